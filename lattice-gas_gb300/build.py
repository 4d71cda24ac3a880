"""Build the engine: generate the collision circuit, compile the CUDA sources
for sm_103a and link lattice_gas/liblgx.so (the C-ABI library).

    python lattice-gas_gb300/build.py            # incremental
    python lattice-gas_gb300/build.py --force    # rebuild everything

nvcc compiles each translation unit in parallel; there is no cmake.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lattice_gas", "liblgx.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I" + CSRC, "-I" + INCLUDE]
SOURCES = ["lgx_step.cu", "lgx_temporal.cu", "lgx_field.cu", "lgx_batch.cu", "lgx_bytes.cu",
           "lgx_noalloc.cu", "lgx_init.cu", "lgx_profile.cu", "lgx_transport.cpp",
           "lgx_resident.cu", "lgx_resident_fixed.cu", "lgx_tune.cpp", "lgx_probe.cu",
           "lgx_lattice.cpp", "lgx_batch_host.cpp", "lgx_server.cpp", "lgx_setup.cpp"]


def _deps():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    deps += [os.path.join(CSRC, "generated", f) for f in os.listdir(os.path.join(CSRC, "generated"))]
    deps.append(os.path.join(INCLUDE, "lgx.h"))
    return deps


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def _compile(src, force, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not force and not _stale(obj, [src] + _deps()):
        return obj, None
    cmd = [NVCC] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, (r.stdout + r.stderr)


def generate():
    r = subprocess.run([sys.executable, os.path.join(HERE, "gen", "collide_gen.py")],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("collision generator failed:\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    generate()
    extra = ["-Xptxas", "-v"] if ptxas_v else []
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, force, extra), srcs))
    objs = [o for o, _ in results]
    for o, log in results:
        if log and (verbose or ptxas_v):
            print(log, file=sys.stderr)
    if force or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-v", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=True, ptxas_v=a.ptxas_v))
