"""The structures that cross the C ABI have the same layout on every side.

A C program compiled with gcc against include/lgx.h prints the size and field
offsets of lgx_step_plan, lgx_batch_class, lgx_transport, lgx_request and
lgx_server_stats.  The Python ctypes mirrors (lattice_gas/__init__.py) and the
Rust #[repr(C)] mirrors that INTEGRATION.md gives a maintainer for src/cuda.rs
must match it field for field; the Rust extern "C" declarations there must name
functions the header declares, with the same number of arguments.  No GPU is
needed.
"""
import json
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RUST_TO_C = {"LgxStepPlan": "lgx_step_plan", "LgxBatchClass": "lgx_batch_class",
             "LgxTransport": "lgx_transport", "LgxRequest": "lgx_request",
             "LgxServerStats": "lgx_server_stats"}

# (size, alignment) of the Rust field types the mirrors use, on a 64-bit target
RUST_TYPES = {"c_int": (4, 4), "i32": (4, 4), "u32": (4, 4), "f32": (4, 4), "u64": (8, 8),
              "i64": (8, 8), "usize": (8, 8), "f64": (8, 8), "u8": (1, 1)}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    exe = str(d / "abi_layout")
    subprocess.run([cc, "-std=c11", "-O0", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "native", "abi_layout.c"), "-o", exe],
                   check=True)
    return json.loads(subprocess.run([exe], check=True, capture_output=True,
                                     text=True).stdout)


def _rust_type(t):
    t = t.strip()
    if t.startswith("*"):
        return 8, 8
    m = re.fullmatch(r"\[(\w+);\s*(\d+)\]", t)
    if m:
        size, align = RUST_TYPES[m.group(1)]
        return size * int(m.group(2)), align
    return RUST_TYPES[t]


def rust_structs():
    """#[repr(C)] structs with fields, from the Rust code blocks of INTEGRATION.md,
    laid out by C rules (which #[repr(C)] follows)."""
    txt = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    out = {}
    for m in re.finditer(r"#\[repr\(C\)\]\s*pub struct (\w+)\s*\{(.*?)\}", txt, re.S):
        body = m.group(2)
        fields = re.findall(r"pub (\w+):\s*([^,]+?)\s*(?:,|$)", body.replace("\n", " "))
        if not fields:
            continue    # opaque handle types
        off, align_max, layout = 0, 1, {}
        for name, ty in fields:
            size, align = _rust_type(ty)
            off = (off + align - 1) // align * align
            layout[name] = [off, size]
            off += size
            align_max = max(align_max, align)
        out[m.group(1)] = {"__size__": (off + align_max - 1) // align_max * align_max,
                           "fields": layout}
    return out


def header_arity():
    txt = open(os.path.join(ROOT, "include", "lgx.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(lgx_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt, re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_python_mirrors_match_the_header(c_layout, engine_lib):
    import ctypes as C
    LG = engine_lib
    mirrors = {"lgx_step_plan": LG.StepPlan, "lgx_batch_class": LG.BatchClass,
               "lgx_transport": LG.Transport, "lgx_request": LG.Request,
               "lgx_server_stats": LG.ServerStats}
    for cname, cls in mirrors.items():
        want = c_layout[cname]
        assert C.sizeof(cls) == want["__size__"], cname
        names = [f[0] for f in cls._fields_]
        assert names == list(want["fields"]), cname
        for name, (off, size) in want["fields"].items():
            assert getattr(cls, name).offset == off, (cname, name)
            assert getattr(cls, name).size == size, (cname, name)


def test_rust_mirrors_match_the_header(c_layout):
    rs = rust_structs()
    assert set(RUST_TO_C) <= set(rs), "INTEGRATION.md lacks a Rust mirror: %s" % (
        sorted(set(RUST_TO_C) - set(rs)))
    for rname, cname in RUST_TO_C.items():
        assert rs[rname] == c_layout[cname], (rname, rs[rname], c_layout[cname])


def test_rust_declarations_match_the_header():
    txt = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    decl = header_arity()
    seen = 0
    for m in re.finditer(r"\bfn (lgx_[a-z0-9_]+)\(([^)]*)\)\s*->", txt, re.S):
        name, args = m.group(1), m.group(2).strip()
        assert name in decl, "%s is not declared in include/lgx.h" % name
        n = 0 if not args else len([a for a in args.split(",") if a.strip()])
        assert n == decl[name], (name, n, decl[name])
        seen += 1
    assert seen >= 30
    assert "lgx_advance" in re.findall(r"\bfn (lgx_[a-z0-9_]+)\(", txt)
