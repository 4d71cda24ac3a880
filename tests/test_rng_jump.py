"""The generator jumps the device byte path and the equilibrium fill rely on
(lattice-gas_gb300/csrc/lgx_rng.cuh), checked on the host: the characteristic
polynomial of the xorshift64 state update, jump polynomials z^k mod P and the
GF(2) matrix jumps all equal stepping the generator (src/rng.rs:8-34) k times.
Compiles a host-only harness with nvcc; no GPU needed."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_jumps_equal_serial_steps(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc is not available")
    exe = tmp_path / "rng_jump_check"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "lattice-gas_gb300", "csrc"),
                    os.path.join(HERE, "native", "rng_jump_check.cu"), "-o", str(exe)],
                   check=True, capture_output=True, timeout=300)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
