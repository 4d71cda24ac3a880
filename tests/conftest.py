"""Shared test setup.

`-m "not gpu"` runs on any machine: the oracle against the reference's golden
vectors, the circuit generator, the host-side setup code and the C ABI's
exports.  `-m gpu` runs the CUDA engine against the oracle and needs a GPU.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "lattice-gas_gb300"),
          os.path.join(ROOT, "lattice-gas_gb300", "gen"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def O():
    import oracle as O_
    O_.lib()
    return O_


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if needed) and load liblgx.so."""
    import build as B
    B.build()
    import lattice_gas as LG
    LG.lib()
    return LG


def _have_gpu():
    try:
        import ctypes
        rt = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if rt is None:
            return False
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def LG(engine_lib):
    """The engine on a GPU: fails loudly (no skip) when the marker says gpu."""
    return engine_lib
