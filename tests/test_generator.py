"""The collision-circuit generator and the circuit it emits.

The emitted header is compiled as host C++ here and checked, word for word,
against the oracle's lane-by-lane class rule on random planes and on the
exhaustive KAT domain (src/gpu.rs:775-820).
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GEN_OUT = os.path.join(ROOT, "lattice-gas_gb300", "csrc", "generated", "collide.cuh")

HOST_SHIM = r"""
#include <stdint.h>
#include "collide.cuh"
extern "C" void host_collide(int rest, const uint32_t* n, const uint32_t* s, uint32_t* o) {
  if (rest) lgx_collide_rest(n, s[0], s + 1, s + 4, o);
  else lgx_collide_norest(n, s[0], s + 1, s + 4, o);
}
"""


@pytest.fixture(scope="module")
def host_circuit():
    import ctypes as C
    d = tempfile.mkdtemp(prefix="lgx_gen_")
    src = os.path.join(d, "shim.cpp")
    open(src, "w").write(HOST_SHIM)
    so = os.path.join(d, "shim.so")
    subprocess.run(["g++", "-O1", "-shared", "-fPIC", "-I", os.path.dirname(GEN_OUT), src, "-o", so],
                   check=True)
    L = C.CDLL(so)
    L.host_collide.restype = None
    return L


def test_generator_output_is_committed_and_current():
    import collide_gen as G
    src, report = G.generate()
    assert open(GEN_OUT).read() == src, "regenerate with gen/collide_gen.py"
    assert report["lgx_collide_rest"]["checked"] == 6144
    # the mapped circuit must stay well under the reference's 685 two-input operators
    assert report["lgx_collide_rest"]["lop3"] < 300


@pytest.mark.parametrize("rest", [True, False])
def test_emitted_circuit_matches_lane_rule_on_random_words(O, host_circuit, rest):
    import ctypes as C
    rng = np.random.default_rng(1234 + rest)
    for it in range(400):
        n = rng.integers(0, 2 ** 32, 7, dtype=np.uint64).astype(np.uint32)
        s = np.zeros(9, np.uint32)
        O.lib().lgo_draws(int(rng.integers(0, 2 ** 32)), O.ptr(s, C.c_uint32))
        want = np.zeros(7, np.uint32)
        got = np.zeros(7, np.uint32)
        O.lib().lgo_collide_word(int(rest), O.ptr(n, C.c_uint32), O.ptr(s, C.c_uint32),
                                 O.ptr(want, C.c_uint32))
        host_circuit.host_collide(int(rest), n.ctypes.data_as(C.POINTER(C.c_uint32)),
                                  s.ctypes.data_as(C.POINTER(C.c_uint32)),
                                  got.ctypes.data_as(C.POINTER(C.c_uint32)))
        assert np.array_equal(want, got), (it, n, s)


@pytest.mark.parametrize("rest", [True, False])
def test_emitted_circuit_exhaustive(O, host_circuit, rest):
    """All-lanes-equal inputs for every (state, two, three, five), as lgca_verify."""
    import ctypes as C
    n_states = 128 if rest else 64
    for state in range(n_states):
        for two in (0, 1):
            for three in range(4):
                for five in range(6):
                    n = np.array([0xFFFFFFFF if state >> d & 1 else 0 for d in range(7)], np.uint32)
                    s = np.zeros(9, np.uint32)
                    s[0] = 0xFFFFFFFF if two else 0
                    if three < 3:
                        s[1 + three] = 0xFFFFFFFF
                    if five < 5:
                        s[4 + five] = 0xFFFFFFFF
                    o = np.zeros(7, np.uint32)
                    host_circuit.host_collide(int(rest), n.ctypes.data_as(C.POINTER(C.c_uint32)),
                                              s.ctypes.data_as(C.POINTER(C.c_uint32)),
                                              o.ctypes.data_as(C.POINTER(C.c_uint32)))
                    assert all(v in (0, 0xFFFFFFFF) for v in o)
                    got = sum(1 << d for d in range(7) if o[d])
                    assert got == O.lib().lgo_collide_lane(int(rest), state, two, three, five)
