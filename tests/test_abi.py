"""The C ABI: the library builds, loads and exports every entry point that
include/*.h declares; the host-side setup functions reproduce the oracle's;
and without a device the engine refuses loudly rather than falling back."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(lgx_[a-z0-9_]+)\s*\(", txt):
            syms.add(m.group(1))
    return syms


def test_library_exports_every_declared_symbol(engine_lib):
    L = engine_lib.lib()
    syms = declared_symbols()
    assert len(syms) > 20
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, missing


def test_thresholds_match_oracle(O, engine_lib):
    for density, ux, uy in ((0.22, 0.3, 0.0), (0.3, 0.2, 0.0), (0.5, 0.0, 0.2), (0.1, -0.4, 0.3),
                            (0.0, 0.0, 0.0), (1.2, 0.9, 0.0), (float("nan"), 0.0, 0.0)):
        for rest in (False, True):
            assert np.array_equal(engine_lib.thresholds(density, ux, uy, rest),
                                  O.thresholds(density, ux, uy, rest))


def test_init_equilibrium_matches_oracle(O, engine_lib):
    w, h = 300, 64
    cells = np.zeros(w * h, np.uint8)
    engine_lib.add_box(cells, w, h, 60.0, 64.0, 10.0, 40.0)
    engine_lib.add_circle(cells, w, h, 150.0, 27.7, 11.5)
    ref = np.zeros(w * h, np.uint8)
    O.lib().lgo_add_box(O.ptr(ref, C.c_uint8), w, h, 60.0, 64.0, 10.0, 40.0, 0)
    O.lib().lgo_add_circle(O.ptr(ref, C.c_uint8), w, h, 150.0, 27.7, 11.5)
    assert np.array_equal(cells, ref) and (cells == 0x80).sum() > 100
    engine_lib.init_equilibrium(cells, 0.3, 0.2, 0.0, True, 0x5EED)
    want = O.init_equilibrium_cells(ref, 0.3, 0.2, 0.0, True, 0x5EED)
    assert np.array_equal(cells, want)


def test_shear_wave_matches_oracle(O, engine_lib):
    w, h = 64, 40
    k = np.float32(2 * np.pi) / (np.float32(h) * np.float32(0.8660254))
    ux = (np.float32(0.05) * np.sin(k * np.arange(h, dtype=np.float32) * np.float32(0.8660254))
          ).astype(np.float32)
    a = engine_lib.shear_wave(w, h, 0.22, ux, True, 0x5EED ^ 0xBEEF)
    b = O.shear_wave_cells(w, h, 0.22, ux, True, 0x5EED ^ 0xBEEF)
    assert np.array_equal(a, b)


def test_bad_arguments_are_errors_not_crashes(engine_lib):
    LG = engine_lib
    with pytest.raises(LG.LgxError):
        LG.GpuLattice(64, 33, True, 1)    # odd row count (src/gpu.rs:480)
    with pytest.raises(LG.LgxError):
        LG.GpuLattice(4, 64, True, 1)     # too small (src/gpu.rs:481)


def _gpu_present():
    from conftest import _have_gpu
    return _have_gpu()


@pytest.mark.skipif(_gpu_present(), reason="checks the no-device path")
def test_no_device_is_a_loud_error(engine_lib):
    LG = engine_lib
    with pytest.raises(LG.LgxError) as e:
        LG.GpuLattice(64, 64, True, 1)
    assert e.value.code == 3


def test_new_entry_points_refuse_bad_arguments(engine_lib):
    """Argument checks come before any device work, so they hold without a GPU."""
    LG = engine_lib
    L = LG.lib()
    ARG = 1
    d = np.array([0.22], np.float32)
    out = (LG.Transport * 1)()
    dp = d.ctypes.data_as(C.POINTER(C.c_float))
    assert L.lgx_transport_measure(dp, 1, 1, 5, 7, out) == ARG      # odd size
    assert L.lgx_transport_measure(dp, 1, 1, 5, 4, out) == ARG      # too small
    assert L.lgx_transport_measure(dp, 0, 1, 5, 64, out) == ARG     # no densities
    assert L.lgx_transport_measure(None, 1, 1, 5, 64, out) == ARG
    assert L.lgx_transport_measure(dp, 9000, 1, 5, 64, out) == ARG  # too many for one batch
    h = C.c_void_p()
    arr = (C.c_void_p * 1)(None)
    assert L.lgx_batch_create_ex(arr, 1, 9, C.byref(h)) == ARG      # unknown policy
    assert L.lgx_batch_create_ex(arr, 0, 0, C.byref(h)) == ARG      # no lattices
    assert L.lgx_batch_create_ex(arr, 1, 0, C.byref(h)) == ARG      # null lattice
    n = C.c_size_t()
    assert L.lgx_batch_plan(None, None, 0, C.byref(n)) == ARG
    assert L.lgx_get_step_plan(None, None) == ARG
    u = np.zeros(8, np.float32)
    assert L.lgx_row_ux(None, u.ctypes.data_as(C.POINTER(C.c_float)), 8) == ARG
    assert L.lgx_column_uy(None, u.ctypes.data_as(C.POINTER(C.c_float)), 8) == ARG
    assert L.lgx_line_sums(None, None, 0, None, 0) == ARG
    assert L.lgx_init_equilibrium(None, 0.3, 0.0, 0.0, 1) == ARG
    assert L.lgx_byte_init_equilibrium(None) == ARG
    fx, fy = C.c_float(), C.c_float()
    assert L.lgx_mean_velocity(None, C.byref(fx), C.byref(fy)) == ARG
    assert L.lgx_byte_mean_velocity(None, C.byref(fx), C.byref(fy)) == ARG
    assert L.lgx_set_step_mode(None, 4) == ARG                    # LGX_STEP_GRAPH, no lattice
    # the allocation-free step refuses sizes beyond 32 bits before any arithmetic on them
    # (the buffer arguments are never touched on this path)
    nz = [C.c_void_p(0x1000 * (i + 1)) for i in range(4)]
    th = np.zeros(7, np.uint32).ctypes.data_as(C.POINTER(C.c_uint32))
    step = L.lgx_step_planes_noalloc
    step.restype = C.c_int
    step.argtypes = [C.c_void_p] * 4 + [C.c_size_t, C.c_size_t, C.c_int, C.c_size_t,
                                        C.POINTER(C.c_uint32), C.c_uint64, C.c_uint64,
                                        C.c_void_p]
    for w, h, cols in ((2 ** 32 + 64, 64, 0), (64, 2 ** 32 + 64, 0), (64, 64, 2 ** 32 + 8),
                       (2 ** 64 - 1, 64, 0)):
        assert step(*nz, w, h, 1, cols, th, 1, 0, None) == ARG, (w, h, cols)
        assert b"32 bits" in L.lgx_last_error()
    for w, h in ((64, 63), (4, 64)):
        assert step(*nz, w, h, 1, 0, th, 1, 0, None) == ARG, (w, h)
    assert step(None, *nz[1:], 64, 64, 1, 0, th, 1, 0, None) == ARG
    assert step(nz[0], nz[0], nz[2], nz[3], 64, 64, 1, 0, th, 1, 0, None) == ARG  # aliased


@pytest.mark.skipif(_gpu_present(), reason="checks the no-device path")
def test_transport_without_a_device_is_an_error(engine_lib):
    LG = engine_lib
    with pytest.raises(LG.LgxError):
        LG.transport_measure([0.22], size=64)
