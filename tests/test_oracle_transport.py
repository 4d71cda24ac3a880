"""The oracle's transport profiles (src/transport.rs:51-91) against a numpy
restatement of the WITH_WALLS moments, and its measurement's invariants: the
same inputs give the same result, the windows and intervals obey
transport.rs:131-165, and the realised start speed is the start's mean."""
import numpy as np

from test_gpu_transport import line_sums_numpy

SQRT3_2 = np.float32(0.8660254)


def test_profiles_match_numpy(O):
    rng = np.random.default_rng(3)
    w, h = 70, 24
    cells = rng.integers(0, 256, w * h, dtype=np.uint8)  # solid cells keep their particles
    rows, cols = line_sums_numpy(cells, w, h)
    mass, px2 = rows[0], rows[1]
    want_ux = np.where(mass > 0, (px2.astype(np.float32) * np.float32(0.5)) /
                       np.maximum(mass, 1).astype(np.float32), np.float32(0))
    np.testing.assert_array_equal(O.row_ux(cells, w, h), want_ux.astype(np.float32))
    cm, cpy = cols[0], cols[2]
    want_uy = np.where(cm > 0, (cpy.astype(np.float32) * SQRT3_2) /
                       np.maximum(cm, 1).astype(np.float32), np.float32(0))
    np.testing.assert_array_equal(O.column_uy(cells, w, h), want_uy.astype(np.float32))


def test_measure_is_deterministic_and_well_formed(O):
    a = O.transport_measure(0.22, True, 2, 0x5EED, 32, gpu=False)
    b = O.transport_measure(0.22, True, 2, 0x5EED, 32, gpu=False)
    assert (a.nu, a.g, a.window_nu, a.window_g) == (b.nu, b.g, b.window_nu, b.window_g)
    for wdw in (a.window_nu, a.window_g):
        assert 80 <= wdw <= 30000
    # u_actual is the mean x-velocity of start(0)
    w = h = 32
    k = np.float32(2.0) * np.float32(np.pi) / np.float32(w)
    uy = (np.float32(0.05) * np.sin(k * np.arange(w, dtype=np.float32))).astype(np.float32)
    seed0 = 0x5EED ^ 0x1357
    cells = O.column_wave_cells(w, h, 0.22, 0.25, uy, True, seed0 ^ 0xF00D)
    m, px, _ = O.invariants(cells)
    assert np.float32(a.u_actual) == np.float32(np.float32(px) * np.float32(0.5) / np.float32(m))
