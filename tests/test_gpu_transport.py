"""Transport observables on the device: row_ux / column_uy / line sums
(src/transport.rs:51-91) against the oracle on the stored cells, and
lgx_transport_measure against the oracle's transport::measure on the bitplane
path (src/transport.rs:131-319), bit for bit: windows, averaged modes, nu, g.
Needs a GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CX2 = np.array([2, 1, -1, -2, -1, 1], np.int64)
CY2 = np.array([0, 1, 1, 0, -1, -1], np.int64)


def line_sums_numpy(cells, w, h):
    """WITH_WALLS (mass, px2, py2) per row and per column (src/moments.rs:37-74)."""
    c = cells.reshape(h, w)
    bits = [((c >> d) & 1).astype(np.int64) for d in range(7)]
    mass = sum(bits)
    px2 = sum(CX2[d] * bits[d] for d in range(6))
    py2 = sum(CY2[d] * bits[d] for d in range(6))
    rows = np.stack([mass.sum(1), px2.sum(1), py2.sum(1)])
    cols = np.stack([mass.sum(0), px2.sum(0), py2.sum(0)])
    return rows, cols


@pytest.mark.parametrize("w,h,rest,obstacle,steps", [
    (64, 32, True, False, 0),
    (100, 38, True, True, 17),     # ragged last word, walls holding particles
    (33, 10, False, False, 5),
    (1000, 602, True, True, 40),   # many row bands, 32 words per row
    (4096, 64, False, False, 3),   # wide: several column passes per thread
])
def test_profiles_match_the_oracle(LG, O, w, h, rest, obstacle, steps):
    rng = np.random.default_rng(w * 7 + h)
    cells = rng.integers(0, 128 if rest else 64, w * h, dtype=np.uint8)
    if obstacle:
        LG.add_circle(cells, w, h, w / 3.0, h * 0.4, min(w, h) / 4.0)
        LG.add_box(cells, w, h, 0.0, float(w), 0.0, 1.5)
    g = LG.GpuLattice(w, h, rest, 0xABC)
    g.load(cells)
    g.advance(steps)
    now = g.store()
    np.testing.assert_array_equal(g.row_ux(), O.row_ux(now, w, h))
    np.testing.assert_array_equal(g.column_uy(), O.column_uy(now, w, h))
    rows, cols = g.line_sums()
    want_rows, want_cols = line_sums_numpy(now, w, h)
    np.testing.assert_array_equal(rows, want_rows)
    np.testing.assert_array_equal(cols, want_cols)
    # twice: the column sums are cleared for the next use
    np.testing.assert_array_equal(g.column_uy(), O.column_uy(now, w, h))


def check_same(got, want):
    assert got.window_nu == want.window_nu
    assert got.window_g == want.window_g
    assert np.float32(got.u_actual) == np.float32(want.u_actual)
    np.testing.assert_array_equal(np.array(got.mode_nu), np.array(want.mode_nu))
    np.testing.assert_array_equal(np.array(got.mode_g), np.array(want.mode_g))
    assert np.float32(got.nu) == np.float32(want.nu)
    assert np.float32(got.g) == np.float32(want.g)


@pytest.mark.parametrize("density,rest,size", [(0.22, True, 64), (0.3, False, 48)])
def test_measure_matches_the_oracle(LG, O, density, rest, size):
    got = LG.transport_measure([density], rest=rest, seed=0x5EED, size=size)[0]
    want = O.transport_measure(density, rest, 4, 0x5EED, size, gpu=True)
    check_same(got, want)


def test_density_scan_is_each_measure(LG, O):
    """Several densities in one batch: each result is the single measurement's."""
    ds = [0.12, 0.22, 0.35]
    got = LG.transport_measure(ds, rest=True, seed=0x1234, size=64)
    for d, r in zip(ds, got):
        check_same(r, O.transport_measure(d, True, 4, 0x1234, 64, gpu=True))
