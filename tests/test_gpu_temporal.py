"""Temporal blocking: k steps per pass over HBM must give exactly the lattice,
block sums and field of k single steps, and of the oracle.  Needs a GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(LG, w, h, cells, seed, inlet, mode, k, plan, block=16):
    g = LG.GpuLattice(w, h, True, seed)
    g.set_step_mode(mode)
    if mode == 3:
        g.set_temporal_depth(k)
    if inlet:
        g.set_inlet(inlet, 0.3, (0.2, 0.0), True)
    g.attach_field(block, block)
    g.load(cells)
    for n, every in plan:
        g.advance_sampling(n, every, 0.5)
    out = (g.store(), g.read_block_sums(), g.read_field().ux.copy(), g.steps,
           g.total_particles())
    g.close()
    return out


def same(a, b):
    assert np.array_equal(a[0], b[0]), "lattices differ in %d cells" % int((a[0] != b[0]).sum())
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)
    assert np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32))
    assert a[3] == b[3] and a[4] == b[4]


@pytest.mark.parametrize("k", [4, 8])
@pytest.mark.parametrize("w,h,inlet", [
    (2048, 256, 8),      # 64 words per row: the smallest width the blocked kernel takes
    (2049, 130, 40),     # one valid bit in the last word, two-word inlet
    (3000, 200, 0),      # several strips, ragged last strip, no inlet
])
def test_temporal_equals_single_steps(LG, w, h, inlet, k):
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w * 0.3, h * 0.4, 20.0)
    LG.add_circle(cells, w, h, 5.0, h * 0.7, 9.0)      # an obstacle across the x wrap
    LG.init_equilibrium(cells, 0.3, 0.2, 0.0, True, 11 + w)
    seed = 0x5EED0000 + w
    plan = [(37, 10), (64, 0), (3, 0), (100, 50)]
    a = run(LG, w, h, cells, seed, inlet, 1, k, plan)
    b = run(LG, w, h, cells, seed, inlet, 3, k, plan)
    same(a, b)


def test_temporal_matches_the_oracle(LG, O):
    w, h, inlet = 2080, 96, 8
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, 700.0, 40.0, 15.0)
    LG.init_equilibrium(cells, 0.25, 0.2, 0.0, True, 3)
    g = LG.GpuLattice(w, h, True, 77)
    g.set_step_mode(3)
    g.set_temporal_depth(8)
    g.set_inlet(inlet, 0.3, (0.2, 0.0), True)
    g.load(cells)
    g.advance(40)
    o = O.BitplaneLattice(w, h, True, 77, 8)
    o.set_inlet(inlet, 0.3, (0.2, 0.0), True)
    o.load(cells)
    o.advance(40)
    assert np.array_equal(g.store(), o.store())


def test_roofline_case_as_stated_against_the_oracle_on_a_band(LG, O):
    """The roofline case as stated: 32768 x 16384, 200 circles, 8-column inflow,
    2,000 steps.  Temporal blocking (k = 4 and 8) gives the single-step kernel's
    lattice after 2,000 steps, every cell; and a 1024-row band containing obstacles
    and the inflow equals the oracle's over the last 64 steps: the oracle takes the
    device's whole lattice after 1,936 steps and steps only the band (widened by the
    steps left), which is exact on the band (lgo_bp_advance_window)."""
    import os
    from lattice_gas import workloads as W
    wl = W.roofline_case()
    n, tail, y0, y1 = 2000, 64, 7680, 8704
    assert (wl.cells[y0 * wl.w:y1 * wl.w] & 0x80).any()
    finals = {}
    for mode, k in ((1, 0), (3, 4), (3, 8)):
        g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
        g.set_step_mode(mode)
        if k:
            g.set_temporal_depth(k)
        g.set_inlet(wl.inlet_cols, wl.density, wl.inflow, True)
        g.load(wl.cells)
        if mode == 1:
            g.advance(n - tail)
            o = O.BitplaneLattice(wl.w, wl.h, True, wl.seed, max(1, min(16, os.cpu_count() or 1)))
            o.set_inlet(wl.inlet_cols, wl.density, wl.inflow, True)
            o.load(g.store())
            o.set_steps(n - tail)
            o.advance_window(tail, y0, y1)
            g.advance(tail)
            band = o.store_rows(y0, y1)
            del o
            got = g.store()
            assert np.array_equal(got[y0 * wl.w:y1 * wl.w], band), \
                "the band differs from the oracle in %d cells" % int(
                    (got[y0 * wl.w:y1 * wl.w] != band).sum())
        else:
            g.advance(n)
            got = g.store()
        assert g.steps == n
        finals[k] = got
        g.close()
    for k in (4, 8):
        assert np.array_equal(finals[0], finals[k]), \
            "temporal k=%d differs from single steps in %d cells" % (
                k, int((finals[0] != finals[k]).sum()))


def test_full_size_roofline_case_temporal_equals_single(LG):
    """32768 x 16384 with 200 circles and the inflow, 24 steps: blocked (k = 8)
    against single steps, compared through the exact block sums and count."""
    from lattice_gas import workloads as W
    wl = W.roofline_case(steps=24)
    out = []
    for mode in (1, 3):
        g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
        g.set_step_mode(mode)
        if mode == 3:
            g.set_temporal_depth(8)
        g.set_inlet(wl.inlet_cols, wl.density, wl.inflow, True)
        g.attach_field(32, 32)
        g.load(wl.cells)
        g.advance_sampling(24, 24, 1.0)
        out.append((g.read_block_sums(), g.total_particles()))
        g.close()
    for x, y in zip(out[0][0], out[1][0]):
        assert np.array_equal(x, y)
    assert out[0][1] == out[1][1]
