"""The reference's byte-per-cell update on the device (lgx_byte_*): its golden
tests (tests/golden.rs) through the engine, bit for bit, and agreement with the
oracle's Lattice::step on other sizes, thread bands, obstacles and inflows.
Needs a GPU."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden_byte.json")))
DENSITY = np.float32(float(GOLD["constants"]["DENSITY"]))
SPEED = np.float32(float(GOLD["constants"]["SPEED"]))
SEED = int(GOLD["constants"]["SEED"], 16)
BLOCK = int(GOLD["constants"]["BLOCK"])


def golden_cells(LG, c):
    """tests/golden.rs:76-86 with the engine's own host setup."""
    w, h = c["w"], c["h"]
    cells = np.zeros(w * h, np.uint8)
    if c["plate"]:
        yc = np.float32(h) * LG.SQRT3_2 / np.float32(2.0)
        x0 = np.float32(w) / np.float32(5.0)
        LG.add_box(cells, w, h, x0, x0 + np.float32(3.0), yc - np.float32(12.0),
                   yc + np.float32(12.0))
    LG.init_equilibrium(cells, DENSITY, SPEED, 0.0, c["rest"], SEED)
    return cells


@pytest.mark.parametrize("case", GOLD["cases"], ids=[c["name"] for c in GOLD["cases"]])
def test_golden_output_on_the_device(LG, O, case):
    g = GOLD["golden"][case["name"]]
    lat = LG.Lattice(case["w"], case["h"], DENSITY, (SPEED, 0.0), case["inlet"], case["rest"],
                     case["threads"], SEED)
    lat.load(golden_cells(LG, case))
    lat.advance(case["steps"])
    cells = lat.store()
    assert O.fnv1a(cells) == int(g["cells"], 16)
    lat.attach_field(BLOCK, BLOCK)
    lat.sample_field(1.0)
    f = lat.read_field()
    fb = b"".join(a.astype("<f4").tobytes() for a in (f.ux, f.uy, f.rho, f.solid))
    assert O.fnv1a(fb) == int(g["field"], 16)
    assert O.invariants(cells) == (g["mass"], g["px"], g["py"])
    assert lat.total_particles() == g["mass"]
    ux, uy = lat.mean_velocity()  # tests/golden.rs:130, 217: the record's six decimals
    assert abs(ux - g["ux"]) < 5e-7 and abs(uy - g["uy"]) < 5e-7
    assert lat.steps == case["steps"]


@pytest.mark.parametrize("w,h,threads,inlet,rest", [
    (300, 64, 3, 40, True),     # partial last segment, two-word inlet
    (129, 18, 5, 8, True),      # odd width, bands of 4 rows with a short last band
    (64, 64, 8, 0, False),      # six-direction rule
    (1000, 40, 1, 70, True),    # one band, many segments per row
    (48, 48, 48, 0, True),      # a band per row
    (16640, 8, 3, 20, True),    # rows wider than one tile: two tiles across, word loads
    (16390, 6, 2, 5, False),    # two tiles across, byte loads, a 6-cell last segment
    (200, 30, 30, 0, True),     # four segments and eight rows per tile, eight bands in it
])
def test_device_byte_path_matches_the_oracle(LG, O, w, h, threads, inlet, rest):
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w / 3.0, h * 0.4, min(w, h) / 6.0)
    LG.init_equilibrium(cells, 0.3, 0.15, 0.0, rest, 99 + w)
    seed = 0xFEEDFACE + w
    lat = LG.Lattice(w, h, 0.3, (0.15, 0.0), inlet, rest, threads, seed)
    lat.load(cells)
    ref = O.Lattice(w, h, 0.3, (0.15, 0.0), inlet, rest, threads, seed)
    ref.set_cells(cells)
    for n in (1, 13, 60):
        lat.advance(n)
        ref.advance(n)
        got = lat.store()
        assert np.array_equal(got, ref.cells), "differs in %d cells" % int((got != ref.cells).sum())


@pytest.mark.parametrize("threads", [1, 3])
def test_periodic_box_on_the_byte_path(LG, O, threads):
    """The plain CPU-runnable case on the device byte stream: a 256 x 128 periodic
    FHP-III box, no obstacle, every channel Bernoulli(0.25) (Lattice::new(256, 128,
    0.25, (0, 0), 0, true, T, seed) and init_equilibrium, filled on the device), 500
    steps at T = 1 and T = 3 thread bands.  The device's cells equal the oracle's
    Lattice::step bit for bit; the 8 x 8 field and the exact integer block sums formed
    on the device equal the oracle's; mass and momentum are conserved exactly."""
    w, h, seed, bs = 256, 128, 0x5EED, 8
    lat = LG.Lattice(w, h, 0.25, (0.0, 0.0), 0, True, threads, seed)
    lat.load(np.zeros(w * h, np.uint8))
    lat.init_equilibrium()
    ref = O.Lattice(w, h, 0.25, (0.0, 0.0), 0, True, threads, seed)
    ref.init_equilibrium()
    start = lat.store()
    assert np.array_equal(start, ref.cells)
    assert (start & 0x80).sum() == 0 and (start & 0x7F).any()
    before = O.invariants(start)
    lat.advance(500)
    ref.advance(500)
    got = lat.store()
    assert np.array_equal(got, ref.cells), "differs in %d cells" % int((got != ref.cells).sum())
    assert O.invariants(got) == before
    assert lat.total_particles() == before[0] and lat.steps == 500
    lat.attach_field(bs, bs)
    lat.sample_field(1.0)
    f = lat.read_field()
    want = O.Field(w, h, bs, bs)
    want.sample(ref.cells, w, h, 1.0)
    for a, b in zip((f.ux, f.uy, f.rho, f.solid), (want.ux, want.uy, want.rho, want.solid)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    g = LG.GpuLattice(w, h, True, seed)
    g.attach_field(bs, bs)
    g.load(got)
    g.sample_field(1.0)
    sums = g.read_block_sums()
    for a, b in zip(sums, O.block_sums(ref.cells, w, h, bs, bs)):
        assert np.array_equal(a, b)
    assert tuple(int(s.sum(dtype=np.int64)) for s in sums[:3]) == before
    g.close()
    lat.close()


def test_restart_and_thread_invariance_of_conserved_quantities(LG, O):
    """tests/golden.rs:262-297 on the device: closed box, 1/2/3/5/8 bands."""
    for rest in (False, True):
        expected = None
        cells = np.zeros(64 * 64, np.uint8)
        LG.init_equilibrium(cells, DENSITY, SPEED, 0.0, rest, SEED)
        before = O.invariants(cells)
        for threads in (1, 2, 3, 5, 8):
            lat = LG.Lattice(64, 64, DENSITY, (SPEED, 0.0), 0, rest, threads, SEED)
            lat.restart(cells, SEED)
            lat.advance(100)
            after = O.invariants(lat.store())
            assert after == before
            if expected is None:
                expected = after
            assert after == expected


def test_full_size_wake_run_on_the_byte_path(LG, O):
    """4096 x 2304, the full-size wake run on the reference's byte stream (16 bands, the
    plate, walls, an 8-column inflow): the device equals the oracle's Lattice::step after
    1, 4 and 12 steps, and the obstacles and walls stay in place."""
    from lattice_gas import workloads as W
    wl = W.wake_run()
    lat = LG.Lattice(wl.w, wl.h, wl.density, wl.inflow, wl.inlet_cols, wl.rest, 16, wl.seed)
    lat.load(wl.cells)
    ref = O.Lattice(wl.w, wl.h, wl.density, wl.inflow, wl.inlet_cols, wl.rest, 16, wl.seed)
    ref.set_cells(wl.cells)
    solid = (np.asarray(wl.cells) & 0x80) != 0
    for n in (1, 3, 8):
        lat.advance(n)
        ref.advance(n)
        got = lat.store()
        assert np.array_equal(got, ref.cells), "differs in %d cells" % int((got != ref.cells).sum())
        assert np.array_equal((got & 0x80) != 0, solid)
    assert lat.total_particles() == ref.total_particles()


def test_full_size_fill_then_step_on_the_byte_path(LG, O):
    """The wake run's geometry filled on the device (init_equilibrium), then 5 steps: the
    same cells as the oracle's fill and steps."""
    from lattice_gas import workloads as W
    wl = W.wake_run()
    lat = LG.Lattice(wl.w, wl.h, wl.density, wl.inflow, wl.inlet_cols, wl.rest, 16, wl.seed)
    lat.load(wl.cells)
    lat.init_equilibrium()
    ref = O.Lattice(wl.w, wl.h, wl.density, wl.inflow, wl.inlet_cols, wl.rest, 16, wl.seed)
    ref.set_cells(wl.cells)
    ref.init_equilibrium()
    assert np.array_equal(lat.store(), ref.cells)
    lat.advance(5)
    ref.advance(5)
    assert np.array_equal(lat.store(), ref.cells)


@pytest.mark.parametrize("w,h,threads,inlet,rest", [(300, 64, 3, 40, True), (129, 18, 5, 8, False),
                                                    (2048, 1280, 12, 8, True)])
def test_lattice_mean_velocity_on_the_device(LG, O, w, h, threads, inlet, rest):
    """Lattice::mean_velocity (src/lattice.rs:286-294) of the device byte lattice and of
    a bitplane lattice holding the same cells equals the oracle's, bit for bit; an
    empty lattice gives (0, 0)."""
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w / 3.0, h * 0.4, min(w, h) / 6.0)
    LG.init_equilibrium(cells, 0.3, 0.15, 0.05, rest, 7 + w)
    lat = LG.Lattice(w, h, 0.3, (0.15, 0.0), inlet, rest, threads, 11)
    lat.load(cells)
    lat.advance(17)
    ref = O.Lattice(w, h, 0.3, (0.15, 0.0), inlet, rest, threads, 11)
    ref.set_cells(lat.store())
    want = [np.float32(v).view(np.uint32) for v in ref.mean_velocity()]
    assert [np.float32(v).view(np.uint32) for v in lat.mean_velocity()] == want
    g = LG.GpuLattice(w, h, rest, 3)
    g.load(lat.store())
    assert [np.float32(v).view(np.uint32) for v in g.lattice_mean_velocity()] == want
    g.load(np.zeros(w * h, np.uint8))
    assert g.lattice_mean_velocity() == (0.0, 0.0)
