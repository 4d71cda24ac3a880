"""The CUDA engine against the oracle, through the C ABI.

Bit-exact: after N steps from the same cells and seed, the lattice state, the
integer block sums, the f32 field and the particle count are identical to the
oracle's restatement of the reference's bitplane path (src/gpu.rs).  The
reference's own GPU tests (src/gpu.rs:773-1451) are restated against the
engine as well.  Every test here needs a GPU.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DX_EVEN = (1, 0, -1, -1, -1, 0)
DX_ODD = (1, 1, 0, -1, 0, 1)
DY = (0, 1, 1, 0, -1, -1)
THREADS = max(1, min(16, os.cpu_count() or 1))


def pair(LG, O, w, h, rest, seed, cells, inlet=None, block=None, mode=0):
    g = LG.GpuLattice(w, h, rest, seed)
    g.set_step_mode(mode)
    o = O.BitplaneLattice(w, h, rest, seed, THREADS)
    if inlet:
        g.set_inlet(*inlet)
        o.set_inlet(*inlet)
    if block:
        g.attach_field(block, block)
        o.attach_field(block, block)
    g.load(cells)
    o.load(cells)
    return g, o


def assert_same(g, o, with_field=True):
    a, b = g.store(), o.store()
    if not np.array_equal(a, b):
        bad = np.nonzero(a != b)[0]
        raise AssertionError("%d cells differ; first at %d (x=%d, y=%d): gpu %02x oracle %02x"
                             % (bad.size, bad[0], bad[0] % g.w, bad[0] // g.w, a[bad[0]],
                                b[bad[0]]))
    assert g.total_particles() == o.total_particles()
    assert g.steps == o.steps
    if with_field and g._field is not None:
        for x, y in zip(g.read_block_sums(), o.read_block_sums()):
            assert np.array_equal(x, y)
        f = g.read_field()
        for x, y in zip((f.ux, f.uy, f.rho, f.solid), o.read_field()):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


# ---- the reference's GPU tests, restated ---------------------------------

@pytest.mark.parametrize("rest", [True, False])
def test_the_device_rule_matches_the_enumeration(LG, O, rest):
    """src/gpu.rs:775-820, on the circuit the step kernel runs."""
    got = LG.verify_circuit(rest)
    L = O.lib()
    for i, v in enumerate(got):
        five, three, two, state = i % 6, (i // 6) % 4, (i // 24) % 2, i // 48
        assert v >> 16 == 0, "lanes disagreed on state %d" % state
        assert (v & 0xFF) == L.lgo_collide_lane(int(rest), state, two, three, five)


@pytest.mark.parametrize("w", [64, 80, 20, 33, 100])
def test_a_single_particle_travels_in_a_straight_line(LG, w):
    """src/gpu.rs:826-863, plus one-word (w=20) and one-bit-tail (w=33) rows."""
    h, steps = 48, 8
    for d in range(6):
        for start_row in (10, 11):
            g = LG.GpuLattice(w, h, True, 1)
            cells = np.zeros(w * h, np.uint8)
            x0, y0 = min(24, w - 2), start_row
            cells[y0 * w + x0] = 1 << d
            g.load(cells)
            g.advance(steps)
            out = g.store()
            live = np.nonzero(out & 0x7F)[0]
            assert len(live) == 1 and out[live[0]] == 1 << d
            x, y = x0, y0
            for _ in range(steps):
                x = (x + (DX_ODD[d] if y & 1 else DX_EVEN[d])) % w
                y = (y + DY[d]) % h
            assert live[0] == y * w + x, (w, d, start_row)


def test_walls_reverse_particles(LG):
    """src/gpu.rs:867-885."""
    w, h = 64, 48
    g = LG.GpuLattice(w, h, True, 1)
    cells = np.zeros(w * h, np.uint8)
    cells[24 * w + 23] = 0x80
    cells[24 * w + 20] = 1
    g.load(cells)
    g.advance(6)
    out = g.store()
    live = np.nonzero(out & 0x7F)[0]
    assert len(live) == 1 and out[live[0]] & 0x7F == 1 << 3 and live[0] == 24 * w + 20


@pytest.mark.parametrize("rest", [True, False])
def test_a_periodic_box_conserves_mass_and_momentum(LG, O, rest):
    """src/gpu.rs:889-924."""
    w, h = 128, 64
    d = np.zeros(w * h, np.uint64)
    O.lib().lgo_rng_draws(7, O.ptr(d, O.C.c_uint64), d.size)
    cells = ((d >> np.uint64(32)) & np.uint64(0xFF)).astype(np.uint8) & (0x7F if rest else 0x3F)
    before = O.invariants(cells)
    g = LG.GpuLattice(w, h, rest, 0xC0FFEE)
    g.load(cells)
    g.advance(250)
    assert O.invariants(g.store()) == before


@pytest.mark.parametrize("w", [64, 100, 33, 20])
def test_load_and_store_round_trip(LG, O, w):
    """src/gpu.rs:929-948."""
    h = 16
    d = np.zeros(w * h, np.uint64)
    O.lib().lgo_rng_draws(11, O.ptr(d, O.C.c_uint64), d.size)
    b = ((d >> np.uint64(32)) & np.uint64(0xFF)).astype(np.uint8)
    want = np.where(b & 0x80, 0x80, b & 0x7F).astype(np.uint8)
    g = LG.GpuLattice(w, h, True, 1)
    g.load(want)
    assert np.array_equal(g.store(), want)


@pytest.mark.parametrize("w,h,block", [(256, 128, 20), (200, 96, 16)])
def test_the_gpu_coarse_grains_the_same_field(LG, O, w, h, block):
    """src/gpu.rs:955-994, bit-exact against the CPU Field::sample."""
    cpu = O.Lattice(w, h, 0.22, (0.3, 0.0), 0, True, 4, 0x5EED)
    yc = np.float32(h) * O.SQRT3_2 / np.float32(2.0)
    cpu.add_circle(np.float32(60.0), yc, np.float32(18.0))
    cpu.init_equilibrium()
    cpu.advance(30)
    want = O.Field(w, h, block, block)
    want.sample(cpu.cells, w, h, 1.0)
    g = LG.GpuLattice(w, h, True, 1)
    g.attach_field(block, block)
    g.load(cpu.cells.copy())
    g.sample_field(1.0)
    f = g.read_field()
    for a, b in zip((want.ux, want.uy, want.rho, want.solid), (f.ux, f.uy, f.rho, f.solid)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    for a, b in zip(O.block_sums(cpu.cells, w, h, block, block), g.read_block_sums()):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("w,h,bx,by", [
    (200, 40, 15, 8),      # below 16 columns: one warp per block
    (256, 64, 16, 16), (250, 42, 16, 7), (300, 40, 17, 20), (2048, 80, 20, 20),
    (263, 66, 31, 33), (4096, 64, 32, 32), (330, 36, 33, 1), (500, 50, 48, 5),
    (1000, 24, 100, 12), (900, 30, 250, 3),
    (2400, 14, 1100, 7),   # one block per CTA, its words past one warp's lanes
])
def test_the_coarse_graining_tiles_match_the_oracle(LG, O, w, h, bx, by):
    """Field::sample (src/gpu.rs:324-377) for block widths on either side of the
    tiled kernel's 16 columns, blocks that straddle words and tiles, narrow and tall
    blocks and a partial last block column, with obstacles: the block sums and the
    running average after two blended samples, bit for bit, through both the
    waiting call (sample_field) and the sampling steps (advance_sampling)."""
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w * 0.37, h * 0.5, h * 0.3)
    LG.add_box(cells, w, h, w * 0.7, w * 0.75, 0.0, h * 0.4, False)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.05, True, 91)
    want = O.Field(w, h, bx, by)
    want.sample(cells, w, h, np.float32(0.3))
    g = LG.GpuLattice(w, h, True, 3)
    g.attach_field(bx, by)
    g.load(cells)
    g.sample_field(0.3)
    o = O.BitplaneLattice(w, h, True, 3, THREADS)
    o.attach_field(bx, by)
    o.load(cells)
    g.advance_sampling(12, 5, 0.6)
    o.advance_sampling(12, 5, 0.6)
    assert_same(g, o, with_field=False)
    for x, y in zip(g.read_block_sums(), o.read_block_sums()):
        assert np.array_equal(x, y)
    h2 = LG.GpuLattice(w, h, True, 3)
    h2.attach_field(bx, by)
    h2.load(cells)
    h2.sample_field(0.3)
    h2.advance(7)
    cur = h2.store()
    want.sample(cur, w, h, np.float32(0.7))
    h2.sample_field(0.7)
    f = h2.read_field()
    for a, b in zip((want.ux, want.uy, want.rho, want.solid), (f.ux, f.uy, f.rho, f.solid)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    for a, b in zip(O.block_sums(cur, w, h, bx, by), h2.read_block_sums()):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("block,separate", [(20, 1), (8, 10)])
def test_sampling_points_ride_in_the_next_steps_grid(LG, O, block, separate):
    """With one launch per step, a sampling point that another step of the run
    follows is coarse-grained inside that step's grid (20-column blocks: only the
    run's last point launches on its own); 8-column blocks take a sampling launch
    at every point.  The field matches the oracle either way."""
    w, h = 256, 64
    cells = np.zeros(w * h, np.uint8)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.0, True, 7)
    g, o = pair(LG, O, w, h, True, 9, cells, block=block, mode=1)
    n0 = g.launches
    g.advance_sampling(50, 5, 0.3)
    o.advance_sampling(50, 5, 0.3)
    assert g.launches - n0 == 50 + separate
    assert_same(g, o)


def test_the_gpu_field_averages_over_time(LG, O):
    """src/gpu.rs:999-1032, bit-exact."""
    ALPHA = 0.2
    w, h, block = 192, 96, 16
    cpu = O.Lattice(w, h, 0.22, (0.3, 0.0), 4, True, 1, 0x5EED)
    cpu.init_equilibrium()
    want = O.Field(w, h, block, block)
    g = LG.GpuLattice(w, h, True, 1)
    g.attach_field(block, block)
    g.load(cpu.cells.copy())
    for _ in range(6):
        want.sample(cpu.cells, w, h, ALPHA)
        g.sample_field(ALPHA)
        cpu.advance(5)
        g.load(cpu.cells.copy())
    f = g.read_field()
    assert np.array_equal(want.ux, f.ux) and np.array_equal(want.rho, f.rho)


@pytest.mark.parametrize("w,h", [(256, 64), (100, 32), (129, 18)])
def test_the_gpu_counts_the_same_particles(LG, O, w, h):
    """src/gpu.rs:1036-1053."""
    cpu = O.Lattice(w, h, 0.3, (0.2, 0.0), 0, True, 1, 0x5EED)
    cpu.add_box(20.0, 30.0, 5.0, 15.0, strict=True)
    cpu.init_equilibrium()
    cpu.advance(20)
    g = LG.GpuLattice(w, h, True, 1)
    g.load(cpu.cells.copy())
    assert g.total_particles() == cpu.total_particles()


@pytest.mark.parametrize("cols", [8, 40])
def test_the_inlet_reseeds_at_the_requested_equilibrium(LG, O, cols):
    """src/gpu.rs:1058-1103."""
    w, h, steps = 128, 64, 60
    g = LG.GpuLattice(w, h, True, 0xC0FFEE)
    g.set_inlet(cols, 0.22, (0.4, 0.0), True)
    g.load(np.zeros(w * h, np.uint8))
    hits = np.zeros(7)
    n = 0
    for _ in range(steps):
        g.advance(1)
        c = g.store().reshape(h, w)[:, :cols]
        for d in range(7):
            hits[d] += ((c >> d) & 1).sum()
        n += c.size
    want = O.thresholds(0.22, 0.4, 0.0, True)
    for d in range(7):
        p = float(want[d]) / 2 ** 24
        assert abs(hits[d] / n - p) < 5 * (p * (1 - p) / n) ** 0.5


def test_the_inlet_does_not_seed_obstacles(LG):
    """src/gpu.rs:1109-1125."""
    w, h = 96, 32
    g = LG.GpuLattice(w, h, True, 5)
    g.set_inlet(w, 0.4, (0.3, 0.0), True)
    g.load(np.full(w * h, 0x80, np.uint8))
    g.advance(10)
    assert (g.store() == 0x80).all()


def test_the_inlet_leaves_the_rest_of_the_lattice_alone(LG):
    """src/gpu.rs:1129-1152."""
    w, h, cols = 128, 32, 8
    g = LG.GpuLattice(w, h, True, 9)
    g.set_inlet(cols, 0.4, (0.3, 0.0), True)
    g.load(np.zeros(w * h, np.uint8))
    g.advance(1)
    c = g.store().reshape(h, w)
    assert (c[:, cols:] == 0).all() and (c[:, :cols] != 0).sum() > h * cols / 2


def test_the_gpu_agrees_with_the_cpu_on_the_bulk_numbers(LG, O):
    """src/gpu.rs:1424-1451."""
    w, h = 256, 128
    cpu = O.Lattice(w, h, 0.22, (0.3, 0.0), 0, True, 4, 0x5EED)
    cpu.init_equilibrium()
    g = LG.GpuLattice(w, h, True, 0x5EED)
    g.load(cpu.cells.copy())
    cpu.advance(120)
    g.advance(120)
    gl = O.Lattice(w, h, 0.22, (0.3, 0.0), 0, True, 1, 1)
    gl.set_cells(g.store())
    (ax, ay), (bx, by) = cpu.mean_velocity(), gl.mean_velocity()
    assert abs(ax - bx) < 0.02 and abs(ay - by) < 0.02
    assert abs(cpu.total_particles() - gl.total_particles()) / cpu.total_particles() < 0.01


# ---- bit-exact against the oracle ----------------------------------------

def test_periodic_box_bit_exact(LG, O):
    """256x128 periodic FHP-III box, Bernoulli(0.25), 500 steps, 8x8 block sums."""
    from lattice_gas import workloads as W
    wl = W.periodic_box()
    g, o = pair(LG, O, wl.w, wl.h, True, wl.seed, wl.cells, block=8)
    before = O.invariants(wl.cells)
    g.advance_sampling(500, 100, 1.0)
    o.advance_sampling(500, 100, 1.0)
    assert_same(g, o)
    assert O.invariants(g.store()) == before
    mass, px, py, _ = g.read_block_sums()
    assert (int(mass.sum()), int(px.sum()), int(py.sum())) == before


MODES = [1, 2]   # one launch per step (programmatic dependent launch), persistent waves


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("w,h,inlet,rest", [
    (100, 34, 40, True),    # ragged width, two-word inlet
    (33, 20, 8, True),      # one valid bit in the last word
    (20, 16, 8, True),      # one word per row: both wraps hit the same word
    (64, 18, 0, False),     # no rest particles
    (129, 40, 70, False),   # no rest, three-word inlet, ragged
    (1000, 64, 8, True),    # many warps per row, rows straddling warps
])
def test_small_lattices_bit_exact(LG, O, w, h, inlet, rest, mode):
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w / 2.0, h * 0.43, min(w, h) / 5.0)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.0, rest, 1234 + w)
    g, o = pair(LG, O, w, h, rest, 0xDEADBEEF12345678 + w, cells,
                inlet=(inlet, 0.3, (0.2, 0.0), rest) if inlet else None, block=8, mode=mode)
    for chunk in (1, 7, 64, 100, 300):   # crosses inlet draw chunks and launch lengths
        g.advance_sampling(chunk, 10, 0.3)
        o.advance_sampling(chunk, 10, 0.3)
        assert_same(g, o)


SHAPES = [1, 2, 3, 4]   # chunk of one / two per warp, two / four consecutive words per lane


@pytest.mark.parametrize("block", [4, 20])  # a warp per field block; tiles, in the step's grid
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("w,h,inlet,rest", [
    (128, 34, 40, True),    # four words per row: one four-word group per row
    (250, 20, 8, True),     # eight words per row, 26 valid bits in the last
    (60, 16, 8, True),      # two words per row: both wraps inside one lane's pair
    (190, 24, 70, False),   # six words per row: pairs apply, fours fall back
    (1000, 40, 8, True),    # 32 words per row: a warp spans several rows
    (4000, 12, 40, False),  # 125 words per row: neither applies
])
def test_step_shapes_bit_exact(LG, O, w, h, inlet, rest, shape, block):
    """Every kernel shape, pinned, against the oracle: obstacles, inflows,
    ragged rows and both rules, across inlet chunks and sampling points (with
    20-column blocks a sampling point inside a run is coarse-grained by the next
    step's grid; 4 x 4 blocks take the sampling kernel)."""
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w / 2.0, h * 0.43, min(w, h) / 5.0)
    LG.add_box(cells, w, h, w // 5, w // 5 + 2, 0, h // 3)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.0, rest, 4321 + w)
    g, o = pair(LG, O, w, h, rest, 0xC0FFEE + w, cells,
                inlet=(inlet, 0.3, (0.2, 0.0), rest) if inlet else None, block=block, mode=1)
    g.set_step_shape(shape)
    for chunk in (1, 7, 64, 130):
        g.advance_sampling(chunk, 10, 0.3)
        o.advance_sampling(chunk, 10, 0.3)
        assert_same(g, o)


@pytest.mark.parametrize("shape", SHAPES)
def test_step_shapes_on_the_full_wake_run(LG, O, shape):
    """4096 x 2304 (128 words per row), 24 steps in each shape against the oracle."""
    from lattice_gas import workloads as W
    wl = W.wake_run()
    g, o = pair(LG, O, wl.w, wl.h, True, wl.seed, wl.cells,
                inlet=(wl.inlet_cols, wl.density, wl.inflow, True), block=wl.block, mode=1)
    g.set_step_shape(shape)
    g.advance_sampling(24, 12, wl.alpha)
    o.advance_sampling(24, 12, wl.alpha)
    assert_same(g, o)


def test_restart_resets_the_stream(LG, O):
    w, h = 96, 32
    cells = np.zeros(w * h, np.uint8)
    LG.init_equilibrium(cells, 0.3, 0.1, 0.0, True, 5)
    g, o = pair(LG, O, w, h, True, 1, cells, inlet=(8, 0.3, (0.1, 0.0), True))
    g.advance(37)
    o.advance(37)
    g.restart(cells, 99)
    o.restart(cells, 99)
    g.advance(20)
    o.advance(20)
    assert_same(g, o)


@pytest.mark.parametrize("mode", MODES)
def test_wake_run_reduced_bit_exact(LG, O, mode):
    """The wake run's geometry (plate, inflow, walls) at 512 x 288, 300 steps."""
    from lattice_gas import workloads as W
    wl = W.wake_run(w=512, h=288, steps=300)
    g, o = pair(LG, O, wl.w, wl.h, True, wl.seed, wl.cells,
                inlet=(wl.inlet_cols, wl.density, wl.inflow, True), block=wl.block, mode=mode)
    g.advance_sampling(300, wl.sample_every, wl.alpha)
    o.advance_sampling(300, wl.sample_every, wl.alpha)
    assert_same(g, o)


def test_wake_run_full_size_bit_exact(LG, O):
    """4096 x 2304, the full-size wake run, 40 steps against the oracle."""
    from lattice_gas import workloads as W
    wl = W.wake_run()
    g, o = pair(LG, O, wl.w, wl.h, True, wl.seed, wl.cells,
                inlet=(wl.inlet_cols, wl.density, wl.inflow, True), block=wl.block)
    g.advance_sampling(40, 20, wl.alpha)
    o.advance_sampling(40, 20, wl.alpha)
    assert_same(g, o)


def test_roofline_geometry_reduced_bit_exact(LG, O):
    """Circles + inflow (the roofline case's geometry) at 2048 x 1024, 30 steps."""
    from lattice_gas import workloads as W
    wl = W.roofline_case(w=2048, h=1024, n_circles=12)
    g, o = pair(LG, O, wl.w, wl.h, True, wl.seed, wl.cells,
                inlet=(wl.inlet_cols, wl.density, wl.inflow, True), block=32)
    g.advance_sampling(30, 10, 1.0)
    o.advance_sampling(30, 10, 1.0)
    assert_same(g, o)


def test_transport_sweep_members_bit_exact(LG, O):
    """Three lattices of the transport sweep (shear-wave starts), 200 steps."""
    from lattice_gas import workloads as W
    for wl in W.transport_sweep(n=3, wmax=600, hmax=400):
        g, o = pair(LG, O, wl.w, wl.h, True, wl.seed, wl.cells, block=wl.block)
        g.advance_sampling(200, wl.sample_every, wl.alpha)
        o.advance_sampling(200, wl.sample_every, wl.alpha)
        assert_same(g, o)


def test_step_modes_agree_on_the_full_wake_run(LG):
    """4096 x 2304, 1000 steps with sampling: persistent launches and one launch
    per step give the same lattice, field and block sums."""
    from lattice_gas import workloads as W
    wl = W.wake_run()
    out = []
    for mode in (1, 2):
        g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
        g.set_step_mode(mode)
        g.set_inlet(wl.inlet_cols, wl.density, wl.inflow, True)
        g.attach_field(wl.block, wl.block)
        g.load(wl.cells)
        g.advance_sampling(1000, wl.sample_every, wl.alpha)
        f = g.read_field()
        out.append((g.store(), g.read_block_sums(), f.ux.copy(), g.steps))
        g.close()
    assert np.array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)
    assert np.array_equal(out[0][2], out[1][2]) and out[0][3] == out[1][3] == 1000


def test_full_size_periodic_conservation(LG, O):
    """32768 x 16384 without inlet: mass and momentum exact after 20 steps (the
    roofline case's size; a size-independent invariant)."""
    w, h = 32768, 16384
    cells = np.zeros(w * h, np.uint8)
    LG.init_equilibrium(cells, 0.2, 0.0, 0.0, True, 77)
    before = O.invariants(cells)
    g = LG.GpuLattice(w, h, True, 77)
    g.attach_field(32, 32)
    g.load(cells)
    del cells
    g.advance_sampling(20, 20, 1.0)
    mass, px, py, _ = g.read_block_sums()
    assert (int(mass.sum(dtype=np.int64)), int(px.sum(dtype=np.int64)),
            int(py.sum(dtype=np.int64))) == before
    assert g.total_particles() == before[0]
