"""The bitplane oracle against the reference's Metal-path tests (src/gpu.rs:773-1451).

The oracle restates lgca_step / lgca_sample / lgca_count and GpuLattice's host
side; these pin it the way the reference pins its shader: the exhaustive rule
check, straight-line flight, walls, conservation, round trips, coarse-graining
against the CPU's Field::sample, the particle count, and the inlet's statistics.
"""
import numpy as np
import pytest

DX_EVEN = (1, 0, -1, -1, -1, 0)
DX_ODD = (1, 1, 0, -1, 0, 1)
DY = (0, 1, 1, 0, -1, -1)


def rng_bytes(O, seed, n):
    d = np.zeros(n, np.uint64)
    O.lib().lgo_rng_draws(seed, O.ptr(d, O.C.c_uint64), n)
    return ((d >> np.uint64(32)) & np.uint64(0xFF)).astype(np.uint8)


@pytest.mark.parametrize("rest", [True, False])
def test_lane_rule_matches_enumeration_rule(O, rest):
    """Two independent statements of the KAT (gpu.rs:799-817) agree."""
    import collide_gen as G
    L = O.lib()
    for state in range(128 if rest else 64):
        for two in (0, 1):
            for three in range(4):
                for five in range(6):
                    assert L.lgo_collide_lane(int(rest), state, two, three, five) == \
                        G.rule(rest, state, two, three, five)


@pytest.mark.parametrize("w", [64, 80])
def test_a_single_particle_travels_in_a_straight_line(O, w):
    """gpu.rs:826-863 on the oracle."""
    h, steps = 48, 8
    for d in range(6):
        for start_row in (10, 11):
            g = O.BitplaneLattice(w, h, True, 1)
            cells = np.zeros(w * h, np.uint8)
            x0, y0 = 24, start_row
            cells[y0 * w + x0] = 1 << d
            g.load(cells)
            g.advance(steps)
            out = g.store()
            live = np.nonzero(out & 0x7F)[0]
            assert len(live) == 1 and out[live[0]] == 1 << d
            x, y = x0, y0
            for _ in range(steps):
                dx = DX_ODD[d] if y & 1 else DX_EVEN[d]
                x = (x + dx) % w
                y = (y + DY[d]) % h
            assert live[0] == y * w + x


def test_walls_reverse_particles(O):
    """gpu.rs:867-885."""
    w, h = 64, 48
    g = O.BitplaneLattice(w, h, True, 1)
    cells = np.zeros(w * h, np.uint8)
    x0, y0 = 20, 24
    cells[y0 * w + x0 + 3] = 0x80
    cells[y0 * w + x0] = 1
    g.load(cells)
    g.advance(6)
    out = g.store()
    live = np.nonzero(out & 0x7F)[0]
    assert len(live) == 1 and out[live[0]] & 0x7F == 1 << 3 and live[0] == y0 * w + x0


@pytest.mark.parametrize("rest", [True, False])
def test_a_periodic_box_conserves_mass_and_momentum(O, rest):
    """gpu.rs:889-924."""
    w, h = 128, 64
    g = O.BitplaneLattice(w, h, rest, 0xC0FFEE)
    cells = rng_bytes(O, 7, w * h) & (0x7F if rest else 0x3F)
    before = O.invariants(cells)
    g.load(cells)
    g.advance(250)
    assert O.invariants(g.store()) == before


@pytest.mark.parametrize("w", [64, 100])
def test_load_and_store_round_trip(O, w):
    """gpu.rs:929-948."""
    h = 16
    g = O.BitplaneLattice(w, h, True, 1)
    b = rng_bytes(O, 11, w * h)
    want = np.where(b & 0x80, 0x80, b & 0x7F).astype(np.uint8)
    g.load(want)
    assert np.array_equal(g.store(), want)


@pytest.mark.parametrize("w,h,block", [(256, 128, 20), (200, 96, 16)])
def test_coarse_grain_matches_field_sample_exactly(O, w, h, block):
    """gpu.rs:955-994, tightened from 1e-5 to bit equality (same integer sums,
    same f32 formula)."""
    cpu = O.Lattice(w, h, 0.22, (0.3, 0.0), 0, True, 4, 0x5EED)
    yc = np.float32(h) * O.SQRT3_2 / np.float32(2.0)
    cpu.add_circle(np.float32(60.0), yc, np.float32(18.0))
    cpu.init_equilibrium()
    cpu.advance(30)
    want = O.Field(w, h, block, block)
    want.sample(cpu.cells, w, h, 1.0)
    g = O.BitplaneLattice(w, h, True, 1)
    g.attach_field(block, block)
    g.load(cpu.cells)
    g.sample_field(1.0)
    got = g.read_field()
    for a, b in zip((want.ux, want.uy, want.rho, want.solid), got):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    sums = g.read_block_sums()
    ref = O.block_sums(cpu.cells, w, h, block, block)
    for a, b in zip(ref, sums):
        assert np.array_equal(a, b)


def test_the_field_averages_over_time(O):
    """gpu.rs:999-1032, exact."""
    ALPHA = 0.2
    w, h, block = 192, 96, 16
    cpu = O.Lattice(w, h, 0.22, (0.3, 0.0), 4, True, 1, 0x5EED)
    cpu.init_equilibrium()
    want = O.Field(w, h, block, block)
    g = O.BitplaneLattice(w, h, True, 1)
    g.attach_field(block, block)
    g.load(cpu.cells)
    for _ in range(6):
        want.sample(cpu.cells, w, h, ALPHA)
        g.sample_field(ALPHA)
        cpu.advance(5)
        g.load(cpu.cells)
    got = g.read_field()
    assert np.array_equal(want.ux, got[0]) and np.array_equal(want.rho, got[2])


@pytest.mark.parametrize("w,h", [(256, 64), (100, 32), (129, 18)])
def test_counts_the_same_particles(O, w, h):
    """gpu.rs:1036-1053."""
    cpu = O.Lattice(w, h, 0.3, (0.2, 0.0), 0, True, 1, 0x5EED)
    cpu.add_box(20.0, 30.0, 5.0, 15.0, strict=True)
    cpu.init_equilibrium()
    cpu.advance(20)
    g = O.BitplaneLattice(w, h, True, 1)
    g.load(cpu.cells)
    assert g.total_particles() == cpu.total_particles()


@pytest.mark.parametrize("cols", [8, 40])
def test_the_inlet_reseeds_at_the_requested_equilibrium(O, cols):
    """gpu.rs:1058-1103."""
    DENSITY, SPEED = 0.22, 0.4
    w, h, steps = 128, 64, 60
    g = O.BitplaneLattice(w, h, True, 0xC0FFEE)
    g.set_inlet(cols, DENSITY, (SPEED, 0.0), True)
    g.load(np.zeros(w * h, np.uint8))
    hits = np.zeros(7)
    n = 0
    for _ in range(steps):
        g.advance(1)
        c = g.store().reshape(h, w)[:, :cols]
        for d in range(7):
            hits[d] += ((c >> d) & 1).sum()
        n += c.size
    want = O.thresholds(DENSITY, SPEED, 0.0, True)
    for d in range(7):
        p = float(want[d]) / 2 ** 24
        sigma = (p * (1 - p) / n) ** 0.5
        assert abs(hits[d] / n - p) < 5 * sigma


def test_the_inlet_does_not_seed_obstacles(O):
    """gpu.rs:1109-1125."""
    w, h = 96, 32
    g = O.BitplaneLattice(w, h, True, 5)
    g.set_inlet(w, 0.4, (0.3, 0.0), True)
    g.load(np.full(w * h, 0x80, np.uint8))
    g.advance(10)
    assert (g.store() == 0x80).all()


def test_the_inlet_leaves_the_rest_of_the_lattice_alone(O):
    """gpu.rs:1129-1152."""
    w, h, cols = 128, 32, 8
    g = O.BitplaneLattice(w, h, True, 9)
    g.set_inlet(cols, 0.4, (0.3, 0.0), True)
    g.load(np.zeros(w * h, np.uint8))
    g.advance(1)
    c = g.store().reshape(h, w)
    assert (c[:, cols:] == 0).all()
    assert (c[:, :cols] != 0).sum() > h * cols / 2


def test_agrees_with_the_cpu_on_the_bulk_numbers(O):
    """gpu.rs:1424-1451."""
    w, h = 256, 128
    cpu = O.Lattice(w, h, 0.22, (0.3, 0.0), 0, True, 4, 0x5EED)
    cpu.init_equilibrium()
    g = O.BitplaneLattice(w, h, True, 0x5EED)
    g.load(cpu.cells.copy())
    cpu.advance(120)
    g.advance(120)
    gl = O.Lattice(w, h, 0.22, (0.3, 0.0), 0, True, 1, 1)
    gl.set_cells(g.store())
    (ax, ay), (bx, by) = cpu.mean_velocity(), gl.mean_velocity()
    assert abs(ax - bx) < 0.02 and abs(ay - by) < 0.02
    ma, mb = cpu.total_particles(), gl.total_particles()
    assert abs(ma - mb) / ma < 0.01


def test_step_parameters(O):
    """GpuLattice::params (gpu.rs:547-568) for a ragged width and a two-word inlet."""
    P = np.zeros(18, np.uint32)
    th = np.arange(7, dtype=np.uint32) + 100
    O.lib().lgo_bp_params(100, 32, 0x1234_5678_9ABC_DEF0, 7, 40, O.ptr(th, O.C.c_uint32),
                          O.ptr(P, O.C.c_uint32))
    seed32 = (0x1234_5678_9ABC_DEF0 ^ (7 * 0x9E3779B97F4A7C15)) & 0xFFFFFFFF
    assert list(P[:11]) == [4, 32, seed32, 3, 3, 0xF, 128, 2, 40, 64, 2]
    assert list(P[11:]) == list(th)


@pytest.mark.parametrize("y0,y1", [(20, 44), (0, 16), (50, 64)])
def test_a_window_stepped_alone_equals_the_whole_lattice(O, y0, y1):
    """The windowed advance (the check of a band of a lattice too large to step whole
    on the host) leaves the band exactly as full steps do, including bands that
    touch the periodic edge rows, with an obstacle, an inflow and a continued step
    count."""
    w, h, n = 200, 64, 12
    cells = O.init_equilibrium_cells(np.zeros(w * h, np.uint8), 0.3, 0.2, 0.0, True, 5)
    O.lib().lgo_add_circle(O.ptr(cells, O.C.c_uint8), w, h, 90.0, 30.0, 9.0)
    full = O.BitplaneLattice(w, h, True, 0xABCDEF, 3)
    part = O.BitplaneLattice(w, h, True, 0xABCDEF, 3)
    for g in (full, part):
        g.set_inlet(40, 0.3, (0.2, 0.0), True)
        g.load(cells)
        g.set_steps(17)
    full.advance(n)
    part.advance_window(n, y0, y1)
    assert full.steps == part.steps == 17 + n
    assert np.array_equal(full.store()[y0 * w:y1 * w], part.store_rows(y0, y1))
    assert not np.array_equal(full.store(), part.store())   # the rest went stale
