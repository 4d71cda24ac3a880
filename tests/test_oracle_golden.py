"""The CPU oracle against the reference's golden vectors and unit tests.

Pins: tests/golden.rs:141-147 (five exact FNV-1a checksums of cells and
field, exact mass/momentum), tests/golden.rs:207-297 (behaviour, determinism,
thread-count invariance), src/collision.rs:127-151, src/moments.rs:147-211,
src/lattice.rs:396-559.
"""
import json
import os

import numpy as np
import pytest

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden_byte.json")))
DENSITY = np.float32(float(GOLD["constants"]["DENSITY"]))
SPEED = np.float32(float(GOLD["constants"]["SPEED"]))
SEED = int(GOLD["constants"]["SEED"], 16)
BLOCK = int(GOLD["constants"]["BLOCK"])


def build_case(O, c, seed=SEED):
    """tests/golden.rs:76-86."""
    lat = O.Lattice(c["w"], c["h"], DENSITY, (SPEED, 0.0), c["inlet"], c["rest"], c["threads"],
                    seed)
    if c["plate"]:
        yc = np.float32(c["h"]) * O.SQRT3_2 / np.float32(2.0)
        x0 = np.float32(c["w"]) / np.float32(5.0)
        x1 = x0 + np.float32(3.0)
        lat.add_box(x0, x1, yc - np.float32(12.0), yc + np.float32(12.0))
    lat.init_equilibrium()
    return lat


def run_case(O, c, seed=SEED):
    lat = build_case(O, c, seed)
    lat.advance(c["steps"])
    f = O.Field(c["w"], c["h"], BLOCK, BLOCK)
    f.sample(lat.cells, c["w"], c["h"], 1.0)
    return dict(cells=O.fnv1a(lat.cells), field=O.fnv1a(f.checksum_bytes()),
                inv=O.invariants(lat.cells), u=lat.mean_velocity())


@pytest.mark.parametrize("case", GOLD["cases"], ids=[c["name"] for c in GOLD["cases"]])
def test_golden_output_is_unchanged(O, case):
    g = GOLD["golden"][case["name"]]
    got = run_case(O, case)
    assert got["cells"] == int(g["cells"], 16)
    assert got["field"] == int(g["field"], 16)
    assert got["inv"] == (g["mass"], g["px"], g["py"])
    # printed with six decimals in the reference
    assert abs(got["u"][0] - g["ux"]) < 5e-7 and abs(got["u"][1] - g["uy"]) < 5e-7


def test_stepping_is_deterministic(O):
    for c in GOLD["cases"]:
        assert run_case(O, c) == run_case(O, c)


@pytest.mark.parametrize("rest", [False, True])
def test_thread_count_does_not_change_conserved_quantities(O, rest):
    expected = None
    for threads in (1, 2, 3, 5, 8):
        c = dict(w=64, h=64, rest=rest, inlet=0, plate=False, threads=threads, steps=100)
        lat = build_case(O, c)
        before = O.invariants(lat.cells)
        lat.advance(c["steps"])
        after = O.invariants(lat.cells)
        assert before == after
        if expected is None:
            expected = after
        assert expected == after


@pytest.mark.parametrize("rest", [False, True])
def test_collisions_conserve_mass_and_momentum(O, rest):
    L = O.lib()
    stride = L.lgo_table_stride(int(rest))
    assert stride == (30 if rest else 6)
    for s in range(128 if rest else 64):
        for k in range(stride):
            rand = ((k << 32) + (1 << 31)) // stride  # lands in slot k
            out = L.lgo_table_apply(int(rest), s, rand)
            assert O.invariants(np.array([s], np.uint8)) == O.invariants(np.array([out], np.uint8))


def test_groups_are_closed(O):
    L = O.lib()
    stride = L.lgo_table_stride(1)
    row = lambda s: {L.lgo_table_apply(1, s, ((k << 32) + (1 << 31)) // stride)
                     for k in range(stride)}
    for s in range(128):
        for out in row(s):
            assert s in row(out)


def test_class_census(O):
    for rest, n, nonsingle, states in ((True, 80, 28, 76), (False, 53, 9, 20)):
        cl = O.classes(rest)
        big = [c for c in cl if len(c) > 1]
        assert (len(cl), len(big), sum(map(len, big))) == (n, nonsingle, states)
        assert sorted(len(c) for c in big) == sorted([2] * 12 + [3] * 14 + [5] * 2
                                                     if rest else [2] * 7 + [3] * 2)


def test_moments_table_agrees_bit_by_bit(O):
    for s in range(256):
        c = np.array([s], np.uint8)
        out = np.zeros(4, np.int64)
        O.lib().lgo_moments_sum(O.ptr(c, O.C.c_uint8), 1, 0, O.ptr(out, O.C.c_int64))
        if s & 0x80:
            assert tuple(out[:3]) == (0, 0, 0) and out[3] == 1
        else:
            m = sum(1 for d in range(7) if s >> d & 1)
            px = sum(O.CX2[d] for d in range(6) if s >> d & 1)
            py = sum(O.CY2[d] for d in range(6) if s >> d & 1)
            assert tuple(out) == (m, px, py, 0)


def test_rng_known_sequence(O):
    # Rng::new(7) draws, first values: a self-consistency pin that the C restatement
    # matches a direct Python evaluation of src/rng.rs.
    M = 2 ** 64 - 1
    s = 7 ^ 0x9E3779B97F4A7C15
    s = ((s ^ (s >> 30)) * 0xBF58476D1CE4E5B9) & M
    s = ((s ^ (s >> 27)) * 0x94D049BB133111EB) & M
    s = (s ^ (s >> 31)) | 1
    want = []
    for _ in range(8):
        s ^= (s << 13) & M
        s ^= s >> 7
        s ^= (s << 17) & M
        want.append((s * 0x2545F4914F6CDD1D) & M)
    out = np.zeros(8, np.uint64)
    O.lib().lgo_rng_draws(7, O.ptr(out, O.C.c_uint64), 8)
    assert [int(v) for v in out] == want


def test_single_particle_travels_in_a_straight_line(O):
    """src/lattice.rs:408-439."""
    CXF = (1.0, 0.5, -0.5, -1.0, -0.5, 0.5)
    CYF = (0.0, 0.8660254, 0.8660254, 0.0, -0.8660254, -0.8660254)
    for d in range(6):
        for start_row in (10, 11):
            lat = O.Lattice(48, 48, 0.2, (0.0, 0.0), 0, False, 1, 1)
            x0, y0 = 24, start_row
            cells = np.zeros(48 * 48, np.uint8)
            cells[y0 * 48 + x0] = 1 << d
            lat.set_cells(cells)
            lat.advance(8)
            occ = np.nonzero(lat.cells & 0x7F)[0]
            assert len(occ) == 1 and lat.cells[occ[0]] == 1 << d
            x, y = occ[0] % 48, occ[0] // 48
            px, py = x + (0.5 if y & 1 else 0.0), y * 0.8660254
            sx, sy = x0 + (0.5 if y0 & 1 else 0.0), y0 * 0.8660254
            assert abs(px - (sx + 8 * CXF[d])) < 1e-3 and abs(py - (sy + 8 * CYF[d])) < 1e-3


def test_walls_reverse_particles(O):
    """src/lattice.rs:443-465."""
    lat = O.Lattice(48, 48, 0.2, (0.0, 0.0), 0, False, 1, 1)
    cells = np.zeros(48 * 48, np.uint8)
    x0, y0 = 20, 24
    cells[y0 * 48 + x0 + 3] = 0x80
    cells[y0 * 48 + x0] = 1
    lat.set_cells(cells)
    lat.advance(6)
    occ = np.nonzero(lat.cells & 0x7F)[0]
    assert len(occ) == 1 and (lat.cells[occ[0]] & 0x7F) == 1 << 3 and occ[0] == y0 * 48 + x0


def test_every_direction_hits_its_requested_rate(O):
    """src/lattice.rs:471-499."""
    N = 1_000_000
    CXF = np.array([1.0, 0.5, -0.5, -1.0, -0.5, 0.5], np.float32)
    CYF = np.array([0.0, 0.8660254, 0.8660254, 0.0, -0.8660254, -0.8660254], np.float32)
    for density, ux, uy in ((0.22, 0.3, 0.0), (0.5, 0.0, 0.2)):
        for rest in (False, True):
            bias = np.float32(2.0 * 7.0 / 6.0) if rest else np.float32(2.0)
            out = np.zeros(N, np.uint8)
            O.lib().lgo_equilibrium_samples(density, ux, uy, int(rest), 0xC0FFEE,
                                            O.ptr(out, O.C.c_uint8), N)
            for d in range(6):
                want = float(np.float32(density) * (np.float32(1.0) + bias * (
                    CXF[d] * np.float32(ux) + CYF[d] * np.float32(uy))))
                got = float(((out >> d) & 1).mean())
                sigma = (want * (1 - want) / N) ** 0.5
                assert abs(got - want) < 5 * sigma


def test_paired_directions_are_uncorrelated(O):
    """src/lattice.rs:503-531."""
    N = 1_000_000
    out = np.zeros(N, np.uint8)
    O.lib().lgo_equilibrium_samples(0.5, 0.0, 0.0, 0, 0xBEEF, O.ptr(out, O.C.c_uint8), N)
    bits = np.stack([(out >> d) & 1 for d in range(6)]).astype(np.float64)
    for a in range(6):
        for b in range(a + 1, 6):
            pa, pb = bits[a].mean(), bits[b].mean()
            pab = (bits[a] * bits[b]).mean()
            corr = (pab - pa * pb) / ((pa * (1 - pa)) ** 0.5 * (pb * (1 - pb)) ** 0.5)
            assert abs(corr) < 0.01


@pytest.mark.parametrize("rest", [False, True])
def test_periodic_box_conserves(O, rest):
    """src/lattice.rs:387-404 (a 32x32 box of random bytes, 200 steps)."""
    lat = O.Lattice(32, 32, 0.2, (0.0, 0.0), 0, rest, 1, 12345)
    draws = np.zeros(32 * 32, np.uint64)
    O.lib().lgo_rng_draws(7, O.ptr(draws, O.C.c_uint64), draws.size)
    mask = 0x7F if rest else 0x3F
    lat.set_cells(((draws >> np.uint64(32)).astype(np.uint32) & 0xFF).astype(np.uint8) & mask)
    before = O.invariants(lat.cells)
    lat.advance(200)
    assert O.invariants(lat.cells) == before
