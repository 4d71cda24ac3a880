"""Batches: many uneven lattices advanced together must give, lattice by
lattice, exactly what advancing each alone gives (and what the oracle gives).
Every test here needs a GPU."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(LG, specs):
    """specs: (w, h, rest, inlet_cols, obstacle, block, seed)"""
    out = []
    for w, h, rest, inlet, obstacle, block, seed in specs:
        cells = np.zeros(w * h, np.uint8)
        if obstacle:
            LG.add_circle(cells, w, h, w / 3.0, h * 0.43, min(w, h) / 6.0)
        LG.init_equilibrium(cells, 0.3, 0.15, 0.0, rest, seed)
        out.append((w, h, rest, inlet, block, seed, cells))
    return out


def build(LG, spec):
    w, h, rest, inlet, block, seed, cells = spec
    g = LG.GpuLattice(w, h, rest, seed)
    if inlet:
        g.set_inlet(inlet, 0.3, (0.15, 0.0), rest)
    if block:
        g.attach_field(block, block)
    g.load(cells)
    return g


def snapshot(g):
    out = [g.store(), g.steps, g.total_particles()]
    if g._field is not None:
        out += g.read_block_sums()
        f = g.read_field()
        out += [f.ux.copy(), f.uy.copy(), f.rho.copy(), f.solid.copy()]
    return out


def same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        if isinstance(x, np.ndarray):
            assert np.array_equal(x.view(np.uint8), y.view(np.uint8))
        else:
            assert x == y


SPECS = [
    (256, 256, True, 0, False, 16, 11),
    (100, 34, True, 40, True, 8, 12),     # ragged, two-word inlet, obstacle
    (33, 20, True, 8, False, 0, 13),      # one-bit tail, no field
    (1000, 64, True, 8, True, 32, 14),
    (64, 18, False, 0, False, 8, 15),     # six-direction rule in the same batch
    (129, 40, False, 70, True, 16, 16),
    (2048, 1024, True, 0, False, 16, 17),
]


POLICIES = [0, 1, 2]  # LG.BATCH_AUTO, BATCH_PER_STEP, BATCH_RESIDENT


@pytest.mark.parametrize("policy", POLICIES)
@pytest.mark.parametrize("n,every", [(1, 0), (37, 0), (300, 50), (257, 100), (400, 500)])
def test_batch_equals_each_lattice_alone(LG, n, every, policy):
    specs = make(LG, SPECS)
    alone = [build(LG, s) for s in specs]
    for g in alone:
        g.advance_sampling(n, every, 0.4)
    together = [build(LG, s) for s in specs]
    b = LG.Batch(together, policy)
    b.advance_sampling(n, every, 0.4)
    for x, y in zip(alone, together):
        same(snapshot(x), snapshot(y))
    b.close()


WIDE_SPECS = [  # every lattice a multiple of 4 words per row; 2,560 blocks of 256 words
    (2048, 1280, True, 40, True, 32, 21),
    (2048, 1280, False, 8, False, 16, 22),   # six-direction rule: a mixed-rule launch
    (4096, 640, True, 8, True, 32, 23),
    (2048, 1280, True, 0, True, 0, 24),
    (2048, 1280, True, 70, False, 20, 25),
    (4096, 640, False, 0, True, 16, 26),
    (2048, 1280, True, 8, True, 32, 27),
    (2048, 1280, True, 0, False, 16, 28),
]


@pytest.mark.parametrize("inflows", [True, False])
@pytest.mark.parametrize("policy", [0, 1])
def test_wide_batch_of_four_word_rows_equals_alone(LG, policy, inflows):
    """Each launch chain covers at least a full wave of blocks and every row is a
    multiple of four words, so the batched step takes four words per lane: with
    inflows in the chains, and without any (the kernel compiled without them)."""
    wide = WIDE_SPECS if inflows else [(w, h, r, 0, o, b, s) for w, h, r, _, o, b, s in WIDE_SPECS]
    specs = make(LG, wide)
    alone = [build(LG, s) for s in specs]
    for g in alone:
        g.advance_sampling(130, 40, 0.4)
    together = [build(LG, s) for s in specs]
    b = LG.Batch(together, policy)
    b.advance_sampling(130, 40, 0.4)
    for x, y in zip(alone, together):
        same(snapshot(x), snapshot(y))
    b.close()


def test_resident_policy_plans_small_classes(LG):
    """Every class of up to 32768 words is listed; under BATCH_RESIDENT those with
    a usable cluster shape run resident, under BATCH_PER_STEP none does."""
    specs = make(LG, SPECS)
    lats = [build(LG, s) for s in specs]
    plan = LG.Batch(lats, LG.BATCH_RESIDENT).plan
    words = sorted({c["words"] for c in plan})
    assert words == sorted({max(64, 1 << (((w + 31) // 32 * h) - 1).bit_length())
                            for w, h, *_ in SPECS if (w + 31) // 32 * h <= 32768})
    assert all(c["resident"] == (c["cluster"] > 0) for c in plan)
    assert any(c["resident"] for c in plan)
    assert sum(c["lattices"] for c in plan) == sum(
        1 for w, h, *_ in SPECS if (w + 31) // 32 * h <= 32768)
    lats2 = [build(LG, s) for s in specs]
    assert not any(c["resident"] for c in LG.Batch(lats2, LG.BATCH_PER_STEP).plan)


@pytest.mark.parametrize("policy", POLICIES)
def test_batch_replays_and_continues(LG, policy):
    """Several calls (graph replays, mixed lengths), then a plain advance after
    the batch: still identical to the lattices run alone throughout."""
    specs = make(LG, SPECS[:4])
    alone = [build(LG, s) for s in specs]
    together = [build(LG, s) for s in specs]
    b = LG.Batch(together, policy)
    for n, every in ((100, 50), (100, 50), (33, 0), (150, 50)):
        for g in alone:
            g.advance_sampling(n, every, 1.0)
        b.advance_sampling(n, every, 1.0)
    b.close()
    for g in alone + together:
        g.advance(10)
    for x, y in zip(alone, together):
        same(snapshot(x), snapshot(y))


@pytest.mark.parametrize("policy", [1, 2])
def test_batch_matches_oracle(LG, O, policy):
    specs = make(LG, SPECS[:5])
    together = [build(LG, s) for s in specs]
    b = LG.Batch(together, policy)
    b.advance_sampling(120, 40, 0.5)
    for (w, h, rest, inlet, block, seed, cells), g in zip(specs, together):
        o = O.BitplaneLattice(w, h, rest, seed, 4)
        if inlet:
            o.set_inlet(inlet, 0.3, (0.15, 0.0), rest)
        if block:
            o.attach_field(block, block)
        o.load(cells)
        o.advance_sampling(120, 40, 0.5)
        assert np.array_equal(g.store(), o.store())
        if block:
            for x, y in zip(g.read_block_sums(), o.read_block_sums()):
                assert np.array_equal(x, y)


def test_transport_sweep_batch_equals_alone(LG):
    """The 64-lattice transport sweep (shear-wave starts, 16x16 blocks every 50
    steps), 200 steps: batch == each alone, under every policy."""
    from lattice_gas import workloads as W
    wls = W.transport_sweep()
    def mk(wl):
        g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
        g.attach_field(wl.block, wl.block)
        g.load(wl.cells)
        return g
    alone = [mk(wl) for wl in wls]
    for g in alone:
        g.advance_sampling(200, 50, 1.0)
    for policy in POLICIES:
        together = [mk(wl) for wl in wls]
        b = LG.Batch(together, policy)
        b.advance_sampling(200, 50, 1.0)
        for x, y in zip(alone, together):
            same(snapshot(x), snapshot(y))
        b.close()


def test_batch_rejects_bad_arguments(LG):
    g = LG.GpuLattice(64, 64, True, 1)
    with pytest.raises(LG.LgxError):
        LG.Batch([g, g])
    with pytest.raises(LG.LgxError):
        LG.Batch([])


_STEPS_CHILD = r'''
import os, sys
import numpy as np
sys.path.insert(0, os.path.join(sys.argv[1], "lattice-gas_gb300"))
import lattice_gas as LG
specs = [  # (w, h, rest, inlet, obstacle, block, seed)
    (256, 256, True, 0, True, 16, 41),
    (128, 128, True, 8, False, 8, 42),     # bands of 8 rows on 16 CTAs
    (100, 96, True, 40, True, 8, 43),      # ragged rows, two-word inflow
    (300, 64, False, 8, True, 16, 44),     # six-direction rule
    (1000, 64, True, 0, False, 0, 45),     # no field
    (64, 36, True, 8, False, 4, 46),       # short bands: fewer steps per barrier
]
def build(s):
    w, h, rest, inlet, obstacle, block, seed = s
    cells = np.zeros(w * h, np.uint8)
    if obstacle:
        LG.add_circle(cells, w, h, w / 3.0, h * 0.43, min(w, h) / 6.0)
    LG.init_equilibrium(cells, 0.3, 0.15, 0.0, rest, seed)
    g = LG.GpuLattice(w, h, rest, seed)
    if inlet:
        g.set_inlet(inlet, 0.3, (0.15, 0.0), rest)
    if block:
        g.attach_field(block, block)
    g.load(cells)
    return g
def snap(g):
    out = [g.store(), g.steps, g.total_particles()]
    if g._field is not None:
        out += list(g.read_block_sums())
        f = g.read_field()
        out += [f.ux.copy(), f.uy.copy(), f.rho.copy(), f.solid.copy()]
    return out
k = int(os.environ["LGX_RESIDENT_STEPS"])
fixed = os.environ["LGX_RESIDENT_FIXED"]
for n, every in ((37, 0), (300, 7), (257, 50)):
    alone = [build(s) for s in specs]
    for g in alone:
        g.set_step_mode(1)
        g.advance_sampling(n, every, 0.4)
    together = [build(s) for s in specs]
    b = LG.Batch(together, LG.BATCH_RESIDENT)
    multi = [c for c in b.plan if c["resident"] and c["cluster"] > 1 and c["steps_per_barrier"] > 1]
    assert multi or k == 1, b.plan
    assert all(c["steps_per_barrier"] <= k for c in b.plan), b.plan
    per_thread = [c for c in b.plan if c["resident"] and c["word_per_thread"]]
    if fixed == "0":
        assert not per_thread, b.plan
    else:
        assert per_thread, b.plan
        if k > 1:
            assert any(c["cluster"] > 1 for c in per_thread), b.plan
    summary = [(c["words"], c["cluster"], c["threads"], c["steps_per_barrier"],
                c["word_per_thread"]) for c in b.plan if c["resident"]]
    b.advance_sampling(n, every, 0.4)
    for s, x, y in zip(specs, alone, together):
        for u, v in zip(snap(x), snap(y)):
            if isinstance(u, np.ndarray):
                assert np.array_equal(u.view(np.uint8), v.view(np.uint8)), (s, n, every)
            else:
                assert u == v, (s, n, every, u, v)
    b.close()
print("steps per barrier", k, "fixed", fixed, "ok:", summary)
'''


@pytest.mark.parametrize("fixed", ["0", "2"])
@pytest.mark.parametrize("k", [1, 2, 4, 8])
def test_resident_steps_per_cluster_barrier_equal_alone(k, fixed):
    """The resident kernels with k steps between cluster barriers (halo rows
    recomputed): every lattice as each alone, across sampling points and short
    bands (where the batch takes fewer steps per barrier); on the kernels that
    keep each thread on one word of its band (fixed "2": the tuner times only
    shapes that take them) and on the others (fixed "0").  k = 1 covers the
    single-CTA shapes.  The tuner caches its plans per process, so each pinned
    setting runs in a child process."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, LGX_RESIDENT_STEPS=str(k), LGX_RESIDENT_FIXED=fixed)
    r = subprocess.run([sys.executable, "-c", _STEPS_CHILD, root], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "ok" in r.stdout


def test_small_lattices_take_the_one_word_per_thread_kernels(LG):
    """Under the tuner's own choice, a batch of 64 x 64 lattices and one 256 x 256
    lattice run resident on the kernels that keep each thread on one word of its
    band (about twice as fast as the others there, so the choice does not flip), and
    one lattice of 256 x 256 steps through its one-lattice batch."""
    lats = [LG.GpuLattice(64, 64, True, i) for i in range(8)]
    plan = LG.Batch(lats, LG.BATCH_AUTO).plan
    assert len(plan) == 1 and plan[0]["resident"] and plan[0]["word_per_thread"], plan
    one = LG.Batch([LG.GpuLattice(256, 256, True, 9)], LG.BATCH_AUTO).plan
    assert one[0]["resident"] and one[0]["word_per_thread"] and one[0]["cluster"] > 1, one
    g = LG.GpuLattice(256, 256, True, 10)
    g.advance(8)
    assert g.step_plan["mode"] == g.STEP_GRAPH, g.step_plan
