"""The step-mode tuner behind LGX_STEP_AUTO: it reports a plan for every size class,
picks the fastest mode it timed, and a lattice stepped in AUTO equals the same lattice
stepped one launch per step.  Needs a GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("w,h", [(64, 64), (300, 96), (4096, 256), (190, 96)])
def test_auto_picks_the_fastest_timed_mode(LG, w, h):
    g = LG.GpuLattice(w, h, True, 3)
    p = g.step_plan
    wpr = (w + 31) // 32
    assert p["single1_us"] > 0 and p["single2_us"] > 0
    # the lane shapes are timed exactly where the words per row allow them
    assert (p["lanes2_us"] > 0) == (wpr % 2 == 0)
    assert (p["lanes4_us"] > 0) == (wpr % 4 == 0)
    shapes = {1: p["single1_us"], 2: p["single2_us"], 3: p["lanes2_us"], 4: p["lanes4_us"]}
    assert p["single_us"] == min(t for t in shapes.values() if t > 0)
    assert shapes[p["words"]] == p["single_us"]
    if (w + 31) // 32 >= 64:
        assert p["temporal4_us"] > 0 and p["temporal8_us"] > 0
    else:
        assert p["temporal4_us"] == 0 and p["temporal8_us"] == 0
    # the one-lattice batch is offered below one full wave of step blocks
    assert p["graph_us"] > 0
    chosen = {1: p["single_us"], 2: p["wave_us"],
              3: p["temporal4_us"] if p["depth"] == 4 else p["temporal8_us"],
              4: p["graph_us"]}[p["mode"]]
    others = min(t for t in (p["single_us"], p["wave_us"], p["temporal4_us"],
                             p["temporal8_us"]) if t > 0)
    if p["mode"] == 4:  # graph replays win ties within 5%
        assert chosen < 1.05 * others
    else:
        assert chosen == others and not (0 < p["graph_us"] < 1.05 * others)
    assert g.step_plan == p  # cached for the size class


@pytest.mark.parametrize("w,h,inlet", [(2048, 128, 8), (100, 40, 0)])
def test_auto_equals_single(LG, O, w, h, inlet):
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w / 3.0, h * 0.4, h / 6.0)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.0, True, 9)
    out = []
    for mode in (0, 1):
        g = LG.GpuLattice(w, h, True, 21)
        g.set_step_mode(mode)
        if inlet:
            g.set_inlet(inlet, 0.3, (0.2, 0.0), True)
        g.attach_field(16, 8)
        g.load(cells)
        g.advance_sampling(203, 50, 0.5)
        out.append((g.store(), g.read_block_sums()))
    assert np.array_equal(out[0][0], out[1][0])
    for x, y in zip(out[0][1], out[1][1]):
        assert np.array_equal(x, y)


def test_graph_is_not_offered_to_lattices_that_fill_the_gpu(LG):
    """4096 x 2304 (the wake run) is more than one wave of step blocks: no graph timing."""
    g = LG.GpuLattice(4096, 2304, True, 3)
    assert g.step_plan["graph_us"] == 0


def _run(LG, cells, w, h, rest, inlet, mode, script):
    g = LG.GpuLattice(w, h, rest, 21)
    g.set_step_mode(mode)
    if inlet:
        g.set_inlet(inlet, 0.3, (0.2, 0.0), rest)
    g.attach_field(16, 8)
    g.load(cells)
    for op, *args in script:
        if op == "adv":
            g.advance_sampling(*args)
        elif op == "mode":
            g.set_step_mode(mode if args[0] is None else args[0])
        elif op == "inlet":
            g.set_inlet(args[0], 0.25, (0.3, 0.0), rest)
        elif op == "field":
            g.attach_field(*args)
    return g.store(), g.read_block_sums(), g.total_particles(), g.steps, g.launches


@pytest.mark.parametrize("w,h,rest,inlet", [
    (2048, 1280, True, 8),   # the reference's production size
    (256, 256, True, 0),     # a resident-kernel class
    (300, 96, False, 40),    # ragged width, six-direction rule, two-word inlet
    (100, 40, True, 0),      # smaller than one step block
])
def test_graph_mode_equals_one_launch_per_step(LG, w, h, rest, inlet):
    """LGX_STEP_GRAPH (the lattice as a batch of one: captured graphs or the resident
    kernel) gives the same cells, block sums and particle count as one launch per
    step, with sampling every 20 (a graph per interval), runs shorter than the graph
    threshold, and sampling every 7 (too often for graphs: one launch per step)."""
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w / 3.0, h * 0.4, h / 6.0)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.0, rest, 9)
    script = [("adv", 157, 20, 0.5), ("adv", 5, 20, 0.5), ("adv", 64, 0, 0.0),
              ("adv", 30, 7, 0.5), ("adv", 41, 16, 0.25)]
    a = _run(LG, cells, w, h, rest, inlet, 4, script)
    b = _run(LG, cells, w, h, rest, inlet, 1, script)
    assert np.array_equal(a[0], b[0])
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)
    assert a[2:4] == b[2:4]
    assert a[4] > 0


def test_graph_mode_follows_reconfiguration(LG):
    """Switching modes, changing the inlet and re-attaching the field between graph
    runs (the one-lattice batch is rebuilt) matches one launch per step throughout."""
    w, h = 512, 200
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w / 4.0, h / 2.0, 20.0)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.0, True, 5)
    script = [("adv", 40, 16, 0.3), ("inlet", 12), ("adv", 33, 17, 0.3), ("mode", 1),
              ("adv", 9, 0, 0.0), ("mode", None), ("field", 8, 8), ("adv", 50, 25, 1.0)]
    a = _run(LG, cells, w, h, True, 6, 4, script)
    b = _run(LG, cells, w, h, True, 6, 1, [s if s[0] != "mode" else ("mode", 1) for s in script])
    assert np.array_equal(a[0], b[0])
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)
    assert a[2:4] == b[2:4]
