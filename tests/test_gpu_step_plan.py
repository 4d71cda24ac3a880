"""The step-mode tuner behind LGX_STEP_AUTO: it reports a plan for every size class,
picks the fastest mode it timed, and a lattice stepped in AUTO equals the same lattice
stepped one launch per step.  Needs a GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("w,h", [(64, 64), (300, 96), (4096, 256)])
def test_auto_picks_the_fastest_timed_mode(LG, w, h):
    g = LG.GpuLattice(w, h, True, 3)
    p = g.step_plan
    assert p["single1_us"] > 0 and p["single2_us"] > 0
    assert p["single_us"] == min(p["single1_us"], p["single2_us"])
    assert p["words"] == (1 if p["single_us"] == p["single1_us"] else 2)
    if (w + 31) // 32 >= 64:
        assert p["temporal4_us"] > 0 and p["temporal8_us"] > 0
    else:
        assert p["temporal4_us"] == 0 and p["temporal8_us"] == 0
    chosen = {1: p["single_us"], 2: p["wave_us"],
              3: p["temporal4_us"] if p["depth"] == 4 else p["temporal8_us"]}[p["mode"]]
    assert chosen == min(t for t in (p["single_us"], p["wave_us"], p["temporal4_us"],
                                     p["temporal8_us"]) if t > 0)
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
