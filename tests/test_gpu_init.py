"""Lattice::init_equilibrium on the device (lgx_init_equilibrium, lgx_byte_init_equilibrium):
bit-identical to the oracle's host fill (src/lattice.rs:197-208) on ragged and large
lattices, with and without obstacles and rest particles, and through the reference's
golden runs (tests/golden.rs) with the fill done on the device.  Needs a GPU."""
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


def obstacles(LG, w, h, kind, seed=7):
    """Solid cells (and junk particle bits the fill must overwrite)."""
    rng = np.random.default_rng(seed)
    cells = rng.integers(0, 128, w * h, dtype=np.uint8)  # particles, no solid bit
    if kind == "circle":
        LG.add_circle(cells, w, h, w / 3.0, h * 0.43, min(w, h) / 5.0)
    elif kind == "random":
        cells[rng.random(w * h) < 0.3] |= 0x80
    elif kind == "rows":  # whole solid rows: segments with no fluid at all
        cells.reshape(h, w)[: h // 4] |= 0x80
        cells.reshape(h, w)[-3:] = 0x80
    return cells


CASES = [
    (64, 32, True, "none"),
    (100, 38, True, "circle"),       # ragged last word
    (33, 10, False, "random"),       # one valid bit in the last word
    (257, 130, True, "rows"),
    (1000, 602, False, "circle"),
    (4096, 2048, True, "random"),    # draw indices past 2^24
]


@pytest.mark.parametrize("w,h,rest,kind", CASES)
def test_bitplane_fill_matches_the_oracle(LG, O, w, h, rest, kind):
    cells = obstacles(LG, w, h, kind)
    seed = 0xC0FFEE ^ w
    want = O.init_equilibrium_cells(cells, 0.31, 0.17, -0.05, rest, seed)
    g = LG.GpuLattice(w, h, rest, 99)
    g.load(cells)
    g.init_equilibrium(0.31, (0.17, -0.05), seed)
    got = g.store()
    np.testing.assert_array_equal(got, want)
    assert g.steps == 0


@pytest.mark.parametrize("w,h,rest,kind", CASES[:5])
def test_byte_fill_matches_the_oracle(LG, O, w, h, rest, kind):
    cells = obstacles(LG, w, h, kind)
    seed = 0x5EED + h
    want = O.init_equilibrium_cells(cells, 0.22, 0.3, 0.0, rest, seed)
    lat = LG.Lattice(w, h, 0.22, (0.3, 0.0), 0, rest, 4, seed)
    lat.load(cells)
    lat.init_equilibrium()
    np.testing.assert_array_equal(lat.store(), want)


def test_large_fill_matches_the_oracle(LG, O):
    """8192 x 8192 cells: draw indices near 2^28, 8 words per thread over 2M words."""
    w = h = 8192
    cells = obstacles(LG, w, h, "circle")
    want = O.init_equilibrium_cells(cells, 0.3, 0.2, 0.0, True, 1234)
    g = LG.GpuLattice(w, h, True, 5)
    g.load(cells)
    g.init_equilibrium(0.3, (0.2, 0.0), 1234)
    got = g.store()
    assert O.fnv1a(got) == O.fnv1a(want)


@pytest.mark.parametrize("case", GOLD["cases"], ids=[c["name"] for c in GOLD["cases"]])
def test_golden_runs_with_the_fill_on_the_device(LG, O, case):
    """tests/golden.rs:76-86, except that init_equilibrium runs on the device."""
    g = GOLD["golden"][case["name"]]
    w, h = case["w"], case["h"]
    cells = np.zeros(w * h, np.uint8)
    if case["plate"]:
        yc = np.float32(h) * LG.SQRT3_2 / np.float32(2.0)
        x0 = np.float32(w) / np.float32(5.0)
        LG.add_box(cells, w, h, x0, x0 + np.float32(3.0), yc - np.float32(12.0),
                   yc + np.float32(12.0))
    lat = LG.Lattice(w, h, DENSITY, (SPEED, 0.0), case["inlet"], case["rest"], case["threads"],
                     SEED)
    lat.load(cells)
    lat.init_equilibrium()
    lat.advance(case["steps"])
    out = lat.store()
    assert O.fnv1a(out) == int(g["cells"], 16)
    assert O.invariants(out) == (g["mass"], g["px"], g["py"])
