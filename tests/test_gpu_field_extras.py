"""Field::vorticity and Field::mean_velocity (src/render.rs:127-161) on the device,
against the oracle's restatement applied to the same field, bit for bit (NaN where
the reference divides 0 by 0, a one-column block grid).  Needs a GPU."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("w,h,bx,by", [(256, 128, 16, 16), (300, 96, 20, 8), (128, 64, 32, 32),
                                       (64, 40, 64, 10),
                                       (2048, 1280, 20, 20),   # 6528 blocks: 13 segments of 512
                                       (2048, 1024, 8, 8),     # 32,768 blocks: 16 of 2048
                                       (4096, 2304, 16, 16),   # 36,864 blocks: 16 of 2304
                                       (4096, 2304, 8, 8)])    # 147,456: the single-chain kernel
def test_vorticity_and_mean_velocity_match_the_oracle(LG, O, w, h, bx, by):
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w / 3.0, h * 0.43, h / 5.0)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.05, True, 77)
    g = LG.GpuLattice(w, h, True, 5)
    g.set_inlet(8, 0.3, (0.2, 0.0), True)
    g.attach_field(bx, by)
    g.load(cells)
    g.advance_sampling(150, 30, 0.5)
    f = g.read_field()
    bw, bh = w // bx, h // by
    want = O.field_vorticity(f.ux, f.uy, bw, bh, bx, by)
    got = g.vorticity()
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.array_equal(got[ok].view(np.uint32), want[ok].view(np.uint32))
    mx, my = g.mean_velocity()
    wx, wy = O.field_mean_velocity(f.ux, f.uy, f.solid)
    assert np.float32(mx).view(np.uint32) == np.float32(wx).view(np.uint32)
    assert np.float32(my).view(np.uint32) == np.float32(wy).view(np.uint32)
    vort2, (mx2, my2) = g.field_analyses()      # both in one launch
    assert np.array_equal(vort2.view(np.uint32), got.view(np.uint32))
    assert (np.float32(mx2).view(np.uint32), np.float32(my2).view(np.uint32)) == (
        np.float32(mx).view(np.uint32), np.float32(my).view(np.uint32))


def test_field_analyses_refuse_bad_requests(LG):
    import ctypes as C
    g = LG.GpuLattice(64, 32, True, 1)
    L = LG.lib()
    fx, fy = C.c_float(), C.c_float()
    out = np.zeros(8, np.float32)               # the 4 x 2 blocks of a 16 x 16 field
    p = out.ctypes.data_as(C.POINTER(C.c_float))
    assert L.lgx_field_analyses(g.handle, p, 8, C.byref(fx), C.byref(fy)) == 4   # no field
    g.attach_field(16, 16)
    assert L.lgx_field_analyses(g.handle, p, 3, C.byref(fx), C.byref(fy)) == 1   # wrong count
    assert L.lgx_field_analyses(g.handle, None, 0, None, None) == 1               # nothing asked
    assert L.lgx_field_analyses(g.handle, None, 0, C.byref(fx), None) == 1        # half asked
    assert L.lgx_field_analyses(g.handle, p, 8, None, None) == 0                  # vorticity only
    assert L.lgx_field_analyses(g.handle, None, 0, C.byref(fx), C.byref(fy)) == 0
    assert (fx.value, fy.value) == (0.0, 0.0)     # an empty lattice: no particles, zero field


_SPEC_CHILD = r'''
import os, sys
import numpy as np
root = sys.argv[1]
sys.path.insert(0, os.path.join(root, "lattice-gas_gb300"))
sys.path.insert(0, os.path.join(root, "oracle"))
import lattice_gas as LG
import oracle as O
cases = [(2048, 1280, 20, 20, 0.2, 0.0), (2048, 1280, 20, 20, 0.0, 0.0), (1024, 512, 8, 8, 0.05, -0.03),
         (600, 300, 4, 4, 0.0, 0.1)]
for w, h, bx, by, ux, uy in cases:
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, w / 3.0, h * 0.43, h / 5.0)
    LG.init_equilibrium(cells, 0.3, ux, uy, True, 91)
    g = LG.GpuLattice(w, h, True, 6)
    g.attach_field(bx, by)
    g.load(cells)
    g.advance_sampling(60, 20, 0.5)
    f = g.read_field()
    for _ in range(3):
        mx, my = g.mean_velocity()
        wx, wy = O.field_mean_velocity(f.ux, f.uy, f.solid)
        assert np.float32(mx).view(np.uint32) == np.float32(wx).view(np.uint32), (w, h, mx, wx)
        assert np.float32(my).view(np.uint32) == np.float32(wy).view(np.uint32), (w, h, my, wy)
    g.close()
print("ok")
'''


@pytest.mark.parametrize("mode", ["0", "2"])
def test_mean_velocity_segments_summed_in_order_equal_the_oracle(mode):
    """The segmented mean velocity with its guess tables ignored (mode "0": every
    segment summed in order from the exact partial sum) or taken for even
    segments only ("2": misses and hits alternate), on fields whose mean is zero
    in one or both components (partial sums near zero, where guesses miss most):
    bit-equal to the oracle, three calls each (the block counter returns to zero
    between launches).  The mode is read once per process, so each runs in a
    child process."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, LGX_MEAN_SPECULATE=mode)
    r = subprocess.run([sys.executable, "-c", _SPEC_CHILD, root], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "ok" in r.stdout
