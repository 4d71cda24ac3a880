"""Field::vorticity and Field::mean_velocity (src/render.rs:127-161) on the device,
against the oracle's restatement applied to the same field, bit for bit (NaN where
the reference divides 0 by 0, a one-column block grid).  Needs a GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("w,h,bx,by", [(256, 128, 16, 16), (300, 96, 20, 8), (128, 64, 32, 32),
                                       (64, 40, 64, 10),
                                       (2048, 1280, 20, 20),   # 6528 blocks: four staged chunks, the last partial
                                       (4096, 2304, 8, 8)])    # 147,456 blocks
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
