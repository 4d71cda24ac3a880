"""The oracle's Field::vorticity and Field::mean_velocity (src/render.rs:127-161)
against a numpy restatement in float32."""
import numpy as np

SQRT3_2 = np.float32(0.8660254)


def vorticity_numpy(ux, uy, bw, bh, bx, by):
    ux = ux.reshape(bh, bw)
    uy = uy.reshape(bh, bw)
    dx = np.float32(bx)
    dy = np.float32(by) * SQRT3_2
    out = np.zeros((bh, bw), np.float32)
    for j in range(bh):
        for i in range(bw):
            ip, im = min(i + 1, bw - 1), max(i - 1, 0)
            jp, jm = (j + 1) % bh, (j - 1) % bh
            with np.errstate(invalid="ignore", divide="ignore"):
                dvdx = (uy[j, ip] - uy[j, im]) / (np.float32(ip - im) * dx)
                dudy = (ux[jp, i] - ux[jm, i]) / (np.float32(2.0) * dy)
            out[j, i] = np.float32(dvdx - dudy)
    return out.reshape(-1)


def test_vorticity_and_mean_velocity(O):
    rng = np.random.default_rng(5)
    for bw, bh, bx, by in ((9, 6, 16, 8), (1, 4, 32, 32), (5, 1, 8, 8)):
        ux = rng.normal(0, 0.1, bw * bh).astype(np.float32)
        uy = rng.normal(0, 0.1, bw * bh).astype(np.float32)
        sol = rng.random(bw * bh).astype(np.float32)
        got = O.field_vorticity(ux, uy, bw, bh, bx, by)
        want = vorticity_numpy(ux, uy, bw, bh, bx, by)
        assert np.array_equal(np.isnan(got), np.isnan(want))
        ok = ~np.isnan(want)
        assert np.array_equal(got[ok], want[ok])
        mx, my = O.field_mean_velocity(ux, uy, sol)
        sx = sy = n = np.float32(0)
        for k in range(bw * bh):
            if sol[k] < np.float32(0.5):
                sx, sy, n = np.float32(sx + ux[k]), np.float32(sy + uy[k]), np.float32(n + 1)
        assert (mx, my) == ((sx / n, sy / n) if n else (0.0, 0.0))
