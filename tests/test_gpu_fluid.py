"""The reference's acceptance tests of the bitplane stream as a fluid, restated
against the engine (src/gpu.rs:1154-1419).

The bitplane step draws a counter-based random stream that no recorded output
of the reference pins; the reference accepts it because it is the *same fluid*
as the golden-pinned byte-per-cell CPU path.  Two transport coefficients are
measured the same way on both paths from identical starting cells, averaged
over 16 realisations before the fit:

* viscosity: a transverse shear wave in a periodic 256 x 256 box decays as
  exp(-nu k^2 t); the log amplitude's slope gives nu.  |dnu| / nu < 12%
  (src/gpu.rs:1176-1281).
* advection factor: a wave riding on a uniform stream U0 = 0.25 drifts at g U0;
  the unwrapped phase's slope gives g.  |dg| / g < 3% (src/gpu.rs:1304-1419).

The bitplane arm is the engine through the C ABI (lgx_create, lgx_load,
lgx_advance, and the profiles lgx_row_ux / lgx_column_uy formed on the device).
The CPU arm is the oracle's byte-per-cell Lattice (src/lattice.rs, 4 thread
bands as the reference's test), whose stream the reference's golden checksums
pin.  The CPU arm runs the 16 realisations four at a time on host threads
(about 10 s of host time for both tests on 16 cores).
"""
import concurrent.futures as cf
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F = np.float32
SQRT3_2 = F(0.8660254)
SIZE = 256
DENSITY = F(0.22)
TRANSIENT = 200
SAMPLES = 20
REPS = 16
AMP = F(0.05)
M64 = 2 ** 64 - 1


def _rep_bits(rep):
    """rep.wrapping_mul(0x9E37_79B9) << 20 in u64 (src/gpu.rs:1220, 1359)."""
    return (((rep * 0x9E3779B9) & M64) << 20) & M64


def _fit_slope(pts):
    n = float(len(pts))
    sx = sum(p[0] for p in pts)
    sy = sum(p[1] for p in pts)
    sxx = sum(p[0] * p[0] for p in pts)
    sxy = sum(p[0] * p[1] for p in pts)
    return (n * sxy - sx * sy) / (n * sxx - sx * sx)


def _project(u, phase):
    """Mode amplitude (a, b) of a profile u against cos/sin of an f32 phase, the
    products in f32 and the sums in f64 (src/gpu.rs:1206-1217, 1340-1350)."""
    a = float(np.sum((u * np.cos(phase)).astype(np.float64)))
    b = float(np.sum((u * np.sin(phase)).astype(np.float64)))
    return 2.0 * a / u.size, 2.0 * b / u.size


def _run_cpu(O, start, seed, inflow, interval, profile, phase, restart):
    """One realisation on the oracle's byte path: TRANSIENT steps, then SAMPLES
    profiles INTERVAL steps apart."""
    cpu = O.Lattice(SIZE, SIZE, DENSITY, inflow, 0, True, 4, seed)
    if restart:
        cpu.restart(start, seed)
    else:
        cpu.set_cells(start)
    cpu.advance(TRANSIENT)
    trace = []
    for _ in range(SAMPLES):
        trace.append(_project(profile(cpu.cells.copy()), phase))
        cpu.advance(interval)
    return trace


def _run_engine(LG, start, seed, interval, profile, phase):
    g = LG.GpuLattice(SIZE, SIZE, True, seed)
    g.load(start)
    g.advance(TRANSIENT)
    trace = []
    for _ in range(SAMPLES):
        trace.append(_project(profile(g), phase))
        g.advance(interval)
    g.close()
    return trace


def _average(traces):
    out = [(0.0, 0.0)] * SAMPLES
    for t in traces:
        out = [(x + a / REPS, y + b / REPS) for (x, y), (a, b) in zip(out, t)]
    return out


def _both_arms(LG, O, starts, seeds, inflow, interval, cpu_profile, gpu_profile, phase,
               restart):
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        futs = [ex.submit(_run_cpu, O, starts[r], seeds[r], inflow, interval, cpu_profile,
                          phase, restart) for r in range(REPS)]
        gpu = [_run_engine(LG, starts[r], seeds[r], interval, gpu_profile, phase)
               for r in range(REPS)]
        cpu = [f.result() for f in futs]
    return _average(cpu), _average(gpu)


def test_the_gpu_fluid_has_the_same_viscosity(LG, O):
    """src/gpu.rs:1176-1281: 256^2, density 0.22, transient 200, 20 samples 250
    steps apart, 16 realisations; nu within 12% of the CPU path's."""
    interval = 250
    h = SIZE
    k = F(2.0) * F(math.pi) / (F(h) * SQRT3_2)
    phase = (k * np.arange(h, dtype=F) * SQRT3_2).astype(F)
    ux_row = (AMP * np.sin(phase)).astype(F)
    starts, seeds = [], []
    for rep in range(REPS):
        s = 0x5EED ^ _rep_bits(rep)
        starts.append(O.shear_wave_cells(SIZE, SIZE, DENSITY, ux_row, True, s ^ 0xBEEF))
        seeds.append(0x5EED ^ (rep << 20))
    cpu, gpu = _both_arms(LG, O, starts, seeds, (0.0, 0.0), interval,
                          lambda c: O.row_ux(c, SIZE, SIZE), lambda g: g.row_ux(), phase,
                          restart=False)

    def fit(trace):
        pts = [(float(i * interval), math.log(max(math.sqrt(a * a + b * b), 1e-12)))
               for i, (a, b) in enumerate(trace)]
        return -_fit_slope(pts) / float(k * k)

    nu_cpu, nu_gpu = fit(cpu), fit(gpu)
    rel = abs(nu_gpu - nu_cpu) / nu_cpu
    print("viscosity: cpu nu = %.4f, gpu nu = %.4f (%.1f%% apart)" % (nu_cpu, nu_gpu,
                                                                       100 * rel))
    assert rel < 0.12, "the GPU is a different fluid: nu = %.4f against the CPU's %.4f" % (
        nu_gpu, nu_cpu)


def test_the_gpu_fluid_has_the_same_advection_factor(LG, O):
    """src/gpu.rs:1304-1419: 256^2, density 0.22, U0 = 0.25, transient 200, 20
    samples 100 steps apart, 16 realisations; g within 3% of the CPU path's."""
    interval = 100
    u0 = F(0.25)
    w = SIZE
    k = F(2.0) * F(math.pi) / F(w)
    phase = (k * np.arange(w, dtype=F)).astype(F)
    uy_col = (AMP * np.sin(phase)).astype(F)
    starts, seeds = [], []
    for rep in range(REPS):
        s = 0x5EED ^ _rep_bits(rep) ^ 0x1357
        starts.append(O.column_wave_cells(SIZE, SIZE, DENSITY, u0, uy_col, True, s ^ 0xF00D))
        seeds.append(0x5EED ^ (rep << 20))
    m = np.zeros(4, np.int64)
    O.lib().lgo_moments_sum(O.ptr(starts[0], O.C.c_uint8), starts[0].size, 1,
                            O.ptr(m, O.C.c_int64))
    u_actual = F(F(m[1]) * F(0.5)) / F(m[0])     # Moments::velocity (src/moments.rs:91-97)
    cpu, gpu = _both_arms(LG, O, starts, seeds, (float(u0), 0.0), interval,
                          lambda c: O.column_uy(c, SIZE, SIZE), lambda g: g.column_uy(), phase,
                          restart=True)

    def fit(trace):
        unwrapped = 0.0
        prev = math.atan2(trace[0][0], trace[0][1])
        pts = []
        for i, (a, b) in enumerate(trace):
            delta = math.atan2(a, b) - prev
            while delta > math.pi:
                delta -= 2 * math.pi
            while delta < -math.pi:
                delta += 2 * math.pi
            unwrapped += delta
            prev = math.atan2(a, b)
            pts.append((float(i * interval), unwrapped))
        return -_fit_slope(pts) / float(F(k * u_actual))

    g_cpu, g_gpu = fit(cpu), fit(gpu)
    rel = abs(g_gpu - g_cpu) / g_cpu
    print("advection: cpu g = %.4f, gpu g = %.4f (%.1f%% apart)" % (g_cpu, g_gpu, 100 * rel))
    assert rel < 0.03, "the GPU advects differently: g = %.4f against the CPU's %.4f" % (
        g_gpu, g_cpu)
