"""Synthetic workloads, expressed in the reference's own primitives.

No public dataset exists for this path; each workload is a seeded lattice
built the way the reference builds one (Lattice::new + add_solid +
init_equilibrium, src/lattice.rs; the shear-wave start of
src/transport.rs:188-200; the obstacle shapes of src/main.rs:582-595).
Every builder returns plain byte cells plus the run parameters, so the same
input can be handed to the engine and to the oracle.

  wake_run        4096 x 2304 wake behind a plate, inflow, walls (the default
                  single-lattice GPU run)
  periodic_box    256 x 128 periodic FHP-III box, Bernoulli(0.25) channels
  transport_sweep 64 periodic shear-wave lattices, 256..2048 x 256..1024
  roofline_case   32768 x 16384 with 200 circular obstacles and inflow
  request_stream  a Poisson stream of simulation requests
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import SQRT3_2, add_box, add_circle, init_equilibrium, shear_wave

F = np.float32


@dataclass
class Workload:
    name: str
    w: int
    h: int
    rest: bool
    seed: int
    cells: np.ndarray
    density: float
    inflow: tuple
    inlet_cols: int
    steps: int
    sample_every: int
    block: int
    alpha: float
    meta: dict = field(default_factory=dict)

    @property
    def sites(self) -> int:
        return self.w * self.h


def _alpha(sample_every: int) -> float:
    """The reference's default EMA weight, clamp(every / 25, 0.02, 1) (src/main.rs:502-507)."""
    return float(min(max(F(sample_every) / F(25.0), F(0.02)), F(1.0)))


def periodic_box(seed: int = 0x5EED, w: int = 256, h: int = 128, steps: int = 500) -> Workload:
    """256x128 periodic box, no obstacle; each of the 7 channels Bernoulli(0.25):
    Equilibrium(0.25, 0, 0, rest) gives threshold ceil(0.25 * 2^24) for all seven."""
    cells = np.zeros(w * h, np.uint8)
    init_equilibrium(cells, 0.25, 0.0, 0.0, True, seed)
    return Workload("periodic_box", w, h, True, seed, cells, 0.25, (0.0, 0.0), 0, steps, 100, 8,
                    1.0)


def wake_run(seed: int = 0x5EED, w: int = 4096, h: int = 2304, steps: int = 20000,
             density: float = 0.3, speed: float = 0.2, every: int = 100,
             block: int = 32) -> Workload:
    """Flow past a flat plate: plate of one eighth of the channel height at x = w/8
    (512 at the default width), 4 columns thick as src/main.rs:584-588; inflow of
    8 columns (src/main.rs:576); walls as solid rows y = 0 and y = h - 1."""
    cells = np.zeros(w * h, np.uint8)
    yc = F(h) * SQRT3_2 / F(2.0)
    height = F(h) * SQRT3_2
    half = height / F(16.0)
    x0 = F(w // 8)
    add_box(cells, w, h, x0, x0 + F(4.0), yc - half, yc + half)
    cells[:w] = 0x80
    cells[(h - 1) * w:] = 0x80
    init_equilibrium(cells, density, speed, 0.0, True, seed)
    return Workload("wake_run", w, h, True, seed, cells, density, (speed, 0.0), 8, steps, every,
                    block, _alpha(every), dict(plate_x=float(x0), plate_half=float(half)))


def roofline_case(seed: int = 0x5EED, w: int = 32768, h: int = 16384, steps: int = 2000,
                  n_circles: int = 200, density: float = 0.2, speed: float = 0.2) -> Workload:
    """Large lattice: 200 circles, centre uniform and radius U[16, 64] from the seed,
    in site_position coordinates; inflow as the wake run."""
    rng = np.random.default_rng(seed)
    cells = np.zeros(w * h, np.uint8)
    height = float(F(h) * SQRT3_2)
    circles = []
    for _ in range(n_circles):
        cx = F(rng.uniform(0.0, w))
        cy = F(rng.uniform(0.0, height))
        r = F(rng.uniform(16.0, 64.0))
        add_circle(cells, w, h, cx, cy, r)
        circles.append((float(cx), float(cy), float(r)))
    init_equilibrium(cells, density, speed, 0.0, True, seed)
    return Workload("roofline_case", w, h, True, seed, cells, density, (speed, 0.0), 8, steps,
                    100, 32, 1.0, dict(circles=circles))


def shear_wave_rows(h: int, amp: float = 0.05) -> np.ndarray:
    """ux(y) = amp * sin(k y sqrt(3)/2), k = 2 pi / (h sqrt(3)/2), in f32.  Computed
    once on the host and shared by engine and oracle."""
    k = F(2.0 * math.pi) / (F(h) * SQRT3_2)
    y = np.arange(h, dtype=np.float32)
    return (F(amp) * np.sin((k * y * SQRT3_2).astype(np.float32))).astype(np.float32)


def transport_sweep(seed: int = 0x5EED, n: int = 64, steps: int = 5000, every: int = 50,
                    block: int = 16, wmin=256, wmax=2048, hmin=256, hmax=1024):
    """64 independent periodic lattices, sizes log-uniform, densities U(0.1, 0.5),
    each started from a shear wave (src/transport.rs:188-200)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w = int(round(math.exp(rng.uniform(math.log(wmin), math.log(wmax)))))
        h = int(round(math.exp(rng.uniform(math.log(hmin), math.log(hmax)))))
        h += h & 1
        density = float(F(rng.uniform(0.1, 0.5)))
        s = (seed ^ ((i * 0x9E3779B9) << 20)) & (2 ** 64 - 1)
        cells = shear_wave(w, h, density, shear_wave_rows(h), True, s ^ 0xBEEF)
        out.append(Workload("sweep_%02d" % i, w, h, True, s, cells, density, (0.0, 0.0), 0, steps,
                            every, block, _alpha(every)))
    return out


@dataclass
class Request:
    rid: int
    arrival: float     # seconds from stream start
    work: Workload


def request_stream(seed: int = 0x5EED, n: int = 2000, rate: float = 200.0,
                   wmin=128, wmax=4096, hmin=128, hmax=2048, smin=1000, smax=50000,
                   size_scale: float = 1.0, step_scale: float = 1.0):
    """Poisson arrivals; size log-uniform; density U(0.1, 0.4); obstacle none /
    plate / circle; steps log-uniform; sampling period U{50..500}; block U{8..32}.
    size_scale and step_scale shrink a stream for tests (1.0 = as specified)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        w = int(round(math.exp(rng.uniform(math.log(wmin), math.log(wmax))) * size_scale))
        h = int(round(math.exp(rng.uniform(math.log(hmin), math.log(hmax))) * size_scale))
        w = max(w, 8)
        h = max(h + (h & 1), 8)
        density = float(F(rng.uniform(0.1, 0.4)))
        obstacle = int(rng.integers(0, 3))
        steps = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax))) * step_scale))
        steps = max(steps, 1)
        every = int(rng.integers(50, 501))
        block = int(rng.integers(8, 33))
        s = int(rng.integers(0, 2 ** 63))
        cells = np.zeros(w * h, np.uint8)
        yc = F(h) * SQRT3_2 / F(2.0)
        if obstacle == 1:
            half = F(h) * SQRT3_2 / F(16.0)
            add_box(cells, w, h, F(w // 8), F(w // 8) + F(4.0), yc - half, yc + half)
        elif obstacle == 2:
            r = F(rng.uniform(0.05, 0.2) * min(w, h))
            add_circle(cells, w, h, F(w // 4), yc, r)
        init_equilibrium(cells, density, 0.1, 0.0, True, s)
        inlet = 8 if obstacle else 0
        reqs.append(Request(i, t, Workload("req_%04d" % i, w, h, True, s, cells, density,
                                           (0.1, 0.0), inlet, steps, every, block,
                                           _alpha(every), dict(obstacle=obstacle))))
    return reqs
