#!/usr/bin/env python3
"""Benchmark: the wake run (4096 x 2304 FHP-III lattice, plate, inflow, walls,
20,000 steps, 32 x 32 coarse-graining every 100 steps) in Gsite-updates/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One bench step is one whole wake run: 20,000 lattice steps plus 200 samples.
`value` is device time (CUDA events on the lattice's stream) with the initial
state already resident in HBM; `e2e` is the same run through the public API
from page-locked host buffers: load the cells, run, read the field and the
block sums back, every step.  Between timed steps a 256 MiB buffer is written
to flush L2 (129 MB).  `--impl reference` times the reference's CPU update
(the byte-per-cell Lattice::step, restated in C in oracle/) on the host's
cores for a bounded sample of the same run.

Under torchrun with N > 1 every rank runs its own replica of the run on its
own GPU (the path has no exchange step); timings are maxed over ranks and the
value counts the site-updates of all ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "lattice-gas_gb300"))

METRIC = "Gsite-updates/s (wake run, plain per-lattice step)"
UNIT = "Gsite-updates/s"
ALGO_BYTES_PER_SITE = 1.75   # 7 bits read + 7 bits written per site-update


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# Figures from ncu captures of the wake run's step kernel in the shape the tuner
# picks there, four words per lane (lgx_step_lanes_kernel; one launch = one
# step): DRAM bytes read + written per launch (cold cache under ncu, the mean of
# three launches; the 18 MB of planes stay in L2 between steps of a timed run) and
# the ALU-pipe warp instructions per launch, which do not depend on timing; and,
# for the roofline case, DRAM bytes per site-update from a 16384 x 8192 capture of
# the same kernel (the mean of two launches; the full 32768 x 16384 case scales
# with its sites).  They hold for the kernel sources they were captured from:
# STEP_SOURCES hashed to CAPTURED_SOURCES_SHA.  When the sources differ the line
# says "stale": true.
STEP_TRAFFIC_BYTES = (9317120 + 8649472 + 8640256) // 3
STEP_ALU_WARP_INSTR = 3024084
BIG_DRAM_BYTES_PER_SITE = (125232512 + 73479680) / (16384 * 8192)
STEP_SOURCES = ("lgx_step.cu", "lgx_step_impl.cuh", "lgx_device.cuh",
                os.path.join("generated", "collide.cuh"))
CAPTURED_SOURCES_SHA = "fe082445883e4dcc"


def step_sources_sha() -> str:
    """sha256 (16 hex digits) over the step kernel's source files, in order."""
    import hashlib
    h = hashlib.sha256()
    for f in STEP_SOURCES:
        with open(os.path.join(ROOT, "lattice-gas_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu),
                                      "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for name, v in zip(names, s[4:8]):
                if v.strip().lower() in ("active", "1", "yes"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(world, x: float) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(world, x: float) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class L2Flusher:
    """Writes a buffer larger than L2 on the device between timed steps."""

    def __init__(self, device: int, nbytes: int = 256 << 20):
        import torch
        self.torch = torch
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda:%d" % device)

    def __call__(self):
        self.buf.fill_(1)
        self.torch.cuda.synchronize()


def cpu_reference_rate(wl, seconds: float, threads: int, chunk: int = 20):
    """Site-updates/s of the reference's CPU update (oracle restatement of
    Lattice::step, banded over `threads`) on the same lattice, sampling every
    `wl.sample_every` steps, for about `seconds` of work."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O
    lat = O.Lattice(wl.w, wl.h, wl.density, wl.inflow, wl.inlet_cols, wl.rest, threads, wl.seed)
    lat.set_cells(wl.cells)
    field = O.Field(wl.w, wl.h, wl.block, wl.block)
    steps = 0
    t0 = time.perf_counter()
    while True:
        lat.advance(chunk)
        steps += chunk
        if steps % wl.sample_every == 0:
            field.sample(lat.cells, wl.w, wl.h, wl.alpha)
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return wl.sites * steps / dt, steps, dt


def cpu_bitplane_rate(wl, seconds: float, threads: int, chunk: int = 20):
    """Site-updates/s of the bitplane update restated in C (the oracle's
    GpuLattice, the same words and draws as the engine) on the host's cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    g = O.BitplaneLattice(wl.w, wl.h, wl.rest, wl.seed, threads)
    g.set_inlet(wl.inlet_cols, wl.density, wl.inflow, wl.rest)
    g.attach_field(wl.block, wl.block)
    g.load(wl.cells)
    steps = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        g.advance_sampling(chunk, wl.sample_every, wl.alpha)
        steps += chunk
    dt = time.perf_counter() - t0
    return wl.sites * steps / dt, steps, dt


def wake_config(steps: int, world: int) -> dict:
    """The headline workload's config, the same for both arms."""
    return {"workload": "wake_run: 4096x2304 FHP-III, plate at x=512 of 1/8 channel height, "
                        "8-column inflow u=0.2, density 0.3, walls at rows 0 and h-1; 20000 "
                        "steps, 32x32 blocks every 100 steps",
            "w": 4096, "h": 2304, "lattice_steps_per_bench_step": steps,
            "sample_every": 100, "block": 32,
            "l2": "flushed between timed steps (256 MiB write)",
            "parallelism": "replicas x%d" % world}


def run_reference(args, world, rank):
    """The reference's CPU update on the host's cores.  Nothing of the engine is
    loaded: the cells come from the oracle's restatement of the reference's setup
    (add_solid, init_equilibrium) and the step is the oracle's Lattice::step."""
    if rank != 0:
        return 0
    from types import SimpleNamespace
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    w, h, every = 4096, 2304, 100
    wl = SimpleNamespace(w=w, h=h, rest=True, seed=0x5EED, density=0.3, inflow=(0.2, 0.0),
                         inlet_cols=8, block=32, sample_every=every, alpha=1.0, sites=w * h,
                         steps=args.lattice_steps, cells=O.wake_run_cells(w, h, 0.3, 0.2, 0x5EED))
    threads = os.cpu_count() or 1
    # each bench step: a bounded sample of the run (~2 s of the host's cores)
    for _ in range(args.warmup):
        cpu_reference_rate(wl, 0.5, threads)
    rates = []
    total_steps = 0
    total_t = 0.0
    for _ in range(args.steps):
        r, n, dt = cpu_reference_rate(wl, 2.0, threads)
        rates.append(r)
        total_steps += n
        total_t += dt
    value = wl.sites * total_steps / total_t / 1e9
    sample = ("%d lattice steps of the wake run in %d samples of ~2 s (a bounded sample of the "
              "20000-step run; the metric is a rate), byte-per-cell Lattice::step restated in C "
              "(oracle/), %d threads, 32x32 field sampled every 100 steps"
              % (total_steps, args.steps, threads))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * total_t / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": wake_config(args.lattice_steps, world),
        "sample": sample,
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def bench_batched(LG, W, steps: int):
    """The transport sweep: 64 periodic shear-wave lattices, 256..2048 x 256..1024,
    16x16 blocks every 50 steps; once one lattice per launch (each lattice's
    run in turn), once as one batch (a replayed CUDA graph per interval)."""
    wls = W.transport_sweep(steps=steps)
    sites = sum(w.sites for w in wls)

    def mk(wl, mode):
        g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
        g.set_step_mode(mode)
        g.attach_field(wl.block, wl.block)
        g.load(wl.cells)
        return g

    plain = [mk(wl, 1) for wl in wls]
    for g in plain:
        g.advance_sampling(100, 50, 1.0)
    t0 = time.perf_counter()
    for g in plain:
        g.advance_sampling(steps, 50, 1.0)
    t_plain = time.perf_counter() - t0
    together = [mk(wl, 0) for wl in wls]
    b = LG.Batch(together)
    b.advance_sampling(100, 50, 1.0)
    k0, g0 = b.launches
    b.timing_mark(0)
    b.advance_sampling(steps, 50, 1.0)
    b.timing_mark(1)
    t_batch = b.timing_elapsed(0, 1) / 1e3
    k1, g1 = b.launches
    same = all(np.array_equal(x.store(), y.store()) for x, y in zip(plain, together))
    # end to end through the public API: every lattice loaded from host memory,
    # the batch run, every field read back
    t0 = time.perf_counter()
    for g, wl in zip(together, wls):
        g.restart(wl.cells, wl.seed)
    b.advance_sampling(steps, 50, 1.0)
    for g in together:
        g.read_field()
    t_e2e = time.perf_counter() - t0
    out = {"workload": "transport sweep: 64 shear-wave lattices 256..2048 x 256..1024, "
                       "%d steps, 16x16 blocks every 50" % steps,
           "sites": sites, "value": round(sites * steps / t_batch / 1e9, 2),
           "plain_value": round(sites * steps / t_plain / 1e9, 2),
           "speedup_vs_plain": round(t_plain / t_batch, 2), "unit": UNIT,
           "batched_s": round(t_batch, 4), "plain_s": round(t_plain, 4),
           "e2e_value": round(sites * steps / t_e2e / 1e9, 2),
           "e2e_note": "host cells in, fields out, through GpuLattice.restart / Batch / "
                       "read_field; the plain figure is host-timed the same way",
           "kernel_launches": k1 - k0, "graph_launches": g1 - g0,
           "bit_exact_vs_plain": bool(same),
           "size_classes": [{k: (round(v, 2) if isinstance(v, float) else v)
                             for k, v in c.items()} for c in b.plan],
           "size_class_note": "the tuner's per-step times, one launch per step vs the "
                              "resident kernel, for each class of small lattices"}
    b.close()
    for g in plain + together:
        g.close()
    return out


def bench_roofline_case(LG, W, steps: int):
    """The 32768 x 16384 roofline case (200 circles, inflow): one launch per
    step, and temporal blocking of 4 and 8 steps per pass over HBM."""
    wl = W.roofline_case()
    out = {"workload": "roofline case: 32768x16384, 200 circles r 16..64, 8-column inflow, "
                       "density 0.2; %d steps timed per mode" % steps, "sites": wl.sites}
    states = {}
    for mode, k, name in ((1, 0, "single"), (3, 4, "temporal4"), (3, 8, "temporal8")):
        g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
        g.set_step_mode(mode)
        if k:
            g.set_temporal_depth(k)
        g.set_inlet(wl.inlet_cols, wl.density, wl.inflow, True)
        g.load(wl.cells)
        g.advance(16)
        g.timing_mark(0)
        g.advance(steps)
        g.timing_mark(1)
        ms = g.timing_elapsed(0, 1) / steps
        states[name] = g.store()
        out[name] = {"ms_per_step": round(ms, 4),
                     "value": round(wl.sites / (ms * 1e-3) / 1e9, 1),
                     "algorithmic_GBps": round(wl.sites * ALGO_BYTES_PER_SITE / (ms * 1e-3) / 1e9, 1)}
        g.close()
    probe = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
    out["step_plan"] = {k: (round(v, 3) if isinstance(v, float) else v)
                        for k, v in probe.step_plan.items()}
    probe.close()
    out["single"]["dram_GBps_from_ncu"] = round(
        wl.sites * BIG_DRAM_BYTES_PER_SITE / (out["single"]["ms_per_step"] * 1e-3) / 1e9, 1)
    out["bit_exact_temporal_vs_single"] = bool(
        np.array_equal(states["single"], states["temporal4"]) and
        np.array_equal(states["single"], states["temporal8"]))
    out["unit"] = UNIT
    return out


def bench_transport(LG, cpu: bool):
    """transport::measure (src/transport.rs:291-319), the caller that synchronises
    most: one measurement at the reference's sizes (its own bench times 64 and 256,
    benches/speed.rs:676-683) and main.rs's 22-density scan as one batch.  The CPU
    reference is the oracle's byte-path measure, the reference's CPU path."""
    import time
    out = {"unit": "s per call", "density": 0.22, "rest": True}
    for size in (64, 256):
        best = None
        for _ in range(3):
            t = time.perf_counter()
            r = LG.transport_measure([0.22], rest=True, seed=0x5EED, size=size)[0]
            dt = time.perf_counter() - t
            best = dt if best is None else min(best, dt)
        out["measure_%d" % size] = {"engine_s": round(best, 4), "nu": round(r.nu, 5),
                                    "g": round(r.g, 5), "window_nu": r.window_nu,
                                    "window_g": r.window_g}
    ds = [0.04 + 0.02 * i for i in range(22)]
    t = time.perf_counter()
    LG.transport_measure(ds, rest=True, seed=0x5EED, size=256)
    out["scan_22_densities_256"] = {"engine_s": round(time.perf_counter() - t, 4),
                                    "densities": "0.04..0.46 step 0.02 (src/main.rs:549-560)"}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        threads = os.cpu_count() or 1
        t = time.perf_counter()
        c = O.transport_measure(0.22, True, threads, 0x5EED, 64, gpu=False)
        dt = time.perf_counter() - t
        out["measure_64"]["cpu_reference_s"] = round(dt, 4)
        out["measure_64"]["cpu"] = {"kind": "port", "cores": threads, "nu": round(c.nu, 5),
                                    "g": round(c.g, 5),
                                    "sample": "transport::measure(0.22, rest, %d threads, "
                                              "0x5EED, 64, cpu) restated in C" % threads}
        out["measure_64"]["speedup_vs_cpu"] = round(dt / out["measure_64"]["engine_s"], 1)
        out["measure_64"]["note"] = (
            "the CPU path draws from the byte stream, the engine from the bitplane stream, so "
            "their estimates are different samples; at 64x64 the decay windows are short and "
            "nu is noise-dominated (the reference's own 64x64 call is a speed benchmark). The "
            "engine's measure equals the oracle's bitplane-path measure bit for bit; at 256x256 "
            "nu sits near the reference's quoted 0.2989 (src/gpu.rs:1172-1175)")
    return out


# The reference's GPU benchmark matrix (benches/speed.rs:480-592) and its figures on
# an Apple M3 Pro through Metal (benches/baseline.txt:21-29), Mcell/s: context, not a
# target (other hardware, other API).
REFERENCE_MATRIX = [
    ("step/gpu/2048x1280/one-per-submit", 16692.3),
    ("step/gpu/2048x1280/batched", 79234.4),
    ("step/gpu/256x256/batched", 9428.9),
    ("step/gpu/4096x2048/batched", 93454.4),
    ("step/gpu/2048x1280/batched+inlet", 76372.2),
    ("step/gpu/2048x1280/batched+inlet+sample", 70812.7),
    ("field/gpu/sample/2048x1280", 20465.0),
    ("lattice/gpu/store/2048x1280", 2611.4),
    ("lattice/gpu/total-particles/2048x1280", 17646.6),
]


# The reference's host-side cases of the same file (benches/speed.rs:606-681) that
# this engine runs on the device, with its M3 Pro figures in ns per call
# (benches/baseline.txt:31-32, 41, 42); cells per call where it counts them.
REFERENCE_HOST_ROWS = [
    ("field/vorticity/2048x1280", 8909.5, 0),
    ("field/mean-velocity/2048x1280", 4751.6, 0),
    ("field/vorticity+mean-velocity/2048x1280 (one call)", 8909.5 + 4751.6, 0),
    ("lattice/init-equilibrium/2048x1280", 17224694.4, 2048 * 1280),
    ("transport/measure/64", 626022417.0, 0),
    ("lattice/total-particles/2048x1280", 44570.5, 2048 * 1280),
    ("lattice/mean-velocity/2048x1280", 501249.2, 2048 * 1280),
]


# The reference's CPU step cases (benches/speed.rs:409-476: the byte-per-cell
# Lattice::step, one step per call) and its M3 Pro figures in Mcell/s
# (benches/baseline.txt:13-20); this engine runs the same stream on the device.
# (w, h, bands, rest, inlet columns, plate); tN is the reference's 12 threads.
REFERENCE_CPU_STEP_ROWS = [
    ("step/512x512/t1", 458.7, (512, 512, 1, True, 0, False)),
    ("step/512x512/tN", 1505.6, (512, 512, 12, True, 0, False)),
    ("step/512x512/t1/no-rest", 463.3, (512, 512, 1, False, 0, False)),
    ("step/512x512/tN/plate", 1502.8, (512, 512, 12, True, 0, True)),
    ("step/512x512/tN/inlet", 1290.9, (512, 512, 12, True, 8, False)),
    ("step/2048x1280/t1", 248.4, (2048, 1280, 1, True, 0, False)),
    ("step/2048x1280/tN", 1844.0, (2048, 1280, 12, True, 0, False)),
    ("step/2048x64/tN", 1061.7, (2048, 64, 12, True, 0, False)),
]


STEP_MODE_NAMES = {1: "single", 2: "wave", 3: "temporal", 4: "graph"}
SHAPE_NAMES = {1: "1 chunk per warp", 2: "2 chunks per warp", 3: "2 words per lane",
               4: "4 words per lane"}
STEP_KERNEL_NAMES = {1: "lgx_step_kernel (1 chunk per warp)",
                     2: "lgx_step_kernel (2 chunks per warp)",
                     3: "lgx_step_lanes_kernel (2 words per lane)",
                     4: "lgx_step_lanes_kernel (4 words per lane)"}


def plan_name(plan: dict) -> str:
    """The step mode the tuner picked, as words."""
    name = STEP_MODE_NAMES.get(plan["mode"], str(plan["mode"]))
    if plan["mode"] == 1:
        name += " (%s)" % SHAPE_NAMES.get(plan["words"], str(plan["words"]))
    elif plan["mode"] == 3:
        name += " k=%d" % plan["depth"]
    return name


def bench_reference_matrix(LG, sample_s: float = 0.1, samples: int = 7):
    """Each case of the reference's GPU benchmark group through this engine's
    GpuLattice, set up as benches/speed.rs does (density 0.22, speed 0.4, 20x20 blocks,
    seed 0x5EED, cells from Lattice::init_equilibrium): warm up, then `samples`
    samples of about `sample_s` seconds each; the value is the median sample, with the
    best beside it (the reference reports its best, benches/speed.rs:150-193). Every
    call waits for the device, as the reference's submit-and-wait does. Throughput in
    Gcell/s (cell updates, or cells processed); step cases name the step mode the
    tuner picked for the lattice."""
    D, S, BLOCK, SEED = 0.22, 0.4, 20, 0x5EED

    def seeded(w, h):
        cells = np.zeros(w * h, np.uint8)
        LG.init_equilibrium(cells, D, S, 0.0, True, SEED)
        g = LG.GpuLattice(w, h, True, SEED)
        g.load(cells)
        return g

    def rate(body, cells_per_iter):
        t0, n = time.perf_counter(), 0
        while time.perf_counter() - t0 < sample_s or n < 3:
            body()
            n += 1
        per = (time.perf_counter() - t0) / n
        iters = max(1, int(round(sample_s / per)))
        ts = []
        for _ in range(samples):
            t = time.perf_counter()
            for _ in range(iters):
                body()
            ts.append((time.perf_counter() - t) / iters)
        return cells_per_iter / statistics.median(ts) / 1e9, cells_per_iter / min(ts) / 1e9

    bw, bh = 2048, 1280
    out = []
    modes = []
    g = seeded(bw, bh)
    got = [rate(lambda: g.advance(1), bw * bh), rate(lambda: g.advance(100), bw * bh * 100)]
    plan = g.step_plan
    modes += ["single (one step per call)", plan_name(plan)]
    g.close()
    g = seeded(256, 256)
    got.append(rate(lambda: g.advance(100), 256 * 256 * 100))
    modes.append(plan_name(g.step_plan))
    g.close()
    g = seeded(4096, 2048)
    got.append(rate(lambda: g.advance(100), 4096 * 2048 * 100))
    modes.append(plan_name(g.step_plan))
    g.close()
    g = seeded(bw, bh)
    g.set_inlet(8, D, (S, 0.0), True)
    got.append(rate(lambda: g.advance(100), bw * bh * 100))
    modes.append(plan_name(g.step_plan))
    g.attach_field(BLOCK, BLOCK)
    got.append(rate(lambda: g.advance_sampling(100, 5, 0.2), bw * bh * 100))
    modes.append(plan_name(g.step_plan) + ", sampling every 5")
    g.close()
    g = seeded(bw, bh)
    g.attach_field(BLOCK, BLOCK)
    got.append(rate(lambda: g.sample_field(0.2), bw * bh))
    buf = np.zeros(bw * bh, np.uint8)
    got.append(rate(lambda: g.store(buf), bw * bh))
    got.append(rate(lambda: g.total_particles(), bw * bh))
    modes += [None, None, None]
    g.close()
    for (name, ref), (v, best), mode in zip(REFERENCE_MATRIX, got, modes):
        row = {"case": name, "value": round(v, 2), "best": round(best, 2),
               "reference_m3pro_metal": round(ref / 1e3, 3), "ratio": round(v * 1e3 / ref, 1)}
        if mode:
            row["step_mode"] = mode
        out.append(row)

    def ns(body):  # rate() gives calls per ns for one unit per call (median sample)
        return 1.0 / rate(body, 1.0)[0]

    host = []
    g = seeded(bw, bh)
    g.attach_field(BLOCK, BLOCK)
    g.advance_sampling(100, 5, 0.2)
    times = [ns(lambda: g.vorticity()), ns(lambda: g.mean_velocity()),
             ns(lambda: g.field_analyses())]
    g.close()
    lat = LG.Lattice(bw, bh, D, (S, 0.0), 8, True, 16, SEED)
    times.append(ns(lambda: lat.init_equilibrium()))
    lat.close()
    best = float("inf")
    for _ in range(3):
        t = time.perf_counter()
        LG.transport_measure([D], rest=True, seed=SEED, size=64)
        best = min(best, time.perf_counter() - t)
    times.append(best * 1e9)
    lat = LG.Lattice(bw, bh, D, (S, 0.0), 0, True, 12, SEED)  # benches/speed.rs:334-346
    lat.init_equilibrium()
    times += [ns(lambda: lat.total_particles()), ns(lambda: lat.mean_velocity())]
    lat.close()
    for (name, ref_ns, n), t in zip(REFERENCE_HOST_ROWS, times):
        row = {"case": name, "ns_per_call": round(t, 1), "reference_m3pro_cpu_ns": ref_ns,
               "ratio": round(ref_ns / t, 2)}
        if n:
            row["gcell_per_s"] = round(n / t, 2)
        host.append(row)
    steps = []
    for name, ref, (w, h, bands, rest, inlet, plate) in REFERENCE_CPU_STEP_ROWS:
        cells = np.zeros(w * h, np.uint8)
        if plate:  # benches/speed.rs:334-341, the binary's plate scaled to the lattice
            yc = np.float32(h) * LG.SQRT3_2 / np.float32(2.0)
            size = np.float32(h) * np.float32(173.0) / np.float32(1280.0)
            x0 = np.float32(w) / np.float32(5.0)
            LG.add_box(cells, w, h, x0, x0 + np.float32(4.0), yc - size / np.float32(2.0),
                       yc + size / np.float32(2.0))
        lat = LG.Lattice(w, h, D, (S, 0.0), inlet, rest, bands, SEED)
        lat.load(cells)
        lat.init_equilibrium()
        v = rate(lambda: lat.advance(1), w * h)[0]
        lat.close()
        steps.append({"case": name, "value": round(v, 2), "reference_m3pro_cpu": round(ref / 1e3, 4),
                      "ratio": round(v * 1e3 / ref, 1)})
    return {"unit": "Gcell/s", "cases": out, "host_cases_on_device": host,
            "byte_step_cases_on_device": steps,
            "step_plan_2048x1280": {k: (round(v, 3) if isinstance(v, float) else v)
                                    for k, v in plan.items()},
            "note": "the reference's own GPU cases (benches/speed.rs) on this engine, median "
                    "of %d samples of ~%.1f s (best beside it); its M3 Pro Metal figures (benches/baseline.txt) are "
                    "other hardware, for context. host_cases_on_device: its CPU cases that "
                    "this engine runs on the device (ns per call, each call a launch and a "
                    "read-back; ratio = reference time / this time). byte_step_cases_on_device: "
                    "its CPU byte-per-cell step cases, the same random stream run by this "
                    "engine's device byte path, one step and a wait per call" % (samples, sample_s)}


def bench_byte_path(LG, W, steps: int, cpu_rate):
    """The reference's own CPU update (byte per cell, its random stream, bands of
    ceil(h / threads) rows, src/lattice.rs:222-364) run on the device on the wake
    run, 16 bands as the reference on 16 host threads: the path whose golden
    checksums (tests/golden.rs) the device reproduces.  Beside it the same update
    on the host cores (the CPU baseline of this line)."""
    wl = W.wake_run(steps=steps)
    lat = LG.Lattice(wl.w, wl.h, wl.density, wl.inflow, wl.inlet_cols, wl.rest, 16, wl.seed)
    lat.load(wl.cells)
    lat.advance(50)
    dt = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        lat.advance(steps)
        lat.store()
        dt = min(dt, time.perf_counter() - t0)
    out = {"workload": "wake run 4096x2304, byte-per-cell update with the reference's random "
                       "stream, 16 bands, %d steps and a read-back, best of 3" % steps,
           "value": round(wl.sites * steps / dt / 1e9, 2), "unit": UNIT,
           "note": "the parity path: each band's draws come from one serial generator, so "
                   "every 64-cell segment jumps its band's state ahead (a jump polynomial) "
                   "and walks its cells in order, one xorshift64* step per cell; the "
                   "bitplane step is the throughput path"}
    if cpu_rate:
        out["cpu_reference"] = round(cpu_rate / 1e9, 4)
        out["speedup_vs_cpu"] = round(wl.sites * steps / dt / cpu_rate, 1)
    lat.close()
    return out


def bench_served(LG, W, n: int, budget: int):
    """The request stream: Poisson arrivals at 200/s, sizes 128x128..4096x2048,
    1k..50k steps, sampling every 50..500 steps with 8..32 blocks, obstacle none
    / plate / circle.  Served with continuous batching, and as the plain
    baseline each request alone on the plain kernel, first come first served."""
    import threading
    reqs = W.request_stream(n=n)
    work = sum(r.work.sites * r.work.steps for r in reqs)
    srv = LG.Server(budget_bytes=budget, max_active=512)
    ids = [None] * len(reqs)
    t0 = time.perf_counter()

    def feed():
        for i, r in enumerate(reqs):
            d = r.arrival - (time.perf_counter() - t0)
            if d > 0:
                time.sleep(d)
            ids[i] = srv.submit_workload(r.work)

    th = threading.Thread(target=feed)
    th.start()
    th.join()
    lat = []
    for rid in ids:
        if srv.wait(rid, 600.0) != LG.REQ_DONE:
            raise RuntimeError("a served request did not complete")
        lat.append(srv.result(rid)["latency"])
    t_served = time.perf_counter() - t0
    st = srv.stats()

    def digest(fields, sums, particles):
        import hashlib
        h = hashlib.blake2b(digest_size=16)
        for a in list(fields) + list(sums):
            h.update(np.ascontiguousarray(a).tobytes())
        h.update(int(particles).to_bytes(8, "little"))
        return h.hexdigest()

    served_digest = []
    for rid in ids:
        res = srv.result(rid)
        served_digest.append(digest((res["ux"], res["uy"], res["rho"], res["solid"]),
                                    (res["mass"], res["px2"], res["py2"], res["nsolid"]),
                                    res["particles"]))
    srv.close()
    # plain: each request alone, one lattice per launch, in arrival order
    clock = 0.0
    plain_lat = []
    busy = 0.0
    same = 0
    for r, sd in zip(reqs, served_digest):
        wl = r.work
        g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
        g.set_step_mode(1)
        if wl.inlet_cols:
            g.set_inlet(wl.inlet_cols, wl.density, wl.inflow, True)
        g.attach_field(wl.block, wl.block)
        t1 = time.perf_counter()
        g.load(wl.cells)
        g.advance_sampling(wl.steps, wl.sample_every, wl.alpha)
        f = g.read_field()
        sums = g.read_block_sums()
        svc = time.perf_counter() - t1
        same += digest((f.ux, f.uy, f.rho, f.solid), sums, g.total_particles()) == sd
        g.close()
        busy += svc
        clock = max(clock, r.arrival) + svc
        plain_lat.append(clock - r.arrival)
    lat.sort()
    plain_lat.sort()
    pct = lambda a, q: a[min(len(a) - 1, int(q * len(a)))]
    return {"workload": "request stream: %d requests, Poisson 200/s, 128x128..4096x2048, "
                        "1k..50k steps, sampling 50..500, blocks 8..32; budget %d MiB"
                        % (n, budget >> 20),
            "site_updates": work, "value": round(work / t_served / 1e9, 2),
            "plain_value": round(work / clock / 1e9, 2),
            "speedup_vs_plain": round(clock / t_served, 2), "unit": UNIT,
            "p50_latency_s": round(pct(lat, 0.5), 4), "p99_latency_s": round(pct(lat, 0.99), 4),
            "plain_p50_latency_s": round(pct(plain_lat, 0.5), 4),
            "plain_p99_latency_s": round(pct(plain_lat, 0.99), 4),
            "served_s": round(t_served, 3), "plain_s": round(clock, 3),
            "ticks": st["ticks"], "kernel_launches": st["kernel_launches"],
            "bit_exact_vs_plain": "%d of %d requests" % (same, len(reqs)),
            "device_busy_s": round(st["gpu_busy_ns"] / 1e9, 4),
            "host_tick_s": round(st["host_tick_ns"] / 1e9, 4),
            "host_wait_s": round(st["host_wait_ns"] / 1e9, 4),
            "latency_note": "includes queueing; the stream offers more work than the GPU "
                            "serves, so the queue grows while it arrives"}


def run_gb300(args, world, rank, local):
    import numpy as np
    import lattice_gas as LG
    from lattice_gas import workloads as W

    LG.select_device(local)
    peak, peak_kind = peaks()
    wl = W.wake_run(steps=args.lattice_steps)
    g = LG.GpuLattice(wl.w, wl.h, wl.rest, wl.seed)
    g.set_inlet(wl.inlet_cols, wl.density, wl.inflow, wl.rest)
    g.attach_field(wl.block, wl.block)
    g.load(wl.cells)
    flush = L2Flusher(local)

    def one_run():
        g.timing_mark(0)
        g.advance_sampling(wl.steps, wl.sample_every, wl.alpha)
        g.timing_mark(1)
        return g.timing_elapsed(0, 1)

    for _ in range(args.warmup):
        one_run()
        flush()

    # ---- device-resident timed region --------------------------------
    clocks = ClockSampler(local)
    launches0 = g.launches
    dist_barrier(world)
    clocks.start()
    ms = []
    for _ in range(args.steps):
        flush()
        ms.append(one_run())
    dist_barrier(world)
    clk = clocks.stop()
    launches = g.launches - launches0
    total_ms = dist_max(world, sum(ms))
    sites_all = dist_sum(world, float(wl.sites * wl.steps * args.steps))
    value = sites_all / (total_ms / 1e3) / 1e9

    # ---- the step kernel alone: average launch duration ----------------
    nk = 2000
    flush()
    g.timing_mark(2)
    g.advance(nk)
    g.timing_mark(3)
    step_ms = g.timing_elapsed(2, 3) / nk
    achieved = wl.sites * ALGO_BYTES_PER_SITE / (step_ms / 1e3) / 1e9

    # ---- end to end through the public API from pinned host memory -----
    nb = (wl.w // wl.block) * (wl.h // wl.block)
    hcells = LG.PinnedBuffer(wl.sites)
    hcells.array[:] = wl.cells
    hout = [LG.PinnedBuffer(nb * 4, np.float32) for _ in range(4)]
    hsum = [LG.PinnedBuffer(nb * 4, np.int32) for _ in range(4)]
    f = LG.Field(wl.w, wl.h, wl.block, wl.block)
    f.ux, f.uy, f.rho, f.solid = (b.array for b in hout)
    e2e_ms = []
    dist_barrier(world)
    for i in range(args.steps + 1):  # the first pass is an untimed warm-up of this path
        flush()
        g.timing_mark(4)
        g.restart(hcells.array, wl.seed)
        g.advance_sampling(wl.steps, wl.sample_every, wl.alpha)
        g.read_field(f)
        LG._check(LG.lib().lgx_read_block_sums(g.handle, *[LG._p(b.array, LG.C.c_int32)
                                                           for b in hsum], nb))
        g.timing_mark(5)
        if i:
            e2e_ms.append(g.timing_elapsed(4, 5))
    dist_barrier(world)
    e2e_total = dist_max(world, sum(e2e_ms))
    e2e_value = sites_all / (e2e_total / 1e3) / 1e9

    # ---- reported CPU baseline (rank 0, N = 1 only) -------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, nsteps, dt = cpu_reference_rate(wl, args.cpu_seconds, threads)
        cpu = {"value": round(rate / 1e9, 4), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d lattice steps of the wake run (%.1f s), byte-per-cell "
                         "Lattice::step restated in C (oracle/), %d threads"
                         % (nsteps, dt, threads)}
        brate, bsteps, bdt = cpu_bitplane_rate(wl, 4.0, threads)
        cpu["bitplane"] = {"value": round(brate / 1e9, 4), "unit": UNIT, "cores": threads,
                           "kind": "port",
                           "sample": "%d lattice steps of the wake run (%.1f s), the bitplane "
                                     "update (GpuLattice's shader) restated in C, %d threads"
                                     % (bsteps, bdt, threads)}

    batched = served = big = transport = byte_path = matrix = None
    if not args.no_patterns:
        batched = bench_batched(LG, W, args.sweep_steps)
        served = bench_served(LG, W, args.requests, args.budget_mib << 20)
        big = bench_roofline_case(LG, W, args.big_steps)
        transport = bench_transport(LG, rank == 0 and world == 1 and not args.no_cpu)
        byte_path = bench_byte_path(LG, W, 1000, rate if cpu else None)
        matrix = bench_reference_matrix(LG)
    lop3_peak = LG.probe_int_rate(0)
    src_sha = step_sources_sha()
    alu_achieved = STEP_ALU_WARP_INSTR * 32 / (step_ms * 1e-3)

    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32 bitplanes (integer)",
        "data": "synthetic (seeded wake-run lattice built with the reference's primitives)",
        "config": wake_config(wl.steps, world),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": STEP_TRAFFIC_BYTES, "peak_kind": peak_kind,
                     "ncu_figures": {"sources_sha": src_sha,
                                     "captured_from_sha": CAPTURED_SOURCES_SHA,
                                     "stale": src_sha != CAPTURED_SOURCES_SHA,
                                     "covers": "traffic, int_pipe.alu_warp_instr_per_launch, "
                                               "roofline_case.single.dram_GBps_from_ncu"},
                     "kernel": STEP_KERNEL_NAMES.get(g.step_plan["words"], "lgx_step_kernel"),
                     "step_kernel_us": round(step_ms * 1e3, 3),
                     "algorithmic_bytes_per_launch": wl.sites * ALGO_BYTES_PER_SITE,
                     "note": "the step is integer-ALU bound, not HBM bound: see int_pipe",
                     "int_pipe": {"achieved": round(alu_achieved / 1e12, 2),
                                  "peak": round(lop3_peak / 1e12, 2), "unit": "Tlane-op/s",
                                  "frac": round(alu_achieved / lop3_peak, 4),
                                  "alu_warp_instr_per_launch": STEP_ALU_WARP_INSTR,
                                  "peak_kind": "measured (lgx_probe_int_rate, lop3)"}},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": wl.sites,
                "d2h_bytes_per_step": 8 * nb * 4},
        "step_plan": {k: (round(v, 3) if isinstance(v, float) else v)
                      for k, v in g.step_plan.items()},
        "gpu_launches": launches,
        "clocks": clk,
        "cpu_baseline": cpu,
        "batched": batched,
        "served": served,
        "roofline_case": big,
        "transport": transport,
        "byte_path": byte_path,
        "reference_matrix": matrix,
        "device": g.device_name(),
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--lattice-steps", type=int, default=20000)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-patterns", action="store_true",
                    help="skip the batched and served measurements")
    ap.add_argument("--sweep-steps", type=int, default=5000)
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--budget-mib", type=int, default=16384)
    ap.add_argument("--big-steps", type=int, default=2000)
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    return run_gb300(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
