"""A fixed run of one workload, for profilers (ncu) to attach to.

    python tests/profile_run.py --case wake --steps 60
    python tests/profile_run.py --case big --steps 20 --mode 1

Cases: `wake` (the 4096 x 2304 wake run), `big` (the roofline case's geometry at
16384 x 8192: planes of 235 MB, larger than L2, a few GB on the device),
`sweep` (the 64-lattice transport sweep as one batch), `analyses` (the field
vorticity and mean velocity of a 2048 x 1280 lattice, --steps calls), `transport` (one
transport::measure at --size, density 0.22), `fill` (init_equilibrium on the
device over the roofline case's geometry at 16384 x 8192), `tiny` (eight --size x
--size lattices as one batch), `bytes` (the wake run on the reference's
byte-per-cell update, 16 bands).  --policy picks the sweep's batch
policy (under a profiler pass 1: the tuner's timings are not meaningful there, and
without one it picks one launch per step for every class of this sweep).  --mode
picks the step
launch mode (1 one launch per step, 2 persistent waves, 3 temporal blocking), --shape
the single-step kernel's shape (1, 2: one or two 32-word chunks per warp; 3, 4: two or
four consecutive words per lane).
"""
import argparse
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "lattice-gas_gb300"))

import numpy as np  # noqa: E402

import lattice_gas as LG  # noqa: E402
from lattice_gas import workloads as W  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="wake",
                    choices=["wake", "big", "sweep", "transport", "fill", "tiny", "bytes",
                             "analyses"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--policy", type=int, default=0,
                    help="batch policy for the sweep: 0 tuned, 1 one launch per step, 2 resident")
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--mode", type=int, default=1)
    ap.add_argument("--depth", type=int, default=4)
    ap.add_argument("--shape", type=int, default=0,
                    help="the single-step kernel's shape (0 by size, 1-4 LGX_SHAPE_*)")
    a = ap.parse_args()
    if a.case == "tiny":
        # --size x --size lattices (8 of them) as one batch under --policy
        lats = [LG.GpuLattice(a.size, a.size, True, i) for i in range(8)]
        b = LG.Batch(lats, a.policy)
        b.advance(a.steps)
        print("tiny: 8 x %d^2, %d steps, policy %d, plan %s" % (a.size, a.steps, a.policy, b.plan))
        return
    if a.case == "analyses":
        # Field::vorticity and Field::mean_velocity of a 2048 x 1280 lattice's
        # 20 x 20 field (6,528 blocks), --steps calls of each
        w, h = 2048, 1280
        cells = np.zeros(w * h, np.uint8)
        LG.init_equilibrium(cells, 0.22, 0.4, 0.0, True, 1)
        g = LG.GpuLattice(w, h, True, 1)
        g.attach_field(20, 20)
        g.load(cells)
        g.advance_sampling(100, 5, 0.2)
        for _ in range(a.steps):
            g.mean_velocity()
            g.vorticity()
        print("analyses: %d x %d, %d calls each, mean %s" % (w, h, a.steps, g.mean_velocity()))
        return
    if a.case == "bytes":
        wl = W.wake_run()
        lat = LG.Lattice(wl.w, wl.h, wl.density, wl.inflow, wl.inlet_cols, wl.rest, 16, wl.seed)
        lat.load(wl.cells)
        lat.advance(a.steps)
        print("bytes: %d x %d, %d steps, %d particles" % (wl.w, wl.h, a.steps,
                                                           lat.total_particles()))
        lat.close()
        return
    if a.case == "fill":
        wl = W.roofline_case(w=16384, h=8192, n_circles=50)
        g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
        g.load(wl.cells)
        for _ in range(3):
            g.init_equilibrium(0.2, (0.1, 0.0), 0x5EED)
        print("fill: %d x %d, %d particles" % (wl.w, wl.h, g.total_particles()))
        return
    if a.case == "transport":
        r = LG.transport_measure([0.22], rest=True, seed=0x5EED, size=a.size)[0]
        print("transport %d: nu %.4f g %.4f windows %d %d" % (a.size, r.nu, r.g, r.window_nu,
                                                             r.window_g))
        return
    if a.case == "sweep":
        wls = W.transport_sweep(steps=a.steps)
        lats = []
        for wl in wls:
            g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
            g.attach_field(wl.block, wl.block)
            g.load(wl.cells)
            lats.append(g)
        b = LG.Batch(lats, a.policy)
        b.advance_sampling(a.steps, 50, 1.0)
        print("sweep: %d lattices, %d steps" % (len(lats), a.steps))
        return
    wl = W.wake_run() if a.case == "wake" else W.roofline_case(w=16384, h=8192, n_circles=50)
    g = LG.GpuLattice(wl.w, wl.h, True, wl.seed)
    g.set_step_mode(a.mode)
    g.set_step_shape(a.shape)
    if a.mode == 3:
        g.set_temporal_depth(a.depth)
    g.set_inlet(wl.inlet_cols, wl.density, wl.inflow, True)
    g.attach_field(wl.block, wl.block)
    g.load(wl.cells)
    g.advance_sampling(a.steps, wl.sample_every, wl.alpha)
    print("%s: %d x %d, %d steps, %d particles" % (a.case, wl.w, wl.h, a.steps,
                                                     g.total_particles()))


if __name__ == "__main__":
    main()
