"""Serving: each result of a request served in the mix is exactly the result
of the same request run alone (lgx_attach_field + lgx_advance_sampling on a
fresh lattice); admission respects the budget; cancellation and an injected
allocation failure leave the rest of the stream unaffected.  Needs a GPU."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_stream(seed, n):
    from lattice_gas import workloads as W
    return W.request_stream(seed=seed, n=n, size_scale=0.12, step_scale=0.02)


def alone(LG, wl):
    g = LG.GpuLattice(wl.w, wl.h, wl.rest, wl.seed)
    if wl.inlet_cols:
        g.set_inlet(wl.inlet_cols, wl.density, wl.inflow, wl.rest)
    g.attach_field(wl.block, wl.block)
    g.load(wl.cells)
    g.advance_sampling(wl.steps, wl.sample_every, wl.alpha)
    f = g.read_field()
    sums = g.read_block_sums()
    out = dict(ux=f.ux, uy=f.uy, rho=f.rho, solid=f.solid, mass=sums[0], px2=sums[1],
               py2=sums[2], nsolid=sums[3], particles=g.total_particles())
    g.close()
    return out


def check_same(a, b):
    for k in ("ux", "uy", "rho", "solid", "mass", "px2", "py2", "nsolid"):
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k
    assert a["particles"] == b["particles"]


def test_each_result_is_the_same_alone_and_in_the_mix(LG):
    reqs = small_stream(7, 24)
    srv = LG.Server(budget_bytes=256 << 20, max_active=64)
    t0 = time.perf_counter()
    ids = []
    for r in reqs:   # Poisson arrivals, compressed 10x
        delay = r.arrival / 10 - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        ids.append(srv.submit_workload(r.work))
    for rid in ids:
        assert srv.wait(rid, 120.0) == LG.REQ_DONE
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    for r, rid in zip(reqs, ids):
        got = srv.result(rid)
        check_same(got, alone(LG, r.work))
        assert got["latency"] > 0
        srv.release(rid)
    srv.close()


def test_budget_limits_residency_but_everything_finishes(LG):
    reqs = small_stream(8, 16)
    # a budget that holds only a few of these lattices at once
    per = max(LG.Server.request_bytes(r.work) for r in reqs)
    srv = LG.Server(budget_bytes=per * 3, max_active=64)
    ids = [srv.submit_workload(r.work) for r in reqs]
    for rid in ids:
        assert srv.wait(rid, 120.0) == LG.REQ_DONE
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert 0 < st["peak_bytes"] <= per * 3
    assert 1 <= st["peak_active"] < len(reqs)   # requests had to wait for room
    for r, rid in zip(reqs[:4], ids[:4]):
        check_same(srv.result(rid), alone(LG, r.work))
    srv.close()


def test_cancel_and_injected_failure_do_not_disturb_the_rest(LG):
    reqs = small_stream(9, 10)
    srv = LG.Server(budget_bytes=1 << 30, max_active=2)
    srv.inject_alloc_failure(1)
    ids = [srv.submit_workload(r.work) for r in reqs]
    srv.cancel(ids[-1])          # still queued (only two resident at a time)
    states = [srv.wait(rid, 120.0) for rid in ids]
    assert states[0] == LG.REQ_FAILED       # the injected allocation failure
    assert states[-1] == LG.REQ_CANCELLED
    for r, rid, st in zip(reqs[1:-1], ids[1:-1], states[1:-1]):
        assert st == LG.REQ_DONE
        check_same(srv.result(rid), alone(LG, r.work))
    with pytest.raises(LG.LgxError):
        srv.result(ids[0])
    srv.close()


def test_oversize_requests_are_refused(LG):
    srv = LG.Server(budget_bytes=1 << 20, max_active=4)
    w, h = 2048, 1024
    cells = np.zeros(w * h, np.uint8)
    with pytest.raises(LG.LgxError) as e:
        srv.submit(cells, w, h, True, 1, 0.2, (0.0, 0.0), 0, 10, 5, 1.0, 16, 16)
    assert e.value.code == 6
    srv.close()


def test_destroy_with_work_in_flight(LG):
    reqs = small_stream(10, 6)
    srv = LG.Server(budget_bytes=1 << 30, max_active=2)
    for r in reqs:
        srv.submit_workload(r.work)
    srv.close()   # cancels what is queued or running, then joins


def test_mixed_rules_in_one_tick(LG):
    """Rest-particle and six-direction requests resident together (one launch per step
    for both rules, two launch chains): each result is still the one it has alone."""
    import dataclasses
    reqs = small_stream(11, 12)
    works = []
    for i, r in enumerate(reqs):
        wl = r.work
        if i % 2:
            cells = wl.cells & np.uint8(0xBF)  # no rest particles in a six-direction lattice
            wl = dataclasses.replace(wl, rest=False, cells=cells)
        works.append(wl)
    srv = LG.Server(budget_bytes=512 << 20, max_active=64)
    ids = [srv.submit_workload(wl) for wl in works]
    for rid in ids:
        assert srv.wait(rid, 120.0) == LG.REQ_DONE
    for wl, rid in zip(works, ids):
        check_same(srv.result(rid), alone(LG, wl))
    srv.close()
