"""The allocation-free step (lgx_step_planes_noalloc), for callers that cannot
let the library allocate device memory: hosts that own every device buffer
through their own arena, and loops that cannot take cudaMalloc's
synchronisation.  The caller owns the planes; the step's inflow draws live in
the library's fixed scratch array.

Two steps in a row through the C ABI must give exactly what the allocating
entry points give (lgx_load + lgx_set_inlet + lgx_advance), bit for bit: the
tolerance for this integer path is zero.  Kept in a file that pytest collects
last, so a run that stops at the first failure has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pack(cells, w, h):
    """Bytes -> (planes[7 * wpr * h], solid[wpr * h], anysolid) in the engine's layout."""
    wpr = (w + 31) // 32
    pad = np.zeros((h, wpr * 32), np.uint8)
    pad[:, :w] = cells.reshape(h, w)
    bits = np.unpackbits(pad[:, :, None], axis=2, bitorder="little")   # (h, wpr*32, 8)
    words = []
    for d in range(8):
        b = bits[:, :, d].reshape(h, wpr, 32).astype(np.uint64)
        words.append((b << np.arange(32, dtype=np.uint64)).sum(axis=2).astype(np.uint32)
                     .reshape(-1))
    planes = np.concatenate(words[:7])
    solid = words[7]
    total = wpr * h
    anysolid = np.zeros((total + 31) // 32, np.uint32)
    nz = np.nonzero(solid)[0]
    np.bitwise_or.at(anysolid, nz >> 5, (np.uint32(1) << (nz & 31).astype(np.uint32)))
    return planes, solid, anysolid


def unpack(planes, solid, w, h):
    wpr = (w + 31) // 32
    total = wpr * h
    out = np.zeros((h, wpr * 32), np.uint8)
    for d in range(8):
        src = planes[d * total:(d + 1) * total] if d < 7 else solid
        bits = ((src.reshape(h, wpr, 1) >> np.arange(32, dtype=np.uint32)) & 1).astype(np.uint8)
        out |= (bits.reshape(h, wpr * 32) << d)
    return out[:, :w].reshape(-1)


def dev(torch, a, offset=0):
    """a on the device, starting `offset` 32-bit words into its allocation (so that
    offset 1 gives a buffer aligned to a word but not to 8 or 16 bytes)."""
    t = torch.zeros(a.size + offset, dtype=torch.int32)
    t[offset:] = torch.from_numpy(a.view(np.int32).copy())
    return t.cuda()


@pytest.mark.parametrize("w,h,inlet,offset", [(300, 64, 40, 0), (300, 64, 0, 0),
                                              (4096, 1856, 8, 0), (4096, 1856, 8, 1),
                                              (300, 64, 40, 1)])
def test_no_alloc_step_matches_the_lattice_api_twice(LG, w, h, inlet, offset):
    """With a two-word inflow (the scratch in use) and without one, on a small
    lattice; and a lattice of a full wave of step blocks, whose step takes the
    kernel shape for large lattices.  offset 1: the caller's buffers start one
    word into their allocations, aligned to 4 bytes only (the step then keeps to
    32-bit accesses)."""
    torch = pytest.importorskip("torch")
    rest = True
    seed = 0xDEADBEEF12345678
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, 120.0, 27.0, 9.0)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.0, rest, 42)
    thresh = LG.thresholds(0.3, 0.2, 0.0, rest)

    # the allocating path
    g = LG.GpuLattice(w, h, rest, seed)
    g.set_step_mode(g.STEP_SINGLE)
    if inlet:
        g.set_inlet(inlet, 0.3, (0.2, 0.0), rest)
    g.load(cells)
    want = []
    for _ in range(2):
        g.advance(1)
        want.append(g.store())

    # the allocation-free path, two calls in a row on caller-owned buffers
    planes, solid, anysolid = pack(cells, w, h)
    assert np.array_equal(unpack(planes, solid, w, h), cells)
    a, b = dev(torch, planes, offset), dev(torch, np.zeros_like(planes), offset)
    s, an = dev(torch, solid, offset), dev(torch, anysolid, offset)
    torch.cuda.synchronize()
    L = LG.lib()
    th = np.ascontiguousarray(thresh, np.uint32)
    src, dst = a, b
    o = 4 * offset
    for step in range(2):
        rc = L.lgx_step_planes_noalloc(src.data_ptr() + o, dst.data_ptr() + o, s.data_ptr() + o,
                                       an.data_ptr() + o, w, h, int(rest), inlet,
                                       th.ctypes.data_as(C.POINTER(C.c_uint32)), seed, step,
                                       None)
        assert rc == 0, L.lgx_last_error().decode()
        torch.cuda.synchronize()
        got = unpack(dst.cpu().numpy().view(np.uint32)[offset:], solid, w, h)
        assert np.array_equal(got, want[step]), "step %d differs in %d cells" % (
            step, int((got != want[step]).sum()))
        src, dst = dst, src


def test_no_alloc_refuses_an_inflow_beyond_its_scratch(LG):
    torch = pytest.importorskip("torch")
    w, h = 128, 16384
    wpr = (w + 31) // 32
    x = torch.zeros(7 * wpr * h, dtype=torch.int32, device="cuda")
    y = torch.zeros_like(x)
    s = torch.zeros(wpr * h, dtype=torch.int32, device="cuda")
    an = torch.zeros((wpr * h + 31) // 32, dtype=torch.int32, device="cuda")
    th = np.zeros(7, np.uint32)
    L = LG.lib()
    # 16384 rows x 3 inflow words x 7 planes > 262144 scratch words
    rc = L.lgx_step_planes_noalloc(x.data_ptr(), y.data_ptr(), s.data_ptr(), an.data_ptr(), w,
                                   h, 1, 96, th.ctypes.data_as(C.POINTER(C.c_uint32)), 1, 0, None)
    assert rc == 1 and b"scratch" in L.lgx_last_error()


def test_no_alloc_steps_replay_from_a_cuda_graph(LG):
    """A warm-up call (the scratch address is looked up there), then two calls,
    a -> b at step 0 and b -> a at step 1, captured into one CUDA graph on a torch
    stream: each replay from the starting planes gives both steps bit for bit as
    the allocating path does (the inflow's scratch is written and read inside the
    graph, in stream order)."""
    torch = pytest.importorskip("torch")
    w, h, inlet, rest, seed = 300, 64, 40, True, 0x1234ABCD9876
    cells = np.zeros(w * h, np.uint8)
    LG.add_circle(cells, w, h, 120.0, 27.0, 9.0)
    LG.init_equilibrium(cells, 0.3, 0.2, 0.0, rest, 43)
    thresh = np.ascontiguousarray(LG.thresholds(0.3, 0.2, 0.0, rest), np.uint32)
    g = LG.GpuLattice(w, h, rest, seed)
    g.set_step_mode(g.STEP_SINGLE)
    g.set_inlet(inlet, 0.3, (0.2, 0.0), rest)
    g.load(cells)
    want = []
    for _ in range(2):
        g.advance(1)
        want.append(g.store())

    planes, solid, anysolid = pack(cells, w, h)
    a, b = dev(torch, planes), dev(torch, np.zeros_like(planes))
    s, an = dev(torch, solid), dev(torch, anysolid)
    start = a.clone()
    L = LG.lib()
    tp = thresh.ctypes.data_as(C.POINTER(C.c_uint32))

    def call(src, dst, step, stream):
        rc = L.lgx_step_planes_noalloc(src.data_ptr(), dst.data_ptr(), s.data_ptr(),
                                       an.data_ptr(), w, h, int(rest), inlet, tp, seed, step,
                                       C.c_void_p(stream.cuda_stream))
        assert rc == 0, L.lgx_last_error().decode()

    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        call(a, b, 0, st)
    st.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=st):
        call(a, b, 0, st)
        call(b, a, 1, st)
    for _ in range(2):
        a.copy_(start)
        b.zero_()
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        got0 = unpack(b.cpu().numpy().view(np.uint32), solid, w, h)
        got1 = unpack(a.cpu().numpy().view(np.uint32), solid, w, h)
        assert np.array_equal(got0, want[0]), "step 0 differs in %d cells" % int(
            (got0 != want[0]).sum())
        assert np.array_equal(got1, want[1]), "step 1 differs in %d cells" % int(
            (got1 != want[1]).sum())
