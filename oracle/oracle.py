"""ctypes binding for the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a plain-C restatement of the reference (daleobrien/lattice-gas):
the byte-per-cell CPU path (src/lattice.rs et al.) and the bitplane path the
Metal shader runs (src/gpu.rs).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use this module; the product library never does.

``build()`` compiles ``oracle/_build/liboracle.so`` with make; ``lib()`` loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lock = threading.Lock()
_lib = None

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f32p = C.POINTER(C.c_float)
sz = C.c_size_t


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


class TransportResult(C.Structure):
    """lgo_transport: transport::Transport and the inputs of its fits."""
    _fields_ = [("nu", C.c_float), ("g", C.c_float), ("window_nu", C.c_uint64),
                ("window_g", C.c_uint64), ("u_actual", C.c_float),
                ("mode_nu", C.c_double * 40), ("mode_g", C.c_double * 40)]


def _sig(lib, name, res, *args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = list(args)


def lib():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        build()
        L = C.CDLL(LIB_PATH)
        _sig(L, "lgo_reverse", C.c_uint8, C.c_uint8)
        _sig(L, "lgo_site_position", None, sz, sz, f32p, f32p)
        _sig(L, "lgo_classes", C.c_int, C.c_int, C.POINTER(C.c_int), u8p)
        _sig(L, "lgo_table_stride", C.c_int, C.c_int)
        _sig(L, "lgo_table_apply", C.c_uint8, C.c_int, C.c_uint8, C.c_uint32)
        _sig(L, "lgo_rng_seed", C.c_uint64, C.c_uint64)
        _sig(L, "lgo_rng_draws", None, C.c_uint64, u64p, sz)
        _sig(L, "lgo_threshold", C.c_uint32, C.c_float)
        _sig(L, "lgo_equilibrium_thresholds", None, C.c_float, C.c_float, C.c_float, C.c_int, u32p)
        _sig(L, "lgo_equilibrium_samples", None, C.c_float, C.c_float, C.c_float, C.c_int,
             C.c_uint64, u8p, sz)
        _sig(L, "lgo_new", C.c_void_p, sz, sz, C.c_float, C.c_float, C.c_float, sz, C.c_int, sz,
             C.c_uint64)
        _sig(L, "lgo_free", None, C.c_void_p)
        _sig(L, "lgo_cells", u8p, C.c_void_p)
        _sig(L, "lgo_steps", C.c_uint64, C.c_void_p)
        _sig(L, "lgo_restart", None, C.c_void_p, u8p, C.c_uint64)
        _sig(L, "lgo_init_equilibrium", None, C.c_void_p)
        _sig(L, "lgo_advance", None, C.c_void_p, C.c_uint64)
        _sig(L, "lgo_total_particles", C.c_uint64, C.c_void_p)
        _sig(L, "lgo_mean_velocity", None, C.c_void_p, f32p, f32p)
        _sig(L, "lgo_add_box", None, u8p, sz, sz, C.c_float, C.c_float, C.c_float, C.c_float,
             C.c_int)
        _sig(L, "lgo_add_circle", None, u8p, sz, sz, C.c_float, C.c_float, C.c_float)
        _sig(L, "lgo_cells_init_equilibrium", None, u8p, sz, C.c_float, C.c_float, C.c_float,
             C.c_int, C.c_uint64)
        _sig(L, "lgo_cells_shear_wave", None, u8p, sz, sz, C.c_float, f32p, C.c_int, C.c_uint64)
        _sig(L, "lgo_cells_column_wave", None, u8p, sz, sz, C.c_float, C.c_float, f32p, C.c_int,
             C.c_uint64)
        _sig(L, "lgo_row_ux", None, u8p, sz, sz, f32p)
        _sig(L, "lgo_field_vorticity", None, f32p, f32p, sz, sz, sz, sz, f32p)
        _sig(L, "lgo_field_mean_velocity", None, f32p, f32p, f32p, sz, f32p, f32p)
        _sig(L, "lgo_column_uy", None, u8p, sz, sz, f32p)
        _sig(L, "lgo_transport_measure", None, C.c_float, C.c_int, sz, C.c_uint64, sz, C.c_int,
             C.POINTER(TransportResult))
        _sig(L, "lgo_moments_sum", None, u8p, sz, C.c_int, i64p)
        _sig(L, "lgo_invariants", None, u8p, sz, i64p)
        _sig(L, "lgo_field_sample", None, u8p, sz, sz, sz, sz, C.c_float, f32p, f32p, f32p, f32p)
        _sig(L, "lgo_block_sums", None, u8p, sz, sz, sz, sz, i32p, i32p, i32p, i32p)
        _sig(L, "lgo_fnv1a", C.c_uint64, u8p, sz)
        _sig(L, "lgo_mix", C.c_uint32, C.c_uint32)
        _sig(L, "lgo_draws", None, C.c_uint32, u32p)
        _sig(L, "lgo_collide_lane", C.c_uint8, C.c_int, C.c_uint8, C.c_int, C.c_int, C.c_int)
        _sig(L, "lgo_collide_word", None, C.c_int, u32p, u32p, u32p)
        _sig(L, "lgo_bp_params", None, sz, sz, C.c_uint64, C.c_uint64, sz, u32p, u32p)
        _sig(L, "lgo_bp_new", C.c_void_p, sz, sz, C.c_int, C.c_uint64, sz)
        _sig(L, "lgo_bp_free", None, C.c_void_p)
        _sig(L, "lgo_bp_set_inlet", None, C.c_void_p, sz, C.c_float, C.c_float, C.c_float, C.c_int)
        _sig(L, "lgo_bp_attach_field", None, C.c_void_p, sz, sz)
        _sig(L, "lgo_bp_load", None, C.c_void_p, u8p)
        _sig(L, "lgo_bp_restart", None, C.c_void_p, u8p, C.c_uint64)
        _sig(L, "lgo_bp_store", None, C.c_void_p, u8p)
        _sig(L, "lgo_bp_advance_sampling", None, C.c_void_p, C.c_uint64, C.c_uint64, C.c_float)
        _sig(L, "lgo_bp_sample_field", None, C.c_void_p, C.c_float)
        _sig(L, "lgo_bp_read_field", None, C.c_void_p, f32p, f32p, f32p, f32p)
        _sig(L, "lgo_bp_read_block_sums", None, C.c_void_p, i32p, i32p, i32p, i32p)
        _sig(L, "lgo_bp_total_particles", C.c_uint64, C.c_void_p)
        _sig(L, "lgo_bp_steps", C.c_uint64, C.c_void_p)
        _sig(L, "lgo_bp_planes", u32p, C.c_void_p)
        _sig(L, "lgo_bp_set_steps", None, C.c_void_p, C.c_uint64)
        _sig(L, "lgo_bp_advance_window", None, C.c_void_p, C.c_uint64, sz, sz)
        _sig(L, "lgo_bp_store_rows", None, C.c_void_p, sz, sz, u8p)
        _lib = L
        return L


def ptr(a: np.ndarray, ct):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ct))


# ---------------------------------------------------------------------------
# Thin Python mirrors of the reference's types, over the C oracle.
# ---------------------------------------------------------------------------

SQRT3_2 = np.float32(0.8660254)
SOLID_BIT = 0x80
REST_BIT = 0x40
STATE_MASK = 0x7F
MOVING_MASK = 0x3F
CX2 = (2, 1, -1, -2, -1, 1)
CY2 = (0, 1, 1, 0, -1, -1)


class Lattice:
    """Byte-per-cell CPU lattice (src/lattice.rs:8-314)."""

    def __init__(self, w, h, density, inflow, inlet_cols, rest, threads, seed):
        L = lib()
        self.w, self.h = w, h
        self.rest = bool(rest)
        self.density = float(density)
        self.inflow = (float(inflow[0]), float(inflow[1]))
        self.inlet_cols = inlet_cols
        self._p = L.lgo_new(w, h, density, inflow[0], inflow[1], inlet_cols, int(rest),
                            threads, seed & (2**64 - 1))
        if not self._p:
            raise ValueError("lattice must have even h, w > 4, h > 4")

    def __del__(self):
        p = getattr(self, "_p", None)
        if p:
            lib().lgo_free(p)
            self._p = None

    @property
    def cells(self) -> np.ndarray:
        """A live numpy view of the cell bytes (changes as the lattice steps)."""
        ptr_ = lib().lgo_cells(self._p)
        return np.ctypeslib.as_array(ptr_, shape=(self.w * self.h,))

    def set_cells(self, cells: np.ndarray):
        self.cells[:] = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)

    @property
    def steps(self) -> int:
        return int(lib().lgo_steps(self._p))

    def restart(self, cells, seed):
        c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
        lib().lgo_restart(self._p, ptr(c, C.c_uint8), seed & (2**64 - 1))

    def init_equilibrium(self):
        lib().lgo_init_equilibrium(self._p)

    def add_box(self, x0, x1, y0, y1, strict=False):
        c = self.cells
        lib().lgo_add_box(c.ctypes.data_as(u8p), self.w, self.h, x0, x1, y0, y1, int(strict))

    def add_circle(self, cx, cy, r):
        c = self.cells
        lib().lgo_add_circle(c.ctypes.data_as(u8p), self.w, self.h, cx, cy, r)

    def advance(self, n):
        lib().lgo_advance(self._p, n)

    def total_particles(self) -> int:
        return int(lib().lgo_total_particles(self._p))

    def mean_velocity(self):
        a, b = C.c_float(), C.c_float()
        lib().lgo_mean_velocity(self._p, C.byref(a), C.byref(b))
        return a.value, b.value


class Field:
    """Coarse-grained field (src/render.rs:22-120)."""

    def __init__(self, w, h, bx, by):
        self.bx, self.by = bx, by
        self.bw, self.bh = w // bx, h // by
        n = self.bw * self.bh
        self.ux = np.zeros(n, np.float32)
        self.uy = np.zeros(n, np.float32)
        self.rho = np.zeros(n, np.float32)
        self.solid = np.zeros(n, np.float32)

    def sample(self, cells: np.ndarray, w: int, h: int, alpha: float):
        assert self.bx * self.by <= 65535 // 8, "block exceeds moments::MAX_BLOCK"
        c = np.ascontiguousarray(cells, dtype=np.uint8)
        lib().lgo_field_sample(ptr(c, C.c_uint8), w, h, self.bx, self.by, alpha,
                               ptr(self.ux, C.c_float), ptr(self.uy, C.c_float),
                               ptr(self.rho, C.c_float), ptr(self.solid, C.c_float))

    def checksum_bytes(self) -> bytes:
        return b"".join(a.astype("<f4").tobytes() for a in (self.ux, self.uy, self.rho, self.solid))


def fnv1a(data) -> int:
    b = np.frombuffer(bytes(data), dtype=np.uint8) if not isinstance(data, np.ndarray) else \
        np.ascontiguousarray(data, dtype=np.uint8).reshape(-1)
    return int(lib().lgo_fnv1a(ptr(b, C.c_uint8), b.size))


def invariants(cells: np.ndarray):
    c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
    out = np.zeros(3, np.int64)
    lib().lgo_invariants(ptr(c, C.c_uint8), c.size, ptr(out, C.c_int64))
    return tuple(int(v) for v in out)


def block_sums(cells, w, h, bx, by):
    bw, bh = w // bx, h // by
    c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
    outs = [np.zeros(bw * bh, np.int32) for _ in range(4)]
    lib().lgo_block_sums(ptr(c, C.c_uint8), w, h, bx, by, *[ptr(o, C.c_int32) for o in outs])
    return outs


def thresholds(density, ux, uy, rest):
    out = np.zeros(7, np.uint32)
    lib().lgo_equilibrium_thresholds(density, ux, uy, int(rest), ptr(out, C.c_uint32))
    return out


def classes(rest):
    sizes = (C.c_int * 128)()
    members = (C.c_uint8 * 128)()
    nc = lib().lgo_classes(int(rest), sizes, members)
    out, pos = [], 0
    for c in range(nc):
        out.append([members[pos + i] for i in range(sizes[c])])
        pos += sizes[c]
    return out


def init_equilibrium_cells(cells, density, ux, uy, rest, seed):
    c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1).copy()
    lib().lgo_cells_init_equilibrium(ptr(c, C.c_uint8), c.size, density, ux, uy, int(rest),
                                     seed & (2**64 - 1))
    return c


def shear_wave_cells(w, h, density, ux_row, rest, rng_seed):
    c = np.zeros(w * h, np.uint8)
    u = np.ascontiguousarray(ux_row, dtype=np.float32)
    lib().lgo_cells_shear_wave(ptr(c, C.c_uint8), w, h, density, ptr(u, C.c_float), int(rest),
                               rng_seed & (2**64 - 1))
    return c


class BitplaneLattice:
    """CPU restatement of GpuLattice (src/gpu.rs:453-755)."""

    def __init__(self, w, h, rest, seed, threads=1):
        self.w, self.h = w, h
        self._p = lib().lgo_bp_new(w, h, int(rest), seed & (2**64 - 1), threads)
        if not self._p:
            raise ValueError("lattice must have even h, w > 4, h > 4")
        self.field_shape = None

    def __del__(self):
        p = getattr(self, "_p", None)
        if p:
            lib().lgo_bp_free(p)
            self._p = None

    def set_inlet(self, cols, density, inflow, rest):
        lib().lgo_bp_set_inlet(self._p, cols, density, inflow[0], inflow[1], int(rest))

    def attach_field(self, bx, by):
        lib().lgo_bp_attach_field(self._p, bx, by)
        self.field_shape = (self.w // bx, self.h // by)

    def load(self, cells):
        c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
        assert c.size == self.w * self.h
        lib().lgo_bp_load(self._p, ptr(c, C.c_uint8))

    def restart(self, cells, seed):
        c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
        lib().lgo_bp_restart(self._p, ptr(c, C.c_uint8), seed & (2**64 - 1))

    def store(self) -> np.ndarray:
        out = np.zeros(self.w * self.h, np.uint8)
        lib().lgo_bp_store(self._p, ptr(out, C.c_uint8))
        return out

    def advance(self, n):
        lib().lgo_bp_advance_sampling(self._p, n, 0, 0.0)

    def advance_sampling(self, n, every, alpha):
        lib().lgo_bp_advance_sampling(self._p, n, every, alpha)

    def sample_field(self, alpha):
        lib().lgo_bp_sample_field(self._p, alpha)

    def read_field(self):
        bw, bh = self.field_shape
        outs = [np.zeros(bw * bh, np.float32) for _ in range(4)]
        lib().lgo_bp_read_field(self._p, *[ptr(o, C.c_float) for o in outs])
        return outs

    def read_block_sums(self):
        bw, bh = self.field_shape
        outs = [np.zeros(bw * bh, np.int32) for _ in range(4)]
        lib().lgo_bp_read_block_sums(self._p, *[ptr(o, C.c_int32) for o in outs])
        return outs

    def total_particles(self) -> int:
        return int(lib().lgo_bp_total_particles(self._p))

    @property
    def steps(self) -> int:
        return int(lib().lgo_bp_steps(self._p))

    def planes(self) -> np.ndarray:
        wpr = (self.w + 31) // 32
        p = lib().lgo_bp_planes(self._p)
        return np.ctypeslib.as_array(p, shape=(7 * wpr * self.h,)).copy()

    def set_steps(self, steps):
        """Continue the random stream of a run that has taken `steps` steps."""
        lib().lgo_bp_set_steps(self._p, int(steps))

    def advance_window(self, n, y0, y1):
        """n steps, exact on rows y0 .. y1-1 only (see lgo_bp_advance_window)."""
        assert y1 - y0 + 2 * n <= self.h
        lib().lgo_bp_advance_window(self._p, int(n), int(y0), int(y1))

    def store_rows(self, y0, y1) -> np.ndarray:
        out = np.zeros((y1 - y0) * self.w, np.uint8)
        lib().lgo_bp_store_rows(self._p, int(y0), int(y1), ptr(out, C.c_uint8))
        return out


def column_wave_cells(w, h, density, u0, uy_col, rest, rng_seed):
    """Transverse-wave start (src/transport.rs:237-251)."""
    c = np.zeros(w * h, np.uint8)
    u = np.ascontiguousarray(uy_col, dtype=np.float32)
    lib().lgo_cells_column_wave(ptr(c, C.c_uint8), w, h, density, u0, ptr(u, C.c_float),
                                int(rest), rng_seed & (2**64 - 1))
    return c


def row_ux(cells, w, h):
    """transport::row_ux (src/transport.rs:87-91)."""
    c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
    out = np.zeros(h, np.float32)
    lib().lgo_row_ux(ptr(c, C.c_uint8), w, h, ptr(out, C.c_float))
    return out


def column_uy(cells, w, h):
    """transport::column_uy (src/transport.rs:51-84)."""
    c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
    out = np.zeros(w, np.float32)
    lib().lgo_column_uy(ptr(c, C.c_uint8), w, h, ptr(out, C.c_float))
    return out


def transport_measure(density, rest, threads, seed, size, gpu):
    """transport::measure (src/transport.rs:291-319) on the byte path (gpu=False) or the
    bitplane path (gpu=True)."""
    r = TransportResult()
    lib().lgo_transport_measure(float(density), int(bool(rest)), int(threads),
                                seed & (2**64 - 1), int(size), int(bool(gpu)), C.byref(r))
    return r


def field_vorticity(ux, uy, bw, bh, bx, by):
    """Field::vorticity (src/render.rs:127-143)."""
    a = np.ascontiguousarray(ux, dtype=np.float32)
    b = np.ascontiguousarray(uy, dtype=np.float32)
    out = np.zeros(bw * bh, np.float32)
    lib().lgo_field_vorticity(ptr(a, C.c_float), ptr(b, C.c_float), bw, bh, bx, by,
                              ptr(out, C.c_float))
    return out


def field_mean_velocity(ux, uy, sol):
    """Field::mean_velocity (src/render.rs:146-161)."""
    a = np.ascontiguousarray(ux, dtype=np.float32)
    b = np.ascontiguousarray(uy, dtype=np.float32)
    c = np.ascontiguousarray(sol, dtype=np.float32)
    mx, my = C.c_float(), C.c_float()
    lib().lgo_field_mean_velocity(ptr(a, C.c_float), ptr(b, C.c_float), ptr(c, C.c_float), a.size,
                                  C.byref(mx), C.byref(my))
    return np.float32(mx.value), np.float32(my.value)


def wake_run_cells(w=4096, h=2304, density=0.3, speed=0.2, seed=0x5EED):
    """The wake run's starting cells built with the oracle's own setup: a plate one
    eighth of the channel height at x = w/8, four columns thick (src/main.rs:582-588,
    add_solid with a box on site_position), walls as solid rows 0 and h-1, then
    Lattice::init_equilibrium (src/lattice.rs:197-208).  The same cells as the
    engine's workload builder makes, for the CPU arm that must not load the engine."""
    F = np.float32
    cells = np.zeros(w * h, np.uint8)
    yc = F(h) * SQRT3_2 / F(2.0)
    half = F(h) * SQRT3_2 / F(16.0)
    x0 = F(w // 8)
    lib().lgo_add_box(ptr(cells, C.c_uint8), w, h, x0, x0 + F(4.0), yc - half, yc + half, 0)
    cells[:w] = SOLID_BIT
    cells[(h - 1) * w:] = SOLID_BIT
    lib().lgo_cells_init_equilibrium(ptr(cells, C.c_uint8), cells.size, density, speed, 0.0, 1,
                                     seed & (2**64 - 1))
    return cells
