"""lattice_gas -- Python host mirror of the GB300 lattice-gas engine.

A ctypes binding of the C ABI in include/lgx.h (liblgx.so, built by
lattice-gas_gb300/build.py).  The names follow the reference crate
(daleobrien/lattice-gas): ``GpuLattice`` is ``lattice_gas::gpu::GpuLattice``
(src/gpu.rs:453-755) with the same methods, argument meaning and panics turned
into ``LgxError``; ``Field`` is ``render::Field``'s data; ``Batch`` and
``Server`` are the batched and served front ends.

There is no CPU fallback: if liblgx.so is missing or no CUDA device is
present, the first call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblgx.so")

__all__ = ["GpuLattice", "Lattice", "Batch", "Server", "Field", "LgxError", "lib", "thresholds", "init_equilibrium",
           "add_box", "add_circle", "shear_wave", "verify_circuit", "SQRT3_2"]

SQRT3_2 = np.float32(0.8660254)
SOLID_BIT = 0x80
REST_BIT = 0x40
STATE_MASK = 0x7F

_lock = threading.Lock()
_lib = None

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
i32p = C.POINTER(C.c_int32)
f32p = C.POINTER(C.c_float)
sz = C.c_size_t
vp = C.c_void_p


class Request(C.Structure):
    """lgx_request (include/lgx.h)."""
    _fields_ = [("w", C.c_size_t), ("h", C.c_size_t), ("rest_particles", C.c_int),
                ("seed", C.c_uint64), ("cells", C.POINTER(C.c_uint8)), ("density", C.c_float),
                ("ux", C.c_float), ("uy", C.c_float), ("inlet_cols", C.c_size_t),
                ("steps", C.c_uint64), ("sample_every", C.c_uint64), ("alpha", C.c_float),
                ("bx", C.c_size_t), ("by", C.c_size_t)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("completed", "failed", "cancelled", "active", "queued",
                                          "ticks", "kernel_launches", "site_updates",
                                          "bytes_in_use", "peak_bytes", "peak_active",
                                          "gpu_busy_ns", "host_tick_ns", "host_wait_ns")]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_CANCELLED, REQ_FAILED = range(5)


TRANSPORT_SAMPLES = 20


class Transport(C.Structure):
    """lgx_transport: transport::Transport (src/transport.rs:31-37) and its fit inputs."""
    _fields_ = [("nu", C.c_float), ("g", C.c_float), ("window_nu", C.c_uint64),
                ("window_g", C.c_uint64), ("u_actual", C.c_float),
                ("mode_nu", C.c_double * (2 * TRANSPORT_SAMPLES)),
                ("mode_g", C.c_double * (2 * TRANSPORT_SAMPLES))]


BATCH_AUTO, BATCH_PER_STEP, BATCH_RESIDENT = 0, 1, 2


class BatchClass(C.Structure):
    """lgx_batch_class: one size class of a batch and the tuner's timings."""
    _fields_ = [("words", C.c_uint32), ("lattices", C.c_uint32), ("rest", C.c_int),
                ("resident", C.c_int), ("cluster", C.c_uint32), ("threads", C.c_uint32),
                ("step_us", C.c_float), ("resident_us", C.c_float),
                ("steps_per_barrier", C.c_uint32), ("word_per_thread", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StepPlan(C.Structure):
    """lgx_step_plan: what LGX_STEP_AUTO resolves to and the tuner's times per step."""
    _fields_ = [("mode", C.c_int), ("depth", C.c_uint32), ("words", C.c_uint32),
                ("single_us", C.c_float), ("single1_us", C.c_float), ("single2_us", C.c_float),
                ("wave_us", C.c_float), ("temporal4_us", C.c_float),
                ("temporal8_us", C.c_float), ("graph_us", C.c_float),
                ("lanes2_us", C.c_float), ("lanes4_us", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LgxError(RuntimeError):
    """A C-ABI call returned a non-zero lgx_status."""

    def __init__(self, code, msg):
        super().__init__("lgx error %d: %s" % (code, msg))
        self.code = code


def _sig(L, name, *args):
    f = getattr(L, name)
    f.restype = C.c_int
    f.argtypes = list(args)


def lib():
    """Load liblgx.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError("liblgx.so is not built; run lattice-gas_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        L.lgx_last_error.restype = C.c_char_p
        L.lgx_last_error.argtypes = []
        _sig(L, "lgx_create", sz, sz, C.c_int, C.c_uint64, C.POINTER(vp))
        _sig(L, "lgx_destroy", vp)
        _sig(L, "lgx_device_name", vp, C.c_char_p, sz)
        _sig(L, "lgx_set_inlet", vp, sz, C.c_float, C.c_float, C.c_float, C.c_int)
        _sig(L, "lgx_attach_field", vp, sz, sz)
        _sig(L, "lgx_load", vp, u8p, sz)
        _sig(L, "lgx_restart", vp, u8p, sz, C.c_uint64)
        _sig(L, "lgx_store", vp, u8p, sz)
        _sig(L, "lgx_init_equilibrium", vp, C.c_float, C.c_float, C.c_float, C.c_uint64)
        _sig(L, "lgx_advance", vp, C.c_uint64)
        _sig(L, "lgx_advance_sampling", vp, C.c_uint64, C.c_uint64, C.c_float)
        _sig(L, "lgx_sample_field", vp, C.c_float)
        _sig(L, "lgx_set_step_mode", vp, C.c_int)
        _sig(L, "lgx_set_temporal_depth", vp, C.c_int)
        _sig(L, "lgx_set_step_shape", vp, C.c_int)
        _sig(L, "lgx_get_step_plan", vp, C.POINTER(StepPlan))
        _sig(L, "lgx_read_field", vp, f32p, f32p, f32p, f32p, sz)
        _sig(L, "lgx_read_block_sums", vp, i32p, i32p, i32p, i32p, sz)
        _sig(L, "lgx_total_particles", vp, C.POINTER(C.c_uint64))
        _sig(L, "lgx_row_ux", vp, f32p, sz)
        _sig(L, "lgx_field_vorticity", vp, f32p, sz)
        _sig(L, "lgx_field_mean_velocity", vp, f32p, f32p)
        _sig(L, "lgx_field_analyses", vp, f32p, sz, f32p, f32p)
        _sig(L, "lgx_mean_velocity", vp, f32p, f32p)
        _sig(L, "lgx_column_uy", vp, f32p, sz)
        _sig(L, "lgx_line_sums", vp, i32p, sz, i32p, sz)
        _sig(L, "lgx_steps", vp, C.POINTER(C.c_uint64))
        _sig(L, "lgx_stream", vp, C.POINTER(vp))
        _sig(L, "lgx_launch_count", vp, C.POINTER(C.c_uint64))
        _sig(L, "lgx_timing_mark", vp, C.c_int)
        _sig(L, "lgx_timing_elapsed", vp, C.c_int, C.c_int, C.POINTER(C.c_float))
        _sig(L, "lgx_verify_circuit", C.c_int, u32p, sz)
        _sig(L, "lgx_select_device", C.c_int)
        _sig(L, "lgx_server_create", sz, sz, C.POINTER(vp))
        _sig(L, "lgx_server_destroy", vp)
        _sig(L, "lgx_server_submit", vp, C.POINTER(Request), C.POINTER(C.c_uint64))
        _sig(L, "lgx_server_poll", vp, C.c_uint64, C.POINTER(C.c_int))
        _sig(L, "lgx_server_wait", vp, C.c_uint64, C.c_double, C.POINTER(C.c_int))
        _sig(L, "lgx_server_result", vp, C.c_uint64, f32p, f32p, f32p, f32p, i32p, i32p, i32p,
             i32p, sz, C.POINTER(C.c_uint64), C.POINTER(C.c_double))
        _sig(L, "lgx_server_cancel", vp, C.c_uint64)
        _sig(L, "lgx_server_release", vp, C.c_uint64)
        _sig(L, "lgx_server_get_stats", vp, C.POINTER(ServerStats))
        _sig(L, "lgx_server_inject_alloc_failure", vp, C.c_int)
        _sig(L, "lgx_request_device_bytes", C.POINTER(Request), C.POINTER(C.c_size_t))
        _sig(L, "lgx_step_planes_noalloc", vp, vp, vp, vp, sz, sz, C.c_int, sz, u32p,
             C.c_uint64, C.c_uint64, vp)
        _sig(L, "lgx_byte_create", sz, sz, C.c_float, C.c_float, C.c_float, sz, C.c_int, sz,
             C.c_uint64, C.POINTER(vp))
        _sig(L, "lgx_byte_destroy", vp)
        _sig(L, "lgx_byte_load", vp, u8p, sz)
        _sig(L, "lgx_byte_restart", vp, u8p, sz, C.c_uint64)
        _sig(L, "lgx_byte_store", vp, u8p, sz)
        _sig(L, "lgx_byte_init_equilibrium", vp)
        _sig(L, "lgx_byte_advance", vp, C.c_uint64)
        _sig(L, "lgx_byte_attach_field", vp, sz, sz)
        _sig(L, "lgx_byte_sample_field", vp, C.c_float)
        _sig(L, "lgx_byte_read_field", vp, f32p, f32p, f32p, f32p, sz)
        _sig(L, "lgx_byte_total_particles", vp, C.POINTER(C.c_uint64))
        _sig(L, "lgx_byte_mean_velocity", vp, C.POINTER(C.c_float), C.POINTER(C.c_float))
        _sig(L, "lgx_byte_steps", vp, C.POINTER(C.c_uint64))
        _sig(L, "lgx_batch_create", C.POINTER(vp), sz, C.POINTER(vp))
        _sig(L, "lgx_batch_create_ex", C.POINTER(vp), sz, C.c_int, C.POINTER(vp))
        _sig(L, "lgx_batch_plan", vp, C.POINTER(BatchClass), sz, C.POINTER(sz))
        _sig(L, "lgx_batch_destroy", vp)
        _sig(L, "lgx_batch_advance_sampling", vp, C.c_uint64, C.c_uint64, C.c_float)
        _sig(L, "lgx_batch_advance", vp, C.c_uint64)
        _sig(L, "lgx_batch_launch_count", vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64))
        _sig(L, "lgx_batch_timing_mark", vp, C.c_int)
        _sig(L, "lgx_batch_timing_elapsed", vp, C.c_int, C.c_int, C.POINTER(C.c_float))
        _sig(L, "lgx_probe_int_rate", C.c_int, C.POINTER(C.c_double))
        _sig(L, "lgx_transport_measure", f32p, sz, C.c_int, C.c_uint64, sz,
             C.POINTER(Transport))
        _sig(L, "lgx_host_alloc", sz, C.POINTER(vp))
        _sig(L, "lgx_host_free", vp)
        _sig(L, "lgx_equilibrium_thresholds", C.c_float, C.c_float, C.c_float, C.c_int, u32p)
        _sig(L, "lgx_cells_init_equilibrium", u8p, sz, C.c_float, C.c_float, C.c_float, C.c_int,
             C.c_uint64)
        _sig(L, "lgx_cells_add_box", u8p, sz, sz, C.c_float, C.c_float, C.c_float, C.c_float,
             C.c_int)
        _sig(L, "lgx_cells_add_circle", u8p, sz, sz, C.c_float, C.c_float, C.c_float)
        _sig(L, "lgx_cells_shear_wave", u8p, sz, sz, C.c_float, f32p, C.c_int, C.c_uint64)
        _lib = L
        return L


def _check(rc):
    if rc != 0:
        raise LgxError(rc, lib().lgx_last_error().decode(errors="replace"))


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _u64(x):
    return int(x) & (2 ** 64 - 1)


class Field:
    """The coarse-grained field's arrays (render::Field, src/render.rs:22-48)."""

    def __init__(self, w, h, bx, by):
        self.bx, self.by = bx, by
        self.bw, self.bh = w // bx, h // by
        n = self.bw * self.bh
        self.ux = np.zeros(n, np.float32)
        self.uy = np.zeros(n, np.float32)
        self.rho = np.zeros(n, np.float32)
        self.solid = np.zeros(n, np.float32)


class GpuLattice:
    """The lattice on the GPU, as bitplanes (src/gpu.rs:453-755)."""

    def __init__(self, w: int, h: int, rest_particles: bool, seed: int):
        L = lib()
        self.w, self.h = int(w), int(h)
        self.rest = bool(rest_particles)
        self._h = vp()
        _check(L.lgx_create(self.w, self.h, int(self.rest), _u64(seed), C.byref(self._h)))
        self._field = None

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().lgx_destroy(self._h)
            self._h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def device_name(self) -> str:
        buf = C.create_string_buffer(256)
        _check(lib().lgx_device_name(self._h, buf, 256))
        return buf.value.decode()

    def set_inlet(self, cols, density, inflow, rest):
        _check(lib().lgx_set_inlet(self._h, int(cols), float(density), float(inflow[0]),
                                   float(inflow[1]), int(bool(rest))))

    def attach_field(self, bx, by):
        _check(lib().lgx_attach_field(self._h, int(bx), int(by)))
        self._field = (int(bx), int(by), self.w // int(bx), self.h // int(by))

    def load(self, cells):
        c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
        _check(lib().lgx_load(self._h, _p(c, C.c_uint8), c.size))

    def restart(self, cells, seed):
        c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
        _check(lib().lgx_restart(self._h, _p(c, C.c_uint8), c.size, _u64(seed)))

    def store(self, out=None) -> np.ndarray:
        if out is None:
            out = np.zeros(self.w * self.h, np.uint8)
        _check(lib().lgx_store(self._h, _p(out, C.c_uint8), out.size))
        return out

    def vorticity(self) -> np.ndarray:
        """Field::vorticity (src/render.rs:127-143) of the attached field, on the device."""
        bx, by, bw, bh = self._field
        out = np.zeros(bw * bh, np.float32)
        _check(lib().lgx_field_vorticity(self._h, _p(out, C.c_float), out.size))
        return out

    def mean_velocity(self):
        """Field::mean_velocity (src/render.rs:146-161) of the attached field."""
        ux, uy = C.c_float(), C.c_float()
        _check(lib().lgx_field_mean_velocity(self._h, C.byref(ux), C.byref(uy)))
        return np.float32(ux.value), np.float32(uy.value)

    def field_analyses(self):
        """Field::vorticity and Field::mean_velocity together: one launch, one read-back."""
        bx, by, bw, bh = self._field
        out = np.zeros(bw * bh, np.float32)
        ux, uy = C.c_float(), C.c_float()
        _check(lib().lgx_field_analyses(self._h, _p(out, C.c_float), out.size, C.byref(ux),
                                        C.byref(uy)))
        return out, (np.float32(ux.value), np.float32(uy.value))

    def lattice_mean_velocity(self):
        """Lattice::mean_velocity (src/lattice.rs:286-294) of this lattice's cells: momentum
        per particle over every site, obstacle sites included."""
        ux, uy = C.c_float(), C.c_float()
        _check(lib().lgx_mean_velocity(self._h, C.byref(ux), C.byref(uy)))
        return np.float32(ux.value), np.float32(uy.value)

    @property
    def step_plan(self) -> dict:
        """What the default step mode resolves to for this lattice's size class."""
        p = StepPlan()
        _check(lib().lgx_get_step_plan(self._h, C.byref(p)))
        return p.as_dict()

    def row_ux(self) -> np.ndarray:
        """transport::row_ux (src/transport.rs:87-91), reduced on the device."""
        out = np.zeros(self.h, np.float32)
        _check(lib().lgx_row_ux(self._h, _p(out, C.c_float), out.size))
        return out

    def column_uy(self) -> np.ndarray:
        """transport::column_uy (src/transport.rs:51-84), reduced on the device."""
        out = np.zeros(self.w, np.float32)
        _check(lib().lgx_column_uy(self._h, _p(out, C.c_float), out.size))
        return out

    def line_sums(self):
        """Exact WITH_WALLS (mass, px2, py2) of every row ([3, h]) and column ([3, w])."""
        rows = np.zeros(3 * self.h, np.int32)
        cols = np.zeros(3 * self.w, np.int32)
        _check(lib().lgx_line_sums(self._h, _p(rows, C.c_int32), rows.size, _p(cols, C.c_int32),
                                   cols.size))
        return rows.reshape(3, self.h), cols.reshape(3, self.w)

    def init_equilibrium(self, density, inflow, seed):
        """Lattice::init_equilibrium (src/lattice.rs:197-208) on the device: fluid cells
        get equilibrium samples from Rng::new(seed ^ 0xA5A51234), obstacles stay."""
        _check(lib().lgx_init_equilibrium(self._h, float(density), float(inflow[0]),
                                          float(inflow[1]), _u64(seed)))

    def advance(self, n):
        _check(lib().lgx_advance(self._h, int(n)))

    def advance_sampling(self, n, sample_every, alpha):
        _check(lib().lgx_advance_sampling(self._h, int(n), int(sample_every), float(alpha)))

    STEP_AUTO, STEP_SINGLE, STEP_WAVE, STEP_TEMPORAL, STEP_GRAPH = 0, 1, 2, 3, 4
    SHAPE_AUTO, SHAPE_CHUNK1, SHAPE_CHUNK2, SHAPE_LANES2, SHAPE_LANES4 = 0, 1, 2, 3, 4

    def set_step_mode(self, mode: int):
        _check(lib().lgx_set_step_mode(self._h, int(mode)))

    def set_step_shape(self, shape: int):
        """Pin the single-step kernel's shape (SHAPE_*; 0: tuner / by size)."""
        _check(lib().lgx_set_step_shape(self._h, int(shape)))

    def set_temporal_depth(self, k: int):
        _check(lib().lgx_set_temporal_depth(self._h, int(k)))

    def sample_field(self, alpha):
        _check(lib().lgx_sample_field(self._h, float(alpha)))

    def read_field(self, f: Field | None = None) -> Field:
        if self._field is None:
            raise LgxError(4, "no field attached to this lattice")
        bx, by, bw, bh = self._field
        if f is None:
            f = Field(self.w, self.h, bx, by)
        if (f.bw, f.bh, f.bx, f.by) != (bw, bh, bx, by):
            raise LgxError(1, "the field on the device has a different block grid from the "
                              "one being filled")
        _check(lib().lgx_read_field(self._h, _p(f.ux, C.c_float), _p(f.uy, C.c_float),
                                    _p(f.rho, C.c_float), _p(f.solid, C.c_float), bw * bh))
        return f

    def read_block_sums(self):
        if self._field is None:
            raise LgxError(4, "no field attached to this lattice")
        _, _, bw, bh = self._field
        outs = [np.zeros(bw * bh, np.int32) for _ in range(4)]
        _check(lib().lgx_read_block_sums(self._h, *[_p(o, C.c_int32) for o in outs], bw * bh))
        return outs

    def total_particles(self) -> int:
        v = C.c_uint64()
        _check(lib().lgx_total_particles(self._h, C.byref(v)))
        return int(v.value)

    @property
    def steps(self) -> int:
        v = C.c_uint64()
        _check(lib().lgx_steps(self._h, C.byref(v)))
        return int(v.value)

    @property
    def launches(self) -> int:
        v = C.c_uint64()
        _check(lib().lgx_launch_count(self._h, C.byref(v)))
        return int(v.value)

    @property
    def stream(self) -> int:
        v = vp()
        _check(lib().lgx_stream(self._h, C.byref(v)))
        return int(v.value or 0)

    def timing_mark(self, slot):
        _check(lib().lgx_timing_mark(self._h, int(slot)))

    def timing_elapsed(self, a, b) -> float:
        ms = C.c_float()
        _check(lib().lgx_timing_elapsed(self._h, int(a), int(b), C.byref(ms)))
        return float(ms.value)


class Lattice:
    """The reference's byte-per-cell lattice (src/lattice.rs), on the device:
    the CPU path's own random stream, bands of ceil(h / threads) rows."""

    def __init__(self, w, h, density, inflow, inlet_cols, rest_particles, threads, seed):
        self.w, self.h = int(w), int(h)
        self._h = vp()
        _check(lib().lgx_byte_create(self.w, self.h, float(density), float(inflow[0]),
                                     float(inflow[1]), int(inlet_cols), int(bool(rest_particles)),
                                     int(threads), _u64(seed), C.byref(self._h)))
        self._field = None

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().lgx_byte_destroy(self._h)
            self._h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, cells):
        c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
        _check(lib().lgx_byte_load(self._h, _p(c, C.c_uint8), c.size))

    def restart(self, cells, seed):
        c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
        _check(lib().lgx_byte_restart(self._h, _p(c, C.c_uint8), c.size, _u64(seed)))

    def store(self) -> np.ndarray:
        out = np.zeros(self.w * self.h, np.uint8)
        _check(lib().lgx_byte_store(self._h, _p(out, C.c_uint8), out.size))
        return out

    def init_equilibrium(self):
        """Lattice::init_equilibrium (src/lattice.rs:197-208), on the device."""
        _check(lib().lgx_byte_init_equilibrium(self._h))

    def advance(self, n):
        _check(lib().lgx_byte_advance(self._h, int(n)))

    def attach_field(self, bx, by):
        _check(lib().lgx_byte_attach_field(self._h, int(bx), int(by)))
        self._field = (int(bx), int(by), self.w // int(bx), self.h // int(by))

    def sample_field(self, alpha):
        _check(lib().lgx_byte_sample_field(self._h, float(alpha)))

    def read_field(self) -> Field:
        bx, by, bw, bh = self._field
        f = Field(self.w, self.h, bx, by)
        _check(lib().lgx_byte_read_field(self._h, _p(f.ux, C.c_float), _p(f.uy, C.c_float),
                                         _p(f.rho, C.c_float), _p(f.solid, C.c_float), bw * bh))
        return f

    def total_particles(self) -> int:
        v = C.c_uint64()
        _check(lib().lgx_byte_total_particles(self._h, C.byref(v)))
        return int(v.value)

    def mean_velocity(self):
        """Lattice::mean_velocity (src/lattice.rs:286-294), on the device."""
        ux, uy = C.c_float(), C.c_float()
        _check(lib().lgx_byte_mean_velocity(self._h, C.byref(ux), C.byref(uy)))
        return np.float32(ux.value), np.float32(uy.value)

    @property
    def steps(self) -> int:
        v = C.c_uint64()
        _check(lib().lgx_byte_steps(self._h, C.byref(v)))
        return int(v.value)


class Batch:
    """Many lattices advanced together: one launch per step for all of them,
    each sampling interval a replayed CUDA graph.  The lattices stay owned by
    the caller; advance them only through the batch while it is alive."""

    def __init__(self, lattices, policy=BATCH_AUTO):
        self.lattices = list(lattices)
        arr = (vp * len(self.lattices))(*[l.handle.value for l in self.lattices])
        self._h = vp()
        _check(lib().lgx_batch_create_ex(arr, len(self.lattices), int(policy),
                                         C.byref(self._h)))

    @property
    def plan(self):
        """The size classes of the batch's small lattices, as the tuner planned them."""
        n = C.c_size_t()
        _check(lib().lgx_batch_plan(self._h, None, 0, C.byref(n)))
        out = (BatchClass * max(n.value, 1))()
        _check(lib().lgx_batch_plan(self._h, out, n.value, C.byref(n)))
        return [out[i].as_dict() for i in range(n.value)]

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().lgx_batch_destroy(self._h)
            self._h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def advance(self, n):
        _check(lib().lgx_batch_advance(self._h, int(n)))

    def advance_sampling(self, n, sample_every, alpha):
        _check(lib().lgx_batch_advance_sampling(self._h, int(n), int(sample_every),
                                                float(alpha)))

    @property
    def launches(self):
        k, g = C.c_uint64(), C.c_uint64()
        _check(lib().lgx_batch_launch_count(self._h, C.byref(k), C.byref(g)))
        return int(k.value), int(g.value)

    def timing_mark(self, slot):
        _check(lib().lgx_batch_timing_mark(self._h, int(slot)))

    def timing_elapsed(self, a, b) -> float:
        ms = C.c_float()
        _check(lib().lgx_batch_timing_elapsed(self._h, int(a), int(b), C.byref(ms)))
        return float(ms.value)


class Server:
    """A request loop with continuous batching (lgx_server_*).  Requests are
    admitted against a device-memory budget, resident lattices advance
    together, and only the moments come back."""

    def __init__(self, budget_bytes: int, max_active: int = 256):
        self._h = vp()
        _check(lib().lgx_server_create(int(budget_bytes), int(max_active), C.byref(self._h)))
        self._shape = {}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().lgx_server_destroy(self._h)
            self._h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, cells, w, h, rest, seed, density, inflow, inlet_cols, steps, sample_every,
               alpha, bx, by) -> int:
        c = np.ascontiguousarray(cells, dtype=np.uint8).reshape(-1)
        q = Request(w, h, int(bool(rest)), _u64(seed), _p(c, C.c_uint8), float(density),
                    float(inflow[0]), float(inflow[1]), int(inlet_cols), int(steps),
                    int(sample_every), float(alpha), int(bx), int(by))
        rid = C.c_uint64()
        _check(lib().lgx_server_submit(self._h, C.byref(q), C.byref(rid)))
        self._shape[int(rid.value)] = (w // bx) * (h // by)
        return int(rid.value)

    def submit_workload(self, wl) -> int:
        return self.submit(wl.cells, wl.w, wl.h, wl.rest, wl.seed, wl.density, wl.inflow,
                           wl.inlet_cols, wl.steps, wl.sample_every, wl.alpha, wl.block, wl.block)

    def poll(self, rid) -> int:
        st = C.c_int()
        _check(lib().lgx_server_poll(self._h, int(rid), C.byref(st)))
        return st.value

    def wait(self, rid, timeout=-1.0) -> int:
        st = C.c_int()
        _check(lib().lgx_server_wait(self._h, int(rid), float(timeout), C.byref(st)))
        return st.value

    def result(self, rid) -> dict:
        nb = self._shape[int(rid)]
        f = [np.zeros(nb, np.float32) for _ in range(4)]
        m = [np.zeros(nb, np.int32) for _ in range(4)]
        part = C.c_uint64()
        lat = C.c_double()
        _check(lib().lgx_server_result(self._h, int(rid), *[_p(a, C.c_float) for a in f],
                                       *[_p(a, C.c_int32) for a in m], nb, C.byref(part),
                                       C.byref(lat)))
        return dict(ux=f[0], uy=f[1], rho=f[2], solid=f[3], mass=m[0], px2=m[1], py2=m[2],
                    nsolid=m[3], particles=int(part.value), latency=float(lat.value))

    def cancel(self, rid):
        _check(lib().lgx_server_cancel(self._h, int(rid)))

    def release(self, rid):
        _check(lib().lgx_server_release(self._h, int(rid)))
        self._shape.pop(int(rid), None)

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().lgx_server_get_stats(self._h, C.byref(st)))
        return {n: int(getattr(st, n)) for n, _ in ServerStats._fields_}

    @staticmethod
    def request_bytes(wl) -> int:
        """Device memory the workload occupies while resident."""
        q = Request(wl.w, wl.h, int(bool(wl.rest)), 0, None, 0.0, 0.0, 0.0, int(wl.inlet_cols),
                    int(wl.steps), int(wl.sample_every), 1.0, int(wl.block), int(wl.block))
        out = C.c_size_t()
        _check(lib().lgx_request_device_bytes(C.byref(q), C.byref(out)))
        return int(out.value)

    def inject_alloc_failure(self, count: int):
        _check(lib().lgx_server_inject_alloc_failure(self._h, int(count)))


# ---- host-side setup (src/lattice.rs, src/hex.rs, src/transport.rs) --------

def thresholds(density, ux, uy, rest):
    out = np.zeros(7, np.uint32)
    _check(lib().lgx_equilibrium_thresholds(float(density), float(ux), float(uy), int(bool(rest)),
                                            _p(out, C.c_uint32)))
    return out


def init_equilibrium(cells, density, ux, uy, rest, seed):
    """Lattice::init_equilibrium on a byte array (in place; returns it)."""
    assert cells.dtype == np.uint8 and cells.flags["C_CONTIGUOUS"]
    _check(lib().lgx_cells_init_equilibrium(_p(cells, C.c_uint8), cells.size, float(density),
                                            float(ux), float(uy), int(bool(rest)), _u64(seed)))
    return cells


def add_box(cells, w, h, x0, x1, y0, y1, strict=False):
    _check(lib().lgx_cells_add_box(_p(cells, C.c_uint8), w, h, float(x0), float(x1), float(y0),
                                   float(y1), int(bool(strict))))
    return cells


def add_circle(cells, w, h, cx, cy, r):
    _check(lib().lgx_cells_add_circle(_p(cells, C.c_uint8), w, h, float(cx), float(cy), float(r)))
    return cells


def shear_wave(w, h, density, ux_row, rest, rng_seed):
    cells = np.zeros(w * h, np.uint8)
    u = np.ascontiguousarray(ux_row, dtype=np.float32)
    _check(lib().lgx_cells_shear_wave(_p(cells, C.c_uint8), w, h, float(density),
                                      _p(u, C.c_float), int(bool(rest)), _u64(rng_seed)))
    return cells


def probe_int_rate(op: int) -> float:
    """Measured integer throughput (instructions/s) for op 0 lop3, 1 imad, 2 shf, 3 add."""
    v = C.c_double()
    _check(lib().lgx_probe_int_rate(int(op), C.byref(v)))
    return float(v.value)


def select_device(ordinal: int):
    _check(lib().lgx_select_device(int(ordinal)))


class PinnedBuffer:
    """A page-locked host buffer viewed as a numpy array."""

    def __init__(self, nbytes: int, dtype=np.uint8):
        self._p = vp()
        _check(lib().lgx_host_alloc(int(nbytes), C.byref(self._p)))
        self.nbytes = int(nbytes)
        buf = (C.c_uint8 * max(self.nbytes, 1)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=np.uint8)[:self.nbytes].view(dtype)

    def free(self):
        if self._p and self._p.value:
            lib().lgx_host_free(self._p)
            self._p = vp()
            self.array = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def verify_circuit(rest) -> np.ndarray:
    n = 48 * (128 if rest else 64)
    out = np.zeros(n, np.uint32)
    _check(lib().lgx_verify_circuit(int(bool(rest)), _p(out, C.c_uint32), n))
    return out


def transport_measure(densities, rest=True, seed=0x5EED, size=256):
    """transport::measure on the device for each density (src/transport.rs:291-319).
    Returns a list of Transport records (nu, g, windows, averaged modes)."""
    d = np.ascontiguousarray(np.atleast_1d(densities), dtype=np.float32)
    out = (Transport * d.size)()
    _check(lib().lgx_transport_measure(_p(d, C.c_float), d.size, int(bool(rest)), _u64(seed),
                                       int(size), out))
    return list(out)
