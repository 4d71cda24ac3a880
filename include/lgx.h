/*
 * lgx.h -- C ABI of the GB300 FHP lattice-gas engine.
 *
 * Drop-in for the reference's bitplane lattice, `GpuLattice` in src/gpu.rs
 * (daleobrien/lattice-gas), which the reference drives through `Sim`
 * (src/sim.rs:35-174).  Every function returns an lgx_status (0 = success);
 * on failure lgx_last_error() describes the error for the calling thread.  No
 * C++ exception crosses this boundary.  A handle is used from one host thread
 * at a time; each lattice owns one CUDA stream on the device that was current
 * when it was created, and every call that the reference makes blocking
 * (advance, load, store, read_field, total_particles) is blocking here too.
 *
 * Cell bytes follow src/hex.rs: bits 0-5 the six directions (0 = east, then
 * counter-clockwise), bit 6 the rest particle, bit 7 the obstacle flag.
 * Rows are w cells, row-major, h rows; h even, w > 4, h > 4.
 */
#ifndef LGX_H
#define LGX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  LGX_OK = 0,
  LGX_ERR_ARG = 1,       /* size or argument mismatch (the reference asserts) */
  LGX_ERR_CUDA = 2,      /* a CUDA call failed */
  LGX_ERR_NO_DEVICE = 3, /* no CUDA device (the reference: "no Metal device") */
  LGX_ERR_STATE = 4,     /* e.g. reading a field that was never attached */
  LGX_ERR_ALLOC = 5,     /* device or host allocation failed */
  LGX_ERR_BUSY = 6       /* server: over budget or queue full */
} lgx_status;

typedef struct lgx_lattice lgx_lattice;

/* Last error message of the calling thread ("" if none). */
const char *lgx_last_error(void);

/* ---- the lattice (replaces GpuLattice, src/gpu.rs:453-755) -------------- */

/* Make `ordinal` the device that later lgx_create calls on this thread use
 * (the reference takes the system default Metal device, src/metal.rs:121). */
int lgx_select_device(int ordinal);
/* Page-locked host buffers, so load/store/read_field copies are true DMA. */
int lgx_host_alloc(size_t bytes, void **out);
int lgx_host_free(void *p);

/* GpuLattice::new (src/gpu.rs:479-515): 7 bitplanes x 2 (ping-pong), solid
 * plane, anysolid summary.  rest_particles selects the FHP-III rule. */
int lgx_create(size_t w, size_t h, int rest_particles, uint64_t seed, lgx_lattice **out);
/* Drop of GpuLattice: frees every device buffer and the stream. */
int lgx_destroy(lgx_lattice *lat);
/* GpuLattice::device_name (src/gpu.rs:517-519). */
int lgx_device_name(lgx_lattice *lat, char *buf, size_t len);
/* GpuLattice::set_inlet (src/gpu.rs:525-528): re-seed the leftmost `cols`
 * columns from Equilibrium(density, (ux, uy), rest) every step. */
int lgx_set_inlet(lgx_lattice *lat, size_t cols, float density, float ux, float uy,
                  int rest_particles);
/* GpuLattice::attach_field (src/gpu.rs:532-545): a (w/bx) x (h/by) block field
 * on the device, zero-initialised. */
int lgx_attach_field(lgx_lattice *lat, size_t bx, size_t by);
/* GpuLattice::load (src/gpu.rs:572-610): n must be w*h. */
int lgx_load(lgx_lattice *lat, const uint8_t *cells, size_t n);
/* GpuLattice::restart (src/gpu.rs:616-620): load, then seed = seed, steps = 0. */
int lgx_restart(lgx_lattice *lat, const uint8_t *cells, size_t n, uint64_t seed);
/* Lattice::init_equilibrium (src/lattice.rs:197-208) applied to the lattice on the
 * device, for callers that today run it on the host and then GpuLattice::load:
 * every fluid cell gets an equilibrium sample for (density, ux, uy) from
 * Rng::new(seed ^ 0xA5A51234), in row-major cell order; obstacles keep no
 * particles.  The result equals init_equilibrium on the stored cells followed by
 * lgx_load.  seed is the host Lattice's seed; steps are unchanged. */
int lgx_init_equilibrium(lgx_lattice *lat, float density, float ux, float uy, uint64_t seed);
/* GpuLattice::store (src/gpu.rs:630-652): n must be w*h. */
int lgx_store(lgx_lattice *lat, uint8_t *cells, size_t n);
/* GpuLattice::advance (src/gpu.rs:657-659). */
int lgx_advance(lgx_lattice *lat, uint64_t n);
/* GpuLattice::advance_sampling (src/gpu.rs:668-706): n steps, folding the
 * lattice into the attached field every sample_every steps and after the last
 * one; sample_every == 0 never samples. */
int lgx_advance_sampling(lgx_lattice *lat, uint64_t n, uint64_t sample_every, float alpha);
/* How steps are launched.  SINGLE launches one kernel per step, as the
 * reference dispatches one lgca_step per step, with programmatic dependent
 * launch so each step's state-independent draws overlap the previous step's
 * tail.  WAVE runs up to 128 steps per cooperative launch of a persistent
 * kernel (each block owns a fixed range of words and waits, with a bounded
 * spin, only for the blocks owning the rows next to its own).  TEMPORAL: see
 * lgx_set_temporal_depth.  GRAPH runs advances of 8 steps or more, sampling
 * every 16 steps or less often, as a batch of this lattice alone (lgx_batch_*;
 * other advances take SINGLE's path): intervals replayed from captured CUDA
 * graphs, or the resident kernel for a small lattice, on the lattice's own
 * stream; for lattices that do not fill the GPU, where one launch per step
 * is bound by the host's launch rate.  AUTO (default) uses whichever of
 * SINGLE, WAVE, TEMPORAL with depth 4 or 8 and (below one full wave of step
 * blocks) GRAPH a tuner measured fastest for the lattice's size class (timed
 * on a scratch lattice of the same shape at its first advance, cached for the
 * process; lgx_get_step_plan).  Results are identical in every mode. */
enum {
  LGX_STEP_AUTO = 0,
  LGX_STEP_SINGLE = 1,
  LGX_STEP_WAVE = 2,
  LGX_STEP_TEMPORAL = 3,
  LGX_STEP_GRAPH = 4
};
int lgx_set_step_mode(lgx_lattice *lat, int mode);
/* TEMPORAL: runs of k steps (k = 4 or 8, lgx_set_temporal_depth) in one pass
 * over HBM, the intermediate steps kept in registers (lattices at least 64
 * words wide; other runs, and steps up to a sampling point, go one at a time). */
int lgx_set_temporal_depth(lgx_lattice *lat, int k);
/* Pins the single-step kernel's shape (no counterpart in the reference, whose
 * lgca_step has one, src/gpu.rs:203-310).  0: the step-mode tuner's choice (or,
 * outside AUTO, by size).  1, 2: a word per lane, one or two 32-word chunks per
 * warp.  3, 4: two or four consecutive words per lane in 64- or 128-bit loads
 * and stores, for lattices whose words per row are a multiple of that count
 * (otherwise the shape by size runs).  Results are identical in every shape. */
enum {
  LGX_SHAPE_AUTO = 0,
  LGX_SHAPE_CHUNK1 = 1,
  LGX_SHAPE_CHUNK2 = 2,
  LGX_SHAPE_LANES2 = 3,
  LGX_SHAPE_LANES4 = 4
};
int lgx_set_step_shape(lgx_lattice *lat, int shape);
/* What AUTO resolves to for this lattice, and the tuner's times per step (0 where a
 * mode does not apply); tunes the size class now if it has not been. */
typedef struct lgx_step_plan {
  int mode;
  uint32_t depth;
  uint32_t words;          /* the single-step kernel's shape (LGX_SHAPE_*) */
  float single_us;         /* one launch per step, with that shape */
  float single1_us, single2_us;  /* one launch per step, one and two chunks per warp */
  float wave_us, temporal4_us, temporal8_us;
  float graph_us;          /* the one-lattice batch (GRAPH) */
  float lanes2_us, lanes4_us;  /* one launch per step, two and four words per lane */
} lgx_step_plan;
int lgx_get_step_plan(lgx_lattice *lat, lgx_step_plan *out);
/* GpuLattice::sample_field (src/gpu.rs:710-721). */
int lgx_sample_field(lgx_lattice *lat, float alpha);
/* GpuLattice::read_field (src/gpu.rs:725-736): n_blocks must be bw*bh. */
int lgx_read_field(lgx_lattice *lat, float *ux, float *uy, float *rho, float *sol,
                   size_t n_blocks);
/* Field::vorticity (src/render.rs:127-143) of the attached field, on the device:
 * n_blocks must be bw*bh. */
int lgx_field_vorticity(lgx_lattice *lat, float *w, size_t n_blocks);
/* Field::mean_velocity (src/render.rs:146-161): the mean of the blocks whose solid
 * fraction is below one half, summed in block order as the reference does. */
int lgx_field_mean_velocity(lgx_lattice *lat, float *ux, float *uy);
/* Both of the above in one launch and one read-back, for a caller that wants the
 * two per frame (the reference computes them one after the other on the host,
 * src/render.rs:127-161): w gets n_blocks = bw*bh vorticity values and (ux, uy)
 * the mean velocity; w may be null, or ux and uy both null, not all three. */
int lgx_field_analyses(lgx_lattice *lat, float *w, size_t n_blocks, float *ux, float *uy);
/* Lattice::mean_velocity (src/lattice.rs:286-294) of this lattice's cells, on the
 * device: momentum per particle over every site, obstacle sites included (the
 * WITH_WALLS moments summed exactly, then Moments::velocity's f32 arithmetic).
 * The reference applies it to a GpuLattice's cells after store
 * (src/gpu.rs:1439-1446); here it needs no copy. */
int lgx_mean_velocity(lgx_lattice *lat, float *ux, float *uy);
/* New: the exact integer block sums (FLUID view, src/moments.rs:37-74) of the
 * most recent sample: mass, px2 (half units), py2 (units of sqrt(3)/2), and
 * the count of obstacle cells.  n_blocks must be bw*bh. */
int lgx_read_block_sums(lgx_lattice *lat, int32_t *mass, int32_t *px2, int32_t *py2,
                        int32_t *nsolid, size_t n_blocks);
/* transport::row_ux (src/transport.rs:87-91) of the lattice as it stands: the mean
 * x-velocity of each row, WITH_WALLS moments (src/moments.rs:37-74), formed on the
 * device; the reference stores the whole lattice to the host for it (Sim::cells,
 * src/sim.rs:100-114).  n must be h. */
int lgx_row_ux(lgx_lattice *lat, float *ux, size_t n);
/* transport::column_uy (src/transport.rs:51-84): the mean y-velocity of each
 * column, 0 for a column without particles.  n must be w. */
int lgx_column_uy(lgx_lattice *lat, float *uy, size_t n);
/* New: the exact integer WITH_WALLS moments behind those profiles: rows gets
 * mass[h] | px2[h] | py2[h] (n_rows = 3h), cols mass[w] | px2[w] | py2[w]
 * (n_cols = 3w); either may be null. */
int lgx_line_sums(lgx_lattice *lat, int32_t *rows, size_t n_rows, int32_t *cols, size_t n_cols);
/* GpuLattice::total_particles (src/gpu.rs:740-754), counted in 64 bits. */
int lgx_total_particles(lgx_lattice *lat, uint64_t *out);
/* GpuLattice::steps (pub field, src/gpu.rs:471). */
int lgx_steps(lgx_lattice *lat, uint64_t *out);
/* Kernels this lattice has launched since it was created (instrumentation). */
int lgx_launch_count(lgx_lattice *lat, uint64_t *out);
/* The lattice's CUDA stream (cudaStream_t), for callers that order their own
 * work after the engine's. */
int lgx_stream(lgx_lattice *lat, void **stream);
/* Device-time instrumentation: record event `slot` (0..7) on the lattice's
 * stream; elapsed milliseconds between two recorded slots (waits for b). */
int lgx_timing_mark(lgx_lattice *lat, int slot);
int lgx_timing_elapsed(lgx_lattice *lat, int a, int b, float *ms);

/* The exhaustive check of the circuit the step kernel runs, evaluated on the
 * device (the lgca_verify kernel, src/gpu.rs:399-417): out[i], i < n_states*48,
 * is the output state for state i/48 and draw (i/24%2, i/6%4, i%6), with bit
 * 16 set if lanes disagreed.  n must be 48 * (rest ? 128 : 64). */
int lgx_verify_circuit(int rest_particles, uint32_t *out, size_t n);

/* Instrumentation: the current device's throughput, in instructions per
 * second, of one integer instruction kind issued from eight independent
 * chains per thread on every SM: op 0 = lop3, 1 = 32-bit multiply-add,
 * 2 = funnel shift, 3 = add, 4 = high-half multiply.  The denominators of the step's integer roofline. */
int lgx_probe_int_rate(int op, double *ops_per_s);

/* ---- one step with no allocation ------------------------------------------ */

/* No counterpart in the reference.  One step of a lattice whose buffers the
 * caller owns, for callers that cannot let a library allocate device memory:
 * hosts that hand out every buffer from their own arena and treat any other
 * allocation as a fault, and loops that cannot afford the synchronisation
 * cudaMalloc/cudaFree imply.  Buffers, all device memory: planes_in /
 * planes_out hold 7 planes of ceil(w/32)*h words each, plane-major, bit k of
 * word y*ceil(w/32)+j being column 32j+k (planes_out receives the step; it
 * must not alias planes_in); solid has one plane of the same shape, anysolid
 * one bit per word of it (bit g%32 of word g/32 set when solid word g is
 * non-zero).  thresh are the inflow's seven 24-bit thresholds
 * (lgx_equilibrium_thresholds), read only when inlet_cols > 0; seed and steps
 * (steps taken before this one) key the draws as lgx_advance does.  w, h and
 * inlet_cols above 2^32 - 1 are refused with LGX_ERR_ARG.  The work is
 * enqueued on `stream` (a cudaStream_t, 0 for the default stream) and the call
 * returns without waiting.
 *
 * The inflow's per-step draws, h * ceil(inlet_cols/32) * 7 words, go to one
 * scratch array of 262144 words (1 MiB) compiled into the library and held
 * by every device that loads it; larger inflows are refused with
 * LGX_ERR_ARG.  Every call shares that array and overwrites it completely
 * before reading it, so calls whose work overlaps on the GPU (on different
 * streams, or on different host threads) race and must be ordered by the
 * caller.  The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current, and so does the first call
 * after the device's context has been destroyed and made again (for instance
 * by cudaDeviceReset), since the array may then sit at another address; make
 * that first call before any stream capture. */
int lgx_step_planes_noalloc(const uint32_t *planes_in, uint32_t *planes_out,
                            const uint32_t *solid, const uint32_t *anysolid, size_t w, size_t h,
                            int rest_particles, size_t inlet_cols, const uint32_t thresh[7],
                            uint64_t seed, uint64_t steps, void *stream);

/* ---- batches: many lattices advanced together ---------------------------- */

/* A batch borrows lattices made with lgx_create (planes, fields, inlets) and
 * advances them together: one kernel launch steps every lattice, and a
 * sampling interval's launches are one CUDA graph, captured on first use and
 * replayed.  The reference runs independent lattices one per host thread and
 * Metal queue (src/transport.rs:299-313).  While a lattice belongs to a live
 * batch, advance it only through the batch. */
typedef struct lgx_batch lgx_batch;
int lgx_batch_create(lgx_lattice *const *lats, size_t n, lgx_batch **out);
/* How a batch steps its lattices.  AUTO: lattices of up to 32768 words are grouped
 * into size classes (words rounded up to a power of two, and the rule), and a
 * tuner times each class both ways on synthetic lattices of its size and count --
 * one batched launch per step, or the resident kernel (a thread-block cluster per
 * lattice, every step of an interval in one launch) over its cluster shapes -- and
 * the faster is used; larger lattices always take one launch per step.  PER_STEP:
 * every lattice one launch per step.  RESIDENT: every class that has a usable
 * cluster shape on the resident kernel.  Results are identical under all three. */
#define LGX_BATCH_AUTO 0
#define LGX_BATCH_PER_STEP 1
#define LGX_BATCH_RESIDENT 2
int lgx_batch_create_ex(lgx_lattice *const *lats, size_t n, int policy, lgx_batch **out);
/* One size class of a batch and the tuner's finding for it. */
typedef struct lgx_batch_class {
  uint32_t words;       /* words per plane per lattice, rounded up to a power of two */
  uint32_t lattices;    /* members of the batch in the class */
  int rest;             /* the class's rule: 1 with rest particles */
  int resident;         /* 1: resident kernel, 0: one batched launch per step */
  uint32_t cluster;     /* the resident kernel's best cluster shape: CTAs per lattice */
  uint32_t threads;     /* and threads per CTA */
  float step_us;        /* tuner's time per step of the class, one launch per step */
  float resident_us;    /* and on the resident kernel (0: no usable shape) */
  uint32_t steps_per_barrier;  /* the resident kernel's steps between cluster barriers */
  int word_per_thread;  /* 1: the resident kernel that keeps each thread on one word of
                         * its band for the whole launch (every member fits it) */
} lgx_batch_class;
/* The classes of small lattices (larger ones are not listed): *n is their number,
 * the first min(cap, *n) are written. */
int lgx_batch_plan(lgx_batch *b, lgx_batch_class *out, size_t cap, size_t *n);
int lgx_batch_destroy(lgx_batch *b);
/* Every lattice advances n steps, sampling into its own attached field every
 * sample_every steps and after the last (as lgx_advance_sampling). */
int lgx_batch_advance_sampling(lgx_batch *b, uint64_t n, uint64_t sample_every, float alpha);
int lgx_batch_advance(lgx_batch *b, uint64_t n);
/* Instrumentation: kernels and graph launches issued so far; device-time
 * events on the batch's stream (as lgx_timing_mark / lgx_timing_elapsed). */
int lgx_batch_launch_count(lgx_batch *b, uint64_t *kernels, uint64_t *graphs);
int lgx_batch_timing_mark(lgx_batch *b, int slot);
int lgx_batch_timing_elapsed(lgx_batch *b, int a, int c, float *ms);

/* ---- transport coefficients (src/transport.rs) ---------------------------- */
#define LGX_TRANSPORT_SAMPLES 20
/* transport::Transport (src/transport.rs:31-37) and what its fits were made from. */
typedef struct lgx_transport {
  float nu;                 /* kinematic viscosity, lattice units */
  float g;                  /* advection factor */
  uint64_t window_nu;       /* decay windows, steps (decay_window, transport.rs:131-150) */
  uint64_t window_g;
  float u_actual;           /* realised mean speed of the advection start */
  double mode_nu[2 * LGX_TRANSPORT_SAMPLES];  /* averaged mode (a, b) per sample */
  double mode_g[2 * LGX_TRANSPORT_SAMPLES];
} lgx_transport;
/* transport::measure(density, rest, threads, seed, size, gpu = true) (src/transport.rs:
 * 291-319) for each of n densities, out[i] for densities[i]; n = 1 is measure, a range
 * of densities is main.rs's density scan (src/main.rs:549-560).  All realisations of
 * all measurements run as one batch on the current device, with the mode's profiles
 * formed on the device; nu and g are those the reference computes on the bitplane
 * path (its `threads` only shapes the CPU path).  size: the box side, even, 8..16384. */
int lgx_transport_measure(const float *densities, size_t n, int rest, uint64_t seed,
                          size_t size, lgx_transport *out);

/* ---- serving: a request loop with continuous batching ---------------------- */

/* One simulation request: a lattice's cells (copied at submit), its rule and
 * seed, the inflow (inlet_cols == 0: none), the run length, and the field to
 * sample (every sample_every steps and after the last, blocks of bx x by,
 * running average weight alpha).  The result is exactly what
 * lgx_attach_field + lgx_advance_sampling give on a fresh lattice. */
typedef struct {
  size_t w, h;
  int rest_particles;
  uint64_t seed;
  const uint8_t *cells;
  float density, ux, uy;
  size_t inlet_cols;
  uint64_t steps;
  uint64_t sample_every;
  float alpha;
  size_t bx, by;
} lgx_request;

enum {
  LGX_REQ_QUEUED = 0,
  LGX_REQ_RUNNING = 1,
  LGX_REQ_DONE = 2,
  LGX_REQ_CANCELLED = 3,
  LGX_REQ_FAILED = 4
};

typedef struct {
  uint64_t completed, failed, cancelled, active, queued;
  uint64_t ticks, kernel_launches, site_updates;
  uint64_t bytes_in_use, peak_bytes, peak_active;
  uint64_t gpu_busy_ns;  /* device time of the ticks run so far (start to end of each) */
  uint64_t host_tick_ns; /* host time the server thread spent in ticks */
  uint64_t host_wait_ns; /* of which waiting for the device to free a descriptor slot */
} lgx_server_stats;

typedef struct lgx_server lgx_server;
/* A server thread on the current device.  Requests are admitted, first fit in
 * arrival order, while their device memory fits `budget_bytes` and at most
 * `max_active` are resident; resident lattices advance together (one batched
 * launch per step) and finished ones make room for waiting ones.  No
 * counterpart in the reference beyond running one lattice per request. */
int lgx_server_create(size_t budget_bytes, size_t max_active, lgx_server **out);
/* Cancels what is still queued or running, then stops the thread. */
int lgx_server_destroy(lgx_server *s);
/* LGX_ERR_BUSY if the lattice alone exceeds the budget. */
int lgx_server_submit(lgx_server *s, const lgx_request *req, uint64_t *id);
int lgx_server_poll(lgx_server *s, uint64_t id, int *state);
/* Waits until the request leaves the queued/running states (timeout_s < 0:
 * forever); LGX_ERR_BUSY on timeout. */
int lgx_server_wait(lgx_server *s, uint64_t id, double timeout_s, int *state);
/* The final field, exact block sums and particle count of a finished request,
 * and its latency (completion minus submission, seconds).  Null outputs are
 * skipped; n_blocks must be (w/bx)*(h/by). */
int lgx_server_result(lgx_server *s, uint64_t id, float *ux, float *uy, float *rho, float *sol,
                      int32_t *mass, int32_t *px2, int32_t *py2, int32_t *nsolid,
                      size_t n_blocks, uint64_t *particles, double *latency_s);
int lgx_server_cancel(lgx_server *s, uint64_t id);
/* Frees a finished request's result buffers. */
int lgx_server_release(lgx_server *s, uint64_t id);
int lgx_server_get_stats(lgx_server *s, lgx_server_stats *out);
/* Device memory one request occupies while resident (what admission counts
 * against the budget). */
int lgx_request_device_bytes(const lgx_request *req, size_t *out);
/* Test hook: the next `count` admissions fail as if device allocation had
 * failed; those requests end LGX_REQ_FAILED and serving continues. */
int lgx_server_inject_alloc_failure(lgx_server *s, int count);

/* ---- the reference's byte-per-cell update, on the device ------------------- */

/* The reference's CPU lattice (src/lattice.rs): one byte per cell, collisions
 * from the padded lookup table with one xorshift64* generator per band of
 * ceil(h / threads) rows, the inflow re-seeded from one serial generator each
 * step.  The same random stream as the reference's CPU path, so its golden
 * checksums (tests/golden.rs) reproduce bit for bit; the bitplane lattice
 * above draws a different (counter-based) stream, as the reference's GPU path
 * does.  `threads` only fixes the band structure of the stream. */
typedef struct lgx_byte_lattice lgx_byte_lattice;
/* Lattice::new (src/lattice.rs:127-152). */
int lgx_byte_create(size_t w, size_t h, float density, float ux, float uy, size_t inlet_cols,
                    int rest_particles, size_t threads, uint64_t seed, lgx_byte_lattice **out);
int lgx_byte_destroy(lgx_byte_lattice *lat);
/* Cells (with SOLID_BIT on obstacles); n must be w*h. */
int lgx_byte_load(lgx_byte_lattice *lat, const uint8_t *cells, size_t n);
/* Lattice::restart (src/lattice.rs:188-193). */
int lgx_byte_restart(lgx_byte_lattice *lat, const uint8_t *cells, size_t n, uint64_t seed);
/* Lattice::init_equilibrium (src/lattice.rs:197-208) on the device, with the
 * lattice's own density, inflow and seed. */
int lgx_byte_init_equilibrium(lgx_byte_lattice *lat);
int lgx_byte_store(lgx_byte_lattice *lat, uint8_t *cells, size_t n);
/* Lattice::advance (src/lattice.rs:222-264, with apply_inlet 270-285). */
int lgx_byte_advance(lgx_byte_lattice *lat, uint64_t n);
/* Field::new / Field::sample (src/render.rs:35-120) on the device, and the copy out. */
int lgx_byte_attach_field(lgx_byte_lattice *lat, size_t bx, size_t by);
int lgx_byte_sample_field(lgx_byte_lattice *lat, float alpha);
int lgx_byte_read_field(lgx_byte_lattice *lat, float *ux, float *uy, float *rho, float *sol,
                        size_t n_blocks);
/* Lattice::total_particles (src/lattice.rs:299-312). */
int lgx_byte_total_particles(lgx_byte_lattice *lat, uint64_t *out);
/* Lattice::mean_velocity (src/lattice.rs:286-294), on the device. */
int lgx_byte_mean_velocity(lgx_byte_lattice *lat, float *ux, float *uy);
int lgx_byte_steps(lgx_byte_lattice *lat, uint64_t *out);

/* ---- host-side lattice setup (src/lattice.rs, src/hex.rs) ---------------- */

/* Equilibrium::new(..).thresholds() (src/lattice.rs:72-92): 24-bit thresholds,
 * six directions then rest (0 without rest particles). */
int lgx_equilibrium_thresholds(float density, float ux, float uy, int rest_particles,
                               uint32_t out[7]);
/* Lattice::init_equilibrium (src/lattice.rs:197-208) on caller-owned cells:
 * one generator Rng::new(seed ^ 0xA5A51234) in cell order; obstacle cells
 * become exactly SOLID_BIT. */
int lgx_cells_init_equilibrium(uint8_t *cells, size_t n, float density, float ux, float uy,
                               int rest_particles, uint64_t seed);
/* Lattice::add_solid (src/lattice.rs:210-220) with a box predicate on
 * hex::site_position (inclusive bounds, or strict when strict != 0). */
int lgx_cells_add_box(uint8_t *cells, size_t w, size_t h, float x0, float x1, float y0, float y1,
                      int strict);
/* Lattice::add_solid with the disc (x-cx)^2 + (y-cy)^2 <= r^2 (src/main.rs:590). */
int lgx_cells_add_circle(uint8_t *cells, size_t w, size_t h, float cx, float cy, float r);
/* Shear-wave start of transport::viscosity (src/transport.rs:188-200): row y
 * drawn from Equilibrium(density, ux_row[y], 0) with one Rng::new(rng_seed). */
int lgx_cells_shear_wave(uint8_t *cells, size_t w, size_t h, float density, const float *ux_row,
                         int rest_particles, uint64_t rng_seed);

#ifdef __cplusplus
}
#endif
#endif /* LGX_H */
