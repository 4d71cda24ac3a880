/*
 * lg_oracle.h -- CPU oracle for the FHP lattice gas (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C restatement of the reference (daleobrien/lattice-gas) that
 * the CUDA engine is tested against.  Nothing in the product library links or
 * calls it; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it.
 *
 * Two paths are restated:
 *   - the byte-per-cell CPU path (src/lattice.rs, src/collision.rs, src/rng.rs,
 *     src/moments.rs, src/render.rs Field::sample).  Pinned bit for bit by the
 *     reference's golden FNV-1a checksums (tests/golden.rs:141-147).
 *   - the bitplane path the Metal shader runs (src/gpu.rs:144-418 and the host
 *     side gpu.rs:479-754).  No recorded microstate exists for it in the
 *     reference; it is pinned by the exhaustive collision known-answer test
 *     (gpu.rs:775-820) and the structural tests (gpu.rs:826-1152).
 *
 * All floating point is f32 with no contraction (built with -ffp-contract=off),
 * matching Rust, which never fuses multiply-add.
 */
#ifndef LG_ORACLE_H
#define LG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- geometry and rule (src/hex.rs, src/collision.rs) ------------------- */
uint8_t lgo_reverse(uint8_t state);                                  /* hex.rs:45 */
void lgo_site_position(size_t x, size_t y, float *px, float *py);     /* hex.rs:52 */
/* Classes in the reference's BTreeMap order; states ascending within each.
 * Writes class sizes to sizes[] and members back to back to members[].
 * Returns the number of classes (collision.rs:62-69). */
int lgo_classes(int rest, int *sizes, uint8_t *members);
int lgo_table_stride(int rest);                                       /* collision.rs:110-113 */
uint8_t lgo_table_apply(int rest, uint8_t state, uint32_t rand);      /* collision.rs:115-119 */

/* ---- RNG (src/rng.rs) ---------------------------------------------------- */
uint64_t lgo_rng_seed(uint64_t seed);                                 /* rng.rs:9-15 */
/* Draw n successive next_u64 values from a generator built with Rng::new(seed). */
void lgo_rng_draws(uint64_t seed, uint64_t *out, size_t n);

/* ---- equilibrium (src/lattice.rs:41-116) --------------------------------- */
uint32_t lgo_threshold(float p);                                      /* lattice.rs:59 */
void lgo_equilibrium_thresholds(float density, float ux, float uy, int rest,
                                uint32_t out[7]);                    /* lattice.rs:72-92 */
/* n samples from Equilibrium::sample with one generator Rng::new(seed). */
void lgo_equilibrium_samples(float density, float ux, float uy, int rest,
                             uint64_t seed, uint8_t *out, size_t n);

/* ---- byte-path lattice (src/lattice.rs) ---------------------------------- */
typedef struct lgo_lattice lgo_lattice;
lgo_lattice *lgo_new(size_t w, size_t h, float density, float ux, float uy,
                     size_t inlet_cols, int rest, size_t threads, uint64_t seed);
void lgo_free(lgo_lattice *lat);
uint8_t *lgo_cells(lgo_lattice *lat);
uint64_t lgo_steps(const lgo_lattice *lat);
void lgo_restart(lgo_lattice *lat, const uint8_t *cells, uint64_t seed);   /* lattice.rs:188 */
void lgo_init_equilibrium(lgo_lattice *lat);                               /* lattice.rs:197 */
void lgo_advance(lgo_lattice *lat, uint64_t n);                            /* lattice.rs:222 */
uint64_t lgo_total_particles(const lgo_lattice *lat);                      /* lattice.rs:299 */
void lgo_mean_velocity(const lgo_lattice *lat, float *ux, float *uy);      /* lattice.rs:292 */

/* Obstacles on any byte lattice (add_solid, lattice.rs:210-220, with the
 * predicates the reference's callers use).  Box: x0<=x<=x1 && y0<=y<=y1, or
 * strict inequalities when strict != 0.  Circle: (x-cx)^2+(y-cy)^2 <= r*r. */
void lgo_add_box(uint8_t *cells, size_t w, size_t h, float x0, float x1,
                 float y0, float y1, int strict);
void lgo_add_circle(uint8_t *cells, size_t w, size_t h, float cx, float cy, float r);
/* Rng::new(seed ^ 0xA5A51234) over every cell; solid cells keep SOLID_BIT. */
void lgo_cells_init_equilibrium(uint8_t *cells, size_t n, float density, float ux,
                                float uy, int rest, uint64_t seed);
/* Shear-wave start (src/transport.rs:188-200): row y drawn from
 * Equilibrium(density, amp_row[y], 0) with one generator Rng::new(rng_seed). */
void lgo_cells_shear_wave(uint8_t *cells, size_t w, size_t h, float density,
                          const float *ux_row, int rest, uint64_t rng_seed);

/* Transverse-wave start (src/transport.rs:237-251): column x drawn from
 * Equilibrium(density, u0, uy_col[x]), cells in row-major order, one generator
 * Rng::new(rng_seed). */
void lgo_cells_column_wave(uint8_t *cells, size_t w, size_t h, float density, float u0,
                           const float *uy_col, int rest, uint64_t rng_seed);

/* ---- moments and coarse-graining (src/moments.rs, src/render.rs:61-120) --- */
/* Exact (mass, px2, py2, solid) of a byte slice through the FLUID (walls=0) or
 * WITH_WALLS (walls=1) table. */
void lgo_moments_sum(const uint8_t *cells, size_t n, int walls, int64_t out[4]);
void lgo_invariants(const uint8_t *cells, size_t n, int64_t out[3]);
/* Field::sample over caller-owned arrays of bw*bh floats. */
void lgo_field_sample(const uint8_t *cells, size_t w, size_t h, size_t bx, size_t by,
                      float alpha, float *ux, float *uy, float *rho, float *sol);
/* Exact integer block sums (FLUID view): mass, px2, py2, nsolid per block. */
void lgo_block_sums(const uint8_t *cells, size_t w, size_t h, size_t bx, size_t by,
                    int32_t *mass, int32_t *px2, int32_t *py2, int32_t *nsolid);
uint64_t lgo_fnv1a(const uint8_t *bytes, size_t n);                   /* golden.rs:40 */
/* Field::vorticity and Field::mean_velocity (render.rs:127-161) of a field. */
void lgo_field_vorticity(const float *ux, const float *uy, size_t bw, size_t bh, size_t bx,
                         size_t by, float *out);
void lgo_field_mean_velocity(const float *ux, const float *uy, const float *sol, size_t nb,
                             float *mx, float *my);


/* ---- bitplane path (src/gpu.rs) ------------------------------------------ */
uint32_t lgo_mix(uint32_t x);                                          /* gpu.rs:147 */
/* s[0]=s2, s[1..3]=s3, s[4..8]=s5 (gpu.rs:157-180). */
void lgo_draws(uint32_t key, uint32_t s[9]);
/* The collision rule for one lane: class pick by selector (gpu.rs:46-139 as
 * specified by the KAT at gpu.rs:799-817).  two: 0/1; three: 0..3 (3 = none);
 * five: 0..5 (5 = none). */
uint8_t lgo_collide_lane(int rest, uint8_t state, int two, int three, int five);
/* Word-wide collision: 7 planes in, 7 out, selectors as lgo_draws. */
void lgo_collide_word(int rest, const uint32_t n[7], const uint32_t s[9], uint32_t o[7]);
/* The 18 step parameters of GpuLattice::params (gpu.rs:547-568). */
void lgo_bp_params(size_t w, size_t h, uint64_t seed, uint64_t steps,
                   size_t inlet_cols, const uint32_t thresh[7], uint32_t P[18]);

typedef struct lgo_bp lgo_bp;                                           /* GpuLattice */
lgo_bp *lgo_bp_new(size_t w, size_t h, int rest, uint64_t seed, size_t threads);
void lgo_bp_free(lgo_bp *g);
void lgo_bp_set_inlet(lgo_bp *g, size_t cols, float density, float ux, float uy, int rest);
void lgo_bp_attach_field(lgo_bp *g, size_t bx, size_t by);
void lgo_bp_load(lgo_bp *g, const uint8_t *cells);
void lgo_bp_restart(lgo_bp *g, const uint8_t *cells, uint64_t seed);
void lgo_bp_store(const lgo_bp *g, uint8_t *cells);
void lgo_bp_advance_sampling(lgo_bp *g, uint64_t n, uint64_t sample_every, float alpha);
void lgo_bp_sample_field(lgo_bp *g, float alpha);
void lgo_bp_read_field(const lgo_bp *g, float *ux, float *uy, float *rho, float *sol);
void lgo_bp_read_block_sums(const lgo_bp *g, int32_t *mass, int32_t *px2,
                            int32_t *py2, int32_t *nsolid);
uint64_t lgo_bp_total_particles(const lgo_bp *g);
uint64_t lgo_bp_steps(const lgo_bp *g);
/* Raw planes (7 * wpr * h words, plane-major) for word-level comparisons. */
const uint32_t *lgo_bp_planes(const lgo_bp *g);
/* Set the step counter (GpuLattice::steps, a public field, gpu.rs:471). */
void lgo_bp_set_steps(lgo_bp *g, uint64_t steps);
/* n steps of rows y0 .. y1-1 only (the window widened by the steps left on each
 * side, so those rows end exact); y1 - y0 + 2n <= h. */
void lgo_bp_advance_window(lgo_bp *g, uint64_t n, size_t y0, size_t y1);
/* Cells of rows y0 .. y1-1, (y1 - y0) * w bytes. */
void lgo_bp_store_rows(const lgo_bp *g, size_t y0, size_t y1, uint8_t *cells);

/* ---- transport.rs ------------------------------------------------------- */
/* row_ux / column_uy (transport.rs:51-91) of byte cells. */
void lgo_row_ux(const uint8_t *cells, size_t w, size_t h, float *out);
void lgo_column_uy(const uint8_t *cells, size_t w, size_t h, float *out);
#define LGO_TRANSPORT_SAMPLES 20
typedef struct lgo_transport {
    float nu, g;
    uint64_t window_nu, window_g;
    float u_actual;
    double mode_nu[2 * LGO_TRANSPORT_SAMPLES];
    double mode_g[2 * LGO_TRANSPORT_SAMPLES];
} lgo_transport;
/* transport::measure (transport.rs:291-319) on the CPU byte path (gpu = 0, whose
 * random stream depends on threads) or on the bitplane path (gpu = 1). */
void lgo_transport_measure(float density, int rest, size_t threads, uint64_t seed, size_t size,
                           int gpu, lgo_transport *out);

#ifdef __cplusplus
}
#endif
#endif
