/*
 * lg_byte.c -- CPU oracle, byte-per-cell path (TEST INFRASTRUCTURE ONLY).
 *
 * Restates, in C, the reference's CPU update and everything it is built from:
 *   src/hex.rs       geometry, bit layout, reverse, site_position
 *   src/rng.rs       xorshift64* with a splitmix-style seed scramble
 *   src/collision.rs momentum classes and the padded lookup table
 *   src/lattice.rs   Equilibrium, Lattice::{step, apply_inlet, init_equilibrium,
 *                    add_solid, total_particles, mean_velocity}
 *   src/moments.rs   packed integer moments (FLUID / WITH_WALLS)
 *   src/render.rs    Field::sample (coarse-graining)
 *   tests/golden.rs  FNV-1a
 * The oracle the CUDA engine is tested against; the product never calls it.
 */
#include "lg_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define NDIR 6
#define REST_BIT 0x40u
#define SOLID_BIT 0x80u
#define STATE_MASK 0x7Fu
#define MOVING_MASK 0x3Fu
#define SQRT3_2 0.8660254f /* hex.rs:25, 0.866_025_4 as f32 */

static const int CX2[NDIR] = {2, 1, -1, -2, -1, 1};  /* hex.rs:29 */
static const int CY2[NDIR] = {0, 1, 1, 0, -1, -1};   /* hex.rs:30 */
static const float CXF[NDIR] = {1.0f, 0.5f, -0.5f, -1.0f, -0.5f, 0.5f};
static const float CYF[NDIR] = {0.0f, SQRT3_2, SQRT3_2, 0.0f, -SQRT3_2, -SQRT3_2};
static const int OPP[NDIR] = {3, 4, 5, 0, 1, 2};     /* hex.rs:36 */
static const int DX_EVEN[NDIR] = {1, 0, -1, -1, -1, 0}; /* hex.rs:39 */
static const int DX_ODD[NDIR] = {1, 1, 0, -1, 0, 1};    /* hex.rs:40 */
static const int DY[NDIR] = {0, 1, 1, 0, -1, -1};       /* hex.rs:41 */

uint8_t lgo_reverse(uint8_t s) {
    uint8_t m = s & MOVING_MASK;
    return (uint8_t)((s & REST_BIT) | ((((unsigned)m << 3) | (m >> 3)) & MOVING_MASK));
}

void lgo_site_position(size_t x, size_t y, float *px, float *py) {
    *px = (float)x + ((y & 1) ? 0.5f : 0.0f);
    *py = (float)y * SQRT3_2;
}

/* ---- rng.rs ---------------------------------------------------------------- */
uint64_t lgo_rng_seed(uint64_t seed) {
    uint64_t s = seed ^ 0x9E3779B97F4A7C15ull;
    s = (s ^ (s >> 30)) * 0xBF58476D1CE4E5B9ull;
    s = (s ^ (s >> 27)) * 0x94D049BB133111EBull;
    return (s ^ (s >> 31)) | 1ull;
}

static inline uint64_t rng_next(uint64_t *st) {
    uint64_t x = *st;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    *st = x;
    return x * 0x2545F4914F6CDD1Dull;
}

static inline uint32_t rng_next_u32(uint64_t *st) { return (uint32_t)(rng_next(st) >> 32); }

void lgo_rng_draws(uint64_t seed, uint64_t *out, size_t n) {
    uint64_t st = lgo_rng_seed(seed);
    for (size_t i = 0; i < n; ++i) out[i] = rng_next(&st);
}

/* ---- collision.rs -------------------------------------------------------- */
static void invariants(uint8_t s, int *mass, int *px, int *py) {
    int m = 0, x = 0, y = 0;
    for (int d = 0; d < NDIR; ++d)
        if (s & (1u << d)) { m++; x += CX2[d]; y += CY2[d]; }
    if (s & REST_BIT) m++;
    *mass = m; *px = x; *py = y;
}

/* Key order of the reference's BTreeMap<(u32, i32, i32), _>: lexicographic. */
static int key_cmp(uint8_t a, uint8_t b) {
    int ma, xa, ya, mb, xb, yb;
    invariants(a, &ma, &xa, &ya);
    invariants(b, &mb, &xb, &yb);
    if (ma != mb) return ma < mb ? -1 : 1;
    if (xa != xb) return xa < xb ? -1 : 1;
    if (ya != yb) return ya < yb ? -1 : 1;
    return 0;
}

int lgo_classes(int rest, int *sizes, uint8_t *members) {
    int n_states = rest ? 128 : 64;
    uint8_t order[128];
    for (int s = 0; s < n_states; ++s) order[s] = (uint8_t)s;
    /* stable insertion sort by key keeps states ascending within a class */
    for (int i = 1; i < n_states; ++i) {
        uint8_t v = order[i];
        int j = i - 1;
        while (j >= 0 && key_cmp(order[j], v) > 0) { order[j + 1] = order[j]; --j; }
        order[j + 1] = v;
    }
    int nc = 0, pos = 0;
    for (int i = 0; i < n_states;) {
        int j = i;
        while (j < n_states && key_cmp(order[i], order[j]) == 0) {
            members[pos++] = order[j];
            ++j;
        }
        sizes[nc++] = j - i;
        i = j;
    }
    return nc;
}

typedef struct {
    int stride;
    int n_states;
    uint8_t data[128 * 30];
} table_t;

static table_t g_table[2];
static pthread_once_t g_table_once = PTHREAD_ONCE_INIT;

static int gcd_i(int a, int b) { return b == 0 ? a : gcd_i(b, a % b); }

static void build_table(table_t *t, int rest) {
    int sizes[128];
    uint8_t members[128];
    int nc = lgo_classes(rest, sizes, members);
    int stride = 1;
    for (int c = 0; c < nc; ++c) stride = stride / gcd_i(stride, sizes[c]) * sizes[c];
    t->stride = stride;
    t->n_states = rest ? 128 : 64;
    int pos = 0;
    for (int c = 0; c < nc; ++c) {
        for (int i = 0; i < sizes[c]; ++i) {
            int s = members[pos + i];
            for (int k = 0; k < stride; ++k) t->data[s * stride + k] = members[pos + k % sizes[c]];
        }
        pos += sizes[c];
    }
}

static void build_tables(void) {
    build_table(&g_table[0], 0);
    build_table(&g_table[1], 1);
}

static const table_t *get_table(int rest) {
    pthread_once(&g_table_once, build_tables);
    return &g_table[rest ? 1 : 0];
}

int lgo_table_stride(int rest) { return get_table(rest)->stride; }

static inline uint8_t table_apply(const table_t *t, uint8_t state, uint32_t rand) {
    uint32_t k = (uint32_t)(((uint64_t)rand * (uint64_t)t->stride) >> 32);
    return t->data[state * t->stride + k];
}

uint8_t lgo_table_apply(int rest, uint8_t state, uint32_t rand) {
    return table_apply(get_table(rest), state, rand);
}

/* ---- lattice.rs: Equilibrium ------------------------------------------- */
uint32_t lgo_threshold(float p) {
    const float ONE = 16777216.0f;
    float t = ceilf(p * ONE);
    if (t >= ONE) return (uint32_t)ONE;
    if (t > 0.0f) return (uint32_t)t;
    return 0; /* also NaN */
}

typedef struct {
    uint32_t thresh[NDIR];
    int has_rest;
    uint32_t rest;
} equilibrium_t;

static void eq_new(equilibrium_t *e, float density, float ux, float uy, int rest) {
    float bias = rest ? 2.0f * 7.0f / 6.0f : 2.0f;
    for (int d = 0; d < NDIR; ++d) {
        float a = CXF[d] * ux;
        float b = CYF[d] * uy;
        float s = a + b;
        float q = bias * s;
        float r = 1.0f + q;
        e->thresh[d] = lgo_threshold(density * r);
    }
    e->has_rest = rest;
    e->rest = rest ? lgo_threshold(density) : 0;
}

static inline uint8_t eq_sample(const equilibrium_t *e, uint64_t *st) {
    uint8_t s = 0;
    for (int d = 0; d < NDIR; d += 2) {
        uint64_t r = rng_next(st);
        s |= (uint8_t)(((uint32_t)(r >> 40) < e->thresh[d]) << d);
        s |= (uint8_t)(((((uint32_t)(r >> 16)) & 0xFFFFFFu) < e->thresh[d + 1]) << (d + 1));
    }
    if (e->has_rest) {
        if ((uint32_t)(rng_next(st) >> 40) < e->rest) s |= REST_BIT;
    }
    return s;
}

void lgo_equilibrium_thresholds(float density, float ux, float uy, int rest, uint32_t out[7]) {
    equilibrium_t e;
    eq_new(&e, density, ux, uy, rest);
    for (int d = 0; d < NDIR; ++d) out[d] = e.thresh[d];
    out[NDIR] = e.has_rest ? e.rest : 0;
}

void lgo_equilibrium_samples(float density, float ux, float uy, int rest, uint64_t seed,
                             uint8_t *out, size_t n) {
    equilibrium_t e;
    eq_new(&e, density, ux, uy, rest);
    uint64_t st = lgo_rng_seed(seed);
    for (size_t i = 0; i < n; ++i) out[i] = eq_sample(&e, &st);
}

/* ---- lattice.rs: Lattice -------------------------------------------------- */
struct lgo_lattice {
    size_t w, h;
    uint8_t *cells, *scratch;
    int rest;
    float density, ux, uy;
    size_t inlet_cols;
    uint64_t steps;
    size_t threads;
    uint64_t seed;
};

lgo_lattice *lgo_new(size_t w, size_t h, float density, float ux, float uy,
                     size_t inlet_cols, int rest, size_t threads, uint64_t seed) {
    if (h % 2 != 0 || w <= 4 || h <= 4) return NULL; /* lattice.rs:137-138 */
    lgo_lattice *l = (lgo_lattice *)calloc(1, sizeof(*l));
    l->w = w; l->h = h;
    l->cells = (uint8_t *)calloc(w * h, 1);
    l->scratch = (uint8_t *)calloc(w * h, 1);
    l->rest = rest ? 1 : 0;
    l->density = density; l->ux = ux; l->uy = uy;
    l->inlet_cols = inlet_cols;
    l->steps = 0;
    l->threads = threads ? threads : 1;
    l->seed = seed;
    return l;
}

void lgo_free(lgo_lattice *l) {
    if (!l) return;
    free(l->cells);
    free(l->scratch);
    free(l);
}

uint8_t *lgo_cells(lgo_lattice *l) { return l->cells; }
uint64_t lgo_steps(const lgo_lattice *l) { return l->steps; }

void lgo_restart(lgo_lattice *l, const uint8_t *cells, uint64_t seed) {
    memcpy(l->cells, cells, l->w * l->h);
    l->seed = seed;
    l->steps = 0;
}

void lgo_cells_init_equilibrium(uint8_t *cells, size_t n, float density, float ux, float uy,
                                int rest, uint64_t seed) {
    uint64_t st = lgo_rng_seed(seed ^ 0xA5A51234ull);
    equilibrium_t e;
    eq_new(&e, density, ux, uy, rest);
    for (size_t i = 0; i < n; ++i)
        cells[i] = (cells[i] & SOLID_BIT) ? (uint8_t)SOLID_BIT : eq_sample(&e, &st);
}

void lgo_init_equilibrium(lgo_lattice *l) {
    lgo_cells_init_equilibrium(l->cells, l->w * l->h, l->density, l->ux, l->uy, l->rest, l->seed);
}

void lgo_cells_shear_wave(uint8_t *cells, size_t w, size_t h, float density,
                          const float *ux_row, int rest, uint64_t rng_seed) {
    uint64_t st = lgo_rng_seed(rng_seed);
    for (size_t y = 0; y < h; ++y) {
        equilibrium_t e;
        eq_new(&e, density, ux_row[y], 0.0f, rest);
        for (size_t x = 0; x < w; ++x) cells[y * w + x] = eq_sample(&e, &st);
    }
}

void lgo_cells_column_wave(uint8_t *cells, size_t w, size_t h, float density, float u0,
                           const float *uy_col, int rest, uint64_t rng_seed) {
    equilibrium_t *cols = (equilibrium_t *)malloc(w * sizeof(equilibrium_t));
    for (size_t x = 0; x < w; ++x) eq_new(&cols[x], density, u0, uy_col[x], rest);
    uint64_t st = lgo_rng_seed(rng_seed);
    for (size_t y = 0; y < h; ++y)
        for (size_t x = 0; x < w; ++x) cells[y * w + x] = eq_sample(&cols[x], &st);
    free(cols);
}

void lgo_add_box(uint8_t *cells, size_t w, size_t h, float x0, float x1, float y0, float y1,
                 int strict) {
    for (size_t y = 0; y < h; ++y)
        for (size_t x = 0; x < w; ++x) {
            float px, py;
            lgo_site_position(x, y, &px, &py);
            int in = strict ? (px > x0 && px < x1 && py > y0 && py < y1)
                            : (px >= x0 && px <= x1 && py >= y0 && py <= y1);
            if (in) cells[y * w + x] = SOLID_BIT;
        }
}

void lgo_add_circle(uint8_t *cells, size_t w, size_t h, float cx, float cy, float r) {
    float rr = r * r;
    for (size_t y = 0; y < h; ++y)
        for (size_t x = 0; x < w; ++x) {
            float px, py;
            lgo_site_position(x, y, &px, &py);
            float dx = px - cx, dy = py - cy;
            float a = dx * dx, b = dy * dy;
            if (a + b <= rr) cells[y * w + x] = SOLID_BIT;
        }
}

/* One row of the fused propagate-then-collide gather (lattice.rs:324-364). */
static void stream_and_collide_row(const uint8_t *old, uint8_t *out, const table_t *t,
                                   uint64_t *rng, size_t y, size_t w, size_t h) {
    const int *dxtab = (y & 1) ? DX_ODD : DX_EVEN;
    int sdx[NDIR];
    size_t srow[NDIR];
    for (int d = 0; d < NDIR; ++d) {
        int back = OPP[d];
        sdx[d] = dxtab[back];
        long sy = ((long)y + DY[back]) % (long)h;
        if (sy < 0) sy += (long)h;
        srow[d] = (size_t)sy * w;
    }
    size_t row = y * w;
    for (size_t x = 0; x < w; ++x) {
        uint8_t here = old[row + x];
        uint8_t state = here & REST_BIT;
        for (int d = 0; d < NDIR; ++d) {
            long sx = (long)x + sdx[d];
            if (sx < 0) sx += (long)w;
            if (sx >= (long)w) sx -= (long)w;
            state |= old[srow[d] + (size_t)sx] & (uint8_t)(1u << d);
        }
        out[x] = (here & SOLID_BIT) ? (uint8_t)(SOLID_BIT | lgo_reverse(state))
                                    : table_apply(t, state, rng_next_u32(rng));
    }
}

typedef struct {
    const uint8_t *old;
    uint8_t *out;
    const table_t *t;
    uint64_t seed;
    size_t y0, rows, w, h;
} band_job;

static void *band_worker(void *arg) {
    band_job *j = (band_job *)arg;
    uint64_t rng = lgo_rng_seed(j->seed);
    for (size_t r = 0; r < j->rows; ++r)
        stream_and_collide_row(j->old, j->out + r * j->w, j->t, &rng, j->y0 + r, j->w, j->h);
    return NULL;
}

static void apply_inlet(lgo_lattice *l) {
    if (l->inlet_cols == 0) return;
    equilibrium_t e;
    eq_new(&e, l->density, l->ux, l->uy, l->rest);
    uint64_t st = lgo_rng_seed(l->seed ^ (l->steps * 0xD1B54A32D192ED03ull));
    size_t cols = l->inlet_cols < l->w ? l->inlet_cols : l->w;
    for (size_t y = 0; y < l->h; ++y)
        for (size_t x = 0; x < cols; ++x) {
            size_t i = y * l->w + x;
            if (!(l->cells[i] & SOLID_BIT)) l->cells[i] = eq_sample(&e, &st);
        }
}

/* Lattice::step (lattice.rs:228-264): one generator per band of rows, bands of
 * ceil(h / min(threads, h)) rows, seeded base_seed ^ ((band + 1) << 32). */
static void lattice_step(lgo_lattice *l) {
    size_t w = l->w, h = l->h;
    const table_t *t = get_table(l->rest);
    size_t nthreads = l->threads < h ? l->threads : h;
    uint64_t base_seed = l->seed ^ (l->steps * 0x9E3779B97F4A7C15ull);
    size_t band = (h + nthreads - 1) / nthreads;
    size_t nbands = (h + band - 1) / band;
    band_job jobs[1024];
    pthread_t tid[1024];
    if (nbands > 1024) nbands = 1024; /* not reachable for h <= 1024 * band */
    for (size_t b = 0; b < nbands; ++b) {
        size_t y0 = b * band;
        size_t rows = (y0 + band <= h) ? band : h - y0;
        jobs[b] = (band_job){l->cells, l->scratch + y0 * w, t,
                             base_seed ^ ((uint64_t)(b + 1) << 32), y0, rows, w, h};
    }
    if (nbands == 1) {
        band_worker(&jobs[0]);
    } else {
        for (size_t b = 0; b < nbands; ++b) pthread_create(&tid[b], NULL, band_worker, &jobs[b]);
        for (size_t b = 0; b < nbands; ++b) pthread_join(tid[b], NULL);
    }
    uint8_t *tmp = l->cells;
    l->cells = l->scratch;
    l->scratch = tmp;
    l->steps += 1;
    apply_inlet(l);
}

void lgo_advance(lgo_lattice *l, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) lattice_step(l);
}

uint64_t lgo_total_particles(const lgo_lattice *l) {
    uint64_t n = 0;
    size_t N = l->w * l->h;
    for (size_t i = 0; i < N; ++i) n += (uint64_t)__builtin_popcount(l->cells[i] & STATE_MASK);
    return n;
}

/* ---- moments.rs ----------------------------------------------------------- */
void lgo_moments_sum(const uint8_t *cells, size_t n, int walls, int64_t out[4]) {
    int64_t mass = 0, px = 0, py = 0, solid = 0;
    for (size_t i = 0; i < n; ++i) {
        uint8_t c = cells[i];
        int is_solid = (c & SOLID_BIT) != 0;
        if (walls || !is_solid) {
            int m, x, y;
            invariants(c & STATE_MASK, &m, &x, &y);
            mass += m; px += x; py += y;
        }
        solid += is_solid;
    }
    out[0] = mass; out[1] = px; out[2] = py; out[3] = solid;
}

void lgo_invariants(const uint8_t *cells, size_t n, int64_t out[3]) {
    int64_t s[4];
    lgo_moments_sum(cells, n, 1, s);
    out[0] = s[0]; out[1] = s[1]; out[2] = s[2];
}

/* Moments::velocity (moments.rs:91-97). */
static void velocity(int64_t mass, int64_t px2, int64_t py2, float *vx, float *vy) {
    if (mass == 0) { *vx = 0.0f; *vy = 0.0f; return; }
    float m = (float)mass;
    float a = (float)px2 * 0.5f;
    float b = (float)py2 * SQRT3_2;
    *vx = a / m;
    *vy = b / m;
}

void lgo_mean_velocity(const lgo_lattice *l, float *ux, float *uy) {
    int64_t s[4];
    lgo_moments_sum(l->cells, l->w * l->h, 1, s);
    velocity(s[0], s[1], s[2], ux, uy);
}

void lgo_block_sums(const uint8_t *cells, size_t w, size_t h, size_t bx, size_t by,
                    int32_t *mass, int32_t *px2, int32_t *py2, int32_t *nsolid) {
    size_t bw = w / bx, bh = h / by;
    for (size_t jb = 0; jb < bh; ++jb)
        for (size_t ib = 0; ib < bw; ++ib) {
            int64_t m = 0, x = 0, yy = 0, s = 0;
            for (size_t y = jb * by; y < (jb + 1) * by; ++y) {
                int64_t t[4];
                lgo_moments_sum(cells + y * w + ib * bx, bx, 0, t);
                m += t[0]; x += t[1]; yy += t[2]; s += t[3];
            }
            size_t k = jb * bw + ib;
            mass[k] = (int32_t)m; px2[k] = (int32_t)x; py2[k] = (int32_t)yy; nsolid[k] = (int32_t)s;
        }
}

void lgo_field_sample(const uint8_t *cells, size_t w, size_t h, size_t bx, size_t by,
                      float alpha, float *ux, float *uy, float *rho, float *sol) {
    size_t bw = w / bx, bh = h / by;
    if (bw == 0 || bh == 0) return;
    size_t nb = bw * bh;
    int32_t *m = (int32_t *)malloc(nb * 4 * sizeof(int32_t));
    lgo_block_sums(cells, w, h, bx, by, m, m + nb, m + 2 * nb, m + 3 * nb);
    float n = (float)(bx * by);
    for (size_t k = 0; k < nb; ++k) {
        float vx, vy;
        velocity(m[k], m[nb + k], m[2 * nb + k], &vx, &vy);
        ux[k] += alpha * (vx - ux[k]);
        uy[k] += alpha * (vy - uy[k]);
        rho[k] += alpha * ((float)m[k] / n - rho[k]);
        sol[k] = (float)m[3 * nb + k] / n;
    }
    free(m);
}

uint64_t lgo_fnv1a(const uint8_t *bytes, size_t n) {
    uint64_t h = 0xcbf29ce484222325ull;
    for (size_t i = 0; i < n; ++i) {
        h ^= bytes[i];
        h *= 0x1000000001b3ull; /* the reference's multiplier, golden.rs:44 */
    }
    return h;
}

/* ---- render.rs: Field::vorticity, Field::mean_velocity ---------------------- */
void lgo_field_vorticity(const float *ux, const float *uy, size_t bw, size_t bh, size_t bx,
                         size_t by, float *out) {
    float dx = (float)bx;
    float dy = (float)by * SQRT3_2;
    for (size_t j = 0; j < bh; ++j)
        for (size_t i = 0; i < bw; ++i) {
            size_t ip = i + 1 < bw - 1 ? i + 1 : bw - 1;
            size_t im = i > 0 ? i - 1 : 0;
            size_t jp = j + 1 < bh ? j + 1 : 0;
            size_t jm = j == 0 ? bh - 1 : j - 1;
            float num = uy[j * bw + ip] - uy[j * bw + im];
            float den = (float)(ip - im) * dx;
            float dvdx = num / den;
            float num2 = ux[jp * bw + i] - ux[jm * bw + i];
            float den2 = 2.0f * dy;
            float dudy = num2 / den2;
            out[j * bw + i] = dvdx - dudy;
        }
}

void lgo_field_mean_velocity(const float *ux, const float *uy, const float *sol, size_t nb,
                             float *mx, float *my) {
    float sx = 0.0f, sy = 0.0f, n = 0.0f;
    for (size_t k = 0; k < nb; ++k)
        if (sol[k] < 0.5f) {
            sx += ux[k];
            sy += uy[k];
            n += 1.0f;
        }
    *mx = n == 0.0f ? 0.0f : sx / n;
    *my = n == 0.0f ? 0.0f : sy / n;
}
