/*
 * lg_bitplane.c -- CPU oracle, bitplane path (TEST INFRASTRUCTURE ONLY).
 *
 * A word-for-word restatement of what the reference's Metal path computes
 * (src/gpu.rs): the stateless hash and selectors (gpu.rs:147-198), the step
 * kernel lgca_step (gpu.rs:203-310), the coarse-graining kernel lgca_sample
 * (gpu.rs:324-377), the particle count lgca_count (gpu.rs:381-395), and the
 * host side of GpuLattice (params, load, store, advance_sampling;
 * gpu.rs:547-754).
 *
 * The collision is NOT the generated circuit: it is the class rule the
 * reference's known-answer test states (gpu.rs:799-817), evaluated lane by
 * lane from the class enumeration.  That keeps this oracle independent of
 * the circuit generator it checks.
 */
#include "lg_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define NDIR 6
#define PLANES 7
#define REST_BIT 0x40u
#define SOLID_BIT 0x80u
#define SQRT3_2 0.8660254f

static const int CX2[NDIR] = {2, 1, -1, -2, -1, 1};
static const int CY2[NDIR] = {0, 1, 1, 0, -1, -1};
static const int OPP[NDIR] = {3, 4, 5, 0, 1, 2};
static const int DXE[NDIR] = {1, 0, -1, -1, -1, 0};
static const int DXO[NDIR] = {1, 1, 0, -1, 0, 1};
static const int DYT[NDIR] = {0, 1, 1, 0, -1, -1};

uint32_t lgo_mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

void lgo_draws(uint32_t key, uint32_t s[9]) {
    uint32_t r = lgo_mix(key);
    s[0] = r;
    uint32_t s3[3] = {0, 0, 0};
    uint32_t open = 0xffffffffu;
    for (int k = 0; k < 3; ++k) {
        r = lgo_mix(r);
        uint32_t a = r;
        r = lgo_mix(r);
        uint32_t b = r;
        s3[0] |= open & ~a & ~b;
        s3[1] |= open & a & ~b;
        s3[2] |= open & ~a & b;
        open &= a & b;
    }
    uint32_t s5[5] = {0, 0, 0, 0, 0};
    uint32_t open5 = 0xffffffffu;
    for (int k = 0; k < 4; ++k) {
        r = lgo_mix(r);
        uint32_t a = r;
        r = lgo_mix(r);
        uint32_t b = r;
        r = lgo_mix(r);
        uint32_t c = r;
        s5[0] |= open5 & ~a & ~b & ~c;
        s5[1] |= open5 & a & ~b & ~c;
        s5[2] |= open5 & ~a & b & ~c;
        s5[3] |= open5 & a & b & ~c;
        s5[4] |= open5 & ~a & ~b & c;
        open5 &= c & (a | b);
    }
    for (int i = 0; i < 3; ++i) s[1 + i] = s3[i];
    for (int i = 0; i < 5; ++i) s[4 + i] = s5[i];
}

static uint32_t bernoulli(uint32_t t, uint32_t *r) {
    if (t == 0u) return 0u;
    if (t >= (1u << 24)) return 0xffffffffu;
    uint32_t x = 0u;
    for (uint32_t j = 0; j < 24u; ++j) {
        *r = lgo_mix(*r);
        x = ((t >> j) & 1u) ? (*r | x) : (*r & x);
    }
    return x;
}

/* class_of[rest][state] -> (offset into members, size) */
typedef struct {
    int size[128];
    int off[128];
    uint8_t members[128];
} classmap_t;

static classmap_t g_cm[2];
static pthread_once_t g_cm_once = PTHREAD_ONCE_INIT;

static void build_cm_one(classmap_t *cm, int rest) {
    int sizes[128];
    int nc = lgo_classes(rest, sizes, cm->members);
    int pos = 0;
    for (int c = 0; c < nc; ++c) {
        for (int i = 0; i < sizes[c]; ++i) {
            cm->size[cm->members[pos + i]] = sizes[c];
            cm->off[cm->members[pos + i]] = pos;
        }
        pos += sizes[c];
    }
}

static void build_cm(void) {
    build_cm_one(&g_cm[0], 0);
    build_cm_one(&g_cm[1], 1);
}

uint8_t lgo_collide_lane(int rest, uint8_t state, int two, int three, int five) {
    pthread_once(&g_cm_once, build_cm);
    const classmap_t *cm = &g_cm[rest ? 1 : 0];
    /* Without rest particles the rule reads six bits; bit 6 passes through. */
    uint8_t keep_hi = rest ? 0 : (state & REST_BIT);
    uint8_t s = rest ? (state & 0x7F) : (state & 0x3F);
    int size = cm->size[s];
    const uint8_t *g = &cm->members[cm->off[s]];
    uint8_t out = s;
    if (size == 2) out = g[two ? 0 : 1];
    else if (size == 3) out = (three < 3) ? g[three] : s;
    else if (size == 5) out = (five < 5) ? g[five] : s;
    return (uint8_t)(out | keep_hi);
}

void lgo_collide_word(int rest, const uint32_t n[7], const uint32_t s[9], uint32_t o[7]) {
    for (int d = 0; d < 7; ++d) o[d] = 0;
    for (int b = 0; b < 32; ++b) {
        uint8_t st = 0;
        for (int d = 0; d < 7; ++d) st |= (uint8_t)(((n[d] >> b) & 1u) << d);
        int two = (s[0] >> b) & 1u;
        int three = 3, five = 5;
        for (int k = 2; k >= 0; --k)
            if ((s[1 + k] >> b) & 1u) three = k;
        for (int k = 4; k >= 0; --k)
            if ((s[4 + k] >> b) & 1u) five = k;
        uint8_t out = lgo_collide_lane(rest, st, two, three, five);
        for (int d = 0; d < 7; ++d) o[d] |= (uint32_t)((out >> d) & 1u) << b;
    }
}

void lgo_bp_params(size_t w, size_t h, uint64_t seed, uint64_t steps, size_t inlet_cols,
                   const uint32_t thresh[7], uint32_t P[18]) {
    size_t wpr = (w + 31) / 32;
    uint32_t lastword = (uint32_t)((w - 1) / 32);
    uint32_t lastbit = (uint32_t)((w - 1) % 32);
    uint32_t tail = (lastbit == 31) ? 0xffffffffu : ((1u << (lastbit + 1)) - 1u);
    size_t iw = (inlet_cols + 31) / 32;
    P[0] = (uint32_t)wpr;
    P[1] = (uint32_t)h;
    P[2] = (uint32_t)(seed ^ (steps * 0x9E3779B97F4A7C15ull));
    P[3] = lastword;
    P[4] = lastbit;
    P[5] = tail;
    P[6] = (uint32_t)(wpr * h);
    P[7] = (uint32_t)iw;
    P[8] = (uint32_t)inlet_cols;
    P[9] = (uint32_t)(iw * h);
    P[10] = (uint32_t)((wpr - iw) > 0 ? (wpr - iw) : 1);
    for (int d = 0; d < 7; ++d) P[11 + d] = thresh[d];
}

/* lgca_step for one lattice word (gpu.rs:229-309). */
static void step_word(const uint32_t *a, uint32_t *b, const uint32_t *solid,
                      const uint32_t *anysolid, const uint32_t *P, int rest, uint32_t y,
                      uint32_t j) {
    uint32_t wpr = P[0], hh = P[1], total = P[6], lastword = P[3], lastbit = P[4];
    uint32_t n[7];
    for (int d = 0; d < 6; ++d) {
        int bk = OPP[d];
        int dx = (y & 1u) ? DXO[bk] : DXE[bk];
        int sy = (int)y + DYT[bk];
        if (sy < 0) sy += (int)hh;
        if (sy >= (int)hh) sy -= (int)hh;
        size_t base = (size_t)d * total + (size_t)sy * wpr;
        uint32_t w = a[base + j];
        uint32_t v;
        if (dx == 0) {
            v = w;
        } else if (dx > 0) {
            uint32_t hi = (j + 1u < wpr) ? a[base + j + 1u] : 0u;
            v = (w >> 1) | (hi << 31);
            if (j == lastword) v = (v & ~(1u << lastbit)) | ((a[base] & 1u) << lastbit);
        } else {
            uint32_t lo = (j > 0u) ? a[base + j - 1u] : 0u;
            v = (w << 1) | (lo >> 31);
            if (j == 0u) v = (v & ~1u) | ((a[base + lastword] >> lastbit) & 1u);
        }
        n[d] = v;
    }
    size_t word = (size_t)y * wpr + j;
    n[6] = a[6u * (size_t)total + word];
    uint32_t s[9];
    lgo_draws((uint32_t)word ^ P[2], s);
    uint32_t o[7];
    lgo_collide_word(rest, n, s, o);
    uint32_t sm = 0u;
    if ((anysolid[word >> 5] >> (word & 31u)) & 1u) sm = solid[word];
    uint32_t fluid = ~sm;
    uint32_t res[7];
    for (int d = 0; d < 6; ++d) res[d] = (sm & n[(d + 3) % 6]) | (fluid & o[d]);
    res[6] = (sm & n[6]) | (fluid & o[6]);
    if (j < P[7]) {
        uint32_t span = P[8] - j * 32u;
        if (span > 32u) span = 32u;
        uint32_t imask = (span >= 32u) ? 0xffffffffu : ((1u << span) - 1u);
        uint32_t apply = imask & fluid;
        if (apply != 0u) {
            uint32_t r = lgo_mix((uint32_t)word ^ P[2] ^ 0x9e3779b9u);
            for (int d = 0; d < 7; ++d)
                res[d] = (res[d] & ~apply) | (bernoulli(P[11 + d], &r) & apply);
        }
    }
    uint32_t mask = (j == lastword) ? P[5] : 0xffffffffu;
    for (int d = 0; d < 7; ++d) b[(size_t)d * total + word] = res[d] & mask;
}

struct lgo_bp {
    size_t w, h, wpr, total;
    int rest;
    uint32_t *a, *b, *solid, *anysolid;
    uint64_t steps, seed;
    size_t inlet_cols;
    uint32_t thresh[7];
    size_t threads;
    /* field */
    size_t bx, by, bw, bh;
    float *ux, *uy, *rho, *sol;
    int32_t *bsum; /* 4 * bw * bh: mass, px2, py2, nsolid of the last sample */
};

lgo_bp *lgo_bp_new(size_t w, size_t h, int rest, uint64_t seed, size_t threads) {
    if (h % 2 != 0 || w <= 4 || h <= 4) return NULL; /* gpu.rs:480-481 */
    lgo_bp *g = (lgo_bp *)calloc(1, sizeof(*g));
    g->w = w; g->h = h;
    g->wpr = (w + 31) / 32;
    g->total = g->wpr * h;
    g->rest = rest ? 1 : 0;
    g->a = (uint32_t *)calloc(g->total * PLANES, 4);
    g->b = (uint32_t *)calloc(g->total * PLANES, 4);
    g->solid = (uint32_t *)calloc(g->total, 4);
    g->anysolid = (uint32_t *)calloc((g->total + 31) / 32, 4);
    g->seed = seed;
    g->threads = threads ? threads : 1;
    return g;
}

void lgo_bp_free(lgo_bp *g) {
    if (!g) return;
    free(g->a); free(g->b); free(g->solid); free(g->anysolid);
    free(g->ux); free(g->uy); free(g->rho); free(g->sol); free(g->bsum);
    free(g);
}

void lgo_bp_set_inlet(lgo_bp *g, size_t cols, float density, float ux, float uy, int rest) {
    g->inlet_cols = cols < g->w ? cols : g->w;
    lgo_equilibrium_thresholds(density, ux, uy, rest, g->thresh);
}

void lgo_bp_attach_field(lgo_bp *g, size_t bx, size_t by) {
    g->bx = bx; g->by = by;
    g->bw = g->w / bx; g->bh = g->h / by;
    size_t n = g->bw * g->bh;
    free(g->ux); free(g->uy); free(g->rho); free(g->sol); free(g->bsum);
    g->ux = (float *)calloc(n ? n : 1, 4);
    g->uy = (float *)calloc(n ? n : 1, 4);
    g->rho = (float *)calloc(n ? n : 1, 4);
    g->sol = (float *)calloc(n ? n : 1, 4);
    g->bsum = (int32_t *)calloc(4 * (n ? n : 1), 4);
}

void lgo_bp_load(lgo_bp *g, const uint8_t *cells) {
    size_t w = g->w, wpr = g->wpr, total = g->total;
    memset(g->a, 0, total * PLANES * 4);
    memset(g->solid, 0, total * 4);
    memset(g->anysolid, 0, ((total + 31) / 32) * 4);
    for (size_t y = 0; y < g->h; ++y)
        for (size_t x = 0; x < w; ++x) {
            uint8_t c = cells[y * w + x];
            size_t word = y * wpr + x / 32;
            uint32_t bit = 1u << (x % 32);
            for (int d = 0; d < 7; ++d)
                if (c & (1u << d)) g->a[d * total + word] |= bit;
            if (c & SOLID_BIT) g->solid[word] |= bit;
        }
    for (size_t i = 0; i < total; ++i)
        if (g->solid[i]) g->anysolid[i >> 5] |= 1u << (i & 31);
}

void lgo_bp_restart(lgo_bp *g, const uint8_t *cells, uint64_t seed) {
    lgo_bp_load(g, cells);
    g->seed = seed;
    g->steps = 0;
}

void lgo_bp_store(const lgo_bp *g, uint8_t *cells) {
    size_t w = g->w, wpr = g->wpr, total = g->total;
    for (size_t y = 0; y < g->h; ++y)
        for (size_t x = 0; x < w; ++x) {
            size_t word = y * wpr + x / 32;
            uint32_t k = (uint32_t)(x % 32);
            uint8_t c = 0;
            for (int d = 0; d < 7; ++d) c |= (uint8_t)(((g->a[d * total + word] >> k) & 1u) << d);
            c |= (uint8_t)(((g->solid[word] >> k) & 1u) << 7);
            cells[y * w + x] = c;
        }
}

typedef struct {
    lgo_bp *g;
    const uint32_t *P;
    uint32_t y0, y1;
} step_job;

static void *step_worker(void *arg) {
    step_job *j = (step_job *)arg;
    lgo_bp *g = j->g;
    for (uint32_t y = j->y0; y < j->y1; ++y)
        for (uint32_t x = 0; x < (uint32_t)g->wpr; ++x)
            step_word(g->a, g->b, g->solid, g->anysolid, j->P, g->rest, y, x);
    return NULL;
}

static void bp_step(lgo_bp *g) {
    uint32_t P[18];
    lgo_bp_params(g->w, g->h, g->seed, g->steps, g->inlet_cols, g->thresh, P);
    size_t nt = g->threads < g->h ? g->threads : g->h;
    if (nt > 256) nt = 256;
    step_job jobs[256];
    pthread_t tid[256];
    size_t band = (g->h + nt - 1) / nt;
    size_t nj = 0;
    for (size_t y = 0; y < g->h; y += band) {
        size_t y1 = y + band < g->h ? y + band : g->h;
        jobs[nj++] = (step_job){g, P, (uint32_t)y, (uint32_t)y1};
    }
    if (nj == 1) step_worker(&jobs[0]);
    else {
        for (size_t i = 0; i < nj; ++i) pthread_create(&tid[i], NULL, step_worker, &jobs[i]);
        for (size_t i = 0; i < nj; ++i) pthread_join(tid[i], NULL);
    }
    uint32_t *t = g->a;
    g->a = g->b;
    g->b = t;
    g->steps += 1;
}

/* lgca_sample (gpu.rs:324-377) for every block. */
static void bp_sample(lgo_bp *g, float alpha) {
    if (!g->ux) return;
    size_t wpr = g->wpr, total = g->total, bx = g->bx, by = g->by, bw = g->bw, bh = g->bh;
    size_t nb = bw * bh;
    for (size_t gid = 0; gid < nb; ++gid) {
        size_t jb = gid / bw, ib = gid - jb * bw;
        uint32_t x0 = (uint32_t)(ib * bx), x1 = (uint32_t)(x0 + bx);
        uint32_t w0 = x0 >> 5, w1 = (x1 - 1u) >> 5;
        int mass = 0, px = 0, py = 0;
        uint32_t nsolid = 0;
        for (size_t y = jb * by; y < (jb + 1) * by; ++y) {
            size_t base = y * wpr;
            for (uint32_t wi = w0; wi <= w1; ++wi) {
                uint32_t lo = (x0 > (wi << 5) ? x0 : (wi << 5)) - (wi << 5);
                uint32_t hi = (x1 < ((wi + 1u) << 5) ? x1 : ((wi + 1u) << 5)) - (wi << 5);
                uint32_t m = (hi - lo >= 32u) ? 0xffffffffu : (((1u << (hi - lo)) - 1u) << lo);
                uint32_t sm = g->solid[base + wi] & m;
                nsolid += (uint32_t)__builtin_popcount(sm);
                uint32_t fm = m & ~sm;
                for (int d = 0; d < 6; ++d) {
                    int c = __builtin_popcount(g->a[d * total + base + wi] & fm);
                    mass += c;
                    px += CX2[d] * c;
                    py += CY2[d] * c;
                }
                mass += __builtin_popcount(g->a[6 * total + base + wi] & fm);
            }
        }
        g->bsum[gid] = mass;
        g->bsum[nb + gid] = px;
        g->bsum[2 * nb + gid] = py;
        g->bsum[3 * nb + gid] = (int32_t)nsolid;
        float n = (float)(bx * by);
        float m = (float)mass;
        float vx = 0.0f, vy = 0.0f;
        if (mass > 0) {
            float t = (float)px * 0.5f;
            vx = t / m;
            float u = (float)py * SQRT3_2;
            vy = u / m;
        }
        g->ux[gid] += alpha * (vx - g->ux[gid]);
        g->uy[gid] += alpha * (vy - g->uy[gid]);
        g->rho[gid] += alpha * (m / n - g->rho[gid]);
        g->sol[gid] = (float)nsolid / n;
    }
}

void lgo_bp_advance_sampling(lgo_bp *g, uint64_t n, uint64_t sample_every, float alpha) {
    uint64_t left = n, since = 0;
    while (left > 0) {
        bp_step(g);
        left -= 1;
        since += 1;
        if (sample_every > 0 && (since >= sample_every || left == 0)) {
            since = 0;
            bp_sample(g, alpha);
        }
    }
}

void lgo_bp_sample_field(lgo_bp *g, float alpha) { bp_sample(g, alpha); }

void lgo_bp_read_field(const lgo_bp *g, float *ux, float *uy, float *rho, float *sol) {
    size_t n = g->bw * g->bh;
    memcpy(ux, g->ux, n * 4);
    memcpy(uy, g->uy, n * 4);
    memcpy(rho, g->rho, n * 4);
    memcpy(sol, g->sol, n * 4);
}

void lgo_bp_read_block_sums(const lgo_bp *g, int32_t *mass, int32_t *px2, int32_t *py2,
                            int32_t *nsolid) {
    size_t n = g->bw * g->bh;
    memcpy(mass, g->bsum, n * 4);
    memcpy(px2, g->bsum + n, n * 4);
    memcpy(py2, g->bsum + 2 * n, n * 4);
    memcpy(nsolid, g->bsum + 3 * n, n * 4);
}

/* lgca_count (gpu.rs:381-395), summed in 64 bits. */
uint64_t lgo_bp_total_particles(const lgo_bp *g) {
    uint32_t lastbit = (uint32_t)((g->w - 1) % 32);
    uint32_t lastword = (uint32_t)((g->w - 1) / 32);
    uint32_t tail = (lastbit == 31) ? 0xffffffffu : ((1u << (lastbit + 1)) - 1u);
    uint64_t n = 0;
    for (int d = 0; d < 7; ++d)
        for (size_t y = 0; y < g->h; ++y)
            for (size_t j = 0; j < g->wpr; ++j)
                n += (uint64_t)__builtin_popcount(g->a[d * g->total + y * g->wpr + j] &
                                                  ((j == lastword) ? tail : 0xffffffffu));
    return n;
}

uint64_t lgo_bp_steps(const lgo_bp *g) { return g->steps; }
const uint32_t *lgo_bp_planes(const lgo_bp *g) { return g->a; }

/* GpuLattice::steps is a public field (gpu.rs:471); a lattice loaded from a run
 * that has already taken `steps` steps continues that run's random stream. */
void lgo_bp_set_steps(lgo_bp *g, uint64_t steps) { g->steps = steps; }

typedef struct {
    lgo_bp *g;
    const uint32_t *P;
    long r0, r1; /* rows r0 .. r1-1 of the lattice, taken mod h */
} window_job;

static void *window_worker(void *arg) {
    window_job *j = (window_job *)arg;
    lgo_bp *g = j->g;
    long h = (long)g->h;
    for (long r = j->r0; r < j->r1; ++r) {
        uint32_t y = (uint32_t)(((r % h) + h) % h);
        for (uint32_t x = 0; x < (uint32_t)g->wpr; ++x)
            step_word(g->a, g->b, g->solid, g->anysolid, j->P, g->rest, y, x);
    }
    return NULL;
}

/* n steps of the rows y0 .. y1-1 only, exactly as n full steps would leave them.
 * A row depends on rows y-1, y, y+1 of the step before, so step s of n updates the
 * window widened by n-1-s rows on each side; rows outside it go stale and are never
 * read by the rows that matter.  For checking a sub-window of a lattice too large to
 * step whole on the host.  Requires y1 - y0 + 2n <= h. */
void lgo_bp_advance_window(lgo_bp *g, uint64_t n, size_t y0, size_t y1) {
    for (uint64_t s = 0; s < n; ++s) {
        uint32_t P[18];
        lgo_bp_params(g->w, g->h, g->seed, g->steps, g->inlet_cols, g->thresh, P);
        long halo = (long)(n - 1 - s);
        long r0 = (long)y0 - halo, r1 = (long)y1 + halo;
        size_t nt = g->threads ? g->threads : 1;
        if (nt > 256) nt = 256;
        long rows = r1 - r0;
        long band = (rows + (long)nt - 1) / (long)nt;
        window_job jobs[256];
        pthread_t tid[256];
        size_t nj = 0;
        for (long r = r0; r < r1; r += band)
            jobs[nj++] = (window_job){g, P, r, r + band < r1 ? r + band : r1};
        if (nj == 1) window_worker(&jobs[0]);
        else {
            for (size_t i = 0; i < nj; ++i) pthread_create(&tid[i], NULL, window_worker, &jobs[i]);
            for (size_t i = 0; i < nj; ++i) pthread_join(tid[i], NULL);
        }
        uint32_t *t = g->a;
        g->a = g->b;
        g->b = t;
        g->steps += 1;
    }
}

/* The cells of rows y0 .. y1-1 (lgo_bp_store restricted to a band). */
void lgo_bp_store_rows(const lgo_bp *g, size_t y0, size_t y1, uint8_t *cells) {
    size_t w = g->w, wpr = g->wpr, total = g->total;
    for (size_t y = y0; y < y1; ++y)
        for (size_t x = 0; x < w; ++x) {
            size_t word = y * wpr + x / 32;
            uint32_t k = (uint32_t)(x % 32);
            uint8_t c = 0;
            for (int d = 0; d < 7; ++d) c |= (uint8_t)(((g->a[d * total + word] >> k) & 1u) << d);
            c |= (uint8_t)(((g->solid[word] >> k) & 1u) << 7);
            cells[(y - y0) * w + x] = c;
        }
}
