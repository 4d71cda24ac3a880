/*
 * lg_transport.c -- CPU oracle for transport::measure (TEST INFRASTRUCTURE ONLY).
 *
 * A plain restatement of src/transport.rs: the row and column velocity
 * profiles (transport.rs:51-91), the two Fourier-mode measurements
 * (viscosity 183-221, advection_factor 225-289) with their decay window
 * (131-150), trajectories (107-127) and averaging (152-172), over either
 * backend of Sim (src/sim.rs): the byte-per-cell CPU lattice or the bitplane
 * lattice the GPU runs.  f32 arithmetic is not contracted (-ffp-contract=off),
 * sinf/cosf/atan2/log/sqrt are the C library's, as Rust's f32/f64 methods are.
 */
#include "lg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define TRANSIENT 200u     /* transport.rs:24-29 */
#define MIN_INTERVAL 4u
#define SAMPLES LGO_TRANSPORT_SAMPLES
#define REPS 4u
#define MAX_WINDOW 30000u

static const float SQRT3_2 = 0.8660254f;
static const float PI32 = 3.14159265358979323846f;

/* ---- row_ux / column_uy (transport.rs:51-91) ---------------------------- */
void lgo_row_ux(const uint8_t *cells, size_t w, size_t h, float *out) {
    for (size_t y = 0; y < h; ++y) {
        int64_t m[4];
        lgo_moments_sum(cells + y * w, w, 1, m);
        /* Moments::velocity().0 (moments.rs:91-97) */
        if (m[0] == 0) {
            out[y] = 0.0f;
        } else {
            float a = (float)m[1] * 0.5f;
            out[y] = a / (float)m[0];
        }
    }
}

void lgo_column_uy(const uint8_t *cells, size_t w, size_t h, float *out) {
    int64_t *mass = (int64_t *)calloc(w, sizeof(int64_t));
    int64_t *py2 = (int64_t *)calloc(w, sizeof(int64_t));
    for (size_t y = 0; y < h; ++y)
        for (size_t x = 0; x < w; ++x) {
            int64_t m[4];
            lgo_moments_sum(cells + y * w + x, 1, 1, m);
            mass[x] += m[0];
            py2[x] += m[2];
        }
    for (size_t x = 0; x < w; ++x) {
        if (mass[x] > 0) {
            float b = (float)py2[x] * SQRT3_2;
            out[x] = b / (float)mass[x];
        } else {
            out[x] = 0.0f;
        }
    }
    free(mass);
    free(py2);
}

/* ---- Sim over either backend (sim.rs) ----------------------------------- */
typedef struct {
    int gpu;
    size_t w, h;
    lgo_lattice *cpu;
    lgo_bp *bp;
    uint8_t *cache;
} sim_t;

/* box_of (transport.rs:176-179): Lattice::new(size, size, density, (0,0), 0,
 * rest, threads, 1), then Sim::new (sim.rs:35-67). */
static void sim_box(sim_t *s, size_t size, float density, int rest, size_t threads, int gpu) {
    memset(s, 0, sizeof(*s));
    s->gpu = gpu;
    s->w = s->h = size;
    s->cache = (uint8_t *)calloc(size * size, 1);
    if (gpu) {
        s->bp = lgo_bp_new(size, size, rest, 1, threads);
        lgo_bp_set_inlet(s->bp, 0, density, 0.0f, 0.0f, rest);
        lgo_bp_load(s->bp, s->cache);
    } else {
        s->cpu = lgo_new(size, size, density, 0.0f, 0.0f, 0, rest, threads, 1);
    }
}

static void sim_free(sim_t *s) {
    if (s->bp) lgo_bp_free(s->bp);
    if (s->cpu) lgo_free(s->cpu);
    free(s->cache);
}

static void sim_restart(sim_t *s, const uint8_t *cells, uint64_t seed) {
    if (s->gpu)
        lgo_bp_restart(s->bp, cells, seed);
    else
        lgo_restart(s->cpu, cells, seed);
}

static void sim_advance(sim_t *s, uint64_t n) {
    if (s->gpu)
        lgo_bp_advance_sampling(s->bp, n, 0, 0.0f);
    else
        lgo_advance(s->cpu, n);
}

static const uint8_t *sim_cells(sim_t *s) {
    if (s->gpu) {
        lgo_bp_store(s->bp, s->cache);
        return s->cache;
    }
    return lgo_cells(s->cpu);
}

/* ---- one measurement ---------------------------------------------------- */
typedef struct {
    int adv;
    float density, k;
    int rest;
    uint64_t seed;
    size_t n;
    float *cs, *sn, *wave;  /* cos, sin of the phase; the start's velocity wave */
    float *u;
} meas_t;

static void project(const meas_t *m, const uint8_t *cells, double *a_out, double *b_out) {
    if (m->adv)
        lgo_column_uy(cells, m->n, m->n, m->u);
    else
        lgo_row_ux(cells, m->n, m->n, m->u);
    double a = 0.0, b = 0.0;
    for (size_t i = 0; i < m->n; ++i) {
        float ca = m->u[i] * m->cs[i];
        float sb = m->u[i] * m->sn[i];
        a += (double)ca;
        b += (double)sb;
    }
    *a_out = 2.0 * a / (double)m->n;
    *b_out = 2.0 * b / (double)m->n;
}

static uint64_t start_seed(const meas_t *m, uint64_t rep) {
    uint64_t s = m->seed ^ ((rep * 0x9E3779B9ull) << 20);
    return m->adv ? s ^ 0x1357ull : s;
}

/* The start closures (transport.rs:187-200, 235-252). */
static void start_cells(const meas_t *m, uint64_t rep, uint8_t *cells) {
    uint64_t s = start_seed(m, rep);
    if (m->adv)
        lgo_cells_column_wave(cells, m->n, m->n, m->density, 0.25f, m->wave, m->rest,
                              s ^ 0xF00Dull);
    else
        lgo_cells_shear_wave(cells, m->n, m->n, m->density, m->wave, m->rest, s ^ 0xBEEFull);
}

static uint64_t decay_window(sim_t *sim, const meas_t *m, uint8_t *cells) {
    start_cells(m, 0, cells);
    sim_restart(sim, cells, start_seed(m, 0));
    sim_advance(sim, TRANSIENT);
    double a, b;
    project(m, sim_cells(sim), &a, &b);
    double a0 = sqrt(a * a + b * b);
    if (a0 < 1e-12) a0 = 1e-12;
    uint64_t t = 0;
    while (t < MAX_WINDOW) {
        sim_advance(sim, 25);
        t += 25;
        project(m, sim_cells(sim), &a, &b);
        if (sqrt(a * a + b * b) < a0 / 3.0) break;
    }
    if (t < (uint64_t)SAMPLES * MIN_INTERVAL) t = (uint64_t)SAMPLES * MIN_INTERVAL;
    if (t > MAX_WINDOW) t = MAX_WINDOW;
    return t;
}

/* averaged (transport.rs:152-172): mode[2 * i], mode[2 * i + 1]. */
static uint64_t averaged(sim_t *sim, const meas_t *m, double *mode, uint64_t *window) {
    uint8_t *cells = (uint8_t *)malloc(m->n * m->n);
    *window = decay_window(sim, m, cells);
    uint64_t interval = *window / SAMPLES;
    if (interval < MIN_INTERVAL) interval = MIN_INTERVAL;
    memset(mode, 0, 2 * SAMPLES * sizeof(double));
    for (uint64_t rep = 0; rep < REPS; ++rep) {
        start_cells(m, rep, cells);
        sim_restart(sim, cells, start_seed(m, rep));
        sim_advance(sim, TRANSIENT);
        for (int i = 0; i < SAMPLES; ++i) {
            double a, b;
            project(m, sim_cells(sim), &a, &b);
            mode[2 * i] += a / (double)REPS;
            mode[2 * i + 1] += b / (double)REPS;
            sim_advance(sim, interval);
        }
    }
    free(cells);
    return interval;
}

static double fit_slope(const double *x, const double *y, int n) {
    double N = (double)n, sx = 0.0, sy = 0.0, sxx = 0.0, sxy = 0.0;
    for (int i = 0; i < n; ++i) sx += x[i];
    for (int i = 0; i < n; ++i) sy += y[i];
    for (int i = 0; i < n; ++i) sxx += x[i] * x[i];
    for (int i = 0; i < n; ++i) sxy += x[i] * y[i];
    return (N * sxy - sx * sy) / (N * sxx - sx * sx);
}

static void meas_init(meas_t *m, int adv, float density, int rest, uint64_t seed, size_t size) {
    m->adv = adv;
    m->density = density;
    m->rest = rest;
    m->seed = seed;
    m->n = size;
    m->cs = (float *)malloc(size * sizeof(float));
    m->sn = (float *)malloc(size * sizeof(float));
    m->wave = (float *)malloc(size * sizeof(float));
    m->u = (float *)malloc(size * sizeof(float));
    if (adv) {
        m->k = 2.0f * PI32 / (float)size;
    } else {
        float hs = (float)size * SQRT3_2;
        m->k = 2.0f * PI32 / hs;
    }
    for (size_t i = 0; i < size; ++i) {
        float p = m->k * (float)i;
        if (!adv) p = p * SQRT3_2;
        m->cs[i] = cosf(p);
        m->sn[i] = sinf(p);
        m->wave[i] = 0.05f * sinf(p);
    }
}

static void meas_free(meas_t *m) {
    free(m->cs);
    free(m->sn);
    free(m->wave);
    free(m->u);
}

void lgo_transport_measure(float density, int rest, size_t threads, uint64_t seed, size_t size,
                           int gpu, lgo_transport *out) {
    memset(out, 0, sizeof(*out));
    double t[SAMPLES], y[SAMPLES];
    /* viscosity (transport.rs:183-221) */
    {
        meas_t m;
        meas_init(&m, 0, density, rest, seed, size);
        sim_t sim;
        sim_box(&sim, size, density, rest, threads, gpu);
        uint64_t interval = averaged(&sim, &m, out->mode_nu, &out->window_nu);
        for (int i = 0; i < SAMPLES; ++i) {
            double a = out->mode_nu[2 * i], b = out->mode_nu[2 * i + 1];
            double r = sqrt(a * a + b * b);
            t[i] = (double)((uint64_t)i * interval);
            y[i] = log(r > 1e-12 ? r : 1e-12);
        }
        float kk = m.k * m.k;
        out->nu = (float)(-fit_slope(t, y, SAMPLES) / (double)kk);
        sim_free(&sim);
        meas_free(&m);
    }
    /* advection_factor (transport.rs:225-289) */
    {
        meas_t m;
        meas_init(&m, 1, density, rest, seed, size);
        uint8_t *cells = (uint8_t *)malloc(size * size);
        start_cells(&m, 0, cells);
        int64_t s[4];
        lgo_moments_sum(cells, size * size, 1, s);
        float u_actual = 0.0f;
        if (s[0] != 0) {
            float a = (float)s[1] * 0.5f;
            u_actual = a / (float)s[0];
        }
        free(cells);
        out->u_actual = u_actual;
        sim_t sim;
        sim_box(&sim, size, density, rest, threads, gpu);
        uint64_t interval = averaged(&sim, &m, out->mode_g, &out->window_g);
        double unwrapped = 0.0;
        double prev = atan2(out->mode_g[0], out->mode_g[1]);
        for (int i = 0; i < SAMPLES; ++i) {
            double ph = atan2(out->mode_g[2 * i], out->mode_g[2 * i + 1]);
            double delta = ph - prev;
            while (delta > M_PI) delta -= 2.0 * M_PI;
            while (delta < -M_PI) delta += 2.0 * M_PI;
            unwrapped += delta;
            prev = ph;
            t[i] = (double)((uint64_t)i * interval);
            y[i] = unwrapped;
        }
        float ku = m.k * u_actual;
        out->g = (float)(-fit_slope(t, y, SAMPLES) / (double)ku);
        sim_free(&sim);
        meas_free(&m);
    }
}
