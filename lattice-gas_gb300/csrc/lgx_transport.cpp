// lgx_transport.cpp -- transport::measure (src/transport.rs:31-319) on the engine.
//
// The reference measures the fluid's viscosity nu and advection factor g by
// watching one Fourier mode of a periodic box: a shear wave (row_ux projected
// on the mode along y) for nu, a transverse wave on a uniform stream
// (column_uy projected along x) for g.  On the GPU path it restarts one
// lattice per realisation and gathers the whole lattice to the host for every
// sample.  Here every realisation of every measurement is a lattice of one
// batch: the starts are filled on the device, each lattice's profile is
// formed on the device at its own sample points inside the batch's captured
// graphs, and only the profiles come back.  The projections, the averaging and
// the fits are the reference's f32 / f64 arithmetic on the host, in the same
// order, so nu and g are those transport::measure finds on the bitplane path.
//
// Two phases, as transport::averaged (transport.rs:152-172) runs them:
//  1. decay windows: start(0) of every measurement, TRANSIENT steps, then the
//     mode every 25 steps until it falls below a third of its first value
//     (decay_window, transport.rs:131-150).  All windows are searched at once;
//     the lattices run ahead in chunks, and a sample past a lattice's crossing
//     is never looked at, so the windows are the reference's.
//  2. trajectories: REPS realisations of every measurement, each measurement
//     with its own interval max(window / SAMPLES, MIN_INTERVAL), SAMPLES
//     samples after the transient (trajectory, transport.rs:107-127).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include "../../include/lgx.h"
#include "lgx_batch.hpp"
#include "lgx_handle.hpp"
#include "lgx_profile.hpp"

namespace {

constexpr uint64_t kTransient = 200;   // transport.rs:24-29
constexpr uint64_t kMinInterval = 4;
constexpr int kSamples = LGX_TRANSPORT_SAMPLES;
constexpr uint64_t kReps = 4;
constexpr uint64_t kMaxWindow = 30000;
constexpr uint64_t kBlock = 25;        // decay_window's step between looks
constexpr uint64_t kWindowLooks = kMaxWindow / kBlock;
constexpr float kPi = 3.14159265358979323846f;  // std::f32::consts::PI
constexpr double kPi64 = 3.14159265358979323846;
constexpr float kSqrt3_2 = 0.8660254f;

int cuda_fail(cudaError_t e, const char* what) {
  lgx::set_error(std::string("lgx_transport_measure: ") + what + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? LGX_ERR_ALLOC : LGX_ERR_CUDA;
}

#define LGX_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

#define LGX_RC(call)          \
  do {                        \
    const int rc_ = (call);   \
    if (rc_) return rc_;      \
  } while (0)

// One measurement: the viscosity (shear wave, rows) or the advection factor
// (transverse wave, columns) at one density.
struct Meas {
  bool adv = false;
  float density = 0;
  uint64_t seed = 0;
  uint32_t n = 0;            // profile length: h for rows, w for columns
  float k = 0;
  std::vector<float> cs, sn; // cos and sin of the mode's phase at each row / column
  uint32_t* d_thresh = nullptr;  // start thresholds, [n][7]
  uint64_t window = 0, interval = 0;
  bool found = false;
  double a0 = 0;
  float u_actual = 0;
  std::vector<double> mode;  // averaged (a, b) per sample
};

// The projection closures of viscosity and advection_factor
// (transport.rs:202-211, 255-264).
void project(const Meas& m, const float* u, double* a_out, double* b_out) {
  double a = 0.0, b = 0.0;
  for (uint32_t i = 0; i < m.n; ++i) {
    const float ca = u[i] * m.cs[i];
    const float sb = u[i] * m.sn[i];
    a += (double)ca;
    b += (double)sb;
  }
  *a_out = 2.0 * a / (double)m.n;
  *b_out = 2.0 * b / (double)m.n;
}

// fit_slope (transport.rs:93-100).
double fit_slope(const std::vector<double>& x, const std::vector<double>& y) {
  const double n = (double)x.size();
  double sx = 0.0, sy = 0.0, sxx = 0.0, sxy = 0.0;
  for (double v : x) sx += v;
  for (double v : y) sy += v;
  for (double v : x) sxx += v * v;
  for (size_t i = 0; i < x.size(); ++i) sxy += x[i] * y[i];
  return (n * sxy - sx * sy) / (n * sxx - sx * sx);
}

// The seed of realisation `rep` (transport.rs:188, 236).
uint64_t start_seed(const Meas& m, uint64_t rep) {
  const uint64_t s = m.seed ^ ((rep * 0x9E3779B9ull) << 20);
  return m.adv ? s ^ 0x1357ull : s;
}

struct Run {
  std::vector<Meas> meas;
  std::vector<lgx_lattice*> lats;  // [meas][rep]
  std::vector<void*> dev;          // device allocations
  lgx_batch* batch = nullptr;
  lgx::ProfDesc* d_prof = nullptr;
  uint32_t nprof = 0, max_h = 0;
  int device = 0;

  ~Run() {
    if (batch) lgx_batch_destroy(batch);
    for (lgx_lattice* l : lats)
      if (l) lgx_destroy(l);
    cudaSetDevice(device);
    for (void* p : dev) cudaFree(p);
  }
  int alloc(void** p, size_t bytes) {
    LGX_CUDA(cudaMalloc(p, bytes));
    dev.push_back(*p);
    return LGX_OK;
  }
};

cudaError_t profile_hook(void* ctx, cudaStream_t st, const uint64_t* base, uint32_t k_after) {
  Run* r = (Run*)ctx;
  const lgx::ProfArgs pa{r->d_prof, r->nprof, base, k_after};
  return lgx::launch_profile(pa, r->max_h, st);
}

// Restart lattice l from realisation `rep` of measurement m, on the device:
// Sim::restart(start.cells, start.seed) with the start's cells drawn as
// transport.rs:189-199 (rows) or 237-251 (columns) draw them.
int restart(Meas& m, uint64_t rep, lgx_lattice* l) {
  const uint64_t s = start_seed(m, rep);
  lgx::EqFill f{};
  f.planes = l->planes[l->cur];
  f.solid = l->solid;
  f.dm = l->dm;
  f.seed = s ^ (m.adv ? 0xF00Dull : 0xBEEFull);
  f.rest = l->rest;
  if (m.adv)
    f.thresh_cols = m.d_thresh;
  else
    f.thresh_rows = m.d_thresh;
  LGX_CUDA(ensure_fill_scratch(l));
  f.scratch = l->fill_scratch;
  LGX_CUDA(lgx::launch_equilibrium_fill(f, l->stream));
  l->launches += 2;
  l->seed = s;
  l->steps = 0;
  l->inlet_valid = 0;
  return LGX_OK;
}

// Profile descriptors for lattices lats[i], with trajectories traj[i] of
// `count` samples at phase steps first + j * every[i]; offset = phase steps
// already run.  Uploaded before each advance: the planes' parity moves.
int upload_profiles(Run& r, const std::vector<lgx_lattice*>& lats,
                    const std::vector<const Meas*>& ms, const std::vector<float*>& traj,
                    const std::vector<int32_t*>& scratch, const std::vector<uint64_t>& every,
                    uint32_t count, uint64_t offset) {
  std::vector<lgx::ProfDesc> d(lats.size());
  for (size_t i = 0; i < lats.size(); ++i) {
    lgx_lattice* l = lats[i];
    lgx::ProfDesc& p = d[i];
    p.planes[0] = l->planes[l->cur];
    p.planes[1] = l->planes[l->cur ^ 1];
    p.cur0 = 0;
    p.dm = l->dm;
    p.rows = scratch[i];
    p.cols = p.rows + 3 * (size_t)l->dm.h;
    p.done = (uint32_t*)(p.cols + 3 * (size_t)l->dm.w);
    p.row_u = ms[i]->adv ? nullptr : traj[i];
    p.col_u = ms[i]->adv ? traj[i] : nullptr;
    p.col_sums = nullptr;
    p.offset = offset;
    p.first = kTransient;
    p.every = every[i];
    p.count = count;
  }
  LGX_CUDA(cudaMemcpy(r.d_prof, d.data(), d.size() * sizeof(lgx::ProfDesc),
                      cudaMemcpyHostToDevice));
  r.nprof = (uint32_t)d.size();
  return LGX_OK;
}

// per_step: the profile hook after every step (every lattice one launch per
// step); otherwise at the end of every interval, which the advances end at
// the sampling points, with the size classes stepped as the tuner finds fastest.
int new_batch(Run& r, const std::vector<lgx_lattice*>& lats, bool per_step) {
  if (r.batch) {
    lgx_batch_destroy(r.batch);
    r.batch = nullptr;
  }
  LGX_RC(lgx_batch_create_ex(lats.data(), lats.size(),
                             per_step ? LGX_BATCH_PER_STEP : LGX_BATCH_AUTO, &r.batch));
  return lgx::batch_set_step_hook(r.batch, profile_hook, &r, per_step);
}

int measure(const float* densities, size_t n, int rest, uint64_t seed, size_t size,
            lgx_transport* out) {
  Run r;
  LGX_CUDA(cudaGetDevice(&r.device));
  const uint32_t N = (uint32_t)size;
  r.max_h = N;
  // the measurements: nu then g for each density
  r.meas.resize(2 * n);
  for (size_t i = 0; i < 2 * n; ++i) {
    Meas& m = r.meas[i];
    m.adv = (i & 1) != 0;
    m.density = densities[i / 2];
    m.seed = seed;
    m.n = N;
    std::vector<uint32_t> t((size_t)N * 7);
    if (!m.adv) {
      // viscosity: k = 2 pi / (h sqrt(3)/2); row y at u_x = amp sin(k y sqrt(3)/2)
      m.k = 2.0f * kPi / ((float)N * kSqrt3_2);
      for (uint32_t y = 0; y < N; ++y) {
        const float p = m.k * (float)y * kSqrt3_2;
        m.cs.push_back(cosf(p));
        m.sn.push_back(sinf(p));
        const float ux = 0.05f * sinf(p);
        lgx::equilibrium_thresholds(m.density, ux, 0.0f, rest != 0, &t[(size_t)y * 7]);
      }
    } else {
      // advection: k = 2 pi / w; column x at (u0, amp sin(k x))
      m.k = 2.0f * kPi / (float)N;
      for (uint32_t x = 0; x < N; ++x) {
        const float p = m.k * (float)x;
        m.cs.push_back(cosf(p));
        m.sn.push_back(sinf(p));
        const float uy = 0.05f * sinf(p);
        lgx::equilibrium_thresholds(m.density, 0.25f, uy, rest != 0, &t[(size_t)x * 7]);
      }
    }
    void* p = nullptr;
    LGX_RC(r.alloc(&p, t.size() * 4));
    m.d_thresh = (uint32_t*)p;
    LGX_CUDA(cudaMemcpy(m.d_thresh, t.data(), t.size() * 4, cudaMemcpyHostToDevice));
  }
  // lattices: box_of (transport.rs:176-179): a quiescent periodic box, no inflow
  const size_t M = r.meas.size();
  r.lats.assign(M * kReps, nullptr);
  for (size_t i = 0; i < M * kReps; ++i) {
    LGX_RC(lgx_create(N, N, rest, 1, &r.lats[i]));
    LGX_RC(lgx_set_inlet(r.lats[i], 0, r.meas[i / kReps].density, 0.0f, 0.0f, rest));
  }
  {
    void* p = nullptr;
    LGX_RC(r.alloc(&p, M * kReps * sizeof(lgx::ProfDesc)));
    r.d_prof = (lgx::ProfDesc*)p;
  }
  // profile scratch per lattice (column sums and counter start at zero)
  const size_t scratch_words = lgx::profile_scratch_words(N, N);
  std::vector<int32_t*> scratch(M * kReps);
  for (size_t i = 0; i < M * kReps; ++i) {
    void* p = nullptr;
    LGX_RC(r.alloc(&p, scratch_words * 4));
    LGX_CUDA(cudaMemset(p, 0, scratch_words * 4));
    scratch[i] = (int32_t*)p;
  }

  // ---- phase 1: decay windows, from start(0) ----
  std::vector<lgx_lattice*> l1(M);
  std::vector<const Meas*> m1(M);
  std::vector<float*> traj1(M);
  std::vector<int32_t*> s1(M);
  std::vector<uint64_t> ev1(M, kBlock);
  const uint32_t looks = (uint32_t)kWindowLooks + 1;  // a0 and up to 1200 looks
  for (size_t i = 0; i < M; ++i) {
    l1[i] = r.lats[i * kReps];
    m1[i] = &r.meas[i];
    s1[i] = scratch[i * kReps];
    void* p = nullptr;
    LGX_RC(r.alloc(&p, (size_t)looks * N * 4));
    traj1[i] = (float*)p;
    LGX_RC(restart(r.meas[i], 0, l1[i]));
  }
  // the realised mean speed of the advection start (transport.rs:267-268)
  for (size_t i = 0; i < M; ++i) {
    if (!r.meas[i].adv) continue;
    std::vector<int32_t> rows(3 * (size_t)N);
    LGX_RC(lgx_line_sums(l1[i], rows.data(), rows.size(), nullptr, 0));
    int64_t mass = 0, px2 = 0;
    for (uint32_t y = 0; y < N; ++y) {
      mass += rows[y];
      px2 += rows[N + y];
    }
    r.meas[i].u_actual = mass ? (float)px2 * 0.5f / (float)mass : 0.0f;
  }
  LGX_RC(new_batch(r, l1, false));
  uint64_t ran = 0, seen = 0;  // phase steps run; looks evaluated (slot index)
  std::vector<float> u((size_t)looks * N);
  size_t pending = M;
  while (pending) {
    const uint64_t last = kTransient + kBlock * kWindowLooks;
    const uint64_t target = std::min(last, ran == 0 ? kTransient + kBlock * 40 : ran + 2000);
    LGX_RC(upload_profiles(r, l1, m1, traj1, s1, ev1, looks, ran));
    // intervals of 25 steps: every phase step that is a multiple of 25 ends one
    LGX_RC(lgx_batch_advance_sampling(r.batch, target - ran, kBlock, 0.0f));
    ran = target;
    const uint64_t avail = (ran - kTransient) / kBlock + 1;  // slots written
    for (size_t i = 0; i < M; ++i) {
      Meas& m = r.meas[i];
      if (m.found) continue;
      LGX_CUDA(cudaMemcpy(u.data() + seen * N, traj1[i] + seen * N, (avail - seen) * N * 4,
                          cudaMemcpyDeviceToHost));
      for (uint64_t j = seen; j < avail && !m.found; ++j) {
        double a, b;
        project(m, u.data() + j * N, &a, &b);
        const double amp = sqrt(a * a + b * b);
        if (j == 0) {
          m.a0 = std::max(amp, 1e-12);
        } else if (amp < m.a0 / 3.0) {
          m.window = j * kBlock;
          m.found = true;
        }
      }
      if (!m.found && avail == looks) {
        m.window = kMaxWindow;
        m.found = true;
      }
      if (m.found) {
        m.window = std::min(std::max(m.window, (uint64_t)kSamples * kMinInterval), kMaxWindow);
        m.interval = std::max(m.window / kSamples, kMinInterval);
        --pending;
      }
    }
    seen = avail;
  }

  // ---- phase 2: REPS trajectories of every measurement ----
  std::vector<lgx_lattice*> l2(M * kReps);
  std::vector<const Meas*> m2(M * kReps);
  std::vector<float*> traj2(M * kReps);
  std::vector<uint64_t> ev2(M * kReps);
  uint64_t longest = 0;
  for (size_t i = 0; i < M * kReps; ++i) {
    Meas& m = r.meas[i / kReps];
    l2[i] = r.lats[i];
    m2[i] = &m;
    ev2[i] = m.interval;
    longest = std::max(longest, m.interval);
    traj2[i] = traj1[i / kReps] + (size_t)(i % kReps) * kSamples * N;  // reuse phase-1 space
    LGX_RC(restart(m, i % kReps, l2[i]));
  }
  // The last sample is taken after TRANSIENT + (SAMPLES - 1) * interval steps;
  // the reference's final advance after it changes nothing it looks at.  With
  // few sampling points (of any measurement) the batch advances from one to the
  // next, each advance one interval ending at the point (a host round trip per
  // point); with many, one advance runs every step with the profile hook after
  // each (an extra launch per step, the lattices' own sampling steps picked on
  // the device).
  std::vector<uint64_t> points;
  for (const Meas& m : r.meas)
    for (int j = 0; j < kSamples; ++j) points.push_back(kTransient + (uint64_t)j * m.interval);
  std::sort(points.begin(), points.end());
  points.erase(std::unique(points.begin(), points.end()), points.end());
  const uint64_t total = kTransient + (kSamples - 1) * longest;
  const bool per_step = points.size() * 16 > total;
  LGX_RC(new_batch(r, l2, per_step));
  if (per_step) {
    LGX_RC(upload_profiles(r, l2, m2, traj2, scratch, ev2, kSamples, 0));
    LGX_RC(lgx_batch_advance(r.batch, total));
  } else {
    ran = 0;
    for (uint64_t pt : points) {
      LGX_RC(upload_profiles(r, l2, m2, traj2, scratch, ev2, kSamples, ran));
      LGX_RC(lgx_batch_advance_sampling(r.batch, pt - ran, pt - ran, 0.0f));
      ran = pt;
    }
  }
  std::vector<float> tr((size_t)kSamples * N);
  for (size_t mi = 0; mi < M; ++mi) {
    Meas& m = r.meas[mi];
    m.mode.assign(2 * kSamples, 0.0);
    for (uint64_t rep = 0; rep < kReps; ++rep) {
      LGX_CUDA(cudaMemcpy(tr.data(), traj2[mi * kReps + rep], tr.size() * 4,
                          cudaMemcpyDeviceToHost));
      for (int j = 0; j < kSamples; ++j) {
        double a, b;
        project(m, tr.data() + (size_t)j * N, &a, &b);
        m.mode[2 * j] += a / (double)kReps;
        m.mode[2 * j + 1] += b / (double)kReps;
      }
    }
  }

  // ---- the fits (transport.rs:213-220, 270-289) ----
  for (size_t d = 0; d < n; ++d) {
    const Meas& mv = r.meas[2 * d];
    const Meas& mg = r.meas[2 * d + 1];
    lgx_transport& o = out[d];
    memset(&o, 0, sizeof(o));
    std::vector<double> t(kSamples), y(kSamples);
    for (int j = 0; j < kSamples; ++j) {
      t[j] = (double)((uint64_t)j * mv.interval);
      const double a = mv.mode[2 * j], b = mv.mode[2 * j + 1];
      y[j] = log(std::max(sqrt(a * a + b * b), 1e-12));
    }
    o.nu = (float)(-fit_slope(t, y) / (double)(mv.k * mv.k));
    double unwrapped = 0.0;
    double prev = atan2(mg.mode[0], mg.mode[1]);
    for (int j = 0; j < kSamples; ++j) {
      t[j] = (double)((uint64_t)j * mg.interval);
      const double ph = atan2(mg.mode[2 * j], mg.mode[2 * j + 1]);
      double delta = ph - prev;
      while (delta > kPi64) delta -= 2.0 * kPi64;
      while (delta < -kPi64) delta += 2.0 * kPi64;
      unwrapped += delta;
      prev = ph;
      y[j] = unwrapped;
    }
    o.g = (float)(-fit_slope(t, y) / (double)(mg.k * mg.u_actual));
    o.window_nu = mv.window;
    o.window_g = mg.window;
    o.u_actual = mg.u_actual;
    for (int j = 0; j < 2 * kSamples; ++j) {
      o.mode_nu[j] = mv.mode[j];
      o.mode_g[j] = mg.mode[j];
    }
  }
  return LGX_OK;
}

}  // namespace

extern "C" int lgx_transport_measure(const float* densities, size_t n, int rest, uint64_t seed,
                                     size_t size, lgx_transport* out) {
  if (!densities || !out || n == 0) {
    lgx::set_error("lgx_transport_measure: need densities and one result per density");
    return LGX_ERR_ARG;
  }
  if (size < 8 || size % 2 != 0 || size > 16384) {
    lgx::set_error("lgx_transport_measure: size must be even, 8 .. 16384");
    return LGX_ERR_ARG;
  }
  if (n * 2 * kReps > 65535) {
    lgx::set_error("lgx_transport_measure: too many densities for one batch");
    return LGX_ERR_ARG;
  }
  return measure(densities, n, rest, seed, size, out);
}
