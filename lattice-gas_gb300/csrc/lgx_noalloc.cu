// lgx_noalloc.cu -- one lattice step that allocates no memory.
//
// Some callers cannot let a library call cudaMalloc behind their back: a host
// engine that carves every device buffer out of one arena it sized at start-up
// (and treats any other allocation as a bug), and loops that cannot afford the
// implicit device synchronisation cudaMalloc and cudaFree bring.  For them
// lgx_step_planes_noalloc advances a lattice whose buffers the caller owns, and
// keeps the one piece of scratch the step needs -- the inflow's Bernoulli words
// for the step, h x ceil(inlet_cols / 32) x 7 words -- in a fixed array compiled
// into this library instead of a per-call allocation.
//
// The array is a file-scope __device__ variable, so every GPU that loads the
// library holds it (kScratchWords words, 1 MiB) until the process exits.  Host
// code cannot use the array's name as a device address; the first call on each
// device looks the address up with cudaGetSymbolAddress while that device is
// current, and later calls reuse it.  The address belongs to the device's
// context: when that context has been destroyed and made again (cudaDeviceReset),
// the module is loaded afresh and the array may sit elsewhere, so the lookup is
// keyed on the context's unique id and repeated for a new context.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/lgx.h"
#include "lgx_internal.hpp"

namespace {

// Scratch capacity in 32-bit words: h * ceil(inlet_cols / 32) * 7 must fit.
constexpr size_t kScratchWords = 262144;  // 1 MiB

static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// The process-unique id of the context current on this thread, or 0 when there
// is none or the driver cannot say.  The driver entry points come through the
// runtime, so the library does not link the driver library itself.
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)f;
    cudaGetLastError();
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  unsigned long long id = 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_noalloc_scratch on the current device: looked up at the
// first call on the device, and again when the device's context is a new one
// (or its id cannot be read, in which case every call looks it up).
int scratch_address(int dev, uint32_t** out) {
  std::lock_guard<std::mutex> g(g_scratch_mu);
  unsigned long long ctx = current_context_id();
  if (!g_scratch_addr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      lgx::set_error(std::string("lgx_step_planes_noalloc: cudaGetSymbolAddress: ") +
                     cudaGetErrorString(e));
      return LGX_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
    g_scratch_ctx[dev] = current_context_id();  // the lookup makes the context current
  }
  *out = (uint32_t*)g_scratch_addr[dev];
  return LGX_OK;
}

}  // namespace

extern "C" int lgx_step_planes_noalloc(const uint32_t* planes_in, uint32_t* planes_out,
                                       const uint32_t* solid, const uint32_t* anysolid,
                                       size_t w, size_t h, int rest_particles,
                                       size_t inlet_cols, const uint32_t thresh[7],
                                       uint64_t seed, uint64_t steps, void* stream) {
  if (!planes_in || !planes_out || !solid || !anysolid || planes_in == planes_out) {
    lgx::set_error("lgx_step_planes_noalloc: null or aliased buffers");
    return LGX_ERR_ARG;
  }
  if (w > UINT32_MAX || h > UINT32_MAX || inlet_cols > UINT32_MAX) {
    lgx::set_error("lgx_step_planes_noalloc: w, h and inlet_cols must fit in 32 bits");
    return LGX_ERR_ARG;
  }
  if (h % 2 != 0 || w <= 4 || h <= 4 || ((w + 31) / 32) * h * 7 >= (1ull << 32)) {
    lgx::set_error("lgx_step_planes_noalloc: h must be even, w > 4, h > 4, and the lattice "
                   "within 32-bit word indices");
    return LGX_ERR_ARG;
  }
  const lgx::Dims dm = lgx::make_dims((uint32_t)w, (uint32_t)h, (uint32_t)inlet_cols);
  const size_t need = (size_t)dm.h * dm.iw * 7;
  if (need > kScratchWords) {
    lgx::set_error("lgx_step_planes_noalloc: the inflow needs " + std::to_string(need) +
                   " scratch words (h * ceil(inlet_cols / 32) * 7), more than the " +
                   std::to_string(kScratchWords) + " this entry point holds");
    return LGX_ERR_ARG;
  }
  if (dm.iw && !thresh) {
    lgx::set_error("lgx_step_planes_noalloc: an inflow needs its seven thresholds");
    return LGX_ERR_ARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    lgx::set_error("lgx_step_planes_noalloc: no usable current device");
    return LGX_ERR_NO_DEVICE;
  }
  uint32_t* scratch = nullptr;
  const int rc = scratch_address(dev, &scratch);  // first call on this device: the lookup
  if (rc) return rc;
  const cudaStream_t st = (cudaStream_t)stream;
  if (dm.iw) {
    // Every word the step reads is written here first; nothing needs zeroing.
    lgx::InletArgs ia;
    ia.out = scratch;
    ia.dm = dm;
    ia.seed = seed;
    ia.steps = steps;
    ia.nsteps = 1;
    for (int d = 0; d < 7; ++d) ia.thresh[d] = thresh[d];
    e = lgx::launch_inlet(ia, st);
    if (e != cudaSuccess) {
      lgx::set_error(std::string("lgx_step_planes_noalloc: ") + cudaGetErrorString(e));
      return LGX_ERR_CUDA;
    }
  }
  lgx::StepArgs sa;
  sa.a = planes_in;
  sa.b = planes_out;
  sa.solid = solid;
  sa.anysolid = anysolid;
  sa.inlet = dm.iw ? scratch : nullptr;
  sa.dm = dm;
  sa.seed = seed;
  sa.steps = steps;
  sa.words = 0;
  e = lgx::launch_step(sa, rest_particles != 0, st);
  if (e != cudaSuccess) {
    lgx::set_error(std::string("lgx_step_planes_noalloc: ") + cudaGetErrorString(e));
    return LGX_ERR_CUDA;
  }
  return LGX_OK;
}
