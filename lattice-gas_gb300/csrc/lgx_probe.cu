// lgx_probe.cu -- integer-pipe throughput probes for the roofline.
//
// The step kernel is a chain of 32-bit logic (lop3), shifts and multiplies,
// with 14 bits of memory traffic per cell, so its ceiling is the integer
// issue rate rather than HBM.  These kernels measure that rate on the device
// at hand: every thread runs eight independent dependency chains of one
// instruction kind, enough blocks fill every SM, and CUDA events time it.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lgx.h"
#include "lgx_internal.hpp"

namespace lgx {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

template <int OP>
__global__ void __launch_bounds__(256) probe_kernel(uint32_t seed, uint32_t* sink) {
  uint32_t x[kChains];
  const uint32_t y = seed ^ threadIdx.x, z = seed * 3u + blockIdx.x;
#pragma unroll
  for (int i = 0; i < kChains; ++i) x[i] = seed + i * 0x9e3779b9u + threadIdx.x;
#pragma unroll 1
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) {
      if (OP == 0)
        asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(x[i]) : "r"(y), "r"(z));
      else if (OP == 1)
        asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(x[i]) : "r"(y), "r"(z));
      else if (OP == 2)
        asm volatile("shf.r.wrap.b32 %0, %0, %1, 13;" : "+r"(x[i]) : "r"(y));
      else if (OP == 3)
        asm volatile("add.u32 %0, %0, %1;" : "+r"(x[i]) : "r"(y));
      else
        asm volatile("mul.hi.u32 %0, %0, %1;" : "+r"(x[i]) : "r"(y));
    }
  }
  uint32_t acc = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) acc ^= x[i];
  if (acc == 0x12345678u) sink[0] = acc;  // keeps the chains live
}

}  // namespace
}  // namespace lgx

extern "C" int lgx_probe_int_rate(int op, double* ops_per_s) {
  if (!ops_per_s || op < 0 || op > 4) {
    lgx::set_error("lgx_probe_int_rate: op must be 0..4");
    return LGX_ERR_ARG;
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    lgx::set_error("no CUDA device on this machine");
    return LGX_ERR_NO_DEVICE;
  }
  uint32_t* sink = nullptr;
  cudaEvent_t a, b;
  if (cudaMalloc(&sink, 4) != cudaSuccess) {
    lgx::set_error("lgx_probe_int_rate: cudaMalloc failed");
    return LGX_ERR_ALLOC;
  }
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = sms * 8, threads = 256;
  auto launch = [&](void) {
    switch (op) {
      case 0: lgx::probe_kernel<0><<<blocks, threads>>>(7u, sink); break;
      case 1: lgx::probe_kernel<1><<<blocks, threads>>>(7u, sink); break;
      case 2: lgx::probe_kernel<2><<<blocks, threads>>>(7u, sink); break;
      case 3: lgx::probe_kernel<3><<<blocks, threads>>>(7u, sink); break;
      default: lgx::probe_kernel<4><<<blocks, threads>>>(7u, sink); break;
    }
  };
  launch();  // warm-up
  cudaEventRecord(a);
  for (int r = 0; r < 5; ++r) launch();
  cudaEventRecord(b);
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  if (e != cudaSuccess) {
    lgx::set_error(std::string("lgx_probe_int_rate: ") + cudaGetErrorString(e));
    return LGX_ERR_CUDA;
  }
  const double ops = 5.0 * blocks * threads * (double)lgx::kIters * lgx::kChains;
  *ops_per_s = ops / (ms * 1e-3);
  return LGX_OK;
}
