// lgx_resident.cu -- many steps of small lattices in one launch.
//
// A lattice of a few thousand words is too small to fill the GPU for one step,
// so stepping it one launch per step costs a launch's latency per step however
// little work the step is.  Here one thread-block cluster owns one lattice for
// a whole interval: its CTAs split the lattice's 32-word chunks between them,
// run the step on their chunks, meet at a cluster barrier (release / acquire at
// cluster scope, so every CTA's stores of the step are visible to the others'
// loads of the next; the next step's draws are made between arrive and wait),
// and go on to the next step, all inside one launch.  The
// planes are read through L2 (ld.global.cg), never the read-only path, since
// they change during the launch.  Sampling points are handled by the cluster
// itself between steps: each CTA coarse-grains a fixed share of the field
// blocks after the steps where its lattice is due.
//
// Clusters never wait on one another, so any number of lattices can share the
// launch; clusters the GPU cannot hold at once run when others finish.
#include <cooperative_groups.h>

#include "lgx_batch.hpp"
#include "lgx_step_impl.cuh"

namespace cg = cooperative_groups;

namespace lgx {
namespace {

template <int THREADS>
__global__ void __launch_bounds__(THREADS) lgx_resident_kernel(const ResidentArgs p) {
  const cg::cluster_group cluster = cg::this_cluster();
  const uint32_t csize = cluster.num_blocks(), rank = cluster.block_rank();
  const uint32_t li = p.first_lat + blockIdx.x / csize;
  const LatDesc& d = p.descs[li];
  const ResSched sch = p.sched[li];
  const Dims& dm = d.dm;
  const uint32_t nchunks = (dm.total + 31u) >> 5;
  const uint32_t c0 = (uint32_t)(((uint64_t)rank * nchunks) / csize);
  const uint32_t c1 = (uint32_t)(((uint64_t)(rank + 1u) * nchunks) / csize);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = THREADS / 32;
  const uint64_t base = p.base ? *p.base : 0ull;
  const uint32_t nb = d.bw * d.bh;

  // The draws of a warp's first chunk for step k are made while the cluster
  // barrier of step k - 1 is pending: they depend on (word, step) only.
  const uint32_t cfirst = c0 + warp;
  const uint32_t gfirst = min(cfirst * 32u + lane, dm.total - 1u);
  Draws first = draws(gfirst ^ step_seed32(d.seed, d.steps0 + base));
  for (uint32_t k = 0; k < p.len; ++k) {
    const uint64_t local = base + k;
    const uint32_t par = (d.cur0 + (uint32_t)local) & 1u;
    const uint32_t* src = par ? d.planes[1] : d.planes[0];
    uint32_t* dst = par ? d.planes[0] : d.planes[1];
    const uint32_t seed32 = step_seed32(d.seed, d.steps0 + local);
    const uint32_t* inlet = dm.iw ? d.inlet + (size_t)k * dm.h * dm.iw * 7u : nullptr;
    for (uint32_t c = cfirst; c < c1; c += nw) {
      uint32_t g = c * 32u + lane;
      const bool live = g < dm.total;
      if (!live) g = dm.total - 1u;
      const Draws s = c == cfirst ? first : draws(g ^ seed32);
      if (d.rest)
        step_word<true, true>(src, dst, d.solid, d.anysolid, inlet, dm, s, g, live);
      else
        step_word<false, true>(src, dst, d.solid, d.anysolid, inlet, dm, s, g, live);
    }
    // arrive (stores released at cluster scope), draw ahead, then wait
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    if (k + 1u < p.len) first = draws(gfirst ^ step_seed32(d.seed, d.steps0 + local + 1u));
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    // sampling point after step k + 1 of this launch
    const uint32_t t = k + 1u;
    const bool due = nb && sch.every &&
                     ((sch.since + t) % sch.every == 0u || t == sch.left);
    if (due) {
      SampleArgs sa;
      sa.a = dst;
      sa.solid = d.solid;
      sa.dm = dm;
      sa.bx = d.bx;
      sa.by = d.by;
      sa.bw = d.bw;
      sa.bh = d.bh;
      sa.alpha = d.alpha;
      sa.ux = d.field;
      sa.uy = d.field + nb;
      sa.rho = d.field + 2 * nb;
      sa.sol = d.field + 3 * nb;
      sa.sums = d.sums;
      for (uint32_t b = rank * nw + warp; b < nb; b += csize * nw) sample_block(sa, b);
    }
  }
}

template <int THREADS>
cudaError_t launch_resident_t(const ResidentArgs& a, uint32_t nlat, uint32_t csize,
                              cudaStream_t st) {
  if (csize > 8) {  // 16-CTA clusters are an opt-in per kernel (and device)
    cudaError_t e = cudaFuncSetAttribute(lgx_resident_kernel<THREADS>,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nlat * csize);
  cfg.blockDim = dim3(THREADS);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, lgx_resident_kernel<THREADS>, a);
}

}  // namespace

bool resident_config_valid(uint32_t csize, uint32_t threads) {
  return (csize == 1 || csize == 2 || csize == 4 || csize == 8 || csize == 16) &&
         (threads == 128 || threads == 256 || threads == 512 || threads == 1024);
}

cudaError_t launch_resident(const ResidentArgs& a, uint32_t nlat, uint32_t csize,
                            uint32_t threads, cudaStream_t st) {
  if (nlat == 0 || a.len == 0) return cudaSuccess;
  if (!resident_config_valid(csize, threads)) return cudaErrorInvalidValue;
  switch (threads) {
    case 128: return launch_resident_t<128>(a, nlat, csize, st);
    case 256: return launch_resident_t<256>(a, nlat, csize, st);
    case 512: return launch_resident_t<512>(a, nlat, csize, st);
    default: return launch_resident_t<1024>(a, nlat, csize, st);
  }
}

}  // namespace lgx
