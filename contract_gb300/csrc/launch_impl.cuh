// Launch helpers shared by the kernel translation units.
#pragma once

#include <algorithm>
#include <mutex>

#include "launch.hpp"

namespace cgb {

// Tile geometry for an op with `sites` sites per tile, its chunks dealt
// round-robin to `ctas` persistent CTAs.  About `chunks_per_cta` chunks per
// CTA keeps the round-robin tail (CTAs that draw one chunk more than others)
// near 1/chunks_per_cta of a CTA's work; chunks never span segments and hold
// at most 64 tiles.
inline TileGeom make_geom(const Job &job, int sites, long long ctas, int chunks_per_cta)
{
  TileGeom g {};
  g.volume = job.volume;
  if (job.per_site) {
    g.seg_len = job.volume;
    g.num_segs = 1;
    g.per_site = 1;
  } else {
    g.seg_len = job.half_slice;
    g.num_segs = 2 * job.lt;
    g.per_site = 0;
  }
  g.tiles_per_seg = (int)((g.seg_len + sites - 1) / sites);
  const long long tiles = (long long)g.tiles_per_seg * g.num_segs;
  long long ct = tiles / (std::max(1LL, ctas) * chunks_per_cta);
  g.chunk_tiles = (int)std::max(1LL, std::min(ct, 64LL));
  g.chunk_tiles = std::min(g.chunk_tiles, g.tiles_per_seg);
  g.chunks_per_seg = (g.tiles_per_seg + g.chunk_tiles - 1) / g.chunk_tiles;
  g.total_chunks = g.chunks_per_seg * g.num_segs;
  g.wait_ns = job.wait_ns ? job.wait_ns : kWaitLimitNs;
  g.withhold_chunk = job.withhold_chunk;
  return g;
}

// Chunks per resident CTA of the per-call kernels.  Measured at 24^3 x 64
// (fused, triangle, loop, meson, diquark kernels): 8 chunks per SM (one to
// three per CTA) left 3-10 % of the time in the round-robin tail; 24 to 96
// per SM ran 3-10 % faster, the chunk partials' extra finalisation costing
// no more than a few microseconds.
constexpr int kChunksPerCta = 12;

template <class K> struct KernelAttr {
  int bps[64] = {};  // resident CTAs per SM, per device ordinal (0 = not yet queried)
};

template <class Op, class K> cudaError_t prepare(K kernel, size_t smem, int &bps_out)
{
  static KernelAttr<K> cache;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 64 && cache.bps[dev] > 0) {
    bps_out = cache.bps[dev];
    return cudaSuccess;
  }
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int bps = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, Op::THREADS, smem);
  if (e != cudaSuccess) return e;
  if (bps < 1) return cudaErrorInvalidConfiguration;
  if (dev < 64) cache.bps[dev] = bps;
  bps_out = bps;
  return cudaSuccess;
}

struct OutPtrs {
  double2 *p[16];
};

constexpr int kFinThreads = 64;  // finalize_kernel's block: the partials of one (output, timeslice)
__global__ void finalize_kernel(const double2 *__restrict__ partial, OutPtrs out, int nout, int lt, int chunks_per_seg);

template <class Op> cudaError_t run_scalar(const Job &job, OpParams<typename Op::R> p)
{
  if (job.volume == 0) return cudaSuccess;
  constexpr size_t smem = engine_smem_bytes<Op>();
  static_assert(smem <= 232448, "op does not fit in shared memory");
  int bps = 0;
  cudaError_t e = prepare<Op>(scalar_kernel<Op>, smem, bps);
  if (e != cudaSuccess) return e;
  const long long ctas = (long long)job.num_sms * bps;
  p.geom = make_geom(job, Op::SITES, ctas, kChunksPerCta);
  p.status = job.status;
  static_assert(Op::NOUT <= 16, "at most 16 outputs per site");
  OutPtrs user_out {};
  for (int o = 0; o < Op::NOUT; ++o) user_out.p[o] = static_cast<double2 *>(p.out[o]);
  double2 *partial = nullptr;
  if (!job.per_site) {
    if (!job.ws) return cudaErrorInvalidValue;
    partial = static_cast<double2 *>(job.ws->get((size_t)p.geom.total_chunks * Op::CW * Op::NOUT * sizeof(double2)));
    if (!partial) return cudaErrorMemoryAllocation;
    p.out[0] = partial;
  }
  const int grid = (int)std::min<long long>(p.geom.total_chunks, ctas);
  scalar_kernel<Op><<<grid, Op::THREADS, smem, job.stream>>>(p);
  e = cudaGetLastError();
  if (e != cudaSuccess || job.per_site) return e;
  // partial is [segment][chunk][consumer warp][NOUT]: fold the warps into the chunk count.
  finalize_kernel<<<Op::NOUT * job.lt, kFinThreads, 0, job.stream>>>(partial, user_out, Op::NOUT, job.lt,
                                                                      p.geom.chunks_per_seg * Op::CW);
  return cudaGetLastError();
}

template <class Op> cudaError_t run_field(const Job &job, OpParams<typename Op::R> p)
{
  if (job.volume == 0) return cudaSuccess;
  Job j = job;
  j.per_site = true;
  constexpr size_t smem = engine_smem_bytes<Op>();
  static_assert(smem <= 232448, "op does not fit in shared memory");
  int bps = 0;
  cudaError_t e = prepare<Op>(field_kernel<Op>, smem, bps);
  if (e != cudaSuccess) return e;
  const long long ctas = (long long)job.num_sms * bps;
  p.geom = make_geom(j, Op::SITES, ctas, kChunksPerCta);
  p.status = job.status;
  const int grid = (int)std::min<long long>(p.geom.total_chunks, ctas);
  field_kernel<Op><<<grid, Op::THREADS, smem, job.stream>>>(p);
  return cudaGetLastError();
}

} // namespace cgb
