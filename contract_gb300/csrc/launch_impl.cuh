// Launch helpers shared by the kernel translation units.
#pragma once

#include <algorithm>
#include <mutex>

#include "launch.hpp"

namespace cgb {

// Tile geometry for an op with `sites` sites per tile.
inline TileGeom make_geom(const Job &job, int sites, int num_sms)
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
  // About 8 chunks per persistent CTA keeps the round-robin tail under ~1/8
  // of a CTA's work; chunks never span segments.
  long long ct = tiles / ((long long)num_sms * 8);
  g.chunk_tiles = (int)std::max(1LL, std::min(ct, 64LL));
  g.chunk_tiles = std::min(g.chunk_tiles, g.tiles_per_seg);
  g.chunks_per_seg = (g.tiles_per_seg + g.chunk_tiles - 1) / g.chunk_tiles;
  g.total_chunks = g.chunks_per_seg * g.num_segs;
  g.wait_ns = job.wait_ns ? job.wait_ns : kWaitLimitNs;
  g.withhold_chunk = job.withhold_chunk;
  return g;
}

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
  p.geom = make_geom(job, Op::SITES, job.num_sms);
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
  constexpr size_t smem = engine_smem_bytes<Op>();
  static_assert(smem <= 232448, "op does not fit in shared memory");
  int bps = 0;
  cudaError_t e = prepare<Op>(scalar_kernel<Op>, smem, bps);
  if (e != cudaSuccess) return e;
  const int grid = (int)std::min<long long>(p.geom.total_chunks, (long long)job.num_sms * bps);
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
  p.geom = make_geom(j, Op::SITES, job.num_sms);
  p.status = job.status;
  constexpr size_t smem = engine_smem_bytes<Op>();
  static_assert(smem <= 232448, "op does not fit in shared memory");
  int bps = 0;
  cudaError_t e = prepare<Op>(field_kernel<Op>, smem, bps);
  if (e != cudaSuccess) return e;
  const int grid = (int)std::min<long long>(p.geom.total_chunks, (long long)job.num_sms * bps);
  field_kernel<Op><<<grid, Op::THREADS, smem, job.stream>>>(p);
  return cudaGetLastError();
}

} // namespace cgb
