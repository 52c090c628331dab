// Site-tile pipeline shared by every contraction kernel.
//
// Work decomposition
// ------------------
// The lattice is a flat array of `volume` sites (PyQUDA even/odd order,
// [2][Lt][Lz][Ly][Lx/2]).  It is cut into `num_segs` segments of `seg_len`
// sites (one half-timeslice per segment when results are reduced per
// timeslice; a single segment otherwise).  A segment is cut into tiles of
// SITES consecutive sites, and CHUNK_TILES consecutive tiles form a chunk.
// Chunks are dealt to persistent CTAs round-robin; a CTA streams its tiles
// through an NST-stage shared-memory ring.
//
// Data movement
// -------------
// Each site of each input propagator (144 complex: 2304 B in complex128,
// 1152 B in complex64) is one cp.async.bulk (TMA) copy into its own padded
// shared-memory slot (+16 B, which staggers consecutive sites across banks).
// Thread 0 arms an mbarrier per stage with the expected byte count; all
// threads wait on it with a time limit.  A timed-out wait sets a bit in the
// device status word, drains this CTA's outstanding copies (again with a time
// limit) and returns: no trap, no unbounded spin.
//
// Outputs
// -------
// Scalar ops (mesons, baryons) produce NOUT complex numbers per site: either
// written per site (the reference's per-site output) or summed in FP64 per
// chunk into `partial[chunk][NOUT]`, which `finalize_segments` reduces per
// timeslice in a fixed order (deterministic).
// Field ops (diquark, sequential sources) produce a propagator-shaped site:
// threads write it to a shared-memory staging slot, and thread 0 stores the
// tile with cp.async.bulk shared->global copies (double-buffered).
#pragma once

#include "common.cuh"

namespace cgb {

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per mbarrier wait

struct TileGeom {
  long long volume;
  long long seg_len;
  int num_segs;
  int tiles_per_seg;
  int chunk_tiles;
  int chunks_per_seg;
  int total_chunks;
  int per_site;  // 1: per-site outputs; 0: per-chunk FP64 partial sums
};

template <int SITES> struct TileIter {
  int chunk, k, ntiles;

  __device__ __forceinline__ void set_chunk(const TileGeom &g, int c)
  {
    chunk = c;
    k = 0;
    ntiles = 0;
    if (c < g.total_chunks) {
      const int cc = c % g.chunks_per_seg;
      ntiles = min(g.chunk_tiles, g.tiles_per_seg - cc * g.chunk_tiles);
    }
  }
  __device__ __forceinline__ bool valid(const TileGeom &g) const { return chunk < g.total_chunks; }
  __device__ __forceinline__ bool last_in_chunk() const { return k == ntiles - 1; }
  __device__ __forceinline__ void next(const TileGeom &g)
  {
    if (++k == ntiles) set_chunk(g, chunk + gridDim.x);
  }
  __device__ __forceinline__ void sites(const TileGeom &g, long long &first, int &n) const
  {
    const int seg = chunk / g.chunks_per_seg;
    const int cc = chunk % g.chunks_per_seg;
    const long long t = (long long)cc * g.chunk_tiles + k;
    first = (long long)seg * g.seg_len + t * SITES;
    n = (int)min((long long)SITES, g.seg_len - t * SITES);
  }
};

template <class S> struct SiteLayout {
  static constexpr uint32_t SITE_BYTES = 144 * sizeof(S);
  static constexpr uint32_t SLOT = SITE_BYTES + 16;
};

// Shared-memory bytes used by the engines (op scratch excluded).
template <class Op> constexpr size_t engine_smem_bytes()
{
  using L = SiteLayout<typename Op::S>;
  size_t b = 128 + (size_t)Op::NST * Op::NIN * Op::SITES * L::SLOT;
  b += (size_t)Op::EXTRA_SLOTS * Op::SITES * L::SLOT;
  if constexpr (Op::FIELD) b += 2ull * Op::SITES * L::SLOT;
  else b += 2ull * Op::SITES * Op::NOUT * sizeof(double2);
  return b;
}

// Issue the bulk copies of one tile into `stage` (called by one thread).
template <class Op>
__device__ __forceinline__ void issue_tile(const typename Op::Params &p, unsigned char *stage_ptr, uint64_t *bar,
                                           long long first, int n)
{
  using L = SiteLayout<typename Op::S>;
  mbar_arrive_expect_tx(bar, (uint32_t)n * Op::NIN * L::SITE_BYTES);
  for (int q = 0; q < Op::NIN; ++q) {
    const char *src = static_cast<const char *>(p.in[q]) + first * L::SITE_BYTES;
    unsigned char *dst = stage_ptr + (size_t)q * Op::SITES * L::SLOT;
    for (int s = 0; s < n; ++s) bulk_g2s(dst + (size_t)s * L::SLOT, src + (size_t)s * L::SITE_BYTES, L::SITE_BYTES, bar);
  }
}

// Wait (bounded) for the copies of tiles [from, issued) so none is still
// writing this CTA's shared memory when it exits after an error.
template <int NST> __device__ void drain(uint64_t *full, int from, int issued)
{
  for (int u = from; u < issued; ++u) mbar_wait_bounded(&full[u % NST], (u / NST) & 1, kWaitLimitNs / 4);
}

// ------------------------------------------------------------ scalar ops --
template <class Op> __global__ void __launch_bounds__(Op::THREADS, 1) scalar_kernel(const __grid_constant__ typename Op::Params p)
{
  using S = typename Op::S;
  using R = typename Op::R;
  using L = SiteLayout<S>;
  constexpr int NIN = Op::NIN, SITES = Op::SITES, TPS = Op::TPS, NST = Op::NST, NOUT = Op::NOUT;
  constexpr size_t STAGE = (size_t)NIN * SITES * L::SLOT;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  unsigned char *stages = smem + 128;
  unsigned char *extra = stages + NST * STAGE;
  double2 *tile_vals = reinterpret_cast<double2 *>(extra + (size_t)Op::EXTRA_SLOTS * SITES * L::SLOT);

  const TileGeom &g = p.geom;
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) mbar_init(&full[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  TileIter<SITES> prod, cons;
  prod.set_chunk(g, blockIdx.x);
  cons.set_chunk(g, blockIdx.x);
  int issued = 0;
  if (tid == 0) {
    for (int s = 0; s < NST && prod.valid(g); ++s) {
      long long f;
      int n;
      prod.sites(g, f, n);
      issue_tile<Op>(p, stages + s * STAGE, &full[s], f, n);
      prod.next(g);
      ++issued;
    }
  }

  const int site = tid / TPS, sub = tid % TPS;
  double2 chunk_acc = make_double2(0.0, 0.0);
  for (int it = 0; cons.valid(g); ++it) {
    const int stage = it % NST;
    long long first;
    int n;
    cons.sites(g, first, n);
    const bool ok = mbar_wait_bounded(&full[stage], (it / NST) & 1, kWaitLimitNs);

    const unsigned char *sb = stages + stage * STAGE;
    const S *in[NIN];
#pragma unroll
    for (int q = 0; q < NIN; ++q) in[q] = reinterpret_cast<const S *>(sb + ((size_t)q * SITES + site) * L::SLOT);
    cx<R> vals[NOUT];
    Op::site(p, in, reinterpret_cast<S *>(extra + (size_t)site * Op::EXTRA_SLOTS * L::SLOT), sub, vals);
#pragma unroll
    for (int o = 0; o < NOUT; ++o) vals[o] = group_sum<TPS>(vals[o]);
    if (sub == 0 && site < n) {
      if (g.per_site) {
#pragma unroll
        for (int o = 0; o < NOUT; ++o)
          static_cast<double2 *>(p.out[o])[first + site] = make_double2(double(vals[o].x), double(vals[o].y));
      } else {
#pragma unroll
        for (int o = 0; o < NOUT; ++o)
          tile_vals[((it & 1) * SITES + site) * NOUT + o] = make_double2(double(vals[o].x), double(vals[o].y));
      }
    }
    if (!__syncthreads_and(ok)) {
      if (tid == 0) {
        report(p.status, kDevErrWaitTimeout, (unsigned int)cons.chunk);
        drain<NST>(full, it, issued);
      }
      return;
    }
    if (!g.per_site && tid < NOUT) {
      for (int s = 0; s < n; ++s) {
        const double2 v = tile_vals[((it & 1) * SITES + s) * NOUT + tid];
        chunk_acc.x += v.x;
        chunk_acc.y += v.y;
      }
      if (cons.last_in_chunk()) {
        static_cast<double2 *>(p.out[0])[(size_t)cons.chunk * NOUT + tid] = chunk_acc;
        chunk_acc = make_double2(0.0, 0.0);
      }
    }
    if (tid == 0 && prod.valid(g)) {
      long long f;
      int nn;
      prod.sites(g, f, nn);
      issue_tile<Op>(p, stages + stage * STAGE, &full[stage], f, nn);
      prod.next(g);
      ++issued;
    }
    cons.next(g);
  }
}

// ------------------------------------------------------------- field ops --
template <class Op> __global__ void __launch_bounds__(Op::THREADS, 1) field_kernel(const __grid_constant__ typename Op::Params p)
{
  using S = typename Op::S;
  using L = SiteLayout<S>;
  constexpr int NIN = Op::NIN, SITES = Op::SITES, TPS = Op::TPS, NST = Op::NST;
  constexpr size_t STAGE = (size_t)NIN * SITES * L::SLOT;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  unsigned char *stages = smem + 128;
  unsigned char *extra = stages + NST * STAGE;
  unsigned char *outbuf = extra + (size_t)Op::EXTRA_SLOTS * SITES * L::SLOT;  // [2][SITES][SLOT]

  const TileGeom &g = p.geom;
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) mbar_init(&full[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  TileIter<SITES> prod, cons;
  prod.set_chunk(g, blockIdx.x);
  cons.set_chunk(g, blockIdx.x);
  int issued = 0;
  if (tid == 0) {
    for (int s = 0; s < NST && prod.valid(g); ++s) {
      long long f;
      int n;
      prod.sites(g, f, n);
      issue_tile<Op>(p, stages + s * STAGE, &full[s], f, n);
      prod.next(g);
      ++issued;
    }
  }

  const int site = tid / TPS, sub = tid % TPS;
  for (int it = 0; cons.valid(g); ++it) {
    const int stage = it % NST;
    long long first;
    int n;
    cons.sites(g, first, n);
    const bool ok = mbar_wait_bounded(&full[stage], (it / NST) & 1, kWaitLimitNs);

    const unsigned char *sb = stages + stage * STAGE;
    const S *in[NIN];
#pragma unroll
    for (int q = 0; q < NIN; ++q) in[q] = reinterpret_cast<const S *>(sb + ((size_t)q * SITES + site) * L::SLOT);
    S *out = reinterpret_cast<S *>(outbuf + ((size_t)(it & 1) * SITES + site) * L::SLOT);
    Op::site(p, in, reinterpret_cast<S *>(extra + (size_t)site * Op::EXTRA_SLOTS * L::SLOT), sub, out);
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      if (ok) {
        for (int s = 0; s < n; ++s)
          bulk_s2g(static_cast<char *>(p.out[0]) + (first + s) * L::SITE_BYTES,
                   outbuf + ((size_t)(it & 1) * SITES + s) * L::SLOT, L::SITE_BYTES);
      }
      bulk_commit();
      bulk_wait_read<1>();  // the other staging buffer is free again
    }
    if (!__syncthreads_and(ok)) {
      if (tid == 0) {
        report(p.status, kDevErrWaitTimeout, (unsigned int)cons.chunk);
        drain<NST>(full, it, issued);
        bulk_wait<0>();
      }
      return;
    }
    if (tid == 0 && prod.valid(g)) {
      long long f;
      int nn;
      prod.sites(g, f, nn);
      issue_tile<Op>(p, stages + stage * STAGE, &full[stage], f, nn);
      prod.next(g);
      ++issued;
    }
    cons.next(g);
  }
  if (tid == 0) bulk_wait<0>();
}

} // namespace cgb
