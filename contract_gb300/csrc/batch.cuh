// Persistent batched launch over a device work queue.
//
// A batch is up to kMaxBatch work items -- one per (source position,
// propagator triple, lattice) -- that share one op and its spin tables.  The
// items travel as a kernel parameter (so a CUDA graph captures them by
// value).  Each item's chunks are laid end to end in one global chunk space,
// and the queue is a counter in device memory over that space (zeroed by the
// host before every launch): each CTA's producer warp takes the next chunk
// with an atomic add whenever it has room in its ring, so CTAs that finish
// early take more chunks and items of very different sizes balance without a
// static schedule.  The producer looks up the chunk's item (binary search on
// chunk_begin) for its geometry, inputs and partial-sum buffer, and hands
// every tile to the consumer warps through a descriptor in shared memory
// beside the ring stage; a final descriptor tells them the queue is empty.
//
// Every item is validated on the device before use (extents, chunk ranges,
// 16-byte alignment); a chunk of a bad item is skipped and reported through
// the status word as kDevErrBadWork.
#pragma once

#include "ops.cuh"

namespace cgb {

constexpr int kMaxBatch = 128;

struct BatchItem {
  const void *in[3];
  double2 *partial;  // [chunks][CW][NOUT] of this item
  TileGeom geom;     // per_site == 0: segments are half-timeslices
  int chunk_begin;   // first global chunk of this item
  int lt;            // timeslices (for the finalisation)
  double2 *out;      // [NOUT][lt] complex128 result
};

template <class R> struct BatchParams {
  OpParams<R> op;  // spin tables; op.in/op.out unused
  DeviceStatus *status;
  unsigned int *queue;  // next global chunk (zero at launch)
  int n_items;
  int total_chunks;
  BatchItem items[kMaxBatch];
};

// One tile as the producer hands it to the consumers.
struct TileDesc {
  long long first;  // first site of the tile in its item's volume
  int item;         // work item
  int local;        // chunk within the item
  int n;            // sites in the tile
  int flags;        // kTileLast: last tile of its chunk; kQueueEmpty: no more tiles
};
constexpr int kTileLast = 1, kQueueEmpty = 2;

// Structural checks of one descriptor (identical in producer and consumers).
template <int SITES, int NIN> __device__ __forceinline__ bool item_ok(const BatchItem &it)
{
  const TileGeom &g = it.geom;
  if (g.seg_len <= 0 || g.num_segs <= 0 || g.chunk_tiles <= 0 || g.chunks_per_seg <= 0) return false;
  if ((long long)g.tiles_per_seg * SITES < g.seg_len || (long long)(g.tiles_per_seg - 1) * SITES >= g.seg_len) return false;
  if (g.total_chunks != g.chunks_per_seg * g.num_segs) return false;
  if ((long long)g.seg_len * g.num_segs != g.volume) return false;
  for (int q = 0; q < NIN; ++q)
    if (!it.in[q] || (reinterpret_cast<uintptr_t>(it.in[q]) & 15)) return false;
  return it.partial != nullptr;
}

template <class P> __device__ __forceinline__ int find_item(const P &p, int chunk)
{
  int lo = 0, hi = p.n_items - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (p.items[mid].chunk_begin <= chunk) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <int SITES, int NIN> struct BatchIter {
  int chunk, item, local, k, ntiles;
  bool ok;

  template <class P> __device__ __forceinline__ void set_chunk(const P &p, int c)
  {
    chunk = c;
    k = 0;
    ntiles = 0;
    ok = false;
    if (c >= p.total_chunks) return;
    item = find_item(p, c);
    const BatchItem &it = p.items[item];
    local = c - it.chunk_begin;
    ok = local >= 0 && local < it.geom.total_chunks && item_ok<SITES, NIN>(it);
    if (ok) {
      const int cc = local % it.geom.chunks_per_seg;
      ntiles = min(it.geom.chunk_tiles, it.geom.tiles_per_seg - cc * it.geom.chunk_tiles);
      ok = ntiles > 0;
    }
  }
  template <class P> __device__ __forceinline__ void sites(const P &p, long long &first, int &n) const
  {
    const TileGeom &g = p.items[item].geom;
    const int seg = local / g.chunks_per_seg;
    const int cc = local % g.chunks_per_seg;
    const long long t = (long long)cc * g.chunk_tiles + k;
    first = (long long)seg * g.seg_len + t * SITES;
    n = (int)min((long long)SITES, g.seg_len - t * SITES);
  }
};

template <class Op>
__device__ __forceinline__ void produce_batch(const BatchParams<typename Op::R> &p, unsigned char *smem, uint64_t *full,
                                              uint64_t *empty, TileDesc *desc, volatile int *abort_flag)
{
  using L = OpLayout<Op>;
  constexpr int NST = Op::NST, NIN = Op::NIN, SITES = Op::SITES;
  const int lane = threadIdx.x & 31;
  // Wait (bounded) until ring slot u is free again; false after a timeout or abort.
  auto slot_free = [&](int u) -> bool {
    if (u >= NST) {
      const bool ok = mbar_wait_bounded_backoff(&empty[u % NST], ((u / NST) - 1) & 1, kWaitLimitNs, kProducerSleepNs);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) {
          *abort_flag = 1;
          report(p.status, kDevErrWaitTimeout, (unsigned int)u);
        }
        return false;
      }
    }
    return !*abort_flag;
  };
  int u = 0;
  for (;;) {
    unsigned int c = 0;
    if (lane == 0) c = atomicAdd(p.queue, 1u);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= (unsigned int)p.total_chunks) break;
    BatchIter<SITES, NIN> it;
    it.set_chunk(p, (int)c);
    if (!it.ok) {  // a rejected item: its chunks are skipped
      if (lane == 0) report(p.status, kDevErrBadWork, c);
      continue;
    }
    for (; it.k < it.ntiles; ++it.k, ++u) {
      if (!slot_free(u)) return;
      const int stage = u % NST;
      long long first;
      int n;
      it.sites(p, first, n);
      const BatchItem &item = p.items[it.item];
      if (lane == 0) {
        desc[stage] = TileDesc {first, it.item, it.local, n, it.k == it.ntiles - 1 ? kTileLast : 0};
        mbar_arrive_expect_tx(&full[stage], (uint32_t)n * NIN * L::SITE_BYTES);
      }
      __syncwarp();
      unsigned char *dst = smem + Smem<Op>::STAGES + stage * Smem<Op>::STAGE;
      for (int q0 = lane; q0 < n * NIN; q0 += 32) {
        const int q = q0 / n, s = q0 - q * n;
        bulk_g2s(dst + ((size_t)q * SITES + s) * L::SLOT,
                 static_cast<const char *>(item.in[q]) + (first + s) * L::SITE_BYTES, L::SITE_BYTES, &full[stage]);
      }
    }
  }
  // the queue is empty: one more slot tells the consumers so
  if (!slot_free(u)) return;
  if (lane == 0) {
    desc[u % NST] = TileDesc {0, 0, 0, 0, kQueueEmpty};
    mbar_arrive(&full[u % NST]);
  }
}

template <class Op>
__global__ void __launch_bounds__(Op::THREADS, min_blocks<Op>()) batch_scalar_kernel(
  const __grid_constant__ BatchParams<typename Op::R> p)
{
  using S = typename Op::S;
  using R = typename Op::R;
  using L = OpLayout<Op>;
  constexpr int NIN = Op::NIN, SITES = Op::SITES, TPS = Op::TPS, NST = Op::NST, NOUT = Op::NOUT;
  constexpr int SPW = 32 / TPS, CW = Op::CW;

  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(16) typename Op::Params ps;
  __shared__ TileDesc desc[NST];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *empty = full + NST;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + 120);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], CW);
    }
    *abort_flag = 0;
    fence_barrier_init();
  }
  copy_params(ps, p.op);
  __syncthreads();
  if (warp == 0) {
    produce_batch<Op>(p, smem, full, empty, desc, abort_flag);
    return;
  }

  const int w = warp - 1;
  const int local = lane / TPS, sub = lane % TPS;
  const int site = w * SPW + local;
  cx<R> *sv = reinterpret_cast<cx<R> *>(smem + Smem<Op>::TAIL) + (size_t)w * SPW * NOUT;
  S *scratch = reinterpret_cast<S *>(smem + Smem<Op>::EXTRA + (size_t)site * Op::EXTRA_BYTES);
  ChunkSum<R> chunk_acc;

  for (int u = 0;; ++u) {
    const int stage = u % NST;
    const bool ok = mbar_wait_bounded(&full[stage], (u / NST) & 1, kWaitLimitNs);
    if (!__all_sync(0xffffffffu, ok) || *abort_flag) {
      if (lane == 0) {
        *abort_flag = 1;
        report(p.status, kDevErrWaitTimeout, (unsigned int)u);
        drain<NST>(full, u, kWaitLimitNs);
      }
      return;
    }
    const TileDesc d = desc[stage];  // read before the stage is released
    if (d.flags & kQueueEmpty) return;
    const unsigned char *sb = smem + Smem<Op>::STAGES + stage * Smem<Op>::STAGE;
    const S *in[NIN];
#pragma unroll
    for (int q = 0; q < NIN; ++q) in[q] = reinterpret_cast<const S *>(sb + ((size_t)q * SITES + site) * L::SLOT);
    cx<R> vals[NOUT];
    Op::site(ps, in, scratch, sub, vals);
    const bool valid = site < d.n;
    if constexpr (kScatterSums<TPS, NOUT>) {
      // many outputs: thread sub keeps the site sum of output sub
      const cx<R> mine = group_reduce_scatter<TPS, NOUT>(vals, sub);
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[stage]);
      if (sub < NOUT) sv[local * NOUT + sub] = valid ? mine : czero<R>();
    } else {
#pragma unroll
      for (int o = 0; o < NOUT; ++o) vals[o] = group_sum<TPS>(vals[o]);
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[stage]);
      if (sub == 0) {
#pragma unroll
        for (int o = 0; o < NOUT; ++o) sv[local * NOUT + o] = valid ? vals[o] : czero<R>();
      }
    }
    __syncwarp();
    if (lane < NOUT) {
#pragma unroll
      for (int s = 0; s < SPW; ++s) chunk_acc.add(sv[s * NOUT + lane]);
      if (d.flags & kTileLast) {
        p.items[d.item].partial[((size_t)d.local * CW + w) * NOUT + lane] = chunk_acc.value();
        chunk_acc.reset();
      }
    }
    __syncwarp();
  }
}

// out_i[o][t] = sum over parity and the item's (chunk, warp) partials, FP64,
// fixed order.  Grid: (items, ceil(nout * max_lt / 128)).
template <class R>
__global__ void batch_finalize_kernel(const __grid_constant__ BatchParams<R> p, int nout, int cw)
{
  const int i = blockIdx.x;
  const BatchItem &it = p.items[i];
  const int idx = blockIdx.y * blockDim.x + threadIdx.x;
  if (idx >= nout * it.lt || it.geom.chunks_per_seg <= 0) return;
  const int o = idx / it.lt, t = idx % it.lt;
  const int per_seg = it.geom.chunks_per_seg * cw;
  double sx = 0.0, sy = 0.0;
  for (int par = 0; par < 2; ++par) {
    const double2 *row = it.partial + ((size_t)(par * it.lt + t) * per_seg) * nout + o;
    for (int c = 0; c < per_seg; ++c) {
      const double2 v = row[(size_t)c * nout];
      sx += v.x;
      sy += v.y;
    }
  }
  it.out[(size_t)o * it.lt + t] = make_double2(sx, sy);
}

} // namespace cgb
