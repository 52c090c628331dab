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
// Warp 0 of every CTA is the producer: for each tile it waits until the ring
// stage is free (`empty` mbarrier, one arrival per consumer warp), arms the
// stage's `full` mbarrier with the tile's byte count and has its 32 lanes
// issue the tile's cp.async.bulk (TMA) copies -- one per site and input, each
// into its own padded shared-memory slot (+16 B, or the op's SLOT_PAD, which
// staggers consecutive sites across banks).  The CW consumer warps each own
// SPW = 32/TPS sites of every tile; they wait on `full`, compute, and release
// the stage.  Warps never meet at a CTA-wide barrier, so a slow warp only
// delays itself.
//
// Every wait is bounded in wall time.  A timed-out wait sets a bit in the
// device status word and a CTA-local abort flag, waits (bounded again) for
// the copies that may still be in flight into this CTA's shared memory, and
// returns: no trap, no unbounded spin.
//
// Outputs
// -------
// Scalar ops (mesons, baryons) produce NOUT complex numbers per site: either
// written per site (the reference's per-site output) or summed per warp and
// accumulated in FP64 per chunk into `partial[chunk][warp][NOUT]`, which
// `finalize_kernel` reduces per timeslice in a fixed order (deterministic).
// Field ops (diquark, sequential sources) produce a propagator-shaped site:
// lanes write it to a per-warp shared-memory staging slot (double-buffered)
// and lane 0 stores it with cp.async.bulk shared->global copies.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace cgb {

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per mbarrier wait (the default)
constexpr unsigned kProducerSleepNs = 128;          // producer's sleep between polls of a busy stage

struct TileGeom {
  long long volume;
  long long seg_len;
  int num_segs;
  int tiles_per_seg;
  int chunk_tiles;
  int chunks_per_seg;
  int total_chunks;
  int per_site;  // 1: per-site outputs; 0: per-chunk FP64 partial sums
  unsigned long long wait_ns;  // wall-time limit of every mbarrier wait
  // Test hook: the producer never copies (nor arms the barrier of) the first
  // tile of this chunk, so its consumers' wait runs out; -1 in normal use.
  int withhold_chunk;
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

// One site's propagator in a ring stage: 144 complex values, then PAD bytes so
// that consecutive sites start in different shared-memory banks (a multiple of
// 16, as the bulk copies need).
template <class S, int PAD = 16> struct SiteLayout {
  static constexpr uint32_t SITE_BYTES = 144 * sizeof(S);
  static constexpr uint32_t SLOT = SITE_BYTES + PAD;
  static_assert(SLOT % 16 == 0, "site slots must stay 16-byte aligned");
};
// An op's slot layout: its SLOT_PAD if it declares one, else 16 bytes.
template <class Op, class = void> struct SlotPad {
  static constexpr int value = 16;
};
template <class Op> struct SlotPad<Op, std::void_t<decltype(Op::SLOT_PAD)>> {
  static constexpr int value = Op::SLOT_PAD;
};
template <class Op> using OpLayout = SiteLayout<typename Op::S, SlotPad<Op>::value>;

// Per-site output block of a field op: OUT_ELEMS complex values (a
// propagator-shaped 144 for diquark/sequential, 256 for the all-gamma meson).
template <class Op> struct OutLayout {
  static constexpr uint32_t BYTES = Op::OUT_ELEMS * sizeof(typename Op::S);
  static constexpr uint32_t SLOT = BYTES + 16;
};

// Shared-memory map of an engine kernel:
//   [0, 128)        full[NST], empty[NST] mbarriers, abort flag
//   stages          NST x NIN x SITES slots
//   extra           SITES x EXTRA_BYTES (per-site op scratch)
//   tail            scalar ops: per-warp site values [CW][SPW][NOUT] (cx<R>)
//                   field ops:  per-warp output staging [CW][2][SPW] slots
template <class Op> struct Smem {
  using L = OpLayout<Op>;
  static constexpr size_t STAGE = (size_t)Op::NIN * Op::SITES * L::SLOT;
  static constexpr size_t STAGES = 128;
  static constexpr size_t EXTRA = STAGES + Op::NST * STAGE;
  static constexpr size_t TAIL = EXTRA + (size_t)Op::EXTRA_BYTES * Op::SITES;
  static constexpr size_t tail_bytes()
  {
    if constexpr (Op::FIELD && Op::DIRECT_OUT) return 0;
    else if constexpr (Op::FIELD) return 2ull * Op::SITES * OutLayout<Op>::SLOT;
    else return (size_t)Op::SITES * Op::NOUT * 2 * sizeof(typename Op::R);
  }
  static constexpr size_t BYTES = TAIL + tail_bytes();
  static_assert(2 * Op::NST * 8 + 4 <= 128, "too many stages for the barrier block");
};

template <class Op> constexpr size_t engine_smem_bytes() { return Smem<Op>::BYTES; }

// FP32 ops ask for two CTAs per SM when their shared memory fits (228 KB per
// SM, 1 KB reserved per CTA), which caps registers at 128 per thread; FP64 ops
// are bound by the FP64 pipe and keep one CTA with the full register file.  An
// op may ask for more (MIN_CTAS), trading registers for warps.
template <class Op> constexpr int min_blocks()
{
  if constexpr (Op::MIN_CTAS > 0) return Op::MIN_CTAS;
  return (sizeof(typename Op::R) == 4 && 2 * (Smem<Op>::BYTES + sizeof(typename Op::Params) + 1024) <= 233472) ? 2
                                                                                                              : 1;
}

// The op parameters, copied to shared memory once per CTA.  Gamma tables are
// indexed by each lane's own spin indices; from the kernel-parameter
// (constant) space such lane-divergent loads serialise, from shared memory
// they do not.
template <class P> __device__ __forceinline__ void copy_params(P &dst, const P &src)
{
  static_assert(sizeof(P) % 4 == 0, "parameter block must be word-sized");
  const uint32_t *s = reinterpret_cast<const uint32_t *>(&src);
  uint32_t *d = reinterpret_cast<uint32_t *>(&dst);
  for (int k = threadIdx.x; k < (int)(sizeof(P) / 4); k += blockDim.x) d[k] = s[k];
}

// Running sum in the op's precision.  FP32 uses a compensated (two-sum)
// accumulator so that chunk sums lose nothing before they reach FP64; FP64 is
// a plain sum.
template <class R> struct ChunkSum;
template <> struct ChunkSum<float> {
  float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f;
  __device__ __forceinline__ static void two_sum(float &h, float &l, float v)
  {
    const float s = h + v;
    const float bp = s - h;
    l += (h - (s - bp)) + (v - bp);
    h = s;
  }
  __device__ __forceinline__ void add(cx<float> v)
  {
    two_sum(hx, lx, v.x);
    two_sum(hy, ly, v.y);
  }
  __device__ __forceinline__ double2 value() const { return make_double2((double)hx + (double)lx, (double)hy + (double)ly); }
  __device__ __forceinline__ void reset() { hx = lx = hy = ly = 0.f; }
};
template <> struct ChunkSum<double> {
  double x = 0.0, y = 0.0;
  __device__ __forceinline__ void add(cx<double> v)
  {
    x += v.x;
    y += v.y;
  }
  __device__ __forceinline__ double2 value() const { return make_double2(x, y); }
  __device__ __forceinline__ void reset() { x = y = 0.0; }
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Producer warp: stream this CTA's tiles into the ring.
template <class Op>
__device__ __forceinline__ void produce(const typename Op::Params &p, unsigned char *smem, uint64_t *full,
                                        uint64_t *empty, volatile int *abort_flag)
{
  using L = OpLayout<Op>;
  constexpr int NST = Op::NST, NIN = Op::NIN, SITES = Op::SITES;
  const TileGeom &g = p.geom;
  const int lane = threadIdx.x & 31;
  TileIter<SITES> it;
  it.set_chunk(g, blockIdx.x);
  for (int u = 0; it.valid(g); ++u) {
    const int stage = u % NST;
    if (u >= NST) {
      const bool ok = mbar_wait_bounded_backoff(&empty[stage], ((u / NST) - 1) & 1, g.wait_ns, kProducerSleepNs);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) {
          *abort_flag = 1;
          report(p.status, kDevErrWaitTimeout, (unsigned int)it.chunk);
        }
        return;
      }
    }
    if (*abort_flag) return;
    if (it.k == 0 && it.chunk == g.withhold_chunk) {  // test hook: this tile never arrives
      it.next(g);
      continue;
    }
    long long first;
    int n;
    it.sites(g, first, n);
    if (lane == 0) mbar_arrive_expect_tx(&full[stage], (uint32_t)n * NIN * L::SITE_BYTES);
    __syncwarp();
    unsigned char *dst = smem + Smem<Op>::STAGES + stage * Smem<Op>::STAGE;
    for (int c = lane; c < n * NIN; c += 32) {
      const int q = c / n, s = c - q * n;
      bulk_g2s(dst + ((size_t)q * SITES + s) * L::SLOT,
               static_cast<const char *>(p.in[q]) + (first + s) * L::SITE_BYTES, L::SITE_BYTES, &full[stage]);
    }
    it.next(g);
  }
}

// A consumer warp that gave up: wait (bounded) for the copies of the next
// NST-1 tiles, which the producer may already have issued.
template <int NST> __device__ void drain(uint64_t *full, int from, unsigned long long wait_ns)
{
  for (int u = from; u < from + NST; ++u) mbar_wait_bounded(&full[u % NST], (u / NST) & 1, wait_ns / 8);
}

// ------------------------------------------------------------ scalar ops --
template <class Op>
__global__ void __launch_bounds__(Op::THREADS, min_blocks<Op>()) scalar_kernel(const __grid_constant__ typename Op::Params p)
{
  using S = typename Op::S;
  using R = typename Op::R;
  using L = OpLayout<Op>;
  constexpr int NIN = Op::NIN, SITES = Op::SITES, TPS = Op::TPS, NST = Op::NST, NOUT = Op::NOUT;
  constexpr int SPW = 32 / TPS, CW = Op::CW;

  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(16) typename Op::Params ps;
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
  copy_params(ps, p);
  __syncthreads();
  if (warp == 0) {
    produce<Op>(p, smem, full, empty, abort_flag);
    return;
  }

  const TileGeom &g = p.geom;
  const int w = warp - 1;
  const int local = lane / TPS, sub = lane % TPS;
  const int site = w * SPW + local;
  cx<R> *sv = reinterpret_cast<cx<R> *>(smem + Smem<Op>::TAIL) + (size_t)w * SPW * NOUT;  // [SPW][NOUT]
  S *scratch = reinterpret_cast<S *>(smem + Smem<Op>::EXTRA + (size_t)site * Op::EXTRA_BYTES);
  ChunkSum<R> chunk_acc;  // lane o < NOUT: output o

  TileIter<SITES> it;
  it.set_chunk(g, blockIdx.x);
  for (int u = 0; it.valid(g); ++u) {
    const int stage = u % NST;
    long long first;
    int n;
    it.sites(g, first, n);
    const bool ok = mbar_wait_bounded(&full[stage], (u / NST) & 1, g.wait_ns);
    if (!__all_sync(0xffffffffu, ok) || *abort_flag) {
      if (lane == 0) {
        *abort_flag = 1;
        report(p.status, kDevErrWaitTimeout, (unsigned int)it.chunk);
        drain<NST>(full, u, g.wait_ns);
      }
      return;
    }
    const unsigned char *sb = smem + Smem<Op>::STAGES + stage * Smem<Op>::STAGE;
    const S *in[NIN];
#pragma unroll
    for (int q = 0; q < NIN; ++q) in[q] = reinterpret_cast<const S *>(sb + ((size_t)q * SITES + site) * L::SLOT);
    cx<R> vals[NOUT];
    Op::site(ps, in, scratch, sub, vals);
    if constexpr (kScatterSums<TPS, NOUT>) {
      // many outputs: thread sub keeps the site sum of output sub
      const cx<R> mine = group_reduce_scatter<TPS, NOUT>(vals, sub);
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[stage]);  // inputs consumed; only registers below
      const bool valid = site < n;
      if (g.per_site) {
        if (sub < NOUT && valid)
          static_cast<double2 *>(p.out[sub])[first + site] = make_double2(double(mine.x), double(mine.y));
      } else {
        if (sub < NOUT) sv[local * NOUT + sub] = valid ? mine : czero<R>();
        __syncwarp();
        if (lane < NOUT) {
#pragma unroll
          for (int s = 0; s < SPW; ++s) chunk_acc.add(sv[s * NOUT + lane]);
          if (it.last_in_chunk()) {
            static_cast<double2 *>(p.out[0])[((size_t)it.chunk * CW + w) * NOUT + lane] = chunk_acc.value();
            chunk_acc.reset();
          }
        }
        __syncwarp();
      }
      it.next(g);
      continue;
    }
#pragma unroll
    for (int o = 0; o < NOUT; ++o) vals[o] = group_sum<TPS>(vals[o]);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[stage]);  // inputs consumed; only registers below
    const bool valid = site < n;
    if (g.per_site) {
      if (sub == 0 && valid) {
#pragma unroll
        for (int o = 0; o < NOUT; ++o)
          static_cast<double2 *>(p.out[o])[first + site] = make_double2(double(vals[o].x), double(vals[o].y));
      }
    } else {
      if (sub == 0) {
#pragma unroll
        for (int o = 0; o < NOUT; ++o) sv[local * NOUT + o] = valid ? vals[o] : czero<R>();
      }
      __syncwarp();
      if (lane < NOUT) {
#pragma unroll
        for (int s = 0; s < SPW; ++s) chunk_acc.add(sv[s * NOUT + lane]);
        if (it.last_in_chunk()) {
          static_cast<double2 *>(p.out[0])[((size_t)it.chunk * CW + w) * NOUT + lane] = chunk_acc.value();
          chunk_acc.reset();
        }
      }
      __syncwarp();
    }
    it.next(g);
  }
}

// ------------------------------------------------------------- field ops --
template <class Op>
__global__ void __launch_bounds__(Op::THREADS, min_blocks<Op>()) field_kernel(const __grid_constant__ typename Op::Params p)
{
  using S = typename Op::S;
  using L = OpLayout<Op>;
  constexpr int NIN = Op::NIN, SITES = Op::SITES, TPS = Op::TPS, NST = Op::NST;
  constexpr int SPW = 32 / TPS, CW = Op::CW;

  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(16) typename Op::Params ps;
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
  copy_params(ps, p);
  __syncthreads();
  if (warp == 0) {
    produce<Op>(p, smem, full, empty, abort_flag);
    return;
  }

  const TileGeom &g = p.geom;
  const int w = warp - 1;
  const int local = lane / TPS, sub = lane % TPS;
  const int site = w * SPW + local;
  S *scratch = reinterpret_cast<S *>(smem + Smem<Op>::EXTRA + (size_t)site * Op::EXTRA_BYTES);
  using O = OutLayout<Op>;
  unsigned char *outbuf = smem + Smem<Op>::TAIL + (size_t)w * 2 * SPW * O::SLOT;  // [2][SPW] slots

  TileIter<SITES> it;
  it.set_chunk(g, blockIdx.x);
  for (int u = 0; it.valid(g); ++u) {
    const int stage = u % NST;
    long long first;
    int n;
    it.sites(g, first, n);
    const bool ok = mbar_wait_bounded(&full[stage], (u / NST) & 1, g.wait_ns);
    if (!__all_sync(0xffffffffu, ok) || *abort_flag) {
      if (lane == 0) {
        *abort_flag = 1;
        report(p.status, kDevErrWaitTimeout, (unsigned int)it.chunk);
        drain<NST>(full, u, g.wait_ns);
        bulk_wait<0>();
      }
      return;
    }
    const unsigned char *sb = smem + Smem<Op>::STAGES + stage * Smem<Op>::STAGE;
    const S *in[NIN];
#pragma unroll
    for (int q = 0; q < NIN; ++q) in[q] = reinterpret_cast<const S *>(sb + ((size_t)q * SITES + site) * L::SLOT);
    if constexpr (Op::DIRECT_OUT) {
      // The op stores its outputs itself: pass this site's destination, or
      // nullptr past the tile's end or for a destination outside the volume.
      S *dst = nullptr;
      if (site < n) {
        const long long d = Op::out_index(ps, first + site);
        if (d >= 0 && d < g.volume) dst = Op::out_ptr(ps, d, static_cast<S *>(p.out[0]));
        else if (sub == 0) report(p.status, kDevErrBadWork, (unsigned int)(first + site));
      }
      Op::site(ps, in, scratch, sub, dst);
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[stage]);
      __syncwarp();
      it.next(g);
      continue;
    }
    unsigned char *ob = outbuf + (size_t)(u & 1) * SPW * O::SLOT;
    Op::site(ps, in, scratch, sub, reinterpret_cast<S *>(ob + (size_t)local * O::SLOT));
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(&empty[stage]);
      for (int s = 0; s < SPW; ++s) {
        if (w * SPW + s >= n) continue;
        // Destination site (identity, or a reordering such as lexicographic):
        // checked against the volume so a bad layout cannot store out of bounds.
        const long long dst = Op::out_index(ps, first + w * SPW + s);
        if (dst < 0 || dst >= g.volume) {
          report(p.status, kDevErrBadWork, (unsigned int)(first + w * SPW + s));
          continue;
        }
        bulk_s2g(static_cast<char *>(p.out[0]) + dst * O::BYTES, ob + (size_t)s * O::SLOT, O::BYTES);
      }
      bulk_commit();
      bulk_wait_read<1>();  // the other staging buffer is free again
    }
    __syncwarp();
    it.next(g);
  }
  if (lane == 0) bulk_wait<0>();
}

} // namespace cgb
