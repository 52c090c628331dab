// Momentum projection on the tensor cores (tcgen05), complex64 storage.
//
// Per timeslice t the projection is the complex GEMM
//   D[p][n] = sum_s Phi[p][s] C[s][n],   Phi[p][s] = exp(+2 pi i (nx x / Lx + ny y / Ly + nz z / Lz)),
// s the lexicographic site of the timeslice and n the 256 (Gamma_ij, Gamma_kl)
// pairs.  It runs as one real GEMM with the momentum rows doubled and the
// site columns interleaved (re, im):
//   A'[2p  ][2s] =  Re Phi   A'[2p  ][2s+1] = -Im Phi   ->  D'[2p  ][n] = Re D[p][n]
//   A'[2p+1][2s] =  Im Phi   A'[2p+1][2s+1] =  Re Phi   ->  D'[2p+1][n] = Im D[p][n]
//   B'[n][2s + c] = (Re C[s][n], Im C[s][n])[c]
// Every operand value x is split into three bf16 terms, hi = bf16(x),
// mid = bf16(x - hi) and lo = bf16(x - hi - mid) (24 significant bits, an
// FP32 value's), and the product keeps every term pair down to second order:
// hi*hi + hi*mid + mid*hi + mid*mid + hi*lo + lo*hi ("split bf16, six
// products"); the terms dropped are of order 2^-24 of the product.  The
// tensor core accumulates in FP32 in tensor memory.  A k-step is 8 sites
// (K = 16 of the real GEMM).
//
// Work: units (momentum group of 128, block of k-steps, t, pair half) are
// dealt round-robin to persistent CTAs, so the CTAs running together share
// the same phase tiles (L2-resident; the phase matrix does not depend on t).
// Roles in a CTA (352 threads):
//   warp 0     one bulk copy per k-step of the 8 sites x 128 pairs (8 KB) of
//              the complex64 field, stored pair-half-major so that it is
//              contiguous, into an 8-deep staging ring (HBM latency)
//   warp 10    bulk copies of the 24 KB phase tile per k-step (both m-tiles,
//              hi, mid and lo, pre-tiled in global memory) into a 4-deep
//              operand ring
//   warp 1     allocates the 512 TMEM columns and issues the MMAs: six
//              M=128 (pairs), N=256 (momentum rows), K=16 MMAs per k-step
//              (the six term pairs above) into one of two accumulator
//              buffers of 256 columns
//   warps 2-9  convert the staged FP32 values into the bf16 hi/mid/lo field tile
//              of the operand ring (four groups of two warps, each taking every
//              fourth k-step), and all eight drain each accumulator buffer
//              (kTcFlush k-steps of MMAs) into FP32 registers (tcgen05.ld) a
//              few k-steps after its window ends, releasing it; at the end of
//              a unit they store its 128 x 256 FP32 partial
// A final kernel sums the partials of each (t, p, n) in FP64 in a fixed order.
// Every mbarrier wait is bounded; on a timeout the CTA stops, reports
// kDevErrWaitTimeout, waits (bounded) for its copies and MMAs and frees TMEM.
#include <cuda_bf16.h>

#include "engine.cuh"
#include "momentum.hpp"
#include "tc.cuh"

namespace cgb {

namespace {

constexpr int kTcOpStages = 4;    // operand ring: phase tile + converted field tile
constexpr int kTcStgStages = 8;   // staging ring: complex64 field rows (HBM latency)
constexpr int kTcFlush = 2;       // k-steps per accumulator window (see the MMA issuer)
constexpr int kTcGroups = 4;      // converter groups of two warps, one k-step each in turn
constexpr int kTcDrainLag = 3;    // k-steps converted past a window's end before draining it (< kTcOpStages)
constexpr int kTcThreads = 352;   // 11 warps
constexpr int kTcHeader = 1024;   // barriers, TMEM slot, abort flag
constexpr int kTcTerms = 3;       // bf16 terms per operand value
constexpr int kTcABytes = kTcTerms * 8192;  // phase tile: {hi, mid, lo} x 256 rows x 16 bf16
constexpr int kTcBBytes = kTcTerms * 4096;  // field tile: {hi, mid, lo} x 128 pairs x 16 bf16
constexpr int kTcOpBytes = kTcABytes + kTcBBytes;
constexpr int kTcStgBytes = 8192; // 8 sites x 128 pairs x complex64
constexpr int kTcSmem = kTcHeader + kTcOpStages * kTcOpBytes + kTcStgStages * kTcStgBytes;
static_assert(kTcSmem <= 232448, "tensor-core projection does not fit in shared memory");
static_assert(kTcDrainLag < kTcOpStages, "a window is drained before its operand slots are reused");
// D[pair][row] (+)= field[pair][k] * phase[row][k]: M = 128 pairs, N = 256 rows.
constexpr uint32_t kTcIdesc = umma_idesc_bf16(128, 256);
constexpr uint32_t kTcLbo128 = 16 * 128, kTcLbo256 = 32 * 128, kTcSbo = 128;

struct TcParams {
  const float2 *field;          // [Lt][2 pair halves][V3][128] complex64, lexicographic sites
  const unsigned char *atiles;  // [MG][J][hi, mid, lo][256 rows x 16 bf16, core-matrix layout]
  float *partial;               // [U][128 pairs][256 momentum rows]
  DeviceStatus *status;
  TcGeom g;
};

struct Unit {
  int mg, jb, t, h, j0, j1;
};

__device__ __forceinline__ Unit decode(const TcGeom &g, int u)
{
  Unit w;
  w.h = u & 1;
  int r = u >> 1;
  w.t = r % g.lt;
  r /= g.lt;
  w.jb = r % g.jb;
  w.mg = r / g.jb;
  w.j0 = w.jb * g.ku;
  w.j1 = min(g.j, w.j0 + g.ku);
  return w;
}

__device__ __forceinline__ uint32_t bf16x2_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t *>(&v); }

// (a, b) -> packed bf16 hi, mid and lo terms (a in the low half); the
// remainders a - hi and a - hi - mid are exact in FP32.
__device__ __forceinline__ void split3(float a, float b, uint32_t &hi, uint32_t &mid, uint32_t &lo)
{
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  const float ra = a - hf.x, rb = b - hf.y;
  const __nv_bfloat162 m = __floats2bfloat162_rn(ra, rb);
  const float2 mf = __bfloat1622float2(m);
  hi = bf16x2_bits(h);
  mid = bf16x2_bits(m);
  lo = bf16x2_bits(__floats2bfloat162_rn(ra - mf.x, rb - mf.y));
}

__device__ __forceinline__ void tc_abort(volatile int *abort_flag, DeviceStatus *st, unsigned int where)
{
  *abort_flag = 1;
  report(st, kDevErrWaitTimeout, where);
}

__global__ void __launch_bounds__(kTcThreads, 1) momentum_gemm_tc(const __grid_constant__ TcParams p)
{
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *stg_full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *stg_empty = stg_full + kTcStgStages;
  uint64_t *a_full = stg_empty + kTcStgStages;
  uint64_t *op_full = a_full + kTcOpStages;
  uint64_t *op_empty = op_full + kTcOpStages;
  uint64_t *acc_full = op_empty + kTcOpStages;
  uint64_t *acc_empty = acc_full + 2;
  uint64_t *fin = acc_empty + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 512);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + 516);
  unsigned char *ops = smem + kTcHeader;
  unsigned char *stgs = ops + kTcOpStages * kTcOpBytes;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const TcGeom &g = p.g;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kTcStgStages; ++s) {
      mbar_init(&stg_full[s], 1);
      mbar_init(&stg_empty[s], 8 / kTcGroups);
    }
    for (int s = 0; s < kTcOpStages; ++s) {
      mbar_init(&a_full[s], 1);
      mbar_init(&op_full[s], 8 / kTcGroups);
      mbar_init(&op_empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 8);
    }
    mbar_init(fin, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 || warp == 10) {
    // ------------------------------------------- bulk-copy producers
    // warp 0: field rows into the staging ring (released by the converters);
    // warp 10: phase tiles into the operand ring (released by MMA completion).
    const bool field = warp == 0;
    const int nst = field ? kTcStgStages : kTcOpStages;
    uint64_t *full = field ? stg_full : a_full;
    uint64_t *empty = field ? stg_empty : op_empty;
    uint32_t gi = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < g.units && ok; u += gridDim.x) {
      const Unit w = decode(g, u);
      for (int j = w.j0; j < w.j1; ++j, ++gi) {
        const int s = gi % nst;
        if (gi >= (uint32_t)nst) {
          ok = __all_sync(0xffffffffu, mbar_wait_bounded(&empty[s], ((gi / nst) - 1) & 1, kWaitLimitNs));
          if (!ok) {
            if (lane == 0) tc_abort(abort_flag, p.status, (field ? 0x100000u : 0x600000u) | (unsigned)u);
            break;
          }
        }
        if (*abort_flag) {
          ok = false;
          break;
        }
        if (field) {
          // the step's sites of this pair half are contiguous: [t][half][site][128 pairs]
          const long long s0 = (long long)j * 8;
          const int nvalid = (int)min(8LL, g.v3 - s0);
          if (lane == 0) {
            mbar_arrive_expect_tx(&full[s], (uint32_t)(nvalid * 1024));
            bulk_g2s(stgs + s * kTcStgBytes, p.field + (((size_t)w.t * 2 + w.h) * g.v3 + s0) * 128,
                     (uint32_t)(nvalid * 1024), &full[s]);
          }
        } else if (lane == 0) {
          mbar_arrive_expect_tx(&full[s], (uint32_t)kTcABytes);
          bulk_g2s(ops + s * kTcOpBytes, p.atiles + ((size_t)w.mg * g.j + j) * kTcABytes, kTcABytes, &full[s]);
        }
      }
    }
    if (!ok) {  // let the copies already issued land before the CTA exits
      const uint32_t from = gi > (uint32_t)nst ? gi - nst : 0;
      for (uint32_t k = from; k < gi; ++k) mbar_wait_bounded(&full[k % nst], (k / nst) & 1, kWaitLimitNs / 8);
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    // A window is kTcFlush k-steps into one accumulator buffer.  Its MMAs run
    // small terms first: the five second-order term pairs of every k-step of
    // the window, then the hi x hi products.  The tensor core's FP32
    // accumulation truncates toward zero relative to the accumulator, so the
    // small terms accumulate while it is small and only kTcFlush truncations
    // fall at the scale of the window's sum.
    uint32_t gi = 0, win = 0;
    bool ok = true;
    const uint32_t sbase = smem_addr(ops);
    for (int u = blockIdx.x; u < g.units && ok; u += gridDim.x) {
      const Unit w = decode(g, u);
      const int n = w.j1 - w.j0;
      for (int i0 = 0; i0 < n && ok; i0 += kTcFlush) {
        const int nw = min(kTcFlush, n - i0);
        const uint32_t buf = win & 1, d = tmem + buf * 256;
        bool okw = win < 2 || mbar_wait_bounded(&acc_empty[buf], ((win >> 1) - 1) & 1, kWaitLimitNs);
        for (int i = 0; i < nw; ++i) {
          const uint32_t gk = gi + i;
          const int s = gk % kTcOpStages;
          okw = okw && mbar_wait_bounded(&a_full[s], (gk / kTcOpStages) & 1, kWaitLimitNs);
          okw = okw && mbar_wait_bounded(&op_full[s], (gk / kTcOpStages) & 1, kWaitLimitNs);
          ok = __all_sync(0xffffffffu, okw) && !*abort_flag;
          if (!ok) {
            if (lane == 0) tc_abort(abort_flag, p.status, 0x200000u | (unsigned)u);
            break;
          }
          tc_fence_after();
          if (lane == 0) {
            const uint32_t st = sbase + s * kTcOpBytes;
            const uint64_t ph = umma_desc(st, kTcLbo256, kTcSbo);              // phase tile, hi
            const uint64_t pm = umma_desc(st + 8192, kTcLbo256, kTcSbo);       // phase tile, mid
            const uint64_t pl = umma_desc(st + 2 * 8192, kTcLbo256, kTcSbo);   // phase tile, lo
            const uint64_t fh = umma_desc(st + kTcABytes, kTcLbo128, kTcSbo);  // field tile, hi
            const uint64_t fm = umma_desc(st + kTcABytes + 4096, kTcLbo128, kTcSbo);
            const uint64_t fl = umma_desc(st + kTcABytes + 2 * 4096, kTcLbo128, kTcSbo);
            umma_bf16(d, fh, pm, kTcIdesc, i == 0 ? 0u : 1u);
            umma_bf16(d, fm, ph, kTcIdesc, 1u);
            umma_bf16(d, fm, pm, kTcIdesc, 1u);
            umma_bf16(d, fh, pl, kTcIdesc, 1u);
            umma_bf16(d, fl, ph, kTcIdesc, 1u);
          }
          __syncwarp();
        }
        if (!ok) break;
        if (lane == 0) {
          for (int i = 0; i < nw; ++i) {
            const int s = (gi + i) % kTcOpStages;
            const uint32_t st = sbase + s * kTcOpBytes;
            umma_bf16(d, umma_desc(st + kTcABytes, kTcLbo128, kTcSbo), umma_desc(st, kTcLbo256, kTcSbo), kTcIdesc,
                      1u);
            umma_commit(&op_empty[s]);  // the k-step's operands are free once its MMAs complete
          }
          umma_commit(&acc_full[buf]);
        }
        __syncwarp();
        gi += nw;
        ++win;
      }
    }
    // every MMA issued by this CTA completes before TMEM is released
    if (lane == 0) umma_commit(fin);
    __syncwarp();
    mbar_wait_bounded(fin, 0, kWaitLimitNs);
  } else {
    // ---------------------------------------- convert + accumulate + store
    const int wi = warp - 2;
    const int q = warp & 3, mt = wi >> 2, row = 32 * q + lane;  // TMEM lane quarter of this warp
    // conversion: group gp converts every kTcGroups-th k-step; its 64 threads
    // take pairs t64 and t64 + 64 over all 8 sites of the step
    const int gp = wi >> 1, t64 = ((wi & 1) << 5) | lane;
    float run[128];
#pragma unroll
    for (int k = 0; k < 128; ++k) run[k] = 0.f;
    uint32_t gi = 0, win = 0;
    // Windows whose MMAs are issued but not yet drained (at most two, one per
    // accumulator buffer): window index, unit, last window of the unit, and
    // the k-step that ended it.
    int nq = 0, qw0 = 0, qw1 = 0, qu0 = 0, qu1 = 0;
    bool ql0 = false, ql1 = false;
    uint32_t qe0 = 0, qe1 = 0;
    bool ok = true;

    auto flush = [&](int wdx) -> bool {
      const uint32_t b = wdx & 1;
      const bool okw = __all_sync(0xffffffffu, mbar_wait_bounded(&acc_full[b], (wdx >> 1) & 1, kWaitLimitNs));
      if (!okw || *abort_flag) return false;
      tc_fence_after();
      const uint32_t base = tmem + ((uint32_t)(32 * q) << 16) + b * 256 + mt * 128;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        float v[32];
        tmem_ld32(base + 32 * k, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) run[32 * k + i] += v[i];
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[b]);
      return true;
    };
    auto store = [&](int unit) {  // this thread: pair `row`, momentum rows mt*128 .. mt*128 + 127
      float4 *dst = reinterpret_cast<float4 *>(p.partial + ((size_t)unit * 128 + row) * 256 + mt * 128);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        dst[k] = make_float4(run[4 * k], run[4 * k + 1], run[4 * k + 2], run[4 * k + 3]);
        run[4 * k] = run[4 * k + 1] = run[4 * k + 2] = run[4 * k + 3] = 0.f;
      }
    };
    // Drain the oldest pending window: its accumulator into `run`, and the
    // unit's partial when it was the unit's last window.
    auto drain_front = [&]() -> bool {
      if (!flush(qw0)) return false;
      if (ql0) store(qu0);
      qw0 = qw1;
      qu0 = qu1;
      ql0 = ql1;
      qe0 = qe1;
      --nq;
      return true;
    };

    for (int u = blockIdx.x; u < g.units && ok; u += gridDim.x) {
      const Unit w = decode(g, u);
      const int n = w.j1 - w.j0;
      for (int i = 0; i < n; ++i, ++gi) {
        if ((int)(gi % kTcGroups) == gp) {
          const int ss = gi % kTcStgStages, so = gi % kTcOpStages;
          bool okw = mbar_wait_bounded(&stg_full[ss], (gi / kTcStgStages) & 1, kWaitLimitNs);
          // the operand slot's field tile is free once the MMAs of k-step gi - kTcOpStages completed
          if (gi >= (uint32_t)kTcOpStages)
            okw = okw && mbar_wait_bounded(&op_empty[so], ((gi / kTcOpStages) - 1) & 1, kWaitLimitNs);
          ok = __all_sync(0xffffffffu, okw) && !*abort_flag;
          if (!ok) {
            if (lane == 0) tc_abort(abort_flag, p.status, 0x300000u | (unsigned)u);
            break;
          }
          const unsigned char *stg = stgs + ss * kTcStgBytes;
          unsigned char *bt = ops + so * kTcOpBytes + kTcABytes;
          const long long s0 = (long long)(w.j0 + i) * 8;
#pragma unroll
          for (int pp = 0; pp < 2; ++pp) {
            const int pair = t64 + 64 * pp;
#pragma unroll
            for (int sh = 0; sh < 2; ++sh) {
              uint32_t hi[4], mid[4], lo[4];
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                const int s8 = sh * 4 + k;
                float2 c = make_float2(0.f, 0.f);
                if (s0 + s8 < g.v3) c = reinterpret_cast<const float2 *>(stg + s8 * 1024)[pair];
                split3(c.x, c.y, hi[k], mid[k], lo[k]);
              }
              const uint32_t off = (sh * 16 + (pair >> 3)) * 128 + (pair & 7) * 16;
              *reinterpret_cast<uint4 *>(bt + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
              *reinterpret_cast<uint4 *>(bt + 4096 + off) = make_uint4(mid[0], mid[1], mid[2], mid[3]);
              *reinterpret_cast<uint4 *>(bt + 2 * 4096 + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
            }
          }
          fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(&stg_empty[ss]);
            mbar_arrive(&op_full[so]);
          }
        }
        if ((i % kTcFlush) == kTcFlush - 1 || i == n - 1) {  // this k-step ends a window
          if (nq == 0) {
            qw0 = (int)win++;
            qu0 = u;
            ql0 = i == n - 1;
            qe0 = gi;
          } else {
            qw1 = (int)win++;
            qu1 = u;
            ql1 = i == n - 1;
            qe1 = gi;
          }
          ++nq;
        }
        // Drain a window once kTcDrainLag more k-steps are converted (the MMAs
        // have then caught up with it), or at once when both buffers are pending.
        while (nq > 0 && (nq == 2 || gi - qe0 >= (uint32_t)kTcDrainLag)) {
          if (!drain_front()) {
            ok = false;
            break;
          }
        }
        if (!ok) {
          if (lane == 0) tc_abort(abort_flag, p.status, 0x400000u | (unsigned)u);
          break;
        }
      }
    }
    while (ok && nq > 0) {
      if (!drain_front()) {
        ok = false;
        if (lane == 0) tc_abort(abort_flag, p.status, 0x500000u);
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, 512);
}

// Phase tiles: for momentum group mg and k-step j, the two 128-row m-tiles
// (64 momenta x {Re, Im} rows each) over the 8 sites of the step, bf16 hi,
// mid and lo, in the K-major core-matrix layout.  Phi = ex * ey * ez in FP64 from the
// FP64 tables exp(2 pi i k / L), k = (n * x) mod L exactly.
__global__ void __launch_bounds__(256) momentum_phase_tiles(unsigned char *__restrict__ atiles,
                                                            const __grid_constant__ MomPlan plan, long long v3, int nj)
{
  const int j = blockIdx.x, mg = blockIdx.y;
  const int mt = threadIdx.x >> 7, r = threadIdx.x & 127;
  const int pm = mg * 128 + mt * 64 + (r >> 1), comp = r & 1;
  const int lx = plan.latt[0], ly = plan.latt[1], lz = plan.latt[2];
  // The threads index the tables at different places: read them from shared
  // memory, not from the (constant-bank) kernel parameters.
  __shared__ double tab[6][kMomMaxL];
  for (int e = threadIdx.x; e < 6 * kMomMaxL; e += blockDim.x) {
    const int q = e / kMomMaxL, k = e % kMomMaxL;
    const double *src = q == 0 ? plan.cosx : q == 1 ? plan.sinx : q == 2 ? plan.cosy : q == 3 ? plan.siny
                        : q == 4 ? plan.cosz : plan.sinz;
    tab[q][k] = src[k];
  }
  __syncthreads();
  const bool live = pm < plan.np;
  int nx = 0, ny = 0, nz = 0;
  if (live) {
    const int qq = plan.p_q[pm];
    nx = plan.px[plan.q_ix[qq]];
    ny = plan.q_ny[qq];
    nz = plan.p_nz[pm];
  }
  uint32_t w[2][kTcTerms][4];
  // site coordinates and phase indices k = (n * x) mod L, advanced site by site
  const long long s_first = (long long)j * 8;
  int x = (int)(s_first % lx), y = (int)((s_first / lx) % ly), z = (int)(s_first / ((long long)lx * ly));
  const int sx = ((nx % lx) + lx) % lx, sy = ((ny % ly) + ly) % ly;
  int kx = (int)(((long long)sx * x) % lx), ky = (int)(((long long)sy * y) % ly);
#pragma unroll
  for (int s8 = 0; s8 < 8; ++s8) {
    const long long s = s_first + s8;
    double re = 0.0, im = 0.0;
    if (live && s < v3) {
      const int kz = ((nz * z) % lz + lz) % lz;
      const double axr = tab[0][kx], axi = tab[1][kx], ayr = tab[2][ky], ayi = tab[3][ky];
      const double azr = tab[4][kz], azi = tab[5][kz];
      const double xyr = axr * ayr - axi * ayi, xyi = axr * ayi + axi * ayr;
      re = xyr * azr - xyi * azi;
      im = xyr * azi + xyi * azr;
    }
    // next site: x + 1, carrying into y and z
    if (++x == lx) {
      x = 0;
      kx = 0;
      if (++y == ly) {
        y = 0;
        ky = 0;
        ++z;
      } else if ((ky += sy) >= ly) {
        ky -= ly;
      }
    } else if ((kx += sx) >= lx) {
      kx -= lx;
    }
    const double a0 = comp ? im : re, a1 = comp ? re : -im;  // columns 2s (Re C) and 2s+1 (Im C)
    // three bf16 terms, each the rounded FP64 remainder of the ones before
    double r0 = a0, r1 = a1;
#pragma unroll
    for (int tm = 0; tm < kTcTerms; ++tm) {
      const __nv_bfloat162 h = __floats2bfloat162_rn((float)r0, (float)r1);
      const float2 hf = __bfloat1622float2(h);
      w[s8 >> 2][tm][s8 & 3] = bf16x2_bits(h);
      r0 -= (double)hf.x;
      r1 -= (double)hf.y;
    }
  }
  // one 256-row tile per term (hi, mid, lo): row mt * 128 + r
  unsigned char *tile = atiles + ((size_t)mg * nj + j) * kTcABytes;
  const int row = mt * 128 + r;
#pragma unroll
  for (int kc = 0; kc < 2; ++kc) {
    const uint32_t off = (kc * 32 + (row >> 3)) * 128 + (row & 7) * 16;
#pragma unroll
    for (int tm = 0; tm < kTcTerms; ++tm)
      *reinterpret_cast<uint4 *>(tile + tm * 8192 + off) =
        make_uint4(w[kc][tm][0], w[kc][tm][1], w[kc][tm][2], w[kc][tm][3]);
  }
}

// out[p][t][n] = sum over the k-blocks of the unit partials, FP64, fixed order.
// One CTA per (pair-local n, half h, t + Lt * group); thread = momentum row.
__global__ void __launch_bounds__(256) momentum_tc_reduce(const float *__restrict__ partial, double *__restrict__ out,
                                                          const __grid_constant__ TcGeom g, int np)
{
  const int pl = blockIdx.x, h = blockIdx.y, t = blockIdx.z % g.lt, mg = blockIdx.z / g.lt, r = threadIdx.x;
  const int pm = mg * 128 + (r >> 1);
  double acc = 0.0;
  for (int jb = 0; jb < g.jb; ++jb) {
    const long long u = ((long long)(mg * g.jb + jb) * g.lt + t) * 2 + h;
    acc += (double)partial[((size_t)u * 128 + pl) * 256 + r];
  }
  if (pm < np) out[(((size_t)pm * g.lt + t) * 256 + h * 128 + pl) * 2 + (r & 1)] = acc;
}

} // namespace

TcGeom make_tc_geom(const MomPlan &plan, int unit_steps)
{
  TcGeom g {};
  g.v3 = (long long)plan.latt[0] * plan.latt[1] * plan.latt[2];
  g.lt = plan.latt[3];
  g.j = (int)((g.v3 + 7) / 8);
  g.ku = g.j < unit_steps ? g.j : unit_steps;
  g.jb = (g.j + g.ku - 1) / g.ku;
  g.mg = (plan.np + 127) / 128;
  g.units = g.mg * g.jb * g.lt * 2;
  return g;
}

size_t tc_phase_bytes(const TcGeom &g) { return (size_t)g.mg * g.j * kTcABytes; }
size_t tc_partial_bytes(const TcGeom &g) { return (size_t)g.units * 2 * 128 * 128 * sizeof(float); }

cudaError_t launch_momentum_tc(const Job &job, const MomPlan &plan, const TcGeom &g, const void *field,
                               unsigned char *atiles, float *partial, void *out, bool tiles_ready)
{
  static bool attr_set[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 64 && !attr_set[dev]) {
    e = cudaFuncSetAttribute(momentum_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
    if (e != cudaSuccess) return e;
    attr_set[dev] = true;
  }
  if (!tiles_ready) {
    momentum_phase_tiles<<<dim3(g.j, g.mg), 256, 0, job.stream>>>(atiles, plan, g.v3, g.j);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  TcParams tp;
  tp.field = static_cast<const float2 *>(field);
  tp.atiles = atiles;
  tp.partial = partial;
  tp.status = job.status;
  tp.g = g;
  const int grid = g.units < job.num_sms ? g.units : job.num_sms;
  momentum_gemm_tc<<<grid, kTcThreads, kTcSmem, job.stream>>>(tp);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  momentum_tc_reduce<<<dim3(128, 2, g.lt * g.mg), 256, 0, job.stream>>>(partial, static_cast<double *>(out), g,
                                                                        plan.np);
  return cudaGetLastError();
}

} // namespace cgb
