// Device-side building blocks shared by every contraction kernel (sm_103a).
//
//  * cx<R>        complex value in registers, R = float (mixed form) or double (plain form)
//  * phase codes  {0,1,2,3} <-> {+1, +i, -1, -i}; every entry of a DeGrand-Rossi gamma
//                 matrix is one of these, so multiplying by one is a swap plus sign
//                 flips done with integer ops -- no FP64/FP32 pipe work
//  * mbarrier + cp.async.bulk (TMA 1D bulk copies) helpers, with time-bounded waits
//  * the device status word kernels report errors through
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cgb {

// ------------------------------------------------------------------ status --
// Bits OR-ed into DeviceStatus::flags by kernels; read back by contract_get_last_error().
enum : unsigned int {
  kDevErrWaitTimeout = 1u << 0,   // an mbarrier wait ran past its time limit
  kDevErrBadWork = 1u << 1,       // a work-queue descriptor failed validation
};

struct DeviceStatus {
  unsigned int flags;
  unsigned int where;   // kernel-defined detail (e.g. tile index of the first failure)
};

__device__ __forceinline__ void report(DeviceStatus *st, unsigned int bit, unsigned int where)
{
  if (st) {
    if ((atomicOr(&st->flags, bit) & bit) == 0) atomicExch(&st->where, where);
  }
}

// ----------------------------------------------------------------- complex --
template <class R> struct cx {
  R x, y;
};

template <class R> __device__ __forceinline__ cx<R> czero() { return {R(0), R(0)}; }

template <class R> __device__ __forceinline__ cx<R> cadd(cx<R> a, cx<R> b) { return {a.x + b.x, a.y + b.y}; }

template <class R> __device__ __forceinline__ cx<R> cmul(cx<R> a, cx<R> b)
{
  return {fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x)};
}

// acc += a * b
template <class R> __device__ __forceinline__ void cfma(cx<R> &acc, cx<R> a, cx<R> b)
{
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}

// acc -= a * b
template <class R> __device__ __forceinline__ void cfms(cx<R> &acc, cx<R> a, cx<R> b)
{
  acc.x = fma(-a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(-a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}

// acc += a * conj(b)
template <class R> __device__ __forceinline__ void cfma_conj(cx<R> &acc, cx<R> a, cx<R> b)
{
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.y, b.x, acc.y);
  acc.y = fma(-a.x, b.y, acc.y);
}

__device__ __forceinline__ float flip_sign(float v, uint32_t s)
{
  return __uint_as_float(__float_as_uint(v) ^ (s << 31));
}
__device__ __forceinline__ double flip_sign(double v, uint32_t s)
{
  return __longlong_as_double(__double_as_longlong(v) ^ ((unsigned long long)s << 63));
}

// z * i^p for a phase code p in {0,1,2,3}: (x,y) (-y,x) (-x,-y) (y,-x).
template <class R> __device__ __forceinline__ cx<R> mul_phase(cx<R> z, uint32_t p)
{
  const bool swap = p & 1u;
  const R a = swap ? z.y : z.x;
  const R b = swap ? z.x : z.y;
  return {flip_sign(a, ((p + 1u) >> 1) & 1u), flip_sign(b, p >> 1)};
}

template <class R> __device__ __forceinline__ cx<R> conj(cx<R> z) { return {z.x, -z.y}; }

// Storage <-> register conversions.  Propagators are stored as interleaved
// (re, im) pairs: complex128 (double2) in the plain form, complex64 (float2) in
// the mixed form.
template <class R> __device__ __forceinline__ cx<R> ld(const double2 *p)
{
  const double2 v = *p;
  return {R(v.x), R(v.y)};
}
template <class R> __device__ __forceinline__ cx<R> ld(const float2 *p)
{
  const float2 v = *p;
  return {R(v.x), R(v.y)};
}
__device__ __forceinline__ void st(double2 *p, cx<double> v) { *p = make_double2(v.x, v.y); }
__device__ __forceinline__ void st(double2 *p, cx<float> v) { *p = make_double2(v.x, v.y); }
__device__ __forceinline__ void st(float2 *p, cx<float> v) { *p = make_float2(v.x, v.y); }
__device__ __forceinline__ void st(float2 *p, cx<double> v) { *p = make_float2(float(v.x), float(v.y)); }

template <class R> __device__ __forceinline__ cx<R> shfl_xor(cx<R> v, int lane_mask)
{
  return {__shfl_xor_sync(0xffffffffu, v.x, lane_mask), __shfl_xor_sync(0xffffffffu, v.y, lane_mask)};
}

// Sum v over the TPS consecutive lanes of a group (TPS a power of two <= 32).
template <int TPS, class R> __device__ __forceinline__ cx<R> group_sum(cx<R> v)
{
#pragma unroll
  for (int o = TPS / 2; o > 0; o >>= 1) v = cadd(v, shfl_xor(v, o));
  return v;
}

// Sum each of NOUT values over the TPS threads of a site and leave the sum of
// value o with the thread whose sub == o (o < NOUT <= TPS), by recursive
// halving: at the step of lane distance h the thread keeps the upper or lower
// half of its values as (sub & h) says and receives its partner's share of
// that half, so TPS - 1 shuffles in all instead of NOUT log2(TPS).
template <int TPS, int NOUT> constexpr bool kScatterSums = NOUT > TPS / 2 && NOUT <= TPS;
template <int TPS, int NOUT, class R>
__device__ __forceinline__ cx<R> group_reduce_scatter(const cx<R> (&vals)[NOUT], int sub)
{
  static_assert(NOUT <= TPS && (TPS & (TPS - 1)) == 0, "one value per thread, TPS a power of two");
  cx<R> v[TPS];
#pragma unroll
  for (int i = 0; i < TPS; ++i) v[i] = i < NOUT ? vals[i] : czero<R>();
#pragma unroll
  for (int h = TPS / 2; h > 0; h >>= 1) {
    const bool hi = (sub & h) != 0;
#pragma unroll
    for (int i = 0; i < h; ++i) {
      const cx<R> send = hi ? v[i] : v[h + i], keep = hi ? v[h + i] : v[i];
      v[i] = cadd(keep, shfl_xor(send, h));
    }
  }
  return v[0];
}

// ------------------------------------------------------------ colour maths --
// 3x3 colour blocks are 9 consecutive complex numbers, row = sink colour.

// d += x ^ y, where (x ^ y)[a][e] = sum_{b,c,f,g} eps_abc eps_efg x[b][f] y[c][g].
// For each (a, e) that is four products:
//   x[a1][e1] y[a2][e2] - x[a1][e2] y[a2][e1] - x[a2][e1] y[a1][e2] + x[a2][e2] y[a1][e1]
// with a1 = a+1, a2 = a+2, e1 = e+1, e2 = e+2 (mod 3).
template <class R> __device__ __forceinline__ void wedge_acc(cx<R> d[9], const cx<R> x[9], const cx<R> y[9])
{
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int a1 = (a + 1) % 3, a2 = (a + 2) % 3;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const int e1 = (e + 1) % 3, e2 = (e + 2) % 3;
      cx<R> &o = d[3 * a + e];
      cfma(o, x[3 * a1 + e1], y[3 * a2 + e2]);
      cfms(o, x[3 * a1 + e2], y[3 * a2 + e1]);
      cfms(o, x[3 * a2 + e1], y[3 * a1 + e2]);
      cfma(o, x[3 * a2 + e2], y[3 * a1 + e1]);
    }
  }
}

// sum_ad x[ad] * y[ad]
template <class R> __device__ __forceinline__ cx<R> dot9(const cx<R> x[9], const cx<R> y[9])
{
  cx<R> s = czero<R>();
#pragma unroll
  for (int k = 0; k < 9; ++k) cfma(s, x[k], y[k]);
  return s;
}

// Complex64 forms on packed FP32x2 FMAs (one instruction updates both lanes
// of a (re, im) pair; the issue slots of the products halve).
//   x * y = x y.x + (i x) y.y: x and i x = (-x.y, x.x) as pairs, y.x and y.y
//   broadcast to both lanes.
__device__ __forceinline__ float2 bcast2(float v) { return make_float2(v, v); }

__device__ __forceinline__ void wedge_acc(cx<float> d[9], const cx<float> x[9], const cx<float> y[9])
{
  float2 xn[9], xr[9], o[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    xn[q] = make_float2(x[q].x, x[q].y);
    xr[q] = make_float2(-x[q].y, x[q].x);
    o[q] = make_float2(d[q].x, d[q].y);
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int a1 = (a + 1) % 3, a2 = (a + 2) % 3;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      const int e1 = (e + 1) % 3, e2 = (e + 2) % 3;
      float2 &t = o[3 * a + e];
      const cx<float> p = y[3 * a2 + e2], m1 = y[3 * a2 + e1], m2 = y[3 * a1 + e2], p2 = y[3 * a1 + e1];
      t = __ffma2_rn(xn[3 * a1 + e1], bcast2(p.x), t);
      t = __ffma2_rn(xr[3 * a1 + e1], bcast2(p.y), t);
      t = __ffma2_rn(xn[3 * a1 + e2], bcast2(-m1.x), t);
      t = __ffma2_rn(xr[3 * a1 + e2], bcast2(-m1.y), t);
      t = __ffma2_rn(xn[3 * a2 + e1], bcast2(-m2.x), t);
      t = __ffma2_rn(xr[3 * a2 + e1], bcast2(-m2.y), t);
      t = __ffma2_rn(xn[3 * a2 + e2], bcast2(p2.x), t);
      t = __ffma2_rn(xr[3 * a2 + e2], bcast2(p2.y), t);
    }
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) d[q] = {o[q].x, o[q].y};
}

// sum x[k] y[k] = (A.x - B.y, A.y + B.x) with A = sum x.x y, B = sum x.y y.
__device__ __forceinline__ cx<float> dot9(const cx<float> x[9], const cx<float> y[9])
{
  float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const float2 yv = make_float2(y[k].x, y[k].y);
    A = __ffma2_rn(yv, bcast2(x[k].x), A);
    B = __ffma2_rn(yv, bcast2(x[k].y), B);
  }
  return {A.x - B.y, A.y + B.x};
}

template <class R, class S> __device__ __forceinline__ void load9(cx<R> out[9], const S *blk)
{
#pragma unroll
  for (int k = 0; k < 9; ++k) out[k] = ld<R>(blk + k);
}

// A 9-complex colour block of a site slot whose spin-block index parity is
// known at compile time.  Slots are 16-byte aligned and blocks are 72 bytes
// apart, so an even block starts on a 16-byte boundary and an odd one 8 bytes
// past it: complex64 blocks load as four 16-byte vectors plus one 8-byte
// value (5 loads instead of 9).  Complex128 values are 16 bytes already.
template <bool ODD, class R> __device__ __forceinline__ void load9p(cx<R> out[9], const float2 *blk)
{
  if constexpr (!ODD) {
    const float4 *v = reinterpret_cast<const float4 *>(blk);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 t = v[q];
      out[2 * q] = {R(t.x), R(t.y)};
      out[2 * q + 1] = {R(t.z), R(t.w)};
    }
    out[8] = ld<R>(blk + 8);
  } else {
    out[0] = ld<R>(blk);
    const float4 *v = reinterpret_cast<const float4 *>(blk + 1);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 t = v[q];
      out[1 + 2 * q] = {R(t.x), R(t.y)};
      out[2 + 2 * q] = {R(t.z), R(t.w)};
    }
  }
}
template <bool ODD, class R> __device__ __forceinline__ void load9p(cx<R> out[9], const double2 *blk)
{
  load9(out, blk);
}

// Two consecutive complex values to a 16-byte (complex64) or 32-byte
// (complex128) aligned address, as vector stores.
__device__ __forceinline__ void st2(float2 *p, cx<float> a, cx<float> b)
{
  *reinterpret_cast<float4 *>(p) = make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void st2(double2 *p, cx<double> a, cx<double> b)
{
  p[0] = make_double2(a.x, a.y);
  p[1] = make_double2(b.x, b.y);
}

template <class R> __device__ __forceinline__ void phase9(cx<R> v[9], uint32_t p)
{
#pragma unroll
  for (int k = 0; k < 9; ++k) v[k] = mul_phase(v[k], p);
}

// ---------------------------------------------------- mbarrier / bulk copy --
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
  uint32_t done;
  asm volatile(
    "{\n\t.reg .pred p;\n\t"
    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
    "selp.u32 %0, 1, 0, p;\n\t}"
    : "=r"(done)
    : "r"(smem_addr(bar)), "r"(parity)
    : "memory");
  return done != 0;
}

__device__ __forceinline__ uint64_t global_timer_ns()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Wait for phase `parity` of an mbarrier, giving up after `limit_ns`
// nanoseconds of wall time (and, as a backstop, after 2^26 polls).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint64_t limit_ns)
{
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  for (uint32_t it = 0; it < (1u << 26); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63u) == 63u && global_timer_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// The same for a waiter that is normally early (a producer waiting for a ring
// stage to be released): between polls it sleeps about `sleep_ns`, so that
// its polling does not take issue slots from the warps it waits for.
__device__ __forceinline__ bool mbar_wait_bounded_backoff(uint64_t *bar, uint32_t parity, uint64_t limit_ns,
                                                          unsigned sleep_ns)
{
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  for (uint32_t it = 0; it < (1u << 26); ++it) {
    __nanosleep(sleep_ns);
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 15u) == 15u && global_timer_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// Global -> shared bulk copy (TMA, non-tensor form).  Both addresses 16-byte
// aligned, bytes a multiple of 16; completion is signalled on `bar`.
__device__ __forceinline__ void bulk_g2s(void *sdst, const void *gsrc, uint32_t bytes, uint64_t *bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                 smem_addr(sdst)),
               "l"(gsrc), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Shared -> global bulk copy; tracked by the issuing thread's bulk group.
__device__ __forceinline__ void bulk_s2g(void *gdst, const void *ssrc, uint32_t bytes)
{
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_addr(ssrc)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Wait until at most N committed store groups still read shared memory.
template <int N> __device__ __forceinline__ void bulk_wait_read()
{
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
template <int N> __device__ __forceinline__ void bulk_wait()
{
  asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory");
}

} // namespace cgb
