// Propagators in QUDA's native device order <-> PyQUDA even/odd propagators,
// and an in-place change of spin basis.
//
// A propagator on QUDA's side is twelve colour-spinor fields, one per source
// (spin k, colour d), field f = 3 k + d, as its solver leaves them on the
// device.  Each field is in QUDA's native "FloatN" order
//   [parity][chunk][stride][16 bytes],
// a chunk holding 16 bytes of the site's spin-colour vector (sink spin s,
// sink colour c), complex entry e = 3 s + c:
//   complex128 (QUDA_FLOAT2_FIELD_ORDER): chunk q = entry q        (12 chunks)
//   complex64  (QUDA_FLOAT4_FIELD_ORDER): chunk q = entries 2q, 2q+1 (6 chunks)
// and stride >= V/2 the (padded) checkerboard length.  QUDA's checkerboard
// index of site (x, y, z, t) is ((t Lz + z) Ly + y) (Lx/2) + x/2 with parity
// (x + y + z + t) & 1 -- exactly the PyQUDA even/odd site order, so a site
// keeps its index and only the 144 complex entries move:
//   P[p * V/2 + x_cb][s][k][c][d] = field[3k + d][p][chunk of (s, c)][x_cb].
//
// A CTA moves tiles of TS consecutive checkerboard sites of one parity through
// shared memory: it reads every (field, chunk) run of TS sites (TS x 16
// contiguous bytes) and writes TS whole sites (contiguous), or the reverse.
// Pure data movement: conversions in both directions are bit-exact.
#include <algorithm>

#include "launch.hpp"

namespace cgb {

namespace {

template <int ES> struct QudaShape {
  static constexpr int NQ = ES == 16 ? 12 : 6;       // chunks per field and parity
  static constexpr int EPC = 16 / ES;                // complex entries per chunk
  static constexpr int TS = ES == 16 ? 16 : 32;      // sites per tile
  static constexpr int SITE = 144 * ES;              // bytes per propagator site
  static constexpr int SMEM = TS * SITE;             // 36 KB either way
};

// Byte offset, within a site of the PyQUDA propagator, of complex entry
// e = 3 s + c of field f = 3 k + d.
template <int ES> __device__ __forceinline__ int prop_entry_offset(int f, int e)
{
  const int k = f / 3, d = f - 3 * k, s = e / 3, c = e - 3 * s;
  return (((s * 4 + k) * 3 + c) * 3 + d) * ES;
}

struct QudaFields {
  char *f[12];
};

template <class R> struct Cplx { using type = double2; };
template <> struct Cplx<float> { using type = float2; };

template <int ES, bool FROM_QUDA>
__global__ void __launch_bounds__(256) quda_layout_kernel(char *__restrict__ prop, const QudaFields fields,
                                                          long long half_volume, long long stride)
{
  using Sh = QudaShape<ES>;
  extern __shared__ __align__(16) unsigned char qsm[];
  const long long tiles_per_parity = (half_volume + Sh::TS - 1) / Sh::TS;
  const long long tiles = 2 * tiles_per_parity;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int par = (int)(tile / tiles_per_parity);
    const long long x0 = (tile - par * tiles_per_parity) * Sh::TS;
    const int n = (int)(half_volume - x0 < Sh::TS ? half_volume - x0 : Sh::TS);
    char *site0 = prop + ((long long)par * half_volume + x0) * Sh::SITE;
    if (!FROM_QUDA) {  // whole sites in, contiguous
      const uint4 *src = reinterpret_cast<const uint4 *>(site0);
      for (int w = threadIdx.x; w < n * Sh::SITE / 16; w += blockDim.x)
        reinterpret_cast<uint4 *>(qsm)[w] = src[w];
      __syncthreads();
    }
    // (field, chunk, site) pieces; consecutive threads take consecutive sites
    for (int w = threadIdx.x; w < 12 * Sh::NQ * Sh::TS; w += blockDim.x) {
      const int x = w % Sh::TS, fq = w / Sh::TS, f = fq / Sh::NQ, q = fq - f * Sh::NQ;
      if (x >= n) continue;
      uint4 *g = reinterpret_cast<uint4 *>(fields.f[f]) + ((long long)par * Sh::NQ + q) * stride + x0 + x;
      unsigned char *site = qsm + x * Sh::SITE;
      if (FROM_QUDA) {
        const uint4 v = *g;
        if (ES == 16) {
          *reinterpret_cast<uint4 *>(site + prop_entry_offset<16>(f, q)) = v;
        } else {
          *reinterpret_cast<uint2 *>(site + prop_entry_offset<8>(f, 2 * q)) = make_uint2(v.x, v.y);
          *reinterpret_cast<uint2 *>(site + prop_entry_offset<8>(f, 2 * q + 1)) = make_uint2(v.z, v.w);
        }
      } else {
        uint4 v;
        if (ES == 16) {
          v = *reinterpret_cast<const uint4 *>(site + prop_entry_offset<16>(f, q));
        } else {
          const uint2 a = *reinterpret_cast<const uint2 *>(site + prop_entry_offset<8>(f, 2 * q));
          const uint2 b = *reinterpret_cast<const uint2 *>(site + prop_entry_offset<8>(f, 2 * q + 1));
          v = make_uint4(a.x, a.y, b.x, b.y);
        }
        *g = v;
      }
    }
    __syncthreads();
    if (FROM_QUDA) {  // whole sites out, contiguous
      uint4 *dst = reinterpret_cast<uint4 *>(site0);
      for (int w = threadIdx.x; w < n * Sh::SITE / 16; w += blockDim.x)
        dst[w] = reinterpret_cast<const uint4 *>(qsm)[w];
      __syncthreads();
    }
  }
}

// P'[s][k] = sum_{s', k'} U[s][s'] P[s'][k'] conj(U[k][k']) for every colour
// pair (c, d).  One thread per (site, c, d): its 16 spin entries are a 4 x 4
// matrix M, and M' = U M U^dagger as two 4 x 4 products.  U is uniform across
// the grid, so its zero entries (most spin-basis changes have two nonzeros
// per row) are skipped by uniform branches.
template <class R> struct SpinRotation {
  R u[4][4][2];
  int nz[4][4];
};

template <class R> __device__ __forceinline__ void cmac(R &re, R &im, R ar, R ai, R br, R bi)
{
  re = fma(ar, br, re);
  re = fma(-ai, bi, re);
  im = fma(ar, bi, im);
  im = fma(ai, br, im);
}

template <class R>
__global__ void __launch_bounds__(256) spin_rotation_kernel(typename Cplx<R>::type *__restrict__ prop, long long volume,
                                                            const SpinRotation<R> rot)
{
  using C = typename Cplx<R>::type;
  const long long n = volume * 9;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < n; w += (long long)gridDim.x * blockDim.x) {
    const long long site = w / 9;
    const int cd = (int)(w - site * 9);
    C *p = prop + site * 144 + cd;  // entry (s, k, c, d) at p[(4 s + k) * 9]
    R m[4][4][2];
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const C v = p[(4 * s + k) * 9];
        m[s][k][0] = v.x;
        m[s][k][1] = v.y;
      }
    R a[4][4][2];  // U M
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        R re = R(0), im = R(0);
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (rot.nz[s][t]) cmac(re, im, rot.u[s][t][0], rot.u[s][t][1], m[t][k][0], m[t][k][1]);
        a[s][k][0] = re;
        a[s][k][1] = im;
      }
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        R re = R(0), im = R(0);
#pragma unroll
        for (int t = 0; t < 4; ++t)  // (U M U^dagger)[s][k] = sum_t (U M)[s][t] conj(U[k][t])
          if (rot.nz[k][t]) cmac(re, im, a[s][t][0], a[s][t][1], rot.u[k][t][0], -rot.u[k][t][1]);
        C v;
        v.x = re;
        v.y = im;
        p[(4 * s + k) * 9] = v;
      }
  }
}

} // namespace

cudaError_t launch_quda_layout(const Job &job, void *prop, void *const *fields, long long stride, bool from_quda,
                               int entry_bytes)
{
  if (job.volume == 0) return cudaSuccess;
  QudaFields f {};
  for (int k = 0; k < 12; ++k) f.f[k] = static_cast<char *>(fields[k]);
  const long long half = job.volume / 2;
  const long long tiles = 2 * ((half + 15) / 16);
  const int grid = (int)std::min<long long>(tiles, (long long)job.num_sms * 6);
  char *p = static_cast<char *>(prop);
  if (entry_bytes == 16) {
    constexpr int smem = QudaShape<16>::SMEM;
    if (from_quda) quda_layout_kernel<16, true><<<grid, 256, smem, job.stream>>>(p, f, half, stride);
    else quda_layout_kernel<16, false><<<grid, 256, smem, job.stream>>>(p, f, half, stride);
  } else {
    constexpr int smem = QudaShape<8>::SMEM;
    if (from_quda) quda_layout_kernel<8, true><<<grid, 256, smem, job.stream>>>(p, f, half, stride);
    else quda_layout_kernel<8, false><<<grid, 256, smem, job.stream>>>(p, f, half, stride);
  }
  return cudaGetLastError();
}

cudaError_t launch_spin_rotation(const Job &job, void *prop, const double *u)
{
  if (job.volume == 0) return cudaSuccess;
  const long long n = job.volume * 9;
  const int grid = (int)std::min<long long>((n + 255) / 256, (long long)job.num_sms * 8);
  if (job.prec == Prec::C128) {
    SpinRotation<double> r {};
    for (int s = 0; s < 4; ++s)
      for (int t = 0; t < 4; ++t) {
        r.u[s][t][0] = u[(s * 4 + t) * 2];
        r.u[s][t][1] = u[(s * 4 + t) * 2 + 1];
        r.nz[s][t] = r.u[s][t][0] != 0.0 || r.u[s][t][1] != 0.0;
      }
    spin_rotation_kernel<double><<<grid, 256, 0, job.stream>>>(static_cast<double2 *>(prop), job.volume, r);
  } else {
    SpinRotation<float> r {};
    for (int s = 0; s < 4; ++s)
      for (int t = 0; t < 4; ++t) {
        r.u[s][t][0] = (float)u[(s * 4 + t) * 2];
        r.u[s][t][1] = (float)u[(s * 4 + t) * 2 + 1];
        r.nz[s][t] = r.u[s][t][0] != 0.0f || r.u[s][t][1] != 0.0f;
      }
    spin_rotation_kernel<float><<<grid, 256, 0, job.stream>>>(static_cast<float2 *>(prop), job.volume, r);
  }
  return cudaGetLastError();
}

} // namespace cgb
