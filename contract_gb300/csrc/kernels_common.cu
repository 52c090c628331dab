// Per-timeslice finalisation and precision conversion kernels.
#include "launch_impl.cuh"
#include "momentum.hpp"

namespace cgb {

__device__ DeviceStatus g_device_status;

cudaError_t device_status_ptr(DeviceStatus **out) { return cudaGetSymbolAddress((void **)out, g_device_status); }

// out.p[o][t] = sum_{parity, chunk} partial[((parity*lt + t)*chunks_per_seg + chunk)*nout + o]
// Segments are half-timeslices in PyQUDA order [parity][t][...].  One block of
// kFinThreads threads per (o, t), block index o * lt + t: thread k sums the
// partials k, k + kFinThreads, ... of the 2 * chunks_per_seg (parity-major) in
// FP64, then a fixed shuffle tree and one shared-memory step join the threads.
// The order is the same on every call, so results are bitwise reproducible.
// (One thread per (o, t) walking every partial in turn left the sum's latency
// chain on the critical path: 108 dependent loads per thread for a per-call
// triangle at 24^3 x 64.)
__global__ void __launch_bounds__(kFinThreads) finalize_kernel(const double2 *__restrict__ partial, OutPtrs out,
                                                               int nout, int lt, int chunks_per_seg)
{
  const int o = blockIdx.x / lt, t = blockIdx.x - o * lt;
  const int n = 2 * chunks_per_seg;
  double sx = 0.0, sy = 0.0;
  for (int k = threadIdx.x; k < n; k += kFinThreads) {
    const int par = k >= chunks_per_seg ? 1 : 0, c = k - par * chunks_per_seg;
    const double2 v = partial[((size_t)(par * lt + t) * chunks_per_seg + c) * nout + o];
    sx += v.x;
    sy += v.y;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    sx += __shfl_down_sync(0xffffffffu, sx, off);
    sy += __shfl_down_sync(0xffffffffu, sy, off);
  }
  __shared__ double2 wsum[kFinThreads / 32];
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = make_double2(sx, sy);
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 r = wsum[0];
#pragma unroll
    for (int w = 1; w < kFinThreads / 32; ++w) {
      r.x += wsum[w].x;
      r.y += wsum[w].y;
    }
    out.p[o][t] = r;
  }
}

// complex128 <-> complex64, one complex per thread step, grid-stride.
__global__ void c128_to_c64(float2 *__restrict__ dst, const double2 *__restrict__ src, long long n)
{
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const double2 v = src[k];
    dst[k] = make_float2((float)v.x, (float)v.y);
  }
}

__global__ void c64_to_c128(double2 *__restrict__ dst, const float2 *__restrict__ src, long long n)
{
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const float2 v = src[k];
    dst[k] = make_double2((double)v.x, (double)v.y);
  }
}

int meson_variants(Prec prec, const char *const **names);
int meson_all_variants(Prec prec, bool source, const char *const **names);
int baryon_variants(Prec prec, int form, const char *const **names);
int fused_variants(Prec prec, int nw, const char *const **names);
int field_variants(Prec prec, bool sequential, const char *const **names);

int launch_variants(Kind kind, Prec prec, int aux, const char *const **names)
{
  switch (kind) {
  case Kind::Meson: return meson_variants(prec, names);
  case Kind::BaryonLoop: return baryon_variants(prec, 0, names);
  case Kind::BaryonTri: return baryon_variants(prec, aux + 1, names);
  case Kind::BaryonFused: return fused_variants(prec, aux, names);
  case Kind::Diquark: return field_variants(prec, false, names);
  case Kind::Sequential: return field_variants(prec, true, names);
  case Kind::MesonAll: return meson_all_variants(prec, aux != 0, names);
  case Kind::Momentum: return momentum_variants(prec, aux, names);
  }
  return 1;
}

// Site reordering between lexicographic ((t*Lz + z)*Ly + y)*Lx + x and PyQUDA
// even/odd ((par*Lt + t)*Lz + z)*Ly + y)*(Lx/2) + x/2, par = (x+y+z+t) & 1.
// One thread per 16-byte piece of a site; a site's pieces are consecutive, so
// reads and writes are contiguous runs of a whole site.
__global__ void layout_kernel(uint4 *__restrict__ dst, const uint4 *__restrict__ src, long long volume,
                              int pieces, int lx, int ly, int lz, int lt, int to_eo)
{
  const long long n = volume * pieces;
  const int half = lx / 2;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long site = k / pieces;
    const int w = (int)(k - site * pieces);
    long long d;
    if (to_eo) {
      long long r = site;
      const int x = (int)(r % lx);
      r /= lx;
      const int y = (int)(r % ly);
      r /= ly;
      const int z = (int)(r % lz);
      const int t = (int)(r / lz);
      const int par = (x + y + z + t) & 1;
      d = ((((long long)par * lt + t) * lz + z) * ly + y) * half + x / 2;
    } else {
      long long r = site;
      const int xh = (int)(r % half);
      r /= half;
      const int y = (int)(r % ly);
      r /= ly;
      const int z = (int)(r % lz);
      r /= lz;
      const int t = (int)(r % lt);
      const int par = (int)(r / lt);
      const int x = 2 * xh + ((par + t + z + y) & 1);
      d = (((long long)t * lz + z) * ly + y) * lx + x;
    }
    dst[d * pieces + w] = src[k];
  }
}

cudaError_t launch_layout(const Job &job, void *dst, const void *src, const int *latt, bool to_eo, int site_bytes)
{
  if (job.volume == 0) return cudaSuccess;
  const int pieces = site_bytes / 16;
  layout_kernel<<<job.num_sms * 8, 256, 0, job.stream>>>(static_cast<uint4 *>(dst), static_cast<const uint4 *>(src),
                                                        job.volume, pieces, latt[0], latt[1], latt[2], latt[3],
                                                        to_eo ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_convert(const Job &job, void *dst, const void *src, bool to_c64)
{
  const long long n = job.volume * 144;
  if (n == 0) return cudaSuccess;
  const int grid = job.num_sms * 8;
  if (to_c64) c128_to_c64<<<grid, 256, 0, job.stream>>>(static_cast<float2 *>(dst), static_cast<const double2 *>(src), n);
  else c64_to_c128<<<grid, 256, 0, job.stream>>>(static_cast<double2 *>(dst), static_cast<const float2 *>(src), n);
  return cudaGetLastError();
}

} // namespace cgb
