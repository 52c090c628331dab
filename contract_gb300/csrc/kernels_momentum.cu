// Meson all-gamma (16 x 16) correlators projected to momenta.
//
//   out[p][t][a][b] = sum_{x in t} exp(+2 pi i (nx x/Lx + ny y/Ly + nz z/Lz)) C_ab(x)
//
// The phase factorises over x, y and z, so instead of one dense
// [momenta x V3] x [V3 x 256] product per timeslice (8 M N K flop) the
// projection runs as three short transforms:
//   1. MesonAllGammaOp (tile engine): C_ab(x) for all 256 pairs, written in
//      lexicographic site order (HBM-bound: two propagators in, 256 complex out)
//   2. plane_kernel: per (t, z) plane, X then Y transform of every C_ab into
//      H[(nx, ny)][ab], in the form's arithmetic (FP64 planes for complex128,
//      FP32 planes for the mixed form)
//   3. momentum_finalize: Z transform and the sum over planes, returned in FP64.
// The mixed form normally fuses 1 and 2 (kernels_momentum_fused.cu), so the
// per-site values never reach HBM.
// For 32^3 x 64 and 125 momenta that is ~25 GFLOP instead of 537 GFLOP.
// Phase tables exp(2 pi i k / L) are computed in FP64 on the host from the
// exact integer index k = (n * x) mod L.
#include <algorithm>
#include <cstdlib>

#include "launch_variants.cuh"
#include "momentum.hpp"

namespace cgb {

template <class R> struct Vec2 { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

using MesonAllGammaP = MesonAllGammaOp<double, double2, 4, 3>;
using MesonAllGammaM = MesonAllGammaOp<float, float2, 8, 2>;
// field of the tensor-core path: the spin-colour products, pair halves apart
using MesonProductsSplitM = MesonAllGammaOp<float, float2, 8, 2, true, true>;

// One CTA per (z, t, chunk of (nx, ny) pairs); one thread per gamma pair.
// X transform: NG groups of +nx / -nx (C = sum cos * v, S = sum sin * v; the
// group count is a template argument so that no predicated-off FMA is
// issued).  Each thread's X values G[nx] go through its own column of shared
// memory, so the Y step reads G[q_ix[q]] with one load; the Y step runs over
// QC (>= the chunk's pair count) pairs.
template <class R> constexpr size_t plane_smem_bytes() { return (size_t)kMomMaxPx * 256 * 2 * sizeof(R); }

template <class R, class S, int NG, int QC>
__global__ void __launch_bounds__(256) plane_kernel(const S *__restrict__ c, typename Vec2<R>::type *__restrict__ planes,
                                                    const __grid_constant__ MomPlan plan)
{
  const int z = blockIdx.x, t = blockIdx.y, q0 = blockIdx.z * kMomQChunk, g = threadIdx.x;
  const int lx = plan.latt[0], ly = plan.latt[1], lz = plan.latt[2];
  const int nq = min(kMomQChunk, plan.nq - q0);
  __shared__ R phx[NG][kMomMaxL][2];
  __shared__ R phy[QC][kMomMaxL][2];
  extern __shared__ __align__(16) unsigned char plane_dyn[];
  cx<R> *gxs = reinterpret_cast<cx<R> *>(plane_dyn);  // [kMomMaxPx][256]
  __shared__ int qix[QC];
  if (g < QC) qix[g] = g < nq ? plan.q_ix[q0 + g] : 0;
  for (int e = g; e < NG * kMomMaxL; e += blockDim.x) {  // per X group: cos, sin of 2 pi k x / Lx
    const int gi = e / kMomMaxL, x = e % kMomMaxL;
    if (x < lx) {
      const int k = (plan.gx_k[gi] * x) % lx;
      phx[gi][x][0] = R(plan.cosx[k]);
      phx[gi][x][1] = R(plan.sinx[k]);
    }
  }
  for (int e = g; e < QC * kMomMaxL; e += blockDim.x) {
    const int q = e / kMomMaxL, y = e % kMomMaxL;
    if (y < ly) {
      const int k = q < nq ? ((plan.q_ny[q0 + q] * y) % ly + ly) % ly : 0;
      phy[q][y][0] = q < nq ? R(plan.cosy[k]) : R(0);
      phy[q][y][1] = q < nq ? R(plan.siny[k]) : R(0);
    }
  }
  __syncthreads();
  cx<R> h[QC];
#pragma unroll
  for (int q = 0; q < QC; ++q) h[q] = czero<R>();
  const S *row = c + ((size_t)(t * lz + z) * ly * lx) * 256 + g;
  constexpr int XB = 8;  // loads in flight per thread
  for (int y = 0; y < ly; ++y) {
    cx<R> gc[NG], gs[NG];
#pragma unroll
    for (int gi = 0; gi < NG; ++gi) gc[gi] = gs[gi] = czero<R>();
    const S *rowy = row + (size_t)y * lx * 256;
    for (int x0 = 0; x0 < lx; x0 += XB) {
      cx<R> v[XB];
#pragma unroll
      for (int u = 0; u < XB; ++u) v[u] = (x0 + u < lx) ? ld<R>(rowy + (size_t)(x0 + u) * 256) : czero<R>();
#pragma unroll
      for (int u = 0; u < XB; ++u) {
        if (x0 + u >= lx) break;
#pragma unroll
        for (int gi = 0; gi < NG; ++gi) {
          const R cs = phx[gi][x0 + u][0], sn = phx[gi][x0 + u][1];
          gc[gi].x = fma(cs, v[u].x, gc[gi].x);
          gc[gi].y = fma(cs, v[u].y, gc[gi].y);
          gs[gi].x = fma(sn, v[u].x, gs[gi].x);
          gs[gi].y = fma(sn, v[u].y, gs[gi].y);
        }
      }
    }
    // G(+k) = C + iS, G(-k) = C - iS
#pragma unroll
    for (int gi = 0; gi < NG; ++gi) {
      if (plan.gx_plus[gi] >= 0) gxs[plan.gx_plus[gi] * 256 + g] = {gc[gi].x - gs[gi].y, gc[gi].y + gs[gi].x};
      if (plan.gx_minus[gi] >= 0) gxs[plan.gx_minus[gi] * 256 + g] = {gc[gi].x + gs[gi].y, gc[gi].y - gs[gi].x};
    }
#pragma unroll
    for (int q = 0; q < QC; ++q) cfma(h[q], cx<R> {phy[q][y][0], phy[q][y][1]}, gxs[qix[q] * 256 + g]);
  }
#pragma unroll
  for (int q = 0; q < QC; ++q)
    if (q < nq)
      planes[((size_t)(t * lz + z) * plan.nq + q0 + q) * 256 + g] = {h[q].x, h[q].y};
}

template <int NG> cudaError_t set_plane_smem_attr_ng()
{
  const int b = (int)plane_smem_bytes<double>();
  cudaError_t e = cudaFuncSetAttribute(plane_kernel<double, double2, NG, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(plane_kernel<double, double2, NG, 9>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(plane_kernel<double, double2, NG, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(plane_kernel<double, double2, NG, kMomQChunk>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  return e;
}

inline cudaError_t set_plane_smem_attr()
{
  cudaError_t e = set_plane_smem_attr_ng<1>();
  if (e == cudaSuccess) e = set_plane_smem_attr_ng<2>();
  if (e == cudaSuccess) e = set_plane_smem_attr_ng<3>();
  if (e == cudaSuccess) e = set_plane_smem_attr_ng<4>();
  if (e == cudaSuccess) e = set_plane_smem_attr_ng<5>();
  if (e == cudaSuccess) e = set_plane_smem_attr_ng<6>();
  if (e == cudaSuccess) e = set_plane_smem_attr_ng<7>();
  if (e == cudaSuccess) e = set_plane_smem_attr_ng<8>();
  return e;
}

template <class R, class S, int NG>
cudaError_t launch_plane_qc(const Job &job, const S *field, typename Vec2<R>::type *planes, const MomPlan &plan,
                            dim3 grid)
{
  const int qc = plan.nq < kMomQChunk ? plan.nq : kMomQChunk;
  const size_t smem = plane_smem_bytes<R>();
  if (qc <= 4) plane_kernel<R, S, NG, 4><<<grid, 256, smem, job.stream>>>(field, planes, plan);
  else if (qc <= 9) plane_kernel<R, S, NG, 9><<<grid, 256, smem, job.stream>>>(field, planes, plan);
  else if (qc <= 16) plane_kernel<R, S, NG, 16><<<grid, 256, smem, job.stream>>>(field, planes, plan);
  else plane_kernel<R, S, NG, kMomQChunk><<<grid, 256, smem, job.stream>>>(field, planes, plan);
  return cudaGetLastError();
}

template <class R, class S>
cudaError_t launch_plane(const Job &job, const S *field, typename Vec2<R>::type *planes, const MomPlan &plan,
                         dim3 grid)
{
  switch (plan.ngx) {
  case 1: return launch_plane_qc<R, S, 1>(job, field, planes, plan, grid);
  case 2: return launch_plane_qc<R, S, 2>(job, field, planes, plan, grid);
  case 3: return launch_plane_qc<R, S, 3>(job, field, planes, plan, grid);
  case 4: return launch_plane_qc<R, S, 4>(job, field, planes, plan, grid);
  case 5: return launch_plane_qc<R, S, 5>(job, field, planes, plan, grid);
  case 6: return launch_plane_qc<R, S, 6>(job, field, planes, plan, grid);
  case 7: return launch_plane_qc<R, S, 7>(job, field, planes, plan, grid);
  case 8: return launch_plane_qc<R, S, 8>(job, field, planes, plan, grid);
  default: return cudaErrorInvalidValue;
  }
}

// out[p][t][g] = sum_z exp(2 pi i nz z / Lz) planes[t][z][q(p)][g].
// One CTA per ((nx, ny) pair q, t).  Each plane value is read once per pass
// and feeds up to CNT Z groups of the pair; a group of +n and -n accumulates
// C = sum cos * v and S = sum sin * v once for both momenta.
//   R = double (complex128 planes): FP64 phases and FMAs.
//   R = float (complex64 planes, whose values are FP32 sums): FP32 phases and
//     products, summed with a compensated (two-sum) accumulator and returned
//     in FP64, so the sum over z adds no rounding beyond the products'.  The
//     FP64 pipe (1/64 of the FP32 rate on this part) would otherwise bound
//     the kernel.
__device__ __forceinline__ void zacc(ChunkSum<double> &a, double c, double2 v)
{
  a.x = fma(c, v.x, a.x);
  a.y = fma(c, v.y, a.y);
}
__device__ __forceinline__ void zacc(ChunkSum<float> &a, float c, float2 v) { a.add(cx<float> {c * v.x, c * v.y}); }

//   TMAP (planes of the fused kernel, which projects the spin-colour products
//     T[i][j][k][l] instead of the Gamma pairs): each momentum's 256 sums go
//     through shared memory as unevaluated FP32 sums hi + lo (the compensated
//     accumulator's two words) and become the Gamma pairs (map_pairs) with
//     compensated sums again.  A Gamma pair is a signed sum of 16 products
//     that can cancel to well below the products themselves (at zero momentum
//     with one field in both slots the diagonal products are sums of positive
//     values); rounding each product to FP32 before that sum would leave an
//     error of the products' size.
__constant__ GammaTables kMomGamma = build_gamma_tables();

// Gamma pair (A, B) from the 256 projected products:
//   sum_{j,k} i^(ph_A(j) + ph_B(k)) T[perm_A(j)][j][k][perm_B(k)],
// ph_n(r) the phase of (g5 Gamma(n)) at (perm_n(r), r).  The phase factorises,
// so the map runs in two stages of four terms each instead of one of sixteen:
//   stage 1, thread 16 (4 i + j) + B:  U[i][j][B] = sum_k i^ph_B(k) T[i][j][k][perm_B(k)]
//   stage 2, thread 16 A + B:          pair(A, B) = sum_j i^ph_A(j) U[perm_A(j)][j][B]
// Products are staged at index p + p / 16 (rows of 16 padded by one against
// bank conflicts), U at 16 (4 i + j) + B; high and low words in separate arrays.
template <int NS> struct PairSmem {  // NS momenta mapped at a time
  float2 th[NS][272], tl[NS][272];
  float2 uh[NS][256], ul[NS][256];
  uint8_t perm[16][4], ph[16][4];
  __device__ __forceinline__ void load_tables(int g)
  {
    if (g < 64) {
      perm[g >> 2][g & 3] = kMomGamma.perm[g >> 2][g & 3];
      ph[g >> 2][g & 3] = kMomGamma.ph_g5g_t[g >> 2][g & 3];
    }
  }
};
struct PairMap {
  int s1[4], s2[4];  // each stage's source indices
  uint32_t ph;       // 2-bit phases: stage 1 in bits 0-7, stage 2 in bits 8-15
};
template <int NS> __device__ __forceinline__ PairMap pair_map(const PairSmem<NS> &s, int g)
{
  PairMap m;
  m.ph = 0u;
  const int i = g >> 6, j = (g >> 4) & 3, A = g >> 4, B = g & 15;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int lb = s.perm[B][r], ia = s.perm[A][r];
    m.s1[r] = (r * 4 + lb) * 17 + (i ^ j) * 4 + i;
    m.s2[r] = (ia * 4 + r) * 16 + B;
    m.ph |= ((uint32_t)s.ph[B][lb] & 3u) << (2 * r);
    m.ph |= ((uint32_t)s.ph[A][ia] & 3u) << (8 + 2 * r);
  }
  return m;
}
// One term hi + lo times i^ph (exact: a swap and sign flips); the high words
// meet in a two-sum, the low words in a plain FP32 sum (they are of the order
// of the high words' rounding).
__device__ __forceinline__ void add_term(ChunkSum<float> &o, float2 h, float2 l, uint32_t ph)
{
  const cx<float> lp = mul_phase(cx<float> {l.x, l.y}, ph);
  o.lx += lp.x;
  o.ly += lp.y;
  o.add(mul_phase(cx<float> {h.x, h.y}, ph));
}
// The Gamma pairs of the NS staged momenta, thread g's pair (A, B) = (g / 16,
// g % 16) of each.  Call after a barrier that follows the staging; contains
// one barrier (between the stages).
template <int NS>
__device__ __forceinline__ void map_pairs(PairSmem<NS> &s, const PairMap &m, int g, double2 (&out)[NS])
{
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    ChunkSum<float> u;
#pragma unroll
    for (int r = 0; r < 4; ++r) add_term(u, s.th[n][m.s1[r]], s.tl[n][m.s1[r]], (m.ph >> (2 * r)) & 3u);
    s.uh[n][g] = make_float2(u.hx, u.hy);
    s.ul[n][g] = make_float2(u.lx, u.ly);
  }
  __syncthreads();
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    ChunkSum<float> o;
#pragma unroll
    for (int r = 0; r < 4; ++r) add_term(o, s.uh[n][m.s2[r]], s.ul[n][m.s2[r]], (m.ph >> (8 + 2 * r)) & 3u);
    out[n] = o.value();
  }
}

// Stage the projected products of one Z group for momenta +n (n = 0) and -n
// (n = 1) from the compensated cosine and sine sums: G(+-n) = C +- i S, the
// high words joined by a two-sum.
__device__ __forceinline__ void stage_products(const ChunkSum<float> &c, const ChunkSum<float> &s, int g,
                                               PairSmem<2> &ps)
{
  const int slot = g + (g >> 4);
#pragma unroll
  for (int n = 0; n < 2; ++n) {
    // +n: (C.re - S.im, C.im + S.re); -n: (C.re + S.im, C.im - S.re)
    const float fx = n ? 1.f : -1.f, fy = -fx;
    float hx = c.hx, lx = c.lx + fx * s.ly, hy = c.hy, ly = c.ly + fy * s.lx;
    ChunkSum<float>::two_sum(hx, lx, fx * s.hy);
    ChunkSum<float>::two_sum(hy, ly, fy * s.hx);
    ps.th[n][slot] = make_float2(hx, hy);
    ps.tl[n][slot] = make_float2(lx, ly);
  }
}

// In place over rows of 256 (one (momentum, timeslice) each): projected
// products -> Gamma pairs.  Used after the tensor-core projection of products,
// whose FP64 sums are split into FP32 words hi + lo for the staging.
__global__ void __launch_bounds__(256) pair_map_kernel(double2 *__restrict__ rows, long long nrows)
{
  const int g = threadIdx.x;
  __shared__ PairSmem<1> ps;
  ps.load_tables(g);
  __syncthreads();
  const PairMap m = pair_map(ps, g);
  for (long long r = blockIdx.x; r < nrows; r += gridDim.x) {
    const double2 v = rows[r * 256 + g];
    __syncthreads();  // the previous row's reads of the staging are done
    const float hx = float(v.x), hy = float(v.y);
    ps.th[0][g + (g >> 4)] = make_float2(hx, hy);
    ps.tl[0][g + (g >> 4)] = make_float2(float(v.x - hx), float(v.y - hy));
    __syncthreads();
    double2 o[1];
    map_pairs<1>(ps, m, g, o);
    rows[r * 256 + g] = o[0];
  }
}

template <class R, int CNT, bool TMAP>
__global__ void __launch_bounds__(256) momentum_finalize(const typename Vec2<R>::type *__restrict__ planes,
                                                          double2 *__restrict__ out, const __grid_constant__ MomPlan plan)
{
  const int q = blockIdx.x, t = blockIdx.y, g = threadIdx.x;
  const int lz = plan.latt[2], lt = plan.latt[3];
  __shared__ R cz[kMomMaxL], sz[kMomMaxL];
  __shared__ PairSmem<2> ps;  // TMAP: the pair map of one Z group (+n and -n)
  if (TMAP) ps.load_tables(g);
  for (int k = g; k < lz; k += blockDim.x) {
    cz[k] = R(plan.cosz[k]);
    sz[k] = R(plan.sinz[k]);
  }
  __syncthreads();
  const int g0 = plan.q_g0[q], g1 = plan.q_g0[q + 1];
  for (int base = g0; base < g1; base += CNT) {
    const int cnt = min(CNT, g1 - base);
    ChunkSum<R> ca[CNT], sa[CNT];
    int kk[CNT], step[CNT];
#pragma unroll
    for (int k = 0; k < CNT; ++k) {
      kk[k] = 0;
      step[k] = k < cnt ? plan.gz_k[base + k] : 0;
    }
    using V2 = typename Vec2<R>::type;
    constexpr int ZB = 4;  // plane loads in flight per thread
    for (int z0 = 0; z0 < lz; z0 += ZB) {
      V2 v[ZB];
#pragma unroll
      for (int u = 0; u < ZB; ++u)
        if (z0 + u < lz) v[u] = planes[((size_t)(t * lz + z0 + u) * plan.nq + q) * 256 + g];
#pragma unroll
      for (int u = 0; u < ZB; ++u) {
        if (z0 + u >= lz) break;
#pragma unroll
        for (int k = 0; k < CNT; ++k) {
          if (k < cnt) {
            zacc(ca[k], cz[kk[k]], v[u]);
            zacc(sa[k], sz[kk[k]], v[u]);
            if ((kk[k] += step[k]) >= lz) kk[k] -= lz;  // k * z mod Lz
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < CNT; ++k) {
      if (k >= cnt) break;  // block-uniform
      if constexpr (TMAP) {
        __syncthreads();  // the previous group's reads of the staging are done
        stage_products(ca[k], sa[k], g, ps);
        __syncthreads();
        double2 o[2];
        map_pairs<2>(ps, pair_map(ps, g), g, o);
#pragma unroll
        for (int sg = 0; sg < 2; ++sg) {
          const int pm = sg ? plan.gz_minus[base + k] : plan.gz_plus[base + k];
          if (pm >= 0) out[((size_t)pm * lt + t) * 256 + g] = o[sg];
        }
      } else {
        const double2 c = ca[k].value(), sn = sa[k].value();
        const int pp = plan.gz_plus[base + k], pn = plan.gz_minus[base + k];
        if (pp >= 0) out[((size_t)pp * lt + t) * 256 + g] = make_double2(c.x - sn.y, c.y + sn.x);
        if (pn >= 0) out[((size_t)pn * lt + t) * 256 + g] = make_double2(c.x + sn.y, c.y - sn.x);
      }
    }
  }
}

template <class R, bool TMAP>
cudaError_t launch_finalize(const Job &job, const typename Vec2<R>::type *planes, double2 *out, const MomPlan &plan)
{
  int most = 1;  // Z groups of the pair with the most
  for (int q = 0; q < plan.nq; ++q) most = std::max(most, plan.q_g0[q + 1] - plan.q_g0[q]);
  const dim3 grid(plan.nq, plan.latt[3]);
  if (most <= 1) momentum_finalize<R, 1, TMAP><<<grid, 256, 0, job.stream>>>(planes, out, plan);
  else if (most <= 2) momentum_finalize<R, 2, TMAP><<<grid, 256, 0, job.stream>>>(planes, out, plan);
  else if (most <= 3) momentum_finalize<R, 3, TMAP><<<grid, 256, 0, job.stream>>>(planes, out, plan);
  else if (most <= 4) momentum_finalize<R, 4, TMAP><<<grid, 256, 0, job.stream>>>(planes, out, plan);
  else momentum_finalize<R, 8, TMAP><<<grid, 256, 0, job.stream>>>(planes, out, plan);
  return cudaGetLastError();
}

// ------------------------------------------------ batched finalisation --
// One launch for what the batched site kernels leave: blocks [0, bf.total_blocks)
// sum the baryon items' partials per (output, timeslice) in the order of
// batch_finalize_kernel (kernels_batch.cu), 256 values a block; the blocks
// after them take one (item, pair q, timeslice) each and do what
// momentum_finalize<float, CNT, true> does for one call: the Z transform of
// the item's planes with a compensated FP32 sum, then the product -> Gamma
// pair map, FP64 out.  Phase tables come from the batch's per-extent tables
// (the same FP32 values as the per-call path).
template <int CNT>
__global__ void __launch_bounds__(256) batch_finalize_combined(const __grid_constant__ MomBatchParams mp,
                                                                const __grid_constant__ BaryonFinParams bf)
{
  const int g = threadIdx.x;
  if ((int)blockIdx.x < bf.total_blocks) {
    int lo = 0, hi = bf.n_items - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (bf.items[mid].blk_begin <= (int)blockIdx.x) lo = mid;
      else hi = mid - 1;
    }
    const BaryonFinItem &it = bf.items[lo];
    const int idx = ((int)blockIdx.x - it.blk_begin) * 256 + g;
    if (idx >= bf.nout * it.lt || it.per_seg <= 0) return;
    const int o = idx / it.lt, t = idx % it.lt;
    double sx = 0.0, sy = 0.0;
    for (int par = 0; par < 2; ++par) {
      const double2 *row = it.partial + ((size_t)(par * it.lt + t) * it.per_seg) * bf.nout + o;
      for (int c = 0; c < it.per_seg; ++c) {
        const double2 v = row[(size_t)c * bf.nout];
        sx += v.x;
        sy += v.y;
      }
    }
    it.out[(size_t)o * it.lt + t] = make_double2(sx, sy);
    return;
  }
  const int b = (int)blockIdx.x - bf.total_blocks;
  int lo = 0, hi = mp.n_items - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mp.items[mid].fin_begin <= b) lo = mid;
    else hi = mid - 1;
  }
  const MomBatchItem &it = mp.items[lo];
  const int lz = it.latt[2], lt = it.latt[3];
  const int local = b - it.fin_begin, q = local / lt, t = local - q * lt;
  if (q >= mp.nq) return;  // block-uniform
  __shared__ float cz[kMomMaxL], sz[kMomMaxL];
  __shared__ PairSmem<2> ps;
  ps.load_tables(g);
  for (int k = g; k < lz; k += blockDim.x) {
    cz[k] = mp.tab[it.tz][k].x;
    sz[k] = mp.tab[it.tz][k].y;
  }
  __syncthreads();
  const PairMap pm_terms = pair_map(ps, g);
  const int g0 = mp.q_g0[q], g1 = mp.q_g0[q + 1];
  for (int base = g0; base < g1; base += CNT) {
    const int cnt = min(CNT, g1 - base);
    ChunkSum<float> ca[CNT], sa[CNT];
    int kk[CNT], step[CNT];
#pragma unroll
    for (int k = 0; k < CNT; ++k) {
      kk[k] = 0;
      step[k] = k < cnt ? mp.gz_k[base + k] : 0;
    }
    constexpr int ZB = 4;  // plane loads in flight per thread
    for (int z0 = 0; z0 < lz; z0 += ZB) {
      float2 v[ZB];
#pragma unroll
      for (int u = 0; u < ZB; ++u)
        if (z0 + u < lz) v[u] = it.planes[((size_t)(t * lz + z0 + u) * mp.nq + q) * 256 + g];
#pragma unroll
      for (int u = 0; u < ZB; ++u) {
        if (z0 + u >= lz) break;
#pragma unroll
        for (int k = 0; k < CNT; ++k) {
          if (k < cnt) {
            zacc(ca[k], cz[kk[k]], v[u]);
            zacc(sa[k], sz[kk[k]], v[u]);
            if ((kk[k] += step[k]) >= lz) kk[k] -= lz;
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < CNT; ++k) {
      if (k >= cnt) break;  // block-uniform
      __syncthreads();  // the previous group's reads of the staging are done
      stage_products(ca[k], sa[k], g, ps);
      __syncthreads();
      double2 o[2];
      map_pairs<2>(ps, pm_terms, g, o);
#pragma unroll
      for (int sg = 0; sg < 2; ++sg) {
        const int pm = sg ? mp.gz_minus[base + k] : mp.gz_plus[base + k];
        if (pm >= 0) it.out[((size_t)pm * lt + t) * 256 + g] = o[sg];
      }
    }
  }
}

cudaError_t launch_batch_finalize(const Job &job, const MomBatchParams &mp, const BaryonFinParams &bf)
{
  const long long blocks = (long long)bf.total_blocks + (mp.n_items > 0 ? mp.total_fin : 0);
  if (blocks <= 0) return cudaSuccess;
  int most = 1;  // Z groups of the pair with the most
  for (int q = 0; q < mp.nq; ++q) most = std::max(most, mp.q_g0[q + 1] - mp.q_g0[q]);
  const unsigned grid = (unsigned)blocks;
  if (mp.n_items == 0 || most <= 1) batch_finalize_combined<1><<<grid, 256, 0, job.stream>>>(mp, bf);
  else if (most <= 2) batch_finalize_combined<2><<<grid, 256, 0, job.stream>>>(mp, bf);
  else if (most <= 3) batch_finalize_combined<3><<<grid, 256, 0, job.stream>>>(mp, bf);
  else if (most <= 4) batch_finalize_combined<4><<<grid, 256, 0, job.stream>>>(mp, bf);
  else batch_finalize_combined<8><<<grid, 256, 0, job.stream>>>(mp, bf);
  return cudaGetLastError();
}

// CONTRACT_MOMENTUM_UNFUSED=1 selects the three-kernel mixed form (site
// values through HBM), for comparison.
static bool fused_disabled()
{
  static const bool off = [] {
    const char *v = getenv("CONTRACT_MOMENTUM_UNFUSED");
    return v && v[0] == '1';
  }();
  return off;
}

static const char *const kMomFusedNames[] = {"fused.site8.xy8", "three-kernel", "fused.site16.xy8"};
static const char *const kMomTcNames[] = {"tc.unit128", "tc.unit64", "tc.unit192"};
static const int kMomTcSteps[] = {128, 64, 192};

int momentum_variants(Prec prec, int aux, const char *const **names)
{
  if ((aux & 2) && prec == Prec::C64) {
    *names = kMomTcNames;
    return 3;
  }
  if ((aux & 1) && prec == Prec::C64) {
    *names = kMomFusedNames;
    return 3;
  }
  return 1;
}

cudaError_t launch_meson_momentum(const Job &job, const OpParams<double> &p, const MomPlan &plan, void *out,
                                  bool tensor_cores)
{
  if (job.volume == 0) return cudaSuccess;
  if (tensor_cores && job.prec != Prec::C64) return cudaErrorInvalidValue;
  // job.variant (autotuner): complex64 -- 1 runs the three-kernel form, 2 the
  // fused kernel with 16 site warps, 0 with 8; tensor cores -- the k-steps per
  // work unit.  With no variant chosen, two fields take 16 site warps and one
  // field passed twice 8 (the tuner's choices at 32^3 x 64).
  const bool fused = !tensor_cores && job.prec == Prec::C64 && momentum_fused_supported(plan) && !fused_disabled() &&
                     job.variant != 1;
  const size_t elem = job.prec == Prec::C128 ? sizeof(double2) : sizeof(float2);
  const size_t c_bytes = fused ? 0 : ((size_t)job.volume * 256 * elem + 255) / 256 * 256;
  const int lz = plan.latt[2], lt = plan.latt[3];
  const int tcv = tensor_cores && job.variant >= 0 && job.variant < 3 ? job.variant : 0;
  const TcGeom tg = make_tc_geom(plan, kMomTcSteps[tcv]);
  const size_t a_bytes = (tc_phase_bytes(tg) + 255) / 256 * 256;
  const size_t tile_bytes = job.tc_tiles ? 0 : a_bytes;  // phase tiles kept by the caller, or in the workspace
  const size_t plane_bytes = tensor_cores ? tile_bytes + tc_partial_bytes(tg)
                                          : (size_t)lt * lz * plan.nq * 256 * 2 * (job.prec == Prec::C128 ? 8 : 4);
  char *ws = static_cast<char *>(job.ws->get(c_bytes + plane_bytes));
  if (!ws) return cudaErrorMemoryAllocation;
  double2 *planes = reinterpret_cast<double2 *>(ws + c_bytes);  // complex128 form
  float2 *planes_m = reinterpret_cast<float2 *>(ws + c_bytes);   // mixed form

  if (fused) {
    const bool sw16 = job.variant == 2 || (job.variant < 0 && p.in[0] != p.in[1]);
    cudaError_t e = launch_momentum_fused(job, p.in[0], p.in[1], planes_m, plan, sw16 ? 16 : 8);
    if (e != cudaSuccess) return e;
    return launch_finalize<float, true>(job, planes_m, static_cast<double2 *>(out), plan);
  }

  OpParams<double> q = p;
  q.out[0] = ws;
  for (int k = 0; k < 4; ++k) q.latt[k] = plan.latt[k];
  cudaError_t e;
  if (job.prec == Prec::C128) e = run_field<MesonAllGammaP>(job, q);
  else if (tensor_cores) e = run_field<MesonProductsSplitM>(job, convert_params<float>(q));
  else e = run_field<MesonAllGammaM>(job, convert_params<float>(q));
  if (e != cudaSuccess) return e;
  if (tensor_cores) {
    unsigned char *tiles = job.tc_tiles ? static_cast<unsigned char *>(job.tc_tiles)
                                        : reinterpret_cast<unsigned char *>(ws + c_bytes);
    e = launch_momentum_tc(job, plan, tg, ws, tiles, reinterpret_cast<float *>(ws + c_bytes + tile_bytes), out,
                           job.tc_tiles != nullptr && job.tc_tiles_ready);
    if (e != cudaSuccess) return e;
    const long long nrows = (long long)plan.np * lt;
    const int grid = (int)std::min<long long>(nrows, (long long)job.num_sms * 8);
    pair_map_kernel<<<grid, 256, 0, job.stream>>>(static_cast<double2 *>(out), nrows);
    return cudaGetLastError();
  }

  const dim3 grid(lz, lt, (plan.nq + kMomQChunk - 1) / kMomQChunk);
  if (job.prec == Prec::C128) {
    // the complex128 form needs more than the default 48 KB of shared memory
    static bool attr[64] = {};
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 64 || !attr[dev]) {
      e = set_plane_smem_attr();
      if (e != cudaSuccess) return e;
      if (dev < 64) attr[dev] = true;
    }
    e = launch_plane<double, double2>(job, reinterpret_cast<const double2 *>(ws), planes, plan, grid);
    if (e != cudaSuccess) return e;
    return launch_finalize<double, false>(job, planes, static_cast<double2 *>(out), plan);
  }
  e = launch_plane<float, float2>(job, reinterpret_cast<const float2 *>(ws), planes_m, plan, grid);
  if (e != cudaSuccess) return e;
  return launch_finalize<float, false>(job, planes_m, static_cast<double2 *>(out), plan);
}

} // namespace cgb
