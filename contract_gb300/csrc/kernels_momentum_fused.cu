// Fused all-gamma meson momentum projection, mixed form (complex64 storage,
// FP32 arithmetic): the per-site spin-colour products behind the 16 x 16 meson
// values and the X and Y transforms of the separable projection in one
// kernel, so the 256 complex values per site live only in shared memory.  The
// three-kernel form writes the meson values to HBM (2 KB per site) and reads
// them back; here HBM traffic is the two propagators (2 x 1152 B per site)
// plus one FP32 plane per (t, z).
//
// One persistent CTA per SM walks (t, z) planes.  A plane's sites are taken
// in row order -- for each y, both parities' half-rows -- in tiles of 16:
//
//   warps 0-7    site warps: each fetches its own two sites of a tile with
//                cp.async.bulk into a per-warp kFNst-stage ring (its own full
//                mbarriers, kFNst - 1 tiles ahead), forms their 256 spin-colour
//                products T (site_products) and leaves them in one of two
//                shared output buffers (ofull / oempty mbarriers)
//   warps 8-15   transform warps: thread g owns product g; for each site of
//                a row, C += cos(k x) v and S += sin(k x) v per X group; at
//                the end of a row G(nx) -> shared column, then
//                H[q] += exp(i ky y) G(nx(q)) for every (nx, ny) pair q
//
// Sixteen warps (no separate producer) leave 128 registers per thread.  At the
// end of a plane each transform thread writes H[q] (FP32) to the plane buffer;
// momentum_finalize applies the Z transform with a compensated sum, then the
// product -> Gamma-pair combination, and returns FP64.  Every mbarrier wait is
// bounded in wall time; a timed-out wait reports kDevErrWaitTimeout, raises
// the CTA's abort flag and returns.
#include "engine.cuh"
#include "momentum.hpp"

namespace cgb {

namespace {

// The 256 spin-colour products of a site,
//   T[i][j][k][l] = sum_c S1[i][k][c] conj(S2[j][l][c]),
// from which every Gamma pair is a signed sum of 16 (see momentum_finalize).
// That combination is linear and the same at every site, so it commutes with
// the projection: the kernel projects T, and the finalize applies it once per
// momentum and timeslice instead of once per site.  Thread sub = 4 s + i of a
// site computes the 16 products of (i, j = i ^ s) and stores T[k][l] at index
// (4 k + l) * 16 + sub, so a warp's stores and the transform's loads are
// consecutive.
__device__ __forceinline__ void site_products(const float2 *in0, const float2 *in1, int sub, float2 *dst)
{
  const int s = sub >> 2, i = sub & 3, j = i ^ s;
  cx<float> T[4][4];
  conj_products_f32x2<4>(T, in0 + i * 36, in1 + j * 36);
  if (!dst) return;
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int l = 0; l < 4; ++l) dst[(k * 4 + l) * 16 + sub] = make_float2(T[k][l].x, T[k][l].y);
}

// The same with a site split over 32 threads: thread sub = 8 s + 2 i + h
// computes the 8 products of (i, j = i ^ s) with k = 2 h, 2 h + 1.
__device__ __forceinline__ void site_products_half(const float2 *in0, const float2 *in1, int sub, float2 *dst)
{
  const int s = sub >> 3, i = (sub >> 1) & 3, h = sub & 1, j = i ^ s;
  cx<float> T[2][4];
  conj_products_f32x2<2>(T, in0 + i * 36 + h * 18, in1 + j * 36);
  if (!dst) return;
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int l = 0; l < 4; ++l) dst[((2 * h + k) * 4 + l) * 16 + s * 4 + i] = make_float2(T[k][l].x, T[k][l].y);
}

// P_i and P_j one field (S1 = S2 = S): T[j][i][l][k] = conj(T[i][j][k][l]),
// so 136 of the 256 products are independent.  Thread sub = 4 s + i
// (j = i ^ s) computes rows r0, r0 + 1 of the block T[X][Y], X = min(i, j),
// Y = max(i, j), and stores each product and its conjugate transpose: r0 = 0
// for the lower spin's thread and 2 for the higher one's.  For s = 0
// (X = Y = i) the block is Hermitian: rows 0 and 1 give its upper triangle
// (the lower entries of those rows are the conjugates of stored ones and are
// not stored), and the three entries left, T[i][i][2][2], [2][3] and [3][3],
// fall one each to the threads (s, i) with s = 1, 2, 3.  Every product is
// stored once; a thread forms at most 9 dots instead of 16.
__device__ __forceinline__ void same_field_extra(const float2 *in, int s, int i, float2 *dst)
{
  const int ea = s == 3 ? 3 : 2, eb = s == 1 ? 2 : 3;  // (2, 2), (2, 3), (3, 3) for s = 1, 2, 3
  cx<float> E[1][1];
  conj_products_f32x2<1, 1>(E, in + (i * 4 + ea) * 9, in + (i * 4 + eb) * 9);
  if (!dst) return;
  dst[(ea * 4 + eb) * 16 + i] = make_float2(E[0][0].x, E[0][0].y);
  if (ea != eb) dst[(eb * 4 + ea) * 16 + i] = make_float2(E[0][0].x, -E[0][0].y);
}

// Stores rows k0 .. k0 + NK - 1 of T[X][Y] (and their conjugate transposes in
// T[Y][X]) for the threads of class s, as described above.
template <int NK>
__device__ __forceinline__ void store_same_field(const cx<float> (&T)[NK][4], int s, int X, int Y, int k0,
                                                 float2 *dst)
{
#pragma unroll
  for (int r = 0; r < NK; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int k = k0 + r;
      if (s == 0 && c < k) continue;  // lower triangle of the Hermitian T[i][i]
      dst[(k * 4 + c) * 16 + 4 * s + X] = make_float2(T[r][c].x, T[r][c].y);
      if (s != 0 || c > k) dst[(c * 4 + k) * 16 + 4 * s + Y] = make_float2(T[r][c].x, -T[r][c].y);
    }
}

__device__ __forceinline__ void site_products_same(const float2 *in, int sub, float2 *dst)
{
  const int s = sub >> 2, i = sub & 3, j = i ^ s;
  const int X = min(i, j), Y = max(i, j), k0 = i > j ? 2 : 0;
  cx<float> T[2][4];
  conj_products_f32x2<2>(T, in + X * 36 + k0 * 9, in + Y * 36);
  if (s != 0) same_field_extra(in, s, i, dst);
  if (dst) store_same_field<2>(T, s, X, Y, k0, dst);
}

// The same over 32 threads: thread sub = 8 s + 2 i + h computes row k0 + h
// of T[X][Y]; the threads with h = 0 and s != 0 take the three entries left.
__device__ __forceinline__ void site_products_same_half(const float2 *in, int sub, float2 *dst)
{
  const int s = sub >> 3, i = (sub >> 1) & 3, h = sub & 1, j = i ^ s;
  const int X = min(i, j), Y = max(i, j), k0 = (i > j ? 2 : 0) + h;
  cx<float> T[1][4];
  conj_products_f32x2<1>(T, in + X * 36 + k0 * 9, in + Y * 36);
  if (s != 0 && h == 0) same_field_extra(in, s, i, dst);
  if (dst) store_same_field<1>(T, s, X, Y, k0, dst);
}

constexpr int kFTW = 8;     // transform warps (256 threads: one per product)
constexpr int kFMaxSW = 16;  // site warps: 8 (two sites a warp) or 16 (one site a warp)
constexpr int kFSites = 16;  // sites per tile
constexpr int kFNst = 3;     // input ring stages
using FL = SiteLayout<float2>;
constexpr size_t kFStage = 2ull * kFSites * FL::SLOT;
constexpr size_t kFOut = (size_t)kFSites * 256 * sizeof(float2);  // 32 KB per output buffer
// mbarriers: full[SW][kFNst], ofull[2], oempty[2] (and tsync in the batched kernel); abort flag at 504
constexpr size_t kFStagesOff = 512;
constexpr size_t kFOutOff = kFStagesOff + kFNst * kFStage;
constexpr size_t kFGxOff = kFOutOff + 2 * kFOut;
constexpr size_t kFSmem = kFGxOff + (size_t)kMomMaxPx * 256 * sizeof(float2);
static_assert((kFMaxSW * kFNst + 5) * 8 <= 504, "mbarrier block overlaps the abort flag");

// Register split of the 16-site-warp shape (setmaxnreg, per warpgroup): the
// launch gives 768 threads 80 registers each (61 440); site warps drop to 56
// and transform warps rise to 128: 16 x 32 x 56 + 8 x 32 x 128 = 61 440.
constexpr int kFLaunchRegs16 = 80, kFSiteRegs16 = 56, kFTransformRegs16 = 128;
static_assert(kFMaxSW * 32 * kFSiteRegs16 + kFTW * 32 * kFTransformRegs16 <= (kFMaxSW + kFTW) * 32 * kFLaunchRegs16,
              "register split exceeds the launch's registers");

template <int SW> struct FusedShape {
  static_assert(SW == 8 || SW == 16, "8 or 16 site warps");
  static constexpr int THREADS = 32 * (SW + kFTW);
  static constexpr int SPW = kFSites / SW;  // sites per site warp
  static constexpr int TPS = 32 / SPW;      // threads per site
};

struct FusedArgs {
  const char *in[2];  // complex64 propagators, PyQUDA even/odd order
  float2 *planes;     // [Lt][Lz][nq][256], FP32 sums
  DeviceStatus *status;
  int tiles_per_plane;
};

static_assert(sizeof(FusedArgs) + sizeof(MomPlan) <= 32764, "kernel parameters exceed 32764 bytes");
static_assert(kFSmem + sizeof(float) * 2 * kMomMaxL * (3 + kMomQChunk) + 4 * kMomQChunk <= 232448,
              "fused momentum kernel does not fit in shared memory");

// Site j (0 <= j < Lx Ly) of plane (t, z) in row order: y = j / Lx, then the
// parity-0 half-row, then the parity-1 half-row.  Returns its even/odd index.
__device__ __forceinline__ long long plane_site(const MomPlan &pl, int t, int z, int j)
{
  const int lx = pl.latt[0], ly = pl.latt[1], lz = pl.latt[2], lt = pl.latt[3], half = lx >> 1;
  const int y = j / lx, r = j - y * lx, par = r >= half ? 1 : 0, xh = r - par * half;
  return ((((long long)par * lt + t) * lz + z) * ly + y) * half + xh;
}

template <int SW, int NG, int QC, bool SAME>
__global__ void __launch_bounds__(FusedShape<SW>::THREADS, 1)
  momentum_fused_kernel(const __grid_constant__ FusedArgs a, const __grid_constant__ MomPlan plan)
{
  using Shape = FusedShape<SW>;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);  // [SW][kFNst]
  uint64_t *ofull = full + SW * kFNst;
  uint64_t *oempty = ofull + 2;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + 504);
  float2 *obuf = reinterpret_cast<float2 *>(smem + kFOutOff);  // [2][kFSites][256]
  __shared__ float phx[NG][kMomMaxL][2];
  __shared__ float phy[QC][kMomMaxL][2];
  __shared__ int qix[QC];

  const int lx = plan.latt[0], ly = plan.latt[1], lz = plan.latt[2], lt = plan.latt[3];
  const int units = lt * lz, tpp = a.tiles_per_plane, nsites = lx * ly;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < SW * kFNst; ++s) mbar_init(&full[s], 1);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&ofull[b], SW);
      mbar_init(&oempty[b], kFTW);
    }
    *abort_flag = 0;
    fence_barrier_init();
  }
  for (int q = threadIdx.x; q < QC; q += blockDim.x) qix[q] = q < plan.nq ? plan.q_ix[q] : 0;
  for (int e = threadIdx.x; e < NG * kMomMaxL; e += blockDim.x) {  // cos, sin of 2 pi k x / Lx per X group
    const int gi = e / kMomMaxL, x = e % kMomMaxL;
    const int k = x < lx ? (plan.gx_k[gi] * x) % lx : 0;
    phx[gi][x][0] = float(plan.cosx[k]);
    phx[gi][x][1] = float(plan.sinx[k]);
  }
  for (int e = threadIdx.x; e < QC * kMomMaxL; e += blockDim.x) {
    const int q = e / kMomMaxL, y = e % kMomMaxL;
    const bool on = q < plan.nq && y < ly;
    const int k = on ? ((plan.q_ny[q] * y) % ly + ly) % ly : 0;
    phy[q][y][0] = on ? float(plan.cosy[k]) : 0.f;
    phy[q][y][1] = on ? float(plan.siny[k]) : 0.f;
  }
  __syncthreads();

  // This CTA's tiles, numbered u = 0, 1, ...: tile k of its i-th plane
  // (plane blockIdx.x + i * gridDim.x) is u = i * tpp + k.
  const int my_units = blockIdx.x < units ? (units - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int ntiles = my_units * tpp;

  if (warp < SW) {
    // ---------------------------------------------------------- site warps
    if constexpr (SW == 16) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kFSiteRegs16));
    constexpr int SPW = Shape::SPW, TPS = Shape::TPS;
    const int w = warp, local = lane / TPS, sub = lane % TPS, site = w * SPW + local;
    uint64_t *wfull = full + w * kFNst;
    // Issue the copies of this warp's sites of tile v into stage v % kFNst.
    auto fetch = [&](int v) {
      const int unit = blockIdx.x + (v / tpp) * gridDim.x, k = v % tpp;
      const int t = unit / lz, z = unit - t * lz;
      const int j0 = k * kFSites + w * SPW, n = max(0, min(SPW, nsites - j0));
      const int stage = v % kFNst, nin = SAME ? 1 : 2;  // one field: one copy per site
      if (lane == 0) mbar_arrive_expect_tx(&wfull[stage], (uint32_t)n * nin * FL::SITE_BYTES);
      __syncwarp();
      if (lane < nin * n) {
        const int q = lane / n, s = lane - q * n;
        bulk_g2s(smem + kFStagesOff + stage * kFStage + ((size_t)q * kFSites + w * SPW + s) * FL::SLOT,
                 a.in[q] + plane_site(plan, t, z, j0 + s) * FL::SITE_BYTES, FL::SITE_BYTES, &wfull[stage]);
      }
    };
    for (int v = 0; v < kFNst - 1 && v < ntiles; ++v) fetch(v);
    for (int u = 0; u < ntiles; ++u) {
      const int stage = u % kFNst, ob = u & 1;
      if (u + kFNst - 1 < ntiles) {
        // stage (u - 1) % kFNst: this warp finished reading it in tile u - 1
        fence_proxy_async_smem();
        __syncwarp();
        fetch(u + kFNst - 1);
      }
      bool ok = mbar_wait_bounded(&wfull[stage], (u / kFNst) & 1, kWaitLimitNs);
      if (ok && u >= 2) ok = mbar_wait_bounded(&oempty[ob], ((u >> 1) - 1) & 1, kWaitLimitNs);
      if (!__all_sync(0xffffffffu, ok) || *abort_flag) {
        if (lane == 0) {
          *abort_flag = 1;
          report(a.status, kDevErrWaitTimeout, (unsigned int)u);
          // copies this warp issued and has not waited for: tiles u .. u + kFNst - 1
          for (int v = u; v < u + kFNst && v < ntiles; ++v)
            mbar_wait_bounded(&wfull[v % kFNst], (v / kFNst) & 1, kWaitLimitNs / 8);
        }
        return;
      }
      const int n = min(kFSites, nsites - (u % tpp) * kFSites);
      const unsigned char *sb = smem + kFStagesOff + stage * kFStage;
      const float2 *in[2] = {reinterpret_cast<const float2 *>(sb + (size_t)site * FL::SLOT),
                             reinterpret_cast<const float2 *>(sb + ((size_t)kFSites + site) * FL::SLOT)};
      float2 *dst = site < n ? obuf + ((size_t)ob * kFSites + site) * 256 : nullptr;
      if constexpr (SAME && SW == 8) site_products_same(in[0], sub, dst);
      else if constexpr (SAME) site_products_same_half(in[0], sub, dst);
      else if constexpr (SW == 8) site_products(in[0], in[1], sub, dst);
      else site_products_half(in[0], in[1], sub, dst);
      __syncwarp();  // the lanes' product stores, then lane 0's arrive (release) publishes them
      if (lane == 0) mbar_arrive(&ofull[ob]);
    }
    return;
  }

  // ------------------------------------------------------ transform warps
  if constexpr (SW == 16) asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kFTransformRegs16));
  const int g = threadIdx.x - 32 * SW;
  const int half = lx >> 1;
  const bool aligned = half % kFSites == 0;  // every tile lies in one half-row
  const bool zero0 = plan.gx_k[0] == 0;      // X group 0 is nx = 0: C = sum v, S = 0
  cx<float> *gxs = reinterpret_cast<cx<float> *>(smem + kFGxOff);  // [kMomMaxPx][256], column g is this thread's
  int u = 0;
  for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
    const int t = unit / lz, z = unit - t * lz;
    cx<float> h[QC];
#pragma unroll
    for (int q = 0; q < QC; ++q) h[q] = czero<float>();
    cx<float> gc[NG], gs[NG];
#pragma unroll
    for (int gi = 0; gi < NG; ++gi) gc[gi] = gs[gi] = czero<float>();
    int y = 0, r = 0;  // row and position in the row of the next site
    auto xstep = [&](int gi, float cs, float sn, cx<float> v) {  // packed FP32x2: (re, im) lanes
      const float2 vv = make_float2(v.x, v.y);
      const float2 c2 = __ffma2_rn(vv, make_float2(cs, cs), make_float2(gc[gi].x, gc[gi].y));
      const float2 s2 = __ffma2_rn(vv, make_float2(sn, sn), make_float2(gs[gi].x, gs[gi].y));
      gc[gi] = {c2.x, c2.y};
      gs[gi] = {s2.x, s2.y};
    };
    // row y complete: G(+k) = C + iS, G(-k) = C - iS, then the Y step
    auto end_row = [&]() {
#pragma unroll
      for (int gi = 0; gi < NG; ++gi) {
        if (plan.gx_plus[gi] >= 0) gxs[plan.gx_plus[gi] * 256 + g] = {gc[gi].x - gs[gi].y, gc[gi].y + gs[gi].x};
        if (plan.gx_minus[gi] >= 0) gxs[plan.gx_minus[gi] * 256 + g] = {gc[gi].x + gs[gi].y, gc[gi].y - gs[gi].x};
        gc[gi] = gs[gi] = czero<float>();
      }
#pragma unroll
      for (int q = 0; q < QC; ++q) cfma(h[q], cx<float> {phy[q][y][0], phy[q][y][1]}, gxs[qix[q] * 256 + g]);
      ++y;
    };
    for (int k = 0; k < tpp; ++k, ++u) {
      const int ob = u & 1;
      const bool ok = mbar_wait_bounded(&ofull[ob], (u >> 1) & 1, kWaitLimitNs);
      if (!__all_sync(0xffffffffu, ok) || *abort_flag) {
        if (lane == 0) {
          *abort_flag = 1;
          report(a.status, kDevErrWaitTimeout, (unsigned int)u);
        }
        return;
      }
      const cx<float> *col = reinterpret_cast<const cx<float> *>(obuf + (size_t)ob * kFSites * 256) + g;
      if (aligned) {
        // the tile is 16 sites of one half-row: x = x0, x0 + 2, ..., x0 + 30
        const int r0 = (k * kFSites) % lx, par = r0 >= half ? 1 : 0;
        const int x0 = 2 * (r0 - par * half) + ((par + t + z + y) & 1);
        if (zero0) {
#pragma unroll 8
          for (int s = 0; s < kFSites; ++s) {
            const cx<float> v = col[s * 256];
            gc[0].x += v.x;
            gc[0].y += v.y;
#pragma unroll
            for (int gi = 1; gi < NG; ++gi) xstep(gi, phx[gi][x0 + 2 * s][0], phx[gi][x0 + 2 * s][1], v);
          }
        } else {
#pragma unroll 8
          for (int s = 0; s < kFSites; ++s) {
            const cx<float> v = col[s * 256];
#pragma unroll
            for (int gi = 0; gi < NG; ++gi) xstep(gi, phx[gi][x0 + 2 * s][0], phx[gi][x0 + 2 * s][1], v);
          }
        }
        if (r0 + kFSites == lx) end_row();
      } else {
        const int n = min(kFSites, nsites - k * kFSites);
        for (int s = 0; s < n; ++s) {
          const int par = r >= half ? 1 : 0;
          const int x = 2 * (r - par * half) + ((par + t + z + y) & 1);
          const cx<float> v = col[s * 256];
#pragma unroll
          for (int gi = 0; gi < NG; ++gi) xstep(gi, phx[gi][x][0], phx[gi][x][1], v);
          if (++r == lx) {
            end_row();
            r = 0;
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&oempty[ob]);
    }
#pragma unroll
    for (int q = 0; q < QC; ++q)
      if (q < plan.nq) a.planes[((size_t)unit * plan.nq + q) * 256 + g] = make_float2(h[q].x, h[q].y);
  }
}

// ---------------------------------------------------------------- batched --
// The kernel above over many items (MomBatchParams): the same site and
// transform warps, with the plane geometry, inputs, plane buffer and phase
// tables taken per unit from its item.  Site warps follow their tiles with a
// cursor (unit, item, tile) that crosses plane and item boundaries, so the
// copy ring runs ahead across them; transform warps reload their phase tables
// (behind a barrier of their own) when the item changes.

__device__ __forceinline__ int batch_item_of(const MomBatchParams &p, int unit)
{
  int lo = 0, hi = p.n_items - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (p.items[mid].unit_begin <= unit) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Site j of plane (t, z) of a lattice with extents l (row order, as plane_site).
__device__ __forceinline__ long long plane_site_l(const int *l, int t, int z, int j)
{
  const int lx = l[0], ly = l[1], lz = l[2], lt = l[3], half = lx >> 1;
  const int y = j / lx, r = j - y * lx, par = r >= half ? 1 : 0, xh = r - par * half;
  return ((((long long)par * lt + t) * lz + z) * ly + y) * half + xh;
}

struct BatchCursor {
  int unit, item, k;
  __device__ __forceinline__ void start(const MomBatchParams &p)
  {
    unit = blockIdx.x;
    k = 0;
    item = unit < p.total_units ? batch_item_of(p, unit) : 0;
  }
  __device__ __forceinline__ bool valid(const MomBatchParams &p) const { return unit < p.total_units; }
  __device__ __forceinline__ void advance(const MomBatchParams &p)
  {
    if (++k < p.items[item].tpp) return;
    k = 0;
    unit += gridDim.x;
    if (unit < p.total_units) item = batch_item_of(p, unit);
  }
};

template <int SW, int NG, int QC, bool SAME>
__global__ void __launch_bounds__(FusedShape<SW>::THREADS, 1)
  momentum_batch_kernel(const __grid_constant__ MomBatchParams p)
{
  using Shape = FusedShape<SW>;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);  // [SW][kFNst]
  uint64_t *ofull = full + SW * kFNst;
  uint64_t *oempty = ofull + 2;
  uint64_t *tsync = oempty + 2;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + 504);
  float2 *obuf = reinterpret_cast<float2 *>(smem + kFOutOff);  // [2][kFSites][256]
  __shared__ float phx[NG][kMomMaxL][2];
  __shared__ float phy[QC][kMomMaxL][2];
  __shared__ int qix[QC];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < SW * kFNst; ++s) mbar_init(&full[s], 1);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&ofull[b], SW);
      mbar_init(&oempty[b], kFTW);
    }
    mbar_init(tsync, kFTW);
    *abort_flag = 0;
    fence_barrier_init();
  }
  for (int q = threadIdx.x; q < QC; q += blockDim.x) qix[q] = q < p.nq ? p.q_ix[q] : 0;
  __syncthreads();

  if (warp < SW) {
    // ---------------------------------------------------------- site warps
    if constexpr (SW == 16) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kFSiteRegs16));
    constexpr int SPW = Shape::SPW, TPS = Shape::TPS;
    const int w = warp, local = lane / TPS, sub = lane % TPS, site = w * SPW + local;
    uint64_t *wfull = full + w * kFNst;
    // Issue the copies of this warp's sites of the tile at cursor c into stage v % kFNst.
    auto fetch = [&](int v, const BatchCursor &c) {
      const MomBatchItem &it = p.items[c.item];
      const int lz = it.latt[2], local_unit = c.unit - it.unit_begin;
      const int t = local_unit / lz, z = local_unit - t * lz, nsites = it.latt[0] * it.latt[1];
      const int j0 = c.k * kFSites + w * SPW, n = max(0, min(SPW, nsites - j0));
      const int stage = v % kFNst, nin = SAME ? 1 : 2;
      if (lane == 0) mbar_arrive_expect_tx(&wfull[stage], (uint32_t)n * nin * FL::SITE_BYTES);
      __syncwarp();
      if (lane < nin * n) {
        const int q = lane / n, s = lane - q * n;
        bulk_g2s(smem + kFStagesOff + stage * kFStage + ((size_t)q * kFSites + w * SPW + s) * FL::SLOT,
                 it.in[q] + plane_site_l(it.latt, t, z, j0 + s) * FL::SITE_BYTES, FL::SITE_BYTES, &wfull[stage]);
      }
    };
    BatchCursor fc, cc;
    fc.start(p);
    cc.start(p);
    int issued = 0;
    for (; issued < kFNst - 1 && fc.valid(p); ++issued, fc.advance(p)) fetch(issued, fc);
    for (int u = 0; cc.valid(p); ++u, cc.advance(p)) {
      const int stage = u % kFNst, ob = u & 1;
      if (fc.valid(p)) {
        // stage (u - 1) % kFNst: this warp finished reading it in tile u - 1
        fence_proxy_async_smem();
        __syncwarp();
        fetch(issued++, fc);
        fc.advance(p);
      }
      bool ok = mbar_wait_bounded(&wfull[stage], (u / kFNst) & 1, kWaitLimitNs);
      if (ok && u >= 2) ok = mbar_wait_bounded(&oempty[ob], ((u >> 1) - 1) & 1, kWaitLimitNs);
      if (!__all_sync(0xffffffffu, ok) || *abort_flag) {
        if (lane == 0) {
          *abort_flag = 1;
          report(p.status, kDevErrWaitTimeout, (unsigned int)u);
          for (int v = u; v < issued; ++v) mbar_wait_bounded(&wfull[v % kFNst], (v / kFNst) & 1, kWaitLimitNs / 8);
        }
        return;
      }
      const int nsites = p.items[cc.item].latt[0] * p.items[cc.item].latt[1];
      const int n = min(kFSites, nsites - cc.k * kFSites);
      const unsigned char *sb = smem + kFStagesOff + stage * kFStage;
      const float2 *in[2] = {reinterpret_cast<const float2 *>(sb + (size_t)site * FL::SLOT),
                             reinterpret_cast<const float2 *>(sb + ((size_t)kFSites + site) * FL::SLOT)};
      float2 *dst = site < n ? obuf + ((size_t)ob * kFSites + site) * 256 : nullptr;
      if constexpr (SAME && SW == 8) site_products_same(in[0], sub, dst);
      else if constexpr (SAME) site_products_same_half(in[0], sub, dst);
      else if constexpr (SW == 8) site_products(in[0], in[1], sub, dst);
      else site_products_half(in[0], in[1], sub, dst);
      __syncwarp();  // the lanes' product stores, then lane 0's arrive (release) publishes them
      if (lane == 0) mbar_arrive(&ofull[ob]);
    }
    return;
  }

  // ------------------------------------------------------ transform warps
  if constexpr (SW == 16) asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kFTransformRegs16));
  const int g = threadIdx.x - 32 * SW;
  const bool zero0 = p.gx_k[0] == 0;  // X group 0 is nx = 0: C = sum v, S = 0
  cx<float> *gxs = reinterpret_cast<cx<float> *>(smem + kFGxOff);
  int u = 0, loaded = -1, tphase = 0;
  // All transform warps at one point (an mbarrier with a bounded wait, so that
  // a warp that gave up elsewhere cannot hold the others forever).
  auto tbarrier = [&]() -> bool {
    __syncwarp();
    if (lane == 0) mbar_arrive(tsync);
    const bool ok = mbar_wait_bounded(tsync, tphase & 1, kWaitLimitNs);
    ++tphase;
    if (__all_sync(0xffffffffu, ok) && !*abort_flag) return true;
    if (lane == 0) {
      *abort_flag = 1;
      report(p.status, kDevErrWaitTimeout, (unsigned int)u);
    }
    return false;
  };
  for (int unit = blockIdx.x; unit < p.total_units; unit += gridDim.x) {
    const int item = batch_item_of(p, unit);
    const MomBatchItem &it = p.items[item];
    const int lx = it.latt[0], ly = it.latt[1], lz = it.latt[2], half = lx >> 1;
    const int nsites = lx * ly, tpp = it.tpp;
    if (item != loaded) {  // the item's phase tables, between two barriers of the transform warps
      if (!tbarrier()) return;
      for (int e = g; e < NG * kMomMaxL; e += kFTW * 32) {
        const int gi = e / kMomMaxL, x = e % kMomMaxL;
        const float2 v = p.tab[it.tx][x < lx ? (p.gx_k[gi] * x) % lx : 0];
        phx[gi][x][0] = v.x;
        phx[gi][x][1] = v.y;
      }
      for (int e = g; e < QC * kMomMaxL; e += kFTW * 32) {
        const int q = e / kMomMaxL, y = e % kMomMaxL;
        const bool on = q < p.nq && y < ly;
        const float2 v = p.tab[it.ty][on ? ((p.q_ny[q] * y) % ly + ly) % ly : 0];
        phy[q][y][0] = on ? v.x : 0.f;
        phy[q][y][1] = on ? v.y : 0.f;
      }
      if (!tbarrier()) return;
      loaded = item;
    }
    const bool aligned = half % kFSites == 0;
    const int local_unit = unit - it.unit_begin, t = local_unit / lz, z = local_unit - t * lz;
    cx<float> h[QC];
#pragma unroll
    for (int q = 0; q < QC; ++q) h[q] = czero<float>();
    cx<float> gc[NG], gs[NG];
#pragma unroll
    for (int gi = 0; gi < NG; ++gi) gc[gi] = gs[gi] = czero<float>();
    int y = 0, r = 0;
    auto xstep = [&](int gi, float cs, float sn, cx<float> v) {
      const float2 vv = make_float2(v.x, v.y);
      const float2 c2 = __ffma2_rn(vv, make_float2(cs, cs), make_float2(gc[gi].x, gc[gi].y));
      const float2 s2 = __ffma2_rn(vv, make_float2(sn, sn), make_float2(gs[gi].x, gs[gi].y));
      gc[gi] = {c2.x, c2.y};
      gs[gi] = {s2.x, s2.y};
    };
    auto end_row = [&]() {
#pragma unroll
      for (int gi = 0; gi < NG; ++gi) {
        if (p.gx_plus[gi] >= 0) gxs[p.gx_plus[gi] * 256 + g] = {gc[gi].x - gs[gi].y, gc[gi].y + gs[gi].x};
        if (p.gx_minus[gi] >= 0) gxs[p.gx_minus[gi] * 256 + g] = {gc[gi].x + gs[gi].y, gc[gi].y - gs[gi].x};
        gc[gi] = gs[gi] = czero<float>();
      }
#pragma unroll
      for (int q = 0; q < QC; ++q) cfma(h[q], cx<float> {phy[q][y][0], phy[q][y][1]}, gxs[qix[q] * 256 + g]);
      ++y;
    };
    for (int k = 0; k < tpp; ++k, ++u) {
      const int ob = u & 1;
      const bool ok = mbar_wait_bounded(&ofull[ob], (u >> 1) & 1, kWaitLimitNs);
      if (!__all_sync(0xffffffffu, ok) || *abort_flag) {
        if (lane == 0) {
          *abort_flag = 1;
          report(p.status, kDevErrWaitTimeout, (unsigned int)u);
        }
        return;
      }
      const cx<float> *col = reinterpret_cast<const cx<float> *>(obuf + (size_t)ob * kFSites * 256) + g;
      if (aligned) {
        const int r0 = (k * kFSites) % lx, par = r0 >= half ? 1 : 0;
        const int x0 = 2 * (r0 - par * half) + ((par + t + z + y) & 1);
        if (zero0) {
#pragma unroll 8
          for (int s = 0; s < kFSites; ++s) {
            const cx<float> v = col[s * 256];
            gc[0].x += v.x;
            gc[0].y += v.y;
#pragma unroll
            for (int gi = 1; gi < NG; ++gi) xstep(gi, phx[gi][x0 + 2 * s][0], phx[gi][x0 + 2 * s][1], v);
          }
        } else {
#pragma unroll 8
          for (int s = 0; s < kFSites; ++s) {
            const cx<float> v = col[s * 256];
#pragma unroll
            for (int gi = 0; gi < NG; ++gi) xstep(gi, phx[gi][x0 + 2 * s][0], phx[gi][x0 + 2 * s][1], v);
          }
        }
        if (r0 + kFSites == lx) end_row();
      } else {
        const int n = min(kFSites, nsites - k * kFSites);
        for (int s = 0; s < n; ++s) {
          const int par = r >= half ? 1 : 0;
          const int x = 2 * (r - par * half) + ((par + t + z + y) & 1);
          const cx<float> v = col[s * 256];
#pragma unroll
          for (int gi = 0; gi < NG; ++gi) xstep(gi, phx[gi][x][0], phx[gi][x][1], v);
          if (++r == lx) {
            end_row();
            r = 0;
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&oempty[ob]);
    }
#pragma unroll
    for (int q = 0; q < QC; ++q)
      if (q < p.nq) it.planes[((size_t)local_unit * p.nq + q) * 256 + g] = make_float2(h[q].x, h[q].y);
  }
}

template <int SW, int NG, int QC, bool SAME> cudaError_t launch_batch_qc(const Job &job, const MomBatchParams &p)
{
  static int attr_set[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64 || !attr_set[dev]) {
    e = cudaFuncSetAttribute(momentum_batch_kernel<SW, NG, QC, SAME>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kFSmem);
    if (e != cudaSuccess) return e;
    if constexpr (SW == 16) {
      cudaFuncAttributes fa {};
      e = cudaFuncGetAttributes(&fa, momentum_batch_kernel<SW, NG, QC, SAME>);
      if (e != cudaSuccess) return e;
      if (fa.numRegs != kFLaunchRegs16) return cudaErrorInvalidConfiguration;
    }
    if (dev < 64) attr_set[dev] = 1;
  }
  const int grid = p.total_units < job.num_sms ? p.total_units : job.num_sms;
  momentum_batch_kernel<SW, NG, QC, SAME><<<grid, FusedShape<SW>::THREADS, kFSmem, job.stream>>>(p);
  return cudaGetLastError();
}

template <int SW, int NG, bool SAME> cudaError_t launch_batch_ng(const Job &job, const MomBatchParams &p)
{
  if (p.nq <= 4) return launch_batch_qc<SW, NG, 4, SAME>(job, p);
  if (p.nq <= 9) return launch_batch_qc<SW, NG, 9, SAME>(job, p);
  if (p.nq <= 16) return launch_batch_qc<SW, NG, 16, SAME>(job, p);
  return launch_batch_qc<SW, NG, kMomQChunk, SAME>(job, p);
}

template <int SW, bool SAME> cudaError_t launch_batch_sw(const Job &job, const MomBatchParams &p)
{
  switch (p.ngx) {
  case 1: return launch_batch_ng<SW, 1, SAME>(job, p);
  case 2: return launch_batch_ng<SW, 2, SAME>(job, p);
  case 3: return launch_batch_ng<SW, 3, SAME>(job, p);
  default: return cudaErrorInvalidValue;
  }
}

template <int SW, int NG, int QC, bool SAME>
cudaError_t launch_fused_qc(const Job &job, const FusedArgs &a, const MomPlan &plan)
{
  static int attr_set[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64 || !attr_set[dev]) {
    e = cudaFuncSetAttribute(momentum_fused_kernel<SW, NG, QC, SAME>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kFSmem);
    if (e != cudaSuccess) return e;
    if constexpr (SW == 16) {
      // the register split above assumes exactly this many registers per thread at launch
      cudaFuncAttributes fa {};
      e = cudaFuncGetAttributes(&fa, momentum_fused_kernel<SW, NG, QC, SAME>);
      if (e != cudaSuccess) return e;
      if (fa.numRegs != kFLaunchRegs16) return cudaErrorInvalidConfiguration;
    }
    if (dev < 64) attr_set[dev] = 1;
  }
  const int units = plan.latt[3] * plan.latt[2];
  const int grid = units < job.num_sms ? units : job.num_sms;
  momentum_fused_kernel<SW, NG, QC, SAME><<<grid, FusedShape<SW>::THREADS, kFSmem, job.stream>>>(a, plan);
  return cudaGetLastError();
}

template <int SW, int NG, bool SAME>
cudaError_t launch_fused_ng(const Job &job, const FusedArgs &a, const MomPlan &plan)
{
  if (plan.nq <= 4) return launch_fused_qc<SW, NG, 4, SAME>(job, a, plan);
  if (plan.nq <= 9) return launch_fused_qc<SW, NG, 9, SAME>(job, a, plan);
  if (plan.nq <= 16) return launch_fused_qc<SW, NG, 16, SAME>(job, a, plan);
  return launch_fused_qc<SW, NG, kMomQChunk, SAME>(job, a, plan);
}

template <int SW, bool SAME> cudaError_t launch_fused_sw(const Job &job, const FusedArgs &a, const MomPlan &plan)
{
  switch (plan.ngx) {
  case 1: return launch_fused_ng<SW, 1, SAME>(job, a, plan);
  case 2: return launch_fused_ng<SW, 2, SAME>(job, a, plan);
  case 3: return launch_fused_ng<SW, 3, SAME>(job, a, plan);
  default: return cudaErrorInvalidValue;
  }
}

} // namespace

bool momentum_fused_supported(const MomPlan &plan)
{
  return plan.ngx >= 1 && plan.ngx <= 3 && plan.nq >= 1 && plan.nq <= kMomQChunk && plan.latt[0] >= 2 &&
         plan.latt[0] % 2 == 0;
}

cudaError_t launch_momentum_fused(const Job &job, const void *in_i, const void *in_j, float2 *planes,
                                  const MomPlan &plan, int site_warps)
{
  if (!momentum_fused_supported(plan)) return cudaErrorInvalidValue;
  FusedArgs a {};
  a.in[0] = static_cast<const char *>(in_i);
  a.in[1] = static_cast<const char *>(in_j);
  a.planes = planes;
  a.status = job.status;
  a.tiles_per_plane = (plan.latt[0] * plan.latt[1] + kFSites - 1) / kFSites;
  // P_i and P_j one field: the Hermitian form of the site products
  if (in_i == in_j) return site_warps == 16 ? launch_fused_sw<16, true>(job, a, plan) : launch_fused_sw<8, true>(job, a, plan);
  return site_warps == 16 ? launch_fused_sw<16, false>(job, a, plan) : launch_fused_sw<8, false>(job, a, plan);
}

cudaError_t launch_momentum_batch(const Job &job, const MomBatchParams &p, bool same_field, int site_warps)
{
  if (p.total_units <= 0) return cudaSuccess;
  if (p.ngx < 1 || p.ngx > 3 || p.nq < 1 || p.nq > kMomQChunk) return cudaErrorInvalidValue;
  if (same_field) return site_warps == 16 ? launch_batch_sw<16, true>(job, p) : launch_batch_sw<8, true>(job, p);
  return site_warps == 16 ? launch_batch_sw<16, false>(job, p) : launch_batch_sw<8, false>(job, p);
}

} // namespace cgb
