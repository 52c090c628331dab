// Per-site contraction routines and the kernel "ops" that plug them into the
// tile engines (engine.cuh).
//
// Notation (one lattice site): a propagator P[s0][s1][c0][c1] is 16 colour
// blocks of 9 complex numbers; block (s0, s1) starts at (4*s0 + s1)*9.
// Gamma coefficients are phase codes (powers of i) and permutations:
//   c1(i) on spin row i with partner j = perm1[i]   (from Gamma_ij)
//   c2(l) on spin column l with partner k = perm2[l] (from Gamma_kl)
//
// Baryon two-point, canonical forms (F = eps.eps trilinear form, X ^ Y the
// colour wedge of common.cuh, W the 4x4 Gamma_mn/projector operand):
//   loop     C = sum_{i,l} c1(i) c2(l) F(A[i][perm2 l], B[perm1 i][l], Q),
//            Q = sum_{m,n} W[m][n] N[n][m]
//   triangle C = sum_{i,l} c1(i) c2(l) A[i][perm2 l] . sum_m (B[perm1 i][m] ^ N'[m][l]),
//            N'[m][l] = sum_n W[m][n] N[n][l]
// The six contract_enum.h types map onto these (CLQCD/contract
// include/baryon.cuh:43-83, baryon_general.cuh:45-93):
//   IK_JL_NM loop (A=P_i, B=P_j, c1 = Gamma_ij,   c2 = Gamma_kl^T)
//   IL_JK_NM loop (A=P_i, B=P_j, c1 = Gamma_ij,   c2 = Gamma_kl)
//   IK_JM_NL tri  (A=P_i, B=P_j, c1 = Gamma_ij,   c2 = Gamma_kl^T)
//   IL_JM_NK tri  (A=P_i, B=P_j, c1 = Gamma_ij,   c2 = Gamma_kl)
//   IM_JK_NL tri  (A=P_j, B=P_i, c1 = Gamma_ij^T, c2 = Gamma_kl^T)
//   IM_JL_NK tri  (A=P_j, B=P_i, c1 = Gamma_ij^T, c2 = Gamma_kl)
// Types that differ only in c2 share every wedge, which the fused kernel
// exploits: IK_JL/IL_JK, IK_JM/IL_JM and IM_JK/IM_JL each cost one evaluation.
//
// Thread mapping: TPS threads per site; thread `sub` owns spin row
// i = sub / (TPS/4) and LPT = 16/TPS consecutive columns l.
#pragma once

#include "engine.cuh"
#include "gamma.hpp"

namespace cgb {

// Projector operand W[m][n] (the Gamma_mn slot).  When W is a phased
// permutation (always true for a Gamma matrix) the kernels use perm/ph and
// do no multiplications with it.
template <class R> struct ProjOperand {
  R w[16][2];
  uint8_t perm[4];
  uint8_t ph[4];
  int is_perm;
  uint8_t nzk[16];  // indices m*4 + n of W's nonzero entries, in order
  int nnz;
  uint32_t nzmask;  // bit m*4 + n set where W[m][n] != 0
};

// Up to two projectors written in the gamma basis, W_w = sum_k coef[w][k] Gamma(g_k):
// N'_w[m][l] = sum_k coef[w][k] i^ph[k][m] N[perm[k][m]][l], so the triangle
// form needs one spin-permuted pass over N per basis term and no N' buffer.
template <class R> struct CliffordSet {
  int ng;
  uint8_t perm[16][4];
  uint8_t ph[16][4];
  uint8_t has_phase[16];
  R coef[2][16][2];
  R qc[2][16][4][2];  // coef[w][k] * i^ph[k][m]: the coefficient of N[perm[k][m]][m] in Q_w
};

// A projector of rank r <= 2 as W = sum_r x_r y_r^T (W[m][n] = sum_r x_r[m] y_r[n]).
// Each vector is a list of nnz (index, coefficient) entries, padded with zero
// coefficients: [side 0: x_r over rows m, side 1: y_r over columns n][r][k].
template <class R> struct RankForm {
  int r;  // 0: the projector is not of this form
  int nnz;
  uint8_t idx[2][2][4];
  R c[2][2][4][2];
  // unit: every coefficient is scale_v i^ph and scale_x * scale_y is one value
  // `scale` for every r (true for (1 +- g4)/2 and the polarised projectors):
  // the complex128 builds then add phased blocks and the triangle values take
  // `scale` (rank_unit_form).  complex64 keeps the coefficients.
  int unit;
  uint8_t ph[2][2][4];
  R scale;
};

template <class R> struct BaryonSpin {
  uint8_t perm1[4], perm2[4];
  uint8_t ph1[2][4];  // [0]: c1 for A = P_i groups, [1]: c1 for the swapped (IM_*) group
  uint8_t ph2[2][4];  // c2 variants (one per output of a loop/tri evaluation)
  ProjOperand<R> proj[2];
  CliffordSet<R> cl;
  RankForm<R> rk;  // proj[0] factored, for the triangle form
};

template <class R> struct MesonSpin {
  uint8_t perm1[4], perm2[4];
  uint8_t ph1[4], ph2[4];
};

template <class R> struct OpParams {
  const void *in[3];
  void *out[16];
  TileGeom geom;
  DeviceStatus *status;
  BaryonSpin<R> b;
  MesonSpin<R> m;
  int latt[4];  // Lx, Ly, Lz, Lt where an op needs site coordinates
};

template <int TPS> struct Lanes {
  static constexpr int TPI = TPS / 4;  // threads per spin row
  static constexpr int LPT = 4 / TPI;  // spin columns per thread
  static_assert(TPS == 4 || TPS == 8 || TPS == 16, "TPS must be 4, 8 or 16");
};

// Q_w[ad] = sum_{m,n} W[m][n] N[n][m][ad], one entry per thread, into smem q[w*9 + ad].
template <class R, class S, int TPS, int NW>
__device__ __forceinline__ void build_q(const BaryonSpin<R> &b, const S *N, S *q, int sub)
{
  for (int e = sub; e < 9 * NW; e += TPS) {
    const int w = e / 9, ad = e % 9;
    const ProjOperand<R> &pw = b.proj[w];
    cx<R> s = czero<R>();
    if (pw.is_perm) {
#pragma unroll
      for (int m = 0; m < 4; ++m) s = cadd(s, mul_phase(ld<R>(N + (pw.perm[m] * 4 + m) * 9 + ad), pw.ph[m]));
    } else if constexpr (sizeof(R) == 8) {
      // complex128: W's nonzero entries from the host's list.  Testing each
      // entry here takes FP64 compares on the FP64 pipe, which bounds these
      // kernels (the loop form with (1 + g4)/2: 7.55 ms against 5.72 ms).
#pragma unroll 1
      for (int t = 0; t < pw.nnz; ++t) {
        const int k = pw.nzk[t];  // W[m][n], m = k / 4, n = k % 4, times N[n][m]
        cfma(s, cx<R> {pw.w[k][0], pw.w[k][1]}, ld<R>(N + ((k & 3) * 4 + (k >> 2)) * 9 + ad));
      }
    } else {
      // complex64: unrolled over W with the host's nonzero mask (a list loop
      // measured 2 % slower on this HBM-bound form).
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int n = 0; n < 4; ++n)
          if ((pw.nzmask >> (m * 4 + n)) & 1u)
            cfma(s, cx<R> {pw.w[m * 4 + n][0], pw.w[m * 4 + n][1]}, ld<R>(N + (n * 4 + m) * 9 + ad));
    }
    st(q + e, s);
  }
}

// Q_w from the gamma-basis form: Q_w = sum_k coef[w][k] sum_m i^ph[k][m] N[perm[k][m]][m].
template <class R, class S, int TPS, int NW>
__device__ __forceinline__ void build_q_cliff(const BaryonSpin<R> &b, const S *N, S *q, int sub)
{
  // One colour entry ad per thread, all NW projectors at once: each N value is
  // loaded once and scaled by the precombined coefficients qc.
  const CliffordSet<R> &cl = b.cl;
  for (int ad = sub; ad < 9; ad += TPS) {
    cx<R> s[NW];
#pragma unroll
    for (int w = 0; w < NW; ++w) s[w] = czero<R>();
    for (int k = 0; k < cl.ng; ++k) {
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const cx<R> n = ld<R>(N + (cl.perm[k][m] * 4 + m) * 9 + ad);
#pragma unroll
        for (int w = 0; w < NW; ++w) cfma(s[w], cx<R> {cl.qc[w][k][m][0], cl.qc[w][k][m][1]}, n);
      }
    }
#pragma unroll
    for (int w = 0; w < NW; ++w) st(q + w * 9 + ad, s[w]);
  }
}

// Largest gamma-basis term count for which build_nprime takes the basis form:
// ng terms cost ng x 9 complex FMA per N' block, the row form four x 9.
constexpr int kNprimeCliffTerms = 4;

// N'_w[m][l] = sum_n W[m][n] N[n][l] into the w-th scratch slot.  With
// `cliff` (b.cl filled for these projectors, few terms) each block is built
// from the gamma basis instead, N'_w[m][l] = sum_k qc[w][k][m] N[perm[k][m]][l]:
// cl.ng iterations that every lane takes, where the row form skips W's zero
// entries per lane and so runs all four n for a warp whose lanes hold
// different rows m.
template <class R, class S, int TPS, int NW>
__device__ __forceinline__ void build_nprime(const BaryonSpin<R> &b, const S *N, S *np, int sub, bool cliff = false)
{
  for (int e = sub; e < 16 * NW; e += TPS) {
    const int w = e / 16, blk = e % 16, m = blk / 4, l = blk % 4;
    const ProjOperand<R> &pw = b.proj[w];
    S *dst = np + (size_t)w * 144 + blk * 9;
    if (cliff) {
      const CliffordSet<R> &cl = b.cl;
      cx<R> o[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) o[k] = czero<R>();
#pragma unroll 1
      for (int k = 0; k < cl.ng; ++k) {
        const S *src = N + (cl.perm[k][m] * 4 + l) * 9;
        const cx<R> c {cl.qc[w][k][m][0], cl.qc[w][k][m][1]};
#pragma unroll
        for (int q = 0; q < 9; ++q) cfma(o[q], c, ld<R>(src + q));
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) st(dst + k, o[k]);
    } else if (pw.is_perm) {
      const S *src = N + (pw.perm[m] * 4 + l) * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) st(dst + k, mul_phase(ld<R>(src + k), pw.ph[m]));
    } else {
      cx<R> o[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) o[k] = czero<R>();
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        if (!((pw.nzmask >> (m * 4 + n)) & 1u)) continue;
        const cx<R> wv {pw.w[m * 4 + n][0], pw.w[m * 4 + n][1]};
#pragma unroll
        for (int k = 0; k < 9; ++k) cfma(o[k], wv, ld<R>(N + (n * 4 + l) * 9 + k));
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) st(dst + k, o[k]);
    }
  }
}

// Loop form.  Writes vals[v*NW + w] (partial over this thread's (i, l) pairs).
template <class R, class S, int TPS, int NV, int NW>
__device__ __forceinline__ void loop_site(const BaryonSpin<R> &b, const S *A, const S *B, const S *q, int sub, int c1sel,
                                          cx<R> *vals)
{
  using Ln = Lanes<TPS>;
  const int i = sub / Ln::TPI, l0 = (sub % Ln::TPI) * Ln::LPT;
  const int j = b.perm1[i];
  if constexpr (Ln::LPT == 1) {
    // One (i, l) pair per thread: contract the wedge with Q first and apply
    // the (i, l) phases to the NV x NW scalars only.
    cx<R> x[9], y[9], t[9];
    load9(x, A + (i * 4 + b.perm2[l0]) * 9);
    load9(y, B + (j * 4 + l0) * 9);
#pragma unroll
    for (int k = 0; k < 9; ++k) t[k] = czero<R>();
    wedge_acc(t, x, y);
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      cx<R> qw[9];
      load9(qw, q + w * 9);
      const cx<R> s = dot9(t, qw);
#pragma unroll
      for (int v = 0; v < NV; ++v) vals[v * NW + w] = mul_phase(s, (b.ph1[c1sel][i] + b.ph2[v][l0]) & 3u);
    }
    return;
  }
  cx<R> r[NV][9];
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int k = 0; k < 9; ++k) r[v][k] = czero<R>();
#pragma unroll
  for (int lo = 0; lo < Ln::LPT; ++lo) {
    const int l = l0 + lo;
    cx<R> x[9], y[9];
    load9(x, A + (i * 4 + b.perm2[l]) * 9);
    load9(y, B + (j * 4 + l) * 9);
    if constexpr (NV == 1) {
      phase9(x, b.ph2[0][l]);
      wedge_acc(r[0], x, y);
    } else {
      cx<R> t[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) t[k] = czero<R>();
      wedge_acc(t, x, y);
#pragma unroll
      for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int k = 0; k < 9; ++k) r[v][k] = cadd(r[v][k], mul_phase(t[k], b.ph2[v][l]));
    }
  }
  const uint32_t p1 = b.ph1[c1sel][i];
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    cx<R> qw[9];
    load9(qw, q + w * 9);
#pragma unroll
    for (int v = 0; v < NV; ++v) vals[v * NW + w] = mul_phase(dot9(r[v], qw), p1);
  }
}

// Triangle form over N' (NW slots of 144 complex).  Writes vals[v*NW + w].
// Loop order l -> m -> w: each B block is loaded once and feeds every
// projector; with two projectors the wedge a ^ B_m is shared between them.
template <class R, class S, int TPS, int NV, int NW>
__device__ __forceinline__ void triangle_site(const BaryonSpin<R> &b, const S *A, const S *B, const S *np, int sub,
                                              int c1sel, cx<R> *vals)
{
  using Ln = Lanes<TPS>;
  const int i = sub / Ln::TPI, l0 = (sub % Ln::TPI) * Ln::LPT;
  const int j = b.perm1[i];
  cx<R> acc[NV][NW];
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int w = 0; w < NW; ++w) acc[v][w] = czero<R>();

  constexpr bool kCacheB = Ln::LPT > 1;
  cx<R> brow[kCacheB ? 4 : 1][9];
  if constexpr (kCacheB) {
#pragma unroll
    for (int m = 0; m < 4; ++m) load9(brow[m], B + (j * 4 + m) * 9);
  }
#pragma unroll
  for (int lo = 0; lo < Ln::LPT; ++lo) {
    const int l = l0 + lo;
    if constexpr (NW >= 2) {
      // a . (B_m ^ N'_w) = N'_w . (a ^ B_m): one wedge per m shared by the projectors.
      cx<R> a[9];
      load9(a, A + (i * 4 + b.perm2[l]) * 9);
      cx<R> sw[NW];
#pragma unroll
      for (int w = 0; w < NW; ++w) sw[w] = czero<R>();
#pragma unroll 1
      for (int m = 0; m < 4; ++m) {
        cx<R> e[9];
        {
          cx<R> bm[9];
          if constexpr (kCacheB) {
#pragma unroll
            for (int k = 0; k < 9; ++k) bm[k] = brow[m][k];
          } else {
            load9(bm, B + (j * 4 + m) * 9);
          }
#pragma unroll
          for (int k = 0; k < 9; ++k) e[k] = czero<R>();
          wedge_acc(e, a, bm);
        }
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          cx<R> nn[9];
          load9(nn, np + (size_t)w * 144 + (m * 4 + l) * 9);
          const cx<R> t = dot9(nn, e);
          sw[w] = cadd(sw[w], t);
        }
      }
#pragma unroll
      for (int w = 0; w < NW; ++w)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v][w] = cadd(acc[v][w], mul_phase(sw[w], b.ph2[v][l]));
    } else {
      cx<R> d[NW][9];
#pragma unroll
      for (int w = 0; w < NW; ++w)
#pragma unroll
        for (int k = 0; k < 9; ++k) d[w][k] = czero<R>();
      // Not unrolled: keeps one B block and one N' block live (register pressure).
#pragma unroll 1
      for (int m = 0; m < 4; ++m) {
        cx<R> bm[9];
        if constexpr (kCacheB) {
#pragma unroll
          for (int k = 0; k < 9; ++k) bm[k] = brow[m][k];
        } else {
          load9(bm, B + (j * 4 + m) * 9);
        }
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          cx<R> nn[9];
          load9(nn, np + (size_t)w * 144 + (m * 4 + l) * 9);
          wedge_acc(d[w], bm, nn);
        }
      }
      cx<R> a[9];
      load9(a, A + (i * 4 + b.perm2[l]) * 9);
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        const cx<R> s = dot9(a, d[w]);
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v][w] = cadd(acc[v][w], mul_phase(s, b.ph2[v][l]));
      }
    }
  }
  const uint32_t p1 = b.ph1[c1sel][i];
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int w = 0; w < NW; ++w) vals[v * NW + w] = mul_phase(acc[v][w], p1);
}

// Triangle form with a projector of rank r <= 2 (RankForm).  By bilinearity
// of the wedge,
//   sum_m B[j][m] ^ N'[m][l] = sum_r X_r[j] ^ Y_r[l],
//   X_r[j] = sum_m x_r[m] B[j][m],  Y_r[l] = sum_n y_r[n] N[n][l],
// so each (i, l) pair takes r wedges and one dot where the N' form takes four
// wedges.  build_rank writes X_r[j] (from B) at block r*4 + j of xy, Y_r[l] at
// block 8 + r*4 + l and, when B2 is given, X_r[j] from B2 at block 16 + r*4 + j.
// Whether the factored form runs on unit-modulus phases: complex128 only, where
// the FP64 pipe bounds the kernels (9.81 -> 9.32 ms for (1 + g4)/2 at
// 24^3 x 64); the complex64 build, on packed FP32 FMAs, measured 2-4 % slower so.
template <class R> __device__ __forceinline__ bool rank_unit_form(const RankForm<R> &rk)
{
  return sizeof(R) == 8 && rk.unit;
}

template <class R, class S, int TPS>
__device__ __forceinline__ void build_rank(const RankForm<R> &rk, const S *B, const S *N, const S *B2, S *xy,
                                           int sub)
{
  const int nb = 4 * rk.r, sides = B2 ? 3 : 2;
  for (int e = sub; e < sides * nb; e += TPS) {
    const int side = e / nb, rem = e - side * nb, rr = rem / 4, q = rem % 4;
    const int ycol = side == 1;  // Y: N[n][q] at block n*4 + q; X: B[q][m] at block q*4 + m
    const S *base = ycol ? N + q * 9 : (side ? B2 : B) + q * 36;
    const int stride = ycol ? 36 : 9;
    cx<R> o[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) o[k] = czero<R>();
    const bool unit = rank_unit_form(rk);
    if (unit) {
#pragma unroll 1
      for (int k = 0; k < rk.nnz; ++k) {
        const S *src = base + rk.idx[ycol][rr][k] * stride;
        const uint32_t ph = rk.ph[ycol][rr][k];
#pragma unroll
        for (int t = 0; t < 9; ++t) o[t] = cadd(o[t], mul_phase(ld<R>(src + t), ph));
      }
    }
#pragma unroll 1
    for (int k = 0; k < (unit ? 0 : rk.nnz); ++k) {
      const S *src = base + rk.idx[ycol][rr][k] * stride;
      const cx<R> c {rk.c[ycol][rr][k][0], rk.c[ycol][rr][k][1]};
#pragma unroll
      for (int t = 0; t < 9; ++t) cfma(o[t], c, ld<R>(src + t));
    }
    S *dst = xy + ((side * 2 + rr) * 4 + q) * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) st(dst + k, o[k]);
  }
}

// Triangle values for the NV c2 variants from X_r (block r*4 + j of X) and
// Y_r (block r*4 + l of Y); c1 from ph1[c1sel].
template <class R, class S, int TPS, int NV>
__device__ __forceinline__ void triangle_rank_site(const BaryonSpin<R> &b, const S *A, const S *X, const S *Y, int sub,
                                                   int c1sel, cx<R> *vals)
{
  using Ln = Lanes<TPS>;
  const int i = sub / Ln::TPI, l0 = (sub % Ln::TPI) * Ln::LPT;
  const int j = b.perm1[i];
  cx<R> acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = czero<R>();
#pragma unroll
  for (int lo = 0; lo < Ln::LPT; ++lo) {
    const int l = l0 + lo;
    cx<R> d[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) d[k] = czero<R>();
#pragma unroll 1
    for (int rr = 0; rr < b.rk.r; ++rr) {
      cx<R> x[9], y[9];
      load9(x, X + (rr * 4 + j) * 9);
      load9(y, Y + (rr * 4 + l) * 9);
      wedge_acc(d, x, y);
    }
    cx<R> a[9];
    load9(a, A + (i * 4 + b.perm2[l]) * 9);
    const cx<R> t = dot9(a, d);
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = cadd(acc[v], mul_phase(t, b.ph2[v][l]));
  }
  const R sc = rank_unit_form(b.rk) ? b.rk.scale : R(1);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const cx<R> z = mul_phase(acc[v], b.ph1[c1sel][i]);
    vals[v] = cx<R> {z.x * sc, z.y * sc};
  }
}

// Triangle form with the projectors in the gamma basis (CliffordSet):
//   D_k = sum_m B[perm1 i][m] ^ (i^ph[k][m] N[perm[k][m]][l]),  s_k = A[i][perm2 l] . D_k
//   vals[v*NW + w] = c1(i) sum_l c2_v(l) sum_k coef[w][k] s_k
// With two or more basis terms the wedge a ^ B[perm1 i][m] is formed once
// per m and dotted with each term's N block; with one term the basis term
// runs outermost so that one D accumulator is live.
template <class R, class S, int TPS, int NV, int NW>
__device__ __forceinline__ void triangle_cliff_site(const BaryonSpin<R> &b, const S *A, const S *B, const S *N, int sub,
                                                    int c1sel, cx<R> *vals)
{
  using Ln = Lanes<TPS>;
  const CliffordSet<R> &cl = b.cl;
  const int i = sub / Ln::TPI, l0 = (sub % Ln::TPI) * Ln::LPT;
  const int j = b.perm1[i];
  cx<R> acc[NV][NW];
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int w = 0; w < NW; ++w) acc[v][w] = czero<R>();
#pragma unroll
  for (int lo = 0; lo < Ln::LPT; ++lo) {
    const int l = l0 + lo;
    cx<R> a[9];
    load9(a, A + (i * 4 + b.perm2[l]) * 9);
    cx<R> u[NW];  // sum_k coef[w][k] s_k for this l
#pragma unroll
    for (int w = 0; w < NW; ++w) u[w] = czero<R>();
    if (cl.ng >= 2) {
      // The triple product a . (b ^ n) is symmetric in a, b, n, so
      // s_k = sum_m n_km . E_m with E_m = a ^ B[perm1 i][m] shared by every
      // basis term: 4 wedges + 4 ng dots instead of 4 ng wedges + ng dots.
#pragma unroll 1
      for (int m = 0; m < 4; ++m) {
        cx<R> e[9];
        {
          cx<R> bm[9];
          load9(bm, B + (j * 4 + m) * 9);
#pragma unroll
          for (int q = 0; q < 9; ++q) e[q] = czero<R>();
          wedge_acc(e, a, bm);
        }
#pragma unroll 1
        for (int k = 0; k < cl.ng; ++k) {
          cx<R> nn[9];
          load9(nn, N + (cl.perm[k][m] * 4 + l) * 9);
          const cx<R> s = mul_phase(dot9(nn, e), cl.ph[k][m]);
#pragma unroll
          for (int w = 0; w < NW; ++w) cfma(u[w], cx<R> {cl.coef[w][k][0], cl.coef[w][k][1]}, s);
        }
      }
    } else {
#pragma unroll 1
      for (int k = 0; k < cl.ng; ++k) {
        cx<R> d[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) d[e] = czero<R>();
        const bool phased = cl.has_phase[k];
#pragma unroll 1
        for (int m = 0; m < 4; ++m) {
          cx<R> bm[9], nn[9];
          load9(bm, B + (j * 4 + m) * 9);
          load9(nn, N + (cl.perm[k][m] * 4 + l) * 9);
          if (phased) phase9(nn, cl.ph[k][m]);
          wedge_acc(d, bm, nn);
        }
        const cx<R> s = dot9(a, d);
#pragma unroll
        for (int w = 0; w < NW; ++w) cfma(u[w], cx<R> {cl.coef[w][k][0], cl.coef[w][k][1]}, s);
      }
    }
#pragma unroll
    for (int w = 0; w < NW; ++w)
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[v][w] = cadd(acc[v][w], mul_phase(u[w], b.ph2[v][l]));
  }
  const uint32_t p1 = b.ph1[c1sel][i];
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int w = 0; w < NW; ++w) vals[v * NW + w] = mul_phase(acc[v][w], p1);
}

// One triangle pass of the fused kernel (one (i, l) pair per thread) with the
// gamma-basis projectors, on the shared-wedge order of triangle_cliff_site.
// The m loop starts at m = l: with (A, B) = (P_i, P_j) its first wedge
// A[i][perm2 l] ^ B[perm1 i][l] is the loop form's, so LOOP folds the two loop
// types (dots with Q_w) into that iteration.  out[v*NW + w] = triangle values,
// loop[v*NW + w] = loop values.
template <class R, class S, int NW, bool LOOP>
__device__ __forceinline__ void fused_triangle_pass(const BaryonSpin<R> &b, const S *A, const S *B, const S *N,
                                                    const S *q, int i, int l, int c1sel, cx<R> *out, cx<R> *loop)
{
  const CliffordSet<R> &cl = b.cl;
  const int j = b.perm1[i];
  cx<R> a[9];
  load9(a, A + (i * 4 + b.perm2[l]) * 9);
  cx<R> u[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) u[w] = czero<R>();
  const bool two = cl.ng == 2;
  cx<R> s0 = czero<R>(), s1 = czero<R>();  // per-term sums when there are two terms
#pragma unroll 1
  for (int mm = 0; mm < 4; ++mm) {
    const int m = (l + mm) & 3;
    cx<R> e[9];
    {
      cx<R> bm[9];
      load9(bm, B + (j * 4 + m) * 9);
#pragma unroll
      for (int k = 0; k < 9; ++k) e[k] = czero<R>();
      wedge_acc(e, a, bm);
    }
    if constexpr (LOOP) {
      if (mm == 0) {
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          cx<R> qw[9];
          load9(qw, q + w * 9);
          const cx<R> sq = dot9(e, qw);
#pragma unroll
          for (int v = 0; v < 2; ++v) loop[v * NW + w] = mul_phase(sq, (b.ph1[c1sel][i] + b.ph2[v][l]) & 3u);
        }
      }
    }
    if (two) {
      cx<R> nn[9];
      load9(nn, N + (cl.perm[0][m] * 4 + l) * 9);
      s0 = cadd(s0, mul_phase(dot9(nn, e), cl.ph[0][m]));
      load9(nn, N + (cl.perm[1][m] * 4 + l) * 9);
      s1 = cadd(s1, mul_phase(dot9(nn, e), cl.ph[1][m]));
    } else {
#pragma unroll 1
      for (int k = 0; k < cl.ng; ++k) {
        cx<R> nn[9];
        load9(nn, N + (cl.perm[k][m] * 4 + l) * 9);
        const cx<R> s = mul_phase(dot9(nn, e), cl.ph[k][m]);
#pragma unroll
        for (int w = 0; w < NW; ++w) cfma(u[w], cx<R> {cl.coef[w][k][0], cl.coef[w][k][1]}, s);
      }
    }
  }
  if (two) {
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      cfma(u[w], cx<R> {cl.coef[w][0][0], cl.coef[w][0][1]}, s0);
      cfma(u[w], cx<R> {cl.coef[w][1][0], cl.coef[w][1][1]}, s1);
    }
  }
  const uint32_t p1 = b.ph1[c1sel][i];
#pragma unroll
  for (int w = 0; w < NW; ++w)
#pragma unroll
    for (int v = 0; v < 2; ++v) out[v * NW + w] = mul_phase(u[w], (p1 + b.ph2[v][l]) & 3u);
}

// Both triangle passes of the fused kernel in one m loop: with
// a1 = P_i[i][perm2 l] and a2 = P_j[i][perm2 l], each N block n_km is loaded
// once and dotted with both a1 ^ P_j[perm1 i][m] and a2 ^ P_i[perm1 i][m].
// The loop form is folded into the m = l wedge of the first pass as in
// fused_triangle_pass.  vals[type * NW + w], types in contract_enum.h order.
template <class R, class S, int NW, bool SAMEIJ = false>
__device__ __forceinline__ void fused_merged_site(const BaryonSpin<R> &b, const S *Pi, const S *Pj, const S *N,
                                                  const S *q, int i, int l, cx<R> *vals)
{
  const CliffordSet<R> &cl = b.cl;
  const int j = b.perm1[i];
  cx<R> a1[9], a2[9];
  load9(a1, Pi + (i * 4 + b.perm2[l]) * 9);
  if constexpr (!SAMEIJ) load9(a2, Pj + (i * 4 + b.perm2[l]) * 9);
  cx<R> u1[NW], u2[NW];
  S *lps = const_cast<S *>(q) + 9 * NW + (i * 4 + l) * 2 * NW;  // loop values, parked in shared memory
#pragma unroll
  for (int w = 0; w < NW; ++w) u1[w] = u2[w] = czero<R>();
  const bool two = cl.ng == 2, phased = cl.has_phase[0] || cl.has_phase[1];
  cx<R> s10 = czero<R>(), s11 = czero<R>(), s20 = czero<R>(), s21 = czero<R>();
#pragma unroll 1
  for (int mm = 0; mm < 4; ++mm) {
    const int m = (l + mm) & 3;
    cx<R> e1[9], e2[9];
    {
      cx<R> bm[9];
      load9(bm, Pj + (j * 4 + m) * 9);
#pragma unroll
      for (int k = 0; k < 9; ++k) e1[k] = czero<R>();
      wedge_acc(e1, a1, bm);
      if constexpr (!SAMEIJ) {
        load9(bm, Pi + (j * 4 + m) * 9);
#pragma unroll
        for (int k = 0; k < 9; ++k) e2[k] = czero<R>();
        wedge_acc(e2, a2, bm);
      }
    }
    if (mm == 0) {
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        cx<R> qw[9];
        load9(qw, q + w * 9);
        const cx<R> sq = dot9(e1, qw);
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          const cx<R> lv = mul_phase(sq, (b.ph1[0][i] + b.ph2[v][l]) & 3u);
          lps[v * NW + w] = S {lv.x, lv.y};
        }
      }
    }
    if (two && !phased) {  // e.g. (1 +- g4)/2 = (Gamma(0) +- Gamma(8))/2: no phases to apply
      cx<R> nn[9];
      load9(nn, N + (cl.perm[0][m] * 4 + l) * 9);
      s10 = cadd(s10, dot9(nn, e1));
      if constexpr (!SAMEIJ) s20 = cadd(s20, dot9(nn, e2));
      load9(nn, N + (cl.perm[1][m] * 4 + l) * 9);
      s11 = cadd(s11, dot9(nn, e1));
      if constexpr (!SAMEIJ) s21 = cadd(s21, dot9(nn, e2));
    } else if (two) {
      cx<R> nn[9];
      load9(nn, N + (cl.perm[0][m] * 4 + l) * 9);
      s10 = cadd(s10, mul_phase(dot9(nn, e1), cl.ph[0][m]));
      if constexpr (!SAMEIJ) s20 = cadd(s20, mul_phase(dot9(nn, e2), cl.ph[0][m]));
      load9(nn, N + (cl.perm[1][m] * 4 + l) * 9);
      s11 = cadd(s11, mul_phase(dot9(nn, e1), cl.ph[1][m]));
      if constexpr (!SAMEIJ) s21 = cadd(s21, mul_phase(dot9(nn, e2), cl.ph[1][m]));
    } else {
#pragma unroll 1
      for (int k = 0; k < cl.ng; ++k) {
        cx<R> nn[9];
        load9(nn, N + (cl.perm[k][m] * 4 + l) * 9);
        const cx<R> t1 = mul_phase(dot9(nn, e1), cl.ph[k][m]);
#pragma unroll
        for (int w = 0; w < NW; ++w) cfma(u1[w], cx<R> {cl.coef[w][k][0], cl.coef[w][k][1]}, t1);
        if constexpr (!SAMEIJ) {
          const cx<R> t2 = mul_phase(dot9(nn, e2), cl.ph[k][m]);
#pragma unroll
          for (int w = 0; w < NW; ++w) cfma(u2[w], cx<R> {cl.coef[w][k][0], cl.coef[w][k][1]}, t2);
        }
      }
    }
  }
  if (two) {
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      const cx<R> c0 {cl.coef[w][0][0], cl.coef[w][0][1]}, c1 {cl.coef[w][1][0], cl.coef[w][1][1]};
      cfma(u1[w], c0, s10);
      cfma(u1[w], c1, s11);
      if constexpr (!SAMEIJ) {
        cfma(u2[w], c0, s20);
        cfma(u2[w], c1, s21);
      }
    }
  }
  if constexpr (SAMEIJ) {  // P_i and P_j are one field: both passes give the same sums
#pragma unroll
    for (int w = 0; w < NW; ++w) u2[w] = u1[w];
  }
  const uint32_t p1 = b.ph1[0][i], p2 = b.ph1[1][i];
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    vals[0 * NW + w] = cx<R> {lps[0 * NW + w].x, lps[0 * NW + w].y};  // IK_JL_NM
    vals[2 * NW + w] = cx<R> {lps[1 * NW + w].x, lps[1 * NW + w].y};  // IL_JK_NM
    vals[1 * NW + w] = mul_phase(u1[w], (p1 + b.ph2[0][l]) & 3u);      // IK_JM_NL
    vals[3 * NW + w] = mul_phase(u1[w], (p1 + b.ph2[1][l]) & 3u);      // IL_JM_NK
    vals[4 * NW + w] = mul_phase(u2[w], (p2 + b.ph2[0][l]) & 3u);      // IM_JK_NL
    vals[5 * NW + w] = mul_phase(u2[w], (p2 + b.ph2[1][l]) & 3u);      // IM_JL_NK
  }
}

// Both triangle passes from one set of wedges.  The wedge is symmetric
// (X ^ Y = Y ^ X) and every gamma permutation is an involution, so the second
// pass's wedge P_j[i][perm2 l] ^ P_i[perm1 i][m] is the first pass's wedge
// E[i'][x][n] = P_i[i'][x] ^ P_j[perm1 i'][n] at i' = perm1 i, x = m,
// n = perm2 l.  Thread (i, x) forms its four wedges E[i][x][n] once and
// dots each with the N blocks of both passes:
//   pass 1 (IK_JM_NL, IL_JM_NK; target (i, l = perm2 x), m = n):
//     N[perm_k n][l], coefficient coef_k i^ph_k(n), output phase fixed per thread;
//   pass 2 (IM_JK_NL, IM_JL_NK; target (perm1 i, perm2 n), m = x):
//     N[perm_k x][perm2 n], coefficient coef_k i^ph_k(x) = qc[.][k][x], output
//     phase i^(ph1[1][perm1 i] + ph2[0][perm2 n]) applied per n.
// The outputs are summed over the site's 16 threads, so a thread may add
// terms that belong to another (i, l).  The loop types use the n = l wedge
// (the loop form's A[i][perm2 l] ^ B[perm1 i][l]) as in fused_merged_site.
// Every Gamma(n) of the DeGrand-Rossi basis is symmetric or antisymmetric, so
// the Gamma_kl and Gamma_kl^T variants of each type differ by one sign:
// IL_JK_NM, IL_JM_NK and IM_JL_NK are i^v1 times IK_JL_NM, IK_JM_NL and
// IM_JK_NL, v1 = ph2[1] - ph2[0] (0 or 2, the same in every column; the
// launcher checks it).  Per site: 64 wedges + 256 dots + 32 loop dots (4 898
// complex FMA with two two-term projectors) instead of 128 wedges + 256 dots
// + 32 (7 382).
template <class R, class S, int NW, bool PHASED>
__device__ __forceinline__ void shared_wedge_loop(const BaryonSpin<R> &b, const cx<R> (&a)[9], const S *Pjj,
                                                  const S *Nl, const S *const (&Nx)[NW], const S *q, S *lps,
                                                  int l, uint32_t p2base, cx<R> (&s1)[NW], cx<R> (&s2)[NW])
{
  const CliffordSet<R> &cl = b.cl;
  const int ng = cl.ng;
#pragma unroll 1
  for (int mm = 0; mm < 4; ++mm) {
    const int n = (l + mm) & 3;
    cx<R> e[9];
    {
      cx<R> bn[9];
      load9(bn, Pjj + n * 9);
#pragma unroll
      for (int k = 0; k < 9; ++k) e[k] = czero<R>();
      wedge_acc(e, a, bn);
    }
    if (mm == 0) {  // n = l: the loop form's wedge
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        cx<R> qw[9];
        load9(qw, q + w * 9);
        const cx<R> sq = dot9(e, qw);
        lps[w] = S {sq.x, sq.y};
      }
    }
    const int ln = b.perm2[n];
    const uint32_t q0 = (p2base + b.ph2[0][ln]) & 3u;
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      if (k < ng) {
        cx<R> nn[9];
        load9(nn, Nl + cl.perm[k][n] * 36);  // pass 1
        const cx<R> d = dot9(e, nn);
        s1[k] = cadd(s1[k], PHASED ? mul_phase(d, cl.ph[k][n]) : d);
        load9(nn, Nx[k] + ln * 9);  // pass 2
        s2[k] = cadd(s2[k], mul_phase(dot9(e, nn), q0));
      }
    }
  }
}

template <class R, class S, int NW>
__device__ __forceinline__ void fused_shared_wedge_site(const BaryonSpin<R> &b, const S *Pi, const S *Pj, const S *N,
                                                        const S *q, int i, int x, cx<R> *vals)
{
  const CliffordSet<R> &cl = b.cl;
  const int j = b.perm1[i];
  const int l = b.perm2[x];
  const int ng = cl.ng;  // <= NW gamma-basis terms
  cx<R> a[9];
  load9(a, Pi + (i * 4 + x) * 9);
  S *lps = const_cast<S *>(q) + 9 * NW + (i * 4 + x) * NW;  // loop values, parked in shared memory
  const S *Nx[NW];
#pragma unroll
  for (int k = 0; k < NW; ++k) Nx[k] = N + (k < ng ? cl.perm[k][x] : 0) * 36;
  cx<R> s1[NW], s2[NW];
#pragma unroll
  for (int k = 0; k < NW; ++k) s1[k] = s2[k] = czero<R>();
  const uint32_t p2base = b.ph1[1][j];
  if (cl.has_phase[0] || cl.has_phase[1])
    shared_wedge_loop<R, S, NW, true>(b, a, Pj + j * 36, N + l * 9, Nx, q, lps, l, p2base, s1, s2);
  else
    shared_wedge_loop<R, S, NW, false>(b, a, Pj + j * 36, N + l * 9, Nx, q, lps, l, p2base, s1, s2);
  const uint32_t p1 = (b.ph1[0][i] + b.ph2[0][l]) & 3u, v1 = (b.ph2[1][0] - b.ph2[0][0]) & 3u;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    cx<R> u1 = czero<R>(), u2 = czero<R>();
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      if (k < ng) {
        cfma(u1, cx<R> {cl.coef[w][k][0], cl.coef[w][k][1]}, s1[k]);
        cfma(u2, cx<R> {cl.qc[w][k][x][0], cl.qc[w][k][x][1]}, s2[k]);
      }
    }
    const cx<R> lv = mul_phase(cx<R> {lps[w].x, lps[w].y}, p1);
    const cx<R> t1 = mul_phase(u1, p1);
    vals[0 * NW + w] = lv;                  // IK_JL_NM
    vals[2 * NW + w] = mul_phase(lv, v1);   // IL_JK_NM
    vals[1 * NW + w] = t1;                  // IK_JM_NL
    vals[3 * NW + w] = mul_phase(t1, v1);   // IL_JM_NK
    vals[4 * NW + w] = u2;                  // IM_JK_NL
    vals[5 * NW + w] = mul_phase(u2, v1);   // IM_JL_NK
  }
}

// One field P for P_i and P_j (the proton's two u quarks), with perm1 free of
// fixed points (Gamma_ij = C g5 and most others): the wedge E[i][x][n] =
// P[i][x] ^ P[perm1 i][n] is also the wedge of slot (perm1 i, n, x), and with
// one field the second triangle pass equals the first.  So eight threads per
// site, thread (i, x) with i < perm1 i, form the 32 distinct wedges once and
// each wedge serves two slots:
//   own slot (i, x, n):           target (i, l = perm2 x), m = n  -- as pass 1 above
//   partner slot (perm1 i, n, x): target (perm1 i, perm2 n), m = x -- the N blocks
//                                 and coefficients of pass 2 above
// Both targets feed all four triangle types (IK_JM_NL with the Gamma_ij phase
// row of P_i first, IM_JK_NL with the transposed row; the Gamma_kl^T variants
// by the sign i^v1 as above); the n = l wedge gives the loop values of both
// targets.  Per site: 32 wedges + 128 dots + 16 loop dots (2 592 complex FMA
// with two two-term projectors) instead of the one-pass form's 64 + 128 + 32
// (3 744).
template <class R, class S, int NW, bool PHASED>
__device__ __forceinline__ void shared_wedge_same_loop(const BaryonSpin<R> &b, const cx<R> (&a)[9], const S *Pjj,
                                                       const S *Nl, const S *const (&Nx)[NW], const S *q, S *lps,
                                                       int l, uint32_t lph, cx<R> (&s1)[NW], cx<R> (&s2)[NW])
{
  const CliffordSet<R> &cl = b.cl;
  const int ng = cl.ng;
#pragma unroll 1
  for (int mm = 0; mm < 4; ++mm) {
    const int n = (l + mm) & 3;
    cx<R> e[9];
    {
      cx<R> bn[9];
      load9(bn, Pjj + n * 9);
#pragma unroll
      for (int k = 0; k < 9; ++k) e[k] = czero<R>();
      wedge_acc(e, a, bn);
    }
    if (mm == 0) {  // n = l: the loop wedge of (i, l) and of the partner target (j, x)
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        cx<R> qw[9];
        load9(qw, q + w * 9);
        const cx<R> sq = dot9(e, qw);
        const cx<R> lv = cadd(sq, mul_phase(sq, lph));  // own phase factored out: 1 + i^(partner - own)
        lps[w] = S {lv.x, lv.y};
      }
    }
    const int ln = b.perm2[n];
    const uint32_t q0 = b.ph2[0][ln];
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      if (k < ng) {
        cx<R> nn[9];
        load9(nn, Nl + cl.perm[k][n] * 36);  // own slot
        const cx<R> d = dot9(e, nn);
        s1[k] = cadd(s1[k], PHASED ? mul_phase(d, cl.ph[k][n]) : d);
        load9(nn, Nx[k] + ln * 9);  // partner slot
        s2[k] = cadd(s2[k], mul_phase(dot9(e, nn), q0));
      }
    }
  }
}

template <class R, class S, int NW>
__device__ __forceinline__ void fused_shared_wedge_same_site(const BaryonSpin<R> &b, const S *P, const S *N,
                                                             const S *q, int sub, cx<R> *vals)
{
  const CliffordSet<R> &cl = b.cl;
  const int i = (sub >> 2) == 0 ? 0 : (b.perm1[0] == 1 ? 2 : 1);  // the two rows with i < perm1 i
  const int x = sub & 3;
  const int j = b.perm1[i];
  const int l = b.perm2[x];
  const int ng = cl.ng;
  cx<R> a[9];
  load9(a, P + (i * 4 + x) * 9);
  S *lps = const_cast<S *>(q) + 9 * NW + sub * NW;  // loop values, parked in shared memory
  const S *Nx[NW];
#pragma unroll
  for (int k = 0; k < NW; ++k) Nx[k] = N + (k < ng ? cl.perm[k][x] : 0) * 36;
  cx<R> s1[NW], s2[NW];
#pragma unroll
  for (int k = 0; k < NW; ++k) s1[k] = s2[k] = czero<R>();
  const uint32_t own = (b.ph1[0][i] + b.ph2[0][l]) & 3u;   // IK_JM_NL / loop phase of target (i, l)
  const uint32_t part = (b.ph1[0][j] + b.ph2[0][x]) & 3u;  // loop phase of the partner target (j, x)
  if (cl.has_phase[0] || cl.has_phase[1])
    shared_wedge_same_loop<R, S, NW, true>(b, a, P + j * 36, N + l * 9, Nx, q, lps, l, (part - own) & 3u, s1, s2);
  else
    shared_wedge_same_loop<R, S, NW, false>(b, a, P + j * 36, N + l * 9, Nx, q, lps, l, (part - own) & 3u, s1, s2);
  // the IM_* group takes the transposed Gamma_ij phase row: a fixed offset per row
  const uint32_t di = (b.ph1[1][i] - b.ph1[0][i]) & 3u, dj = (b.ph1[1][j] - b.ph1[0][j]) & 3u;
  const uint32_t v1 = (b.ph2[1][0] - b.ph2[0][0]) & 3u;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    cx<R> u1 = czero<R>(), u2 = czero<R>();
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      if (k < ng) {
        cfma(u1, cx<R> {cl.coef[w][k][0], cl.coef[w][k][1]}, s1[k]);
        cfma(u2, cx<R> {cl.qc[w][k][x][0], cl.qc[w][k][x][1]}, s2[k]);
      }
    }
    const cx<R> o1 = mul_phase(u1, own);   // target (i, l)
    const cx<R> o2 = mul_phase(u2, b.ph1[0][j]);  // target (j, perm2 n): its column phase is already in s2
    const cx<R> lv = mul_phase(cx<R> {lps[w].x, lps[w].y}, own);
    const cx<R> t1 = cadd(o1, o2);
    const cx<R> t2 = cadd(mul_phase(o1, di), mul_phase(o2, dj));
    vals[0 * NW + w] = lv;                  // IK_JL_NM
    vals[2 * NW + w] = mul_phase(lv, v1);   // IL_JK_NM
    vals[1 * NW + w] = t1;                  // IK_JM_NL
    vals[3 * NW + w] = mul_phase(t1, v1);   // IL_JM_NK
    vals[4 * NW + w] = t2;                  // IM_JK_NL
    vals[5 * NW + w] = mul_phase(t2, v1);   // IM_JL_NK
  }
}

// ------------------------------------------------------------------ ops --
// Common compile-time configuration of an op: CW consumer warps (plus one
// producer warp), TPS threads per site, NST ring stages.
template <class R_, class S_, int CW_, int TPS_, int NST_> struct OpBase {
  using R = R_;
  using S = S_;
  using Params = OpParams<R_>;
  static constexpr int CW = CW_, TPS = TPS_, NST = NST_;
  static constexpr int SITES = CW_ * (32 / TPS_);
  static constexpr int THREADS = 32 * (CW_ + 1);
  // Field ops: true when site() stores its outputs to global memory itself
  // (the engine then passes the destination, or nullptr for a site to skip).
  static constexpr bool DIRECT_OUT = false;
  // Resident CTAs per SM that the launch bounds ask for (0: the engine's rule).
  static constexpr int MIN_CTAS = 0;
  static_assert(32 % TPS_ == 0, "a site's threads must sit in one warp");
};

// Bytes of n complex values of storage type S, rounded up to 16.
template <class S> constexpr int cbytes(int n) { return (int)((n * sizeof(S) + 15) / 16 * 16); }

// One baryon contraction type per launch, loop form (IK_JL_NM, IL_JK_NM).
template <class R, class S, int CW, int TPS, int NST>
struct BaryonLoopOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 3, NOUT = 1, EXTRA_BYTES = cbytes<S>(9);
  static constexpr bool FIELD = false;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, cx<R> *vals)
  {
    build_q<R, S, TPS, 1>(p.b, in[2], scratch, sub);
    __syncwarp();
    loop_site<R, S, TPS, 1, 1>(p.b, in[0], in[1], scratch, sub, 0, vals);
  }
};

// One baryon contraction type per launch, triangle form (the other four
// types), with N' = W N materialised per site (any 4x4 projector).
template <class R, class S, int CW, int TPS, int NST>
struct BaryonTriOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 3, NOUT = 1, EXTRA_BYTES = cbytes<S>(144) + 16;  // +16: bank stagger
  static constexpr bool FIELD = false;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, cx<R> *vals)
  {
    build_nprime<R, S, TPS, 1>(p.b, in[2], scratch, sub, p.b.cl.ng <= kNprimeCliffTerms);
    __syncwarp();
    triangle_site<R, S, TPS, 1, 1>(p.b, in[0], in[1], scratch, sub, 0, vals);
  }
};

// Triangle form, one type per launch, with W of rank <= 2 (e.g. (1 +- g4)/2,
// rank 2; a polarised projector, rank 1): X_r and Y_r blocks in scratch.
template <class R, class S, int CW, int TPS, int NST>
struct BaryonTriRankOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 3, NOUT = 1, EXTRA_BYTES = cbytes<S>(144) + 16;  // +16: bank stagger
  static constexpr bool FIELD = false;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, cx<R> *vals)
  {
    build_rank<R, S, TPS>(p.b.rk, in[1], in[2], nullptr, scratch, sub);
    __syncwarp();
    triangle_rank_site<R, S, TPS, 1>(p.b, in[0], scratch, scratch + 72, sub, 0, vals);
  }
};

// Triangle form, one type per launch, with W a combination of few gamma
// matrices (always one for baryon_two_point): no N' buffer.
template <class R, class S, int CW, int TPS, int NST>
struct BaryonTriCliffOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 3, NOUT = 1, EXTRA_BYTES = 0;
  static constexpr bool FIELD = false;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *, int sub, cx<R> *vals)
  {
    triangle_cliff_site<R, S, TPS, 1, 1>(p.b, in[0], in[1], in[2], sub, 0, vals);
  }
};

// All six types x NW projectors in one pass over (P_i, P_j, P_n), projectors
// in the gamma basis (e.g. (1 +- g4)/2 = (Gamma(0) +- Gamma(8))/2).
// Output o = type * NW + w, types in contract_enum.h order.
template <class R, class S, int CW, int TPS, int NST, int NW>
struct BaryonFusedCliffOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 3, NOUT = 6 * NW, EXTRA_BYTES = cbytes<S>(9 * NW);
  static constexpr bool FIELD = false;
  static_assert(TPS == 16, "one (i, l) pair per thread");
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, cx<R> *vals)
  {
    build_q_cliff<R, S, TPS, NW>(p.b, in[2], scratch, sub);
    __syncwarp();
    const int i = sub >> 2, l = sub & 3;
    cx<R> t[2 * NW], lp[2 * NW];
    // IK_JM_NL, IL_JM_NK, with IK_JL_NM, IL_JK_NM folded into the first wedge
    fused_triangle_pass<R, S, NW, true>(p.b, in[0], in[1], in[2], scratch, i, l, 0, t, lp);
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      vals[0 * NW + w] = lp[0 * NW + w];
      vals[2 * NW + w] = lp[1 * NW + w];
      vals[1 * NW + w] = t[0 * NW + w];
      vals[3 * NW + w] = t[1 * NW + w];
    }
    fused_triangle_pass<R, S, NW, false>(p.b, in[1], in[0], in[2], scratch, i, l, 1, t, lp);  // IM_JK_NL, IM_JL_NK
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      vals[4 * NW + w] = t[0 * NW + w];
      vals[5 * NW + w] = t[1 * NW + w];
    }
  }
};

// The same six types x NW projectors with both triangle passes in one m loop
// (fused_merged_site): fewer N loads, more live registers.
template <class R, class S, int CW, int TPS, int NST, int NW, int MINB = 0, bool SAMEIJ = false>
struct BaryonFusedCliffMergedOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 3, NOUT = 6 * NW, EXTRA_BYTES = cbytes<S>(9 * NW + 16 * 2 * NW);
  static constexpr bool FIELD = false;
  static constexpr int MIN_CTAS = MINB;
  static_assert(TPS == 16, "one (i, l) pair per thread");
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, cx<R> *vals)
  {
    build_q_cliff<R, S, TPS, NW>(p.b, in[2], scratch, sub);
    __syncwarp();
    fused_merged_site<R, S, NW, SAMEIJ>(p.b, in[0], in[1], in[2], scratch, sub >> 2, sub & 3, vals);
  }
};

// The same six types x NW projectors with every wedge shared by both triangle
// passes (fused_shared_wedge_site): a third fewer FMAs than the merged form.
template <class R, class S, int CW, int TPS, int NST, int NW, int MINB = 0>
struct BaryonFusedSharedWedgeOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 3, NOUT = 6 * NW, EXTRA_BYTES = cbytes<S>(9 * NW + 16 * NW);
  static constexpr bool FIELD = false;
  static constexpr int MIN_CTAS = MINB;
  static_assert(TPS == 16, "one (i, x) pair per thread");
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, cx<R> *vals)
  {
    build_q_cliff<R, S, TPS, NW>(p.b, in[2], scratch, sub);
    __syncwarp();
    fused_shared_wedge_site<R, S, NW>(p.b, in[0], in[1], in[2], scratch, sub >> 2, sub & 3, vals);
  }
};

// One field for P_i and P_j and perm1 without fixed points: eight threads per
// site, each wedge serving two slots (fused_shared_wedge_same_site).  Two
// inputs, in[0] = P and in[1] = P_n: the field is staged once per site.
template <class R, class S, int CW, int NST, int NW, int MINB = 0>
struct BaryonFusedSharedWedgeSameOp : OpBase<R, S, CW, 8, NST> {
  static constexpr int NIN = 2, NOUT = 6 * NW, EXTRA_BYTES = cbytes<S>(9 * NW + 8 * NW);
  static constexpr bool FIELD = false;
  // Four sites share a warp here.  Their threads load colour blocks 4 i + x
  // (x = 0..3, two rows i), 8-byte values at block * 72 bytes: with 1168-byte
  // slots the next site's blocks land 16 bytes on, in banks the first site's
  // blocks already use; 1184-byte slots move them 32 bytes on, clear of those.
  static constexpr int SLOT_PAD = 32;
  static constexpr int MIN_CTAS = MINB;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, cx<R> *vals)
  {
    build_q_cliff<R, S, 8, NW>(p.b, in[1], scratch, sub);
    __syncwarp();
    fused_shared_wedge_same_site<R, S, NW>(p.b, in[0], in[1], scratch, sub, vals);
  }
};

// All six types for one projector of rank <= 2 that is not one gamma matrix
// (e.g. (1 + g4)/2 alone): the loop types through Q, the triangle types through
// the factored form, with X_r from P_j for the first triangle pass and from P_i
// for the swapped one, Y_r from P_n shared by both.  Output o = type.
template <class R, class S, int CW, int TPS, int NST>
struct BaryonFusedRankOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 3, NOUT = 6, EXTRA_BYTES = cbytes<S>(216) + cbytes<S>(9);
  static constexpr bool FIELD = false;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, cx<R> *vals)
  {
    S *q = scratch + 216;  // after the 24 X, Y, X' blocks
    build_q<R, S, TPS, 1>(p.b, in[2], q, sub);
    build_rank<R, S, TPS>(p.b.rk, in[1], in[2], in[0], scratch, sub);
    __syncwarp();
    cx<R> t[2];
    loop_site<R, S, TPS, 2, 1>(p.b, in[0], in[1], q, sub, 0, t);  // IK_JL_NM, IL_JK_NM
    vals[0] = t[0];
    vals[2] = t[1];
    triangle_rank_site<R, S, TPS, 2>(p.b, in[0], scratch, scratch + 72, sub, 0, t);  // IK_JM_NL, IL_JM_NK
    vals[1] = t[0];
    vals[3] = t[1];
    triangle_rank_site<R, S, TPS, 2>(p.b, in[1], scratch + 144, scratch + 72, sub, 1, t);  // IM_JK_NL, IM_JL_NK
    vals[4] = t[0];
    vals[5] = t[1];
  }
};

// All six types x NW projectors with N'_w = W_w N materialised per site
// (projectors that are not short gamma-basis combinations).
template <class R, class S, int CW, int TPS, int NST, int NW>
struct BaryonFusedOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 3, NOUT = 6 * NW, EXTRA_BYTES = cbytes<S>(144) * NW + cbytes<S>(9 * NW);
  static constexpr bool FIELD = false;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, cx<R> *vals)
  {
    S *q = reinterpret_cast<S *>(reinterpret_cast<char *>(scratch) + cbytes<S>(144) * NW);
    build_nprime<R, S, TPS, NW>(p.b, in[2], scratch, sub, p.b.cl.ng <= kNprimeCliffTerms);
    build_q<R, S, TPS, NW>(p.b, in[2], q, sub);
    __syncwarp();
    cx<R> t[2 * NW];
    loop_site<R, S, TPS, 2, NW>(p.b, in[0], in[1], q, sub, 0, t);  // IK_JL_NM, IL_JK_NM
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      vals[0 * NW + w] = t[0 * NW + w];
      vals[2 * NW + w] = t[1 * NW + w];
    }
    triangle_site<R, S, TPS, 2, NW>(p.b, in[0], in[1], scratch, sub, 0, t);  // IK_JM_NL, IL_JM_NK
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      vals[1 * NW + w] = t[0 * NW + w];
      vals[3 * NW + w] = t[1 * NW + w];
    }
    triangle_site<R, S, TPS, 2, NW>(p.b, in[1], in[0], scratch, sub, 1, t);  // IM_JK_NL, IM_JL_NK
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      vals[4 * NW + w] = t[0 * NW + w];
      vals[5 * NW + w] = t[1 * NW + w];
    }
  }
};

// Meson two-point: C = sum_{i,l} c1(i) c2(l) sum_ad A[i][perm2 l][ad] conj(B[perm1 i][l][ad])
// with c from (g5 Gamma)^T (include/meson.cuh:33-50).
template <class R, class S, int CW, int TPS, int NST>
struct MesonOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 2, NOUT = 1, EXTRA_BYTES = 0;
  static constexpr bool FIELD = false;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *, int sub, cx<R> *vals)
  {
    using Ln = Lanes<TPS>;
    const MesonSpin<R> &m = p.m;
    const int i = sub / Ln::TPI, l0 = (sub % Ln::TPI) * Ln::LPT;
    const int j = m.perm1[i];
    cx<R> acc = czero<R>();
#pragma unroll
    for (int lo = 0; lo < Ln::LPT; ++lo) {
      const int l = l0 + lo;
      const S *x = in[0] + (i * 4 + m.perm2[l]) * 9;
      const S *y = in[1] + (j * 4 + l) * 9;
      cx<R> t = czero<R>();
#pragma unroll
      for (int k = 0; k < 9; ++k) cfma_conj(t, ld<R>(x + k), ld<R>(y + k));
      acc = cadd(acc, mul_phase(t, m.ph2[l]));
    }
    vals[0] = mul_phase(acc, m.ph1[i]);
  }
};

// x . conj(y) over a colour block.  Complex64: packed FP32x2 FMAs on two
// accumulators, A = sum x.re y and B = sum x.im y (y as a pair, x broadcast),
// then (A.x + B.y, B.x - A.y): no operand needs reordering.
template <class R> __device__ __forceinline__ cx<R> conj_dot9(const cx<R> x[9], const cx<R> y[9])
{
  cx<R> t = czero<R>();
#pragma unroll
  for (int e = 0; e < 9; ++e) cfma_conj(t, x[e], y[e]);
  return t;
}
template <> __device__ __forceinline__ cx<float> conj_dot9<float>(const cx<float> x[9], const cx<float> y[9])
{
  float2 A = make_float2(0.f, 0.f), B = A;
#pragma unroll
  for (int e = 0; e < 9; ++e) {
    const float2 yv = make_float2(y[e].x, y[e].y);
    A = __ffma2_rn(yv, bcast2(x[e].x), A);
    B = __ffma2_rn(yv, bcast2(x[e].y), B);
  }
  return {A.x + B.y, B.x - A.y};
}

template <class R> __device__ __forceinline__ cx<R> pick4(const cx<R> t[4], int k)
{
  return k == 0 ? t[0] : (k == 1 ? t[1] : (k == 2 ? t[2] : t[3]));
}

// meson_all_source_two_point: Gamma_ij fixed (perm1/ph1), all 16 Gamma_kl.
// Thread = spin row i (TPS = 4); the 4 x 4 colour dots T[k][l] for j = perm1[i]
// are shared by all 16 outputs (include/meson_all.cuh:53-73 recomputes them per Gamma).
template <class R, class S, int CW, int NST>
struct MesonAllSourceOp : OpBase<R, S, CW, 4, NST> {
  static constexpr int NIN = 2, NOUT = 16, EXTRA_BYTES = 0;
  static constexpr bool FIELD = false;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *, int sub, cx<R> *vals)
  {
    constexpr GammaTables G = build_gamma_tables();
    const int i = sub, j = p.m.perm1[i];
#pragma unroll
    for (int g = 0; g < 16; ++g) vals[g] = czero<R>();
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      cx<R> t[4], y[9];
      if (l & 1) load9p<true>(y, in[1] + (j * 4 + l) * 9);  // block parity = parity of l
      else load9p<false>(y, in[1] + (j * 4 + l) * 9);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        cx<R> x[9];
        if (k & 1) load9p<true>(x, in[0] + (i * 4 + k) * 9);
        else load9p<false>(x, in[0] + (i * 4 + k) * 9);
        t[k] = conj_dot9<R>(x, y);
      }
#pragma unroll
      for (int g = 0; g < 16; ++g) vals[g] = cadd(vals[g], mul_phase(pick4(t, G.perm[g][l]), G.ph_g5g_t[g][l]));
    }
    const uint32_t p1 = p.m.ph1[i];
#pragma unroll
    for (int g = 0; g < 16; ++g) vals[g] = mul_phase(vals[g], p1);
  }
};

// meson_all_sink_two_point: Gamma_kl fixed (perm2/ph2), all 16 Gamma_ij.
// Thread = spin column l (TPS = 4).
template <class R, class S, int CW, int NST>
struct MesonAllSinkOp : OpBase<R, S, CW, 4, NST> {
  static constexpr int NIN = 2, NOUT = 16, EXTRA_BYTES = 0;
  static constexpr bool FIELD = false;
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *, int sub, cx<R> *vals)
  {
    constexpr GammaTables G = build_gamma_tables();
    const int l = sub, k = p.m.perm2[l];
#pragma unroll
    for (int g = 0; g < 16; ++g) vals[g] = czero<R>();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      cx<R> t[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        cx<R> x[9], y[9];
        load9(x, in[0] + (i * 4 + k) * 9);
        load9(y, in[1] + (j * 4 + l) * 9);
        t[j] = conj_dot9<R>(x, y);
      }
#pragma unroll
      for (int g = 0; g < 16; ++g) vals[g] = cadd(vals[g], mul_phase(pick4(t, G.perm[g][i]), G.ph_g5g_t[g][i]));
    }
    const uint32_t p2 = p.m.ph2[l];
#pragma unroll
    for (int g = 0; g < 16; ++g) vals[g] = mul_phase(vals[g], p2);
  }
};

// ----------------------------------------------------------- field ops --
// Diquark (include/diquark.cuh:33-57):
//   D[m][l][ad] = g5[m] g5[l] conj( c2(l) sum_i c1(i) (P_i[i][perm2 l] ^ P_j[perm1 i][m])[ad] )
// with c1 from Gamma_ij, c2 from Gamma_kl^T.  Thread handles 16/TPS blocks (m, l).
template <class R, class S, int CW, int TPS, int NST, bool DIRECT = false>
struct DiquarkOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 2, EXTRA_BYTES = 0, OUT_ELEMS = 144;
  static constexpr bool FIELD = true;
  // DIRECT: each thread stores its blocks straight to HBM (72 contiguous bytes
  // a block) instead of staging the site in shared memory for a bulk store.
  static constexpr bool DIRECT_OUT = DIRECT;
  __device__ static long long out_index(const OpParams<R> &, long long site) { return site; }
  __device__ static S *out_ptr(const OpParams<R> &, long long d, S *base) { return base + d * OUT_ELEMS; }
  __device__ static void site(const OpParams<R> &p, const S *const *in, S *, int sub, S *out)
  {
    const BaryonSpin<R> &b = p.b;
    if (!out) return;  // a site past the end of the tile (no cross-thread work below)
    for (int blk = sub; blk < 16; blk += TPS) {
      const int m = blk / 4, l = blk % 4, k = b.perm2[l];
      cx<R> d[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) d[e] = czero<R>();
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        cx<R> x[9], y[9];
        load9(x, in[0] + (i * 4 + k) * 9);
        load9(y, in[1] + (b.perm1[i] * 4 + m) * 9);
        phase9(x, b.ph1[0][i]);
        wedge_acc(d, x, y);
      }
      // g5[m] g5[l] = -1 when exactly one of m, l is a lower spin component.
      const uint32_t sgn = ((m >> 1) ^ (l >> 1)) & 1u;
      const uint32_t p2 = b.ph2[0][l];
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        cx<R> v = conj(mul_phase(d[e], p2));
        v.x = flip_sign(v.x, sgn);
        v.y = flip_sign(v.y, sgn);
        st(out + blk * 9 + e, v);
      }
    }
  }
};

// Sequential source: the slot's propagator is overwritten with dC/dP_slot
// (include/baryon_sequential.cuh:36-163).  With the canonical forms above,
// A/B/N denote the roles; `role` is which one is differentiated.  Inputs are
// the two other roles in (A, B, N) order.  W is always a Gamma matrix here.
//   loop, d/dA[i][perm2 l] = c1 c2 (B[perm1 i][l] ^ Q)
//   loop, d/dB[perm1 i][l] = c1 c2 (A[i][perm2 l] ^ Q)
//   loop, d/dN[perm(m)][m] = W[m][perm m] * sum_{i,l} c1 c2 (A ^ B)
//   tri,  d/dA[i][perm2 l] = c1 c2 sum_m B[perm1 i][m] ^ N'[m][l]
//   tri,  d/dB[perm1 i][m] = c1 sum_l c2 (A[i][perm2 l] ^ N'[m][l])
//   tri,  d/dN[perm(m)][l] = W[m][perm m] sum_i c1 c2 (A[i][perm2 l] ^ B[perm1 i][m])
template <class R, class S, int CW, int TPS, int NST, bool LOOP, int ROLE>
struct SequentialOp : OpBase<R, S, CW, TPS, NST> {
  static constexpr int NIN = 2, EXTRA_BYTES = cbytes<S>(144) + 16, OUT_ELEMS = 144;
  static constexpr bool FIELD = true;
  __device__ static long long out_index(const OpParams<R> &, long long site) { return site; }
  __device__ static S *out_ptr(const OpParams<R> &, long long d, S *base) { return base + d * OUT_ELEMS; }

  __device__ static void site(const OpParams<R> &p, const S *const *in, S *scratch, int sub, S *out)
  {
    const BaryonSpin<R> &b = p.b;
    const ProjOperand<R> &pw = b.proj[0];
    const S *A = ROLE == 0 ? nullptr : in[0];
    const S *B = ROLE == 1 ? nullptr : (ROLE == 0 ? in[0] : in[1]);
    const S *N = ROLE == 2 ? nullptr : in[1];
    if constexpr (LOOP && ROLE != 2) {
      build_q<R, S, TPS, 1>(b, N, scratch, sub);
      __syncwarp();
    }
    if constexpr (!LOOP && ROLE != 2) {
      build_nprime<R, S, TPS, 1>(b, N, scratch, sub);
      __syncwarp();
    }
    if constexpr (LOOP && ROLE == 2) {
      // R = sum_{i,l} c1 c2 (A ^ B): each thread its (i, l) share, then a group sum.
      using Ln = Lanes<TPS>;
      const int i = sub / Ln::TPI, l0 = (sub % Ln::TPI) * Ln::LPT, j = b.perm1[i];
      cx<R> r[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) r[e] = czero<R>();
#pragma unroll
      for (int lo = 0; lo < Ln::LPT; ++lo) {
        const int l = l0 + lo;
        cx<R> x[9], y[9];
        load9(x, A + (i * 4 + b.perm2[l]) * 9);
        load9(y, B + (j * 4 + l) * 9);
        phase9(x, (b.ph1[0][i] + b.ph2[0][l]) & 3u);
        wedge_acc(r, x, y);
      }
#pragma unroll
      for (int e = 0; e < 9; ++e) r[e] = group_sum<TPS>(r[e]);
      // out[n][m] = W[m][n] R for n = perm(m); every other block is zero.
      for (int blk = sub; blk < 16; blk += TPS) {
        const int n = blk / 4, m = blk % 4;
        const bool hit = pw.perm[m] == n;
        if (!out) continue;  // a site past the end of the tile
#pragma unroll
        for (int e = 0; e < 9; ++e) st(out + blk * 9 + e, hit ? mul_phase(r[e], pw.ph[m]) : czero<R>());
      }
    } else {
      field_blocks(b, pw, A, B, scratch, sub, out);
    }
  }

  __device__ static void field_blocks(const BaryonSpin<R> &b, const ProjOperand<R> &pw, const S *A, const S *B,
                                      const S *scratch, int sub, S *out)
  {
    if (!out) return;  // a site past the end of the tile (no cross-thread work below)
    for (int blk = sub; blk < 16; blk += TPS) {
      cx<R> d[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) d[e] = czero<R>();
      int dst;
      if constexpr (LOOP) {
        cx<R> q[9];
        load9(q, scratch);
        if constexpr (ROLE == 0) {  // block (i, k), k = perm2 l
          const int i = blk / 4, k = blk % 4, l = b.perm2[k], j = b.perm1[i];
          cx<R> y[9];
          load9(y, B + (j * 4 + l) * 9);
          phase9(y, (b.ph1[0][i] + b.ph2[0][l]) & 3u);
          wedge_acc(d, y, q);
        } else {  // block (j, l), i = perm1 j
          const int j = blk / 4, l = blk % 4, i = b.perm1[j];
          cx<R> x[9];
          load9(x, A + (i * 4 + b.perm2[l]) * 9);
          phase9(x, (b.ph1[0][i] + b.ph2[0][l]) & 3u);
          wedge_acc(d, x, q);
        }
        dst = blk;
      } else if constexpr (ROLE == 0) {  // block (i, k)
        const int i = blk / 4, k = blk % 4, l = b.perm2[k], j = b.perm1[i];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          cx<R> y[9], nn[9];
          load9(y, B + (j * 4 + m) * 9);
          load9(nn, scratch + (m * 4 + l) * 9);
          wedge_acc(d, y, nn);
        }
        phase9(d, (b.ph1[0][i] + b.ph2[0][l]) & 3u);
        dst = blk;
      } else if constexpr (ROLE == 1) {  // block (j, m), i = perm1 j
        const int j = blk / 4, m = blk % 4, i = b.perm1[j];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          cx<R> x[9], nn[9];
          load9(x, A + (i * 4 + b.perm2[l]) * 9);
          phase9(x, b.ph2[0][l]);
          load9(nn, scratch + (m * 4 + l) * 9);
          wedge_acc(d, x, nn);
        }
        phase9(d, b.ph1[0][i]);
        dst = blk;
      } else {  // ROLE 2, triangle: block (n, l), n = perm(m)
        const int n = blk / 4, l = blk % 4, m = pw.perm[n];  // perm is an involution
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          cx<R> x[9], y[9];
          load9(x, A + (i * 4 + b.perm2[l]) * 9);
          load9(y, B + (b.perm1[i] * 4 + m) * 9);
          phase9(x, b.ph1[0][i]);
          wedge_acc(d, x, y);
        }
        phase9(d, (b.ph2[0][l] + pw.ph[m]) & 3u);
        dst = blk;
      }
#pragma unroll
      for (int e = 0; e < 9; ++e) st(out + dst * 9 + e, d[e]);
    }
  }
};

// All 16 x 16 meson gamma pairs per site, C[a][b] = meson_two_point(Gamma_a, Gamma_b)
// (include/meson.cuh:33-50 for every pair), written as a 256-entry block per
// site in lexicographic site order ((t*Lz + z)*Ly + y)*Lx + x for the
// momentum projection.  Every Gamma permutes spin rows by XOR with a class
// s = perm(0) in {0,1,2,3}.  Thread (s, i) of a site computes the 16 colour
// dots T[k][l] = P_i[i][k] . conj(P_j[i^s][l]) -- the 256 dots of the site
// exactly once -- then
//   V[b] = sum_l c_b(l) T[l ^ s_b][l]                    (all 16 Gamma_b)
//   C[a][b] += c_a(i) V[b]   for the four Gamma_a of class s,
// summed over the four threads i by a halving shuffle exchange.
// The permutation of every Gamma(n) is r -> r ^ s for its class s, and
// within a class the (g5 Gamma(a))^T row phases factor as
//   ph(a, r) = beta_s(r) + alpha_a + 2 popcount(h_a & r)  (mod 4)
// with h_a running over 0..3 (Walsh functions).  Hence the sum over spin
// rows r of the four members of a class is one phase i^beta per row and a
// four-point Walsh-Hadamard transform across the rows' threads, followed by
// i^alpha per member.  ClassWalsh holds, per (class s, Walsh index h), the
// member a and alpha, and beta per (s, r); built and checked at compile time.
// T[k][l] = sum_e x_k[e] conj(y_l[e]) for the four colour blocks x_k = xr[9k..]
// and y_l = yr[9l..] of one spin row each, with packed FP32x2 FMAs (two lanes
// of one instruction: (re, im) += (a.x, a.y) b.x and (a.y, -a.x) b.y), which
// halves the issue slots of the products.  Colour index outermost, so only
// one colour of each block is live; per element the FMA order is that of
// cfma_conj, so the sums are the same to the bit.
// NK consecutive colour blocks of the spin row (xr[9k..] for k < NK): the
// half-row form serves a site split over two threads.  NL < 4 takes the
// first NL blocks of yr.
template <int NK, int NL = 4>
__device__ __forceinline__ void conj_products_f32x2(cx<float> (&T)[NK][NL], const float2 *xr, const float2 *yr)
{
  float2 acc[NK][NL];
#pragma unroll
  for (int k = 0; k < NK; ++k)
#pragma unroll
    for (int l = 0; l < NL; ++l) acc[k][l] = make_float2(0.f, 0.f);
#pragma unroll 3  // fully unrolled, the loads of later colours run ahead and spill at 128 registers
  for (int e = 0; e < 9; ++e) {
    float2 a[NK], ar[NK], b[NL];
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      a[k] = xr[k * 9 + e];
      ar[k] = make_float2(a[k].y, -a[k].x);
    }
#pragma unroll
    for (int l = 0; l < NL; ++l) b[l] = yr[l * 9 + e];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const float2 bx = make_float2(b[l].x, b[l].x), by = make_float2(b[l].y, b[l].y);
#pragma unroll
      for (int k = 0; k < NK; ++k) {
        acc[k][l] = __ffma2_rn(a[k], bx, acc[k][l]);
        acc[k][l] = __ffma2_rn(ar[k], by, acc[k][l]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < NK; ++k)
#pragma unroll
    for (int l = 0; l < NL; ++l) T[k][l] = {acc[k][l].x, acc[k][l].y};
}

struct ClassWalsh {
  uint32_t beta;     // 2 bits per (s, r), index 4 s + r
  uint64_t member;   // 4 bits per (s, h), index 4 s + h
  uint32_t alpha;    // 2 bits per (s, h)
  bool ok;
};
CGB_HD constexpr ClassWalsh class_walsh()
{
  constexpr GammaTables G = build_gamma_tables();
  ClassWalsh w {0u, 0ull, 0u, true};
  for (int s = 0; s < 4; ++s) {
    int base = -1, seen = 0;
    for (int a = 0; a < 16; ++a) {
      if (G.perm[a][0] != s) continue;
      for (int r = 0; r < 4; ++r)
        if (G.perm[a][r] != (r ^ s)) w.ok = false;
      if (base < 0) {
        base = a;
        for (int r = 0; r < 4; ++r) w.beta |= (uint32_t)G.ph_g5g_t[a][r] << (2 * (4 * s + r));
      }
      int d[4] = {0, 0, 0, 0};
      for (int r = 0; r < 4; ++r) d[r] = (G.ph_g5g_t[a][r] - G.ph_g5g_t[base][r] + 4) & 3;
      const int alpha = d[0];
      const int h0 = ((d[1] - alpha + 4) & 3) >> 1, h1 = ((d[2] - alpha + 4) & 3) >> 1;
      for (int r = 0; r < 4; ++r) {
        const int pc = ((r & 1) & h0) + (((r >> 1) & 1) & h1);
        if (d[r] != ((alpha + 2 * pc) & 3)) w.ok = false;
      }
      const int h = h0 | (h1 << 1);
      if (seen & (1 << h)) w.ok = false;
      seen |= 1 << h;
      w.member |= (uint64_t)a << (4 * (4 * s + h));
      w.alpha |= (uint32_t)alpha << (2 * (4 * s + h));
    }
    if (seen != 15) w.ok = false;
  }
  return w;
}
static_assert(class_walsh().ok, "gamma classes must have the Walsh phase structure");

// SPLIT selects the layout [t][pair half][site][128 pairs] (pairs 0-127 and
// 128-255 of a timeslice in separate planes) that the tensor-core projection
// streams as contiguous 8-site tiles; otherwise [t][site][256 pairs].
// PRODUCTS (complex64): store the 256 spin-colour products
//   T[i][j][k][l] = sum_c S1[i][k][c] conj(S2[j][l][c])
// instead of the Gamma pairs, product (i, j = i ^ s, k, l) at index
// (4 k + l) * 16 + 4 s + i.  Each pair is a signed sum of 16 products, the same
// at every site, so a linear consumer (the momentum projection) forms the pairs
// once from its sums (pair_from_products in kernels_momentum.cu).
template <class R, class S, int CW, int NST, bool SPLIT = false, bool PRODUCTS = false>
struct MesonAllGammaOp : OpBase<R, S, CW, 16, NST> {
  static constexpr int NIN = 2, EXTRA_BYTES = 0, OUT_ELEMS = 256;
  static constexpr bool FIELD = true;
  static_assert(!PRODUCTS || sizeof(R) == 4, "the product form is complex64 only");
  // Each thread's 16 outputs are four 32-byte runs: stored straight to HBM.
  static constexpr bool DIRECT_OUT = true;

  __device__ static long long sites_per_slice(const OpParams<R> &p)
  {
    return (long long)p.latt[0] * p.latt[1] * p.latt[2];
  }
  // Destination of site `d` (lexicographic index, 0 <= d < volume): the start
  // of its 256 pairs, or with SPLIT of its first 128 (the second 128 follow
  // one timeslice plane later).
  __device__ static S *out_ptr(const OpParams<R> &p, long long d, S *base)
  {
    if constexpr (SPLIT) {
      const long long v3 = sites_per_slice(p), t = d / v3;
      return base + (d + t * v3) * 128;
    } else {
      return base + d * OUT_ELEMS;
    }
  }

  __device__ static long long out_index(const OpParams<R> &p, long long site)
  {
    const long long lx = p.latt[0], ly = p.latt[1], lz = p.latt[2], lt = p.latt[3];
    if (lx < 2 || ly < 1 || lz < 1 || lt < 1) return -1;  // no lattice: the engine skips and reports
    const long long half = lx / 2;
    long long r = site / half;
    const long long xh = site - r * half;
    const long long y = r % ly;
    r /= ly;
    const long long z = r % lz;
    r /= lz;
    const long long t = r % lt, par = r / lt;
    const long long x = 2 * xh + ((par + t + z + y) & 1);
    return ((t * lz + z) * ly + y) * lx + x;
  }


  __device__ static void site(const OpParams<R> &ps_, const S *const *in, S *, int sub, S *out)
  {
    constexpr GammaTables G = build_gamma_tables();
    constexpr ClassWalsh CW8 = class_walsh();
    const int s = sub >> 2, i = sub & 3, j = i ^ s;
    cx<R> T[4][4];
    if constexpr (sizeof(R) == 4) {
      conj_products_f32x2(T, in[0] + i * 36, in[1] + j * 36);
      if constexpr (PRODUCTS) {
        if (!out) return;
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
          for (int l = 0; l < 4; ++l) {
            const int g = (k * 4 + l) * 16 + sub;
            S *dst;
            if constexpr (SPLIT) dst = out + (g >> 7) * sites_per_slice(ps_) * 128 + (g & 127);
            else dst = out + g;
            *dst = S {T[k][l].x, T[k][l].y};
          }
        return;
      }
    } else {
      // Block (i, k) has the parity of k and block (j, l) that of l, so every
      // colour block loads as 16-byte vectors.
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        cx<R> x[9];
        if (k & 1) load9p<true>(x, in[0] + (i * 4 + k) * 9);
        else load9p<false>(x, in[0] + (i * 4 + k) * 9);
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          cx<R> y[9];
          if (l & 1) load9p<true>(y, in[1] + (j * 4 + l) * 9);
          else load9p<false>(y, in[1] + (j * 4 + l) * 9);
          cx<R> t = czero<R>();
#pragma unroll
          for (int e = 0; e < 9; ++e) cfma_conj(t, x[e], y[e]);
          T[k][l] = t;
        }
      }
    }
    // V[b] = i^beta_s(i) sum_l (g5 Gamma(b))^T-phase(l) T[perm_b(l)][l]
    const uint32_t beta = (CW8.beta >> (2 * (4 * s + i))) & 3u;
    cx<R> V[16];
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      cx<R> v = czero<R>();
#pragma unroll
      for (int l = 0; l < 4; ++l) v = cadd(v, mul_phase(T[G.perm[b][l]][l], G.ph_g5g_t[b][l]));
      V[b] = mul_phase(v, beta);
    }
    // Walsh-Hadamard over the row bits of i (lanes ^1, ^2), reduce-scattering b:
    // this thread ends with X[h][kk] for b = 8 i0 + 4 i1 + kk.
    const uint32_t i0 = i & 1, i1 = (i >> 1) & 1;
    cx<R> Y0[8], Y1[8];  // Walsh bit h0 = 0, 1 for b in [8 i0, 8 i0 + 8)
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const cx<R> own = i0 ? V[8 + k] : V[k], send = i0 ? V[k] : V[8 + k];
      const cx<R> recv = shfl_xor(send, 1);
      Y0[k] = cadd(own, recv);
      const cx<R> d = {own.x - recv.x, own.y - recv.y};
      Y1[k] = {flip_sign(d.x, i0), flip_sign(d.y, i0)};
    }
    cx<R> X[4][4];
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
      for (int h0 = 0; h0 < 2; ++h0) {
        const cx<R> *Y = h0 ? Y1 : Y0;
        const cx<R> own = i1 ? Y[4 + kk] : Y[kk], send = i1 ? Y[kk] : Y[4 + kk];
        const cx<R> recv = shfl_xor(send, 2);
        X[h0][kk] = cadd(own, recv);
        const cx<R> d = {own.x - recv.x, own.y - recv.y};
        X[2 + h0][kk] = {flip_sign(d.x, i1), flip_sign(d.y, i1)};
      }
    }
    const int b0 = 8 * i0 + 4 * i1;
    if (!out) return;  // a site past the end of the tile (the shuffles above still ran)
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int idx = 4 * s + h;
      const int a = (int)((CW8.member >> (4 * idx)) & 15u);
      const uint32_t alpha = (CW8.alpha >> (2 * idx)) & 3u;
      S *dst;  // 32-byte aligned
      if constexpr (SPLIT) dst = out + (a >> 3) * sites_per_slice(ps_) * 128 + (a & 7) * 16 + b0;
      else dst = out + a * 16 + b0;
      st2(dst, mul_phase(X[h][0], alpha), mul_phase(X[h][1], alpha));
      st2(dst + 2, mul_phase(X[h][2], alpha), mul_phase(X[h][3], alpha));
    }
  }
};

} // namespace cgb
