/*
 * Plain-C FP64 restatement of CLQCD/contract's per-site contractions.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for the CUDA path and the CPU
 * baseline timed by bench.py.  Nothing in the product links or calls it.
 *
 * It restates the reference's per-site algorithm -- a loop over the 16 spin
 * pairs (i, l) with j = perm(Gamma_ij, i), k = perm(Gamma_kl, l), and an
 * epsilon-epsilon colour contraction per (a, d) -- in C99 complex arithmetic:
 *   meson_local            include/meson.cuh:33-50
 *   meson all-gamma loops  include/meson_all.cuh:53-103
 *   baryon_local           include/baryon.cuh:34-83 (+ load swap :95-105)
 *   baryon_general_local   include/baryon_general.cuh:36-93
 *   diquark_local          include/diquark.cuh:33-57
 *   baryon_sequential      include/baryon_sequential.cuh:36-163, restated as
 *                          the gradient dC(x)/dP_slot(x) it equals.
 * The gamma index/phase tables are derived at load time from the four
 * DeGrand-Rossi gamma matrices, not copied.
 *
 * Sites are independent; OpenMP parallelises over them.
 */
#include <complex.h>
#include <stddef.h>
#include <string.h>

typedef double _Complex cplx;

#define SITE 144 /* 4 x 4 spin x 3 x 3 colour */

/* ---------------------------------------------------------------- gamma -- */

static int g_index[16][4];       /* column of the nonzero entry of row r     */
static cplx g_data[16][4];       /* Gamma[r][g_index[r]]                     */
static cplx g_mat[16][4][4];     /* dense Gamma(n)                           */
static int g_ready = 0;

static void matmul4(cplx out[4][4], cplx a[4][4], cplx b[4][4])
{
  cplx t[4][4];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      cplx s = 0;
      for (int k = 0; k < 4; ++k) s += a[r][k] * b[k][c];
      t[r][c] = s;
    }
  memcpy(out, t, sizeof(t));
}

static void gamma_init(void)
{
  if (g_ready) return;
  /* Euclidean DeGrand-Rossi basis. */
  cplx g[4][4][4];
  memset(g, 0, sizeof(g));
  g[0][0][3] = I; g[0][1][2] = I; g[0][2][1] = -I; g[0][3][0] = -I;   /* gamma_1 */
  g[1][0][3] = -1; g[1][1][2] = 1; g[1][2][1] = 1; g[1][3][0] = -1;   /* gamma_2 */
  g[2][0][2] = I; g[2][1][3] = -I; g[2][2][0] = -I; g[2][3][1] = I;   /* gamma_3 */
  g[3][0][2] = 1; g[3][1][3] = 1; g[3][2][0] = 1; g[3][3][1] = 1;     /* gamma_4 */
  for (int n = 0; n < 16; ++n) {
    cplx m[4][4];
    memset(m, 0, sizeof(m));
    for (int r = 0; r < 4; ++r) m[r][r] = 1;
    for (int bit = 0; bit < 4; ++bit)
      if ((n >> bit) & 1) matmul4(m, m, g[bit]);
    memcpy(g_mat[n], m, sizeof(m));
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c)
        if (cabs(m[r][c]) > 0.5) {
          g_index[n][r] = c;
          g_data[n][r] = m[r][c];
        }
  }
  g_ready = 1;
}

void oracle_gamma_tables(int *index, cplx *data)
{
  gamma_init();
  for (int n = 0; n < 16; ++n)
    for (int r = 0; r < 4; ++r) {
      index[n * 4 + r] = g_index[n][r];
      data[n * 4 + r] = g_data[n][r];
    }
}

/* ------------------------------------------------------ colour helpers -- */

/* (x ^ y)[a][d] = sum_{b,c,e,f} eps_abc eps_def x[b][e] y[c][f] for one (a, d):
 * the same four products the reference sums per (a, d). */
static inline cplx wedge_ad(const cplx *x, const cplx *y, int a, int d)
{
  const int b = (a + 1) % 3, c = (a + 2) % 3, e = (d + 1) % 3, f = (d + 2) % 3;
  return (x[3 * b + e] * y[3 * c + f] + x[3 * c + f] * y[3 * b + e]) -
         (x[3 * c + e] * y[3 * b + f] + x[3 * b + f] * y[3 * c + e]);
}

static inline const cplx *blk(const cplx *p, int s0, int s1) { return p + (s0 * 4 + s1) * 9; }
static inline cplx *blkw(cplx *p, int s0, int s1) { return p + (s0 * 4 + s1) * 9; }

/* ------------------------------------------------------------- mesons -- */

/* (g5 Gamma)^T [r][perm(r)] = g5[c][c] Gamma[c][r] with c = perm(r): the
 * coefficient meson_local applies (g5 = diag(1, 1, -1, -1)). */
static inline cplx g5g_t(int g, int r)
{
  const int c = g_index[g][r];
  return (c < 2 ? 1.0 : -1.0) * g_mat[g][c][r];
}

static inline cplx meson_site(const cplx *pi, const cplx *pj, int gij, int gkl)
{
  cplx acc = 0;
  for (int i = 0; i < 4; ++i)
    for (int l = 0; l < 4; ++l) {
      const int j = g_index[gij][i], k = g_index[gkl][l];
      const cplx c = g5g_t(gij, i) * g5g_t(gkl, l);
      const cplx *x = blk(pi, i, k), *y = blk(pj, j, l);
      cplx t = 0;
      for (int ad = 0; ad < 9; ++ad) t += x[ad] * conj(y[ad]);
      acc += c * t;
    }
  return acc;
}

void oracle_meson_two_point(cplx *correl, const cplx *pi, const cplx *pj, size_t volume, int gamma_ij,
                            int gamma_kl)
{
  gamma_init();
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x) correl[x] = meson_site(pi + x * SITE, pj + x * SITE, gamma_ij, gamma_kl);
}

void oracle_meson_all_source(cplx *correl, const cplx *pi, const cplx *pj, size_t volume, int gamma_ij)
{
  gamma_init();
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x)
    for (int g = 0; g < 16; ++g) correl[g * volume + x] = meson_site(pi + x * SITE, pj + x * SITE, gamma_ij, g);
}

void oracle_meson_all_sink(cplx *correl, const cplx *pi, const cplx *pj, size_t volume, int gamma_kl)
{
  gamma_init();
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x)
    for (int g = 0; g < 16; ++g) correl[g * volume + x] = meson_site(pi + x * SITE, pj + x * SITE, g, gamma_kl);
}

/* ------------------------------------------------------------ baryons -- */

/* Contraction-type structure (contract_enum.h:1-8).  Types 0 and 2 contract
 * P_n with itself through the Gamma_mn operand; types 1, 3, 4, 5 form a spin
 * triangle.  IM_* types exchange the roles of P_i and P_j; IL_* / IM_JL_*
 * types use Gamma_kl transposed (baryon.cuh:43-51). */
static inline int type_loop(int t) { return t == 0 || t == 2; }
static inline int type_swap_ij(int t) { return t == 4 || t == 5; }
static inline int type_swap_kl(int t) { return t == 2 || t == 3 || t == 5; }

/* Coefficient of Gamma (or Gamma^T when transpose) on row r at its nonzero column. */
static inline cplx gcoef(int g, int r, int transpose)
{
  const int c = g_index[g][r];
  return transpose ? g_mat[g][c][r] : g_mat[g][r][c];
}

/* w[m][n]: the Gamma_mn operand as the kernel weights P_n[n][m] (type 0/2)
 * or eps(P_j[j][m], P_n[n][l]) (types 1/3/4/5).  Zero entries are skipped. */
static cplx baryon_site(const cplx *pi, const cplx *pj, const cplx *pn, int type, int gij, int gkl,
                        const cplx w[4][4])
{
  const int sij = type_swap_ij(type), skl = type_swap_kl(type);
  const cplx *pa = sij ? pj : pi, *pb = sij ? pi : pj;
  cplx acc = 0;
  for (int i = 0; i < 4; ++i)
    for (int l = 0; l < 4; ++l) {
      const int j = g_index[gij][i], k = g_index[gkl][l];
      const cplx c = gcoef(gij, i, sij) * gcoef(gkl, l, !skl);
      const cplx *a_ik = blk(pa, i, k);
      for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d) {
          const int ad = 3 * a + d;
          cplx tmp = 0;
          if (type_loop(type)) {
            for (int n = 0; n < 4; ++n)
              for (int m = 0; m < 4; ++m)
                if (w[m][n] != 0) tmp += w[m][n] * blk(pn, n, m)[ad];
            acc += c * tmp * wedge_ad(a_ik, blk(pb, j, l), a, d);
          } else {
            for (int n = 0; n < 4; ++n)
              for (int m = 0; m < 4; ++m)
                if (w[m][n] != 0) tmp += w[m][n] * wedge_ad(blk(pb, j, m), blk(pn, n, l), a, d);
            acc += c * tmp * a_ik[ad];
          }
        }
    }
  return acc;
}

void oracle_baryon_general(cplx *correl, const cplx *pi, const cplx *pj, const cplx *pn, int type, size_t volume,
                           int gamma_ij, int gamma_kl, const cplx *w_nm)
{
  gamma_init();
  cplx w[4][4]; /* w[m][n] = operand[m][n] */
  for (int m = 0; m < 4; ++m)
    for (int n = 0; n < 4; ++n) w[m][n] = w_nm[m * 4 + n];
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x)
    correl[x] = baryon_site(pi + x * SITE, pj + x * SITE, pn + x * SITE, type, gamma_ij, gamma_kl, w);
}

void oracle_baryon_two_point(cplx *correl, const cplx *pi, const cplx *pj, const cplx *pn, int type, size_t volume,
                             int gamma_ij, int gamma_kl, int gamma_mn)
{
  gamma_init();
  oracle_baryon_general(correl, pi, pj, pn, type, volume, gamma_ij, gamma_kl, &g_mat[gamma_mn][0][0]);
}

/* ------------------------------------------------------------ diquark -- */

void oracle_baryon_diquark(cplx *diquark, const cplx *pi, const cplx *pj, size_t volume, int gamma_ij, int gamma_kl)
{
  gamma_init();
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x) {
    const cplx *a = pi + x * SITE, *b = pj + x * SITE;
    cplx *out = diquark + x * SITE;
    for (int m = 0; m < 4; ++m)
      for (int l = 0; l < 4; ++l) {
        const int k = g_index[gamma_kl][l];
        const cplx ckl = gcoef(gamma_kl, l, 1);
        const double s = ((m >> 1) ^ (l >> 1)) ? -1.0 : 1.0; /* g5[m][m] g5[l][l] */
        for (int ad = 0; ad < 9; ++ad) {
          cplx tmp = 0;
          for (int i = 0; i < 4; ++i) {
            const int j = g_index[gamma_ij][i];
            tmp += gcoef(gamma_ij, i, 0) * wedge_ad(blk(a, i, k), blk(b, j, m), ad / 3, ad % 3);
          }
          blkw(out, m, l)[ad] = s * conj(ckl * tmp);
        }
      }
  }
}

/* --------------------------------------------------------- sequential -- */

/* out += c * (x ^ y) over all (a, d). */
static inline void wedge_acc(cplx *out, cplx c, const cplx *x, const cplx *y)
{
  for (int ad = 0; ad < 9; ++ad) out[ad] += c * wedge_ad(x, y, ad / 3, ad % 3);
}

/* dC(x)/dP_slot(x) for one site; `out` (144 complex) is fully written.
 * The baryon is trilinear in (P_a, P_b, P_n) through eps.eps, which is
 * symmetric in its three colour matrices, so the derivative with respect to
 * one operand is the colour wedge of the other two. */
static void sequential_site(cplx *out, const cplx *pi, const cplx *pj, const cplx *pn, int type, int slot, int gij,
                            int gkl, const cplx w[4][4])
{
  const int sij = type_swap_ij(type), skl = type_swap_kl(type);
  const cplx *pa = sij ? pj : pi, *pb = sij ? pi : pj;
  /* which operand the slot is: 0 = A (P_i, or P_j when swapped), 1 = B, 2 = P_n */
  const int op = slot == 2 ? 2 : ((slot == 0) != sij ? 0 : 1);
  memset(out, 0, sizeof(cplx) * SITE);
  cplx q[9] = {0};
  if (type_loop(type))
    for (int n = 0; n < 4; ++n)
      for (int m = 0; m < 4; ++m)
        if (w[m][n] != 0)
          for (int ad = 0; ad < 9; ++ad) q[ad] += w[m][n] * blk(pn, n, m)[ad];
  for (int i = 0; i < 4; ++i)
    for (int l = 0; l < 4; ++l) {
      const int j = g_index[gij][i], k = g_index[gkl][l];
      const cplx c = gcoef(gij, i, sij) * gcoef(gkl, l, !skl);
      if (type_loop(type)) {
        /* C += c F(A_ik, B_jl, Q),  Q = sum w[m][n] P_n[n][m] */
        if (op == 0) wedge_acc(blkw(out, i, k), c, blk(pb, j, l), q);
        else if (op == 1) wedge_acc(blkw(out, j, l), c, blk(pa, i, k), q);
        else {
          cplx r[9] = {0};
          wedge_acc(r, c, blk(pa, i, k), blk(pb, j, l));
          for (int n = 0; n < 4; ++n)
            for (int m = 0; m < 4; ++m)
              if (w[m][n] != 0)
                for (int ad = 0; ad < 9; ++ad) blkw(out, n, m)[ad] += w[m][n] * r[ad];
        }
      } else {
        /* C += c w[m][n] F(A_ik, B_jm, P_n[n][l]) */
        for (int n = 0; n < 4; ++n)
          for (int m = 0; m < 4; ++m) {
            if (w[m][n] == 0) continue;
            const cplx cw = c * w[m][n];
            if (op == 0) wedge_acc(blkw(out, i, k), cw, blk(pb, j, m), blk(pn, n, l));
            else if (op == 1) wedge_acc(blkw(out, j, m), cw, blk(pa, i, k), blk(pn, n, l));
            else wedge_acc(blkw(out, n, l), cw, blk(pa, i, k), blk(pb, j, m));
          }
      }
    }
}

void oracle_baryon_sequential(cplx *pi, cplx *pj, cplx *pn, int type, int slot, size_t volume, int gamma_ij,
                              int gamma_kl, int gamma_mn)
{
  gamma_init();
  cplx w[4][4];
  for (int m = 0; m < 4; ++m)
    for (int n = 0; n < 4; ++n) w[m][n] = g_mat[gamma_mn][m][n];
  cplx *target = slot == 0 ? pi : (slot == 1 ? pj : pn);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x) {
    cplx out[SITE];
    sequential_site(out, pi + x * SITE, pj + x * SITE, pn + x * SITE, type, slot, gamma_ij, gamma_kl, w);
    memcpy(target + x * SITE, out, sizeof(out));
  }
}
