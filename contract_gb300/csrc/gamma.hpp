// DeGrand-Rossi gamma algebra as exact signed permutations (host + device).
//
// Every product of gamma matrices has exactly one nonzero entry per row, and
// that entry is a power of i.  A matrix is therefore stored as
//     M[r][perm[r]] = i^ph[r]      (perm a permutation of 0..3, ph in 0..3)
// and products/transposes are computed with integer arithmetic only, so the
// tables are exact by construction.  The 16 matrices are
//     Gamma(n) = g1^(n&1) g2^((n>>1)&1) g3^((n>>2)&1) g4^((n>>3)&1),
// the indexing used by CLQCD/contract (include/gamma.cuh:58-127), with
// Gamma(15) = g5 = diag(1, 1, -1, -1).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define CGB_HD __host__ __device__
#else
#define CGB_HD
#endif

namespace cgb {

struct SignedPerm {
  int perm[4];
  int ph[4];
};

CGB_HD constexpr SignedPerm sp_identity() { return {{0, 1, 2, 3}, {0, 0, 0, 0}}; }

// (a b)[r][c] = a[r][pa(r)] b[pa(r)][pb(pa(r))]
CGB_HD constexpr SignedPerm sp_mul(const SignedPerm &a, const SignedPerm &b)
{
  SignedPerm o {};
  for (int r = 0; r < 4; ++r) {
    o.perm[r] = b.perm[a.perm[r]];
    o.ph[r] = (a.ph[r] + b.ph[a.perm[r]]) & 3;
  }
  return o;
}

// (a^T)[r][c] = a[c][r]: row r is nonzero at the c with perm(c) = r.
CGB_HD constexpr SignedPerm sp_transpose(const SignedPerm &a)
{
  SignedPerm o {};
  for (int c = 0; c < 4; ++c) {
    o.perm[a.perm[c]] = c;
    o.ph[a.perm[c]] = a.ph[c];
  }
  return o;
}

// Euclidean DeGrand-Rossi basis g1..g4 (mu = 0..3); phases as powers of i.
CGB_HD constexpr SignedPerm sp_basis(int mu)
{
  switch (mu) {
  case 0: return {{3, 2, 1, 0}, {1, 1, 3, 3}};  // g1: +i +i -i -i on the anti-diagonal
  case 1: return {{3, 2, 1, 0}, {2, 0, 0, 2}};  // g2: -1 +1 +1 -1 on the anti-diagonal
  case 2: return {{2, 3, 0, 1}, {1, 3, 3, 1}};  // g3: +i -i -i +i
  default: return {{2, 3, 0, 1}, {0, 0, 0, 0}}; // g4: +1 everywhere
  }
}

CGB_HD constexpr SignedPerm sp_gamma(int n)
{
  SignedPerm m = sp_identity();
  for (int mu = 0; mu < 4; ++mu)
    if ((n >> mu) & 1) m = sp_mul(m, sp_basis(mu));
  return m;
}

struct GammaTables {
  uint8_t perm[16][4];      // perm of Gamma(n) (shared by every variant below)
  uint8_t ph[16][4];        // Gamma(n)[r][perm r]
  uint8_t ph_t[16][4];      // Gamma(n)^T[r][perm r]
  uint8_t ph_g5g_t[16][4];  // (g5 Gamma(n))^T[r][perm r]
};

CGB_HD constexpr GammaTables build_gamma_tables()
{
  GammaTables t {};
  const SignedPerm g5 = sp_gamma(15);
  for (int n = 0; n < 16; ++n) {
    const SignedPerm g = sp_gamma(n);
    const SignedPerm gt = sp_transpose(g);
    const SignedPerm g5gt = sp_transpose(sp_mul(g5, g));
    for (int r = 0; r < 4; ++r) {
      t.perm[n][r] = (uint8_t)g.perm[r];
      t.ph[n][r] = (uint8_t)g.ph[r];
      t.ph_t[n][r] = (uint8_t)gt.ph[r];
      t.ph_g5g_t[n][r] = (uint8_t)g5gt.ph[r];
    }
  }
  return t;
}

// Gamma matrices are involutive permutations, so Gamma, Gamma^T and
// (g5 Gamma)^T share one permutation; these checks run at compile time.
CGB_HD constexpr bool gamma_tables_consistent()
{
  for (int n = 0; n < 16; ++n) {
    const SignedPerm g = sp_gamma(n);
    const SignedPerm gt = sp_transpose(g);
    const SignedPerm g5gt = sp_transpose(sp_mul(sp_gamma(15), g));
    for (int r = 0; r < 4; ++r)
      if (g.perm[g.perm[r]] != r || gt.perm[r] != g.perm[r] || g5gt.perm[r] != g.perm[r]) return false;
  }
  const SignedPerm g5 = sp_gamma(15);
  return g5.perm[0] == 0 && g5.perm[3] == 3 && g5.ph[0] == 0 && g5.ph[1] == 0 && g5.ph[2] == 2 && g5.ph[3] == 2;
}
static_assert(gamma_tables_consistent(), "gamma algebra tables are inconsistent");

} // namespace cgb
