// Export the reference's gamma switch tables (include/gamma.cuh:58-127,225-271)
// so the oracle's derived tables can be pinned bit-exactly.
#include <gamma.cuh>
#include "ref_common.h"

extern "C" void ref_gamma_tables(int *index, cplx *data, cplx *data_t, cplx *g_g5, cplx *g5_g_t)
{
  using contract::Complex;
  for (int g = 0; g < 16; ++g) {
    for (int r = 0; r < 4; ++r) {
      int o = g * 4 + r;
      index[o] = contract::gamma_index(g, r);
      Complex<double> v = contract::gamma_data<false, double>(g, r);
      data[o] = cplx(v.real(), v.imag());
      v = contract::gamma_data<true, double>(g, r);
      data_t[o] = cplx(v.real(), v.imag());
      v = contract::gamma_gamma5_data<false, double>(g, r);
      g_g5[o] = cplx(v.real(), v.imag());
      v = contract::gamma_gamma5_data<true, double>(g, r);
      g5_g_t[o] = cplx(v.real(), v.imag());
    }
  }
}
