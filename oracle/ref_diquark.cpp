// Host build of the reference's diquark_local (include/diquark.cuh:33-57).
#include <diquark.cuh>
#include "ref_common.h"

template <int GAMMA_IJ>
static void run(cplx *diquark, const cplx *pi, const cplx *pj, std::size_t volume, int gamma_kl)
{
  using T = contract::Complex<double>;
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x) {
    auto a = reinterpret_cast<const T(*)[Nc * Nc]>(pi + x * kSite);
    auto b = reinterpret_cast<const T(*)[Nc * Nc]>(pj + x * kSite);
    T out[Ns * Ns][Nc * Nc];
    for (int idx = 0; idx < 16; ++idx) contract::diquark_local<GAMMA_IJ, double>(out, a, b, gamma_kl, idx);
    for (int s = 0; s < 16; ++s)
      for (int c = 0; c < 9; ++c) diquark[x * kSite + s * 9 + c] = cplx(out[s][c].real(), out[s][c].imag());
  }
}

extern "C" int ref_baryon_diquark(cplx *diquark, const cplx *pi, const cplx *pj, std::size_t volume, int gamma_ij,
                                  int gamma_kl)
{
  return dispatch_int<16>(gamma_ij, [&](auto g) { run<decltype(g)::value>(diquark, pi, pj, volume, gamma_kl); })
           ? 0 : -1;
}
