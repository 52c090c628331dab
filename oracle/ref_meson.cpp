// Host build of the reference's meson_local (include/meson.cuh:33-50): one
// call per spin pair idx = i*4+l, then the 16 partial results are summed as
// the device tile reduction does (include/load_store.cuh:50-62).
#include <meson.cuh>
#include "ref_common.h"

extern "C" void ref_meson_two_point(cplx *correl, const cplx *pi, const cplx *pj, std::size_t volume, int gamma_ij,
                                    int gamma_kl)
{
  using T = contract::Complex<double>;
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x) {
    auto a = reinterpret_cast<const T(*)[Nc * Nc]>(pi + x * kSite);
    auto b = reinterpret_cast<const T(*)[Nc * Nc]>(pj + x * kSite);
    T part[Ns * Ns];
    for (int idx = 0; idx < 16; ++idx) contract::meson_local<double>(part, a, b, gamma_ij, gamma_kl, idx);
    T sum = part[0];
    for (int idx = 1; idx < 16; ++idx) sum += part[idx];
    correl[x] = cplx(sum.real(), sum.imag());
  }
}
