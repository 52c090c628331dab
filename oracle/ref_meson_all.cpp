// Host build of the reference's all-gamma meson loops (include/meson_all.cuh:53-103).
#include <meson_all.cuh>
#include "ref_common.h"

static void meson_all(cplx *correl, const cplx *pi, const cplx *pj, std::size_t volume, int gamma, bool source)
{
  using T = contract::Complex<double>;
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x) {
    auto a = reinterpret_cast<const T(*)[Nc * Nc]>(pi + x * kSite);
    auto b = reinterpret_cast<const T(*)[Nc * Nc]>(pj + x * kSite);
    for (int g = 0; g < 16; ++g) {
      T part[Ns * Ns];
      for (int idx = 0; idx < 16; ++idx) {
        if (source) contract::meson_local<double>(part, a, b, gamma, g, idx);
        else contract::meson_local<double>(part, a, b, g, gamma, idx);
      }
      T sum = part[0];
      for (int idx = 1; idx < 16; ++idx) sum += part[idx];
      correl[g * volume + x] = cplx(sum.real(), sum.imag());
    }
  }
}

extern "C" void ref_meson_all_source(cplx *correl, const cplx *pi, const cplx *pj, std::size_t volume, int gamma_ij)
{
  meson_all(correl, pi, pj, volume, gamma_ij, true);
}

extern "C" void ref_meson_all_sink(cplx *correl, const cplx *pi, const cplx *pj, std::size_t volume, int gamma_kl)
{
  meson_all(correl, pi, pj, volume, gamma_kl, false);
}
