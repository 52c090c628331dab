// Host build of the reference's baryon_local (include/baryon.cuh:34-83).  The
// i/j operand swap of the IM_* types happens at load time in the device
// kernel (baryon.cuh:95-105) and is reproduced here.
#include <baryon.cuh>
#include "ref_common.h"

template <BaryonContractType CONTRACT, int GAMMA_MN>
static void run(cplx *correl, const cplx *pi, const cplx *pj, const cplx *pn, std::size_t volume, int gamma_ij,
                int gamma_kl)
{
  using T = contract::Complex<double>;
  constexpr bool swap_ij = (CONTRACT == IM_JK_NL || CONTRACT == IM_JL_NK);
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x) {
    auto a = reinterpret_cast<const T(*)[Nc * Nc]>((swap_ij ? pj : pi) + x * kSite);
    auto b = reinterpret_cast<const T(*)[Nc * Nc]>((swap_ij ? pi : pj) + x * kSite);
    auto n = reinterpret_cast<const T(*)[Nc * Nc]>(pn + x * kSite);
    T part[Ns * Ns];
    for (int idx = 0; idx < 16; ++idx)
      contract::baryon_local<CONTRACT, GAMMA_MN, double>(part, a, b, n, gamma_ij, gamma_kl, idx);
    T sum = part[0];
    for (int idx = 1; idx < 16; ++idx) sum += part[idx];
    correl[x] = cplx(sum.real(), sum.imag());
  }
}

extern "C" int ref_baryon_two_point(cplx *correl, const cplx *pi, const cplx *pj, const cplx *pn, int contract_type,
                                    std::size_t volume, int gamma_ij, int gamma_kl, int gamma_mn)
{
  bool ok = false;
  dispatch_int<6>(contract_type, [&](auto c) {
    ok = dispatch_int<16>(gamma_mn, [&](auto g) {
      run<static_cast<BaryonContractType>(decltype(c)::value), decltype(g)::value>(correl, pi, pj, pn, volume,
                                                                                  gamma_ij, gamma_kl);
    });
  });
  return ok ? 0 : -1;
}
