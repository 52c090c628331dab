// Host build of the reference's baryon_general_local (include/baryon_general.cuh:36-93),
// with the load-time i/j swap of baryon_general.cuh:101-111.
#include <baryon_general.cuh>
#include "ref_common.h"

template <BaryonContractType CONTRACT>
static void run(cplx *correl, const cplx *pi, const cplx *pj, const cplx *pn, std::size_t volume, int gamma_ij,
                int gamma_kl, const cplx *project_mn)
{
  using T = contract::Complex<double>;
  constexpr bool swap_ij = (CONTRACT == IM_JK_NL || CONTRACT == IM_JL_NK);
  T proj[16];
  for (int k = 0; k < 16; ++k) proj[k] = T(project_mn[k].real(), project_mn[k].imag());
#pragma omp parallel for schedule(static)
  for (long x = 0; x < (long)volume; ++x) {
    auto a = reinterpret_cast<const T(*)[Nc * Nc]>((swap_ij ? pj : pi) + x * kSite);
    auto b = reinterpret_cast<const T(*)[Nc * Nc]>((swap_ij ? pi : pj) + x * kSite);
    auto n = reinterpret_cast<const T(*)[Nc * Nc]>(pn + x * kSite);
    T part[Ns * Ns];
    for (int idx = 0; idx < 16; ++idx)
      contract::baryon_general_local<CONTRACT, double>(part, a, b, n, gamma_ij, gamma_kl, proj, idx);
    T sum = part[0];
    for (int idx = 1; idx < 16; ++idx) sum += part[idx];
    correl[x] = cplx(sum.real(), sum.imag());
  }
}

extern "C" int ref_baryon_general_two_point(cplx *correl, const cplx *pi, const cplx *pj, const cplx *pn,
                                            int contract_type, std::size_t volume, int gamma_ij, int gamma_kl,
                                            const cplx *project_mn)
{
  return dispatch_int<6>(contract_type, [&](auto c) {
           run<static_cast<BaryonContractType>(decltype(c)::value)>(correl, pi, pj, pn, volume, gamma_ij, gamma_kl,
                                                                    project_mn);
         }) ? 0 : -1;
}
