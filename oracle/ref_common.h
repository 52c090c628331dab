// Shared helpers for the host builds of the reference's per-site functions
// (test infrastructure only; see ref_shim/kernel.cuh).
#pragma once
#include <complex>
#include <cstddef>
#include <utility>

using cplx = std::complex<double>;

// One propagator site: [Ns*Ns][Nc*Nc] complex, i.e. 144 complex numbers.
static constexpr std::size_t kSite = 144;

// Call f(std::integral_constant<int, K>{}) for the runtime value k in [0, N).
template <int N, typename F, int... K>
inline bool dispatch_int(int k, F &&f, std::integer_sequence<int, K...>)
{
  bool hit = false;
  ((k == K ? (f(std::integral_constant<int, K> {}), hit = true) : false), ...);
  return hit;
}
template <int N, typename F> inline bool dispatch_int(int k, F &&f)
{
  return dispatch_int<N>(k, std::forward<F>(f), std::make_integer_sequence<int, N> {});
}
