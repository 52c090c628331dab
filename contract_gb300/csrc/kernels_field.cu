// Field-valued kernels: diquark and sequential sources.
// Template arguments: <R, S, consumer warps, threads per site, ring stages>.
#include "launch_impl.cuh"

namespace cgb {

template <class R, class S, int CW, int TPS>
static cudaError_t seq_dispatch(const Job &job, bool loop, int role, const OpParams<R> &p)
{
  constexpr int NST = 3;
  if (loop) {
    switch (role) {
    case 0: return run_field<SequentialOp<R, S, CW, TPS, NST, true, 0>>(job, p);
    case 1: return run_field<SequentialOp<R, S, CW, TPS, NST, true, 1>>(job, p);
    default: return run_field<SequentialOp<R, S, CW, TPS, NST, true, 2>>(job, p);
    }
  }
  switch (role) {
  case 0: return run_field<SequentialOp<R, S, CW, TPS, NST, false, 0>>(job, p);
  case 1: return run_field<SequentialOp<R, S, CW, TPS, NST, false, 1>>(job, p);
  default: return run_field<SequentialOp<R, S, CW, TPS, NST, false, 2>>(job, p);
  }
}

cudaError_t launch_diquark(const Job &job, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) return run_field<DiquarkOp<double, double2, 4, 16, 3>>(job, p);
  return run_field<DiquarkOp<float, float2, 8, 16, 3>>(job, convert_params<float>(p));
}

cudaError_t launch_sequential(const Job &job, bool loop, int role, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) return seq_dispatch<double, double2, 4, 16>(job, loop, role, p);
  return seq_dispatch<float, float2, 8, 16>(job, loop, role, convert_params<float>(p));
}

} // namespace cgb
