// Meson kernels: one Gamma pair per site, and the all-source / all-sink forms.
// Template arguments: <R, S, consumer warps, threads per site, ring stages>.
#include "launch_impl.cuh"

namespace cgb {

// complex128: FP64-pipe bound; 8 sites per tile, two CTAs per SM.
using MesonP = MesonOp<double, double2, 2, 8, 3>;
// complex64: HBM bound; 16 sites per tile, 4-deep ring.
using MesonM = MesonOp<float, float2, 4, 8, 4>;
using MesonAllSrcP = MesonAllSourceOp<double, double2, 1, 3>;
using MesonAllSnkP = MesonAllSinkOp<double, double2, 1, 3>;
using MesonAllSrcM = MesonAllSourceOp<float, float2, 2, 4>;
using MesonAllSnkM = MesonAllSinkOp<float, float2, 2, 4>;

cudaError_t launch_meson(const Job &job, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) return run_scalar<MesonP>(job, p);
  return run_scalar<MesonM>(job, convert_params<float>(p));
}

cudaError_t launch_meson_all(const Job &job, bool source, const OpParams<double> &p)
{
  if (job.prec == Prec::C128)
    return source ? run_scalar<MesonAllSrcP>(job, p) : run_scalar<MesonAllSnkP>(job, p);
  const OpParams<float> q = convert_params<float>(p);
  return source ? run_scalar<MesonAllSrcM>(job, q) : run_scalar<MesonAllSnkM>(job, q);
}

} // namespace cgb
