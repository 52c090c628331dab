// Meson kernels: one Gamma pair per site, and the all-source / all-sink forms.
#include "launch_impl.cuh"

namespace cgb {

// complex128: FP64-pipe bound, 64 threads x 16 sites per tile.
using MesonP = MesonOp<double, double2, 16, 4, 3>;
// complex64: HBM bound, 128 threads x 16 sites, 4-deep ring.
using MesonM = MesonOp<float, float2, 16, 8, 4>;
using MesonAllSrcP = MesonAllSourceOp<double, double2, 16, 2>;
using MesonAllSnkP = MesonAllSinkOp<double, double2, 16, 2>;
using MesonAllSrcM = MesonAllSourceOp<float, float2, 16, 4>;
using MesonAllSnkM = MesonAllSinkOp<float, float2, 16, 4>;

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
