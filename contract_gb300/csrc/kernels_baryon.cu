// Baryon two-point kernels, one contraction type per launch.
// Template arguments: <R, S, consumer warps, threads per site, ring stages>.
#include "launch_impl.cuh"

namespace cgb {

// complex128: 8 sites per tile, one (i, l) spin pair per thread.
using LoopP = BaryonLoopOp<double, double2, 4, 16, 3>;
using TriP = BaryonTriOp<double, double2, 4, 16, 3>;
// complex64: 16 sites per tile, eight consumer warps.
using LoopM = BaryonLoopOp<float, float2, 8, 16, 3>;
using TriM = BaryonTriOp<float, float2, 8, 16, 3>;

cudaError_t launch_baryon(const Job &job, bool loop, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) return loop ? run_scalar<LoopP>(job, p) : run_scalar<TriP>(job, p);
  const OpParams<float> q = convert_params<float>(p);
  return loop ? run_scalar<LoopM>(job, q) : run_scalar<TriM>(job, q);
}

} // namespace cgb
