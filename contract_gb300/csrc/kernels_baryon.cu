// Baryon two-point kernels, one contraction type per launch.
#include "launch_impl.cuh"

namespace cgb {

// complex128: 8 sites x 16 threads (one (i, l) spin pair per thread).
using LoopP = BaryonLoopOp<double, double2, 8, 16, 3>;
using TriP = BaryonTriOp<double, double2, 8, 16, 3>;
// complex64: 16 sites x 8 threads (spin row i, two columns per thread).
using LoopM = BaryonLoopOp<float, float2, 16, 8, 3>;
using TriM = BaryonTriOp<float, float2, 16, 8, 3>;

cudaError_t launch_baryon(const Job &job, bool loop, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) return loop ? run_scalar<LoopP>(job, p) : run_scalar<TriP>(job, p);
  const OpParams<float> q = convert_params<float>(p);
  return loop ? run_scalar<LoopM>(job, q) : run_scalar<TriM>(job, q);
}

} // namespace cgb
