// Baryon two-point kernels, one contraction type per launch.
// Template arguments: <R, S, consumer warps, threads per site, ring stages>.
#include "launch_impl.cuh"

namespace cgb {

// complex128 (FP64-pipe bound): 8 sites per tile, one (i, l) spin pair per thread.
using LoopP = BaryonLoopOp<double, double2, 4, 16, 3>;
using TriP = BaryonTriOp<double, double2, 4, 16, 3>;
using TriCliffP = BaryonTriCliffOp<double, double2, 4, 16, 3>;
// complex64: 14 sites per tile, two CTAs (14 consumer warps) per SM.
using LoopM = BaryonLoopOp<float, float2, 7, 16, 2>;
using TriM = BaryonTriOp<float, float2, 7, 16, 3>;
using TriCliffM = BaryonTriCliffOp<float, float2, 7, 16, 2>;

cudaError_t launch_baryon(const Job &job, bool loop, const OpParams<double> &p)
{
  // A projector that is one gamma matrix (baryon_two_point) needs no N' buffer.
  const bool cliff = p.b.cl.ng == 1;
  if (job.prec == Prec::C128) {
    if (loop) return run_scalar<LoopP>(job, p);
    return cliff ? run_scalar<TriCliffP>(job, p) : run_scalar<TriP>(job, p);
  }
  const OpParams<float> q = convert_params<float>(p);
  if (loop) return run_scalar<LoopM>(job, q);
  return cliff ? run_scalar<TriCliffM>(job, q) : run_scalar<TriM>(job, q);
}

} // namespace cgb
