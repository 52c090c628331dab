// All six baryon contraction types (x up to two projectors) in one pass.
// Template arguments: <R, S, consumer warps, threads per site, ring stages, projectors>.
#include "launch_impl.cuh"

namespace cgb {

using Fused1P = BaryonFusedOp<double, double2, 4, 16, 2, 1>;
using Fused2P = BaryonFusedOp<double, double2, 4, 16, 2, 2>;
using Fused1M = BaryonFusedOp<float, float2, 8, 16, 2, 1>;
using Fused2M = BaryonFusedOp<float, float2, 8, 16, 2, 2>;

cudaError_t launch_baryon_fused(const Job &job, int nw, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) return nw == 1 ? run_scalar<Fused1P>(job, p) : run_scalar<Fused2P>(job, p);
  const OpParams<float> q = convert_params<float>(p);
  return nw == 1 ? run_scalar<Fused1M>(job, q) : run_scalar<Fused2M>(job, q);
}

} // namespace cgb
