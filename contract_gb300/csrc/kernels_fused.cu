// All six baryon contraction types (x up to two projectors) in one pass.
// Template arguments: <R, S, consumer warps, threads per site, ring stages, projectors>.
#include "launch_impl.cuh"

namespace cgb {

// Projectors spanned by at most `nw` gamma matrices (e.g. (1 +- g4)/2): no N' buffers.
using FusedCliff1P = BaryonFusedCliffOp<double, double2, 4, 16, 2, 1>;
using FusedCliff2P = BaryonFusedCliffOp<double, double2, 4, 16, 2, 2>;
using FusedCliff1M = BaryonFusedCliffOp<float, float2, 7, 16, 2, 1>;
using FusedCliff2M = BaryonFusedCliffOp<float, float2, 7, 16, 2, 2>;
// General projectors: N'_w = W_w N materialised per site.
using Fused1P = BaryonFusedOp<double, double2, 4, 16, 2, 1>;
using Fused2P = BaryonFusedOp<double, double2, 4, 16, 2, 2>;
using Fused1M = BaryonFusedOp<float, float2, 8, 16, 2, 1>;
using Fused2M = BaryonFusedOp<float, float2, 8, 16, 2, 2>;

cudaError_t launch_baryon_fused(const Job &job, int nw, const OpParams<double> &p)
{
  const bool cliff = p.b.cl.ng <= nw;
  if (job.prec == Prec::C128) {
    if (cliff) return nw == 1 ? run_scalar<FusedCliff1P>(job, p) : run_scalar<FusedCliff2P>(job, p);
    return nw == 1 ? run_scalar<Fused1P>(job, p) : run_scalar<Fused2P>(job, p);
  }
  const OpParams<float> q = convert_params<float>(p);
  if (cliff) return nw == 1 ? run_scalar<FusedCliff1M>(job, q) : run_scalar<FusedCliff2M>(job, q);
  return nw == 1 ? run_scalar<Fused1M>(job, q) : run_scalar<Fused2M>(job, q);
}

} // namespace cgb
