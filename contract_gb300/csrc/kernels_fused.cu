// All six baryon contraction types (x up to two projectors) in one pass.
// Op template arguments: <R, S, consumer warps, threads per site, ring stages, projectors>.
#include "launch_variants.cuh"

namespace cgb {

// Projectors spanned by at most `nw` gamma matrices (e.g. (1 +- g4)/2): no N' buffers.
using FusedCliff1P = BaryonFusedCliffOp<double, double2, 4, 16, 2, 1>;
using FusedCliff2P = BaryonFusedCliffOp<double, double2, 4, 16, 2, 2>;
// General projectors: N'_w = W_w N materialised per site.
using Fused1P = BaryonFusedOp<double, double2, 4, 16, 2, 1>;
using Fused2P = BaryonFusedOp<double, double2, 4, 16, 2, 2>;
using Fused1M = BaryonFusedOp<float, float2, 8, 16, 2, 1>;
using Fused2M = BaryonFusedOp<float, float2, 8, 16, 2, 2>;

// complex64, FP32-issue bound: consumer warps per SM vs registers per thread.  The
// shared-wedge variants form each P_i ^ P_j wedge once for both triangle passes;
// the merged variants run both passes in one m loop with a wedge each.
static const VariantSet<float, 12> kFusedCliff1M = {
  {run_scalar<BaryonFusedSharedWedgeOp<float, float2, 4, 16, 2, 1, 3>>,
   run_scalar<BaryonFusedSharedWedgeOp<float, float2, 3, 16, 2, 1, 4>>,
   run_scalar<BaryonFusedSharedWedgeOp<float, float2, 5, 16, 2, 1, 2>>,
   run_scalar<BaryonFusedSharedWedgeOp<float, float2, 2, 16, 3, 1, 6>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 1, 3>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 3, 16, 2, 1, 4>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 1>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 5, 16, 2, 1>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 3, 16, 2, 1>>,
   run_scalar<BaryonFusedCliffOp<float, float2, 7, 16, 2, 1>>,
   run_scalar<BaryonFusedCliffOp<float, float2, 5, 16, 2, 1>>,
   run_scalar<BaryonFusedCliffOp<float, float2, 3, 16, 3, 1>>},
  {"shared.cw4.tps16.st2.occ3", "shared.cw3.tps16.st2.occ4", "shared.cw5.tps16.st2.occ2",
   "shared.cw2.tps16.st3.occ6", "merged.cw4.tps16.st2.occ3", "merged.cw3.tps16.st2.occ4", "merged.cw4.tps16.st2",
   "merged.cw5.tps16.st2", "merged.cw3.tps16.st2", "cw7.tps16.st2", "cw5.tps16.st2", "cw3.tps16.st3"},
  0};
static const VariantSet<float, 12> kFusedCliff2M = {
  {run_scalar<BaryonFusedSharedWedgeOp<float, float2, 4, 16, 2, 2, 3>>,
   run_scalar<BaryonFusedSharedWedgeOp<float, float2, 3, 16, 2, 2, 4>>,
   run_scalar<BaryonFusedSharedWedgeOp<float, float2, 5, 16, 2, 2, 2>>,
   run_scalar<BaryonFusedSharedWedgeOp<float, float2, 2, 16, 3, 2, 6>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 2, 3>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 3, 16, 2, 2, 4>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 2>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 5, 16, 2, 2>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 3, 16, 2, 2>>,
   run_scalar<BaryonFusedCliffOp<float, float2, 7, 16, 2, 2>>,
   run_scalar<BaryonFusedCliffOp<float, float2, 5, 16, 2, 2>>,
   run_scalar<BaryonFusedCliffOp<float, float2, 3, 16, 3, 2>>},
  {"shared.cw4.tps16.st2.occ3", "shared.cw3.tps16.st2.occ4", "shared.cw5.tps16.st2.occ2",
   "shared.cw2.tps16.st3.occ6", "merged.cw4.tps16.st2.occ3", "merged.cw3.tps16.st2.occ4", "merged.cw4.tps16.st2",
   "merged.cw5.tps16.st2", "merged.cw3.tps16.st2", "cw7.tps16.st2", "cw5.tps16.st2", "cw3.tps16.st3"},
  0};

// P_i and P_j the same field (one pointer, e.g. the u quark of a proton): the
// second triangle pass equals the first, and only one is evaluated.
static const VariantSet<float, 3> kFusedCliff1MSame = {
  {run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 1, 3, true>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 3, 16, 2, 1, 4, true>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 1, 0, true>>},
  {"same.cw4.tps16.st2.occ3", "same.cw3.tps16.st2.occ4", "same.cw4.tps16.st2"},
  0};
static const VariantSet<float, 3> kFusedCliff2MSame = {
  {run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 2, 3, true>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 3, 16, 2, 2, 4, true>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 2, 0, true>>},
  {"same.cw4.tps16.st2.occ3", "same.cw3.tps16.st2.occ4", "same.cw4.tps16.st2"},
  0};

cudaError_t launch_baryon_fused(const Job &job, int nw, const OpParams<double> &p)
{
  const bool cliff = p.b.cl.ng <= nw;
  if (job.prec == Prec::C128) {
    if (cliff) return nw == 1 ? run_scalar<FusedCliff1P>(job, p) : run_scalar<FusedCliff2P>(job, p);
    return nw == 1 ? run_scalar<Fused1P>(job, p) : run_scalar<Fused2P>(job, p);
  }
  const OpParams<float> q = convert_params<float>(p);
  if (cliff && fused_same_ij(p)) return nw == 1 ? kFusedCliff1MSame.launch(job, q) : kFusedCliff2MSame.launch(job, q);
  if (cliff) return nw == 1 ? kFusedCliff1M.launch(job, q) : kFusedCliff2M.launch(job, q);
  return nw == 1 ? run_scalar<Fused1M>(job, q) : run_scalar<Fused2M>(job, q);
}

// aux = nw + 4 * (P_i and P_j one field)
int fused_variants(Prec prec, int aux, const char *const **names)
{
  if (prec == Prec::C128) return 1;
  const int nw = aux & 3;
  if (aux & 4) return nw == 1 ? kFusedCliff1MSame.describe(names) : kFusedCliff2MSame.describe(names);
  return nw == 1 ? kFusedCliff1M.describe(names) : kFusedCliff2M.describe(names);
}

} // namespace cgb
