// All six baryon contraction types (x up to two projectors) in one pass.
// Op template arguments: <R, S, consumer warps, threads per site, ring stages, projectors>.
#include "launch_variants.cuh"

namespace cgb {

// Projectors spanned by at most `nw` gamma matrices (e.g. (1 +- g4)/2): no N' buffers.
using FusedCliff1P = BaryonFusedCliffOp<double, double2, 4, 16, 2, 1>;
using FusedCliff2P = BaryonFusedCliffOp<double, double2, 4, 16, 2, 2>;
// complex128 runs on the FP64 pipe, so its time follows the FP64 FMA count: the
// shared-wedge forms do a third fewer (5 078 complex FMA per site with two
// two-term projectors against 7 382), and with one field for P_i and P_j the
// one-pass form about half.
// The smaller tiles let two CTAs share an SM; the default (last field) is the
// six-site tile, the tuner's choice at 24^3 x 64.
static const VariantSet<double, 3> kSharedWedge1P = {
  {run_scalar<BaryonFusedSharedWedgeOp<double, double2, 4, 16, 2, 1>>,
   run_scalar<BaryonFusedSharedWedgeOp<double, double2, 3, 16, 2, 1>>,
   run_scalar<BaryonFusedSharedWedgeOp<double, double2, 2, 16, 3, 1>>},
  {"shared.cw4.tps16.st2", "shared.cw3.tps16.st2", "shared.cw2.tps16.st3"},
  1};
static const VariantSet<double, 3> kSharedWedge2P = {
  {run_scalar<BaryonFusedSharedWedgeOp<double, double2, 4, 16, 2, 2>>,
   run_scalar<BaryonFusedSharedWedgeOp<double, double2, 3, 16, 2, 2>>,
   run_scalar<BaryonFusedSharedWedgeOp<double, double2, 2, 16, 3, 2>>},
  {"shared.cw4.tps16.st2", "shared.cw3.tps16.st2", "shared.cw2.tps16.st3"},
  1};
using SharedSame1P = BaryonFusedSharedWedgeSameOp<double, double2, 4, 2, 1>;
using SharedSame2P = BaryonFusedSharedWedgeSameOp<double, double2, 4, 2, 2>;
// General projectors: N'_w = W_w N materialised per site.
using Fused1P = BaryonFusedOp<double, double2, 4, 16, 2, 1>;
using Fused2P = BaryonFusedOp<double, double2, 4, 16, 2, 2>;
using Fused1M = BaryonFusedOp<float, float2, 8, 16, 2, 1>;
using Fused2M = BaryonFusedOp<float, float2, 8, 16, 2, 2>;
// One projector of rank <= 2 that is not one gamma matrix: factored triangles.
using FusedRank1P = BaryonFusedRankOp<double, double2, 3, 16, 2>;
using FusedRank1M = BaryonFusedRankOp<float, float2, 4, 16, 2>;

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
// second triangle pass equals the first, and only one is evaluated.  The
// shared-wedge form also forms each distinct wedge once (eight threads per
// site); it needs a Gamma_ij permutation without fixed points and takes the
// one-pass merged form otherwise.
template <class Op> cudaError_t run_same_field(const Job &job, OpParams<typename Op::R> q)
{
  using R = typename Op::R;
  if (q.b.perm1[0] == 0) {  // XOR permutations: a fixed point at 0 means the identity
    constexpr int kMinb = sizeof(R) == 4 ? 3 : 0;
    using Fallback = BaryonFusedCliffMergedOp<R, typename Op::S, 4, 16, 2, Op::NOUT / 6, kMinb, true>;
    return run_scalar<Fallback>(job, q);
  }
  q.in[1] = q.in[2];  // inputs: the field once, then P_n
  return run_scalar<Op>(job, q);
}

static const VariantSet<float, 7> kFusedCliff1MSame = {
  {run_same_field<BaryonFusedSharedWedgeSameOp<float, float2, 3, 2, 1, 3>>,
   run_same_field<BaryonFusedSharedWedgeSameOp<float, float2, 2, 2, 1, 4>>,
   run_same_field<BaryonFusedSharedWedgeSameOp<float, float2, 4, 2, 1, 2>>,
   run_same_field<BaryonFusedSharedWedgeSameOp<float, float2, 5, 2, 1, 2>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 1, 3, true>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 3, 16, 2, 1, 4, true>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 1, 0, true>>},
  {"shared_same.cw3.tps8.st2.occ3", "shared_same.cw2.tps8.st2.occ4", "shared_same.cw4.tps8.st2.occ2",
   "shared_same.cw5.tps8.st2.occ2", "same.cw4.tps16.st2.occ3", "same.cw3.tps16.st2.occ4", "same.cw4.tps16.st2"},
  0};
static const VariantSet<float, 7> kFusedCliff2MSame = {
  {run_same_field<BaryonFusedSharedWedgeSameOp<float, float2, 3, 2, 2, 3>>,
   run_same_field<BaryonFusedSharedWedgeSameOp<float, float2, 2, 2, 2, 4>>,
   run_same_field<BaryonFusedSharedWedgeSameOp<float, float2, 4, 2, 2, 2>>,
   run_same_field<BaryonFusedSharedWedgeSameOp<float, float2, 5, 2, 2, 2>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 2, 3, true>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 3, 16, 2, 2, 4, true>>,
   run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 2, 0, true>>},
  {"shared_same.cw3.tps8.st2.occ3", "shared_same.cw2.tps8.st2.occ4", "shared_same.cw4.tps8.st2.occ2",
   "shared_same.cw5.tps8.st2.occ2", "same.cw4.tps16.st2.occ3", "same.cw3.tps16.st2.occ4", "same.cw4.tps16.st2"},
  2};

// The shared-wedge forms derive the Gamma_kl^T variant of each type from the
// Gamma_kl one by the phase ph2[1] - ph2[0], which is the same in every column
// because every Gamma(n) is symmetric or antisymmetric; checked here all the same.
template <class R> static bool kl_transpose_is_sign(const OpParams<R> &q)
{
  const int d = (q.b.ph2[1][0] - q.b.ph2[0][0]) & 3;
  for (int c = 1; c < 4; ++c)
    if (((q.b.ph2[1][c] - q.b.ph2[0][c]) & 3) != d) return false;
  return d == 0 || d == 2;
}

cudaError_t launch_baryon_fused(const Job &job, int nw, const OpParams<double> &p)
{
  const bool cliff = p.b.cl.ng <= nw;
  if (nw == 1 && !cliff && p.b.rk.r > 0)
    return job.prec == Prec::C128 ? run_scalar<FusedRank1P>(job, p) : run_scalar<FusedRank1M>(job, convert_params<float>(p));
  if (job.prec == Prec::C128) {
    if (cliff && kl_transpose_is_sign(p)) {
      if (fused_same_ij(p))
        return nw == 1 ? run_same_field<SharedSame1P>(job, p) : run_same_field<SharedSame2P>(job, p);
      return nw == 1 ? kSharedWedge1P.launch(job, p) : kSharedWedge2P.launch(job, p);
    }
    if (cliff) return nw == 1 ? run_scalar<FusedCliff1P>(job, p) : run_scalar<FusedCliff2P>(job, p);
    return nw == 1 ? run_scalar<Fused1P>(job, p) : run_scalar<Fused2P>(job, p);
  }
  const OpParams<float> q = convert_params<float>(p);
  if (cliff && !kl_transpose_is_sign(q)) {  // never for DeGrand-Rossi gammas: the merged forms need no such relation
    if (fused_same_ij(p))
      return nw == 1 ? run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 1, 3, true>>(job, q)
                     : run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 2, 3, true>>(job, q);
    return nw == 1 ? run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 1, 3>>(job, q)
                   : run_scalar<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 2, 3>>(job, q);
  }
  if (cliff && fused_same_ij(p)) return nw == 1 ? kFusedCliff1MSame.launch(job, q) : kFusedCliff2MSame.launch(job, q);
  if (cliff) return nw == 1 ? kFusedCliff1M.launch(job, q) : kFusedCliff2M.launch(job, q);
  return nw == 1 ? run_scalar<Fused1M>(job, q) : run_scalar<Fused2M>(job, q);
}

// aux = nw + 4 * (P_i and P_j one field)
int fused_variants(Prec prec, int aux, const char *const **names)
{
  const int nw = aux & 3;
  // complex128: the shapes of the two-field shared-wedge form (the form the
  // launcher picks for gamma-basis projectors; the others run one shape)
  if (prec == Prec::C128) return (aux & 4) ? 1 : (nw == 1 ? kSharedWedge1P.describe(names) : kSharedWedge2P.describe(names));
  if (aux & 4) return nw == 1 ? kFusedCliff1MSame.describe(names) : kFusedCliff2MSame.describe(names);
  return nw == 1 ? kFusedCliff1M.describe(names) : kFusedCliff2M.describe(names);
}

} // namespace cgb
