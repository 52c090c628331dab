// Baryon two-point kernels, one contraction type per launch.
// Op template arguments: <R, S, consumer warps, threads per site, ring stages>.
#include "launch_variants.cuh"

namespace cgb {

// complex128 (FP64-pipe bound), one (i, l) spin pair per thread: four consumer
// warps and three ring stages (one CTA per SM: 8 sites x 3 inputs x 2 320 B per
// stage), or smaller tiles and rings so that two or three CTAs fit.  The
// default (used with autotuning off) is three consumer warps and two stages,
// the tuner's choice at 24^3 x 64.
static const VariantSet<double, 4> kLoopP = {
  {run_scalar<BaryonLoopOp<double, double2, 4, 16, 3>>, run_scalar<BaryonLoopOp<double, double2, 3, 16, 2>>,
   run_scalar<BaryonLoopOp<double, double2, 2, 16, 3>>, run_scalar<BaryonLoopOp<double, double2, 2, 16, 2>>},
  {"cw4.tps16.st3", "cw3.tps16.st2", "cw2.tps16.st3", "cw2.tps16.st2"},
  1};
static const VariantSet<double, 4> kTriP = {
  {run_scalar<BaryonTriOp<double, double2, 4, 16, 3>>, run_scalar<BaryonTriOp<double, double2, 3, 16, 2>>,
   run_scalar<BaryonTriOp<double, double2, 2, 16, 3>>, run_scalar<BaryonTriOp<double, double2, 2, 16, 2>>},
  {"cw4.tps16.st3", "cw3.tps16.st2", "cw2.tps16.st3", "cw2.tps16.st2"},
  1};
static const VariantSet<double, 4> kTriRankP = {
  {run_scalar<BaryonTriRankOp<double, double2, 4, 16, 3>>, run_scalar<BaryonTriRankOp<double, double2, 3, 16, 2>>,
   run_scalar<BaryonTriRankOp<double, double2, 2, 16, 3>>, run_scalar<BaryonTriRankOp<double, double2, 2, 16, 2>>},
  {"cw4.tps16.st3", "cw3.tps16.st2", "cw2.tps16.st3", "cw2.tps16.st2"},
  1};
static const VariantSet<double, 4> kTriCliffP = {
  {run_scalar<BaryonTriCliffOp<double, double2, 4, 16, 3>>, run_scalar<BaryonTriCliffOp<double, double2, 3, 16, 2>>,
   run_scalar<BaryonTriCliffOp<double, double2, 2, 16, 3>>, run_scalar<BaryonTriCliffOp<double, double2, 2, 16, 2>>},
  {"cw4.tps16.st3", "cw3.tps16.st2", "cw2.tps16.st3", "cw2.tps16.st2"},
  1};

// complex64 variants: sites per tile x ring depth x CTAs per SM; the default
// (last field) is the tuner's choice at 24^3 x 64.
static const VariantSet<float, 4> kLoopM = {
  {run_scalar<BaryonLoopOp<float, float2, 7, 16, 2>>, run_scalar<BaryonLoopOp<float, float2, 5, 16, 3>>,
   run_scalar<BaryonLoopOp<float, float2, 4, 8, 3>>, run_scalar<BaryonLoopOp<float, float2, 3, 16, 3>>},
  {"cw7.tps16.st2", "cw5.tps16.st3", "cw4.tps8.st3", "cw3.tps16.st3"},
  3};
// General projector (N' materialised per site).
static const VariantSet<float, 4> kTriM = {
  {run_scalar<BaryonTriOp<float, float2, 6, 16, 2>>, run_scalar<BaryonTriOp<float, float2, 7, 16, 3>>,
   run_scalar<BaryonTriOp<float, float2, 4, 16, 3>>, run_scalar<BaryonTriOp<float, float2, 3, 16, 2>>},
  {"cw6.tps16.st2", "cw7.tps16.st3", "cw4.tps16.st3", "cw3.tps16.st2"},
  3};
// Projector of rank <= 2 (X_r, Y_r blocks per site).
static const VariantSet<float, 5> kTriRankM = {
  {run_scalar<BaryonTriRankOp<float, float2, 3, 16, 2>>, run_scalar<BaryonTriRankOp<float, float2, 4, 16, 3>>,
   run_scalar<BaryonTriRankOp<float, float2, 6, 16, 2>>, run_scalar<BaryonTriRankOp<float, float2, 7, 16, 2>>,
   run_scalar<BaryonTriRankOp<float, float2, 4, 8, 2>>},
  {"cw3.tps16.st2", "cw4.tps16.st3", "cw6.tps16.st2", "cw7.tps16.st2", "cw4.tps8.st2"},
  0};
static const VariantSet<float, 5> kTriCliffM = {
  {run_scalar<BaryonTriCliffOp<float, float2, 7, 16, 2>>, run_scalar<BaryonTriCliffOp<float, float2, 5, 16, 3>>,
   run_scalar<BaryonTriCliffOp<float, float2, 4, 8, 2>>, run_scalar<BaryonTriCliffOp<float, float2, 3, 16, 2>>,
   run_scalar<BaryonTriCliffOp<float, float2, 4, 16, 3>>},
  {"cw7.tps16.st2", "cw5.tps16.st3", "cw4.tps8.st2", "cw3.tps16.st2", "cw4.tps16.st3"},
  3};

cudaError_t launch_baryon(const Job &job, bool loop, const OpParams<double> &p)
{
  // A projector that is one gamma matrix (baryon_two_point) needs no N' buffer;
  // one of rank <= 2 takes the factored form.
  const bool cliff = p.b.cl.ng == 1, rank = !cliff && p.b.rk.r > 0;
  if (job.prec == Prec::C128) {
    if (loop) return kLoopP.launch(job, p);
    if (rank) return kTriRankP.launch(job, p);
    return cliff ? kTriCliffP.launch(job, p) : kTriP.launch(job, p);
  }
  const OpParams<float> q = convert_params<float>(p);
  if (loop) return kLoopM.launch(job, q);
  if (rank) return kTriRankM.launch(job, q);
  return cliff ? kTriCliffM.launch(job, q) : kTriM.launch(job, q);
}

// form: 0 loop, 1 triangle with one gamma, 2 triangle with N' materialised,
// 3 triangle with a projector of rank <= 2.
int baryon_variants(Prec prec, int form, const char *const **names)
{
  if (prec == Prec::C128) {
    if (form == 0) return kLoopP.describe(names);
    if (form == 3) return kTriRankP.describe(names);
    return form == 1 ? kTriCliffP.describe(names) : kTriP.describe(names);
  }
  if (form == 0) return kLoopM.describe(names);
  if (form == 3) return kTriRankM.describe(names);
  return form == 1 ? kTriCliffM.describe(names) : kTriM.describe(names);
}

} // namespace cgb
