// Meson kernels: one Gamma pair per site, and the all-source / all-sink forms.
// Op template arguments: <R, S, consumer warps, threads per site, ring stages>.
#include "launch_variants.cuh"

namespace cgb {

// complex128: FP64-pipe bound.  The shapes trade ring depth against CTAs per
// SM; the default is the set's last field.
static const VariantSet<double, 4> kMesonP = {
  {run_scalar<MesonOp<double, double2, 2, 8, 3>>, run_scalar<MesonOp<double, double2, 4, 8, 2>>,
   run_scalar<MesonOp<double, double2, 2, 8, 2>>, run_scalar<MesonOp<double, double2, 3, 8, 3>>},
  {"cw2.tps8.st3", "cw4.tps8.st2", "cw2.tps8.st2", "cw3.tps8.st3"},
  0};
static const VariantSet<double, 3> kMesonAllSrcP = {
  {run_scalar<MesonAllSourceOp<double, double2, 1, 3>>, run_scalar<MesonAllSourceOp<double, double2, 2, 2>>,
   run_scalar<MesonAllSourceOp<double, double2, 1, 2>>},
  {"cw1.tps4.st3", "cw2.tps4.st2", "cw1.tps4.st2"},
  1};
static const VariantSet<double, 3> kMesonAllSnkP = {
  {run_scalar<MesonAllSinkOp<double, double2, 1, 3>>, run_scalar<MesonAllSinkOp<double, double2, 2, 2>>,
   run_scalar<MesonAllSinkOp<double, double2, 1, 2>>},
  {"cw1.tps4.st3", "cw2.tps4.st2", "cw1.tps4.st2"},
  1};

// complex64: HBM bound; the variants trade ring depth against CTAs per SM.
static const VariantSet<float, 4> kMesonM = {
  {run_scalar<MesonOp<float, float2, 4, 8, 2>>, run_scalar<MesonOp<float, float2, 4, 8, 4>>,
   run_scalar<MesonOp<float, float2, 3, 8, 3>>, run_scalar<MesonOp<float, float2, 6, 16, 2>>},
  {"cw4.tps8.st2", "cw4.tps8.st4", "cw3.tps8.st3", "cw6.tps16.st2"},
  0};

cudaError_t launch_meson(const Job &job, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) return kMesonP.launch(job, p);
  return kMesonM.launch(job, convert_params<float>(p));
}

// complex64 all-source / all-sink: four threads (one spin row) per site, so a
// consumer warp holds 8 sites (18.7 KB per ring stage).  Two CTAs of two
// consumer warps with two stages, or one CTA of four or five.
static const VariantSet<float, 4> kMesonAllSrcM = {
  {run_scalar<MesonAllSourceOp<float, float2, 2, 2>>, run_scalar<MesonAllSourceOp<float, float2, 5, 2>>,
   run_scalar<MesonAllSourceOp<float, float2, 4, 2>>, run_scalar<MesonAllSourceOp<float, float2, 2, 4>>},
  {"cw2.tps4.st2", "cw5.tps4.st2", "cw4.tps4.st2", "cw2.tps4.st4"},
  0};
static const VariantSet<float, 4> kMesonAllSnkM = {
  {run_scalar<MesonAllSinkOp<float, float2, 2, 2>>, run_scalar<MesonAllSinkOp<float, float2, 5, 2>>,
   run_scalar<MesonAllSinkOp<float, float2, 4, 2>>, run_scalar<MesonAllSinkOp<float, float2, 2, 4>>},
  {"cw2.tps4.st2", "cw5.tps4.st2", "cw4.tps4.st2", "cw2.tps4.st4"},
  0};

cudaError_t launch_meson_all(const Job &job, bool source, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) return source ? kMesonAllSrcP.launch(job, p) : kMesonAllSnkP.launch(job, p);
  const OpParams<float> q = convert_params<float>(p);
  return source ? kMesonAllSrcM.launch(job, q) : kMesonAllSnkM.launch(job, q);
}

int meson_all_variants(Prec prec, bool source, const char *const **names)
{
  if (prec == Prec::C128) return source ? kMesonAllSrcP.describe(names) : kMesonAllSnkP.describe(names);
  return source ? kMesonAllSrcM.describe(names) : kMesonAllSnkM.describe(names);
}

int meson_variants(Prec prec, const char *const **names)
{
  if (prec == Prec::C128) return kMesonP.describe(names);
  return kMesonM.describe(names);
}

} // namespace cgb
