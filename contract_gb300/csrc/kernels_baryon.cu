// Baryon two-point kernels, one contraction type per launch.
// Op template arguments: <R, S, consumer warps, threads per site, ring stages>.
#include "launch_variants.cuh"

namespace cgb {

// complex128 (FP64-pipe bound): 8 sites per tile, one (i, l) spin pair per thread.
using LoopP = BaryonLoopOp<double, double2, 4, 16, 3>;
using TriP = BaryonTriOp<double, double2, 4, 16, 3>;
using TriCliffP = BaryonTriCliffOp<double, double2, 4, 16, 3>;

// complex64 variants: sites per tile x ring depth x CTAs per SM.
static const VariantSet<float, 4> kLoopM = {
  {run_scalar<BaryonLoopOp<float, float2, 7, 16, 2>>, run_scalar<BaryonLoopOp<float, float2, 5, 16, 3>>,
   run_scalar<BaryonLoopOp<float, float2, 4, 8, 3>>, run_scalar<BaryonLoopOp<float, float2, 3, 16, 3>>},
  {"cw7.tps16.st2", "cw5.tps16.st3", "cw4.tps8.st3", "cw3.tps16.st3"},
  0};
// General projector (N' materialised per site).
static const VariantSet<float, 4> kTriM = {
  {run_scalar<BaryonTriOp<float, float2, 6, 16, 2>>, run_scalar<BaryonTriOp<float, float2, 7, 16, 3>>,
   run_scalar<BaryonTriOp<float, float2, 4, 16, 3>>, run_scalar<BaryonTriOp<float, float2, 3, 16, 2>>},
  {"cw6.tps16.st2", "cw7.tps16.st3", "cw4.tps16.st3", "cw3.tps16.st2"},
  0};
static const VariantSet<float, 5> kTriCliffM = {
  {run_scalar<BaryonTriCliffOp<float, float2, 7, 16, 2>>, run_scalar<BaryonTriCliffOp<float, float2, 5, 16, 3>>,
   run_scalar<BaryonTriCliffOp<float, float2, 4, 8, 2>>, run_scalar<BaryonTriCliffOp<float, float2, 3, 16, 2>>,
   run_scalar<BaryonTriCliffOp<float, float2, 4, 16, 3>>},
  {"cw7.tps16.st2", "cw5.tps16.st3", "cw4.tps8.st2", "cw3.tps16.st2", "cw4.tps16.st3"},
  0};

cudaError_t launch_baryon(const Job &job, bool loop, const OpParams<double> &p)
{
  // A projector that is one gamma matrix (baryon_two_point) needs no N' buffer.
  const bool cliff = p.b.cl.ng == 1;
  if (job.prec == Prec::C128) {
    if (loop) return run_scalar<LoopP>(job, p);
    return cliff ? run_scalar<TriCliffP>(job, p) : run_scalar<TriP>(job, p);
  }
  const OpParams<float> q = convert_params<float>(p);
  if (loop) return kLoopM.launch(job, q);
  return cliff ? kTriCliffM.launch(job, q) : kTriM.launch(job, q);
}

int baryon_variants(Prec prec, int form, const char *const **names)
{
  if (prec == Prec::C128) return 1;
  if (form == 0) return kLoopM.describe(names);
  return form == 1 ? kTriCliffM.describe(names) : kTriM.describe(names);
}

} // namespace cgb
