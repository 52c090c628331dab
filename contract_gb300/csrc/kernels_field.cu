// Field-valued kernels: diquark and sequential sources.
// Op template arguments: <R, S, consumer warps, threads per site, ring stages>.
#include "launch_variants.cuh"

namespace cgb {

template <class R, class S, int CW, int TPS, int NST>
static cudaError_t seq_dispatch(const Job &job, bool loop, int role, const OpParams<R> &p)
{
  if (loop) {
    switch (role) {
    case 0: return run_field<SequentialOp<R, S, CW, TPS, NST, true, 0>>(job, p);
    case 1: return run_field<SequentialOp<R, S, CW, TPS, NST, true, 1>>(job, p);
    default: return run_field<SequentialOp<R, S, CW, TPS, NST, true, 2>>(job, p);
    }
  }
  switch (role) {
  case 0: return run_field<SequentialOp<R, S, CW, TPS, NST, false, 0>>(job, p);
  case 1: return run_field<SequentialOp<R, S, CW, TPS, NST, false, 1>>(job, p);
  default: return run_field<SequentialOp<R, S, CW, TPS, NST, false, 2>>(job, p);
  }
}

// complex64 variants: the two-CTA shapes keep more tiles (and stores) in flight;
// the default (last field) is the tuner's choice at 24^3 x 64.
static const VariantSet<float, 6> kDiquarkM = {
  {run_field<DiquarkOp<float, float2, 6, 16, 2>>, run_field<DiquarkOp<float, float2, 8, 16, 3>>,
   run_field<DiquarkOp<float, float2, 6, 16, 2, true>>, run_field<DiquarkOp<float, float2, 8, 16, 3, true>>,
   run_field<DiquarkOp<float, float2, 4, 16, 2, true>>, run_field<DiquarkOp<float, float2, 3, 16, 3, true>>},
  {"cw6.tps16.st2", "cw8.tps16.st3", "cw6.tps16.st2.direct", "cw8.tps16.st3.direct", "cw4.tps16.st2.direct",
   "cw3.tps16.st3.direct"},
  5};

// complex128 (FP64-pipe bound): the first shape is the default.
static const VariantSet<double, 3> kDiquarkP = {
  {run_field<DiquarkOp<double, double2, 4, 16, 3>>, run_field<DiquarkOp<double, double2, 3, 16, 2>>,
   run_field<DiquarkOp<double, double2, 2, 16, 3>>},
  {"cw4.tps16.st3", "cw3.tps16.st2", "cw2.tps16.st3"},
  0};

cudaError_t launch_diquark(const Job &job, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) return kDiquarkP.launch(job, p);
  return kDiquarkM.launch(job, convert_params<float>(p));
}

cudaError_t launch_sequential(const Job &job, bool loop, int role, const OpParams<double> &p)
{
  if (job.prec == Prec::C128) {  // default (no variant chosen): three consumer warps, two stages
    if (job.variant == 0) return seq_dispatch<double, double2, 4, 16, 3>(job, loop, role, p);
    if (job.variant == 2) return seq_dispatch<double, double2, 2, 16, 3>(job, loop, role, p);
    return seq_dispatch<double, double2, 3, 16, 2>(job, loop, role, p);
  }
  const OpParams<float> q = convert_params<float>(p);
  if (job.variant == 1) return seq_dispatch<float, float2, 8, 16, 3>(job, loop, role, q);
  if (job.variant == 2) return seq_dispatch<float, float2, 3, 16, 3>(job, loop, role, q);
  return seq_dispatch<float, float2, 5, 16, 2>(job, loop, role, q);
}

static const char *const kSequentialNames[3] = {"cw5.tps16.st2", "cw8.tps16.st3", "cw3.tps16.st3"};
static const char *const kSequentialNamesP[3] = {"cw4.tps16.st3", "cw3.tps16.st2", "cw2.tps16.st3"};

int field_variants(Prec prec, bool sequential, const char *const **names)
{
  if (prec == Prec::C128) {
    if (!sequential) return kDiquarkP.describe(names);
    if (names) *names = kSequentialNamesP;
    return 3;
  }
  if (!sequential) return kDiquarkM.describe(names);
  if (names) *names = kSequentialNames;
  return 3;
}

} // namespace cgb
