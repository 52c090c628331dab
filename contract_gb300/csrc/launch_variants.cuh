// Tables of compiled tile-shape variants for one op (used by the launchers).
#pragma once

#include "launch_impl.cuh"

namespace cgb {

template <class R> using Runner = cudaError_t (*)(const Job &, OpParams<R>);

template <class R, int N> struct VariantSet {
  Runner<R> run[N];
  const char *names[N];
  int def;

  cudaError_t launch(const Job &job, const OpParams<R> &p) const
  {
    const int v = (job.variant >= 0 && job.variant < N) ? job.variant : def;
    return run[v](job, p);
  }
  int describe(const char *const **out) const
  {
    if (out) *out = names;
    return N;
  }
};

} // namespace cgb
