// Host interface of the batched launches (kernels_batch.cu).
#pragma once

#include "launch.hpp"

namespace cgb {

struct BatchSpec {
  const void *in[3];  // P_i, P_j, P_n (device)
  double2 *out;       // [6][nw][Lt] complex128
  int latt[4];
};

struct BaryonFinParams;

// All six baryon types x nw projectors (gamma-basis projectors, or one
// projector of rank <= 2) for n items in one persistent launch plus one
// finalisation launch -- or, with
// fin != nullptr, without it: fin then describes the partial sums for the
// caller's combined finalisation (launch_batch_finalize).  job.variant picks
// the tile shape (batch_variants; -1 the default).
cudaError_t launch_baryon_fused_batch(const Job &job, int nw, const OpParams<double> &p, const BatchSpec *specs, int n,
                                      BaryonFinParams *fin = nullptr);
// Names of the batched launch's tile shapes (the one-pass form when every
// item passes one field as P_i and P_j, and Gamma_ij allows it).
int batch_variants(bool same_field, const char *const **names);
bool batch_same_field(const OpParams<double> &p, const BatchSpec *specs, int n);
// One projector of rank <= 2 that is not one gamma matrix: the factored
// triangle form, one tile shape (job.variant is not used).
bool batch_rank_form(int nw, const OpParams<double> &p);

} // namespace cgb
