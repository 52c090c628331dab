// Host interface of the batched launches (kernels_batch.cu).
#pragma once

#include "launch.hpp"

namespace cgb {

struct BatchSpec {
  const void *in[3];  // P_i, P_j, P_n (device)
  double2 *out;       // [6][nw][Lt] complex128
  int latt[4];
};

// All six baryon types x nw projectors (gamma-basis projectors only) for n
// items in one persistent launch plus one finalisation launch.
cudaError_t launch_baryon_fused_batch(const Job &job, int nw, const OpParams<double> &p, const BatchSpec *specs, int n);

} // namespace cgb
