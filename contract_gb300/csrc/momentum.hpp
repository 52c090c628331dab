// Momentum-projection plan shared by the host (abi.cpp) and kernels_momentum.cu.
#pragma once

#include "launch.hpp"

namespace cgb {

constexpr int kMomMaxL = 64;     // largest spatial extent
constexpr int kMomMaxPx = 8;     // distinct nx values per call
constexpr int kMomMaxQ = 128;    // distinct (nx, ny) pairs per call
constexpr int kMomMaxP = 1024;   // momenta per call
constexpr int kMomQChunk = 25;   // (nx, ny) pairs per plane-kernel CTA

struct MomPlan {
  int latt[4];
  int npx, nq, np;
  int px[kMomMaxPx];                // distinct nx
  int q_ix[kMomMaxQ], q_ny[kMomMaxQ];  // pair q: index into px, ny
  int p_q[kMomMaxP], p_nz[kMomMaxP];   // momentum p: pair index, nz
  double cosx[kMomMaxL], sinx[kMomMaxL];  // exp(2 pi i k / Lx)
  double cosy[kMomMaxL], siny[kMomMaxL];
  double cosz[kMomMaxL], sinz[kMomMaxL];
};

// All-gamma meson correlators at the plan's momenta: out[p][t][16*16]
// complex128 (device).  Uses job.ws for the per-site values and plane sums.
cudaError_t launch_meson_momentum(const Job &job, const OpParams<double> &p, const MomPlan &plan, void *out);

} // namespace cgb
