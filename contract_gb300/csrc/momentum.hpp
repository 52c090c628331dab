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
  // The exp(+i theta) and exp(-i theta) transforms share C = sum cos(theta) v
  // and S = sum sin(theta) v: n -> C + iS, -n -> C - iS.  Groups pair a
  // momentum component n (mod L) with -n; an absent partner is -1.
  int ngx;                                                        // X groups
  int gx_k[kMomMaxPx], gx_plus[kMomMaxPx], gx_minus[kMomMaxPx];  // k in [0, Lx/2]; px indices
  int q_g0[kMomMaxQ + 1];                                // Z groups of pair q: [q_g0[q], q_g0[q+1])
  int gz_k[kMomMaxP], gz_plus[kMomMaxP], gz_minus[kMomMaxP];     // k in [0, Lz/2]; momentum indices
};

// Geometry of the tensor-core projection (kernels_momentum_tc.cu): k-steps of
// 8 sites per timeslice, k-steps per work unit (a tile-shape choice: 512 by
// default, 256 and 1024 as autotuner variants), units.
constexpr int kTcUnitSteps = 512;
struct TcGeom {
  long long v3;  // sites per timeslice
  int lt;        // timeslices
  int j;         // k-steps per timeslice, ceil(v3 / 8)
  int ku;        // k-steps per unit
  int jb;        // units per (momentum group, t, pair half)
  int mg;        // momentum groups of 128
  int units;     // mg * jb * lt * 2
};
TcGeom make_tc_geom(const MomPlan &plan, int unit_steps = kTcUnitSteps);
size_t tc_phase_bytes(const TcGeom &g);
size_t tc_partial_bytes(const TcGeom &g);
cudaError_t launch_momentum_tc(const Job &job, const MomPlan &plan, const TcGeom &g, const void *field,
                               unsigned char *atiles, float *partial, void *out);

// Fused site + X/Y transform kernel of the mixed form (kernels_momentum_fused.cu):
// writes the FP32 planes [Lt][Lz][nq][256] straight from the two complex64
// propagators.  Supported for up to three X groups and kMomQChunk pairs.
bool momentum_fused_supported(const MomPlan &plan);
cudaError_t launch_momentum_fused(const Job &job, const void *in_i, const void *in_j, float2 *planes,
                                  const MomPlan &plan, int site_warps = 8);

// Tile-shape variants of the projection for the autotuner (Kind::Momentum).
// aux = 2 * tensor_cores + (fused form supported) + 4 * (P_i and P_j one field):
//   1, 5: complex64 fused with 8 or 16 site warps, or three kernels;
//   2, 3: tensor-core unit sizes.
int momentum_variants(Prec prec, int aux, const char *const **names);

// All-gamma meson correlators at the plan's momenta: out[p][t][16*16]
// complex128 (device).  Uses job.ws for the per-site values and the plane
// sums, or (tensor_cores, complex64 only) the phase tiles and unit partials
// of the tensor-core projection.
cudaError_t launch_meson_momentum(const Job &job, const OpParams<double> &p, const MomPlan &plan, void *out,
                                  bool tensor_cores = false);

} // namespace cgb
