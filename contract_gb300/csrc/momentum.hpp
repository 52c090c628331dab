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
// 8 sites per timeslice, k-steps per work unit (a tile-shape choice: 128 by
// default, 64 and 192 as autotuner variants), units.  A unit's sum is kept in
// FP32 registers, window by window, and leaves as an FP32 partial that the
// reduction adds in FP64: short units bound the FP32 rounding.
constexpr int kTcUnitSteps = 128;
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
// tiles_ready: atiles already holds this plan's phase tiles (kept by the
// caller across calls), so they are not rebuilt.
cudaError_t launch_momentum_tc(const Job &job, const MomPlan &plan, const TcGeom &g, const void *field,
                               unsigned char *atiles, float *partial, void *out, bool tiles_ready = false);

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

// ------------------------------------------------------------ batched form --
// Many (P_i, P_j) pairs, on lattices of different extents, in one persistent
// launch of the fused complex64 kernel: every item's (t, z) planes are laid
// end to end in one unit space (unit_begin) that persistent CTAs walk.  The
// momentum list is the same for every item, and so is the structure of its
// plan (X groups, (nx, ny) pairs, Z groups) -- the host checks it -- while
// extents and phase tables differ; the tables are held once per distinct
// extent, (cos, sin)(2 pi k / L) rounded to FP32 from the FP64 values of the
// per-call plan, so an item's planes are the per-call kernel's.
constexpr int kMomBatchMaxItems = 128;
constexpr int kMomBatchMaxExt = 8;   // distinct spatial extents per batch
constexpr int kMomBatchMaxG = 256;   // Z groups (at most the momenta) per batch

struct MomBatchItem {
  const char *in[2];    // complex64 propagators (PyQUDA even/odd order)
  float2 *planes;       // [Lt][Lz][nq][256] FP32 plane sums (workspace)
  double2 *out;         // [np][Lt][256] complex128 correlators
  int latt[4];
  int unit_begin;       // first (t, z) plane of this item in the batch's unit space
  int tpp;              // tiles of 16 sites per plane
  int fin_begin;        // first finalisation block of this item (nq * Lt blocks)
  uint8_t tx, ty, tz;   // phase table of the x, y and z extents
};

struct MomBatchParams {
  DeviceStatus *status;
  int n_items, total_units, total_fin;
  int ngx, nq, np;
  int gx_k[kMomMaxPx], gx_plus[kMomMaxPx], gx_minus[kMomMaxPx];
  int q_ix[kMomQChunk], q_ny[kMomQChunk];
  int q_g0[kMomQChunk + 1];
  int gz_k[kMomBatchMaxG], gz_plus[kMomBatchMaxG], gz_minus[kMomBatchMaxG];
  float2 tab[kMomBatchMaxExt][kMomMaxL];
  MomBatchItem items[kMomBatchMaxItems];
};

// The per-timeslice finalisation of batched baryon items (kernels_batch.cu),
// carried by the combined finalisation launch below: out[o][t] = sum of the
// item's partials [2 Lt segments][per_seg][nout] in a fixed order.
struct BaryonFinItem {
  const double2 *partial;
  double2 *out;
  int lt, per_seg;
  int blk_begin;  // first finalisation block of this item
};
struct BaryonFinParams {
  int n_items, nout, total_blocks;
  BaryonFinItem items[kMomBatchMaxItems];
};

// One persistent launch of the fused site + X/Y kernel over every item's
// planes (site_warps 8 or 16).
cudaError_t launch_momentum_batch(const Job &job, const MomBatchParams &p, bool same_field, int site_warps);
// One launch for the rest: the Z transform and Gamma-pair map of every
// momentum item, and the per-timeslice sums of every baryon item in bf (n_items
// may be 0 on either side).
cudaError_t launch_batch_finalize(const Job &job, const MomBatchParams &mp, const BaryonFinParams &bf);

// All-gamma meson correlators at the plan's momenta: out[p][t][16*16]
// complex128 (device).  Uses job.ws for the per-site values and the plane
// sums, or (tensor_cores, complex64 only) the phase tiles and unit partials
// of the tensor-core projection.
cudaError_t launch_meson_momentum(const Job &job, const OpParams<double> &p, const MomPlan &plan, void *out,
                                  bool tensor_cores = false);

} // namespace cgb
