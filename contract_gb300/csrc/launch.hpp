// Internal host interface between the C ABI (abi.cpp) and the kernel
// translation units.  Not part of the public headers.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "ops.cuh"

namespace cgb {

enum class Prec { C128 = 0, C64 = 1 };

// Device scratch provider (partial sums of the per-timeslice reductions).
struct Workspace {
  virtual ~Workspace() = default;
  // Returns a device buffer of at least `bytes`, or nullptr on failure.
  virtual void *get(size_t bytes) = 0;
};

struct Job {
  Prec prec = Prec::C128;
  cudaStream_t stream = 0;
  DeviceStatus *status = nullptr;
  int num_sms = 1;
  long long volume = 0;
  // Per-site outputs (the reference's semantics) or per-timeslice sums.
  bool per_site = true;
  int lt = 0;                // timeslices (per_site == false)
  long long half_slice = 0;  // sites per (parity, t) segment = Lx*Ly*Lz/2
  Workspace *ws = nullptr;
  int variant = -1;          // tile-shape variant (-1: the launcher's default)
  unsigned long long wait_ns = 0;  // mbarrier wait limit of the site engines (0: kWaitLimitNs)
  int withhold_chunk = -1;         // test hook of the site engines (TileGeom::withhold_chunk)
  // Tensor-core momentum projection: a buffer the caller keeps for the phase
  // tiles of one (lattice, momentum list), and whether it already holds them.
  void *tc_tiles = nullptr;
  bool tc_tiles_ready = false;
};

// Ops whose launchers offer several compiled tile shapes (consumer warps,
// threads per site, ring stages); the autotuner in abi.cpp picks among them.
enum class Kind {
  Meson = 0,
  BaryonLoop = 1,
  BaryonTri = 2,
  BaryonFused = 3,
  Diquark = 4,
  Sequential = 5,
  MesonAll = 6,
  Momentum = 7
};

// Number of variants (and their names) for an op at a precision; `aux` is
// the projector count for BaryonFused and, for BaryonTri, 0 for the
// gamma-basis form, 1 for the materialised-N' form and 2 for the form with a
// projector of rank <= 2.  1 means there is nothing to tune.
int launch_variants(Kind kind, Prec prec, int aux, const char *const **names);

// Every launcher fills the geometry for its own tile shape and returns the
// CUDA error of the launch (cudaSuccess when volume == 0).
cudaError_t launch_meson(const Job &job, const OpParams<double> &p);
cudaError_t launch_meson_all(const Job &job, bool source, const OpParams<double> &p);
cudaError_t launch_baryon(const Job &job, bool loop, const OpParams<double> &p);
cudaError_t launch_baryon_fused(const Job &job, int nw, const OpParams<double> &p);
// The fused complex64 pass takes its one-pass form when P_i and P_j are the
// same device pointer.
inline bool fused_same_ij(const OpParams<double> &p) { return p.in[0] == p.in[1]; }
cudaError_t launch_diquark(const Job &job, const OpParams<double> &p);
cudaError_t launch_sequential(const Job &job, bool loop, int role, const OpParams<double> &p);
cudaError_t launch_convert(const Job &job, void *dst, const void *src, bool to_c64);
// Propagator site order lexicographic <-> PyQUDA even/odd (site_bytes per site).
cudaError_t launch_layout(const Job &job, void *dst, const void *src, const int *latt, bool to_eo, int site_bytes);
// Propagator <-> twelve colour-spinor fields in QUDA's native order (stride:
// the fields' checkerboard length in 16-byte chunks; entry_bytes 16 or 8).
cudaError_t launch_quda_layout(const Job &job, void *prop, void *const *fields, long long stride, bool from_quda,
                               int entry_bytes);
// In place P -> U P U^dagger on the spin indices; u: host 4 x 4 complex128, row-major.
cudaError_t launch_spin_rotation(const Job &job, void *prop, const double *u);
// Address of this device's status word (a __device__ variable of the library).
cudaError_t device_status_ptr(DeviceStatus **out);
// Device address and size of the fixed scratch array used by the
// allocation-free entry point (noalloc.cu).
cudaError_t static_scratch(void **ptr, size_t *bytes);

// ---- helpers shared by the launcher TUs --------------------------------------
template <class R> OpParams<R> convert_params(const OpParams<double> &p)
{
  OpParams<R> o {};
  for (int k = 0; k < 3; ++k) o.in[k] = p.in[k];
  for (int k = 0; k < 16; ++k) o.out[k] = p.out[k];
  o.geom = p.geom;
  o.status = p.status;
  for (int k = 0; k < 4; ++k) o.latt[k] = p.latt[k];
  for (int k = 0; k < 4; ++k) {
    o.b.perm1[k] = p.b.perm1[k];
    o.b.perm2[k] = p.b.perm2[k];
    o.m.perm1[k] = p.m.perm1[k];
    o.m.perm2[k] = p.m.perm2[k];
    o.m.ph1[k] = p.m.ph1[k];
    o.m.ph2[k] = p.m.ph2[k];
    for (int v = 0; v < 2; ++v) {
      o.b.ph1[v][k] = p.b.ph1[v][k];
      o.b.ph2[v][k] = p.b.ph2[v][k];
    }
  }
  for (int w = 0; w < 2; ++w) {
    const ProjOperand<double> &s = p.b.proj[w];
    ProjOperand<R> &d = o.b.proj[w];
    for (int k = 0; k < 16; ++k) {
      d.w[k][0] = R(s.w[k][0]);
      d.w[k][1] = R(s.w[k][1]);
    }
    for (int k = 0; k < 4; ++k) {
      d.perm[k] = s.perm[k];
      d.ph[k] = s.ph[k];
    }
    d.is_perm = s.is_perm;
    d.nnz = s.nnz;
    d.nzmask = s.nzmask;
    for (int k = 0; k < 16; ++k) d.nzk[k] = s.nzk[k];
  }
  o.b.cl.ng = p.b.cl.ng;
  for (int k = 0; k < 16; ++k) {
    o.b.cl.has_phase[k] = p.b.cl.has_phase[k];
    for (int r = 0; r < 4; ++r) {
      o.b.cl.perm[k][r] = p.b.cl.perm[k][r];
      o.b.cl.ph[k][r] = p.b.cl.ph[k][r];
    }
    for (int w = 0; w < 2; ++w) {
      o.b.cl.coef[w][k][0] = R(p.b.cl.coef[w][k][0]);
      o.b.cl.coef[w][k][1] = R(p.b.cl.coef[w][k][1]);
      for (int m = 0; m < 4; ++m) {
        o.b.cl.qc[w][k][m][0] = R(p.b.cl.qc[w][k][m][0]);
        o.b.cl.qc[w][k][m][1] = R(p.b.cl.qc[w][k][m][1]);
      }
    }
  }
  o.b.rk.r = p.b.rk.r;
  o.b.rk.nnz = p.b.rk.nnz;
  o.b.rk.unit = p.b.rk.unit;
  o.b.rk.scale = R(p.b.rk.scale);
  for (int s = 0; s < 2; ++s)
    for (int r = 0; r < 2; ++r)
      for (int k = 0; k < 4; ++k) {
        o.b.rk.idx[s][r][k] = p.b.rk.idx[s][r][k];
        o.b.rk.ph[s][r][k] = p.b.rk.ph[s][r][k];
        o.b.rk.c[s][r][k][0] = R(p.b.rk.c[s][r][k][0]);
        o.b.rk.c[s][r][k][1] = R(p.b.rk.c[s][r][k][1]);
      }
  return o;
}

} // namespace cgb
