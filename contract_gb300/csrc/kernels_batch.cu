// Batched all-types baryon contractions: many sources / lattices per launch.
#include <mutex>
#include <tuple>

#include "batch.cuh"
#include "launch_impl.cuh"
#include "batch.hpp"
#include "momentum.hpp"

namespace cgb {

// One persistent launch over the n items, then (fin == nullptr) the
// finalisation launch, or (fin != nullptr) the finalisation left to the
// caller's combined launch: fin receives each item's partials and outputs.
template <class Op>
static cudaError_t run_batch(const Job &job, const OpParams<typename Op::R> &op, const BatchSpec *specs, int n,
                             BaryonFinParams *fin)
{
  using R = typename Op::R;
  if (n <= 0) return cudaSuccess;
  if (n > kMaxBatch) return cudaErrorInvalidValue;
  static BatchParams<R> bp;  // large (~10 KB): built on the host, passed by value
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  bp = {};
  bp.op = op;
  bp.status = job.status;
  bp.n_items = n;
  size_t partial_total = 0;
  int chunks = 0;
  long long max_lt = 0;
  for (int i = 0; i < n; ++i) {
    Job ji = job;
    ji.volume = (long long)specs[i].latt[0] * specs[i].latt[1] * specs[i].latt[2] * specs[i].latt[3];
    ji.per_site = false;
    ji.lt = specs[i].latt[3];
    ji.half_slice = (long long)specs[i].latt[0] * specs[i].latt[1] * specs[i].latt[2] / 2;
    BatchItem &it = bp.items[i];
    for (int q = 0; q < 3; ++q) it.in[q] = specs[i].in[q];
    it.geom = make_geom(ji, Op::SITES, job.num_sms, 8);  // the device queue balances the CTAs
    it.chunk_begin = chunks;
    it.lt = ji.lt;
    it.out = specs[i].out;
    chunks += it.geom.total_chunks;
    partial_total += (size_t)it.geom.total_chunks * Op::CW * Op::NOUT;
    max_lt = std::max<long long>(max_lt, ji.lt);
  }
  bp.total_chunks = chunks;
  // the partial sums, then the queue's counter
  const size_t partial_bytes = (partial_total * sizeof(double2) + 255) / 256 * 256;
  char *ws = static_cast<char *>(job.ws->get(partial_bytes + 256));
  if (!ws) return cudaErrorMemoryAllocation;
  double2 *partial = reinterpret_cast<double2 *>(ws);
  bp.queue = reinterpret_cast<unsigned int *>(ws + partial_bytes);
  size_t off = 0;
  for (int i = 0; i < n; ++i) {
    bp.items[i].partial = partial + off;
    off += (size_t)bp.items[i].geom.total_chunks * Op::CW * Op::NOUT;
  }
  constexpr size_t smem = engine_smem_bytes<Op>();
  int bps = 0;
  cudaError_t e = prepare<Op>(batch_scalar_kernel<Op>, smem, bps);
  if (e != cudaSuccess) return e;
  const int grid = (int)std::min<long long>(chunks, (long long)job.num_sms * bps);
  e = cudaMemsetAsync(bp.queue, 0, sizeof(unsigned int), job.stream);
  if (e != cudaSuccess) return e;
  batch_scalar_kernel<Op><<<grid, Op::THREADS, smem, job.stream>>>(bp);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (fin) {
    fin->n_items = n;
    fin->nout = Op::NOUT;
    int blocks = 0;
    for (int i = 0; i < n; ++i) {
      BaryonFinItem &f = fin->items[i];
      f.partial = bp.items[i].partial;
      f.out = bp.items[i].out;
      f.lt = bp.items[i].lt;
      f.per_seg = bp.items[i].geom.chunks_per_seg * Op::CW;
      f.blk_begin = blocks;
      blocks += (Op::NOUT * f.lt + 255) / 256;
    }
    fin->total_blocks = blocks;
    return cudaSuccess;
  }
  const dim3 fg(n, (unsigned)((Op::NOUT * max_lt + 127) / 128));
  batch_finalize_kernel<R><<<fg, 128, 0, job.stream>>>(bp, Op::NOUT, Op::CW);
  return cudaGetLastError();
}

// Tile shapes of the batched launch (the autotuner's choice per batch: one
// shape serves every item of a launch).
template <int NW> struct BatchShapes {
  using Two = std::tuple<BaryonFusedSharedWedgeOp<float, float2, 4, 16, 2, NW, 3>,
                         BaryonFusedSharedWedgeOp<float, float2, 3, 16, 2, NW, 4>,
                         BaryonFusedSharedWedgeOp<float, float2, 2, 16, 3, NW, 6>>;
  using Same = std::tuple<BaryonFusedSharedWedgeSameOp<float, float2, 2, 2, NW, 4>,
                          BaryonFusedSharedWedgeSameOp<float, float2, 3, 2, NW, 3>,
                          BaryonFusedSharedWedgeSameOp<float, float2, 4, 2, NW, 2>>;
};
static const char *const kBatchShapeNames[] = {"shared.cw4.tps16.st2.occ3", "shared.cw3.tps16.st2.occ4",
                                               "shared.cw2.tps16.st3.occ6"};
static const char *const kBatchSameShapeNames[] = {"shared_same.cw2.tps8.st2.occ4", "shared_same.cw3.tps8.st2.occ3",
                                                   "shared_same.cw4.tps8.st2.occ2"};

template <class Tuple>
static cudaError_t run_shape(int v, const Job &job, const OpParams<float> &q, const BatchSpec *specs, int n,
                             BaryonFinParams *fin)
{
  switch (v) {
  case 1: return run_batch<std::tuple_element_t<1, Tuple>>(job, q, specs, n, fin);
  case 2: return run_batch<std::tuple_element_t<2, Tuple>>(job, q, specs, n, fin);
  default: return run_batch<std::tuple_element_t<0, Tuple>>(job, q, specs, n, fin);
  }
}

int batch_variants(bool same_field, const char *const **names)
{
  if (names) *names = same_field ? kBatchSameShapeNames : kBatchShapeNames;
  return 3;
}

bool batch_same_field(const OpParams<double> &p, const BatchSpec *specs, int n)
{
  bool same = n > 0;  // every item's P_i and P_j one field: the one-pass form
  for (int i = 0; i < n; ++i) same = same && specs[i].in[0] == specs[i].in[1];
  return same && p.b.perm1[0] != 0;
}

bool batch_rank_form(int nw, const OpParams<double> &p) { return nw == 1 && p.b.cl.ng > 1 && p.b.rk.r > 0; }

cudaError_t launch_baryon_fused_batch(const Job &job, int nw, const OpParams<double> &p, const BatchSpec *specs, int n,
                                      BaryonFinParams *fin)
{
  // One projector of rank <= 2 that is not one gamma matrix: factored triangles.
  if (batch_rank_form(nw, p)) {
    if (job.prec == Prec::C128) return run_batch<BaryonFusedRankOp<double, double2, 3, 16, 2>>(job, p, specs, n, fin);
    return run_batch<BaryonFusedRankOp<float, float2, 4, 16, 2>>(job, convert_params<float>(p), specs, n, fin);
  }
  // Otherwise gamma-basis projectors only (e.g. (1 +- g4)/2): no per-site N' buffers.
  if (p.b.cl.ng > nw) return cudaErrorInvalidValue;
  if (job.prec == Prec::C128) {
    return nw == 1 ? run_batch<BaryonFusedCliffOp<double, double2, 4, 16, 2, 1>>(job, p, specs, n, fin)
                   : run_batch<BaryonFusedCliffOp<double, double2, 4, 16, 2, 2>>(job, p, specs, n, fin);
  }
  const OpParams<float> q = convert_params<float>(p);
  bool same = n > 0;
  for (int i = 0; i < n; ++i) same = same && specs[i].in[0] == specs[i].in[1];
  // The shared-wedge forms take the Gamma_kl^T variants as a sign (every
  // Gamma(n) is symmetric or antisymmetric); the one-field form also needs a
  // Gamma_ij permutation without fixed points (XOR permutations: perm1[0] != 0).
  const int v = job.variant;
  if (same && q.b.perm1[0] != 0) {
    static BatchSpec two[kMaxBatch];  // inputs: the field once, then P_n
    static std::mutex mu2;
    std::lock_guard<std::mutex> lk(mu2);
    if (n > kMaxBatch) return cudaErrorInvalidValue;
    for (int i = 0; i < n; ++i) {
      two[i] = specs[i];
      two[i].in[1] = specs[i].in[2];
    }
    return nw == 1 ? run_shape<BatchShapes<1>::Same>(v, job, q, two, n, fin)
                   : run_shape<BatchShapes<2>::Same>(v, job, q, two, n, fin);
  }
  if (same)
    return nw == 1 ? run_batch<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 1, 3, true>>(job, q, specs, n, fin)
                   : run_batch<BaryonFusedCliffMergedOp<float, float2, 4, 16, 2, 2, 3, true>>(job, q, specs, n, fin);
  return nw == 1 ? run_shape<BatchShapes<1>::Two>(v, job, q, specs, n, fin)
                 : run_shape<BatchShapes<2>::Two>(v, job, q, specs, n, fin);
}

} // namespace cgb
