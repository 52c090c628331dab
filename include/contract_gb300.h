/*
 * contract_gb300.h -- extensions of the libcontract.so C ABI (GB300 build).
 *
 * None of these entry points exists in CLQCD/contract; they add what its
 * callers otherwise do themselves (per-timeslice sums, many contraction types
 * per pass, precision choice) plus error reporting and stream control.
 *
 * Shared conventions (see also contract.h):
 *  - precision: CONTRACT_C128 propagators are complex128 (the drop-in format);
 *    CONTRACT_C64 propagators are complex64 and the arithmetic is FP32 with
 *    FP64 per-timeslice reduction ("mixed" form).
 *  - lattice: int[4] = {Lx, Ly, Lz, Lt} of the local lattice in PyQUDA
 *    even/odd site order, site = (((p*Lt + t)*Lz + z)*Ly + y)*(Lx/2) + xh,
 *    Lx even.  When a call takes `lattice`, passing NULL selects per-site
 *    output (one complex128 per site, `volume` sites); non-NULL selects
 *    per-timeslice sums (Lt complex128 values, the reduction in FP64).
 *  - correlator outputs are always complex128 device buffers.
 */
#ifndef CONTRACT_GB300_H
#define CONTRACT_GB300_H

#include <stddef.h>

#include "contract.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  CONTRACT_C128 = 0,
  CONTRACT_C64 = 1,
  /* contract_meson_all_gamma_momentum only: complex64 propagators, FP32
   * site arithmetic, and the projection as a tensor-core GEMM with each
   * operand split into two bf16 terms (hi*hi + hi*lo + lo*hi), FP32
   * accumulation and an FP64 sum per timeslice. */
  CONTRACT_C64_TC = 2,
};

/* ----------------------------------------------------------- errors ---- */
enum {
  CONTRACT_SUCCESS = 0,
  CONTRACT_ERROR_INVALID_ARGUMENT = 1,
  CONTRACT_ERROR_CUDA = 2,             /* a CUDA runtime call failed */
  CONTRACT_ERROR_DEVICE_TIMEOUT = 3,   /* a kernel gave up waiting on its own copies */
  CONTRACT_ERROR_OUT_OF_MEMORY = 4,    /* the workspace could not grow */
  CONTRACT_ERROR_BAD_WORK = 5,         /* a batched work descriptor failed validation */
};

enum {
  CONTRACT_ERRORS_EXIT = 0,    /* reference behaviour: message on stderr, exit(-1) (CUDA errors: exit(code)) */
  CONTRACT_ERRORS_RECORD = 1,  /* record the error, skip the call, return */
};

/* Select how invalid calls are handled.  The default is CONTRACT_ERRORS_EXIT
 * unless the environment variable CONTRACT_ERROR_MODE=record is set. */
void contract_set_error_mode(int mode);
int contract_get_error_mode(void);

/* First error recorded since the last clear (sticky), and its message. */
int contract_last_error(void);
const char *contract_last_error_message(void);
void contract_clear_error(void);

/* Synchronise the current stream, then fold the device status word (errors
 * reported by kernels, e.g. a timed-out wait) into the sticky error. */
int contract_check_device(void);

/* Wall-time limit, in nanoseconds, of every wait of the site kernels on their
 * own copies (0 = the default, 2 s).  A wait that runs out sets the timeout
 * bit that contract_check_device() reports; the kernel then waits (bounded)
 * for its copies still in flight and returns, so the context stays usable. */
void contract_set_wait_limit(unsigned long long ns);
/* Test hook for the timeout path: in the next call only, the site kernel's
 * producer never issues (nor announces) the copies of the first tile of work
 * chunk `chunk`, so the consumers waiting for that tile run out of time.  The
 * call's results are then incomplete and contract_check_device() reports
 * CONTRACT_ERROR_DEVICE_TIMEOUT.  A negative chunk cancels it. */
void contract_test_withhold_chunk(int chunk);

/* ---------------------------------------------------------- streams ---- */
/* All later calls (drop-in ones included) queue work on `stream`
 * (a cudaStream_t; NULL = legacy default stream, the reference's choice). */
void contract_set_stream(void *stream);
void *contract_get_stream(void);

/* Tile-shape autotuning (consumer warps, threads per site, ring stages) of
 * the complex64 kernels: when enabled, the first call for a new (op, shape)
 * times each compiled variant on its own data and keeps the fastest.  Also
 * enabled by CONTRACT_AUTOTUNE=1; CONTRACT_TUNE_CACHE=<file> persists the
 * choices across processes.  Never tunes during stream capture. */
void contract_set_autotune(int enable);
/* Writes "key<TAB>variant<TAB>ms" lines of the current choices into buf
 * (NUL-terminated, truncated to n); returns the number of entries. */
int contract_autotune_report(char *buf, size_t n);
/* Names of the compiled tile-shape variants of an op, space-separated in
 * variant order (the order a tune-cache line's variant index refers to), into
 * buf (NUL-terminated, truncated to n); returns their number (1: nothing to
 * tune).  op: 0 meson, 1 baryon loop form, 2 baryon triangle form, 3 all
 * types in one pass, 4 diquark, 5 sequential, 6 meson all-source/sink,
 * 7 meson all-gamma momentum projection; precision CONTRACT_C128 or
 * CONTRACT_C64; aux as in the tune-cache keys (for op 2, 0: Gamma_mn one
 * gamma matrix, 1: N' = W N formed per site, 2: a projector of rank <= 2, see
 * contract_projector_rank; the projector count for op 3, +4 when P_i and P_j
 * are one field; for op 7, 2 selects the tensor-core form).  Unknown op or
 * precision: an error, and 0. */
int contract_variant_names(int op, int precision, int aux, char *buf, size_t n);

/* Reserve `bytes` of the per-device workspace used by per-timeslice
 * reductions, so that later calls (e.g. inside CUDA graph capture) do not
 * allocate.  Returns CONTRACT_SUCCESS or an error code. */
int contract_workspace_reserve(size_t bytes);
/* Workspace bytes a per-timeslice call with `noutputs` correlators needs. */
size_t contract_workspace_bytes(const int *lattice, int noutputs);

/* ------------------------------------------------------ gamma algebra -- */
/* perm[16*4], phase[16*4]: Gamma(n)[r][perm[n*4+r]] = i^phase[n*4+r]. */
void contract_gamma_table(int *perm, int *phase);
/* How the per-call triangle kernels apply a projector W (project_mn of
 * baryon_general_two_point: 16 complex128, row-major W[m][n]): 1 or 2 when W
 * factors exactly as sum_r x_r y_r^T of that rank, found by elimination with
 * complete pivoting whose remainder is exactly zero ((1 +- g4)/2: 2; a
 * polarised projector such as (1 + g4)(1 - i g1 g2)/4: 1), so that each spin
 * pair takes r colour wedges instead of four; 0 when they form N' = W N per
 * site instead (rank above 2, W = 0, or project_mn NULL). */
int contract_projector_rank(const void *project_mn);

/* ------------------------------------------------------- conversion ---- */
/* complex128 <-> complex64 propagator copy of `volume` sites on the device. */
void contract_convert_precision(void *dst, const void *src, size_t volume, int to_c64);

/* Propagator site order on the device: to_eo != 0 reorders a lexicographic
 * propagator (site ((t*Lz + z)*Ly + y)*Lx + x, e.g. QUDA's lexicographic or a
 * gathered numpy field) into PyQUDA even/odd order [2][Lt][Lz][Ly][Lx/2]
 * (parity (x+y+z+t) & 1); to_eo == 0 goes back.  Whole sites are moved
 * (144 complex of `precision`); dst and src must not overlap.  No
 * counterpart in the reference. */
void contract_convert_layout(void *dst, const void *src, const int *lattice, int to_eo, int precision);

/* Propagators as QUDA's solver leaves them on the device: twelve
 * colour-spinor fields, one per source (spin k, colour d), field 3k + d, each
 * in QUDA's native order [parity][chunk][stride][16 bytes], a chunk holding 16
 * bytes of the site's spin-colour vector (complex entry 3s + c, sink spin s,
 * sink colour c): one entry per chunk in complex128 (QUDA_FLOAT2_FIELD_ORDER),
 * two in complex64 (QUDA_FLOAT4_FIELD_ORDER).  QUDA's checkerboard site index
 * is the PyQUDA even/odd order's, so sites keep their index.  fields: HOST
 * array of 12 device pointers; stride: checkerboard length of the fields in
 * sites, >= volume/2 (0 = volume/2, no padding).  The pad sites of the fields
 * are neither read nor written.  Bit-exact both ways.  The baryon_2pt.py
 * example receives its propagators from PyQUDA's invert (baryon_2pt.py:63),
 * which converts QUDA's fields on the host; these calls do it on the device.
 * No counterpart in the reference. */
void contract_convert_from_quda(void *propag, void *const *fields, const int *lattice, size_t stride, int precision);
void contract_convert_to_quda(void *const *fields, const void *propag, const int *lattice, size_t stride,
                              int precision);

/* In place change of spin basis of `volume` propagator sites:
 * P[s][k] -> sum U[s][s'] P[s'][k'] conj(U[k][k']) for every colour pair;
 * rotation: HOST 4 x 4 complex128, row-major (e.g. the unitary that takes a
 * solver's gamma basis to DeGrand-Rossi, the basis every contraction here
 * assumes).  FP64 arithmetic for complex128, FP32 for complex64.  No
 * counterpart in the reference. */
void contract_rotate_spin_basis(void *propag, size_t volume, const void *rotation, int precision);

/* ------------------------------------------------------ contractions --- */
/* meson_two_point with a precision and optional per-timeslice output. */
void contract_meson(void *correl, const void *propag_i, const void *propag_j, size_t volume, int gamma_ij,
                    int gamma_kl, int precision, const int *lattice);

/* meson_all_{source,sink}_two_point: correl is a HOST array of 16 device
 * pointers; `source` != 0 fixes gamma_ij = fixed_gamma and loops gamma_kl,
 * else fixes gamma_kl and loops gamma_ij. */
void contract_meson_all(void **correl, const void *propag_i, const void *propag_j, size_t volume, int fixed_gamma,
                        int source, int precision, const int *lattice);

/* baryon_two_point / baryon_general_two_point in one call: project_mn (HOST,
 * 16 complex128, row-major) replaces Gamma(gamma_mn) when non-NULL. */
void contract_baryon(void *correl, const void *propag_i, const void *propag_j, const void *propag_n,
                     BaryonContractType contract_type, size_t volume, int gamma_ij, int gamma_kl, int gamma_mn,
                     const void *project_mn, int precision, const int *lattice);

/* All six contraction types for `nproj` (1 or 2) projectors in one pass over
 * the three propagators.  projectors: HOST, nproj x 16 complex128.
 * correl: device complex128 [6][nproj][Lt] (lattice given) or
 * [6][nproj][volume] (lattice NULL); types in BaryonContractType order. */
void contract_baryon_all_types(void *correl, const void *propag_i, const void *propag_j, const void *propag_n,
                               size_t volume, int gamma_ij, int gamma_kl, int nproj, const void *projectors,
                               int precision, const int *lattice);

/* contract_baryon_all_types from HOST complex128 propagators (pinned memory
 * for full speed) into a HOST correl [6][nproj][Lt]; lattice required.
 * Timeslice chunks of the three propagators are copied back to back on one copy stream
 * while earlier chunks are converted (CONTRACT_C64) and contracted on the
 * library stream, so the copies overlap the work.  Asynchronous like every
 * other call: synchronise the library stream before reading correl or
 * changing the inputs.  Uses its own growable staging memory on the device.
 * No counterpart in the reference. */
void contract_baryon_all_types_host(void *correl, const void *propag_i, const void *propag_j, const void *propag_n,
                                    size_t volume, int gamma_ij, int gamma_kl, int nproj, const void *projectors,
                                    int precision, const int *lattice);

/* contract_baryon_all_types with a non-NULL lattice, for callers that cannot
 * let the library allocate device memory (a pool allocator in the host
 * framework owns the free memory, cudaMalloc's implicit synchronisation is
 * not acceptable, or the host requires an allocation-free library as the
 * reference library is).  No counterpart in the reference.
 *
 * The per-timeslice partial sums go into a fixed 16 MiB static device array
 * that every GPU loading the library holds until exit; nothing is allocated
 * or freed.  The array is fully overwritten by each call (nothing needs to
 * start at zero), and all calls share it: calls that overlap on the GPU (on
 * different streams, or in different host threads) race.  The first call on
 * a device looks up the array's device address; make it before any stream
 * capture.  A lattice whose partial sums do not fit the array is rejected
 * with CONTRACT_ERROR_INVALID_ARGUMENT and a message naming both sizes (each
 * of the 2 Lt half-timeslices needs at least 1344 bytes with two projectors,
 * so Lt beyond about 6000 never fits; a 48^3 x 96 lattice does).  Returns
 * CONTRACT_SUCCESS or the error code (errors also follow the error mode, like
 * every other call). */
int contract_baryon_all_types_noalloc(void *correl, const void *propag_i, const void *propag_j,
                                      const void *propag_n, size_t volume, int gamma_ij, int gamma_kl, int nproj,
                                      const void *projectors, int precision, const int *lattice);

/* One work item of a batched launch: a source position / propagator triple
 * on its own lattice (extents may differ between items). */
typedef struct {
  const void *propag_i, *propag_j, *propag_n;  /* device, `precision` storage */
  void *correl;                                /* device complex128 [6][nproj][Lt] */
  int lattice[4];                              /* Lx, Ly, Lz, Lt (PyQUDA even/odd order) */
} ContractBaryonBatchItem;

/* contract_baryon_all_types (per-timeslice) for up to 128 items in one
 * persistent launch driven by a device work queue, plus one finalisation
 * launch; items is a HOST array.  Projectors must be spanned by at most
 * nproj gamma matrices (e.g. (1 +- g4)/2 with nproj = 2), or be one projector
 * of rank <= 2 (contract_projector_rank; e.g. (1 + g4)/2 alone with
 * nproj = 1, which runs the factored triangle form in both passes and one
 * tile shape).  No host synchronisation: after a
 * warm-up call (and contract_workspace_reserve) the sequence can be captured
 * in a CUDA graph.  When EVERY item passes one pointer as both propag_i and
 * propag_j, the launch evaluates one triangle pass per site (the second is
 * the same values); a single item with two distinct fields sends the whole
 * batch to the two-pass form.  The two forms agree to FP32 rounding. */
void contract_baryon_all_types_batch(const ContractBaryonBatchItem *items, int nitems, int gamma_ij, int gamma_kl,
                                     int nproj, const void *projectors, int precision);

/* One work item of a batched meson momentum projection: a (P_i, P_j) pair on
 * its own lattice (extents may differ between items). */
typedef struct {
  const void *propag_i, *propag_j;  /* device, complex64 */
  void *correl;                     /* device complex128 [nmom][Lt][256] */
  int lattice[4];                   /* Lx, Ly, Lz, Lt (PyQUDA even/odd order) */
} ContractMesonMomentumBatchItem;

/* contract_meson_all_gamma_momentum (CONTRACT_C64) for up to 128 items with
 * one momentum list: one persistent launch over every item's (t, z) planes
 * and one finalisation launch.  The list must give every item's lattice the
 * same structure of +n/-n groups (any list with 2|n| < L in each direction
 * does; e.g. n in {-1, 0, 1}^3 on L >= 3); at most 8 distinct spatial
 * extents.  When every item passes one field as propag_i and propag_j, the
 * launch forms the Hermitian site products.  No host synchronisation after a
 * warm-up call; the workspace holds every item's FP32 planes. */
void contract_meson_all_gamma_momentum_batch(const ContractMesonMomentumBatchItem *items, int nitems,
                                             const int *moms, int nmom, int precision);

/* The batched baryon and meson workloads of one set of sources together
 * (CONTRACT_C64): the baryon items' all-types contraction (as
 * contract_baryon_all_types_batch) in one persistent launch, the meson items'
 * momentum projection (as contract_meson_all_gamma_momentum_batch) in
 * another, and a single finalisation launch for both -- three kernel launches
 * for any number of items.  With autotuning enabled, each launch's tile
 * shape is chosen per lattice extent: every extent class is timed alone, and
 * the launch takes the shape with the least total over its items (reported
 * by contract_autotune_report per class and per batch).  Either count may be
 * 0.  No counterpart in the reference, whose callers issue one launch per
 * contraction (include/kernel.cuh:173-183). */
void contract_batch_mixed(const ContractBaryonBatchItem *baryon_items, int nbaryon, int gamma_ij, int gamma_kl,
                          int nproj, const void *projectors, const ContractMesonMomentumBatchItem *meson_items,
                          int nmeson, const int *moms, int nmom, int precision);

/* All 16 x 16 meson correlators (C(x) of meson_two_point for every
 * (gamma_ij, gamma_kl)) projected to momenta, per timeslice:
 *   correl[p][t][gamma_ij * 16 + gamma_kl] =
 *       sum_{x in t} exp(+2 pi i (nx x/Lx + ny y/Ly + nz z/Lz)) C(x),
 * moms: HOST int[nmom][3] = (nx, ny, nz); lattice required, spatial extents
 * <= 64, at most 8 distinct nx and 128 distinct (nx, ny) per call.  correl:
 * device complex128 [nmom][Lt][256].  Uses the per-device workspace for
 * V x 256 site values and the per-plane partial sums (FP64), or with
 * CONTRACT_C64_TC the bf16 phase tiles and the FP32 partials of the
 * tensor-core projection. */
void contract_meson_all_gamma_momentum(void *correl, const void *propag_i, const void *propag_j, size_t volume,
                                       const int *lattice, const int *moms, int nmom, int precision);

/* baryon_diquark / baryon_sequential_two_point with a storage precision
 * (fields are read and written in that precision). */
void contract_diquark(void *diquark, const void *propag_i, const void *propag_j, size_t volume, int gamma_ij,
                      int gamma_kl, int precision);
void contract_sequential(void *propag_i, void *propag_j, void *propag_n, BaryonContractType contract_type,
                         BaryonSequentialType sequential_type, size_t volume, int gamma_ij, int gamma_kl,
                         int gamma_mn, int precision);

/* Sequential source inserted at the sink timeslice t_sink: the selected
 * propagator is overwritten with dC(x)/dP(x) on the sites of timeslice
 * t_sink and with zeros everywhere else (PyQUDA even/odd order, lattice
 * required). */
void contract_sequential_sink(void *propag_i, void *propag_j, void *propag_n, BaryonContractType contract_type,
                              BaryonSequentialType sequential_type, size_t volume, const int *lattice, int t_sink,
                              int gamma_ij, int gamma_kl, int gamma_mn, int precision);

#ifdef __cplusplus
}
#endif

#endif /* CONTRACT_GB300_H */
