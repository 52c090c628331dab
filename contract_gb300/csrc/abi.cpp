// C ABI of libcontract.so: the contract.h drop-in entry points and the
// contract_gb300.h extensions.  Validates arguments, builds the gamma
// coefficient tables of each call, and hands the work to the kernel launchers.
//
// Error behaviour (CLQCD/contract lib/target/runtime_api_cuda.cpp:5-12 and the
// launchers, e.g. lib/baryon/baryon.cu:43-45): an invalid selector prints a
// message and exits with -1, a failed CUDA call exits with its error code.
// That stays the default; contract_set_error_mode(CONTRACT_ERRORS_RECORD)
// (or CONTRACT_ERROR_MODE=record) records the error and skips the call instead.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <cmath>
#include <fstream>
#include <functional>
#include <memory>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "contract_gb300.h"
#include "gamma.hpp"
#include "launch.hpp"
#include "momentum.hpp"
#include "batch.hpp"

namespace {

using cgb::OpParams;

std::mutex g_mu;
int g_mode = -1;
int g_err = CONTRACT_SUCCESS;
std::string g_msg;
cudaStream_t g_stream = nullptr;
unsigned long long g_wait_ns = 0;  // 0: the engines' default limit
int g_withhold_chunk = -1;         // test hook for the next call (contract_test_withhold_chunk)

constexpr cgb::GammaTables kG = cgb::build_gamma_tables();

constexpr int kPipeSlots = 3;  // staging slots of the host-input pipeline

struct DevState {
  int num_sms = 0;
  cgb::DeviceStatus *status = nullptr;
  void *ws = nullptr;
  size_t ws_bytes = 0;
  // Host-input pipeline (contract_baryon_all_types_host): staging buffers,
  // the copy stream and the slots' events; created on first use.
  void *pipe = nullptr;
  size_t pipe_bytes = 0;
  cudaStream_t copy = nullptr;  // host-to-device copies of the host-input pipeline
  cudaEvent_t copied[kPipeSlots] = {}, freed[kPipeSlots] = {}, start = nullptr;
  // Tensor-core momentum projection: the phase tiles of the last (lattice,
  // momentum list), kept so that repeated calls do not rebuild them.
  void *tc_tiles = nullptr;
  size_t tc_tiles_bytes = 0;
  std::string tc_key;
};
DevState g_dev[64];
std::mutex g_dev_mu;  // guards the first-use set-up of g_dev entries

int error_mode()
{
  if (g_mode < 0) {
    const char *e = std::getenv("CONTRACT_ERROR_MODE");
    g_mode = (e && std::strcmp(e, "record") == 0) ? CONTRACT_ERRORS_RECORD : CONTRACT_ERRORS_EXIT;
  }
  return g_mode;
}

// Report an error according to the error mode.  Always returns false.
bool fail(int code, int exit_code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (error_mode() == CONTRACT_ERRORS_EXIT) {
    std::fprintf(stderr, "Error: %s\n", buf);
    std::exit(exit_code);
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_err == CONTRACT_SUCCESS) {
    g_err = code;
    g_msg = buf;
  }
  return false;
}

bool invalid(const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return fail(CONTRACT_ERROR_INVALID_ARGUMENT, -1, "%s", buf);
}

bool cuda_ok(cudaError_t e, const char *what)
{
  if (e == cudaSuccess) return true;
  if (e == cudaErrorMemoryAllocation)
    return fail(CONTRACT_ERROR_OUT_OF_MEMORY, (int)e, "CUDA error in %s: %s", what, cudaGetErrorString(e));
  return fail(CONTRACT_ERROR_CUDA, (int)e, "CUDA error in %s: %s", what, cudaGetErrorString(e));
}

DevState *dev_state()
{
  int d = 0;
  if (!cuda_ok(cudaGetDevice(&d), "cudaGetDevice")) return nullptr;
  if (d < 0 || d >= 64) {
    invalid("device ordinal %d out of range", d);
    return nullptr;
  }
  DevState &s = g_dev[d];
  // first use on a device: two host threads may get here at once
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (s.num_sms == 0) {
    int sms = 0;
    if (!cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d), "cudaDeviceGetAttribute"))
      return nullptr;
    cgb::DeviceStatus *st = nullptr;
    if (!cuda_ok(cgb::device_status_ptr(&st), "cudaGetSymbolAddress")) return nullptr;
    s.status = st;
    s.num_sms = sms;
  }
  return &s;
}

// Per-device scratch for per-timeslice partial sums; grows, never shrinks.
struct DeviceWorkspace : cgb::Workspace {
  DevState *s;
  explicit DeviceWorkspace(DevState *st) : s(st) { }
  void *get(size_t bytes) override
  {
    if (bytes <= s->ws_bytes) return s->ws;
    size_t want = bytes > 2 * s->ws_bytes ? bytes : 2 * s->ws_bytes;
    want = (want + 4095) & ~size_t(4095);
    if (s->ws) {
      // Kernels queued earlier may still read the old buffer.
      if (cudaDeviceSynchronize() != cudaSuccess) return nullptr;
      cudaFree(s->ws);
      s->ws = nullptr;
      s->ws_bytes = 0;
    }
    void *p = nullptr;
    if (cudaMalloc(&p, want) != cudaSuccess) return nullptr;
    s->ws = p;
    s->ws_bytes = want;
    return p;
  }
};

// Hands out the library's fixed static scratch array; never allocates.  A
// request larger than the array is remembered and refused.
struct StaticWorkspace : cgb::Workspace {
  void *base = nullptr;
  size_t cap = 0;
  size_t requested = 0;
  void *get(size_t bytes) override
  {
    requested = bytes;
    return bytes <= cap ? base : nullptr;
  }
};

// ------------------------------------------------------------- autotuner --
// Ops with several compiled tile shapes (Kind in launch.hpp) are tuned per
// (op, precision, projector count, lattice shape): the first call with a new
// key times every variant on the call's own data (one warm-up launch, then two
// timed launches each, CUDA events on the library's stream), keeps the fastest
// and re-launches it so the output is that variant's.  Choices live in memory
// and, when CONTRACT_TUNE_CACHE names a file, are appended there and read
// back by later processes.  Tuning is off unless CONTRACT_AUTOTUNE=1 or
// contract_set_autotune(1); it never runs during stream capture.  Untuned
// calls use each launcher's default variant.
struct TuneEntry {
  int variant;
  float ms;
  std::string name;
};

struct Tuner {
  std::mutex mu;
  std::map<std::string, TuneEntry> choice;
  // batched launches: per lattice class, the time of every tile shape
  std::map<std::string, std::vector<float>> class_ms;
  int enabled = -1;
  bool loaded = false;
  std::string path;
};
Tuner g_tune;

bool autotune_enabled()
{
  if (g_tune.enabled < 0) {
    const char *e = std::getenv("CONTRACT_AUTOTUNE");
    g_tune.enabled = (e && e[0] == '1') ? 1 : 0;
  }
  return g_tune.enabled == 1;
}

std::string tune_key(cgb::Kind kind, const cgb::Job &job, int aux)
{
  std::ostringstream k;
  k << "kind=" << (int)kind << ",prec=" << (int)job.prec << ",aux=" << aux << ",volume=" << job.volume
    << ",lt=" << (job.per_site ? 0 : job.lt) << ",half=" << job.half_slice;
  return k.str();
}

// Caller holds g_tune.mu.
void tune_load_locked()
{
  if (g_tune.loaded) return;
  g_tune.loaded = true;
  const char *p = std::getenv("CONTRACT_TUNE_CACHE");
  if (!p || !*p) return;
  g_tune.path = p;
  std::ifstream f(g_tune.path);
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ls(line);
    std::string key, name;
    int v = -1;
    float ms = 0;
    if (std::getline(ls, key, '\t') && (ls >> v >> name >> ms)) g_tune.choice[key] = {v, ms, name};
  }
}

bool stream_capturing(cudaStream_t s)
{
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) return true;
  return st != cudaStreamCaptureStatusNone;
}

template <class Launch> cudaError_t tuned_launch(cgb::Kind kind, cgb::Job job, int aux, Launch launch)
{
  const char *const *names = nullptr;
  const int n = cgb::launch_variants(kind, job.prec, aux, &names);
  if (n <= 1 || job.volume == 0) return launch(job);
  const std::string key = tune_key(kind, job, aux);
  int v = -1;
  {
    std::lock_guard<std::mutex> lk(g_tune.mu);
    tune_load_locked();
    auto it = g_tune.choice.find(key);
    if (it != g_tune.choice.end() && it->second.variant < n && it->second.name == names[it->second.variant])
      v = it->second.variant;
  }
  if (v < 0 && autotune_enabled() && !stream_capturing(job.stream)) {
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return cudaGetLastError();
    if (cudaEventCreate(&e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      return cudaGetLastError();
    }
    float best = INFINITY;
    for (int c = 0; c < n; ++c) {
      job.variant = c;
      if (launch(job) != cudaSuccess) continue;
      cudaEventRecord(e0, job.stream);
      cudaError_t e = launch(job);
      if (e == cudaSuccess) e = launch(job);
      cudaEventRecord(e1, job.stream);
      if (e != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) continue;
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms / 2 < best) {
        best = ms / 2;
        v = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (v >= 0) {
      std::lock_guard<std::mutex> lk(g_tune.mu);
      g_tune.choice[key] = {v, best, names[v]};
      if (!g_tune.path.empty()) {
        std::ofstream f(g_tune.path, std::ios::app);
        f << key << '\t' << v << ' ' << names[v] << ' ' << best << '\n';
      }
    }
  }
  job.variant = v;
  return launch(job);
}

// Tile shape of a batched launch, tuned per lattice extent: each class of
// items (one lattice shape) is timed alone under every shape (one item of
// the class, a warm-up run and two timed runs), which gives that class's
// best shape in the report; one launch serves every item, so the batch takes
// the shape with the least sum over its items of their class's time.
// classes: (class key, item count); run_one(c, v) runs one item of class c
// under shape v.  Returns the shape, or -1 (the launcher's default) when
// tuning is off and nothing is cached.
int tune_batch(const std::string &tag, int nvariants, const char *const *names,
               const std::vector<std::pair<std::string, int>> &classes,
               const std::function<cudaError_t(int, int)> &run_one, cudaStream_t stream)
{
  std::string comp = tag + ",batch=";
  for (const auto &c : classes) comp += c.first + "x" + std::to_string(c.second) + ";";
  std::vector<std::vector<float>> times(classes.size());
  bool have_all = true;
  {
    std::lock_guard<std::mutex> lk(g_tune.mu);
    tune_load_locked();
    for (size_t c = 0; c < classes.size(); ++c) {
      auto it = g_tune.class_ms.find(tag + ",latt=" + classes[c].first);
      if (it != g_tune.class_ms.end() && (int)it->second.size() == nvariants) times[c] = it->second;
      else have_all = false;
    }
    if (!have_all) {
      auto it = g_tune.choice.find(comp);
      if (it != g_tune.choice.end() && it->second.variant < nvariants && it->second.name == names[it->second.variant])
        return it->second.variant;
    }
  }
  if (!have_all) {
    if (!autotune_enabled() || stream_capturing(stream)) return -1;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return -1;
    if (cudaEventCreate(&e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      return -1;
    }
    for (size_t c = 0; c < classes.size(); ++c) {
      if (!times[c].empty()) continue;
      std::vector<float> ms(nvariants, INFINITY);
      for (int v = 0; v < nvariants; ++v) {
        if (run_one((int)c, v) != cudaSuccess) continue;
        cudaEventRecord(e0, stream);
        cudaError_t e = run_one((int)c, v);
        if (e == cudaSuccess) e = run_one((int)c, v);
        cudaEventRecord(e1, stream);
        if (e != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) continue;
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        ms[v] = t / 2;
      }
      times[c] = ms;
      const int best = (int)(std::min_element(ms.begin(), ms.end()) - ms.begin());
      const std::string key = tag + ",latt=" + classes[c].first;
      std::lock_guard<std::mutex> lk(g_tune.mu);
      g_tune.class_ms[key] = ms;
      g_tune.choice[key] = {best, ms[best], names[best]};
      if (!g_tune.path.empty()) {
        std::ofstream f(g_tune.path, std::ios::app);
        f << key << '\t' << best << ' ' << names[best] << ' ' << ms[best] << '\n';
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  int v = 0;
  float best = INFINITY;
  for (int cand = 0; cand < nvariants; ++cand) {
    float sum = 0;
    for (size_t c = 0; c < classes.size(); ++c) sum += classes[c].second * times[c][cand];
    if (sum < best) {
      best = sum;
      v = cand;
    }
  }
  if (!std::isfinite(best)) return -1;
  std::lock_guard<std::mutex> lk(g_tune.mu);
  g_tune.choice[comp] = {v, best, names[v]};
  if (!g_tune.path.empty()) {
    std::ofstream f(g_tune.path, std::ios::app);
    f << comp << '\t' << v << ' ' << names[v] << ' ' << best << '\n';
  }
  return v;
}

bool gamma_ok(int g, const char *name)
{
  if (g >= 0 && g < 16) return true;
  return invalid("Invalid %s value %d", name, g);
}

bool prec_ok(int p)
{
  if (p == CONTRACT_C128 || p == CONTRACT_C64) return true;
  return invalid("Invalid precision value %d", p);
}

// Device buffers are moved with 16-byte bulk copies and 16-byte stores, so
// every pointer must be 16-byte aligned (any complex128 array is; a complex64
// view starting at an odd element is not).
bool ptr_ok(const void *p, size_t volume, const char *name)
{
  if (volume == 0) return true;
  if (p == nullptr) return invalid("%s is NULL", name);
  if (reinterpret_cast<uintptr_t>(p) & 15u) return invalid("%s must be 16-byte aligned", name);
  return true;
}

// Build the job: per-site (lattice == nullptr) or per-timeslice.  The
// arguments are validated before any CUDA call is made.
bool make_job(cgb::Job &job, int precision, size_t volume, const int *lattice, DevState **state = nullptr)
{
  job.per_site = lattice == nullptr;
  if (lattice) {
    const long long lx = lattice[0], ly = lattice[1], lz = lattice[2], lt = lattice[3];
    if (lx <= 0 || ly <= 0 || lz <= 0 || lt <= 0 || (lx & 1))
      return invalid("invalid lattice {%lld, %lld, %lld, %lld} (positive extents, Lx even)", lx, ly, lz, lt);
    if (lx * ly * lz * lt != (long long)volume)
      return invalid("volume %zu does not match lattice {%lld, %lld, %lld, %lld}", volume, lx, ly, lz, lt);
    job.lt = (int)lt;
    job.half_slice = lx * ly * lz / 2;
  }
  DevState *s = dev_state();
  if (!s) return false;
  job.prec = precision == CONTRACT_C64 ? cgb::Prec::C64 : cgb::Prec::C128;
  job.stream = g_stream;
  job.status = s->status;
  job.num_sms = s->num_sms;
  job.volume = (long long)volume;
  job.wait_ns = g_wait_ns;
  job.withhold_chunk = g_withhold_chunk;  // one call only
  g_withhold_chunk = -1;
  if (state) *state = s;
  return true;
}

void set_row(uint8_t dst[4], const uint8_t src[4])
{
  for (int k = 0; k < 4; ++k) dst[k] = src[k];
}

// Fill the projector operand from Gamma(gamma_mn) or a host 4x4 complex array.
void fill_proj(cgb::ProjOperand<double> &w, int gamma_mn, const double *project_mn)
{
  w = {};
  if (!project_mn) {
    const cgb::SignedPerm g = cgb::sp_gamma(gamma_mn);
    static const double re[4] = {1, 0, -1, 0}, im[4] = {0, 1, 0, -1};
    for (int m = 0; m < 4; ++m) {
      w.perm[m] = (uint8_t)g.perm[m];
      w.ph[m] = (uint8_t)g.ph[m];
      w.w[m * 4 + g.perm[m]][0] = re[g.ph[m]];
      w.w[m * 4 + g.perm[m]][1] = im[g.ph[m]];
    }
    w.is_perm = 1;
    return;
  }
  for (int k = 0; k < 16; ++k) {
    w.w[k][0] = project_mn[2 * k];
    w.w[k][1] = project_mn[2 * k + 1];
    if (w.w[k][0] != 0.0 || w.w[k][1] != 0.0) {
      w.nzk[w.nnz++] = (uint8_t)k;
      w.nzmask |= 1u << k;
    }
  }
  // A phased permutation (one entry in {1, i, -1, -i} per row, distinct
  // columns) is applied with index/sign operations instead of multiplies.
  bool perm = true;
  int used = 0;
  for (int m = 0; m < 4 && perm; ++m) {
    int nz = 0, col = -1;
    for (int n = 0; n < 4; ++n)
      if (w.w[m * 4 + n][0] != 0.0 || w.w[m * 4 + n][1] != 0.0) {
        ++nz;
        col = n;
      }
    if (nz != 1 || (used >> col) & 1) {
      perm = false;
      break;
    }
    used |= 1 << col;
    const double a = w.w[m * 4 + col][0], b = w.w[m * 4 + col][1];
    int ph = -1;
    if (a == 1.0 && b == 0.0) ph = 0;
    else if (a == 0.0 && b == 1.0) ph = 1;
    else if (a == -1.0 && b == 0.0) ph = 2;
    else if (a == 0.0 && b == -1.0) ph = 3;
    if (ph < 0) perm = false;
    w.perm[m] = (uint8_t)col;
    w.ph[m] = (uint8_t)(ph < 0 ? 0 : ph);
  }
  w.is_perm = perm ? 1 : 0;
}

// Write the projectors W_w (w < nw, each 16 complex row-major, or Gamma(gamma_mn)
// when `projs` is null) in the gamma basis: W = sum_g c_g Gamma(g) with
// c_g = Tr(Gamma(g)^dagger W) / 4 = (1/4) sum_m i^(-ph_g(m)) W[m][perm_g(m)].
void fill_clifford(cgb::CliffordSet<double> &cl, const double *const *projs, int nw, int gamma_mn)
{
  cl = {};
  static const double re[4] = {1, 0, -1, 0}, im[4] = {0, 1, 0, -1};
  double c[2][16][2] = {};
  bool used[16] = {};
  for (int w = 0; w < nw; ++w) {
    if (!projs) {
      c[w][gamma_mn][0] = 1.0;
      used[gamma_mn] = true;
      continue;
    }
    for (int g = 0; g < 16; ++g) {
      const cgb::SignedPerm sp = cgb::sp_gamma(g);
      double x = 0, y = 0;
      for (int m = 0; m < 4; ++m) {
        const double *wv = projs[w] + 2 * (m * 4 + sp.perm[m]);
        // multiply by conj(i^ph) = i^(-ph)
        const double cr = re[sp.ph[m]], ci = -im[sp.ph[m]];
        x += cr * wv[0] - ci * wv[1];
        y += cr * wv[1] + ci * wv[0];
      }
      c[w][g][0] = x / 4;
      c[w][g][1] = y / 4;
      if (x != 0.0 || y != 0.0) used[g] = true;
    }
  }
  for (int g = 0; g < 16; ++g) {
    if (!used[g]) continue;
    const int k = cl.ng++;
    const cgb::SignedPerm sp = cgb::sp_gamma(g);
    for (int m = 0; m < 4; ++m) {
      cl.perm[k][m] = (uint8_t)sp.perm[m];
      cl.ph[k][m] = (uint8_t)sp.ph[m];
      if (sp.ph[m]) cl.has_phase[k] = 1;
    }
    for (int w = 0; w < nw; ++w) {
      cl.coef[w][k][0] = c[w][g][0];
      cl.coef[w][k][1] = c[w][g][1];
      for (int m = 0; m < 4; ++m) {  // coef * i^ph[k][m]
        const double pr = re[cl.ph[k][m]], pi = im[cl.ph[k][m]];
        cl.qc[w][k][m][0] = c[w][g][0] * pr - c[w][g][1] * pi;
        cl.qc[w][k][m][1] = c[w][g][0] * pi + c[w][g][1] * pr;
      }
    }
  }
}

// A projector W (4x4 complex, row-major) of rank r <= 2 as W = sum_r x_r y_r^T,
// by elimination with complete pivoting: pivot (p, q) of the remainder E,
// x_r = E[., q] / E[p][q], y_r = E[p][.], E -= x_r y_r^T.  Taken only when the
// remainder after at most two steps is exactly zero, so that the factors give W
// back to rounding; otherwise rk.r stays 0 and the triangle form uses N'.
void fill_rank(cgb::RankForm<double> &rk, const double *w)
{
  rk = {};
  double e[4][4][2], x[2][4][2] = {}, y[2][4][2] = {};
  std::memcpy(e, w, sizeof(e));
  for (int k = 0; k < 32; ++k)
    if (!std::isfinite(w[k])) return;  // N' carries NaN and Inf through as the reference does
  int r = 0;
  for (;;) {
    int p = -1, q = -1;
    double best = 0.0;
    for (int m = 0; m < 4; ++m)
      for (int n = 0; n < 4; ++n) {
        const double a = e[m][n][0] * e[m][n][0] + e[m][n][1] * e[m][n][1];
        if (a > best) {
          best = a;
          p = m;
          q = n;
        }
      }
    if (p < 0) break;    // the remainder is zero: rank r
    if (r == 2) return;  // rank > 2
    const double pr = e[p][q][0], pi = e[p][q][1];
    for (int m = 0; m < 4; ++m) {  // E[m][q] / E[p][q]
      x[r][m][0] = (e[m][q][0] * pr + e[m][q][1] * pi) / best;
      x[r][m][1] = (e[m][q][1] * pr - e[m][q][0] * pi) / best;
    }
    x[r][p][0] = 1.0;
    x[r][p][1] = 0.0;
    for (int n = 0; n < 4; ++n) {
      y[r][n][0] = e[p][n][0];
      y[r][n][1] = e[p][n][1];
    }
    for (int m = 0; m < 4; ++m)
      for (int n = 0; n < 4; ++n) {
        e[m][n][0] -= x[r][m][0] * y[r][n][0] - x[r][m][1] * y[r][n][1];
        e[m][n][1] -= x[r][m][0] * y[r][n][1] + x[r][m][1] * y[r][n][0];
      }
    for (int k = 0; k < 4; ++k) {  // row p and column q are eliminated
      e[p][k][0] = e[p][k][1] = 0.0;
      e[k][q][0] = e[k][q][1] = 0.0;
    }
    ++r;
  }
  if (r == 0) return;
  int nnz = 1;
  for (int side = 0; side < 2; ++side)
    for (int k = 0; k < r; ++k) {
      const double(*v)[2] = side ? y[k] : x[k];
      int c = 0;
      for (int t = 0; t < 4; ++t)
        if (v[t][0] != 0.0 || v[t][1] != 0.0) {
          rk.idx[side][k][c] = (uint8_t)t;
          rk.c[side][k][c][0] = v[t][0];
          rk.c[side][k][c][1] = v[t][1];
          ++c;
        }
      nnz = std::max(nnz, c);
    }
  rk.r = r;
  rk.nnz = nnz;
  // Unit form: within each vector every nonzero entry is the same modulus times
  // a power of i, and the product of a pair's two moduli is the same for every r.
  rk.unit = 1;
  double scale = 0.0;
  for (int k = 0; k < r && rk.unit; ++k) {
    double mod[2];
    for (int side = 0; side < 2 && rk.unit; ++side) {
      mod[side] = 0.0;
      for (int t = 0; t < nnz && rk.unit; ++t) {
        const double a = rk.c[side][k][t][0], b = rk.c[side][k][t][1];
        if (a == 0.0 && b == 0.0) {  // a padded list: the device adds every entry
          rk.unit = 0;
          break;
        }
        const double m = std::fabs(a) + std::fabs(b);  // one of a, b is zero for a phase
        if (mod[side] == 0.0) mod[side] = m;
        int ph = -1;
        if (a == m && b == 0.0) ph = 0;
        else if (a == 0.0 && b == m) ph = 1;
        else if (a == -m && b == 0.0) ph = 2;
        else if (a == 0.0 && b == -m) ph = 3;
        if (ph < 0 || m != mod[side]) rk.unit = 0;
        else rk.ph[side][k][t] = (uint8_t)ph;
      }
    }
    if (!rk.unit) break;
    const double s = mod[0] * mod[1];
    if (k == 0) scale = s;
    else if (s != scale) rk.unit = 0;
  }
  rk.scale = rk.unit ? scale : 1.0;
}

// Contraction type -> canonical form (see ops.cuh): loop or triangle, whether
// P_i and P_j swap roles, and the c1/c2 phase rows.
struct TypeForm {
  bool loop, swap_ij;
  const uint8_t *c1, *c2;
};

TypeForm type_form(int type, int gij, int gkl)
{
  const bool sij = type == IM_JK_NL || type == IM_JL_NK;
  const bool skl = type == IL_JK_NM || type == IL_JM_NK || type == IM_JL_NK;
  TypeForm f;
  f.loop = type == IK_JL_NM || type == IL_JK_NM;
  f.swap_ij = sij;
  f.c1 = sij ? kG.ph_t[gij] : kG.ph[gij];
  f.c2 = skl ? kG.ph[gkl] : kG.ph_t[gkl];
  return f;
}

bool type_ok(int type)
{
  if (type >= 0 && type < 6) return true;
  return invalid("Invalid contract_type value %d", type);
}

void do_meson(void *correl, const void *pi, const void *pj, size_t volume, int gij, int gkl, int prec,
              const int *lattice)
{
  if (!gamma_ok(gij, "gamma_ij") || !gamma_ok(gkl, "gamma_kl") || !prec_ok(prec)) return;
  if (!ptr_ok(correl, volume, "correl") || !ptr_ok(pi, volume, "propag_i") || !ptr_ok(pj, volume, "propag_j")) return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, prec, volume, lattice, &s)) return;
  DeviceWorkspace ws(s);
  job.ws = &ws;
  OpParams<double> p {};
  p.in[0] = pi;
  p.in[1] = pj;
  p.out[0] = correl;
  set_row(p.m.perm1, kG.perm[gij]);
  set_row(p.m.ph1, kG.ph_g5g_t[gij]);
  set_row(p.m.perm2, kG.perm[gkl]);
  set_row(p.m.ph2, kG.ph_g5g_t[gkl]);
  cuda_ok(tuned_launch(cgb::Kind::Meson, job, 0, [&](const cgb::Job &j) { return cgb::launch_meson(j, p); }),
          "meson_two_point");
}

void do_meson_all(void **correl, const void *pi, const void *pj, size_t volume, int gamma, bool source, int prec,
                  const int *lattice)
{
  if (!gamma_ok(gamma, source ? "gamma_ij" : "gamma_kl") || !prec_ok(prec)) return;
  if (!correl) {
    invalid("correl pointer array is NULL");
    return;
  }
  for (int g = 0; g < 16; ++g)
    if (!ptr_ok(correl[g], volume, "correl[g]")) return;
  if (!ptr_ok(pi, volume, "propag_i") || !ptr_ok(pj, volume, "propag_j")) return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, prec, volume, lattice, &s)) return;
  DeviceWorkspace ws(s);
  job.ws = &ws;
  OpParams<double> p {};
  p.in[0] = pi;
  p.in[1] = pj;
  for (int g = 0; g < 16; ++g) p.out[g] = correl[g];
  set_row(p.m.perm1, kG.perm[gamma]);
  set_row(p.m.ph1, kG.ph_g5g_t[gamma]);
  set_row(p.m.perm2, kG.perm[gamma]);
  set_row(p.m.ph2, kG.ph_g5g_t[gamma]);
  cuda_ok(tuned_launch(cgb::Kind::MesonAll, job, source ? 1 : 0,
                       [&](const cgb::Job &j) { return cgb::launch_meson_all(j, source, p); }),
          source ? "meson_all_source_two_point" : "meson_all_sink_two_point");
}

void do_baryon(void *correl, const void *pi, const void *pj, const void *pn, int type, size_t volume, int gij, int gkl,
               int gmn, const double *proj, int prec, const int *lattice)
{
  if (!type_ok(type)) return;
  if (!proj && !gamma_ok(gmn, "gamma_mn")) return;
  if (!gamma_ok(gij, "gamma_ij") || !gamma_ok(gkl, "gamma_kl") || !prec_ok(prec)) return;
  if (!ptr_ok(correl, volume, "correl") || !ptr_ok(pi, volume, "propag_i") || !ptr_ok(pj, volume, "propag_j") ||
      !ptr_ok(pn, volume, "propag_n"))
    return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, prec, volume, lattice, &s)) return;
  DeviceWorkspace ws(s);
  job.ws = &ws;
  const TypeForm f = type_form(type, gij, gkl);
  OpParams<double> p {};
  p.in[0] = f.swap_ij ? pj : pi;
  p.in[1] = f.swap_ij ? pi : pj;
  p.in[2] = pn;
  p.out[0] = correl;
  set_row(p.b.perm1, kG.perm[gij]);
  set_row(p.b.perm2, kG.perm[gkl]);
  set_row(p.b.ph1[0], f.c1);
  set_row(p.b.ph2[0], f.c2);
  fill_proj(p.b.proj[0], gmn, proj);
  fill_clifford(p.b.cl, proj ? &proj : nullptr, 1, gmn);
  if (proj) fill_rank(p.b.rk, proj);
  const cgb::Kind kind = f.loop ? cgb::Kind::BaryonLoop : cgb::Kind::BaryonTri;
  auto run = [&](const cgb::Job &j) { return cgb::launch_baryon(j, f.loop, p); };
  // aux 0: gamma-basis triangle (one gamma), 1: triangle with N' materialised,
  // 2: triangle with a projector of rank <= 2
  const int aux = (f.loop || p.b.cl.ng == 1) ? 0 : (p.b.rk.r > 0 ? 2 : 1);
  const cudaError_t e = tuned_launch(kind, job, aux, run);
  cuda_ok(e, proj ? "baryon_general_two_point" : "baryon_two_point");
}

void do_diquark(void *dq, const void *pi, const void *pj, size_t volume, int gij, int gkl, int prec)
{
  if (gij < 0 || gij >= 16) {
    // The reference silently skips an unknown gamma_ij (lib/baryon/diquark.cu:40).
    if (error_mode() == CONTRACT_ERRORS_RECORD) invalid("Invalid gamma_ij value %d", gij);
    return;
  }
  if (!gamma_ok(gkl, "gamma_kl") || !prec_ok(prec)) return;
  if (!ptr_ok(dq, volume, "diquark") || !ptr_ok(pi, volume, "propag_i") || !ptr_ok(pj, volume, "propag_j")) return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, prec, volume, nullptr, &s)) return;
  OpParams<double> p {};
  p.in[0] = pi;
  p.in[1] = pj;
  p.out[0] = dq;
  set_row(p.b.perm1, kG.perm[gij]);
  set_row(p.b.ph1[0], kG.ph[gij]);
  set_row(p.b.perm2, kG.perm[gkl]);
  set_row(p.b.ph2[0], kG.ph_t[gkl]);
  cuda_ok(tuned_launch(cgb::Kind::Diquark, job, 0, [&](const cgb::Job &j) { return cgb::launch_diquark(j, p); }),
          "baryon_diquark");
}

void do_sequential(void *pi, void *pj, void *pn, int type, int seq, size_t volume, int gij, int gkl, int gmn, int prec)
{
  if (seq < 0 || seq > 2) {
    // The reference silently skips an unknown sequential_type (lib/contract.cpp:60).
    if (error_mode() == CONTRACT_ERRORS_RECORD) invalid("Invalid sequential_type value %d", seq);
    return;
  }
  if (!type_ok(type) || !gamma_ok(gmn, "gamma_mn") || !gamma_ok(gij, "gamma_ij") || !gamma_ok(gkl, "gamma_kl") ||
      !prec_ok(prec))
    return;
  if (!ptr_ok(pi, volume, "propag_i") || !ptr_ok(pj, volume, "propag_j") || !ptr_ok(pn, volume, "propag_n")) return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, prec, volume, nullptr, &s)) return;
  const TypeForm f = type_form(type, gij, gkl);
  const void *a = f.swap_ij ? pj : pi, *b = f.swap_ij ? pi : pj;
  // Differentiated role: 0 = A, 1 = B, 2 = P_n.
  const int role = seq == SEQUENTIAL_N ? 2 : (((seq == SEQUENTIAL_I) != f.swap_ij) ? 0 : 1);
  OpParams<double> p {};
  if (role == 0) {
    p.in[0] = b;
    p.in[1] = pn;
  } else if (role == 1) {
    p.in[0] = a;
    p.in[1] = pn;
  } else {
    p.in[0] = a;
    p.in[1] = b;
  }
  p.out[0] = seq == SEQUENTIAL_I ? pi : (seq == SEQUENTIAL_J ? pj : pn);
  set_row(p.b.perm1, kG.perm[gij]);
  set_row(p.b.perm2, kG.perm[gkl]);
  set_row(p.b.ph1[0], f.c1);
  set_row(p.b.ph2[0], f.c2);
  fill_proj(p.b.proj[0], gmn, nullptr);
  cuda_ok(tuned_launch(cgb::Kind::Sequential, job, (f.loop ? 3 : 0) + role,
                       [&](const cgb::Job &j) { return cgb::launch_sequential(j, f.loop, role, p); }),
          "baryon_sequential_two_point");
}

// Build the momentum plan: distinct nx, distinct (nx, ny) pairs, FP64 phase tables.
bool make_mom_plan(cgb::MomPlan &plan, const int *lattice, const int *moms, int nmom)
{
  plan = {};
  for (int k = 0; k < 4; ++k) plan.latt[k] = lattice[k];
  if (lattice[0] > cgb::kMomMaxL || lattice[1] > cgb::kMomMaxL || lattice[2] > cgb::kMomMaxL)
    return invalid("momentum projection supports spatial extents up to %d", cgb::kMomMaxL);
  if (nmom < 1 || nmom > cgb::kMomMaxP) return invalid("nmom must be 1..%d (got %d)", cgb::kMomMaxP, nmom);
  plan.np = nmom;
  for (int p = 0; p < nmom; ++p) {
    const int nx = moms[3 * p], ny = moms[3 * p + 1], nz = moms[3 * p + 2];
    int ix = -1;
    for (int k = 0; k < plan.npx; ++k)
      if (plan.px[k] == nx) ix = k;
    if (ix < 0) {
      if (plan.npx == cgb::kMomMaxPx) return invalid("at most %d distinct x momenta per call", cgb::kMomMaxPx);
      ix = plan.npx++;
      plan.px[ix] = nx;
    }
    int iq = -1;
    for (int k = 0; k < plan.nq; ++k)
      if (plan.q_ix[k] == ix && plan.q_ny[k] == ny) iq = k;
    if (iq < 0) {
      if (plan.nq == cgb::kMomMaxQ) return invalid("at most %d distinct (x, y) momentum pairs per call", cgb::kMomMaxQ);
      iq = plan.nq++;
      plan.q_ix[iq] = ix;
      plan.q_ny[iq] = ny;
    }
    plan.p_q[p] = iq;
    plan.p_nz[p] = nz;
  }
  // +n / -n groups of the X and Z transforms (see MomPlan).  k = min(m, L - m) for m = n mod L; the sign
  // is + when m == k.  A momentum joins an open group of its k and sign slot,
  // else starts one (duplicates get groups of their own).
  auto key = [](int n, int L, bool &plus) {
    const int m = ((n % L) + L) % L, k = m <= L - m ? m : L - m;
    plus = m == k;
    return k;
  };
  plan.ngx = 0;
  for (int ip = 0; ip < plan.npx; ++ip) {
    bool plus;
    const int k = key(plan.px[ip], lattice[0], plus);
    int gsel = -1;
    for (int gi = 0; gi < plan.ngx && gsel < 0; ++gi)
      if (plan.gx_k[gi] == k && (plus ? plan.gx_plus[gi] : plan.gx_minus[gi]) < 0) gsel = gi;
    if (gsel < 0) {
      gsel = plan.ngx++;
      plan.gx_k[gsel] = k;
      plan.gx_plus[gsel] = plan.gx_minus[gsel] = -1;
    }
    (plus ? plan.gx_plus[gsel] : plan.gx_minus[gsel]) = ip;
  }
  for (int gi = 1; gi < plan.ngx; ++gi)  // the nx = 0 group first: its transform is a plain sum
    if (plan.gx_k[gi] == 0) {
      std::swap(plan.gx_k[0], plan.gx_k[gi]);
      std::swap(plan.gx_plus[0], plan.gx_plus[gi]);
      std::swap(plan.gx_minus[0], plan.gx_minus[gi]);
    }
  int ng = 0;
  for (int q = 0; q < plan.nq; ++q) {
    plan.q_g0[q] = ng;
    for (int pm = 0; pm < nmom; ++pm) {
      if (plan.p_q[pm] != q) continue;
      bool plus;
      const int k = key(plan.p_nz[pm], lattice[2], plus);
      int gsel = -1;
      for (int gi = plan.q_g0[q]; gi < ng && gsel < 0; ++gi)
        if (plan.gz_k[gi] == k && (plus ? plan.gz_plus[gi] : plan.gz_minus[gi]) < 0) gsel = gi;
      if (gsel < 0) {
        gsel = ng++;
        plan.gz_k[gsel] = k;
        plan.gz_plus[gsel] = plan.gz_minus[gsel] = -1;
      }
      (plus ? plan.gz_plus[gsel] : plan.gz_minus[gsel]) = pm;
    }
  }
  plan.q_g0[plan.nq] = ng;
  const double two_pi = 6.283185307179586476925286766559;
  for (int k = 0; k < lattice[0]; ++k) {
    plan.cosx[k] = std::cos(two_pi * k / lattice[0]);
    plan.sinx[k] = std::sin(two_pi * k / lattice[0]);
  }
  for (int k = 0; k < lattice[1]; ++k) {
    plan.cosy[k] = std::cos(two_pi * k / lattice[1]);
    plan.siny[k] = std::sin(two_pi * k / lattice[1]);
  }
  for (int k = 0; k < lattice[2]; ++k) {
    plan.cosz[k] = std::cos(two_pi * k / lattice[2]);
    plan.sinz[k] = std::sin(two_pi * k / lattice[2]);
  }
  return true;
}

// Arguments shared by the all-types entry points.
bool all_types_args_ok(int gamma_ij, int gamma_kl, int nproj, const void *projectors, int precision)
{
  if (nproj < 1 || nproj > 2) return invalid("nproj must be 1 or 2 (got %d)", nproj);
  if (!projectors) return invalid("projectors is NULL");
  return gamma_ok(gamma_ij, "gamma_ij") && gamma_ok(gamma_kl, "gamma_kl") && prec_ok(precision);
}

// Inputs, outputs (nproj x 6 rows of `stride` values), spin tables and
// projectors of the fused all-types op.
void fill_all_types(OpParams<double> &p, const void *pi, const void *pj, const void *pn, void *correl, size_t stride,
                    int gamma_ij, int gamma_kl, int nproj, const void *projectors)
{
  p.in[0] = pi;
  p.in[1] = pj;
  p.in[2] = pn;
  for (int o = 0; o < 6 * nproj; ++o) p.out[o] = correl ? static_cast<char *>(correl) + o * stride * 16 : nullptr;
  set_row(p.b.perm1, kG.perm[gamma_ij]);
  set_row(p.b.perm2, kG.perm[gamma_kl]);
  set_row(p.b.ph1[0], kG.ph[gamma_ij]);    // A = P_i groups
  set_row(p.b.ph1[1], kG.ph_t[gamma_ij]);  // IM_* group (A = P_j)
  set_row(p.b.ph2[0], kG.ph_t[gamma_kl]);  // IK_JL_NM, IK_JM_NL, IM_JK_NL
  set_row(p.b.ph2[1], kG.ph[gamma_kl]);    // IL_JK_NM, IL_JM_NK, IM_JL_NK
  const double *pr = static_cast<const double *>(projectors);
  const double *pw[2] = {pr, pr + 32};
  for (int w = 0; w < nproj; ++w) fill_proj(p.b.proj[w], 0, pw[w]);
  fill_clifford(p.b.cl, pw, nproj, 0);
  if (nproj == 1) fill_rank(p.b.rk, pw[0]);
}

cudaError_t run_all_types(const cgb::Job &job, const OpParams<double> &p, int nproj)
{
  auto run = [&](const cgb::Job &j) { return cgb::launch_baryon_fused(j, nproj, p); };
  const int aux = nproj + (cgb::fused_same_ij(p) ? 4 : 0);
  return p.b.cl.ng <= nproj ? tuned_launch(cgb::Kind::BaryonFused, job, aux, run) : run(job);
}

// Staging memory, copy stream and events of the host-input pipeline.
bool pipeline_ready(DevState *s, size_t bytes)
{
  if (!s->copy) {
    if (!cuda_ok(cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking), "cudaStreamCreateWithFlags")) return false;
    for (int b = 0; b < kPipeSlots; ++b) {
      if (!cuda_ok(cudaEventCreateWithFlags(&s->copied[b], cudaEventDisableTiming), "cudaEventCreateWithFlags") ||
          !cuda_ok(cudaEventCreateWithFlags(&s->freed[b], cudaEventDisableTiming), "cudaEventCreateWithFlags"))
        return false;
    }
    if (!cuda_ok(cudaEventCreateWithFlags(&s->start, cudaEventDisableTiming), "cudaEventCreateWithFlags")) return false;
  }
  if (bytes <= s->pipe_bytes) return true;
  if (s->pipe) {
    // Copies and kernels of an earlier call may still use the old buffer.
    if (!cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize")) return false;
    cudaFree(s->pipe);
    s->pipe = nullptr;
    s->pipe_bytes = 0;
  }
  if (cudaMalloc(&s->pipe, bytes) != cudaSuccess) {
    s->pipe = nullptr;
    return fail(CONTRACT_ERROR_OUT_OF_MEMORY, -1, "cannot allocate %zu bytes for the host-input pipeline", bytes);
  }
  s->pipe_bytes = bytes;
  return true;
}

// ------------------------------------------------------ batched launches --
struct BaryonBatch {
  std::vector<cgb::BatchSpec> specs;
  OpParams<double> p {};
};

// Validates baryon batch items and builds the launch's specs and spin tables.
bool baryon_batch_setup(BaryonBatch &bb, const ContractBaryonBatchItem *items, int nitems, int gamma_ij, int gamma_kl,
                        int nproj, const void *projectors, int precision)
{
  if (nitems < 0 || nitems > 128) return invalid("nitems must be 0..128 (got %d)", nitems);
  if (!items || !projectors) return invalid("items and projectors are required");
  if (nproj < 1 || nproj > 2) return invalid("nproj must be 1 or 2 (got %d)", nproj);
  if (!gamma_ok(gamma_ij, "gamma_ij") || !gamma_ok(gamma_kl, "gamma_kl") || !prec_ok(precision)) return false;
  bb.specs.assign(nitems, cgb::BatchSpec {});
  for (int i = 0; i < nitems; ++i) {
    const ContractBaryonBatchItem &it = items[i];
    const int *l = it.lattice;
    if (l[0] <= 0 || l[1] <= 0 || l[2] <= 0 || l[3] <= 0 || (l[0] & 1))
      return invalid("batch item %d: invalid lattice {%d, %d, %d, %d}", i, l[0], l[1], l[2], l[3]);
    const size_t v = (size_t)l[0] * l[1] * l[2] * l[3];
    if (!ptr_ok(it.correl, v, "correl") || !ptr_ok(it.propag_i, v, "propag_i") ||
        !ptr_ok(it.propag_j, v, "propag_j") || !ptr_ok(it.propag_n, v, "propag_n"))
      return false;
    cgb::BatchSpec &sp = bb.specs[i];
    sp.in[0] = it.propag_i;
    sp.in[1] = it.propag_j;
    sp.in[2] = it.propag_n;
    sp.out = static_cast<double2 *>(it.correl);
    for (int k = 0; k < 4; ++k) sp.latt[k] = l[k];
  }
  OpParams<double> &p = bb.p;
  p = {};
  set_row(p.b.perm1, kG.perm[gamma_ij]);
  set_row(p.b.perm2, kG.perm[gamma_kl]);
  set_row(p.b.ph1[0], kG.ph[gamma_ij]);
  set_row(p.b.ph1[1], kG.ph_t[gamma_ij]);
  set_row(p.b.ph2[0], kG.ph_t[gamma_kl]);
  set_row(p.b.ph2[1], kG.ph[gamma_kl]);
  const double *pr = static_cast<const double *>(projectors);
  const double *pw[2] = {pr, pr + 32};
  for (int w = 0; w < nproj; ++w) fill_proj(p.b.proj[w], 0, pw[w]);
  fill_clifford(p.b.cl, pw, nproj, 0);
  if (nproj == 1) fill_rank(p.b.rk, pw[0]);
  if (p.b.cl.ng > nproj && !(nproj == 1 && p.b.rk.r > 0))
    return invalid("batched contractions need projectors spanned by at most nproj gamma matrices, or one projector "
                   "of rank <= 2 (got %d terms)",
                   p.b.cl.ng);
  return true;
}

// Validates meson momentum batch items and fills the launch parameters (all
// but the plane buffers).  Every item's momentum plan must have the structure
// of the first item's (true for any list of components n with 2|n| < L in
// every direction); phase tables are kept once per distinct extent.
bool meson_batch_setup(cgb::MomBatchParams &mp, size_t &plane_floats, const ContractMesonMomentumBatchItem *items,
                       int nitems, const int *moms, int nmom)
{
  if (nitems < 0 || nitems > cgb::kMomBatchMaxItems)
    return invalid("nmeson must be 0..%d (got %d)", cgb::kMomBatchMaxItems, nitems);
  mp = {};
  plane_floats = 0;
  if (nitems == 0) return true;
  if (!items || !moms) return invalid("meson items and moms are required");
  std::vector<int> ext;  // distinct extents
  auto ext_index = [&](int L) {
    for (size_t e = 0; e < ext.size(); ++e)
      if (ext[e] == L) return (int)e;
    ext.push_back(L);
    return (int)ext.size() - 1;
  };
  cgb::MomPlan first;
  int units = 0, fin = 0;
  for (int i = 0; i < nitems; ++i) {
    const ContractMesonMomentumBatchItem &it = items[i];
    const int *l = it.lattice;
    if (l[0] <= 0 || l[1] <= 0 || l[2] <= 0 || l[3] <= 0 || (l[0] & 1))
      return invalid("meson item %d: invalid lattice {%d, %d, %d, %d}", i, l[0], l[1], l[2], l[3]);
    const size_t v = (size_t)l[0] * l[1] * l[2] * l[3];
    if (!ptr_ok(it.correl, v, "correl") || !ptr_ok(it.propag_i, v, "propag_i") || !ptr_ok(it.propag_j, v, "propag_j"))
      return false;
    cgb::MomPlan plan;
    if (!make_mom_plan(plan, l, moms, nmom)) return false;
    if (i == 0) {
      first = plan;
      if (!cgb::momentum_fused_supported(plan))
        return invalid("batched momentum projection supports up to 3 X groups and %d (nx, ny) pairs", cgb::kMomQChunk);
      if (plan.q_g0[plan.nq] > cgb::kMomBatchMaxG)
        return invalid("batched momentum projection supports up to %d z groups", cgb::kMomBatchMaxG);
    } else {
      bool same = plan.npx == first.npx && plan.nq == first.nq && plan.ngx == first.ngx;
      for (int k = 0; same && k < plan.ngx; ++k)
        same = plan.gx_k[k] == first.gx_k[k] && plan.gx_plus[k] == first.gx_plus[k] &&
               plan.gx_minus[k] == first.gx_minus[k];
      for (int q = 0; same && q <= plan.nq; ++q) same = plan.q_g0[q] == first.q_g0[q];
      for (int q = 0; same && q < plan.nq; ++q) same = plan.q_ix[q] == first.q_ix[q] && plan.q_ny[q] == first.q_ny[q];
      for (int g = 0; same && g < plan.q_g0[plan.nq]; ++g)
        same = plan.gz_k[g] == first.gz_k[g] && plan.gz_plus[g] == first.gz_plus[g] &&
               plan.gz_minus[g] == first.gz_minus[g];
      if (!same)
        return invalid("meson item %d: the momentum list has another structure on lattice {%d, %d, %d, %d} "
                       "than on the first item's", i, l[0], l[1], l[2], l[3]);
    }
    cgb::MomBatchItem &b = mp.items[i];
    b.in[0] = static_cast<const char *>(it.propag_i);
    b.in[1] = static_cast<const char *>(it.propag_j);
    b.out = static_cast<double2 *>(it.correl);
    for (int k = 0; k < 4; ++k) b.latt[k] = l[k];
    b.unit_begin = units;
    b.tpp = (l[0] * l[1] + 15) / 16;
    b.fin_begin = fin;
    const int ex = ext_index(l[0]), ey = ext_index(l[1]), ez = ext_index(l[2]);
    if ((int)ext.size() > cgb::kMomBatchMaxExt)
      return invalid("batched momentum projection supports up to %d distinct spatial extents", cgb::kMomBatchMaxExt);
    b.tx = (uint8_t)ex;
    b.ty = (uint8_t)ey;
    b.tz = (uint8_t)ez;
    // the phase tables of the per-call plan, FP32 as the kernels use them
    for (int k = 0; k < l[0]; ++k) mp.tab[ex][k] = make_float2((float)plan.cosx[k], (float)plan.sinx[k]);
    for (int k = 0; k < l[1]; ++k) mp.tab[ey][k] = make_float2((float)plan.cosy[k], (float)plan.siny[k]);
    for (int k = 0; k < l[2]; ++k) mp.tab[ez][k] = make_float2((float)plan.cosz[k], (float)plan.sinz[k]);
    units += l[2] * l[3];
    fin += first.nq * l[3];
    plane_floats += (size_t)l[2] * l[3] * first.nq * 256 * 2;
  }
  mp.n_items = nitems;
  mp.total_units = units;
  mp.total_fin = fin;
  mp.ngx = first.ngx;
  mp.nq = first.nq;
  mp.np = first.np;
  for (int k = 0; k < first.ngx; ++k) {
    mp.gx_k[k] = first.gx_k[k];
    mp.gx_plus[k] = first.gx_plus[k];
    mp.gx_minus[k] = first.gx_minus[k];
  }
  for (int q = 0; q < first.nq; ++q) {
    mp.q_ix[q] = first.q_ix[q];
    mp.q_ny[q] = first.q_ny[q];
  }
  for (int q = 0; q <= first.nq; ++q) mp.q_g0[q] = first.q_g0[q];
  for (int g = 0; g < first.q_g0[first.nq]; ++g) {
    mp.gz_k[g] = first.gz_k[g];
    mp.gz_plus[g] = first.gz_plus[g];
    mp.gz_minus[g] = first.gz_minus[g];
  }
  return true;
}

std::string latt_key(const int *l)
{
  return std::to_string(l[0]) + "," + std::to_string(l[1]) + "," + std::to_string(l[2]) + "," + std::to_string(l[3]);
}

// A workspace view `off` bytes into another (the momentum planes sit below
// the baryon partials of a mixed batch).
struct OffsetWorkspace : cgb::Workspace {
  cgb::Workspace *base;
  size_t off;
  OffsetWorkspace(cgb::Workspace *b, size_t o) : base(b), off(o) { }
  void *get(size_t bytes) override
  {
    char *p = static_cast<char *>(base->get(off + bytes));
    return p ? p + off : nullptr;
  }
};

// Baryon items and meson momentum items (complex64), each kind in one
// persistent launch with its tile shape tuned per extent, then one combined
// finalisation launch.
void run_mixed_batch(const ContractBaryonBatchItem *bitems, int nb, int gamma_ij, int gamma_kl, int nproj,
                     const void *projectors, const ContractMesonMomentumBatchItem *mitems, int nm, const int *moms,
                     int nmom, int precision, const char *what)
{
  if (precision != CONTRACT_C64) {
    invalid("%s needs CONTRACT_C64 propagators (got precision %d)", what, precision);
    return;
  }
  if (nb < 0 || nb > 128 || nm < 0 || nm > cgb::kMomBatchMaxItems) {
    invalid("%s: item counts must be 0..128 (got %d baryon, %d meson)", what, nb, nm);
    return;
  }
  BaryonBatch bb;
  if (nb > 0 && !baryon_batch_setup(bb, bitems, nb, gamma_ij, gamma_kl, nproj, projectors, precision)) return;
  auto mp = std::make_unique<cgb::MomBatchParams>();
  size_t plane_floats = 0;
  if (!meson_batch_setup(*mp, plane_floats, mitems, nm, moms, nmom)) return;
  if (nb == 0 && nm == 0) return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, precision, 0, nullptr, &s)) return;
  DeviceWorkspace ws(s);
  const size_t plane_bytes = (plane_floats * sizeof(float) + 255) / 256 * 256;
  OffsetWorkspace bws(&ws, plane_bytes);
  mp->status = job.status;

  // per-extent tile shapes
  int bvar = -1, mvar = -1;
  const bool msame = [&] {
    bool same = nm > 0;
    for (int i = 0; i < nm; ++i) same = same && mitems[i].propag_i == mitems[i].propag_j;
    return same;
  }();
  // one projector of rank <= 2 (not one gamma matrix) runs its one shape
  if (nb > 0 && !cgb::batch_rank_form(nproj, bb.p)) {
    const bool same = cgb::batch_same_field(bb.p, bb.specs.data(), nb);
    const char *const *names = nullptr;
    const int nv = cgb::batch_variants(same, &names);
    std::vector<std::pair<std::string, int>> classes;
    std::vector<int> rep;  // first item of each class
    for (int i = 0; i < nb; ++i) {
      const std::string k = latt_key(bb.specs[i].latt);
      auto it = std::find_if(classes.begin(), classes.end(), [&](const auto &c) { return c.first == k; });
      if (it == classes.end()) {
        classes.push_back({k, 1});
        rep.push_back(i);
      } else {
        ++it->second;
      }
    }
    const std::string tag = std::string("batch=baryon,nproj=") + std::to_string(nproj) + ",same=" + (same ? "1" : "0");
    cgb::Job tj = job;
    tj.ws = &bws;
    bvar = tune_batch(tag, nv, names, classes, [&](int c, int v) {
      tj.variant = v;
      return cgb::launch_baryon_fused_batch(tj, nproj, bb.p, &bb.specs[rep[c]], 1);
    }, job.stream);
  }
  if (nm > 0) {
    static const char *const kMomBatchNames[] = {"fused.site8.xy8", "fused.site16.xy8"};
    std::vector<std::pair<std::string, int>> classes;
    std::vector<int> rep;
    for (int i = 0; i < nm; ++i) {
      const std::string k = latt_key(mitems[i].lattice);
      auto it = std::find_if(classes.begin(), classes.end(), [&](const auto &c) { return c.first == k; });
      if (it == classes.end()) {
        classes.push_back({k, 1});
        rep.push_back(i);
      } else {
        ++it->second;
      }
    }
    const std::string tag = std::string("batch=meson_momentum,nmom=") + std::to_string(nmom) +
                            ",same=" + (msame ? "1" : "0");
    auto one = std::make_unique<cgb::MomBatchParams>();
    mvar = tune_batch(tag, 2, kMomBatchNames, classes, [&](int c, int v) {
      // one item of class c alone: its own plane buffer at the workspace start
      *one = *mp;
      one->n_items = 1;
      one->items[0] = mp->items[rep[c]];
      one->items[0].unit_begin = 0;
      one->items[0].fin_begin = 0;
      const int *l = one->items[0].latt;
      one->total_units = l[2] * l[3];
      one->total_fin = mp->nq * l[3];
      float2 *pl = static_cast<float2 *>(ws.get((size_t)l[2] * l[3] * mp->nq * 256 * sizeof(float2)));
      if (!pl) return cudaErrorMemoryAllocation;
      one->items[0].planes = pl;
      cudaError_t e = cgb::launch_momentum_batch(job, *one, msame, v == 1 ? 16 : 8);
      if (e != cudaSuccess) return e;
      cgb::BaryonFinParams none {};
      return cgb::launch_batch_finalize(job, *one, none);
    }, job.stream);
  }

  // the launches: baryon items, meson items, one finalisation
  auto bf = std::make_unique<cgb::BaryonFinParams>();
  *bf = {};
  if (nb > 0) {
    cgb::Job bj = job;
    bj.ws = &bws;
    bj.variant = bvar;
    if (!cuda_ok(cgb::launch_baryon_fused_batch(bj, nproj, bb.p, bb.specs.data(), nb, bf.get()), what)) return;
  }
  if (nm > 0) {
    // after the baryon launch's workspace request, so this one does not move the buffer
    char *planes = static_cast<char *>(ws.get(plane_bytes));
    if (!planes) {
      fail(CONTRACT_ERROR_OUT_OF_MEMORY, (int)cudaErrorMemoryAllocation, "%s: workspace of %zu bytes", what,
           plane_bytes);
      return;
    }
    size_t off = 0;
    for (int i = 0; i < nm; ++i) {
      mp->items[i].planes = reinterpret_cast<float2 *>(planes + off);
      const int *l = mp->items[i].latt;
      off += (size_t)l[2] * l[3] * mp->nq * 256 * sizeof(float2);
    }
    if (!cuda_ok(cgb::launch_momentum_batch(job, *mp, msame, mvar == 1 ? 16 : 8), what)) return;
  }
  cuda_ok(cgb::launch_batch_finalize(job, *mp, *bf), what);
}

} // namespace

// Only the C ABI is exported (the library is built with -fvisibility=hidden).
#pragma GCC visibility push(default)
extern "C" {

// ------------------------------------------------------------ contract.h --
void init(int device) { cuda_ok(cudaSetDevice(device), "cudaSetDevice"); }

void meson_two_point(void *correl, void *propag_i, void *propag_j, unsigned long volume, int gamma_ij, int gamma_kl)
{
  do_meson(correl, propag_i, propag_j, volume, gamma_ij, gamma_kl, CONTRACT_C128, nullptr);
}

void meson_all_source_two_point(void **correl, void *propag_i, void *propag_j, unsigned long volume, int gamma_ij)
{
  do_meson_all(correl, propag_i, propag_j, volume, gamma_ij, true, CONTRACT_C128, nullptr);
}

void meson_all_sink_two_point(void **correl, void *propag_i, void *propag_j, unsigned long volume, int gamma_kl)
{
  do_meson_all(correl, propag_i, propag_j, volume, gamma_kl, false, CONTRACT_C128, nullptr);
}

void baryon_diquark(void *diquark, void *propag_i, void *propag_j, size_t volume, int gamma_ij, int gamma_kl)
{
  do_diquark(diquark, propag_i, propag_j, volume, gamma_ij, gamma_kl, CONTRACT_C128);
}

void baryon_two_point(void *correl, void *propag_i, void *propag_j, void *propag_n, BaryonContractType contract_type,
                      unsigned long volume, int gamma_ij, int gamma_kl, int gamma_mn)
{
  do_baryon(correl, propag_i, propag_j, propag_n, (int)contract_type, volume, gamma_ij, gamma_kl, gamma_mn, nullptr,
            CONTRACT_C128, nullptr);
}

void baryon_general_two_point(void *correl, void *propag_i, void *propag_j, void *propag_n,
                              BaryonContractType contract_type, size_t volume, int gamma_ij, int gamma_kl,
                              void *project_mn)
{
  if (!project_mn) {
    invalid("project_mn is NULL");
    return;
  }
  do_baryon(correl, propag_i, propag_j, propag_n, (int)contract_type, volume, gamma_ij, gamma_kl, 0,
            static_cast<const double *>(project_mn), CONTRACT_C128, nullptr);
}

void baryon_sequential_two_point(void *propag_i, void *propag_j, void *propag_n, BaryonContractType contract_type,
                                 BaryonSequentialType sequential_type, size_t volume, int gamma_ij, int gamma_kl,
                                 int gamma_mn)
{
  do_sequential(propag_i, propag_j, propag_n, (int)contract_type, (int)sequential_type, volume, gamma_ij, gamma_kl,
                gamma_mn, CONTRACT_C128);
}

// ------------------------------------------------------ contract_gb300.h --
void contract_set_error_mode(int mode)
{
  g_mode = mode == CONTRACT_ERRORS_RECORD ? CONTRACT_ERRORS_RECORD : CONTRACT_ERRORS_EXIT;
}

int contract_get_error_mode(void) { return error_mode(); }

int contract_last_error(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  return g_err;
}

const char *contract_last_error_message(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  return g_msg.c_str();
}

void contract_clear_error(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  g_err = CONTRACT_SUCCESS;
  g_msg.clear();
}

int contract_check_device(void)
{
  DevState *s = dev_state();
  if (!s) return contract_last_error();
  if (!cuda_ok(cudaStreamSynchronize(g_stream), "cudaStreamSynchronize")) return contract_last_error();
  cgb::DeviceStatus st {};
  if (!cuda_ok(cudaMemcpy(&st, s->status, sizeof(st), cudaMemcpyDeviceToHost), "status readback"))
    return contract_last_error();
  if (st.flags) {
    const cgb::DeviceStatus zero {};
    cudaMemcpy(s->status, &zero, sizeof(zero), cudaMemcpyHostToDevice);
    if (st.flags & cgb::kDevErrWaitTimeout)
      fail(CONTRACT_ERROR_DEVICE_TIMEOUT, -1, "a kernel timed out waiting for its copies (chunk %u)", st.where);
    else
      fail(CONTRACT_ERROR_BAD_WORK, -1, "a work descriptor failed validation (item %u)", st.where);
  }
  return contract_last_error();
}

void contract_set_stream(void *stream) { g_stream = static_cast<cudaStream_t>(stream); }

void contract_set_wait_limit(unsigned long long ns) { g_wait_ns = ns; }

void contract_test_withhold_chunk(int chunk) { g_withhold_chunk = chunk < 0 ? -1 : chunk; }

void contract_set_autotune(int enable) { g_tune.enabled = enable ? 1 : 0; }

int contract_autotune_report(char *buf, size_t n)
{
  std::lock_guard<std::mutex> lk(g_tune.mu);
  std::ostringstream o;
  for (const auto &kv : g_tune.choice) o << kv.first << '\t' << kv.second.name << '\t' << kv.second.ms << '\n';
  const std::string r = o.str();
  if (buf && n) {
    const size_t m = r.size() < n - 1 ? r.size() : n - 1;
    std::memcpy(buf, r.data(), m);
    buf[m] = '\0';
  }
  return (int)g_tune.choice.size();
}

int contract_variant_names(int op, int precision, int aux, char *buf, size_t n)
{
  if (op < 0 || op > 7) return invalid("Invalid op value %d", op), 0;
  if (!prec_ok(precision)) return 0;
  const char *const *names = nullptr;
  const int cnt = cgb::launch_variants(static_cast<cgb::Kind>(op), static_cast<cgb::Prec>(precision), aux, &names);
  std::string r;
  for (int v = 0; names && v < cnt; ++v) r += (v ? " " : "") + std::string(names[v]);
  if (buf && n) {
    const size_t m = r.size() < n - 1 ? r.size() : n - 1;
    std::memcpy(buf, r.data(), m);
    buf[m] = '\0';
  }
  return cnt;
}

void *contract_get_stream(void) { return g_stream; }

size_t contract_workspace_bytes(const int *lattice, int noutputs)
{
  if (!lattice || noutputs <= 0) return 0;
  const long long half = (long long)lattice[0] * lattice[1] * lattice[2] / 2;
  // One partial per (chunk, consumer warp): a chunk holds at least one tile of
  // CW * SPW sites with SPW >= 2 and CW <= 16, so a half-timeslice yields at
  // most half/2 + 16 partials.
  return (size_t)(half / 2 + 16) * 2 * lattice[3] * noutputs * 16;
}

int contract_workspace_reserve(size_t bytes)
{
  DevState *s = dev_state();
  if (!s) return contract_last_error();
  DeviceWorkspace ws(s);
  if (!ws.get(bytes)) {
    fail(CONTRACT_ERROR_OUT_OF_MEMORY, (int)cudaErrorMemoryAllocation, "workspace of %zu bytes", bytes);
    return contract_last_error();
  }
  return CONTRACT_SUCCESS;
}

int contract_projector_rank(const void *project_mn)
{
  if (!project_mn) return 0;
  cgb::RankForm<double> rk;
  fill_rank(rk, static_cast<const double *>(project_mn));
  return rk.r;
}

void contract_gamma_table(int *perm, int *phase)
{
  for (int n = 0; n < 16; ++n)
    for (int r = 0; r < 4; ++r) {
      if (perm) perm[n * 4 + r] = kG.perm[n][r];
      if (phase) phase[n * 4 + r] = kG.ph[n][r];
    }
}

void contract_convert_precision(void *dst, const void *src, size_t volume, int to_c64)
{
  if (!ptr_ok(dst, volume, "dst") || !ptr_ok(src, volume, "src")) return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, CONTRACT_C128, volume, nullptr, &s)) return;
  cuda_ok(cgb::launch_convert(job, dst, src, to_c64 != 0), "contract_convert_precision");
}

void contract_convert_layout(void *dst, const void *src, const int *lattice, int to_eo, int precision)
{
  if (!lattice) {
    invalid("contract_convert_layout needs the lattice");
    return;
  }
  if (!prec_ok(precision)) return;
  const size_t volume = (size_t)std::max(0, lattice[0]) * std::max(0, lattice[1]) * std::max(0, lattice[2]) *
                        std::max(0, lattice[3]);
  if (!ptr_ok(dst, volume, "dst") || !ptr_ok(src, volume, "src")) return;
  const size_t bytes = volume * 144 * (precision == CONTRACT_C64 ? 8 : 16);
  const char *d = static_cast<const char *>(dst), *s = static_cast<const char *>(src);
  if (volume && d < s + bytes && s < d + bytes) {
    invalid("contract_convert_layout: dst and src overlap");
    return;
  }
  cgb::Job job;
  if (!make_job(job, precision, volume, lattice)) return;
  cuda_ok(cgb::launch_layout(job, dst, src, lattice, to_eo != 0, precision == CONTRACT_C64 ? 1152 : 2304),
          "contract_convert_layout");
}

// Shared checks of the QUDA-order conversions: the lattice, the stride, the
// twelve field pointers (16-byte aligned, disjoint from each other and from
// the propagator).  Returns the stride in 16-byte chunks, or -1.
static long long quda_fields_ok(void *const *fields, const void *propag, const int *lattice, size_t stride,
                                int precision, size_t &volume)
{
  if (!lattice) {
    invalid("the QUDA-order conversions need the lattice");
    return -1;
  }
  if (!prec_ok(precision)) return -1;
  volume = (size_t)std::max(0, lattice[0]) * std::max(0, lattice[1]) * std::max(0, lattice[2]) *
           std::max(0, lattice[3]);
  const size_t half = volume / 2;
  if (stride == 0) stride = half;
  if (stride < half) {
    invalid("QUDA field stride %zu is shorter than the checkerboard length %zu", stride, half);
    return -1;
  }
  if (!fields) {
    invalid("fields is NULL (a host array of 12 device pointers)");
    return -1;
  }
  if (!ptr_ok(propag, volume, "propagator")) return -1;
  const size_t esz = precision == CONTRACT_C64 ? 8 : 16;
  const size_t fbytes = 2 * 12 * esz * stride;  // [2 parities][12 entries * esz / 16 chunks][stride][16 B]
  const size_t pbytes = volume * 144 * esz;
  for (int k = 0; k < 12; ++k) {
    if (!ptr_ok(fields[k], volume, "QUDA field")) return -1;
    if (!volume) continue;
    const char *a = static_cast<const char *>(fields[k]), *p = static_cast<const char *>(propag);
    if (a < p + pbytes && p < a + fbytes) {
      invalid("QUDA field %d overlaps the propagator", k);
      return -1;
    }
    for (int j = 0; j < k; ++j) {
      const char *b = static_cast<const char *>(fields[j]);
      if (a < b + fbytes && b < a + fbytes) {
        invalid("QUDA fields %d and %d overlap", j, k);
        return -1;
      }
    }
  }
  return (long long)stride;
}

void contract_convert_from_quda(void *propag, void *const *fields, const int *lattice, size_t stride, int precision)
{
  size_t volume = 0;
  const long long st = quda_fields_ok(fields, propag, lattice, stride, precision, volume);
  if (st < 0) return;
  cgb::Job job;
  if (!make_job(job, precision, volume, lattice)) return;
  cuda_ok(cgb::launch_quda_layout(job, propag, fields, st, true, precision == CONTRACT_C64 ? 8 : 16),
          "contract_convert_from_quda");
}

void contract_convert_to_quda(void *const *fields, const void *propag, const int *lattice, size_t stride,
                              int precision)
{
  size_t volume = 0;
  const long long st = quda_fields_ok(fields, propag, lattice, stride, precision, volume);
  if (st < 0) return;
  cgb::Job job;
  if (!make_job(job, precision, volume, lattice)) return;
  cuda_ok(cgb::launch_quda_layout(job, const_cast<void *>(propag), fields, st, false,
                                  precision == CONTRACT_C64 ? 8 : 16),
          "contract_convert_to_quda");
}

void contract_rotate_spin_basis(void *propag, size_t volume, const void *rotation, int precision)
{
  if (!prec_ok(precision)) return;
  if (!rotation) {
    invalid("rotation is NULL (a host array of 16 complex128)");
    return;
  }
  if (!ptr_ok(propag, volume, "propagator")) return;
  cgb::Job job;
  if (!make_job(job, precision, volume, nullptr)) return;
  cuda_ok(cgb::launch_spin_rotation(job, propag, static_cast<const double *>(rotation)),
          "contract_rotate_spin_basis");
}

void contract_meson(void *correl, const void *propag_i, const void *propag_j, size_t volume, int gamma_ij,
                    int gamma_kl, int precision, const int *lattice)
{
  do_meson(correl, propag_i, propag_j, volume, gamma_ij, gamma_kl, precision, lattice);
}

void contract_meson_all(void **correl, const void *propag_i, const void *propag_j, size_t volume, int fixed_gamma,
                        int source, int precision, const int *lattice)
{
  do_meson_all(correl, propag_i, propag_j, volume, fixed_gamma, source != 0, precision, lattice);
}

void contract_baryon(void *correl, const void *propag_i, const void *propag_j, const void *propag_n,
                     BaryonContractType contract_type, size_t volume, int gamma_ij, int gamma_kl, int gamma_mn,
                     const void *project_mn, int precision, const int *lattice)
{
  do_baryon(correl, propag_i, propag_j, propag_n, (int)contract_type, volume, gamma_ij, gamma_kl, gamma_mn,
            static_cast<const double *>(project_mn), precision, lattice);
}

void contract_baryon_all_types(void *correl, const void *propag_i, const void *propag_j, const void *propag_n,
                               size_t volume, int gamma_ij, int gamma_kl, int nproj, const void *projectors,
                               int precision, const int *lattice)
{
  if (!all_types_args_ok(gamma_ij, gamma_kl, nproj, projectors, precision)) return;
  if (!ptr_ok(correl, volume, "correl") || !ptr_ok(propag_i, volume, "propag_i") ||
      !ptr_ok(propag_j, volume, "propag_j") || !ptr_ok(propag_n, volume, "propag_n"))
    return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, precision, volume, lattice, &s)) return;
  DeviceWorkspace ws(s);
  job.ws = &ws;
  OpParams<double> p {};
  const size_t stride = lattice ? (size_t)lattice[3] : volume;
  fill_all_types(p, propag_i, propag_j, propag_n, correl, stride, gamma_ij, gamma_kl, nproj, projectors);
  cuda_ok(run_all_types(job, p, nproj), "contract_baryon_all_types");
}

void contract_baryon_all_types_host(void *correl, const void *propag_i, const void *propag_j, const void *propag_n,
                                    size_t volume, int gamma_ij, int gamma_kl, int nproj, const void *projectors,
                                    int precision, const int *lattice)
{
  if (!all_types_args_ok(gamma_ij, gamma_kl, nproj, projectors, precision)) return;
  if (!lattice) {
    invalid("contract_baryon_all_types_host needs the lattice");
    return;
  }
  if (!correl || !propag_i || !propag_j || !propag_n) {
    invalid("contract_baryon_all_types_host: NULL host pointer");
    return;
  }
  cgb::Job full;
  DevState *s = nullptr;
  if (!make_job(full, precision, volume, lattice, &s)) return;
  if (volume == 0) return;
  const int lt = lattice[3];
  const size_t half = (size_t)full.half_slice;  // sites per (parity, t)
  const size_t site_in = 2304, site_c = precision == CONTRACT_C64 ? 1152 : 2304;
  // Chunks of timeslices of about 256 MB of complex128 per propagator, and
  // at least four chunks so that copies overlap the contractions.
  size_t per_t = 2 * half * site_in;
  int chunk = (int)std::max<size_t>(1, (256u << 20) / per_t);
  chunk = std::min(chunk, std::max(1, (lt + 3) / 4));
  chunk = std::min(chunk, lt);
  const size_t chunk_sites = (size_t)chunk * 2 * half;
  const size_t stage_bytes = ((chunk_sites * site_in + 255) / 256) * 256;
  const size_t conv_bytes = precision == CONTRACT_C64 ? ((chunk_sites * site_c + 255) / 256) * 256 : 0;
  const size_t out_bytes = ((size_t)6 * nproj * chunk * 16 + 255) / 256 * 256;
  const size_t slot_bytes = 3 * stage_bytes + 3 * conv_bytes + out_bytes;
  if (!pipeline_ready(s, kPipeSlots * slot_bytes)) return;

  OpParams<double> p {};
  fill_all_types(p, nullptr, nullptr, nullptr, nullptr, 0, gamma_ij, gamma_kl, nproj, projectors);
  const void *host[3] = {propag_i, propag_j, propag_n};
  const bool same_ij = propag_i == propag_j;
  DeviceWorkspace ws(s);
  // Nothing of an earlier call may still read the staging buffers.
  if (!cuda_ok(cudaEventRecord(s->start, g_stream), "cudaEventRecord")) return;
  if (!cuda_ok(cudaStreamWaitEvent(s->copy, s->start, 0), "cudaStreamWaitEvent")) return;
  // One copy stream keeps the link busy with back-to-back chunks; a chunk's
  // slot is reused kPipeSlots chunks later, long after its conversion, so the
  // copies never wait on the contractions.
  const int nchunk = (lt + chunk - 1) / chunk;
  for (int c = 0; c < nchunk; ++c) {
    const int b = c % kPipeSlots, t0 = c * chunk, nt = std::min(chunk, lt - t0);
    char *slot = static_cast<char *>(s->pipe) + b * slot_bytes;
    char *stage[3], *conv[3];
    for (int q = 0; q < 3; ++q) {
      stage[q] = slot + q * stage_bytes;
      conv[q] = slot + 3 * stage_bytes + q * conv_bytes;
    }
    char *out = slot + 3 * stage_bytes + 3 * conv_bytes;
    cudaStream_t cs = s->copy;
    if (c >= kPipeSlots && !cuda_ok(cudaStreamWaitEvent(cs, s->freed[b], 0), "cudaStreamWaitEvent")) return;
    // timeslices [t0, t0 + nt) of each parity, packed as a [2][nt][half] lattice;
    // P_j given as the same host buffer as P_i is copied and converted once
    const size_t piece = (size_t)nt * half * site_in;
    for (int q = 0; q < 3; ++q)
      for (int par = 0; par < 2; ++par) {
        if (q == 1 && same_ij) continue;
        const char *src = static_cast<const char *>(host[q]) + ((size_t)par * lt + t0) * half * site_in;
        if (!cuda_ok(cudaMemcpyAsync(stage[q] + par * piece, src, piece, cudaMemcpyHostToDevice, cs),
                     "cudaMemcpyAsync"))
          return;
      }
    if (!cuda_ok(cudaEventRecord(s->copied[b], cs), "cudaEventRecord") ||
        !cuda_ok(cudaStreamWaitEvent(g_stream, s->copied[b], 0), "cudaStreamWaitEvent"))
      return;
    const int clatt[4] = {lattice[0], lattice[1], lattice[2], nt};
    cgb::Job job;
    if (!make_job(job, precision, (size_t)nt * 2 * half, clatt)) return;
    job.ws = &ws;
    const char *in[3] = {stage[0], stage[1], stage[2]};
    if (precision == CONTRACT_C64) {
      for (int q = 0; q < 3; ++q) {
        if (q == 1 && same_ij) continue;
        if (!cuda_ok(cgb::launch_convert(job, conv[q], stage[q], true), "contract_baryon_all_types_host")) return;
        in[q] = conv[q];
      }
      if (!cuda_ok(cudaEventRecord(s->freed[b], g_stream), "cudaEventRecord")) return;
    }
    if (same_ij) in[1] = in[0];
    p.in[0] = in[0];
    p.in[1] = in[1];
    p.in[2] = in[2];
    for (int o = 0; o < 6 * nproj; ++o) p.out[o] = out + (size_t)o * nt * 16;
    if (!cuda_ok(run_all_types(job, p, nproj), "contract_baryon_all_types_host")) return;
    if (precision != CONTRACT_C64 && !cuda_ok(cudaEventRecord(s->freed[b], g_stream), "cudaEventRecord")) return;
    // out[o][t0 + t] for t < nt: rows of nt values into rows of Lt
    if (!cuda_ok(cudaMemcpy2DAsync(static_cast<char *>(correl) + (size_t)t0 * 16, (size_t)lt * 16, out,
                                   (size_t)nt * 16, (size_t)nt * 16, 6 * nproj, cudaMemcpyDeviceToHost, g_stream),
                 "cudaMemcpy2DAsync"))
      return;
  }
}

int contract_baryon_all_types_noalloc(void *correl, const void *propag_i, const void *propag_j,
                                      const void *propag_n, size_t volume, int gamma_ij, int gamma_kl, int nproj,
                                      const void *projectors, int precision, const int *lattice)
{
  if (!lattice) {
    invalid("contract_baryon_all_types_noalloc needs a lattice (per-site output needs no scratch: "
            "use contract_baryon_all_types)");
    return CONTRACT_ERROR_INVALID_ARGUMENT;
  }
  if (nproj < 1 || nproj > 2) {
    invalid("nproj must be 1 or 2 (got %d)", nproj);
    return CONTRACT_ERROR_INVALID_ARGUMENT;
  }
  if (!projectors) {
    invalid("projectors is NULL");
    return CONTRACT_ERROR_INVALID_ARGUMENT;
  }
  if (!gamma_ok(gamma_ij, "gamma_ij") || !gamma_ok(gamma_kl, "gamma_kl") || !prec_ok(precision) ||
      !ptr_ok(correl, volume, "correl") || !ptr_ok(propag_i, volume, "propag_i") ||
      !ptr_ok(propag_j, volume, "propag_j") || !ptr_ok(propag_n, volume, "propag_n"))
    return CONTRACT_ERROR_INVALID_ARGUMENT;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, precision, volume, lattice, &s)) return contract_last_error();
  StaticWorkspace ws;
  if (!cuda_ok(cgb::static_scratch(&ws.base, &ws.cap), "static scratch address")) return contract_last_error();
  job.ws = &ws;
  OpParams<double> p {};
  p.in[0] = propag_i;
  p.in[1] = propag_j;
  p.in[2] = propag_n;
  for (int o = 0; o < 6 * nproj; ++o) p.out[o] = static_cast<char *>(correl) + o * (size_t)lattice[3] * 16;
  set_row(p.b.perm1, kG.perm[gamma_ij]);
  set_row(p.b.perm2, kG.perm[gamma_kl]);
  set_row(p.b.ph1[0], kG.ph[gamma_ij]);
  set_row(p.b.ph1[1], kG.ph_t[gamma_ij]);
  set_row(p.b.ph2[0], kG.ph_t[gamma_kl]);
  set_row(p.b.ph2[1], kG.ph[gamma_kl]);
  const double *pr = static_cast<const double *>(projectors);
  const double *pw[2] = {pr, pr + 32};
  for (int w = 0; w < nproj; ++w) fill_proj(p.b.proj[w], 0, pw[w]);
  fill_clifford(p.b.cl, pw, nproj, 0);
  if (nproj == 1) fill_rank(p.b.rk, pw[0]);
  const cudaError_t e = cgb::launch_baryon_fused(job, nproj, p);
  if (e != cudaSuccess && ws.requested > ws.cap) {
    invalid("lattice {%d, %d, %d, %d} needs %zu bytes of partial sums, more than the %zu-byte static scratch of "
            "contract_baryon_all_types_noalloc (use contract_baryon_all_types)",
            lattice[0], lattice[1], lattice[2], lattice[3], ws.requested, ws.cap);
    return CONTRACT_ERROR_INVALID_ARGUMENT;
  }
  if (!cuda_ok(e, "contract_baryon_all_types_noalloc")) return contract_last_error();
  return CONTRACT_SUCCESS;
}

void contract_diquark(void *diquark, const void *propag_i, const void *propag_j, size_t volume, int gamma_ij,
                      int gamma_kl, int precision)
{
  do_diquark(diquark, propag_i, propag_j, volume, gamma_ij, gamma_kl, precision);
}

void contract_sequential(void *propag_i, void *propag_j, void *propag_n, BaryonContractType contract_type,
                         BaryonSequentialType sequential_type, size_t volume, int gamma_ij, int gamma_kl,
                         int gamma_mn, int precision)
{
  do_sequential(propag_i, propag_j, propag_n, (int)contract_type, (int)sequential_type, volume, gamma_ij, gamma_kl,
                gamma_mn, precision);
}

void contract_meson_all_gamma_momentum(void *correl, const void *propag_i, const void *propag_j, size_t volume,
                                       const int *lattice, const int *moms, int nmom, int precision)
{
  if (!lattice || !moms) {
    invalid("lattice and moms are required");
    return;
  }
  const bool tensor_cores = precision == CONTRACT_C64_TC;
  if (tensor_cores) precision = CONTRACT_C64;
  if (!prec_ok(precision) || !ptr_ok(correl, volume, "correl") || !ptr_ok(propag_i, volume, "propag_i") ||
      !ptr_ok(propag_j, volume, "propag_j"))
    return;
  cgb::MomPlan plan;
  if (!make_mom_plan(plan, lattice, moms, nmom)) return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, precision, volume, lattice, &s)) return;
  DeviceWorkspace ws(s);
  job.ws = &ws;
  OpParams<double> p {};
  p.in[0] = propag_i;
  p.in[1] = propag_j;
  const bool fused = job.prec == cgb::Prec::C64 && cgb::momentum_fused_supported(plan);
  const int aux = tensor_cores ? 2 : (fused ? 1 + (propag_i == propag_j ? 4 : 0) : 0);
  std::string tc_key;
  if (tensor_cores && volume) {
    // phase tiles: rebuilt only when the lattice or the momentum list changes
    tc_key = std::to_string(lattice[0]) + "," + std::to_string(lattice[1]) + "," + std::to_string(lattice[2]) + ":";
    for (int k = 0; k < 3 * nmom; ++k) tc_key += std::to_string(moms[k]) + ",";
    const size_t need = cgb::tc_phase_bytes(cgb::make_tc_geom(plan));
    if (s->tc_tiles_bytes < need) {
      if (s->tc_tiles) {
        if (!cuda_ok(cudaDeviceSynchronize(), "contract_meson_all_gamma_momentum")) return;
        cudaFree(s->tc_tiles);
        s->tc_tiles = nullptr;
        s->tc_tiles_bytes = 0;
      }
      if (cudaMalloc(&s->tc_tiles, need) != cudaSuccess) {
        s->tc_tiles = nullptr;
        fail(CONTRACT_ERROR_OUT_OF_MEMORY, (int)cudaErrorMemoryAllocation, "phase tiles of %zu bytes", need);
        return;
      }
      s->tc_tiles_bytes = need;
      s->tc_key.clear();
    }
    job.tc_tiles = s->tc_tiles;
    job.tc_tiles_ready = s->tc_key == tc_key;
  }
  const bool ok = cuda_ok(
    tuned_launch(cgb::Kind::Momentum, job, aux,
                 [&](const cgb::Job &j) { return cgb::launch_meson_momentum(j, p, plan, correl, tensor_cores); }),
    "contract_meson_all_gamma_momentum");
  if (tensor_cores && volume) s->tc_key = ok ? tc_key : std::string();
}

void contract_baryon_all_types_batch(const ContractBaryonBatchItem *items, int nitems, int gamma_ij, int gamma_kl,
                                     int nproj, const void *projectors, int precision)
{
  if (nitems == 0) return;
  BaryonBatch bb;
  if (!baryon_batch_setup(bb, items, nitems, gamma_ij, gamma_kl, nproj, projectors, precision)) return;
  cgb::Job job;
  DevState *s = nullptr;
  if (!make_job(job, precision, 0, nullptr, &s)) return;
  DeviceWorkspace ws(s);
  job.ws = &ws;
  cuda_ok(cgb::launch_baryon_fused_batch(job, nproj, bb.p, bb.specs.data(), nitems), "contract_baryon_all_types_batch");
}

void contract_meson_all_gamma_momentum_batch(const ContractMesonMomentumBatchItem *items, int nitems,
                                             const int *moms, int nmom, int precision)
{
  run_mixed_batch(nullptr, 0, 0, 0, 1, nullptr, items, nitems, moms, nmom, precision,
                  "contract_meson_all_gamma_momentum_batch");
}

void contract_batch_mixed(const ContractBaryonBatchItem *baryon_items, int nbaryon, int gamma_ij, int gamma_kl,
                          int nproj, const void *projectors, const ContractMesonMomentumBatchItem *meson_items,
                          int nmeson, const int *moms, int nmom, int precision)
{
  run_mixed_batch(baryon_items, nbaryon, gamma_ij, gamma_kl, nproj, projectors, meson_items, nmeson, moms, nmom,
                  precision, "contract_batch_mixed");
}

void contract_sequential_sink(void *propag_i, void *propag_j, void *propag_n, BaryonContractType contract_type,
                              BaryonSequentialType sequential_type, size_t volume, const int *lattice, int t_sink,
                              int gamma_ij, int gamma_kl, int gamma_mn, int precision)
{
  if (!lattice) {
    invalid("lattice is required");
    return;
  }
  if ((int)sequential_type < 0 || (int)sequential_type > 2) {
    invalid("Invalid sequential_type value %d", (int)sequential_type);
    return;
  }
  if (t_sink < 0 || t_sink >= lattice[3]) {
    invalid("t_sink %d outside 0..%d", t_sink, lattice[3] - 1);
    return;
  }
  if (!type_ok((int)contract_type) || !gamma_ok(gamma_mn, "gamma_mn") || !gamma_ok(gamma_ij, "gamma_ij") ||
      !gamma_ok(gamma_kl, "gamma_kl") || !prec_ok(precision))
    return;
  if (!ptr_ok(propag_i, volume, "propag_i") || !ptr_ok(propag_j, volume, "propag_j") ||
      !ptr_ok(propag_n, volume, "propag_n"))
    return;
  cgb::Job check;
  DevState *s = nullptr;
  if (!make_job(check, precision, volume, lattice, &s)) return;
  const size_t site_bytes = precision == CONTRACT_C64 ? 1152 : 2304;
  const size_t half = (size_t)check.half_slice;
  void *bufs[3] = {propag_i, propag_j, propag_n};
  // Zero the whole output field, then fill the sink timeslice's two
  // (parity) segments, each a contiguous run of half-timeslice sites.
  if (!cuda_ok(cudaMemsetAsync(bufs[(int)sequential_type], 0, volume * site_bytes, g_stream), "cudaMemsetAsync"))
    return;
  for (int par = 0; par < 2; ++par) {
    const size_t off = ((size_t)par * lattice[3] + t_sink) * half * site_bytes;
    do_sequential(static_cast<char *>(propag_i) + off, static_cast<char *>(propag_j) + off,
                  static_cast<char *>(propag_n) + off, (int)contract_type, (int)sequential_type, half, gamma_ij,
                  gamma_kl, gamma_mn, precision);
  }
}

} // extern "C"
#pragma GCC visibility pop
