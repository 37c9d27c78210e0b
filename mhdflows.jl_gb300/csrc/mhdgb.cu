// Host orchestration and C ABI of the GB300-native MHD RK4 / LSRK4 step.
//
// One right-hand-side evaluation (MHDcalcN!, src/pgen.jl:153-162 of MHDFlows.jl) is six kernels:
//   z_inverse  (state -> colbuf, 6 fields, pruned input; no normalisation anywhere in the passes,
//              the 1/n^6 of the two transforms is applied to the products in the epilogue)
//   y_inverse  (colbuf -> rowbuf, 6 fields, pruned input)
//   x_fused    (rowbuf -> rowbuf: c2r, 8 quadratic products, r2c; physical fields never leave chip)
//   y_forward  (rowbuf -> colbuf, 8 products, pruned output)
//   z_forward  (colbuf -> compact product spectra: z r2c of the 8 products, pruned output)
//   rk_epilogue (Leray projection, curl, -nu k^2 / -eta k^2 and the RK stage update, streaming)
// The state is kept only on the retained (2/3-rule) band, which is all the reference's dynamics
// ever read: dealias! zeroes the alias band of the stage state before every RHS evaluation.
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <functional>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/mhdgb.h"
#include "ops.cuh"
#include "step_kernels.cuh"

using namespace mhdgb;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define MHD_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      return fail(e_ == cudaErrorMemoryAllocation ? MHD_ERR_OOM : MHD_ERR_CUDA,          \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                   \
    }                                                                                    \
  } while (0)

// pass-buffer slots per (z, ky') / (z, y): 8 products, plus 6 penalty fields with VP
int slots_of(bool vp) { return vp ? 14 : 8; }

OpsBase* make_ops(int n) {
  switch (n) {
    case 16: return make_ops_16();
    case 32: return make_ops_32();
    case 48: return make_ops_48();
    case 64: return make_ops_64();
    case 96: return make_ops_96();
    case 128: return make_ops_128();
    case 256: return make_ops_256();
    case 512: return make_ops_512();
    default: return nullptr;
  }
}

bool supported(int n) { return n == 16 || n == 32 || n == 48 || n == 64 || n == 96 || n == 128 || n == 256 || n == 512; }

// Alias ranges of FourierFlows' getaliasedwavenumbers with aliased_fraction = 1/3 (same double
// arithmetic as Julia): 1-based iL = floor((1-a)/2*n)+1, iR = ceil((1+a)/2*n).
void kept_modes(int n, int* kx, int* kp, int* kn) {
  const double a = 1.0 / 3.0;
  const double lo = (1 - a) / 2, hi = (1 + a) / 2;
  const int iL = (int)std::floor(lo * n) + 1;
  const int iR = (int)std::ceil(hi * n);
  *kx = iL - 1;
  *kp = iL - 1;
  *kn = n - iR;
}

Geom make_geom(int n, double L) {
  Geom g;
  g.n = n;
  kept_modes(n, &g.kx, &g.kp, &g.kn);
  g.kxp = (g.kx + 3) / 4 * 4;
  g.k2 = g.kp + g.kn;
  g.kscale = (float)(2.0 * M_PI / L);
  return g;
}

// Kernel classes for per-launch timing (KClass of ops.cuh).
const char* kClassNames[KC_COUNT] = {"z_inverse", "y_inverse", "x_fused", "y_forward", "z_forward", "rk_epilogue",
                                     "other"};

const double kLsA[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                        -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
const double kLsB[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                        1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                        2277821191437.0 / 14882151754819.0};

struct Sizes {
  long long fs;      // one compact field (complex)
  long long state;   // six fields (slot stride of sol / xs / acc)
  long long colbuf;  // colbuf complex elements per slot
  long long rowbuf;  // rowbuf complex elements per slot
  long long ref;     // reference-layout sol (complex)
  long long phys;    // one physical field (floats)
  int diag_blocks;
};

Sizes sizes_of(const Geom& g, int ns) {
  Sizes s;
  s.fs = (long long)g.k2 * g.k2 * g.kxp;
  s.state = 6 * s.fs;
  s.colbuf = (long long)g.n * g.k2 * ns * g.kxp;
  s.rowbuf = (long long)g.n * g.n * ns * g.kxp;
  s.ref = 6LL * (g.n / 2 + 1) * g.n * g.n;
  s.phys = (long long)g.n * g.n * g.n;
  long long b = (s.fs + kDiagThreads - 1) / kDiagThreads;
  s.diag_blocks = (int)(b < 1216 ? b : 1216);
  return s;
}

// Device bytes of one slot (state, stage arrays, pass buffers; with VP the mask and the six wall
// fields) and of the per-class staging.
long long slot_bytes(const Geom& g, bool vp = false, bool hydro = false) {
  Sizes s = sizes_of(g, slots_of(vp && !hydro));
  return (3 * s.state + s.fs + s.colbuf + s.rowbuf) * 8 + 16 * 4 + (vp ? 7 * s.phys * 4 : 0);
}
long long class_bytes(const Geom& g) {
  Sizes s = sizes_of(g, 8);
  return s.ref * 8 + s.phys * 4 + 6LL * g.n * 8 + (long long)s.diag_blocks * kDiagSlots * 8 + 256;
}
long long footprint(const Geom& g, int cap, bool vp = false, bool hydro = false) {
  return class_bytes(g) + (long long)cap * slot_bytes(g, vp, hydro);
}

}  // namespace

namespace mhdgb {
int report_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace mhdgb

namespace {

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// 5-D tensor map over 8-byte elements (complex float pairs), no swizzle, zero fill out of range
bool make_tmap(CUtensorMap* m, void* base, const cuuint64_t (&dims)[5], const cuuint64_t (&strides)[4],
               const cuuint32_t (&box)[5]) {
  auto enc = tmap_encoder();
  if (!enc) return false;
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

}  // namespace

namespace {

// ------------------------------------------------------------------------------------------
// Autotuner results: the selected variant name of each tuned kernel class, keyed by device
// (name and SM count) and grid size.  Kept for the process and, unless disabled, in a text file
// ($MHDGB_TUNE_CACHE, else $XDG_CACHE_HOME/mhdgb/tune.txt, else $HOME/.cache/mhdgb/tune.txt; an
// empty $MHDGB_TUNE_CACHE turns the file off).  One line per entry:
//   <device name>|<sm count>|<n>|<variant of z_inverse>|...|<variant of z_forward>
// ------------------------------------------------------------------------------------------
std::mutex g_tune_mtx;
std::map<std::string, std::vector<std::string>> g_tuned;

std::string tune_file() {
  const char* e = std::getenv("MHDGB_TUNE_CACHE");
  if (e) return std::string(e);
  const char* x = std::getenv("XDG_CACHE_HOME");
  if (x && *x) return std::string(x) + "/mhdgb/tune.txt";
  const char* h = std::getenv("HOME");
  if (h && *h) return std::string(h) + "/.cache/mhdgb/tune.txt";
  return "";
}

std::string tune_key(int device, int n, int prec, int vp, int hd = 0) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return "";
  std::string name(prop.name);
  for (auto& c : name) if (c == '|' || c == '\n') c = ' ';
  return name + "|" + std::to_string(prop.multiProcessorCount) + "|" + std::to_string(n) + (prec ? "p" + std::to_string(prec) : "") +
         (vp ? "v" + std::to_string(vp) : "") + (hd ? "h" : "");
}

std::vector<std::string> split_bar(const std::string& line) {
  std::vector<std::string> out;
  size_t a = 0;
  while (true) {
    size_t b = line.find('|', a);
    out.push_back(line.substr(a, b == std::string::npos ? std::string::npos : b - a));
    if (b == std::string::npos) break;
    a = b + 1;
  }
  return out;
}

// variant names of a key: the process cache, else the file
bool tuned_lookup(const std::string& key, std::vector<std::string>* names) {
  std::lock_guard<std::mutex> lock(g_tune_mtx);
  auto it = g_tuned.find(key);
  if (it != g_tuned.end()) { *names = it->second; return true; }
  const std::string path = tune_file();
  if (path.empty()) return false;
  std::FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return false;
  char buf[4096];
  bool found = false;
  while (std::fgets(buf, sizeof(buf), f)) {
    std::string line(buf);
    while (!line.empty() && (line.back() == '\n' || line.back() == '\r')) line.pop_back();
    std::vector<std::string> parts = split_bar(line);
    if (parts.size() != 3 + (size_t)kTunedClasses) continue;
    if (parts[0] + "|" + parts[1] + "|" + parts[2] != key) continue;
    names->assign(parts.begin() + 3, parts.end());
    found = true;  // the last line of a key wins
  }
  std::fclose(f);
  if (found) g_tuned[key] = *names;
  return found;
}

void tuned_store(const std::string& key, const std::vector<std::string>& names, bool persist) {
  std::lock_guard<std::mutex> lock(g_tune_mtx);
  g_tuned[key] = names;
  if (!persist) return;
  const std::string path = tune_file();
  if (path.empty()) return;
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos && slash > 0) {  // create the directory chain, ignore failures
    std::string dir = path.substr(0, slash);
    for (size_t p = 1; p <= dir.size(); ++p)
      if (p == dir.size() || dir[p] == '/') mkdir(dir.substr(0, p).c_str(), 0755);
  }
  std::FILE* f = std::fopen(path.c_str(), "a");
  if (!f) return;
  std::string line = key;
  for (const auto& nm : names) line += "|" + nm;
  std::fprintf(f, "%s\n", line.c_str());
  std::fclose(f);
}

}  // namespace

// A size class: `cap` slots of one grid size and scheme, stepped together.  The single-problem
// API is the capacity-1 case with slot 0 active.
struct mhd_problem {
  mhd_params p{};
  Geom g{};
  Sizes sz{};
  int cap = 1;
  std::unique_ptr<OpsBase> ops;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // slot pools
  float2* sol = nullptr;
  float2* xs = nullptr;
  float2* acc = nullptr;
  float2* aux = nullptr;
  float2* colbuf = nullptr;
  float2* rowbuf = nullptr;
  // per-class staging and reductions (one slot at a time)
  float2* ref = nullptr;
  float* phys = nullptr;
  double* diag_partial = nullptr;
  double* diag_out = nullptr;
  unsigned int* maxabs = nullptr;
  // work lists
  SlotParams* dparams = nullptr;
  int* dlist = nullptr;
  // on-device CFL: per-slot maxima of |u|, |B| (float bits) and device clock
  unsigned int* dvmax = nullptr;
  double* dtime = nullptr;
  // per-slot step counters on the device (the random forcing's call counter) and whether any
  // slot is forced (the step then ends with step_tick_kernel)
  long long* dstep = nullptr;
  bool forcing = false;
  // volume penalisation (mhd_params.vp): ns pass-buffer slots, per-slot mask and wall fields in
  // physical space, which slots have walls set, and whether each step ends with the divergence
  // corrections of TimeIntegrator!
  int ns = 8;
  float* vchi = nullptr;
  float* vwall = nullptr;
  std::vector<char> walls;
  bool divcorr = false;
  // TMA sources of the column passes (used when a TMA-fed variant is selected) and the device
  // word a timed-out tile wait is recorded in
  TmaPass tm_zinv_sol, tm_zinv_xs, tm_yinv, tm_yfwd, tm_zfwd;
  int* derr = nullptr;
  bool cfl = false;
  double cfl_coef = 0.3;
  int graph_version = 0;   // active slots, then the identity list (cap each), then counts
  std::vector<SlotParams> hparams;
  std::vector<char> used;
  std::vector<int> active;
  std::vector<double> t;
  std::vector<long long> stepc;
  bool list_dirty = true;
  // step graph
  cudaGraphExec_t graph = nullptr;
  // ordering events of the device-pointer state transfers (created on first use)
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  // source of the copy-engine zeros of get_state into mapped host memory (created on first use):
  // a zeroed device buffer and the side stream its copies run on
  void* zeros = nullptr;
  size_t zbytes = 0;
  cudaStream_t zstream = nullptr;
  cudaEvent_t ev_z = nullptr;  // orders the copy-engine side stream against the handle's stream
  int ensure_zero_source() {
    if (zeros) return MHD_OK;
    const size_t want = size_t(16) << 20;
    MHD_CUDA(cudaMalloc(&zeros, want));
    MHD_CUDA(cudaMemset(zeros, 0, want));
    zbytes = want;
    if (!zstream) MHD_CUDA(cudaStreamCreateWithFlags(&zstream, cudaStreamNonBlocking));
    if (!ev_z) MHD_CUDA(cudaEventCreateWithFlags(&ev_z, cudaEventDisableTiming));
    return MHD_OK;
  }
  // guard bands: every large buffer is allocated kGuardBytes longer and the tail filled with
  // kGuardByte, so that a kernel writing past a buffer's end shows up in mhd_check_guards
  static constexpr size_t kGuardBytes = 4096;
  static constexpr unsigned char kGuardByte = 0xA5;
  std::vector<std::pair<unsigned char*, size_t>> guards;
  template <typename T>
  cudaError_t alloc_guarded(T** p, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes + kGuardBytes);
    if (e != cudaSuccess) return e;
    e = cudaMemset(static_cast<unsigned char*>(q) + bytes, kGuardByte, kGuardBytes);
    if (e != cudaSuccess) { cudaFree(q); return e; }
    *p = static_cast<T*>(q);
    guards.emplace_back(static_cast<unsigned char*>(q) + bytes, kGuardBytes);
    return cudaSuccess;
  }
  // on-device diagnostics history: every diag_freq-th step of mhd_step ends with the batched
  // diagnostics into sample *dhist_count (graph_diag is that step's graph); the host logs the
  // step and clock of each sample as it launches them
  int diag_freq = 0, diag_capacity = 0;
  double* dhist = nullptr;
  double* dhist_partial = nullptr;
  int* dhist_count = nullptr;
  long long hsteps = 0;
  std::vector<long long> hist_step;
  std::vector<std::vector<double>> hist_t;
  cudaGraphExec_t graph_diag = nullptr;
  // profiling
  bool profiling = false;
  struct Rec { int cls; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  long long prof_launches[KC_COUNT] = {0};
  double prof_ms[KC_COUNT] = {0};

  ~mhd_problem() { release(); }

  void release() {
    cudaSetDevice(device);
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    if (graph_diag) cudaGraphExecDestroy(graph_diag);
    graph_diag = nullptr;
    free_history();
    for (auto& r : recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    recs.clear();
    for (auto e : pool) cudaEventDestroy(e);
    pool.clear();
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    ev_in = ev_out = nullptr;
    if (zstream) cudaStreamSynchronize(zstream), cudaStreamDestroy(zstream);
    if (zeros) cudaFree(zeros);
    if (ev_z) cudaEventDestroy(ev_z);
    zstream = nullptr;
    zeros = nullptr;
    ev_z = nullptr;
    void* ptrs[] = {sol, xs, acc, aux, colbuf, rowbuf, ref, phys, diag_partial, diag_out, maxabs, dparams, dlist, dvmax, dtime,
                    dstep, derr, vchi, vwall};
    for (void* q : ptrs) if (q) cudaFree(q);
    vchi = vwall = nullptr;
    sol = xs = acc = aux = colbuf = rowbuf = ref = nullptr;
    guards.clear();
    phys = nullptr; diag_partial = nullptr; diag_out = nullptr; maxabs = nullptr; dparams = nullptr; dlist = nullptr;
    dvmax = nullptr; dtime = nullptr; dstep = nullptr; derr = nullptr;
    if (own_stream) cudaStreamDestroy(own_stream);
    own_stream = nullptr;
  }

  // device work lists: dlist[0..cap) active, dlist[cap..2cap) identity, dlist[2cap] active count, dlist[2cap+1] = 1
  BatchRef active_ref() const { return BatchRef{dlist, dlist + 2 * cap}; }
  BatchRef slot_ref(int slot) const { return BatchRef{dlist + cap + slot, dlist + 2 * cap + 1}; }

  int sync_lists() {
    if (!list_dirty) return MHD_OK;
    std::vector<int> h(2 * cap + 2, 0);
    for (size_t i = 0; i < active.size(); ++i) h[i] = active[i];
    for (int i = 0; i < cap; ++i) h[cap + i] = i;
    h[2 * cap] = (int)active.size();
    h[2 * cap + 1] = 1;
    MHD_CUDA(cudaMemcpyAsync(dlist, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, stream));
    MHD_CUDA(cudaMemcpyAsync(dparams, hparams.data(), hparams.size() * sizeof(SlotParams), cudaMemcpyHostToDevice, stream));
    list_dirty = false;
    return MHD_OK;
  }

  cudaEvent_t get_event() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e; cudaEventCreate(&e); return e;
  }
  int fold_records() {
    if (recs.empty()) return MHD_OK;
    MHD_CUDA(cudaStreamSynchronize(stream));
    for (auto& r : recs) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r.a, r.b);
      prof_launches[r.cls] += 1;
      prof_ms[r.cls] += ms;
      pool.push_back(r.a); pool.push_back(r.b);
    }
    recs.clear();
    return MHD_OK;
  }
  template <class F>
  int launch(int cls, F&& f) {
    if (profiling) {
      Rec r{cls, get_event(), get_event()};
      cudaEventRecord(r.a, stream);
      f();
      cudaEventRecord(r.b, stream);
      recs.push_back(r);
      if (recs.size() > (1u << 16)) { int rc = fold_records(); if (rc) return rc; }
    } else {
      f();
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("kernel launch (") + kClassNames[cls] + "): " + cudaGetErrorString(e));
    return MHD_OK;
  }

  // ---- strides (complex elements)
  long long FS() const { return sz.fs; }
  long long ST() const { return sz.state; }
  long long AZ() const { return (long long)g.k2 * ns * g.kxp; }
  long long BZ() const { return (long long)g.n * ns * g.kxp; }
  long long SLK() const { return (long long)ns * g.kxp; }

  // compact fields (src + slot*sI, nf fields at stride FS) -> colbuf slots 0..nf-1
  int z_inverse(const float2* src, long long sI, int nf, BatchRef br) {
    ColArgs a{src, colbuf, FS(), (long long)g.kxp, (long long)g.k2 * g.kxp, (long long)g.kxp, SLK(), AZ(), sI, sz.colbuf};
    // the maps cover all six fields of a pool: only the right-hand side's call can use them
    const TmaPass* tp = (nf == 6 && sI == ST()) ? (src == sol ? &tm_zinv_sol : src == xs ? &tm_zinv_xs : nullptr) : nullptr;
    return launch(KC_ZINV, [&] { ops->col(KC_ZINV, a, g, g.k2, nf, br, cap, stream, tp); });
  }
  int y_inverse(int nf, BatchRef br) {
    ColArgs a{colbuf, rowbuf, (long long)g.kxp, AZ(), SLK(), (long long)g.kxp, BZ(), SLK(), sz.colbuf, sz.rowbuf};
    return launch(KC_YINV, [&] { ops->col(KC_YINV, a, g, g.n, nf, br, cap, stream, &tm_yinv); });
  }
  int x_fused(BatchRef br, unsigned int* vmax) {
    // the six field rows of a physical row are contiguous (slot stride == kxp)
    const VpRef vp{vchi, vwall, sz.phys};
    return launch(KC_XFUSED, [&] { ops->x_fused(rowbuf, g, SLK(), g.kxp, sz.rowbuf, br, cap, vmax, vp, stream); });
  }
  int y_forward(int nf, BatchRef br) {
    ColArgs a{rowbuf, colbuf, (long long)g.kxp, BZ(), SLK(), (long long)g.kxp, AZ(), SLK(), sz.rowbuf, sz.colbuf};
    return launch(KC_YFWD, [&] { ops->col(KC_YFWD, a, g, g.n, nf, br, cap, stream, &tm_yfwd); });
  }
  // colbuf slots -> compact planes (nf fields/products) at dst + slot*dI, pruned output
  // hx: the stage state whose kx = 0 Hermitian part the pass also writes into aux (the
  // right-hand side's call), or nullptr
  int z_forward(float2* dst, long long dI, int nf, BatchRef br, const float2* hx = nullptr) {
    ColArgs a{colbuf, dst, (long long)g.kxp, SLK(), AZ(), FS(), (long long)g.kxp, (long long)g.k2 * g.kxp, sz.colbuf, dI};
    a.hx = hx;
    a.hout = aux;
    a.hfs = FS();
    a.hsI = ST();
    a.hoI = FS();
    return launch(KC_ZFWD, [&] { ops->col(KC_ZFWD, a, g, g.k2, nf, br, cap, stream, &tm_zfwd); });
  }
  // Stage epilogue: RHS from the 8 compact product planes (in rowbuf; 14 with the VP penalty
  // fields) and the stage state X.
  RkArgs rk_args(const float2* X, float2* xn, int op, float hf, float ca, float cb, int stage) const {
    RkArgs a{};
    a.prod = rowbuf;
    a.X = X;
    a.H = aux;
    a.sol = sol;
    a.acc = acc;
    a.xn = xn;
    a.sp = dparams;
    a.fs = FS();
    a.stI = ST();
    a.prodI = sz.rowbuf;
    a.hI = FS();
    a.hf = hf;
    a.ca = ca;
    a.cb = cb;
    a.op = op;
    a.step = dstep;
    a.stage = stage;
    a.hydro = p.hydro_only;
    const double n3 = (double)g.n * g.n * g.n;
    a.pscale = (float)(1.0 / (n3 * n3));
    a.vscale = (float)(1.0 / n3);
    return a;
  }
  // HDcalcN! (src/pgen.jl:176-182) calls addforcing! before HDcalcN_advection!, whose UᵢUpdate!
  // starts by zeroing the velocity right-hand side: a hydrodynamic problem is unforced
  bool forced() const { return forcing && !p.hydro_only; }
  // xn: where the stage update writes (the next stage state, or sol; it may be X itself, so the
  // Hermitian part of X's kx = 0 plane was copied out into aux by the z_forward before it)
  int epilogue(const float2* X, float2* xn, int op, float hf, float ca, float cb, BatchRef br, int stage) {
    const RkArgs a = rk_args(X, xn, op, hf, ca, cb, stage);
    const int bx = g.kx <= 256 ? (g.kx + 31) / 32 * 32 : 256;
    const dim3 grid((g.kx + bx - 1) / bx, g.k2, g.k2 * cap);
    const bool f = forced(), v = p.vp != 0;
    return launch(KC_RKEPI, [&] {
      if (hd_form() && v) launch_epilogue<false, true, true>(op, grid, bx, a, br);
      else if (hd_form()) launch_epilogue<false, false, true>(op, grid, bx, a, br);
      else if (f && v) launch_epilogue<true, true>(op, grid, bx, a, br);
      else if (f) launch_epilogue<true, false>(op, grid, bx, a, br);
      else if (v) launch_epilogue<false, true>(op, grid, bx, a, br);
      else launch_epilogue<false, false>(op, grid, bx, a, br);
    });
  }
  // record: the stage whose physical fields getCFL! reads (the last one of a step)
  template <bool F, bool V, bool H = false>
  void launch_epilogue(int op, dim3 grid, int bx, const RkArgs& a, BatchRef br) {
    switch (op) {
      case OP_RHS: rk_epilogue_kernel<OP_RHS, F, V, H><<<grid, bx, 0, stream>>>(a, g, br); break;
      case OP_RK4_FIRST: rk_epilogue_kernel<OP_RK4_FIRST, F, V, H><<<grid, bx, 0, stream>>>(a, g, br); break;
      case OP_RK4_MID: rk_epilogue_kernel<OP_RK4_MID, F, V, H><<<grid, bx, 0, stream>>>(a, g, br); break;
      case OP_RK4_LAST: rk_epilogue_kernel<OP_RK4_LAST, F, V, H><<<grid, bx, 0, stream>>>(a, g, br); break;
      case OP_LS_FIRST: rk_epilogue_kernel<OP_LS_FIRST, F, V, H><<<grid, bx, 0, stream>>>(a, g, br); break;
      default: rk_epilogue_kernel<OP_LS, F, V, H><<<grid, bx, 0, stream>>>(a, g, br); break;
    }
  }
  // DivVCorrection! / DivBCorrection! of the slots in br (mask: 1 u, 2 B)
  int div_correct(BatchRef br, int ninst, int mask) {
    const int bx = g.kx <= 256 ? (g.kx + 31) / 32 * 32 : 256;
    const dim3 grid((g.kx + bx - 1) / bx, g.k2, g.k2 * ninst);
    return launch(KC_OTHER, [&] { div_correct_kernel<<<grid, bx, 0, stream>>>(sol, g, FS(), ST(), br, mask); });
  }
  // stage: right-hand-side evaluation within the step (7 outside a step)
  int rhs(const float2* X, float2* xn, int op, float hf, float ca, float cb, BatchRef br, int stage, bool record = false) {
    int rc;
    const int nin = hd_form() ? 3 : 6, nout = hd_form() ? (p.vp ? 8 : 5) : ns;
    if ((rc = z_inverse(X, ST(), nin, br))) return rc;
    if ((rc = y_inverse(nin, br))) return rc;
    if ((rc = x_fused(br, (record && cfl) ? dvmax : nullptr))) return rc;
    if ((rc = y_forward(nout, br))) return rc;
    if ((rc = z_forward(rowbuf, sz.rowbuf, nout, br, X))) return rc;
    return epilogue(X, xn, op, hf, ca, cb, br, stage);
  }
  // One step of every active slot (launches only; see run_steps for graphs and clocks).
  int issue_step(bool with_diag = false) {
    const BatchRef br = active_ref();
    int rc;
    if (p.scheme == MHD_RK4) {
      if ((rc = rhs(sol, xs, OP_RK4_FIRST, 0.5f, 0.f, 0.f, br, 0))) return rc;
      if ((rc = rhs(xs, xs, OP_RK4_MID, 0.5f, 0.f, 0.f, br, 1))) return rc;
      if ((rc = rhs(xs, xs, OP_RK4_MID, 1.0f, 0.f, 0.f, br, 2))) return rc;
      if ((rc = rhs(xs, sol, OP_RK4_LAST, 0.f, 0.f, 0.f, br, 3, true))) return rc;
    } else {
      for (int i = 0; i < 5; ++i)
        if ((rc = rhs(sol, sol, i == 0 ? OP_LS_FIRST : OP_LS, 0.f, (float)kLsA[i], (float)kLsB[i], br, i, i == 4))) return rc;
    }
    if (forcing && (rc = launch(KC_OTHER, [&] {
          step_tick_kernel<<<(cap + 127) / 128, 128, 0, stream>>>(br, dstep);
        })))
      return rc;
    if (divcorr) {
      // TimeIntegrator! with VP (src/integrator.jl:118-122): DivVCorrection!, and DivBCorrection!
      // for MHD, after every step; they also refresh vars, which the next getCFL! reads
      if ((rc = div_correct(br, cap, p.hydro_only ? 1 : 3))) return rc;
      if (cfl && (rc = cfl_prime())) return rc;
    }
    if (cfl && (rc = cfl_update(1))) return rc;
    if (with_diag) return record_diagnostics(br);
    return MHD_OK;
  }
  // the diagnostics of every active slot's state into the next history sample
  int record_diagnostics(BatchRef br) {
    int rc;
    const int nb = sz.diag_blocks;
    const double n3 = (double)g.n * g.n * g.n, dx = p.L / g.n;
    const double scale = dx * dx * dx / n3;
    if ((rc = launch(KC_OTHER, [&] {
           diag_partial_batch_kernel<<<dim3(nb, cap), kDiagThreads, 0, stream>>>(sol, ST(), g, br, dhist_partial);
         })))
      return rc;
    if ((rc = launch(KC_OTHER, [&] {
           diag_record_kernel<<<cap, kDiagThreads, 0, stream>>>(dhist_partial, nb, br, cap, dhist, dhist_count,
                                                                diag_capacity, cfl ? dtime : nullptr, scale);
         })))
      return rc;
    return launch(KC_OTHER, [&] { hist_tick_kernel<<<1, 32, 0, stream>>>(dhist_count); });
  }
  void free_history() {
    if (dhist) cudaFree(dhist);
    if (dhist_partial) cudaFree(dhist_partial);
    if (dhist_count) cudaFree(dhist_count);
    dhist = dhist_partial = nullptr;
    dhist_count = nullptr;
  }
  int cfl_update(int advance) {
    const float coef_dx = (float)(cfl_coef * p.L / g.n);
    const float vscale = (float)(1.0 / ((double)g.n * g.n * g.n));
    return launch(KC_OTHER, [&] {
      cfl_update_kernel<<<(cap + 127) / 128, 128, 0, stream>>>(active_ref(), dparams, dvmax, dtime, coef_dx, vscale,
                                                              advance);
    });
  }
  // maxima of the current state's physical fields (the first CFL step's vars)
  int cfl_prime() {
    int rc;
    MHD_CUDA(cudaMemsetAsync(dvmax, 0, 2 * (size_t)cap * sizeof(unsigned int), stream));
    for (int s : active)
      for (int f = 0; f < 6; ++f) {
        if ((rc = inverse_field(sol + f * sz.fs, sz.state, s, 1.0f))) return rc;  // raw units, like x_fused
        unsigned int* out = dvmax + 2 * s + (f < 3 ? 0 : 1);
        if ((rc = launch(KC_OTHER, [&] { maxabs_into_kernel<<<1216, 256, 0, stream>>>(phys, sz.phys, out); }))) return rc;
      }
    return MHD_OK;
  }
  // ---- autotuner: each candidate is timed inside real right-hand-side evaluations (z_inverse ..
  // z_forward, the kx = 0 Hermitian part and the epilogue in its RHS-only form, which writes
  // only the scratch pass buffers and acc, never the state), with CUDA events around every
  // launch.  Round r selects variant r of every class that has one (the others keep their
  // current choice); the per-class time of a candidate is the best over two sweeps.
  int tune_rounds(std::vector<std::vector<double>>& best) {
    const BatchRef br = active_ref();
    int maxv = 0;
    for (int c = 0; c < kTunedClasses; ++c) maxv = std::max(maxv, ops->variant_count(c));
    best.assign(kTunedClasses, std::vector<double>(maxv, 1e300));
    int base[kTunedClasses];
    std::memcpy(base, ops->sel, sizeof(base));
    int rc = MHD_OK;
    profiling = true;
    for (int sweep = 0; sweep < 2 && rc == MHD_OK; ++sweep)
      for (int r = 0; r < maxv && rc == MHD_OK; ++r) {
        for (int c = 0; c < kTunedClasses; ++c) ops->sel[c] = ops->variant_ok(c, r) ? r : base[c];
        // one evaluation to warm up, then three timed ones
        for (int k = 0; k < 4 && rc == MHD_OK; ++k) {
          if (k == 1) {
            if ((rc = fold_records())) break;
            for (int c = 0; c < KC_COUNT; ++c) { prof_launches[c] = 0; prof_ms[c] = 0; }
          }
          rc = rhs(sol, acc, OP_RHS, 0.f, 0.f, 0.f, br, 7);
        }
        if (rc == MHD_OK) rc = fold_records();
        for (int c = 0; c < kTunedClasses && rc == MHD_OK; ++c)
          if (ops->variant_ok(c, r) && prof_launches[c] > 0)
            best[c][r] = std::min(best[c][r], prof_ms[c] / prof_launches[c]);
      }
    profiling = false;
    for (auto& rec : recs) { pool.push_back(rec.a); pool.push_back(rec.b); }
    recs.clear();
    for (int c = 0; c < KC_COUNT; ++c) { prof_launches[c] = 0; prof_ms[c] = 0; }
    std::memcpy(ops->sel, base, sizeof(base));
    return rc;
  }
  std::vector<std::string> selected_names() const {
    std::vector<std::string> v;
    for (int c = 0; c < kTunedClasses; ++c) v.push_back(ops->variant_name(c, ops->sel[c]));
    return v;
  }
  int apply_names(const std::vector<std::string>& names) {
    if ((int)names.size() != kTunedClasses) return MHD_ERR_INVALID;
    int saved[kTunedClasses];
    std::memcpy(saved, ops->sel, sizeof(saved));
    for (int c = 0; c < kTunedClasses; ++c)
      if (ops->select_by_name(c, names[c]) != MHD_OK) {  // a stale entry: keep the defaults
        std::memcpy(ops->sel, saved, sizeof(saved));
        g_err.clear();
        return MHD_ERR_INVALID;
      }
    invalidate_graph();
    return MHD_OK;
  }
  int autotune(bool force, bool persist) {
    if (profiling) return fail(MHD_ERR_STATE, "autotune does not run with per-kernel profiling enabled");
    int rc;
    if ((rc = sync_lists())) return rc;
    const std::string key = tune_key(device, g.n, p.precision, ops->vp, ops->hd);
    std::vector<std::string> names;
    if (!force && !key.empty() && tuned_lookup(key, &names) && apply_names(names) == MHD_OK) return MHD_OK;
    if (active.empty()) return fail(MHD_ERR_STATE, "autotune needs at least one active slot");
    std::vector<std::vector<double>> best;
    if ((rc = tune_rounds(best))) return rc;
    for (int c = 0; c < kTunedClasses; ++c) {
      int pick = ops->sel[c];
      for (int i = 0; i < (int)best[c].size(); ++i)
        if (best[c][i] < best[c][pick]) pick = i;
      ops->sel[c] = pick;
    }
    if (!key.empty()) tuned_store(key, selected_names(), persist);
    invalidate_graph();
    return MHD_OK;
  }
  int build_graph(bool with_diag = false) {
    cudaGraphExec_t& out = with_diag ? graph_diag : graph;
    if (out) return MHD_OK;
    cudaGraph_t gr = nullptr;
    MHD_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = issue_step(with_diag);
    cudaError_t e = cudaStreamEndCapture(stream, &gr);
    if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
    if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&out, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) { out = nullptr; return fail(MHD_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)); }
    return MHD_OK;
  }
  void advance_clocks() {
    for (int s : active) {
      if (!cfl) t[s] += hparams[s].dt;  // with the on-device CFL the clock lives on the device
      stepc[s] += 1;
    }
  }
  void invalidate_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    if (graph_diag) cudaGraphExecDestroy(graph_diag);
    graph_diag = nullptr;
    ++graph_version;
  }
  int run_steps(int nsteps) {
    int rc;
    if ((rc = sync_lists())) return rc;
    if (active.empty()) return MHD_OK;
    if (!profiling && (rc = build_graph())) return rc;
    for (int i = 0; i < nsteps; ++i) {
      const bool rec = diag_freq > 0 && (hsteps + 1) % diag_freq == 0;
      if (profiling) {
        if ((rc = issue_step(rec))) return rc;
      } else {
        if (rec && (rc = build_graph(true))) return rc;
        MHD_CUDA(cudaGraphLaunch(rec ? graph_diag : graph, stream));
      }
      advance_clocks();
      ++hsteps;
      if (rec) {
        hist_step.push_back(hsteps);
        std::vector<double> tt(cap, 0.0);
        for (int s2 : active) tt[s2] = t[s2];
        hist_t.push_back(tt);
      }
    }
    return MHD_OK;
  }
  // One field of one slot: compact (src) -> physical staging, normalised inverse.
  // scale < 0: the normalised inverse (1/n^3)
  int inverse_field(const float2* src, long long sI, int slot, float scale = -1.f) {
    int rc;
    const BatchRef br = slot_ref(slot);
    if ((rc = z_inverse(src, sI, 1, br))) return rc;
    if ((rc = y_inverse(1, br))) return rc;
    float2* rb = rowbuf + slot * sz.rowbuf;
    const float sc = scale < 0.f ? (float)(1.0 / ((double)g.n * g.n * g.n)) : scale;
    return launch(KC_OTHER, [&] { ops->x_c2r(rb, phys, g, SLK(), sc, stream); });
  }
  // One field of one slot: physical staging -> compact (dst + slot*dI), unnormalised forward.
  int forward_field(float2* dst, long long dI, int slot) {
    int rc;
    const BatchRef br = slot_ref(slot);
    float2* rb = rowbuf + slot * sz.rowbuf;
    if ((rc = launch(KC_OTHER, [&] { ops->x_r2c(phys, rb, g, SLK(), stream); }))) return rc;
    if ((rc = y_forward(1, br))) return rc;
    return z_forward(dst, dI, 1, br);
  }
  bool valid_slot(int s) const { return s >= 0 && s < cap && used[s]; }
  // Tensor maps of the column passes' sources (coordinates: kx first, then the dimensions
  // named; rows = the transformed axis).  A map that cannot be encoded leaves the pass on the
  // cp.async kernels.
  void build_tma() {
    const cuuint64_t E = sizeof(float2), kxp = g.kxp, k2 = g.k2, n = g.n, C = cap;
    const cuuint32_t kp = g.kp, rb = g.n <= 256 ? g.n : 256;
    auto set = [&](TmaPass& t, void* base, const cuuint64_t (&d)[5], const cuuint64_t (&st)[4],
                   const cuuint32_t (&box)[5], TmaCoords tc) {
      t.ok = make_tmap(&t.map, base, d, st, box);
      t.tc = tc;
      t.err = derr;
    };
    // z_inverse over sol / xs [slot][f][kz'][ky'][kx]: rows kz', outer ky'
    const cuuint64_t dz[5] = {kxp, k2, k2, 6, C};
    const cuuint64_t sz5[4] = {kxp * E, k2 * kxp * E, (cuuint64_t)sz.fs * E, (cuuint64_t)sz.state * E};
    const cuuint32_t bz[5] = {16, 1, kp, 1, 1};
    set(tm_zinv_sol, sol, dz, sz5, bz, TmaCoords{2, 1, 3, 4, (int)kp});
    set(tm_zinv_xs, xs, dz, sz5, bz, TmaCoords{2, 1, 3, 4, (int)kp});
    // colbuf [slot][z][ky'][ns][kx] and rowbuf [slot][z][y][ns][kx]
    const cuuint64_t S = ns;
    const cuuint64_t dc[5] = {kxp, S, k2, n, C};
    const cuuint64_t sc[4] = {kxp * E, S * kxp * E, k2 * S * kxp * E, (cuuint64_t)sz.colbuf * E};
    const cuuint64_t dr[5] = {kxp, S, n, n, C};
    const cuuint64_t sr[4] = {kxp * E, S * kxp * E, n * S * kxp * E, (cuuint64_t)sz.rowbuf * E};
    const cuuint32_t by_in[5] = {16, 1, kp, 1, 1};
    const cuuint32_t by_out[5] = {16, 1, rb, 1, 1};
    const cuuint32_t bz_out[5] = {16, 1, 1, rb, 1};
    set(tm_yinv, colbuf, dc, sc, by_in, TmaCoords{2, 3, 1, 4, (int)kp});      // rows ky', outer z
    set(tm_yfwd, rowbuf, dr, sr, by_out, TmaCoords{2, 3, 1, 4, (int)rb});     // rows y, outer z
    set(tm_zfwd, colbuf, dc, sc, bz_out, TmaCoords{3, 2, 1, 4, (int)rb});     // rows z, outer ky'
  }
  // a TMA tile wait that timed out on the device (checked where the library synchronises)
  int check_device_error() {
    int e = 0;
    MHD_CUDA(cudaMemcpy(&e, derr, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) return fail(MHD_ERR_CUDA, e == 2 ? "TMA buffer misaligned in shared memory" : "a TMA tile wait timed out on the device");
    if (ops->x_device_error()) return fail(MHD_ERR_CUDA, "a tensor-core completion wait of the x rows timed out on the device");
    return MHD_OK;
  }
  // Hydrodynamics runs the MHD kernels with B = 0: the epilogue sets the induction right-hand
  // side to zero, so B stays exactly zero, and the momentum right-hand side is HDcalcN!'s (the
  // x rows pair uz with bx in one transform, so they see FP32 roundoff in place of bx = 0; its
  // products enter the momentum at ~1e-14 relative).  Only the three velocity fields cross the
  // boundary.
  int nfields() const { return p.hydro_only ? 3 : 6; }
  // the dedicated hydrodynamic passes (three fields in, five products out; with volume
  // penalisation also the three velocity penalty fields, in the spare slots 5..7)
  bool hd_form() const { return p.hydro_only != 0; }
  long long ref_elems() const { return sz.ref / 6 * nfields(); }
};

namespace {

int check_handle(mhd_handle h) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  return MHD_OK;
}

int check_slot(mhd_handle h, int slot) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!h->valid_slot(slot)) return fail(MHD_ERR_INVALID, "slot " + std::to_string(slot) + " is not active");
  return h->sync_lists();
}

int validate(const mhd_params* p) {
  if (!p) return fail(MHD_ERR_INVALID, "null params");
  if (!supported(p->n)) return fail(MHD_ERR_INVALID, "unsupported grid size n=" + std::to_string(p->n) + " (supported: 16,32,48,64,96,128,256,512)");
  if (!(p->L > 0) || !std::isfinite(p->L)) return fail(MHD_ERR_INVALID, "box size L must be positive");
  if (!(p->nu >= 0) || !(p->eta >= 0)) return fail(MHD_ERR_INVALID, "nu and eta must be non-negative");
  if (p->nnu > 1 || p->neta > 1) return fail(MHD_ERR_INVALID, "hyper-diffusion (nnu > 1 or neta > 1) is not on this path");
  if (!std::isfinite(p->dt)) return fail(MHD_ERR_INVALID, "dt must be finite");
  if (p->scheme != MHD_RK4 && p->scheme != MHD_LSRK4) return fail(MHD_ERR_INVALID, "scheme must be MHD_RK4 or MHD_LSRK4");
  if (p->hydro_only != 0 && p->hydro_only != 1) return fail(MHD_ERR_INVALID, "hydro_only must be 0 or 1");
  if (p->precision != MHD_PREC_FP32 && p->precision != MHD_PREC_SPLIT_FP16 && p->precision != MHD_PREC_SPLIT_BF16 &&
      p->precision != MHD_PREC_SPLIT_TF32)
    return fail(MHD_ERR_INVALID,
                "precision must be MHD_PREC_FP32, MHD_PREC_SPLIT_FP16, MHD_PREC_SPLIT_BF16 or MHD_PREC_SPLIT_TF32");
  if ((p->precision == MHD_PREC_SPLIT_FP16 || p->precision == MHD_PREC_SPLIT_BF16) && p->n != 128 && p->n != 256 &&
      p->n != 512)
    return fail(MHD_ERR_INVALID, "the split FP16 / BF16 tensor-core forms exist for n = 128, 256, 512");
  if (p->precision == MHD_PREC_SPLIT_TF32 && p->n != 256)
    return fail(MHD_ERR_INVALID, "the split TF32 tcgen05 form exists for n = 256");
  if (p->vp != 0 && p->vp != 1) return fail(MHD_ERR_INVALID, "vp must be 0 or 1");
  if (p->vp && p->precision != MHD_PREC_FP32)
    return fail(MHD_ERR_INVALID, "volume penalisation runs in the FP32 form only");
  return MHD_OK;
}

int create_class(const mhd_params* params, int cap, mhd_handle* out) {
  g_err.clear();
  if (!out) return fail(MHD_ERR_INVALID, "null output handle");
  *out = nullptr;
  int rc = validate(params);
  if (rc) return rc;
  if (cap < 1 || cap > 4096) return fail(MHD_ERR_INVALID, "capacity must be 1..4096");
  {
    const Geom g0 = make_geom(params->n, params->L);
    if ((long long)g0.k2 * cap > 65535) return fail(MHD_ERR_INVALID, "capacity too large for this grid size");
  }
  std::unique_ptr<mhd_problem> h(new (std::nothrow) mhd_problem());
  if (!h) return fail(MHD_ERR_OOM, "host allocation failed");
  h->p = *params;
  h->cap = cap;
  h->device = params->device;
  MHD_CUDA(cudaSetDevice(h->device));
  h->g = make_geom(params->n, params->L);
  h->ns = slots_of(params->vp != 0 && !params->hydro_only);
  h->sz = sizes_of(h->g, h->ns);
  h->ops.reset(make_ops(params->n));
  if (!h->ops) return fail(MHD_ERR_INVALID, "no plan for n");
  h->ops->prec = params->precision;
  h->ops->vp_capable = params->vp != 0;
  h->ops->hd = h->hd_form() ? 1 : 0;
  if ((rc = h->ops->setup(h->g))) return rc;
  if (params->vp && (rc = h->ops->set_vp(1))) return rc;  // mask only until walls are set
  {
    // a selection the autotuner made earlier for this device and grid size (this process or the
    // tuning file); the defaults otherwise
    const std::string key = tune_key(h->device, h->g.n, params->precision, h->ops->vp, h->ops->hd);
    std::vector<std::string> names;
    if (!key.empty() && tuned_lookup(key, &names)) h->apply_names(names);
  }
  MHD_CUDA(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
  h->stream = h->own_stream;
  const Sizes& s = h->sz;
  const size_t c = (size_t)cap;
  MHD_CUDA(h->alloc_guarded(&h->sol, c * s.state * sizeof(float2)));
  MHD_CUDA(h->alloc_guarded(&h->xs, c * s.state * sizeof(float2)));
  MHD_CUDA(h->alloc_guarded(&h->acc, c * s.state * sizeof(float2)));
  MHD_CUDA(h->alloc_guarded(&h->aux, c * s.fs * sizeof(float2)));
  MHD_CUDA(h->alloc_guarded(&h->colbuf, c * s.colbuf * sizeof(float2)));
  MHD_CUDA(h->alloc_guarded(&h->rowbuf, c * s.rowbuf * sizeof(float2)));
  MHD_CUDA(h->alloc_guarded(&h->ref, s.ref * sizeof(float2)));
  MHD_CUDA(h->alloc_guarded(&h->phys, s.phys * sizeof(float)));
  MHD_CUDA(cudaMalloc(&h->diag_partial, (size_t)s.diag_blocks * kDiagSlots * sizeof(double)));
  MHD_CUDA(cudaMalloc(&h->diag_out, 16 * sizeof(double)));
  MHD_CUDA(cudaMalloc(&h->maxabs, 16 * sizeof(unsigned int)));
  MHD_CUDA(cudaMalloc(&h->dparams, c * sizeof(SlotParams)));
  MHD_CUDA(cudaMalloc(&h->dlist, (2 * c + 2) * sizeof(int)));
  MHD_CUDA(cudaMalloc(&h->dvmax, 2 * c * sizeof(unsigned int)));
  MHD_CUDA(cudaMalloc(&h->dtime, c * sizeof(double)));
  MHD_CUDA(cudaMalloc(&h->dstep, c * sizeof(long long)));
  MHD_CUDA(cudaMalloc(&h->derr, sizeof(int)));
  MHD_CUDA(cudaMemsetAsync(h->derr, 0, sizeof(int), h->stream));
  MHD_CUDA(cudaMemsetAsync(h->dstep, 0, c * sizeof(long long), h->stream));
  MHD_CUDA(cudaMemsetAsync(h->dvmax, 0, 2 * c * sizeof(unsigned int), h->stream));
  MHD_CUDA(cudaMemsetAsync(h->dtime, 0, c * sizeof(double), h->stream));
  MHD_CUDA(cudaMemsetAsync(h->sol, 0, c * s.state * sizeof(float2), h->stream));
  MHD_CUDA(cudaMemsetAsync(h->xs, 0, c * s.state * sizeof(float2), h->stream));
  MHD_CUDA(cudaMemsetAsync(h->acc, 0, c * s.state * sizeof(float2), h->stream));
  if (params->vp) {
    MHD_CUDA(h->alloc_guarded(&h->vchi, c * s.phys * sizeof(float)));
    MHD_CUDA(h->alloc_guarded(&h->vwall, 6 * c * s.phys * sizeof(float)));
    MHD_CUDA(cudaMemsetAsync(h->vchi, 0, c * s.phys * sizeof(float), h->stream));
    MHD_CUDA(cudaMemsetAsync(h->vwall, 0, 6 * c * s.phys * sizeof(float), h->stream));
  }
  h->walls.assign(cap, 0);
  h->build_tma();
  h->hparams.assign(cap, SlotParams{0.f, 0.f, 0.f, 0.f});
  h->used.assign(cap, 0);
  h->t.assign(cap, 0.0);
  h->stepc.assign(cap, 0);
  h->list_dirty = true;
  if ((rc = h->sync_lists())) return rc;
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  *out = h.release();
  return MHD_OK;
}

int add_slot(mhd_handle h, double nu, double eta, double dt, int* slot) {
  if (!(nu >= 0) || !(eta >= 0) || !std::isfinite(dt)) return fail(MHD_ERR_INVALID, "nu, eta >= 0 and finite dt required");
  int s = -1;
  for (int i = 0; i < h->cap; ++i) if (!h->used[i]) { s = i; break; }
  if (s < 0) return fail(MHD_ERR_STATE, "size class is full (capacity " + std::to_string(h->cap) + ")");
  h->used[s] = 1;
  h->active.push_back(s);
  const double dl = h->p.L / h->g.n, vi = nu > eta ? nu : eta;
  h->hparams[s] = SlotParams{(float)nu, (float)eta, (float)dt, vi > 0 ? (float)(h->cfl_coef * dl * dl / vi) : 0.f};
  if (h->cfl) MHD_CUDA(cudaMemsetAsync(h->dtime + s, 0, sizeof(double), h->stream));
  MHD_CUDA(cudaMemsetAsync(h->dstep + s, 0, sizeof(long long), h->stream));
  h->t[s] = 0.0;
  h->stepc[s] = 0;
  h->list_dirty = true;
  MHD_CUDA(cudaMemsetAsync(h->sol + s * h->sz.state, 0, h->sz.state * sizeof(float2), h->stream));
  if (slot) *slot = s;
  return MHD_OK;
}

}  // namespace

extern "C" {

const char* mhd_last_error(void) { return g_err.c_str(); }

int mhd_supported_n(int n) { return supported(n) ? 1 : 0; }

int mhd_kept_modes(int n, int* kx, int* kp, int* kn) {
  if (n < 4 || n % 2 || !kx || !kp || !kn) return fail(MHD_ERR_INVALID, "n must be even and >= 4, outputs non-null");
  kept_modes(n, kx, kp, kn);
  return MHD_OK;
}

int mhd_footprint_bytes(const mhd_params* params, long long* bytes) {
  int rc = validate(params);
  if (rc) return rc;
  if (!bytes) return fail(MHD_ERR_INVALID, "null output");
  *bytes = footprint(make_geom(params->n, params->L), 1, params->vp != 0, params->hydro_only != 0);
  return MHD_OK;
}

int mhd_slot_bytes(const mhd_params* params, long long* per_slot, long long* per_class) {
  int rc = validate(params);
  if (rc) return rc;
  const Geom g = make_geom(params->n, params->L);
  if (per_slot) *per_slot = slot_bytes(g, params->vp != 0, params->hydro_only != 0);
  if (per_class) *per_class = class_bytes(g);
  return MHD_OK;
}

int mhd_create(const mhd_params* params, mhd_handle* out) {
  int rc = create_class(params, 1, out);
  if (rc) return rc;
  if ((rc = add_slot(*out, params->nu, params->eta, params->dt, nullptr))) {
    delete *out;
    *out = nullptr;
    return rc;
  }
  return (*out)->sync_lists();
}

int mhd_batch_create(const mhd_params* params, int capacity, mhd_handle* out) {
  return create_class(params, capacity, out);
}

int mhd_destroy(mhd_handle h) {
  if (!h) return MHD_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  delete h;
  return MHD_OK;
}

int mhd_batch_add(mhd_handle h, double nu, double eta, double dt, int* slot) {
  int rc = check_handle(h);
  if (rc) return rc;
  return add_slot(h, nu, eta, dt, slot);
}

int mhd_batch_remove(mhd_handle h, int slot) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!h->valid_slot(slot)) return fail(MHD_ERR_INVALID, "slot " + std::to_string(slot) + " is not active");
  h->used[slot] = 0;
  for (size_t i = 0; i < h->active.size(); ++i)
    if (h->active[i] == slot) { h->active.erase(h->active.begin() + i); break; }
  h->list_dirty = true;
  return MHD_OK;
}

int mhd_batch_info(mhd_handle h, int* capacity, int* active) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  if (capacity) *capacity = h->cap;
  if (active) *active = (int)h->active.size();
  return MHD_OK;
}

}  // extern "C"

namespace {

// Device address of a host buffer of `bytes` bytes that kernels can read and write directly:
// page-locked memory mapped into the device address space (mhd_host_alloc, cudaHostAlloc,
// cudaHostRegister), where a kernel reaches the host over NVLink-C2C / PCIe without a staging
// copy.  Both ends of the range must lie in one mapping.  nullptr for anything else (pageable
// memory goes through the staging buffer and cudaMemcpyAsync).
void* mapped_host(const void* p, size_t bytes) {
  cudaPointerAttributes a0, a1;
  const char* q = static_cast<const char*>(p);
  if (cudaPointerGetAttributes(&a0, q) != cudaSuccess || cudaPointerGetAttributes(&a1, q + bytes - 1) != cudaSuccess) {
    cudaGetLastError();  // clear the error of a pointer the runtime does not know
    return nullptr;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
    return nullptr;
  if (static_cast<char*>(a1.devicePointer) - static_cast<char*>(a0.devicePointer) != (ptrdiff_t)(bytes - 1))
    return nullptr;
  return a0.devicePointer;
}

// Host worker threads for zeroing host memory (created on first use and kept: starting threads
// on every call costs tens of microseconds each).  run(n, fn) calls fn(i) for i in [0, n) on
// the workers and the calling thread and returns when every call has finished; one run at a time.
// A forked child has none of its parent's workers, so a process gets its own pool.
class HostPool {
 public:
  static HostPool& get() {
    static std::mutex mk;
    static HostPool* pool = nullptr;
    static pid_t owner = 0;
    std::lock_guard<std::mutex> lk(mk);
    if (!pool || owner != getpid()) {
      // $MHDGB_HOST_THREADS threads in all (the caller included), else the hardware threads, at
      // most 16 (on the 16-core Grace host, 8 threads left the zeros of get_state less hidden
      // behind the step: 4.0-4.4 ms per e2e step against 4.0-4.15 ms, 4 threads 6 ms)
      const unsigned hw = std::thread::hardware_concurrency();
      int nt = (int)std::min<unsigned>(16, hw ? hw : 1);
      if (const char* e = std::getenv("MHDGB_HOST_THREADS")) nt = std::max(1, std::min(64, std::atoi(e)));
      pool = new HostPool(nt - 1);  // never destroyed: the workers sleep until the process ends
      owner = getpid();
    }
    return *pool;
  }
  int threads() const { return (int)workers_.size() + 1; }
  void run(int n, const std::function<void(int)>& fn) {
    std::lock_guard<std::mutex> one(call_);
    {
      std::lock_guard<std::mutex> lk(m_);
      fn_ = &fn;
      n_ = n;
      next_.store(0);
      busy_ = (int)workers_.size();
      ++gen_;
    }
    cv_.notify_all();
    drain();
    std::unique_lock<std::mutex> lk(m_);
    done_.wait(lk, [&] { return busy_ == 0; });
    fn_ = nullptr;
  }

 private:
  explicit HostPool(int workers) {
    for (int i = 0; i < workers; ++i) workers_.emplace_back([this] { loop(); });
    for (auto& t : workers_) t.detach();
  }
  void drain() {
    for (int i = next_.fetch_add(1); i < n_; i = next_.fetch_add(1)) (*fn_)(i);
  }
  void loop() {
    unsigned seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
      }
      drain();
      std::lock_guard<std::mutex> lk(m_);
      if (--busy_ == 0) done_.notify_all();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex call_, m_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* fn_ = nullptr;
  int n_ = 0, busy_ = 0;
  unsigned gen_ = 0;
  std::atomic<int> next_{0};
};

// The alias band of a reference-layout state (nf, n, n, nkr) outside the retained band (the
// complement of scatter_retained_kernel) has three parts per field: the z-planes of the alias
// band [kp, n - kn) (one contiguous block), a block of alias rows [kp, n - kn) in every kept
// z-plane, and the tail kx >= Kx of every kept row.  zero_alias_host zeroes the tails on the
// host pool, and the alias z-planes (planes_too) and row blocks (blocks) when asked, in pieces
// of about 1 MB; zero_alias_blocks writes the others from the copy engine.
void zero_alias_host(float2* ref, const Geom& g, int nf, bool planes_too, bool blocks) {
  const size_t nkr = g.n / 2 + 1, row = nkr * sizeof(float2), plane = (size_t)g.n * row;
  const size_t tail = (nkr - g.kx) * sizeof(float2);
  const size_t na = (size_t)(g.n - g.kp - g.kn);
  char* base = reinterpret_cast<char*>(ref);
  struct Piece { char* p; size_t bytes; };
  std::vector<Piece> big;                 // contiguous pieces
  constexpr size_t kChunk = size_t(1) << 20;
  if (planes_too)
    for (int f = 0; f < nf; ++f) {
      char* p = base + ((size_t)f * g.n + g.kp) * plane;  // alias z-planes
      for (size_t left = na * plane; left > 0;) {
        const size_t b = std::min(left, kChunk);
        big.push_back({p, b});
        p += b;
        left -= b;
      }
    }
  const int planes = nf * g.k2;  // kept z-planes: alias row block and row tails
  const int per_task = std::max(1, (int)(kChunk / (na * row + (size_t)g.k2 * tail)));
  const int ptasks = (planes + per_task - 1) / per_task;
  auto kept_plane = [&](int q) {
    const int f = q / g.k2, jz = q % g.k2;
    char* p = base + ((size_t)f * g.n + freq_of_kept(g, jz)) * plane;
    if (blocks) std::memset(p + (size_t)g.kp * row, 0, na * row);
    for (int j = 0; j < g.k2; ++j) std::memset(p + (size_t)freq_of_kept(g, j) * row + g.kx * sizeof(float2), 0, tail);
  };
  const int nbig = (int)big.size();
  HostPool::get().run(nbig + ptasks, [&](int i) {
    if (i < nbig) {
      std::memset(big[i].p, 0, big[i].bytes);
    } else {
      const int q0 = (i - nbig) * per_task, q1 = std::min(planes, q0 + per_task);
      for (int q = q0; q < q1; ++q) kept_plane(q);
    }
  });
}

// Which path writes the alias-band zeros of get_state into mapped host memory
// ($MHDGB_HOST_ZEROS, read once).  The copy engine's zeros share the host link with the retained
// band (about 193 GB/s device to host); the host pool writes at about 120 GB/s on its own.
//   split (default) copy engine: the alias z-planes; host pool: the row blocks and row tails
//   ce     copy engine: the z-planes and the row blocks; host pool: the row tails
//   host   host pool: everything
enum class ZeroPath { Split, CopyEngine, Host };
ZeroPath zero_path() {
  static const ZeroPath z = [] {
    const char* e = std::getenv("MHDGB_HOST_ZEROS");
    if (e && std::strcmp(e, "ce") == 0) return ZeroPath::CopyEngine;
    if (e && std::strcmp(e, "host") == 0) return ZeroPath::Host;
    return ZeroPath::Split;
  }();
  return z;
}

// Copy-engine writes of zeros from `zeros` (zbytes of zeroed device memory) into the alias planes
// and (blocks) the alias row blocks of a host reference-layout state, on stream s.
cudaError_t zero_alias_blocks(float2* ref, const Geom& g, int nf, const void* zeros, size_t zbytes, cudaStream_t s,
                              bool blocks) {
  const size_t nkr = g.n / 2 + 1, row = nkr * sizeof(float2), plane = (size_t)g.n * row;
  const size_t na = (size_t)(g.n - g.kp - g.kn);
  char* base = reinterpret_cast<char*>(ref);
  for (int f = 0; f < nf; ++f) {
    // the alias z-planes of field f: one contiguous block, in pieces of at most zbytes
    char* p = base + ((size_t)f * g.n + g.kp) * plane;
    for (size_t left = na * plane; left > 0;) {
      const size_t b = std::min(left, zbytes);
      const cudaError_t e = cudaMemcpyAsync(p, zeros, b, cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) return e;
      p += b;
      left -= b;
    }
    if (!blocks) continue;
    // the alias row block of every kept z-plane: width na rows, one plane apart, in groups of
    // planes that fit the zero buffer
    const size_t width = na * row;
    const size_t per = std::max<size_t>(1, zbytes / width);
    const int z0[2] = {0, g.n - g.kn}, zc[2] = {g.kp, g.kn};
    for (int r = 0; r < 2; ++r)
      for (int z = 0; z < zc[r]; z += (int)per) {
        const size_t h = std::min<size_t>(per, (size_t)(zc[r] - z));
        char* d = base + (((size_t)f * g.n + z0[r] + z) * g.n + g.kp) * row;
        const cudaError_t e = cudaMemcpy2DAsync(d, plane, zeros, width, width, h, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return e;
      }
  }
  return cudaSuccess;
}

// How state transfers to and from page-locked host buffers mapped into the device address space
// move their bytes ($MHDGB_HOST_TRANSFER, read once; other host memory always takes the copy path):
//   mapped (default) kernels read and write the caller's array directly: set_state gathers the
//          retained band of half the fields over the link while the copy engine brings the other
//          half; get_state writes the alias-band zeros from the copy engine (the alias z-planes,
//          from a zeroed device buffer) and from the host pool (row blocks and row tails) while
//          the step still runs, then the retained band crosses on both paths at once.
//   copy   the copy engines only (about 200 GB/s over the host link): set_state copies the
//          retained band of the caller's array into the device staging array (one 3-D copy per
//          field and ky / kz range) and gathers it there; get_state scatters into the staging
//          array at HBM speed and brings the whole array back in one contiguous copy.
bool mapped_transfers() {
  static const bool m = [] {
    const char* e = std::getenv("MHDGB_HOST_TRANSFER");
    return !(e && std::strcmp(e, "copy") == 0);
  }();
  return m;
}

// The retained band of a reference-layout state (nf, n, n, nkr) between two arrays of that
// layout: for each field, the kept ky and kz ranges [0, kp) and [n - kn, n) form four boxes of
// kx < Kx rows (one cudaMemcpy3DAsync each).
cudaError_t copy_retained(void* dst, const void* src, const Geom& g, int nf, cudaMemcpyKind kind, cudaStream_t s) {
  const size_t pitch = (size_t)(g.n / 2 + 1) * sizeof(float2);
  const int r0[2] = {0, g.n - g.kn}, rc[2] = {g.kp, g.kn};
  for (int f = 0; f < nf; ++f)
    for (int bz = 0; bz < 2; ++bz)
      for (int by = 0; by < 2; ++by) {
        if (rc[bz] == 0 || rc[by] == 0) continue;
        cudaMemcpy3DParms p = {};
        p.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), pitch, pitch, g.n);
        p.dstPtr = make_cudaPitchedPtr(dst, pitch, pitch, g.n);
        p.srcPos = make_cudaPos(0, r0[by], (size_t)f * g.n + r0[bz]);
        p.dstPos = p.srcPos;
        p.extent = make_cudaExtent((size_t)g.kx * sizeof(float2), rc[by], rc[bz]);
        p.kind = kind;
        const cudaError_t e = cudaMemcpy3DAsync(&p, s);
        if (e != cudaSuccess) return e;
      }
  return cudaSuccess;
}

// Device memory (or managed memory) that kernels of the current device can use, of `bytes`.
bool is_device_memory(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" {

int mhd_slot_set_state(mhd_handle h, int slot, const float* sol) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (!sol) return fail(MHD_ERR_INVALID, "null sol");
  const int nf = h->nfields();
  const size_t bytes = h->ref_elems() * sizeof(float2);
  const long long fref = h->ref_elems() / nf;  // one field of the reference layout
  float2* dst = h->sol + slot * h->sz.state;
  const float2* mapped = mapped_transfers() ? static_cast<const float2*>(mapped_host(sol, bytes)) : nullptr;
  if (mapped) {
    // the retained band crosses the host link on two paths at once: the gather kernel reads the
    // first half of the fields straight from the mapped array, while the copy engine brings the
    // retained band of the other half into the staging array, gathered from there
    if ((rc = h->ensure_zero_source())) return rc;
    const int hf = nf / 2;
    MHD_CUDA(cudaEventRecord(h->ev_z, h->stream));  // the staging array is free once earlier work is done
    MHD_CUDA(cudaStreamWaitEvent(h->zstream, h->ev_z, 0));
    const cudaError_t e = copy_retained(h->ref + hf * fref, reinterpret_cast<const float2*>(sol) + hf * fref, h->g,
                                        nf - hf, cudaMemcpyHostToDevice, h->zstream);
    if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("set_state copy: ") + cudaGetErrorString(e));
    MHD_CUDA(cudaEventRecord(h->ev_z, h->zstream));
    if ((rc = h->launch(KC_OTHER, [&] { gather_state_kernel<<<1216, 256, 0, h->stream>>>(mapped, dst, h->g, hf); }))) return rc;
    MHD_CUDA(cudaStreamWaitEvent(h->stream, h->ev_z, 0));
    if ((rc = h->launch(KC_OTHER, [&] {
           gather_state_kernel<<<1216, 256, 0, h->stream>>>(h->ref + hf * fref, dst + hf * h->sz.fs, h->g, nf - hf);
         })))
      return rc;
  } else {
    // only the retained band crosses the link (29% of the array), into the staging array
    const cudaError_t e = copy_retained(h->ref, sol, h->g, nf, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("set_state copy: ") + cudaGetErrorString(e));
    if ((rc = h->launch(KC_OTHER, [&] { gather_state_kernel<<<1216, 256, 0, h->stream>>>(h->ref, dst, h->g, nf); }))) return rc;
  }
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_slot_get_state(mhd_handle h, int slot, float* sol) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (!sol) return fail(MHD_ERR_INVALID, "null sol");
  const int nf = h->nfields();
  const float2* src = h->sol + slot * h->sz.state;
  const size_t bytes = h->ref_elems() * sizeof(float2);
  const long long fref = h->ref_elems() / nf;
  float2* out = mapped_transfers() ? static_cast<float2*>(mapped_host(sol, bytes)) : nullptr;
  if (out && bytes < (size_t(16) << 20)) {
    // small mapped buffers: the device writes every element
    if ((rc = h->launch(KC_OTHER, [&] {
           scatter_state_kernel<<<1216, 256, 0, h->stream>>>(src, out, h->g, nf);
         })))
      return rc;
  } else if (out) {
    // mapped memory.  The zeros of the alias band do not wait for the step: the copy engine
    // writes the alias z-planes from a zeroed device buffer on a side stream, and the host pool
    // zeroes the alias row blocks and row tails, both while the handle's stream still runs
    // (zero_path).  After the step the retained band (29% of the bytes) crosses on two paths at
    // once: the device writes the first half of the fields straight into the mapping, and the
    // other half is scattered into the staging array and brought over by the copy engine.
    if ((rc = h->ensure_zero_source())) return rc;
    const int hf = nf / 2;
    float2* host = reinterpret_cast<float2*>(sol);
    const ZeroPath zp = zero_path();
    if (zp != ZeroPath::Host)
      MHD_CUDA(zero_alias_blocks(host, h->g, nf, h->zeros, h->zbytes, h->zstream, zp == ZeroPath::CopyEngine));
    if ((rc = h->launch(KC_OTHER, [&] {
           scatter_retained_kernel<<<1216, 256, 0, h->stream>>>(src + hf * h->sz.fs, h->ref + hf * fref, h->g, nf - hf);
         })))
      return rc;
    MHD_CUDA(cudaEventRecord(h->ev_z, h->stream));
    MHD_CUDA(cudaStreamWaitEvent(h->zstream, h->ev_z, 0));
    MHD_CUDA(copy_retained(host + hf * fref, h->ref + hf * fref, h->g, nf - hf, cudaMemcpyDeviceToHost, h->zstream));
    if ((rc = h->launch(KC_OTHER, [&] {
           scatter_retained_kernel<<<1216, 256, 0, h->stream>>>(src, out, h->g, hf);
         })))
      return rc;
    zero_alias_host(host, h->g, nf, zp == ZeroPath::Host, zp != ZeroPath::CopyEngine);
    MHD_CUDA(cudaStreamSynchronize(h->zstream));
  } else {
    // the full array is assembled in the staging buffer at HBM speed, zeros included, and comes
    // back in one contiguous copy
    if ((rc = h->launch(KC_OTHER, [&] {
           scatter_state_kernel<<<1216, 256, 0, h->stream>>>(src, h->ref, h->g, nf);
         })))
      return rc;
    MHD_CUDA(cudaMemcpyAsync(sol, h->ref, bytes, cudaMemcpyDeviceToHost, h->stream));
  }
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

// prob.sol as a device array: the gather / scatter kernels read or write the caller's array
// directly, ordered on `stream` after the handle's earlier work and before its later work.
static int state_device(mhd_handle h, int slot, float* sol_dev, void* stream, bool to_state) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (!sol_dev) return fail(MHD_ERR_INVALID, "null device array");
  if (reinterpret_cast<uintptr_t>(sol_dev) % 16 != 0) return fail(MHD_ERR_INVALID, "the device array must be 16-byte aligned");
  if (!is_device_memory(sol_dev)) return fail(MHD_ERR_INVALID, "sol_dev is not device memory");
  // the caller's stream as given: 0 is the legacy default stream (torch's default, CUDA C's
  // default), which the handle's non-blocking stream does not synchronise with by itself
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (s != h->stream) {
    if (!h->ev_in) MHD_CUDA(cudaEventCreateWithFlags(&h->ev_in, cudaEventDisableTiming));
    if (!h->ev_out) MHD_CUDA(cudaEventCreateWithFlags(&h->ev_out, cudaEventDisableTiming));
    MHD_CUDA(cudaEventRecord(h->ev_in, h->stream));
    MHD_CUDA(cudaStreamWaitEvent(s, h->ev_in, 0));
  }
  float2* st = h->sol + slot * h->sz.state;
  float2* ref = reinterpret_cast<float2*>(sol_dev);
  if (to_state) gather_state_kernel<<<1216, 256, 0, s>>>(ref, st, h->g, h->nfields());
  else scatter_state_kernel<<<1216, 256, 0, s>>>(st, ref, h->g, h->nfields());
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string(to_state ? "gather" : "scatter") + " launch: " + cudaGetErrorString(e));
  if (s != h->stream) {
    MHD_CUDA(cudaEventRecord(h->ev_out, s));
    MHD_CUDA(cudaStreamWaitEvent(h->stream, h->ev_out, 0));
  }
  return MHD_OK;
}

int mhd_slot_set_state_device(mhd_handle h, int slot, const float* sol_dev, void* stream) {
  return state_device(h, slot, const_cast<float*>(sol_dev), stream, true);
}
int mhd_slot_get_state_device(mhd_handle h, int slot, float* sol_dev, void* stream) {
  return state_device(h, slot, sol_dev, stream, false);
}
int mhd_set_state_device(mhd_handle h, const float* sol_dev, void* stream) {
  return mhd_slot_set_state_device(h, 0, sol_dev, stream);
}
int mhd_get_state_device(mhd_handle h, float* sol_dev, void* stream) {
  return mhd_slot_get_state_device(h, 0, sol_dev, stream);
}

int mhd_slot_set_physical(mhd_handle h, int slot, int field, const float* phys) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (field < 0 || field >= h->nfields())
    return fail(MHD_ERR_INVALID, h->p.hydro_only ? "field must be 0..2 (ux uy uz)" : "field must be 0..5 (ux uy uz bx by bz)");
  if (!phys) return fail(MHD_ERR_INVALID, "null field array");
  MHD_CUDA(cudaMemcpyAsync(h->phys, phys, h->sz.phys * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  if ((rc = h->forward_field(h->sol + field * h->sz.fs, h->sz.state, slot))) return rc;
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_slot_get_physical(mhd_handle h, int slot, int field, float* phys) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (field < 0 || field >= h->nfields())
    return fail(MHD_ERR_INVALID, h->p.hydro_only ? "field must be 0..2 (ux uy uz)" : "field must be 0..5 (ux uy uz bx by bz)");
  if (!phys) return fail(MHD_ERR_INVALID, "null field array");
  if ((rc = h->inverse_field(h->sol + field * h->sz.fs, h->sz.state, slot))) return rc;
  MHD_CUDA(cudaMemcpyAsync(phys, h->phys, h->sz.phys * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_slot_get_clock(mhd_handle h, int slot, double* t, long long* step, double* dt) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  if (!h->valid_slot(slot)) return fail(MHD_ERR_INVALID, "slot " + std::to_string(slot) + " is not active");
  if (h->cfl) {  // dt and t are advanced on the device
    int rc = check_handle(h);
    if (rc) return rc;
    SlotParams sp;
    MHD_CUDA(cudaMemcpyAsync(&h->t[slot], h->dtime + slot, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    MHD_CUDA(cudaMemcpyAsync(&sp, h->dparams + slot, sizeof(SlotParams), cudaMemcpyDeviceToHost, h->stream));
    MHD_CUDA(cudaStreamSynchronize(h->stream));
    h->hparams[slot].dt = sp.dt;
  }
  if (t) *t = h->t[slot];
  if (step) *step = h->stepc[slot];
  if (dt) *dt = h->hparams[slot].dt;
  return MHD_OK;
}

int mhd_slot_set_clock(mhd_handle h, int slot, double t, long long step, double dt) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  if (!h->valid_slot(slot)) return fail(MHD_ERR_INVALID, "slot " + std::to_string(slot) + " is not active");
  if (!std::isfinite(t) || !std::isfinite(dt)) return fail(MHD_ERR_INVALID, "t and dt must be finite");
  h->t[slot] = t;
  h->stepc[slot] = step;
  {
    int rc = check_handle(h);
    if (rc) return rc;
    MHD_CUDA(cudaMemcpyAsync(h->dstep + slot, &h->stepc[slot], sizeof(long long), cudaMemcpyHostToDevice, h->stream));
    MHD_CUDA(cudaStreamSynchronize(h->stream));
  }
  if ((float)dt != h->hparams[slot].dt) {
    h->hparams[slot].dt = (float)dt;
    h->list_dirty = true;
  }
  if (h->cfl) {
    int rc = check_handle(h);
    if (rc) return rc;
    MHD_CUDA(cudaMemcpyAsync(h->dtime + slot, &h->t[slot], sizeof(double), cudaMemcpyHostToDevice, h->stream));
    MHD_CUDA(cudaStreamSynchronize(h->stream));
  }
  return MHD_OK;
}

int mhd_slot_set_forcing(mhd_handle h, int slot, double P, double kf, double sigma, double b,
                         unsigned long long seed) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (!std::isfinite(P) || P < 0 || !std::isfinite(kf) || !(sigma > 0) || !std::isfinite(sigma) || !(b > 0) ||
      !std::isfinite(b))
    return fail(MHD_ERR_INVALID, "forcing needs P >= 0, finite kf, sigma > 0 and b > 0");
  SlotParams& sp = h->hparams[slot];
  if (P == 0) {
    sp.fA = 0.f;
  } else {
    // SetUpFk! (src/pgen/A99ForceDriving_GPU.jl:24-48): A = sqrt(P 3 (L/dx)^3 / I / dx^3) with
    // I = sum over the (nkr, n, n) grid of exp(-(k - kf)^2 / sigma^2) / (k + 1)^2
    const int n = h->g.n, nkr = n / 2 + 1;
    const double ks = 2.0 * M_PI / h->p.L, dx = h->p.L / n;
    double integral = 0.0;
    for (int z = 0; z < n; ++z) {
      const double kz = ks * (z < (n + 1) / 2 ? z : z - n);
      for (int y = 0; y < n; ++y) {
        const double ky = ks * (y < (n + 1) / 2 ? y : y - n);
        for (int x = 0; x < nkr; ++x) {
          const double kx = ks * x;
          const double k = std::sqrt(kx * kx + ky * ky + kz * kz);
          integral += std::exp(-(k - kf) * (k - kf) / (sigma * sigma)) / ((k + 1) * (k + 1));
        }
      }
    }
    sp.fA = (float)std::sqrt(P * 3.0 * (double)n * n * n / integral * (1.0 / (dx * dx * dx)));
    sp.fkf = (float)b;  // SetUpFk! stores kf = b (src/pgen/A99ForceDriving_GPU.jl:46), kept as is
    sp.fs2 = (float)(sigma * sigma);
    sp.fb = (float)b;
    sp.fseed = seed;
  }
  h->list_dirty = true;
  bool any = false;
  for (int s = 0; s < h->cap; ++s) any = any || (h->used[s] && h->hparams[s].fA != 0.f);
  if (any != h->forcing) {
    h->forcing = any;
    h->invalidate_graph();
  }
  return h->sync_lists();
}

int mhd_set_forcing(mhd_handle h, double P, double kf, double sigma, double b, unsigned long long seed) {
  return mhd_slot_set_forcing(h, 0, P, kf, sigma, b, seed);
}

int mhd_slot_set_vp(mhd_handle h, int slot, const float* chi, const float* U0, const float* B0) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (!h->p.vp) return fail(MHD_ERR_STATE, "volume penalisation is off for this handle (mhd_params.vp = 0)");
  const long long n3 = h->sz.phys;
  const size_t fb = (size_t)n3 * sizeof(float);
  float* c = h->vchi + slot * n3;
  float* w = h->vwall + 6 * slot * n3;
  if (chi) MHD_CUDA(cudaMemcpyAsync(c, chi, fb, cudaMemcpyHostToDevice, h->stream));
  else MHD_CUDA(cudaMemsetAsync(c, 0, fb, h->stream));
  const float* src[2] = {U0, B0};
  for (int k = 0; k < 2; ++k) {
    if (src[k]) MHD_CUDA(cudaMemcpyAsync(w + 3 * k * n3, src[k], 3 * fb, cudaMemcpyHostToDevice, h->stream));
    else MHD_CUDA(cudaMemsetAsync(w + 3 * k * n3, 0, 3 * fb, h->stream));
  }
  h->walls[slot] = (U0 || B0) ? 1 : 0;
  bool any = false;
  for (int s = 0; s < h->cap; ++s) any = any || h->walls[s];
  const int mode = any ? 2 : 1;
  if (mode != h->ops->vp) {
    if ((rc = h->ops->set_vp(mode))) return rc;
    // a tuned selection of the new form, if one is known
    const std::string key = tune_key(h->device, h->g.n, h->p.precision, mode);
    std::vector<std::string> names;
    if (!key.empty() && tuned_lookup(key, &names)) h->apply_names(names);
    h->invalidate_graph();
  }
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_set_vp(mhd_handle h, const float* chi, const float* U0, const float* B0) {
  return mhd_slot_set_vp(h, 0, chi, U0, B0);
}

int mhd_slot_div_correct(mhd_handle h, int slot, int fields) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (fields < 0 || fields > 3) return fail(MHD_ERR_INVALID, "fields must be a mask of MHD_DIV_U and MHD_DIV_B");
  if (h->p.hydro_only) fields &= MHD_DIV_U;
  if (fields && (rc = h->div_correct(h->slot_ref(slot), 1, fields))) return rc;
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_div_correct(mhd_handle h, int fields) { return mhd_slot_div_correct(h, 0, fields); }

int mhd_set_div_correction(mhd_handle h, int on) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (on != 0 && on != 1) return fail(MHD_ERR_INVALID, "on must be 0 or 1");
  if ((on != 0) != h->divcorr) {
    MHD_CUDA(cudaStreamSynchronize(h->stream));
    h->divcorr = on != 0;
    h->invalidate_graph();
  }
  return MHD_OK;
}

int mhd_set_diag_history(mhd_handle h, int freq, int capacity) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (freq < 0 || capacity < 0 || (freq > 0 && capacity < 1))
    return fail(MHD_ERR_INVALID, "freq >= 0 and, with freq > 0, capacity >= 1 required");
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  h->free_history();
  h->hist_step.clear();
  h->hist_t.clear();
  h->hsteps = 0;
  h->diag_freq = freq;
  h->diag_capacity = freq > 0 ? capacity : 0;
  if (freq > 0) {
    const size_t c = (size_t)h->cap;
    MHD_CUDA(cudaMalloc(&h->dhist, (size_t)capacity * c * kHistVals * sizeof(double)));
    MHD_CUDA(cudaMalloc(&h->dhist_partial, c * h->sz.diag_blocks * kDiagSlots * sizeof(double)));
    MHD_CUDA(cudaMalloc(&h->dhist_count, sizeof(int)));
    MHD_CUDA(cudaMemsetAsync(h->dhist_count, 0, sizeof(int), h->stream));
    MHD_CUDA(cudaStreamSynchronize(h->stream));
  }
  h->invalidate_graph();
  return MHD_OK;
}

int mhd_get_diag_history(mhd_handle h, int slot, double* out, int max_samples, int* count) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (!count || (max_samples > 0 && !out)) return fail(MHD_ERR_INVALID, "null output");
  if (h->diag_freq <= 0) {
    *count = 0;
    return MHD_OK;
  }
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  int total = 0;
  MHD_CUDA(cudaMemcpy(&total, h->dhist_count, sizeof(int), cudaMemcpyDeviceToHost));
  const int stored = std::min(std::min(total, h->diag_capacity), (int)h->hist_step.size());
  *count = stored;
  const int n = std::min(stored, max_samples);
  if (n <= 0) return MHD_OK;
  std::vector<double> buf((size_t)n * h->cap * kHistVals);
  MHD_CUDA(cudaMemcpy(buf.data(), h->dhist, buf.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int k = 0; k < n; ++k) {
    const double* o = buf.data() + ((size_t)k * h->cap + slot) * kHistVals;
    double* r = out + (size_t)k * 8;
    r[0] = (double)h->hist_step[k];
    r[1] = o[6] >= 0 ? o[6] : h->hist_t[k][slot];
    for (int v = 0; v < 6; ++v) r[2 + v] = o[v];
  }
  return MHD_OK;
}

int mhd_check_guards(mhd_handle h, long long* bad_bytes) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!bad_bytes) return fail(MHD_ERR_INVALID, "null output");
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  unsigned long long* d = nullptr;
  MHD_CUDA(cudaMalloc(&d, sizeof(unsigned long long)));
  MHD_CUDA(cudaMemset(d, 0, sizeof(unsigned long long)));
  for (auto& gd : h->guards)
    guard_check_kernel<<<(unsigned)((gd.second + 255) / 256), 256>>>(gd.first, (long long)gd.second, mhd_problem::kGuardByte, d);
  unsigned long long bad = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(&bad, d, sizeof(bad), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("guard check: ") + cudaGetErrorString(e));
  *bad_bytes = (long long)bad;
  return MHD_OK;
}

int mhd_check_bounded_wait(int device, double limit_ms, int* timed_out, double* waited_ms) {
  if (!timed_out || !waited_ms) return fail(MHD_ERR_INVALID, "null output");
  if (!(limit_ms > 0) || limit_ms > 1000) return fail(MHD_ERR_INVALID, "limit_ms must be in (0, 1000]");
  MHD_CUDA(cudaSetDevice(device));
  unsigned long long* d = nullptr;
  MHD_CUDA(cudaMalloc(&d, 2 * sizeof(unsigned long long)));
  bounded_wait_check_kernel<<<1, 32>>>((unsigned long long)(limit_ms * 1e6), d);
  unsigned long long hbuf[2] = {0, 0};
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(hbuf, d, sizeof(hbuf), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("bounded wait check: ") + cudaGetErrorString(e));
  *timed_out = (int)hbuf[0];
  *waited_ms = (double)hbuf[1] * 1e-6;
  return MHD_OK;
}

int mhd_get_forcing(mhd_handle h, int slot, double* A, double* kf_used) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  if (!h->valid_slot(slot)) return fail(MHD_ERR_INVALID, "slot " + std::to_string(slot) + " is not active");
  if (A) *A = h->hparams[slot].fA;
  if (kf_used) *kf_used = h->hparams[slot].fkf;
  return MHD_OK;
}

int mhd_set_cfl(mhd_handle h, int enable, double coef) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (enable && !(coef > 0 && std::isfinite(coef))) return fail(MHD_ERR_INVALID, "CFL coefficient must be positive");
  if ((rc = h->sync_lists())) return rc;
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  if (enable) {
    h->cfl_coef = coef;
    const double dl = h->p.L / h->g.n;
    for (int s = 0; s < h->cap; ++s) {
      const double vi = h->hparams[s].nu > h->hparams[s].eta ? h->hparams[s].nu : h->hparams[s].eta;
      h->hparams[s].tdiff = vi > 0 ? (float)(coef * dl * dl / vi) : 0.f;
    }
    h->list_dirty = true;
    if ((rc = h->sync_lists())) return rc;
    MHD_CUDA(cudaMemcpyAsync(h->dtime, h->t.data(), h->cap * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    h->cfl = true;
    if ((rc = h->cfl_prime())) { h->cfl = false; return rc; }
    if ((rc = h->cfl_update(0))) { h->cfl = false; return rc; }
    std::vector<SlotParams> dev(h->cap);
    MHD_CUDA(cudaMemcpyAsync(dev.data(), h->dparams, h->cap * sizeof(SlotParams), cudaMemcpyDeviceToHost, h->stream));
    MHD_CUDA(cudaStreamSynchronize(h->stream));
    for (int s = 0; s < h->cap; ++s) h->hparams[s].dt = dev[s].dt;
  } else if (h->cfl) {
    std::vector<SlotParams> dev(h->cap);
    MHD_CUDA(cudaMemcpyAsync(h->t.data(), h->dtime, h->cap * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    MHD_CUDA(cudaMemcpyAsync(dev.data(), h->dparams, h->cap * sizeof(SlotParams), cudaMemcpyDeviceToHost, h->stream));
    MHD_CUDA(cudaStreamSynchronize(h->stream));
    for (int s = 0; s < h->cap; ++s) h->hparams[s].dt = dev[s].dt;
    h->cfl = false;
  }
  h->invalidate_graph();
  return MHD_OK;
}

int mhd_slot_diagnostics(mhd_handle h, int slot, double* out, int nout) {
  int rc = check_slot(h, slot);
  if (rc) return rc;
  if (!out || nout < 8) return fail(MHD_ERR_INVALID, "diagnostics needs an output array of >= 8 doubles");
  const Sizes& s = h->sz;
  const float2* st = h->sol + slot * s.state;
  float2* aux = h->aux + slot * s.fs;
  if ((rc = h->launch(KC_OTHER, [&] { diag_partial_kernel<<<s.diag_blocks, kDiagThreads, 0, h->stream>>>(st, h->g, h->diag_partial); }))) return rc;
  if ((rc = h->launch(KC_OTHER, [&] { diag_final_kernel<<<1, kDiagThreads, 0, h->stream>>>(h->diag_partial, s.diag_blocks, h->diag_out); }))) return rc;
  if ((rc = h->launch(KC_OTHER, [&] { divb_spectrum_kernel<<<1216, 256, 0, h->stream>>>(st, aux, h->g); }))) return rc;
  if ((rc = h->inverse_field(h->aux, s.fs, slot))) return rc;
  MHD_CUDA(cudaMemsetAsync(h->maxabs, 0, sizeof(unsigned int), h->stream));
  if ((rc = h->launch(KC_OTHER, [&] { maxabs_kernel<<<1216, 256, 0, h->stream>>>(h->phys, s.phys, h->maxabs); }))) return rc;
  double d[kDiagSlots];
  unsigned int mx = 0;
  MHD_CUDA(cudaMemcpyAsync(d, h->diag_out, sizeof(d), cudaMemcpyDeviceToHost, h->stream));
  MHD_CUDA(cudaMemcpyAsync(&mx, h->maxabs, sizeof(mx), cudaMemcpyDeviceToHost, h->stream));
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  const double n3 = (double)h->g.n * h->g.n * h->g.n;
  const double dx = h->p.L / h->g.n;
  const double scale = dx * dx * dx / n3;
  float mxf;
  std::memcpy(&mxf, &mx, sizeof(mxf));
  out[0] = d[0] * scale;
  out[1] = d[1] * scale;
  out[2] = d[2] * scale;
  out[3] = d[3];
  out[4] = d[4];
  out[5] = (double)mxf;
  out[6] = d[5];
  out[7] = h->t[slot];
  if (d[5] > 0 || !std::isfinite(out[0]) || !std::isfinite(out[1])) return fail(MHD_ERR_NONFINITE, "detected NaN! Quit the simulation right now.");
  return MHD_OK;
}

// ---- single-problem API (slot 0)
int mhd_set_state(mhd_handle h, const float* sol) { return mhd_slot_set_state(h, 0, sol); }
int mhd_get_state(mhd_handle h, float* sol) { return mhd_slot_get_state(h, 0, sol); }
int mhd_set_physical(mhd_handle h, int field, const float* phys) { return mhd_slot_set_physical(h, 0, field, phys); }
int mhd_get_physical(mhd_handle h, int field, float* phys) { return mhd_slot_get_physical(h, 0, field, phys); }
int mhd_get_clock(mhd_handle h, double* t, long long* step, double* dt) { return mhd_slot_get_clock(h, 0, t, step, dt); }
int mhd_set_clock(mhd_handle h, double t, long long step, double dt) { return mhd_slot_set_clock(h, 0, t, step, dt); }
int mhd_diagnostics(mhd_handle h, double* out, int nout) { return mhd_slot_diagnostics(h, 0, out, nout); }

int mhd_step(mhd_handle h, int nsteps) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (nsteps < 0) return fail(MHD_ERR_INVALID, "nsteps must be >= 0");
  return h->run_steps(nsteps);
}

int mhd_compute_rhs(mhd_handle h, float* rhs_out) {
  int rc = check_slot(h, 0);
  if (rc) return rc;
  if (!rhs_out) return fail(MHD_ERR_INVALID, "null output");
  if ((rc = h->rhs(h->sol, h->acc, OP_RHS, 0.f, 0.f, 0.f, h->slot_ref(0), 7))) return rc;
  if ((rc = h->launch(KC_OTHER, [&] { scatter_state_kernel<<<1216, 256, 0, h->stream>>>(h->acc, h->ref, h->g, h->nfields()); }))) return rc;
  MHD_CUDA(cudaMemcpyAsync(rhs_out, h->ref, h->ref_elems() * sizeof(float2), cudaMemcpyDeviceToHost, h->stream));
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_synchronize(mhd_handle h) {
  int rc = check_handle(h);
  if (rc) return rc;
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return h->check_device_error();
}

int mhd_set_stream(mhd_handle h, void* stream) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return MHD_OK;
}

void* mhd_get_stream(mhd_handle h) { return h ? (void*)h->stream : nullptr; }

int mhd_memory_bytes(mhd_handle h, long long* bytes) {
  if (!h || !bytes) return fail(MHD_ERR_INVALID, "null argument");
  *bytes = footprint(h->g, h->cap, h->p.vp != 0, h->p.hydro_only != 0);
  return MHD_OK;
}

int mhd_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return fail(MHD_ERR_INVALID, "null output");
  *ptr = nullptr;
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) return fail(MHD_ERR_OOM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
  return MHD_OK;
}

int mhd_host_free(void* ptr) {
  if (!ptr) return MHD_OK;
  MHD_CUDA(cudaFreeHost(ptr));
  return MHD_OK;
}

int mhd_profile_enable(mhd_handle h, int enable) {
  int rc = check_handle(h);
  if (rc) return rc;
  if ((rc = h->fold_records())) return rc;
  if (enable) {
    for (int c = 0; c < KC_COUNT; ++c) { h->prof_launches[c] = 0; h->prof_ms[c] = 0; }
  }
  h->profiling = enable != 0;
  return MHD_OK;
}

int mhd_profile_read(mhd_handle h, long long* launches, double* ms, int nclass) {
  int rc = check_handle(h);
  if (rc) return rc;
  if ((rc = h->fold_records())) return rc;
  for (int c = 0; c < nclass && c < KC_COUNT; ++c) {
    if (launches) launches[c] = h->prof_launches[c];
    if (ms) ms[c] = h->prof_ms[c];
  }
  return MHD_OK;
}

const char* mhd_kernel_class_name(int cls) { return (cls >= 0 && cls < KC_COUNT) ? kClassNames[cls] : ""; }
int mhd_kernel_class_count(void) { return KC_COUNT; }

int mhd_kernel_class_bytes(mhd_handle h, int cls, double* bytes) {
  if (!h || !bytes) return fail(MHD_ERR_INVALID, "null argument");
  const double n = h->g.n, kx = h->g.kx, k2 = h->g.k2, c = 8.0;
  const double inst = (double)(h->active.empty() ? 1 : h->active.size());
  const double state_field = k2 * k2 * kx * c;
  double b = 0;
  // state arrays (6 fields each) one epilogue launch touches, averaged over the scheme's stages
  const double arrays = h->p.scheme == MHD_RK4 ? (3 + 5 + 5 + 4) / 4.0 : (3 + 4 * 4) / 5.0;
  // out-going planes (8 products, 14 with the VP penalty fields) and the VP mask / wall reads
  // the hydrodynamic form moves 3 fields in and 5 products out (6 product slots leave x_fused;
  // with VP 8 slots, the penalty fields in 5..7)
  const bool hd = h->hd_form();
  const bool vp = h->p.vp != 0;
  const double ns = hd ? (vp ? 8 : 5) : h->ns, nin = hd ? 3 : 6, xout = hd ? (vp ? 8 : 6) : ns;
  const double vpin = vp ? (h->ops->vp == 2 ? (hd ? 4.0 : 7.0) : 1.0) * n * n * n * 4.0 : 0.0;
  switch (cls) {
    case KC_ZINV: b = nin * (state_field + n * k2 * kx * c); break;
    case KC_YINV: b = nin * (n * k2 * kx * c + n * n * kx * c); break;
    case KC_XFUSED: b = (nin + xout) * n * n * kx * c + vpin; break;
    case KC_YFWD: b = ns * (n * n * kx * c + n * k2 * kx * c); break;
    case KC_ZFWD: b = ns * (n * k2 * kx * c + state_field) + 2 * 6 * k2 * k2 * c; break;  // + the kx = 0 Hermitian part
    case KC_RKEPI: b = ns * state_field + arrays * nin * state_field + nin * k2 * k2 * c; break;
    default: b = 0;
  }
  *bytes = b * inst;
  return MHD_OK;
}

int mhd_step_timed(mhd_handle h, int nsteps, double* ms_per_step) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (nsteps < 1 || !ms_per_step) return fail(MHD_ERR_INVALID, "nsteps >= 1 and a non-null output are required");
  if ((rc = h->sync_lists())) return rc;
  if (!h->profiling && (rc = h->build_graph())) return rc;
  std::vector<cudaEvent_t> ev(nsteps + 1);
  for (auto& e : ev) MHD_CUDA(cudaEventCreate(&e));
  cudaEventRecord(ev[0], h->stream);
  for (int i = 0; i < nsteps && rc == MHD_OK; ++i) {
    rc = h->run_steps(1);
    cudaEventRecord(ev[i + 1], h->stream);
  }
  cudaError_t e = cudaEventSynchronize(ev[nsteps]);
  for (int i = 0; i < nsteps; ++i) {
    float f = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&f, ev[i], ev[i + 1]);
    ms_per_step[i] = f;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("cudaEventSynchronize: ") + cudaGetErrorString(e));
  return MHD_OK;
}

int mhd_time_steps(mhd_handle h, int nsteps, double* ms) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!ms) return fail(MHD_ERR_INVALID, "null output");
  if ((rc = h->sync_lists())) return rc;
  if (!h->profiling && (rc = h->build_graph())) return rc;
  cudaEvent_t a, b;
  MHD_CUDA(cudaEventCreate(&a));
  MHD_CUDA(cudaEventCreate(&b));
  cudaEventRecord(a, h->stream);
  rc = h->run_steps(nsteps);
  cudaEventRecord(b, h->stream);
  cudaError_t e = cudaEventSynchronize(b);
  float f = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&f, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("cudaEventSynchronize: ") + cudaGetErrorString(e));
  *ms = f;
  return MHD_OK;
}

int mhd_autotune(mhd_handle h, int flags) {
  int rc = check_handle(h);
  if (rc) return rc;
  return h->autotune((flags & MHD_TUNE_FORCE) != 0, (flags & MHD_TUNE_NO_FILE) == 0);
}

int mhd_variant_count(mhd_handle h, int cls, int* count) {
  if (!h || !count) return fail(MHD_ERR_INVALID, "null argument");
  if (cls < 0 || cls >= kTunedClasses) return fail(MHD_ERR_INVALID, "class must be 0..4 (the FFT pass classes)");
  *count = h->ops->variant_count(cls);
  return MHD_OK;
}

int mhd_variant_name(mhd_handle h, int cls, int idx, char* buf, int len) {
  if (!h || !buf || len < 1) return fail(MHD_ERR_INVALID, "null argument");
  if (cls < 0 || cls >= kTunedClasses) return fail(MHD_ERR_INVALID, "class must be 0..4 (the FFT pass classes)");
  if (idx < 0) idx = h->ops->sel[cls];
  if (idx >= h->ops->variant_count(cls)) return fail(MHD_ERR_INVALID, "no such variant");
  const std::string name = h->ops->variant_name(cls, idx);
  std::snprintf(buf, (size_t)len, "%s", name.c_str());
  return MHD_OK;
}

int mhd_select_variant(mhd_handle h, int cls, int idx) {
  int rc = check_handle(h);
  if (rc) return rc;
  if ((rc = h->ops->select(cls, idx))) return rc;
  h->invalidate_graph();
  return MHD_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// Ensembles: several size classes stepped concurrently.  One step of every class is captured
// into a single CUDA graph: the classes fork onto their own streams and join on the first one,
// so small boxes run alongside large ones instead of one class after another.
// ------------------------------------------------------------------------------------------
struct mhd_ensemble_s {
  std::vector<mhd_handle> hs;
  std::vector<int> versions;
  cudaGraphExec_t graph = nullptr;
  std::vector<cudaEvent_t> evs;
  ~mhd_ensemble_s() {
    if (graph) cudaGraphExecDestroy(graph);
    for (auto e : evs) cudaEventDestroy(e);
  }
};

extern "C" {

int mhd_ensemble_create(mhd_handle* hs, int nh, mhd_ensemble* out) {
  if (!out || !hs || nh < 1) return fail(MHD_ERR_INVALID, "need >= 1 handles and an output");
  *out = nullptr;
  for (int i = 0; i < nh; ++i) {
    if (!hs[i]) return fail(MHD_ERR_INVALID, "null handle in ensemble");
    if (hs[i]->device != hs[0]->device) return fail(MHD_ERR_INVALID, "ensemble members must share a device");
    for (int j = 0; j < i; ++j) if (hs[j] == hs[i]) return fail(MHD_ERR_INVALID, "duplicate handle in ensemble");
  }
  std::unique_ptr<mhd_ensemble_s> e(new (std::nothrow) mhd_ensemble_s());
  if (!e) return fail(MHD_ERR_OOM, "host allocation failed");
  e->hs.assign(hs, hs + nh);
  *out = e.release();
  return MHD_OK;
}

int mhd_ensemble_destroy(mhd_ensemble e) {
  if (!e) return MHD_OK;
  delete e;
  return MHD_OK;
}

int mhd_ensemble_step(mhd_ensemble e, int nsteps) {
  if (!e) return fail(MHD_ERR_INVALID, "null ensemble");
  if (nsteps < 0) return fail(MHD_ERR_INVALID, "nsteps must be >= 0");
  mhd_handle h0 = e->hs[0];
  int rc = check_handle(h0);
  if (rc) return rc;
  for (auto h : e->hs) {
    if ((rc = h->sync_lists())) return rc;
    if (h->profiling) return fail(MHD_ERR_STATE, "ensemble steps do not run with per-kernel profiling enabled");
  }
  // the lists are uploaded on each member's stream: order them before the graph's first node
  for (size_t i = 1; i < e->hs.size(); ++i) {
    cudaEvent_t ev;
    MHD_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, e->hs[i]->stream);
    cudaStreamWaitEvent(h0->stream, ev, 0);
    cudaEventDestroy(ev);
  }
  {
    std::vector<int> v;
    for (auto h : e->hs) v.push_back(h->graph_version);
    if (e->graph && v != e->versions) {  // a member changed what one of its steps launches
      cudaGraphExecDestroy(e->graph);
      e->graph = nullptr;
    }
    e->versions = v;
  }
  if (!e->graph) {
    const size_t m = e->hs.size();
    e->evs.resize(m + 1);
    for (auto& ev : e->evs) MHD_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaGraph_t gr = nullptr;
    MHD_CUDA(cudaStreamBeginCapture(h0->stream, cudaStreamCaptureModeThreadLocal));
    cudaEventRecord(e->evs[m], h0->stream);
    for (size_t i = 0; i < m && rc == MHD_OK; ++i) {
      mhd_handle h = e->hs[i];
      if (i > 0) cudaStreamWaitEvent(h->stream, e->evs[m], 0);
      rc = h->issue_step();
      if (i > 0) {
        cudaEventRecord(e->evs[i], h->stream);
        cudaStreamWaitEvent(h0->stream, e->evs[i], 0);
      }
    }
    cudaError_t err = cudaStreamEndCapture(h0->stream, &gr);
    if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
    if (err != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("ensemble capture: ") + cudaGetErrorString(err));
    err = cudaGraphInstantiate(&e->graph, gr, 0);
    cudaGraphDestroy(gr);
    if (err != cudaSuccess) { e->graph = nullptr; return fail(MHD_ERR_CUDA, std::string("ensemble instantiate: ") + cudaGetErrorString(err)); }
  }
  for (int s = 0; s < nsteps; ++s) {
    MHD_CUDA(cudaGraphLaunch(e->graph, h0->stream));
    for (auto h : e->hs) h->advance_clocks();
  }
  // later work on any member's own stream follows the ensemble's steps
  for (size_t i = 1; i < e->hs.size(); ++i) {
    cudaEvent_t ev;
    MHD_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, h0->stream);
    cudaStreamWaitEvent(e->hs[i]->stream, ev, 0);
    cudaEventDestroy(ev);
  }
  return MHD_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// Allocation-free diagnostics.
//
// Some callers of this code cannot call cudaMalloc.  A Julia program whose CuArrays come from
// CUDA.jl's memory pool, or a Python program whose tensors come from PyTorch's caching
// allocator, hands the library device pointers but expects all device memory to go through
// that pool: a raw cudaMalloc behind the pool's back can fail once the pool has reserved the
// free memory, and it makes the process's memory use invisible to the pool's accounting.
// Real-time loops that must not block on the allocator, and code running where the driver
// forbids allocation, are in the same position.  mhd_diagnostics_noalloc serves them: it reads
// a caller-owned device copy of prob.sol, writes six doubles to caller-owned device memory, and
// the only scratch it uses is the fixed array below, compiled into the library.
// ------------------------------------------------------------------------------------------
namespace {

// Per-block partial sums of the reduction: at most kNoAllocBlocks blocks x kDiagSlots doubles
// (1216 x 6 x 8 B = 58,368 bytes).  Every GPU that loads the library holds it until the process
// exits.  Each call overwrites the partials it uses before reading them, so nothing has to be
// zeroed between calls, but all calls share this one array: calls whose kernels overlap on the
// GPU (two streams, or two host threads) race on it and must be serialised by the caller.
constexpr int kNoAllocBlocks = 1216;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocBlocks * kDiagSlots];

// Device address of g_noalloc_partials, looked up once per CUDA context.  A __device__ variable
// has its own address in every context that loads the module (a caller's own context on a
// device as well as the device's primary context, and a new one after cudaDeviceReset), so the
// cache is keyed by the unique id of the context current at the call (cuCtxGetId: never reused
// within a process, unlike a context handle), not by the device ordinal.
std::mutex g_noalloc_mtx;
std::map<unsigned long long, double*> g_noalloc_ptr;

// Driver entry points through the runtime (the library does not link libcuda).
template <class F>
F driver_fn(const char* name, int version) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, version, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return reinterpret_cast<F>(p);
}

// Id of the context current on this thread; 0 if there is none or the query fails.
unsigned long long current_ctx_id() {
  static const auto get_ctx = driver_fn<PFN_cuCtxGetCurrent_v4000>("cuCtxGetCurrent", 4000);
  static const auto get_id = driver_fn<PFN_cuCtxGetId_v12000>("cuCtxGetId", 12000);
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_ctx || !get_id || get_ctx(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Partial sums over a reference-layout half spectrum sol[f][kz][ky][kx] (nkr = n/2+1 fastest),
// restricted to the retained band, with the weights and sums of diag_partial_kernel.
__global__ void __launch_bounds__(kDiagThreads) diag_partial_ref_kernel(const float2* __restrict__ sol, Geom geo,
                                                                        double* partial) {
  const int nkr = geo.n / 2 + 1;
  const long long plane = (long long)geo.n * geo.n * nkr;  // one field
  double acc[kDiagSlots] = {0, 0, 0, 0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < plane; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nkr);
    if (x >= geo.kx) continue;
    const long long r = i / nkr;
    const int fy = (int)(r % geo.n);
    const int fz = (int)(r / geo.n);
    const int jy = kept_of_freq(geo, fy), jz = kept_of_freq(geo, fz);
    if (jy < 0 || jz < 0) continue;
    const double w = x == 0 ? 1.0 : 2.0;
    const double kx = (double)geo.kscale * x;
    const double ky = (double)geo.kscale * signed_of_kept(geo, jy);
    const double kz = (double)geo.kscale * signed_of_kept(geo, jz);
    double2 ku = make_double2(0, 0), kb = make_double2(0, 0);
    double eu = 0, eb = 0, hc = 0;
    bool bad = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 u = sol[c * plane + i], b = sol[(c + 3) * plane + i];
      bad |= !isfinite(u.x) || !isfinite(u.y) || !isfinite(b.x) || !isfinite(b.y);
      eu += (double)u.x * u.x + (double)u.y * u.y;
      eb += (double)b.x * b.x + (double)b.y * b.y;
      hc += (double)u.x * b.x + (double)u.y * b.y;
      const double kc = c == 0 ? kx : (c == 1 ? ky : kz);
      ku.x += kc * u.x; ku.y += kc * u.y;
      kb.x += kc * b.x; kb.y += kc * b.y;
    }
    acc[0] += w * eu;
    acc[1] += w * eb;
    acc[2] += w * hc;
    acc[3] = fmax(acc[3], sqrt(ku.x * ku.x + ku.y * ku.y));
    acc[4] = fmax(acc[4], sqrt(kb.x * kb.x + kb.y * kb.y));
    acc[5] += bad ? 1.0 : 0.0;
  }
  block_reduce_diag(acc, partial + (long long)blockIdx.x * kDiagSlots);
}

// Reduce the partials in block order and scale the three sums by dV / n^3 into out[0..6).
__global__ void __launch_bounds__(kDiagThreads) diag_final_scaled_kernel(const double* __restrict__ partial, int nblocks,
                                                                         double scale, double* out) {
  __shared__ double res[kDiagSlots];
  double acc[kDiagSlots] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
    for (int s = 0; s < kDiagSlots; ++s) {
      const double x = partial[b * kDiagSlots + s];
      acc[s] = (s == 3 || s == 4) ? fmax(acc[s], x) : acc[s] + x;
    }
  }
  block_reduce_diag(acc, res);
  __syncthreads();
  if (threadIdx.x < kDiagSlots) out[threadIdx.x] = threadIdx.x < 3 ? res[threadIdx.x] * scale : res[threadIdx.x];
}

}  // namespace

extern "C" int mhd_diagnostics_noalloc(const float* sol_dev, int n, double L, double* out_dev, void* stream) {
  if (!sol_dev || !out_dev) return fail(MHD_ERR_INVALID, "sol_dev and out_dev must be device pointers");
  if (!supported(n)) {
    return fail(MHD_ERR_INVALID, "n=" + std::to_string(n) + " is beyond what this entry point handles (n in 16,32,48,64,96,128,256,512)");
  }
  if (!(L > 0) || !std::isfinite(L)) return fail(MHD_ERR_INVALID, "box size L must be positive");
  {
    // an error left by earlier work on this thread is reported as such, not blamed on the
    // launches below (their check would otherwise return and clear it)
    const cudaError_t pre = cudaGetLastError();
    if (pre != cudaSuccess)
      return fail(MHD_ERR_CUDA, std::string("a CUDA error was pending before mhd_diagnostics_noalloc: ") + cudaGetErrorString(pre));
  }
  double* partials = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mtx);
    unsigned long long ctx = current_ctx_id();
    auto it = ctx ? g_noalloc_ptr.find(ctx) : g_noalloc_ptr.end();
    if (it == g_noalloc_ptr.end()) {
      // first call in this context: resolve the scratch array's device address here.  With no
      // context current yet, this runtime call makes the current device's primary context
      // current, and the address belongs to that context.
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_partials): ") + cudaGetErrorString(e));
      if (!ctx) ctx = current_ctx_id();
      if (!ctx) return fail(MHD_ERR_CUDA, "no current CUDA context (cuCtxGetCurrent / cuCtxGetId)");
      it = g_noalloc_ptr.emplace(ctx, static_cast<double*>(p)).first;
    }
    partials = it->second;
  }
  const Geom g = make_geom(n, L);
  const long long plane = (long long)n * n * (n / 2 + 1);
  long long blocks = (plane + kDiagThreads - 1) / kDiagThreads;
  if (blocks > kNoAllocBlocks) blocks = kNoAllocBlocks;  // grid-stride loop covers the rest
  if (blocks < 1 || blocks > kNoAllocBlocks) return fail(MHD_ERR_INVALID, "reduction needs more partial sums than the scratch holds");
  cudaStream_t s = (cudaStream_t)stream;
  const double dx = L / n;
  const double scale = dx * dx * dx / ((double)n * n * n);
  diag_partial_ref_kernel<<<(unsigned)blocks, kDiagThreads, 0, s>>>(reinterpret_cast<const float2*>(sol_dev), g, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("diag_partial_ref_kernel launch: ") + cudaGetErrorString(e));
  diag_final_scaled_kernel<<<1, kDiagThreads, 0, s>>>(partials, (int)blocks, scale, out_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("diag_final_scaled_kernel launch: ") + cudaGetErrorString(e));
  return MHD_OK;
}
