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

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/mhdgb.h"
#include "passes.cuh"

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

// ------------------------------------------------------------------------------------------
// Per-size plans: column passes (y, z) and x rows.
// ------------------------------------------------------------------------------------------
template <int N>
struct Cfg;
template <> struct Cfg<16>  { using C = Plan<16, 4, 4, 4>;       using R = Plan<16, 4, 4, 4>;       static constexpr int TX = 16, TXE = 16, ROWS = 32; };
template <> struct Cfg<32>  { using C = Plan<32, 4, 8, 4>;       using R = Plan<32, 4, 8, 4>;       static constexpr int TX = 16, TXE = 16, ROWS = 32; };
template <> struct Cfg<48>  { using C = Plan<48, 4, 12, 4>;      using R = Plan<48, 4, 12, 4>;      static constexpr int TX = 16, TXE = 16, ROWS = 32; };
template <> struct Cfg<64>  { using C = Plan<64, 8, 8, 8>;       using R = Plan<64, 8, 8, 8>;       static constexpr int TX = 16, TXE = 16, ROWS = 16; };
template <> struct Cfg<96>  { using C = Plan<96, 8, 12, 4, 2>;   using R = Plan<96, 8, 12, 4, 2>;   static constexpr int TX = 16, TXE = 16, ROWS = 16; };
template <> struct Cfg<128> { using C = Plan<128, 8, 16, 8>;     using R = Plan<128, 16, 8, 4, 4>;  static constexpr int TX = 16, TXE = 16, ROWS = 8; };
template <> struct Cfg<256> { using C = Plan<256, 16, 16, 16>;   using R = Plan<256, 32, 8, 8, 4>;  static constexpr int TX = 16, TXE = 16, ROWS = 4; };
template <> struct Cfg<512> { using C = Plan<512, 32, 16, 8, 4>; using R = Plan<512, 64, 8, 8, 8>;  static constexpr int TX = 8, TXE = 8, ROWS = 2; };

constexpr int kSlots = 8;

struct OpsBase {
  virtual ~OpsBase() {}
  virtual int setup(const Geom& g) = 0;
  virtual void col_inv(const ColArgs& a, const Geom& g, int outer, int nf, cudaStream_t s) = 0;
  virtual void col_fwd(const ColArgs& a, const Geom& g, int outer, int nf, cudaStream_t s) = 0;
  virtual void x_fused(float2* buf, const Geom& g, long long rowstride, long long slot, cudaStream_t s) = 0;
  virtual void x_c2r(const float2* src, float* dst, const Geom& g, long long srow, float scale, cudaStream_t s) = 0;
  virtual void x_r2c(const float* src, float2* dst, const Geom& g, long long drow, cudaStream_t s) = 0;
};

// Host construction of a plan's stage-twiddle table (PlanTw layout), in double precision.
template <class P>
void plan_twiddles(std::vector<float2>& out) {
  constexpr int N = P::N, R0 = P::R0, R1 = P::R1, R2 = P::R2;
  out.assign(PlanTw<P>::SIZE, make_float2(1.f, 0.f));
  auto w = [](long long j) {
    const double ang = 2.0 * M_PI * (double)(j % N) / (double)N;
    return make_float2((float)std::cos(ang), (float)std::sin(ang));
  };
  for (int n1 = 0; n1 < R1; ++n1)
    for (int k0 = 0; k0 < R0; ++k0) out[n1 * R0 + k0] = w((long long)((n1 * k0) % (R0 * R1)) * R2);
  if (R2 > 1)
    for (int k1 = 0; k1 < R1; ++k1)
      for (int n2 = 0; n2 < R2; ++n2)
        for (int k0 = 0; k0 < R0; ++k0) out[R0 * R1 + k1 * (R0 * R2) + k0 + R0 * n2] = w((long long)n2 * (k0 + R0 * k1));
}

template <class K>
int set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
  }
  return MHD_OK;
}

// Resident CTAs of a kernel on the whole device (persistent grid size).
template <class K>
int resident_ctas(K kernel, int threads, size_t smem, int* out) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("occupancy query: ") + cudaGetErrorString(e));
  *out = (per < 1 ? 1 : per) * sms;
  return MHD_OK;
}

template <int N>
struct Ops : OpsBase {
  using C = typename Cfg<N>::C;
  using R = typename Cfg<N>::R;
  using RR = typename Reverse<R>::type;
  using XC = XCfg<R>;
  static constexpr int TX = Cfg<N>::TX;
  static constexpr int GROUPS = XC::TPG >= 64 ? 2 : 4;  // x row groups per CTA (128 threads)
  static constexpr size_t kColSmem = sizeof(float2) * 2 * N * TX;
  static constexpr size_t kRowSmem = sizeof(float2) * RowCfg<R>::TS;
  size_t x_smem = 0;
  int col_inv_ctas = 0, col_fwd_ctas = 0, x_ctas = 0;
  float2* tw_all = nullptr;
  const float2 *twC = nullptr, *twR = nullptr, *twRR = nullptr;

  ~Ops() override {
    if (tw_all) cudaFree(tw_all);
  }

  int setup(const Geom& g) override {
    int rc = MHD_OK;
    std::vector<float2> tc, tr, trr;
    plan_twiddles<C>(tc);
    plan_twiddles<R>(tr);
    plan_twiddles<RR>(trr);
    std::vector<float2> all(tc);
    all.insert(all.end(), tr.begin(), tr.end());
    all.insert(all.end(), trr.begin(), trr.end());
    MHD_CUDA(cudaMalloc(&tw_all, all.size() * sizeof(float2)));
    MHD_CUDA(cudaMemcpy(tw_all, all.data(), all.size() * sizeof(float2), cudaMemcpyHostToDevice));
    twC = tw_all;
    twR = tw_all + tc.size();
    twRR = twR + tr.size();
    x_smem = sizeof(float2) * (size_t)GROUPS * XC::group_words(g.kxp);
    if ((rc = set_smem(col_pass_kernel<C, TX, +1, true, false>, kColSmem))) return rc;
    if ((rc = set_smem(col_pass_kernel<C, TX, -1, false, true>, kColSmem))) return rc;
    if ((rc = set_smem(x_fused_kernel<R, GROUPS>, x_smem))) return rc;
    if ((rc = set_smem(x_c2r_kernel<R, Cfg<N>::ROWS>, kRowSmem * Cfg<N>::ROWS))) return rc;
    if ((rc = set_smem(x_r2c_kernel<R, Cfg<N>::ROWS>, kRowSmem * Cfg<N>::ROWS))) return rc;
    if ((rc = resident_ctas(col_pass_kernel<C, TX, +1, true, false>, TX * C::G, kColSmem, &col_inv_ctas))) return rc;
    if ((rc = resident_ctas(col_pass_kernel<C, TX, -1, false, true>, TX * C::G, kColSmem, &col_fwd_ctas))) return rc;
    if ((rc = resident_ctas(x_fused_kernel<R, GROUPS>, GROUPS * XC::TPG, x_smem, &x_ctas))) return rc;
    return MHD_OK;
  }
  void col_inv(const ColArgs& a, const Geom& g, int outer, int nf, cudaStream_t s) override {
    ColWork w{(g.kx + TX - 1) / TX, outer, nf, g.k2};
    const int total = w.tiles_x * w.outer * w.nf;
    col_pass_kernel<C, TX, +1, true, false><<<total < col_inv_ctas ? total : col_inv_ctas, TX * C::G, kColSmem, s>>>(a, g, w, twC);
  }
  void col_fwd(const ColArgs& a, const Geom& g, int outer, int nf, cudaStream_t s) override {
    ColWork w{(g.kx + TX - 1) / TX, outer, nf, N};
    const int total = w.tiles_x * w.outer * w.nf;
    col_pass_kernel<C, TX, -1, false, true><<<total < col_fwd_ctas ? total : col_fwd_ctas, TX * C::G, kColSmem, s>>>(a, g, w, twC);
  }
  void x_fused(float2* buf, const Geom& g, long long rowstride, long long slot, cudaStream_t s) override {
    const long long groups = (long long)N * N / XC::RPG;
    const long long need = (groups + GROUPS - 1) / GROUPS;
    const int grid = (int)(need < x_ctas ? need : x_ctas);
    x_fused_kernel<R, GROUPS><<<grid, GROUPS * XC::TPG, x_smem, s>>>(buf, g, rowstride, slot, twR, twRR);
  }
  void x_c2r(const float2* src, float* dst, const Geom& g, long long srow, float scale, cudaStream_t s) override {
    constexpr int ROWS = Cfg<N>::ROWS;
    const long long pairs = (long long)N * N / 2;
    x_c2r_kernel<R, ROWS><<<(unsigned)(pairs / ROWS), ROWS * R::G, kRowSmem * ROWS, s>>>(src, dst, g, srow, scale, twR);
  }
  void x_r2c(const float* src, float2* dst, const Geom& g, long long drow, cudaStream_t s) override {
    constexpr int ROWS = Cfg<N>::ROWS;
    const long long pairs = (long long)N * N / 2;
    x_r2c_kernel<R, ROWS><<<(unsigned)(pairs / ROWS), ROWS * R::G, kRowSmem * ROWS, s>>>(src, dst, g, drow, twR);
  }
};

OpsBase* make_ops(int n) {
  switch (n) {
    case 16: return new Ops<16>();
    case 32: return new Ops<32>();
    case 48: return new Ops<48>();
    case 64: return new Ops<64>();
    case 96: return new Ops<96>();
    case 128: return new Ops<128>();
    case 256: return new Ops<256>();
    case 512: return new Ops<512>();
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

// Kernel classes for per-launch timing.
enum KClass { KC_ZINV = 0, KC_YINV, KC_XFUSED, KC_YFWD, KC_ZFWD, KC_RKEPI, KC_HERM, KC_OTHER, KC_COUNT };
const char* kClassNames[KC_COUNT] = {"z_inverse", "y_inverse", "x_fused", "y_forward", "z_forward", "rk_epilogue",
                                     "herm_kx0", "other"};

const double kLsA[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                        -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
const double kLsB[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                        1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                        2277821191437.0 / 14882151754819.0};

struct Sizes {
  long long fs;      // one compact field (complex)
  long long state;   // six fields
  long long colbuf;  // colbuf complex elements
  long long rowbuf;  // rowbuf complex elements
  long long ref;     // reference-layout sol (complex)
  long long phys;    // one physical field (floats)
  int diag_blocks;
};

Sizes sizes_of(const Geom& g) {
  Sizes s;
  s.fs = (long long)g.k2 * g.k2 * g.kxp;
  s.state = 6 * s.fs;
  s.colbuf = (long long)g.n * g.k2 * kSlots * g.kxp;
  s.rowbuf = (long long)g.n * g.n * kSlots * g.kxp;
  s.ref = 6LL * (g.n / 2 + 1) * g.n * g.n;
  s.phys = (long long)g.n * g.n * g.n;
  long long b = (s.fs + kDiagThreads - 1) / kDiagThreads;
  s.diag_blocks = (int)(b < 1216 ? b : 1216);
  return s;
}

long long footprint(const Geom& g) {
  Sizes s = sizes_of(g);
  long long bytes = 0;
  bytes += 3 * s.state * 8;          // sol, stage state, accumulator
  bytes += s.fs * 8;                 // aux (div B spectrum)
  bytes += s.colbuf * 8 + s.rowbuf * 8;
  bytes += s.ref * 8;                // reference-layout staging
  bytes += s.phys * 4;               // physical staging
  bytes += 6LL * g.n * 8;            // stage twiddle tables
  bytes += (long long)s.diag_blocks * kDiagSlots * 8 + 16 * 8 + 64;
  return bytes;
}

}  // namespace

struct mhd_problem {
  mhd_params p{};
  Geom g{};
  Sizes sz{};
  std::unique_ptr<OpsBase> ops;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  float2* sol = nullptr;
  float2* xs = nullptr;
  float2* acc = nullptr;
  float2* aux = nullptr;
  float2* colbuf = nullptr;
  float2* rowbuf = nullptr;
  float2* ref = nullptr;
  float* phys = nullptr;
  double* diag_partial = nullptr;
  double* diag_out = nullptr;
  unsigned int* maxabs = nullptr;
  double t = 0.0;
  long long step = 0;
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
    for (auto& r : recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    recs.clear();
    for (auto e : pool) cudaEventDestroy(e);
    pool.clear();
    void* ptrs[] = {sol, xs, acc, aux, colbuf, rowbuf, ref, phys, diag_partial, diag_out, maxabs};
    for (void* q : ptrs) if (q) cudaFree(q);
    sol = xs = acc = aux = colbuf = rowbuf = ref = nullptr;
    phys = nullptr; diag_partial = nullptr; diag_out = nullptr; maxabs = nullptr;
    if (own_stream) cudaStreamDestroy(own_stream);
    own_stream = nullptr;
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
  long long AZ() const { return (long long)g.k2 * kSlots * g.kxp; }
  long long BZ() const { return (long long)g.n * kSlots * g.kxp; }
  long long SLK() const { return (long long)kSlots * g.kxp; }

  // state (nf fields starting at src) -> colbuf slots 0..nf-1
  int z_inverse(const float2* src, int nf) {
    ColArgs a{src, colbuf, FS(), (long long)g.kxp, (long long)g.k2 * g.kxp, (long long)g.kxp, SLK(), AZ()};
    return launch(KC_ZINV, [&] { ops->col_inv(a, g, g.k2, nf, stream); });
  }
  int y_inverse(int nf) {
    ColArgs a{colbuf, rowbuf, (long long)g.kxp, AZ(), SLK(), (long long)g.kxp, BZ(), SLK()};
    return launch(KC_YINV, [&] { ops->col_inv(a, g, g.n, nf, stream); });
  }
  int x_fused() {
    // the six field rows of a physical row are contiguous (slot stride == kxp)
    return launch(KC_XFUSED, [&] { ops->x_fused(rowbuf, g, SLK(), g.kxp, stream); });
  }
  int y_forward(int nf) {
    ColArgs a{rowbuf, colbuf, (long long)g.kxp, BZ(), SLK(), (long long)g.kxp, AZ(), SLK()};
    return launch(KC_YFWD, [&] { ops->col_fwd(a, g, g.n, nf, stream); });
  }
  // colbuf slots -> compact planes (nf fields/products) of dst, pruned output
  int z_forward(float2* dst, int nf) {
    ColArgs a{colbuf, dst, (long long)g.kxp, SLK(), AZ(), FS(), (long long)g.kxp, (long long)g.k2 * g.kxp};
    return launch(KC_ZFWD, [&] { ops->col_fwd(a, g, g.k2, nf, stream); });
  }
  // Stage epilogue: RHS from the 8 compact product planes (in rowbuf) and the stage state X.
  int epilogue(const float2* X, int op, float h, float ca, float cb) {
    int rc = launch(KC_HERM, [&] {
      const int total = 6 * g.k2 * g.k2;
      herm_kx0_kernel<<<(total + 255) / 256, 256, 0, stream>>>(X, aux, g, FS());
    });
    if (rc) return rc;
    RkArgs a{};
    a.prod = rowbuf;
    a.X = X;
    a.H = aux;
    a.sol = sol;
    a.acc = acc;
    a.xn = (op == OP_LS_FIRST || op == OP_LS) ? sol : xs;
    a.fs = FS();
    a.nu = (float)p.nu;
    a.eta = (float)p.eta;
    a.h = h;
    a.dt = (float)p.dt;
    a.ca = ca;
    a.cb = cb;
    a.op = op;
    const double n3 = (double)g.n * g.n * g.n;
    a.pscale = (float)(1.0 / (n3 * n3));
    const int bx = g.kx <= 256 ? (g.kx + 31) / 32 * 32 : 256;
    const dim3 grid((g.kx + bx - 1) / bx, g.k2, g.k2);
    return launch(KC_RKEPI, [&] {
      switch (op) {
        case OP_RHS: rk_epilogue_kernel<OP_RHS><<<grid, bx, 0, stream>>>(a, g); break;
        case OP_RK4_FIRST: rk_epilogue_kernel<OP_RK4_FIRST><<<grid, bx, 0, stream>>>(a, g); break;
        case OP_RK4_MID: rk_epilogue_kernel<OP_RK4_MID><<<grid, bx, 0, stream>>>(a, g); break;
        case OP_RK4_LAST: rk_epilogue_kernel<OP_RK4_LAST><<<grid, bx, 0, stream>>>(a, g); break;
        case OP_LS_FIRST: rk_epilogue_kernel<OP_LS_FIRST><<<grid, bx, 0, stream>>>(a, g); break;
        default: rk_epilogue_kernel<OP_LS><<<grid, bx, 0, stream>>>(a, g); break;
      }
    });
  }
  int epilogues(const float2* X, int op, float h, float ca, float cb) {
    int rc;
    if ((rc = z_forward(rowbuf, kSlots))) return rc;
    return epilogue(X, op, h, ca, cb);
  }
  int rhs_passes(const float2* X) {
    int rc;
    if ((rc = z_inverse(X, 6))) return rc;
    if ((rc = y_inverse(6))) return rc;
    if ((rc = x_fused())) return rc;
    if ((rc = y_forward(kSlots))) return rc;
    return MHD_OK;
  }
  int step_rk4() {
    const float dtf = (float)p.dt;
    const float half = dtf / 2.0f;
    int rc;
    if ((rc = rhs_passes(sol))) return rc;
    if ((rc = epilogues(sol, OP_RK4_FIRST, half, 0.f, 0.f))) return rc;
    if ((rc = rhs_passes(xs))) return rc;
    if ((rc = epilogues(xs, OP_RK4_MID, half, 0.f, 0.f))) return rc;
    if ((rc = rhs_passes(xs))) return rc;
    if ((rc = epilogues(xs, OP_RK4_MID, dtf, 0.f, 0.f))) return rc;
    if ((rc = rhs_passes(xs))) return rc;
    if ((rc = epilogues(xs, OP_RK4_LAST, 0.f, 0.f, 0.f))) return rc;
    return MHD_OK;
  }
  int step_lsrk4() {
    int rc;
    for (int i = 0; i < 5; ++i) {
      if ((rc = rhs_passes(sol))) return rc;
      if ((rc = epilogues(sol, i == 0 ? OP_LS_FIRST : OP_LS, 0.f, (float)kLsA[i], (float)kLsB[i]))) return rc;
    }
    return MHD_OK;
  }
  // One field: compact (src, field slot) -> physical staging (normalised inverse).
  int inverse_field(const float2* src) {
    int rc;
    if ((rc = z_inverse(src, 1))) return rc;
    if ((rc = y_inverse(1))) return rc;
    return launch(KC_OTHER, [&] { ops->x_c2r(rowbuf, phys, g, SLK(), (float)(1.0 / ((double)g.n * g.n * g.n)), stream); });
  }
  // One field: physical staging -> compact dst (unnormalised forward).
  int forward_field(float2* dst) {
    int rc;
    if ((rc = launch(KC_OTHER, [&] { ops->x_r2c(phys, rowbuf, g, SLK(), stream); }))) return rc;
    if ((rc = y_forward(1))) return rc;
    return z_forward(dst, 1);
  }
};

namespace {

int check_handle(mhd_handle h) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return fail(MHD_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  return MHD_OK;
}

int validate(const mhd_params* p) {
  if (!p) return fail(MHD_ERR_INVALID, "null params");
  if (!supported(p->n)) return fail(MHD_ERR_INVALID, "unsupported grid size n=" + std::to_string(p->n) + " (supported: 16,32,48,64,96,128,256,512)");
  if (!(p->L > 0) || !std::isfinite(p->L)) return fail(MHD_ERR_INVALID, "box size L must be positive");
  if (!(p->nu >= 0) || !(p->eta >= 0)) return fail(MHD_ERR_INVALID, "nu and eta must be non-negative");
  if (p->nnu > 1 || p->neta > 1) return fail(MHD_ERR_INVALID, "hyper-diffusion (nnu > 1 or neta > 1) is not on this path");
  if (!std::isfinite(p->dt)) return fail(MHD_ERR_INVALID, "dt must be finite");
  if (p->scheme != MHD_RK4 && p->scheme != MHD_LSRK4) return fail(MHD_ERR_INVALID, "scheme must be MHD_RK4 or MHD_LSRK4");
  if (p->precision != MHD_PREC_FP32) return fail(MHD_ERR_INVALID, "only MHD_PREC_FP32 is available");
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
  *bytes = footprint(make_geom(params->n, params->L));
  return MHD_OK;
}

int mhd_create(const mhd_params* params, mhd_handle* out) {
  g_err.clear();
  if (!out) return fail(MHD_ERR_INVALID, "null output handle");
  *out = nullptr;
  int rc = validate(params);
  if (rc) return rc;
  std::unique_ptr<mhd_problem> h(new (std::nothrow) mhd_problem());
  if (!h) return fail(MHD_ERR_OOM, "host allocation failed");
  h->p = *params;
  h->device = params->device;
  MHD_CUDA(cudaSetDevice(h->device));
  h->g = make_geom(params->n, params->L);
  h->sz = sizes_of(h->g);
  h->ops.reset(make_ops(params->n));
  if (!h->ops) return fail(MHD_ERR_INVALID, "no plan for n");
  if ((rc = h->ops->setup(h->g))) return rc;
  MHD_CUDA(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
  h->stream = h->own_stream;
  const Sizes& s = h->sz;
  MHD_CUDA(cudaMalloc(&h->sol, s.state * sizeof(float2)));
  MHD_CUDA(cudaMalloc(&h->xs, s.state * sizeof(float2)));
  MHD_CUDA(cudaMalloc(&h->acc, s.state * sizeof(float2)));
  MHD_CUDA(cudaMalloc(&h->aux, s.fs * sizeof(float2)));
  MHD_CUDA(cudaMalloc(&h->colbuf, s.colbuf * sizeof(float2)));
  MHD_CUDA(cudaMalloc(&h->rowbuf, s.rowbuf * sizeof(float2)));
  MHD_CUDA(cudaMalloc(&h->ref, s.ref * sizeof(float2)));
  MHD_CUDA(cudaMalloc(&h->phys, s.phys * sizeof(float)));
  MHD_CUDA(cudaMalloc(&h->diag_partial, (size_t)s.diag_blocks * kDiagSlots * sizeof(double)));
  MHD_CUDA(cudaMalloc(&h->diag_out, 16 * sizeof(double)));
  MHD_CUDA(cudaMalloc(&h->maxabs, 16 * sizeof(unsigned int)));
  MHD_CUDA(cudaMemsetAsync(h->sol, 0, s.state * sizeof(float2), h->stream));
  MHD_CUDA(cudaMemsetAsync(h->xs, 0, s.state * sizeof(float2), h->stream));
  MHD_CUDA(cudaMemsetAsync(h->acc, 0, s.state * sizeof(float2), h->stream));
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  *out = h.release();
  return MHD_OK;
}

int mhd_destroy(mhd_handle h) {
  if (!h) return MHD_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  delete h;
  return MHD_OK;
}

int mhd_set_state(mhd_handle h, const float* sol) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!sol) return fail(MHD_ERR_INVALID, "null sol");
  MHD_CUDA(cudaMemcpyAsync(h->ref, sol, h->sz.ref * sizeof(float2), cudaMemcpyHostToDevice, h->stream));
  if ((rc = h->launch(KC_OTHER, [&] { gather_state_kernel<<<1216, 256, 0, h->stream>>>(h->ref, h->sol, h->g, 6); }))) return rc;
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_get_state(mhd_handle h, float* sol) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!sol) return fail(MHD_ERR_INVALID, "null sol");
  if ((rc = h->launch(KC_OTHER, [&] { scatter_state_kernel<<<1216, 256, 0, h->stream>>>(h->sol, h->ref, h->g, 6); }))) return rc;
  MHD_CUDA(cudaMemcpyAsync(sol, h->ref, h->sz.ref * sizeof(float2), cudaMemcpyDeviceToHost, h->stream));
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_set_physical(mhd_handle h, int field, const float* phys) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (field < 0 || field > 5) return fail(MHD_ERR_INVALID, "field must be 0..5 (ux uy uz bx by bz)");
  if (!phys) return fail(MHD_ERR_INVALID, "null field array");
  MHD_CUDA(cudaMemcpyAsync(h->phys, phys, h->sz.phys * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  if ((rc = h->forward_field(h->sol + field * h->sz.fs))) return rc;
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_get_physical(mhd_handle h, int field, float* phys) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (field < 0 || field > 5) return fail(MHD_ERR_INVALID, "field must be 0..5 (ux uy uz bx by bz)");
  if (!phys) return fail(MHD_ERR_INVALID, "null field array");
  if ((rc = h->inverse_field(h->sol + field * h->sz.fs))) return rc;
  MHD_CUDA(cudaMemcpyAsync(phys, h->phys, h->sz.phys * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_step(mhd_handle h, int nsteps) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (nsteps < 0) return fail(MHD_ERR_INVALID, "nsteps must be >= 0");
  for (int i = 0; i < nsteps; ++i) {
    rc = h->p.scheme == MHD_RK4 ? h->step_rk4() : h->step_lsrk4();
    if (rc) return rc;
    h->t += h->p.dt;
    h->step += 1;
  }
  return MHD_OK;
}

int mhd_compute_rhs(mhd_handle h, float* rhs_out) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!rhs_out) return fail(MHD_ERR_INVALID, "null output");
  if ((rc = h->rhs_passes(h->sol))) return rc;
  if ((rc = h->epilogues(h->sol, OP_RHS, 0.f, 0.f, 0.f))) return rc;
  if ((rc = h->launch(KC_OTHER, [&] { scatter_state_kernel<<<1216, 256, 0, h->stream>>>(h->acc, h->ref, h->g, 6); }))) return rc;
  MHD_CUDA(cudaMemcpyAsync(rhs_out, h->ref, h->sz.ref * sizeof(float2), cudaMemcpyDeviceToHost, h->stream));
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_get_clock(mhd_handle h, double* t, long long* step, double* dt) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  if (t) *t = h->t;
  if (step) *step = h->step;
  if (dt) *dt = h->p.dt;
  return MHD_OK;
}

int mhd_set_clock(mhd_handle h, double t, long long step, double dt) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  if (!std::isfinite(t) || !std::isfinite(dt)) return fail(MHD_ERR_INVALID, "t and dt must be finite");
  h->t = t;
  h->step = step;
  h->p.dt = dt;
  return MHD_OK;
}

int mhd_diagnostics(mhd_handle h, double* out, int nout) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (!out || nout < 8) return fail(MHD_ERR_INVALID, "diagnostics needs an output array of >= 8 doubles");
  const Sizes& s = h->sz;
  if ((rc = h->launch(KC_OTHER, [&] { diag_partial_kernel<<<s.diag_blocks, kDiagThreads, 0, h->stream>>>(h->sol, h->g, h->diag_partial); }))) return rc;
  if ((rc = h->launch(KC_OTHER, [&] { diag_final_kernel<<<1, kDiagThreads, 0, h->stream>>>(h->diag_partial, s.diag_blocks, h->diag_out); }))) return rc;
  if ((rc = h->launch(KC_OTHER, [&] { divb_spectrum_kernel<<<1216, 256, 0, h->stream>>>(h->sol, h->aux, h->g); }))) return rc;
  if ((rc = h->inverse_field(h->aux))) return rc;
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
  out[7] = h->t;
  if (d[5] > 0 || !std::isfinite(out[0]) || !std::isfinite(out[1])) return fail(MHD_ERR_NONFINITE, "detected NaN! Quit the simulation right now.");
  return MHD_OK;
}

int mhd_synchronize(mhd_handle h) {
  int rc = check_handle(h);
  if (rc) return rc;
  MHD_CUDA(cudaStreamSynchronize(h->stream));
  return MHD_OK;
}

int mhd_set_stream(mhd_handle h, void* stream) {
  if (!h) return fail(MHD_ERR_INVALID, "null handle");
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return MHD_OK;
}

void* mhd_get_stream(mhd_handle h) { return h ? (void*)h->stream : nullptr; }

int mhd_memory_bytes(mhd_handle h, long long* bytes) {
  if (!h || !bytes) return fail(MHD_ERR_INVALID, "null argument");
  *bytes = footprint(h->g);
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
  const double state_field = k2 * k2 * kx * c;
  double b = 0;
  // state arrays (6 fields each) one epilogue launch touches, averaged over the scheme's stages
  const double arrays = h->p.scheme == MHD_RK4 ? (3 + 5 + 5 + 4) / 4.0 : (3 + 4 * 4) / 5.0;
  switch (cls) {
    case KC_ZINV: b = 6 * (state_field + n * k2 * kx * c); break;
    case KC_YINV: b = 6 * (n * k2 * kx * c + n * n * kx * c); break;
    case KC_XFUSED: b = (6 + 8) * n * n * kx * c; break;
    case KC_YFWD: b = 8 * (n * n * kx * c + n * k2 * kx * c); break;
    case KC_ZFWD: b = 8 * (n * k2 * kx * c + state_field); break;
    case KC_RKEPI: b = 8 * state_field + arrays * 6 * state_field + 6 * k2 * k2 * c; break;
    case KC_HERM: b = 2 * 6 * k2 * k2 * c; break;
    default: b = 0;
  }
  *bytes = b;
  return MHD_OK;
}

int mhd_step_timed(mhd_handle h, int nsteps, double* ms_per_step) {
  int rc = check_handle(h);
  if (rc) return rc;
  if (nsteps < 1 || !ms_per_step) return fail(MHD_ERR_INVALID, "nsteps >= 1 and a non-null output are required");
  std::vector<cudaEvent_t> ev(nsteps + 1);
  for (auto& e : ev) MHD_CUDA(cudaEventCreate(&e));
  cudaEventRecord(ev[0], h->stream);
  for (int i = 0; i < nsteps && rc == MHD_OK; ++i) {
    rc = mhd_step(h, 1);
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
  cudaEvent_t a, b;
  MHD_CUDA(cudaEventCreate(&a));
  MHD_CUDA(cudaEventCreate(&b));
  cudaEventRecord(a, h->stream);
  rc = mhd_step(h, nsteps);
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

}  // extern "C"
