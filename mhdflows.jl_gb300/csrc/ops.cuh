// Per-grid-size pass kernels and their variants (sm_103a).
//
// Every grid size has a default configuration of each FFT pass.  For the sizes where the choice
// matters there are further candidates (radix plans, kx columns per tile, transforms per
// exchange round, occupancy bounds); mhd_autotune times them on the device and selects one per
// kernel class.  Each grid size is compiled in its own translation unit (ops_*.cu) through the
// make_ops_<n> factories below.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "passes.cuh"
#include "tc5_rows.cuh"
#include "tc_rows.cuh"

namespace mhdgb {

// Kernel classes of one right-hand-side evaluation (also the per-launch profiling classes).
enum KClass { KC_ZINV = 0, KC_YINV, KC_XFUSED, KC_YFWD, KC_ZFWD, KC_RKEPI, KC_OTHER, KC_COUNT };
constexpr int kTunedClasses = 5;  // z_inverse .. z_forward

// Error reporting of the library (defined with the C ABI): stores the message, returns code.
int report_error(int code, const std::string& msg);

using XFn = void (*)(float2*, Geom, long long, long long, long long, BatchRef, const float2*, const float2*,
                     unsigned int*, VpRef);
using ColFn = void (*)(ColArgs, Geom, ColWork, BatchRef, const float2*);
using TmaColFn = void (*)(ColArgs, Geom, ColWork, BatchRef, const float2*, CUtensorMap, TmaCoords, int*);

// A TMA source description for one column pass: the tensor map over the pass's source array,
// its coordinate roles, and the device word a timed-out tile wait is recorded in.
struct TmaPass {
  CUtensorMap map;
  TmaCoords tc;
  int* err = nullptr;
  bool ok = false;
};
using C2RFn = void (*)(const float2*, float*, Geom, long long, float, const float2*);
using R2CFn = void (*)(const float*, float2*, Geom, long long, const float2*);

struct XVariant {
  std::string name;
  XFn fn = nullptr;
  int threads = 0, rpg = 1, groups = 1;
  int (*group_words)(int) = nullptr;  // shared-memory words of one row group for a padded row length
  size_t tw = 0, twr = 0;             // offsets of the plan's twiddles and of its reverse's
  size_t smem = 0;
  int ctas = 0;                       // resident CTAs on the device (0: does not fit)
  // precision form: 0 FP32, 1 split FP16 tensor cores, 2 split BF16 tensor cores; the split
  // forms read a per-device constant table (DFT fragments, twiddles) built by build_table
  int prec = 0;
  // volume penalisation (x_fused_kernel's VPM): 0 none, 1 mask only, 2 mask and wall fields
  int vp = 0;
  // hydrodynamic form (x_fused_kernel's HDX): three fields in, five products out
  int hd = 0;
  size_t table_words = 0;
  int (*build_table)(uint32_t* table) = nullptr;
  uint32_t* table = nullptr;
  int err_word = -1;  // index of a device error word in the table (bounded waits), -1: none
  bool max_carveout = false;  // ask for the largest shared-memory carveout of the L1 array
};

struct ColVariant {
  std::string name;
  ColFn inv = nullptr, fwd = nullptr;
  TmaColFn inv_tma = nullptr, fwd_tma = nullptr;  // set for TMA-fed variants (inv / fwd unused then)
  int threads = 0, tx = 0;
  size_t tw = 0;
  size_t smem = 0;
  int ctas_inv = 0, ctas_fwd = 0;
};

class OpsBase {
 public:
  virtual ~OpsBase();
  int setup(const Geom& g);
  // cap: upper bound of the active instances (the grid covers cap instances; the kernels read
  // the actual count from the BatchRef)
  // tp: the TMA source of this call (nullptr or !ok: a TMA-fed selection falls back to variant 0)
  void col(int cls, const ColArgs& a, const Geom& g, int outer, int nf, BatchRef br, int cap, cudaStream_t s,
           const TmaPass* tp = nullptr) const;
  void x_fused(float2* pool, const Geom& g, long long rowstride, long long slot, long long istride, BatchRef br,
               int cap, unsigned int* vmax, VpRef vp, cudaStream_t s) const;
  void x_c2r(const float2* src, float* dst, const Geom& g, long long srow, float scale, cudaStream_t s) const;
  void x_r2c(const float* src, float2* dst, const Geom& g, long long drow, cudaStream_t s) const;
  // a bounded device wait of the selected x-row kernel that ran out (its table's error word);
  // 0 when none (reads device memory: call where the library synchronises)
  int x_device_error() const;

  int n = 0;
  int prec = 0;  // precision form of the x rows (mhd_params.precision)
  int vp = 0;    // volume-penalisation form of the x rows (XVariant::vp)
  bool vp_capable = false;  // set before setup: prepare the penalty forms too
  int hd = 0;    // set before setup: 1 selects the hydrodynamic x-row form (XVariant::hd)
  // switch the volume-penalisation form; the x-row class falls back to its first variant of the
  // new form (MHD_OK, or MHD_ERR_INVALID when this grid size has none)
  int set_vp(int mode);
  std::vector<XVariant> xv;
  std::vector<ColVariant> cv;
  int sel[kTunedClasses] = {0, 0, 0, 0, 0};  // selected variant of each tuned class
  int variant_count(int cls) const;
  bool variant_ok(int cls, int i) const;
  std::string variant_name(int cls, int i) const;
  int select(int cls, int i);                 // MHD_OK or MHD_ERR_INVALID
  int select_by_name(int cls, const std::string& name);

 protected:
  // plain row transforms (staging of set_physical / get_physical / diagnostics)
  C2RFn c2r = nullptr;
  R2CFn r2c = nullptr;
  int rows = 1, row_threads = 0;
  size_t row_smem = 0, row_tw = 0;
  std::vector<float2> tw_host;
  std::map<std::string, size_t> tw_index;
  float2* tw_dev = nullptr;
};

// Host construction of a plan's stage-twiddle table (PlanTw layout of fft_core.cuh), double
// precision rounded to FP32.
template <class P>
void plan_twiddles(std::vector<float2>& out) {
  constexpr int N = P::N, R0 = P::R0, R1 = P::R1, R2 = P::R2;
  out.assign(PlanTw<P>::SIZE, make_float2(1.f, 0.f));
  auto w = [](long long j) {
    const double ang = 2.0 * 3.14159265358979323846 * (double)(j % N) / (double)N;
    return make_float2((float)std::cos(ang), (float)std::sin(ang));
  };
  for (int n1 = 0; n1 < R1; ++n1)
    for (int k0 = 0; k0 < R0; ++k0) out[n1 * R0 + k0] = w((long long)((n1 * k0) % (R0 * R1)) * R2);
  if (R2 > 1)
    for (int k1 = 0; k1 < R1; ++k1)
      for (int n2 = 0; n2 < R2; ++n2)
        for (int k0 = 0; k0 < R0; ++k0) out[R0 * R1 + k1 * (R0 * R2) + k0 + R0 * n2] = w((long long)n2 * (k0 + R0 * k1));
}

template <class P>
std::string plan_name() {
  std::string s = std::to_string(P::R0) + "x" + std::to_string(P::R1);
  if (P::R2 > 1) s += "x" + std::to_string(P::R2);
  return s + "/g" + std::to_string(P::G);
}

// Builder of one grid size's variant lists (used by the ops_*.cu translation units).
template <int N>
class Ops : public OpsBase {
 public:
  Ops() { n = N; }

  template <class P>
  size_t twiddles() {
    const std::string key = plan_name<P>();
    auto it = tw_index.find(key);
    if (it != tw_index.end()) return it->second;
    std::vector<float2> t;
    plan_twiddles<P>(t);
    const size_t off = tw_host.size();
    tw_host.insert(tw_host.end(), t.begin(), t.end());
    tw_index[key] = off;
    return off;
  }

  // x rows: plan R (inverse; the forward uses its reverse), GROUPS row groups per CTA, NTI / NTF
  // transforms per exchange round, MINB CTAs per SM.
  template <class R, int GROUPS, int NTI, int NTF, int MINB>
  void add_x() {
    add_x_form<R, GROUPS, NTI, NTF, MINB, false>();
  }
  // DIRECT: field rows loaded from global memory into registers, no staging copy ("/d")
  template <class R, int GROUPS, int NTI, int NTF, int MINB, bool DIRECT>
  void add_x_form() {
    constexpr int NTS = NTI > NTF ? NTI : NTF;
    using XC = XCfg<R, NTS, DIRECT>;
    XVariant v;
    v.name = "x:" + plan_name<R>() + "/nt" + std::to_string(NTI) + std::to_string(NTF) + "/c" +
             std::to_string(GROUPS) + "/b" + std::to_string(MINB) + (DIRECT ? "/d" : "");
    v.fn = x_fused_kernel<R, GROUPS, NTI, NTF, MINB, 0, false, DIRECT>;
    v.threads = GROUPS * XC::TPG;
    v.rpg = XC::RPG;
    v.groups = GROUPS;
    v.group_words = &XC::group_words;
    v.tw = twiddles<R>();
    v.twr = twiddles<typename Reverse<R>::type>();
    xv.push_back(v);
  }

  // x rows with the volume-penalisation pairs: the mask-only and the mask-and-walls forms of a
  // plan, one forward transform per exchange round
  template <class R, int GROUPS, int NTI, int MINB>
  void add_x_vp() {
    add_x_vp_one<R, GROUPS, NTI, MINB, 1>();
    add_x_vp_one<R, GROUPS, NTI, MINB, 2>();
  }
  template <class R, int GROUPS, int NTI, int MINB, int VPM>
  void add_x_vp_one() {
    using XC = XCfg<R, NTI>;
    XVariant v;
    v.name = "xvp" + std::to_string(VPM) + ":" + plan_name<R>() + "/nt" + std::to_string(NTI) + "1/c" +
             std::to_string(GROUPS) + "/b" + std::to_string(MINB);
    v.fn = x_fused_kernel<R, GROUPS, NTI, 1, MINB, VPM>;
    v.threads = GROUPS * XC::TPG;
    v.rpg = XC::RPG;
    v.groups = GROUPS;
    v.group_words = &XC::group_words;
    v.tw = twiddles<R>();
    v.twr = twiddles<typename Reverse<R>::type>();
    v.vp = VPM;
    xv.push_back(v);
  }

  // x rows of the hydrodynamic form (one transform per exchange round); VPM > 0 adds the
  // velocity penalty fields (VP on hydrodynamics)
  template <class R, int GROUPS, int MINB, int VPM = 0>
  void add_x_hd() {
    using XC = XCfg<R, 1>;
    XVariant v;
    v.name = std::string(VPM ? "xhdvp" + std::to_string(VPM) : "xhd") + ":" + plan_name<R>() + "/nt11/c" +
             std::to_string(GROUPS) + "/b" + std::to_string(MINB);
    v.fn = x_fused_kernel<R, GROUPS, 1, 1, MINB, VPM, true>;
    v.threads = GROUPS * XC::TPG;
    v.rpg = XC::RPG;
    v.groups = GROUPS;
    v.group_words = &XC::group_words;
    v.tw = twiddles<R>();
    v.twr = twiddles<typename Reverse<R>::type>();
    v.hd = 1;
    v.vp = VPM;
    xv.push_back(v);
  }
  // both penalisation forms (mask only, mask and walls) of the hydrodynamic x rows
  template <class R, int GROUPS, int MINB>
  void add_x_hdvp() {
    add_x_hd<R, GROUPS, MINB, 1>();
    add_x_hd<R, GROUPS, MINB, 2>();
  }

  // x rows on the tensor cores (split FP16 or BF16 operands), GROUPS warps (rows) per CTA
  template <int KIND, int GROUPS, int MINB>
  void add_x_tc() {
    XVariant v;
    v.name = std::string("xtc:") + (KIND == SPLIT_F16 ? "f16" : "bf16") + "/16x" + std::to_string(N / 16) + "/c" +
             std::to_string(GROUPS) + "/b" + std::to_string(MINB);
    v.fn = x_fused_tc_kernel<N, KIND, GROUPS, MINB>;
    v.threads = GROUPS * 32;
    v.rpg = 1;
    v.groups = GROUPS;
    v.group_words = &tc_group_words<N>;
    v.prec = KIND == SPLIT_F16 ? 1 : 2;
    v.table_words = TcLayout<N>::WORDS;
    v.build_table = &tc_build_table<N, KIND>;
    xv.push_back(v);
  }

  // x rows on the fifth-generation tensor cores (tcgen05, split TF32 operands, n = 256 only)
  void add_x_tc5() {
    static_assert(N == 256, "the tcgen05 x rows are built for n = 256");
    XVariant v;
    v.name = "xtc5:tf32/16x16/m128";
    v.fn = x_fused_tc5_kernel<N>;
    v.threads = Tc5Layout::THREADS;
    v.rpg = Tc5Layout::TILE_ROWS;
    v.groups = 1;
    v.group_words = &tc5_group_words;
    v.prec = 3;
    v.table_words = Tc5Layout::WORDS;
    v.build_table = &tc5_build_table<N>;
    v.err_word = Tc5Layout::ERR;
    v.max_carveout = true;
    xv.push_back(v);
  }

  // column passes (y and z): plan C, TX kx columns per tile, MINB CTAs per SM, NBUF tile buffers
  // TWS: stage twiddles in shared memory (behind the tiles)
  template <class C, int TX, int MINB, int NBUF = 2, bool TWS = false>
  void add_col() {
    ColVariant c;
    c.name = "col:" + plan_name<C>() + "/tx" + std::to_string(TX) + "/b" + std::to_string(MINB) +
             (NBUF == 2 ? std::string() : "/q" + std::to_string(NBUF)) + (TWS ? "/ts" : "");
    c.inv = col_pass_kernel<C, TX, +1, true, false, MINB, NBUF, TWS>;
    c.fwd = col_pass_kernel<C, TX, -1, false, true, MINB, NBUF, TWS>;
    c.threads = TX * C::G;
    c.tx = TX;
    c.smem = sizeof(float2) * (NBUF * (size_t)N * TX + (TWS ? PlanTw<C>::SIZE : 0));
    c.tw = twiddles<C>();
    cv.push_back(c);
  }

  // TMA-fed column passes (16 kx columns: 128-byte box rows keep every box destination aligned)
  template <class C, int MINB, int NBUF, bool TWS = false>
  void add_col_tma() {
    constexpr int TX = 16;
    ColVariant c;
    c.name = "coltma:" + plan_name<C>() + "/tx" + std::to_string(TX) + "/b" + std::to_string(MINB) + "/q" +
             std::to_string(NBUF) + (TWS ? "/ts" : "");
    c.inv_tma = col_pass_tma_kernel<C, TX, +1, true, false, MINB, NBUF, TWS>;
    c.fwd_tma = col_pass_tma_kernel<C, TX, -1, false, true, MINB, NBUF, TWS>;
    c.threads = TX * C::G;
    c.tx = TX;
    c.smem = sizeof(float2) * NBUF * (size_t)N * TX + NBUF * sizeof(unsigned long long) + 16 +
             (TWS ? sizeof(float2) * PlanTw<C>::SIZE : 0);
    c.tw = twiddles<C>();
    cv.push_back(c);
  }

  // plain row c2r / r2c kernels, ROWS row pairs per CTA
  template <class R, int ROWS>
  void set_rows() {
    c2r = x_c2r_kernel<R, ROWS>;
    r2c = x_r2c_kernel<R, ROWS>;
    rows = ROWS;
    row_threads = ROWS * R::G;
    row_smem = sizeof(float2) * (size_t)RowCfg<R>::TS * ROWS;
    row_tw = twiddles<R>();
  }
};

OpsBase* make_ops_16();
OpsBase* make_ops_32();
OpsBase* make_ops_48();
OpsBase* make_ops_64();
OpsBase* make_ops_96();
OpsBase* make_ops_128();
OpsBase* make_ops_256();
OpsBase* make_ops_512();

}  // namespace mhdgb
