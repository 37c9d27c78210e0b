// Set-up, launch and selection of the pass-kernel variants of one grid size.
#include <string>

#include "../../include/mhdgb.h"
#include "ops.cuh"

namespace mhdgb {

OpsBase::~OpsBase() {
  if (tw_dev) cudaFree(tw_dev);
  for (auto& x : xv)
    if (x.table) cudaFree(x.table);
}

namespace {

int set_smem(const void* fn, size_t bytes) {
  if (bytes <= 48 * 1024) return MHD_OK;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return report_error(MHD_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
  return MHD_OK;
}

// Resident CTAs of a kernel on the whole device (persistent grid size); 0 when it does not fit.
int resident_ctas(const void* fn, int threads, size_t smem, int sms, int* out) {
  int per = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem);
  if (e != cudaSuccess) return report_error(MHD_ERR_CUDA, std::string("occupancy query: ") + cudaGetErrorString(e));
  *out = per * sms;
  return MHD_OK;
}

bool is_col(int cls) { return cls == KC_ZINV || cls == KC_YINV || cls == KC_YFWD || cls == KC_ZFWD; }
bool is_inv(int cls) { return cls == KC_ZINV || cls == KC_YINV; }

}  // namespace

int OpsBase::setup(const Geom& g) {
  if (g.kx != kept_kx_of(n) || g.kp != kept_kx_of(n) || g.kn != kept_kn_of(n))
    return report_error(MHD_ERR_INVALID, "kept-mode counts differ from the compiled pass plans");
  int rc = MHD_OK, dev = 0, sms = 0, smem_max = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return report_error(MHD_ERR_CUDA, std::string("device query: ") + cudaGetErrorString(e));
  e = cudaMalloc(&tw_dev, tw_host.size() * sizeof(float2));
  if (e != cudaSuccess) return report_error(MHD_ERR_OOM, std::string("twiddle tables: ") + cudaGetErrorString(e));
  e = cudaMemcpy(tw_dev, tw_host.data(), tw_host.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return report_error(MHD_ERR_CUDA, std::string("twiddle upload: ") + cudaGetErrorString(e));
  for (auto& x : xv) {
    x.smem = sizeof(float2) * (size_t)x.groups * x.group_words(g.kxp);
    x.ctas = 0;
    if (x.prec != prec || (int)x.smem > smem_max) continue;  // only this problem's precision form
    if (x.vp && !vp_capable) continue;                       // penalty forms only with VP on
    if (x.hd != hd) continue;                                // this problem's field set only
    if (x.build_table) {
      e = cudaMalloc(&x.table, x.table_words * sizeof(uint32_t));
      if (e != cudaSuccess) return report_error(MHD_ERR_OOM, std::string("tensor-core tables: ") + cudaGetErrorString(e));
      if (x.build_table(x.table)) return report_error(MHD_ERR_CUDA, "building the tensor-core DFT tables failed");
    }
    if ((rc = set_smem((const void*)x.fn, x.smem))) return rc;
    if (x.max_carveout) {
      // the whole unified L1 / shared array as shared memory: two CTAs per SM fit only then
      e = cudaFuncSetAttribute((const void*)x.fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      if (e != cudaSuccess) return report_error(MHD_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
    }
    if ((rc = resident_ctas((const void*)x.fn, x.threads, x.smem, sms, &x.ctas))) return rc;
  }
  for (auto& c : cv) {
    c.ctas_inv = c.ctas_fwd = 0;
    if ((int)c.smem > smem_max) continue;
    const void* fi = c.inv_tma ? (const void*)c.inv_tma : (const void*)c.inv;
    const void* ff = c.fwd_tma ? (const void*)c.fwd_tma : (const void*)c.fwd;
    if ((rc = set_smem(fi, c.smem))) return rc;
    if ((rc = set_smem(ff, c.smem))) return rc;
    if ((rc = resident_ctas(fi, c.threads, c.smem, sms, &c.ctas_inv))) return rc;
    if ((rc = resident_ctas(ff, c.threads, c.smem, sms, &c.ctas_fwd))) return rc;
  }
  if (!cv.empty() && cv[0].inv_tma) return report_error(MHD_ERR_INVALID, "the default column variant must not be TMA-fed");
  if ((rc = set_smem((const void*)c2r, row_smem))) return rc;
  if ((rc = set_smem((const void*)r2c, row_smem))) return rc;
  // the default of each class is its first variant that fits on this device
  for (int cls = 0; cls < kTunedClasses; ++cls) {
    int i = 0;
    while (i < variant_count(cls) && !variant_ok(cls, i)) ++i;
    if (i == variant_count(cls))
      return report_error(cls == KC_XFUSED && prec ? MHD_ERR_INVALID : MHD_ERR_CUDA,
                          cls == KC_XFUSED && prec ? "no x-row kernel of this precision form for this grid size"
                                                   : "no pass-kernel variant fits on this device");
    sel[cls] = i;
  }
  return MHD_OK;
}

int OpsBase::set_vp(int mode) {
  if (mode == vp) return MHD_OK;
  const int old = vp;
  vp = mode;
  for (int i = 0; i < (int)xv.size(); ++i)
    if (variant_ok(KC_XFUSED, i)) { sel[KC_XFUSED] = i; return MHD_OK; }
  vp = old;
  return report_error(MHD_ERR_INVALID, "no x-row kernel of this volume-penalisation form for this grid size");
}

int OpsBase::variant_count(int cls) const {
  if (cls == KC_XFUSED) return (int)xv.size();
  return is_col(cls) ? (int)cv.size() : 0;
}

bool OpsBase::variant_ok(int cls, int i) const {
  if (i < 0 || i >= variant_count(cls)) return false;
  if (cls == KC_XFUSED) return xv[i].ctas > 0 && xv[i].prec == prec && xv[i].vp == vp && xv[i].hd == hd;
  return is_inv(cls) ? cv[i].ctas_inv > 0 : cv[i].ctas_fwd > 0;
}

std::string OpsBase::variant_name(int cls, int i) const {
  if (i < 0 || i >= variant_count(cls)) return "";
  return cls == KC_XFUSED ? xv[i].name : cv[i].name;
}

int OpsBase::select(int cls, int i) {
  if (cls < 0 || cls >= kTunedClasses || !variant_ok(cls, i))
    return report_error(MHD_ERR_INVALID, "no such kernel variant (class " + std::to_string(cls) + ", index " +
                                             std::to_string(i) + ")");
  sel[cls] = i;
  return MHD_OK;
}

int OpsBase::select_by_name(int cls, const std::string& name) {
  for (int i = 0; i < variant_count(cls); ++i)
    if (variant_name(cls, i) == name) return select(cls, i);
  return report_error(MHD_ERR_INVALID, "no kernel variant named " + name);
}

void OpsBase::col(int cls, const ColArgs& a, const Geom& g, int outer, int nf, BatchRef br, int cap,
                  cudaStream_t s, const TmaPass* tp) const {
  const bool tma_sel = cv[sel[cls]].inv_tma != nullptr;
  const ColVariant& c = (tma_sel && !(tp && tp->ok)) ? cv[0] : cv[sel[cls]];
  const bool inv = is_inv(cls);
  if (c.inv_tma) {
    const ColWork w{(g.kx + c.tx - 1) / c.tx, outer, nf, inv ? g.k2 : n};
    const long long total = (long long)cap * w.tiles_x * w.outer * w.nf;
    const int ctas = inv ? c.ctas_inv : c.ctas_fwd;
    const int grid = (int)(total < ctas ? total : ctas);
    const TmaColFn f = inv ? c.inv_tma : c.fwd_tma;
    f<<<grid, c.threads, c.smem, s>>>(a, g, w, br, tw_dev + c.tw, tp->map, tp->tc, tp->err);
    return;
  }
  const ColWork w{(g.kx + c.tx - 1) / c.tx, outer, nf, inv ? g.k2 : n};
  const long long total = (long long)cap * w.tiles_x * w.outer * w.nf;
  const int ctas = inv ? c.ctas_inv : c.ctas_fwd;
  const int grid = (int)(total < ctas ? total : ctas);
  const ColFn f = inv ? c.inv : c.fwd;
  f<<<grid, c.threads, c.smem, s>>>(a, g, w, br, tw_dev + c.tw);
}

void OpsBase::x_fused(float2* pool, const Geom& g, long long rowstride, long long slot, long long istride,
                      BatchRef br, int cap, unsigned int* vmax, VpRef vp, cudaStream_t s) const {
  const XVariant& x = xv[sel[KC_XFUSED]];
  const long long groups = (long long)cap * n * n / x.rpg;
  const long long need = (groups + x.groups - 1) / x.groups;
  const int grid = (int)(need < x.ctas ? need : x.ctas);
  const float2* t1 = x.table ? reinterpret_cast<const float2*>(x.table) : tw_dev + x.tw;
  const float2* t2 = x.table ? nullptr : tw_dev + x.twr;
  x.fn<<<grid, x.threads, x.smem, s>>>(pool, g, rowstride, slot, istride, br, t1, t2, vmax, vp);
}

int OpsBase::x_device_error() const {
  const XVariant& x = xv[sel[KC_XFUSED]];
  if (!x.table || x.err_word < 0) return 0;
  uint32_t e = 0;
  if (cudaMemcpy(&e, x.table + x.err_word, sizeof(e), cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
  return e != 0;
}

void OpsBase::x_c2r(const float2* src, float* dst, const Geom& g, long long srow, float scale, cudaStream_t s) const {
  const long long pairs = (long long)n * n / 2;
  c2r<<<(unsigned)(pairs / rows), row_threads, row_smem, s>>>(src, dst, g, srow, scale, tw_dev + row_tw);
}

void OpsBase::x_r2c(const float* src, float2* dst, const Geom& g, long long drow, cudaStream_t s) const {
  const long long pairs = (long long)n * n / 2;
  r2c<<<(unsigned)(pairs / rows), row_threads, row_smem, s>>>(src, dst, g, drow, tw_dev + row_tw);
}

}  // namespace mhdgb
