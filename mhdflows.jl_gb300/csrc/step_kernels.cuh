// Spectral epilogue, layout conversion, CFL and diagnostics kernels of the MHD step (sm_103a).
// Included by the library's main translation unit only (the non-template kernels here have one
// definition); the FFT pass kernels are in passes.cuh.
#pragma once
#include "stage_math.cuh"

namespace mhdgb {

// grid (ceil(kx / blockDim.x), k2, k2): one thread per retained mode, no index division.
// HD: the hydrodynamic form (three fields, five product planes; B is neither read nor written).
template <int OP, bool FORCED, bool VPEN, bool HD = false>
__global__ void __launch_bounds__(256) rk_epilogue_kernel(RkArgs a, Geom geo, BatchRef br) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= geo.kx) return;
  const int inst = blockIdx.z / geo.k2;
  if (inst >= *br.count) return;
  const int slot = br.list[inst];
  const int jy = blockIdx.y, jz = blockIdx.z - inst * geo.k2;
  const long long fs = a.fs;
  const long long i = ((long long)jz * geo.k2 + jy) * geo.kxp + x;
  const float2* prod = a.prod + slot * a.prodI;
  const float kxv = geo.kscale * (float)x;
  const float kyv = geo.kscale * (float)signed_of_kept(geo, jy);
  const float kzv = geo.kscale * (float)signed_of_kept(geo, jz);
  float2 p[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) p[q] = (HD && q >= 5) ? make_float2(0.f, 0.f) : cscale(__ldcs(prod + q * fs + i), a.pscale);
  const float2 dxz = p[0], dyz = p[1], txy = p[2], txz = p[3], tyz = p[4];
  const float2 axy = p[5], axz = p[6], ayz = p[7];
  ModeSums m;
  m.Vx = make_float2(kxv * dxz.x + kyv * txy.x + kzv * txz.x, kxv * dxz.y + kyv * txy.y + kzv * txz.y);
  m.Vy = make_float2(kxv * txy.x + kyv * dyz.x + kzv * tyz.x, kxv * txy.y + kyv * dyz.y + kzv * tyz.y);
  m.Vz = make_float2(kxv * txz.x + kyv * tyz.x, kxv * txz.y + kyv * tyz.y);
  m.Wx = make_float2(kyv * axy.x + kzv * axz.x, kyv * axy.y + kzv * axz.y);
  m.Wy = make_float2(kzv * ayz.x - kxv * axy.x, kzv * ayz.y - kxv * axy.y);
  m.Wz = make_float2(-(kxv * axz.x + kyv * ayz.x), -(kxv * axz.y + kyv * ayz.y));
  finish_mode<OP, FORCED, VPEN, HD>(a, geo, slot, jz, jy, x, i, kxv, kyv, kzv, m, prod);
}

// On-device getCFL! (src/integrator.jl:158-198 of MHDFlows.jl) after a step of every active
// slot: t += dt of the step just taken; next dt = min(coef * dx / max(|u|max, |B|max), tdiff)
// from the maxima x_fused recorded on the step's last stage; the maxima are cleared for the next
// step.  A slot with no finite positive maximum keeps its dt.
// vmax holds maxima of the unnormalised fields the passes work with (n^3 times the physical
// values); vscale = 1/n^3 converts them.
__global__ void cfl_update_kernel(BatchRef br, SlotParams* sp, unsigned int* vmax, double* t, float coef_dx,
                                  float vscale, int advance) {
  const int n = *br.count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = br.list[i];
    SlotParams p = sp[s];
    if (advance) t[s] += (double)p.dt;
    const float vm = vscale * fmaxf(__uint_as_float(vmax[2 * s]), __uint_as_float(vmax[2 * s + 1]));
    if (vm > 0.f && isfinite(vm)) {
      float dt = coef_dx / vm;
      if (p.tdiff > 0.f) dt = fminf(dt, p.tdiff);
      p.dt = dt;
      sp[s] = p;
    }
    vmax[2 * s] = 0u;
    vmax[2 * s + 1] = 0u;
  }
}

// one step of every active slot taken: advance the per-slot step counters (random forcing)
__global__ void step_tick_kernel(BatchRef br, long long* steps) {
  const int n = *br.count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) steps[br.list[i]] += 1;
}

// max |field| of one physical field into vmax[which] (initial fields before the first CFL step).
__global__ void maxabs_into_kernel(const float* __restrict__ a, long long n, unsigned int* out) {
  unsigned int m = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    m = max(m, __float_as_uint(fabsf(a[i])));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// ------------------------------------------------------------------------------------------
// Layout conversion between the reference's column-major sol[kx, ky, kz, f] (half spectrum,
// nkr = n/2+1) and the compact retained-band state.
// ------------------------------------------------------------------------------------------
__global__ void gather_state_kernel(const float2* __restrict__ ref, float2* __restrict__ S, Geom geo, int nf) {
  const long long total = (long long)nf * geo.k2 * geo.k2 * geo.kxp;
  const int nkr = geo.n / 2 + 1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % geo.kxp);
    long long r = i / geo.kxp;
    const int jy = (int)(r % geo.k2); r /= geo.k2;
    const int jz = (int)(r % geo.k2);
    const int f = (int)(r / geo.k2);
    float2 val = make_float2(0.f, 0.f);
    if (x < geo.kx) {
      const int fy = freq_of_kept(geo, jy), fz = freq_of_kept(geo, jz);
      val = ref[(((long long)f * geo.n + fz) * geo.n + fy) * nkr + x];
    }
    S[i] = val;
  }
}

// One element of the reference layout from the compact state (zero in the alias band).
__device__ __forceinline__ float2 ref_value(const float2* __restrict__ S, const Geom& geo, long long i, int nkr) {
  const int x = (int)(i % nkr);
  long long r = i / nkr;
  const int fy = (int)(r % geo.n); r /= geo.n;
  const int fz = (int)(r % geo.n);
  const int f = (int)(r / geo.n);
  const int jy = kept_of_freq(geo, fy), jz = kept_of_freq(geo, fz);
  if (x < geo.kx && jy >= 0 && jz >= 0) return S[(((long long)f * geo.k2 + jz) * geo.k2 + jy) * geo.kxp + x];
  return make_float2(0.f, 0.f);
}

// Compact state -> reference layout, two elements (one 16-byte store) per thread and step: the
// element count nf n^2 nkr is even and ref is 16-byte aligned, so every pair is aligned.  The
// output may be mapped host memory, where wide stores use the host link better.
__global__ void scatter_state_kernel(const float2* __restrict__ S, float2* __restrict__ ref, Geom geo, int nf) {
  const int nkr = geo.n / 2 + 1;
  const long long pairs = (long long)nf * geo.n * geo.n * nkr / 2;
  float4* out = reinterpret_cast<float4*>(ref);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < pairs; p += (long long)gridDim.x * blockDim.x) {
    const float2 a = ref_value(S, geo, 2 * p, nkr), b = ref_value(S, geo, 2 * p + 1, nkr);
    out[p] = make_float4(a.x, a.y, b.x, b.y);
  }
}

// Compact state -> the retained elements of the reference layout (kx < Kx, ky and kz kept),
// 8-byte stores; every other element is zero and the caller fills it.
__global__ void scatter_retained_kernel(const float2* __restrict__ S, float2* __restrict__ ref, Geom geo, int nf) {
  const int nkr = geo.n / 2 + 1;
  const long long total = (long long)nf * geo.k2 * geo.k2 * geo.kx;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total; p += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(p % geo.kx);
    long long r = p / geo.kx;
    const int jy = (int)(r % geo.k2); r /= geo.k2;
    const int jz = (int)(r % geo.k2);
    const int f = (int)(r / geo.k2);
    const long long row = ((long long)f * geo.n + freq_of_kept(geo, jz)) * geo.n + freq_of_kept(geo, jy);
    ref[row * nkr + x] = S[(((long long)f * geo.k2 + jz) * geo.k2 + jy) * geo.kxp + x];
  }
}

// ------------------------------------------------------------------------------------------
// Diagnostics.
// ------------------------------------------------------------------------------------------
// Per-block partial sums over the compact state (double accumulation, fixed order):
//   [0] sum w|u|^2  [1] sum w|b|^2  [2] sum w Re(u.conj b)  [3] max|k.u|  [4] max|k.b|  [5] non-finite count
// w = 1 on the kx = 0 plane and 2 elsewhere (the half spectrum stands for both +-kx).
constexpr int kDiagSlots = 6;
constexpr int kDiagThreads = 256;

__device__ __forceinline__ void block_reduce_diag(double (&acc)[kDiagSlots], double* out) {
  __shared__ double red[kDiagThreads / 32][kDiagSlots];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < kDiagSlots; ++s) {
    double x = acc[s];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_down_sync(0xffffffffu, x, o);
      x = (s == 3 || s == 4) ? fmax(x, y) : x + y;
    }
    if (lane == 0) red[wid][s] = x;
  }
  __syncthreads();
  if (threadIdx.x < kDiagSlots) {
    const int s = threadIdx.x;
    double x = red[0][s];
    for (int w = 1; w < kDiagThreads / 32; ++w) x = (s == 3 || s == 4) ? fmax(x, red[w][s]) : x + red[w][s];
    out[s] = x;
  }
}

__global__ void __launch_bounds__(kDiagThreads) diag_partial_kernel(const float2* __restrict__ S, Geom geo, double* partial) {
  const long long plane = (long long)geo.k2 * geo.k2 * geo.kxp;  // one field
  double acc[kDiagSlots] = {0, 0, 0, 0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < plane; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % geo.kxp);
    if (x >= geo.kx) continue;
    long long r = i / geo.kxp;
    const int jy = (int)(r % geo.k2);
    const int jz = (int)(r / geo.k2);
    const double w = x == 0 ? 1.0 : 2.0;
    const double kx = (double)geo.kscale * x;
    const double ky = (double)geo.kscale * signed_of_kept(geo, jy);
    const double kz = (double)geo.kscale * signed_of_kept(geo, jz);
    double2 ku = make_double2(0, 0), kb = make_double2(0, 0);
    double eu = 0, eb = 0, hc = 0;
    bool bad = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 u = S[c * plane + i], b = S[(c + 3) * plane + i];
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

// Second pass: reduce the block partials in block order (deterministic).
__global__ void __launch_bounds__(kDiagThreads) diag_final_kernel(const double* __restrict__ partial, int nblocks, double* out) {
  double acc[kDiagSlots] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
    for (int s = 0; s < kDiagSlots; ++s) {
      const double x = partial[b * kDiagSlots + s];
      acc[s] = (s == 3 || s == 4) ? fmax(acc[s], x) : acc[s] + x;
    }
  }
  block_reduce_diag(acc, out);
}

// On-device diagnostics history (getCFL! / increment!(diags) without host synchronisation):
// grid (blocks, cap), blockIdx.y = instance; the partial sums of slot s go to
// partial[(s * gridDim.x + block) * kDiagSlots].
__global__ void __launch_bounds__(kDiagThreads) diag_partial_batch_kernel(const float2* __restrict__ pool, long long stI,
                                                                          Geom geo, BatchRef br, double* partial) {
  const int inst = blockIdx.y;
  if (inst >= *br.count) return;
  const int slot = br.list[inst];
  const float2* S = pool + slot * stI;
  const long long plane = (long long)geo.k2 * geo.k2 * geo.kxp;
  double acc[kDiagSlots] = {0, 0, 0, 0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < plane; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % geo.kxp);
    if (x >= geo.kx) continue;
    long long r = i / geo.kxp;
    const int jy = (int)(r % geo.k2);
    const int jz = (int)(r / geo.k2);
    const double w = x == 0 ? 1.0 : 2.0;
    const double kx = (double)geo.kscale * x;
    const double ky = (double)geo.kscale * signed_of_kept(geo, jy);
    const double kz = (double)geo.kscale * signed_of_kept(geo, jz);
    double2 ku = make_double2(0, 0), kb = make_double2(0, 0);
    double eu = 0, eb = 0, hc = 0;
    bool bad = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 u = S[c * plane + i], b = S[(c + 3) * plane + i];
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
  block_reduce_diag(acc, partial + ((long long)slot * gridDim.x + blockIdx.x) * kDiagSlots);
}

// grid (cap): one block per instance reduces its slot's partials (block order, deterministic)
// into sample *count of the history: hist[(sample * cap + slot) * kHistVals + v] with v =
// E_u, E_B, H_c (times scale = dV / n^3), max|k.u|, max|k.B|, non-finite count, device time
// (dtime[slot], or -1 without the on-device clock).  Samples past `capacity` are counted, not
// stored.  hist_tick_kernel advances the count after every slot has read it.
constexpr int kHistVals = 7;
__global__ void __launch_bounds__(kDiagThreads) diag_record_kernel(const double* __restrict__ partial, int nblocks, BatchRef br,
                                                                   int cap, double* hist, const int* count, int capacity,
                                                                   const double* dtime, double scale) {
  const int inst = blockIdx.x;
  if (inst >= *br.count) return;
  const int slot = br.list[inst];
  double acc[kDiagSlots] = {0, 0, 0, 0, 0, 0};
  const double* p = partial + (long long)slot * nblocks * kDiagSlots;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
    for (int s = 0; s < kDiagSlots; ++s) {
      const double x = p[b * kDiagSlots + s];
      acc[s] = (s == 3 || s == 4) ? fmax(acc[s], x) : acc[s] + x;
    }
  }
  __shared__ double red[kDiagSlots];
  block_reduce_diag(acc, red);
  __syncthreads();
  const int sample = *count;
  if (threadIdx.x == 0 && sample < capacity) {
    double* o = hist + ((long long)sample * cap + slot) * kHistVals;
    o[0] = red[0] * scale;
    o[1] = red[1] * scale;
    o[2] = red[2] * scale;
    o[3] = red[3];
    o[4] = red[4];
    o[5] = red[5];
    o[6] = dtime ? dtime[slot] : -1.0;
  }
}
__global__ void hist_tick_kernel(int* count) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *count += 1;
}

// i k.B into a one-field compact buffer (input of the div B inverse transform).
__global__ void divb_spectrum_kernel(const float2* __restrict__ S, float2* __restrict__ out, Geom geo) {
  const long long plane = (long long)geo.k2 * geo.k2 * geo.kxp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < plane; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % geo.kxp);
    long long r = i / geo.kxp;
    const int jy = (int)(r % geo.k2);
    const int jz = (int)(r / geo.k2);
    const float kx = geo.kscale * x, ky = geo.kscale * signed_of_kept(geo, jy), kz = geo.kscale * signed_of_kept(geo, jz);
    const float2 bx = S[3 * plane + i], by = S[4 * plane + i], bz = S[5 * plane + i];
    const float re = kx * bx.x + ky * by.x + kz * bz.x;
    const float im = kx * bx.y + ky * by.y + kz * bz.y;
    out[i] = x < geo.kx ? make_float2(-im, re) : make_float2(0.f, 0.f);
  }
}

// DivVCorrection! / DivBCorrection! (src/Solver/VPSolver.jl:60-138): u (mask bit 0) and B (bit 1)
// of every active slot lose their gradient part, X -= k (k.X) / k^2 with 1/k^2 = 0 at k = 0.
// grid (ceil(kx / blockDim.x), k2, k2 * cap): one thread per retained mode.
__global__ void div_correct_kernel(float2* __restrict__ pool, Geom geo, long long fs, long long stI, BatchRef br,
                                   int mask) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= geo.kx) return;
  const int inst = blockIdx.z / geo.k2;
  if (inst >= *br.count) return;
  const int jy = blockIdx.y, jz = blockIdx.z - inst * geo.k2;
  float2* X = pool + br.list[inst] * stI + ((long long)jz * geo.k2 + jy) * geo.kxp + x;
  const float kx = geo.kscale * (float)x;
  const float ky = geo.kscale * (float)signed_of_kept(geo, jy);
  const float kz = geo.kscale * (float)signed_of_kept(geo, jz);
  const float k2 = kx * kx + ky * ky + kz * kz;
  const float ik2 = k2 > 0.f ? 1.0f / k2 : 0.f;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    if (!(mask & (1 << h))) continue;
    float2* F = X + 3 * h * fs;
    const float2 a = F[0], b = F[fs], c = F[2 * fs];
    const float pr = (kx * a.x + ky * b.x + kz * c.x) * ik2;
    const float pi = (kx * a.y + ky * b.y + kz * c.y) * ik2;
    F[0] = make_float2(a.x - kx * pr, a.y - kx * pi);
    F[fs] = make_float2(b.x - ky * pr, b.y - ky * pi);
    F[2 * fs] = make_float2(c.x - kz * pr, c.y - kz * pi);
  }
}

// Check of the bounded wait the TMA-fed passes use: one thread waits on an mbarrier that nothing
// arrives on, with a limit of limit_ns, and records in out[0] whether the wait gave up (1) and in
// out[1] the nanoseconds it waited.  The kernel then returns like a pass that timed out.
__global__ void bounded_wait_check_kernel(unsigned long long limit_ns, unsigned long long* out) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  const unsigned int b = smem_u32(&bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  const unsigned long long t0 = global_ns();
  const bool done = mbar_wait(b, 0u, limit_ns);
  out[0] = done ? 0ull : 1ull;
  out[1] = global_ns() - t0;
}

// Bytes of a guard band that differ from its fill value, added to *bad.
__global__ void guard_check_kernel(const unsigned char* __restrict__ g, long long n, unsigned char fill,
                                   unsigned long long* bad) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const unsigned int b = (i < n && g[i] != fill) ? 1u : 0u;
  const unsigned int cnt = __popc(__ballot_sync(0xffffffffu, b));
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(bad, (unsigned long long)cnt);
}

// max |x| over a float array via the ordered bit pattern of non-negative floats (NaN wins).
__global__ void maxabs_kernel(const float* __restrict__ a, long long n, unsigned int* out) {
  unsigned int m = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned int b = __float_as_uint(fabsf(a[i]));
    m = b > m ? b : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned int y = __shfl_down_sync(0xffffffffu, m, o);
    m = y > m ? y : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

}  // namespace mhdgb
