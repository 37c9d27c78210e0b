// Spectral epilogue, layout conversion, CFL and diagnostics kernels of the MHD step (sm_103a).
// Included by the library's main translation unit only (the non-template kernels here have one
// definition); the FFT pass kernels are in passes.cuh.
#pragma once
#include "passes.cuh"

namespace mhdgb {

// Runge-Kutta stage operations of the epilogue.
enum StageOp : int {
  OP_RHS = 0,       // out <- R
  OP_RK4_FIRST = 1, // acc <- R/6 ; xn <- sol + h R            (X = sol)
  OP_RK4_MID = 2,   // acc <- acc + R/3 ; xn <- sol + h R
  OP_RK4_LAST = 3,  // sol <- sol + dt (acc + R/6)
  OP_LS_FIRST = 4,  // du <- dt R ; u <- u + b du              (X = u)
  OP_LS = 5,        // du <- a du + dt R ; u <- u + b du
};

// ------------------------------------------------------------------------------------------
// Streaming right-hand side + Runge-Kutta stage update over the compact retained band.
// prod: compact spectra of the 8 products [p][kz'][ky'][kx] (Dxz Dyz Txy Txz Tyz Axy Axz Ayz).
// Momentum: R_u = i (V - k (k.V)/k^2) - nu k^2 X_u with V = (kx Dxz + ky Txy + kz Txz,
// kx Txy + ky Dyz + kz Tyz, kx Txz + ky Tyz) (the stress tensor minus Tzz*I, whose gradient the
// projection removes).  Induction: R_b = i k x E - eta k^2 X_b with E = (Ayz, -Axz, Axy) = u x B.
// ------------------------------------------------------------------------------------------
struct RkArgs {
  const float2* prod;   // 8 compact product planes, then 6 penalty planes with VP (slot stride prodI)
  const float2* X;      // stage state (6 fields, slot stride stI)
  const float2* H;      // Hermitian part of X on the kx = 0 plane, [f][kz'][ky'] (slot stride hI)
  float2* sol;          // RK4 step-start state
  float2* acc;          // RK4 accumulator / LSRK4 du / OP_RHS output
  float2* xn;           // RK4 next stage state / LSRK4 u
  const SlotParams* sp; // per-slot nu, eta, dt
  long long fs;         // compact field stride (complex elements)
  long long stI, prodI, hI;
  float hf;             // RK4 stage fraction of dt (1/2 or 1)
  float ca, cb;         // LSRK4 coefficients of the stage
  float pscale;         // 1/n^6: the column and row passes are unnormalised in both directions
  int op;
  const long long* step; // per-slot step counters (random forcing: call = 8 * step + stage)
  int stage;             // right-hand-side evaluation within the step (7: outside a step)
  int hydro;             // hydrodynamics: the induction right-hand side is zero, B stays zero
  float vscale;          // 1/n^3: the penalty planes are n^3 times the reference's rfft
};

// ------------------------------------------------------------------------------------------
// A99 random solenoidal forcing (src/pgen/A99ForceDriving_GPU.jl:76-130 of MHDFlows.jl), with
// a counter-based generator in place of the device rand(): uniform numbers from the SplitMix64
// finaliser of (seed, call, mode index in the reference's (nkr, n, n) layout, draw).
// ------------------------------------------------------------------------------------------
__host__ __device__ inline unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ float a99_uniform(unsigned long long key, unsigned long long index, int draw) {
  const unsigned long long z = mix64(key ^ (index * 4ull + (unsigned long long)draw));
  return (float)(z >> 40) * (1.0f / 16777216.0f);
}
// forcing of the three velocity components at wavenumber (kx, ky, kz)
__device__ __forceinline__ void a99_force(const SlotParams& sp, unsigned long long key, unsigned long long index,
                                          float kx, float ky, float kz, float2 (&F)[3]) {
  constexpr float kPi = 3.14159265358979f;
  const float k = sqrtf(kx * kx + ky * ky + kz * kz);
  const float kp = sqrtf(kx * kx + kz * kz);
  const float kinv = k > 0.f ? 1.f / k : 0.f;
  const float pinv = kp > 0.f ? 1.f / kp : 0.f;
  const float dk = k - sp.fkf;
  const float Fk = sp.fA * sqrtf(expf(-dk * dk / sp.fs2) / 2.f / kPi) * kinv;
  const float e1x = kz * pinv, e1z = -kx * pinv;
  const float e2x = kx * ky * pinv * kinv, e2y = -kp * kinv, e2z = kz * ky * pinv * kinv;
  const float th1 = a99_uniform(key, index, 0) * 2.f * kPi;
  const float phi = a99_uniform(key, index, 1) * kPi;
  const float th2 = a99_uniform(key, index, 2) * 2.f * kPi;
  float gi = -tanhf(sp.fb * (phi - kPi / 2)) / tanhf(sp.fb * kPi / 2);
  if (fabsf(gi) >= 1.f) gi = copysignf(1.f, gi);
  const float gj = sqrtf(1.f - gi * gi);
  float s1, c1, s2, c2;
  sincosf(th1, &s1, &c1);
  sincosf(th2, &s2, &c2);
  const float amp = sp.fA * Fk;
  const float a1 = amp * gi, a2 = amp * gj;
  F[0] = make_float2(a1 * e1x * c1 + a2 * e2x * c2, a1 * e1x * s1 + a2 * e2x * s2);
  F[1] = make_float2(a2 * e2y * c2, a2 * e2y * s2);
  F[2] = make_float2(a1 * e1z * c1 + a2 * e2z * c2, a1 * e1z * s1 + a2 * e2z * s2);
}

struct RkSlot {
  float2* sol;
  float2* acc;
  float2* xn;
  float h, dt, ca, cb;
};

template <int OP>
__device__ __forceinline__ void rk_apply(const RkSlot& a, long long o, float2 x, float2 R) {
  if constexpr (OP == OP_RHS) {
    a.acc[o] = R;
  } else if constexpr (OP == OP_RK4_FIRST) {
    a.acc[o] = make_float2(R.x / 6.f, R.y / 6.f);
    a.xn[o] = make_float2(x.x + a.h * R.x, x.y + a.h * R.y);
  } else if constexpr (OP == OP_RK4_MID) {
    const float2 s = a.sol[o], q = a.acc[o];
    a.acc[o] = make_float2(q.x + R.x / 3.f, q.y + R.y / 3.f);
    a.xn[o] = make_float2(s.x + a.h * R.x, s.y + a.h * R.y);
  } else if constexpr (OP == OP_RK4_LAST) {
    const float2 s = a.sol[o], q = a.acc[o];
    const float2 tot = make_float2(q.x + R.x / 6.f, q.y + R.y / 6.f);
    a.sol[o] = make_float2(s.x + a.dt * tot.x, s.y + a.dt * tot.y);
  } else if constexpr (OP == OP_LS_FIRST) {
    const float2 du = make_float2(a.dt * R.x, a.dt * R.y);
    a.acc[o] = du;
    a.xn[o] = make_float2(x.x + a.cb * du.x, x.y + a.cb * du.y);
  } else if constexpr (OP == OP_LS) {
    const float2 q = a.acc[o];
    const float2 du = make_float2(a.ca * q.x + a.dt * R.x, a.ca * q.y + a.dt * R.y);
    a.acc[o] = du;
    a.xn[o] = make_float2(x.x + a.cb * du.x, x.y + a.cb * du.y);
  }
}

// grid (ceil(kx / blockDim.x), k2, k2): one thread per retained mode, no index division.
// HD: the hydrodynamic form (three fields, five product planes; B is neither read nor written).
template <int OP, bool FORCED, bool VPEN, bool HD = false>
__global__ void __launch_bounds__(256) rk_epilogue_kernel(RkArgs a, Geom geo, BatchRef br) {
  constexpr int NF = HD ? 3 : 6;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= geo.kx) return;
  const int inst = blockIdx.z / geo.k2;
  if (inst >= *br.count) return;
  const int slot = br.list[inst];
  const int jy = blockIdx.y, jz = blockIdx.z - inst * geo.k2;
  const long long fs = a.fs;
  const long long i = ((long long)jz * geo.k2 + jy) * geo.kxp + x;
  const SlotParams sp = a.sp[slot];
  const long long so = slot * a.stI;
  RkSlot rs{a.sol + so, a.acc + so, a.xn + so, a.hf * sp.dt, sp.dt, a.ca, a.cb};
  const float2* X = a.X + so;
  const float2* prod = a.prod + slot * a.prodI;
  const float kxv = geo.kscale * (float)x;
  const float kyv = geo.kscale * (float)signed_of_kept(geo, jy);
  const float kzv = geo.kscale * (float)signed_of_kept(geo, jz);
  const float k2 = kxv * kxv + kyv * kyv + kzv * kzv;
  float2 p[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) p[q] = (HD && q >= 5) ? make_float2(0.f, 0.f) : cscale(__ldcs(prod + q * fs + i), a.pscale);
  float2 xv[6], xd[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) xv[c] = xd[c] = c < NF ? X[c * fs + i] : make_float2(0.f, 0.f);
  if (x == 0) {
    const long long p = (long long)jz * geo.k2 + jy, pl = (long long)geo.k2 * geo.k2;
    const float2* H = a.H + slot * a.hI;
#pragma unroll
    for (int c = 0; c < NF; ++c) xd[c] = H[c * pl + p];
  }
  const float2 dxz = p[0], dyz = p[1], txy = p[2], txz = p[3], tyz = p[4];
  const float2 axy = p[5], axz = p[6], ayz = p[7];
  float2 Vx, Vy, Vz;
  Vx.x = kxv * dxz.x + kyv * txy.x + kzv * txz.x;  Vx.y = kxv * dxz.y + kyv * txy.y + kzv * txz.y;
  Vy.x = kxv * txy.x + kyv * dyz.x + kzv * tyz.x;  Vy.y = kxv * txy.y + kyv * dyz.y + kzv * tyz.y;
  Vz.x = kxv * txz.x + kyv * tyz.x;                Vz.y = kxv * txz.y + kyv * tyz.y;
  const float ik2 = k2 > 0.f ? 1.0f / k2 : 0.f;
  const float kvx = (kxv * Vx.x + kyv * Vy.x + kzv * Vz.x) * ik2;
  const float kvy = (kxv * Vx.y + kyv * Vy.y + kzv * Vz.y) * ik2;
  float2 nl[6];
  nl[0] = make_float2(-(Vx.y - kxv * kvy), Vx.x - kxv * kvx);
  nl[1] = make_float2(-(Vy.y - kyv * kvy), Vy.x - kyv * kvx);
  nl[2] = make_float2(-(Vz.y - kzv * kvy), Vz.x - kzv * kvx);
  // W = i k x E with E = (Ayz, -Axz, Axy): Wx = i(ky Axy + kz Axz), Wy = i(kz Ayz - kx Axy), Wz = -i(kx Axz + ky Ayz)
  const float2 wx = make_float2(kyv * axy.x + kzv * axz.x, kyv * axy.y + kzv * axz.y);
  const float2 wy = make_float2(kzv * ayz.x - kxv * axy.x, kzv * ayz.y - kxv * axy.y);
  const float2 wz = make_float2(-(kxv * axz.x + kyv * ayz.x), -(kxv * axz.y + kyv * ayz.y));
  nl[3] = make_float2(-wx.y, wx.x);
  nl[4] = make_float2(-wy.y, wy.x);
  nl[5] = make_float2(-wz.y, wz.x);
  const float du = -sp.nu * k2, db = -sp.eta * k2;
  float2 R[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const float dk = c < 3 ? du : db;
    R[c] = make_float2(nl[c].x + dk * xd[c].x, nl[c].y + dk * xd[c].y);
  }
  if constexpr (VPEN) {
    // VP_UᵢUpdate! / VP_BᵢUpdate! (src/Solver/VPSolver.jl:20-58): N_a += -(δ_aj - k_a k_j / k^2) F_j
    // with F = rfft(chi / eta (u - U0)) (and chi / eta (B - B0)), eta = 13 dt / 7, 1/k^2 = 0 at k = 0
    const float sc = -a.vscale * 7.f / (13.f * sp.dt);
    float2 F[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) F[q] = cscale(__ldcs(prod + (8 + q) * fs + i), sc);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float2 f0 = F[3 * h], f1 = F[3 * h + 1], f2 = F[3 * h + 2];
      const float px = (kxv * f0.x + kyv * f1.x + kzv * f2.x) * ik2;
      const float py = (kxv * f0.y + kyv * f1.y + kzv * f2.y) * ik2;
      R[3 * h] = make_float2(R[3 * h].x + f0.x - kxv * px, R[3 * h].y + f0.y - kxv * py);
      R[3 * h + 1] = make_float2(R[3 * h + 1].x + f1.x - kyv * px, R[3 * h + 1].y + f1.y - kyv * py);
      R[3 * h + 2] = make_float2(R[3 * h + 2].x + f2.x - kzv * px, R[3 * h + 2].y + f2.y - kzv * py);
    }
  }
  if (FORCED && sp.fA != 0.f) {  // addforcing!: N[u] += F, then the kx = 0 plane keeps its real part
    const unsigned long long call = 8ull * (unsigned long long)a.step[slot] + (unsigned long long)a.stage;
    const unsigned long long key = mix64(sp.fseed ^ mix64(call));
    const int nkr = geo.n / 2 + 1;
    const unsigned long long index =
        (unsigned long long)x + (unsigned long long)nkr * ((unsigned long long)freq_of_kept(geo, jy) +
                                                            (unsigned long long)geo.n * freq_of_kept(geo, jz));
    float2 F[3];
    a99_force(sp, key, index, kxv, kyv, kzv, F);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      R[c] = make_float2(R[c].x + F[c].x, R[c].y + F[c].y);
      if (x == 0) R[c].y = 0.f;
    }
  }
  if (!HD && a.hydro) {  // B = 0: only roundoff of the paired x-row transforms would feed it
#pragma unroll
    for (int c = 3; c < 6; ++c) R[c] = make_float2(0.f, 0.f);
  }
#pragma unroll
  for (int c = 0; c < NF; ++c) rk_apply<OP>(rs, c * fs + i, xv[c], R[c]);
}

// Hermitian part of the kx = 0 plane of the six fields: H(k) = (X(k) + conj X(-k)) / 2, with
// X(-k) = 0 when -k is in the alias band.  The reference's diffusion term is computed from the
// re-transformed physical field, rfft(irfft(X)), which is exactly this on the kx = 0 plane.
__global__ void herm_kx0_kernel(const float2* __restrict__ Xpool, float2* __restrict__ Hpool, Geom geo, long long fs,
                                long long stI, long long hI, BatchRef br) {
  // grid (ceil(K2 / blockDim.x), K2, cap): one thread per (ky', kz') of one instance, all six
  // fields in flight
  const int jy = blockIdx.x * blockDim.x + threadIdx.x;
  const int jz = blockIdx.y;
  const int inst = blockIdx.z;
  if (jy >= geo.k2 || inst >= *br.count) return;
  const int slot = br.list[inst];
  const float2* X = Xpool + slot * stI;
  float2* H = Hpool + slot * hI;
  const int py = kept_of_signed(geo, -signed_of_kept(geo, jy));
  const int pz = kept_of_signed(geo, -signed_of_kept(geo, jz));
  const bool partner = py >= 0 && pz >= 0;
  const long long own = ((long long)jz * geo.k2 + jy) * geo.kxp;
  const long long par = partner ? ((long long)pz * geo.k2 + py) * geo.kxp : own;
  const long long pl = (long long)geo.k2 * geo.k2;
  float2 xk[6], xp[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    xk[c] = X[c * fs + own];
    xp[c] = X[c * fs + par];
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const float2 q = partner ? xp[c] : make_float2(0.f, 0.f);
    H[c * pl + (long long)jz * geo.k2 + jy] = make_float2(0.5f * (xk[c].x + q.x), 0.5f * (xk[c].y - q.y));
  }
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
