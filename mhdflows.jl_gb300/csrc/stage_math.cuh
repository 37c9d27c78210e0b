// Spectral right-hand side of one retained mode and the Runge-Kutta stage update (sm_103a):
// templates and inline functions only (the spectral epilogue kernel is in step_kernels.cuh).
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


// The stress and induction sums of one retained mode (already scaled to the reference's rfft):
// V = (kx Dxz + ky Txy + kz Txz, kx Txy + ky Dyz + kz Tyz, kx Txz + ky Tyz) and
// W = k x E with E = (Ayz, -Axz, Axy): Wx = ky Axy + kz Axz, Wy = kz Ayz - kx Axy,
// Wz = -(kx Axz + ky Ayz).  The nonlinear terms are i (V - k (k.V)/k^2) and i W.
struct ModeSums {
  float2 Vx, Vy, Vz, Wx, Wy, Wz;
};

// The right-hand side of one retained mode (jz, jy, x) of a slot from its sums, the stage state
// (the kx = 0 plane diffuses its Hermitian part), volume penalisation, forcing, and the stage
// update.  i is the mode's offset in a compact field; prod the slot's product planes (VPEN only).
template <int OP, bool FORCED, bool VPEN, bool HD>
__device__ __forceinline__ void finish_mode(const RkArgs& a, const Geom& geo, int slot, int jz, int jy, int x, long long i,
                                            float kxv, float kyv, float kzv, const ModeSums& m, const float2* prod) {
  constexpr int NF = HD ? 3 : 6;
  const long long fs = a.fs;
  const SlotParams sp = a.sp[slot];
  const long long so = slot * a.stI;
  RkSlot rs{a.sol + so, a.acc + so, a.xn + so, a.hf * sp.dt, sp.dt, a.ca, a.cb};
  const float2* X = a.X + so;
  const float k2 = kxv * kxv + kyv * kyv + kzv * kzv;
  float2 xv[6], xd[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) xv[c] = xd[c] = c < NF ? X[c * fs + i] : make_float2(0.f, 0.f);
  if (x == 0) {
    const long long p = (long long)jz * geo.k2 + jy, pl = (long long)geo.k2 * geo.k2;
    const float2* H = a.H + slot * a.hI;
#pragma unroll
    for (int c = 0; c < NF; ++c) xd[c] = H[c * pl + p];
  }
  const float ik2 = k2 > 0.f ? 1.0f / k2 : 0.f;
  const float kvx = (kxv * m.Vx.x + kyv * m.Vy.x + kzv * m.Vz.x) * ik2;
  const float kvy = (kxv * m.Vx.y + kyv * m.Vy.y + kzv * m.Vz.y) * ik2;
  float2 nl[6];
  nl[0] = make_float2(-(m.Vx.y - kxv * kvy), m.Vx.x - kxv * kvx);
  nl[1] = make_float2(-(m.Vy.y - kyv * kvy), m.Vy.x - kyv * kvx);
  nl[2] = make_float2(-(m.Vz.y - kzv * kvy), m.Vz.x - kzv * kvx);
  nl[3] = make_float2(-m.Wx.y, m.Wx.x);
  nl[4] = make_float2(-m.Wy.y, m.Wy.x);
  nl[5] = make_float2(-m.Wz.y, m.Wz.x);
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
    // MHD: the six penalty planes are 8..13 (u x, u y, u z, B x, B y, B z), n^3 times the
    // reference's rfft; the hydrodynamic form keeps u in the spare product slots 6, 7, 5 (x, y, z)
    // at the products' scale, n^6
    const float sc = -(HD ? a.pscale : a.vscale) * 7.f / (13.f * sp.dt);
    float2 F[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const int plane = HD ? (q == 0 ? 6 : q == 1 ? 7 : 5) : 8 + q;
      F[q] = (HD && q >= 3) ? make_float2(0.f, 0.f) : cscale(__ldcs(prod + plane * fs + i), sc);
    }
#pragma unroll
    for (int h = 0; h < (HD ? 1 : 2); ++h) {
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

}  // namespace mhdgb
