// Register-resident mixed-radix FFT building blocks for the MHD pass kernels (sm_103a).
//
// A length-N transform is spread over G cooperating threads that each hold V = N/G complex
// values in registers.  N = R0*R1*R2 (R2 may be 1) and every radix divides V, so each stage is
// V/R_s small DFTs per thread, done fully unrolled in registers (Cooley-Tukey codelets built from
// radix-2/3/4 butterflies, in the paired FP32 instructions of the sm_100 family where the inputs
// are run-time values).  Between stages the values are exchanged through shared memory; the
// stage twiddles W_N^j come from a per-size table computed in double precision on the host.
//
// Index conventions (DIR = -1 forward, +1 inverse, X[k] = sum_n x[n] exp(DIR*2*pi*i*n*k/N)):
//   input  n = n0*(R1*R2) + n1*R2 + n2        (stage-1 label l1 = n1*R2 + n2 = n mod R1*R2)
//   output k = k0 + k1*R0 + k2*R0*R1          (last-stage label lF = k mod (N/RF))
// A thread with lane g owns labels l = g + G*d, d = 0..V/R-1, for every stage, so a transform
// with radices (R0,R1,R2) leaves its outputs exactly where a transform with the reversed radices
// (R2,R1,R0) expects its inputs: the physical-space product step between an inverse and a
// forward row transform needs no data movement at all.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mhdgb {

// ------------------------------------------------------------------------------------------
// Compile-time trigonometry (Taylor series in double, argument reduced to [-pi, pi]) used only
// to build the constant twiddles inside the small register codelets.
// ------------------------------------------------------------------------------------------
__host__ __device__ constexpr double k_pi() { return 3.141592653589793238462643383279502884; }

__host__ __device__ constexpr double taylor_sin(double x) {
  double term = x, sum = x;
  for (int i = 1; i < 28; ++i) {
    term *= -x * x / ((2.0 * i) * (2.0 * i + 1.0));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double taylor_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int i = 1; i < 28; ++i) {
    term *= -x * x / ((2.0 * i - 1.0) * (2.0 * i));
    sum += term;
  }
  return sum;
}
// cos / sin of 2*pi*j/R with exact values on the axes.
__host__ __device__ constexpr double unit_cos(int j, int R) {
  j %= R; if (j < 0) j += R;
  if (4 * j == 0) return 1.0;
  if (4 * j == R || 4 * j == 3 * R) return 0.0;
  if (2 * j == R) return -1.0;
  int jj = (2 * j > R) ? j - R : j;
  return taylor_cos(2.0 * k_pi() * jj / R);
}
__host__ __device__ constexpr double unit_sin(int j, int R) {
  j %= R; if (j < 0) j += R;
  if (j == 0 || 2 * j == R) return 0.0;
  if (4 * j == R) return 1.0;
  if (4 * j == 3 * R) return -1.0;
  int jj = (2 * j > R) ? j - R : j;
  return taylor_sin(2.0 * k_pi() * jj / R);
}

template <int R>
struct TwTab {
  float c[R];
  float s[R];
  __host__ __device__ constexpr TwTab() : c(), s() {
    for (int j = 0; j < R; ++j) {
      c[j] = (float)unit_cos(j, R);
      s[j] = (float)unit_sin(j, R);
    }
  }
};

// ------------------------------------------------------------------------------------------
// Complex helpers
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// a * (c + i*DIR*s)
template <int DIR>
__device__ __forceinline__ float2 cmul_cs(float2 a, float c, float s) {
  const float ds = DIR * s;
  return make_float2(fmaf(a.x, c, -a.y * ds), fmaf(a.x, ds, a.y * c));
}
// a * (DIR * i)
template <int DIR>
__device__ __forceinline__ float2 cmul_diri(float2 a) {
  return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// Paired FP32 arithmetic of the sm_100 family: one instruction updates both components of a
// complex value, each component rounded exactly like the scalar operation.  The codelets below
// use it wherever their inputs are run-time values (PK = true); a stage whose inputs include
// compile-time zeros (the pruned first stage of an inverse transform) keeps the scalar forms,
// which fold those zeros away.
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b: b * (-1) is exact, so the fused form rounds once, like a - b
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
// a + m * b, componentwise, one rounding per component
__device__ __forceinline__ float2 paxpy(float2 b, float2 m, float2 a) { return __ffma2_rn(b, m, a); }
template <bool PK>
__device__ __forceinline__ float2 kadd(float2 a, float2 b) { return PK ? padd(a, b) : cadd(a, b); }
template <bool PK>
__device__ __forceinline__ float2 ksub(float2 a, float2 b) { return PK ? psub(a, b) : csub(a, b); }
// (a.y - b.y, a.x - b.x): the difference with its components exchanged, as two scalar
// subtractions that write the pair in exchanged order (no register moves)
__device__ __forceinline__ float2 csub_swapped(float2 a, float2 b) { return make_float2(a.y - b.y, a.x - b.x); }

// ------------------------------------------------------------------------------------------
// Small in-register DFT codelets: x[0..R) in place, natural-order output.
// ------------------------------------------------------------------------------------------
template <int R>
struct FirstFactor {
  static constexpr int value = (R % 4 == 0 && R != 4) ? 4 : (R % 2 == 0 && R != 2) ? 2 : (R % 3 == 0 && R != 3) ? 3 : R;
};

template <int R, int DIR, bool PK = true>
struct Dft;

template <int DIR, bool PK>
struct Dft<1, DIR, PK> {
  template <int S, int O, int A>
  __device__ __forceinline__ static void run(float2 (&)[A]) {}
};

template <int DIR, bool PK>
struct Dft<2, DIR, PK> {
  // operates on x[O], x[O+S]
  template <int S, int O, int A>
  __device__ __forceinline__ static void run(float2 (&x)[A]) {
    float2 a = x[O], b = x[O + S];
    x[O] = kadd<PK>(a, b);
    x[O + S] = ksub<PK>(a, b);
  }
};

template <int DIR, bool PK>
struct Dft<3, DIR, PK> {
  template <int S, int O, int A>
  __device__ __forceinline__ static void run(float2 (&x)[A]) {
    const float h = 0.86602540378443864676f;  // sqrt(3)/2
    float2 x0 = x[O], x1 = x[O + S], x2 = x[O + 2 * S];
    if constexpr (PK) {
      // X1,2 = t2 +- DIR i h (x1 - x2) = t2 + (-+DIR h (x1-x2).y, +-DIR h (x1-x2).x)
      const float2 t1 = padd(x1, x2);
      const float2 t2 = paxpy(t1, make_float2(-0.5f, -0.5f), x0);
      const float2 ds = csub_swapped(x1, x2);
      x[O] = padd(x0, t1);
      x[O + S] = paxpy(ds, make_float2(-DIR * h, DIR * h), t2);
      x[O + 2 * S] = paxpy(ds, make_float2(DIR * h, -DIR * h), t2);
    } else {
      float2 t1 = cadd(x1, x2);
      float2 t2 = make_float2(fmaf(-0.5f, t1.x, x0.x), fmaf(-0.5f, t1.y, x0.y));
      float2 d = csub(x1, x2);
      float2 t3 = cmul_diri<DIR>(cscale(d, h));
      x[O] = cadd(x0, t1);
      x[O + S] = cadd(t2, t3);
      x[O + 2 * S] = csub(t2, t3);
    }
  }
};

template <int DIR, bool PK>
struct Dft<4, DIR, PK> {
  template <int S, int O, int A>
  __device__ __forceinline__ static void run(float2 (&x)[A]) {
    float2 x0 = x[O], x1 = x[O + S], x2 = x[O + 2 * S], x3 = x[O + 3 * S];
    if constexpr (PK) {
      // X1,3 = b +- DIR i e with e = x1 - x3: (b.x -+ DIR e.y, b.y +- DIR e.x)
      const float2 a = padd(x0, x2), b = psub(x0, x2), c = padd(x1, x3);
      const float2 es = csub_swapped(x1, x3);
      x[O] = padd(a, c);
      x[O + 2 * S] = psub(a, c);
      x[O + S] = paxpy(es, make_float2((float)-DIR, (float)DIR), b);
      x[O + 3 * S] = paxpy(es, make_float2((float)DIR, (float)-DIR), b);
    } else {
      float2 a = cadd(x0, x2), b = csub(x0, x2);
      float2 c = cadd(x1, x3), d = cmul_diri<DIR>(csub(x1, x3));
      x[O] = cadd(a, c);
      x[O + 2 * S] = csub(a, c);
      x[O + S] = cadd(b, d);
      x[O + 3 * S] = csub(b, d);
    }
  }
};

// Radix 8 in paired arithmetic: X[k] = E[k] + W^k O[k], X[k+4] = E[k] - W^k O[k] with E, O the
// 4-point DFTs of the even and odd inputs and W = exp(DIR 2 pi i / 8).  The odd-side products
// W^k O[k] are formed componentwise before the last fused step:
//   W^1 O = c (O.x - DIR O.y, O.y + DIR O.x),   W^3 O = c (-O.x - DIR O.y, DIR O.x - O.y),
//   W^2 O = DIR i O,  c = sqrt(1/2).
template <int DIR>
struct Dft<8, DIR, true> {
  template <int S, int O, int A>
  __device__ __forceinline__ static void run(float2 (&x)[A]) {
    constexpr float c = 0.70710678118654752440f;
    float2 e[4] = {x[O], x[O + 2 * S], x[O + 4 * S], x[O + 6 * S]};
    float2 o[4] = {x[O + S], x[O + 3 * S], x[O + 5 * S], x[O + 7 * S]};
    Dft<4, DIR, true>::template run<1, 0>(e);
    Dft<4, DIR, true>::template run<1, 0>(o);
    x[O] = padd(e[0], o[0]);
    x[O + 4 * S] = psub(e[0], o[0]);
    const float2 u1 = make_float2(o[1].x - DIR * o[1].y, o[1].y + DIR * o[1].x);
    x[O + S] = paxpy(u1, make_float2(c, c), e[1]);
    x[O + 5 * S] = paxpy(u1, make_float2(-c, -c), e[1]);
    const float2 o2s = make_float2(o[2].y, o[2].x);
    x[O + 2 * S] = paxpy(o2s, make_float2((float)-DIR, (float)DIR), e[2]);
    x[O + 6 * S] = paxpy(o2s, make_float2((float)DIR, (float)-DIR), e[2]);
    const float2 u3 = make_float2(-o[3].x - DIR * o[3].y, DIR * o[3].x - o[3].y);
    x[O + 3 * S] = paxpy(u3, make_float2(c, c), e[3]);
    x[O + 7 * S] = paxpy(u3, make_float2(-c, -c), e[3]);
  }
};

// Composite R = P*Q (P = FirstFactor): x[n], n = Q*a + b;  X[k], k = ka + P*kb.
// The element set is x[O + S*i], i = 0..R-1 (strided view inside a register array).
template <int R, int DIR, bool PK>
struct Dft {
  static constexpr int P = FirstFactor<R>::value;
  static constexpr int Q = R / P;
  static_assert(P * Q == R && P > 1 && Q > 1, "unsupported radix");

  template <int S, int O, int A>
  __device__ __forceinline__ static void run(float2 (&x)[A]) {
    constexpr TwTab<R> tw{};
    // step 1: Q DFTs of size P over a (elements O + S*(Q*a + b))
#pragma unroll
    for (int b = 0; b < Q; ++b) {
      float2 t[P];
#pragma unroll
      for (int a = 0; a < P; ++a) t[a] = x[O + S * (Q * a + b)];
      Dft<P, DIR, PK>::template run<1, 0>(t);
      // twiddle W_R^{b*ka}; multiples of a quarter turn are exact sign/swap operations
#pragma unroll
      for (int ka = 0; ka < P; ++ka) {
        const int e = (b * ka) % R;
        if (e != 0) {
          if ((4 * e) % R == 0) {
            const int q = (4 * e) / R;  // W = (DIR i)^q
            if (q == 2) t[ka] = make_float2(-t[ka].x, -t[ka].y);
            else if (q == 1) t[ka] = cmul_diri<DIR>(t[ka]);
            else t[ka] = cmul_diri<-DIR>(t[ka]);
          } else {
            t[ka] = cmul_cs<DIR>(t[ka], tw.c[e], tw.s[e]);
          }
        }
        x[O + S * (Q * ka + b)] = t[ka];
      }
    }
    // step 2: P DFTs of size Q over b (elements O + S*(Q*ka + b)), output k = ka + P*kb
    float2 out[R];
#pragma unroll
    for (int ka = 0; ka < P; ++ka) {
      float2 t[Q];
#pragma unroll
      for (int b = 0; b < Q; ++b) t[b] = x[O + S * (Q * ka + b)];
      Dft<Q, DIR, PK>::template run<1, 0>(t);
#pragma unroll
      for (int kb = 0; kb < Q; ++kb) out[ka + P * kb] = t[kb];
    }
#pragma unroll
    for (int k = 0; k < R; ++k) x[O + S * k] = out[k];
  }
};

// Run DFT-R on each of the D = A/R contiguous groups of a register array.
template <int R, int DIR, bool PK, int A>
__device__ __forceinline__ void dft_groups(float2 (&x)[A]) {
  static_assert(A % R == 0, "radix must divide the per-thread count");
#pragma unroll
  for (int d = 0; d < A / R; ++d) {
    float2 t[R];
#pragma unroll
    for (int r = 0; r < R; ++r) t[r] = x[d * R + r];
    Dft<R, DIR, PK>::template run<1, 0>(t);
#pragma unroll
    for (int r = 0; r < R; ++r) x[d * R + r] = t[r];
  }
}

// ------------------------------------------------------------------------------------------
// Multi-stage thread-distributed plan.
// ------------------------------------------------------------------------------------------
template <int N_, int G_, int R0_, int R1_, int R2_ = 1>
struct Plan {
  static constexpr int N = N_, G = G_, V = N_ / G_;
  static constexpr int R0 = R0_, R1 = R1_, R2 = R2_;
  static_assert(R0 * R1 * R2 == N, "radices must multiply to N");
  static_assert(V * G == N, "G must divide N");
  static_assert(V % R0 == 0 && V % R1 == 0 && V % R2 == 0, "radices must divide V");
  static constexpr int STAGES = (R2 == 1) ? 2 : 3;
  static constexpr int RF = (R2 == 1) ? R1 : R2;      // last radix
  static constexpr int LI = N / R0;                    // input label count
  static constexpr int LF = N / RF;                    // output label count
  static constexpr int DI = V / R0;                    // input slots per thread
  static constexpr int DF = V / RF;                    // output slots per thread
  // Shared-memory exchange strides.  Padding spreads the 8-byte words a half-warp touches over the
  // 16 bank pairs when consecutive lanes hold consecutive labels (row layouts): stage-2 readers
  // of one instruction differ in k0 (stride E1S) and n2 (stride 1), so E1S = 16/R0 (mod 16)
  // interleaves them; stage-3 writers differ in k0 (stride 1) and n2 (stride E2S), so E2S = R0.
  static constexpr bool kPow2R0 = R0 <= 16 && (16 % R0) == 0;
  static constexpr int P1 = kPow2R0 ? ((16 / R0) % 16 - (R1 * R2) % 16 + 32) % 16 : 1;
  static constexpr int E1S = R1 * R2 + P1;
  static constexpr int P2 = kPow2R0 ? ((R0 % 16) - (R0 * R1) % 16 + 32) % 16 : 0;
  static constexpr int E2S = R0 * R1 + P2;
  static constexpr int SMEM1 = R0 * E1S;              // words used by exchange 1
  static constexpr int SMEM2 = R2 * E2S;              // words used by exchange 2
  static constexpr int SMEM = (STAGES == 3 && SMEM2 > SMEM1) ? SMEM2 : SMEM1;
};

// The same plan without bank padding: column layouts put the TX columns of a tile in consecutive
// words, so any exchange address pattern is conflict-free and the exchange fits in N*TX words.
template <class P>
struct Unpadded : P {
  static constexpr int E1S = P::R1 * P::R2;
  static constexpr int E2S = P::R0 * P::R1;
  static constexpr int SMEM = P::N;
};

// Reversed-radix plan: its input layout equals the output layout of P.
template <class P>
struct Reverse;
template <int N, int G, int R0, int R1>
struct Reverse<Plan<N, G, R0, R1, 1>> { using type = Plan<N, G, R1, R0, 1>; };
template <int N, int G, int R0, int R1, int R2>
struct Reverse<Plan<N, G, R0, R1, R2>> { using type = Plan<N, G, R2, R1, R0>; };

__device__ __forceinline__ float2 ldtw(const float2* __restrict__ tw, int j) { return __ldg(tw + j); }

// 16-byte asynchronous global -> shared copy (L2 only) and its group fences.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const unsigned int d = (unsigned int)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND) : "memory"); }

// Stage twiddles of a plan, laid out in the order the lanes of a warp read them, so one warp
// load touches one or two 128-byte lines:
//   tw[n1*R0 + k0]                    = W_N^{(n1 k0 mod R0R1) R2}       (before stage 2)
//   tw[R0R1 + k1*R0R2 + k0 + R0*n2]   = W_N^{n2 (k0 + R0 k1) mod N}     (before stage 3)
// with W_N^j = cos(2 pi j/N) + i sin(2 pi j/N); the transform direction conjugates on use.
template <class P>
struct PlanTw {
  static constexpr int T2 = P::R0 * P::R1;
  static constexpr int SIZE = T2 + (P::R2 > 1 ? P::N : 0);
};

// Executes stages of plan P on NT independent transforms held as v[t][V] by this thread.
// Shared memory word address of logical element a for transform t is  buf[t*TS + a*STR + OFF].
// SYNC() must be a barrier over every thread that shares buf.  tw is the plan's PlanTw table.
// TWS: tw lies in shared memory (plain loads).
// PK1: the first stage in paired arithmetic; false where its inputs hold compile-time zeros
// (pruned alias-band inputs), which fold away only in scalar code.
// Input: v[t][d*R0 + n0] = x[l1 + LI*n0] with l1 = g + G*d.
// Output: v[t][d*RF + e] = X[lF + LF*e] with lF = g + G*d.
template <class P, int DIR, int NT, int TS, int STR, bool PK1 = true, bool TWS = false, class SyncF>
__device__ __forceinline__ void fft_run(float2 (&v)[NT][P::V], float2* buf, int off, int g,
                                        const float2* __restrict__ tw, SyncF SYNC) {
  constexpr int V = P::V, G = P::G, R0 = P::R0, R1 = P::R1, R2 = P::R2;
  // ---- stage 1: DFT-R0 over n0
#pragma unroll
  for (int t = 0; t < NT; ++t) dft_groups<R0, DIR, PK1>(v[t]);
  // ---- exchange 1: write Y1[k0; l1] at k0*E1S + l1
#pragma unroll
  for (int t = 0; t < NT; ++t)
#pragma unroll
    for (int d = 0; d < V / R0; ++d) {
      const int l1 = g + G * d;
#pragma unroll
      for (int k0 = 0; k0 < R0; ++k0) buf[t * TS + (k0 * P::E1S + l1) * STR + off] = v[t][d * R0 + k0];
    }
  SYNC();
  // ---- read for stage 2: label l2 = k0 + R0*n2, elements n1
#pragma unroll
  for (int d = 0; d < V / R1; ++d) {
    const int l2 = g + G * d;
    const int k0 = l2 % R0, n2 = l2 / R0;
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) {
      float2 w = make_float2(1.f, 0.f);
      if (n1 != 0) w = TWS ? tw[n1 * R0 + k0] : ldtw(tw, n1 * R0 + k0);  // W_{R0R1}^{n1 k0}
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        float2 a = buf[t * TS + (k0 * P::E1S + n1 * R2 + n2) * STR + off];
        if (n1 != 0) a = cmul_cs<DIR>(a, w.x, w.y);
        v[t][d * R1 + n1] = a;
      }
    }
  }
  // ---- stage 2: DFT-R1 over n1
#pragma unroll
  for (int t = 0; t < NT; ++t) dft_groups<R1, DIR, true>(v[t]);
  if constexpr (P::STAGES == 3) {
    SYNC();  // every thread finished reading exchange 1
    // twiddle W_N^{n2 (k0 + R0 k1)} and exchange 2: write at n2*E2S + l3, l3 = k0 + R0*k1
#pragma unroll
    for (int d = 0; d < V / R1; ++d) {
      const int l2 = g + G * d;
      const int k0 = l2 % R0, n2 = l2 / R0;
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) {
        const int l3 = k0 + R0 * k1;
        const int j = PlanTw<P>::T2 + k1 * (R0 * R2) + l2;
        const float2 w = TWS ? tw[j] : ldtw(tw, j);  // W_N^{n2 l3}
#pragma unroll
        for (int t = 0; t < NT; ++t) {
          const float2 a = cmul_cs<DIR>(v[t][d * R1 + k1], w.x, w.y);
          buf[t * TS + (n2 * P::E2S + l3) * STR + off] = a;
        }
      }
    }
    SYNC();
#pragma unroll
    for (int t = 0; t < NT; ++t)
#pragma unroll
      for (int d = 0; d < V / R2; ++d) {
        const int l3 = g + G * d;
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) v[t][d * R2 + n2] = buf[t * TS + (n2 * P::E2S + l3) * STR + off];
      }
#pragma unroll
    for (int t = 0; t < NT; ++t) dft_groups<R2, DIR, true>(v[t]);
  }
}

}  // namespace mhdgb
