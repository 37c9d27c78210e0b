// Split-precision tensor-core x rows (precision forms MHD_PREC_SPLIT_FP16 / MHD_PREC_SPLIT_BF16).
//
// The fused x-row pass (3 inverse c2r pairs -> 8 products -> 4 forward r2c pairs) with every
// length-N transform computed as two small dense complex DFT matrix products on the tensor cores
// (mma.sync m16n8k16, 16-bit operands, FP32 accumulation).  N = 16 Q, Q in {8, 16, 32}.
//
// Inverse, n = Q n1 + n2, k = k1 + 16 k2:
//   stage A  Y[k1][n2]  = sum_n1 F16[k1][n1] x[Q n1 + n2]           A = F16 (constant), B = data
//   twiddle  Y'[k1][n2] = Y[k1][n2] W_N^{n2 k1}
//   stage B  X[k1][k2]  = sum_n2 Y'[k1][n2] FQ[n2][k2]              A = data, B = FQ (constant)
// Forward, input at the inverse's output positions n = r + 16 c, read as n = 16 a + b:
//   stage A' Y[k1][b]   = sum_a FQ*[k1][a] x[16 a + b]              A = FQ* (constant), B = data^T
//   twiddle  Y'[k1][b]  = Y[k1][b] W_N^{-b k1}
//   stage B' X[k1+Q k2] = sum_b Y'[k1][b] F16*[b][k2]               A = data, B = F16* (constant)
// Complex products use the real embedding [[Re,-Im],[Im,Re]] of the left factor (or
// [[Re,Im],[-Im,Re]] of the right one).  The accumulator fragment of one stage is the A operand
// of the next (the m16n8 C layout of two adjacent n-tiles is the m16k16 A layout), and the
// inverse's output fragments read as the forward's B operand transposed, so a row never leaves
// the registers of its warp between the input load and the forward output.
//
// Precision: each 16-bit operand v is split v = hi + lo (hi = rn(v), lo = rn(v - hi)) and a
// product is hi*hi + hi*lo + lo*hi (the lo*lo term is below FP32 rounding for FP16 and is
// dropped for BF16 as well).  FP16 operands are scaled per transform by a power of two so that
// the largest input component is 2^10 (no overflow through a 16- or 32-point stage); BF16 needs
// no scaling.  The constant fragments (hi, lo) and the twiddles are built once per device by
// tc_tables_kernel and read through the read-only cache.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "passes.cuh"

namespace mhdgb {

enum SplitKind : int { SPLIT_F16 = 0, SPLIT_BF16 = 1 };

template <int KIND>
__device__ __forceinline__ uint32_t pack16(float a, float b) {
  if constexpr (KIND == SPLIT_F16) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  } else {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  }
}
template <int KIND>
__device__ __forceinline__ float2 unpack16(uint32_t u) {
  if constexpr (KIND == SPLIT_F16) {
    __half2 h = *reinterpret_cast<__half2*>(&u);
    return __half22float2(h);
  } else {
    __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&u);
    return __bfloat1622float2(h);
  }
}
// (a, b) -> hi and lo 16-bit pairs.  FP16: hi keeps the leading 11 significant bits of each
// value (a mask, so hi converts exactly and no half -> float conversion is needed) and lo is the
// rounded remainder; BF16: hi is the rounded value, unpacked by a shift.
template <int KIND>
__device__ __forceinline__ void split_pair(float a, float b, uint32_t& hi, uint32_t& lo) {
  if constexpr (KIND == SPLIT_F16) {
    const float ah = __uint_as_float(__float_as_uint(a) & 0xffffe000u);
    const float bh = __uint_as_float(__float_as_uint(b) & 0xffffe000u);
    hi = pack16<KIND>(ah, bh);
    lo = pack16<KIND>(a - ah, b - bh);
  } else {
    hi = pack16<KIND>(a, b);
    const float ah = __uint_as_float(hi << 16), bh = __uint_as_float(hi & 0xffff0000u);
    lo = pack16<KIND>(a - ah, b - bh);
  }
}

template <int KIND>
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  if constexpr (KIND == SPLIT_F16) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
  } else {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
  }
}
// d += A B with both factors split, for NB independent B operands (one A): the three terms
// lo*hi, hi*lo, hi*hi go term by term across the NB tiles, so consecutive MMAs are independent
template <int KIND, int NB>
__device__ __forceinline__ void mma3n(float (&d)[NB][4], const uint32_t (&ah)[4], const uint32_t (&al)[4],
                                      const uint32_t (&bh)[NB][2], const uint32_t (&bl)[NB][2]) {
#pragma unroll
  for (int j = 0; j < NB; ++j) mma16816<KIND>(d[j], al, bh[j][0], bh[j][1]);
#pragma unroll
  for (int j = 0; j < NB; ++j) mma16816<KIND>(d[j], ah, bl[j][0], bl[j][1]);
#pragma unroll
  for (int j = 0; j < NB; ++j) mma16816<KIND>(d[j], ah, bh[j][0], bh[j][1]);
}

// ------------------------------------------------------------------------------------------
// Constant tables (32-bit words), per lane so that one lane's fragment is one 8- or 16-byte load:
//   invA  [mt 2][kb 2][hl 2][lane][4]          F16 inverse, left factor          (A fragments)
//   invB  [kb 2Q/16][nt 2Q/8][hl 2][lane][2]   FQ inverse, right factor          (B fragments)
//   fwdA  [mt MQ][kb 2Q/16][hl 2][lane][4]     FQ forward, left factor, MQ = max(2Q/16, 1)
//   fwdB  [kb 2][nt 4][hl 2][lane][2]          F16 forward, right factor
//   twI   [j Q/8][lane][4 complex]             W_N^{+n2 k1} at the inverse stage-A fragment
//   twF   [mr MR][nb 2][lane][4 complex]       W_N^{-b k1} at the forward stage-A' fragment
// (complex twiddles are float pairs, 2 words each)
// ------------------------------------------------------------------------------------------
template <int N>
struct TcLayout {
  static constexpr int Q = N / 16;
  static_assert(N == 16 * Q && (Q == 8 || Q == 16 || Q == 32), "tensor-core rows need N = 16 Q, Q in {8,16,32}");
  static constexpr int KBQ = 2 * Q / 16;                 // k-blocks of a 2Q-wide real embedding
  static constexpr int NTQ = 2 * Q / 8;                  // n-tiles of a 2Q-wide real embedding
  static constexpr int MQ = KBQ;                         // m-tiles of FQ (2Q rows)
  static constexpr int MR = Q >= 16 ? Q / 16 : 1;        // stage-A' m-tiles holding real parts
  static constexpr int INVA = 0;
  static constexpr int INVB = INVA + 2 * 2 * 2 * 32 * 4;
  static constexpr int FWDA = INVB + KBQ * NTQ * 2 * 32 * 2;
  static constexpr int FWDB = FWDA + MQ * KBQ * 2 * 32 * 4;
  static constexpr int TWI = FWDB + 2 * 4 * 2 * 32 * 2;
  static constexpr int TWF = TWI + (Q / 8) * 32 * 8;
  static constexpr int WORDS = TWF + MR * 2 * 32 * 8;
};

// exp(i 2 pi s j / m) in double, rounded to float
__device__ __forceinline__ double2 unit_root(long long j, int m, int s) {
  long long r = ((j % m) + m) % m;
  double sn, cs;
  sincospi(2.0 * (double)r / (double)m, &sn, &cs);
  return make_double2(cs, s * sn);
}

// Entry (row, col) of the real embedding of a DFT matrix F[a][b] = exp(i 2 pi s a b / m):
// left factor L = [[Re, -Im], [Im, Re]], right factor R = [[Re, Im], [-Im, Re]].
__device__ __forceinline__ float embed_entry(int row, int col, int m, int s, bool left) {
  const int a = row % m, b = col % m;
  const bool ri = row >= m, ci = col >= m;
  const double2 w = unit_root((long long)a * b, m, s);
  if (!ri && !ci) return (float)w.x;
  if (ri && ci) return (float)w.x;
  if (left) return (float)(ri ? w.y : -w.y);  // [1][0] = Im, [0][1] = -Im
  return (float)(ri ? -w.y : w.y);            // [1][0] = -Im, [0][1] = Im
}

template <int KIND>
__device__ __forceinline__ void store_split(uint32_t* hi, uint32_t* lo, float a, float b) {
  uint32_t h, l;
  split_pair<KIND>(a, b, h, l);
  *hi = h;
  *lo = l;
}

// One thread per lane slot of every table entry; N, Q from the layout.
template <int N, int KIND>
__global__ void tc_tables_kernel(uint32_t* t) {
  using L = TcLayout<N>;
  constexpr int Q = L::Q;
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, tq = lane & 3;
  const int idx = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);  // fragment index
  // A fragment (m16 x k16, rows mt*16.., cols kb*16..) of a left embedding of size 2m
  auto a_frag = [&](uint32_t* base, int mt, int kb, int m, int s) {
    const int r0 = mt * 16 + g, c0 = kb * 16 + 2 * tq;
    uint32_t* hi = base + lane * 4;
    uint32_t* lo = base + 32 * 4 + lane * 4;
    const int rr[4] = {r0, r0 + 8, r0, r0 + 8};
    const int cc[4] = {c0, c0, c0 + 8, c0 + 8};
    for (int i = 0; i < 4; ++i)
      store_split<KIND>(hi + i, lo + i, embed_entry(rr[i], cc[i], m, s, true), embed_entry(rr[i], cc[i] + 1, m, s, true));
  };
  // B fragment (k16 x n8, rows kb*16.., cols nt*8..) of a right embedding of size 2m
  auto b_frag = [&](uint32_t* base, int kb, int nt, int m, int s) {
    const int k0 = kb * 16 + 2 * tq, n0 = nt * 8 + g;
    uint32_t* hi = base + lane * 2;
    uint32_t* lo = base + 32 * 2 + lane * 2;
    store_split<KIND>(hi + 0, lo + 0, embed_entry(k0, n0, m, s, false), embed_entry(k0 + 1, n0, m, s, false));
    store_split<KIND>(hi + 1, lo + 1, embed_entry(k0 + 8, n0, m, s, false), embed_entry(k0 + 9, n0, m, s, false));
  };
  int f = idx;
  if (f < 4) { a_frag(t + L::INVA + f * 2 * 32 * 4, f / 2, f % 2, 16, +1); return; }
  f -= 4;
  if (f < L::KBQ * L::NTQ) { b_frag(t + L::INVB + f * 2 * 32 * 2, f / L::NTQ, f % L::NTQ, Q, +1); return; }
  f -= L::KBQ * L::NTQ;
  if (f < L::MQ * L::KBQ) { a_frag(t + L::FWDA + f * 2 * 32 * 4, f / L::KBQ, f % L::KBQ, Q, -1); return; }
  f -= L::MQ * L::KBQ;
  if (f < 8) { b_frag(t + L::FWDB + f * 2 * 32 * 2, f / 4, f % 4, 16, -1); return; }
  f -= 8;
  if (f < Q / 8) {  // inverse stage-A twiddles: rows k1 = g, g+8; cols n2 = 8 f + 2 tq + {0,1}
    float* w = reinterpret_cast<float*>(t + L::TWI + (f * 32 + lane) * 8);
    const int n2 = 8 * f + 2 * tq;
    const int k1s[4] = {g, g, g + 8, g + 8}, n2s[4] = {n2, n2 + 1, n2, n2 + 1};
    for (int i = 0; i < 4; ++i) {
      const double2 z = unit_root((long long)n2s[i] * k1s[i], N, +1);
      w[2 * i] = (float)z.x;
      w[2 * i + 1] = (float)z.y;
    }
    return;
  }
  f -= Q / 8;
  if (f < L::MR * 2) {  // forward stage-A' twiddles: rows k1 = 16 mr + g (+8), cols b = 8 nb + 2 tq + {0,1}
    const int mr = f / 2, nb = f % 2;
    float* w = reinterpret_cast<float*>(t + L::TWF + (f * 32 + lane) * 8);
    const int b = 8 * nb + 2 * tq;
    const int k1 = 16 * mr + g;
    const int k1s[4] = {k1, k1, k1 + 8, k1 + 8}, bs[4] = {b, b + 1, b, b + 1};
    for (int i = 0; i < 4; ++i) {
      const double2 z = unit_root((long long)bs[i] * k1s[i], N, -1);
      w[2 * i] = (float)z.x;
      w[2 * i + 1] = (float)z.y;
    }
  }
}

template <int N>
constexpr int tc_table_fragments() {
  using L = TcLayout<N>;
  return 4 + L::KBQ * L::NTQ + L::MQ * L::KBQ + 8 + L::Q / 8 + L::MR * 2;
}

// A fragment (hi at f, lo 128 words further), one 16-byte load each
__device__ __forceinline__ void ldfrag4(const uint32_t* f, uint32_t (&hi)[4], uint32_t (&lo)[4]) {
  const uint4 h = __ldg(reinterpret_cast<const uint4*>(f));
  const uint4 l = __ldg(reinterpret_cast<const uint4*>(f + 32 * 4));
  hi[0] = h.x; hi[1] = h.y; hi[2] = h.z; hi[3] = h.w;
  lo[0] = l.x; lo[1] = l.y; lo[2] = l.z; lo[3] = l.w;
}

// padded index of element k of a forward output buffer: 4 pad words after every 16 elements
// make the accumulator-layout writes free of bank conflicts
__host__ __device__ constexpr int tc_pad(int k) { return k + 4 * (k >> 4); }

// shared-memory words (float2) of one warp's row: two staging buffers and the forward output
template <int N>
int tc_group_words(int kxp) { return 2 * 6 * kxp + tc_pad(N); }

// Build the constant table of (N, KIND) into device memory (one warp per fragment).
template <int N, int KIND>
int tc_build_table(uint32_t* table) {
  constexpr int frags = tc_table_fragments<N>();
  tc_tables_kernel<N, KIND><<<(frags + 3) / 4, 128>>>(table);
  if (cudaGetLastError() != cudaSuccess) return 1;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

// ------------------------------------------------------------------------------------------
// One length-N transform pair (inverse) or product pair (forward) per call, one row per warp.
// ------------------------------------------------------------------------------------------
// Power-of-two scale bringing a bound m of the largest |component| of a transform's input to
// [2^9, 2^10) (FP16 only; BF16 has the FP32 exponent range): one 16- or 32-point stage then stays
// below 2^16 and the split operands stay in the FP16 range.  m is the same on every lane.
template <int KIND>
__device__ __forceinline__ float tc_scale(float m) {
  if constexpr (KIND != SPLIT_F16) {
    return 1.f;
  } else {
    if (!(m > 0.f) || !isfinite(m)) return 1.f;
    const int e = (int)((__float_as_uint(m) >> 23) & 0xff) - 127;  // floor(log2 m) for normal m
    int p = 9 - e;
    p = p < -100 ? -100 : (p > 100 ? 100 : p);
    return __uint_as_float((unsigned)(127 + p) << 23);
  }
}
// exact reciprocal of a power-of-two scale
__device__ __forceinline__ float pow2_inv(float s) { return __uint_as_float(0x7f000000u - __float_as_uint(s)); }

__device__ __forceinline__ float warp_max(float m) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  return m;
}

// Inverse transform of one row held as B fragments, inputs scaled by s.
// in:  zr/zi[nt][4] = z[Q n1 + n2] for n2 = 8 nt + g and n1 = 2tq, 2tq+1, 2tq+8, 2tq+9
// out: xr/xi[nt2][4] = x[k1 + 16 k2] for k2 = 8 nt2 + 2tq + {0,1}, k1 = g (elements 0,1) or
//      g + 8 (elements 2,3) -- the m16n8 accumulator layout
template <int N, int KIND>
__device__ __forceinline__ void tc_inverse(const float (&zr)[N / 128][4], const float (&zi)[N / 128][4], float s,
                                           float (&xr)[N / 128][4], float (&xi)[N / 128][4],
                                           const uint32_t* __restrict__ tab, int lane) {
  using L = TcLayout<N>;
  constexpr int NT = L::Q / 8;
  // stage A: C[mt][nt] (mt 0 = real rows, 1 = imaginary rows) = sum_kb F16e[mt][kb] Z[kb][nt]
  float c[2][NT][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) c[mt][nt][i] = 0.f;
#pragma unroll
  for (int kb = 0; kb < 2; ++kb) {  // kb 0: real parts of z, kb 1: imaginary parts
    uint32_t bh[NT][2], bl[NT][2];
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const float* v = kb ? zi[nt] : zr[nt];
      split_pair<KIND>(s * v[0], s * v[1], bh[nt][0], bl[nt][0]);
      split_pair<KIND>(s * v[2], s * v[3], bh[nt][1], bl[nt][1]);
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      uint32_t ah[4], al[4];
      ldfrag4(tab + L::INVA + (mt * 2 + kb) * 2 * 32 * 4 + lane * 4, ah, al);
      mma3n<KIND, NT>(c[mt], ah, al, bh, bl);
    }
  }
  // twiddle W_N^{n2 k1}
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    const float4* w4 = reinterpret_cast<const float4*>(tab + L::TWI + (nt * 32 + lane) * 8);
    const float4 wa = __ldg(w4), wb = __ldg(w4 + 1);
    const float w[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float wr = w[2 * i], wi = w[2 * i + 1];
      const float a = c[0][nt][i], b = c[1][nt][i];
      c[0][nt][i] = a * wr - b * wi;
      c[1][nt][i] = a * wi + b * wr;
    }
  }
  // stage B: X = [Y'r | Y'i] (16 x 2Q) * FQe (2Q x 2Q); the A operand's k-block kb is the pair of
  // accumulator tiles (2 kb, 2 kb + 1) of the list [real tiles 0..NT-1, imaginary tiles 0..NT-1]
  const float inv = pow2_inv(s);
  float d[L::NTQ][4];
#pragma unroll
  for (int nt2 = 0; nt2 < L::NTQ; ++nt2)
#pragma unroll
    for (int i = 0; i < 4; ++i) d[nt2][i] = 0.f;
#pragma unroll
  for (int kb = 0; kb < L::KBQ; ++kb) {
    uint32_t ah[4], al[4];
    const int j0 = 2 * kb, j1 = 2 * kb + 1;
    const float* t0 = c[j0 / NT][j0 % NT];
    const float* t1 = c[j1 / NT][j1 % NT];
    split_pair<KIND>(t0[0], t0[1], ah[0], al[0]);
    split_pair<KIND>(t0[2], t0[3], ah[1], al[1]);
    split_pair<KIND>(t1[0], t1[1], ah[2], al[2]);
    split_pair<KIND>(t1[2], t1[3], ah[3], al[3]);
    uint32_t bh[L::NTQ][2], bl[L::NTQ][2];
#pragma unroll
    for (int nt2 = 0; nt2 < L::NTQ; ++nt2) {
      const uint2* f = reinterpret_cast<const uint2*>(tab + L::INVB + (kb * L::NTQ + nt2) * 2 * 32 * 2);
      const uint2 h = __ldg(f + lane), l = __ldg(f + 32 + lane);
      bh[nt2][0] = h.x; bh[nt2][1] = h.y; bl[nt2][0] = l.x; bl[nt2][1] = l.y;
    }
    mma3n<KIND, L::NTQ>(d, ah, al, bh, bl);
  }
#pragma unroll
  for (int nt2 = 0; nt2 < L::NTQ; ++nt2) {
    float* out = nt2 < NT ? xr[nt2] : xi[nt2 - NT];
#pragma unroll
    for (int i = 0; i < 4; ++i) out[i] = d[nt2][i] * inv;
  }
}

// Forward transform of one row whose input element (tile nt, element i) of the inverse's output
// layout is prod(nt, i) (a float2: real, imaginary), scaled by s; the result X[k1 + Q k2] goes to
// buf[tc_pad(k)] in natural order.
template <int N, int KIND, class Prod>
__device__ __forceinline__ void tc_forward(Prod prod, float s, float2* buf, const uint32_t* __restrict__ tab,
                                           int lane) {
  using L = TcLayout<N>;
  constexpr int Q = L::Q, NT = Q / 8;
  const int g = lane >> 2, tq = lane & 3;
  // stage A': C[mt][nb] = sum_kb FQe*[mt][kb] B[kb][nb].  The B operand (K = 2Q: a real 0..Q-1,
  // a imaginary; N = 16: b) is the input read transposed: k-block kb, n-tile nb takes elements
  // (0,1) (nb = 0) or (2,3) (nb = 1) of tiles 2kb, 2kb+1 of the list [real tiles, imaginary tiles].
  float c[L::MQ][2][4];
#pragma unroll
  for (int mt = 0; mt < L::MQ; ++mt)
#pragma unroll
    for (int nb = 0; nb < 2; ++nb)
#pragma unroll
      for (int i = 0; i < 4; ++i) c[mt][nb][i] = 0.f;
#pragma unroll
  for (int kb = 0; kb < L::KBQ; ++kb) {
    uint32_t bh[2][2], bl[2][2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j = 2 * kb + h;
      const int nt = j % NT;
      const bool im = j >= NT;
#pragma unroll
      for (int nb = 0; nb < 2; ++nb) {
        const float2 p0 = prod(nt, 2 * nb), p1 = prod(nt, 2 * nb + 1);
        const float v0 = im ? p0.y : p0.x, v1 = im ? p1.y : p1.x;
        split_pair<KIND>(s * v0, s * v1, bh[nb][h], bl[nb][h]);
      }
    }
#pragma unroll
    for (int mt = 0; mt < L::MQ; ++mt) {
      uint32_t ah[4], al[4];
      ldfrag4(tab + L::FWDA + (mt * L::KBQ + kb) * 2 * 32 * 4 + lane * 4, ah, al);
      mma3n<KIND, 2>(c[mt], ah, al, bh, bl);
    }
  }
  // twiddle W_N^{-b k1}: real part of row k1 at tile (k1 / 16, element 0/1 or 2/3), imaginary
  // part at tile (k1 + Q) / 16; for Q = 8 both live in the one tile (real elements 0,1, imaginary 2,3)
#pragma unroll
  for (int mr = 0; mr < L::MR; ++mr)
#pragma unroll
    for (int nb = 0; nb < 2; ++nb) {
      const float4* w4 = reinterpret_cast<const float4*>(tab + L::TWF + ((mr * 2 + nb) * 32 + lane) * 8);
      const float4 wa = __ldg(w4), wb = __ldg(w4 + 1);
      const float w[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
      if constexpr (Q >= 16) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float wr = w[2 * i], wi = w[2 * i + 1];
          float& a = c[mr][nb][i];
          float& b = c[mr + Q / 16][nb][i];
          const float ar = a, bi = b;
          a = ar * wr - bi * wi;
          b = ar * wi + bi * wr;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const float wr = w[2 * i], wi = w[2 * i + 1];
          float& a = c[0][nb][i];
          float& b = c[0][nb][i + 2];
          const float ar = a, bi = b;
          a = ar * wr - bi * wi;
          b = ar * wi + bi * wr;
        }
      }
    }
  // stage B': X = [Y'r | Y'i] (Q x 32) * F16e* (32 x 32); A operand of m-tile mt: k-block 0 from
  // the real tiles of rows 16mt.., k-block 1 from the imaginary ones (Q = 8: rows 8..15 padding)
  const float inv = pow2_inv(s);
  constexpr int MT = Q >= 16 ? Q / 16 : 1;
#pragma unroll
  for (int mt = 0; mt < MT; ++mt) {
    uint32_t ah[2][4], al[2][4];
#pragma unroll
    for (int kb = 0; kb < 2; ++kb) {
      float t0[4], t1[4];
      if constexpr (Q >= 16) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          t0[i] = c[mt + kb * (Q / 16)][0][i];
          t1[i] = c[mt + kb * (Q / 16)][1][i];
        }
      } else {  // real rows are elements 0,1 of the tile, imaginary rows elements 2,3
        t0[0] = c[0][0][2 * kb]; t0[1] = c[0][0][2 * kb + 1]; t0[2] = 0.f; t0[3] = 0.f;
        t1[0] = c[0][1][2 * kb]; t1[1] = c[0][1][2 * kb + 1]; t1[2] = 0.f; t1[3] = 0.f;
      }
      split_pair<KIND>(t0[0], t0[1], ah[kb][0], al[kb][0]);
      split_pair<KIND>(t0[2], t0[3], ah[kb][1], al[kb][1]);
      split_pair<KIND>(t1[0], t1[1], ah[kb][2], al[kb][2]);
      split_pair<KIND>(t1[2], t1[3], ah[kb][3], al[kb][3]);
    }
#pragma unroll
    for (int nh = 0; nh < 2; ++nh) {  // output columns k2 = 8 nh + ..: real tile nh, imaginary tile nh + 2
      float d[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
      for (int kb = 0; kb < 2; ++kb) {
        uint32_t bh[2][2], bl[2][2];
#pragma unroll
        for (int ri = 0; ri < 2; ++ri) {
          const uint2* f = reinterpret_cast<const uint2*>(tab + L::FWDB + (kb * 4 + nh + 2 * ri) * 2 * 32 * 2);
          const uint2 h = __ldg(f + lane), l = __ldg(f + 32 + lane);
          bh[ri][0] = h.x; bh[ri][1] = h.y; bl[ri][0] = l.x; bl[ri][1] = l.y;
        }
        mma3n<KIND, 2>(d, ah[kb], al[kb], bh, bl);
      }
      // element (row k1, col k2): rows 16 mt + g (+8), cols 8 nh + 2 tq + {0,1}
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int k1 = 16 * mt + g + (i >= 2 ? 8 : 0);
        const int k2 = 8 * nh + 2 * tq + (i & 1);
        if (k1 < Q) buf[tc_pad(k1 + Q * k2)] = make_float2(d[0][i] * inv, d[1][i] * inv);
      }
    }
  }
}

// ------------------------------------------------------------------------------------------
// Fused x rows on the tensor cores: same contract as x_fused_kernel (one row per warp, GROUPS
// warps per CTA, cp.async double-buffered staging of the six field rows), with the transforms of
// tc_inverse / tc_forward.  tab is the tc_tables_kernel output of this N and KIND.
// ------------------------------------------------------------------------------------------
template <int N, int KIND, int GROUPS, int MINB>
__global__ void __launch_bounds__(GROUPS * 32, MINB)
    x_fused_tc_kernel(float2* pool, Geom geo, long long rowstride, long long slot, long long istride, BatchRef br,
                      const float2* __restrict__ tabf, const float2* __restrict__ unused, unsigned int* vmax,
                      VpRef) {
  constexpr int Q = N / 16, NT = Q / 8;
  constexpr int KX = kept_kx_of(N);
  const uint32_t* __restrict__ tab = reinterpret_cast<const uint32_t*>(tabf);
  extern __shared__ float2 smem[];
  const int kxp = geo.kxp;
  const int grp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tq = lane & 3;
  const int sw = 6 * kxp;                       // staging words of one row
  float2* gs = smem + grp * (2 * sw + tc_pad(N));
  float2* ob = gs + 2 * sw;                     // forward output of one transform (padded)
  constexpr int GPI = N * N;                    // rows per instance
  const long long nrows = (long long)(*br.count) * GPI;
  const int chunks_row = 3 * kxp;
  auto row_ptr = [&](long long q) {
    const int inst = (int)(q / GPI);
    return pool + br.list[inst] * istride + (q - (long long)inst * GPI) * rowstride;
  };
  auto prefetch = [&](long long q, float2* dst) {
    const float2* src = row_ptr(q);
    for (int c = lane; c < chunks_row; c += 32) cp_async16(dst + 2 * c, src + 2 * c);
  };
  long long q = (long long)blockIdx.x * GROUPS + grp;
  const long long qstep = (long long)gridDim.x * GROUPS;
  if (q < nrows) prefetch(q, gs);
  cp_async_commit();
  for (int it = 0; q < nrows; q += qstep, ++it) {
    const float2* cur = gs + (it & 1) * sw;
    if (q + qstep < nrows) prefetch(q + qstep, gs + ((it + 1) & 1) * sw);
    cp_async_commit();
    cp_async_wait<1>();
    __syncwarp();
    // scale of the three inverse transforms: the largest |component| of the six spectral rows
    float sc = 1.f;
    if constexpr (KIND == SPLIT_F16) {
      float m = 0.f;
      for (int c = lane; c < 6 * KX; c += 32) {
        const float2 z = cur[(c / KX) * kxp + c % KX];
        m = fmaxf(m, fmaxf(fabsf(z.x), fabsf(z.y)));
      }
      sc = tc_scale<KIND>(2.f * warp_max(m));  // |F1 +- i F2| components are at most twice that
    }
    // inverse inputs: z[n] = F1[n] + i F2[n] (Hermitian extension, kx = 0 imaginary parts dropped)
    float ur[3][NT][4], ui[3][NT][4];
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      const float2* f1 = cur + (2 * t) * kxp;
      const float2* f2 = cur + (2 * t + 1) * kxp;
      float zr[NT][4], zi[NT][4];
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int n1 = 2 * tq + (i & 1) + (i >= 2 ? 8 : 0);
          const int n = Q * n1 + 8 * nt + g;
          float2 z = make_float2(0.f, 0.f);
          if (n < KX) {
            float2 a = f1[n], b = f2[n];
            if (n == 0) { a.y = 0.f; b.y = 0.f; }
            z = make_float2(a.x - b.y, a.y + b.x);
          } else if (n > N - KX) {
            const int m = N - n;
            const float2 a = f1[m], b = f2[m];
            z = make_float2(a.x + b.y, b.x - a.y);
          }
          zr[nt][i] = z.x;
          zi[nt][i] = z.y;
        }
      tc_inverse<N, KIND>(zr, zi, sc, ur[t], ui[t], tab, lane);
    }
    __syncwarp();  // staging reads done before the buffer is refilled two rows later
    float mu = 0.f, mb = 0.f;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        mu = fmaxf(mu, fmaxf(fabsf(ur[0][nt][i]), fmaxf(fabsf(ui[0][nt][i]), fabsf(ur[1][nt][i]))));
        mb = fmaxf(mb, fmaxf(fabsf(ui[1][nt][i]), fmaxf(fabsf(ur[2][nt][i]), fabsf(ui[2][nt][i]))));
      }
    if (vmax) {
      unsigned int bu = __float_as_uint(mu), bb = __float_as_uint(mb);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        bu = max(bu, __shfl_xor_sync(0xffffffffu, bu, o));
        bb = max(bb, __shfl_xor_sync(0xffffffffu, bb, o));
      }
      if (lane == 0) {
        const int inst = (int)(q / GPI);
        atomicMax(vmax + 2 * br.list[inst], bu);
        atomicMax(vmax + 2 * br.list[inst] + 1, bb);
      }
    }
    // every product is bounded by 4 max(|u|, |B|)^2
    float scp = 1.f;
    if constexpr (KIND == SPLIT_F16) {
      const float mm = warp_max(fmaxf(mu, mb));
      scp = tc_scale<KIND>(4.f * mm * mm);
    }
    float2* rowp = row_ptr(q);
#pragma unroll 1
    for (int t = 0; t < 4; ++t) {  // not unrolled: one forward transform's working set at a time
      auto prod = [&](int nt, int i) -> float2 {
        const float ux = ur[0][nt][i], uy = ui[0][nt][i], uz = ur[1][nt][i];
        const float bx = ui[1][nt][i], by = ur[2][nt][i], bz = ui[2][nt][i];
        if (t == 0) {
          const float tzz = bz * bz - uz * uz;
          return make_float2((bx * bx - ux * ux) - tzz, (by * by - uy * uy) - tzz);
        } else if (t == 1) {
          return make_float2(bx * by - ux * uy, bx * bz - ux * uz);
        } else if (t == 2) {
          return make_float2(by * bz - uy * uz, ux * by - bx * uy);
        } else {
          return make_float2(ux * bz - bx * uz, uy * bz - by * uz);
        }
      };
      tc_forward<N, KIND>(prod, scp, ob, tab, lane);
      __syncwarp();
      {
        float2* outa = rowp + (2 * t) * slot;
        float2* outb = rowp + (2 * t + 1) * slot;
        for (int k = lane; k < KX; k += 32) {
          const float2 z = ob[tc_pad(k)];
          const float2 zc = cconj(ob[tc_pad((N - k) % N)]);
          const float2 sm = cadd(z, zc), df = csub(z, zc);
          outa[k] = make_float2(0.5f * sm.x, 0.5f * sm.y);
          outb[k] = make_float2(0.5f * df.y, -0.5f * df.x);
        }
      }
      __syncwarp();
    }
  }
  cp_async_wait<0>();
}

}  // namespace mhdgb
