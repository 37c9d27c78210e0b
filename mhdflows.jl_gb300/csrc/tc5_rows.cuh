// x rows on the fifth-generation tensor cores (precision form MHD_PREC_SPLIT_TF32, n = 256).
//
// Each 256-point row transform is two 16-point stages (N = 16 * 16), and each stage is one
// matrix product on the tensor cores: tcgen05.mma kind::tf32 with M = 128 rows, N = 32, K = 32,
// the A operand (the data) in tensor memory, the B operand (a 16-point DFT matrix in its real
// embedding) in shared memory, and the FP32 accumulator in tensor memory.  FP32 accuracy comes
// from a split of both operands into TF32 hi + lo parts, x = hi + lo with hi = x rounded to TF32:
// D = A_hi B_hi + A_hi B_lo + A_lo B_hi, FP32 accumulation (the dropped A_lo B_lo is below 2^-22).
//
// A CTA of 128 threads (4 warps) takes 8 physical rows at a time; thread m owns tensor-memory lane
// m, which is row r = m / 16 of the tile and index j = m % 16 inside it (the 16 lanes of a row sit
// in one warp).  With n = 16 a + b (inverse input index) and k = c + 16 d (inverse output index):
//   stage 1  lane (r, b):  Y[b, c] = sum_a z[16 a + b] w16^(a c)      (A row: z[16 a + b], a = 0..15)
//   twiddle                Y[b, c] *= w256^(b c)
//   transpose (shared memory, inside the warp) to lane (r, c): Y[., c]
//   stage 2  lane (r, c):  X[c + 16 d] = sum_b Y[b, c] w16^(b d)
// so after an inverse transform lane (r, c) holds the physical points x = c + 16 d, d = 0..15.
// The forward transform of a product row starts from exactly that layout: stage 1 runs over d on
// the lane's own points, the twiddle is the conjugate of the same table, and after the transpose
// stage 2 leaves Z[q0 + 16 q1] on lane (r, q0).  The Hermitian two-for-one split pairs lane q0
// with lane 16 - q0 through shuffles.  Between the inverse and the forward transforms the six
// physical fields stay in tensor memory (the second-stage products write there directly).
//
// Tensor memory (256 columns per CTA, two CTAs per SM):
//   [0, 32)    twiddles w256^(j c) of the lane's j = m % 16, c = 0..15: cos then sin
//   [32, 128)  physical fields of the three inverse pairs (ux uy | uz bx | by bz), re then im
//   [128, 160) A operand hi, [160, 192) A operand lo, [192, 224) accumulator D
// Shared memory: the four B matrices (inverse / forward x hi / lo), the transpose buffer, and two
// buffers of the tile's six spectral field rows (cp.async, the next tile's while this one runs).
//
// Every wait on the MMA completion barrier is bounded (about one second of %globaltimer); on a
// timeout the CTA records an error word in the table, stops, lets its copies land and frees its
// tensor memory before it returns.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "passes.cuh"

namespace mhdgb {

// The table of the TF32 x rows: four 32 x 32 B matrices in the tensor cores' no-swizzle K-major
// layout (core matrices of 8 rows x 4 words, 128 bytes each; core (row group g, k chunk c) at
// word (g * 8 + c) * 32), then an error word.
struct Tc5Layout {
  static constexpr int MAT = 32 * 32;
  static constexpr int ERR = 4 * MAT;   // word index of the error word
  static constexpr int WORDS = 4 * MAT + 32;
  static constexpr int TILE_ROWS = 8;   // physical rows per tile (M = 8 * 16 = 128)
  static constexpr int THREADS = 128;
  static constexpr int TMEM_COLS = 256;
  static constexpr int C_TW = 0, C_PHYS = 32, C_AHI = 128, C_ALO = 160, C_D = 192;
};

__host__ __device__ constexpr int tc5_core_word(int n, int k) { return ((n / 8) * 8 + k / 4) * 32 + (n % 8) * 4 + k % 4; }

// Shared-memory bytes of one CTA (tc5_smem_words in float2 units for the variant table).
__host__ __device__ constexpr int tc5_smem_bytes(int kxp) {
  return 4 * Tc5Layout::MAT * 4                       // B matrices
         + Tc5Layout::TILE_ROWS * 16 * 16 * 8         // transpose buffer
         + 2 * Tc5Layout::TILE_ROWS * 6 * kxp * 8     // two staging buffers of the spectral rows
         + 64;                                        // barrier, tensor-memory base, flags
}
// (about 100 KB at n = 256: two CTAs per SM, which is also what the 2 x 256 tensor-memory columns
// of an SM allow)
inline int tc5_group_words(int kxp) { return (tc5_smem_bytes(kxp) + 7) / 8; }

// B matrices of the 16-point DFT, real embedding, rows N (output c: re 0..15, im 16..31), columns
// K (input a: re 0..15, im 16..31), direction DIR: entry of (c, a) is e^(DIR 2 pi i a c / 16).
// Matrix s: 0 inverse hi, 1 inverse lo, 2 forward hi, 3 forward lo; hi = TF32 rounding of the
// FP64 value, lo = TF32 rounding of the rest.  Twiddle generation in FP64 on the device.
__device__ __forceinline__ uint32_t tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
template <int N>
__global__ void tc5_tables_kernel(uint32_t* table) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * Tc5Layout::MAT) {
    if (i < 2 * Tc5Layout::MAT + 32) table[Tc5Layout::ERR + (i - 2 * Tc5Layout::MAT)] = 0u;
    return;
  }
  const int dirsel = i / Tc5Layout::MAT, e = i % Tc5Layout::MAT;
  const int n = e / 32, k = e % 32;  // row (output), column (input)
  const int c = n % 16, a = k % 16;
  const double dir = dirsel == 0 ? 1.0 : -1.0;
  double s, co;
  sincospi(dir * 2.0 * (double)((a * c) % 16) / 16.0, &s, &co);
  // [re_out] = re_in cos - im_in sin ; [im_out] = re_in sin + im_in cos
  double v;
  if (n < 16) v = k < 16 ? co : -s;
  else v = k < 16 ? s : co;
  const uint32_t hi = tf32_round((float)v);
  const uint32_t lo = tf32_round((float)(v - (double)__uint_as_float(hi)));
  table[(2 * dirsel) * Tc5Layout::MAT + tc5_core_word(n, k)] = hi;
  table[(2 * dirsel + 1) * Tc5Layout::MAT + tc5_core_word(n, k)] = lo;
}
template <int N>
int tc5_build_table(uint32_t* table) {
  tc5_tables_kernel<N><<<(2 * Tc5Layout::MAT + 32 + 127) / 128, 128>>>(table);
  if (cudaGetLastError() != cudaSuccess) return 1;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

// ---- tcgen05 / tensor-memory primitives (PTX) ---------------------------------------------
__device__ __forceinline__ uint64_t tc5_smem_desc(uint32_t addr) {
  // no swizzle; leading byte offset 128 (next core matrix along K), stride byte offset 1024 (next
  // group of 8 rows); descriptor version 1 at bit 46
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46);
}
// kind::tf32 instruction descriptor: FP32 accumulator, TF32 A and B, both K-major, N = 32, M = 128
constexpr uint32_t kTc5Idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc5_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc5_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc5_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]),
      "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]),
      "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}
__device__ __forceinline__ void tc5_ld32(uint32_t taddr, float (&f)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) f[i] = __uint_as_float(r[i]);
}

// x = hi + lo with hi the TF32 rounding of x (lo exact in FP32; the tensor core reads its top bits)
__device__ __forceinline__ void tc5_split(const float (&x)[32], uint32_t (&hi)[32], uint32_t (&lo)[32]) {
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    hi[i] = tf32_round(x[i]);
    lo[i] = __float_as_uint(x[i] - __uint_as_float(hi[i]));
  }
}
__device__ __forceinline__ void tc5_store_operand(uint32_t tlane, const float (&x)[32]) {
  uint32_t hi[32], lo[32];
  tc5_split(x, hi, lo);
  tc5_st32(tlane + Tc5Layout::C_AHI, hi);
  tc5_st32(tlane + Tc5Layout::C_ALO, lo);
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// One 16-point stage for the whole CTA: every thread has stored its A row; the elected thread
// issues D = A_hi B_hi + A_hi B_lo + A_lo B_hi (four K = 8 steps each) into column dcol and
// commits to the barrier; that thread waits for the phase (bounded) and the CTA barrier releases
// the others.  Returns false on a timeout.
__device__ __forceinline__ bool tc5_stage(uint32_t tbase, uint32_t dcol, uint32_t bhi, uint32_t blo, uint32_t bar,
                                          uint32_t phase) {
  tc5_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc5_fence_after();
    const uint32_t d = tbase + dcol;
#pragma unroll
    for (int term = 0; term < 3; ++term) {
      const uint32_t a = tbase + (term == 2 ? Tc5Layout::C_ALO : Tc5Layout::C_AHI);
      const uint32_t b = term == 1 ? blo : bhi;
#pragma unroll
      for (int kc = 0; kc < 4; ++kc) {
        const uint64_t bd = tc5_smem_desc(b + kc * 256);
        const uint32_t acc = (term | kc) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d),
            "r"(a + kc * 8), "l"(bd), "r"(kTc5Idesc), "r"(acc)
            : "memory");
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
  }
  // one thread polls the barrier (bounded); the others wait at the CTA barrier without issuing
  const bool ok = threadIdx.x == 0 ? mbar_wait(bar, phase & 1u) : true;
  const bool all = __syncthreads_and(ok ? 1 : 0) != 0;
  tc5_fence_after();
  return all;
}

// Transpose of a 16 x 16 complex block between the 16 lanes of a row (inside one warp): lane j
// holds v[c] (c = 0..15) of row j; afterwards lane j holds the column j, v[b] = old row b's v[j].
// 16-byte chunks are swizzled by the row so that both the row writes and the column reads touch
// each bank once per 8 lanes.
__device__ __forceinline__ void tc5_transpose(float2* tb, int j, float (&re)[16], float (&im)[16]) {
  float4* row = reinterpret_cast<float4*>(tb + j * 16);
#pragma unroll
  for (int q = 0; q < 8; ++q) row[q ^ (j & 7)] = make_float4(re[2 * q], im[2 * q], re[2 * q + 1], im[2 * q + 1]);
  __syncwarp();
#pragma unroll
  for (int b = 0; b < 16; ++b) {
    const float2 v = tb[b * 16 + 2 * ((j >> 1) ^ (b & 7)) + (j & 1)];
    re[b] = v.x;
    im[b] = v.y;
  }
  __syncwarp();
}

// The Hermitian two-for-one input of an inverse transform (two spectral rows f1, f2 with KX kept
// modes): z[n] = F1[n] + i F2[n] with F[-n] = conj F[n], kx = 0 imaginary parts dropped.
template <int N, int KX>
__device__ __forceinline__ float2 tc5_herm(const float2* f1, const float2* f2, int n) {
  if (n < KX) {
    float2 a = f1[n], b = f2[n];
    if (n == 0) { a.y = 0.f; b.y = 0.f; }
    return make_float2(a.x - b.y, a.y + b.x);
  }
  if (n > N - KX) {
    const float2 a = f1[N - n], b = f2[N - n];
    return make_float2(a.x + b.y, b.x - a.y);
  }
  return make_float2(0.f, 0.f);
}

// The fused x pass of one right-hand side on the tensor cores (same inputs, outputs and products
// as x_fused_kernel: 3 inverse pairs -> 6 fields -> 8 products -> 4 forward pairs).
// tw carries the table (B matrices, error word); twr is unused.
template <int N>
__global__ void __launch_bounds__(128, 2)
    x_fused_tc5_kernel(float2* pool, Geom geo, long long rowstride, long long slot, long long istride, BatchRef br,
                       const float2* tw, const float2* /*twr*/, unsigned int* vmax, VpRef /*vp*/) {
  static_assert(N == 256, "two 16-point stages: n = 256");
  constexpr int KX = kept_kx_of(N), R = Tc5Layout::TILE_ROWS;
  using L = Tc5Layout;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  uint32_t* table = const_cast<uint32_t*>(reinterpret_cast<const uint32_t*>(tw));
  const int kxp = geo.kxp;
  float* bmat = reinterpret_cast<float*>(smem_raw);                                     // 16 KB
  float2* tbuf = reinterpret_cast<float2*>(smem_raw + 4 * L::MAT * 4);                   // 16 KB
  float2* stage = reinterpret_cast<float2*>(smem_raw + 4 * L::MAT * 4 + R * 256 * 8);    // 2 x 8 rows x 6 fields
  unsigned char* misc = smem_raw + 4 * L::MAT * 4 + R * 256 * 8 + 2 * R * 6 * kxp * 8;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(misc);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(misc + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r = tid >> 4, j = tid & 15;  // row of the tile, index inside the row

  // ---- set-up: B matrices, tensor memory, barrier, twiddles
  for (int i = tid; i < 4 * L::MAT; i += blockDim.x) bmat[i] = __uint_as_float(table[i]);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "n"(L::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B matrices visible to the tensor cores
  tc5_fence_before();
  __syncthreads();
  tc5_fence_after();
  const uint32_t tbase = *tmem_slot;
  const uint32_t tlane = tbase + ((uint32_t)(warp * 32) << 16);
  {
    float w[32];
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      double s, co;
      sincospi((double)(j * c) / 128.0, &s, &co);  // w256^(j c)
      w[c] = (float)co;
      w[16 + c] = (float)s;
    }
    uint32_t u[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) u[c] = __float_as_uint(w[c]);
    tc5_st32(tlane + L::C_TW, u);
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
  }
  const uint32_t b_inv_hi = smem_u32(bmat), b_inv_lo = b_inv_hi + L::MAT * 4;
  const uint32_t b_fwd_hi = b_inv_hi + 2 * L::MAT * 4, b_fwd_lo = b_inv_hi + 3 * L::MAT * 4;
  const uint32_t barp = smem_u32(bar);
  uint32_t phase = 0;
  bool ok = true;

  constexpr int GPI = N * N / R;  // tiles per instance
  const long long ntiles = (long long)(*br.count) * GPI;
  const int chunks_row = 6 * kxp / 2;  // 16-byte chunks of a row's six contiguous field rows
  auto tile_rows = [&](long long q) {  // first row of tile q (taken from the last one down)
    q = ntiles - 1 - q;
    const int inst = (int)(q / GPI);
    return pool + br.list[inst] * istride + (q - (long long)inst * GPI) * R * rowstride;
  };
  auto prefetch = [&](long long q, float2* dst) {
    const float2* src = tile_rows(q);
    for (int c = tid; c < R * chunks_row; c += blockDim.x) {
      const int rr = c / chunks_row, cc = c - rr * chunks_row;
      cp_async16(dst + rr * 6 * kxp + 2 * cc, src + rr * rowstride + 2 * cc);
    }
  };
  long long q = blockIdx.x;
  if (q < ntiles) prefetch(q, stage);
  cp_async_commit();
  for (int it = 0; q < ntiles && ok; q += gridDim.x, ++it) {
    const float2* cur = stage + (it & 1) * R * 6 * kxp;
    if (q + gridDim.x < ntiles) prefetch(q + gridDim.x, stage + ((it + 1) & 1) * R * 6 * kxp);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const float2* rin = cur + r * 6 * kxp;
    float2* tb = tbuf + r * 256;
    float tw_c[16], tw_s[16];
    {
      float w[32];
      tc5_ld32(tlane + L::C_TW, w);
#pragma unroll
      for (int c = 0; c < 16; ++c) { tw_c[c] = w[c]; tw_s[c] = w[16 + c]; }
    }
    // ---- inverse transforms of the pairs (ux uy), (uz bx), (by bz)
#pragma unroll 1
    for (int p = 0; p < 3 && ok; ++p) {
      float a[32];
#pragma unroll
      for (int s = 0; s < 16; ++s) {  // lane (r, b = j): z[16 s + j]
        const float2 z = tc5_herm<N, KX>(rin + 2 * p * kxp, rin + (2 * p + 1) * kxp, 16 * s + j);
        a[s] = z.x;
        a[16 + s] = z.y;
      }
      tc5_store_operand(tlane, a);
      ok = tc5_stage(tbase, L::C_D, b_inv_hi, b_inv_lo, barp, phase++);
      if (!ok) break;
      float d[32];
      tc5_ld32(tlane + L::C_D, d);
      float re[16], im[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {  // Y[j, c] w256^(j c)
        re[c] = d[c] * tw_c[c] - d[16 + c] * tw_s[c];
        im[c] = d[c] * tw_s[c] + d[16 + c] * tw_c[c];
      }
      tc5_transpose(tb, j, re, im);  // lane (r, c = j) now holds Y[b, j], b = 0..15
#pragma unroll
      for (int b = 0; b < 16; ++b) { a[b] = re[b]; a[16 + b] = im[b]; }
      tc5_store_operand(tlane, a);
      ok = tc5_stage(tbase, L::C_PHYS + 32 * p, b_inv_hi, b_inv_lo, barp, phase++);
    }
    // ---- products and forward transforms: lane (r, c = j) holds the points x = j + 16 d
    float2* rowp = tile_rows(q) + r * rowstride;
#pragma unroll 1
    for (int t = 0; t < 4 && ok; ++t) {
      float a[32];
      {
        float f0[32], f1[32], f2[32];
        tc5_ld32(tlane + L::C_PHYS, f0);
        tc5_ld32(tlane + L::C_PHYS + 32, f1);
        tc5_ld32(tlane + L::C_PHYS + 64, f2);
        if (vmax && t == 0) {
          // max |u_i| and max |B_i| (getCFL! on the last stage's fields), as bit patterns
          float mu = 0.f, mb = 0.f;
#pragma unroll
          for (int d = 0; d < 16; ++d) {
            mu = fmaxf(mu, fmaxf(fabsf(f0[d]), fmaxf(fabsf(f0[16 + d]), fabsf(f1[d]))));
            mb = fmaxf(mb, fmaxf(fabsf(f1[16 + d]), fmaxf(fabsf(f2[d]), fabsf(f2[16 + d]))));
          }
          unsigned int bu = __float_as_uint(mu), bb = __float_as_uint(mb);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            bu = max(bu, __shfl_xor_sync(0xffffffffu, bu, o));
            bb = max(bb, __shfl_xor_sync(0xffffffffu, bb, o));
          }
          if (lane == 0) {
            const int inst = (int)((ntiles - 1 - q) / GPI);
            atomicMax(vmax + 2 * br.list[inst], bu);
            atomicMax(vmax + 2 * br.list[inst] + 1, bb);
          }
        }
#pragma unroll
        for (int d = 0; d < 16; ++d) {
          const float ux = f0[d], uy = f0[16 + d], uz = f1[d], bx = f1[16 + d], by = f2[d], bz = f2[16 + d];
          float pr, pi;
          if (t == 0) {
            const float tzz = bz * bz - uz * uz;
            pr = (bx * bx - ux * ux) - tzz;
            pi = (by * by - uy * uy) - tzz;
          } else if (t == 1) {
            pr = bx * by - ux * uy;
            pi = bx * bz - ux * uz;
          } else if (t == 2) {
            pr = by * bz - uy * uz;
            pi = ux * by - bx * uy;
          } else {
            pr = ux * bz - bx * uz;
            pi = uy * bz - by * uz;
          }
          a[d] = pr;
          a[16 + d] = pi;
        }
      }
      tc5_store_operand(tlane, a);
      ok = tc5_stage(tbase, L::C_D, b_fwd_hi, b_fwd_lo, barp, phase++);
      if (!ok) break;
      float d[32];
      tc5_ld32(tlane + L::C_D, d);
      float re[16], im[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {  // Z1[j, c] w256^(-j c)
        re[c] = d[c] * tw_c[c] + d[16 + c] * tw_s[c];
        im[c] = d[16 + c] * tw_c[c] - d[c] * tw_s[c];
      }
      tc5_transpose(tb, j, re, im);
#pragma unroll
      for (int b = 0; b < 16; ++b) { a[b] = re[b]; a[16 + b] = im[b]; }
      tc5_store_operand(tlane, a);
      ok = tc5_stage(tbase, L::C_D, b_fwd_hi, b_fwd_lo, barp, phase++);
      if (!ok) break;
      tc5_ld32(tlane + L::C_D, d);  // lane (r, q0 = j): Z[j + 16 q1], re d[q1], im d[16 + q1]
      // two-for-one split: A[k] = (Z[k] + conj Z[N-k]) / 2, B[k] = (Z[k] - conj Z[N-k]) / (2 i),
      // k = j + 16 q1 < KX; Z[N - k] sits on lane 16 - j at q1' = 15 - q1 (j > 0) or on this lane
      // at (16 - q1) mod 16 (j = 0)
      float2* outa = rowp + (2 * t) * slot;
      float2* outb = rowp + (2 * t + 1) * slot;
      const int src_lane = (lane & 16) | ((16 - j) & 15);
#pragma unroll
      for (int q1 = 0; q1 * 16 < KX; ++q1) {
        const float prx = __shfl_sync(0xffffffffu, d[15 - q1], src_lane);
        const float pry = __shfl_sync(0xffffffffu, d[31 - q1], src_lane);
        const int self = (16 - q1) & 15;
        const float2 pz = j == 0 ? make_float2(d[self], d[16 + self]) : make_float2(prx, pry);
        const int k = j + 16 * q1;
        if (k < KX) {
          const float2 z = make_float2(d[q1], d[16 + q1]);
          const float2 zc = make_float2(pz.x, -pz.y);
          const float2 s = cadd(z, zc), df = csub(z, zc);
          outa[k] = make_float2(0.5f * s.x, 0.5f * s.y);
          outb[k] = make_float2(0.5f * df.y, -0.5f * df.x);
        }
      }
    }
  }
  if (!ok && tid == 0) atomicExch(table + L::ERR, 1u);
  cp_async_wait<0>();
  tc5_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "n"(L::TMEM_COLS) : "memory");
  }
}

}  // namespace mhdgb
