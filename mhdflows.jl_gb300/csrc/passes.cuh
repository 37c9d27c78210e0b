// Pass kernels of the pruned pseudospectral MHD right-hand side (sm_103a).
//
// Data layouts in HBM (complex = float2, kx fastest everywhere, rows padded to kxp):
//   state   S[f][kz'][ky'][kx]          retained band only (kx < Kx, ky', kz' kept indices)
//   colbuf  A[z][ky'][slot][kx]         after the z pass (inverse) / before it (forward)
//   rowbuf  B[z][y][slot][kx]           after the y pass (inverse) / before it (forward)
// 8 slots per (z, ky') and (z, y): fields 0..5 on the way in, products 0..7 on the way out; with
// volume penalisation 14 slots, the six penalty fields in slots 8..13 on the way out.
// A kept index j maps to frequency index j (j < Kp) or j + n - K2 (negative wavenumbers).
#pragma once
#include <cuda.h>

#include "fft_core.cuh"

namespace mhdgb {

struct Geom {
  int n;      // points per axis
  int kx;     // kept rfft-axis modes
  int kxp;    // padded row length
  int kp;     // kept non-negative full-axis modes
  int kn;     // kept negative full-axis modes
  int k2;     // kp + kn
  float kscale;  // 2*pi/L
};

__host__ __device__ inline int kept_of_freq(const Geom& g, int f) {
  return f < g.kp ? f : (f >= g.n - g.kn ? f - g.n + g.k2 : -1);
}
__host__ __device__ inline int freq_of_kept(const Geom& g, int j) { return j < g.kp ? j : j + g.n - g.k2; }
__host__ __device__ inline int signed_of_kept(const Geom& g, int j) { return j < g.kp ? j : j - g.k2; }
// kept index of a signed wavenumber, -1 if it lies in the alias band
__host__ __device__ inline int kept_of_signed(const Geom& g, int s) {
  return s >= 0 ? (s < g.kp ? s : -1) : (s >= -g.kn ? s + g.k2 : -1);
}

// Kept modes of the 2/3 rule for n points as compile-time constants, with the double arithmetic of
// FourierFlows' getaliasedwavenumbers at aliased fraction 1/3: the alias band of an axis is the
// 1-based index range floor((1-a)/2 n)+1 .. ceil((1+a)/2 n).  kept_kx_of is the number of kept
// rfft-axis modes and of kept non-negative full-axis modes; kept_kn_of the kept negative ones.
__host__ __device__ constexpr int kept_kx_of(int n) { return (int)((1.0 - 1.0 / 3.0) / 2.0 * n); }
__host__ __device__ constexpr int kept_kn_of(int n) {
  const double hi = (1.0 + 1.0 / 3.0) / 2.0 * n;
  const int c = (int)hi;
  return n - (c < hi ? c + 1 : c);
}

struct BlockSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

// Barrier over the threads that share one row's shared-memory buffers: a warp when a row (or
// several rows) fits in one warp, otherwise a named barrier over the row's G threads.
template <int G>
struct RowSync {
  int id;
  __device__ __forceinline__ void operator()() const {
    if constexpr (G <= 32) {
      __syncwarp();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(G) : "memory");
    }
  }
};

// Batched work: the kernels walk the active instances list[0..*count) of a size class; an
// instance's buffers sit at slot * (slot stride) inside pools shared by the class.  Reading the
// count from device memory lets membership change between steps without new launches.
struct BatchRef {
  const int* list;   // active slots
  const int* count;  // number of active slots
};

// Volume-penalisation inputs of the x rows (src/Solver/VPSolver.jl): per slot the mask chi
// (n^3 floats) and the wall fields U0x U0y U0z B0x B0y B0z (6 n^3 floats), all in the reference's
// (x, y, z) order, x fastest: the row of physical (y, z) starts at (z n + y) n.
struct VpRef {
  const float* chi;
  const float* wall;
  long long cs;  // n^3: field stride; slot strides cs (chi) and 6 cs (wall)
};

struct SlotParams {
  float nu, eta, dt;
  float tdiff;  // diffusive time-step limit of the on-device CFL (0: none)
  // A99 random forcing of the velocity (fA = 0: off): amplitude, spectrum peak, width^2,
  // shape parameter b and generator seed
  float fA, fkf, fs2, fb;
  unsigned long long fseed;
};

struct ColArgs {
  const float2* src;
  float2* dst;
  long long sF, sO, sR;  // source strides (complex elements): field/slot, outer, row
  long long dF, dO, dR;  // destination strides
  long long sI, dI;      // source / destination slot strides (instances of a size class)
  // the right-hand side's z_forward only (else hx == nullptr): once its tiles are done, the pass
  // writes the Hermitian part of the stage state's kx = 0 plane (herm_kx0_items) from the state
  // pool hx (field stride hfs, slot stride hsI) into hout (slot stride hoI)
  const float2* hx;
  float2* hout;
  long long hfs, hsI, hoI;
};

// Hermitian part of the kx = 0 plane of the six fields of every active instance:
// H(k) = (X(k) + conj X(-k)) / 2, with X(-k) = 0 when -k is in the alias band, stored as
// H[f][kz'][ky'].  The reference's diffusion term is computed from the re-transformed physical
// field, rfft(irfft(X)), which is exactly this on the kx = 0 plane.  Items (instance, field, kz',
// ky') with ky' fastest, threads t0, t0 + stride, ... of a grid-stride walk.
__device__ __forceinline__ void herm_kx0_items(const float2* __restrict__ Xpool, float2* __restrict__ Hpool,
                                               const Geom& geo, long long fs, long long stI, long long hI,
                                               BatchRef br, long long t0, long long stride) {
  const long long pl = (long long)geo.k2 * geo.k2;
  const long long total = (long long)(*br.count) * 6 * pl;
  for (long long i = t0; i < total; i += stride) {
    const int inst = (int)(i / (6 * pl));
    const long long r = i - inst * 6 * pl;
    const int c = (int)(r / pl);
    const long long p = r - c * pl;
    const int jz = (int)(p / geo.k2), jy = (int)(p - (long long)jz * geo.k2);
    const int slot = br.list[inst];
    const float2* X = Xpool + slot * stI + c * fs;
    const int py = kept_of_signed(geo, -signed_of_kept(geo, jy));
    const int pz = kept_of_signed(geo, -signed_of_kept(geo, jz));
    const float2 xk = X[((long long)jz * geo.k2 + jy) * geo.kxp];
    const float2 q = (py >= 0 && pz >= 0) ? X[((long long)pz * geo.k2 + py) * geo.kxp] : make_float2(0.f, 0.f);
    Hpool[slot * hI + c * pl + p] = make_float2(0.5f * (xk.x + q.x), 0.5f * (xk.y - q.y));
  }
}

// ------------------------------------------------------------------------------------------
// Column pass: one length-n transform per (field, outer index, kx column); TX columns per tile.
// Persistent CTAs walk the tiles; the next tile's rows are fetched with cp.async into a second
// shared-memory buffer while the current one is transformed, and the buffer that was just read
// into registers doubles as the exchange space of the transform.
// PIN: input rows are kept indices (pruned inverse input).  POUT: only kept outputs stored.
// ------------------------------------------------------------------------------------------
struct ColWork {
  int tiles_x;  // kx tiles
  int outer;    // outer index count
  int nf;       // fields / slots
  int rows_in;  // rows staged per tile (K2 for pruned input, n otherwise)
};

// Rows 0..rows-1 of a TX-column tile starting at column col0 -> buf[row'][TX] (16-byte chunks;
// chunks past the padded row length are skipped).  Each thread keeps one chunk column.  With
// PIN the rows are kept indices and land at their frequency position row' (non-negative modes
// in place, negative modes at row + n - K2); the alias rows in between are zero-filled, so the
// transform reads every row unconditionally.
template <int TX, int NT, int N, bool PIN, int G>
__device__ __forceinline__ void col_prefetch(float2* buf, const float2* src, long long sR, int rows, int col0,
                                             const Geom& geo) {
  constexpr int CH = TX / 2;       // 16-byte chunks per row
  constexpr int RSTEP = NT / CH;   // rows advanced per sweep
  const int q = threadIdx.x % CH;
  int row = threadIdx.x / CH;
  if (PIN) {
    // the transform reads the alias rows only inside lane groups (G consecutive rows) that also
    // hold kept rows; groups wholly inside the alias band are compile-time zeros
    constexpr int KP = kept_kx_of(N), KN = kept_kn_of(N);
    float4* zb = reinterpret_cast<float4*>(buf + KP * TX);
    constexpr int nz = (N - KP - KN) * CH;
    for (int c = threadIdx.x; c < nz; c += NT) {
      const int r = KP + c / CH;
      const int gs = r / G * G;
      if (gs < KP || gs + G - 1 >= N - KN) zb[c] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  if (col0 + 2 * q >= geo.kxp) return;
  const float2* s = src + row * sR + col0 + 2 * q;
  for (; row < rows; row += RSTEP, s += RSTEP * sR) {
    const int drow = PIN ? (row < geo.kp ? row : row + N - geo.k2) : row;
    cp_async16(buf + drow * TX + 2 * q, s);
  }
}

// NBUF tile buffers: NBUF - 1 tiles are being fetched while one is transformed.  TWS: the
// stage twiddles are copied into shared memory behind the tile buffers (plain shared loads in
// the exchanges instead of read-only global loads).
template <class P0, int TX, int DIR, bool PIN, bool POUT, int MINB, int NBUF, bool TWS = false>
__global__ void __launch_bounds__(TX * P0::G, MINB)
    col_pass_kernel(ColArgs a, Geom geo, ColWork w, BatchRef br, const float2* __restrict__ tw) {
  static_assert(NBUF >= 2 && NBUF <= 4, "two to four tile buffers");
  using P = Unpadded<P0>;
  extern __shared__ float2 smem[];
  constexpr int G = P::G, V = P::V, N = P::N, NT = TX * P0::G;
  const int tx = threadIdx.x % TX, g = threadIdx.x / TX;
  const int per = w.tiles_x * w.outer * w.nf;  // tiles of one instance
  const int total = *br.count * per;
  // Kept band along the transformed axis (compile-time; the host checks geo.kp / geo.kn): an
  // element group (d, n0) of the input or (d, e) of the output covers the frequencies
  // G*d + LI*n0 + g (or G*d + LF*e + g) of the G lanes; a group inside the alias band for every
  // lane is a compile-time zero (pruned input) or never stored (pruned output), so the first or
  // last transform stage is pruned by constant folding.
  constexpr int KP = kept_kx_of(N), KN = kept_kn_of(N);
  const int dR = (int)a.dR;  // row offsets inside one buffer fit 32 bits for n <= 512
  const int shift = (N - KP - KN) * dR;
  // Tile index t = tx_t + tiles_x*(f + nf*(o + outer*inst)): the outer index (z of the y passes)
  // varies slowest, so the last tiles of a pass write the last outer planes, the part of its
  // output still in L2 when the next pass starts.  The grid-stride walk advances t by gridDim.x
  // with a carrying mixed-radix add, so divisions happen once per CTA.
  struct Cur { int tx, o, f, inst; };
  auto decompose = [&](int t) {
    Cur c;
    c.tx = t % w.tiles_x;
    int r = t / w.tiles_x;
    c.f = r % w.nf;
    r /= w.nf;
    c.o = r % w.outer;
    c.inst = r / w.outer;
    return c;
  };
  const Cur gstep = decompose(gridDim.x);
  auto advance = [&](Cur c) {
    int carry;
    c.tx += gstep.tx; carry = c.tx >= w.tiles_x; if (carry) c.tx -= w.tiles_x;
    c.f += gstep.f + carry; carry = c.f >= w.nf; if (carry) c.f -= w.nf;
    c.o += gstep.o + carry; carry = c.o >= w.outer; if (carry) c.o -= w.outer;
    c.inst += gstep.inst + carry;
    return c;
  };
  // instance offsets: list lookups only when the instance changes (a dependent global load on
  // every tile's address otherwise)
  int src_inst = -1, dst_inst = -1;
  long long src_off = 0, dst_off = 0;
  auto tile_src = [&](const Cur& c) {
    if (c.inst != src_inst) {
      src_inst = c.inst;
      src_off = br.list[c.inst] * a.sI;
    }
    return a.src + src_off + c.f * a.sF + (long long)c.o * a.sO;
  };
  float2* tws = smem + NBUF * (N * TX);
  if constexpr (TWS)
    for (int i = threadIdx.x; i < PlanTw<P0>::SIZE; i += NT) tws[i] = __ldg(tw + i);
  int t = blockIdx.x;
  Cur cur_t = decompose(t);
  // prologue: the first NBUF - 1 tiles of this CTA (one commit group each, empty past the end)
  int tp = t;
  Cur pre_t = cur_t;
#pragma unroll
  for (int j = 0; j < NBUF - 1; ++j) {
    if (tp < total) col_prefetch<TX, NT, N, PIN, P::G>(smem + j * (N * TX), tile_src(pre_t), a.sR, w.rows_in, pre_t.tx * TX, geo);
    cp_async_commit();
    tp += gridDim.x;
    pre_t = advance(pre_t);
  }
  for (int it = 0; t < total; t += gridDim.x, ++it) {
    float2* cur = smem + (it % NBUF) * (N * TX);
    // tile it + NBUF - 1 into the buffer that tile it - 1 used (freed by the barrier ending the
    // previous iteration)
    if (tp < total)
      col_prefetch<TX, NT, N, PIN, P::G>(smem + ((it + NBUF - 1) % NBUF) * (N * TX), tile_src(pre_t), a.sR, w.rows_in,
                                         pre_t.tx * TX, geo);
    cp_async_commit();
    tp += gridDim.x;
    pre_t = advance(pre_t);
    cp_async_wait<NBUF - 1>();
    __syncthreads();
    const int inst = cur_t.inst, f = cur_t.f, o = cur_t.o;
    const int kxg = cur_t.tx * TX + tx;
    cur_t = advance(cur_t);
    float2 v[1][V];
#pragma unroll
    for (int d = 0; d < P::DI; ++d)
#pragma unroll
      for (int n0 = 0; n0 < P::R0; ++n0) {
        const int rmin = G * d + P::LI * n0;
        if (PIN && rmin >= KP && rmin + G - 1 < N - KN)
          v[0][d * P::R0 + n0] = make_float2(0.f, 0.f);
        else
          v[0][d * P::R0 + n0] = cur[(g + rmin) * TX + tx];
      }
    __syncthreads();  // cur is now free: reuse it as the exchange buffer
    fft_run<P, DIR, 1, 0, TX, !PIN, TWS>(v, cur, tx, g, TWS ? tws : tw, BlockSync{});
    if (kxg < geo.kx) {
      if (inst != dst_inst) {
        dst_inst = inst;
        dst_off = br.list[inst] * a.dI;
      }
      float2* dst = a.dst + dst_off + f * a.dF + (long long)o * a.dO + kxg;
#pragma unroll
      for (int d = 0; d < P::DF; ++d) {
        const int base = (g + G * d) * dR;
#pragma unroll
        for (int e = 0; e < P::RF; ++e) {
          const int kmin = G * d + P::LF * e;
          if (POUT && kmin >= KP && kmin + G - 1 < N - KN) continue;  // no lane keeps this group
          const int k = g + kmin;
          const int off = base + e * (P::LF * dR);
          if (!POUT || k < KP) {
            dst[off] = v[0][d * P::RF + e];
          } else if (k >= N - KN) {
            dst[off - shift] = v[0][d * P::RF + e];
          }
        }
      }
    }
    __syncthreads();  // all exchange reads of cur done before it is refilled
  }
  cp_async_wait<0>();
  if (a.hx) herm_kx0_items(a.hx, a.hout, geo, a.hfs, a.hsI, a.hoI, br, (long long)blockIdx.x * NT + threadIdx.x,
                           (long long)gridDim.x * NT);
}

// ------------------------------------------------------------------------------------------
// TMA-fed column pass: the same transform as col_pass_kernel, with each tile brought into
// shared memory by one thread's cp.async.bulk.tensor copies (a 5-D tensor map over the pass's
// source array) completing on an mbarrier per buffer.  Pruned inputs take two boxes (the kept
// non-negative rows, then the kept negative rows at their frequency position); full inputs one
// box, or two of 256 rows.  Every wait is bounded (about one second of %globaltimer): on a
// timeout the kernel records the failure in *err, stops taking tiles, waits (bounded again) for
// the copies it issued and returns.
// ------------------------------------------------------------------------------------------
struct TmaCoords {
  int rowdim, odim, fdim, idim;  // tensor-map dimensions of the transformed axis, outer index, field, slot
  int rb;                        // rows per box
};

__device__ __forceinline__ unsigned int smem_u32(const void* p) { return (unsigned int)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// true when the barrier's phase `parity` completed within limit_ns (about a second by default)
__device__ __forceinline__ bool mbar_wait(unsigned int bar, unsigned int parity,
                                          unsigned long long limit_ns = 1000000000ull) {
  const unsigned long long t0 = global_ns();
  while (true) {
    unsigned int done;
    asm volatile(
        "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n selp.u32 %0, 1, 0, P;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}
__device__ __forceinline__ void tma_load5(unsigned int dst, const void* map, int c0, int c1, int c2, int c3, int c4,
                                          unsigned int bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
      "[%7];\n" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}

// TWS: the stage twiddles are copied into shared memory behind the barriers.
template <class P0, int TX, int DIR, bool PIN, bool POUT, int MINB, int NBUF, bool TWS = false>
__global__ void __launch_bounds__(TX * P0::G, MINB)
    col_pass_tma_kernel(ColArgs a, Geom geo, ColWork w, BatchRef br, const float2* __restrict__ tw,
                        const __grid_constant__ CUtensorMap map, TmaCoords tc, int* err) {
  static_assert(NBUF >= 2 && NBUF <= 4, "two to four tile buffers");
  using P = Unpadded<P0>;
  // dynamic shared memory only (its base is then 1024-byte aligned): NBUF tile buffers, then the
  // NBUF mbarriers and the abort flag (16 bytes), then with TWS the stage twiddles
  extern __shared__ __align__(128) float2 smem[];
  constexpr int G = P::G, V = P::V, N = P::N, NT = TX * P0::G;
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + NBUF * N * TX);
  volatile int& abort_flag = *reinterpret_cast<volatile int*>(bars + NBUF);
  float2* tws = smem + NBUF * N * TX + NBUF + 2;
  if constexpr (TWS)
    for (int i = threadIdx.x; i < PlanTw<P0>::SIZE; i += NT) tws[i] = __ldg(tw + i);
  constexpr int KP = kept_kx_of(N), KN = kept_kn_of(N);
  const int tx = threadIdx.x % TX, g = threadIdx.x / TX;
  const int per = w.tiles_x * w.outer * w.nf;
  const int total = *br.count * per;
  const int dR = (int)a.dR;
  const int shift = (N - KP - KN) * dR;
  const unsigned int tx_bytes = PIN ? 2u * tc.rb * TX * 8u : (unsigned int)N * TX * 8u;
  if (threadIdx.x == 0) {
    abort_flag = (smem_u32(smem) & 127u) != 0;  // TMA destinations must be 128-byte aligned
    if (abort_flag) atomicExch(err, 2);
    for (int b = 0; b < NBUF; ++b)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[b])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (abort_flag) return;
  struct Cur { int tx, o, f, inst; };
  auto decompose = [&](int t) {
    Cur c;
    c.tx = t % w.tiles_x;
    int r = t / w.tiles_x;
    c.f = r % w.nf;
    r /= w.nf;
    c.o = r % w.outer;
    c.inst = r / w.outer;
    return c;
  };
  const Cur gstep = decompose(gridDim.x);
  auto advance = [&](Cur c) {
    int carry;
    c.tx += gstep.tx; carry = c.tx >= w.tiles_x; if (carry) c.tx -= w.tiles_x;
    c.f += gstep.f + carry; carry = c.f >= w.nf; if (carry) c.f -= w.nf;
    c.o += gstep.o + carry; carry = c.o >= w.outer; if (carry) c.o -= w.outer;
    c.inst += gstep.inst + carry;
    return c;
  };
  // tile c into buffer b: zero the alias rows the transform reads (all threads), then thread 0
  // arms the barrier and issues the box copies
  auto issue = [&](const Cur& c, int b) {
    float2* buf = smem + b * (N * TX);
    if (PIN) {
      constexpr int CH = TX / 2;
      float4* zb = reinterpret_cast<float4*>(buf + KP * TX);
      constexpr int nz = (N - KP - KN) * CH;
      for (int q = threadIdx.x; q < nz; q += NT) {
        const int r = KP + q / CH;
        const int gs = r / G * G;
        if (gs < KP || gs + G - 1 >= N - KN) zb[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    if (threadIdx.x == 0) {
      const unsigned int bar = smem_u32(&bars[b]);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier generic reads of buf
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(tx_bytes) : "memory");
      int cc[5] = {c.tx * TX, 0, 0, 0, 0};
      cc[tc.odim] = c.o;
      cc[tc.fdim] = c.f;
      cc[tc.idim] = br.list[c.inst];
      if (PIN) {
        cc[tc.rowdim] = 0;
        tma_load5(smem_u32(buf), &map, cc[0], cc[1], cc[2], cc[3], cc[4], bar);
        cc[tc.rowdim] = KP;
        tma_load5(smem_u32(buf + (N - KN) * TX), &map, cc[0], cc[1], cc[2], cc[3], cc[4], bar);
      } else {
        for (int r0 = 0; r0 < N; r0 += tc.rb) {
          cc[tc.rowdim] = r0;
          tma_load5(smem_u32(buf + r0 * TX), &map, cc[0], cc[1], cc[2], cc[3], cc[4], bar);
        }
      }
    }
  };
  int t = blockIdx.x;
  Cur cur_t = decompose(t);
  int tp = t;
  Cur pre_t = cur_t;
  int issued = 0;  // tiles issued by this CTA (tile k uses buffer k % NBUF, phase (k / NBUF) & 1)
#pragma unroll
  for (int j = 0; j < NBUF - 1; ++j) {
    if (tp < total) { issue(pre_t, j); ++issued; }
    tp += gridDim.x;
    pre_t = advance(pre_t);
  }
  int dst_inst = -1;
  long long dst_off = 0;
  int it = 0;
  for (; t < total; t += gridDim.x, ++it) {
    if (tp < total) { issue(pre_t, (it + NBUF - 1) % NBUF); ++issued; }
    tp += gridDim.x;
    pre_t = advance(pre_t);
    if (!mbar_wait(smem_u32(&bars[it % NBUF]), (unsigned int)((it / NBUF) & 1))) {
      atomicExch(err, 1);
      abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag) break;
    float2* cur = smem + (it % NBUF) * (N * TX);
    const int inst = cur_t.inst, f = cur_t.f, o = cur_t.o;
    const int kxg = cur_t.tx * TX + tx;
    cur_t = advance(cur_t);
    float2 v[1][V];
#pragma unroll
    for (int d = 0; d < P::DI; ++d)
#pragma unroll
      for (int n0 = 0; n0 < P::R0; ++n0) {
        const int rmin = G * d + P::LI * n0;
        if (PIN && rmin >= KP && rmin + G - 1 < N - KN)
          v[0][d * P::R0 + n0] = make_float2(0.f, 0.f);
        else
          v[0][d * P::R0 + n0] = cur[(g + rmin) * TX + tx];
      }
    __syncthreads();  // cur is now free: reuse it as the exchange buffer
    fft_run<P, DIR, 1, 0, TX, !PIN, TWS>(v, cur, tx, g, TWS ? tws : tw, BlockSync{});
    if (kxg < geo.kx) {
      if (inst != dst_inst) {  // list lookup only when the instance changes
        dst_inst = inst;
        dst_off = br.list[inst] * a.dI;
      }
      float2* dst = a.dst + dst_off + f * a.dF + (long long)o * a.dO + kxg;
#pragma unroll
      for (int d = 0; d < P::DF; ++d) {
        const int base = (g + G * d) * dR;
#pragma unroll
        for (int e = 0; e < P::RF; ++e) {
          const int kmin = G * d + P::LF * e;
          if (POUT && kmin >= KP && kmin + G - 1 < N - KN) continue;
          const int k = g + kmin;
          const int off = base + e * (P::LF * dR);
          if (!POUT || k < KP) {
            dst[off] = v[0][d * P::RF + e];
          } else if (k >= N - KN) {
            dst[off - shift] = v[0][d * P::RF + e];
          }
        }
      }
    }
    __syncthreads();  // all exchange reads of cur done before it is refilled
  }
  // after an abort: let the copies this CTA issued and did not consume land before exiting
  if (abort_flag && threadIdx.x == 0) {
    for (int k = it; k < issued; ++k) (void)mbar_wait(smem_u32(&bars[k % NBUF]), (unsigned int)((k / NBUF) & 1));
  }
  if (a.hx) herm_kx0_items(a.hx, a.hout, geo, a.hfs, a.hsI, a.hoI, br, (long long)blockIdx.x * NT + threadIdx.x,
                           (long long)gridDim.x * NT);
}

// ------------------------------------------------------------------------------------------
// x rows: Hermitian two-for-one helpers.
// ------------------------------------------------------------------------------------------
// Input of an inverse (c2r) transform of two half-spectrum rows f1, f2 with KX kept modes
// (plain loads: the rows may live in global or in shared memory):
// z[n] = F1[n] + i F2[n] with F[n-n] = conj(F[n]); the kx = 0 imaginary parts are dropped,
// which is what a c2r transform does with a non-Hermitian kx = 0 plane.  Elements whose index
// lies in the alias band for every lane are compile-time zeros, so the first stage of the
// transform is pruned by constant folding.
// ZB: the second field is zero (f2 is not read).
template <class P, int KX, bool ZB = false>
__device__ __forceinline__ void load_herm_pair(float2 (&v)[P::V], const float2* __restrict__ f1,
                                               const float2* __restrict__ f2, int g) {
#pragma unroll
  for (int d = 0; d < P::DI; ++d)
#pragma unroll
    for (int n0 = 0; n0 < P::R0; ++n0) {
      const int nmin = P::G * d + P::LI * n0;  // element index of lane 0
      float2 z = make_float2(0.f, 0.f);
      if (nmin < KX || nmin + P::G - 1 > P::N - KX) {  // some lane holds a kept mode
        const int n = g + nmin;
        if (n < KX) {
          float2 a = f1[n], b = ZB ? make_float2(0.f, 0.f) : f2[n];
          if (n == 0) { a.y = 0.f; b.y = 0.f; }
          z = make_float2(a.x - b.y, a.y + b.x);
        } else if (n > P::N - KX) {
          const int m = P::N - n;
          float2 a = f1[m], b = ZB ? make_float2(0.f, 0.f) : f2[m];
          z = make_float2(a.x + b.y, b.x - a.y);
        }
      }
      v[d * P::R0 + n0] = z;
    }
}

// Split Z = FFT(pa + i pb) into the half spectra of pa and pb for k < kx and store them.
// sb holds Z[k] for every needed k (k < kx and k > n - kx).
__device__ __forceinline__ void store_split_pair(const float2* sb, int n, int kx, int g, int G,
                                                 float2* outa, float2* outb) {
  for (int k = g; k < kx; k += G) {
    const float2 z = sb[k];
    const float2 zc = cconj(sb[(n - k) % n]);
    const float2 s = cadd(z, zc), df = csub(z, zc);
    outa[k] = make_float2(0.5f * s.x, 0.5f * s.y);
    outb[k] = make_float2(0.5f * df.y, -0.5f * df.x);
  }
}

// The same split straight from the registers of a forward transform whose G lanes sit in one
// warp (G <= 32, lanes rowbase .. rowbase+G-1).  With the output layout of fft_run,
// register (m % DF)*RF + m / DF of lane g holds Z[g + G m], and Z[N - g - G m] sits in lane
// (G - g) % G at index V-1-m (g > 0) or in lane 0 itself at index (V-m) % V (g = 0): one
// shuffle per needed output, no shared memory.  Outputs of every lane past the kept band are
// never read, so the last stage of the transform is pruned as dead code.
template <class P, int KX>
__device__ __forceinline__ void store_split_shfl(const float2 (&v)[P::V], int g, int rowbase, float2* outa,
                                                 float2* outb) {
  constexpr int G = P::G, V = P::V, DF = P::DF, RF = P::RF;
  static_assert(G <= 32, "the shuffle split needs the row inside one warp");
  const int partner = rowbase + (G - g) % G;
#pragma unroll
  for (int m = 0; m < V; ++m) {
    if (G * m >= KX) break;  // no lane holds a kept output from here on (compile-time)
    const float2 z = v[(m % DF) * RF + m / DF];
    const int mp = V - 1 - m, m0 = (V - m) % V;
    const float2 pz = v[(mp % DF) * RF + mp / DF];
    float2 p;
    p.x = __shfl_sync(0xffffffffu, pz.x, partner);
    p.y = __shfl_sync(0xffffffffu, pz.y, partner);
    if (g == 0) p = v[(m0 % DF) * RF + m0 / DF];
    const int k = g + G * m;
    if (k < KX) {
      const float2 zc = cconj(p);
      const float2 s = cadd(z, zc), df = csub(z, zc);
      outa[k] = make_float2(0.5f * s.x, 0.5f * s.y);
      outb[k] = make_float2(0.5f * df.y, -0.5f * df.x);
    }
  }
}

template <class P>
struct RowCfg {
  using PR = typename Reverse<P>::type;
  static constexpr int a = P::SMEM > PR::SMEM ? P::SMEM : PR::SMEM;
  static constexpr int b = a > P::N ? a : P::N;
  static constexpr int TS = (b + 1) / 2 * 2;  // words per transform buffer (even: 16-byte aligned)
};

// Fused x pass: per physical row (z, y): 3 inverse c2r pairs -> 6 physical fields -> 8 products
// -> 4 forward r2c pairs -> 8 half-spectrum rows, written back over the same row slots.
// Products: Dxz = (bx^2-ux^2)-(bz^2-uz^2), Dyz = (by^2-uy^2)-(bz^2-uz^2), Txy, Txz, Tyz with
// Tij = bi*bj - ui*uj, and Axy, Axz, Ayz with Aij = ui*bj - bi*uj.
// A row group is RPG = max(1, 32/G) consecutive rows handled by one warp (G <= 32) or one row
// handled by G/32 warps.  Groups are persistent: while a group transforms its rows, cp.async
// brings the six field rows of its next rows into the other half of a double buffer.
// DIRECT: the field rows are read from global memory straight into registers (coalesced across
// the lanes of a row), with no staging copy in shared memory.
template <class P, int NTS = 1, bool DIRECT = false>
struct XCfg {
  static constexpr int G = P::G;
  static constexpr int RPG = G >= 32 ? 1 : 32 / G;        // rows per group
  static constexpr int TPG = G >= 32 ? G : 32;            // threads per group
  static constexpr int TS = RowCfg<P>::TS;                // exchange words per transform
  static __host__ __device__ int stage_words(int kxp) { return DIRECT ? 0 : RPG * 6 * kxp; }
  // two staging buffers of the six field rows, then NTS exchange buffers per row
  static __host__ __device__ int group_words(int kxp) { return 2 * stage_words(kxp) + RPG * NTS * TS; }
};

// Variants (chosen per grid size by the autotuner): NTI inverse transforms (1 or 3) and NTF
// forward transforms (1, 2 or 4) go through the stages together, sharing the twiddle loads and
// the barriers and giving each thread more independent work; MINB is the occupancy bound.
//
// VPM (volume penalisation, VP_UᵢUpdate! / VP_BᵢUpdate! of src/Solver/VPSolver.jl:20-58): 0 off;
// 1 adds the penalty fields chi u and chi B (walls U0 = B0 = 0); 2 adds chi (u - U0), chi (B - B0).
// They leave as three more forward pairs in slots 8..13; the epilogue scales and projects them.
// HDX (hydrodynamics, HDcalcN!): three fields in (ux uy | uz), B = 0 folded at compile time, two
// inverse and three forward transforms; the products are the first five of the MHD set (the
// sixth slot written is zero).
template <class P, int GROUPS, int NTI, int NTF, int MINB, int VPM = 0, bool HDX = false, bool DIRECT = false>
__global__ void __launch_bounds__(GROUPS * XCfg<P>::TPG, MINB)
    x_fused_kernel(float2* pool, Geom geo, long long rowstride, long long slot, long long istride, BatchRef br,
                   const float2* __restrict__ tw, const float2* __restrict__ twr, unsigned int* vmax, VpRef vp) {
  using PR = typename Reverse<P>::type;
  constexpr int NTS = NTI > NTF ? NTI : NTF;
  using XC = XCfg<P, NTS, DIRECT>;
  static_assert(NTI == 1 || NTI == 3, "inverse transforms go one or three at a time");
  static_assert(NTF == 1 || NTF == 2 || NTF == 4, "forward transforms go one, two or four at a time");
  static_assert(NTF == 1 || P::G <= 32, "batched forward transforms need the row inside one warp");
  static_assert(VPM == 0 || NTF == 1, "the penalty pairs go one at a time");
  static_assert(!HDX || (NTI == 1 && NTF == 1), "the hydrodynamic form goes one transform at a time");
  // forward transform pairs per row; the hydrodynamic form with penalisation fills the three
  // spare product slots: pair 2 = (-uy uz, n^3 chi (uz - U0z)), pair 3 = n^3 (chi (ux - U0x),
  // chi (uy - U0y))
  constexpr int NPAIR = HDX ? (VPM ? 4 : 3) : VPM ? 7 : 4;
  constexpr int NINV = HDX ? 2 : 3;             // inverse transforms (field pairs) per row
  constexpr int G = P::G, V = P::V, N = P::N, RPG = XC::RPG, TPG = XC::TPG, TS = XC::TS;
  constexpr int KX = kept_kx_of(N);  // the host checks geo.kx == KX
  extern __shared__ float2 smem[];
  const int kxp = geo.kxp;
  const int grp = threadIdx.x / TPG;
  const int gt = threadIdx.x % TPG;          // thread within group
  const int rr = gt / G, g = gt % G;         // row within group, lane within row
  const int sw = XC::stage_words(kxp);
  float2* gs = smem + grp * XC::group_words(kxp);
  float2* sb = gs + 2 * sw + rr * NTS * TS;
  const RowSync<G> sync{1 + grp};
  constexpr int GPI = N * N / RPG;  // row groups per instance
  const long long ngroups = (long long)(*br.count) * GPI;
  const int chunks_row = (HDX ? 3 : 6) * kxp / 2;  // 16-byte chunks of the contiguous field rows (slot == kxp)
  // first row of row group q, inside its instance's rowbuf.  Groups are taken from the last one
  // down: the y pass before this kernel wrote the last z planes last (still in L2), and the y
  // pass after it reads the first z planes first (written here last).
  auto group_rows = [&](long long q) {
    q = ngroups - 1 - q;
    const int inst = (int)(q / GPI);
    return pool + br.list[inst] * istride + (q - (long long)inst * GPI) * RPG * rowstride;
  };

  // rows q*RPG .. q*RPG+RPG-1 -> dst (each row's six fields contiguous)
  auto prefetch = [&](long long q, float2* dst) {
    const float2* src = group_rows(q);
    for (int c = gt; c < RPG * chunks_row; c += TPG) {
      const int r = RPG == 1 ? 0 : c / chunks_row;
      const int cc = RPG == 1 ? c : c - r * chunks_row;
      cp_async16(dst + r * 6 * kxp + 2 * cc, src + r * rowstride + 2 * cc);
    }
  };

  long long q = (long long)blockIdx.x * GROUPS + grp;
  const long long qstep = (long long)gridDim.x * GROUPS;
  if (!DIRECT && q < ngroups) prefetch(q, gs);
  cp_async_commit();
  for (int it = 0; q < ngroups; q += qstep, ++it) {
    const float2* rin;
    if constexpr (DIRECT) {
      // this row's own slots (slot stride == kxp); every lane loads its inputs before any lane
      // stores an output over them (the stores follow the transforms)
      rin = group_rows(q) + rr * rowstride;
    } else {
      const float2* cur = gs + (it & 1) * sw;
      if (q + qstep < ngroups) prefetch(q + qstep, gs + ((it + 1) & 1) * sw);
      cp_async_commit();
      cp_async_wait<1>();
      sync();
      rin = cur + rr * 6 * kxp;
    }
    float2 v[3][V];
#pragma unroll
    for (int t = 0; t < NINV; ++t) {
      if (HDX && t == 1) load_herm_pair<P, KX, true>(v[t], rin + (2 * t) * kxp, nullptr, g);
      else load_herm_pair<P, KX>(v[t], rin + (2 * t) * kxp, rin + (2 * t + 1) * kxp, g);
    }
    if constexpr (NTI == 3) {
      fft_run<P, +1, 3, TS, 1, false>(v, sb, 0, g, tw, sync);
      sync();
    } else {
#pragma unroll
      for (int t = 0; t < NINV; ++t) {
        fft_run<P, +1, 1, TS, 1, false>(reinterpret_cast<float2(&)[1][V]>(v[t]), sb, 0, g, tw, sync);
        sync();
      }
    }
    if constexpr (HDX) {  // B = 0: the second half of pair 1 is zero up to roundoff, pair 2 unused
#pragma unroll
      for (int i = 0; i < V; ++i) {
        v[1][i].y = 0.f;
        v[2][i] = make_float2(0.f, 0.f);
      }
    }
    if (vmax) {
      // max |u_i| and max |B_i| over the physical fields (getCFL! on the last stage's fields);
      // non-negative floats order like their bit patterns, NaN above +inf
      float mu = 0.f, mb = 0.f;
#pragma unroll
      for (int i = 0; i < V; ++i) {
        mu = fmaxf(mu, fmaxf(fabsf(v[0][i].x), fmaxf(fabsf(v[0][i].y), fabsf(v[1][i].x))));
        mb = fmaxf(mb, fmaxf(fabsf(v[1][i].y), fmaxf(fabsf(v[2][i].x), fabsf(v[2][i].y))));
      }
      unsigned int bu = __float_as_uint(mu), bb = __float_as_uint(mb);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        bu = max(bu, __shfl_xor_sync(0xffffffffu, bu, o));
        bb = max(bb, __shfl_xor_sync(0xffffffffu, bb, o));
      }
      if ((threadIdx.x & 31) == 0) {
        const int inst = (int)((ngroups - 1 - q) / GPI);  // the instance of group_rows(q)
        atomicMax(vmax + 2 * br.list[inst], bu);
        atomicMax(vmax + 2 * br.list[inst] + 1, bb);
      }
    }
    float2* rowp = group_rows(q) + rr * rowstride;
    // the penalty inputs of this row at the physical points this thread holds: x = lF + LF e for
    // register d RF + e (the inverse plan's output layout)
    float chi[VPM ? V : 1];
    const float* wrow = nullptr;
    if constexpr (VPM > 0) {
      const long long qr = ngroups - 1 - q;  // the group group_rows(q) addresses
      const int inst = (int)(qr / GPI);
      const long long s = br.list[inst];
      const long long r = (qr - (long long)inst * GPI) * RPG + rr;  // z n + y
      const float* crow = vp.chi + s * vp.cs + r * N;
      if constexpr (VPM == 2) wrow = vp.wall + 6 * s * vp.cs + r * N;
#pragma unroll
      for (int d = 0; d < P::DF; ++d)
#pragma unroll
        for (int e = 0; e < P::RF; ++e) chi[d * P::RF + e] = __ldg(crow + g + G * d + P::LF * e);
    }
    // NTF product pairs at a time: the six fields stay live, each pair is formed just before its
    // forward transform (fewer live registers than all eight products at once)
#pragma unroll
    for (int t0 = 0; t0 < NPAIR; t0 += NTF) {
      float2 w[NTF][V];
#pragma unroll
      for (int j = 0; j < NTF; ++j) {
        const int t = t0 + j;
#pragma unroll
        for (int i = 0; i < V; ++i) {
          const float ux = v[0][i].x, uy = v[0][i].y, uz = v[1][i].x;
          const float bx = v[1][i].y, by = v[2][i].x, bz = v[2][i].y;
          if (HDX && VPM > 0 && t >= 2) {
            if constexpr (HDX && VPM > 0) {
              constexpr float n3 = (float)N * (float)N * (float)N;
              const int x = g + G * (i / P::RF) + P::LF * (i % P::RF);
              auto wall = [&](int c) { return VPM == 2 ? n3 * __ldg(wrow + c * vp.cs + x) : 0.f; };
              // scaled by n^3 to the products' magnitude (n^6 times physical): a pair whose halves
              // differ by n^3 would lose the small half to the large one's rounding in the split
              const float c3 = n3 * chi[i];
              if (t == 2) w[j][i] = make_float2(-uy * uz, c3 * (uz - wall(2)));
              else w[j][i] = make_float2(c3 * (ux - wall(0)), c3 * (uy - wall(1)));
            }
          } else if (t >= 4) {  // penalty pair t - 4: (u x, u y), (u z, B x), (B y, B z) of the field pairs
            if constexpr (VPM > 0) {
              float2 f = v[t - 4][i];
              if constexpr (VPM == 2) {  // the fields are n^3 times physical: so are the walls
                constexpr float n3 = (float)N * (float)N * (float)N;
                const int x = g + G * (i / P::RF) + P::LF * (i % P::RF);
                const long long c0 = (long long)(2 * (t - 4)) * vp.cs;
                f.x = fmaf(-n3, __ldg(wrow + c0 + x), f.x);
                f.y = fmaf(-n3, __ldg(wrow + c0 + vp.cs + x), f.y);
              }
              w[j][i] = make_float2(chi[i] * f.x, chi[i] * f.y);
            }
          } else if (t == 0) {
            const float tzz = bz * bz - uz * uz;
            w[j][i] = make_float2((bx * bx - ux * ux) - tzz, (by * by - uy * uy) - tzz);
          } else if (t == 1) {
            w[j][i] = make_float2(bx * by - ux * uy, bx * bz - ux * uz);
          } else if (t == 2) {
            w[j][i] = make_float2(by * bz - uy * uz, ux * by - bx * uy);
          } else {
            w[j][i] = make_float2(ux * bz - bx * uz, uy * bz - by * uz);
          }
        }
      }
      fft_run<PR, -1, NTF, TS, 1>(w, sb, 0, g, twr, sync);
      if constexpr (G <= 32) {
#pragma unroll
        for (int j = 0; j < NTF; ++j)
          store_split_shfl<PR, KX>(w[j], g, (threadIdx.x & 31) - g, rowp + (2 * (t0 + j)) * slot,
                                   rowp + (2 * (t0 + j) + 1) * slot);
        sync();  // the next transform's first exchange overwrites sb
      } else {
        sync();
#pragma unroll
        for (int d = 0; d < PR::DF; ++d)
#pragma unroll
          for (int e = 0; e < PR::RF; ++e) {
            const int k = g + G * d + PR::LF * e;
            if (k < KX || k > N - KX) sb[k] = w[0][d * PR::RF + e];
          }
        sync();
        store_split_pair(sb, N, KX, g, G, rowp + (2 * t0) * slot, rowp + (2 * t0 + 1) * slot);
        sync();
      }
    }
  }
  cp_async_wait<0>();
}

// Plain c2r of row pairs: spectral rows (2q, 2q+1) -> physical rows times scale (1/n^3: the
// column passes do not normalise).
template <class P, int ROWS>
__global__ void __launch_bounds__(ROWS * P::G) x_c2r_kernel(const float2* src, float* dst, Geom geo, long long srow,
                                                              float scale, const float2* __restrict__ tw) {
  constexpr int G = P::G, V = P::V, N = P::N;
  constexpr int TS = RowCfg<P>::TS;
  extern __shared__ float2 smem[];
  const int r = threadIdx.x / G, g = threadIdx.x % G;
  const long long q = (long long)blockIdx.x * ROWS + r;
  float2 v[1][V];
  load_herm_pair<P, kept_kx_of(P::N)>(v[0], src + (2 * q) * srow, src + (2 * q + 1) * srow, g);
  fft_run<P, +1, 1, TS, 1, false>(v, smem + r * TS, 0, g, tw, RowSync<G>{1 + r});
  float* da = dst + (2 * q) * N;
  float* db = dst + (2 * q + 1) * N;
#pragma unroll
  for (int d = 0; d < P::DF; ++d)
#pragma unroll
    for (int e = 0; e < P::RF; ++e) {
      const int x = g + G * d + P::LF * e;
      da[x] = scale * v[0][d * P::RF + e].x;
      db[x] = scale * v[0][d * P::RF + e].y;
    }
}

// Plain r2c of row pairs: physical rows (2q, 2q+1) -> half-spectrum rows (kx kept modes).
template <class P, int ROWS>
__global__ void __launch_bounds__(ROWS * P::G) x_r2c_kernel(const float* src, float2* dst, Geom geo, long long drow,
                                                              const float2* __restrict__ tw) {
  constexpr int G = P::G, V = P::V, N = P::N;
  constexpr int TS = RowCfg<P>::TS;
  extern __shared__ float2 smem[];
  const int r = threadIdx.x / G, g = threadIdx.x % G;
  const long long q = (long long)blockIdx.x * ROWS + r;
  const float* sa = src + (2 * q) * N;
  const float* sbp = src + (2 * q + 1) * N;
  float2 v[1][V];
#pragma unroll
  for (int d = 0; d < P::DI; ++d)
#pragma unroll
    for (int n0 = 0; n0 < P::R0; ++n0) {
      const int x = g + G * d + P::LI * n0;
      v[0][d * P::R0 + n0] = make_float2(__ldg(sa + x), __ldg(sbp + x));
    }
  float2* sb = smem + r * TS;
  const RowSync<G> sync{1 + r};
  fft_run<P, -1, 1, TS, 1>(v, sb, 0, g, tw, sync);
  sync();
#pragma unroll
  for (int d = 0; d < P::DF; ++d)
#pragma unroll
    for (int e = 0; e < P::RF; ++e) {
      const int k = g + G * d + P::LF * e;
      if (k < geo.kx || k > N - geo.kx) sb[k] = v[0][d * P::RF + e];
    }
  sync();
  store_split_pair(sb, N, geo.kx, g, G, dst + (2 * q) * drow, dst + (2 * q + 1) * drow);
}

}  // namespace mhdgb
