// Pass kernels of the pruned pseudospectral MHD right-hand side (sm_103a).
//
// Data layouts in HBM (complex = float2, kx fastest everywhere, rows padded to kxp):
//   state   S[f][kz'][ky'][kx]          retained band only (kx < Kx, ky', kz' kept indices)
//   colbuf  A[z][ky'][slot][kx]         after the z pass (inverse) / before it (forward)
//   rowbuf  B[z][y][slot][kx]           after the y pass (inverse) / before it (forward)
// 8 slots per (z, ky') and (z, y): fields 0..5 on the way in, products 0..7 on the way out.
// A kept index j maps to frequency index j (j < Kp) or j + n - K2 (negative wavenumbers).
#pragma once
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

__host__ __device__ __forceinline__ int kept_of_freq(const Geom& g, int f) {
  return f < g.kp ? f : (f >= g.n - g.kn ? f - g.n + g.k2 : -1);
}
__host__ __device__ __forceinline__ int freq_of_kept(const Geom& g, int j) { return j < g.kp ? j : j + g.n - g.k2; }
__host__ __device__ __forceinline__ int signed_of_kept(const Geom& g, int j) { return j < g.kp ? j : j - g.k2; }
// kept index of a signed wavenumber, -1 if it lies in the alias band
__host__ __device__ __forceinline__ int kept_of_signed(const Geom& g, int s) {
  return s >= 0 ? (s < g.kp ? s : -1) : (s >= -g.kn ? s + g.k2 : -1);
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

struct SlotParams {
  float nu, eta, dt;
  float tdiff;  // diffusive time-step limit of the on-device CFL (0: none)
};

struct ColArgs {
  const float2* src;
  float2* dst;
  long long sF, sO, sR;  // source strides (complex elements): field/slot, outer, row
  long long dF, dO, dR;  // destination strides
  long long sI, dI;      // source / destination slot strides (instances of a size class)
};

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
template <int TX, int NT, int N, bool PIN>
__device__ __forceinline__ void col_prefetch(float2* buf, const float2* src, long long sR, int rows, int col0,
                                             const Geom& geo) {
  constexpr int CH = TX / 2;       // 16-byte chunks per row
  constexpr int RSTEP = NT / CH;   // rows advanced per sweep
  const int q = threadIdx.x % CH;
  int row = threadIdx.x / CH;
  if (PIN) {
    float4* zb = reinterpret_cast<float4*>(buf + geo.kp * TX);
    const int nz = (N - geo.k2) * CH;
    for (int c = threadIdx.x; c < nz; c += NT) zb[c] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (col0 + 2 * q >= geo.kxp) return;
  const float2* s = src + row * sR + col0 + 2 * q;
  for (; row < rows; row += RSTEP, s += RSTEP * sR) {
    const int drow = PIN ? (row < geo.kp ? row : row + N - geo.k2) : row;
    cp_async16(buf + drow * TX + 2 * q, s);
  }
}

template <class P0, int TX, int DIR, bool PIN, bool POUT, int MINB>
__global__ void __launch_bounds__(TX * P0::G, MINB)
    col_pass_kernel(ColArgs a, Geom geo, ColWork w, BatchRef br, const float2* __restrict__ tw) {
  using P = Unpadded<P0>;
  extern __shared__ float2 smem[];
  constexpr int G = P::G, V = P::V, N = P::N, NT = TX * P0::G;
  const int tx = threadIdx.x % TX, g = threadIdx.x / TX;
  const int per = w.tiles_x * w.outer * w.nf;  // tiles of one instance
  const int total = *br.count * per;
  // Kept-output bookkeeping (loop invariant): output element e of slot d has frequency
  // k = g + G*d + LF*e; it is kept for e < e_lo[d] (k < Kp) or e >= e_hi[d] (k >= n - Kn),
  // and its kept index is k (first range) or k - (n - K2) (second range).
  int e_lo[P::DF], e_hi[P::DF];
#pragma unroll
  for (int d = 0; d < P::DF; ++d) {
    const int l = g + G * d;
    e_lo[d] = POUT ? (geo.kp - l + P::LF - 1) / P::LF : P::RF;
    e_hi[d] = POUT ? (N - geo.kn - l + P::LF - 1) / P::LF : P::RF;
  }
  const int dR = (int)a.dR;  // row offsets inside one buffer fit 32 bits for n <= 512
  const int shift = (N - geo.k2) * dR;
  // Tile index t = tx_t + tiles_x*(o + outer*(f + nf*inst)).  The grid-stride walk advances it
  // by gridDim.x with a carrying mixed-radix add, so divisions happen once per CTA.
  struct Cur { int tx, o, f, inst; };
  auto decompose = [&](int t) {
    Cur c;
    c.tx = t % w.tiles_x;
    int r = t / w.tiles_x;
    c.o = r % w.outer;
    r /= w.outer;
    c.f = r % w.nf;
    c.inst = r / w.nf;
    return c;
  };
  const Cur gstep = decompose(gridDim.x);
  auto advance = [&](Cur c) {
    int carry;
    c.tx += gstep.tx; carry = c.tx >= w.tiles_x; if (carry) c.tx -= w.tiles_x;
    c.o += gstep.o + carry; carry = c.o >= w.outer; if (carry) c.o -= w.outer;
    c.f += gstep.f + carry; carry = c.f >= w.nf; if (carry) c.f -= w.nf;
    c.inst += gstep.inst + carry;
    return c;
  };
  auto tile_src = [&](const Cur& c) {
    return a.src + br.list[c.inst] * a.sI + c.f * a.sF + (long long)c.o * a.sO;
  };
  int t = blockIdx.x;
  Cur cur_t = decompose(t);
  if (t < total) col_prefetch<TX, NT, N, PIN>(smem, tile_src(cur_t), a.sR, w.rows_in, cur_t.tx * TX, geo);
  cp_async_commit();
  for (int it = 0; t < total; t += gridDim.x, ++it) {
    float2* cur = smem + (it & 1) * (N * TX);
    const int tn = t + gridDim.x;
    const Cur nxt = advance(cur_t);
    if (tn < total)
      col_prefetch<TX, NT, N, PIN>(smem + ((it + 1) & 1) * (N * TX), tile_src(nxt), a.sR, w.rows_in, nxt.tx * TX, geo);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const int inst = cur_t.inst, f = cur_t.f, o = cur_t.o;
    const int kxg = cur_t.tx * TX + tx;
    cur_t = nxt;
    float2 v[1][V];
#pragma unroll
    for (int d = 0; d < P::DI; ++d)
#pragma unroll
      for (int n0 = 0; n0 < P::R0; ++n0) v[0][d * P::R0 + n0] = cur[(g + G * d + P::LI * n0) * TX + tx];
    __syncthreads();  // cur is now free: reuse it as the exchange buffer
    fft_run<P, DIR, 1, 0, TX>(v, cur, tx, g, tw, BlockSync{});
    if (kxg < geo.kx) {
      float2* dst = a.dst + br.list[inst] * a.dI + f * a.dF + (long long)o * a.dO + kxg;
#pragma unroll
      for (int d = 0; d < P::DF; ++d) {
        const int base = (g + G * d) * dR;
#pragma unroll
        for (int e = 0; e < P::RF; ++e) {
          const int off = base + e * (P::LF * dR);
          if (!POUT) {
            dst[off] = v[0][d * P::RF + e];
          } else if (e < e_lo[d]) {
            dst[off] = v[0][d * P::RF + e];
          } else if (e >= e_hi[d]) {
            dst[off - shift] = v[0][d * P::RF + e];
          }
        }
      }
    }
    __syncthreads();  // all exchange reads of cur done before it is refilled
  }
  cp_async_wait<0>();
}

// ------------------------------------------------------------------------------------------
// x rows: Hermitian two-for-one helpers.
// ------------------------------------------------------------------------------------------
// Kept rfft-axis modes of the 2/3 rule for n points, as a compile-time constant (the same double
// arithmetic as FourierFlows' getaliasedwavenumbers with aliased fraction 1/3: floor(n/3 + tiny)).
__host__ __device__ constexpr int kept_kx_of(int n) { return (int)((1.0 - 1.0 / 3.0) / 2.0 * n); }

// Input of an inverse (c2r) transform of two half-spectrum rows f1, f2 with KX kept modes
// (plain loads: the rows may live in global or in shared memory):
// z[n] = F1[n] + i F2[n] with F[n-n] = conj(F[n]); the kx = 0 imaginary parts are dropped,
// which is what a c2r transform does with a non-Hermitian kx = 0 plane.  Elements whose index
// lies in the alias band for every lane are compile-time zeros, so the first stage of the
// transform is pruned by constant folding.
template <class P, int KX>
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
          float2 a = f1[n], b = f2[n];
          if (n == 0) { a.y = 0.f; b.y = 0.f; }
          z = make_float2(a.x - b.y, a.y + b.x);
        } else if (n > P::N - KX) {
          const int m = P::N - n;
          float2 a = f1[m], b = f2[m];
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
template <class P>
struct XCfg {
  static constexpr int G = P::G;
  static constexpr int RPG = G >= 32 ? 1 : 32 / G;        // rows per group
  static constexpr int TPG = G >= 32 ? G : 32;            // threads per group
  static constexpr int TS = RowCfg<P>::TS;                // exchange words per row
  static __host__ __device__ int stage_words(int kxp) { return RPG * 6 * kxp; }
  static __host__ __device__ int group_words(int kxp) { return 2 * stage_words(kxp) + RPG * TS; }
};

template <class P, int GROUPS>
__global__ void __launch_bounds__(GROUPS * XCfg<P>::TPG, (P::V > 8 ? 2 : 4))
    x_fused_kernel(float2* pool, Geom geo, long long rowstride, long long slot, long long istride, BatchRef br,
                   const float2* __restrict__ tw, const float2* __restrict__ twr, unsigned int* vmax) {
  using PR = typename Reverse<P>::type;
  using XC = XCfg<P>;
  constexpr int G = P::G, V = P::V, N = P::N, RPG = XC::RPG, TPG = XC::TPG, TS = XC::TS;
  constexpr int KX = kept_kx_of(N);  // the host checks geo.kx == KX
  extern __shared__ float2 smem[];
  const int kxp = geo.kxp;
  const int grp = threadIdx.x / TPG;
  const int gt = threadIdx.x % TPG;          // thread within group
  const int rr = gt / G, g = gt % G;         // row within group, lane within row
  const int sw = XC::stage_words(kxp);
  float2* gs = smem + grp * XC::group_words(kxp);
  float2* sb = gs + 2 * sw + rr * TS;
  const RowSync<G> sync{1 + grp};
  constexpr int GPI = N * N / RPG;  // row groups per instance
  const long long ngroups = (long long)(*br.count) * GPI;
  const int chunks_row = 3 * kxp;  // 16-byte chunks of the six contiguous field rows (slot == kxp)
  // first row of row group q, inside its instance's rowbuf
  auto group_rows = [&](long long q) {
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
  if (q < ngroups) prefetch(q, gs);
  cp_async_commit();
  for (int it = 0; q < ngroups; q += qstep, ++it) {
    const float2* cur = gs + (it & 1) * sw;
    if (q + qstep < ngroups) prefetch(q + qstep, gs + ((it + 1) & 1) * sw);
    cp_async_commit();
    cp_async_wait<1>();
    sync();
    const float2* rin = cur + rr * 6 * kxp;
    float2 v[3][V];
#pragma unroll
    for (int t = 0; t < 3; ++t) load_herm_pair<P, KX>(v[t], rin + (2 * t) * kxp, rin + (2 * t + 1) * kxp, g);
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      fft_run<P, +1, 1, TS, 1>(reinterpret_cast<float2(&)[1][V]>(v[t]), sb, 0, g, tw, sync);
      sync();
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
        const int inst = (int)(q / GPI);
        atomicMax(vmax + 2 * br.list[inst], bu);
        atomicMax(vmax + 2 * br.list[inst] + 1, bb);
      }
    }
    float2* rowp = group_rows(q) + rr * rowstride;
    // one product pair at a time: the six fields stay live, the pair is formed just before its
    // forward transform (fewer live registers than all eight products at once)
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      float2 w[1][V];
#pragma unroll
      for (int i = 0; i < V; ++i) {
        const float ux = v[0][i].x, uy = v[0][i].y, uz = v[1][i].x;
        const float bx = v[1][i].y, by = v[2][i].x, bz = v[2][i].y;
        if (t == 0) {
          const float tzz = bz * bz - uz * uz;
          w[0][i] = make_float2((bx * bx - ux * ux) - tzz, (by * by - uy * uy) - tzz);
        } else if (t == 1) {
          w[0][i] = make_float2(bx * by - ux * uy, bx * bz - ux * uz);
        } else if (t == 2) {
          w[0][i] = make_float2(by * bz - uy * uz, ux * by - bx * uy);
        } else {
          w[0][i] = make_float2(ux * bz - bx * uz, uy * bz - by * uz);
        }
      }
      fft_run<PR, -1, 1, TS, 1>(w, sb, 0, g, twr, sync);
      float2* oa = rowp + (2 * t) * slot;
      float2* ob = rowp + (2 * t + 1) * slot;
      if constexpr (G <= 32) {
        store_split_shfl<PR, KX>(w[0], g, (threadIdx.x & 31) - g, oa, ob);
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
        store_split_pair(sb, N, KX, g, G, oa, ob);
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
  fft_run<P, +1, 1, TS, 1>(v, smem + r * TS, 0, g, tw, RowSync<G>{1 + r});
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
  const float2* prod;   // 8 compact planes (slot stride prodI)
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
};

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
template <int OP>
__global__ void __launch_bounds__(256) rk_epilogue_kernel(RkArgs a, Geom geo, BatchRef br) {
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
  for (int q = 0; q < 8; ++q) p[q] = cscale(__ldcs(prod + q * fs + i), a.pscale);
  float2 xv[6], xd[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) xv[c] = xd[c] = X[c * fs + i];
  if (x == 0) {
    const long long p = (long long)jz * geo.k2 + jy, pl = (long long)geo.k2 * geo.k2;
    const float2* H = a.H + slot * a.hI;
#pragma unroll
    for (int c = 0; c < 6; ++c) xd[c] = H[c * pl + p];
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
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const float dk = c < 3 ? du : db;
    rk_apply<OP>(rs, c * fs + i, xv[c], make_float2(nl[c].x + dk * xd[c].x, nl[c].y + dk * xd[c].y));
  }
}

// Hermitian part of the kx = 0 plane of the six fields: H(k) = (X(k) + conj X(-k)) / 2, with
// X(-k) = 0 when -k is in the alias band.  The reference's diffusion term is computed from the
// re-transformed physical field, rfft(irfft(X)), which is exactly this on the kx = 0 plane.
__global__ void herm_kx0_kernel(const float2* __restrict__ Xpool, float2* __restrict__ Hpool, Geom geo, long long fs,
                                long long stI, long long hI, BatchRef br) {
  const int per = 6 * geo.k2 * geo.k2;
  const int total = *br.count * per;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int inst = t / per, i = t - inst * per;
    const int slot = br.list[inst];
    const float2* X = Xpool + slot * stI;
    float2* H = Hpool + slot * hI;
    const int jy = i % geo.k2;
    const int r = i / geo.k2;
    const int jz = r % geo.k2, c = r / geo.k2;
    const long long base = (long long)c * fs;
    const float2 xk = X[base + ((long long)jz * geo.k2 + jy) * geo.kxp];
    const int py = kept_of_signed(geo, -signed_of_kept(geo, jy));
    const int pz = kept_of_signed(geo, -signed_of_kept(geo, jz));
    float2 xp = make_float2(0.f, 0.f);
    if (py >= 0 && pz >= 0) xp = X[base + ((long long)pz * geo.k2 + py) * geo.kxp];
    H[i] = make_float2(0.5f * (xk.x + xp.x), 0.5f * (xk.y - xp.y));
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

__global__ void scatter_state_kernel(const float2* __restrict__ S, float2* __restrict__ ref, Geom geo, int nf) {
  const int nkr = geo.n / 2 + 1;
  const long long total = (long long)nf * geo.n * geo.n * nkr;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nkr);
    long long r = i / nkr;
    const int fy = (int)(r % geo.n); r /= geo.n;
    const int fz = (int)(r % geo.n);
    const int f = (int)(r / geo.n);
    float2 val = make_float2(0.f, 0.f);
    const int jy = kept_of_freq(geo, fy), jz = kept_of_freq(geo, fz);
    if (x < geo.kx && jy >= 0 && jz >= 0) val = S[(((long long)f * geo.k2 + jz) * geo.k2 + jy) * geo.kxp + x];
    ref[i] = val;
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
