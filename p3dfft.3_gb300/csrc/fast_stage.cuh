// Specialised stage kernels for the hot transform kinds (C2C, even-length R2C and C2R) at FFT
// lengths N = 2^a 3^b 5^c from 16 to 512 and 1024, 2048: one instantiation per (arithmetic,
// kind, length), with the radix plan and every index computed at compile time.
//
// Same contract as k_stage (one reference transplan stage: gather a tile of lines along the
// transform dimension from the input memory order, transform, scatter into the output memory
// order), organised for instruction economy:
//   - one tile of TB lines per CTA, lines numbered across both batch dims (a tile may span two
//     rows of the tile dim, so no lanes idle when that dim is short); twiddles through the
//     read-only cache
//   - every thread owns V = N/T points of one line (the same points for load, FFT and store)
//   - loads go to registers first; float-float tiles are scaled by a power of two chosen from
//     the tile's largest exponent (block-wide max) before conversion, which keeps any finite
//     input in range
//   - Stockham passes of radix 8/4/2 then 5/3 in registers, one padded shared-memory scatter
//     per pass; in a pass of radix R each thread does ceil(N/R / T) butterflies
//   - R2C / C2R half-length packing and the fused i*k derivative are done on the way in / out
//   - DCT-I / DST-I (FFTW REDFT00 / RODFT00) are the FFT of the line's even / odd extension,
//     built on the way in; real lines are transformed two at a time as the real and imaginary
//     parts of one complex line (both transforms are real-linear)
//   - DCT / DST II-IV (FFTW REDFT10/01/11, RODFT10/01/11) are one FFT of length 2n of the
//     pre-twiddled, zero-padded real line and a post-twiddle on the way out; a complex line is
//     two real lines (its real and imaginary parts)
#pragma once
#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>

#include <type_traits>

#include "kernels.h"
#include "stage_common.cuh"

namespace p3d {

enum FastKind { FK_C2C = 0, FK_R2C = 1, FK_C2R = 2, FK_R2R1 = 3, FK_R2RG = 4 };

struct FParams {
  const void *in;
  void *out;
  const void *tw;   // W_{tabN}^m, tabN = N (C2C) or 2N (R2C / C2R), m < tabN
  const void *ptw;  // per-pass twiddle rows (fast_pass_offset)
  long long iL, it, io, oL, ot, oo;  // element strides
  int dt;                            // size of the tile dim; line g is (g % dt, g / dt)
  int nlines, ntotal;                // lines in total, CTAs
  int sign;                          // C2C: -1 forward, +1 backward
  int deriv, dg, dmid;               // fused derivative (compute_deriv_loc wavenumbers)
  int load_Lmajor, store_Lmajor;
  // FK_R2R1: r2r_odd 0 DCT-I (N = 2(n-1)), 1 DST-I (N = 2(n+1)); pair 1 for real lines, taken
  // two at a time (lines 2g and 2g+1 of nreal form FFT line g), 0 for complex lines
  int r2r_odd, pair, nreal;
  // FK_R2RG: y_k = 2 Re or -2 Im of W_{8n}^{a2 (2k + b2)} U_k, U = FFT_{2n}(x_j W_{8n}^{2 b2 j},
  // j < n, x_0 / x_{n-1} halved when half0 / half1), aux = the W_{8n} table; cplx: FFT line g is
  // part g & 1 of complex line g >> 1
  const void *aux;
  int rg_n, rg_a2, rg_b2, rg_sin, rg_half0, rg_half1, rg_cplx;
  // Float-float intermediate fields (DFP kernels, FK_C2C / FK_R2C out / FK_C2R in).  ffin: the
  // input holds packed float-float values, each scaled by 2^sin[i] of the line that stored it,
  // i = j * fi_j + (g % dt) * fi_t + (g / dt) * fi_o for point j of line g.  ffout: store packed
  // float-float values at this tile's scale and each line's scale at sout[(g % dt) * fo_t +
  // (g / dt) * fo_o].
  int ffin, ffout;
  const int *sin;
  int *sout;
  long long fi_j, fi_t, fi_o, fo_t, fo_o;
  // TMA-staged loads (k_fast_tma): the wait for the tile's bytes gives up after tma_timeout_ns
  // and sets *status to 1; tma_extra adds bytes the copies never deliver (a wait that runs out,
  // for the failure-path test)
  long long tma_timeout_ns;
  int tma_extra;
  int tma_d1;    // lines along the tensor map's line dim (line g at (g % tma_d1, g / tma_d1))
  int tma_store;  // 1: the tile's outputs leave by TMA (C2C, tile dim contiguous in the output)
  int tma_mode;  // 1: lines contiguous (boxes of one line's floats x TB lines); 2: tile dim
                 // contiguous (C2C: boxes of TB points' floats x rows of the line dim)
  int *status;
  // k_fast_persist: a zeroed counter from which the CTAs take their tiles after the first (the
  // CTA that finishes first takes the next), or nullptr for a fixed grid stride
  int *tile_ctr;
};

// The FP32 split-twiddle policy the build instantiates: twiddle powers read from the tables
// (FAST_FS_CHAIN 0, the default) or chained in float-float from W^1 (1: same accuracy, but the
// 512^3 FP32 round trip measured 1.680 against 1.362 ms - the float-float products and the lower
// occupancy they need, 6 CTAs of 40 registers, cost more than the table loads they save)
#ifndef FAST_FS_CHAIN
#define FAST_FS_CHAIN 0
#endif
using FSplit = NativeFS<FAST_FS_CHAIN != 0>;

// Float-float C2R: form the half-length packing pairwise (k, N-k) before the first pass (1:
// half the twiddle products; measured 0.851 -> 0.848 ms at 512^3), or per point as the first pass
// reads (0; kept for FP32, where the extra shared-memory round trip cost 7%)
#ifndef FAST_C2R_PAIRS
#define FAST_C2R_PAIRS 1
#endif

// resident 256-thread CTAs per SM the register allocation is sized for (FP64 and float-float;
// FP32 kernels, with half-width values, can afford more resident CTAs)
#ifndef FAST_MIN_BLOCKS
#define FAST_MIN_BLOCKS 4
#endif
#ifndef FAST_MIN_BLOCKS_FP32
#define FAST_MIN_BLOCKS_FP32 8
#endif
// float-float / FP64 R2C and C2R kernels (the real-data pack / unpack costs registers: at 4 CTAs of
// 64 registers they spill 16-28 bytes per thread; 3 CTAs of 80 registers remove the spills but
// measured slower at 512^3: R2C 0.755 vs 0.720 ms, C2R 0.915 vs 0.847 ms)
#ifndef FAST_MIN_BLOCKS_RC
#define FAST_MIN_BLOCKS_RC FAST_MIN_BLOCKS
#endif

// The FFT lengths with a specialised kernel.
#define P3D_FAST_LENGTHS(X)                                                                              \
  X(16) X(18) X(20) X(24) X(25) X(27) X(30) X(32) X(36) X(40) X(45) X(48) X(50) X(54) X(60) X(64) X(72)   \
  X(75) X(80) X(81) X(90) X(96) X(100) X(108) X(120) X(125) X(128) X(135) X(144) X(150) X(160) X(162)    \
  X(180) X(192) X(200) X(216) X(225) X(240) X(243) X(250) X(256) X(270) X(288) X(300) X(320) X(324)      \
  X(360) X(375) X(384) X(400) X(405) X(432) X(450) X(480) X(486) X(500) X(512) X(1024) X(2048)

// The even lengths (FFT lengths of DCT-I / DST-I extensions).
#define P3D_FAST_EVEN_LENGTHS(X)                                                                         \
  X(16) X(18) X(20) X(24) X(30) X(32) X(36) X(40) X(48) X(50) X(54) X(60) X(64) X(72) X(80) X(90) X(96)   \
  X(100) X(108) X(120) X(128) X(144) X(150) X(160) X(162) X(180) X(192) X(200) X(216) X(240) X(250)     \
  X(256) X(270) X(288) X(300) X(320) X(324) X(360) X(384) X(400) X(432) X(450) X(480) X(486) X(500)     \
  X(512) X(1024) X(2048)

// Radix plan: radix-8 passes, the leftover power of two (4 or 2), then 5s, then 3s.
struct RadixList {
  int n;  // passes, -1 if N has a prime factor above 5
  int r[16];
};
__host__ __device__ constexpr RadixList fast_radices(int N) {
  RadixList L{0, {0}};
  int a = 0, m = N;
  while (m > 1 && m % 2 == 0) {
    m /= 2;
    a++;
  }
  for (int i = 0; i < a / 3; i++) L.r[L.n++] = 8;
  if (a % 3 == 2) L.r[L.n++] = 4;
  if (a % 3 == 1) L.r[L.n++] = 2;
  while (m > 1 && m % 5 == 0) {
    m /= 5;
    L.r[L.n++] = 5;
  }
  while (m > 1 && m % 3 == 0) {
    m /= 3;
    L.r[L.n++] = 3;
  }
  if (m != 1) L.n = -1;
  return L;
}
// points per thread: the largest divisor of N up to 8
__host__ __device__ constexpr int fast_points(int N) {
  for (int d = 8; d > 1; d--)
    if (N % d == 0) return d;
  return 1;
}
// most values a thread holds in one pass
__host__ __device__ constexpr int fast_max_values(int N) {
  const RadixList L = fast_radices(N);
  const int T = N / fast_points(N);
  int m = 0;
  for (int i = 0; i < L.n; i++) {
    const int nb = (N / L.r[i] + T - 1) / T;
    if (nb * L.r[i] > m) m = nb * L.r[i];
  }
  return m;
}

template <int N>
struct FastShape {
  static constexpr int V = fast_points(N);          // points per thread
  static constexpr int T = N / V;                   // threads per line
  static constexpr int TB = T >= 256 ? 1 : 256 / T;  // lines per tile
  static constexpr int USED = TB * T;               // threads with a line
  static constexpr int BLOCK = (USED + 31) / 32 * 32;
  static constexpr int MINB = fast_max_values(N) > 8 ? 3 : FAST_MIN_BLOCKS;
};

// Layout of a line in shared memory.  Padding: one slot after every 2^PS data slots, PS = 3 for
// 16-byte complex elements and 4 for 8-byte ones, i.e. one slot per 128 bytes of line data.
// Swizzle (PS = FK_SWZ, 8-byte elements with FAST_SWIZZLE8): slot i ^ ((i >> 3) & 15), a
// permutation within each aligned block of 16 slots that a wavefront model of the Stockham
// passes finds conflict-free where the padding leaves 1/6 extra wavefronts.  Measured: correct,
// but the FP32 512^3 round trip 15% slower (1.43 vs 1.24 ms), the slots of a thread's points
// being computed one by one instead of by constant steps; so the padding is the default.
#ifndef FAST_SWIZZLE8
#define FAST_SWIZZLE8 0
#endif
constexpr int FK_SWZ = 15;
template <int ESZ>
__host__ __device__ constexpr int fast_pad_shift() {
  return ESZ >= 16 ? 3 : (FAST_SWIZZLE8 ? FK_SWZ : 4);
}
template <int PS>
__host__ __device__ __forceinline__ constexpr int fk_pos(int i) {
  if constexpr (PS == FK_SWZ) return i ^ ((i >> 3) & 15);
  else return PS ? i + (i >> PS) : i;
}
// additive padding (slots of evenly spaced points advance by constant steps)
template <int PS>
__host__ __device__ constexpr bool fk_additive() {
  return PS != FK_SWZ;
}

// Bank-conflict cost of a shared-memory line stride LS (complex slots of ESZ bytes): a warp's
// accesses are served 128 bytes at a time, i.e. by groups of U = 128/ESZ threads whose slots should
// fall in distinct ESZ-byte bank groups (slot mod U).  Summed over the block, for both thread
// mappings of the kernel (consecutive threads along a line, and across the TB lines).
template <int N>
__host__ __device__ constexpr int fast_ls_cost(int LS, int ESZ) {
  using SH = FastShape<N>;
  const int U = 128 / ESZ;
  int cost = 0;
  for (int map = 0; map < 2; map++) {
    for (int g0 = 0; g0 < SH::USED; g0 += U) {
      int cnt[32] = {0};
      int worst = 0;
      for (int t = g0; t < g0 + U && t < SH::USED; t++) {
        const int l = map ? t % SH::TB : t / SH::T;
        const int j = map ? t / SH::TB : t % SH::T;
        const int slot = l * LS + (ESZ >= 16 ? fk_pos<3>(j) : fk_pos<fast_pad_shift<8>()>(j));
        const int c = ++cnt[slot % U];
        worst = c > worst ? c : worst;
      }
      cost += worst;
    }
  }
  return cost;
}

// Line stride: more than the largest slot of points 0..N (N is used by C2R), the cheapest under
// fast_ls_cost among the next 128/ESZ candidates.
template <int N, int ESZ>
__host__ __device__ constexpr int fast_ls() {
  int base = 0;
  for (int i = 0; i <= N; i++) {
    const int sl = fk_pos<fast_pad_shift<ESZ>()>(i);
    base = sl + 1 > base ? sl + 1 : base;
  }
  const int U = 128 / ESZ;
  int best = base, best_cost = 1 << 30;
  for (int ls = base; ls < base + U; ls++) {
    const int c = fast_ls_cost<N>(ls, ESZ);
    if (c < best_cost) {
      best_cost = c;
      best = ls;
    }
  }
  return best;
}

// Per-pass twiddle tables.  Pass I >= 1 of the radix plan (radix R, Ns = product of the earlier
// radices) multiplies by W_{Ns R}^{r k}, r = 1 .. R-1, for its k = jj mod Ns.  They are stored per
// pass as R-1 rows of Ns entries, row r-1 holding W_{Ns R}^{r k} at entry k: the threads of a warp
// (consecutive jj, hence consecutive k) read consecutive entries for each r, so every twiddle load
// of a pass is coalesced.  Pass I starts at fast_pass_offset(N, I) entries.
__host__ __device__ constexpr int fast_pass_offset(int N, int I) {
  const RadixList L = fast_radices(N);
  int off = 0, ns = L.n > 0 ? L.r[0] : 1;
  for (int j = 1; j < I && j < L.n; j++) {
    off += ns * (L.r[j] - 1);
    ns *= L.r[j];
  }
  return off;
}
// total entries of the per-pass tables of length N
__host__ __device__ constexpr int fast_pass_entries(int N) { return fast_pass_offset(N, 32); }

// Twiddles are read through the read-only data cache (the tables are a few KB and stay L1
// resident across the CTAs of an SM); a shared-memory copy per CTA was measured to cost more
// registers and L2 traffic than it saves.
template <class O>
__device__ __forceinline__ typename O::W fk_tw(const typename O::T *tab, int m, int sign) {
  const typename O::W w = O::tw(tab, m);
  return sign < 0 ? w : O::conj(w);
}

// 1: float-float values are normalised each time a pass stores them; 0: only by the output
// conversion.  Unnormalised pass stores measured 3.7% faster on the 512^3 round trip, at
// 2.7e-14 instead of 1.7e-14 relative L2 against native FP64 (the lo parts carry the rounding
// errors of more additions before they are folded back).
#ifndef FAST_PASS_NORM
#define FAST_PASS_NORM 0
#endif

// Barrier between the phases of a tile.  sid = 0: the whole CTA; otherwise only the threads of
// one line, which then exchange data with no other line: a named barrier of the line's T threads
// (sid = 1 + line, T a multiple of 32 above one warp) or the warp (lines of T <= 32 threads that
// divide a warp).
template <int T>
__device__ __forceinline__ void fk_sync(int sid) {
  if (sid == 0) {
    __syncthreads();
  } else if constexpr (T % 32 == 0 && T > 32) {
    asm volatile("bar.sync %0, %1;" ::"r"(sid), "n"(T) : "memory");
  } else {
    __syncwarp();
  }
}

// Stockham pass I (radix R = plan[I], Ns = product of the earlier radices): butterfly jj reads
// x[jj + r N/R], multiplies by W_{Ns R}^{r k} (k = jj mod Ns), applies DFT-R and writes slot
// (jj - k) R + k + r Ns.  Values stay in registers across the barrier; one scatter per pass.
// C2RPRE (first pass of a C2R stage): each value read is the half-length packing
// Z[k] = (X[k] + conj X[N-k]) + i conj(W_2N^k) (X[k] - conj X[N-k]) of the spectrum in the line
// (slots 0..N; imaginary parts of X[0], X[N] ignored), formed as it is read.
template <class O, int N, int TWSTEP, int Ns, int I, bool C2RPRE = false>
__device__ __forceinline__ void fk_pass(typename O::C *line, const typename O::T *tab, const typename O::T *ptab,
                                        int j, bool active, int sign, int sid) {
  using C = typename O::C;
  constexpr int PS = fast_pad_shift<(int)sizeof(C)>();
  constexpr RadixList RL = fast_radices(N);
  constexpr int R = RL.r[I];
  constexpr int T = FastShape<N>::T, M = N / R;
  constexpr int NB = (M + T - 1) / T;  // butterflies per thread
  constexpr bool GUARD = (M % T) != 0;
  C v[NB * R];
  typename O::W w1, w2;  // W_R^1, W_R^2 for the odd radices
  if constexpr (R == 3 || R == 5) w1 = O::tw(tab, (N / R) * TWSTEP);
  if constexpr (R == 5) w2 = O::tw(tab, 2 * (N / R) * TWSTEP);
  if (active) {
#pragma unroll
    for (int b = 0; b < NB; b++) {
      const int jj = j + b * T;
      if (GUARD && jj >= M) break;
      // padded slots: pad(jj + r M) = pad(jj) + r (M + M/2^PS) when M is a multiple of 2^PS
      const int pj = fk_pos<PS>(jj);
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int slot = (fk_additive<PS>() && M % (1 << PS) == 0) ? pj + r * (M + (M >> PS)) : fk_pos<PS>(jj + r * M);
        if constexpr (C2RPRE) {
          const int k = jj + r * M;
          C xa = line[slot], xb = line[fk_pos<PS>(N - k)];
          if (k == 0) {
            xa = O::mk(O::re(xa), O::rzero());
            xb = O::mk(O::re(xb), O::rzero());
          }
          const C xbc = O::conj(xb);
          const C s = O::add(xa, xbc), d = O::sub(xa, xbc);
          v[b * R + r] = O::norm(O::add(s, O::muli(O::mul(d, O::conj(O::tw(tab, k))))));
        } else {
          v[b * R + r] = line[slot];
        }
      }
      if constexpr (Ns > 1) {
        const typename O::T *pt = ptab + fast_pass_offset(N, I) + jj % Ns;
        if constexpr (O::TW_POWERS) {
          // two table twiddles per butterfly, the others as products of at most two of them
          typename O::W w[8];
          w[1] = fk_tw<O>(pt, 0, sign);
          if constexpr (R >= 3) w[2] = O::wmul(w[1], w[1]);
          if constexpr (R >= 4) w[3] = O::wmul(w[2], w[1]);
          if constexpr (R == 5) w[4] = O::wmul(w[2], w[2]);
          if constexpr (R == 8) {
            w[4] = fk_tw<O>(pt, 3 * Ns, sign);
            w[5] = O::wmul(w[4], w[1]);
            w[6] = O::wmul(w[4], w[2]);
            w[7] = O::wmul(w[4], w[3]);
          }
#pragma unroll
          for (int r = 1; r < R; r++) v[b * R + r] = O::mul(v[b * R + r], w[r]);
        } else if constexpr (O::TW_CHAIN) {
          // W^1 from the table, W^r = W^(r-1) W^1 formed one at a time
          const typename O::W w1 = fk_tw<O>(pt, 0, sign);
          typename O::W w = w1;
          v[b * R + 1] = O::mul(v[b * R + 1], w1);
#pragma unroll
          for (int r = 2; r < R; r++) {
            w = O::wmul(w, w1);
            v[b * R + r] = O::mul(v[b * R + r], w);
          }
        } else {
#pragma unroll
          for (int r = 1; r < R; r++) v[b * R + r] = O::mul(v[b * R + r], fk_tw<O>(pt, (r - 1) * Ns, sign));
        }
      }
      if constexpr (R == 3) dft3<O>(&v[b * R], sign, w1);
      else if constexpr (R == 5) dft5<O>(&v[b * R], sign, w1, w2);
      else dft_p2<O, R>(&v[b * R], sign);
    }
  }
  fk_sync<T>(sid);
  if (active) {
#pragma unroll
    for (int b = 0; b < NB; b++) {
      const int jj = j + b * T;
      if (GUARD && jj >= M) break;
      const int k = jj % Ns;
      const int base = (jj - k) * R + k;
      // pad(base + r Ns) = pad(base) + r (Ns + Ns/2^PS) for Ns a multiple of 2^PS, and
      // pad(base) + r in the first pass when R is a power of two up to 2^PS (base = jj R then
      // stays in one padding block)
      constexpr bool NS_AL = fk_additive<PS>() && Ns % (1 << PS) == 0;
      constexpr bool FIRST_AL = fk_additive<PS>() && Ns == 1 && (R & (R - 1)) == 0 && R <= (1 << PS);
      const int pb = fk_pos<PS>(base);
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int slot = NS_AL ? pb + r * (Ns + (Ns >> PS)) : (FIRST_AL ? pb + r : fk_pos<PS>(base + r * Ns));
        line[slot] = FAST_PASS_NORM ? O::norm(v[b * R + r]) : v[b * R + r];
      }
    }
  }
  fk_sync<T>(sid);
  if constexpr (I + 1 < RL.n) fk_pass<O, N, TWSTEP, Ns * R, I + 1>(line, tab, ptab, j, active, sign, sid);
}

// f(e) for e = 0 .. V-1, U iterations unrolled per step of the outer loop
template <int V, int U, class F>
__device__ __forceinline__ void fk_for(F &&f) {
  constexpr int UU = U < 1 ? 1 : (U > V ? V : U);
#pragma unroll 1
  for (int e0 = 0; e0 < V; e0 += UU) {
#pragma unroll
    for (int u = 0; u < UU; u++)
      if (V % UU == 0 || e0 + u < V) f(e0 + u);
  }
}

// Slot of point j0 + e*TT given pj0 = slot(j0): constant steps when TT is a multiple of 2^PS.
template <int PS, int TT>
__device__ __forceinline__ int fk_slot(int j0, int pj0, int e) {
  if constexpr (fk_additive<PS>() && TT % (1 << PS) == 0) return pj0 + e * (TT + (TT >> PS));
  else return fk_pos<PS>(j0 + e * TT);
}
// Slot of point N - (j0 + e*TT) given pn = slot(N - j0), for 0 < j0 + e*TT <= N.
template <int PS, int TT, int N>
__device__ __forceinline__ int fk_slot_rev(int j0, int pn, int e) {
  if constexpr (fk_additive<PS>() && TT % (1 << PS) == 0 && N % (1 << PS) == 0) return pn - e * (TT + (TT >> PS));
  else return fk_pos<PS>(N - j0 - e * TT);
}

template <class O>
__device__ __forceinline__ typename O::C fk_deriv(const FParams &p, typename O::C v, int k) {
  if (!p.deriv) return v;
  if (k == p.dmid) return O::zero();
  return O::iscale(v, (k < p.dmid) ? k : k - p.dg);
}

template <class O, int N, int KIND = FK_C2C>
__host__ __device__ constexpr int fast_min_blocks() {
  // (the chained split twiddles hold two float-float twiddles: 6 CTAs of 40 registers)
  return sizeof(typename O::C) <= 8
             ? ((fast_max_values(N) > 8 || O::TW_CHAIN) ? FAST_MIN_BLOCKS_FP32 * 3 / 4 : FAST_MIN_BLOCKS_FP32)
             : ((KIND == FK_R2C || KIND == FK_C2R) && FAST_MIN_BLOCKS_RC < FastShape<N>::MINB ? FAST_MIN_BLOCKS_RC
                                                                                       : FastShape<N>::MINB);
}

// A launch over the tiles of several stages of independent transforms that share the kernel
// (arithmetic, kind, length) and may differ in everything else (buffers, grids, strides, tables):
// plist holds each stage's parameters, work the (stage, tile) items; one CTA per item
// (k_fast_list).
struct FGroup {
  const struct FParams *plist;
  const struct FWork *work;
  int nwork;
};
struct FWork {
  int stage, tile;
};

// TMA staging of a tile's input (FP32 C2C / R2C with line-contiguous, evenly spaced lines and a
// first radix equal to the points per thread): a 3D tensor map (floats along the line, lines
// along the tile dim, lines along the other batch dim) and NBOX boxes of BOXW floats x TB lines,
// landed densely in the tile's shared-memory region box after box; one mbarrier counts the bytes.
// Threads then read their first butterfly's inputs from shared memory instead of global memory.
template <int N>
struct FastTma {
  static constexpr int FL = 2 * N;  // floats per line (complex points, or packed real pairs)
  static constexpr int BOXW = FL <= 256 ? FL : 256;
  static constexpr int NBOX = FL / BOXW;
  static constexpr bool OK = FL <= 256 || FL % 256 == 0;
  // tile-dim-contiguous tiles: boxes of BOXR rows (the largest divisor of N up to 256)
  static constexpr int BOXR = [] {
    int r = N < 256 ? N : 256;
    while (N % r) r--;
    return r;
  }();
  static constexpr int NBR = N / BOXR;
};
__host__ __device__ constexpr bool fast_tma_length(int n) {
  // even n: a box row of 2n floats is a multiple of 16 bytes
  return n >= 32 && n % 2 == 0 && (2 * n <= 256 || (2 * n) % 256 == 0) && fast_radices(n).n > 0 &&
         fast_radices(n).r[0] == fast_points(n);
}
template <class O, int KIND, int N>
__host__ __device__ constexpr bool fk_tma_variant() {
  return (std::is_same_v<O, Native<float>> || std::is_same_v<O, FSplit>) &&
         (KIND == FK_C2C || KIND == FK_R2C) && fast_tma_length(N);
}
// mbarrier phase wait bounded by the global timer: false after limit_ns
__device__ __forceinline__ bool fk_mbar_wait(unsigned bar, unsigned parity, long long limit_ns) {
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if ((long long)(t - t0) > limit_ns) return false;
  }
}

// One tile of one stage (the body of k_fast and k_fast_list).
// FF: float-float intermediate I/O of the DFP kernels, bit 0 input, bit 1 output (FParams ffin /
// ffout); separate instantiations (fk_ff_variants), so that the IEEE-only kernels carry none of it
// TMA: the tile's input arrives by the tensor map *tm (fk_tma_variant kernels only).
template <class O, int KIND, int N, int FF = 0, bool TMA = false>
__device__ __forceinline__ void fk_tile(const FParams &p, const int tile, const void *in, void *out,
                                        const CUtensorMap *tm = nullptr, const CUtensorMap *tmo = nullptr) {
  using C = typename O::C;
  using T = typename O::T;
  using G = typename O::G;
  using RAW = typename O::RAW;
  using SH = FastShape<N>;
  constexpr int TWSTEP = (KIND == FK_C2C || KIND == FK_R2R1 || KIND == FK_R2RG) ? 1 : 2;  // W_N^m = tab[m * TWSTEP]
  constexpr int LS = fast_ls<N, (int)sizeof(C)>(), TB = SH::TB, TT = SH::T, V = SH::V;
  constexpr int PS = fast_pad_shift<(int)sizeof(C)>();
  extern __shared__ __align__(128) unsigned char smem_raw[];
  C *buf = reinterpret_cast<C *>(smem_raw);
  __shared__ int red[32], red2[32];
  // float-float tiles whose lines differ widely in magnitude: each line's largest biased
  // exponent (finite values), so that every line gets its own power-of-two scale
  __shared__ int lfin[TB];
  const T *tab = reinterpret_cast<const T *>(p.tw);
  const T *ptab = reinterpret_cast<const T *>(p.ptw);
  // threads past TB*T (BLOCK rounded up to whole warps) hold no line
  const bool valid = SH::BLOCK == SH::USED || (int)threadIdx.x < SH::USED;
  unsigned tbar_addr = 0;
  // TMA writes to 128-byte aligned shared memory only; a tile region placed otherwise is loaded by
  // the threads (the same values, by the per-thread path)
  const bool tma_on = TMA && ((unsigned)__cvta_generic_to_shared(smem_raw) & 127u) == 0;
  if constexpr (TMA) {
    // one thread starts the tile's copies first thing; the others meet it at the barrier below
    __shared__ __align__(8) unsigned long long tbar;
    using TM = FastTma<N>;
    tbar_addr = (unsigned)__cvta_generic_to_shared(&tbar);
    if (threadIdx.x == 0 && tma_on) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tbar_addr) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      constexpr unsigned BYTES = (unsigned)(TM::NBOX * TB * TM::BOXW * 4);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tbar_addr),
                   "r"(BYTES + (unsigned)p.tma_extra)
                   : "memory");
      const int g0 = tile * TB, ct = g0 % p.tma_d1, co = g0 / p.tma_d1;
      const unsigned dst0 = (unsigned)__cvta_generic_to_shared(smem_raw);
      if (p.tma_mode == 2) {
        // rows r of the line dim, TB points of the tile dim each: element (line l, point j) at
        // float 2 (j TB + l)
#pragma unroll 1
        for (int b = 0; b < TM::NBR; b++)
          asm volatile(
              "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
              "%4}], [%5];" ::"r"(dst0 + (unsigned)(b * TM::BOXR * TB * 8)),
              "l"(reinterpret_cast<unsigned long long>(tm)), "r"(2 * ct), "r"(b * TM::BOXR), "r"(co), "r"(tbar_addr)
              : "memory");
      } else {
#pragma unroll 1
        for (int b = 0; b < TM::NBOX; b++)
          asm volatile(
              "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
              "%4}], [%5];" ::"r"(dst0 + (unsigned)(b * TB * TM::BOXW * 4)),
              "l"(reinterpret_cast<unsigned long long>(tm)), "r"(b * TM::BOXW), "r"(ct), "r"(co), "r"(tbar_addr)
              : "memory");
      }
    }
    __syncthreads();
  }

  // The float-float FFT passes of a tile synchronise per line when each line's threads are whole
  // warps or share one warp and the load gives each line to consecutive threads (then the passes
  // of different lines run independently: -2.6% on the 512^3 round trip); otherwise, around the
  // block-wide steps, and for the FP32 kernels (measured 9% slower per line), per CTA.
  constexpr bool LSYNC = O::SCALED && SH::BLOCK == SH::USED && ((TT % 32 == 0 && TB <= 15) || (32 % TT == 0));
  // this thread's line and first point: the same V points j0 + e*TT for load, FFT and store
  int l, j0;
  if (p.load_Lmajor) {
    l = threadIdx.x / TT;
    j0 = threadIdx.x - l * TT;
  } else {
    l = threadIdx.x % TB;
    j0 = threadIdx.x / TB;
  }
  int ls, js;  // store-side mapping
  if (p.store_Lmajor) {
    ls = threadIdx.x / TT;
    js = threadIdx.x - ls * TT;
  } else {
    ls = threadIdx.x % TB;
    js = threadIdx.x / TB;
  }
  const G *gin = reinterpret_cast<const G *>(in);
  G *gout = reinterpret_cast<G *>(out);
  // barrier of this thread's FFT passes (fk_sync): per line only after a line-contiguous load
  // (remapping the FFT phase of a tile-dim-contiguous load to lines, with the float-float
  // conversion after the block-wide barrier, measured 1% slower on those stages)
  const int sid = (LSYNC && p.load_Lmajor) ? (TT > 32 ? 1 + l : -1) : 0;

  // One tile per CTA: a persistent loop over tiles was measured to keep ~80 more registers live.
  {
    const int g0 = tile * TB;
    const int gl = g0 + l;
    const bool act = valid && gl < p.nlines;
    // element offset of line g's first point; paired real lines: lines 2g and 2g+1 (the last
    // line of an odd count is paired with itself and its second result is not stored)
    auto line_base = [&](int g, long long st, long long so) -> long long {
      return (long long)(g % p.dt) * st + (long long)(g / p.dt) * so;
    };
    long long ibase, ibase2 = 0;
    if (KIND == FK_R2R1 && p.pair) {
      ibase = line_base(2 * gl, p.it, p.io);
      ibase2 = line_base(min(2 * gl + 1, p.nreal - 1), p.it, p.io);
    } else if (KIND == FK_R2RG && p.rg_cplx) {
      ibase = 2 * line_base(gl >> 1, p.it, p.io) + (gl & 1);  // in reals: one part of a complex line
    } else {
      ibase = line_base(gl, p.it, p.io);
    }
    // raw value of FFT input point j of this thread's line
    const G *src = gin + ((KIND == FK_R2C || (KIND == FK_R2R1 && p.pair) || KIND == FK_R2RG) ? ibase : 2 * ibase);
    const long long rstride = (KIND == FK_R2RG && p.rg_cplx) ? 2 * p.iL : p.iL;  // FK_R2RG, in reals
    const T *raux = reinterpret_cast<const T *>(p.aux);
    // FK_R2RG: the pre-twiddled, zero-padded input point j
    auto rg_pre = [&](C x, int j) -> C {
      if (j >= p.rg_n) return O::zero();
      if ((p.rg_half0 && j == 0) || (p.rg_half1 && j == p.rg_n - 1)) x = O::half(x);
      return O::mul(x, O::tw(raux, 2 * p.rg_b2 * j));
    };
    auto load_raw = [&](int j) -> RAW {
      if constexpr (KIND == FK_R2C) {  // packed z[j] = x[2j] + i x[2j+1]
        if (p.iL == 1) return O::ldraw(src + 2 * j);
        return O::ldraw2(src + (long long)(2 * j) * p.iL, src + (long long)(2 * j + 1) * p.iL);
      } else if constexpr (KIND == FK_R2R1) {
        // even extension x[0..n-1], x[n-2..1]; odd extension 0, x[0..n-1], 0, -x[n-1..0]
        int m = j;
        bool neg = false;
        if (!p.r2r_odd) {
          if (j > N / 2) m = N - j;
        } else {
          if (j == 0 || j == N / 2) return RAW{};
          if (j < N / 2) m = j - 1;
          else {
            m = N - j - 1;
            neg = true;
          }
        }
        RAW r = p.pair ? O::ldraw2(src + (long long)m * p.iL, gin + ibase2 + (long long)m * p.iL)
                       : O::ldraw(src + 2 * (long long)m * p.iL);
        return neg ? O::rneg(r) : r;
      } else if constexpr (KIND == FK_R2RG) {
        return j < p.rg_n ? O::ldraw1(src + (long long)j * rstride) : RAW{};
      } else {
        return O::ldraw(src + 2 * (long long)j * p.iL);
      }
    };

    // float-float input: producer-line scale of point j of this thread's line
    constexpr bool ffin = O::SCALED && (KIND == FK_C2C || KIND == FK_C2R) && (FF & 1);
    // (32-bit indices: a side array holds one scale per line, fewer than 2^31 - the launch checks)
    const int sib = ffin ? (gl % p.dt) * (int)p.fi_t + (gl / p.dt) * (int)p.fi_o : 0;
    auto sp_of = [&](int j) -> int { return __ldg(p.sin + (sib + j * (int)p.fi_j)); };
    // the scales of this thread's points, loaded with the points and kept in registers for the
    // conversion (a second load there would put an L2 round trip after the block reduction)
    int spv[V > 0 ? V : 1] = {};  // per-slot input line scales (float-float input only)
    int spn = 0;
    C *lb = buf + (size_t)l * LS;
    const int fsign = KIND == FK_C2C ? p.sign : ((KIND == FK_R2C || KIND == FK_R2R1 || KIND == FK_R2RG) ? -1 : 1);
    constexpr RadixList RL = fast_radices(N);
    // Native arithmetic, no C2R packing, and a first radix equal to the points per thread: the
    // values a thread loads are exactly the inputs of its first butterfly, so the first pass runs
    // on them in registers and the tile's first trip through shared memory is skipped.
    constexpr bool FUSE1 = !O::SCALED && KIND != FK_C2R && KIND != FK_R2R1 && KIND != FK_R2RG && RL.r[0] == V;
    static_assert(!TMA || FUSE1, "TMA staging feeds the first pass in registers");
    if constexpr (FUSE1) {
      constexpr int R0 = RL.r[0];
      C x[V];
      bool staged = false;
      if constexpr (TMA) {
        if (tma_on) {
          using TM = FastTma<N>;
          // every thread's wait ends (bytes arrived, or the time limit); the CTA agrees on the outcome
          const bool got = __syncthreads_and(fk_mbar_wait(tbar_addr, 0, p.tma_timeout_ns));
          if (!got) {
            // the tile is skipped; its copies get a second bounded wait before the CTA exits
            if (threadIdx.x == 0) {
              if (p.status) atomicExch(p.status, 1);
              fk_mbar_wait(tbar_addr, 0, p.tma_timeout_ns);
            }
            return;
          }
          if (act) {
            const float *stg = reinterpret_cast<const float *>(smem_raw);
#pragma unroll
            for (int e = 0; e < V; e++) {
              const int j = j0 + e * TT;
              const int f = 2 * j;  // point j = floats 2j, 2j + 1 of the line
              const int off = p.tma_mode == 2 ? 2 * (j * TB + l)
                                              : (f / TM::BOXW) * (TB * TM::BOXW) + l * TM::BOXW + f % TM::BOXW;
              x[e] = O::from_raw(*reinterpret_cast<const RAW *>(stg + off), 0);
            }
          }
          __syncthreads();  // the first pass below overwrites the staged tile
          staged = true;
        }
      }
      if (!staged && act) {
#pragma unroll
        for (int e = 0; e < V; e++) x[e] = O::from_raw(load_raw(j0 + e * TT), 0);
      }
      if (act) {
        if constexpr (R0 == 3) dft3<O>(x, fsign, O::tw(tab, (N / 3) * TWSTEP));
        else if constexpr (R0 == 5) dft5<O>(x, fsign, O::tw(tab, (N / 5) * TWSTEP), O::tw(tab, 2 * (N / 5) * TWSTEP));
        else dft_p2<O, R0>(x, fsign);
        const int pb = fk_pos<PS>(j0 * R0);
#pragma unroll
        for (int r = 0; r < R0; r++)
          lb[(fk_additive<PS>() && (R0 & (R0 - 1)) == 0 && R0 <= (1 << PS)) ? pb + r : fk_pos<PS>(j0 * R0 + r)] = O::norm(x[r]);
      }
      fk_sync<TT>(sid);
      if constexpr (RL.n > 1) fk_pass<O, N, TWSTEP, R0, 1>(lb, tab, ptab, j0, act, fsign, sid);
    }
    int sc_out = 0;  // the stored line's power-of-two scale (float-float)
    if constexpr (!FUSE1) {
    // ---------------- load the tile into shared memory ----------------
    // Raw input values go straight to their slot (slot N holds X[N] for C2R).  Float-float lines
    // are converted in place once their largest exponent is known.
    RAW *lr = reinterpret_cast<RAW *>(lb);
    int emax = 0;
    const int pj0 = fk_pos<PS>(j0);
    if (act && KIND == FK_R2R1) {
      // extensions: each input element is read once and written to slots j and N - j
      const int pn0 = fk_pos<PS>(N - j0);
      fk_for<V, O::IO_UNROLL>([&](int e) {
        const int j = j0 + e * TT;
        if (j > N / 2) return;
        const RAW r = load_raw(j);
        const bool mirror = j > 0 && j < N / 2;
        const RAW rm = (mirror && p.r2r_odd) ? O::rneg(r) : r;
        const int sj = fk_slot<PS, TT>(j0, pj0, e);
        const int sm = mirror ? fk_slot_rev<PS, TT, N>(j0, pn0, e) : sj;
        if (O::SCALED) {
          emax = max(emax, O::rexp(r));
          lr[sj] = r;
          lr[sm] = rm;
        } else {
          lb[sj] = O::from_raw(r, 0);
          lb[sm] = O::from_raw(rm, 0);
        }
      });
    } else if (act) {
      fk_for<V, O::IO_UNROLL>([&](int e) {
        const int sj = fk_slot<PS, TT>(j0, pj0, e);
        const RAW r = load_raw(j0 + e * TT);
        if (O::SCALED) {
          if constexpr (ffin) {
            spv[e] = sp_of(j0 + e * TT);
            emax = max(emax, O::rexp_ff(r, spv[e]));
          } else {
            emax = max(emax, O::rexp(r));
          }
          lr[sj] = r;
        } else if (KIND == FK_R2RG) {
          lb[sj] = rg_pre(O::from_raw(r, 0), j0 + e * TT);
        } else {
          lb[sj] = O::from_raw(r, 0);
        }
      });
      if (KIND == FK_C2R && j0 == 0) {
        RAW r = O::ldraw(src + 2 * (long long)N * p.iL);
        if (O::SCALED) {
          if constexpr (ffin) {
            spn = sp_of(N);
            emax = max(emax, O::rexp_ff(r, spn));
          } else {
            emax = max(emax, O::rexp(r));
          }
          lr[fk_pos<PS>(N)] = r;
        } else {
          lb[fk_pos<PS>(N)] = O::from_raw(r, 0);
        }
      }
    }
    int sc = 0;
    bool perline = false;  // lines scaled one by one (wide spread of magnitudes, or non-finite input)
    if constexpr (O::SCALED) {
      // The tile's largest exponent and the smallest of its threads' largest nonzero ones: when
      // they are within 2^40 (the usual case) one scale 2^sc brings the tile maximum near 2^20 and
      // keeps every line's precision (values are flushed only 2^94 below the tile maximum, so at
      // least 2^54 below their own line's).  Otherwise (rare, block-uniform) each line takes its own
      // scale from its finite values and keeps non-finite values, so that a line far smaller than
      // its neighbours keeps its precision and an infinity or NaN reaches only its own line.
      int emin = (act && emax > 0) ? emax : 0x7ff;
      const int wmax = __reduce_max_sync(0xffffffffu, emax), wmin = __reduce_min_sync(0xffffffffu, emin);
      if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = wmax;
        red2[threadIdx.x >> 5] = wmin;
      }
      __syncthreads();
      int tmax = 0, tmin = 0x7ff;
#pragma unroll
      for (int w = 0; w < SH::BLOCK / 32; w++) {
        tmax = max(tmax, red[w]);
        tmin = min(tmin, red2[w]);
      }
      perline = tmax == 0x7ff || tmax - tmin > 40;
      if (perline) {
        if ((int)threadIdx.x < TB) lfin[threadIdx.x] = 0;
        __syncthreads();
        int em = 0;
        if (act) {
          if (ffin) {
            fk_for<V, 1>([&](int e) {
              em = max(em, O::rexp_ff_finite(lr[fk_slot<PS, TT>(j0, pj0, e)], sp_of(j0 + e * TT)));
            });
            if (KIND == FK_C2R && j0 == 0) em = max(em, O::rexp_ff_finite(lr[fk_pos<PS>(N)], sp_of(N)));
          } else {
            fk_for<V, 1>([&](int e) { em = max(em, O::rexp_finite(lr[fk_slot<PS, TT>(j0, pj0, e)])); });
            if (KIND == FK_C2R && j0 == 0) em = max(em, O::rexp_finite(lr[fk_pos<PS>(N)]));
          }
        }
        {
          const unsigned grp = __match_any_sync(0xffffffffu, l);
          const int lm = __reduce_max_sync(grp, em);
          if (act && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(&lfin[l], lm);
        }
        __syncthreads();
        sc = 1043 - lfin[l];
        if (act) {
          fk_for<V, 1>([&](int e) {
            const int j = fk_slot<PS, TT>(j0, pj0, e);
            const C x = ffin ? O::from_ff(lr[j], sc - sp_of(j0 + e * TT)) : O::from_raw_nf(lr[j], sc);
            lb[j] = KIND == FK_R2RG ? rg_pre(x, j0 + e * TT) : x;
          });
          if (KIND == FK_C2R && j0 == 0)
            lb[fk_pos<PS>(N)] = ffin ? O::from_ff(lr[fk_pos<PS>(N)], sc - sp_of(N)) : O::from_raw_nf(lr[fk_pos<PS>(N)], sc);
        }
      } else {
        sc = 1043 - tmax;
        if (act) {
          // each thread converts its own slots in place (C2R: and slot N, which thread j0 = 0 loaded)
          fk_for<V, O::IO_UNROLL>([&](int e) {
            const int j = fk_slot<PS, TT>(j0, pj0, e);
            const C x = ffin ? O::from_ff(lr[j], sc - spv[e]) : O::from_raw(lr[j], sc);
            lb[j] = KIND == FK_R2RG ? rg_pre(x, j0 + e * TT) : x;
          });
          if (KIND == FK_C2R && j0 == 0)
            lb[fk_pos<PS>(N)] = ffin ? O::from_ff(lr[fk_pos<PS>(N)], sc - spn) : O::from_raw(lr[fk_pos<PS>(N)], sc);
        }
      }
    }
    fk_sync<TT>(sid);

    // ---------------- FFT (C2R: the half-length packing first) ----
    if constexpr (KIND == FK_C2R && FAST_C2R_PAIRS && O::SCALED) {
      // Z[k] = s + t and Z[N-k] = conj(s - t) from the pair X[k], X[N-k]: s = X[k] + conj X[N-k],
      // t = i conj(W_2N^k) (X[k] - conj X[N-k]); one twiddle product per pair, in place
      // (imaginary parts of X[0], X[N] ignored; slot N keeps a value no pass reads)
      if (act) {
#pragma unroll 1
        for (int k = j0; k <= N / 2; k += TT) {
          const int pk = fk_pos<PS>(k), pm = fk_pos<PS>(N - k);
          C xa = lb[pk], xb = lb[pm];
          if (k == 0) {
            xa = O::mk(O::re(xa), O::rzero());
            xb = O::mk(O::re(xb), O::rzero());
          }
          const C xbc = O::conj(xb);
          const C sv = O::add(xa, xbc), dv = O::sub(xa, xbc);
          const C tv = O::muli(O::mul(dv, O::conj(O::tw(tab, k))));
          lb[pk] = O::norm(O::add(sv, tv));
          if (2 * k != N) lb[pm] = O::norm(O::conj(O::sub(sv, tv)));
        }
      }
      fk_sync<TT>(sid);
      fk_pass<O, N, TWSTEP, 1, 0, false>(lb, tab, ptab, j0, act, fsign, sid);
    } else {
      // (the half-length packing formed as the first pass reads)
      fk_pass<O, N, TWSTEP, 1, 0, KIND == FK_C2R>(lb, tab, ptab, j0, act, fsign, sid);
    }
    // the scale of the line this thread stores (the store may map threads to other lines)
    if constexpr (O::SCALED) sc_out = perline ? 1043 - lfin[ls] : sc;
    }
    // a store that gives each thread points of other lines than the load waits for all of them
    if (sid != 0 && !p.store_Lmajor) __syncthreads();

    // ---------------- post-processing + store ----------------
    if constexpr (TMA && KIND == FK_C2C) {
      if (tma_on && p.tma_store) {
        // The tile leaves by TMA: each thread takes its points into registers, the CTA lays the
        // tile out over the region the FFT used as rows of TB points (row k: point k of the
        // tile's lines), and one thread stores the rows box by box, then waits until the copy
        // has read shared memory before the CTA exits.  (Full tiles only: the host checks.)
        using TM = FastTma<N>;
        const bool sact = valid;
        const int pjs = fk_pos<PS>(js);
        C yv[V];
        if (sact) {
          const C *Y = buf + (size_t)ls * LS;
#pragma unroll
          for (int e = 0; e < V; e++) yv[e] = fk_deriv<O>(p, Y[fk_slot<PS, TT>(js, pjs, e)], js + e * TT);
        }
        __syncthreads();
        RAW *stg = reinterpret_cast<RAW *>(smem_raw);
        if (sact) {
#pragma unroll
          for (int e = 0; e < V; e++) stg[(js + e * TT) * TB + ls] = O::to_raw(yv[e], 0);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
          const int ct = g0 % p.dt, co = g0 / p.dt;
          const unsigned src0 = (unsigned)__cvta_generic_to_shared(smem_raw);
#pragma unroll 1
          for (int b = 0; b < TM::NBR; b++)
            asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                             reinterpret_cast<unsigned long long>(tmo)),
                         "r"(2 * ct), "r"(b * TM::BOXR), "r"(co), "r"(src0 + (unsigned)(b * TM::BOXR * TB * 8))
                         : "memory");
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
        return;
      }
    }
    const int gs = g0 + ls;
    const bool sact = valid && gs < p.nlines;
    if (sact) {
      const C *Y = buf + (size_t)ls * LS;
      long long obase, obase2 = 0;
      bool second = false;  // paired real lines: the second line exists
      if (KIND == FK_R2R1 && p.pair) {
        obase = line_base(2 * gs, p.ot, p.oo);
        second = 2 * gs + 1 < p.nreal;
        obase2 = second ? line_base(2 * gs + 1, p.ot, p.oo) : 0;
      } else if (KIND == FK_R2RG && p.rg_cplx) {
        obase = 2 * line_base(gs >> 1, p.ot, p.oo) + (gs & 1);  // in reals
      } else {
        obase = line_base(gs, p.ot, p.oo);
      }
      const long long ostride = (KIND == FK_R2RG && p.rg_cplx) ? 2 * p.oL : p.oL;  // FK_R2RG, in reals
      const int pjs = fk_pos<PS>(js), pns = fk_pos<PS>(N - js);
      // float-float output: values at this line's scale, the scale beside them
      constexpr bool ffout = O::SCALED && (KIND == FK_C2C || KIND == FK_R2C) && (FF & 2);
      if (ffout && js == 0) p.sout[(gs % p.dt) * (int)p.fo_t + (gs / p.dt) * (int)p.fo_o] = sc_out;
      auto store_c = [&](G *ptr, C v) {
        if constexpr (ffout) O::stff(ptr, v);
        else O::straw(ptr, O::to_raw(v, sc_out));
      };
      if constexpr (KIND == FK_R2C && V % 2 == 0) {
        // X[k] = 1/2 (s - i t), X[N-k] = 1/2 conj(s + i t), with s = Z_k + conj Z_{N-k} and
        // t = W_2N^k (Z_k - conj Z_{N-k}): each thread unpacks the pairs (k, N-k), k < N/2,
        // k = 0 giving X[0] and X[N]; X[N/2] (its own partner) by the thread with js = 0
        auto put = [&](int k, C x) { store_c(gout + 2 * (obase + (long long)k * p.oL), fk_deriv<O>(p, x, k)); };
        fk_for<V / 2, O::IO_UNROLL>([&](int e) {
          const int k = js + e * TT;
          const C a = Y[fk_slot<PS, TT>(js, pjs, e)];
          const C b = O::conj(Y[k == 0 ? fk_pos<PS>(0) : fk_slot_rev<PS, TT, N>(js, pns, e)]);
          const C sv = O::add(a, b);
          const C it = O::muli(O::mul(O::sub(a, b), O::tw(tab, k)));
          put(k, O::half(O::sub(sv, it)));
          put(N - k, O::half(O::conj(O::add(sv, it))));
        });
        if (js == 0) {
          const C a = Y[fk_pos<PS>(N / 2)], b = O::conj(a);
          put(N / 2, O::half(O::sub(O::add(a, b), O::muli(O::mul(O::sub(a, b), O::tw(tab, N / 2))))));
        }
      } else
      fk_for<V, O::IO_UNROLL>([&](int e) {
        const int k = js + e * TT;
        const int sk = fk_slot<PS, TT>(js, pjs, e);
        if (KIND == FK_C2C) {
          store_c(gout + 2 * (obase + (long long)k * p.oL), fk_deriv<O>(p, Y[sk], k));
        } else if (KIND == FK_R2C) {
          // X[k] = 1/2 [(Z_k + conj Z_{N-k}) - i W_2N^k (Z_k - conj Z_{N-k})]
          C a = Y[sk], b = O::conj(Y[k == 0 ? 0 : fk_slot_rev<PS, TT, N>(js, pns, e)]);
          C s = O::add(a, b), d = O::sub(a, b);
          C x = O::half(O::sub(s, O::muli(O::mul(d, O::tw(tab, k)))));
          store_c(gout + 2 * (obase + (long long)k * p.oL), fk_deriv<O>(p, x, k));
          if (k == 0) {  // X[N] = Re Z_0 - Im Z_0
            C z0 = Y[fk_pos<PS>(0)];
            C xn = O::mk(O::re(O::norm(O::sub(O::mk(O::re(z0), O::rzero()), O::mk(O::im(z0), O::rzero())))), O::rzero());
            store_c(gout + 2 * (obase + (long long)N * p.oL), fk_deriv<O>(p, xn, N));
          }
        } else if (KIND == FK_R2R1) {
          // DCT-I: Y[k], k <= N/2; DST-I: i Y[k+1], k < N/2 - 1
          int ko = k;
          C y = Y[sk];
          if (!p.r2r_odd) {
            if (k > N / 2) return;
          } else {
            if (k == 0 || k >= N / 2) return;
            ko = k - 1;
            y = O::muli(y);
          }
          const RAW r = O::to_raw(y, sc_out);
          if (!p.pair) {
            O::straw(gout + 2 * (obase + (long long)ko * p.oL), r);
          } else if (second) {
            O::straw2(gout + obase + (long long)ko * p.oL, gout + obase2 + (long long)ko * p.oL, r);
          } else {
            O::strawx(gout + obase + (long long)ko * p.oL, r);
          }
        } else if (KIND == FK_R2RG) {
          // y_k = S+ + S- (cosine kinds) or -i (S+ - S-) (sine kinds), S- = W^{a2 (2k+b2)} U_k, S+ = conj S-
          if (k >= p.rg_n) return;
          const C sm = O::mul(Y[sk], O::tw(raux, p.rg_a2 * (2 * k + p.rg_b2)));
          const C sp = O::conj(sm);
          const C v = p.rg_sin ? O::mulmi(O::sub(sp, sm)) : O::add(sp, sm);
          O::strawx(gout + obase + (long long)k * ostride, O::to_raw(v, sc_out));
        } else {  // C2R: reals 2k, 2k+1 = z[k]
          RAW r = O::to_raw(Y[sk], sc_out);
          if (p.oL == 1) O::straw(gout + obase + 2 * k, r);
          else O::straw2(gout + obase + (long long)(2 * k) * p.oL, gout + obase + (long long)(2 * k + 1) * p.oL, r);
        }
      });
    }
  }
}

template <class O, int KIND, int N, int FF = 0>
__global__ void __launch_bounds__(FastShape<N>::BLOCK, fast_min_blocks<O, N, KIND>()) k_fast(FParams p) {
  fk_tile<O, KIND, N, FF>(p, blockIdx.x, p.in, p.out);
}

// Persistent form: a grid smaller than the tile count, each CTA walking the tiles with a grid
// stride, which bounds the SMs held by a stage that moves its data over the host link while the
// neighbour stage runs beside it.  A separate kernel: inside a loop the tile body no longer fits
// 64 registers and spills, so the one-tile-per-CTA kernel stays loop-free, and this one is
// compiled for 2 resident CTAs per SM (128 registers; a link stage needs few CTAs).
// Instantiated for the end stages of real-to-complex plans on the large-field lengths: R2C
// reading IEEE values (FF 0, or 2 with a float-float output) and C2R writing them (FF 0 or 1).
template <int KIND, int N>
constexpr bool fk_persist_variant() {
  return (KIND == FK_R2C || KIND == FK_C2R) &&
         (N == 64 || N == 128 || N == 256 || N == 512 || N == 1024 || N == 2048);
}
// Whether a launch of this kind, length and float-float sides can be capped (host side).
inline bool fast_persist_ok(int kind, int n, int ffin, int ffout) {
  const bool len = n == 64 || n == 128 || n == 256 || n == 512 || n == 1024 || n == 2048;
  return len && ((kind == FK_R2C && !ffin) || (kind == FK_C2R && !ffout));
}
#ifndef FAST_PERSIST_MINB
#define FAST_PERSIST_MINB 2  // resident CTAs per SM the persistent kernels are compiled for
#endif
template <class O, int KIND, int N, int FF = 0>
__global__ void __launch_bounds__(FastShape<N>::BLOCK, FAST_PERSIST_MINB)
    k_fast_persist(FParams p) {
  __shared__ int nxt;
  for (int t = blockIdx.x;;) {
    fk_tile<O, KIND, N, FF>(p, t, p.in, p.out);
    if (p.tile_ctr) {
      if (threadIdx.x == 0) nxt = (int)gridDim.x + atomicAdd(p.tile_ctr, 1);
      __syncthreads();
      t = nxt;
    } else {
      t += gridDim.x;
    }
    if (t >= p.ntotal) break;
    __syncthreads();
  }
}

// The tile's input staged by the tensor-memory accelerator (fk_tma_variant lengths and kinds).
template <class O, int KIND, int N>
__global__ void __launch_bounds__(FastShape<N>::BLOCK, fast_min_blocks<O, N, KIND>())
    k_fast_tma(FParams p, const __grid_constant__ CUtensorMap tm, const __grid_constant__ CUtensorMap tmo) {
  if constexpr (fk_tma_variant<O, KIND, N>()) fk_tile<O, KIND, N, 0, true>(p, blockIdx.x, p.in, p.out, &tm, &tmo);
}

// Lengths and kinds with float-float intermediate variants (DFP: C2C in / out / both, R2C out,
// C2R in; the power-of-two lengths from 64, which carry the large fields)
template <class O, int KIND, int N>
constexpr bool fk_ff_variants() {
  return std::is_same_v<O, DFP> && (KIND == FK_C2C || KIND == FK_R2C || KIND == FK_C2R) &&
         (N == 64 || N == 128 || N == 256 || N == 512 || N == 1024 || N == 2048);
}
inline bool fast_ff_length(int n) { return n == 64 || n == 128 || n == 256 || n == 512 || n == 1024 || n == 2048; }

// Work-list launch: item w is tile work[w].tile of the stage whose parameters are
// plist[work[w].stage]; the parameters are staged in shared memory for the tile.  One CTA per
// item.  No CTA waits on another.
// (A grid-stride loop over the list, for a grid smaller than the list, was measured no faster
// and makes the tile body spill: inside a loop it no longer fits 64 registers.)
template <class O, int KIND, int N>
__global__ void __launch_bounds__(FastShape<N>::BLOCK, fast_min_blocks<O, N, KIND>())
    k_fast_list(const FParams *plist, const FWork *work, int nwork) {
  __shared__ FParams sp;
  constexpr int NW = (int)(sizeof(FParams) / sizeof(int));
  static_assert(sizeof(FParams) % sizeof(int) == 0, "FParams copied as ints");
  const int w = blockIdx.x;
  if (w >= nwork) return;
  const FWork it = work[w];
  const int *src = reinterpret_cast<const int *>(plist + it.stage);
  for (int i = threadIdx.x; i < NW; i += blockDim.x) reinterpret_cast<int *>(&sp)[i] = __ldg(src + i);
  __syncthreads();
  fk_tile<O, KIND, N>(sp, it.tile, sp.in, sp.out);
}

// ------------------------------------------------------------------------------------------
// host side
struct FastArgs {
  int kind;  // FastKind
  int n;     // complex FFT length N
  FParams p;
  int split = 0;  // FP32 only: split-twiddle kernels (NativeFS; table format 2)
  int tma = 0;    // single launches only: the tile's input staged by TMA through tm[0] (k_fast_tma)
  CUtensorMap tm[2];  // the input's tensor map and (p.tma_store) the output's
};

template <class O>
struct is_split_policy : std::false_type {};
template <bool P>
struct is_split_policy<NativeFS<P>> : std::true_type {};

// FFT lengths of the FP32 split-twiddle kernels (the long lines)
#define P3D_FAST_SPLIT_LENGTHS(X) X(512) X(1024) X(2048)
inline bool fast_split_length(int n) { return n == 512 || n == 1024 || n == 2048; }

template <class O, int KIND, int N>
constexpr size_t fk_smem() {
  return sizeof(typename O::C) * (size_t)FastShape<N>::TB * fast_ls<N, (int)sizeof(typename O::C)>();
}

// Sets the kernel's dynamic shared-memory limit once; this also loads the kernel's module (which
// CUDA otherwise does lazily at the first launch).
template <class O, int KIND, int N>
static int fk_configure() {
  static_assert(fast_radices(N).n > 0, "length must be 2^a 3^b 5^c");
  static bool configured = false;
  if (!configured) {
    if (cudaFuncSetAttribute(k_fast<O, KIND, N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)fk_smem<O, KIND, N>()) != cudaSuccess ||
        cudaFuncSetAttribute(k_fast_list<O, KIND, N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)fk_smem<O, KIND, N>()) != cudaSuccess)
      return E_CUDA;
    if constexpr (fk_tma_variant<O, KIND, N>()) {
      if (cudaFuncSetAttribute(k_fast_tma<O, KIND, N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)fk_smem<O, KIND, N>()) != cudaSuccess)
        return E_CUDA;
    }
    if constexpr (fk_ff_variants<O, KIND, N>()) {
      const int sm = (int)fk_smem<O, KIND, N>();
      if (cudaFuncSetAttribute(k_fast<O, KIND, N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) != cudaSuccess ||
          cudaFuncSetAttribute(k_fast<O, KIND, N, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) != cudaSuccess ||
          cudaFuncSetAttribute(k_fast<O, KIND, N, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) != cudaSuccess)
        return E_CUDA;
    }
    if constexpr (fk_persist_variant<KIND, N>()) {
      const int sm = (int)fk_smem<O, KIND, N>();
      if (cudaFuncSetAttribute(k_fast_persist<O, KIND, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) !=
          cudaSuccess)
        return E_CUDA;
      if constexpr (fk_ff_variants<O, KIND, N>()) {
        constexpr int FFV = KIND == FK_R2C ? 2 : 1;
        if (cudaFuncSetAttribute(k_fast_persist<O, KIND, N, FFV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 sm) != cudaSuccess)
          return E_CUDA;
      }
    }
    configured = true;
  }
  return E_OK;
}

template <class O, int KIND, int N>
static int fk_launch(const FParams &p, const FGroup *g, int ctas, cudaStream_t st, const CUtensorMap *tm) {
  if (fk_configure<O, KIND, N>() != E_OK) return E_CUDA;
  if (g) {
    if (ctas <= 0) return E_OK;
    k_fast_list<O, KIND, N><<<(unsigned)g->nwork, FastShape<N>::BLOCK, fk_smem<O, KIND, N>(), st>>>(
        g->plist, g->work, g->nwork);
  } else {
    if (p.ntotal <= 0) return E_OK;
    const int ff = (p.ffin ? 1 : 0) | (p.ffout ? 2 : 0);
    const unsigned nb = (unsigned)p.ntotal;
    constexpr int BL = FastShape<N>::BLOCK;
    constexpr size_t SM = fk_smem<O, KIND, N>();
    // ctas > 0 caps the grid of a single launch at that many persistent CTAs (the lengths, kinds
    // and float-float sides of k_fast_persist; fast_persist_ok tells which)
    if constexpr (fk_persist_variant<KIND, N>()) {
      if (ctas > 0 && !tm && ctas < p.ntotal) {
        const unsigned pb = (unsigned)ctas;
        constexpr int FFV = KIND == FK_R2C ? 2 : 1;
        if (ff == 0) {
          k_fast_persist<O, KIND, N><<<pb, BL, SM, st>>>(p);
          return cudaGetLastError() == cudaSuccess ? E_OK : E_CUDA;
        }
        if constexpr (fk_ff_variants<O, KIND, N>()) {
          if (ff == FFV) {
            k_fast_persist<O, KIND, N, FFV><<<pb, BL, SM, st>>>(p);
            return cudaGetLastError() == cudaSuccess ? E_OK : E_CUDA;
          }
        }
      }
    }
    if (tm) {
      if constexpr (fk_tma_variant<O, KIND, N>()) {
        if (ff) return E_UNSUPPORTED;
        k_fast_tma<O, KIND, N><<<nb, BL, SM, st>>>(p, tm[0], tm[1]);
        return cudaGetLastError() == cudaSuccess ? E_OK : E_CUDA;
      } else {
        return E_UNSUPPORTED;
      }
    }
    if constexpr (fk_ff_variants<O, KIND, N>()) {
      if (ff == 1) k_fast<O, KIND, N, 1><<<nb, BL, SM, st>>>(p);
      else if (ff == 2) k_fast<O, KIND, N, 2><<<nb, BL, SM, st>>>(p);
      else if (ff == 3) k_fast<O, KIND, N, 3><<<nb, BL, SM, st>>>(p);
      else k_fast<O, KIND, N><<<nb, BL, SM, st>>>(p);
    } else {
      if (ff) return E_UNSUPPORTED;
      k_fast<O, KIND, N><<<nb, BL, SM, st>>>(p);
    }
  }
  return cudaGetLastError() == cudaSuccess ? E_OK : E_CUDA;
}

// The float-float kernels are the slowest to compile; their translation units are split in two
// by length (alternate entries of P3D_FAST_LENGTHS), so that the halves compile in parallel.
template <class O>
constexpr int fast_nparts() {
  return std::is_same_v<O, DFP> ? 2 : 1;
}
#define P3D_FAST_ITEM(L) L,
constexpr int kFastLengths[] = {P3D_FAST_LENGTHS(P3D_FAST_ITEM)};
#undef P3D_FAST_ITEM
constexpr int fast_length_index(int n) {
  for (int i = 0; i < (int)(sizeof(kFastLengths) / sizeof(int)); i++)
    if (kFastLengths[i] == n) return i;
  return -1;
}
template <class O>
constexpr int fast_part_of(int n) {
  return fast_length_index(n) < 0 ? 0 : fast_length_index(n) % fast_nparts<O>();
}

// Lengths of part PART: n > 0 launches the length-n kernel (one stage, or a group of stages when g
// is set); n == 0 configures (loads) every length's kernels.
template <class O, int KIND, int PART>
static int fk_dispatch_n(int n, const FParams &p, const FGroup *g, int ctas, cudaStream_t st, const CUtensorMap *tm) {
  if constexpr (is_split_policy<O>::value) {  // long lines only
    if (n == 0) {
      int rc = E_OK;
#define P3D_FAST_CASE(L) \
  if (fk_configure<O, KIND, L>() != E_OK) rc = E_CUDA;
      P3D_FAST_SPLIT_LENGTHS(P3D_FAST_CASE)
#undef P3D_FAST_CASE
      return rc;
    }
#define P3D_FAST_CASE(L) \
  case L: return fk_launch<O, KIND, L>(p, g, ctas, st, tm);
    switch (n) {
      P3D_FAST_SPLIT_LENGTHS(P3D_FAST_CASE)
      default: return E_UNSUPPORTED;
    }
#undef P3D_FAST_CASE
  }
  if (n == 0) {
    int rc = E_OK;
#define P3D_FAST_CASE(L)                                                      \
  if constexpr (fast_part_of<O>(L) == PART) {                                 \
    if (fk_configure<O, KIND, L>() != E_OK) rc = E_CUDA;                      \
  }
    if constexpr (KIND == FK_R2R1 || KIND == FK_R2RG) {
      P3D_FAST_EVEN_LENGTHS(P3D_FAST_CASE)
    } else {
      P3D_FAST_LENGTHS(P3D_FAST_CASE)
    }
#undef P3D_FAST_CASE
    return rc;
  }
#define P3D_FAST_CASE(L)                                                      \
  case L:                                                                     \
    if constexpr (fast_part_of<O>(L) == PART) return fk_launch<O, KIND, L>(p, g, ctas, st, tm); \
    else return E_UNSUPPORTED;
  if constexpr (KIND == FK_R2R1 || KIND == FK_R2RG) {
    switch (n) {
      P3D_FAST_EVEN_LENGTHS(P3D_FAST_CASE)
      default: return E_UNSUPPORTED;
    }
  } else {
    switch (n) {
      P3D_FAST_LENGTHS(P3D_FAST_CASE)
      default: return E_UNSUPPORTED;
    }
  }
#undef P3D_FAST_CASE
}

// One (arithmetic, kind, part) per translation unit (fast_inst.cu), so they compile in parallel.
template <class O, int KIND, int PART>
int fast_launch_part(int n, const FParams &p, const FGroup *g, int ctas, cudaStream_t st, const CUtensorMap *tm);
#define P3D_FAST_DECL(O, K, P) \
  template <>                  \
  int fast_launch_part<O, K, P>(int, const FParams &, const FGroup *, int, cudaStream_t, const CUtensorMap *);
#define P3D_FAST_DECL_KINDS(O, P) \
  P3D_FAST_DECL(O, FK_C2C, P)     \
  P3D_FAST_DECL(O, FK_R2C, P)     \
  P3D_FAST_DECL(O, FK_C2R, P)     \
  P3D_FAST_DECL(O, FK_R2R1, P)    \
  P3D_FAST_DECL(O, FK_R2RG, P)
P3D_FAST_DECL_KINDS(DFP, 0)
P3D_FAST_DECL_KINDS(DFP, 1)
P3D_FAST_DECL_KINDS(Native<double>, 0)
P3D_FAST_DECL_KINDS(Native<float>, 0)
P3D_FAST_DECL_KINDS(FSplit, 0)
#undef P3D_FAST_DECL_KINDS
#undef P3D_FAST_DECL

template <class O, int KIND>
inline int fast_launch_kind(int n, const FParams &p, const FGroup *g, int ctas, cudaStream_t st,
                            const CUtensorMap *tm) {
  if constexpr (fast_nparts<O>() == 1) {
    return fast_launch_part<O, KIND, 0>(n, p, g, ctas, st, tm);
  } else {
    static_assert(fast_nparts<O>() == 2, "two parts");
    if (n == 0) {
      const int r0 = fast_launch_part<O, KIND, 0>(0, p, g, ctas, st, tm);
      const int r1 = fast_launch_part<O, KIND, 1>(0, p, g, ctas, st, tm);
      return r0 != E_OK ? r0 : r1;
    }
    return fast_part_of<O>(n) == 0 ? fast_launch_part<O, KIND, 0>(n, p, g, ctas, st, tm)
                                   : fast_launch_part<O, KIND, 1>(n, p, g, ctas, st, tm);
  }
}

template <class O>
inline int fast_launch_arith(const FastArgs &a, const FGroup *g, int ctas, cudaStream_t st) {
  const CUtensorMap *tm = (a.tma && !g) ? a.tm : nullptr;
  switch (a.kind) {
    case FK_C2C: return fast_launch_kind<O, FK_C2C>(a.n, a.p, g, ctas, st, tm);
    case FK_R2C: return fast_launch_kind<O, FK_R2C>(a.n, a.p, g, ctas, st, tm);
    case FK_C2R: return fast_launch_kind<O, FK_C2R>(a.n, a.p, g, ctas, st, tm);
    case FK_R2R1: return fast_launch_kind<O, FK_R2R1>(a.n, a.p, g, ctas, st, tm);
    case FK_R2RG: return fast_launch_kind<O, FK_R2RG>(a.n, a.p, g, ctas, st, tm);
    default: return E_UNSUPPORTED;
  }
}

// Loads every specialised kernel of one arithmetic (prec 4, or prec 8 with arith).
inline int fast_preload(int prec, int arith) {
  FastArgs a{};
  int rc = E_OK;
  for (int k = FK_C2C; k <= FK_R2RG; k++) {
    a.kind = k;
    a.n = 0;
    int r;
    if (prec == 4) {
      r = fast_launch_arith<Native<float>>(a, nullptr, 0, 0);
      const int r2 = fast_launch_arith<FSplit>(a, nullptr, 0, 0);
      if (r2 != E_OK) r = r2;
    } else if (arith == AR_DF) r = fast_launch_arith<DFP>(a, nullptr, 0, 0);
    else r = fast_launch_arith<Native<double>>(a, nullptr, 0, 0);
    if (r != E_OK) rc = r;
  }
  return rc;
}

// prec 4: FP32; prec 8: float-float (arith AR_DF) or native FP64.  With g set, one launch of
// `ctas` CTAs covers the group of stages g describes (a.kind and a.n select the kernel); without
// g, ctas > 0 caps the stage's grid at that many persistent CTAs.
inline int launch_fast(int prec, int arith, const FastArgs &a, cudaStream_t st, const FGroup *g = nullptr,
                       int ctas = 0) {
  if (prec == 4) {
    if (a.split) return fast_launch_arith<FSplit>(a, g, ctas, st);
    return fast_launch_arith<Native<float>>(a, g, ctas, st);
  }
  if (arith == AR_DF) return fast_launch_arith<DFP>(a, g, ctas, st);
  return fast_launch_arith<Native<double>>(a, g, ctas, st);
}

inline bool fast_supported(int n, int kind = FK_C2C) {
  if ((kind == FK_R2R1 || kind == FK_R2RG) && n % 2) return false;
  switch (n) {
#define P3D_FAST_CASE(L) case L:
    P3D_FAST_LENGTHS(P3D_FAST_CASE)
#undef P3D_FAST_CASE
    return true;
    default: return false;
  }
}
inline int fast_tile_lines(int n) {
  const int T = n / fast_points(n);
  return T >= 256 ? 1 : 256 / T;
}

}  // namespace p3d
