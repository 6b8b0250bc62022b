// Specialised stage kernels for the hot transform kinds (C2C, even-length R2C and C2R) at
// power-of-two FFT lengths 32..4096, one instantiation per (arithmetic, kind, length).
//
// Same contract as k_stage (one reference transplan stage: gather a tile of lines along the
// transform dimension from the input memory order, transform, scatter into the output memory
// order), organised for instruction economy:
//   - one tile of TB lines per CTA; twiddles through the read-only cache
//   - every thread owns V points of one line (the same points for load, FFT and store), so all
//     index arithmetic is compile-time except the per-tile base offsets
//   - loads go to registers first; float-float tiles are scaled by a power of two chosen from
//     the tile's largest exponent (block-wide max) before conversion, which keeps any finite
//     input in range
//   - radix-8/4/2 butterflies in registers, one padded shared-memory scatter per pass
//   - R2C / C2R half-length packing and the fused i*k derivative are done on the way in / out
#pragma once
#include <cuda_runtime.h>

#include "kernels.h"
#include "stage_common.cuh"

namespace p3d {

enum FastKind { FK_C2C = 0, FK_R2C = 1, FK_C2R = 2 };

struct FParams {
  const void *in;
  void *out;
  const void *tw;  // W_{tabN}^m, tabN = N (C2C) or 2N (R2C / C2R), m < tabN
  long long iL, it, io, oL, ot, oo;  // element strides
  int dt, ntile, ntotal;             // tile-dim size, tiles along it, tiles in total
  int sign;                          // C2C: -1 forward, +1 backward
  int deriv, dg, dmid;               // fused derivative (compute_deriv_loc wavenumbers)
  int load_Lmajor, store_Lmajor;
};

// resident 256-thread CTAs per SM the register allocation is sized for
#ifndef FAST_MIN_BLOCKS
#define FAST_MIN_BLOCKS 4
#endif

template <int N, int V>
struct FastShape {
  static constexpr int T = N / V;                      // threads per line
  static constexpr int TB = T >= 256 ? 1 : 256 / T;    // lines per tile
  static constexpr int BLOCK = TB * T;
  // Padded line stride (complex slots, > N + N/8 so slot N fits): chosen so that the TB lines of
  // a t-major access (consecutive threads on consecutive lines) fall in distinct 16-byte bank
  // groups, LS = 8/TB mod 8 (odd when TB >= 8).
  static constexpr int BASE = N + N / 8;
  static constexpr int TGT = TB >= 8 ? 1 : 8 / TB;
  static constexpr int ADJ = ((TGT - BASE % 8) % 8 + 8) % 8;
  static constexpr int LS = BASE + (ADJ == 0 ? 8 : ADJ);
};

// Twiddles are read through the read-only data cache (the table is a few KB and stays L1
// resident across the CTAs of an SM); a shared-memory copy per CTA was measured to cost more
// registers and L2 traffic than it saves.
template <class O>
__device__ __forceinline__ typename O::C fk_tw(const typename O::T *tab, int m, int sign) {
  typename O::C w = O::tw(tab, m);
  return sign < 0 ? w : O::conj(w);
}

// Stockham passes in registers with a padded shared-memory scatter per pass (cf. fixed_pass).
template <class O, int N, int V, int TWSTEP, int Ns, int R, int... Rest>
__device__ __forceinline__ void fk_pass(typename O::C *line, const typename O::T *tab, int j, bool active, int sign) {
  using C = typename O::C;
  constexpr int T = N / V, NB = V / R, M = N / R;
  C v[V];
  if (active) {
#pragma unroll
    for (int b = 0; b < NB; b++) {
      const int jj = j + b * T;
#pragma unroll
      for (int r = 0; r < R; r++) v[b * R + r] = line[pad<3>(jj + r * M)];
      if (Ns > 1) {
        const int k = jj & (Ns - 1);
#pragma unroll
        for (int r = 1; r < R; r++)
          v[b * R + r] = O::mul(v[b * R + r], fk_tw<O>(tab, r * k * (N / (Ns * R)) * TWSTEP, sign));
      }
      dft_p2<O, R>(&v[b * R], sign);
    }
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int b = 0; b < NB; b++) {
      const int jj = j + b * T;
      const int k = jj & (Ns - 1);
      const int base = (jj - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) line[pad<3>(base + r * Ns)] = O::norm(v[b * R + r]);
    }
  }
  __syncthreads();
  if constexpr (sizeof...(Rest) > 0) fk_pass<O, N, V, TWSTEP, Ns * R, Rest...>(line, tab, j, active, sign);
}

template <class O>
__device__ __forceinline__ typename O::C fk_deriv(const FParams &p, typename O::C v, int k) {
  if (!p.deriv) return v;
  if (k == p.dmid) return O::zero();
  return O::iscale(v, (k < p.dmid) ? k : k - p.dg);
}

template <class O, int KIND, int N, int V, int... Rs>
__global__ void __launch_bounds__(FastShape<N, V>::BLOCK, FAST_MIN_BLOCKS * 256 / FastShape<N, V>::BLOCK)
    k_fast(FParams p) {
  using C = typename O::C;
  using T = typename O::T;
  using G = typename O::G;
  using RAW = typename O::RAW;
  using SH = FastShape<N, V>;
  constexpr int TWSTEP = (KIND == FK_C2C) ? 1 : 2;  // FFT twiddle W_N^m = tab[m * TWSTEP]
  constexpr int LS = SH::LS, TB = SH::TB, TT = SH::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf = reinterpret_cast<C *>(smem_raw);
  __shared__ int red[32];
  const T *tab = reinterpret_cast<const T *>(p.tw);

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
  const G *gin = reinterpret_cast<const G *>(p.in);
  G *gout = reinterpret_cast<G *>(p.out);

  // One tile per CTA: a persistent loop over tiles was measured to keep ~80 more registers live.
  {
    const int tile = blockIdx.x;
    const int tt = tile % p.ntile, oth = tile / p.ntile;
    const int t0 = tt * TB;
    const int nlines = min(TB, p.dt - t0);
    const bool act = l < nlines;
    const long long ibase = (long long)(t0 + l) * p.it + (long long)oth * p.io;

    // ---------------- load the tile into shared memory ----------------
    // Raw input values go straight to their slot (slot N holds X[N] for C2R).  Float-float tiles
    // are converted in place once the block-wide largest exponent is known.
    C *lb = buf + (size_t)l * LS;
    RAW *lr = reinterpret_cast<RAW *>(lb);
    int emax = 0;
    if (act) {
      const G *src = gin + (KIND == FK_R2C ? ibase : 2 * ibase);
#pragma unroll 2
      for (int e = 0; e < V; e++) {
        const int j = j0 + e * TT;
        RAW r;
        if (KIND == FK_R2C) {  // packed z[j] = x[2j] + i x[2j+1]
          if (p.iL == 1) r = O::ldraw(src + 2 * j);
          else r = O::ldraw2(src + (long long)(2 * j) * p.iL, src + (long long)(2 * j + 1) * p.iL);
        } else {
          r = O::ldraw(src + 2 * (long long)j * p.iL);
        }
        if (O::SCALED) {
          emax = max(emax, O::rexp(r));
          lr[pad<3>(j)] = r;
        } else {
          lb[pad<3>(j)] = O::from_raw(r, 0);
        }
      }
      if (KIND == FK_C2R && j0 == 0) {
        RAW r = O::ldraw(src + 2 * (long long)N * p.iL);
        if (O::SCALED) {
          emax = max(emax, O::rexp(r));
          lr[pad<3>(N)] = r;
        } else {
          lb[pad<3>(N)] = O::from_raw(r, 0);
        }
      }
    }
    int sc = 0;
    if (O::SCALED) {
      // block-wide max exponent -> scale 2^sc bringing the tile maximum near 2^20
      emax = __reduce_max_sync(0xffffffffu, emax);
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = emax;
      __syncthreads();
      emax = 0;
#pragma unroll
      for (int w = 0; w < SH::BLOCK / 32; w++) emax = max(emax, red[w]);
      sc = 1043 - emax;
      if (act && KIND != FK_C2R) {
#pragma unroll 2
        for (int e = 0; e < V; e++) {
          const int j = pad<3>(j0 + e * TT);
          lb[j] = O::from_raw(lr[j], sc);
        }
      }
    }
    if (KIND == FK_C2R) {
      // Z'[k] = (X[k] + conj X[N-k]) + i conj(W_2N^k) (X[k] - conj X[N-k]); imag of X[0], X[N] ignored
      __syncthreads();
      C z[V];
      if (act) {
#pragma unroll
        for (int e = 0; e < V; e++) {
          const int k = j0 + e * TT;
          C a, b;
          if (O::SCALED) {
            a = O::from_raw(lr[pad<3>(k)], sc);
            b = O::from_raw(lr[pad<3>(N - k)], sc);
          } else {
            a = lb[pad<3>(k)];
            b = lb[pad<3>(N - k)];
          }
          if (k == 0) {
            a.y = O::rzero();
            b.y = O::rzero();
          }
          C bc = O::conj(b);
          C s = O::add(a, bc), d = O::sub(a, bc);
          C w = O::conj(O::tw(tab, k));
          z[e] = O::norm(O::add(s, O::muli(O::mul(w, d))));
        }
      }
      __syncthreads();
      if (act) {
#pragma unroll
        for (int e = 0; e < V; e++) lb[pad<3>(j0 + e * TT)] = z[e];
      }
    }
    __syncthreads();

    // ---------------- FFT ----------------
    fk_pass<O, N, V, TWSTEP, 1, Rs...>(lb, tab, j0, act, KIND == FK_C2C ? p.sign : (KIND == FK_R2C ? -1 : 1));

    // ---------------- post-processing + store ----------------
    const bool sact = ls < nlines;
    if (sact) {
      const C *Y = buf + (size_t)ls * LS;
      const long long obase = (long long)(t0 + ls) * p.ot + (long long)oth * p.oo;
#pragma unroll 2
      for (int e = 0; e < V; e++) {
        const int k = js + e * TT;
        if (KIND == FK_C2C) {
          O::straw(gout + 2 * (obase + (long long)k * p.oL), O::to_raw(fk_deriv<O>(p, Y[pad<3>(k)], k), sc));
        } else if (KIND == FK_R2C) {
          // X[k] = 1/2 [(Z_k + conj Z_{N-k}) - i W_2N^k (Z_k - conj Z_{N-k})]
          C a = Y[pad<3>(k)], b = O::conj(Y[pad<3>(k == 0 ? 0 : N - k)]);
          C s = O::add(a, b), d = O::sub(a, b);
          C x = O::half(O::sub(s, O::muli(O::mul(O::tw(tab, k), d))));
          O::straw(gout + 2 * (obase + (long long)k * p.oL), O::to_raw(fk_deriv<O>(p, x, k), sc));
          if (k == 0) {  // X[N] = Re Z_0 - Im Z_0
            C z0 = Y[pad<3>(0)];
            C xn = O::mk(O::norm(O::sub(O::mk(z0.x, O::rzero()), O::mk(z0.y, O::rzero()))).x, O::rzero());
            O::straw(gout + 2 * (obase + (long long)N * p.oL), O::to_raw(fk_deriv<O>(p, xn, N), sc));
          }
        } else {  // C2R: reals 2k, 2k+1 = z[k]
          RAW r = O::to_raw(Y[pad<3>(k)], sc);
          if (p.oL == 1) O::straw(gout + obase + 2 * k, r);
          else O::straw2(gout + obase + (long long)(2 * k) * p.oL, gout + obase + (long long)(2 * k + 1) * p.oL, r);
        }
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------
// host side
struct FastArgs {
  int kind;  // FastKind
  int n;     // complex FFT length N
  FParams p;
};

template <class O, int KIND, int N, int V, int... Rs>
static int fk_launch(const FParams &p, cudaStream_t st) {
  using SH = FastShape<N, V>;
  const size_t smem = sizeof(typename O::C) * (size_t)SH::TB * SH::LS;
  static bool configured = false;
  auto kern = k_fast<O, KIND, N, V, Rs...>;
  if (!configured) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return E_CUDA;
    configured = true;
  }
  if (p.ntotal <= 0) return E_OK;
  kern<<<(unsigned)p.ntotal, SH::BLOCK, smem, st>>>(p);
  return cudaGetLastError() == cudaSuccess ? E_OK : E_CUDA;
}

template <class O, int KIND>
static int fk_dispatch_n(int n, const FParams &p, cudaStream_t st) {
  switch (n) {
    case 32: return fk_launch<O, KIND, 32, 8, 8, 4>(p, st);
    case 64: return fk_launch<O, KIND, 64, 8, 8, 8>(p, st);
    case 128: return fk_launch<O, KIND, 128, 8, 8, 8, 2>(p, st);
    case 256: return fk_launch<O, KIND, 256, 8, 8, 8, 4>(p, st);
    case 512: return fk_launch<O, KIND, 512, 8, 8, 8, 8>(p, st);
    case 1024: return fk_launch<O, KIND, 1024, 8, 8, 8, 8, 2>(p, st);
    case 2048: return fk_launch<O, KIND, 2048, 8, 8, 8, 8, 4>(p, st);
    default: return E_UNSUPPORTED;
  }
}

template <class O>
static int fk_dispatch(const FastArgs &a, cudaStream_t st) {
  switch (a.kind) {
    case FK_C2C: return fk_dispatch_n<O, FK_C2C>(a.n, a.p, st);
    case FK_R2C: return fk_dispatch_n<O, FK_R2C>(a.n, a.p, st);
    case FK_C2R: return fk_dispatch_n<O, FK_C2R>(a.n, a.p, st);
    default: return E_UNSUPPORTED;
  }
}

int launch_fast_df(const FastArgs &a, cudaStream_t st);
int launch_fast_f64(const FastArgs &a, cudaStream_t st);
int launch_fast_f32(const FastArgs &a, cudaStream_t st);

inline bool fast_supported(int n) { return n >= 32 && n <= 2048 && (n & (n - 1)) == 0; }
inline int fast_tile_lines(int n) {
  const int T = n / 8;
  return T >= 256 ? 1 : 256 / T;
}

}  // namespace p3d
