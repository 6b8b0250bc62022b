// sm_103a kernels for the P3DFFT++ stage pipeline.
//
// One kernel family, `k_stage`, executes a whole reference "transplan" stage
// (build/exec.C:522-702): it gathers a tile of TB lines along the transform dimension L from
// the input memory order, runs the 1D transform in shared memory (Stockham autosort, mixed
// radix 2/3/4/5/7/8 + generic odd radix), applies the kind's pre/post-processing (R2C/C2R
// half-length packing, DCT/DST extensions, the fused i*k derivative of compute_deriv_loc,
// build/exec.C:228-287) and scatters the tile into the output memory order.  Each stage
// therefore reads and writes HBM exactly once; the reference's reorder_trans/reorder_out
// transposes (build/exec.C:737-2032) are folded into the tile gather/scatter.
//
// The arithmetic is a policy template:
//   Native<double>  FP64 data, DFMA arithmetic
//   Native<float>   FP32 data, FFMA arithmetic, twiddles rounded from FP64/long-double tables
//   DF              FP64 data, float-float arithmetic on the FP32 pipe (df_arith.cuh)
#include <cuda_runtime.h>
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <mutex>
#include <vector>

#include "fast_stage.cuh"
#include "kernels.h"
#include "stage_common.cuh"

namespace p3d {

// ------------------------------------------------------------------------------------------
struct KParams {
  const void *in;
  void *out;
  const void *tw;   // W_tabN^m, m < tabN (forward sign)
  const void *aux;  // generic r2r: W_{8n'}^m
  int kind, r2r, sign;
  int nfft, twstep;  // W_nfft^m = tw[m * twstep]
  int nrad;
  int rad[24];
  int nin, nout, nlog;  // line lengths (elements) in / out, logical length
  int ls;               // shared-memory line stride (complex slots)
  int TB, nfl;          // data lines per CTA, FFT lines per data line (1 or 2)
  int ntile, dt, dother;
  long long iL, it, io, oL, ot, oo;
  int load_Lmajor, store_Lmajor;
  int deriv, dg, dmid;
  int r2r_np, r2r_a2, r2r_b2, r2r_sin, r2r_halffirst, r2r_halflast;
  int in_complex, out_complex;
  // Bluestein engine: convolution length bM (power of two), its radix plan, and its tables
  // [W_bM^k, k < bM][chirp W_m, m < nfft][transform of the forward chirp kernel][of the backward]
  int bM, bnrad;
  int brad[12];
  const void *baux;
};

// B selects the Bluestein engine's convolution FFT (length bM, its own twiddle table).
template <class O, bool B = false>
__device__ __forceinline__ typename O::C twid(const KParams &p, int m, int sign) {
  typename O::C w = B ? O::tw(reinterpret_cast<const typename O::T *>(p.baux), m)
                      : O::tw(reinterpret_cast<const typename O::T *>(p.tw), m * p.twstep);
  return sign < 0 ? w : O::conj(w);
}

// DFT of radix R in registers, sign -1 forward.  Odd R uses the twiddle table for W_R^q.
template <class O, int R, bool B = false>
__device__ __forceinline__ void dft_reg(typename O::C *v, int sign, const KParams &p) {
  const int nf = B ? p.bM : p.nfft;
  using C = typename O::C;
  if (R == 2) {
    C a = v[0], b = v[1];
    v[0] = O::add(a, b);
    v[1] = O::sub(a, b);
  } else if (R == 4) {
    C t0 = O::add(v[0], v[2]), t1 = O::sub(v[0], v[2]);
    C t2 = O::add(v[1], v[3]), t3 = O::sub(v[1], v[3]);
    t3 = sign < 0 ? O::mulmi(t3) : O::muli(t3);
    v[0] = O::add(t0, t2);
    v[2] = O::sub(t0, t2);
    v[1] = O::add(t1, t3);
    v[3] = O::sub(t1, t3);
  } else if (R == 8) {
    C e[4], o[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      e[k] = v[2 * k];
      o[k] = v[2 * k + 1];
    }
    dft_reg<O, 4, B>(e, sign, p);
    dft_reg<O, 4, B>(o, sign, p);
    // o[k] *= W8^k (forward), conj for backward
    C o1 = O::rsqrt2(sign < 0 ? O::add(o[1], O::mulmi(o[1])) : O::add(o[1], O::muli(o[1])));
    C o2 = sign < 0 ? O::mulmi(o[2]) : O::muli(o[2]);
    C o3 = O::rsqrt2(sign < 0 ? O::sub(O::mulmi(o[3]), o[3]) : O::sub(O::muli(o[3]), o[3]));
    v[0] = O::add(e[0], o[0]);
    v[4] = O::sub(e[0], o[0]);
    v[1] = O::add(e[1], o1);
    v[5] = O::sub(e[1], o1);
    v[2] = O::add(e[2], o2);
    v[6] = O::sub(e[2], o2);
    v[3] = O::add(e[3], o3);
    v[7] = O::sub(e[3], o3);
  } else if (R == 3) {
    dft3<O>(v, sign, twid<O, B>(p, nf / 3, -1));
  } else if (R == 5) {
    dft5<O>(v, sign, twid<O, B>(p, nf / 5, -1), twid<O, B>(p, 2 * (nf / 5), -1));
  } else {
    // other odd radix: direct sum with W_R^q from the table (index q * nfft/R)
    C out[R];
    const int unit = nf / R;
#pragma unroll
    for (int q = 0; q < R; q++) {
      C acc = v[0];
#pragma unroll
      for (int r = 1; r < R; r++) acc = O::add(acc, O::mul(v[r], twid<O, B>(p, ((r * q) % R) * unit, sign)));
      out[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < R; q++) v[q] = out[q];
  }
}

template <class O, int R, bool B = false>
__device__ __forceinline__ void bfly(const typename O::C *src, typename O::C *dst, int j, int T, int Ns,
                                     int sign, const KParams &p) {
  using C = typename O::C;
  C v[R];
  int k = j % Ns;
#pragma unroll
  for (int r = 0; r < R; r++) v[r] = src[j + r * T];
  if (Ns > 1) {
    int unit = k * ((B ? p.bM : p.nfft) / (Ns * R));
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = O::mul(v[r], twid<O, B>(p, r * unit, sign));
  }
  dft_reg<O, R, B>(v, sign, p);
  int base = (j - k) * R + k;
#pragma unroll
  for (int r = 0; r < R; r++) dst[base + r * Ns] = O::norm(v[r]);
}

template <class O, bool B = false>
__device__ void bfly_generic(const typename O::C *src, typename O::C *dst, int j, int T, int Ns, int R,
                             int sign, const KParams &p) {
  using C = typename O::C;
  const int nf = B ? p.bM : p.nfft;
  int k = j % Ns;
  int unit = k * (nf / (Ns * R));
  int runit = nf / R;
  int base = (j - k) * R + k;
  for (int q = 0; q < R; q++) {
    C acc = O::zero();
    for (int r = 0; r < R; r++) {
      C x = src[j + r * T];
      int m = r * unit + ((r * q) % R) * runit;  // twiddle * W_R^{rq}
      m %= nf;
      // (normalised at every term: a float-float sum of R terms left unnormalised collects the
      // rounding of every lo part, which cost 1e-12 relative at R = 2039)
      acc = O::norm(O::add(acc, O::mul(x, twid<O, B>(p, m, sign))));
    }
    dst[base + q * Ns] = O::norm(acc);
  }
}

// Runs the radix passes over `nlines` lines; returns the buffer index holding the result.
template <class O, bool B = false>
__device__ int fft_passes(const KParams &p, typename O::C *b0, typename O::C *b1, int nlines, int sign) {
  using C = typename O::C;
  int Ns = 1, cur = 0;
  const int nrad = B ? p.bnrad : p.nrad;
  for (int s = 0; s < nrad; s++) {
    const int R = B ? p.brad[s] : p.rad[s];
    const int T = (B ? p.bM : p.nfft) / R;
    const C *src = cur ? b1 : b0;
    C *dst = cur ? b0 : b1;
    const int total = nlines * T;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      int lt = idx / T, j = idx - lt * T;
      const C *sl = src + (size_t)lt * p.ls;
      C *dl = dst + (size_t)lt * p.ls;
      switch (R) {
        case 2: bfly<O, 2, B>(sl, dl, j, T, Ns, sign, p); break;
        case 3: bfly<O, 3, B>(sl, dl, j, T, Ns, sign, p); break;
        case 4: bfly<O, 4, B>(sl, dl, j, T, Ns, sign, p); break;
        case 5: bfly<O, 5, B>(sl, dl, j, T, Ns, sign, p); break;
        case 7: bfly<O, 7, B>(sl, dl, j, T, Ns, sign, p); break;
        case 8: bfly<O, 8, B>(sl, dl, j, T, Ns, sign, p); break;
        default: bfly_generic<O, B>(sl, dl, j, T, Ns, R, sign, p); break;
      }
    }
    __syncthreads();
    cur ^= 1;
    Ns *= R;
  }
  return cur;
}

// Element offsets of a line position in global memory (elements, not reals)
__device__ __forceinline__ long long in_off(const KParams &p, int lt, int j, int t0, int ioth) {
  return (long long)j * p.iL + (long long)(t0 + lt) * p.it + (long long)ioth * p.io;
}
__device__ __forceinline__ long long out_off(const KParams &p, int lt, int k, int t0, int ioth) {
  return (long long)k * p.oL + (long long)(t0 + lt) * p.ot + (long long)ioth * p.oo;
}

__device__ __forceinline__ void map_idx(int idx, int n, int nlines, int Lmajor, int &lt, int &j) {
  if (Lmajor) {
    lt = idx / n;
    j = idx - lt * n;
  } else {
    j = idx / nlines;
    lt = idx - j * nlines;
  }
}

template <class O>
__device__ __forceinline__ typename O::C apply_deriv(const KParams &p, typename O::C v, int k) {
  if (!p.deriv) return v;
  if (k == p.dmid) return O::zero();
  int kk = (k < p.dmid) ? k : k - p.dg;
  return O::iscale(v, kk);
}


// ------------------------------------------------------------------------------------------
// FFT engines.  An engine runs the complex FFT of length nfft on every line of the tile held in
// shared memory and returns which of the two buffers holds the result.
//
// GenericFFT: runtime mixed-radix plan (any length), ping-pong buffers, 256 threads.
struct GenericFFT {
  static constexpr int PADSH = 0;
  static constexpr bool FIXED = false;
  template <class O>
  __device__ static int run(const KParams &p, typename O::C *b0, typename O::C *b1, int nflines, int sign) {
    return fft_passes<O>(p, b0, b1, nflines, sign);
  }
};

// BluesteinFFT: the DFT of a length n with a large prime factor as a circular convolution of
// length bM (a power of two >= 2n-1), computed with two bM-point radix FFTs (Bluestein, 1970):
//   W_m = exp(s i pi m^2 / n)  (s = sign),  a_j = x_j W_j,  b_m = conj(W_m) for |m| < n,
//   X_k = W_k (a (*) b)_k,  k < n.
// The bM-point transforms of b for both signs are precomputed on the host (long double).
struct BluesteinFFT {
  static constexpr int PADSH = 0;
  static constexpr bool FIXED = false;
  template <class O>
  __device__ static int run(const KParams &p, typename O::C *b0, typename O::C *b1, int nlines, int sign) {
    using C = typename O::C;
    using T = typename O::T;
    const int n = p.nfft, M = p.bM;
    const T *tab = reinterpret_cast<const T *>(p.baux);
    const T *chirp = tab + M;
    const T *kern = tab + M + n + (sign < 0 ? 0 : M);
    int total = nlines * M;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      const int lt = idx / M, k = idx - lt * M;
      C v = O::zero();
      if (k < n) {
        const C w = O::tw(chirp, k);
        v = O::mul(b0[(size_t)lt * p.ls + k], sign < 0 ? w : O::conj(w));
      }
      b1[(size_t)lt * p.ls + k] = O::norm(v);
    }
    __syncthreads();
    int cur = fft_passes<O, true>(p, b1, b0, nlines, -1);
    C *A = cur ? b0 : b1, *other = cur ? b1 : b0;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      const int lt = idx / M, k = idx - lt * M;
      C *a = A + (size_t)lt * p.ls + k;
      *a = O::norm(O::mul(*a, O::tw(kern, k)));
    }
    __syncthreads();
    cur = fft_passes<O, true>(p, A, other, nlines, 1);
    C *c = cur ? other : A;
    const float inv = 1.0f / (float)M;  // exact: M is a power of two
    total = nlines * n;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      const int lt = idx / n, k = idx - lt * n;
      C *y = c + (size_t)lt * p.ls + k;
      const C w = O::tw(chirp, k);
      *y = O::norm(O::scalef(O::mul(*y, sign < 0 ? w : O::conj(w)), inv));
    }
    __syncthreads();
    return c == b0 ? 0 : 1;
  }
};

// Register engine for power-of-two lengths known at compile time: each line is processed by
// N/V threads holding V points in registers; pass s applies V/R radix-R butterflies per thread
// (twiddle multiply + DFT-R in registers) and one scatter through shared memory.
template <class O, int N, int V, int Ns, int R, int... Rest>
__device__ __forceinline__ void fixed_pass(const KParams &p, typename O::C *line, int j, bool active, int sign) {
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
        for (int r = 1; r < R; r++) v[b * R + r] = O::mul(v[b * R + r], twid<O>(p, r * k * (N / (Ns * R)), sign));
      }
      dft_reg<O, R>(&v[b * R], sign, p);
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
  if constexpr (sizeof...(Rest) > 0) fixed_pass<O, N, V, Ns * R, Rest...>(p, line, j, active, sign);
}

template <int N_, int V_, int... Rs>
struct FixedFFT {
  static constexpr int PADSH = 3;
  static constexpr bool FIXED = true;
  static constexpr int N = N_, V = V_, T = N_ / V_;
  template <class O>
  __device__ static int run(const KParams &p, typename O::C *b0, typename O::C *, int nflines, int sign) {
    const int l = threadIdx.x / T, j = threadIdx.x - l * T;
    fixed_pass<O, N, V, 1, Rs...>(p, b0 + (size_t)l * p.ls, j, l < nflines, sign);
    return 0;
  }
};

// ------------------------------------------------------------------------------------------
template <class O, class E>
__global__ void __launch_bounds__(256) k_stage(KParams p) {
  using C = typename O::C;
  using S = typename O::S;
  using G = typename O::G;
  constexpr int SH = E::PADSH;
  extern __shared__ __align__(128) unsigned char smem_raw[];  // (as declared in fast_stage.cuh)
  C *b0 = reinterpret_cast<C *>(smem_raw);
  C *b1 = b0 + (size_t)p.TB * p.nfl * p.ls;
  const int tile = blockIdx.x % p.ntile;
  const int ioth = blockIdx.x / p.ntile;
  const int t0 = tile * p.TB;
  const int nlines = min(p.TB, p.dt - t0);
  const G *gin = reinterpret_cast<const G *>(p.in);
  G *gout = reinterpret_cast<G *>(p.out);
  const int kind = p.kind;

  // ---------------- gather + pre-processing into b0 ----------------
  const bool direct = (kind == K_C2C_FWD || kind == K_C2C_BWD || kind == K_R2C ||
                       (kind == K_C2R && (p.nlog & 1)));
  {
    C *dstbuf = direct ? b0 : b1;
    const int total = nlines * p.nin;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      int lt, j;
      map_idx(idx, p.nin, nlines, p.load_Lmajor, lt, j);
      long long off = in_off(p, lt, j, t0, ioth);
      C *line = dstbuf + (size_t)lt * p.nfl * p.ls;
      if (p.in_complex) {
        line[pad<SH>(j)] = O::ldc(gin + 2 * off);
      } else if (kind == K_R2C && !(p.nlog & 1)) {
        S v = O::ld(gin + off);  // packed z[n] = x[2n] + i x[2n+1]
        if (j & 1) line[pad<SH>(j >> 1)].y = v;
        else line[pad<SH>(j >> 1)].x = v;
      } else {
        line[pad<SH>(j)] = O::mk(O::ld(gin + off), O::rzero());
      }
    }
  }
  __syncthreads();
  if (!direct) {
    if (kind == K_C2R) {  // even N: Z'[k] = (X[k]+conj X[M-k]) + i conj(W_N^k) (X[k]-conj X[M-k])
      const int M = p.nfft;
      const int total = nlines * M;
      for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int lt = idx / M, k = idx - lt * M;
        const C *X = b1 + (size_t)lt * p.ls;
        C a = X[pad<SH>(k)], b = X[pad<SH>(M - k)];
        if (k == 0) {
          a.y = O::rzero();
          b.y = O::rzero();
        }
        C bc = O::conj(b);
        C s = O::add(a, bc), d = O::sub(a, bc);
        C w = O::conj(O::tw(reinterpret_cast<const typename O::T *>(p.tw), k));  // W_N^-k
        b0[(size_t)lt * p.ls + pad<SH>(k)] = O::add(s, O::muli(O::mul(w, d)));
      }
    } else if (kind == K_R2R && p.r2r == REDFT00) {
      // even extension of length M = 2(n-1)
      const int n = p.nin, M = p.nfft;
      const int total = nlines * M;
      for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int lt = idx / M, j = idx - lt * M;
        const C *x = b1 + (size_t)lt * p.ls;
        b0[(size_t)lt * p.ls + pad<SH>(j)] = (j < n) ? x[pad<SH>(j)] : x[pad<SH>(M - j)];
      }
    } else if (kind == K_R2R && p.r2r == RODFT00) {
      // odd extension of length M = 2(n+1): [0, x0..x_{n-1}, 0, -x_{n-1}..-x0]
      const int n = p.nin, M = p.nfft;
      const int total = nlines * M;
      for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int lt = idx / M, j = idx - lt * M;
        const C *x = b1 + (size_t)lt * p.ls;
        C v;
        if (j == 0 || j == n + 1) v = O::zero();
        else if (j <= n) v = x[pad<SH>(j - 1)];
        else v = O::neg(x[pad<SH>(M - j - 1)]);
        b0[(size_t)lt * p.ls + pad<SH>(j)] = v;
      }
    } else if (kind == K_R2R) {
      // generic kinds II/III/IV: u_j = x_j exp(-i pi beta j / n'), zero padded to 2n'.
      // complex data: FFT line 2lt holds u(x), line 2lt+1 holds u(conj x).
      const int n = p.nin, M = p.nfft;
      const int total = nlines * M;
      const typename O::T *aux = reinterpret_cast<const typename O::T *>(p.aux);
      for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        int lt = idx / M, j = idx - lt * M;
        const C *x = b1 + (size_t)lt * p.nfl * p.ls;
        C u = O::zero(), uc = O::zero();
        if (j < n) {
          C xv = x[pad<SH>(j)];
          if ((p.r2r_halffirst && j == 0) || (p.r2r_halflast && j == n - 1)) xv = O::half(xv);
          C w = O::tw(aux, 2 * p.r2r_b2 * j);
          u = O::mul(xv, w);
          uc = O::mul(O::conj(xv), w);
        }
        C *fl = b0 + (size_t)lt * p.nfl * p.ls;
        fl[pad<SH>(j)] = u;
        if (p.nfl == 2) fl[p.ls + pad<SH>(j)] = uc;
      }
    }
    __syncthreads();
  } else if (kind == K_C2R) {
    // odd N: Hermitian extension X[N-k] = conj X[k], imag of DC ignored
    const int N = p.nlog, h = (N + 1) / 2;
    const int total = nlines * N;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      int lt = idx / N, k = idx - lt * N;
      C *X = b0 + (size_t)lt * p.ls;
      if (k == 0) X[0].y = O::rzero();
      else if (k >= h) X[pad<SH>(k)] = O::conj(X[pad<SH>(N - k)]);
    }
    __syncthreads();
  }

  // ---------------- FFT ----------------
  const int cur = E::template run<O>(p, b0, b1, nlines * p.nfl, p.sign);
  const C *res = cur ? b1 : b0;

  // ---------------- post-processing + scatter ----------------
  const int total = nlines * p.nout;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int lt, k;
    map_idx(idx, p.nout, nlines, p.store_Lmajor, lt, k);
    const C *Y = res + (size_t)lt * p.nfl * p.ls;
    long long off = out_off(p, lt, k, t0, ioth);
    if (kind == K_C2C_FWD || kind == K_C2C_BWD) {
      O::stc(gout + 2 * off, apply_deriv<O>(p, Y[pad<SH>(k)], k));
    } else if (kind == K_R2C) {
      C v;
      if (p.nlog & 1) {
        v = Y[pad<SH>(k)];
      } else {
        const int M = p.nfft;
        const int k1 = (k == M) ? 0 : k, k2 = (k == 0) ? 0 : M - k;
        C a = Y[pad<SH>(k1)], b = O::conj(Y[pad<SH>(k2)]);
        C w = O::tw(reinterpret_cast<const typename O::T *>(p.tw), k);  // W_N^k
        C s = O::add(a, b), d = O::sub(a, b);
        v = O::half(O::sub(s, O::muli(O::mul(w, d))));
      }
      O::stc(gout + 2 * off, apply_deriv<O>(p, v, k));
    } else if (kind == K_C2R) {
      S v;
      if (p.nlog & 1) v = Y[pad<SH>(k)].x;
      else v = (k & 1) ? Y[pad<SH>(k >> 1)].y : Y[pad<SH>(k >> 1)].x;
      O::st(gout + off, v);
    } else {  // K_R2R
      C v;
      if (p.r2r == REDFT00) {
        v = Y[pad<SH>(k)];
      } else if (p.r2r == RODFT00) {
        v = O::muli(Y[pad<SH>(k + 1)]);
      } else {
        const typename O::T *aux = reinterpret_cast<const typename O::T *>(p.aux);
        C w = O::tw(aux, p.r2r_a2 * (2 * k + p.r2r_b2));
        C sm = O::mul(w, Y[pad<SH>(k)]);  // S-_k
        C sp;
        if (p.nfl == 2) sp = O::conj(O::mul(w, Y[p.ls + pad<SH>(k)]));
        else sp = O::conj(sm);
        v = p.r2r_sin ? O::mulmi(O::sub(sp, sm)) : O::add(sp, sm);
      }
      if (p.out_complex) O::stc(gout + 2 * off, apply_deriv<O>(p, v, k));
      else O::st(gout + off, v.x);
    }
  }
}

// ------------------------------------------------------------------------------------------
// EMPTY stages: pure permutation (reorder_out / reorder_in, build/exec.C:1858-2266)
template <class E>
__global__ void __launch_bounds__(256) k_permute(const E *__restrict__ in, E *__restrict__ out, int da, int db,
                                                 long long ia, long long ib, long long ic, long long oa,
                                                 long long ob, long long oc, int ta, int tb) {
  // a = input-fastest dim, b = output-fastest dim, c = remaining dim (one CTA per 32x32 tile)
  __shared__ E tile[32][33];
  const int bx = blockIdx.x % ta, by = (blockIdx.x / ta) % tb;
  const long long c = blockIdx.x / ((long long)ta * tb);
  const int a0 = bx * 32, b0 = by * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    int a = a0 + threadIdx.x, b = b0 + y;
    if (a < da && b < db) tile[y][threadIdx.x] = in[a * ia + b * ib + c * ic];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    int b = b0 + threadIdx.x, a = a0 + y;
    if (a < da && b < db) out[a * oa + b * ob + c * oc] = tile[threadIdx.x][y];
  }
}

// Standalone derivative on a complex field: storage-order traversal, multiply by i*k along
// logical dim idir (build/deriv.C:85-184 with GlobStart = 0).
template <class R>
__global__ void k_deriv(const R *in, R *out, long long n, int sd0, int sd1, int pos, int g, int mid) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (; q < n; q += stride) {
    long long c0 = q % sd0, r = q / sd0, c1 = r % sd1, c2 = r / sd1;
    int k = (int)(pos == 0 ? c0 : (pos == 1 ? c1 : c2));
    R x = in[2 * q], y = in[2 * q + 1];
    R rx, ry;
    if (k == mid) {
      rx = 0;
      ry = 0;
    } else {
      R kk = (R)((k < mid) ? k : k - g);
      rx = -kk * y;
      ry = kk * x;
    }
    out[2 * q] = rx;
    out[2 * q + 1] = ry;
  }
}

// ------------------------------------------------------------------------------------------
// Host side: twiddle tables W_N^k = exp(-2 pi i k / N), generated in long double and stored as
// double pairs (fmt 0), float pairs (fmt 1) or float-float pairs (fmt 2).
// bytes per table entry: format 0 double, 1 float, 2 float-float, 3 packed float-float in
// product form (pcw: (c, c), (-s, s) for the hi parts, then the lo parts)
static size_t entry_bytes(int fmt) { return fmt == 1 ? 8 : (fmt == 3 ? 32 : 16); }

size_t table_bytes(int N, int fmt) { return (size_t)N * entry_bytes(fmt); }

static const long double TWO_PI_L = 6.283185307179586476925286766559005768L;

// entry i of a table: the complex value c + i s in format fmt
static void put_value(unsigned char *host, size_t i, long double c, long double s, int fmt) {
  if (fmt == 0) {
    double v[2] = {(double)c, (double)s};
    memcpy(&host[i * 16], v, 16);
  } else if (fmt == 1) {
    float v[2] = {(float)c, (float)s};
    memcpy(&host[i * 8], v, 8);
  } else if (fmt == 2) {
    float ch = (float)c, sh = (float)s;
    float v[4] = {ch, (float)(c - (long double)ch), sh, (float)(s - (long double)sh)};
    memcpy(&host[i * 16], v, 16);
  } else {
    const float ch = (float)c, sh = (float)s;
    const float cl = (float)(c - (long double)ch), sl = (float)(s - (long double)sh);
    float v[8] = {ch, ch, -sh, sh, cl, cl, -sl, sl};
    memcpy(&host[i * 32], v, 32);
  }
}

// entry i of a table: W_M^m = exp(-2 pi i m / M) in format fmt
static void put_twiddle(unsigned char *host, size_t i, long long m, long long M, int fmt) {
  const long double a = TWO_PI_L * (long double)(m % M) / (long double)M;
  put_value(host, i, cosl(a), -sinl(a), fmt);
}

// Bluestein: convolution length (power of two >= 2n - 1)
static int blue_len(int n) {
  int M = 1;
  while (M < 2 * n - 1) M <<= 1;
  return M;
}

static int largest_prime_factor(int n) {
  int m = n, lp = 1;
  for (int f = 2; (long long)f * f <= m; f++)
    while (m % f == 0) {
      lp = f;
      m /= f;
    }
  return m > 1 ? std::max(lp, m) : lp;
}

size_t blue_table_bytes(int n, int fmt) { return (size_t)(3 * blue_len(n) + n) * entry_bytes(fmt); }

// In-place forward DFT (exp(-2 pi i jk/M)) of a power-of-two length, in long double.
static void ld_fft(std::vector<long double> &re, std::vector<long double> &im) {
  const size_t n = re.size();
  for (size_t i = 1, j = 0; i < n; i++) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      std::swap(re[i], re[j]);
      std::swap(im[i], im[j]);
    }
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    for (size_t j = 0; j < len / 2; j++) {
      const long double a = -TWO_PI_L * (long double)j / (long double)len, wr = cosl(a), wi = sinl(a);
      for (size_t i = 0; i < n; i += len) {
        const size_t u = i + j, v = i + j + len / 2;
        const long double xr = re[v] * wr - im[v] * wi, xi = re[v] * wi + im[v] * wr;
        re[v] = re[u] - xr;
        im[v] = im[u] - xi;
        re[u] += xr;
        im[u] += xi;
      }
    }
  }
}

// [W_M^k, k < M][W_m = exp(-i pi m^2 / n), m < n][FFT_M of b_m = conj(W_m)][FFT_M of b_m = W_m],
// b placed circularly (b_{M-m} = b_m, 0 < m < n).
void fill_blue_table(int n, int fmt, void *dst) {
  unsigned char *host = static_cast<unsigned char *>(dst);
  const int M = blue_len(n);
  for (int k = 0; k < M; k++) put_twiddle(host, k, k, M, fmt);
  std::vector<long double> wr(n), wi(n);
  for (int m = 0; m < n; m++) {
    const long long q = ((long long)m * m) % (2LL * n);  // exp(-i pi m^2 / n) = W_{2n}^{m^2}
    const long double a = TWO_PI_L * (long double)q / (long double)(2 * n);
    wr[m] = cosl(a);
    wi[m] = -sinl(a);
    put_value(host, (size_t)M + m, wr[m], wi[m], fmt);
  }
  for (int sgn = 0; sgn < 2; sgn++) {  // 0: b = conj(W) (forward), 1: b = W (backward)
    std::vector<long double> br(M, 0.0L), bi(M, 0.0L);
    for (int m = 0; m < n; m++) {
      const long double im = sgn == 0 ? -wi[m] : wi[m];
      br[m] = wr[m];
      bi[m] = im;
      if (m > 0) {
        br[M - m] = wr[m];
        bi[M - m] = im;
      }
    }
    ld_fft(br, bi);
    for (int k = 0; k < M; k++) put_value(host, (size_t)M + n + (size_t)sgn * M + k, br[k], bi[k], fmt);
  }
}

void fill_table(int N, int fmt, void *dst) {
  unsigned char *host = static_cast<unsigned char *>(dst);
  for (int k = 0; k < N; k++) put_twiddle(host, k, k, N, fmt);
}

size_t pass_table_bytes(int N, int fmt) {
  return (size_t)std::max(1, fast_pass_entries(N)) * entry_bytes(fmt);
}

// Pass I >= 1: entry (r-1) Ns + k holds W_{Ns R}^{r k}, r = 1 .. R-1, k < Ns.
void fill_pass_table(int N, int fmt, void *dst) {
  unsigned char *host = static_cast<unsigned char *>(dst);
  memset(host, 0, pass_table_bytes(N, fmt));
  const RadixList L = fast_radices(N);
  if (L.n <= 0) return;
  int ns = L.r[0];
  for (int i = 1; i < L.n; i++) {
    const int R = L.r[i], off = fast_pass_offset(N, i);
    for (int r = 1; r < R; r++)
      for (int k = 0; k < ns; k++)
        put_twiddle(host, (size_t)off + (size_t)(r - 1) * ns + k, (long long)r * k, (long long)ns * R, fmt);
    ns *= R;
  }
}

// Kept resident per device; the map owns device allocations made on first use of each length.
struct DeviceTables {
  std::mutex mu;
  // key: (N, format + 8 pass) format 0 = double, 1 = float, 2 = float-float, 3 = packed float-float
  std::map<std::pair<int, int>, void *> tabs;
  int *status = nullptr;  // device status word: nonzero after a kernel's bounded wait ran out
  int *ctrs = nullptr;    // kTileCounters tile counters of capped launches
  ~DeviceTables() {
    for (auto &kv : tabs) cudaFree(kv.second);
    if (status) cudaFree(status);
    if (ctrs) cudaFree(ctrs);
  }
  // pass = 1: the specialised kernels' per-pass twiddle rows of FFT length N; pass = 2: the
  // Bluestein engine's tables for length N
  const void *get(int N, int fmt, int *err, int pass = 0) {
    std::lock_guard<std::mutex> g(mu);
    auto key = std::make_pair(N, fmt + 8 * pass);
    auto it = tabs.find(key);
    if (it != tabs.end()) return it->second;
    size_t bytes = pass == 2 ? blue_table_bytes(N, fmt) : (pass ? pass_table_bytes(N, fmt) : table_bytes(N, fmt));
    std::vector<unsigned char> host(bytes);
    if (pass == 2) fill_blue_table(N, fmt, host.data());
    else if (pass) fill_pass_table(N, fmt, host.data());
    else fill_table(N, fmt, host.data());
    void *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) {
      *err = E_CUDA;
      return nullptr;
    }
    if (cudaMemcpy(d, host.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaFree(d);
      *err = E_CUDA;
      return nullptr;
    }
    tabs[key] = d;
    return d;
  }
};

DeviceTables *tables_create() {
  DeviceTables *t = new DeviceTables();
  if (cudaMalloc(&t->status, sizeof(int)) != cudaSuccess || cudaMemset(t->status, 0, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    if (t->status) cudaFree(t->status);
    t->status = nullptr;  // no status word: the kernels with bounded waits are not used
  }
  return t;
}
void tables_destroy(DeviceTables *t) { delete t; }
int *tile_counters(DeviceTables *t) {
  if (!t) return nullptr;
  std::lock_guard<std::mutex> g(t->mu);
  if (!t->ctrs && cudaMalloc(&t->ctrs, sizeof(int) * kTileCounters) != cudaSuccess) {
    cudaGetLastError();
    t->ctrs = nullptr;
  }
  return t->ctrs;
}

int device_status(DeviceTables *t, bool clear) {
  if (!t || !t->status) return 0;
  int v = 0;
  if (cudaMemcpy(&v, t->status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (clear && v && cudaMemset(t->status, 0, sizeof(int)) != cudaSuccess) return -1;
  return v;
}

// Radix plan of a length (8s first, then 4, 2, 3, 5, 7, larger primes); returns the count or -1
// when more than `cap` factors would be needed.
static int factorize(int n, int *rad, int cap) {
  int k = 0;
  auto push = [&](int f) {
    if (k < cap) rad[k] = f;
    k++;
  };
  while (n % 8 == 0) { push(8); n /= 8; }
  while (n % 4 == 0) { push(4); n /= 4; }
  while (n % 2 == 0) { push(2); n /= 2; }
  const int small[3] = {3, 5, 7};
  for (int f : small)
    while (n % f == 0) { push(f); n /= f; }
  for (int f = 11; (long long)f * f <= n; f += 2)
    while (n % f == 0) { push(f); n /= f; }
  if (n > 1) push(n);
  return k <= cap ? k : -1;
}

int max_line_len(int prec) { return prec == 8 ? 6144 : 12288; }

// FP32 split twiddles on the long lines (P3DFFT_GB300_FP32_SPLIT_TWIDDLES=0 turns them off)
static int g_fp32_split = -1;
bool fp32_split_twiddles() {
  if (g_fp32_split < 0) {
    const char *e = getenv("P3DFFT_GB300_FP32_SPLIT_TWIDDLES");
    g_fp32_split = (e && e[0] == '0') ? 0 : 1;
  }
  return g_fp32_split == 1;
}
void set_fp32_split_twiddles(bool on) { g_fp32_split = on ? 1 : 0; }

// FP32 stages whose tile is TB evenly spaced, contiguous lines in device memory load it by TMA
// (P3DFFT_GB300_FP32_TMA=0 turns it off)
static int g_fp32_tma = -1;
bool fp32_tma() {
  if (g_fp32_tma < 0) {
    const char *e = getenv("P3DFFT_GB300_FP32_TMA");
    g_fp32_tma = (e && e[0] == '0') ? 0 : 1;
  }
  return g_fp32_tma == 1;
}
void set_fp32_tma(bool on) { g_fp32_tma = on ? 1 : 0; }
// TMA stores of tile-dim-contiguous outputs with the TMA loads (P3DFFT_GB300_FP32_TMA_STORE=0 off)
static int g_fp32_tma_store = -1;
static bool fp32_tma_store() {
  if (g_fp32_tma_store < 0) {
    const char *e = getenv("P3DFFT_GB300_FP32_TMA_STORE");
    g_fp32_tma_store = (e && e[0] == '0') ? 0 : 1;
  }
  return g_fp32_tma_store == 1;
}
static std::atomic<int> g_tma_stall(0);
void inject_tma_stall() { g_tma_stall = 1; }

static PFN_cuTensorMapEncodeTiled_v12000 tma_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// Sets fa up for a TMA-staged load when the stage qualifies (FP32 C2C / R2C on a
// fast_tma_length, 16-byte aligned device memory and strides):
// - mode 1, lines contiguous (unit stride) and the tile's lines evenly spaced: either all lines
//   are (the other batch dim's stride is the tile dim's times its size; a partial last tile is
//   filled with zeros) or the tile dim is a multiple of the tile's lines;
// - mode 2 (C2C), the tile dim contiguous and a multiple of the tile's (even) line count.
static std::atomic<long long> g_tma_launches(0);
long long tma_launches() { return g_tma_launches.load(); }
static bool fast_tma_setup(FastArgs &fa, const void *in, void *out, DeviceTables *tabs) {
  FParams &q = fa.p;
  if (!fp32_tma() || !tabs || !tabs->status || (fa.kind != FK_C2C && fa.kind != FK_R2C) || !fast_tma_length(fa.n))
    return false;
  if (q.ffin || q.ffout || q.nlines <= 0 || reinterpret_cast<uintptr_t>(in) % 16) return false;
  const int TB = fast_tile_lines(fa.n);
  const long long esz = fa.kind == FK_R2C ? 4 : 8;  // R2C strides count reals, C2C complex points
  long long nout = (q.nlines + q.dt - 1) / q.dt;
  cuuint64_t dims[3];
  cuuint64_t strides[2];
  cuuint32_t box[3];
  int mode, d1;
  if (q.load_Lmajor && q.iL == 1) {  // lines contiguous
    long long n1, s1, s2;
    if (nout == 1 || q.io == q.it * q.dt) {  // every line evenly spaced
      n1 = q.nlines;
      s1 = q.it * esz;
      s2 = s1 * n1;
      nout = 1;
    } else if (q.dt % TB == 0 && q.nlines % q.dt == 0) {
      n1 = q.dt;
      s1 = q.it * esz;
      s2 = q.io * esz;
    } else {
      return false;
    }
    if (n1 > 0x7fffffffLL || s1 % 16 || s2 % 16 || s1 < 8 * fa.n) return false;
    const int fl = 2 * fa.n;
    dims[0] = (cuuint64_t)fl;
    dims[1] = (cuuint64_t)n1;
    dims[2] = (cuuint64_t)nout;
    strides[0] = (cuuint64_t)s1;
    strides[1] = (cuuint64_t)s2;
    box[0] = (cuuint32_t)(fl <= 256 ? fl : 256);
    box[1] = (cuuint32_t)TB;
    box[2] = 1u;
    mode = 1;
    d1 = (int)n1;
  } else if (!q.load_Lmajor && q.it == 1 && fa.kind == FK_C2C && TB % 2 == 0 && q.dt % TB == 0 &&
             q.nlines % q.dt == 0) {
    // tile dim contiguous (C2C): rows of TB points along the tile dim (an even count, so that a
    // row is a multiple of 16 bytes and starts on one), one row per point of the lines
    const long long s1 = q.iL * 8, s2 = q.io * 8;
    if (s1 % 16 || s2 % 16 || q.dt > 0x3fffffffLL) return false;
    int boxr = fa.n < 256 ? fa.n : 256;
    while (fa.n % boxr) boxr--;
    dims[0] = (cuuint64_t)(2 * q.dt);
    dims[1] = (cuuint64_t)fa.n;
    dims[2] = (cuuint64_t)nout;
    strides[0] = (cuuint64_t)s1;
    strides[1] = (cuuint64_t)s2;
    box[0] = (cuuint32_t)(2 * TB);
    box[1] = (cuuint32_t)boxr;
    box[2] = 1u;
    mode = 2;
    d1 = q.dt;
  } else {
    return false;
  }
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, in) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type != cudaMemoryTypeDevice) return false;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tma_encoder();
  if (!enc) return false;
  cuuint32_t estr[3] = {1u, 1u, 1u};
  if (enc(&fa.tm[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(in), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  q.tma_mode = mode;
  // the output by TMA too (C2C whose output tile dim is contiguous: each tile leaves as rows of
  // TB points, full tiles only, 16-byte aligned rows)
  memset(&fa.tm[1], 0, sizeof(fa.tm[1]));
  q.tma_store = 0;
  if (fp32_tma_store() && fa.kind == FK_C2C && !q.store_Lmajor && q.ot == 1 && TB % 2 == 0 && q.dt % TB == 0 &&
      q.nlines % q.dt == 0 && reinterpret_cast<uintptr_t>(out) % 16 == 0 && (q.oL * 8) % 16 == 0 &&
      (q.oo * 8) % 16 == 0 && q.dt <= 0x3fffffff) {
    cudaPointerAttributes ao;
    const bool dev_out = cudaPointerGetAttributes(&ao, out) == cudaSuccess && ao.type == cudaMemoryTypeDevice;
    cudaGetLastError();
    int boxr = fa.n < 256 ? fa.n : 256;
    while (fa.n % boxr) boxr--;
    cuuint64_t od[3] = {(cuuint64_t)(2 * q.dt), (cuuint64_t)fa.n, (cuuint64_t)(q.nlines / q.dt)};
    cuuint64_t os[2] = {(cuuint64_t)(q.oL * 8), (cuuint64_t)(q.oo * 8)};
    cuuint32_t ob[3] = {(cuuint32_t)(2 * TB), (cuuint32_t)boxr, 1u};
    if (dev_out && enc(&fa.tm[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, out, od, os, ob, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                       CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
      q.tma_store = 1;
  }
  // a stall injected for the failure-path test: 16 bytes more than the copies deliver, so the
  // tile's wait runs out after 20 ms
  const bool stall = g_tma_stall.exchange(0) != 0;
  q.tma_extra = stall ? 16 : 0;
  q.tma_timeout_ns = stall ? 20000000LL : 1000000000LL;
  q.status = tabs->status;
  q.tma_d1 = d1;
  fa.tma = 1;
  g_tma_launches++;
  return true;
}

template <class O, class E>
static int launch_k(const KParams &p, size_t smem, int grid, int threads, cudaStream_t st) {
  static int configured_smem = 0;  // per instantiation
  if ((int)smem > configured_smem) {
    if (cudaFuncSetAttribute(k_stage<O, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return E_CUDA;
    configured_smem = (int)smem;
  }
  k_stage<O, E><<<grid, threads, smem, st>>>(p);
  return cudaGetLastError() == cudaSuccess ? E_OK : E_CUDA;
}

// Register engines available for a complex FFT length (power-of-two lengths 16..2048: 8 points
// per thread within k_stage's 256 threads)
static bool fixed_engine_len(int n) {
  switch (n) {
    case 16: case 32: case 64: case 128: case 256: case 512: case 1024: case 2048: return true;
    default: return false;
  }
}

template <class O>
static int launch_fixed(const KParams &p, size_t smem, int grid, int threads, cudaStream_t st) {
  switch (p.nfft) {
    case 16: return launch_k<O, FixedFFT<16, 4, 4, 4>>(p, smem, grid, threads, st);
    case 32: return launch_k<O, FixedFFT<32, 8, 8, 4>>(p, smem, grid, threads, st);
    case 64: return launch_k<O, FixedFFT<64, 8, 8, 8>>(p, smem, grid, threads, st);
    case 128: return launch_k<O, FixedFFT<128, 8, 8, 8, 2>>(p, smem, grid, threads, st);
    case 256: return launch_k<O, FixedFFT<256, 8, 8, 8, 4>>(p, smem, grid, threads, st);
    case 512: return launch_k<O, FixedFFT<512, 8, 8, 8, 8>>(p, smem, grid, threads, st);
    case 1024: return launch_k<O, FixedFFT<1024, 8, 8, 8, 8, 2>>(p, smem, grid, threads, st);
    case 2048: return launch_k<O, FixedFFT<2048, 8, 8, 8, 8, 4>>(p, smem, grid, threads, st);
    default: return E_UNSUPPORTED;
  }
}

template <class O>
static int launch_any(const KParams &p, bool fixed, bool blue, size_t smem, int grid, int threads, cudaStream_t st) {
  if (fixed) return launch_fixed<O>(p, smem, grid, threads, st);
  if (blue) return launch_k<O, BluesteinFFT>(p, smem, grid, threads, st);
  return launch_k<O, GenericFFT>(p, smem, grid, threads, st);
}

int launch_stage(const StageDesc &d, const void *in, void *out, int arith, cudaStream_t stream,
                 DeviceTables *tabs, int *kernels_launched, const void *tw_given, const void *aux_given,
                 TableNeed *tabs_out, FastArgs *fast_prep) {
  const int L = d.L;
  const int a = (L + 1) % 3, b = (L + 2) % 3;
  if (d.d1[a] != d.d2[a] || d.d1[b] != d.d2[b]) return E_BAD_ARG;
  KParams p;
  memset(&p, 0, sizeof(p));
  p.in = in;
  p.out = out;
  p.kind = d.kind;
  p.r2r = d.r2r;
  p.nin = d.d1[L];
  p.nout = d.d2[L];
  p.in_complex = d.dt1 == 2;
  p.out_complex = d.dt2 == 2;
  p.nfl = 1;
  p.sign = -1;
  int tabN = 0;
  switch (d.kind) {
    case K_C2C_FWD:
    case K_C2C_BWD:
      if (p.nin != p.nout) return E_BAD_ARG;
      p.nlog = p.nin;
      p.nfft = p.nin;
      tabN = p.nfft;
      p.twstep = 1;
      p.sign = d.kind == K_C2C_FWD ? -1 : 1;
      break;
    case K_R2C:
      p.nlog = p.nin;
      if (p.nout != p.nlog / 2 + 1) return E_BAD_ARG;
      if (p.nlog % 2 == 0 && p.nlog >= 2) {
        p.nfft = p.nlog / 2;
        tabN = p.nlog;
        p.twstep = 2;
      } else {
        p.nfft = p.nlog;
        tabN = p.nlog;
        p.twstep = 1;
      }
      break;
    case K_C2R:
      p.nlog = p.nout;
      if (p.nin != p.nlog / 2 + 1) return E_BAD_ARG;
      p.sign = 1;
      if (p.nlog % 2 == 0 && p.nlog >= 2) {
        p.nfft = p.nlog / 2;
        tabN = p.nlog;
        p.twstep = 2;
      } else {
        p.nfft = p.nlog;
        tabN = p.nlog;
        p.twstep = 1;
      }
      break;
    case K_R2R: {
      if (p.nin != p.nout) return E_BAD_ARG;
      int n = p.nin;
      p.nlog = n;
      if (d.r2r == REDFT00) {
        if (n < 2) return E_UNSUPPORTED;
        p.nfft = 2 * (n - 1);
      } else if (d.r2r == RODFT00) {
        p.nfft = 2 * (n + 1);
      } else {
        p.nfft = 2 * n;
        p.r2r_np = n;
        p.nfl = p.in_complex ? 2 : 1;
        switch (d.r2r) {
          case REDFT10: p.r2r_a2 = 1; p.r2r_b2 = 0; break;
          case REDFT01: p.r2r_a2 = 0; p.r2r_b2 = 1; p.r2r_halffirst = 1; break;
          case REDFT11: p.r2r_a2 = 1; p.r2r_b2 = 1; break;
          case RODFT10: p.r2r_a2 = 1; p.r2r_b2 = 2; p.r2r_sin = 1; break;
          case RODFT01: p.r2r_a2 = 2; p.r2r_b2 = 1; p.r2r_sin = 1; p.r2r_halflast = 1; break;
          case RODFT11: p.r2r_a2 = 1; p.r2r_b2 = 1; p.r2r_sin = 1; break;
          default: return E_BAD_ARG;
        }
      }
      tabN = p.nfft;
      p.twstep = 1;
      break;
    }
    default:
      return E_BAD_ARG;
  }
  if (p.nfft > max_line_len(d.prec)) return E_TOO_LARGE;
  p.nrad = factorize(p.nfft, p.rad, 24);
  if (p.nrad < 0) return E_UNSUPPORTED;

  // engine: the specialised kernels for C2C / even R2C / even C2R at their lengths, else the
  // register engine (powers of two) or the generic engine; complex vector I/O needs element-aligned
  // base pointers
  const uintptr_t align_need = (d.prec == 8) ? 16 : 8;
  const bool aligned = (((uintptr_t)in | (uintptr_t)out) % align_need) == 0;
  const bool even = (p.nlog % 2) == 0;
  // DCT-I / DST-I run as the FFT of the extended line (no fused derivative on that path)
  const bool r2r1 = d.kind == K_R2R && (d.r2r == REDFT00 || d.r2r == RODFT00) && !(d.deriv && d.dt2 == 2);
  // DCT / DST II-IV: FFT of the pre-twiddled, zero-padded line; it reads a third table (W_8n), so
  // it is not used where the caller supplies the tables or groups the launch
  const bool r2rg = d.kind == K_R2R && p.r2r_np > 0 && !(d.deriv && d.dt2 == 2) && !tw_given && !tabs_out && !fast_prep;
  const int fkind = r2r1 ? FK_R2R1 : (r2rg ? FK_R2RG : FK_C2C);
  const bool fast_kind = d.kind == K_C2C_FWD || d.kind == K_C2C_BWD || ((d.kind == K_R2C || d.kind == K_C2R) && even) || r2r1 || r2rg;
  const bool generic_only = getenv("P3DFFT_GB300_GENERIC_ONLY") != nullptr;
  const bool fast_ok = fast_kind && fast_supported(p.nfft, fkind) && aligned;
  if (d.engine == ENG_FAST && !fast_ok) return E_UNSUPPORTED;
  if (d.engine == ENG_FIXED && !fixed_engine_len(p.nfft)) return E_UNSUPPORTED;
  const bool use_fast = fast_ok && (d.engine == ENG_FAST || (d.engine == ENG_AUTO && !generic_only));
  // Bluestein for lengths with a prime factor above 16 (radix passes would spend O(p^2) work per
  // butterfly), when its tables come from the cache and its convolution fits in shared memory
  const int bM = blue_len(p.nfft);
  const bool use_blue = !use_fast && !tw_given && !tabs_out && !fast_prep && !generic_only &&
                        (d.engine == ENG_AUTO || d.engine == ENG_BLUESTEIN) && largest_prime_factor(p.nfft) > 16 &&
                        bM <= (d.prec == 4 ? 8192 : 4096);  // two buffers of bM: 128 KB
  if (d.engine == ENG_BLUESTEIN && !use_blue) return E_UNSUPPORTED;

  // FP32 specialised kernels on long lines: split (compensated) twiddle products, tables in
  // float-float pairs (format 2)
  const bool split = d.prec == 4 && use_fast && fp32_split_twiddles() && fast_split_length(p.nfft);
  // float-float tables: packed product form for the specialised kernels
  const int fmt = d.prec == 4 ? (split ? 2 : 1) : (arith == AR_DF ? (use_fast ? 3 : 2) : 0);
  if (tabs_out) {  // caller supplies the tables: report what is needed, launch nothing
    tabs_out->fmt = fmt;
    // the specialised float-float kernel of this length has float-float intermediate variants
    tabs_out->ff = (use_fast && d.prec == 8 && arith == AR_DF && !r2r1 && !r2rg && fast_ff_length(p.nfft) &&
                    (d.kind == K_C2C_FWD || d.kind == K_C2C_BWD || d.kind == K_R2C || d.kind == K_C2R)) ? 1 : 0;
    tabs_out->tabN = tabN;
    tabs_out->auxN = use_fast ? p.nfft : ((d.kind == K_R2R && p.r2r_np > 0) ? 8 * p.r2r_np : 0);
    tabs_out->aux_pass = use_fast ? 1 : 0;
    return E_OK;
  }
  int err = E_OK;
  if (tw_given) {
    p.tw = tw_given;
    p.aux = aux_given;
  } else {
    p.tw = tabs->get(tabN, fmt, &err);
    if (!p.tw) return err;
    if (use_fast) {
      p.aux = tabs->get(p.nfft, fmt, &err, 1);
      if (!p.aux) return err;
    } else if (d.kind == K_R2R && p.r2r_np > 0) {
      p.aux = tabs->get(8 * p.r2r_np, fmt, &err);
      if (!p.aux) return err;
    }
    if (use_blue) {
      p.bM = bM;
      p.bnrad = factorize(bM, p.brad, 12);
      p.baux = tabs->get(p.nfft, fmt, &err, 2);
      if (!p.baux || p.bnrad < 0) return err ? err : E_UNSUPPORTED;
    }
  }
  if (d.deriv && d.dt2 == 2) {
    p.deriv = 1;
    p.dg = (d.kind == K_R2C) ? (p.nout - 1) * 2 : p.nout;  // exec.C:240-243
    p.dmid = p.dg / 2;
  }
  // tile selection: t = batch dim along which consecutive lines are taken
  p.iL = d.s1[L];
  p.oL = d.s2[L];
  // t: with lines contiguous on input (L-major load) the tile dim only matters for the store, so
  // it is the batch dim with the smaller output stride (a t-major store when that dim is
  // contiguous); otherwise the batch dim with the smaller input stride (t-major load)
  int t = (d.s1[L] == 1) ? (d.s2[a] <= d.s2[b] ? a : b) : (d.s1[a] <= d.s1[b] ? a : b);
  if (d.talt) t = (t == a) ? b : a;
  const int o = (t == a) ? b : a;
  p.load_Lmajor = d.s1[L] == 1 ? 1 : 0;
  p.store_Lmajor = (d.s2[L] == 1) ? 1 : ((d.s2[t] == 1) ? 0 : 1);
  p.it = d.s1[t];
  p.io = d.s1[o];
  p.ot = d.s2[t];
  p.oo = d.s2[o];
  p.dt = d.d1[t];
  p.dother = d.d1[o];

  if (!aligned && (p.in_complex || p.out_complex)) return E_ALIGN;
  // float-float intermediates: only the specialised float-float C2C / R2C (out) / C2R (in) kernels
  if ((d.ffin || d.ffout) &&
      (!use_fast || arith != AR_DF || d.prec != 8 || r2r1 || r2rg || fast_prep || !fast_ff_length(p.nfft) ||
       (d.ffin && d.kind == K_R2C) ||
       (d.ffout && d.kind == K_C2R) || !(d.kind == K_C2C_FWD || d.kind == K_C2C_BWD || d.kind == K_R2C || d.kind == K_C2R)))
    return E_UNSUPPORTED;
  if (d.ffin || d.ffout) {  // the kernels index the scale arrays with 32-bit offsets
    long long span = 0;
    for (int i = 0; i < 3; i++) span += (long long)(d.d1[i] - 1) * std::max(d.mi[i], d.mo[i]);
    if (span >= 0x7fffffffLL) return E_UNSUPPORTED;
  }

  if (use_fast) {
    FastArgs fa;
    fa.split = split ? 1 : 0;
    fa.kind = (r2r1 || r2rg) ? fkind : ((d.kind == K_R2C) ? FK_R2C : (d.kind == K_C2R ? FK_C2R : FK_C2C));
    fa.n = p.nfft;
    FParams &q = fa.p;
    q.in = in;
    q.out = out;
    q.tw = p.tw;
    q.ptw = p.aux;
    q.iL = p.iL;
    q.it = p.it;
    q.io = p.io;
    q.oL = p.oL;
    q.ot = p.ot;
    q.oo = p.oo;
    q.dt = p.dt;
    const int TB = fast_tile_lines(p.nfft);
    const long long nreal = (long long)p.dt * p.dother;
    q.r2r_odd = (r2r1 && d.r2r == RODFT00) ? 1 : 0;
    q.pair = (r2r1 && !p.in_complex) ? 1 : 0;  // real lines, two per FFT line
    q.aux = nullptr;
    q.rg_n = q.rg_a2 = q.rg_b2 = q.rg_sin = q.rg_half0 = q.rg_half1 = q.rg_cplx = 0;
    if (r2rg) {
      q.aux = tabs->get(8 * p.r2r_np, fmt, &err);
      if (!q.aux) return err;
      q.rg_n = p.r2r_np;
      q.rg_a2 = p.r2r_a2;
      q.rg_b2 = p.r2r_b2;
      q.rg_sin = p.r2r_sin;
      q.rg_half0 = p.r2r_halffirst;
      q.rg_half1 = p.r2r_halflast;
      q.rg_cplx = p.in_complex ? 1 : 0;  // each part of a complex line is one FFT line
    }
    const long long nl = q.pair ? (nreal + 1) / 2 : (q.rg_cplx ? 2 * nreal : nreal);
    if (2 * nreal + TB > 0x7fffffffLL) return E_TOO_LARGE;
    q.nreal = (int)nreal;
    q.nlines = (int)nl;
    q.ntotal = (int)((nl + TB - 1) / TB);
    q.sign = p.sign;
    q.deriv = p.deriv;
    q.dg = p.dg;
    q.dmid = p.dmid;
    q.load_Lmajor = p.load_Lmajor;
    q.store_Lmajor = p.store_Lmajor;
    q.ffin = d.ffin;
    q.ffout = d.ffout;
    q.sin = d.sin;
    q.sout = d.sout;
    q.fi_j = d.mi[L];
    q.fi_t = d.mi[t];
    q.fi_o = d.mi[o];
    q.fo_t = d.mo[t];
    q.fo_o = d.mo[o];
    q.tma_timeout_ns = 0;
    q.tma_extra = 0;
    q.tma_d1 = 0;
    q.tma_mode = 0;
    q.tma_store = 0;
    q.status = nullptr;
    q.tile_ctr = d.max_ctas > 0 ? d.tile_ctr : nullptr;
    fa.tma = 0;
    if (fast_prep) {
      *fast_prep = fa;
      return E_OK;
    }
    if (q.ntotal == 0) return E_OK;
    // (a capped grid runs the persistent k_fast: the TMA kernels take one tile per CTA)
    if (d.prec == 4 && d.max_ctas <= 0) fast_tma_setup(fa, in, out, tabs);
    const int rc = launch_fast(d.prec, arith, fa, stream, nullptr, std::max(0, d.max_ctas));
    if (rc == E_OK && kernels_launched) (*kernels_launched)++;
    return rc;
  }
  if (fast_prep) return E_UNSUPPORTED;

  const size_t csz = (d.prec == 4) ? 8 : 16;
  // (k_stage runs at most 256 threads: two FFT lines of 2048 points per data line take the generic
  // engine unless the register engine is asked for explicitly)
  const bool fixed_fits = (p.nfft / (p.nfft == 16 ? 4 : 8)) * p.nfl <= 256;
  const bool fixed = !use_blue && fixed_engine_len(p.nfft) &&
                     (d.engine == ENG_FIXED || (d.engine == ENG_AUTO && !generic_only && fixed_fits));
  int slots = p.nfft;
  if (use_blue) slots = std::max(slots, bM);
  if (p.nin > slots) slots = p.nin;
  if (p.nout > slots) slots = p.nout;
  if (d.kind == K_C2R) slots = std::max(slots, p.nfft + 1);
  if (fixed) slots += slots / 8 + 1;  // padding slots of the register engine
  p.ls = slots;
  // the register engine needs the second buffer only for kinds with a pre-processing step
  const bool need_b1 = !fixed || d.kind == K_R2R || (d.kind == K_C2R && !(p.nlog & 1));
  const size_t per_line = (need_b1 ? 2 : 1) * (size_t)p.nfl * p.ls * csz;
  const size_t smem_cap = 110 * 1024;
  int TB, threads = 256;
  if (fixed) {
    const int T = p.nfft / (p.nfft == 16 ? 4 : 8);  // threads per FFT line
    TB = std::max(1, 256 / (T * p.nfl));
    while (TB > 1 && per_line * TB > smem_cap) TB /= 2;
    threads = TB * p.nfl * T;
    if (threads > 256 || threads < 32) return E_UNSUPPORTED;  // k_stage runs at most 256 threads
  } else if (!p.load_Lmajor || !p.store_Lmajor) {
    int esz = (int)((p.in_complex ? 2 : 1) * d.prec);
    TB = std::max(2, 64 / esz);
  } else {
    TB = std::max(1, 2048 / std::max(1, p.nfft));
  }
  while (!fixed && TB > 1 && per_line * TB > smem_cap) TB--;
  if (per_line * TB > 227 * 1024) return E_TOO_LARGE;
  if (!fixed && TB > p.dt) TB = p.dt;
  if (TB < 1) TB = 1;
  p.TB = TB;
  p.ntile = (p.dt + TB - 1) / TB;
  long long grid = (long long)p.ntile * p.dother;
  if (grid <= 0) return E_OK;
  if (grid > 0x7fffffffLL) return E_TOO_LARGE;
  size_t smem = per_line * TB;
  int rc;
  if (d.prec == 4) rc = launch_any<Native<float>>(p, fixed, use_blue, smem, (int)grid, threads, stream);
  else if (arith == AR_DF) rc = launch_any<DF>(p, fixed, use_blue, smem, (int)grid, threads, stream);
  else rc = launch_any<Native<double>>(p, fixed, use_blue, smem, (int)grid, threads, stream);
  if (rc == E_OK && kernels_launched) (*kernels_launched)++;
  return rc;
}

bool stage_cap_ok(const StageDesc &d, const void *in, void *out, int arith, DeviceTables *tabs) {
  StageDesc q = d;
  q.ffin = q.ffout = 0;  // (the query form takes none; fast_persist_ok checks the sides)
  q.sin = nullptr;
  q.sout = nullptr;
  FastArgs fa;
  if (launch_stage(q, in, out, arith, 0, tabs, nullptr, nullptr, nullptr, nullptr, &fa) != E_OK) return false;
  return fast_persist_ok(fa.kind, fa.n, d.ffin, d.ffout);
}

template <class E>
static int permute_t(const int d[3], const long long s1[3], const long long s2[3], const void *in, void *out,
                     cudaStream_t st) {
  int a = 0, b = 0;
  for (int i = 0; i < 3; i++) {
    if (s1[i] < s1[a]) a = i;
    if (s2[i] < s2[b]) b = i;
  }
  if (a == b) b = (a + 1) % 3;
  int c = 3 - a - b;
  int ta = (d[a] + 31) / 32, tb = (d[b] + 31) / 32;
  long long grid = (long long)ta * tb * d[c];
  if (grid <= 0) return E_OK;
  if (grid > 0x7fffffffLL) return E_TOO_LARGE;
  dim3 blk(32, 8);
  k_permute<E><<<(unsigned)grid, blk, 0, st>>>((const E *)in, (E *)out, d[a], d[b], s1[a], s1[b], s1[c], s2[a],
                                               s2[b], s2[c], ta, tb);
  return cudaGetLastError() == cudaSuccess ? E_OK : E_CUDA;
}

// ------------------------------------------------------------------------------------------
// Grouped launches
struct LaunchItem {
  int group;  // >= 0: member of group `group`; -1: launched alone
  StageLaunch st;
  std::vector<int> members;  // positions in the level's input list that this launch runs
};
struct LaunchGroupInfo {
  FastArgs fa;  // the first member's launch (kernel selection)
  int prec, arith;
  int count;  // members
  // the members' parameters [pfirst, pfirst + count) and (member, tile) items
  // [wfirst, wfirst + nwork) in the set's device arrays
  int pfirst = 0, wfirst = 0, nwork = 0;
};
struct LaunchSet {
  std::vector<std::vector<LaunchItem>> levels;
  std::vector<LaunchGroupInfo> groups;
  FParams *dev_params = nullptr;  // every group's members' parameters
  FWork *dev_work = nullptr;      // and (member, tile) items
  DeviceTables *tabs = nullptr;
};

// everything of a specialised launch but its buffers
static std::vector<long long> fast_key(const StageLaunch &st, const FastArgs &fa) {
  const FParams &q = fa.p;
  return {st.d.prec, st.d.prec == 8 ? st.arith : 0, fa.kind, fa.n, (long long)(uintptr_t)q.tw,
          (long long)(uintptr_t)q.ptw, q.iL, q.it, q.io, q.oL, q.ot, q.oo, q.dt, q.nlines, q.ntotal, q.sign,
          q.deriv, q.dg, q.dmid, q.load_Lmajor, q.store_Lmajor, q.r2r_odd, q.pair, q.nreal,
          (long long)(uintptr_t)q.aux, q.rg_n, q.rg_a2, q.rg_b2, q.rg_sin, q.rg_half0, q.rg_half1, q.rg_cplx};
}

// the kernel a specialised launch runs: arithmetic, kind, length, twiddle form
static std::vector<long long> kernel_key(const StageLaunch &st, const FastArgs &fa) {
  return {st.d.prec, st.d.prec == 8 ? st.arith : 0, fa.kind, fa.n, fa.split};
}

LaunchSet *launch_set_build(const std::vector<std::vector<StageLaunch>> &levels, DeviceTables *tabs, int *err,
                            bool work_list) {
  LaunchSet *S = new LaunchSet();
  S->tabs = tabs;
  std::vector<FParams> params;
  std::vector<FWork> work;
  for (const auto &lv : levels) {
    std::vector<LaunchItem> items;
    struct Member {
      FastArgs fa;
      StageLaunch st;
      int pos;
    };
    std::map<std::vector<long long>, std::vector<Member>> by_kernel;
    for (size_t pos = 0; pos < lv.size(); pos++) {
      const StageLaunch &st = lv[pos];
      FastArgs fa;
      int rc = E_UNSUPPORTED;
      if (st.d.kind != K_EMPTY)
        rc = launch_stage(st.d, st.src, st.dst, st.arith, 0, tabs, nullptr, nullptr, nullptr, nullptr, &fa);
      if (rc == E_OK && fa.p.ntotal > 0) {
        by_kernel[work_list ? kernel_key(st, fa) : fast_key(st, fa)].push_back({fa, st, (int)pos});
      } else if (rc == E_OK || rc == E_UNSUPPORTED) {
        items.push_back({-1, st, {(int)pos}});
      } else {
        *err = rc;
        delete S;
        return nullptr;
      }
    }
    for (auto &kv : by_kernel) {
      if (kv.second.size() == 1) {  // nothing to group
        items.push_back({-1, kv.second[0].st, {kv.second[0].pos}});
        continue;
      }
      LaunchGroupInfo g;
      g.fa = kv.second[0].fa;
      g.prec = (int)kv.first[0];
      g.arith = (int)kv.first[1];
      g.count = (int)kv.second.size();
      g.pfirst = (int)params.size();
      g.wfirst = (int)work.size();
      std::vector<int> members;
      for (auto &m : kv.second) {
        const int member = (int)params.size() - g.pfirst;
        params.push_back(m.fa.p);
        for (int t = 0; t < m.fa.p.ntotal; t++) work.push_back({member, t});
        members.push_back(m.pos);
      }
      g.nwork = (int)work.size() - g.wfirst;
      items.push_back({(int)S->groups.size(), kv.second[0].st, members});
      S->groups.push_back(g);
    }
    // largest launches first, so that concurrent streams finish together
    auto work = [&](const LaunchItem &it) -> double {
      const StageDesc &d = it.st.d;
      const double n = (double)d.d1[0] * d.d1[1] * d.d1[2];
      return it.group >= 0 ? n * S->groups[it.group].count : n;
    };
    std::stable_sort(items.begin(), items.end(),
                     [&](const LaunchItem &a, const LaunchItem &b) { return work(a) > work(b); });
    S->levels.push_back(items);
  }
  if (!params.empty()) {
    const size_t pb = params.size() * sizeof(FParams), wb = work.size() * sizeof(FWork);
    if (cudaMalloc(&S->dev_params, pb) != cudaSuccess || cudaMalloc(&S->dev_work, wb) != cudaSuccess ||
        cudaMemcpy(S->dev_params, params.data(), pb, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(S->dev_work, work.data(), wb, cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      launch_set_destroy(S);
      *err = E_CUDA;
      return nullptr;
    }
  }
  return S;
}

static int run_launch_item(LaunchSet *S, const LaunchItem &it, cudaStream_t st, int *kernels);

int launch_set_run(LaunchSet *S, cudaStream_t st, int *kernels) {
  for (size_t l = 0; l < S->levels.size(); l++)
    for (const LaunchItem &it : S->levels[l]) {
      const int rc = run_launch_item(S, it, st, kernels);
      if (rc != E_OK) return rc;
    }
  return E_OK;
}

int launch_set_levels(const LaunchSet *S) { return (int)S->levels.size(); }
int launch_set_items(const LaunchSet *S, int l) { return (int)S->levels[l].size(); }
int launch_set_run_item(LaunchSet *S, int l, int i, cudaStream_t st, int *kernels) {
  return run_launch_item(S, S->levels[l][i], st, kernels);
}
const std::vector<int> &launch_set_item_members(const LaunchSet *S, int l, int i) { return S->levels[l][i].members; }

static int run_launch_item(LaunchSet *S, const LaunchItem &it, cudaStream_t st, int *kernels) {
  if (it.group >= 0) {
    const LaunchGroupInfo &g = S->groups[it.group];
    FGroup fg;
    fg.plist = S->dev_params + g.pfirst;
    fg.work = S->dev_work + g.wfirst;
    fg.nwork = g.nwork;
    const long long ctas = g.nwork;  // one CTA per item
    if (ctas > 0x7fffffffLL) return E_TOO_LARGE;
    const int rc = launch_fast(g.prec, g.arith, g.fa, st, &fg, (int)ctas);
    if (rc == E_OK && kernels) (*kernels)++;
    return rc;
  }
  const StageDesc &d = it.st.d;
  if (d.kind == K_EMPTY) {
    const bool same = d.s1[0] == d.s2[0] && d.s1[1] == d.s2[1] && d.s1[2] == d.s2[2];
    const size_t bytes = (size_t)d.d1[0] * d.d1[1] * d.d1[2] * d.dt1 * d.prec;
    if (!same) return launch_permute(d.d1, d.s1, d.s2, d.dt1 * d.prec, it.st.src, it.st.dst, st, kernels);
    if (it.st.src == it.st.dst) return E_OK;
    return cudaMemcpyAsync(it.st.dst, it.st.src, bytes, cudaMemcpyDefault, st) == cudaSuccess ? E_OK : E_CUDA;
  }
  return launch_stage(d, it.st.src, it.st.dst, it.st.arith, st, S->tabs, kernels);
}

int launch_set_groups(const LaunchSet *S) { return (int)S->groups.size(); }

void launch_set_destroy(LaunchSet *S) {
  if (!S) return;
  if (S->dev_params) cudaFree(S->dev_params);
  if (S->dev_work) cudaFree(S->dev_work);
  delete S;
}

int preload_kernels() {
  int rc = fast_preload(4, AR_NATIVE);
  if (fast_preload(8, AR_DF) != E_OK) rc = E_CUDA;
  if (fast_preload(8, AR_NATIVE) != E_OK) rc = E_CUDA;
  return rc;
}

int launch_permute(const int d[3], const long long s1[3], const long long s2[3], int esize, const void *in,
                   void *out, cudaStream_t stream, int *kernels_launched) {
  int rc;
  switch (esize) {
    case 4: rc = permute_t<float>(d, s1, s2, in, out, stream); break;
    case 8: rc = permute_t<double>(d, s1, s2, in, out, stream); break;
    case 16: rc = permute_t<double2>(d, s1, s2, in, out, stream); break;
    default: return E_BAD_ARG;
  }
  if (rc == E_OK && kernels_launched) (*kernels_launched)++;
  return rc;
}

int launch_deriv(int prec, const int d[3], const long long s[3], int idir, int g, int ref_axis, const void *in,
                 void *out, cudaStream_t stream, int *kernels_launched) {
  // storage dims (fastest first) and the storage position of idir
  int order[3] = {0, 1, 2};
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (s[order[j]] < s[order[i]]) std::swap(order[i], order[j]);
  int pos = 0;
  for (int i = 0; i < 3; i++)
    if (order[i] == idir) pos = i;
  // deriv.C:89-93 takes ldir with MemOrder[ldir] == idir and uses it as the storage axis
  if (ref_axis) pos = order[idir];
  long long n = (long long)d[0] * d[1] * d[2];
  if (n == 0) return E_OK;
  int mid = g / 2;
  int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  if (prec == 8)
    k_deriv<double><<<blocks, 256, 0, stream>>>((const double *)in, (double *)out, n, d[order[0]], d[order[1]], pos, g, mid);
  else
    k_deriv<float><<<blocks, 256, 0, stream>>>((const float *)in, (float *)out, n, d[order[0]], d[order[1]], pos, g, mid);
  if (kernels_launched) (*kernels_launched)++;
  return cudaGetLastError() == cudaSuccess ? E_OK : E_CUDA;
}

}  // namespace p3d
