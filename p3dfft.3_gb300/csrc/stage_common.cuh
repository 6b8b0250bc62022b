// Arithmetic policies shared by the stage kernels (generic engine in stage_kernels.cu, the
// specialised fast kernels in fast_stage.cuh).
//   Native<double>  FP64 data, DFMA arithmetic
//   Native<float>   FP32 data, FFMA arithmetic, twiddles rounded from long-double tables
//   DF              FP64 data, float-float arithmetic on the FP32 pipe (df_arith.cuh)
#pragma once
#include <cuda_runtime.h>

#include "df_arith.cuh"
#include "kernels.h"

namespace p3d {

// Loads / stores per thread that the specialised kernels keep in flight together (loop unroll
// of their global-memory I/O).  All of a thread's points for every arithmetic: with the packed
// FP32x2 float-float arithmetic those kernels are latency- rather than issue-bound as well.
#ifndef FAST_IO_UNROLL_NATIVE
#define FAST_IO_UNROLL_NATIVE 8
#endif
#ifndef FAST_IO_UNROLL_DF
#define FAST_IO_UNROLL_DF 8
#endif
#ifndef FAST_TW_POWERS_FP32
#define FAST_TW_POWERS_FP32 1
#endif

// ------------------------------------------------------------------------------------------
// Arithmetic policies
template <class R>
struct __align__(2 * sizeof(R)) cx {
  R x, y;
};

__device__ __forceinline__ cx<double> ldg_c(const cx<double> *p) {
  double2 v = __ldg(reinterpret_cast<const double2 *>(p));
  cx<double> r;
  r.x = v.x;
  r.y = v.y;
  return r;
}
__device__ __forceinline__ cx<float> ldg_c(const cx<float> *p) {
  float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  cx<float> r;
  r.x = v.x;
  r.y = v.y;
  return r;
}

template <class R>
struct Native {
  using G = R;       // global real type
  using S = R;       // shared-memory real type
  using C = cx<R>;   // working complex
  using T = cx<R>;   // twiddle-table entry
  static __device__ __forceinline__ C mk(S a, S b) { C c; c.x = a; c.y = b; return c; }
  static __device__ __forceinline__ C add(C a, C b) { return mk(a.x + b.x, a.y + b.y); }
  static __device__ __forceinline__ C sub(C a, C b) { return mk(a.x - b.x, a.y - b.y); }
  static __device__ __forceinline__ C mul(C a, C b) {
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
  }
  static __device__ __forceinline__ C muli(C a) { return mk(-a.y, a.x); }
  static __device__ __forceinline__ C mulmi(C a) { return mk(a.y, -a.x); }
  static __device__ __forceinline__ C conj(C a) { return mk(a.x, -a.y); }
  static __device__ __forceinline__ C half(C a) { return mk(a.x * R(0.5), a.y * R(0.5)); }
  static __device__ __forceinline__ C neg(C a) { return mk(-a.x, -a.y); }
  static __device__ __forceinline__ C rsqrt2(C a) {
    const R c = R(0.70710678118654752440084436210485);
    return mk(a.x * c, a.y * c);
  }
  static __device__ __forceinline__ C rmul(C a, S c) { return mk(a.x * c, a.y * c); }  // real scalar
  static __device__ __forceinline__ C scalef(C a, float f) { return mk(a.x * (R)f, a.y * (R)f); }  // power of 2
  static __device__ __forceinline__ C iscale(C a, int k) {  // a * (i*k)
    R kk = R(k);
    return mk(-kk * a.y, kk * a.x);
  }
  static __device__ __forceinline__ S rzero() { return R(0); }
  static __device__ __forceinline__ C zero() { return mk(R(0), R(0)); }
  static __device__ __forceinline__ S negs(S a) { return -a; }
  static __device__ __forceinline__ S halfs(S a) { return a * R(0.5); }
  static __device__ __forceinline__ S ld(const G *p) { return __ldg(p); }
  static __device__ __forceinline__ C ldc(const G *p) {
    cx<R> v = ldg_c(reinterpret_cast<const cx<R> *>(p));
    return mk(v.x, v.y);
  }
  static __device__ __forceinline__ void st(G *p, S v) { *p = v; }
  static __device__ __forceinline__ void stc(G *p, C v) {
    cx<R> w; w.x = v.x; w.y = v.y;
    *reinterpret_cast<cx<R> *>(p) = w;
  }
  static __device__ __forceinline__ C tw(const T *t, int k) {
    T v = ldg_c(t + k);
    return mk(v.x, v.y);
  }
  static __device__ __forceinline__ C norm(C a) { return a; }
  static __device__ __forceinline__ C tws(const T *t, int k) { return t[k]; }
  // twiddles in registers are plain complex values; real and imaginary parts
  using W = C;
  static __device__ __forceinline__ S re(C a) { return a.x; }
  static __device__ __forceinline__ S im(C a) { return a.y; }
  static __device__ __forceinline__ S wre(C w) { return w.x; }
  static __device__ __forceinline__ S wim(C w) { return w.y; }
  // register-level I/O of the specialised kernels (no tile scaling for native arithmetic)
  static constexpr bool SCALED = false;
  static constexpr int IO_UNROLL = FAST_IO_UNROLL_NATIVE;
  // FP32: build most pass twiddles as products of two table entries (fewer loads through L1,
  // the FP32 kernels' bottleneck; at most two roundings more per twiddle)
  static constexpr bool TW_POWERS = sizeof(R) == 4 && FAST_TW_POWERS_FP32;
  static constexpr bool TW_CHAIN = false;
  // product of two twiddles (twiddle powers formed in registers)
  static __device__ __forceinline__ C wmul(C a, C b) { return mul(a, b); }
  using RAW = cx<R>;
  static __device__ __forceinline__ RAW ldraw(const G *p) { return ldg_c(reinterpret_cast<const cx<R> *>(p)); }
  static __device__ __forceinline__ RAW ldraw2(const G *p0, const G *p1) {
    RAW r;
    r.x = __ldg(p0);
    r.y = __ldg(p1);
    return r;
  }
  static __device__ __forceinline__ RAW ldraw1(const G *p) {  // one real, imaginary part 0
    RAW r;
    r.x = __ldg(p);
    r.y = R(0);
    return r;
  }
  static __device__ __forceinline__ int rexp(RAW) { return 0; }
  static __device__ __forceinline__ C from_raw(RAW r, int) { return mk(r.x, r.y); }
  static __device__ __forceinline__ RAW to_raw(C v, int) {
    RAW r;
    r.x = v.x;
    r.y = v.y;
    return r;
  }
  static __device__ __forceinline__ void straw(G *p, RAW r) { *reinterpret_cast<cx<R> *>(p) = r; }
  static __device__ __forceinline__ void straw2(G *p0, G *p1, RAW r) {
    *p0 = r.x;
    *p1 = r.y;
  }
  static __device__ __forceinline__ void strawx(G *p, RAW r) { *p = r.x; }  // real part only
  static __device__ __forceinline__ RAW rneg(RAW r) {
    r.x = -r.x;
    r.y = -r.y;
    return r;
  }
  // float-float intermediate fields exist only for the float-float kernels (DFP)
  static __device__ __forceinline__ int rexp_ff(RAW, int) { return 0; }
  static __device__ __forceinline__ int rexp_ff_finite(RAW, int) { return 0; }
  static __device__ __forceinline__ C from_ff(RAW r, int) { return mk(r.x, r.y); }
  static __device__ __forceinline__ void stff(G *p, C v) { straw(p, to_raw(v, 0)); }
};

// FP32 data with split twiddles (the specialised kernels on long lines): each twiddle is the pair
// (hi, lo) of FP32 values whose sum is its long-double value to ~48 bits (table format 2), and a
// product a * w is formed as a * hi + (a * lo), the small term first, so the twiddle adds no
// rounding of its own beyond that of the product ("compensated" twiddle products).  CHAIN = false
// reads every pass twiddle W^r (r = 1 .. R-1) from the tables; CHAIN = true reads W^1 and forms
// W^r = W^(r-1) W^1 as float-float products, one at a time (two twiddles live, ~2^-44 relative
// after the six products of a radix-8 butterfly, far below the FP32 data's 2^-24), trading the
// table loads through the L1 data path, which bounds the FP32 kernels, for FMA-pipe work.
template <bool CHAIN>
struct NativeFS : Native<float> {
  using T = cff;
  using W = cff;
  using Native<float>::conj;
  using Native<float>::mul;
  static __device__ __forceinline__ W tw(const T *t, int k) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(t + k));
    return W{ff{v.x, v.y}, ff{v.z, v.w}};
  }
  static __device__ __forceinline__ W conj(const W &w) { return W{w.x, ff{-w.y.hi, -w.y.lo}}; }
  static __device__ __forceinline__ C mul(C a, const W &w) {
    const float cr = __fmaf_rn(a.x, w.x.lo, -a.y * w.y.lo);
    const float ci = __fmaf_rn(a.x, w.y.lo, a.y * w.x.lo);
    return mk(__fmaf_rn(a.x, w.x.hi, __fmaf_rn(-a.y, w.y.hi, cr)), __fmaf_rn(a.x, w.y.hi, __fmaf_rn(a.y, w.x.hi, ci)));
  }
  static __device__ __forceinline__ S wre(const W &w) { return w.x.hi; }
  static __device__ __forceinline__ S wim(const W &w) { return w.y.hi; }
  static constexpr bool TW_POWERS = false;
  static constexpr bool TW_CHAIN = CHAIN;
  static __device__ __forceinline__ W wmul(const W &a, const W &b) { return cff_mul(a, b); }
};

// float-float arithmetic for FP64 data (see df_arith.cuh), scalar form: the generic engines
// (k_stage); the specialised kernels use the packed form DFP below
struct DF {
  using G = double;
  using S = ff;
  using C = cff;
  using T = cff;
  static __device__ __forceinline__ C mk(S a, S b) { C c; c.x = a; c.y = b; return c; }
  // sums are left unnormalised inside a butterfly; norm() is applied before values are stored
  static __device__ __forceinline__ C add(C a, C b) { return mk(ff_add_nn(a.x, b.x), ff_add_nn(a.y, b.y)); }
  static __device__ __forceinline__ C sub(C a, C b) {
    return mk(ff_add_nn(a.x, ff_neg(b.x)), ff_add_nn(a.y, ff_neg(b.y)));
  }
  static __device__ __forceinline__ C norm(C a) { return mk(ff_norm(a.x), ff_norm(a.y)); }
  static __device__ __forceinline__ C mul(C a, C b) { return cff_mul_nn(a, b); }
  static __device__ __forceinline__ C muli(C a) { return mk(ff_neg(a.y), a.x); }
  static __device__ __forceinline__ C mulmi(C a) { return mk(a.y, ff_neg(a.x)); }
  static __device__ __forceinline__ C conj(C a) { return mk(a.x, ff_neg(a.y)); }
  static __device__ __forceinline__ C half(C a) { return mk(ff_half(a.x), ff_half(a.y)); }
  static __device__ __forceinline__ C neg(C a) { return mk(ff_neg(a.x), ff_neg(a.y)); }
  static __device__ __forceinline__ C rsqrt2(C a) {
    return mk(ff_mul_const_nn(a.x, FF_RSQRT2_HI, FF_RSQRT2_LO), ff_mul_const_nn(a.y, FF_RSQRT2_HI, FF_RSQRT2_LO));
  }
  static __device__ __forceinline__ C iscale(C a, int k) {
    return mk(ff_neg(ff_mul_int(a.y, k)), ff_mul_int(a.x, k));
  }
  static __device__ __forceinline__ C scalef(C a, float f) {  // by a power of two: exact
    return mk(ff{a.x.hi * f, a.x.lo * f}, ff{a.y.hi * f, a.y.lo * f});
  }
  static __device__ __forceinline__ C rmul(C a, S c) {  // real scalar, unnormalised
    return mk(ff_mul_const_nn(a.x, c.hi, c.lo), ff_mul_const_nn(a.y, c.hi, c.lo));
  }
  static __device__ __forceinline__ S rzero() { return ff{0.f, 0.f}; }
  static __device__ __forceinline__ C zero() { return mk(rzero(), rzero()); }
  static __device__ __forceinline__ S negs(S a) { return ff_neg(a); }
  static __device__ __forceinline__ S halfs(S a) { return ff_half(a); }
  static __device__ __forceinline__ S ld(const G *p) { return ff_from_double_bits(__ldg(reinterpret_cast<const long long *>(p))); }
  static __device__ __forceinline__ C ldc(const G *p) {
    longlong2 v = __ldg(reinterpret_cast<const longlong2 *>(p));
    return mk(ff_from_double_bits(v.x), ff_from_double_bits(v.y));
  }
  static __device__ __forceinline__ void st(G *p, S v) {
    *reinterpret_cast<long long *>(p) = ff_to_double_bits(ff_norm(v));
  }
  static __device__ __forceinline__ void stc(G *p, C v) {
    longlong2 w;
    w.x = ff_to_double_bits(ff_norm(v.x));
    w.y = ff_to_double_bits(ff_norm(v.y));
    *reinterpret_cast<longlong2 *>(p) = w;
  }
  static __device__ __forceinline__ C tws(const T *t, int k) { return t[k]; }
  static __device__ __forceinline__ C tw(const T *t, int k) {
    float4 v = __ldg(reinterpret_cast<const float4 *>(t + k));
    C c;
    c.x = ff{v.x, v.y};
    c.y = ff{v.z, v.w};
    return c;
  }
  using W = C;
  static __device__ __forceinline__ S re(C a) { return a.x; }
  static __device__ __forceinline__ S im(C a) { return a.y; }
  static __device__ __forceinline__ S wre(C w) { return w.x; }
  static __device__ __forceinline__ S wim(C w) { return w.y; }
};

// Float-float for FP64 data with packed FP32x2 arithmetic (the specialised kernels): the same
// operations as DF, the real and imaginary parts issued together (df_arith.cuh, pcf).  Twiddle
// tables hold pcw entries (table format 3).
struct DFP {
  using G = double;
  using S = ff;
  using C = pcf;
  using T = pcw;
  using W = pcw;
  static __device__ __forceinline__ C mk(S a, S b) { return C{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)}; }
  static __device__ __forceinline__ S re(C a) { return ff{a.hi.x, a.lo.x}; }
  static __device__ __forceinline__ S im(C a) { return ff{a.hi.y, a.lo.y}; }
  static __device__ __forceinline__ C add(C a, C b) { return pcf_add_nn(a, b); }
  static __device__ __forceinline__ C sub(C a, C b) { return pcf_sub_nn(a, b); }
  static __device__ __forceinline__ C norm(C a) { return pcf_norm(a); }
  static __device__ __forceinline__ C mul(C a, const W &w) { return pcf_mul_nn(a, w); }
  static __device__ __forceinline__ C muli(C a) {
    return C{make_float2(-a.hi.y, a.hi.x), make_float2(-a.lo.y, a.lo.x)};
  }
  static __device__ __forceinline__ C mulmi(C a) {
    return C{make_float2(a.hi.y, -a.hi.x), make_float2(a.lo.y, -a.lo.x)};
  }
  static __device__ __forceinline__ C conj(C a) { return C{make_float2(a.hi.x, -a.hi.y), make_float2(a.lo.x, -a.lo.y)}; }
  static __device__ __forceinline__ W conj(const W &w) { return W{w.xh, f2neg(w.yh), w.xl, f2neg(w.yl)}; }
  static __device__ __forceinline__ C half(C a) { return C{f2mul(a.hi, f2dup(0.5f)), f2mul(a.lo, f2dup(0.5f))}; }
  static __device__ __forceinline__ C neg(C a) { return C{f2neg(a.hi), f2neg(a.lo)}; }
  static __device__ __forceinline__ C rsqrt2(C a) {
    return pcf_rmul_nn(a, f2dup(FF_RSQRT2_HI), f2dup(FF_RSQRT2_LO));
  }
  static __device__ __forceinline__ C rmul(C a, S c) { return pcf_rmul_nn(a, f2dup(c.hi), f2dup(c.lo)); }
  static __device__ __forceinline__ C iscale(C a, int k) {  // a * (i k), normalised like ff_mul_int
    const float2 kk = make_float2(-(float)k, (float)k);
    const float2 as = f2swap(a.hi);
    const float2 p = f2mul(as, kk);
    float2 e = f2fma(as, kk, f2neg(p));
    e = f2fma(f2swap(a.lo), kk, e);
    return pcf_norm(C{p, e});
  }
  static __device__ __forceinline__ S rzero() { return ff{0.f, 0.f}; }
  static __device__ __forceinline__ C zero() { return C{make_float2(0.f, 0.f), make_float2(0.f, 0.f)}; }
  static __device__ __forceinline__ S negs(S a) { return ff_neg(a); }
  // twiddle re / im parts (the radix-3 and radix-5 butterflies' cos / sin constants)
  static __device__ __forceinline__ S wre(const W &w) { return ff{w.xh.x, w.xl.x}; }
  static __device__ __forceinline__ S wim(const W &w) { return ff{w.yh.y, w.yl.y}; }
  static __device__ __forceinline__ W tw(const T *t, int k) {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(t + k));
    const float4 b = __ldg(reinterpret_cast<const float4 *>(t + k) + 1);
    return W{make_float2(a.x, a.y), make_float2(a.z, a.w), make_float2(b.x, b.y), make_float2(b.z, b.w)};
  }
  static constexpr bool SCALED = true;
  static constexpr int IO_UNROLL = FAST_IO_UNROLL_DF;
  static constexpr bool TW_POWERS = false;
  static constexpr bool TW_CHAIN = false;
  using RAW = longlong2;
  static __device__ __forceinline__ RAW ldraw(const G *p) { return __ldg(reinterpret_cast<const longlong2 *>(p)); }
  static __device__ __forceinline__ RAW ldraw2(const G *p0, const G *p1) {
    RAW r;
    r.x = __ldg(reinterpret_cast<const long long *>(p0));
    r.y = __ldg(reinterpret_cast<const long long *>(p1));
    return r;
  }
  static __device__ __forceinline__ RAW ldraw1(const G *p) {  // one real, imaginary part 0
    RAW r;
    r.x = __ldg(reinterpret_cast<const long long *>(p));
    r.y = 0;
    return r;
  }
  static __device__ __forceinline__ int rexp(RAW r) { return max(dbl_biased_exp(r.x), dbl_biased_exp(r.y)); }
  static __device__ __forceinline__ C from_raw(RAW r, int sc) {
    return mk(ff_from_bits_scaled(r.x, sc), ff_from_bits_scaled(r.y, sc));
  }
  // tiles holding infinities or NaNs: the scale from the finite values, non-finite values kept
  static __device__ __forceinline__ int rexp_finite(RAW r) {
    return max(dbl_biased_exp_finite(r.x), dbl_biased_exp_finite(r.y));
  }
  static __device__ __forceinline__ C from_raw_nf(RAW r, int sc) {
    return mk(ff_from_bits_scaled_nf(r.x, sc), ff_from_bits_scaled_nf(r.y, sc));
  }
  static __device__ __forceinline__ RAW to_raw(C v, int sc) {
    const C n = pcf_norm(v);
    RAW r;
    r.x = ff_to_bits_scaled(ff{n.hi.x, n.lo.x}, sc);
    r.y = ff_to_bits_scaled(ff{n.hi.y, n.lo.y}, sc);
    return r;
  }
  static __device__ __forceinline__ void straw(G *p, RAW r) { *reinterpret_cast<longlong2 *>(p) = r; }
  static __device__ __forceinline__ void straw2(G *p0, G *p1, RAW r) {
    *reinterpret_cast<long long *>(p0) = r.x;
    *reinterpret_cast<long long *>(p1) = r.y;
  }
  static __device__ __forceinline__ void strawx(G *p, RAW r) { *reinterpret_cast<long long *>(p) = r.x; }
  static __device__ __forceinline__ RAW rneg(RAW r) {
    r.x ^= (long long)0x8000000000000000ull;
    r.y ^= (long long)0x8000000000000000ull;
    return r;
  }
  // Float-float intermediate fields: a complex element is its packed value (hi.x, hi.y, lo.x,
  // lo.y as four floats, the 16 bytes of a complex double) scaled by 2^sp, sp the scale of the
  // line that stored it.  rexp_ff gives the biased double exponent the value stands for (0 for
  // zero, 0x7ff for an infinity or NaN); from_ff rescales by 2^d, d = consumer scale - sp (the
  // clamp only matters for values far below every line maximum, which flush as in from_raw).
  static __device__ __forceinline__ unsigned ff_hexp(RAW r, int part) {
    const unsigned u = part ? (unsigned)((unsigned long long)r.x >> 32) : (unsigned)r.x;
    return (u >> 23) & 0xffu;
  }
  static __device__ __forceinline__ int rexp_ff(RAW r, int sp) {
    const unsigned fx = ff_hexp(r, 0), fy = ff_hexp(r, 1);
    const unsigned fm = fx > fy ? fx : fy;
    if (fm == 0xffu) return 0x7ff;
    return fm ? (int)fm + 896 - sp : 0;
  }
  static __device__ __forceinline__ int rexp_ff_finite(RAW r, int sp) {
    unsigned fx = ff_hexp(r, 0), fy = ff_hexp(r, 1);
    fx = fx == 0xffu ? 0u : fx;
    fy = fy == 0xffu ? 0u : fy;
    const unsigned fm = fx > fy ? fx : fy;
    return fm ? (int)fm + 896 - sp : 0;
  }
  static __device__ __forceinline__ C from_ff(RAW r, int d) {
    d = d < -126 ? -126 : (d > 127 ? 127 : d);
    const float2 f = f2dup(__int_as_float((d + 127) << 23));
    const C v = *reinterpret_cast<const C *>(&r);
    return C{f2mul(v.hi, f), f2mul(v.lo, f)};
  }
  static __device__ __forceinline__ void stff(G *p, C v) { *reinterpret_cast<C *>(p) = pcf_norm(v); }
};


// Shared-memory slot of line element i: one padding slot every 2^SH elements (SH = 0: none),
// which keeps the Stockham scatter of the register engines free of bank conflicts.
template <int SH>
__device__ __forceinline__ int pad(int i) {
  return SH ? i + (i >> SH) : i;
}

// In-register DFTs of radix 2, 4 and 8 (sign -1 forward, +1 backward); results normalised.
template <class O, int R>
__device__ __forceinline__ void dft_p2(typename O::C *v, int sign) {
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
  } else {  // R == 8
    C e[4], o[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      e[k] = v[2 * k];
      o[k] = v[2 * k + 1];
    }
    dft_p2<O, 4>(e, sign);
    dft_p2<O, 4>(o, sign);
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
  }
}

// Radix-3 and radix-5 DFTs (sign -1 forward, +1 backward).  The real constants cos/sin(2 pi q/R)
// come from twiddle-table entries w1 = W_R^1 = (cos 2pi/R, -sin 2pi/R) and w2 = W_R^2, so they
// carry the table's precision.  Pairing x_j with x_{R-j} leaves one real multiply per constant:
//   y_q = x0 + sum_j cos(2pi jq/R) (x_j + x_{R-j}) + sign*i sum_j sin(2pi jq/R) (x_j - x_{R-j}).
template <class O>
__device__ __forceinline__ void dft3(typename O::C *v, int sign, const typename O::W &w1) {
  using C = typename O::C;
  const C a = O::add(v[1], v[2]), b = O::sub(v[1], v[2]);
  const C m = O::sub(v[0], O::half(a));  // x0 + cos(2pi/3) a, cos(2pi/3) = -1/2
  C t = O::rmul(b, O::negs(O::wim(w1)));  // sin(2pi/3) b
  t = sign < 0 ? O::mulmi(t) : O::muli(t);
  v[0] = O::add(v[0], a);
  v[1] = O::add(m, t);
  v[2] = O::sub(m, t);
}

template <class O>
__device__ __forceinline__ void dft5(typename O::C *v, int sign, const typename O::W &w1, const typename O::W &w2) {
  using C = typename O::C;
  using S = typename O::S;
  const S c1 = O::wre(w1), s1 = O::negs(O::wim(w1)), c2 = O::wre(w2), s2 = O::negs(O::wim(w2));
  const C a1 = O::add(v[1], v[4]), b1 = O::sub(v[1], v[4]);
  const C a2 = O::add(v[2], v[3]), b2 = O::sub(v[2], v[3]);
  const C m1 = O::add(v[0], O::add(O::rmul(a1, c1), O::rmul(a2, c2)));
  const C m2 = O::add(v[0], O::add(O::rmul(a1, c2), O::rmul(a2, c1)));
  C t1 = O::add(O::rmul(b1, s1), O::rmul(b2, s2));
  C t2 = O::sub(O::rmul(b1, s2), O::rmul(b2, s1));
  t1 = sign < 0 ? O::mulmi(t1) : O::muli(t1);
  t2 = sign < 0 ? O::mulmi(t2) : O::muli(t2);
  v[0] = O::add(v[0], O::add(a1, a2));
  v[1] = O::add(m1, t1);
  v[4] = O::sub(m1, t1);
  v[2] = O::add(m2, t2);
  v[3] = O::sub(m2, t2);
}

}  // namespace p3d
