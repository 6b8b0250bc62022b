// Float-float ("double-float") arithmetic on the FP32 pipe, used for FP64 data on GB300 where
// native DFMA issues at under 2 instructions per SM per clock versus ~128 for FFMA.
//
// A value is hi + lo with |lo| <= ulp(hi)/2 after normalisation, giving a ~48-bit significand.
// The error-free transformations are the classical ones (Knuth TwoSum, Dekker/FMA TwoProd,
// FastTwoSum); no CUDA math-library routine is involved.
//
// Conversions to and from IEEE double use integer bit manipulation only, so that no
// instruction is issued to the FP64 pipe.  Supported magnitude range: 2^-100 <= |x| < 2^126
// (values below are flushed to zero, values above saturate to infinity).
#pragma once
#include <cstdint>

namespace p3d {

struct __align__(8) ff {
  float hi, lo;
};
struct __align__(16) cff {
  ff x, y;
};

// 1/sqrt(2) = FF_RSQRT2_HI + FF_RSQRT2_LO
#define FF_RSQRT2_HI __int_as_float(0x3f3504f3)
#define FF_RSQRT2_LO __int_as_float(0x324fe77a)

__device__ __forceinline__ ff ff_fast2sum(float s, float e) {
  float h = s + e;
  return ff{h, e - (h - s)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  return ff_fast2sum(s, e);
}
// Unnormalised sum: the hi parts are added exactly (TwoSum), the rounding error and both lo parts
// collect in lo.  Used inside a butterfly; ff_norm restores |lo| <= ulp(hi)/2 afterwards.
__device__ __forceinline__ ff ff_add_nn(ff a, ff b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  return ff{s, e + (a.lo + b.lo)};
}
__device__ __forceinline__ ff ff_norm(ff a) { return ff_fast2sum(a.hi, a.lo); }
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_half(ff a) { return ff{a.hi * 0.5f, a.lo * 0.5f}; }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  float p = a.hi * b.hi;
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ff_fast2sum(p, e);
}
__device__ __forceinline__ ff ff_mul_const(ff a, float chi, float clo) { return ff_mul(a, ff{chi, clo}); }
__device__ __forceinline__ ff ff_mul_int(ff a, int k) {
  float kf = (float)k;  // exact for |k| < 2^24
  float p = a.hi * kf;
  float e = __fmaf_rn(a.hi, kf, -p);
  e = __fmaf_rn(a.lo, kf, e);
  return ff_fast2sum(p, e);
}
// a.x*b.x - a.y*b.y (+i ...) with one TwoSum per component
__device__ __forceinline__ cff cff_mul(cff a, cff b) {
  cff r;
  {
    float p1 = a.x.hi * b.x.hi, e1 = __fmaf_rn(a.x.hi, b.x.hi, -p1);
    float p2 = -a.y.hi * b.y.hi, e2 = __fmaf_rn(-a.y.hi, b.y.hi, -p2);
    float s = p1 + p2, bb = s - p1, e3 = (p1 - (s - bb)) + (p2 - bb);
    float lo = (e1 + e2) + e3;
    lo = __fmaf_rn(a.x.hi, b.x.lo, lo);
    lo = __fmaf_rn(a.x.lo, b.x.hi, lo);
    lo = __fmaf_rn(-a.y.hi, b.y.lo, lo);
    lo = __fmaf_rn(-a.y.lo, b.y.hi, lo);
    r.x = ff_fast2sum(s, lo);
  }
  {
    float p1 = a.x.hi * b.y.hi, e1 = __fmaf_rn(a.x.hi, b.y.hi, -p1);
    float p2 = a.y.hi * b.x.hi, e2 = __fmaf_rn(a.y.hi, b.x.hi, -p2);
    float s = p1 + p2, bb = s - p1, e3 = (p1 - (s - bb)) + (p2 - bb);
    float lo = (e1 + e2) + e3;
    lo = __fmaf_rn(a.x.hi, b.y.lo, lo);
    lo = __fmaf_rn(a.x.lo, b.y.hi, lo);
    lo = __fmaf_rn(a.y.hi, b.x.lo, lo);
    lo = __fmaf_rn(a.y.lo, b.x.hi, lo);
    r.y = ff_fast2sum(s, lo);
  }
  return r;
}

// Unnormalised products for use inside a butterfly (the sums that follow do not need |lo| <=
// ulp(hi)/2; values are normalised before they are stored).
__device__ __forceinline__ cff cff_mul_nn(cff a, cff b) {
  cff r;
  {
    float p1 = a.x.hi * b.x.hi, e1 = __fmaf_rn(a.x.hi, b.x.hi, -p1);
    float p2 = -a.y.hi * b.y.hi, e2 = __fmaf_rn(-a.y.hi, b.y.hi, -p2);
    float s = p1 + p2, bb = s - p1, e3 = (p1 - (s - bb)) + (p2 - bb);
    float lo = (e1 + e2) + e3;
    lo = __fmaf_rn(a.x.hi, b.x.lo, lo);
    lo = __fmaf_rn(a.x.lo, b.x.hi, lo);
    lo = __fmaf_rn(-a.y.hi, b.y.lo, lo);
    lo = __fmaf_rn(-a.y.lo, b.y.hi, lo);
    r.x = ff{s, lo};
  }
  {
    float p1 = a.x.hi * b.y.hi, e1 = __fmaf_rn(a.x.hi, b.y.hi, -p1);
    float p2 = a.y.hi * b.x.hi, e2 = __fmaf_rn(a.y.hi, b.x.hi, -p2);
    float s = p1 + p2, bb = s - p1, e3 = (p1 - (s - bb)) + (p2 - bb);
    float lo = (e1 + e2) + e3;
    lo = __fmaf_rn(a.x.hi, b.y.lo, lo);
    lo = __fmaf_rn(a.x.lo, b.y.hi, lo);
    lo = __fmaf_rn(a.y.hi, b.x.lo, lo);
    lo = __fmaf_rn(a.y.lo, b.x.hi, lo);
    r.y = ff{s, lo};
  }
  return r;
}
__device__ __forceinline__ ff ff_mul_const_nn(ff a, float chi, float clo) {
  float p = a.hi * chi;
  float e = __fmaf_rn(a.hi, chi, -p);
  e = __fmaf_rn(a.hi, clo, e);
  e = __fmaf_rn(a.lo, chi, e);
  return ff{p, e};
}

// IEEE double bits -> float-float (truncating split of the 53-bit significand into 24 + 24 bits)
__device__ __forceinline__ ff ff_from_double_bits(long long bits) {
  const unsigned long long b = (unsigned long long)bits;
  const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
  const int E = (int)((b >> 52) & 0x7ff);
  const int e = E - 1023;
  if (e < -100) return ff{__int_as_float(sign), 0.f};
  if (E == 0x7ff && (b & 0xfffffffffffffull)) return ff{__int_as_float(sign | 0x7fc00000u), 0.f};  // NaN
  if (e > 127) return ff{__int_as_float(sign | 0x7f800000u), 0.f};
  const unsigned long long m = b & 0xfffffffffffffull;
  const unsigned int hib = sign | ((unsigned int)(e + 127) << 23) | (unsigned int)(m >> 29);
  const unsigned int r = (unsigned int)(m & 0x1fffffffu);  // 29 bits below hi, weight 2^(e-52)
  float lo = 0.f;
  if (r) {
    const int lz = __clz(r) - 3;  // leading zeros inside the 29-bit field
    const unsigned int nrm = r << lz;  // leading one at bit 28
    const int el = e - 24 - lz;        // exponent of that leading one
    if (el >= -126) lo = __int_as_float(sign | ((unsigned int)(el + 127) << 23) | ((nrm >> 5) & 0x7fffffu));
  }
  return ff{__int_as_float(hib), lo};
}

// Scaled conversions of the specialised stage kernels.  Each line of a tile is multiplied by
// 2^sc (an integer added to every exponent field) so that its largest value is near 2^20; values
// more than 2^94 below the line's maximum are flushed to zero.  Only integer and FP32 pipe
// instructions are used.
__device__ __forceinline__ int dbl_biased_exp(long long bits) { return (int)(((unsigned long long)bits >> 52) & 0x7ff); }

__device__ __forceinline__ ff ff_from_bits_scaled(long long bits, int sc) {
  const unsigned H = (unsigned)((unsigned long long)bits >> 32), Lw = (unsigned)bits;
  const unsigned sign = H & 0x80000000u;
  const int E0 = (int)((H >> 20) & 0x7ff);
  const int E = E0 + sc;  // scaled biased exponent
  if (E0 == 0 || E < 949) return ff{0.f, 0.f};
  const unsigned t = ((H & 0x000fffffu) | ((unsigned)E << 20)) - (896u << 20);
  const float hi = __uint_as_float(__funnelshift_l(Lw, t, 3) | sign);
  const float rf = __uint2float_rz(Lw & 0x1fffffffu);
  const float lo = rf * __uint_as_float((unsigned)(E - 948) << 23);
  return ff{hi, __uint_as_float(__float_as_uint(lo) ^ sign)};
}

// Non-finite inputs of a tile (exponent field 0x7ff): the tile's scale is taken from its finite
// values and these convert to the float infinity or NaN of the same sign.
__device__ __forceinline__ int dbl_biased_exp_finite(long long bits) {
  const int e = dbl_biased_exp(bits);
  return e == 0x7ff ? 0 : e;
}
__device__ __forceinline__ ff ff_from_bits_scaled_nf(long long bits, int sc) {
  const unsigned long long b = (unsigned long long)bits;
  if (((b >> 52) & 0x7ff) == 0x7ff) {
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const unsigned nan = (b & 0xfffffffffffffull) ? 0x00400000u : 0u;
    return ff{__uint_as_float(sign | 0x7f800000u | nan), 0.f};
  }
  return ff_from_bits_scaled(bits, sc);
}

// normalised float-float times 2^-sc -> IEEE double bits (round to nearest on the lo part);
// a float infinity or NaN in hi gives the double infinity or NaN
__device__ __forceinline__ long long ff_to_bits_scaled(ff v, int sc) {
  const unsigned uh = __float_as_uint(v.hi);
  const unsigned Ef = (uh >> 23) & 0xff;
  const unsigned sign = uh & 0x80000000u;
  if (Ef - 1u >= 254u) {  // zero, or infinity / NaN (one unsigned comparison for both)
    if (Ef == 0) return 0;
    return (long long)(((unsigned long long)sign << 32) | 0x7ff0000000000000ull |
                       ((uh & 0x7fffffu) ? 0x0008000000000000ull : 0ull));
  }
  const int E = (int)Ef + 896 - sc;
  if (E <= 0) return (long long)((unsigned long long)sign << 32);
  const unsigned H = sign | ((unsigned)E << 20) | ((uh & 0x7fffffu) >> 3);
  const unsigned L = uh << 29;
  const float kf = v.lo * __uint_as_float((306u - Ef) << 23);  // lo in units of ulp_double(hi)
  int k = __float2int_rn(kf);
  if (sign) k = -k;
  if ((uh & 0x7fffffu) == 0 && k < 0) k *= 2;  // sum lies in the binade below hi
  unsigned long long bits = ((unsigned long long)H << 32) | L;
  bits += (unsigned long long)(long long)k;
  return (long long)bits;
}

// float (normal or zero) bits -> double bits
__device__ __forceinline__ long long f_to_double_bits(float f) {
  unsigned int u = __float_as_uint(f);
  unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
  unsigned int E = (u >> 23) & 0xff;
  if (E == 0) return (long long)s;
  if (E == 0xff) return (long long)(s | 0x7ff0000000000000ull | ((unsigned long long)(u & 0x7fffff) << 29));
  return (long long)(s | ((unsigned long long)(E - 127 + 1023) << 52) | ((unsigned long long)(u & 0x7fffff) << 29));
}

// float-float -> IEEE double bits (hi + lo, truncated to 53 bits).  Requires a normalised pair.
__device__ __forceinline__ long long ff_to_double_bits(ff v) {
  const unsigned int uh = __float_as_uint(v.hi);
  const unsigned int Eh = (uh >> 23) & 0xff;
  if (Eh == 0 || Eh == 0xff) return f_to_double_bits(v.hi);
  const unsigned int ul = __float_as_uint(v.lo);
  const unsigned int El = (ul >> 23) & 0xff;
  // significand of hi in units of 2^(eh-52): (2^23 | mant) << 29
  long long S = (long long)((0x800000u | (uh & 0x7fffffu))) << 29;
  if (El != 0) {
    long long ml = (long long)(0x800000u | (ul & 0x7fffffu));
    int sh = (int)El - (int)Eh + 29;  // lo = ml * 2^(el-23); in units 2^(eh-52): shift el-eh+29
    long long add = sh >= 0 ? (sh < 40 ? (ml << sh) : 0) : (sh > -32 ? (ml >> (-sh)) : 0);
    if ((uh ^ ul) & 0x80000000u) S -= add;
    else S += add;
  }
  int eh = (int)Eh - 127;
  // renormalise to [2^52, 2^53)
  if (S >= (1ll << 53)) {
    S >>= 1;
    eh += 1;
  }
  while (S < (1ll << 52) && S > 0) {
    S <<= 1;
    eh -= 1;
  }
  const unsigned long long sign = (unsigned long long)(uh & 0x80000000u) << 32;
  return (long long)(sign | ((unsigned long long)(eh + 1023) << 52) | ((unsigned long long)S & 0xfffffffffffffull));
}

// ------------------------------------------------------------------------------------------
// Packed float-float complex values for the FP32x2 instructions of sm_100 and later
// (add/sub/mul/fma .f32x2: two FP32 operations per instruction issue).  A complex value keeps
// its real and imaginary parts side by side, hi = (re.hi, im.hi) and lo = (re.lo, im.lo), so the
// componentwise operations of an FFT (sums, differences, real scalings) issue once for both parts.
// The arithmetic of each lane is that of the scalar float-float operations above.
struct __align__(16) pcf {
  float2 hi, lo;
};
// A twiddle w = wx + i wy in product form: xh = (wx.hi, wx.hi), yh = (-wy.hi, wy.hi), and the same
// for the lo parts, so that a * w = a (wx, wx) + swap(a) (-wy, wy) lane by lane.
struct __align__(16) pcw {
  float2 xh, yh, xl, yl;
};

__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
  unsigned long long ua = *reinterpret_cast<const unsigned long long *>(&a);
  unsigned long long ub = *reinterpret_cast<const unsigned long long *>(&b);
  unsigned long long ud;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(ud) : "l"(ua), "l"(ub));
  return *reinterpret_cast<const float2 *>(&ud);
}
__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 f2swap(float2 a) { return make_float2(a.y, a.x); }
__device__ __forceinline__ float2 f2dup(float a) { return make_float2(a, a); }

// unnormalised sum / difference (TwoSum on the hi parts, as ff_add_nn)
__device__ __forceinline__ pcf pcf_add_nn(pcf a, pcf b) {
  const float2 s = f2add(a.hi, b.hi);
  const float2 bb = f2sub(s, a.hi);
  const float2 e = f2add(f2sub(a.hi, f2sub(s, bb)), f2sub(b.hi, bb));
  return pcf{s, f2add(e, f2add(a.lo, b.lo))};
}
__device__ __forceinline__ pcf pcf_sub_nn(pcf a, pcf b) {
  const float2 s = f2sub(a.hi, b.hi);
  const float2 bb = f2sub(s, a.hi);
  const float2 e = f2sub(f2sub(a.hi, f2sub(s, bb)), f2add(b.hi, bb));
  return pcf{s, f2add(e, f2sub(a.lo, b.lo))};
}
__device__ __forceinline__ pcf pcf_norm(pcf a) {
  const float2 h = f2add(a.hi, a.lo);
  return pcf{h, f2sub(a.lo, f2sub(h, a.hi))};
}
// a * w, unnormalised (the terms of cff_mul_nn, lane by lane)
__device__ __forceinline__ pcf pcf_mul_nn(pcf a, const pcw &w) {
  const float2 as = f2swap(a.hi), als = f2swap(a.lo);
  const float2 p = f2mul(a.hi, w.xh), q = f2mul(as, w.yh);
  const float2 e1 = f2fma(a.hi, w.xh, f2neg(p)), e2 = f2fma(as, w.yh, f2neg(q));
  const float2 s = f2add(p, q), bb = f2sub(s, p);
  const float2 e3 = f2add(f2sub(p, f2sub(s, bb)), f2sub(q, bb));
  float2 lo = f2add(f2add(e1, e2), e3);
  lo = f2fma(a.hi, w.xl, lo);
  lo = f2fma(a.lo, w.xh, lo);
  lo = f2fma(as, w.yl, lo);
  lo = f2fma(als, w.yh, lo);
  return pcf{s, lo};
}
// a * (c.hi + c.lo) for a real float-float c, unnormalised
__device__ __forceinline__ pcf pcf_rmul_nn(pcf a, float2 ch, float2 cl) {
  const float2 p = f2mul(a.hi, ch);
  float2 e = f2fma(a.hi, ch, f2neg(p));
  e = f2fma(a.hi, cl, e);
  e = f2fma(a.lo, ch, e);
  return pcf{p, e};
}

}  // namespace p3d
