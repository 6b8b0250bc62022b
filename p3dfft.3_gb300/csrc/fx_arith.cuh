// Fixed-point 64-bit arithmetic for FP64 data on GB300 (the FX arithmetic of the stage kernels).
//
// A tile of lines is converted from IEEE double to two's-complement int64 with one common scale
// 2^sc, chosen so that every value of the tile stays below 2^59 in magnitude through the whole
// transform (headroom of log2(length) + 4 bits).  Additions are then exact 64-bit integer
// additions; products with twiddle factors (stored as w * 2^61) use 31-bit limbs and 32x32->64
// multiply-accumulates, truncating about two units in the last place per product.  With ~50
// significant bits per value the stage error is ~1e-14 relative L2, and no instruction is
// issued to the FP64 pipe.  Conversions back to double round to nearest.
#pragma once
#include <cstdint>

namespace p3d {

struct __align__(16) cfx {
  long long x, y;
};
// twiddle entry w = (wr, wi) * 2^61, each split as h*2^31 + l with 0 <= l < 2^31
struct __align__(16) tfx {
  int rh, rl, ih, il;
};

__device__ __forceinline__ long long fx_mw(int a, int b) { return (long long)a * (long long)b; }

__device__ __forceinline__ void fx_split(long long v, int &h, int &l) {
  h = (int)(v >> 31);
  l = (int)(v & 0x7fffffffll);
}

// (a * w) / 2^61 for a complex a (|a| < 2^59) and twiddle w
__device__ __forceinline__ cfx fx_cmul(cfx a, tfx w) {
  int arh, arl, aih, ail;
  fx_split(a.x, arh, arl);
  fx_split(a.y, aih, ail);
  const long long tre = fx_mw(arh, w.rh) - fx_mw(aih, w.ih);
  const long long sre = fx_mw(arh, w.rl) + fx_mw(arl, w.rh) - fx_mw(aih, w.il) - fx_mw(ail, w.ih);
  const long long tim = fx_mw(arh, w.ih) + fx_mw(aih, w.rh);
  const long long sim = fx_mw(arh, w.il) + fx_mw(arl, w.ih) + fx_mw(aih, w.rl) + fx_mw(ail, w.rh);
  cfx r;
  r.x = 2 * tre + (sre >> 30);
  r.y = 2 * tim + (sim >> 30);
  return r;
}

// (a * c) / 2^61 for a real constant c = ch*2^31 + cl
__device__ __forceinline__ long long fx_rmul(long long a, int ch, int cl) {
  int ah, al;
  fx_split(a, ah, al);
  return 2 * fx_mw(ah, ch) + ((fx_mw(ah, cl) + fx_mw(al, ch)) >> 30);
}

// 2^61 / sqrt(2) rounded = 1630477228166597777, split into 31-bit limbs
#define FX_RSQRT2_H 759250124
#define FX_RSQRT2_L 2134625425

// IEEE double bits -> round(x * 2^sc)
__device__ __forceinline__ long long fx_from_bits(long long bits, int sc) {
  const unsigned long long u = (unsigned long long)bits;
  int E = (int)((u >> 52) & 0x7ff);
  unsigned long long m = u & 0xfffffffffffffull;
  if (E) m |= 1ull << 52;
  else E = 1;
  const int sh = E - 1075 + sc;
  long long v;
  if (sh >= 0) {
    v = sh < 11 ? (long long)(m << sh) : 0x3fffffffffffffffll;  // sh >= 11 cannot occur for in-range tiles
  } else {
    const int r = -sh;
    v = r >= 62 ? 0 : (long long)((m + (1ull << (r - 1))) >> r);
  }
  return (u >> 63) ? -v : v;
}

// round_to_double(v * 2^-sc) as IEEE bits
__device__ __forceinline__ long long fx_to_bits(long long v, int sc) {
  if (v == 0) return 0;
  const unsigned long long s = (unsigned long long)v & 0x8000000000000000ull;
  const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  const int lz = __clzll((long long)a);
  const unsigned long long r = a << lz;
  const unsigned long long m = (r >> 11) + ((r >> 10) & 1ull);  // may round up to 2^53
  const long long E = 1023 + (63 - lz) - sc;
  return (long long)(s | (((unsigned long long)(E - 1) << 52) + m));
}

// round_to_double(v * k * 2^-sc) as IEEE bits, |k| < 2^31 (the fused derivative's i*k factor)
__device__ __forceinline__ long long fx_to_bits_mul(long long v, int k, int sc) {
  if (v == 0 || k == 0) return 0;
  const unsigned long long s = ((unsigned long long)v ^ ((unsigned long long)(long long)k)) & 0x8000000000000000ull;
  const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  const unsigned long long b = (unsigned long long)(k < 0 ? -k : k);
  const unsigned long long lo = a * b, hi = __umul64hi(a, b);
  unsigned long long r;
  int top;  // bit index of the leading one in the 128-bit product
  if (hi) {
    const int lz = __clzll((long long)hi);
    r = (hi << lz) | (lo >> (64 - lz));
    top = 127 - lz;
  } else {
    const int lz = __clzll((long long)lo);
    r = lo << lz;
    top = 63 - lz;
  }
  const unsigned long long m = (r >> 11) + ((r >> 10) & 1ull);
  const long long E = 1023 + top - sc;
  return (long long)(s | (((unsigned long long)(E - 1) << 52) + m));
}

}  // namespace p3d
