// Floor and fraction of a lattice coordinate from the bits of its FP64 value.
//
// The mixed form keeps vertex positions in FP64 and needs, per coordinate,
// floor(P), the fraction (float)(P - floor(P)) and floor(P + 0.5).  With FP64
// instructions (floor, subtract, two conversions) that is four FP64-pipe
// operations per axis, and this GPU's FP64 pipe takes 16 SM cycles per warp
// instruction.  The same results follow exactly from the IEEE-754 fields of P
// with 32-bit integer operations and one 32-bit conversion:
//   for 1 <= P < 2^20, P = m * 2^-s with m the 53-bit significand and
//   s = 52 - e in [33, 52];
//   floor(P) = m >> s, and the fraction is F * 2^-s with F = m mod 2^s;
//   P - floor(P) is exact in FP64 (Sterbenz), so its conversion to float is F
//   rounded to 24 significant bits, to nearest, ties to even: F's leading 32
//   bits with a sticky bit for the rest convert to the same float;
//   floor(P + 0.5) = floor(P) + (F >= 2^(s-1)): P + 0.5 is exact in FP64 for
//   these P, or rounds within [2^(e+1), 2^(e+1) + 0.5) when it crosses the
//   binade, which has the same floor.
// Outside [1, 2^20) (negative coordinates on a periodic axis, the first unit
// interval, coordinates beyond a million nodes, non-finite values) split()
// returns false and the caller takes the FP64 instructions.  Host and device compile the same code; a CPU test
// compares it bit for bit with the FP64 operations.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define HC_POS_HD __host__ __device__ __forceinline__
#else
#define HC_POS_HD inline
#endif

namespace hcpos {

HC_POS_HD void double_words(double x, uint32_t& hi, uint32_t& lo) {
#ifdef __CUDA_ARCH__
  hi = (uint32_t)__double2hiint(x);
  lo = (uint32_t)__double2loint(x);
#else
  uint64_t b;
  memcpy(&b, &x, sizeof b);
  hi = (uint32_t)(b >> 32);
  lo = (uint32_t)b;
#endif
}

HC_POS_HD float float_from_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, sizeof f);
  return f;
#endif
}

HC_POS_HD int leading_zeros32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __clz((int)x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}

// (hi:lo) >> n for 0 <= n <= 31, low 32 bits
HC_POS_HD uint32_t shift_right_pair(uint32_t lo, uint32_t hi, int n) {
#ifdef __CUDA_ARCH__
  return __funnelshift_r(lo, hi, n);
#else
  return n == 0 ? lo : (lo >> n) | (hi << (32 - n));
#endif
}

HC_POS_HD float uint_to_float_rn(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __uint2float_rn(x);
#else
  return (float)x;  // round to nearest under the default rounding mode
#endif
}

// 2^k as a float, -126 <= k <= 127
HC_POS_HD float pow2f(int k) { return float_from_bits((uint32_t)(k + 127) << 23); }

// The fields of a coordinate 1 <= P < 2^20 (every lattice coordinate in
// practice): floor q, the fraction F * 2^-s with F = fh:fl (s = 33..52
// fraction bits, so fh holds the top s - 32 of them), and up = 1 when the
// fraction is at least 0.5.  Returns false for every other P.
struct FractionBits {
  int q, s, up;
  uint32_t fh, fl;
};
HC_POS_HD bool fraction_bits(double P, FractionBits& b) {
  uint32_t hi, lo;
  double_words(P, hi, lo);
  const int be = (int)(hi >> 20);  // sign bit and biased exponent
  if ((unsigned)(be - 1023) > 19u) return false;
  b.s = 1075 - be;                                  // fraction bits, 33..52
  const int t = b.s - 32;                           // fraction bits in the high word, 1..20
  const uint32_t mh = (hi & 0xFFFFFu) | 0x100000u;  // significand bits 32..52
  b.q = (int)(mh >> t);
  b.fh = mh & ((1u << t) - 1u);
  b.fl = lo;
  b.up = (int)((b.fh >> (t - 1)) & 1u);
  return true;
}

// The fraction rounded to float, to nearest, ties to even: F's leading 32
// bits (all of F when fh is zero) with a sticky bit for the rest.
HC_POS_HD float fraction_to_float(const FractionBits& b) {
  const int n = 32 - leading_zeros32(b.fh);  // bits of fh, 0..20
  uint32_t top = shift_right_pair(b.fl, b.fh, n);
  if (b.fl & ((1u << n) - 1u)) top |= 1u;
  return uint_to_float_rn(top) * pow2f(n - b.s);
}

// For 1 <= P < 2^20: q = floor(P), fr = (float)(P - floor(P)) rounded as the
// FP64 conversion rounds it, up = 1 when P - floor(P) >= 0.5 (so that
// floor(P + 0.5) = q + up).  Returns false, leaving the outputs unset, for
// every other P.
HC_POS_HD bool split(double P, int& q, float& fr, int& up) {
  FractionBits b;
  if (!fraction_bits(P, b)) return false;
  q = b.q;
  up = b.up;
  fr = fraction_to_float(b);
  return true;
}

// The two linear weights of the mixed form's stencil along one axis, for
// 1 <= P < 2^20: w1 = (float)(P - floor(P)) and w0 = 1 - w1, except when the
// fraction rounds to 1: w0 is then the rounded exact complement
// 1 - (P - floor(P)) = (2^s - F) * 2^-s, not zero (2^s - F < 2^(s-24) then
// fits 32 bits, and is -fl modulo 2^32 since s >= 32).  Returns false for
// every other P.
HC_POS_HD bool split_weights(double P, int& q, float& w0, float& w1) {
  FractionBits b;
  if (!fraction_bits(P, b)) return false;
  q = b.q;
  w1 = fraction_to_float(b);
  const uint32_t g = 0u - b.fl;
  w0 = w1 == 1.0f ? uint_to_float_rn(g) * pow2f(-b.s) : 1.0f - w1;
  return true;
}

// floor(P + 0.5) as a 64-bit integer, exactly as the FP64 expression gives it.
HC_POS_HD long long nearest(double P) {
  int q, up;
  float fr;
  if (split(P, q, fr, up)) return (long long)q + up;
  return (long long)floor(P + 0.5);
}

}  // namespace hcpos
