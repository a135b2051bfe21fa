// Checks hcpos::split, hcpos::split_weights and hcpos::nearest
// (hemocell_gb300/csrc/hc_posbits.h) against the FP64 operations they
// replace: floor(P), (float)(P - floor(P)), the stencil's complement weight
// and floor(P + 0.5), on random coordinates (the integer path over [1, 2^20),
// the FP64 fallback of nearest() elsewhere), on coordinates a few ulps from
// integers and half-integers, on fractions whose float rounding is an exact
// tie, just off one or rounds to one, and on the coordinates split() refuses.
// Prints "ok <cases>" or the first mismatch; exit status 0 only when all agree.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <limits>

#include "hc_posbits.h"

static uint64_t rng_state = 0x9E3779B97F4A7C15ull;
static uint64_t next_u64() {  // splitmix64
  uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double from_bits(uint64_t b) {
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
}
static uint32_t fbits(float f) {
  uint32_t b;
  memcpy(&b, &f, sizeof b);
  return b;
}

static long long cases = 0, rounded_to_one = 0;

static bool check(double P) {
  ++cases;
  int q = 0, up = 0;
  float fr = 0.f;
  const bool ok = hcpos::split(P, q, fr, up);
  const bool in_range = P >= 1.0 && P < 1048576.0;
  if (ok != in_range) {
    printf("split accepted=%d for P=%.17g\n", (int)ok, P);
    return false;
  }
  if (!std::isfinite(P)) return true;
  const double q0 = std::floor(P);
  const long long near = (long long)std::floor(P + 0.5);
  if (hcpos::nearest(P) != near) {
    printf("nearest %lld != %lld for P=%.17g\n", hcpos::nearest(P), near, P);
    return false;
  }
  if (!ok) return true;
  const float fr_ref = (float)(P - q0);
  if ((double)q != q0 || fbits(fr) != fbits(fr_ref) || (long long)q + up != near) {
    printf("mismatch P=%.17g: q %d/%.0f fr %.9g/%.9g (bits %08x/%08x) up %d near %lld\n", P, q, q0, (double)fr,
           (double)fr_ref, fbits(fr), fbits(fr_ref), up, near);
    return false;
  }
  // the stencil weights: w1 = the rounded fraction, w0 = 1 - w1 or, when the
  // fraction rounds to one, the rounded exact complement
  int qw = 0;
  float w0 = 0.f, w1 = 0.f;
  if (!hcpos::split_weights(P, qw, w0, w1)) {
    printf("split_weights refused P=%.17g\n", P);
    return false;
  }
  const float w0_ref = fr_ref == 1.0f ? (float)(1.0 - (P - q0)) : 1.0f - fr_ref;
  if (qw != q || fbits(w1) != fbits(fr_ref) || fbits(w0) != fbits(w0_ref)) {
    printf("weights P=%.17g: w0 %.9g/%.9g w1 %.9g/%.9g\n", P, (double)w0, (double)w0_ref, (double)w1,
           (double)fr_ref);
    return false;
  }
  if (fr_ref == 1.0f) ++rounded_to_one;
  return true;
}

int main() {
  // random coordinates, log-uniform over [2^-4, 2^32), both signs
  for (int k = 0; k < 3000000; ++k) {
    const int e = (int)(next_u64() % 36) - 4;
    const uint64_t mant = next_u64() & 0xFFFFFFFFFFFFFull;
    double P = from_bits(((uint64_t)(1023 + e) << 52) | mant);
    if (k % 7 == 0) P = -P;
    if (!check(P)) return 1;
  }
  // a few ulps around integers and half-integers, lattice-sized and large
  const double bases[] = {1.0,   2.0,    3.0,    7.0,     63.0,      64.0,       127.0,      255.0,
                          256.0, 1023.0, 4095.0, 65535.0, 1048575.0, 16777215.0, 16777216.0, 2147483647.0};
  for (double b : bases) {
    for (double off : {0.0, 0.5}) {
      double P = b + off;
      for (int k = 0; k < 64; ++k) P = std::nextafter(P, 0.0);
      for (int k = 0; k < 128; ++k) {
        if (!check(P)) return 1;
        P = std::nextafter(P, std::numeric_limits<double>::infinity());
      }
    }
  }
  // fractions at, just below and just above a 24-bit rounding tie, with the
  // leading fraction bit anywhere (both halves of the significand), and
  // all-ones fractions that round up to 1.0f
  for (int k = 0; k < 600000; ++k) {
    const int e = (int)(next_u64() % 20);  // P in [2^e, 2^(e+1))
    const int s = 52 - e;
    const int lead = (int)(next_u64() % (uint64_t)s);  // leading one of the fraction
    uint64_t F = (1ull << lead) | (next_u64() & ((1ull << lead) - 1));
    if (lead > 24) {
      const int sh = lead - 23;
      F &= ~((1ull << sh) - 1);
      F |= 1ull << (sh - 1);  // an exact tie
      const int kind = (int)(next_u64() % 3);
      if (kind == 1) F -= 1;            // just below it
      if (kind == 2 && sh > 1) F |= 1;  // just above it (a sticky bit far below)
    }
    if (k % 5 == 0) F = (1ull << s) - 1;
    const uint64_t ipart = (next_u64() << s) & 0xFFFFFFFFFFFFFull;
    const double P = from_bits(((uint64_t)(1023 + e) << 52) | ipart | F);
    if (!check(P)) return 1;
  }
  // values split() refuses
  const double refused[] = {0.0, -0.0, 0.25, 0.5, 0.999999999, -1.0, -0.5, 1048576.0, 2147483648.0, 4e9, 1e300,
                            std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                            std::numeric_limits<double>::quiet_NaN(), std::numeric_limits<double>::denorm_min()};
  for (double P : refused)
    if (!check(P)) return 1;
  if (rounded_to_one < 1000) {
    printf("only %lld fractions rounded to one\n", rounded_to_one);
    return 1;
  }
  printf("ok %lld\n", cases);
  return 0;
}
