// Checks the integer float64 quantizer and dequantizer (szp_f64.h) against
// this CPU's binary64 multiply and truncating conversion, the arithmetic the
// reference's szp_double.cc / szpd_double.cc run.  usage: f64_arith_check N SEED
// Prints "ok <cases>" or the first mismatch and exits 1.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "szp_f64.h"

using namespace szp::f64i;

static uint64_t rng_state;
static uint64_t next() {  // splitmix64
  uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// The reference quantizer: (int)(x * inv) behind the range test; out of range
// gives what x86's cvttsd2si gives, 0x80000000.
static int32_t quantize_ref(double x, double inv, bool& bad) {
  volatile double p = x * inv;
  if (p > -2147483649.0 && p < 2147483648.0) return (int32_t)p;
  bad = true;
  return INT32_MIN;
}

static double rand_double_any() {
  switch (next() % 8) {
    case 0: return double_of(next());  // any bit pattern
    case 1: return double_of(next() & 0x800FFFFFFFFFFFFFull);  // subnormal or zero
    case 2: {  // small integer-valued significand (exact products, ties)
      const double m = (double)(int64_t)(next() >> (11 + next() % 30));
      return (next() & 1 ? -m : m) * double_of((uint64_t)(1023 + (int)(next() % 80) - 40) << 52);
    }
    case 3: return (double)(int32_t)next() + (double)(next() % 4) * 0.25;
    default: {  // moderate magnitudes
      const uint64_t e = 1023 + (next() % 90) - 60;
      return double_of((next() & 0x800FFFFFFFFFFFFFull) | (e << 52));
    }
  }
}

static double rand_inv() {
  switch (next() % 6) {
    case 0: return double_of(next() & 0x7FFFFFFFFFFFFFFFull);  // any positive, inf and NaN included
    case 1: return double_of((uint64_t)(1023 + (int)(next() % 64) - 8) << 52);  // a power of two
    case 2: return (double)(next() % 100000 + 1);  // integer, odd ones give ties
    case 3: return -double_of((next() & 0xFFFFFFFFFFFFFull) | ((uint64_t)(1023 + next() % 40) << 52));
    default: return 1.0 / double_of((next() & 0xFFFFFFFFFFFFFull) | ((uint64_t)(1023 - 1 - next() % 40) << 52));
  }
}

static double rand_eb() {
  switch (next() % 5) {
    case 0: return double_of(((next() % 2014) + 1) << 52 | (next() & 0xFFFFFFFFFFFFFull));  // any accepted
    case 1: return double_of((uint64_t)(1023 - (int)(next() % 60)) << 52);  // a power of two
    case 2: return -double_of(((1023 - next() % 40) << 52) | (next() & 0xFFFFFFFFFFFFFull));
    case 3: return (double)(next() % 1000 + 1) * 1e-6;
    default: return double_of(((1023 - next() % 40) << 52) | (next() & 0xFFFFFFFFFFFFFull));
  }
}

static int32_t rand_q() {
  switch (next() % 5) {
    case 0: return (int32_t)next();
    case 1: return (int32_t)(next() % 64) - 32;
    case 2: return (int32_t)((next() & 1) ? INT32_MIN + (int32_t)(next() % 4) : INT32_MAX - (int32_t)(next() % 4));
    default: return (int32_t)((int64_t)(next() >> (33 + next() % 31)) * ((next() & 1) ? 1 : -1));
  }
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  rng_state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
  long cases = 0;
  for (long i = 0; i < n; i++) {
    // quantizer: one inverse per few hundred values, like one eb per field
    const double inv = rand_inv();
    const Operand io = unpack(bits_of(inv));
    const Inverse iv = prepare_inverse(bits_of(inv));
    for (int k = 0; k < 8; k++, cases++) {
      double x = rand_double_any();
      if (k == 7) {  // a product within a few ulps of a boundary (integer or half-integer)
        static const double edge[] = {2147483648.0, 2147483647.0, 2147483647.5, -2147483648.0, -2147483648.5,
                                      -2147483649.0, -2147483647.5, 1.0, -1.0, 0.5, -0.5};
        const double target = (next() & 1) ? edge[next() % 11]
                                           : (double)(int32_t)next() + ((next() & 1) ? 0.5 : 0.0);
        x = target / inv;
        uint64_t u = bits_of(x);
        const int64_t d = (int64_t)(next() % 5) - 2;
        u += (uint64_t)d;
        x = double_of(u);
      }
      bool b1 = false, b2 = false, b3 = false;
      const int32_t r = quantize_ref(x, inv, b1);
      const int32_t g = quantize(bits_of(x), io, b2);
      const int32_t f = quantize_fast(bits_of(x), iv, b3);
      if (r != g || b1 != b2 || r != f || b1 != b3) {
        printf("quantize mismatch x=%a inv=%a ref=%d(%d) got=%d(%d) fast=%d(%d)\n", x, inv, r, (int)b1, g, (int)b2, f,
               (int)b3);
        return 1;
      }
    }
    // dequantizer
    const double eb = rand_eb();
    const uint64_t ebb = bits_of(eb);
    if (!dequant_fast_ok(ebb)) {
      printf("eb %a rejected\n", eb);
      return 1;
    }
    const uint64_t mb = (ebb & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const uint32_t ef = (uint32_t)(ebb >> 52) & 0x7FFu;
    for (int k = 0; k < 8; k++, cases++) {
      const int32_t q = rand_q();
      volatile double want = (double)q * eb;
      const uint64_t got = dequant_bits(q, mb, ef, ebb & 0x8000000000000000ull);
      if (bits_of(want) != got) {
        printf("dequant mismatch q=%d eb=%a want=%a got=%a\n", q, eb, want, double_of(got));
        return 1;
      }
    }
  }
  // the fast path's edges: the largest eb it takes times the largest |q|,
  // the smallest normal eb times 1
  const double edges[] = {double_of((uint64_t)(1023 + 991) << 52 | 0xFFFFFFFFFFFFFull), double_of(1ull << 52),
                          -double_of(1ull << 52), double_of((uint64_t)(1023 + 991) << 52)};
  const int32_t qs[] = {INT32_MIN, INT32_MAX, 1, -1, 0, 3, -3};
  for (double eb : edges) {
    const uint64_t ebb = bits_of(eb);
    if (!dequant_fast_ok(ebb)) {
      printf("edge eb %a rejected\n", eb);
      return 1;
    }
    for (int32_t q : qs) {
      volatile double want = (double)q * eb;
      const uint64_t got = dequant_bits(q, (ebb & 0xFFFFFFFFFFFFFull) | (1ull << 52), (uint32_t)(ebb >> 52) & 0x7FFu,
                                        ebb & 0x8000000000000000ull);
      if (bits_of(want) != got) {
        printf("dequant edge mismatch q=%d eb=%a want=%a got=%a\n", q, eb, want, double_of(got));
        return 1;
      }
      cases++;
    }
  }
  if (dequant_fast_ok(bits_of(double_of((uint64_t)(1023 + 992) << 52))) || dequant_fast_ok(bits_of(4.9e-324)) ||
      dequant_fast_ok(bits_of(1.0 / 0.0))) {
    printf("fast path accepts an eb it cannot take\n");
    return 1;
  }
  printf("ok %ld\n", cases);
  return 0;
}
