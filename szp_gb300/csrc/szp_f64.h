// Float64 quantization and dequantization in integer arithmetic.
//
// GB300 retires a warp-wide FP64 instruction about once every 16 cycles per
// SM, so the four FP64 instructions of the float64 quantizer (the product
// x * (1/eb), two range compares, the truncating conversion) and the two of
// the dequantizer ((double)q, the product with eb) bound the float64 kernels.
// The same results come out of 64-bit integer arithmetic on the operands'
// fields: the exact 106-bit product of the significands rounded to nearest,
// ties to even, at 53 bits, which is binary64 multiplication as IEEE 754-2008
// defines it (sections 4.3.1 and 5.4.1).
//
// The header is plain C++ as well as CUDA so that the host test suite checks
// it against the CPU's own binary64 multiply.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SZP_F64_FN __host__ __device__ __forceinline__
#else
#define SZP_F64_FN static inline
#endif

namespace szp {
namespace f64i {

SZP_F64_FN uint64_t bits_of(double v) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t u;
  memcpy(&u, &v, 8);
  return u;
#endif
}

SZP_F64_FN double double_of(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double v;
  memcpy(&v, &u, 8);
  return v;
#endif
}

SZP_F64_FN int clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)v);
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

SZP_F64_FN int clz32(uint32_t v) {
#if defined(__CUDA_ARCH__)
  return __clz((int)v);
#else
  return v ? __builtin_clz(v) : 32;
#endif
}

// a * b for a < 2^32, b < 2^53 as hi:lo (the product is below 2^85).
SZP_F64_FN void mul_32x53(uint32_t a, uint64_t b, uint64_t& hi, uint64_t& lo) {
  const uint64_t p0 = (uint64_t)a * (uint32_t)b;          // < 2^64
  const uint64_t p1 = (uint64_t)a * (uint32_t)(b >> 32);  // < 2^53
  lo = p0 + (p1 << 32);
  hi = (p1 >> 32) + (lo < p0 ? 1u : 0u);
}

// a * b for a, b < 2^53 as hi:lo.
SZP_F64_FN void mul_53x53(uint64_t a, uint64_t b, uint64_t& hi, uint64_t& lo) {
  lo = a * b;
#if defined(__CUDA_ARCH__)
  hi = __umul64hi(a, b);
#else
  hi = (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// A binary64 operand as (-1)^sign * m * 2^e, m in [2^52, 2^53) when finite
// and nonzero (subnormals normalised).  cls: 0 zero, 1 finite nonzero,
// 2 infinity or NaN.
struct Operand {
  uint64_t m;
  int32_t e;
  uint32_t sign, cls;
};

SZP_F64_FN Operand unpack(uint64_t u) {
  Operand o;
  o.sign = (uint32_t)(u >> 63);
  const uint32_t ef = (uint32_t)(u >> 52) & 0x7FFu;
  const uint64_t f = u & 0xFFFFFFFFFFFFFull;
  o.m = f | (1ull << 52);
  o.e = (int32_t)ef - 1075;
  o.cls = ef == 0x7FFu ? 2u : 1u;
  if (ef == 0) {
    if (f == 0) {
      o.cls = 0;
    } else {  // subnormal: f * 2^-1074
      const int sh = clz64(f) - 11;
      o.m = f << sh;
      o.e = -1074 - sh;
    }
  }
  return o;
}

// The float64 quantizer: with p = x * inv rounded as binary64, q = trunc(p)
// when -2^31 - 1 < p < 2^31; otherwise (NaN, infinity, too large) *bad is set
// and q is INT32_MIN, what x86's truncating conversion gives.
SZP_F64_FN int32_t quantize(uint64_t xb, const Operand& inv, bool& bad) {
  const Operand x = unpack(xb);
  if (x.cls == 2 || inv.cls == 2) {
    bad = true;
    return INT32_MIN;
  }
  if (x.cls == 0 || inv.cls == 0) return 0;
  uint64_t hi, lo;
  mul_53x53(x.m, inv.m, hi, lo);           // P in [2^104, 2^106)
  const uint32_t t = (uint32_t)(hi >> 41);  // P >= 2^105
  const uint32_t sh = 52 + t;
  uint64_t s = (hi << (12 - t)) | (lo >> sh);  // top 53 bits of P
  // Rounding s up moves trunc(p) only when (s + 1) * 2^f is an integer, and
  // then s is odd, which a tie rounds up too: ties need no test here.
  s += (lo & ((1ull << sh) - 1)) >= (1ull << (sh - 1)) ? 1u : 0u;  // s in [2^52, 2^53]
  const int32_t f = x.e + inv.e + (int32_t)sh;                      // p = s * 2^f
  if (f >= 0) {  // |p| >= 2^52
    bad = true;
    return INT32_MIN;
  }
  const uint64_t i = f <= -54 ? 0 : s >> (uint32_t)(-f);  // trunc(|p|)
  const uint32_t neg = x.sign ^ inv.sign;
  if (i > 0x7FFFFFFFull + neg) {
    bad = true;
    return INT32_MIN;
  }
  return (int32_t)(neg ? 0u - (uint32_t)i : (uint32_t)i);
}

// 1/eb prepared for quantize_fast: significand, exponent field, sign, and
// whether it is normal (quantize_fast needs that; otherwise quantize()).
struct Inverse {
  Operand op;  // for quantize()
  uint64_t m;
  uint32_t ef, sign;
  bool normal;
};

SZP_F64_FN Inverse prepare_inverse(uint64_t u) {
  Inverse v;
  v.op = unpack(u);
  v.m = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  v.ef = (uint32_t)(u >> 52) & 0x7FFu;
  v.sign = (uint32_t)(u >> 63);
  v.normal = v.ef >= 1 && v.ef <= 2046;
  return v;
}

// quantize() in fewer steps for a normal x and a normal inverse (others take
// quantize()).  With P = mx * mi in [2^104, 2^106) and p = P * 2^E, rounding
// to 53 bits is adding half an ulp at bit sh (52 + [P >= 2^105]) and
// truncating there (ties up, which as quantize() notes never moves the
// truncated value), and truncating again at -E >= 64 composes with it:
// trunc(RN(p)) = (P + 2^(sh-1)) >> -E, which reads only the high word of the
// sum.
SZP_F64_FN int32_t quantize_fast(uint64_t xb, const Inverse& inv, bool& bad) {
  const uint32_t xh = (uint32_t)(xb >> 32);
  const uint32_t ex = (xh >> 20) & 0x7FFu;
  if (ex - 1u >= 0x7FEu || !inv.normal) return quantize(xb, inv.op, bad);  // zero, subnormal, inf, NaN
  uint64_t hi, lo;
  mul_53x53((xb & 0xFFFFFFFFFFFFFull) | (1ull << 52), inv.m, hi, lo);
  const uint64_t half = 1ull << (51 + (uint32_t)(hi >> 41));
  const uint64_t lo2 = lo + half;
  const uint64_t hi2 = hi + (lo2 < lo ? 1u : 0u);
  const int32_t k = 2086 - (int32_t)ex - (int32_t)inv.ef;  // -E - 64
  const uint32_t neg = (xh >> 31) ^ inv.sign;
  if (k < 0) {  // |p| >= 2^40
    bad = true;
    return INT32_MIN;
  }
  const uint64_t i = k >= 64 ? 0 : hi2 >> (uint32_t)k;
  if (i > 0x7FFFFFFFull + neg) {
    bad = true;
    return INT32_MIN;
  }
  return (int32_t)(neg ? 0u - (uint32_t)i : (uint32_t)i);
}

// Whether dequant_bits applies to eb: eb normal and small enough that no
// product |q| * eb with |q| <= 2^31 leaves the normal range.
SZP_F64_FN bool dequant_fast_ok(uint64_t ebb) {
  const uint32_t ef = (uint32_t)(ebb >> 52) & 0x7FFu;
  return ef >= 1 && ef <= 1023 + 991;
}

// (double)q * eb rounded as binary64, as bits, for an eb that
// dequant_fast_ok accepts; mb is eb's significand (with the leading one),
// ef its exponent field and sgn its sign bit in place.
SZP_F64_FN uint64_t dequant_bits(int32_t q, uint64_t mb, uint32_t ef, uint64_t sgn) {
  if (q == 0) return sgn;  // +0 * eb
  const uint64_t sg = ((uint64_t)((uint32_t)q >> 31) << 63) ^ sgn;
  uint32_t a = q < 0 ? 0u - (uint32_t)q : (uint32_t)q;  // |q| in [1, 2^31]
  const int c = clz32(a);
  a <<= c;  // [2^31, 2^32)
  // P = a * mb in [2^83, 2^85) as w * 2^32 + l, w in [2^51, 2^53)
  const uint64_t p0 = (uint64_t)a * (uint32_t)mb;
  const uint64_t w = (uint64_t)a * (uint32_t)(mb >> 32) + (p0 >> 32);
  const uint32_t l = (uint32_t)p0;
  const uint32_t t = (uint32_t)(w >> 52);  // P >= 2^84: round at bit 32, else at bit 31
  // the 53 kept bits, and the dropped bits scaled to 32 (their half is 2^31)
  uint64_t s = t ? w : ((w << 1) | (l >> 31));
  const uint32_t r = t ? l : (l << 1);
  s += (r > 0x80000000u || (r == 0x80000000u && (s & 1))) ? 1u : 0u;  // s in [2^52, 2^53]
  // |q| * eb = s * 2^(31 + t - c + ef - 1075): biased exponent ef + 31 + t - c;
  // a rounded-up s = 2^53 carries into the exponent field
  const uint64_t e = (uint64_t)(ef + 31 + t - (uint32_t)c);
  return sg | (((e - 1) << 52) + s);
}

}  // namespace f64i
}  // namespace szp
