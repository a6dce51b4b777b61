// FP64 division and square root, rounded to nearest-even, computed on the integer and FP32
// pipes.  GB300 issues FP64 at a small fraction of its FP32 and integer rates, and a
// correctly rounded FP64 division or square root costs the FP64 pipe about ten operations;
// the assembly's bit-exact cotangents need nine divisions and six square roots per
// triangle.  These routines give the same bits as the IEEE operations (__ddiv_rn,
// __dsqrt_rn) for every input.  (Additions and multiplications stay on the FP64 pipe: an
// integer multiplication of two 53-bit significands -- a 64-bit high and low product plus
// the rounding -- measured no cheaper than the FP64 multiply it would replace.)
//
// Method: Newton-Raphson on the integer result with an exact residual, then an exact
// remainder test for the rounding (the classical scheme for correctly rounded division and
// square root, e.g. J.-M. Muller et al., Handbook of Floating-Point Arithmetic, 2nd ed.,
// ch. 4 and 9): for a / b with significands ma, mb (53 bits, ma scaled so that ma / mb is
// in [1, 2)) the target is Q = floor(ma 2^53 / mb), a 54-bit integer; for sqrt(x) with
// significand m (scaled so that the exponent is even) S = floor(sqrt(m 2^54)).  An FP32
// seed gives 22 bits; each correction adds the exact 128-bit residual N - Q mb (N - S^2)
// scaled by an FP32 reciprocal of mb (of 2S), which leaves the estimate within one unit
// after two steps; a bounded fix-up against the exact remainder pins the floor, and the
// low bit of Q (S) with the remainder decides round-to-nearest-even (exact ties cannot
// occur for normal quotients or square roots, the even rule is kept all the same).
// Zeros, subnormals, infinities, NaNs, negative square roots and quotients that may leave
// the normal range are handed to the hardware operation.
#pragma once

#include <cstdint>

namespace ruv {

struct I128 {  // two's complement, hi:lo
  uint64_t hi, lo;
};

// (nhi:nlo) - a * b
__device__ __forceinline__ I128 i128_sub_mul(uint64_t nhi, uint64_t nlo, uint64_t a, uint64_t b) {
  const uint64_t phi = __umul64hi(a, b), plo = a * b;
  I128 r;
  r.lo = nlo - plo;
  r.hi = nhi - phi - (nlo < plo ? 1ull : 0ull);
  return r;
}
__device__ __forceinline__ bool i128_neg(I128 r) { return (int64_t)r.hi < 0; }
__device__ __forceinline__ I128 i128_add(I128 r, uint64_t v) {
  I128 o;
  o.lo = r.lo + v;
  o.hi = r.hi + (o.lo < v ? 1ull : 0ull);
  return o;
}
__device__ __forceinline__ I128 i128_sub(I128 r, uint64_t v) {
  I128 o;
  o.lo = r.lo - v;
  o.hi = r.hi - (r.lo < v ? 1ull : 0ull);
  return o;
}
// r >= v for a non-negative v below 2^64
__device__ __forceinline__ bool i128_ge(I128 r, uint64_t v) { return !i128_neg(r) && (r.hi != 0 || r.lo >= v); }
// float(r / 2^32), for |r| < 2^95, from two 32-bit conversions (64-bit integer <-> float
// conversions would run on the FP64 pipe); about 2^-23 relative, enough for a correction
__device__ __forceinline__ float i128_f32_shr32(I128 r) {
  const long long v = (long long)((r.hi << 32) | (r.lo >> 32));
  return __fmaf_rn(__int2float_rn((int)(v >> 32)), 4294967296.0f, __uint2float_rn((unsigned)v));
}
// c rounded to an integer multiple of 2^SH, for |c| < 2^(31 + SH), via a 32-bit conversion
template <int SH>
__device__ __forceinline__ uint64_t f32_to_step(float c) {
  return (uint64_t)(long long)__float2int_rn(__fmul_rn(c, 1.0f / (float)(1u << SH))) << SH;
}

constexpr uint64_t kFp64Frac = (1ull << 52) - 1;
constexpr uint64_t kFp64Hidden = 1ull << 52;

__device__ __forceinline__ double div_rn(double a, double b) {
  const uint64_t ua = (uint64_t)__double_as_longlong(a), ub = (uint64_t)__double_as_longlong(b);
  const int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
  if (ea == 0 || eb == 0 || ea == 0x7ff || eb == 0x7ff) return __ddiv_rn(a, b);
  uint64_t ma = (ua & kFp64Frac) | kFp64Hidden;
  const uint64_t mb = (ub & kFp64Frac) | kFp64Hidden;
  int e = ea - eb + 1022;  // biased exponent of the quotient
  if (ma >= mb) {
    e += 1;
  } else {
    ma <<= 1;
  }
  if (e <= 0 || e >= 2046) return __ddiv_rn(a, b);  // subnormal, or may round up to infinity
  // Q = floor(N / mb), N = ma 2^53 (107 bits), Q in [2^53, 2^54)
  const uint64_t nhi = ma >> 11, nlo = ma << 53;
  const float rb = __frcp_rn(__uint2float_rn((uint32_t)(mb >> 29)));  // ~ 2^29 / mb
  // seed: (ma 2^-30) (2^29 / mb) ~ (ma / mb) / 2 in [0.5, 1], times 2^54 (error below 2^33)
  uint64_t q = (uint64_t)__float2uint_rz(__fmul_rn(__fmul_rn(__uint2float_rn((uint32_t)(ma >> 30)), rb), 2147483648.0f))
               << 23;
  const float rb8 = __fmul_rn(rb, 8.0f);  // (r / 2^32) * rb8 ~ r / mb
  // first correction to a multiple of 2^8 (error then below 2^11), second exact to one unit
  q += f32_to_step<8>(__fmul_rn(i128_f32_shr32(i128_sub_mul(nhi, nlo, q, mb)), rb8));
  q += f32_to_step<0>(__fmul_rn(i128_f32_shr32(i128_sub_mul(nhi, nlo, q, mb)), rb8));
  I128 r = i128_sub_mul(nhi, nlo, q, mb);
  for (int k = 0; k < 3 && i128_neg(r); ++k) {
    q -= 1;
    r = i128_add(r, mb);
  }
  for (int k = 0; k < 3 && i128_ge(r, mb); ++k) {
    q += 1;
    r = i128_sub(r, mb);
  }
  if (i128_neg(r) || i128_ge(r, mb)) return __ddiv_rn(a, b);  // (not reached)
  uint64_t m = q >> 1;
  if ((q & 1ull) && ((r.hi | r.lo) != 0ull || (m & 1ull))) m += 1;
  if (m >> 53) {
    m >>= 1;
    e += 1;
  }
  const uint64_t sign = (ua ^ ub) & 0x8000000000000000ull;
  return __longlong_as_double((long long)(sign | ((uint64_t)e << 52) | (m & kFp64Frac)));
}

__device__ __forceinline__ double sqrt_rn(double x) {
  const uint64_t ux = (uint64_t)__double_as_longlong(x);
  const int ex = (int)(ux >> 52);  // the sign bit included: negative inputs land above 0x7ff
  if (ex == 0 || ex >= 0x7ff) return __dsqrt_rn(x);
  uint64_t m = (ux & kFp64Frac) | kFp64Hidden;
  int e = ex - 1023;
  if (e & 1) {
    m <<= 1;
    e -= 1;
  }
  // S = floor(sqrt(N)), N = m 2^54 (108 bits), S in [2^53, 2^54); sqrt(x) = S 2^(e/2 - 53)
  const uint64_t nhi = m >> 10, nlo = m << 54;
  const float sf = __fsqrt_rn(__uint2float_rn((uint32_t)(m >> 30)));  // ~ sqrt(m) 2^-15
  uint64_t s = (uint64_t)__float2uint_rz(__fmul_rn(sf, 1048576.0f)) << 22;  // error below 2^31
  // (r / 2^32) * k2s ~ r / 2S: k2s = 2^31 / S ~ 2 / (S >> 30)
  const float k2s = __fmul_rn(__frcp_rn(__uint2float_rn((uint32_t)(s >> 30))), 2.0f);
  s += f32_to_step<8>(__fmul_rn(i128_f32_shr32(i128_sub_mul(nhi, nlo, s, s)), k2s));
  s += f32_to_step<0>(__fmul_rn(i128_f32_shr32(i128_sub_mul(nhi, nlo, s, s)), k2s));
  I128 r = i128_sub_mul(nhi, nlo, s, s);  // floor: 0 <= N - S^2 < 2S + 1
  for (int k = 0; k < 3 && i128_neg(r); ++k) {
    r = i128_add(r, 2 * s - 1);
    s -= 1;
  }
  for (int k = 0; k < 3 && i128_ge(r, 2 * s + 1); ++k) {
    r = i128_sub(r, 2 * s + 1);
    s += 1;
  }
  if (i128_neg(r) || i128_ge(r, 2 * s + 1)) return __dsqrt_rn(x);  // (not reached)
  uint64_t m53 = s >> 1;
  if ((s & 1ull) && ((r.hi | r.lo) != 0ull || (m53 & 1ull))) m53 += 1;
  int eo = e / 2 + 1023;
  if (m53 >> 53) {
    m53 >>= 1;
    eo += 1;
  }
  return __longlong_as_double((long long)(((uint64_t)eo << 52) | (m53 & kFp64Frac)));
}

}  // namespace ruv
