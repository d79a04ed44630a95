// oz_common.cuh -- building blocks of the split-operand ("Ozaki") tensor-core
// kernels oz_xc.cu and oz_gram.cu: FP64-accurate products of FP64 (and
// FP32) blocks computed exactly on the bf16 tensor cores.
//
// The error-free splitting (Ozaki, Ogita, Oishi and Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012): every
// value v of a group that shares one power-of-two scale 2^E (a row of the
// left factor, a column of the right one, a column over a 64-row chunk) is
// written in fixed point with F = 7 s fractional bits,
//     v ~= 2^E * sum_t d_t 2^(-7 (t + 1)),   t = 0 .. s-1,
// with integer digits of at most 128 in magnitude (rounded, so mostly within
// +-64), each held exactly by a bf16.  A digit product has at most 14
// bits, so the sums of digit products over a short contraction stay below
// 2^22 and the tensor cores' FP32 accumulation is exact: the products of
// level L = t + u are summed in one TMEM accumulator, and only the levels
// L < s are formed (the rest lie below 2^(-7 s) of the scale).
//
// Everything between the FP64 values and the digits, and back, is integer or
// FP32 arithmetic on the bit patterns: this GPU's FP64 pipe runs at 1/64 of
// its FP32 rate, so no FP64 instruction is spent per element.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tc_common.cuh"

// instruction descriptor of tcgen05.mma.kind::f16: D = F32, A = B = BF16,
// both K-major, M x N (the same fields as tf32_idesc with type code 1)
static __host__ __device__ constexpr uint32_t bf16_idesc(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

static __device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                                uint32_t idesc, uint32_t accumulate)
{
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arm an mbarrier with one arrival and the bytes the bulk copies will deliver
static __device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// contiguous global -> shared bulk copy (16-byte aligned addresses, size a
// multiple of 16), completion counted on the mbarrier
static __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                                uint64_t* bar)
{
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ----------------------------------------------------------------- digits

// biased FP64 exponent field (0 for zeros and subnormals, which split to 0)
static __device__ __forceinline__ int oz_bexp64(double v)
{
  return (int)((__double_as_longlong(v) >> 52) & 0x7FF);
}
// the same scale for an FP32 value, on the FP64 exponent scale
static __device__ __forceinline__ int oz_bexp32(float v)
{
  const int e = (int)((__float_as_uint(v) >> 23) & 0xFF);
  return e ? e + 896 : 0;
}

// |v| in fixed point with F fractional bits relative to 2^(E - 1022), E the
// group's largest biased exponent: U = round(|v| 2^(F - (E - 1022))),
// 0 <= U <= 2^F.  F <= 52.
template <int F>
static __device__ __forceinline__ uint64_t oz_fixed64(double v, int E)
{
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  const int be = (int)((b >> 52) & 0x7FF);
  if (be == 0) return 0;
  const uint64_t M = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;  // 53 bits
  const int sh = 53 - F + (E - be);  // >= 1 since F <= 52 and be <= E
  if (sh >= 64) return 0;
  return (M + (1ull << (sh - 1))) >> sh;
}
template <int F>
static __device__ __forceinline__ uint64_t oz_fixed32(float v, int E)
{
  const uint32_t b = __float_as_uint(v);
  const int be = (int)((b >> 23) & 0xFF);
  if (be == 0) return 0;
  const uint64_t M = (uint64_t)((b & 0x7FFFFFu) | 0x800000u);  // 24 bits
  const int sh = 24 - F + (E - (be + 896));
  if (sh <= 0) return M << (-sh);
  if (sh >= 64) return 0;
  return (M + (1ull << (sh - 1))) >> sh;
}

// bf16 bit pattern of the integer d, |d| <= 256 (exact), negated when neg
// (a digit of a negative value)
static __device__ __forceinline__ uint32_t oz_bf16_of(int d, uint32_t neg)
{
  const float f = __uint_as_float(0x4B000000u + (uint32_t)(d + 256)) - 8388864.0f;  // 2^23 + 256
  return (__float_as_uint(f) >> 16) ^ (neg << 15);
}

// the S balanced digits of U (< 2^(7 S)), most significant first, as bf16
// bit patterns carrying the value's sign
template <int S>
static __device__ __forceinline__ void oz_digits(uint64_t U, uint32_t neg, uint32_t (&d)[S])
{
  // add 64 to every digit below the top one, so that the field values minus
  // 64 are the balanced digits (the carry lands in the top digit)
  uint64_t bias = 0;
#pragma unroll
  for (int t = 1; t < S; t++) bias |= 64ull << (7 * (S - 1 - t));
  const uint64_t V = U + bias;
  d[0] = oz_bf16_of((int)(V >> (7 * (S - 1))), neg);
#pragma unroll
  for (int t = 1; t < S; t++) d[t] = oz_bf16_of((int)((V >> (7 * (S - 1 - t))) & 127) - 64, neg);
}

// exact integer value of an FP32 accumulator entry, |x| < 2^22
static __device__ __forceinline__ int oz_int_of(float x)
{
  return (int)__float_as_uint(x + 12582912.0f) - 0x4B400000;  // 1.5 * 2^23
}

// round-to-nearest-even FP64 of T * 2^base for a signed 64-bit T (|T| < 2^63),
// from integer operations only
static __device__ __forceinline__ double oz_to_double(long long T, int base)
{
  if (T == 0) return 0.0;
  const uint64_t sign = T < 0 ? 1ull : 0ull;
  uint64_t A = sign ? (uint64_t)(-T) : (uint64_t)T;
  const int lz = __clzll((long long)A);
  const uint64_t top = A << lz;  // bit 63 set
  uint64_t mant = top >> 11;     // 53 bits
  const uint64_t rest = top & 0x7FFull;
  if (rest > 0x400ull || (rest == 0x400ull && (mant & 1))) mant++;
  int e = 63 - lz + base + 1023;  // biased exponent of the leading bit
  if (mant >> 53) {
    mant >>= 1;
    e++;
  }
  if (e <= 0) return 0.0;  // below the normal range: negligible here
  if (e >= 2047) return __longlong_as_double((long long)((sign << 63) | 0x7FF0000000000000ull));
  return __longlong_as_double((long long)((sign << 63) | ((uint64_t)e << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// v = m * 2^e with m a signed integer mantissa: FP64 and FP32 inputs
static __device__ __forceinline__ void oz_unpack64(double v, long long& m, int& e)
{
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  const int be = (int)((b >> 52) & 0x7FF);
  if (be == 0) {
    m = 0;
    e = 0;
    return;
  }
  const long long M = (long long)((b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull);
  m = (b >> 63) ? -M : M;
  e = be - 1075;
}
static __device__ __forceinline__ void oz_unpack32(float v, long long& m, int& e)
{
  const uint32_t b = __float_as_uint(v);
  const int be = (int)((b >> 23) & 0xFF);
  if (be == 0) {
    m = 0;
    e = 0;
    return;
  }
  const long long M = (long long)((b & 0x7FFFFFu) | 0x800000u);
  m = (b >> 31) ? -M : M;
  e = be - 150;
}

// FP32 nearest to an FP64 value whose magnitude lies in FP32's normal range
// (smaller magnitudes give 0), from integer operations
static __device__ __forceinline__ float oz_to_float(double v)
{
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  const int be = (int)((b >> 52) & 0x7FF);
  const uint32_t sign = (uint32_t)(b >> 63);
  if (be == 0x7FF) return __uint_as_float((sign << 31) | 0x7F800000u | (uint32_t)((b & 0xFFFFFFFFFFFFFull) != 0));
  int e = be - 1023 + 127;
  if (e <= 0) return __uint_as_float(sign << 31);
  uint64_t mant = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;  // 53 bits
  uint32_t m24 = (uint32_t)(mant >> 29);
  const uint32_t rest = (uint32_t)(mant & 0x1FFFFFFFu);
  if (rest > 0x10000000u || (rest == 0x10000000u && (m24 & 1))) m24++;
  if (m24 >> 24) {
    m24 >>= 1;
    e++;
  }
  if (e >= 255) return __uint_as_float((sign << 31) | 0x7F800000u);
  return __uint_as_float((sign << 31) | ((uint32_t)e << 23) | (m24 & 0x7FFFFFu));
}

// ------------------------------------------- four digits with FP32 arithmetic
// The same balanced 7-bit digits (S = 4, 28 fraction bits), cut with FP32
// round-to-nearest arithmetic instead of integer shifts: rint(x) is
// (x + 1.5 * 2^23) - 1.5 * 2^23 for |x| < 2^22, and every remainder is
// formed exactly by an FMA.  The digits come out as floats holding small
// integers (|d| <= 128) whose bf16 patterns are their top 16 bits.
//   u = v 2^(28 - (E - 1022)),  |u| < 2^28
//   h = rint(u / 2^14), l = u - 2^14 h
//   d0 = rint(h / 2^7), d1 = h - 2^7 d0, d2 = rint(l / 2^7), d3 = rint(l - 2^7 d2)
// so u ~= 2^21 d0 + 2^14 d1 + 2^7 d2 + d3 to within 1/2.

#define OZ_RINT_MAGIC 12582912.0f  // 1.5 * 2^23

static __device__ __forceinline__ void oz_digits4_hl(float h, float l, float (&d)[4])
{
  d[0] = fmaf(h, 0.0078125f, OZ_RINT_MAGIC) - OZ_RINT_MAGIC;
  d[1] = fmaf(d[0], -128.0f, h);
  d[2] = fmaf(l, 0.0078125f, OZ_RINT_MAGIC) - OZ_RINT_MAGIC;
  d[3] = (fmaf(d[2], -128.0f, l) + OZ_RINT_MAGIC) - OZ_RINT_MAGIC;
}

// FP32 value; scale = 2^(28 - (E - 1022)) as a float (E in [923, 1176])
static __device__ __forceinline__ void oz_digits4_f32(float v, float scale, float (&d)[4])
{
  const float u = v * scale;
  const float h = fmaf(u, 0.00006103515625f, OZ_RINT_MAGIC) - OZ_RINT_MAGIC;  // 2^-14
  const float l = fmaf(h, -16384.0f, u);
  oz_digits4_hl(h, l, d);
}

// the scale of oz_digits4_f32 for a group exponent E, 0 when E is outside the
// range the float can hold (the caller then takes the integer path)
static __device__ __forceinline__ float oz_scale4(int E)
{
  const int f = 28 + 1022 - E + 127;
  return (f >= 1 && f <= 254) ? __uint_as_float((uint32_t)f << 23) : 0.0f;
}

// a 28-bit fixed point magnitude U (<= 2^28) with sign bit sg (bit 31): its
// two 14-bit halves as exact floats, then the digits (here l is in
// [0, 2^14), so d2 reaches 128; the digit products stay below 2^14)
static __device__ __forceinline__ void oz_digits4_u(uint32_t U, uint32_t sg, float (&d)[4])
{
  const float h = __uint_as_float(__float_as_uint(__uint_as_float(0x4B000000u | (U >> 14)) - 8388608.0f) ^ sg);
  const float l = __uint_as_float(__float_as_uint(__uint_as_float(0x4B000000u | (U & 0x3FFFu)) - 8388608.0f) ^ sg);
  oz_digits4_hl(h, l, d);
}

// FP64 value: the 28-bit fixed point integer from its bits, then as above
static __device__ __forceinline__ void oz_digits4_f64(double v, int E, float (&d)[4])
{
  oz_digits4_u((uint32_t)oz_fixed64<28>(v, E), (uint32_t)((uint64_t)__double_as_longlong(v) >> 63) << 31, d);
}

// ------------------------------------ four 8-bit digits (32 fraction bits)
// The Gram's digits: with its 64-row chunks the level sums of 8-bit digits
// stay exact in FP32 (|d0| <= 256, |d_t| <= 128 after, or d2 <= 256 on the
// integer path: every level below 2^24 over 64 rows), so a fourth bit per
// digit costs nothing and makes the products 16 times more accurate.
//   u = v 2^(32 - (E - 1022)),  |u| < 2^32 (exact: v's 24 bits, scaled)
//   h = rint(u / 2^16), l = u - 2^16 h
//   d0 = rint(h / 2^8), d1 = h - 2^8 d0, d2 = rint(l / 2^8), d3 = rint(l - 2^8 d2)
// so u ~= 2^24 d0 + 2^16 d1 + 2^8 d2 + d3 to within 1/2.
static __device__ __forceinline__ void oz_digits4x8_hl(float h, float l, float (&d)[4])
{
  d[0] = fmaf(h, 0.00390625f, OZ_RINT_MAGIC) - OZ_RINT_MAGIC;
  d[1] = fmaf(d[0], -256.0f, h);
  d[2] = fmaf(l, 0.00390625f, OZ_RINT_MAGIC) - OZ_RINT_MAGIC;
  d[3] = (fmaf(d[2], -256.0f, l) + OZ_RINT_MAGIC) - OZ_RINT_MAGIC;
}

// FP32 value; scale = 2^(32 - (E - 1022)) as a float
static __device__ __forceinline__ void oz_digits4x8_f32(float v, float scale, float (&d)[4])
{
  const float u = v * scale;
  const float h = fmaf(u, 0.0000152587890625f, OZ_RINT_MAGIC) - OZ_RINT_MAGIC;  // 2^-16
  const float l = fmaf(h, -65536.0f, u);
  oz_digits4x8_hl(h, l, d);
}

// the scale of oz_digits4x8_f32 for a group exponent E, 0 when E is outside
// the range the float can hold (the caller then takes the integer path)
static __device__ __forceinline__ float oz_scale4x8(int E)
{
  const int f = 32 + 1022 - E + 127;
  return (f >= 1 && f <= 254) ? __uint_as_float((uint32_t)f << 23) : 0.0f;
}

// a 32-bit fixed point magnitude U (<= 2^32) with sign bit sg (bit 31): its
// two 16-bit halves as exact floats (h <= 2^16), then the digits
static __device__ __forceinline__ void oz_digits4x8_u(uint64_t U, uint32_t sg, float (&d)[4])
{
  const float h = __uint_as_float(__float_as_uint(__uint_as_float(0x4B000000u | (uint32_t)(U >> 16)) - 8388608.0f) ^ sg);
  const float l = __uint_as_float(__float_as_uint(__uint_as_float(0x4B000000u | (uint32_t)(U & 0xFFFFu)) - 8388608.0f) ^ sg);
  oz_digits4x8_hl(h, l, d);
}

// FP64 value: the 32-bit fixed point integer from its bits, then as above
static __device__ __forceinline__ void oz_digits4x8_f64(double v, int E, float (&d)[4])
{
  oz_digits4x8_u(oz_fixed64<32>(v, E), (uint32_t)((uint64_t)__double_as_longlong(v) >> 63) << 31, d);
}

// two digits (floats holding integers) as one word of two bf16 patterns
static __device__ __forceinline__ uint32_t oz_pack_bf16(float lo, float hi)
{
  return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}
