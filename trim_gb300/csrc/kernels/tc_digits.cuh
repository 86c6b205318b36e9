// Digit slicing shared by the tensor-core GEMM kernels: the power-of-two
// row/column scale, the 7 balanced signed 7-bit digits of an FP64 value as
// exact BF16 values, and the 128-byte swizzled K-major operand layout of
// tcgen05 shared-memory descriptors.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace tn {
namespace {

__device__ __forceinline__ uint32_t swz_off(int r, int c) {  // row r (0..), 16-byte chunk c (0..7)
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

// power-of-two exponent e with |x| < 2^e for every x of a row/column whose
// largest magnitude has bit pattern maxbits (0 -> 0)
__device__ __forceinline__ int exp_of(uint64_t maxbits) {
  if (maxbits == 0) return 0;
  int ef = (int)(maxbits >> 52);
  if (ef == 0) return (63 - __clzll((long long)maxbits)) - 1073;  // subnormal: |x| < 2^(msb+1-1074)
  return ef - 1022;
}

// ---------------------------------------------------------------- slicing
// 8 consecutive-k values of one row -> NS slices of 8 bf16 (packed in uint4).
//
// NS = 7: X = |x| * 2^(49 - e) rounded to the nearest integer (X <= 2^49),
// V = +-X, and the balanced base-128 digits of V (d_1..d_6 in [-64, 63],
// d_0 = the rest, |d_0| <= 129).  They are the plain base-128 digits of
// Y = V + 64 * (1 + 128 + ... + 128^5), each minus 64 (the representation is
// unique, so this equals peeling digits off from the bottom), read out of the
// two 32-bit halves of Y by shifts and masks.  d * 2^-7s is formed exactly in
// FP32 from the bit pattern of 1.5 * 2^(23-7s) + d * 2^-7s (integer add into
// the mantissa, one exact subtraction); it has at most 8 significant bits, so
// its BF16 pattern is the top half of the FP32 pattern.
// NS = 1 (fast mode): the BF16 rounding of the FP32 rounding of x * 2^(7-e),
// the scaling done on the exponent field.
template <int NS>
__device__ __forceinline__ void make_slices(const double (&x)[8], int e, uint4 (&out)[NS]) {
  static_assert(NS == 1 || NS == 7, "7 digits (split) or one BF16 slice (fast)");
  uint32_t hbits[NS][8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint64_t bits = (uint64_t)__double_as_longlong(x[i]);
    const int ef = (int)((bits >> 52) & 0x7FF);
    if (NS == 1) {
      float f;
      const int nex = ef + 7 - e;  // biased exponent of x * 2^(7-e)
      if (ef != 0 && nex >= 1 && nex <= 2046)
        f = __double2float_rn(__longlong_as_double(
            (long long)((bits & ~(0x7FFull << 52)) | ((uint64_t)nex << 52))));
      else
        f = (float)ldexp(x[i], 7 - e);  // zero, subnormal or far below the row's scale
      hbits[0][i] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(f)) << 16;
    } else {
      uint64_t mant = bits & ((1ull << 52) - 1);
      int E = -1022;
      if (ef) {
        mant |= 1ull << 52;
        E = ef - 1023;
      }
      const int sh = 3 + e - E;  // X = mant * 2^(E - 52) * 2^(49 - e)
      const uint64_t X = (sh >= 64) ? 0ull : (sh > 0 ? ((mant + (1ull << (sh - 1))) >> sh) : (mant << (-sh)));
      const long long V = (bits >> 63) ? -(long long)X : (long long)X;
      const uint64_t Y = (uint64_t)(V + 2216338399296ll);  // + 64 * (128^6 - 1) / 127
      const uint32_t lo = (uint32_t)Y, hi = (uint32_t)(Y >> 32);
      int d[7];
      d[6] = (int)(lo & 127u) - 64;
      d[5] = (int)((lo >> 7) & 127u) - 64;
      d[4] = (int)((lo >> 14) & 127u) - 64;
      d[3] = (int)((lo >> 21) & 127u) - 64;
      d[2] = (int)(__funnelshift_r(lo, hi, 28) & 127u) - 64;
      d[1] = (int)((hi >> 3) & 127u) - 64;
      d[0] = (int)hi >> 10;
#pragma unroll
      for (int s = 0; s < 7; s++) {
        const float magic = __uint_as_float(0x4B400000u - ((uint32_t)(7 * s) << 23));  // 1.5 * 2^(23-7s)
        hbits[s][i] = __float_as_uint(__uint_as_float(__float_as_uint(magic) + (uint32_t)d[s]) - magic);
      }
    }
  }
#pragma unroll
  for (int s = 0; s < NS; s++)
    out[s] = make_uint4(__byte_perm(hbits[s][0], hbits[s][1], 0x7632), __byte_perm(hbits[s][2], hbits[s][3], 0x7632),
                        __byte_perm(hbits[s][4], hbits[s][5], 0x7632), __byte_perm(hbits[s][6], hbits[s][7], 0x7632));
}

// TF32 fast mode: 8 consecutive-k values of one row as TF32 patterns of
// x * 2^(7 - e) (FP32 with the 13 low mantissa bits rounded off, to nearest,
// ties away from zero), packed as two 16-byte chunks.  The scaling is done on
// the exponent field as in the BF16 fast mode.
__device__ __forceinline__ void make_tf32(const double (&x)[8], int e, uint4 (&out)[2]) {
  uint32_t w[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint64_t bits = (uint64_t)__double_as_longlong(x[i]);
    const int ef = (int)((bits >> 52) & 0x7FF);
    const int nex = ef + 7 - e;
    float f;
    if (ef != 0 && nex >= 1 && nex <= 2046)
      f = __double2float_rn(__longlong_as_double((long long)((bits & ~(0x7FFull << 52)) | ((uint64_t)nex << 52))));
    else
      f = (float)ldexp(x[i], 7 - e);  // zero, subnormal or far below the row's scale
    const uint32_t u = __float_as_uint(f);
    w[i] = ((u & 0x7F800000u) == 0x7F800000u) ? u : ((u + 0x1000u) & 0xFFFFE000u);
  }
  out[0] = make_uint4(w[0], w[1], w[2], w[3]);
  out[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

// S * 2^q as the nearest double (ties to even), integer operations only (the
// FP64 units and FP64 conversions run at ~2 per clock per SM on GB300)
__device__ __forceinline__ double fixed_to_double(long long S, int q) {
  if (S == 0) return 0.0;
  const uint64_t sign = (uint64_t)S & (1ull << 63);
  uint64_t mag = S < 0 ? (uint64_t)(-S) : (uint64_t)S;
  const int lz = __clzll((long long)mag);
  mag <<= lz;                                        // leading one at bit 63
  const int E = 63 - lz + q;                         // value = mag * 2^(E - 63)
  const uint32_t rem = (uint32_t)mag & 0x7FFu;
  const uint64_t r = (mag >> 11) + (uint64_t)((rem > 0x400u) | ((rem == 0x400u) & (uint32_t)(mag >> 11)));  // ties to even; may reach 2^53
  if (E < -1021 || E > 1022) return ldexp(__ll2double_rn(S), q);     // near the ends of the range: slow path
  // the hidden bit of r adds one to the exponent field (two when r carried to 2^53)
  return __longlong_as_double((long long)(sign | (((uint64_t)(E + 1022) << 52) + r)));
}


// d * 2^q for a finite double d, the exponent field adjusted as an integer
// when the result stays normal (else ldexp)
__device__ __forceinline__ double scale_pow2(double d, int q) {
  const uint64_t b = (uint64_t)__double_as_longlong(d);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0 || ex + q < 1 || ex + q > 2046) return ldexp(d, q);
  return __longlong_as_double((long long)(b + ((uint64_t)(int64_t)q << 52)));
}

}  // namespace
}  // namespace tn
