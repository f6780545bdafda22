// Conversions between FP64 and FP32 done with integer instructions.
//
// On this GPU every instruction that reads or writes an FP64 value in the
// FP64 unit -- arithmetic and also the conversions F2F.F32.F64,
// F2F.F64.F32 and F2I.F64 -- runs at about 2 lanes per clock per SM, 1/64
// of the FP32 rate.  The integer pipe is much faster, so the kernels that
// turn FP64 state into FP32 working copies (and back) use these
// bit-manipulation forms instead of the hardware conversions.
//
// Range: normal FP32 numbers and zero.  Inputs below the FP32 normal range
// become (signed) zero; infinities and NaNs are not handled (the state
// never holds them on these paths).  Rounding: soft_d2f truncates toward
// zero, soft_d2f_rn rounds to nearest (ties away from zero); soft_f2d is
// exact.
#pragma once
#include <cstdint>
#include <cstring>
#ifdef __CUDACC__
#include <cuda_runtime.h>
#endif

namespace mdsc {

__host__ __device__ __forceinline__ uint32_t soft_hi(double x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2hiint(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return (uint32_t)(u >> 32);
#endif
}
__host__ __device__ __forceinline__ uint32_t soft_lo(double x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2loint(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return (uint32_t)u;
#endif
}
__host__ __device__ __forceinline__ double soft_hilo(uint32_t hi, uint32_t lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t u = ((uint64_t)hi << 32) | lo;
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
__host__ __device__ __forceinline__ float soft_uf(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
__host__ __device__ __forceinline__ uint32_t soft_fu(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
__host__ __device__ __forceinline__ uint32_t soft_shl3(uint32_t lo, uint32_t hi) {
  // (hi << 3) | (lo >> 29): a funnel shift
#ifdef __CUDA_ARCH__
  return __funnelshift_l(lo, hi, 3);
#else
  return (hi << 3) | (lo >> 29);
#endif
}

// FP64 -> FP32, truncated toward zero
__host__ __device__ __forceinline__ float soft_d2f(double x) {
  const uint32_t hi = soft_hi(x), lo = soft_lo(x);
  const uint32_t ah = hi & 0x7fffffffu;  // exponent (11 bits) | top 20 mantissa bits
  // rebias the exponent (1023 -> 127) and keep 23 mantissa bits
  uint32_t f = soft_shl3(lo, ah - (896u << 20));
  f = ah < (897u << 20) ? 0u : f;  // below the FP32 normal range: zero
  return soft_uf(f | (hi & 0x80000000u));
}

// FP64 -> FP32, rounded to nearest (ties away from zero), so that FP32
// working copies carry no bias
__host__ __device__ __forceinline__ float soft_d2f_rn(double x) {
  const uint32_t hi = soft_hi(x), lo = soft_lo(x);
  const uint32_t ah = hi & 0x7fffffffu;
  uint32_t f = soft_shl3(lo, ah - (896u << 20)) + ((lo >> 28) & 1u);  // a carry moves up the exponent
  f = ah < (897u << 20) ? 0u : f;
  return soft_uf(f | (hi & 0x80000000u));
}

// FP32 -> FP64, exact
__host__ __device__ __forceinline__ double soft_f2d(float f) {
  const uint32_t u = soft_fu(f);
  const uint32_t au = u & 0x7fffffffu;
  uint32_t hi = (au >> 3) + (896u << 20);  // exponent 127 -> 1023, top 20 mantissa bits
  uint32_t lo = u << 29;                   // the low 3 mantissa bits
  const bool zero = au < 0x00800000u;      // zero (subnormals flushed)
  hi = zero ? 0u : hi;
  lo = zero ? 0u : lo;
  return soft_hilo(hi | (u & 0x80000000u), lo);
}

// x split into two FP32 numbers, hi + lo = x to ~48 bits: hi holds the top
// 24 bits of the significand, lo the next 24 (truncated).
__host__ __device__ __forceinline__ void soft_split(double x, float& hi, float& lo) {
  hi = soft_d2f(x);
  const uint32_t h = soft_hi(x), l = soft_lo(x);
  const uint32_t e = (h >> 20) & 0x7ffu;  // biased FP64 exponent
  // the 29 significand bits below hi's 23: value rem * 2^(e - 1075)
  const uint32_t rem = l & 0x1fffffffu;
  // 2^(e - 1075) as an FP32 number: biased FP32 exponent e - 1075 + 127
  const int ee = (int)e - 948;
  float scale = soft_uf((uint32_t)(ee > 0 ? ee : 0) << 23);
  float r = (float)rem * scale;
  r = (e < 949u) ? 0.f : r;  // scale below the FP32 normal range (or x == 0)
  lo = (h & 0x80000000u) ? -r : r;
}

// low 32 bits of floor(y) for |y| < 2^52 (two's complement), the fixed-point
// image of a coordinate
__host__ __device__ __forceinline__ uint32_t soft_floor_u32(double y) {
  const uint32_t h = soft_hi(y), l = soft_lo(y);
  const bool neg = (h >> 31) != 0;
  const int e = (int)((h >> 20) & 0x7ffu) - 1023;  // unbiased exponent
  const uint32_t mh = (h & 0x000fffffu) | 0x00100000u;  // 53-bit significand, top word
  // integer part = M >> (52 - e) for 0 <= e <= 52; fraction = the bits shifted out
  const int s = 52 - e;
  uint32_t ip, frac;
  if (s >= 32) {
    const int t = s - 32;  // 0..20 for e >= 0
    ip = t >= 21 ? 0u : (mh >> t);
    frac = l | (t >= 21 ? mh : (mh & ((1u << t) - 1u)));
  } else {
    // s in 0..31: low word of (mh:l) >> s
    ip = s == 0 ? l : ((l >> s) | (mh << (32 - s)));
    frac = s == 0 ? 0u : (l & ((1u << s) - 1u));
  }
  if (e < 0) {  // |y| < 1
    ip = 0u;
    frac = (h & 0x7fffffffu) | l;
  }
  // floor of a negative number: -(integer part) - (fraction != 0)
  const uint32_t mag = ip + ((neg && frac != 0u) ? 1u : 0u);
  return neg ? 0u - mag : mag;
}

}  // namespace mdsc
