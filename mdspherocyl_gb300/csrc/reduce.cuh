// Deterministic reductions.  FP64 arithmetic and FP64 conversions run at
// 1/64 of the FP32 rate on this GPU, so block-level sums of FP64 values are
// done in float-float (a hi/lo pair of FP32 numbers combined with
// error-free TwoSum, ~48 significant bits), entered and left by integer
// conversions, with one FP64 addition per value at the end.  The tree shape
// is fixed, so results are bitwise reproducible.
#pragma once
#include <cuda_runtime.h>

#include "softcvt.cuh"

namespace mdsc {

struct FF {
  float hi, lo;
};

// x as a float-float pair (48 bits), by integer instructions
__device__ __forceinline__ FF ff_from(double x) {
  FF r;
  soft_split(x, r.hi, r.lo);
  return r;
}

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b.hi - bb);
  const float lo = a.lo + b.lo + err;
  FF r;
  r.hi = s + lo;
  r.lo = lo - (r.hi - s);
  return r;
}

__device__ __forceinline__ FF ff_warp_sum(FF v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    FF o;
    o.hi = __shfl_xor_sync(0xffffffffu, v.hi, off);
    o.lo = __shfl_xor_sync(0xffffffffu, v.lo, off);
    v = ff_add(v, o);
  }
  return v;
}

// Sums NV float-float values over a block of NT threads (an FP32 value x
// enters as {x, 0}); thread 0 gets the totals in out[].  The warps' sums are
// added in float-float too, so each value costs one FP64 addition, at the
// end.  sh must hold NV * NT/32 doubles.
template <int NV, int NT>
__device__ __forceinline__ void block_sum(const FF (&v)[NV], double* sh, double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  FF* shf = reinterpret_cast<FF*>(sh);
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    FF w = ff_warp_sum(v[c]);
    if (lane == 0) shf[c * (NT / 32) + warp] = w;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      FF s = shf[c * (NT / 32)];
      for (int k = 1; k < NT / 32; ++k) s = ff_add(s, shf[c * (NT / 32) + k]);
      out[c] = soft_f2d(s.hi) + soft_f2d(s.lo);
    }
  }
  __syncthreads();
}

// Same, for FP64 values (split into float-float by integer instructions,
// 48 bits).
template <int NV, int NT>
__device__ __forceinline__ void block_sum(const double (&v)[NV], double* sh, double* out) {
  FF f[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) f[c] = ff_from(v[c]);
  block_sum<NV, NT>(f, sh, out);
}

__device__ __forceinline__ FF ff_of(float x) {
  FF r;
  r.hi = x;
  r.lo = 0.f;
  return r;
}

// Per-block maximum of non-negative values.
template <int NT>
__device__ __forceinline__ float block_max(float v, float* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  float m = 0.f;
  if (threadIdx.x == 0)
    for (int k = 0; k < NT / 32; ++k) m = fmaxf(m, sh[k]);
  __syncthreads();
  return m;
}

}  // namespace mdsc
