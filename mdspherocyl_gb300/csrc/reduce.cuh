// Deterministic reductions.  FP64 arithmetic runs at a small fraction of
// the FP32 rate on this GPU, so warp-level sums of FP64 values are done in
// float-float (a hi/lo pair of FP32 numbers combined with error-free
// TwoSum, ~48 significant bits) and only the per-warp results are added in
// FP64.  The tree shape is fixed, so results are bitwise reproducible.
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

// Sums NV FP64 values over a block of NT threads; thread 0 gets the totals
// in out[].  sh must hold NV * NT/32 doubles.
template <int NV, int NT>
__device__ __forceinline__ void block_sum(const double (&v)[NV], double* sh, double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    FF w = ff_warp_sum(ff_from(v[c]));
    if (lane == 0) sh[c * (NT / 32) + warp] = soft_f2d(w.hi) + soft_f2d(w.lo);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      double s = 0.0;
      for (int k = 0; k < NT / 32; ++k) s += sh[c * (NT / 32) + k];
      out[c] = s;
    }
  }
  __syncthreads();
}

// Same, for values already in float-float form (an FP32 value x enters as
// {x, 0} and costs no FP64 instruction).
template <int NV, int NT>
__device__ __forceinline__ void block_sum(const FF (&v)[NV], double* sh, double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    FF w = ff_warp_sum(v[c]);
    if (lane == 0) sh[c * (NT / 32) + warp] = soft_f2d(w.hi) + soft_f2d(w.lo);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      double s = 0.0;
      for (int k = 0; k < NT / 32; ++k) s += sh[c * (NT / 32) + k];
      out[c] = s;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ FF ff_of(float x) {
  FF r;
  r.hi = x;
  r.lo = 0.f;
  return r;
}

// Same, for a per-block maximum of non-negative values.
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
