// The FP32 screen of force_sc's pairs (v25/functions.cpp:1397-1553),
// partners from the Verlet list: in the WCA screen kernel, and in the
// neighbour pass of the systems with a real-space cutoff.
//
// Each thread screens its particle i against the partners q > i the
// iterator yields in ascending order: FP32 segment distance against
// 2^(1/3) sigma^2 with a margin for the FP32 arithmetic.  Candidates go to
// i's slots (wcand) in that order; each partner learns where its share of
// the pair will be (win, wincnt); the warp appends (slot, system) items to
// the work list of the FP64 evaluation with one atomic.  Every lane of the
// warp must call it (shuffles).
#pragma once
#include "mdsc_dev.cuh"
#include "seg_dist.cuh"

namespace mdsc {

template <class Next>
__device__ __forceinline__ void wca_screen_one(const Batch& b, const SysDev& P, int s, int i, bool ok,
                                               Next&& next) {
  const int lane = threadIdx.x & 31;
  const int N = b.ntot;
  int err = 0;
  int nc = 0;
  if (ok) {
    const uint32_t ux = b.pfx[i], uy = b.pfx[N + i], uz = b.pfx[2 * N + i];
    const float4 ai = b.pax[i];
    const float di = b.pdia[i];
    for (int q = next(); q >= 0; q = next()) {
      if (q < i) continue;
      const float dx = fix_diff(ux, b.pfx[q], P.Lfix[0]);
      const float dy = fix_diff(uy, b.pfx[N + q], P.Lfix[1]);
      const float dz = fix_diff(uz, b.pfx[2 * N + q], P.Lfix[2]);
      const float4 aj = b.pax[q];
      const float sg = 0.5f * (di + b.pdia[q]);
      const float d2 = seg_dist_fast(dx, dy, dz, ai.x, ai.y, ai.z, ai.w, aj.x, aj.y, aj.z, aj.w);
      // 2^(1/3) sigma^2, with a margin for the FP32 screen
      if (d2 >= 1.2599211f * sg * sg * 1.002f) continue;
      if (nc < kMaxC) {
        b.wcand[(long long)i * kMaxC + nc] = q;
        // the partner learns where its share of this pair will be
        const int k = atomicAdd(&b.wincnt[q], 1);
        if (k < kMaxC)
          b.win[(long long)q * kMaxC + k] = i * kMaxC + nc;
        else
          err |= kErrListOverflow;
      }
      ++nc;
    }
    if (nc > kMaxC) {
      err |= kErrListOverflow;
      nc = kMaxC;
    }
    b.wcnt[i] = nc;
  }
  // room on the work list for the warp's candidates: one atomic per warp
  int inc = nc;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += v;
  }
  const int wtot = __shfl_sync(0xffffffffu, inc, 31);
  int base = 0;
  if (lane == 31 && wtot > 0) base = atomicAdd(b.wlist_n, wtot);
  base = __shfl_sync(0xffffffffu, base, 31);
  const int off = base + inc - nc;
  for (int kk = 0; kk < nc; ++kk) b.wlist[off + kk] = make_int2(i * kMaxC + kk, s);
  if (err) atomicOr(&b.st[s].status, err);
}

}  // namespace mdsc
