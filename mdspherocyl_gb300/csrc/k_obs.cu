// Observables outside the step -- the GPU form of acc_correl
// (v25/functions.cpp:2400-2470) and of the sums behind oo_params
// (:2702-2748, Qmat_3d :3426-3445).
//
// Pair histograms (acc_correl): every unordered pair of particles adds its
// terms to its distance bin floor(r / bar_w) of the functions 000, 110, 112
// and 220 -- 2, 2 dot, 2 (3 doti dotj - dot), 3 dot^2 - 1 to its species'
// histogram when both particles are of one species, and 1, dot,
// 3 doti dotj - dot, (3 dot^2 - 1) / 2 to the histogram of the species pair
// otherwise.  Species are contiguous blocks of particles, as the reference
// numbers them (calc_II / rev_II); a system's histograms are its nc species
// blocks, then the nc (nc - 1) / 2 pair blocks in the order (0,1), (0,2), ...,
// (1,2), ..., each 4 x nbins.
// One block per particle block of 128: each thread holds one particle i and
// meets every j > i of its system, 128 at a time from shared memory.  The
// sums are integers -- the counts exactly, the three others in fixed point
// with 2^24 units -- so they are the same whatever order the atomics land
// in.  The bins live in shared memory when they fit (kCorrSmemBins per
// block), else directly in global memory.
//
#include "mdsc_dev.cuh"
#include "reduce.cuh"

namespace mdsc {

constexpr int kCorrSmemBins = 1024;  // histogram bins (x 4 functions x 8 B = 32 KB) in shared memory
constexpr float kCorrScale = 16777216.f;  // 2^24: fixed-point unit of the non-count sums

template <bool SMEM>
__global__ void __launch_bounds__(kPartBlock) corr_kernel(Batch b, const CorrSys* __restrict__ cs,
                                                          const unsigned char* __restrict__ species, double bar_w,
                                                          unsigned long long* __restrict__ hist) {
  extern __shared__ unsigned long long shist[];
  __shared__ uint32_t sx[kPartBlock], sy[kPartBlock], sz[kPartBlock];
  __shared__ float4 sa[kPartBlock];
  __shared__ unsigned char ssp[kPartBlock];
  const int2 bk = b.blk[blockIdx.x];
  const int s = bk.x;
  const SysDev& P = b.sys[s];
  const CorrSys C = cs[s];
  const int nbins = C.nbins, nc = C.nsp;
  const int nwords = (nc + nc * (nc - 1) / 2) * 4 * nbins;
  unsigned long long* gh = hist + C.off;
  unsigned long long* h = SMEM ? shist : gh;
  if (SMEM) {
    for (int k = threadIdx.x; k < nwords; k += blockDim.x) shist[k] = 0ull;
    __syncthreads();
  }
  const int N = b.ntot;
  const int i = bk.y + threadIdx.x;
  const int iend = P.part_off + P.n;
  const bool ok = i < iend;
  uint32_t ux = 0, uy = 0, uz = 0;
  float4 ai = make_float4(0.f, 0.f, 1.f, 0.f);
  int spi = 0;
  if (ok) {
    ux = b.pfx[i];
    uy = b.pfx[N + i];
    uz = b.pfx[2 * N + i];
    ai = b.pax[i];
    spi = species[i];
  }
  const float ibw = (float)(1.0 / bar_w);
  // how far the FP32 t = r / bar_w may be from the reference's: ~8 roundings
  // relative (bounded by 1e-6 t) plus the fixed-point quantum of each
  // coordinate difference (L / 2^32 per axis, doubled)
  const float q0 = (float)(4.0 * fmax(P.L[0], fmax(P.L[1], P.L[2])) / 4294967296.0 / bar_w) + 1e-6f;
  for (int j0 = bk.y; j0 < iend; j0 += kPartBlock) {
    const int nj = min(kPartBlock, iend - j0);
    __syncthreads();
    if (threadIdx.x < nj) {
      const int q = j0 + threadIdx.x;
      sx[threadIdx.x] = b.pfx[q];
      sy[threadIdx.x] = b.pfx[N + q];
      sz[threadIdx.x] = b.pfx[2 * N + q];
      sa[threadIdx.x] = b.pax[q];
      ssp[threadIdx.x] = species[q];
    }
    __syncthreads();
    if (!ok) continue;
    for (int k = 0; k < nj; ++k) {
      const int j = j0 + k;
      if (j <= i) continue;
      const float dx = fix_diff(ux, sx[k], P.Lfix[0]);
      const float dy = fix_diff(uy, sy[k], P.Lfix[1]);
      const float dz = fix_diff(uz, sz[k], P.Lfix[2]);
      const float4 aj = sa[k];
      float r = sqrtf(dx * dx + dy * dy + dz * dz);
      const float t = r * ibw;
      int bin = (int)floorf(t);
      const float fr = t - (float)bin;
      const float edge = 1e-6f * t + q0;
      if (fr < edge || fr > 1.f - edge) {
        // near a bin edge: the reference's distance in FP64, rounded step
        // by step as it is (no fused multiply-adds)
        double D[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const double X = __dsub_rn(b.r[3 * i + a], b.r[3 * j + a]);
          D[a] = __dsub_rn(X, __dmul_rn(P.L[a], floor(__dadd_rn(X / P.L[a], 0.5))));
        }
        const double R = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(D[0], D[0]), __dmul_rn(D[1], D[1])),
                                        __dmul_rn(D[2], D[2])));
        bin = (int)floor(R / bar_w);
      }
      if (bin < 0 || bin >= nbins) continue;
      const float dot = ai.x * aj.x + ai.y * aj.y + ai.z * aj.z;
      const float ir = r > 0.f ? 1.f / r : 0.f;
      const float doti = (ai.x * dx + ai.y * dy + ai.z * dz) * ir;
      const float dotj = (aj.x * dx + aj.y * dy + aj.z * dz) * ir;
      // i < j and species ascend with the index, so spi <= spj
      const int spj = ssp[k];
      const bool intra = spi == spj;
      // pair block (m, n), m < n: after the nc species blocks, in row order
      const int blkno = intra ? spi : nc + spi * (2 * nc - spi - 1) / 2 + (spj - spi - 1);
      const float w = intra ? 2.f : 1.f;
      const int v110 = __float2int_rn(w * dot * kCorrScale);
      const int v112 = __float2int_rn(w * (3.f * doti * dotj - dot) * kCorrScale);
      const int v220 = __float2int_rn(0.5f * w * (3.f * dot * dot - 1.f) * kCorrScale);
      unsigned long long* hb = h + (size_t)blkno * 4 * nbins;
      atomicAdd(&hb[0 * nbins + bin], intra ? 2ull : 1ull);
      atomicAdd(&hb[1 * nbins + bin], (unsigned long long)(long long)v110);
      atomicAdd(&hb[2 * nbins + bin], (unsigned long long)(long long)v112);
      atomicAdd(&hb[3 * nbins + bin], (unsigned long long)(long long)v220);
    }
  }
  if (SMEM) {
    __syncthreads();
    for (int k = threadIdx.x; k < nwords; k += blockDim.x)
      if (shist[k] != 0ull) atomicAdd(&gh[k], shist[k]);
  }
}

// Per particle block: sum of the rod axes (3), of their outer products (6,
// the Q tensor's input) and of the dipole moment vectors mu O^T o_body (3),
// in FP64, then float-float over the block.
__global__ void __launch_bounds__(kPartBlock) order_sums_kernel(Batch b, double* __restrict__ out) {
  __shared__ double sh[12 * kPartBlock / 32];
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  const int i = bk.y + threadIdx.x;
  double v[12];
#pragma unroll
  for (int c = 0; c < 12; ++c) v[c] = 0.0;
  if (i < P.part_off + P.n) {
    const double* O = b.O + 9 * i;
    const double o0 = O[6], o1 = O[7], o2 = O[8];
    v[0] = o0;
    v[1] = o1;
    v[2] = o2;
    v[3] = o0 * o0;
    v[4] = o0 * o1;
    v[5] = o0 * o2;
    v[6] = o1 * o1;
    v[7] = o1 * o2;
    v[8] = o2 * o2;
    const int g0 = P.dip_off + (i - P.part_off) * P.nd;
    for (int w = 0; w < P.nd; ++w) {
      const int g = g0 + w;
      const double ox = b.dob[3 * g], oy = b.dob[3 * g + 1], oz = b.dob[3 * g + 2], mu = b.dmu[g];
      v[9] += mu * (O[0] * ox + O[3] * oy + O[6] * oz);
      v[10] += mu * (O[1] * ox + O[4] * oy + O[7] * oz);
      v[11] += mu * (O[2] * ox + O[5] * oy + O[8] * oz);
    }
  }
  double tot[12];
  block_sum<12, kPartBlock>(v, sh, tot);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < 12; ++c) out[12 * blk_slot(P, bk) + c] = tot[c];
  }
}

// max_bins: the largest (species blocks + pair blocks) x nbins of any system
void launch_correlations(const Batch& b, const CorrSys* c, const unsigned char* species, double bar_w,
                         int max_bins, unsigned long long* hist, cudaStream_t s) {
  if (!b.nblk) return;
  if (max_bins <= kCorrSmemBins)
    corr_kernel<true><<<b.nblk, kPartBlock, 4 * max_bins * sizeof(unsigned long long), s>>>(b, c, species, bar_w,
                                                                                             hist);
  else
    corr_kernel<false><<<b.nblk, kPartBlock, 0, s>>>(b, c, species, bar_w, hist);
}

void launch_order_sums(const Batch& b, double* out, cudaStream_t s) {
  if (b.nblk) order_sums_kernel<<<b.nblk, kPartBlock, 0, s>>>(b, out);
}

}  // namespace mdsc
