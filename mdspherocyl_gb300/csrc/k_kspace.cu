// Reciprocal-space Ewald dipolar sum -- the GPU form of force_dipK
// (v25/functions.cpp:1706-1961) with wave_v's prefactors (:1963-1990).
//
// k-set.  The reference loops n_x, n_y, n_z in [0, K_max-1] with four sign
// patterns (+-k_x, +-k_y, +k_z) and divides by 2 or 4 where components are
// zero (:1725-1744,1845-1850); that visits every distinct +-k pair of the
// cube exactly once with weight 2*Kvec/V.  The host enumerates the same
// distinct vectors once each (one representative per +-k pair) with that
// weight, optionally masked to |n|^2 <= ksq_max.
//
// Per k the structure factor is S(k) = k . U(k) with
// U_c(k) = sum_dipoles mu o_c exp(-i k.r) (the reference's uve); the
// reference removes each particle's own interaction per k with
// self(k) = sum_i |S_i(k)|^2 and uvslf_c(k) = sum_i Re(conj(S_i) U_ic).
//
// Phases.  Dipole positions are 32-bit box fractions u, so for
// k = 2 pi n / L the phase k.r = 2 pi (n . u) / 2^32 and the integer n . u
// wraps modulo 2^32 exactly: the phase is reduced exactly to [-pi, pi) for
// any box size and any k, and only the final sine/cosine is rounded.
//
// Kernels: ksum (partial sums over chunks of kKChunk particles, one k per
// thread), kcombine (chunks -> FP64 sums per k, energy and pressure-tensor
// terms per k), kgather (per particle over all k: force and torque).
#include "mdsc_dev.cuh"
#include "reduce.cuh"

namespace mdsc {

__device__ __forceinline__ void phase_exp(uint32_t ux, uint32_t uy, uint32_t uz, int4 n, float& c,
                                          float& s) {
  const uint32_t ph = (uint32_t)n.x * ux + (uint32_t)n.y * uy + (uint32_t)n.z * uz;
  // (int)ph * 2^-31 * pi: the phase, already reduced to [-pi, pi); the
  // hardware sine/cosine is accurate to ~4e-7 absolute on that range
  const float x = (float)(int32_t)ph * 1.4629180792671596e-09f;
  __sincosf(x, &s, &c);
}

// grid: one block per (system, particle chunk, k tile); work list kwork.
// With one dipole per particle the per-particle self terms need no per-k
// work: |S_i(k)|^2 = (m_i.k)^2 and Re(conj(S_i) U_ic) = (m_i.k) m_ic, so
// self(k) = k^T G k and uvslf(k) = G k with G = sum_i m_i m_i^T, which the
// first k tile of every chunk sums once.
template <int ND>
__global__ void __launch_bounds__(kKBlock) ksum_kernel(Batch b, const int4* __restrict__ kwork) {
  __shared__ uint32_t sx[kKChunk * ND], sy[kKChunk * ND], sz[kKChunk * ND];
  __shared__ float smx[kKChunk * ND], smy[kKChunk * ND], smz[kKChunk * ND];
  __shared__ double shG[6 * kKBlock / 32];
  const int4 w = kwork[blockIdx.x];
  const SysDev& P = b.sys[w.x];
  const int chunk = w.y;
  const int kl = w.z * kKBlock + threadIdx.x;
  const int ND_all = b.ndtot;
  const int p0 = chunk * kKChunk;
  const int np = min(kKChunk, P.n - p0);
  const int nd = P.nd;
  for (int q = threadIdx.x; q < np * nd; q += kKBlock) {
    const int g = P.dip_off + p0 * nd + q;
    sx[q] = b.dfx[g];
    sy[q] = b.dfx[ND_all + g];
    sz[q] = b.dfx[2 * ND_all + g];
    smx[q] = b.dm[g];
    smy[q] = b.dm[ND_all + g];
    smz[q] = b.dm[2 * ND_all + g];
  }
  __syncthreads();
  if (ND == 1 && w.z == 0) {
    double gl[6] = {0, 0, 0, 0, 0, 0};
    for (int q = threadIdx.x; q < np; q += kKBlock) {
      const double mx = smx[q], my = smy[q], mz = smz[q];
      gl[0] += mx * mx; gl[1] += mx * my; gl[2] += mx * mz;
      gl[3] += my * my; gl[4] += my * mz; gl[5] += mz * mz;
    }
    double tot[6];
    block_sum<6, kKBlock>(gl, shG, tot);
    if (threadIdx.x == 0) {
#pragma unroll
      for (int c = 0; c < 6; ++c) b.kG[((long long)P.gch_off + chunk) * 6 + c] = tot[c];
    }
  }
  if (kl >= P.nk) return;
  const int4 n = b.kn[P.k_off + kl];
  const float4 kv = b.kv[P.k_off + kl];
  float acc[10];
#pragma unroll
  for (int c = 0; c < 10; ++c) acc[c] = 0.f;
  if (ND == 1) {
    for (int p = 0; p < np; ++p) {
      float c, s;
      phase_exp(sx[p], sy[p], sz[p], n, c, s);
      // E = exp(-i k.r) = (c, -s); U_c += m_c E
      const float mx = smx[p], my = smy[p], mz = smz[p];
      acc[0] += mx * c; acc[1] -= mx * s;
      acc[2] += my * c; acc[3] -= my * s;
      acc[4] += mz * c; acc[5] -= mz * s;
    }
  } else {
    for (int p = 0; p < np; ++p) {
      float Sr = 0.f, Si = 0.f, Ur[3] = {0.f, 0.f, 0.f}, Ui[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        if (d < nd) {
          const int q = p * nd + d;
          float c, s;
          phase_exp(sx[q], sy[q], sz[q], n, c, s);
          const float mx = smx[q], my = smy[q], mz = smz[q];
          const float a = mx * kv.x + my * kv.y + mz * kv.z;
          Sr += a * c;
          Si -= a * s;
          Ur[0] += mx * c; Ui[0] -= mx * s;
          Ur[1] += my * c; Ui[1] -= my * s;
          Ur[2] += mz * c; Ui[2] -= mz * s;
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        acc[2 * c] += Ur[c];
        acc[2 * c + 1] += Ui[c];
        acc[7 + c] += Sr * Ur[c] + Si * Ui[c];
      }
      acc[6] += Sr * Sr + Si * Si;
    }
  }
  float* out = b.kpart + ((long long)P.kchunk_off + (long long)chunk * P.nk + kl) * 10;
  const int nout = ND == 1 ? 6 : 10;
#pragma unroll
  for (int c = 0; c < 10; ++c)
    if (c < nout) out[c] = acc[c];
}

// one thread per k over the whole batch: chunk sums in FP64, S(k), and the
// energy and pressure-tensor terms of that k (v25/functions.cpp:1839-1952)
template <int ND>
__global__ void kcombine_kernel(Batch b, const int2* __restrict__ kowner, double* __restrict__ kE) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.nktot) return;
  const int2 ow = kowner[k];  // (system, k index within the system)
  const SysDev& P = b.sys[ow.x];
  const int kl = ow.y;
  const int nv = ND == 1 ? 6 : 10;
  double s[10];
#pragma unroll
  for (int c = 0; c < 10; ++c) s[c] = 0.0;
  for (int ch = 0; ch < P.nkchunk; ++ch) {
    const float* in = b.kpart + ((long long)P.kchunk_off + (long long)ch * P.nk + kl) * 10;
#pragma unroll
    for (int c = 0; c < 10; ++c)
      if (c < nv) s[c] += (double)in[c];
  }
  const double kx = b.kvec[3 * k], ky = b.kvec[3 * k + 1], kz = b.kvec[3 * k + 2];
  if (ND == 1) {
    double G[6] = {0, 0, 0, 0, 0, 0};
    for (int ch = 0; ch < P.nkchunk; ++ch) {
      const double* g = b.kG + ((long long)P.gch_off + ch) * 6;
#pragma unroll
      for (int c = 0; c < 6; ++c) G[c] += g[c];
    }
    const double gx = G[0] * kx + G[1] * ky + G[2] * kz;
    const double gy = G[1] * kx + G[3] * ky + G[4] * kz;
    const double gz = G[2] * kx + G[4] * ky + G[5] * kz;
    s[6] = kx * gx + ky * gy + kz * gz;
    s[7] = gx;
    s[8] = gy;
    s[9] = gz;
  }
  double* ks = b.ksum + (long long)k * 10;
#pragma unroll
  for (int c = 0; c < 10; ++c) ks[c] = s[c];
  const double Sr = kx * s[0] + ky * s[2] + kz * s[4];
  const double Si = kx * s[1] + ky * s[3] + kz * s[5];
  const double val = b.kval[k];
  const double nrm = Sr * Sr + Si * Si;
  const double self = s[6];
  const double en = val * 0.5 * (nrm - self);
  b.kS[k] = make_float2((float)(val * Sr), (float)(val * Si));
  const double pval = b.kpre[k];
  const double kk[3] = {kx, ky, kz};
  double* e = kE + (long long)k * 10;
  e[0] = en;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    // Re(conj(S) U_j) - uvslf_j
    const double re = Sr * s[2 * j] + Si * s[2 * j + 1] - s[7 + j];
#pragma unroll
    for (int q = 0; q < 3; ++q)
      e[1 + 3 * j + q] =
          val * 0.5 * (((j == q ? 1.0 : 0.0) - pval * kk[j] * kk[q]) * (nrm - self) + 2.0 * re * kk[q]);
  }
}

// per particle over all k of its system: force and torque (:1853-1925)
template <int ND>
__global__ void __launch_bounds__(kPartBlock) kgather_kernel(Batch b) {
  __shared__ int4 skn[kKBlock];
  __shared__ float4 skv[kKBlock];
  __shared__ float2 sks[kKBlock];
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  const int i = bk.y + threadIdx.x;  // batch particle index
  const bool ok = i < P.part_off + P.n;
  const int nd = P.nd;
  const int ND_all = b.ndtot;
  uint32_t ux[ND], uy[ND], uz[ND];
  float mx[ND], my[ND], mz[ND];
  const int gd0 = P.dip_off + (i - P.part_off) * nd;
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    const bool v = ok && d < nd;
    const int g = v ? gd0 + d : 0;
    ux[d] = b.dfx[g];
    uy[d] = b.dfx[ND_all + g];
    uz[d] = b.dfx[2 * ND_all + g];
    mx[d] = v ? b.dm[g] : 0.f;
    my[d] = v ? b.dm[ND_all + g] : 0.f;
    mz[d] = v ? b.dm[2 * ND_all + g] : 0.f;
  }
  // outer accumulators (Kahan-compensated) and per-tile FP32 sums
  float fo[ND][6], fc[ND][6];
#pragma unroll
  for (int d = 0; d < ND; ++d)
#pragma unroll
    for (int c = 0; c < 6; ++c) fo[d][c] = fc[d][c] = 0.f;

  for (int k0 = 0; k0 < P.nk; k0 += kKBlock) {
    const int nk = min(kKBlock, P.nk - k0);
    __syncthreads();
    for (int q = threadIdx.x; q < nk; q += blockDim.x) {
      skn[q] = b.kn[P.k_off + k0 + q];
      skv[q] = b.kv[P.k_off + k0 + q];
      sks[q] = b.kS[P.k_off + k0 + q];
    }
    __syncthreads();
    float ft[ND][6];
#pragma unroll
    for (int d = 0; d < ND; ++d)
#pragma unroll
      for (int c = 0; c < 6; ++c) ft[d][c] = 0.f;
    for (int q = 0; q < nk; ++q) {
      const int4 n = skn[q];
      const float4 kv = skv[q];  // kx, ky, kz, val
      const float2 vS = sks[q];  // val * S(k)
      float Ec[ND], Es[ND], a[ND];
      float Sr = 0.f, Si = 0.f;
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        if (d < nd) {
          phase_exp(ux[d], uy[d], uz[d], n, Ec[d], Es[d]);
          a[d] = mx[d] * kv.x + my[d] * kv.y + mz[d] * kv.z;
          Sr += a[d] * Ec[d];
          Si -= a[d] * Es[d];
        }
      }
      // D = conj(val S) - val conj(S_i)
      const float Dr = vS.x - kv.w * Sr;
      const float Di = -vS.y + kv.w * Si;
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        if (d < nd) {
          // Z = E D with E = (c, -s)
          const float Zr = Ec[d] * Dr + Es[d] * Di;
          const float Zi = Ec[d] * Di - Es[d] * Dr;
          const float fF = -a[d] * Zi;
          const float fT = -Zr;
          ft[d][0] += fF * kv.x;
          ft[d][1] += fF * kv.y;
          ft[d][2] += fF * kv.z;
          ft[d][3] += fT * kv.x;
          ft[d][4] += fT * kv.y;
          ft[d][5] += fT * kv.z;
        }
      }
    }
#pragma unroll
    for (int d = 0; d < ND; ++d)
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const float y = ft[d][c] - fc[d][c];
        const float t = fo[d][c] + y;
        fc[d][c] = (t - fo[d][c]) - y;
        fo[d][c] = t;
      }
  }
  if (!ok) return;
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    if (d < nd) {
      const int g = gd0 + d;
      b.Fk[3 * g + 0] = (double)fo[d][0] - (double)fc[d][0];
      b.Fk[3 * g + 1] = (double)fo[d][1] - (double)fc[d][1];
      b.Fk[3 * g + 2] = (double)fo[d][2] - (double)fc[d][2];
      b.Gk[3 * g + 0] = (double)fo[d][3] - (double)fc[d][3];
      b.Gk[3 * g + 1] = (double)fo[d][4] - (double)fc[d][4];
      b.Gk[3 * g + 2] = (double)fo[d][5] - (double)fc[d][5];
    }
  }
}

template <int ND>
static void launch_kspace_nd(const Batch& b, const int4* kwork, int nkwork, const int2* kowner,
                             double* kE, cudaStream_t s) {
  if (b.nktot == 0) return;
  if (nkwork > 0) ksum_kernel<ND><<<nkwork, kKBlock, 0, s>>>(b, kwork);
  kcombine_kernel<ND><<<cdiv(b.nktot, 128), 128, 0, s>>>(b, kowner, kE);
  kgather_kernel<ND><<<b.nblk, kPartBlock, 0, s>>>(b);
}

template <int ND>
static void kspace_part_nd(const Batch& b, const int4* kwork, int nkwork, const int2* kowner,
                           double* kE, int part, cudaStream_t s) {
  if (b.nktot == 0) return;
  if (part == 0 && nkwork > 0) ksum_kernel<ND><<<nkwork, kKBlock, 0, s>>>(b, kwork);
  if (part == 1) kcombine_kernel<ND><<<cdiv(b.nktot, 128), 128, 0, s>>>(b, kowner, kE);
  if (part == 2) kgather_kernel<ND><<<b.nblk, kPartBlock, 0, s>>>(b);
}

// one of the three k-space kernels (0: ksum, 1: kcombine, 2: kgather)
void launch_kspace_parts(const Batch& b, int maxnd, const int4* kwork, int nkwork, const int2* kowner,
                         double* kE, int part, cudaStream_t s) {
  if (maxnd <= 1)
    kspace_part_nd<1>(b, kwork, nkwork, kowner, kE, part, s);
  else if (maxnd == 2)
    kspace_part_nd<2>(b, kwork, nkwork, kowner, kE, part, s);
  else
    kspace_part_nd<4>(b, kwork, nkwork, kowner, kE, part, s);
}

void launch_kspace(const Batch& b, int maxnd, const int4* kwork, int nkwork, const int2* kowner,
                   double* kE, cudaStream_t s) {
  if (maxnd <= 1)
    launch_kspace_nd<1>(b, kwork, nkwork, kowner, kE, s);
  else if (maxnd == 2)
    launch_kspace_nd<2>(b, kwork, nkwork, kowner, kE, s);
  else
    launch_kspace_nd<4>(b, kwork, nkwork, kowner, kE, s);
}

}  // namespace mdsc
