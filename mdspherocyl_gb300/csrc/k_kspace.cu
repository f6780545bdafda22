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

__device__ __forceinline__ void phase_cs(uint32_t ph, float& c, float& s) {
  // (int)ph * 2^-31 * pi: the phase, already reduced to [-pi, pi); the
  // hardware sine/cosine is accurate to ~4e-7 absolute on that range
  const float x = (float)(int32_t)ph * 1.4629180792671596e-09f;
  __sincosf(x, &s, &c);
}
__device__ __forceinline__ uint32_t phase_of(uint32_t ux, uint32_t uy, uint32_t uz, int4 n) {
  return (uint32_t)n.x * ux + (uint32_t)n.y * uy + (uint32_t)n.z * uz;
}
__device__ __forceinline__ void phase_exp(uint32_t ux, uint32_t uy, uint32_t uz, int4 n, float& c,
                                          float& s) {
  phase_cs(phase_of(ux, uy, uz, n), c, s);
}
// the gathers walk their k-vectors in order: where a k-vector is the last
// one plus (1, 0, 0) (n.w = 1, marked at layout) the phase advances by u_x,
// the same integer modulo 2^32 as the three products
__device__ __forceinline__ uint32_t phase_next(uint32_t ph, bool have, uint32_t ux, uint32_t uy, uint32_t uz,
                                               int4 n) {
  return (have && n.w) ? ph + ux : phase_of(ux, uy, uz, n);
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
  if ((ND > 1 && P.nd <= 1) || at_limit(b, w.x)) return;  // single-dipole systems: ksum1_kernel
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

// Single-dipole systems: as ksum_kernel<1>, with each thread taking two
// k-vectors (kl and kl + 64 of the block's k tile) in the halves of float2
// values, so every particle read from shared memory serves two k's and the
// six multiply-adds of U(k) issue once for both.
__global__ void __launch_bounds__(kKBlock / 2) ksum1_kernel(Batch b, const int4* __restrict__ kwork) {
  __shared__ uint32_t sx[kKChunk], sy[kKChunk], sz[kKChunk];
  __shared__ float4 sm[kKChunk];
  __shared__ double shG[6 * (kKBlock / 2) / 32];
  const int4 w = kwork[blockIdx.x];
  const SysDev& P = b.sys[w.x];
  if (P.nd != 1 || at_limit(b, w.x)) return;  // other systems: ksum_kernel<ND>
  const int chunk = w.y;
  const int t = threadIdx.x;
  const int kl0 = w.z * kKBlock + t, kl1 = kl0 + kKBlock / 2;
  const int ND_all = b.ndtot;
  const int p0 = chunk * kKChunk;
  const int np = min(kKChunk, P.n - p0);
  for (int q = t; q < np; q += kKBlock / 2) {
    const int g = P.dip_off + p0 + q;
    sx[q] = b.dfx[g];
    sy[q] = b.dfx[ND_all + g];
    sz[q] = b.dfx[2 * ND_all + g];
    sm[q] = make_float4(b.dm[g], b.dm[ND_all + g], b.dm[2 * ND_all + g], 0.f);
  }
  __syncthreads();
  if (w.z == 0) {
    double gl[6] = {0, 0, 0, 0, 0, 0};
    for (int q = t; q < np; q += kKBlock / 2) {
      const double mx = soft_f2d(sm[q].x), my = soft_f2d(sm[q].y), mz = soft_f2d(sm[q].z);
      gl[0] += mx * mx; gl[1] += mx * my; gl[2] += mx * mz;
      gl[3] += my * my; gl[4] += my * mz; gl[5] += mz * mz;
    }
    double tot[6];
    block_sum<6, kKBlock / 2>(gl, shG, tot);
    if (t == 0) {
#pragma unroll
      for (int c = 0; c < 6; ++c) b.kG[((long long)P.gch_off + chunk) * 6 + c] = tot[c];
      // the last chunk of the system to finish adds all chunks in chunk
      // order (the same bits whichever block it is) and rearms the counter
      __threadfence();
      if (atomicAdd(&b.kgcnt[w.x], 1) == P.nkchunk - 1) {
        __threadfence();
        double g[6] = {0, 0, 0, 0, 0, 0};
        for (int ch = 0; ch < P.nkchunk; ++ch)
#pragma unroll
          for (int c = 0; c < 6; ++c) g[c] += __ldcg(&b.kG[((long long)P.gch_off + ch) * 6 + c]);
#pragma unroll
        for (int c = 0; c < 6; ++c) b.kGs[6 * w.x + c] = g[c];
        b.kgcnt[w.x] = 0;
      }
    }
  }
  const bool v0 = kl0 < P.nk, v1 = kl1 < P.nk;
  if (!v0) return;
  const int4 n0 = b.kn[P.k_off + kl0];
  const int4 n1 = v1 ? b.kn[P.k_off + kl1] : n0;
  float2 acc[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) acc[c] = make_float2(0.f, 0.f);
#pragma unroll 2
  for (int p = 0; p < np; ++p) {
    float c0, s0, c1, s1;
    phase_exp(sx[p], sy[p], sz[p], n0, c0, s0);
    phase_exp(sx[p], sy[p], sz[p], n1, c1, s1);
    const float2 c = make_float2(c0, c1), sn = make_float2(-s0, -s1);
    // E = exp(-i k.r) = (c, -s); U_c += m_c E
    const float4 m = sm[p];
    acc[0] = __ffma2_rn(make_float2(m.x, m.x), c, acc[0]);
    acc[1] = __ffma2_rn(make_float2(m.x, m.x), sn, acc[1]);
    acc[2] = __ffma2_rn(make_float2(m.y, m.y), c, acc[2]);
    acc[3] = __ffma2_rn(make_float2(m.y, m.y), sn, acc[3]);
    acc[4] = __ffma2_rn(make_float2(m.z, m.z), c, acc[4]);
    acc[5] = __ffma2_rn(make_float2(m.z, m.z), sn, acc[5]);
  }
  float* out0 = b.kpart + ((long long)P.kchunk_off + (long long)chunk * P.nk + kl0) * 10;
#pragma unroll
  for (int c = 0; c < 6; ++c) out0[c] = acc[c].x;
  if (v1) {
    float* out1 = b.kpart + ((long long)P.kchunk_off + (long long)chunk * P.nk + kl1) * 10;
#pragma unroll
    for (int c = 0; c < 6; ++c) out1[c] = acc[c].y;
  }
}

template <int ND>
static void launch_ksum(const Batch& b, const int4* kwork, int nkwork, cudaStream_t s) {
  // every single-dipole system through the single-dipole kernel, in any
  // batch, so that it gives the same bits alone and beside multi-dipole ones
  ksum1_kernel<<<nkwork, kKBlock / 2, 0, s>>>(b, kwork);
  if (ND > 1) ksum_kernel<ND><<<nkwork, kKBlock, 0, s>>>(b, kwork);
}

// one thread per k over the whole batch: chunk sums in FP64, S(k), and the
// energy and pressure-tensor terms of that k (v25/functions.cpp:1839-1952)
template <int ND>
__global__ void kcombine_kernel(Batch b, const int2* __restrict__ kowner, double* __restrict__ kE) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.nktot) return;
  const int2 ow = kowner[k];  // (system, k index within the system)
  if (at_limit(b, ow.x)) return;
  const SysDev& P = b.sys[ow.x];
  const int kl = ow.y;
  // single-dipole systems (all of them when ND = 1): 6 sums per chunk and
  // the self terms from the moment tensor, as ksum1_kernel leaves them
  const bool one = ND == 1 || P.nd == 1;
  const int nv = one ? 6 : 10;
  // chunk sums in float-float (FP32 instructions; ~48 bits), then FP64
  FF sf[10];
#pragma unroll
  for (int c = 0; c < 10; ++c) sf[c].hi = sf[c].lo = 0.f;
  for (int ch = 0; ch < P.nkchunk; ++ch) {
    const float* in = b.kpart + ((long long)P.kchunk_off + (long long)ch * P.nk + kl) * 10;
#pragma unroll
    for (int c = 0; c < 10; ++c)
      if (c < nv) {
        FF v;
        v.hi = in[c];
        v.lo = 0.f;
        sf[c] = ff_add(sf[c], v);
      }
  }
  double s[10];
#pragma unroll
  for (int c = 0; c < 10; ++c) s[c] = c < nv ? soft_f2d(sf[c].hi) + soft_f2d(sf[c].lo) : 0.0;
  const double kx = b.kvec[3 * k], ky = b.kvec[3 * k + 1], kz = b.kvec[3 * k + 2];
  if (one) {
    const double* G = b.kGs + 6 * ow.x;
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
  b.kS[k] = make_float2(soft_d2f_rn(val * Sr), soft_d2f_rn(val * Si));
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

// k-space results of one dipole from its Kahan sums (sum = fo - fc): the
// force as float-float, and the torque m x G (G the second triple) with the
// FP32 moment -- as accurate as the FP32 sums it is built from
__device__ __forceinline__ void store_kout(const Batch& b, int g, const float* fo, const float* fc,
                                           float mx, float my, float mz) {
#pragma unroll
  for (int c = 0; c < 3; ++c) b.Fk[3 * g + c] = make_float2(fo[c], -fc[c]);
  const float gx = fo[3], gy = fo[4], gz = fo[5];
  const float lx = -fc[3], ly = -fc[4], lz = -fc[5];
  b.Tk[3 * g + 0] = make_float2(my * gz - mz * gy, my * lz - mz * ly);
  b.Tk[3 * g + 1] = make_float2(mz * gx - mx * gz, mz * lx - mx * lz);
  b.Tk[3 * g + 2] = make_float2(mx * gy - my * gx, mx * ly - my * lx);
}

// per particle over all k of its system: force and torque (:1853-1925)
template <int ND>
__global__ void __launch_bounds__(kPartBlock) kgather_kernel(Batch b) {
  __shared__ int4 skn[kKBlock];
  __shared__ float4 skv[kKBlock];
  __shared__ float2 sks[kKBlock];
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  if ((ND > 1 && P.nd <= 1) || at_limit(b, bk.x)) return;  // single-dipole systems: kgather1 / kgather1s
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

  uint32_t ph[ND];
#pragma unroll
  for (int d = 0; d < ND; ++d) ph[d] = 0u;
  bool have = false;
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
          ph[d] = phase_next(ph[d], have, ux[d], uy[d], uz[d], n);
          phase_cs(ph[d], Ec[d], Es[d]);
          a[d] = mx[d] * kv.x + my[d] * kv.y + mz[d] * kv.z;
          Sr += a[d] * Ec[d];
          Si -= a[d] * Es[d];
        }
      }
      have = true;
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
  for (int d = 0; d < ND; ++d)
    if (d < nd) store_kout(b, gd0 + d, fo[d], fc[d], mx[d], my[d], mz[d]);
}

// Split gathers (large single-dipole systems, SysDev::kgs > 1): block part
// ks of a particle block takes the k tiles [ks tpk, (ks + 1) tpk), tpk =
// ceil(tiles / kgs), and leaves its Kahan sums (fo, fc per component) in
// its partial set; the block that finishes last adds the parts in part
// order (Kahan over the sums, the compensations apart) and stores the
// result, so the order of the sums does not depend on which block ends last.
__device__ __forceinline__ void kpart_range(const SysDev& P, int ks, int& k0, int& k1) {
  const int tpk = cdiv(cdiv(P.nk, kKBlock), P.kgs) * kKBlock;
  k0 = min(P.nk, ks * tpk);
  k1 = min(P.nk, (ks + 1) * tpk);
}
__device__ __forceinline__ float* kpart_set(const Batch& b, const SysDev& P, int slot, int ks) {
  return b.kgpart + ((long long)P.kgp_off + (long long)(slot - P.blk_off) * P.kgs + ks) * kPartBlock * 12;
}
// the parts of local particle p of a particle block, added in part order
__device__ __forceinline__ void kpart_combine(const Batch& b, const SysDev& P, int slot, int p, float* fo,
                                              float* fc) {
  float cs[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) fo[c] = fc[c] = cs[c] = 0.f;
  for (int q = 0; q < P.kgs; ++q) {
    const float* part = kpart_set(b, P, slot, q) + p * 12;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const float y = __fadd_rn(__ldcg(part + c), -fc[c]);
      const float tt = __fadd_rn(fo[c], y);
      fc[c] = __fadd_rn(__fadd_rn(tt, -fo[c]), -y);
      fo[c] = tt;
      cs[c] = __fadd_rn(cs[c], __ldcg(part + 6 + c));
    }
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) fc[c] = __fadd_rn(fc[c], cs[c]);
}

// Single-dipole systems: a thread takes two particles, i and i + 64 of its
// block, and runs them side by side in the halves of float2 values with
// the paired FP32 instructions, so every k read from shared memory serves
// two particles and the force/torque arithmetic issues once for both.
// With D = conj(val S) - val conj(S_i) (S_i = a e^{-ik.r}, a = m.k) the
// k-term is Z = e^{-ik.r} D; fF = -a Im Z, fT = -Re Z, written below with
// Dr = Re(val S) - val a cos, Dn = Im(val S) + val a sin.
namespace {
__device__ __forceinline__ float2 pk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
}  // namespace

__global__ void __launch_bounds__(kPartBlock / 2) kgather1_kernel(Batch b) {
  __shared__ int4 skn[kKBlock];
  __shared__ float4 skv[kKBlock];
  __shared__ float2 sks[kKBlock];
  __shared__ int last;
  const int2 wk = b.kgwork[blockIdx.x];  // (particle block, part)
  const int2 bk = b.blk[wk.x];
  const SysDev& P = b.sys[bk.x];
  if (P.nd != 1 || at_limit(b, bk.x)) return;  // other systems: kgather_kernel<ND>
  int kb, ke;
  kpart_range(P, wk.y, kb, ke);
  const int t = threadIdx.x;
  const int i0 = bk.y + t, i1 = i0 + kPartBlock / 2;
  const int iend = P.part_off + P.n;
  const bool ok0 = i0 < iend, ok1 = i1 < iend;
  const int ND_all = b.ndtot;
  // single dipole: dipole index = dip_off + (particle - part_off)
  const int g0 = ok0 ? P.dip_off + (i0 - P.part_off) : 0;
  const int g1 = ok1 ? P.dip_off + (i1 - P.part_off) : 0;
  const uint32_t ux0 = b.dfx[g0], uy0 = b.dfx[ND_all + g0], uz0 = b.dfx[2 * ND_all + g0];
  const uint32_t ux1 = b.dfx[g1], uy1 = b.dfx[ND_all + g1], uz1 = b.dfx[2 * ND_all + g1];
  const float2 mx = pk(ok0 ? b.dm[g0] : 0.f, ok1 ? b.dm[g1] : 0.f);
  const float2 my = pk(ok0 ? b.dm[ND_all + g0] : 0.f, ok1 ? b.dm[ND_all + g1] : 0.f);
  const float2 mz = pk(ok0 ? b.dm[2 * ND_all + g0] : 0.f, ok1 ? b.dm[2 * ND_all + g1] : 0.f);
  // outer accumulators (Kahan-compensated) of the per-tile sums
  float2 fo[6], fc[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) fo[c] = fc[c] = bc(0.f);

  uint32_t ph0 = 0u, ph1 = 0u;
  bool have = false;  // a phase from the previous k-vector (the first of the range computes its own)
  for (int k0 = kb; k0 < ke; k0 += kKBlock) {
    const int nk = min(kKBlock, ke - k0);
    __syncthreads();
    for (int q = t; q < nk; q += kPartBlock / 2) {
      skn[q] = b.kn[P.k_off + k0 + q];
      skv[q] = b.kv[P.k_off + k0 + q];
      sks[q] = b.kS[P.k_off + k0 + q];
    }
    __syncthreads();
    float2 ft[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) ft[c] = bc(0.f);
#pragma unroll 2
    for (int q = 0; q < nk; ++q) {
      const int4 n = skn[q];
      const float4 kv = skv[q];  // kx, ky, kz, val
      const float2 vS = sks[q];  // val * S(k)
      float c0, s0, c1, s1;
      ph0 = phase_next(ph0, have, ux0, uy0, uz0, n);
      ph1 = phase_next(ph1, have, ux1, uy1, uz1, n);
      have = true;
      phase_cs(ph0, c0, s0);
      phase_cs(ph1, c1, s1);
      const float2 c = pk(c0, c1), sn = pk(s0, s1);
      const float2 a = __ffma2_rn(mz, bc(kv.z), __ffma2_rn(my, bc(kv.y), __fmul2_rn(mx, bc(kv.x))));
      const float2 va = __fmul2_rn(bc(kv.w), a);
      const float2 Dr = __ffma2_rn(pk(-va.x, -va.y), c, bc(vS.x));
      const float2 Dn = __ffma2_rn(va, sn, bc(vS.y));
      const float2 fF = __fmul2_rn(a, __ffma2_rn(c, Dn, __fmul2_rn(sn, Dr)));
      const float2 fT = __ffma2_rn(sn, Dn, __fmul2_rn(pk(-c.x, -c.y), Dr));
      ft[0] = __ffma2_rn(fF, bc(kv.x), ft[0]);
      ft[1] = __ffma2_rn(fF, bc(kv.y), ft[1]);
      ft[2] = __ffma2_rn(fF, bc(kv.z), ft[2]);
      ft[3] = __ffma2_rn(fT, bc(kv.x), ft[3]);
      ft[4] = __ffma2_rn(fT, bc(kv.y), ft[4]);
      ft[5] = __ffma2_rn(fT, bc(kv.z), ft[5]);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const float2 y = __fadd2_rn(ft[c], pk(-fc[c].x, -fc[c].y));
      const float2 tt = __fadd2_rn(fo[c], y);
      fc[c] = __fadd2_rn(__fadd2_rn(tt, pk(-fo[c].x, -fo[c].y)), pk(-y.x, -y.y));
      fo[c] = tt;
    }
  }
  float a0[6], c0[6], a1[6], c1[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    a0[c] = fo[c].x;
    c0[c] = fc[c].x;
    a1[c] = fo[c].y;
    c1[c] = fc[c].y;
  }
  if (P.kgs > 1) {  // a part: leave the sums, the last part combines
    const int slot = blk_slot(P, bk);
    float* mine = kpart_set(b, P, slot, wk.y);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      mine[t * 12 + c] = a0[c];
      mine[t * 12 + 6 + c] = c0[c];
      mine[(t + kPartBlock / 2) * 12 + c] = a1[c];
      mine[(t + kPartBlock / 2) * 12 + 6 + c] = c1[c];
    }
    __threadfence();
    __syncthreads();
    if (t == 0) last = atomicAdd(&b.kgdone[slot], 1) == P.kgs - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    kpart_combine(b, P, slot, t, a0, c0);
    kpart_combine(b, P, slot, t + kPartBlock / 2, a1, c1);
    if (t == 0) b.kgdone[slot] = 0;
  }
  if (ok0) store_kout(b, g0, a0, c0, mx.x, my.x, mz.x);
  if (ok1) store_kout(b, g1, a1, c1, mx.y, my.y, mz.y);
}

// The same gather with one particle per thread (128 threads per block):
// twice the warps of the packed form and no paired instructions.  Every
// particle goes through the same IEEE operations in the same order as in
// the packed kernel (explicit _rn intrinsics, no contraction), so the two
// forms give identical bits and the autotuner may pick either.
__global__ void __launch_bounds__(kPartBlock) kgather1s_kernel(Batch b) {
  __shared__ int4 skn[kKBlock];
  __shared__ float4 skv[kKBlock];
  __shared__ float2 sks[kKBlock];
  __shared__ int last;
  const int2 wk = b.kgwork[blockIdx.x];  // (particle block, part)
  const int2 bk = b.blk[wk.x];
  const SysDev& P = b.sys[bk.x];
  if (P.nd != 1 || at_limit(b, bk.x)) return;  // other systems: kgather_kernel<ND>
  int kb, ke;
  kpart_range(P, wk.y, kb, ke);
  const int t = threadIdx.x;
  const int i0 = bk.y + t;
  const bool ok0 = i0 < P.part_off + P.n;
  const int ND_all = b.ndtot;
  const int g0 = ok0 ? P.dip_off + (i0 - P.part_off) : 0;
  const uint32_t ux0 = b.dfx[g0], uy0 = b.dfx[ND_all + g0], uz0 = b.dfx[2 * ND_all + g0];
  const float mx = ok0 ? b.dm[g0] : 0.f, my = ok0 ? b.dm[ND_all + g0] : 0.f,
              mz = ok0 ? b.dm[2 * ND_all + g0] : 0.f;
  float fo[6], fc[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) fo[c] = fc[c] = 0.f;
  uint32_t ph = 0u;
  bool have = false;
  for (int k0 = kb; k0 < ke; k0 += kKBlock) {
    const int nk = min(kKBlock, ke - k0);
    __syncthreads();
    for (int q = t; q < nk; q += kPartBlock) {
      skn[q] = b.kn[P.k_off + k0 + q];
      skv[q] = b.kv[P.k_off + k0 + q];
      sks[q] = b.kS[P.k_off + k0 + q];
    }
    __syncthreads();
    float ft[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) ft[c] = 0.f;
#pragma unroll 2
    for (int q = 0; q < nk; ++q) {
      const int4 n = skn[q];
      const float4 kv = skv[q];
      const float2 vS = sks[q];
      float c, sn;
      ph = phase_next(ph, have, ux0, uy0, uz0, n);
      have = true;
      phase_cs(ph, c, sn);
      const float a = __fmaf_rn(mz, kv.z, __fmaf_rn(my, kv.y, __fmul_rn(mx, kv.x)));
      const float va = __fmul_rn(kv.w, a);
      const float Dr = __fmaf_rn(-va, c, vS.x);
      const float Dn = __fmaf_rn(va, sn, vS.y);
      const float fF = __fmul_rn(a, __fmaf_rn(c, Dn, __fmul_rn(sn, Dr)));
      const float fT = __fmaf_rn(sn, Dn, __fmul_rn(-c, Dr));
      ft[0] = __fmaf_rn(fF, kv.x, ft[0]);
      ft[1] = __fmaf_rn(fF, kv.y, ft[1]);
      ft[2] = __fmaf_rn(fF, kv.z, ft[2]);
      ft[3] = __fmaf_rn(fT, kv.x, ft[3]);
      ft[4] = __fmaf_rn(fT, kv.y, ft[4]);
      ft[5] = __fmaf_rn(fT, kv.z, ft[5]);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const float y = __fadd_rn(ft[c], -fc[c]);
      const float tt = __fadd_rn(fo[c], y);
      fc[c] = __fadd_rn(__fadd_rn(tt, -fo[c]), -y);
      fo[c] = tt;
    }
  }
  if (P.kgs > 1) {  // a part: leave the sums, the last part combines
    const int slot = blk_slot(P, bk);
    float* mine = kpart_set(b, P, slot, wk.y) + t * 12;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      mine[c] = fo[c];
      mine[6 + c] = fc[c];
    }
    __threadfence();
    __syncthreads();
    if (t == 0) last = atomicAdd(&b.kgdone[slot], 1) == P.kgs - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    kpart_combine(b, P, slot, t, fo, fc);
    if (t == 0) b.kgdone[slot] = 0;
  }
  if (ok0) store_kout(b, g0, fo, fc, mx, my, mz);
}

template <int ND>
static void launch_kgather(const Batch& b, cudaStream_t s) {
  if (b.tune.kg_scalar)
    kgather1s_kernel<<<b.nkgwork, kPartBlock, 0, s>>>(b);
  else
    kgather1_kernel<<<b.nkgwork, kPartBlock / 2, 0, s>>>(b);
  if (ND > 1) kgather_kernel<ND><<<b.nblk, kPartBlock, 0, s>>>(b);
}

template <int ND>
static void launch_kspace_nd(const Batch& b, const int4* kwork, int nkwork, const int2* kowner,
                             double* kE, cudaStream_t s) {
  if (b.nktot == 0) return;
  if (nkwork > 0) launch_ksum<ND>(b, kwork, nkwork, s);
  kcombine_kernel<ND><<<cdiv(b.nktot, 128), 128, 0, s>>>(b, kowner, kE);
  launch_kgather<ND>(b, s);
}

template <int ND>
static void kspace_part_nd(const Batch& b, const int4* kwork, int nkwork, const int2* kowner,
                           double* kE, int part, cudaStream_t s) {
  if (b.nktot == 0) return;
  if (part == 0 && nkwork > 0) launch_ksum<ND>(b, kwork, nkwork, s);
  if (part == 1) kcombine_kernel<ND><<<cdiv(b.nktot, 128), 128, 0, s>>>(b, kowner, kE);
  if (part == 2) launch_kgather<ND>(b, s);
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
