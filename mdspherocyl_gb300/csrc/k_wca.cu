// Verlet list, WCA core forces and cluster bonds -- the GPU form of
// neigh_list / check_list (v25/functions.cpp:1298-1394), force_sc
// (:1397-1553) and the cluster criterion of clust_conf (:2987-3016), plus
// an energy criterion for clusters (pair energy below a threshold).
//
// List: each particle keeps every partner (both directions, ascending
// index) whose segment distance is below r_list = max(2^(1/6) sigma_max,
// sigma_max + min_s) + skin.  It is rebuilt when any rod end may have moved
// by more than skin/2 since the last build (centre displacement plus half
// the length times the axis change); the reference's own test looks at the
// centres only (v25/functions.cpp:1386-1387), which is not enough once the
// list radius is tight.  The build scans every particle of the system in
// FP32 (fixed-point separations, exact minimum image).  Systems of
// kCellMinRods rods or more whose box holds at least 3 cells along every
// axis bin their rods into cells no smaller than the largest reach of a
// list entry and scan only the 27 cells around each rod's own: O(N) per
// build instead of O(N^2).  A cell's rods are staged in cell order (the
// fixed-point position with the rod's index, and the axis with the
// length), and the two warps of a cell read each neighbour cell's slots
// together, the same address across the warp.  The tests are the same FP32
// expressions on the same values as the all-pairs scan, and each list is
// sorted by index before it is written, so both scans give the same lists.
//
// WCA: the force is non-zero only for segment distance < 2^(1/6) sigma_ij.
// A pair is first screened in FP32; pairs that pass are evaluated exactly as
// the reference does, in FP64 and with the reference's segment-distance
// routine and sentinels, always with the lower index as particle i so both
// members of a pair see the same numbers.  Each particle sums its own pairs
// in ascending partner order -- the order in which force_sc adds them.
#include "mdsc_dev.cuh"
#include "reduce.cuh"
#include "seg_dist.cuh"
#include "wca_screen.cuh"

namespace mdsc {

// Rebuild decision of every system (the same in every block of a system),
// and, for a system that rebuilds on cells, its cell counts zeroed.
__global__ void __launch_bounds__(kPartBlock) list_prep_kernel(Batch b, int force_all) {
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  SysState& S = b.st[bk.x];
  bool need = (force_all || S.force_list) && !at_limit(b, bk.x);
  if (!need && !at_limit(b, bk.x)) {
    double m = 0.0;
    for (int k = 0; k < P.nblk; ++k) m = fmax(m, b.dmax[P.blk_off + k]);
    need = 2.0 * m > P.skin;
  }
  const int j = blk_slot(P, bk) - P.blk_off;
  if (j == 0 && threadIdx.x == 0) {
    S.rebuild = need ? 1 : 0;
    S.cell_ovf = 0;
  }
  if (!need || P.ncell == 0) return;
  for (int c = j * kPartBlock + threadIdx.x; c < P.ncell; c += P.nblk * kPartBlock) b.ccnt[P.cell_off + c] = 0;
}

// cell of a fixed-point position: floor(fraction x cells), exact
__device__ __forceinline__ int cell_of(const SysDev& P, uint32_t ux, uint32_t uy, uint32_t uz) {
  const int cx = (int)(((unsigned long long)ux * (unsigned)P.cnx) >> 32);
  const int cy = (int)(((unsigned long long)uy * (unsigned)P.cny) >> 32);
  const int cz = (int)(((unsigned long long)uz * (unsigned)P.cnz) >> 32);
  return (cz * P.cny + cy) * P.cnx + cx;
}

// Each rod of a rebuilding cell system into a slot of its cell (any order).
__global__ void __launch_bounds__(kPartBlock) cell_bin_kernel(Batch b) {
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  SysState& S = b.st[bk.x];
  if (!S.rebuild || P.ncell == 0) return;
  const int i = bk.y + threadIdx.x;
  if (i >= P.part_off + P.n) return;
  const int N = b.ntot;
  const uint32_t ux = b.pfx[i], uy = b.pfx[N + i], uz = b.pfx[2 * N + i];
  const int c = P.cell_off + cell_of(P, ux, uy, uz);
  const int slot = atomicAdd(&b.ccnt[c], 1);
  if (slot < kCellSlots) {
    b.cpos[(long long)c * kCellSlots + slot] = make_uint4(ux, uy, uz, (uint32_t)i);
    b.cax[(long long)c * kCellSlots + slot] = b.pax[i];
  } else {
    atomicExch(&S.cell_ovf, 1);
  }
}

// ascending insertion sort of a short list
template <class A>
__device__ __forceinline__ void sort_small(A& v, int n) {
  for (int a = 1; a < n; ++a) {
    const int x = v[a];
    int c = a - 1;
    while (c >= 0 && v[c] > x) {
      v[c + 1] = v[c];
      --c;
    }
    v[c + 1] = x;
  }
}

// The cell scan: blocks of two cells (two warps each), a thread per slot.
__device__ void list_cells(const Batch& b) {
  const int2 cb = b.cellblk[blockIdx.x - b.nblk];
  const SysDev& P = b.sys[cb.x];
  SysState& S = b.st[cb.x];
  if (!S.rebuild || P.ncell == 0 || S.cell_ovf) return;
  const int c = cb.y + (threadIdx.x >> 6);
  if (c >= P.ncell) return;
  const int t = threadIdx.x & 63;
  const int cnt0 = b.ccnt[P.cell_off + c];
  const bool ok = t < cnt0;
  uint4 me = make_uint4(0u, 0u, 0u, 0u);
  float4 ai = make_float4(0.f, 0.f, 1.f, 0.f);
  if (ok) {
    me = b.cpos[(long long)(P.cell_off + c) * kCellSlots + t];
    ai = b.cax[(long long)(P.cell_off + c) * kCellSlots + t];
  }
  const int i = (int)me.w;
  const float rl = (float)P.r_list;
  const float rl2 = rl * rl;
  const float Lx = P.Lfix[0], Ly = P.Lfix[1], Lz = P.Lfix[2];
  const bool rcut = P.rc_real > 0.0;
  int lst[kMaxNb];
  int cnt = 0, rcnt = 0;
  int* rout = b.rnb + (long long)i * kMaxR;
  const int cx = c % P.cnx, cy = (c / P.cnx) % P.cny, cz = c / (P.cnx * P.cny);
  for (int dz = -1; dz <= 1; ++dz) {
    const int qz = (cz + dz + P.cnz) % P.cnz;
    for (int dy = -1; dy <= 1; ++dy) {
      const int qy = (cy + dy + P.cny) % P.cny;
      for (int dx0 = -1; dx0 <= 1; ++dx0) {
        const int qx = (cx + dx0 + P.cnx) % P.cnx;
        const long long q = P.cell_off + (qz * P.cny + qy) * P.cnx + qx;
        const int m = b.ccnt[q];
        const uint4* cp = b.cpos + q * kCellSlots;
        const float4* ca = b.cax + q * kCellSlots;
        for (int k = 0; k < m; ++k) {
          const uint4 pj = cp[k];
          const float4 aj = ca[k];
          if (!ok || pj.w == me.w) continue;
          const float dx = fix_diff(me.x, pj.x, Lx);
          const float dy = fix_diff(me.y, pj.y, Ly);
          const float dz2 = fix_diff(me.z, pj.z, Lz);
          const float r2 = dx * dx + dy * dy + dz2 * dz2;
          if (rcut && r2 < P.rl_r2) {
            if (rcnt < kMaxR) rout[rcnt] = (int)pj.w;
            ++rcnt;
          }
          const float reach = rl + 0.5f * (ai.w + aj.w);
          if (!(r2 < reach * reach)) continue;
          const float d2 = seg_dist_fast(dx, dy, dz2, ai.x, ai.y, ai.z, ai.w, aj.x, aj.y, aj.z, aj.w);
          if (d2 < rl2) {
            if (cnt < kMaxNb) lst[cnt] = (int)pj.w;
            ++cnt;
          }
        }
      }
    }
  }
  if (!ok) return;
  int err = (cnt > kMaxNb || rcnt > kMaxR) ? kErrListOverflow : 0;
  cnt = min(cnt, kMaxNb);
  sort_small(lst, cnt);
  int* out = b.nb + (long long)i * kMaxNb;
  for (int k = 0; k < cnt; ++k) out[k] = lst[k];
  b.nbc[i] = cnt;
  if (rcut) {
    rcnt = min(rcnt, kMaxR);
    sort_small(rout, rcnt);
    b.rnbc[i] = rcnt;
  }
  if (err) atomicOr(&S.status, err);
  const int N = b.ntot;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    b.fsave[3 * i + a] = b.pfx[a * N + i];
    b.usave[3 * i + a] = a == 0 ? ai.x : (a == 1 ? ai.y : ai.z);
  }
}

// The list build: blocks below nblk scan all pairs of their particle block
// (systems without cells, or whose cells overflowed this build); the rest
// scan cells.
__global__ void __launch_bounds__(kPartBlock) list_build_kernel(Batch b) {
  __shared__ uint32_t sx[kPartBlock], sy[kPartBlock], sz[kPartBlock];
  __shared__ float4 sa[kPartBlock];
  if ((int)blockIdx.x >= b.nblk) {
    list_cells(b);
    return;
  }
  const int2 bk = b.blk[blockIdx.x];
  const int s = bk.x;
  const SysDev& P = b.sys[s];
  SysState& S = b.st[s];
  if (!S.rebuild || (b.cells && P.ncell > 0 && !S.cell_ovf)) return;
  const int i = bk.y + threadIdx.x;
  const bool ok = i < P.part_off + P.n;
  const int N = b.ntot;
  uint32_t ux = 0, uy = 0, uz = 0;
  float4 ai = make_float4(0.f, 0.f, 1.f, 0.f);
  if (ok) {
    ux = b.pfx[i];
    uy = b.pfx[N + i];
    uz = b.pfx[2 * N + i];
    ai = b.pax[i];
  }
  const float rl = (float)P.r_list;
  const float rl2 = rl * rl;
  const float Lx = P.Lfix[0], Ly = P.Lfix[1], Lz = P.Lfix[2];
  const int first = P.part_off, n = P.n;
  int cnt = 0;
  int* out = b.nb + (long long)i * kMaxNb;
  // real-space neighbours (systems with a real-space cutoff): every rod whose
  // centre is within rl_r2, in ascending order, both directions
  const bool rcut = P.rc_real > 0.0;
  int rcnt = 0;
  int* rout = b.rnb + (long long)i * kMaxR;
  for (int q0 = 0; q0 < n; q0 += kPartBlock) {
    const int nq = min(kPartBlock, n - q0);
    __syncthreads();
    if (threadIdx.x < nq) {
      const int q = first + q0 + threadIdx.x;
      sx[threadIdx.x] = b.pfx[q];
      sy[threadIdx.x] = b.pfx[N + q];
      sz[threadIdx.x] = b.pfx[2 * N + q];
      sa[threadIdx.x] = b.pax[q];
    }
    __syncthreads();
    if (!ok) continue;
    if (rcut) {
      for (int k = 0; k < nq; ++k) {
        const float dx = fix_diff(ux, sx[k], Lx);
        const float dy = fix_diff(uy, sy[k], Ly);
        const float dz = fix_diff(uz, sz[k], Lz);
        if (dx * dx + dy * dy + dz * dz < P.rl_r2 && first + q0 + k != i) {
          if (rcnt < kMaxR) rout[rcnt] = first + q0 + k;
          ++rcnt;
        }
      }
    }
    // 1. centre distance against the reach of the two rods, branch-free,
    //    into a mask of the chunk's 128 candidates: nearly every warp has a
    //    lane with some candidate in reach, so testing the segments inside
    //    this loop would run the segment routine for every candidate
    uint32_t m[4];
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      uint32_t bits = 0u;
#pragma unroll 8
      for (int kk = 0; kk < 32; ++kk) {
        const int k = 32 * w + kk;
        const float dx = fix_diff(ux, sx[k], Lx);
        const float dy = fix_diff(uy, sy[k], Ly);
        const float dz = fix_diff(uz, sz[k], Lz);
        const float reach = rl + 0.5f * (ai.w + sa[k].w);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const bool in = k < nq && r2 < reach * reach && first + q0 + k != i;
        bits |= (uint32_t)in << kk;
      }
      m[w] = bits;
    }
    // 2. segment distance of the candidates in reach, in ascending order
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      for (uint32_t bits = m[w]; bits; bits &= bits - 1u) {
        const int k = 32 * w + __ffs(bits) - 1;
        const float dx = fix_diff(ux, sx[k], Lx);
        const float dy = fix_diff(uy, sy[k], Ly);
        const float dz = fix_diff(uz, sz[k], Lz);
        const float4 aj = sa[k];
        const float d2 = seg_dist_fast(dx, dy, dz, ai.x, ai.y, ai.z, ai.w, aj.x, aj.y, aj.z, aj.w);
        if (d2 < rl2) {
          if (cnt < kMaxNb) out[cnt] = first + q0 + k;
          ++cnt;
        }
      }
    }
  }
  if (!ok) return;
  int err = (cnt > kMaxNb || rcnt > kMaxR) ? kErrListOverflow : 0;
  b.nbc[i] = min(cnt, kMaxNb);
  if (rcut) {
    b.rnbc[i] = min(rcnt, kMaxR);
  }
  if (err) atomicOr(&S.status, err);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    b.fsave[3 * i + a] = b.pfx[a * N + i];
    b.usave[3 * i + a] = a == 0 ? ai.x : (a == 1 ? ai.y : ai.z);
  }
}

__device__ __forceinline__ void load_rod(const Batch& b, int i, RodD& R) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    R.r[a] = b.r[3 * i + a];
    R.o[a] = b.O[9 * i + 6 + a];
  }
  R.len = b.len[i];
}

// WCA pair (v25/functions.cpp:1438-1540) for A < B; returns false when the
// pair does not interact.  fA: force on A; tA, tB: torques; ev: U, W and
// the pressure tensor.  This file is compiled without FMA contraction (the
// cluster test must repeat the reference's roundings); the force path asks
// for its FMAs explicitly.
__device__ bool wca_pair(const Batch& b, const SysDev& P, int A, int B, double* fA, double* tA,
                         double* tB, double* ev, int& err) {
  RodD ra, rb;
  load_rod(b, A, ra);
  load_rod(b, B, rb);
  const double shA0 = ra.len, shB0 = rb.len;
  const double sigma = (b.dia[A] + b.dia[B]) / 2;
  const double sig_sq = sigma * sigma;
  const double srt = 1.122462048309373;   // 2^(1/6)
  const double rsh = srt * srt * sig_sq;
  double rij[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    rij[a] = ra.r[a] - rb.r[a];
    rij[a] = fma(-P.L[a], floor(fma(rij[a], P.invL[a], 0.5)), rij[a]);
  }
  const double rsq = fma(rij[2], rij[2], fma(rij[1], rij[1], rij[0] * rij[0]));
  double dij[3], st[2];
  const double dsq = seg_dist_wca(ra, rb, P.L, rij, dij, st);
  if (dsq < 0.49 * sig_sq || dsq > rsq * 1.00001) err |= kErrOverlap;
  if (!(dsq < rsh)) return false;
  // one reciprocal instead of the reference's three divisions; FIJ = W / ddr
  // reduces to 6 (pot + 4 SR6^2) / dsq, NaN where ddr = 0 as in the reference
  const double inv_dsq = 1.0 / dsq;
  const double SR2s = sig_sq * inv_dsq;
  const double SR6s = SR2s * SR2s * SR2s;
  const double pot = fma(4 * SR6s, SR6s, -4 * SR6s);
  const double ddr = fma(rij[2], dij[2], fma(rij[1], dij[1], rij[0] * dij[0]));
  const double fw = 6 * fma(4 * SR6s, SR6s, pot) * inv_dsq;
  const double FIJ = (ddr != 0.0) ? fw : __longlong_as_double(0x7ff8000000000000LL);
  if (!(fabs(FIJ) < 1e300)) err |= kErrNan;
  ev[0] = pot + 1.;
  ev[1] = fw * ddr;
#pragma unroll
  for (int a = 0; a < 3; ++a) fA[a] = FIJ * dij[a];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) ev[2 + 3 * a + c] = rij[a] * fA[c];
  const double *oi = ra.o, *oj = rb.o;
  const double icroj[3] = {fma(oi[1], oj[2], -oi[2] * oj[1]), fma(oi[2], oj[0], -oi[0] * oj[2]),
                           fma(oi[0], oj[1], -oi[1] * oj[0])};
  const double icror[3] = {fma(oi[1], rij[2], -oi[2] * rij[1]), fma(oi[2], rij[0], -oi[0] * rij[2]),
                           fma(oi[0], rij[1], -oi[1] * rij[0])};
  const double jcror[3] = {fma(oj[1], rij[2], -oj[2] * rij[1]), fma(oj[2], rij[0], -oj[0] * rij[2]),
                           fma(oj[0], rij[1], -oj[1] * rij[0])};
  double fact1 = (st[0] - 0.5) * shA0;
  double fact2 = -(st[1] - 0.5) * shB0;
  if (st[0] == -1.e+6) fact1 = fact2 = 0.;
  // as in the reference, -3e10 is tested twice (v25/functions.cpp:1526,1529),
  // so the (-/+) end-point sentinel keeps the lever arms computed above
  if (st[0] == -1.e+10) {
    fact1 = 0.5 * shA0;
    fact2 = 0.5 * shB0;
  } else if (st[0] == -2.e+10) {
    fact1 = -0.5 * shA0;
    fact2 = -0.5 * shB0;
  } else if (st[0] == -3.e+10) {
    fact1 = 0.5 * shA0;
    fact2 = -0.5 * shB0;
  }
  const double fmul = fact1 * fact2;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    tA[a] = FIJ * fma(fact1, icror[a], fmul * icroj[a]);
    tB[a] = FIJ * fma(fact2, jcror[a], -fmul * icroj[a]);
  }
  return true;
}

// WCA in two kernels.  (1) wca_screen: each thread screens its particle's
// partners of higher index (each pair once) in FP32, keeps the candidates in
// ascending index in its slots (wcand) and appends (slot, system) items to
// a work list, one atomic per warp.  (2) wca_eval: every thread of a fixed
// grid takes list items and evaluates them in FP64 -- only pairs that can
// touch reach the FP64 unit (1/64 of the FP32 rate on this GPU), densely
// packed, with no block-wide synchronisation.  Each item writes its own
// share (force and torque on the lower index), its partner's share and its
// energy/virial terms to the candidate's slot.  The finalize kernel adds a
// particle's own shares in slot order and its partners' shares in partner
// order, and the per-system reduction adds the slots' energies in particle
// and slot order, so the list order (which depends on warp timing) does not
// reach any result.
__global__ void __launch_bounds__(kPartBlock) wca_screen_kernel(Batch b) {
  const int2 bk = b.blk[blockIdx.x];
  const int s = bk.x;
  const SysDev& P = b.sys[s];
  if (P.rc_real > 0.0 || at_limit(b, s)) return;  // cutoff systems: screened in their neighbour pass
  const int i = bk.y + threadIdx.x;
  const bool ok = i < P.part_off + P.n;
  const int nl = ok ? b.nbc[i] : 0;
  const int* lst = b.nb + (long long)i * kMaxNb;
  int k = 0;
  wca_screen_one(b, P, s, i, ok, [&]() { return k < nl ? lst[k++] : -1; });
}

__global__ void __launch_bounds__(128) wca_eval_kernel(Batch b) {
  const int n = *(volatile const int*)b.wlist_n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int2 it = b.wlist[e];
    const int slot = it.x, s = it.y;
    const int p = slot / kMaxC;
    const SysDev& P = b.sys[s];
    const int q = b.wcand[slot];
    int err = 0;
    double fA[3], tA[3], tB[3], ev[11];
    if (!wca_pair(b, P, p, q, fA, tA, tB, ev, err)) {
#pragma unroll
      for (int a = 0; a < 3; ++a) fA[a] = tA[a] = tB[a] = 0.0;
#pragma unroll
      for (int c = 0; c < 11; ++c) ev[c] = 0.0;
    }
    double* own = b.wown + (long long)slot * 6;
    double* rec = b.wrec + (long long)slot * 6;
    double* evo = b.wev + (long long)slot * 11;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      own[a] = fA[a];
      own[3 + a] = tA[a];
      rec[a] = -fA[a];
      rec[3 + a] = tB[a];
    }
#pragma unroll
    for (int c = 0; c < 11; ++c) evo[c] = ev[c];
    if (err) atomicOr(&b.st[s].status, err);
  }
}

// ---- clusters (v25/functions.cpp:2987-3016,3282-3324) ----------------
// bond flags for list entries q > i: segment distance < (D_i + D_j)/2 + min_s,
// evaluated in FP64 with the reference's routine (lower index first)
__global__ void __launch_bounds__(kPartBlock) cluster_bonds_kernel(Batch b) {
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  const int i = bk.y + threadIdx.x;
  if (i >= P.part_off + P.n) return;
  b.comp[i] = i;
  if (P.cl_mode) return;  // energy criterion: ebond_kernel
  const int nc = b.nbc[i];
  const int* lst = b.nb + (long long)i * kMaxNb;
  unsigned char* fl = b.eflag + (long long)i * kMaxNb;
  RodD ri;
  load_rod(b, i, ri);
  for (int k = 0; k < nc; ++k) {
    const int q = lst[k];
    unsigned char bond = 0;
    if (q > i) {
      RodD rq;
      load_rod(b, q, rq);
      const double sigma = (b.dia[i] + b.dia[q]) / 2 + P.min_s;
      double rij[3], dij[3], st[2];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        rij[a] = ri.r[a] - rq.r[a];
        rij[a] -= P.L[a] * floor(rij[a] / P.L[a] + 0.5);
      }
      const double dsq = seg_dist_ref<true>(ri, rq, P.L, rij, dij, st);
      bond = dsq < sigma * sigma ? 1 : 0;
    }
    fl[k] = bond;
  }
}

// ---- energy criterion (an extension; the reference's test is geometric) --
// U_pair = the WCA pair energy of force_sc (v25/functions.cpp:1436-1483) +
// the bare dipole-dipole energy of every dipole pair of the two rods at the
// minimum image of the sites, mu_a mu_b (o_a.o_b - 3 (o_a.r)(o_b.r)/r^2)/r^3,
// in FP64 with the operations in the oracle's order (A < B; this file is
// compiled without FMA contraction, and sqrt and division round correctly).
__device__ void dip_lab_ref(const Batch& b, const SysDev& P, int i, int w, double pos[3], double ori[3],
                            double* mu) {
  const int g = P.dip_off + (i - P.part_off) * P.nd + w;
  const double* O = b.O + 9 * (long long)i;
  const double d0 = b.dpc[g];
#pragma unroll
  for (int a = 0; a < 3; ++a) pos[a] = b.r[3 * i + a] + d0 * O[6 + a];
#pragma unroll
  for (int m = 0; m < 3; ++m) {  // transpose(O) times the body direction, summed from 0
    double acc = 0.;
    acc += O[m] * b.dob[3 * g];
    acc += O[3 + m] * b.dob[3 * g + 1];
    acc += O[6 + m] * b.dob[3 * g + 2];
    ori[m] = acc;
  }
  *mu = b.dmu[g];
}

__device__ double pair_energy_ref(const Batch& b, const SysDev& P, int A, int B) {
  RodD ra, rb;
  load_rod(b, A, ra);
  load_rod(b, B, rb);
  double rij[3], dij[3], st[2];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    rij[a] = ra.r[a] - rb.r[a];
    rij[a] -= P.L[a] * floor(rij[a] / P.L[a] + 0.5);
  }
  const double dsq = seg_dist_ref<true>(ra, rb, P.L, rij, dij, st);
  const double sigma = (b.dia[A] + b.dia[B]) / 2;
  const double sig_sq = sigma * sigma;
  const double srt = 1.122462048309373;  // 2^(1/6)
  double U = 0.;
  if (dsq < srt * srt * sig_sq) {
    const double SR2s = sig_sq / dsq;
    const double SR6s = SR2s * SR2s * SR2s;
    U = 4 * SR6s * (SR6s - 1.) + 1.;
  }
  for (int a = 0; a < P.nd; ++a) {
    double pa[3], oa[3], ma;
    dip_lab_ref(b, P, A, a, pa, oa, &ma);
    if (ma == 0.) continue;
    for (int c = 0; c < P.nd; ++c) {
      double pb[3], ob[3], mb;
      dip_lab_ref(b, P, B, c, pb, ob, &mb);
      if (mb == 0.) continue;
      double r[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) r[k] = dmimg(pa[k] - pb[k], P.L[k]);
      const double r2 = ddot(r, r);
      const double ir = 1. / sqrt(r2);
      const double ir3 = ir * ir * ir;
      const double dd = ddot(oa, ob), da = ddot(oa, r), db = ddot(ob, r);
      U += ma * mb * (dd - 3. * da * db / r2) * ir3;
    }
  }
  return U;
}

// Candidates for bonds U_pair < -cl_ubond among the higher indices of the
// system: an FP32 screen on the centres (fixed-point minimum image) keeps
// the pairs that can bond, |U_dd| <= 2 M_i M_j / (r - e_i - e_j)^3 with M
// the sum of a rod's moments and e its largest dipole offset, U_WCA >= 0.
// Ascending order; ebond_eval_kernel evaluates them exactly.
__global__ void __launch_bounds__(kPartBlock) ebond_screen_kernel(Batch b) {
  __shared__ uint32_t sx[kPartBlock], sy[kPartBlock], sz[kPartBlock];
  __shared__ float2 sme[kPartBlock];
  const int2 bk = b.blk[blockIdx.x];
  const int s = bk.x;
  const SysDev& P = b.sys[s];
  if (P.cl_mode != 1) return;  // the same for the whole block
  const int first = P.part_off, n = P.n, N = b.ntot;
  const int i = bk.y + threadIdx.x;
  const bool ok = i < first + n;
  auto bound = [&](int q) {
    float m = 0.f, e = 0.f;
    for (int w = 0; w < P.nd; ++w) {
      const int g = P.dip_off + (q - first) * P.nd + w;
      const float ob = (float)sqrt(b.dob[3 * g] * b.dob[3 * g] + b.dob[3 * g + 1] * b.dob[3 * g + 1] +
                                   b.dob[3 * g + 2] * b.dob[3 * g + 2]);
      m += fabsf((float)b.dmu[g]) * ob;
      e = fmaxf(e, fabsf((float)b.dpc[g]));
    }
    return make_float2(m * 1.0001f, e * 1.0001f);
  };
  uint32_t ux = 0, uy = 0, uz = 0;
  float2 mi = make_float2(0.f, 0.f);
  if (ok) {
    ux = b.pfx[i];
    uy = b.pfx[N + i];
    uz = b.pfx[2 * N + i];
    mi = bound(i);
  }
  const float Lx = P.Lfix[0], Ly = P.Lfix[1], Lz = P.Lfix[2];
  const float thr = (float)P.cl_ubond * 0.999f;
  int* out = b.ecand + (long long)i * kMaxE;
  int cnt = 0;
  for (int q0 = (bk.y - first) / kPartBlock * kPartBlock; q0 < n; q0 += kPartBlock) {
    __syncthreads();
    if (q0 + (int)threadIdx.x < n) {
      const int q = first + q0 + threadIdx.x;
      sx[threadIdx.x] = b.pfx[q];
      sy[threadIdx.x] = b.pfx[N + q];
      sz[threadIdx.x] = b.pfx[2 * N + q];
      sme[threadIdx.x] = bound(q);
    }
    __syncthreads();
    if (!ok || mi.x == 0.f) continue;
    const int nq = min(kPartBlock, n - q0);
    for (int t = 0; t < nq; ++t) {
      const int j = first + q0 + t;
      const float2 mj = sme[t];
      const float dx = fix_diff(ux, sx[t], Lx), dy = fix_diff(uy, sy[t], Ly), dz = fix_diff(uz, sz[t], Lz);
      const float gap = sqrtf(dx * dx + dy * dy + dz * dz) * 0.9999f - mi.y - mj.y;
      const bool cand = j > i && mj.x != 0.f && (gap <= 0.f || 2.f * mi.x * mj.x >= thr * gap * gap * gap);
      if (cand) {
        if (cnt < kMaxE) out[cnt] = j;
        ++cnt;
      }
    }
  }
  if (ok) {
    b.ecnt[i] = min(cnt, kMaxE);
    if (cnt > kMaxE) atomicOr(&b.eovf[s], 1);
  }
}

// the screened candidates of each rod, exactly: a bond where the FP64 pair
// energy (pair_energy_ref, lower index first) is below -cl_ubond
__global__ void __launch_bounds__(kPartBlock) ebond_eval_kernel(Batch b) {
  const int2 bk = b.blk[blockIdx.x];
  const int s = bk.x;
  const SysDev& P = b.sys[s];
  if (P.cl_mode != 1) return;
  const int i = bk.y + threadIdx.x;
  if (i >= P.part_off + P.n) return;
  const int nc = b.ecnt[i];
  const int* cand = b.ecand + (long long)i * kMaxE;
  int* out = b.ebond + (long long)i * kMaxC;
  int cnt = 0;
  for (int k = 0; k < nc; ++k) {
    const int j = cand[k];
    if (pair_energy_ref(b, P, i, j) < -P.cl_ubond) {
      if (cnt < kMaxC) out[cnt] = j;
      ++cnt;
    }
  }
  b.ebcnt[i] = min(cnt, kMaxC);
  if (cnt > kMaxC) atomicOr(&b.eovf[s], 1);
}

__device__ __forceinline__ int find_root(const int* comp, int x) {
  int p = comp[x];
  while (p != x) {
    x = p;
    p = comp[x];
  }
  return x;
}

// hook: for every bond, attach the larger root to the smaller one
__global__ void __launch_bounds__(kPartBlock) cluster_hook_kernel(Batch b) {
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  const int i = bk.y + threadIdx.x;
  if (i >= P.part_off + P.n) return;
  const bool en = P.cl_mode == 1;
  const int nc = en ? b.ebcnt[i] : b.nbc[i];
  const int* lst = en ? b.ebond + (long long)i * kMaxC : b.nb + (long long)i * kMaxNb;
  const unsigned char* fl = en ? nullptr : b.eflag + (long long)i * kMaxNb;
  for (int k = 0; k < nc; ++k) {
    if (fl && !fl[k]) continue;
    int ra = find_root(b.comp, i), rb = find_root(b.comp, lst[k]);
    while (ra != rb) {
      const int hi = max(ra, rb), lo = min(ra, rb);
      const int old = atomicMin(&b.comp[hi], lo);
      if (old == hi) {
        *b.flag = 1;
        break;
      }
      ra = find_root(b.comp, old);
      rb = find_root(b.comp, lo);
    }
  }
}

__global__ void __launch_bounds__(kPartBlock) cluster_compress_kernel(Batch b) {
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  const int i = bk.y + threadIdx.x;
  if (i >= P.part_off + P.n) return;
  b.comp[i] = find_root(b.comp, i);
}

void launch_list_build(const Batch& b, int force_all, cudaStream_t s) {
  if (!b.nblk) return;
  list_prep_kernel<<<b.nblk, kPartBlock, 0, s>>>(b, force_all);
  const int ncb = b.cells ? b.ncellblk : 0;
  if (ncb) cell_bin_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
  list_build_kernel<<<b.nblk + ncb, kPartBlock, 0, s>>>(b);
}
void launch_near_pass(const Batch& b, int mode, cudaStream_t s);  // k_real.cu

void launch_wca(const Batch& b, int near_mode, cudaStream_t s) {
  if (!b.nblk) return;
  cudaMemsetAsync(b.wlist_n, 0, sizeof(int), s);
  cudaMemsetAsync(b.wincnt, 0, sizeof(int) * b.ntot, s);
  // cutoff systems: the WCA screen over their Verlet list in their
  // neighbour pass (with their real space when near_mode says so); the
  // others: in the screen kernel
  launch_near_pass(b, 2 | near_mode, s);
  wca_screen_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
  // a fixed grid (chosen by the autotuner); each thread loops over the list
  wca_eval_kernel<<<b.tune.wca_blocks, 128, 0, s>>>(b);
}
void launch_cluster_bonds(const Batch& b, cudaStream_t s) {
  if (b.nblk) cluster_bonds_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
}
void launch_ebond(const Batch& b, cudaStream_t s) {
  if (!b.nblk || !b.ecand) return;
  ebond_screen_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
  ebond_eval_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
}
void launch_cluster_hook(const Batch& b, cudaStream_t s) {
  if (b.nblk) cluster_hook_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
}
void launch_cluster_compress(const Batch& b, cudaStream_t s) {
  if (b.nblk) cluster_compress_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
}

}  // namespace mdsc
