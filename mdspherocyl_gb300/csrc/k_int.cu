// Integrator, force assembly and per-system reductions -- the GPU form of
// moveTher / moveP / moveX / renorm / ext_field and of the driver's
// bookkeeping (v25/functions.cpp:1992-2025,2071-2218; v25/classes.cpp:228-325;
// v25/main.cpp:558-649).
//
// Precision: the master state (r, p, l, O, F, T) is FP64.  FP64 runs at a
// small fraction of the FP32 rate on this GPU, so the free-rotor update
// (five plane rotations in the body frame, J. Chem. Phys. 107, 5840, as
// Spherocyl::rotate does) is composed in FP32 as M = I + D, with every
// rotation entered as cos-1 = -2 sin^2(a/2) and sin a so that D keeps full
// FP32 *relative* precision (|D| ~ 1e-3 -> ~1e-10 absolute), and is applied
// to the FP64 orientation as O += D O.  Kicks, drifts and the thermostat
// scalars stay in FP64.
#include <algorithm>
#include <vector>

#include "mdsc_dev.cuh"
#include "reduce.cuh"

namespace mdsc {

// ---------------------------------------------------------------------
// working copies: fixed-point positions, FP32 axes and dipole vectors
// ---------------------------------------------------------------------
__device__ __forceinline__ void derive_particle(const Batch& b, const SysDev& P, int i,
                                                const double* r, const double* O, uint32_t* u) {
  const int N = b.ntot, ND = b.ndtot;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    u[a] = to_fix(r[a], P.invL32[a]);
    b.pfx[a * N + i] = u[a];
  }
  // FP32 copies by integer instructions (the FP64 unit is the scarce one)
  float Of[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Of[k] = soft_d2f_rn(O[k]);
  b.pax[i] = make_float4(Of[6], Of[7], Of[8], soft_d2f_rn(b.len[i]));
  b.pdia[i] = soft_d2f_rn(b.dia[i]);
  const int nd = P.nd;
  const int g0 = P.dip_off + (i - P.part_off) * nd;
  for (int w = 0; w < nd; ++w) {
    const int g = g0 + w;
    const double pc = b.dpc[g];
    if (pc == 0.0) {
#pragma unroll
      for (int a = 0; a < 3; ++a) b.dfx[a * ND + g] = u[a];
    } else {
#pragma unroll
      for (int a = 0; a < 3; ++a) b.dfx[a * ND + g] = to_fix(r[a] + pc * O[6 + a], P.invL32[a]);
    }
    // lab direction O^T o_body (Spherocyl::set_dip, v25/classes.cpp:166-170), times the moment
    const float ox = soft_d2f_rn(b.dob[3 * g]), oy = soft_d2f_rn(b.dob[3 * g + 1]),
                oz = soft_d2f_rn(b.dob[3 * g + 2]);
    const float mu = soft_d2f_rn(b.dmu[g]);
#pragma unroll
    for (int a = 0; a < 3; ++a) b.dm[a * ND + g] = mu * (Of[a] * ox + Of[3 + a] * oy + Of[6 + a] * oz);
  }
}

// how far the rod's ends may have moved since the last list build: the
// centre's move from the fixed-point coordinates (exact minimum image, no
// FP64 arithmetic) plus half the length times the axis change
__device__ __forceinline__ float displacement(const Batch& b, const SysDev& P, int i, const uint32_t* u,
                                              const double* O) {
  float dr2 = 0.f, du2 = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float d = fix_diff(u[a], b.fsave[3 * i + a], P.Lfix[a]);
    const float e = soft_d2f_rn(O[6 + a]) - b.usave[3 * i + a];
    dr2 += d * d;
    du2 += e * e;
  }
  return sqrtf(dr2) + 0.5f * soft_d2f_rn(b.len[i]) * sqrtf(du2);
}

__global__ void __launch_bounds__(kPartBlock) derive_kernel(Batch b) {
  __shared__ float shm[kPartBlock / 32];
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  const int i = bk.y + threadIdx.x;
  float disp = 0.f;
  if (i < P.part_off + P.n) {
    double r[3], O[9];
#pragma unroll
    for (int a = 0; a < 3; ++a) r[a] = b.r[3 * i + a];
#pragma unroll
    for (int k = 0; k < 9; ++k) O[k] = b.O[9 * i + k];
    uint32_t u[3];
    derive_particle(b, P, i, r, O, u);
    disp = displacement(b, P, i, u, O);
  }
  const float m = block_max<kPartBlock>(disp, shm);
  if (threadIdx.x == 0) b.dmax[blk_slot(P, bk)] = soft_f2d(m);
}

// Spherocyl::renorm, v25/classes.cpp:307-325
__device__ __forceinline__ void renorm_O(double* o) {
  double norm = sqrt(o[6] * o[6] + o[7] * o[7] + o[8] * o[8]);
  o[6] /= norm; o[7] /= norm; o[8] /= norm;
  const double Up[3] = {o[6] + o[3], o[7] + o[4], o[8] + o[5]};
  const double d = Up[0] * o[6] + Up[1] * o[7] + Up[2] * o[8];
  o[3] = Up[0] - d * o[6];
  o[4] = Up[1] - d * o[7];
  o[5] = Up[2] - d * o[8];
  norm = sqrt(o[3] * o[3] + o[4] * o[4] + o[5] * o[5]);
  o[3] /= norm; o[4] /= norm; o[5] /= norm;
  o[0] = o[4] * o[8] - o[7] * o[5];
  o[1] = o[5] * o[6] - o[8] * o[3];
  o[2] = o[3] * o[7] - o[6] * o[4];
}

// one plane rotation of the composition: rows/components (i, j) turn by a
__device__ __forceinline__ void plane_rot(float a, int i, int j, float* lb, float* D) {
  float sh, ch;
  sincosf(0.5f * a, &sh, &ch);
  const float s = 2.f * sh * ch;
  const float cm1 = -2.f * sh * sh;  // cos a - 1 with full relative precision
  const float li = lb[i], lj = lb[j];
  lb[i] = li + (cm1 * li - s * lj);
  lb[j] = lj + (s * li + cm1 * lj);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float di = D[3 * i + c], dj = D[3 * j + c];
    float ni = di + (cm1 * di - s * dj);
    float nj = dj + (s * di + cm1 * dj);
    if (c == i) { ni += cm1; nj += s; }
    if (c == j) { ni -= s; nj += cm1; }
    D[3 * i + c] = ni;
    D[3 * j + c] = nj;
  }
}

// translate + rotate (Spherocyl::translate / rotate, v25/classes.cpp:228-304)
__device__ __forceinline__ void move_x(const Batch& b, int i, double dt, double* r, const double* p,
                                       double* O, const double* l) {
  const double im = b.invm[i];
#pragma unroll
  for (int a = 0; a < 3; ++a) r[a] += dt * p[a] * im;
  const float iI0 = soft_d2f_rn(b.invI[3 * i]), iI1 = soft_d2f_rn(b.invI[3 * i + 1]),
              iI2 = soft_d2f_rn(b.invI[3 * i + 2]);
  const float fdt = soft_d2f_rn(dt), h = 0.5f * fdt;
  float lb[3], Of[9];
  const float lf[3] = {soft_d2f_rn(l[0]), soft_d2f_rn(l[1]), soft_d2f_rn(l[2])};
#pragma unroll
  for (int k = 0; k < 9; ++k) Of[k] = soft_d2f_rn(O[k]);
#pragma unroll
  for (int a = 0; a < 3; ++a) lb[a] = Of[3 * a] * lf[0] + Of[3 * a + 1] * lf[1] + Of[3 * a + 2] * lf[2];
  float D[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) D[k] = 0.f;
  plane_rot(-lb[0] * h * iI0, 1, 2, lb, D);   // Rx
  plane_rot(-lb[1] * h * iI1, 2, 0, lb, D);   // Ry
  plane_rot(-lb[2] * fdt * iI2, 0, 1, lb, D); // Rz
  plane_rot(-lb[1] * h * iI1, 2, 0, lb, D);   // Ry
  plane_rot(-lb[0] * h * iI0, 1, 2, lb, D);   // Rx
  // O += D O: the increment (|D| ~ 1e-3) in FP32, ~1e-10 absolute like D
  // itself, added to the FP64 orientation
  float inc[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) inc[3 * a + c] = D[3 * a] * Of[c] + D[3 * a + 1] * Of[3 + c] + D[3 * a + 2] * Of[6 + c];
#pragma unroll
  for (int k = 0; k < 9; ++k) O[k] += soft_f2d(inc[k]);
}

// K_r = l^T (O^T I^-1 O) l = sum_a (O l)_a^2 / I_a  (v25/functions.cpp:2123-2148)
__device__ __forceinline__ double rot_kin(const Batch& b, int i, const double* O, const double* l) {
  double kr = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double lb = O[3 * a] * l[0] + O[3 * a + 1] * l[1] + O[3 * a + 2] * l[2];
    kr += lb * lb * b.invI[3 * i + a];
  }
  return kr;
}

// thermostat coordinates used by the second half kick: moveTher 0 then 1
// (v25/functions.cpp:2193-2206), from the first-half kinetic energies of
// every block of the system (read from L2: other blocks wrote them)
__device__ __forceinline__ void xi_mid(const Batch& b, const SysDev& P, const SysState& S, int s,
                                       double* xi2, double* Kf) {
  double K0 = 0.0, K1 = 0.0;
  for (int k = 0; k < P.nblk; ++k) {
    K0 += __ldcg(&b.kin1[2 * (P.blk_off + k)]);
    K1 += __ldcg(&b.kin1[2 * (P.blk_off + k) + 1]);
  }
  Kf[0] = 0.5 * K0;
  Kf[1] = 0.5 * K1;
  const double* nz = b.noise + ((long long)S.iter * b.nsys + s) * 4;
  const double x1t = P.ex1 * S.xi[0] + P.cnoise * nz[0];
  const double x1r = P.ex1 * S.xi[1] + P.cnoise * nz[2];
  xi2[0] = x1t + P.dt * (2. * Kf[0] - P.ntemp3) / P.Q;
  xi2[1] = x1r + P.dt * (2. * Kf[1] - P.ntemp3) / P.Q;
}

// ---------------------------------------------------------------------
// first half of the step: moveTher(0), [renorm], moveP(first), moveX
// ---------------------------------------------------------------------
// 8 blocks per SM (64 registers, 76 B of spills) instead of 6 (80): the
// state reads' latency is hidden by more warps, 0.047 to 0.045 ms on the
// 256-replica mix (the same bound on finalize made it 12% slower)
__global__ void __launch_bounds__(kPartBlock, 8) integrate_first_kernel(Batch b) {
  __shared__ double sh[2 * kPartBlock / 32];
  __shared__ float shm[kPartBlock / 32];
  __shared__ double sfac[2];
  const int2 bk = b.blk[blockIdx.x];
  const int s = bk.x;
  if (at_limit(b, s)) return;
  const SysDev& P = b.sys[s];
  const SysState& S = b.st[s];
  const int i = bk.y + threadIdx.x;
  const bool ok = i < P.part_off + P.n;
  if (threadIdx.x == 0) {
    // moveTher mode 0 (v25/functions.cpp:2193-2202); noise drawn on the host
    const double* nz = b.noise + ((long long)S.iter * b.nsys + s) * 4;
    const double xt = P.ex1 * S.xi[0] + P.cnoise * nz[0];
    const double xr = P.ex1 * S.xi[1] + P.cnoise * nz[2];
    sfac[0] = 1.0 / (1.0 + 0.5 * P.dt * xt);
    sfac[1] = 1.0 / (1.0 + 0.5 * P.dt * xr);
  }
  __syncthreads();
  double kin[2] = {0.0, 0.0};
  float disp = 0.f;
  if (ok) {
    const double h = 0.5 * P.dt;
    double r[3], p[3], l[3], O[9];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      r[a] = b.r[3 * i + a];
      p[a] = b.p[3 * i + a];
      l[a] = b.l[3 * i + a];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) O[k] = b.O[9 * i + k];
    if (S.step % 100 == 0) renorm_O(O);  // v25/main.cpp:556-563
    // moveP first half (v25/functions.cpp:2129-2149)
    double psq = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      p[a] = (p[a] + h * b.F[3 * i + a]) * sfac[0];
      psq += p[a] * p[a];
      l[a] = (l[a] + h * b.T[3 * i + a]) * sfac[1];
    }
    kin[0] = psq * b.invm[i];
    kin[1] = rot_kin(b, i, O, l);
    // moveX (v25/functions.cpp:2071-2092)
    move_x(b, i, P.dt, r, p, O, l);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      b.r[3 * i + a] = r[a];
      b.p[3 * i + a] = p[a];
      b.l[3 * i + a] = l[a];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) b.O[9 * i + k] = O[k];
    uint32_t u[3];
    derive_particle(b, P, i, r, O, u);
    disp = displacement(b, P, i, u, O);
  }
  double tot[2];
  block_sum<2, kPartBlock>(kin, sh, tot);
  const float m = block_max<kPartBlock>(disp, shm);
  if (threadIdx.x == 0) {
    const int lb = blk_slot(P, bk);
    b.kin1[2 * lb] = tot[0];
    b.kin1[2 * lb + 1] = tot[1];
    b.dmax[lb] = soft_f2d(m);
    // the system's last block to finish computes the second-half thermostat
    // coordinates once (blocks' sums in block order: the same bits whichever
    // block is last) and rearms the counter
    __threadfence();
    if (atomicAdd(&b.icnt[s], 1) == P.nblk - 1) {
      __threadfence();
      SysState& Sw = b.st[s];
      double xi2[2], Kf[2];
      xi_mid(b, P, Sw, s, xi2, Kf);
      Sw.xi_mid[0] = xi2[0];
      Sw.xi_mid[1] = xi2[1];
      Sw.K_first[0] = Kf[0];
      Sw.K_first[1] = Kf[1];
      b.icnt[s] = 0;
    }
  }
}


// ---------------------------------------------------------------------
// force assembly (+ ext_field) and optionally moveP(last)
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(kPartBlock, 6) finalize_kernel(Batch b, int mode) {
  __shared__ double sh[20 * kPartBlock / 32];
  const int2 bk = b.blk[blockIdx.x];
  const int s = bk.x;
  if (at_limit(b, s)) return;
  const SysDev& P = b.sys[s];
  const SysState& S = b.st[s];
  const int i = bk.y + threadIdx.x;
  const bool ok = i < P.part_off + P.n;
  // block sums: K_t, K_r, PT_kin (6), U_ext, then the WCA terms U, W, PT (9)
  // of this block's own candidate pairs
  FF acc[20];
#pragma unroll
  for (int c = 0; c < 20; ++c) acc[c].hi = acc[c].lo = 0.f;
  if (ok) {
    double F[3], T[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      F[a] = (mode & kFlagAccum) ? b.F[3 * i + a] : 0.0;
      T[a] = (mode & kFlagAccum) ? b.T[3 * i + a] : 0.0;
    }
    if (mode & kMaskWca) {
      // its own shares of its candidate pairs (higher-index partners), in
      // slot order, as force_sc adds them
      {
        const int nc = b.wcnt[i];
        const double* own = b.wown + (long long)i * kMaxC * 6;
        const double* ev = b.wev + (long long)i * kMaxC * 11;
        for (int c = 0; c < nc; ++c) {
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            F[a] += own[6 * c + a];
            T[a] += own[6 * c + 3 + a];
          }
#pragma unroll
          for (int q = 0; q < 11; ++q) acc[9 + q] = ff_add(acc[9 + q], ff_from(ev[11 * c + q]));
        }
      }
      // shares of the pairs this particle forms with lower-index partners,
      // left by the WCA kernel in the partner's records.  The screen listed
      // their slots here in arrival order; sorted, the slots ascend with the
      // partner (slot = partner * kMaxC + c), the order force_sc adds them.
      const int nin = min(b.wincnt[i], kMaxC);
      int sl[kMaxC];
      for (int k = 0; k < nin; ++k) {
        const int v = b.win[(long long)i * kMaxC + k];
        int m = k;
        while (m > 0 && sl[m - 1] > v) {
          sl[m] = sl[m - 1];
          --m;
        }
        sl[m] = v;
      }
      for (int k = 0; k < nin; ++k) {
        const double* rec = b.wrec + (long long)sl[k] * 6;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          F[a] += rec[a];
          T[a] += rec[3 + a];
        }
      }
    }
    double ax[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) ax[a] = b.O[9 * i + 6 + a];
    const int nd = P.nd;
    const int loc0 = (i - P.part_off) * nd;
    // the field term needs the FP64 moment; without a field it adds nothing
    const bool ext = (mode & kMaskExt) && (P.B[0] != 0.0 || P.B[1] != 0.0 || P.B[2] != 0.0);
    double uext = 0.0;
    for (int w = 0; w < nd; ++w) {
      const int loc = loc0 + w;
      const int g = P.dip_off + loc;
      // real- and reciprocal-space force and torque of this dipole in
      // float-float (FP32 instructions), one conversion to FP64 at the end
      FF acc6[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) acc6[c].hi = acc6[c].lo = 0.f;
      if (mode & kMaskReal) {
        // this dipole's tile partials summed over all partner strips
        // (real_sum_kernel)
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const float2 v = b.rsum[(long long)c * b.ndtot + g];
          acc6[c].hi = v.x;
          acc6[c].lo = v.y;
        }
      }
      if (mode & kMaskK) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float2 fk = b.Fk[3 * g + c], tk = b.Tk[3 * g + c];
          FF v;
          v.hi = fk.x;
          v.lo = fk.y;
          acc6[c] = ff_add(acc6[c], v);
          v.hi = tk.x;
          v.lo = tk.y;
          acc6[3 + c] = ff_add(acc6[3 + c], v);
        }
      }
      double f[3], t[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        f[c] = soft_f2d(acc6[c].hi) + soft_f2d(acc6[c].lo);
        t[c] = soft_f2d(acc6[3 + c].hi) + soft_f2d(acc6[3 + c].lo);
      }
      if (ext) {
        // ext_field: torque mu o x B, energy -mu o.B (v25/functions.cpp:2014-2020),
        // with the dipole vector mu O^T o_body in FP64
        const double* O = b.O + 9 * i;
        const double ox = b.dob[3 * g], oy = b.dob[3 * g + 1], oz = b.dob[3 * g + 2], mu = b.dmu[g];
        const double mx = mu * (O[0] * ox + O[3] * oy + O[6] * oz);
        const double my = mu * (O[1] * ox + O[4] * oy + O[7] * oz);
        const double mz = mu * (O[2] * ox + O[5] * oy + O[8] * oz);
        t[0] += my * P.B[2] - mz * P.B[1];
        t[1] += mz * P.B[0] - mx * P.B[2];
        t[2] += mx * P.B[1] - my * P.B[0];
        uext -= mx * P.B[0] + my * P.B[1] + mz * P.B[2];
      }
      // lever arm of an off-centre dipole: d x f (v25/classes.hpp:135-136)
      const double pc = b.dpc[g];
      if (pc != 0.0) {
        const double d[3] = {pc * ax[0], pc * ax[1], pc * ax[2]};
        t[0] += d[1] * f[2] - d[2] * f[1];
        t[1] += d[2] * f[0] - d[0] * f[2];
        t[2] += d[0] * f[1] - d[1] * f[0];
      }
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        F[a] += f[a];
        T[a] += t[a];
      }
    }
    acc[8] = ff_from(uext);
    double p[3], l[3];
    if (mode & kFlagMoveP) {
      // moveP last half (v25/functions.cpp:2150-2173)
      const double h = 0.5 * P.dt;
      // xi after moveTher 0 and 1, set by the first-half kernel
      const double ft = 1. - h * S.xi_mid[0], fr = 1. - h * S.xi_mid[1];
      double psq = 0.0;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        p[a] = b.p[3 * i + a] * ft + h * F[a];
        psq += p[a] * p[a];
        l[a] = b.l[3 * i + a] * fr + h * T[a];
        b.p[3 * i + a] = p[a];
        b.l[3 * i + a] = l[a];
      }
      double O[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) O[k] = b.O[9 * i + k];
      const double im = b.invm[i];
      acc[0] = ff_from(psq * im);
      acc[1] = ff_from(rot_kin(b, i, O, l));
      // kinetic pressure tensor p_a p_b / m: FP32 products, float-float sums
      const float pf[3] = {soft_d2f_rn(p[0]), soft_d2f_rn(p[1]), soft_d2f_rn(p[2])};
      const float imf = soft_d2f_rn(im);
      acc[2] = ff_of(pf[0] * pf[0] * imf);
      acc[3] = ff_of(pf[0] * pf[1] * imf);
      acc[4] = ff_of(pf[0] * pf[2] * imf);
      acc[5] = ff_of(pf[1] * pf[1] * imf);
      acc[6] = ff_of(pf[1] * pf[2] * imf);
      acc[7] = ff_of(pf[2] * pf[2] * imf);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      b.F[3 * i + a] = F[a];
      b.T[3 * i + a] = T[a];
    }
  }
  double tot[20];
  block_sum<20, kPartBlock>(acc, sh, tot);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < 9; ++c) b.kin2[9 * blk_slot(P, bk) + c] = tot[c];
    if (mode & kMaskWca) {
#pragma unroll
      for (int c = 0; c < 11; ++c) b.wcaE[11 * blk_slot(P, bk) + c] = tot[9 + c];
    }
  }
}

// ---------------------------------------------------------------------
// oo_params' terms (v25/functions.cpp:2720-2760, Qmat_3d :3426-3445) per
// particle block, from the FP32 working copies of this step's orientations:
// the rod axis o, o o^T and the dipole vectors mu o_dipole, float-float
// block sums.  Its own small kernel, early in the step on the WCA stream:
// widening finalize's sums cost that kernel occupancy.
__global__ void __launch_bounds__(kPartBlock) order_terms_kernel(Batch b) {
  __shared__ double sh[12 * kPartBlock / 32];
  const int2 bk = b.blk[blockIdx.x];
  if (at_limit(b, bk.x)) return;
  const SysDev& P = b.sys[bk.x];
  const int i = bk.y + threadIdx.x;
  FF v[12];
#pragma unroll
  for (int c = 0; c < 12; ++c) v[c].hi = v[c].lo = 0.f;
  if (i < P.part_off + P.n) {
    const float4 q = b.pax[i];
    const float t[9] = {q.x, q.y, q.z, q.x * q.x, q.x * q.y, q.x * q.z, q.y * q.y, q.y * q.z, q.z * q.z};
#pragma unroll
    for (int c = 0; c < 9; ++c) v[c] = ff_of(t[c]);
    const int ND = b.ndtot, g0 = P.dip_off + (i - P.part_off) * P.nd;
    for (int w = 0; w < P.nd; ++w) {
#pragma unroll
      for (int a = 0; a < 3; ++a) v[9 + a] = ff_add(v[9 + a], ff_of(b.dm[a * ND + g0 + w]));
    }
  }
  double tot[12];
  block_sum<12, kPartBlock>(v, sh, tot);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < 12; ++c) b.obk[12 * blk_slot(P, bk) + c] = tot[c];
  }
}

// ---------------------------------------------------------------------
// per-system sums and the thermostat's last update.  kRedGroups blocks per
// system, one per group of sums (real-space tiles, k-vectors, WCA blocks,
// kinetic terms, order parameters), each in float-float with a fixed order;
// the kinetic block also closes the step's thermostat and bookkeeping.
constexpr int kRedThreads = 128;
__global__ void __launch_bounds__(kRedThreads) reduce_obs_kernel(Batch b, int mode) {
  __shared__ double sh[12 * kRedThreads / 32];
  const int s = blockIdx.x / kRedGroups, grp = blockIdx.x % kRedGroups;
  if (at_limit(b, s)) return;
  const SysDev& P = b.sys[s];
  SysState& S = b.st[s];
  SysObs& ob = b.obs[s];
  FF v[12];
#pragma unroll
  for (int c = 0; c < 12; ++c) v[c].hi = v[c].lo = 0.f;
  {
    // the rows of one per-system table, column by column: real-space tiles
    // (U, PT; FP32) or, in large systems, strips (each strip's tiles summed
    // in float-float by strip_energy), k-vectors (U, PT), WCA blocks (U, W, PT), kinetic
    // blocks (K_t, K_r, PT_kin, U_ext) or order-parameter blocks.  One code
    // path for the five keeps the kernel small: its blocks are short, and a
    // larger kernel waited on instruction fetch.
    const float* fsrc = nullptr;
    const double* dsrc = nullptr;
    int nrow, ncol;
    if (grp == 0 && P.rc_real > 0.0) {  // the neighbour pass's block sums (real_cut)
      dsrc = b.rlE + (long long)P.blk_off * 10;
      nrow = P.nblk;
      ncol = 10;
    } else if (grp == 0 && P.nstrip > kStripRows) {  // the strips' sums of their tiles (strip_energy)
      dsrc = b.stripE + (long long)P.strip_off * 10;
      nrow = P.nstrip;
      ncol = 10;
    } else if (grp == 0) {  // the tiles themselves
      fsrc = b.tileE + (long long)P.tile_off * 10;
      nrow = P.ntile;
      ncol = 10;
    } else if (grp == 1) {
      dsrc = b.kE + (long long)P.k_off * 10;
      nrow = P.nk;
      ncol = 10;
    } else if (grp == 2) {
      dsrc = b.wcaE + (long long)P.blk_off * 11;
      nrow = P.nblk;
      ncol = 11;
    } else if (grp == 4) {
      dsrc = b.obk + (long long)P.blk_off * 12;
      nrow = P.nblk;
      ncol = 12;
    } else {
      dsrc = b.kin2 + (long long)P.blk_off * 9;
      nrow = P.nblk;
      ncol = 9;
    }
    for (int t = threadIdx.x; t < nrow; t += kRedThreads) {
#pragma unroll
      for (int c = 0; c < 12; ++c) {
        if (c < ncol) {
          const long long e = (long long)t * ncol + c;
          v[c] = ff_add(v[c], fsrc ? ff_of(fsrc[e]) : ff_from(dsrc[e]));
        }
      }
    }
  }
  double out[12];
  block_sum<12, kRedThreads>(v, sh, out);
  if (threadIdx.x != 0) return;
  if (grp == 0) {
    ob.U_dipR = out[0];
    for (int c = 0; c < 9; ++c) ob.PT_dipR[c] = out[1 + c];
  } else if (grp == 1) {
    ob.U_dipK = out[0];
    for (int c = 0; c < 9; ++c) ob.PT_dipK[c] = out[1 + c];
  } else if (grp == 2) {
    ob.U_ss = out[0];
    ob.W_ss = out[1];
    for (int c = 0; c < 9; ++c) ob.PT_ss[c] = out[2 + c];
  } else if (grp == 4) {
    for (int c = 0; c < 12; ++c) ob.osum[c] = out[c];
  } else {
    ob.U_ext = out[8];
    ob.U_self = P.Uself;
    if (mode & kRedStep) {
      ob.K[0] = 0.5 * out[0];
      ob.K[1] = 0.5 * out[1];
      const double pt6[6] = {out[2], out[3], out[4], out[5], out[6], out[7]};
      const int map[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};
      for (int c = 0; c < 9; ++c) ob.PT_kin[c] = pt6[map[c]];
      // moveTher mode 2 (v25/functions.cpp:2207-2213) closes the step
      const double* nz = b.noise + ((long long)S.iter * b.nsys + s) * 4;
      S.xi[0] = P.ex1 * S.xi_mid[0] + P.cnoise * nz[1];
      S.xi[1] = P.ex1 * S.xi_mid[1] + P.cnoise * nz[3];
      S.strn[0] = nz[1];
      S.strn[1] = nz[3];
      S.step += 1;
      S.iter += 1;
      if (S.rebuild) S.list_builds += 1;
      S.force_list = 0;
    }
    ob.xi[0] = S.xi[0];
    ob.xi[1] = S.xi[1];
    ob.step = S.step;
    ob.status = S.status;
    ob.list_builds = S.list_builds;
  }
}

// ---------------------------------------------------------------------
// function-level entry points
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(kPartBlock) movex_kernel(Batch b) {
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  const int i = bk.y + threadIdx.x;
  if (i >= P.part_off + P.n) return;
  double r[3], p[3], l[3], O[9];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    r[a] = b.r[3 * i + a];
    p[a] = b.p[3 * i + a];
    l[a] = b.l[3 * i + a];
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) O[k] = b.O[9 * i + k];
  move_x(b, i, P.dt, r, p, O, l);
#pragma unroll
  for (int a = 0; a < 3; ++a) b.r[3 * i + a] = r[a];
#pragma unroll
  for (int k = 0; k < 9; ++k) b.O[9 * i + k] = O[k];
  uint32_t u[3];
  derive_particle(b, P, i, r, O, u);
}

__global__ void __launch_bounds__(kPartBlock) renorm_kernel(Batch b) {
  const int2 bk = b.blk[blockIdx.x];
  const SysDev& P = b.sys[bk.x];
  const int i = bk.y + threadIdx.x;
  if (i >= P.part_off + P.n) return;
  double O[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) O[k] = b.O[9 * i + k];
  renorm_O(O);
#pragma unroll
  for (int k = 0; k < 9; ++k) b.O[9 * i + k] = O[k];
}

// moveP with caller-given thermostat coordinates xi[2*sys]; partial sums
// K_t, K_r, PT (6) per block into kin2
__global__ void __launch_bounds__(kPartBlock) movep_kernel(Batch b, const double* __restrict__ xi,
                                                          int last) {
  __shared__ double sh[9 * kPartBlock / 32];
  const int2 bk = b.blk[blockIdx.x];
  const int s = bk.x;
  const SysDev& P = b.sys[s];
  const int i = bk.y + threadIdx.x;
  double acc[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) acc[c] = 0.0;
  if (i < P.part_off + P.n) {
    const double h = 0.5 * P.dt;
    double p[3], l[3], O[9];
    double psq = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) O[k] = b.O[9 * i + k];
    const double xt = xi[2 * s], xr = xi[2 * s + 1];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double p0 = b.p[3 * i + a], l0 = b.l[3 * i + a];
      const double f = b.F[3 * i + a], t = b.T[3 * i + a];
      if (!last) {
        p[a] = (p0 + h * f) / (1. + h * xt);
        l[a] = (l0 + h * t) / (1. + h * xr);
      } else {
        p[a] = p0 * (1. - h * xt) + h * f;
        l[a] = l0 * (1. - h * xr) + h * t;
      }
      psq += p[a] * p[a];
      b.p[3 * i + a] = p[a];
      b.l[3 * i + a] = l[a];
    }
    const double im = b.invm[i];
    acc[0] = psq * im;
    acc[1] = rot_kin(b, i, O, l);
    if (last) {
      acc[2] = p[0] * p[0] * im;
      acc[3] = p[0] * p[1] * im;
      acc[4] = p[0] * p[2] * im;
      acc[5] = p[1] * p[1] * im;
      acc[6] = p[1] * p[2] * im;
      acc[7] = p[2] * p[2] * im;
    }
  }
  double tot[9];
  block_sum<9, kPartBlock>(acc, sh, tot);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < 9; ++c) b.kin2[9 * blk_slot(P, bk) + c] = tot[c];
  }
}

__global__ void reset_iter_kernel(Batch b) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < b.nsys) b.st[s].iter = 0;
}

// ---------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------
void launch_reset_iter(const Batch& b, cudaStream_t s) {
  if (b.nsys) reset_iter_kernel<<<cdiv(b.nsys, 128), 128, 0, s>>>(b);
}
void launch_derive(const Batch& b, cudaStream_t s) {
  if (b.nblk) derive_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
}
void launch_integrate_first(const Batch& b, cudaStream_t s) {
  if (b.nblk) integrate_first_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
}
void launch_finalize(const Batch& b, int mode, cudaStream_t s) {
  if (b.nblk) finalize_kernel<<<b.nblk, kPartBlock, 0, s>>>(b, mode);
}
void launch_order_terms(const Batch& b, cudaStream_t s) {
  if (b.nblk) order_terms_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
}
void launch_reduce_obs(const Batch& b, int mode, cudaStream_t s) {
  if (b.nsys) reduce_obs_kernel<<<kRedGroups * b.nsys, kRedThreads, 0, s>>>(b, mode);
}
void launch_movex(const Batch& b, cudaStream_t s) {
  if (b.nblk) movex_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
}
void launch_renorm(const Batch& b, cudaStream_t s) {
  if (b.nblk) renorm_kernel<<<b.nblk, kPartBlock, 0, s>>>(b);
}
void launch_movep(const Batch& b, const double* xi, int last, cudaStream_t s) {
  if (b.nblk) movep_kernel<<<b.nblk, kPartBlock, 0, s>>>(b, xi, last);
}

}  // namespace mdsc

// ---------------------------------------------------------------------
// systems moved between batches (mdsc_transfer_many): the particle state,
// forces, shapes and dipoles of each (destination slot, source slot) pair,
// the dipole owners for the destination's layout, and the mutable state
// with a list rebuild requested.  One launch per kTransferChunk pairs,
// grid.y over the pairs.
// ---------------------------------------------------------------------
namespace mdsc {

constexpr int kTransferChunk = 256;
struct TransferPairs {
  int n;
  int2 p[kTransferChunk];  // (destination system, source system)
};

__global__ void transfer_kernel(Batch dst, Batch src, TransferPairs tp) {
  const int k = blockIdx.y;
  if (k >= tp.n) return;
  const int d = tp.p[k].x, q = tp.p[k].y;
  const SysDev& Pd = dst.sys[d];
  const SysDev& Ps = src.sys[q];
  const int n = Pd.n, ndip = Pd.ndip;
  const long long is = Ps.part_off, id = Pd.part_off, gs = Ps.dip_off, gd = Pd.dip_off;
  const int stride = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 9 * n; t += stride) {
    dst.O[9 * id + t] = src.O[9 * is + t];
    if (t < 3 * n) {
      dst.r[3 * id + t] = src.r[3 * is + t];
      dst.p[3 * id + t] = src.p[3 * is + t];
      dst.l[3 * id + t] = src.l[3 * is + t];
      dst.F[3 * id + t] = src.F[3 * is + t];
      dst.T[3 * id + t] = src.T[3 * is + t];
      dst.inert[3 * id + t] = src.inert[3 * is + t];
      dst.invI[3 * id + t] = src.invI[3 * is + t];
    }
    if (t < n) {
      dst.len[id + t] = src.len[is + t];
      dst.dia[id + t] = src.dia[is + t];
      dst.mass[id + t] = src.mass[is + t];
      dst.invm[id + t] = src.invm[is + t];
    }
    if (t < 3 * ndip) dst.dob[3 * gd + t] = src.dob[3 * gs + t];
    if (t < ndip) {
      dst.dpc[gd + t] = src.dpc[gs + t];
      dst.dmu[gd + t] = src.dmu[gs + t];
      dst.downer[gd + t] = (int)id + t / max(Pd.nd, 1);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    SysState st = src.st[q];
    st.force_list = 1;
    st.rebuild = 0;
    st.iter = 0;
    dst.st[d] = st;
  }
}

cudaError_t launch_transfer(const Batch& dst, const Batch& src, const std::vector<int2>& pairs, cudaStream_t s) {
  for (size_t k0 = 0; k0 < pairs.size(); k0 += kTransferChunk) {
    TransferPairs tp;
    tp.n = (int)std::min<size_t>(kTransferChunk, pairs.size() - k0);
    for (int k = 0; k < tp.n; ++k) tp.p[k] = pairs[k0 + k];
    // enough threads for the largest system of the batch: 9 values per rod
    const int grid_x = std::min(64, cdiv(9 * std::max(dst.ntot, 1), 256));
    transfer_kernel<<<dim3(grid_x, tp.n), 256, 0, s>>>(dst, src, tp);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace mdsc
