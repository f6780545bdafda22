// Closest points of two spherocylinder axes under the minimum image.
//
// seg_dist_ref: the reference's spherocyl_dist (v25/functions.cpp:89-489),
// in FP64, with its branch structure and its sentinels for parallel rods
// (s = t = -1e6: no unique closest pair; -1e10, -2e10, -3e10, -4e10: the
// (+/+), (-/-), (+/-), (-/+) end-point pairs).  force_sc and the cluster
// test read those sentinels, so the exact path keeps them.
//
// seg_dist_fast: a plain closest-points-of-two-segments routine in FP32
// (clamped line parameters; Ericson, Real-Time Collision Detection 5.1.9)
// used only to pre-filter candidate pairs with a margin.
#pragma once
#include <cuda_runtime.h>

namespace mdsc {

struct RodD {
  double r[3];  // centre (unwrapped, as the reference keeps it)
  double o[3];  // axis
  double len;
};

__device__ inline double ddot(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
__device__ inline double dmimg(double x, double L) { return x - L * floor(x / L + 0.5); }

// returns d^2; dAB = closest-approach vector (from B to A); st = (s, t).
// EXACT: divide by det as the reference does (the cluster test, whose labels
// must equal the reference's); otherwise multiply by one reciprocal (the WCA
// forces, within ~1e-16 of the reference).
template <bool EXACT>
__device__ inline double seg_dist_ref(const RodD& A, const RodD& B, const double L[3],
                                      const double rAB[3], double dAB[3], double st[2]) {
  const double *oA = A.o, *oB = B.o;
  const double lA = A.len, lB = B.len;
  const double doto = ddot(oA, oB);
  const double dotrA = ddot(rAB, oA);
  const double dotrB = ddot(rAB, oB);
  const double a = lA * lA;
  const double b = doto * lA * lB;
  const double c = lB * lB;
  const double d = dotrA * lA - a / 2 + b / 2;
  const double e = dotrB * lB + c / 2 - b / 2;
  const double det = a * c - b * b;
  double s = b * e - c * d;
  double t = a * e - b * d;
  double dsq = 0.;
  auto seg = [&](double sv, double tv, double* out) {
    for (int i = 0; i < 3; ++i) out[i] = rAB[i] + (sv - 0.5) * lA * oA[i] - (tv - 0.5) * lB * oB[i];
  };
  if (det > 1.e-12) {
    double dis[3];
    const double inv_det = EXACT ? 0.0 : 1.0 / det;
    double s0 = EXACT ? s / det : s * inv_det, t0 = EXACT ? t / det : t * inv_det;
    seg(s0, t0, dis);
    double dsq0 = ddot(dis, dis);
    if (dsq0 < 1.e-12) {
      // the axis lines intersect: end point to segment (v25/functions.cpp:127-276)
      double pp[4][3];
      for (int q = 0; q < 3; ++q) {
        pp[0][q] = A.r[q] + lA * oA[q] / 2;
        pp[1][q] = A.r[q] - lA * oA[q] / 2;
        pp[2][q] = B.r[q] + lB * oB[q] / 2;
        pp[3][q] = B.r[q] - lB * oB[q] / 2;
      }
      double dv[4][3], dd[4];
      for (int q = 0; q < 3; ++q) {
        dv[0][q] = dmimg(pp[0][q] - pp[2][q], L[q]);
        dv[1][q] = dmimg(pp[0][q] - pp[3][q], L[q]);
        dv[2][q] = dmimg(pp[1][q] - pp[2][q], L[q]);
        dv[3][q] = dmimg(pp[1][q] - pp[3][q], L[q]);
      }
      int im = 0;
      double mind = 1.e6;
      for (int k = 0; k < 4; ++k) {
        dd[k] = ddot(dv[k], dv[k]);
        if (dd[k] < mind) {
          im = k;
          mind = dd[k];
        }
      }
      const double tfix = (im == 0 || im == 2) ? 1. : 0.;
      const int pB = (im == 0 || im == 2) ? 2 : 3;
      const double sfix = (im == 0 || im == 1) ? 1. : 0.;
      const int pA = (im == 0 || im == 1) ? 0 : 1;
      double vec[3];
      t = tfix;
      for (int q = 0; q < 3; ++q) vec[q] = dmimg(pp[1][q] - pp[pB][q], L[q]);
      s = ddot(vec, oA) / -lA;
      if (s >= 0 && s <= 1) {
        seg(s, t, dAB);
      } else {
        s = sfix;
        for (int q = 0; q < 3; ++q) vec[q] = dmimg(pp[3][q] - pp[pA][q], L[q]);
        t = ddot(vec, oB) / -lB;
        if (t >= 0 && t <= 1) {
          seg(s, t, dAB);
        } else {
          t = tfix;
          for (int q = 0; q < 3; ++q) dAB[q] = dv[im][q];
        }
      }
      dsq = ddot(dAB, dAB);
    } else {
      int region;
      if (s >= 0) {
        if (s <= det)
          region = (t >= 0) ? ((t <= det) ? 5 : 6) : 4;
        else
          region = (t >= 0) ? ((t <= det) ? 2 : 3) : 1;
      } else {
        region = (t >= 0) ? ((t <= det) ? 8 : 9) : 7;
      }
      switch (region) {
        case 2:
          s = 1; t = (e + b) / c;
          t = t > 1 ? 1 : (t < 0 ? 0 : t);
          seg(s, t, dAB);
          break;
        case 8:
          s = 0; t = e / c;
          t = t > 1 ? 1 : (t < 0 ? 0 : t);
          seg(s, t, dAB);
          break;
        case 6:
          t = 1; s = -(d - b) / a;
          s = s > 1 ? 1 : (s < 0 ? 0 : s);
          seg(s, t, dAB);
          break;
        case 4:
          t = 0; s = -d / a;
          s = s > 1 ? 1 : (s < 0 ? 0 : s);
          seg(s, t, dAB);
          break;
        case 1:
        case 3:
        case 7:
        case 9: {
          if (region == 1 || region == 3) {
            s = 1; t = (e + b) / c;
            t = t < 0 ? 0 : (t > 1 ? 1 : t);
            t0 = (region == 1) ? 0 : 1;
            s0 = (region == 1) ? -d / a : -(d - b) / a;
            s0 = s0 < 0 ? 0 : (s0 > 1 ? 1 : s0);
          } else {
            t = (region == 7) ? 0 : 1;
            s = (region == 7) ? -d / a : -(d - b) / a;
            s = s < 0 ? 0 : (s > 1 ? 1 : s);
            s0 = 0; t0 = e / c;
            t0 = t0 < 0 ? 0 : (t0 > 1 ? 1 : t0);
          }
          seg(s, t, dAB);
          dsq = ddot(dAB, dAB);
          seg(s0, t0, dis);
          dsq0 = ddot(dis, dis);
          if (dsq0 < dsq) {
            for (int q = 0; q < 3; ++q) dAB[q] = dis[q];
            s = s0;
            t = t0;
          }
          break;
        }
        default:  // 5
          s = s0;
          t = t0;
          seg(s, t, dAB);
          break;
      }
      dsq = ddot(dAB, dAB);
    }
  } else {
    const double le = (lA + lB) / 2;
    if (fabs(dotrA) < le) {
      for (int i = 0; i < 3; ++i) dAB[i] = rAB[i] - dotrA * oA[i];
      s = t = -1.e+6;
    } else {
      double d2[3];
      const double sg = doto > 0 ? 1.0 : -1.0;
      for (int i = 0; i < 3; ++i) {
        dAB[i] = rAB[i] + lA * oA[i] / 2 + sg * lB * oB[i] / 2;
        d2[i] = rAB[i] - lA * oA[i] / 2 - sg * lB * oB[i] / 2;
      }
      const double dq = ddot(dAB, dAB), dq0 = ddot(d2, d2);
      s = t = (doto > 0) ? -1.e+10 : -3.e+10;
      if (dq0 < dq) {
        for (int q = 0; q < 3; ++q) dAB[q] = d2[q];
        s = t = (doto > 0) ? -2.e+10 : -4.e+10;
      }
    }
    dsq = ddot(dAB, dAB);
  }
  st[0] = s;
  st[1] = t;
  return dsq;
}

// seg_dist_ref<false> without divergence, for the WCA forces.  The
// reference's nine regions reduce to three candidate points: the interior
// solution (s0, t0); s held at an end, S = 1 if s > det else 0, with
// t = clamp((e + b S)/c); t held at an end, T = 1 if t > det else 0, with
// s = clamp((b T - d)/a).  Regions 2/8 take the s-held point, 4/6 the
// t-held one, 5 the interior one, and the corners 1/3/7/9 the nearer of the
// two held points, ties going as in the reference (1/3 keep the s-held
// point, 7/9 the t-held one).  Every lane computes all three and selects,
// so a warp of contacts in different regions runs one instruction stream.
// Parallel axes (det <= 1e-12) and intersecting axis lines fall back to
// seg_dist_ref<false>.  Products are contracted to FMAs and the three
// divisions share one reciprocal: the closest points agree with the
// reference's to a few ulps.
__device__ inline double seg_dist_wca(const RodD& A, const RodD& B, const double L[3],
                                      const double rAB[3], double dAB[3], double st[2]) {
  const double *oA = A.o, *oB = B.o;
  const double lA = A.len, lB = B.len;
  const double doto = fma(oA[2], oB[2], fma(oA[1], oB[1], oA[0] * oB[0]));
  const double dotrA = fma(rAB[2], oA[2], fma(rAB[1], oA[1], rAB[0] * oA[0]));
  const double dotrB = fma(rAB[2], oB[2], fma(rAB[1], oB[1], rAB[0] * oB[0]));
  const double a = lA * lA;
  const double b = doto * lA * lB;
  const double c = lB * lB;
  const double d = fma(dotrA, lA, -0.5 * a) + 0.5 * b;
  const double e = fma(dotrB, lB, 0.5 * c) - 0.5 * b;
  const double det = fma(a, c, -b * b);
  const double s = fma(b, e, -c * d);
  const double t = fma(a, e, -b * d);
  const bool par = !(det > 1.e-12);
  const double dets = par ? 1.0 : det;
  const double ac = a * c;
  const double inv = 1.0 / (dets * ac);
  const double inv_det = inv * ac, inv_a = inv * dets * c, inv_c = inv * dets * a;
  double laA[3], lbB[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    laA[q] = lA * oA[q];
    lbB[q] = lB * oB[q];
  }
  auto seg = [&](double sv, double tv, double* out) {
    const double sm = sv - 0.5, tm = 0.5 - tv;
#pragma unroll
    for (int q = 0; q < 3; ++q) out[q] = fma(tm, lbB[q], fma(sm, laA[q], rAB[q]));
    return fma(out[2], out[2], fma(out[1], out[1], out[0] * out[0]));
  };
  const double s0 = s * inv_det, t0 = t * inv_det;
  double vI[3];
  const double dI = seg(s0, t0, vI);
  if (par || dI < 1.e-12) return seg_dist_ref<false>(A, B, L, rAB, dAB, st);
  const bool sneg = s < 0.0, sbig = s > det, tneg = t < 0.0, tbig = t > det;
  const double S = sbig ? 1.0 : 0.0, T = tbig ? 1.0 : 0.0;
  double tS = fma(b, S, e) * inv_c;
  tS = tS > 1.0 ? 1.0 : (tS < 0.0 ? 0.0 : tS);
  double sT = fma(b, T, -d) * inv_a;
  sT = sT > 1.0 ? 1.0 : (sT < 0.0 ? 0.0 : sT);
  double vS[3], vT[3];
  const double dS = seg(S, tS, vS);
  const double dT = seg(sT, T, vT);
  const bool sout = sneg || sbig, tout = tneg || tbig;
  // 0: interior, 1: s held, 2: t held
  int pick;
  if (!sout && !tout) pick = 0;
  else if (!tout) pick = 1;
  else if (!sout) pick = 2;
  else if (sbig) pick = (dT < dS) ? 2 : 1;
  else pick = (dS < dT) ? 1 : 2;
#pragma unroll
  for (int q = 0; q < 3; ++q) dAB[q] = pick == 0 ? vI[q] : (pick == 1 ? vS[q] : vT[q]);
  st[0] = pick == 0 ? s0 : (pick == 1 ? S : sT);
  st[1] = pick == 0 ? t0 : (pick == 1 ? tS : T);
  return pick == 0 ? dI : (pick == 1 ? dS : dT);
}

// FP32 closest distance^2 of two segments c_A + s lA oA, c_B + t lB oB
// (s, t in [-1/2, 1/2]); r = c_A - c_B.  Pre-filter only.
__device__ __forceinline__ float seg_dist_fast(float rx, float ry, float rz, float ax, float ay,
                                               float az, float la, float bx, float by, float bz,
                                               float lb) {
  // segment A: p1 = -la/2 * oA relative to A's centre; direction d1 = la oA
  // segment B relative to A's centre: p2 = -r - lb/2 oB, d2 = lb oB
  const float d1x = la * ax, d1y = la * ay, d1z = la * az;
  const float d2x = lb * bx, d2y = lb * by, d2z = lb * bz;
  const float p1x = -0.5f * d1x, p1y = -0.5f * d1y, p1z = -0.5f * d1z;
  const float p2x = -rx - 0.5f * d2x, p2y = -ry - 0.5f * d2y, p2z = -rz - 0.5f * d2z;
  const float wx = p1x - p2x, wy = p1y - p2y, wz = p1z - p2z;
  const float a = d1x * d1x + d1y * d1y + d1z * d1z;
  const float e = d2x * d2x + d2y * d2y + d2z * d2z;
  const float f = d2x * wx + d2y * wy + d2z * wz;
  const float c = d1x * wx + d1y * wy + d1z * wz;
  const float b = d1x * d2x + d1y * d2y + d1z * d2z;
  const float den = a * e - b * b;
  float s = den > 1e-6f * a * e ? fminf(fmaxf((b * f - c * e) / den, 0.f), 1.f) : 0.f;
  float t = (b * s + f) / e;
  if (t < 0.f) {
    t = 0.f;
    s = fminf(fmaxf(-c / a, 0.f), 1.f);
  } else if (t > 1.f) {
    t = 1.f;
    s = fminf(fmaxf((b - c) / a, 0.f), 1.f);
  }
  const float qx = wx + s * d1x - t * d2x, qy = wy + s * d1y - t * d2y, qz = wz + s * d1z - t * d2z;
  return qx * qx + qy * qy + qz * qz;
}

}  // namespace mdsc
