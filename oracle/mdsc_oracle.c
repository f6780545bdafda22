/*
 * CPU restatement of the reference's MD-step routines -- the oracle.
 * TEST INFRASTRUCTURE ONLY; see mdsc_oracle.h.  Every function cites the
 * reference routine it restates (file:line within the reference project)
 * and keeps its order of floating-point operations.
 */
#include "mdsc_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;
void mdsc_or_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

/* dot and cros, v25/functions.cpp:3411-3419 */
static inline double dot3(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline void cros3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
static inline double mimg(double x, double L) { return x - L * floor(x / L + 0.5); }

/* rod axis = row 2 of the orientation matrix (Spherocyl::get_ori) */
static inline const double* axis(const mdsc_oracle_state* s, int i) { return &s->O[9 * i + 6]; }

/* dipole w of particle i in the lab frame (Spherocyl::set_dip / rotate,
   v25/classes.cpp:162-171,292-302) */
static inline void dip_lab(const mdsc_oracle_state* s, int i, int w, double pos[3], double ori[3],
                           double lev[3], double* mu) {
  const double* d = &s->dip[(i * s->nd + w) * 5];
  const double* O = &s->O[9 * i];
  const double* r = &s->r[3 * i];
  pos[0] = r[0] + d[0] * O[6];
  pos[1] = r[1] + d[0] * O[7];
  pos[2] = r[2] + d[0] * O[8];
  /* transpose(m_ori) * l0, accumulated from 0 as Matrix::operator* does */
  for (int m = 0; m < 3; ++m) {
    double acc = 0.;
    acc += O[0 * 3 + m] * d[1];
    acc += O[1 * 3 + m] * d[2];
    acc += O[2 * 3 + m] * d[3];
    ori[m] = acc;
  }
  /* Spherocyl::get_lev, v25/classes.hpp:135-136 */
  lev[0] = d[0] * O[6];
  lev[1] = d[0] * O[7];
  lev[2] = d[0] * O[8];
  *mu = d[4];
}

/* ------------------------------------------------------------------ */
/* spherocyl_dist, v25/functions.cpp:89-489                            */
/* ------------------------------------------------------------------ */
#define SEG(dst, sv, tv)                                                     \
  for (int i_ = 0; i_ < 3; ++i_)                                             \
    (dst)[i_] = rAB[i_] + ((sv)-0.5) * lA * oA[i_] - ((tv)-0.5) * lB * oB[i_];

double mdsc_or_seg_dist(const mdsc_oracle_state* S, int iA, int iB, const double rAB[3],
                        double dAB[3], double st[2]) {
  const double* oA = axis(S, iA);
  const double* oB = axis(S, iB);
  const double lA = S->len[iA], lB = S->len[iB];
  const double* L = S->L;
  double doto = dot3(oA, oB);
  double dotrA = dot3(rAB, oA);
  double dotrB = dot3(rAB, oB);

  double a = lA * lA;
  double b = doto * lA * lB;
  double c = lB * lB;
  double d = dotrA * lA - a / 2 + b / 2;
  double e = dotrB * lB + c / 2 - b / 2;

  double det = a * c - b * b;
  double s = b * e - c * d;
  double t = a * e - b * d;
  double dis[3], dsq = 0.;
  if (det > 1.e-12) { /* not parallel */
    double s0, t0, dsq0;
    s0 = s / det;
    t0 = t / det;
    for (int i = 0; i < 3; ++i) dis[i] = rAB[i] + (s0 - 0.5) * lA * oA[i] - (t0 - 0.5) * lB * oB[i];
    dsq0 = dot3(dis, dis);

    if (dsq0 < 1.e-12) { /* the lines intersect: segment-to-endpoint cases, :127-276 */
      const double* rA = &S->r[3 * iA];
      const double* rB = &S->r[3 * iB];
      double pp[4][3];
      for (int q = 0; q < 3; ++q) {
        pp[0][q] = rA[q] + lA * oA[q] / 2;
        pp[1][q] = rA[q] - lA * oA[q] / 2;
        pp[2][q] = rB[q] + lB * oB[q] / 2;
        pp[3][q] = rB[q] - lB * oB[q] / 2;
      }
      double dd[4], dv[4][3];
      for (int q = 0; q < 3; ++q) {
        dv[0][q] = mimg(pp[0][q] - pp[2][q], L[q]);
        dv[1][q] = mimg(pp[0][q] - pp[3][q], L[q]);
        dv[2][q] = mimg(pp[1][q] - pp[2][q], L[q]);
        dv[3][q] = mimg(pp[1][q] - pp[3][q], L[q]);
      }
      for (int k = 0; k < 4; ++k) dd[k] = dot3(dv[k], dv[k]);
      int im = 0;
      double mind = 1.e6;
      for (int k = 0; k < 4; ++k)
        if (dd[k] < mind) {
          im = k;
          mind = dd[k];
        }
      double vec[3];
      /* t fixed at its end point, s from the projection of the other end;
         cases 0..3 of :155-275 differ in which end points they use */
      double tfix = (im == 0 || im == 2) ? 1. : 0.;
      int pB = (im == 0 || im == 2) ? 2 : 3;
      double sfix = (im == 0 || im == 1) ? 1. : 0.;
      int pA = (im == 0 || im == 1) ? 0 : 1;
      t = tfix;
      for (int q = 0; q < 3; ++q) vec[q] = mimg(pp[1][q] - pp[pB][q], L[q]);
      s = dot3(vec, oA);
      s /= -lA;
      if (s >= 0 && s <= 1) {
        SEG(dAB, s, t);
        dsq = dot3(dAB, dAB);
      } else {
        s = sfix;
        for (int q = 0; q < 3; ++q) vec[q] = mimg(pp[3][q] - pp[pA][q], L[q]);
        t = dot3(vec, oB);
        t /= -lB;
        if (t >= 0 && t <= 1) {
          SEG(dAB, s, t);
          dsq = dot3(dAB, dAB);
        } else {
          t = tfix;
          for (int q = 0; q < 3; ++q) dAB[q] = dv[im][q];
          dsq = dot3(dAB, dAB);
        }
      }
    } else { /* the lines do not intersect: 9 regions, :277-445 */
      int region;
      if (s >= 0) {
        if (s <= det) {
          if (t >= 0)
            region = (t <= det) ? 5 : 6;
          else
            region = 4;
        } else {
          if (t >= 0)
            region = (t <= det) ? 2 : 3;
          else
            region = 1;
        }
      } else {
        if (t >= 0)
          region = (t <= det) ? 8 : 9;
        else
          region = 7;
      }
      switch (region) {
        case 2:
          s = 1;
          t = (e + b) / c;
          if (t > 1) t = 1;
          else if (t < 0) t = 0;
          SEG(dAB, s, t);
          dsq = dot3(dAB, dAB);
          break;
        case 8:
          s = 0;
          t = e / c;
          if (t > 1) t = 1;
          else if (t < 0) t = 0;
          SEG(dAB, s, t);
          dsq = dot3(dAB, dAB);
          break;
        case 6:
          t = 1;
          s = -(d - b) / a;
          if (s > 1) s = 1;
          else if (s < 0) s = 0;
          SEG(dAB, s, t);
          dsq = dot3(dAB, dAB);
          break;
        case 4:
          t = 0;
          s = -d / a;
          if (s > 1) s = 1;
          else if (s < 0) s = 0;
          SEG(dAB, s, t);
          dsq = dot3(dAB, dAB);
          break;
        case 1:
        case 3:
        case 7:
        case 9: {
          /* two candidate edges; the first is kept unless the second is closer */
          if (region == 1 || region == 3) {
            s = 1;
            t = (e + b) / c;
            if (t < 0) t = 0;
            else if (t > 1) t = 1;
          } else {
            t = (region == 7) ? 0 : 1;
            s = (region == 7) ? -d / a : -(d - b) / a;
            if (s < 0) s = 0;
            else if (s > 1) s = 1;
          }
          SEG(dAB, s, t);
          dsq = dot3(dAB, dAB);
          if (region == 1 || region == 3) {
            t0 = (region == 1) ? 0 : 1;
            s0 = (region == 1) ? -d / a : -(d - b) / a;
            if (s0 < 0) s0 = 0;
            else if (s0 > 1) s0 = 1;
          } else {
            s0 = 0;
            t0 = e / c;
            if (t0 < 0) t0 = 0;
            else if (t0 > 1) t0 = 1;
          }
          SEG(dis, s0, t0);
          dsq0 = dot3(dis, dis);
          if (dsq0 < dsq) {
            for (int q = 0; q < 3; ++q) dAB[q] = dis[q];
            s = s0;
            t = t0;
            dsq = dsq0;
          }
          break;
        }
        case 5:
        default:
          s /= det;
          t /= det;
          SEG(dAB, s, t);
          dsq = dot3(dAB, dAB);
          break;
      }
    }
  } else { /* parallel, :447-486 */
    double le = (lA + lB) / 2;
    if (fabs(dotrA) < le) { /* no unique closest pair */
      for (int i = 0; i < 3; ++i) dAB[i] = rAB[i] - dotrA * oA[i];
      dsq = dot3(dAB, dAB);
      s = t = -1.e+6;
    } else {
      double d2[3], dsq0;
      if (doto > 0) {
        for (int i = 0; i < 3; ++i) {
          dAB[i] = rAB[i] + lA * oA[i] / 2 + lB * oB[i] / 2;
          d2[i] = rAB[i] - lA * oA[i] / 2 - lB * oB[i] / 2;
        }
        dsq = dot3(dAB, dAB);
        dsq0 = dot3(d2, d2);
        s = t = -1.e+10;
        if (dsq0 < dsq) {
          for (int q = 0; q < 3; ++q) dAB[q] = d2[q];
          dsq = dsq0;
          s = t = -2.e+10;
        }
      } else {
        for (int i = 0; i < 3; ++i) {
          dAB[i] = rAB[i] + lA * oA[i] / 2 - lB * oB[i] / 2;
          d2[i] = rAB[i] - lA * oA[i] / 2 + lB * oB[i] / 2;
        }
        dsq = dot3(dAB, dAB);
        dsq0 = dot3(d2, d2);
        s = t = -3.e+10;
        if (dsq0 < dsq) {
          for (int q = 0; q < 3; ++q) dAB[q] = d2[q];
          dsq = dsq0;
          s = t = -4.e+10;
        }
      }
    }
  }
  st[0] = s;
  st[1] = t;
  return dsq;
}

/* ------------------------------------------------------------------ */
/* neigh_list, v25/functions.cpp:1298-1334                             */
/* ------------------------------------------------------------------ */
int mdsc_or_neigh_list(const mdsc_oracle_state* s, double r_list, int* counts, int* idx, int cap) {
  const int n = s->n;
  const double rl_sq = r_list * r_list;
  int tot = 0;
  for (int f = 0; f < n; ++f) {
    counts[f] = 0;
    if (f == n - 1) break;
    const double* ri = &s->r[3 * f];
    for (int g = f + 1; g < n; ++g) {
      const double* rj = &s->r[3 * g];
      double rij[3], st[2], dij[3];
      for (int a = 0; a < 3; ++a) rij[a] = mimg(ri[a] - rj[a], s->L[a]);
      /* screen: the segment distance is at least the centre distance less
         both half lengths; pairs clearly beyond r_list that way are not
         listed by the segment test either (the margin is far above
         rounding), so the list is the same */
      const double reach = 0.5 * (s->len[f] + s->len[g]) + r_list;
      if (rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2] > reach * reach * (1. + 1e-9) + 1e-9) continue;
      double dsq = mdsc_or_seg_dist(s, f, g, rij, dij, st);
      if (dsq < rl_sq) {
        if (tot < cap) idx[tot] = g;
        ++tot;
        ++counts[f];
      }
    }
  }
  if (n > 0) counts[n - 1] = 0;
  return tot;
}

/* ------------------------------------------------------------------ */
/* force_sc, v25/functions.cpp:1397-1553                               */
/* ------------------------------------------------------------------ */
int mdsc_or_force_sc_list(mdsc_oracle_state* s, double r_cut, const int* start, const int* idx,
                          double* U, double* W, double PT[9]) {
  const int n = s->n;
  const double r_cut_sq = r_cut * r_cut;
  double Uc = 0., Wc = 0.;
  double P[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const double srt = pow(2., 1. / 6);
  const double srtsq = srt * srt;
  int abort_ = 0;
  for (int id = 0; id < n && !abort_; ++id) {
    const double* ri = &s->r[3 * id];
    const double* oi = axis(s, id);
    for (int k = start[id]; k < start[id + 1]; ++k) {
      int jd = idx[k];
      const double* rj = &s->r[3 * jd];
      const double* oj = axis(s, jd);
      double shi0 = s->len[id], shi1 = s->dia[id];
      double shj0 = s->len[jd], shj1 = s->dia[jd];
      double sigma = (shi1 + shj1) / 2;
      double sig_sq = sigma * sigma;
      double rsh = srtsq * sig_sq;
      double rij[3], rsq = 0;
      for (int a = 0; a < 3; ++a) {
        rij[a] = ri[a] - rj[a];
        rij[a] -= s->L[a] * floor(rij[a] / s->L[a] + 0.5);
        rsq += rij[a] * rij[a];
      }
      double st[2], dij[3];
      double dsq = mdsc_or_seg_dist(s, id, jd, rij, dij, st);
      if (dsq < 0.49 * sig_sq) abort_ = 1;   /* overlap, :1454-1465 */
      if (dsq > rsq * 1.00001) abort_ = 1;   /* distance check, :1466-1473 */
      if (dsq < r_cut_sq) {
        double SR2s = sig_sq / dsq;
        double SR6s = SR2s * SR2s * SR2s;
        double pot = 4 * SR6s * (SR6s - 1.);
        double UIJ = 0., WIJ = 0.;
        double ddr = dot3(rij, dij);
        if (dsq < rsh) {
          UIJ = pot + 1.;
          WIJ = 6 * (pot + 4 * SR6s * SR6s) * ddr / dsq;
        }
        Uc += UIJ;
        Wc += WIJ;
        double FIJ = WIJ / ddr;
        double f[3];
        for (int a = 0; a < 3; ++a) f[a] = FIJ * dij[a];
        for (int a = 0; a < 3; ++a) s->F[3 * id + a] += f[a];
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) P[3 * a + b] += rij[a] * f[b];
        for (int a = 0; a < 3; ++a) f[a] *= -1;
        for (int a = 0; a < 3; ++a) s->F[3 * jd + a] += f[a];
        double icroj[3], icror[3], jcror[3], t[3];
        cros3(oi, oj, icroj);
        cros3(oi, rij, icror);
        cros3(oj, rij, jcror);
        double fact1 = (st[0] - 0.5) * shi0;
        double fact2 = -(st[1] - 0.5) * shj0;
        if (st[0] == -1.e+6) fact1 = fact2 = 0.;
        /* the reference tests -3e10 twice (:1526,1529), so the (-/+) end
           points (-4e10) keep the lever arms computed from s, t above */
        if (st[0] == -1.e+10) {
          fact1 = 0.5 * shi0;
          fact2 = 0.5 * shj0;
        } else if (st[0] == -2.e+10) {
          fact1 = -0.5 * shi0;
          fact2 = -0.5 * shj0;
        } else if (st[0] == -3.e+10) {
          fact1 = 0.5 * shi0;
          fact2 = -0.5 * shj0;
        }
        double fmul = fact1 * fact2;
        for (int a = 0; a < 3; ++a) t[a] = FIJ * (fact1 * icror[a] + fmul * icroj[a]);
        for (int a = 0; a < 3; ++a) s->T[3 * id + a] += t[a];
        for (int a = 0; a < 3; ++a) t[a] = FIJ * (fact2 * jcror[a] - fmul * icroj[a]);
        for (int a = 0; a < 3; ++a) s->T[3 * jd + a] += t[a];
      }
    }
  }
  if (abort_) return 0;
  *U = Uc;
  *W = Wc;
  for (int k = 0; k < 9; ++k) PT[k] = P[k];
  return 1;
}

int mdsc_or_force_sc(mdsc_oracle_state* s, double r_cut, double r_list, double* U, double* W,
                     double PT[9]) {
  const int n = s->n;
  int* counts = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
  int cap = 64 * n + 64;
  int* idx = (int*)malloc(sizeof(int) * cap);
  int tot = mdsc_or_neigh_list(s, r_list, counts, idx, cap);
  if (tot > cap) {
    free(idx);
    cap = tot;
    idx = (int*)malloc(sizeof(int) * cap);
    mdsc_or_neigh_list(s, r_list, counts, idx, cap);
  }
  int* start = (int*)malloc(sizeof(int) * (n + 1));
  start[0] = 0;
  for (int i = 0; i < n; ++i) start[i + 1] = start[i] + counts[i];
  int ok = mdsc_or_force_sc_list(s, r_cut, start, idx, U, W, PT);
  free(counts);
  free(idx);
  free(start);
  return ok;
}

/* The real-space cutoff of this library's rc_real: tabul's table with the
   entries beyond rc zeroed (entry i-1 holds r = 0.5 * extL * i / 32768). */
void mdsc_or_mask_table(double* tab, double rc) {
  if (!(rc > 0)) return;
  double extL = 200 * 1.001;
  for (int i = 1; i < 32769; i++)
    if (0.5 * extL * i / 32768 > rc) tab[3 * (i - 1)] = tab[3 * (i - 1) + 1] = tab[3 * (i - 1) + 2] = 0.;
}

/* ------------------------------------------------------------------ */
/* tabul, v25/functions.cpp:1680-1704                                  */
/* ------------------------------------------------------------------ */
void mdsc_or_tabul(double alpha, double* tab) {
  double extL = 200 * 1.001;
  double alsq = alpha * alpha;
  double alft = alsq * alsq;
  double spi = sqrt(M_PI);
  for (int i = 1; i < 32769; i++) {
    double r = 0.5 * extL * i / 32768;
    double rsq = r * r;
    double sr1 = 1.0 / r;
    double sr2 = sr1 * sr1;
    double sr3 = sr2 * sr1;
    double ERFC = erfc(alpha * r);
    double aer = 2.0 * alpha * exp(-alsq * rsq) / spi;
    double aa = 2.0 * alsq + 3.0 * sr2;
    tab[3 * (i - 1) + 0] = ERFC * sr3 + aer * sr2;
    tab[3 * (i - 1) + 1] = (3.0 * ERFC * sr3 + aer * aa) * sr2;
    tab[3 * (i - 1) + 2] = 4. * alft * aer;
  }
}

/* ------------------------------------------------------------------ */
/* force_dipR, v25/functions.cpp:1555-1678                             */
/* ------------------------------------------------------------------ */
void mdsc_or_force_dipR(mdsc_oracle_state* s, const double* Tab, double* U, double PT[9]) {
  const int n = s->n, nd = s->nd;
  double Uc = 0.;
  double P00 = 0., P01 = 0., P02 = 0., P10 = 0., P11 = 0., P12 = 0., P20 = 0., P21 = 0., P22 = 0.;
  const double Lh = 0.5 * (200 * 1.001) / 32768;
  const int nt = g_threads;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt) if (nt > 1) \
    reduction(+ : Uc, P00, P01, P02, P10, P11, P12, P20, P21, P22)
  for (int k = 0; k < n - 1; ++k) {
    for (int lp = k + 1; lp < n; ++lp) {
      for (int v = 0; v < nd; ++v) {
        double ri[3], oi[3], di[3], mui;
        dip_lab(s, k, v, ri, oi, di, &mui);
        if (mui == 0.) continue;
        for (int w = 0; w < nd; ++w) {
          double rj[3], oj[3], dj[3], muj;
          dip_lab(s, lp, w, rj, oj, dj, &muj);
          if (muj == 0.) continue;
          double rij[3], f[3], t[3];
          for (int a = 0; a < 3; ++a) {
            rij[a] = ri[a] - rj[a];
            rij[a] -= s->L[a] * floor(rij[a] / s->L[a] + 0.5);
          }
          double RIJSQ = dot3(rij, rij);
          double uu = mui * muj;
          double SR2 = 1. / RIJSQ;
          double RIJ = sqrt(RIJSQ);
          int ix = (int)floor(RIJ / Lh);
          double R_L0 = RIJ - Lh * ix;
          double R_L1 = RIJ - Lh * (ix + 1);
          double A = (Tab[3 * ix + 0] * R_L0 - Tab[3 * (ix - 1) + 0] * R_L1) / Lh;
          double B = (Tab[3 * ix + 1] * R_L0 - Tab[3 * (ix - 1) + 1] * R_L1) / Lh;
          double C = (Tab[3 * ix + 2] * R_L0 - Tab[3 * (ix - 1) + 2] * R_L1) / Lh;
          double UIR = dot3(oi, rij);
          double UJR = dot3(oj, rij);
          double UIJR = UIR * UJR;
          double UIUJ = dot3(oi, oj);
          double UIJ = uu * (UIUJ * A - UIJR * B);
          Uc += UIJ;
          double fact = (UIUJ - 5. * UIJR * SR2) * B - UIJR * SR2 * C;
          for (int a = 0; a < 3; ++a) f[a] = uu * (fact * rij[a] + (UIR * oj[a] + UJR * oi[a]) * B);
          for (int a = 0; a < 3; ++a) {
#pragma omp atomic
            s->F[3 * k + a] += f[a];
          }
          P00 += rij[0] * f[0]; P01 += rij[0] * f[1]; P02 += rij[0] * f[2];
          P10 += rij[1] * f[0]; P11 += rij[1] * f[1]; P12 += rij[1] * f[2];
          P20 += rij[2] * f[0]; P21 += rij[2] * f[1]; P22 += rij[2] * f[2];
          for (int a = 0; a < 3; ++a) f[a] *= -1;
          for (int a = 0; a < 3; ++a) {
#pragma omp atomic
            s->F[3 * lp + a] += f[a];
          }
          double icror[3], dicror[3], dicroi[3], jcror[3], djcror[3], djcroj[3];
          double dicroj[3], djcroi[3], icroj[3];
          cros3(oi, rij, icror);
          cros3(di, rij, dicror);
          cros3(di, oi, dicroi);
          cros3(oj, rij, jcror);
          cros3(dj, rij, djcror);
          cros3(dj, oj, djcroj);
          cros3(di, oj, dicroj);
          cros3(dj, oi, djcroi);
          cros3(oi, oj, icroj);
          for (int a = 0; a < 3; ++a) icroj[a] *= A;
          fact = -UIR * UJR * (5 * B + C) * SR2 + UIUJ * B;
          double fact1;
          for (int a = 0; a < 3; ++a) {
            fact1 = (UJR * (icror[a] + dicroi[a]) + UIR * dicroj[a]) * B;
            t[a] = uu * (fact * dicror[a] + fact1 - icroj[a]);
          }
          for (int a = 0; a < 3; ++a) {
#pragma omp atomic
            s->T[3 * k + a] += t[a];
          }
          for (int a = 0; a < 3; ++a) {
            fact1 = (UIR * (jcror[a] - djcroj[a]) - UJR * djcroi[a]) * B;
            t[a] = uu * (-fact * djcror[a] + fact1 + icroj[a]);
          }
          for (int a = 0; a < 3; ++a) {
#pragma omp atomic
            s->T[3 * lp + a] += t[a];
          }
        }
      }
    }
  }
  *U = Uc;
  PT[0] = P00; PT[1] = P01; PT[2] = P02;
  PT[3] = P10; PT[4] = P11; PT[5] = P12;
  PT[6] = P20; PT[7] = P21; PT[8] = P22;
}

/* ------------------------------------------------------------------ */
/* wave_v, v25/functions.cpp:1963-1990                                 */
/* ------------------------------------------------------------------ */
void mdsc_or_wave_v(double* kvec, const double L[3], double alpha, int K_max, int ksq_max) {
  const int K1 = K_max + 1;
  double c = 4. * alpha * alpha;
  double P2[3] = {2. * M_PI / L[0], 2. * M_PI / L[1], 2. * M_PI / L[2]};
  memset(kvec, 0, sizeof(double) * K1 * K1 * K1);
  for (int nz = 0; nz <= K_max; ++nz) {
    double Kz = P2[2] * nz;
    for (int ny = 0; ny <= K_max; ++ny) {
      double Ky = P2[1] * ny;
      for (int nx = 0; nx <= K_max; ++nx) {
        double Kx = P2[0] * nx;
        double Ksq = Kx * Kx + Ky * Ky + Kz * Kz;
        if (Ksq != 0.) kvec[(nx * K1 + ny) * K1 + nz] = 4. * M_PI * exp(-Ksq / c) / Ksq;
        if (ksq_max > 0 && nx * nx + ny * ny + nz * nz > ksq_max) kvec[(nx * K1 + ny) * K1 + nz] = 0.;
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* force_dipK, v25/functions.cpp:1706-1961                             */
/* complex arithmetic is written out as libstdc++ std::complex<double>  */
/* evaluates it (product: (ac-bd, ad+bc); norm: re^2+im^2)              */
/* ------------------------------------------------------------------ */
typedef struct {
  double re, im;
} cplx;

void mdsc_or_force_dipK(mdsc_oracle_state* s, int K_max, double alpha, const double* Kvec,
                        double* U, double PT[9]) {
  const int n = s->n, nd = s->nd;
  const int K1 = K_max + 1;
  const double* L = s->L;
  double V = L[0] * L[1] * L[2];
  double P2[3] = {2. * M_PI / L[0], 2. * M_PI / L[1], 2. * M_PI / L[2]};
  int K_max2 = K_max * K_max;
  int K_max3 = K_max2 * K_max;
  double a4 = 1. / (4. * alpha);
  double Uc = 0.;
  double P00 = 0., P01 = 0., P02 = 0., P10 = 0., P11 = 0., P12 = 0., P20 = 0., P21 = 0., P22 = 0.;
  const int nt = g_threads;
#pragma omp parallel num_threads(nt) if (nt > 1)
  {
    cplx* M = (cplx*)malloc(sizeof(cplx) * 4 * (size_t)n * (nd > 0 ? nd : 1));
#pragma omp for schedule(dynamic, 50) reduction(+ : Uc, P00, P01, P02, P10, P11, P12, P20, P21, P22)
    for (int kn = 0; kn < K_max3; ++kn) {
      int nz = (int)floor((float)kn / K_max2);
      float lf = kn - K_max2 * nz;
      int ny = (int)floor(lf / K_max);
      int nx = (int)lf - K_max * ny;
      double Kz = P2[2] * nz, Ky = P2[1] * ny, Kx = P2[0] * nx;
      double Ksq = Kx * Kx + Ky * Ky + Kz * Kz;
      if (Ksq == 0) continue;
      double KK = Kvec[(nx * K1 + ny) * K1 + nz];
      double val = 2. * KK / V;
      double pval = 2 * (a4 + 1. / Ksq);
      double K[4][3] = {{Kx, Ky, Kz}, {-Kx, Ky, Kz}, {Kx, -Ky, Kz}, {-Kx, -Ky, Kz}};
      cplx sum[4], uve[4][3];
      double self[4], uvslf[4][3];
      for (int b = 0; b < 4; ++b) {
        sum[b].re = sum[b].im = 0.;
        self[b] = 0.;
        for (int k = 0; k < 3; ++k) {
          uve[b][k].re = uve[b][k].im = 0.;
          uvslf[b][k] = 0.;
        }
      }
      for (size_t q = 0; q < 4 * (size_t)n * nd; ++q) M[q].re = M[q].im = 0.;
#define MIDX(b, i, w) M[((size_t)(b) * n + (i)) * nd + (w)]
      for (int i = 0; i < n; ++i) {
        cplx selfpart[4], uvslfpart[4][3];
        for (int b = 0; b < 4; ++b) {
          selfpart[b].re = selfpart[b].im = 0.;
          for (int k = 0; k < 3; ++k) uvslfpart[b][k].re = uvslfpart[b][k].im = 0.;
        }
        for (int w = 0; w < nd; ++w) {
          double ri[3], oi[3], di[3], mu;
          dip_lab(s, i, w, ri, oi, di, &mu);
          for (int k = 0; k < 3; ++k) ri[k] -= L[k] * floor(ri[k] / L[k] + 0.5);
          if (mu != 0.) {
            double RIK[4], UIK[4];
            cplx z[4];
            for (int b = 0; b < 4; ++b) {
              RIK[b] = dot3(ri, K[b]);
              UIK[b] = dot3(oi, K[b]);
              UIK[b] *= mu;
              z[b].re = cos(RIK[b]);
              z[b].im = sin(RIK[b]);
            }
            for (int b = 0; b < 4; ++b) {
              cplx m = {z[b].re, -z[b].im};
              MIDX(b, i, w) = m;
              cplx uk = {UIK[b] * m.re, UIK[b] * m.im};
              sum[b].re += uk.re;
              sum[b].im += uk.im;
              selfpart[b].re += uk.re;
              selfpart[b].im += uk.im;
              for (int k = 0; k < 3; ++k) {
                double fac = mu * oi[k];
                cplx u2 = {fac * m.re, fac * m.im};
                uve[b][k].re += u2.re;
                uve[b][k].im += u2.im;
                uvslfpart[b][k].re += u2.re;
                uvslfpart[b][k].im += u2.im;
              }
            }
          }
        }
        for (int b = 0; b < 4; ++b) {
          self[b] += selfpart[b].re * selfpart[b].re + selfpart[b].im * selfpart[b].im;
          for (int k = 0; k < 3; ++k)
            uvslf[b][k] += selfpart[b].re * uvslfpart[b][k].re - (-selfpart[b].im) * uvslfpart[b][k].im;
        }
      }
      cplx adds[4];
      double addslf[4];
      for (int b = 0; b < 4; ++b) {
        adds[b].re = 0. + sum[b].re;
        adds[b].im = 0. + sum[b].im;
        addslf[b] = 0. + self[b];
      }
      double Upar = 0;
      for (int b = 0; b < 4; ++b) {
        double nrm = adds[b].re * adds[b].re + adds[b].im * adds[b].im;
        double en = val * 0.5 * (nrm - addslf[b]);
        Upar += en;
      }
      int w4 = (nx == 0 && ny == 0) || (nx == 0 && nz == 0) || (ny == 0 && nz == 0);
      int w2 = (nz == 0 && nx != 0 && ny != 0) || (ny == 0 && nz != 0 && nx != 0) ||
               (nx == 0 && ny != 0 && nz != 0);
      if (w4) Upar /= 4.;
      else if (w2) Upar /= 2.;
      Uc += Upar;

      /* force and torque, :1853-1925 */
      for (int i = 0; i < n; ++i) {
        double UIKw[4][8];
        cplx local_adds[4];
        for (int b = 0; b < 4; ++b) {
          local_adds[b].re = local_adds[b].im = 0.;
          for (int w = 0; w < nd; ++w) {
            double ri[3], oi[3], di[3], mu;
            dip_lab(s, i, w, ri, oi, di, &mu);
            if (mu != 0) {
              UIKw[b][w] = dot3(oi, K[b]);
              UIKw[b][w] *= mu;
              cplx m = MIDX(b, i, w);
              local_adds[b].re += UIKw[b][w] * m.re;
              local_adds[b].im += UIKw[b][w] * m.im;
            }
          }
        }
        for (int w = 0; w < nd; ++w) {
          double ri[3], oi[3], di[3], mu;
          dip_lab(s, i, w, ri, oi, di, &mu);
          if (mu == 0) continue;
          double icrok[4][3], dicrok[4][3];
          for (int b = 0; b < 4; ++b) {
            cros3(di, K[b], dicrok[b]);
            cros3(oi, K[b], icrok[b]);
            for (int j = 0; j < 3; ++j) icrok[b][j] *= mu;
          }
          double f[3] = {0., 0., 0.}, t[3] = {0., 0., 0.};
          for (int b = 0; b < 4; ++b) {
            cplx m = MIDX(b, i, w);
            cplx dc = {adds[b].re - local_adds[b].re, (-adds[b].im) - (-local_adds[b].im)};
            cplx um = {UIKw[b][w] * m.re, UIKw[b][w] * m.im};
            double im_ = um.re * dc.im + um.im * dc.re;
            double factF = -val * im_;
            for (int j = 0; j < 3; ++j) f[j] += factF * K[b][j];
            double re_ = m.re * dc.re - m.im * dc.im;
            double factT = -val * re_;
            for (int j = 0; j < 3; ++j) t[j] += factT * icrok[b][j] + factF * dicrok[b][j];
          }
          if (w4) {
            for (int j = 0; j < 3; ++j) {
              f[j] /= 4.;
              t[j] /= 4.;
            }
          } else if (w2) {
            for (int j = 0; j < 3; ++j) {
              f[j] /= 2.;
              t[j] /= 2.;
            }
          }
          for (int j = 0; j < 3; ++j) {
#pragma omp atomic
            s->F[3 * i + j] += f[j];
          }
          for (int j = 0; j < 3; ++j) {
#pragma omp atomic
            s->T[3 * i + j] += t[j];
          }
        }
      }
#undef MIDX
      /* pressure tensor, :1926-1952 */
      double P[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int b = 0; b < 4; ++b) {
        double nrm = adds[b].re * adds[b].re + adds[b].im * adds[b].im;
        for (int j = 0; j < 3; ++j) {
          for (int k = 0; k < 3; ++k) {
            double re_ = adds[b].re * uve[b][j].re - (-adds[b].im) * uve[b][j].im;
            P[j][k] += val * 0.5 *
                       (((double)(j == k) - pval * K[b][j] * K[b][k]) * (nrm - addslf[b]) +
                        2 * (re_ - uvslf[b][j]) * K[b][k]);
          }
        }
      }
      if (w4) {
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k) P[j][k] /= 4.;
      } else if (w2) {
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k) P[j][k] /= 2.;
      }
      P00 += P[0][0]; P01 += P[0][1]; P02 += P[0][2];
      P10 += P[1][0]; P11 += P[1][1]; P12 += P[1][2];
      P20 += P[2][0]; P21 += P[2][1]; P22 += P[2][2];
    }
    free(M);
  }
  *U = Uc;
  PT[0] = P00; PT[1] = P01; PT[2] = P02;
  PT[3] = P10; PT[4] = P11; PT[5] = P12;
  PT[6] = P20; PT[7] = P21; PT[8] = P22;
}

/* ------------------------------------------------------------------ */
/* ext_field, v25/functions.cpp:1992-2025                              */
/* ------------------------------------------------------------------ */
void mdsc_or_ext_field(mdsc_oracle_state* s, const double B[3], double* U) {
  double Uext = 0.;
  for (int k = 0; k < s->n; ++k) {
    for (int w = 0; w < s->nd; ++w) {
      double ri[3], oi[3], di[3], mu, t[3];
      dip_lab(s, k, w, ri, oi, di, &mu);
      double doti = dot3(oi, B);
      Uext -= mu * doti;
      cros3(oi, B, t);
      t[0] *= mu;
      t[1] *= mu;
      t[2] *= mu;
      for (int a = 0; a < 3; ++a) s->T[3 * k + a] += t[a];
    }
  }
  *U = Uext;
}

/* ------------------------------------------------------------------ */
/* self_ener, v25/functions.cpp:2027-2069 (per particle, one species)  */
/* ------------------------------------------------------------------ */
double mdsc_or_self_ener(const mdsc_oracle_state* s) {
  /* the reference evaluates particle 0 of each species and multiplies by
     the species count; with one species that is particle 0 times n */
  if (s->n == 0) return 0.;
  double Un = 0.;
  for (int v = 0; v < s->nd - 1; ++v) {
    double ri[3], oi[3], di[3], mui;
    dip_lab(s, 0, v, ri, oi, di, &mui);
    for (int w = v + 1; w < s->nd; ++w) {
      double rj[3], oj[3], dj[3], muj;
      dip_lab(s, 0, w, rj, oj, dj, &muj);
      double uu = mui * muj;
      double rij[3];
      for (int a = 0; a < 3; ++a) rij[a] = ri[a] - rj[a];
      double RIJSQ = dot3(rij, rij);
      double RIJ = sqrt(RIJSQ);
      double SR2 = 1. / RIJSQ;
      double SR3 = SR2 / RIJ;
      double UIUJ = dot3(oi, oj);
      double UIR = dot3(oi, rij);
      double UJR = dot3(oj, rij);
      Un += uu * (UIUJ * SR3 - 3. * UIR * UJR * SR2 * SR3);
    }
  }
  return 0. + s->n * Un;
}

/* ------------------------------------------------------------------ */
/* integrator                                                          */
/* ------------------------------------------------------------------ */
/* Matrix<double>::operator* on 3x3 operands (v25/Matrix.hpp:383-393) */
static void mm3(const double* A, const double* B, double* C) {
  double R[9];
  for (int m = 0; m < 3; ++m)
    for (int n = 0; n < 3; ++n) {
      double acc = 0;
      for (int i = 0; i < 3; ++i) acc += A[3 * m + i] * B[3 * i + n];
      R[3 * m + n] = acc;
    }
  memcpy(C, R, sizeof(R));
}
static void mv3(const double* A, const double* x, double* y) {
  double R[3];
  for (int m = 0; m < 3; ++m) {
    double acc = 0;
    for (int i = 0; i < 3; ++i) acc += A[3 * m + i] * x[i];
    R[m] = acc;
  }
  memcpy(y, R, sizeof(R));
}

/* set_inertia, v25/classes.cpp:175-185 */
void mdsc_or_inertia(double L, double D, double mass, double I[3]) {
  double R = D / 2;
  double Rsq = R * R;
  double Rft = Rsq * Rsq;
  double Lsq = L * L;
  double vol = M_PI * Rsq * (L + 3. * R / 4);
  double mdens = mass / vol;
  I[0] = mdens * M_PI * (Lsq * L * Rsq / 12 + Lsq * Rsq * R / 3 + L * Rft / 4 + 8. * Rft * R / 15);
  I[1] = I[0];
  I[2] = mdens * M_PI * (L * Rft / 2 + 8. * Rft * R / 15);
}

/* translate + rotate, v25/classes.cpp:228-304 */
static void move_one(mdsc_oracle_state* s, int id, double dt) {
  double* r = &s->r[3 * id];
  const double* p = &s->p[3 * id];
  double* O = &s->O[9 * id];
  const double* l = &s->l[3 * id];
  double I[3];
  mdsc_or_inertia(s->len[id], s->dia[id], s->mass[id], I);
  for (int j = 0; j < 3; j++) r[j] += dt * p[j] / s->mass[id];

  double R[9], Q[9], l0[3], l1[3];
  double ang, cosa, sina, dt2 = dt / 2;
  mv3(O, l, l1);
  /* Rx */
  ang = -l1[0] * dt2 / I[0];
  cosa = cos(ang); sina = sin(ang);
  R[0] = 1.; R[1] = 0.; R[2] = 0.;
  R[3] = 0.; R[4] = cosa; R[5] = -sina;
  R[6] = 0.; R[7] = sina; R[8] = cosa;
  mv3(R, l1, l0);
  mm3(R, O, Q);
  /* Ry */
  ang = -l0[1] * dt2 / I[1];
  cosa = cos(ang); sina = sin(ang);
  R[0] = cosa; R[1] = 0.; R[2] = sina;
  R[3] = 0.; R[4] = 1.; R[5] = 0.;
  R[6] = -sina; R[7] = 0.; R[8] = cosa;
  mv3(R, l0, l1);
  mm3(R, Q, O);
  /* Rz */
  ang = -l1[2] * dt / I[2];
  cosa = cos(ang); sina = sin(ang);
  R[0] = cosa; R[1] = -sina; R[2] = 0.;
  R[3] = sina; R[4] = cosa; R[5] = 0.;
  R[6] = 0.; R[7] = 0.; R[8] = 1.;
  mv3(R, l1, l0);
  mm3(R, O, Q);
  /* Ry */
  ang = -l0[1] * dt2 / I[1];
  cosa = cos(ang); sina = sin(ang);
  R[0] = cosa; R[1] = 0.; R[2] = sina;
  R[3] = 0.; R[4] = 1.; R[5] = 0.;
  R[6] = -sina; R[7] = 0.; R[8] = cosa;
  mv3(R, l0, l1);
  mm3(R, Q, O);
  /* Rx */
  ang = -l1[0] * dt2 / I[0];
  cosa = cos(ang); sina = sin(ang);
  R[0] = 1.; R[1] = 0.; R[2] = 0.;
  R[3] = 0.; R[4] = cosa; R[5] = -sina;
  R[6] = 0.; R[7] = sina; R[8] = cosa;
  mv3(R, l1, l0);
  mm3(R, O, Q);
  memcpy(O, Q, sizeof(Q));
}

void mdsc_or_moveX(mdsc_oracle_state* s, double dt) {
  const int nt = g_threads;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
  for (int id = 0; id < s->n; ++id) move_one(s, id, dt);
}

void mdsc_or_moveP(mdsc_oracle_state* s, const double xi[2], double Dt, int last, double Kout[2],
                   double PT[9]) {
  double Dt2 = Dt / 2;
  double Kc0 = 0., Kc1 = 0.;
  double P00 = 0., P01 = 0., P02 = 0., P11 = 0., P12 = 0., P22 = 0.;
  const int nt = g_threads;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1) \
    reduction(+ : Kc0, Kc1, P00, P01, P02, P11, P12, P22)
  for (int id = 0; id < s->n; ++id) {
    double m = s->mass[id];
    double I[3];
    mdsc_or_inertia(s->len[id], s->dia[id], m, I);
    double* p = &s->p[3 * id];
    const double* f = &s->F[3 * id];
    double* l = &s->l[3 * id];
    const double* t = &s->T[3 * id];
    const double* o = &s->O[9 * id];
    /* Ib = transpose(o) * I0 * o */
    double I0[9] = {1. / I[0], 0, 0, 0, 1. / I[1], 0, 0, 0, 1. / I[2]};
    double oT[9], tmp[9], Ib[9];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) oT[3 * a + b] = o[3 * b + a];
    mm3(oT, I0, tmp);
    mm3(tmp, o, Ib);
    double psq = 0., lsq = 0.;
    double sfac;
    if (!last) {
      sfac = 1. + Dt2 * xi[0];
      for (int j = 0; j < 3; j++) {
        p[j] = (p[j] + Dt2 * f[j]) / sfac;
        psq += p[j] * p[j];
      }
      sfac = 1. + Dt2 * xi[1];
      for (int j = 0; j < 3; j++) l[j] = (l[j] + Dt2 * t[j]) / sfac;
    } else {
      sfac = 1. - Dt2 * xi[0];
      for (int j = 0; j < 3; j++) {
        p[j] = p[j] * sfac + Dt2 * f[j];
        psq += p[j] * p[j];
      }
      P00 += p[0] * p[0] / m; P01 += p[0] * p[1] / m; P02 += p[0] * p[2] / m;
      P11 += p[1] * p[1] / m; P12 += p[1] * p[2] / m;
      P22 += p[2] * p[2] / m;
      sfac = 1. - Dt2 * xi[1];
      for (int j = 0; j < 3; j++) l[j] = l[j] * sfac + Dt2 * t[j];
    }
    /* lres = transpose(ll) * Ib * ll */
    double v[3];
    for (int nn = 0; nn < 3; ++nn) {
      double acc = 0;
      for (int i = 0; i < 3; ++i) acc += l[i] * Ib[3 * i + nn];
      v[nn] = acc;
    }
    double lres = 0;
    for (int i = 0; i < 3; ++i) lres += v[i] * l[i];
    lsq += lres;
    Kc0 += psq / m;
    Kc1 += lsq;
  }
  Kout[0] = Kc0 / 2;
  Kout[1] = Kc1 / 2;
  PT[0] = P00; PT[1] = P01; PT[2] = P02;
  PT[3] = P01; PT[4] = P11; PT[5] = P12;
  PT[6] = P02; PT[7] = P12; PT[8] = P22;
}

/* renorm, v25/classes.cpp:307-325 */
void mdsc_or_renorm(mdsc_oracle_state* s) {
  for (int i = 0; i < s->n; ++i) {
    double* o = &s->O[9 * i];
    double norm = sqrt(o[6] * o[6] + o[7] * o[7] + o[8] * o[8]);
    o[6] /= norm; o[7] /= norm; o[8] /= norm;
    double Up[3] = {o[6] + o[3], o[7] + o[4], o[8] + o[5]};
    double d = Up[0] * o[6] + Up[1] * o[7] + Up[2] * o[8];
    o[3] = Up[0] - d * o[6];
    o[4] = Up[1] - d * o[7];
    o[5] = Up[2] - d * o[8];
    norm = sqrt(o[3] * o[3] + o[4] * o[4] + o[5] * o[5]);
    o[3] /= norm; o[4] /= norm; o[5] /= norm;
    o[0] = o[4] * o[8] - o[7] * o[5];
    o[1] = o[5] * o[6] - o[8] * o[3];
    o[2] = o[3] * o[7] - o[6] * o[4];
  }
}

/* gauss, v25/functions.cpp:1149-1156 */
void mdsc_or_gauss(double variance, double* rnd1, double* rnd2) {
  double rndA = sqrt(-2 * log(*rnd1)) * cos(2 * M_PI * *rnd2);
  double rndB = sqrt(-2 * log(*rnd1)) * sin(2 * M_PI * *rnd2);
  double sqrtVar = sqrt(variance);
  *rnd1 = rndA * sqrtVar;
  *rnd2 = rndB * sqrtVar;
}

void mdsc_or_thermo_init(mdsc_or_thermo* th, double Q, double gamma, double xi0) {
  th->Q = Q;
  th->g = gamma;
  th->xi[0] = th->xi[1] = xi0;
  th->strn[0] = th->strn[1] = 0.;
  mdsc_mt_seed(&th->rng[0], 1);
  mdsc_mt_seed(&th->rng[1], 2);
}

/* moveTher, v25/functions.cpp:2186-2218 */
void mdsc_or_moveTher(mdsc_or_thermo* th, double temp, double Dt, const double K[2], double Tpart,
                      int mode) {
  for (int i = 0; i < 2; ++i) {
    double Q = th->Q, g, ex1, s;
    switch (mode) {
      case 0: {
        double rnd[2];
        rnd[0] = mdsc_mt_uniform(&th->rng[i]);
        rnd[1] = mdsc_mt_uniform(&th->rng[i]);
        mdsc_or_gauss(1, &rnd[0], &rnd[1]);
        th->strn[i] = rnd[1];
        g = th->g;
        ex1 = exp(-g * Dt / 2);
        s = ex1 * th->xi[i] + sqrt(2. * temp * g * Dt / Q) * rnd[0];
        th->xi[i] = s;
        break;
      }
      case 1:
        s = th->xi[i] + Dt * (2. * K[i] - 3. * Tpart * temp) / Q;
        th->xi[i] = s;
        break;
      case 2: {
        double rnd1 = th->strn[i];
        g = th->g;
        ex1 = exp(-g * Dt / 2);
        s = ex1 * th->xi[i] + sqrt(2. * temp * g * Dt / Q) * rnd1;
        th->xi[i] = s;
        break;
      }
      default:
        break;
    }
  }
}

/* ------------------------------------------------------------------ */
/* clust_conf, v25/functions.cpp:2950-3148,3282-3324                   */
/* ------------------------------------------------------------------ */
/* dist_test, v25/functions.cpp:2987-3016 */
static int dist_test(const mdsc_oracle_state* s, int A, int B, double min_s) {
  const double* ri = &s->r[3 * A];
  const double* rj = &s->r[3 * B];
  double sigma = (s->dia[A] + s->dia[B]) / 2 + min_s;
  double sig_sq = sigma * sigma;
  double rij[3], st[2], dij[3];
  for (int a = 0; a < 3; ++a) {
    rij[a] = ri[a] - rj[a];
    rij[a] -= s->L[a] * floor(rij[a] / s->L[a] + 0.5);
  }
  double dsq = mdsc_or_seg_dist(s, A, B, rij, dij, st);
  return dsq < sig_sq;
}

/* The pair energy of the energy criterion for clusters -- an extension: the
   reference's own criterion is the geometric one above.  U_pair = the WCA
   pair energy of force_sc (v25/functions.cpp:1436-1483, 2^(1/6) sigma range,
   shifted by 1) + the bare dipole-dipole energy of every dipole pair of the
   two rods, at the minimum image of the dipole sites:
     mu_a mu_b (o_a.o_b - 3 (o_a.r)(o_b.r) / r^2) / r^3.
   A is the lower index.  Zero-moment dipoles are skipped. */
double mdsc_or_pair_energy(const mdsc_oracle_state* s, int A, int B) {
  const double* ri = &s->r[3 * A];
  const double* rj = &s->r[3 * B];
  double rij[3], dij[3], st[2];
  for (int a = 0; a < 3; ++a) {
    rij[a] = ri[a] - rj[a];
    rij[a] -= s->L[a] * floor(rij[a] / s->L[a] + 0.5);
  }
  const double dsq = mdsc_or_seg_dist(s, A, B, rij, dij, st);
  const double sigma = (s->dia[A] + s->dia[B]) / 2;
  const double sig_sq = sigma * sigma;
  const double srt = 1.122462048309373; /* 2^(1/6) */
  double U = 0.;
  if (dsq < srt * srt * sig_sq) {
    const double SR2s = sig_sq / dsq;
    const double SR6s = SR2s * SR2s * SR2s;
    U = 4 * SR6s * (SR6s - 1.) + 1.;
  }
  for (int a = 0; a < s->nd; ++a) {
    double pa[3], oa[3], la[3], ma;
    dip_lab(s, A, a, pa, oa, la, &ma);
    if (ma == 0.) continue;
    for (int b = 0; b < s->nd; ++b) {
      double pb[3], ob[3], lb[3], mb;
      dip_lab(s, B, b, pb, ob, lb, &mb);
      if (mb == 0.) continue;
      double r[3];
      for (int k = 0; k < 3; ++k) r[k] = mimg(pa[k] - pb[k], s->L[k]);
      const double r2 = dot3(r, r);
      const double ir = 1. / sqrt(r2);
      const double ir3 = ir * ir * ir;
      const double dd = dot3(oa, ob), da = dot3(oa, r), db = dot3(ob, r);
      U += ma * mb * (dd - 3. * da * db / r2) * ir3;
    }
  }
  return U;
}

/* the bond test of a labelling: geometric (dist_test, min_s) or energy
   (U_pair < -u_bond, lower index first) */
typedef struct {
  int energy;
  double v;
} bond_rule;

static int bonded(const mdsc_oracle_state* s, int A, int B, const bond_rule* br) {
  if (!br->energy) return dist_test(s, A, B, br->v);
  return (A < B ? mdsc_or_pair_energy(s, A, B) : mdsc_or_pair_energy(s, B, A)) < -br->v;
}

/* Partners j that the geometric test can bond to A, ascending: the segment
   distance is at least the centre distance less both half lengths, so a
   pair whose minimum-image centres lie further apart than
   (L_A + L_B)/2 + sigma (with a margin far above rounding) cannot pass
   dist_test.  Only a screen: the bond itself is still dist_test, and the
   partners come in the order the reference's j loop visits them. */
static void geometric_candidates(const mdsc_oracle_state* s, double min_s, int** start_out, int** list_out) {
  const int TP = s->n;
  int* cnt = (int*)calloc((size_t)TP + 1, sizeof(int));
  int* tmp_n = (int*)calloc(TP > 0 ? TP : 1, sizeof(int));
  int** tmp = (int**)calloc(TP > 0 ? TP : 1, sizeof(int*));
#pragma omp parallel for schedule(dynamic, 64)
  for (int A = 0; A < TP; ++A) {
    int cap = 16, m = 0;
    int* v = (int*)malloc(sizeof(int) * cap);
    for (int B = 0; B < TP; ++B) {
      if (B == A) continue;
      double r2 = 0.;
      for (int a = 0; a < 3; ++a) {
        double d = s->r[3 * A + a] - s->r[3 * B + a];
        d -= s->L[a] * floor(d / s->L[a] + 0.5);
        r2 += d * d;
      }
      const double reach = 0.5 * (s->len[A] + s->len[B]) + (s->dia[A] + s->dia[B]) / 2 + min_s;
      if (r2 > reach * reach * (1. + 1e-9) + 1e-9) continue;
      if (m == cap) {
        cap *= 2;
        v = (int*)realloc(v, sizeof(int) * cap);
      }
      v[m++] = B;
    }
    tmp[A] = v;
    tmp_n[A] = m;
  }
  for (int A = 0; A < TP; ++A) cnt[A + 1] = cnt[A] + tmp_n[A];
  int* list = (int*)malloc(sizeof(int) * (cnt[TP] > 0 ? cnt[TP] : 1));
  for (int A = 0; A < TP; ++A) {
    memcpy(list + cnt[A], tmp[A], sizeof(int) * tmp_n[A]);
    free(tmp[A]);
  }
  free(tmp);
  free(tmp_n);
  *start_out = cnt;
  *list_out = list;
}

static int clust_bfs(mdsc_oracle_state* s, const bond_rule* br, mdsc_mt19937* ran) {
  const int TP = s->n;
  /* the geometric test visits only the partners within reach (same order) */
  int *cstart = NULL, *clist = NULL;
  if (!br->energy) geometric_candidates(s, br->v, &cstart, &clist);
  int* NI = (int*)malloc(sizeof(int) * (TP > 0 ? TP : 1)); /* remaining, ascending */
  int nrem = TP;
  for (int j = 0; j < TP; ++j) NI[j] = j;
  char* added = (char*)calloc(TP > 0 ? TP : 1, 1);
  char* locadd = (char*)malloc(TP > 0 ? TP : 1);
  int* queue = (int*)malloc(sizeof(int) * (TP > 0 ? TP : 1));
  int n_clust = 0;
  while (nrem > 0) {
    /* rnd_part, :2950-2970 */
    double rnd = mdsc_mt_uniform(ran);
    int ip = (int)floor(rnd * nrem);
    int I = NI[ip];
    memset(locadd, 0, TP);
    added[I] = 1;
    locadd[I] = 1;
    if (s->clust) s->clust[I] = n_clust;
    memmove(&NI[ip], &NI[ip + 1], sizeof(int) * (nrem - ip - 1));
    --nrem;
    int qh = 0, qt = 0;
    queue[qt++] = I;
    /* clust_gen breadth-first growth, :3074-3145 */
    while (qh < qt) {
      int ii = queue[qh];
      const int jn = cstart ? cstart[ii + 1] - cstart[ii] : TP;
      for (int q = 0; q < jn; ++q) {
        const int j = cstart ? clist[cstart[ii] + q] : q;
        if (locadd[j]) continue;
        if (bonded(s, ii, j, br)) {
          if (!added[j]) {
            queue[qt++] = j;
            int loc = 0;
            for (int q = 0; q < nrem; ++q)
              if (NI[q] == j) {
                loc = q;
                break;
              }
            memmove(&NI[loc], &NI[loc + 1], sizeof(int) * (nrem - loc - 1));
            --nrem;
            locadd[j] = 1;
            added[j] = 1;
            if (s->clust) s->clust[j] = n_clust;
          }
          /* else: the reference logs "classifies for 2 clusters" and moves on */
        }
      }
      ++qh;
    }
    ++n_clust;
  }
  free(NI);
  free(added);
  free(locadd);
  free(queue);
  free(cstart);
  free(clist);
  return n_clust;
}

int mdsc_or_clust_conf(mdsc_oracle_state* s, double min_s, mdsc_mt19937* ran) {
  const bond_rule br = {0, min_s};
  return clust_bfs(s, &br, ran);
}

/* clust_conf's labelling over the energy criterion: bonds U_pair < -u_bond */
int mdsc_or_clust_energy(mdsc_oracle_state* s, double u_bond, mdsc_mt19937* ran) {
  const bond_rule br = {1, u_bond};
  return clust_bfs(s, &br, ran);
}

void* mdsc_or_rng_new(unsigned long seed) {
  mdsc_mt19937* g = (mdsc_mt19937*)malloc(sizeof(mdsc_mt19937));
  mdsc_mt_seed(g, seed);
  return g;
}
double mdsc_or_rng_uniform(void* g) { return mdsc_mt_uniform((mdsc_mt19937*)g); }
void mdsc_or_rng_free(void* g) { free(g); }
int mdsc_or_clust_conf_rng(mdsc_oracle_state* s, double min_s, void* g) {
  return mdsc_or_clust_conf(s, min_s, (mdsc_mt19937*)g);
}
int mdsc_or_clust_energy_rng(mdsc_oracle_state* s, double u_bond, void* g) {
  return mdsc_or_clust_energy(s, u_bond, (mdsc_mt19937*)g);
}

/* ------------------------------------------------------------------ */
/* driver loop body, v25/main.cpp:458-708                              */
/* ------------------------------------------------------------------ */
static double round12(double x) {
  /* compConf.dat keeps positions with 12 decimals (v25/functions.cpp:1344) */
  char buf[64];
  snprintf(buf, sizeof(buf), "%.12f", x);
  return strtod(buf, NULL);
}

static int md_build_list(mdsc_or_md* md, mdsc_oracle_state* s) {
  int n = s->n;
  int* counts = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
  int tot = mdsc_or_neigh_list(s, md->r_list_max, counts, md->nb_idx, md->nb_cap);
  if (tot > md->nb_cap) {
    free(md->nb_idx);
    md->nb_cap = tot + 1024;
    md->nb_idx = (int*)malloc(sizeof(int) * md->nb_cap);
    mdsc_or_neigh_list(s, md->r_list_max, counts, md->nb_idx, md->nb_cap);
  }
  md->nb_start[0] = 0;
  for (int i = 0; i < n; ++i) md->nb_start[i + 1] = md->nb_start[i] + counts[i];
  free(counts);
  for (int k = 0; k < 3 * n; ++k) md->saved_r[k] = round12(s->r[k]);
  md->list_builds++;
  return 1;
}

/* check_list, v25/functions.cpp:1356-1394, against the saved positions */
static int md_check_list(mdsc_or_md* md, const mdsc_oracle_state* s) {
  double dismax = 0.;
  for (int i = 0; i < s->n; ++i) {
    for (int a = 0; a < 3; ++a) {
      double D = s->r[3 * i + a] - md->saved_r[3 * i + a];
      D -= s->L[a] * floor(D / s->L[a] + 0.5);
      if (fabs(D) > dismax) dismax = fabs(D);
    }
  }
  dismax = 2. * sqrt(3. * dismax * dismax);
  return dismax > md->r_list_max - md->r_list_min;
}

static int md_forces(mdsc_or_md* md, mdsc_oracle_state* s) {
  for (int k = 0; k < 3 * s->n; ++k) s->F[k] = s->T[k] = 0.;
  md->Uss = md->Wss = 0.;
  if (!mdsc_or_force_sc_list(s, md->sr_cut, md->nb_start, md->nb_idx, &md->Uss, &md->Wss, md->PTss))
    return 0;
  md->UdipR = 0.;
  mdsc_or_force_dipR(s, md->tab, &md->UdipR, md->PTdipR);
  md->UdipK = 0.;
  mdsc_or_force_dipK(s, md->K_max, md->alpha, md->kvec, &md->UdipK, md->PTdipK);
  mdsc_or_ext_field(s, md->B, &md->Uext);
  return 1;
}

int mdsc_or_md_init(mdsc_or_md* md, mdsc_oracle_state* s, double dt, double temp, double Q,
                    double gamma, double xi0, double sr_cut, int K_max, int ksq_max, double alpha,
                    const double B[3], int cl_fr, double min_s) {
  memset(md, 0, sizeof(*md));
  md->dt = dt;
  md->temp = temp;
  md->sr_cut = sr_cut;
  md->alpha = alpha;
  md->K_max = K_max;
  md->ksq_max = ksq_max;
  md->cl_fr = cl_fr;
  md->min_s = min_s;
  for (int a = 0; a < 3; ++a) md->B[a] = B[a];
  mdsc_or_thermo_init(&md->thermo, Q, gamma, xi0);
  mdsc_mt_seed(&md->ran, 1);
  /* list radii, v25/main.cpp:460-463 (d_min, d_max over all particles) */
  double dmax = 0, dmin = 1.e+6;
  for (int i = 0; i < s->n; ++i) {
    if (s->len[i] + s->dia[i] > dmax) dmax = s->len[i] + s->dia[i];
    if (s->dia[i] < dmin) dmin = s->dia[i];
  }
  md->r_list_min = sr_cut + 0.1 * dmin;
  if (md->r_list_min < 1.5 * dmax) md->r_list_min = 1.5 * dmax;
  md->r_list_max = md->r_list_min + 0.9 * dmin;
  md->tab = (double*)malloc(sizeof(double) * 32768 * 3);
  mdsc_or_tabul(alpha, md->tab);
  md->kvec = (double*)malloc(sizeof(double) * (K_max + 1) * (K_max + 1) * (K_max + 1));
  mdsc_or_wave_v(md->kvec, s->L, alpha, K_max, ksq_max);
  md->nb_start = (int*)malloc(sizeof(int) * (s->n + 1));
  md->nb_cap = 64 * s->n + 1024;
  md->nb_idx = (int*)malloc(sizeof(int) * md->nb_cap);
  md->saved_r = (double*)malloc(sizeof(double) * 3 * (s->n > 0 ? s->n : 1));
  md_build_list(md, s);
  if (!md_forces(md, s)) return 0;
  md->Uself = mdsc_or_self_ener(s);
  return 1;
}

int mdsc_or_md_step(mdsc_or_md* md, mdsc_oracle_state* s) {
  double K[2] = {0., 0.};
  if (md->step % 100 == 0) mdsc_or_renorm(s);
  mdsc_or_moveTher(&md->thermo, md->temp, md->dt, K, s->n, 0);
  mdsc_or_moveP(s, md->thermo.xi, md->dt, 0, K, md->PTkin);
  mdsc_or_moveTher(&md->thermo, md->temp, md->dt, K, s->n, 1);
  mdsc_or_moveX(s, md->dt);
  if (!md_forces(md, s)) return 0;
  mdsc_or_moveP(s, md->thermo.xi, md->dt, 1, K, md->PTkin);
  mdsc_or_moveTher(&md->thermo, md->temp, md->dt, K, s->n, 2);
  md->K[0] = K[0];
  md->K[1] = K[1];
  if (md_check_list(md, s)) md_build_list(md, s);
  if (md->cl_fr > 0 && md->step % md->cl_fr == 0) mdsc_or_clust_conf(s, md->min_s, &md->ran);
  md->step++;
  return 1;
}

void mdsc_or_md_obs(const mdsc_or_md* md, double* out) {
  /* K_t, K_r, Uss, Wss, UdipR, UdipK, Uext, Uself, xi_t, xi_r, steps, list builds */
  out[0] = md->K[0];
  out[1] = md->K[1];
  out[2] = md->Uss;
  out[3] = md->Wss;
  out[4] = md->UdipR;
  out[5] = md->UdipK;
  out[6] = md->Uext;
  out[7] = md->Uself;
  out[8] = md->thermo.xi[0];
  out[9] = md->thermo.xi[1];
  out[10] = (double)md->step;
  out[11] = (double)md->list_builds;
  for (int k = 0; k < 9; ++k) {
    out[12 + k] = md->PTkin[k];
    out[21 + k] = md->PTss[k];
    out[30 + k] = md->PTdipR[k];
    out[39 + k] = md->PTdipK[k];
  }
}

void mdsc_or_md_set_thermo(mdsc_or_md* md, const double xi[2], const double strn[2]) {
  md->thermo.xi[0] = xi[0];
  md->thermo.xi[1] = xi[1];
  md->thermo.strn[0] = strn[0];
  md->thermo.strn[1] = strn[1];
}

/* the step's real-space table with entries beyond rc zeroed, and the
   forces of the current state again with it (as mdsc_or_md_init left them) */
int mdsc_or_md_mask_table(mdsc_or_md* md, mdsc_oracle_state* s, double rc) {
  mdsc_or_mask_table(md->tab, rc);
  return md_forces(md, s);
}

void mdsc_or_md_free(mdsc_or_md* md) {
  free(md->tab);
  free(md->kvec);
  free(md->nb_start);
  free(md->nb_idx);
  free(md->saved_r);
  memset(md, 0, sizeof(*md));
}

/* ------------------------------------------------------------------ */
/* observables outside the step                                        */
/* ------------------------------------------------------------------ */
/* acc_correl (v25/functions.cpp:2400-2470) for one species: the intra
   histograms, pair by pair (i < j) in the reference's order and arithmetic.
   hist[f * nbins + bin], f = 000, 110, 112, 220, accumulates.  Pairs whose
   bin is >= nbins (distance at the very corner of the box) are skipped. */
void mdsc_or_acc_correl(const mdsc_oracle_state* s, double bar_w, int nbins, double* hist) {
  const double* L = s->L;
  for (int f = 0; f < s->n - 1; ++f) {
    const double* ri = s->r + 3 * f;
    const double* oi = s->O + 9 * f + 6;
    for (int g = f + 1; g < s->n; ++g) {
      const double* rj = s->r + 3 * g;
      const double* oj = s->O + 9 * g + 6;
      double XIJ = ri[0] - rj[0];
      XIJ -= L[0] * floor(XIJ / L[0] + 0.5);
      double YIJ = ri[1] - rj[1];
      YIJ -= L[1] * floor(YIJ / L[1] + 0.5);
      double ZIJ = ri[2] - rj[2];
      ZIJ -= L[2] * floor(ZIJ / L[2] + 0.5);
      const double RIJSQ = XIJ * XIJ + YIJ * YIJ + ZIJ * ZIJ;
      const double RIJ = sqrt(RIJSQ);
      const double dot = oi[0] * oj[0] + oi[1] * oj[1] + oi[2] * oj[2];
      const double dotsq = dot * dot;
      const double doti = (oi[0] * XIJ + oi[1] * YIJ + oi[2] * ZIJ) / RIJ;
      const double dotj = (oj[0] * XIJ + oj[1] * YIJ + oj[2] * ZIJ) / RIJ;
      const int bin = (int)floor(RIJ / bar_w);
      if (bin < 0 || bin >= nbins) continue;
      hist[0 * nbins + bin] += 2.;
      hist[1 * nbins + bin] += 2. * dot;
      hist[2 * nbins + bin] += 2. * (3. * doti * dotj - dot);
      hist[3 * nbins + bin] += 3. * dotsq - 1.;
    }
  }
}

/* acc_correl (v25/functions.cpp:2400-2470) with nsp species, contiguous
   blocks of counts[k] particles (calc_II / rev_II numbering).  hist: the
   nsp species blocks (intra: 2, 2 dot, 2 (3 doti dotj - dot), 3 dot^2 - 1),
   then the species-pair blocks (0,1), (0,2), ..., (1,2), ... (inter: 1, dot,
   3 doti dotj - dot, (3 dot^2 - 1) / 2), each 4 x nbins; accumulates. */
void mdsc_or_acc_correl_species(const mdsc_oracle_state* s, int nsp, const int* counts, double bar_w,
                                int nbins, double* hist) {
  const double* L = s->L;
  int* sp = (int*)malloc(sizeof(int) * (s->n > 0 ? s->n : 1));
  int q = 0;
  for (int k = 0; k < nsp; ++k)
    for (int c = 0; c < counts[k]; ++c) sp[q++] = k;
  for (int f = 0; f < s->n - 1; ++f) {
    const double* ri = s->r + 3 * f;
    const double* oi = s->O + 9 * f + 6;
    for (int g = f + 1; g < s->n; ++g) {
      const double* rj = s->r + 3 * g;
      const double* oj = s->O + 9 * g + 6;
      double XIJ = ri[0] - rj[0];
      XIJ -= L[0] * floor(XIJ / L[0] + 0.5);
      double YIJ = ri[1] - rj[1];
      YIJ -= L[1] * floor(YIJ / L[1] + 0.5);
      double ZIJ = ri[2] - rj[2];
      ZIJ -= L[2] * floor(ZIJ / L[2] + 0.5);
      const double RIJSQ = XIJ * XIJ + YIJ * YIJ + ZIJ * ZIJ;
      const double RIJ = sqrt(RIJSQ);
      const double dot = oi[0] * oj[0] + oi[1] * oj[1] + oi[2] * oj[2];
      const double dotsq = dot * dot;
      const double doti = (oi[0] * XIJ + oi[1] * YIJ + oi[2] * ZIJ) / RIJ;
      const double dotj = (oj[0] * XIJ + oj[1] * YIJ + oj[2] * ZIJ) / RIJ;
      const int bin = (int)floor(RIJ / bar_w);
      if (bin < 0 || bin >= nbins) continue;
      const int m = sp[f], n = sp[g];
      if (m == n) {
        double* h = hist + (size_t)m * 4 * nbins;
        h[0 * nbins + bin] += 2.;
        h[1 * nbins + bin] += 2. * dot;
        h[2 * nbins + bin] += 2. * (3. * doti * dotj - dot);
        h[3 * nbins + bin] += 3. * dotsq - 1.;
      } else {
        /* the reference's Vc table numbers the pairs m < n row by row */
        const int cc = m * (2 * nsp - m - 1) / 2 + (n - m - 1);
        double* h = hist + (size_t)(nsp + cc) * 4 * nbins;
        h[0 * nbins + bin] += 1.;
        h[1 * nbins + bin] += dot;
        h[2 * nbins + bin] += 3. * doti * dotj - dot;
        h[3 * nbins + bin] += (3. * dotsq - 1.) / 2;
      }
    }
  }
  free(sp);
}

/* eigenvalues d[3] and eigenvectors (columns of V) of a symmetric 3x3
   matrix by cyclic Jacobi rotations (Golub & Van Loan, Matrix
   Computations, 8.5): each rotation zeroes one off-diagonal element. */
static void sym3_eigen(const double A_in[3][3], double d[3], double V[3][3]) {
  double A[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      A[i][j] = A_in[i][j];
      V[i][j] = i == j ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 64; ++sweep) {
    const double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
    const double scale = fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]) + 1e-300;
    if (off <= 1e-15 * scale) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (A[p][q] == 0.0) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 3; ++k) {  /* A <- A J */
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - sn * akq;
          A[k][q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {  /* A <- J^T A */
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - sn * aqk;
          A[q][k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {  /* V <- V J */
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - sn * vkq;
          V[k][q] = sn * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) d[i] = A[i][i];
}

/* oo_params (v25/functions.cpp:2702-2748) with Qmat_3d (:3426-3445): the
   total dipole moment M = sum mu o (lab frame), the nematic order G2 = the
   largest |eigenvalue| of Q = sum (3 o o^T - 1) / (2 N) (accumulated in
   FP32 as Qmat_3d does) and G1 = |sum o . e| / N along its eigenvector.
   The eigen solver is this file's own (sym3_eigen), not the reference's, so
   G1 and G2 agree with the reference to FP32 precision, not bit for bit. */
void mdsc_or_oo_params(const mdsc_oracle_state* s, double* G1, double* G2, double M[3]) {
  for (int a = 0; a < 3; ++a) M[a] = 0.0;
  for (int i = 0; i < s->n; ++i)
    for (int w = 0; w < s->nd; ++w) {
      double pos[3], ori[3], lev[3], mu;
      dip_lab(s, i, w, pos, ori, lev, &mu);
      for (int a = 0; a < 3; ++a) M[a] += mu * ori[a];
    }
  float Q[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int k = 0; k < s->n; ++k) {
    const double* o = s->O + 9 * k + 6;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        Q[i][j] += ((float)(3 * o[i] * o[j]) - (float)(i == j ? 1 : 0)) / (2 * s->n);
  }
  double Qd[3][3], d[3], V[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Qd[i][j] = Q[i][j];
  sym3_eigen(Qd, d, V);
  const double e1 = fabs(d[0]), e2 = fabs(d[1]), e3 = fabs(d[2]);
  int c;
  if (e1 >= e2 && e1 >= e3) c = 0;
  else if (e2 > e1 && e2 >= e3) c = 1;
  else c = 2;
  *G2 = fabs(d[c]);
  double Ve[3] = {V[0][c], V[1][c], V[2][c]};
  const double nv = sqrt(Ve[0] * Ve[0] + Ve[1] * Ve[1] + Ve[2] * Ve[2]);
  for (int a = 0; a < 3; ++a) Ve[a] /= nv;
  double g1 = 0.0;
  for (int k = 0; k < s->n; ++k) {
    const double* o = s->O + 9 * k + 6;
    g1 += Ve[0] * o[0] + Ve[1] * o[1] + Ve[2] * o[2];
  }
  *G1 = fabs(g1) / s->n;
}
