// Function-level harness around the reference's own, unmodified hot-path
// routines (v25/functions.cpp, v25/classes.cpp).  TEST INFRASTRUCTURE ONLY:
// it is compiled by oracle/build_ref.sh into oracle/_ref/libmdsc_ref.so,
// together with the reference sources where they lie, and is used to pin
// the C restatement (oracle/mdsc_oracle.c) and to make golden fixtures.
//
// The caller describes one system as structure-of-arrays (mdsc_ref_state,
// identical to mdsc_oracle_state in oracle/mdsc_oracle.h).  Each call builds
// the reference's particle container with one species and per-particle
// shape, mass, inertia and dipoles -- the reference reads all of these per
// particle on the hot path (v25/functions.cpp:1432-1433,1584-1595,2113-2114)
// -- calls the reference routine, and writes the state back.

#include "functions.hpp"
#include <vector>
#include <deque>
#include <algorithm>
#include <cmath>

extern "C" {

struct mdsc_ref_state {
  int n;         // particles
  int nd;        // dipoles per particle
  double L[3];   // box edges
  double* r;     // n*3 centre of mass
  double* p;     // n*3 momentum
  double* O;     // n*9 rows = body axes in the lab frame (row 2 = rod axis)
  double* l;     // n*3 angular momentum (lab frame)
  double* F;     // n*3 force
  double* T;     // n*3 torque
  const double* len;   // n rod length L
  const double* dia;   // n diameter D
  const double* mass;  // n
  const double* dip;   // n*nd*5: offset along axis, body-frame direction (3), moment
  int* clust;          // n cluster label
};

}  // extern "C"

namespace {

void build_part(const mdsc_ref_state* s, Dynvec<Dynvec<Spherocyl> >& part, part_num& NP) {
  Dynvec<int> np(1);
  np[0] = s->n;
  NP.init(1, np);
  part.set_size(1);
  part[0].set_size(s->n);
  for (int i = 0; i < s->n; ++i) {
    Spherocyl& P = part[0][i];
    double sh[2] = {s->len[i], s->dia[i]};
    P.set_id(i);
    P.set_shape(sh);
    P.set_mass(s->mass[i]);
    P.set_inertia();
    P.set_pos(&s->r[3 * i]);
    P.set_mom(&s->p[3 * i]);
    Matrix<double> o(3, 3);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) o[a][b] = s->O[9 * i + 3 * a + b];
    P.set_omat(o);
    P.set_angm(&s->l[3 * i]);
    P.set_F(&s->F[3 * i]);
    P.set_T(&s->T[3 * i]);
    Matrix<double> u(s->nd, 5);
    for (int w = 0; w < s->nd; ++w)
      for (int c = 0; c < 5; ++c) u[w][c] = s->dip[(i * s->nd + w) * 5 + c];
    P.set_dip(u);
    P.set_clust(s->clust ? s->clust[i] : 0);
  }
}

void write_back(mdsc_ref_state* s, Dynvec<Dynvec<Spherocyl> >& part) {
  for (int i = 0; i < s->n; ++i) {
    Spherocyl& P = part[0][i];
    P.get_pos(&s->r[3 * i]);
    P.get_mom(&s->p[3 * i]);
    Matrix<double> o(3, 3);
    P.get_omat(o);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) s->O[9 * i + 3 * a + b] = o[a][b];
    P.get_angm(&s->l[3 * i]);
    P.get_F(&s->F[3 * i]);
    P.get_T(&s->T[3 * i]);
    if (s->clust) s->clust[i] = P.get_clust();
  }
}

void copy_pt(double PT[3][3], double* out) {
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) out[3 * a + b] = PT[a][b];
}

double g_tab[32768][3];  // tabul() table, v25/main.cpp:429-433

}  // namespace

extern "C" {

// The reference sizes its dynamic OpenMP chunks as floor(N / (16 * threads))
// (e.g. v25/functions.cpp:1412-1414); for N < 16 * threads that chunk is 0
// and the loop never finishes, so the harness runs with one thread unless
// told otherwise.  One thread is also what makes it deterministic.
void mdsc_ref_set_threads(int n) { omp_set_num_threads(n < 1 ? 1 : n); }

// spherocyl_dist (v25/functions.cpp:89-489) for particles i, j of the state
double mdsc_ref_seg_dist(mdsc_ref_state* s, int i, int j, double* dAB, double* st) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  double ri[3], rj[3], rij[3];
  part[0][i].get_pos(ri);
  part[0][j].get_pos(rj);
  for (int a = 0; a < 3; ++a) {
    rij[a] = ri[a] - rj[a];
    rij[a] -= s->L[a] * floor(rij[a] / s->L[a] + 0.5);
  }
  return spherocyl_dist(part[0][i], part[0][j], s->L, rij, dAB, st);
}

// neigh_list (v25/functions.cpp:1298-1334); out: CSR of the half list
int mdsc_ref_neigh_list(mdsc_ref_state* s, double r_list, int* counts, int* idx, int cap) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  std::vector<std::deque<int> > nb(s->n);
  neigh_list(part, NP, s->L, nb.data(), r_list);
  int tot = 0;
  for (int i = 0; i < s->n; ++i) {
    counts[i] = (int)nb[i].size();
    for (size_t k = 0; k < nb[i].size(); ++k) {
      if (tot < cap) idx[tot] = nb[i][k];
      ++tot;
    }
  }
  return tot;
}

// force_sc (v25/functions.cpp:1397-1553) over the list neigh_list builds
// with radius r_list.  F and T accumulate as in the reference.
int mdsc_ref_force_sc(mdsc_ref_state* s, double r_cut, double r_list, double* U, double* W,
                      double* PT) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  std::vector<std::deque<int> > nb(s->n);
  neigh_list(part, NP, s->L, nb.data(), r_list);
  double pt[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double u = 0, w = 0;
  bool ok = force_sc(part, NP, s->L, r_cut, u, w, pt, nb.data());
  *U = u;
  *W = w;
  copy_pt(pt, PT);
  write_back(s, part);
  return ok ? 1 : 0;
}

// tabul (v25/functions.cpp:1680-1704): 32768 x 3 table
void mdsc_ref_tabul(double alpha, double* tab_out) {
  tabul(g_tab, alpha);
  for (int i = 0; i < 32768; ++i)
    for (int c = 0; c < 3; ++c) tab_out[3 * i + c] = g_tab[i][c];
}

// force_dipR (v25/functions.cpp:1555-1678) with the table of tabul(alpha)
void mdsc_ref_force_dipR(mdsc_ref_state* s, double alpha, double* U, double* PT) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  tabul(g_tab, alpha);
  double pt[3][3];
  double u = 0;
  force_dipR(part, NP, s->L, g_tab, u, pt);
  *U = u;
  copy_pt(pt, PT);
  write_back(s, part);
}

// force_dipR with tabul's table zeroed beyond rc (entry i-1 holds
// r = 0.5 * 200.2 * i / 32768): the real-space cutoff of this library's
// rc_real, through the reference's own routine
void mdsc_ref_force_dipR_cut(mdsc_ref_state* s, double alpha, double rc, double* U, double* PT) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  tabul(g_tab, alpha);
  const double extL = 200 * 1.001;
  for (int i = 1; i < 32769; i++)
    if (0.5 * extL * i / 32768 > rc) g_tab[i - 1][0] = g_tab[i - 1][1] = g_tab[i - 1][2] = 0.;
  double pt[3][3];
  double u = 0;
  force_dipR(part, NP, s->L, g_tab, u, pt);
  *U = u;
  copy_pt(pt, PT);
  write_back(s, part);
}

// force_dipK (v25/functions.cpp:1706-1961) with Kvec from wave_v
// (v25/functions.cpp:1963-1990).  ksq_max > 0 zeroes Kvec outside
// nx^2+ny^2+nz^2 <= ksq_max, giving a spherical k-set.
void mdsc_ref_force_dipK(mdsc_ref_state* s, int K_max, double alpha, int ksq_max, double* U,
                         double* PT) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  Dynvec<Matrix<double> > Kvec;
  Kvec.set_size(K_max + 1);
  for (int i = 0; i < K_max + 1; ++i) {
    Kvec[i].set_size(K_max + 1, K_max + 1);
    Kvec[i].set_to(0.);
  }
  wave_v(Kvec, s->L, alpha, K_max);
  if (ksq_max > 0) {
    for (int x = 0; x <= K_max; ++x)
      for (int y = 0; y <= K_max; ++y)
        for (int z = 0; z <= K_max; ++z)
          if (x * x + y * y + z * z > ksq_max) Kvec[x][y][z] = 0.;
  }
  double pt[3][3];
  double u = 0;
  force_dipK(part, NP, s->L, K_max, alpha, Kvec, u, pt);
  *U = u;
  copy_pt(pt, PT);
  write_back(s, part);
}

// ext_field (v25/functions.cpp:1992-2025)
void mdsc_ref_ext_field(mdsc_ref_state* s, const double* B, double* U) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  double u = 0;
  ext_field(part, NP, B, u);
  *U = u;
  write_back(s, part);
}

// self_ener (v25/functions.cpp:2027-2069)
double mdsc_ref_self_ener(mdsc_ref_state* s) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  return self_ener(part, NP);
}

// moveX (v25/functions.cpp:2071-2092 -> v25/classes.cpp:228-304)
void mdsc_ref_moveX(mdsc_ref_state* s, double dt) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  moveX(part, NP, dt);
  write_back(s, part);
}

// moveP (v25/functions.cpp:2094-2184).  xi = thermostat coordinates.
void mdsc_ref_moveP(mdsc_ref_state* s, const double* xi, double dt, int last, double* K,
                    double* PT) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  Thermostat th[2];
  th[0].set_coo(xi[0]);
  th[1].set_coo(xi[1]);
  double pt[3][3];
  moveP(part, th, NP, dt, K, pt, last != 0);
  copy_pt(pt, PT);
  write_back(s, part);
}

// renorm (v25/classes.cpp:307-325) for every particle
void mdsc_ref_renorm(mdsc_ref_state* s) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  for (int i = 0; i < s->n; ++i) part[0][i].renorm();
  write_back(s, part);
}

// ---- random generators (gsl_rng stand-in) ----
void* mdsc_ref_rng_new(unsigned long seed) {
  gsl_rng* r = gsl_rng_alloc(gsl_rng_mt19937);
  gsl_rng_set(r, seed);
  return r;
}
double mdsc_ref_rng_uniform(void* r) { return gsl_rng_uniform((gsl_rng*)r); }
void mdsc_ref_rng_free(void* r) { gsl_rng_free((gsl_rng*)r); }

// clust_conf (v25/functions.cpp:3282-3324) with p_check = false, as the
// driver calls it (v25/main.cpp:703-708); labels land in s->clust.
void mdsc_ref_clust_conf(mdsc_ref_state* s, double min_s, void* rng) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  double dmax = 0;
  for (int i = 0; i < s->n; ++i) dmax = std::max(dmax, s->len[i] + s->dia[i]);
  clust_conf(part, NP, s->L, min_s, dmax, (gsl_rng*)rng, false);
  write_back(s, part);
}

// moveTher (v25/functions.cpp:2186-2218) on two thermostats whose state
// is (xi, stored normal) and whose generators are rng0 / rng1.
void mdsc_ref_moveTher(double* xi, double* strn, double Q, double gamma, void* rng0, void* rng1,
                       double temp, double dt, const double* K, double tpart, int mode) {
  // Thermostat objects own their generator and free it on destruction, so
  // the state is moved through heap objects that are never destroyed here.
  Thermostat* th = new Thermostat[2];
  gsl_rng* own[2];
  for (int i = 0; i < 2; ++i) {
    th[i].set_mass(Q);
    th[i].set_shr(gamma);
    th[i].set_coo(xi[i]);
    th[i].set_strn(strn[i]);
  }
  // swap our generators in: Thermostat keeps its generator in m_ran
  struct ThermoView {
    double m_Q, m_s, m_g;
    gsl_rng* m_ran;
    double m_strn;
  };
  static_assert(sizeof(ThermoView) == sizeof(Thermostat), "Thermostat layout");
  for (int i = 0; i < 2; ++i) {
    ThermoView* v = reinterpret_cast<ThermoView*>(&th[i]);
    own[i] = v->m_ran;
    v->m_ran = (gsl_rng*)(i == 0 ? rng0 : rng1);
  }
  moveTher(th, temp, dt, K, tpart, mode);
  for (int i = 0; i < 2; ++i) {
    xi[i] = th[i].get_coo();
    strn[i] = th[i].get_strn();
    ThermoView* v = reinterpret_cast<ThermoView*>(&th[i]);
    v->m_ran = own[i];
  }
  delete[] th;
}

}  // extern "C"

// acc_correl (v25/functions.cpp:2400-2470), one species: the intra
// histograms of this state added to hist[4*nbins] (000, 110, 112, 220).
// acc_correl does not check the bin against the matrix, so the matrix here
// reaches the largest minimum-image distance, half the box diagonal; only
// the first nbins bins are returned.
extern "C" void mdsc_ref_acc_correl(mdsc_ref_state* s, double bar_w, int nbins, double* hist) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  const double diag = 0.5 * sqrt(s->L[0] * s->L[0] + s->L[1] * s->L[1] + s->L[2] * s->L[2]);
  const int nfull = std::max(nbins, (int)floor(diag / bar_w) + 2);
  Dynvec<Matrix<double> > Hista(1), Histe(1);
  Hista[0].set_size(4, nfull);
  Hista[0].set_to(0.);
  acc_correl(part, Hista, Histe, s->L, bar_w, NP, nullptr);
  for (int f = 0; f < 4; ++f)
    for (int b = 0; b < nbins; ++b) hist[f * nbins + b] += Hista[0][f][b];
}

// oo_params (v25/functions.cpp:2702-2748): G1, G2 and the total moment M
extern "C" void mdsc_ref_oo_params(mdsc_ref_state* s, double* G1, double* G2, double* M) {
  Dynvec<Dynvec<Spherocyl> > part;
  part_num NP;
  build_part(s, part, NP);
  double g1 = 0, g2 = 0, m[3] = {0, 0, 0};
  oo_params(part, NP, g1, g2, m);
  *G1 = g1;
  *G2 = g2;
  for (int a = 0; a < 3; ++a) M[a] = m[a];
}

// acc_correl with nsp species of counts[k] contiguous particles: Hista per
// species, Histe per species pair (the driver's Vc numbering, v25/main.cpp:
// 118-143); hist gets the species blocks, then the pair blocks, 4 x nbins
// each (+=).
extern "C" void mdsc_ref_acc_correl_species(mdsc_ref_state* s, int nsp, const int* counts, double bar_w,
                                            int nbins, double* hist) {
  Dynvec<int> np(nsp);
  for (int k = 0; k < nsp; ++k) np[k] = counts[k];
  part_num NP;
  NP.init(nsp, np);
  Dynvec<Dynvec<Spherocyl> > part(nsp);
  int i = 0;
  for (int k = 0; k < nsp; ++k) {
    part[k].set_size(counts[k]);
    for (int q = 0; q < counts[k]; ++q, ++i) {
      Spherocyl& P = part[k][q];
      double sh[2] = {s->len[i], s->dia[i]};
      P.set_id(i);
      P.set_shape(sh);
      P.set_mass(s->mass[i]);
      P.set_inertia();
      P.set_pos(&s->r[3 * i]);
      Matrix<double> o(3, 3);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) o[a][b] = s->O[9 * i + 3 * a + b];
      P.set_omat(o);
    }
  }
  const int ns = nsp * (nsp - 1) / 2;
  cross* Vc = new cross[nsp];
  if (nsp > 1) {
    for (int n = 0; n < nsp; ++n) {
      Vc[n].C.set_size(nsp - 1);
      Vc[n].P.set_size(nsp - 1);
      Vc[n].T.set_size(nsp - 1);
    }
    std::vector<int> cct(nsp, 0);
    int cnt = 0;
    for (int m = 0; m < nsp - 1; ++m)
      for (int n = m + 1; n < nsp; ++n) {
        Vc[m].C[cct[m]] = cnt;
        Vc[m].P[cct[m]] = n;
        Vc[m].T[cct[m]] = true;
        cct[m]++;
        Vc[n].C[cct[n]] = cnt;
        Vc[n].P[cct[n]] = m;
        Vc[n].T[cct[n]] = false;
        cct[n]++;
        cnt++;
      }
  }
  const double diag = 0.5 * sqrt(s->L[0] * s->L[0] + s->L[1] * s->L[1] + s->L[2] * s->L[2]);
  const int nfull = std::max(nbins, (int)floor(diag / bar_w) + 2);
  Dynvec<Matrix<double> > Hista(nsp), Histe(ns > 0 ? ns : 1);
  for (int k = 0; k < nsp; ++k) {
    Hista[k].set_size(4, nfull);
    Hista[k].set_to(0.);
  }
  for (int k = 0; k < (ns > 0 ? ns : 1); ++k) {
    Histe[k].set_size(4, nfull);
    Histe[k].set_to(0.);
  }
  acc_correl(part, Hista, Histe, s->L, bar_w, NP, Vc);
  for (int k = 0; k < nsp + ns; ++k)
    for (int f = 0; f < 4; ++f)
      for (int b = 0; b < nbins; ++b)
        hist[((size_t)k * 4 + f) * nbins + b] += k < nsp ? Hista[k][f][b] : Histe[k - nsp][f][b];
  delete[] Vc;
}
