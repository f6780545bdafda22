/*
 * CPU restatement of the reference's MD-step routines, in plain C, FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle (the checker) for the GPU
 * path: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
 * it; the product library never links, loads or calls it.  Each routine
 * follows the reference function named beside it (file:line in the
 * reference project) operation for operation, so that, single-threaded and
 * built with -ffp-contract=off, it reproduces the reference bit for bit.
 * It is pinned against the reference itself (oracle/_ref, built from the
 * reference's unmodified sources by oracle/build_ref.sh) and against golden
 * fixtures made from it (tests/golden/).
 *
 * One system, structure of arrays, one species with per-particle shape,
 * mass and dipoles (the reference reads all of these per particle on the
 * hot path).  O holds the orientation matrix row-major; its rows are the
 * body axes in the lab frame and row 2 is the rod axis (v25/classes.hpp:74).
 */
#ifndef MDSC_ORACLE_H
#define MDSC_ORACLE_H

#include "mt19937.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int n;        /* particles */
  int nd;       /* dipoles per particle */
  double L[3];  /* box edges */
  double* r;    /* n*3 */
  double* p;    /* n*3 */
  double* O;    /* n*9 */
  double* l;    /* n*3 */
  double* F;    /* n*3 */
  double* T;    /* n*3 */
  const double* len;  /* n */
  const double* dia;  /* n */
  const double* mass; /* n */
  const double* dip;  /* n*nd*5: offset along the axis, body-frame direction (3), moment */
  int* clust;         /* n, may be NULL */
} mdsc_oracle_state;

/* spherocyl_dist, v25/functions.cpp:89-489 */
double mdsc_or_seg_dist(const mdsc_oracle_state* s, int A, int B, const double rAB[3],
                        double dAB[3], double st[2]);
/* neigh_list, v25/functions.cpp:1298-1334: half list as CSR (counts, idx);
   returns the number of entries (idx holds at most cap of them) */
int mdsc_or_neigh_list(const mdsc_oracle_state* s, double r_list, int* counts, int* idx, int cap);
/* force_sc, v25/functions.cpp:1397-1553, over the half list of radius
   r_list.  F, T accumulate.  Returns 1, or 0 on the reference's abort. */
int mdsc_or_force_sc(mdsc_oracle_state* s, double r_cut, double r_list, double* U, double* W,
                     double PT[9]);
/* same, over a given CSR half list */
int mdsc_or_force_sc_list(mdsc_oracle_state* s, double r_cut, const int* start, const int* idx,
                          double* U, double* W, double PT[9]);
/* tabul, v25/functions.cpp:1680-1704 (32768 x 3) */
void mdsc_or_tabul(double alpha, double* tab);
/* tabul's table with the entries beyond a real-space cutoff rc zeroed */
void mdsc_or_mask_table(double* tab, double rc);
/* force_dipR, v25/functions.cpp:1555-1678 */
void mdsc_or_force_dipR(mdsc_oracle_state* s, const double* tab, double* U, double PT[9]);
/* wave_v, v25/functions.cpp:1963-1990, into kvec[(nx*(K+1)+ny)*(K+1)+nz];
   ksq_max > 0 zeroes entries outside nx^2+ny^2+nz^2 <= ksq_max */
void mdsc_or_wave_v(double* kvec, const double L[3], double alpha, int K_max, int ksq_max);
/* force_dipK, v25/functions.cpp:1706-1961 */
void mdsc_or_force_dipK(mdsc_oracle_state* s, int K_max, double alpha, const double* kvec,
                        double* U, double PT[9]);
/* ext_field, v25/functions.cpp:1992-2025 */
void mdsc_or_ext_field(mdsc_oracle_state* s, const double B[3], double* U);
/* self_ener, v25/functions.cpp:2027-2069 */
double mdsc_or_self_ener(const mdsc_oracle_state* s);
/* moveX, v25/functions.cpp:2071-2092 with translate/rotate, v25/classes.cpp:228-304 */
void mdsc_or_moveX(mdsc_oracle_state* s, double dt);
/* moveP, v25/functions.cpp:2094-2184 */
void mdsc_or_moveP(mdsc_oracle_state* s, const double xi[2], double dt, int last, double K[2],
                   double PT[9]);
/* renorm, v25/classes.cpp:307-325, every particle */
void mdsc_or_renorm(mdsc_oracle_state* s);
/* set_inertia, v25/classes.cpp:175-185 */
void mdsc_or_inertia(double L, double D, double mass, double I[3]);
/* gauss, v25/functions.cpp:1149-1156 */
void mdsc_or_gauss(double variance, double* rnd1, double* rnd2);

/* Thermostat pair (v25/classes.hpp:145-182): coordinate, stored normal and
   its MT19937 generator; seeds 1 and 2 in the driver (v25/main.cpp:179-188) */
typedef struct {
  double Q, g;
  double xi[2];
  double strn[2];
  mdsc_mt19937 rng[2];
} mdsc_or_thermo;
void mdsc_or_thermo_init(mdsc_or_thermo* th, double Q, double gamma, double xi0);
/* moveTher, v25/functions.cpp:2186-2218 */
void mdsc_or_moveTher(mdsc_or_thermo* th, double temp, double dt, const double K[2], double tpart,
                      int mode);

/* clust_conf with p_check = false, v25/functions.cpp:2950-3148,3282-3324:
   labels into s->clust, draws from ran.  Returns the number of clusters. */
int mdsc_or_clust_conf(mdsc_oracle_state* s, double min_s, mdsc_mt19937* ran);
/* energy criterion (an extension): pair energy, lower index A; labelling over
   bonds U_pair < -u_bond */
double mdsc_or_pair_energy(const mdsc_oracle_state* s, int A, int B);
int mdsc_or_clust_energy(mdsc_oracle_state* s, double u_bond, mdsc_mt19937* ran);

/* heap generator handles for callers without the struct layout */
void* mdsc_or_rng_new(unsigned long seed);
double mdsc_or_rng_uniform(void* g);
void mdsc_or_rng_free(void* g);
int mdsc_or_clust_conf_rng(mdsc_oracle_state* s, double min_s, void* g);
int mdsc_or_clust_energy_rng(mdsc_oracle_state* s, double u_bond, void* g);

/* One MD step of the reference driver's loop body, v25/main.cpp:520-708
   (no file output).  The context keeps what the driver keeps between
   steps: thermostats, neighbour list and its reference positions. */
typedef struct {
  double dt, temp, sr_cut, alpha, min_s, B[3];
  int K_max, ksq_max, cl_fr;
  double r_list_min, r_list_max;
  mdsc_or_thermo thermo;
  mdsc_mt19937 ran; /* cluster seeds, seeded 1 (v25/main.cpp:209-211) */
  double* tab;      /* 32768*3 */
  double* kvec;     /* (K+1)^3 */
  int* nb_start;    /* n+1 */
  int* nb_idx;
  int nb_cap;
  double* saved_r;  /* n*3, positions at the last list build, 12 decimals */
  long step;
  int list_builds;
  double Uself;
  /* observables of the last step (v25/main.cpp:626-649), totals not per particle */
  double K[2], Uss, Wss, UdipR, UdipK, Uext;
  double PTkin[9], PTss[9], PTdipR[9], PTdipK[9];
} mdsc_or_md;
int mdsc_or_md_init(mdsc_or_md* md, mdsc_oracle_state* s, double dt, double temp, double Q,
                    double gamma, double xi0, double sr_cut, int K_max, int ksq_max, double alpha,
                    const double B[3], int cl_fr, double min_s);
int mdsc_or_md_mask_table(mdsc_or_md* md, mdsc_oracle_state* s, double rc);
int mdsc_or_md_step(mdsc_or_md* md, mdsc_oracle_state* s);
void mdsc_or_md_free(mdsc_or_md* md);
/* observables of the last step: K_t, K_r, Uss, Wss, UdipR, UdipK, Uext,
   Uself, xi_t, xi_r, steps, list builds, then PTkin, PTss, PTdipR, PTdipK
   (9 each) -- 48 doubles */
void mdsc_or_md_obs(const mdsc_or_md* md, double* out);
void mdsc_or_md_set_thermo(mdsc_or_md* md, const double xi[2], const double strn[2]);

/* number of OpenMP threads the routines may use (1 = serial, bit-exact) */
void mdsc_or_set_threads(int n);

/* acc_correl, v25/functions.cpp:2400-2470 (one species): hist[4*nbins] += */
void mdsc_or_acc_correl(const mdsc_oracle_state* s, double bar_w, int nbins, double* hist);
/* the same with nsp species of counts[k] contiguous particles: the species
   blocks, then the species-pair blocks, each 4 x nbins (+=) */
void mdsc_or_acc_correl_species(const mdsc_oracle_state* s, int nsp, const int* counts, double bar_w,
                                int nbins, double* hist);
/* oo_params, v25/functions.cpp:2702-2748: G1, G2 and the total moment M */
void mdsc_or_oo_params(const mdsc_oracle_state* s, double* G1, double* G2, double M[3]);

#ifdef __cplusplus
}
#endif
#endif
