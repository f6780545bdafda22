// gb300_bridge.cpp -- the reference's hot path (v25/functions.hpp) on a
// GB300 through the C ABI of include/mdsc.h.
//
// A maintainer of the reference adds this file next to v25/main.cpp and
// links the program against libmdsc.so:
//
//   g++ -O2 -fopenmp -I. -I<repo>/include main.cpp classes.cpp functions.cpp \
//       jacobi.c gb300_bridge.cpp -L<repo>/mdspherocyl_gb300/_lib -lmdsc -lgsl
//
// Two forms are offered.
//  * gb300::step replaces the loop body of v25/main.cpp:558-708 for any
//    number of steps: the state stays on the GPU, and only the observables
//    come back unless the driver asks for the configuration.
//  * gb300::force_sc, force_dipR, force_dipK, ext_field, self_ener, moveX,
//    moveP, clust_conf keep the reference's own signatures
//    (v25/functions.hpp:38-52,107-108).  Each uploads the particles, runs
//    the function on the GPU and writes the results back, so one function
//    at a time can be checked against the original.
//
// Particles are flattened in the reference's own global order (rev_II).
// Dipoles travel in the body frame -- offset along the axis, direction in
// body axes, moment -- the table Spherocyl::set_dip takes
// (v25/classes.cpp:148-173).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <vector>

#include "classes.hpp"
#include "functions.hpp"
#include "mdsc.h"

namespace gb300 {

struct Bridge {
  mdsc_batch* b = nullptr;
  int n = 0, nd = 0;
  std::vector<double> r, p, O, l, F, T, len, dia, mass, dip;
  std::vector<int> clust;
  mdsc_host_state hs{};
};
static Bridge B;

static void check(mdsc_status s, const char* what) {
  if (s == MDSC_OK) return;
  char msg[512] = "";
  if (B.b) mdsc_last_error(B.b, msg, sizeof msg);
  std::fprintf(stderr, "%s: status %d %s\n", what, (int)s, msg);
  if (s != MDSC_ERR_OVERLAP) std::exit(1);  // overlap: the caller decides, as with force_sc's false
}

// The largest dipole count of any particle (the batch's dipoles per particle).
int max_dipoles(const Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP) {
  int nd = 0;
  for (int k = 0; k < NP.get_Tpart(); ++k) {
    int m = 0, i = 0;
    rev_II(NP, m, i, k);
    if (part[m][i].get_ndips() > nd) nd = part[m][i].get_ndips();
  }
  return nd;
}

// Host buffers for n particles of nd dipoles each (no GPU involved).
void size_buffers(int n, int nd) {
  B.n = n;
  B.nd = nd;
  const size_t m = n;
  B.r.assign(3 * m, 0.0); B.p.assign(3 * m, 0.0); B.O.assign(9 * m, 0.0); B.l.assign(3 * m, 0.0);
  B.F.assign(3 * m, 0.0); B.T.assign(3 * m, 0.0);
  B.len.assign(m, 0.0); B.dia.assign(m, 0.0); B.mass.assign(m, 0.0);
  B.dip.assign(m * (nd > 0 ? nd : 1) * 5, 0.0);
  B.clust.assign(m, 0);
  B.hs.r = B.r.data(); B.hs.p = B.p.data(); B.hs.O = B.O.data(); B.hs.l = B.l.data();
  B.hs.F = B.F.data(); B.hs.T = B.T.data();
  B.hs.len = B.len.data(); B.hs.dia = B.dia.data(); B.hs.mass = B.mass.data();
  B.hs.dip = B.dip.data(); B.hs.clust = B.clust.data();
}

// Called once after r_input / chrg_conf with the run's parameters
// (input.txt, v25/functions.cpp:26-82).
void init(const part_num& NP, const Dynvec<Dynvec<Spherocyl> >& part, const double L[3], double alpha,
          int K_max, double dt, double temp, double Q, double gamma, double xi0, const double Bf[3],
          double min_s, int cl_fr, double sr_cut) {
  size_buffers(NP.get_Tpart(), max_dipoles(part, NP));
  mdsc_system_desc d;
  std::memset(&d, 0, sizeof d);
  d.n = B.n;
  d.nd = B.nd;
  for (int a = 0; a < 3; ++a) {
    d.box[a] = L[a];
    d.B[a] = Bf[a];
  }
  d.alpha = alpha;
  d.K_max = K_max;
  d.ksq_max = 0;  // 0: the reference's full k cube
  d.sr_cut = sr_cut;
  d.dt = dt;
  d.temp = temp;
  d.Q = Q;
  d.gamma = gamma;
  d.xi0 = xi0;
  d.min_s = min_s;
  d.cl_fr = cl_fr;
  d.rc_real = 0;  // all minimum-image pairs, as force_dipR sums them (> 0: its table zeroed beyond rc_real)
  d.thermo_seed[0] = 1;
  d.thermo_seed[1] = 2;
  d.cluster_seed = 1;
  d.cluster_skip = 0;
  check(mdsc_create(&d, 1, /*device*/ 0, &B.b), "mdsc_create");
}

// Dynvec<Dynvec<Spherocyl> > -> structure of arrays, flat index k in rev_II
// order.  Particles with fewer dipoles than nd get zero-moment dipoles,
// which contribute nothing.
void pack(const Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP) {
  for (int k = 0; k < B.n; ++k) {
    int m = 0, i = 0;
    rev_II(NP, m, i, k);
    const Spherocyl& s = part[m][i];
    s.get_pos(&B.r[3 * k]);
    s.get_mom(&B.p[3 * k]);
    s.get_angm(&B.l[3 * k]);
    s.get_F(&B.F[3 * k]);
    s.get_T(&B.T[3 * k]);
    Matrix<double> o(3, 3);
    s.get_omat(o);
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) B.O[9 * k + 3 * a + c] = o[a][c];
    double sh[2];
    s.get_shape(sh);
    B.len[k] = sh[0];
    B.dia[k] = sh[1];
    B.mass[k] = s.get_mass();
    B.clust[k] = s.get_clust();
    double ax[3];
    s.get_ori(ax);
    for (int w = 0; w < B.nd; ++w) {
      double* q = &B.dip[((size_t)k * B.nd + w) * 5];
      if (w >= s.get_ndips()) {
        q[0] = 0; q[1] = 0; q[2] = 0; q[3] = 1; q[4] = 0;
        continue;
      }
      const Dipole u = s.get_dip(w);
      double lev[3], uo[3];
      s.get_lev(w, lev);
      u.get_ori(uo);
      q[0] = lev[0] * ax[0] + lev[1] * ax[1] + lev[2] * ax[2];
      for (int a = 0; a < 3; ++a) q[1 + a] = o[a][0] * uo[0] + o[a][1] * uo[1] + o[a][2] * uo[2];
      q[4] = u.get_dip();
    }
  }
}

// structure of arrays -> Dynvec<Dynvec<Spherocyl> > (state, forces, cluster
// labels; the lab-frame dipoles follow from the new position and axes)
void unpack(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP) {
  for (int k = 0; k < B.n; ++k) {
    int m = 0, i = 0;
    rev_II(NP, m, i, k);
    Spherocyl& s = part[m][i];
    s.set_pos(&B.r[3 * k]);
    s.set_mom(&B.p[3 * k]);
    s.set_angm(&B.l[3 * k]);
    s.set_F(&B.F[3 * k]);
    s.set_T(&B.T[3 * k]);
    Matrix<double> o(3, 3);
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) o[a][c] = B.O[9 * k + 3 * a + c];
    s.set_omat(o);
    const int nk = s.get_ndips();
    if (nk > 0) {
      Matrix<double> u(nk, 5);
      for (int w = 0; w < nk; ++w)
        for (int c = 0; c < 5; ++c) u[w][c] = B.dip[((size_t)k * B.nd + w) * 5 + c];
      s.set_dip(u);
    }
    s.set_clust(B.clust[k]);
  }
}

static void to_pt(const double* v, double PT[3][3]) {
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) PT[a][c] = v[3 * a + c];
}

static void upload(const Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP) {
  pack(part, NP);
  check(mdsc_upload(B.b, 0, &B.hs), "mdsc_upload");
}

static void download(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP) {
  check(mdsc_download(B.b, 0, &B.hs), "mdsc_download");
  unpack(part, NP);
}

// Replacement of the loop body v25/main.cpp:558-708 for `steps` steps.
// The state stays on the GPU.  Download only when the driver prints or
// saves a configuration.
bool step(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP, int steps, bool download_state,
          double Ktr[2], double& Uss, double& Wss, double& UdipR, double& UdipK, double& Uext,
          double PTkin[3][3], double PTss[3][3], double PTdipR[3][3], double PTdipK[3][3]) {
  mdsc_observables ob;
  const mdsc_status s = mdsc_step(B.b, steps, &ob);
  check(s, "mdsc_step");
  Ktr[0] = ob.K[0];
  Ktr[1] = ob.K[1];
  Uss = ob.U_ss;
  Wss = ob.W_ss;
  UdipR = ob.U_dipR;
  UdipK = ob.U_dipK;
  Uext = ob.U_ext;
  to_pt(ob.PT_kin, PTkin);
  to_pt(ob.PT_ss, PTss);
  to_pt(ob.PT_dipR, PTdipR);
  to_pt(ob.PT_dipK, PTdipK);
  if (download_state) download(part, NP);
  return s != MDSC_ERR_OVERLAP;  // force_sc's false ends the run (main.cpp:591-595)
}

// ---- per-function replacements with the reference's signatures ----------
// Forces and torques accumulate into what the particles hold, as in the
// reference (the caller zeroes them first, v25/main.cpp:582-588).

// force_sc (v25/functions.hpp:38-39): the GPU keeps its own Verlet list, so
// r_cut and the host's nblist are not needed.
bool force_sc(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP, const double[3], double, double& U,
              double& W, double PT[3][3], const std::deque<int>[]) {
  upload(part, NP);
  double u = 0, w = 0, pt[9];
  const mdsc_status s = mdsc_force_sc(B.b, &u, &w, pt);
  check(s, "mdsc_force_sc");
  download(part, NP);
  U = u;
  W = w;
  to_pt(pt, PT);
  return s != MDSC_ERR_OVERLAP;
}

// force_dipR (v25/functions.hpp:40-41): the table is built on the GPU side
// from alpha with tabul's expressions.
void force_dipR(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP, const double[3],
                const double (*)[3] /* Tab */, double& U, double PT[3][3]) {
  upload(part, NP);
  double u = 0, pt[9];
  check(mdsc_force_dipR(B.b, &u, pt), "mdsc_force_dipR");
  download(part, NP);
  U = u;
  to_pt(pt, PT);
}

// force_dipK (v25/functions.hpp:42-43): K_max, alpha and the k table were
// fixed at init (wave_v's vectors are generated on the GPU side).
void force_dipK(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP, const double[3], int, double,
                const Dynvec<Matrix<double> >&, double& U, double PT[3][3]) {
  upload(part, NP);
  double u = 0, pt[9];
  check(mdsc_force_dipK(B.b, &u, pt), "mdsc_force_dipK");
  download(part, NP);
  U = u;
  to_pt(pt, PT);
}

// ext_field (v25/functions.hpp:44): the field was fixed at init.
void ext_field(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP, const double[3], double& U) {
  upload(part, NP);
  double u = 0;
  check(mdsc_ext_field(B.b, &u), "mdsc_ext_field");
  download(part, NP);
  U = u;
}

// self_ener (v25/functions.hpp:45)
double self_ener(const Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP) {
  upload(part, NP);
  double u = 0;
  check(mdsc_self_ener(B.b, &u), "mdsc_self_ener");
  return u;
}

// moveX (v25/functions.hpp:50): Dt was fixed at init.
void moveX(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP, double) {
  upload(part, NP);
  check(mdsc_moveX(B.b), "mdsc_moveX");
  download(part, NP);
}

// moveP (v25/functions.hpp:51-52): the thermostats' coordinates are passed
// as they stand; Dt was fixed at init.
void moveP(Dynvec<Dynvec<Spherocyl> >& part, Thermostat ther[2], const part_num& NP, double, double K[2],
           double PT[3][3], bool last) {
  upload(part, NP);
  const double xi[2] = {ther[0].get_coo(), ther[1].get_coo()};
  double pt[9];
  check(mdsc_moveP(B.b, xi, last ? 1 : 0, K, pt), "mdsc_moveP");
  download(part, NP);
  to_pt(pt, PT);
}

// clust_conf (v25/functions.hpp:107-108): labels from the GPU's bonds and
// the batch's own generator (seeded at init), written to every particle.
bool clust_conf(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP, const double[3], double, double,
                const gsl_rng*, bool) {
  upload(part, NP);
  int ncl = 0;
  check(mdsc_clust_conf(B.b, 0, B.clust.data(), &ncl), "mdsc_clust_conf");
  for (int k = 0; k < B.n; ++k) {
    int m = 0, i = 0;
    rev_II(NP, m, i, k);
    part[m][i].set_clust(B.clust[k]);
  }
  return true;
}

void shutdown() {
  if (B.b) mdsc_destroy(B.b);
  B.b = nullptr;
}

}  // namespace gb300
