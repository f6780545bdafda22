// Host-side check of integration/gb300_bridge.cpp against the reference's
// own particle classes (v25/classes.hpp), run by tests/test_bridge.py.
//
// Two species (3 rods with two off-centre, tilted dipoles; 4 rods with one
// axial dipole), every field set to distinct values and the orientation a
// general rotation.  gb300::pack flattens them in rev_II order, then
// gb300::unpack writes the arrays into a copy whose state was cleared.
// State, forces, shapes and labels must come back bit for bit; the
// lab-frame dipoles, which set_dip recomputes from the body-frame table,
// to a few roundings.  No GPU is involved.
#include <cmath>
#include <cstdio>
#include <deque>

#include "classes.hpp"
#include "functions.hpp"

namespace gb300 {
void size_buffers(int n, int nd);
int max_dipoles(const Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP);
void pack(const Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP);
void unpack(Dynvec<Dynvec<Spherocyl> >& part, const part_num& NP);
}  // namespace gb300

static int bad = 0;

static void same(const char* what, int k, const double* a, const double* b, int n, double tol) {
  for (int c = 0; c < n; ++c) {
    const double d = std::fabs(a[c] - b[c]);
    if (tol == 0.0 ? a[c] != b[c] : d > tol) {
      std::printf("mismatch %s particle %d component %d: %.17g vs %.17g\n", what, k, c, a[c], b[c]);
      ++bad;
    }
  }
}

static void rotation(double ax, double ay, double az, double O[3][3]) {
  const double cx = std::cos(ax), sx = std::sin(ax), cy = std::cos(ay), sy = std::sin(ay), cz = std::cos(az),
               sz = std::sin(az);
  const double Rx[3][3] = {{1, 0, 0}, {0, cx, -sx}, {0, sx, cx}};
  const double Ry[3][3] = {{cy, 0, sy}, {0, 1, 0}, {-sy, 0, cy}};
  const double Rz[3][3] = {{cz, -sz, 0}, {sz, cz, 0}, {0, 0, 1}};
  double T[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T[i][j] = 0;
      for (int k = 0; k < 3; ++k) T[i][j] += Ry[i][k] * Rz[k][j];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      O[i][j] = 0;
      for (int k = 0; k < 3; ++k) O[i][j] += Rx[i][k] * T[k][j];
    }
}

// Both containers are built the same way (the reference's operator= does
// not copy the dipole count, v25/classes.cpp:187-208); the copy that
// receives unpack's output starts from a cleared state.
static void fill(Dynvec<Dynvec<Spherocyl> >& part, const Dynvec<int>& np, bool state) {
  part.set_size(2);
  const int ndips[2] = {2, 1};
  for (int m = 0; m < 2; ++m) {
    part[m].set_size(np[m]);
    for (int i = 0; i < np[m]; ++i) {
      Spherocyl& s = part[m][i];
      const double t = state ? 0.37 * (m * 10 + i + 1) : 0.0;
      const double sh[2] = {2.0 + 0.5 * m + 0.01 * i, 1.0};
      s.set_id(i);
      s.set_shape(sh);
      s.set_mass(1.0 + 0.1 * i);
      s.set_inertia();
      const double r[3] = {1.1 * t, -0.7 * t, 2.3 * (t != 0) + t}, p[3] = {0.3 * (t != 0) - t, 0.2 * t, -0.1 * t};
      const double l[3] = {0.05 * t, -0.4 * t, 0.9 * t}, F[3] = {t, 2 * t, -3 * t}, T[3] = {-t, 0.5 * t, t * t};
      s.set_pos(r);
      s.set_mom(p);
      s.set_angm(l);
      s.set_F(F);
      s.set_T(T);
      double O[3][3];
      if (state) {
        rotation(0.3 + t, 1.1 - 0.5 * t, 0.7 * t, O);
      } else {
        for (int a = 0; a < 3; ++a)
          for (int c = 0; c < 3; ++c) O[a][c] = a == c ? 1.0 : 0.0;
      }
      Matrix<double> o(3, 3);
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) o[a][c] = O[a][c];
      s.set_omat(o);
      Matrix<double> u(ndips[m], 5);
      for (int w = 0; w < ndips[m]; ++w) {
        const double th = 0.4 + 0.9 * w, ph = 0.2 * i;
        u[w][0] = m == 0 ? (w == 0 ? 0.6 : -0.45) : 0.0;
        u[w][1] = m == 0 ? std::sin(th) * std::cos(ph) : 0.0;
        u[w][2] = m == 0 ? std::sin(th) * std::sin(ph) : 0.0;
        u[w][3] = m == 0 ? std::cos(th) : 1.0;
        u[w][4] = 1.5 + 0.25 * w;
      }
      s.set_dip(u);
      s.set_clust(state ? 100 + m * 10 + i : -1);
    }
  }
}

int main() {
  part_num NP;
  Dynvec<int> np(2);
  np[0] = 3;
  np[1] = 4;
  NP.init(2, np);
  Dynvec<Dynvec<Spherocyl> > part, back;
  fill(part, np, true);
  fill(back, np, false);
  gb300::size_buffers(NP.get_Tpart(), gb300::max_dipoles(part, NP));
  gb300::pack(part, NP);
  gb300::unpack(back, NP);
  for (int k = 0; k < NP.get_Tpart(); ++k) {
    int m = 0, i = 0;
    rev_II(NP, m, i, k);
    const Spherocyl &a = part[m][i], &b = back[m][i];
    double va[9], vb[9];
    a.get_pos(va); b.get_pos(vb); same("r", k, va, vb, 3, 0.0);
    a.get_mom(va); b.get_mom(vb); same("p", k, va, vb, 3, 0.0);
    a.get_angm(va); b.get_angm(vb); same("l", k, va, vb, 3, 0.0);
    a.get_F(va); b.get_F(vb); same("F", k, va, vb, 3, 0.0);
    a.get_T(va); b.get_T(vb); same("T", k, va, vb, 3, 0.0);
    Matrix<double> oa(3, 3), ob(3, 3);
    a.get_omat(oa);
    b.get_omat(ob);
    for (int r = 0; r < 3; ++r) same("O", k, oa[r], ob[r], 3, 0.0);
    const double ca = a.get_clust(), cb = b.get_clust();
    same("clust", k, &ca, &cb, 1, 0.0);
    if (a.get_ndips() != b.get_ndips()) {
      std::printf("dipole count differs at particle %d\n", k);
      ++bad;
      continue;
    }
    for (int w = 0; w < a.get_ndips(); ++w) {
      const Dipole da = a.get_dip(w), db = b.get_dip(w);
      da.get_pos(va); db.get_pos(vb); same("dipole position", k, va, vb, 3, 1e-13);
      da.get_ori(va); db.get_ori(vb); same("dipole direction", k, va, vb, 3, 1e-13);
      const double ua = da.get_dip(), ub = db.get_dip();
      same("dipole moment", k, &ua, &ub, 1, 0.0);
    }
  }
  if (bad) {
    std::printf("%d mismatches\n", bad);
    return 1;
  }
  std::printf("bridge round trip OK: %d particles, %d dipoles per particle at most\n", NP.get_Tpart(),
              gb300::max_dipoles(part, NP));
  return 0;
}
