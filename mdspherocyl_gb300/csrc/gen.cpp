// Seeded random non-overlapping placement of spherocylinders (host code).
// Sequential rejection: each rod gets a uniform centre and a uniform axis and
// is kept if its segment distance to every rod already placed is at least
// (D_i + D_j)/2 + gap; a cell grid limits the test to nearby rods.  Closest
// points of two segments as in Ericson, Real-Time Collision Detection,
// sec. 5.1.9.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "mdsc.h"

namespace {

double seg_dist2(const double* p1, const double* d1, const double* p2, const double* d2) {
  double r[3], a = 0, e = 0, f = 0, c = 0, b = 0;
  for (int k = 0; k < 3; ++k) {
    r[k] = p1[k] - p2[k];
    a += d1[k] * d1[k];
    e += d2[k] * d2[k];
    f += d2[k] * r[k];
    c += d1[k] * r[k];
    b += d1[k] * d2[k];
  }
  const double den = a * e - b * b;
  double s = den > 1e-12 * a * e ? std::clamp((b * f - c * e) / den, 0.0, 1.0) : 0.0;
  double t = (b * s + f) / e;
  if (t < 0) {
    t = 0;
    s = std::clamp(-c / a, 0.0, 1.0);
  } else if (t > 1) {
    t = 1;
    s = std::clamp((b - c) / a, 0.0, 1.0);
  }
  double q = 0;
  for (int k = 0; k < 3; ++k) {
    const double v = r[k] + s * d1[k] - t * d2[k];
    q += v * v;
  }
  return q;
}

}  // namespace

extern "C" int mdsc_place_rods(int n, const double* len, const double* dia, const double* box,
                               unsigned long long seed, double gap, int max_attempts, double* r,
                               double* O) {
  if (n < 0 || !len || !dia || !box || !r || !O) return MDSC_ERR_BAD_ARG;
  std::mt19937_64 g(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  std::normal_distribution<double> N(0.0, 1.0);
  double reach = gap;
  double lmax = 0, dmax = 0;
  for (int i = 0; i < n; ++i) {
    lmax = std::max(lmax, len[i]);
    dmax = std::max(dmax, dia[i]);
  }
  reach += lmax + dmax;
  int nc[3];
  double cw[3];
  for (int a = 0; a < 3; ++a) {
    nc[a] = std::max(1, (int)std::floor(box[a] / reach));
    cw[a] = box[a] / nc[a];
  }
  std::vector<std::vector<int>> cells((size_t)nc[0] * nc[1] * nc[2]);
  auto cell_of = [&](const double* x, int* c) {
    for (int a = 0; a < 3; ++a) {
      int k = (int)std::floor(x[a] / cw[a]);
      c[a] = ((k % nc[a]) + nc[a]) % nc[a];
    }
  };
  long long attempts = 0;
  const long long limit = (long long)max_attempts + 100LL * n;
  for (int i = 0; i < n; ++i) {
    for (;;) {
      if (++attempts > limit) return MDSC_ERR_TOO_LARGE;
      double x[3] = {U(g) * box[0], U(g) * box[1], U(g) * box[2]};
      double u[3] = {N(g), N(g), N(g)};
      double nu = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
      if (nu < 1e-12) continue;
      for (auto& v : u) v /= nu;
      int c[3];
      cell_of(x, c);
      bool ok = true;
      const double di[3] = {len[i] * u[0], len[i] * u[1], len[i] * u[2]};
      const double p1[3] = {-0.5 * di[0], -0.5 * di[1], -0.5 * di[2]};
      int rng[3][3], cnt[3];
      for (int a = 0; a < 3; ++a) {
        cnt[a] = 0;
        if (nc[a] >= 3) {
          for (int d = -1; d <= 1; ++d) rng[a][cnt[a]++] = ((c[a] + d) % nc[a] + nc[a]) % nc[a];
        } else {
          for (int d = 0; d < nc[a]; ++d) rng[a][cnt[a]++] = d;
        }
      }
      for (int ix = 0; ix < cnt[0] && ok; ++ix)
        for (int iy = 0; iy < cnt[1] && ok; ++iy)
          for (int iz = 0; iz < cnt[2] && ok; ++iz) {
            const auto& cl = cells[((size_t)rng[0][ix] * nc[1] + rng[1][iy]) * nc[2] + rng[2][iz]];
            for (int j : cl) {
              double rij[3], dj[3], p2[3];
              for (int a = 0; a < 3; ++a) {
                rij[a] = x[a] - r[3 * j + a];
                rij[a] -= box[a] * std::floor(rij[a] / box[a] + 0.5);
                dj[a] = len[j] * O[9 * j + 6 + a];
                p2[a] = -rij[a] - 0.5 * dj[a];
              }
              const double lim = 0.5 * (dia[i] + dia[j]) + gap;
              if (seg_dist2(p1, di, p2, dj) < lim * lim) {
                ok = false;
                break;
              }
            }
          }
      if (!ok) continue;
      // body frame: row 2 = axis, rows 0 and 1 complete a right-handed basis
      double a0[3] = {N(g), N(g), N(g)};
      const double dt = a0[0] * u[0] + a0[1] * u[1] + a0[2] * u[2];
      for (int a = 0; a < 3; ++a) a0[a] -= dt * u[a];
      const double na = std::sqrt(a0[0] * a0[0] + a0[1] * a0[1] + a0[2] * a0[2]);
      if (na < 1e-9) continue;
      for (auto& v : a0) v /= na;
      const double b0[3] = {u[1] * a0[2] - u[2] * a0[1], u[2] * a0[0] - u[0] * a0[2],
                            u[0] * a0[1] - u[1] * a0[0]};
      for (int a = 0; a < 3; ++a) {
        r[3 * i + a] = x[a];
        O[9 * i + a] = a0[a];
        O[9 * i + 3 + a] = b0[a];
        O[9 * i + 6 + a] = u[a];
      }
      cells[((size_t)c[0] * nc[1] + c[1]) * nc[2] + c[2]].push_back(i);
      break;
    }
  }
  return MDSC_OK;
}
