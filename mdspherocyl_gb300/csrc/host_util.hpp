// Host-side helpers of the library: the random generator the reference
// draws from, its Gaussian transform, and the per-particle constants the
// reference computes on the host.
#pragma once
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

namespace mdsc {

// The reference's generator is GSL's MT19937 (v25/classes.hpp:150-181,
// v25/main.cpp:209-211): init_genrand seeding with seed 0 mapped to 4357,
// uniform = 32-bit output / 2^32.  std::mt19937 implements the same
// generator and seeding.
class Mt19937 {
 public:
  // MT19937 (Matsumoto & Nishimura, ACM TOMACS 8(1), 1998) with GSL's state
  // layout and seeding, so that a state read from the reference's generator
  // files continues the same sequence: 624 words and the position of the
  // next word; a seed of 0 means 4357 (gsl_rng_set).
  static constexpr int kN = 624;
  explicit Mt19937(unsigned long seed = 1) { seed_with(seed); }
  void seed_with(unsigned long seed) {
    uint32_t s = (uint32_t)(seed & 0xffffffffUL);
    if (s == 0) s = 4357u;
    mt_[0] = s;
    for (int i = 1; i < kN; ++i) mt_[i] = 1812433253u * (mt_[i - 1] ^ (mt_[i - 1] >> 30)) + (uint32_t)i;
    mti_ = kN;
  }
  uint32_t next() {
    if (mti_ >= kN) refill();
    uint32_t y = mt_[mti_++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
  double uniform() { return (double)next() / 4294967296.0; }
  void discard(unsigned long long n) {
    for (unsigned long long k = 0; k < n; ++k) next();
  }
  void get_state(uint32_t* mt, int* mti) const {
    for (int i = 0; i < kN; ++i) mt[i] = mt_[i];
    *mti = mti_;
  }
  bool set_state(const uint32_t* mt, int mti) {
    if (mti < 0 || mti > kN) return false;
    for (int i = 0; i < kN; ++i) mt_[i] = mt[i];
    mti_ = mti;
    return true;
  }

 private:
  void refill() {
    constexpr uint32_t kUpper = 0x80000000u, kLower = 0x7fffffffu, kMatrix = 0x9908b0dfu;
    constexpr int kM = 397;
    for (int k = 0; k < kN; ++k) {
      const uint32_t y = (mt_[k] & kUpper) | (mt_[(k + 1) % kN] & kLower);
      mt_[k] = mt_[(k + kM) % kN] ^ (y >> 1) ^ ((y & 1u) ? kMatrix : 0u);
    }
    mti_ = 0;
  }
  uint32_t mt_[kN];
  int mti_ = kN;
};

// gauss(1, rnd1, rnd2): Box-Muller as v25/functions.cpp:1149-1156 does it
inline void box_muller(double& rnd1, double& rnd2) {
  const double a = std::sqrt(-2 * std::log(rnd1)) * std::cos(2 * M_PI * rnd2);
  const double b = std::sqrt(-2 * std::log(rnd1)) * std::sin(2 * M_PI * rnd2);
  rnd1 = a;
  rnd2 = b;
}

// Spherocyl::set_inertia, v25/classes.cpp:175-185
inline void spherocyl_inertia(double L, double D, double mass, double I[3]) {
  const double R = D / 2, Rsq = R * R, Rft = Rsq * Rsq, Lsq = L * L;
  const double vol = M_PI * Rsq * (L + 3. * R / 4);
  const double mdens = mass / vol;
  I[0] = mdens * M_PI * (Lsq * L * Rsq / 12 + Lsq * Rsq * R / 3 + L * Rft / 4 + 8. * Rft * R / 15);
  I[1] = I[0];
  I[2] = mdens * M_PI * (L * Rft / 2 + 8. * Rft * R / 15);
}

// Fenwick tree over 0/1 flags: order statistics of the remaining particles
// for the cluster-label replay.
class Fenwick {
 public:
  explicit Fenwick(int n) : n_(n), t_(n + 1, 0) {
    for (int i = 1; i <= n; ++i) {
      t_[i] += 1;
      const int j = i + (i & -i);
      if (j <= n) t_[j] += t_[i];
    }
  }
  void remove(int i) {
    for (++i; i <= n_; i += i & -i) t_[i] -= 1;
  }
  // index of the k-th (0-based) remaining element
  int kth(int k) const {
    int pos = 0, step = 1;
    while (step * 2 <= n_) step *= 2;
    for (; step; step >>= 1) {
      if (pos + step <= n_ && t_[pos + step] <= k) {
        pos += step;
        k -= t_[pos];
      }
    }
    return pos;
  }

 private:
  int n_;
  std::vector<int> t_;
};

}  // namespace mdsc
