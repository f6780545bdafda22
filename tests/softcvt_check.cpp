// CPU check of the integer FP64<->FP32 conversions in softcvt.cuh against
// the IEEE casts (compiled with g++ by test_softcvt.py).
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <random>

#define __host__
#define __device__
#define __forceinline__ inline
#include "../mdspherocyl_gb300/csrc/softcvt.cuh"

using namespace mdsc;

static float trunc_cast(double x) {
  float f = (float)x;
  if (std::fabs((double)f) > std::fabs(x)) f = std::nextafterf(f, 0.f);
  return f;
}

int main() {
  std::mt19937_64 g(12345);
  std::uniform_real_distribution<double> u(-1.0, 1.0), ex(-60.0, 60.0);
  long bad = 0, n = 0;
  for (int k = 0; k < 2000000; ++k) {
    double x = u(g) * std::ldexp(1.0, (int)ex(g));
    if (k % 97 == 0) x = std::floor(x);
    if (k % 101 == 0) x = std::floor(x) + 0.5;
    if (k == 0) x = 0.0;
    if (k == 1) x = -0.0;
    if (k == 2) x = (double)FLT_MIN;
    if (k == 3) x = -(double)FLT_MIN * 1.5;
    ++n;
    // d2f: truncation inside the FP32 normal range
    if (std::fabs(x) >= FLT_MIN || x == 0.0) {
      const float a = soft_d2f(x), b = trunc_cast(x);
      if (std::memcmp(&a, &b, 4) != 0 && !(a == 0.f && b == 0.f)) {
        if (bad++ < 10) std::printf("d2f %.17g: %.9g vs %.9g\n", x, a, b);
      }
      // d2f_rn: IEEE round-to-nearest except at exact ties (ties go away from zero)
      {
        const float c = soft_d2f_rn(x), d = (float)x;
        const double dc = std::fabs((double)c - x), dd = std::fabs((double)d - x);
        if (std::memcmp(&c, &d, 4) != 0 && !(c == 0.f && d == 0.f) && dc != dd) {
          if (bad++ < 10) std::printf("d2f_rn %.17g: %.9g vs %.9g\n", x, c, d);
        }
      }
      // f2d exact on FP32 values
      const double c = soft_f2d(b), d = (double)b;
      if (c != d || std::signbit(c) != std::signbit(d)) {
        if (bad++ < 10) std::printf("f2d %.9g: %.17g vs %.17g\n", b, c, d);
      }
      // split: hi + lo = x to 2^-47 relative
      float hi, lo;
      soft_split(x, hi, lo);
      const double err = std::fabs(((double)hi + (double)lo) - x);
      if (err > std::ldexp(std::fabs(x), -47) && std::fabs(x) > std::ldexp(1.0, -70)) {
        if (bad++ < 10) std::printf("split %.17g: %.9g + %.9g (err %.3g)\n", x, hi, lo, err);
      }
    }
    // floor modulo 2^32 for |y| < 2^52
    const double y = x * 1e3;
    if (std::fabs(y) < std::ldexp(1.0, 52)) {
      const uint32_t a = soft_floor_u32(y), b = (uint32_t)(int64_t)std::floor(y);
      if (a != b) {
        if (bad++ < 10) std::printf("floor %.17g: %u vs %u\n", y, a, b);
      }
    }
  }
  std::printf("checked %ld values, %ld mismatches\n", n, bad);
  return bad == 0 ? 0 : 1;
}
