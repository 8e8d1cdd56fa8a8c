// Host check of the integer-pipe FP64 <-> FP32 conversions of kernels.cuh (f64_to_f32i,
// f32_to_f64i): every result within half an FP32 ulp of the exact value, signed zeros for
// magnitudes below the FP32 normal range, Inf / NaN kept, and f32 -> f64 exact.  Built and run
// by tests/test_conversions.py.
#include "kernels.cuh"
#include <cstdio>
#include <cmath>
#include <random>
#include <limits>
using namespace gmk;
int main() {
  std::mt19937_64 rng(1);
  long bad = 0, n = 0;
  auto check = [&](double x) {
    float a = f64_to_f32i(x);
    float ref = (float)x;
    ++n;
    if (std::isnan(x)) { if (!std::isnan(a)) ++bad; return; }
    if (std::fabs(ref) < 1.1754943508222875e-38f) { if (a != 0.0f || std::signbit(a) != std::signbit(x)) ++bad; return; }
    double err = std::fabs((double)a - x), ulp = std::ldexp(1.0, std::ilogb(x) - 23);
    if (std::isinf(ref)) { if (!(std::isinf(a) && std::signbit(a) == std::signbit(x))) ++bad; return; }
    if (err > 0.5 * ulp * (1 + 1e-12) || std::signbit(a) != std::signbit(x)) { if (bad < 5) printf("f64->f32 %.17g -> %.9g ref %.9g\n", x, a, ref); ++bad; }
    double back = f32_to_f64i(a);
    if (back != (double)a) { if (bad < 5) printf("f32->f64 %.9g -> %.17g\n", a, back); ++bad; }
  };
  double specials[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38, 1e39, -1e39,
                       1.1754943508222875e-38, 1.1754942e-38, 1e-40, 5e-324, 2.220446049250313e-16, 1e300,
                       std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                       std::numeric_limits<double>::quiet_NaN(), 0.1, 1.0 / 3.0, 16777217.0, 16777215.5};
  for (double x : specials) check(x);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-140, 140);
  for (int i = 0; i < 4000000; ++i) check(std::ldexp(u(rng), ex(rng)));
  // exact halfway cases: round half away from zero
  for (int i = 0; i < 100000; ++i) {
    float f = std::ldexp((float)u(rng), ex(rng) / 2);
    if (f == 0 || !std::isfinite(f)) continue;
    double h = (double)f + std::ldexp(1.0, std::ilogb(f) - 24) * (f > 0 ? 1 : -1);
    check(h);
  }
  printf("checked %ld, bad %ld\n", n, bad);
  return bad != 0;
}
