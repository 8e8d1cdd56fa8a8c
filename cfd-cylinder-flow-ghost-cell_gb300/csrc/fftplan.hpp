// Host-side FFT plans for the shared-memory Stockham transforms (transforms.cuh):
// radix factorisation, the exact-division magic numbers of every stage and the plan's
// twiddle table.
#pragma once
#include <cmath>
#include <stdexcept>
#include <vector>

#include "transforms.cuh"

namespace gmk {

inline FftPlan make_plan(int M) {
  FftPlan p{};
  p.M = M;
  int m = M, s = 0;
  while (m % 8 == 0) { p.radix[s++] = 8; m /= 8; }
  while (m % 4 == 0) { p.radix[s++] = 4; m /= 4; }
  while (m % 2 == 0) { p.radix[s++] = 2; m /= 2; }
  while (m % 5 == 0) { p.radix[s++] = 5; m /= 5; }
  while (m % 3 == 0) { p.radix[s++] = 3; m /= 3; }
  for (int f = 7; m > 1; f += 2)
    while (m % f == 0) {
      if (f > 64) throw std::runtime_error("FFT length has a prime factor above 64");
      p.radix[s++] = f;
      m /= f;
    }
  p.nstages = s;
  if (M > 65536) throw std::runtime_error("FFT length above 65536");
  long long Ns = 1;
  int off = 0;
  bool generic = false;
  for (int k = 0; k < s; ++k) {
    p.ns_magic[k] = Ns == 1 ? 0u : (unsigned)(((1ull << 32) + (unsigned long long)Ns - 1) / (unsigned long long)Ns);
    const int R = p.radix[k];
    if (R == 2 || R == 3 || R == 4 || R == 5 || R == 8) {
      p.tw_off[k] = off;
      off += (int)Ns * (R - 1);
    } else {
      generic = true;
    }
    Ns *= R;
  }
  for (int k = 0; k < s; ++k) {
    const int R = p.radix[k];
    if (!(R == 2 || R == 3 || R == 4 || R == 5 || R == 8)) p.tw_off[k] = off;  // the full table follows
  }
  p.tw_len = off + (generic ? M : 0);
  return p;
}

// The plan's twiddle table (see FftPlan), interleaved (re, im), forward sign exp(-2 pi i t / M).
inline std::vector<double> plan_twiddles(const FftPlan& p) {
  std::vector<double> t(2 * (size_t)p.tw_len);
  const long double PI = 3.14159265358979323846264338327950288L;
  auto put = [&](int at, long long e) {
    const long double a = -2.0L * PI * (long double)(e % p.M) / (long double)p.M;
    t[2 * (size_t)at] = (double)std::cos(a);
    t[2 * (size_t)at + 1] = (double)std::sin(a);
  };
  long long Ns = 1;
  bool generic = false;
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s];
    if (R == 2 || R == 3 || R == 4 || R == 5 || R == 8) {
      const long long tws = p.M / (Ns * R);
      for (long long k = 0; k < Ns; ++k)
        for (int r = 1; r < R; ++r) put(p.tw_off[s] + (int)(k * (R - 1) + r - 1), r * k * tws);
    } else {
      generic = true;
    }
    Ns *= R;
  }
  if (generic) {
    int base = p.tw_len - p.M;
    for (int e = 0; e < p.M; ++e) put(base + e, e);
  }
  return t;
}

}  // namespace gmk
