// Host-side 1D FFT planning: radix factorisation of a length and its twiddle table.
//
// Twiddles are generated in double precision from an octant-reduced argument evaluated in long
// double, so that every entry is the correctly rounded (or within one ulp) double value of
// exp(-2 pi i m / n). Single-precision and double-float kernels round these double values; no
// kernel evaluates trigonometric functions itself.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

namespace spfft {
namespace gb300 {

constexpr int kMaxStages = 24;

struct RadixPlan {
  int n = 1;
  int numStages = 0;
  int radix[kMaxStages] = {0};
};

// Radices are applied in the order stored. Powers of two are grouped into radix 8 (with a 4*4 or a
// 4 in place of a trailing 8*2 or 2*2), then 3, 5, 7 are taken, then any remaining prime factor
// becomes one generic-radix stage.
inline RadixPlan make_radix_plan(int n) {
  RadixPlan p;
  p.n = n;
  if (n <= 1) return p;
  int m = n;
  int twos = 0;
  while (m % 2 == 0) {
    m /= 2;
    ++twos;
  }
  std::vector<int> radices;
  int eights = twos / 3, rest = twos % 3;
  if (rest == 1 && eights > 0) {  // 8*2 -> 4*4
    --eights;
    radices.push_back(4);
    radices.push_back(4);
  } else if (rest == 1) {
    radices.push_back(2);
  } else if (rest == 2) {
    radices.push_back(4);
  }
  for (int i = 0; i < eights; ++i) radices.insert(radices.begin(), 8);
  for (int r : {3, 5, 7}) {
    while (m % r == 0) {
      radices.push_back(r);
      m /= r;
    }
  }
  for (int f = 11; m > 1;) {
    if (static_cast<long long>(f) * f > m) {  // m is prime
      radices.push_back(m);
      break;
    }
    if (m % f == 0) {
      radices.push_back(f);
      m /= f;
    } else {
      f += 2;
    }
  }
  p.numStages = static_cast<int>(radices.size());
  for (int i = 0; i < p.numStages; ++i) p.radix[i] = radices[i];
  return p;
}

// Radix plans the autotuner may choose from for the generic (runtime-radix) kernels, the default of
// make_radix_plan first; then the same stages in reverse order, the powers of two as radix-4 stages
// (and one radix 2), and for at most ten factors of two radix-2 stages only -- each followed by
// the odd factors in the default order. Every plan's radices multiply to n; duplicates are dropped.
inline std::vector<RadixPlan> radix_plan_candidates(int n) {
  std::vector<RadixPlan> out;
  auto add = [&](const std::vector<int>& r) {
    if (static_cast<int>(r.size()) > kMaxStages) return;
    RadixPlan p;
    p.n = n;
    p.numStages = static_cast<int>(r.size());
    for (int i = 0; i < p.numStages; ++i) p.radix[i] = r[i];
    for (const RadixPlan& q : out) {
      bool same = q.numStages == p.numStages;
      for (int i = 0; same && i < p.numStages; ++i) same = q.radix[i] == p.radix[i];
      if (same) return;
    }
    out.push_back(p);
  };
  const RadixPlan d = make_radix_plan(n);
  std::vector<int> def(d.radix, d.radix + d.numStages);
  add(def);
  add(std::vector<int>(def.rbegin(), def.rend()));
  int twos = 0;
  for (int m = n; m > 1 && m % 2 == 0; m /= 2) ++twos;
  std::vector<int> odd;
  for (int r : def)
    if (r % 2 != 0) odd.push_back(r);
  if (twos > 0) {
    std::vector<int> fours(static_cast<size_t>(twos / 2), 4);
    if (twos % 2) fours.push_back(2);
    fours.insert(fours.end(), odd.begin(), odd.end());
    add(fours);
    if (twos <= 10) {
      std::vector<int> pairs(static_cast<size_t>(twos), 2);
      pairs.insert(pairs.end(), odd.begin(), odd.end());
      add(pairs);
    }
  }
  return out;
}

// exp(-2 pi i m / n) for m in [0, n), as (cos, sin) pairs in double precision.
inline std::vector<double> make_twiddles(int n) {
  std::vector<double> w(2 * static_cast<size_t>(n > 0 ? n : 1));
  const long double twoPi = 6.283185307179586476925286766559005768L;
  for (int m = 0; m < n; ++m) {
    // Reduce m/n to the first octant so that sin/cos are evaluated on |angle| <= pi/4.
    long long num8 = 8LL * m;  // angle = 2*pi*m/n = (pi/4) * (8m/n)
    long long oct = num8 / n;  // octant 0..7
    long long remNum = num8 - oct * n;  // angle within octant = (pi/4) * remNum / n
    long double a = (twoPi / 8.0L) * static_cast<long double>(remNum) / static_cast<long double>(n);
    long double c, s;
    // Use the complementary angle in odd octants so the argument stays small.
    if (oct % 2 == 1) {
      long double b = (twoPi / 8.0L) * static_cast<long double>(n - remNum) / static_cast<long double>(n);
      // angle = (oct+1)*pi/4 - b
      long double cb = cosl(b), sb = sinl(b);
      // cos/sin of k*pi/4 - b expressed by swapping; handled via the generic rotation below.
      long double ck, sk;
      switch ((oct + 1) % 8) {
        case 0: ck = 1; sk = 0; break;
        case 2: ck = 0; sk = 1; break;
        case 4: ck = -1; sk = 0; break;
        default: ck = 0; sk = -1; break;  // 6
      }
      c = ck * cb + sk * sb;
      s = sk * cb - ck * sb;
    } else {
      long double ca = cosl(a), sa = sinl(a);
      long double ck, sk;
      switch (oct % 8) {
        case 0: ck = 1; sk = 0; break;
        case 2: ck = 0; sk = 1; break;
        case 4: ck = -1; sk = 0; break;
        default: ck = 0; sk = -1; break;  // 6
      }
      c = ck * ca - sk * sa;
      s = sk * ca + ck * sa;
    }
    // Forward sign: exp(-i angle).
    w[2 * m] = static_cast<double>(c);
    w[2 * m + 1] = static_cast<double>(-s);
  }
  return w;
}

}  // namespace gb300
}  // namespace spfft
