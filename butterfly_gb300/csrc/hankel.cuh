// Hankel functions of the first kind of orders 0 and 1 for real x > 0:
//   H0(x) = J0(x) + i Y0(x),   H1(x) = J1(x) + i Y1(x).
//
// The reference evaluates these with glibc's j0/y0/j1/y1 (bessel.c:284-308).
// This evaluator is written from published methods only; no library's
// internal constants are used.  Three regimes:
//
//   x < kSeriesMax      ascending power series (Abramowitz & Stegun 9.1.10,
//                       9.1.11, 9.1.13), with psi(k+1) = -gamma + H_k.
//   x < kAsymptoticMin  Miller's backward recurrence J_{n-1} = (2n/x) J_n -
//                       J_{n+1} from a start index far above x, normalised by
//                       J0 + 2 sum J_2k = 1 (A&S 9.1.46); Y0 from the Neumann
//                       series Y0 = (2/pi)[(ln(x/2)+gamma) J0 - 2 sum (-1)^k
//                       J_2k / k] (A&S 9.1.88) and Y1 = -Y0' from the
//                       derivative of that series.
//   otherwise           Hankel's asymptotic expansion (A&S 9.2.5-9.2.10):
//                       H_nu(x) ~ sqrt(2/(pi x)) (P + i Q) exp(i chi),
//                       chi = x - (nu/2 + 1/4) pi, with the terms
//                       t_k = t_{k-1} (4 nu^2 - (2k-1)^2) / (8 k x) summed
//                       until they fall below 1e-17.  exp(i chi) is formed
//                       from sincos(x) and the exact rotation by pi/4 or
//                       3 pi/4, so no rounding of x - chi enters.
//
// The same source compiles for the host (tests) and the device (kernels).
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define BFG_HD __host__ __device__ __forceinline__
#else
#define BFG_HD inline
#endif

namespace bfg {

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kTwoOverPi = 0.636619772367581343075535053490057448;
constexpr double kEulerGamma = 0.577215664901532860606512090082402431;
constexpr double kInvSqrt2 = 0.707106781186547524400844362104849039;
constexpr double kSeriesMax = 0.25;
constexpr double kAsymptoticMin = 20.0;

struct Bessel01 {
  double j0, y0, j1, y1;
};

BFG_HD void bfgSincos(double x, double *s, double *c) {
#if defined(__CUDA_ARCH__)
  sincos(x, s, c);
#else
  *s = sin(x);
  *c = cos(x);
#endif
}

// x < kSeriesMax: ascending series.  q = x^2/4 <= 1/64, so eight terms
// reach below 1e-20 relative.
BFG_HD Bessel01 besselSeries(double x) {
  double const h = 0.5 * x;
  double const q = h * h;
  double lnh = log(h);
  // J0 = sum (-q)^k/(k!)^2 ; J1 = h sum (-q)^k / (k!(k+1)!)
  // Y0 tail: sum_{k>=1} (-1)^{k+1} H_k q^k/(k!)^2
  // Y1 tail: sum_{k>=0} (psi(k+1)+psi(k+2)) (-q)^k / (k!(k+1)!)
  double t0 = 1.0;            // (-q)^k/(k!)^2
  double t1 = 1.0;            // (-q)^k/(k!(k+1)!)
  double j0 = 1.0, j1s = 1.0;
  double harm = 0.0;          // H_k
  double y0tail = 0.0;
  double psi1 = -kEulerGamma;            // psi(k+1)
  double psi2 = -kEulerGamma + 1.0;      // psi(k+2)
  double y1tail = psi1 + psi2;
  for (int k = 1; k <= 8; ++k) {
    double const dk = (double)k;
    t0 *= -q / (dk * dk);
    t1 *= -q / (dk * (dk + 1.0));
    harm += 1.0 / dk;
    psi1 += 1.0 / dk;
    psi2 += 1.0 / (dk + 1.0);
    j0 += t0;
    j1s += t1;
    y0tail -= harm * t0;   // (-1)^{k+1} H_k q^k/(k!)^2 = -H_k t0
    y1tail += (psi1 + psi2) * t1;
  }
  Bessel01 b;
  b.j0 = j0;
  b.j1 = h * j1s;
  b.y0 = kTwoOverPi * ((lnh + kEulerGamma) * j0 + y0tail);
  b.y1 = -kTwoOverPi / x + kTwoOverPi * lnh * b.j1 - h * y1tail / kPi;
  return b;
}

// kSeriesMax <= x < kAsymptoticMin: Miller's algorithm + Neumann series.
BFG_HD Bessel01 besselMiller(double x) {
  int const nStart = 2 * (int)(0.5 * (x + 36.0));   // even, > x + 34
  double const twoOverX = 2.0 / x;
  double jn1 = 0.0;     // J_{n+1}
  double jn = 1e-30;    // J_n, arbitrary small start at n = nStart
  double norm = 0.0;    // 2 sum_{even n>=2} J_n
  double s0 = 0.0;      // sum_{even n>=2} (-1)^{n/2} (4/n) J_n
  double s1 = 0.0;      // sum_{odd  n>=3} (-1)^{(n+1)/2} 4n/(n^2-1) J_n
  double j1 = 0.0;
  // account for J_nStart itself (even)
  {
    int const n = nStart;
    double const sgn = ((n >> 1) & 1) ? -1.0 : 1.0;
    norm += 2.0 * jn;
    s0 += sgn * (4.0 / n) * jn;
  }
  for (int n = nStart; n >= 1; --n) {
    double const jm1 = (double)n * twoOverX * jn - jn1;   // J_{n-1}
    jn1 = jn;
    jn = jm1;
    int const m = n - 1;                 // index of the value just formed
    if (m == 0) break;
    if ((m & 1) == 0) {
      double const sgn = ((m >> 1) & 1) ? -1.0 : 1.0;
      norm += 2.0 * jn;
      s0 += sgn * (4.0 / m) * jn;
    } else if (m == 1) {
      j1 = jn;
    } else {
      double const sgn = (((m + 1) >> 1) & 1) ? -1.0 : 1.0;
      s1 += sgn * (4.0 * m / ((double)m * m - 1.0)) * jn;
    }
  }
  double const j0 = jn;
  double const scale = 1.0 / (j0 + norm);
  Bessel01 b;
  b.j0 = j0 * scale;
  b.j1 = j1 * scale;
  double const l = log(0.5 * x) + kEulerGamma;
  b.y0 = kTwoOverPi * (l * b.j0 - s0 * scale);
  // Y1 = (2/pi) [ -J0/x + l J1 + (-J1 + s1) ]
  b.y1 = kTwoOverPi * (-b.j0 / x + l * b.j1 - b.j1 + s1 * scale);
  return b;
}

// x >= kAsymptoticMin: Hankel's expansion; order 1 only when kOrder1.
template <bool kOrder1 = true>
BFG_HD Bessel01 besselAsymptotic(double x) {
  double const inv8x = 0.125 / x;
  // order 0: mu = 0; order 1: mu = 4
  double t0 = 1.0, t1 = 1.0;
  double p0 = 1.0, q0 = 0.0, p1 = 1.0, q1 = 0.0;
  for (int k = 1; k <= 60; ++k) {
    double const odd = (double)(2 * k - 1);
    double const f = inv8x / (double)k;
    t0 *= (0.0 - odd * odd) * f;
    if (kOrder1) t1 *= (4.0 - odd * odd) * f;
    // k odd -> Q with sign (-1)^{(k-1)/2}; k even -> P with sign (-1)^{k/2}
    int const r = k & 3;
    if (r == 1) { q0 += t0; q1 += t1; }
    else if (r == 2) { p0 -= t0; p1 -= t1; }
    else if (r == 3) { q0 -= t0; q1 -= t1; }
    else { p0 += t0; p1 += t1; }
    if (fabs(t0) < 1e-17 && (!kOrder1 || fabs(t1) < 1e-17)) break;
  }
  double s, c;
  bfgSincos(x, &s, &c);
  double const amp = sqrt(kTwoOverPi / x);
  // chi0 = x - pi/4, chi1 = x - 3pi/4
  double const c0 = (c + s) * kInvSqrt2, s0 = (s - c) * kInvSqrt2;
  double const c1 = (s - c) * kInvSqrt2, s1 = -(s + c) * kInvSqrt2;
  Bessel01 b;
  b.j0 = amp * (p0 * c0 - q0 * s0);
  b.y0 = amp * (p0 * s0 + q0 * c0);
  if (kOrder1) {
    b.j1 = amp * (p1 * c1 - q1 * s1);
    b.y1 = amp * (p1 * s1 + q1 * c1);
  } else {
    b.j1 = b.y1 = 0.0;
  }
  return b;
}

// J0, Y0 (and J1, Y1 when kOrder1) at x > 0.
template <bool kOrder1 = true>
BFG_HD Bessel01 bessel01(double x) {
  if (x >= kAsymptoticMin) return besselAsymptotic<kOrder1>(x);
  if (x >= kSeriesMax) return besselMiller(x);
  return besselSeries(x);
}

}  // namespace bfg
