// cnoidal.h -- Jacobi elliptic cn and the complete elliptic integrals K, E by
// the arithmetic-geometric mean, for the LEF_CON boundary wave.
//
// Restates cnoidal_cn, cnoidal_ck and cnoidal_ce (src/waves.F:225-370):
// the AGM sequence a_n, b_n, c_n of the parameter m runs until |c_n| < 1e-15
// (a single-precision literal there); K = (pi/2)/a_N; E = K (1 - sum_n
// 2^(n-2) c_n^2); cn(u|m) = cos(phi_1), with phi_N = 2^(N-1) a_N u and the
// descending Landen step phi_{n} = (phi_{n+1} + asin(c_{n+1}/a_{n+1}
// sin phi_{n+1}))/2.  Used by the host set-up (Newton iteration for m,
// start phase) and by the boundary-wave kernel once per step.
//
// For 0 <= m <= 1 the sequence ends by n = 52 (at m = 1, b stays 0 and
// c_n = 2^(1-n)); kCnMax bounds the arrays, and the host set-up rejects a
// parameter whose sequence would not fit.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define NHW_HD __host__ __device__
#else
#define NHW_HD
#endif

namespace nhw {

constexpr int kCnMax = 64;
constexpr double kCnEps = (double)1.0e-15f;     // the 1.0e-15 of the AGM stop test (default real)
constexpr double kCnPi = (double)3.1415926535897932384626f;   // the pi literal of cnoidal_ck / _ce

// Length N of the AGM sequence of m (N <= kCnMax - 1 when 0 <= m <= 1).
NHW_HD inline int cn_agm(double m, double* a, double* c) {
  double a0 = 1.0, b0 = sqrt(1.0 - m), c0 = sqrt(m);
  int n = 1;
  a[n] = a0;
  c[n] = c0;
  while (!(fabs(c0) < kCnEps) && n < kCnMax - 1) {
    ++n;
    const double a1 = (a0 + b0) / 2.0, b1 = sqrt(a0 * b0), c1 = (a0 - b0) / 2.0;
    a0 = a1; b0 = b1; c0 = c1;
    a[n] = a0;
    c[n] = c0;
  }
  return n;
}

NHW_HD inline double cnoidal_ck(double m) {
  double a[kCnMax], c[kCnMax];
  const int n = cn_agm(m, a, c);
  return kCnPi / 2.0 / a[n];
}

NHW_HD inline double cnoidal_ce(double m) {
  double a[kCnMax], c[kCnMax];
  const int n = cn_agm(m, a, c);
  const double ck = kCnPi / 2.0 / a[n];
  double sum = 0.0;
  for (int k1 = 1; k1 <= n; ++k1) sum = sum + ldexp(1.0, k1 - 2) * (c[k1] * c[k1]);
  return ck * (1.0 - sum);
}

// cn keeps only the ratios c_n / a_n of the descending steps (half the
// local memory of the boundary kernel's thread)
NHW_HD inline double cnoidal_cn(double u, double m) {
  double r[kCnMax];
  double a0 = 1.0, b0 = sqrt(1.0 - m), c0 = sqrt(m);
  int n = 1;
  r[n] = c0 / a0;
  while (!(fabs(c0) < kCnEps) && n < kCnMax - 1) {
    ++n;
    const double a1 = (a0 + b0) / 2.0, b1 = sqrt(a0 * b0), c1 = (a0 - b0) / 2.0;
    a0 = a1; b0 = b1; c0 = c1;
    r[n] = c0 / a0;
  }
  double y = ldexp(1.0, n - 1) * a0 * u;
  for (int i = n - 1; i >= 1; --i) y = (y + asin(r[i + 1] * sin(y))) / 2.0;
  return cos(y);
}

}  // namespace nhw
