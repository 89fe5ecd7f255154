// Device/host math for the OPTIMET sphere path: complex arithmetic, spherical
// Bessel/Hankel functions, normalised associated Legendre functions and the
// Wigner d functions of OPTIMET's AuxCoefficients.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#define OM_HD __host__ __device__ __forceinline__

namespace om {

constexpr double kPi = 3.14159265358979323846;
constexpr int kMaxNmax = 15;                 // lanes hold l <= 2 nMax <= 30
constexpr int kMaxOrder = 2 * kMaxNmax + 2;  // Bessel orders 0..2 nMax + 1

struct zd {
  double re, im;
};
OM_HD zd mk(double r, double i) {
  zd z;
  z.re = r;
  z.im = i;
  return z;
}
OM_HD zd operator+(zd a, zd b) { return mk(a.re + b.re, a.im + b.im); }
OM_HD zd operator-(zd a, zd b) { return mk(a.re - b.re, a.im - b.im); }
OM_HD zd operator-(zd a) { return mk(-a.re, -a.im); }
OM_HD zd operator*(zd a, zd b) { return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
OM_HD zd operator*(double s, zd a) { return mk(s * a.re, s * a.im); }
OM_HD zd operator*(zd a, double s) { return mk(s * a.re, s * a.im); }
OM_HD zd conj(zd a) { return mk(a.re, -a.im); }
OM_HD double norm2(zd a) { return a.re * a.re + a.im * a.im; }
OM_HD double cabs(zd a) { return hypot(a.re, a.im); }
// a * conj(b)
OM_HD zd mulc(zd a, zd b) { return mk(a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im); }
// Smith's division
OM_HD zd operator/(zd a, zd b) {
  if(fabs(b.re) >= fabs(b.im)) {
    double r = b.im / b.re, d = b.re + b.im * r;
    return mk((a.re + a.im * r) / d, (a.im - a.re * r) / d);
  }
  double r = b.re / b.im, d = b.re * r + b.im;
  return mk((a.re * r + a.im) / d, (a.im * r - a.re) / d);
}
OM_HD zd operator/(double a, zd b) { return mk(a, 0.0) / b; }
OM_HD zd operator/(zd a, double s) { return mk(a.re / s, a.im / s); }
OM_HD zd cexp_i(zd z) {  // exp(i z)
  double s, c;
  sincos(z.re, &s, &c);
  double e = exp(-z.im);
  return mk(e * c, e * s);
}
OM_HD zd csin(zd z) {
  double s, c;
  sincos(z.re, &s, &c);
  return mk(s * cosh(z.im), c * sinh(z.im));
}
OM_HD zd ccos(zd z) {
  double s, c;
  sincos(z.re, &s, &c);
  return mk(c * cosh(z.im), -s * sinh(z.im));
}

// ---------------------------------------------------------------------------
// Spherical Bessel functions of complex argument, orders 0..L1.
// j_n: Miller's backward recurrence for the ratios r_n = j_n / j_{n-1},
//      r_n = z / (2n + 1 - z r_{n+1}), started well above max(L1, |z|), then a
//      forward product normalised at the larger of the closed forms
//      j_0 = sin z / z, j_1 = (sin z / z - cos z) / z (j_0 only for |z| < 1).
// h_n (first kind): closed forms h_0 = -i e^{iz}/z, h_1 = -e^{iz}(z + i)/z^2,
//      then the upward recurrence h_{n+1} = (2n+1)/z h_n - h_{n-1}.
// ---------------------------------------------------------------------------
OM_HD void sph_j(zd z, int L1, zd *f) {
  double az = cabs(z);
  int N = (L1 > (int)az ? L1 : (int)az) + 30 + (int)(4.0 * cbrt(az));
  zd r = mk(0.0, 0.0);
  zd keep[kMaxOrder + 1];
  for(int n = N; n >= 1; --n) {
    r = z / (mk(double(2 * n + 1), 0.0) - z * r);
    if(n <= L1)
      keep[n] = r;
  }
  zd s = csin(z), c = ccos(z);
  zd j0 = s / z;
  f[0] = j0;
  if(L1 == 0)
    return;
  zd j1 = (s / z - c) / z;
  if(az >= 1.0 && norm2(j1) > norm2(j0))
    f[1] = j1;
  else
    f[1] = j0 * keep[1];
  for(int n = 2; n <= L1; ++n)
    f[n] = f[n - 1] * keep[n];
}

OM_HD void sph_h1(zd z, int L1, zd *f) {
  zd e = cexp_i(z);
  const zd rz = 1.0 / z;
  f[0] = mk(e.im, -e.re) * rz;  // -i e / z
  if(L1 == 0)
    return;
  f[1] = -(e * (z + mk(0.0, 1.0))) * (rz * rz);
  for(int n = 1; n < L1; ++n)
    f[n + 1] = double(2 * n + 1) * (rz * f[n]) - f[n - 1];
}

// Values and derivatives for orders 0..L the way OPTIMET's bessel<> wrapper
// assembles them (srcAna/Bessel.h:58-143): zero-argument branch for |z| <= 1e-10,
// derivative z_n' = -z_{n+1} + (n/z) z_n, imaginary parts cleared for j_n of a
// real argument. type 0 = Bessel j, 1 = Hankel h^(1).
OM_HD void bessel_deriv(int type, zd z, int L, zd *data, zd *ddata) {
  if(cabs(z) <= 1e-10) {
    for(int i = 0; i <= L; ++i) {
      data[i] = mk(0.0, 0.0);
      ddata[i] = mk(0.0, 0.0);
    }
    if(type == 0)
      data[0] = mk(1.0, 0.0);
  } else {
    zd f[kMaxOrder + 2];
    if(type == 0)
      sph_j(z, L + 1, f);
    else
      sph_h1(z, L + 1, f);
    for(int i = 0; i <= L; ++i) {
      data[i] = f[i];
      if(ddata)
        ddata[i] = (double(i) / z) * f[i] - f[i + 1];
    }
  }
  if(z.im == 0.0 && type == 0) {
    for(int i = 0; i <= L; ++i) {
      data[i].im = 0.0;
      if(ddata)
        ddata[i].im = 0.0;
    }
  }
}

// ---------------------------------------------------------------------------
// Wigner d functions of AuxCoefficients::VIGdVIG (srcAna/AuxCoefficients.cpp:217-290),
// including its theta nudge (applied after the m < 0 reflection) and the
// final-order derivative term. W, dW: orders 0..nMax.
// ---------------------------------------------------------------------------
OM_HD double factorial_d(unsigned n) {
  double r = 1.0;
  for(unsigned i = 2; i <= n; ++i)
    r *= i;
  return r;
}

OM_HD void vigdvig(int nMaxI, int mI, double the, double *W, double *dW) {
  unsigned long nMax = nMaxI;
  for(unsigned long i = 0; i <= nMax; ++i) {
    W[i] = 0.0;
    dW[i] = 0.0;
  }
  bool neg = mI < 0;
  int m = mI < 0 ? -mI : mI;
  unsigned long n_min = (unsigned long)m;
  double vig_the = neg ? kPi - the : the;
  if((fabs(the) < 1e-10) || (fabs(the) - kPi + 1e-10 > 0.0))
    vig_the = vig_the + 1e-6;
  double x = cos(vig_the);
  double sv = sin(vig_the);
  W[n_min] = pow(2.0, -m) * (sqrt(factorial_d(2u * unsigned(m))) / factorial_d(unsigned(m))) *
             pow(1.0 - x, m / 2.0) * pow(1.0 + x, m / 2.0);
  unsigned long s = n_min, mm = (unsigned long)(m * m);
  if(n_min == 0 && nMax > 0) {
    W[1] = x * W[0];
    s = 1;
  }
  for(; s < nMax; ++s) {
    W[s + 1] = ((2 * s + 1) * x * W[s] - sqrt(double(s * s - mm)) * W[s - 1]) /
               sqrt(double((s + 1) * (s + 1) - mm));
    dW[s] = (((s * sqrt(double((s + 1) * (s + 1) - mm)) * W[s + 1]) / (2 * s + 1)) -
             (((s + 1) * sqrt(double(s * s * (s * s - mm))) * W[s - 1]) / (s * (2 * s + 1)))) /
            sv;
  }
  if(nMax > 0) {
    double Wn = ((2 * nMax + 1) * x * W[nMax] - sqrt(double(nMax * nMax - mm)) * W[nMax - 1]) /
                sqrt(double((nMax + 1) * (nMax + 1) - mm));
    dW[nMax] = (((nMax * sqrt(double((nMax + 1) * (nMax + 1) - mm)) * Wn) / (2 * nMax + 1)) -
                (((nMax + 1) * sqrt(double(nMax * nMax * (nMax * nMax - mm))) * W[nMax - 1]) /
                 (nMax * (2 * nMax + 1)))) /
               sv;
  }
  if(neg) {
    for(unsigned long i = 0; i <= nMax; ++i) {
      double c = (i & 1) ? -1.0 : 1.0;
      W[i] *= c;
      dW[i] *= -c;
    }
  }
}

// Cartesian <-> spherical as OPTIMET's Tools/Spherical do it.
OM_HD void to_spherical(double x, double y, double z, double *r, double *t, double *p) {
  double rl = sqrt(x * x + y * y + z * z);
  if(rl > 0.0) {
    *r = rl;
    *t = acos(z / rl);
    *p = atan2(y, x);
  } else {
    *r = 0.0;
    *t = 0.0;
    *p = 0.0;
  }
}
OM_HD void to_cartesian(double r, double t, double p, double *x, double *y, double *z) {
  *x = r * sin(t) * cos(p);
  *y = r * sin(t) * sin(p);
  *z = r * cos(t);
}

OM_HD int flat(int n, int m) { return n * (n + 1) - m - 1; }
OM_HD int pmax(int nmax) { return nmax * (nmax + 2); }

}  // namespace om
