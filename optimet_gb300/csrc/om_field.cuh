// Vector spherical wave sums shared by the FF and SH field kernels.
#pragma once

#include "om_math.cuh"

namespace om {

// Geometry-independent tables of the field kernels, one copy per CTA in
// shared memory: the Wigner-d recurrence of AuxCoefficients::VIGdVIG
// (AuxCoefficients.cpp:217-290) rewritten with precomputed ratios,
//   W[s+1] = ra[m][s] x W[s] - rb[m][s] W[s-1],
//   dW[s]  = (rc[m][s] W[s+1] - rd[m][s] W[s-1]) / sin(theta),
// its starting values w0[m] = 2^-m sqrt((2m)!) / m! (times
// ((1-x)(1+x))^(m/2)), and the VSWF normalisation dn[n]
// (AuxCoefficients::compute_dn, AuxCoefficients.cpp:31-39).
struct WigTab {
  double ra[kMaxNmax + 1][kMaxNmax + 1], rb[kMaxNmax + 1][kMaxNmax + 1];
  double rc[kMaxNmax + 1][kMaxNmax + 1], rd[kMaxNmax + 1][kMaxNmax + 1];
  double w0[kMaxNmax + 1], dn[kMaxNmax + 1];
};

__device__ inline void wigtab_fill(WigTab &t) {
  constexpr int S = kMaxNmax + 1;
  for(int idx = threadIdx.x; idx < S * S; idx += blockDim.x) {
    const int m = idx / S, s = idx - m * S;
    const double mm = (double)m * m, s1 = sqrt((double)(s + 1) * (s + 1) - mm);
    const double s0 = s >= m ? sqrt((double)s * s - mm) : 0.0;
    t.ra[m][s] = (2.0 * s + 1.0) / s1;
    t.rb[m][s] = s0 / s1;
    t.rc[m][s] = s * s1 / (2.0 * s + 1.0);
    t.rd[m][s] = s >= 1 && s >= m ? (s + 1.0) * sqrt((double)s * s * ((double)s * s - mm)) /
                                         (s * (2.0 * s + 1.0))
                                   : 0.0;
  }
  for(int m = threadIdx.x; m < S; m += blockDim.x) {
    double f = 1.0;
    for(int i = 2; i <= 2 * m; ++i)
      f *= i;
    double g = 1.0;
    for(int i = 2; i <= m; ++i)
      g *= i;
    t.w0[m] = pow(2.0, -m) * sqrt(f) / g;
    t.dn[m] = m ? sqrt((2.0 * m + 1.0) / (4.0 * kPi * (double)(m * (m + 1)))) : 0.0;
  }
}

// sum_p (M_p c_p + N_p d_p) and sum_p (N_p c_p + M_p d_p) of one AuxCoefficients
// expansion (AuxCoefficients.cpp:292-343) about a centre, in local spherical
// components (projected to Cartesian by the caller, Tools::toProjection).
// NM >= nmax is the compile-time bound that keeps the Wigner values in
// registers; zs is this thread's slice of shared memory for the radial
// factors (3 (NM + 1) complex values, stride `zst` between entries).
// The radial factors fold the normalisation: Z1 = dn z_n,
// Z2 = dn (Kr z_n' + z_n) / Kr, Z3 = n (n + 1) dn z_n / Kr, so that for each m
// the six sums are real-weighted combinations of Z1..Z3 with c_p, d_p,
// multiplied once by (-1)^m e^{i m phi}.
template <int NM>
__device__ void vswf_point(const WigTab &T, zd *zs, int zst, double r, double th, double ph, zd k,
                           int regular, int nmax, const zd *c, const zd *d, zd eloc[3],
                           zd hloc[3]) {
  zd *Z1 = zs, *Z2 = zs + (NM + 1) * zst, *Z3 = zs + 2 * (NM + 1) * zst;
  const zd Kr = k * r;
  const zd invKr = 1.0 / Kr;
  if(regular) {
    zd z[kMaxNmax + 2], dz[kMaxNmax + 2];
    bessel_deriv(0, r * k, nmax, z, dz);
    for(int n = 1; n <= nmax; ++n) {
      const double dn = T.dn[n];
      Z1[n * zst] = dn * z[n];
      Z2[n * zst] = (dn * (Kr * dz[n] + z[n])) * invKr;
      Z3[n * zst] = (double(n * (n + 1)) * dn * z[n]) * invKr;
    }
  } else {
    // h_n(z), h_n'(z) by the upward recurrence of sph_h1 / bessel_deriv
    const zd zz = r * k;
    if(cabs(zz) <= 1e-10) {
      for(int n = 1; n <= nmax; ++n)
        Z1[n * zst] = Z2[n * zst] = Z3[n * zst] = mk(0.0, 0.0);
    } else {
      const zd e = cexp_i(zz), rz = 1.0 / zz;
      zd f0 = mk(e.im, -e.re) * rz;
      zd f1 = -(e * (zz + mk(0.0, 1.0))) * (rz * rz);
      for(int n = 1; n <= nmax; ++n) {
        const zd f2 = double(2 * n + 1) * (rz * f1) - f0;  // h_{n+1}
        const zd dz = (double(n) * rz) * f1 - f2;
        const double dn = T.dn[n];
        Z1[n * zst] = dn * f1;
        Z2[n * zst] = (dn * (Kr * dz + f1)) * invKr;
        Z3[n * zst] = (double(n * (n + 1)) * dn * f1) * invKr;
        f0 = f1;
        f1 = f2;
      }
    }
  }
  const bool pole = fabs(th) < 1e-10 || (fabs(th) - kPi + 1e-10) > 0.0;
  const double inv_trig = pole ? 1.0 / cos(th) : 1.0 / sin(th);
  // VIGdVIG's angle: theta (m >= 0) or pi - theta (m < 0), nudged at the poles
  double xs[2], svi[2], q[2];
  for(int g = 0; g < 2; ++g) {
    double vt = g ? kPi - th : th;
    if(pole)
      vt += 1e-6;
    const double x = cos(vt);
    xs[g] = x;
    svi[g] = 1.0 / sin(vt);
    q[g] = sqrt(1.0 - x) * sqrt(1.0 + x);
  }
  double sp, cp;
  sincos(ph, &sp, &cp);
  const zd e1 = mk(cp, sp);
  zd em;  // e^{i m phi}, advanced by e^{i phi} per m
  {
    double s0, c0;
    sincos(-nmax * ph, &s0, &c0);
    em = mk(c0, s0);
  }
  for(int t = 0; t < 3; ++t) {
    eloc[t] = mk(0.0, 0.0);
    hloc[t] = mk(0.0, 0.0);
  }
  for(int m = -nmax; m <= nmax; ++m, em = em * e1) {
    const int am = m < 0 ? -m : m, g = m < 0;
    const double x = xs[g], isv = svi[g];
    double qm = 1.0;
    for(int i = 0; i < am; ++i)
      qm *= q[g];
    double W[NM + 2], dW[NM + 1];
#pragma unroll
    for(int s = 0; s <= NM; ++s) {
      W[s] = (s == am) ? T.w0[am] * qm : 0.0;
      dW[s] = 0.0;
    }
    W[NM + 1] = 0.0;
#pragma unroll
    for(int s = 0; s <= NM; ++s) {
      // VIGdVIG: for m = 0 the first step is W[1] = x W[0] (no dW[0])
      if(s >= am && s <= nmax) {
        const double wm1 = s > 0 ? W[s > 0 ? s - 1 : 0] : 0.0;
        const double wp = (am == 0 && s == 0) ? x * W[0] : T.ra[am][s] * x * W[s] - T.rb[am][s] * wm1;
        if(s < nmax || (am == 0 && s == 0))
          W[s + 1] = wp;
        if(!(am == 0 && s == 0))
          dW[s] = (T.rc[am][s] * wp - T.rd[am][s] * wm1) * isv;
      }
    }
    if(g) {
#pragma unroll
      for(int s = 0; s <= NM; ++s) {
        if(s & 1) {
          W[s] = -W[s];
        } else {
          dW[s] = -dW[s];
        }
      }
    }
    zd S[6];
    for(int t = 0; t < 6; ++t)
      S[t] = mk(0.0, 0.0);
#pragma unroll
    for(int n = 1; n <= NM; ++n) {
      if(n >= am && n <= nmax) {
        const double A = (m == 0) ? 0.0 : (pole ? m * inv_trig * dW[n] : m * inv_trig * W[n]);
        const zd z1 = Z1[n * zst], z2 = Z2[n * zst], z3 = Z3[n * zst];
        const int p = flat(n, m);
        const zd cc = c[p], dd = d[p];
        const zd wz3 = W[n] * z3, dwz2 = dW[n] * z2, dwz1 = dW[n] * z1;
        const zd iaz1 = mk(-A * z1.im, A * z1.re), iaz2 = mk(-A * z2.im, A * z2.re);
        S[0] = S[0] + wz3 * dd;
        S[1] = S[1] + iaz1 * cc + dwz2 * dd;
        S[2] = S[2] + iaz2 * dd - dwz1 * cc;
        S[3] = S[3] + wz3 * cc;
        S[4] = S[4] + dwz2 * cc + iaz1 * dd;
        S[5] = S[5] + iaz2 * cc - dwz1 * dd;
      }
    }
    // (-1)^m e^{i m phi}
    const zd ep = ((am & 1) ? -1.0 : 1.0) * em;
    for(int t = 0; t < 3; ++t) {
      eloc[t] = eloc[t] + ep * S[t];
      hloc[t] = hloc[t] + ep * S[3 + t];
    }
  }
}

__device__ __forceinline__ void project_add(double th, double ph, const zd v[3], zd s, zd out[3]) {
  const double st = sin(th), ct = cos(th), sp = sin(ph), cp = cos(ph);
  zd x = st * cp * v[0] + ct * cp * v[1] - sp * v[2];
  zd y = st * sp * v[0] + ct * sp * v[1] + cp * v[2];
  zd zz = ct * v[0] - st * v[1];
  out[0] = out[0] + x * s;
  out[1] = out[1] + y * s;
  out[2] = out[2] + zz * s;
}

}  // namespace om
