// Vector spherical wave sums shared by the FF and SH field kernels.
#pragma once

#include "om_math.cuh"

namespace om {

// sum_p (M_p c_p + N_p d_p) and sum_p (N_p c_p + M_p d_p) of one AuxCoefficients
// expansion (AuxCoefficients.cpp:292-343) about a centre, in local spherical
// components; projected to Cartesian by the caller (Tools::toProjection).
__device__ inline void vswf_sum(double r, double th, double ph, zd k, int regular, int nmax, const zd *c,
                         const zd *d, zd eloc[3], zd hloc[3]) {
  zd z[kMaxNmax + 2], dz[kMaxNmax + 2];
  const zd Kr = k * r;
  bessel_deriv(regular ? 0 : 1, r * k, nmax, z, dz);
  const zd invKr = 1.0 / Kr;
  double W[kMaxNmax + 1], dW[kMaxNmax + 1];
  const bool pole = fabs(th) < 1e-10 || (fabs(th) - kPi + 1e-10) > 0.0;
  const double inv_trig = pole ? 1.0 / cos(th) : 1.0 / sin(th);
  const int P = pmax(nmax);
  for(int q = 0; q < 3; ++q) {
    eloc[q] = mk(0.0, 0.0);
    hloc[q] = mk(0.0, 0.0);
  }
  for(int m = nmax; m >= -nmax; --m) {
    vigdvig(nmax, m, th, W, dW);
    const double dm = (m & 1) ? -1.0 : 1.0;
    double sn, cs;
    sincos(m * ph, &sn, &cs);
    const zd e = mk(cs, sn);
    for(int n = (m < 0 ? -m : m); n <= nmax; ++n) {
      if(n == 0)
        continue;
      const double A = (m == 0) ? 0.0 : (pole ? m * inv_trig * dW[n] : m * inv_trig * W[n]);
      const double dn = sqrt((2.0 * n + 1.0) / (4.0 * kPi * (double)(n * (n + 1))));
      const zd ct = (dm * dn) * e;
      const zd cz = ct * z[n];
      // M = ct z_n C_n, C_n = (0, iA, -dW)
      const zd Mt = mk(-cz.im * A, cz.re * A), Mp = -dW[n] * cz;
      // N = (1/Kr) dm dn (n(n+1) z_n P_n + (Kr z_n' + z_n) B_n) e, B_n = (0, dW, iA)
      const zd pre = invKr * ct;
      const zd rad = Kr * dz[n] + z[n];
      const zd Nr = pre * (double(n * (n + 1)) * W[n] * z[n]);
      const zd prad = pre * rad;
      const zd Nt = dW[n] * prad, Np = mk(-prad.im * A, prad.re * A);
      const int p = flat(n, m);
      const zd cp = c[p], dp = d[p];
      eloc[0] = eloc[0] + Nr * dp;
      eloc[1] = eloc[1] + Mt * cp + Nt * dp;
      eloc[2] = eloc[2] + Mp * cp + Np * dp;
      hloc[0] = hloc[0] + Nr * cp;
      hloc[1] = hloc[1] + Nt * cp + Mt * dp;
      hloc[2] = hloc[2] + Np * cp + Mp * dp;
    }
  }
  (void)P;
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
