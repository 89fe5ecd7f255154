// Post-processing of the OPTIMET sphere path on the device: internal
// coefficients, the four cross sections and the near-field summation.
#include "om_internal.h"

namespace om {

namespace {

// convertInternal (Solver.cpp:57-77): X_int = X_sca (.) Iaux
__global__ void k_internal(const zd *X, const zd *iaux, int nmax, long n, zd *Xint) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(idx >= n)
    return;
  const int P = pmax(nmax);
  const long j = idx / (2 * P);
  const int r = (int)(idx - j * 2 * P);
  const int p = r < P ? r : r - P;
  const int nn = (int)sqrt((double)(p + 1));
  Xint[idx] = X[idx] * iaux[j * 2 * (nmax + 1) + 2 * nn + (r < P ? 0 : 1)];
}

// getExtinctionCrossSection / getScatteringCrossSection / getAbsorptionCrossSection
// (Result.cpp:541-631), one CTA, fixed-order reduction (deterministic).
__global__ void __launch_bounds__(256) k_cross_sections(const zd *X, const zd *incloc,
                                                        const double *wsca, const double *cabs,
                                                        int N, int nmax, double kr2, double *out) {
  __shared__ double red[3][256];
  const int P = pmax(nmax);
  double e = 0.0, s = 0.0, a = 0.0;
  for(long idx = threadIdx.x; idx < (long)N * P; idx += blockDim.x) {
    const long j = idx / P;
    const int p = (int)(idx - j * P);
    const int nn = (int)sqrt((double)(p + 1));
    const zd cte = X[j * 2 * P + p], ctm = X[j * 2 * P + P + p];
    const zd qte = incloc[j * 2 * P + p], qtm = incloc[j * 2 * P + P + p];
    e += (conj(qte) * cte + conj(qtm) * ctm).re;
    const double n_te = norm2(cte), n_tm = norm2(ctm);
    s += wsca[j * P + p] * (n_te + n_tm);
    a += n_te * cabs[j * 2 * (nmax + 1) + 2 * nn] + n_tm * cabs[j * 2 * (nmax + 1) + 2 * nn + 1];
  }
  red[0][threadIdx.x] = e;
  red[1][threadIdx.x] = s;
  red[2][threadIdx.x] = a;
  __syncthreads();
  for(int w = blockDim.x / 2; w > 0; w >>= 1) {
    if(threadIdx.x < w)
      for(int c = 0; c < 3; ++c)
        red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    out[0] = (-1. / kr2) * red[0][0];
    out[1] = (1. / kr2) * red[1][0];
    out[2] = out[0] - out[1];
    out[3] = (1 / kr2) * red[2][0];
  }
}

struct FieldArgs {
  const double *xyz;      // points, Cartesian (after the reader's spherical round trip)
  int npts;
  const double *cart;     // sphere centres
  const double *radius;
  int N, nmax;
  const zd *X, *Xint, *inc;
  zd waveK;               // background wave number
  zd iZ;                  // -i / sqrt(mu_b / eps_b)
  const zd *k_in;         // per sphere: waveK_0 sqrt(eps_r mu_r)
  const zd *iZ_in;        // per sphere: -i / sqrt(mu / eps)
  zd *E, *H;
};

// sum_p (M_p c_p + N_p d_p) and sum_p (N_p c_p + M_p d_p) of one AuxCoefficients
// expansion (AuxCoefficients.cpp:292-343) about a centre, in local spherical
// components; projected to Cartesian by the caller (Tools::toProjection).
__device__ void vswf_sum(double r, double th, double ph, zd k, int regular, int nmax, const zd *c,
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

// Result::getEHFields, fundamental frequency, Cartesian components
// (Result.cpp:74-301) with Geometry::checkInner (Geometry.cpp:147-163).
__global__ void __launch_bounds__(128) k_near_field(FieldArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= a.npts)
    return;
  const int P = pmax(a.nmax);
  const double px = a.xyz[3 * i], py = a.xyz[3 * i + 1], pz = a.xyz[3 * i + 2];
  zd E[3] = {mk(0, 0), mk(0, 0), mk(0, 0)}, H[3] = {mk(0, 0), mk(0, 0), mk(0, 0)};
  int inner = -1;
  for(int j = 0; j < a.N; ++j) {
    double r, t, p;
    to_spherical(px - a.cart[3 * j], py - a.cart[3 * j + 1], pz - a.cart[3 * j + 2], &r, &t, &p);
    if(r <= a.radius[j]) {
      inner = j;
      break;
    }
  }
  const zd one = mk(1.0, 0.0);
  zd el[3], hl[3];
  if(inner < 0) {
    double r, t, p;
    to_spherical(px, py, pz, &r, &t, &p);
    vswf_sum(r, t, p, a.waveK, 1, a.nmax, a.inc, a.inc + P, el, hl);
    zd Ei[3] = {mk(0, 0), mk(0, 0), mk(0, 0)}, Hi[3] = {mk(0, 0), mk(0, 0), mk(0, 0)};
    project_add(t, p, el, one, Ei);
    project_add(t, p, hl, a.iZ, Hi);
    for(int j = 0; j < a.N; ++j) {
      to_spherical(px - a.cart[3 * j], py - a.cart[3 * j + 1], pz - a.cart[3 * j + 2], &r, &t, &p);
      const zd *c = a.X + (size_t)j * 2 * P;
      vswf_sum(r, t, p, a.waveK, 0, a.nmax, c, c + P, el, hl);
      project_add(t, p, el, one, E);
      project_add(t, p, hl, a.iZ, H);
    }
    for(int q = 0; q < 3; ++q) {
      E[q] = Ei[q] + E[q];
      H[q] = Hi[q] + H[q];
    }
  } else {
    double r, t, p;
    to_spherical(px - a.cart[3 * inner], py - a.cart[3 * inner + 1], pz - a.cart[3 * inner + 2],
                 &r, &t, &p);
    const zd *c = a.Xint + (size_t)inner * 2 * P;
    vswf_sum(r, t, p, a.k_in[inner], 1, a.nmax, c, c + P, el, hl);
    project_add(t, p, el, one, E);
    project_add(t, p, hl, a.iZ_in[inner], H);
  }
  for(int q = 0; q < 3; ++q) {
    a.E[3 * (size_t)i + q] = E[q];
    a.H[3 * (size_t)i + q] = H[q];
  }
}

}  // namespace

void launch_internal(om_problem *pr) {
  k_internal<<<blocks_for(pr->n, 256), 256, 0, pr->ctx->stream>>>(pr->d_X, pr->d_iaux, pr->nmax,
                                                                 pr->n, pr->d_Xint);
  pr->ctx->last_launches++;
}

void launch_cross_sections(om_problem *pr) {
  double kr = pr->waveK.real();
  k_cross_sections<<<1, 256, 0, pr->ctx->stream>>>(pr->d_X, pr->d_incloc, pr->d_wsca, pr->d_cabs,
                                                   pr->N, pr->nmax, kr * kr, pr->d_xsec);
  pr->ctx->last_launches++;
}

void launch_near_field(om_problem *pr, const double *d_xyz, int npts, zd *d_E, zd *d_H) {
  FieldArgs a;
  a.xyz = d_xyz;
  a.npts = npts;
  a.cart = pr->d_cart;
  a.radius = pr->d_radius;
  a.N = pr->N;
  a.nmax = pr->nmax;
  a.X = pr->d_X;
  a.Xint = pr->d_Xint;
  a.inc = pr->d_inc;
  a.waveK = mk(pr->waveK.real(), pr->waveK.imag());
  a.iZ = mk(pr->iZ.real(), pr->iZ.imag());
  a.k_in = pr->d_kin;
  a.iZ_in = pr->d_izin;
  a.E = d_E;
  a.H = d_H;
  k_near_field<<<blocks_for(npts, 128), 128, 0, pr->ctx->stream>>>(a);
  pr->ctx->last_launches++;
}

}  // namespace om
