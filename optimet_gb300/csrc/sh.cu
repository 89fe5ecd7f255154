// Second harmonic on the device: the nine coupling tables (Wigner 3j/6j/9j),
// the SH source terms u', v', u'' and their analytic part, SH internal
// coefficients and the SH cross sections.
//
// Tables: Symbol.cpp:1036-1451 (computed once per nMax and context; entries
// with M != M1 + M2 vanish through their Clebsch-Gordan factor and are left 0).
// Source: Symbol.cpp:155-353 with Geometry.cpp:250-310 and
// PreconditionedMatrix.cpp:1347-1436; every bilinear form only visits the
// (p, q) with m_q = M - m_p.
#include <cmath>
#include <stdexcept>
#include <vector>

#include "om_field.cuh"
#include "om_internal.h"

namespace om {

namespace {

enum { T_C10m1, T_C11m1, T_C00m1, T_C01m1, T_Wm1m1, T_W11, T_W00, T_W10, T_W01 };

// Wigner symbols from their Racah formulas (zero outside the triangle and
// projection rules); f is a factorial table in shared memory.
__device__ __forceinline__ bool tri(int a, int b, int c) { return c >= abs(a - b) && c <= a + b; }
__device__ __forceinline__ double fk(const double *f, int n) { return n < 0 ? 0.0 : f[n]; }

__device__ __noinline__ double w3j(const double *f, int j1, int j2, int j3, int m1, int m2, int m3) {
  if(j1 < 0 || j2 < 0 || j3 < 0 || !tri(j1, j2, j3) || m1 + m2 + m3 != 0 || abs(m1) > j1 ||
     abs(m2) > j2 || abs(m3) > j3)
    return 0.0;
  const double delta = sqrt(fk(f, j1 + j2 - j3) * fk(f, j1 - j2 + j3) * fk(f, -j1 + j2 + j3) /
                            fk(f, j1 + j2 + j3 + 1));
  const double pre = sqrt(fk(f, j1 + m1) * fk(f, j1 - m1) * fk(f, j2 + m2) * fk(f, j2 - m2) *
                          fk(f, j3 + m3) * fk(f, j3 - m3));
  const int kmin = max(0, max(j2 - j3 - m1, j1 - j3 + m2));
  const int kmax = min(j1 + j2 - j3, min(j1 - m1, j2 + m2));
  double sum = 0.0;
  for(int k = kmin; k <= kmax; ++k) {
    const double den = fk(f, k) * fk(f, j3 - j2 + k + m1) * fk(f, j3 - j1 + k - m2) *
                       fk(f, j1 + j2 - j3 - k) * fk(f, j1 - k - m1) * fk(f, j2 - k + m2);
    sum += ((k & 1) ? -1.0 : 1.0) / den;
  }
  return (((j1 - j2 - m3) & 1) ? -1.0 : 1.0) * delta * pre * sum;
}

__device__ __forceinline__ double tdelta(const double *f, int a, int b, int c) {
  return sqrt(fk(f, a + b - c) * fk(f, a - b + c) * fk(f, -a + b + c) / fk(f, a + b + c + 1));
}

__device__ __noinline__ double w6j(const double *f, int j1, int j2, int j3, int j4, int j5, int j6) {
  if(j1 < 0 || j2 < 0 || j3 < 0 || j4 < 0 || j5 < 0 || j6 < 0)
    return 0.0;
  if(!tri(j1, j2, j3) || !tri(j1, j5, j6) || !tri(j4, j2, j6) || !tri(j4, j5, j3))
    return 0.0;
  const int a1 = j1 + j2 + j3, a2 = j1 + j5 + j6, a3 = j4 + j2 + j6, a4 = j4 + j5 + j3;
  const int b1 = j1 + j2 + j4 + j5, b2 = j2 + j3 + j5 + j6, b3 = j3 + j1 + j6 + j4;
  const int tmin = max(max(a1, a2), max(a3, a4)), tmax = min(b1, min(b2, b3));
  double sum = 0.0;
  for(int t = tmin; t <= tmax; ++t) {
    const double den = fk(f, t - a1) * fk(f, t - a2) * fk(f, t - a3) * fk(f, t - a4) *
                       fk(f, b1 - t) * fk(f, b2 - t) * fk(f, b3 - t);
    sum += ((t & 1) ? -1.0 : 1.0) * fk(f, t + 1) / den;
  }
  return tdelta(f, j1, j2, j3) * tdelta(f, j1, j5, j6) * tdelta(f, j4, j2, j6) *
         tdelta(f, j4, j5, j3) * sum;
}

__device__ __noinline__ double w9j(const double *f, int a, int b, int c, int d, int e, int g6, int g, int h, int i) {
  if(a < 0 || b < 0 || c < 0 || d < 0 || e < 0 || g6 < 0 || g < 0 || h < 0 || i < 0)
    return 0.0;
  const int xmin = max(abs(a - i), max(abs(h - d), abs(b - g6)));
  const int xmax = min(a + i, min(h + d, b + g6));
  double sum = 0.0;
  for(int x = xmin; x <= xmax; ++x)
    sum += (2 * x + 1) * w6j(f, a, d, g, h, i, x) * w6j(f, b, e, h, d, x, g6) *
           w6j(f, c, g6, i, x, a, b);
  return sum;
}

// Symbol.cpp:39-43 and :110-116
__device__ __noinline__ double cg(const double *f, int j, int m, int j1, int m1, int j2, int m2) {
  return (((m + j1 - j2) & 1) ? -1.0 : 1.0) * sqrt(2.0 * j + 1.0) * w3j(f, j1, j2, j, m1, m2, -m);
}
__device__ __noinline__ double Wf(const double *f, int L1, int J1, int M1, int L2, int J2, int M2, int L, int M) {
  return (((J2 + L1 + L) & 1) ? -1.0 : 1.0) *
         sqrt((2.0 * J1 + 1.0) * (2.0 * J2 + 1.0) * (2.0 * L1 + 1.0) * (2.0 * L2 + 1.0) /
              (4.0 * kPi * (2.0 * L + 1.0))) *
         w6j(f, L1, L2, L, J2, J1, 1) * cg(f, L, 0, L1, 0, L2, 0) * cg(f, L, M, J1, M1, J2, M2);
}

__host__ __device__ __forceinline__ void nm_of(int p, int &n, int &m) {
  n = (int)sqrtf((float)(p + 1));
  while(n * n > p + 1)
    --n;
  while((n + 1) * (n + 1) <= p + 1)
    ++n;
  m = -(p + 1) + n * (n + 1);
}

// One CTA per SH harmonic k; threads over (p, m2 fixed by M - m1, n2).
__global__ void __launch_bounds__(256) k_clg_tables(int nmax, double *out) {
  __shared__ double f[171];
  if(threadIdx.x == 0) {
    f[0] = 1.0;
    for(int i = 1; i <= 170; ++i)
      f[i] = f[i - 1] * i;
  }
  __syncthreads();
  const int P = pmax(nmax);
  const size_t sz = (size_t)P * P * P;
  const int k = blockIdx.x;
  int J, M;
  nm_of(k, J, M);
  const double s32 = sqrt(3.0 / 2.0 / kPi);
  for(int idx = threadIdx.x; idx < P * P; idx += blockDim.x) {
    const int p = idx / P, q = idx - p * P;
    int J1, M1, J2, M2;
    nm_of(p, J1, M1);
    nm_of(q, J2, M2);
    if(M != M1 + M2)
      continue;
    const size_t at = ((size_t)k * P + p) * P + q;
    const double c = cg(f, J, M, J1, M1, J2, M2);
    const double jp = sqrt(J / (2.0 * J + 1.0)), jm = sqrt((J + 1) / (2.0 * J + 1.0));
    const double r2m = sqrt(J2 * (2.0 * J2 - 1.0)), r2p = sqrt((J2 + 1.0) * (2.0 * J2 + 3.0));
    out[T_C10m1 * sz + at] =
        s32 * (2.0 * J1 + 1.0) * c *
        (r2m * w9j(f, J1, J1, 1, J2, J2 - 1, 1, J, J + 1, 1) * cg(f, J + 1, 0, J1, 0, J2 - 1, 0) * jp -
         r2p * w9j(f, J1, J1, 1, J2, J2 + 1, 1, J, J + 1, 1) * cg(f, J + 1, 0, J1, 0, J2 + 1, 0) * jp +
         r2m * w9j(f, J1, J1, 1, J2, J2 - 1, 1, J, J - 1, 1) * cg(f, J - 1, 0, J1, 0, J2 - 1, 0) * jm -
         r2p * w9j(f, J1, J1, 1, J2, J2 + 1, 1, J, J - 1, 1) * cg(f, J - 1, 0, J1, 0, J2 + 1, 0) * jm);
    const double s_mm = sqrt((J1 + 1.0) * J2 * (2.0 * J1 - 1.0) * (2.0 * J2 - 1.0));
    const double s_mp = sqrt((J1 + 1.0) * (J2 + 1) * (2.0 * J1 - 1.0) * (2.0 * J2 + 3.0));
    const double s_pm = sqrt((double)(J1 * J2) * (2.0 * J1 + 3.0) * (2.0 * J2 - 1.0));
    const double s_pp = sqrt((double)(J1 * (J2 + 1)) * (2.0 * J1 + 3.0) * (2.0 * J2 + 3.0));
    out[T_C11m1 * sz + at] =
        s32 * c *
        (s_mm * w9j(f, J1, J1 - 1, 1, J2, J2 - 1, 1, J, J + 1, 1) * cg(f, J + 1, 0, J1 - 1, 0, J2 - 1, 0) * jp -
         s_mp * w9j(f, J1, J1 - 1, 1, J2, J2 + 1, 1, J, J + 1, 1) * cg(f, J + 1, 0, J1 - 1, 0, J2 + 1, 0) * jp +
         s_pm * w9j(f, J1, J1 + 1, 1, J2, J2 - 1, 1, J, J + 1, 1) * cg(f, J + 1, 0, J1 + 1, 0, J2 - 1, 0) * jp -
         s_pp * w9j(f, J1, J1 + 1, 1, J2, J2 + 1, 1, J, J + 1, 1) * cg(f, J + 1, 0, J1 + 1, 0, J2 + 1, 0) * jp +
         s_mm * w9j(f, J1, J1 - 1, 1, J2, J2 - 1, 1, J, J - 1, 1) * cg(f, J - 1, 0, J1 - 1, 0, J2 - 1, 0) * jm -
         s_mp * w9j(f, J1, J1 - 1, 1, J2, J2 + 1, 1, J, J - 1, 1) * cg(f, J - 1, 0, J1 - 1, 0, J2 + 1, 0) * jm +
         s_pm * w9j(f, J1, J1 + 1, 1, J2, J2 - 1, 1, J, J - 1, 1) * cg(f, J - 1, 0, J1 + 1, 0, J2 - 1, 0) * jm -
         s_pp * w9j(f, J1, J1 + 1, 1, J2, J2 + 1, 1, J, J - 1, 1) * cg(f, J - 1, 0, J1 + 1, 0, J2 + 1, 0) * jm);
    out[T_C00m1 * sz + at] =
        s32 * (2.0 * J1 + 1.0) * c *
        (r2m * w9j(f, J1, J1, 1, J2, J2 - 1, 1, J, J, 1) * cg(f, J, 0, J1, 0, J2 - 1, 0) -
         r2p * w9j(f, J1, J1, 1, J2, J2 + 1, 1, J, J, 1) * cg(f, J, 0, J1, 0, J2 + 1, 0));
    out[T_C01m1 * sz + at] =
        s32 * c *
        (s_mm * w9j(f, J1, J1 - 1, 1, J2, J2 - 1, 1, J, J, 1) * cg(f, J, 0, J1 - 1, 0, J2 - 1, 0) -
         s_mp * w9j(f, J1, J1 - 1, 1, J2, J2 + 1, 1, J, J, 1) * cg(f, J, 0, J1 - 1, 0, J2 + 1, 0) +
         s_pm * w9j(f, J1, J1 + 1, 1, J2, J2 - 1, 1, J, J, 1) * cg(f, J, 0, J1 + 1, 0, J2 - 1, 0) -
         s_pp * w9j(f, J1, J1 + 1, 1, J2, J2 + 1, 1, J, J, 1) * cg(f, J, 0, J1 + 1, 0, J2 + 1, 0));
    const double a1 = sqrt(J1 / (2.0 * J1 + 1.0)), b1 = sqrt((J1 + 1) / (2.0 * J1 + 1.0));
    const double a2 = sqrt(J2 / (2.0 * J2 + 1.0)), b2 = sqrt((J2 + 1) / (2.0 * J2 + 1.0));
    out[T_Wm1m1 * sz + at] = a1 * a2 * Wf(f, J1 - 1, J1, M1, J2 - 1, J2, M2, J, M) +
                             b1 * b2 * Wf(f, J1 + 1, J1, M1, J2 + 1, J2, M2, J, M) -
                             a1 * b2 * Wf(f, J1 - 1, J1, M1, J2 + 1, J2, M2, J, M) -
                             b1 * a2 * Wf(f, J1 + 1, J1, M1, J2 - 1, J2, M2, J, M);
    out[T_W11 * sz + at] = b1 * b2 * Wf(f, J1 - 1, J1, M1, J2 - 1, J2, M2, J, M) +
                           a1 * a2 * Wf(f, J1 + 1, J1, M1, J2 + 1, J2, M2, J, M) +
                           b1 * a2 * Wf(f, J1 - 1, J1, M1, J2 + 1, J2, M2, J, M) +
                           a1 * b2 * Wf(f, J1 + 1, J1, M1, J2 - 1, J2, M2, J, M);
    out[T_W00 * sz + at] = Wf(f, J1, J1, M1, J2, J2, M2, J, M);
    out[T_W10 * sz + at] = b1 * Wf(f, J1 - 1, J1, M1, J2, J2, M2, J, M) +
                           a1 * Wf(f, J1 + 1, J1, M1, J2, J2, M2, J, M);
    out[T_W01 * sz + at] = b2 * Wf(f, J1, J1, M1, J2 - 1, J2, M2, J, M) +
                           a2 * Wf(f, J1, J1, M1, J2 + 1, J2, M2, J, M);
  }
}

// Per sphere: A_0, A_1, A_m1 of Symbol.cpp:46-64 times conj(internal coefficients)
// (the solve passes them conjugated, PreconditionedMatrixSolver.h:65-70).
__global__ void k_sh_vectors(const ShScalars *shs, const zd *Xint, int nmax, zd *vec) {
  const int j = blockIdx.x, P = pmax(nmax);
  __shared__ zd J[kMaxNmax + 2], dJ[kMaxNmax + 2];
  const ShScalars c = shs[j];
  if(threadIdx.x == 0)
    bessel_deriv(0, c.R * c.k1, nmax, J, dJ);
  __syncthreads();
  const zd I = mk(0.0, 1.0);
  const zd rk = 1.0 / c.k1;
  for(int p = threadIdx.x; p < P; p += blockDim.x) {
    int n, m;
    nm_of(p, n, m);
    const zd cc = conj(Xint[(size_t)j * 2 * P + p]), dd = conj(Xint[(size_t)j * 2 * P + P + p]);
    zd *v = vec + (size_t)j * 3 * P;
    v[p] = J[n] * cc;
    v[P + p] = I * rk * (c.k1 * dJ[n] + J[n] / c.R) * dd;
    v[2 * P + p] = I * sqrt(n * (n + 1.0)) * (rk / c.R) * J[n] * dd;
  }
}

// u', v', u'' per (sphere, SH harmonic) and K, K1ana (source_vectorSH, K1ana).
// One CTA per sphere, one warp per SH harmonic k at a time: the lanes walk
// k's (p, q) pairs of the compact coupling table (coalesced), each keeping
// partial sums of the bilinear forms, which a warp reduction combines.
__global__ void __launch_bounds__(256) k_sh_source(const ShScalars *shs, const zd *vec, const int *off,
                                                   const int2 *pq, const double *val, long count,
                                                   const zd *shf, int nmax, zd *K, zd *K1) {
  extern __shared__ zd sv[];
  const int j = blockIdx.x, P = pmax(nmax);
  for(int t = threadIdx.x; t < 3 * P; t += blockDim.x)
    sv[t] = vec[(size_t)j * 3 * P + t];
  __syncthreads();
  const zd *a0 = sv, *a1 = sv + P, *am1 = sv + 2 * P;
  const ShScalars c = shs[j];
  const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  for(int k = threadIdx.x >> 5; k < P; k += warps) {
    zd up = mk(0, 0), vp = mk(0, 0), gmn = mk(0, 0), fmn = mk(0, 0);
    for(int t = off[k] + lane; t < off[k + 1]; t += 32) {
      const int p = pq[t].x, q = pq[t].y;
      const double *v = val + t;
      const zd a1am = a1[p] * am1[q], a0am = a0[p] * am1[q];
      up = up + a1am * v[T_C10m1 * count] + a0am * v[T_C11m1 * count];
      vp = vp + a1am * v[T_C00m1 * count] + a0am * v[T_C01m1 * count];
      gmn = gmn + am1[p] * am1[q] * v[T_Wm1m1 * count];
      fmn = fmn + a1[p] * a1[q] * v[T_W11 * count] + a0[p] * a0[q] * v[T_W00 * count] +
            a1[p] * a0[q] * v[T_W10 * count] + a0[p] * a1[q] * v[T_W01 * count];
    }
    for(int o = 16; o > 0; o >>= 1) {
      up.re += __shfl_down_sync(0xffffffffu, up.re, o);
      up.im += __shfl_down_sync(0xffffffffu, up.im, o);
      vp.re += __shfl_down_sync(0xffffffffu, vp.re, o);
      vp.im += __shfl_down_sync(0xffffffffu, vp.im, o);
      gmn.re += __shfl_down_sync(0xffffffffu, gmn.re, o);
      gmn.im += __shfl_down_sync(0xffffffffu, gmn.im, o);
      fmn.re += __shfl_down_sync(0xffffffffu, fmn.re, o);
      fmn.im += __shfl_down_sync(0xffffffffu, fmn.im, o);
    }
    if(lane == 0) {
      int J, M;
      nm_of(k, J, M);
      const double snn = sqrt((double)(J * (J + 1)));
      const zd u1 = up * c.c_up, v1 = vp * c.c_vp;
      const zd u2 = (c.c_g1 * snn) * gmn + (c.c_g2 * snn) * (gmn + fmn);
      const zd *f = shf + ((size_t)j * (nmax + 1) + J) * 8;
      const size_t o = (size_t)j * 2 * P;
      K[o + k] = f[0] * v1;               // + T2_TE * v'' (v'' = 0, Geometry.cpp:296)
      K[o + P + k] = f[1] * u1 + f[3] * u2;
      K1[o + k] = mk(0.0, 0.0);           // IauxSH2_TE * v''
      K1[o + P + k] = f[7] * u2;
    }
  }
}

// Gathers the compact table's coefficients from the dense tables.
__global__ void k_clg_compact(const double *tab, int P, const int2 *pq, const int *kof, long count,
                              double *val) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(t >= count)
    return;
  const size_t sz = (size_t)P * P * P;
  const size_t at = ((size_t)kof[t] * P + pq[t].x) * P + pq[t].y;
  for(int e = 0; e < 9; ++e)
    val[e * count + t] = tab[e * sz + at];
}

// convertInternal_SH (Solver.cpp:95-116)
__global__ void k_sh_internal(const zd *X, const zd *K1, const zd *shf, int nmax, long n, zd *Xi) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(idx >= n)
    return;
  const int P = pmax(nmax);
  const long j = idx / (2 * P);
  const int r = (int)(idx - j * 2 * P);
  const int p = r < P ? r : r - P;
  int nn, mm;
  nm_of(p, nn, mm);
  const zd f = shf[((size_t)j * (nmax + 1) + nn) * 8 + (r < P ? 4 : 5)];
  Xi[idx] = X[idx] * f - K1[idx];
}

// The bulk (gamma) sums CXm1 / CXp1 (Symbol.cpp:478-620) for SH harmonic k =
// (J, M) of one sphere at radius r; xi = that sphere's FF internal
// coefficients [c | d], d/dd/ddd = j_n(k1 r) and its first two derivatives.
// Only the (p, q) with m_q = M - m_p are visited (the tables vanish elsewhere).
__device__ void cx_sums(int k, int J, int M, int nmax, const zd *xi, const double *tab,
                        const zd *d, const zd *dd, const zd *ddd, zd k1, double r, zd c_bulk,
                        zd &Xm1, zd &Xp1) {
  const int P = pmax(nmax);
  const size_t sz = (size_t)P * P * P;
  const double sn = sqrt((double)(J * (J + 1)));
  const zd rk2 = 1.0 / (k1 * k1);
  Xm1 = mk(0.0, 0.0);
  Xp1 = mk(0.0, 0.0);
  for(int p = 0; p < P; ++p) {
    int n1, m1;
    nm_of(p, n1, m1);
    const int m2 = M - m1;
    if(m2 < -nmax || m2 > nmax)
      continue;
    const zd c1 = xi[p], d1 = xi[P + p];
    for(int n2 = max(1, abs(m2)); n2 <= nmax; ++n2) {
      const int q = flat(n2, m2);
      const size_t at = ((size_t)k * P + p) * P + q;
      const double Wm = tab[T_Wm1m1 * sz + at], W1 = tab[T_W11 * sz + at], W0 = tab[T_W00 * sz + at];
      const zd c2 = xi[q], d2 = xi[P + q];
      const zd F00 = d[n1] * dd[n2];
      const zd F11 = (k1 * dd[n2] + d[n2] / r) * (k1 * dd[n1] + d[n1] / r);
      const zd Fm = (1.0 / (r * r)) * (d[n1] * d[n2]);
      const zd Fd00 = d[n1] * dd[n2] * k1 + k1 * dd[n1] * d[n2];
      const zd Fd11 = ((k1 * k1) * ddd[n1] - (1.0 / (r * r)) * d[n1] + (1.0 / r) * k1 * dd[n1]) *
                          (k1 * dd[n2] + d[n2] / r) +
                      ((k1 * k1) * ddd[n2] - (1.0 / (r * r)) * d[n2] + (1.0 / r) * k1 * dd[n2]) *
                          (k1 * dd[n1] + d[n1] / r);
      const zd Fdm = (1.0 / (r * r)) * (k1 * dd[n1] * d[n2] + d[n1] * k1 * dd[n2]) -
                     (2.0 / (r * r * r)) * (d[n1] * d[n2]);
      const double sq = sqrt((double)(n1 * n2 * (n1 + 1) * (n2 + 1)));
      Xm1 = Xm1 + c_bulk * (c1 * c2 * W0 * Fd00 + d1 * d2 * rk2 * (W1 * Fd11 + Wm * sq * Fdm));
      Xp1 = Xp1 + c_bulk * (c1 * c2 * W0 * sn * (1.0 / r) * F00 +
                            d1 * d2 * rk2 * (W1 * sn * (1.0 / r) * F11 + Wm * sq * sn * (1.0 / r) * Fm));
    }
  }
}

// j_n(z), j_n'(z), j_n''(z) for n <= nmax (bessel3der, Bessel.h:145-245).
__device__ void bessel_j012(zd z, int nmax, zd *d, zd *dd, zd *ddd) {
  bessel_deriv(0, z, nmax, d, dd);
  ddd[0] = mk(0.0, 0.0);
  for(int i = 1; i <= nmax; ++i) {
    ddd[i] = -((double(i) / z) * dd[i]) + (double(i) / (z * z)) * d[i] + dd[i - 1];
    if(z.im == 0.0)
      ddd[i].im = 0.0;
  }
}

// ACSshcoeff (Symbol.cpp:358-477) per (sphere, SH harmonic): 4-point
// Gauss-Legendre radial integral.
__global__ void __launch_bounds__(256) k_sh_abs(const ShScalars *shs, const zd *Xint,
                                                const zd *Xish, const double *tab, int nmax,
                                                double omega, zd *acs) {
  const int j = blockIdx.x, P = pmax(nmax);
  __shared__ zd d[4][kMaxNmax + 2], dd[4][kMaxNmax + 2], ddd[4][kMaxNmax + 2];
  __shared__ zd ds[4][kMaxNmax + 2], dds[4][kMaxNmax + 2];
  const double xi[4] = {-0.3399810435848563, 0.3399810435848563, -0.8611363115940526,
                        0.8611363115940526};
  const double wi[4] = {0.6521451548625461, 0.6521451548625461, 0.3478548451374538,
                        0.3478548451374538};
  const ShScalars c = shs[j];
  const double R = c.R;
  if(threadIdx.x < 4) {
    const int g = threadIdx.x;
    const double r = (R / 2.0) * xi[g] + R / 2.0;
    const zd z = r * c.k1;
    bessel_j012(z, nmax, d[g], dd[g], ddd[g]);
    bessel_deriv(0, r * c.kSH, nmax, ds[g], dds[g]);
  }
  __syncthreads();
  const zd k1 = c.k1;
  for(int k = threadIdx.x; k < P; k += blockDim.x) {
    int J, M;
    nm_of(k, J, M);
    const double sn = sqrt((double)(J * (J + 1)));
    const zd cmn = Xish[(size_t)j * 2 * P + k], dmn = Xish[(size_t)j * 2 * P + P + k];
    zd integral = mk(0.0, 0.0);
    for(int g = 0; g < 4; ++g) {
      const double r = (R / 2.0) * xi[g] + R / 2.0;
      zd Xm1 = mk(0.0, 0.0), Xp1 = mk(0.0, 0.0);
      if(c.has_gamma)
        cx_sums(k, J, M, nmax, Xint + (size_t)j * 2 * P, tab, d[g], dd[g], ddd[g], k1, r, c.c_bulk,
                Xm1, Xp1);
      const zd w01 = c.w01;
      const zd rkSH = 1.0 / c.kSH;
      const zd Xm1SH = w01 * dmn * rkSH * sn * (1.0 / r) * ds[g][J];
      const zd X0 = -(w01 * cmn * ds[g][J]);
      const zd Xp1SH = w01 * dmn * rkSH * ((1.0 / r) * ds[g][J] + dds[g][J]);
      const zd a = Xm1 + Xm1SH, b = Xp1 + Xp1SH;
      integral = integral + wi[g] * (r * r) * (a * conj(a) + X0 * conj(X0) + b * conj(b));
    }
    acs[(size_t)j * P + k] = integral * (R / 2.0);
  }
}

// C_sca_SH (Result.cpp:662-745) and C_abs_SH (Result.cpp:747-778): one CTA,
// fixed-order reductions.
__global__ void __launch_bounds__(256) k_sh_xsec(const ShScalars *shs, const zd *X, const double *w,
                                                 const zd *acs, int N, int nmax, double arbcf,
                                                 zd eta, double *out) {
  __shared__ double red[2][256];
  const int P = pmax(nmax);
  double s = 0.0, a = 0.0;
  for(long idx = threadIdx.x; idx < (long)N * P; idx += blockDim.x) {
    const long j = idx / P;
    const int p = (int)(idx - j * P);
    s += w[j * P + p] * (norm2(X[j * 2 * P + p]) + norm2(X[j * 2 * P + P + p]));
  }
  for(int j = threadIdx.x; j < N; j += blockDim.x) {
    zd sum = mk(0.0, 0.0);
    for(int k = 0; k < P; ++k)
      sum = sum + acs[(size_t)j * P + k];
    a += ((2.0 * eta) * 0.5 * shs[j].sigma * sum).re;
  }
  red[0][threadIdx.x] = s;
  red[1][threadIdx.x] = a;
  __syncthreads();
  for(int st = blockDim.x / 2; st > 0; st >>= 1) {
    if(threadIdx.x < st) {
      red[0][threadIdx.x] += red[0][threadIdx.x + st];
      red[1][threadIdx.x] += red[1][threadIdx.x + st];
    }
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    out[0] = (1.0 / (4.0 * arbcf)) * red[0][0];
    out[1] = red[1][0];
  }
}

struct ShFieldArgs {
  const double *xyz;     // points, Cartesian (after the reader's spherical round trip)
  int npts;
  const double *cart;    // sphere centres
  const double *radius;
  int N, nmax;
  const zd *Xsh, *Xish;  // SH scattered / internal coefficients
  const zd *Xint;        // FF internal coefficients (particular solution)
  const ShScalars *shs;
  const double *tab;     // the nine SH coupling tables
  zd k2b;                // 2 waveK (background, second harmonic)
  zd iZw;                // iZ waveK_0 (background)
  zd w0;                 // waveK_0
  const zd *k_in;        // per sphere: 2 waveK_0 sqrt(eps_r_SH mu_r_SH)
  const zd *iZw_in;      // per sphere: -i / sqrt(mu_SH / eps_SH) waveK_0
  int *inner;            // per point: index of the sphere holding it, or -1
  zd *E, *H;
};

// Result::getEHFields, second-harmonic half (Result.cpp:166-199 outside,
// 237-276 inside), without the particular solution (k_near_field_sh_gamma).
// Same structure as the fundamental field kernel (vswf_point).
template <int NM>
__global__ void k_near_field_sh(ShFieldArgs a) {
  extern __shared__ double fsm[];
  WigTab &T = *reinterpret_cast<WigTab *>(fsm);
  zd *zs = reinterpret_cast<zd *>(fsm + sizeof(WigTab) / sizeof(double)) + threadIdx.x;
  const int zst = blockDim.x;
  wigtab_fill(T);
  __syncthreads();
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
  zd el[3], hl[3];
  if(inner < 0) {
    for(int j = 0; j < a.N; ++j) {
      double r, t, p;
      to_spherical(px - a.cart[3 * j], py - a.cart[3 * j + 1], pz - a.cart[3 * j + 2], &r, &t, &p);
      const zd *c = a.Xsh + (size_t)j * 2 * P;
      vswf_point<NM>(T, zs, zst, r, t, p, a.k2b, 0, a.nmax, c, c + P, el, hl);
      project_add(t, p, el, a.w0, E);
      project_add(t, p, hl, a.iZw, H);
    }
  } else {
    double r, t, p;
    to_spherical(px - a.cart[3 * inner], py - a.cart[3 * inner + 1], pz - a.cart[3 * inner + 2],
                 &r, &t, &p);
    const zd *c = a.Xish + (size_t)inner * 2 * P;
    vswf_point<NM>(T, zs, zst, r, t, p, a.k_in[inner], 1, a.nmax, c, c + P, el, hl);
    project_add(t, p, el, a.w0, E);
    project_add(t, p, hl, a.iZw_in[inner], H);
  }
  a.inner[i] = inner;
  for(int q = 0; q < 3; ++q) {
    a.E[3 * (size_t)i + q] = E[q];
    a.H[3 * (size_t)i + q] = H[q];
  }
}

template <int NM> void launch_nf_sh(const ShFieldArgs &a, cudaStream_t st) {
  const int threads = NM <= 8 ? 128 : 64;
  const size_t smem = sizeof(WigTab) + 3 * (NM + 1) * threads * sizeof(zd);
  cudaFuncSetAttribute(k_near_field_sh<NM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_near_field_sh<NM><<<blocks_for(a.npts, threads), threads, smem, st>>>(a);
}

// The particular solution inside spheres with a bulk chi(2) (gamma != 0):
// E_SH += sum_k (Xm_k CXm1_k + Xp_k CXp1_k) (Result.cpp:260-262 with
// Result::setFields / Geometry::COEFFpartSH, Result.cpp:906-919,
// Geometry.cpp:458-491; Xm, Xp: AuxCoefficients.cpp:134-176). One CTA per
// point; points outside every such sphere return at once.
__global__ void __launch_bounds__(128) k_near_field_sh_gamma(ShFieldArgs a) {
  const int i = blockIdx.x;
  const int j = a.inner[i];
  if(j < 0 || !a.shs[j].has_gamma)
    return;
  const int P = pmax(a.nmax), nmax = a.nmax;
  __shared__ zd d[kMaxNmax + 2], dd[kMaxNmax + 2], ddd[kMaxNmax + 2];
  __shared__ zd red[3][128];
  double r, t, ph;
  to_spherical(a.xyz[3 * i] - a.cart[3 * j], a.xyz[3 * i + 1] - a.cart[3 * j + 1],
               a.xyz[3 * i + 2] - a.cart[3 * j + 2], &r, &t, &ph);
  const ShScalars c = a.shs[j];
  if(threadIdx.x == 0)
    bessel_j012(r * c.k1, nmax, d, dd, ddd);
  __syncthreads();
  zd acc[3] = {mk(0, 0), mk(0, 0), mk(0, 0)};
  const bool pole = fabs(t) < 1e-10 || (fabs(t) - kPi + 1e-10) > 0.0;
  const double inv_trig = pole ? 1.0 / cos(t) : 1.0 / sin(t);
  for(int k = threadIdx.x; k < P; k += blockDim.x) {
    int J, M;
    nm_of(k, J, M);
    zd cxm, cxp;
    cx_sums(k, J, M, nmax, a.Xint + (size_t)j * 2 * P, a.tab, d, dd, ddd, c.k1, r, c.c_bulk, cxm,
            cxp);
    double W[kMaxNmax + 1], dW[kMaxNmax + 1];
    vigdvig(nmax, M, t, W, dW);
    const double A = (M == 0) ? 0.0 : (pole ? M * inv_trig * dW[J] : M * inv_trig * W[J]);
    const double dn = sqrt((2.0 * J + 1.0) / (4.0 * kPi * (double)(J * (J + 1))));
    double sn, cs;
    sincos(M * ph, &sn, &cs);
    const zd cb = (((M & 1) ? -1.0 : 1.0) * dn) * mk(cs, sn);
    const zd cx = sqrt((double)(J * (J + 1))) * cb;
    // Xm = cx (W, 0, 0), Xp = cb (0, dW, iA), in local spherical components
    const zd xm[3] = {cx * W[J], mk(0, 0), mk(0, 0)};
    const zd cbA = cb * A;
    const zd xp[3] = {mk(0, 0), cb * dW[J], mk(-cbA.im, cbA.re)};
    project_add(t, ph, xm, cxm, acc);
    project_add(t, ph, xp, cxp, acc);
  }
  for(int q = 0; q < 3; ++q)
    red[q][threadIdx.x] = acc[q];
  __syncthreads();
  if(threadIdx.x < 3) {
    zd s = mk(0, 0);
    for(int u = 0; u < (int)blockDim.x; ++u)
      s = s + red[threadIdx.x][u];
    a.E[3 * (size_t)i + threadIdx.x] = a.E[3 * (size_t)i + threadIdx.x] + s;
  }
}

}  // namespace

const double *clg_tables_dev(om_context *ctx, int nmax) {
  if(ctx->parent) {
    bool cached = false;
    for(auto &t : ctx->parent->clg)
      cached |= t.first == nmax;
    const double *d = clg_tables_dev(ctx->parent, nmax);
    if(!cached)  // built on the parent's stream: finish before this context uses it
      cudaStreamSynchronize(ctx->parent->stream);
    return d;
  }
  for(auto &t : ctx->clg)
    if(t.first == nmax)
      return t.second;
  const size_t P = pmax(nmax), count = 9 * P * P * P;
  double *d = nullptr;
  if(ctx->budget && ctx->used + count * sizeof(double) > ctx->budget)
    throw std::runtime_error("device-memory budget exceeded by the SH coupling tables");
  if(cudaMalloc(&d, count * sizeof(double)) != cudaSuccess)
    throw std::runtime_error("cudaMalloc failed for the SH coupling tables");
  ctx->used += count * sizeof(double);
  cudaMemsetAsync(d, 0, count * sizeof(double), ctx->stream);
  k_clg_tables<<<(unsigned)P, 256, 0, ctx->stream>>>(nmax, d);
  ctx->last_launches++;
  ctx->clg.push_back({nmax, d});
  return d;
}

// The compact form of the SH coupling tables for nmax (cached per context;
// a context with a parent uses the parent's, finished before it returns).
const ClgCompact &clg_compact_dev(om_context *ctx, int nmax) {
  if(ctx->parent) {
    bool cached = false;
    for(auto &t : ctx->parent->clgc)
      cached |= t.nmax == nmax;
    const ClgCompact &c = clg_compact_dev(ctx->parent, nmax);
    if(!cached)
      cudaStreamSynchronize(ctx->parent->stream);
    return c;
  }
  for(auto &t : ctx->clgc)
    if(t.nmax == nmax)
      return t;
  const double *tab = clg_tables_dev(ctx, nmax);
  const int P = pmax(nmax);
  std::vector<int> off(P + 1, 0), kof;
  std::vector<int2> pq;
  for(int k = 0; k < P; ++k) {
    int J, M;
    nm_of(k, J, M);
    off[k] = (int)pq.size();
    for(int p = 0; p < P; ++p) {
      int n1, m1;
      nm_of(p, n1, m1);
      const int m2 = M - m1;
      if(m2 < -nmax || m2 > nmax)
        continue;
      for(int n2 = std::max(1, std::abs(m2)); n2 <= nmax; ++n2) {
        pq.push_back(make_int2(p, flat(n2, m2)));
        kof.push_back(k);
      }
    }
  }
  off[P] = (int)pq.size();
  ClgCompact c;
  c.nmax = nmax;
  c.count = (long)pq.size();
  int *d_kof = nullptr;
  if(cudaMalloc(&c.off, sizeof(int) * (P + 1)) != cudaSuccess ||
     cudaMalloc(&c.pq, sizeof(int2) * pq.size()) != cudaSuccess ||
     cudaMalloc(&c.val, sizeof(double) * 9 * pq.size()) != cudaSuccess ||
     cudaMalloc(&d_kof, sizeof(int) * kof.size()) != cudaSuccess)
    throw std::runtime_error("cudaMalloc failed for the compact SH coupling tables");
  cudaMemcpy(c.off, off.data(), sizeof(int) * (P + 1), cudaMemcpyHostToDevice);
  cudaMemcpy(c.pq, pq.data(), sizeof(int2) * pq.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(d_kof, kof.data(), sizeof(int) * kof.size(), cudaMemcpyHostToDevice);
  k_clg_compact<<<blocks_for(c.count, 256), 256, 0, ctx->stream>>>(tab, P, c.pq, d_kof, c.count, c.val);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(d_kof);
  ctx->last_launches++;
  ctx->clgc.push_back(c);
  return ctx->clgc.back();
}

void launch_sh_source(om_problem *pr) {
  om_context *ctx = pr->ctx;
  const ClgCompact c = clg_compact_dev(ctx, pr->nmax);
  const int P = pr->P;
  k_sh_vectors<<<pr->N, 128, 0, ctx->stream>>>(pr->d_shs, pr->d_Xint, pr->nmax, pr->d_shvec);
  k_sh_source<<<pr->N, 256, 3 * P * sizeof(zd), ctx->stream>>>(pr->d_shs, pr->d_shvec, c.off, c.pq,
                                                               c.val, c.count, pr->d_shf, pr->nmax,
                                                               pr->d_K, pr->d_K1);
  ctx->last_launches += 2;
}

void launch_sh_internal(om_problem *pr) {
  k_sh_internal<<<blocks_for(pr->n, 256), 256, 0, pr->ctx->stream>>>(
      pr->d_Xsh, pr->d_K1, pr->d_shf, pr->nmax, pr->n, pr->d_Xish);
  pr->ctx->last_launches++;
}

void launch_sh_cross_sections(om_problem *pr, double *d_out2) {
  om_context *ctx = pr->ctx;
  const double *tab = clg_tables_dev(ctx, pr->nmax);
  launch_sh_weights(pr);
  k_sh_abs<<<pr->N, 256, 0, ctx->stream>>>(pr->d_shs, pr->d_Xint, pr->d_Xish, tab, pr->nmax,
                                           pr->omega, pr->d_acs);
  const double arbcf = pr->bg_eps_r.real() * pr->bg_mu_r.real();
  k_sh_xsec<<<1, 256, 0, ctx->stream>>>(pr->d_shs, pr->d_Xsh, pr->d_wsh, pr->d_acs, pr->N, pr->nmax,
                                        arbcf, mk(pr->eta.real(), pr->eta.imag()), d_out2);
  ctx->last_launches += 2;
}

void launch_near_field_sh(om_problem *pr, const double *d_xyz, int npts, cplx w0, const zd *d_kin,
                          const zd *d_izw, int *d_inner, zd *d_E, zd *d_H) {
  om_context *ctx = pr->ctx;
  ShFieldArgs a;
  a.xyz = d_xyz;
  a.npts = npts;
  a.cart = pr->d_cart;
  a.radius = pr->d_radius;
  a.N = pr->N;
  a.nmax = pr->nmax;
  a.Xsh = pr->d_Xsh;
  a.Xish = pr->d_Xish;
  a.Xint = pr->d_Xint;
  a.shs = pr->d_shs;
  a.tab = nullptr;
  const cplx k2b = cplx(2.0, 0.0) * pr->waveK, iZw = pr->iZ * w0;
  a.k2b = mk(k2b.real(), k2b.imag());
  a.iZw = mk(iZw.real(), iZw.imag());
  a.w0 = mk(w0.real(), w0.imag());
  a.k_in = d_kin;
  a.iZw_in = d_izw;
  a.inner = d_inner;
  a.E = d_E;
  a.H = d_H;
  if(a.nmax <= 4)
    launch_nf_sh<4>(a, ctx->stream);
  else if(a.nmax <= 8)
    launch_nf_sh<8>(a, ctx->stream);
  else if(a.nmax <= 12)
    launch_nf_sh<12>(a, ctx->stream);
  else
    launch_nf_sh<15>(a, ctx->stream);
  ctx->last_launches++;
  bool gamma = false;
  for(const auto &g : pr->gamma)
    gamma = gamma || g != cplx(0.0, 0.0);
  if(gamma) {
    a.tab = clg_tables_dev(ctx, pr->nmax);
    k_near_field_sh_gamma<<<npts, 128, 0, ctx->stream>>>(a);
    ctx->last_launches++;
  }
}

}  // namespace om
