// Post-processing of the OPTIMET sphere path on the device: internal
// coefficients, the four cross sections and the near-field summation.
#include "om_field.cuh"
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

// Result::getEHFields, fundamental frequency, Cartesian components
// (Result.cpp:74-301) with Geometry::checkInner (Geometry.cpp:147-163).
// One thread per point; the CTA shares the Wigner tables and holds each
// thread's radial factors (see vswf_point) in dynamic shared memory.
template <int NM>
__global__ void k_near_field(FieldArgs a) {
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
  const zd one = mk(1.0, 0.0);
  zd el[3], hl[3];
  if(inner < 0) {
    double r, t, p;
    to_spherical(px, py, pz, &r, &t, &p);
    vswf_point<NM>(T, zs, zst, r, t, p, a.waveK, 1, a.nmax, a.inc, a.inc + P, el, hl);
    zd Ei[3] = {mk(0, 0), mk(0, 0), mk(0, 0)}, Hi[3] = {mk(0, 0), mk(0, 0), mk(0, 0)};
    project_add(t, p, el, one, Ei);
    project_add(t, p, hl, a.iZ, Hi);
    for(int j = 0; j < a.N; ++j) {
      to_spherical(px - a.cart[3 * j], py - a.cart[3 * j + 1], pz - a.cart[3 * j + 2], &r, &t, &p);
      const zd *c = a.X + (size_t)j * 2 * P;
      vswf_point<NM>(T, zs, zst, r, t, p, a.waveK, 0, a.nmax, c, c + P, el, hl);
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
    vswf_point<NM>(T, zs, zst, r, t, p, a.k_in[inner], 1, a.nmax, c, c + P, el, hl);
    project_add(t, p, el, one, E);
    project_add(t, p, hl, a.iZ_in[inner], H);
  }
  for(int q = 0; q < 3; ++q) {
    a.E[3 * (size_t)i + q] = E[q];
    a.H[3 * (size_t)i + q] = H[q];
  }
}

template <int NM> void launch_nf(const FieldArgs &a, cudaStream_t st) {
  const int threads = NM <= 8 ? 128 : 64;
  const size_t smem = sizeof(WigTab) + 3 * (NM + 1) * threads * sizeof(zd);
  cudaFuncSetAttribute(k_near_field<NM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_near_field<NM><<<blocks_for(a.npts, threads), threads, smem, st>>>(a);
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
  if(a.nmax <= 4)
    launch_nf<4>(a, pr->ctx->stream);
  else if(a.nmax <= 8)
    launch_nf<8>(a, pr->ctx->stream);
  else if(a.nmax <= 12)
    launch_nf<12>(a, pr->ctx->stream);
  else
    launch_nf<15>(a, pr->ctx->stream);
  pr->ctx->last_launches++;
}

}  // namespace om
