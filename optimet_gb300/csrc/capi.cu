// C ABI of liboptimet_gpu: host-side model set-up (the Reader / Geometry /
// Excitation state of OPTIMET-3D), device-memory ownership and the call
// sequence of one wavelength-solve.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "om_internal.h"

using om::cplx;
using om::zd;

namespace {

// srcAna/constants.cpp:19-41
const double kPi = 3.14159265358979323846;
const double kC = 299792458;
const double kMu0 = 4.0 * kPi * 1e-7;
const double kEps0 = 1.0 / (kMu0 * kC * kC);

zd Z(cplx c) { return om::mk(c.real(), c.imag()); }

int cuda_fail(om_context *ctx, cudaError_t e, const char *what) {
  ctx->err = std::string(what) + ": " + cudaGetErrorString(e);
  return OM_ERR_CUDA;
}

int check_launch(om_context *ctx, const char *what) {
  cudaError_t e = cudaGetLastError();
  if(e != cudaSuccess)
    return cuda_fail(ctx, e, what);
  return OM_OK;
}

template <typename T> int dev_alloc(om_context *ctx, T **p, size_t count) {
  return om::dev_malloc(ctx, (void **)p, std::max<size_t>(count, 1) * sizeof(T));
}

template <typename T> void dev_free(om_context *ctx, T *&p, size_t count) {
  om::dev_release(ctx, p, std::max<size_t>(count, 1) * sizeof(T));
  p = nullptr;
}

void to_sph(double x, double y, double z, double *o) { om::to_spherical(x, y, z, o, o + 1, o + 2); }

// The per-wavelength scalars: Excitation (Excitation.cpp:31-45,132-137),
// per-sphere wave numbers (Scatterer.cpp:39-161, Result.cpp:206-213).
int update_wave(om_problem *pr) {
  om_context *ctx = pr->ctx;
  const cplx eps_b = pr->bg_eps_r * kEps0, mu_b = pr->bg_mu_r * kMu0;
  const double k0 = 2 * kPi / pr->lambda;  // vKInc.rrr
  pr->waveK = k0 * std::sqrt(pr->bg_eps_r * pr->bg_mu_r);
  pr->omega = kC * k0;
  pr->iZ = cplx(0.0, -1.0) / std::sqrt(mu_b / eps_b);
  const double w = pr->omega;
  const cplx waveK_0 = w * std::sqrt(kEps0 * kMu0);
  // the previous upload from these buffers must be done before they change
  if(!pr->h_scal.empty())
    cudaStreamSynchronize(ctx->stream);
  std::vector<om::SphereScalars> &sc = pr->h_scal;
  std::vector<om::ShScalars> &shs = pr->h_shs;
  std::vector<zd> &kin = pr->h_kin, &izin = pr->h_izin;
  sc.assign(pr->N, om::SphereScalars{});
  shs.assign(pr->N, om::ShScalars{});
  kin.assign(pr->N, zd{});
  izin.assign(pr->N, zd{});
  pr->eta = std::sqrt(mu_b / eps_b);
  for(int i = 0; i < pr->N; ++i) {
    const cplx eps_s = pr->eps_r[i] * kEps0, mu_s = pr->mu_r[i] * kMu0;
    const cplx eps_sh = pr->eps_r_sh[i] * kEps0;
    const cplx k_s = w * std::sqrt(eps_s * mu_s);
    const cplx k_b = w * std::sqrt(eps_b * mu_b);
    const cplx k_s2 = 2.0 * w * std::sqrt(eps_sh * mu_s);
    const cplx k_b2 = 2.0 * w * std::sqrt(eps_b * mu_b);
    om::SphereScalars &s = sc[i];
    s.rho = Z(k_s / k_b);
    s.r0 = Z(k_b * pr->radius[i]);
    s.mu_sob = Z(mu_s / mu_b);
    s.mu_j = Z(mu_s);
    s.mu_0 = Z(mu_b);
    s.rho_sh = Z(k_s2 / k_b2);
    s.r0_sh = Z(k_b2 * pr->radius[i]);
    s.mu_sob_sh = Z(mu_s / mu_b);
    // SH outer / internal factors (Scatterer.cpp:163-412)
    s.x_b2 = Z(k_b2 * pr->radius[i]);
    s.x_i2 = Z(k_s2 * pr->radius[i]);
    s.zeta = Z(std::sqrt(mu_b / eps_b) / std::sqrt(mu_s / eps_sh));
    // SH source and absorption scalars (Symbol.cpp:155-477)
    om::ShScalars &h = shs[i];
    const cplx mu_0 = kMu0, eps_0 = kEps0;
    const cplx imp = std::sqrt(mu_b / eps_b) / std::sqrt(mu_0 / eps_0);
    const cplx waveK_01 = w * std::sqrt(eps_0 * mu_0);
    const double R = pr->radius[i];
    h.k1 = Z(w * std::sqrt(eps_s * mu_s));
    h.kSH = Z(2.0 * w * std::sqrt(eps_sh * mu_s));
    h.c_up = Z(cplx(2.0, 0.0) * cplx(0.0, 1.0) * pr->ksiparppar[i] * imp);
    h.c_vp = Z(cplx(2.0, 0.0) * pr->ksiparppar[i] * imp);
    h.c_g1 = Z(cplx(0.0, 1.0) * pr->ksippp[i] / waveK_01 / R);
    h.c_g2 = Z(cplx(0.0, 1.0) * pr->gamma[i] * (eps_0 / eps_sh) / waveK_01 / R);
    h.c_bulk = Z((-eps_0 / eps_sh) * pr->gamma[i]);
    h.sigma = Z(-cplx(0.0, 1.0) * kEps0 * 2.0 * w * (pr->eps_r_sh[i] - 1.0));
    h.w01 = Z(waveK_01);
    h.R = R;
    h.has_gamma = pr->gamma[i] != cplx(0.0, 0.0);
    kin[i] = Z(waveK_0 * std::sqrt(pr->eps_r[i] * pr->mu_r[i]));
    izin[i] = Z(cplx(0.0, -1.0) / std::sqrt(mu_s / eps_s));
  }
  cudaMemcpyAsync(pr->d_scal, sc.data(), sizeof(om::SphereScalars) * pr->N, cudaMemcpyHostToDevice,
                  ctx->stream);
  cudaMemcpyAsync(pr->d_kin, kin.data(), sizeof(zd) * pr->N, cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(pr->d_shs, shs.data(), sizeof(om::ShScalars) * pr->N, cudaMemcpyHostToDevice,
                  ctx->stream);
  cudaMemcpyAsync(pr->d_izin, izin.data(), sizeof(zd) * pr->N, cudaMemcpyHostToDevice, ctx->stream);
  om::launch_sphere_terms(pr);
  // Einc = toProjection((0, theta, phi), (0, E_theta, E_phi)) (Reader.cpp:815-827)
  const double st = std::sin(pr->theta), ct = std::cos(pr->theta), sp = std::sin(pr->phi),
               cp = std::cos(pr->phi);
  const cplx Et = pr->e_theta, Ep = pr->e_phi;
  const cplx ex = ct * cp * Et - sp * Ep, ey = ct * sp * Et + cp * Ep, ez = -st * Et;
  double *einc = pr->h_einc;
  einc[0] = ex.real();
  einc[1] = ex.imag();
  einc[2] = ey.real();
  einc[3] = ey.imag();
  einc[4] = ez.real();
  einc[5] = ez.imag();
  om::launch_incident(pr, einc);
  pr->have_source = false;
  pr->have_solution = false;
  pr->have_sh = false;
  pr->S_prec[0] = pr->S_prec[1] = -1;
  return check_launch(ctx, "per-sphere / incident kernels");
}

void free_problem(om_problem *pr) {
  om_context *ctx = pr->ctx;
  const size_t N = pr->N, P = pr->P, n = pr->n, nm = 2 * (pr->nmax + 1);
  dev_free(ctx, pr->d_cart, 3 * N);
  dev_free(ctx, pr->d_radius, N);
  dev_free(ctx, pr->d_kin, N);
  dev_free(ctx, pr->d_izin, N);
  dev_free(ctx, pr->d_scal, N);
  dev_free(ctx, pr->d_T, N * nm);
  dev_free(ctx, pr->d_Tsh, N * nm);
  dev_free(ctx, pr->d_iaux, N * nm);
  dev_free(ctx, pr->d_cabs, N * nm);
  dev_free(ctx, pr->d_inc, 2 * P);
  dev_free(ctx, pr->d_incloc, n);
  dev_free(ctx, pr->d_wsca, N * P);
  dev_free(ctx, pr->d_Q, n);
  dev_free(ctx, pr->d_X, n);
  dev_free(ctx, pr->d_Xint, n);
  dev_free(ctx, pr->d_xsec, 16);
  dev_free(ctx, pr->d_shs, N);
  dev_free(ctx, pr->d_shf, N * (nm / 2) * 8);
  dev_free(ctx, pr->d_shvec, 3 * N * P);
  dev_free(ctx, pr->d_K, n);
  dev_free(ctx, pr->d_K1, n);
  dev_free(ctx, pr->d_Xsh, n);
  dev_free(ctx, pr->d_Xish, n);
  if(pr->d_Srows)
    om::dev_release(ctx, pr->d_Srows, pr->rows_bytes);
  pr->d_Srows = nullptr;
  dev_free(ctx, pr->d_wsh, N * P);
  dev_free(ctx, pr->d_acs, N * P);
  for(int h = 0; h < 2; ++h) {
    om::dev_release(ctx, pr->d_S[h], sizeof(double2) * n * n);
    pr->d_S[h] = nullptr;
    om::dev_release(ctx, pr->d_S32[h], sizeof(float2) * n * n);
    pr->d_S32[h] = nullptr;
  }
  om::aca_free(pr);
}

int make_problem(om_context *ctx, const om_sphere *spheres, int n_spheres, const om_medium *bg,
                 const om_plane_wave *wave, om_problem **out) {
  if(!ctx || !out)
    return OM_ERR_INVALID;
  *out = nullptr;
  if(!spheres || n_spheres < 1 || !wave) {
    ctx->err = "need at least one sphere and a plane wave";
    return OM_ERR_INVALID;
  }
  const int nmax = spheres[0].nmax;
  for(int i = 0; i < n_spheres; ++i)
    if(spheres[i].nmax != nmax) {
      ctx->err = "All objects must have same number of harmonics";
      return OM_ERR_INVALID;
    }
  if(nmax < 1 || nmax > om::kMaxNmax) {
    ctx->err = "nmax must be in [1, " + std::to_string(om::kMaxNmax) + "]";
    return OM_ERR_INVALID;
  }
  if(!(wave->wavelength > 0)) {
    ctx->err = "wavelength must be positive";
    return OM_ERR_INVALID;
  }
  om_problem *pr = new(std::nothrow) om_problem();
  if(!pr)
    return OM_ERR_INVALID;
  pr->ctx = ctx;
  pr->N = n_spheres;
  pr->nmax = nmax;
  pr->P = om::pmax(nmax);
  pr->n = 2L * pr->P * n_spheres;
  for(int i = 0; i < n_spheres; ++i) {
    const om_sphere &s = spheres[i];
    if(!(s.radius > 0)) {
      ctx->err = "sphere " + std::to_string(i) + " has no positive radius";
      delete pr;
      return OM_ERR_INVALID;
    }
    double sp[3];
    to_sph(s.x, s.y, s.z, sp);
    // Geometry::pushObject (Geometry.cpp:39-51)
    for(int j = 0; j < i; ++j) {
      double a[3], b[3];
      om::to_cartesian(pr->sph[3 * j], pr->sph[3 * j + 1], pr->sph[3 * j + 2], a, a + 1, a + 2);
      om::to_cartesian(sp[0], sp[1], sp[2], b, b + 1, b + 2);
      double d = std::sqrt(std::pow(b[0] - a[0], 2.0) + std::pow(b[1] - a[1], 2.0) +
                           std::pow(b[2] - a[2], 2.0));
      if(d <= s.radius + pr->radius[j]) {
        ctx->err = "The sphere at index " + std::to_string(i) + " overlaps with the one at index " +
                   std::to_string(j);
        delete pr;
        return OM_ERR_OVERLAP;
      }
    }
    pr->sph.insert(pr->sph.end(), sp, sp + 3);
    double c[3];
    om::to_cartesian(sp[0], sp[1], sp[2], c, c + 1, c + 2);
    pr->cart.insert(pr->cart.end(), c, c + 3);
    pr->radius.push_back(s.radius);
    pr->eps_r.push_back(cplx(s.eps_r[0], s.eps_r[1]));
    pr->mu_r.push_back(cplx(s.mu_r[0], s.mu_r[1]));
    pr->eps_r_sh.push_back(cplx(s.eps_r_sh[0], s.eps_r_sh[1]));
    pr->ksippp.push_back(cplx(s.ksippp[0], s.ksippp[1]));
    pr->ksiparppar.push_back(cplx(s.ksiparppar[0], s.ksiparppar[1]));
    pr->gamma.push_back(cplx(s.gamma[0], s.gamma[1]));
  }
  pr->bg_eps_r = bg ? cplx(bg->eps_r[0], bg->eps_r[1]) : cplx(1.0, 0.0);
  pr->bg_mu_r = bg ? cplx(bg->mu_r[0], bg->mu_r[1]) : cplx(1.0, 0.0);
  pr->lambda = wave->wavelength;
  pr->theta = wave->theta;
  pr->phi = wave->phi;
  pr->e_theta = cplx(wave->e_theta[0], wave->e_theta[1]);
  pr->e_phi = cplx(wave->e_phi[0], wave->e_phi[1]);
  pr->sh = wave->sh;
  const size_t N = pr->N, P = pr->P, n = pr->n, nm = 2 * (nmax + 1);
  int rc = OM_OK;
  if(!rc) rc = dev_alloc(ctx, &pr->d_cart, 3 * N);
  if(!rc) rc = dev_alloc(ctx, &pr->d_radius, N);
  if(!rc) rc = dev_alloc(ctx, &pr->d_kin, N);
  if(!rc) rc = dev_alloc(ctx, &pr->d_izin, N);
  if(!rc) rc = dev_alloc(ctx, &pr->d_scal, N);
  if(!rc) rc = dev_alloc(ctx, &pr->d_T, N * nm);
  if(!rc) rc = dev_alloc(ctx, &pr->d_Tsh, N * nm);
  if(!rc) rc = dev_alloc(ctx, &pr->d_iaux, N * nm);
  if(!rc) rc = dev_alloc(ctx, &pr->d_cabs, N * nm);
  if(!rc) rc = dev_alloc(ctx, &pr->d_inc, 2 * P);
  if(!rc) rc = dev_alloc(ctx, &pr->d_incloc, n);
  if(!rc) rc = dev_alloc(ctx, &pr->d_wsca, N * P);
  if(!rc) rc = dev_alloc(ctx, &pr->d_Q, n);
  if(!rc) rc = dev_alloc(ctx, &pr->d_X, n);
  if(!rc) rc = dev_alloc(ctx, &pr->d_Xint, n);
  if(!rc) rc = dev_alloc(ctx, &pr->d_xsec, 16);
  if(!rc) rc = dev_alloc(ctx, &pr->d_shs, N);
  if(!rc) rc = dev_alloc(ctx, &pr->d_shf, N * (nm / 2) * 8);
  if(rc) {
    free_problem(pr);
    delete pr;
    return rc;
  }
  cudaMemcpyAsync(pr->d_cart, pr->cart.data(), sizeof(double) * 3 * N, cudaMemcpyHostToDevice,
                  ctx->stream);
  cudaMemcpyAsync(pr->d_radius, pr->radius.data(), sizeof(double) * N, cudaMemcpyHostToDevice,
                  ctx->stream);
  rc = update_wave(pr);
  if(rc) {
    free_problem(pr);
    delete pr;
    return rc;
  }
  *out = pr;
  return OM_OK;
}

// The plain form keeps the complex128 matrix, the precision form only the
// complex64 one (its refinement works on that system; the cross sections of
// the rounded system differ from FP64 by ~1e-9, far inside the 1e-6 target).
int ensure_matrix(om_problem *pr, int harmonic, int precision) {
  om_context *ctx = pr->ctx;
  const size_t nn = (size_t)pr->n * pr->n;
  if(precision == OM_C128 && !pr->d_S[harmonic]) {
    double2 *p = nullptr;
    int rc = dev_alloc(ctx, &p, nn);
    if(rc)
      return rc;
    pr->d_S[harmonic] = p;
  }
  if(precision == OM_C64 && !pr->d_S32[harmonic]) {
    float2 *p = nullptr;
    int rc = dev_alloc(ctx, &p, nn);
    if(rc)
      return rc;
    pr->d_S32[harmonic] = p;
  }
  return OM_OK;
}

}  // namespace

namespace om {
// Device memory is stream-ordered (cudaMallocAsync / cudaFreeAsync on the
// context's stream, from the device's default pool): a release never waits
// for other streams, so contexts that run side by side on one device (the
// serving slots) do not serialise each other through allocation.
int dev_malloc(om_context *ctx, void **p, size_t bytes) {
  *p = nullptr;
  if(ctx->budget && ctx->used + bytes > ctx->budget) {
    ctx->err = "device-memory budget exceeded (" + std::to_string(ctx->used + bytes) + " > " +
               std::to_string(ctx->budget) + " bytes)";
    return OM_ERR_BUDGET;
  }
  cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
  if(e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    ctx->err = std::string("cudaMallocAsync(") + std::to_string(bytes) +
               " bytes): " + cudaGetErrorString(e);
    return OM_ERR_BUDGET;
  }
  ctx->used += bytes;
  return OM_OK;
}

void dev_release(om_context *ctx, void *p, size_t bytes) {
  if(!p)
    return;
  cudaFreeAsync(p, ctx->stream);
  ctx->used -= bytes;
}

// Drop one harmonic's matrix storage (the server frees the FF matrix before
// the SH assembly).
void release_matrix(om_problem *pr, int harmonic) {
  const size_t nn = (size_t)pr->n * pr->n;
  dev_release(pr->ctx, pr->d_S[harmonic], sizeof(double2) * nn);
  pr->d_S[harmonic] = nullptr;
  dev_release(pr->ctx, pr->d_S32[harmonic], sizeof(float2) * nn);
  pr->d_S32[harmonic] = nullptr;
  pr->S_prec[harmonic] = -1;
}

int sh_alloc(om_problem *pr) {
  om_context *ctx = pr->ctx;
  const size_t N = pr->N, P = pr->P, n = pr->n;
  int rc = OM_OK;
  if(!rc && !pr->d_shvec) rc = dev_alloc(ctx, &pr->d_shvec, 3 * N * P);
  if(!rc && !pr->d_K) rc = dev_alloc(ctx, &pr->d_K, n);
  if(!rc && !pr->d_K1) rc = dev_alloc(ctx, &pr->d_K1, n);
  if(!rc && !pr->d_Xsh) rc = dev_alloc(ctx, &pr->d_Xsh, n);
  if(!rc && !pr->d_Xish) rc = dev_alloc(ctx, &pr->d_Xish, n);
  if(!rc && !pr->d_wsh) rc = dev_alloc(ctx, &pr->d_wsh, N * P);
  if(!rc && !pr->d_acs) rc = dev_alloc(ctx, &pr->d_acs, N * P);
  return rc;
}

void collect_timers(om_context *ctx) {
  auto fold = [](std::vector<std::pair<cudaEvent_t, cudaEvent_t>> &v, double &t, long &n) {
    for(auto &e : v) {
      float ms = 0;
      cudaEventSynchronize(e.second);
      cudaEventElapsedTime(&ms, e.first, e.second);
      t += ms;
      ++n;
      cudaEventDestroy(e.first);
      cudaEventDestroy(e.second);
    }
    v.clear();
  };
  fold(ctx->ev_mv64, ctx->t_mv64, ctx->n_mv64);
  fold(ctx->ev_mv32, ctx->t_mv32, ctx->n_mv32);
  fold(ctx->ev_asm, ctx->t_asm, ctx->n_asm);
  fold(ctx->ev_mvdf, ctx->t_mvdf, ctx->n_mvdf);
  fold(ctx->ev_mv16, ctx->t_mv16, ctx->n_mv16);
  fold(ctx->ev_mvcp, ctx->t_mvcp, ctx->n_mvcp);
  fold(ctx->ev_luf, ctx->t_luf, ctx->n_luf);
  fold(ctx->ev_lup, ctx->t_lup, ctx->n_lup);
  fold(ctx->ev_luu, ctx->t_luu, ctx->n_luu);
  fold(ctx->ev_lus, ctx->t_lus, ctx->n_lus);
}
}  // namespace om

extern "C" {

int om_context_mark(om_context *ctx, double *ms) {
  if(!ctx)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaEvent_t e;
  if(cudaEventCreate(&e) != cudaSuccess)
    return cuda_fail(ctx, cudaGetLastError(), "event");
  cudaEventRecord(e, ctx->stream);
  cudaError_t err = cudaEventSynchronize(e);
  if(err != cudaSuccess)
    return cuda_fail(ctx, err, "mark");
  float t = 0;
  if(ctx->mark) {
    cudaEventElapsedTime(&t, ctx->mark, e);
    cudaEventDestroy(ctx->mark);
  }
  ctx->mark = e;
  if(ms)
    *ms = t;
  return OM_OK;
}

int om_context_tune(om_context *ctx, const om_tuning *t) {
  if(!ctx || !t || t->matvec_ctas_per_sm > 64 || t->matvec_df_ctas_per_sm > 64 ||
     t->assemble_carveout > 100 || t->matvec_carveout > 100)
    return OM_ERR_INVALID;
  if(t->matvec_ctas_per_sm > 0)
    ctx->mv_ctas = t->matvec_ctas_per_sm;
  if(t->matvec_df_ctas_per_sm > 0)
    ctx->mv_ctas_df = t->matvec_df_ctas_per_sm;
  if(t->assemble_carveout >= 0)
    ctx->carve_asm = t->assemble_carveout;
  if(t->matvec_carveout >= 0)
    ctx->carve_mv = t->matvec_carveout;
  if(t->lu_tensor_cores >= 0)
    ctx->lu_tc = std::min(t->lu_tensor_cores, 3);
  if(t->matvec_tma >= 0)
    ctx->mv_tma = t->matvec_tma ? 1 : 0;
  if(t->assemble_rotation >= 0)
    ctx->asm_rot = t->assemble_rotation ? 1 : 0;
  if(t->lu_persistent > 0)
    ctx->lu_persist = std::min(t->lu_persistent, 3);
  if(t->batch_tiles >= 0)
    ctx->batch_tiles = std::min(t->batch_tiles, 8);
  if(t->batch_fused >= 0)
    ctx->batch_fused = std::min(t->batch_fused, 2);
  if(t->inner_half >= 0)
    ctx->inner_half = t->inner_half ? 1 : 0;
  return OM_OK;
}

int om_matvec_inner_c64(om_context *ctx, long n, const float *S, const float *x, float *y, int products) {
  if(!ctx || !S || !x || !y || n < 1 || products < 1)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  float2 *dS = nullptr, *dx = nullptr, *dy = nullptr;
  const size_t nn = (size_t)n * n;
  int rc = dev_alloc(ctx, &dS, nn);
  if(!rc) rc = dev_alloc(ctx, &dx, (size_t)n);
  if(!rc) rc = dev_alloc(ctx, &dy, (size_t)n);
  if(!rc) {
    cudaMemcpyAsync(dS, S, sizeof(float2) * nn, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(dx, x, sizeof(float2) * n, cudaMemcpyHostToDevice, ctx->stream);
    rc = om::inner_products(ctx, dS, n, dx, dy, products);
    if(!rc) {
      cudaMemcpyAsync(y, dy, sizeof(float2) * n, cudaMemcpyDeviceToHost, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if(e != cudaSuccess)
        rc = cuda_fail(ctx, e, "inner product");
    }
  }
  cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, dS, nn);
  dev_free(ctx, dx, (size_t)n);
  dev_free(ctx, dy, (size_t)n);
  return rc;
}

int om_cgemm_sub_c64(om_context *ctx, long m, long n, int k, const float *A, long lda,
                     const float *B, long ldb, float *C, long ldc) {
  if(!ctx || !A || !B || !C || m < 1 || n < 1 || k < 1 || lda < m || ldb < k || ldc < m)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  float2 *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int *derr = nullptr;
  unsigned char *dS = nullptr;
  const size_t na = (size_t)lda * k, nbb = (size_t)ldb * n, nc = (size_t)ldc * n;
  // operands split once, then streamed by bulk copies (the LU's path)
  const size_t ns = om::cgemm_sub_tc_split_bytes(m, n, k);
  int rc = dev_alloc(ctx, &dA, na);
  if(!rc) rc = dev_alloc(ctx, &dB, nbb);
  if(!rc) rc = dev_alloc(ctx, &dC, nc);
  if(!rc) rc = dev_alloc(ctx, &derr, 1);
  if(!rc) rc = dev_alloc(ctx, &dS, ns);
  if(!rc) {
    cudaMemcpyAsync(dA, A, sizeof(float2) * na, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(dB, B, sizeof(float2) * nbb, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(dC, C, sizeof(float2) * nc, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(derr, 0, sizeof(int), ctx->stream);
    om::launch_cgemm_sub_tc_split(ctx, dA, lda, dB, ldb, dC, ldc, m, n, k, dS, derr);
    rc = check_launch(ctx, "tensor-core update");
    int herr = 0;
    if(!rc) {
      cudaMemcpyAsync(C, dC, sizeof(float2) * nc, cudaMemcpyDeviceToHost, ctx->stream);
      cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if(e != cudaSuccess)
        rc = cuda_fail(ctx, e, "tensor-core update");
      else if(herr) {
        ctx->err = "tensor-core update timed out";
        rc = OM_ERR_CUDA;
      }
    }
  }
  cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, dA, na);
  dev_free(ctx, dB, nbb);
  dev_free(ctx, dC, nc);
  dev_free(ctx, derr, 1);
  if(dS)
    dev_free(ctx, dS, ns);
  return rc;
}

int om_context_timers(om_context *ctx, int enable, double *out) {
  if(!ctx)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  om::collect_timers(ctx);
  if(out) {
    out[0] = ctx->t_asm;
    out[1] = (double)ctx->n_asm;
    out[2] = ctx->t_mv64;
    out[3] = (double)ctx->n_mv64;
    out[4] = ctx->t_mv32;
    out[5] = (double)ctx->n_mv32;
    out[6] = ctx->t_mvdf;
    out[7] = (double)ctx->n_mvdf;
  }
  ctx->t_asm = ctx->t_mv64 = ctx->t_mv32 = ctx->t_mvdf = 0;
  ctx->n_asm = ctx->n_mv64 = ctx->n_mv32 = ctx->n_mvdf = 0;
  ctx->timing = enable != 0;
  return OM_OK;
}

int om_context_inner_timers(om_context *ctx, double *out) {
  if(!ctx)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  om::collect_timers(ctx);
  if(out) {
    out[0] = ctx->t_mv16;
    out[1] = (double)ctx->n_mv16;
    out[2] = ctx->t_mvcp;
    out[3] = (double)ctx->n_mvcp;
  }
  ctx->t_mv16 = ctx->t_mvcp = 0;
  ctx->n_mv16 = ctx->n_mvcp = 0;
  return OM_OK;
}

int om_context_lu_timers(om_context *ctx, double *out) {
  if(!ctx)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  om::collect_timers(ctx);
  if(out) {
    out[0] = ctx->t_luf;
    out[1] = (double)ctx->n_luf;
    out[2] = ctx->t_lup;
    out[3] = (double)ctx->n_lup;
    out[4] = ctx->t_luu;
    out[5] = (double)ctx->n_luu;
    out[6] = ctx->t_lus;
    out[7] = (double)ctx->n_lus;
  }
  ctx->t_luf = ctx->t_lup = ctx->t_luu = ctx->t_lus = 0;
  ctx->n_luf = ctx->n_lup = ctx->n_luu = ctx->n_lus = 0;
  return OM_OK;
}

int om_context_create(int device, size_t budget_bytes, om_context **out) {
  if(!out)
    return OM_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if(cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return OM_ERR_CUDA;
  }
  if(cudaSetDevice(device) != cudaSuccess)
    return OM_ERR_CUDA;
  om_context *ctx = new(std::nothrow) om_context();
  if(!ctx)
    return OM_ERR_INVALID;
  ctx->device = device;
  ctx->budget = budget_bytes;
  if(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    ctx->sm_count = 1;
  // the context's stream at the highest priority, the assembly stream at the
  // lowest: when contexts share the device, pending solve blocks are
  // dispatched ahead of pending assembly blocks
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  if(cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, hi) != cudaSuccess ||
     cudaStreamCreateWithPriority(&ctx->stream_lo, cudaStreamNonBlocking, lo) != cudaSuccess ||
     cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
     cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    if(ctx->stream) cudaStreamDestroy(ctx->stream);
    if(ctx->stream_lo) cudaStreamDestroy(ctx->stream_lo);
    delete ctx;
    return OM_ERR_CUDA;
  }
  if(cudaMalloc(&ctx->d_tile_counter, 256) == cudaSuccess) {
    ctx->d_tma_err = reinterpret_cast<int *>(ctx->d_tile_counter + 1);
    cudaMemset(ctx->d_tile_counter, 0, 256);
  } else {
    cudaGetLastError();
    cudaStreamDestroy(ctx->stream);
    cudaStreamDestroy(ctx->stream_lo);
    cudaEventDestroy(ctx->ev_fork);
    cudaEventDestroy(ctx->ev_join);
    delete ctx;
    return OM_ERR_CUDA;
  }
  // keep freed blocks in the default pool (process-local setting) so that
  // repeated solves reuse them instead of returning memory to the driver
  cudaMemPool_t pool;
  if(cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    unsigned long long keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cudaGetLastError();
  *out = ctx;
  return OM_OK;
}

void om_context_destroy(om_context *ctx) {
  if(!ctx)
    return;
  cudaSetDevice(ctx->device);
  om::batch_release(ctx);
  for(om_context *a : ctx->aux)
    om_context_destroy(a);
  ctx->aux.clear();
  cudaStreamSynchronize(ctx->stream);
  // problems still alive belong to the context and go with it
  while(!ctx->problems.empty())
    om_problem_destroy(ctx->problems.back());
  for(auto &t : ctx->tables) {
    cudaFree(t.rec);
    cudaFree(t.qf);
    cudaFree(t.pf);
    cudaFree(t.legc);
    cudaFree(t.rot_i);
    cudaFree(t.rot_d);
    cudaFree(t.rot_z);
  }
  for(auto &t : ctx->clg)
    cudaFree(t.second);
  for(auto &t : ctx->clgc) {
    cudaFree(t.off);
    cudaFree(t.pq);
    cudaFree(t.val);
  }
  if(ctx->mark)
    cudaEventDestroy(ctx->mark);
  cudaEventDestroy(ctx->ev_fork);
  cudaEventDestroy(ctx->ev_join);
  cudaFree(ctx->d_tile_counter);
  cudaStreamDestroy(ctx->stream_lo);
  cudaStreamDestroy(ctx->stream);
  // hand unused pool memory back (live allocations of other contexts stay)
  cudaMemPool_t pool;
  if(cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess)
    cudaMemPoolTrimTo(pool, 0);
  cudaGetLastError();
  delete ctx;
}

const char *om_context_last_error(const om_context *ctx) { return ctx ? ctx->err.c_str() : ""; }

int om_context_last_launches(const om_context *ctx) { return ctx ? ctx->last_launches : 0; }

int om_context_synchronize(om_context *ctx) {
  if(!ctx)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? OM_OK : cuda_fail(ctx, e, "synchronize");
}

int om_problem_create(om_context *ctx, const om_sphere *spheres, int n_spheres,
                      const om_medium *background, const om_plane_wave *wave, om_problem **out) {
  if(!ctx)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  try {
    int rc = make_problem(ctx, spheres, n_spheres, background, wave, out);
    if(rc == OM_OK)
      ctx->problems.push_back(*out);
    return rc;
  } catch(std::exception &e) {
    ctx->err = e.what();
    return OM_ERR_CUDA;
  }
}

void om_problem_destroy(om_problem *pr) {
  if(!pr)
    return;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_problem(pr);
  auto &v = ctx->problems;
  v.erase(std::remove(v.begin(), v.end(), pr), v.end());
  delete pr;
}

long om_problem_size(const om_problem *pr) { return pr ? pr->n : 0; }

int om_problem_set_wavelength(om_problem *pr, double wavelength) {
  if(!pr || !(wavelength > 0))
    return OM_ERR_INVALID;
  cudaSetDevice(pr->ctx->device);
  pr->ctx->last_launches = 0;
  pr->lambda = wavelength;
  return update_wave(pr);
}

int om_problem_set_wave(om_problem *pr, const om_plane_wave *wave) {
  if(!pr || !wave || !(wave->wavelength > 0))
    return OM_ERR_INVALID;
  cudaSetDevice(pr->ctx->device);
  pr->ctx->last_launches = 0;
  pr->lambda = wave->wavelength;
  pr->theta = wave->theta;
  pr->phi = wave->phi;
  pr->e_theta = cplx(wave->e_theta[0], wave->e_theta[1]);
  pr->e_phi = cplx(wave->e_phi[0], wave->e_phi[1]);
  pr->sh = wave->sh;
  return update_wave(pr);
}

int om_coupling(om_context *ctx, const double *rel_xyz, int count, double k_re, double k_im,
                int nmax, int regular, double *A, double *B) {
  if(!ctx || !rel_xyz || count < 1 || !A || !B || nmax < 1 || nmax > om::kMaxNmax)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  const size_t P = om::pmax(nmax);
  double *d_rel = nullptr;
  zd *d_A = nullptr, *d_B = nullptr;
  int rc = dev_alloc(ctx, &d_rel, 3 * (size_t)count);
  if(!rc) rc = dev_alloc(ctx, &d_A, P * P * count);
  if(!rc) rc = dev_alloc(ctx, &d_B, P * P * count);
  if(!rc) {
    // the reference takes a Spherical displacement; mirror its Cartesian round trip
    std::vector<double> rel(3 * (size_t)count);
    for(int e = 0; e < count; ++e) {
      double s[3];
      to_sph(rel_xyz[3 * e], rel_xyz[3 * e + 1], rel_xyz[3 * e + 2], s);
      om::to_cartesian(s[0], s[1], s[2], &rel[3 * e], &rel[3 * e + 1], &rel[3 * e + 2]);
    }
    cudaMemcpyAsync(d_rel, rel.data(), sizeof(double) * rel.size(), cudaMemcpyHostToDevice,
                    ctx->stream);
    try {
      om::launch_coupling(ctx, d_rel, count, om::mk(k_re, k_im), nmax, regular ? 1 : 0, d_A, d_B);
      rc = check_launch(ctx, "coupling kernel");
    } catch(std::exception &ex) {
      ctx->err = ex.what();
      rc = OM_ERR_CUDA;
    }
    if(!rc) {
      cudaMemcpyAsync(A, d_A, sizeof(zd) * P * P * count, cudaMemcpyDeviceToHost, ctx->stream);
      cudaMemcpyAsync(B, d_B, sizeof(zd) * P * P * count, cudaMemcpyDeviceToHost, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if(e != cudaSuccess)
        rc = cuda_fail(ctx, e, "coupling");
    }
  }
  dev_free(ctx, d_rel, 3 * (size_t)count);
  dev_free(ctx, d_A, P * P * count);
  dev_free(ctx, d_B, P * P * count);
  return rc;
}

int om_tmatrix(om_problem *pr, int harmonic, double *T) {
  if(!pr || !T || (harmonic != OM_FF && harmonic != OM_SH))
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  const int nm = 2 * (pr->nmax + 1);
  std::vector<zd> h((size_t)pr->N * nm);
  cudaMemcpyAsync(h.data(), harmonic == OM_SH ? pr->d_Tsh : pr->d_T, sizeof(zd) * h.size(),
                  cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if(e != cudaSuccess)
    return cuda_fail(ctx, e, "tmatrix");
  // expand to the reference's 2P diagonal (Scatterer.cpp:86-95)
  zd *out = reinterpret_cast<zd *>(T);
  for(int i = 0; i < pr->N; ++i)
    for(int p = 0; p < pr->P; ++p) {
      int n = (int)std::sqrt(p + 1.0);
      out[(size_t)i * 2 * pr->P + p] = h[(size_t)i * nm + 2 * n];
      out[(size_t)i * 2 * pr->P + pr->P + p] = h[(size_t)i * nm + 2 * n + 1];
    }
  return OM_OK;
}

int om_incident_coefficients(om_problem *pr, double *ab) {
  if(!pr || !ab)
    return OM_ERR_INVALID;
  cudaSetDevice(pr->ctx->device);
  cudaMemcpyAsync(ab, pr->d_inc, sizeof(zd) * 2 * pr->P, cudaMemcpyDeviceToHost, pr->ctx->stream);
  cudaError_t e = cudaStreamSynchronize(pr->ctx->stream);
  return e == cudaSuccess ? OM_OK : cuda_fail(pr->ctx, e, "incident coefficients");
}

int om_assemble(om_problem *pr, int harmonic, int precision) {
  if(!pr || (harmonic != OM_FF && harmonic != OM_SH) ||
     (precision != OM_C128 && precision != OM_C64 && precision != OM_ACA))
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  if(precision == OM_ACA) {
    int rc;
    try {
      rc = om::aca_build(pr, harmonic);
    } catch(std::exception &e) {
      ctx->err = e.what();
      rc = OM_ERR_CUDA;
    }
    if(!rc)
      rc = check_launch(ctx, "ACA compression");
    if(rc)
      return rc;
    pr->S_prec[harmonic] = OM_ACA;
    if(harmonic == OM_FF)
      pr->have_solution = false;
    return OM_OK;
  }
  int rc = ensure_matrix(pr, harmonic, precision);
  if(rc)
    return rc;
  try {
    om::launch_assemble(pr, harmonic, precision);
  } catch(std::exception &e) {
    ctx->err = e.what();
    return OM_ERR_CUDA;
  }
  rc = check_launch(ctx, "assembly kernel");
  if(rc)
    return rc;
  pr->S_prec[harmonic] = precision;
  if(harmonic == OM_FF)
    pr->have_solution = false;
  return OM_OK;
}

int om_aca_info(om_problem *pr, int harmonic, double *store_bytes, int *compressed, int *dense,
                double *mean_rank, int *max_rank) {
  if(!pr || (harmonic != OM_FF && harmonic != OM_SH))
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  if(pr->S_prec[harmonic] != OM_ACA) {
    ctx->err = "matrix not assembled with OM_ACA";
    return OM_ERR_STATE;
  }
  cudaSetDevice(ctx->device);
  const size_t NN = (size_t)pr->N * pr->N;
  std::vector<int> r(NN);
  cudaMemcpyAsync(r.data(), pr->aca[harmonic].rank, sizeof(int) * NN, cudaMemcpyDeviceToHost,
                  ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if(e != cudaSuccess)
    return cuda_fail(ctx, e, "ACA info");
  int nc = 0, nd = 0, mx = 0;
  double sum = 0.0;
  for(int v : r) {
    if(v == -1)
      ++nd;
    else if(v >= 0) {
      ++nc;
      sum += v;
      mx = std::max(mx, v);
    }
  }
  if(store_bytes) *store_bytes = (double)pr->aca[harmonic].used * sizeof(double2);
  if(compressed) *compressed = nc;
  if(dense) *dense = nd;
  if(mean_rank) *mean_rank = nc ? sum / nc : 0.0;
  if(max_rank) *max_rank = mx;
  return OM_OK;
}

int om_copy_matrix(om_problem *pr, int harmonic, double *S) {
  if(!pr || !S || (harmonic != OM_FF && harmonic != OM_SH))
    return OM_ERR_INVALID;
  if(pr->S_prec[harmonic] < 0 || pr->S_prec[harmonic] == OM_ACA) {
    pr->ctx->err = pr->S_prec[harmonic] < 0 ? "matrix not assembled"
                                             : "an ACA-compressed matrix has no dense copy";
    return OM_ERR_STATE;
  }
  cudaSetDevice(pr->ctx->device);
  const size_t nn = (size_t)pr->n * pr->n;
  if(pr->S_prec[harmonic] == OM_C128) {
    cudaMemcpyAsync(S, pr->d_S[harmonic], sizeof(double2) * nn, cudaMemcpyDeviceToHost,
                    pr->ctx->stream);
    cudaError_t e = cudaStreamSynchronize(pr->ctx->stream);
    return e == cudaSuccess ? OM_OK : cuda_fail(pr->ctx, e, "copy matrix");
  }
  // complex64 storage: widen on the host, in place from the back
  float *f = reinterpret_cast<float *>(S) + 2 * nn;  // second half of the buffer
  cudaMemcpyAsync(f, pr->d_S32[harmonic], sizeof(float2) * nn, cudaMemcpyDeviceToHost,
                  pr->ctx->stream);
  cudaError_t e = cudaStreamSynchronize(pr->ctx->stream);
  if(e != cudaSuccess)
    return cuda_fail(pr->ctx, e, "copy matrix");
  for(size_t i = 0; i < 2 * nn; ++i)
    S[i] = (double)f[i];
  return OM_OK;
}

int om_source_vector(om_problem *pr, double *Q) {
  if(!pr)
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  try {
    om::launch_source(pr);
  } catch(std::exception &e) {
    ctx->err = e.what();
    return OM_ERR_CUDA;
  }
  int rc = check_launch(ctx, "source kernel");
  if(rc)
    return rc;
  pr->have_source = true;
  if(Q) {
    cudaMemcpyAsync(Q, pr->d_Q, sizeof(zd) * pr->n, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if(e != cudaSuccess)
      return cuda_fail(ctx, e, "source vector");
  }
  return OM_OK;
}

static int solve_impl(om_problem *pr, int harmonic, const om_solve_options *o, const double2 *b,
                      double2 *x, om_solve_stats *st) {
  om_context *ctx = pr->ctx;
  if(pr->S_prec[harmonic] < 0) {
    ctx->err = "matrix not assembled";
    return OM_ERR_STATE;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, ctx->stream);
  int rc;
  switch(o->method) {
  case OM_SOLVE_LU:
    if(pr->S_prec[harmonic] != OM_C128) {
      ctx->err = "LU solve needs the matrix assembled with OM_C128";
      rc = OM_ERR_STATE;
    } else
      rc = om::solve_lu_rhs(pr, harmonic, b, x, st);
    break;
  case OM_SOLVE_GMRES:
    rc = om::solve_gmres_rhs(pr, harmonic, o, b, x, st);
    break;
  case OM_SOLVE_FGMRES_MIXED:
  case OM_SOLVE_LU_MIXED:
    if(pr->S_prec[harmonic] != OM_C64) {
      ctx->err = "mixed solves need the matrix assembled with OM_C64";
      rc = OM_ERR_STATE;
    } else if(o->method == OM_SOLVE_FGMRES_MIXED)
      rc = om::solve_fgmres_rhs(pr, harmonic, o, b, x, st);
    else
      rc = om::solve_lu_mixed_rhs(pr, harmonic, o, b, x, st);
    break;
  default:
    ctx->err = "unknown solve method";
    rc = OM_ERR_INVALID;
  }
  cudaEventRecord(e1, ctx->stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if(st)
    st->seconds = ms * 1e-3;
  if(!rc)
    rc = check_launch(ctx, "solve");
  // a TMA matvec whose bounded wait ran out leaves a flag
  int tma_err = 0;
  cudaMemcpyAsync(&tma_err, ctx->d_tma_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  if(tma_err) {
    cudaMemsetAsync(ctx->d_tma_err, 0, sizeof(int), ctx->stream);
    ctx->err = "a TMA matrix-vector product timed out";
    rc = OM_ERR_CUDA;
  }
  return rc;
}

int om_solve(om_problem *pr, const om_solve_options *opts, om_solve_stats *stats) {
  if(!pr || !opts)
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  if(!pr->have_source) {
    ctx->err = "source vector not computed";
    return OM_ERR_STATE;
  }
  om_solve_stats st{};
  int rc;
  try {
    rc = solve_impl(pr, OM_FF, opts, (const double2 *)pr->d_Q, (double2 *)pr->d_X, &st);
  } catch(std::exception &e) {
    ctx->err = e.what();
    rc = OM_ERR_CUDA;
  }
  if(stats)
    *stats = st;
  if(rc && rc != OM_ERR_NOT_CONVERGED)
    return rc;
  om::launch_internal(pr);
  int rc2 = check_launch(ctx, "internal coefficients");
  if(rc2)
    return rc2;
  pr->have_solution = true;
  return rc;
}

int om_solve_rhs(om_problem *pr, int harmonic, const om_solve_options *opts, const double *b,
                 double *x, om_solve_stats *stats) {
  if(!pr || !opts || !b || !x || (harmonic != OM_FF && harmonic != OM_SH))
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  double2 *db = nullptr, *dx = nullptr;
  int rc = dev_alloc(ctx, &db, pr->n);
  if(!rc)
    rc = dev_alloc(ctx, &dx, pr->n);
  om_solve_stats st{};
  if(!rc) {
    cudaMemcpyAsync(db, b, sizeof(double2) * pr->n, cudaMemcpyHostToDevice, ctx->stream);
    try {
      rc = solve_impl(pr, harmonic, opts, db, dx, &st);
    } catch(std::exception &e) {
      ctx->err = e.what();
      rc = OM_ERR_CUDA;
    }
    cudaMemcpyAsync(x, dx, sizeof(double2) * pr->n, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if(!rc && e != cudaSuccess)
      rc = cuda_fail(ctx, e, "solve_rhs");
  }
  if(stats)
    *stats = st;
  dev_free(ctx, db, pr->n);
  dev_free(ctx, dx, pr->n);
  return rc;
}

int om_get_coefficients(om_problem *pr, double *X_sca, double *X_int) {
  if(!pr)
    return OM_ERR_INVALID;
  if(!pr->have_solution) {
    pr->ctx->err = "no solution";
    return OM_ERR_STATE;
  }
  cudaSetDevice(pr->ctx->device);
  if(X_sca)
    cudaMemcpyAsync(X_sca, pr->d_X, sizeof(zd) * pr->n, cudaMemcpyDeviceToHost, pr->ctx->stream);
  if(X_int)
    cudaMemcpyAsync(X_int, pr->d_Xint, sizeof(zd) * pr->n, cudaMemcpyDeviceToHost,
                    pr->ctx->stream);
  cudaError_t e = cudaStreamSynchronize(pr->ctx->stream);
  return e == cudaSuccess ? OM_OK : cuda_fail(pr->ctx, e, "coefficients");
}

int om_cross_sections(om_problem *pr, double out[4]) {
  if(!pr || !out)
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  if(!pr->have_solution) {
    ctx->err = "no solution";
    return OM_ERR_STATE;
  }
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  om::launch_cross_sections(pr);
  cudaMemcpyAsync(out, pr->d_xsec, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if(e != cudaSuccess)
    return cuda_fail(ctx, e, "cross sections");
  return check_launch(ctx, "cross sections");
}

int om_near_field(om_problem *pr, const double *xyz, int npts, double *E, double *H) {
  if(!pr || !xyz || npts < 1 || !E || !H)
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  if(!pr->have_solution) {
    ctx->err = "no solution";
    return OM_ERR_STATE;
  }
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  // grid points reach getEHFields as Spherical (OutputGrid.cpp:147-153) and are
  // converted back to Cartesian inside Tools::toPoint
  std::vector<double> pts(3 * (size_t)npts);
  for(int i = 0; i < npts; ++i) {
    double s[3];
    to_sph(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], s);
    om::to_cartesian(s[0], s[1], s[2], &pts[3 * i], &pts[3 * i + 1], &pts[3 * i + 2]);
  }
  double *d_xyz = nullptr;
  zd *d_E = nullptr, *d_H = nullptr;
  int rc = dev_alloc(ctx, &d_xyz, 3 * (size_t)npts);
  if(!rc) rc = dev_alloc(ctx, &d_E, 3 * (size_t)npts);
  if(!rc) rc = dev_alloc(ctx, &d_H, 3 * (size_t)npts);
  if(!rc) {
    cudaMemcpyAsync(d_xyz, pts.data(), sizeof(double) * pts.size(), cudaMemcpyHostToDevice,
                    ctx->stream);
    om::launch_near_field(pr, d_xyz, npts, d_E, d_H);
    rc = check_launch(ctx, "near field");
    if(!rc) {
      cudaMemcpyAsync(E, d_E, sizeof(zd) * 3 * npts, cudaMemcpyDeviceToHost, ctx->stream);
      cudaMemcpyAsync(H, d_H, sizeof(zd) * 3 * npts, cudaMemcpyDeviceToHost, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if(e != cudaSuccess)
        rc = cuda_fail(ctx, e, "near field");
    }
  }
  dev_free(ctx, d_xyz, 3 * (size_t)npts);
  dev_free(ctx, d_E, 3 * (size_t)npts);
  dev_free(ctx, d_H, 3 * (size_t)npts);
  return rc;
}


int om_solve_sh(om_problem *pr, const om_solve_options *opts, om_solve_stats *stats) {
  if(!pr || !opts)
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  if(!pr->have_solution) {
    ctx->err = "the SH source needs the fundamental solution (om_solve first)";
    return OM_ERR_STATE;
  }
  if(pr->S_prec[OM_SH] < 0) {
    ctx->err = "SH matrix not assembled (om_assemble with OM_SH)";
    return OM_ERR_STATE;
  }
  int rc = om::sh_alloc(pr);
  if(rc)
    return rc;
  om_solve_stats st{};
  try {
    om::launch_sh_source(pr);
    rc = check_launch(ctx, "SH source");
    if(!rc)
      rc = solve_impl(pr, OM_SH, opts, (const double2 *)pr->d_K, (double2 *)pr->d_Xsh, &st);
  } catch(std::exception &e) {
    ctx->err = e.what();
    rc = OM_ERR_CUDA;
  }
  if(stats)
    *stats = st;
  if(rc && rc != OM_ERR_NOT_CONVERGED)
    return rc;
  om::launch_sh_internal(pr);
  int rc2 = check_launch(ctx, "SH internal coefficients");
  if(rc2)
    return rc2;
  pr->have_sh = true;
  return rc;
}

int om_get_sh_vectors(om_problem *pr, double *K, double *K1ana, double *X_sca_SH,
                      double *X_int_SH) {
  if(!pr)
    return OM_ERR_INVALID;
  if(!pr->have_sh) {
    pr->ctx->err = "no SH solution";
    return OM_ERR_STATE;
  }
  cudaSetDevice(pr->ctx->device);
  const size_t b = sizeof(zd) * pr->n;
  if(K) cudaMemcpyAsync(K, pr->d_K, b, cudaMemcpyDeviceToHost, pr->ctx->stream);
  if(K1ana) cudaMemcpyAsync(K1ana, pr->d_K1, b, cudaMemcpyDeviceToHost, pr->ctx->stream);
  if(X_sca_SH) cudaMemcpyAsync(X_sca_SH, pr->d_Xsh, b, cudaMemcpyDeviceToHost, pr->ctx->stream);
  if(X_int_SH) cudaMemcpyAsync(X_int_SH, pr->d_Xish, b, cudaMemcpyDeviceToHost, pr->ctx->stream);
  cudaError_t e = cudaStreamSynchronize(pr->ctx->stream);
  return e == cudaSuccess ? OM_OK : cuda_fail(pr->ctx, e, "SH vectors");
}

int om_near_field_sh(om_problem *pr, const double *xyz, int npts, double *E, double *H) {
  if(!pr || !xyz || npts < 1 || !E || !H)
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  if(!pr->have_sh) {
    ctx->err = "no SH solution";
    return OM_ERR_STATE;
  }
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  std::vector<double> pts(3 * (size_t)npts);
  for(int i = 0; i < npts; ++i) {
    double s[3];
    to_sph(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], s);
    om::to_cartesian(s[0], s[1], s[2], &pts[3 * i], &pts[3 * i + 1], &pts[3 * i + 2]);
  }
  // Result.cpp:237-244: interior SH wave number and impedance per sphere
  const cplx w0 = pr->omega * std::sqrt(kEps0 * kMu0);
  std::vector<zd> kin(pr->N), izw(pr->N);
  for(int j = 0; j < pr->N; ++j) {
    const cplx k = cplx(2.0, 0.0) * w0 * std::sqrt(pr->eps_r_sh[j] * pr->mu_r[j]);
    const cplx mu_sh = pr->mu_r[j] * kMu0, eps_sh = pr->eps_r_sh[j] * kEps0;
    const cplx iz = (cplx(0.0, -1.0) / std::sqrt(mu_sh / eps_sh)) * w0;
    kin[j] = om::mk(k.real(), k.imag());
    izw[j] = om::mk(iz.real(), iz.imag());
  }
  double *d_xyz = nullptr;
  zd *d_E = nullptr, *d_H = nullptr, *d_k = nullptr;
  int *d_inner = nullptr;
  const size_t np = (size_t)npts;
  int rc = dev_alloc(ctx, &d_xyz, 3 * np);
  if(!rc) rc = dev_alloc(ctx, &d_E, 3 * np);
  if(!rc) rc = dev_alloc(ctx, &d_H, 3 * np);
  if(!rc) rc = dev_alloc(ctx, &d_k, 2 * (size_t)pr->N);
  if(!rc) rc = dev_alloc(ctx, &d_inner, np);
  if(!rc) {
    cudaMemcpyAsync(d_xyz, pts.data(), sizeof(double) * pts.size(), cudaMemcpyHostToDevice,
                    ctx->stream);
    cudaMemcpyAsync(d_k, kin.data(), sizeof(zd) * pr->N, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(d_k + pr->N, izw.data(), sizeof(zd) * pr->N, cudaMemcpyHostToDevice,
                    ctx->stream);
    try {
      om::launch_near_field_sh(pr, d_xyz, npts, w0, d_k, d_k + pr->N, d_inner, d_E, d_H);
      rc = check_launch(ctx, "SH near field");
    } catch(std::exception &e) {
      ctx->err = e.what();
      rc = OM_ERR_CUDA;
    }
    if(!rc) {
      cudaMemcpyAsync(E, d_E, sizeof(zd) * 3 * np, cudaMemcpyDeviceToHost, ctx->stream);
      cudaMemcpyAsync(H, d_H, sizeof(zd) * 3 * np, cudaMemcpyDeviceToHost, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if(e != cudaSuccess)
        rc = cuda_fail(ctx, e, "SH near field");
    }
  }
  cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, d_xyz, 3 * np);
  dev_free(ctx, d_E, 3 * np);
  dev_free(ctx, d_H, 3 * np);
  dev_free(ctx, d_k, 2 * (size_t)pr->N);
  dev_free(ctx, d_inner, np);
  return rc;
}

int om_sh_cross_sections(om_problem *pr, double out[2]) {
  if(!pr || !out)
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  if(!pr->have_sh) {
    ctx->err = "no SH solution";
    return OM_ERR_STATE;
  }
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  try {
    om::launch_sh_cross_sections(pr, pr->d_xsec + 4);
  } catch(std::exception &e) {
    ctx->err = e.what();
    return OM_ERR_CUDA;
  }
  cudaMemcpyAsync(out, pr->d_xsec + 4, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if(e != cudaSuccess)
    return cuda_fail(ctx, e, "SH cross sections");
  return check_launch(ctx, "SH cross sections");
}

int om_clg_tables(om_context *ctx, int nmax, double *out) {
  if(!ctx || !out || nmax < 1 || nmax > om::kMaxNmax)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  try {
    const double *d = om::clg_tables_dev(ctx, nmax);
    const size_t P = om::pmax(nmax);
    cudaMemcpyAsync(out, d, sizeof(double) * 9 * P * P * P, cudaMemcpyDeviceToHost, ctx->stream);
  } catch(std::exception &e) {
    ctx->err = e.what();
    return OM_ERR_BUDGET;
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? check_launch(ctx, "tables") : cuda_fail(ctx, e, "tables");
}

int om_wavelength_solve_sh(om_context *ctx, const om_sphere *spheres, int n_spheres,
                           const om_medium *background, const om_plane_wave *wave,
                           const om_solve_options *opts, int precision, double xsec[4],
                           double xsec_sh[2], om_solve_stats *stats) {
  if(!ctx || !opts || !xsec || !wave)
    return OM_ERR_INVALID;
  om_problem *pr = nullptr;
  int rc = om_problem_create(ctx, spheres, n_spheres, background, wave, &pr);
  if(rc)
    return rc;
  int launches = ctx->last_launches;
  auto step = [&](int r) {
    launches += ctx->last_launches;
    return r;
  };
  rc = step(om_source_vector(pr, nullptr));
  if(!rc) rc = step(om_assemble(pr, OM_FF, precision));
  int solve_rc = OM_OK;
  if(!rc) {
    solve_rc = step(om_solve(pr, opts, stats));
    if(solve_rc && solve_rc != OM_ERR_NOT_CONVERGED)
      rc = solve_rc;
  }
  if(!rc) rc = step(om_cross_sections(pr, xsec));
  if(!rc && wave->sh && xsec_sh) {
    rc = step(om_assemble(pr, OM_SH, precision));
    if(!rc) {
      int r2 = step(om_solve_sh(pr, opts, nullptr));
      if(r2 && r2 != OM_ERR_NOT_CONVERGED)
        rc = r2;
      else if(r2)
        solve_rc = r2;
    }
    if(!rc) rc = step(om_sh_cross_sections(pr, xsec_sh));
  }
  std::string err = ctx->err;
  om_problem_destroy(pr);
  ctx->err = err;
  ctx->last_launches = launches;
  return rc ? rc : solve_rc;
}

int om_wavelength_solve(om_context *ctx, const om_sphere *spheres, int n_spheres,
                        const om_medium *background, const om_plane_wave *wave,
                        const om_solve_options *opts, int precision, double xsec[4],
                        double *X_sca, double *X_int, om_solve_stats *stats) {
  if(!ctx || !opts || !xsec)
    return OM_ERR_INVALID;
  om_problem *pr = nullptr;
  int rc = om_problem_create(ctx, spheres, n_spheres, background, wave, &pr);
  if(rc)
    return rc;
  int launches = ctx->last_launches;
  rc = om_source_vector(pr, nullptr);
  launches += ctx->last_launches;
  if(!rc) {
    rc = om_assemble(pr, OM_FF, precision);
    launches += ctx->last_launches;
  }
  int solve_rc = OM_OK;
  if(!rc) {
    solve_rc = om_solve(pr, opts, stats);
    launches += ctx->last_launches;
    if(solve_rc && solve_rc != OM_ERR_NOT_CONVERGED)
      rc = solve_rc;
  }
  if(!rc) {
    rc = om_cross_sections(pr, xsec);
    launches += ctx->last_launches;
  }
  if(!rc && (X_sca || X_int))
    rc = om_get_coefficients(pr, X_sca, X_int);
  std::string err = ctx->err;
  om_problem_destroy(pr);
  ctx->err = err;
  ctx->last_launches = launches;
  return rc ? rc : solve_rc;
}

}  // extern "C"
