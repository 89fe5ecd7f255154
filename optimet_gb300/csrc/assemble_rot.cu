// Precision-form assembly of the scattering matrix by rotations.
//
// The coupling blocks of a displacement R = (r, theta, phi) are rotated z-axis
// translations: A(R) = U A(r z) U^H and B(R) = U B(r z) U^H, with U block
// diagonal over the degree n, U[(n, m'), (n, m)] = d^n_{m'm}(theta) e^{i m' phi}
// (Wigner small-d), and the z-axis blocks A(r z), B(r z) diagonal in m. Only the
// d = m - k = 0 slice of the Stout recurrences
// (TranslationAdditionCoefficients.cpp:71-124) survives on the z axis. That
// slice is linear in its seeds alpha(0,0,p,0) = (-1)^p sqrt(2p+1) h_p(k r)
// (:102-111) with geometry-independent coefficients, so the host runs the
// recurrence once per nMax on unit seeds and the kernel applies the resulting
// sparse map, alpha(n,m,l,m) = sum_p C^p_{nml} h_p(k r) with
// p = |n-l|, |n-l|+2, ..., n+l, to each pair's Hankel values. The block of S
// (PreconditionedMatrix.cpp:369-397) is then
//
//   S_ij[(l,k'), (n,m')] = -T_i(l) e^{i(m'-k')phi} M_A(m', k'),
//   M_A(m', k') = sum_m d^n_{m'm} Az_m(n,l) d^l_{k'm}
//
// (B likewise, on the TM/TE off-diagonal blocks), and S_ji follows from the
// parity A(-R) = (-1)^{n+l} A(R), B(-R) = -(-1)^{n+l} B(R). For a real wave
// number Az_{-m} = Az_m and Bz_{-m} = -Bz_m, and with
// d^n_{-m',-m} = (-1)^{m'+m} d^n_{m'm} this gives
// M_A(-m',-k') = (-1)^{m'+k'} M_A(m',k'), M_B(-m',-k') = -(-1)^{m'+k'} M_B(m',k'):
// only the columns m' >= 0 are computed and each also writes its mirror.
//
// FP64 is scarce on this part (about 1/60 of the FP32 rate) and the FP32 work
// is issue-bound, so: every FP64 step runs with its lanes full, and the FP32
// products use the packed fma.rn.f32x2 (two FP32 lanes per instruction). One
// CTA of 128 threads takes kPPC work items (unordered sphere pairs i < j,
// identity diagonal blocks, or idle padding of a batch size class):
//  prologue, once per CTA, FP64, one lane per pair: geometry and the Hankel
//     values h_p(k r), p <= 2 nMax; then one lane per (pair, m): the phases
//     e^{i m phi} and the powers of cos, sin (theta / 2);
//  per pair, FP64: one warp (two above nMax 8) runs the Wigner d^n(theta),
//     n <= nMax, by the three-term recurrence in n over the wedge m' >= |m|
//     (host-built step coefficients, chains balanced over the lanes; the rest
//     of d by its symmetries) while the other warps apply the z-axis map
//     (rounded once to complex64);
//  per pair, FP32: Az, Bz (the coupling formulas of Coupling.cpp:30-51 with
//     k = m, from a host-built table of the three alpha terms and their
//     factors), then the rotation products, register-blocked over a run of up
//     to 9 column harmonics m' of one degree n per thread and row p, scaled by
//     -T(l) and the phases and stored column by column (coalesced rows) for
//     S_ij and S_ji.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <vector>

#include "om_internal.h"

namespace om {

namespace {

constexpr int kRotThreads = 128;
constexpr int kPPC = 8;       // work items (pairs) per CTA
constexpr int kChunk = 9;     // column harmonics m' per thread (register block)
constexpr int kMaxGroups = 48;

struct RotArgs {
  const double *cart;
  const zd *T;  // N x (nmax+1) x 2
  const int *ti;     // rotation tables (ints), see rotation_tables
  const double *td;  // rotation tables (doubles)
  const float4 *tz;  // Az / Bz formation table, 3 float4 per entry
  int N, nmax;
  zd waveK;
  long ld;
  long items;        // work items in the grid (pairs + identity blocks, or the batch table's)
  const BatchMat *batch;
  int per_mat;
  int nwl, nent, ent_base, onl_base, naz;
  int ngf, ngh;      // column groups: all m' (complex k) / m' >= 0 (real k)
  signed char gn[2][kMaxGroups], gm0[2][kMaxGroups], gcnt[2][kMaxGroups];
};

// Shared-memory layout (bytes), the same on host and device.
struct RotLayout {
  int ncomp;   // compact (m, n, l) alpha entries: |m| <= n, l <= nMax (plus a zero slot)
  int naz;     // Az / Bz entries: per (n, l), m = -min(n,l) .. min(n,l)
  int nw;      // Wigner entries: sum_{n=1}^{nMax} (2n+1)^2
  int o_alz, o_az, o_bz, o_w, o_e, o_pw, o_t, o_wo, o_onl, o_geo, o_hk, o_grp, o_item;
  int bytes;
};

__host__ __device__ inline RotLayout rot_layout(int nmax) {
  RotLayout y;
  int nc = 0;
  for(int m = -nmax; m <= nmax; ++m) {
    const int w = nmax - (m < 0 ? -m : m) + 1;
    nc += w * w;
  }
  y.ncomp = nc;
  int na = 0;
  for(int n = 1; n <= nmax; ++n)
    for(int l = 1; l <= nmax; ++l)
      na += 2 * (n < l ? n : l) + 1;
  y.naz = na;
  int nw = 0;
  for(int n = 1; n <= nmax; ++n)
    nw += (2 * n + 1) * (2 * n + 1);
  y.nw = nw;
  const int L1 = 2 * nmax + 1;
  int o = 0;
  auto take = [&](int bytes) {
    const int at = o;
    o += (bytes + 15) & ~15;
    return at;
  };
  y.o_alz = take(8 * (nc + 1));
  y.o_az = take(8 * na);
  y.o_bz = take(8 * na);
  y.o_w = take(8 * nw);               // (d, d) pairs for the packed products
  y.o_e = take(8 * kPPC * L1);        // e^{i m phi}, m = -nMax..nMax, FP32, per pair
  y.o_pw = take(16 * kPPC * L1);      // c^k, s^k, k <= 2 nMax, FP64, per pair
  y.o_t = take(8 * 4 * (nmax + 1));
  y.o_wo = take(4 * (nmax + 2));
  y.o_onl = take(4 * (nmax + 1) * (nmax + 1));
  y.o_geo = take(8 * 8 * kPPC);
  y.o_hk = take(16 * 2 * L1 * kPPC);  // h_p(k r) and, for complex k, h_p(-conj(k) r)
  y.o_grp = take(4 * 2 * kMaxGroups);
  y.o_item = take(16 * kPPC);
  y.bytes = o;
  return y;
}

// --- packed FP32 pairs (fma.rn.f32x2 / mul.rn.f32x2) ---
__device__ __forceinline__ unsigned long long u64(float2 a) { return *reinterpret_cast<unsigned long long *>(&a); }
__device__ __forceinline__ float2 f2(unsigned long long a) { return *reinterpret_cast<float2 *>(&a); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(u64(a)), "l"(u64(b)), "l"(u64(c)));
  return f2(d);
}
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(u64(a)), "l"(u64(b)));
  return f2(d);
}
// complex a * b: (a.x, a.x) * b + (a.y, a.y) * (-b.y, b.x)
__device__ __forceinline__ float2 cm(float2 a, float2 b) {
  return f2fma(make_float2(a.x, a.x), b, f2mul(make_float2(a.y, a.y), make_float2(-b.y, b.x)));
}
__device__ __forceinline__ float2 negf(float2 a) { return make_float2(-a.x, -a.y); }

// A work item: its matrix and what the CTA does for it.
struct Item {
  int kind;  // 0 idle, 1 pair, 2 identity block
  int i, j;  // spheres (pair) or the diagonal block (identity)
  int mat;   // matrix (batch table entry), 0 without a batch
};

__device__ Item decode(const RotArgs &a, long w) {
  Item it{0, 0, 0, 0};
  if(w >= a.items)
    return it;
  long b = w;
  int N = a.N;
  if(a.batch) {
    it.mat = (int)(w / a.per_mat);
    b = w % a.per_mat;
    N = a.batch[it.mat].N;
    if(b >= (long)N * (N + 1) / 2)  // padding of the size class or an empty entry
      return it;
  }
  const long npairs = (long)N * (N - 1) / 2;
  if(b >= npairs) {
    it.kind = 2;
    it.i = it.j = (int)(b - npairs);
    return it;
  }
  // b -> (i, j), i < j: b = j (j - 1) / 2 + i
  int j = (int)((1.0 + sqrt(1.0 + 8.0 * (double)b)) * 0.5);
  while((long)j * (j - 1) / 2 > b)
    --j;
  while((long)(j + 1) * j / 2 <= b)
    ++j;
  it.kind = 1;
  it.i = (int)(b - (long)j * (j - 1) / 2);
  it.j = j;
  return it;
}

// Spherical Hankel functions h_0 .. h_L of a real argument x > 0: the closed
// forms of h_0, h_1 and the upward recurrence h_{p+1} = (2p+1)/x h_p - h_{p-1}
// on real and imaginary parts (the recurrence of sph_h1 for a real argument).
__device__ void hankel_real(double x, int L, zd *h) {
  double sx, cx;
  sincos(x, &sx, &cx);
  const double rx = 1.0 / x;
  zd h0 = mk(sx * rx, -cx * rx);
  h[0] = h0;
  if(L == 0)
    return;
  zd h1 = mk((h0.re - cx) * rx, (h0.im - sx) * rx);
  h[1] = h1;
  for(int p = 1; p < L; ++p) {
    const double c = (2 * p + 1) * rx;
    const zd h2 = mk(fma(c, h1.re, -h0.re), fma(c, h1.im, -h0.im));
    h[p + 1] = h2;
    h0 = h1;
    h1 = h2;
  }
}

// c^k by binary powering (k >= 0)
__device__ __forceinline__ double ipow(double c, int k) {
  double r = 1.0;
  while(k) {
    if(k & 1)
      r *= c;
    c *= c;
    k >>= 1;
  }
  return r;
}

// Products of one run: cnt <= C column harmonics m' = m0 .. m0 - cnt + 1 of
// degree n for row (l, k'): accA[c] = sum_m d^n_{m'm} Az_m(n,l) d^l_{k'm},
// accB likewise. W2 holds (d, d) pairs so that one packed FMA updates re and im.
template <int C>
__device__ __forceinline__ void products(const float2 *wl, int sl, const float2 *wn, int sn, const float2 *azp,
                                         const float2 *bzp, int cntm, int cnt, float2 *accA, float2 *accB) {
#pragma unroll
  for(int c = 0; c < C; ++c) {
    accA[c] = make_float2(0.f, 0.f);
    accB[c] = make_float2(0.f, 0.f);
  }
  for(int it = 0; it < cntm; ++it) {
    const float2 dl = *wl;
    wl += sl;
    const float2 xa = f2mul(azp[it], dl), xb = f2mul(bzp[it], dl);
#pragma unroll
    for(int c = 0; c < C; ++c) {
      if(c < cnt) {
        const float2 dn = wn[-c];  // m' = m0 - c
        accA[c] = f2fma(dn, xa, accA[c]);
        accB[c] = f2fma(dn, xb, accB[c]);
      }
    }
    wn += sn;
  }
}

// The eight S entries of (row p, column q) for the run's columns; then, for a
// real wave number, the eight of each mirror (row p', column q'), m' > 0.
template <int C>
__device__ __forceinline__ void store_run(float2 *bi, float2 *bj, size_t LD, size_t PLD, int P, int p, int pm,
                                          int n, int m0, int cnt, const float2 *E, int nmax, const float2 *accA,
                                          const float2 *accB, const float2 *Tl, int nT, int l, int kp, bool mirror) {
  const float2 tei = Tl[2 * l], tmi = Tl[2 * l + 1], tej = Tl[nT + 2 * l], tmj = Tl[nT + 2 * l + 1];
  const float sgn = ((n + l) & 1) ? 1.f : -1.f;  // -(-1)^{n+l}
  {
    // S_ij's row factors -T_i(l) e^{-ik'phi}; S_ji's -(-1)^{n+l} T_j(l) e^{-ik'phi}
    const float2 ek = E[nmax - kp];
    const float2 ci_te = cm(negf(tei), ek), ci_tm = cm(negf(tmi), ek);
    const float2 cj_te = cm(make_float2(sgn * tej.x, sgn * tej.y), ek);
    const float2 cj_tm = cm(make_float2(sgn * tmj.x, sgn * tmj.y), ek);
#pragma unroll
    for(int c = 0; c < C; ++c) {
      if(c < cnt) {
        const int mp = m0 - c;
        const int q = n * (n + 1) - mp - 1;
        const float2 A = cm(E[nmax + mp], accA[c]), B = cm(E[nmax + mp], accB[c]);
        float2 *ci = bi + (size_t)q * LD, *cj = bj + (size_t)q * LD;
        ci[p] = cm(ci_te, A);
        ci[PLD + P + p] = cm(ci_tm, A);
        ci[PLD + p] = cm(ci_te, B);
        ci[P + p] = cm(ci_tm, B);
        // S_ji: A -> (-1)^{n+l} A, B -> -(-1)^{n+l} B, rows of sphere j
        cj[p] = cm(cj_te, A);
        cj[PLD + P + p] = cm(cj_tm, A);
        cj[PLD + p] = cm(negf(cj_te), B);
        cj[P + p] = cm(negf(cj_tm), B);
      }
    }
  }
  if(!mirror)
    return;
  {
    // mirror (-m', -k'): A_m = (-1)^{m'} conj(em) M_A, B_m = -(-1)^{m'} conj(em) M_B;
    // (-1)^{k'} and e^{+ik'phi} go into the mirror row factors
    const float2 ekm = E[nmax + kp];
    const float sk = (kp & 1) ? -1.f : 1.f;
    const float2 mi_te = cm(make_float2(-sk * tei.x, -sk * tei.y), ekm);
    const float2 mi_tm = cm(make_float2(-sk * tmi.x, -sk * tmi.y), ekm);
    const float2 mj_te = cm(make_float2(sk * sgn * tej.x, sk * sgn * tej.y), ekm);
    const float2 mj_tm = cm(make_float2(sk * sgn * tmj.x, sk * sgn * tmj.y), ekm);
#pragma unroll
    for(int c = 0; c < C; ++c) {
      const int mp = m0 - c;
      if(c < cnt && mp > 0) {
        const float2 emc = E[nmax - mp];  // conj(e^{i m' phi})
        const float2 dA = cm(emc, accA[c]), dB = cm(emc, accB[c]);
        const bool odd = mp & 1;
        const float2 Am = odd ? negf(dA) : dA, Bm = odd ? dB : negf(dB);
        const int qm = n * (n + 1) + mp - 1;
        float2 *mi = bi + (size_t)qm * LD, *mj = bj + (size_t)qm * LD;
        mi[pm] = cm(mi_te, Am);
        mi[PLD + P + pm] = cm(mi_tm, Am);
        mi[PLD + pm] = cm(mi_te, Bm);
        mi[P + pm] = cm(mi_tm, Bm);
        mj[pm] = cm(mj_te, Am);
        mj[PLD + P + pm] = cm(mj_tm, Am);
        mj[PLD + pm] = cm(negf(mj_te), Bm);
        mj[P + pm] = cm(negf(mj_tm), Bm);
      }
    }
  }
}

template <int C>
__device__ __forceinline__ void run_item(float2 *bi, float2 *bj, size_t LD, size_t PLD, int P, int p, int pm, int n,
                                         int m0, int cnt, int l, int kp, const float2 *W2, const int *wo,
                                         const float2 *az, const float2 *bz, const int *onl, int nmax,
                                         const float2 *E, const float2 *Tl, int nT, bool mirror) {
  float2 accA[C], accB[C];
  const int mn = n < l ? n : l;
  const float2 *wl = W2 + wo[l] + (l - mn) * (2 * l + 1) + (kp + l);
  const float2 *wn = W2 + wo[n] + (n - mn) * (2 * n + 1) + (m0 + n);
  const int e0 = onl[n * (nmax + 1) + l];
  products<C>(wl, 2 * l + 1, wn, 2 * n + 1, az + e0, bz + e0, 2 * mn + 1, cnt, accA, accB);
  store_run<C>(bi, bj, LD, PLD, P, p, pm, n, m0, cnt, E, nmax, accA, accB, Tl, nT, l, kp, mirror);
}

__global__ void __launch_bounds__(kRotThreads, 5) k_assemble_rot(RotArgs a, float2 *S0) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int nmax = a.nmax;
  const RotLayout y = rot_layout(nmax);
  float2 *alz = reinterpret_cast<float2 *>(sm + y.o_alz);
  float2 *az = reinterpret_cast<float2 *>(sm + y.o_az);
  float2 *bz = reinterpret_cast<float2 *>(sm + y.o_bz);
  float2 *W2 = reinterpret_cast<float2 *>(sm + y.o_w);
  float2 *Eall = reinterpret_cast<float2 *>(sm + y.o_e);
  double *pwall = reinterpret_cast<double *>(sm + y.o_pw);
  float2 *Tl = reinterpret_cast<float2 *>(sm + y.o_t);
  int *wo = reinterpret_cast<int *>(sm + y.o_wo);
  int *onl = reinterpret_cast<int *>(sm + y.o_onl);
  double *geoall = reinterpret_cast<double *>(sm + y.o_geo);
  zd *hkall = reinterpret_cast<zd *>(sm + y.o_hk);
  int *grp = reinterpret_cast<int *>(sm + y.o_grp);
  int4 *items = reinterpret_cast<int4 *>(sm + y.o_item);

  const int t = threadIdx.x, warp = t >> 5;
  const int P = nmax * (nmax + 2);
  const int L1 = 2 * nmax + 1;
  const long w0 = (long)blockIdx.x * kPPC;

  // --- prologue: tables, then per pair (one lane each) geometry and Hankel values ---
  if(t == 0) {
    int q = 0;
    wo[0] = 0;
    for(int n = 1; n <= nmax; ++n) {
      wo[n] = q;
      q += (2 * n + 1) * (2 * n + 1);
    }
    alz[y.ncomp] = make_float2(0.f, 0.f);  // the zero slot of absent alpha terms
  }
  for(int v = t; v < (nmax + 1) * (nmax + 1); v += blockDim.x)
    onl[v] = a.ti[a.onl_base + v];
  if(t < 2 * kMaxGroups) {
    const int s = t / kMaxGroups, g = t - s * kMaxGroups;
    grp[t] = (int)a.gn[s][g] | ((int)(unsigned char)a.gm0[s][g] << 8) | ((int)a.gcnt[s][g] << 16);
  }
  if(t < kPPC) {
    const Item it = decode(a, w0 + t);
    items[t] = make_int4(it.kind, it.i, it.j, it.mat);
    if(it.kind == 1) {
      const double *cart = a.batch ? a.batch[it.mat].cart : a.cart;
      const zd waveK = a.batch ? a.batch[it.mat].waveK : a.waveK;
      const double dx = cart[3 * it.i] - cart[3 * it.j], dy = cart[3 * it.i + 1] - cart[3 * it.j + 1],
                   dz = cart[3 * it.i + 2] - cart[3 * it.j + 2];
      const double rho2 = dx * dx + dy * dy, r = sqrt(rho2 + dz * dz), rho = sqrt(rho2);
      const double rr = 1.0 / r;
      // cos(theta/2), sin(theta/2) without cancellation on either hemisphere
      double c, s;
      if(dz >= 0.0) {
        c = sqrt(0.5 * (1.0 + dz * rr));
        s = 0.5 * rho * rr / c;
      } else {
        s = sqrt(0.5 * (1.0 - dz * rr));
        c = 0.5 * rho * rr / s;
      }
      double *geo = geoall + 8 * t;
      geo[0] = r;
      geo[1] = dz * rr;  // cos theta
      geo[2] = c;
      geo[3] = s;
      geo[4] = rho > 0.0 ? dx / rho : 1.0;  // cos phi
      geo[5] = rho > 0.0 ? dy / rho : 0.0;  // sin phi
      zd *h = hkall + 2 * L1 * t;
      if(waveK.im == 0.0) {
        hankel_real(waveK.re * r, 2 * nmax, h);
      } else {
        zd f[kMaxOrder + 2];
        sph_h1(r * waveK, 2 * nmax, f);
        for(int p = 0; p <= 2 * nmax; ++p)
          h[p] = f[p];
        sph_h1(r * (-conj(waveK)), 2 * nmax, f);  // the conjugate wave (TranslationAdditionCoefficients.h:72-74)
        for(int p = 0; p <= 2 * nmax; ++p)
          h[L1 + p] = f[p];
      }
    }
  }
  __syncthreads();
  // phases e^{i m phi} (m >= 0, binary powering in FP64; m < 0 by conjugation)
  // and the powers c^k, s^k of the Wigner edges: one lane per (pair, m) / (pair, k)
  for(int v = t; v < kPPC * (nmax + 1); v += blockDim.x) {
    const int u = v / (nmax + 1), m = v - u * (nmax + 1);
    if(items[u].x != 1)
      continue;
    const double *geo = geoall + 8 * u;
    zd z = mk(geo[4], geo[5]), e = mk(1.0, 0.0);
    for(int k = m; k; k >>= 1) {
      if(k & 1)
        e = e * z;
      z = z * z;
    }
    float2 *E = Eall + u * L1;
    E[nmax + m] = make_float2((float)e.re, (float)e.im);
    E[nmax - m] = make_float2((float)e.re, (float)-e.im);
  }
  for(int v = t; v < kPPC * L1; v += blockDim.x) {
    const int u = v / L1, k = v - u * L1;
    if(items[u].x != 1)
      continue;
    const double *geo = geoall + 8 * u;
    double *pw = pwall + 2 * L1 * u;
    pw[k] = ipow(geo[2], k);
    pw[L1 + k] = ipow(geo[3], k);
  }
  __syncthreads();

  const int *wl_off = a.ti;              // Wigner lanes: chain lists
  const int *ent = a.ti + a.ent_base;    // z-axis map entries
  const double *wcoef = a.td;            // Wigner step coefficients, then the map's
  const int nT = 2 * (nmax + 1);
  for(int u = 0; u < kPPC; ++u) {
    const int4 iv = items[u];
    if(iv.x == 0)
      continue;
    const int i = iv.y, j = iv.z;
    float2 *S = a.batch ? (float2 *)a.batch[iv.w].S : S0;
    const size_t LD = (size_t)(a.batch ? a.batch[iv.w].ld : a.ld);
    if(iv.x == 2) {
      const size_t x0 = 2ul * P * i;
      for(int idx = t; idx < 4 * P * P; idx += blockDim.x) {
        const int c = idx / (2 * P), r = idx - c * 2 * P;
        S[(x0 + c) * LD + x0 + r] = make_float2(r == c ? 1.f : 0.f, 0.f);
      }
      continue;
    }
    const zd *Tg = a.batch ? a.batch[iv.w].T : a.T;
    const bool real_k = (a.batch ? a.batch[iv.w].waveK.im : a.waveK.im) == 0.0;
    const double *geo = geoall + 8 * u;
    const zd *hk = hkall + 2 * L1 * u;
    const float2 *E = Eall + u * L1;

    // --- FP64: Wigner wedge (warps < nwl / 32) beside the z-axis map (other warps) ---
    const int wwarps = a.nwl >> 5;
    if(warp < wwarps) {
      const double ct = geo[1];
      const double *pw = pwall + 2 * L1 * u;
      for(int c = wl_off[t]; c < wl_off[t + 1]; ++c) {
        const int cv = wl_off[a.nwl + 1 + c];
        const int mp = cv & 0xff, m = ((cv >> 8) & 0xff) - 128, co = cv >> 16;
        const bool flip = (mp - m) & 1;
        const double *cf = wcoef + co;
        double cur = __ldg(cf) * pw[mp + m] * pw[L1 + mp - m], prev = 0.0;
        auto put = [&](int n, double d) {
          const int w = 2 * n + 1, b = wo[n];
          const float f = (float)d, g = flip ? -f : f;
          W2[b + (m + n) * w + (mp + n)] = make_float2(f, f);    // d_{m' m}
          W2[b + (-mp + n) * w + (-m + n)] = make_float2(f, f);  // d_{-m, -m'}
          W2[b + (mp + n) * w + (m + n)] = make_float2(g, g);    // d_{m m'}
          W2[b + (-m + n) * w + (-mp + n)] = make_float2(g, g);  // d_{-m', -m}
        };
        if(mp >= 1)
          put(mp, cur);
        for(int n = mp + 1; n <= nmax; ++n) {
          const double *k3 = cf + 1 + 3 * (n - mp - 1);
          const double nx = fma(fma(__ldg(k3), ct, -__ldg(k3 + 1)), cur, -__ldg(k3 + 2) * prev);
          prev = cur;
          cur = nx;
          put(n, nx);
        }
      }
    } else {
      for(int e = t - 32 * wwarps; e < a.nent; e += blockDim.x - 32 * wwarps) {
        const int4 ev = reinterpret_cast<const int4 *>(ent)[e];
        const int ip = ev.x & 0xffff, im = ev.x >> 16;
        const int p0 = ev.y & 0xff, cnt = (ev.y >> 8) & 0xff, odd = ev.y >> 16;
        const double *cf = wcoef + ev.z;
        zd acc = mk(0.0, 0.0);
        for(int q = 0; q < cnt; ++q) {
          const double c = __ldg(cf + q);
          const zd h = hk[p0 + 2 * q];
          acc.re = fma(c, h.re, acc.re);
          acc.im = fma(c, h.im, acc.im);
        }
        alz[ip] = make_float2((float)acc.re, (float)acc.im);
        if(real_k) {
          alz[im] = make_float2((float)acc.re, (float)acc.im);
        } else if(im != ip) {
          // conjugate wave: alpha(n,-m,l,-m) = (-1)^{n+l} conj(alpha_neg(n,m,l,m))
          zd an = mk(0.0, 0.0);
          for(int q = 0; q < cnt; ++q) {
            const double c = __ldg(cf + q);
            const zd h = hk[L1 + p0 + 2 * q];
            an.re = fma(c, h.re, an.re);
            an.im = fma(c, h.im, an.im);
          }
          const float sg = odd ? -1.f : 1.f;
          alz[im] = make_float2(sg * (float)an.re, -sg * (float)an.im);
        }
      }
      for(int v = t - 32 * wwarps; v < 2 * nT; v += blockDim.x - 32 * wwarps) {
        const zd tv = Tg[(size_t)(v < nT ? i : j) * nT + (v < nT ? v : v - nT)];
        Tl[v] = make_float2((float)tv.re, (float)tv.im);
      }
    }
    __syncthreads();

    // --- FP32: the z-axis coupling blocks (Coupling.cpp:30-51, k = m) from the
    //     table {alpha indices t0, t+, t-, u0, u+, u- (the zero slot where a term
    //     is absent), factors f0, f1, f2, g0, g1, g2} ---
    for(int e = t; e < y.naz; e += blockDim.x) {
      const float4 r0 = __ldg(a.tz + 3 * e), f = __ldg(a.tz + 3 * e + 1), g = __ldg(a.tz + 3 * e + 2);
      const int i0 = __float_as_int(r0.x), i1 = __float_as_int(r0.y), i2 = __float_as_int(r0.z);
      const float2 t0 = alz[i0 & 0xffff], tp = alz[i0 >> 16], tm = alz[i1 & 0xffff];
      const float2 u0 = alz[i1 >> 16], up = alz[i2 & 0xffff], um = alz[i2 >> 16];
      az[e] = make_float2(fmaf(f.x, t0.x, fmaf(f.y, tp.x, f.z * tm.x)), fmaf(f.x, t0.y, fmaf(f.y, tp.y, f.z * tm.y)));
      const float sre = fmaf(f.w, u0.x, fmaf(g.x, up.x, -g.y * um.x));
      const float sim = fmaf(f.w, u0.y, fmaf(g.x, up.y, -g.y * um.y));
      bz[e] = make_float2(sim, -sre);  // B = -i s
    }
    __syncthreads();

    // --- FP32: rotation products and the S_ij / S_ji stores ---
    const int gs = real_k ? 1 : 0, ng = real_k ? a.ngh : a.ngf;
    float2 *bi = S + (size_t)2 * P * j * LD + (size_t)2 * P * i;  // S_ij: rows of i, columns of j
    float2 *bj = S + (size_t)2 * P * i * LD + (size_t)2 * P * j;  // S_ji
    const size_t PLD = (size_t)P * LD;
    const int nitems = ng * P;
    for(int it = t; it < nitems; it += blockDim.x) {
      const int g = it / P, p = it - g * P;
      const int gv = grp[gs * kMaxGroups + g];
      const int n = gv & 0xff, m0 = (int)(signed char)((gv >> 8) & 0xff), cnt = gv >> 16;
      // row harmonic p = (l, k'): p = l(l+1) - k' - 1; mirror row (l, -k')
      int l = (int)sqrtf((float)(p + 1));
      while(l * l - 1 > p)
        --l;
      while((l + 1) * (l + 1) - 1 <= p)
        ++l;
      const int kp = l * (l + 1) - 1 - p, pm = l * (l + 1) + kp - 1;
      if(cnt <= 4)
        run_item<4>(bi, bj, LD, PLD, P, p, pm, n, m0, cnt, l, kp, W2, wo, az, bz, onl, nmax, E, Tl, nT, real_k);
      else
        run_item<kChunk>(bi, bj, LD, PLD, P, p, pm, n, m0, cnt, l, kp, W2, wo, az, bz, onl, nmax, E, Tl, nT, real_k);
    }
    __syncthreads();
  }
}

// Column groups: per degree n, the harmonics m' = n .. -n (all; complex wave
// number) or m' = n .. 0 (real wave number, mirrors derived) split into
// ceil(count / 9) near-equal runs.
void fill_groups(RotArgs &a, int nmax) {
  for(int s = 0; s < 2; ++s) {
    int g = 0;
    for(int n = 1; n <= nmax; ++n) {
      const int w = s ? n + 1 : 2 * n + 1, lo = s ? 0 : -n;
      const int nch = (w + kChunk - 1) / kChunk;
      const int sz = (w + nch - 1) / nch;
      int m0 = n;
      for(int c = 0; c < nch; ++c) {
        const int cnt = std::min(sz, m0 - lo + 1);
        if(g >= kMaxGroups)
          throw std::runtime_error("rotation assembly: too many column groups");
        a.gn[s][g] = (signed char)n;
        a.gm0[s][g] = (signed char)m0;
        a.gcnt[s][g] = (signed char)cnt;
        ++g;
        m0 -= cnt;
      }
    }
    for(int k = g; k < kMaxGroups; ++k)
      a.gn[s][k] = a.gm0[s][k] = a.gcnt[s][k] = 0;
    (s ? a.ngh : a.ngf) = g;
  }
}

// The dynamic shared-memory ceiling is a process-wide attribute of the kernel:
// always raised to the device's opt-in limit (never one launch's size), so
// that host threads launching it with different nMax cannot undercut each other.
void set_rot_smem(om_context *ctx) {
  int dev = 0, lim = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncSetAttribute(k_assemble_rot, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  if(ctx->carve_asm >= 0)
    cudaFuncSetAttribute(k_assemble_rot, cudaFuncAttributePreferredSharedMemoryCarveout, ctx->carve_asm);
}

int wigner_lanes(int nmax) { return nmax <= 8 ? 32 : 64; }

RotArgs rot_args(om_context *ctx, int nmax) {
  const CoefTables &ct = coef_tables(ctx, nmax);
  RotArgs a{};
  a.ti = ct.rot_i;
  a.td = ct.rot_d;
  a.tz = reinterpret_cast<const float4 *>(ct.rot_z);
  a.nmax = nmax;
  a.batch = nullptr;
  a.per_mat = 1;
  a.nwl = wigner_lanes(nmax);
  a.nent = ct.rot_nent;
  a.ent_base = ct.rot_ent_base;
  a.onl_base = ct.rot_onl_base;
  a.naz = rot_layout(nmax).naz;
  fill_groups(a, nmax);
  return a;
}

// Stout recurrence coefficients (TranslationAdditionCoefficients.cpp:34-61)
double ra_plus(int n, int m) {
  if(n < 0 || std::abs(m) > n)
    return 0.0;
  return -std::sqrt(double((n + m + 1) * (n - m + 1)) / double((2 * n + 1) * (2 * n + 3)));
}
double ra_minus(int n, int m) {
  if(n < 0 || std::abs(m) > n)
    return 0.0;
  return std::sqrt(double((n + m) * (n - m)) / double((2 * n + 1) * (2 * n - 1)));
}
double rb_plus(int n, int m) {
  if(n < 0 || std::abs(m) > n)
    return 0.0;
  return std::sqrt(double((n + m + 2) * (n + m + 1)) / double((2 * n + 1) * (2 * n + 3)));
}
double rb_minus(int n, int m) {
  if(n < 0 || std::abs(m) > n)
    return 0.0;
  return std::sqrt(double((n - m) * (n - m - 1)) / double((2 * n + 1) * (2 * n - 1)));
}

}  // namespace

// Host-built tables of the rotation assembly for one nMax.
//
// The z-axis map: the d = 0 slice of the Stout recurrences (diagonal step
// alpha(mu,mu,l,mu) from alpha(mu-1,mu-1,l+-1,mu-1), off-diagonal step
// alpha(n,mu,l,mu) from alpha(n-1,mu,l+-1,mu) and alpha(n-2,mu,l,mu)) run in
// FP64 on each unit seed e_p, p <= 2 nMax, gives alpha(n,m,l,m) = sum_p C^p
// seed_p; with seed_p = (-1)^p sqrt(2p+1) h_p(k r) (the z-axis value of
// sqrt(4 pi) (-1)^p Y_p^0 h_p) folded in, alpha = sum_p c^p h_p with
// p = |n-l| + 2q, q = 0 .. min(n,l).
//
// ti: [0, nwl]: first chain of each Wigner lane; [nwl + 1, ...): the chains
//     (m' | (m + 128) << 8 | coefficient offset << 16); at ent_base: the map
//     entries, 4 ints each (compact index of +m | of -m << 16,
//     p0 | count << 8 | (n + l odd) << 16, coefficient offset, 0), sorted by
//     count so that the lanes of a warp do equal work; at onl_base: the first
//     Az / Bz entry of each (n, l), (nMax+1)^2 ints.
// td: per chain {(-1)^{m'-m} sqrt(C(2m', m'+m)), then per step n = m'+1 ..
//     nMax: a, a m m' / (n (n-1)), a b} for the recurrence
//     d^n = (a cos theta - a m m' / (n(n-1))) d^{n-1} - a b d^{n-2},
//     a = n (2n-1) / sqrt((n^2-m^2)(n^2-m'^2)),
//     b = sqrt(((n-1)^2-m^2)((n-1)^2-m'^2)) / ((n-1)(2n-1));
//     then the map coefficients.
// tz: per Az / Bz entry (n, l, m), m = -min(n,l) .. min(n,l): the compact
//     alpha indices of t0 = alpha(n,m,l), t+ = alpha(n,m+1,l),
//     t- = alpha(n,m-1,l), u0 = alpha(n,m,l-1), u+ = alpha(n,m+1,l-1),
//     u- = alpha(n,m-1,l-1) (the zero slot ncomp where Coupling.cpp drops a
//     term), and the factors of Az = f0 t0 + f1 t+ + f2 t- and
//     Bz = -i (g0 u0 + g1 u+ - g2 u-), as 12 floats (3 float4).
void rotation_tables(int nmax, std::vector<int> &ti, std::vector<double> &td, std::vector<float> &tz, int &nent,
                     int &ent_base, int &onl_base) {
  ti.clear();
  td.clear();
  tz.clear();
  // --- Wigner chains over the wedge m' >= |m|, balanced over the lanes (longest first) ---
  const int nwl = wigner_lanes(nmax);
  struct Chain {
    int mp, m, steps;
  };
  std::vector<Chain> ch;
  for(int mp = 0; mp <= nmax; ++mp)
    for(int m = -mp; m <= mp; ++m)
      ch.push_back({mp, m, nmax - mp + 1});
  std::stable_sort(ch.begin(), ch.end(), [](const Chain &x, const Chain &y) { return x.steps > y.steps; });
  std::vector<std::vector<int>> lane(nwl);
  std::vector<int> load(nwl, 0);
  for(int c = 0; c < (int)ch.size(); ++c) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    lane[k].push_back(c);
    load[k] += ch[c].steps;
  }
  std::vector<int> chain_off(ch.size());
  for(size_t c = 0; c < ch.size(); ++c) {
    const int mp = ch[c].mp, m = ch[c].m;
    chain_off[c] = (int)td.size();
    double bin = 1.0;
    for(int u = 1; u <= mp + m; ++u)
      bin = bin * double(mp - m + u) / double(u);
    td.push_back((((mp - m) & 1) ? -1.0 : 1.0) * std::sqrt(bin));
    for(int n = mp + 1; n <= nmax; ++n) {
      const double A = double(n) * (2 * n - 1) / std::sqrt(double(n * n - m * m) * double(n * n - mp * mp));
      double A2 = 0.0, A3 = 0.0;
      if(n > 1) {
        A2 = A * double(m * mp) / (double(n) * (n - 1));
        A3 = A * std::sqrt(double((n - 1) * (n - 1) - m * m) * double((n - 1) * (n - 1) - mp * mp)) /
             (double(n - 1) * (2 * n - 1));
      }
      td.push_back(A);
      td.push_back(A2);
      td.push_back(A3);
    }
  }
  if(td.size() >= (1u << 15))
    throw std::runtime_error("rotation tables: Wigner coefficients exceed the packed offset");
  ti.assign(nwl + 1, 0);
  int pos = 0;
  std::vector<int> list;
  for(int k = 0; k < nwl; ++k) {
    ti[k] = pos;
    for(int c : lane[k]) {
      list.push_back(ch[c].mp | ((ch[c].m + 128) << 8) | (chain_off[c] << 16));
      ++pos;
    }
  }
  ti[nwl] = pos;
  ti.insert(ti.end(), list.begin(), list.end());
  // --- the z-axis map ---
  const int L = 2 * nmax;
  std::vector<int> off(2 * nmax + 2);
  int ncomp = 0;
  for(int m = -nmax; m <= nmax; ++m) {
    off[m + nmax] = ncomp;
    const int w = nmax - std::abs(m) + 1;
    ncomp += w * w;
  }
  auto cidx_h = [&](int m, int n, int l) {
    const int am = std::abs(m);
    return off[m + nmax] + (n - am) * (nmax - am + 1) + (l - am);
  };
  // coefficient C^p of alpha(n, mu, l, mu), mu >= 0, n <= nMax, l <= nMax
  std::vector<double> C((size_t)(nmax + 1) * (nmax + 1) * (nmax + 1) * (L + 1), 0.0);
  auto Cat = [&](int n, int mu, int l, int p) -> double & {
    return C[(((size_t)n * (nmax + 1) + mu) * (nmax + 1) + l) * (L + 1) + p];
  };
  for(int p = 0; p <= L; ++p) {
    std::vector<double> D(L + 2, 0.0), Dn(L + 2), O1(L + 2), O2(L + 2), On(L + 2);
    D[p] = 1.0;
    for(int mu = 0; mu <= nmax; ++mu) {
      if(mu > 0) {
        for(int l = 0; l <= L; ++l) {
          const double dm = l >= 1 ? D[l - 1] : 0.0, dp = D[l + 1];
          Dn[l] = (dm * rb_plus(l - 1, mu - 1) + dp * rb_minus(l + 1, mu - 1)) / rb_plus(mu - 1, mu - 1);
        }
        Dn[L + 1] = 0.0;
        D = Dn;
      }
      for(int l = mu; l <= nmax; ++l)
        Cat(mu, mu, l, p) = D[l];
      O2.assign(L + 2, 0.0);
      O1 = D;
      for(int n = mu + 1; n <= nmax; ++n) {
        for(int l = 0; l <= L; ++l) {
          const double om = l >= 1 ? O1[l - 1] : 0.0, op = O1[l + 1];
          On[l] = (om * ra_plus(l - 1, mu) + op * ra_minus(l + 1, mu) - O2[l] * ra_minus(n - 1, mu)) /
                  ra_plus(n - 1, mu);
        }
        On[L + 1] = 0.0;
        O2 = O1;
        O1 = On;
        for(int l = mu; l <= nmax; ++l)
          Cat(n, mu, l, p) = On[l];
      }
    }
  }
  struct Ent {
    int ip, im, p0, cnt, odd;
    std::vector<double> c;
  };
  std::vector<Ent> es;
  for(int mu = 0; mu <= nmax; ++mu)
    for(int n = std::max(mu, 1); n <= nmax; ++n)
      for(int l = mu; l <= nmax; ++l) {
        Ent e;
        e.ip = cidx_h(mu, n, l);
        e.im = cidx_h(-mu, n, l);
        e.p0 = std::abs(n - l);
        e.cnt = std::min(n, l) + 1;
        e.odd = (n + l) & 1;
        for(int q = 0; q < e.cnt; ++q) {
          const int p = e.p0 + 2 * q;
          e.c.push_back(Cat(n, mu, l, p) * ((p & 1) ? -1.0 : 1.0) * std::sqrt(2.0 * p + 1.0));
        }
        es.push_back(e);
      }
  std::stable_sort(es.begin(), es.end(), [](const Ent &x, const Ent &y) { return x.cnt > y.cnt; });
  while(ti.size() % 4)  // int4-aligned entries
    ti.push_back(0);
  ent_base = (int)ti.size();
  nent = (int)es.size();
  for(const Ent &e : es) {
    ti.push_back(e.ip | (e.im << 16));
    ti.push_back(e.p0 | (e.cnt << 8) | (e.odd << 16));
    ti.push_back((int)td.size());
    ti.push_back(0);
    td.insert(td.end(), e.c.begin(), e.c.end());
  }
  // --- Az / Bz formation (Coupling.cpp:30-51 with k = m) ---
  onl_base = (int)ti.size();
  ti.resize(ti.size() + (size_t)(nmax + 1) * (nmax + 1), 0);
  const int zero = ncomp;
  auto al = [&](int n, int m, int l) {  // alpha(n, m, l, m) index, or the zero slot
    if(l < 0 || std::abs(m) > n || std::abs(m) > l)
      return zero;
    return cidx_h(m, n, l);
  };
  auto pack = [](int a, int b) {
    const int v = a | (b << 16);
    float f;
    std::memcpy(&f, &v, 4);
    return f;
  };
  int e = 0;
  for(int n = 1; n <= nmax; ++n)
    for(int l = 1; l <= nmax; ++l) {
      ti[onl_base + n * (nmax + 1) + l] = e;
      const int mn = std::min(n, l);
      for(int m = -mn; m <= mn; ++m, ++e) {
        // factors: qf / pf of coef_tables for q = (n, m), p = (l, m)
        const double g = 0.5 / std::sqrt(double(n * (n + 1)));
        const double q0 = g * std::sqrt(double((n - m) * (n + m + 1))), q1 = g * std::sqrt(double((n + m) * (n - m + 1))),
                     q2 = g * 2 * m;
        const double gl = 1.0 / std::sqrt(double(l * (l + 1)));
        const double hB = std::sqrt(double(2 * l + 1) / double((2 * l - 1) * l * (l + 1)));
        const double p0 = gl * std::sqrt(double((l - m) * (l + m + 1))), p1 = gl * std::sqrt(double((l + m) * (l - m + 1))),
                     p2 = gl * m, p3 = hB * std::sqrt(double((l - m) * (l + m))),
                     p4 = hB * std::sqrt(double((l - m) * (l - m - 1))), p5 = hB * std::sqrt(double((l + m) * (l + m - 1)));
        const int t0 = al(n, m, l);
        const int tp = (m < n && m < l) ? al(n, m + 1, l) : zero;
        const int tm = (m > -n && m > -l) ? al(n, m - 1, l) : zero;
        const int lm = l - 1;
        const int u0 = (std::abs(m) <= lm) ? al(n, m, lm) : zero;
        const int up = (m < n && std::abs(m + 1) <= lm) ? al(n, m + 1, lm) : zero;
        const int um = (m > -n && std::abs(m - 1) <= lm) ? al(n, m - 1, lm) : zero;
        tz.push_back(pack(t0, tp));
        tz.push_back(pack(tm, u0));
        tz.push_back(pack(up, um));
        tz.push_back(0.f);
        tz.push_back((float)(q2 * p2));
        tz.push_back((float)(q0 * p0));
        tz.push_back((float)(q1 * p1));
        tz.push_back((float)(q2 * p3));
        tz.push_back((float)(q0 * p4));
        tz.push_back((float)(q1 * p5));
        tz.push_back(0.f);
        tz.push_back(0.f);
      }
    }
  if(ncomp >= (1 << 15))
    throw std::runtime_error("rotation tables: alpha indices exceed the packed width");
}

int rot_smem_bytes(int nmax) { return rot_layout(nmax).bytes; }

void launch_assemble_rot(om_problem *pr, int harmonic) {
  om_context *ctx = pr->ctx;
  RotArgs a = rot_args(ctx, pr->nmax);
  a.cart = pr->d_cart;
  a.T = harmonic == OM_SH ? pr->d_Tsh : pr->d_T;
  a.N = pr->N;
  const cplx k = harmonic == OM_SH ? 2.0 * pr->waveK : pr->waveK;
  a.waveK = mk(k.real(), k.imag());
  a.ld = pr->n;
  a.items = (long)pr->N * (pr->N - 1) / 2 + pr->N;
  const int bytes = rot_layout(pr->nmax).bytes;
  set_rot_smem(ctx);
  const dim3 grid((unsigned)((a.items + kPPC - 1) / kPPC));
  timer_begin(ctx, ctx->ev_asm);
  cudaEventRecord(ctx->ev_fork, ctx->stream);
  cudaStreamWaitEvent(ctx->stream_lo, ctx->ev_fork, 0);
  k_assemble_rot<<<grid, kRotThreads, bytes, ctx->stream_lo>>>(a, (float2 *)pr->d_S32[harmonic]);
  cudaEventRecord(ctx->ev_join, ctx->stream_lo);
  cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0);
  timer_end(ctx, ctx->ev_asm);
  ctx->last_launches++;
}

void launch_assemble_rot_batch(om_context *ctx, int nmax, const BatchMat *d_mats, int nmats, int per_mat,
                               cudaStream_t stream) {
  RotArgs a = rot_args(ctx, nmax);
  a.batch = d_mats;
  a.per_mat = per_mat;
  a.items = (long)nmats * per_mat;
  const int bytes = rot_layout(nmax).bytes;
  set_rot_smem(ctx);
  const dim3 grid((unsigned)((a.items + kPPC - 1) / kPPC));
  k_assemble_rot<<<grid, kRotThreads, bytes, stream>>>(a, nullptr);
  ctx->last_launches++;
}

}  // namespace om
