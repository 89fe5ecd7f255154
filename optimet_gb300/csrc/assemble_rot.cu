// Precision-form assembly of the scattering matrix by rotations.
//
// The coupling blocks of a displacement R = (r, theta, phi) are rotated z-axis
// translations: A(R) = U A(r z) U^H and B(R) = U B(r z) U^H, with U block
// diagonal over the degree n, U[(n, m'), (n, m)] = d^n_{m'm}(theta) e^{i m' phi}
// (Wigner small-d), and the z-axis blocks A(r z), B(r z) diagonal in m. Only the
// d = m - k = 0 slice of the Stout recurrences
// (TranslationAdditionCoefficients.cpp:71-124) survives on the z axis, so one
// recurrence chain per pair replaces the 3 nMax + 1 chains of the general
// translation. The block of S (PreconditionedMatrix.cpp:369-397) is then
//
//   S_ij[(l,k'), (n,m')] = -T_i(l) e^{i(m'-k')phi} sum_m d^n_{m'm} Az_m(n,l) d^l_{k'm}
//
// (B likewise, on the TM/TE off-diagonal blocks), and S_ji follows from the
// parity A(-R) = (-1)^{n+l} A(R), B(-R) = -(-1)^{n+l} B(R).
//
// One CTA of 128 threads per unordered sphere pair i < j:
//  1. FP64: the Hankel seeds alpha(0,0,l,0) = (-1)^l sqrt(2l+1) h_l(k r) for
//     l <= 2 nMax, the d = 0 chain on one warp (lanes over l, shuffles for
//     l +- 1), and, on the other warps at the same time, the Wigner d^n(theta)
//     for n <= nMax by the three-term recurrence in n over the wedge
//     m' >= |m| (the rest by the symmetries of d);
//  2. FP64: Az, Bz from the chain (the coupling formulas of Coupling.cpp:30-51
//     with k = m), rounded once to complex64;
//  3. FP32: the rotation products, register-blocked over up to 9 column
//     harmonics m' of one degree n per thread and row p, then scaled by
//     -T_i(l) and the phases and stored column by column (coalesced rows) for
//     S_ij and S_ji.
// The last N CTAs write the identity diagonal blocks.
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

#include "om_internal.h"

namespace om {

namespace {

constexpr int kRotThreads = 128;
constexpr int kChunk = 9;     // column harmonics m' per thread (register block)
constexpr int kMaxGroups = 48;

// Recurrence coefficient table of the Stout chains (same layout as the
// translation kernel's: 6 doubles per (n, m), n <= 2 nMax + 1).
enum { kAP = 0, kAM = 1, kBP = 2, kBM = 3, kRAP = 4, kRBP = 5, kRecStride = 6 };

struct RotArgs {
  const double *cart;
  const zd *T;  // N x (nmax+1) x 2
  const double *rec, *qf, *pf, *wig;
  int N, nmax;
  zd waveK;
  long ld;
  const BatchMat *batch;
  int per_mat;
  int ngroups;
  signed char gn[kMaxGroups], gm0[kMaxGroups], gcnt[kMaxGroups];
};

// Shared-memory layout (bytes), the same on host and device.
struct RotLayout {
  int ncomp;   // compact (m, n, l) entries: |m| <= n, l <= nMax
  int nw;      // Wigner entries: sum_{n=1}^{nMax} (2n+1)^2
  int o_alz, o_az, o_bz, o_w, o_e, o_t, o_off, o_wo, o_geo, o_hk, o_grp;
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
  int nw = 0;
  for(int n = 1; n <= nmax; ++n)
    nw += (2 * n + 1) * (2 * n + 1);
  y.nw = nw;
  int o = 0;
  auto take = [&](int bytes) {
    const int at = o;
    o += (bytes + 15) & ~15;
    return at;
  };
  y.o_alz = take(16 * nc);
  y.o_az = take(8 * nc);
  y.o_bz = take(8 * nc);
  y.o_w = take(4 * nw);
  y.o_e = take(8 * (2 * nmax + 1));
  y.o_t = take(8 * 4 * (nmax + 1));
  y.o_off = take(4 * (2 * nmax + 2));
  y.o_wo = take(4 * (nmax + 2));
  y.o_geo = take(8 * 8);
  y.o_hk = take(16 * 2 * (2 * nmax + 2));
  y.o_grp = take(4 * kMaxGroups);
  y.bytes = o;
  return y;
}

__device__ __forceinline__ double rc(const double *rec, int Lc, int n, int m, int which) {
  if(n < 0 || n > Lc || m > n || m < -n)
    return 0.0;
  return __ldg(rec + kRecStride * (n * n + n + m) + which);
}

__device__ __forceinline__ zd shfl_up_z(zd v) {
  return mk(__shfl_up_sync(0xffffffffu, v.re, 1), __shfl_up_sync(0xffffffffu, v.im, 1));
}
__device__ __forceinline__ zd shfl_down_z(zd v) {
  return mk(__shfl_down_sync(0xffffffffu, v.re, 1), __shfl_down_sync(0xffffffffu, v.im, 1));
}

// Index of (m, n, l) in the compact tables, |m| <= n, l <= nMax.
__device__ __forceinline__ int cidx(const int *off, int nmax, int m, int n, int l) {
  const int am = m < 0 ? -m : m;
  return off[m + nmax] + (n - am) * (nmax - am + 1) + (l - am);
}

// The d = 0 Stout chain on the z axis (one full warp, lane = l <= 2 nMax):
// alpha(n, mu, l, mu) for 0 <= mu <= n <= nMax, l <= nMax. `neg` selects the
// conjugate-wave chain of a complex wave number (TranslationAdditionCoefficients.h:72-74),
// whose results are the m < 0 entries (-1)^{n+l} conj(alpha_neg); for a real
// wave number the m < 0 entries equal the m > 0 ones (d = 0, irregular).
__device__ void zchain(zd *alz, const int *off, const double *rec, const zd *hk, int nmax, bool neg,
                       bool real_k) {
  const int L = 2 * nmax, Lc = 2 * nmax + 1;
  const int l = threadIdx.x & 31;
  zd D = mk(0.0, 0.0);
  if(l <= L) {
    const double f = ((l & 1) ? -1.0 : 1.0) * sqrt(2.0 * l + 1.0);
    D = f * hk[l];
  }
  auto store = [&](int n, int mu, zd v) {
    if(n < 1 || l > nmax || mu > l)
      return;
    if(!neg) {
      alz[cidx(off, nmax, mu, n, l)] = v;
      if(mu > 0 && real_k)
        alz[cidx(off, nmax, -mu, n, l)] = v;
    } else if(mu > 0) {
      zd w = conj(v);
      if((n + l) & 1)
        w = -w;
      alz[cidx(off, nmax, -mu, n, l)] = w;
    }
  };
  for(int mu = 0; mu <= nmax; ++mu) {
    if(mu > 0) {
      const zd Dm = shfl_up_z(D), Dp = shfl_down_z(D);
      const double bp = rc(rec, Lc, l - 1, mu - 1, kBP);
      const double bm = rc(rec, Lc, l + 1, mu - 1, kBM);
      const double rden = rc(rec, Lc, mu - 1, mu - 1, kRBP);
      zd Dn;
      Dn.re = fma(Dm.re, bp, Dp.re * bm) * rden;
      Dn.im = fma(Dm.im, bp, Dp.im * bm) * rden;
      D = (l <= L) ? Dn : mk(0.0, 0.0);
    }
    store(mu, mu, D);
    zd O2 = mk(0.0, 0.0), O1 = D;
    const double apl = rc(rec, Lc, l - 1, mu, kAP);
    const double aml = rc(rec, Lc, l + 1, mu, kAM);
    for(int n = mu + 1; n <= nmax; ++n) {
      const zd Om = shfl_up_z(O1), Op = shfl_down_z(O1);
      const double amn = rc(rec, Lc, n - 1, mu, kAM);
      const double rapn = rc(rec, Lc, n - 1, mu, kRAP);
      zd On;
      On.re = fma(Om.re, apl, fma(Op.re, aml, -O2.re * amn)) * rapn;
      On.im = fma(Om.im, apl, fma(Op.im, aml, -O2.im * amn)) * rapn;
      if(l > L)
        On = mk(0.0, 0.0);
      O2 = O1;
      O1 = On;
      store(n, mu, On);
    }
  }
}

// Wigner table offsets of the FP64 coefficient array `wig` (built on the host
// per nMax, see wigner_tables):
//   sq[j][a]  = sqrt(j^2 - a^2)            at j (nMax+1) + a
//   rs[j][a]  = 1 / sqrt(j^2 - a^2), a < j at (nMax+1)^2 + j (nMax+1) + a
//   cj[j]     = {j (2j-1), 1/(j (j-1)), 1/((j-1)(2j-1))} at 2 (nMax+1)^2 + 3 j
//   bin[m'][m] = sqrt(C(2m', m'+m))        at 2 (nMax+1)^2 + 3 (nMax+1) + m' (2 nMax+1) + m + nMax
//
// One wedge chain (m', m), m' >= |m|: d^n_{m'm} for n = m' .. nMax, started
// from d^{m'}_{m'm} = (-1)^{m'-m} sqrt(C(2m', m'+m)) c^{m'+m} s^{m'-m}
// (c, s = cos, sin of theta/2) and continued by
//   d^j = j(2j-1) / sqrt((j^2-m^2)(j^2-m'^2)) *
//         [ (cos theta - m m' / (j(j-1))) d^{j-1}
//           - sqrt(((j-1)^2-m^2)((j-1)^2-m'^2)) / ((j-1)(2j-1)) d^{j-2} ].
// Each value goes to the four table places the symmetries of d give:
// d_{m'm} = d_{-m,-m'} = (-1)^{m'-m} d_{m m'} = (-1)^{m'-m} d_{-m',-m}.
// Table layout: d^n_{m'm} at wo[n] + (m + n)(2n + 1) + (m' + n) (m' fastest).
__device__ void wigner_chain(float *W, const int *wo, const double *wig, int nmax, int mp, int m,
                             double ct, double c, double s) {
  const int S = nmax + 1;
  const double *sq = wig, *rs = wig + S * S, *cj = wig + 2 * S * S, *bin = wig + 2 * S * S + 3 * S;
  const int am = m < 0 ? -m : m;
  double v = __ldg(bin + mp * (2 * nmax + 1) + m + nmax);
  for(int i = 0; i < mp + m; ++i)
    v *= c;
  for(int i = 0; i < mp - m; ++i)
    v *= s;
  if((mp - m) & 1)
    v = -v;
  const double sg = ((mp - m) & 1) ? -1.0 : 1.0;
  auto put = [&](int n, double d) {
    const int w = 2 * n + 1, b = wo[n];
    const float f = (float)d, g = (float)(sg * d);
    W[b + (m + n) * w + (mp + n)] = f;    // d_{m' m}
    W[b + (-mp + n) * w + (-m + n)] = f;  // d_{-m, -m'}
    W[b + (mp + n) * w + (m + n)] = g;    // d_{m m'}
    W[b + (-m + n) * w + (-mp + n)] = g;  // d_{-m', -m}
  };
  if(mp >= 1)
    put(mp, v);
  double prev = 0.0, cur = v;
  for(int j = mp + 1; j <= nmax; ++j) {
    const double a = __ldg(cj + 3 * j) * __ldg(rs + j * S + am) * __ldg(rs + j * S + mp);
    double t1 = ct, b = 0.0;
    if(j > 1) {
      t1 -= (double)(m * mp) * __ldg(cj + 3 * j + 1);
      b = __ldg(sq + (j - 1) * S + am) * __ldg(sq + (j - 1) * S + mp) * __ldg(cj + 3 * j + 2);
    }
    const double nx = a * fma(t1, cur, -b * prev);
    prev = cur;
    cur = nx;
    put(j, nx);
  }
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__global__ void __launch_bounds__(kRotThreads, 4) k_assemble_rot(RotArgs a, float2 *S) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int nmax = a.nmax;
  const RotLayout y = rot_layout(nmax);
  zd *alz = reinterpret_cast<zd *>(sm + y.o_alz);
  float2 *az = reinterpret_cast<float2 *>(sm + y.o_az);
  float2 *bz = reinterpret_cast<float2 *>(sm + y.o_bz);
  float *W = reinterpret_cast<float *>(sm + y.o_w);
  float2 *E = reinterpret_cast<float2 *>(sm + y.o_e);
  float2 *Tl = reinterpret_cast<float2 *>(sm + y.o_t);
  int *off = reinterpret_cast<int *>(sm + y.o_off);
  int *wo = reinterpret_cast<int *>(sm + y.o_wo);
  double *geo = reinterpret_cast<double *>(sm + y.o_geo);
  zd *hk = reinterpret_cast<zd *>(sm + y.o_hk);
  int *grp = reinterpret_cast<int *>(sm + y.o_grp);

  const double *cart = a.cart;
  const zd *Tg = a.T;
  int N = a.N;
  zd waveK = a.waveK;
  long ld = a.ld;
  long b = blockIdx.x;
  if(a.batch) {
    const BatchMat &bm = a.batch[blockIdx.x / a.per_mat];
    b = blockIdx.x % a.per_mat;
    cart = bm.cart;
    Tg = bm.T;
    N = bm.N;
    waveK = bm.waveK;
    ld = bm.ld;
    S = (float2 *)bm.S;
    if(b >= (long)N * (N + 1) / 2)  // idle: padding of the size class or an empty entry
      return;
  }
  const int P = nmax * (nmax + 2);
  const long npairs = (long)N * (N - 1) / 2;
  const int t = threadIdx.x;
  if(b >= npairs) {
    const int i = (int)(b - npairs);
    const size_t x0 = 2ul * P * i;
    for(int idx = t; idx < 4 * P * P; idx += blockDim.x) {
      const int c = idx / (2 * P), r = idx - c * 2 * P;
      S[(x0 + c) * (size_t)ld + x0 + r] = make_float2(r == c ? 1.f : 0.f, 0.f);
    }
    return;
  }
  // b -> (i, j), i < j: b = j (j - 1) / 2 + i
  int j = (int)((1.0 + sqrt(1.0 + 8.0 * (double)b)) * 0.5);
  while((long)j * (j - 1) / 2 > b)
    --j;
  while((long)(j + 1) * j / 2 <= b)
    ++j;
  const int i = (int)(b - (long)j * (j - 1) / 2);
  const bool real_k = waveK.im == 0.0;

  // --- set-up: geometry, offsets, T factors, phase table ---
  if(t == 0) {
    double r, th, ph;
    to_spherical(cart[3 * i] - cart[3 * j], cart[3 * i + 1] - cart[3 * j + 1],
                 cart[3 * i + 2] - cart[3 * j + 2], &r, &th, &ph);
    geo[0] = r;
    geo[1] = th;
    geo[2] = ph;
    geo[3] = cos(th);
    sincos(0.5 * th, &geo[5], &geo[4]);
    int o = 0;
    for(int m = -nmax; m <= nmax; ++m) {
      off[m + nmax] = o;
      const int w = nmax - (m < 0 ? -m : m) + 1;
      o += w * w;
    }
    int q = 0;
    wo[0] = 0;
    for(int n = 1; n <= nmax; ++n) {
      wo[n] = q;
      q += (2 * n + 1) * (2 * n + 1);
    }
  }
  if(t < a.ngroups)
    grp[t] = (int)a.gn[t] | ((int)(unsigned char)a.gm0[t] << 8) | ((int)a.gcnt[t] << 16);
  const int nT = 2 * (nmax + 1);
  for(int u = t; u < 2 * nT; u += blockDim.x) {
    const zd v = Tg[(size_t)(u < nT ? i : j) * nT + (u < nT ? u : u - nT)];
    Tl[u] = make_float2((float)v.re, (float)v.im);
  }
  __syncthreads();
  const double r = geo[0], ph = geo[2];
  if(t < 2 * nmax + 1) {
    double sn, cs;
    sincos((double)(t - nmax) * ph, &sn, &cs);
    E[t] = make_float2((float)cs, (float)sn);
  }
  // Hankel seeds: warp 0 lane 0 for the wave, warp 1 lane 0 for the
  // conjugate wave of a complex wave number (k -> -conj(k))
  const int warp = t >> 5;
  if((t == 0) || (t == 32 && !real_k)) {
    const zd k = (t == 0) ? waveK : -conj(waveK);
    zd f[kMaxOrder + 2];
    sph_h1(r * k, 2 * nmax, f);
    zd *dst = hk + (t == 0 ? 0 : (2 * nmax + 2));
    for(int l = 0; l <= 2 * nmax; ++l)
      dst[l] = f[l];
  }
  __syncthreads();

  // --- FP64: the z-axis chain(s) and, beside them, the Wigner wedge ---
  const int chain_warps = real_k ? 1 : 2;
  if(warp == 0) {
    zchain(alz, off, a.rec, hk, nmax, false, real_k);
  } else if(warp == 1 && !real_k) {
    zchain(alz, off, a.rec, hk + (2 * nmax + 2), nmax, true, real_k);
  } else {
    const double ct = geo[3], c2 = geo[4], s2 = geo[5];
    const int nwedge = (nmax + 1) * (nmax + 1);
    for(int c = t - 32 * chain_warps; c < nwedge; c += blockDim.x - 32 * chain_warps) {
      const int mp = (int)sqrtf((float)c);  // c = mp^2 + (m + mp)
      int mpp = mp;
      while(mpp * mpp > c)
        --mpp;
      while((mpp + 1) * (mpp + 1) <= c)
        ++mpp;
      const int m = c - mpp * mpp - mpp;
      wigner_chain(W, wo, a.wig, nmax, mpp, m, ct, c2, s2);
    }
  }
  __syncthreads();

  // --- FP64: the z-axis coupling blocks (Coupling.cpp:30-51, k = m), rounded once ---
  for(int e = t; e < y.ncomp; e += blockDim.x) {
    int m = -nmax;
    while(m < nmax && off[m + 1 + nmax] <= e)
      ++m;
    const int am = m < 0 ? -m : m, w = nmax - am + 1;
    const int rel = e - off[m + nmax];
    const int n = am + rel / w, l = am + rel % w;
    if(n < 1 || l < 1) {
      az[e] = make_float2(0.f, 0.f);
      bz[e] = make_float2(0.f, 0.f);
      continue;
    }
    const double *qf = a.qf + kQfacStride * flat(n, m);
    const double *pf = a.pf + kPfacStride * flat(l, m);
    const double q0 = __ldg(qf), q1 = __ldg(qf + 1), q2 = __ldg(qf + 2);
    const zd t0 = alz[cidx(off, nmax, m, n, l)];
    const zd tp = (m < n && m < l) ? alz[cidx(off, nmax, m + 1, n, l)] : mk(0.0, 0.0);
    const zd tm = (m > -n && m > -l) ? alz[cidx(off, nmax, m - 1, n, l)] : mk(0.0, 0.0);
    const double f0 = q2 * __ldg(pf + 2), f1 = q0 * __ldg(pf), f2 = q1 * __ldg(pf + 1);
    const zd A = f0 * t0 + f1 * tp + f2 * tm;
    const int lm = l - 1;
    const zd u0 = (am <= lm) ? alz[cidx(off, nmax, m, n, lm)] : mk(0.0, 0.0);
    const zd up = (m < n && abs(m + 1) <= lm) ? alz[cidx(off, nmax, m + 1, n, lm)] : mk(0.0, 0.0);
    const zd um = (m > -n && abs(m - 1) <= lm) ? alz[cidx(off, nmax, m - 1, n, lm)] : mk(0.0, 0.0);
    const double g0 = q2 * __ldg(pf + 3), g1 = q0 * __ldg(pf + 4), g2 = q1 * __ldg(pf + 5);
    const zd s = g0 * u0 + g1 * up - g2 * um;
    az[e] = make_float2((float)A.re, (float)A.im);
    bz[e] = make_float2((float)s.im, (float)-s.re);  // B = -i s
  }
  __syncthreads();

  // --- FP32: rotation products and the S_ij / S_ji stores ---
  const size_t xi = 2ul * P * i, xj = 2ul * P * j;
  const size_t LD = (size_t)ld;
  const int nitems = a.ngroups * P;
  for(int it = t; it < nitems; it += blockDim.x) {
    const int g = it / P, p = it - g * P;
    const int gv = grp[g];
    const int n = gv & 0xff, m0 = (int)(signed char)((gv >> 8) & 0xff), cnt = gv >> 16;
    // row harmonic p = (l, k'): p = l(l+1) - k' - 1
    int l = (int)sqrtf((float)(p + 1));
    while(l * (l + 1) - l - 1 > p)
      --l;
    while((l + 1) * (l + 2) - (l + 1) - 1 <= p)
      ++l;
    const int kp = l * (l + 1) - 1 - p;
    const int mn = n < l ? n : l;
    float2 accA[kChunk], accB[kChunk];
#pragma unroll
    for(int c = 0; c < kChunk; ++c) {
      accA[c] = make_float2(0.f, 0.f);
      accB[c] = make_float2(0.f, 0.f);
    }
    const float *Wl = W + wo[l] + (kp + l);
    const float *Wn = W + wo[n] + (m0 + n);
    for(int m = -mn; m <= mn; ++m) {
      const float dl = Wl[(m + l) * (2 * l + 1)];
      const int e = cidx(off, nmax, m, n, l);
      const float2 va = az[e], vb = bz[e];
      const float2 xa = make_float2(va.x * dl, va.y * dl), xb = make_float2(vb.x * dl, vb.y * dl);
      const float *wn = Wn + (m + n) * (2 * n + 1);
#pragma unroll
      for(int c = 0; c < kChunk; ++c) {
        if(c < cnt) {
          const float dn = wn[-c];  // m' = m0 - c
          accA[c].x = fmaf(dn, xa.x, accA[c].x);
          accA[c].y = fmaf(dn, xa.y, accA[c].y);
          accB[c].x = fmaf(dn, xb.x, accB[c].x);
          accB[c].y = fmaf(dn, xb.y, accB[c].y);
        }
      }
    }
    // row factors -T(l) e^{-i k' phi}; S_ji's carry the parity: -(-1)^{n+l} T_j(l) e^{-i k' phi}
    const float2 ek = E[nmax - kp];
    const float2 tei = Tl[2 * l], tmi = Tl[2 * l + 1], tej = Tl[nT + 2 * l], tmj = Tl[nT + 2 * l + 1];
    const float sgn = ((n + l) & 1) ? 1.f : -1.f;  // -(-1)^{n+l}
    const float2 ci_te = cmulf(make_float2(-tei.x, -tei.y), ek);
    const float2 ci_tm = cmulf(make_float2(-tmi.x, -tmi.y), ek);
    const float2 cj_te = cmulf(make_float2(sgn * tej.x, sgn * tej.y), ek);
    const float2 cj_tm = cmulf(make_float2(sgn * tmj.x, sgn * tmj.y), ek);
#pragma unroll
    for(int c = 0; c < kChunk; ++c) {
      if(c < cnt) {
        const int mp = m0 - c;
        const int q = n * (n + 1) - mp - 1;
        const float2 em = E[nmax + mp];
        const float2 A = cmulf(em, accA[c]), B = cmulf(em, accB[c]);
        const size_t cte_i = (xj + q) * LD + xi, ctm_i = (xj + P + q) * LD + xi;
        S[cte_i + p] = cmulf(ci_te, A);
        S[ctm_i + P + p] = cmulf(ci_tm, A);
        S[ctm_i + p] = cmulf(ci_te, B);
        S[cte_i + P + p] = cmulf(ci_tm, B);
        // S_ji: A -> (-1)^{n+l} A, B -> -(-1)^{n+l} B, rows of sphere j
        const size_t cte_j = (xi + q) * LD + xj, ctm_j = (xi + P + q) * LD + xj;
        S[cte_j + p] = cmulf(cj_te, A);
        S[ctm_j + P + p] = cmulf(cj_tm, A);
        S[ctm_j + p] = cmulf(make_float2(-cj_te.x, -cj_te.y), B);
        S[cte_j + P + p] = cmulf(make_float2(-cj_tm.x, -cj_tm.y), B);
      }
    }
  }
}

// Column groups: per degree n, the 2n+1 harmonics m' = n .. -n split into
// ceil((2n+1)/9) near-equal runs.
void fill_groups(RotArgs &a, int nmax) {
  int g = 0;
  for(int n = 1; n <= nmax; ++n) {
    const int w = 2 * n + 1;
    const int nch = (w + kChunk - 1) / kChunk;
    const int sz = (w + nch - 1) / nch;
    int m0 = n;
    for(int c = 0; c < nch; ++c) {
      const int cnt = std::min(sz, m0 + n + 1);
      if(g >= kMaxGroups)
        throw std::runtime_error("rotation assembly: too many column groups");
      a.gn[g] = (signed char)n;
      a.gm0[g] = (signed char)m0;
      a.gcnt[g] = (signed char)cnt;
      ++g;
      m0 -= cnt;
    }
  }
  a.ngroups = g;
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

RotArgs rot_args(om_context *ctx, int nmax) {
  const CoefTables &ct = coef_tables(ctx, nmax);
  RotArgs a{};
  a.rec = ct.rec;
  a.qf = ct.qf;
  a.pf = ct.pf;
  a.wig = ct.wig;
  a.nmax = nmax;
  a.batch = nullptr;
  a.per_mat = 1;
  fill_groups(a, nmax);
  return a;
}

}  // namespace

std::vector<double> wigner_tables(int nmax) {
  const int S = nmax + 1;
  std::vector<double> w(2 * S * S + 3 * S + S * (2 * nmax + 1), 0.0);
  for(int j = 0; j <= nmax; ++j)
    for(int a = 0; a <= j; ++a) {
      w[j * S + a] = std::sqrt(double(j * j - a * a));
      if(a < j)
        w[S * S + j * S + a] = 1.0 / std::sqrt(double(j * j - a * a));
    }
  for(int j = 0; j <= nmax; ++j) {
    double *c = &w[2 * S * S + 3 * j];
    c[0] = double(j) * (2 * j - 1);
    c[1] = j > 1 ? 1.0 / (double(j) * (j - 1)) : 0.0;
    c[2] = j > 1 ? 1.0 / (double(j - 1) * (2 * j - 1)) : 0.0;
  }
  for(int mp = 0; mp <= nmax; ++mp)
    for(int m = -mp; m <= mp; ++m) {
      // C(2m', m'+m) in floating point (exact below 2^53 for nMax <= 15)
      double c = 1.0;
      const int kk = mp + m, nn = 2 * mp;
      for(int u = 1; u <= kk; ++u)
        c = c * double(nn - kk + u) / double(u);
      w[2 * S * S + 3 * S + mp * (2 * nmax + 1) + m + nmax] = std::sqrt(c);
    }
  return w;
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
  const int bytes = rot_layout(pr->nmax).bytes;
  set_rot_smem(ctx);
  const dim3 grid((unsigned)((long)pr->N * (pr->N - 1) / 2 + pr->N));
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
  const int bytes = rot_layout(nmax).bytes;
  set_rot_smem(ctx);
  const dim3 grid((unsigned)((long)nmats * per_mat));
  k_assemble_rot<<<grid, kRotThreads, bytes, stream>>>(a, nullptr);
  ctx->last_launches++;
}

}  // namespace om
