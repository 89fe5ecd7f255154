// Translation-addition coefficients, coupling blocks, scattering-matrix
// assembly and source vector for the OPTIMET sphere path.
//
// One CTA per translation (an ordered sphere pair for the matrix, a sphere
// for the source vector). Inside a CTA:
//  1. seeds alpha(0,0,l,k) = sqrt(4 pi) (-1)^{l+k} Y_l^{-k}(theta,phi) z_l(kR) for
//     l <= 2 nMax (TranslationAdditionCoefficients.cpp:102-111);
//  2. the Stout recurrences (:113-124). Both the diagonal recurrence
//     (n,n,l,k) <- (n-1,n-1,l+-1,k-1) and the off-diagonal one
//     (n,m,l,k) <- (n-1,m,l+-1,k), (n-2,m,l,k) keep d = m - k fixed, so each
//     "slice" d is an independent chain: one warp per chain, lanes over l,
//     warp shuffles for the l+-1 neighbours, state in registers. Negative m
//     comes from the conjugate-wave chains (:128-135). Results with l <= nMax
//     go to a shared-memory table alpha[(n,m)][(l,k)];
//  3. A and B (Coupling.cpp:30-51) are formed from that table and, for the
//     matrix, scaled by -T_i and written as the 2P x 2P block of S
//     (PreconditionedMatrix.cpp:369-397) with coalesced column stores.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <stdexcept>
#include <type_traits>

#include "om_internal.h"

namespace om {

namespace {

// --- host coefficient formulas (TranslationAdditionCoefficients.cpp:34-61) ---
bool valid2(int n, int m) { return n >= 0 && std::abs(m) <= n; }
double h_a_plus(int n, int m) {
  if(!valid2(n, m))
    return 0e0;
  return -std::sqrt(static_cast<double>((n + m + 1) * (n - m + 1)) /
                    static_cast<double>((2 * n + 1) * (2 * n + 3)));
}
double h_a_minus(int n, int m) {
  if(!valid2(n, m))
    return 0e0;
  return std::sqrt(static_cast<double>((n + m) * (n - m)) /
                   static_cast<double>((2 * n + 1) * (2 * n - 1)));
}
double h_b_plus(int n, int m) {
  if(!valid2(n, m))
    return 0e0;
  return std::sqrt(static_cast<double>((n + m + 2) * (n + m + 1)) /
                   static_cast<double>((2 * n + 1) * (2 * n + 3)));
}
double h_b_minus(int n, int m) {
  if(!valid2(n, m))
    return 0e0;
  return std::sqrt(static_cast<double>((n - m) * (n - m - 1)) /
                   static_cast<double>((2 * n + 1) * (2 * n - 1)));
}

enum { kAP = 0, kAM = 1, kBP = 2, kBM = 3, kRAP = 4, kRBP = 5, kRecStride = 6 };

// Shared-memory layout of a translation CTA (offsets in doubles).
struct Layout {
  int nmax, P, L, Lc, W;
  int rec, qf, pf, leg, legc, eph, geo, zb, seed, tl, qf32, pf32, tl32, tab;
  int rows_cap;
  int tab_elem;  // bytes per table entry: 16 (complex128) or 8 (complex64, precision form)
  int qf_global; // the factor tables qf / pf stay in global memory (large nMax)
  size_t bytes;
};

Layout make_layout_with(int nmax, size_t smem_limit, bool mixed, bool qf_global) {
  Layout y;
  y.tab_elem = mixed ? 8 : 16;
  y.nmax = nmax;
  y.P = pmax(nmax);
  y.L = 2 * nmax;
  y.Lc = 2 * nmax + 1;
  y.W = (nmax + 1) * (nmax + 1);
  y.qf_global = qf_global ? 1 : 0;
  int o = 0;
  auto take = [&](int n) {
    int at = o;
    o += (n + 1) & ~1;  // keep 16-byte alignment for complex entries
    return at;
  };
  y.rec = take(kRecStride * (y.Lc + 1) * (y.Lc + 1));
  y.qf = take(qf_global ? 0 : kQfacStride * y.P);
  y.pf = take(qf_global ? 0 : kPfacStride * y.P);
  y.leg = take((y.L + 1) * (y.L + 2) / 2);
  y.legc = take((y.L + 1) * (y.L + 2));
  y.eph = take(2 * (y.L + 1));
  y.geo = take(8);
  y.zb = take(2 * 2 * (y.L + 1));
  y.seed = take(2 * 2 * (y.L + 1) * (y.L + 1));
  y.tl = take(2 * 2 * 2 * (nmax + 1));  // T of both spheres of a pair
  y.qf32 = mixed ? take((kQfacStride * y.P + 1) / 2) : o;
  y.pf32 = mixed ? take((kPfacStride * y.P + 1) / 2) : o;
  y.tl32 = mixed ? take(2 * 2 * (nmax + 1)) : o;
  y.tab = o;
  size_t fixed = size_t(o) * sizeof(double);
  size_t row_bytes = size_t(y.W) * y.tab_elem;
  size_t avail = smem_limit > fixed ? smem_limit - fixed : 0;
  int cap = (int)std::min<size_t>(avail / row_bytes, (size_t)y.P);
  y.rows_cap = cap;
  y.bytes = fixed + size_t(cap) * row_bytes;
  return y;
}

// Shared-memory layout of the translation kernels. When the top harmonic level
// does not fit next to the tables (nMax >= 14 in FP64), the coefficient
// factor tables are read from global memory instead.
Layout make_layout(int nmax, size_t smem_limit, bool mixed = false) {
  Layout y = make_layout_with(nmax, smem_limit, mixed, false);
  if(y.rows_cap < 2 * nmax + 1)
    y = make_layout_with(nmax, smem_limit, mixed, true);
  return y;
}

// Chunks of whole n-levels whose rows fit the table.
std::vector<std::pair<int, int>> make_chunks(const Layout &y) {
  std::vector<std::pair<int, int>> out;
  int n = 1;
  while(n <= y.nmax) {
    int lo = n, rows = 0;
    while(n <= y.nmax && rows + (2 * n + 1) <= y.rows_cap) {
      rows += 2 * n + 1;
      ++n;
    }
    if(n == lo)
      throw std::runtime_error("shared memory too small for one harmonic level");
    out.push_back({lo, n - 1});
  }
  return out;
}

struct Smem {
  double *rec, *qf, *pf, *leg, *legc, *geo;
  zd *eph, *zb, *seed, *tl, *tab;
  float *qf32, *pf32;
  float2 *tl32;
};

__device__ Smem smem_view(double *base, const Layout &y, const double *gqf, const double *gpf) {
  Smem s;
  s.rec = base + y.rec;
  s.qf = y.qf_global ? const_cast<double *>(gqf) : base + y.qf;
  s.pf = y.qf_global ? const_cast<double *>(gpf) : base + y.pf;
  s.leg = base + y.leg;
  s.legc = base + y.legc;
  s.eph = reinterpret_cast<zd *>(base + y.eph);
  s.geo = base + y.geo;
  s.qf32 = reinterpret_cast<float *>(base + y.qf32);
  s.pf32 = reinterpret_cast<float *>(base + y.pf32);
  s.tl32 = reinterpret_cast<float2 *>(base + y.tl32);
  s.zb = reinterpret_cast<zd *>(base + y.zb);
  s.seed = reinterpret_cast<zd *>(base + y.seed);
  s.tl = reinterpret_cast<zd *>(base + y.tl);
  s.tab = reinterpret_cast<zd *>(base + y.tab);
  return s;
}

__device__ __forceinline__ double rcoef(const Smem &s, int Lc, int n, int m, int which) {
  if(n < 0 || n > Lc || m > n || m < -n)
    return 0.0;
  return s.rec[kRecStride * (n * n + n + m) + which];
}

__device__ __forceinline__ zd shfl_up1(zd v) {
  return mk(__shfl_up_sync(0xffffffffu, v.re, 1), __shfl_up_sync(0xffffffffu, v.im, 1));
}
__device__ __forceinline__ zd shfl_down1(zd v) {
  return mk(__shfl_down_sync(0xffffffffu, v.re, 1), __shfl_down_sync(0xffffffffu, v.im, 1));
}

// Copy the geometry-independent tables into shared memory.
__device__ void load_tables(const Smem &s, const Layout &y, const double *rec, const double *qf,
                            const double *pf, const double *legc) {
  int nrec = kRecStride * (y.Lc + 1) * (y.Lc + 1);
  for(int i = threadIdx.x; i < nrec; i += blockDim.x)
    s.rec[i] = rec[i];
  for(int i = threadIdx.x; i < (y.L + 1) * (y.L + 2); i += blockDim.x)
    s.legc[i] = legc[i];
  if(y.qf_global)
    return;
  for(int i = threadIdx.x; i < kQfacStride * y.P; i += blockDim.x)
    s.qf[i] = qf[i];
  for(int i = threadIdx.x; i < kPfacStride * y.P; i += blockDim.x)
    s.pf[i] = pf[i];
}

// Seeds for the positive (waveK) and conjugate-wave recurrences.
// geo[0..2] must hold (r, theta, phi) before the call.
__device__ void make_seeds(const Smem &s, const Layout &y, zd waveK, int hankel) {
  const int L = y.L;
  const int t = threadIdx.x;
  const double r = s.geo[0], th = s.geo[1], ph = s.geo[2];
  if(t == 0 || t == 32) {
    zd k = (t == 0) ? waveK : (hankel ? -conj(waveK) : conj(waveK));
    zd z = r * k;
    zd f[kMaxOrder + 2];
    bessel_deriv(hankel ? 1 : 0, z, L, f, nullptr);
    zd *dst = s.zb + (t == 0 ? 0 : (L + 1));
    for(int l = 0; l <= L; ++l)
      dst[l] = f[l];
  }
  if(t >= 64 && t < 64 + L + 1) {
    // normalised associated Legendre functions with the Condon-Shortley phase;
    // legc holds, at l(l+1)/2 + k: {P_kk / sin^k, sqrt(2k+3)} for l = k and
    // {a_lk, b_lk} of the three-term recurrence for l >= k + 2 (host-computed)
    const int k = t - 64;
    const double x = cos(th), st = sin(th);
    double v = s.legc[2 * (k * (k + 1) / 2 + k)];
    for(int i = 1; i <= k; ++i)
      v *= st;
    s.leg[k * (k + 1) / 2 + k] = v;
    if(k + 1 <= L) {
      double v0 = v, v1 = s.legc[2 * (k * (k + 1) / 2 + k) + 1] * x * v;
      s.leg[(k + 1) * (k + 2) / 2 + k] = v1;
      for(int l = k + 2; l <= L; ++l) {
        const double a = s.legc[2 * (l * (l + 1) / 2 + k)];
        const double b = s.legc[2 * (l * (l + 1) / 2 + k) + 1];
        double v2 = a * fma(x, v1, -b * v0);
        s.leg[l * (l + 1) / 2 + k] = v2;
        v0 = v1;
        v1 = v2;
      }
    }
  }
  if(t >= 128 && t < 128 + L + 1) {
    double sn, cs;
    sincos((t - 128) * ph, &sn, &cs);
    s.eph[t - 128] = mk(cs, sn);
  }
  __syncthreads();
  const double s4pi = sqrt(4e0 * kPi);
  for(int idx = t; idx < (L + 1) * (L + 1); idx += blockDim.x) {
    int l = (int)sqrtf((float)idx);
    while(l * l > idx)
      --l;
    while((l + 1) * (l + 1) <= idx)
      ++l;
    int k = idx - l * l - l;  // idx = l*l + l + k
    zd zp = s.zb[l], zn = s.zb[L + 1 + l];
    if(l == 0) {
      s.seed[idx] = zp;
      s.seed[(L + 1) * (L + 1) + idx] = zn;
      continue;
    }
    int am = k < 0 ? -k : k;  // |mu| with mu = -k
    double pre = s.leg[l * (l + 1) / 2 + am];
    const zd e = s.eph[am];
    double re = pre * e.re, im = pre * e.im;
    if(k > 0) {  // mu = -k < 0: Y_l^{-|m|} = (-1)^|m| conj(Y_l^{|m|})
      if(am & 1)
        re = -re;
      else
        im = -im;
    }
    double factor = s4pi * (((l + k) % 2 == 0) ? 1 : -1);
    zd fy = mk(factor * re, factor * im);
    s.seed[idx] = fy * zp;
    s.seed[(L + 1) * (L + 1) + idx] = fy * zn;
  }
  __syncthreads();
}

template <typename T> struct Tab;
template <> struct Tab<zd> {
  static __device__ __forceinline__ zd get(const zd *t, int i) { return t[i]; }
  static __device__ __forceinline__ void put(zd *t, int i, zd v) { t[i] = v; }
};
template <> struct Tab<float2> {
  static __device__ __forceinline__ float2 get(const float2 *t, int i) { return t[i]; }
  static __device__ __forceinline__ void put(float2 *t, int i, zd v) {
    t[i] = make_float2((float)v.re, (float)v.im);
  }
};

template <int W> __device__ __forceinline__ zd shfl_up_w(zd v) {
  return mk(__shfl_up_sync(0xffffffffu, v.re, 1, W), __shfl_up_sync(0xffffffffu, v.im, 1, W));
}
template <int W> __device__ __forceinline__ zd shfl_down_w(zd v) {
  return mk(__shfl_down_sync(0xffffffffu, v.re, 1, W), __shfl_down_sync(0xffffffffu, v.im, 1, W));
}

// The recurrence chains; stores alpha(n, m, l, k) for n in [n_lo, n_hi], l <= nMax.
// For a real wave number the conjugate-wave chains (TranslationAdditionCoefficients.h:72-74)
// follow from the positive ones: regular: alpha_neg = alpha_pos; irregular (Hankel
// h_l(-x) = (-1)^l conj(h_l(x))): alpha_neg(n,m,l,k) = (-1)^{n+l} e^{2 i d phi}
// conj(alpha_pos(n,m,l,k)), d = m - k (the recurrence keeps n + l parity and d);
// only the positive chains then run.
//
// kW = 32: one warp per chain, lane = l <= 2 nMax.
// kW = 16 (nMax <= 8): two chains per warp, lane & 15 = l. Level n >= 1 only
// needs l <= 2 nMax - 1 <= 15; the level-0 neighbours (l up to 16) are read
// from the seed table. Both halves run the same (warp-uniform) loop bounds and
// predicate their stores.
template <int kW, typename TabT>
__device__ void run_chains(const Smem &s, TabT *tab, const Layout &y, int hankel, bool real_k,
                           int n_lo, int n_hi) {
  const int nmax = y.nmax, L = y.L, Lc = y.Lc, W = y.W;
  const int sub = threadIdx.x / kW, nsub = blockDim.x / kW;
  const int l = threadIdx.x & (kW - 1);
  const int npos = 3 * nmax + 1, nneg = real_k ? 0 : 3 * nmax;
  const int nchains = npos + nneg;
  const int base = n_lo * n_lo - 1;  // flat(n_lo, n_lo)
  const double phi = s.geo[2];
  // chains ordered d = 2 nMax .. -nMax (positive), then the conjugate-wave ones,
  // so that neighbouring chains (paired in a warp) have equal loop lengths
  const int rounds = (nchains + nsub - 1) / nsub;
  for(int r = 0; r < rounds; ++r) {
    const int c = sub + r * nsub;
    const bool active = c < nchains;
    const bool neg = active && c >= npos;
    const int d = !active ? 0 : (neg ? 2 * nmax - (c - npos) : 2 * nmax - c);
    const zd *seed = s.seed + (neg ? (L + 1) * (L + 1) : 0);
    auto seed_at = [&](int ll) {
      return (active && ll >= 0 && ll <= L && (d < 0 ? -d : d) <= ll) ? seed[ll * ll + ll - d]
                                                                      : mk(0.0, 0.0);
    };
    double e2s, e2c;
    sincos(-2.0 * d * phi, &e2s, &e2c);
    const zd e2 = mk(e2c, e2s);
    const float2 e2f = make_float2((float)e2c, (float)e2s);
    zd D = seed_at(l);
    const int mu_end = active ? min(min(nmax, d + nmax), n_hi) : -1;
    int mu_end_w = mu_end;
    if(kW == 16)
      mu_end_w = max(mu_end, __shfl_xor_sync(0xffffffffu, mu_end, 16));
    for(int mu = 0; mu <= mu_end_w; ++mu) {
      const int kap = mu - d;
      const bool live = mu <= mu_end;
      if(mu > 0) {
        zd Dm, Dp;
        if(kW == 16 && mu == 1) {
          Dm = seed_at(l - 1);
          Dp = seed_at(l + 1);
        } else {
          Dm = shfl_up_w<kW>(D);
          Dp = shfl_down_w<kW>(D);
        }
        const double bp = rcoef(s, Lc, l - 1, kap - 1, kBP);
        const double bm = rcoef(s, Lc, l + 1, kap - 1, kBM);
        const double rden = rcoef(s, Lc, mu - 1, mu - 1, kRBP);
        zd Dn;
        Dn.re = fma(Dm.re, bp, Dp.re * bm) * rden;
        Dn.im = fma(Dm.im, bp, Dp.im * bm) * rden;
        D = (l <= L) ? Dn : mk(0.0, 0.0);
      }
      // store alpha(n, mu, l, kap) and, from the positive chains of a real
      // wave number, the negative-m image (n, -mu, l, -kap). With a complex64
      // table (precision form) the image is formed in FP32 from the rounded
      // entry: the recurrence stays FP64, only the stored values are FP32.
      auto store = [&](int n, zd v) {
        if(!live || n < n_lo || n > n_hi || l > nmax || kap > l || kap < -l)
          return;
        const int m = -mu, k = -kap;
        const int sign = hankel ? (n + m + l + k) : (k + m);
        if constexpr(std::is_same<TabT, float2>::value) {
          const float2 vf = make_float2((float)v.re, (float)v.im);
          if(!neg)
            tab[(flat(n, mu) - base) * W + l * (l + 1) - kap] = vf;
          if(mu == 0 || (!neg && !real_k))
            return;
          float2 wf;
          if(!neg && hankel) {
            wf = make_float2(fmaf(e2f.x, vf.x, -e2f.y * vf.y), fmaf(e2f.x, vf.y, e2f.y * vf.x));
            if((n + l) & 1)
              wf = make_float2(-wf.x, -wf.y);
          } else {
            wf = make_float2(vf.x, -vf.y);
          }
          if(sign & 1)
            wf = make_float2(-wf.x, -wf.y);
          tab[(flat(n, m) - base) * W + l * (l + 1) - k] = wf;
        } else {
          if(!neg)
            Tab<TabT>::put(tab, (flat(n, mu) - base) * W + l * (l + 1) - kap, v);
          if(mu == 0 || (!neg && !real_k))
            return;
          zd w;
          if(neg) {
            w = conj(v);
          } else if(hankel) {
            w = e2 * v;  // conj(alpha_neg) = (-1)^{n+l} e^{-2 i d phi} alpha_pos
            if((n + l) & 1)
              w = -w;
          } else {
            w = conj(v);
          }
          if(sign & 1)
            w = -w;
          Tab<TabT>::put(tab, (flat(n, m) - base) * W + l * (l + 1) - k, w);
        }
      };
      store(mu, D);
      zd O2 = mk(0.0, 0.0), O1 = D;
      const double apl = rcoef(s, Lc, l - 1, kap, kAP);
      const double aml = rcoef(s, Lc, l + 1, kap, kAM);
      for(int n = mu + 1; n <= n_hi; ++n) {
        zd Om, Op;
        if(kW == 16 && n == 1) {
          Om = seed_at(l - 1);
          Op = seed_at(l + 1);
        } else {
          Om = shfl_up_w<kW>(O1);
          Op = shfl_down_w<kW>(O1);
        }
        const double amn = rcoef(s, Lc, n - 1, mu, kAM);
        const double rapn = rcoef(s, Lc, n - 1, mu, kRAP);
        zd O;
        O.re = fma(Om.re, apl, fma(Op.re, aml, -O2.re * amn)) * rapn;
        O.im = fma(Om.im, apl, fma(Op.im, aml, -O2.im * amn)) * rapn;
        if(l > L)
          O = mk(0.0, 0.0);
        O2 = O1;
        O1 = O;
        store(n, O);
      }
    }
  }
}

template <typename TabT>
__device__ void chains(const Smem &s, TabT *tab, const Layout &y, int hankel, bool real_k,
                       int n_lo, int n_hi) {
  if(y.nmax <= 8)
    run_chains<16, TabT>(s, tab, y, hankel, real_k, n_lo, n_hi);
  else
    run_chains<32, TabT>(s, tab, y, hankel, real_k, n_lo, n_hi);
}

// A(q, p) and B(q, p) of Coupling.cpp:30-51 for q = (n, m) in the table chunk
// starting at flat index `base`, p = (l, k). The reference's coefficient
// products c_i * factor are split into a row factor (qf) and a column factor (pf).
template <typename R> struct CT {
  R re, im;
};
template <typename R> __device__ __forceinline__ CT<R> ld(const zd *t, int i) {
  return CT<R>{(R)t[i].re, (R)t[i].im};
}
template <typename R> __device__ __forceinline__ CT<R> ld(const float2 *t, int i) {
  return CT<R>{(R)t[i].x, (R)t[i].y};
}

template <typename R> struct Fac;
template <> struct Fac<double> {
  static __device__ __forceinline__ const double *q(const Smem &s) { return s.qf; }
  static __device__ __forceinline__ const double *p(const Smem &s) { return s.pf; }
};
template <> struct Fac<float> {
  static __device__ __forceinline__ const float *q(const Smem &s) { return s.qf32; }
  static __device__ __forceinline__ const float *p(const Smem &s) { return s.pf32; }
};

template <typename R, typename TabT>
__device__ __forceinline__ void coupling_entry(const Smem &s, const TabT *tab, const Layout &y,
                                               int base, int q, int p, CT<R> &A, CT<R> &B) {
  const R *qf = Fac<R>::q(s) + q * kQfacStride;
  const R *pf = Fac<R>::p(s) + p * kPfacStride;
  const int n = (int)qf[3], m = (int)qf[4], l = (int)pf[6], k = (int)pf[7];
  const int W = y.W;
  const int row = (q - base) * W;
  const R z = 0;
  const int c0 = row + l * (l + 1) - k;
  const CT<R> t0 = ld<R>(tab, c0);
  const CT<R> tp = (m < n && k < l) ? ld<R>(tab, c0 - 1 - W) : CT<R>{z, z};
  const CT<R> tm = (m > -n && k > -l) ? ld<R>(tab, c0 + 1 + W) : CT<R>{z, z};
  const R f0 = qf[2] * pf[2], f1 = qf[0] * pf[0], f2 = qf[1] * pf[1];
  A.re = fma(f0, t0.re, fma(f1, tp.re, f2 * tm.re));
  A.im = fma(f0, t0.im, fma(f1, tp.im, f2 * tm.im));
  const int c1 = row + (l - 1) * l - k;
  const int lm = l - 1;
  const CT<R> u0 = (k <= lm && k >= -lm) ? ld<R>(tab, c1) : CT<R>{z, z};
  const CT<R> up = (m < n && k + 1 <= lm && k + 1 >= -lm) ? ld<R>(tab, c1 - 1 - W) : CT<R>{z, z};
  const CT<R> um = (m > -n && k - 1 >= -lm && k - 1 <= lm) ? ld<R>(tab, c1 + 1 + W) : CT<R>{z, z};
  const R g0 = qf[2] * pf[3], g1 = qf[0] * pf[4], g2 = qf[1] * pf[5];
  const R sre = fma(g0, u0.re, fma(g1, up.re, -g2 * um.re));
  const R sim = fma(g0, u0.im, fma(g1, up.im, -g2 * um.im));
  B.re = sim;  // -i * s
  B.im = -sre;
}

// zd-typed wrapper used by the source and coupling kernels (FP64 table)
__device__ __forceinline__ void coupling_entry(const Smem &s, const Layout &y, int base, int q, int p,
                                               zd &A, zd &B) {
  CT<double> a, b;
  coupling_entry<double, zd>(s, s.tab, y, base, q, p, a, b);
  A = mk(a.re, a.im);
  B = mk(b.re, b.im);
}

// -(t * v) for the T-matrix row scaling
template <typename R> __device__ __forceinline__ CT<R> neg_mul(CT<R> t, CT<R> v) {
  return CT<R>{fma(-t.re, v.re, t.im * v.im), fma(-t.re, v.im, -(t.im * v.re))};
}

struct AssembleArgs {
  const double *cart;
  const zd *T;  // N x (nmax+1) x 2
  const double *rec, *qf, *pf, *legc;
  int N;
  zd waveK;
  long ld;
  int nchunks;
  int2 chunks[kMaxNmax];
  // pair-scratch mode (ACA batches): CTA b handles unordered pair pair0 + b and
  // writes S_ij, S_ji as two consecutive 2P x 2P column-major blocks at
  // S + 2 b (2P)^2 (ld = 2P); no identity blocks
  int scratch;
  long pair0;
  // batch mode (batch != nullptr): CTA b works on matrix b / per_mat of the
  // table, local index b % per_mat (pairs, then identity blocks, then idle
  // CTAs of the size class's padding); the table's entry replaces cart, T,
  // N, waveK, ld and S
  const BatchMat *batch;
  int per_mat;
  // row-block mode (row1 > row0): the rows of spheres row0 .. row1 - 1 only,
  // into a (2P (row1 - row0)) x 2PN column-major block (ld = its rows);
  // CTA b handles the ordered pair (row0 + b / N, b % N)
  int row0, row1;
};

template <typename O> __device__ __forceinline__ void put_out(O *S, size_t at, double re, double im);
template <> __device__ __forceinline__ void put_out<double2>(double2 *S, size_t at, double re, double im) {
  S[at] = make_double2(re, im);
}
template <> __device__ __forceinline__ void put_out<float2>(float2 *S, size_t at, double re, double im) {
  S[at] = make_float2((float)re, (float)im);
}

// kMixed = false: complex128 table, FP64 block forming, complex128 S.
// kMixed = true (precision form): the recurrences still run in FP64; their
// results are rounded into a complex64 table and the blocks are formed in FP32
// straight into the complex64 S.
//
// One CTA per unordered pair {i, j}, i < j: the table is built for
// R = r_i - r_j and serves both S_ij and S_ji, because Y_l^m(-R) = (-1)^l Y_l^m(R)
// and the recurrences keep the parity of n + l, so alpha(n,m,l,k; -R) =
// (-1)^{n+l} alpha(n,m,l,k; R): A(-R) = (-1)^{n+l} A(R), B(-R) = -(-1)^{n+l} B(R).
// The last N CTAs write the identity diagonal blocks.
template <bool kMixed>
__global__ void __launch_bounds__(256) k_assemble(AssembleArgs a, Layout y,
                                                  typename std::conditional<kMixed, float2, double2>::type *S) {
  typedef typename std::conditional<kMixed, float2, double2>::type OutT;
  typedef typename std::conditional<kMixed, float2, zd>::type TabT;
  typedef typename std::conditional<kMixed, float, double>::type R;
  extern __shared__ double smem[];
  const double *cart = a.cart;
  const zd *Tg = a.T;
  int N = a.N;
  zd waveK = a.waveK;
  long ld = a.ld;
  long b = blockIdx.x + (a.scratch ? a.pair0 : 0);
  if(a.batch) {
    const BatchMat &bm = a.batch[blockIdx.x / a.per_mat];
    b = blockIdx.x % a.per_mat;
    cart = bm.cart;
    Tg = bm.T;
    N = bm.N;
    waveK = bm.waveK;
    ld = bm.ld;
    S = (OutT *)bm.S;
    if(b >= (long)N * (N + 1) / 2)  // idle: padding of the size class or an empty entry
      return;
  }
  const long npairs = (long)N * (N - 1) / 2;
  const int P = y.P;
  const bool rowblk = a.row1 > a.row0;
  int i, j;
  if(rowblk) {
    i = a.row0 + (int)(b / N);
    j = (int)(b % N);
    if(i == j) {
      const long r0 = 2L * P * (i - a.row0), c0 = 2L * P * i;
      for(int idx = threadIdx.x; idx < 4 * P * P; idx += blockDim.x) {
        int c = idx / (2 * P), r = idx - c * 2 * P;
        put_out<OutT>(S, (c0 + c) * ld + r0 + r, r == c ? 1.0 : 0.0, 0.0);
      }
      return;
    }
  } else {
    if(!a.scratch && b >= npairs) {
      const int d = (int)(b - npairs);
      const long x0 = 2L * P * d;
      for(int idx = threadIdx.x; idx < 4 * P * P; idx += blockDim.x) {
        int c = idx / (2 * P), r = idx - c * 2 * P;
        put_out<OutT>(S, (x0 + c) * ld + x0 + r, r == c ? 1.0 : 0.0, 0.0);
      }
      return;
    }
    // b -> (i, j), i < j: b = j (j - 1) / 2 + i
    j = (int)((1.0 + sqrt(1.0 + 8.0 * (double)b)) * 0.5);
    while((long)j * (j - 1) / 2 > b)
      --j;
    while((long)(j + 1) * j / 2 <= b)
      ++j;
    i = (int)(b - (long)j * (j - 1) / 2);
  }
  const long xi = a.scratch ? 0 : 2L * P * (rowblk ? i - a.row0 : i), xj = a.scratch ? 0 : 2L * P * j;
  OutT *Sij = S, *Sji = S;
  if(a.scratch) {
    Sij = S + (size_t)(2 * blockIdx.x) * (4L * P * P);
    Sji = Sij + 4L * P * P;
  }
  Smem s = smem_view(smem, y, a.qf, a.pf);
  TabT *tab = reinterpret_cast<TabT *>(s.tab);
  load_tables(s, y, a.rec, a.qf, a.pf, a.legc);
  const int nT = 2 * (y.nmax + 1);
  for(int t = threadIdx.x; t < 2 * nT; t += blockDim.x)  // T_i then T_j
    s.tl[t] = Tg[(size_t)(t < nT ? i : j) * nT + (t < nT ? t : t - nT)];
  if(kMixed) {
    for(int t = threadIdx.x; t < kQfacStride * y.P; t += blockDim.x)
      s.qf32[t] = (float)a.qf[t];
    for(int t = threadIdx.x; t < kPfacStride * y.P; t += blockDim.x)
      s.pf32[t] = (float)a.pf[t];
    for(int t = threadIdx.x; t < 2 * nT; t += blockDim.x) {
      const zd v = Tg[(size_t)(t < nT ? i : j) * nT + (t < nT ? t : t - nT)];
      s.tl32[t] = make_float2((float)v.re, (float)v.im);
    }
  }
  if(threadIdx.x == 0) {
    double dx = cart[3 * i] - cart[3 * j], dy = cart[3 * i + 1] - cart[3 * j + 1],
           dz = cart[3 * i + 2] - cart[3 * j + 2];
    to_spherical(dx, dy, dz, &s.geo[0], &s.geo[1], &s.geo[2]);
  }
  __syncthreads();
  make_seeds(s, y, waveK, 1);
  for(int c = 0; c < a.nchunks; ++c) {
    const int n_lo = a.chunks[c].x, n_hi = a.chunks[c].y;
    chains<TabT>(s, tab, y, 1, waveK.im == 0.0, n_lo, n_hi);
    __syncthreads();
    const int base = n_lo * n_lo - 1;
    const int rows = (n_hi + 1) * (n_hi + 1) - 1 - base;
    for(int idx = threadIdx.x; idx < rows * P; idx += blockDim.x) {
      const int qr = idx / P, p = idx - qr * P, q = base + qr;
      CT<R> A, B;
      coupling_entry<R, TabT>(s, tab, y, base, q, p, A, B);
      const int l = (int)s.pf[p * kPfacStride + 6];
      const int n = (int)s.qf[q * kQfacStride + 3];
      CT<R> tei, tmi, tej, tmj;
      if(kMixed) {
        tei = CT<R>{(R)s.tl32[2 * l].x, (R)s.tl32[2 * l].y};
        tmi = CT<R>{(R)s.tl32[2 * l + 1].x, (R)s.tl32[2 * l + 1].y};
        tej = CT<R>{(R)s.tl32[nT + 2 * l].x, (R)s.tl32[nT + 2 * l].y};
        tmj = CT<R>{(R)s.tl32[nT + 2 * l + 1].x, (R)s.tl32[nT + 2 * l + 1].y};
      } else {
        tei = CT<R>{(R)s.tl[2 * l].re, (R)s.tl[2 * l].im};
        tmi = CT<R>{(R)s.tl[2 * l + 1].re, (R)s.tl[2 * l + 1].im};
        tej = CT<R>{(R)s.tl[nT + 2 * l].re, (R)s.tl[nT + 2 * l].im};
        tmj = CT<R>{(R)s.tl[nT + 2 * l + 1].re, (R)s.tl[nT + 2 * l + 1].im};
      }
      // S_ij (rows of sphere i, columns of sphere j), translation r_i - r_j
      size_t col_te = (xj + q) * ld + xi, col_tm = (xj + P + q) * ld + xi;
      CT<R> v = neg_mul(tei, A);
      put_out<OutT>(Sij, col_te + p, v.re, v.im);
      v = neg_mul(tmi, A);
      put_out<OutT>(Sij, col_tm + P + p, v.re, v.im);
      v = neg_mul(tei, B);
      put_out<OutT>(Sij, col_tm + p, v.re, v.im);
      v = neg_mul(tmi, B);
      put_out<OutT>(Sij, col_te + P + p, v.re, v.im);
      if(rowblk)
        continue;
      // S_ji, translation r_j - r_i
      if((n + l) & 1) {
        A.re = -A.re;
        A.im = -A.im;
      } else {
        B.re = -B.re;
        B.im = -B.im;
      }
      col_te = (xi + q) * ld + xj;
      col_tm = (xi + P + q) * ld + xj;
      v = neg_mul(tej, A);
      put_out<OutT>(Sji, col_te + p, v.re, v.im);
      v = neg_mul(tmj, A);
      put_out<OutT>(Sji, col_tm + P + p, v.re, v.im);
      v = neg_mul(tej, B);
      put_out<OutT>(Sji, col_tm + p, v.re, v.im);
      v = neg_mul(tmj, B);
      put_out<OutT>(Sji, col_te + P + p, v.re, v.im);
    }
    __syncthreads();
  }
}

struct SourceArgs {
  const double *cart;
  const zd *T;
  int weights_only;  // 1: only the C_sca weights (SH cross section at 2k)
  const zd *inc;  // 2P
  const double *rec, *qf, *pf, *legc;
  zd waveK;
  zd *incloc, *Q;
  double *wsca;
  int nchunks;
  int2 chunks[kMaxNmax];
};

// getIncLocal (Excitation.cpp:79-129) + source_vector (PreconditionedMatrix.cpp:1327-1345)
// + the per-sphere weights of getScatteringCrossSection (Result.cpp:563-631).
__global__ void __launch_bounds__(256) k_source(SourceArgs a, Layout y) {
  extern __shared__ double smem[];
  const int i = blockIdx.x;
  const int P = y.P, t = threadIdx.x;
  Smem s = smem_view(smem, y, a.qf, a.pf);
  load_tables(s, y, a.rec, a.qf, a.pf, a.legc);
  for(int u = t; u < 2 * (y.nmax + 1); u += blockDim.x)
    s.tl[u] = a.T[(size_t)i * 2 * (y.nmax + 1) + u];
  if(t == 0)
    to_spherical(a.cart[3 * i], a.cart[3 * i + 1], a.cart[3 * i + 2], &s.geo[0], &s.geo[1],
                 &s.geo[2]);
  __syncthreads();
  zd te = mk(0.0, 0.0), tm = mk(0.0, 0.0);
  double w = 0.0;
  const bool at_origin = fabs(s.geo[0]) < 1e-10;  // Coupling.cpp:82-84: A = I, B = 0
  if(at_origin) {
    if(t < P) {
      if(!a.weights_only) {
        te = a.inc[t];
        tm = a.inc[P + t];
      }
      w = 1.0;
    }
  } else {
    make_seeds(s, y, a.waveK, 0);
    for(int c = 0; c < a.nchunks; ++c) {
      const int n_lo = a.chunks[c].x, n_hi = a.chunks[c].y;
      chains<zd>(s, s.tab, y, 0, a.waveK.im == 0.0, n_lo, n_hi);
      __syncthreads();
      const int base = n_lo * n_lo - 1;
      const int qend = (n_hi + 1) * (n_hi + 1) - 1;
      if(t < P && !a.weights_only) {
        for(int q = base; q < qend; ++q) {  // IncLocal[p] = sum_q A(q,p) a_q + B(q,p) b_q
          zd A, B;
          coupling_entry(s, y, base, q, t, A, B);
          te = te + A * a.inc[q] + B * a.inc[P + q];
          tm = tm + B * a.inc[q] + A * a.inc[P + q];
        }
      }
      if(t >= base && t < qend) {
        for(int p = 0; p < P; ++p) {
          zd A, B;
          coupling_entry(s, y, base, t, p, A, B);
          w += norm2(A) + norm2(B);
        }
      }
      __syncthreads();
    }
  }
  if(t < P && a.weights_only) {
    a.wsca[(size_t)i * P + t] = w;
  } else if(t < P) {
    const size_t o = (size_t)i * 2 * P;
    const int l = (int)s.pf[t * kPfacStride + 6];
    a.incloc[o + t] = te;
    a.incloc[o + P + t] = tm;
    a.Q[o + t] = s.tl[2 * l] * te;
    a.Q[o + P + t] = s.tl[2 * l + 1] * tm;
    a.wsca[(size_t)i * P + t] = w;
  }
}

struct CouplingArgs {
  const double *rel;  // count x 3 Cartesian
  const double *rec, *qf, *pf, *legc;
  zd waveK;
  int hankel;
  zd *A, *B;  // count x P x P
  int nchunks;
  int2 chunks[kMaxNmax];
};

__global__ void __launch_bounds__(256) k_coupling(CouplingArgs a, Layout y) {
  extern __shared__ double smem[];
  const int e = blockIdx.x, P = y.P;
  Smem s = smem_view(smem, y, a.qf, a.pf);
  zd *A = a.A + (size_t)e * P * P, *B = a.B + (size_t)e * P * P;
  load_tables(s, y, a.rec, a.qf, a.pf, a.legc);
  if(threadIdx.x == 0)
    to_spherical(a.rel[3 * e], a.rel[3 * e + 1], a.rel[3 * e + 2], &s.geo[0], &s.geo[1],
                 &s.geo[2]);
  __syncthreads();
  if(fabs(s.geo[0]) < 1e-10) {
    for(int idx = threadIdx.x; idx < P * P; idx += blockDim.x) {
      A[idx] = mk((idx / P) == (idx % P) ? 1.0 : 0.0, 0.0);
      B[idx] = mk(0.0, 0.0);
    }
    return;
  }
  make_seeds(s, y, a.waveK, a.hankel);
  for(int c = 0; c < a.nchunks; ++c) {
    const int n_lo = a.chunks[c].x, n_hi = a.chunks[c].y;
    chains<zd>(s, s.tab, y, a.hankel, a.waveK.im == 0.0, n_lo, n_hi);
    __syncthreads();
    const int base = n_lo * n_lo - 1;
    const int rows = (n_hi + 1) * (n_hi + 1) - 1 - base;
    for(int idx = threadIdx.x; idx < rows * P; idx += blockDim.x) {
      const int qr = idx / P, p = idx - qr * P, q = base + qr;
      zd va, vb;
      coupling_entry(s, y, base, q, p, va, vb);
      A[(size_t)p * P + q] = va;  // row q = (n,m), column p = (l,k)
      B[(size_t)p * P + q] = vb;
    }
    __syncthreads();
  }
}

// Per sphere and n: T-matrix (FF, SH), internal factors and the Mie
// absorption factors (Scatterer.cpp:39-271, Geometry.cpp:86-145). One CTA
// per sphere: six threads evaluate the Bessel sequences j(r0), j(rho r0),
// h(r0) of both harmonics side by side, then one thread per (harmonic, n)
// forms that order's factors.
__global__ void __launch_bounds__(64) k_sphere_terms(const SphereScalars *sc, int N, int nmax, zd *T,
                                                     zd *Tsh, zd *iaux, double *cabs_out, zd *shf) {
  __shared__ zd Bv[2][3][kMaxNmax + 2], dBv[2][3][kMaxNmax + 2];
  const int i = blockIdx.x;
  if(i >= N)
    return;
  const SphereScalars c = sc[i];
  if(threadIdx.x < 6) {
    const int h = threadIdx.x / 3, w = threadIdx.x % 3;
    const zd r0 = h ? c.r0_sh : c.r0, rho = h ? c.rho_sh : c.rho;
    bessel_deriv(w == 2 ? 1 : 0, w == 1 ? rho * r0 : r0, nmax, Bv[h][w], dBv[h][w]);
  }
  __syncthreads();
  for(int t = threadIdx.x; t < 2 * (nmax + 1); t += blockDim.x) {
    const int h = t / (nmax + 1), n = t % (nmax + 1);
    zd *Tout = (h ? Tsh : T) + (size_t)i * 2 * (nmax + 1);
    if(n == 0) {
      Tout[0] = mk(0.0, 0.0);
      Tout[1] = mk(0.0, 0.0);
      continue;
    }
    const zd r0 = h ? c.r0_sh : c.r0, rho = h ? c.rho_sh : c.rho, mu_sob = h ? c.mu_sob_sh : c.mu_sob;
    const zd *J = Bv[h][0], *dJ = dBv[h][0], *Jr = Bv[h][1], *dJr = dBv[h][1], *H = Bv[h][2],
             *dH = dBv[h][2];
    zd psi = r0 * J[n];
    zd dpsi = r0 * dJ[n] + J[n];
    zd ksi = r0 * H[n];
    zd dksi = r0 * dH[n] + H[n];
    zd psirho = r0 * rho * Jr[n];
    zd dpsirho = r0 * rho * dJr[n] + Jr[n];
    zd TE = (psi / ksi) * (mu_sob * dpsi / psi - rho * dpsirho / psirho) /
            (rho * dpsirho / psirho - mu_sob * dksi / ksi);
    zd TM = (psi / ksi) * (mu_sob * dpsirho / psirho - rho * dpsi / psi) /
            (rho * dksi / ksi - mu_sob * dpsirho / psirho);
    Tout[2 * n] = TE;
    Tout[2 * n + 1] = TM;
    if(h == 1 && shf) {
      // getTLocalSH1_outer / SH2_outer / getIauxSH1 / getIauxSH2 (Scatterer.cpp:163-412)
      const zd x_b2 = c.x_b2, x_i2 = c.x_i2, z = c.zeta;
      zd *f = shf + ((size_t)i * (nmax + 1) + n) * 8;
      const zd den_te = z * ksi * dpsirho - psirho * dksi;
      const zd den_tm = z * psirho * dksi - ksi * dpsirho;
      f[0] = -(x_b2 * psirho) / den_te;
      f[1] = -(x_b2 * dpsirho) / den_tm;
      f[2] = z * x_b2 * dpsirho / den_te;
      f[3] = z * x_b2 * psirho / den_tm;
      const zd i1te = (-x_i2 * ksi) / (x_b2 * psirho);
      const zd i1tm = (-x_i2 * dksi) / (x_b2 * dpsirho);
      f[4] = i1te;
      f[5] = i1tm;
      const zd bnpp = (z * x_b2 * dpsirho) / den_te;
      const zd anpp = (z * x_b2 * psirho) / den_tm;
      f[6] = bnpp * ((-x_i2 * ksi) / (x_b2 * psirho) + (x_i2 * dksi) / (z * x_b2 * dpsirho));
      f[7] = anpp * ((-x_i2 * dksi) / (x_b2 * dpsirho) + (x_i2 * ksi) / (z * x_b2 * psirho));
    }
    if(h == 0) {
      const zd mu_j = c.mu_j, mu_0 = c.mu_0, I = mk(0.0, 1.0);
      zd ia_te = (mu_j * rho) / (mu_0 * rho * dpsirho * psi - mu_j * psirho * dpsi) * I;
      zd ia_tm = (mu_j * rho) / (mu_j * psi * dpsirho - mu_0 * rho * psirho * dpsi) * I;
      iaux[(size_t)i * 2 * (nmax + 1) + 2 * n] = ia_te;
      iaux[(size_t)i * 2 * (nmax + 1) + 2 * n + 1] = ia_tm;
      zd t1 = I * rho * mu_0 * conj(mu_j) * conj(psirho) * dpsirho;
      double t2 = cabs(mu_j * psirho * dpsi - mu_0 * rho * dpsirho * psi);
      t2 *= t2;
      cabs_out[(size_t)i * 2 * (nmax + 1) + 2 * n] = t1.re / t2;
      t1 = I * conj(rho) * mu_0 * mu_j * conj(psirho) * dpsirho;
      t2 = cabs(mu_0 * rho * psirho * dpsi - mu_j * dpsirho * psi);
      t2 *= t2;
      cabs_out[(size_t)i * 2 * (nmax + 1) + 2 * n + 1] = t1.re / t2;
    }
  }
}

// Excitation::populate (Excitation.cpp:48-75): one thread per m.
__global__ void k_incident(int nmax, double theta, double phi, const double *einc, zd *inc) {
  const int t = threadIdx.x;
  if(t > 2 * nmax)
    return;
  const int m = nmax - t;
  const int P = pmax(nmax);
  double W[kMaxNmax + 1], dW[kMaxNmax + 1];
  vigdvig(nmax, m, theta, W, dW);
  const double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
  const zd E0 = mk(einc[0], einc[1]), E1 = mk(einc[2], einc[3]), E2 = mk(einc[4], einc[5]);
  const double sgn_m = (m & 1) ? -1.0 : 1.0;
  double ps, pc;
  sincos(-(double)m * phi, &ps, &pc);
  const zd ph = mk(pc, ps);
  for(int n = (m < 0 ? -m : m); n <= nmax; ++n) {
    if(n == 0)
      continue;
    double A;
    if(m == 0)
      A = 0.0;
    else if(fabs(theta) < 1e-10 || (fabs(theta) - kPi + 1e-10) > 0.0)
      A = m / cos(theta) * dW[n];
    else
      A = m / sin(theta) * W[n];
    // local (r, theta, phi) components of C_n and B_n, projected to Cartesian
    const zd Cr = mk(0.0, 0.0), Ct = mk(0.0, A), Cp = mk(-dW[n], 0.0);
    const zd Br = mk(0.0, 0.0), Bt = mk(dW[n], 0.0), Bp = mk(0.0, A);
    zd Cx = st * cp * Cr + ct * cp * Ct - sp * Cp, Cy = st * sp * Cr + ct * sp * Ct + cp * Cp,
       Cz = ct * Cr - st * Ct;
    zd Bx = st * cp * Br + ct * cp * Bt - sp * Bp, By = st * sp * Br + ct * sp * Bt + cp * Bp,
       Bz = ct * Br - st * Bt;
    zd cdot = conj(Cx) * E0 + conj(Cy) * E1 + conj(Cz) * E2;
    zd bdot = conj(Bx) * E0 + conj(By) * E1 + conj(Bz) * E2;
    const double dn = sqrt((2.0 * n + 1.0) / (4.0 * kPi * (double)((unsigned long)n * (n + 1))));
    const zd i_pow[4] = {mk(1, 0), mk(0, 1), mk(-1, 0), mk(0, -1)};
    const zd in = i_pow[n & 3], in1 = i_pow[(n + 3) & 3];
    const int p = flat(n, m);
    inc[p] = 4 * kPi * sgn_m * in * dn * cdot * ph;
    inc[P + p] = 4 * kPi * sgn_m * in1 * dn * bdot * ph;
  }
}

std::atomic<size_t> g_smem_limit{0};

size_t smem_limit() {
  size_t v = g_smem_limit.load();
  if(!v) {
    int dev = 0, lim = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    v = (size_t)lim;
    g_smem_limit.store(v);
  }
  return v;
}

template <typename Args> void fill_chunks(Args &a, const Layout &y) {
  auto ch = make_chunks(y);
  a.nchunks = (int)ch.size();
  for(size_t c = 0; c < ch.size(); ++c)
    a.chunks[c] = make_int2(ch[c].first, ch[c].second);
}

// The dynamic shared-memory ceiling of a kernel is a process-wide attribute:
// it is always raised to the largest layout (smem_limit), never set to one
// launch's size, so that contexts launching the same kernel from several host
// threads with different nMax cannot undercut each other's launches.
template <typename K> void set_smem(K kernel, size_t bytes, int carveout = -1) {
  (void)bytes;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_limit());
  if(carveout >= 0)
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, carveout);
}

}  // namespace

const CoefTables &coef_tables(om_context *ctx, int nmax) {
  if(ctx->parent)  // built with synchronous copies: ready for any stream
    return coef_tables(ctx->parent, nmax);
  for(auto &t : ctx->tables)
    if(t.nmax == nmax)
      return t;
  CoefTables t;
  t.nmax = nmax;
  const int Lc = 2 * nmax + 1, P = pmax(nmax);
  std::vector<double> rec(kRecStride * (Lc + 1) * (Lc + 1), 0.0);
  for(int n = 0; n <= Lc; ++n)
    for(int m = -n; m <= n; ++m) {
      int i = n * n + n + m;
      rec[kRecStride * i + kAP] = h_a_plus(n, m);
      rec[kRecStride * i + kAM] = h_a_minus(n, m);
      rec[kRecStride * i + kBP] = h_b_plus(n, m);
      rec[kRecStride * i + kBM] = h_b_minus(n, m);
      rec[kRecStride * i + kRAP] = h_a_plus(n, m) != 0.0 ? 1.0 / h_a_plus(n, m) : 0.0;
      rec[kRecStride * i + kRBP] = h_b_plus(n, m) != 0.0 ? 1.0 / h_b_plus(n, m) : 0.0;
    }
  std::vector<double> qf(kQfacStride * P), pf(kPfacStride * P);
  for(int n = 1; n <= nmax; ++n)
    for(int m = -n; m <= n; ++m) {
      int i = flat(n, m);
      double g = 0.5 / std::sqrt(double(n * (n + 1)));
      qf[kQfacStride * i + 0] = g * std::sqrt(double((n - m) * (n + m + 1)));
      qf[kQfacStride * i + 1] = g * std::sqrt(double((n + m) * (n - m + 1)));
      qf[kQfacStride * i + 2] = g * 2 * m;
      qf[kQfacStride * i + 3] = n;
      qf[kQfacStride * i + 4] = m;
      qf[kQfacStride * i + 5] = g;
      int l = n, k = m;
      double gl = 1.0 / std::sqrt(double(l * (l + 1)));
      double hB = std::sqrt(double(2 * l + 1) / double((2 * l - 1) * l * (l + 1)));
      pf[kPfacStride * i + 0] = gl * std::sqrt(double((l - k) * (l + k + 1)));
      pf[kPfacStride * i + 1] = gl * std::sqrt(double((l + k) * (l - k + 1)));
      pf[kPfacStride * i + 2] = gl * k;
      pf[kPfacStride * i + 3] = hB * std::sqrt(double((l - k) * (l + k)));
      pf[kPfacStride * i + 4] = hB * std::sqrt(double((l - k) * (l - k - 1)));
      pf[kPfacStride * i + 5] = hB * std::sqrt(double((l + k) * (l + k - 1)));
      pf[kPfacStride * i + 6] = l;
      pf[kPfacStride * i + 7] = k;
    }
  const int L = 2 * nmax;
  std::vector<double> legc((L + 1) * (L + 2), 0.0);
  for(int k = 0; k <= L; ++k) {
    double c = 1.0 / std::sqrt(4.0 * kPi);
    for(int i = 1; i <= k; ++i)
      c *= -std::sqrt(double(2 * i + 1) / double(2 * i));
    legc[2 * (k * (k + 1) / 2 + k)] = c;
    legc[2 * (k * (k + 1) / 2 + k) + 1] = std::sqrt(double(2 * k + 3));
    for(int l = k + 2; l <= L; ++l) {
      legc[2 * (l * (l + 1) / 2 + k)] = std::sqrt(double(4 * l * l - 1) / double(l * l - k * k));
      legc[2 * (l * (l + 1) / 2 + k) + 1] =
          std::sqrt(double((l - 1) * (l - 1) - k * k) / double(4 * (l - 1) * (l - 1) - 1));
    }
  }
  auto up = [](const std::vector<double> &v) {
    double *d = nullptr;
    if(cudaMalloc(&d, v.size() * sizeof(double)) != cudaSuccess)
      throw std::runtime_error("cudaMalloc failed for coefficient tables");
    cudaMemcpy(d, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice);
    return d;
  };
  t.rec = up(rec);
  t.qf = up(qf);
  t.pf = up(pf);
  t.legc = up(legc);
  {
    std::vector<int> ti;
    std::vector<double> td;
    std::vector<float> tz;
    rotation_tables(nmax, ti, td, tz, t.rot_nent, t.rot_ent_base, t.rot_onl_base);
    t.rot_d = up(td);
    if(cudaMalloc(&t.rot_i, ti.size() * sizeof(int)) != cudaSuccess ||
       cudaMalloc(&t.rot_z, tz.size() * sizeof(float)) != cudaSuccess)
      throw std::runtime_error("cudaMalloc failed for rotation tables");
    cudaMemcpy(t.rot_i, ti.data(), ti.size() * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(t.rot_z, tz.data(), tz.size() * sizeof(float), cudaMemcpyHostToDevice);
  }
  ctx->tables.push_back(t);
  return ctx->tables.back();
}

void launch_sphere_terms(om_problem *pr) {
  k_sphere_terms<<<pr->N, 64, 0, pr->ctx->stream>>>(
      pr->d_scal, pr->N, pr->nmax, pr->d_T, pr->d_Tsh, pr->d_iaux, pr->d_cabs, pr->d_shf);
  pr->ctx->last_launches++;
}

void launch_incident(om_problem *pr, const double einc[6]) {
  double *d_e = nullptr;
  // the field vector is passed through a small device buffer owned by the problem
  d_e = pr->d_xsec + 8;
  cudaMemcpyAsync(d_e, einc, 6 * sizeof(double), cudaMemcpyHostToDevice, pr->ctx->stream);
  k_incident<<<1, 32, 0, pr->ctx->stream>>>(pr->nmax, pr->theta, pr->phi, d_e, pr->d_inc);
  pr->ctx->last_launches++;
}

void launch_assemble(om_problem *pr, int harmonic, int precision) {
  om_context *ctx = pr->ctx;
  const bool mixed = precision == OM_C64;
  if(mixed && ctx->asm_rot) {
    launch_assemble_rot(pr, harmonic);
    return;
  }
  const CoefTables &ct = coef_tables(ctx, pr->nmax);
  Layout y = make_layout(pr->nmax, smem_limit(), mixed);
  AssembleArgs a{};
  a.cart = pr->d_cart;
  a.T = harmonic == OM_SH ? pr->d_Tsh : pr->d_T;
  a.rec = ct.rec;
  a.qf = ct.qf;
  a.pf = ct.pf;
  a.legc = ct.legc;
  a.N = pr->N;
  cplx k = harmonic == OM_SH ? 2.0 * pr->waveK : pr->waveK;
  a.waveK = mk(k.real(), k.imag());
  a.ld = pr->n;
  a.scratch = 0;
  a.pair0 = 0;
  a.batch = nullptr;
  a.per_mat = 1;
  fill_chunks(a, y);
  dim3 grid((unsigned)((long)pr->N * (pr->N - 1) / 2 + pr->N));
  timer_begin(ctx, ctx->ev_asm);
  // the assembly runs on the context's low-priority stream, ordered after and
  // before the work of `stream`
  cudaEventRecord(ctx->ev_fork, ctx->stream);
  cudaStreamWaitEvent(ctx->stream_lo, ctx->ev_fork, 0);
  if(mixed) {
    set_smem(k_assemble<true>, y.bytes, ctx->carve_asm);
    k_assemble<true><<<grid, 256, y.bytes, ctx->stream_lo>>>(a, y, (float2 *)pr->d_S32[harmonic]);
  } else {
    set_smem(k_assemble<false>, y.bytes, ctx->carve_asm);
    k_assemble<false><<<grid, 256, y.bytes, ctx->stream_lo>>>(a, y, (double2 *)pr->d_S[harmonic]);
  }
  cudaEventRecord(ctx->ev_join, ctx->stream_lo);
  cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0);
  timer_end(ctx, ctx->ev_asm);
  ctx->last_launches++;
}

void launch_assemble_pairs(om_problem *pr, int harmonic, long pair0, int count, double2 *scratch) {
  om_context *ctx = pr->ctx;
  const CoefTables &ct = coef_tables(ctx, pr->nmax);
  Layout y = make_layout(pr->nmax, smem_limit(), false);
  AssembleArgs a{};
  a.cart = pr->d_cart;
  a.T = harmonic == OM_SH ? pr->d_Tsh : pr->d_T;
  a.rec = ct.rec;
  a.qf = ct.qf;
  a.pf = ct.pf;
  a.legc = ct.legc;
  a.N = pr->N;
  cplx k = harmonic == OM_SH ? 2.0 * pr->waveK : pr->waveK;
  a.waveK = mk(k.real(), k.imag());
  a.ld = 2L * pr->P;
  a.scratch = 1;
  a.pair0 = pair0;
  a.batch = nullptr;
  a.per_mat = 1;
  fill_chunks(a, y);
  set_smem(k_assemble<false>, y.bytes, ctx->carve_asm);
  k_assemble<false><<<count, 256, y.bytes, ctx->stream>>>(a, y, scratch);
  ctx->last_launches++;
}

void launch_assemble_rows(om_problem *pr, int harmonic, int sphere0, int sphere1, double2 *Srows) {
  om_context *ctx = pr->ctx;
  const CoefTables &ct = coef_tables(ctx, pr->nmax);
  Layout y = make_layout(pr->nmax, smem_limit(), false);
  AssembleArgs a{};
  a.cart = pr->d_cart;
  a.T = harmonic == OM_SH ? pr->d_Tsh : pr->d_T;
  a.rec = ct.rec;
  a.qf = ct.qf;
  a.pf = ct.pf;
  a.legc = ct.legc;
  a.N = pr->N;
  cplx k = harmonic == OM_SH ? 2.0 * pr->waveK : pr->waveK;
  a.waveK = mk(k.real(), k.imag());
  a.ld = 2L * pr->P * (sphere1 - sphere0);
  a.per_mat = 1;
  a.row0 = sphere0;
  a.row1 = sphere1;
  fill_chunks(a, y);
  set_smem(k_assemble<false>, y.bytes, ctx->carve_asm);
  k_assemble<false><<<(unsigned)((long)(sphere1 - sphere0) * pr->N), 256, y.bytes, ctx->stream>>>(a, y, Srows);
  ctx->last_launches++;
}

void launch_assemble_batch(om_context *ctx, int nmax, int precision, const BatchMat *d_mats,
                           int nmats, int per_mat, cudaStream_t stream) {
  const bool mixed = precision == OM_C64;
  if(mixed && ctx->asm_rot) {
    launch_assemble_rot_batch(ctx, nmax, d_mats, nmats, per_mat, stream);
    return;
  }
  const CoefTables &ct = coef_tables(ctx, nmax);
  Layout y = make_layout(nmax, smem_limit(), mixed);
  AssembleArgs a{};
  a.rec = ct.rec;
  a.qf = ct.qf;
  a.pf = ct.pf;
  a.legc = ct.legc;
  a.scratch = 0;
  a.pair0 = 0;
  a.batch = d_mats;
  a.per_mat = per_mat;
  fill_chunks(a, y);
  const dim3 grid((unsigned)((long)nmats * per_mat));
  if(mixed) {
    set_smem(k_assemble<true>, y.bytes, ctx->carve_asm);
    k_assemble<true><<<grid, 256, y.bytes, stream>>>(a, y, nullptr);
  } else {
    set_smem(k_assemble<false>, y.bytes, ctx->carve_asm);
    k_assemble<false><<<grid, 256, y.bytes, stream>>>(a, y, nullptr);
  }
  ctx->last_launches++;
}

void launch_source(om_problem *pr) {
  om_context *ctx = pr->ctx;
  const CoefTables &ct = coef_tables(ctx, pr->nmax);
  Layout y = make_layout(pr->nmax, smem_limit());
  SourceArgs a;
  a.cart = pr->d_cart;
  a.T = pr->d_T;
  a.inc = pr->d_inc;
  a.rec = ct.rec;
  a.qf = ct.qf;
  a.pf = ct.pf;
  a.legc = ct.legc;
  a.waveK = mk(pr->waveK.real(), pr->waveK.imag());
  a.incloc = pr->d_incloc;
  a.Q = pr->d_Q;
  a.wsca = pr->d_wsca;
  a.weights_only = 0;
  fill_chunks(a, y);
  set_smem(k_source, y.bytes);
  k_source<<<pr->N, 256, y.bytes, ctx->stream>>>(a, y);
  ctx->last_launches++;
}

// Per-sphere weights sum_p |T^reg_pq(2k)|^2 of getScatteringCrossSection_SH
// (Result.cpp:662-745): the regular translation at twice the wave number.
void launch_sh_weights(om_problem *pr) {
  om_context *ctx = pr->ctx;
  const CoefTables &ct = coef_tables(ctx, pr->nmax);
  Layout y = make_layout(pr->nmax, smem_limit());
  SourceArgs a;
  a.cart = pr->d_cart;
  a.T = pr->d_T;
  a.inc = nullptr;
  a.rec = ct.rec;
  a.qf = ct.qf;
  a.pf = ct.pf;
  a.legc = ct.legc;
  const cplx k2 = 2.0 * pr->waveK;
  a.waveK = mk(k2.real(), k2.imag());
  a.incloc = nullptr;
  a.Q = nullptr;
  a.wsca = pr->d_wsh;
  a.weights_only = 1;
  fill_chunks(a, y);
  set_smem(k_source, y.bytes);
  k_source<<<pr->N, 256, y.bytes, ctx->stream>>>(a, y);
  ctx->last_launches++;
}

int launch_coupling(om_context *ctx, const double *d_rel, int count, zd waveK, int nmax,
                    int hankel, zd *d_A, zd *d_B) {
  const CoefTables &ct = coef_tables(ctx, nmax);
  Layout y = make_layout(nmax, smem_limit());
  CouplingArgs a;
  a.rel = d_rel;
  a.rec = ct.rec;
  a.qf = ct.qf;
  a.pf = ct.pf;
  a.legc = ct.legc;
  a.waveK = waveK;
  a.hankel = hankel;
  a.A = d_A;
  a.B = d_B;
  fill_chunks(a, y);
  set_smem(k_coupling, y.bytes);
  k_coupling<<<count, 256, y.bytes, ctx->stream>>>(a, y);
  ctx->last_launches++;
  return 0;
}

}  // namespace om
