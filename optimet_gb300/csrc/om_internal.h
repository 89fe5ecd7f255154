// Internal declarations shared by the CUDA translation units of liboptimet_gpu.
#pragma once

#include <complex>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "om_math.cuh"
#include "../../include/optimet_gpu.h"

namespace om {

using cplx = std::complex<double>;

// Geometry-independent coefficient tables for one nMax (device memory), built
// once per context and nMax:
//  rec   : a+, a-, b+, b- of the Stout recurrences (TranslationAdditionCoefficients.cpp:34-61)
//          for n <= 2 nMax + 1, index 4 * (n*n + n + m) + {0,1,2,3}
//  qfac  : per row harmonic q = (n, m): {0.5/sqrt(n(n+1)) * u1, * u2, * 2m, n, m} with
//          u1 = sqrt((n-m)(n+m+1)), u2 = sqrt((n+m)(n-m+1)) (Coupling.cpp:30-51 factorised)
//  pfac  : per column harmonic p = (l, k): {v1/sqrt(l(l+1)), v2/sqrt(l(l+1)), k/sqrt(l(l+1)),
//          hB*w0, hB*w1, hB*w2, l, k} with hB = sqrt((2l+1)/((2l-1) l (l+1)))
struct CoefTables {
  int nmax = -1;
  double *rec = nullptr;
  double *qf = nullptr;
  double *pf = nullptr;
  double *legc = nullptr;  // normalised-Legendre recurrence coefficients for l <= 2 nMax
  // rotation assembly (assemble_rot.cu, rotation_tables): Wigner d step
  // coefficients and lane schedule, the z-axis translation map, the Az / Bz table
  int *rot_i = nullptr;
  double *rot_d = nullptr;
  float *rot_z = nullptr;
  int rot_nent = 0, rot_ent_base = 0, rot_onl_base = 0;
};
constexpr int kQfacStride = 6;
constexpr int kPfacStride = 8;

// Per-sphere scalars computed on the host from the reference's formulas
// (Scatterer.cpp:39-412), consumed by the T-matrix kernel.
struct SphereScalars {
  zd r0, rho, mu_sob, mu_j, mu_0;           // fundamental
  zd r0_sh, rho_sh, mu_sob_sh;              // second harmonic
  zd x_b2, x_i2, zeta;                      // SH outer / internal factors
};

// Per-sphere scalars of the SH source and absorption (Symbol.cpp:155-477).
struct ShScalars {
  zd k1;          // omega sqrt(eps_j mu_j)
  zd kSH;         // 2 omega sqrt(eps_SH mu_SH)
  zd c_up, c_vp;  // 2 i ksiparppar imp, 2 ksiparppar imp; imp = sqrt(mu_b/eps_b)/sqrt(mu_0/eps_0)
  zd c_g1, c_g2;  // i ksippp / waveK_01 / R, i gamma (eps_0/eps_SH) / waveK_01 / R
  zd c_bulk;      // (-eps_0 / eps_SH) gamma
  zd sigma;       // -i eps_0 2 omega (eps_r_SH - 1)
  zd w01;         // waveK_01 = omega sqrt(eps_0 mu_0)
  double R;
  int has_gamma;
};

struct Arena;

// ACA-compressed operator of one harmonic (aca.cu)
struct AcaData {
  double2 *store = nullptr;  // packed blocks (complex128)
  size_t cap = 0, used = 0;  // capacity / used, complex values
  long long *off = nullptr;  // per ordered block (i N + j): offset in the store
  int *rank = nullptr;       // per ordered block: rank, -1 dense, -2 identity
  char *ctl = nullptr;       // bump offset (8 bytes) + overflow flag
};
struct AcaOp {
  int N, kmax;
  const long long *off;
  const int *rank;
  const double2 *store;
};

// One matrix of a batched assembly (batch.cu): the spheres' centres and
// T-matrix factors (FF or SH), the wave number and the column-major output
// (ld = 2 P N). N = 0 marks an unused entry.
struct BatchMat {
  const double *cart;
  const zd *T;
  void *S;
  long ld;
  zd waveK;
  int N;
};
struct BatchClass;

// The SH coupling tables in compact form (sh.cu): for SH harmonic k the pairs
// (p, q) with m_p + m_q = M_k, n_q >= |m_q|, in the order p ascending, n_q
// ascending (entries off[k] .. off[k+1]-1 of pq), and the nine coefficients
// of each pair (val[t * count + e], t = table).
struct ClgCompact {
  int nmax = -1;
  long count = 0;
  int *off = nullptr;
  int2 *pq = nullptr;
  double *val = nullptr;
};

}  // namespace om

struct om_context {
  int device = 0;
  cudaStream_t stream = nullptr;     // every call's work, in order (highest priority)
  cudaStream_t stream_lo = nullptr;  // matrix assembly, forked from / joined to `stream`
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int sm_count = 1;
  // matvec grid caps, CTAs per SM (the kernels walk their tiles with a grid
  // stride): below the SM's capacity so that another slot's assembly fits
  int mv_ctas = 8, mv_ctas_df = 8;
  unsigned long long *d_tile_counter = nullptr;  // matvec tile counter (device)
  int *d_tma_err = nullptr;                      // set by a TMA matvec whose wait timed out
  int mv_tma = 1;                                // complex64 matvecs staged by TMA
  int carve_asm = -1, carve_mv = -1;  // preferred smem carveout (percent), -1 = driver's choice
  // complex64 LU updates on the tensor cores: 3 the persistent kernel for the
  // rank-256 trailing updates and one CTA per tile for the rank-32 ones,
  // 1 persistent for all, 2 one CTA per tile for all, 0 off (FP32 CUDA cores)
  int lu_tc = 3;
  // LU kernels: 1 one cooperative launch per tall panel (its rows in shared
  // memory when they fit) and one launch per triangular sweep, 2 per-column
  // panel launches and per-block sweep launches, 3 as 1 with the panel rows
  // always in global memory
  int lu_persist = 1;
  // batched matvec tiles: 0 autotuned per size class, k > 0 candidate k - 1
  int batch_tiles = 0;
  // batched solves: 1 one cooperative launch per solve (k_b_fused) for the
  // classes of at most 1,024 padded unknowns, 2 for those of at most 4,096,
  // 0 the lockstep graphs for every class
  int batch_fused = 1;
  // precision form: the inner FP32 products read a 4-byte copy of the
  // complex64 matrix when 1 (FGMRES: bf16, written by the first product; the
  // batching form: scaled fp16, written after the batch's assembly)
  int inner_half = 1;
  int asm_rot = 1;  // precision-form assembly by rotated z-axis translations (assemble_rot.cu)
  size_t budget = 0;
  size_t used = 0;
  std::string err;
  std::vector<om::CoefTables> tables;  // by nmax
  std::vector<std::pair<int, double *>> clg;  // SH coupling tables by nmax
  std::vector<om::ClgCompact> clgc;           // their compact forms
  int last_launches = 0;               // kernels launched by the last API call
  // kernel timers (CUDA events on `stream`), reset by om_context_timers
  bool timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_mv64, ev_mv32, ev_mvdf, ev_asm;
  double t_mv64 = 0, t_mv32 = 0, t_mvdf = 0, t_asm = 0;  // accumulated milliseconds
  cudaEvent_t mark = nullptr;                // last om_context_mark event
  long n_mv64 = 0, n_mv32 = 0, n_mvdf = 0, n_asm = 0;
  // inner products on the bf16 copy, and the complex64 products that write it
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_mv16, ev_mvcp;
  double t_mv16 = 0, t_mvcp = 0;
  long n_mv16 = 0, n_mvcp = 0;
  // LU phases: whole factorizations, panels, trailing updates, triangular solves
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_luf, ev_lup, ev_luu, ev_lus;
  double t_luf = 0, t_lup = 0, t_luu = 0, t_lus = 0;
  long n_luf = 0, n_lup = 0, n_luu = 0, n_lus = 0;
  std::vector<om_problem *> problems;  // live problems, destroyed with the context
  // auxiliary contexts of the batched solver (streams for per-request work);
  // a context with a parent takes its coefficient tables from the parent
  om_context *parent = nullptr;
  std::vector<om_context *> aux;
};

struct om_problem {
  om_context *ctx = nullptr;
  int N = 0, nmax = 0, P = 0;
  long n = 0;  // 2 P N
  // host model (Reader/Geometry/Excitation state)
  std::vector<double> sph;  // (r, theta, phi) per sphere as the XML reader stores it
  std::vector<double> cart; // toCartesian(sph)
  std::vector<double> radius;
  std::vector<om::cplx> eps_r, mu_r, eps_r_sh;
  om::cplx bg_eps_r, bg_mu_r;
  double lambda = 0, theta = 0, phi = 0;
  om::cplx e_theta, e_phi;
  om::cplx waveK;
  double omega = 0;
  int sh = 0;
  // device state
  double *d_cart = nullptr;
  double *d_radius = nullptr;
  om::zd *d_kin = nullptr;    // per sphere: waveK_0 sqrt(eps_r mu_r) (interior wave number)
  om::zd *d_izin = nullptr;   // per sphere: -i / sqrt(mu / eps)
  om::cplx iZ;                // -i / sqrt(mu_b / eps_b)
  om::SphereScalars *d_scal = nullptr;
  om::zd *d_T = nullptr;      // N x (nmax+1) x 2 : TE, TM per n (FF)
  om::zd *d_Tsh = nullptr;    // same at the second harmonic
  om::zd *d_iaux = nullptr;   // N x (nmax+1) x 2
  double *d_cabs = nullptr;   // N x (nmax+1) x 2
  om::zd *d_inc = nullptr;    // 2P incident coefficients [a | b]
  om::zd *d_incloc = nullptr; // n: IncLocal per sphere
  double *d_wsca = nullptr;   // N x P: sum_p |T^reg_pq|^2 (Result.cpp:563-631)
  om::zd *d_Q = nullptr;      // n
  void *d_S[2] = {nullptr, nullptr};    // complex128 matrix per harmonic (plain form)
  void *d_Srows = nullptr;              // a block of sphere rows (om_assemble_rows), complex128
  int rows0 = 0, rows1 = 0, rows_harmonic = -1;
  size_t rows_bytes = 0;
  void *d_S32[2] = {nullptr, nullptr};  // complex64 matrix per harmonic (precision form)
  int S_prec[2] = {-1, -1};             // which of the two holds the current assembly
  om::zd *d_X = nullptr, *d_Xint = nullptr;
  double *d_xsec = nullptr;   // 4 + scratch
  // second harmonic
  std::vector<om::cplx> ksippp, ksiparppar, gamma;
  om::ShScalars *d_shs = nullptr;
  om::zd *d_shf = nullptr;    // N x (nmax+1) x 8: T1 TE/TM, T2 TE/TM, IauxSH1 TE/TM, IauxSH2 TE/TM
  om::zd *d_shvec = nullptr;  // N x 3P: A_0, A_1, A_m1 vectors
  om::zd *d_K = nullptr, *d_K1 = nullptr, *d_Xsh = nullptr, *d_Xish = nullptr;
  double *d_wsh = nullptr;    // N x P: SH scattering weights
  om::zd *d_acs = nullptr;    // N x P: ACSshcoeff
  om::cplx eta;
  bool have_sh = false;
  bool have_source = false, have_solution = false;
  om::AcaData aca[2];
  // host copies of what update_wave uploads (kept until the next update, so
  // that no asynchronous copy reads freed host memory)
  std::vector<om::SphereScalars> h_scal;
  std::vector<om::ShScalars> h_shs;
  std::vector<om::zd> h_kin, h_izin;
  double h_einc[6] = {0, 0, 0, 0, 0, 0};
};

namespace om {

// translate.cu
const CoefTables &coef_tables(om_context *ctx, int nmax);
void launch_sphere_terms(om_problem *pr);
void launch_incident(om_problem *pr, const double einc[6]);
void launch_assemble(om_problem *pr, int harmonic, int precision);
// unordered pairs pair0 .. pair0 + count - 1 (pair b = j (j - 1) / 2 + i, i < j):
// S_ij and S_ji as 2P x 2P column-major blocks at scratch + 2 (b - pair0) (2P)^2
void launch_assemble_pairs(om_problem *pr, int harmonic, long pair0, int count, double2 *scratch);
// batched assembly: matrix e of the table d_mats (device) is assembled by CTAs
// e per_mat .. (e + 1) per_mat - 1; per_mat >= N (N + 1) / 2 for every entry
// the block rows of spheres sphere0 .. sphere1 - 1 of S (complex128), into a
// (2P (sphere1 - sphere0)) x 2PN column-major block
void launch_assemble_rows(om_problem *pr, int harmonic, int sphere0, int sphere1, double2 *Srows);
void launch_assemble_batch(om_context *ctx, int nmax, int precision, const BatchMat *d_mats,
                           int nmats, int per_mat, cudaStream_t stream);
void launch_source(om_problem *pr);

// assemble_rot.cu: the precision-form (complex64) assembly by rotations and
// its host-built tables for one nMax
void rotation_tables(int nmax, std::vector<int> &ti, std::vector<double> &td, std::vector<float> &tz, int &nent,
                     int &ent_base, int &onl_base);
int rot_smem_bytes(int nmax);
void launch_assemble_rot(om_problem *pr, int harmonic);
void launch_assemble_rot_batch(om_context *ctx, int nmax, const BatchMat *d_mats, int nmats, int per_mat,
                               cudaStream_t stream);
void launch_sh_weights(om_problem *pr);
int launch_coupling(om_context *ctx, const double *d_rel, int count, zd waveK, int nmax,
                    int hankel, zd *d_A, zd *d_B);

// sh.cu
const double *clg_tables_dev(om_context *ctx, int nmax);
int sh_alloc(om_problem *pr);
void launch_sh_source(om_problem *pr);
void launch_sh_internal(om_problem *pr);
void launch_sh_cross_sections(om_problem *pr, double *d_out2);
// w0 = waveK_0; d_kin / d_izw per sphere: 2 waveK_0 sqrt(eps_r_SH mu_r) and
// waveK_0 (-i) / sqrt(mu_SH / eps_SH); d_inner: npts ints of scratch.
void launch_near_field_sh(om_problem *pr, const double *d_xyz, int npts, cplx w0, const zd *d_kin,
                          const zd *d_izw, int *d_inner, zd *d_E, zd *d_H);

// field.cu
void launch_internal(om_problem *pr);
void launch_cross_sections(om_problem *pr);
void launch_near_field(om_problem *pr, const double *d_xyz, int npts, zd *d_E, zd *d_H);

// solve.cu
int solve_lu_rhs(om_problem *pr, int harmonic, const double2 *b, double2 *x, om_solve_stats *st);
int solve_gmres_rhs(om_problem *pr, int harmonic, const om_solve_options *o, const double2 *b,
                    double2 *x, om_solve_stats *st);
int solve_fgmres_rhs(om_problem *pr, int harmonic, const om_solve_options *o, const double2 *b,
                     double2 *x, om_solve_stats *st);
int solve_lu_mixed_rhs(om_problem *pr, int harmonic, const om_solve_options *o, const double2 *b,
                       double2 *x, om_solve_stats *st);

// tc_gemm.cu: C (m x n) -= A (m x k) B (k x n), any k >= 1, complex64, column-major,
// on the tensor cores from operands split once into fp16 hi / lo parts of
// power-of-two scaled rows and columns (FP32 accumulation); three launches:
// the two splits and the update kernel; *d_err set on a timed-out wait;
// scratch: cgemm_sub_tc_split_bytes(m, n, k) bytes of device memory, 16-byte
// aligned.
size_t cgemm_sub_tc_split_bytes(long m, long n, int k);
void launch_cgemm_sub_tc_split(om_context *ctx, const float2 *A, long lda, const float2 *B, long ldb,
                               float2 *C, long ldc, long m, long n, int k, void *scratch, int *d_err);

// aca.cu
int aca_build(om_problem *pr, int harmonic);
void aca_free(om_problem *pr);
AcaOp aca_op(const om_problem *pr, int harmonic);
// y = S x, or y = b - S x when b is given
void aca_matvec(om_context *ctx, const AcaOp &op, const double2 *x, double2 *y, const double2 *b);

// batch.cu: device bytes of one request in the batching form (0: not batchable);
// release of the class workspaces a context keeps between calls
size_t batch_request_bytes(const om_request &rq);
void batch_release(om_context *ctx);

// tma_matvec.cu: complex64 matvec with TMA-staged matrix tiles; false when the
// tensor map cannot be encoded
// cuTensorMapEncodeTiled through the runtime's driver entry point (nullptr
// when the driver does not provide it)
void *tensor_map_encoder();
// (writing the bf16 copy of S into `copy`, ld ldc, when that is not null)
bool launch_matvec_tma(om_context *ctx, const float2 *S, long n, const float2 *x, float2 *part, int row_tiles,
                       long tiles, int cols, unsigned grid, void *copy, long ldc);
// solve.cu: `products` inner FP32 GMRES products on device buffers (the first
// writes the bf16 copy when ctx->inner_half is set, the later ones read it)
int inner_products(om_context *ctx, const float2 *S, long n, const float2 *x, float2 *y, int products);
// the same product on the bf16 copy (Bf16c entries, ld ldh a multiple of 4)
bool launch_matvec_bf16(om_context *ctx, const void *H, long n, long ldh, const float2 *x, float2 *part,
                        int row_tiles, long tiles, int cols, unsigned grid);

// capi.cu: stream-ordered device memory counted against the context budget
int dev_malloc(om_context *ctx, void **p, size_t bytes);
void dev_release(om_context *ctx, void *p, size_t bytes);
void release_matrix(om_problem *pr, int harmonic);

inline int blocks_for(long n, int threads) { return (int)((n + threads - 1) / threads); }

// Event pair around a launch when timing is enabled; folded by collect_timers.
inline void timer_begin(om_context *ctx, std::vector<std::pair<cudaEvent_t, cudaEvent_t>> &v) {
  if(!ctx->timing)
    return;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, ctx->stream);
  v.push_back({a, b});
}
inline void timer_end(om_context *ctx, std::vector<std::pair<cudaEvent_t, cudaEvent_t>> &v) {
  if(!ctx->timing || v.empty())
    return;
  cudaEventRecord(v.back().second, ctx->stream);
}
void collect_timers(om_context *ctx);

}  // namespace om
