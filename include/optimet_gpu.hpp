/* C++ interface over liboptimet_gpu (header only, C++17).
 *
 * optimet_gpu::Solver plays the role of the reference's
 * solver::AbstractSolver (srcAna/Solver.h:62-144) for one cluster: update()
 * re-expands the excitation (AbstractSolver::update, Solver.h:93-103) and
 * solve() fills the scattered and internal coefficients of the fundamental
 * and, when the wave asks for it, the second harmonic
 * (AbstractSolver::solve, Solver.h:86-87; the coefficient layout of
 * Result::init, Result.cpp:41-58: per sphere [TE | TM], p = n(n+1) - m - 1).
 * Cross sections follow Result::getExtinctionCrossSection /
 * getScatteringCrossSection / getAbsorptionCrossSection (Result.cpp:541-778)
 * and the near field Result::getEHFields (Result.cpp:74-301). Errors throw
 * optimet_gpu::Error (a std::runtime_error, as the reference's solvers
 * throw) carrying the library's status code and message. */
#ifndef OPTIMET_GPU_HPP
#define OPTIMET_GPU_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "optimet_gpu.h"

namespace optimet_gpu {

using cplx = std::complex<double>;

class Error : public std::runtime_error {
public:
  Error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

private:
  int code_;
};

// One GPU: a device context (stream, tables, memory budget in bytes, 0 = none).
class Context {
public:
  explicit Context(int device = 0, size_t budget = 0) {
    const int rc = om_context_create(device, budget, &ctx_);
    if(rc)
      throw Error(rc, "om_context_create failed on device " + std::to_string(device));
  }
  ~Context() { om_context_destroy(ctx_); }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  om_context *get() const { return ctx_; }
  void check(int rc, const char *what) const {
    if(rc != OM_OK)
      throw Error(rc, std::string(what) + ": " + om_context_last_error(ctx_));
  }

private:
  om_context *ctx_ = nullptr;
};

// How the reference was built, which decides its solver (solver::factory,
// Solver.cpp:30-54): Serial (no MPI) -> PreconditionedMatrix; Scalapack (MPI
// with ScaLAPACK, no Belos) -> Scalapack; Belos (MPI with Belos and
// ScaLAPACK) -> by the parameter list's "Solver": "eigen" ->
// PreconditionedMatrix, "scalapack" -> Scalapack, otherwise MatrixBelos.
enum class Build { Serial, Scalapack, Belos };

// The run's solver inputs: the build, the <ParameterList> entries the
// reference reads (read_parameter_list, Reader.cpp:909-921; defaults of
// gmres_linear_system, LinearSystemSolver.hpp:149-160) and the <ACA
// compression="yes"> flag (Geometry::ACA_cond_).
struct SolverChoice {
  Build build = Build::Serial;
  std::string solver = "GMRES";   // "Solver": "GMRES" | "scalapack" | "eigen"
  double tolerance = 1e-10;       // "Convergence Tolerance"
  int max_iterations = 4000;      // "Maximum Iterations"
  int num_blocks = 1000;          // "Num Blocks" (the restart length)
  bool aca = false;
};

// What the GPU runs for a SolverChoice: the matrix form and the solve.
//  - direct solvers (PreconditionedMatrix's colPivHouseholderQr,
//    PreconditionedMatrixSolver.h:45-79; Scalapack's pzgesv,
//    ScalapackSolver.cpp:54-130): OM_C128 with OM_SOLVE_LU;
//  - MatrixBelos (MatrixBelosSolver.cpp:26-104): OM_C128 with OM_SOLVE_GMRES,
//    restart length "Num Blocks" (at most 1000), "Maximum Iterations" in total,
//    "Convergence Tolerance";
//  - with ACA each class runs Gmres_Zcomp on the compressed operator with its
//    own constants (tolerance, iterations per cycle, cycles):
//    PreconditionedMatrix 1e-6, 240, 2 (PreconditionedMatrixSolver.h:48-51),
//    Scalapack 1e-7, 250, 3 (ScalapackSolver.cpp:58-60), MatrixBelos 1e-6,
//    340, 1 (MatrixBelosSolver.cpp:35-37): OM_ACA with OM_SOLVE_GMRES.
struct Plan {
  int precision;
  om_solve_options opts;
};

inline Plan plan(const SolverChoice &c) {
  enum { PM, SC, MB } role = PM;
  if(c.build == Build::Scalapack)
    role = SC;
  else if(c.build == Build::Belos)
    role = c.solver == "eigen" ? PM : (c.solver == "scalapack" ? SC : MB);
  Plan p{OM_C128, om_solve_options{OM_SOLVE_LU, 0, 0, 0, 0.0, 0.0}};
  if(c.aca) {
    p.precision = OM_ACA;
    p.opts.method = OM_SOLVE_GMRES;
    if(role == PM)
      p.opts = om_solve_options{OM_SOLVE_GMRES, 240, 2, 0, 1e-6, 0.0};
    else if(role == SC)
      p.opts = om_solve_options{OM_SOLVE_GMRES, 250, 3, 0, 1e-7, 0.0};
    else
      p.opts = om_solve_options{OM_SOLVE_GMRES, 340, 1, 0, 1e-6, 0.0};
    return p;
  }
  if(role != MB)
    return p;
  const int m = std::max(1, std::min(c.num_blocks, 1000));
  p.opts = om_solve_options{OM_SOLVE_GMRES, m, std::max(1, (c.max_iterations + m - 1) / m), 0, c.tolerance, 0.0};
  return p;
}

// (E_theta, E_phi) of a plane wave from the Cartesian field the reference's
// Excitation keeps (Excitation::Einc = Tools::toProjection of (0, E_theta,
// E_phi), Reader.cpp:818-827): Tools::fromProjection's theta and phi rows
// (Tools.cpp:290-301) at the propagation direction (theta, phi).
inline std::pair<cplx, cplx> polarisation(double theta, double phi, cplx ex, cplx ey, cplx ez) {
  const double st = std::sin(theta), ct = std::cos(theta), sp = std::sin(phi), cp = std::cos(phi);
  return {ct * cp * ex + ct * sp * ey - st * ez, cp * ey - sp * ex};
}

// A cluster of spheres, a background medium and a plane wave, with the
// solver options and the matrix form (OM_C128 plain FP64; OM_ACA the
// compressed FP64 operator, GMRES only; OM_C64 the precision form with
// OM_SOLVE_FGMRES_MIXED or OM_SOLVE_LU_MIXED).
class Solver {
public:
  // the solver the reference would pick for `choice` (plan())
  Solver(Context &ctx, std::vector<om_sphere> spheres, om_medium background, om_plane_wave wave,
         const SolverChoice &choice)
      : Solver(ctx, std::move(spheres), background, wave, plan(choice).opts, plan(choice).precision) {}

  Solver(Context &ctx, std::vector<om_sphere> spheres, om_medium background, om_plane_wave wave,
         om_solve_options opts, int precision = OM_C128)
      : ctx_(ctx), spheres_(std::move(spheres)), bg_(background), wave_(wave), opts_(opts),
        precision_(precision) {
    ctx_.check(om_problem_create(ctx_.get(), spheres_.data(), (int)spheres_.size(), &bg_, &wave_, &pr_),
               "om_problem_create");
  }
  ~Solver() { om_problem_destroy(pr_); }
  Solver(const Solver &) = delete;
  Solver &operator=(const Solver &) = delete;

  // a new wavelength / direction / polarisation for the same cluster
  void update(const om_plane_wave &wave) {
    wave_ = wave;
    ctx_.check(om_problem_set_wave(pr_, &wave_), "om_problem_set_wave");
    solved_ = false;
  }

  // 2 nMax (nMax + 2) N, the length of each coefficient vector
  long scattering_size() const { return om_problem_size(pr_); }

  // source vector, assembly, solve, internal coefficients; the SH chain
  // when the wave asks for it
  void solve(std::vector<cplx> &X_sca, std::vector<cplx> &X_int, std::vector<cplx> &X_sca_SH,
             std::vector<cplx> &X_int_SH) {
    run();
    const long n = scattering_size();
    X_sca.assign(n, 0.0);
    X_int.assign(n, 0.0);
    ctx_.check(om_get_coefficients(pr_, dp(X_sca), dp(X_int)), "om_get_coefficients");
    X_sca_SH.assign(wave_.sh ? n : 0, 0.0);
    X_int_SH.assign(wave_.sh ? n : 0, 0.0);
    if(wave_.sh)
      ctx_.check(om_get_sh_vectors(pr_, nullptr, nullptr, dp(X_sca_SH), dp(X_int_SH)),
                 "om_get_sh_vectors");
  }

  // {C_ext, C_sca, C_ext - C_sca, C_abs from the Mie factors}
  std::array<double, 4> cross_sections() {
    run();
    std::array<double, 4> out{};
    ctx_.check(om_cross_sections(pr_, out.data()), "om_cross_sections");
    return out;
  }

  // {C_sca,SH, C_abs,SH} (SH waves only)
  std::array<double, 2> sh_cross_sections() {
    run();
    std::array<double, 2> out{};
    ctx_.check(om_sh_cross_sections(pr_, out.data()), "om_sh_cross_sections");
    return out;
  }

  // E and H (3 components per point) at Cartesian points xyz (3 per point)
  void near_field(const std::vector<double> &xyz, std::vector<cplx> &E, std::vector<cplx> &H) {
    run();
    const int npts = (int)(xyz.size() / 3);
    E.assign(3 * (size_t)npts, 0.0);
    H.assign(3 * (size_t)npts, 0.0);
    ctx_.check(om_near_field(pr_, xyz.data(), npts, dp(E), dp(H)), "om_near_field");
  }

  const om_solve_stats &stats() const { return stats_; }

private:
  static double *dp(std::vector<cplx> &v) { return reinterpret_cast<double *>(v.data()); }

  void run() {
    if(solved_)
      return;
    ctx_.check(om_source_vector(pr_, nullptr), "om_source_vector");
    ctx_.check(om_assemble(pr_, OM_FF, precision_), "om_assemble");
    const int rc = om_solve(pr_, &opts_, &stats_);
    ctx_.check(rc, "om_solve");
    if(wave_.sh) {
      ctx_.check(om_assemble(pr_, OM_SH, precision_), "om_assemble (SH)");
      ctx_.check(om_solve_sh(pr_, &opts_, nullptr), "om_solve_sh");
    }
    solved_ = true;
  }

  Context &ctx_;
  std::vector<om_sphere> spheres_;
  om_medium bg_;
  om_plane_wave wave_;
  om_solve_options opts_;
  int precision_;
  om_problem *pr_ = nullptr;
  om_solve_stats stats_{};
  bool solved_ = false;
};

}  // namespace optimet_gpu

#endif /* OPTIMET_GPU_HPP */
