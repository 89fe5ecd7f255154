// The solver-role mapping of include/optimet_gpu.hpp (plan, polarisation)
// printed for the cases tests/test_cpp_interface.py checks; no library call.
#include <cstdio>

#include "optimet_gpu.hpp"

int main() {
  using optimet_gpu::Build;
  struct Case {
    Build b;
    const char *solver;
    bool aca;
  } cases[] = {{Build::Serial, "GMRES", false},   {Build::Scalapack, "GMRES", false}, {Build::Belos, "GMRES", false},
               {Build::Belos, "eigen", false},    {Build::Belos, "scalapack", false}, {Build::Serial, "GMRES", true},
               {Build::Scalapack, "GMRES", true}, {Build::Belos, "GMRES", true},      {Build::Belos, "eigen", true}};
  for(const auto &c : cases) {
    optimet_gpu::SolverChoice ch;
    ch.build = c.b;
    ch.solver = c.solver;
    ch.aca = c.aca;
    ch.tolerance = 1e-9;
    ch.max_iterations = 700;
    ch.num_blocks = 300;
    const auto p = optimet_gpu::plan(ch);
    std::printf("%d %s %d : %d %d %d %d %.3g\n", (int)c.b, c.solver, (int)c.aca, p.precision, p.opts.method,
                p.opts.max_iter, p.opts.restarts, p.opts.tol);
  }
  const auto e = optimet_gpu::polarisation(0.7, -1.1, {0.3, 0.1}, {-0.2, 0.4}, {0.5, -0.6});
  std::printf("pol %.17g %.17g %.17g %.17g\n", e.first.real(), e.first.imag(), e.second.real(), e.second.imag());
  return 0;
}
