// A wavelength-solve through the C++ interface (optimet_gpu::Solver), the
// way a reference-side caller drives it: spheres, background, the wave with
// its Cartesian field as the reference's Excitation keeps it, and the solver
// inputs of a Run (the build, the <ParameterList> entries, the ACA flag), from
// a small text file; the solve, then the four cross sections on stdout.
//
// Input lines:  sphere x y z radius eps_re eps_im
//               nmax n
//               wave wavelength theta phi
//               einc ex_re ex_im ey_re ey_im ez_re ez_im   (Cartesian E, after `wave`)
//               background eps_re eps_im mu_re mu_im
//               role serial|scalapack|belos
//               solver GMRES|scalapack|eigen
//               tolerance t
//               iterations max_iterations num_blocks
//               aca yes|no
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "optimet_gpu.hpp"

int main(int argc, char **argv) {
  if(argc != 2) {
    std::fprintf(stderr, "usage: %s case.txt\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1]);
  std::vector<om_sphere> spheres;
  om_medium bg{{1.0, 0.0}, {1.0, 0.0}};
  om_plane_wave wave{};
  optimet_gpu::SolverChoice choice;
  int nmax = 0;
  std::string line;
  while(std::getline(in, line)) {
    std::istringstream ss(line);
    std::string key;
    ss >> key;
    if(key == "sphere") {
      om_sphere s{};
      ss >> s.x >> s.y >> s.z >> s.radius >> s.eps_r[0] >> s.eps_r[1];
      s.mu_r[0] = 1.0;
      s.eps_r_sh[0] = s.eps_r[0];
      s.eps_r_sh[1] = s.eps_r[1];
      spheres.push_back(s);
    } else if(key == "nmax") {
      ss >> nmax;
    } else if(key == "wave") {
      ss >> wave.wavelength >> wave.theta >> wave.phi;
    } else if(key == "einc") {
      double v[6];
      for(double &d : v)
        ss >> d;
      const auto p = optimet_gpu::polarisation(wave.theta, wave.phi, {v[0], v[1]}, {v[2], v[3]}, {v[4], v[5]});
      wave.e_theta[0] = p.first.real();
      wave.e_theta[1] = p.first.imag();
      wave.e_phi[0] = p.second.real();
      wave.e_phi[1] = p.second.imag();
    } else if(key == "background") {
      ss >> bg.eps_r[0] >> bg.eps_r[1] >> bg.mu_r[0] >> bg.mu_r[1];
    } else if(key == "role") {
      std::string r;
      ss >> r;
      choice.build = r == "belos" ? optimet_gpu::Build::Belos
                                  : (r == "scalapack" ? optimet_gpu::Build::Scalapack : optimet_gpu::Build::Serial);
    } else if(key == "solver") {
      ss >> choice.solver;
    } else if(key == "tolerance") {
      ss >> choice.tolerance;
    } else if(key == "iterations") {
      ss >> choice.max_iterations >> choice.num_blocks;
    } else if(key == "aca") {
      std::string a;
      ss >> a;
      choice.aca = a == "yes";
    }
  }
  for(auto &s : spheres)
    s.nmax = nmax;
  try {
    optimet_gpu::Context ctx(0);
    optimet_gpu::Solver solver(ctx, spheres, bg, wave, choice);
    std::vector<std::complex<double>> xs, xi, xs_sh, xi_sh;
    solver.solve(xs, xi, xs_sh, xi_sh);
    const auto c = solver.cross_sections();
    const auto p = optimet_gpu::plan(choice);
    std::printf("unknowns %ld\n", solver.scattering_size());
    std::printf("plan %d %d %d %d %.17g\n", p.precision, p.opts.method, p.opts.max_iter, p.opts.restarts, p.opts.tol);
    std::printf("xsec %.17g %.17g %.17g %.17g\n", c[0], c[1], c[2], c[3]);
    for(const auto &v : xs)
      std::printf("x %.17g %.17g\n", v.real(), v.imag());
  } catch(const optimet_gpu::Error &e) {
    std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
    return 1;
  }
  return 0;
}
