// A wavelength-solve through the C++ interface (optimet_gpu::Solver), the
// way a reference-side caller drives it: spheres, background and wave from a
// small text file, the solve, then the four cross sections on stdout.
//
// Input lines:  sphere x y z radius eps_re eps_im
//               nmax n
//               wave wavelength theta phi e_theta_re e_theta_im e_phi_re e_phi_im
//               background eps_re eps_im mu_re mu_im
//               method lu|gmres
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
  om_solve_options opts{OM_SOLVE_LU, 200, 10, 40, 1e-12, 1e-4};
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
      ss >> wave.wavelength >> wave.theta >> wave.phi >> wave.e_theta[0] >> wave.e_theta[1] >>
          wave.e_phi[0] >> wave.e_phi[1];
    } else if(key == "background") {
      ss >> bg.eps_r[0] >> bg.eps_r[1] >> bg.mu_r[0] >> bg.mu_r[1];
    } else if(key == "method") {
      std::string m;
      ss >> m;
      opts.method = m == "gmres" ? OM_SOLVE_GMRES : OM_SOLVE_LU;
    }
  }
  for(auto &s : spheres)
    s.nmax = nmax;
  try {
    optimet_gpu::Context ctx(0);
    optimet_gpu::Solver solver(ctx, spheres, bg, wave, opts, OM_C128);
    std::vector<std::complex<double>> xs, xi, xs_sh, xi_sh;
    solver.solve(xs, xi, xs_sh, xi_sh);
    const auto c = solver.cross_sections();
    std::printf("unknowns %ld\n", solver.scattering_size());
    std::printf("xsec %.17g %.17g %.17g %.17g\n", c[0], c[1], c[2], c[3]);
    std::printf("x0 %.17g %.17g\n", xs[0].real(), xs[0].imag());
  } catch(const optimet_gpu::Error &e) {
    std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
    return 1;
  }
  return 0;
}
