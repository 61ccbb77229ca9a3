// C++ host program running VUMPS sweeps through include/imps_vumps.hpp (no Python): reads a
// model and an initial state from a text file, runs the sweeps and prints, per sweep, the two
// bond energies, the gradient norms and the precisions.
//
// Input (whitespace separated): d nsym; I2K (d x nsym ints); for bonds 0 and 1: nsectors, then per
// sector nsym ints and the dimension; nnz, then per nonzero row col value; nsweeps fixed_tol
// InvETol eig_margin autotune(0/1) concurrent(0/1); then the flat AL(0), AL(1), AR(0), AR(1), C[0], C[1] (their
// lengths follow from the layouts).  Per sweep it also prints the wall time of the sweep
// (synchronised) in ms and the Lanczos applies so far.
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>

#include "../../include/imps_vumps.hpp"

int main(int argc, char** argv) {
  if (argc < 2) { std::fprintf(stderr, "usage: %s input\n", argv[0]); return 2; }
  std::ifstream in(argv[1]);
  imps_cpp::model m;
  int nsym = 0;
  in >> m.d >> nsym;
  m.I2K.assign(m.d, imps_cpp::charge(nsym));
  for (auto& q : m.I2K) for (auto& x : q) in >> x;
  std::array<imps_cpp::bond_dims, 2> dims;
  for (int b = 0; b < 2; ++b) {
    int ns = 0;
    in >> ns;
    for (int i = 0; i < ns; ++i) {
      imps_cpp::charge q(nsym);
      for (auto& x : q) in >> x;
      int dim = 0;
      in >> dim;
      dims[b][q] = dim;
    }
  }
  int nnz = 0;
  in >> nnz;
  for (int i = 0; i < nnz; ++i) {
    imps_cpp::hnonzero z{};
    in >> z.row >> z.col >> z.val;
    m.h.push_back(z);
  }
  int nsweeps = 0;
  imps_cpp::vumps_options o;
  int tune = 0, conc = 1;
  in >> nsweeps >> o.fixed_tol >> o.InvETol >> o.eig_margin >> tune >> conc;
  o.autotune = tune != 0;
  o.concurrent = conc != 0;
  std::array<std::vector<double>, 6> init;
  for (int n = 0; n < 2; ++n) {
    const int64_t na = imps_cpp::layout(nsym, imps_cpp::mps_blocks(m.I2K, dims[n], dims[1 - n])).nelem();
    init[n].resize(na);
    init[2 + n].resize(na);
    init[4 + n].resize(imps_cpp::layout(nsym, imps_cpp::bd_blocks(dims[n])).nelem());
  }
  for (int k : {0, 1, 2, 3, 4, 5})
    for (double& x : init[k]) in >> x;
  if (!in) { std::fprintf(stderr, "cpp_vumps_check: malformed input\n"); return 2; }
  try {
    imps_cpp::context ctx(0);
    imps_cpp::vumps v(ctx, m, dims, init, o);
    for (int s = 0; s < nsweeps; ++s) {
      cudaDeviceSynchronize();
      const auto t0 = std::chrono::steady_clock::now();
      const auto E = v.sweep();
      cudaDeviceSynchronize();
      const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      std::printf("sweep %d %.17g %.17g %.17g %.17g %.17g %.17g %.3f %d\n", s, E[0], E[1], v.F[0], v.F[1], v.prec[0],
                  v.prec[1], ms, v.lanczos_applies);
    }
    std::printf("cpp vumps check ok: %d Lanczos applies, %d GMRES iterations\n", v.lanczos_applies, v.gmres_iters);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "cpp_vumps_check: %s\n", e.what());
    return 1;
  }
  return 0;
}
