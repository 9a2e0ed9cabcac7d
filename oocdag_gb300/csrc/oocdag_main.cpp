// Command-line driver with the reference's interface (oocdag.cpp:223-370):
//
//   oocdag N NB memsize_MB [--verify] [--uniform ALPHA] [--seed S]
//
// generates the reference's test matrix (pdmatgen('Symm','Diag'), seed 100, as
// oocdag.cpp:298-302 does; --uniform switches to (R+R^T)/2 + ALPHA I), factors it out of
// core through a device budget of memsize_MB MiB with the drop-in Cholesky() entry, and
// prints the reference's result line (its GFLOPS convention: (N/3 + 0.5) N^2 / t / 2^30)
// followed by TFLOP/s with n^3/3 flops and the LAPACK info.  --verify regenerates A tile by
// tile and prints the scaled residual ||A - L L^T||_F / (n eps ||A||_F) (the reference's
// VERIFY block, oocdag.cpp:379-464, checks with dpotrs instead).
//
// Only the library's C-ABI is used (include/oocdag_gb300.h); the host matrix is ordinary
// pageable memory, page-locked by the library for the call.

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "oocdag_gb300.h"

static int usage() {
  std::fprintf(stderr, "invalid arguments N NB memsize(M) [--verify] [--uniform ALPHA] [--seed S]\n");
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 4) return usage();
  const long long N = std::atoll(argv[1]);
  const int NB = std::atoi(argv[2]);
  const size_t memsize = (size_t)std::atoll(argv[3]) * 1024 * 1024;
  bool verify = false, uniform = false;
  double alpha = 0.0;
  long long seed = 100;  // IASEED, oocdag.cpp:233
  for (int i = 4; i < argc; i++) {
    if (!std::strcmp(argv[i], "--verify")) verify = true;
    else if (!std::strcmp(argv[i], "--uniform") && i + 1 < argc) { uniform = true; alpha = std::atof(argv[++i]); }
    else if (!std::strcmp(argv[i], "--seed") && i + 1 < argc) seed = std::atoll(argv[++i]);
    else return usage();
  }
  if (N <= 0 || NB <= 0 || memsize == 0) return usage();
  ooc_handle* h = nullptr;
  int rc = ooc_create(&h, 0);
  if (rc) {
    std::fprintf(stderr, "ooc_create failed (%d): %s\n", rc, ooc_last_error_string());
    return 2;
  }
  std::vector<double> A((size_t)N * N);
  rc = uniform ? ooc_dmatgen_uniform(h, A.data(), N, N, (uint64_t)seed, alpha)
               : ooc_dmatgen_pdmatgen(h, A.data(), N, N, (int)seed);
  if (rc) {
    std::fprintf(stderr, "matrix generation failed (%d): %s\n", rc, ooc_last_error_string());
    return 2;
  }
  const double t = Cholesky(h, A.data(), (int)N, NB, (int)N, memsize);
  if (t < 0) {
    std::fprintf(stderr, "Cholesky failed (%d): %s\n", (int)t, ooc_last_error_string());
    return 2;
  }
  const int info = ooc_last_info(h);
  const double n = (double)N;
  const double gflops = (n / 3.0 + 0.5) * n * n / t / 1024.0 / 1024.0 / 1024.0;
  std::printf("N NB memsize(MB) streams time Gflops\n%lld %d %lf %d %lf %lf\n", N, NB,
              (double)memsize / 1024 / 1024, 3, t, gflops);
  std::printf("TFLOP/s (n^3/3) %.4f info %d\n", n * n * n / 3.0 / t / 1e12, info);
  if (verify && info == 0) {
    double r = 0.0;
    rc = ooc_dresidual(h, A.data(), N, N, uniform ? 0 : 1, (uint64_t)seed, alpha, &r);
    if (rc) {
      std::fprintf(stderr, "residual failed (%d): %s\n", rc, ooc_last_error_string());
      return 2;
    }
    std::printf("scaled residual ||A - L L^T||_F / (n eps ||A||_F) = %.3f\n", r);
  }
  ooc_destroy(h);
  return info == 0 ? 0 : 3;
}
