// Harness around the reference's own Cholesky() (oocdag.cpp:18-112, compiled unmodified
// from the reference tree together with oocquark.cpp by oracle/ref_build.py).
//
// TEST INFRASTRUCTURE ONLY: its outputs check the oracle (tests/test_ref_build.py) and
// make the golden fixtures of tests/golden/gen_ref_run.py.  One factorization per
// process, because the reference's find_Yn keeps a function-local static between calls
// (oocdag.cpp:480).
//
//   oocdag_ref plan N NB memsize_bytes
//       Dry run: Cholesky's panel loop runs and inserts every task, none is executed and
//       no matrix memory is touched except the element the driver prints at the end.
//       Prints the driver's own per-panel line ("bb .. jb .. YM .. YN .. Ym .. Yn ..")
//       and one "tasks" line with the count per task body.
//   oocdag_ref run N NB LDA memsize_bytes blas_path blas_prefix in.f64 out.f64
//       Reads A (LDA x N, column-major FP64) from in.f64, factors it with the reference's
//       Cholesky on the host stand-ins, writes A (L in the lower triangle) to out.f64,
//       then prints the "tasks" line and "info <first failing dpotrf info>".

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <unistd.h>

#include "oocdag.h"
#include "shim.h"

double Cholesky(Quark* quark, double* A, int N, int NB, int LDA, size_t memsize);

static void print_tasks() {
  printf("tasks H2D %lld D2H %lld potrf %lld trsm %lld syrk %lld gemm %lld\n", ooc_shim_task_count(CORE_H2D),
         ooc_shim_task_count(CORE_D2H), ooc_shim_task_count(CORE_incore_dpotrf),
         ooc_shim_task_count(CORE_incore_dtrsm), ooc_shim_task_count(CORE_incore_dsyrk),
         ooc_shim_task_count(CORE_incore_dgemm));
}

static int plan(int N, int NB, size_t memsize) {
  ooc_shim_set_dry(1);
  const size_t LDA = (size_t)N;
  const size_t bytes = LDA * (size_t)N * sizeof(double);
  // The matrix is an inaccessible range except for the page of the one element the
  // driver reads, for its closing printf (oocdag.cpp:92).  That index is formed in int
  // arithmetic, (N-1)*LDA + N-1, which wraps for N > 46341; the element read is then up
  // to 16 GiB before or after A, so that much inaccessible room is reserved on each
  // side and the page of the wrapped address is made readable.
  const size_t guard = (size_t)1 << 34;
  char* R = (char*)mmap(nullptr, bytes + 2 * guard, PROT_NONE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
  if (R == MAP_FAILED) {
    perror("mmap");
    return 2;
  }
  char* A = R + guard;
  const long long wrapped = (long long)(int)(unsigned)((unsigned long long)(N - 1) * LDA) + (N - 1);
  const long long idx = (long long)(int)(unsigned)(unsigned long long)wrapped;
  const size_t pg = (size_t)sysconf(_SC_PAGESIZE);
  char* at = A + idx * (long long)sizeof(double);
  char* page = R + ((size_t)(at - R) / pg) * pg;
  if (mprotect(page, pg, PROT_READ | PROT_WRITE) != 0) {
    perror("mprotect");
    return 2;
  }
  Quark* q = QUARK_New(OOC_NTHREADS);
  Cholesky(q, (double*)A, N, NB, (int)LDA, memsize);
  QUARK_Delete(q);
  print_tasks();
  munmap(R, bytes + 2 * guard);
  return 0;
}

static int run(int N, int NB, int LDA, size_t memsize, const char* blas, const char* prefix, const char* in,
               const char* out) {
  if (ooc_shim_init_blas(blas, prefix) != 0) return 3;
  const size_t count = (size_t)LDA * (size_t)N;
  double* A = (double*)aligned_alloc(64, ((count * sizeof(double) + 63) / 64) * 64);
  FILE* f = fopen(in, "rb");
  if (!f || fread(A, sizeof(double), count, f) != count) {
    fprintf(stderr, "cannot read %zu doubles from %s\n", count, in);
    return 4;
  }
  fclose(f);
  for (int r = 0; r < OOC_NTHREADS; r++) cublasCreate(&worker_handle[r]);
  Quark* q = QUARK_New(OOC_NTHREADS);
  double t = Cholesky(q, A, N, NB, LDA, memsize);
  QUARK_Delete(q);
  for (int r = 0; r < OOC_NTHREADS; r++) cublasDestroy(worker_handle[r]);
  f = fopen(out, "wb");
  if (!f || fwrite(A, sizeof(double), count, f) != count) {
    fprintf(stderr, "cannot write %s\n", out);
    return 5;
  }
  fclose(f);
  free(A);
  print_tasks();
  printf("info %d\nseconds %.6f\n", ooc_shim_first_potrf_failure(), t);
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 5 && !strcmp(argv[1], "plan")) return plan(atoi(argv[2]), atoi(argv[3]), strtoull(argv[4], 0, 10));
  if (argc == 10 && !strcmp(argv[1], "run"))
    return run(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), strtoull(argv[5], 0, 10), argv[6], argv[7], argv[8],
               argv[9]);
  fprintf(stderr,
          "usage: %s plan N NB memsize_bytes\n"
          "       %s run N NB LDA memsize_bytes blas_path blas_prefix in.f64 out.f64\n",
          argv[0], argv[0]);
  return 1;
}
