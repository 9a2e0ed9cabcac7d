// Host implementations behind the stand-in headers in include/ (QUARK, cuBLAS v2, the
// CUDA runtime's cudaMalloc/cudaFree, MPI_Wtime, MKL dpotrf_, BLACS), so that the
// reference's own oocdag.cpp and oocquark.cpp compile and run unmodified on the CPU.
//
// TEST INFRASTRUCTURE ONLY (the compiled reference in oracle/_ref checks the oracle).
// The level-3 BLAS and dpotrf_ forward to a host BLAS/LAPACK loaded at run time
// (ooc_shim_init_blas); tasks run at insertion, in program order (see quark.h).

#include "shim.h"

#include <dlfcn.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <time.h>

#include <map>
#include <string>
#include <vector>

#include "cublas_v2.h"
#include "mkl.h"
#include "mkl_blacs.h"
#include "mpi.h"
#include "quark.h"

// ---- host BLAS / LAPACK (Fortran ABI, LP64, trailing hidden string lengths) ----------
typedef void (*dgemm_t)(const char*, const char*, const int*, const int*, const int*, const double*,
                        const double*, const int*, const double*, const int*, const double*, double*,
                        const int*, size_t, size_t);
typedef void (*dsyrk_t)(const char*, const char*, const int*, const int*, const double*, const double*,
                        const int*, const double*, double*, const int*, size_t, size_t);
typedef void (*dtrsm_t)(const char*, const char*, const char*, const char*, const int*, const int*,
                        const double*, const double*, const int*, double*, const int*, size_t, size_t,
                        size_t, size_t);
typedef void (*dpotrf_t)(const char*, const int*, double*, const int*, int*, size_t);
typedef void (*nthreads_t)(int);

static dgemm_t p_dgemm;
static dsyrk_t p_dsyrk;
static dtrsm_t p_dtrsm;
static dpotrf_t p_dpotrf;

int ooc_shim_init_blas(const char* path, const char* prefix) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    fprintf(stderr, "ref shim: dlopen(%s): %s\n", path, dlerror());
    return -1;
  }
  std::string p(prefix ? prefix : "");
  p_dgemm = (dgemm_t)dlsym(h, (p + "dgemm_").c_str());
  p_dsyrk = (dsyrk_t)dlsym(h, (p + "dsyrk_").c_str());
  p_dtrsm = (dtrsm_t)dlsym(h, (p + "dtrsm_").c_str());
  p_dpotrf = (dpotrf_t)dlsym(h, (p + "dpotrf_").c_str());
  nthreads_t nt = (nthreads_t)dlsym(h, (p + "openblas_set_num_threads").c_str());
  if (!p_dgemm || !p_dsyrk || !p_dtrsm || !p_dpotrf) {
    fprintf(stderr, "ref shim: BLAS symbols with prefix '%s' missing in %s\n", p.c_str(), path);
    return -2;
  }
  if (nt) nt(1);  // one thread per task body, as the reference links sequential MKL
  return 0;
}

// ---- dry run: tasks are counted, never executed; "device" memory is never touched -----
static int g_dry = 0;
void ooc_shim_set_dry(int dry) { g_dry = dry; }

// ---- QUARK ------------------------------------------------------------------------------
struct ooc_shim_quark {
  int nthreads = 1;
  std::vector<unsigned char> args;  // packed arguments of the task now running
};
static std::map<void (*)(Quark*), long long> g_task_counts;

long long ooc_shim_task_count(void (*fn)(Quark*)) {
  auto it = g_task_counts.find(fn);
  return it == g_task_counts.end() ? 0 : it->second;
}

Quark* QUARK_New(int nthreads) {
  Quark* q = new Quark;
  q->nthreads = nthreads;
  return q;
}
void QUARK_Delete(Quark* q) { delete q; }
void QUARK_Barrier(Quark*) {}  // every task has already run
int QUARK_Thread_Rank(Quark*) { return 0; }
void QUARK_DOT_DAG_Enable(Quark*, int) {}
int quark_getenv_int(const char* name, int dflt) {
  const char* v = getenv(name);
  return v ? atoi(v) : dflt;
}
Quark_Task_Flags* QUARK_Task_Flag_Set(Quark_Task_Flags* f, int flag, intptr_t val) {
  switch (flag) {
    case TASK_COLOR: f->color = val; break;
    case TASK_LABEL: f->label = val; break;
    case TASK_PRIORITY: f->priority = val; break;
    case TASK_LOCK_TO_THREAD_MASK: f->thread_mask = val; break;
    case TASK_LOCK_TO_THREAD: f->thread = val; break;
    default: break;
  }
  return f;
}

// Argument list: (size, pointer, mode) triples ended by a size of 0.  The sizes are
// sizeof expressions (size_t) and the terminator an int literal; like QUARK, read
// each size as an int (the low half of the 64-bit argument slot on LP64 targets).
unsigned long long QUARK_Insert_Task(Quark* q, void (*fn)(Quark*), Quark_Task_Flags* flags, ...) {
  g_task_counts[fn]++;
  if (g_dry) return 0;
  std::vector<unsigned char> packed;
  va_list ap;
  va_start(ap, flags);
  for (;;) {
    int size = va_arg(ap, int);
    if (size == 0) break;
    void* ptr = va_arg(ap, void*);
    int mode = va_arg(ap, int);
    const unsigned char* src;
    size_t len;
    if (mode & VALUE) {
      src = (const unsigned char*)ptr;
      len = (size_t)size;
    } else {
      src = (const unsigned char*)&ptr;
      len = sizeof(void*);
    }
    packed.insert(packed.end(), src, src + len);
  }
  va_end(ap);
  std::vector<unsigned char> saved;
  saved.swap(q->args);
  q->args.swap(packed);
  fn(q);
  q->args.swap(saved);
  return g_task_counts[fn];
}
const unsigned char* ooc_shim_task_args(Quark* q) { return q->args.data(); }

// ---- CUDA runtime: "device" memory -----------------------------------------------------
static std::map<void*, size_t> g_maps;
cudaError_t cudaMalloc(void** p, size_t bytes) {
  size_t len = bytes ? bytes : 1;
  void* a = mmap(nullptr, len, g_dry ? PROT_NONE : (PROT_READ | PROT_WRITE),
                 MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
  if (a == MAP_FAILED) return cudaErrorMemoryAllocation;
  g_maps[a] = len;
  *p = a;
  return cudaSuccess;
}
cudaError_t cudaFree(void* p) {
  auto it = g_maps.find(p);
  if (it == g_maps.end()) return cudaErrorMemoryAllocation;
  munmap(p, it->second);
  g_maps.erase(it);
  return cudaSuccess;
}

// ---- cuBLAS v2 ---------------------------------------------------------------------------
struct ooc_shim_cublas {
  int unused;
};
cublasStatus_t cublasCreate(cublasHandle_t* h) {
  *h = new ooc_shim_cublas{0};
  return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDestroy(cublasHandle_t h) {
  delete h;
  return CUBLAS_STATUS_SUCCESS;
}
static cublasStatus_t copy2d(int rows, int cols, int es, const void* A, int lda, void* B, int ldb) {
  if (rows < 0 || cols < 0 || es <= 0 || lda < rows || ldb < rows) return CUBLAS_STATUS_INVALID_VALUE;
  for (int j = 0; j < cols; j++)
    memcpy((char*)B + (size_t)j * ldb * es, (const char*)A + (size_t)j * lda * es, (size_t)rows * es);
  return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasSetMatrix(int rows, int cols, int es, const void* A, int lda, void* B, int ldb) {
  return copy2d(rows, cols, es, A, lda, B, ldb);
}
cublasStatus_t cublasGetMatrix(int rows, int cols, int es, const void* A, int lda, void* B, int ldb) {
  return copy2d(rows, cols, es, A, lda, B, ldb);
}
static const char* op_char(cublasOperation_t t) { return t == CUBLAS_OP_N ? "N" : t == CUBLAS_OP_T ? "T" : "C"; }
cublasStatus_t cublasDtrsm_v2(cublasHandle_t, cublasSideMode_t side, cublasFillMode_t uplo, cublasOperation_t trans,
                              cublasDiagType_t diag, int m, int n, const double* alpha, const double* A, int lda,
                              double* B, int ldb) {
  p_dtrsm(side == CUBLAS_SIDE_LEFT ? "L" : "R", uplo == CUBLAS_FILL_MODE_LOWER ? "L" : "U", op_char(trans),
          diag == CUBLAS_DIAG_UNIT ? "U" : "N", &m, &n, alpha, A, &lda, B, &ldb, 1, 1, 1, 1);
  return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDsyrk_v2(cublasHandle_t, cublasFillMode_t uplo, cublasOperation_t trans, int n, int k,
                              const double* alpha, const double* A, int lda, const double* beta, double* C,
                              int ldc) {
  p_dsyrk(uplo == CUBLAS_FILL_MODE_LOWER ? "L" : "U", op_char(trans), &n, &k, alpha, A, &lda, beta, C, &ldc, 1, 1);
  return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDgemm_v2(cublasHandle_t, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                              const double* alpha, const double* A, int lda, const double* B, int ldb,
                              const double* beta, double* C, int ldc) {
  p_dgemm(op_char(ta), op_char(tb), &m, &n, &k, alpha, A, &lda, B, &ldb, beta, C, &ldc, 1, 1);
  return CUBLAS_STATUS_SUCCESS;
}

// ---- MKL LAPACK, MPI, BLACS ----------------------------------------------------------------
static int g_last_potrf_info = 0;
int ooc_shim_first_potrf_failure(void) { return g_last_potrf_info; }
void dpotrf_(const char* uplo, const int* n, double* A, const int* lda, int* info) {
  p_dpotrf(uplo, n, A, lda, info, 1);
  if (*info != 0 && g_last_potrf_info == 0) g_last_potrf_info = *info;
}
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
void blacs_pinfo_(int* iam, int* nprocs) { *iam = 0; *nprocs = 1; }
void blacs_get_(const int*, const int*, int* val) { *val = 0; }
void blacs_gridinit_(int*, const char*, const int*, const int*) {}
void blacs_gridinfo_(const int*, int* nprow, int* npcol, int* myrow, int* mycol) {
  *nprow = *npcol = 1;
  *myrow = *mycol = 0;
}
void blacs_gridexit_(const int*) {}
void blacs_exit_(const int*) {}

// The reference's main() (compiled, never run here) calls the ScaLAPACK test-matrix
// generator, which is Fortran (LIN/pdmatgen.f) and not built; the recipe feeds
// Cholesky() its matrices directly.
extern "C" void pdmatgen(int*, char*, char*, int*, int*, int*, int*, double*, int*, int*, int*, int*, int*, int*,
                         int*, int*, int*, int*, int*, int*) {
  fprintf(stderr, "ref shim: pdmatgen is not part of the compiled reference path\n");
  abort();
}
