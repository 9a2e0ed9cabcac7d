// The reference's tile-offload interface (ooc_offload.h:28-64 / ooc_offload.cpp:13-684) on
// the GB300: device memory instead of MIC memory, one CUDA stream per worker rank `r`
// instead of a per-thread bounce buffer, and the library's own FP64 kernels instead of
// MKL inside offload regions.  Every call is synchronous with respect to its caller,
// as the reference's offload regions were.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/ooc_offload.h"
#include "common.cuh"

namespace {

// ---------------------------------------------------------------------------------
// General FP64 contraction for the BLAS-shaped calls:
//   C = alpha * opA * opB^T + beta * C  on all of C, its lower (mask 1) or upper (mask 2)
// triangle, where opA(i,k) = A[i*sar + k*sak] (m x k) and opB(j,k) = B[j*sbr + k*sbk]
// (n x k).  Same DMMA m8n8k4 tiling as the panel update, with strided loads.
// ---------------------------------------------------------------------------------
constexpr int GBM = 64, GBK = 16, GLDS = GBM + 4, GTHR = 128;

__device__ __forceinline__ void dmma(double& c0, double& c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

__device__ __forceinline__ void load_strided(double* S, const double* M, i64 sr, i64 sk, int r0, int rows, int k0,
                                             int kmax) {
  if (sk == 1) {  // k contiguous: walk k fastest
    for (int idx = threadIdx.x; idx < GBM * GBK; idx += GTHR) {
      const int kc = idx % GBK, r = idx / GBK;
      const int gr = r0 + r, gk = k0 + kc;
      S[kc * GLDS + r] = (gr < rows && gk < kmax) ? M[(i64)gr * sr + gk] : 0.0;
    }
  } else {
    for (int idx = threadIdx.x; idx < GBM * GBK; idx += GTHR) {
      const int kc = idx / GBM, r = idx % GBM;
      const int gr = r0 + r, gk = k0 + kc;
      S[kc * GLDS + r] = (gr < rows && gk < kmax) ? M[(i64)gr * sr + (i64)gk * sk] : 0.0;
    }
  }
}

__global__ void __launch_bounds__(GTHR) k_gemm_general(const double* __restrict__ A, i64 sar, i64 sak,
                                                       const double* __restrict__ B, i64 sbr, i64 sbk,
                                                       double* __restrict__ C, i64 ldc, int m, int n, int k,
                                                       double alpha, double beta, int mask) {
  __shared__ __align__(16) double As[GBK * GLDS];
  __shared__ __align__(16) double Bs[GBK * GLDS];
  const int mblocks = (m + GBM - 1) / GBM;
  const int m0 = (blockIdx.x % mblocks) * GBM;
  const int n0 = (blockIdx.x / mblocks) * GBM;
  if (mask == 1 && n0 > m0 + GBM - 1) return;
  if (mask == 2 && m0 > n0 + GBM - 1) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wm = warp & 1, wn = warp >> 1, g = lane >> 2, tig = lane & 3;
  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j][0] = acc[i][j][1] = 0.0;
  for (int k0 = 0; k0 < k; k0 += GBK) {
    load_strided(As, A, sar, sak, m0, m, k0, k);
    load_strided(Bs, B, sbr, sbk, n0, n, k0, k);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; kk += 4) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[(kk + tig) * GLDS + wm * 32 + i * 8 + g];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[(kk + tig) * GLDS + wn * 32 + j * 8 + g];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) dmma(acc[i][j][0], acc[i][j][1], a[i], b[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int r = m0 + wm * 32 + i * 8 + g;
    if (r >= m) continue;
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int c = n0 + wn * 32 + j * 8 + 2 * tig + h;
        if (c >= n || (mask == 1 && c > r) || (mask == 2 && c < r)) continue;
        double* p = C + r + (i64)c * ldc;
        *p = (beta == 0.0) ? alpha * acc[i][j][h] : fma(alpha, acc[i][j][h], beta * *p);
      }
  }
}

// C = beta * C on a triangle or all of it (k == 0 or alpha == 0 BLAS cases).
__global__ void k_scale(double* C, i64 ldc, int m, int n, double beta, int mask) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  for (int c = blockIdx.y; c < n; c += gridDim.y) {
    if ((mask == 1 && c > r) || (mask == 2 && c < r)) continue;
    double* p = C + r + (i64)c * ldc;
    *p = (beta == 0.0) ? 0.0 : beta * *p;
  }
}

// Lower-form copy of a triangular matrix: L(i,j) = T(i,j) (uplo L) or T(j,i) (uplo U) for
// i >= j, with a unit diagonal when requested; zero above.
// Lower triangle M (order n, zero above the diagonal) read from the triangle T through one
// of four index maps, so that every dtrsm form becomes the column solve W := W M^-T:
//   mode 0: M = L          M(i,j) = T(i, j)
//   mode 1: M = U^T        M(i,j) = T(j, i)
//   mode 2: M = J L^T J    M(i,j) = T(n-1-j, n-1-i)   (J reverses the order)
//   mode 3: M = J U J      M(i,j) = T(n-1-i, n-1-j)
// A unit diagonal is written as ones (T's diagonal is not read).
__global__ void k_tri_form(const double* T, i64 ldt, double* M, i64 ldm, int n, int mode, int unit) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int j = blockIdx.y; j < n; j += gridDim.y) {
    double v = 0.0;
    if (i > j || (i == j && !unit)) {
      int r = i, c = j;
      if (mode == 1) { r = j; c = i; }
      else if (mode == 2) { r = n - 1 - j; c = n - 1 - i; }
      else if (mode == 3) { r = n - 1 - i; c = n - 1 - j; }
      v = T[r + (i64)c * ldt];
    } else if (i == j) {
      v = 1.0;
    }
    M[i + (i64)j * ldm] = v;
  }
}

// W (rows x cols, ld ldw) <-> B: W(i, j) sits at S(i, rev ? cols-1-j : j) with S = B or B^T.
// TO_W: W = alpha * that element; otherwise the element = W(i, j).
template <bool TO_W>
__global__ void k_b_map(double* B, i64 ldb, double* W, i64 ldw, int rows, int cols, int trans, int rev,
                        double alpha) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  for (int j = blockIdx.y; j < cols; j += gridDim.y) {
    const int jj = rev ? cols - 1 - j : j;
    double* e = trans ? &B[jj + (i64)i * ldb] : &B[i + (i64)jj * ldb];
    if (TO_W) W[i + (i64)j * ldw] = alpha * *e;
    else *e = W[i + (i64)j * ldw];
  }
}

// Transposed copy of the upper triangle into / out of lower form.
__global__ void k_upper_to_lower(const double* A, i64 lda, double* L, i64 ldl, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int j = blockIdx.y; j <= i && j < n; j += gridDim.y) L[i + (i64)j * ldl] = A[j + (i64)i * lda];
}
__global__ void k_lower_to_upper(const double* L, i64 ldl, double* A, i64 lda, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int j = blockIdx.y; j <= i && j < n; j += gridDim.y) A[j + (i64)i * lda] = L[i + (i64)j * ldl];
}

// ---------------------------------------------------------------------------------
// Per-thread state: the device chosen by offload_init, a stream and a status word per
// worker rank, and the last error.
// ---------------------------------------------------------------------------------
constexpr int MAX_R = 64;
int g_device = 0;
std::mutex g_mu;
struct Slot {
  cudaStream_t s = nullptr;
  int* status = nullptr;
};
Slot g_slot[MAX_R];
thread_local int t_err = 0;

bool ok_char(char c, const char* set) { return std::strchr(set, c) != nullptr && c != 0; }
char up(char c) { return (c >= 'a' && c <= 'z') ? (char)(c - 32) : c; }

Slot* slot(int r) {
  if (r < 0 || r >= MAX_R) { t_err = OOC_ERR_INTERNAL; return nullptr; }
  std::lock_guard<std::mutex> lk(g_mu);
  cudaSetDevice(g_device);
  Slot& sl = g_slot[r];
  if (!sl.s) {
    if (cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&sl.status, sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      t_err = OOC_ERR_CUDA;
      return nullptr;
    }
  }
  return &sl;
}

int finish(cudaStream_t s) {
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    ooc_set_last_error(e, "offload call", __FILE__, __LINE__);
    t_err = OOC_ERR_CUDA;
    return OOC_ERR_CUDA;
  }
  return OOC_OK;
}

void gemm_general(const double* A, i64 sar, i64 sak, const double* B, i64 sbr, i64 sbk, double* C, i64 ldc, int m,
                  int n, int k, double alpha, double beta, int mask, cudaStream_t s) {
  if (m <= 0 || n <= 0) return;
  if (k <= 0 || alpha == 0.0) {
    if (beta != 1.0)
      k_scale<<<dim3((m + 255) / 256, std::min(n, 4096)), 256, 0, s>>>(C, ldc, m, n, beta, mask);
    return;
  }
  const int mb = (m + GBM - 1) / GBM, nbk = (n + GBM - 1) / GBM;
  k_gemm_general<<<mb * nbk, GTHR, 0, s>>>(A, sar, sak, B, sbr, sbk, C, ldc, m, n, k, alpha, beta, mask);
}

}  // namespace

// =================================================================================
// C-ABI
// =================================================================================
extern "C" int ooc_offload_last_error(void) { return t_err; }

extern "C" void offload_init(int* myrank, int* mydevice) {
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd <= 0) {
    cudaGetLastError();
    t_err = OOC_ERR_NODEVICE;
    if (mydevice) *mydevice = -1;
    return;
  }
  const int rank = myrank ? *myrank : 0;
  g_device = ((rank % nd) + nd) % nd;  // ooc_offload.cpp:15-19
  if (mydevice) *mydevice = g_device;
  cudaSetDevice(g_device);
  t_err = 0;
}
extern "C" void offload_init_(int* myrank, int* mydevice) { offload_init(myrank, mydevice); }

extern "C" void offload_destroy(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  cudaSetDevice(g_device);
  for (Slot& sl : g_slot) {
    if (sl.s) { cudaStreamSynchronize(sl.s); cudaStreamDestroy(sl.s); sl.s = nullptr; }
    if (sl.status) { cudaFree(sl.status); sl.status = nullptr; }
  }
}
extern "C" void offload_destroy_(void) { offload_destroy(); }

extern "C" intptr_t offload_Alloc(size_t size, int r) {
  (void)r;
  cudaSetDevice(g_device);
  void* p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(size, 1)) != cudaSuccess) {
    cudaGetLastError();
    t_err = OOC_ERR_NOMEM;
    return 0;
  }
  return (intptr_t)p;
}

// The reference reads every byte on the MIC to fault the pages in (ooc_offload.cpp:49-78);
// device memory from cudaMalloc is resident, so there is nothing to do.
extern "C" void offload_touch(void* p, size_t size, int r) { (void)p; (void)size; (void)r; }

extern "C" void offload_Free(void* p, int r) {
  (void)r;
  cudaSetDevice(g_device);
  if (p && cudaFree(p) != cudaSuccess) { cudaGetLastError(); t_err = OOC_ERR_CUDA; }
}

static void vec_copy(int n, const double* x, int incx, double* y, int incy, int r, cudaMemcpyKind kind) {
  if (n <= 0) return;
  if (incx <= 0 || incy <= 0) { t_err = -3; return; }
  Slot* sl = slot(r);
  if (!sl) return;
  if (cudaMemcpy2DAsync(y, (size_t)incy * 8, x, (size_t)incx * 8, 8, n, kind, sl->s) != cudaSuccess) {
    cudaGetLastError();
    t_err = OOC_ERR_CUDA;
    return;
  }
  finish(sl->s);
}

extern "C" void offload_dSetVector(int n, double* x, int incx, double* y, int incy, int r) {
  vec_copy(n, x, incx, y, incy, r, cudaMemcpyHostToDevice);
}
extern "C" void offload_dGetVector(int n, double* x, int incx, double* y, int incy, int r) {
  // ooc_offload.cpp:128-176: x on the device, y on the host
  vec_copy(n, x, incx, y, incy, r, cudaMemcpyDeviceToHost);
}
extern "C" void offload_dcopy(int n, const double* x, int incx, double* y, int incy, int r) {
  vec_copy(n, x, incx, y, incy, r, cudaMemcpyDeviceToDevice);
}

static void mat_copy(int rows, int cols, const double* A, int lda, double* B, int ldb, int r, cudaMemcpyKind kind) {
  if (rows <= 0 || cols <= 0) return;
  if (lda < rows || ldb < rows) { t_err = -4; return; }
  Slot* sl = slot(r);
  if (!sl) return;
  if (cudaMemcpy2DAsync(B, (size_t)ldb * 8, A, (size_t)lda * 8, (size_t)rows * 8, cols, kind, sl->s) != cudaSuccess) {
    cudaGetLastError();
    t_err = OOC_ERR_CUDA;
    return;
  }
  finish(sl->s);
}

extern "C" void offload_dSetMatrix(int rows, int cols, double* A, int lda, double* B, int ldb, int r) {
  mat_copy(rows, cols, A, lda, B, ldb, r, cudaMemcpyHostToDevice);
}
extern "C" void offload_dGetMatrix(int rows, int cols, double* A, int lda, double* B, int ldb, int r) {
  mat_copy(rows, cols, A, lda, B, ldb, r, cudaMemcpyDeviceToHost);
}

// Triangular (trapezoidal) copies: lower = rows j..rows-1 of columns j < min(rows, cols);
// upper = rows 0..min(j, rows-1) of each column (ooc_offload.cpp:398-605).
static void tr_copy(char uplo, int rows, int cols, const double* A, int lda, double* B, int ldb, int r,
                    cudaMemcpyKind kind) {
  if (rows <= 0 || cols <= 0) return;
  const char u = up(uplo);
  if (u != 'L' && u != 'U') { t_err = -1; return; }
  if (lda < rows || ldb < rows) { t_err = -5; return; }
  Slot* sl = slot(r);
  if (!sl) return;
  const int nc = (u == 'L') ? std::min(rows, cols) : cols;
  for (int j = 0; j < nc; j++) {
    const int r0 = (u == 'L') ? j : 0;
    const int r1 = (u == 'L') ? rows : std::min(j + 1, rows);
    if (r1 <= r0) continue;
    if (cudaMemcpyAsync(B + r0 + (i64)j * ldb, A + r0 + (i64)j * lda, (size_t)(r1 - r0) * 8, kind, sl->s) !=
        cudaSuccess) {
      cudaGetLastError();
      t_err = OOC_ERR_CUDA;
      return;
    }
  }
  finish(sl->s);
}

extern "C" void offload_dtrSetMatrix(char uplo, int rows, int cols, double* A, int lda, double* B, int ldb, int r) {
  tr_copy(uplo, rows, cols, A, lda, B, ldb, r, cudaMemcpyHostToDevice);
}
extern "C" void offload_dtrGetMatrix(char uplo, int rows, int cols, double* A, int lda, double* B, int ldb, int r) {
  tr_copy(uplo, rows, cols, A, lda, B, ldb, r, cudaMemcpyDeviceToHost);
}

extern "C" void offload_dgemm(const char* transa, const char* transb, const MKL_INT* m, const MKL_INT* n,
                              const MKL_INT* k, const double* alpha, const double* a, const MKL_INT* lda,
                              const double* b, const MKL_INT* ldb, const double* beta, double* c,
                              const MKL_INT* ldc, int r) {
  const char ta = up(*transa), tb = up(*transb);
  if (!ok_char(ta, "NTC")) { t_err = -1; return; }
  if (!ok_char(tb, "NTC")) { t_err = -2; return; }
  if (*m < 0) { t_err = -3; return; }
  if (*n < 0) { t_err = -4; return; }
  if (*k < 0) { t_err = -5; return; }
  if (*ldc < std::max(1, *m)) { t_err = -13; return; }
  Slot* sl = slot(r);
  if (!sl) return;
  // opA(i,kk): N -> a[i + kk*lda], T -> a[kk + i*lda]
  const i64 sar = (ta == 'N') ? 1 : *lda, sak = (ta == 'N') ? *lda : 1;
  // opB as (n x k): opB(kk, j) = N -> b[kk + j*ldb], T -> b[j + kk*ldb]
  const i64 sbr = (tb == 'N') ? *ldb : 1, sbk = (tb == 'N') ? 1 : *ldb;
  gemm_general(a, sar, sak, b, sbr, sbk, c, *ldc, *m, *n, *k, *alpha, *beta, 0, sl->s);
  finish(sl->s);
}

extern "C" void offload_dsyrk(const char* uplo, const char* trans, const MKL_INT* n, const MKL_INT* k,
                              const double* alpha, const double* a, const MKL_INT* lda, const double* beta, double* c,
                              const MKL_INT* ldc, int r) {
  const char u = up(*uplo), t = up(*trans);
  if (u != 'L' && u != 'U') { t_err = -1; return; }
  if (!ok_char(t, "NTC")) { t_err = -2; return; }
  if (*n < 0) { t_err = -3; return; }
  if (*k < 0) { t_err = -4; return; }
  if (*ldc < std::max(1, *n)) { t_err = -10; return; }
  Slot* sl = slot(r);
  if (!sl) return;
  // trans N: C = alpha A A^T + beta C, A n x k; trans T: C = alpha A^T A + beta C, A k x n
  const i64 sr = (t == 'N') ? 1 : *lda, sk = (t == 'N') ? *lda : 1;
  gemm_general(a, sr, sk, a, sr, sk, c, *ldc, *n, *n, *k, *alpha, *beta, u == 'L' ? 1 : 2, sl->s);
  finish(sl->s);
}

extern "C" void offload_dtrsm(const char* side, const char* uplo, const char* transa, const char* diag,
                              const MKL_INT* m, const MKL_INT* n, const double* alpha, const double* a,
                              const MKL_INT* lda, double* b, const MKL_INT* ldb, int r) {
  const char sd = up(*side), u = up(*uplo), t = up(*transa), d = up(*diag);
  if (sd != 'L' && sd != 'R') { t_err = -1; return; }
  if (u != 'L' && u != 'U') { t_err = -2; return; }
  if (!ok_char(t, "NTC")) { t_err = -3; return; }
  if (d != 'N' && d != 'U') { t_err = -4; return; }
  if (*m < 0) { t_err = -5; return; }
  if (*n < 0) { t_err = -6; return; }
  const int kdim = (sd == 'L') ? *m : *n;
  if (*lda < std::max(1, kdim)) { t_err = -9; return; }
  if (*ldb < std::max(1, *m)) { t_err = -11; return; }
  if (*m == 0 || *n == 0) return;
  Slot* sl = slot(r);
  if (!sl) return;
  cudaStream_t s = sl->s;
  cudaMemsetAsync(sl->status, 0, sizeof(int), s);
  if (sd == 'R' && u == 'L' && t != 'N' && d == 'N') {
    // The form the reference uses (oocquark.cpp:407): B := alpha B L^-T, the library's
    // blocked column solve directly.
    if (*alpha != 1.0) gemm_general(nullptr, 0, 0, nullptr, 0, 0, b, *ldb, *m, *n, 0, 0.0, *alpha, 0, s);
    int rc = launch_trsm_col(a, *lda, TileCol{b, *ldb, 0}, 1, *m, *m, *n, sl->status, s);
    if (rc) t_err = rc;
    finish(s);
    return;
  }
  // Every other form is the same column solve (substitution, no explicit inverse) on
  // rearranged copies.  Side L transposes first: op(T) X = B  <=>  X^T op(T)^T = B^T.
  // On side R, X op(T) = B with op(T) = L^T is the direct form (M = L); U = (U^T)^T gives
  // M = U^T; a lower (or upper-transposed) right factor is reversed into an upper one,
  // X L J = B J  <=>  (X J)(J L J) = B J, whose transpose-lower form is M = J L^T J
  // (J U J for X U^T = B), with the columns of B and of the result in reverse order.
  const bool tr = (sd == 'L');
  const char te = tr ? (t == 'N' ? 'T' : 'N') : (t == 'N' ? 'N' : 'T');  // the side-R form's op
  const int mode = (u == 'L') ? (te == 'T' ? 0 : 2) : (te == 'N' ? 1 : 3);
  const int rev = mode >= 2;
  const int rows = tr ? *n : *m;  // W = alpha * (B or B^T), rows x kdim, columns maybe reversed
  double *M = nullptr, *W = nullptr;
  if (cudaMalloc(&M, (size_t)kdim * kdim * 8) != cudaSuccess || cudaMalloc(&W, (size_t)rows * kdim * 8) != cudaSuccess) {
    cudaGetLastError();
    if (M) cudaFree(M);
    t_err = OOC_ERR_NOMEM;
    return;
  }
  dim3 gm((kdim + 255) / 256, std::min(kdim, 4096)), gw((rows + 255) / 256, std::min(kdim, 4096));
  k_tri_form<<<gm, 256, 0, s>>>(a, *lda, M, kdim, kdim, mode, d == 'U');
  k_b_map<true><<<gw, 256, 0, s>>>(b, *ldb, W, rows, rows, kdim, tr, rev, *alpha);
  int rc = launch_trsm_col(M, kdim, TileCol{W, rows, 0}, 1, rows, rows, kdim, sl->status, s);
  if (rc) t_err = rc;
  k_b_map<false><<<gw, 256, 0, s>>>(b, *ldb, W, rows, rows, kdim, tr, rev, 1.0);
  if (cudaGetLastError() != cudaSuccess) t_err = OOC_ERR_CUDA;
  finish(s);
  cudaFree(M);
  cudaFree(W);
}

extern "C" void offload_dpotrf(const char* uplo, const MKL_INT* n, double* a, const MKL_INT* lda, MKL_INT* info,
                               int r) {
  const char u = up(*uplo);
  if (!info) return;
  *info = 0;
  if (u != 'L' && u != 'U') { *info = -1; return; }
  if (*n < 0) { *info = -2; return; }
  if (*lda < std::max(1, *n)) { *info = -4; return; }
  if (*n == 0) return;
  Slot* sl = slot(r);
  if (!sl) { *info = t_err; return; }
  cudaStream_t s = sl->s;
  cudaMemsetAsync(sl->status, 0, sizeof(int), s);
  int rc;
  if (u == 'L') {
    rc = launch_potrf_tile(a, *lda, *n, 0, sl->status, s);
  } else {
    // A = U^T U: factor the transposed upper triangle as a lower one, then write U back.
    double* Lw = nullptr;
    if (cudaMalloc(&Lw, (size_t)(*n) * (*n) * 8) != cudaSuccess) {
      cudaGetLastError();
      *info = OOC_ERR_NOMEM;
      return;
    }
    dim3 g2((*n + 255) / 256, std::min(*n, 4096));
    k_upper_to_lower<<<g2, 256, 0, s>>>(a, *lda, Lw, *n, *n);
    rc = launch_potrf_tile(Lw, *n, *n, 0, sl->status, s);
    k_lower_to_upper<<<g2, 256, 0, s>>>(Lw, *n, a, *lda, *n);
    cudaStreamSynchronize(s);
    cudaFree(Lw);
  }
  int st = 0;
  cudaMemcpyAsync(&st, sl->status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (finish(s) != OOC_OK) { *info = OOC_ERR_CUDA; return; }
  *info = rc ? rc : st;  // returned through an out clause in the reference (ooc_offload.cpp:679)
}
