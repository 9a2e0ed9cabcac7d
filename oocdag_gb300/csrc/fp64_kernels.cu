// FP64 tile kernels for the out-of-core Cholesky on GB300 (sm_103a).
//
// GB300 executes FP64 at about 1/1800 of its dense BF16 tensor rate: the measured
// FP64 DMMA rate is ~1.05 TFLOP/s per GPU (about two FP64 FMAs per clock per SM).  At
// that rate every FP64 tile operation is bound by the FP64 pipe, not by HBM or shared
// memory, so the kernels here are built to keep the DMMA pipe issuing:
//   * the contraction (gemm / syrk, oocquark.cpp:130,176,222 use cuBLAS there) runs on
//     FP64 tensor-core MMAs (mma.sync m8n8k4 f64) with 64x64 output blocks per CTA,
//     16-deep K slabs double-buffered in shared memory by cp.async;
//   * the diagonal-tile factor (host dpotrf_ at oocquark.cpp:87 in the reference) and
//     the column solve (cublasDtrsm at oocquark.cpp:130) are blocked into 64-wide steps
//     so that almost all of their flops go through the same contraction kernel, with
//     only the 64x64 diagonal pieces done in shared memory.
// Every kernel reads the device status word first and returns at once when an earlier
// step has reported a non-positive-definite minor.

#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"

namespace {

constexpr int BM = 64;
constexpr int BN = 64;
constexpr int BK = 16;
constexpr int PAD = 4;               // row length BM+PAD makes fragment loads conflict-free
constexpr int GEMM_THREADS = 128;    // 4 warps in a 2 x 2 arrangement, 32 x 32 each

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void dmma884(double& c0, double& c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

// Loads rows [r0, r0+BMX) x columns [k0, k0+16) of the column-major operand M (rows
// valid below `rows`, columns below `kmax`) into S[k][r] (row length BMX + PAD).
template <bool VEC, int BMX = BM>
__device__ __forceinline__ void load_slab(double* S, const double* M, i64 ld, int r0, int rows,
                                          int k0, int kmax) {
  constexpr int L = BMX + PAD;
  const int t = threadIdx.x;
  if (VEC) {
#pragma unroll
    for (int it = 0; it < (BMX * BK / 2) / GEMM_THREADS; it++) {
      int idx = t + it * GEMM_THREADS;
      int kc = idx / (BMX / 2);
      int r = (idx % (BMX / 2)) * 2;
      int gr = r0 + r, gk = k0 + kc;
      int nvalid = 0;
      if (gk < kmax) nvalid = min(max(rows - gr, 0), 2);
      const double* src = (nvalid > 0) ? (M + gr + (i64)gk * ld) : M;
      cp_async16(S + kc * L + r, src, nvalid * 8);
    }
  } else {
    for (int idx = t; idx < BMX * BK; idx += GEMM_THREADS) {
      int kc = idx / BMX;
      int r = idx % BMX;
      int gr = r0 + r, gk = k0 + kc;
      S[kc * L + r] = (gr < rows && gk < kmax) ? M[gr + (i64)gk * ld] : 0.0;
    }
  }
}

// C[m0:m0+BMX, n0:n0+BMX] += alpha * A[m0:, 0:k] * B[n0:, 0:k]^T, restricted to the lower
// triangle (row >= column) when `lower` is set.  Four warps in a 2 x 2 arrangement, each
// (BMX/2) x (BMX/2) as (BMX/16)^2 DMMA tiles.  BMX = 32 gives four times as many CTAs for
// the same output (for launches too small to fill the GPU with 64 x 64 blocks); every
// output element takes the same DMMA steps in the same order either way.
template <bool VEC, int BMX = BM>
__device__ __forceinline__ void gemm_block(const double* __restrict__ A, i64 lda,
                                           const double* __restrict__ B, i64 ldb,
                                           double* __restrict__ C, i64 ldc, int m, int n, int k,
                                           int m0, int n0, int lower, double alpha) {
  constexpr int L = BMX + PAD;
  constexpr int TI = BMX / 16;  // DMMA tiles per warp dimension
  constexpr int WT = BMX / 2;   // warp tile
  __shared__ __align__(16) double As[2][BK * L];
  __shared__ __align__(16) double Bs[2][BK * L];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wm = warp & 1, wn = warp >> 1;
  const int g = lane >> 2, tig = lane & 3;

  double acc[TI][TI][2];
#pragma unroll
  for (int i = 0; i < TI; i++)
#pragma unroll
    for (int j = 0; j < TI; j++) acc[i][j][0] = acc[i][j][1] = 0.0;

  const int nslab = (k + BK - 1) / BK;
  if (nslab > 0) {
    load_slab<VEC, BMX>(As[0], A, lda, m0, m, 0, k);
    load_slab<VEC, BMX>(Bs[0], B, ldb, n0, n, 0, k);
    if (VEC) cp_async_commit();
  }
  for (int s = 0; s < nslab; s++) {
    const int cur = s & 1;
    if (s + 1 < nslab) {
      load_slab<VEC, BMX>(As[cur ^ 1], A, lda, m0, m, (s + 1) * BK, k);
      load_slab<VEC, BMX>(Bs[cur ^ 1], B, ldb, n0, n, (s + 1) * BK, k);
      if (VEC) { cp_async_commit(); cp_async_wait<1>(); }
    } else {
      if (VEC) cp_async_wait<0>();
    }
    __syncthreads();
    const double* as = As[cur];
    const double* bs = Bs[cur];
#pragma unroll
    for (int kk = 0; kk < BK; kk += 4) {
      double a[TI], b[TI];
#pragma unroll
      for (int i = 0; i < TI; i++) a[i] = as[(kk + tig) * L + wm * WT + i * 8 + g];
#pragma unroll
      for (int j = 0; j < TI; j++) b[j] = bs[(kk + tig) * L + wn * WT + j * 8 + g];
#pragma unroll
      for (int i = 0; i < TI; i++)
#pragma unroll
        for (int j = 0; j < TI; j++) dmma884(acc[i][j][0], acc[i][j][1], a[i], b[j]);
    }
    __syncthreads();
  }

  // Epilogue, one 8-row group at a time: its loads of C first, then its stores (a load
  // after a store to a possibly aliasing address would wait for memory each time).
#pragma unroll
  for (int i = 0; i < TI; i++) {
    const int r = m0 + wm * WT + i * 8 + g;
    double cv[TI][2];
#pragma unroll
    for (int j = 0; j < TI; j++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int c = n0 + wn * WT + j * 8 + 2 * tig + h;
        const bool ok = r < m && c < n && !(lower && c > r);
        cv[j][h] = ok ? C[r + (i64)c * ldc] : 0.0;
      }
#pragma unroll
    for (int j = 0; j < TI; j++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int c = n0 + wn * WT + j * 8 + 2 * tig + h;
        if (r < m && c < n && !(lower && c > r)) C[r + (i64)c * ldc] = fma(alpha, acc[i][j][h], cv[j][h]);
      }
  }
}

// ---------------------------------------------------------------------------------
// Panel update: every tile pair (i >= j) of a trapezoid, one launch per X column.
// grid.x = 64x64 blocks within a tile, grid.y = tile pair.
// ---------------------------------------------------------------------------------
template <bool VEC>
__global__ void __launch_bounds__(GEMM_THREADS)
k_panel_update(TileCol X, TileMap Cm, int Ht, int Kt, i64 H, i64 Kcols, int K, const int* status) {
  if (status && *(volatile const int*)status) return;
  int p = blockIdx.y;
  int j = 0;
  while (j < Kt && p >= Ht - j) { p -= Ht - j; j++; }
  if (j >= Kt) return;
  const int i = j + p;
  const int nb = Cm.nb;
  const int LM = (int)min((i64)nb, H - (i64)i * nb);
  const int LN = (int)min((i64)nb, Kcols - (i64)j * nb);
  const int mblocks = (nb + BM - 1) / BM;
  const int m0 = (blockIdx.x % mblocks) * BM;
  const int n0 = (blockIdx.x / mblocks) * BN;
  if (m0 >= LM || n0 >= LN) return;
  const int lower = (i == j);
  if (lower && n0 > m0 + BM - 1) return;
  const double* Xi = X.base + (i64)i * X.stride;
  const double* Xj = X.base + (i64)j * X.stride;
  double* Cij = tile_ptr(Cm, i, j);
  gemm_block<VEC>(Xi, X.ld, Xj, X.ld, Cij, Cm.ld, LM, LN, K, m0, n0, lower, -1.0);
}

// ---------------------------------------------------------------------------------
// Batched generic NT gemm: C_z += alpha A_z B_z^T, z = blockIdx.y; the last batch entry
// may have a different row count (m_last).
// ---------------------------------------------------------------------------------
struct GemmBatch {
  const double* A; i64 lda, sA;
  const double* B; i64 ldb, sB;
  double* C; i64 ldc, sC;
  int m, m_last, n, k, lower, batch;
  double alpha;
  int tri_b;  // B lower triangular (B(j, kk) = 0 for kk > j): skip the zero K range
};

template <bool VEC, int BMX = BM>
__global__ void __launch_bounds__(GEMM_THREADS) k_gemm_batched(GemmBatch gb, const int* status) {
  if (status && *(volatile const int*)status) return;
  const int z = blockIdx.y;
  const int m = (z == gb.batch - 1) ? gb.m_last : gb.m;
  const int mblocks = (max(gb.m, gb.m_last) + BMX - 1) / BMX;
  const int m0 = (blockIdx.x % mblocks) * BMX;
  const int n0 = (blockIdx.x / mblocks) * BMX;
  if (m0 >= m || n0 >= gb.n) return;
  if (gb.lower && n0 > m0 + BMX - 1) return;
  const int kmax = gb.tri_b ? min(gb.k, n0 + BMX) : gb.k;
  gemm_block<VEC, BMX>(gb.A + (i64)z * gb.sA, gb.lda, gb.B + (i64)z * gb.sB, gb.ldb,
                       gb.C + (i64)z * gb.sC, gb.ldc, m, gb.n, kmax, m0, n0, gb.lower, gb.alpha);
}

// ---------------------------------------------------------------------------------
// Unblocked lower Cholesky of an n x n block (n <= 64) in shared memory, right-looking.
// LAPACK convention: a pivot that is not > 0 (or is NaN) stops the factorization and
// reports info = col0 + j + 1.
// ---------------------------------------------------------------------------------
constexpr int SB = 64;

__global__ void __launch_bounds__(256) k_potrf_small(double* A, i64 ld, int n, i64 col0, int* status) {
  if (*(volatile int*)status) return;
  __shared__ double S[SB][SB + 1];  // S[col][row]
  __shared__ int failed;
  __shared__ double s_inv;
  const int t = threadIdx.x;
  {  // 64 rows x 4 column groups: 16 loads in flight per thread
    const int r = t & (SB - 1), cg = t >> 6;
#pragma unroll
    for (int i = 0; i < SB / 4; i++) {
      const int c = cg + 4 * i;
      if (r < n && c < n && r >= c) S[c][r] = A[r + (i64)c * ld];
    }
  }
  // Column j's pivot (one FP64 square root and one division, by thread 0).  Thread 0 also
  // owns element (j+1, j+1) in column j's trailing update (row j + 1 + 0, first column
  // group), so it takes the next pivot as soon as that element is final, while the other
  // threads are still updating: two barriers per column, and the serial pivot mostly off
  // the barrier-to-barrier path.
  auto pivot = [&](int j) {
    const double d = S[j][j];
    if (!(d > 0.0)) {
      failed = 1;
      atomicCAS(status, 0, (int)(col0 + j + 1));
    } else {
      const double sq = sqrt(d);
      S[j][j] = sq;
      s_inv = 1.0 / sq;
    }
  };
  if (t == 0) {
    failed = 0;
    if (n > 0) pivot(0);
  }
  __syncthreads();
  for (int j = 0; j < n; j++) {
    if (failed) break;
    const double inv = s_inv;  // read before the barrier below; thread 0 rewrites it after
    for (int r = j + 1 + t; r < n; r += blockDim.x) S[j][r] *= inv;
    __syncthreads();
    // trailing lower triangle: thread t takes row j + 1 + (t mod 64) and every fourth
    // column from j + 1 + (t / 64) up to that row (independent updates, no index division)
    {
      const int r = j + 1 + (t & (SB - 1));
      if (r < n) {
        const double lr = S[j][r];
#pragma unroll 4
        for (int c = j + 1 + (t >> 6); c <= r; c += 4) S[c][r] -= lr * S[j][c];
      }
    }
    if (t == 0 && j + 1 < n) pivot(j + 1);
    __syncthreads();
  }
  // Columns factored before a failure are written back as well (LAPACK leaves the
  // leading part of the factor in place).
  for (int idx = t; idx < n * n; idx += blockDim.x) {
    int c = idx / n, r = idx % n;
    if (r >= c) A[r + (i64)c * ld] = S[c][r];
  }
}

// ---------------------------------------------------------------------------------
// B := B L^-T for a block of up to 64 columns: L is n x n lower (n <= 64), B rows are
// independent.  Four lanes per row, each holding every fourth column in registers, 32 rows
// per CTA of 128 threads; z = blockIdx.y walks a batch of row panels (tiles) with stride
// sB, the last of which has m_last rows.  FP64 issues from each SM sub-partition at about
// one FMA per two clocks, so a row group must spread over the sub-partitions: one thread
// per row left three of them idle and took ~100 us per 64-column step.  Right-looking:
// once x_c is final (computed by its owner lane and passed to the row's other lanes by a
// shuffle), every later column takes its FMA with it, in increasing c, as a substitution
// does.  L sits in shared memory, padded to 64 with the identity, and is read by broadcast;
// x_c = v * (1 / L(c,c)).
// ---------------------------------------------------------------------------------
constexpr int TS_ROWS = 32;                  // rows per CTA
constexpr int TS_LPR = 4;                    // lanes per row
constexpr int TS_THREADS = TS_ROWS * TS_LPR;
constexpr int TS_C = SB / TS_LPR;            // columns per lane

__global__ void __launch_bounds__(TS_THREADS) k_trsm_small(const double* L, i64 ldl, double* B, i64 ldb, i64 sB,
                                                           int m, int m_last, int batch, int n,
                                                           const int* status) {
  if (status && *(volatile const int*)status) return;
  __shared__ __align__(16) double Ls[SB * SB];  // Ls[c * SB + r] = L(r, c)
  __shared__ double Rinv[SB];
  const int t = threadIdx.x, lane = t & 31;
  const int s = t & (TS_LPR - 1);   // this lane holds columns s, s + 4, ...
  const int z = blockIdx.y;
  const int mz = (z == batch - 1) ? m_last : m;
  const int r0 = blockIdx.x * TS_ROWS;
  if (r0 >= mz) return;
  double* Bz = B + (i64)z * sB;
  {  // L column by column, threads down the rows (two columns per pass), 8 loads in flight
    const int r = t & (SB - 1), cg = t / SB;
#pragma unroll 8
    for (int c = cg; c < SB; c += TS_THREADS / SB) {
      double v = (r == c) ? 1.0 : 0.0;
      if (r < n && c < n && r >= c) v = L[r + (i64)c * ldl];
      Ls[c * SB + r] = v;
    }
  }
  __syncthreads();
  if (t < SB) Rinv[t] = 1.0 / Ls[t * SB + t];
  const int row = r0 + t / TS_LPR;
  const int nl = (row < mz) ? n : 0;  // columns this row loads and stores
  double* p = Bz + (row < mz ? row : 0);
  double x[TS_C];
#pragma unroll
  for (int j = 0; j < TS_C; j++) {
    const int q = TS_LPR * j + s;
    x[j] = (q < nl) ? p[(i64)q * ldb] : 0.0;
  }
  __syncthreads();
  const int zero = n >> 30;  // n <= 64: 0 at run time, opaque to the compiler
  const int base = lane & ~(TS_LPR - 1);
#pragma unroll
  for (int c = 0; c < SB; c++) {
    const int i = c / TS_LPR, sc = c % TS_LPR;
    const double xc = __shfl_sync(0xffffffffu, x[i] * Rinv[c], base | sc);  // the owner's x_c
    if (s == sc) x[i] = xc;
    // column c's loads of L wait for x_c (not all hoisted into registers)
    const double* lc = Ls + c * SB + (zero & __double2hiint(xc));
#pragma unroll
    for (int j = 0; j < TS_C; j++) {
      const int q = TS_LPR * j + s;
      if (q > c) x[j] = fma(-xc, lc[q], x[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < TS_C; j++) {
    const int q = TS_LPR * j + s;
    if (q < nl) p[(i64)q * ldb] = x[j];
  }
}

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

}  // namespace

// =================================================================================
// Launchers
// =================================================================================

int launch_panel_update(const TileCol& X, const TileMap& C, int Ht, int Kt, i64 H, i64 Kcols, int K,
                        const int* status, cudaStream_t s) {
  if (Ht <= 0 || Kt <= 0 || K <= 0) return OOC_OK;
  i64 npairs = (i64)Kt * Ht - ((i64)Kt * (Kt - 1)) / 2;
  if (npairs > 65535) return OOC_ERR_INTERNAL;  // a panel never has that many tile pairs
  const int mblocks = (C.nb + BM - 1) / BM;
  const int nblocks = (C.nb + BN - 1) / BN;
  dim3 grid(mblocks * nblocks, (unsigned)npairs);
  bool vec = aligned16(X.base) && aligned16(C.base) && (X.ld % 2 == 0) && (C.ld % 2 == 0) &&
             (X.stride % 2 == 0);
  if (vec) k_panel_update<true><<<grid, GEMM_THREADS, 0, s>>>(X, C, Ht, Kt, H, Kcols, K, status);
  else k_panel_update<false><<<grid, GEMM_THREADS, 0, s>>>(X, C, Ht, Kt, H, Kcols, K, status);
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

static int launch_gemm_batched(const GemmBatch& gb, const int* status, cudaStream_t s) {
  if (gb.batch <= 0 || gb.n <= 0 || (gb.m <= 0 && gb.m_last <= 0)) return OOC_OK;
  if (gb.batch > 65535) return OOC_ERR_INTERNAL;
  const int mb = (max(gb.m, gb.m_last) + BM - 1) / BM;
  const int nbk = (gb.n + BN - 1) / BN;
  dim3 grid(mb * nbk, gb.batch);
  bool vec = aligned16(gb.A) && aligned16(gb.B) && aligned16(gb.C) && gb.lda % 2 == 0 &&
             gb.ldb % 2 == 0 && gb.sA % 2 == 0 && gb.sB % 2 == 0;
  if (gb.k <= 0) return OOC_OK;
  // Fewer 64 x 64 blocks than two per SM: 32 x 32 blocks, four times as many CTAs (the
  // FP64 pipe of an SM does ~2 FMAs per clock, so a 64 x 64 x 64 block alone takes ~75 us)
  static int nsm = [] {
    int d = 0, v = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d);
    return v > 0 ? v : 1;
  }();
  if ((i64)mb * nbk * gb.batch < 2LL * nsm && (i64)gb.batch <= 65535) {
    const int mb32 = (max(gb.m, gb.m_last) + 31) / 32, nb32 = (gb.n + 31) / 32;
    dim3 g32(mb32 * nb32, gb.batch);
    if (vec) k_gemm_batched<true, 32><<<g32, GEMM_THREADS, 0, s>>>(gb, status);
    else k_gemm_batched<false, 32><<<g32, GEMM_THREADS, 0, s>>>(gb, status);
  } else if (vec) {
    k_gemm_batched<true><<<grid, GEMM_THREADS, 0, s>>>(gb, status);
  } else {
    k_gemm_batched<false><<<grid, GEMM_THREADS, 0, s>>>(gb, status);
  }
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

int launch_gemm_nt(const double* A, i64 lda, const double* B, i64 ldb, double* C, i64 ldc, int m, int n,
                   int k, int lower, double alpha, const int* status, cudaStream_t s) {
  GemmBatch gb{A, lda, 0, B, ldb, 0, C, ldc, 0, m, m, n, k, lower, 1, alpha, 0};
  return launch_gemm_batched(gb, status, s);
}

int launch_gemm_nt_trib(const double* A, i64 lda, const double* B, i64 ldb, double* C, i64 ldc, int m, int n, int k,
                        double alpha, const int* status, cudaStream_t s) {
  GemmBatch gb{A, lda, 0, B, ldb, 0, C, ldc, 0, m, m, n, k, 0, 1, alpha, 1};
  return launch_gemm_batched(gb, status, s);
}

static int launch_trsm_small(const double* L, i64 ldl, double* B, i64 ldb, i64 sB, int m, int m_last,
                             int batch, int n, const int* status, cudaStream_t s) {
  if (batch <= 0 || n <= 0) return OOC_OK;
  if (n > SB) return OOC_ERR_INTERNAL;
  dim3 grid((max(m, m_last) + TS_ROWS - 1) / TS_ROWS, batch);
  k_trsm_small<<<grid, TS_THREADS, 0, s>>>(L, ldl, B, ldb, sB, m, m_last, batch, n, status);
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

int launch_potrf_tile(double* A, i64 ld, int n, i64 col0, int* status, cudaStream_t s) {
  for (int k = 0; k < n; k += SB) {
    const int kb = min(SB, n - k);
    double* Akk = A + k + (i64)k * ld;
    k_potrf_small<<<1, 256, 0, s>>>(Akk, ld, kb, col0 + k, status);
    OOC_CUDA_TRY(cudaGetLastError());
    const int rest = n - k - kb;
    if (rest > 0) {
      double* Bp = A + (k + kb) + (i64)k * ld;  // rows below the block, columns k..k+kb
      int rc = launch_trsm_small(Akk, ld, Bp, ld, 0, rest, rest, 1, kb, status, s);
      if (rc) return rc;
      double* Ct = A + (k + kb) + (i64)(k + kb) * ld;
      rc = launch_gemm_nt(Bp, ld, Bp, ld, Ct, ld, rest, rest, kb, 1, -1.0, status, s);
      if (rc) return rc;
    }
  }
  return OOC_OK;
}

int launch_trsm_col(const double* L, i64 ldl, const TileCol& B, int ntiles, int nb, int m_last, int n,
                    const int* status, cudaStream_t s) {
  if (ntiles <= 0) return OOC_OK;
  double* Bb = const_cast<double*>(B.base);
  for (int k = 0; k < n; k += SB) {
    const int kb = min(SB, n - k);
    const double* Lkk = L + k + (i64)k * ldl;
    int rc = launch_trsm_small(Lkk, ldl, Bb + (i64)k * B.ld, B.ld, B.stride, nb, m_last, ntiles, kb,
                               status, s);
    if (rc) return rc;
    const int rest = n - k - kb;
    if (rest > 0) {
      // B[:, k+kb:n] -= B[:, k:k+kb] L[k+kb:n, k:k+kb]^T for every tile of the column.
      GemmBatch gb{Bb + (i64)k * B.ld, B.ld, B.stride,
                   L + (k + kb) + (i64)k * ldl, ldl, 0,
                   Bb + (i64)(k + kb) * B.ld, B.ld, B.stride,
                   nb, m_last, rest, kb, 0, ntiles, -1.0, 0};
      rc = launch_gemm_batched(gb, status, s);
      if (rc) return rc;
    }
  }
  return OOC_OK;
}
