// Batched factor + solve of many small SPD systems in ONE persistent launch.
//
// Thousands of uneven matrices (n in [16, 512]) are too small for the tile pipeline:
// each would be a handful of tiny launches.  Here every CTA of a persistent grid (one
// launch per size class) takes the next matrix from a queue sorted by decreasing size
// (largest first balances the tail), factors it with a blocked right-looking Cholesky
// inside the CTA, solves for its right-hand side, and moves on.  FP32 (factor_f32): the
// diagonal block factored by one warp in registers, the panel solved a row per thread in
// registers and kept transposed in shared memory, the trailing update by 32 x 32 blocks
// with a 4 x 8 register tile per lane, the forward substitution inside the factorization
// and the backward sweep on the vector in shared memory.  FP64 (factor_one): the diagonal
// block column by column by the CTA, the panel solve a row per thread, the trailing update
// from a row copy of the panel with 4 x 4 register tiles, then both sweeps (solve_one).
// Per-matrix LAPACK info goes to an array; a failed matrix is skipped.  The panel width is
// chosen per size bucket by the autotuner (oocdag_gb300/autotune.py).
//
// The per-tile arithmetic restates the reference's task bodies at small n: the
// diagonal dpotrf (oocquark.cpp:87), the column dtrsm R/L/T/N (:130) and the
// dsyrk/dgemm trailing update (:176,222), followed by the dpotrs of its VERIFY block
// (oocdag.cpp:439).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace {

constexpr int BT = 256;        // threads per CTA
constexpr int NMAX = 512;      // largest matrix order supported
constexpr int NBUCKETS = 16;   // size buckets of 32: n in [32 q, 32 q + 31]

struct Item {
  void* a;    // the matrix (column-major, ld = n): A on entry, L on exit
  void* b;    // its right-hand side (overwritten by the solution)
  int n;
  int blk;    // panel width for this matrix
  int mode;   // 0: factor + solve, 1: solve with an L already in `a`
};

template <typename T>
__device__ __forceinline__ T tsqrt(T x) { return sqrt(x); }
template <>
__device__ __forceinline__ float tsqrt<float>(float x) { return sqrtf(x); }

// Cholesky of the kb x kb (kb <= 32) block at rows/columns off.. of D (lower, column-major,
// ld 65) in one warp: lane r holds row r in registers, and the current column is published
// through the padding slots D[c * 65 + 64] (row 64 of D is never data), so the warp needs no
// block-wide barrier.  A non-positive pivot is replaced by 1 so the steps stay finite;
// returns the first one (kb if none), and writes the block back only if it factored.
template <typename T>
__device__ int chol32_warp(T* D, int off, int kb, int lane) {
  T a[32];
#pragma unroll
  for (int c = 0; c < 32; c++)
    a[c] = (lane < kb && c <= lane) ? D[(off + c) * 65 + off + lane] : ((c == lane) ? T(1) : T(0));
  int bad = kb;
#pragma unroll
  for (int j = 0; j < 32; j++) {
    D[lane * 65 + 64] = a[j];  // column j as it stands
    __syncwarp();
    T d = D[j * 65 + 64];
    if (!(d > T(0))) {
      if (j < kb) bad = min(bad, j);
      d = T(1);
    }
    const T sq = tsqrt(d), inv = T(1) / sq;
    const T lj = (lane == j) ? sq : a[j] * inv;  // L(lane, j)
    if (lane >= j) a[j] = lj;
#pragma unroll
    for (int c = j + 1; c < 32; c++)  // A(lane, c) -= L(lane, j) L(c, j)
      if (lane >= c) a[c] -= lj * (D[c * 65 + 64] * inv);
    __syncwarp();
  }
  if (bad == kb) {
#pragma unroll
    for (int c = 0; c < 32; c++)
      if (lane < kb && c <= lane) D[(off + c) * 65 + off + lane] = a[c];
  }
  return bad;
}

// FP64 factorization of one matrix by the CTA.  Shared layout: D[64][65] (diagonal block),
// P[NMAX][blk+1] (panel copy).  BLK is the panel width (a compile-time constant, so that
// the panel solve keeps its row in registers).
template <typename T, int BLK>
__device__ int factor_one(T* __restrict__ A, int n, T* D, T* P, int* s_fail) {
  constexpr int blk = BLK;
  const int t = threadIdx.x;
  const int ldp = blk + 1;
  for (int k = 0; k < n; k += blk) {
    const int kb = min(blk, n - k);
    // 1. diagonal block -> shared, unblocked right-looking Cholesky
    for (int idx = t; idx < kb * kb; idx += BT) {
      const int c = idx / kb, r = idx % kb;
      if (r >= c) D[c * 65 + r] = A[(k + r) + (i64)(k + c) * n];
    }
    if (t == 0) *s_fail = 0;
    __syncthreads();
    // column by column over the CTA (a warp form would spill its doubles)
    for (int j = 0; j < kb; j++) {
      if (t == 0) {
        const T d = D[j * 65 + j];
        if (!(d > T(0))) *s_fail = k + j + 1;
        else D[j * 65 + j] = tsqrt(d);
      }
      __syncthreads();
      if (*s_fail) break;
      const T inv = T(1) / D[j * 65 + j];
      for (int r = j + 1 + t; r < kb; r += BT) D[j * 65 + r] *= inv;
      __syncthreads();
      const int w = kb - j - 1;
      for (int idx = t; idx < w * w; idx += BT) {
        const int c = j + 1 + idx / w, r = j + 1 + idx % w;
        if (r >= c) D[c * 65 + r] -= D[j * 65 + r] * D[j * 65 + c];
      }
      __syncthreads();
    }
    for (int idx = t; idx < kb * kb; idx += BT) {
      const int c = idx / kb, r = idx % kb;
      if (r >= c) A[(k + r) + (i64)(k + c) * n] = D[c * 65 + r];
    }
    const int fail = *s_fail;
    __syncthreads();
    if (fail) return fail;
    const int m = n - k - kb;
    if (m <= 0) break;
    // 2. panel: rows below, B := B L_kk^-T, one thread per row held in registers (the
    // dependent chain then waits on FMAs, not on shared-memory loads); result kept in P.
    // Columns c >= kb are computed from stale D entries and discarded.
    for (int i = t; i < m; i += BT) {
      const int gi = k + kb + i;
      T r[BLK];
#pragma unroll
      for (int c = 0; c < BLK; c++) r[c] = (c < kb) ? A[gi + (i64)(k + c) * n] : T(0);
#pragma unroll
      for (int c = 0; c < BLK; c++) {
        T v = r[c];
#pragma unroll
        for (int q = 0; q < c; q++) v -= r[q] * D[q * 65 + c];
        r[c] = (c < kb) ? v / D[c * 65 + c] : T(0);
      }
      T* row = P + i * ldp;
#pragma unroll
      for (int c = 0; c < BLK; c++)
        if (c < kb) {
          row[c] = r[c];
          A[gi + (i64)(k + c) * n] = r[c];
        }
    }
    __syncthreads();
    // 3. trailing update of the lower triangle from P (4 x 4 tiles per thread)
    const int Tt = (m + 3) / 4;
    const int ntile = Tt * (Tt + 1) / 2;
    for (int tile = t; tile < ntile; tile += BT) {
      int ti = (int)((sqrtf(8.f * (float)tile + 1.f) - 1.f) * 0.5f);
      while ((ti + 1) * (ti + 2) / 2 <= tile) ti++;
      while (ti * (ti + 1) / 2 > tile) ti--;
      const int tj = tile - ti * (ti + 1) / 2;
      T acc[4][4];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = T(0);
      const int r0 = ti * 4, c0 = tj * 4;
      for (int q = 0; q < kb; q++) {
        T ra[4], cb[4];
#pragma unroll
        for (int a = 0; a < 4; a++) ra[a] = (r0 + a < m) ? P[(r0 + a) * ldp + q] : T(0);
#pragma unroll
        for (int b = 0; b < 4; b++) cb[b] = (c0 + b < m) ? P[(c0 + b) * ldp + q] : T(0);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int b = 0; b < 4; b++) acc[a][b] = fma(ra[a], cb[b], acc[a][b]);
      }
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
          const int r = r0 + a, c = c0 + b;
          if (r < m && c < m && c <= r) {
            T* p = A + (k + kb + r) + (i64)(k + kb + c) * n;
            *p -= acc[a][b];
          }
        }
    }
    __syncthreads();
  }
  return 0;
}

// FP32 factorization of one matrix by the CTA, in steps of BLK (16 or 32) columns:
//   1. the diagonal block is factored by one warp in registers (chol32_warp), and the
//      reciprocals of its diagonal are kept; from the second step on this happens inside
//      the previous step's trailing update (warp 0 updates the block that holds it and
//      factors it while the other warps update the rest);
//   2. every row below solves against L_kk^T, one thread per row with the row in registers,
//      right-looking (each column's FMAs independent of the others'); the result goes to
//      the matrix and, transposed, to PT (PT[c ldt + i] = L(k + kb + i, k + c)), zero-padded
//      to a multiple of 32 rows;
//   3. the trailing lower triangle is updated by 32 x 32 blocks, a warp a block, each lane a
//      4 x 8 register tile fed by 16-byte shared loads of PT (ten FMAs per shared load); the
//      block's elements of the matrix are loaded before the products and stored after.
// The trailing matrix stays in global memory (up to 1 MB per matrix); every element of it is
// read and written once per step.
__device__ __forceinline__ void bt_block_ij(int b, int& I, int& J) {
  int i = (int)((sqrtf(8.f * (float)b + 1.f) - 1.f) * 0.5f);
  if ((i + 1) * (i + 2) / 2 <= b) i++;
  if (i * (i + 1) / 2 > b) i--;
  I = i;
  J = b - i * (i + 1) / 2;
}

template <int BLK>
__device__ int factor_f32(float* __restrict__ A, int n, float* D, float* PT, int ldt, float* bs, int* s_fail) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  float* rinv = D + 40 * 65;  // a column of D that a <= 32-wide block never uses
  const int r0 = (lane & 7) * 4, c0 = (lane >> 3) * 8;
  const int zero = n >> 30;  // n <= 512
  // warp 0: factor the kb x kb diagonal block at column k (already in D), keep the
  // reciprocals of its diagonal and write L_kk to the matrix
  auto diag = [&](int k, int kb) {
    const int b = chol32_warp(D, 0, kb, lane);
    if (lane == 0) *s_fail = (b < kb) ? k + b + 1 : 0;
    const float ri = (lane < kb) ? 1.f / D[lane * 65 + lane] : 0.f;
    if (lane < BLK) rinv[lane] = ri;
    if (b == kb) {
      for (int idx = lane; idx < kb * kb; idx += 32) {
        const int c = idx / kb, r = idx % kb;
        if (r >= c) A[(k + r) + (i64)(k + c) * n] = D[c * 65 + r];
      }
      if (bs) {  // forward sweep, this block: y_k = L_kk^{-1} b_k (b_k is final: every
                 // earlier step's row solve has already subtracted its panel's share)
        float v = (lane < kb) ? bs[k + lane] : 0.f;
        for (int j = 0; j < kb; j++) {
          const float yj = __shfl_sync(0xffffffffu, v * ri, j);
          if (lane == j) v = yj;
          else if (lane > j) v = fmaf(-D[j * 65 + lane], yj, v);
        }
        if (lane < kb) bs[k + lane] = v;
      }
    }
  };
  {
    const int kb = min(BLK, n);
    for (int idx = t; idx < kb * kb; idx += BT) {
      const int c = idx / kb, r = idx % kb;
      if (r >= c) D[c * 65 + r] = A[r + (i64)c * n];
    }
    __syncthreads();
    if (warp == 0) diag(0, kb);
    __syncthreads();
  }
  for (int k = 0; k < n; k += BLK) {
    const int kb = min(BLK, n - k);
    const int fail = *s_fail;
    if (fail) return fail;
    const int m = n - k - kb;
    if (m <= 0) break;
    const int m32 = (m + 31) & ~31;
    for (int i = t; i < m32; i += BT) {
      float r[BLK];
      float* g = A + (k + kb + i);
      const bool live = i < m;
#pragma unroll
      for (int c = 0; c < BLK; c++) r[c] = (live && c < kb) ? g[(i64)(k + c) * n] : 0.f;
      float fw = 0.f;  // forward sweep: b_i -= L(i, k..) y_k (y_k sits in bs[k..])
      const float* yk = bs ? bs + k : rinv;
#pragma unroll
      for (int c = 0; c < BLK; c++) {
        r[c] *= rinv[c];
        // zero at run time: column c's loads of L_kk wait for r[c] (not all hoisted into registers)
        const int z = zero & __float_as_int(r[c]);
        const float* lc = D + c * 65 + z;
#pragma unroll
        for (int q = c + 1; q < BLK; q++) r[q] = fmaf(-r[c], lc[q], r[q]);
        const float v = (live && c < kb) ? r[c] : 0.f;
        PT[c * ldt + i] = v;
        if (live && c < kb) g[(i64)(k + c) * n] = v;
        if (c < kb) fw = fmaf(v, yk[c + z], fw);  // never reads past the vector
      }
      if (bs && live) bs[k + kb + i] -= fw;
    }
    __syncthreads();
    // Trailing update.  Warp 0 takes block (0, 0), which holds the next diagonal block: it
    // also leaves that block's kn x kn corner in D and factors it at once, while warps
    // 1.. update the other blocks; the next step's row solve follows the barrier directly.
    const int nb32 = m32 >> 5, nblk = nb32 * (nb32 + 1) / 2;
    const int kn = min(BLK, m);
    float* C = A + (k + kb) + (i64)(k + kb) * n;
    for (int b = (warp == 0) ? 0 : warp; b < nblk; b += (warp == 0) ? nblk : BT / 32 - 1) {
      int I, J;
      bt_block_ij(b, I, J);
      const int rb = I * 32 + r0, cb = J * 32 + c0;
      float cv[4][8];
#pragma unroll
      for (int ii = 0; ii < 4; ii++)
#pragma unroll
        for (int jj = 0; jj < 8; jj++) {
          const int row = rb + ii, col = cb + jj;
          cv[ii][jj] = (row < m && col <= row) ? C[row + (i64)col * n] : 0.f;
        }
      float acc[4][8] = {};
#pragma unroll 8
      for (int q = 0; q < BLK; q++) {
        const float4 a = *reinterpret_cast<const float4*>(PT + q * ldt + rb);
        const float4 b0 = *reinterpret_cast<const float4*>(PT + q * ldt + cb);
        const float4 b1 = *reinterpret_cast<const float4*>(PT + q * ldt + cb + 4);
        const float av[4] = {a.x, a.y, a.z, a.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int ii = 0; ii < 4; ii++)
#pragma unroll
          for (int jj = 0; jj < 8; jj++) acc[ii][jj] = fmaf(av[ii], bv[jj], acc[ii][jj]);
      }
#pragma unroll
      for (int ii = 0; ii < 4; ii++)
#pragma unroll
        for (int jj = 0; jj < 8; jj++) {
          const int row = rb + ii, col = cb + jj;
          if (row < m && col <= row) {
            const float v = cv[ii][jj] - acc[ii][jj];
            C[row + (i64)col * n] = v;
            if (b == 0 && row < kn) D[col * 65 + row] = v;
          }
        }
    }
    if (warp == 0) {
      __syncwarp();
      diag(k + kb, kn);
    }
    __syncthreads();
  }
  return 0;
}

// Backward sweep L^T x = y for the vector in shared memory (FP32 path; the forward sweep
// ran inside the factorization), blocks of 32 rows from the last.  Once x_K is known,
// warp 0 takes its share off the rows of block K-1 and solves that block at once (a
// 32 x 32 triangular system with shuffles), while the other warps take x_K's share off the
// rows above; one barrier per block.  Every row receives the same subtractions in the same
// order whichever warp performs them.
__device__ __forceinline__ void back_share(const float* __restrict__ L, int n, float* bs, int k, int kb, int i) {
  const float* li = L + k + (i64)i * n;  // L(k.., i): contiguous rows of column i
  float s0 = 0.f, s1 = 0.f;
#pragma unroll 8
  for (int j = 0; j + 1 < kb; j += 2) {
    s0 = fmaf(li[j], bs[k + j], s0);
    s1 = fmaf(li[j + 1], bs[k + j + 1], s1);
  }
  if (kb & 1) s0 = fmaf(li[kb - 1], bs[k + kb - 1], s0);
  bs[i] -= s0 + s1;
}

__device__ __forceinline__ void back_block(const float* __restrict__ L, int n, float* bs, int k, int lane) {
  const int kb = min(32, n - k);
  float v = (lane < kb) ? bs[k + lane] : 0.f;
  const float ljj = (lane < kb) ? L[(k + lane) + (i64)(k + lane) * n] : 1.f;
  for (int j = kb - 1; j >= 0; j--) {
    const float xj = __shfl_sync(0xffffffffu, v / ljj, j);
    if (lane == j) v = xj;
    else if (lane < j) v = fmaf(-L[(k + j) + (i64)(k + lane) * n], xj, v);  // (L^T)(lane, j) = L(j, lane)
  }
  if (lane < kb) bs[k + lane] = v;
}

__device__ void solve_back_f32(const float* __restrict__ L, int n, float* bs) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  int k = ((n - 1) / 32) * 32;
  if (warp == 0) back_block(L, n, bs, k, lane);
  __syncthreads();
  for (; k > 0; k -= 32) {  // x for rows k.. is final
    const int kb = min(32, n - k);
    if (warp == 0) {
      back_share(L, n, bs, k, kb, k - 32 + lane);
      __syncwarp();
      back_block(L, n, bs, k - 32, lane);
    } else {
      for (int i = t - 32; i < k - 32; i += BT - 32) back_share(L, n, bs, k, kb, i);
    }
    __syncthreads();
  }
}

// L L^T x = b in place (b in global), blocks of 32 rows: one warp solves the diagonal
// block with shuffles, all threads update the rest.
template <typename T>
__device__ void solve_one(const T* __restrict__ L, int n, T* __restrict__ b) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  // forward
  for (int k = 0; k < n; k += 32) {
    const int kb = min(32, n - k);
    if (warp == 0) {
      T v = (lane < kb) ? b[k + lane] : T(0);
      for (int j = 0; j < kb; j++) {
        T yj = __shfl_sync(0xffffffffu, v, j);
        if (lane == j) { yj = v / L[(k + j) + (i64)(k + j) * n]; v = yj; }
        yj = __shfl_sync(0xffffffffu, v, j);
        if (lane > j && lane < kb) v -= L[(k + lane) + (i64)(k + j) * n] * yj;
      }
      if (lane < kb) b[k + lane] = v;
    }
    __syncthreads();
    for (int i = k + kb + t; i < n; i += BT) {
      T s = T(0);
      for (int j = 0; j < kb; j++) s = fma(L[i + (i64)(k + j) * n], b[k + j], s);
      b[i] -= s;
    }
    __syncthreads();
  }
  // backward: L^T x = y
  for (int k = ((n - 1) / 32) * 32; k >= 0; k -= 32) {
    const int kb = min(32, n - k);
    if (warp == 0) {
      T v = (lane < kb) ? b[k + lane] : T(0);
      for (int j = kb - 1; j >= 0; j--) {
        T xj = __shfl_sync(0xffffffffu, v, j);
        if (lane == j) { xj = v / L[(k + j) + (i64)(k + j) * n]; v = xj; }
        xj = __shfl_sync(0xffffffffu, v, j);
        if (lane < j) v -= L[(k + j) + (i64)(k + lane) * n] * xj;  // (L^T)(lane, j) = L(j, lane)
      }
      if (lane < kb) b[k + lane] = v;
    }
    __syncthreads();
    for (int i = t; i < k; i += BT) {
      T s = T(0);
      for (int j = 0; j < kb; j++) s = fma(L[(k + j) + (i64)i * n], b[k + j], s);
      b[i] -= s;
    }
    __syncthreads();
  }
}

// MINB resident CTAs per SM requested from the register allocator: 2 for FP32 (whose
// shared memory, sized per size class, lets two CTAs share an SM up to n = 256), 1 for FP64.
template <typename T, int MINB>
__global__ void __launch_bounds__(BT, MINB) k_batched_posv(const Item* __restrict__ items, int count, int* info,
                                                           int* counter, int do_solve, int ldt) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  T* D = (T*)smem_raw;
  T* P = D + 64 * 65;
  __shared__ int s_idx, s_fail;
  for (;;) {
    if (threadIdx.x == 0) s_idx = atomicAdd(counter, 1);
    __syncthreads();
    const int idx = s_idx;
    __syncthreads();
    if (idx >= count) break;
    const Item it = items[idx];
    T* a = (T*)it.a;
    int f = 0;
    bool solved = false;
    if (it.mode == 0) {
      if constexpr (sizeof(T) == 4) {  // 16- or 32-wide steps (the autotuner's choice)
        // the right-hand side in shared memory: the forward sweep runs inside the
        // factorization, the backward sweep after it
        float* bs = do_solve ? P + 32 * ldt : nullptr;
        if (bs) {
          for (int i = threadIdx.x; i < it.n; i += BT) bs[i] = ((const float*)it.b)[i];
          __syncthreads();
        }
        if (it.blk <= 16) f = factor_f32<16>(a, it.n, D, P, ldt, bs, &s_fail);
        else f = factor_f32<32>(a, it.n, D, P, ldt, bs, &s_fail);
        if (bs && f == 0) {
          solve_back_f32(a, it.n, bs);
          for (int i = threadIdx.x; i < it.n; i += BT) ((float*)it.b)[i] = bs[i];
        }
        solved = true;
      } else {
        switch (it.blk) {  // the widths the autotuner chooses from (others fall back to 32)
          case 8: f = factor_one<T, 8>(a, it.n, D, P, &s_fail); break;
          case 16: f = factor_one<T, 16>(a, it.n, D, P, &s_fail); break;
          default: f = factor_one<T, 32>(a, it.n, D, P, &s_fail); break;
        }
      }
    }
    if (threadIdx.x == 0) info[idx] = f;
    if (f == 0 && do_solve && !solved) solve_one<T>(a, it.n, (T*)it.b);
    __syncthreads();
  }
}

// Scatter per-matrix info from sorted order back to the caller's order.
__global__ void k_scatter_info(const int* sorted_info, const int* order, int count, int* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[order[i]] = sorted_info[i];
}

// Shared memory of a launch whose matrices have orders <= nmax and panel widths <= blk.
// FP32 keeps the panel transposed (up to 32 rows of ldt floats, ldt = the class's largest
// order rounded up to 32, plus 4) and the right-hand side (ldt floats); FP64 keeps the
// panel row by row (nmax rows of blk + 1).
inline int ldt_for(int nmax) { return (nmax + 31) / 32 * 32 + 4; }
template <typename T>
size_t smem_for(int blk, int nmax = NMAX) {
  if (sizeof(T) == 4) return (size_t)(64 * 65 + 33 * ldt_for(nmax)) * sizeof(T);  // D, PT (<= 32 rows), b
  return (size_t)(64 * 65 + nmax * (blk + 1)) * sizeof(T);
}
template <typename T>
constexpr int minb() { return sizeof(T) == 4 ? 2 : 1; }

template <typename T>
int run_items(cudaStream_t s, int dev, std::vector<Item>& items_in, int* info_host, const int* blk_table,
              int ctas_per_sm, int do_solve, double* seconds, int (*wait)(void*, cudaStream_t), void* wait_arg,
              GrowBuf* ws);

template <typename T>
int run_batched(ooc_handle* h, int count, const int* n, const int64_t* a_off, const int64_t* b_off, T* A, T* B,
                int* info_host, const int* blk_table, int ctas_per_sm, int do_solve, double* seconds) {
  std::vector<Item> items(count);
  for (int i = 0; i < count; i++) items[i] = Item{(void*)(A + a_off[i]), (void*)(B + b_off[i]), n[i], 0, 0};
  return run_items<T>(ooc_compute_stream(h), ooc_device(h), items, info_host, blk_table, ctas_per_sm, do_solve, seconds,
                      [](void* hh, cudaStream_t st) { return ooc_wait_stream((ooc_handle*)hh, st); }, (void*)h,
                      ooc_handle_batch_ws(h));
}

// Sorts the items by decreasing order, picks each one's panel width from the table, and
// runs them in persistent launches on `s`, one per size class; info_host receives LAPACK
// info per item in the caller's order.
template <typename T>
int run_items(cudaStream_t s, int dev, std::vector<Item>& items_in, int* info_host, const int* blk_table,
              int ctas_per_sm, int do_solve, double* seconds, int (*wait)(void*, cudaStream_t), void* wait_arg,
              GrowBuf* ws) {
  const int count = (int)items_in.size();
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return items_in[x].n > items_in[y].n; });
  std::vector<Item> items(count);
  for (int i = 0; i < count; i++) {
    const int j = order[i];
    const int bucket = std::min(NBUCKETS - 1, items_in[j].n / 32);
    int blk = blk_table ? blk_table[bucket] : (sizeof(T) == 8 ? 32 : 64);
    blk = std::max(1, std::min(blk, 32));
    blk = sizeof(T) == 4 ? (blk <= 16 ? 16 : 32) : (blk <= 8 ? 8 : blk <= 16 ? 16 : 32);  // the compiled widths
    items[i] = items_in[j];
    items[i].blk = blk;
  }
  // Size classes (orders in (0,64], (64,128], (128,256], (256,384], (384,512]; the items
  // are sorted by decreasing order, so a class is a contiguous range): one persistent
  // launch each, its shared memory sized for the class's largest order and panel width,
  // so that the small classes fit several CTAs per SM.
  const int bounds[] = {512, 384, 256, 128, 64};
  std::vector<std::pair<int, int>> classes;  // [first, one past the last) in sorted order
  {
    int i = 0;
    for (int ci = 0; ci < 5 && i < count; ci++) {
      const int lo = ci + 1 < 5 ? bounds[ci + 1] : 0;
      int j = i;
      while (j < count && items[j].n > lo) j++;
      if (j > i) classes.emplace_back(i, j);
      i = j;
    }
  }
  const int ncls = (int)classes.size();
  // the launch tables, in the caller's workspace (kept across calls): items, then four
  // int arrays (info, order, scattered info, one counter per class), each 256-byte aligned
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t b_items = up(sizeof(Item) * (size_t)count), b_int = up(sizeof(int) * (size_t)count);
  int rc = ws->ensure(b_items + 3 * b_int + 256);
  Item* d_items = nullptr;
  int *d_info = nullptr, *d_order = nullptr, *d_out = nullptr, *d_counter = nullptr;
  if (!rc) {
    char* base = (char*)ws->p;
    d_items = (Item*)base;
    d_info = (int*)(base + b_items);
    d_order = (int*)(base + b_items + b_int);
    d_out = (int*)(base + b_items + 2 * b_int);
    d_counter = (int*)(base + b_items + 3 * b_int);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (!rc) {
    cudaMemcpyAsync(d_items, items.data(), sizeof(Item) * count, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_order, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(d_counter, 0, sizeof(int) * 8, s);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    for (int ci = 0; ci < ncls && !rc; ci++) {
      const int i0 = classes[ci].first, i1 = classes[ci].second;
      int cmax = 1, cblk = 1;
      for (int i = i0; i < i1; i++) {
        cmax = std::max(cmax, items[i].n);
        cblk = std::max(cblk, items[i].blk);
      }
      const size_t sm = smem_for<T>(cblk, cmax);
      if (cudaFuncSetAttribute(k_batched_posv<T, minb<T>()>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
          cudaSuccess) {
        cudaGetLastError();
        rc = OOC_ERR_UNSUPPORTED;
        break;
      }
      int occ = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched_posv<T, minb<T>()>, BT, sm);
      const int per = std::max(1, std::min(ctas_per_sm > 0 ? ctas_per_sm : occ, std::max(occ, 1)));
      const int grid = std::max(1, std::min(i1 - i0, nsm * per));
      k_batched_posv<T, minb<T>()><<<grid, BT, sm, s>>>(d_items + i0, i1 - i0, d_info + i0, d_counter + ci, do_solve,
                                                         ldt_for(cmax));
    }
    cudaEventRecord(e1, s);
    if (!rc) k_scatter_info<<<(count + 255) / 256, 256, 0, s>>>(d_info, d_order, count, d_out);
    cudaError_t e = cudaGetLastError();
    if (!rc && e != cudaSuccess) { ooc_set_last_error(e, "k_batched_posv", __FILE__, __LINE__); rc = OOC_ERR_CUDA; }
  }
  if (!rc) {
    cudaMemcpyAsync(info_host, d_out, sizeof(int) * count, cudaMemcpyDeviceToHost, s);
    rc = wait(wait_arg, s);
  }
  if (!rc && seconds) {
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    *seconds = ms * 1e-3;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return rc;
}

template <typename T>
int check_args(int count, const int* n, const int64_t* a_off, const int64_t* b_off, const T* A, const T* B,
               int* info) {
  if (count < 0) return -3;
  if (count > 0 && (!n || !a_off || !b_off)) return -4;
  if (count > 0 && (!A || !B)) return -7;
  if (!info && count > 0) return -9;
  for (int i = 0; i < count; i++)
    if (n[i] < 1 || n[i] > NMAX) return -4;
  return OOC_OK;
}

}  // namespace

// Server hook: FP64 items given by absolute device pointers (mode 0 factor+solve, 1 solve).
// `ws`: the caller's workspace for the launch tables (kept across calls).
int ooc_batched_run_ptrs(cudaStream_t s, int dev, int count, double* const* a, double* const* b, const int* n,
                         const int* mode, int* info_host, const int* blk_table, GrowBuf* ws) {
  std::vector<Item> items(count);
  for (int i = 0; i < count; i++) items[i] = Item{(void*)a[i], (void*)b[i], n[i], 0, mode[i]};
  return run_items<double>(s, dev, items, info_host, blk_table, 0, 1, nullptr,
                           [](void*, cudaStream_t st) -> int {
                             cudaError_t e = cudaStreamSynchronize(st);
                             return e == cudaSuccess ? OOC_OK : OOC_ERR_CUDA;
                           },
                           nullptr, ws);
}

extern "C" int ooc_batched_dposv(ooc_handle* h, int count, const int* n, const int64_t* a_off, const int64_t* b_off,
                                 double* A, double* B, int* info, const int* blk_table, int ctas_per_sm,
                                 double* seconds) {
  if (!h) return -1;
  int rc = check_args<double>(count, n, a_off, b_off, A, B, info);
  if (rc) return rc;
  if (count == 0) return OOC_OK;
  cudaSetDevice(ooc_device(h));
  return run_batched<double>(h, count, n, a_off, b_off, A, B, info, blk_table, ctas_per_sm, 1, seconds);
}

extern "C" int ooc_batched_sposv(ooc_handle* h, int count, const int* n, const int64_t* a_off, const int64_t* b_off,
                                 float* A, float* B, int* info, const int* blk_table, int ctas_per_sm,
                                 double* seconds) {
  if (!h) return -1;
  int rc = check_args<float>(count, n, a_off, b_off, A, B, info);
  if (rc) return rc;
  if (count == 0) return OOC_OK;
  cudaSetDevice(ooc_device(h));
  return run_batched<float>(h, count, n, a_off, b_off, A, B, info, blk_table, ctas_per_sm, 1, seconds);
}
