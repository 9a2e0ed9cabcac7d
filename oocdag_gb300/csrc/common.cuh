// Shared definitions for the GB300 out-of-core Cholesky library.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <stdint.h>
#include <stdio.h>

#include "../../include/oocdag_gb300.h"

typedef int64_t i64;

// Packed panel layout: the lower trapezoid of a panel of Ym tile rows, column of tiles
// after column of tiles, each tile nb x nb with leading dimension nb.  Tile (i, j),
// i >= j, starts at tile index i + j*Ym - j*(j+1)/2 (the layout of oocquark.cpp:256).
__host__ __device__ inline i64 packed_tile_index(int i, int j, int Ym) {
  return (i64)i + (i64)j * Ym - ((i64)j * (j + 1)) / 2;
}

// Addressing of a grid of nb x nb tiles.  Either packed (as above, ld = nb) or strided
// (a column-major matrix with leading dimension ld; tile (i, j) starts at row i*nb,
// column j*nb).
struct TileMap {
  double* base;
  i64 ld;      // leading dimension of every tile
  int packed;  // 1: packed trapezoid, 0: strided
  int Ym;      // packed: tile rows of the panel
  int nb;
};

__host__ __device__ inline double* tile_ptr(const TileMap& m, int i, int j) {
  if (m.packed) return m.base + packed_tile_index(i, j, m.Ym) * (i64)m.nb * m.nb;
  return m.base + (i64)i * m.nb + (i64)j * m.nb * m.ld;
}

// A single column of tiles: tile i starts at base + i*stride (stride in elements).
struct TileCol {
  const double* base;
  i64 ld;
  i64 stride;
};

#define OOC_CUDA_TRY(expr)                                              \
  do {                                                                  \
    cudaError_t _e = (expr);                                            \
    if (_e != cudaSuccess) {                                            \
      ooc_set_last_error(_e, #expr, __FILE__, __LINE__);                \
      return OOC_ERR_CUDA;                                              \
    }                                                                   \
  } while (0)

void ooc_set_last_error(cudaError_t e, const char* what, const char* file, int line);
void ooc_set_last_message(const char* msg);

// ---------------------------------------------------------------------------------
// FP64 kernel launchers (fp64_kernels.cu).  All run on `s`, read the status word
// `status` first and return without touching memory once it is non-zero.
// ---------------------------------------------------------------------------------

// C(i, j) -= X(i) X(j)^T for every tile pair of a trapezoid of Ht tile rows and Kt
// tile columns (i >= j); X is a column of Ht tiles, each with K columns.  H and Kcols
// are the element extents (the last tile row / column may be ragged).  Diagonal pairs
// update only their lower triangle.
int launch_panel_update(const TileCol& X, const TileMap& C, int Ht, int Kt, i64 H, i64 Kcols,
                        int K, const int* status, cudaStream_t s);

// Generic C[m x n] -= A[m x k] * B[n x k]^T (column-major, any leading dimensions);
// lower = 1 restricts the update to the lower triangle (m == n, syrk).
int launch_gemm_nt(const double* A, i64 lda, const double* B, i64 ldb, double* C, i64 ldc, int m,
                   int n, int k, int lower, double alpha, const int* status, cudaStream_t s);

// C[m x n] += alpha * A[m x k] * B[n x k]^T with B lower triangular (B(j, kk) = 0 for
// kk > j): the zero part of K is skipped, so a triangular product costs its own flops.
int launch_gemm_nt_trib(const double* A, i64 lda, const double* B, i64 ldb, double* C, i64 ldc, int m, int n, int k,
                        double alpha, const int* status, cudaStream_t s);

// Lower Cholesky of an n x n tile in place (leading dimension ld).  On failure writes
// status = col0 + (1-based local column) unless status is already non-zero.
int launch_potrf_tile(double* A, i64 ld, int n, i64 col0, int* status, cudaStream_t s);

// B(t) := B(t) L^-T for every tile t of a column of `ntiles` tiles with `m_last` rows in
// the last one (all others nb rows) and n columns; L is the n x n lower tile.
int launch_trsm_col(const double* L, i64 ldl, const TileCol& B, int ntiles, int nb, int m_last,
                    int n, const int* status, cudaStream_t s);

// ---------------------------------------------------------------------------------
// Handle accessors shared between translation units (ooc_driver.cu).
// ---------------------------------------------------------------------------------
cudaStream_t ooc_compute_stream(ooc_handle* h);
int ooc_device(ooc_handle* h);
int ooc_wait_stream(ooc_handle* h, cudaStream_t s);  // bounded by the handle's timeout
ooc_handle* ooc_default_handle();
// The handle's device-buffer cache (devpool.cuh), shared with the factor objects it creates.
struct DevPool;
std::shared_ptr<DevPool> ooc_handle_pool(ooc_handle* h);

// Device scratch that only grows: kept across calls and reallocated only when a call needs
// more than it holds (by at least half again, so that a slowly growing need reallocates a
// few times only).  Reallocation frees the old buffer first; callers make sure no work that
// uses it is still queued (every entry point waits for its streams before it returns).
struct GrowBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t b) {
    if (b <= bytes) return OOC_OK;
    const size_t want = std::max(b, bytes + bytes / 2);
    release();
    if (cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return OOC_ERR_NOMEM;
    }
    bytes = want;
    return OOC_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  ~GrowBuf() { release(); }
};
// The handle's workspace for the batched solvers' launch tables.
GrowBuf* ooc_handle_batch_ws(ooc_handle* h);
// The handle's workspace for solves with a stored factor (ooc_dpotrs_L).
GrowBuf* ooc_handle_solve_ws(ooc_handle* h);
// Backward error of a solution x of A x = b (device vectors) for the uniform test matrix
// of `seed` (mixed.cu), A regenerated on the fly.
int ooc_seeded_backward_error(ooc_handle* h, int64_t n, uint64_t seed, double alpha, const double* B, const double* X,
                              double* berr);

// Generators (matgen.cu): fill the block of global rows [r0, r0+m) and columns
// [c0, c0+nc) of the n x n test matrix into the device buffer B (leading dimension ldb).
int launch_gen_uniform_block(double* B, i64 ldb, i64 n, uint64_t seed, double alpha, i64 r0, i64 c0, i64 m,
                             i64 nc, cudaStream_t s);
int launch_gen_pdmatgen_block(double* B, i64 ldb, i64 n, int seed, i64 r0, i64 c0, i64 m, i64 nc,
                              cudaStream_t s);

// ---------------------------------------------------------------------------------
// The uniform test matrix A = (R + R^T)/2 + alpha I element by element (the generator of
// ooc_dmatgen_uniform), for kernels that regenerate A instead of storing it.
// R(i,j) = u - 1/2, u = top 53 bits of SplitMix64 output number i + j*n, state started at
// mix(seed); exact in binary64, so every user of these helpers sees the same bits.
// ---------------------------------------------------------------------------------
__host__ __device__ inline uint64_t ooc_sm64_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__host__ __device__ inline uint64_t ooc_uniform_key(uint64_t seed) { return ooc_sm64_mix(seed + 0x9E3779B97F4A7C15ULL); }
__device__ inline double ooc_r_elem(uint64_t key, uint64_t c) {
  const uint64_t z = ooc_sm64_mix(key + (c + 1) * 0x9E3779B97F4A7C15ULL);
  return __dadd_rn((double)(z >> 11) * 0x1.0p-53, -0.5);
}
// Off-diagonal elements are integer multiples of 2^-54: A(i,j) = (r(i,j) + r(j,i)) / 2 with
// r = u 2^-53 - 1/2 (u the top 53 bits of the SplitMix64 output) equals
// (u(i,j) + u(j,i) - 2^53) 2^-54 exactly, since the sum of the two r's is exact in binary64.
__device__ inline long long ooc_uniform_offdiag_int(uint64_t key, i64 n, i64 i, i64 j) {
  const uint64_t u1 = ooc_sm64_mix(key + ((uint64_t)(i + j * n) + 1) * 0x9E3779B97F4A7C15ULL) >> 11;
  const uint64_t u2 = ooc_sm64_mix(key + ((uint64_t)(j + i * n) + 1) * 0x9E3779B97F4A7C15ULL) >> 11;
  return (long long)(u1 + u2) - (1LL << 53);
}
// ---- conversions on the integer pipe ------------------------------------------------
// FP64 arithmetic and FP64 conversions share a pipe that runs at ~1/64 of FP32 on this
// part, so the reduced-precision paths convert with integer operations (round to nearest
// even, from the IEEE 754 encodings); the rare values outside the FP32 normal range take
// the hardware conversion.
__device__ __forceinline__ float ooc_f64_to_f32(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e < 1023 - 126 || e > 1023 + 127) return __double2float_rn(x);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFULL;
  unsigned int f = ((unsigned int)(b >> 63) << 31) | ((unsigned int)(e - 1023 + 127) << 23) | (unsigned int)(m >> 29);
  const unsigned long long rem = m & 0x1FFFFFFFULL, half = 0x10000000ULL;
  if (rem > half || (rem == half && (f & 1u))) f += 1u;  // a carry moves into the exponent (inf on overflow)
  return __uint_as_float(f);
}
__device__ __forceinline__ double ooc_f32_to_f64(float x) {
  const unsigned int f = __float_as_uint(x);
  const unsigned int e = (f >> 23) & 0xFFu;
  if ((f & 0x7FFFFFFFu) == 0) return __longlong_as_double((long long)((unsigned long long)(f >> 31) << 63));
  if (e == 0 || e == 255) return (double)x;  // subnormal, inf, nan
  const unsigned long long b = ((unsigned long long)(f >> 31) << 63) | ((unsigned long long)(e - 127 + 1023) << 52) |
                               ((unsigned long long)(f & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)b);
}
// RN_f32(v 2^scale) for an integer |v| < 2^62 whose result is an FP32 normal number.
__device__ __forceinline__ float ooc_i64_to_f32_scaled(long long v, int scale) {
  if (v == 0) return 0.f;
  const unsigned int sgn = v < 0 ? 1u : 0u;
  unsigned long long a = sgn ? (unsigned long long)(-v) : (unsigned long long)v;
  const int lz = __clzll((long long)a);
  a <<= lz;  // leading one at bit 63
  unsigned int f = (sgn << 31) | ((unsigned int)(63 - lz + scale + 127) << 23) | ((unsigned int)(a >> 40) & 0x7FFFFFu);
  const unsigned long long rem = a & 0xFFFFFFFFFFULL, half = 0x8000000000ULL;
  if (rem > half || (rem == half && (f & 1u))) f += 1u;
  return __uint_as_float(f);
}

__device__ inline double ooc_uniform_elem(uint64_t key, i64 n, double alpha, i64 i, i64 j) {
  if (i == j) return __dadd_rn(ooc_r_elem(key, (uint64_t)(i + j * n)), alpha);
  return (double)ooc_uniform_offdiag_int(key, n, i, j) * 0x1.0p-54;
}
// RN_f32 of the same element (exact integer path off the diagonal).
__device__ inline float ooc_uniform_elem_f32(uint64_t key, i64 n, double alpha, i64 i, i64 j) {
  if (i == j) return ooc_f64_to_f32(__dadd_rn(ooc_r_elem(key, (uint64_t)(i + j * n)), alpha));
  return ooc_i64_to_f32_scaled(ooc_uniform_offdiag_int(key, n, i, j), -54);
}
// b(i) ~ N(0,1) for right-hand sides: Box-Muller on two SplitMix64 uniforms of stream
// `key`, element index i (column-major over the right-hand sides).
__device__ inline double ooc_normal_elem(uint64_t key, uint64_t i) {
  const uint64_t z1 = ooc_sm64_mix(key + (2 * i + 1) * 0x9E3779B97F4A7C15ULL);
  const uint64_t z2 = ooc_sm64_mix(key + (2 * i + 2) * 0x9E3779B97F4A7C15ULL);
  const double u1 = ((double)(z1 >> 11) + 0.5) * 0x1.0p-53;  // (0, 1)
  const double u2 = (double)(z2 >> 11) * 0x1.0p-53;
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// Lower-triangular blocks (bi, bj), bj in [lo, hi), bi in [bj, T), enumerated column by
// column: column c holds T - c blocks and S(c) = c T - c (c - 1) / 2 blocks precede it.
__host__ __device__ inline i64 ooc_lower_blocks_before(i64 c, i64 T) { return c * T - c * (c - 1) / 2; }
__device__ inline void ooc_lower_block_decode(i64 t, int T, int lo, int* bi, int* bj) {
  const i64 u = t + ooc_lower_blocks_before(lo, T);
  const double b = 2.0 * T + 1.0;
  i64 c = (i64)floor((b - sqrt(fmax(b * b - 8.0 * (double)u, 0.0))) * 0.5);
  if (c < 0) c = 0;
  while (c > 0 && ooc_lower_blocks_before(c, T) > u) c--;
  while (ooc_lower_blocks_before(c + 1, T) <= u) c++;
  *bj = (int)c;
  *bi = (int)(c + (u - ooc_lower_blocks_before(c, T)));
}
