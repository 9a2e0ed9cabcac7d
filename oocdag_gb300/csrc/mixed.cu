// Mixed-precision factorization and FP64 solves with iterative refinement.
//
// Factor objects.  OOC_PREC_FP64 is the plain path's right-looking factorization (device
// potrf, inverse-based column solve and DMMA updates).  The reduced precisions keep the
// reference's per-panel structure (diagonal-tile potrf, column solve, trailing syrk/gemm:
// oocquark.cpp:393-410, 346, 351) on an FP32 working matrix that becomes the factor:
//   diagonal tile  : FP32 Cholesky and inverse in one CTA (k_diag_s256 for tiles of up to
//                    256 columns, held in shared memory; k_diag_f32 for wider ones);
//   column solve   : the panel times the tile's inverse, in FP32 (k_colsolve_f32) or as
//                    three split-BF16 tensor-core products (k_trsm2_bf16x3, tc_bf16x3.cu);
//   trailing update: OOC_PREC_FP32 - FP32 FFMA products (k_syrk_f32);
//                    OOC_PREC_BF16X3 - hi/lo BF16 planes of the panel, three tensor-core
//                    products (hi*hi + hi*lo + lo*hi) accumulated in FP32 in TMEM and added
//                    into the FP32 trailing matrix by TMA reductions (k_syrk2_bf16x3).
// Split-BF16 factors use nb/2-wide panels for the last OOC_OPT_TAIL_ORDER orders.
// Solves use the kept inverses of the diagonal tiles (solve_with).  The refinement
// computes residuals in FP64 against the FP64 matrix (device, or the lower triangle of a
// host matrix copied once), and corrects with the FP32 factor until the normwise backward
// error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) reaches the tolerance.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <mutex>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "devpool.cuh"

namespace {

// ---------------------------------------------------------------------------------
// FP32 lower-triangular rank-K update: C (FP32 or FP64, lower) -= X X^T with X (m x K, FP32,
// column-major, ld ldx).  128 x 128 output blocks, lower-triangular block grid.
// ---------------------------------------------------------------------------------
constexpr int FB = 128, FK = 16, FTHR = 256;

__device__ __forceinline__ void cp_async16f(void* smem, const void* gmem, int src_bytes) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes));
}

__device__ __forceinline__ void load_slab_f32(float* S, const float* X, i64 ldx, int r0, int m, int k0, int K) {
  // 128 rows x 16 k; each k column holds 128 contiguous floats = 32 x 16 B.
  for (int idx = threadIdx.x; idx < FK * (FB / 4); idx += FTHR) {
    const int kc = idx / (FB / 4);
    const int r = (idx % (FB / 4)) * 4;
    const int gr = r0 + r, gk = k0 + kc;
    int nv = 0;
    if (gk < K) nv = min(max(m - gr, 0), 4);
    const float* src = nv > 0 ? X + gr + (i64)gk * ldx : X;
    cp_async16f(S + kc * FB + r, src, nv * 4);
  }
}

template <typename TC>
__global__ void __launch_bounds__(FTHR) k_syrk_f32(const float* __restrict__ X, i64 ldx, TC* __restrict__ C,
                                                   i64 ldc, int m, int K, int T, int bj_lo, const int* status) {
  if (status && *(volatile const int*)status) return;
  int bi, bj;
  ooc_lower_block_decode((i64)blockIdx.x, T, bj_lo, &bi, &bj);
  const int m0 = bi * FB, n0 = bj * FB;
  // 32 KB: double-buffered A and B slabs, reused afterwards to stage the result.
  __shared__ __align__(16) float smem[4 * FK * FB];
  float* As[2] = {smem, smem + FK * FB};
  float* Bs[2] = {smem + 2 * FK * FB, smem + 3 * FK * FB};
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int j = 0; j < 8; j++) acc[i][j] = 0.f;
  const int nslab = (K + FK - 1) / FK;
  load_slab_f32(As[0], X, ldx, m0, m, 0, K);
  load_slab_f32(Bs[0], X, ldx, n0, m, 0, K);
  asm volatile("cp.async.commit_group;\n" ::);
  for (int s = 0; s < nslab; s++) {
    const int cur = s & 1;
    if (s + 1 < nslab) {
      load_slab_f32(As[cur ^ 1], X, ldx, m0, m, (s + 1) * FK, K);
      load_slab_f32(Bs[cur ^ 1], X, ldx, n0, m, (s + 1) * FK, K);
      asm volatile("cp.async.commit_group;\n" ::);
      asm volatile("cp.async.wait_group 1;\n" ::);
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::);
    }
    __syncthreads();
    const float* as = As[cur];
    const float* bs = Bs[cur];
#pragma unroll
    for (int k = 0; k < FK; k++) {
      const float4 a0 = *reinterpret_cast<const float4*>(as + k * FB + ty * 4);
      const float4 a1 = *reinterpret_cast<const float4*>(as + k * FB + 64 + ty * 4);
      const float4 b0 = *reinterpret_cast<const float4*>(bs + k * FB + tx * 4);
      const float4 b1 = *reinterpret_cast<const float4*>(bs + k * FB + 64 + tx * 4);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  // Stage the block through shared memory, 32 columns at a time (stride 129 floats),
  // so that the FP64 read-modify-write of C walks whole columns (coalesced).
  // Thread columns: quarter 0 = tx*4+j for tx < 8, quarter 1 = tx*4+j for tx >= 8,
  // quarters 2/3 the same shifted by 64.
  float* stage = smem;
  const int warp = tid >> 5, lane = tid & 31;
#pragma unroll
  for (int qtr = 0; qtr < 4; qtr++) {
    const int half = qtr >> 1;      // which group of 4 accumulator columns
    const int lo_tx = (qtr & 1) * 8;  // threads whose columns fall in this quarter
    if (tx >= lo_tx && tx < lo_tx + 8) {
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const int rr = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int cc = (tx - lo_tx) * 4 + j;  // 0..31 inside this quarter
          stage[cc * 129 + rr] = acc[i][half * 4 + j];
        }
      }
    }
    __syncthreads();
    // each warp: 4 columns x 128 rows; all loads before the stores
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int cc = warp * 4 + u;
      const int c = n0 + half * 64 + (qtr & 1) * 32 + cc;
      TC cv[4];
      bool ok[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int r = m0 + lane + 32 * q;
        ok[q] = (c < m) && (r < m) && !(bi == bj && c > r);
        cv[q] = ok[q] ? C[r + (i64)c * ldc] : TC(0);
      }
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int rr = lane + 32 * q;
        if (ok[q]) C[m0 + rr + (i64)c * ldc] = cv[q] - (TC)stage[cc * 129 + rr];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// Column solve of a reduced-precision factor, in place:  P (m x LN, FP32, ld ldp) :=
// P X^T with X = L_jj^{-1} (LN x LN, FP32, lower, exact zeros above the diagonal), given
// row-major in Xr (ld ldxr).  This is the dtrsm task (oocquark.cpp:130) as a product with
// the kept inverse.  One CTA per 64-row block walks the 128-column blocks from the last to
// the first: output block cb needs P's columns k < 128 (cb + 1) only, which no block
// written before it touches.
// ---------------------------------------------------------------------------------
constexpr int CS_ROWS = 64;           // rows per CTA
constexpr int CS_COLS = 128;          // output columns per pass
constexpr int CS_BP = CS_COLS + 4;    // B slab row stride: float4-aligned, few bank conflicts on the transposed store

__global__ void __launch_bounds__(FTHR, 2) k_colsolve_f32(float* __restrict__ P, i64 ldp, const float* __restrict__ Xr,
                                                          i64 ldxr, int m, int LN, const int* status) {
  if (status && *(volatile const int*)status) return;
  __shared__ __align__(16) float smem[2 * FK * CS_ROWS + 2 * FK * CS_BP];  // A, B slabs (x2), then output stage
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;  // 8 columns (tx*4.., 64+tx*4..) x 4 rows (ty*4..)
  const int warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.x * CS_ROWS;
  constexpr int PA = FK * CS_ROWS / FTHR;  // 4 A elements per thread and slab
  constexpr int PB = FK * CS_COLS / FTHR;  // 8 B elements per thread and slab
  for (int cb = (LN - 1) / CS_COLS; cb >= 0; cb--) {
    const int c0 = cb * CS_COLS;
    const int kend = min(LN, c0 + CS_COLS);
    const int nslab = (kend + FK - 1) / FK;
    float acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 8; j++) acc[i][j] = 0.f;
    float ra[PA], rb[PB];
    auto fetch = [&](int k0) {
#pragma unroll
      for (int u = 0; u < PA; u++) {
        const int idx = tid + u * FTHR;
        const int kc = idx / CS_ROWS, x = idx % CS_ROWS;
        const int gk = k0 + kc;
        ra[u] = (r0 + x < m && gk < kend) ? P[(r0 + x) + (i64)gk * ldp] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < PB; u++) {
        const int idx = tid + u * FTHR;
        const int xb = idx / FK, kb2 = idx % FK;  // consecutive threads read consecutive k of X's row c
        rb[u] = (c0 + xb < LN && k0 + kb2 < kend) ? Xr[(i64)(c0 + xb) * ldxr + k0 + kb2] : 0.f;  // (X^T)(k, c)
      }
    };
    fetch(0);
    for (int s = 0; s < nslab; s++) {
      float* as_w = smem + (s & 1) * FK * CS_ROWS;
      float* bs_w = smem + 2 * FK * CS_ROWS + (s & 1) * FK * CS_BP;
#pragma unroll
      for (int u = 0; u < PA; u++) as_w[tid + u * FTHR] = ra[u];
#pragma unroll
      for (int u = 0; u < PB; u++) {
        const int idx = tid + u * FTHR;
        bs_w[(idx % FK) * CS_BP + idx / FK] = rb[u];
      }
      __syncthreads();
      if (s + 1 < nslab) fetch((s + 1) * FK);
#pragma unroll
      for (int k = 0; k < FK; k++) {
        const float4 a0 = *reinterpret_cast<const float4*>(as_w + k * CS_ROWS + ty * 4);
        const float4 b0 = *reinterpret_cast<const float4*>(bs_w + k * CS_BP + tx * 4);
        const float4 b1 = *reinterpret_cast<const float4*>(bs_w + k * CS_BP + 64 + tx * 4);
        const float a[4] = {a0.x, a0.y, a0.z, a0.w};
        const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 8; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
      }
    }
    __syncthreads();  // every read of P's columns < kend is done before any store below
    // Store through shared memory 32 columns at a time (stride CS_ROWS + 1) so each warp
    // writes whole column segments (coalesced).
    float* stage = smem;
#pragma unroll
    for (int qtr = 0; qtr < 4; qtr++) {
      const int half = qtr >> 1;
      const int lo_tx = (qtr & 1) * 8;
      if (tx >= lo_tx && tx < lo_tx + 8) {
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) stage[((tx - lo_tx) * 4 + j) * (CS_ROWS + 1) + ty * 4 + i] = acc[i][half * 4 + j];
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int cc = warp * 4 + u;
        const int c = c0 + half * 64 + (qtr & 1) * 32 + cc;
#pragma unroll
        for (int q = 0; q < 2; q++) {
          const int rr = lane + 32 * q;
          if (c < LN && r0 + rr < m) P[(r0 + rr) + (i64)c * ldp] = stage[cc * (CS_ROWS + 1) + rr];
        }
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------------
// Diagonal tile of a reduced-precision factor, fused in one CTA and in FP32:
//   L_jj = chol(D) (the dpotrf task, oocquark.cpp:87/393), X = L_jj^{-1},
// in place in the FP32 working matrix: D's lower triangle := L_jj, Dinv := X^T (upper,
// zeros below, ld lde), Xr := X row-major (ld LN; the column solve reads it).
// Both phases are left-looking over 32-wide blocks, so every element is computed in
// registers from finished data (D itself and Xr, a row-major FP32 scratch copy of X with
// ld LN, both L2-resident) and written once:
//   phase 1, block column K: C = A(K:, K) - L(K:, :K) L(K, :K)^T (thread per row, the
//            32 L(K, :K) rows staged in shared memory), one warp factors C's 32 x 32 top
//            in registers, one thread per row solves the rows below;
//   phase 2, block row I:    X(I, j) = -L_II^{-1} sum_q L(I, q) X(q, j) (thread per
//            column j, the L(I, :I) rows staged), X(I, I) = L_II^{-1}.
// A non-positive pivot writes info = col0 + j + 1 to the status word and stops.
// ---------------------------------------------------------------------------------
constexpr int DG_THREADS = 512, DG_B = 32, DG_LD = 33, DG_MAX = 512;
constexpr int DG_WARPS = DG_THREADS / 32;
constexpr int DG_STEPS = 2 * (DG_MAX / DG_B);  // phase 1 and phase 2 steps
constexpr size_t DG_SMEM =
    (size_t)(DG_MAX * DG_B + DG_MAX * DG_LD + DG_WARPS * 32 * DG_LD + 2 * DG_B * DG_LD + DG_B) * sizeof(float) +
    (size_t)DG_STEPS * DG_WARPS * sizeof(int4);


// acc[c] += sum over q in [qa, qb) of v(q) S[q * 32 + c], v(q) = src[q * stride] for
// q >= qmask, else 0; qa is a multiple of 8 and the same for the whole warp.
__device__ __forceinline__ void dg_dot_range(float acc[DG_B], const float* src, i64 stride, int qa, int qb,
                                             int qmask, const float* __restrict__ S) {
  if (qa >= qb) return;
  float nx[8];
#pragma unroll
  for (int u = 0; u < 8; u++) {
    const int q = qa + u;
    nx[u] = (q >= qmask && q < qb) ? src[q * stride] : 0.f;
  }
  for (int q0 = qa; q0 < qb; q0 += 8) {
    float x[8];
#pragma unroll
    for (int u = 0; u < 8; u++) x[u] = nx[u];
    if (q0 + 8 < qb) {
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int q = q0 + 8 + u;
        nx[u] = (q >= qmask && q < qb) ? src[q * stride] : 0.f;
      }
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const float4* b4 = reinterpret_cast<const float4*>(S + (q0 + u) * DG_B);
#pragma unroll
      for (int v = 0; v < DG_B / 4; v++) {
        const float4 bb = b4[v];
        acc[4 * v + 0] = fmaf(x[u], bb.x, acc[4 * v + 0]);
        acc[4 * v + 1] = fmaf(x[u], bb.y, acc[4 * v + 1]);
        acc[4 * v + 2] = fmaf(x[u], bb.z, acc[4 * v + 2]);
        acc[4 * v + 3] = fmaf(x[u], bb.w, acc[4 * v + 3]);
      }
    }
  }
}

// Splits `njobs` reductions of len[j] 32-wide steps over the CTA's warps: every job gets
// one chunk, the rest go one at a time to the job with the longest chunk (ties to the
// lower job).  For each warp w: its job (-1: none), its chunk's step range [a, b) and the
// number of chunks of its job (the chunks of a job are consecutive warps).
__device__ void dg_plan_all(const int* len, int njobs, int* job, int* qa, int* qb, int* nch) {
  int ch[DG_WARPS];
  for (int j = 0; j < DG_WARPS; j++) ch[j] = (j < njobs) ? 1 : 0;
  for (int extra = DG_WARPS - njobs; extra > 0; extra--) {
    int best = -1;
    for (int j = 0; j < njobs; j++)
      if (len[j] > ch[j] && (best < 0 || len[j] * ch[best] > len[best] * ch[j])) best = j;
    if (best < 0) break;
    ch[best]++;
  }
  int w = 0;
  for (int j = 0; j < njobs; j++)
    for (int c = 0; c < ch[j]; c++, w++) {
      job[w] = j;
      nch[w] = ch[j];
      qa[w] = (len[j] * c) / ch[j];
      qb[w] = (len[j] * (c + 1)) / ch[j];
    }
  for (; w < DG_WARPS; w++) { job[w] = -1; nch[w] = 0; qa[w] = 1; qb[w] = 0; }
}

// S[q * 32 + c] = Lw(r0 + c, q) for q < nq, c < cb (0 for c >= cb): every load of the
// thread is issued before the first store (a loop with one load per iteration would
// wait an L2 round trip per element).
__device__ __forceinline__ void dg_stage(float* __restrict__ S, const float* Lw, i64 ldw, int r0, int nq, int cb) {
  constexpr int PER = DG_MAX * DG_B / DG_THREADS;  // 32 elements per thread at most
  float v[PER];
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int idx = threadIdx.x + u * DG_THREADS;
    const int q = idx >> 5, c = idx & 31;
    v[u] = (q < nq && c < cb) ? Lw[(r0 + c) + q * ldw] : 0.f;
  }
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int idx = threadIdx.x + u * DG_THREADS;
    if ((idx >> 5) < nq) S[idx] = v[u];
  }
}

// hi/lo BF16 split of one element of the inverse (the tensor-core column solve's operand)
__device__ __forceinline__ void dg_split_store(__nv_bfloat16* Xh, __nv_bfloat16* Xl, i64 idx, float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  Xh[idx] = h;
  Xl[idx] = __float2bfloat16_rn(v - __bfloat162float(h));
}

__global__ void __launch_bounds__(DG_THREADS, 1)
    k_diag_f32(float* D, i64 ldd, int LN, i64 col0, float* __restrict__ Dinv, i64 lde, float* __restrict__ Xr,
               __nv_bfloat16* __restrict__ Xh, __nv_bfloat16* __restrict__ Xl, int* status) {
  if (*(volatile int*)status) return;
  extern __shared__ __align__(16) float dsm[];
  float* S = dsm;                      // staged rows, q-major: S[q * 32 + r]
  float* Cs = S + DG_MAX * DG_B;       // phase 1: the block column being finished, Cs[t * DG_LD + c]
  float* Ps = Cs + DG_MAX * DG_LD;     // per-warp partial sums, Ps[(w * 32 + lane) * DG_LD + c]
  float* Dk = Ps + DG_WARPS * 32 * DG_LD;  // L(K, K), Dk[r * DG_LD + c]
  float* Li = Dk + DG_B * DG_LD;       // phase 2: L_II^{-1}, Li[r * DG_LD + c]
  float* dinv = Li + DG_B * DG_LD;     // 1 / L(k + c, k + c)
  int4* plan = reinterpret_cast<int4*>(dinv + DG_B);  // [step][warp] = (job, qa, qb, nch)
  __shared__ int s_fail;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  float* Lw = D;  // L overwrites A in place
  const i64 ldw = ldd;
  const i64 ldx = LN;  // Xr
  if (t == 0) s_fail = 0;
  // Work plans of all steps, one thread per step (phase 1: block column K, jobs = row tiles
  // of length K; phase 2: block row I, jobs = column tiles jt of length I - jt).
  const int nsteps = (LN + DG_B - 1) / DG_B;
  if (t < 2 * nsteps) {
    int len[DG_WARPS], job[DG_WARPS], qa[DG_WARPS], qb[DG_WARPS], nch[DG_WARPS];
    int njobs;
    if (t < nsteps) {
      const int K = t;
      njobs = (LN - K * DG_B + DG_B - 1) / DG_B;
      for (int j = 0; j < DG_WARPS; j++) len[j] = K;
    } else {
      const int I = t - nsteps;
      njobs = I < DG_WARPS ? I : DG_WARPS;
      for (int j = 0; j < DG_WARPS; j++) len[j] = I - j;
    }
    dg_plan_all(len, njobs, job, qa, qb, nch);
    for (int w = 0; w < DG_WARPS; w++) plan[t * DG_WARPS + w] = make_int4(job[w], qa[w], qb[w], nch[w]);
  }
  __syncthreads();
  // ---- phase 1: L = chol(D), block columns left to right.  Block column K: the row tiles
  // below k0 are the jobs, each a reduction over the K earlier block columns, split across
  // the warps; the chunks' partial sums are added in order by the job's first warp.
  for (int k0 = 0; k0 < LN; k0 += DG_B) {
    const int kb = min(DG_B, LN - k0), mK = LN - k0;
    const int K = k0 / DG_B;
    dg_stage(S, Lw, ldw, k0, k0, kb);
    __syncthreads();
    const int4 pw = plan[K * DG_WARPS + warp];
    const int job = pw.x, qa = pw.y, qb = pw.z, nch = pw.w;
    if (job >= 0) {
      const int rr = job * DG_B + lane;  // row within the block column
      float acc[DG_B];
#pragma unroll
      for (int c = 0; c < DG_B; c++) acc[c] = 0.f;
      if (rr < mK) dg_dot_range(acc, Lw + k0 + rr, ldw, qa * DG_B, qb * DG_B, 0, S);
#pragma unroll
      for (int c = 0; c < DG_B; c++) Ps[(warp * 32 + lane) * DG_LD + c] = acc[c];
    }
    __syncthreads();
    if (job >= 0 && qa == 0) {  // C = A - sum of the chunks, in chunk order
      const int rr = job * DG_B + lane;
      if (rr < mK) {
        const int i = k0 + rr;
        float cv[DG_B];
#pragma unroll
        for (int c = 0; c < DG_B; c++) cv[c] = (c < kb && c <= rr) ? Lw[i + (i64)(k0 + c) * ldw] : 0.f;
        for (int w2 = warp; w2 < warp + nch; w2++)
#pragma unroll
          for (int c = 0; c < DG_B; c++) cv[c] -= Ps[(w2 * 32 + lane) * DG_LD + c];
#pragma unroll
        for (int c = 0; c < DG_B; c++) Cs[rr * DG_LD + c] = cv[c];
      }
    }
    __syncthreads();
    if (warp == 0) {
      // 32 x 32 Cholesky in registers: lane r holds row r.  Column j is published through
      // shared memory (one store, then independent broadcast loads), not shuffles whose
      // latency each update would wait for.  Straight-line code: a non-positive pivot is
      // recorded and replaced by 1 so the remaining steps stay finite; the first is reported.
      float a[DG_B];
      float* colb = Li;  // free during phase 1
#pragma unroll
      for (int c = 0; c < DG_B; c++) a[c] = (lane < kb && c <= lane) ? Cs[lane * DG_LD + c] : ((c == lane) ? 1.f : 0.f);
      int first_bad = DG_B;
#pragma unroll
      for (int j = 0; j < DG_B; j++) {
        colb[lane] = a[j];
        __syncwarp();
        float d = colb[j];
        if (!(d > 0.f)) {
          first_bad = min(first_bad, j);
          d = 1.f;
        }
        const float inv = rsqrtf(d);
        const float lj = (lane == j) ? d * inv : a[j] * inv;  // L(lane, j)
        const float ljs = lj * inv;                             // L(lane, j) / sqrt(d)
        if (lane == j) dinv[j] = inv;
        a[j] = (lane >= j) ? lj : a[j];
#pragma unroll
        for (int c = j + 1; c < DG_B; c++)  // A(lane, c) -= L(lane, j) L(c, j), L(c, j) = A(c, j) / sqrt(d)
          if (lane >= c) a[c] = fmaf(-ljs, colb[c], a[c]);
        __syncwarp();
      }
      if (first_bad < kb && lane == 0) { s_fail = 1; atomicCAS(status, 0, (int)(col0 + k0 + first_bad + 1)); }
#pragma unroll
      for (int c = 0; c < DG_B; c++) Dk[lane * DG_LD + c] = (c <= lane) ? a[c] : 0.f;
    }
    __syncthreads();
    if (s_fail) break;
    if (t < mK) {
      const int i = k0 + t;
      float row[DG_B];
      if (t < kb) {
#pragma unroll
        for (int c = 0; c < DG_B; c++) row[c] = Dk[t * DG_LD + c];
      } else {  // B := B L_KK^{-T}, one thread per row
#pragma unroll
        for (int c = 0; c < DG_B; c++) row[c] = Cs[t * DG_LD + c];
#pragma unroll
        for (int c = 0; c < DG_B; c++) {
          float v = row[c];
#pragma unroll
          for (int q = 0; q < c; q++) v = fmaf(-row[q], Dk[c * DG_LD + q], v);
          row[c] = v * dinv[c];
        }
      }
#pragma unroll
      for (int c = 0; c < DG_B; c++)
        if (c < kb && c <= t) Lw[i + (k0 + c) * ldw] = row[c];
    }
    __syncthreads();
  }
  if (s_fail) return;
  // ---- phase 2: X = L^{-1}, block rows top to bottom.  Block row I: the column tiles jt < I
  // are the jobs, each a reduction over the block rows jt .. I-1, split across the warps.
  for (int i0 = 0; i0 < LN; i0 += DG_B) {
    const int ib = min(DG_B, LN - i0), I = i0 / DG_B;
    dg_stage(S, Lw, ldw, i0, i0, ib);
    for (int idx = t; idx < DG_B * DG_B; idx += DG_THREADS) {
      const int r = idx >> 5, c = idx & 31;
      Dk[r * DG_LD + c] = (r < ib && c <= r) ? Lw[(i0 + r) + (i0 + c) * ldw] : 0.f;
    }
    __syncthreads();
    const int4 pw = plan[(nsteps + I) * DG_WARPS + warp];
    const int job = pw.x, qa = pw.y, qb = pw.z, nch = pw.w;
    if (warp == DG_WARPS - 1) {  // L_II^{-1}: lane c solves L_II x = e_c (concurrently with the chunks)
      float x[DG_B];
#pragma unroll
      for (int r = 0; r < DG_B; r++) {
        float v = (r == lane) ? 1.f : 0.f;
#pragma unroll
        for (int q = 0; q < r; q++) v = fmaf(-Dk[r * DG_LD + q], x[q], v);
        x[r] = (r < ib) ? v / Dk[r * DG_LD + r] : 0.f;
      }
#pragma unroll
      for (int r = 0; r < DG_B; r++) Li[r * DG_LD + lane] = x[r];
    }
    if (job >= 0) {
      const int j = job * DG_B + lane;  // column of X
      float acc[DG_B];
#pragma unroll
      for (int r = 0; r < DG_B; r++) acc[r] = 0.f;
      // acc[r] = sum_q L(i0 + r, q) X(q, j) over the chunk's block rows jt + qa .. jt + qb - 1
      dg_dot_range(acc, Xr + j, ldx, (job + qa) * DG_B, (job + qb) * DG_B, j, S);
#pragma unroll
      for (int r = 0; r < DG_B; r++) Ps[(warp * 32 + lane) * DG_LD + r] = acc[r];
    }
    __syncthreads();
    if (job >= 0 && qa == 0) {
      const int j = job * DG_B + lane;
      float acc[DG_B];
#pragma unroll
      for (int r = 0; r < DG_B; r++) acc[r] = 0.f;
      for (int w2 = warp; w2 < warp + nch; w2++)
#pragma unroll
        for (int r = 0; r < DG_B; r++) acc[r] += Ps[(w2 * 32 + lane) * DG_LD + r];
      float y[DG_B];
#pragma unroll
      for (int r = 0; r < DG_B; r++) {
        float v = 0.f;
#pragma unroll
        for (int s2 = 0; s2 <= r; s2++) v = fmaf(Li[r * DG_LD + s2], acc[s2], v);
        y[r] = -v;
      }
#pragma unroll
      for (int r = 0; r < DG_B; r++)
        if (r < ib) {
          Xr[(i0 + r) * ldx + j] = y[r];
          Dinv[j + (i64)(i0 + r) * lde] = y[r];
          if (Xh) dg_split_store(Xh, Xl, (i0 + r) * ldx + j, y[r]);
        }
    }
    if (t >= i0 && t < LN) {
      const int c = t - i0;  // diagonal block column (c < ib) or right of it (zeros)
#pragma unroll
      for (int r = 0; r < DG_B; r++)
        if (r < ib) {
          const float y = (c < ib && r >= c) ? Li[r * DG_LD + c] : 0.f;
          Xr[(i0 + r) * ldx + t] = y;
          Dinv[t + (i64)(i0 + r) * lde] = y;
          if (Xh) dg_split_store(Xh, Xl, (i0 + r) * ldx + t, y);
        }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// The same outputs for a diagonal tile of at most 256 columns, with the whole tile in
// shared memory: its lower block triangle as 32 x 32 blocks (row-major, pitch 36), padded
// to a multiple of 32 with the identity.  k_diag_f32 re-reads the finished columns from L2
// in every step, and beside the trailing update (which loads L2 heavily) those round trips,
// not its arithmetic, set its time; here no step waits on L2, and every block product runs
// from registers (a 4 x 8 tile per lane, 16-byte shared loads).
//   phase 1, block column K (right-looking): one warp factors L_KK in registers; one
//            thread per row below solves its row against L_KK^T (the solved rows also
//            go, transposed, into PT, and to D) while a warp forms X_KK = L_KK^{-1}; then
//            each block (I, J), K < J <= I, takes -= L(I,K) L(J,K)^T, a warp a block.
//   phase 2, X = L^{-1} in place (right-looking): block row K of X is X_KK times the
//            finished block row; then each block (I, J), I > K, J <= K, takes
//            -= L(I,K) X(K,J) (for J = K: := -L(I,K) X_KK).
// Phase 2 runs one step behind phase 1, in the warps that the serial parts of phase 1
// leave idle (its products of step K-1 beside the Cholesky of block K, while PT still holds
// L(., K-1)), so the two phases share their barriers.
// Dinv (= X^T), and X row-major as BF16 planes (or in FP32 into Xr when no planes are
// asked for), at the end.  A non-positive pivot writes
// info = col0 + j + 1 to the status word and stops, the columns left of the failed block
// written, the others left as they were (as k_diag_f32).
// ---------------------------------------------------------------------------------
constexpr int DS_MAX = 256, DS_NBK = DS_MAX / DG_B, DS_P = 36, DS_BLK = DG_B * DS_P;
constexpr int DS_NBLK = DS_NBK * (DS_NBK + 1) / 2;
constexpr int DS_PTLD = DS_MAX - DG_B + 4;  // rows below a block column, 16-byte multiple
constexpr size_t DS_SMEM =
    (size_t)((DS_NBLK + DS_NBK) * DS_BLK + DG_B * DS_PTLD + 2 * DG_B) * sizeof(float);
static_assert(DS_SMEM + 64 <= 227 * 1024 && DG_SMEM + 64 <= 227 * 1024,
              "a diagonal kernel's shared memory exceeds the 227 KB a CTA may opt in to");

// block b of a lower block triangle stored row by row -> (I, J), J <= I
__device__ __forceinline__ void ds_block_ij(int b, int& I, int& J) {
  int i = (int)((sqrtf(8.f * (float)b + 1.f) - 1.f) * 0.5f);
  if ((i + 1) * (i + 2) / 2 <= b) i++;
  if (i * (i + 1) / 2 > b) i--;
  I = i;
  J = b - i * (i + 1) / 2;
}

// acc[i][j] += sum over k < 32 of A[k lda + r0 + i] B[k ldb + c0 + j]: lane's 4 x 8 tile of
// a 32 x 32 block product (A and B k-major, rows 16-byte aligned)
__device__ __forceinline__ void ds_mm32(float acc[4][8], const float* A, int lda, const float* B, int ldb, int r0,
                                        int c0) {
#pragma unroll 8
  for (int k = 0; k < DG_B; k++) {
    const float4 a = *reinterpret_cast<const float4*>(A + k * lda + r0);
    const float4 b0 = *reinterpret_cast<const float4*>(B + k * ldb + c0);
    const float4 b1 = *reinterpret_cast<const float4*>(B + k * ldb + c0 + 4);
    const float av[4] = {a.x, a.y, a.z, a.w};
    const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 8; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
  }
}

// the lane's tile of block C (pitch DS_P) := C - acc (mode 0), -acc (mode 1) or acc (mode 2)
__device__ __forceinline__ void ds_put(float* C, const float acc[4][8], int r0, int c0, int mode) {
#pragma unroll
  for (int i = 0; i < 4; i++) {
    float4* p = reinterpret_cast<float4*>(C + (r0 + i) * DS_P + c0);
    float v[8];
    if (mode == 0) {
      const float4 u = p[0], w = p[1];
      const float cv[8] = {u.x, u.y, u.z, u.w, w.x, w.y, w.z, w.w};
#pragma unroll
      for (int j = 0; j < 8; j++) v[j] = cv[j] - acc[i][j];
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) v[j] = (mode == 1) ? -acc[i][j] : acc[i][j];
    }
    p[0] = make_float4(v[0], v[1], v[2], v[3]);
    p[1] = make_float4(v[4], v[5], v[6], v[7]);
  }
}

// 32 x 32 Cholesky of a diagonal block (pitch DS_P) by one warp, in registers (lane r = row
// r, as in k_diag_f32): the block's lower triangle := L (zeros above), dinv := 1 / diag(L).
// Rows and columns from kb on are taken as the identity.  A non-positive pivot in the first
// kb columns sets *fail and writes info = colg + j + 1 to the status word.
__device__ __forceinline__ void ds_chol32(float* Tb, int kb, i64 colg, float* colb, float* dinv, int* fail,
                                          int* status, int lane) {
  float a[DG_B];
#pragma unroll
  for (int c = 0; c < DG_B; c++) a[c] = (lane < kb && c <= lane) ? Tb[lane * DS_P + c] : ((c == lane) ? 1.f : 0.f);
  int first_bad = DG_B;
#pragma unroll
  for (int j = 0; j < DG_B; j++) {
    colb[lane] = a[j];
    __syncwarp();
    float d = colb[j];
    if (!(d > 0.f)) {
      first_bad = min(first_bad, j);
      d = 1.f;
    }
    const float inv = rsqrtf(d);
    const float lj = (lane == j) ? d * inv : a[j] * inv;  // L(lane, j)
    const float ljs = lj * inv;                             // L(lane, j) / sqrt(d)
    if (lane == j) dinv[j] = inv;
    a[j] = (lane >= j) ? lj : a[j];
#pragma unroll
    for (int c = j + 1; c < DG_B; c++)
      if (lane >= c) a[c] = fmaf(-ljs, colb[c], a[c]);
    __syncwarp();
  }
  if (first_bad < kb && lane == 0) {
    *fail = 1;
    atomicCAS(status, 0, (int)(colg + first_bad + 1));
  }
#pragma unroll
  for (int c = 0; c < DG_B; c++) Tb[lane * DS_P + c] = (c <= lane) ? a[c] : 0.f;
}

__global__ void __launch_bounds__(DG_THREADS, 1)
    k_diag_s256(float* D, i64 ldd, int LN, i64 col0, float* __restrict__ Dinv, i64 lde, float* __restrict__ Xr,
                __nv_bfloat16* __restrict__ Xh, __nv_bfloat16* __restrict__ Xl, int* status) {
  if (*(volatile int*)status) return;
  extern __shared__ __align__(16) float dss[];
  float* T = dss;                         // block (I, J) at (I (I + 1) / 2 + J) DS_BLK
  float* XD = T + DS_NBLK * DS_BLK;       // X_KK transposed: XD[K DS_BLK + k DS_P + r] = X_KK(r, k)
  float* PT = XD + DS_NBK * DS_BLK;       // block column K below its diagonal, transposed
  float* dinv = PT + DG_B * DS_PTLD;      // 1 / L(k0 + c, k0 + c)
  float* colb = dinv + DG_B;              // the warp Cholesky's column broadcast
  __shared__ int s_fail;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int NBK = (LN + DG_B - 1) / DG_B;
  const int r0 = (lane & 7) * 4, c0 = (lane >> 3) * 8;  // the lane's tile of a block product
  auto blk = [&](int I, int J) -> float* { return T + (I * (I + 1) / 2 + J) * DS_BLK; };
  if (t == 0) s_fail = 0;
  {  // the lower block triangle, 24 loads in flight per thread (lanes down a column)
    constexpr int U = 24;
    const int total = NBK * (NBK + 1) / 2 * DG_B * DG_B;
    for (int base = 0; base < total; base += U * DG_THREADS) {
      float v[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int idx = base + u * DG_THREADS + t;
        float x = 0.f;
        if (idx < total) {
          int I, J;
          ds_block_ij(idx >> 10, I, J);
          const int i = I * DG_B + (idx & 31), j = J * DG_B + ((idx >> 5) & 31);
          if (i < LN && j < LN) {
            if (i >= j) x = D[i + (i64)j * ldd];
          } else if (i == j) {
            x = 1.f;
          }
        }
        v[u] = x;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int idx = base + u * DG_THREADS + t;
        if (idx < total) T[(idx >> 10) * DS_BLK + (idx & 31) * DS_P + ((idx >> 5) & 31)] = v[u];
      }
    }
  }
  __syncthreads();
  // ---- Phase 1 (L = chol(D)) step K and phase 2 (X = L^{-1}) step K-1 run together in
  // iteration K: the phase-2 products of step K-1 beside the warp Cholesky of block K (PT
  // still holds L(., K-1) transposed), and block row K of X beside the trailing update.
  int K = 0;
  for (; K < NBK; K++) {
    const int k0 = K * DG_B, kb = min(DG_B, LN - k0), nI = NBK - 1 - K;
    float* Tkk = blk(K, K);
    if (warp == 0) {
      ds_chol32(Tkk, kb, col0 + k0, colb, dinv, &s_fail, status, lane);
    } else if (K > 0) {  // phase 2, step K-1: block (K+ii, J) -= L(K+ii, K-1) X(K-1, J), J < K-1;
                         // block (K+ii, K-1) := -L(K+ii, K-1) X_{K-1}
      for (int it = warp - 1; it < (NBK - K) * K; it += DG_WARPS - 1) {
        const int ii = it / K, J = it - ii * K;
        float acc[4][8] = {};
        ds_mm32(acc, PT + ii * DG_B, DS_PTLD, blk(K - 1, J), DS_P, r0, c0);
        ds_put(blk(K + ii, J), acc, r0, c0, J < K - 1 ? 0 : 1);
      }
    }
    __syncthreads();
    if (s_fail) return;  // D holds L left of block K (written below), the rest as it was
    if (t < nI * DG_B) {  // row t below: B := B L_KK^{-T}, into the tile, PT and D
      const int i = (K + 1) * DG_B + t;
      float* Trow = blk(K + 1 + (t >> 5), K) + (t & 31) * DS_P;
      float row[DG_B];
#pragma unroll
      for (int c4 = 0; c4 < DG_B / 4; c4++) {
        const float4 q = reinterpret_cast<const float4*>(Trow)[c4];
        row[4 * c4 + 0] = q.x;
        row[4 * c4 + 1] = q.y;
        row[4 * c4 + 2] = q.z;
        row[4 * c4 + 3] = q.w;
      }
#pragma unroll
      for (int c = 0; c < DG_B; c++) {
        float v = row[c];
#pragma unroll
        for (int q = 0; q < c; q++) v = fmaf(-row[q], Tkk[c * DS_P + q], v);
        row[c] = v * dinv[c];
      }
#pragma unroll
      for (int c4 = 0; c4 < DG_B / 4; c4++)
        reinterpret_cast<float4*>(Trow)[c4] =
            make_float4(row[4 * c4 + 0], row[4 * c4 + 1], row[4 * c4 + 2], row[4 * c4 + 3]);
#pragma unroll
      for (int c = 0; c < DG_B; c++) PT[c * DS_PTLD + t] = row[c];
      if (i < LN) {  // a block column with rows below is full width
#pragma unroll
        for (int c = 0; c < DG_B; c++) D[i + (i64)(k0 + c) * ldd] = row[c];
      }
    } else if (warp == DG_WARPS - 1) {  // X_KK by columns: lane c solves L_KK x = e_c
      float x[DG_B];
#pragma unroll
      for (int r = 0; r < DG_B; r++) {
        float v = (r == lane) ? 1.f : 0.f;
#pragma unroll
        for (int q = 0; q < r; q++) v = fmaf(-Tkk[r * DS_P + q], x[q], v);
        x[r] = v * dinv[r];
      }
      float* Xk = XD + K * DS_BLK;
#pragma unroll
      for (int r = 0; r < DG_B; r++) Xk[lane * DS_P + r] = x[r];
    } else if (warp == DG_WARPS - 2) {  // L_KK into D, lanes down the rows
      for (int c = 0; c < kb; c++)
        if (lane >= c && lane < kb) D[(k0 + lane) + (i64)(k0 + c) * ldd] = Tkk[lane * DS_P + c];
    }
    __syncthreads();
    // trailing lower block triangle: block (K+1+ii, K+1+jj) -= L(., K) L(., K)^T; then phase
    // 2, step K: X(K, J) = X_KK B(K, J) for J < K (B(K, J) is final), and X(K, K) = X_KK
    const int ntr = nI * (nI + 1) / 2;
    for (int it = warp; it <= ntr + K; it += DG_WARPS) {
      if (it < ntr) {
        int ii, jj;
        ds_block_ij(it, ii, jj);
        float acc[4][8] = {};
        ds_mm32(acc, PT + ii * DG_B, DS_PTLD, PT + jj * DG_B, DS_PTLD, r0, c0);
        ds_put(blk(K + 1 + ii, K + 1 + jj), acc, r0, c0, 0);
      } else {
        const float* Xk = XD + K * DS_BLK;
        const int J = it - ntr;
        if (J < K) {
          float* Bkj = blk(K, J);
          float acc[4][8] = {};
          ds_mm32(acc, Xk, DS_P, Bkj, DS_P, r0, c0);
          __syncwarp();
          ds_put(Bkj, acc, r0, c0, 2);
        } else {
#pragma unroll 4
          for (int c = 0; c < DG_B; c++) Tkk[lane * DS_P + c] = (c <= lane) ? Xk[c * DS_P + lane] : 0.f;
        }
      }
    }
    __syncthreads();
  }
  // Dinv = X^T (zeros below its diagonal), X row-major as BF16 planes or in FP32
  for (int i = warp; i < LN; i += DG_WARPS)
    for (int j = lane; j < LN; j += 32) {
      const float x = (j <= i) ? blk(i >> 5, j >> 5)[(i & 31) * DS_P + (j & 31)] : 0.f;
      Dinv[j + (i64)i * lde] = x;
      if (Xh) dg_split_store(Xh, Xl, (i64)i * LN + j, x);
      else Xr[(i64)i * LN + j] = x;
    }
}

// FP32 column panel (m x K, ld ldx) -> copy with ld ldy.
__global__ void k_copy_f32(const float* __restrict__ X, i64 ldx, float* __restrict__ Y, i64 ldy, int m, int K) {
  const i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  for (int k = blockIdx.y; k < K; k += gridDim.y) Y[r + k * ldy] = X[r + k * ldx];
}

// FP64 column panel (m x K, ld ldx) -> FP32 copy (ld ldy).
__global__ void k_to_f32(const double* __restrict__ X, i64 ldx, float* __restrict__ Y, i64 ldy, int m, int K) {
  const i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  for (int k = blockIdx.y; k < K; k += gridDim.y) Y[r + k * ldy] = ooc_f64_to_f32(X[r + k * ldx]);
}

// ---------------------------------------------------------------------------------
// Small-right-hand-side products (r <= 16 columns), accumulated in TC:
//   NN:  C[m x r] = beta C + alpha A[m x k] B[k x r]        thread per row
//   TN:  C[m x r] = beta C + alpha A[k x m]^T B[k x r]      warp per row
// (beta is 0 or 1).  For NN the long dimension k can be split across blockIdx.y into a
// partial buffer P (nslice x m x r) that k_reduce_slices sums in slice order, so results
// never depend on scheduling.
// ---------------------------------------------------------------------------------
constexpr int RMAX = 16;
constexpr int NN_KCHUNK = 256;

// Optional copy done by the first CTA of a small product: dst(0:n, 0:r) := src (the
// block a triangular-solve step has just finished, moved into place without a launch).
template <typename TC>
struct CopyOut {
  const TC* src = nullptr;
  i64 lds = 0;
  TC* dst = nullptr;
  i64 ldd = 0;
  int n = 0;
};

template <typename TA, typename TC, int R>
__global__ void __launch_bounds__(256) k_gemm_nn_small(const TA* __restrict__ A, i64 lda, const TC* __restrict__ B,
                                                       i64 ldb, TC* __restrict__ C, i64 ldc, int m, int k, int r,
                                                       int kslice, TC* __restrict__ P, TC alpha, TC beta,
                                                       CopyOut<TC> co) {
  // CTA: 32 rows x 8 warps; warp w sums its eighth of the CTA's k slice for the 32 rows
  // (lane = row, so each load is 32 consecutive rows of one column); the eight partial
  // sums are then added in warp order.
  __shared__ TC Bs[NN_KCHUNK * R];  // also the 8 x 32 x R partial sums at the end
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const i64 row = (i64)blockIdx.x * 32 + lane;
  const int k0 = blockIdx.y * kslice;
  const int k1 = min(k, k0 + kslice);
  if (co.n > 0 && blockIdx.x == 0 && blockIdx.y == 0)
    for (int idx = threadIdx.x; idx < co.n * r; idx += blockDim.x) {
      const int q = idx / co.n, i = idx % co.n;
      co.dst[i + (i64)q * co.ldd] = co.src[i + (i64)q * co.lds];
    }
  TC acc[R];
#pragma unroll
  for (int q = 0; q < R; q++) acc[q] = 0;
  const TA* Arow = A + (row < m ? row : 0);
  for (int kc = k0; kc < k1; kc += NN_KCHUNK) {
    const int kn = min(NN_KCHUNK, k1 - kc);
    __syncthreads();
    for (int idx = threadIdx.x; idx < kn * R; idx += blockDim.x) {
      const int q = idx / kn, kk = idx % kn;
      Bs[kk * R + q] = (q < r) ? B[(kc + kk) + (i64)q * ldb] : TC(0);
    }
    __syncthreads();
    const int kw = (kn + 7) / 8;
    const int ka = warp * kw, kb = min(kn, ka + kw);
    if (row < m) {
      int kk = ka;
      for (; kk + 8 <= kb; kk += 8) {
        TC a[8];
#pragma unroll
        for (int u = 0; u < 8; u++) a[u] = (TC)Arow[(i64)(kc + kk + u) * lda];
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
          for (int q = 0; q < R; q++) acc[q] = fma(a[u], Bs[(kk + u) * R + q], acc[q]);
      }
      for (; kk < kb; kk++) {
        const TC a = (TC)Arow[(i64)(kc + kk) * lda];
#pragma unroll
        for (int q = 0; q < R; q++) acc[q] = fma(a, Bs[kk * R + q], acc[q]);
      }
    }
  }
  static_assert(NN_KCHUNK == 8 * 32, "partial sums reuse the B chunk buffer");
  __syncthreads();
#pragma unroll
  for (int q = 0; q < R; q++) Bs[(warp * 32 + lane) * R + q] = acc[q];
  __syncthreads();
  if (warp != 0 || row >= m) return;
#pragma unroll
  for (int q = 0; q < R; q++) {
    TC v = Bs[lane * R + q];
#pragma unroll
    for (int w = 1; w < 8; w++) v += Bs[(w * 32 + lane) * R + q];
    acc[q] = v;
  }
  if (P) {
    TC* Pz = P + (i64)blockIdx.y * m * r;
#pragma unroll
    for (int q = 0; q < R; q++)
      if (q < r) Pz[row + (i64)q * m] = acc[q];
  } else {
#pragma unroll
    for (int q = 0; q < R; q++) {
      if (q >= r) break;
      TC* c = C + row + (i64)q * ldc;
      *c = (beta != TC(0)) ? fma(alpha, acc[q], *c) : alpha * acc[q];
    }
  }
}

template <typename TC>
__global__ void k_reduce_slices(const TC* __restrict__ P, int nslice, TC* __restrict__ C, i64 ldc, int m, int r,
                                TC alpha, TC beta) {
  const i64 row = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= m) return;
  for (int q = 0; q < r; q++) {
    TC sum = 0;
    for (int z = 0; z < nslice; z++) sum += P[(i64)z * m * r + row + (i64)q * m];
    TC* c = C + row + (i64)q * ldc;
    *c = (beta != TC(0)) ? fma(alpha, sum, *c) : alpha * sum;
  }
}

template <typename TA, typename TC, int R>
__global__ void __launch_bounds__(256) k_gemm_tn_small(const TA* __restrict__ A, i64 lda, const TC* __restrict__ B,
                                                       i64 ldb, TC* __restrict__ C, i64 ldc, int m, int k, int r,
                                                       TC alpha, TC beta, CopyOut<TC> co) {
  __shared__ TC Bs[NN_KCHUNK * R];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (co.n > 0 && blockIdx.x == 0)
    for (int idx = threadIdx.x; idx < co.n * r; idx += blockDim.x) {
      const int q = idx / co.n, i = idx % co.n;
      co.dst[i + (i64)q * co.ldd] = co.src[i + (i64)q * co.lds];
    }
  const i64 row = (i64)blockIdx.x * (blockDim.x / 32) + warp;
  TC acc[R];
#pragma unroll
  for (int q = 0; q < R; q++) acc[q] = 0;
  const TA* Acol = A + (row < m ? row : 0) * lda;
  for (int kc = 0; kc < k; kc += NN_KCHUNK) {
    const int kn = min(NN_KCHUNK, k - kc);
    __syncthreads();
    for (int idx = threadIdx.x; idx < kn * R; idx += blockDim.x) {
      const int q = idx / kn, kk = idx % kn;
      Bs[q * NN_KCHUNK + kk] = (q < r) ? B[(kc + kk) + (i64)q * ldb] : TC(0);  // q-major: lanes read
    }                                                                         // consecutive kk
    __syncthreads();
    if (row < m) {
      int kk = lane;  // eight loads in flight, then four, then one (k ascending either way)
      for (; kk + 224 < kn; kk += 256) {
        TC a[8];
#pragma unroll
        for (int u = 0; u < 8; u++) a[u] = (TC)Acol[kc + kk + 32 * u];
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
          for (int q = 0; q < R; q++) acc[q] = fma(a[u], Bs[q * NN_KCHUNK + kk + 32 * u], acc[q]);
      }
      for (; kk + 96 < kn; kk += 128) {
        TC a[4];
#pragma unroll
        for (int u = 0; u < 4; u++) a[u] = (TC)Acol[kc + kk + 32 * u];
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int q = 0; q < R; q++) acc[q] = fma(a[u], Bs[q * NN_KCHUNK + kk + 32 * u], acc[q]);
      }
      for (; kk < kn; kk += 32) {
        const TC a = (TC)Acol[kc + kk];
#pragma unroll
        for (int q = 0; q < R; q++) acc[q] = fma(a, Bs[q * NN_KCHUNK + kk], acc[q]);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < R; q++) {
    TC v = acc[q];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    acc[q] = v;
  }
  if (row >= m || lane != 0) return;
#pragma unroll
  for (int q = 0; q < R; q++) {
    if (q >= r) break;
    TC* c = C + row + (i64)q * ldc;
    *c = (beta != TC(0)) ? fma(alpha, acc[q], *c) : alpha * acc[q];
  }
}

// One right-hand side through a diagonal block's inverse: x = U^T b (TRANS) or x = U b,
// U = Dinv_J = L_JJ^{-T} (LN x LN, ld ldu, upper triangular), so output i takes only
// k <= i (TRANS) or k >= i.  CTA = 32 outputs x 16 warps, warp w takes k in [32w, 32w+32):
// all of a thread's loads are issued before its first FMA (one round trip instead of a
// walk), the 16 warp sums added in warp order.  TRANS: lane = k, 32 outputs per lane, then
// a transposing butterfly leaves lane l with its warp's sum for output l; otherwise lane =
// output row, b(k) passed along the warp by shuffles.  LN <= 512.
constexpr int DMV_WARPS = 16;
// a[0..S) := the lane's kept half plus the partner's passed half (partner = lane ^ S)
template <typename T, int S>
__device__ __forceinline__ void dmv_fold(T (&a)[32], int lane) {
  const bool hi = (lane & S) != 0;
#pragma unroll
  for (int j = 0; j < S; j++) {
    const T send = hi ? a[j] : a[j + S];
    const T keep = hi ? a[j + S] : a[j];
    a[j] = keep + __shfl_xor_sync(0xffffffffu, send, S);
  }
}

template <typename T, bool TRANS>
__global__ void __launch_bounds__(DMV_WARPS * 32) k_dinv_mv(const T* __restrict__ U, i64 ldu, int LN,
                                                           const T* __restrict__ b, T* __restrict__ x) {
  __shared__ T part[DMV_WARPS][33];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i0 = blockIdx.x * 32, k0 = warp * 32;
  const int kl = k0 + lane;
  const T bk = (kl < LN) ? b[kl] : T(0);
  T acc;
  if (TRANS) {
    T a[32];
#pragma unroll
    for (int j = 0; j < 32; j++) {
      const int i = i0 + j;
      a[j] = (kl < LN && i < LN && kl <= i) ? U[kl + (i64)i * ldu] : T(0);
    }
#pragma unroll
    for (int j = 0; j < 32; j++) a[j] *= bk;
    dmv_fold<T, 16>(a, lane);  // keep half, pass half: lane l ends with index l
    dmv_fold<T, 8>(a, lane);
    dmv_fold<T, 4>(a, lane);
    dmv_fold<T, 2>(a, lane);
    dmv_fold<T, 1>(a, lane);
    acc = a[0];
  } else {
    const int i = i0 + lane;
    T v[32];
#pragma unroll
    for (int u = 0; u < 32; u++) {
      const int k = k0 + u;
      v[u] = (i < LN && k < LN && k >= i) ? U[i + (i64)k * ldu] : T(0);
    }
    acc = T(0);
#pragma unroll
    for (int u = 0; u < 32; u++) acc = fma(v[u], __shfl_sync(0xffffffffu, bk, u), acc);
  }
  part[warp][lane] = acc;
  __syncthreads();
  if (warp == 0 && i0 + lane < LN) {
    T sum = part[0][lane];
#pragma unroll
    for (int w = 1; w < DMV_WARPS; w++) sum += part[w][lane];
    x[i0 + lane] = sum;
  }
}

// D (n x n, ld ldd) -> E = D^T (ld lde).
__global__ void k_transpose(const double* __restrict__ D, i64 ldd, double* __restrict__ E, i64 lde, int n) {
  __shared__ double t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int r = bx + threadIdx.x, c = by + yy;
    t[yy][threadIdx.x] = (r < n && c < n) ? D[r + (i64)c * ldd] : 0.0;
  }
  __syncthreads();
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int r = by + threadIdx.x, c = bx + yy;  // E(r, c) = D(c, r)
    if (r < n && c < n) E[r + (i64)c * lde] = t[threadIdx.x][yy];
  }
}

// Identity into a (n x n, ld) block.
template <typename T>
__global__ void k_set_identity(T* D, i64 ld, int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int c = blockIdx.y; c < n; c += gridDim.y) D[r + (i64)c * ld] = (r == c) ? T(1) : T(0);
}

// Copy with conversion (column-major blocks).

// Lower triangle (columns [c0, c0 + w), rows >= column) between the FP64 input/output and the
// FP32 working matrix, converted on the integer pipe; `zero_upper` writes 0 above it.
__device__ __forceinline__ float to_f32(double x) { return ooc_f64_to_f32(x); }
__device__ __forceinline__ double to_f64(float x) { return ooc_f32_to_f64(x); }
template <typename TS, typename TD>
__global__ void k_lower_conv(const TS* __restrict__ S, i64 lds, TD* __restrict__ D, i64 ldd, i64 n, i64 c0, int w,
                             int zero_upper) {
  const i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  constexpr int U = 4;  // columns per pass, their loads issued before the first store
  for (int cb = blockIdx.y; cb < w; cb += U * gridDim.y) {
    TS v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int cc = cb + u * gridDim.y;
      v[u] = (cc < w && r >= c0 + cc) ? S[r + (i64)cc * lds] : TS(0);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int cc = cb + u * gridDim.y;
      if (cc >= w) break;
      if (r >= c0 + cc) {
        if constexpr (sizeof(TD) == 4) D[r + (i64)cc * ldd] = to_f32(v[u]);
        else D[r + (i64)cc * ldd] = to_f64(v[u]);
      } else if (zero_upper) {
        D[r + (i64)cc * ldd] = TD(0);
      }
    }
  }
}
// The uniform test matrix's lower triangle, rounded to FP32 (the same values as rounding
// the FP64 generator's output).
__global__ void k_gen_uniform_f32_lower(float* __restrict__ D, i64 ldd, i64 n, uint64_t key, double alpha) {
  const i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (i64 c = blockIdx.y; c <= r && c < n; c += gridDim.y) D[r + c * ldd] = ooc_uniform_elem_f32(key, n, alpha, r, c);
}

// x += d (columns), and per-column max |.| of x, r and b for the backward error.
__global__ void k_axpy_cols(double* X, i64 ldx, const double* D, i64 ldd, int n, int r) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int q = 0; q < r; q++) X[i + q * ldx] += D[i + q * ldd];
}

__global__ void k_colmax_abs(const double* V, i64 ld, int n, int r, double* out /* r per CTA */) {
  __shared__ double sm[256];
  for (int q = 0; q < r; q++) {
    double mx = 0;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
      mx = fmax(mx, fabs(V[i + q * ld]));
    sm[threadIdx.x] = mx;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(i64)blockIdx.x * r + q] = sm[0];
    __syncthreads();
  }
}


// R(:, q) -= A(seed) X(:, q) over the columns [blockIdx.y * kslice, ...) of A, with A
// regenerated element by element (uniform generator) instead of read from memory.
// Partial sums per column slice go to P (nslice x m x r) for an ordered reduction.
// The uniform test matrix's off-diagonal elements are integer multiples of 2^-54
// (ooc_uniform_offdiag_int): the kernels below accumulate the integers and apply 2^-54 once
// per row (a power of two commutes with rounding), one conversion per element.
// P[slice](row, q) = sum over the slice's columns c of A(row, c) X(c, q), A regenerated.
template <int R>
__global__ void __launch_bounds__(256) k_resid_gen(uint64_t key, i64 n, double alpha, const double* __restrict__ X,
                                                   i64 ldx, int r, int kslice, double* __restrict__ P) {
  __shared__ double Xs[NN_KCHUNK * R];
  const i64 row = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  const int k0 = blockIdx.y * kslice;
  const int k1 = (int)min((i64)k0 + kslice, n);
  double acc[R];  // in units of 2^-54
#pragma unroll
  for (int q = 0; q < R; q++) acc[q] = 0;
  for (int kc = k0; kc < k1; kc += NN_KCHUNK) {
    const int kn = min(NN_KCHUNK, k1 - kc);
    __syncthreads();
    for (int idx = threadIdx.x; idx < kn * R; idx += blockDim.x) {
      const int q = idx / kn, kk = idx % kn;
      Xs[kk * R + q] = (q < r) ? X[(kc + kk) + (i64)q * ldx] : 0.0;
    }
    __syncthreads();
    if (row < n) {
      for (int kk = 0; kk < kn; kk++) {
        const i64 c = kc + kk;
        const double a = (c == row) ? 0.0 : (double)ooc_uniform_offdiag_int(key, n, row, c);
#pragma unroll
        for (int q = 0; q < R; q++) acc[q] = fma(a, Xs[kk * R + q], acc[q]);
      }
    }
  }
  if (row >= n) return;
  const bool has_diag = row >= k0 && row < k1;
  const double aii = has_diag ? ooc_uniform_elem(key, n, alpha, row, row) : 0.0;
  double* Pz = P + (i64)blockIdx.y * n * r;
  for (int q = 0; q < r; q++) {
    double v = acc[q] * 0x1.0p-54;
    if (has_diag) v = fma(aii, X[row + (i64)q * ldx], v);
    Pz[row + (i64)q * n] = v;
  }
}

// P[slice](row) = sum over the slice's columns of |A(row, c)|: integer sums of at most 512
// terms (< 2^62), each converted once.
__global__ void __launch_bounds__(256) k_rowsum_gen(uint64_t key, i64 n, double alpha, int kslice,
                                                    double* __restrict__ P) {
  const i64 row = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  const int k0 = blockIdx.y * kslice;
  const int k1 = (int)min((i64)k0 + kslice, n);
  double s = 0;
  for (int c0 = k0; c0 < k1; c0 += 512) {
    const int c1 = min(k1, c0 + 512);
    unsigned long long is = 0;
    for (int c = c0; c < c1; c++) {
      if (c == row) continue;
      const long long v = ooc_uniform_offdiag_int(key, n, row, c);
      is += (unsigned long long)(v < 0 ? -v : v);
    }
    s += (double)is;
  }
  s *= 0x1.0p-54;
  if (row >= k0 && row < k1) s += fabs(ooc_uniform_elem(key, n, alpha, row, row));
  P[(i64)blockIdx.y * n + row] = s;
}

__global__ void k_sum_slices_rows(const double* __restrict__ P, int nslice, i64 n, double* __restrict__ out) {
  const i64 row = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  double s = 0;
  for (int z = 0; z < nslice; z++) s += P[(i64)z * n + row];
  out[row] = s;
}

// B(i, q) = N(0,1) sample of stream `key`, element i + q*n.
__global__ void k_gen_normal(double* B, i64 ldb, i64 n, int r, uint64_t key) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int q = 0; q < r; q++) B[i + q * ldb] = ooc_normal_elem(key, (uint64_t)(i + q * n));
}

}  // namespace

// =================================================================================
// Host-side pieces
// =================================================================================

int launch_syrk_bf16x3(const double* X, i64 ldx, double* C, i64 ldc, int m, int K, const int* status,
                       cudaStream_t s, void* work, size_t work_bytes, int bj_lo, int bj_hi, int do_split,
                       int reserve_sms);
int launch_syrk_bf16x3_f32(const float* X, i64 ldx, float* C, i64 ldc, int m, int K, const int* status,
                           cudaStream_t s, void* work, size_t work_bytes, int bj_lo, int bj_hi, int do_split,
                           int reserve_sms);
size_t bf16x3_work_bytes(int m, int K);
int launch_split_bf16_f32(const float* X, i64 ldx, int m, int K, void* work, size_t work_bytes, cudaStream_t s);
int launch_trsm_bf16x3_f32(void* uwork, size_t ubytes, const void* xhi, const void* xlo, float* P, i64 ldp, int m,
                           int K, void* swork, size_t sbytes, const int* status, cudaStream_t s);
int launch_trsm_bf16x3_f32_to(void* uwork, size_t ubytes, const void* xhi, const void* xlo, float* P, i64 ldp, int m,
                              int K, void* ohi, void* olo, i64 ldo, const int* status, cudaStream_t s);
int launch_syrk_planes_f32(const void* hi, const void* lo, i64 ldk, int m, int K, float* C, i64 ldc,
                           const int* status, cudaStream_t s, unsigned long long* tickets, int bj_lo, int bj_hi,
                           int reserve_sms);

namespace {

// Device scratch that grows on demand.  With a pool (a factor object's buffers), the
// buffer comes from the handle's cache and returns to it on destruction; a buffer replaced
// by a larger one is freed at once (work queued on it may still be pending).
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevPool* pool = nullptr;
  ~DevBuf() {
    if (!p) return;
    if (pool) pool->release(p);
    else cudaFree(p);
  }
  int ensure(size_t b) {
    if (bytes >= b) return OOC_OK;
    if (p) {
      if (pool) pool->drop(p);
      else cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
    if (pool) {
      p = pool->alloc(b);
    } else if (cudaMalloc(&p, b) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    if (!p) return OOC_ERR_NOMEM;
    bytes = b;
    return OOC_OK;
  }
  // gives the buffer back (to the pool, or freed) once the work queued on it is done
  void release() {
    if (!p) return;
    if (pool) pool->release(p);
    else cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

// C (lower, m x m) -= X X^T restricted to the 128-wide block columns [bj_lo, bj_hi) (bj_hi < 0
// = all) in reduced precision.  `prepare` converts / splits X first; a second call on the
// same X (another block-column range) may skip it.
// reserve_sms: SMs the persistent tensor-core kernel leaves free for concurrent work on
// another stream (the next panel's diagonal factor).
int syrk_lowprec(int prec, const double* X, i64 ldx, double* C, i64 ldc, int m, int K, const int* status,
                 cudaStream_t s, DevBuf& work, int bj_lo = 0, int bj_hi = -1, int prepare = 1, int reserve_sms = 0) {
  if (m <= 0 || K <= 0) return OOC_OK;
  if (prec == OOC_PREC_FP32) {
    const i64 ldy = ((i64)m + 3) / 4 * 4;
    if (prepare) {
      int rc = work.ensure((size_t)ldy * K * sizeof(float));
      if (rc) return rc;
    }
    float* Y = (float*)work.p;
    if (prepare)
      k_to_f32<<<dim3((unsigned)((m + 255) / 256), (unsigned)std::min(K, 1024)), 256, 0, s>>>(X, ldx, Y, ldy, m, K);
    const i64 T = ((i64)m + FB - 1) / FB;
    const i64 hi = std::min<i64>(bj_hi < 0 ? T : bj_hi, T);
    if (bj_lo >= hi) return OOC_OK;
    const i64 nblk = ooc_lower_blocks_before(hi, T) - ooc_lower_blocks_before(bj_lo, T);
    if (nblk > 0x7fffffff) return OOC_ERR_INTERNAL;
    k_syrk_f32<double><<<(unsigned)nblk, FTHR, 0, s>>>(Y, ldy, C, ldc, m, K, (int)T, bj_lo, status);
    OOC_CUDA_TRY(cudaGetLastError());
    return OOC_OK;
  }
  if (prec == OOC_PREC_BF16X3) {
    if (prepare) {
      int rc = work.ensure(bf16x3_work_bytes(m, K));
      if (rc) return rc;
    }
    return launch_syrk_bf16x3(X, ldx, C, ldc, m, K, status, s, work.p, work.bytes, bj_lo, bj_hi, prepare,
                              reserve_sms);
  }
  return OOC_ERR_UNSUPPORTED;
}

// The same for the FP32 working matrix of a reduced-precision factor: C (FP32) -= X X^T
// with X the FP32 column panel (no conversions).
int syrk_f32(int prec, const float* X, i64 ldx, float* C, i64 ldc, int m, int K, const int* status, cudaStream_t s,
             DevBuf& work, int bj_lo = 0, int bj_hi = -1, int prepare = 1, int reserve_sms = 0) {
  if (m <= 0 || K <= 0) return OOC_OK;
  if (prec == OOC_PREC_FP32) {
    const i64 T = ((i64)m + FB - 1) / FB;
    const i64 hi = std::min<i64>(bj_hi < 0 ? T : bj_hi, T);
    if (bj_lo >= hi) return OOC_OK;
    const i64 nblk = ooc_lower_blocks_before(hi, T) - ooc_lower_blocks_before(bj_lo, T);
    if (nblk > 0x7fffffff) return OOC_ERR_INTERNAL;
    // k_syrk_f32 stages X with 16-byte copies: a panel whose base or leading dimension is
    // not 16-byte compatible is first copied to an aligned buffer (once per panel).
    const float* Xs = X;
    i64 lds = ldx;
    if ((reinterpret_cast<uintptr_t>(X) % 16) != 0 || (ldx % 4) != 0) {
      lds = ((i64)m + 3) / 4 * 4;
      if (prepare) {
        int rc = work.ensure((size_t)lds * K * sizeof(float));
        if (rc) return rc;
        k_copy_f32<<<dim3((unsigned)((m + 255) / 256), (unsigned)std::min(K, 1024)), 256, 0, s>>>(X, ldx, (float*)work.p,
                                                                                              lds, m, K);
      }
      Xs = (const float*)work.p;
    }
    k_syrk_f32<float><<<(unsigned)nblk, FTHR, 0, s>>>(Xs, lds, C, ldc, m, K, (int)T, bj_lo, status);
    OOC_CUDA_TRY(cudaGetLastError());
    return OOC_OK;
  }
  if (prec == OOC_PREC_BF16X3) {
    if (prepare) {
      int rc = work.ensure(bf16x3_work_bytes(m, K));
      if (rc) return rc;
    }
    return launch_syrk_bf16x3_f32(X, ldx, C, ldc, m, K, status, s, work.p, work.bytes, bj_lo, bj_hi, prepare,
                                  reserve_sms);
  }
  return OOC_ERR_UNSUPPORTED;
}

// Instantiates a small-RHS kernel for the smallest of 1, 4, 16 columns covering r.
#define NN_DISPATCH(r, launch)          \
  do {                                  \
    if ((r) <= 1) {                     \
      constexpr int RR = 1;             \
      launch;                           \
    } else if ((r) <= 4) {              \
      constexpr int RR = 4;             \
      launch;                           \
    } else {                            \
      constexpr int RR = 16;            \
      launch;                           \
    }                                   \
  } while (0)

template <typename TA, typename TC>
int gemm_nn_small(const TA* A, i64 lda, const TC* B, i64 ldb, TC* C, i64 ldc, int m, int k, int r, TC alpha, TC beta,
                  cudaStream_t s, DevBuf* part, CopyOut<TC> co = CopyOut<TC>()) {
  if (m <= 0 || r <= 0) return OOC_OK;
  if (r > RMAX) return OOC_ERR_UNSUPPORTED;
  if (k <= 0) {
    if (beta == TC(0)) {
      for (int q = 0; q < r; q++) OOC_CUDA_TRY(cudaMemsetAsync(C + (i64)q * ldc, 0, sizeof(TC) * m, s));
    }
    return OOC_OK;
  }
  const int rows_blocks = (m + 31) / 32;
  // Long k: slices of at most 2048 (each warp then walks <= 256 columns) in grid.y, their
  // partial sums added in slice order by k_reduce_slices.
  int nslice = part ? (k + 2047) / 2048 : 1;
  if (nslice > 1) {
    const int kslice = ((k + nslice - 1) / nslice + NN_KCHUNK - 1) / NN_KCHUNK * NN_KCHUNK;
    nslice = (k + kslice - 1) / kslice;
    int rc = part->ensure((size_t)nslice * m * r * sizeof(TC));
    if (rc) return rc;
    NN_DISPATCH(r, (k_gemm_nn_small<TA, TC, RR><<<dim3(rows_blocks, nslice), 256, 0, s>>>(
                       A, lda, B, ldb, C, ldc, m, k, r, kslice, (TC*)part->p, alpha, beta, co)));
    k_reduce_slices<TC><<<(m + 255) / 256, 256, 0, s>>>((const TC*)part->p, nslice, C, ldc, m, r, alpha, beta);
  } else {
    NN_DISPATCH(r, (k_gemm_nn_small<TA, TC, RR><<<dim3(rows_blocks, 1), 256, 0, s>>>(
                       A, lda, B, ldb, C, ldc, m, k, r, k, nullptr, alpha, beta, co)));
  }
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

template <typename TA, typename TC>
int gemm_tn_small(const TA* A, i64 lda, const TC* B, i64 ldb, TC* C, i64 ldc, int m, int k, int r, TC alpha, TC beta,
                  cudaStream_t s, CopyOut<TC> co = CopyOut<TC>()) {
  if (m <= 0 || r <= 0) return OOC_OK;
  if (r > RMAX) return OOC_ERR_UNSUPPORTED;
  NN_DISPATCH(r, (k_gemm_tn_small<TA, TC, RR><<<(m + 7) / 8, 256, 0, s>>>(A, lda, B, ldb, C, ldc, m, k, r, alpha,
                                                                        beta, co)));
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

// ---- symmetric products reading only the lower triangle of A (FP64): the refinement's
// residual Y = A X = tril(A) X + strict(A)^T X, and with ABS the row sums of |A| for the
// infinity norm (X null, r = 1): |a| rounded to FP32 on the integer pipe and summed in FP32
// over runs of at most 32 elements, the runs added in FP64 (relative error < 1e-5, which the
// backward error's denominator does not notice; an FP64 operation per element would cost
// ~2 ms per 10^9 elements on this part).  Nothing above the diagonal is loaded, so the
// strict upper triangle may hold anything.
//   k_symv_rows: CTA = 32 rows x a column slice (j <= i), warp w sums its eighth of each
//                chunk; one partial sum per slice (as k_gemm_nn_small).
//   k_symv_cols: one warp per column j, the dot products of A(j+1:n, j) with the rows of X
//                (lane order, then a fixed shuffle tree).
// The partial sums are added in slice order by k_symv_combine: the result is deterministic.
template <bool ABS>
__device__ __forceinline__ double symv_elem(double a) {
  return ABS ? fabs(a) : a;
}

template <bool ABS, int R>
__global__ void __launch_bounds__(256) k_symv_rows(const double* __restrict__ A, i64 lda,
                                                   const double* __restrict__ X, i64 ldx, int n, int r, int kslice,
                                                   double* __restrict__ P) {
  __shared__ double Xs[R * NN_KCHUNK];  // q-major chunk of X; also the 8 x 32 x R partial sums
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i0 = blockIdx.x * 32;
  const int row = i0 + lane;
  const int k0 = blockIdx.y * kslice;
  const int k1 = min(min(n, k0 + kslice), i0 + 32);  // columns j <= the block's last row
  double acc[R];
#pragma unroll
  for (int q = 0; q < R; q++) acc[q] = 0;
  const double* Arow = A + (row < n ? row : 0);
  for (int kc = k0; kc < k1; kc += NN_KCHUNK) {
    const int kn = min(NN_KCHUNK, k1 - kc);
    __syncthreads();
    for (int idx = threadIdx.x; idx < kn * R; idx += blockDim.x) {
      const int q = idx / kn, kk = idx % kn;
      Xs[q * NN_KCHUNK + kk] = (q < r) ? (X ? X[(kc + kk) + (i64)q * ldx] : 1.0) : 0.0;
    }
    __syncthreads();
    const int kw = (kn + 7) / 8;
    const int ka = warp * kw, kb = min(kn, ka + kw);
    if (ABS && row < n) {  // |a| rounded to FP32 (integer pipe), FP32 run of <= 32 per chunk
      float f = 0.f;
      int kk = ka;
      for (; kk + 8 <= kb; kk += 8) {
        double a[8];
#pragma unroll
        for (int u = 0; u < 8; u++) a[u] = (kc + kk + u <= row) ? Arow[(i64)(kc + kk + u) * lda] : 0.0;
#pragma unroll
        for (int u = 0; u < 8; u++) f += fabsf(ooc_f64_to_f32(a[u]));
      }
      for (; kk < kb; kk++)
        if (kc + kk <= row) f += fabsf(ooc_f64_to_f32(Arow[(i64)(kc + kk) * lda]));
      acc[0] += ooc_f32_to_f64(f);
    } else if (row < n) {
      int kk = ka;
      for (; kk + 8 <= kb; kk += 8) {
        double a[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
          const int j = kc + kk + u;
          a[u] = (j <= row) ? symv_elem<ABS>(Arow[(i64)j * lda]) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
          for (int q = 0; q < R; q++) acc[q] = fma(a[u], Xs[q * NN_KCHUNK + kk + u], acc[q]);
      }
      for (; kk < kb; kk++) {
        const int j = kc + kk;
        const double a = (j <= row) ? symv_elem<ABS>(Arow[(i64)j * lda]) : 0.0;
#pragma unroll
        for (int q = 0; q < R; q++) acc[q] = fma(a, Xs[q * NN_KCHUNK + kk], acc[q]);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < R; q++) Xs[(warp * 32 + lane) * R + q] = acc[q];
  __syncthreads();
  if (warp != 0 || row >= n) return;
  double* Pz = P + (i64)blockIdx.y * n * r;
#pragma unroll
  for (int q = 0; q < R; q++) {
    if (q >= r) break;
    double v = Xs[lane * R + q];
#pragma unroll
    for (int w = 1; w < 8; w++) v += Xs[(w * 32 + lane) * R + q];
    Pz[row + (i64)q * n] = v;
  }
}

template <bool ABS, int R>
__global__ void __launch_bounds__(256) k_symv_cols(const double* __restrict__ A, i64 lda,
                                                   const double* __restrict__ X, i64 ldx, int n, int r,
                                                   double* __restrict__ Q) {
  __shared__ double Xs[R * NN_KCHUNK];  // q-major chunk of X rows
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int jmin = blockIdx.x * 8;
  const int j = jmin + warp;
  double acc[R];
#pragma unroll
  for (int q = 0; q < R; q++) acc[q] = 0;
  const double* Acol = A + (i64)(j < n ? j : 0) * lda;
  for (int ic = jmin + 1; ic < n; ic += NN_KCHUNK) {
    const int kn = min(NN_KCHUNK, n - ic);
    __syncthreads();
    for (int idx = threadIdx.x; idx < kn * R; idx += blockDim.x) {
      const int q = idx / kn, ii = idx % kn;
      Xs[q * NN_KCHUNK + ii] = (q < r) ? (X ? X[(ic + ii) + (i64)q * ldx] : 1.0) : 0.0;
    }
    __syncthreads();
    if (ABS && j < n) {  // |a| rounded to FP32, FP32 run of <= 8 per chunk
      float f = 0.f;
      int ii = lane;
      for (; ii + 96 < kn; ii += 128) {
        double a[4];
#pragma unroll
        for (int u = 0; u < 4; u++) a[u] = (ic + ii + 32 * u > j) ? Acol[ic + ii + 32 * u] : 0.0;
#pragma unroll
        for (int u = 0; u < 4; u++) f += fabsf(ooc_f64_to_f32(a[u]));
      }
      for (; ii < kn; ii += 32)
        if (ic + ii > j) f += fabsf(ooc_f64_to_f32(Acol[ic + ii]));
      acc[0] += ooc_f32_to_f64(f);
    } else if (j < n) {
      int ii = lane;
      for (; ii + 96 < kn; ii += 128) {
        double a[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int i = ic + ii + 32 * u;
          a[u] = (i > j) ? symv_elem<ABS>(Acol[i]) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int q = 0; q < R; q++) acc[q] = fma(a[u], Xs[q * NN_KCHUNK + ii + 32 * u], acc[q]);
      }
      for (; ii < kn; ii += 32) {
        const int i = ic + ii;
        const double a = (i > j) ? symv_elem<ABS>(Acol[i]) : 0.0;
#pragma unroll
        for (int q = 0; q < R; q++) acc[q] = fma(a, Xs[q * NN_KCHUNK + ii], acc[q]);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < R; q++) {
    double v = acc[q];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    acc[q] = v;
  }
  if (j >= n || lane != 0) return;
#pragma unroll
  for (int q = 0; q < R; q++)
    if (q < r) Q[j + (i64)q * n] = acc[q];
}

// C = beta C + alpha (sum of the nslice partials in order + Q)
__global__ void k_symv_combine(const double* __restrict__ P, int nslice, const double* __restrict__ Q, double* C,
                               i64 ldc, int n, int r, double alpha, double beta) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int q = 0; q < r; q++) {
    double v = 0;
    for (int z = 0; z < nslice; z++) v += P[(i64)z * n * r + i + (i64)q * n];
    v += Q[i + (i64)q * n];
    double* c = C + i + (i64)q * ldc;
    *c = (beta != 0.0) ? fma(alpha, v, beta * *c) : alpha * v;
  }
}

// C (n x r, ld ldc) = beta C + alpha A X with A symmetric, given by its lower triangle
// (ld lda).  abs: |A| instead of A; X null: a column of ones (r = 1).
int symv_lower(bool abs, const double* A, i64 lda, const double* X, i64 ldx, double* C, i64 ldc, int n, int r,
               double alpha, double beta, cudaStream_t s, DevBuf& part) {
  if (n <= 0 || r <= 0) return OOC_OK;
  if (r > RMAX || (!X && r != 1)) return OOC_ERR_UNSUPPORTED;
  int nslice = (n + 2047) / 2048;
  const int kslice = ((n + nslice - 1) / nslice + NN_KCHUNK - 1) / NN_KCHUNK * NN_KCHUNK;
  nslice = (n + kslice - 1) / kslice;
  int rc = part.ensure((size_t)(nslice + 1) * n * r * sizeof(double));
  if (rc) return rc;
  double* P = (double*)part.p;
  double* Q = P + (size_t)nslice * n * r;
  const dim3 grow((unsigned)((n + 31) / 32), (unsigned)nslice);
  const unsigned gcol = (unsigned)((n + 7) / 8);
  if (abs) {
    k_symv_rows<true, 1><<<grow, 256, 0, s>>>(A, lda, X, ldx, n, r, kslice, P);
    k_symv_cols<true, 1><<<gcol, 256, 0, s>>>(A, lda, X, ldx, n, r, Q);
  } else {
    NN_DISPATCH(r, (k_symv_rows<false, RR><<<grow, 256, 0, s>>>(A, lda, X, ldx, n, r, kslice, P)));
    NN_DISPATCH(r, (k_symv_cols<false, RR><<<gcol, 256, 0, s>>>(A, lda, X, ldx, n, r, Q)));
  }
  k_symv_combine<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, nslice, Q, C, ldc, n, r, alpha, beta);
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

// Panel schedule of a reduced-precision factor: nb-wide panels up to column tail0 (a
// multiple of nb), then nb2-wide panels (tail0 = n: uniform nb).  Panel p starts at J0,
// is LN wide, and its diagonal tile's inverse sits at Dinv + off with leading dimension ld
// (the panel's nominal width): the tiles are stored one after the other.
struct Panels {
  i64 n = 0, tail0 = 0;
  int nb = 0, nb2 = 0;
  int count() const {
    if (tail0 >= n) return (int)((n + nb - 1) / nb);
    return (int)(tail0 / nb + (n - tail0 + nb2 - 1) / nb2);
  }
  void get(int p, i64* J0, int* LN, i64* off, int* ld) const {
    const int hc = tail0 >= n ? count() : (int)(tail0 / nb);
    if (p < hc) {
      *J0 = (i64)p * nb;
      *LN = (int)std::min<i64>(nb, n - *J0);
      *off = (i64)p * nb * nb;
      *ld = nb;
    } else {
      const int t = p - hc;
      *J0 = tail0 + (i64)t * nb2;
      *LN = (int)std::min<i64>(nb2, n - *J0);
      *off = (i64)hc * nb * nb + (i64)t * nb2 * nb2;
      *ld = nb2;
    }
  }
};

// Solve L L^T X = B in place (B: n x r, ld ldb) using the inverses of the diagonal
// tiles.  Dinv_J holds L_JJ^{-T} (column-major, upper), i.e. the transpose of
// L_JJ^{-1}; tmp holds nb x r (nb = the widest panel).
// B := (L L^T)^{-1} B with the factor's L and kept diagonal inverses (r <= 16 columns):
// the dpotrs of the reference's VERIFY block (oocdag.cpp:439).  Two launches per block
// step: the product with the block's inverse into tmp, then the panel product, whose
// first CTA also moves tmp into place.
template <typename T>
int solve_with(const T* L, i64 ldl, const T* Dinv, const Panels& P, T* B, i64 ldb, int r, T* tmp, cudaStream_t s,
               DevBuf* part) {
  const i64 n = P.n;
  const int nt = P.nb;  // ld of tmp
  const int bb = P.count();
  int rc;
  // forward: L y = b
  for (int J = 0; J < bb; J++) {
    i64 J0, off;
    int LN, ld;
    P.get(J, &J0, &LN, &off, &ld);
    if (r == 1 && LN <= DMV_WARPS * 32) {  // Dinv_J^T b_J
      k_dinv_mv<T, true><<<(LN + 31) / 32, DMV_WARPS * 32, 0, s>>>(Dinv + off, ld, LN, B + J0, tmp);
      OOC_CUDA_TRY(cudaGetLastError());
    } else {
      rc = gemm_tn_small<T, T>(Dinv + off, ld, B + J0, ldb, tmp, nt, LN, LN, r, T(1), T(0), s);
      if (rc) return rc;
    }
    const i64 rows = n - J0 - LN;
    if (rows > 0) {
      rc = gemm_nn_small<T, T>(L + (J0 + LN) + J0 * ldl, ldl, tmp, nt, B + J0 + LN, ldb, (int)rows, LN, r, T(-1),
                               T(1), s, part, CopyOut<T>{tmp, nt, B + J0, ldb, LN});
      if (rc) return rc;
    } else {
      OOC_CUDA_TRY(cudaMemcpy2DAsync(B + J0, ldb * sizeof(T), tmp, nt * sizeof(T), LN * sizeof(T), r,
                                     cudaMemcpyDeviceToDevice, s));
    }
  }
  // backward: L^T x = y
  for (int J = bb - 1; J >= 0; J--) {
    i64 J0, off;
    int LN, ld;
    P.get(J, &J0, &LN, &off, &ld);
    if (r == 1 && LN <= DMV_WARPS * 32) {  // Dinv_J y_J
      k_dinv_mv<T, false><<<(LN + 31) / 32, DMV_WARPS * 32, 0, s>>>(Dinv + off, ld, LN, B + J0, tmp);
      OOC_CUDA_TRY(cudaGetLastError());
    } else {
      rc = gemm_nn_small<T, T>(Dinv + off, ld, B + J0, ldb, tmp, nt, LN, LN, r, T(1), T(0), s, nullptr);
      if (rc) return rc;
    }
    if (J0 > 0) {  // y_{<J} -= L_{J,<J}^T x_J
      rc = gemm_tn_small<T, T>(L + J0, ldl, tmp, nt, B, ldb, (int)J0, LN, r, T(-1), T(1), s,
                               CopyOut<T>{tmp, nt, B + J0, ldb, LN});
      if (rc) return rc;
    } else {
      OOC_CUDA_TRY(cudaMemcpy2DAsync(B + J0, ldb * sizeof(T), tmp, nt * sizeof(T), LN * sizeof(T), r,
                                     cudaMemcpyDeviceToDevice, s));
    }
  }
  return OOC_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------
// Solver state: a factor with the inverses of its diagonal tiles (FP64), and FP32
// copies of both for the correction solves of the refinement.
// ---------------------------------------------------------------------------------
struct ooc_factor {
  int device = 0;
  i64 n = 0;
  int nb = 0;
  int prec = OOC_PREC_FP64;
  // OOC_PREC_FP64: L and Dinv in FP64.  Reduced precision: the FP32 working matrix Lf is
  // the factor (lower triangle; the strict upper triangle is not kept) and Dinvf its
  // diagonal inverses; the FP64 members stay null.
  double* L = nullptr;     // n x n, ld n (owned); lower = factor
  double* Dinv = nullptr;  // bb tiles of nb x nb: L_JJ^{-T}
  float* Lf = nullptr;     // n x n FP32, ld `ld`
  i64 ld = 0;              // leading dimension of Lf (n for a factor object)
  bool owns_Lf = true;     // false when Lf is a caller's matrix (ooc_spotrf_L)
  float* Dinvf = nullptr;
  // panel schedule (reduced precision): nb-wide panels up to column tail0, then nb2-wide
  i64 tail0 = 0;
  int nb2 = 0;
  Panels panels() const {
    Panels P;
    P.n = n;
    P.nb = nb;
    P.tail0 = (Lf && tail0 < n) ? tail0 : n;
    P.nb2 = nb2 > 0 ? nb2 : nb;
    return P;
  }
  double* tmp = nullptr;   // nb x 16
  float* tmpf = nullptr;
  int* status = nullptr;   // device status word of the factorization
  int info = 0;
  // the handle's device-buffer cache (null: plain cudaMalloc / cudaFree); declared before
  // the DevBufs so that it outlives them
  std::shared_ptr<DevPool> pool;
  DevBuf part, partf, work, scratch;
  DevBuf work2;  // BF16 planes of the panel before its tensor-core column solve
  // Solves share the buffers above: calls on one factor from several threads take turns.
  std::mutex solve_mu;
  DevBuf rws;    // refinement workspace (residual, FP32 correction, reductions), kept
  DevBuf sws;    // FP32 right-hand sides of ooc_factor_solve on a reduced factor, kept
  DevBuf part2;  // partial sums of the refinement's norm (second stream)
  // FP64 copy of a host A's lower triangle (ld n), kept for the refinement
  // (OOC_OPT_KEEP_A); A64_src / A64_lda identify the host matrix it came from.
  double* A64 = nullptr;
  const double* A64_src = nullptr;
  i64 A64_lda = 0;
  // a device buffer of the factor, from the pool when there is one
  template <typename T>
  int alloc(T** p, size_t bytes) {
    *p = nullptr;
    if (pool) {
      *p = (T*)pool->alloc(bytes);
    } else if (cudaMalloc((void**)p, bytes) != cudaSuccess) {
      cudaGetLastError();
      *p = nullptr;
    }
    return *p ? OOC_OK : OOC_ERR_NOMEM;
  }
  void release(void* p) {
    if (!p) return;
    if (pool) pool->release(p);
    else cudaFree(p);
  }
  // destroyed after its device work is done (ooc_factor_destroy synchronises the device)
  ~ooc_factor() {
    release(A64);
    release(L);
    release(Dinv);
    if (owns_Lf) release(Lf);
    release(Dinvf);
    release(tmp);
    release(tmpf);
    release(status);
  }
};

namespace {

int alloc_factor(ooc_factor* F, i64 n, int nb, bool reduced) {
  const int bb = (int)((n + nb - 1) / nb);
  const size_t tiles = (size_t)bb * nb * nb;
  bool ok = !F->alloc(&F->status, sizeof(int)) && !F->alloc(&F->tmp, (size_t)nb * RMAX * sizeof(double));
  if (ok && !reduced)
    ok = !F->alloc(&F->L, (size_t)n * n * sizeof(double)) && !F->alloc(&F->Dinv, tiles * sizeof(double));
  if (ok && reduced)
    ok = !F->alloc(&F->Lf, (size_t)n * n * sizeof(float)) && !F->alloc(&F->Dinvf, tiles * sizeof(float)) &&
         !F->alloc(&F->tmpf, (size_t)nb * RMAX * sizeof(float));
  return ok ? OOC_OK : OOC_ERR_NOMEM;
}

struct MixedProf {
  bool on = false;
  std::vector<cudaEvent_t> ev;  // pairs: [2k] start, [2k+1] end (on the segment's stream)
  std::vector<int> kind;        // 0 = FP64 factor + column solve, 1 = trailing update
  std::vector<double> flops;    // algorithmic flops of each update
  cudaEvent_t h2d0 = nullptr, h2d1 = nullptr;  // first copy's start, last copy's end
  double h2d_bytes = 0;         // bytes of a streamed host matrix copied to the device
  void mark(cudaStream_t s) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    ev.push_back(e);
  }
  ~MixedProf() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    if (h2d0) cudaEventDestroy(h2d0);
    if (h2d1) cudaEventDestroy(h2d1);
  }
};

// Right-looking in-core FP64 factorization of F->L (ld n) (the reference's ooc_incore over
// the whole matrix, oocquark.cpp:389-419, with the dsyrk/dgemm tasks as one lower-
// triangular update).  The column solve B := B L_jj^{-T} runs as one FP64 DMMA product
// with the tile's inverse (kept for the solves, formed from the diagonal tile alone),
// B := W (L_jj^{-1})^T with W a copy of B and the triangular half of K skipped.
// Look-ahead on two streams: the diagonal work of panel j (potrf, inverse, column solve)
// runs on `s1` while `s0` performs the bulk of the trailing update of panel j-1; `s0` first
// updates only the next panel's columns and signals `s1`, then updates the rest.
int factor_mixed(ooc_factor* F, int prec, cudaStream_t s0, cudaStream_t s1, int64_t* launches, MixedProf* prof) {
  const i64 n = F->n;
  const int nb = F->nb;
  const int bb = (int)((n + nb - 1) / nb);
  double* A = F->L;
  const i64 lda = n;
  const i64 tile = (i64)nb * nb;
  int rc = F->scratch.ensure((size_t)n * nb * sizeof(double) + (size_t)tile * sizeof(double));
  if (rc) return rc;
  double* W = (double*)F->scratch.p;   // copy of the column panel (m x nb, ld n)
  double* E = W + (size_t)n * nb;      // L_jj^{-1} (lower, ld nb)
  (void)prec;
  cudaEvent_t evA, evP;  // A: next panel's columns updated (s0 -> s1); P: panel solved (s1 -> s0)
  OOC_CUDA_TRY(cudaEventCreateWithFlags(&evA, cudaEventDisableTiming));
  OOC_CUDA_TRY(cudaEventCreateWithFlags(&evP, cudaEventDisableTiming));
  struct EvGuard {
    cudaEvent_t a, b;
    ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
  } guard{evA, evP};
  OOC_CUDA_TRY(cudaEventRecord(evA, s0));  // the matrix was filled on s0
  for (int j = 0; j < bb; j++) {
    const i64 J0 = (i64)j * nb;
    const int LN = (int)std::min<i64>(nb, n - J0);
    double* Djj = A + J0 + J0 * lda;
    // ---- s1: FP64 diagonal tile, its inverse, the column solve
    OOC_CUDA_TRY(cudaStreamWaitEvent(s1, evA, 0));
    if (prof->on) { prof->mark(s1); prof->kind.push_back(0); }
    rc = launch_potrf_tile(Djj, lda, LN, J0, F->status, s1);
    if (rc) return rc;
    double* Dj = F->Dinv + (i64)j * tile;  // Dinv_j = I L_jj^{-T} = L_jj^{-T}; E = Dinv_j^T = L_jj^{-1}
    k_set_identity<double><<<dim3((LN + 255) / 256, std::min(LN, 1024)), 256, 0, s1>>>(Dj, nb, LN);
    rc = launch_trsm_col(Djj, lda, TileCol{Dj, nb, tile}, 1, LN, LN, LN, F->status, s1);
    if (rc) return rc;
    k_transpose<<<dim3((LN + 31) / 32, (LN + 31) / 32), dim3(32, 8), 0, s1>>>(Dj, nb, E, nb, LN);
    const i64 m = n - J0 - LN;
    double* Pn = Djj + LN;  // the panel below the diagonal tile
    if (m > 0) {
      OOC_CUDA_TRY(cudaMemcpy2DAsync(W, n * sizeof(double), Pn, lda * sizeof(double), m * sizeof(double), LN,
                                     cudaMemcpyDeviceToDevice, s1));
      OOC_CUDA_TRY(cudaMemset2DAsync(Pn, lda * sizeof(double), 0, m * sizeof(double), LN, s1));
      rc = launch_gemm_nt_trib(W, n, E, nb, Pn, lda, (int)m, LN, LN, 1.0, F->status, s1);
      if (rc) return rc;
    }
    if (prof->on) prof->mark(s1);
    OOC_CUDA_TRY(cudaEventRecord(evP, s1));
    // ---- s0: trailing update, next panel's columns first
    OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evP, 0));
    if (m > 0) {
      double* C = A + (J0 + LN) * (1 + lda);
      const int below = bb - j - 1;
      if (prof->on) {
        prof->mark(s0);
        prof->kind.push_back(1);
        prof->flops.push_back((double)m * (double)(m + 1) * LN);
      }
      TileMap Cm{C, lda, 0, below, nb};
      rc = launch_panel_update(TileCol{Pn, lda, nb}, Cm, below, 1, m, m, LN, F->status, s0);
      if (rc) return rc;
      OOC_CUDA_TRY(cudaEventRecord(evA, s0));
      if (below > 1) {
        TileMap Cr{C + nb * (1 + lda), lda, 0, below - 1, nb};
        rc = launch_panel_update(TileCol{Pn + nb, lda, nb}, Cr, below - 1, below - 1, m - nb, m - nb, LN,
                                 F->status, s0);
      }
      if (rc) return rc;
      if (prof->on) prof->mark(s0);
    }
    if (launches) *launches += 5 * ((LN + 63) / 64) + 8;
  }
  // s0 continues only after the last diagonal work on s1
  OOC_CUDA_TRY(cudaEventRecord(evP, s1));
  OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evP, 0));
  return OOC_OK;
}

// Reduced-precision factorization of the FP32 working matrix F->Lf (ld n), right-looking
// over nb-wide panels (nb <= 512):
//   s1: the diagonal tile's Cholesky and inverse in one FP32 CTA (k_diag_f32), beside the
//       bulk update of the previous panel (the persistent tensor-core update leaves
//       kChainSMs SMs free for it);
//   s0: the column solve (product with the inverse), then the trailing update in `prec` --
//       the next panel's block columns first (an event lets s1 start on its diagonal
//       tile), then the rest.
// Split-BF16 factors with nb a multiple of 128 solve the panel on the tensor cores
// (k_trsm2_bf16x3, the update's three products): the panel is split into BF16 planes
// while its diagonal tile is factored (right after the previous narrow update, on s0),
// the diagonal kernel also writes the planes of the inverse, and the solve writes the FP32
// panel together with the planes the update reads.  Otherwise the solve is an FP32
// product on the CUDA cores (k_colsolve_f32) and the update splits the panel itself.
constexpr int kChainSMs = 1;  // the diagonal kernel is one CTA

int factor_f32(ooc_factor* F, int prec, cudaStream_t s0, cudaStream_t s1, int64_t* launches, MixedProf* prof) {
  const i64 n = F->n;
  const int nb = F->nb;
  const Panels P = F->panels();
  const int bb = P.count();
  float* A = F->Lf;
  const i64 lda = F->ld;
  const i64 tile = (i64)nb * nb;
  if (nb > DG_MAX) return OOC_ERR_UNSUPPORTED;
  const bool split = (nb % 128 == 0) && (P.nb2 % 128 == 0);
  const bool tc_solve = split && prec == OOC_PREC_BF16X3 && n > nb;
  int rc = F->scratch.ensure((size_t)tile * (sizeof(float) + (tc_solve ? 2 * sizeof(__nv_bfloat16) : 0)));
  if (rc) return rc;
  float* Xr = (float*)F->scratch.p;  // L_jj^{-1}, row-major (ld LN), from the diagonal kernel
  __nv_bfloat16* Xh = tc_solve ? reinterpret_cast<__nv_bfloat16*>(Xr + tile) : nullptr;  // its hi, lo planes
  __nv_bfloat16* Xl = tc_solve ? Xh + tile : nullptr;
  if (tc_solve) {  // planes of the panel before (work2) and after (work) the solve
    const size_t pb = bf16x3_work_bytes((int)(n - std::min(nb, P.nb2)), nb);
    if ((rc = F->work.ensure(pb)) || (rc = F->work2.ensure(pb))) return rc;
  }
  OOC_CUDA_TRY(cudaFuncSetAttribute(k_diag_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DG_SMEM));
  OOC_CUDA_TRY(cudaFuncSetAttribute(k_diag_s256, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DS_SMEM));
  cudaEvent_t evA, evP;  // A: next panel's columns updated (s0 -> s1); P: diagonal tile done (s1 -> s0)
  OOC_CUDA_TRY(cudaEventCreateWithFlags(&evA, cudaEventDisableTiming));
  OOC_CUDA_TRY(cudaEventCreateWithFlags(&evP, cudaEventDisableTiming));
  struct EvGuard {
    cudaEvent_t a, b;
    ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
  } guard{evA, evP};
  auto width = [&](int p) -> int {  // width of panel p (0 past the last)
    if (p >= bb) return 0;
    i64 J0, off;
    int LN, ld;
    P.get(p, &J0, &LN, &off, &ld);
    return LN;
  };
  OOC_CUDA_TRY(cudaEventRecord(evA, s0));  // the matrix was filled on s0
  if (tc_solve) {  // panel 0 below its diagonal tile, beside the first diagonal kernel
    const int w0 = width(0);
    rc = launch_split_bf16_f32(A + w0, lda, (int)(n - w0), w0, F->work2.p, F->work2.bytes, s0);
    if (rc) return rc;
  }
  for (int j = 0; j < bb; j++) {
    i64 J0, off;
    int LN, ldd;
    P.get(j, &J0, &LN, &off, &ldd);
    const int LNn = width(j + 1);              // the next panel's width
    const int bjn = (LNn + 127) / 128;         // its 128-wide block columns in the trailing matrix
    float* Djj = A + J0 + J0 * lda;
    OOC_CUDA_TRY(cudaStreamWaitEvent(s1, evA, 0));
    if (prof->on) { prof->mark(s1); prof->kind.push_back(0); }
    if (LN <= DS_MAX)  // the tile fits in shared memory
      k_diag_s256<<<1, DG_THREADS, DS_SMEM, s1>>>(Djj, lda, LN, J0, F->Dinvf + off, ldd, Xr, Xh, Xl, F->status);
    else
      k_diag_f32<<<1, DG_THREADS, DG_SMEM, s1>>>(Djj, lda, LN, J0, F->Dinvf + off, ldd, Xr, Xh, Xl, F->status);
    OOC_CUDA_TRY(cudaGetLastError());
    if (prof->on) prof->mark(s1);
    OOC_CUDA_TRY(cudaEventRecord(evP, s1));
    OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evP, 0));
    const i64 m = n - J0 - LN;
    if (m > 0) {
      float* Pn = Djj + LN;
      if (prof->on) { prof->mark(s0); prof->kind.push_back(0); }
      if (tc_solve) {
        rc = launch_trsm_bf16x3_f32(F->work2.p, F->work2.bytes, Xh, Xl, Pn, lda, (int)m, LN, F->work.p,
                                    F->work.bytes, F->status, s0);
        if (rc) return rc;
      } else {
        k_colsolve_f32<<<(unsigned)((m + CS_ROWS - 1) / CS_ROWS), FTHR, 0, s0>>>(Pn, lda, Xr, LN, (int)m, LN,
                                                                                F->status);
        OOC_CUDA_TRY(cudaGetLastError());
      }
      if (prof->on) {
        prof->mark(s0);
        prof->mark(s0);
        prof->kind.push_back(1);
        prof->flops.push_back((double)m * (double)(m + 1) * LN);
      }
      float* C = A + (J0 + LN) * (1 + lda);
      if (tc_solve) {  // the planes come from the solve
        rc = syrk_f32(prec, Pn, lda, C, lda, (int)m, LN, F->status, s0, F->work, 0, bjn, 0, 0);
        if (rc) return rc;
        OOC_CUDA_TRY(cudaEventRecord(evA, s0));
        // panel j+1 is final now: its planes (rows below its diagonal tile), then the bulk
        if (m - LNn > 0) {
          rc = launch_split_bf16_f32(C + LNn, lda, (int)(m - LNn), LNn, F->work2.p, F->work2.bytes, s0);
          if (rc) return rc;
        }
        rc = syrk_f32(prec, Pn, lda, C, lda, (int)m, LN, F->status, s0, F->work, bjn, -1, 0, kChainSMs);
      } else if (split) {
        rc = syrk_f32(prec, Pn, lda, C, lda, (int)m, LN, F->status, s0, F->work, 0, bjn, 1, 0);
        if (rc) return rc;
        OOC_CUDA_TRY(cudaEventRecord(evA, s0));
        rc = syrk_f32(prec, Pn, lda, C, lda, (int)m, LN, F->status, s0, F->work, bjn, -1, 0, kChainSMs);
      } else {
        rc = syrk_f32(prec, Pn, lda, C, lda, (int)m, LN, F->status, s0, F->work);
        if (rc) return rc;
        OOC_CUDA_TRY(cudaEventRecord(evA, s0));
      }
      if (rc) return rc;
      if (prof->on) prof->mark(s0);
    }
    if (launches) *launches += 5;
  }
  OOC_CUDA_TRY(cudaEventRecord(evP, s1));
  OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evP, 0));
  return OOC_OK;
}

// Lower-triangle elements of an m x m trailing matrix in columns [a, b): the useful
// outputs of an update restricted to those columns (2 K flops each).
double lower_elems(i64 m, i64 a, i64 b) {
  b = std::min(b, m);
  if (a >= b) return 0.0;
  return (double)(b - a) * (double)m - ((double)b * (double)(b - 1) - (double)a * (double)(a - 1)) / 2.0;
}

// Where the columns of a left-looking factorization come from: a page-locked host matrix
// (copied on the copy stream, into the kept FP64 copy or through a ring of staging
// slots) or a device matrix (converted in place).  Every column block reaches the FP32
// working matrix through k_lower_conv on the compute stream.
struct LbSource {
  const double* A = nullptr;
  i64 lda = 0;
  bool on_device = false;
  double* keep = nullptr;    // FP64 copy of the lower triangle (ld n), kept for the refinement
  double* stage = nullptr;   // otherwise: `slots` staging slots of n x chunk doubles
  int slots = 0;
  i64 chunk = 512;           // columns per copy (at most 256 MB of full column height)
};

// Split-BF16 factorization of the FP32 working matrix F->Lf over left-looking column
// blocks (the reference's panel streaming, oocdag.cpp:59-87: A2Y of a panel, its update by
// every finished column, then the in-core factorization; here a block of whole panels).
// Block b covers columns [c0, c1); F_b is its first panel, F_{b+1} the next block's.
//   sc  copies the host matrix's lower triangle, chunk after chunk in column order, as
//       far ahead as the staging allows (all of it when a kept copy is the destination),
//       and, for a device matrix or a kept copy, converts each group of columns to FP32
//       right behind its copies (beside s0's tensor-core work);
//   s0  converts staged chunks to FP32 when they are needed, or waits for the group's
//       conversion on sc.  At block b's start F_b is already
//       up to date, so s1 factors its diagonal tile at once while s0 catches the rest of
//       the block and F_{b+1} up with all panels before the block (long-K tensor-core
//       updates from the plane store, at most kCatchK columns of K per launch).  The
//       block's panels then go right-looking: column solve (writing its BF16 planes into
//       the plane store: row r, column k of L at r * ldk + k), the next panel's columns
//       first (an event lets s1 start on its diagonal tile), then the rest of the block
//       and F_{b+1}, so that F_{b+1} is final when the block ends.  The in-block updates
//       span at most a block's width, so the panels are narrow (nb/2 where nb is a
//       multiple of 256): their diagonal tiles are factored in shared memory, quickly
//       enough to hide behind those updates;
//   s1  the one-CTA diagonal kernels, beside s0's bulk updates, as in factor_f32.
// Long-K catch-ups move C once per kCatchK columns of K instead of once per panel, which
// is what makes the tensor pipe busier than in the right-looking factor_f32.
// Requires the tensor-core column solve (nb and nb2 multiples of 128).
constexpr i64 kCatchK = 8192;

int factor_f32_lb(ooc_factor* F, cudaStream_t s0, cudaStream_t s1, cudaStream_t sc, cudaStream_t sc2, i64 block_cols,
                  const LbSource& src, int64_t* launches, MixedProf* prof) {
  const i64 n = F->n;
  const int nb = F->nb;
  const Panels P = F->panels();
  const int bb = P.count();
  float* A = F->Lf;
  const i64 lda = F->ld;
  const i64 tile = (i64)nb * nb;
  if (nb > DG_MAX || nb % 128 || P.nb2 % 128 || n <= nb || lda != n) return OOC_ERR_UNSUPPORTED;
  if (!src.on_device && !src.keep && (!src.stage || src.slots < 1)) return OOC_ERR_INTERNAL;
  int rc = F->scratch.ensure((size_t)tile * (sizeof(float) + 2 * sizeof(__nv_bfloat16)));
  if (rc) return rc;
  float* Xr = (float*)F->scratch.p;
  __nv_bfloat16* Xh = reinterpret_cast<__nv_bfloat16*>(Xr + tile);
  __nv_bfloat16* Xl = Xh + tile;
  const size_t pb = bf16x3_work_bytes((int)(n - std::min(nb, P.nb2)), nb);
  if ((rc = F->work2.ensure(pb))) return rc;
  // plane store: hi then lo, n rows of ldk BF16 each, then the update launches' tickets
  const i64 ldk = (n + 63) / 64 * 64;
  const size_t plane = (size_t)n * (size_t)ldk;
  if ((rc = F->work.ensure(2 * plane * sizeof(__nv_bfloat16) + 256))) return rc;
  __nv_bfloat16* Ghi = (__nv_bfloat16*)F->work.p;
  __nv_bfloat16* Glo = Ghi + plane;
  unsigned long long* tickets = reinterpret_cast<unsigned long long*>(Glo + plane);
  OOC_CUDA_TRY(cudaFuncSetAttribute(k_diag_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DG_SMEM));
  OOC_CUDA_TRY(cudaFuncSetAttribute(k_diag_s256, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DS_SMEM));
  auto panel = [&](int p, i64* J0, int* LN) {
    i64 off;
    int ld;
    P.get(p, J0, LN, &off, &ld);
  };
  auto col_of = [&](int q) -> i64 {  // first column of panel q (n past the last)
    if (q >= bb) return n;
    i64 J0;
    int LN;
    panel(q, &J0, &LN);
    return J0;
  };
  // blocks of whole panels: [first panel, one past the last)
  std::vector<std::pair<int, int>> blocks;
  for (int p = 0; p < bb;) {
    const i64 c0 = col_of(p);
    int q = p + 1;
    while (q < bb && (block_cols <= 0 || col_of(q) - c0 < block_cols)) q++;
    blocks.emplace_back(p, q);
    p = q;
  }
  const int nblocks = (int)blocks.size();
  // chunks (the unit of copy and conversion): each panel's columns, split to at most
  // src.chunk columns, in column order -- the order s0 converts them in
  struct Chunk { i64 c0, c1; };
  std::vector<Chunk> chunks;
  std::vector<std::pair<int, int>> panel_chunks(bb);  // [first chunk, one past the last)
  const i64 cw = src.on_device ? n : std::max<i64>(1, src.chunk);
  for (int q = 0; q < bb; q++) {
    const int k0 = (int)chunks.size();
    const i64 a = col_of(q), e = col_of(q + 1);
    for (i64 c = a; c < e; c += cw) chunks.push_back({c, std::min(e, c + cw)});
    panel_chunks[q] = {k0, (int)chunks.size()};
  }
  const int nchunks = (int)chunks.size();
  std::vector<cudaEvent_t> evs;  // every event this call creates (destroyed on return)
  struct EvGuard {
    std::vector<cudaEvent_t>* v;
    ~EvGuard() { for (cudaEvent_t e : *v) cudaEventDestroy(e); }
  } guard{&evs};
  auto new_event = [&](cudaEvent_t* e) -> int {
    OOC_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    evs.push_back(*e);
    return OOC_OK;
  };
  cudaEvent_t evA, evP;
  if ((rc = new_event(&evA)) || (rc = new_event(&evP))) return rc;
  std::vector<cudaEvent_t> evCopied(nchunks, nullptr), evFree(src.slots > 0 ? src.slots : 1, nullptr);
  if (!src.on_device) {
    for (auto& e : evCopied) if ((rc = new_event(&e))) return rc;
    for (auto& e : evFree) if ((rc = new_event(&e))) return rc;
  }
  const unsigned gx = (unsigned)((n + 255) / 256);
  // copies are enqueued in chunk order; with staging slots, chunk k waits until the
  // conversion of chunk k - slots has freed its slot (enqueued on s0 before it)
  int next_copy = 0, next_conv = 0;
  OOC_CUDA_TRY(cudaEventRecord(evP, s0));  // the factor's buffers were set up on s0
  OOC_CUDA_TRY(cudaStreamWaitEvent(sc, evP, 0));
  // Device matrices and kept host copies ("side" mode): the copies and every conversion
  // run on sc, group after group in the order the compute stream needs them, so the
  // conversions (HBM-bound) overlap the compute stream's tensor-core work; s0 only waits
  // for a group's event before it uses the group's columns.  A group is F_0, then for each
  // block the rest of its panels and the next block's first panel.
  const bool side = src.on_device || src.keep;
  auto enqueue_copies = [&]() -> int {
    if (src.on_device || side) return OOC_OK;
    while (next_copy < nchunks && (src.keep || next_copy < next_conv + src.slots)) {
      const Chunk& c = chunks[next_copy];
      double* dst;
      if (src.keep) {
        dst = src.keep + c.c0 * n;
      } else {
        const int slot = next_copy % src.slots;
        if (next_copy >= src.slots) OOC_CUDA_TRY(cudaStreamWaitEvent(sc, evFree[slot], 0));
        dst = src.stage + (size_t)slot * (size_t)n * (size_t)src.chunk;
      }
      if (prof->on && next_copy == 0) {
        OOC_CUDA_TRY(cudaEventCreate(&prof->h2d0));
        OOC_CUDA_TRY(cudaEventRecord(prof->h2d0, sc));
      }
      OOC_CUDA_TRY(cudaMemcpy2DAsync(dst + c.c0, n * sizeof(double), src.A + c.c0 + c.c0 * src.lda,
                                     src.lda * sizeof(double), (n - c.c0) * sizeof(double), c.c1 - c.c0,
                                     cudaMemcpyHostToDevice, sc));
      OOC_CUDA_TRY(cudaEventRecord(evCopied[next_copy], sc));
      prof->h2d_bytes += (double)(n - c.c0) * (double)(c.c1 - c.c0) * sizeof(double);
      if (prof->on && next_copy == nchunks - 1) {
        OOC_CUDA_TRY(cudaEventCreate(&prof->h2d1));
        OOC_CUDA_TRY(cudaEventRecord(prof->h2d1, sc));
      }
      next_copy++;
    }
    return OOC_OK;
  };
  auto convert_panel = [&](int q) -> int {
    for (int k = panel_chunks[q].first; k < panel_chunks[q].second; k++) {
      const Chunk& c = chunks[k];
      const int w = (int)(c.c1 - c.c0);
      const double* from;
      i64 ldf = n;
      if (src.on_device) {
        from = src.A + c.c0 * src.lda;
        ldf = src.lda;
      } else {
        OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evCopied[k], 0));
        from = src.keep ? src.keep + c.c0 * n : src.stage + (size_t)(k % src.slots) * (size_t)n * (size_t)src.chunk;
      }
      k_lower_conv<double, float><<<dim3(gx, (unsigned)std::min(w, 1024)), 256, 0, s0>>>(from, ldf, A + c.c0 * lda,
                                                                                       lda, n, c.c0, w, 0);
      OOC_CUDA_TRY(cudaGetLastError());
      if (!src.on_device && !src.keep) OOC_CUDA_TRY(cudaEventRecord(evFree[k % src.slots], s0));
      next_conv = k + 1;
      if (launches) *launches += 1;
      if ((rc = enqueue_copies())) return rc;
    }
    return OOC_OK;
  };
  // panels q0..q1 into the FP32 matrix: one conversion over their columns (a device
  // matrix, or the kept copy once its last chunk has arrived), or chunk by chunk through
  // the staging slots
  std::vector<int> group_of(bb, -1);
  std::vector<cudaEvent_t> evConv, evCopy1, evCopy2;
  if (side) {
    OOC_CUDA_TRY(cudaStreamWaitEvent(sc2, evP, 0));
    std::vector<std::pair<int, int>> groups{{0, 0}};
    for (const auto& bk : blocks) {
      const int q1 = std::min(bk.second, bb - 1);
      if (q1 >= bk.first + 1) groups.emplace_back(bk.first + 1, q1);
    }
    evConv.resize(groups.size());
    evCopy1.resize(groups.size());
    evCopy2.resize(groups.size());
    for (size_t g = 0; g < groups.size(); g++) {
      const int q0 = groups[g].first, q1 = groups[g].second;
      for (int q = q0; q <= q1; q++) group_of[q] = (int)g;
      if ((rc = new_event(&evConv[g])) || (rc = new_event(&evCopy1[g])) || (rc = new_event(&evCopy2[g]))) return rc;
      if (!src.on_device) {  // this group's chunks into the kept FP64 copy, in column order,
                             // alternately on the two copy streams (two copy engines in flight)
        if (prof->on && g == 0) {
          OOC_CUDA_TRY(cudaEventCreate(&prof->h2d0));
          OOC_CUDA_TRY(cudaEventRecord(prof->h2d0, sc));
          OOC_CUDA_TRY(cudaStreamWaitEvent(sc2, prof->h2d0, 0));
        }
        // the second stream starts a group only when the first has issued the previous
        // group's copies: both engines then work on the group the compute stream needs
        // next, instead of the second racing ahead on later groups and sharing the link
        if (g > 0 && sc2 != sc) OOC_CUDA_TRY(cudaStreamWaitEvent(sc2, evCopy1[g - 1], 0));
        for (int k = panel_chunks[q0].first; k < panel_chunks[q1].second; k++) {
          const Chunk& c = chunks[k];
          OOC_CUDA_TRY(cudaMemcpy2DAsync(src.keep + c.c0 + c.c0 * n, n * sizeof(double), src.A + c.c0 + c.c0 * src.lda,
                                         src.lda * sizeof(double), (n - c.c0) * sizeof(double), c.c1 - c.c0,
                                         cudaMemcpyHostToDevice, (k & 1) ? sc2 : sc));
          prof->h2d_bytes += (double)(n - c.c0) * (double)(c.c1 - c.c0) * sizeof(double);
        }
        OOC_CUDA_TRY(cudaEventRecord(evCopy1[g], sc));
        OOC_CUDA_TRY(cudaEventRecord(evCopy2[g], sc2));  // sc converts after both streams' copies
        OOC_CUDA_TRY(cudaStreamWaitEvent(sc, evCopy2[g], 0));
        if (prof->on && panel_chunks[q1].second == nchunks) {
          OOC_CUDA_TRY(cudaEventCreate(&prof->h2d1));
          OOC_CUDA_TRY(cudaEventRecord(prof->h2d1, sc));
        }
      }
      const i64 c0 = col_of(q0), c1 = col_of(q1 + 1);
      const double* from = src.on_device ? src.A + c0 * src.lda : src.keep + c0 * n;
      k_lower_conv<double, float><<<dim3(gx, (unsigned)std::min<i64>(c1 - c0, 1024)), 256, 0, sc>>>(
          from, src.on_device ? src.lda : n, A + c0 * lda, lda, n, c0, (int)(c1 - c0), 0);
      OOC_CUDA_TRY(cudaGetLastError());
      OOC_CUDA_TRY(cudaEventRecord(evConv[g], sc));
      if (launches) *launches += 1;
    }
  }
  auto convert_panels = [&](int q0, int q1) -> int {
    if (q1 < q0) return OOC_OK;
    if (side) {  // converted on sc: wait for the group that holds them
      OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evConv[group_of[q1]], 0));
      return OOC_OK;
    }
    if (src.on_device || src.keep) {
      const int k1 = panel_chunks[q1].second - 1;
      const i64 c0 = col_of(q0), c1 = col_of(q1 + 1);
      const double* from = src.on_device ? src.A + c0 * src.lda : src.keep + c0 * n;
      if (!src.on_device) OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evCopied[k1], 0));  // copies land in order
      k_lower_conv<double, float><<<dim3(gx, (unsigned)std::min<i64>(c1 - c0, 1024)), 256, 0, s0>>>(
          from, src.on_device ? src.lda : n, A + c0 * lda, lda, n, c0, (int)(c1 - c0), 0);
      OOC_CUDA_TRY(cudaGetLastError());
      next_conv = k1 + 1;
      if (launches) *launches += 1;
      return OOC_OK;
    }
    for (int q = q0; q <= q1; q++) {
      int r = convert_panel(q);
      if (r) return r;
    }
    return OOC_OK;
  };
  // C = trailing matrix from column `c` (rows c..n-1), columns [c, c + w), minus the
  // contribution of the finished panels in columns [0, K): long-K updates from the store
  auto catch_up = [&](i64 c, i64 w, i64 K) -> int {
    if (K <= 0 || w <= 0) return OOC_OK;
    const i64 m = n - c;
    float* C = A + c * (1 + lda);
    if (prof->on) {
      prof->mark(s0);
      prof->kind.push_back(1);
      prof->flops.push_back(2.0 * (double)K * lower_elems(m, 0, w));
    }
    for (i64 k0 = 0; k0 < K; k0 += kCatchK) {
      const i64 kw = std::min(kCatchK, K - k0);
      int r = launch_syrk_planes_f32(Ghi + c * ldk + k0, Glo + c * ldk + k0, ldk, (int)m, (int)kw, C, lda, F->status,
                                     s0, tickets, 0, (int)((w + 127) / 128), kChainSMs);
      if (r) return r;
      if (launches) *launches += 1;
    }
    if (prof->on) prof->mark(s0);
    return OOC_OK;
  };
  auto split_raw = [&](i64 J0, int LN) -> int {  // panel's rows below its diagonal tile -> work2
    const i64 m = n - J0 - LN;
    if (m <= 0) return OOC_OK;
    if (launches) *launches += 1;
    return launch_split_bf16_f32(A + J0 + LN + J0 * lda, lda, (int)m, LN, F->work2.p, F->work2.bytes, s0);
  };
  if ((rc = enqueue_copies())) return rc;
  if ((rc = convert_panels(0, 0))) return rc;  // F_0
  OOC_CUDA_TRY(cudaEventRecord(evA, s0));
  {
    i64 J0;
    int LN;
    panel(0, &J0, &LN);
    if ((rc = split_raw(J0, LN))) return rc;
  }
  for (int b = 0; b < nblocks; b++) {
    const int p0 = blocks[b].first, p1 = blocks[b].second;
    const i64 c0 = col_of(p0), cf = col_of(p0 + 1), c1 = col_of(p1);
    const int plast = std::min(p1, bb - 1);  // the block's panels after F_b, and F_{b+1}
    const i64 cn = col_of(plast + 1);         // end of the columns the block's updates reach
    // F_b is final: s1 may factor its diagonal tile (after evA) while s0 converts the rest
    // of the block and F_{b+1} and catches them up with every panel before the block.
    if ((rc = convert_panels(p0 + 1, plast))) return rc;
    if ((rc = catch_up(c1, cn - c1, c0))) return rc;  // F_{b+1}
    if ((rc = catch_up(cf, c1 - cf, c0))) return rc;  // the rest of block b
    for (int j = p0; j < p1; j++) {
      i64 J0, off;
      int LN, ldd;
      P.get(j, &J0, &LN, &off, &ldd);
      float* Djj = A + J0 + J0 * lda;
      OOC_CUDA_TRY(cudaStreamWaitEvent(s1, evA, 0));
      if (prof->on) { prof->mark(s1); prof->kind.push_back(0); }
      if (LN <= DS_MAX)
        k_diag_s256<<<1, DG_THREADS, DS_SMEM, s1>>>(Djj, lda, LN, J0, F->Dinvf + off, ldd, Xr, Xh, Xl, F->status);
      else
        k_diag_f32<<<1, DG_THREADS, DG_SMEM, s1>>>(Djj, lda, LN, J0, F->Dinvf + off, ldd, Xr, Xh, Xl, F->status);
      OOC_CUDA_TRY(cudaGetLastError());
      if (prof->on) prof->mark(s1);
      OOC_CUDA_TRY(cudaEventRecord(evP, s1));
      OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evP, 0));
      if (launches) *launches += 1;
      const i64 m = n - J0 - LN;
      if (m <= 0) continue;
      float* Pn = Djj + LN;
      __nv_bfloat16* gh = Ghi + (J0 + LN) * ldk + J0;  // this panel's rows below its diagonal tile
      __nv_bfloat16* gl = Glo + (J0 + LN) * ldk + J0;
      if (prof->on) { prof->mark(s0); prof->kind.push_back(0); }
      rc = launch_trsm_bf16x3_f32_to(F->work2.p, F->work2.bytes, Xh, Xl, Pn, lda, (int)m, LN, gh, gl, ldk, F->status,
                                     s0);
      if (rc) return rc;
      if (prof->on) prof->mark(s0);
      if (launches) *launches += 1;
      // right-looking inside the block, and into F_{b+1}: columns [J0 + LN, cn)
      i64 J0n;
      int LNn;
      panel(j + 1, &J0n, &LNn);
      const i64 wa = cn - J0 - LN;
      const int bjn = (LNn + 127) / 128;
      const int bjh = (int)((wa + 127) / 128);
      float* C = A + (J0 + LN) * (1 + lda);
      if (prof->on) {
        prof->mark(s0);
        prof->kind.push_back(1);
        prof->flops.push_back(2.0 * (double)LN * lower_elems(m, 0, wa));
      }
      rc = launch_syrk_planes_f32(gh, gl, ldk, (int)m, LN, C, lda, F->status, s0, tickets, 0, bjn, 0);
      if (rc) return rc;
      OOC_CUDA_TRY(cudaEventRecord(evA, s0));
      if ((rc = split_raw(J0n, LNn))) return rc;
      rc = launch_syrk_planes_f32(gh, gl, ldk, (int)m, LN, C, lda, F->status, s0, tickets, bjn, bjh, kChainSMs);
      if (rc) return rc;
      if (prof->on) prof->mark(s0);
      if (launches) *launches += 2;
    }
  }
  OOC_CUDA_TRY(cudaEventRecord(evP, s1));
  OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evP, 0));
  return OOC_OK;
}

int read_int(const int* d, int* h, cudaStream_t s) {
  OOC_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, s));
  OOC_CUDA_TRY(cudaStreamSynchronize(s));
  return OOC_OK;
}

}  // namespace

static int create_impl(ooc_handle* h, const double* A, int64_t n, int64_t lda, bool gen, uint64_t seed, double alpha,
                       int nb, int prec, ooc_factor** out, int* info, ooc_stats* stats) {
  if (!h) return -1;
  if (!gen && !A && n > 0) return -2;
  if (n <= 0) return -3;
  if (!gen && lda < n) return -4;
  if (prec != OOC_PREC_FP64 && prec != OOC_PREC_FP32 && prec != OOC_PREC_BF16X3) return -6;
  const bool reduced = prec != OOC_PREC_FP64;
  if (nb <= 0 || (reduced && nb > DG_MAX)) return -5;
  if (!out) return -7;
  if (!info) return -8;
  *out = nullptr;
  *info = 0;
  if (stats) memset(stats, 0, sizeof(*stats));
  cudaSetDevice(ooc_device(h));
  cudaStream_t s = ooc_compute_stream(h);
  ooc_factor* F = new ooc_factor();
  F->device = ooc_device(h);
  F->n = n;
  F->ld = n;
  F->nb = nb;
  F->prec = prec;
  F->tail0 = n;
  F->nb2 = nb;
  // Left-looking column blocks (OOC_OPT_BLOCK_COLS) for split-BF16 factors of a stored
  // matrix: the blocks are filled on the third stream while earlier ones are factored.
  bool on_device = false, pinned = false;
  if (!gen) {
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, A) == cudaSuccess) {
      on_device = pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged;
      pinned = pa.type == cudaMemoryTypeHost;
    }
    cudaGetLastError();
  }
  i64 bcols = 0;
  {
    int64_t opt = -1;
    ooc_get_option(h, OOC_OPT_BLOCK_COLS, &opt);
    // automatic: 4096-column blocks for device and page-locked host matrices of more
    // than two blocks (faster long-K updates; for a host matrix, copies overlapped)
    bcols = opt >= 0 ? opt : ((pinned || on_device) && n > 2 * 4096 ? 4096 : 0);
  }
  const bool lb = !gen && bcols > 0 && prec == OOC_PREC_BF16X3 && nb % 128 == 0 && n > nb && (on_device || pinned);
  if (lb && nb % 256 == 0) {  // left-looking blocks: nb/2-wide panels throughout
    F->tail0 = 0;
    F->nb2 = nb / 2;
  } else if (prec == OOC_PREC_BF16X3 && nb % 256 == 0 && n > nb) {  // nb/2-wide tail panels
    int64_t tail = 0;
    ooc_get_option(h, OOC_OPT_TAIL_ORDER, &tail);
    if (tail > 0) {
      const i64 t0 = std::max<i64>(0, n - tail);
      F->tail0 = std::min<i64>(n, (t0 + nb - 1) / nb * nb);
      F->nb2 = nb / 2;
    }
  }
  F->pool = ooc_handle_pool(h);
  for (DevBuf* b : {&F->part, &F->partf, &F->work, &F->scratch, &F->work2, &F->part2, &F->rws, &F->sws})
    b->pool = F->pool.get();
  int rc = alloc_factor(F, n, nb, reduced);
  if (rc) { delete F; return rc; }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // A (generated, host or device) into the factor's storage
  rc = OOC_OK;
  if (cudaMemsetAsync(F->status, 0, sizeof(int), s) != cudaSuccess) rc = OOC_ERR_CUDA;
  int64_t keep = 0;
  if (!gen && !on_device) ooc_get_option(h, OOC_OPT_KEEP_A, &keep);
  if (!rc && keep && reduced) {
    if (F->alloc(&F->A64, (size_t)n * n * sizeof(double))) {
      rc = OOC_ERR_NOMEM;
    } else {
      F->A64_src = A;
      F->A64_lda = lda;
    }
  }
  DevBuf stage;  // host columns on their way to the FP32 matrix when no copy is kept
  const unsigned gx = (unsigned)((n + 255) / 256);
  // columns [c0, c1) of A (rows c0..n-1) into the FP32 working matrix, on stream `st`
  std::function<int(i64, i64, cudaStream_t)> fill = [&](i64 c0, i64 c1, cudaStream_t st) -> int {
    if (on_device) {
      k_lower_conv<double, float><<<dim3(gx, (unsigned)std::min<i64>(c1 - c0, 1024)), 256, 0, st>>>(
          A + c0 * lda, lda, F->Lf + c0 * n, n, n, c0, (int)(c1 - c0), 0);
      return cudaGetLastError() == cudaSuccess ? OOC_OK : OOC_ERR_CUDA;
    }
    // chunks of at most 256 MB of a full column height: the copy follows the lower
    // triangle chunk by chunk (rows k0..n-1 of columns k0..k0+wc-1)
    const i64 w = std::max<i64>(1, std::min<i64>(c1 - c0, (256LL << 20) / (8 * n)));
    if (!keep) {
      int r = stage.ensure((size_t)n * w * sizeof(double));
      if (r) return r;
    }
    for (i64 k0 = c0; k0 < c1; k0 += w) {  // the lower part of each column block (rows k0..n-1)
      const int wc = (int)std::min<i64>(w, c1 - k0);
      double* dst = keep ? F->A64 + k0 * n : (double*)stage.p;  // column k0 of the block, ld n
      if (cudaMemcpy2DAsync(dst + k0, n * sizeof(double), A + k0 + k0 * lda, lda * sizeof(double),
                            (n - k0) * sizeof(double), wc, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return OOC_ERR_CUDA;
      k_lower_conv<double, float><<<dim3(gx, (unsigned)std::min(wc, 1024)), 256, 0, st>>>(dst, n, F->Lf + k0 * n, n,
                                                                                        n, k0, wc, 0);
    }
    return cudaGetLastError() == cudaSuccess ? OOC_OK : OOC_ERR_CUDA;
  };
  if (!rc && !reduced) {
    if (gen) {
      rc = launch_gen_uniform_block(F->L, n, n, seed, alpha, 0, 0, n, n, s);
    } else if (cudaMemcpy2DAsync(F->L, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), n,
                                 cudaMemcpyDefault, s) != cudaSuccess) {
      rc = OOC_ERR_CUDA;
    }
  } else if (!rc && !lb) {
    if (gen) {
      k_gen_uniform_f32_lower<<<dim3(gx, (unsigned)std::min<i64>(n, 1024)), 256, 0, s>>>(
          F->Lf, n, n, ooc_uniform_key(seed), alpha);
    } else {
      rc = fill(0, n, s);
      if (!rc && !on_device && cudaStreamSynchronize(s) != cudaSuccess) rc = OOC_ERR_CUDA;  // before `stage` goes
    }
    if (!rc && cudaGetLastError() != cudaSuccess) rc = OOC_ERR_CUDA;
  }
  int64_t launches = 0;
  MixedProf prof;
  {
    int64_t pv = 0;
    ooc_get_option(h, OOC_OPT_PROFILE, &pv);
    prof.on = pv != 0;
  }
  if (!rc) {
    cudaEventRecord(e0, s);
    void* s1p = nullptr;
    ooc_get_stream(h, 1, &s1p);
    if (lb) {
      void* s2p = nullptr;
      void* s3p = nullptr;
      ooc_get_stream(h, 2, &s2p);
      int64_t ncs = 1;
      ooc_get_option(h, OOC_OPT_COPY_STREAMS, &ncs);
      ooc_get_stream(h, ncs > 1 ? 3 : 2, &s3p);  // one stream: sc2 is sc itself
      LbSource src;
      src.A = A;
      src.lda = lda;
      src.on_device = on_device;
      src.keep = keep ? F->A64 : nullptr;
      src.chunk = std::max<i64>(1, std::min<i64>(n, (256LL << 20) / (8 * n)));
      if (!on_device && !keep) {  // a ring of staging slots for the copies
        src.slots = 8;
        rc = stage.ensure((size_t)src.slots * (size_t)n * (size_t)src.chunk * sizeof(double));
        src.stage = (double*)stage.p;
      }
      if (!rc) rc = factor_f32_lb(F, s, (cudaStream_t)s1p, (cudaStream_t)s2p, (cudaStream_t)s3p, bcols, src, &launches, &prof);
    } else {
      rc = reduced ? factor_f32(F, prec, s, (cudaStream_t)s1p, &launches, &prof)
                   : factor_mixed(F, prec, s, (cudaStream_t)s1p, &launches, &prof);
    }
    cudaEventRecord(e1, s);
  }
  int st = 0;
  if (!rc) rc = read_int(F->status, &st, s);
  if (lb) F->work.release();  // the plane store: the factor is complete
  if (!rc) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { ooc_set_last_error(e, "mixed factorization", __FILE__, __LINE__); rc = OOC_ERR_CUDA; }
  }
  float ms = 0;
  if (!rc) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) { delete F; return rc; }
  F->info = st;
  *info = st;
  if (stats) {
    stats->seconds = ms * 1e-3;
    stats->flops = (double)n * n * n / 3.0;
    stats->npanels = 1;
    stats->info = st;
    stats->kernel_launches = launches;
    stats->h2d_bytes = prof.h2d_bytes;
    if (prof.h2d0 && prof.h2d1) {
      float t = 0;
      cudaEventElapsedTime(&t, prof.h2d0, prof.h2d1);
      stats->h2d_ms = t;
    }
    if (prof.on) {
      size_t fi = 0;
      for (size_t k = 0; k < prof.kind.size(); k++) {
        float t = 0;
        cudaEventElapsedTime(&t, prof.ev[2 * k], prof.ev[2 * k + 1]);
        if (prof.kind[k] == 0) stats->factor_ms += t;
        else { stats->update_ms += t; stats->update_launches++; stats->update_flops += prof.flops[fi++]; }
      }
    }
  }
  *out = F;
  return OOC_OK;
}

extern "C" int ooc_factor_create(ooc_handle* h, const double* A, int64_t n, int64_t lda, int nb, int prec,
                                 ooc_factor** out, int* info, ooc_stats* stats) {
  return create_impl(h, A, n, lda, false, 0, 0.0, nb, prec, out, info, stats);
}

extern "C" int ooc_factor_create_gen(ooc_handle* h, int64_t n, uint64_t seed, double alpha, int nb, int prec,
                                     ooc_factor** out, int* info, ooc_stats* stats) {
  return create_impl(h, nullptr, n, n, true, seed, alpha, nb, prec, out, info, stats);
}

extern "C" int64_t ooc_factor_bytes(int64_t n, int nb, int prec) {
  if (n <= 0 || nb <= 0) return 0;
  const int64_t bb = (n + nb - 1) / nb;
  int64_t b = (int64_t)nb * 16 * 8 + 256;  // tmp, status
  if (prec == OOC_PREC_FP64) return b + n * n * 8 + bb * nb * nb * 8 + n * nb * 8 + (int64_t)nb * nb * 8;
  b += n * n * 4 + bb * nb * nb * 4 + (int64_t)nb * 16 * 4 + 2 * (int64_t)nb * nb * 4;  // Lf, Dinvf, tmpf, scratch
  if (prec == OOC_PREC_BF16X3) {
    const int64_t planes = 2 * ((n + 127) / 128 * 128) * ((nb + 63) / 64 * 64) * 2 + 256;  // hi + lo
    b += planes;
    if (nb % 128 == 0 && n > nb) b += planes + 2 * (int64_t)nb * nb * 2;  // tensor-core column solve
  }
  return b;
}

extern "C" int ooc_factor_destroy(ooc_factor* F) {
  if (!F) return OOC_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(F->device);
  // No device-wide synchronisation: every call that used the factor waited for its own
  // streams before returning, so its buffers are idle and go back to the handle's cache
  // without stalling other pipelines' work.
  delete F;
  cudaSetDevice(prev);
  return OOC_OK;
}

namespace {
__global__ void k_residual_init(const double* B, i64 ldb, double* R, i64 ldr, int n, int r) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int q = 0; q < r; q++) R[i + q * ldr] = B[i + q * ldb];
}
__global__ void k_f32_to_f64_cols(const float* S, i64 lds, double* D, i64 ldd, int n, int r) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int q = 0; q < r; q++) D[i + q * ldd] = ooc_f32_to_f64(S[i + q * lds]);
}
__global__ void k_to_f32_cols(const double* S, i64 lds, float* D, i64 ldd, int n, int r) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int q = 0; q < r; q++) D[i + q * ldd] = ooc_f64_to_f32(S[i + q * lds]);
}
__global__ void k_add_f32_cols(double* X, i64 ldx, const float* D, i64 ldd, int n, int r) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int q = 0; q < r; q++) X[i + q * ldx] += ooc_f32_to_f64(D[i + q * ldd]);
}

double host_max(const std::vector<double>& v, int r, int q, int nb) {
  double m = 0;
  for (int b = 0; b < nb; b++) m = std::max(m, v[(size_t)b * r + q]);
  return m;
}
}  // namespace

extern "C" int ooc_factor_copy_L(ooc_factor* F, double* L, int64_t ldl) {
  if (!F) return -1;
  if (!L) return -2;
  if (ldl < F->n) return -3;
  cudaSetDevice(F->device);
  const i64 n = F->n;
  if (!F->Lf) {
    OOC_CUDA_TRY(cudaMemcpy2D(L, ldl * sizeof(double), F->L, n * sizeof(double), n * sizeof(double), n,
                              cudaMemcpyDefault));
    return OOC_OK;
  }
  // reduced precision: the FP32 factor widened to FP64, zeros above the diagonal, through a
  // staging buffer of column blocks
  cudaPointerAttributes pa{};
  const bool on_device = cudaPointerGetAttributes(&pa, L) == cudaSuccess && pa.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  const unsigned gx = (unsigned)((n + 255) / 256);
  if (on_device) {
    k_lower_conv<float, double><<<dim3(gx, (unsigned)std::min<i64>(n, 1024)), 256>>>(F->Lf, n, L, ldl, n, 0, (int)n, 1);
    OOC_CUDA_TRY(cudaGetLastError());
    OOC_CUDA_TRY(cudaDeviceSynchronize());
    return OOC_OK;
  }
  const int w = (int)std::max<i64>(1, std::min<i64>(n, (256LL << 20) / (8 * n)));
  DevBuf stage;
  int rc = stage.ensure((size_t)n * w * sizeof(double));
  if (rc) return rc;
  for (i64 c0 = 0; c0 < n; c0 += w) {
    const int wc = (int)std::min<i64>(w, n - c0);
    k_lower_conv<float, double><<<dim3(gx, (unsigned)std::min(wc, 1024)), 256>>>(F->Lf + c0 * n, n, (double*)stage.p, n,
                                                                                 n, c0, wc, 1);
    OOC_CUDA_TRY(cudaGetLastError());
    OOC_CUDA_TRY(cudaMemcpy2D(L + c0 * ldl, ldl * sizeof(double), stage.p, n * sizeof(double), n * sizeof(double), wc,
                              cudaMemcpyDeviceToHost));
  }
  return OOC_OK;
}

// Plain solve with the factor: B := A^{-1} B, B on the device (FP64 triangular solves; for a
// reduced-precision factor the solves run in FP32 on a rounded copy of B).
extern "C" int ooc_factor_solve(ooc_handle* h, ooc_factor* F, double* B, int64_t ldb, int nrhs) {
  if (!h) return -1;
  if (!F) return -2;
  if (!B) return -3;
  if (ldb < F->n) return -4;
  if (nrhs < 0 || nrhs > RMAX) return -5;
  if (F->info != 0) return OOC_ERR_UNSUPPORTED;
  if (nrhs == 0) return OOC_OK;
  cudaSetDevice(F->device);
  std::lock_guard<std::mutex> solve_lock(F->solve_mu);
  cudaStream_t s = ooc_compute_stream(h);
  const i64 n = F->n;
  int rc;
  if (F->Lf) {
    rc = F->sws.ensure((size_t)n * RMAX * sizeof(float));
    if (rc) return rc;
    float* bf = (float*)F->sws.p;
    const unsigned gb = (unsigned)((n + 255) / 256);
    k_to_f32_cols<<<gb, 256, 0, s>>>(B, ldb, bf, n, (int)n, nrhs);
    rc = solve_with<float>(F->Lf, n, F->Dinvf, F->panels(), bf, n, nrhs, F->tmpf, s, &F->partf);
    if (!rc) k_f32_to_f64_cols<<<gb, 256, 0, s>>>((const float*)bf, n, B, ldb, (int)n, nrhs);
    if (!rc) rc = ooc_wait_stream(h, s);
    return rc;
  }
  rc = solve_with<double>(F->L, n, F->Dinv, F->panels(), B, ldb, nrhs, F->tmp, s, &F->part);
  if (rc) return rc;
  return ooc_wait_stream(h, s);
}



// B := A^{-1} B with the lower factor L of A as ooc_dpotrf_L leaves it (host or device,
// ld ldl): the forward sweep L Y = B and the backward sweep L^T X = Y over nb-wide column
// panels, each panel's inverse diagonal tile formed on the device (identity, then the
// library's column solve: L_JJ^{-T}), then a small product with the panel below it.  A host
// L is streamed: each sweep copies the panels' lower parts (rows J0..n-1) through two device
// panel buffers on the host-to-device stream, the copy of the next panel beside the
// compute of this one -- the dpotrs of the reference's VERIFY block (oocdag.cpp:436-439)
// with the factor left where the out-of-core factorization put it.
extern "C" int ooc_dpotrs_L(ooc_handle* h, const double* L, int64_t n, int64_t ldl, int nb, size_t dev_budget,
                            double* B, int64_t ldb, int nrhs) {
  if (!h) return -1;
  if (!L && n > 0) return -2;
  if (n < 0) return -3;
  if (ldl < std::max<int64_t>(1, n)) return -4;
  if (nb <= 0) return -5;
  if (!B && n > 0) return -7;
  if (ldb < std::max<int64_t>(1, n)) return -8;
  if (nrhs < 0 || nrhs > RMAX) return -9;
  if (n == 0 || nrhs == 0) return OOC_OK;
  cudaSetDevice(ooc_device(h));
  cudaStream_t s = ooc_compute_stream(h);
  void* scp = nullptr;
  ooc_get_stream(h, 1, &scp);
  cudaStream_t sc = (cudaStream_t)scp;
  auto on_device = [](const void* p) {
    cudaPointerAttributes pa{};
    const bool d = cudaPointerGetAttributes(&pa, p) == cudaSuccess &&
                   (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    return d;
  };
  const bool l_dev = on_device(L), b_dev = on_device(B);
  nb = (int)std::min<i64>(nb, n);
  const int bb = (int)((n + nb - 1) / nb);
  const i64 tile = (i64)nb * nb;
  // workspace: status word, L_JJ^{-T}, nb x RMAX products, B's device copy, two panels
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t b_stat = 256, b_dinv = up(tile * 8), b_tmp = up((size_t)nb * RMAX * 8);
  const size_t b_B = b_dev ? 0 : up((size_t)n * nrhs * 8), b_pan = l_dev ? 0 : up((size_t)n * nb * 8);
  const size_t need = b_stat + b_dinv + b_tmp + b_B + 2 * b_pan;
  if (dev_budget > 0 && need > dev_budget) {
    char buf[200];
    snprintf(buf, sizeof(buf), "ooc_dpotrs_L: n=%lld nb=%d needs %zu device bytes (two panels), budget %zu",
             (long long)n, nb, need, dev_budget);
    ooc_set_last_message(buf);
    return OOC_ERR_BUDGET;
  }
  GrowBuf* ws = ooc_handle_solve_ws(h);
  int rc = ws->ensure(need);
  if (rc) return rc;
  char* base = (char*)ws->p;
  int* status = (int*)base;
  double* D = (double*)(base + b_stat);
  double* tmp = (double*)(base + b_stat + b_dinv);
  double* Bd = b_dev ? B : (double*)(base + b_stat + b_dinv + b_tmp);
  const i64 ldbd = b_dev ? ldb : n;
  double* Pbuf[2] = {nullptr, nullptr};
  if (!l_dev) {
    Pbuf[0] = (double*)(base + b_stat + b_dinv + b_tmp + b_B);
    Pbuf[1] = (double*)((char*)Pbuf[0] + b_pan);
  }
  struct EvGuard {  // copied (per slot), slot free (per slot), inputs ready
    cudaEvent_t e[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    ~EvGuard() { for (cudaEvent_t x : e) if (x) cudaEventDestroy(x); }
  } ev;
  for (cudaEvent_t& x : ev.e) OOC_CUDA_TRY(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
  cudaEvent_t* evc = ev.e;
  cudaEvent_t* evf = ev.e + 2;
  cudaEvent_t ev0 = ev.e[4];
  OOC_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), s));
  if (!b_dev)
    OOC_CUDA_TRY(cudaMemcpy2DAsync(Bd, n * sizeof(double), B, ldb * sizeof(double), n * sizeof(double), nrhs,
                                   cudaMemcpyHostToDevice, s));
  OOC_CUDA_TRY(cudaEventRecord(ev0, s));
  OOC_CUDA_TRY(cudaStreamWaitEvent(sc, ev0, 0));
  auto panel_cols = [&](int J, i64* J0, int* LN) {
    *J0 = (i64)J * nb;
    *LN = (int)std::min<i64>(nb, n - *J0);
  };
  // panel J's lower part on the device: its address and leading dimension
  auto fetch = [&](int J, int slot, int uses) -> int {  // uses: sweeps that used the slot before
    if (l_dev) return OOC_OK;
    i64 J0;
    int LN;
    panel_cols(J, &J0, &LN);
    if (uses > 0) OOC_CUDA_TRY(cudaStreamWaitEvent(sc, evf[slot], 0));
    OOC_CUDA_TRY(cudaMemcpy2DAsync(Pbuf[slot], n * sizeof(double), L + J0 + J0 * ldl, ldl * sizeof(double),
                                   (n - J0) * sizeof(double), LN, cudaMemcpyHostToDevice, sc));
    OOC_CUDA_TRY(cudaEventRecord(evc[slot], sc));
    return OOC_OK;
  };
  int slot_uses[2] = {0, 0};
  for (int sweep = 0; sweep < 2 && !rc; sweep++) {
    // panel order: forward left to right, backward right to left
    auto pj = [&](int t) { return sweep == 0 ? t : bb - 1 - t; };
    if ((rc = fetch(pj(0), 0, slot_uses[0]))) break;
    for (int t = 0; t < bb && !rc; t++) {
      const int J = pj(t), slot = t % 2;
      if (t + 1 < bb && (rc = fetch(pj(t + 1), (t + 1) % 2, slot_uses[(t + 1) % 2]))) break;
      i64 J0;
      int LN;
      panel_cols(J, &J0, &LN);
      const double* Pj;
      i64 ldp;
      if (l_dev) {
        Pj = L + J0 + J0 * ldl;
        ldp = ldl;
      } else {
        OOC_CUDA_TRY(cudaStreamWaitEvent(s, evc[slot], 0));
        Pj = Pbuf[slot];
        ldp = n;
      }
      const i64 rows = n - J0 - LN;
      k_set_identity<double><<<dim3((LN + 255) / 256, std::min(LN, 1024)), 256, 0, s>>>(D, nb, LN);
      rc = launch_trsm_col(Pj, ldp, TileCol{D, nb, tile}, 1, LN, LN, LN, status, s);  // D = L_JJ^{-T}
      if (rc) break;
      if (sweep == 0) {  // y_J = L_JJ^{-1} b_J, then b_below -= L_below y_J
        if (nrhs == 1 && LN <= DMV_WARPS * 32) {
          k_dinv_mv<double, true><<<(LN + 31) / 32, DMV_WARPS * 32, 0, s>>>(D, nb, LN, Bd + J0, tmp);
          OOC_CUDA_TRY(cudaGetLastError());
        } else if ((rc = gemm_tn_small<double, double>(D, nb, Bd + J0, ldbd, tmp, nb, LN, LN, nrhs, 1.0, 0.0, s))) {
          break;
        }
        if (rows > 0) {
          rc = gemm_nn_small<double, double>(Pj + LN, ldp, tmp, nb, Bd + J0 + LN, ldbd, (int)rows, LN, nrhs, -1.0, 1.0,
                                             s, nullptr, CopyOut<double>{tmp, nb, Bd + J0, ldbd, LN});
          if (rc) break;
        } else {
          OOC_CUDA_TRY(cudaMemcpy2DAsync(Bd + J0, ldbd * sizeof(double), tmp, nb * sizeof(double), LN * sizeof(double),
                                         nrhs, cudaMemcpyDeviceToDevice, s));
        }
      } else {  // y_J -= L_below^T x_below, then x_J = L_JJ^{-T} y_J
        if (rows > 0 && (rc = gemm_tn_small<double, double>(Pj + LN, ldp, Bd + J0 + LN, ldbd, Bd + J0, ldbd, LN,
                                                            (int)rows, nrhs, -1.0, 1.0, s)))
          break;
        if (nrhs == 1 && LN <= DMV_WARPS * 32) {
          k_dinv_mv<double, false><<<(LN + 31) / 32, DMV_WARPS * 32, 0, s>>>(D, nb, LN, Bd + J0, tmp);
          OOC_CUDA_TRY(cudaGetLastError());
        } else if ((rc = gemm_nn_small<double, double>(D, nb, Bd + J0, ldbd, tmp, nb, LN, LN, nrhs, 1.0, 0.0, s,
                                                       nullptr))) {
          break;
        }
        OOC_CUDA_TRY(cudaMemcpy2DAsync(Bd + J0, ldbd * sizeof(double), tmp, nb * sizeof(double), LN * sizeof(double),
                                       nrhs, cudaMemcpyDeviceToDevice, s));
      }
      if (!l_dev) {
        OOC_CUDA_TRY(cudaEventRecord(evf[slot], s));
        slot_uses[slot]++;
      }
    }
  }
  if (!rc && !b_dev)
    OOC_CUDA_TRY(cudaMemcpy2DAsync(B, ldb * sizeof(double), Bd, n * sizeof(double), n * sizeof(double), nrhs,
                                   cudaMemcpyDeviceToHost, s));
  const int wrc = ooc_wait_stream(h, s);  // every queued use of the workspace is done
  if (!rc) rc = wrc;
  if (!rc) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      ooc_set_last_error(e, "ooc_dpotrs_L", __FILE__, __LINE__);
      rc = OOC_ERR_CUDA;
    }
  }
  return rc;
}

// Iterative refinement to a normwise backward error <= tol: X0 from the factor in FP64,
// then repeat R = B - A X (FP64), D = A_F^{-1} R with the factor (FP32 copy for a
// reduced-precision factor, FP64 otherwise), X += D.  A is either stored (Astore != null,
// ld lda) or regenerated from the uniform generator (key, alpha) inside the residual.
static int refine_impl(ooc_handle* h, ooc_factor* F, const double* Astore, i64 lda, bool gen, uint64_t key,
                       double alpha, const double* B, i64 ldb, double* X, i64 ldx, int r, double tol, int maxiter,
                       int* iters, double* berr) {
  cudaSetDevice(F->device);
  std::lock_guard<std::mutex> solve_lock(F->solve_mu);
  cudaStream_t s = ooc_compute_stream(h);
  const i64 n = F->n;
  // the residual R (n x RMAX FP64), its FP32 copy, the row sums and the reduction words, in
  // the factor's workspace (sized once for RMAX columns and kept across calls)
  const int nred = 152;
  const size_t bR = (size_t)n * RMAX * sizeof(double), bRf = ((size_t)n * RMAX * sizeof(float) + 255) / 256 * 256;
  const size_t bRows = ((size_t)n * sizeof(double) + 255) / 256 * 256;
  if (F->rws.ensure(bR + bRf + bRows + (size_t)nred * (RMAX + 1) * sizeof(double))) return OOC_ERR_NOMEM;
  double* R = (double*)F->rws.p;
  float* Rf = (float*)((char*)F->rws.p + bR);
  double* rows = (double*)((char*)F->rws.p + bR + bRf);
  double* red = (double*)((char*)F->rws.p + bR + bRf + bRows);
  int rc = OOC_OK;
  // A given on the host: the lower triangle the factor kept (same pointer and lda), else
  // a device copy of the lower triangle, column block by column block.
  double* Atmp = nullptr;
  if (!gen) {
    cudaPointerAttributes pa{};
    const bool on_device = cudaPointerGetAttributes(&pa, Astore) == cudaSuccess && pa.type == cudaMemoryTypeDevice;
    cudaGetLastError();
    if (!on_device) {
      if (F->A64 && Astore == F->A64_src && lda == F->A64_lda) {
        Astore = F->A64;
        lda = n;
      } else if (F->alloc(&Atmp, (size_t)n * n * sizeof(double))) {
        rc = OOC_ERR_NOMEM;
      } else {
        const i64 w = std::max<i64>(1, std::min<i64>(n, (256LL << 20) / (8 * n)));
        for (i64 c0 = 0; !rc && c0 < n; c0 += w) {
          const i64 wc = std::min<i64>(w, n - c0);
          if (cudaMemcpy2DAsync(Atmp + c0 + c0 * n, n * sizeof(double), Astore + c0 + c0 * lda, lda * sizeof(double),
                                (n - c0) * sizeof(double), wc, cudaMemcpyHostToDevice, s) != cudaSuccess)
            rc = OOC_ERR_CUDA;
        }
        Astore = Atmp;
        lda = n;
      }
    }
  }
  std::vector<double> hv((size_t)nred * r);
  const unsigned gb = (unsigned)((n + 255) / 256);
  // column slices of the generated products (enough CTAs to fill the GPU)
  const int gslices = std::max(1, std::min((int)((n + 1023) / 1024), (int)((4 * 304 + gb - 1) / gb)));
  const int gks = (int)((n + gslices - 1) / gslices);
  auto colmax = [&](const double* V, i64 ld, int cols, std::vector<double>& out) -> int {
    k_colmax_abs<<<nred, 256, 0, s>>>(V, ld, (int)n, cols, red);
    OOC_CUDA_TRY(cudaMemcpyAsync(hv.data(), red, (size_t)nred * cols * sizeof(double), cudaMemcpyDeviceToHost, s));
    int e = ooc_wait_stream(h, s);
    if (e) return e;
    out.assign(cols, 0.0);
    for (int q = 0; q < cols; q++) out[q] = host_max(hv, cols, q, nred);
    return OOC_OK;
  };
  // The FP32 triangular solve on Rf is ~4 launches per block step: captured once into a
  // CUDA graph and replayed for X0 and every correction (launch-bound otherwise).
  cudaGraphExec_t solve_graph = nullptr;
  bool graph_failed = false;
  auto solve32 = [&]() -> int {
    if (!solve_graph && !graph_failed) {
      cudaGraph_t g = nullptr;
      int crc = OOC_OK;
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        crc = OOC_ERR_CUDA;
      } else {
        crc = solve_with<float>(F->Lf, n, F->Dinvf, F->panels(), Rf, n, r, F->tmpf, s, nullptr);
        if (cudaStreamEndCapture(s, &g) != cudaSuccess) crc = OOC_ERR_CUDA;
      }
      if (!crc && cudaGraphInstantiate(&solve_graph, g, 0) != cudaSuccess) {
        solve_graph = nullptr;
        crc = OOC_ERR_CUDA;
      }
      if (g) cudaGraphDestroy(g);
      if (crc) {  // capture not available: launch directly from now on
        cudaGetLastError();
        graph_failed = true;
      }
    }
    if (solve_graph) return cudaGraphLaunch(solve_graph, s) == cudaSuccess ? OOC_OK : OOC_ERR_CUDA;
    return solve_with<float>(F->Lf, n, F->Dinvf, F->panels(), Rf, n, r, F->tmpf, s, &F->partf);
  };
  // ||A||_inf
  // ||A||_inf on the handle's second stream, beside X0's solve (a chain of small launches
  // that leaves most of the GPU idle): row sums into `rows`, their maximum per CTA into
  // the last nred words of `red`, read once X0 has been issued.
  double normA = 0;
  double* red_norm = red + (size_t)nred * r;
  cudaStream_t s2 = s;
  {
    void* p2 = nullptr;
    if (ooc_get_stream(h, 1, &p2) == OOC_OK && p2) s2 = (cudaStream_t)p2;
  }
  cudaEvent_t ev_in = nullptr;
  if (!rc && s2 != s) {
    if (cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming) != cudaSuccess || cudaEventRecord(ev_in, s) != cudaSuccess ||
        cudaStreamWaitEvent(s2, ev_in, 0) != cudaSuccess)
      rc = OOC_ERR_CUDA;
  }
  if (!rc) {
    if (gen) {
      rc = F->part2.ensure((size_t)gslices * n * sizeof(double));
      if (!rc) {
        k_rowsum_gen<<<dim3(gb, gslices), 256, 0, s2>>>(key, n, alpha, gks, (double*)F->part2.p);
        k_sum_slices_rows<<<gb, 256, 0, s2>>>((const double*)F->part2.p, gslices, n, rows);
      }
    } else {  // |A| 1 from the lower triangle
      rc = symv_lower(true, Astore, lda, nullptr, 0, rows, n, (int)n, 1, 1.0, 0.0, s2, F->part2);
    }
    if (!rc) k_colmax_abs<<<nred, 256, 0, s2>>>(rows, n, (int)n, 1, red_norm);
  }
  std::vector<double> nb_(r), nx(r), nr(r);
  if (!rc) rc = colmax(B, ldb, r, nb_);
  if (!rc && F->Lf) {  // X0 from the FP32 factor
    k_to_f32_cols<<<gb, 256, 0, s>>>(B, ldb, Rf, n, (int)n, r);
    rc = solve32();
    if (!rc) k_f32_to_f64_cols<<<gb, 256, 0, s>>>(Rf, n, X, ldx, (int)n, r);
  } else if (!rc) {  // (no early return: the buffers above are freed at the end)
    const cudaError_t e = cudaMemcpy2DAsync(X, ldx * sizeof(double), B, ldb * sizeof(double), n * sizeof(double), r,
                                            cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) {
      ooc_set_last_error(e, "cudaMemcpy2DAsync (X := B)", __FILE__, __LINE__);
      rc = OOC_ERR_CUDA;
    } else {
      rc = solve_with<double>(F->L, n, F->Dinv, F->panels(), X, ldx, r, F->tmp, s, &F->part);
    }
  }
  if (!rc) rc = ooc_wait_stream(h, s2);
  if (!rc) {
    std::vector<double> hn(nred);
    if (cudaMemcpy(hn.data(), red_norm, (size_t)nred * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = OOC_ERR_CUDA;
    for (int b = 0; !rc && b < nred; b++) normA = std::max(normA, hn[b]);
  }
  int it = 0;
  double be = 0;
  while (!rc) {
    // R = B - A X (FP64)
    k_residual_init<<<gb, 256, 0, s>>>(B, ldb, R, n, (int)n, r);
    if (gen) {
      rc = F->part.ensure((size_t)gslices * n * r * sizeof(double));
      if (rc) break;
      NN_DISPATCH(r, (k_resid_gen<RR><<<dim3(gb, gslices), 256, 0, s>>>(key, n, alpha, X, ldx, r, gks,
                                                                         (double*)F->part.p)));
      k_reduce_slices<double><<<gb, 256, 0, s>>>((const double*)F->part.p, gslices, R, n, (int)n, r, -1.0, 1.0);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) { ooc_set_last_error(e, "generated residual", __FILE__, __LINE__); rc = OOC_ERR_CUDA; break; }
    } else {
      rc = symv_lower(false, Astore, lda, X, ldx, R, n, (int)n, r, -1.0, 1.0, s, F->part);
      if (rc) break;
    }
    rc = colmax(R, n, r, nr);
    if (rc) break;
    rc = colmax(X, ldx, r, nx);
    if (rc) break;
    be = 0;
    for (int q = 0; q < r; q++) {
      const double den = normA * nx[q] + nb_[q];
      be = std::max(be, den > 0 ? nr[q] / den : 0.0);
    }
    if (be <= tol || it >= maxiter) break;
    if (F->Lf) {
      k_to_f32_cols<<<gb, 256, 0, s>>>(R, n, Rf, n, (int)n, r);
      rc = solve32();
      if (rc) break;
      k_add_f32_cols<<<gb, 256, 0, s>>>(X, ldx, Rf, n, (int)n, r);
    } else {
      rc = solve_with<double>(F->L, n, F->Dinv, F->panels(), R, n, r, F->tmp, s, &F->part);
      if (rc) break;
      k_axpy_cols<<<gb, 256, 0, s>>>(X, ldx, R, n, (int)n, r);
    }
    it++;
  }
  if (!rc) rc = ooc_wait_stream(h, s);
  if (s2 != s) cudaStreamSynchronize(s2);  // the norm's buffers may go now
  if (ev_in) cudaEventDestroy(ev_in);
  if (solve_graph) cudaGraphExecDestroy(solve_graph);
  if (Atmp) {
    cudaStreamSynchronize(s);
    F->release(Atmp);
  }
  if (rc) return rc;
  if (iters) *iters = it;
  if (berr) *berr = be;
  return OOC_OK;
}

// Normwise backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) of one
// solution x (device) of A x = b (device) for the uniform test matrix of `seed` and alpha,
// with A regenerated inside the residual and the norm (no copy of A).  For solutions
// computed without a factor object (the out-of-core path of the serving runtime).
int ooc_seeded_backward_error(ooc_handle* h, int64_t n, uint64_t seed, double alpha, const double* B, const double* X,
                              double* berr) {
  cudaSetDevice(ooc_device(h));
  cudaStream_t s = ooc_compute_stream(h);
  const uint64_t key = ooc_uniform_key(seed);
  const unsigned gb = (unsigned)((n + 255) / 256);
  const int gslices = std::max(1, std::min((int)((n + 1023) / 1024), (int)((4 * 304 + gb - 1) / gb)));
  const int gks = (int)((n + gslices - 1) / gslices);
  const int nred = 152;
  GrowBuf* ws = ooc_handle_solve_ws(h);
  const size_t bvec = ((size_t)n * 8 + 255) / 256 * 256;
  int rc = ws->ensure(2 * bvec + (size_t)gslices * n * 8 + (size_t)nred * 3 * 8);
  if (rc) return rc;
  double* R = (double*)ws->p;
  double* rows = (double*)((char*)ws->p + bvec);
  double* part = (double*)((char*)ws->p + 2 * bvec);
  double* red = part + (size_t)gslices * n;
  k_residual_init<<<gb, 256, 0, s>>>(B, n, R, n, (int)n, 1);
  k_resid_gen<1><<<dim3(gb, gslices), 256, 0, s>>>(key, n, alpha, X, n, 1, gks, part);
  k_reduce_slices<double><<<gb, 256, 0, s>>>(part, gslices, R, n, (int)n, 1, -1.0, 1.0);
  k_rowsum_gen<<<dim3(gb, gslices), 256, 0, s>>>(key, n, alpha, gks, part);
  k_sum_slices_rows<<<gb, 256, 0, s>>>(part, gslices, n, rows);
  k_colmax_abs<<<nred, 256, 0, s>>>(R, n, (int)n, 1, red);
  k_colmax_abs<<<nred, 256, 0, s>>>(X, n, (int)n, 1, red + nred);
  k_colmax_abs<<<nred, 256, 0, s>>>(B, n, (int)n, 1, red + 2 * nred);
  k_colmax_abs<<<nred, 256, 0, s>>>(rows, n, (int)n, 1, red + 3 * nred);
  OOC_CUDA_TRY(cudaGetLastError());
  std::vector<double> hv((size_t)nred * 4);
  OOC_CUDA_TRY(cudaMemcpyAsync(hv.data(), red, hv.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  rc = ooc_wait_stream(h, s);
  if (rc) return rc;
  double m[4] = {0, 0, 0, 0};
  for (int k = 0; k < 4; k++)
    for (int b = 0; b < nred; b++) m[k] = std::max(m[k], hv[(size_t)k * nred + b]);
  const double den = m[3] * m[1] + m[2];
  *berr = den > 0 ? m[0] / den : 0.0;
  return OOC_OK;
}

extern "C" int ooc_solve_refine(ooc_handle* h, ooc_factor* F, const double* A, int64_t lda, const double* B,
                                int64_t ldb, double* X, int64_t ldx, int nrhs, double tol, int maxiter, int* iters,
                                double* berr) {
  if (!h) return -1;
  if (!F) return -2;
  if (!A) return -3;
  if (lda < F->n) return -4;
  if (!B) return -5;
  if (ldb < F->n) return -6;
  if (!X) return -7;
  if (ldx < F->n) return -8;
  if (nrhs <= 0 || nrhs > RMAX) return -9;
  if (F->info != 0) return OOC_ERR_UNSUPPORTED;
  return refine_impl(h, F, A, lda, false, 0, 0.0, B, ldb, X, ldx, nrhs, tol, maxiter, iters, berr);
}

extern "C" int ooc_solve_refine_gen(ooc_handle* h, ooc_factor* F, uint64_t seed, double alpha, const double* B,
                                    int64_t ldb, double* X, int64_t ldx, int nrhs, double tol, int maxiter,
                                    int* iters, double* berr) {
  if (!h) return -1;
  if (!F) return -2;
  if (!B) return -5;
  if (ldb < F->n) return -6;
  if (!X) return -7;
  if (ldx < F->n) return -8;
  if (nrhs <= 0 || nrhs > RMAX) return -9;
  if (F->info != 0) return OOC_ERR_UNSUPPORTED;
  return refine_impl(h, F, nullptr, 0, true, ooc_uniform_key(seed), alpha, B, ldb, X, ldx, nrhs, tol, maxiter, iters,
                     berr);
}

extern "C" int ooc_gen_normal(ooc_handle* h, double* B, int64_t n, int64_t ldb, int nrhs, uint64_t seed) {
  if (!h) return -1;
  if (!B && n > 0) return -2;
  if (n < 0) return -3;
  if (ldb < std::max<int64_t>(1, n)) return -4;
  if (nrhs < 0) return -5;
  if (n == 0 || nrhs == 0) return OOC_OK;
  cudaSetDevice(ooc_device(h));
  cudaStream_t s = ooc_compute_stream(h);
  k_gen_normal<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(B, ldb, n, nrhs, ooc_uniform_key(seed));
  OOC_CUDA_TRY(cudaGetLastError());
  return ooc_wait_stream(h, s);
}

// C (lower, n x n, device) := C - A A^T with A (n x k, device), trailing-update kernels of
// the given precision.  The dsyrk('L','N', alpha=-1, beta=1) task body of the reference
// (oocquark.cpp:176), exposed as a tile call.
extern "C" int ooc_dsyrk_ln(ooc_handle* h, int prec, int n, int k, const double* A, int64_t lda, double* C,
                            int64_t ldc) {
  if (!h) return -1;
  if (prec != OOC_PREC_FP64 && prec != OOC_PREC_FP32 && prec != OOC_PREC_BF16X3) return -2;
  if (n < 0) return -3;
  if (k < 0) return -4;
  if (!A && n > 0) return -5;
  if (lda < std::max(1, n)) return -6;
  if (!C && n > 0) return -7;
  if (ldc < std::max(1, n)) return -8;
  if (n == 0 || k == 0) return OOC_OK;
  cudaSetDevice(ooc_device(h));
  cudaStream_t s = ooc_compute_stream(h);
  int* status = nullptr;
  if (cudaMalloc(&status, sizeof(int)) != cudaSuccess) { cudaGetLastError(); return OOC_ERR_NOMEM; }
  cudaMemsetAsync(status, 0, sizeof(int), s);
  DevBuf work;
  int rc;
  if (prec == OOC_PREC_FP64) {
    rc = launch_gemm_nt(A, lda, A, lda, C, ldc, n, n, k, 1, -1.0, status, s);
  } else {
    rc = syrk_lowprec(prec, A, lda, C, ldc, n, k, status, s, work);
  }
  int st = 0;
  if (!rc) rc = read_int(status, &st, s);
  if (!rc) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { ooc_set_last_error(e, "ooc_dsyrk_ln", __FILE__, __LINE__); rc = OOC_ERR_CUDA; }
  }
  cudaFree(status);
  if (rc) return rc;
  return st == 0 ? OOC_OK : OOC_ERR_TIMEOUT;
}

// ---------------------------------------------------------------------------------
// FP32 Cholesky of a caller's matrix, in place (the reference has no FP32 entry): the
// reduced-precision factor pipeline with FP32 trailing updates (k_syrk_f32), on the
// matrix itself (device) or on a device copy of it (host, when it fits in dev_budget).
// ---------------------------------------------------------------------------------
namespace {
// FP32 lower Cholesky of a HOST matrix through `budget` device bytes: the reference's
// left-looking panel loop (oocdag.cpp:59-87) with panels of W columns (W from the budget:
// the panel and two copies of earlier columns, each n x W floats).  Per panel, on the
// compute stream s: the panel's lower part arrives (copy stream sc), every earlier panel's
// columns arrive W at a time through two X buffers and update it (FP32 k_syrk_f32 restricted
// to the panel's columns: the A2X + ooc_syrk tasks, oocquark.cpp:301-356), then the panel is
// factored in core right-looking (FP32 diagonal tile, column solve, updates inside the
// panel: ooc_incore, oocquark.cpp:358-421) and copied back (stream sd) before any later
// panel reads its columns from the host.
int spotrf_host_ooc(ooc_handle* h, float* A, i64 n, i64 lda, int nb, size_t budget, int* info, ooc_stats* stats) {
  const i64 W = (i64)(budget / ((size_t)3 * n * sizeof(float))) / nb * nb;
  if (W < nb) {
    char buf[200];
    snprintf(buf, sizeof(buf), "ooc_spotrf_L: budget %zu bytes below one panel (3 n nb floats = %zu)", budget,
             (size_t)3 * n * nb * sizeof(float));
    ooc_set_last_message(buf);
    return OOC_ERR_BUDGET;
  }
  cudaStream_t s = ooc_compute_stream(h);
  void *p1 = nullptr, *p2 = nullptr;
  ooc_get_stream(h, 1, &p1);
  ooc_get_stream(h, 2, &p2);
  cudaStream_t sc = (cudaStream_t)p1, sd = (cudaStream_t)p2;
  auto pool = ooc_handle_pool(h);
  DevBuf Pb, Xb[2], work, aux;
  for (DevBuf* b : {&Pb, &Xb[0], &Xb[1], &work, &aux}) b->pool = pool.get();
  const i64 tile = (i64)nb * nb;
  int rc;
  if ((rc = Pb.ensure((size_t)n * W * sizeof(float))) || (rc = Xb[0].ensure((size_t)n * W * sizeof(float))) ||
      (rc = Xb[1].ensure((size_t)n * W * sizeof(float))) ||
      (rc = aux.ensure((size_t)2 * tile * sizeof(float) + 256)))
    return rc;
  float* P = (float*)Pb.p;
  float* Dinv = (float*)aux.p;      // the diagonal kernel's inverse output (not kept)
  float* Xr = Dinv + tile;          // L_jj^{-1}, row-major, for the column solve
  int* status = (int*)(Xr + tile);
  OOC_CUDA_TRY(cudaFuncSetAttribute(k_diag_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DG_SMEM));
  OOC_CUDA_TRY(cudaFuncSetAttribute(k_diag_s256, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DS_SMEM));
  struct Ev {
    cudaEvent_t e[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    ~Ev() { for (cudaEvent_t x : e) if (x) cudaEventDestroy(x); }
  } ev;
  for (cudaEvent_t& x : ev.e) OOC_CUDA_TRY(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
  cudaEvent_t evPin = ev.e[0], evPdone = ev.e[1], evPfree = ev.e[2], evXin[2] = {ev.e[3], ev.e[4]},
              evXfree[2] = {ev.e[5], ev.e[6]};
  cudaEvent_t t0, t1;
  OOC_CUDA_TRY(cudaEventCreate(&t0));
  OOC_CUDA_TRY(cudaEventCreate(&t1));
  struct T2 {
    cudaEvent_t a, b;
    ~T2() { cudaEventDestroy(a); cudaEventDestroy(b); }
  } tguard{t0, t1};
  OOC_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), s));
  OOC_CUDA_TRY(cudaEventRecord(t0, s));
  OOC_CUDA_TRY(cudaEventRecord(evPfree, s));  // the panel buffer is free
  int xuses[2] = {0, 0}, xslot = 0;
  double h2d = 0, d2h = 0;
  int64_t launches = 0;
  int npanels = 0;
  for (i64 J0 = 0; J0 < n; J0 += W, npanels++) {
    const i64 Wp = std::min(W, n - J0), m = n - J0;
    // the panel's lower part (A2Y)
    OOC_CUDA_TRY(cudaStreamWaitEvent(sc, evPfree, 0));
    OOC_CUDA_TRY(cudaMemcpy2DAsync(P, n * sizeof(float), A + J0 + J0 * lda, lda * sizeof(float), m * sizeof(float),
                                   Wp, cudaMemcpyHostToDevice, sc));
    OOC_CUDA_TRY(cudaEventRecord(evPin, sc));
    h2d += (double)m * Wp * 4;
    OOC_CUDA_TRY(cudaStreamWaitEvent(s, evPin, 0));
    const int bjp = (int)((Wp + 127) / 128);
    // left-looking: the finished columns [K0, K0 + Kw), rows J0..n-1 (A2X + ooc_syrk)
    for (i64 K0 = 0; K0 < J0; K0 += W) {
      const i64 Kw = std::min(W, J0 - K0);
      const int sl = xslot;
      xslot ^= 1;
      if (xuses[sl]) OOC_CUDA_TRY(cudaStreamWaitEvent(sc, evXfree[sl], 0));
      float* X = (float*)Xb[sl].p;
      OOC_CUDA_TRY(cudaMemcpy2DAsync(X, n * sizeof(float), A + J0 + K0 * lda, lda * sizeof(float), m * sizeof(float),
                                     Kw, cudaMemcpyHostToDevice, sc));
      OOC_CUDA_TRY(cudaEventRecord(evXin[sl], sc));
      h2d += (double)m * Kw * 4;
      OOC_CUDA_TRY(cudaStreamWaitEvent(s, evXin[sl], 0));
      if ((rc = syrk_f32(OOC_PREC_FP32, X, n, P, n, (int)m, (int)Kw, status, s, work, 0, bjp))) return rc;
      OOC_CUDA_TRY(cudaEventRecord(evXfree[sl], s));
      xuses[sl]++;
      launches++;
    }
    // in-core factorization of the panel, right-looking inside it (ooc_incore)
    for (i64 q0 = 0; q0 < Wp; q0 += nb) {
      const int LN = (int)std::min<i64>(nb, Wp - q0);
      float* Djj = P + q0 + q0 * n;
      if (LN <= DS_MAX)
        k_diag_s256<<<1, DG_THREADS, DS_SMEM, s>>>(Djj, n, LN, J0 + q0, Dinv, LN, Xr, nullptr, nullptr, status);
      else
        k_diag_f32<<<1, DG_THREADS, DG_SMEM, s>>>(Djj, n, LN, J0 + q0, Dinv, LN, Xr, nullptr, nullptr, status);
      OOC_CUDA_TRY(cudaGetLastError());
      const i64 mq = m - q0 - LN;
      launches++;
      if (mq <= 0) continue;
      float* Pn = Djj + LN;
      k_colsolve_f32<<<(unsigned)((mq + CS_ROWS - 1) / CS_ROWS), FTHR, 0, s>>>(Pn, n, Xr, LN, (int)mq, LN, status);
      OOC_CUDA_TRY(cudaGetLastError());
      launches++;
      const i64 wrest = Wp - q0 - LN;  // the panel's columns right of this step
      if (wrest > 0) {
        if ((rc = syrk_f32(OOC_PREC_FP32, Pn, n, Pn + LN * n, n, (int)mq, LN, status, s, work, 0,
                           (int)((wrest + 127) / 128))))
          return rc;
        launches++;
      }
    }
    // the factored panel back to the host (Y2A), before later panels read its columns
    OOC_CUDA_TRY(cudaEventRecord(evPdone, s));
    OOC_CUDA_TRY(cudaStreamWaitEvent(sd, evPdone, 0));
    OOC_CUDA_TRY(cudaMemcpy2DAsync(A + J0 + J0 * lda, lda * sizeof(float), P, n * sizeof(float), m * sizeof(float), Wp,
                                   cudaMemcpyDeviceToHost, sd));
    OOC_CUDA_TRY(cudaEventRecord(evPfree, sd));
    d2h += (double)m * Wp * 4;
  }
  OOC_CUDA_TRY(cudaStreamWaitEvent(s, evPfree, 0));
  OOC_CUDA_TRY(cudaEventRecord(t1, s));
  int st = 0;
  if ((rc = read_int(status, &st, s))) return rc;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ooc_set_last_error(e, "ooc_spotrf_L (out of core)", __FILE__, __LINE__);
    return OOC_ERR_CUDA;
  }
  *info = st;
  if (stats) {
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    stats->seconds = ms * 1e-3;
    stats->flops = (double)n * n * n / 3.0;
    stats->npanels = npanels;
    stats->info = st;
    stats->kernel_launches = launches;
    stats->h2d_bytes = h2d;
    stats->d2h_bytes = d2h;
  }
  return OOC_OK;
}
}  // namespace

extern "C" int ooc_spotrf_L(ooc_handle* h, float* A, int64_t n, int64_t lda, int nb, size_t dev_budget, int* info,
                            ooc_stats* stats) {
  if (!h) return -1;
  if (!A && n > 0) return -2;
  if (n < 0) return -3;
  if (lda < std::max<int64_t>(1, n)) return -4;
  if (nb <= 0 || nb > DG_MAX) return -5;
  if (!info) return -7;
  *info = 0;
  if (stats) memset(stats, 0, sizeof(*stats));
  if (n == 0) return OOC_OK;
  cudaSetDevice(ooc_device(h));
  cudaStream_t s = ooc_compute_stream(h);
  cudaPointerAttributes pa{};
  const bool on_device = cudaPointerGetAttributes(&pa, A) == cudaSuccess && pa.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  ooc_factor F;
  F.device = ooc_device(h);
  F.n = n;
  F.nb = nb;
  F.prec = OOC_PREC_FP32;
  F.owns_Lf = on_device ? false : true;
  const int bb = (int)((n + nb - 1) / nb);
  if (on_device) {
    F.Lf = A;
    F.ld = lda;
  } else {
    const size_t bytes = (size_t)n * n * sizeof(float);
    size_t budget = dev_budget;
    if (budget == 0) {
      size_t fr = 0, tot = 0;
      cudaMemGetInfo(&fr, &tot);
      budget = fr / 4 * 3;
    }
    if (bytes > budget)  // out of core: left-looking panels streamed through the budget
      return spotrf_host_ooc(h, A, n, lda, nb, budget, info, stats);
    if (cudaMalloc(&F.Lf, bytes) != cudaSuccess) { cudaGetLastError(); F.Lf = nullptr; return OOC_ERR_NOMEM; }
    F.ld = n;
    OOC_CUDA_TRY(cudaMemcpy2DAsync(F.Lf, n * sizeof(float), A, lda * sizeof(float), n * sizeof(float), n,
                                   cudaMemcpyHostToDevice, s));
  }
  if (cudaMalloc(&F.Dinvf, (size_t)bb * nb * nb * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&F.status, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return OOC_ERR_NOMEM;
  }
  OOC_CUDA_TRY(cudaMemsetAsync(F.status, 0, sizeof(int), s));
  cudaEvent_t e0, e1;
  OOC_CUDA_TRY(cudaEventCreate(&e0));
  OOC_CUDA_TRY(cudaEventCreate(&e1));
  OOC_CUDA_TRY(cudaEventRecord(e0, s));
  void* s1p = nullptr;
  ooc_get_stream(h, 1, &s1p);
  MixedProf prof;
  int64_t launches = 0;
  int rc = factor_f32(&F, OOC_PREC_FP32, s, (cudaStream_t)s1p, &launches, &prof);
  if (!rc) rc = cudaEventRecord(e1, s) == cudaSuccess ? OOC_OK : OOC_ERR_CUDA;
  int st = 0;
  if (!rc) rc = read_int(F.status, &st, s);
  if (!rc && !on_device)
    rc = cudaMemcpy2D(A, lda * sizeof(float), F.Lf, n * sizeof(float), n * sizeof(float), n, cudaMemcpyDeviceToHost) ==
                 cudaSuccess ? OOC_OK : OOC_ERR_CUDA;
  if (!rc) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { ooc_set_last_error(e, "ooc_spotrf_L", __FILE__, __LINE__); rc = OOC_ERR_CUDA; }
  }
  float ms = 0;
  if (!rc) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  *info = st;
  if (stats) {
    stats->seconds = ms * 1e-3;
    stats->flops = (double)n * n * n / 3.0;
    stats->npanels = 1;
    stats->info = st;
    stats->kernel_launches = launches;
    stats->h2d_bytes = on_device ? 0.0 : (double)n * n * 4;
    stats->d2h_bytes = on_device ? 0.0 : (double)n * n * 4;
  }
  return OOC_OK;
}
