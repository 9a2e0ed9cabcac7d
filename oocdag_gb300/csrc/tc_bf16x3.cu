// Split-BF16 tensor-core kernels on Blackwell (tcgen05 + TMA + TMEM) for the mixed path:
//   k_split_bf16        hi/lo BF16 planes of a column panel (K-major);
//   k_syrk_bf16x3<TC>   trailing update C (lower) -= X X^T in 128 x 128 blocks with a
//                       read-modify-write epilogue: FP64 C, and FP32 C whose base or
//                       leading dimension is not 16-byte aligned;
//   k_syrk2_bf16x3<TC>  the same for 16-byte-aligned FP32 C (the working matrix of
//                       reduced-precision factors) in 256 x 128 blocks, C updated by TMA
//                       reductions, blocks taken from a run-time ticket counter;
//   k_syrk2t_bf16x3     the same update for long K (the left-looking catch-ups), issued
//                       as N=256 MMAs with C transposed in TMEM, fed by four 48 KB stages
//                       of K = 32 (64-byte swizzle);
//   k_trsm2_bf16x3      the column solve P = U X^T with the same three products.
// Each kernel's own comment gives its layout; the 128 x 128 update is described here.
//
//   C (FP64, lower triangle) -= X X^T,   X = m x K (FP64, column-major)
//
// X is split once per update into BF16 hi/lo planes (x = hi + lo + O(2^-17 |x|)), stored
// K-major (each row's K values contiguous) so that TMA can stage 128 x 64 tiles with the
// 128-byte swizzle the tensor core reads.  For every 128 x 128 block of the lower
// triangle the kernel accumulates, in TMEM (FP32),
//     D = sum_k  Ahi Bhi^T + Ahi Blo^T + Alo Bhi^T
// with tcgen05.mma kind::f16 (M=128, N=128, K=16) and subtracts D from the FP64 block.
//
// Persistent and warp-specialised: one CTA per SM walks the blocks in strips of 16 block
// columns (row by row inside a strip, so the strip's B operands stay in L2 and each A
// operand is reused by up to 16 consecutive blocks).  Warp 0 issues the TMA loads into a
// three-stage ring, warp 1 (one elected thread) issues the MMAs into one of two TMEM
// accumulators, and sixteen epilogue warps drain the other accumulator (tcgen05.ld) and do
// the FP64 read-modify-write of C, so the HBM traffic of one block overlaps the MMAs of
// the next.
//
// Every mbarrier wait is bounded.  A wait that runs out records an error code in the
// status word (so every later kernel of the factorization returns at once), raises a
// CTA-wide abort flag that ends every other role's loop, waits (bounded) for the MMAs and
// TMA loads already issued, frees its TMEM and returns.

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "common.cuh"

namespace {

constexpr int TB = 128;        // output block (rows = cols)
constexpr int TK = 64;         // K per stage: 64 bf16 = one 128-byte swizzle row
constexpr int STAGES = 3;
constexpr int PLANE_BYTES = TB * TK * 2;          // 16 KB: one 128 x 64 bf16 tile
constexpr int STAGE_BYTES = 4 * PLANE_BYTES;      // Ahi, Alo, Bhi, Blo
constexpr int NACC = 2;                           // TMEM accumulators (double buffer)
constexpr int TMEM_COLS = NACC * TB;
constexpr int EPI_WARPS = 16;                     // four per TMEM lane quadrant (32 columns each)
constexpr int THREADS = 64 + 32 * EPI_WARPS;      // producer warp, MMA warp, epilogue
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
// barriers, TMEM address and abort flag must end before the two counters at offset 128
static_assert((2 * STAGES + 2 * NACC + 1) * 8 + 8 <= 128, "control block overflow");
constexpr int STRIP = 16;                         // block columns per scheduling strip
constexpr long long WAIT_LIMIT = 1LL << 22;       // polls before a wait is declared stuck
constexpr int ERR_TIMEOUT_CODE = -1000003;        // status value written on a stuck wait

// --------------------------------- PTX helpers -----------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// Bounded parity wait: true when the phase with `parity` has completed; false when the
// poll limit runs out or another role raised the CTA's abort flag.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, const volatile int* abort_flag) {
  const uint32_t a = smem_u32(bar);
  for (long long i = 0; i < WAIT_LIMIT; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (abort_flag && *abort_flag) return false;
  }
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];\n" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

// C (global, FP32) += box at smem `src`, added in L2 (TMA reduction); coordinates are
// (row, column) of the box's first element, rows innermost.
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap* map, const void* src, int c0, int c1) {
  asm volatile("cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.bulk_group [%0, {%2, %3}], [%1];\n" ::"l"(
                   (uint64_t)map),
               "r"(smem_u32(src)), "r"(c0), "r"(c1)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// the bulk groups committed so far, all but the newest N, have finished reading shared memory
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ void named_bar_sync(uint32_t id, uint32_t count) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(count) : "memory");
}
// barrier over `count` threads that also returns the AND of their predicates
__device__ __forceinline__ bool named_bar_and(uint32_t id, uint32_t count, bool p) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred a, b;\n setp.ne.u32 a, %1, 0;\n bar.red.and.pred b, %2, %3, a;\n selp.u32 %0, 1, 0, b;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)p), "r"(id), "r"(count)
      : "memory");
  return r != 0;
}

// Shared-memory matrix descriptor: K-major operand in 128-byte-swizzled atoms of
// 8 rows x 128 bytes (stride between atoms 1024 bytes).
__device__ __forceinline__ uint64_t umma_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);          // start address
  d |= (uint64_t)(16 >> 4) << 16;                   // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                 // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                           // fixed 0b001
  d |= (uint64_t)2 << 61;                           // 128-byte swizzle
  return d;
}

// Instruction descriptor: kind::f16 with BF16 A/B, FP32 D, both K-major, M=128, N=128.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TB >> 3) << 17) | ((uint32_t)(TB >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(IDESC), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
               : "memory");
}

// ------------------------------------ kernels ------------------------------------
// Split: X (m x K, FP64 or FP32, column-major) -> hi/lo planes (Mp x Kp BF16, row-major,
// zero pad).  FP32 input stays on the FP32 pipe (x - hi is exact in FP32).
template <typename TX>
__global__ void k_split_bf16(const TX* __restrict__ X, i64 ldx, __nv_bfloat16* __restrict__ hi,
                             __nv_bfloat16* __restrict__ lo, int m, int K, int Mp, int Kp) {
  __shared__ TX t[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  // read 32 x 32 (rows r0.., cols k0..) coalesced along rows
  for (int c = threadIdx.y; c < 32; c += blockDim.y) {
    const int r = r0 + threadIdx.x, k = k0 + c;
    t[c][threadIdx.x] = (r < m && k < K) ? X[r + (i64)k * ldx] : TX(0);
  }
  __syncthreads();
  // write rows, coalesced along k
  for (int rr = threadIdx.y; rr < 32; rr += blockDim.y) {
    const int r = r0 + rr, k = k0 + threadIdx.x;
    if (r < Mp && k < Kp) {
      const TX x = t[threadIdx.x][rr];
      __nv_bfloat16 h, l;
      if constexpr (sizeof(TX) == 4) {
        h = __float2bfloat16_rn(x);
        l = __float2bfloat16_rn(x - __bfloat162float(h));
      } else {
        h = __double2bfloat16(x);
        l = __double2bfloat16(x - (double)__bfloat162float(h));
      }
      hi[(i64)r * Kp + k] = h;
      lo[(i64)r * Kp + k] = l;
    }
  }
}

// Block t of the lower-triangular block range [bj_lo, bj_hi) x rows (up to T), in strip
// order: strips of STRIP block columns, and inside a strip row by row (the first rows of
// a strip form its triangle).  Same set of blocks as ooc_lower_block_decode, other order.
__device__ __forceinline__ void strip_block_decode(i64 t, int T, int bj_lo, int bj_hi, int* bi, int* bj) {
  const int Tl = T - bj_lo, Wc = bj_hi - bj_lo;
  for (int J0 = 0; J0 < Wc; J0 += STRIP) {
    const i64 w = min(STRIP, Wc - J0);
    const i64 tri = w * (w + 1) / 2;
    const i64 cnt = tri + (i64)(Tl - J0 - w) * w;
    if (t < cnt) {
      int r, c;
      if (t < tri) {
        r = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);  // t < 136: exact enough, corrected below
        while ((i64)(r + 1) * (r + 2) / 2 <= t) r++;
        while ((i64)r * (r + 1) / 2 > t) r--;
        c = (int)(t - (i64)r * (r + 1) / 2);
      } else {
        const i64 u = t - tri;
        r = (int)(w + u / w);
        c = (int)(u % w);
      }
      *bi = bj_lo + J0 + r;
      *bj = bj_lo + J0 + c;
      return;
    }
    t -= cnt;
  }
  *bi = *bj = 0;  // not reached for t < number of blocks
}

template <typename TC>
__global__ void __launch_bounds__(THREADS, 1)
    k_syrk_bf16x3(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
                  TC* __restrict__ C, i64 ldc, int m, int Kp, int T, int bj_lo, int bj_hi, i64 nblk,
                  int* status) {
  if (*(volatile int*)status) return;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);  // TMA -> MMA, per stage
  uint64_t* empty = full + STAGES;                            // MMA -> TMA, per stage
  uint64_t* tfull = empty + STAGES;                           // MMA -> epilogue, per accumulator
  uint64_t* tempty = tfull + NACC;                            // epilogue -> MMA, per accumulator
  uint64_t* done = tempty + NACC;                             // drain after an abort
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  volatile long long* n_issued = (volatile long long*)(smem + STAGES * STAGE_BYTES + 128);  // stages loaded
  volatile long long* n_consumed = n_issued + 1;  // stages whose load the MMA thread saw complete

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = Kp / TK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < NACC; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], EPI_WARPS);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    *n_issued = 0;
    *n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---- TMA producer (lane 0; the warp stays converged around it)
    long long c = 0;
    bool ok = true;
    for (i64 t = blockIdx.x; ok && t < nblk; t += gridDim.x) {
      int bi, bj;
      strip_block_decode(t, T, bj_lo, bj_hi, &bi, &bj);
      const bool diag = (bi == bj);
      for (int kc = 0; kc < nk; kc++, c++) {
        if (lane == 0) {
          const int s = (int)(c % STAGES);
          const uint32_t ph = (uint32_t)((c / STAGES) & 1);
          if (!mbar_wait(&empty[s], ph ^ 1, abort_flag)) {
            ok = false;
          } else {
            uint8_t* st = smem + s * STAGE_BYTES;
            mbar_expect_tx(&full[s], diag ? 2 * PLANE_BYTES : STAGE_BYTES);
            tma_load_2d(st + 0 * PLANE_BYTES, &map_hi, &full[s], kc * TK, bi * TB);
            tma_load_2d(st + 1 * PLANE_BYTES, &map_lo, &full[s], kc * TK, bi * TB);
            if (!diag) {  // a diagonal block's B operand is its A operand
              tma_load_2d(st + 2 * PLANE_BYTES, &map_hi, &full[s], kc * TK, bj * TB);
              tma_load_2d(st + 3 * PLANE_BYTES, &map_lo, &full[s], kc * TK, bj * TB);
            }
            *n_issued = c + 1;
          }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
      }
    }
    if (!ok && lane == 0) *abort_flag = 1;
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer
      long long c = 0;
      int tl = 0;
      bool ok = true;
      for (i64 t = blockIdx.x; ok && t < nblk; t += gridDim.x, tl++) {
        int bi, bj;
        strip_block_decode(t, T, bj_lo, bj_hi, &bi, &bj);
        const bool diag = (bi == bj);
        const int acc = tl % NACC;
        if (!mbar_wait(&tempty[acc], (uint32_t)(((tl / NACC) & 1) ^ 1), abort_flag)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        const uint32_t dt = tmem + (uint32_t)(acc * TB);
        for (int kc = 0; kc < nk; kc++, c++) {
          const int s = (int)(c % STAGES);
          const uint32_t ph = (uint32_t)((c / STAGES) & 1);
          if (!mbar_wait(&full[s], ph, abort_flag)) { ok = false; break; }
          *n_consumed = c + 1;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
          const uint32_t base = smem_u32(smem + s * STAGE_BYTES);
          const uint32_t a_hi = base, a_lo = base + PLANE_BYTES;
          const uint32_t b_hi = diag ? a_hi : base + 2 * PLANE_BYTES;
          const uint32_t b_lo = diag ? a_lo : base + 3 * PLANE_BYTES;
#pragma unroll
          for (int kk = 0; kk < TK / 16; kk++) {
            const uint32_t off = kk * 32;  // 16 bf16 = 32 bytes along K inside the swizzle row
            const uint32_t acc0 = (kc > 0 || kk > 0) ? 1u : 0u;
            umma_bf16(dt, umma_desc_sw128(a_hi + off), umma_desc_sw128(b_hi + off), acc0);
            umma_bf16(dt, umma_desc_sw128(a_hi + off), umma_desc_sw128(b_lo + off), 1u);
            umma_bf16(dt, umma_desc_sw128(a_lo + off), umma_desc_sw128(b_hi + off), 1u);
          }
          umma_commit(&empty[s]);  // stage free once these MMAs have read it
        }
        if (!ok) break;
        umma_commit(&tfull[acc]);  // accumulator ready once every MMA above has completed
      }
      if (!ok) *abort_flag = 1;
    }
  } else {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (block rows) and one quarter
    // of the columns.  Each thread loads its 32 C values of the next block as soon as it
    // has stored the current one, so the loads overlap that block's MMAs.
    const int quad = warp & 3;
    const int cq = ((warp - 2) >> 2) * 32;
    int tl = 0;
    i64 t = blockIdx.x;
    int bi = 0, bj = 0;
    TC cv[32];
    if (t < nblk) strip_block_decode(t, T, bj_lo, bj_hi, &bi, &bj);
    {
      const int row = bi * TB + quad * 32 + lane, c0 = bj * TB + cq;
      const bool diag = (bi == bj);
      const TC* base = C + row + (i64)c0 * ldc;
#pragma unroll
      for (int q = 0; q < 32; q++) {
        const int col = c0 + q;
        cv[q] = (t < nblk && row < m && col < m && (!diag || col <= row)) ? base[(i64)q * ldc] : TC(0);
      }
    }
    for (; t < nblk; t += gridDim.x, tl++) {
      const int acc = tl % NACC;
      const bool got = mbar_wait(&tfull[acc], (uint32_t)((tl / NACC) & 1), abort_flag);
      if (!__all_sync(0xffffffffu, got)) {
        if (lane == 0) *abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      // two halves of 16 columns: the first is stored before the second is read, which
      // keeps the thread's registers within the 18-warp budget
      const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(acc * TB + cq);
      const int row = bi * TB + quad * 32 + lane, c0 = bj * TB + cq;
      const bool diag = (bi == bj);
      TC* base = C + row + (i64)c0 * ldc;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        uint32_t v[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(taddr + (uint32_t)(16 * h)));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
        if (h == 1) {
          asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
          __syncwarp();
          if (lane == 0) mbar_arrive(&tempty[acc]);  // the accumulator may be overwritten now
        }
        if (row < m) {
#pragma unroll
          for (int q = 0; q < 16; q++) {
            const int col = c0 + 16 * h + q;
            if (col < m && (!diag || col <= row))
              base[(i64)(16 * h + q) * ldc] = cv[16 * h + q] - (TC)__uint_as_float(v[q]);
          }
        }
      }
      const i64 tn = t + gridDim.x;
      if (tn < nblk) {
        strip_block_decode(tn, T, bj_lo, bj_hi, &bi, &bj);
        const int row = bi * TB + quad * 32 + lane, c0 = bj * TB + cq;
        const bool diag = (bi == bj);
        const TC* base = C + row + (i64)c0 * ldc;
#pragma unroll
        for (int q = 0; q < 32; q++) {
          const int col = c0 + q;
          cv[q] = (row < m && col < m && (!diag || col <= row)) ? base[(i64)q * ldc] : TC(0);
        }
      }
    }
  }

  // ---- teardown
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  if (*abort_flag) {
    if (threadIdx.x == 0) atomicCAS(status, 0, ERR_TIMEOUT_CODE);
    if (warp == 1 && lane == 0) {
      umma_commit(done);  // fires once every MMA this thread issued has completed
      (void)mbar_wait(done, 0, nullptr);
    }
    if (warp == 0 && lane == 0) {
      // Let loads still in flight land (bounded) before the CTA's shared memory goes away.
      for (long long c = *n_consumed; c < *n_issued; c++)
        (void)mbar_wait(&full[c % STAGES], (uint32_t)((c / STAGES) & 1), nullptr);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// ---------------------------------------------------------------------------------
// 256 x 128 blocks: two M=128 accumulators (rows 256 bi2 .. +127 and +128 .. +255) share
// the B operand, so a stage carries 25 % fewer operand bytes per MMA than two 128 x 128
// blocks.  Eight epilogue warps (two per TMEM lane quadrant, 64 columns each) stage -D in
// shared memory and add it into C with TMA reductions (cp.reduce.async.bulk.tensor .add):
// the read-modify-write of C happens in L2 on whole 1 KB column runs of a 256-row block,
// where per-thread loads and stores of one row across 64 columns reached only about half
// of the HBM bandwidth.  The FP32 additions in L2 round to nearest; like the L2's other
// FP32 atomics they may flush subnormal values (|x| < 2^-126) to zero.  Used for FP32 C (the
// working matrix of reduced-precision factors) with a 16-byte-aligned base and leading
// dimension.
//
// Blocks are scheduled at run time from a ticket counter (zeroed on the stream before each
// launch): with the diagonal-tile kernel running beside the update on another stream, the
// SMs of that kernel's GPC run about 20 % slower, and a static round-robin assignment
// made the whole launch wait for them.
// ---------------------------------------------------------------------------------
constexpr int TM2 = 256;
constexpr int STAGES2 = 2;
constexpr int A2_PLANE = TM2 * TK * 2;                    // 32 KB
constexpr int B2_PLANE = TB * TK * 2;                     // 16 KB
constexpr int STAGE2_BYTES = 2 * A2_PLANE + 2 * B2_PLANE; // Ahi, Alo, Bhi, Blo
constexpr int NSLOT2 = 2;                                 // blocks in flight in TMEM
constexpr int NID2 = 4;                                   // block-index ring entries
constexpr int TMEM_COLS2 = NSLOT2 * 2 * TB;               // 512: the whole TMEM
constexpr int EPI2_WARPS = 8;
constexpr int THREADS2 = 64 + 32 * EPI2_WARPS;
constexpr int SMEM2_BYTES = STAGES2 * STAGE2_BYTES + 1024 + 256;
static_assert((2 * STAGES2 + 2 * NSLOT2 + 1) * 8 + 8 <= 128, "control block overflow");
// counters at +128, index ring (2 NID2 barriers + NID2 indices) at +160, all inside the 256
static_assert(160 + 3 * NID2 * 8 <= 256, "index ring overflow");
// Update epilogue (FP32 C): per column group of four warps, two staging boxes of 256 rows x
// CB_COLS columns after the control block, handed to TMA reductions.
constexpr int CB_COLS = 8;
constexpr int CB_FLOATS = TM2 * CB_COLS;                       // 8 KB
constexpr int SMEM2U_BYTES = SMEM2_BYTES + 2 * 2 * CB_FLOATS * 4;  // 230,656
static_assert(SMEM2U_BYTES <= 232448, "update kernel shared memory");

// Block t of the block columns [bj_lo, bj_hi) (128 wide) x row blocks bi2 (256 high) with
// 2 bi2 + 1 >= bj, in strips of STRIP block columns, row by row inside a strip.
__device__ __forceinline__ void strip2_decode(i64 t, int T, int bj_lo, int bj_hi, int* bi2, int* bj) {
  const int T2 = (T + 1) / 2;
  for (int J0 = bj_lo; J0 < bj_hi; J0 += STRIP) {
    const int w = min(STRIP, bj_hi - J0);
    const int r0 = J0 / 2;
    const int a = min(w, 2 * r0 + 2 - J0);
    const int Kt = (w - a + 1) / 2;  // rows with fewer than w blocks
    const int rows = T2 - r0;
    const int kt = min(Kt, rows);
    const i64 tri_full = (i64)Kt * a + (i64)Kt * (Kt - 1);
    const i64 cnt = (i64)kt * a + (i64)kt * (kt - 1) + (i64)max(0, rows - Kt) * w;
    if (t < cnt) {
      int k, c;
      if (t < tri_full) {  // k^2 + (a-1) k <= t
        k = (int)((-(float)(a - 1) + sqrtf((float)((a - 1) * (a - 1)) + 4.f * (float)t)) * 0.5f);
        while ((i64)(k + 1) * (k + 1) + (i64)(a - 1) * (k + 1) <= t) k++;
        while ((i64)k * k + (i64)(a - 1) * k > t) k--;
        c = (int)(t - ((i64)k * k + (i64)(a - 1) * k));
      } else {
        const i64 u = t - tri_full;
        k = (int)(Kt + u / w);
        c = (int)(u % w);
      }
      *bi2 = r0 + k;
      *bj = J0 + c;
      return;
    }
    t -= cnt;
  }
  *bi2 = *bj = 0;  // not reached for t < number of blocks
}

template <typename TC>
__global__ void __launch_bounds__(THREADS2, 1)
    k_syrk2_bf16x3(const __grid_constant__ CUtensorMap map_ahi, const __grid_constant__ CUtensorMap map_alo,
                   const __grid_constant__ CUtensorMap map_bhi, const __grid_constant__ CUtensorMap map_blo,
                   const __grid_constant__ CUtensorMap map_c, int m, int Kp, int T, int bj_lo, int bj_hi, i64 nblk,
                   unsigned long long* __restrict__ tickets, int* status) {
  static_assert(sizeof(TC) == 4, "the reduction epilogue adds into FP32 C");
  if (*(volatile int*)status) return;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES2 * STAGE2_BYTES);
  uint64_t* empty = full + STAGES2;
  uint64_t* tfull = empty + STAGES2;
  uint64_t* tempty = tfull + NSLOT2;
  uint64_t* done = tempty + NSLOT2;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  volatile long long* n_issued = (volatile long long*)(smem + STAGES2 * STAGE2_BYTES + 128);
  volatile long long* n_consumed = n_issued + 1;
  // block-index ring: the producer publishes each block it starts (-1: no more blocks)
  uint64_t* idfull = (uint64_t*)(smem + STAGES2 * STAGE2_BYTES + 160);
  uint64_t* idempty = idfull + NID2;
  volatile long long* ids = (volatile long long*)(idempty + NID2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = Kp / TK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES2; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < NSLOT2; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], EPI2_WARPS);
    }
    for (int a = 0; a < NID2; a++) {
      mbar_init(&idfull[a], 1);
      mbar_init(&idempty[a], 1 + EPI2_WARPS);  // the MMA thread and every epilogue warp
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    *n_issued = 0;
    *n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS2));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---- TMA producer (lane 0; the warp stays converged around it).  Blocks are handed out
    // at run time: a CTA's first block is blockIdx.x, each later one gridDim.x + the next
    // ticket of the launch's counter, so that CTAs slowed by other work beside them (a
    // kernel on another stream shares their GPC's path to L2) take fewer blocks instead of
    // holding back the end of the launch.  Every block started is published in the ring.
    long long c = 0;
    bool ok = true;
    i64 t = blockIdx.x;
    for (int tl = 0; ok; tl++) {
      const i64 tp = t < nblk ? t : -1;
      if (lane == 0) {
        const int r = tl % NID2;
        if (!mbar_wait(&idempty[r], (uint32_t)(((tl / NID2) & 1) ^ 1), abort_flag)) {
          ok = false;
        } else {
          ids[r] = tp;
          mbar_arrive(&idfull[r]);
        }
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok || tp < 0) break;
      int bi2, bj;
      strip2_decode(t, T, bj_lo, bj_hi, &bi2, &bj);
      const bool b_in_a = (bj == 2 * bi2 || bj == 2 * bi2 + 1);  // B is one half of A
      for (int kc = 0; kc < nk; kc++, c++) {
        if (lane == 0) {
          const int s = (int)(c % STAGES2);
          const uint32_t ph = (uint32_t)((c / STAGES2) & 1);
          if (!mbar_wait(&empty[s], ph ^ 1, abort_flag)) {
            ok = false;
          } else {
            uint8_t* st = smem + s * STAGE2_BYTES;
            mbar_expect_tx(&full[s], b_in_a ? 2 * A2_PLANE : STAGE2_BYTES);
            tma_load_2d(st, &map_ahi, &full[s], kc * TK, bi2 * TM2);
            tma_load_2d(st + A2_PLANE, &map_alo, &full[s], kc * TK, bi2 * TM2);
            if (!b_in_a) {
              tma_load_2d(st + 2 * A2_PLANE, &map_bhi, &full[s], kc * TK, bj * TB);
              tma_load_2d(st + 2 * A2_PLANE + B2_PLANE, &map_blo, &full[s], kc * TK, bj * TB);
            }
            *n_issued = c + 1;
          }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
      }
      if (!ok) break;
      unsigned long long nx = 0;
      if (lane == 0) nx = atomicAdd(tickets, 1ull);
      nx = __shfl_sync(0xffffffffu, nx, 0);
      t = (i64)gridDim.x + (i64)nx;
    }
    if (!ok && lane == 0) *abort_flag = 1;
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer: per stage and K-step, three products into each active half
      long long c = 0;
      bool ok = true;
      for (int tl = 0;; tl++) {
        const int r = tl % NID2;
        if (!mbar_wait(&idfull[r], (uint32_t)((tl / NID2) & 1), abort_flag)) { ok = false; break; }
        const i64 t = ids[r];
        mbar_arrive(&idempty[r]);
        if (t < 0) break;
        int bi2, bj;
        strip2_decode(t, T, bj_lo, bj_hi, &bi2, &bj);
        const bool act0 = (2 * bi2 < T) && (2 * bi2 >= bj), act1 = (2 * bi2 + 1 < T) && (2 * bi2 + 1 >= bj);
        const int slot = tl % NSLOT2;
        if (!mbar_wait(&tempty[slot], (uint32_t)(((tl / NSLOT2) & 1) ^ 1), abort_flag)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        const uint32_t d0 = tmem + (uint32_t)(slot * 2 * TB), d1 = d0 + (uint32_t)TB;
        for (int kc = 0; kc < nk; kc++, c++) {
          const int s = (int)(c % STAGES2);
          const uint32_t ph = (uint32_t)((c / STAGES2) & 1);
          if (!mbar_wait(&full[s], ph, abort_flag)) { ok = false; break; }
          *n_consumed = c + 1;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
          const uint32_t base = smem_u32(smem + s * STAGE2_BYTES);
          const uint32_t a_hi = base, a_lo = base + A2_PLANE;
          const uint32_t half_b = (uint32_t)(TB * 128);  // 128 rows x 128 bytes
          uint32_t b_hi = base + 2 * A2_PLANE, b_lo = base + 2 * A2_PLANE + B2_PLANE;
          if (bj == 2 * bi2) { b_hi = a_hi; b_lo = a_lo; }
          if (bj == 2 * bi2 + 1) { b_hi = a_hi + half_b; b_lo = a_lo + half_b; }
#pragma unroll
          for (int kk = 0; kk < TK / 16; kk++) {
            const uint32_t off = kk * 32;
            const uint32_t acc0 = (kc > 0 || kk > 0) ? 1u : 0u;
            if (act0) {
              umma_bf16(d0, umma_desc_sw128(a_hi + off), umma_desc_sw128(b_hi + off), acc0);
              umma_bf16(d0, umma_desc_sw128(a_hi + off), umma_desc_sw128(b_lo + off), 1u);
              umma_bf16(d0, umma_desc_sw128(a_lo + off), umma_desc_sw128(b_hi + off), 1u);
            }
            if (act1) {
              umma_bf16(d1, umma_desc_sw128(a_hi + half_b + off), umma_desc_sw128(b_hi + off), acc0);
              umma_bf16(d1, umma_desc_sw128(a_hi + half_b + off), umma_desc_sw128(b_lo + off), 1u);
              umma_bf16(d1, umma_desc_sw128(a_lo + half_b + off), umma_desc_sw128(b_hi + off), 1u);
            }
          }
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&tfull[slot]);
      }
      if (!ok) *abort_flag = 1;
    }
  } else {
    // ---- epilogue: the four warps of a column group (64 columns; warp w reads TMEM lanes
    // 32 (w % 4) .. +31 of both halves) stage -D in boxes of 256 rows x CB_COLS columns, and
    // one thread adds each box into C with a TMA reduction: L2 does the read-modify-write in
    // 1 KB column runs, and the SM keeps no C values.  Elements outside the lower triangle
    // (above the diagonal in a diagonal block, or a half above it) are staged as -0.0, which
    // leaves any value unchanged; rows and columns past m are clipped by the tensor map.
    // Every decision to stop is a vote of the group (bar.red), so that all four warps always
    // meet the same named barriers.
    const int quad = warp & 3;
    const int grp = (warp - 2) >> 2;
    const int cg = grp * 64;
    const uint32_t gbar = 1 + (uint32_t)grp;  // named barrier of the column group (128 threads)
    const bool issuer = (warp == 2 + 4 * grp) && lane == 0;
    float* cbox = reinterpret_cast<float*>(smem + STAGES2 * STAGE2_BYTES + 256) + grp * 2 * CB_FLOATS;
    // index of the CTA's u-th block from the ring: -1 when none is left, -2 on abort
    auto next_id = [&](int u) -> i64 {
      const int r = u % NID2;
      const bool got = mbar_wait(&idfull[r], (uint32_t)((u / NID2) & 1), abort_flag);
      i64 v = -2;
      if (__all_sync(0xffffffffu, got)) v = ids[r];
      __syncwarp();
      if (lane == 0 && v != -2) mbar_arrive(&idempty[r]);
      return named_bar_and(gbar, 128, v != -2) ? v : -2;
    };
    int nbox = 0;
    i64 t = next_id(0);
    for (int tl = 0; t >= 0; tl++) {
      int bi2, bj;
      strip2_decode(t, T, bj_lo, bj_hi, &bi2, &bj);
      const int slot = tl % NSLOT2;
      const bool got = mbar_wait(&tfull[slot], (uint32_t)((tl / NSLOT2) & 1), abort_flag);
      if (!named_bar_and(gbar, 128, __all_sync(0xffffffffu, got))) {
        t = -2;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      const int r0 = quad * 32 + lane;  // row within a half
      const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(slot * 2 * TB + cg);
#pragma unroll 1
      for (int ch = 0; ch < 4; ch++) {
        uint32_t v0[16], v1[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
            : "=r"(v0[0]), "=r"(v0[1]), "=r"(v0[2]), "=r"(v0[3]), "=r"(v0[4]), "=r"(v0[5]), "=r"(v0[6]), "=r"(v0[7]),
              "=r"(v0[8]), "=r"(v0[9]), "=r"(v0[10]), "=r"(v0[11]), "=r"(v0[12]), "=r"(v0[13]), "=r"(v0[14]),
              "=r"(v0[15])
            : "r"(taddr + (uint32_t)(16 * ch)));
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
            : "=r"(v1[0]), "=r"(v1[1]), "=r"(v1[2]), "=r"(v1[3]), "=r"(v1[4]), "=r"(v1[5]), "=r"(v1[6]), "=r"(v1[7]),
              "=r"(v1[8]), "=r"(v1[9]), "=r"(v1[10]), "=r"(v1[11]), "=r"(v1[12]), "=r"(v1[13]), "=r"(v1[14]),
              "=r"(v1[15])
            : "r"(taddr + (uint32_t)(TB + 16 * ch)));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
#pragma unroll
        for (int sub = 0; sub < 16 / CB_COLS; sub++) {
          float* box = cbox + (nbox & 1) * CB_FLOATS;
          if (issuer) bulk_wait_read<1>();  // the reduction that last read this box is done with it
          named_bar_sync(gbar, 128);
          const int col0 = bj * TB + cg + 16 * ch + CB_COLS * sub;
#pragma unroll
          for (int c = 0; c < CB_COLS; c++) {
            const int col = col0 + c;
#pragma unroll
            for (int h = 0; h < 2; h++) {
              const int blk = 2 * bi2 + h, row = blk * TB + r0;
              const bool keep = blk < T && blk >= bj && (blk != bj || col <= row);
              const uint32_t u = h ? v1[CB_COLS * sub + c] : v0[CB_COLS * sub + c];
              box[c * TM2 + h * TB + r0] = keep ? -__uint_as_float(u) : -0.0f;
            }
          }
          fence_proxy_async_smem();
          named_bar_sync(gbar, 128);
          if (issuer) {
            tma_reduce_add_2d(&map_c, box, bi2 * TM2, col0);
            bulk_commit();
          }
          nbox++;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[slot]);  // both halves read: the slot may be reused
      t = next_id(tl + 1);
    }
    if (issuer) bulk_wait_all();  // every reduction of this CTA has landed
    if (t == -2 && lane == 0) *abort_flag = 1;
  }

  // ---- teardown (as in k_syrk_bf16x3)
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  if (*abort_flag) {
    if (threadIdx.x == 0) atomicCAS(status, 0, ERR_TIMEOUT_CODE);
    if (warp == 1 && lane == 0) {
      umma_commit(done);
      (void)mbar_wait(done, 0, nullptr);
    }
    if (warp == 0 && lane == 0) {
      for (long long c = *n_consumed; c < *n_issued; c++)
        (void)mbar_wait(&full[c % STAGES2], (uint32_t)((c / STAGES2) & 1), nullptr);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS2));
  }
}

// ---------------------------------------------------------------------------------
// The same update for long K (the left-looking factor's catch-ups), issued transposed: per
// K step and product ONE M=128, N=256 MMA with the 128-row B tile as the M operand and the
// 256-row A tile as the N operand, so TMEM holds the block transposed (lane = C column,
// TMEM column = C row) and each MMA reads 12 KB of operands from shared memory for 128 x
// 256 outputs where two M=N=128 MMAs read 16 KB (the MMA stream measured 1.39x faster in
// isolation).  Same producer, rings, block tickets, bounded waits and teardown as
// k_syrk2_bf16x3; halves of a block that lie above the diagonal are computed and masked.
// Epilogue: warp (quad q, group g) reads TMEM lanes 32q.. (32 C columns) and TMEM columns
// 128g.. (128 C rows) in four 32-row pieces; a thread owns one C column, so a piece is a
// 32 x 32 box stored column by column with the 128-byte swizzle (conflict-free 16-byte
// stores) and added into C by one TMA reduction.  Its per-block cost is higher than the
// K=512 kernel's, which is why only launches with a long K use it.
// ---------------------------------------------------------------------------------
constexpr uint32_t IDESC_N256 =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(TB >> 4) << 24);
__device__ __forceinline__ void umma_bf16_n256(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(IDESC_N256), "r"(accumulate));
}
// Operand ring of the transposed kernel: four stages of K = 32 (64-byte rows, 64-byte
// swizzle), 48 KB each, where the K = 64 kernels hold two stages of 96 KB: the same bytes
// in flight, but the MMA can start on a stage as soon as half as many bytes have landed
// and the producer refills a stage after half as many MMAs.
constexpr int TK_T = 32;
constexpr int STAGES_T = 4;
constexpr int A_T_PLANE = TM2 * TK_T * 2;                      // 16 KB
constexpr int B_T_PLANE = TB * TK_T * 2;                       // 8 KB
constexpr int STAGE_T_BYTES = 2 * A_T_PLANE + 2 * B_T_PLANE;   // 48 KB
static_assert(STAGES_T * STAGE_T_BYTES == STAGES2 * STAGE2_BYTES, "the transposed ring keeps the smem budget");
static_assert(A_T_PLANE % 512 == 0 && B_T_PLANE % 512 == 0, "64-byte swizzle atoms are 512-byte aligned");
// Shared-memory matrix descriptor for a K-major BF16 tile with the 64-byte swizzle: rows
// of 64 bytes, 8-row atoms of 512 bytes one after another along M/N.
__device__ __forceinline__ uint64_t umma_desc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);          // start address
  d |= (uint64_t)(16 >> 4) << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;                  // stride byte offset: 8 rows x 64 B
  d |= (uint64_t)1 << 46;                           // fixed 0b001
  d |= (uint64_t)4 << 61;                           // 64-byte swizzle
  return d;
}
constexpr int TBOX = 32;  // 32 x 32 FP32 C boxes (4 KB, 1024-byte aligned for the swizzle)
constexpr int BOX2T_OFF = STAGES_T * STAGE_T_BYTES + 1024;  // after the control block, padded
constexpr int SMEM2T_BYTES = BOX2T_OFF + EPI2_WARPS * TBOX * TBOX * 4 + 1024 /*align*/;  // 231,424
static_assert(SMEM2T_BYTES <= 232448, "transposed update kernel shared memory");

__global__ void __launch_bounds__(THREADS2, 1)
    k_syrk2t_bf16x3(const __grid_constant__ CUtensorMap map_ahi, const __grid_constant__ CUtensorMap map_alo,
                    const __grid_constant__ CUtensorMap map_bhi, const __grid_constant__ CUtensorMap map_blo,
                    const __grid_constant__ CUtensorMap map_c, int m, int Kp, int T, int bj_lo, int bj_hi, i64 nblk,
                    unsigned long long* __restrict__ tickets, int* status) {
  if (*(volatile int*)status) return;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES_T * STAGE_T_BYTES);
  uint64_t* empty = full + STAGES_T;
  uint64_t* tfull = empty + STAGES_T;
  uint64_t* tempty = tfull + NSLOT2;
  uint64_t* done = tempty + NSLOT2;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  volatile long long* n_issued = (volatile long long*)(smem + STAGES_T * STAGE_T_BYTES + 128);
  volatile long long* n_consumed = n_issued + 1;
  uint64_t* idfull = (uint64_t*)(smem + STAGES_T * STAGE_T_BYTES + 160);
  uint64_t* idempty = idfull + NID2;
  volatile long long* ids = (volatile long long*)(idempty + NID2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = Kp / TK_T;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES_T; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < NSLOT2; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], EPI2_WARPS);
    }
    for (int a = 0; a < NID2; a++) {
      mbar_init(&idfull[a], 1);
      mbar_init(&idempty[a], 1 + EPI2_WARPS);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    *n_issued = 0;
    *n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS2));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---- TMA producer: as in k_syrk2_bf16x3
    long long c = 0;
    bool ok = true;
    i64 t = blockIdx.x;
    for (int tl = 0; ok; tl++) {
      const i64 tp = t < nblk ? t : -1;
      if (lane == 0) {
        const int r = tl % NID2;
        if (!mbar_wait(&idempty[r], (uint32_t)(((tl / NID2) & 1) ^ 1), abort_flag)) {
          ok = false;
        } else {
          ids[r] = tp;
          mbar_arrive(&idfull[r]);
        }
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok || tp < 0) break;
      int bi2, bj;
      strip2_decode(t, T, bj_lo, bj_hi, &bi2, &bj);
      const bool b_in_a = (bj == 2 * bi2 || bj == 2 * bi2 + 1);
      for (int kc = 0; kc < nk; kc++, c++) {
        if (lane == 0) {
          const int s = (int)(c % STAGES_T);
          const uint32_t ph = (uint32_t)((c / STAGES_T) & 1);
          if (!mbar_wait(&empty[s], ph ^ 1, abort_flag)) {
            ok = false;
          } else {
            uint8_t* st = smem + s * STAGE_T_BYTES;
            mbar_expect_tx(&full[s], b_in_a ? 2 * A_T_PLANE : STAGE_T_BYTES);
            tma_load_2d(st, &map_ahi, &full[s], kc * TK_T, bi2 * TM2);
            tma_load_2d(st + A_T_PLANE, &map_alo, &full[s], kc * TK_T, bi2 * TM2);
            if (!b_in_a) {
              tma_load_2d(st + 2 * A_T_PLANE, &map_bhi, &full[s], kc * TK_T, bj * TB);
              tma_load_2d(st + 2 * A_T_PLANE + B_T_PLANE, &map_blo, &full[s], kc * TK_T, bj * TB);
            }
            *n_issued = c + 1;
          }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
      }
      if (!ok) break;
      unsigned long long nx = 0;
      if (lane == 0) nx = atomicAdd(tickets, 1ull);
      nx = __shfl_sync(0xffffffffu, nx, 0);
      t = (i64)gridDim.x + (i64)nx;
    }
    if (!ok && lane == 0) *abort_flag = 1;
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer: per stage and K-step, the three products as N=256 MMAs (D transposed)
      long long c = 0;
      bool ok = true;
      for (int tl = 0;; tl++) {
        const int r = tl % NID2;
        if (!mbar_wait(&idfull[r], (uint32_t)((tl / NID2) & 1), abort_flag)) { ok = false; break; }
        const i64 t = ids[r];
        mbar_arrive(&idempty[r]);
        if (t < 0) break;
        int bi2, bj;
        strip2_decode(t, T, bj_lo, bj_hi, &bi2, &bj);
        const int slot = tl % NSLOT2;
        if (!mbar_wait(&tempty[slot], (uint32_t)(((tl / NSLOT2) & 1) ^ 1), abort_flag)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        const uint32_t d = tmem + (uint32_t)(slot * 2 * TB);
        for (int kc = 0; kc < nk; kc++, c++) {
          const int s = (int)(c % STAGES_T);
          const uint32_t ph = (uint32_t)((c / STAGES_T) & 1);
          if (!mbar_wait(&full[s], ph, abort_flag)) { ok = false; break; }
          *n_consumed = c + 1;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
          const uint32_t base = smem_u32(smem + s * STAGE_T_BYTES);
          const uint32_t a_hi = base, a_lo = base + A_T_PLANE;
          const uint32_t half_b = (uint32_t)(TB * TK_T * 2);
          uint32_t b_hi = base + 2 * A_T_PLANE, b_lo = base + 2 * A_T_PLANE + B_T_PLANE;
          if (bj == 2 * bi2) { b_hi = a_hi; b_lo = a_lo; }
          if (bj == 2 * bi2 + 1) { b_hi = a_hi + half_b; b_lo = a_lo + half_b; }
#pragma unroll
          for (int kk = 0; kk < TK_T / 16; kk++) {
            const uint32_t off = kk * 32;
            const uint32_t acc0 = (kc > 0 || kk > 0) ? 1u : 0u;
            umma_bf16_n256(d, umma_desc_sw64(b_hi + off), umma_desc_sw64(a_hi + off), acc0);
            umma_bf16_n256(d, umma_desc_sw64(b_hi + off), umma_desc_sw64(a_lo + off), 1u);
            umma_bf16_n256(d, umma_desc_sw64(b_lo + off), umma_desc_sw64(a_hi + off), 1u);
          }
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&tfull[slot]);
      }
      if (!ok) *abort_flag = 1;
    }
  } else {
    // ---- epilogue: warp (quad q, group g): C columns bj*128 + 32q + lane, C rows
    // bi2*256 + 128g + 32 piece + (0..31); one 32 x 32 box per piece, 128-byte swizzled.
    const int quad = warp & 3;
    const int grp = (warp - 2) >> 2;
    float* box = reinterpret_cast<float*>(smem + BOX2T_OFF) + (warp - 2) * TBOX * TBOX;
    auto next_id = [&](int u) -> i64 {
      const int r = u % NID2;
      const bool got = mbar_wait(&idfull[r], (uint32_t)((u / NID2) & 1), abort_flag);
      i64 v = -2;
      if (__all_sync(0xffffffffu, got)) v = ids[r];
      __syncwarp();
      if (lane == 0 && v != -2) mbar_arrive(&idempty[r]);
      return v;
    };
    i64 t = next_id(0);
    for (int tl = 0; t >= 0; tl++) {
      int bi2, bj;
      strip2_decode(t, T, bj_lo, bj_hi, &bi2, &bj);
      const int slot = tl % NSLOT2;
      const bool got = mbar_wait(&tfull[slot], (uint32_t)((tl / NSLOT2) & 1), abort_flag);
      if (!__all_sync(0xffffffffu, got)) {
        t = -2;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      const int col = bj * TB + quad * 32 + lane;  // this thread's C column
      const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(slot * 2 * TB + grp * 128);
#pragma unroll 1
      for (int piece = 0; piece < 4; piece++) {
        uint32_t v[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(taddr + (uint32_t)(32 * piece)));
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
            : "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
              "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
              "=r"(v[30]), "=r"(v[31])
            : "r"(taddr + (uint32_t)(32 * piece + 16)));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
        const int row0 = bi2 * TM2 + grp * 128 + piece * 32;
        if (lane == 0) bulk_wait_read<0>();  // the previous piece's reduction has read the box
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 8; j++) {  // 16-byte chunk j: rows row0 + 4j .. +3
          float4 q4;
          float* f = reinterpret_cast<float*>(&q4);
#pragma unroll
          for (int e = 0; e < 4; e++) {
            const int row = row0 + 4 * j + e;
            f[e] = (col <= row) ? -__uint_as_float(v[4 * j + e]) : -0.0f;
          }
          *reinterpret_cast<float4*>(box + lane * TBOX + ((j ^ (lane & 7)) * 4)) = q4;
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) {
          tma_reduce_add_2d(&map_c, box, row0, bj * TB + quad * 32);
          bulk_commit();
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[slot]);
      t = next_id(tl + 1);
    }
    if (lane == 0) bulk_wait_all();
    if (t == -2 && lane == 0) *abort_flag = 1;
  }

  // ---- teardown (as in k_syrk2_bf16x3)
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  if (*abort_flag) {
    if (threadIdx.x == 0) atomicCAS(status, 0, ERR_TIMEOUT_CODE);
    if (warp == 1 && lane == 0) {
      umma_commit(done);
      (void)mbar_wait(done, 0, nullptr);
    }
    if (warp == 0 && lane == 0) {
      for (long long c = *n_consumed; c < *n_issued; c++)
        (void)mbar_wait(&full[c % STAGES_T], (uint32_t)((c / STAGES_T) & 1), nullptr);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS2));
  }
}

// ---------------------------------------------------------------------------------
// Column solve of a panel on the tensor cores: P = U X^T (m x nb), U the panel before the
// solve and X = L_jj^{-1} (lower triangular), both given as BF16 hi/lo planes (K-major),
// with the update's three products.  Block t = (row tile bi2 of 256 rows, column block cb
// of 128): K runs over [0, 128 (cb + 1)) only, since X(c, k) = 0 for k > c.  The epilogue
// writes the FP32 result into the panel (column-major, ld ldp) and its hi/lo split into the
// planes the trailing update reads (Mp x Kp, row-major), so the update needs no split pass.
// Same roles, rings, bounded waits, run-time block tickets and teardown as k_syrk2_bf16x3.
// ---------------------------------------------------------------------------------
__global__ void __launch_bounds__(THREADS2, 1)
    k_trsm2_bf16x3(const __grid_constant__ CUtensorMap map_uhi, const __grid_constant__ CUtensorMap map_ulo,
                   const __grid_constant__ CUtensorMap map_xhi, const __grid_constant__ CUtensorMap map_xlo,
                   float* __restrict__ P, i64 ldp, __nv_bfloat16* __restrict__ shi, __nv_bfloat16* __restrict__ slo,
                   i64 lds, int Kp, int m, int ncb, i64 nblk, unsigned long long* __restrict__ tickets, int* status) {
  if (*(volatile int*)status) return;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES2 * STAGE2_BYTES);
  uint64_t* empty = full + STAGES2;
  uint64_t* tfull = empty + STAGES2;
  uint64_t* tempty = tfull + NSLOT2;
  uint64_t* done = tempty + NSLOT2;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  volatile long long* n_issued = (volatile long long*)(smem + STAGES2 * STAGE2_BYTES + 128);
  volatile long long* n_consumed = n_issued + 1;
  uint64_t* idfull = (uint64_t*)(smem + STAGES2 * STAGE2_BYTES + 160);
  uint64_t* idempty = idfull + NID2;
  volatile long long* ids = (volatile long long*)(idempty + NID2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES2; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < NSLOT2; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], EPI2_WARPS);
    }
    for (int a = 0; a < NID2; a++) {
      mbar_init(&idfull[a], 1);
      mbar_init(&idempty[a], 1 + EPI2_WARPS);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    *n_issued = 0;
    *n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS2));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---- TMA producer (lane 0; the warp stays converged around it)
    long long c = 0;
    bool ok = true;
    i64 t = blockIdx.x;
    for (int tl = 0; ok; tl++) {
      const i64 tp = t < nblk ? t : -1;
      if (lane == 0) {
        const int r = tl % NID2;
        if (!mbar_wait(&idempty[r], (uint32_t)(((tl / NID2) & 1) ^ 1), abort_flag)) {
          ok = false;
        } else {
          ids[r] = tp;
          mbar_arrive(&idfull[r]);
        }
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok || tp < 0) break;
      const int bi2 = (int)(t / ncb), cb = (int)(t % ncb);
      const int nk = 2 * (cb + 1);
      for (int kc = 0; kc < nk; kc++, c++) {
        if (lane == 0) {
          const int s = (int)(c % STAGES2);
          const uint32_t ph = (uint32_t)((c / STAGES2) & 1);
          if (!mbar_wait(&empty[s], ph ^ 1, abort_flag)) {
            ok = false;
          } else {
            uint8_t* st = smem + s * STAGE2_BYTES;
            mbar_expect_tx(&full[s], STAGE2_BYTES);
            tma_load_2d(st, &map_uhi, &full[s], kc * TK, bi2 * TM2);
            tma_load_2d(st + A2_PLANE, &map_ulo, &full[s], kc * TK, bi2 * TM2);
            tma_load_2d(st + 2 * A2_PLANE, &map_xhi, &full[s], kc * TK, cb * TB);
            tma_load_2d(st + 2 * A2_PLANE + B2_PLANE, &map_xlo, &full[s], kc * TK, cb * TB);
            *n_issued = c + 1;
          }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
      }
      if (!ok) break;
      unsigned long long nx = 0;
      if (lane == 0) nx = atomicAdd(tickets, 1ull);
      nx = __shfl_sync(0xffffffffu, nx, 0);
      t = (i64)gridDim.x + (i64)nx;
    }
    if (!ok && lane == 0) *abort_flag = 1;
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer
      long long c = 0;
      bool ok = true;
      for (int tl = 0;; tl++) {
        const int r = tl % NID2;
        if (!mbar_wait(&idfull[r], (uint32_t)((tl / NID2) & 1), abort_flag)) { ok = false; break; }
        const i64 t = ids[r];
        mbar_arrive(&idempty[r]);
        if (t < 0) break;
        const int bi2 = (int)(t / ncb), cb = (int)(t % ncb);
        const int nk = 2 * (cb + 1);
        const bool act1 = (2 * bi2 + 1) * TB < m;
        const int slot = tl % NSLOT2;
        if (!mbar_wait(&tempty[slot], (uint32_t)(((tl / NSLOT2) & 1) ^ 1), abort_flag)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        const uint32_t d0 = tmem + (uint32_t)(slot * 2 * TB), d1 = d0 + (uint32_t)TB;
        for (int kc = 0; kc < nk; kc++, c++) {
          const int s = (int)(c % STAGES2);
          const uint32_t ph = (uint32_t)((c / STAGES2) & 1);
          if (!mbar_wait(&full[s], ph, abort_flag)) { ok = false; break; }
          *n_consumed = c + 1;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
          const uint32_t base = smem_u32(smem + s * STAGE2_BYTES);
          const uint32_t a_hi = base, a_lo = base + A2_PLANE;
          const uint32_t half_a = (uint32_t)(TB * 128);  // 128 rows x 128 bytes
          const uint32_t b_hi = base + 2 * A2_PLANE, b_lo = base + 2 * A2_PLANE + B2_PLANE;
#pragma unroll
          for (int kk = 0; kk < TK / 16; kk++) {
            const uint32_t off = kk * 32;
            const uint32_t acc0 = (kc > 0 || kk > 0) ? 1u : 0u;
            umma_bf16(d0, umma_desc_sw128(a_hi + off), umma_desc_sw128(b_hi + off), acc0);
            umma_bf16(d0, umma_desc_sw128(a_hi + off), umma_desc_sw128(b_lo + off), 1u);
            umma_bf16(d0, umma_desc_sw128(a_lo + off), umma_desc_sw128(b_hi + off), 1u);
            if (act1) {
              umma_bf16(d1, umma_desc_sw128(a_hi + half_a + off), umma_desc_sw128(b_hi + off), acc0);
              umma_bf16(d1, umma_desc_sw128(a_hi + half_a + off), umma_desc_sw128(b_lo + off), 1u);
              umma_bf16(d1, umma_desc_sw128(a_lo + half_a + off), umma_desc_sw128(b_hi + off), 1u);
            }
          }
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&tfull[slot]);
      }
      if (!ok) *abort_flag = 1;
    }
  } else {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 of both halves, 64 columns;
    // a thread owns one row: FP32 stores coalesce along the column, and each plane gets
    // 32-byte runs of the row.
    const int quad = warp & 3;
    const int cg = ((warp - 2) >> 2) * 64;
    auto next_id = [&](int u) -> i64 {
      const int r = u % NID2;
      const bool got = mbar_wait(&idfull[r], (uint32_t)((u / NID2) & 1), abort_flag);
      if (!__all_sync(0xffffffffu, got)) return -2;
      const i64 v = ids[r];
      __syncwarp();
      if (lane == 0) mbar_arrive(&idempty[r]);
      return v;
    };
    i64 t = next_id(0);
    for (int tl = 0; t >= 0; tl++) {
      const int bi2 = (int)(t / ncb), cb = (int)(t % ncb);
      const int slot = tl % NSLOT2;
      const bool got = mbar_wait(&tfull[slot], (uint32_t)((tl / NSLOT2) & 1), abort_flag);
      if (!__all_sync(0xffffffffu, got)) {
        t = -2;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
#pragma unroll
      for (int h = 0; h < 2; h++) {
        if ((2 * bi2 + h) * TB >= m) continue;  // uniform: this half was not computed
        const int row = (2 * bi2 + h) * TB + quad * 32 + lane, c0 = cb * TB + cg;
        float* pb = P + row + (i64)c0 * ldp;
        __nv_bfloat16* hb = shi + (i64)row * lds + c0;
        __nv_bfloat16* lb = slo + (i64)row * lds + c0;
        const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(slot * 2 * TB + h * TB + cg);
#pragma unroll
        for (int ch = 0; ch < 4; ch++) {
          uint32_t v[16];
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
              : "r"(taddr + (uint32_t)(16 * ch)));
          asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
          if (row < m) {
            uint32_t ph[8], pl[8];
#pragma unroll
            for (int q = 0; q < 16; q += 2) {
              const float f0 = __uint_as_float(v[q]), f1 = __uint_as_float(v[q + 1]);
              pb[(i64)(16 * ch + q) * ldp] = f0;
              pb[(i64)(16 * ch + q + 1) * ldp] = f1;
              const __nv_bfloat16 h0 = __float2bfloat16_rn(f0), h1 = __float2bfloat16_rn(f1);
              const __nv_bfloat16 l0 = __float2bfloat16_rn(f0 - __bfloat162float(h0));
              const __nv_bfloat16 l1 = __float2bfloat16_rn(f1 - __bfloat162float(h1));
              ph[q / 2] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
              pl[q / 2] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
            }
            uint4* h4 = reinterpret_cast<uint4*>(hb + 16 * ch);
            uint4* l4 = reinterpret_cast<uint4*>(lb + 16 * ch);
            h4[0] = make_uint4(ph[0], ph[1], ph[2], ph[3]);
            h4[1] = make_uint4(ph[4], ph[5], ph[6], ph[7]);
            l4[0] = make_uint4(pl[0], pl[1], pl[2], pl[3]);
            l4[1] = make_uint4(pl[4], pl[5], pl[6], pl[7]);
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[slot]);
      t = next_id(tl + 1);
    }
    if (t == -2 && lane == 0) *abort_flag = 1;
  }

  // ---- teardown (as in k_syrk_bf16x3)
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  if (*abort_flag) {
    if (threadIdx.x == 0) atomicCAS(status, 0, ERR_TIMEOUT_CODE);
    if (warp == 1 && lane == 0) {
      umma_commit(done);
      (void)mbar_wait(done, 0, nullptr);
    }
    if (warp == 0 && lane == 0) {
      for (long long c = *n_consumed; c < *n_issued; c++)
        (void)mbar_wait(&full[c % STAGES2], (uint32_t)((c / STAGES2) & 1), nullptr);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS2));
  }
}

// ------------------------------ host: tensor maps --------------------------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

int get_encode() {
  std::call_once(g_encode_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  });
  return g_encode ? OOC_OK : OOC_ERR_UNSUPPORTED;
}

// BF16 plane of `rows` rows of K values (row-major, `ldk` elements between rows; ldk = K
// when omitted): boxes of TK x box_rows, 128-byte swizzle (or TK_T x box_rows with the
// 64-byte swizzle for the transposed kernel's ring).  Rows and K past the plane read as zeros.
int make_map(CUtensorMap* map, void* base, int rows, int K, int box_rows = TB, i64 ldk = 0, bool k32 = false) {
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ldk > 0 ? ldk : K) * 2};
  cuuint32_t box[2] = {(cuuint32_t)(k32 ? TK_T : TK), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, k32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? OOC_OK : OOC_ERR_CUDA;
}

// FP32 C (m x m, column-major, ld ldc) for the update's TMA reductions: boxes of 256 rows x
// CB_COLS columns, rows innermost.
int make_map_c32(CUtensorMap* map, float* C, int m, i64 ldc) {
  cuuint64_t dims[2] = {(cuuint64_t)m, (cuuint64_t)m};
  cuuint64_t strides[1] = {(cuuint64_t)ldc * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)TM2, (cuuint32_t)CB_COLS};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? OOC_OK : OOC_ERR_CUDA;
}

// FP32 C for the transposed update's reductions: 32 x 32 boxes (rows innermost), 128-byte
// swizzle (the epilogue stores each box column by column with the same swizzle).
int make_map_c32t(CUtensorMap* map, float* C, int m, i64 ldc) {
  cuuint64_t dims[2] = {(cuuint64_t)m, (cuuint64_t)m};
  cuuint64_t strides[1] = {(cuuint64_t)ldc * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)TBOX, (cuuint32_t)TBOX};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? OOC_OK : OOC_ERR_CUDA;
}

// Number of 256 x 128 blocks of k_syrk2_bf16x3 for block columns [bj_lo, bj_hi).
i64 count_blocks2(int T, int bj_lo, int bj_hi) {
  const int T2 = (T + 1) / 2;
  i64 total = 0;
  for (int J0 = bj_lo; J0 < bj_hi; J0 += STRIP) {
    const int w = std::min(STRIP, bj_hi - J0);
    const int r0 = J0 / 2;
    const int a = std::min(w, 2 * r0 + 2 - J0);
    const int Kt = (w - a + 1) / 2;
    const int rows = T2 - r0;
    const int kt = std::min(Kt, rows);
    total += (i64)kt * a + (i64)kt * (kt - 1) + (i64)std::max(0, rows - Kt) * w;
  }
  return total;
}

}  // namespace

size_t bf16x3_work_bytes(int m, int K) {
  const size_t Mp = ((size_t)m + TB - 1) / TB * TB;
  const size_t Kp = ((size_t)K + TK - 1) / TK * TK;
  return 2 * Mp * Kp * sizeof(__nv_bfloat16) + 256;
}

namespace {
template <typename TX, typename TC>
int launch_syrk_t(const TX* X, i64 ldx, TC* C, i64 ldc, int m, int K, const int* status, cudaStream_t s, void* work,
                  size_t work_bytes, int bj_lo, int bj_hi, int do_split, int reserve_sms) {
  if (m <= 0 || K <= 0) return OOC_OK;
  if (!status) return OOC_ERR_INTERNAL;
  int rc = get_encode();
  if (rc) return rc;
  const int Mp = (m + TB - 1) / TB * TB;
  const int Kp = (K + TK - 1) / TK * TK;
  if (work_bytes < bf16x3_work_bytes(m, K)) return OOC_ERR_INTERNAL;
  __nv_bfloat16* hi = (__nv_bfloat16*)work;
  __nv_bfloat16* lo = hi + (size_t)Mp * Kp;
  if (do_split) {
    dim3 sg((unsigned)(Kp / 32), (unsigned)(Mp / 32));
    k_split_bf16<TX><<<sg, dim3(32, 8), 0, s>>>(X, ldx, hi, lo, m, K, Mp, Kp);
    OOC_CUDA_TRY(cudaGetLastError());
  }
  CUtensorMap mh, ml;
  if (make_map(&mh, hi, Mp, Kp) || make_map(&ml, lo, Mp, Kp)) {
    ooc_set_last_message("cuTensorMapEncodeTiled failed for the BF16 split planes");
    return OOC_ERR_CUDA;
  }
  // per device: set on every launch (cheap)
  OOC_CUDA_TRY(cudaFuncSetAttribute(k_syrk_bf16x3<TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
  const i64 T = Mp / TB;
  bj_hi = (int)std::min<i64>(bj_hi < 0 ? T : bj_hi, T);
  if (bj_lo >= bj_hi) return OOC_OK;
  const i64 nblk = ooc_lower_blocks_before(bj_hi, T) - ooc_lower_blocks_before(bj_lo, T);
  int dev = 0, nsm = 0;
  OOC_CUDA_TRY(cudaGetDevice(&dev));
  OOC_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  // FP32 trailing matrix with a 16-byte-aligned base and leading dimension (the TMA
  // reduction's requirements): 256 x 128 blocks; otherwise the 128 x 128 kernel.
  if constexpr (sizeof(TC) == 4) {
    if (reinterpret_cast<uintptr_t>(C) % 16 == 0 && (ldc * (i64)sizeof(TC)) % 16 == 0) {
      CUtensorMap ah, al, mc;
      if (make_map(&ah, hi, Mp, Kp, TM2) || make_map(&al, lo, Mp, Kp, TM2) || make_map_c32(&mc, C, m, ldc)) {
        ooc_set_last_message("cuTensorMapEncodeTiled failed for the update operands");
        return OOC_ERR_CUDA;
      }
      const i64 nblk2 = count_blocks2((int)T, bj_lo, bj_hi);
      if (nblk2 <= 0) return OOC_OK;
      OOC_CUDA_TRY(
          cudaFuncSetAttribute(k_syrk2_bf16x3<TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2U_BYTES));
      const i64 grid2 = std::max<i64>(1, std::min<i64>(nblk2, std::max(1, nsm - std::max(0, reserve_sms))));
      // the launch's block tickets live in the 256 bytes after the two planes
      unsigned long long* tickets = reinterpret_cast<unsigned long long*>(lo + (size_t)Mp * Kp);
      OOC_CUDA_TRY(cudaMemsetAsync(tickets, 0, sizeof(unsigned long long), s));
      k_syrk2_bf16x3<TC><<<(unsigned)grid2, THREADS2, SMEM2U_BYTES, s>>>(ah, al, mh, ml, mc, m, Kp, (int)T, bj_lo,
                                                                         bj_hi, nblk2, tickets,
                                                                         const_cast<int*>(status));
      OOC_CUDA_TRY(cudaGetLastError());
      return OOC_OK;
    }
  }
  const i64 grid = std::max<i64>(1, std::min<i64>(nblk, std::max(1, nsm - std::max(0, reserve_sms))));
  k_syrk_bf16x3<TC><<<(unsigned)grid, THREADS, SMEM_BYTES, s>>>(mh, ml, C, ldc, m, Kp, (int)T, bj_lo, bj_hi, nblk,
                                                            const_cast<int*>(status));
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}
}  // namespace

int launch_syrk_bf16x3(const double* X, i64 ldx, double* C, i64 ldc, int m, int K, const int* status, cudaStream_t s,
                       void* work, size_t work_bytes, int bj_lo, int bj_hi, int do_split, int reserve_sms) {
  return launch_syrk_t<double, double>(X, ldx, C, ldc, m, K, status, s, work, work_bytes, bj_lo, bj_hi, do_split,
                                       reserve_sms);
}

// FP32 trailing matrix (reduced-precision factors): C (FP32) -= X X^T, X FP32.
int launch_syrk_bf16x3_f32(const float* X, i64 ldx, float* C, i64 ldc, int m, int K, const int* status,
                           cudaStream_t s, void* work, size_t work_bytes, int bj_lo, int bj_hi, int do_split,
                           int reserve_sms) {
  return launch_syrk_t<float, float>(X, ldx, C, ldc, m, K, status, s, work, work_bytes, bj_lo, bj_hi, do_split,
                                     reserve_sms);
}

// FP32 panel X (m x K, column-major, ld ldx) -> BF16 hi/lo planes at `work` (the layout of
// bf16x3_work_bytes(m, K): Mp x Kp row-major hi, then lo, zero-padded).
int launch_split_bf16_f32(const float* X, i64 ldx, int m, int K, void* work, size_t work_bytes, cudaStream_t s) {
  if (m <= 0 || K <= 0) return OOC_OK;
  if (work_bytes < bf16x3_work_bytes(m, K)) return OOC_ERR_INTERNAL;
  const int Mp = (m + TB - 1) / TB * TB;
  const int Kp = (K + TK - 1) / TK * TK;
  __nv_bfloat16* hi = (__nv_bfloat16*)work;
  __nv_bfloat16* lo = hi + (size_t)Mp * Kp;
  k_split_bf16<float><<<dim3((unsigned)(Kp / 32), (unsigned)(Mp / 32)), dim3(32, 8), 0, s>>>(X, ldx, hi, lo, m, K, Mp,
                                                                                          Kp);
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

// Column solve of an FP32 panel on the tensor cores, P = U X^T (k_trsm2_bf16x3).  `uwork`
// holds the planes of the panel before the solve (launch_split_bf16_f32, m x K) followed by
// the 256 bytes of block tickets; `xhi`, `xlo` the hi and lo planes of X = L_jj^{-1}
// (K x K, row-major, ld K).  The result goes to P (ld ldp) and, split, to the planes `ohi`,
// `olo` (row r's K values at r * ldo; rows past m are not written).  K must be a multiple
// of 128.
int launch_trsm_bf16x3_f32_to(void* uwork, size_t ubytes, const void* xhi, const void* xlo, float* P, i64 ldp, int m,
                              int K, void* ohi, void* olo, i64 ldo, const int* status, cudaStream_t s) {
  if (m <= 0 || K <= 0) return OOC_OK;
  if (K % TB != 0) return OOC_ERR_UNSUPPORTED;
  if (!status || !uwork || !xhi || !xlo || !ohi || !olo || ldo < K) return OOC_ERR_INTERNAL;
  if (ubytes < bf16x3_work_bytes(m, K)) return OOC_ERR_INTERNAL;
  int rc = get_encode();
  if (rc) return rc;
  const int Mp = (m + TB - 1) / TB * TB, Kp = K;
  __nv_bfloat16* uh = (__nv_bfloat16*)uwork;
  __nv_bfloat16* ul = uh + (size_t)Mp * Kp;
  unsigned long long* tickets = reinterpret_cast<unsigned long long*>(ul + (size_t)Mp * Kp);
  __nv_bfloat16* xh = (__nv_bfloat16*)const_cast<void*>(xhi);
  __nv_bfloat16* xl = (__nv_bfloat16*)const_cast<void*>(xlo);
  CUtensorMap mu_h, mu_l, mx_h, mx_l;
  if (make_map(&mu_h, uh, Mp, Kp, TM2) || make_map(&mu_l, ul, Mp, Kp, TM2) || make_map(&mx_h, xh, K, K, TB) ||
      make_map(&mx_l, xl, K, K, TB)) {
    ooc_set_last_message("cuTensorMapEncodeTiled failed for the column-solve planes");
    return OOC_ERR_CUDA;
  }
  const int ncb = K / TB;
  const i64 nblk = (i64)((Mp + TM2 - 1) / TM2) * ncb;
  int dev = 0, nsm = 0;
  OOC_CUDA_TRY(cudaGetDevice(&dev));
  OOC_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const i64 grid = std::max<i64>(1, std::min<i64>(nblk, nsm));
  OOC_CUDA_TRY(cudaFuncSetAttribute(k_trsm2_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2_BYTES));
  OOC_CUDA_TRY(cudaMemsetAsync(tickets, 0, sizeof(unsigned long long), s));
  k_trsm2_bf16x3<<<(unsigned)grid, THREADS2, SMEM2_BYTES, s>>>(mu_h, mu_l, mx_h, mx_l, P, ldp, (__nv_bfloat16*)ohi,
                                                              (__nv_bfloat16*)olo, ldo, Kp, m, ncb, nblk, tickets,
                                                              const_cast<int*>(status));
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

// The same with the result planes in `swork`, in the layout launch_syrk_bf16x3_f32 reads
// with do_split = 0 (Mp x K, hi then lo).
int launch_trsm_bf16x3_f32(void* uwork, size_t ubytes, const void* xhi, const void* xlo, float* P, i64 ldp, int m,
                           int K, void* swork, size_t sbytes, const int* status, cudaStream_t s) {
  if (m <= 0 || K <= 0) return OOC_OK;
  if (!swork || sbytes < bf16x3_work_bytes(m, K)) return OOC_ERR_INTERNAL;
  const size_t Mp = ((size_t)m + TB - 1) / TB * TB;
  __nv_bfloat16* sh = (__nv_bfloat16*)swork;
  return launch_trsm_bf16x3_f32_to(uwork, ubytes, xhi, xlo, P, ldp, m, K, sh, sh + Mp * (size_t)K, K, status, s);
}

// FP32 trailing matrix C (m x m, lower, ld ldc) -= X X^T restricted to the 128-wide block
// columns [bj_lo, bj_hi) (bj_hi < 0 = all), with X given as BF16 hi/lo planes already split:
// row r's K values at hi + r * ldk, lo + r * ldk (for example a window of a matrix-wide
// plane store: rows from the trailing matrix's first row, K over any run of finished
// panels).  `tickets` is 8 bytes of device memory for the launch's block counter.
int g_long_k = 2048;  // K from which the transposed kernel is used (OOC_SYRK_LONG_K overrides)
int launch_syrk_planes_f32(const void* hi, const void* lo, i64 ldk, int m, int K, float* C, i64 ldc,
                           const int* status, cudaStream_t s, unsigned long long* tickets, int bj_lo, int bj_hi,
                           int reserve_sms) {
  static const int kLongK = [] {
    const char* e = getenv("OOC_SYRK_LONG_K");
    return e ? atoi(e) : g_long_k;
  }();
  if (m <= 0 || K <= 0) return OOC_OK;
  if (!status || !hi || !lo || !tickets || K % TK != 0 || ldk < K) return OOC_ERR_INTERNAL;
  if ((reinterpret_cast<uintptr_t>(hi) | reinterpret_cast<uintptr_t>(lo) | (uintptr_t)(ldk * 2)) % 16 != 0)
    return OOC_ERR_INTERNAL;
  int rc = get_encode();
  if (rc) return rc;
  void* h = const_cast<void*>(hi);
  void* l = const_cast<void*>(lo);
  const i64 T = ((i64)m + TB - 1) / TB;
  bj_hi = (int)std::min<i64>(bj_hi < 0 ? T : bj_hi, T);
  if (bj_lo >= bj_hi) return OOC_OK;
  int dev = 0, nsm = 0;
  OOC_CUDA_TRY(cudaGetDevice(&dev));
  OOC_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const bool c16 = reinterpret_cast<uintptr_t>(C) % 16 == 0 && (ldc * (i64)sizeof(float)) % 16 == 0;
  // long K (catch-ups): the transposed N=256 kernel with its K=32 ring; short K: the K=512-tuned one
  const bool tr = c16 && K >= kLongK;
  CUtensorMap mh, ml;
  if (make_map(&mh, h, m, K, TB, ldk, tr) || make_map(&ml, l, m, K, TB, ldk, tr)) {
    ooc_set_last_message("cuTensorMapEncodeTiled failed for the plane-store window");
    return OOC_ERR_CUDA;
  }
  if (c16) {
    CUtensorMap ah, al, mc;
    if (make_map(&ah, h, m, K, TM2, ldk, tr) || make_map(&al, l, m, K, TM2, ldk, tr) ||
        (tr ? make_map_c32t(&mc, C, m, ldc) : make_map_c32(&mc, C, m, ldc))) {
      ooc_set_last_message("cuTensorMapEncodeTiled failed for the update operands");
      return OOC_ERR_CUDA;
    }
    const i64 nblk2 = count_blocks2((int)T, bj_lo, bj_hi);
    if (nblk2 <= 0) return OOC_OK;
    const i64 grid2 = std::max<i64>(1, std::min<i64>(nblk2, std::max(1, nsm - std::max(0, reserve_sms))));
    OOC_CUDA_TRY(cudaMemsetAsync(tickets, 0, sizeof(unsigned long long), s));
    if (tr) {
      OOC_CUDA_TRY(cudaFuncSetAttribute(k_syrk2t_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2T_BYTES));
      k_syrk2t_bf16x3<<<(unsigned)grid2, THREADS2, SMEM2T_BYTES, s>>>(ah, al, mh, ml, mc, m, K, (int)T, bj_lo, bj_hi,
                                                                       nblk2, tickets, const_cast<int*>(status));
    } else {
      OOC_CUDA_TRY(
          cudaFuncSetAttribute(k_syrk2_bf16x3<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2U_BYTES));
      k_syrk2_bf16x3<float><<<(unsigned)grid2, THREADS2, SMEM2U_BYTES, s>>>(ah, al, mh, ml, mc, m, K, (int)T, bj_lo,
                                                                            bj_hi, nblk2, tickets,
                                                                            const_cast<int*>(status));
    }
    OOC_CUDA_TRY(cudaGetLastError());
    return OOC_OK;
  }
  const i64 nblk = ooc_lower_blocks_before(bj_hi, T) - ooc_lower_blocks_before(bj_lo, T);
  OOC_CUDA_TRY(cudaFuncSetAttribute(k_syrk_bf16x3<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
  const i64 grid = std::max<i64>(1, std::min<i64>(nblk, std::max(1, nsm - std::max(0, reserve_sms))));
  k_syrk_bf16x3<float><<<(unsigned)grid, THREADS, SMEM_BYTES, s>>>(mh, ml, C, ldc, m, K, (int)T, bj_lo, bj_hi, nblk,
                                                                  const_cast<int*>(status));
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}
