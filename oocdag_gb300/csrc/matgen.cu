// Test-matrix generators, the scaled residual, and the FP64 peak probe.
//
// Generators write straight into device memory (or, through a device staging block,
// into host memory), so that a matrix that only fits in host memory is produced at
// copy-engine speed instead of on the host cores.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace {

// ---------------------------------------------------------------------------------
// Uniform generator: R(i,j) = u - 1/2, u = top 53 bits of SplitMix64 output number
// c = i + j*n (state started at mix(seed)); A = (R + R^T)/2 + alpha I.
// ---------------------------------------------------------------------------------
__host__ __device__ inline uint64_t sm64_mix(uint64_t z) { return ooc_sm64_mix(z); }

__global__ void k_gen_uniform(double* B, i64 ldb, i64 n, uint64_t key, double alpha, i64 r0, i64 c0,
                              i64 m, i64 nc) {
  const i64 ii = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= m) return;
  const i64 i = r0 + ii;
  for (i64 jj = blockIdx.y; jj < nc; jj += gridDim.y) B[ii + jj * ldb] = ooc_uniform_elem(key, n, alpha, i, c0 + jj);
}

// ---------------------------------------------------------------------------------
// pdmatgen('Symm','Diag') on a 1 x 1 grid: x_{k+1} = a x_k + c mod 2^31, u_k = x_k/2^31,
// A(i,j) = 1 - 2 u[min(i,j) n + max(i,j)], A(i,i) = |A(i,i)| + n.
// A thread owns one row and a run of columns; along the run it steps the stream by n
// (below the diagonal, index j*n + i) or by 1 (above it, index i*n + j).
// ---------------------------------------------------------------------------------
constexpr uint64_t LCG_A = 1103515245ULL, LCG_C = 12345ULL, LCG_M = 0x7FFFFFFFULL;

__host__ __device__ inline void lcg_jump(uint64_t k, uint64_t* ak, uint64_t* ck) {
  uint64_t ra = 1, rc = 0, ba = LCG_A, bc = LCG_C;
  while (k) {
    if (k & 1) { rc = (ba * rc + bc) & LCG_M; ra = (ba * ra) & LCG_M; }
    bc = (ba * bc + bc) & LCG_M;
    ba = (ba * ba) & LCG_M;
    k >>= 1;
  }
  *ak = ra;
  *ck = rc;
}

constexpr int PDM_RUN = 64;

__global__ void k_gen_pdmatgen(double* B, i64 ldb, i64 n, uint64_t x0, uint64_t an, uint64_t cn, i64 r0,
                               i64 c0, i64 m, i64 nc) {
  const i64 ii = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= m) return;
  const i64 i = r0 + ii;
  const i64 jj0 = (i64)blockIdx.y * PDM_RUN;
  if (jj0 >= nc) return;
  const i64 jj1 = min(nc, jj0 + PDM_RUN);
  i64 j = c0 + jj0;
  uint64_t ak, ck;
  lcg_jump((uint64_t)(j <= i ? j * n + i : i * n + j), &ak, &ck);
  uint64_t x = (ak * x0 + ck) & LCG_M;
  for (i64 jj = jj0; jj < jj1; jj++, j++) {
    double v = 1.0 - 2.0 * ((double)x / 2147483648.0);
    if (i == j) v = fabs(v) + (double)n;
    B[ii + jj * ldb] = v;
    // advance to column j+1 of row i
    if (j < i) x = (an * x + cn) & LCG_M;          // index (j+1)*n + i
    else x = (LCG_A * x + LCG_C) & LCG_M;          // index i*n + j + 1 (j >= i)
  }
}

// ---------------------------------------------------------------------------------
// Sum of squares of a (m x nc) block (and of a second block of the same shape):
// one partial per CTA, summed on the host in a fixed order.
// ---------------------------------------------------------------------------------
__global__ void k_sumsq2(const double* P, const double* A, i64 ld, i64 m, i64 nc, double* partial) {
  __shared__ double s1[256], s2[256];
  double a1 = 0, a2 = 0;
  const i64 total = m * nc;
  for (i64 idx = (i64)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (i64)gridDim.x * blockDim.x) {
    const i64 c = idx / m, r = idx % m;
    const double p = P[r + c * ld];
    a1 = fma(p, p, a1);
    const double a = A[r + c * ld];
    a2 = fma(a, a, a2);
  }
  s1[threadIdx.x] = a1;
  s2[threadIdx.x] = a2;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = s1[0];
    partial[2 * blockIdx.x + 1] = s2[0];
  }
}

// Copies the lower triangle of L (columns [c0, c0+w)) into Z (ld n), zeroing above.
__global__ void k_lower_copy(const double* L, i64 ldl, double* Z, i64 ldz, i64 n, i64 c0, i64 w) {
  const i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (i64 cc = blockIdx.y; cc < w; cc += gridDim.y) {
    const i64 c = c0 + cc;
    Z[r + c * ldz] = (r >= c) ? L[r + c * ldl] : 0.0;
  }
}

// FP64 DMMA issue loop for the peak probe: eight independent accumulator chains per
// thread so that MMA latency is hidden and only the pipe's issue rate remains.
__global__ void __launch_bounds__(256) k_dmma_probe(double* out, int iters) {
  double a = 1.0 + threadIdx.x * 1e-6, b = 1.0 - threadIdx.x * 1e-6;
  double c[16];
#pragma unroll
  for (int q = 0; q < 16; q++) c[q] = 0.0;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int q = 0; q < 8; q++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c[2 * q]), "+d"(c[2 * q + 1])
                   : "d"(a), "d"(b));
  }
  double s = 0;
#pragma unroll
  for (int q = 0; q < 16; q++) s += c[q];
  out[(i64)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

bool is_device_ptr(const void* p) {
  cudaPointerAttributes attr;
  memset(&attr, 0, sizeof(attr));
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

}  // namespace

int launch_gen_uniform_block(double* B, i64 ldb, i64 n, uint64_t seed, double alpha, i64 r0, i64 c0, i64 m,
                             i64 nc, cudaStream_t s) {
  if (m <= 0 || nc <= 0) return OOC_OK;
  const uint64_t key = sm64_mix(seed + 0x9E3779B97F4A7C15ULL);
  dim3 grid((unsigned)((m + 255) / 256), (unsigned)std::min<i64>(nc, 4096));
  k_gen_uniform<<<grid, 256, 0, s>>>(B, ldb, n, key, alpha, r0, c0, m, nc);
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

int launch_gen_pdmatgen_block(double* B, i64 ldb, i64 n, int seed, i64 r0, i64 c0, i64 m, i64 nc,
                              cudaStream_t s) {
  if (m <= 0 || nc <= 0) return OOC_OK;
  const uint64_t x0 = (LCG_A * (uint64_t)(uint32_t)seed + LCG_C) & LCG_M;
  uint64_t an, cn;
  lcg_jump((uint64_t)n, &an, &cn);
  const i64 runs = (nc + PDM_RUN - 1) / PDM_RUN;
  if (runs > 65535) return OOC_ERR_INTERNAL;
  dim3 grid((unsigned)((m + 127) / 128), (unsigned)runs);
  k_gen_pdmatgen<<<grid, 128, 0, s>>>(B, ldb, n, x0, an, cn, r0, c0, m, nc);
  OOC_CUDA_TRY(cudaGetLastError());
  return OOC_OK;
}

namespace {

// Generates the whole matrix into A (device, or host through a staging block).
int gen_matrix(ooc_handle* h, double* A, i64 n, i64 lda, int kind, uint64_t seed, double alpha) {
  cudaStream_t s = ooc_compute_stream(h);
  auto gen = [&](double* B, i64 ldb, i64 c0, i64 nc) {
    return kind == 0 ? launch_gen_uniform_block(B, ldb, n, seed, alpha, 0, c0, n, nc, s)
                     : launch_gen_pdmatgen_block(B, ldb, n, (int)seed, 0, c0, n, nc, s);
  };
  if (is_device_ptr(A)) {
    for (i64 c0 = 0; c0 < n; c0 += 65535 * PDM_RUN / 2) {
      const i64 nc = std::min<i64>(n - c0, 65535 * PDM_RUN / 2);
      int rc = gen(A + c0 * lda, lda, c0, nc);
      if (rc) return rc;
    }
    return ooc_wait_stream(h, s);
  }
  // Host destination: two staging blocks of ~256 MB, generated and copied alternately.
  const i64 w = std::max<i64>(1, std::min<i64>(n, (i64)(256LL << 20) / (8 * n)));
  double* stage = nullptr;
  if (cudaMalloc(&stage, 2 * (size_t)w * n * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return OOC_ERR_NOMEM;
  }
  int rc = OOC_OK;
  int b = 0;
  for (i64 c0 = 0; c0 < n && rc == OOC_OK; c0 += w, b ^= 1) {
    const i64 nc = std::min<i64>(w, n - c0);
    double* B = stage + (size_t)b * w * n;
    rc = gen(B, n, c0, nc);
    if (rc) break;
    cudaError_t e = cudaMemcpy2DAsync(A + c0 * lda, lda * sizeof(double), B, n * sizeof(double),
                                      n * sizeof(double), nc, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) { ooc_set_last_error(e, "cudaMemcpy2DAsync", __FILE__, __LINE__); rc = OOC_ERR_CUDA; }
  }
  int rc2 = ooc_wait_stream(h, s);
  cudaFree(stage);
  return rc ? rc : rc2;
}

}  // namespace

extern "C" int ooc_dmatgen_uniform(ooc_handle* h, double* A, int64_t n, int64_t lda, uint64_t seed,
                                   double alpha) {
  if (!h) return -1;
  if (!A && n > 0) return -2;
  if (n < 0) return -3;
  if (lda < std::max<int64_t>(1, n)) return -4;
  if (n == 0) return OOC_OK;
  cudaSetDevice(ooc_device(h));
  return gen_matrix(h, A, n, lda, 0, seed, alpha);
}

extern "C" int ooc_dmatgen_pdmatgen(ooc_handle* h, double* A, int64_t n, int64_t lda, int seed) {
  if (!h) return -1;
  if (!A && n > 0) return -2;
  if (n < 0) return -3;
  if (lda < std::max<int64_t>(1, n)) return -4;
  if (n == 0) return OOC_OK;
  cudaSetDevice(ooc_device(h));
  return gen_matrix(h, A, n, lda, 1, (uint64_t)(uint32_t)seed, 0.0);
}

// ||A - L L^T||_F / (n eps ||A||_F).  The lower triangle of L is copied into a zero-
// padded device copy Z; then for every block column J (width t), the block
// P = A(J:, J) - Z(J:, 0:J+t) Z(J, 0:J+t)^T is formed with A regenerated in place and
// its squares summed (diagonal block once, blocks below twice, by symmetry).
extern "C" int ooc_dresidual(ooc_handle* h, const double* L, int64_t n, int64_t lda, int kind, uint64_t seed,
                             double alpha, double* resid) {
  if (!h) return -1;
  if (!L && n > 0) return -2;
  if (n < 0) return -3;
  if (lda < std::max<int64_t>(1, n)) return -4;
  if (kind != 0 && kind != 1) return -5;
  if (!resid) return -8;
  *resid = 0;
  if (n == 0) return OOC_OK;
  cudaSetDevice(ooc_device(h));
  cudaStream_t s = ooc_compute_stream(h);
  const int t = 512;
  double *Z = nullptr, *P = nullptr, *Ablk = nullptr, *part = nullptr;
  const int nparts = 304;
  size_t zbytes = (size_t)n * n * sizeof(double);
  if (cudaMalloc(&Z, zbytes) != cudaSuccess || cudaMalloc(&P, (size_t)n * t * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&Ablk, (size_t)n * t * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&part, 2 * nparts * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    if (Z) cudaFree(Z);
    if (P) cudaFree(P);
    if (Ablk) cudaFree(Ablk);
    return OOC_ERR_NOMEM;
  }
  int rc = OOC_OK;
  const bool dev = is_device_ptr(L);
  double* Lsrc = nullptr;
  if (!dev) {
    // Host factor: stage it column block by column block.
    if (cudaMalloc(&Lsrc, (size_t)n * t * sizeof(double)) != cudaSuccess) { cudaGetLastError(); rc = OOC_ERR_NOMEM; }
  }
  for (i64 c0 = 0; c0 < n && rc == OOC_OK; c0 += t) {
    const i64 w = std::min<i64>(t, n - c0);
    const double* src = L + c0 * lda;
    i64 lds = lda;
    if (!dev) {
      if (cudaMemcpy2DAsync(Lsrc, n * sizeof(double), src, lda * sizeof(double), n * sizeof(double), w,
                            cudaMemcpyHostToDevice, s) != cudaSuccess) { rc = OOC_ERR_CUDA; break; }
      src = Lsrc;
      lds = n;
      k_lower_copy<<<dim3((unsigned)((n + 255) / 256), (unsigned)w), 256, 0, s>>>(src - c0 * lds, lds, Z, n, n, c0, w);
    } else {
      k_lower_copy<<<dim3((unsigned)((n + 255) / 256), (unsigned)w), 256, 0, s>>>(L, lda, Z, n, n, c0, w);
    }
  }
  std::vector<double> hp(2 * nparts);
  double sumR = 0, sumA = 0;
  for (i64 J = 0; J < n && rc == OOC_OK; J += t) {
    const i64 w = std::min<i64>(t, n - J);
    const i64 m = n - J;
    rc = (kind == 0) ? launch_gen_uniform_block(P, n, n, seed, alpha, J, J, m, w, s)
                     : launch_gen_pdmatgen_block(P, n, n, (int)seed, J, J, m, w, s);
    if (rc) break;
    if (cudaMemcpyAsync(Ablk, P, (size_t)n * w * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      rc = OOC_ERR_CUDA;
      break;
    }
    rc = launch_gemm_nt(Z + J, n, Z + J, n, P, n, (int)m, (int)w, (int)(J + w), 0, -1.0, nullptr, s);
    if (rc) break;
    // diagonal block (rows J..J+w) once, the rest twice: two reductions.
    double sums[4] = {0, 0, 0, 0};
    for (int part_i = 0; part_i < 2; part_i++) {
      const i64 r0 = part_i == 0 ? 0 : w;
      const i64 rows = part_i == 0 ? w : m - w;
      if (rows <= 0) continue;
      k_sumsq2<<<nparts, 256, 0, s>>>(P + r0, Ablk + r0, n, rows, w, part);
      if (cudaMemcpyAsync(hp.data(), part, 2 * nparts * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) {
        rc = OOC_ERR_CUDA;
        break;
      }
      rc = ooc_wait_stream(h, s);
      if (rc) break;
      for (int q = 0; q < nparts; q++) { sums[2 * part_i] += hp[2 * q]; sums[2 * part_i + 1] += hp[2 * q + 1]; }
    }
    sumR += sums[0] + 2 * sums[2];
    sumA += sums[1] + 2 * sums[3];
  }
  if (rc == OOC_OK) rc = ooc_wait_stream(h, s);
  cudaFree(Z);
  cudaFree(P);
  cudaFree(Ablk);
  cudaFree(part);
  if (Lsrc) cudaFree(Lsrc);
  if (rc) return rc;
  *resid = std::sqrt(sumR) / ((double)n * 0x1.0p-53 * std::sqrt(sumA));
  return OOC_OK;
}

extern "C" int ooc_fp64_peak_probe(ooc_handle* h, double ms, double* tflops) {
  if (!h) return -1;
  if (!(ms > 0)) return -2;
  if (!tflops) return -3;
  cudaSetDevice(ooc_device(h));
  int dev = ooc_device(h), nsm = 0;
  OOC_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = nsm * 4, threads = 256;
  double* out = nullptr;
  OOC_CUDA_TRY(cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaStream_t s = ooc_compute_stream(h);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int iters = 256;
  float el = 0;
  double rate = 0;
  for (int rep = 0; rep < 8; rep++) {
    cudaEventRecord(e0, s);
    k_dmma_probe<<<blocks, threads, 0, s>>>(out, iters);
    cudaEventRecord(e1, s);
    int rc = ooc_wait_stream(h, s);
    if (rc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      cudaFree(out);
      return rc;
    }
    cudaEventElapsedTime(&el, e0, e1);
    double flops = 2.0 * 8 * 8 * 4 * 8.0 * iters * (double)blocks * (threads / 32);
    rate = flops / (el * 1e-3) / 1e12;
    if (el >= ms) break;
    iters = (int)std::min(1e8, iters * std::max(2.0, ms / std::max(el, 1e-3f) * 1.1));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaError_t e = cudaGetLastError();
  cudaFree(out);
  if (e != cudaSuccess) { ooc_set_last_error(e, "k_dmma_probe", __FILE__, __LINE__); return OOC_ERR_CUDA; }
  *tflops = rate;
  return OOC_OK;
}
