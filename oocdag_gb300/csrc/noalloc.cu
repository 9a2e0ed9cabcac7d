// Out-of-core Cholesky entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: a process whose device memory is owned by another
// allocator (a framework's caching pool that has already reserved the GPU's memory, so a
// fresh allocation fails or fragments it), or a latency-sensitive server that must not
// let cudaMalloc / cudaFree synchronize the device while its other streams run.
// ooc_dpotrf_L needs a device panel buffer and a status word, which its handle allocates;
// this variant takes both from a fixed-size array in the library's own static device
// memory instead, and runs entirely on the caller's stream.
//
// The array is OOC_STATIC_PANEL_BYTES (64 MiB) of device memory that every GPU which
// loads this library holds until the process exits.  All calls share it and it keeps
// whatever the last call left there, so the status word is cleared at the start of every
// call; two calls whose work overlaps on the GPU (for example from two host threads on
// two streams) race on the array and must be serialized by the caller.

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <mutex>
#include <string>
#include <thread>

#include "common.cuh"

namespace {

constexpr size_t kStaticBytes = (size_t)OOC_STATIC_PANEL_BYTES;
static_assert(kStaticBytes % 256 == 0, "static panel size must keep 256-byte alignment");

// Static device scratch: the panel buffer, and the status word in its own small array.
static __device__ __align__(256) double g_static_panel[kStaticBytes / sizeof(double)];
static __device__ __align__(256) int g_static_status[64];

// Device addresses of the arrays above, looked up (set-up) once per device context with
// that context current.  In host code the array names are host-side stand-ins, never
// device addresses: only these looked-up pointers are passed to kernels and copies.
// The cache is keyed by the driver's context ID, not by the device number: when a
// caller resets the device (cudaDeviceReset, or another library resetting the primary
// context), the next context loads the module afresh and the arrays may sit at other
// addresses, so a new context ID means a new lookup.  IDs are never reused within a
// process.  Without the driver entry points the lookup runs on every call (it
// allocates nothing).
struct StaticPtrs {
  double* panel = nullptr;
  int* status = nullptr;
  unsigned long long ctx_id = 0;
  bool ready = false;
};
std::mutex g_mu;
StaticPtrs g_ptrs[64];

typedef CUresult (*ctx_get_current_t)(CUcontext*);
typedef CUresult (*ctx_get_id_t)(CUcontext, unsigned long long*);
ctx_get_current_t g_ctx_current = nullptr;
ctx_get_id_t g_ctx_id = nullptr;
std::once_flag g_entry_once;

// ID of the context current on this thread; false if there is none or it is unknown.
bool current_context_id(unsigned long long* id) {
  std::call_once(g_entry_once, [] {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qb == cudaDriverEntryPointSuccess) {
      g_ctx_current = (ctx_get_current_t)a;
      g_ctx_id = (ctx_get_id_t)b;
    }
  });
  if (!g_ctx_current || !g_ctx_id) return false;
  CUcontext ctx = nullptr;
  if (g_ctx_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
  return g_ctx_id(ctx, id) == CUDA_SUCCESS;
}

int static_setup(int dev, StaticPtrs* out) {
  if (dev < 0 || dev >= 64) return OOC_ERR_NODEVICE;
  std::lock_guard<std::mutex> lk(g_mu);
  StaticPtrs& p = g_ptrs[dev];
  unsigned long long id = 0;
  if (p.ready && current_context_id(&id) && id == p.ctx_id) {
    *out = p;
    return OOC_OK;
  }
  p.ready = false;
  void* a = nullptr;
  void* b = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&a, g_static_panel);  // also initialises the context
  if (e != cudaSuccess) {
    ooc_set_last_error(e, "cudaGetSymbolAddress(g_static_panel)", __FILE__, __LINE__);
    return OOC_ERR_CUDA;
  }
  e = cudaGetSymbolAddress(&b, g_static_status);
  if (e != cudaSuccess) {
    ooc_set_last_error(e, "cudaGetSymbolAddress(g_static_status)", __FILE__, __LINE__);
    return OOC_ERR_CUDA;
  }
  p.panel = (double*)a;
  p.status = (int*)b;
  p.ready = current_context_id(&p.ctx_id);  // cached only when the context is known
  *out = p;
  return OOC_OK;
}

// Panel width as the reference chooses it (oocdag.cpp:478-492) with its single X buffer.
int width_one_x(int bb, i64 memBlock, int jb, int* state) {
  int Yn = *state;
  const i64 Ym = bb - jb;
  const i64 room = (memBlock - Ym) * 2;
  if (Ym * (Ym + 1) <= room) {
    Yn = (int)Ym;
  } else {
    while (room >= (2 * Ym - Yn) * (i64)(Yn + 1)) {
      if (Yn == Ym) break;
      Yn++;
    }
  }
  *state = Yn;
  return Yn;
}

// Waits for the caller's stream without creating an event, bounded in time.
int wait_stream_bounded(cudaStream_t s, int64_t timeout_ms) {
  auto t0 = std::chrono::steady_clock::now();
  for (int spin = 0;; spin++) {
    cudaError_t q = cudaStreamQuery(s);
    if (q == cudaSuccess) return OOC_OK;
    if (q != cudaErrorNotReady) {
      ooc_set_last_error(q, "cudaStreamQuery", __FILE__, __LINE__);
      return OOC_ERR_CUDA;
    }
    auto el = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0);
    if (el.count() > timeout_ms) return OOC_ERR_TIMEOUT;
    if (spin > 64) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

// One panel update, split by tile columns when the trapezoid has more tile pairs than a
// launch's grid.y can hold (only with very small tiles).
int update_split(const TileCol& X, const TileMap& C, int Ht, int Kt, i64 H, i64 Kc, int K, const int* status,
                 cudaStream_t s) {
  int j0 = 0;
  while (j0 < Kt) {
    int j1 = j0;
    i64 cnt = 0;
    while (j1 < Kt && cnt + (Ht - j1) <= 65535) { cnt += Ht - j1; j1++; }
    TileMap Cs = C;
    Cs.base = tile_ptr(C, j0, j0);
    Cs.Ym = C.Ym - j0;
    TileCol Xs = X;
    Xs.base = X.base + (i64)j0 * X.stride;
    int rc = launch_panel_update(Xs, Cs, Ht - j0, j1 - j0, H - (i64)j0 * C.nb, Kc - (i64)j0 * C.nb, K, status, s);
    if (rc) return rc;
    j0 = j1;
  }
  return OOC_OK;
}

#define NA_TRY(expr)                                         \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) {                                 \
      ooc_set_last_error(_e, #expr, __FILE__, __LINE__);     \
      return OOC_ERR_CUDA;                                   \
    }                                                        \
  } while (0)

// The panel rule with one X buffer needs at least 2 * ceil(n/nb) tiles for the first
// panel (oocdag.cpp:483-486 with Yn = 1: (memBlock - Ym) * 2 >= 2 * Ym).  Host only.
int check_fits(i64 n, int nb) {
  const i64 bb = (n + nb - 1) / nb;
  const i64 memBlock = (i64)(kStaticBytes / sizeof(double) / ((size_t)nb * (size_t)nb));
  if (memBlock < 2 * bb) {
    char buf[256];
    snprintf(buf, sizeof(buf),
             "ooc_dpotrf_L_static: n=%lld with nb=%d needs more than the %zu-byte static panel buffer "
             "(%lld tiles of %d x %d available, at least %lld needed)",
             (long long)n, nb, kStaticBytes, (long long)memBlock, nb, nb, 2LL * bb);
    ooc_set_last_message(buf);
    return OOC_ERR_BUDGET;
  }
  return OOC_OK;
}

int run_static(double* A, i64 n, i64 lda, int nb, cudaStream_t s, const StaticPtrs& P, int* info) {
  const int bb = (int)((n + nb - 1) / nb);
  const i64 tile = (i64)nb * nb;
  const i64 memBlock = (i64)(kStaticBytes / sizeof(double) / (size_t)tile);
  double* Y = P.panel;
  int* status = P.status;
  NA_TRY(cudaMemsetAsync(status, 0, sizeof(int), s));  // the shared word keeps the last call's value
  int state = 0;
  i64 JB = 0;
  int jb = 0;
  while (JB < n) {
    const int Ym = bb - jb;
    const int Yn = width_one_x(bb, memBlock, jb, &state);
    const i64 YM = n - JB;
    const i64 YN = std::min<i64>((i64)(jb + Yn) * nb, n) - JB;
    double* X = Y + (memBlock - Ym) * tile;
    double* Apan = A + JB + JB * lda;
    TileMap Pm{Y, nb, 1, Ym, nb};
    // panel in (oocquark.cpp:253-275)
    for (int j = 0; j < Yn; j++) {
      const i64 LN = std::min<i64>(nb, YN - (i64)j * nb);
      for (int i = j; i < Ym; i++) {
        const i64 LM = std::min<i64>(nb, YM - (i64)i * nb);
        NA_TRY(cudaMemcpy2DAsync(tile_ptr(Pm, i, j), nb * sizeof(double), Apan + (i64)i * nb + (i64)j * nb * lda,
                                 lda * sizeof(double), LM * sizeof(double), LN, cudaMemcpyDefault, s));
      }
    }
    // left-looking updates, one X column at a time through the single X buffer
    for (int jjb = 0; jjb < jb; jjb++) {
      const double* Acol = A + JB + (i64)jjb * nb * lda;
      for (int i = 0; i < Ym; i++) {
        const i64 LM = std::min<i64>(nb, YM - (i64)i * nb);
        NA_TRY(cudaMemcpy2DAsync(X + i * tile, nb * sizeof(double), Acol + (i64)i * nb, lda * sizeof(double),
                                 LM * sizeof(double), nb, cudaMemcpyDefault, s));
      }
      int rc = update_split(TileCol{X, nb, tile}, Pm, Ym, Yn, YM, YN, nb, status, s);
      if (rc) return rc;
    }
    // in-panel factorization with copy-back (oocquark.cpp:389-419)
    for (int j = 0; j < Yn; j++) {
      const int LN = (int)std::min<i64>(nb, YN - (i64)j * nb);
      double* Djj = tile_ptr(Pm, j, j);
      int rc = launch_potrf_tile(Djj, nb, LN, JB + (i64)j * nb, status, s);
      if (rc) return rc;
      if (Ym - j - 1 > 0) {
        const int m_last = (int)(YM - (i64)(Ym - 1) * nb);
        rc = launch_trsm_col(Djj, nb, TileCol{tile_ptr(Pm, j + 1, j), nb, tile}, Ym - j - 1, nb, m_last, LN,
                             status, s);
        if (rc) return rc;
      }
      for (int i = j; i < Ym; i++) {
        const i64 LM = std::min<i64>(nb, YM - (i64)i * nb);
        NA_TRY(cudaMemcpy2DAsync(Apan + (i64)i * nb + (i64)j * nb * lda, lda * sizeof(double), tile_ptr(Pm, i, j),
                                 nb * sizeof(double), LM * sizeof(double), LN, cudaMemcpyDefault, s));
      }
      if (j + 1 < Yn) {
        TileMap C = Pm;
        C.base = tile_ptr(Pm, j + 1, j + 1);
        C.Ym = Ym - j - 1;
        rc = update_split(TileCol{tile_ptr(Pm, j + 1, j), nb, tile}, C, Ym - j - 1, Yn - j - 1,
                                 YM - (i64)(j + 1) * nb, YN - (i64)(j + 1) * nb, nb, status, s);
        if (rc) return rc;
      }
    }
    JB += YN;
    jb += Yn;
  }
  // Wait (bounded) for the stream, then read the status word.  The host word is pageable
  // stack memory, so the copy returns only once it is done; with the stream idle it
  // finishes at once and never waits without bound.
  int rc = wait_stream_bounded(s, 6LL * 3600 * 1000);
  if (rc) return rc;
  int host_status = 0;
  NA_TRY(cudaMemcpyAsync(&host_status, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  rc = wait_stream_bounded(s, 60LL * 1000);
  if (rc) return rc;
  *info = host_status;
  return OOC_OK;
}

}  // namespace

extern "C" int ooc_dpotrf_L_static(double* A, int64_t n, int64_t lda, int nb, void* stream, int* info) {
  if (!A && n > 0) return -1;
  if (n < 0) return -2;
  if (lda < std::max<int64_t>(1, n)) return -3;
  if (nb <= 0) return -4;
  if (!info) return -6;
  *info = 0;
  if (n == 0) return OOC_OK;
  int rc = check_fits(n, nb);  // host arithmetic only: no device call before it
  if (rc) return rc;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    ooc_set_last_error(e, "cudaGetDevice", __FILE__, __LINE__);
    return OOC_ERR_NODEVICE;
  }
  StaticPtrs P;
  rc = static_setup(dev, &P);
  if (rc) return rc;
  return run_static(A, n, lda, nb, (cudaStream_t)stream, P, info);
}
