// Out-of-core left-looking Cholesky driver: the panel loop of the reference
// (oocdag.cpp:18-112) and its task graph (oocquark.cpp:253-421), rebuilt on three CUDA
// streams of one GPU.
//
//   reference (QUARK tasks, 4 threads)        here (streams + events)
//   ---------------------------------------  -------------------------------------------
//   A2Y   H2D task per panel tile              s_h2d: one 2-D async copy per tile from the
//                                            page-locked host matrix into the packed panel
//   A2X   H2D task per tile of column jjb      s_h2d: same, into X buffer jjb % 2, waiting
//         (single X buffer: WAR on X)          on the update that last read that buffer
//   ooc_syrk  dsyrk/dgemm task per tile pair   s_comp: ONE launch per X column covering
//                                            every tile pair of the panel (FP64 DMMA)
//   ooc_incore  host dpotrf round trip,        s_comp: device potrf of the diagonal tile,
//               dtrsm + D2H per tile,          one column solve launch sequence, trailing
//               trailing ooc_syrk              update launch; s_d2h copies each finished
//                                            column back while s_comp moves on
//   QUARK_Barrier                              one bounded wait at the end
//
// Hazards QUARK tracked by tile address become events: Y is reused across panels
// (next panel's copies wait for this panel's compute and copy-back), host tiles written
// back by one panel are read by later panels' A2X (ordered by the same wait), X buffers
// are reused every other column (copy waits for the update that read it).

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <memory>
#include <vector>

#include "common.cuh"
#include "devpool.cuh"

// ---------------------------------------------------------------------------------
// Error reporting
// ---------------------------------------------------------------------------------
static thread_local std::string g_last_error;

void ooc_set_last_error(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  g_last_error = buf;
}

void ooc_set_last_message(const char* msg) { g_last_error = msg; }

extern "C" const char* ooc_last_error_string(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------------
// Handle
// ---------------------------------------------------------------------------------
struct ooc_handle {
  int device = 0;
  cudaStream_t s_h2d = nullptr, s_comp = nullptr, s_d2h = nullptr;
  cudaStream_t s_h2d2 = nullptr;  // a second host-to-device copy stream (two copy engines in flight)
  int* d_status = nullptr;
  int* h_status = nullptr;  // page-locked mirror
  double* d_buf = nullptr;
  size_t d_buf_bytes = 0;
  int x_buffers = 2;
  int64_t timeout_ms = 6LL * 3600 * 1000;
  int profile = 0;
  int pin_host = 1;
  int ref_schedule = 0;
  int keep_a = 0;
  int64_t tail_order = 24576;
  int64_t block_cols = -1;  // OOC_OPT_BLOCK_COLS (-1: by input)
  int copy_streams = 2;      // OOC_OPT_COPY_STREAMS
  std::shared_ptr<DevPool> pool;  // device buffers of the handle's factor objects
  GrowBuf batch_ws;               // launch tables of the batched solvers
  GrowBuf solve_ws;               // panels and vectors of ooc_dpotrs_L
  int last_info = 0;
  std::vector<cudaEvent_t> ev_pool;  // reusable timing-free events
  size_t ev_next = 0;
  std::vector<cudaEvent_t> prof_pool;  // timing events for the profile option
  size_t prof_next = 0;
  cudaEvent_t ev_wait = nullptr;  // used only by bounded stream waits
};

namespace {

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

cudaError_t next_event(ooc_handle* h, cudaEvent_t* ev) {
  if (h->ev_next == h->ev_pool.size()) {
    cudaEvent_t e;
    cudaError_t rc = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (rc != cudaSuccess) return rc;
    h->ev_pool.push_back(e);
  }
  *ev = h->ev_pool[h->ev_next++];
  return cudaSuccess;
}

cudaError_t next_prof_event(ooc_handle* h, cudaEvent_t* ev) {
  if (h->prof_next == h->prof_pool.size()) {
    cudaEvent_t e;
    cudaError_t rc = cudaEventCreate(&e);
    if (rc != cudaSuccess) return rc;
    h->prof_pool.push_back(e);
  }
  *ev = h->prof_pool[h->prof_next++];
  return cudaSuccess;
}

// Bounded wait: polls the event until it completes or the handle's timeout passes.
int wait_event(ooc_handle* h, cudaEvent_t ev) {
  auto t0 = std::chrono::steady_clock::now();
  for (int spin = 0;; spin++) {
    cudaError_t q = cudaEventQuery(ev);
    if (q == cudaSuccess) return OOC_OK;
    if (q != cudaErrorNotReady) {
      ooc_set_last_error(q, "cudaEventQuery", __FILE__, __LINE__);
      return OOC_ERR_CUDA;
    }
    auto el = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0);
    if (el.count() > h->timeout_ms) {
      g_last_error = "bounded wait for the device timed out";
      return OOC_ERR_TIMEOUT;
    }
    if (spin > 64) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

}  // namespace

extern "C" int ooc_create(ooc_handle** out, int device) {
  if (!out) return -1;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    g_last_error = "no CUDA device";
    return OOC_ERR_NODEVICE;
  }
  if (device < 0 || device >= ndev) return OOC_ERR_NODEVICE;
  ooc_handle* h = new (std::nothrow) ooc_handle();
  if (!h) return OOC_ERR_NOMEM;
  h->device = device;
  DeviceGuard g(device);
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  // Copies run at the higher priority, as the reference gives copy tasks priority 1
  // (oocquark.cpp:260).
  if (cudaStreamCreateWithPriority(&h->s_h2d, cudaStreamNonBlocking, hi) != cudaSuccess ||
      cudaStreamCreateWithPriority(&h->s_d2h, cudaStreamNonBlocking, hi) != cudaSuccess ||
      cudaStreamCreateWithPriority(&h->s_h2d2, cudaStreamNonBlocking, hi) != cudaSuccess ||
      cudaStreamCreateWithPriority(&h->s_comp, cudaStreamNonBlocking, lo) != cudaSuccess ||
      cudaMalloc(&h->d_status, sizeof(int)) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_wait, cudaEventDisableTiming) != cudaSuccess ||
      cudaHostAlloc(&h->h_status, sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
    ooc_destroy(h);
    g_last_error = "handle creation failed";
    return OOC_ERR_CUDA;
  }
  h->pool = std::make_shared<DevPool>();
  h->pool->device = device;
  {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    h->pool->cap = tot / 10 * 4;  // default: 40 % of the device memory may stay cached
  }
  *out = h;
  return OOC_OK;
}

std::shared_ptr<DevPool> ooc_handle_pool(ooc_handle* h) { return h ? h->pool : nullptr; }
GrowBuf* ooc_handle_batch_ws(ooc_handle* h) { return h ? &h->batch_ws : nullptr; }
GrowBuf* ooc_handle_solve_ws(ooc_handle* h) { return h ? &h->solve_ws : nullptr; }

extern "C" int ooc_destroy(ooc_handle* h) {
  if (!h) return OOC_OK;
  {
    DeviceGuard g(h->device);
    if (h->s_h2d) cudaStreamSynchronize(h->s_h2d);
    if (h->s_comp) cudaStreamSynchronize(h->s_comp);
    if (h->s_d2h) cudaStreamSynchronize(h->s_d2h);
    if (h->s_h2d2) cudaStreamSynchronize(h->s_h2d2);
    for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : h->prof_pool) cudaEventDestroy(e);
    if (h->ev_wait) cudaEventDestroy(h->ev_wait);
    if (h->d_buf) cudaFree(h->d_buf);
    h->batch_ws.release();
    h->solve_ws.release();
    if (h->d_status) cudaFree(h->d_status);
    if (h->h_status) cudaFreeHost(h->h_status);
    if (h->s_h2d) cudaStreamDestroy(h->s_h2d);
    if (h->s_comp) cudaStreamDestroy(h->s_comp);
    if (h->s_d2h) cudaStreamDestroy(h->s_d2h);
    if (h->s_h2d2) cudaStreamDestroy(h->s_h2d2);
  }
  delete h;
  return OOC_OK;
}

extern "C" int ooc_set_option(ooc_handle* h, int key, int64_t v) {
  if (!h) return -1;
  switch (key) {
    case OOC_OPT_X_BUFFERS:
      if (v != 1 && v != 2) return -3;
      h->x_buffers = (int)v;
      return OOC_OK;
    case OOC_OPT_TIMEOUT_MS:
      if (v <= 0) return -3;
      h->timeout_ms = v;
      return OOC_OK;
    case OOC_OPT_PROFILE: h->profile = v ? 1 : 0; return OOC_OK;
    case OOC_OPT_PIN_HOST: h->pin_host = v ? 1 : 0; return OOC_OK;
    case OOC_OPT_REF_SCHEDULE: h->ref_schedule = v ? 1 : 0; return OOC_OK;
    case OOC_OPT_KEEP_A: h->keep_a = v ? 1 : 0; return OOC_OK;
    case OOC_OPT_TAIL_ORDER:
      if (v < 0) return -3;
      h->tail_order = v;
      return OOC_OK;
    case OOC_OPT_POOL_BYTES:
      if (v < 0) return -3;
      if (h->pool) h->pool->set_cap((size_t)v);
      return OOC_OK;
    case OOC_OPT_BLOCK_COLS:
      if (v < -1) return -3;
      h->block_cols = v;
      return OOC_OK;
    case OOC_OPT_COPY_STREAMS:
      if (v < 1 || v > 2) return -3;
      h->copy_streams = (int)v;
      return OOC_OK;
    default: return -2;
  }
}

extern "C" int ooc_get_option(ooc_handle* h, int key, int64_t* v) {
  if (!h) return -1;
  if (!v) return -3;
  switch (key) {
    case OOC_OPT_X_BUFFERS: *v = h->x_buffers; return OOC_OK;
    case OOC_OPT_TIMEOUT_MS: *v = h->timeout_ms; return OOC_OK;
    case OOC_OPT_PROFILE: *v = h->profile; return OOC_OK;
    case OOC_OPT_PIN_HOST: *v = h->pin_host; return OOC_OK;
    case OOC_OPT_REF_SCHEDULE: *v = h->ref_schedule; return OOC_OK;
    case OOC_OPT_KEEP_A: *v = h->keep_a; return OOC_OK;
    case OOC_OPT_TAIL_ORDER: *v = h->tail_order; return OOC_OK;
    case OOC_OPT_POOL_BYTES: *v = h->pool ? (int64_t)h->pool->cap : 0; return OOC_OK;
    case OOC_OPT_BLOCK_COLS: *v = h->block_cols; return OOC_OK;
    case OOC_OPT_COPY_STREAMS: *v = h->copy_streams; return OOC_OK;
    default: return -2;
  }
}

extern "C" int ooc_last_info(ooc_handle* h) { return h ? h->last_info : 0; }

extern "C" int ooc_get_stream(ooc_handle* h, int which, void** stream) {
  if (!h) return -1;
  if (!stream) return -3;
  switch (which) {
    case 0: *stream = (void*)h->s_comp; return OOC_OK;
    case 1: *stream = (void*)h->s_h2d; return OOC_OK;
    case 2: *stream = (void*)h->s_d2h; return OOC_OK;
    case 3: *stream = (void*)h->s_h2d2; return OOC_OK;
    default: return -2;
  }
}

// Shared with the other translation units.
cudaStream_t ooc_compute_stream(ooc_handle* h) { return h->s_comp; }
int ooc_device(ooc_handle* h) { return h->device; }
int ooc_wait_stream(ooc_handle* h, cudaStream_t s) {
  OOC_CUDA_TRY(cudaEventRecord(h->ev_wait, s));
  return wait_event(h, h->ev_wait);
}

// ---------------------------------------------------------------------------------
// Panel sizing.  With nx = 1 this is the reference's find_Yn (oocdag.cpp:478-492): the
// widest panel whose packed trapezoid plus one X column of Ym tiles fits in memBlock
// tiles, never narrower than the previous panel except for the last.  nx = 2 counts a
// second X buffer so that the copy of column k+1 overlaps the update with column k.
// ---------------------------------------------------------------------------------
static int panel_width(int bb, i64 memBlock, int jb, int nx, int* state) {
  int Yn = *state;
  const i64 Ym = bb - jb;
  const i64 room = (memBlock - nx * Ym) * 2;
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

// Exported for tests: the reference's panel sequence and this library's, as (jb, Ym, Yn)
// triples.  Returns the number of panels, OOC_ERR_BUDGET, or -5 if cap is too small.
extern "C" int ooc_panel_plan(int64_t n, int nb, int64_t memBlock, int nx, int* out, int cap) {
  if (n <= 0 || nb <= 0) return -1;
  const int bb = (int)((n + nb - 1) / nb);
  int state = 0, np = 0;
  i64 JB = 0;
  int jb = 0;
  while (JB < n) {
    const int Ym = bb - jb;
    const int Yn = panel_width(bb, memBlock, jb, nx, &state);
    if (Yn <= 0) return OOC_ERR_BUDGET;
    if (np >= cap) return -5;
    out[3 * np] = jb;
    out[3 * np + 1] = Ym;
    out[3 * np + 2] = Yn;
    np++;
    JB += std::min<i64>((i64)(jb + Yn) * nb, n) - (i64)jb * nb;
    jb += Yn;
  }
  return np;
}

// ---------------------------------------------------------------------------------
// Factorization of one panel held in `Ym` x `Yn` tiles of map `P` (in place), the
// right-looking in-core step of the reference (oocquark.cpp:358-421), with finished
// columns copied back to the host when `host` is set.
// ---------------------------------------------------------------------------------
namespace {

struct Run {
  ooc_handle* h;
  ooc_stats st{};
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> upd_ev, fac_ev;
  std::vector<double> upd_flops;
};

double pair_flops(int Ht, int Kt, i64 H, i64 Kc, int nb, int K) {
  double f = 0;
  for (int j = 0; j < Kt; j++) {
    double LN = (double)std::min<i64>(nb, Kc - (i64)j * nb);
    f += LN * (LN + 1) * K;  // syrk on the diagonal tile
    double rows = (double)std::min<i64>(H - (i64)(j + 1) * nb, (i64)(Ht - j - 1) * nb);
    if (rows > 0) f += 2.0 * rows * LN * K;
  }
  return f;
}

int timed_update(Run& R, const TileCol& X, const TileMap& C, int Ht, int Kt, i64 H, i64 Kc, int K) {
  ooc_handle* h = R.h;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (h->profile) {
    if (next_prof_event(h, &e0) != cudaSuccess || next_prof_event(h, &e1) != cudaSuccess) return OOC_ERR_CUDA;
    OOC_CUDA_TRY(cudaEventRecord(e0, h->s_comp));
  }
  // Large trapezoids are split so that no launch exceeds the grid's y limit.
  const i64 total = (i64)Kt * Ht - ((i64)Kt * (Kt - 1)) / 2;
  int rc;
  if (total <= 65535) {
    rc = launch_panel_update(X, C, Ht, Kt, H, Kc, K, h->d_status, h->s_comp);
    R.st.kernel_launches++;
  } else {
    // Split by tile columns: columns [j0, j1) of the trapezoid form a sub-trapezoid
    // whose pairs start at tile (j0, j0).
    int j0 = 0;
    rc = OOC_OK;
    while (j0 < Kt && rc == OOC_OK) {
      int j1 = j0;
      i64 cnt = 0;
      while (j1 < Kt && cnt + (Ht - j1) <= 65535) { cnt += Ht - j1; j1++; }
      TileMap Cs = C;
      Cs.base = tile_ptr(C, j0, j0);
      if (C.packed) Cs.Ym = C.Ym - j0;
      TileCol Xs = X;
      Xs.base = X.base + (i64)j0 * X.stride;
      rc = launch_panel_update(Xs, Cs, Ht - j0, j1 - j0, H - (i64)j0 * C.nb, Kc - (i64)j0 * C.nb, K,
                               h->d_status, h->s_comp);
      R.st.kernel_launches++;
      j0 = j1;
    }
  }
  if (rc) return rc;
  if (h->profile) {
    OOC_CUDA_TRY(cudaEventRecord(e1, h->s_comp));
    R.upd_ev.push_back({e0, e1});
    R.upd_flops.push_back(pair_flops(Ht, Kt, H, Kc, C.nb, K));
  }
  return OOC_OK;
}

// Copies the (rows x cols) block between host (ld lda) and a device tile (ld ldt).
int copy_h2d(Run& R, double* dst, i64 ldt, const double* src, i64 lda, i64 rows, i64 cols, cudaStream_t s) {
  OOC_CUDA_TRY(cudaMemcpy2DAsync(dst, ldt * sizeof(double), src, lda * sizeof(double), rows * sizeof(double),
                                 cols, cudaMemcpyHostToDevice, s));
  R.st.h2d_bytes += (double)rows * cols * sizeof(double);
  return OOC_OK;
}
int copy_d2h(Run& R, double* dst, i64 lda, const double* src, i64 ldt, i64 rows, i64 cols, cudaStream_t s) {
  OOC_CUDA_TRY(cudaMemcpy2DAsync(dst, lda * sizeof(double), src, ldt * sizeof(double), rows * sizeof(double),
                                 cols, cudaMemcpyDeviceToHost, s));
  R.st.d2h_bytes += (double)rows * cols * sizeof(double);
  return OOC_OK;
}

// In-panel factorization (oocquark.cpp:389-419).  P maps the panel's tiles; YM / YN are
// its element extents; col0 its first global column; hostA (may be null) the host
// address of the panel's tile (0,0) with leading dimension lda.
// Look-ahead, as QUARK's DAG allows it: the diagonal factor and column solve of tile
// column j+1 run on the high-priority stream s1 (the handle's host-to-device stream,
// idle while a panel is factored) beside the bulk of column j's trailing update on
// s_comp, which first updates tile column j+1 alone and signals s1.  Every tile still
// receives the same updates, from the same kernels, in the same order.
int factor_panel(Run& R, const TileMap& P, int Ym, int Yn, i64 YM, i64 YN, i64 col0, double* hostA, i64 lda) {
  ooc_handle* h = R.h;
  const int nb = P.nb;
  const i64 tstride = P.packed ? (i64)nb * nb : (i64)nb;
  cudaStream_t s0 = h->s_comp, s1 = h->s_h2d;
  cudaEvent_t evA, evP;  // A: column j+1 updated by column j (s0 -> s1); P: column j solved (s1 -> s0)
  OOC_CUDA_TRY(next_event(h, &evA));
  OOC_CUDA_TRY(cudaEventRecord(evA, s0));  // the panel's tiles are ready on s0
  for (int j = 0; j < Yn; j++) {
    const int LN = (int)std::min<i64>(nb, YN - (i64)j * nb);
    double* Djj = tile_ptr(P, j, j);
    OOC_CUDA_TRY(cudaStreamWaitEvent(s1, evA, 0));
    cudaEvent_t f0 = nullptr, f1 = nullptr;
    if (h->profile) {
      if (next_prof_event(h, &f0) != cudaSuccess || next_prof_event(h, &f1) != cudaSuccess) return OOC_ERR_CUDA;
      OOC_CUDA_TRY(cudaEventRecord(f0, s1));
    }
    int rc = launch_potrf_tile(Djj, P.ld, LN, col0 + (i64)j * nb, h->d_status, s1);
    if (rc) return rc;
    R.st.kernel_launches += 3 * ((LN + 63) / 64);
    const int below = Ym - j - 1;
    if (below > 0) {
      const int m_last = (int)(YM - (i64)(Ym - 1) * nb);
      TileCol B{tile_ptr(P, j + 1, j), P.ld, tstride};
      rc = launch_trsm_col(Djj, P.ld, B, below, nb, m_last, LN, h->d_status, s1);
      if (rc) return rc;
      R.st.kernel_launches += 2 * ((LN + 63) / 64);
    }
    if (h->profile) {
      OOC_CUDA_TRY(cudaEventRecord(f1, s1));
      R.fac_ev.push_back({f0, f1});
    }
    OOC_CUDA_TRY(next_event(h, &evP));
    OOC_CUDA_TRY(cudaEventRecord(evP, s1));
    OOC_CUDA_TRY(cudaStreamWaitEvent(s0, evP, 0));
    if (hostA) {
      // Column j is final: copy it back while the trailing update proceeds
      // (oocquark.cpp:394,409).
      OOC_CUDA_TRY(cudaStreamWaitEvent(h->s_d2h, evP, 0));
      for (int i = j; i < Ym; i++) {
        const i64 LM = std::min<i64>(nb, YM - (i64)i * nb);
        rc = copy_d2h(R, hostA + (i64)i * nb + (i64)j * nb * lda, lda, tile_ptr(P, i, j), P.ld, LM, LN, h->s_d2h);
        if (rc) return rc;
      }
    }
    if (j + 1 < Yn) {
      // tile column j+1 first, then the rest of the panel's trailing tiles
      TileCol X{tile_ptr(P, j + 1, j), P.ld, tstride};
      TileMap C = P;
      C.base = tile_ptr(P, j + 1, j + 1);
      if (P.packed) C.Ym = Ym - j - 1;
      rc = timed_update(R, X, C, Ym - j - 1, 1, YM - (i64)(j + 1) * nb, std::min<i64>(nb, YN - (i64)(j + 1) * nb), nb);
      if (rc) return rc;
      OOC_CUDA_TRY(next_event(h, &evA));
      OOC_CUDA_TRY(cudaEventRecord(evA, s0));
      if (j + 2 < Yn) {
        TileCol X2{tile_ptr(P, j + 2, j), P.ld, tstride};
        TileMap C2 = P;
        C2.base = tile_ptr(P, j + 2, j + 2);
        if (P.packed) C2.Ym = Ym - j - 2;
        rc = timed_update(R, X2, C2, Ym - j - 2, Yn - j - 2, YM - (i64)(j + 2) * nb, YN - (i64)(j + 2) * nb, nb);
        if (rc) return rc;
      }
    }
  }
  return OOC_OK;
}

int finish_profile(Run& R) {
  for (auto& pr : R.upd_ev) {
    float ms = 0;
    OOC_CUDA_TRY(cudaEventElapsedTime(&ms, pr.first, pr.second));
    R.st.update_ms += ms;
  }
  R.st.update_launches = (int64_t)R.upd_ev.size();
  for (double f : R.upd_flops) R.st.update_flops += f;
  for (auto& pr : R.fac_ev) {
    float ms = 0;
    OOC_CUDA_TRY(cudaEventElapsedTime(&ms, pr.first, pr.second));
    R.st.factor_ms += ms;
  }
  return OOC_OK;
}

int read_status(ooc_handle* h, int* info) {
  OOC_CUDA_TRY(cudaMemcpyAsync(h->h_status, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->s_comp));
  int rc = ooc_wait_stream(h, h->s_comp);
  if (rc) return rc;
  *info = *(volatile int*)h->h_status;
  return OOC_OK;
}

int sync_all(ooc_handle* h) {
  int rc = ooc_wait_stream(h, h->s_h2d);
  if (!rc) rc = ooc_wait_stream(h, h->s_d2h);
  if (!rc) rc = ooc_wait_stream(h, h->s_comp);
  return rc;
}

// In-core: A is device memory.  One panel covering the whole matrix, factored in place.
int dpotrf_device(Run& R, double* A, i64 n, i64 lda, int nb) {
  const int bb = (int)((n + nb - 1) / nb);
  TileMap P{A, lda, 0, bb, nb};
  R.st.npanels = 1;
  return factor_panel(R, P, bb, bb, n, n, 0, nullptr, lda);
}

// Out-of-core: A is host memory.  oocdag.cpp:59-89.
int dpotrf_host(Run& R, double* A, i64 n, i64 lda, int nb, size_t budget) {
  ooc_handle* h = R.h;
  const int bb = (int)((n + nb - 1) / nb);
  const i64 tile_elems = (i64)nb * nb;
  i64 memBlock = (i64)(budget / sizeof(double) / (size_t)tile_elems);
  int nx = h->ref_schedule ? 1 : h->x_buffers;
  {
    int probe = 0;
    if (panel_width(bb, memBlock, 0, nx, &probe) <= 0) {
      if (nx == 2) {
        probe = 0;
        nx = 1;  // the budget only holds the reference's single X buffer
        if (panel_width(bb, memBlock, 0, nx, &probe) <= 0) return OOC_ERR_BUDGET;
      } else {
        return OOC_ERR_BUDGET;
      }
    }
  }
  // A budget larger than one whole-matrix panel plus its X buffers buys nothing: the
  // schedule is the same single panel, so only that much is allocated.
  memBlock = std::min<i64>(memBlock, (i64)bb * (bb + 1) / 2 + (i64)nx * bb);
  const size_t need = (size_t)memBlock * (size_t)tile_elems * sizeof(double);
  if (h->d_buf_bytes < need) {
    if (h->d_buf) cudaFree(h->d_buf);
    h->d_buf = nullptr;
    h->d_buf_bytes = 0;
    if (cudaMalloc(&h->d_buf, need) != cudaSuccess) {
      cudaGetLastError();
      g_last_error = "device panel buffer allocation failed";
      return OOC_ERR_NOMEM;
    }
    h->d_buf_bytes = need;
  }
  double* Y = h->d_buf;
  int state = 0;
  cudaEvent_t ev_prev_comp = nullptr, ev_prev_d2h = nullptr;
  i64 JB = 0;
  int jb = 0;
  int rc = OOC_OK;
  while (JB < n) {
    const int Ym = bb - jb;
    const int Yn = panel_width(bb, memBlock, jb, nx, &state);
    const i64 YM = n - JB;
    const i64 YN = std::min<i64>((i64)(jb + Yn) * nb, n) - JB;
    double* Xb[2] = {Y + (memBlock - Ym) * tile_elems, nullptr};
    if (nx == 2) Xb[1] = Y + (memBlock - 2 * (i64)Ym) * tile_elems;
    double* Apan = A + JB + JB * lda;
    TileMap P{Y, nb, 1, Ym, nb};
    // The previous panel must be done with Y, and its copy-back done with the host
    // tiles this panel reads.
    if (ev_prev_comp) OOC_CUDA_TRY(cudaStreamWaitEvent(h->s_h2d, ev_prev_comp, 0));
    if (ev_prev_d2h) OOC_CUDA_TRY(cudaStreamWaitEvent(h->s_h2d, ev_prev_d2h, 0));
    // A2Y (oocquark.cpp:253-275)
    for (int j = 0; j < Yn; j++) {
      const i64 LN = std::min<i64>(nb, YN - (i64)j * nb);
      for (int i = j; i < Ym; i++) {
        const i64 LM = std::min<i64>(nb, YM - (i64)i * nb);
        rc = copy_h2d(R, tile_ptr(P, i, j), nb, Apan + (i64)i * nb + (i64)j * nb * lda, lda, LM, LN, h->s_h2d);
        if (rc) return rc;
      }
    }
    cudaEvent_t ev_y;
    OOC_CUDA_TRY(next_event(h, &ev_y));
    OOC_CUDA_TRY(cudaEventRecord(ev_y, h->s_h2d));
    OOC_CUDA_TRY(cudaStreamWaitEvent(h->s_comp, ev_y, 0));
    // Left-looking updates with every earlier tile column (oocdag.cpp:73-77).
    cudaEvent_t ev_x_free[2] = {nullptr, nullptr};
    for (int jjb = 0; jjb < jb; jjb++) {
      const int b = (nx == 2) ? (jjb & 1) : 0;
      double* X = Xb[b];
      if (ev_x_free[b]) OOC_CUDA_TRY(cudaStreamWaitEvent(h->s_h2d, ev_x_free[b], 0));
      // A2X (oocquark.cpp:301-319): tile rows jb.. of tile column jjb.
      const double* Acol = A + JB + (i64)jjb * nb * lda;
      for (int i = 0; i < Ym; i++) {
        const i64 LM = std::min<i64>(nb, YM - (i64)i * nb);
        rc = copy_h2d(R, X + i * tile_elems, nb, Acol + (i64)i * nb, lda, LM, nb, h->s_h2d);
        if (rc) return rc;
      }
      cudaEvent_t ev_x;
      OOC_CUDA_TRY(next_event(h, &ev_x));
      OOC_CUDA_TRY(cudaEventRecord(ev_x, h->s_h2d));
      OOC_CUDA_TRY(cudaStreamWaitEvent(h->s_comp, ev_x, 0));
      TileCol Xc{X, nb, tile_elems};
      rc = timed_update(R, Xc, P, Ym, Yn, YM, YN, nb);
      if (rc) return rc;
      cudaEvent_t ev_f;
      OOC_CUDA_TRY(next_event(h, &ev_f));
      OOC_CUDA_TRY(cudaEventRecord(ev_f, h->s_comp));
      ev_x_free[b] = ev_f;
    }
    // In-core factorization of the panel with copy-back (oocdag.cpp:80).
    rc = factor_panel(R, P, Ym, Yn, YM, YN, JB, Apan, lda);
    if (rc) return rc;
    OOC_CUDA_TRY(cudaMemcpyAsync(h->h_status, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->s_comp));
    OOC_CUDA_TRY(next_event(h, &ev_prev_comp));
    OOC_CUDA_TRY(cudaEventRecord(ev_prev_comp, h->s_comp));
    OOC_CUDA_TRY(next_event(h, &ev_prev_d2h));
    OOC_CUDA_TRY(cudaEventRecord(ev_prev_d2h, h->s_d2h));
    R.st.npanels++;
    JB += YN;
    jb += Yn;
    // Stop early once a minor has failed (checked without stalling the pipeline).
    if (cudaEventQuery(ev_prev_comp) == cudaSuccess) {
      if (*(volatile int*)h->h_status) break;
    }
    if (h->ev_next > 4096) {
      // Keep the event pool bounded on very long runs: once everything queued so far
      // has finished, every pooled event may be recorded again.
      rc = sync_all(h);
      if (rc) return rc;
      ev_prev_comp = ev_prev_d2h = nullptr;
      h->ev_next = 0;
    }
  }
  return OOC_OK;
}

}  // namespace

extern "C" int ooc_dpotrf_L(ooc_handle* h, double* A, int64_t n, int64_t lda, int nb, size_t dev_budget,
                            int* info, ooc_stats* stats) {
  if (!h) return -1;
  if (!A && n > 0) return -2;
  if (n < 0) return -3;
  if (lda < std::max<int64_t>(1, n)) return -4;
  if (nb <= 0) return -5;
  if (!info) return -7;
  *info = 0;
  if (stats) memset(stats, 0, sizeof(*stats));
  if (n == 0) return OOC_OK;
  DeviceGuard g(h->device);

  cudaPointerAttributes attr;
  memset(&attr, 0, sizeof(attr));
  if (cudaPointerGetAttributes(&attr, A) != cudaSuccess) {
    cudaGetLastError();
    attr.type = cudaMemoryTypeUnregistered;
  }
  const bool on_device = (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged);
  bool registered = false;
  if (!on_device && attr.type == cudaMemoryTypeUnregistered && h->pin_host) {
    size_t bytes = ((size_t)(n - 1) * (size_t)lda + (size_t)n) * sizeof(double);
    if (cudaHostRegister(A, bytes, cudaHostRegisterDefault) == cudaSuccess) registered = true;
    else cudaGetLastError();  // fall back to pageable copies
  }

  Run R;
  R.h = h;
  h->ev_next = 0;
  h->prof_next = 0;
  int rc = OOC_OK;
  {  // (no early return: a host matrix registered above is unregistered below)
    const cudaError_t e = cudaMemsetAsync(h->d_status, 0, sizeof(int), h->s_comp);
    if (e != cudaSuccess) {
      ooc_set_last_error(e, "cudaMemsetAsync (status word)", __FILE__, __LINE__);
      rc = OOC_ERR_CUDA;
    }
  }
  *h->h_status = 0;
  if (!rc) rc = ooc_wait_stream(h, h->s_comp);
  auto t0 = std::chrono::steady_clock::now();
  if (!rc) rc = on_device ? dpotrf_device(R, A, n, lda, nb) : dpotrf_host(R, A, n, lda, nb, dev_budget);
  int rc2 = sync_all(h);
  if (!rc) rc = rc2;
  auto t1 = std::chrono::steady_clock::now();
  int st = 0;
  if (!rc) rc = read_status(h, &st);
  if (!rc && h->profile) rc = finish_profile(R);
  if (registered) cudaHostUnregister(A);
  h->ev_next = 0;
  h->prof_next = 0;
  if (rc) return rc;
  *info = st;
  h->last_info = st;
  R.st.seconds = std::chrono::duration<double>(t1 - t0).count();
  R.st.flops = (double)n * (double)n * (double)n / 3.0;
  R.st.info = st;
  if (stats) *stats = R.st;
  return OOC_OK;
}

// ---------------------------------------------------------------------------------
// Reference-shaped entry points.
// ---------------------------------------------------------------------------------
static std::mutex g_default_mu;
static ooc_handle* g_default[64] = {nullptr};

ooc_handle* ooc_default_handle() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_default_mu);
  if (!g_default[dev]) {
    ooc_handle* h = nullptr;
    if (ooc_create(&h, dev) != OOC_OK) return nullptr;
    g_default[dev] = h;
  }
  return g_default[dev];
}

extern "C" double Cholesky(void* handle, double* A, int N, int NB, int LDA, size_t memsize) {
  ooc_handle* h = handle ? (ooc_handle*)handle : ooc_default_handle();
  if (!h) return (double)OOC_ERR_NODEVICE;
  int info = 0;
  ooc_stats st;
  int rc = ooc_dpotrf_L(h, A, N, LDA, NB, memsize, &info, &st);
  if (rc) return (double)rc;
  return st.seconds;
}

extern "C" void ooc_pdpotrf_(const char* uplo, const int* n, double* a, const int* ia, const int* ja,
                             const int* desca, int* info) {
  if (!info) return;
  if (!uplo || (*uplo != 'L' && *uplo != 'l')) { *info = -1; return; }
  if (!n || *n < 0) { *info = -2; return; }
  if (!ia || !ja || *ia < 1 || *ja < 1) { *info = -4; return; }
  if (!desca) { *info = -(600 + 1); return; }
  // desc: DTYPE_=0 CTXT_=1 M_=2 N_=3 MB_=4 NB_=5 RSRC_=6 CSRC_=7 LLD_=8 (0-based here)
  const int nbk = desca[5], lld = desca[8];
  if (desca[4] != desca[5]) { *info = -(600 + 5); return; }
  if (nbk <= 0) { *info = -(600 + 6); return; }
  if (lld < std::max(1, desca[2])) { *info = -(600 + 9); return; }
  if (*ia - 1 + *n > desca[2] || *ja - 1 + *n > desca[3]) { *info = -2; return; }
  ooc_handle* h = ooc_default_handle();
  if (!h) { *info = OOC_ERR_NODEVICE; return; }
  size_t budget = 0;
  if (const char* e = getenv("OOC_DEVICE_BUDGET_MB")) budget = (size_t)atoll(e) << 20;
  if (budget == 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    budget = fr / 4 * 3;
  }
  double* A = a + (i64)(*ia - 1) + (i64)(*ja - 1) * lld;
  int lapack_info = 0;
  int rc = ooc_dpotrf_L(h, A, *n, lld, nbk, budget, &lapack_info, nullptr);
  *info = rc ? rc : lapack_info;
}

// The same for FP32 (pspotrf_ argument order): ooc_spotrf_L on the sub-matrix.
extern "C" void ooc_pspotrf_(const char* uplo, const int* n, float* a, const int* ia, const int* ja,
                             const int* desca, int* info) {
  if (!info) return;
  if (!uplo || (*uplo != 'L' && *uplo != 'l')) { *info = -1; return; }
  if (!n || *n < 0) { *info = -2; return; }
  if (!ia || !ja || *ia < 1 || *ja < 1) { *info = -4; return; }
  if (!desca) { *info = -(600 + 1); return; }
  const int nbk = desca[5], lld = desca[8];
  if (desca[4] != desca[5]) { *info = -(600 + 5); return; }
  if (nbk <= 0) { *info = -(600 + 6); return; }
  if (lld < std::max(1, desca[2])) { *info = -(600 + 9); return; }
  if (*ia - 1 + *n > desca[2] || *ja - 1 + *n > desca[3]) { *info = -2; return; }
  ooc_handle* h = ooc_default_handle();
  if (!h) { *info = OOC_ERR_NODEVICE; return; }
  size_t budget = 0;
  if (const char* e = getenv("OOC_DEVICE_BUDGET_MB")) budget = (size_t)atoll(e) << 20;
  float* A = a + (i64)(*ia - 1) + (i64)(*ja - 1) * lld;
  int lapack_info = 0;
  int rc = ooc_spotrf_L(h, A, *n, lld, nbk, budget, &lapack_info, nullptr);
  *info = rc ? rc : lapack_info;
}
