// CPU oracle for the out-of-core (OOC) left-looking tiled Cholesky.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, on the host, the algorithm of the
// reference project (efdazedo/oocdag) so that the GPU library can be checked against
// it.  Only tests, the smoke check and the CPU-baseline leg of the benchmark may load
// it; the GPU product never links, calls or falls back to it.
//
// Parity status: pinned (a) to the reference's own oocdag.cpp/oocquark.cpp compiled
// unmodified with host stand-ins for QUARK, cuBLAS and MKL (oracle/ref_build.py,
// oracle/_ref): this oracle's factor equals that build's bit for bit, and its panel
// plans and task counts equal the reference's; (b) to a literal-loop restatement of the
// reference's Fortran generator (tests/golden); (c) to LAPACK dpotrf.  Tile arithmetic
// is delegated to host BLAS/LAPACK (OpenBLAS bundled with SciPy), standing in for the
// MKL and cuBLAS calls the reference makes at oocquark.cpp:87,130,176,222.
//
// What follows the reference (paths relative to the reference project):
//   orc_find_Yn          oocdag.cpp:478-492  (the function-local `static Yn` becomes
//                        an explicit state argument)
//   orc_cholesky         oocdag.cpp:18-112   (panel loop; device buffer Y = host buffer)
//   a2y / a2x / syrk_dag / incore_dag
//                        oocquark.cpp:253-275, 301-319, 323-356, 358-421
//   task bodies          oocquark.cpp:16-251 (H2D/D2H = strided<->packed copies,
//                        potrf on the host copy of the diagonal tile as under
//                        USE_HOST_DPOTRF, trsm R/L/T/N, syrk L/N, gemm N/T)
//   dependency tracking  QUARK semantics as used at oocquark.cpp:37-44,102-107,145-156,
//                        191-201,238-250: hazards keyed by tile base address with
//                        INPUT / OUTPUT / INOUT modes; copy tasks restricted to
//                        "communication" workers and given priority 1
//                        (oocquark.cpp:10-13,257-261).
//   generators           LIN/pdmatgen.f:223-378,516-543 with LIN/pmatgeninc.f:5-135,
//                        271-313 (closed form of the 31-bit LCG stream), and the
//                        counter-based uniform generator used for (R+R^T)/2 + alpha*I.
//   residual             ||A - L L^T||_F / (n * eps * ||A||_F), eps = 2^-53, A tiles
//                        regenerated from the seed as LIN/pdlaschk.f:238-250 does.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <dlfcn.h>
#include <functional>
#include <mutex>
#include <queue>
#include <thread>
#include <unordered_map>
#include <vector>

typedef int64_t i64;

// ---------------------------------------------------------------------------------
// Host BLAS / LAPACK (Fortran ABI, LP64) resolved from SciPy's bundled OpenBLAS.
// ---------------------------------------------------------------------------------
typedef void (*dgemm_t)(const char*, const char*, const int*, const int*, const int*,
                        const double*, const double*, const int*, const double*, const int*,
                        const double*, double*, const int*, size_t, size_t);
typedef void (*dsyrk_t)(const char*, const char*, const int*, const int*, const double*,
                        const double*, const int*, const double*, double*, const int*,
                        size_t, size_t);
typedef void (*dtrsm_t)(const char*, const char*, const char*, const char*, const int*,
                        const int*, const double*, const double*, const int*, double*,
                        const int*, size_t, size_t, size_t, size_t);
typedef void (*dpotrf_t)(const char*, const int*, double*, const int*, int*, size_t);
typedef void (*dpotrs_t)(const char*, const int*, const int*, const double*, const int*,
                         double*, const int*, int*, size_t);
typedef void (*setthreads_t)(int);
typedef void (*setthreads_local_t)(int);

static dgemm_t p_dgemm = nullptr;
static dsyrk_t p_dsyrk = nullptr;
static dtrsm_t p_dtrsm = nullptr;
static dpotrf_t p_dpotrf = nullptr;
static dpotrs_t p_dpotrs = nullptr;
static setthreads_t p_setthreads = nullptr;

extern "C" int orc_init_blas(const char* libpath) {
  void* h = dlopen(libpath, RTLD_NOW | RTLD_LOCAL);
  if (!h) { fprintf(stderr, "oracle: dlopen(%s) failed: %s\n", libpath, dlerror()); return -1; }
  p_dgemm = (dgemm_t)dlsym(h, "scipy_dgemm_");
  p_dsyrk = (dsyrk_t)dlsym(h, "scipy_dsyrk_");
  p_dtrsm = (dtrsm_t)dlsym(h, "scipy_dtrsm_");
  p_dpotrf = (dpotrf_t)dlsym(h, "scipy_dpotrf_");
  p_dpotrs = (dpotrs_t)dlsym(h, "scipy_dpotrs_");
  p_setthreads = (setthreads_t)dlsym(h, "scipy_openblas_set_num_threads");
  if (!p_dgemm || !p_dsyrk || !p_dtrsm || !p_dpotrf || !p_dpotrs || !p_setthreads) {
    fprintf(stderr, "oracle: missing BLAS symbols in %s\n", libpath);
    return -2;
  }
  return 0;
}

extern "C" void orc_set_blas_threads(int n) { if (p_setthreads) p_setthreads(n); }

static void blas_dgemm_nt(int m, int n, int k, double alpha, const double* A, int lda,
                          const double* B, int ldb, double beta, double* C, int ldc) {
  p_dgemm("N", "T", &m, &n, &k, &alpha, A, &lda, B, &ldb, &beta, C, &ldc, 1, 1);
}
static void blas_dsyrk_ln(int n, int k, double alpha, const double* A, int lda, double beta,
                          double* C, int ldc) {
  p_dsyrk("L", "N", &n, &k, &alpha, A, &lda, &beta, C, &ldc, 1, 1);
}
static void blas_dtrsm_rltn(int m, int n, double alpha, const double* A, int lda, double* B,
                            int ldb) {
  p_dtrsm("R", "L", "T", "N", &m, &n, &alpha, A, &lda, B, &ldb, 1, 1, 1, 1);
}
static int lapack_dpotrf_l(int n, double* A, int lda) {
  int info = 0;
  p_dpotrf("L", &n, A, &lda, &info, 1);
  return info;
}

// ---------------------------------------------------------------------------------
// Panel sizing (oocdag.cpp:478-492).  `state` carries the reference's function-local
// static: the panel width only grows from one panel to the next, except that the
// last panel takes whatever is left.
// ---------------------------------------------------------------------------------
extern "C" int orc_find_Yn(int bb, int memBlock, int jb, int* state) {
  int Yn = *state;
  int Ym = bb - jb;
  if (Ym * (Ym + 1) <= (memBlock - Ym) * 2) {
    Yn = Ym;
  } else {
    while ((memBlock - Ym) * 2 >= (2 * Ym - Yn) * (Yn + 1)) {
      if (Yn == Ym) break;
      Yn++;
    }
  }
  *state = Yn;
  return Yn;
}

// Writes the panel sequence (jb, Ym, Yn) of the driver loop (oocdag.cpp:59-66) for a
// problem of N rows, tile NB and a budget of memBlock tiles.  Returns the number of
// panels, or -1 if `cap` triples do not suffice.
extern "C" int orc_panel_plan(int N, int NB, i64 memBlock, int* out, int cap) {
  int bb = (N + NB - 1) / NB;
  int state = 0;
  int np = 0;
  int JB = 0, jb = 0;
  while (JB < N) {
    int Ym = bb - jb;
    int Yn = orc_find_Yn(bb, (int)memBlock, jb, &state);
    if (Yn <= 0) return -2;
    if (np >= cap) return -1;
    out[3 * np + 0] = jb;
    out[3 * np + 1] = Ym;
    out[3 * np + 2] = Yn;
    np++;
    JB += std::min((jb + Yn) * NB, N) - jb * NB;
    jb += Yn;
  }
  return np;
}

// ---------------------------------------------------------------------------------
// QUARK-like task executor.  Tasks are inserted in program order by the calling
// thread.  Every pointer argument is a hazard key (its base address), with the access
// mode the reference declares for it.  A task runs once every earlier task that
// conflicts on some key has finished: read-after-write, write-after-read and
// write-after-write.  Copy tasks go to "communication" workers at priority 1; compute
// tasks go to the remaining workers (oocquark.cpp:10-13).
// ---------------------------------------------------------------------------------
enum AccessMode { ACC_INPUT = 1, ACC_OUTPUT = 2, ACC_INOUT = 3 };

struct Access { const void* key; int mode; };

class TaskGraph {
 public:
  TaskGraph(int nthreads, int ncomm) : nthreads_(std::max(1, nthreads)) {
    ncomm_ = (nthreads_ >= 2) ? std::max(1, std::min(ncomm, nthreads_ - 1)) : 0;
    for (int t = 0; t < nthreads_; t++) workers_.emplace_back([this, t] { worker(t); });
  }
  ~TaskGraph() {
    barrier();
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& w : workers_) w.join();
  }

  void insert(std::function<void()> body, std::initializer_list<Access> acc, bool comm,
              int prio) {
    std::lock_guard<std::mutex> lk(mu_);
    i64 id = (i64)tasks_.size();
    tasks_.emplace_back();
    Task& t = tasks_.back();
    t.body = std::move(body);
    t.comm = comm;
    t.prio = prio;
    t.npred = 0;
    for (const Access& a : acc) {
      Track& tr = track_[a.key];
      if (a.mode == ACC_INPUT) {
        if (tr.writer >= 0) add_edge(tr.writer, id);
        tr.readers.push_back(id);
      } else {
        if (tr.writer >= 0) add_edge(tr.writer, id);
        for (i64 r : tr.readers) add_edge(r, id);
        tr.readers.clear();
        tr.writer = id;
      }
    }
    pending_++;
    if (t.npred == 0) push_ready(id);
  }

  void barrier() {
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [this] { return pending_ == 0; });
    // All work finished: hazard history can be dropped.
    track_.clear();
  }

 private:
  struct Task {
    std::function<void()> body;
    std::vector<i64> succ;
    int npred;
    int prio;
    bool comm;
    bool done = false;
  };
  struct Track { i64 writer = -1; std::vector<i64> readers; };
  struct Ready {
    int prio; i64 id;
    bool operator<(const Ready& o) const {  // max-heap on priority, then FIFO
      if (prio != o.prio) return prio < o.prio;
      return id > o.id;
    }
  };

  void add_edge(i64 from, i64 to) {
    Task& f = tasks_[from];
    if (f.done) return;
    if (!f.succ.empty() && f.succ.back() == to) return;  // duplicate key in one task
    f.succ.push_back(to);
    tasks_[to].npred++;
  }
  void push_ready(i64 id) {
    Task& t = tasks_[id];
    if (t.comm && ncomm_ > 0) comm_q_.push({t.prio, id});
    else comp_q_.push({t.prio, id});
    cv_.notify_all();
  }
  void worker(int t) {
    bool is_comm = (t >= nthreads_ - ncomm_) && ncomm_ > 0;
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      std::priority_queue<Ready>& q = is_comm ? comm_q_ : comp_q_;
      cv_.wait(lk, [&] { return stop_ || !q.empty(); });
      if (q.empty()) { if (stop_) return; continue; }
      i64 id = q.top().id;
      q.pop();
      std::function<void()> body = std::move(tasks_[id].body);
      lk.unlock();
      body();
      lk.lock();
      Task& tk = tasks_[id];
      tk.done = true;
      for (i64 s : tk.succ) {
        if (--tasks_[s].npred == 0) push_ready(s);
      }
      tk.succ.clear();
      tk.succ.shrink_to_fit();
      if (--pending_ == 0) done_cv_.notify_all();
    }
  }

  int nthreads_, ncomm_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<Task> tasks_;
  std::unordered_map<const void*, Track> track_;
  std::priority_queue<Ready> comm_q_, comp_q_;
  i64 pending_ = 0;
  bool stop_ = false;
  std::vector<std::thread> workers_;
};

// ---------------------------------------------------------------------------------
// Task bodies (oocquark.cpp:16-251).
// ---------------------------------------------------------------------------------
static void copy_tile(int M, int N, const double* src, i64 lds, double* dst, i64 ldd) {
  for (int j = 0; j < N; j++) memcpy(dst + (size_t)j * ldd, src + (size_t)j * lds, sizeof(double) * M);
}

struct OocRun {
  TaskGraph* g;
  std::atomic<int> info{0};
  int first_bad_col = 0;
};

static void q_h2d(OocRun& R, int M, int N, const double* H, int ldh, double* D, int NB) {
  R.g->insert([=] { copy_tile(M, N, H, ldh, D, NB); },
              {{H, ACC_INPUT}, {D, ACC_OUTPUT}}, true, 1);
}
static void q_d2h(OocRun& R, int M, int N, const double* D, int NB, double* H, int ldh) {
  R.g->insert([=] { copy_tile(M, N, D, NB, H, ldh); },
              {{D, ACC_INPUT}, {H, ACC_OUTPUT}}, true, 1);
}
// The diagonal-tile factor runs on the host copy of the tile (USE_HOST_DPOTRF build).
// `col0` is the global index of the tile's first column; a failure is reported as the
// LAPACK info of the whole matrix (first failing leading minor), keeping the smallest.
static void q_potrf(OocRun& R, int N, double* A, int lda, int col0) {
  OocRun* r = &R;
  R.g->insert([=] {
    int info = lapack_dpotrf_l(N, A, lda);
    if (info > 0) {
      int g = col0 + info;
      int cur = r->info.load();
      while ((cur == 0 || g < cur) && !r->info.compare_exchange_weak(cur, g)) {}
    }
  }, {{A, ACC_INOUT}}, false, 0);
}
static void q_trsm(OocRun& R, int M, int N, const double* A, double* B, int NB) {
  R.g->insert([=] { blas_dtrsm_rltn(M, N, 1.0, A, NB, B, NB); },
              {{A, ACC_INPUT}, {B, ACC_INOUT}}, false, 0);
}
static void q_syrk(OocRun& R, int N, int K, const double* A, double* C, int NB) {
  R.g->insert([=] { blas_dsyrk_ln(N, K, -1.0, A, NB, 1.0, C, NB); },
              {{A, ACC_INPUT}, {C, ACC_INOUT}}, false, 0);
}
static void q_gemm(OocRun& R, int M, int N, int K, const double* A, const double* B, double* C,
                   int NB) {
  R.g->insert([=] { blas_dgemm_nt(M, N, K, -1.0, A, NB, B, NB, 1.0, C, NB); },
              {{A, ACC_INPUT}, {B, ACC_INPUT}, {C, ACC_INOUT}}, false, 0);
}

// Packed panel: the panel's lower trapezoid of tiles, each NB x NB with ld = NB, stored
// column of tiles after column of tiles (oocquark.cpp:256,326,361).
static inline i64 ytile(int ib, int jb, int Ym) {
  return (i64)ib + (i64)jb * Ym - ((i64)jb * (jb + 1)) / 2;
}

// oocquark.cpp:253-275
static void a2y(OocRun& R, double* A, double* Y, int LDA, int NB, int M, int N) {
  int Ym = (M + NB - 1) / NB;
  for (int JB = 0, jb = 0; JB < N; JB += NB, jb++) {
    int LN = std::min(JB + NB, N) - JB;
    for (int IB = JB, ib = jb; IB < M; IB += NB, ib++) {
      int LM = std::min(IB + NB, M) - IB;
      q_h2d(R, LM, LN, A + (size_t)jb * NB * LDA + (size_t)ib * NB, LDA,
            Y + ytile(ib, jb, Ym) * NB * NB, NB);
    }
  }
}
// oocquark.cpp:301-319
static void a2x(OocRun& R, double* A, int LDA, double* X, int NB, int K) {
  for (int IB = 0, ib = 0; IB < K; IB += NB, ib++) {
    int LM = std::min(IB + NB, K) - IB;
    q_h2d(R, LM, NB, A + (size_t)ib * NB, LDA, X + (size_t)ib * NB * NB, NB);
  }
}
// oocquark.cpp:323-356: Y(0:H, 0:K) -= X X(0:K)^T with the storage pattern of Y fixed by
// H and NB.
static void syrk_dag(OocRun& R, double* X, double* Y, int H, int K, int NB) {
  int Ym = (H + NB - 1) / NB;
  for (int JB = 0, jb = 0; JB < K; JB += NB, jb++) {
    int LN = std::min(JB + NB, K) - JB;
    q_syrk(R, LN, NB, X + (size_t)jb * NB * NB, Y + ytile(jb, jb, Ym) * NB * NB, NB);
    for (int IB = JB + NB, ib = jb + 1; IB < H; IB += NB, ib++) {
      int LM = std::min(IB + NB, H) - IB;
      q_gemm(R, LM, LN, NB, X + (size_t)ib * NB * NB, X + (size_t)jb * NB * NB,
             Y + ytile(ib, jb, Ym) * NB * NB, NB);
    }
  }
}
// oocquark.cpp:358-421 (USE_HOST_DPOTRF branch).  `col0` is the panel's first global
// column, used only to report the failing leading minor.
static void incore_dag(OocRun& R, double* A, double* Y, int LDA, int NB, int M, int N, int col0) {
  int Ym = (M + NB - 1) / NB;
  for (int JB = 0, jb = 0; JB < N; JB += NB, jb++) {
    int LN = std::min(JB + NB, N) - JB;
    double* Ajj = A + (size_t)jb * NB * LDA + (size_t)jb * NB;
    double* Yjj = Y + ytile(jb, jb, Ym) * NB * NB;
    q_d2h(R, LN, LN, Yjj, NB, Ajj, LDA);
    q_potrf(R, LN, Ajj, LDA, col0 + JB);
    q_h2d(R, LN, LN, Ajj, LDA, Yjj, NB);
    for (int IB = JB + NB, ib = jb + 1; IB < M; IB += NB, ib++) {
      int LM = std::min(IB + NB, M) - IB;
      double* Yij = Y + ytile(ib, jb, Ym) * NB * NB;
      q_trsm(R, LM, LN, Yjj, Yij, NB);
      q_d2h(R, LM, LN, Yij, NB, A + (size_t)jb * NB * LDA + (size_t)ib * NB, LDA);
    }
    if (JB + NB < N) {
      int H = M - JB - NB;
      int K = N - JB - NB;
      syrk_dag(R, Y + ytile(jb + 1, jb, Ym) * NB * NB, Y + ytile(jb + 1, jb + 1, Ym) * NB * NB,
               H, K, NB);
    }
  }
}

// oocdag.cpp:18-112.  Factors the lower triangle of the N x N column-major matrix A
// (leading dimension LDA) in place with a "device" budget of memsize bytes, executing
// the task graph on `nthreads` workers (`ncomm` of them for copies).  Returns the
// factorization time in seconds (buffer allocation excluded, as oocdag.cpp:41,51).
// *info receives the LAPACK-style info (0, or the order of the first leading minor
// that is not positive definite).  The ORC_SEQUENTIAL mode (nthreads == 0) runs every
// task inline in program order.
extern "C" double orc_cholesky(double* A, int N, int NB, int LDA, size_t memsize, int nthreads,
                               int ncomm, int* info, int* npanels) {
  int bb = (N + NB - 1) / NB;
  i64 memBlock = (i64)(memsize / sizeof(double) / NB / NB);
  *info = 0;
  if (npanels) *npanels = 0;
  if (N <= 0) return 0.0;
  {
    // The first panel must get at least one tile column (the reference asserts the
    // equivalent at oocdag.cpp:249-250); otherwise the panel loop cannot advance.
    int probe = 0;
    if (orc_find_Yn(bb, (int)memBlock, 0, &probe) <= 0) { *info = -6; return 0.0; }
  }
  // A budget beyond one whole-matrix panel plus its X column gives the same single-panel
  // schedule; only that much host memory stands in for the device buffer.
  memBlock = std::min<i64>(memBlock, (i64)bb * (bb + 1) / 2 + bb);
  std::vector<double> Ybuf((size_t)memBlock * NB * NB);
  double* Y = Ybuf.data();
  OocRun R;
  TaskGraph* g = new TaskGraph(nthreads <= 0 ? 1 : nthreads, nthreads <= 0 ? 0 : ncomm);
  R.g = g;
  int state = 0;
  auto t0 = std::chrono::steady_clock::now();
  int np = 0;
  for (int JB = 0, jb = 0, YN = 0, Yn = 0; JB < N; JB += YN, jb += Yn) {
    int Ym = bb - jb;
    Yn = orc_find_Yn(bb, (int)memBlock, jb, &state);
    int YM = N - JB;
    YN = std::min((jb + Yn) * NB, N) - jb * NB;
    double* X = Y + (size_t)(memBlock - Ym) * NB * NB;
    double* Ajb = A + (size_t)jb * NB * LDA + (size_t)jb * NB;
    a2y(R, Ajb, Y, LDA, NB, YM, YN);
    for (int jjb = 0; jjb < jb; jjb++) {
      a2x(R, A + (size_t)jjb * NB * LDA + (size_t)jb * NB, LDA, X, NB, YM);
      syrk_dag(R, X, Y, YM, YN, NB);
    }
    incore_dag(R, Ajb, Y, LDA, NB, YM, YN, JB);
    np++;
    if (nthreads <= 0) g->barrier();
  }
  g->barrier();
  auto t1 = std::chrono::steady_clock::now();
  delete g;
  *info = R.info.load();
  if (npanels) *npanels = np;
  return std::chrono::duration<double>(t1 - t0).count();
}

// ---------------------------------------------------------------------------------
// Matrix generators.
// ---------------------------------------------------------------------------------

// Counter-based uniform stream: R element with column-major index c (c = i + j*n) is
// output number c of SplitMix64 (Steele, Lea and Flood, 2014) whose state starts at
// mix(seed); the top 53 bits give u in [0,1) and R = u - 1/2.  A = (R + R^T)/2 + alpha*I
// is then exact in binary64, so any implementation of the same rule produces the same
// bits.
static inline uint64_t sm64_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static inline double r_elem(uint64_t key, uint64_t c) {
  uint64_t z = sm64_mix(key + (c + 1) * 0x9E3779B97F4A7C15ULL);
  return (double)(z >> 11) * 0x1.0p-53 - 0.5;
}
extern "C" uint64_t orc_seed_key(uint64_t seed) { return sm64_mix(seed + 0x9E3779B97F4A7C15ULL); }

// Fills the block of A with global rows [r0, r0+m) and columns [c0, c0+nc) into B
// (column-major, leading dimension ldb) for an n x n matrix.
extern "C" void orc_gen_uniform_block(double* B, i64 ldb, i64 n, uint64_t seed, double alpha,
                                      i64 r0, i64 c0, i64 m, i64 nc) {
  uint64_t key = orc_seed_key(seed);
  for (i64 jj = 0; jj < nc; jj++) {
    i64 j = c0 + jj;
    for (i64 ii = 0; ii < m; ii++) {
      i64 i = r0 + ii;
      double v;
      if (i == j) v = r_elem(key, (uint64_t)(i + j * n)) + alpha;
      else v = 0.5 * (r_elem(key, (uint64_t)(i + j * n)) + r_elem(key, (uint64_t)(j + i * n)));
      B[ii + jj * ldb] = v;
    }
  }
}

// pdmatgen('Symm', 'Diag') on a 1 x 1 process grid with MB = NB and M = N, in closed
// form.  The stream is x_{k+1} = (1103515245 x_k + 12345) mod 2^31 with
// x_0 = (1103515245 seed + 12345) mod 2^31 and u_k = x_k / 2^31
// (LIN/pdmatgen.f:117-119,241-250; LIN/pmatgeninc.f:5-135,271-313);
// A(i,j) = 1 - 2 u[min(i,j) N + max(i,j)] (0-based) and A(i,i) = |A(i,i)| + N
// (LIN/pdmatgen.f:223-378,516-543).
static const uint64_t LCG_A = 1103515245ULL, LCG_C = 12345ULL, LCG_M = 0x7FFFFFFFULL;
static inline void lcg_jump(uint64_t k, uint64_t* ak, uint64_t* ck) {
  // (a, c)^k as an affine map x -> ak x + ck (mod 2^31), by binary powering.
  uint64_t ra = 1, rc = 0, ba = LCG_A, bc = LCG_C;
  while (k) {
    if (k & 1) { rc = (ba * rc + bc) & LCG_M; ra = (ba * ra) & LCG_M; }
    bc = (ba * bc + bc) & LCG_M;
    ba = (ba * ba) & LCG_M;
    k >>= 1;
  }
  *ak = ra; *ck = rc;
}
extern "C" void orc_gen_pdmatgen_block(double* B, i64 ldb, i64 n, int seed, i64 r0, i64 c0,
                                       i64 m, i64 nc) {
  uint64_t x0 = (LCG_A * (uint64_t)(uint32_t)seed + LCG_C) & LCG_M;
  for (i64 jj = 0; jj < nc; jj++) {
    i64 j = c0 + jj;
    for (i64 ii = 0; ii < m; ii++) {
      i64 i = r0 + ii;
      i64 lo = std::min(i, j), hi = std::max(i, j);
      uint64_t ak, ck;
      lcg_jump((uint64_t)(lo * n + hi), &ak, &ck);
      uint64_t x = (ak * x0 + ck) & LCG_M;
      double v = 1.0 - 2.0 * ((double)x / 2147483648.0);
      if (i == j) v = std::fabs(v) + (double)n;
      B[ii + jj * ldb] = v;
    }
  }
}

// ---------------------------------------------------------------------------------
// Scaled residual ||A - L L^T||_F / (n eps ||A||_F), eps = 2^-53, using the lower
// triangle of L (leading dimension ldl).  A is regenerated tile by tile from its seed
// (kind 0: uniform generator with `alpha`; kind 1: pdmatgen with integer seed), so only
// the factor needs to be held in memory.  Tiles are t x t; BLAS threads as set.
// ---------------------------------------------------------------------------------
extern "C" double orc_residual(const double* L, i64 n, i64 ldl, int kind, uint64_t seed,
                               double alpha, int t, double* out_normA, double* out_normR) {
  if (n <= 0) return 0.0;
  std::vector<double> At((size_t)t * t), Pt((size_t)t * t);
  double sumR = 0.0, sumA = 0.0;
  for (i64 J = 0; J < n; J += t) {
    int nj = (int)std::min<i64>(t, n - J);
    for (i64 I = J; I < n; I += t) {
      int mi = (int)std::min<i64>(t, n - I);
      // P = sum_{K <= J} L(I,K) L(J,K)^T, i.e. L(I, 0:J+nj) L(J, 0:J+nj)^T restricted to
      // the lower triangle of L (columns < min(I,J)+... handled by L being lower).
      int kk = (int)(J + nj);
      // L(J, 0:kk) has entries above the diagonal of the J block: the caller's upper
      // part is not zero (it holds A), so copy the needed rows with the upper part
      // masked.
      std::vector<double> LI((size_t)mi * kk), LJ((size_t)nj * kk);
      for (int k = 0; k < kk; k++) {
        for (int r = 0; r < mi; r++) { i64 gi = I + r; LI[r + (size_t)k * mi] = (k <= gi) ? L[gi + k * ldl] : 0.0; }
        for (int r = 0; r < nj; r++) { i64 gj = J + r; LJ[r + (size_t)k * nj] = (k <= gj) ? L[gj + k * ldl] : 0.0; }
      }
      blas_dgemm_nt(mi, nj, kk, 1.0, LI.data(), mi, LJ.data(), nj, 0.0, Pt.data(), mi);
      if (kind == 0) orc_gen_uniform_block(At.data(), mi, n, seed, alpha, I, J, mi, nj);
      else orc_gen_pdmatgen_block(At.data(), mi, n, (int)seed, I, J, mi, nj);
      double w = (I == J) ? 1.0 : 2.0;  // off-diagonal blocks appear twice in the full matrix
      double sr = 0, sa = 0;
      for (int c = 0; c < nj; c++)
        for (int r = 0; r < mi; r++) {
          double a = At[r + (size_t)c * mi];
          double d = a - Pt[r + (size_t)c * mi];
          sr += d * d; sa += a * a;
        }
      sumR += w * sr; sumA += w * sa;
    }
  }
  double nA = std::sqrt(sumA), nR = std::sqrt(sumR);
  if (out_normA) *out_normA = nA;
  if (out_normR) *out_normR = nR;
  return nR / ((double)n * 0x1.0p-53 * nA);
}

// Solve A X = B with the factor L (lower, ld ldl), via LAPACK dpotrs; used by tests for
// the solve paths.
extern "C" int orc_potrs(const double* L, int n, int ldl, double* B, int nrhs, int ldb) {
  int info = 0;
  p_dpotrs("L", &n, &nrhs, L, &ldl, B, &ldb, &info, 1);
  return info;
}
