// Serving runtime: a continuous-batching request loop for factor + solve requests.
//
// Requests (factor a new SPD matrix and solve, or solve again with a resident factor)
// arrive at any time.  A scheduler thread admits them in arrival order against a device
// memory budget (evicting least-recently-used resident factors that nobody is using; a
// request that does not fit yet keeps waiting while later ones that fit are admitted),
// and routes them:
//   * small systems (n <= small_max_n) to a batcher thread that gathers everything admitted
//     within a short window and runs it as ONE persistent batched launch (factor+solve, or
//     solve-only for resident factors), so requests that arrive while a batch runs join
//     the next one;
//   * larger systems to `workers` pipeline threads, each with its own library handle and
//     CUDA streams, so their factorizations and refinements overlap on the device.
// Factors stay resident under the request's key for later repeat solves.  Every answer
// comes with its normwise backward error (FP64 residual against the regenerated matrix).
//
// Matrices are the seeded uniform test matrices A = (R + R^T)/2 + n I, generated on the
// device from their seed, so a request carries a seed, not n^2 numbers.  There is no
// counterpart of this in the reference, which factors one matrix per process.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "devpool.cuh"

int ooc_batched_run_ptrs(cudaStream_t s, int dev, int count, double* const* a, double* const* b, const int* n,
                         const int* mode, int* info_host, const int* blk_table, GrowBuf* ws);

namespace {

// Right-hand sides b ~ N(0,1) of each small item (stream `rhs_key[i]`).
__global__ void k_fill_normals(double* const* b, const int* n, const uint64_t* rhs_key, int count) {
  const int i = blockIdx.x;
  if (i >= count) return;
  for (int r = threadIdx.x; r < n[i]; r += blockDim.x) b[i][r] = ooc_normal_elem(rhs_key[i], (uint64_t)r);
}

// Backward error of each small item: ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)
// with A and b regenerated from their seeds; also sum(x).
__global__ void k_small_berr(double* const* x, const int* n, const uint64_t* a_key, const uint64_t* rhs_key,
                             int count, double* berr, double* xsum) {
  const int i = blockIdx.x;
  if (i >= count) return;
  const int ni = n[i];
  const double alpha = (double)ni;
  const double* xi = x[i];
  __shared__ double s_r[256], s_a[256], s_x[256], s_b[256], s_s[256];
  double mr = 0, ma = 0, mx = 0, mb = 0, sx = 0;
  for (int r = threadIdx.x; r < ni; r += blockDim.x) {
    double acc = ooc_normal_elem(rhs_key[i], (uint64_t)r);
    mb = fmax(mb, fabs(acc));
    double rs = 0;
    for (int c = 0; c < ni; c++) {
      const double a = ooc_uniform_elem(a_key[i], ni, alpha, r, c);
      acc = fma(-a, xi[c], acc);
      rs += fabs(a);
    }
    mr = fmax(mr, fabs(acc));
    ma = fmax(ma, rs);
    mx = fmax(mx, fabs(xi[r]));
    sx += xi[r];
  }
  s_r[threadIdx.x] = mr; s_a[threadIdx.x] = ma; s_x[threadIdx.x] = mx; s_b[threadIdx.x] = mb; s_s[threadIdx.x] = sx;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s_r[threadIdx.x] = fmax(s_r[threadIdx.x], s_r[threadIdx.x + w]);
      s_a[threadIdx.x] = fmax(s_a[threadIdx.x], s_a[threadIdx.x + w]);
      s_x[threadIdx.x] = fmax(s_x[threadIdx.x], s_x[threadIdx.x + w]);
      s_b[threadIdx.x] = fmax(s_b[threadIdx.x], s_b[threadIdx.x + w]);
      s_s[threadIdx.x] += s_s[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double den = s_a[0] * s_x[0] + s_b[0];
    berr[i] = den > 0 ? s_r[0] / den : 0.0;
    xsum[i] = s_s[0];
  }
}

struct Job {
  int64_t id;
  ooc_request r;
  double t_submit = 0, t_admit = 0;
  int64_t reserve = 0;       // bytes reserved at admission
  int64_t factor_bytes = 0;  // part of `reserve` that stays resident afterwards
  bool small = false;
  bool ooc = false;          // factored out of core (host-resident matrix, capped device budget)
  bool hit = false;          // solved with a resident factor
};

struct Entry {
  int64_t n = 0;
  uint64_t seed = 0;
  bool small = false;
  ooc_factor* F = nullptr;  // large
  double* Ls = nullptr;     // small: L in place of A
  int64_t bytes = 0;
  int users = 0;
  double last = 0;
};

}  // namespace

struct ooc_server {
  ooc_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_sched, cv_large, cv_small, cv_done;
  std::deque<Job> pending, large_q;
  std::vector<Job> small_q;
  std::deque<ooc_completion> done;
  std::unordered_map<int64_t, std::vector<double>> sols;
  std::unordered_map<int64_t, Entry> cache;
  int64_t reserved = 0, resident = 0, next_id = 1;
  int64_t budget = 0;
  int running = 0;
  bool stop = false;
  std::thread sched, batcher;
  std::vector<std::thread> workers;
  std::chrono::steady_clock::time_point t0;
  std::string last_error;
  // Device memory in steady state comes from caches, so that a request never frees (a
  // cudaFree synchronises the device under every other pipeline): small systems' factors
  // from `small_pool` (kept by exact size), the batcher's right-hand sides, launch tables
  // and per-system metadata from grow-only buffers.
  std::shared_ptr<DevPool> small_pool;
  GrowBuf bat_b, bat_meta, bat_ws;

  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }

  void release_entry(Entry& e) {  // caller holds mu; device frees happen here
    if (e.F) ooc_factor_destroy(e.F);
    if (e.Ls) small_pool->release(e.Ls);
    e.F = nullptr;
    e.Ls = nullptr;
    resident -= e.bytes;
  }

  bool evict_for(int64_t need, int64_t keep_key) {
    while (reserved + resident + need > budget) {
      int64_t victim = -1;
      double oldest = 1e300;
      for (auto& kv : cache)
        if (kv.second.users == 0 && kv.first != keep_key && kv.second.last < oldest) {
          oldest = kv.second.last;
          victim = kv.first;
        }
      if (victim < 0) return false;
      release_entry(cache[victim]);
      cache.erase(victim);
    }
    return true;
  }

  void complete(const Job& j, int status, int info, int path, int iters, double berr, double xsum,
                std::vector<double>* x) {
    if (status != OOC_OK) {
      const char* m = ooc_last_error_string();
      char buf[96];
      snprintf(buf, sizeof(buf), "request %lld (n=%lld): status %d: ", (long long)j.id, (long long)j.r.n, status);
      last_error = std::string(buf) + (m ? m : "");
    }
    ooc_completion c{};
    c.id = j.id;
    c.status = status;
    c.info = info;
    c.path = path;
    c.factor_reused = j.hit ? 1 : 0;
    c.iterations = iters;
    c.backward_error = berr;
    c.t_submit = j.t_submit;
    c.t_admit = j.t_admit;
    c.t_done = now();
    c.x_sum = xsum;
    done.push_back(c);
    if (x && j.r.keep_solution) sols[j.id] = std::move(*x);
    cv_done.notify_all();
  }

  // ---------------------------------------------------------------- scheduler
  void schedule_loop() {
    cudaSetDevice(cfg.device);
    std::unique_lock<std::mutex> lk(mu);
    while (!stop) {
      cv_sched.wait_for(lk, std::chrono::milliseconds(1));
      bool any_small = false, any_large = false;
      for (size_t i = 0; i < pending.size();) {
        Job& j = pending[i];
        j.small = j.r.n <= cfg.small_max_n;
        auto it = cache.find(j.r.key);
        const bool hit = j.r.kind == 1 && it != cache.end() && it->second.n == j.r.n && (it->second.F || it->second.Ls);
        j.ooc = !hit && !j.small && cfg.ooc_min_n > 0 && j.r.n >= cfg.ooc_min_n;
        const int64_t n = j.r.n;
        // out of core: the factor lives in host memory; the device holds the panel budget
        // and the solve's two panels
        const int64_t need_f = hit || j.ooc ? 0 : (j.small ? 8 * n * n : ooc_factor_bytes(n, cfg.nb, cfg.prec));
        const int64_t need_w = j.small ? 64 * n
                               : j.ooc ? cfg.ooc_budget + 16 * n * cfg.nb + 64 * n + (64LL << 20)
                                       : 64 * n + (64LL << 20);
        const int64_t need = need_f + need_w;
        if (need > budget) {  // can never fit this device budget
          Job jj = j;
          pending.erase(pending.begin() + i);
          complete(jj, OOC_ERR_BUDGET, 0, jj.small ? 0 : jj.ooc ? 2 : 1, 0, 0.0, 0.0, nullptr);
          continue;
        }
        if (!evict_for(need, hit ? j.r.key : -1)) {
          // Does not fit now: it keeps its place; later requests that fit may pass it
          // (a very large request waits until enough memory is free).
          i++;
          continue;
        }
        j.hit = hit;
        j.reserve = need;
        j.factor_bytes = need_f;
        j.t_admit = now();
        reserved += need;
        if (hit) {
          it->second.users++;
          it->second.last = j.t_admit;
        }
        if (j.small) { small_q.push_back(j); any_small = true; }
        else { large_q.push_back(j); any_large = true; }
        pending.erase(pending.begin() + i);
      }
      if (any_small) cv_small.notify_all();
      if (any_large) cv_large.notify_all();
    }
  }

  // ---------------------------------------------------------------- out of core
  // FP64 factorization of a host-resident copy of the matrix through cfg.ooc_budget device
  // bytes (ooc_dpotrf_L, the reference's panel streaming), the solve with the host factor
  // (ooc_dpotrs_L) and the backward error with A regenerated on the device.  One at a time
  // (they share the server's page-locked host matrix, grown to the largest order seen); the
  // host factor is not kept, so a repeat solve of such a key factors again.
  std::mutex ooc_mu;
  double* ooc_host = nullptr;
  size_t ooc_host_bytes = 0;
  void run_ooc(ooc_handle* h, const Job& j, GrowBuf& wbuf) {
    const int64_t n = j.r.n;
    const double alpha = (double)n;
    int status = OOC_OK, info = 0;
    double berr = 0, xsum = 0;
    std::vector<double> x;
    {
      std::lock_guard<std::mutex> olk(ooc_mu);
      const size_t bytes = (size_t)n * n * sizeof(double);
      if (ooc_host_bytes < bytes) {
        if (ooc_host) cudaFreeHost(ooc_host);
        ooc_host = nullptr;
        ooc_host_bytes = 0;
        if (cudaHostAlloc((void**)&ooc_host, bytes, cudaHostAllocDefault) != cudaSuccess) {
          cudaGetLastError();
          ooc_host = nullptr;
          status = OOC_ERR_NOMEM;
        } else {
          ooc_host_bytes = bytes;
        }
      }
      if (status == OOC_OK) status = ooc_dmatgen_uniform(h, ooc_host, n, n, j.r.matrix_seed, alpha);
      if (status == OOC_OK)
        status = ooc_dpotrf_L(h, ooc_host, n, n, cfg.nb, (size_t)cfg.ooc_budget, &info, nullptr);
      double *B = nullptr, *X = nullptr;
      if (status == OOC_OK && info == 0 && (status = wbuf.ensure((size_t)n * 16)) == OOC_OK) {
        B = (double*)wbuf.p;
        X = B + n;
        status = ooc_gen_normal(h, B, n, n, 1, j.r.rhs_seed);
        if (status == OOC_OK && cudaMemcpy(X, B, (size_t)n * 8, cudaMemcpyDeviceToDevice) != cudaSuccess)
          status = OOC_ERR_CUDA;
        if (status == OOC_OK) status = ooc_dpotrs_L(h, ooc_host, n, n, cfg.nb, 0, X, n, 1);
        if (status == OOC_OK) status = ooc_seeded_backward_error(h, n, j.r.matrix_seed, alpha, B, X, &berr);
        if (status == OOC_OK) {
          x.resize(n);
          if (cudaMemcpy(x.data(), X, (size_t)n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) status = OOC_ERR_CUDA;
          for (double v : x) xsum += v;
        }
      }
    }
    std::lock_guard<std::mutex> lk(mu);
    reserved -= j.reserve;
    running--;
    complete(j, status, info, 2, 0, berr, xsum, &x);
  }

  // ---------------------------------------------------------------- large requests
  void worker_loop() {
    cudaSetDevice(cfg.device);
    ooc_handle* h = nullptr;
    if (ooc_create(&h, cfg.device) != OOC_OK) return;
    GrowBuf wbuf;  // this pipeline's right-hand side and solution, kept across requests
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      cv_large.wait(lk, [&] { return stop || !large_q.empty(); });
      if (stop) break;
      Job j = large_q.front();
      large_q.pop_front();
      running++;
      ooc_factor* F = nullptr;
      if (j.hit) F = cache[j.r.key].F;
      lk.unlock();
      if (j.ooc) {
        run_ooc(h, j, wbuf);
        lk.lock();
        continue;
      }
      const int64_t n = j.r.n;
      const double alpha = (double)n;
      int status = OOC_OK, info = 0, iters = 0;
      double berr = 0, xsum = 0;
      std::vector<double> x;
      bool made = false;
      if (!F) {
        status = ooc_factor_create_gen(h, n, j.r.matrix_seed, alpha, cfg.nb, cfg.prec, &F, &info, nullptr);
        made = (status == OOC_OK);
      }
      double *B = nullptr, *X = nullptr;
      if (status == OOC_OK && info == 0) {
        status = wbuf.ensure((size_t)n * 16);
        if (status == OOC_OK) {
          B = (double*)wbuf.p;
          X = B + n;
        }
      }
      if (status == OOC_OK && info == 0) status = ooc_gen_normal(h, B, n, n, 1, j.r.rhs_seed);
      if (status == OOC_OK && info == 0)
        status = ooc_solve_refine_gen(h, F, j.r.matrix_seed, alpha, B, n, X, n, 1, cfg.tol, 30, &iters, &berr);
      if (status == OOC_OK && info == 0) {
        x.resize(n);
        if (cudaMemcpy(x.data(), X, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) status = OOC_ERR_CUDA;
        for (double v : x) xsum += v;
      }
      lk.lock();
      reserved -= j.reserve;
      if (j.hit) {
        Entry& e = cache[j.r.key];
        e.users--;
        e.last = now();
      } else if (made && info == 0 && status == OOC_OK) {
        auto old = cache.find(j.r.key);
        if (old != cache.end() && old->second.users == 0) {
          release_entry(old->second);
          cache.erase(old);
        }
        if (cache.find(j.r.key) == cache.end()) {
          Entry e;
          e.n = n;
          e.seed = j.r.matrix_seed;
          e.F = F;
          e.bytes = j.factor_bytes;
          e.last = now();
          cache[j.r.key] = e;
          resident += e.bytes;
          F = nullptr;
        }
      }
      if (F && made) {  // not kept
        lk.unlock();
        ooc_factor_destroy(F);
        lk.lock();
      }
      running--;
      complete(j, status, info, 1, iters, berr, xsum, &x);
    }
    lk.unlock();
    ooc_destroy(h);
  }

  // ---------------------------------------------------------------- small requests
  void batch_loop() {
    cudaSetDevice(cfg.device);
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      cv_small.wait(lk, [&] { return stop || !small_q.empty(); });
      if (stop) break;
      // let requests that arrive meanwhile join this batch
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds((int64_t)(cfg.batch_window_ms * 1000)));
      lk.lock();
      std::vector<Job> batch;
      batch.swap(small_q);
      running += (int)batch.size();
      std::vector<double*> Ls(batch.size(), nullptr);
      for (size_t i = 0; i < batch.size(); i++)
        if (batch[i].hit) Ls[i] = cache[batch[i].r.key].Ls;
      lk.unlock();
      run_batch(s, batch, Ls);
      lk.lock();
    }
    lk.unlock();
    cudaStreamDestroy(s);
  }

  void run_batch(cudaStream_t s, std::vector<Job>& batch, std::vector<double*>& Ls) {
    const int count = (int)batch.size();
    std::vector<int> n(count), mode(count), info(count, 0);
    std::vector<double*> b(count);
    std::vector<uint64_t> akey(count), bkey(count);
    std::vector<bool> made(count, false);
    int64_t btot = 0;
    for (int i = 0; i < count; i++) {
      n[i] = (int)batch[i].r.n;
      btot += n[i];
      akey[i] = ooc_uniform_key(batch[i].r.matrix_seed);
      bkey[i] = ooc_uniform_key(batch[i].r.rhs_seed);
    }
    int status = OOC_OK;
    double* Bbuf = nullptr;
    void* meta = nullptr;
    if (bat_b.ensure((size_t)std::max<int64_t>(btot, 1) * 8) != OOC_OK ||
        bat_meta.ensure((size_t)count * (8 + 4 + 8 + 8 + 8 + 8) + 64) != OOC_OK) {
      status = OOC_ERR_NOMEM;
    } else {
      Bbuf = (double*)bat_b.p;
      meta = bat_meta.p;
    }
    int64_t off = 0;
    for (int i = 0; i < count && status == OOC_OK; i++) {
      b[i] = Bbuf + off;
      off += n[i];
      if (Ls[i]) {
        mode[i] = 1;
      } else {
        mode[i] = 0;
        Ls[i] = (double*)small_pool->alloc((size_t)n[i] * n[i] * 8);
        if (!Ls[i]) {
          status = OOC_ERR_NOMEM;
          break;
        }
        made[i] = true;
        status = launch_gen_uniform_block(Ls[i], n[i], n[i], batch[i].r.matrix_seed, (double)n[i], 0, 0, n[i], n[i], s);
        if (status != OOC_OK) break;
      }
    }
    std::vector<double> berr(count, 0.0), xsum(count, 0.0);
    if (status == OOC_OK) {
      char* mp = (char*)meta;
      double** d_b = (double**)mp;
      mp += (size_t)count * 8;
      int* d_n = (int*)mp;
      mp += (size_t)count * 4;
      mp = (char*)(((uintptr_t)mp + 7) & ~(uintptr_t)7);
      uint64_t* d_ak = (uint64_t*)mp;
      mp += (size_t)count * 8;
      uint64_t* d_bk = (uint64_t*)mp;
      mp += (size_t)count * 8;
      double* d_be = (double*)mp;
      mp += (size_t)count * 8;
      double* d_xs = (double*)mp;
      auto chk = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess && status == OOC_OK) {
          ooc_set_last_error(e, what, __FILE__, __LINE__);
          status = OOC_ERR_CUDA;
        }
      };
      chk(cudaMemcpyAsync(d_b, b.data(), (size_t)count * 8, cudaMemcpyHostToDevice, s), "copy b pointers");
      chk(cudaMemcpyAsync(d_n, n.data(), (size_t)count * 4, cudaMemcpyHostToDevice, s), "copy n");
      chk(cudaMemcpyAsync(d_ak, akey.data(), (size_t)count * 8, cudaMemcpyHostToDevice, s), "copy matrix keys");
      chk(cudaMemcpyAsync(d_bk, bkey.data(), (size_t)count * 8, cudaMemcpyHostToDevice, s), "copy rhs keys");
      k_fill_normals<<<count, 128, 0, s>>>(d_b, d_n, d_bk, count);
      chk(cudaGetLastError(), "k_fill_normals");
      if (status == OOC_OK)
        status = ooc_batched_run_ptrs(s, cfg.device, count, Ls.data(), b.data(), n.data(), mode.data(), info.data(),
                                      nullptr, &bat_ws);
      if (status == OOC_OK) {
        k_small_berr<<<count, 256, 0, s>>>(d_b, d_n, d_ak, d_bk, count, d_be, d_xs);
        chk(cudaGetLastError(), "k_small_berr");
        chk(cudaMemcpyAsync(berr.data(), d_be, (size_t)count * 8, cudaMemcpyDeviceToHost, s), "copy berr");
        chk(cudaMemcpyAsync(xsum.data(), d_xs, (size_t)count * 8, cudaMemcpyDeviceToHost, s), "copy xsum");
        chk(cudaStreamSynchronize(s), "batch synchronize");
      }
    }
    std::vector<std::vector<double>> xs(count);
    for (int i = 0; i < count && status == OOC_OK; i++)
      if (batch[i].r.keep_solution) {
        xs[i].resize(n[i]);
        cudaMemcpy(xs[i].data(), b[i], (size_t)n[i] * 8, cudaMemcpyDeviceToHost);
      }
    std::lock_guard<std::mutex> lk(mu);
    for (int i = 0; i < count; i++) {
      Job& j = batch[i];
      reserved -= j.reserve;
      if (j.hit) {
        Entry& e = cache[j.r.key];
        e.users--;
        e.last = now();
      } else if (made[i] && status == OOC_OK && info[i] == 0) {
        auto old = cache.find(j.r.key);
        if (old != cache.end() && old->second.users == 0) {
          release_entry(old->second);
          cache.erase(old);
        }
        if (cache.find(j.r.key) == cache.end()) {
          Entry e;
          e.n = n[i];
          e.seed = j.r.matrix_seed;
          e.small = true;
          e.Ls = Ls[i];
          e.bytes = j.factor_bytes;
          e.last = now();
          cache[j.r.key] = e;
          resident += e.bytes;
          made[i] = false;
        }
      }
      if (made[i] && Ls[i]) small_pool->release(Ls[i]);  // not kept
      running--;
      complete(j, status, info[i], 0, 0, berr[i], xsum[i], &xs[i]);
    }
  }
};

extern "C" int ooc_server_create(const ooc_server_config* cfg, ooc_server** out) {
  if (!cfg) return -1;
  if (!out) return -2;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) {
    cudaGetLastError();
    return OOC_ERR_NODEVICE;
  }
  ooc_server* S = new ooc_server();
  S->cfg = *cfg;
  if (S->cfg.workers <= 0) S->cfg.workers = 4;
  if (S->cfg.small_max_n <= 0 || S->cfg.small_max_n > 512) S->cfg.small_max_n = 512;
  if (S->cfg.nb <= 0) S->cfg.nb = 512;
  if (S->cfg.tol <= 0) S->cfg.tol = 1e-14;
  if (S->cfg.batch_window_ms < 0) S->cfg.batch_window_ms = 0;
  cudaSetDevice(S->cfg.device);
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  S->budget = S->cfg.hbm_budget > 0 ? S->cfg.hbm_budget : (int64_t)(fr / 10 * 9);
  if (S->cfg.ooc_budget <= 0) S->cfg.ooc_budget = 24LL << 30;
  S->small_pool = std::make_shared<DevPool>();
  S->small_pool->device = S->cfg.device;
  S->small_pool->cap = (size_t)1 << 30;  // evicted small factors kept for reuse (2 MB each at n=512)
  S->t0 = std::chrono::steady_clock::now();
  S->sched = std::thread([S] { S->schedule_loop(); });
  S->batcher = std::thread([S] { S->batch_loop(); });
  for (int w = 0; w < S->cfg.workers; w++) S->workers.emplace_back([S] { S->worker_loop(); });
  *out = S;
  return OOC_OK;
}

extern "C" int ooc_server_submit(ooc_server* S, const ooc_request* r, int64_t* id) {
  if (!S) return -1;
  if (!r || r->n <= 0 || (r->kind != 0 && r->kind != 1)) return -2;
  std::lock_guard<std::mutex> lk(S->mu);
  Job j;
  j.id = S->next_id++;
  j.r = *r;
  j.t_submit = S->now();
  S->pending.push_back(j);
  if (id) *id = j.id;
  S->cv_sched.notify_all();
  return OOC_OK;
}

extern "C" int ooc_server_poll(ooc_server* S, ooc_completion* out, int max, int* count, int wait_ms) {
  if (!S) return -1;
  if (!out && max > 0) return -2;
  if (!count) return -4;
  std::unique_lock<std::mutex> lk(S->mu);
  if (S->done.empty() && wait_ms > 0)
    S->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !S->done.empty(); });
  int k = 0;
  while (k < max && !S->done.empty()) {
    out[k++] = S->done.front();
    S->done.pop_front();
  }
  *count = k;
  return OOC_OK;
}

extern "C" int ooc_server_solution(ooc_server* S, int64_t id, double* x, int64_t n) {
  if (!S) return -1;
  if (!x) return -3;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->sols.find(id);
  if (it == S->sols.end()) return -2;
  if ((int64_t)it->second.size() != n) return -4;
  memcpy(x, it->second.data(), n * 8);
  S->sols.erase(it);
  return OOC_OK;
}

extern "C" int ooc_server_status(ooc_server* S, int64_t* pending, int64_t* running, int64_t* resident_bytes,
                                 int64_t* reserved_bytes) {
  if (!S) return -1;
  std::lock_guard<std::mutex> lk(S->mu);
  if (pending) *pending = (int64_t)S->pending.size();
  if (running) *running = (int64_t)(S->running + S->large_q.size() + S->small_q.size());
  if (resident_bytes) *resident_bytes = S->resident;
  if (reserved_bytes) *reserved_bytes = S->reserved;
  return OOC_OK;
}

extern "C" double ooc_server_now(ooc_server* S) { return S ? S->now() : 0.0; }

extern "C" const char* ooc_server_last_error(ooc_server* S) {
  if (!S) return "";
  std::lock_guard<std::mutex> lk(S->mu);
  return S->last_error.c_str();
}

extern "C" int ooc_server_destroy(ooc_server* S) {
  if (!S) return OOC_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_sched.notify_all();
  S->cv_large.notify_all();
  S->cv_small.notify_all();
  if (S->sched.joinable()) S->sched.join();
  if (S->batcher.joinable()) S->batcher.join();
  for (auto& t : S->workers)
    if (t.joinable()) t.join();
  cudaSetDevice(S->cfg.device);
  for (auto& kv : S->cache) S->release_entry(kv.second);
  S->cache.clear();
  if (S->ooc_host) cudaFreeHost(S->ooc_host);
  delete S;
  return OOC_OK;
}
