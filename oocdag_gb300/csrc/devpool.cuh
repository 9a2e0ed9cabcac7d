// Device-buffer cache of a handle.
//
// Factor objects take their device buffers from the handle's pool and give them back when
// they are destroyed; a released buffer is kept, keyed by its exact size, and handed to the
// next request of that size.  Freeing a multi-GB buffer costs ~0.4 ms per GB here and
// synchronises the device, so a solve loop that creates and destroys a factor per system
// (one n=65536 split-BF16 factor is 17.6 GB) would otherwise pay it every time.
//
// The cache holds at most `cap` bytes (OOC_OPT_POOL_BYTES); a release beyond that frees.
// An allocation that fails empties the cache and tries once more.  Only buffers whose
// device work has finished may be released into the cache (factor destruction
// synchronises the device first); a buffer replaced while work may still use it is freed
// with cudaFree (drop), which orders itself after that work.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <map>
#include <mutex>
#include <unordered_map>

struct DevPool {
  int device = 0;
  size_t cap = 0;     // bytes the cache may hold
  size_t cached = 0;  // bytes it holds
  std::mutex mu;
  std::multimap<size_t, void*> idle;    // size -> cached buffer
  std::unordered_map<void*, size_t> live;  // buffers handed out -> size

  void* alloc(size_t bytes) {
    std::lock_guard<std::mutex> g(mu);
    auto it = idle.find(bytes);
    if (it != idle.end()) {
      void* p = it->second;
      idle.erase(it);
      cached -= bytes;
      live[p] = bytes;
      return p;
    }
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      flush_locked();
      p = nullptr;
      if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
    }
    live[p] = bytes;
    return p;
  }
  // Back into the cache (the buffer's device work is done).
  void release(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> g(mu);
    auto it = live.find(p);
    if (it == live.end()) {
      cudaFree(p);
      return;
    }
    const size_t b = it->second;
    live.erase(it);
    if (cached + b <= cap) {
      idle.emplace(b, p);
      cached += b;
    } else {
      cudaFree(p);
    }
  }
  // Free now (work may still be pending on it: cudaFree orders itself after that work).
  void drop(void* p) {
    if (!p) return;
    {
      std::lock_guard<std::mutex> g(mu);
      live.erase(p);
    }
    cudaFree(p);
  }
  void set_cap(size_t c) {
    std::lock_guard<std::mutex> g(mu);
    cap = c;
    if (cached > cap) flush_locked();
  }
  void flush_locked() {
    for (auto& kv : idle) cudaFree(kv.second);
    idle.clear();
    cached = 0;
  }
  ~DevPool() {
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(device);
    flush_locked();
    if (prev >= 0) cudaSetDevice(prev);
  }
};
