// ephg_ws.cuh - device workspace cache shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

namespace ephg {

// The library's device memory: one stream-ordered pool per device that keeps
// freed memory (up to half the device) mapped for the next allocation instead
// of returning it at every synchronisation, so that a handle created after
// another one was destroyed, or a request's workspace after the last one's,
// reuses mapped memory: cudaFree / first-touch mapping of gigabytes costs
// milliseconds per call.  Memory above the threshold is returned as usual.
inline cudaMemPool_t lib_pool(int device) {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lk(mu);
  auto it = pools.find(device);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  cudaMemPool_t pool = nullptr;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
    cudaGetLastError();
    if (cudaDeviceGetDefaultMemPool(&pool, device) != cudaSuccess) return nullptr;
  } else {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    uint64_t keep = (uint64_t)tot / 2;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  pools[device] = pool;
  return pool;
}

// bytes from the current device's library pool, ordered on st
inline cudaError_t pool_alloc(void **p, size_t bytes, cudaStream_t st) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaMemPool_t pool = lib_pool(dev);
  if (!pool) return cudaMallocAsync(p, bytes, st);
  return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

// Named device buffers that grow on demand and are reused across calls, so a
// repeated request pays no cudaMalloc.  get() returns 0 or EPHG_ERR_NOMEM (6)
// and leaves the reason in msg: cudaMalloc failed, or growing the cache would
// take its total past `limit` (the serving loop's share of the HBM budget).
// Buffers are allocated and freed stream-ordered on `st` (the library pool,
// cudaFreeAsync): unlike cudaMalloc / cudaFree these do not wait for the other
// streams of the device, so a request that grows its workspace does not stall
// behind the kernels of other requests running concurrently.
struct Workspace {
  std::map<std::string, std::pair<void *, size_t>> bufs;
  std::string msg;
  size_t limit = (size_t)-1;
  cudaStream_t st = nullptr;
  // optional reservation hook (the serving loop's HBM budget): asked before the
  // cache grows by delta > 0 bytes; false refuses the growth (EPHG_ERR_NOMEM).
  // Growth that then fails to allocate is given back with a negative delta.
  // release() does not call it: the owner accounts for released bytes.
  bool (*grow)(void *ctx, int64_t delta) = nullptr;
  void *grow_ctx = nullptr;
  size_t total() const {
    size_t t = 0;
    for (auto &kv : bufs) t += kv.second.second;
    return t;
  }
  int get(const char *name, size_t bytes, void **out) {
    auto it = bufs.find(name);
    if (it != bufs.end() && it->second.second >= bytes) {
      *out = it->second.first;
      return 0;
    }
    const size_t old_bytes = it != bufs.end() ? it->second.second : 0;
    const int64_t delta = (int64_t)(bytes ? bytes : 16) - (int64_t)old_bytes;
    {
      const size_t want = total() - old_bytes + (bytes ? bytes : 16);
      if (want > limit) {
        char b[256];
        snprintf(b, sizeof b, "workspace %s: %zu bytes in total would exceed the budget of %zu bytes", name, want,
                 limit);
        msg = b;
        return 6;
      }
      if (grow && delta > 0 && !grow(grow_ctx, delta)) {
        char b[256];
        snprintf(b, sizeof b, "workspace %s: growing by %lld bytes would exceed the HBM budget", name,
                 (long long)delta);
        msg = b;
        return 6;
      }
    }
    if (it != bufs.end()) {
      cudaFreeAsync(it->second.first, st);
      bufs.erase(it);
    }
    void *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = pool_alloc(&p, bytes, st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      if (grow) grow(grow_ctx, -(int64_t)bytes);   // the old buffer is gone too: give back all
      char b[256];
      snprintf(b, sizeof b, "cudaMallocAsync(%s, %zu bytes): %s", name, bytes, cudaGetErrorString(e));
      msg = b;
      return 6;
    }
    bufs[name] = {p, bytes};
    *out = p;
    return 0;
  }
  void release() {
    for (auto &kv : bufs) cudaFreeAsync(kv.second.first, st);
    bufs.clear();
  }
};

template <typename T>
int wsget(Workspace &ws, const char *name, size_t count, T **out) {
  void *p = nullptr;
  int rc = ws.get(name, count * sizeof(T), &p);
  *out = (T *)p;
  return rc;
}

// Cooperative hand-over point of a long request (the serving loop): called
// between launches; it may drain the caller's stream and block while a
// smaller request owns the GPU.  A default-constructed hook does nothing.
struct Yield {
  void (*fn)(void *) = nullptr;
  void *ctx = nullptr;
  void operator()() const {
    if (fn) fn(ctx);
  }
};

// Device-time accumulator for a family of kernel launches: mark() before and
// after each launch on the launching stream, total_ms() after a stream sync.
struct LaunchTimer {
  std::vector<cudaEvent_t> ev;
  size_t used = 0;
  int n = 0;
  void reset() { used = 0; n = 0; }
  void mark(cudaStream_t st) {
    if (used == ev.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev.push_back(e);
    }
    cudaEventRecord(ev[used++], st);
  }
  void begin(cudaStream_t st) { mark(st); }
  void end(cudaStream_t st) {
    mark(st);
    ++n;
  }
  double total_ms() const {
    double t = 0;
    for (size_t i = 0; i + 1 < used; i += 2) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
      t += ms;
    }
    return t;
  }
  ~LaunchTimer() {
    for (auto e : ev) cudaEventDestroy(e);
  }
};

}  // namespace ephg
