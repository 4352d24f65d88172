// ephg_ws.cuh - device workspace cache shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdio>
#include <map>
#include <string>
#include <utility>
#include <vector>

namespace ephg {

// Named device buffers that grow on demand and are reused across calls, so a
// repeated request pays no cudaMalloc.  get() returns 0 or EPHG_ERR_NOMEM (6)
// and leaves the reason in msg.
struct Workspace {
  std::map<std::string, std::pair<void *, size_t>> bufs;
  std::string msg;
  int get(const char *name, size_t bytes, void **out) {
    auto it = bufs.find(name);
    if (it != bufs.end() && it->second.second >= bytes) {
      *out = it->second.first;
      return 0;
    }
    if (it != bufs.end()) {
      cudaFree(it->second.first);
      bufs.erase(it);
    }
    void *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      char b[256];
      snprintf(b, sizeof b, "cudaMalloc(%s, %zu bytes): %s", name, bytes, cudaGetErrorString(e));
      msg = b;
      return 6;
    }
    bufs[name] = {p, bytes};
    *out = p;
    return 0;
  }
  void release() {
    for (auto &kv : bufs) cudaFree(kv.second.first);
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
