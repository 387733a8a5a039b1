// Host-side declarations shared by the CUDA translation units of libshci_gpu.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "shci_common.cuh"
#include "status.h"

namespace shci {

#define SHCI_CUDA(call)                                                                         \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) {                                                                    \
      throw ::shci::Error(e_ == cudaErrorMemoryAllocation ? ::shci::kErrOOM : ::shci::kErrCuda, \
                          std::string(#call) + ": " + cudaGetErrorString(e_));                  \
    }                                                                                           \
  } while (0)

// Number of kernel launches issued by the library (every launch site ends with
// SHCI_LAUNCH_CHECK()).
extern std::atomic<int64_t> g_launch_count;
#define SHCI_LAUNCH_CHECK()                                                   \
  do {                                                                        \
    ::shci::g_launch_count.fetch_add(1, std::memory_order_relaxed);           \
    SHCI_CUDA(cudaGetLastError());                                            \
  } while (0)

// SHCI_TRACE >= 2 prints the duration of each build phase to stderr (the
// stream is synchronised at every mark only when tracing is on).
int trace_level();
struct PhaseTimer {
  cudaStream_t s;
  double t0;
  explicit PhaseTimer(cudaStream_t st);
  void mark(const char* what);
};

// Device allocation cap (bytes) for out-of-memory emulation in tests; 0 = off.
extern size_t g_alloc_cap;
extern size_t g_alloc_live;
// Device memory. While a context's call runs on this thread (AllocStream
// scope), buffers come from the device's stream-ordered memory pool on that
// context's stream (cudaMallocAsync / cudaFreeAsync): a freed buffer goes back
// to the pool in stream order and the next allocation reuses its pages, so the
// multi-GB temporaries of each Hamiltonian build are not unmapped and mapped
// again (cudaFree of tens of GB costs ~0.4 ms per GB and synchronises the
// device). Outside such a scope, cudaMalloc / cudaFree. `pooled` records which.
void* dev_alloc(size_t bytes, bool* pooled);
void dev_free(void* p, size_t bytes, bool pooled);
struct AllocStream {
  cudaStream_t prev;
  explicit AllocStream(cudaStream_t s);
  ~AllocStream();
};
// Returns the pool's unused memory to the device (after the stream's pending
// frees have completed), e.g. before sizing buffers from cudaMemGetInfo.
void release_pool_memory(cudaStream_t s);

// Owning device buffer.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;    // elements in use
  size_t cap = 0;  // elements allocated
  bool pooled = false;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) dev_free(p, cap * sizeof(T), pooled);
    p = nullptr;
    n = cap = 0;
    pooled = false;
  }
  // Ensure room for `count` elements; contents are not preserved.
  void reserve(size_t count) {
    if (count <= cap) return;
    release();
    size_t c = count < 16 ? 16 : count;
    p = static_cast<T*>(dev_alloc(c * sizeof(T), &pooled));
    cap = c;
  }
  void resize(size_t count) {
    reserve(count);
    n = count;
  }
  // Grow keeping the first `n` elements.
  void grow_keep(size_t count, cudaStream_t s) {
    if (count <= cap) {
      n = count;
      return;
    }
    size_t c = count + count / 2;
    bool qpooled = false;
    T* q = static_cast<T*>(dev_alloc(c * sizeof(T), &qpooled));
    if (p && n) SHCI_CUDA(cudaMemcpyAsync(q, p, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    if (p) dev_free(p, cap * sizeof(T), pooled);
    p = q;
    pooled = qpooled;
    cap = c;
    n = count;
  }
  size_t bytes() const { return n * sizeof(T); }
  void swap(DevBuf& o) {
    std::swap(p, o.p);
    std::swap(n, o.n);
    std::swap(cap, o.cap);
    std::swap(pooled, o.pooled);
  }
};

// Temporaries of the device primitives, owned by one context (calls on one
// context are serialised on its stream). Each primitive has its own buffers so
// that nested calls (sort -> scan) never share storage.
struct Prims {
  DevBuf<unsigned char> scan_lvl[4];  // block sums per recursion level
  DevBuf<uint64_t> sort_k0, sort_k1;  // alternate key words
  DevBuf<uint32_t> sort_v;            // alternate payload
  DevBuf<uint32_t> sort_hist;         // per-tile digit counts
  DevBuf<uint32_t> sort_glob;         // 16 x 256 global digit histogram
  DevBuf<int64_t> uniq_flag, uniq_pos;
  DevBuf<unsigned char> small;        // small host<->device transfers
};

// ---- primitives (kernels_core.cu) -----------------------------------------
void scan_exclusive_i64(const int64_t* in, int64_t* out, size_t n, int64_t* total_host, Prims& pr,
                        cudaStream_t s);
void scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, Prims& pr, cudaStream_t s);
// Stable sort of determinants in Dice's order (signed words, top word first),
// optionally carrying a uint32 payload (vals may be null). Sorted in place.
void sort_dets(Det2* keys, uint32_t* vals, size_t n, Prims& pr, cudaStream_t s);
// Stable sort of uint64 keys (unsigned order) with a uint32 payload, in place.
void sort_u64(uint64_t* keys, uint32_t* vals, size_t n, Prims& pr, cudaStream_t s);
// Stable sort of 128-bit keys (k1 high word, k0 low word; unsigned order)
// with a uint32 payload, in place. A high word that is the same for every key
// is not moved.
void sort_u128(uint64_t* k0, uint64_t* k1, uint32_t* vals, size_t n, Prims& pr, cudaStream_t s);
// Remove adjacent duplicates of sorted determinants; returns the new count.
size_t unique_dets(Det2* keys, size_t n, Prims& pr, cudaStream_t s);

// Determinant hash set over indices into a determinant array.
struct DetHash {
  DevBuf<uint32_t> slots;
  uint64_t mask = 0;
  void build(const Det2* dets, size_t n, cudaStream_t s);
};

}  // namespace shci
