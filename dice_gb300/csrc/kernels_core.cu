// Device primitives for the determinant bookkeeping of the variational loop:
// exclusive scans, a stable LSD radix sort of 128-bit determinant keys in the
// reference's order, unique, and an open-addressing determinant hash set.
//
// The sort replaces std::sort over Determinant::operator< in
// SHCI/SHCIbasics.cpp:992-994 and :1101-1106; unique replaces std::unique at
// :993-994; the hash set replaces the per-candidate binary_search over
// SortedDets in SHCI/SHCIgetdeterminants.cpp:676,727.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "engine.h"

namespace shci {

size_t g_alloc_cap = 0;
size_t g_alloc_live = 0;

namespace {
thread_local cudaStream_t g_alloc_stream = nullptr;

// The device's default pool keeps freed memory for reuse (no release at
// stream synchronisation); set once per device.
cudaMemPool_t device_pool() {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {nullptr};
  int dev = 0;
  SHCI_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) throw Error(kErrInvalid, "device index beyond 63");
  std::lock_guard<std::mutex> lock(mu);
  if (!pools[dev]) {
    cudaMemPool_t pool = nullptr;
    SHCI_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t keep = ~0ull;
    SHCI_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    pools[dev] = pool;
  }
  return pools[dev];
}
}  // namespace

AllocStream::AllocStream(cudaStream_t s) : prev(g_alloc_stream) { g_alloc_stream = s; }
AllocStream::~AllocStream() { g_alloc_stream = prev; }

void release_pool_memory(cudaStream_t s) {
  if (s) SHCI_CUDA(cudaStreamSynchronize(s));
  SHCI_CUDA(cudaMemPoolTrimTo(device_pool(), 0));
}

void* dev_alloc(size_t bytes, bool* pooled) {
  if (g_alloc_cap && g_alloc_live + bytes > g_alloc_cap)
    throw Error(kErrOOM, "device allocation of " + std::to_string(bytes) + " bytes exceeds the configured cap");
  void* p = nullptr;
  const cudaStream_t s = g_alloc_stream;
  cudaError_t e;
  if (s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    SHCI_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) throw Error(kErrState, "device allocation inside a captured region");
    device_pool();
    e = cudaMallocAsync(&p, bytes, s);
    if (e == cudaErrorMemoryAllocation) {  // give the pool's unused pages back, then once more
      cudaGetLastError();
      release_pool_memory(s);
      e = cudaMallocAsync(&p, bytes, s);
    }
  } else {
    e = cudaMalloc(&p, bytes);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(e == cudaErrorMemoryAllocation ? kErrOOM : kErrCuda,
                std::string(s ? "cudaMallocAsync(" : "cudaMalloc(") + std::to_string(bytes) +
                    "): " + cudaGetErrorString(e));
  }
  *pooled = s != nullptr;
  if (reinterpret_cast<uintptr_t>(p) & 255u) {  // the vector loads of the kernels assume cudaMalloc's alignment
    if (s)
      cudaFreeAsync(p, s);
    else
      cudaFree(p);
    throw Error(kErrCuda, "device allocation not 256-byte aligned");
  }
  g_alloc_live += bytes;
  return p;
}
void dev_free(void* p, size_t bytes, bool pooled) {
  if (pooled && g_alloc_stream)
    cudaFreeAsync(p, g_alloc_stream);
  else
    cudaFree(p);
  g_alloc_live -= std::min(bytes, g_alloc_live);
}

static inline unsigned grid_for(size_t n, int threads, size_t max_blocks = 152 * 64) {
  size_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (unsigned)b;
}

// ---------------------------------------------------------------------------
// Exclusive scan: reduce chunks, scan the chunk sums recursively, downsweep.
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanChunk = kScanThreads * kScanItems;

template <class T>
__device__ T block_exclusive_sum(T v, T* smem_warp, T& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < (kScanThreads / 32) ? smem_warp[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(kFull, w, o);
      if (lane >= o) w += y;
    }
    if (lane < (kScanThreads / 32)) smem_warp[lane] = w;
  }
  __syncthreads();
  T warp_off = warp ? smem_warp[warp - 1] : T(0);
  total = smem_warp[kScanThreads / 32 - 1];
  __syncthreads();
  return warp_off + x - v;
}

template <class T>
__global__ void k_scan_reduce(const T* __restrict__ in, size_t n, T* __restrict__ sums) {
  __shared__ T sw[kScanThreads / 32];
  size_t base = (size_t)blockIdx.x * kScanChunk + (size_t)threadIdx.x * kScanItems;
  T acc = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) acc += in[base + i];
  T total;
  block_exclusive_sum<T>(acc, sw, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <class T>
__global__ void k_scan_down(const T* in, size_t n, const T* __restrict__ offs, T* out) {
  __shared__ T sw[kScanThreads / 32];
  size_t base = (size_t)blockIdx.x * kScanChunk + (size_t)threadIdx.x * kScanItems;
  T v[kScanItems];
  T acc = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : T(0);
    acc += v[i];
  }
  T total;
  T run = block_exclusive_sum<T>(acc, sw, total) + (offs ? offs[blockIdx.x] : T(0));
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
}

template <class T>
static void scan_rec(const T* in, T* out, size_t n, Prims& pr, int level, cudaStream_t s) {
  if (n == 0) return;
  size_t nb = (n + kScanChunk - 1) / kScanChunk;
  if (nb == 1) {
    k_scan_down<T><<<1, kScanThreads, 0, s>>>(in, n, nullptr, out);
    SHCI_LAUNCH_CHECK();
    return;
  }
  if (level >= 4) throw Error(kErrInvalid, "scan too large");
  DevBuf<unsigned char>& lb = pr.scan_lvl[level];
  lb.reserve(nb * sizeof(T));
  T* sums = reinterpret_cast<T*>(lb.p);
  k_scan_reduce<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, sums);
  SHCI_LAUNCH_CHECK();
  scan_rec<T>(sums, sums, nb, pr, level + 1, s);
  k_scan_down<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, sums, out);
  SHCI_LAUNCH_CHECK();
}

void scan_exclusive_i64(const int64_t* in, int64_t* out, size_t n, int64_t* total_host, Prims& pr,
                        cudaStream_t s) {
  if (n == 0) {
    if (total_host) *total_host = 0;
    return;
  }
  int64_t last_in = 0;
  if (total_host && in == out)
    SHCI_CUDA(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  if (total_host && in == out) SHCI_CUDA(cudaStreamSynchronize(s));
  if (total_host && in != out) {
    SHCI_CUDA(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  }
  scan_rec<int64_t>(in, out, n, pr, 0, s);
  if (total_host) {
    int64_t last_out = 0;
    SHCI_CUDA(cudaMemcpyAsync(&last_out, out + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    *total_host = last_out + last_in;
  }
}

void scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, Prims& pr, cudaStream_t s) {
  scan_rec<uint32_t>(in, out, n, pr, 0, s);
}

// ---------------------------------------------------------------------------
// LSD radix sort, 8-bit digits, stable. Keys are unsigned 64-bit words (the
// caller maps signed order onto unsigned order by flipping the sign bit).
// ---------------------------------------------------------------------------
constexpr int kRsThreads = 256;
constexpr int kRsItems = 8;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsWarps = kRsThreads / 32;

__global__ void k_rs_global_hist(const uint64_t* __restrict__ k0, const uint64_t* __restrict__ k1, size_t n,
                                 uint32_t* __restrict__ glob) {
  __shared__ uint32_t h[16 * 256];
  for (int j = threadIdx.x; j < 16 * 256; j += blockDim.x) h[j] = 0;
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint64_t a = k0[i];
#pragma unroll
    for (int d = 0; d < 8; ++d) atomicAdd(&h[d * 256 + ((a >> (8 * d)) & 255)], 1u);
    if (k1) {
      uint64_t b = k1[i];
#pragma unroll
      for (int d = 0; d < 8; ++d) atomicAdd(&h[(8 + d) * 256 + ((b >> (8 * d)) & 255)], 1u);
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < 16 * 256; j += blockDim.x)
    if (h[j]) atomicAdd(&glob[j], h[j]);
}

__global__ void k_rs_tile_hist(const uint64_t* __restrict__ key, size_t n, int shift, uint32_t* __restrict__ hist,
                               unsigned ntiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  size_t base = (size_t)blockIdx.x * kRsTile;
#pragma unroll
  for (int r = 0; r < kRsItems; ++r) {
    size_t i = base + (size_t)r * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(key[i] >> shift) & 255], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_rs_tile_scatter(const uint64_t* __restrict__ kin0, const uint64_t* __restrict__ kin1,
                                  const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout0,
                                  uint64_t* __restrict__ kout1, uint32_t* __restrict__ vout, size_t n, int word,
                                  int shift, const uint32_t* __restrict__ hist, unsigned ntiles) {
  __shared__ uint32_t s_off[256];
  __shared__ uint32_t s_tot[256];
  __shared__ uint32_t s_cnt[kRsWarps][256];
  __shared__ uint32_t s_pre[kRsWarps][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned lt = (1u << lane) - 1u;
  s_off[tid] = hist[(size_t)tid * ntiles + blockIdx.x];
  for (int w = 0; w < kRsWarps; ++w) s_cnt[w][tid] = 0;
  __syncthreads();
  size_t base = (size_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsItems; ++r) {
    size_t i = base + (size_t)r * kRsThreads + tid;
    bool valid = i < n;
    uint64_t a = 0, b = 0;
    uint32_t v = 0;
    int digit = 256;
    if (valid) {
      a = kin0[i];
      if (kin1) b = kin1[i];
      if (vin) v = vin[i];
      digit = (int)(((word ? b : a) >> shift) & 255);
    }
    unsigned peers = __match_any_sync(kFull, digit);
    int rank = __popc(peers & lt);
    if (valid && rank == 0) s_cnt[warp][digit] = __popc(peers);
    __syncthreads();
    {
      uint32_t run = 0;
      for (int w = 0; w < kRsWarps; ++w) {
        uint32_t c = s_cnt[w][tid];
        s_pre[w][tid] = run;
        run += c;
        s_cnt[w][tid] = 0;
      }
      s_tot[tid] = run;
    }
    __syncthreads();
    if (valid) {
      uint32_t pos = s_off[digit] + s_pre[warp][digit] + rank;
      kout0[pos] = a;
      if (kout1) kout1[pos] = b;
      if (vout) vout[pos] = v;
    }
    __syncthreads();
    s_off[tid] += s_tot[tid];
    __syncthreads();
  }
}

// Sorts (k0[, k1][, v]) in place by (k1, k0) unsigned lexicographic order.
static void radix_sort_soa(uint64_t* k0, uint64_t* k1, uint32_t* v, size_t n, Prims& pr, cudaStream_t s) {
  if (n <= 1) return;
  if (n >= (size_t)0xffffffffu) throw Error(kErrInvalid, "sort size exceeds 2^32");
  pr.sort_glob.reserve(16 * 256);
  SHCI_CUDA(cudaMemsetAsync(pr.sort_glob.p, 0, 16 * 256 * sizeof(uint32_t), s));
  k_rs_global_hist<<<grid_for(n, 256, 152 * 4), 256, 0, s>>>(k0, k1, n, pr.sort_glob.p);
  SHCI_LAUNCH_CHECK();
  std::vector<uint32_t> glob(16 * 256);
  SHCI_CUDA(cudaMemcpyAsync(glob.data(), pr.sort_glob.p, glob.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  unsigned ntiles = (unsigned)((n + kRsTile - 1) / kRsTile);
  pr.sort_hist.reserve((size_t)256 * ntiles);
  pr.sort_k0.reserve(n);
  if (k1) pr.sort_k1.reserve(n);
  if (v) pr.sort_v.reserve(n);
  // a constant high word needs no moving: every permutation leaves it as is
  bool k1_const = k1 != nullptr;
  for (int d = 8; k1_const && d < 16; ++d) {
    int nz = 0;
    for (int j = 0; j < 256; ++j) nz += glob[d * 256 + j] != 0;
    k1_const = nz <= 1;
  }
  if (k1_const) k1 = nullptr;
  uint64_t *a0 = k0, *a1 = k1, *b0 = pr.sort_k0.p, *b1 = k1 ? pr.sort_k1.p : nullptr;
  uint32_t *av = v, *bv = v ? pr.sort_v.p : nullptr;
  int npass = 0;
  for (int d = 0; d < (k1 ? 16 : 8); ++d) {
    int nz = 0;
    for (int j = 0; j < 256; ++j) nz += glob[d * 256 + j] != 0;
    if (nz <= 1) continue;  // every key has the same digit here
    int word = d >= 8, shift = 8 * (d & 7);
    k_rs_tile_hist<<<ntiles, kRsThreads, 0, s>>>(word ? a1 : a0, n, shift, pr.sort_hist.p, ntiles);
    SHCI_LAUNCH_CHECK();
    scan_exclusive_u32(pr.sort_hist.p, pr.sort_hist.p, (size_t)256 * ntiles, pr, s);
    k_rs_tile_scatter<<<ntiles, kRsThreads, 0, s>>>(a0, a1, av, b0, b1, bv, n, word, shift, pr.sort_hist.p,
                                                    ntiles);
    SHCI_LAUNCH_CHECK();
    std::swap(a0, b0);
    std::swap(a1, b1);
    std::swap(av, bv);
    ++npass;
  }
  if (npass & 1) {
    SHCI_CUDA(cudaMemcpyAsync(k0, a0, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
    if (k1) SHCI_CUDA(cudaMemcpyAsync(k1, a1, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
    if (v) SHCI_CUDA(cudaMemcpyAsync(v, av, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  }
}

constexpr uint64_t kSign = 0x8000000000000000ull;

__global__ void k_dets_split(const Det2* __restrict__ d, size_t n, uint64_t* k0, uint64_t* k1) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    Det2 x = d[i];
    k0[i] = x.w0 ^ kSign;
    k1[i] = x.w1 ^ kSign;
  }
}
__global__ void k_dets_join(const uint64_t* __restrict__ k0, const uint64_t* __restrict__ k1, size_t n, Det2* d) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    d[i] = Det2{k0[i] ^ kSign, k1[i] ^ kSign};
  }
}

void sort_dets(Det2* keys, uint32_t* vals, size_t n, Prims& pr, cudaStream_t s) {
  if (n <= 1) return;
  // Split into two word arrays; the split copies live in temporaries owned by
  // this call so the radix passes can use the Prims buffers.
  DevBuf<uint64_t> k0, k1;
  k0.resize(n);
  k1.resize(n);
  k_dets_split<<<grid_for(n, 256), 256, 0, s>>>(keys, n, k0.p, k1.p);
  SHCI_LAUNCH_CHECK();
  radix_sort_soa(k0.p, k1.p, vals, n, pr, s);
  k_dets_join<<<grid_for(n, 256), 256, 0, s>>>(k0.p, k1.p, n, keys);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));
}

void sort_u64(uint64_t* keys, uint32_t* vals, size_t n, Prims& pr, cudaStream_t s) {
  radix_sort_soa(keys, nullptr, vals, n, pr, s);
}

void sort_u128(uint64_t* k0, uint64_t* k1, uint32_t* vals, size_t n, Prims& pr, cudaStream_t s) {
  radix_sort_soa(k0, k1, vals, n, pr, s);
}

__global__ void k_unique_flags(const Det2* __restrict__ k, size_t n, int64_t* __restrict__ flag) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    flag[i] = (i == 0 || !det_eq(k[i], k[i - 1])) ? 1 : 0;
}
__global__ void k_unique_scatter(const Det2* __restrict__ k, size_t n, const int64_t* __restrict__ flag,
                                 const int64_t* __restrict__ pos, Det2* __restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (flag[i]) out[pos[i]] = k[i];
}

size_t unique_dets(Det2* keys, size_t n, Prims& pr, cudaStream_t s) {
  if (n <= 1) return n;
  pr.uniq_flag.reserve(n);
  pr.uniq_pos.reserve(n);
  k_unique_flags<<<grid_for(n, 256), 256, 0, s>>>(keys, n, pr.uniq_flag.p);
  SHCI_LAUNCH_CHECK();
  int64_t total = 0;
  scan_exclusive_i64(pr.uniq_flag.p, pr.uniq_pos.p, n, &total, pr, s);
  DevBuf<Det2> tmp;
  tmp.resize((size_t)total);
  k_unique_scatter<<<grid_for(n, 256), 256, 0, s>>>(keys, n, pr.uniq_flag.p, pr.uniq_pos.p, tmp.p);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaMemcpyAsync(keys, tmp.p, (size_t)total * sizeof(Det2), cudaMemcpyDeviceToDevice, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  return (size_t)total;
}

// ---------------------------------------------------------------------------
// Hash set: slots hold indices into the determinant array; linear probing.
// ---------------------------------------------------------------------------
__global__ void k_hash_insert(const Det2* __restrict__ dets, size_t n, uint32_t* slots, uint64_t mask) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint64_t h = det_hash(dets[i]) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
      uint32_t prev = atomicCAS(&slots[h], 0xffffffffu, (uint32_t)i);
      if (prev == 0xffffffffu) break;
      h = (h + 1) & mask;
    }
  }
}

void DetHash::build(const Det2* dets, size_t n, cudaStream_t s) {
  uint64_t cap = 1024;
  while (cap < 2 * (uint64_t)n) cap <<= 1;
  slots.resize(cap);
  mask = cap - 1;
  SHCI_CUDA(cudaMemsetAsync(slots.p, 0xff, cap * sizeof(uint32_t), s));
  if (n) {
    k_hash_insert<<<grid_for(n, 256), 256, 0, s>>>(dets, n, slots.p, mask);
    SHCI_LAUNCH_CHECK();
  }
}

}  // namespace shci
