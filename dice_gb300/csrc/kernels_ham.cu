// Hamiltonian-side kernels of the variational loop:
//   * alpha/beta string tables and single-excitation neighbour lists
//     (replaces HamHelpers2::PopulateHelpers, SHCI/SHCImakeHamiltonian.cpp:184-408);
//   * the diagonal energies (Determinant::Energy at SHCI/SHCIbasics.cpp:1145-1154);
//   * the two-pass count/emit build of the sparse Hamiltonian as full-row CSR
//     (replaces MakeHfromSMHelpers2, SHCI/SHCImakeHamiltonian.cpp:486-715);
//   * the matrix-free sigma (replaces HmultDirect::operator(), SHCI/Hmult.h:241-381).
//
// One warp owns one row I. The connected determinants J are found in three
// scans over string groups:
//   1. determinants sharing I's alpha string: beta distance 1 or 2;
//   2. determinants whose alpha string is a single excitation of I's and whose
//      beta string equals I's or is one excitation away;
//   3. determinants sharing I's beta string: alpha distance 2.
// This visits the same (I, J) set as the reference's five helper-list classes
// (single alpha, alpha-beta, single beta, double beta, double alpha).
#include "engine.h"
#include "ham.h"

namespace shci {

static inline unsigned grid_for(size_t n, int threads, size_t max_blocks = 152 * 64) {
  size_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (unsigned)b;
}

// ---------------------------------------------------------------------------
// Strings and groups
// ---------------------------------------------------------------------------
__global__ void k_strings(const Det2* __restrict__ dets, size_t n, uint64_t* __restrict__ astr,
                          uint64_t* __restrict__ bstr, uint64_t* __restrict__ akey, uint64_t* __restrict__ bkey,
                          uint32_t* __restrict__ ia, uint32_t* __restrict__ ib) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    Det2 d = dets[i];
    uint64_t a = det_alpha(d), b = det_beta(d);
    astr[i] = a;
    bstr[i] = b;
    akey[i] = a;
    bkey[i] = b;
    ia[i] = (uint32_t)i;
    ib[i] = (uint32_t)i;
  }
}

__global__ void k_group_flags(const uint64_t* __restrict__ key, size_t n, int64_t* __restrict__ flag) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    flag[i] = (i == 0 || key[i] != key[i - 1]) ? 1 : 0;
}

// seg(p) = inclusive count - 1; writes the unique string, group start, the
// det -> group map and the partner string of every grouped determinant.
__global__ void k_group_fill(const uint64_t* __restrict__ key, const uint32_t* __restrict__ perm, size_t n,
                             const int64_t* __restrict__ flag, const int64_t* __restrict__ excl,
                             uint64_t* __restrict__ ustr, int64_t* __restrict__ start, uint32_t* __restrict__ idx,
                             const uint64_t* __restrict__ partner, uint64_t* __restrict__ group_partner) {
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    int64_t seg = excl[p] + flag[p] - 1;
    if (flag[p]) {
      ustr[seg] = key[p];
      start[seg] = (int64_t)p;
    }
    uint32_t d = perm[p];
    idx[d] = (uint32_t)seg;
    group_partner[p] = partner[d];
  }
}

__device__ __forceinline__ int64_t bsearch_u64(const uint64_t* __restrict__ a, int64_t n, uint64_t x) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    uint64_t v = a[mid];
    if (v < x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < n && a[lo] == x) ? lo : -1;
}

// Single-excitation neighbours of every unique alpha string among the present
// alpha strings (SinglesFromAlpha, SHCI/SHCImakeHamiltonian.cpp:237-252).
// Warp per string; lanes over (occupied i, empty a) pairs.
template <bool kEmit>
__global__ void k_alpha_singles(const uint64_t* __restrict__ ua, int64_t na, int norb, int64_t* __restrict__ counts,
                                const int64_t* __restrict__ offs, uint32_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < na; s += warps) {
    const uint64_t x = ua[s];
    const int nocc = __popcll(x);
    const int nvir = norb - nocc;
    const int total = nocc * nvir;
    int64_t cnt = 0;
    int64_t pos = kEmit ? offs[s] : 0;
    for (int base = 0; base < total; base += 32) {
      int q = base + lane;
      bool hit = false;
      int64_t idx = -1;
      if (q < total) {
        int oi = q / nvir, va = q % nvir;
        // oi-th set bit and va-th clear bit (below norb)
        uint64_t occ = x, vir = (~x) & (norb == 64 ? ~0ull : ((1ull << norb) - 1ull));
        for (int t = 0; t < oi; ++t) occ &= occ - 1;
        for (int t = 0; t < va; ++t) vir &= vir - 1;
        int i = __ffsll((long long)occ) - 1, a = __ffsll((long long)vir) - 1;
        uint64_t y = (x ^ (1ull << i)) | (1ull << a);
        idx = bsearch_u64(ua, na, y);
        hit = idx >= 0;
      }
      unsigned m = __ballot_sync(kFull, hit);
      if (kEmit && hit) out[pos + __popc(m & ((1u << lane) - 1u))] = (uint32_t)idx;
      pos += __popc(m);
      cnt += __popc(m);
    }
    if (!kEmit && lane == 0) counts[s] = cnt;
  }
}

__global__ void k_iota_last(int64_t* start, int64_t n_groups, int64_t n_total) { start[n_groups] = n_total; }

static void build_groups(const uint64_t* str_of_det, const uint64_t* partner_of_det, size_t n, DevBuf<uint64_t>& key,
                         DevBuf<uint32_t>& perm, DevBuf<uint64_t>& ustr, DevBuf<int64_t>& start,
                         DevBuf<uint32_t>& idx, DevBuf<uint64_t>& gpartner, int64_t& ngroups, Prims& pr,
                         cudaStream_t s) {
  sort_u64(key.p, perm.p, n, pr, s);
  DevBuf<int64_t> flag, excl;
  flag.resize(n);
  excl.resize(n);
  k_group_flags<<<grid_for(n, 256), 256, 0, s>>>(key.p, n, flag.p);
  SHCI_LAUNCH_CHECK();
  scan_exclusive_i64(flag.p, excl.p, n, &ngroups, pr, s);
  ustr.resize(ngroups);
  start.resize(ngroups + 1);
  idx.resize(n);
  gpartner.resize(n);
  k_group_fill<<<grid_for(n, 256), 256, 0, s>>>(key.p, perm.p, n, flag.p, excl.p, ustr.p, start.p, idx.p,
                                                 partner_of_det, gpartner.p);
  SHCI_LAUNCH_CHECK();
  k_iota_last<<<1, 1, 0, s>>>(start.p, ngroups, (int64_t)n);
  SHCI_LAUNCH_CHECK();
  (void)str_of_det;
}

void Helpers::build(const Det2* dets, size_t n, int norb, Prims& pr, cudaStream_t s) {
  N = n;
  astr.resize(n);
  bstr.resize(n);
  DevBuf<uint64_t> akey, bkey;
  akey.resize(n);
  bkey.resize(n);
  aDets.resize(n);
  bDets.resize(n);
  k_strings<<<grid_for(n, 256), 256, 0, s>>>(dets, n, astr.p, bstr.p, akey.p, bkey.p, aDets.p, bDets.p);
  SHCI_LAUNCH_CHECK();
  build_groups(astr.p, bstr.p, n, akey, aDets, ua, aStart, aidx, aGroupB, NA, pr, s);
  build_groups(bstr.p, astr.p, n, bkey, bDets, ub, bStart, bidx, bGroupA, NB, pr, s);
  // alpha single-excitation lists
  DevBuf<int64_t> cnt;
  cnt.resize(NA);
  aSingStart.resize(NA + 1);
  k_alpha_singles<false><<<grid_for((size_t)NA * 32, 256), 256, 0, s>>>(ua.p, NA, norb, cnt.p, nullptr, nullptr);
  SHCI_LAUNCH_CHECK();
  int64_t total = 0;
  scan_exclusive_i64(cnt.p, aSingStart.p, NA, &total, pr, s);
  k_iota_last<<<1, 1, 0, s>>>(aSingStart.p, NA, total);
  SHCI_LAUNCH_CHECK();
  aSing.resize(total > 0 ? total : 1);
  k_alpha_singles<true><<<grid_for((size_t)NA * 32, 256), 256, 0, s>>>(ua.p, NA, norb, nullptr, aSingStart.p,
                                                                         aSing.p);
  SHCI_LAUNCH_CHECK();
  nsing = total;
  SHCI_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// Row traversal shared by count, emit and the matrix-free sigma.
// V::step(hit, J) is called by all 32 lanes together.
// ---------------------------------------------------------------------------
template <class V>
__device__ void visit_row(const HelperView& h, uint32_t I, V& v) {
  const int lane = threadIdx.x & 31;
  const uint64_t A = h.astr[I], B = h.bstr[I];
  const uint32_t ia = h.aidx[I], ib = h.bidx[I];
  // 1. same alpha string: beta single or double
  {
    const int64_t p0 = h.aStart[ia], p1 = h.aStart[ia + 1];
    for (int64_t base = p0; base < p1; base += 32) {
      int64_t p = base + lane;
      bool hit = false;
      uint32_t J = 0;
      int d = -1;
      if (p < p1) {
        d = __popcll(h.aGroupB[p] ^ B);
        hit = (d == 2 || d == 4);
        J = h.aDets[p];
      }
      v.step(hit, J, d == 2);
    }
  }
  // 2. alpha single excitation: beta equal (single alpha) or beta single (alpha-beta double)
  {
    const int64_t s0 = h.aSingStart[ia], s1 = h.aSingStart[ia + 1];
    for (int64_t base = s0; base < s1; base += 32) {
      int64_t q = base + lane;
      int64_t g0 = 0, len = 0;
      if (q < s1) {
        uint32_t As = h.aSing[q];
        g0 = h.aStart[As];
        len = h.aStart[As + 1] - g0;
      }
      int64_t incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
      }
      const int64_t total = __shfl_sync(kFull, incl, 31);
      const int64_t excl = incl - len;
      for (int64_t f0 = 0; f0 < total; f0 += 32) {
        const int64_t f = f0 + lane;
        int lo = 0;
#pragma unroll
        for (int st = 16; st >= 1; st >>= 1) {
          int c = lo + st;
          int64_t e = __shfl_sync(kFull, excl, c < 32 ? c : 31);
          if (c < 32 && e <= f) lo = c;
        }
        int64_t gb = __shfl_sync(kFull, g0, lo);
        int64_t eo = __shfl_sync(kFull, excl, lo);
        bool hit = false;
        uint32_t J = 0;
        int d = -1;
        if (f < total) {
          int64_t p = gb + (f - eo);
          d = __popcll(h.aGroupB[p] ^ B);
          hit = (d == 0 || d == 2);
          J = h.aDets[p];
        }
        v.step(hit, J, d == 0);
      }
    }
  }
  // 3. same beta string: alpha double
  {
    const int64_t p0 = h.bStart[ib], p1 = h.bStart[ib + 1];
    for (int64_t base = p0; base < p1; base += 32) {
      int64_t p = base + lane;
      bool hit = false;
      uint32_t J = 0;
      if (p < p1) {
        int d = __popcll(h.bGroupA[p] ^ A);
        hit = (d == 4);
        J = h.bDets[p];
      }
      v.step(hit, J, false);
    }
  }
}

struct CountVisitor {
  int64_t c = 0;
  __device__ void step(bool hit, uint32_t, bool) { c += hit; }
};

__global__ void k_ham_count(HelperView h, int64_t* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t I = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < (int64_t)h.N; I += warps) {
    CountVisitor v;
    visit_row(h, (uint32_t)I, v);
    int64_t c = v.c;
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
    if (lane == 0) counts[I] = c;
  }
}

// Emits (col, value) for one row; H_IJ is evaluated with the higher-index
// determinant as the ket, the element the reference stores in row max(I,J)
// (SHCI/SHCImakeHamiltonian.cpp:565-580).
//
// Connections found by the scans are queued per warp in shared memory, one
// queue for single and one for double excitations; whenever a queue holds 32
// entries all lanes evaluate one Slater-Condon element each, so the FP64 work
// runs on full warps and singles (an O(n_elec) sum) do not wait on doubles.
struct EmitVisitor {
  const Det2* dets;
  IntsView ints;
  Det2 dI;
  uint32_t I;
  int64_t pos;
  int32_t* col;
  double* v64;
  float* vhi;
  float* vlo;
  uint32_t* qs;  // 64 entries: single excitations
  uint32_t* qd;  // 64 entries: double excitations
  int ns, nd;

  __device__ void store(int64_t q, uint32_t J) {
    const Det2 dJ = dets[J];
    const double hv = (J < I) ? hij_any(ints, dJ, dI) : hij_any(ints, dI, dJ);
    col[q] = (int32_t)J;
    if (v64) v64[q] = hv;
    if (vhi) {
      const float hi = (float)hv;
      vhi[q] = hi;
      if (vlo) vlo[q] = (float)(hv - (double)hi);
    }
  }
  // evaluate the first `cnt` (<= 32) entries of queue q, then shift the rest down
  __device__ int drain(uint32_t* q, int n, int cnt) {
    const int lane = threadIdx.x & 31;
    if (lane < cnt) store(pos + lane, q[lane]);
    pos += cnt;
    __syncwarp();
    const int rest = n - cnt;
    uint32_t v = lane < rest ? q[cnt + lane] : 0u;
    __syncwarp();
    if (lane < rest) q[lane] = v;
    __syncwarp();
    return rest;
  }
  __device__ void step(bool hit, uint32_t J, bool single) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned ms = __ballot_sync(kFull, hit && single);
    const unsigned md = __ballot_sync(kFull, hit && !single);
    if (hit && single) qs[ns + __popc(ms & lt)] = J;
    if (hit && !single) qd[nd + __popc(md & lt)] = J;
    ns += __popc(ms);
    nd += __popc(md);
    __syncwarp();
    if (ns >= 32) ns = drain(qs, ns, 32);
    if (nd >= 32) nd = drain(qd, nd, 32);
  }
  __device__ void flush() {
    if (ns) ns = drain(qs, ns, ns);
    if (nd) nd = drain(qd, nd, nd);
  }
};

__global__ void __launch_bounds__(256) k_ham_emit(HelperView h, const Det2* __restrict__ dets, IntsView ints,
                                                  const int64_t* __restrict__ rowptr, int32_t* __restrict__ col,
                                                  double* __restrict__ v64, float* __restrict__ vhi,
                                                  float* __restrict__ vlo) {
  __shared__ uint32_t s_q[8][2][64];
  const int wib = threadIdx.x >> 5;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t I = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < (int64_t)h.N; I += warps) {
    EmitVisitor v{dets, ints, dets[I], (uint32_t)I, rowptr[I], col, v64, vhi, vlo, s_q[wib][0], s_q[wib][1], 0, 0};
    visit_row(h, (uint32_t)I, v);
    v.flush();
  }
}

__global__ void k_set_last(int64_t* rowptr, int64_t n, int64_t total) { rowptr[n] = total; }

void build_ham_csr(const Helpers& hp, const Det2* dets, const IntsView& ints, Csr& H, bool want64, bool want32,
                   bool want_lo, Prims& pr, cudaStream_t s) {
  const size_t N = hp.N;
  HelperView hv = hp.view();
  DevBuf<int64_t> counts;
  counts.resize(N);
  const unsigned blocks = grid_for(N * 32, 256, 152 * 16);
  k_ham_count<<<blocks, 256, 0, s>>>(hv, counts.p);
  SHCI_LAUNCH_CHECK();
  H.rowptr.resize(N + 1);
  int64_t total = 0;
  scan_exclusive_i64(counts.p, H.rowptr.p, N, &total, pr, s);
  k_set_last<<<1, 1, 0, s>>>(H.rowptr.p, (int64_t)N, total);
  SHCI_LAUNCH_CHECK();
  H.N = N;
  H.nnz = total;
  size_t cap = total > 0 ? (size_t)total : 1;
  H.col.resize(cap);
  if (want64) H.v64.resize(cap); else H.v64.release();
  if (want32) H.vhi.resize(cap); else H.vhi.release();
  if (want32 && want_lo) H.vlo.resize(cap); else H.vlo.release();
  k_ham_emit<<<blocks, 256, 0, s>>>(hv, dets, ints, H.rowptr.p, H.col.p, want64 ? H.v64.p : nullptr,
                                    want32 ? H.vhi.p : nullptr, (want32 && want_lo) ? H.vlo.p : nullptr);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// Diagonal energies: thread per determinant, Direct/Exchange in shared memory.
// ---------------------------------------------------------------------------
__global__ void k_diag(const Det2* __restrict__ dets, size_t n, IntsView ints, double* __restrict__ diag) {
  extern __shared__ double sm[];
  const int nn = ints.norb * ints.norb;
  double* sD = sm;
  double* sX = sm + nn;
  for (int j = threadIdx.x; j < nn; j += blockDim.x) {
    sD[j] = ints.Direct[j];
    sX[j] = ints.Exchange[j];
  }
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    diag[i] = det_energy(ints, dets[i], sD, sX);
}

void compute_diag(const Det2* dets, size_t n, const IntsView& ints, double* diag, cudaStream_t s) {
  if (n == 0) return;
  size_t smem = 2 * sizeof(double) * ints.norb * ints.norb;
  SHCI_CUDA(cudaFuncSetAttribute(k_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_diag<<<grid_for(n, 128, 152 * 8), 128, smem, s>>>(dets, n, ints, diag);
  SHCI_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Matrix-free sigma: y[I] = diag[I] x[I] + sum_J H_IJ x[J] with H_IJ
// recomputed for every connection. X and Y are row-interleaved [N][K].
// ---------------------------------------------------------------------------
template <int K>
struct DirectVisitor {
  const Det2* dets;
  IntsView ints;
  Det2 dI;
  uint32_t I;
  const double* x;
  double acc[K];
  __device__ void step(bool hit, uint32_t J, bool) {
    if (hit) {
      Det2 dJ = dets[J];
      double hv = (J < I) ? hij_any(ints, dJ, dI) : hij_any(ints, dI, dJ);
#pragma unroll
      for (int r = 0; r < K; ++r) acc[r] += hv * x[(size_t)J * K + r];
    }
  }
};

template <int K>
__global__ void k_sigma_direct(HelperView h, const Det2* __restrict__ dets, IntsView ints,
                               const double* __restrict__ diag, const double* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t I = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < (int64_t)h.N; I += warps) {
    DirectVisitor<K> v{dets, ints, dets[I], (uint32_t)I, x, {}};
#pragma unroll
    for (int r = 0; r < K; ++r) v.acc[r] = 0.0;
    visit_row(h, (uint32_t)I, v);
#pragma unroll
    for (int r = 0; r < K; ++r) {
      double a = v.acc[r];
#pragma unroll
      for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
      if (lane == 0) y[(size_t)I * K + r] = diag[I] * x[(size_t)I * K + r] + a;
    }
  }
}

void sigma_direct(const Helpers& hp, const Det2* dets, const IntsView& ints, const double* diag, const double* x,
                  double* y, int k, cudaStream_t s) {
  HelperView hv = hp.view();
  const unsigned blocks = grid_for(hp.N * 32, 256, 152 * 16);
  switch (k) {
    case 1: k_sigma_direct<1><<<blocks, 256, 0, s>>>(hv, dets, ints, diag, x, y); break;
    case 2: k_sigma_direct<2><<<blocks, 256, 0, s>>>(hv, dets, ints, diag, x, y); break;
    case 4: k_sigma_direct<4><<<blocks, 256, 0, s>>>(hv, dets, ints, diag, x, y); break;
    default: throw Error(kErrInvalid, "direct sigma supports k in {1,2,4}");
  }
  SHCI_LAUNCH_CHECK();
}

}  // namespace shci
