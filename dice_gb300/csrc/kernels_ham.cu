// Hamiltonian-side kernels of the variational loop:
//   * alpha/beta string tables and single-excitation neighbour lists
//     (replaces HamHelpers2::PopulateHelpers, SHCI/SHCImakeHamiltonian.cpp:184-408);
//   * the diagonal energies (Determinant::Energy at SHCI/SHCIbasics.cpp:1145-1154);
//   * the two-pass count/emit build of the sparse Hamiltonian as full-row CSR
//     (replaces MakeHfromSMHelpers2, SHCI/SHCImakeHamiltonian.cpp:486-715);
//   * the matrix-free sigma (replaces HmultDirect::operator(), SHCI/Hmult.h:241-381).
//
// One warp owns one row I = (A, B). The connected determinants J are found in
// three parts:
//   1. determinants sharing I's alpha string: beta distance 1 or 2 (scan of
//      the alpha group);
//   2. determinants whose alpha string As is a single excitation of A and
//      whose beta string equals B or is one excitation away. Every such J
//      contains the partial string B - b for some occupied b of B, so it is
//      found by looking up the keys (As, B - b) in the partial-string index
//      (a hash table per alpha group As gives each key's run of entries):
//      |B| probes per group As that return (nearly) only connections,
//      instead of a scan over every determinant of the group -- except for
//      groups of at most a few times |B| determinants, which are scanned;
//   3. determinants sharing I's beta string: alpha distance 2 (scan of the
//      beta group).
// This visits the same (I, J) set as the reference's five helper-list classes
// (single alpha, alpha-beta, single beta, double beta, double alpha).
#include <algorithm>
#include <type_traits>

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

// Partial-string index entries, sorted by (alpha group, partial beta string):
// the entries of one key are one run and the runs of one alpha group are
// contiguous, and so are the slots of the group's hash table, so the probes
// of rows of the same alpha string touch the same small regions.
constexpr uint32_t kM1GroupBits = 26;

__global__ void k_m1_count(const uint64_t* __restrict__ bstr, size_t n, int64_t* __restrict__ cnt) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    cnt[i] = __popcll(bstr[i]);
}
__global__ void k_m1_fill(const uint64_t* __restrict__ bstr, const uint32_t* __restrict__ aidx, size_t n,
                          const int64_t* __restrict__ off, uint64_t* __restrict__ key, uint32_t* __restrict__ perm,
                          uint4* __restrict__ ent) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint64_t B = bstr[i];
    const uint32_t g = aidx[i];
    int64_t q = off[i];
    for (uint64_t r = B; r; r &= r - 1) {
      const int b = __ffsll((long long)r) - 1;
      const uint64_t bm = B ^ (1ull << b);
      key[q] = bm;
      perm[q] = (uint32_t)q;
      ent[q] = make_uint4((uint32_t)bm, (uint32_t)(bm >> 32), g | ((uint32_t)b << kM1GroupBits), (uint32_t)i);
      ++q;
    }
  }
}
__global__ void k_m1_group_keys(const uint4* __restrict__ ent, const uint32_t* __restrict__ perm, int64_t n,
                                uint64_t* __restrict__ gk) {
  const uint32_t mask = (1u << kM1GroupBits) - 1u;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    gk[k] = ent[perm[k]].z & mask;
}
__global__ void k_m1_permute(const uint4* __restrict__ src, const uint32_t* __restrict__ perm, int64_t n,
                             uint4* __restrict__ dst) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    dst[k] = src[perm[k]];
}
// Per-group hash tables over the index's distinct keys. Entry k starts a run
// when its key (alpha group, partial string) differs from entry k-1's.
__device__ __forceinline__ bool m1_same_key(const uint4& a, const uint4& b) {
  constexpr uint32_t gmask = (1u << kM1GroupBits) - 1u;
  return a.x == b.x && a.y == b.y && ((a.z ^ b.z) & gmask) == 0;
}
// Fibonacci hashing: the top lg bits of the partial string times 2^64 / phi
// pick the slot; 26 bits of a second product are the slot's fingerprint
__device__ __forceinline__ uint64_t m1_slot(uint64_t bm, unsigned lg) {
  return (bm * 0x9e3779b97f4a7c15ull) >> (64u - lg);
}
__device__ __forceinline__ uint32_t m1_fingerprint(uint64_t bm) {
  return (uint32_t)((bm * 0xc2b2ae3d27d4eb4full) >> 38);
}
constexpr uint32_t kM1Empty = 0xffffffffu;
__global__ void k_m1_heads(const uint4* __restrict__ ent, int64_t n, uint32_t* __restrict__ keys_of_group) {
  constexpr uint32_t gmask = (1u << kM1GroupBits) - 1u;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const uint4 e = ent[k];
    if (k == 0 || !m1_same_key(e, ent[k - 1])) atomicAdd(keys_of_group + (e.z & gmask), 1u);
  }
}
// slots of group g: the power of two >= 2 x its distinct keys, at least 2
__global__ void k_m1_slots(const uint32_t* __restrict__ keys_of_group, int64_t ng, int64_t* __restrict__ slots) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += (int64_t)gridDim.x * blockDim.x) {
    int64_t t = 2;
    while (t < 2 * (int64_t)keys_of_group[g]) t <<= 1;
    slots[g] = t;
  }
}
__global__ void k_m1_dir(const int64_t* __restrict__ slots, const int64_t* __restrict__ first, int64_t ng,
                         uint64_t* __restrict__ dir) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += (int64_t)gridDim.x * blockDim.x)
    dir[g] = ((uint64_t)first[g] << 6) | (uint64_t)(63 - __clzll((long long)slots[g]));
}
// One thread per run: measure the run (at most 64 entries: one per beta
// orbital outside the partial string) and claim a slot of its group's table
// by linear probing; a table more than half empty always has a free slot.
__global__ void k_m1_insert(const uint4* __restrict__ ent, int64_t n, const uint64_t* __restrict__ dir,
                            uint2* __restrict__ tab) {
  constexpr uint32_t gmask = (1u << kM1GroupBits) - 1u;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const uint4 e = ent[k];
    if (k > 0 && m1_same_key(e, ent[k - 1])) continue;
    int64_t f = k + 1;
    while (f < n && m1_same_key(ent[f], e)) ++f;
    const uint64_t d = dir[e.z & gmask];
    const unsigned lg = (unsigned)(d & 63);
    const uint64_t mask = (1ull << lg) - 1;
    uint2* t = tab + (d >> 6);
    const uint64_t bm = ((uint64_t)e.y << 32) | e.x;
    uint64_t q = m1_slot(bm, lg);
    for (uint64_t step = 0; step <= mask; ++step) {
      if (atomicCAS(&t[q].x, kM1Empty, (uint32_t)k) == kM1Empty) {
        t[q].y = ((uint32_t)(f - k - 1) << kM1GroupBits) | m1_fingerprint(bm);
        break;
      }
      q = (q + 1) & mask;
    }
  }
}

// Orders each alpha group's single-excitation list: groups A_s of at most
// kScanFactor x n_beta determinants first (cheaper to scan, one coalesced
// load and popcount per determinant, than to probe the index n_beta times),
// then the rest, each part in its original order; mid[g] is where the large
// groups start. One thread per group. mol36 (498,028 determinants), FP64
// 4-vector matrix-free sigma: 60.7 ms probing every group, 49.7 / 48.8 / 47.5 /
// 47.7 ms with factors 2 / 3 / 4 / 6.
#ifndef SHCI_SCAN_FACTOR
#define SHCI_SCAN_FACTOR 4
#endif
constexpr int kScanFactor = SHCI_SCAN_FACTOR;
__global__ void k_split_singles(const int64_t* __restrict__ sstart, const uint32_t* __restrict__ in,
                                const int64_t* __restrict__ gstart, const uint64_t* __restrict__ gbeta, int64_t na,
                                uint32_t* __restrict__ out, int64_t* __restrict__ mid) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < na; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s0 = sstart[g], s1 = sstart[g + 1];
    const int64_t cap = (int64_t)kScanFactor * __popcll(gbeta[gstart[g]]);
    int64_t w = s0;
    for (int64_t q = s0; q < s1; ++q) {
      const uint32_t As = in[q];
      if (gstart[As + 1] - gstart[As] <= cap) out[w++] = As;
    }
    mid[g] = w;
    for (int64_t q = s0; q < s1; ++q) {
      const uint32_t As = in[q];
      if (gstart[As + 1] - gstart[As] > cap) out[w++] = As;
    }
  }
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
  {
    DevBuf<uint32_t> split;
    split.resize(total > 0 ? total : 1);
    aSingMid.resize(NA);
    k_split_singles<<<grid_for((size_t)NA, 256), 256, 0, s>>>(aSingStart.p, aSing.p, aStart.p, aGroupB.p, NA, split.p,
                                                              aSingMid.p);
    SHCI_LAUNCH_CHECK();
    aSing.swap(split);
  }
  // partial-string index (one entry per determinant and occupied beta orbital)
  {
    DevBuf<int64_t> c1, o1;
    c1.resize(n);
    o1.resize(n + 1);
    k_m1_count<<<grid_for(n, 256), 256, 0, s>>>(bstr.p, n, c1.p);
    SHCI_LAUNCH_CHECK();
    int64_t ne = 0;
    scan_exclusive_i64(c1.p, o1.p, n, &ne, pr, s);
    if (ne >= ((int64_t)1 << 32)) throw Error(kErrInvalid, "partial-string index too large");
    if (NA >= ((int64_t)1 << kM1GroupBits)) throw Error(kErrInvalid, "too many alpha strings for the partial-string index");
    nm1 = ne;
    if (ne > 0) {
      DevBuf<uint64_t> key;
      DevBuf<uint32_t> perm;
      DevBuf<uint4> raw;
      key.resize(ne);
      perm.resize(ne);
      raw.resize(ne);
      m1ent.resize(ne);
      const unsigned eb = grid_for((size_t)ne, 256);
      k_m1_fill<<<grid_for(n, 256), 256, 0, s>>>(bstr.p, aidx.p, n, o1.p, key.p, perm.p, raw.p);
      SHCI_LAUNCH_CHECK();
      sort_u64(key.p, perm.p, (size_t)ne, pr, s);  // by partial string
      k_m1_group_keys<<<eb, 256, 0, s>>>(raw.p, perm.p, ne, key.p);
      SHCI_LAUNCH_CHECK();
      sort_u64(key.p, perm.p, (size_t)ne, pr, s);  // then by alpha group (stable)
      k_m1_permute<<<eb, 256, 0, s>>>(raw.p, perm.p, ne, m1ent.p);
      SHCI_LAUNCH_CHECK();
      // the groups' hash tables
      DevBuf<uint32_t> nkey;
      DevBuf<int64_t> slots, first;
      nkey.resize((size_t)NA);
      slots.resize((size_t)NA);
      first.resize((size_t)NA + 1);
      SHCI_CUDA(cudaMemsetAsync(nkey.p, 0, (size_t)NA * sizeof(uint32_t), s));
      k_m1_heads<<<eb, 256, 0, s>>>(m1ent.p, ne, nkey.p);
      SHCI_LAUNCH_CHECK();
      k_m1_slots<<<grid_for((size_t)NA, 256), 256, 0, s>>>(nkey.p, NA, slots.p);
      SHCI_LAUNCH_CHECK();
      int64_t nslot = 0;
      scan_exclusive_i64(slots.p, first.p, NA, &nslot, pr, s);
      m1dir.resize((size_t)NA);
      k_m1_dir<<<grid_for((size_t)NA, 256), 256, 0, s>>>(slots.p, first.p, NA, m1dir.p);
      SHCI_LAUNCH_CHECK();
      m1tab.resize((size_t)nslot);
      SHCI_CUDA(cudaMemsetAsync(m1tab.p, 0xff, (size_t)nslot * sizeof(uint2), s));
      k_m1_insert<<<eb, 256, 0, s>>>(m1ent.p, ne, m1dir.p, m1tab.p);
      SHCI_LAUNCH_CHECK();
    }
  }
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
  // 2. alpha single excitation: beta equal (single alpha) or beta single
  // (alpha-beta double). I's list of groups A_s holds the small groups first
  // (at most a few times |B| determinants: scanned, one popcount each), then
  // the large ones (found from the partial-string index, |B| probes each).
  {
    const int64_t s0 = h.aSingStart[ia], s1 = h.aSingStart[ia + 1];
    const bool indexed = h.m1ent != nullptr && B != 0;
    const int64_t smid = indexed ? h.aSingMid[ia] : s1;
    // the small groups (every group without the index)
    for (int64_t base = s0; base < smid; base += 32) {
      int64_t q = base + lane;
      int64_t g0 = 0, len = 0;
      if (q < smid) {
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
    if (indexed && smid < s1) {
      const int nb = __popcll(B);
      const int64_t nprobe = (s1 - smid) * nb;
      // Probe t = (excitation sidx, occupied beta orbital `which`): each lane
      // keeps its pair and steps it by 32 probes a round (no division per
      // probe), and lane k holds the k-th occupied beta orbital of B for the
      // others to read (B's orbitals beyond the 32nd, possible only past 32 beta
      // electrons, are found bit by bit)
      int occ_k = 0;
      {
        uint64_t r = B;
        for (int k = 0; k < lane && r; ++k) r &= r - 1;
        occ_k = r ? __ffsll((long long)r) - 1 : 0;
      }
      const int step_q = 32 / nb, step_r = 32 % nb;
      int64_t sidx = lane / nb;
      int which = lane % nb;
      for (int64_t base = 0; base < nprobe; base += 32) {
        const int64_t t = base + lane;
        // each lane locates the entries of its key (As, B - b)
        uint32_t lo = 0;
        int len = 0;  // at most 64: one entry per beta orbital outside the key
        int bq = __shfl_sync(kFull, occ_k, which & 31);  // the beta orbital removed by this probe
        if (which >= 32) {
          uint64_t r = B;
          for (int k = 0; k < which; ++k) r &= r - 1;
          bq = __ffsll((long long)r) - 1;
        }
        const int64_t my_s = sidx;
        const bool first_b = which == 0;
        which += step_r;
        sidx += step_q;
        if (which >= nb) {
          which -= nb;
          ++sidx;
        }
        if (t < nprobe) {
          const uint32_t As = h.aSing[smid + my_s];
          const uint64_t Bm = B ^ (1ull << bq);
          // the slot of Bm in group As's table gives the key's run of entries
          // (a fingerprint match is confirmed on the run's first entry, the
          // entry the flattening below reads first); an empty slot means no
          // determinant of the space has the key
          const uint64_t d = h.m1dir[As];
          const unsigned lg = (unsigned)(d & 63);
          const uint64_t mask = (1ull << lg) - 1;
          const uint2* tab = h.m1tab + (d >> 6);
          const uint32_t fp = m1_fingerprint(Bm);
          uint64_t q = m1_slot(Bm, lg);
          for (uint64_t step = 0; step <= mask; ++step) {
            const uint2 sl = tab[q];
            if (sl.x == kM1Empty) break;
            if ((sl.y & ((1u << kM1GroupBits) - 1u)) == fp) {
              const uint2 k0 = *reinterpret_cast<const uint2*>(h.m1ent + sl.x);
              if (k0.x == (uint32_t)Bm && k0.y == (uint32_t)(Bm >> 32)) {
                lo = sl.x;
                len = (sl.y >> kM1GroupBits) + 1;
                break;
              }
            }
            q = (q + 1) & mask;
          }
        }
        // flatten the lanes' matches and verify them 32 at a time
        int incl = len;
  #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(kFull, incl, o);
          if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        const int excl = incl - len;
        for (int f0 = 0; f0 < total; f0 += 32) {
          const int f = f0 + lane;
          int src = 0;
  #pragma unroll
          for (int st = 16; st >= 1; st >>= 1) {
            const int c = src + st;
            const int e = __shfl_sync(kFull, excl, c < 32 ? c : 31);
            if (c < 32 && e <= f) src = c;
          }
          const uint32_t elo = __shfl_sync(kFull, lo, src);
          const int eo = __shfl_sync(kFull, excl, src);
          const int wb = __shfl_sync(kFull, bq, src);
          const bool fb = __shfl_sync(kFull, first_b, src);
          bool hit = false, single = false;
          uint32_t J = 0;
          if (f < total) {
            // the entry holds J and the orbital b' its beta string has beyond
            // B - b: b' == b means beta equal (found once per occupied b, kept
            // for the first), otherwise a beta single excitation b -> b'
            const uint4 en = h.m1ent[(size_t)elo + (uint32_t)(f - eo)];
            J = en.w;
            single = (int)(en.z >> kM1GroupBits) == wb;
            hit = single ? fb : true;
          }
          v.step(hit, J, single);
        }
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

// Rows [row0, row0 + nr); counts[slot(I)] = number of off-diagonal
// connections, where slot(I) = slot[I] when a slot map is given (the storage
// position of a full build, the local row of a row block), else I - row0.
// order[k], k < nr: those rows in alpha-major order (rows of one
// alpha string probe the same index sections; run together, they share them
// in cache). Output positions stay indexed by the row.
__global__ void k_ham_count(HelperView h, int64_t row0, int64_t nr, const uint32_t* __restrict__ order,
                            const uint32_t* __restrict__ slot, int64_t* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nr; k += warps) {
    const int64_t I = order[k];
    CountVisitor v;
    visit_row(h, (uint32_t)I, v);
    int64_t c = v.c;
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
    if (lane == 0) counts[slot ? (int64_t)slot[I] : I - row0] = c;
  }
}

// H_IJ with the higher-index determinant as the ket, the element the
// reference stores in row max(I,J) (SHCI/SHCImakeHamiltonian.cpp:565-580).
// Kept out of line, taking and returning plain values: the visitors' step()
// is inlined at every scan site of visit_row, and the Slater-Condon code
// copied into each caused instruction-cache misses, while an out-of-line
// member taking the visitor by address kept the visitor's state (queue
// counts, accumulators, output position) in local memory.
__device__ __noinline__ double ham_element(const double* I1, const double* I2, const double* V1, int norb, Det2 dI,
                                           Det2 dJ, bool j_below) {
  const IntsView iv{I1, I2, nullptr, nullptr, norb, nullptr, nullptr, V1, nullptr};
  return j_below ? hij_any(iv, dJ, dI) : hij_any(iv, dI, dJ);
}
__device__ __noinline__ float ham_element_f32(const float* I1f, const float* I2f, const float* V1f, int norb,
                                              Det2 dI, Det2 dJ, bool j_below) {
  const IntsView iv{nullptr, nullptr, nullptr, nullptr, norb, I1f, I2f, nullptr, V1f};
  return j_below ? hij_any_f32(iv, dJ, dI) : hij_any_f32(iv, dI, dJ);
}

// Emits (col, value) for one row (elements from ham_element).
//
// Connections found by the scans are queued per warp in shared memory, one
// queue for single and one for double excitations; whenever a queue holds 32
// entries all lanes evaluate one Slater-Condon element each, so the FP64 work
// runs on full warps and singles (an O(n_elec) sum) do not wait on doubles.
struct EmitVisitor {
  const Det2* dets;
  const uint32_t* cmap;  // determinant index -> storage column
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
    const double hv = ham_element(ints.I1, ints.I2, ints.V1, ints.norb, dI, dets[J], J < I);
    col[q] = (int32_t)cmap[J];
    if (v64) v64[q] = hv;
    if (vhi) {
      const float hi = (float)hv;
      vhi[q] = hi;
      if (vlo) vlo[q] = (float)(hv - (double)hi);
    }
  }
  // evaluate the first `cnt` (<= 32) entries of queue q, then shift the rest
  // down
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

// Rows [row0, row0 + nr) into a CSR whose row pointers are indexed by slot(I)
// (see k_ham_count); columns are storage positions cmap[J].
// Resident blocks per SM the emit and the matrix-free sigma are compiled for.
// Both wait on the latency of index probes and gathers. The emit runs best
// with 6 (at most 40 registers a thread, a few hundred bytes of spills: mol24
// H build 0.98 s, 1.02 s with 4 blocks); the matrix-free sigma, whose
// accumulators stay in registers, with 4 (64 registers, almost no spills:
// mol36, 4 vectors, FP32 64 ms against 70 ms with 6).
#ifndef SHCI_EMIT_MIN_BLOCKS
#define SHCI_EMIT_MIN_BLOCKS 6
#endif
#ifndef SHCI_DIRECT_MIN_BLOCKS
#define SHCI_DIRECT_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(256, SHCI_EMIT_MIN_BLOCKS) k_ham_emit(HelperView h, int64_t row0, int64_t nr,
                                                     const uint32_t* __restrict__ order,
                                                     const uint32_t* __restrict__ slot,
                                                     const uint32_t* __restrict__ cmap,
                                                     const Det2* __restrict__ dets, IntsView ints,
                                                     const int64_t* __restrict__ rowptr, int32_t* __restrict__ col,
                                                     double* __restrict__ v64, float* __restrict__ vhi,
                                                     float* __restrict__ vlo) {
  __shared__ uint32_t s_q[8][2][64];
  const int wib = threadIdx.x >> 5;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nr; k += warps) {
    const int64_t I = order[k];
    EmitVisitor v{dets, cmap, ints, dets[I], (uint32_t)I, rowptr[slot ? (int64_t)slot[I] : I - row0], col, v64, vhi,
                  vlo, s_q[wib][0], s_q[wib][1], 0, 0};
    visit_row(h, (uint32_t)I, v);
    v.flush();
  }
}

__global__ void k_set_last(int64_t* rowptr, int64_t n, int64_t total) { rowptr[n] = total; }

// Sort of one row by column, one block per row. The row's columns become
// 64-bit keys (column << 12 | position in the row) sorted by a bitonic network
// in which each of the 256 threads keeps E consecutive keys in registers: the
// compare-exchange steps between keys of one thread run in registers, only
// the longer-distance steps go through shared memory (36 of the 66 steps for
// a 2048-key row). The values are then gathered from their old positions
// (read into registers before any write, the row is sorted in place). Rows
// longer than kRowSortCap are left in emission order (still correct, only
// with less gather locality in sigma).
constexpr int kRowSortCap = 4096;
constexpr int kSortThreads = 256;

template <int E>
__device__ __forceinline__ void sort_exchange_regs(uint64_t (&v)[E], int g0, int k) {
  // the steps of merge size k with partner distance j < E: partner in the same thread
#pragma unroll
  for (int j = E >> 1; j > 0; j >>= 1) {
    if (j >= k) continue;  // merges smaller than E start at j = k / 2
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int pe = e ^ j;
      if (pe > e) {
        const bool up = ((g0 + e) & k) == 0;
        const uint64_t x = v[e], y = v[pe];
        if ((x > y) == up) {
          v[e] = y;
          v[pe] = x;
        }
      }
    }
  }
}

template <int E>
__device__ void sort_row_keys(uint64_t* sk, int P) {
  // threads [0, P/E) own keys [t*E, t*E+E); others only join the barriers
  const int T = P / E;
  const int t = threadIdx.x;
  const bool act = t < T;
  const int g0 = t * E;
  uint64_t v[E];
  for (int k = 2; k <= P; k <<= 1) {
    // distances j >= E: pairs in shared memory
    for (int j = k >> 1; j >= E; j >>= 1) {
      for (int q = t; q < P / 2; q += blockDim.x) {
        const int lo = ((q & ~(j - 1)) << 1) | (q & (j - 1));  // lower index of the q-th pair (j a power of two)
        const int hi = lo + j;
        const bool up = (lo & k) == 0;
        const uint64_t x = sk[lo], y = sk[hi];
        if ((x > y) == up) {
          sk[lo] = y;
          sk[hi] = x;
        }
      }
      __syncthreads();
    }
    // distances j < E: in registers
    if (E > 1) {
      if (act) {
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = sk[g0 + e];
        sort_exchange_regs<E>(v, g0, k);
#pragma unroll
        for (int e = 0; e < E; ++e) sk[g0 + e] = v[e];
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(kSortThreads) k_row_sort(const int64_t* __restrict__ rowptr, size_t N,
                                                           int32_t* __restrict__ col, double* __restrict__ v64,
                                                           float* __restrict__ vhi, float* __restrict__ vlo) {
  __shared__ uint64_t sk[kRowSortCap];
  constexpr int kPer = kRowSortCap / kSortThreads;  // values gathered per thread
  for (size_t r = blockIdx.x; r < N; r += gridDim.x) {
    const int64_t p0 = rowptr[r], len = rowptr[r + 1] - p0;
    if (len <= 1 || len > kRowSortCap) continue;  // uniform across the block
    int P = 2;
    while (P < len) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x)
      sk[i] = i < len ? ((uint64_t)(uint32_t)col[p0 + i] << 12) | (uint64_t)i : ~0ull;
    __syncthreads();
    if (P >= 16 * kSortThreads)
      sort_row_keys<16>(sk, P);
    else if (P >= 8 * kSortThreads)
      sort_row_keys<8>(sk, P);
    else if (P >= 4 * kSortThreads)
      sort_row_keys<4>(sk, P);
    else if (P >= 2 * kSortThreads)
      sort_row_keys<2>(sk, P);
    else
      sort_row_keys<1>(sk, P);
    // gather the values of this thread's output positions, then write
    uint64_t pay[kPer];
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
      const int i = threadIdx.x + m * kSortThreads;
      pay[m] = 0;
      if (i < len) {
        const int src = (int)(sk[i] & 0xFFFull);
        if (v64) {
          pay[m] = (uint64_t)__double_as_longlong(v64[p0 + src]);
        } else {
          pay[m] = (uint64_t)__float_as_uint(vhi[p0 + src]);
          if (vlo) pay[m] |= (uint64_t)__float_as_uint(vlo[p0 + src]) << 32;
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
      const int i = threadIdx.x + m * kSortThreads;
      if (i < len) {
        col[p0 + i] = (int32_t)(sk[i] >> 12);
        if (v64) {
          v64[p0 + i] = __longlong_as_double((long long)pay[m]);
        } else {
          vhi[p0 + i] = __uint_as_float((uint32_t)pay[m]);
          if (vlo) vlo[p0 + i] = __uint_as_float((uint32_t)(pay[m] >> 32));
        }
      }
    }
    __syncthreads();
  }
}

// Value arrays of a CSR as raw pointers.
struct CsrVals {
  int32_t* col;
  double* v64;
  float* vhi;
  float* vlo;
};

// Rows longer than kRowSortCap: one 1024-thread block per row runs the
// bitonic network on 64-bit keys (column << 32 | position) in a global
// scratch segment (L2-resident), then the values are permuted through a second
// scratch segment. Every row then leaves the build sorted, so the order of a
// row's entries (and of sigma's sums over it) does not depend on the atomic
// order in which the incremental build placed its new columns.
__global__ void k_long_rows(const int64_t* __restrict__ rowptr, size_t N, int cap, uint32_t* __restrict__ list,
                            unsigned long long* __restrict__ count) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x)
    if (rowptr[r + 1] - rowptr[r] > cap) list[atomicAdd(count, 1ull)] = (uint32_t)r;
}
__global__ void __launch_bounds__(1024) k_long_row_sort(const int64_t* __restrict__ rowptr,
                                                        const uint32_t* __restrict__ rows,
                                                        const int64_t* __restrict__ soff, uint64_t* __restrict__ key,
                                                        uint64_t* __restrict__ pay, CsrVals v) {
  const size_t r = rows[blockIdx.x];
  const int64_t p0 = rowptr[r], len = rowptr[r + 1] - p0;
  uint64_t* k = key + soff[blockIdx.x];
  uint64_t* y = pay + soff[blockIdx.x];
  int64_t P = 2;
  while (P < len) P <<= 1;
  for (int64_t i = threadIdx.x; i < P; i += blockDim.x)
    k[i] = i < len ? ((uint64_t)(uint32_t)v.col[p0 + i] << 32) | (uint64_t)i : ~0ull;
  __syncthreads();
  for (int64_t kk = 2; kk <= P; kk <<= 1)
    for (int64_t j = kk >> 1; j > 0; j >>= 1) {
      for (int64_t q = threadIdx.x; q < P / 2; q += blockDim.x) {
        const int64_t lo = ((q & ~(j - 1)) << 1) | (q & (j - 1)), hi = lo + j;  // j a power of two
        const bool up = (lo & kk) == 0;
        const uint64_t a = k[lo], b = k[hi];
        if ((a > b) == up) {
          k[lo] = b;
          k[hi] = a;
        }
      }
      __syncthreads();
    }
  // permute the values through y, then write columns and values back
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
    const int64_t src = (int64_t)(k[i] & 0xFFFFFFFFull);
    uint64_t val;
    if (v.v64) {
      val = (uint64_t)__double_as_longlong(v.v64[p0 + src]);
    } else {
      val = (uint64_t)__float_as_uint(v.vhi[p0 + src]);
      if (v.vlo) val |= (uint64_t)__float_as_uint(v.vlo[p0 + src]) << 32;
    }
    y[i] = val;
  }
  __syncthreads();
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
    v.col[p0 + i] = (int32_t)(k[i] >> 32);
    const uint64_t val = y[i];
    if (v.v64) {
      v.v64[p0 + i] = __longlong_as_double((long long)val);
    } else {
      v.vhi[p0 + i] = __uint_as_float((uint32_t)val);
      if (v.vlo) v.vlo[p0 + i] = __uint_as_float((uint32_t)(val >> 32));
    }
  }
}

__global__ void k_list_lens(const int64_t* __restrict__ rowptr, const uint32_t* __restrict__ rows, size_t n,
                            int64_t* __restrict__ len) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    len[i] = rowptr[rows[i] + 1] - rowptr[rows[i]];
}

static void sort_rows(const int64_t* rowptr, size_t n, const CsrVals& v, cudaStream_t s) {
  if (n == 0) return;
  const unsigned sblocks = (unsigned)std::min<size_t>(n, 152 * 6);
  k_row_sort<<<sblocks, kSortThreads, 0, s>>>(rowptr, n, v.col, v.v64, v.vhi, v.vlo);
  SHCI_LAUNCH_CHECK();
  // rows past the shared-memory cap
  DevBuf<unsigned long long> cnt;
  cnt.resize(1);
  SHCI_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), s));
  DevBuf<uint32_t> list;
  list.resize(n);
  k_long_rows<<<grid_for(n, 256), 256, 0, s>>>(rowptr, n, kRowSortCap, list.p, cnt.p);
  SHCI_LAUNCH_CHECK();
  unsigned long long nl = 0;
  SHCI_CUDA(cudaMemcpyAsync(&nl, cnt.p, sizeof(nl), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  if (nl == 0) return;
  DevBuf<int64_t> lens;
  lens.resize(nl);
  k_list_lens<<<grid_for(nl, 256), 256, 0, s>>>(rowptr, list.p, nl, lens.p);
  SHCI_LAUNCH_CHECK();
  std::vector<int64_t> hl(nl);
  SHCI_CUDA(cudaMemcpyAsync(hl.data(), lens.p, nl * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  std::vector<int64_t> off(nl);
  int64_t tot = 0;
  for (unsigned long long i = 0; i < nl; ++i) {
    int64_t P = 2;
    while (P < hl[i]) P <<= 1;
    off[i] = tot;
    tot += P;
  }
  DevBuf<int64_t> doff;
  doff.resize(nl);
  SHCI_CUDA(cudaMemcpyAsync(doff.p, off.data(), nl * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  DevBuf<uint64_t> key, pay;
  key.resize(tot);
  pay.resize(tot);
  k_long_row_sort<<<(unsigned)nl, 1024, 0, s>>>(rowptr, list.p, doff.p, key.p, pay.p, v);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));  // the scratch is freed on return
}

// Count, emit and sort the full rows [row0, N) into (rowptr, vals); returns nnz.
__global__ void k_order_keys(const uint32_t* __restrict__ aidx, int64_t row0, int64_t nr, uint64_t* __restrict__ key,
                             uint32_t* __restrict__ val) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nr; k += (int64_t)gridDim.x * blockDim.x) {
    key[k] = aidx[row0 + k];
    val[k] = (uint32_t)(row0 + k);
  }
}

// Rows [row0, row1) of the determinant array. slot: storage position of each
// row (full build), local row of a row block, or null (rows at I - row0);
// cmap: determinant index -> storage column.
static int64_t emit_rows(const Helpers& hp, size_t row0, size_t row1, const uint32_t* slot, const uint32_t* cmap,
                         const Det2* dets, const IntsView& ints, DevBuf<int64_t>& rowptr, DevBuf<int32_t>& col,
                         DevBuf<double>& v64, DevBuf<float>& vhi, DevBuf<float>& vlo, bool want64, bool want32,
                         bool want_lo, Prims& pr, cudaStream_t s, PhaseTimer& pt) {
  const size_t nr = row1 - row0;
  HelperView hv = hp.view();
  DevBuf<int64_t> counts;
  counts.resize(nr > 0 ? nr : 1);
  // the new rows in alpha-major order (stable: by row within an alpha string)
  DevBuf<uint32_t> order;
  order.resize(nr > 0 ? nr : 1);
  if (nr) {
    DevBuf<uint64_t> okey;
    okey.resize(nr);
    k_order_keys<<<grid_for(nr, 256), 256, 0, s>>>(hp.aidx.p, (int64_t)row0, (int64_t)nr, okey.p, order.p);
    SHCI_LAUNCH_CHECK();
    sort_u64(okey.p, order.p, nr, pr, s);
  }
  const unsigned blocks = grid_for(nr * 32, 256, 152 * 16);
  if (nr) {
    k_ham_count<<<blocks, 256, 0, s>>>(hv, (int64_t)row0, (int64_t)nr, order.p, slot, counts.p);
    SHCI_LAUNCH_CHECK();
  }
  pt.mark("ham count");
  rowptr.resize(nr + 1);
  int64_t total = 0;
  scan_exclusive_i64(counts.p, rowptr.p, nr, &total, pr, s);
  k_set_last<<<1, 1, 0, s>>>(rowptr.p, (int64_t)nr, total);
  SHCI_LAUNCH_CHECK();
  const size_t cap = total > 0 ? (size_t)total : 1;
  col.resize(cap);
  if (want64) v64.resize(cap); else v64.release();
  if (want32) vhi.resize(cap); else vhi.release();
  if (want32 && want_lo) vlo.resize(cap); else vlo.release();
  CsrVals v{col.p, want64 ? v64.p : nullptr, want32 ? vhi.p : nullptr, (want32 && want_lo) ? vlo.p : nullptr};
  if (nr) {
    k_ham_emit<<<blocks, 256, 0, s>>>(hv, (int64_t)row0, (int64_t)nr, order.p, slot, cmap, dets, ints, rowptr.p,
                                      v.col, v.v64,
                                      v.vhi, v.vlo);
    SHCI_LAUNCH_CHECK();
  }
  pt.mark("ham emit");
  // sort every row by column so that the 32 gathers of one warp instruction in
  // sigma fall on fewer 32-byte sectors of x
  sort_rows(rowptr.p, nr, v, s);
  pt.mark("ham row sort");
  return total;
}

// Storage order: the determinants sorted by (alpha string, beta string);
// perm[i] = determinant at storage position i, spos = its inverse.
__global__ void k_storage_keys(const uint64_t* __restrict__ astr, const uint64_t* __restrict__ bstr, size_t n,
                               uint64_t* __restrict__ k0, uint64_t* __restrict__ k1, uint32_t* __restrict__ v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    k0[i] = bstr[i];
    k1[i] = astr[i];
    v[i] = (uint32_t)i;
  }
}
__global__ void k_invert(const uint32_t* __restrict__ perm, size_t n, uint32_t* __restrict__ inv) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    inv[perm[i]] = (uint32_t)i;
}
static void storage_order(const Helpers& hp, DevBuf<uint32_t>& perm, DevBuf<uint32_t>& spos, Prims& pr,
                          cudaStream_t s) {
  const size_t n = hp.N;
  perm.resize(n > 0 ? n : 1);
  spos.resize(n > 0 ? n : 1);
  if (n == 0) return;
  DevBuf<uint64_t> k0, k1;
  k0.resize(n);
  k1.resize(n);
  k_storage_keys<<<grid_for(n, 256), 256, 0, s>>>(hp.astr.p, hp.bstr.p, n, k0.p, k1.p, perm.p);
  SHCI_LAUNCH_CHECK();
  sort_u128(k0.p, k1.p, perm.p, n, pr, s);
  k_invert<<<grid_for(n, 256), 256, 0, s>>>(perm.p, n, spos.p);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));  // k0, k1 are freed on return
}

// Incremental build helpers. The rows of the new determinants R >= n_old are
// emitted in full (row R at R - n_old, columns in the new storage order);
// their entries whose column is an old determinant C < n_old are the new
// columns of old row C (same value: H_CR is evaluated with R, the higher
// index, as the ket in both places).
// Bit x of `old` = storage position x holds an old determinant (index < n_old).
__global__ void k_old_bits(const uint32_t* __restrict__ perm, int64_t N, int64_t n_old, uint32_t* __restrict__ old) {
  const int64_t nw = (N + 31) >> 5;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = 0;
    for (int b = 0; b < 32 && (w << 5) + b < N; ++b) m |= ((int64_t)perm[(w << 5) + b] < n_old ? 1u : 0u) << b;
    old[w] = m;
  }
}
__device__ __forceinline__ bool is_old(const uint32_t* __restrict__ old, uint32_t x) {
  return (__ldg(old + (x >> 5)) >> (x & 31)) & 1u;
}
// New columns of the old rows, indexed by the old row's new storage position
// (the new rows' columns are storage positions already).
__global__ void k_delta_count(const int64_t* __restrict__ rp_new, size_t nr, const int32_t* __restrict__ col_new,
                              const uint32_t* __restrict__ old, unsigned long long* __restrict__ dcnt) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < (int64_t)nr; r += warps)
    for (int64_t p = rp_new[r] + lane; p < rp_new[r + 1]; p += 32) {
      const uint32_t c = (uint32_t)col_new[p];
      if (is_old(old, c)) atomicAdd(&dcnt[c], 1ull);
    }
}
// The old row at storage position c receives column spos[n_old + r].
__global__ void k_delta_fill(const int64_t* __restrict__ rp_new, size_t nr, CsrVals nv,
                             const uint32_t* __restrict__ old, const uint32_t* __restrict__ spos, int64_t n_old,
                             const int64_t* __restrict__ dptr, unsigned long long* __restrict__ dfill, CsrVals dv) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < (int64_t)nr; r += warps) {
    const int32_t me = (int32_t)spos[n_old + r];
    for (int64_t p = rp_new[r] + lane; p < rp_new[r + 1]; p += 32) {
      const uint32_t c = (uint32_t)nv.col[p];
      if (!is_old(old, c)) continue;
      const int64_t q = dptr[c] + (int64_t)atomicAdd(&dfill[c], 1ull);
      dv.col[q] = me;
      if (dv.v64) dv.v64[q] = nv.v64[p];
      if (dv.vhi) dv.vhi[q] = nv.vhi[p];
      if (dv.vlo) dv.vlo[q] = nv.vlo[p];
    }
  }
}
// rel[o] = new storage position of the determinant at old storage position o.
// Both orders sort by the same key, so rel is increasing.
__global__ void k_relabel(const uint32_t* __restrict__ perm_old, const uint32_t* __restrict__ spos, int64_t n_old,
                          uint32_t* __restrict__ rel) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_old; o += (int64_t)gridDim.x * blockDim.x)
    rel[o] = spos[perm_old[o]];
}
__global__ void k_merged_len(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ spos_old,
                             const int64_t* __restrict__ rp_old, const int64_t* __restrict__ dptr, int64_t n_old,
                             const int64_t* __restrict__ rp_new, int64_t N, int64_t* __restrict__ len) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = perm[i];
    if (u < n_old) {
      const int64_t o = spos_old[u];
      len[i] = (rp_old[o + 1] - rp_old[o]) + (dptr[i + 1] - dptr[i]);
    } else {
      len[i] = rp_new[u - n_old + 1] - rp_new[u - n_old];
    }
  }
}

// Number of lanes whose v (ascending across the warp) is below key.
__device__ __forceinline__ int warp_rank(uint32_t key, uint32_t v) {
  int r = 0;
#pragma unroll
  for (int st = 16; st >= 1; st >>= 1) {
    const uint32_t t = __shfl_sync(kFull, v, r + st - 1);
    if (t < key) r += st;
  }
  const uint32_t last = __shfl_sync(kFull, v, 31);
  if (r == 31 && last < key) r = 32;
  return r;
}

// Merged row at storage position i, warp per row. An old determinant's row is
// its old row A with columns relabelled (still sorted: the relabelling is
// increasing) merged with its new columns B (sorted; disjoint from A), 32
// outputs a step: the next 32 entries of A and of B are ranked against each
// other by shuffles, and those among the 32 smallest of the 64 (the next 32
// of the merged row) are written; the rest are taken up again next step. A
// new determinant's row is copied from the new rows.
// VK: 0 = FP64 values, 1 = FP32 head + tail.
template <int VK>
struct MergeVal;
template <>
struct MergeVal<0> {
  double v;
  __device__ void load(const double* v64, const float*, const float*, int64_t p) { v = v64[p]; }
  __device__ void store(double* v64, float*, float*, int64_t q) const { v64[q] = v; }
};
template <>
struct MergeVal<1> {
  float h, l;
  __device__ void load(const double*, const float* hi, const float* lo, int64_t p) {
    h = hi[p];
    l = lo[p];
  }
  __device__ void store(double*, float* hi, float* lo, int64_t q) const {
    hi[q] = h;
    lo[q] = l;
  }
};
template <int VK>
__global__ void __launch_bounds__(256) k_merge_rows(const uint32_t* __restrict__ perm,
                                                    const uint32_t* __restrict__ spos_old,
                                                    const int64_t* __restrict__ rp_old, CsrVals ov,
                                                    const uint32_t* __restrict__ rel,
                                                    const int64_t* __restrict__ dptr, CsrVals dv,
                                                    const int64_t* __restrict__ rp_new, CsrVals nv, int64_t n_old,
                                                    int64_t N, const int64_t* __restrict__ rp, CsrVals out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  int32_t* __restrict__ ocol = out.col;
  double* __restrict__ o64 = out.v64;
  float* __restrict__ ohi = out.vhi;
  float* __restrict__ olo = out.vlo;
  constexpr uint32_t kNone = 0xffffffffu;  // above every storage position
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += warps) {
    const int64_t d = rp[i];
    const int64_t u = perm[i];
    if (u >= n_old) {  // a new row: copied
      const int64_t a0 = rp_new[u - n_old], la = rp_new[u - n_old + 1] - a0;
      for (int64_t t = lane; t < la; t += 32) {
        MergeVal<VK> v;
        v.load(nv.v64, nv.vhi, nv.vlo, a0 + t);
        ocol[d + t] = nv.col[a0 + t];
        v.store(o64, ohi, olo, d + t);
      }
      continue;
    }
    const int64_t o = spos_old[u];
    const int64_t a0 = rp_old[o], la = rp_old[o + 1] - a0;
    const int64_t b0 = dptr[i], lb = dptr[i + 1] - b0;
    if (lb == 0) {  // no new columns: the old row relabelled
      for (int64_t t = lane; t < la; t += 32) {
        MergeVal<VK> v;
        v.load(ov.v64, ov.vhi, ov.vlo, a0 + t);
        ocol[d + t] = (int32_t)rel[ov.col[a0 + t]];
        v.store(o64, ohi, olo, d + t);
      }
      continue;
    }
    int64_t ia = 0, ib = 0;
    while (ia < la || ib < lb) {
      const bool va = ia + lane < la, vb = ib + lane < lb;
      const uint32_t ka = va ? rel[ov.col[a0 + ia + lane]] : kNone;
      const uint32_t kb = vb ? (uint32_t)dv.col[b0 + ib + lane] : kNone;
      const int pa = lane + warp_rank(ka, kb);  // position among the 64 of this step
      const int pb = lane + warp_rank(kb, ka);
      const bool ea = va && pa < 32, eb = vb && pb < 32;
      const int64_t base = d + ia + ib;
      if (ea) {
        MergeVal<VK> v;
        v.load(ov.v64, ov.vhi, ov.vlo, a0 + ia + lane);
        ocol[base + pa] = (int32_t)ka;
        v.store(o64, ohi, olo, base + pa);
      }
      if (eb) {
        MergeVal<VK> w;
        w.load(dv.v64, dv.vhi, dv.vlo, b0 + ib + lane);
        ocol[base + pb] = (int32_t)kb;
        w.store(o64, ohi, olo, base + pb);
      }
      ia += __popc(__ballot_sync(kFull, ea));
      ib += __popc(__ballot_sync(kFull, eb));
    }
  }
}

void build_ham_csr(const Helpers& hp, const Det2* dets, const IntsView& ints, Csr& H, bool want64, bool want32,
                   bool want_lo, size_t n_old, Prims& pr, cudaStream_t s) {
  const size_t N = hp.N;
  PhaseTimer pt(s);
  const bool incremental = !H.block && n_old > 0 && n_old < N && H.N == n_old && H.perm.n >= n_old &&
                           (want64 ? !want32 : (want32 && want_lo)) &&
                           (H.v64.p != nullptr) == want64 && (H.vhi.p != nullptr) == want32 &&
                           (H.vlo.p != nullptr) == (want32 && want_lo);
  if (!incremental) {
    if (n_old == N && H.N == N && !H.block) return;  // nothing new
    H.clear_block();
    storage_order(hp, H.perm, H.spos, pr, s);
    pt.mark("ham storage order");
    H.nnz = emit_rows(hp, 0, N, H.spos.p, H.spos.p, dets, ints, H.rowptr, H.col, H.v64, H.vhi, H.vlo, want64, want32,
                      want_lo, pr, s, pt);
    H.N = N;
    SHCI_CUDA(cudaStreamSynchronize(s));
    return;
  }
  const size_t nr = N - n_old;
  DevBuf<uint32_t> perm, spos;
  storage_order(hp, perm, spos, pr, s);
  pt.mark("ham storage order");
  Csr Hn;  // rows of the determinants n_old .. N-1
  Hn.nnz = emit_rows(hp, n_old, N, nullptr, spos.p, dets, ints, Hn.rowptr, Hn.col, Hn.v64, Hn.vhi, Hn.vlo, want64,
                     want32, want_lo, pr, s, pt);
  CsrVals nv{Hn.col.p, Hn.v64.p, Hn.vhi.p, Hn.vlo.p};
  // new columns of the old rows, indexed by the old row's new storage position
  DevBuf<uint32_t> oldbits;
  oldbits.resize((N + 31) / 32);
  k_old_bits<<<grid_for((N + 31) / 32, 256), 256, 0, s>>>(perm.p, (int64_t)N, (int64_t)n_old, oldbits.p);
  SHCI_LAUNCH_CHECK();
  DevBuf<unsigned long long> dcnt, dfill;
  dcnt.resize(N);
  dfill.resize(N);
  SHCI_CUDA(cudaMemsetAsync(dcnt.p, 0, N * sizeof(unsigned long long), s));
  SHCI_CUDA(cudaMemsetAsync(dfill.p, 0, N * sizeof(unsigned long long), s));
  const unsigned wblocks = grid_for(nr * 32, 256, 152 * 16);
  k_delta_count<<<wblocks, 256, 0, s>>>(Hn.rowptr.p, nr, Hn.col.p, oldbits.p, dcnt.p);
  SHCI_LAUNCH_CHECK();
  DevBuf<int64_t> dptr;
  dptr.resize(N + 1);
  int64_t dtotal = 0;
  scan_exclusive_i64(reinterpret_cast<const int64_t*>(dcnt.p), dptr.p, N, &dtotal, pr, s);
  k_set_last<<<1, 1, 0, s>>>(dptr.p, (int64_t)N, dtotal);
  SHCI_LAUNCH_CHECK();
  Csr Hd;
  const size_t dcap = dtotal > 0 ? (size_t)dtotal : 1;
  Hd.col.resize(dcap);
  if (want64) Hd.v64.resize(dcap);
  if (want32) Hd.vhi.resize(dcap);
  if (want32 && want_lo) Hd.vlo.resize(dcap);
  CsrVals dv{Hd.col.p, Hd.v64.p, Hd.vhi.p, Hd.vlo.p};
  k_delta_fill<<<wblocks, 256, 0, s>>>(Hn.rowptr.p, nr, nv, oldbits.p, spos.p, (int64_t)n_old, dptr.p, dfill.p, dv);
  SHCI_LAUNCH_CHECK();
  sort_rows(dptr.p, N, dv, s);
  pt.mark("ham new columns");
  // merge in the new storage order
  DevBuf<uint32_t> rel;
  rel.resize(n_old);
  k_relabel<<<grid_for(n_old, 256), 256, 0, s>>>(H.perm.p, spos.p, (int64_t)n_old, rel.p);
  SHCI_LAUNCH_CHECK();
  DevBuf<int64_t> len, rp;
  len.resize(N);
  rp.resize(N + 1);
  k_merged_len<<<grid_for(N, 256), 256, 0, s>>>(perm.p, H.spos.p, H.rowptr.p, dptr.p, (int64_t)n_old, Hn.rowptr.p,
                                                (int64_t)N, len.p);
  SHCI_LAUNCH_CHECK();
  int64_t total = 0;
  scan_exclusive_i64(len.p, rp.p, N, &total, pr, s);
  k_set_last<<<1, 1, 0, s>>>(rp.p, (int64_t)N, total);
  SHCI_LAUNCH_CHECK();
  Csr M;
  const size_t cap = total > 0 ? (size_t)total : 1;
  M.col.resize(cap);
  if (want64) M.v64.resize(cap);
  if (want32) M.vhi.resize(cap);
  if (want32 && want_lo) M.vlo.resize(cap);
  CsrVals ov{H.col.p, H.v64.p, H.vhi.p, H.vlo.p}, mv{M.col.p, M.v64.p, M.vhi.p, M.vlo.p};
  if (want64)
    k_merge_rows<0><<<grid_for(N * 32, 256, 152 * 16), 256, 0, s>>>(perm.p, H.spos.p, H.rowptr.p, ov, rel.p,
                                                                    dptr.p, dv, Hn.rowptr.p, nv, (int64_t)n_old,
                                                                    (int64_t)N, rp.p, mv);
  else
    k_merge_rows<1><<<grid_for(N * 32, 256, 152 * 16), 256, 0, s>>>(perm.p, H.spos.p, H.rowptr.p, ov, rel.p,
                                                                    dptr.p, dv, Hn.rowptr.p, nv, (int64_t)n_old,
                                                                    (int64_t)N, rp.p, mv);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));
  H.rowptr.swap(rp);
  H.col.swap(M.col);
  H.v64.swap(M.v64);
  H.vhi.swap(M.vhi);
  H.vlo.swap(M.vlo);
  H.perm.swap(perm);
  H.spos.swap(spos);
  H.N = N;
  H.nnz = total;
  pt.mark("ham merge");
}

// ---------------------------------------------------------------------------
// Row block: one rank's share of the Hamiltonian in the sharded path, the full
// rows of the determinants [r0, r1) with every column. Local rows are those
// determinants in storage order (alpha-major, as in the whole matrix);
// H.perm[r] is the determinant of local row r, H.xpos[r] its storage position
// (where its own x sits for the diagonal term) and H.xperm the whole storage
// order (storage position -> determinant), through which x is packed. Columns
// are storage positions of the whole space. A row's entries and their order
// are those of the same row in the whole matrix.
// ---------------------------------------------------------------------------
__global__ void k_block_flags(const uint32_t* __restrict__ perm, size_t n, uint32_t r0, uint32_t r1,
                              int64_t* __restrict__ flag) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t d = perm[i];
    flag[i] = (d >= r0 && d < r1) ? 1 : 0;
  }
}
__global__ void k_block_fill(const uint32_t* __restrict__ perm, size_t n, uint32_t r0, uint32_t r1,
                             const int64_t* __restrict__ pos, uint32_t* __restrict__ rows, uint32_t* __restrict__ xpos,
                             uint32_t* __restrict__ slot) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t d = perm[i];
    if (d >= r0 && d < r1) {
      const int64_t q = pos[i];
      rows[q] = d;
      xpos[q] = (uint32_t)i;
      slot[d] = (uint32_t)q;
    }
  }
}

void build_ham_block(const Helpers& hp, const Det2* dets, const IntsView& ints, Csr& H, bool want64, bool want32,
                     bool want_lo, size_t r0, size_t r1, Prims& pr, cudaStream_t s) {
  const size_t N = hp.N;
  if (!(r0 < r1 && r1 <= N)) throw Error(kErrInvalid, "row block [r0, r1) must be a non-empty range of the space");
  const size_t nb = r1 - r0;
  PhaseTimer pt(s);
  DevBuf<uint32_t> perm, spos;
  storage_order(hp, perm, spos, pr, s);
  DevBuf<int64_t> flag, pos;
  flag.resize(N);
  pos.resize(N);
  k_block_flags<<<grid_for(N, 256), 256, 0, s>>>(perm.p, N, (uint32_t)r0, (uint32_t)r1, flag.p);
  SHCI_LAUNCH_CHECK();
  int64_t nflag = 0;
  scan_exclusive_i64(flag.p, pos.p, N, &nflag, pr, s);
  if ((size_t)nflag != nb) throw Error(kErrState, "row block: storage order lost determinants");
  DevBuf<uint32_t> rows, xpos, slot;
  rows.resize(nb);
  xpos.resize(nb);
  slot.resize(N);
  k_block_fill<<<grid_for(N, 256), 256, 0, s>>>(perm.p, N, (uint32_t)r0, (uint32_t)r1, pos.p, rows.p, xpos.p,
                                                slot.p);
  SHCI_LAUNCH_CHECK();
  pt.mark("ham block order");
  H.drop_compressed();
  H.nnz = emit_rows(hp, r0, r1, slot.p, spos.p, dets, ints, H.rowptr, H.col, H.v64, H.vhi, H.vlo, want64, want32,
                    want_lo, pr, s, pt);
  SHCI_CUDA(cudaStreamSynchronize(s));
  H.perm.swap(rows);
  H.xpos.swap(xpos);
  H.xperm.swap(perm);
  H.spos.release();
  H.N = nb;
  H.nfull = N;
  H.row0 = r0;
  H.block = true;
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
// Matrix-free sigma (HmultDirect, SHCI/Hmult.h:241-381): row I's connections
// are found by visit_row and H_IJ is recomputed (ket = max(I, J), so the
// element is the same in both triangles). Hits are queued per warp, singles
// and doubles apart, and evaluated 32 at a time on full warps, as in the H
// build. FP64: the reference's arithmetic. FP32 (the first stage of the
// mixed matrix-free path): FP32 integrals, FP32 elements, compensated FP32
// accumulation of h * x.
template <int K, bool F32>
struct DirectQVisitor {
  using T = typename std::conditional<F32, float, double>::type;
  const Det2* dets;
  IntsView ints;
  Det2 dI;
  uint32_t I;
  const T* x;  // [N][K]
  uint32_t* qs;
  uint32_t* qd;
  int ns, nd;
  Acc a32[K];
  double a64[K];

  __device__ void add(uint32_t J) {
    const Det2 dJ = dets[J];
    if constexpr (F32) {
      const float hv = ham_element_f32(ints.I1f, ints.I2f, ints.V1f, ints.norb, dI, dJ, J < I);
#pragma unroll
      for (int r = 0; r < K; ++r) acc_add(a32[r], hv, x[(size_t)J * K + r]);
    } else {
      const double hv = ham_element(ints.I1, ints.I2, ints.V1, ints.norb, dI, dJ, J < I);
#pragma unroll
      for (int r = 0; r < K; ++r) a64[r] += hv * x[(size_t)J * K + r];
    }
  }
  __device__ int drain(uint32_t* q, int n, int cnt) {
    const int lane = threadIdx.x & 31;
    if (lane < cnt) add(q[lane]);
    __syncwarp();
    const int rest = n - cnt;
    const uint32_t v = lane < rest ? q[cnt + lane] : 0u;
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

template <int K, bool F32>
__global__ void __launch_bounds__(256, SHCI_DIRECT_MIN_BLOCKS) k_sigma_direct(HelperView h, const Det2* __restrict__ dets, IntsView ints,
                                                      const double* __restrict__ diag,
                                                      const typename DirectQVisitor<K, F32>::T* __restrict__ x,
                                                      double* __restrict__ y) {
  __shared__ uint32_t s_q[8][2][64];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  // rows in alpha-major order (the alpha groups' determinant lists): rows of
  // one alpha string run side by side and probe the same sections of the
  // partial-string index, and largely the same connections, from cache
  for (int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < (int64_t)h.N; k += warps) {
    const int64_t I = h.aDets[k];
    DirectQVisitor<K, F32> v;
    v.dets = dets;
    v.ints = ints;
    v.dI = dets[I];
    v.I = (uint32_t)I;
    v.x = x;
    v.qs = s_q[wib][0];
    v.qd = s_q[wib][1];
    v.ns = v.nd = 0;
#pragma unroll
    for (int r = 0; r < K; ++r) {
      v.a32[r] = Acc{0.f, 0.f};
      v.a64[r] = 0.0;
    }
    visit_row(h, (uint32_t)I, v);
    v.flush();
#pragma unroll
    for (int r = 0; r < K; ++r) {
      if constexpr (F32) {
        Acc a = v.a32[r];
        // merge in lane order (a fixed tree); FP64 diagonal term
#pragma unroll
        for (int o = 16; o; o >>= 1) {
          Acc other{__shfl_xor_sync(kFull, a.s, o), __shfl_xor_sync(kFull, a.c, o)};
          if ((lane & o) == 0) {
            acc_merge(a, other);
          } else {
            acc_merge(other, a);
            a = other;
          }
        }
        if (lane == 0) y[(size_t)I * K + r] = diag[I] * (double)x[(size_t)I * K + r] + ((double)a.s + (double)a.c);
      } else {
        double a = v.a64[r];
#pragma unroll
        for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
        if (lane == 0) y[(size_t)I * K + r] = diag[I] * x[(size_t)I * K + r] + a;
      }
    }
  }
}

void sigma_direct(const Helpers& hp, const Det2* dets, const IntsView& ints, const double* diag, const double* x,
                  double* y, int k, cudaStream_t s) {
  HelperView hv = hp.view();
  const unsigned blocks = grid_for(hp.N * 32, 256, 152 * 16);
  switch (k) {
    case 1: k_sigma_direct<1, false><<<blocks, 256, 0, s>>>(hv, dets, ints, diag, x, y); break;
    case 2: k_sigma_direct<2, false><<<blocks, 256, 0, s>>>(hv, dets, ints, diag, x, y); break;
    case 4: k_sigma_direct<4, false><<<blocks, 256, 0, s>>>(hv, dets, ints, diag, x, y); break;
    default: throw Error(kErrInvalid, "direct sigma supports k in {1,2,4}");
  }
  SHCI_LAUNCH_CHECK();
}

void sigma_direct32(const Helpers& hp, const Det2* dets, const IntsView& ints, const double* diag, const float* x,
                    double* y, int k, cudaStream_t s) {
  if (!ints.I1f || !ints.I2f) throw Error(kErrState, "FP32 integrals missing");
  HelperView hv = hp.view();
  const unsigned blocks = grid_for(hp.N * 32, 256, 152 * 16);
  switch (k) {
    case 1: k_sigma_direct<1, true><<<blocks, 256, 0, s>>>(hv, dets, ints, diag, x, y); break;
    case 2: k_sigma_direct<2, true><<<blocks, 256, 0, s>>>(hv, dets, ints, diag, x, y); break;
    case 4: k_sigma_direct<4, true><<<blocks, 256, 0, s>>>(hv, dets, ints, diag, x, y); break;
    default: throw Error(kErrInvalid, "direct sigma supports k in {1,2,4}");
  }
  SHCI_LAUNCH_CHECK();
}

}  // namespace shci
