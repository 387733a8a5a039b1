// Deterministic second-order (Epstein-Nesbet) perturbation theory.
//
// Restates SHCIbasics::DoPerturbativeDeterministic (SHCI/SHCIbasics.cpp:453-728,
// the branch without RDMs) and its generator
// SHCIgetdeterminants::getDeterminantsDeterministicPT
// (SHCI/SHCIgetdeterminants.cpp:40-171). For every variational determinant i
// with epsilon = |eps2 / c_i|:
//   singles  i -> a (same spin): exact H_ai (Hij_1Excite), kept if |H_ai| > epsilon,
//            numerator H_ai c_i;
//   doubles  from the heat-bath list of each occupied pair while |v| >= epsilon,
//            a and b empty, numerator v * sign * c_i with v the list's FP32 value;
//   no ncore/nact filter, only the occupation restrictions.
// Equal determinants are merged by summing numerators, those in the
// variational space removed, and E2 = sum_a N_a^2 / (E0 - E_a).
//
// GPU form (one launch sequence per hash partition):
//   k_pt_gen<false>  one warp per parent (dynamic queue) counts the candidates
//                    outside the variational space (hash probe) that fall in
//                    this partition;
//   exclusive scan   -> each parent's output offset, so the output is in
//                    (parent, generation) order whatever the warp schedule;
//   k_pt_gen<true>   the same walk writes (determinant, numerator);
//   radix sort       stable, by determinant, with the candidate index as payload;
//   k_pt_reduce      one thread per run of equal determinants: numerators summed
//                    in parent order, E_a from the integrals, fixed-grid block
//                    partials summed on the host in block order.
// Results are therefore bitwise reproducible for a given partition count.
// When the candidates do not fit in device memory they are split by a hash of
// the determinant, as the reference splits them over MPI ranks
// (SHCI/SHCIbasics.cpp:519-530); each partition is generated, sorted and
// reduced alone.
#include <algorithm>
#include <cmath>

#include "ham.h"

namespace shci {

namespace {

constexpr int kPtThreads = 256;
constexpr int kPtWarps = kPtThreads / 32;
constexpr unsigned kPtRedBlocks = 152 * 4;
constexpr int kPtRedThreads = 256;
// device bytes per candidate in one partition: determinant (16), numerator (8),
// sort payload (4), the sort's split words and alternates (16 + 16 + 4)
constexpr size_t kPtBytesPerCand = 64;

inline unsigned grid_for(size_t n, int threads, size_t max_blocks = 152 * 64) {
  size_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (unsigned)b;
}

struct PtArgs {
  const Det2* dets;
  const double* c;
  size_t n;
  double eps2;
  IntsView ints;
  HeatBathView hb;
  double maxEntry;
  SelectParams sp;
  const uint32_t* hslots;
  uint64_t hmask;
  uint32_t nparts, part;
  unsigned long long* next;
  int64_t* counts;
  const int64_t* offs;
  Det2* out;
  double* num;
};

__device__ __forceinline__ bool in_part(const PtArgs& a, const Det2& d) {
  return a.nparts == 1 || (uint32_t)((det_hash(d) >> 32) % a.nparts) == a.part;
}

// Determinant::parity(a, b, i, j, sgn) on the excited determinant di
// (SHCI/Determinants.cpp:332-357 as called at SHCIgetdeterminants.cpp:155-157):
// the a<->i transposition counted on di, then b<->j on di with a emptied and
// i refilled.
__device__ __forceinline__ double pt_double_sign(Det2 di, int a, int b, int i, int j) {
  int n1 = occ_between(di, a < i ? a : i, a < i ? i : a);
  det_flip(di, a);
  det_flip(di, i);
  int n2 = occ_between(di, b < j ? b : j, b < j ? j : b);
  return ((n1 + n2) & 1) ? -1.0 : 1.0;
}

// Warp-uniform count / ordered write of the lanes with `keep`. Writes stay
// inside the parent's range [base, lim) of the counting pass.
template <bool EMIT>
__device__ __forceinline__ void pt_put(const PtArgs& a, bool keep, const Det2& cand, double v, int64_t base,
                                       int64_t lim, int64_t& cnt) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(kFull, keep);
  if (EMIT && keep) {
    const int64_t q = base + cnt + __popc(m & ((1u << lane) - 1u));
    if (q < lim) {
      a.out[q] = cand;
      a.num[q] = v;
    }
  }
  cnt += __popc(m);
}

template <bool EMIT>
__global__ void __launch_bounds__(kPtThreads) k_pt_gen(PtArgs a) {
  __shared__ unsigned char s_closed[kPtWarps][kMaxSpin];
  __shared__ unsigned char s_open[kPtWarps][kMaxSpin];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned char* closed = s_closed[wib];
  unsigned char* open = s_open[wib];
  const int n2 = 2 * a.ints.norb;
  const SelectParams& sp = a.sp;
  while (true) {
    unsigned long long pp = 0;
    if (lane == 0) pp = atomicAdd(a.next, 1ull);
    pp = __shfl_sync(kFull, pp, 0);
    if (pp >= (unsigned long long)a.n) break;
    const size_t p = (size_t)pp;
    const Det2 d = a.dets[p];
    const double cp = a.c[p];
    const double eps = fabs(a.eps2 / cp);
    const int64_t base = EMIT ? a.offs[p] : 0;
    const int64_t lim = EMIT ? base + a.counts[p] : 0;
    int64_t cnt = 0;
    if (eps < INFINITY) {  // c_i = 0: nothing passes either threshold
      __syncwarp();
      if (lane == 0) {
        int nc = 0, no = 0;
        for (int q = 0; q < n2; ++q) {
          if (det_getocc(d, q))
            closed[nc++] = (unsigned char)q;
          else
            open[no++] = (unsigned char)q;
        }
      }
      __syncwarp();
      const int nclosed = __popcll(d.w0) + __popcll(d.w1);
      const int nopen = n2 - nclosed;
      int cur[kMaxRestrict];
      for (int r = 0; r < sp.nrestrict; ++r) cur[r] = __popcll(d.w0 & sp.rmask0[r]) + __popcll(d.w1 & sp.rmask1[r]);

      // ---- singles: every same-spin (i, a); the exact element decides
      const int ns = nclosed * nopen;
      for (int b0 = 0; b0 < ns; b0 += 32) {
        const int q = b0 + lane;
        bool keep = false;
        Det2 cand = d;
        double v = 0.0;
        if (q < ns) {
          const int ci = closed[q / nopen], oa = open[q % nopen];
          // a spin flip has a zero element (no alpha-beta block in I1)
          bool ok = (ci & 1) == (oa & 1);
          for (int r = 0; ok && r < sp.nrestrict; ++r) {
            int e = cur[r] - in_mask(sp, r, ci) + in_mask(sp, r, oa);
            ok = e >= sp.rmin[r] && e <= sp.rmax[r];
          }
          if (ok) {
            const double h = hij_single(a.ints, d, oa, ci);
            if (fabs(h) > eps) {
              det_flip(cand, oa);
              det_flip(cand, ci);
              keep = in_part(a, cand) && !hash_contains(a.hslots, a.hmask, a.dets, cand);
              v = h * cp;
            }
          }
        }
        pt_put<EMIT>(a, keep, cand, v, base, lim, cnt);
      }

      // ---- doubles: heat-bath list prefixes, flattened over the warp
      if (!(fabs(a.maxEntry) < eps)) {
        const int npairs = nclosed * (nclosed - 1) / 2;
        for (int pb = 0; pb < npairs; pb += 32) {
          const int q = pb + lane;
          int ci = 0, cj = 0;
          int64_t lstart = 0, len = 0;
          bool same = false;
          if (q < npairs) {
            // q -> (i, j), i > j, q = i(i-1)/2 + j
            int i = (int)((1.0 + sqrt(1.0 + 8.0 * (double)q)) * 0.5);
            while (i * (i - 1) / 2 > q) --i;
            while ((i + 1) * i / 2 <= q) ++i;
            const int j = q - i * (i - 1) / 2;
            ci = closed[i];
            cj = closed[j];
            const int I = ci >> 1, J = cj >> 1;
            const int X = I > J ? I : J, Y = I > J ? J : I;
            const int pair = X * (X + 1) / 2 + Y;
            same = (ci & 1) == (cj & 1);
            const int64_t* st = same ? a.hb.sameStart : a.hb.oppStart;
            const float* vals = same ? a.hb.sameVal : a.hb.oppVal;
            const int64_t s0 = st[pair], s1 = st[pair + 1];
            // first entry with |v| < eps (lists sorted by |v| descending)
            int64_t lo = s0, hi = s1;
            while (lo < hi) {
              const int64_t mid = (lo + hi) >> 1;
              if ((double)fabsf(vals[mid]) < eps)
                hi = mid;
              else
                lo = mid + 1;
            }
            lstart = s0;
            len = lo - s0;
          }
          int64_t incl = len;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
          }
          const int64_t total = __shfl_sync(kFull, incl, 31);
          const int64_t excl = incl - len;
          for (int64_t f0 = 0; f0 < total; f0 += 32) {
            const int64_t f = f0 + lane;
            // owner lane of flattened entry f: last lane with excl <= f
            int lo = 0;
#pragma unroll
            for (int st = 16; st >= 1; st >>= 1) {
              const int c = lo + st;
              const int64_t e = __shfl_sync(kFull, excl, c < 32 ? c : 31);
              if (c < 32 && e <= f) lo = c;
            }
            const int64_t ls = __shfl_sync(kFull, lstart, lo);
            const int64_t eo = __shfl_sync(kFull, excl, lo);
            const int oci = __shfl_sync(kFull, ci, lo);
            const int ocj = __shfl_sync(kFull, cj, lo);
            const bool osame = __shfl_sync(kFull, (int)same, lo) != 0;
            bool keep = false;
            Det2 cand = d;
            double v = 0.0;
            if (f < total) {
              const int64_t index = ls + (f - eo);
              const int16_t* pr = osame ? a.hb.samePairs : a.hb.oppPairs;
              const float* vals = osame ? a.hb.sameVal : a.hb.oppVal;
              const int av = 2 * pr[2 * index] + (oci & 1);
              const int bv = 2 * pr[2 * index + 1] + (ocj & 1);
              bool ok = true;
              for (int r = 0; ok && r < sp.nrestrict; ++r) {
                int e = cur[r] - in_mask(sp, r, oci) - in_mask(sp, r, ocj) + in_mask(sp, r, av) + in_mask(sp, r, bv);
                ok = e >= sp.rmin[r] && e <= sp.rmax[r];
              }
              if (ok && !(det_getocc(d, av) || det_getocc(d, bv))) {
                det_flip(cand, av);
                det_flip(cand, bv);
                det_flip(cand, oci);
                det_flip(cand, ocj);
                keep = in_part(a, cand) && !hash_contains(a.hslots, a.hmask, a.dets, cand);
                if (keep) v = (double)vals[index] * pt_double_sign(cand, av, bv, oci, ocj) * cp;
              }
            }
            pt_put<EMIT>(a, keep, cand, v, base, lim, cnt);
          }
        }
      }
    }
    if (!EMIT && lane == 0) a.counts[p] = cnt;
  }
}

__global__ void k_pt_iota(uint32_t* __restrict__ p, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = (uint32_t)i;
}

// One thread per run of equal determinants in the sorted candidates; block
// partials {E2, |psi1|^2, count} in part[3 * block].
__global__ void __launch_bounds__(kPtRedThreads) k_pt_reduce(const Det2* __restrict__ sorted,
                                                             const uint32_t* __restrict__ perm,
                                                             const double* __restrict__ num, size_t m, IntsView ints,
                                                             double E0, double* __restrict__ part) {
  extern __shared__ double sm[];
  const int nn = ints.norb * ints.norb;
  double* sD = sm;
  double* sX = sm + nn;
  for (int j = threadIdx.x; j < nn; j += blockDim.x) {
    sD[j] = ints.Direct[j];
    sX[j] = ints.Exchange[j];
  }
  __syncthreads();
  double e2 = 0.0, psi = 0.0, cnt = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (size_t)gridDim.x * blockDim.x) {
    const Det2 d = sorted[k];
    if (k > 0 && det_eq(d, sorted[k - 1])) continue;
    double s = num[perm[k]];
    for (size_t j = k + 1; j < m; ++j) {
      if (!det_eq(sorted[j], d)) break;
      s += num[perm[j]];
    }
    const double de = E0 - det_energy(ints, d, sD, sX);
    e2 += s * s / de;
    const double t = s / de;
    psi += t * t;
    cnt += 1.0;
  }
  __shared__ double r0[kPtRedThreads / 32], r1[kPtRedThreads / 32], r2[kPtRedThreads / 32];
  for (int o = 16; o; o >>= 1) {
    e2 += __shfl_xor_sync(kFull, e2, o);
    psi += __shfl_xor_sync(kFull, psi, o);
    cnt += __shfl_xor_sync(kFull, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r0[threadIdx.x >> 5] = e2;
    r1[threadIdx.x >> 5] = psi;
    r2[threadIdx.x >> 5] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0, c = 0.0;
    for (int w = 0; w < kPtRedThreads / 32; ++w) {
      a += r0[w];
      b += r1[w];
      c += r2[w];
    }
    part[3 * blockIdx.x] = a;
    part[3 * blockIdx.x + 1] = b;
    part[3 * blockIdx.x + 2] = c;
  }
}

}  // namespace

PtResult pt_deterministic(const Det2* dets, size_t n, const double* c, double E0, double eps2, const IntsView& ints,
                          const HeatBathView& hb, double maxEntry, const SelectParams& sp, const DetHash& present,
                          int64_t max_candidates, PtWork& w, Prims& pr, cudaStream_t s) {
  PtResult res;
  if (n == 0) return res;
  if (!(eps2 >= 0.0)) throw Error(kErrInvalid, "epsilon2 must be >= 0");
  w.counts.resize(n);
  w.offs.resize(n);
  w.next.resize(1);
  w.part.resize(3 * kPtRedBlocks);
  PtArgs a{};
  a.dets = dets;
  a.c = c;
  a.n = n;
  a.eps2 = eps2;
  a.ints = ints;
  a.hb = hb;
  a.maxEntry = maxEntry;
  a.sp = sp;
  a.hslots = present.slots.p;
  a.hmask = present.mask;
  a.next = w.next.p;
  a.counts = w.counts.p;
  a.offs = w.offs.p;
  const unsigned gen_blocks = 152 * 8;  // one warp per parent from a shared queue
  auto gen = [&](bool emit, uint32_t nparts, uint32_t part) -> int64_t {
    a.nparts = nparts;
    a.part = part;
    SHCI_CUDA(cudaMemsetAsync(w.next.p, 0, sizeof(unsigned long long), s));
    if (emit) {
      a.out = w.cand.p;
      a.num = w.num.p;
      k_pt_gen<true><<<gen_blocks, kPtThreads, 0, s>>>(a);
      SHCI_LAUNCH_CHECK();
      return 0;
    }
    k_pt_gen<false><<<gen_blocks, kPtThreads, 0, s>>>(a);
    SHCI_LAUNCH_CHECK();
    int64_t total = 0;
    scan_exclusive_i64(w.counts.p, w.offs.p, n, &total, pr, s);
    return total;
  };

  // capacity of one partition
  int64_t cap = max_candidates;
  if (cap <= 0) {
    size_t fr = 0, tot = 0;
    SHCI_CUDA(cudaMemGetInfo(&fr, &tot));
    size_t avail = fr;
    if (g_alloc_cap) avail = std::min(avail, g_alloc_cap > g_alloc_live ? g_alloc_cap - g_alloc_live : (size_t)0);
    // what the buffers already hold counts as available to them
    avail += w.cand.cap * sizeof(Det2) + w.num.cap * sizeof(double) + w.perm.cap * sizeof(uint32_t);
    cap = (int64_t)(avail / 4 * 3 / kPtBytesPerCand);
  }
  cap = std::min<int64_t>(cap, (int64_t)0xfffffff0u);
  if (cap < 1) throw Error(kErrOOM, "no device memory left for perturbation candidates");

  PhaseTimer pt(s);
  const int64_t total_all = gen(false, 1, 0);
  pt.mark("pt count");
  uint32_t nparts = total_all <= cap ? 1u : (uint32_t)((total_all + total_all / 8) / cap + 1);
  const size_t smem = 2 * sizeof(double) * ints.norb * ints.norb;
  SHCI_CUDA(cudaFuncSetAttribute(k_pt_reduce, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  std::vector<double> hp(3 * kPtRedBlocks);
  for (int attempt = 0;; ++attempt) {
    res = PtResult();
    res.partitions = (int)nparts;
    bool overflow = false;
    for (uint32_t part = 0; part < nparts; ++part) {
      const int64_t m = nparts == 1 ? total_all : gen(false, nparts, part);
      if (m > cap) {
        overflow = true;
        break;
      }
      res.candidates += m;
      if (m == 0) continue;
      w.cand.reserve((size_t)m);
      w.num.reserve((size_t)m);
      w.perm.resize((size_t)m);
      gen(true, nparts, part);
      pt.mark("pt emit");
      k_pt_iota<<<grid_for((size_t)m, 256), 256, 0, s>>>(w.perm.p, (size_t)m);
      SHCI_LAUNCH_CHECK();
      sort_dets(w.cand.p, w.perm.p, (size_t)m, pr, s);
      pt.mark("pt sort");
      k_pt_reduce<<<kPtRedBlocks, kPtRedThreads, smem, s>>>(w.cand.p, w.perm.p, w.num.p, (size_t)m, ints, E0,
                                                            w.part.p);
      SHCI_LAUNCH_CHECK();
      pt.mark("pt reduce");
      SHCI_CUDA(cudaMemcpyAsync(hp.data(), w.part.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
      for (unsigned b = 0; b < kPtRedBlocks; ++b) {
        res.e2 += hp[3 * b];
        res.psi1_norm += hp[3 * b + 1];
        res.unique += (int64_t)hp[3 * b + 2];
      }
    }
    if (!overflow) break;
    if (attempt >= 8) throw Error(kErrOOM, "perturbation candidates do not fit in device memory");
    nparts *= 2;
  }
  SHCI_CUDA(cudaStreamSynchronize(s));
  return res;
}

}  // namespace shci
