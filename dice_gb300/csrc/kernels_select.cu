// Heat-bath selection of new determinants, one warp per parent determinant.
// Restates SHCIgetdeterminants::getDeterminantsVariationalApprox
// (SHCI/SHCIgetdeterminants.cpp:586-739) as called from the parent loop of
// DoVariational (SHCI/SHCIbasics.cpp:969-982) with threshold eps1/|cMax_i|:
//   singles: for occupied i, empty a (ncore/nact and restriction filters):
//            bound Singles(a,i) > eps, then the exact FP64 Hij_1Excite > eps;
//   doubles: for occupied pairs i > j, the heat-bath list of the pair is
//            scanned while |v| >= eps (list sorted by |float| descending).
// The prefix length of each pair list is found by binary search, and the
// (pair, entry) work is flattened across the 32 lanes.
// Candidates already in the variational space are dropped by a hash lookup
// (the reference's binary_search over SortedDets); sort + unique follow.
#include <cmath>

#include "ham.h"

namespace shci {

struct SelArgs {
  const Det2* dets;
  const double* cmax;
  size_t n;
  double eps1;
  IntsView ints;
  HeatBathView hb;
  double maxEntry;
  SelectParams sp;
  const uint32_t* hslots;
  uint64_t hmask;
  Det2* out;
  int64_t cap;
  int64_t* counter;
};

constexpr int kSelThreads = 256;
constexpr int kSelWarps = kSelThreads / 32;

// Warp-aggregated append of one candidate per lane with `emit` set.
__device__ __forceinline__ void append(const SelArgs& a, bool emit, const Det2& cand) {
  const int lane = threadIdx.x & 31;
  unsigned m = __ballot_sync(kFull, emit);
  if (!m) return;
  int leader = __ffs(m) - 1;
  int64_t base = 0;
  if (lane == leader) base = atomicAdd((unsigned long long*)a.counter, (unsigned long long)__popc(m));
  base = __shfl_sync(kFull, base, leader);
  if (emit) {
    int64_t q = base + __popc(m & ((1u << lane) - 1u));
    if (q < a.cap) a.out[q] = cand;
  }
}

__global__ void __launch_bounds__(kSelThreads) k_select(SelArgs a) {
  __shared__ unsigned char s_closed[kSelWarps][kMaxSpin];
  __shared__ unsigned char s_open[kSelWarps][kMaxSpin];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned char* closed = s_closed[wib];
  unsigned char* open = s_open[wib];
  const int n2 = 2 * a.ints.norb;
  const int64_t warps = (int64_t)gridDim.x * kSelWarps;
  const SelectParams& sp = a.sp;
  for (int64_t p = (int64_t)blockIdx.x * kSelWarps + wib; p < (int64_t)a.n; p += warps) {
    const Det2 d = a.dets[p];
    const double eps = a.eps1 / fabs(a.cmax[p]);
    if (!(eps < INFINITY)) continue;  // |c| = 0: nothing passes any threshold
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

    // ---- singles
    const int ns = nclosed * nopen;
    for (int base = 0; base < ns; base += 32) {
      const int q = base + lane;
      bool emit = false;
      Det2 cand = d;
      if (q < ns) {
        const int ci = closed[q / nopen], oa = open[q % nopen];
        bool ok = (ci >> 1) >= sp.ncore && (oa >> 1) < sp.ncore + sp.nact;
        for (int r = 0; ok && r < sp.nrestrict; ++r) {
          int e = cur[r] - in_mask(sp, r, ci) + in_mask(sp, r, oa);
          ok = e >= sp.rmin[r] && e <= sp.rmax[r];
        }
        if (ok) {
          double integral = a.hb.singles[(size_t)oa * n2 + ci];
          if (fabs(integral) > eps)
            if ((ci & 1) == (oa & 1)) integral = hij_single(a.ints, d, oa, ci);
          if (fabs(integral) > eps) {
            det_flip(cand, oa);
            det_flip(cand, ci);
            emit = !hash_contains(a.hslots, a.hmask, a.dets, cand);
          }
        }
      }
      append(a, emit, cand);
    }

    // ---- doubles
    if (fabs(a.maxEntry) < eps) continue;
    // for a float v, (double)|v| < eps exactly when |v| < eps rounded up to float
    const float eps_f = __double2float_ru(eps);
    const int npairs = nclosed * (nclosed - 1) / 2;
    for (int pb = 0; pb < npairs; pb += 32) {
      const int q = pb + lane;
      int ci = 0, cj = 0;
      int64_t lstart = 0, len = 0;
      bool same = false;
      if (q < npairs) {
        // q -> (i, j), i > j, q = i(i-1)/2 + j
        int i = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)q)) * 0.5f);  // corrected below
        while (i * (i - 1) / 2 > q) --i;
        while ((i + 1) * i / 2 <= q) ++i;
        int j = q - i * (i - 1) / 2;
        ci = closed[i];
        cj = closed[j];
        if ((ci >> 1) >= sp.ncore && (cj >> 1) >= sp.ncore) {
          int I = ci >> 1, J = cj >> 1;
          int X = I > J ? I : J, Y = I > J ? J : I;
          int pair = X * (X + 1) / 2 + Y;
          same = (ci & 1) == (cj & 1);
          const int64_t* st = same ? a.hb.sameStart : a.hb.oppStart;
          const float* vals = same ? a.hb.sameVal : a.hb.oppVal;
          int64_t s0 = st[pair], s1 = st[pair + 1];
          // first index with |v| < eps
          int64_t lo = s0, hi = s1;
          while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if (fabsf(vals[mid]) < eps_f)
              hi = mid;
            else
              lo = mid + 1;
          }
          lstart = s0;
          len = lo - s0;
        }
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
        const int64_t ls = __shfl_sync(kFull, lstart, lo);
        const int64_t eo = __shfl_sync(kFull, excl, lo);
        const int oci = __shfl_sync(kFull, ci, lo);
        const int ocj = __shfl_sync(kFull, cj, lo);
        const bool osame = __shfl_sync(kFull, (int)same, lo) != 0;
        bool emit = false;
        Det2 cand = d;
        if (f < total) {
          const int64_t index = ls + (f - eo);
          const int16_t* pr = osame ? a.hb.samePairs : a.hb.oppPairs;
          const int av = 2 * pr[2 * index] + (oci & 1);
          const int bv = 2 * pr[2 * index + 1] + (ocj & 1);
          bool ok = (av >> 1) < sp.ncore + sp.nact && (bv >> 1) < sp.ncore + sp.nact;
          for (int r = 0; ok && r < sp.nrestrict; ++r) {
            int e = cur[r] - in_mask(sp, r, oci) - in_mask(sp, r, ocj) + in_mask(sp, r, av) + in_mask(sp, r, bv);
            ok = e >= sp.rmin[r] && e <= sp.rmax[r];
          }
          if (ok && !(det_getocc(d, av) || det_getocc(d, bv))) {
            det_flip(cand, av);
            det_flip(cand, bv);
            det_flip(cand, oci);
            det_flip(cand, ocj);
            emit = !hash_contains(a.hslots, a.hmask, a.dets, cand);
          }
        }
        append(a, emit, cand);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// alpha <-> beta flip map. The relabelling a+_{2k} <-> a+_{2k+1} maps the
// ordered creation string of a determinant onto that of its flipped partner
// up to one transposition per doubly occupied orbital, hence the sign.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t hash_find(const uint32_t* __restrict__ slots, uint64_t mask,
                                             const Det2* __restrict__ dets, const Det2& x) {
  uint64_t h = det_hash(x) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    uint32_t s = slots[h];
    if (s == 0xffffffffu) return -1;
    if (det_eq(x, dets[s])) return (int64_t)s;
    h = (h + 1) & mask;
  }
  return -1;
}

__global__ void k_flip_map(const Det2* __restrict__ dets, size_t n, const uint32_t* __restrict__ slots, uint64_t mask,
                           int32_t* __restrict__ flip, int8_t* __restrict__ sign,
                           unsigned long long* __restrict__ missing) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const Det2 d = dets[i];
    const uint64_t a = det_alpha(d), b = det_beta(d);
    const Det2 f = det_from_strings(b, a);
    const int64_t j = hash_find(slots, mask, dets, f);
    if (j < 0) {
      atomicAdd(missing, 1ull);
      flip[i] = (int32_t)i;
    } else {
      flip[i] = (int32_t)j;
    }
    sign[i] = (__popcll(a & b) & 1) ? -1 : 1;
  }
}

bool build_flip_map(const Det2* dets, size_t n, const DetHash& hash, int32_t* flip, int8_t* sign,
                    int64_t* d_missing, cudaStream_t s) {
  SHCI_CUDA(cudaMemsetAsync(d_missing, 0, sizeof(int64_t), s));
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (blocks < 1) blocks = 1;
  k_flip_map<<<(unsigned)blocks, 256, 0, s>>>(dets, n, hash.slots.p, hash.mask, flip, sign,
                                              reinterpret_cast<unsigned long long*>(d_missing));
  SHCI_LAUNCH_CHECK();
  int64_t missing = 0;
  SHCI_CUDA(cudaMemcpyAsync(&missing, d_missing, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  return missing == 0;
}

constexpr unsigned kParBlocks = 152 * 2;

__global__ void k_flip_parity(const double* __restrict__ x, size_t n, const int32_t* __restrict__ flip,
                              const int8_t* __restrict__ sign, double* __restrict__ part) {
  __shared__ double sxy[8], sxx[8];
  double xy = 0.0, xx = 0.0;
  const size_t per = (n + gridDim.x - 1) / gridDim.x;
  const size_t r0 = (size_t)blockIdx.x * per, r1 = r0 + per < n ? r0 + per : n;
  for (size_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
    const double v = x[i];
    xy += v * (double)sign[i] * x[flip[i]];
    xx += v * v;
  }
  for (int o = 16; o; o >>= 1) {
    xy += __shfl_xor_sync(kFull, xy, o);
    xx += __shfl_xor_sync(kFull, xx, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sxy[threadIdx.x >> 5] = xy;
    sxx[threadIdx.x >> 5] = xx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += sxy[w];
      b += sxx[w];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

double flip_parity(const double* x, size_t n, const int32_t* flip, const int8_t* sign, DevBuf<double>& part,
                   cudaStream_t s) {
  part.reserve(2 * kParBlocks);
  k_flip_parity<<<kParBlocks, 256, 0, s>>>(x, n, flip, sign, part.p);
  SHCI_LAUNCH_CHECK();
  std::vector<double> h(2 * kParBlocks);
  SHCI_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  double a = 0.0, b = 0.0;
  for (unsigned k = 0; k < kParBlocks; ++k) {
    a += h[2 * k];
    b += h[2 * k + 1];
  }
  return b > 0.0 ? a / b : 0.0;
}

__global__ void k_flip_apply(const double* __restrict__ x, size_t n, const int32_t* __restrict__ flip,
                             const int8_t* __restrict__ sign, double p, double* __restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = 0.5 * (x[i] + p * (double)sign[i] * x[flip[i]]);
}

void flip_project(double* x, size_t n, const int32_t* flip, const int8_t* sign, double p, double* tmp,
                  cudaStream_t s) {
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (blocks < 1) blocks = 1;
  k_flip_apply<<<(unsigned)blocks, 256, 0, s>>>(x, n, flip, sign, p, tmp);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaMemcpyAsync(x, tmp, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
}

// ---------------------------------------------------------------------------
// Time-reversal symmetry (Treversal). The reference keeps one determinant of
// each alpha <-> beta flipped pair, the "standard" one
// (Determinant::isStandard, SHCI/Determinants.h:241-258: the larger of D and
// its flip, words compared as unsigned integers from the top word down), and
// works in the basis (D + t p(D) D~)/sqrt(2). That basis spans the flip sector
// of the determinant space that holds both members of every pair, so the
// engine keeps both, selects from the standard one as the reference does, and
// projects Davidson into the sector.
// ---------------------------------------------------------------------------
// cMax of the reference's time-reversal run (SHCI/SHCIbasics.cpp:954-965 on
// the coefficients of the symmetrized basis): for a standard determinant
// sqrt(sum over roots of c_i^2 + c_flip(i)^2) (its pair's coefficient is
// sqrt(2) times each member's), c_i alone for a closed shell; 0 for the
// flipped member, which the reference does not hold as a parent.
__global__ void k_trev_cmax(const Det2* __restrict__ dets, const double* __restrict__ ci, size_t ld, int nroots,
                            size_t n, const int32_t* __restrict__ flip, double* __restrict__ out) {
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    const Det2 d = dets[j];
    if (!det_is_standard(d)) {
      out[j] = 0.0;
      continue;
    }
    const size_t f = (size_t)flip[j];
    double s = 0.0;
    for (int r = 0; r < nroots; ++r) {
      const double c = ci[(size_t)r * ld + j];
      s = __dadd_rn(s, __dmul_rn(c, c));
      if (f != j) {
        const double cf = ci[(size_t)r * ld + f];
        s = __dadd_rn(s, __dmul_rn(cf, cf));
      }
    }
    out[j] = sqrt(s);
  }
}
void trev_cmax(const Det2* dets, const double* ci, size_t ld, int nroots, size_t n, const int32_t* flip, double* out,
               cudaStream_t s) {
  size_t blocks = std::min<size_t>((n + 255) / 256, 152 * 32);
  if (blocks < 1) blocks = 1;
  k_trev_cmax<<<(unsigned)blocks, 256, 0, s>>>(dets, ci, ld, nroots, n, flip, out);
  SHCI_LAUNCH_CHECK();
}

__global__ void k_make_standard(Det2* __restrict__ q, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (!det_is_standard(q[i])) q[i] = det_flip_pair(q[i]);
}
// flag[i] = q[i] is absent from the hash set (which == 0), or q[i] has unpaired
// electrons (which == 1)
__global__ void k_trev_flags(const Det2* __restrict__ q, size_t n, const uint32_t* __restrict__ slots,
                             uint64_t mask, const Det2* __restrict__ dets, int which, int64_t* __restrict__ flag) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const Det2 d = q[i];
    if (which == 0) {
      flag[i] = hash_contains(slots, mask, dets, d) ? 0 : 1;
    } else {
      const Det2 f = det_flip_pair(d);
      flag[i] = (f.w0 != d.w0 || f.w1 != d.w1) ? 1 : 0;
    }
  }
}
// out[pos[i]] = q[i] (or its flip) for flagged i
__global__ void k_trev_compact(const Det2* __restrict__ q, size_t n, const int64_t* __restrict__ flag,
                               const int64_t* __restrict__ pos, int flip_it, Det2* __restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (flag[i]) out[pos[i]] = flip_it ? det_flip_pair(q[i]) : q[i];
}

size_t trev_new_dets(Det2* cand, size_t n, const DetHash& present, const Det2* dets, Det2* out, DevBuf<int64_t>& flag,
                     DevBuf<int64_t>& pos, Prims& pr, cudaStream_t s) {
  if (n == 0) return 0;
  size_t blocks = std::min<size_t>((n + 255) / 256, 152 * 32);
  // the standard member of each candidate's pair (SHCI/SHCIbasics.cpp:984-987),
  // sorted and unique (:992-994), without those already present (:996-997)
  k_make_standard<<<(unsigned)blocks, 256, 0, s>>>(cand, n);
  SHCI_LAUNCH_CHECK();
  sort_dets(cand, nullptr, n, pr, s);
  n = unique_dets(cand, n, pr, s);
  blocks = std::min<size_t>((n + 255) / 256, 152 * 32);
  flag.reserve(n);
  pos.reserve(n);
  k_trev_flags<<<(unsigned)blocks, 256, 0, s>>>(cand, n, present.slots.p, present.mask, dets, 0, flag.p);
  SHCI_LAUNCH_CHECK();
  int64_t m = 0;
  scan_exclusive_i64(flag.p, pos.p, n, &m, pr, s);
  k_trev_compact<<<(unsigned)blocks, 256, 0, s>>>(cand, n, flag.p, pos.p, 0, out);
  SHCI_LAUNCH_CHECK();
  // then the flipped partners of the open-shell ones, in the same order (the
  // order in which SHCI/SHCIbasics.cpp:730-781 unpacks them)
  const size_t bm = std::max<size_t>(1, std::min<size_t>(((size_t)m + 255) / 256, 152 * 32));
  int64_t f = 0;
  if (m > 0) {
    k_trev_flags<<<(unsigned)bm, 256, 0, s>>>(out, (size_t)m, present.slots.p, present.mask, dets, 1, flag.p);
    SHCI_LAUNCH_CHECK();
    scan_exclusive_i64(flag.p, pos.p, (size_t)m, &f, pr, s);
    k_trev_compact<<<(unsigned)bm, 256, 0, s>>>(out, (size_t)m, flag.p, pos.p, 1, out + m);
    SHCI_LAUNCH_CHECK();
  }
  SHCI_CUDA(cudaStreamSynchronize(s));
  return (size_t)(m + f);
}

// How many of q[0, n) the hash set holds.
__global__ void k_count_present(const Det2* __restrict__ q, size_t n, const uint32_t* __restrict__ slots,
                                uint64_t mask, const Det2* __restrict__ dets, unsigned long long* __restrict__ cnt) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (hash_contains(slots, mask, dets, q[i])) atomicAdd(cnt, 1ull);
}

int64_t count_present(const Det2* q, size_t n, const DetHash& present, const Det2* dets, int64_t* d_counter,
                      cudaStream_t s) {
  SHCI_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(int64_t), s));
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  k_count_present<<<(unsigned)blocks, 256, 0, s>>>(q, n, present.slots.p, present.mask, dets,
                                                   reinterpret_cast<unsigned long long*>(d_counter));
  SHCI_LAUNCH_CHECK();
  int64_t total = 0;
  SHCI_CUDA(cudaMemcpyAsync(&total, d_counter, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  return total;
}

int64_t select_candidates(const Det2* dets, const double* cmax, size_t n, double eps1, const IntsView& ints,
                          const HeatBathView& hb, double maxEntry, const SelectParams& sp, const DetHash& present,
                          Det2* out, int64_t cap, int64_t* d_counter, cudaStream_t s) {
  SHCI_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(int64_t), s));
  SelArgs a{dets, cmax, n, eps1, ints, hb, maxEntry, sp, present.slots.p, present.mask, out, cap, d_counter};
  size_t blocks = (n + kSelWarps - 1) / kSelWarps;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  k_select<<<(unsigned)blocks, kSelThreads, 0, s>>>(a);
  SHCI_LAUNCH_CHECK();
  int64_t total = 0;
  SHCI_CUDA(cudaMemcpyAsync(&total, d_counter, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  return total;
}

}  // namespace shci
