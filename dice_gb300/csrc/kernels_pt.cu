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
//   k_pt_gen     one warp per parent (dynamic queue); candidates outside the
//                variational space (hash probe) in this partition are
//                appended (warp-aggregated atomics) with their numerator and
//                energy. The energy is updated from the parent's in O(1):
//                with orbital energies F_p = h_pp + sum_{q occupied} V(p, q)
//                and V the same-spin-aware Coulomb-minus-exchange, a single
//                i -> a changes E by F_a - F_i - V(a, i), a double by the
//                analogous pair terms (the reference's EnergyAfterExcitation,
//                SHCI/Determinants.cpp:124-249, sums the same terms in a loop).
//                Singles are screened in FP32 with a rigorous error bound and
//                evaluated exactly (bit-identical to the reference's FP64
//                element) only where the screen cannot decide or keeps them;
//   radix sort   of the determinants (two key words, written apart by the
//                generator) with the candidate index as payload;
//   k_pt_reduce  one thread per run of equal determinants: the numerators are
//                summed exactly in 128-bit fixed point (2^-80 units), so the
//                sum does not depend on the order the atomics left the run in,
//                E_a is the minimum over the run (the copies differ only by
//                rounding), and N^2 / (E0 - E_a) goes into fixed-grid block
//                partials summed on the host in block order.
// E2 is therefore bitwise reproducible for a given partition count.
// Candidates that do not fit in device memory are split by a hash of the
// determinant, as the reference splits them over MPI ranks
// (SHCI/SHCIbasics.cpp:519-530); each partition is generated, sorted and
// reduced alone.
#include <algorithm>
#include <cmath>
#include <random>

#include "ham.h"

namespace shci {

namespace {

constexpr int kPtThreads = 256;
constexpr int kPtWarps = kPtThreads / 32;
constexpr unsigned kPtGenBlocks = 152 * 6;
constexpr unsigned kPtRedBlocks = 152 * 4;
constexpr int kPtRedThreads = 256;
// device bytes per candidate in one partition: determinant (16), numerator (8),
// energy (8), sort payload (4), the sort's alternates (16 + 4)
constexpr size_t kPtBytesPerCand = 56;
constexpr int kFixBits = 80;  // fixed-point numerator sums in units of 2^-80

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
  // dense single-excitation integrals, A fastest so that the lanes of a warp
  // (same I, neighbouring A, the same J sequence) read contiguous addresses:
  const double* coul;   // (AI|JJ) at (I n + J) n + A (spatial)
  const double* exch;   // (AJ|JI) at (I n + J) n + A
  const float* coul32;  // the same rounded to FP32, for the screen
  const float* exch32;
  const float2* coulff;  // and as float pairs
  const float2* exchff;
  unsigned long long* next;     // parent queue
  unsigned long long* counter;  // candidates appended (counts past cap too)
  int64_t cap;
  uint64_t* key0;  // candidate determinant, low word
  uint64_t* key1;  // high word
  float4* ne;   // numerator (x + y) and E_a - E0 (z + w), both float pairs
  float2 e0;    // E0 (without the core energy) as a float pair
  // semistochastic mode (plist != null): the parents are plist[0, n) with
  // weights pw; numerators use the weight, thresholds the coefficient; n2p
  // receives the two numerators in FP64 (their difference cancels to a few
  // digits, so they are kept as the reference computes them) and ne.x the
  // flag |H| > eps2L / |c|
  const int32_t* plist;
  const double* pw;
  double eps2L;
  double nmc;  // number of draws per iteration
  double2* n2p;
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

// ---- float pairs (hi + lo, |lo| <= ulp(hi)/2): the per-candidate arithmetic
// runs on the FP32 pipe (the FP64 pipe of this part issues 2 lanes per clock
// per SM). u = 2^-24 below.
__device__ __forceinline__ float2 ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v)));
}
__device__ __forceinline__ float2 ff_fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
// error below 3 u^2 (|a| + |b|)
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  const float2 t = ff_two_sum(a.x, b.x);
  return ff_fast_two_sum(t.x, __fadd_rn(t.y, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 ff_sub(float2 a, float2 b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  const float e = __fmaf_rn(a.x, b.x, -p);
  return ff_fast_two_sum(p, __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, e)));
}
__device__ __forceinline__ float2 ff_mul_f(float a, float2 b) {
  const float p = __fmul_rn(a, b.x);
  const float e = __fmaf_rn(a, b.x, -p);
  return ff_fast_two_sum(p, __fmaf_rn(a, b.y, e));
}
__device__ __forceinline__ float2 ff_of(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ bool ff_less(float2 a, float2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }
__device__ __forceinline__ float2 shfl_ff(float2 v, int src) {
  return make_float2(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src));
}

// Warp-aggregated append of the lanes with `keep`; slots past cap are counted
// but not written.
__device__ __forceinline__ void pt_put(const PtArgs& a, bool keep, const Det2& cand, float2 v, float2 e,
                                       double2 vs = make_double2(0.0, 0.0), bool present = false) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(kFull, keep);
  if (!m) return;
  const int leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(m));
  base = __shfl_sync(kFull, base, leader);
  if (keep) {
    const unsigned long long q = base + __popc(m & ((1u << lane) - 1u));
    if (q < (unsigned long long)a.cap) {
      a.key0[q] = cand.w0;
      a.key1[q] = cand.w1;
      if (a.n2p) {
        a.ne[q] = make_float4(present ? 1.0f : 0.0f, 0.0f, e.x, e.y);
        a.n2p[q] = vs;
      } else {
        a.ne[q] = make_float4(v.x, v.y, e.x, e.y);
      }
    }
  }
}

// Hij_1Excite(a, i) of `ket` (SHCI/Determinants.cpp:437-469) with the two
// integrals of each term read from the dense tables: the same values summed
// in the same order as hij_single, so bit-identical.
__device__ __forceinline__ double hij_single_rows(const PtArgs& a, const Det2& ket, int ao, int io) {
  const int n = a.ints.norb, n2 = 2 * n;
  const size_t base = (size_t)(io >> 1) * n * n + (ao >> 1);
  double energy = __ldg(a.ints.I1 + (size_t)ao * n2 + io);
  const uint64_t same = (ao & 1) ? 0xaaaaaaaaaaaaaaaaull : 0x5555555555555555ull;
#pragma unroll 1
  for (int w = 0; w < 2; ++w) {
    uint64_t bits = w ? ket.w1 : ket.w0;
    while (bits) {
      const int j = __ffsll((long long)bits) - 1;
      const size_t t = base + (size_t)((j + 64 * w) >> 1) * n;
      const double dd = __ldg(a.coul + t);
      const double x = ((same >> j) & 1ull) ? __ldg(a.exch + t) : 0.0;
      bits &= bits - 1;
      energy = __dadd_rn(energy, __dsub_rn(dd, x));
    }
  }
  const int lo = ao < io ? ao : io, hi = ao < io ? io : ao;
  return (occ_between(ket, lo, hi) & 1) ? -energy : energy;
}

// FP32 screen of |Hij_1Excite(a, i)| against eps: returns +1 when the FP64
// element certainly exceeds eps, -1 when it certainly does not, 0 when the
// FP32 sum is too close to tell. Error bound: with S the sum of |I1_ai| and
// |d|, |x| over the m terms, the rounding of the integrals to FP32 (u per
// value), of each difference and of the running sum stays below (m + 3) u S;
// the margin used is (m + 8) 2u S, and the comparisons round against the
// decision (eps_lo <= eps <= eps_hi are its FP32 neighbours).
__device__ __forceinline__ int single_screen(const PtArgs& a, const Det2& ket, int ao, int io, float eps_lo,
                                             float eps_hi) {
  const int n = a.ints.norb, n2 = 2 * n;
  const size_t base = (size_t)(io >> 1) * n * n + (ao >> 1);
  float h = __double2float_rn(__ldg(a.ints.I1 + (size_t)ao * n2 + io));
  float S = fabsf(h);
  int m = 0;
  const uint64_t same = (ao & 1) ? 0xaaaaaaaaaaaaaaaaull : 0x5555555555555555ull;
#pragma unroll 1
  for (int w = 0; w < 2; ++w) {
    uint64_t bits = w ? ket.w1 : ket.w0;
    while (bits) {
      const int j = __ffsll((long long)bits) - 1;
      const size_t t = base + (size_t)((j + 64 * w) >> 1) * n;
      const float dd = __ldg(a.coul32 + t);
      const float x = ((same >> j) & 1ull) ? __ldg(a.exch32 + t) : 0.0f;
      bits &= bits - 1;
      h = __fadd_rn(h, __fsub_rn(dd, x));
      S = __fadd_rn(S, __fadd_rn(fabsf(dd), fabsf(x)));
      ++m;
    }
  }
  const float margin = __fmul_ru((float)(m + 8) * 1.1920928955078125e-07f, S);
  const float ah = fabsf(h);
  if (__fsub_rd(ah, margin) > eps_hi) return 1;
  if (__fadd_ru(ah, margin) < eps_lo) return -1;
  return 0;
}

// Hij_1Excite(a, i) in float pairs from the float-pair tables, with the
// decision against eps: returns +1 / -1 when |H| certainly is above / not
// above eps, 0 when FP64 must decide. Error bound: every table value carries
// u^2 relative error, every pair addition 3 u^2 (|a| + |b|), so |H_ff - H|
// stays below (7m + 8) u^2 S; the margin used is (8m + 24) u^2 (S + eps).
__device__ __forceinline__ int single_ff(const PtArgs& a, const Det2& ket, int ao, int io, float2 eps_ff,
                                         float2& H) {
  const int n = a.ints.norb, n2 = 2 * n;
  const size_t base = (size_t)(io >> 1) * n * n + (ao >> 1);
  float2 h = ff_of(__ldg(a.ints.I1 + (size_t)ao * n2 + io));
  float S = fabsf(h.x);
  int m = 0;
  const uint64_t same = (ao & 1) ? 0xaaaaaaaaaaaaaaaaull : 0x5555555555555555ull;
#pragma unroll 1
  for (int w = 0; w < 2; ++w) {
    uint64_t bits = w ? ket.w1 : ket.w0;
    while (bits) {
      const int j = __ffsll((long long)bits) - 1;
      const size_t t = base + (size_t)((j + 64 * w) >> 1) * n;
      const float2 dd = __ldg(a.coulff + t);
      bits &= bits - 1;
      if ((same >> j) & 1ull) {
        const float2 x = __ldg(a.exchff + t);
        h = ff_add(h, ff_sub(dd, x));
        S = __fadd_rn(S, __fadd_rn(fabsf(dd.x), fabsf(x.x)));
      } else {
        h = ff_add(h, dd);
        S = __fadd_rn(S, fabsf(dd.x));
      }
      ++m;
    }
  }
  const int lo = ao < io ? ao : io, hi = ao < io ? io : ao;
  if (occ_between(ket, lo, hi) & 1) h = ff_neg(h);
  H = h;
  const float2 ah = h.x < 0.0f ? ff_neg(h) : h;
  const float2 diff = ff_sub(ah, eps_ff);
  const float margin = __fmul_ru((float)(8 * m + 24) * 3.5527136788005009e-15f, __fadd_ru(S, eps_ff.x));
  if (diff.x > margin) return 1;
  if (diff.x < -margin) return -1;
  return 0;
}

// V(p, q): Coulomb (opposite spins) or Coulomb minus exchange (same spin) of
// spin orbitals p, q, from the n x n float-pair tables J and J - K staged in
// shared memory.
__device__ __forceinline__ float2 vpair(const float2* sJ, const float2* sJK, int n, int p, int q) {
  const int o = (p >> 1) * n + (q >> 1);
  return ((p ^ q) & 1) ? sJ[o] : sJK[o];
}

__global__ void __launch_bounds__(kPtThreads) k_pt_gen(PtArgs a) {
  extern __shared__ float2 smf[];
  __shared__ unsigned char s_closed[kPtWarps][kMaxSpin];
  __shared__ unsigned char s_open[kPtWarps][kMaxSpin];   // alpha holes, then beta holes
  __shared__ unsigned char s_cspin[kPtWarps][kMaxSpin];  // alpha electrons, then beta electrons
  __shared__ float2 s_F[kPtWarps][kMaxSpin];
  __shared__ uint32_t s_qo[kPtWarps][64];
  __shared__ float s_qv[kPtWarps][64];
  const int n = a.ints.norb, nn = n * n;
  float2* sD = smf;            // J
  float2* sX = smf + nn;       // J - K
  float2* sH = smf + 2 * nn;   // h_pp, spin orbitals
  for (int j = threadIdx.x; j < nn; j += blockDim.x) {
    sD[j] = ff_of(a.ints.Direct[j]);
    sX[j] = ff_of(__dsub_rn(a.ints.Direct[j], a.ints.Exchange[j]));
  }
  for (int j = threadIdx.x; j < 2 * n; j += blockDim.x) sH[j] = ff_of(a.ints.I1[(size_t)j * (2 * n + 1)]);
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned char* closed = s_closed[wib];
  unsigned char* open = s_open[wib];
  unsigned char* cspin = s_cspin[wib];
  float2* F = s_F[wib];
  const unsigned lt = (1u << lane) - 1u;
  const int n2 = 2 * n;
  const SelectParams& sp = a.sp;
  while (true) {
    unsigned long long pp = 0;
    if (lane == 0) pp = atomicAdd(a.next, 1ull);
    pp = __shfl_sync(kFull, pp, 0);
    if (pp >= (unsigned long long)a.n) break;
    const size_t p = a.plist ? (size_t)a.plist[pp] : (size_t)pp;
    const Det2 d = a.dets[p];
    const double cp = a.c[p];
    const double eps = fabs(a.eps2 / cp);
    if (!(eps < INFINITY)) continue;  // c_i = 0: nothing passes either threshold
    const float eps_lo = __double2float_rd(eps), eps_hi = __double2float_ru(eps);
    // numerator factor: c_i, or the sample weight in the semistochastic mode
    const double ci1 = a.plist ? a.pw[pp] : cp;
    const float2 eps_ff = ff_of(eps), cp_ff = ff_of(ci1);
    const bool stoch = a.plist != nullptr;
    const double epsL = stoch ? fabs(a.eps2L / cp) : INFINITY;
    const float epsL_f = __double2float_rd(epsL);
    // ci1 * Nmc / (Nmc - 1) - ci2 of getDeterminantsStochastic2Epsilon
    const double kfac = stoch ? __dsub_rn(__ddiv_rn(__dmul_rn(ci1, a.nmc), __dsub_rn(a.nmc, 1.0)), cp) : 0.0;
    // occupied list (ascending) and per-spin electron / hole lists, by ballot
    const int nclosed = __popcll(d.w0) + __popcll(d.w1);
    const int ncA = __popcll(d.w0 & 0x5555555555555555ull) + __popcll(d.w1 & 0x5555555555555555ull);
    const int nhA = n - ncA;
    __syncwarp();
    {
      int nc = 0, ea = 0, eb = 0, ha = 0, hb2 = 0;
      for (int base = 0; base < n2; base += 32) {
        const int q = base + lane;
        const bool valid = q < n2;
        const bool occ = valid && det_getocc(d, q);
        const unsigned mo = __ballot_sync(kFull, occ), mv = __ballot_sync(kFull, valid);
        const unsigned mh = mv & ~mo;
        const unsigned evn = 0x55555555u, odd = 0xaaaaaaaau;  // alpha lanes, beta lanes
        if (occ) {
          closed[nc + __popc(mo & lt)] = (unsigned char)q;
          if (q & 1)
            cspin[ncA + eb + __popc(mo & odd & lt)] = (unsigned char)q;
          else
            cspin[ea + __popc(mo & evn & lt)] = (unsigned char)q;
        } else if (valid) {
          if (q & 1)
            open[nhA + hb2 + __popc(mh & odd & lt)] = (unsigned char)q;
          else
            open[ha + __popc(mh & evn & lt)] = (unsigned char)q;
        }
        nc += __popc(mo);
        ea += __popc(mo & evn);
        eb += __popc(mo & odd);
        ha += __popc(mh & evn);
        hb2 += __popc(mh & odd);
      }
    }
    __syncwarp();
    // orbital energies F_q = h_qq + sum over occupied r of V(q, r) (V(q, q) = 0)
    // and the parent's energy relative to E0, sum_occ (h_qq + F_q) / 2 - E0
    float2 ed = make_float2(0.0f, 0.0f);
    for (int q = lane; q < n2; q += 32) {
      float2 f = make_float2(0.0f, 0.0f);
      for (int k = 0; k < nclosed; ++k) f = ff_add(f, vpair(sD, sX, n, q, closed[k]));
      const float2 hq = sH[q];
      F[q] = ff_add(hq, f);
      if (det_getocc(d, q)) {
        const float2 half = ff_add(hq, make_float2(0.5f * f.x, 0.5f * f.y));
        ed = ff_add(ed, half);
      }
    }
    for (int o = 16; o; o >>= 1) ed = ff_add(ed, make_float2(__shfl_xor_sync(kFull, ed.x, o),
                                                         __shfl_xor_sync(kFull, ed.y, o)));
    ed = ff_sub(shfl_ff(ed, 0), a.e0);  // one value for the whole warp
    __syncwarp();
    int cur[kMaxRestrict];
    for (int r = 0; r < sp.nrestrict; ++r) cur[r] = __popcll(d.w0 & sp.rmask0[r]) + __popcll(d.w1 & sp.rmask1[r]);

    // Survivors of the cheap tests wait in a per-warp ring of 64 entries and
    // are processed 32 at a time, so that the costly part (pair-arithmetic
    // element or energy, hash probe, stores) runs on full warps. Entry: the
    // orbitals i | j << 8 | a << 16 | b << 24 (j = b = 0xff for a single) and
    // the heat-bath value of a double.
    uint32_t* qo = s_qo[wib];
    float* qv = s_qv[wib];
    unsigned qh = 0, qn = 0;  // ring head and length (warp-uniform)
    auto push = [&](bool surv, uint32_t w, float val) {
      const unsigned m = __ballot_sync(kFull, surv);
      if (surv) {
        const unsigned slot = (qh + qn + __popc(m & lt)) & 63u;
        qo[slot] = w;
        qv[slot] = val;
      }
      qn += __popc(m);
      __syncwarp();
    };
    auto drain = [&](unsigned cnt) {  // the first cnt (<= 32) entries
      bool keep = false, present = false;
      Det2 cand = d;
      float2 v = make_float2(0.0f, 0.0f), e = v;
      double2 vs = make_double2(0.0, 0.0);
      if ((unsigned)lane < cnt) {
        const unsigned slot = (qh + lane) & 63u;
        const uint32_t w = qo[slot];
        const int oi = w & 0xff, oj = (w >> 8) & 0xff, oa = (w >> 16) & 0xff, ob = w >> 24;
        if (oj == 0xff) {
          // single i -> a: float pairs, then (rarely) the FP64 element
          float2 H = make_float2(0.0f, 0.0f);
          int dec = single_ff(a, d, oa, oi, eps_ff, H);
          if (dec == 0) {
            const double h = hij_single_rows(a, d, oa, oi);
            dec = fabs(h) > eps ? 1 : -1;
            H = ff_of(h);
          }
          if (dec > 0) {
            det_flip(cand, oa);
            det_flip(cand, oi);
            keep = in_part(a, cand) && !hash_contains(a.hslots, a.hmask, a.dets, cand);
            if (keep) {
              v = ff_mul(H, cp_ff);
              if (stoch) {
                // numerators as the reference forms them, from the FP64 element
                const double hd = hij_single_rows(a, d, oa, oi);
                vs = make_double2(__dmul_rn(hd, ci1), __dmul_rn(__dmul_rn(__dmul_rn(hd, hd), ci1), kfac));
                present = fabs(hd) > epsL;
              }
              e = ff_sub(ff_add(ed, ff_sub(F[oa], F[oi])), vpair(sD, sX, n, oa, oi));
            }
          }
        } else {
          // double i -> a, j -> b
          det_flip(cand, oa);
          det_flip(cand, ob);
          det_flip(cand, oi);
          det_flip(cand, oj);
          keep = in_part(a, cand) && !hash_contains(a.hslots, a.hmask, a.dets, cand);
          if (keep) {
            const float vf = qv[slot];
            v = ff_mul_f(pt_double_sign(cand, oa, ob, oi, oj) > 0.0 ? vf : -vf, cp_ff);
            if (stoch) {
              // integrals[index] * sgn * ci1 and integrals[index]^2 (a float
              // product) * ci1 * kfac, as the reference forms them
              const double sg = pt_double_sign(cand, oa, ob, oi, oj);
              const float sq = __fmul_rn(vf, vf);
              vs = make_double2(__dmul_rn(__dmul_rn((double)vf, sg), ci1),
                                __dmul_rn(__dmul_rn((double)sq, ci1), kfac));
              present = fabsf(vf) > epsL_f;  // (double)|v| > epsL exactly
            }
            const float2 fa = ff_add(F[oa], F[ob]), fi = ff_add(F[oi], F[oj]);
            const float2 vin = ff_add(vpair(sD, sX, n, oi, oj), vpair(sD, sX, n, oa, ob));
            const float2 vx = ff_add(ff_add(vpair(sD, sX, n, oa, oi), vpair(sD, sX, n, oa, oj)),
                                     ff_add(vpair(sD, sX, n, ob, oi), vpair(sD, sX, n, ob, oj)));
            e = ff_add(ed, ff_add(ff_sub(fa, fi), ff_sub(vin, vx)));
          }
        }
      }
      pt_put(a, keep, cand, v, e, vs, present);
      qh = (qh + cnt) & 63u;
      qn -= cnt;
      __syncwarp();
    };

    // ---- singles: every same-spin (i, a) (a spin flip has a zero element:
    // I1 has no alpha-beta block); FP32 screen here, the rest when drained
    const int ncB = nclosed - ncA, nhB = n - ncB;
    const int nsA = ncA * nhA, ns = nsA + ncB * nhB;
    for (int b0 = 0; b0 < ns; b0 += 32) {
      const int q = b0 + lane;
      bool surv = false;
      int ci = 0, oa = 0;
      if (q < ns) {
        if (q < nsA) {
          ci = cspin[q / nhA];
          oa = open[q % nhA];
        } else {
          ci = cspin[ncA + (q - nsA) / nhB];
          oa = open[nhA + (q - nsA) % nhB];
        }
        bool ok = true;
        for (int r = 0; ok && r < sp.nrestrict; ++r) {
          int c2 = cur[r] - in_mask(sp, r, ci) + in_mask(sp, r, oa);
          ok = c2 >= sp.rmin[r] && c2 <= sp.rmax[r];
        }
        surv = ok && single_screen(a, d, oa, ci, eps_lo, eps_hi) >= 0;
      }
      push(surv, (uint32_t)ci | 0xff00u | ((uint32_t)oa << 16) | 0xff000000u, 0.0f);
      if (qn >= 32) drain(32);
    }
    while (qn > 0) drain(qn < 32 ? qn : 32);

    // ---- doubles: heat-bath list prefixes, flattened over the warp
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
          if (fabsf(vals[mid]) < eps_f)
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
          const int c2 = lo + st;
          const int64_t e2 = __shfl_sync(kFull, excl, c2 < 32 ? c2 : 31);
          if (c2 < 32 && e2 <= f) lo = c2;
        }
        const int64_t ls = __shfl_sync(kFull, lstart, lo);
        const int64_t eo = __shfl_sync(kFull, excl, lo);
        const int oci = __shfl_sync(kFull, ci, lo);
        const int ocj = __shfl_sync(kFull, cj, lo);
        const bool osame = __shfl_sync(kFull, (int)same, lo) != 0;
        bool surv = false;
        uint32_t w = 0;
        float vf = 0.0f;
        if (f < total) {
          const int64_t index = ls + (f - eo);
          const int16_t* pr = osame ? a.hb.samePairs : a.hb.oppPairs;
          const int av = 2 * pr[2 * index] + (oci & 1);
          const int bv = 2 * pr[2 * index + 1] + (ocj & 1);
          bool ok = true;
          for (int r = 0; ok && r < sp.nrestrict; ++r) {
            int c2 = cur[r] - in_mask(sp, r, oci) - in_mask(sp, r, ocj) + in_mask(sp, r, av) + in_mask(sp, r, bv);
            ok = c2 >= sp.rmin[r] && c2 <= sp.rmax[r];
          }
          surv = ok && !(det_getocc(d, av) || det_getocc(d, bv));
          if (surv) {
            w = (uint32_t)oci | ((uint32_t)ocj << 8) | ((uint32_t)av << 16) | ((uint32_t)bv << 24);
            vf = (osame ? a.hb.sameVal : a.hb.oppVal)[index];
          }
        }
        push(surv, w, vf);
        if (qn >= 32) drain(32);
      }
    }
    while (qn > 0) drain(qn < 32 ? qn : 32);
  }
}

__global__ void k_pt_tables(const double* __restrict__ I2, int n, double* __restrict__ coul,
                            double* __restrict__ exch, float* __restrict__ coul32, float* __restrict__ exch32,
                            float2* __restrict__ coulff, float2* __restrict__ exchff) {
  const size_t nt = (size_t)n * n * n;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (size_t)gridDim.x * blockDim.x) {
    const int A = (int)(t % n), J = (int)((t / n) % n), I = (int)(t / ((size_t)n * n));
    const double c = i2_spatial(I2, A, I, J, J), x = i2_spatial(I2, A, J, J, I);
    coul[t] = c;
    exch[t] = x;
    coul32[t] = (float)c;
    exch32[t] = (float)x;
    coulff[t] = ff_of(c);
    exchff[t] = ff_of(x);
  }
}

__global__ void k_pt_iota(uint32_t* __restrict__ p, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = (uint32_t)i;
}

// x in units of 2^-kFixBits, truncated toward zero (|x| < 2^47).
__device__ __forceinline__ __int128 to_fix(float x) {
  const unsigned b = __float_as_uint(x);
  const int ex = (int)((b >> 23) & 0xff);
  if (ex == 0) return 0;  // zero or subnormal: below the unit
  const unsigned long long m = (b & 0x7fffffu) | 0x800000u;
  const int sh = ex - 150 + kFixBits;
  unsigned __int128 v = 0;
  if (sh >= 0)
    v = (unsigned __int128)m << (sh < 103 ? sh : 103);
  else if (sh > -32)
    v = m >> (-sh);
  return (b >> 31) ? -(__int128)v : (__int128)v;
}
// a float pair exactly (up to the 2^-kFixBits truncation of each part)
__device__ __forceinline__ __int128 to_fix(float2 x) { return to_fix(x.x) + to_fix(x.y); }
// a double (|x| < 2^47), truncated toward zero to the unit
__device__ __forceinline__ __int128 to_fix(double x) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0) return 0;
  const unsigned long long m = ((unsigned long long)b & 0xfffffffffffffull) | (1ull << 52);
  const int sh = ex - 1075 + kFixBits;
  unsigned __int128 v = 0;
  if (sh >= 0)
    v = (unsigned __int128)m << (sh < 74 ? sh : 74);
  else if (sh > -64)
    v = m >> (-sh);
  return b < 0 ? -(__int128)v : (__int128)v;
}

__device__ __forceinline__ double from_fix(__int128 v) {
  const bool neg = v < 0;
  const unsigned __int128 m = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const double d = (double)(unsigned long long)(m >> 64) * 18446744073709551616.0 + (double)(unsigned long long)m;
  return (neg ? -d : d) * 8.271806125530276748714086920699e-25;  // 2^-80
}

// Runs of equal determinants in the sorted candidates, reduced by warps: a
// warp owns the runs whose first element lies in its tile of kPtRedTile
// positions and walks them 32 positions at a time (following the last owned
// run past the tile end). All loads of a round are independent (keys and
// payload in order, numerators and energies gathered), and a segmented
// inclusive scan over the lanes sums the fixed-point numerators and takes
// the minimum energy per run; the lane at a run's end adds its term. Block
// partials {E2, |psi1|^2, count} go to part[3 * block].
constexpr int kPtRedTile = 256;

__device__ __forceinline__ __int128 shfl_up_i128(__int128 v, int o) {
  const unsigned long long lo = __shfl_up_sync(kFull, (unsigned long long)v, o);
  const long long hi = __shfl_up_sync(kFull, (long long)(v >> 64), o);
  return (__int128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}
__device__ __forceinline__ __int128 shfl_i128(__int128 v, int src) {
  const unsigned long long lo = __shfl_sync(kFull, (unsigned long long)v, src);
  const long long hi = __shfl_sync(kFull, (long long)(v >> 64), src);
  return (__int128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}

__global__ void __launch_bounds__(kPtRedThreads) k_pt_reduce(const uint64_t* __restrict__ k0,
                                                             const uint64_t* __restrict__ k1,
                                                             const uint32_t* __restrict__ perm,
                                                             const float4* __restrict__ ne, size_t m,
                                                             double* __restrict__ part) {
  const int lane = threadIdx.x & 31;
  const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  double e2 = 0.0, psi = 0.0, cnt = 0.0;
  __shared__ unsigned long long s_qlo[kPtRedThreads / 32][64];
  __shared__ long long s_qhi[kPtRedThreads / 32][64];
  __shared__ float2 s_qe[kPtRedThreads / 32][64];
  unsigned long long* qlo = s_qlo[threadIdx.x >> 5];
  long long* qhi = s_qhi[threadIdx.x >> 5];
  float2* qe = s_qe[threadIdx.x >> 5];
  unsigned qh = 0, qn = 0;  // finished runs waiting (warp-uniform)
  const unsigned lt = (1u << lane) - 1u;
  auto flush = [&](unsigned c) {
    if ((unsigned)lane < c) {
      const unsigned slot = (qh + lane) & 63u;
      const __int128 v = (__int128)(((unsigned __int128)(unsigned long long)qhi[slot] << 64) | qlo[slot]);
      const float2 e = qe[slot];
      const double sn = from_fix(v);
      const double inv = 1.0 / -((double)e.x + (double)e.y);  // 1 / (E0 - E_a)
      const double t = sn * inv;
      e2 += sn * t;
      psi += t * t;
      cnt += 1.0;
    }
    qh = (qh + c) & 63u;
    qn -= c;
    __syncwarp();
  };
  // head flag of position q (first of its run)
  auto is_head = [&](size_t q) -> bool {
    return q == 0 || k0[q] != k0[q - 1] || k1[q] != k1[q - 1];
  };
  for (size_t t0 = warp * kPtRedTile; t0 < m; t0 += nwarps * kPtRedTile) {
    const size_t t1 = t0 + kPtRedTile < m ? t0 + kPtRedTile : m;
    // first head at or after t0, inside the tile
    size_t b = t0;
    bool found = false;
    for (; b < t1; b += 32) {
      const size_t q = b + lane;
      const unsigned hm = __ballot_sync(kFull, q < t1 && is_head(q));
      if (hm) {
        b += __ffs(hm) - 1;
        found = true;
        break;
      }
    }
    if (!found) continue;
    __int128 cs = 0;     // open run carried from the previous round
    float2 ce = make_float2(INFINITY, 0.0f);
    size_t chead = b;
    bool open = false;
    for (; b < m; b += 32) {
      if (b >= t1 && !(open && chead < t1)) break;
      const size_t q = b + lane;
      const bool valid = q < m;
      bool head = false;
      __int128 v = 0;
      float2 e = make_float2(INFINITY, 0.0f);
      if (valid) {
        head = (lane == 0) ? !open : is_head(q);
        const uint32_t pk = perm[q];
        const float4 x = ne[pk];
        v = to_fix(make_float2(x.x, x.y));
        e = make_float2(x.z, x.w);
      }
      // the run open at the end of the last round continues in lane 0's segment
      if (lane == 0 && open && !head) {
        v += cs;
        if (ff_less(ce, e)) e = ce;
      }
      size_t hp = head ? q : 0;
      bool f = head;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const __int128 nv = shfl_up_i128(v, o);
        const float2 ne = make_float2(__shfl_up_sync(kFull, e.x, o), __shfl_up_sync(kFull, e.y, o));
        const bool nf = __shfl_up_sync(kFull, (int)f, o) != 0;
        const size_t nh = __shfl_up_sync(kFull, (unsigned long long)hp, o);
        if (lane >= o) {
          if (!f) {
            v += nv;
            if (ff_less(ne, e)) e = ne;
          }
          f = f || nf;
          hp = hp > nh ? hp : nh;
        }
      }
      if (!f) hp = chead;  // lanes before the first head of the round
      // does the run of this lane end here? (next position is a head or past the end)
      bool next_head = __shfl_down_sync(kFull, (int)head, 1) != 0;
      if (lane == 31) next_head = (q + 1 >= m) || is_head(q + 1);
      // a finished run waits in the warp's queue, evaluated 32 at a time
      // (the FP64 tail costs a full-warp issue however few lanes take part)
      const bool fin = valid && (q + 1 >= m || next_head) && hp < t1;
      const unsigned fm = __ballot_sync(kFull, fin);
      if (fin) {
        const unsigned slot = (qh + qn + __popc(fm & lt)) & 63u;
        qlo[slot] = (unsigned long long)v;
        qhi[slot] = (long long)(v >> 64);
        qe[slot] = e;
      }
      qn += __popc(fm);
      __syncwarp();
      if (qn >= 32) flush(32);
      // carry lane 31's run when it continues into the next round
      const bool cont = __shfl_sync(kFull, (int)(valid && !(q + 1 >= m || next_head)), 31) != 0;
      cs = shfl_i128(v, 31);
      ce = shfl_ff(e, 31);
      chead = __shfl_sync(kFull, (unsigned long long)hp, 31);
      open = cont;
      if (!open && b + 32 >= t1) break;
    }
  }
  while (qn > 0) flush(qn < 32 ? qn : 32);
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

// Semistochastic estimate over the sorted candidates of one iteration, one
// thread per run of equal determinants: with S1, S2 the sums of the two
// numerators (and S1B, S2B over the contributions flagged as already held by
// the deterministic part), eA = sum (S1^2 f - S2) / (E_a - E0) and eB likewise
// (SHCI/SHCIbasics.cpp:271-363). Sums in fixed point as in k_pt_reduce; block
// partials {eA, eB, runs} in part[3 * block].
__global__ void __launch_bounds__(kPtRedThreads) k_pt_reduce_stoch(const uint64_t* __restrict__ k0,
                                                                   const uint64_t* __restrict__ k1,
                                                                   const uint32_t* __restrict__ perm,
                                                                   const float4* __restrict__ ne,
                                                                   const double2* __restrict__ n2p, size_t m, double f,
                                                                   double* __restrict__ part) {
  double eA = 0.0, eB = 0.0, cnt = 0.0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (size_t)gridDim.x * blockDim.x) {
    const uint64_t d0 = k0[k], d1 = k1[k];
    if (k > 0 && d0 == k0[k - 1] && d1 == k1[k - 1]) continue;
    __int128 s1 = 0, s2 = 0, s1b = 0, s2b = 0;
    float2 e = make_float2(INFINITY, 0.0f);
    for (size_t j = k; j < m; ++j) {
      if (j > k && (k0[j] != d0 || k1[j] != d1)) break;
      const uint32_t pk = perm[j];
      const float4 x = ne[pk];
      const double2 y = n2p[pk];
      const __int128 f1 = to_fix(y.x), f2 = to_fix(y.y);
      s1 += f1;
      s2 += f2;
      if (x.x != 0.0f) {
        s1b += f1;
        s2b += f2;
      }
      const float2 ej = make_float2(x.z, x.w);
      if (ff_less(ej, e)) e = ej;
    }
    const double de = (double)e.x + (double)e.y;  // E_a - E0
    const double n1 = from_fix(s1), n1b = from_fix(s1b);
    eA += (n1 * n1 * f - from_fix(s2)) / de;
    eB += (n1b * n1b * f - from_fix(s2b)) / de;
    cnt += 1.0;
  }
  __shared__ double r0[kPtRedThreads / 32], r1[kPtRedThreads / 32], r2[kPtRedThreads / 32];
  for (int o = 16; o; o >>= 1) {
    eA += __shfl_xor_sync(kFull, eA, o);
    eB += __shfl_xor_sync(kFull, eB, o);
    cnt += __shfl_xor_sync(kFull, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r0[threadIdx.x >> 5] = eA;
    r1[threadIdx.x >> 5] = eB;
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

namespace {

// Fields of PtArgs shared by both modes; builds the dense integral tables on
// first use. Returns the generator's dynamic shared memory size.
size_t pt_prepare(PtArgs& a, const Det2* dets, size_t n, const double* c, double E0, double eps2,
                  const IntsView& ints, const HeatBathView& hb, double maxEntry, const SelectParams& sp,
                  const DetHash& present, PtWork& w, cudaStream_t s) {
  w.next.resize(2);
  w.part.resize(3 * kPtRedBlocks);
  a = PtArgs{};
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
  a.counter = w.next.p + 1;
  a.nparts = 1;
  if (w.tables_of != ints.I2 || w.tables_n != ints.norb) {
    const size_t nt = (size_t)ints.norb * ints.norb * ints.norb;
    w.coul.resize(nt);
    w.exch.resize(nt);
    w.coul32.resize(nt);
    w.exch32.resize(nt);
    w.coulff.resize(nt);
    w.exchff.resize(nt);
    k_pt_tables<<<grid_for(nt, 256), 256, 0, s>>>(ints.I2, ints.norb, w.coul.p, w.exch.p, w.coul32.p, w.exch32.p,
                                                   w.coulff.p, w.exchff.p);
    SHCI_LAUNCH_CHECK();
    w.tables_of = ints.I2;
    w.tables_n = ints.norb;
  }
  a.coul = w.coul.p;
  a.exch = w.exch.p;
  a.coul32 = w.coul32.p;
  a.exch32 = w.exch32.p;
  a.coulff = w.coulff.p;
  a.exchff = w.exchff.p;
  {
    const float h = (float)E0;
    a.e0 = make_float2(h, (float)(E0 - (double)h));
  }
  const size_t gsmem = sizeof(float2) * (2 * ints.norb * ints.norb + 2 * ints.norb);
  SHCI_CUDA(cudaFuncSetAttribute(k_pt_gen, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsmem));
  return gsmem;
}

}  // namespace

PtResult pt_deterministic(const Det2* dets, size_t n, const double* c, double E0, double eps2, const IntsView& ints,
                          const HeatBathView& hb, double maxEntry, const SelectParams& sp, const DetHash& present,
                          int64_t max_candidates, PtWork& w, Prims& pr, cudaStream_t s) {
  PtResult res;
  if (n == 0) return res;
  if (!(eps2 >= 0.0)) throw Error(kErrInvalid, "epsilon2 must be >= 0");
  PtArgs a;
  const size_t gsmem = pt_prepare(a, dets, n, c, E0, eps2, ints, hb, maxEntry, sp, present, w, s);

  // capacity of one partition
  int64_t cap = max_candidates;
  if (cap <= 0) {
    size_t fr = 0, tot = 0;
    release_pool_memory(s);  // freed buffers held for reuse count as free
    SHCI_CUDA(cudaMemGetInfo(&fr, &tot));
    size_t avail = fr;
    if (g_alloc_cap) avail = std::min(avail, g_alloc_cap > g_alloc_live ? g_alloc_cap - g_alloc_live : (size_t)0);
    // what the buffers already hold counts as available to them
    avail += (w.key0.cap + w.key1.cap) * sizeof(uint64_t) + w.ne.cap * sizeof(float4) +
             w.perm.cap * sizeof(uint32_t);
    cap = (int64_t)(avail / 4 * 3 / kPtBytesPerCand);
  }
  cap = std::min<int64_t>(cap, (int64_t)0xfffffff0u);
  if (cap < 1) throw Error(kErrOOM, "no device memory left for perturbation candidates");

  // one generation pass into buffers of `room` candidates; returns the count
  auto gen = [&](uint32_t nparts, uint32_t part, int64_t room) -> int64_t {
    w.key0.reserve((size_t)room);
    w.key1.reserve((size_t)room);
    w.ne.reserve((size_t)room);
    a.nparts = nparts;
    a.part = part;
    a.cap = room;
    a.key0 = w.key0.p;
    a.key1 = w.key1.p;
    a.ne = w.ne.p;
    SHCI_CUDA(cudaMemsetAsync(w.next.p, 0, 2 * sizeof(unsigned long long), s));
    k_pt_gen<<<kPtGenBlocks, kPtThreads, gsmem, s>>>(a);
    SHCI_LAUNCH_CHECK();
    unsigned long long total = 0;
    SHCI_CUDA(cudaMemcpyAsync(&total, w.next.p + 1, sizeof(total), cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    return (int64_t)total;
  };
  PhaseTimer pt(s);
  auto reduce = [&](int64_t m, PtResult& r) {
    w.perm.resize((size_t)m);
    k_pt_iota<<<grid_for((size_t)m, 256), 256, 0, s>>>(w.perm.p, (size_t)m);
    SHCI_LAUNCH_CHECK();
    sort_u128(w.key0.p, w.key1.p, w.perm.p, (size_t)m, pr, s);
    pt.mark("pt sort");
    k_pt_reduce<<<kPtRedBlocks, kPtRedThreads, 0, s>>>(w.key0.p, w.key1.p, w.perm.p, w.ne.p, (size_t)m,
                                                       w.part.p);
    SHCI_LAUNCH_CHECK();
    std::vector<double> hp(3 * kPtRedBlocks);
    SHCI_CUDA(cudaMemcpyAsync(hp.data(), w.part.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    SHCI_CUDA(cudaStreamSynchronize(s));
    for (unsigned b = 0; b < kPtRedBlocks; ++b) {
      r.e2 += hp[3 * b];
      r.psi1_norm += hp[3 * b + 1];
      r.unique += (int64_t)hp[3 * b + 2];
    }
  };

  // first pass into what the buffers hold (at least 64 per parent, at most cap)
  int64_t room = std::min<int64_t>(cap, std::max<int64_t>((int64_t)w.key0.cap, 64 * (int64_t)n));
  int64_t total = gen(1, 0, room);
  pt.mark("pt generate");
  if (total <= cap) {
    if (total > room) {  // buffers too small: regenerate into exact room
      gen(1, 0, total);
      pt.mark("pt regenerate");
    }
    res.partitions = 1;
    res.candidates = total;
    if (total > 0) reduce(total, res);
    pt.mark("pt reduce");
    return res;
  }
  // split by hash; a partition that still overflows doubles the count
  uint32_t nparts = (uint32_t)((total + total / 8) / cap + 1);
  for (int attempt = 0;; ++attempt) {
    res = PtResult();
    res.partitions = (int)nparts;
    bool overflow = false;
    for (uint32_t part = 0; part < nparts && !overflow; ++part) {
      const int64_t m = gen(nparts, part, cap);
      if (m > cap) {
        overflow = true;
        break;
      }
      res.candidates += m;
      if (m > 0) reduce(m, res);
    }
    if (!overflow) break;
    if (attempt >= 8) throw Error(kErrOOM, "perturbation candidates do not fit in device memory");
    nparts *= 2;
  }
  pt.mark("pt partitions");
  return res;
}

// SHCIsampledeterminants::setUpAliasMethod (SHCI/SHCIsampledeterminants.cpp:64-88).
static void alias_setup(const std::vector<double>& ci, double cumulative, std::vector<int>& alias,
                        std::vector<double>& prob) {
  const size_t N = ci.size();
  alias.assign(N, 0);
  prob.assign(N, 0.0);
  std::vector<int> larger, smaller;
  for (size_t i = 0; i < N; i++) {
    prob[i] = fabs(ci[i]) * N / cumulative;
    if (prob[i] < 1.0)
      smaller.push_back((int)i);
    else
      larger.push_back((int)i);
  }
  while (!larger.empty() && !smaller.empty()) {
    const int l = larger.back();
    larger.pop_back();
    const int sm = smaller.back();
    smaller.pop_back();
    alias[sm] = l;
    prob[l] = prob[l] - (1.0 - prob[sm]);
    if (prob[l] < 1.0)
      smaller.push_back(l);
    else
      larger.push_back(l);
  }
}

PtStochResult pt_semistochastic(const Det2* dets, size_t n, const double* c_dev, const std::vector<double>& c_host,
                                double E0, double eps2, double eps2L, int nsample, int max_iter, double target,
                                uint64_t seed, const IntsView& ints, const HeatBathView& hb, double maxEntry,
                                const SelectParams& sp, const DetHash& present, PtWork& w, Prims& pr,
                                cudaStream_t s) {
  PtStochResult res;
  if (n == 0) return res;
  if (!(eps2 >= 0.0)) throw Error(kErrInvalid, "epsilon2 must be >= 0");
  if (nsample < 2) throw Error(kErrInvalid, "sampleN must be at least 2");
  if (max_iter < 1) throw Error(kErrInvalid, "nPTiter must be at least 1");
  if (eps2L < 999) res.e_large = pt_deterministic(dets, n, c_dev, E0, eps2L, ints, hb, maxEntry, sp, present, 0, w,
                                                  pr, s).e2;
  double cumulative = 0.0;
  for (size_t i = 0; i < n; i++) cumulative += fabs(c_host[i]);
  std::vector<int> alias;
  std::vector<double> prob;
  alias_setup(c_host, cumulative, alias, prob);
  PtArgs a;
  const size_t gsmem = pt_prepare(a, dets, n, c_dev, E0, eps2, ints, hb, maxEntry, sp, present, w, s);
  a.eps2L = eps2L;
  a.nmc = (double)nsample;
  DevBuf<int32_t> dlist;
  DevBuf<double> dw;
  dlist.resize((size_t)nsample);
  dw.resize((size_t)nsample);
  // uniform [0, 1) from a 64-bit Mersenne twister (the reference draws
  // rand() / RAND_MAX; any uniform stream gives the same estimator)
  std::mt19937_64 g(seed);
  auto next = [&]() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); };
  std::vector<int32_t> sample((size_t)nsample);
  std::vector<double> wts((size_t)nsample);
  std::vector<double> hp(3 * kPtRedBlocks);
  const double f = (double)nsample / (nsample - 1);
  double avg = 0.0, avg2 = 0.0;
  for (int iter = 0; iter < max_iter; ++iter) {
    // SHCIsampledeterminants::sample_N2_alias (SHCI/SHCIsampledeterminants.cpp:153-190)
    std::fill(sample.begin(), sample.end(), -1);
    std::fill(wts.begin(), wts.end(), 0.0);
    int distinct = 0;
    for (int k = 0; k < nsample; k++) {
      int det = (int)floor(next() * n);
      if (next() >= prob[det]) det = alias[det];
      int at = -1;
      for (int q = 0; q < distinct; ++q)
        if (sample[q] == det) {
          at = q;
          break;
        }
      const double wgt = cumulative * c_host[det] / fabs(c_host[det]);
      if (at < 0) {
        sample[distinct] = det;
        wts[distinct] = wgt;
        distinct++;
      } else {
        wts[at] += wgt;
      }
    }
    for (int k = 0; k < nsample; k++) wts[k] /= nsample;
    SHCI_CUDA(cudaMemcpyAsync(dlist.p, sample.data(), distinct * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    SHCI_CUDA(cudaMemcpyAsync(dw.p, wts.data(), distinct * sizeof(double), cudaMemcpyHostToDevice, s));
    a.plist = dlist.p;
    a.pw = dw.p;
    a.n = (size_t)distinct;
    // generate (twice when the buffers turn out too small)
    int64_t room = std::max<int64_t>((int64_t)w.key0.cap, (int64_t)1 << 20), m = 0;
    for (int pass = 0; pass < 2; ++pass) {
      w.key0.reserve((size_t)room);
      w.key1.reserve((size_t)room);
      w.ne.reserve((size_t)room);
      w.n2p.reserve((size_t)room);
      a.cap = room;
      a.key0 = w.key0.p;
      a.key1 = w.key1.p;
      a.ne = w.ne.p;
      a.n2p = w.n2p.p;
      SHCI_CUDA(cudaMemsetAsync(w.next.p, 0, 2 * sizeof(unsigned long long), s));
      k_pt_gen<<<kPtGenBlocks, kPtThreads, gsmem, s>>>(a);
      SHCI_LAUNCH_CHECK();
      unsigned long long total = 0;
      SHCI_CUDA(cudaMemcpyAsync(&total, w.next.p + 1, sizeof(total), cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
      m = (int64_t)total;
      if (m <= room) break;
      if (m >= (int64_t)0xfffffff0u) throw Error(kErrOOM, "semistochastic sample exceeds 2^32 candidates");
      room = m;
    }
    res.candidates += m;
    double eA = 0.0, eB = 0.0;
    if (m > 0) {
      w.perm.resize((size_t)m);
      k_pt_iota<<<grid_for((size_t)m, 256), 256, 0, s>>>(w.perm.p, (size_t)m);
      SHCI_LAUNCH_CHECK();
      sort_u128(w.key0.p, w.key1.p, w.perm.p, (size_t)m, pr, s);
      k_pt_reduce_stoch<<<kPtRedBlocks, kPtRedThreads, 0, s>>>(w.key0.p, w.key1.p, w.perm.p, w.ne.p, w.n2p.p,
                                                               (size_t)m, f, w.part.p);
      SHCI_LAUNCH_CHECK();
      SHCI_CUDA(cudaMemcpyAsync(hp.data(), w.part.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
      SHCI_CUDA(cudaStreamSynchronize(s));
      for (unsigned b = 0; b < kPtRedBlocks; ++b) {
        eA += hp[3 * b];
        eB += hp[3 * b + 1];
      }
    }
    // SHCI/SHCIbasics.cpp:388-449
    const double est = -eA + eB + res.e_large;
    avg += est;
    avg2 += est * est;
    const int it = iter + 1;
    res.iterations = it;
    res.stddev = it < 5 ? 1e4 : pow((it * avg2 - pow(avg, 2)) / it / (it - 1) / it, 0.5);
    if (res.stddev < target) break;
  }
  res.e2 = avg / res.iterations;
  return res;
}

}  // namespace shci
