// Spatial 1- and 2-RDMs of the variational wavefunction.
//
// Restates SHCIrdm::EvaluateRDM (SHCI/SHCIrdm.cpp:863-993) and
// SHCIrdm::EvaluateOneRDM (:996-1100) with cibra = ciket = c, over the
// connection lists of the stored Hamiltonian (every connected pair J < I of
// the variational space, the pairs the reference's build stores with their
// orbital differences, SHCI/SHCImakeHamiltonian.cpp:578-588):
//   diagonal  every occupied pair of every determinant, weight c_I^2;
//   single    J = I with d -> c: the 1-RDM pair (c, d) and, for every other
//             occupied spectator k of I, the 2-RDM elements of
//             populateSpatialRDM (:846-861), sign of the transposition times
//             -1 when k lies between c and d;
//   double    the two 2-RDM elements of the excitation, sign of
//             Determinant::parity(d1, d0, c1, c0) (SHCI/Determinants.cpp:332-357).
// The sums are kept in 64-bit fixed point (units of 2^-58, elements are
// bounded by 4 in magnitude) and added with integer atomics, so the result
// does not depend on the order of the additions and is bitwise reproducible;
// each term is rounded to the unit (2^-59 error per term).
//
//   k_rdm_diag  thread per determinant; the diagonal elements ((IJ, IJ) and
//               (IJ, JI)) and the 1-RDM diagonal accumulate in shared memory
//               per block, then once per block into the global sums;
//   k_rdm_off   warp per row, lanes over the row's connections J < I (rows
//               and columns in the stored Hamiltonian's storage order: each
//               connected pair is visited once, and its terms are symmetric
//               in the two determinants, so the order does not change the
//               sums);
//   k_rdm_fin   fixed point -> FP64.
#include "ham.h"

namespace shci {

namespace {

constexpr double kRdmUnit = 288230376151711744.0;  // 2^58
constexpr int kRdmThreads = 256;

inline unsigned grid_for(size_t n, int threads, size_t max_blocks = 152 * 32) {
  size_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (unsigned)b;
}

__device__ __forceinline__ void add_fix(unsigned long long* p, long long v) {
  atomicAdd(p, (unsigned long long)v);
}

// populateSpatialRDM(i, j, k, l, v) (SHCI/SHCIrdm.cpp:846-861) on the n^2 x n^2
// matrix s2, element (I n + J, K n + L) at (I n + J) n^2 + K n + L.
__device__ __forceinline__ void pop2(unsigned long long* s2, int n, int i, int j, int k, int l, long long v) {
  const size_t n2 = (size_t)n * n;
  const int I = i >> 1, J = j >> 1, K = k >> 1, L = l >> 1;
  if (((i ^ l) & 1) == 0 && ((j ^ k) & 1) == 0) {
    add_fix(s2 + (size_t)(I * n + J) * n2 + L * n + K, -v);
    add_fix(s2 + (size_t)(J * n + I) * n2 + K * n + L, -v);
  }
  if (((i ^ k) & 1) == 0 && ((l ^ j) & 1) == 0) {
    add_fix(s2 + (size_t)(I * n + J) * n2 + K * n + L, v);
    add_fix(s2 + (size_t)(J * n + I) * n2 + L * n + K, v);
  }
}

__global__ void __launch_bounds__(kRdmThreads) k_rdm_diag(const Det2* __restrict__ dets,
                                                          const double* __restrict__ c, size_t N, int n,
                                                          unsigned long long* __restrict__ s2,
                                                          unsigned long long* __restrict__ s1) {
  extern __shared__ unsigned long long sm[];
  const int nn = n * n;
  unsigned long long* dd = sm;            // (IJ, IJ)
  unsigned long long* dx = sm + nn;       // (IJ, JI)
  unsigned long long* d1 = sm + 2 * nn;   // 1-RDM (I, I)
  for (int t = threadIdx.x; t < 2 * nn + n; t += blockDim.x) sm[t] = 0ull;
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
    const Det2 d = dets[i];
    const long long v = __double2ll_rn(c[i] * c[i] * kRdmUnit);
    // occupied pairs orb1 > orb2: populateSpatialRDM(orb1, orb2, orb1, orb2)
    for (int w1 = 0; w1 < 2; ++w1) {
      uint64_t b1 = w1 ? d.w1 : d.w0;
      while (b1) {
        const int o1 = __ffsll((long long)b1) - 1 + 64 * w1;
        b1 &= b1 - 1;
        const int I = o1 >> 1;
        atomicAdd(&d1[I], (unsigned long long)v);
        for (int w2 = 0; w2 <= w1; ++w2) {
          uint64_t b2 = w2 ? d.w1 : d.w0;
          if (w2 == w1) b2 &= (o1 & 63) ? ((1ull << (o1 & 63)) - 1ull) : 0ull;  // o2 < o1
          while (b2) {
            const int o2 = __ffsll((long long)b2) - 1 + 64 * w2;
            b2 &= b2 - 1;
            const int J = o2 >> 1;
            if (((o1 ^ o2) & 1) == 0) {
              atomicAdd(&dx[I * n + J], (unsigned long long)(-v));
              atomicAdd(&dx[J * n + I], (unsigned long long)(-v));
            }
            atomicAdd(&dd[I * n + J], (unsigned long long)v);
            atomicAdd(&dd[J * n + I], (unsigned long long)v);
          }
        }
      }
    }
  }
  __syncthreads();
  const size_t n2 = (size_t)nn;
  for (int t = threadIdx.x; t < nn; t += blockDim.x) {
    const int I = t / n, J = t % n;
    if (dd[t]) atomicAdd(s2 + (size_t)(I * n + J) * n2 + I * n + J, dd[t]);
    if (dx[t]) atomicAdd(s2 + (size_t)(I * n + J) * n2 + J * n + I, dx[t]);
  }
  for (int t = threadIdx.x; t < n; t += blockDim.x)
    if (d1[t]) atomicAdd(s1 + (size_t)t * n + t, d1[t]);
}

__global__ void __launch_bounds__(kRdmThreads) k_rdm_off(const Det2* __restrict__ dets,
                                                         const double* __restrict__ c, size_t N,
                                                         const int64_t* __restrict__ rowptr,
                                                         const int32_t* __restrict__ col,
                                                         const uint32_t* __restrict__ perm, int n,
                                                         unsigned long long* __restrict__ s2,
                                                         unsigned long long* __restrict__ s1) {
  const int lane = threadIdx.x & 31;
  const size_t warps = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t I = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < N; I += warps) {
    const uint32_t dI = perm[I];
    const Det2 di = dets[dI];
    const double cI = c[dI];
    const int64_t p0 = rowptr[I], p1 = rowptr[I + 1];
    for (int64_t p = p0 + lane; p < p1; p += 32) {
      const int J = col[p];
      if ((size_t)J >= I) continue;
      const uint32_t dJ = perm[J];
      const Det2 dj = dets[dJ];
      // created: in J only; destroyed: in I only (getOrbDiff(Dets[J], Dets[I]))
      const uint64_t cr0 = dj.w0 & ~di.w0, cr1 = dj.w1 & ~di.w1;
      const uint64_t de0 = di.w0 & ~dj.w0, de1 = di.w1 & ~dj.w1;
      const int ncre = __popcll(cr0) + __popcll(cr1);
      const long long v = __double2ll_rn(c[dJ] * cI * kRdmUnit);
      int cre[2], des[2];
      {
        int k = 0;
        for (uint64_t b = cr0; b && k < 2; b &= b - 1) cre[k++] = __ffsll((long long)b) - 1;
        for (uint64_t b = cr1; b && k < 2; b &= b - 1) cre[k++] = __ffsll((long long)b) - 1 + 64;
        k = 0;
        for (uint64_t b = de0; b && k < 2; b &= b - 1) des[k++] = __ffsll((long long)b) - 1;
        for (uint64_t b = de1; b && k < 2; b &= b - 1) des[k++] = __ffsll((long long)b) - 1 + 64;
      }
      if (ncre == 1) {
        const int c0 = cre[0], d0 = des[0];
        const int lo = c0 < d0 ? c0 : d0, hi = c0 < d0 ? d0 : c0;
        const long long v0 = (occ_between(di, lo, hi) & 1) ? -v : v;
        add_fix(s1 + (size_t)(c0 >> 1) * n + (d0 >> 1), v0);
        add_fix(s1 + (size_t)(d0 >> 1) * n + (c0 >> 1), v0);
        for (int w = 0; w < 2; ++w) {
          uint64_t bits = w ? di.w1 : di.w0;
          while (bits) {
            const int k = __ffsll((long long)bits) - 1 + 64 * w;
            bits &= bits - 1;
            if (k == d0) continue;
            const long long vk = (k > lo && k < hi) ? -v0 : v0;
            const int a = k > c0 ? k : c0, b = k > c0 ? c0 : k;
            const int II = k > d0 ? k : d0, JJ = k > d0 ? d0 : k;
            pop2(s2, n, a, b, II, JJ, vk);
            pop2(s2, n, II, JJ, a, b, vk);
          }
        }
      } else if (ncre == 2) {
        const int c0 = cre[0], c1 = cre[1], d0 = des[0], d1 = des[1];
        Det2 t = di;
        int par = occ_between(t, d1 < c1 ? d1 : c1, d1 < c1 ? c1 : d1);
        det_flip(t, d1);
        det_flip(t, c1);
        par += occ_between(t, d0 < c0 ? d0 : c0, d0 < c0 ? c0 : d0);
        const long long vs = (par & 1) ? -v : v;
        pop2(s2, n, c1, c0, d1, d0, vs);
        pop2(s2, n, d1, d0, c1, c0, vs);
      }
    }
  }
}

__global__ void k_rdm_fin(const unsigned long long* __restrict__ fix, size_t m, double* __restrict__ out) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < m; t += (size_t)gridDim.x * blockDim.x)
    out[t] = (double)(long long)fix[t] * (1.0 / kRdmUnit);
}

}  // namespace

void rdm_evaluate(const Det2* dets, const double* c, size_t N, const Csr& H, int n, DevBuf<unsigned long long>& fix,
                  DevBuf<double>& out, cudaStream_t s) {
  const size_t n2 = (size_t)n * n, n4 = n2 * n2;
  fix.resize(n4 + n2);
  out.resize(n4 + n2);
  SHCI_CUDA(cudaMemsetAsync(fix.p, 0, (n4 + n2) * sizeof(unsigned long long), s));
  unsigned long long* s2 = fix.p;
  unsigned long long* s1 = fix.p + n4;
  if (N > 0) {
    const size_t smem = sizeof(unsigned long long) * (2 * n2 + n);
    SHCI_CUDA(cudaFuncSetAttribute(k_rdm_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_rdm_diag<<<grid_for(N, kRdmThreads, 152 * 4), kRdmThreads, smem, s>>>(dets, c, N, n, s2, s1);
    SHCI_LAUNCH_CHECK();
    k_rdm_off<<<grid_for(N * 32, kRdmThreads, 152 * 16), kRdmThreads, 0, s>>>(dets, c, N, H.rowptr.p, H.col.p, H.perm.p,
                                                                              n, s2, s1);
    SHCI_LAUNCH_CHECK();
  }
  k_rdm_fin<<<grid_for(n4 + n2, 256), 256, 0, s>>>(fix.p, n4 + n2, out.p);
  SHCI_LAUNCH_CHECK();
}

}  // namespace shci
