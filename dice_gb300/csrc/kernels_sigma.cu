// Sigma (y = H x) on the stored Hamiltonian and the tall-skinny vector
// kernels of the block Davidson solver.
//
// Sigma replaces Hmult2::operator() (SHCI/Hmult.h:52-150). The reference
// stores the lower triangle and scatters symmetrically into a private
// temporary; here every row is complete (both triangles), so each row is
// owned by VW lanes of one warp and written once, without atomics:
//   y[I] = diag[I] x[I] (FP64) + sum_J h_IJ x[J]
// Mixed path: h in FP32, x in FP32, FP32 accumulation, the FP64 diagonal term
// added in FP64. Plain path: FP64 throughout. k vectors share one pass over
// the matrix (x is row-interleaved, one 4/8/16-byte gather per column index).
//
// The Davidson kernels (Gram products, Ritz combinations, residuals and the
// diagonal preconditioner of SHCI/Davidson.cpp:85-106) reduce in a fixed
// order, so results do not depend on scheduling.
#include <cstdlib>

#include "ham.h"

namespace shci {

static inline unsigned grid_for(size_t n, int threads, size_t max_blocks = 152 * 32) {
  size_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (unsigned)b;
}

// Compensated FP32 accumulation: the running sum s carries an FP32 error term
// c that collects the rounding error of every product (FMA residual) and of
// every addition (TwoSum), so s + c equals the exact sum of the FP32 products
// to about 2^-44 relative, whatever the summation order.
//
// Why it matters: the selected space is closed under the alpha <-> beta flip
// and H commutes with it, so a Davidson run seeded with a flip-even vector
// stays flip-even in exact arithmetic -- and in FP64, which is how the
// reference converges to the state of its reference determinant. A row and
// its flipped partner hold the same products in a different order; plain FP32
// accumulation rounds them differently, breaking the symmetry at 1e-7, and a
// lower flip-odd state (present in some spaces) can then take over the solve.
// (Acc, acc_add and acc_merge live in shci_common.cuh.)

template <int KP>
struct VecF;
template <>
struct VecF<1> {
  __device__ static void fma(Acc* acc, float h, const float* x, int j) { acc_add(acc[0], h, __ldg(x + j)); }
};
template <>
struct VecF<2> {
  __device__ static void fma(Acc* acc, float h, const float* x, int j) {
    float2 v = __ldg(reinterpret_cast<const float2*>(x) + j);
    acc_add_rounded(acc[0], h, v.x);
    acc_add_rounded(acc[1], h, v.y);
  }
};
template <>
struct VecF<4> {
  __device__ static void fma(Acc* acc, float h, const float* x, int j) {
    float4 v = __ldg(reinterpret_cast<const float4*>(x) + j);
    acc_add_rounded(acc[0], h, v.x);
    acc_add_rounded(acc[1], h, v.y);
    acc_add_rounded(acc[2], h, v.z);
    acc_add_rounded(acc[3], h, v.w);
  }
};

// Row walk shared by the stored-matrix sigma kernels; every lane of a warp
// sees the same sequence of row groups (32 / VW rows, VW lanes each), so the
// width-VW shuffles always run on full warps.
//
// Single vector (kBalanced): block b owns the contiguous rows whose nonzeros
// fall in the b-th equal share of all nonzeros -- equal work per block
// whatever the row lengths -- and its warps take the next rows of that range
// from a shared-memory counter. Consecutive rows of the determinant order are
// close determinants with largely the same connections, so the rows one block
// runs together gather the same parts of x and hit in L1 (launched as two
// 1024-thread blocks per SM, one wave).
// Several vectors: the grid strides over the rows (x is k times larger and
// the band of rows the whole GPU works on at once is what stays in cache).
__device__ __forceinline__ size_t lower_bound_i64(const int64_t* __restrict__ a, size_t n, int64_t v) {
  size_t lo = 0, hi = n;
  while (lo < hi) {
    const size_t mid = (lo + hi) >> 1;
    if (a[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

template <int VW, bool kBalanced, class F>
__device__ __forceinline__ void run_rows(const int64_t* __restrict__ rowptr, size_t N, F& row) {
  if constexpr (kBalanced) {
    __shared__ unsigned long long s_next, s_end;
    if (threadIdx.x == 0) {
      const int64_t nnz = rowptr[N];
      const int64_t g = (int64_t)gridDim.x, b = (int64_t)blockIdx.x;
      const size_t r0 = lower_bound_i64(rowptr, N + 1, nnz / g * b + nnz % g * b / g);
      size_t r1 = b + 1 == g ? N : lower_bound_i64(rowptr, N + 1, nnz / g * (b + 1) + nnz % g * (b + 1) / g);
      if (r1 > N) r1 = N;
      s_next = r0 < r1 ? r0 : r1;
      s_end = r1;
    }
    __syncthreads();
    const unsigned long long end = s_end;
    while (true) {
      unsigned long long wr = 0;
      if ((threadIdx.x & 31) == 0) wr = atomicAdd(&s_next, (unsigned long long)(32 / VW));
      wr = __shfl_sync(kFull, wr, 0);
      if (wr >= end) break;
      const size_t pos = wr + (threadIdx.x & 31) / VW;
      row(pos < end ? pos : 0, pos < end);
    }
  } else {
    const size_t rows_per_warp = 32 / VW;
    const size_t stride = ((size_t)gridDim.x * blockDim.x / 32) * rows_per_warp;
    for (size_t wr = (((size_t)blockIdx.x * blockDim.x + threadIdx.x) / 32) * rows_per_warp; wr < N; wr += stride) {
      const size_t r = wr + (threadIdx.x & 31) / VW;
      row(r, r < N);
    }
  }
}

// Opens the per-row body (a lambda over the row r and whether it is live);
// ROW_LOOP_END runs it over the rows with the walk above.
#define ROW_LOOP_BEGIN                         \
  const int sub = threadIdx.x & (VW - 1);      \
  auto row = [&](const size_t r, const bool live) {
#define ROW_LOOP_END \
  }              \
  ;              \
  run_rows<VW, kBalWalk>(rowptr, N, row);

// FP32 sigma on int32 columns. One and two vectors walk balanced row ranges
// (two 1024-thread blocks per SM); four vectors the grid-strided rows, which is
// faster there (mol24, 2.91 M determinants: k = 2 10.8 ms balanced against
// 12.6 ms strided; k = 4 20.6 ms against 16.9 ms).
template <int VW, int KP, bool kBalWalk = (KP <= 2)>
__global__ void __launch_bounds__(kBalWalk ? 1024 : 256) k_sigma_mixed(const int64_t* __restrict__ rowptr,
                                                     const int32_t* __restrict__ col,
                                                     const float* __restrict__ val, const double* __restrict__ diag,
                                                     const float* __restrict__ x, size_t N, int k,
                                                     double* __restrict__ y, size_t ldy,
                                                     const uint32_t* __restrict__ perm,
    const uint32_t* __restrict__ xpos) {
  // The row loop is uniform per warp (rows past the slice run empty) so that
  // the width-VW shuffles below always see all 32 lanes.
  ROW_LOOP_BEGIN
    Acc acc[KP];
#pragma unroll
    for (int c = 0; c < KP; ++c) acc[c] = Acc{0.f, 0.f};
    const int64_t p0 = live ? __ldg(rowptr + r) : 0;
    const int64_t p1 = live ? __ldg(rowptr + r + 1) : 0;
    // Consecutive lanes take consecutive nonzeros: the column and value loads
    // are coalesced, and on a column-sorted row the 32 gathers of one
    // instruction land on as few 32-byte sectors of x as the row allows.
    // Four nonzeros per lane per step keep four gathers in flight.
    int64_t p = p0 + sub;
    for (; p + 3 * VW < p1; p += 4 * VW) {
      const int j0 = __ldcs(col + p), j1 = __ldcs(col + p + VW);
      const int j2 = __ldcs(col + p + 2 * VW), j3 = __ldcs(col + p + 3 * VW);
      const float h0 = __ldcs(val + p), h1 = __ldcs(val + p + VW);
      const float h2 = __ldcs(val + p + 2 * VW), h3 = __ldcs(val + p + 3 * VW);
      VecF<KP>::fma(acc, h0, x, j0);
      VecF<KP>::fma(acc, h1, x, j1);
      VecF<KP>::fma(acc, h2, x, j2);
      VecF<KP>::fma(acc, h3, x, j3);
    }
    for (; p < p1; p += VW) VecF<KP>::fma(acc, __ldcs(val + p), x, __ldcs(col + p));
#pragma unroll
    for (int c = 0; c < KP; ++c) {
#pragma unroll
      for (int o = VW / 2; o; o >>= 1) {
        Acc other{__shfl_xor_sync(kFull, acc[c].s, o, VW), __shfl_xor_sync(kFull, acc[c].c, o, VW)};
        // merge in lane order so that both partners of a pair compute the same value
        if ((threadIdx.x & o) == 0) {
          acc_merge(acc[c], other);
        } else {
          acc_merge(other, acc[c]);
          acc[c] = other;
        }
      }
    }
    if (sub == 0 && live) {
      const size_t o = __ldg(perm + r);
      const size_t xr = xpos ? (size_t)__ldg(xpos + r) : r;  // the row's own x (row blocks: its storage position)
      const double dg = diag[o];
#pragma unroll
      for (int c = 0; c < KP; ++c)
        if (c < k) y[(size_t)c * ldy + o] = dg * (double)x[xr * KP + c] + ((double)acc[c].s + (double)acc[c].c);
    }
  ROW_LOOP_END
}

// Single-vector FP32 sigma on the 16-bit-delta copy (Csr::cdel): the same
// row walk and accumulation as k_sigma_mixed. Rows are padded to multiples of
// four entries and start at multiples of four, so each lane takes four
// consecutive entries with one 8-byte load of deltas and one 16-byte load of
// values; the columns come from the lane's running sum plus one segmented
// prefix sum of the lanes' totals per 4 x VW entries. 6 bytes per entry
// streamed instead of 8.
template <int VW>
__global__ void __launch_bounds__(1024) k_sigma_mixed16(const int64_t* __restrict__ rowptr,
                                                        const int32_t* __restrict__ cbase,
                                                        const uint16_t* __restrict__ cdel,
                                                        const float* __restrict__ val, const double* __restrict__ diag,
                                                        const float* __restrict__ x, size_t N, double* __restrict__ y,
                                                        const uint32_t* __restrict__ perm,
    const uint32_t* __restrict__ xpos) {
  constexpr int KP = 1;
  constexpr bool kBalWalk = true;
  const unsigned seg = VW == 32 ? kFull : (((1u << VW) - 1u) << (threadIdx.x & 31 & ~(VW - 1)));
  ROW_LOOP_BEGIN
    Acc acc{0.f, 0.f};
    const int64_t p0 = live ? __ldg(rowptr + r) : 0;
    const int64_t p1 = live ? __ldg(rowptr + r + 1) : 0;
    int carry = live ? __ldg(cbase + r) : 0;  // column before the chunk's first entry (first delta is 0)
    for (int64_t q = p0; q < p1; q += 4 * VW) {
      const int64_t p = q + 4 * sub;
      const bool ok = p < p1;
      uint2 dd = make_uint2(0u, 0u);
      float4 hh = make_float4(0.f, 0.f, 0.f, 0.f);
      if (ok) {
        dd = __ldcs(reinterpret_cast<const uint2*>(cdel + p));
        hh = __ldcs(reinterpret_cast<const float4*>(val + p));
      }
      const int d0 = (int)(dd.x & 0xFFFFu), d1 = (int)(dd.x >> 16);
      const int d2 = (int)(dd.y & 0xFFFFu), d3 = (int)(dd.y >> 16);
      const int t = d0 + d1 + d2 + d3;
      int incl = t;
#pragma unroll
      for (int o = 1; o < VW; o <<= 1) {
        const int u = __shfl_up_sync(seg, incl, o, VW);
        if (sub >= o) incl += u;
      }
      const int c0 = carry + incl - t + d0, c1 = c0 + d1, c2 = c1 + d2, c3 = c2 + d3;
      carry += __shfl_sync(seg, incl, VW - 1, VW);
      if (ok) {
        const float x0 = hh.x != 0.f ? __ldg(x + c0) : 0.f;
        const float x1 = hh.y != 0.f ? __ldg(x + c1) : 0.f;
        const float x2 = hh.z != 0.f ? __ldg(x + c2) : 0.f;
        const float x3 = hh.w != 0.f ? __ldg(x + c3) : 0.f;
        acc_add(acc, hh.x, x0);
        acc_add(acc, hh.y, x1);
        acc_add(acc, hh.z, x2);
        acc_add(acc, hh.w, x3);
      }
    }
#pragma unroll
    for (int o = VW / 2; o; o >>= 1) {
      Acc other{__shfl_xor_sync(kFull, acc.s, o, VW), __shfl_xor_sync(kFull, acc.c, o, VW)};
      if ((threadIdx.x & o) == 0) {
        acc_merge(acc, other);
      } else {
        acc_merge(other, acc);
        acc = other;
      }
    }
    if (sub == 0 && live) {
      const size_t o = __ldg(perm + r);
      const size_t xr = xpos ? (size_t)__ldg(xpos + r) : r;
      y[o] = diag[o] * (double)x[xr] + ((double)acc.s + (double)acc.c);
    }
  ROW_LOOP_END
}

// ---- building the 16-bit-delta copy ----------------------------------------
// bridges needed before entry p of its row: (gap - 1) / 65535 for a gap >= 65536
// (columns fit 31 bits, so gaps are 32-bit; the division runs only for those)
__global__ void k_c_count(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col, size_t N,
                          int64_t* __restrict__ len) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < (int64_t)N; r += warps) {
    const int64_t p0 = rowptr[r], p1 = rowptr[r + 1];
    int64_t b = 0;
    for (int64_t p = p0 + 1 + lane; p < p1; p += 32) {
      const uint32_t gap = (uint32_t)(col[p] - col[p - 1]);  // >= 1: columns ascend
      if (gap > 65535u) b += (gap - 1u) / 65535u;             // rare: divide only there
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) b += __shfl_xor_sync(kFull, b, o);
    if (lane == 0) len[r] = ((p1 - p0) + b + 3) & ~(int64_t)3;  // padded to a multiple of four
  }
}
__global__ void k_c_fill(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                         const float* __restrict__ vhi, size_t N, const int64_t* __restrict__ crow,
                         int32_t* __restrict__ cbase, uint16_t* __restrict__ cdel, float* __restrict__ cval) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < (int64_t)N; r += warps) {
    const int64_t p0 = rowptr[r], p1 = rowptr[r + 1];
    if (lane == 0) cbase[r] = p1 > p0 ? col[p0] : 0;
    int64_t out0 = crow[r];  // output position of this chunk's first item
    for (int64_t q = p0; q < p1; q += 32) {
      const int64_t p = q + lane;
      uint32_t gap = 0, nb = 0;  // a gap needs (gap - 1) / 65535 bridges, none below 65536
      if (p < p1) {
        gap = p > p0 ? (uint32_t)(col[p] - col[p - 1]) : 0u;
        nb = gap > 65535u ? (gap - 1u) / 65535u : 0u;
      }
      int incl = (p < p1 ? 1 : 0) + (int)nb;  // items this lane writes (bridges + the entry)
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
      }
      if (p < p1) {
        int64_t o = out0 + incl - 1 - (int64_t)nb;
        for (uint32_t t = 0; t < nb; ++t, ++o) {
          cdel[o] = 65535;
          cval[o] = 0.f;
        }
        cdel[o] = (uint16_t)(gap - nb * 65535u);
        cval[o] = vhi[p];
      }
      out0 += __shfl_sync(kFull, incl, 31);
    }
    // padding to the next multiple of four: delta 0 (same column), value 0
    const int64_t end = crow[r + 1];
    if (lane < end - out0) {
      cdel[out0 + lane] = 0;
      cval[out0 + lane] = 0.f;
    }
  }
}

void compress_csr(Csr& H, Prims& pr, cudaStream_t s) {
  H.drop_compressed();
  if (!H.vhi.p || H.N == 0) return;
  const size_t N = H.N;
  DevBuf<int64_t> len;
  len.resize(N);
  const unsigned blocks = grid_for(N * 32, 256, 152 * 16);
  k_c_count<<<blocks, 256, 0, s>>>(H.rowptr.p, H.col.p, N, len.p);
  SHCI_LAUNCH_CHECK();
  H.crow.resize(N + 1);
  int64_t total = 0;
  scan_exclusive_i64(len.p, H.crow.p, N, &total, pr, s);
  SHCI_CUDA(cudaMemcpyAsync(H.crow.p + N, &total, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  H.cbase.resize(N);
  H.cdel.resize(total > 0 ? total : 1);
  H.cval.resize(total > 0 ? total : 1);
  k_c_fill<<<blocks, 256, 0, s>>>(H.rowptr.p, H.col.p, H.vhi.p, N, H.crow.p, H.cbase.p, H.cdel.p, H.cval.p);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));
  H.cnnz = total;
  H.cvalid = true;
}

template <int VW, int KP>
__global__ void __launch_bounds__(KP == 1 ? 1024 : 256) k_sigma_f64(const int64_t* __restrict__ rowptr,
                                                   const int32_t* __restrict__ col,
                                                   const double* __restrict__ v64, const double* __restrict__ diag,
                                                   const double* __restrict__ x, size_t N, int k,
                                                   double* __restrict__ y, size_t ldy,
                                                   const uint32_t* __restrict__ perm,
    const uint32_t* __restrict__ xpos) {
  constexpr bool kBalWalk = KP == 1;
  ROW_LOOP_BEGIN
    double acc[KP];
#pragma unroll
    for (int c = 0; c < KP; ++c) acc[c] = 0.0;
    const int64_t p0 = live ? __ldg(rowptr + r) : 0;
    const int64_t p1 = live ? __ldg(rowptr + r + 1) : 0;
    auto elem = [&](int64_t p, int j) {
      const double h = __ldcs(v64 + p);
#pragma unroll
      for (int c = 0; c < KP; ++c) acc[c] += h * __ldg(x + (size_t)j * KP + c);
    };
    // consecutive lanes on consecutive nonzeros (see k_sigma_mixed)
    int64_t p = p0 + sub;
    for (; p + 3 * VW < p1; p += 4 * VW) {
      const int j0 = __ldcs(col + p), j1 = __ldcs(col + p + VW);
      const int j2 = __ldcs(col + p + 2 * VW), j3 = __ldcs(col + p + 3 * VW);
      elem(p, j0);
      elem(p + VW, j1);
      elem(p + 2 * VW, j2);
      elem(p + 3 * VW, j3);
    }
    for (; p < p1; p += VW) elem(p, __ldcs(col + p));
#pragma unroll
    for (int c = 0; c < KP; ++c) {
#pragma unroll
      for (int o = VW / 2; o; o >>= 1) acc[c] += __shfl_xor_sync(kFull, acc[c], o, VW);
    }
    if (sub == 0 && live) {
      const size_t o = __ldg(perm + r);
      const size_t xr = xpos ? (size_t)__ldg(xpos + r) : r;
      const double dg = diag[o];
#pragma unroll
      for (int c = 0; c < KP; ++c)
        if (c < k) y[(size_t)c * ldy + o] = dg * x[xr * KP + c] + acc[c];
    }
  ROW_LOOP_END
}

// Refinement sigma on the mixed path's head + tail values, in float-float
// arithmetic: x is split as x = xh + xl (two floats) and every product
// (hi + lo)(xh + xl) enters the compensated accumulator as its exactly
// rounded head hi*xh plus the FMA residual and the cross terms hi*xl + lo*xh.
// The result matches the FP64 product sum to ~1e-13 relative while keeping
// every operation of the inner loop on the FP32 pipe (the FP64 pipe of this
// GPU issues about two FMAs per clock per SM, so an FP64 head + tail sum,
// with its two conversions, one add and one FMA per nonzero, runs 3.5x
// slower). The diagonal term is added in FP64 from the unsplit x.
__device__ __forceinline__ void acc_add_ff(Acc& a, float hi, float lo, float xh, float xl) {
  const float p = __fmul_rn(hi, xh);
  const float pe = __fmaf_rn(hi, xh, -p);
  const float small = __fmaf_rn(hi, xl, __fmaf_rn(lo, xh, pe));
  const float t = __fadd_rn(a.s, p);
  const float bp = __fsub_rn(t, a.s);
  const float e = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  a.s = t;
  a.c = __fadd_rn(a.c, __fadd_rn(e, small));
}

template <int KP>
struct VecFF;
template <>
struct VecFF<1> {
  __device__ static void fma(Acc* acc, float hi, float lo, const float* x, int j) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(x) + j);
    acc_add_ff(acc[0], hi, lo, v.x, v.y);
  }
};
template <>
struct VecFF<2> {
  __device__ static void fma(Acc* acc, float hi, float lo, const float* x, int j) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(x) + j);
    acc_add_ff(acc[0], hi, lo, v.x, v.y);
    acc_add_ff(acc[1], hi, lo, v.z, v.w);
  }
};
template <>
struct VecFF<4> {
  __device__ static void fma(Acc* acc, float hi, float lo, const float* x, int j) {
    const float4 v0 = __ldg(reinterpret_cast<const float4*>(x) + 2 * (size_t)j);
    const float4 v1 = __ldg(reinterpret_cast<const float4*>(x) + 2 * (size_t)j + 1);
    acc_add_ff(acc[0], hi, lo, v0.x, v0.y);
    acc_add_ff(acc[1], hi, lo, v0.z, v0.w);
    acc_add_ff(acc[2], hi, lo, v1.x, v1.y);
    acc_add_ff(acc[3], hi, lo, v1.z, v1.w);
  }
};

template <int VW, int KP>
__global__ void __launch_bounds__(KP == 1 ? 1024 : 256) k_sigma_ff(const int64_t* __restrict__ rowptr,
                                                  const int32_t* __restrict__ col,
                                                  const float* __restrict__ vhi, const float* __restrict__ vlo,
                                                  const double* __restrict__ diag, const float* __restrict__ xff,
                                                  const double* __restrict__ xd, size_t ldx, int c0, size_t N, int k,
                                                  double* __restrict__ y, size_t ldy,
                                                  const uint32_t* __restrict__ perm) {
  // same row mapping as the FP64 kernel
  constexpr bool kBalWalk = KP == 1;
  ROW_LOOP_BEGIN
    Acc acc[KP];
#pragma unroll
    for (int c = 0; c < KP; ++c) acc[c] = Acc{0.f, 0.f};
    const int64_t p0 = live ? __ldg(rowptr + r) : 0;
    const int64_t p1 = live ? __ldg(rowptr + r + 1) : 0;
    int64_t p = p0 + sub;
    for (; p + 3 * VW < p1; p += 4 * VW) {
      const int j0 = __ldcs(col + p), j1 = __ldcs(col + p + VW);
      const int j2 = __ldcs(col + p + 2 * VW), j3 = __ldcs(col + p + 3 * VW);
      const float h0 = __ldcs(vhi + p), h1 = __ldcs(vhi + p + VW);
      const float h2 = __ldcs(vhi + p + 2 * VW), h3 = __ldcs(vhi + p + 3 * VW);
      const float l0 = __ldcs(vlo + p), l1 = __ldcs(vlo + p + VW);
      const float l2 = __ldcs(vlo + p + 2 * VW), l3 = __ldcs(vlo + p + 3 * VW);
      VecFF<KP>::fma(acc, h0, l0, xff, j0);
      VecFF<KP>::fma(acc, h1, l1, xff, j1);
      VecFF<KP>::fma(acc, h2, l2, xff, j2);
      VecFF<KP>::fma(acc, h3, l3, xff, j3);
    }
    for (; p < p1; p += VW) VecFF<KP>::fma(acc, __ldcs(vhi + p), __ldcs(vlo + p), xff, __ldcs(col + p));
#pragma unroll
    for (int c = 0; c < KP; ++c) {
#pragma unroll
      for (int o = VW / 2; o; o >>= 1) {
        Acc other{__shfl_xor_sync(kFull, acc[c].s, o, VW), __shfl_xor_sync(kFull, acc[c].c, o, VW)};
        if ((threadIdx.x & o) == 0) {
          acc_merge(acc[c], other);
        } else {
          acc_merge(other, acc[c]);
          acc[c] = other;
        }
      }
    }
    if (sub == 0 && live) {
      const size_t o = __ldg(perm + r);
      const double dg = diag[o];
#pragma unroll
      for (int c = 0; c < KP; ++c)
        if (c < k)
          y[(size_t)c * ldy + o] = dg * xd[(size_t)(c0 + c) * ldx + o] + ((double)acc[c].s + (double)acc[c].c);
    }
  ROW_LOOP_END
}

// Launch shape of the stored-matrix sigma kernels (see run_rows): one vector
// runs as two 1024-thread blocks per SM over nonzero-balanced row ranges;
// several vectors as a grid-strided launch of 256-thread blocks.
struct SigmaLaunch {
  unsigned blocks;
  int threads;
};
static int sm_count() {
  static int n = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      v = 152;
    return v > 0 ? v : 152;
  }();
  return n;
}
static SigmaLaunch sigma_launch(size_t N, int vw, int kp) {
  if (kp == 1) return SigmaLaunch{(unsigned)(2 * sm_count()), 1024};
  return SigmaLaunch{grid_for(N * (size_t)vw, 256, (size_t)sm_count() * 16), 256};
}

static int pick_vw(const Csr& H) {
  double avg = H.N ? (double)H.nnz / (double)H.N : 0.0;
  if (avg >= 96) return 32;
  if (avg >= 40) return 16;
  if (avg >= 14) return 8;
  return 4;
}

template <int KP>
static void launch_mixed(int vw, const Csr& H, const double* diag, const float* x, int k, double* y, size_t ldy,
                         cudaStream_t s) {
  const SigmaLaunch L = KP <= 2 ? sigma_launch(H.N, vw, 1) : sigma_launch(H.N, vw, KP);
  switch (vw) {
    case 32: k_sigma_mixed<32, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, H.vhi.p, diag, x, H.N, k, y, ldy, H.perm.p, H.block ? H.xpos.p : nullptr); break;
    case 16: k_sigma_mixed<16, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, H.vhi.p, diag, x, H.N, k, y, ldy, H.perm.p, H.block ? H.xpos.p : nullptr); break;
    case 8: k_sigma_mixed<8, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, H.vhi.p, diag, x, H.N, k, y, ldy, H.perm.p, H.block ? H.xpos.p : nullptr); break;
    default: k_sigma_mixed<4, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, H.vhi.p, diag, x, H.N, k, y, ldy, H.perm.p, H.block ? H.xpos.p : nullptr); break;
  }
  SHCI_LAUNCH_CHECK();
}

void sigma_csr_mixed(const Csr& H, const double* diag, const float* x32, int kp, int k, double* y, size_t ldy,
                     cudaStream_t s) {
  if (!H.vhi.p) throw Error(kErrState, "Hamiltonian has no FP32 values (built for the FP64 path)");
  if (H.N == 0) return;
  int vw = pick_vw(H);
  if (kp == 1 && H.cvalid) {
    const SigmaLaunch L = sigma_launch(H.N, vw, 1);
    switch (vw) {
      case 32: k_sigma_mixed16<32><<<L.blocks, L.threads, 0, s>>>(H.crow.p, H.cbase.p, H.cdel.p, H.cval.p, diag, x32, H.N, y, H.perm.p, H.block ? H.xpos.p : nullptr); break;
      case 16: k_sigma_mixed16<16><<<L.blocks, L.threads, 0, s>>>(H.crow.p, H.cbase.p, H.cdel.p, H.cval.p, diag, x32, H.N, y, H.perm.p, H.block ? H.xpos.p : nullptr); break;
      case 8: k_sigma_mixed16<8><<<L.blocks, L.threads, 0, s>>>(H.crow.p, H.cbase.p, H.cdel.p, H.cval.p, diag, x32, H.N, y, H.perm.p, H.block ? H.xpos.p : nullptr); break;
      default: k_sigma_mixed16<4><<<L.blocks, L.threads, 0, s>>>(H.crow.p, H.cbase.p, H.cdel.p, H.cval.p, diag, x32, H.N, y, H.perm.p, H.block ? H.xpos.p : nullptr); break;
    }
    SHCI_LAUNCH_CHECK();
    return;
  }
  switch (kp) {
    case 1: launch_mixed<1>(vw, H, diag, x32, k, y, ldy, s); break;
    case 2: launch_mixed<2>(vw, H, diag, x32, k, y, ldy, s); break;
    case 4: launch_mixed<4>(vw, H, diag, x32, k, y, ldy, s); break;
    default: throw Error(kErrInvalid, "sigma block width must be 1, 2 or 4");
  }
}

template <int KP>
static void launch_f64(int vw, const Csr& H, const double* diag, const double* x, int k, double* y, size_t ldy,
                       cudaStream_t s) {
  const SigmaLaunch L = sigma_launch(H.N, vw, KP);
  const double* v64 = H.v64.p;
  switch (vw) {
    case 32: k_sigma_f64<32, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, v64, diag, x, H.N, k, y, ldy, H.perm.p, H.block ? H.xpos.p : nullptr); break;
    case 16: k_sigma_f64<16, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, v64, diag, x, H.N, k, y, ldy, H.perm.p, H.block ? H.xpos.p : nullptr); break;
    case 8: k_sigma_f64<8, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, v64, diag, x, H.N, k, y, ldy, H.perm.p, H.block ? H.xpos.p : nullptr); break;
    default: k_sigma_f64<4, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, v64, diag, x, H.N, k, y, ldy, H.perm.p, H.block ? H.xpos.p : nullptr); break;
  }
  SHCI_LAUNCH_CHECK();
}

void sigma_csr_f64(const Csr& H, const double* diag, const double* x64, int kp, int k, double* y, size_t ldy,
                   cudaStream_t s) {
  if (H.N == 0) return;
  if (!H.v64.p) throw Error(kErrState, "Hamiltonian has no FP64 values");
  const int vw = pick_vw(H);
  switch (kp) {
    case 1: launch_f64<1>(vw, H, diag, x64, k, y, ldy, s); break;
    case 2: launch_f64<2>(vw, H, diag, x64, k, y, ldy, s); break;
    case 4: launch_f64<4>(vw, H, diag, x64, k, y, ldy, s); break;
    default: throw Error(kErrInvalid, "sigma block width must be 1, 2 or 4");
  }
}

template <int KP>
static void launch_ff(int vw, const Csr& H, const double* diag, const float* xff, const double* xd, size_t ldx, int c0,
                      int k, double* y, size_t ldy, cudaStream_t s) {
  const SigmaLaunch L = sigma_launch(H.N, vw, KP);
  const float *vhi = H.vhi.p, *vlo = H.vlo.p;
  switch (vw) {
    case 32: k_sigma_ff<32, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, vhi, vlo, diag, xff, xd, ldx, c0, H.N, k, y, ldy, H.perm.p); break;
    case 16: k_sigma_ff<16, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, vhi, vlo, diag, xff, xd, ldx, c0, H.N, k, y, ldy, H.perm.p); break;
    case 8: k_sigma_ff<8, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, vhi, vlo, diag, xff, xd, ldx, c0, H.N, k, y, ldy, H.perm.p); break;
    default: k_sigma_ff<4, KP><<<L.blocks, L.threads, 0, s>>>(H.rowptr.p, H.col.p, vhi, vlo, diag, xff, xd, ldx, c0, H.N, k, y, ldy, H.perm.p); break;
  }
  SHCI_LAUNCH_CHECK();
}

void sigma_csr_ff(const Csr& H, const double* diag, const float* xff, int kp, const double* xd, size_t ldx, int c0,
                  int k, double* y, size_t ldy, cudaStream_t s) {
  if (H.N == 0) return;
  if (!(H.vhi.p && H.vlo.p)) throw Error(kErrState, "Hamiltonian has no FP32 head/tail values");
  const int vw = pick_vw(H);
  switch (kp) {
    case 1: launch_ff<1>(vw, H, diag, xff, xd, ldx, c0, k, y, ldy, s); break;
    case 2: launch_ff<2>(vw, H, diag, xff, xd, ldx, c0, k, y, ldy, s); break;
    case 4: launch_ff<4>(vw, H, diag, xff, xd, ldx, c0, k, y, ldy, s); break;
    default: throw Error(kErrInvalid, "sigma block width must be 1, 2 or 4");
  }
}

// ---------------------------------------------------------------------------
// Packing between column-major FP64 blocks and row-interleaved vectors
// ---------------------------------------------------------------------------
__global__ void k_pack_f32(const double* __restrict__ A, size_t lda, int c0, int k, int kp, size_t N,
                           float* __restrict__ out, const uint32_t* __restrict__ perm) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x) {
    const size_t src = perm ? (size_t)perm[r] : r;
    for (int c = 0; c < kp; ++c) out[r * kp + c] = c < k ? (float)A[(size_t)(c0 + c) * lda + src] : 0.f;
  }
}
__global__ void k_pack_f64(const double* __restrict__ A, size_t lda, int c0, int k, int kp, size_t N,
                           double* __restrict__ out, const uint32_t* __restrict__ perm) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x) {
    const size_t src = perm ? (size_t)perm[r] : r;
    for (int c = 0; c < kp; ++c) out[r * kp + c] = c < k ? A[(size_t)(c0 + c) * lda + src] : 0.0;
  }
}
__global__ void k_unpack_f64(const double* __restrict__ in, int kp, int k, size_t N, double* __restrict__ A,
                             size_t lda, int c0) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x)
    for (int c = 0; c < k; ++c) A[(size_t)(c0 + c) * lda + r] = in[r * kp + c];
}
__global__ void k_pack_ff(const double* __restrict__ A, size_t lda, int c0, int k, int kp, size_t N,
                          float2* __restrict__ out, const uint32_t* __restrict__ perm) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x)
    for (int c = 0; c < kp; ++c) {
      float2 v = make_float2(0.f, 0.f);
      if (c < k) {
        const double x = A[(size_t)(c0 + c) * lda + (perm ? (size_t)perm[r] : r)];
        v.x = __double2float_rn(x);
        v.y = __double2float_rn(x - (double)v.x);
      }
      out[r * kp + c] = v;
    }
}
void pack_ff(const double* A, size_t lda, int c0, int k, int kp, size_t N, float* out, cudaStream_t s,
             const uint32_t* perm) {
  k_pack_ff<<<grid_for(N, 256), 256, 0, s>>>(A, lda, c0, k, kp, N, reinterpret_cast<float2*>(out), perm);
  SHCI_LAUNCH_CHECK();
}
void pack_f32(const double* A, size_t lda, int c0, int k, int kp, size_t N, float* out, cudaStream_t s,
              const uint32_t* perm) {
  k_pack_f32<<<grid_for(N, 256), 256, 0, s>>>(A, lda, c0, k, kp, N, out, perm);
  SHCI_LAUNCH_CHECK();
}
void pack_f64(const double* A, size_t lda, int c0, int k, int kp, size_t N, double* out, cudaStream_t s,
              const uint32_t* perm) {
  k_pack_f64<<<grid_for(N, 256), 256, 0, s>>>(A, lda, c0, k, kp, N, out, perm);
  SHCI_LAUNCH_CHECK();
}
struct Row32 {
  double2 a, b;
};
template <class T>
__global__ void k_gather_rows(const T* __restrict__ in, const uint32_t* __restrict__ perm, size_t N,
                              T* __restrict__ out) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x)
    out[r] = in[perm[r]];
}
void gather_rows(const void* in, size_t bytes_per_row, const uint32_t* perm, size_t N, void* out, cudaStream_t s) {
  if (N == 0) return;
  const unsigned g = grid_for(N, 256);
  switch (bytes_per_row) {
    case 4: k_gather_rows<float><<<g, 256, 0, s>>>(static_cast<const float*>(in), perm, N, static_cast<float*>(out)); break;
    case 8: k_gather_rows<double><<<g, 256, 0, s>>>(static_cast<const double*>(in), perm, N, static_cast<double*>(out)); break;
    case 16: k_gather_rows<double2><<<g, 256, 0, s>>>(static_cast<const double2*>(in), perm, N, static_cast<double2*>(out)); break;
    case 32: k_gather_rows<Row32><<<g, 256, 0, s>>>(static_cast<const Row32*>(in), perm, N, static_cast<Row32*>(out)); break;
    default: throw Error(kErrInvalid, "gather_rows: row size must be 4, 8, 16 or 32 bytes");
  }
  SHCI_LAUNCH_CHECK();
}
void unpack_f64(const double* in, int kp, int k, size_t N, double* A, size_t lda, int c0, cudaStream_t s) {
  k_unpack_f64<<<grid_for(N, 256), 256, 0, s>>>(in, kp, k, N, A, lda, c0);
  SHCI_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Tall-skinny Gram: G = A^T B. Blocks own contiguous row ranges and write
// one partial per block; a second kernel adds the partials in block order, so
// the result does not depend on scheduling.
// Narrow products (ma * mb <= 16: norms, dots, residual norms) keep every
// pair's sum in registers and stream the rows with independent loads; wider
// ones (the Rayleigh matrix) stage 64-row tiles in shared memory with all
// threads of the block splitting the rows of a tile between them.
// ---------------------------------------------------------------------------
constexpr int kGramMax = 16;
constexpr int kGramRows = 64;
constexpr unsigned kGramBlocks = 152 * 2;
constexpr int kGramRegPairs = 16;

__device__ inline void block_sum_pairs(double* acc, int P, double* __restrict__ out) {
  __shared__ double red[8][kGramRegPairs];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int p = 0; p < kGramRegPairs; ++p) {
    if (p >= P) break;
    double v = acc[p];
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if (lane == 0) red[w][p] = v;
  }
  __syncthreads();
  if ((int)threadIdx.x < P) {
    double v = 0.0;
    for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww) v += red[ww][threadIdx.x];
    out[threadIdx.x] = v;
  }
}

__global__ void __launch_bounds__(256) k_gram_reg(const double* __restrict__ A, size_t lda, int ma,
                                                  const double* __restrict__ B, size_t ldb, int mb, size_t N,
                                                  double* __restrict__ part) {
  double acc[kGramRegPairs];
#pragma unroll
  for (int p = 0; p < kGramRegPairs; ++p) acc[p] = 0.0;
  const int P = ma * mb;
  const size_t per = (N + gridDim.x - 1) / gridDim.x;
  const size_t r0 = (size_t)blockIdx.x * per;
  const size_t r1 = r0 + per < N ? r0 + per : N;
  // repeated loads of one row's entries hit L1; only distinct ones reach L2
  for (size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
#pragma unroll
    for (int p = 0; p < kGramRegPairs; ++p)
      if (p < P) acc[p] += A[(size_t)(p % ma) * lda + r] * B[(size_t)(p / ma) * ldb + r];
  }
  block_sum_pairs(acc, P, part + (size_t)blockIdx.x * P);
}

__global__ void __launch_bounds__(256) k_gram_part(const double* __restrict__ A, size_t lda, int ma,
                                                   const double* __restrict__ B, size_t ldb, int mb, size_t N,
                                                   double* __restrict__ part) {
  __shared__ double sA[kGramMax][kGramRows + 1];
  __shared__ double sB[kGramMax][kGramRows + 1];
  __shared__ double red[256];
  const int t = threadIdx.x;
  const int P = ma * mb;
  const int S = 256 / P;  // threads per pair, splitting the rows of a tile
  const int pp = t % P, q = t / P;
  const int pi = pp % ma, pj = pp / ma;
  const bool active = q < S;
  double acc = 0.0;
  const size_t per = (N + gridDim.x - 1) / gridDim.x;
  const size_t r0 = (size_t)blockIdx.x * per;
  const size_t r1 = r0 + per < N ? r0 + per : N;
  for (size_t base = r0; base < r1; base += kGramRows) {
    for (int e = t; e < ma * kGramRows; e += blockDim.x) {
      const int c = e / kGramRows, rr = e % kGramRows;
      const size_t row = base + rr;
      sA[c][rr] = row < r1 ? A[(size_t)c * lda + row] : 0.0;
    }
    for (int e = t; e < mb * kGramRows; e += blockDim.x) {
      const int c = e / kGramRows, rr = e % kGramRows;
      const size_t row = base + rr;
      sB[c][rr] = row < r1 ? B[(size_t)c * ldb + row] : 0.0;
    }
    __syncthreads();
    if (active)
      for (int rr = q; rr < kGramRows; rr += S) acc += sA[pi][rr] * sB[pj][rr];
    __syncthreads();
  }
  red[t] = active ? acc : 0.0;
  __syncthreads();
  if (t < P) {
    double v = 0.0;
    for (int k = 0; k < S; ++k) v += red[t + k * P];
    part[(size_t)blockIdx.x * P + t] = v;
  }
}

__global__ void k_gram_sum(const double* __restrict__ part, int nblocks, int P, double* __restrict__ G) {
  int t = threadIdx.x;
  if (t < P) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * P + t];
    G[t] = s;
  }
}

void ts_gram(const double* A, size_t lda, int ma, const double* B, size_t ldb, int mb, size_t N, double* G,
             DevBuf<double>& part, cudaStream_t s) {
  if (ma < 1 || mb < 1 || ma > kGramMax || mb > kGramMax) throw Error(kErrInvalid, "Gram block too wide");
  unsigned nb = kGramBlocks;
  if ((size_t)nb * kGramRows > N) nb = (unsigned)((N + kGramRows - 1) / kGramRows);
  if (nb < 1) nb = 1;
  part.reserve((size_t)nb * ma * mb);
  if (ma * mb <= kGramRegPairs)
    k_gram_reg<<<nb, 256, 0, s>>>(A, lda, ma, B, ldb, mb, N, part.p);
  else
    k_gram_part<<<nb, 256, 0, s>>>(A, lda, ma, B, ldb, mb, N, part.p);
  SHCI_LAUNCH_CHECK();
  k_gram_sum<<<1, 256, 0, s>>>(part.p, (int)nb, ma * mb, G);
  SHCI_LAUNCH_CHECK();
}

// Y = alpha * A Q + beta * Y. Each thread owns one row; the row's m entries
// stay in registers (loops unrolled to the 16-column maximum and predicated).
__global__ void __launch_bounds__(256) k_ts_gemm(const double* __restrict__ A, size_t lda, int m,
                                                 const double* __restrict__ Q, int k, size_t N, double alpha,
                                                 double beta, double* __restrict__ Y, size_t ldy) {
  __shared__ double sQ[kGramMax * kGramMax];
  for (int e = threadIdx.x; e < m * k; e += blockDim.x) sQ[e] = Q[e];
  __syncthreads();
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x) {
    double a[kGramMax];
#pragma unroll
    for (int i = 0; i < kGramMax; ++i) a[i] = i < m ? A[(size_t)i * lda + r] : 0.0;
    for (int c = 0; c < k; ++c) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < kGramMax; ++i)
        if (i < m) s += a[i] * sQ[c * m + i];
      double* yp = Y + (size_t)c * ldy + r;
      *yp = (beta == 0.0) ? alpha * s : alpha * s + beta * (*yp);
    }
  }
}
void ts_gemm(const double* A, size_t lda, int m, const double* Q, int k, size_t N, double alpha, double beta,
             double* Y, size_t ldy, cudaStream_t s) {
  if (m > kGramMax || k > kGramMax) throw Error(kErrInvalid, "tall-skinny product too wide");
  k_ts_gemm<<<grid_for(N, 256), 256, 0, s>>>(A, lda, m, Q, k, N, alpha, beta, Y, ldy);
  SHCI_LAUNCH_CHECK();
}

__global__ void k_residual(const double* __restrict__ X, const double* __restrict__ Y, const double* __restrict__ lam,
                           int k, size_t N, size_t ld, double* __restrict__ R) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x)
    for (int c = 0; c < k; ++c) R[(size_t)c * ld + r] = Y[(size_t)c * ld + r] - lam[c] * X[(size_t)c * ld + r];
}
void residual(const double* X, const double* Y, const double* lam, int k, size_t N, size_t ld, double* R,
              cudaStream_t s) {
  k_residual<<<grid_for(N, 256), 256, 0, s>>>(X, Y, lam, k, N, ld, R);
  SHCI_LAUNCH_CHECK();
}

// precondition (SHCI/Davidson.cpp:85-106)
__global__ void k_precondition(const double* __restrict__ diag, const double* __restrict__ lam, int k, size_t N,
                               double* __restrict__ R, size_t ld) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x)
    for (int c = 0; c < k; ++c) {
      double e = lam[c], d = diag[r];
      double* p = R + (size_t)c * ld + r;
      if (fabs(e - d) > 1e-12)
        *p = *p / (e - d);
      else
        *p = *p / (e - d - 1.e-12);
    }
}
void precondition(const double* diag, const double* lam, int k, size_t N, double* R, size_t ld, cudaStream_t s) {
  k_precondition<<<grid_for(N, 256), 256, 0, s>>>(diag, lam, k, N, R, ld);
  SHCI_LAUNCH_CHECK();
}

// Shifted preconditioner r_i / (lam - diag_i - shift_i). The plain denominator
// is kept wherever the shifted one changes sign or shrinks below a fifth of it
// (a shift that would blow the correction up), so the learned or second-order
// shift can only refine the reference's denominator, never replace it wholesale.
__global__ void k_precondition_shift(const double* __restrict__ diag, const double* __restrict__ shift,
                                     const double* __restrict__ lam, int k, size_t N, double* __restrict__ R,
                                     size_t ld) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x)
    for (int c = 0; c < k; ++c) {
      const double e = lam[c], d = diag[r];
      double den = e - d;
      const double d2 = den - shift[r];
      if ((d2 > 0) == (den > 0) && fabs(d2) > 0.2 * fabs(den)) den = d2;
      double* p = R + (size_t)c * ld + r;
      if (fabs(den) > 1e-12)
        *p = *p / den;
      else
        *p = *p / (den - 1.e-12);
    }
}
void precondition_shift(const double* diag, const double* shift, const double* lam, int k, size_t N, double* R,
                        size_t ld, cudaStream_t s) {
  k_precondition_shift<<<grid_for(N, 256), 256, 0, s>>>(diag, shift, lam, k, N, R, ld);
  SHCI_LAUNCH_CHECK();
}

__global__ void k_scale_inv_norm(double* __restrict__ c, size_t N, const double* __restrict__ g) {
  const double nrm = sqrt(g[0]);
  if (!(nrm > 1e-14)) return;  // linearly dependent: left for the host to drop
  const double sc = 1.0 / nrm;
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x)
    c[r] *= sc;
}
void scale_inv_norm(double* c, size_t N, const double* g, cudaStream_t s) {
  k_scale_inv_norm<<<grid_for(N, 256), 256, 0, s>>>(c, N, g);
  SHCI_LAUNCH_CHECK();
}

__global__ void k_scale_cols(double* __restrict__ A, size_t ld, const double* __restrict__ sc, int k, size_t N) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (size_t)gridDim.x * blockDim.x)
    for (int c = 0; c < k; ++c) A[(size_t)c * ld + r] *= sc[c];
}
void scale_cols(double* A, size_t ld, const double* scale, int k, size_t N, cudaStream_t s) {
  k_scale_cols<<<grid_for(N, 256), 256, 0, s>>>(A, ld, scale, k, N);
  SHCI_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Allocation-free sigma (shci_sigma_device_noalloc). The row-interleaved copy
// of x that the sigma kernels gather from lives in this fixed device array
// instead of a context buffer, so a call never allocates. Every GPU that loads
// the library holds the array until the process exits. All calls share it and
// each call overwrites the part it uses (including the zero padding), so
// nothing has to be cleared between calls; calls that overlap on the GPU
// (different streams or contexts at the same time) race on it.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_sigma_pack_scratch[kNoAllocPackBytes];

// Device address of the array on the current device. Host code cannot use
// the symbol itself: on the host it names a stand-in, not device memory. The
// context calls this while it builds a stored Hamiltonian (a call that may
// allocate and load this file's kernels), so the allocation-free sigma itself
// only reads the address the context kept.
void* noalloc_scratch_address() {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_sigma_pack_scratch);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(kErrCuda, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
  }
  return p;
}

void sigma_noalloc(const Csr& H, const double* diag, int mode_mixed, const double* x, size_t ldx, int k, double* y,
                   size_t ldy, void* scratch, cudaStream_t s) {
  const size_t N = H.N;
  const int kp = k == 3 ? 4 : k;
  const size_t need = N * (size_t)kp * (mode_mixed ? sizeof(float) : sizeof(double));
  if (need > kNoAllocPackBytes)
    throw Error(kErrInvalid, "allocation-free sigma: N x k = " + std::to_string(N) + " x " + std::to_string(kp) +
                                 " needs " + std::to_string(need) + " bytes of scratch, the fixed maximum is " +
                                 std::to_string(kNoAllocPackBytes));
  if (!scratch) throw Error(kErrState, "allocation-free sigma: scratch address not set up (build the Hamiltonian)");
  if (mode_mixed) {
    pack_f32(x, ldx, 0, k, kp, N, static_cast<float*>(scratch), s, H.perm.p);
    sigma_csr_mixed(H, diag, static_cast<const float*>(scratch), kp, k, y, ldy, s);
  } else {
    if (H.v64.p) {
      pack_f64(x, ldx, 0, k, kp, N, static_cast<double*>(scratch), s, H.perm.p);
      sigma_csr_f64(H, diag, static_cast<const double*>(scratch), kp, k, y, ldy, s);
    } else {  // head + tail values: float-float refinement sigma (same 8 bytes per entry)
      pack_ff(x, ldx, 0, k, kp, N, static_cast<float*>(scratch), s, H.perm.p);
      sigma_csr_ff(H, diag, static_cast<const float*>(scratch), kp, x, ldx, 0, k, y, ldy, s);
    }
  }
}

}  // namespace shci
