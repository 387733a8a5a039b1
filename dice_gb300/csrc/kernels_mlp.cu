// Learned correction of the Davidson preconditioner (no counterpart in the
// reference, whose preconditioner is r_i / (theta - H_ii), SHCI/Davidson.cpp:85-106).
//
// The correction is a per-determinant shift s_i of the denominator,
//   t_i = r_i / (theta - H_ii - s_i).
// During a variational run the network learns s_i from the (residual,
// correction) pairs Davidson itself generates (pair_targets below): the shift
// that would have turned each recorded residual entry into the correction the
// solve turned out to need. A second target, the second-order level shift of
// determinant i inside the variational space, s_i = sum_j H_ij^2 / (E - H_jj)
// (computed from the stored Hamiltonian at the Davidson energy E), serves the
// explicit training entry point. A small MLP learns s_i from the determinant
// itself:
//   features: per spatial orbital "doubly occupied" and "singly occupied"
//             (2n values, spin-free), (H_ii - E) / 10, and 1;
//   net:      F -> 128 -> 128 -> 1, ReLU, weights stored in BF16,
//             FP32 master weights and Adam moments;
//   target:   s_i / sigma (sigma = RMS of the teacher shifts).
// The forward, backward and Adam kernels below are the project's own; the
// hidden activations are kept in FP32 inside the kernels.
#include <algorithm>
#include <cuda_bf16.h>

#include "ham.h"
#include "mlp.h"

namespace shci {

// ---------------------------------------------------------------------------
// teacher: s_i = sum_j h_ij^2 / (E - d_j) over stored row i. The reciprocals
// 1 / (E - d_j) are formed once per determinant (a division per nonzero would
// run on this GPU's slow FP64 divide path); the row sums run in FP32, ample
// for a level shift that only scales the preconditioner. The reciprocals are
// laid out in the matrix's storage order (inv[j] belongs to determinant
// perm[j]), the shifts in the determinant array's order.
// ---------------------------------------------------------------------------
__global__ void k_pt2_inverse(const double* __restrict__ diag, const uint32_t* __restrict__ perm, size_t N, double E,
                              float* __restrict__ inv) {
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (size_t)gridDim.x * blockDim.x) {
    const double den = E - diag[perm[j]];
    inv[j] = fabs(den) > 1e-8 ? (float)(1.0 / den) : 0.f;
  }
}
template <bool F64>
__global__ void k_pt2_shift(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                            const double* __restrict__ v64, const float* __restrict__ vhi,
                            const float* __restrict__ inv, const uint32_t* __restrict__ perm, size_t N,
                            double* __restrict__ s) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < (int64_t)N; r += warps) {
    float acc = 0.f;
    for (int64_t p = rowptr[r] + lane; p < rowptr[r + 1]; p += 32) {
      const float h = F64 ? (float)v64[p] : vhi[p];
      acc = fmaf(h * h, __ldg(inv + col[p]), acc);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if (lane == 0) s[perm[r]] = (double)acc;
  }
}

void pt2_shift(const Csr& H, const double* diag, double E, double* s, DevBuf<float>& inv, cudaStream_t st) {
  if (H.N == 0) return;
  inv.reserve(H.N);
  k_pt2_inverse<<<(unsigned)std::min<size_t>((H.N + 255) / 256, 152 * 32), 256, 0, st>>>(diag, H.perm.p, H.N, E,
                                                                                       inv.p);
  SHCI_LAUNCH_CHECK();
  size_t blocks = (H.N * 32 + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (H.v64.p)
    k_pt2_shift<true><<<(unsigned)blocks, 256, 0, st>>>(H.rowptr.p, H.col.p, H.v64.p, nullptr, inv.p, H.perm.p, H.N, s);
  else
    k_pt2_shift<false><<<(unsigned)blocks, 256, 0, st>>>(H.rowptr.p, H.col.p, nullptr, H.vhi.p, inv.p, H.perm.p, H.N, s);
  SHCI_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// network
// ---------------------------------------------------------------------------
// Spin-free occupation features: f < n is "orbital f doubly occupied",
// n <= f < 2n is "orbital f-n singly occupied". They are invariant under the
// alpha <-> beta flip, so the predicted shift is too -- a flip-asymmetric
// preconditioner would let a Davidson run leave the flip sector of its start
// vector (see the note on compensated accumulation in kernels_sigma.cu).
__device__ __forceinline__ float feature(const Det2& d, int f, int nspin, float dscaled) {
  const int n = nspin >> 1;
  if (f < n) return (det_getocc(d, 2 * f) && det_getocc(d, 2 * f + 1)) ? 1.f : 0.f;
  if (f < nspin) return (det_getocc(d, 2 * (f - n)) != det_getocc(d, 2 * (f - n) + 1)) ? 1.f : 0.f;
  if (f == nspin) return dscaled;
  if (f == nspin + 1) return 1.f;
  return 0.f;
}

// Shared-memory layout of one block (kHidden threads, one per hidden unit).
struct MlpSmem {
  __nv_bfloat16* W1;  // kHidden x F (row j = unit j)
  __nv_bfloat16* W2;  // kHidden x kHidden
  float* x;           // F
  float* h1;          // kHidden
  float* h2;          // kHidden
  float* red;         // kHidden / 32 partial sums
};

__device__ __forceinline__ MlpSmem carve(unsigned char* base, int F) {
  MlpSmem m;
  m.W1 = reinterpret_cast<__nv_bfloat16*>(base);
  m.W2 = m.W1 + (size_t)kHidden * F;
  float* f = reinterpret_cast<float*>(m.W2 + (size_t)kHidden * kHidden);
  m.x = f;
  m.h1 = m.x + F;
  m.h2 = m.h1 + kHidden;
  m.red = m.h2 + kHidden;
  return m;
}
size_t mlp_fwd_smem(int F) {
  return (size_t)kHidden * F * 2 + (size_t)kHidden * kHidden * 2 + ((size_t)F + 2 * kHidden + kHidden / 32) * 4;
}

__device__ __forceinline__ void load_weights(const MlpView& w, MlpSmem& m, int F) {
  for (int i = threadIdx.x; i < kHidden * F; i += blockDim.x) m.W1[i] = w.W1b[i];
  for (int i = threadIdx.x; i < kHidden * kHidden; i += blockDim.x) m.W2[i] = w.W2b[i];
  __syncthreads();
}

// forward of one sample by the block; returns the output in every thread
__device__ __forceinline__ float forward_one(const MlpView& w, MlpSmem& m, int F) {
  const int j = threadIdx.x;
  float a = w.b1[j];
  for (int f = 0; f < F; ++f) a += __bfloat162float(m.W1[(size_t)j * F + f]) * m.x[f];
  m.h1[j] = fmaxf(a, 0.f);
  __syncthreads();
  float b = w.b2[j];
  for (int k = 0; k < kHidden; ++k) b += __bfloat162float(m.W2[(size_t)j * kHidden + k]) * m.h1[k];
  const float h2 = fmaxf(b, 0.f);
  m.h2[j] = h2;
  float o = w.w3[j] * h2;
#pragma unroll
  for (int s = 16; s; s >>= 1) o += __shfl_xor_sync(kFull, o, s);
  if ((j & 31) == 0) m.red[j >> 5] = o;
  __syncthreads();
  float out = w.b3[0];
  for (int q = 0; q < kHidden / 32; ++q) out += m.red[q];
  __syncthreads();
  return out;
}

__global__ void __launch_bounds__(kHidden) k_mlp_infer(MlpView w, const Det2* __restrict__ dets,
                                                       const double* __restrict__ diag, size_t N, double E,
                                                       double sigma, double* __restrict__ out) {
  extern __shared__ unsigned char sm_raw[];
  const int F = w.F, nspin = w.nspin;
  MlpSmem m = carve(sm_raw, F);
  load_weights(w, m, F);
  for (size_t i = blockIdx.x; i < N; i += gridDim.x) {
    const Det2 d = dets[i];
    const float ds = (float)((diag[i] - E) * 0.1);
    for (int f = threadIdx.x; f < F; f += blockDim.x) m.x[f] = feature(d, f, nspin, ds);
    __syncthreads();
    const float o = forward_one(w, m, F);
    if (threadIdx.x == 0) out[i] = (double)o * sigma;
  }
}

// Gradients of the mean squared error over a batch. Every block keeps its own
// FP32 gradient in shared memory (thread j owns row j of dW1 and dW2) and
// writes it to its slice of `part`; k_mlp_grad_sum adds the slices in block
// order, so the result does not depend on scheduling.
__global__ void __launch_bounds__(kHidden) k_mlp_grad(MlpView w, const Det2* __restrict__ dets,
                                                      const double* __restrict__ diag, const int32_t* __restrict__ idx,
                                                      const float* __restrict__ target, int B, double E,
                                                      float* __restrict__ part, float* __restrict__ loss_part) {
  extern __shared__ unsigned char sm_raw[];
  const int F = w.F, nspin = w.nspin, j = threadIdx.x;
  MlpSmem m = carve(sm_raw, F);
  float* gW1 = reinterpret_cast<float*>(m.red + kHidden / 32);  // kHidden x F
  float* gW2 = gW1 + (size_t)kHidden * F;                        // kHidden x kHidden
  float* dh2 = gW2 + (size_t)kHidden * kHidden;                  // kHidden
  load_weights(w, m, F);
  for (int f = 0; f < F; ++f) gW1[(size_t)j * F + f] = 0.f;
  for (int k = 0; k < kHidden; ++k) gW2[(size_t)j * kHidden + k] = 0.f;
  float gb1 = 0.f, gb2 = 0.f, gw3 = 0.f, gb3 = 0.f, loss = 0.f;
  __syncthreads();
  const float inv = 2.f / (float)B;
  for (int s = blockIdx.x; s < B; s += gridDim.x) {
    const int i = idx[s];
    const Det2 d = dets[i];
    const float ds = (float)((diag[i] - E) * 0.1);
    for (int f = threadIdx.x; f < F; f += blockDim.x) m.x[f] = feature(d, f, nspin, ds);
    __syncthreads();
    const float o = forward_one(w, m, F);
    const float err = o - target[s];
    loss += (j == 0) ? err * err / (float)B : 0.f;
    const float dout = inv * err;
    gb3 += (j == 0) ? dout : 0.f;
    const float h2 = m.h2[j];
    gw3 += dout * h2;
    const float g2 = (h2 > 0.f) ? dout * w.w3[j] : 0.f;
    dh2[j] = g2;
    gb2 += g2;
    for (int k = 0; k < kHidden; ++k) gW2[(size_t)j * kHidden + k] += g2 * m.h1[k];
    __syncthreads();
    // dh1[j] = sum_k dh2[k] W2[k][j]
    float g1 = 0.f;
    for (int k = 0; k < kHidden; ++k) g1 += dh2[k] * __bfloat162float(m.W2[(size_t)k * kHidden + j]);
    g1 = (m.h1[j] > 0.f) ? g1 : 0.f;
    gb1 += g1;
    for (int f = 0; f < F; ++f) gW1[(size_t)j * F + f] += g1 * m.x[f];
    __syncthreads();
  }
  float* mypart = part + (size_t)blockIdx.x * w.nparam;
  for (int f = 0; f < F; ++f) mypart[w.offW1 + (size_t)j * F + f] = gW1[(size_t)j * F + f];
  for (int k = 0; k < kHidden; ++k) mypart[w.offW2 + (size_t)j * kHidden + k] = gW2[(size_t)j * kHidden + k];
  mypart[w.offb1 + j] = gb1;
  mypart[w.offb2 + j] = gb2;
  mypart[w.offw3 + j] = gw3;
  if (j == 0) {
    mypart[w.offb3] = gb3;
    loss_part[blockIdx.x] = loss;
  }
}
size_t mlp_grad_smem(int F) {
  return mlp_fwd_smem(F) + ((size_t)kHidden * F + (size_t)kHidden * kHidden + kHidden) * 4;
}

__global__ void k_mlp_grad_sum(const float* __restrict__ part, int nblocks, int nparam, float* __restrict__ g) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nparam; i += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * nparam + i];
    g[i] = s;
  }
}

// Adam on the FP32 master weights; refreshes the BF16 copies used by the kernels.
__global__ void k_adam(float* __restrict__ p, float* __restrict__ mo, float* __restrict__ ve,
                       const float* __restrict__ g, int n, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ pb, int nb) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float m = b1 * mo[i] + (1.f - b1) * gi;
    const float v = b2 * ve[i] + (1.f - b2) * gi * gi;
    mo[i] = m;
    ve[i] = v;
    const float np = p[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
    p[i] = np;
    if (i < nb) pb[i] = __float2bfloat16_rn(np);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
void Mlp::init(int nspin_, uint64_t seed, cudaStream_t s) {
  nspin = nspin_;
  F = nspin + 2;
  offW1 = 0;
  offW2 = offW1 + kHidden * F;
  offb1 = offW2 + kHidden * kHidden;
  offb2 = offb1 + kHidden;
  offw3 = offb2 + kHidden;
  offb3 = offw3 + kHidden;
  nparam = offb3 + 1;
  std::vector<float> h(nparam, 0.f);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 12345;
  auto rnd = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return (float)(((st >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0);
  };
  const float a1 = std::sqrt(6.f / (float)(F + kHidden)), a2 = std::sqrt(6.f / (2.f * kHidden));
  for (int i = 0; i < kHidden * F; ++i) h[offW1 + i] = a1 * rnd();
  for (int i = 0; i < kHidden * kHidden; ++i) h[offW2 + i] = a2 * rnd();
  for (int i = 0; i < kHidden; ++i) h[offw3 + i] = a2 * rnd();
  set_params(h, s);
  step = 0;
  sigma = 1.0;
  trained = false;
}

void Mlp::set_params(const std::vector<float>& h, cudaStream_t s) {
  if ((int)h.size() != nparam) throw Error(kErrInvalid, "MLP parameter count mismatch");
  params.resize(nparam);
  mom.resize(nparam);
  var.resize(nparam);
  grad.resize(nparam);
  wb.resize((size_t)offb1);  // BF16 copies of W1 and W2 (contiguous at the start)
  SHCI_CUDA(cudaMemcpyAsync(params.p, h.data(), nparam * sizeof(float), cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaMemsetAsync(mom.p, 0, nparam * sizeof(float), s));
  SHCI_CUDA(cudaMemsetAsync(var.p, 0, nparam * sizeof(float), s));
  std::vector<__nv_bfloat16> b(offb1);
  for (int i = 0; i < offb1; ++i) b[i] = __float2bfloat16_rn(h[i]);
  SHCI_CUDA(cudaMemcpyAsync(wb.p, b.data(), offb1 * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  step = 0;
}

std::vector<float> Mlp::get_params(cudaStream_t s) const {
  std::vector<float> h(nparam);
  SHCI_CUDA(cudaMemcpyAsync(h.data(), params.p, nparam * sizeof(float), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  return h;
}

MlpView Mlp::view() const {
  MlpView v;
  v.F = F;
  v.nspin = nspin;
  v.W1b = wb.p + offW1;
  v.W2b = wb.p + offW2;
  v.b1 = params.p + offb1;
  v.b2 = params.p + offb2;
  v.w3 = params.p + offw3;
  v.b3 = params.p + offb3;
  v.nparam = nparam;
  v.offW1 = offW1;
  v.offW2 = offW2;
  v.offb1 = offb1;
  v.offb2 = offb2;
  v.offw3 = offw3;
  v.offb3 = offb3;
  return v;
}

constexpr int kGradBlocks = 152 * 2;

constexpr unsigned kSampleBlocks = 152;
__global__ void k_mlp_sample(const double* __restrict__ teacher, size_t N, int64_t ns, uint64_t seed,
                             int32_t* __restrict__ idx, float* __restrict__ tgt, double* __restrict__ part) {
  __shared__ double red[8];
  double ss = 0.0;
  const int64_t per = (ns + gridDim.x - 1) / gridDim.x;
  const int64_t k0 = (int64_t)blockIdx.x * per, k1 = k0 + per < ns ? k0 + per : ns;
  for (int64_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    const size_t i = (size_t)(mix64(seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(k + 1))) % N);
    const double t = teacher[i];
    idx[k] = (int32_t)i;
    tgt[k] = (float)t;
    ss += t * t;
  }
  for (int o = 16; o; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
    part[blockIdx.x] = v;
  }
}
__global__ void k_mlp_scale_targets(float* __restrict__ tgt, int64_t ns, const double* __restrict__ part, int np) {
  double ss = 0.0;
  for (int b = 0; b < np; ++b) ss += part[b];
  double rms = ns > 0 ? sqrt(ss / (double)ns) : 1.0;
  if (!(rms > 0.0)) rms = 1.0;
  const float inv = (float)(1.0 / rms);
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += (int64_t)gridDim.x * blockDim.x)
    tgt[k] *= inv;
}
double mlp_sample(const double* teacher, size_t N, int64_t ns, uint64_t seed, int32_t* idx, float* tgt,
                  DevBuf<double>& part, cudaStream_t s) {
  if (N == 0 || ns <= 0) return 1.0;
  part.reserve(kSampleBlocks);
  k_mlp_sample<<<kSampleBlocks, 256, 0, s>>>(teacher, N, ns, seed, idx, tgt, part.p);
  SHCI_LAUNCH_CHECK();
  k_mlp_scale_targets<<<kSampleBlocks, 256, 0, s>>>(tgt, ns, part.p, (int)kSampleBlocks);
  SHCI_LAUNCH_CHECK();
  std::vector<double> h(kSampleBlocks);
  SHCI_CUDA(cudaMemcpyAsync(h.data(), part.p, kSampleBlocks * sizeof(double), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  double ss = 0.0;
  for (double v : h) ss += v;
  double rms = std::sqrt(ss / (double)ns);
  return rms > 0.0 ? rms : 1.0;
}

// ---------------------------------------------------------------------------
// Targets from Davidson's own (residual, correction) pairs. At iteration k of
// a solve the Ritz vector x_k has residual r_k = H x_k - theta_k x_k; once the
// solve has converged to x*, the correction that iteration needed is
// e = x* / (x* . x_k) - x_k, and to first order (H - theta_k) e = -r_k. The
// diagonal preconditioner approximates (H - theta)^-1 by 1 / (H_ii - theta);
// the denominator that would have produced e_i from r_i exactly is
// -r_i / e_i = H_ii - theta + s_i, so the per-determinant shift the network
// learns is s_i = -r_i / e_i - (H_ii - theta). Entries where r_i or e_i is
// at the rounding level carry no information and are dropped, as are shifts
// that would flip the sign of the plain denominator or exceed twice its size
// (the preconditioner refuses such shifts anyway).
// ---------------------------------------------------------------------------
__global__ void k_pair_targets(const double* __restrict__ xk, const double* __restrict__ rk,
                               const double* __restrict__ xstar, double inv_ck, const double* __restrict__ diag,
                               double theta, size_t N, double r_floor, double e_floor, double* __restrict__ tgt,
                               int64_t* __restrict__ flag) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
    const double e = xstar[i] * inv_ck - xk[i];
    const double r = rk[i];
    const double d = diag[i] - theta;
    double sh = 0.0;
    bool ok = fabs(e) > e_floor && fabs(r) > r_floor && fabs(d) > 1e-8;
    if (ok) {
      const double den = -r / e;
      sh = den - d;
      ok = (den > 0.0) == (d > 0.0) && fabs(sh) <= 2.0 * fabs(d) && isfinite(sh);
    }
    tgt[i] = ok ? sh : 0.0;
    flag[i] = ok ? 1 : 0;
  }
}
__global__ void k_pair_compact(const double* __restrict__ tgt, const int64_t* __restrict__ flag,
                               const int64_t* __restrict__ pos, size_t N, int64_t base, int32_t* __restrict__ cidx,
                               double* __restrict__ ctgt) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x)
    if (flag[i]) {
      cidx[base + pos[i]] = (int32_t)i;
      ctgt[base + pos[i]] = tgt[i];
    }
}
// Sample of ns pairs drawn (hashed, with replacement) from the m valid ones.
__global__ void k_mlp_sample_pairs(const int32_t* __restrict__ cidx, const double* __restrict__ ctgt, int64_t m,
                                   int64_t ns, uint64_t seed, int32_t* __restrict__ idx, float* __restrict__ tgt,
                                   double* __restrict__ part) {
  __shared__ double red[8];
  double ss = 0.0;
  const int64_t per = (ns + gridDim.x - 1) / gridDim.x;
  const int64_t k0 = (int64_t)blockIdx.x * per, k1 = k0 + per < ns ? k0 + per : ns;
  for (int64_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    const int64_t j = (int64_t)(mix64(seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(k + 1))) % (uint64_t)m);
    const double t = ctgt[j];
    idx[k] = cidx[j];
    tgt[k] = (float)t;
    ss += t * t;
  }
  for (int o = 16; o; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
    part[blockIdx.x] = v;
  }
}

int64_t pair_targets(const double* xk, const double* rk, const double* xstar, double ck, const double* diag,
                     double theta, size_t N, double r_floor, double e_floor, int64_t base, DevBuf<int32_t>& cidx,
                     DevBuf<double>& ctgt, DevBuf<double>& tmp, DevBuf<int64_t>& flag, DevBuf<int64_t>& pos, Prims& pr,
                     cudaStream_t s) {
  tmp.reserve(N);
  flag.reserve(N);
  pos.reserve(N);
  const unsigned blocks = (unsigned)std::min<size_t>((N + 255) / 256, 152 * 16);
  k_pair_targets<<<blocks, 256, 0, s>>>(xk, rk, xstar, 1.0 / ck, diag, theta, N, r_floor, e_floor, tmp.p, flag.p);
  SHCI_LAUNCH_CHECK();
  int64_t m = 0;
  scan_exclusive_i64(flag.p, pos.p, N, &m, pr, s);
  cidx.grow_keep((size_t)(base + m), s);
  ctgt.grow_keep((size_t)(base + m), s);
  k_pair_compact<<<blocks, 256, 0, s>>>(tmp.p, flag.p, pos.p, N, base, cidx.p, ctgt.p);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaStreamSynchronize(s));
  return m;
}

double mlp_sample_pairs(const int32_t* cidx, const double* ctgt, int64_t m, int64_t ns, uint64_t seed, int32_t* idx,
                        float* tgt, DevBuf<double>& part, cudaStream_t s) {
  if (m <= 0 || ns <= 0) return 1.0;
  part.reserve(kSampleBlocks);
  k_mlp_sample_pairs<<<kSampleBlocks, 256, 0, s>>>(cidx, ctgt, m, ns, seed, idx, tgt, part.p);
  SHCI_LAUNCH_CHECK();
  k_mlp_scale_targets<<<kSampleBlocks, 256, 0, s>>>(tgt, ns, part.p, (int)kSampleBlocks);
  SHCI_LAUNCH_CHECK();
  std::vector<double> h(kSampleBlocks);
  SHCI_CUDA(cudaMemcpyAsync(h.data(), part.p, kSampleBlocks * sizeof(double), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  double ss = 0.0;
  for (double v : h) ss += v;
  const double rms = std::sqrt(ss / (double)ns);
  return rms > 0.0 ? rms : 1.0;
}

// The judge: on a recorded iteration (x_k, r_k, theta_k) of a converged solve
// (x*, ck = x* . x_k), how well the plain and the shifted preconditioners
// would have pointed at the correction that iteration needed,
// e = x*/ck - x_k. Sums over the determinants of <t, e>, <t, t> for the plain
// t_i = r_i / (theta - H_ii) and for the shifted one (the shift kept only
// where the preconditioner keeps it, as k_precondition_shift does), and
// <e, e>, per block into part[6 * block].
__global__ void k_judge(const double* __restrict__ xk, const double* __restrict__ rk,
                        const double* __restrict__ xstar, double inv_ck, const double* __restrict__ diag,
                        const double* __restrict__ shift, double theta, size_t N, double* __restrict__ part) {
  __shared__ double red[5][8];
  double a[5] = {0, 0, 0, 0, 0};
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (size_t)gridDim.x * blockDim.x) {
    const double e = xstar[i] * inv_ck - xk[i];
    double den = theta - diag[i];
    if (!(fabs(den) > 1e-12)) den -= 1e-12;
    const double tp = rk[i] / den;
    double dl = den;
    const double d2 = den - shift[i];
    if ((d2 > 0) == (den > 0) && fabs(d2) > 0.2 * fabs(den)) dl = d2;
    const double tl = rk[i] / dl;
    a[0] += tp * e;
    a[1] += tp * tp;
    a[2] += tl * e;
    a[3] += tl * tl;
    a[4] += e * e;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    double v = a[q];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[q][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double v = 0.0;
    for (int u = 0; u < (int)(blockDim.x >> 5); ++u) v += red[threadIdx.x][u];
    part[(size_t)blockIdx.x * 6 + threadIdx.x] = v;
  }
}

void judge_preconditioners(const double* xk, const double* rk, const double* xstar, double ck, const double* diag,
                           const double* shift, double theta, size_t N, DevBuf<double>& part, cudaStream_t s,
                           double* cos_plain, double* cos_learned) {
  const unsigned blocks = (unsigned)std::max<size_t>(1, std::min<size_t>((N + 255) / 256, 152 * 4));
  part.reserve((size_t)blocks * 6);
  k_judge<<<blocks, 256, 0, s>>>(xk, rk, xstar, 1.0 / ck, diag, shift, theta, N, part.p);
  SHCI_LAUNCH_CHECK();
  std::vector<double> h((size_t)blocks * 6);
  SHCI_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  double a[5] = {0, 0, 0, 0, 0};
  for (unsigned b = 0; b < blocks; ++b)
    for (int q = 0; q < 5; ++q) a[q] += h[(size_t)b * 6 + q];
  const double ne = std::sqrt(a[4]);
  *cos_plain = (a[1] > 0 && ne > 0) ? std::fabs(a[0]) / (std::sqrt(a[1]) * ne) : 0.0;
  *cos_learned = (a[3] > 0 && ne > 0) ? std::fabs(a[2]) / (std::sqrt(a[3]) * ne) : 0.0;
}

float Mlp::gradient(const Det2* dets, const double* diag, const int32_t* idx, const float* target, int B, double E,
                    cudaStream_t s, bool want_loss) {
  const size_t smem = mlp_grad_smem(F);
  SHCI_CUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int nb = std::min(kGradBlocks, std::max(1, B));
  part.reserve((size_t)nb * nparam);
  lpart.reserve(nb);
  k_mlp_grad<<<nb, kHidden, smem, s>>>(view(), dets, diag, idx, target, B, E, part.p, lpart.p);
  SHCI_LAUNCH_CHECK();
  k_mlp_grad_sum<<<(nparam + 255) / 256, 256, 0, s>>>(part.p, nb, nparam, grad.p);
  SHCI_LAUNCH_CHECK();
  if (!want_loss) return std::nanf("");
  std::vector<float> lp(nb);
  SHCI_CUDA(cudaMemcpyAsync(lp.data(), lpart.p, nb * sizeof(float), cudaMemcpyDeviceToHost, s));
  SHCI_CUDA(cudaStreamSynchronize(s));
  float loss = 0.f;
  for (float v : lp) loss += v;
  return loss;
}

void Mlp::adam(float lr, cudaStream_t s) {
  ++step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
  k_adam<<<(nparam + 255) / 256, 256, 0, s>>>(params.p, mom.p, var.p, grad.p, nparam, lr, b1, b2, 1e-8f, c1, c2,
                                             wb.p, offb1);
  SHCI_LAUNCH_CHECK();
}

void Mlp::infer(const Det2* dets, const double* diag, size_t N, double E, double* out, cudaStream_t s) const {
  if (N == 0) return;
  const size_t smem = mlp_fwd_smem(F);
  SHCI_CUDA(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned blocks = (unsigned)std::min<size_t>(N, 152 * 8);
  k_mlp_infer<<<blocks, kHidden, smem, s>>>(view(), dets, diag, N, E, sigma, out);
  SHCI_LAUNCH_CHECK();
}

}  // namespace shci
