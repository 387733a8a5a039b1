// Learned preconditioner correction (kernels_mlp.cu).
#pragma once
#include <cuda_bf16.h>

#include "ham.h"

namespace shci {

constexpr int kHidden = 128;

struct MlpView {
  int F, nspin;
  const __nv_bfloat16* W1b;  // kHidden x F
  const __nv_bfloat16* W2b;  // kHidden x kHidden
  const float *b1, *b2, *w3, *b3;
  int nparam, offW1, offW2, offb1, offb2, offw3, offb3;
};

// Second-order level shift of every row of the stored Hamiltonian at energy E:
// s_i = sum_j H_ij^2 / (E - diag_j).
void pt2_shift(const Csr& H, const double* diag, double E, double* s, DevBuf<float>& inv, cudaStream_t st);

// Training sample on the device: idx[k] = a hashed row (with replacement),
// tgt[k] = teacher[idx[k]] / rms; returns the rms (one small read-back).
double mlp_sample(const double* teacher, size_t N, int64_t ns, uint64_t seed, int32_t* idx, float* tgt,
                  DevBuf<double>& part, cudaStream_t s);

// Davidson (residual, correction) pairs of one recorded iteration (x_k, r_k,
// theta_k) against the converged vector x* (ck = x* . x_k): the shifts
// s_i = -r_i / e_i - (H_ii - theta_k), e = x*/ck - x_k, of the informative
// entries are appended to (cidx, ctgt) at `base`; returns how many.
int64_t pair_targets(const double* xk, const double* rk, const double* xstar, double ck, const double* diag,
                     double theta, size_t N, double r_floor, double e_floor, int64_t base, DevBuf<int32_t>& cidx,
                     DevBuf<double>& ctgt, DevBuf<double>& tmp, DevBuf<int64_t>& flag, DevBuf<int64_t>& pos, Prims& pr,
                     cudaStream_t s);
// Training sample of ns pairs from the m collected ones, targets scaled to
// unit rms; returns the rms.
double mlp_sample_pairs(const int32_t* cidx, const double* ctgt, int64_t m, int64_t ns, uint64_t seed, int32_t* idx,
                        float* tgt, DevBuf<double>& part, cudaStream_t s);

// The plain preconditioner as judge of the learned one: on a held-out
// recorded iteration, |cos| of the angle between the correction each would
// have produced (plain r_i / (theta - H_ii), shifted by `shift` where the
// preconditioner keeps the shift) and the correction e = x*/ck - x_k the
// iteration needed.
void judge_preconditioners(const double* xk, const double* rk, const double* xstar, double ck, const double* diag,
                           const double* shift, double theta, size_t N, DevBuf<double>& part, cudaStream_t s,
                           double* cos_plain, double* cos_learned);

struct Mlp {
  int nspin = 0, F = 0, nparam = 0;
  int offW1 = 0, offW2 = 0, offb1 = 0, offb2 = 0, offw3 = 0, offb3 = 0;
  int step = 0;
  double sigma = 1.0;  // target scale: prediction = output * sigma
  bool trained = false;
  DevBuf<float> params, mom, var, grad, part, lpart;
  DevBuf<__nv_bfloat16> wb;

  void init(int nspin, uint64_t seed, cudaStream_t s);
  void set_params(const std::vector<float>& h, cudaStream_t s);
  std::vector<float> get_params(cudaStream_t s) const;
  MlpView view() const;
  // mean squared error of the batch (rows idx, targets already divided by
  // sigma) and its gradient into `grad`
  // Loss (read back, one synchronisation) only when want_loss; NaN otherwise.
  float gradient(const Det2* dets, const double* diag, const int32_t* idx, const float* target, int B, double E,
                 cudaStream_t s, bool want_loss = true);
  void adam(float lr, cudaStream_t s);
  // out[i] = sigma * net(features of det i)
  void infer(const Det2* dets, const double* diag, size_t N, double E, double* out, cudaStream_t s) const;
};

}  // namespace shci
