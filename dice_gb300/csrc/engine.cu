// Engine context, device Davidson solver, the variational driver and the
// C-ABI entry points of libshci_gpu (include/shci_gpu.h).
//
// Davidson (replaces davidson / davidsonDirect, SHCI/Davidson.cpp:111-590):
// the basis V and its sigma W live on the device in FP64 (column-major). Each
// iteration forms G = V^T W (one fused Gram pass), solves the small symmetric
// eigenproblem on the host in FP64, forms Ritz vectors X = V Q, HX = W Q and
// residuals R = HX - lambda X on the device, and appends preconditioned,
// orthogonalised corrections. An iteration is two CUDA graphs, captured once
// per basis size and active-root set and replayed after that: (1) Ritz
// vectors, residuals and their norms; (2) corrections, orthonormalisation,
// collapse, append, sigma and the next Gram matrix. The host reads back only
// the small matrices (two synchronisations per iteration). The basis is only rotated on collapse; the
// subspace sequence is the reference's (same maxCopies, same collapse to the
// lowest nroots+2 Ritz vectors, corrections orthogonalised against the whole
// basis before the collapse). Block mode adds one correction per unconverged
// root and applies sigma to all of them in one k-vector launch.
//
// Mixed precision: sigma runs in FP32 (FP32 CSR values and vectors, FP32
// accumulation, FP64 diagonal term) until the residual tolerance is met; the
// solve then restarts from the converged Ritz vectors with sigma in FP64
// (FP32 head + FP32 tail of every element), which refines the Ritz pairs and
// yields FP64 Rayleigh quotients.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <unordered_map>

#include "../../include/shci_gpu.h"
#include "ham.h"
#include "host_io.h"
#include "mlp.h"

namespace shci {

std::atomic<int64_t> g_launch_count{0};

// Residual norm below which the FP32 stage of the mixed solver may stop on
// stagnation and hand over to the FP64 stage.
constexpr double kStallWindow = 2e-5;
// |<x|F|x>| above which a vector counts as having a definite flip parity.
constexpr double kParityDefinite = 0.999;

// SHCI_TRACE=1 prints one line per Davidson iteration to stderr, 2 also the
// phases of the Hamiltonian build.
int trace_level() {
  static const int level = [] {
    const char* v = std::getenv("SHCI_TRACE");
    return v ? std::atoi(v) : 0;
  }();
  return level;
}
static double wall_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
PhaseTimer::PhaseTimer(cudaStream_t st) : s(st), t0(trace_level() >= 2 ? wall_s() : 0.0) {}
void PhaseTimer::mark(const char* what) {
  if (trace_level() < 2) return;
  cudaStreamSynchronize(s);
  const double t = wall_s();
  std::fprintf(stderr, "[phase] %-16s %9.3f ms\n", what, (t - t0) * 1e3);
  t0 = t;
}

static inline unsigned grid_for(size_t n, int threads, size_t max_blocks = 152 * 32) {
  size_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (unsigned)b;
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Dense symmetric eigensolver (cyclic Jacobi), ascending eigenvalues; A is
// m x m row-major, evecs column-major (column c = eigenvector c).
static void sym_eig(int m, std::vector<double> A, std::vector<double>& evals, std::vector<double>& evecs) {
  std::vector<double> V((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) V[(size_t)i * m + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int p = 0; p < m; ++p) {
      diag += A[(size_t)p * m + p] * A[(size_t)p * m + p];
      for (int q = p + 1; q < m; ++q) off += A[(size_t)p * m + q] * A[(size_t)p * m + q];
    }
    if (off <= 1e-32 * diag || off < 1e-300) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = A[(size_t)p * m + q];
        if (apq == 0.0) continue;
        const double app = A[(size_t)p * m + p], aqq = A[(size_t)q * m + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < m; ++k) {
          double akp = A[(size_t)k * m + p], akq = A[(size_t)k * m + q];
          A[(size_t)k * m + p] = c * akp - s * akq;
          A[(size_t)k * m + q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {
          double apk = A[(size_t)p * m + k], aqk = A[(size_t)q * m + k];
          A[(size_t)p * m + k] = c * apk - s * aqk;
          A[(size_t)q * m + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {
          double vkp = V[(size_t)k * m + p], vkq = V[(size_t)k * m + q];
          V[(size_t)k * m + p] = c * vkp - s * vkq;
          V[(size_t)k * m + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> ord(m);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(),
                   [&](int x, int y) { return A[(size_t)x * m + x] < A[(size_t)y * m + y]; });
  evals.resize(m);
  evecs.assign((size_t)m * m, 0.0);
  for (int c = 0; c < m; ++c) {
    evals[c] = A[(size_t)ord[c] * m + ord[c]];
    for (int i = 0; i < m; ++i) evecs[(size_t)c * m + i] = V[(size_t)i * m + ord[c]];
  }
}

__global__ void k_cmax(const double* __restrict__ ci, size_t ld, int nroots, size_t n, double* __restrict__ out) {
  for (size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < nroots; ++r) {
      double c = fabs(ci[(size_t)r * ld + j]);
      s = __dadd_rn(s, __dmul_rn(c, c));
    }
    out[j] = sqrt(s);
  }
}

__global__ void k_append(const Det2* __restrict__ src, size_t n, Det2* __restrict__ dst) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

struct IterLog {
  int64_t ndets;
  double energy;
  int dav_iters;
  double seconds;
};

// The terms of Hij_1Excite (SHCI/Determinants.cpp:437-469) for every
// spin-orbital pair (a, i) of one spin s and spin orbital j, laid out as
// IntsView::V1 reads them: (ai|jj) - (aj|ji) when j has spin s, (ai|jj)
// otherwise; FP64 (the difference hij_single adds) and FP32 (the FP32 copies'
// difference hij_single_f32 adds), so the table sums are bit-identical.
static void single_terms(const HostInts& h, std::vector<double>& v1, std::vector<float>& v1f) {
  const int n = h.norb, n2 = 2 * n;
  auto pair = [](size_t p, size_t q) { return p > q ? p * (p + 1) / 2 + q : q * (q + 1) / 2 + p; };
  auto i2 = [&](int i, int j, int k, int l) { return h.I2[pair(pair(i, j), pair(k, l))]; };
  v1.assign((size_t)2 * n * n * n2, 0.0);
  v1f.assign(v1.size(), 0.f);
  for (int sp = 0; sp < 2; ++sp)
    for (int a = 0; a < n; ++a)
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n2; ++j) {
          const size_t t = (((size_t)sp * n + a) * n + i) * n2 + j;
          const int jp = j >> 1;
          const double d = i2(a, i, jp, jp);
          if ((j & 1) == sp) {
            const double x = i2(a, jp, jp, i);
            v1[t] = d - x;
            v1f[t] = (float)d - (float)x;
          } else {
            v1[t] = d;
            v1f[t] = (float)d;
          }
        }
}

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;

  HostInts hints;
  HostHeatBath hhb;
  bool have_ints = false;
  DevBuf<double> dI1, dI2, dDirect, dExchange, dSingles;
  DevBuf<float> dI1f, dI2f;  // FP32 copies for the FP32 matrix-free sigma
  DevBuf<double> dV1;        // terms of Hij_1Excite per (a, i, j) (IntsView::V1)
  DevBuf<float> dV1f;
  DevBuf<float> dSameVal, dOppVal;
  DevBuf<int16_t> dSamePairs, dOppPairs;
  DevBuf<int64_t> dSameStart, dOppStart;
  SelectParams sp;

  DevBuf<Det2> dets;
  size_t ndet = 0;
  DetHash hash;
  Helpers helpers;
  bool helpers_ok = false;
  Csr H;
  // device address of the allocation-free sigma's fixed array on this
  // context's device, looked up by every stored build
  void* noalloc_ptr = nullptr;
  int ham_mode = -1;
  bool ham_ok = false;
  DevBuf<double> diag;
  size_t ndiag = 0;
  Prims prims;
  DevBuf<int64_t> counter;
  DevBuf<Det2> cand;
  size_t ncand = 0;  // candidates of the last shci_select_candidates left in cand

  // Davidson workspace
  DevBuf<double> V, W, Vt, Wt, X, Y, R, D, xb64, yb64, gpart, dG, dQ, dlam, dsmall, ftmp;
  DevBuf<float> xb32;

  // alpha <-> beta flip map of the current space (-1 unknown, 0 not closed, 1 closed)
  DevBuf<int32_t> flipidx;
  DevBuf<int8_t> flipsgn;
  int flip_state = -1;
  bool last_stalled = false;  // the last FP32 Davidson stage stopped at its rounding floor
  // time reversal: the flip sector every Davidson vector is kept in (0: none;
  // otherwise +-1, the input's Treversal times (-1)^(beta electrons), in the
  // sign convention of build_flip_map)
  int trev_sector = 0;
  DevBuf<Det2> trev_buf;
  DevBuf<int64_t> trev_flag, trev_pos;

  // preconditioner: 0 the reference's diagonal, 1 diagonal + second-order
  // level shift from the stored H, 2 diagonal + shift predicted by the MLP
  int precond = 0;
  // Davidson subspace: 0 = the reference's (nroots+4 vectors, collapsed to
  // nroots+2 Ritz vectors); otherwise at most basis_max vectors, collapsed to
  // basis_keep (shci_set_davidson_basis)
  int basis_max = 0, basis_keep = 0;
  Mlp mlp;
  DevBuf<double> shift, teacher;
  DevBuf<float> pt2inv;  // 1 / (E - H_jj) for the second-order shift
  bool shift_ready = false;
  DevBuf<int32_t> tr_idx;
  DevBuf<float> tr_tgt;
  int mlp_steps = 60, mlp_batch = 4096;
  // Davidson (residual, correction) pairs for the learned preconditioner: the
  // Ritz vector, residual and Ritz value of root 0 at iterations 2, 4, 8 and
  // 16 of a loose solve, kept until the solve has converged
  static constexpr int kSnaps = 4;
  bool record_pairs = false;
  int n_snap = 0;
  double snap_theta[kSnaps] = {0, 0, 0, 0};
  DevBuf<double> snapX, snapR, pair_tgt, pair_tmp;
  DevBuf<int32_t> pair_idx;
  DevBuf<int64_t> pair_flag, pair_pos;
  int64_t last_pairs = 0;
  // the judge's verdict on the network trained last: its corrections point at
  // the needed one better than the plain preconditioner's on held-out pairs
  bool mlp_ok = false;
  double judge_cos_plain = 0.0, judge_cos_learned = 0.0;
  float mlp_lr = 2e-3f;
  int64_t mlp_sample = 200000;
  double last_loss = 0.0;

  // deterministic perturbation theory
  PtWork ptw;
  PtResult pt_last;
  int64_t pt_max_cand = 0;  // partition capacity override (0: from free memory)
  double t_pt = 0;
  DevBuf<double> ptc;  // coefficients passed from the host

  // reduced density matrices
  DevBuf<unsigned long long> rdm_fix;
  DevBuf<double> rdm_out;
  double t_rdm = 0;

  // run state
  DevBuf<double> ci, cmax;
  int nroots_run = 0;
  std::vector<double> Evar;  // E_var per root of the last run, coreE included
  double run_eps2 = 1e-8;    // the last input's epsilon2
  Schedule run_sched;        // the last input's PT settings
  PtStochResult pts_last;    // last semistochastic PT
  std::vector<IterLog> log;
  double t_select = 0, t_ham = 0, t_dav = 0, t_total = 0, t_sigma = 0, t_mlp = 0;
  int64_t total_dav_iters = 0;
  int64_t n_sigma = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  // captured Davidson iterations: graph per (phase, basis size, active roots)
  bool use_graphs = true;
  bool sigma_deferred = false;  // apply_sigma inside a capture: timing read later
  std::unordered_map<uint64_t, std::pair<cudaGraphExec_t, int64_t>> gcache;
  double* pin = nullptr;  // pinned staging for the small matrices (kPin doubles)
  static constexpr int kPinQ = 0, kPinLam = 256, kPinAct = 272, kPinRR = 288, kPinG = 544, kPinNrm = 800,
                       kPin = 816;
  DevBuf<double> dactlam, drr, dnrm;

  void graphs_clear() {
    for (auto& kv : gcache) cudaGraphExecDestroy(kv.second.first);
    gcache.clear();
  }
  // Run body() on the stream: captured into a graph the first time `key` is
  // seen in this solve, replayed from then on. body() must not synchronise,
  // read device results on the host or allocate.
  template <class F>
  void launch_body(uint64_t key, F&& body) {
    if (!use_graphs) {
      body();
      return;
    }
    auto it = gcache.find(key);
    if (it == gcache.end()) {
      const int64_t l0 = g_launch_count.load();
      SHCI_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      try {
        body();
      } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      cudaGraph_t g = nullptr;
      SHCI_CUDA(cudaStreamEndCapture(stream, &g));
      cudaGraphExec_t ex = nullptr;
      const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
      cudaGraphDestroy(g);
      SHCI_CUDA(e);
      const int64_t nk = g_launch_count.load() - l0;
      g_launch_count.fetch_sub(nk);  // counted once per replay below
      it = gcache.emplace(key, std::make_pair(ex, nk)).first;
    }
    SHCI_CUDA(cudaGraphLaunch(it->second.first, stream));
    g_launch_count.fetch_add(it->second.second);
  }

  ~Context() {
    graphs_clear();
    if (pin) cudaFreeHost(pin);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }

  IntsView ints() const {
    return IntsView{dI1.p, dI2.p, dDirect.p, dExchange.p, hints.norb, dI1f.p, dI2f.p, dV1.p, dV1f.p};
  }
  HeatBathView hb() const {
    return HeatBathView{dSameVal.p, dSamePairs.p, dSameStart.p, dOppVal.p, dOppPairs.p, dOppStart.p, dSingles.p};
  }
  void require_ints() const {
    if (!have_ints) throw Error(kErrState, "no integrals loaded (call shci_read_fcidump first)");
  }
  void require_dets() const {
    if (ndet == 0) throw Error(kErrState, "determinant space is empty");
  }

  template <class T>
  void upload(DevBuf<T>& b, const std::vector<T>& h) {
    b.resize(h.size() ? h.size() : 1);
    if (!h.empty())
      SHCI_CUDA(cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
  }

  void load_fcidump(const std::string& path) {
    HostInts hi;
    read_fcidump(path, hi);
    HostHeatBath hb;
    build_heatbath(hi, hb);
    hints = std::move(hi);
    hhb = std::move(hb);
    upload(dI1, hints.I1);
    upload(dI2, hints.I2);
    {
      const std::vector<float> f1(hints.I1.begin(), hints.I1.end()), f2(hints.I2.begin(), hints.I2.end());
      upload(dI1f, f1);
      upload(dI2f, f2);
      std::vector<double> v1;
      std::vector<float> v1f;
      single_terms(hints, v1, v1f);
      upload(dV1, v1);
      upload(dV1f, v1f);
      SHCI_CUDA(cudaStreamSynchronize(stream));  // the host copies go out of scope
    }
    upload(dDirect, hints.Direct);
    upload(dExchange, hints.Exchange);
    upload(dSingles, hhb.singles);
    upload(dSameVal, hhb.sameVal);
    upload(dOppVal, hhb.oppVal);
    upload(dSamePairs, hhb.samePairs);
    upload(dOppPairs, hhb.oppPairs);
    upload(dSameStart, hhb.sameStart);
    upload(dOppStart, hhb.oppStart);
    SHCI_CUDA(cudaStreamSynchronize(stream));
    have_ints = true;
    ndet = 0;
    helpers_ok = ham_ok = false;
    ndiag = 0;
  }

  void invalidate_space() {
    helpers_ok = false;
    ham_ok = false;
    flip_state = -1;
    Evar.clear();  // the run's coefficients no longer match the space
  }

  // True when the space is closed under the alpha <-> beta flip (equal alpha
  // and beta electron counts and every flipped determinant present).
  bool ensure_flip() {
    if (flip_state >= 0) return flip_state == 1;
    flip_state = 0;
    if (ndet == 0) return false;
    Det2 d0;
    SHCI_CUDA(cudaMemcpyAsync(&d0, dets.p, sizeof(Det2), cudaMemcpyDeviceToHost, stream));
    SHCI_CUDA(cudaStreamSynchronize(stream));
    if (__builtin_popcountll(det_alpha(d0)) != __builtin_popcountll(det_beta(d0))) return false;
    hash.build(dets.p, ndet, stream);
    flipidx.resize(ndet);
    flipsgn.resize(ndet);
    counter.resize(1);
    if (build_flip_map(dets.p, ndet, hash, flipidx.p, flipsgn.p, counter.p, stream)) flip_state = 1;
    return flip_state == 1;
  }
  // Project column c (length ndet) onto the flip sector of sign p.
  void project_parity(double* c, double p) {
    ftmp.reserve(ndet);
    flip_project(c, ndet, flipidx.p, flipsgn.p, p, ftmp.p, stream);
  }

  void set_dets(const uint64_t* h, int64_t n) {
    require_ints();
    H.N = 0;  // the stored Hamiltonian no longer describes a prefix of the space
    H.nnz = 0;
    if (n < 0) throw Error(kErrInvalid, "negative determinant count");
    const int n2 = 2 * hints.norb;
    for (int64_t i = 0; i < n; ++i) {
      uint64_t w0 = h[2 * i], w1 = h[2 * i + 1];
      int ne = __builtin_popcountll(w0) + __builtin_popcountll(w1);
      if (ne != hints.nelec) throw Error(kErrInvalid, "determinant " + std::to_string(i) + " has wrong electron count");
      if (n2 < 128) {
        uint64_t lim0 = n2 >= 64 ? ~0ull : ((1ull << n2) - 1ull);
        uint64_t lim1 = n2 > 64 ? ((1ull << (n2 - 64)) - 1ull) : 0ull;
        if ((w0 & ~lim0) || (w1 & ~lim1))
          throw Error(kErrInvalid, "determinant " + std::to_string(i) + " occupies orbitals beyond NORB");
      }
    }
    dets.resize(n > 0 ? (size_t)n : 1);
    if (n) SHCI_CUDA(cudaMemcpyAsync(dets.p, h, (size_t)n * sizeof(Det2), cudaMemcpyHostToDevice, stream));
    ndet = (size_t)n;
    ndiag = 0;
    invalidate_space();
    SHCI_CUDA(cudaStreamSynchronize(stream));
  }

  // Heat-bath selection from every current determinant; appends new ones.
  int64_t select(const double* cmax_dev, double eps1) {
    const size_t nnew = candidates(cmax_dev, eps1);
    append_candidates(nnew);
    return (int64_t)nnew;
  }

  // Selection with time reversal: candidates from the standard member of each
  // pair (the others have cMax 0), made standard, sorted, unique and absent
  // from the space, then appended followed by their flipped partners, so the
  // space stays closed under the flip (SHCI/SHCIbasics.cpp:969-997).
  int64_t select_trev(const double* cmax_dev, double eps1) {
    const size_t n = candidates(cmax_dev, eps1);
    size_t nnew = 0;
    if (n) {
      trev_buf.reserve(2 * n);
      nnew = trev_new_dets(cand.p, n, hash, dets.p, trev_buf.p, trev_flag, trev_pos, prims, stream);
    }
    ncand = 0;
    if (nnew) {
      if (ndet + nnew >= (size_t)0x7fffffff) throw Error(kErrInvalid, "determinant space exceeds 2^31 entries");
      dets.grow_keep(ndet + nnew, stream);
      k_append<<<grid_for(nnew, 256), 256, 0, stream>>>(trev_buf.p, nnew, dets.p + ndet);
      SHCI_LAUNCH_CHECK();
      ndet += nnew;
      invalidate_space();
    }
    SHCI_CUDA(cudaStreamSynchronize(stream));
    return (int64_t)nnew;
  }

  // The new determinants of a selection (parents with cMax 0 contribute
  // none), sorted in the reference's order and unique, left in cand[0, n).
  size_t candidates(const double* cmax_dev, double eps1) {
    require_ints();
    require_dets();
    hash.build(dets.p, ndet, stream);
    counter.resize(1);
    int64_t cap = (int64_t)std::max<size_t>(cand.cap, std::max<size_t>((size_t)1 << 20, 4 * ndet));
    cand.reserve((size_t)cap);
    cap = (int64_t)cand.cap;
    int64_t total = select_candidates(dets.p, cmax_dev, ndet, eps1, ints(), hb(), hints.maxEntry, sp, hash, cand.p,
                                      cap, counter.p, stream);
    if (total > cap) {
      cand.release();
      cand.reserve((size_t)total + total / 8);
      cap = (int64_t)cand.cap;
      total = select_candidates(dets.p, cmax_dev, ndet, eps1, ints(), hb(), hints.maxEntry, sp, hash, cand.p, cap,
                                counter.p, stream);
      if (total > cap) throw Error(kErrState, "candidate count changed between passes");
    }
    size_t nnew = 0;
    if (total > 0) {
      sort_dets(cand.p, nullptr, (size_t)total, prims, stream);
      nnew = unique_dets(cand.p, (size_t)total, prims, stream);
    }
    SHCI_CUDA(cudaStreamSynchronize(stream));
    ncand = nnew;
    return nnew;
  }

  // Appends cand[0, nnew) to the space (new determinants in sorted order, as
  // the reference appends them, SHCI/SHCIbasics.cpp:1059-1077).
  void append_candidates(size_t nnew) {
    if (nnew) {
      if (ndet + nnew >= (size_t)0x7fffffff) throw Error(kErrInvalid, "determinant space exceeds 2^31 entries");
      dets.grow_keep(ndet + nnew, stream);
      k_append<<<grid_for(nnew, 256), 256, 0, stream>>>(cand.p, nnew, dets.p + ndet);
      SHCI_LAUNCH_CHECK();
      ndet += nnew;
      invalidate_space();
    }
    ncand = 0;
    SHCI_CUDA(cudaStreamSynchronize(stream));
  }

  // Appends host determinants (the merged new determinants of a sharded
  // selection): they must follow the reference's order strictly, carry the
  // right electron count and be absent from the space.
  void append_dets(const uint64_t* h, int64_t n) {
    require_ints();
    require_dets();
    if (n < 0) throw Error(kErrInvalid, "negative determinant count");
    if (n == 0) return;
    for (int64_t i = 0; i < n; ++i) {
      const uint64_t w0 = h[2 * i], w1 = h[2 * i + 1];
      if (__builtin_popcountll(w0) + __builtin_popcountll(w1) != hints.nelec)
        throw Error(kErrInvalid, "appended determinant " + std::to_string(i) + " has the wrong electron count");
      if (i > 0) {  // Determinant::operator<: signed words from the top (SHCI/Determinants.h:490-498)
        const int64_t a1 = (int64_t)h[2 * i - 1], b1 = (int64_t)w1;
        const int64_t a0 = (int64_t)h[2 * i - 2], b0 = (int64_t)w0;
        if (!(a1 < b1 || (a1 == b1 && a0 < b0)))
          throw Error(kErrInvalid, "appended determinants must be sorted and unique");
      }
    }
    hash.build(dets.p, ndet, stream);
    cand.reserve((size_t)n);
    SHCI_CUDA(cudaMemcpyAsync(cand.p, h, (size_t)n * sizeof(Det2), cudaMemcpyHostToDevice, stream));
    counter.resize(1);
    if (count_present(cand.p, (size_t)n, hash, dets.p, counter.p, stream) != 0)
      throw Error(kErrInvalid, "appended determinants must be absent from the space");
    append_candidates((size_t)n);
  }

  void ensure_diag() {
    require_dets();
    if (ndiag >= ndet) return;
    diag.grow_keep(ndet, stream);
    compute_diag(dets.p + ndiag, ndet - ndiag, ints(), diag.p + ndiag, stream);
    ndiag = ndet;
  }

  static bool is_direct(int m) { return m == SHCI_MODE_DIRECT || m == SHCI_MODE_DIRECT_MIXED; }
  // a stored Hamiltonian of the whole space (not matrix-free, not a row block)
  bool whole_ham() const { return ham_ok && !is_direct(ham_mode) && !H.block; }

  // Spatial 2-RDM (n^4) and 1-RDM (n^2) of the wavefunction c (device, ndet
  // entries) to the host (either may be null), over the connection lists of
  // the stored Hamiltonian (built in the mixed form when the current one is
  // matrix-free or stale, as the reference rebuilds helpers for its RDM after
  // a matrix-free Davidson, SHCI/SHCIbasics.cpp:1274-1283).
  void rdm(const double* c, double* s2, double* s1) {
    require_ints();
    require_dets();
    const double t0 = now_s();
    if (!whole_ham()) build_ham(SHCI_MODE_MIXED);
    const size_t n = (size_t)hints.norb, n2 = n * n, n4 = n2 * n2;
    rdm_evaluate(dets.p, c, ndet, H, hints.norb, rdm_fix, rdm_out, stream);
    if (s2) SHCI_CUDA(cudaMemcpyAsync(s2, rdm_out.p, n4 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (s1) SHCI_CUDA(cudaMemcpyAsync(s1, rdm_out.p + n4, n2 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    SHCI_CUDA(cudaStreamSynchronize(stream));
    t_rdm = now_s() - t0;
  }

  // Deterministic PT2 of the current space with coefficients c (device, ndet
  // entries); E0 includes coreE, as in SHCIbasics::DoPerturbativeDeterministic
  // (SHCI/SHCIbasics.cpp:453-728). The selection restrictions apply (the
  // reference's `restrict` fills both lists, SHCI/input.cpp:267-277); ncore and
  // nact do not.
  double perturb(const double* c, double E0, double eps2) {
    require_ints();
    require_dets();
    const double t0 = now_s();
    hash.build(dets.p, ndet, stream);
    SelectParams psp = sp;
    psp.ncore = 0;
    psp.nact = 1 << 30;
    pt_last = pt_deterministic(dets.p, ndet, c, E0 - hints.coreE, eps2, ints(), hb(), hints.maxEntry, psp, hash,
                               pt_max_cand, ptw, prims, stream);
    t_pt = now_s() - t0;
    pts_last = PtStochResult();
    return pt_last.e2;
  }

  // getParityForDiceToAlphaBeta (SHCI/Determinants.cpp:691-706): the sign
  // between Dice's interleaved spin-orbital order and all-alpha-then-beta:
  // (-1)^(alpha electrons in higher orbitals) for every occupied beta orbital.
  static double alpha_beta_parity(const uint64_t* w, int norb) {
    auto occ = [&](int p) { return (w[p >> 6] >> (p & 63)) & 1ull; };
    int nalpha = 0;
    for (int k = 0; k < norb; ++k) nalpha += (int)occ(2 * k);
    double parity = 1.0;
    int before = 0;  // alpha electrons in orbitals below k
    for (int k = 0; k < norb; ++k) {
      if (occ(2 * k + 1)) {
        const int after = nalpha - before - (int)occ(2 * k);
        if (after % 2 == 1) parity = -parity;
      }
      before += (int)occ(2 * k);
    }
    return parity;
  }

  // writeBestDeterminants (SHCI/SHCI.cpp:465-506): the num largest |c| of a
  // root as {int num, int norb, then per determinant the coefficient times
  // the alpha-beta parity (double) and one character per spatial orbital,
  // '0', 'a', 'b' or '2'}. Ties in |c| keep index order (the reference's
  // std::sort leaves their order unspecified).
  void write_best_dets(const double* c, int num, const std::string& path) {
    require_dets();
    std::vector<double> ch(ndet);
    std::vector<uint64_t> dh(2 * ndet);
    SHCI_CUDA(cudaMemcpyAsync(ch.data(), c, ndet * sizeof(double), cudaMemcpyDeviceToHost, stream));
    SHCI_CUDA(cudaMemcpyAsync(dh.data(), dets.p, ndet * sizeof(Det2), cudaMemcpyDeviceToHost, stream));
    SHCI_CUDA(cudaStreamSynchronize(stream));
    num = (int)std::min<size_t>((size_t)std::max(num, 0), ndet);
    std::vector<size_t> idx(ndet);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return std::fabs(ch[a]) > std::fabs(ch[b]); });
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error(kErrIO, "cannot write " + path);
    const int n = hints.norb;
    bool ok = std::fwrite(&num, sizeof(int), 1, f) == 1 && std::fwrite(&n, sizeof(int), 1, f) == 1;
    std::vector<char> occ(n);
    for (int i = 0; ok && i < num; ++i) {
      const size_t m = idx[i];
      const uint64_t* w = &dh[2 * m];
      const double coeff = alpha_beta_parity(w, n) * ch[m];
      for (int k = 0; k < n; ++k) {
        const bool a = (w[(2 * k) >> 6] >> ((2 * k) & 63)) & 1ull, b = (w[(2 * k + 1) >> 6] >> ((2 * k + 1) & 63)) & 1ull;
        occ[k] = a ? (b ? '2' : 'a') : (b ? 'b' : '0');
      }
      ok = std::fwrite(&coeff, sizeof(double), 1, f) == 1 && std::fwrite(occ.data(), 1, n, f) == (size_t)n;
    }
    if (std::fclose(f) != 0 || !ok) throw Error(kErrIO, "error writing " + path);
  }

  // Semistochastic PT2 (E0 with coreE) of the current space with
  // coefficients c (device, ndet entries); restrictions as in perturb().
  double perturb_stoch(const double* c, double E0, double eps2, double eps2L, int nsample, int max_iter,
                       double target, uint64_t seed) {
    require_ints();
    require_dets();
    const double t0 = now_s();
    std::vector<double> ch(ndet);
    SHCI_CUDA(cudaMemcpyAsync(ch.data(), c, ndet * sizeof(double), cudaMemcpyDeviceToHost, stream));
    SHCI_CUDA(cudaStreamSynchronize(stream));
    hash.build(dets.p, ndet, stream);
    SelectParams psp = sp;
    psp.ncore = 0;
    psp.nact = 1 << 30;
    pts_last = pt_semistochastic(dets.p, ndet, c, ch, E0 - hints.coreE, eps2, eps2L, nsample, max_iter, target, seed,
                                 ints(), hb(), hints.maxEntry, psp, hash, ptw, prims, stream);
    pt_last = PtResult();
    pt_last.candidates = pts_last.candidates;
    t_pt = now_s() - t0;
    return pts_last.e2;
  }

  void build_ham(int mode) {
    require_ints();
    require_dets();
    if (mode < 0 || mode > 3) throw Error(kErrInvalid, "unknown Hamiltonian mode");
    PhaseTimer pt(stream);
    if (!helpers_ok) {
      helpers.build(dets.p, ndet, hints.norb, prims, stream);
      helpers_ok = true;
    }
    pt.mark("string tables");
    ensure_diag();
    if (is_direct(mode)) {
      H.drop_compressed();
      H.perm.release();
      H.spos.release();
      H.col.release();
      H.v64.release();
      H.vhi.release();
      H.vlo.release();
      H.rowptr.release();
      H.N = 0;
      H.nnz = 0;
    } else {
      // the stored rows stay valid for the unchanged prefix of the space
      // (selection only appends), so only new rows and columns are built
      const size_t n_old = (ham_mode == mode && !H.block) ? H.N : 0;
      H.drop_compressed();  // stale; rebuilt below (frees its memory before the build)
      build_ham_csr(helpers, dets.p, ints(), H, mode == SHCI_MODE_FP64, mode == SHCI_MODE_MIXED,
                    mode == SHCI_MODE_MIXED, n_old, prims, stream);
      if (mode == SHCI_MODE_MIXED) compress_csr(H, prims, stream);
      pt.mark("ham compress");
      noalloc_ptr = noalloc_scratch_address();
    }
    ham_mode = mode;
    ham_ok = true;
    SHCI_CUDA(cudaStreamSynchronize(stream));
  }

  // One rank's share of the stored Hamiltonian in the sharded path: the full
  // rows of the determinants [r0, r1) (shci_ham_build_rows).
  void build_ham_rows(int mode, size_t r0, size_t r1) {
    require_ints();
    require_dets();
    if (mode != SHCI_MODE_FP64 && mode != SHCI_MODE_MIXED)
      throw Error(kErrInvalid, "a row block is stored: mode must be SHCI_MODE_FP64 or SHCI_MODE_MIXED");
    if (!(r0 < r1 && r1 <= ndet)) throw Error(kErrInvalid, "row block [r0, r1) must be a non-empty range of the space");
    if (!helpers_ok) {
      helpers.build(dets.p, ndet, hints.norb, prims, stream);
      helpers_ok = true;
    }
    ensure_diag();
    ham_ok = false;
    build_ham_block(helpers, dets.p, ints(), H, mode == SHCI_MODE_FP64, mode == SHCI_MODE_MIXED,
                    mode == SHCI_MODE_MIXED, r0, r1, prims, stream);
    if (mode == SHCI_MODE_MIXED) compress_csr(H, prims, stream);
    noalloc_ptr = noalloc_scratch_address();
    ham_mode = mode;
    ham_ok = true;
    SHCI_CUDA(cudaStreamSynchronize(stream));
  }

  // Y[:, yc0 + c] = H A[:, c0 + c], c < k, in the given sigma mode.
  void apply_sigma(int mode, const double* A, size_t lda, int c0, int k, double* Yp, size_t ldy, int yc0) {
    if (!ham_ok) throw Error(kErrState, "Hamiltonian not built for the current space (call shci_ham_build)");
    if (is_direct(mode) && !helpers_ok) throw Error(kErrState, "string tables missing");
    if (!is_direct(mode) && is_direct(ham_mode))
      throw Error(kErrState, "Hamiltonian was built matrix-free; stored sigma unavailable");
    if (mode == SHCI_MODE_MIXED && ham_mode != SHCI_MODE_MIXED)
      throw Error(kErrState, "mixed sigma needs a Hamiltonian built in mixed mode");
    const size_t N = ndet;
    // inside a capture the records must be external to become graph nodes
    const unsigned evflag = sigma_deferred ? cudaEventRecordExternal : 0u;
    SHCI_CUDA(cudaEventRecordWithFlags(ev0, stream, evflag));
    for (int done = 0; done < k;) {
      const int kk = std::min(4, k - done);
      const int kp = kk == 3 ? 4 : kk;
      if (mode == SHCI_MODE_MIXED) {
        xb32.reserve(N * kp);
        pack_f32(A, lda, c0 + done, kk, kp, N, xb32.p, stream, H.pack_perm());
        sigma_csr_mixed(H, diag.p, xb32.p, kp, kk, Yp + (size_t)(yc0 + done) * ldy, ldy, stream);
      } else if (mode == SHCI_MODE_FP64) {
        xb64.reserve(N * kp);
        if (H.v64.p) {
          pack_f64(A, lda, c0 + done, kk, kp, N, xb64.p, stream, H.pack_perm());
          sigma_csr_f64(H, diag.p, xb64.p, kp, kk, Yp + (size_t)(yc0 + done) * ldy, ldy, stream);
        } else {  // mixed-path matrix: float-float refinement sigma on head + tail
          float* xff = reinterpret_cast<float*>(xb64.p);
          pack_ff(A, lda, c0 + done, kk, kp, N, xff, stream, H.pack_perm());
          sigma_csr_ff(H, diag.p, xff, kp, A, lda, c0 + done, kk, Yp + (size_t)(yc0 + done) * ldy, ldy, stream);
        }
      } else if (mode == SHCI_MODE_DIRECT_MIXED) {  // FP32 matrix-free
        xb32.reserve(N * kp);
        yb64.reserve(N * kp);
        pack_f32(A, lda, c0 + done, kk, kp, N, xb32.p, stream);
        sigma_direct32(helpers, dets.p, ints(), diag.p, xb32.p, yb64.p, kp, stream);
        unpack_f64(yb64.p, kp, kk, N, Yp, ldy, yc0 + done, stream);
      } else {
        xb64.reserve(N * kp);
        yb64.reserve(N * kp);
        pack_f64(A, lda, c0 + done, kk, kp, N, xb64.p, stream);
        sigma_direct(helpers, dets.p, ints(), diag.p, xb64.p, yb64.p, kp, stream);
        unpack_f64(yb64.p, kp, kk, N, Yp, ldy, yc0 + done, stream);
      }
      done += kk;
    }
    SHCI_CUDA(cudaEventRecordWithFlags(ev1, stream, evflag));
    if (sigma_deferred) return;  // captured: the caller reads the events after the replay
    SHCI_CUDA(cudaEventSynchronize(ev1));
    float ms = 0.f;
    SHCI_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    t_sigma += ms * 1e-3;
    n_sigma += 1;
  }

  // ---- Davidson -----------------------------------------------------------
  std::vector<double> gram_host(const double* A, size_t lda, int ma, const double* B, size_t ldb, int mb) {
    dG.reserve((size_t)ma * mb);
    ts_gram(A, lda, ma, B, ldb, mb, ndet, dG.p, gpart, stream);
    std::vector<double> g((size_t)ma * mb);
    SHCI_CUDA(cudaMemcpyAsync(g.data(), dG.p, g.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    SHCI_CUDA(cudaStreamSynchronize(stream));
    return g;
  }
  void to_dev(DevBuf<double>& b, const std::vector<double>& h) {
    b.reserve(h.size());
    SHCI_CUDA(cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
  }
  void fill_random(double* col, uint64_t seed) {
    std::vector<double> h(ndet);
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 1;
    for (auto& v : h) {
      s ^= s << 13;
      s ^= s >> 7;
      s ^= s << 17;
      v = ((s >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
    }
    SHCI_CUDA(cudaMemcpyAsync(col, h.data(), ndet * sizeof(double), cudaMemcpyHostToDevice, stream));
    SHCI_CUDA(cudaStreamSynchronize(stream));
  }
  // col_j -= (col_i . col_j) col_i  (device-only)
  void project_out(const double* ci_, double* cj) {
    dsmall.reserve(4);
    ts_gram(ci_, ndet, 1, cj, ndet, 1, ndet, dsmall.p, gpart, stream);
    ts_gemm(ci_, ndet, 1, dsmall.p, 1, ndet, -1.0, 1.0, cj, ndet, stream);
  }
  double norm_host(const double* c) {
    auto g = gram_host(c, ndet, 1, c, ndet, 1);
    return std::sqrt(g[0]);
  }
  void scale_col(double* c, double s) {
    to_dev(dsmall, std::vector<double>{s});
    scale_cols(c, ndet, dsmall.p, 1, ndet, stream);
  }

  // One Davidson solve in a fixed sigma mode. x: device N x nroots (ld N).
  // stall_exit: stop early (returning the current Ritz vectors) once the
  // residual stops decreasing -- the FP32 stage of the mixed path, whose
  // residual floor is set by FP32 rounding in sigma, hands over to the FP64
  // stage there.
  //
  // resume_m > 0: continue on the basis V[:, :resume_m] left by a previous
  // stage (W is recomputed in this stage's sigma mode); x is then ignored on
  // entry. On return basis_m holds the size of the basis left in V.
  void davidson_core(int mode, bool block, int nroots, double* x, int maxCopies, double tol, bool direct_rules,
                     std::vector<double>& E, int& numIter, bool stall_exit = false, int resume_m = 0,
                     int* basis_m = nullptr) {
    const size_t N = ndet;
    const double t_enter = now_s();
    double t_g1 = 0.0, t_g2 = 0.0, t_loop0 = 0.0, sig0 = t_sigma;
    // FP32 stage: when every start vector lies in one alpha <-> beta flip
    // sector, exact arithmetic keeps the iterates there, and so does FP64
    // sigma to rounding; FP32 sigma does not (see the note on compensated
    // accumulation in kernels_sigma.cu), so its corrections are projected
    // back into that sector. Start vectors spanning both sectors (e.g. the
    // random guesses of extra roots) already reach every state: no projection.
    const bool sym = (stall_exit || trev_sector != 0) && ensure_flip();
    if (trev_sector != 0 && !sym)
      throw Error(kErrState, "time reversal needs the flipped partner of every determinant in the space");
    int sector = trev_sector;
    last_stalled = false;
    if (nroots < 1) throw Error(kErrInvalid, "nroots must be >= 1");
    if ((size_t)nroots > N) throw Error(kErrInvalid, "more roots than determinants");
    int mmax = std::max(maxCopies, nroots + 1);
    if (mmax > 16) mmax = 16;
    if ((size_t)mmax > N) mmax = (int)N;
    if (nroots > 16) throw Error(kErrInvalid, "at most 16 roots");
    V.reserve(N * mmax);
    W.reserve(N * mmax);
    Vt.reserve(N * mmax);
    Wt.reserve(N * mmax);
    X.reserve(N * nroots);
    Y.reserve(N * nroots);
    R.reserve(N * nroots);
    D.reserve(N * nroots);
    int m = nroots;
    if (resume_m > 0) {
      m = std::min(resume_m, mmax);
      apply_sigma(mode, V.p, N, 0, m, W.p, N, 0);
    } else {
      // initial block (SHCI/Davidson.cpp:156-180)
      SHCI_CUDA(cudaMemcpyAsync(V.p, x, N * nroots * sizeof(double), cudaMemcpyDeviceToDevice, stream));
      for (int i = 0; i < nroots; ++i) {
        double* bi = V.p + (size_t)i * N;
        if (norm_host(bi) < 1.e-10) {
          fill_random(bi, 1000 + i);
          scale_col(bi, 1.0 / norm_host(bi));
        }
      }
      for (int i = 0; i < nroots; ++i) {
        double* bi = V.p + (size_t)i * N;
        for (int j = 0; j < i; ++j) project_out(V.p + (size_t)j * N, bi);
        if (norm_host(bi) < 1e-8) fill_random(bi, 2000 + i);
        for (int j = 0; j < i; ++j) project_out(V.p + (size_t)j * N, bi);
        scale_col(bi, 1.0 / norm_host(bi));
      }
      if (sym) {
        if (trev_sector == 0) {
          std::vector<double> par(nroots);
          for (int i = 0; i < nroots; ++i)
            par[i] = flip_parity(V.p + (size_t)i * N, N, flipidx.p, flipsgn.p, gpart, stream);
          sector = par[0] > kParityDefinite ? 1 : (par[0] < -kParityDefinite ? -1 : 0);
          for (int i = 1; i < nroots; ++i)
            if (!(par[i] * sector > kParityDefinite)) sector = 0;
        }
        if (sector != 0)
          for (int i = 0; i < nroots; ++i) {
            double* bi = V.p + (size_t)i * N;
            for (int j = 0; j < i; ++j) project_out(V.p + (size_t)j * N, bi);
            project_parity(bi, (double)sector);
            double nb = norm_host(bi);
            if (nb < 1e-8) {  // no component in the sector: a random start there
              fill_random(bi, 3000 + i);
              for (int j = 0; j < i; ++j) project_out(V.p + (size_t)j * N, bi);
              project_parity(bi, (double)sector);
              nb = norm_host(bi);
            }
            if (nb < 1e-8)
              throw Error(kErrInvalid, "the determinant space has no room for root " + std::to_string(i + 1) +
                                           " in the time-reversal (alpha <-> beta flip) sector");
            scale_col(bi, 1.0 / nb);
          }
      }
      apply_sigma(mode, V.p, N, 0, nroots, W.p, N, 0);
    }
    numIter = 0;
    int cR = 0;
    const int soft_cap = (direct_rules ? 400 : 800) * nroots;
    const int hard_cap = (direct_rules ? 400 : 2000) * nroots;
    std::vector<double> lam, Q;
    double best_resid = 1e300;
    int stall = 0, stall_root = 0;
    // everything the captured bodies touch is allocated before the first capture
    graphs_clear();
    dG.reserve(256);
    dQ.reserve(256);
    dlam.reserve(16);
    dactlam.reserve(16);
    drr.reserve(256);
    dnrm.reserve(16);
    dsmall.reserve(16);
    gpart.reserve(256 * 304 + 2 * 304);
    if (mode == SHCI_MODE_MIXED) xb32.reserve(N * 4);
    if (mode == SHCI_MODE_FP64) xb64.reserve(N * 4);
    if (mode == SHCI_MODE_DIRECT) {
      xb64.reserve(N * 4);
      yb64.reserve(N * 4);
    }
    if (mode == SHCI_MODE_DIRECT_MIXED) {
      xb32.reserve(N * 4);
      yb64.reserve(N * 4);
    }
    if (sym) ftmp.reserve(N);
    const double* shiftp = (shift_ready && shift.n >= N) ? shift.p : nullptr;
    std::vector<double> G = gram_host(V.p, N, m, W.p, N, m);
    t_loop0 = now_s();
    while (true) {
      // Rayleigh-Ritz (SHCI/Davidson.cpp:250-269): small eigenproblem on the host
      std::vector<double> hs((size_t)m * m);
      for (int i = 0; i < m; ++i)
        for (int j = i; j < m; ++j) hs[(size_t)i * m + j] = hs[(size_t)j * m + i] = G[(size_t)i + (size_t)j * m];
      sym_eig(m, hs, lam, Q);
      std::memcpy(pin + kPinQ, Q.data(), (size_t)m * m * sizeof(double));
      std::memcpy(pin + kPinLam, lam.data(), (size_t)nroots * sizeof(double));
      // graph 1: Ritz vectors, residuals and the residual Gram matrix
      launch_body(((uint64_t)1 << 60) | (uint64_t)m, [&]() {
        SHCI_CUDA(cudaMemcpyAsync(dQ.p, pin + kPinQ, (size_t)m * m * sizeof(double), cudaMemcpyHostToDevice, stream));
        SHCI_CUDA(cudaMemcpyAsync(dlam.p, pin + kPinLam, (size_t)nroots * sizeof(double), cudaMemcpyHostToDevice,
                                  stream));
        ts_gemm(V.p, N, m, dQ.p, nroots, N, 1.0, 0.0, X.p, N, stream);
        ts_gemm(W.p, N, m, dQ.p, nroots, N, 1.0, 0.0, Y.p, N, stream);
        residual(X.p, Y.p, dlam.p, nroots, N, N, R.p, stream);
        ts_gram(R.p, N, nroots, R.p, N, nroots, N, drr.p, gpart, stream);
        SHCI_CUDA(cudaMemcpyAsync(pin + kPinRR, drr.p, (size_t)nroots * nroots * sizeof(double),
                                  cudaMemcpyDeviceToHost, stream));
      });
      SHCI_CUDA(cudaStreamSynchronize(stream));
      if (trace_level() > 0) t_g1 += now_s() - t_loop0, t_loop0 = now_s();
      std::vector<double> rn(nroots);
      for (int c = 0; c < nroots; ++c) rn[c] = std::sqrt(std::max(0.0, pin[kPinRR + (size_t)c * nroots + c]));
      numIter++;
      if (trace_level() > 0)
        std::fprintf(stderr, "[davidson mode=%d it=%d m=%d] lam0=%.12f res0=%.3e G00=%.12f t=%.3f\n", mode, numIter,
                     m, lam[0], rn[0], G[0], now_s() - t_enter);
      if (record_pairs && n_snap < kSnaps && (numIter == 2 || numIter == 4 || numIter == 8 || numIter == 16)) {
        if (n_snap == 0) {
          snapX.reserve(N * kSnaps);
          snapR.reserve(N * kSnaps);
        }
        SHCI_CUDA(cudaMemcpyAsync(snapX.p + (size_t)n_snap * N, X.p, N * sizeof(double), cudaMemcpyDeviceToDevice,
                                  stream));
        SHCI_CUDA(cudaMemcpyAsync(snapR.p + (size_t)n_snap * N, R.p, N * sizeof(double), cudaMemcpyDeviceToDevice,
                                  stream));
        snap_theta[n_snap++] = lam[0];
      }
      auto finish = [&]() {
        if (basis_m) *basis_m = m;
        E.assign(lam.begin(), lam.begin() + nroots);
        SHCI_CUDA(cudaMemcpyAsync(x, X.p, N * nroots * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        SHCI_CUDA(cudaStreamSynchronize(stream));
        graphs_clear();
        if (trace_level() > 0)
          std::fprintf(stderr,
                       "[davidson-time mode=%d N=%zu iters=%d mmax=%d] total %.2f ms: setup %.2f, ritz %.2f, "
                       "correction+sigma %.2f (sigma %.2f)\n",
                       mode, N, numIter, mmax, 1e3 * (now_s() - t_enter), 1e3 * (t_loop0 - t_enter - t_g1 - t_g2),
                       1e3 * t_g1, 1e3 * t_g2, 1e3 * (t_sigma - sig0));
      };
      if ((size_t)m == N) {
        finish();
        return;
      }
      if (stall_exit) {
        // progress measure: the worked-on root (root-by-root) or the worst root (block)
        double worst = 0.0;
        if (block) {
          for (int c = 0; c < nroots; ++c) worst = std::max(worst, rn[c]);
        } else {
          worst = rn[cR];
          if (cR != stall_root) {
            stall_root = cR;
            best_resid = 1e300;
            stall = 0;
          }
        }
        // One root: only near the FP32 rounding floor (~1e-6); a plateau
        // higher up is ordinary Davidson behaviour and the FP32 stage keeps
        // going. Several roots (block): any plateau of the worst root hands
        // over, with the whole basis, to the refinement stage, which finishes
        // the roots whose FP32 residuals stall above the floor.
        if (worst < 0.8 * best_resid) {
          best_resid = worst;
          stall = 0;
        } else if ((block || worst < kStallWindow) && ++stall >= 8) {
          last_stalled = true;
          finish();
          return;
        }
      }
      std::vector<int> act;
      std::vector<double> act_lam;
      if (!block) {
        // root-by-root scheme of the reference (SHCI/Davidson.cpp:271-323)
        const double ei = lam[cR];
        bool back = false;
        for (int i = 0; i < cR; ++i)
          if (rn[i] > tol) {
            cR = i;
            back = true;
            break;
          }
        double error = rn[cR];
        if (back) {
          // the reference keeps the old eigenvalue for the residual here
          to_dev(dsmall, std::vector<double>{ei});
          residual(X.p + (size_t)cR * N, Y.p + (size_t)cR * N, dsmall.p, 1, N, N, R.p + (size_t)cR * N, stream);
          error = norm_host(R.p + (size_t)cR * N);
        }
        const int rootForR = cR;
        if (error < tol || numIter > soft_cap) {
          if (numIter > hard_cap)
            throw Error(kErrNoConv, "Davidson calculation did not converge for root " + std::to_string(cR + 1));
          cR++;
          if (cR == nroots) {
            finish();
            return;
          }
        }
        act.push_back(rootForR);
        act_lam.push_back(ei);
      } else {
        for (int c = 0; c < nroots; ++c)
          if (!(rn[c] < tol)) {
            act.push_back(c);
            act_lam.push_back(lam[c]);
          }
        if (act.empty() || numIter > soft_cap) {
          if (!act.empty() && numIter > hard_cap) throw Error(kErrNoConv, "block Davidson did not converge");
          finish();
          return;
        }
      }
      const int nact = (int)act.size();
      std::memcpy(pin + kPinAct, act_lam.data(), (size_t)nact * sizeof(double));
      uint64_t amask = 0;
      for (int a : act) amask |= 1ull << a;
      const bool collapse = m + nact > mmax;
      int keep = m;
      if (collapse) {
        keep = basis_keep > 0 ? std::min(basis_keep, mmax - nact)
                              : (block ? mmax - nact : std::min(nroots + 2, mmax - nact));
        if (keep < nroots) keep = nroots;
      }
      const int m1 = collapse ? keep : m;
      // graph 2: corrections, orthonormalisation, collapse, append, sigma, Gram
      sigma_deferred = use_graphs;
      launch_body(((uint64_t)2 << 60) | ((uint64_t)m << 40) | ((uint64_t)keep << 20) | amask, [&]() {
        SHCI_CUDA(cudaMemcpyAsync(dactlam.p, pin + kPinAct, (size_t)nact * sizeof(double), cudaMemcpyHostToDevice,
                                  stream));
        for (int a = 0; a < nact; ++a) {
          // residual with the eigenvalue the reference uses for this root, preconditioned
          double* da = D.p + (size_t)a * N;
          residual(X.p + (size_t)act[a] * N, Y.p + (size_t)act[a] * N, dactlam.p + a, 1, N, N, da, stream);
          if (shiftp)
            precondition_shift(diag.p, shiftp, dactlam.p + a, 1, N, da, N, stream);
          else
            precondition(diag.p, dactlam.p + a, 1, N, da, N, stream);
          if (sector != 0) project_parity(da, (double)sector);  // stay in the start sector
        }
        // orthogonalise against the whole basis (two classical Gram-Schmidt passes)
        for (int pass = 0; pass < 2; ++pass) {
          ts_gram(V.p, N, m, D.p, N, nact, N, dG.p, gpart, stream);
          ts_gemm(V.p, N, m, dG.p, nact, N, -1.0, 1.0, D.p, N, stream);
        }
        for (int a = 0; a < nact; ++a) {
          double* da = D.p + (size_t)a * N;
          for (int b2 = 0; b2 < a; ++b2) project_out(D.p + (size_t)b2 * N, da);
          ts_gram(da, N, 1, da, N, 1, N, dnrm.p + a, gpart, stream);
          scale_inv_norm(da, N, dnrm.p + a, stream);
        }
        SHCI_CUDA(cudaMemcpyAsync(pin + kPinNrm, dnrm.p, (size_t)nact * sizeof(double), cudaMemcpyDeviceToHost,
                                  stream));
        if (collapse) {
          ts_gemm(V.p, N, m, dQ.p, keep, N, 1.0, 0.0, Vt.p, N, stream);
          ts_gemm(W.p, N, m, dQ.p, keep, N, 1.0, 0.0, Wt.p, N, stream);
          SHCI_CUDA(cudaMemcpyAsync(V.p, Vt.p, (size_t)keep * N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
          SHCI_CUDA(cudaMemcpyAsync(W.p, Wt.p, (size_t)keep * N * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        }
        SHCI_CUDA(cudaMemcpyAsync(V.p + (size_t)m1 * N, D.p, (size_t)nact * N * sizeof(double),
                                  cudaMemcpyDeviceToDevice, stream));
        apply_sigma(mode, V.p, N, m1, nact, W.p, N, m1);
        // only the new columns of G = V^T W: (m1 + nact) x nact
        ts_gram(V.p, N, m1 + nact, W.p + (size_t)m1 * N, N, nact, N, dG.p, gpart, stream);
        SHCI_CUDA(cudaMemcpyAsync(pin + kPinG, dG.p, (size_t)(m1 + nact) * nact * sizeof(double),
                                  cudaMemcpyDeviceToHost, stream));
      });
      sigma_deferred = false;
      SHCI_CUDA(cudaStreamSynchronize(stream));
      if (trace_level() > 0) t_g2 += now_s() - t_loop0, t_loop0 = now_s();
      if (use_graphs) {
        float ms = 0.f;
        SHCI_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        t_sigma += ms * 1e-3;
        n_sigma += 1;
      }
      bool dependent = false;
      for (int a = 0; a < nact; ++a) dependent |= !(std::sqrt(pin[kPinNrm + a]) > 1e-14);
      if (!dependent) {
        // G of the new basis: the kept block (rotated on the host after a
        // collapse: Q_k^T G Q_k) plus the new columns from the device
        const int mm = m1 + nact;
        std::vector<double> Gn((size_t)mm * mm, 0.0);
        if (collapse) {
          std::vector<double> T((size_t)m * keep, 0.0);  // hs Q_k (m x keep, column-major)
          for (int b2 = 0; b2 < keep; ++b2)
            for (int i = 0; i < m; ++i) {
              double t = 0.0;
              for (int j = 0; j < m; ++j) t += hs[(size_t)i * m + j] * Q[(size_t)j + (size_t)b2 * m];
              T[(size_t)i + (size_t)b2 * m] = t;
            }
          for (int b2 = 0; b2 < keep; ++b2)
            for (int a2 = 0; a2 < keep; ++a2) {
              double t = 0.0;
              for (int i = 0; i < m; ++i) t += Q[(size_t)i + (size_t)a2 * m] * T[(size_t)i + (size_t)b2 * m];
              Gn[(size_t)a2 + (size_t)b2 * mm] = t;
            }
        } else {
          for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) Gn[(size_t)i + (size_t)j * mm] = G[(size_t)i + (size_t)j * m];
        }
        for (int j = 0; j < nact; ++j)
          for (int i = 0; i < mm; ++i) {
            const double g = pin[kPinG + (size_t)i + (size_t)j * mm];
            Gn[(size_t)i + (size_t)(m1 + j) * mm] = g;
            Gn[(size_t)(m1 + j) + (size_t)i * mm] = g;
          }
        m = mm;
        G.swap(Gn);
        continue;
      }
      // Some correction was linearly dependent on the basis (rare: tiny or
      // exhausted spaces). Drop it, as the reference does, and redo the
      // append and sigma for the others on the stream directly; the rotated
      // basis (if collapsed) is kept.
      int kept = 0;
      for (int a = 0; a < nact; ++a) {
        if (!(std::sqrt(pin[kPinNrm + a]) > 1e-14)) continue;
        if (kept != a)
          SHCI_CUDA(cudaMemcpyAsync(D.p + (size_t)kept * N, D.p + (size_t)a * N, N * sizeof(double),
                                    cudaMemcpyDeviceToDevice, stream));
        ++kept;
      }
      m = m1;
      if (kept == 0) {  // nothing new to add: the subspace is exhausted
        G = gram_host(V.p, N, m, W.p, N, m);
        std::vector<double> hs2((size_t)m * m);
        for (int i = 0; i < m; ++i)
          for (int j = i; j < m; ++j) hs2[(size_t)i * m + j] = hs2[(size_t)j * m + i] = G[(size_t)i + (size_t)j * m];
        sym_eig(m, hs2, lam, Q);
        to_dev(dQ, Q);
        to_dev(dlam, std::vector<double>(lam.begin(), lam.begin() + nroots));
        ts_gemm(V.p, N, m, dQ.p, nroots, N, 1.0, 0.0, X.p, N, stream);
        finish();
        return;
      }
      SHCI_CUDA(cudaMemcpyAsync(V.p + (size_t)m * N, D.p, (size_t)kept * N * sizeof(double),
                                cudaMemcpyDeviceToDevice, stream));
      apply_sigma(mode, V.p, N, m, kept, W.p, N, m);
      m += kept;
      G = gram_host(V.p, N, m, W.p, N, m);
    }
  }

  // Shift of the preconditioner for the current space at energy estimate E
  // (NaN: unknown, plain preconditioner).
  void prepare_shift(double E) {
    shift_ready = false;
    if (precond == 0 || !(E == E) || ndet == 0) return;
    shift.resize(ndet);
    if (precond == 1) {
      if (!whole_ham()) return;
      pt2_shift(H, diag.p, E, shift.p, pt2inv, stream);
      shift_ready = true;
    } else if (precond == 2 && mlp.trained && mlp_ok && mlp.nspin == 2 * hints.norb) {
      mlp.infer(dets.p, diag.p, ndet, E, shift.p, stream);
      shift_ready = true;
    }
  }

  // Trains the MLP on the second-order shifts of (a sample of) the current
  // space at energy E, the pairs the Davidson run itself produced. Returns the
  // final minibatch loss.
  // steps: Adam steps of this call (0 = mlp_steps)
  double train_mlp(double E, int steps = 0) {
    if (!whole_ham()) throw Error(kErrState, "training needs the stored Hamiltonian of the whole space");
    ensure_diag();
    if (mlp.nspin != 2 * hints.norb) mlp.init(2 * hints.norb, 7, stream);
    PhaseTimer pt(stream);
    teacher.resize(ndet);
    pt2_shift(H, diag.p, E, teacher.p, pt2inv, stream);
    pt.mark("mlp teacher");
    const int64_t ns = std::min<int64_t>(mlp_sample, (int64_t)ndet);
    // rows drawn on the device (hashed, with replacement), targets scaled to unit rms
    tr_idx.resize(ns);
    tr_tgt.resize(ns);
    mlp.sigma = shci::mlp_sample(teacher.p, ndet, ns, 0x2545F4914F6CDD1Dull ^ (uint64_t)ndet, tr_idx.p, tr_tgt.p,
                                 gpart, stream);
    pt.mark("mlp sample");
    const int B = (int)std::min<int64_t>(mlp_batch, ns);
    double loss = 0.0;
    const int nsteps = steps > 0 ? steps : mlp_steps;
    for (int s = 0; s < nsteps; ++s) {
      const int64_t off = ((int64_t)s * B) % std::max<int64_t>(1, ns - B + 1);
      loss = mlp.gradient(dets.p, diag.p, tr_idx.p + off, tr_tgt.p + off, B, E, stream, s + 1 == nsteps);
      mlp.adam(mlp_lr, stream);
    }
    SHCI_CUDA(cudaStreamSynchronize(stream));
    pt.mark("mlp steps");
    mlp.trained = true;
    mlp_ok = true;  // trained explicitly on the level-shift target: used as asked
    last_loss = loss;
    return loss;
  }

  // Trains the MLP on the (residual, correction) pairs recorded during the
  // last solve, whose converged root-0 vector is c (device, ndet entries), at
  // energy E (pair_targets in kernels_mlp.cu gives the target of a pair).
  // No stored Hamiltonian is needed, so the matrix-free path uses it too.
  // Returns the final minibatch loss (the previous one when the solve left
  // too few informative pairs).
  double train_mlp_pairs(const double* c, double E, int steps = 0) {
    ensure_diag();
    const size_t N = ndet;
    const int nsnap = n_snap;
    n_snap = 0;
    if (nsnap < 2 || N < 64) return last_loss;  // nothing to hold out for the judge
    PhaseTimer pt(stream);
    if (mlp.nspin != 2 * hints.norb) mlp.init(2 * hints.norb, 7, stream);
    // training pairs from every recorded iteration but the last, which the
    // judge holds out
    int64_t m = 0;
    double cks[kSnaps];
    for (int k = 0; k < nsnap; ++k) {
      const double* xk = snapX.p + (size_t)k * N;
      cks[k] = gram_host(c, N, 1, xk, N, 1)[0];
      if (k == nsnap - 1) break;
      if (!(std::fabs(cks[k]) > 0.5)) continue;  // too far from x* for the first-order relation
      const double* rk = snapR.p + (size_t)k * N;
      // entries far below the rms of r_k or of e = x*/ck - x_k (|e|^2 = 1/ck^2 - 1)
      // are at the rounding level
      const double rrms = norm_host(rk) / std::sqrt((double)N);
      const double erms = std::sqrt(std::max(0.0, 1.0 / (cks[k] * cks[k]) - 1.0)) / std::sqrt((double)N);
      if (!(erms > 0.0)) continue;
      m += pair_targets(xk, rk, c, cks[k], diag.p, snap_theta[k], N, 1e-3 * rrms, 1e-3 * erms, m, pair_idx, pair_tgt,
                        pair_tmp, pair_flag, pair_pos, prims, stream);
    }
    last_pairs = m;
    pt.mark("mlp pairs");
    if (m < 256) return last_loss;
    const int64_t ns = std::min<int64_t>(mlp_sample, m);
    tr_idx.resize(ns);
    tr_tgt.resize(ns);
    mlp.sigma = mlp_sample_pairs(pair_idx.p, pair_tgt.p, m, ns, 0x2545F4914F6CDD1Dull ^ (uint64_t)N, tr_idx.p,
                                 tr_tgt.p, gpart, stream);
    const int B = (int)std::min<int64_t>(mlp_batch, ns);
    double loss = 0.0;
    const int nsteps = steps > 0 ? steps : mlp_steps;
    for (int st = 0; st < nsteps; ++st) {
      const int64_t off = ((int64_t)st * B) % std::max<int64_t>(1, ns - B + 1);
      loss = mlp.gradient(dets.p, diag.p, tr_idx.p + off, tr_tgt.p + off, B, E, stream, st + 1 == nsteps);
      mlp.adam(mlp_lr, stream);
    }
    mlp.trained = true;
    last_loss = loss;
    pt.mark("mlp steps");
    // the judge: the network is used from the next solve on only if, on the
    // held-out iteration, its corrections point at the needed correction
    // better than the plain preconditioner's
    const int kv = nsnap - 1;
    mlp_ok = false;
    // a held-out iteration already at the solution (|e|^2 = 1/ck^2 - 1 at the
    // rounding level) judges nothing
    if (std::fabs(cks[kv]) > 0.5 && 1.0 / (cks[kv] * cks[kv]) - 1.0 > 1e-10) {
      teacher.resize(N);
      mlp.infer(dets.p, diag.p, N, snap_theta[kv], teacher.p, stream);
      judge_preconditioners(snapX.p + (size_t)kv * N, snapR.p + (size_t)kv * N, c, cks[kv], diag.p, teacher.p,
                            snap_theta[kv], N, gpart, stream, &judge_cos_plain, &judge_cos_learned);
      mlp_ok = judge_cos_learned > 1.05 * judge_cos_plain;  // a clear margin, not noise
    }
    if (trace_level() > 0)
      std::fprintf(stderr, "[mlp] %lld pairs, loss %.4f, judge cos plain %.6f learned %.6f -> %s\n", (long long)m,
                   loss, judge_cos_plain, judge_cos_learned, mlp_ok ? "learned" : "plain");
    return loss;
  }

  void davidson(int mode, bool block, int nroots, double* x, int maxCopies, double tol, bool direct_rules,
                std::vector<double>& E, int& iters, double E_est = std::nan("")) {
    if (!ham_ok) throw Error(kErrState, "Hamiltonian not built for the current space (call shci_ham_build)");
    if (H.block)
      throw Error(kErrState, "the stored Hamiltonian is a row block (shci_ham_build_rows); Davidson needs the whole "
                             "matrix on this context (shci_ham_build)");
    ensure_diag();
    prepare_shift(E_est);
    if (mode == SHCI_MODE_MIXED || mode == SHCI_MODE_DIRECT_MIXED) {
      // FP32 stage, then the refinement stage continues on the same basis with
      // W recomputed accurately (stored: head + tail values in float-float;
      // matrix-free: FP64 elements and accumulation)
      const int refine = mode == SHCI_MODE_MIXED ? SHCI_MODE_FP64 : SHCI_MODE_DIRECT;
      int it1 = 0, it2 = 0, m = 0;
      davidson_core(mode, block, nroots, x, maxCopies, tol, direct_rules, E, it1, true, 0, &m);
      // converged in FP32: one accurate sigma of the Ritz vectors usually
      // confirms it; stopped at the FP32 floor: keep the whole basis
      davidson_core(refine, block, nroots, x, maxCopies, tol, direct_rules, E, it2, false, last_stalled ? m : 0);
      iters = it1 + it2;
    } else {
      davidson_core(mode, block, nroots, x, maxCopies, tol, direct_rules, E, iters);
    }
  }

  // ---- variational driver (SHCIbasics::DoVariational) -----------------------
  // ---- checkpoints (writeVariationalResult / readVariationalResult,
  // SHCI/SHCIbasics.cpp:1481-1590): the iteration, the determinants, the
  // coefficients of every root and E0 (core energy excluded), in this
  // library's own binary layout (the reference writes Boost archives).
  static constexpr char kChkMagic[8] = {'S', 'H', 'C', 'I', 'G', 'P', 'U', '1'};
  static std::string checkpoint_path(const Schedule& s) {
    std::string dir = s.prefix.empty() ? std::string(".") : s.prefix;
    if (dir[0] != '/') dir = s.baseDir + "/" + dir;
    return dir + "/shci_gpu-variational.chk";
  }
  void write_checkpoint(const std::string& path, int iter, int nroots, const std::vector<double>& E0) {
    std::vector<uint64_t> hd(2 * ndet);
    std::vector<double> hc((size_t)nroots * ndet);
    SHCI_CUDA(cudaMemcpyAsync(hd.data(), dets.p, ndet * sizeof(Det2), cudaMemcpyDeviceToHost, stream));
    SHCI_CUDA(cudaMemcpyAsync(hc.data(), ci.p, hc.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    SHCI_CUDA(cudaStreamSynchronize(stream));
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error(kErrIO, "cannot write checkpoint " + path);
    const int32_t head[4] = {1, iter, 1, nroots};  // version, iteration, converged (as the reference saves it), roots
    const int64_t n = (int64_t)ndet;
    const int32_t norb = hints.norb;
    bool ok = std::fwrite(kChkMagic, 1, 8, f) == 8 && std::fwrite(head, sizeof(head), 1, f) == 1 &&
              std::fwrite(&n, sizeof(n), 1, f) == 1 && std::fwrite(&norb, sizeof(norb), 1, f) == 1 &&
              std::fwrite(hd.data(), sizeof(uint64_t), hd.size(), f) == hd.size() &&
              std::fwrite(hc.data(), sizeof(double), hc.size(), f) == hc.size() &&
              std::fwrite(E0.data(), sizeof(double), (size_t)nroots, f) == (size_t)nroots;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) throw Error(kErrIO, "failed writing checkpoint " + path);
  }
  // Loads the space and coefficients; returns the saved iteration.
  int read_checkpoint(const std::string& path, int nroots, bool& converged, std::vector<double>& E0) {
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error(kErrIO, "cannot open checkpoint " + path + " (restart needs the files of an earlier run)");
    char magic[8];
    int32_t head[4];
    int64_t n = 0;
    int32_t norb = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kChkMagic, 8) == 0 &&
              std::fread(head, sizeof(head), 1, f) == 1 && std::fread(&n, sizeof(n), 1, f) == 1 &&
              std::fread(&norb, sizeof(norb), 1, f) == 1 && head[0] == 1 && n > 0 && n < ((int64_t)1 << 31);
    if (ok && (norb != hints.norb || head[3] != nroots)) {
      std::fclose(f);
      throw Error(kErrInvalid, "checkpoint " + path + " was written for another system or number of roots");
    }
    std::vector<uint64_t> hd;
    std::vector<double> hc;
    if (ok) {
      hd.resize(2 * (size_t)n);
      hc.resize((size_t)nroots * (size_t)n);
      E0.assign(nroots, 0.0);
      ok = std::fread(hd.data(), sizeof(uint64_t), hd.size(), f) == hd.size() &&
           std::fread(hc.data(), sizeof(double), hc.size(), f) == hc.size() &&
           std::fread(E0.data(), sizeof(double), (size_t)nroots, f) == (size_t)nroots;
    }
    std::fclose(f);
    if (!ok) throw Error(kErrIO, "checkpoint " + path + " is not a complete checkpoint of this library");
    set_dets(hd.data(), n);
    ci.resize(hc.size());
    SHCI_CUDA(cudaMemcpyAsync(ci.p, hc.data(), hc.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    SHCI_CUDA(cudaStreamSynchronize(stream));
    converged = head[2] != 0;
    return head[1];
  }

  void run(const Schedule& s, int mode, bool block, std::vector<double>& Eout) {
    require_ints();
    const double t0 = now_s();
    t_select = t_ham = t_dav = t_sigma = t_mlp = 0;
    n_sigma = 0;
    total_dav_iters = 0;
    shift_ready = false;
    mlp.trained = false;
    mlp_ok = false;
    log.clear();
    if (s.direct)
      mode = (mode == SHCI_MODE_MIXED || mode == SHCI_MODE_DIRECT_MIXED) ? SHCI_MODE_DIRECT_MIXED : SHCI_MODE_DIRECT;
    // selection parameters
    sp.ncore = s.ncore;
    sp.nact = s.nact;
    sp.nrestrict = (int)s.restrictions.size();
    for (int r = 0; r < sp.nrestrict; ++r) {
      sp.rmin[r] = s.restrictions[r].minElec;
      sp.rmax[r] = s.restrictions[r].maxElec;
      uint64_t m0 = 0, m1 = 0;
      for (int k = 0; k < 64; ++k)
        if ((s.restrictions[r].mask >> k) & 1ull) {
          for (int spn = 0; spn < 2; ++spn) {
            int p = 2 * k + spn;
            if (p < 64)
              m0 |= 1ull << p;
            else
              m1 |= 1ull << (p - 64);
          }
        }
      sp.rmask0[r] = m0;
      sp.rmask1[r] = m1;
    }
    // time reversal: off for an odd number of electrons (SHCI/SHCI.cpp:188-195);
    // the sector applies to this run's solves only
    const int trev = (hints.nelec % 2 == 0) ? s.trev : 0;
    trev_sector = 0;
    struct SectorReset {
      int& v;
      ~SectorReset() { v = 0; }
    } sector_reset{trev_sector};
    // reference determinants and initial ci (SHCI/SHCI.cpp:289-399)
    std::vector<uint64_t> hd;
    int lowest = 0;
    double lowestE = 1e300;
    for (size_t d = 0; d < s.occupied.size(); ++d) {
      uint64_t w[2] = {0, 0};
      if ((int)s.occupied[d].size() != hints.nelec)
        throw Error(kErrInvalid, "The number of electrons given in the FCIDUMP should be equal to the nocc given in the shci input file.");
      for (int p : s.occupied[d]) {
        if (p < 0 || p >= 2 * hints.norb) throw Error(kErrInvalid, "orbital index out of range in nocc");
        if ((w[p >> 6] >> (p & 63)) & 1ull)
          throw Error(kErrInvalid, "orbital " + std::to_string(p) + " appears twice in input determinant number " +
                                       std::to_string(d));
        w[p >> 6] |= 1ull << (p & 63);
      }
      if (trev != 0) {  // makeStandard (SHCI/SHCI.cpp:302)
        Det2 dd{w[0], w[1]};
        if (__builtin_popcountll(det_alpha(dd)) != __builtin_popcountll(det_beta(dd)))
          throw Error(kErrInvalid, "time reversal (Treversal) needs as many alpha as beta electrons");
        if (!det_is_standard(dd)) dd = det_flip_pair(dd);
        w[0] = dd.w0;
        w[1] = dd.w1;
      }
      for (size_t e = 0; e < d; ++e)
        if (hd[2 * e] == w[0] && hd[2 * e + 1] == w[1])
          throw Error(kErrInvalid, "Determinant appears twice in the input determinant list.");
      hd.push_back(w[0]);
      hd.push_back(w[1]);
      double E = 0.0;
      {
        std::vector<int> cl;
        for (int p = 0; p < 2 * hints.norb; ++p)
          if ((w[p >> 6] >> (p & 63)) & 1ull) cl.push_back(p);
        const int n2 = 2 * hints.norb;
        for (size_t i = 0; i < cl.size(); ++i) {
          E += hints.I1[(size_t)cl[i] * n2 + cl[i]];
          for (size_t j = i + 1; j < cl.size(); ++j) {
            E += hints.Direct[(size_t)(cl[i] / 2) * hints.norb + cl[j] / 2];
            if ((cl[i] % 2) == (cl[j] % 2)) E -= hints.Exchange[(size_t)(cl[i] / 2) * hints.norb + cl[j] / 2];
          }
        }
      }
      if (E < lowestE) {
        lowestE = E;
        lowest = (int)d;
      }
    }
    if (s.occupied.empty()) throw Error(kErrInvalid, "nocc keyword has to be included.");
    const size_t nin = s.occupied.size();
    // with time reversal the flipped partners of the open-shell input
    // determinants follow them (the pair's basis function is spread over both)
    std::vector<size_t> partner(nin, (size_t)-1);
    if (trev != 0) {
      const int nbeta = __builtin_popcountll(det_beta(Det2{hd[0], hd[1]}));
      trev_sector = trev * ((nbeta % 2) ? -1 : 1);
      for (size_t d = 0; d < nin; ++d) {
        const Det2 dd{hd[2 * d], hd[2 * d + 1]};
        const Det2 f = det_flip_pair(dd);
        if (f.w0 == dd.w0 && f.w1 == dd.w1) continue;
        partner[d] = hd.size() / 2;
        hd.push_back(f.w0);
        hd.push_back(f.w1);
      }
    }
    set_dets(hd.data(), (int64_t)(hd.size() / 2));
    const int nroots = s.nroots;
    if (nroots < 1 || nroots > 16) throw Error(kErrInvalid, "nroots must be in 1..16");
    nroots_run = nroots;
    {
      // the reference's guess over its (symmetrized) basis functions: 1 each,
      // plus the count on the lowest, normalised; a pair's coefficient c goes
      // to its two determinants as c/sqrt(2) and sector * sign * c/sqrt(2)
      const size_t n0 = ndet;
      std::vector<double> c0(n0 * nroots, 0.0);
      for (size_t j = 0; j < nin; ++j) c0[j] = 1.0;
      c0[lowest] += (double)nin;
      double nn = 0.0;
      for (size_t j = 0; j < nin; ++j) nn += c0[j] * c0[j];
      nn = std::sqrt(nn);
      for (size_t j = 0; j < nin; ++j) c0[j] /= nn;
      for (size_t j = 0; j < nin; ++j)
        if (partner[j] != (size_t)-1) {
          const uint64_t a = det_alpha(Det2{hd[2 * j], hd[2 * j + 1]}), b = det_beta(Det2{hd[2 * j], hd[2 * j + 1]});
          const double sgn = (__builtin_popcountll(a & b) & 1) ? -1.0 : 1.0;
          c0[j] /= std::sqrt(2.0);
          c0[partner[j]] = trev_sector * sgn * c0[j];
        }
      ci.resize(n0 * nroots);
      SHCI_CUDA(cudaMemcpyAsync(ci.p, c0.data(), c0.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    }
    std::vector<double> E0(nroots, 0.0);
    const std::string chk = checkpoint_path(s);
    size_t iterstart = 0;
    if (s.restart) {  // SHCI/SHCIbasics.cpp:871-943
      bool converged = false;
      const int saved = read_checkpoint(chk, nroots, converged, E0);
      iterstart = s.restart == 2 ? 0 : (size_t)saved + 1;
      if (s.restart == 1 && converged && saved >= 0 && (size_t)saved < s.epsilon1.size() &&
          s.epsilon1[saved] <= s.epsilon1.back())
        iterstart = s.epsilon1.size();  // converged at the final threshold: nothing left to iterate
    }
    DevBuf<double> X0;
    for (size_t iter = iterstart; iter < s.epsilon1.size(); ++iter) {
      const double eps1 = s.epsilon1[iter];
      const size_t N0 = ndet;
      double ta = now_s();
      cmax.resize(N0);
      if (trev_sector != 0) {
        if (!ensure_flip())
          throw Error(kErrState, "time reversal needs the flipped partner of every determinant in the space");
        trev_cmax(dets.p, ci.p, N0, nroots, N0, flipidx.p, cmax.p, stream);
        select_trev(cmax.p, eps1);
      } else {
        k_cmax<<<grid_for(N0, 256), 256, 0, stream>>>(ci.p, N0, nroots, N0, cmax.p);
        SHCI_LAUNCH_CHECK();
        select(cmax.p, eps1);
      }
      const size_t N = ndet;
      if (trace_level() > 0)
        std::fprintf(stderr, "[select] %zu eps1=%.3e ndets %zu -> %zu in %.3f s\n", iter, eps1, N0, N, now_s() - ta);
      // X0 = [ci; 0]
      X0.resize(N * nroots);
      SHCI_CUDA(cudaMemsetAsync(X0.p, 0, N * nroots * sizeof(double), stream));
      for (int r = 0; r < nroots; ++r)
        SHCI_CUDA(cudaMemcpyAsync(X0.p + (size_t)r * N, ci.p + (size_t)r * N0, N0 * sizeof(double),
                                  cudaMemcpyDeviceToDevice, stream));
      double tb = now_s();
      t_select += tb - ta;
      build_ham(mode);
      double tc = now_s();
      t_ham += tc - tb;
      const double prevE0 = (iter == 0) ? -10.0 : E0[0];
      int numIter = 0;
      const int maxCopies = basis_max > 0 ? basis_max
                            : (block ? std::max(nroots + 4, 3 * nroots) : (s.direct ? nroots + 2 : nroots + 4));
      // the shifted preconditioners need an energy: the previous iteration's
      const double E_est = iter == 0 ? std::nan("") : E0[0];
      n_snap = 0;
      record_pairs = precond == 2;
      davidson(mode, block, nroots, X0.p, maxCopies, s.davidsonTolLoose, s.direct, E0, numIter, E_est);
      record_pairs = false;
      ci.swap(X0);
      double td = now_s();
      t_dav += td - tc;
      log.push_back({(int64_t)N, E0[0] + hints.coreE, numIter, td - t0});
      total_dav_iters += numIter;
      if (trace_level() > 0)  // the reference's per-iteration table line, plus the matrix size
        std::fprintf(stderr, "[iter] %zu eps1=%.3e ndets=%zu nnz=%lld csr_bytes=%zu helper_bytes=%zu E=%.12f "
                             "davidson=%d t=%.3f\n", iter, eps1, N, (long long)H.nnz, H.bytes(), helpers.bytes(),
                     E0[0] + hints.coreE, numIter, td - t0);
      if (precond == 2) {
        // (residual, correction) pairs of this solve, used from the next solve
        // on; later calls refine the network already trained (a third of the
        // steps)
        train_mlp_pairs(ci.p, E0[0], mlp.trained ? std::max(1, mlp_steps / 3) : 0);
        t_mlp += now_s() - td;
      }
      if (std::fabs(E0[0] - prevE0) < s.dE || iter == s.epsilon1.size() - 1) {
        const double t1 = now_s();
        davidson(mode, block, nroots, ci.p,
                 basis_max > 0 ? basis_max : (block ? std::max(nroots + 4, 3 * nroots) : nroots + 4), s.davidsonTol,
                 s.direct, E0, numIter, E0[0]);
        total_dav_iters += numIter;
        t_dav += now_s() - t1;
        if (s.io) write_checkpoint(chk, (int)iter, nroots, E0);
        break;
      }
      if (s.io) write_checkpoint(chk, (int)iter, nroots, E0);
    }
    Eout.resize(nroots);
    for (int r = 0; r < nroots; ++r) Eout[r] = E0[r] + hints.coreE;
    Evar = Eout;
    run_eps2 = s.epsilon2;
    run_sched = s;
    t_total = now_s() - t0;
  }
};

}  // namespace shci

// ===========================================================================
// C-ABI
// ===========================================================================
using shci::Context;
using shci::Error;

struct shci_ctx {
  Context c;
};

namespace {
thread_local std::string g_create_error;

template <class F>
int guarded(shci_ctx* ctx, F&& f) {
  if (!ctx) return SHCI_ERR_INVALID;
  try {
    ctx->c.err.clear();
    cudaSetDevice(ctx->c.device);
    shci::AllocStream scope(ctx->c.stream);  // this call's buffers: the device pool, in this stream's order
    f(ctx->c);
    return SHCI_OK;
  } catch (const Error& e) {
    ctx->c.err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    ctx->c.err = e.what();
    return SHCI_ERR_INVALID;
  }
}
}  // namespace

extern "C" {

int shci_ctx_create(int device, shci_ctx** out) {
  if (!out) return SHCI_ERR_INVALID;
  *out = nullptr;
  try {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      g_create_error = "no CUDA device available";
      return SHCI_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) {
      g_create_error = "device index out of range";
      return SHCI_ERR_INVALID;
    }
    std::unique_ptr<shci_ctx> ctx(new shci_ctx());
    ctx->c.device = device;
    SHCI_CUDA(cudaSetDevice(device));
    SHCI_CUDA(cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking));
    SHCI_CUDA(cudaEventCreate(&ctx->c.ev0));
    SHCI_CUDA(cudaEventCreate(&ctx->c.ev1));
    SHCI_CUDA(cudaMallocHost(&ctx->c.pin, Context::kPin * sizeof(double)));
    *out = ctx.release();
    return SHCI_OK;
  } catch (const Error& e) {
    g_create_error = e.what();
    return e.code;
  }
}

int shci_ctx_destroy(shci_ctx* ctx) {
  if (!ctx) return SHCI_ERR_INVALID;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  delete ctx;
  try {
    shci::release_pool_memory(nullptr);  // the context's memory back to the device
  } catch (const std::exception&) {
  }
  return SHCI_OK;
}

const char* shci_last_error(shci_ctx* ctx) { return ctx ? ctx->c.err.c_str() : g_create_error.c_str(); }

void* shci_ctx_stream(shci_ctx* ctx) { return ctx ? (void*)ctx->c.stream : nullptr; }

int shci_set_alloc_cap(shci_ctx* ctx, uint64_t bytes) {
  return guarded(ctx, [&](Context&) { shci::g_alloc_cap = (size_t)bytes; });
}

int shci_read_fcidump(shci_ctx* ctx, const char* path, int* norb, int* nelec, double* coreE) {
  return guarded(ctx, [&](Context& c) {
    if (!path) throw Error(SHCI_ERR_INVALID, "null path");
    c.load_fcidump(path);
    if (norb) *norb = c.hints.norb;
    if (nelec) *nelec = c.hints.nelec;
    if (coreE) *coreE = c.hints.coreE;
  });
}

int shci_fcidump_info(const char* path, int* norb, int* nelec, double* coreE, int64_t* nnz_i2) {
  try {
    g_create_error.clear();
    if (!path) throw Error(SHCI_ERR_INVALID, "null path");
    shci::HostInts H;
    shci::read_fcidump(path, H);
    if (norb) *norb = H.norb;
    if (nelec) *nelec = H.nelec;
    if (coreE) *coreE = H.coreE;
    if (nnz_i2) {
      int64_t n = 0;
      for (double v : H.I2) n += v != 0.0;
      *nnz_i2 = n;
    }
    return SHCI_OK;
  } catch (const Error& e) {
    g_create_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_create_error = e.what();
    return SHCI_ERR_INVALID;
  }
}

int shci_input_info(const char* path, double* eps1, int cap_eps, int* n_eps, double* tols, int* ints) {
  try {
    g_create_error.clear();
    if (!path) throw Error(SHCI_ERR_INVALID, "null path");
    shci::Schedule s;
    shci::read_input(path, s);
    if (n_eps) *n_eps = (int)s.epsilon1.size();
    for (int i = 0; eps1 && i < cap_eps && i < (int)s.epsilon1.size(); ++i) eps1[i] = s.epsilon1[i];
    if (tols) {
      tols[0] = s.davidsonTol;
      tols[1] = s.davidsonTolLoose;
      tols[2] = s.dE;
    }
    if (ints) {
      ints[0] = s.nroots;
      ints[1] = (int)s.occupied.size();
      ints[2] = s.ncore;
      ints[3] = s.nact;
      ints[4] = s.mode;
      ints[5] = s.block ? 1 : 0;
      ints[6] = s.precond;
      ints[7] = s.basis_max;
    }
    return SHCI_OK;
  } catch (const Error& e) {
    g_create_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_create_error = e.what();
    return SHCI_ERR_INVALID;
  }
}

int shci_heatbath_export(shci_ctx* ctx, int which, int64_t* count, float* vals, int16_t* pairs, int64_t* starts,
                         double* singles) {
  return guarded(ctx, [&](Context& c) {
    c.require_ints();
    const auto& V = which ? c.hhb.sameVal : c.hhb.oppVal;
    const auto& P = which ? c.hhb.samePairs : c.hhb.oppPairs;
    const auto& S = which ? c.hhb.sameStart : c.hhb.oppStart;
    if (count) *count = (int64_t)V.size();
    if (vals) std::memcpy(vals, V.data(), V.size() * sizeof(float));
    if (pairs) std::memcpy(pairs, P.data(), P.size() * sizeof(int16_t));
    if (starts) std::memcpy(starts, S.data(), S.size() * sizeof(int64_t));
    if (singles) std::memcpy(singles, c.hhb.singles.data(), c.hhb.singles.size() * sizeof(double));
  });
}

int shci_set_selection_params(shci_ctx* ctx, int ncore, int nact, int nrestrict, const int* rmin, const int* rmax,
                              const uint64_t* spatial_masks) {
  return guarded(ctx, [&](Context& c) {
    if (nrestrict < 0 || nrestrict > shci::kMaxRestrict) throw Error(SHCI_ERR_INVALID, "at most 4 restrictions");
    if (ncore < 0 || nact < 0) throw Error(SHCI_ERR_INVALID, "ncore/nact must be >= 0");
    c.sp.ncore = ncore;
    c.sp.nact = nact;
    c.sp.nrestrict = nrestrict;
    for (int r = 0; r < nrestrict; ++r) {
      c.sp.rmin[r] = rmin[r];
      c.sp.rmax[r] = rmax[r];
      uint64_t m0 = 0, m1 = 0;
      for (int k = 0; k < 64; ++k)
        if ((spatial_masks[r] >> k) & 1ull)
          for (int s = 0; s < 2; ++s) {
            int p = 2 * k + s;
            if (p < 64) m0 |= 1ull << p; else m1 |= 1ull << (p - 64);
          }
      c.sp.rmask0[r] = m0;
      c.sp.rmask1[r] = m1;
    }
  });
}

int shci_dets_set(shci_ctx* ctx, const uint64_t* dets, int64_t n) {
  return guarded(ctx, [&](Context& c) {
    if (n > 0 && !dets) throw Error(SHCI_ERR_INVALID, "null determinant array");
    c.set_dets(dets, n);
  });
}

int shci_dets_count(shci_ctx* ctx, int64_t* n) {
  return guarded(ctx, [&](Context& c) { *n = (int64_t)c.ndet; });
}

int shci_dets_get(shci_ctx* ctx, uint64_t* out, int64_t cap) {
  return guarded(ctx, [&](Context& c) {
    if (cap < (int64_t)c.ndet) throw Error(SHCI_ERR_INVALID, "output buffer too small");
    if (c.ndet)
      SHCI_CUDA(cudaMemcpyAsync(out, c.dets.p, c.ndet * sizeof(shci::Det2), cudaMemcpyDeviceToHost, c.stream));
    SHCI_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int shci_select(shci_ctx* ctx, const double* cmax, double eps1, int64_t* n_new) {
  return guarded(ctx, [&](Context& c) {
    c.require_dets();
    if (!cmax) throw Error(SHCI_ERR_INVALID, "null cmax");
    c.cmax.resize(c.ndet);
    SHCI_CUDA(cudaMemcpyAsync(c.cmax.p, cmax, c.ndet * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    int64_t k = c.select(c.cmax.p, eps1);
    if (n_new) *n_new = k;
  });
}

int shci_select_candidates(shci_ctx* ctx, const double* cmax, double eps1, int rank, int world, int64_t* n_new) {
  return guarded(ctx, [&](Context& c) {
    c.require_dets();
    if (!cmax) throw Error(SHCI_ERR_INVALID, "null cmax");
    if (world < 1 || rank < 0 || rank >= world) throw Error(SHCI_ERR_INVALID, "need 0 <= rank < world");
    // this rank's parents are the determinants i with i % world == rank
    // (SHCI/SHCIbasics.cpp:969-970); the others get cMax 0, which the
    // selection skips
    std::vector<double> own(c.ndet, 0.0);
    for (size_t i = (size_t)rank; i < c.ndet; i += (size_t)world) own[i] = cmax[i];
    c.cmax.resize(c.ndet);
    SHCI_CUDA(cudaMemcpyAsync(c.cmax.p, own.data(), c.ndet * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    const size_t k = c.candidates(c.cmax.p, eps1);
    if (n_new) *n_new = (int64_t)k;
  });
}

int shci_candidates_get(shci_ctx* ctx, uint64_t* out, int64_t cap) {
  return guarded(ctx, [&](Context& c) {
    if (cap < (int64_t)c.ncand) throw Error(SHCI_ERR_INVALID, "output too small for the candidates");
    if (c.ncand) {
      if (!out) throw Error(SHCI_ERR_INVALID, "null output");
      SHCI_CUDA(cudaMemcpyAsync(out, c.cand.p, c.ncand * sizeof(shci::Det2), cudaMemcpyDeviceToHost, c.stream));
      SHCI_CUDA(cudaStreamSynchronize(c.stream));
    }
  });
}

int shci_dets_append(shci_ctx* ctx, const uint64_t* dets, int64_t n) {
  return guarded(ctx, [&](Context& c) {
    if (n > 0 && !dets) throw Error(SHCI_ERR_INVALID, "null determinants");
    c.append_dets(dets, n);
  });
}

int shci_ham_build(shci_ctx* ctx, int mode, int64_t* nnz) {
  return guarded(ctx, [&](Context& c) {
    c.build_ham(mode);
    if (nnz) *nnz = c.H.nnz;
  });
}

int shci_ham_build_rows(shci_ctx* ctx, int mode, int64_t r0, int64_t r1, int64_t* nnz) {
  return guarded(ctx, [&](Context& c) {
    if (r0 < 0 || r1 < 0) throw Error(SHCI_ERR_INVALID, "negative row index");
    c.build_ham_rows(mode, (size_t)r0, (size_t)r1);
    if (nnz) *nnz = c.H.nnz;
  });
}

int shci_ham_export(shci_ctx* ctx, int64_t* rowptr, int32_t* col, double* val) {
  return guarded(ctx, [&](Context& c) {
    if (!c.whole_ham()) throw Error(SHCI_ERR_STATE, "no stored Hamiltonian of the whole space");
    // the stored matrix is in storage order (sorted by alpha, then beta
    // string); the export is in the determinant order of shci_dets_get with
    // every row's columns ascending
    const size_t N = c.H.N, nnz = (size_t)c.H.nnz;
    std::vector<int64_t> rp(N + 1);
    std::vector<int32_t> cl(nnz);
    std::vector<double> v(nnz);
    std::vector<uint32_t> perm(N), spos(N);
    SHCI_CUDA(cudaMemcpyAsync(rp.data(), c.H.rowptr.p, (N + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, c.stream));
    if (N) {
      SHCI_CUDA(cudaMemcpyAsync(perm.data(), c.H.perm.p, N * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
      SHCI_CUDA(cudaMemcpyAsync(spos.data(), c.H.spos.p, N * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream));
    }
    if (nnz) {
      SHCI_CUDA(cudaMemcpyAsync(cl.data(), c.H.col.p, nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, c.stream));
      if (c.H.v64.p) {
        SHCI_CUDA(cudaMemcpyAsync(v.data(), c.H.v64.p, nnz * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        SHCI_CUDA(cudaStreamSynchronize(c.stream));
      } else {
        std::vector<float> hi(nnz), lo(nnz);
        SHCI_CUDA(cudaMemcpyAsync(hi.data(), c.H.vhi.p, nnz * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
        SHCI_CUDA(cudaMemcpyAsync(lo.data(), c.H.vlo.p, nnz * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
        SHCI_CUDA(cudaStreamSynchronize(c.stream));
        for (size_t i = 0; i < nnz; ++i) v[i] = (double)hi[i] + (double)lo[i];
      }
    }
    SHCI_CUDA(cudaStreamSynchronize(c.stream));
    rowptr[0] = 0;
    for (size_t u = 0; u < N; ++u) rowptr[u + 1] = rowptr[u] + (rp[spos[u] + 1] - rp[spos[u]]);
    std::vector<std::pair<int32_t, double>> row;
    for (size_t u = 0; u < N; ++u) {
      const int64_t p0 = rp[spos[u]], p1 = rp[spos[u] + 1];
      row.clear();
      for (int64_t p = p0; p < p1; ++p) row.emplace_back((int32_t)perm[cl[p]], v[p]);
      std::sort(row.begin(), row.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
      for (size_t t = 0; t < row.size(); ++t) {
        col[rowptr[u] + t] = row[t].first;
        val[rowptr[u] + t] = row[t].second;
      }
    }
  });
}

int shci_diag(shci_ctx* ctx, double* out) {
  return guarded(ctx, [&](Context& c) {
    c.require_ints();
    c.ensure_diag();
    if (out)
      SHCI_CUDA(cudaMemcpyAsync(out, c.diag.p, c.ndet * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SHCI_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int shci_sigma(shci_ctx* ctx, int mode, const double* x, double* y, int k) {
  return guarded(ctx, [&](Context& c) {
    if (k < 1 || k > 4) throw Error(SHCI_ERR_INVALID, "k must be in 1..4");
    if (!x || !y) throw Error(SHCI_ERR_INVALID, "null vector");
    const size_t N = c.ndet;
    c.X.reserve(N * k);
    c.Y.reserve(N * k);
    SHCI_CUDA(cudaMemcpyAsync(c.X.p, x, N * k * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    c.ensure_diag();
    c.apply_sigma(mode, c.X.p, N, 0, k, c.Y.p, N, 0);
    SHCI_CUDA(cudaMemcpyAsync(y, c.Y.p, N * k * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SHCI_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int shci_sigma_device(shci_ctx* ctx, int mode, const double* x_dev, double* y_dev, int k, int64_t ld) {
  return guarded(ctx, [&](Context& c) {
    if (k < 1 || k > 4) throw Error(SHCI_ERR_INVALID, "k must be in 1..4");
    if (ld < (int64_t)c.ndet) throw Error(SHCI_ERR_INVALID, "leading dimension smaller than N");
    if (!x_dev || !y_dev) throw Error(SHCI_ERR_INVALID, "null vector");
    c.ensure_diag();
    c.apply_sigma(mode, x_dev, (size_t)ld, 0, k, y_dev, (size_t)ld, 0);
  });
}

int shci_sigma_packed_device(shci_ctx* ctx, int mode, const void* x_packed, int kp, int k, double* y_dev,
                             int64_t ld) {
  return guarded(ctx, [&](Context& c) {
    if (!(kp == 1 || kp == 2 || kp == 4) || k < 1 || k > kp) throw Error(SHCI_ERR_INVALID, "need k <= kp in {1,2,4}");
    if (!x_packed || !y_dev) throw Error(SHCI_ERR_INVALID, "null vector");
    if (!c.whole_ham()) throw Error(SHCI_ERR_STATE, "no stored Hamiltonian of the whole space");
    if (ld < (int64_t)c.ndet) throw Error(SHCI_ERR_INVALID, "leading dimension smaller than N");
    c.ensure_diag();
    // x_packed is in the determinant array's order: its rows are gathered
    // into the stored Hamiltonian's storage order first
    const size_t N = c.ndet;
    if (mode == SHCI_MODE_MIXED) {
      c.xb32.reserve(N * kp);
      shci::gather_rows(x_packed, sizeof(float) * kp, c.H.perm.p, N, c.xb32.p, c.stream);
      shci::sigma_csr_mixed(c.H, c.diag.p, c.xb32.p, kp, k, y_dev, (size_t)ld, c.stream);
    } else if (mode == SHCI_MODE_FP64) {
      // the FP64 values of a plain build; a mixed build's refinement sigma
      // (float-float, shci_sigma_device) needs the column-major FP64 x
      if (!c.H.v64.p)
        throw Error(SHCI_ERR_STATE, "packed FP64 sigma needs a Hamiltonian built in FP64 mode (a mixed build's "
                                    "FP64 refinement sigma is shci_sigma_device)");
      c.xb64.reserve(N * kp);
      shci::gather_rows(x_packed, sizeof(double) * kp, c.H.perm.p, N, c.xb64.p, c.stream);
      shci::sigma_csr_f64(c.H, c.diag.p, c.xb64.p, kp, k, y_dev, (size_t)ld, c.stream);
    } else {
      throw Error(SHCI_ERR_INVALID, "packed sigma supports the stored modes only");
    }
  });
}

int shci_sigma_device_noalloc(shci_ctx* ctx, int mode, const double* x_dev, double* y_dev, int k, int64_t ld) {
  return guarded(ctx, [&](Context& c) {
    if (k < 1 || k > 4) throw Error(SHCI_ERR_INVALID, "k must be in 1..4");
    if (mode != SHCI_MODE_MIXED && mode != SHCI_MODE_FP64)
      throw Error(SHCI_ERR_INVALID, "the allocation-free sigma supports the stored modes (MIXED, FP64) only");
    const size_t need = c.ndet * (size_t)(k == 3 ? 4 : k) * (mode == SHCI_MODE_MIXED ? sizeof(float) : sizeof(double));
    if (need > shci::kNoAllocPackBytes)
      throw Error(SHCI_ERR_INVALID, "allocation-free sigma: N x k needs " + std::to_string(need) +
                                        " bytes of scratch, more than its fixed " +
                                        std::to_string(shci::kNoAllocPackBytes) + " bytes");
    if (!c.whole_ham()) throw Error(SHCI_ERR_STATE, "no stored Hamiltonian of the whole space");
    if (mode == SHCI_MODE_MIXED && c.ham_mode != SHCI_MODE_MIXED)
      throw Error(SHCI_ERR_STATE, "mixed sigma needs a Hamiltonian built in mixed mode");
    if (c.ndiag < c.ndet) throw Error(SHCI_ERR_STATE, "diagonal not computed (call shci_ham_build first)");
    if (ld < (int64_t)c.ndet) throw Error(SHCI_ERR_INVALID, "leading dimension smaller than N");
    if (!x_dev || !y_dev) throw Error(SHCI_ERR_INVALID, "null vector");
    shci::sigma_noalloc(c.H, c.diag.p, mode == SHCI_MODE_MIXED, x_dev, (size_t)ld, k, y_dev, (size_t)ld,
                        c.noalloc_ptr, c.stream);
  });
}

int shci_ham_bytes(shci_ctx* ctx, int64_t* csr_bytes, int64_t* helper_bytes) {
  return guarded(ctx, [&](Context& c) {
    if (csr_bytes) *csr_bytes = (int64_t)c.H.bytes();
    if (helper_bytes) *helper_bytes = (int64_t)c.helpers.bytes();
  });
}

int shci_sigma_bytes(shci_ctx* ctx, int mode, int k, int64_t* bytes) {
  return guarded(ctx, [&](Context& c) {
    if (!bytes || k < 1 || k > 4) throw Error(SHCI_ERR_INVALID, "need bytes and 1 <= k <= 4");
    if (!c.whole_ham()) throw Error(SHCI_ERR_STATE, "no stored Hamiltonian of the whole space");
    const int64_t N = (int64_t)c.H.N, nnz = c.H.nnz;
    int64_t b = 0;
    if (mode == SHCI_MODE_MIXED && k == 1 && c.H.cvalid)  // 16-bit deltas + FP32 values, row bases
      b = c.H.cnnz * 6 + 8 * (N + 1) + 4 * N + 8 * N + 4 * N + 8 * N;
    else if (mode == SHCI_MODE_MIXED)
      b = nnz * 8 + 8 * (N + 1) + 8 * N + (int64_t)k * N * (4 + 8);
    else if (mode == SHCI_MODE_FP64 && c.H.v64.p)
      b = nnz * 12 + 8 * (N + 1) + 8 * N + (int64_t)k * N * (8 + 8);
    else if (mode == SHCI_MODE_FP64)  // float-float on head + tail: split x, FP64 x for the diagonal
      b = nnz * 12 + 8 * (N + 1) + 8 * N + (int64_t)k * N * (8 + 8 + 8);
    else
      throw Error(SHCI_ERR_INVALID, "stored sigma modes only");
    // the storage-order permutation read by the sigma kernel, and the gather
    // of x into storage order (permutation, x read and written)
    b += 8 * N + 2 * (int64_t)k * N * (mode == SHCI_MODE_MIXED ? 4 : 8);
    *bytes = b;
  });
}

int shci_davidson(shci_ctx* ctx, int mode, int block, int nroots, double* x0, int max_copies, double tol, double* E,
                  int* iters) {
  return guarded(ctx, [&](Context& c) {
    if (!x0 || !E) throw Error(SHCI_ERR_INVALID, "null argument");
    const size_t N = c.ndet;
    shci::DevBuf<double> x;
    x.resize(N * nroots);
    SHCI_CUDA(cudaMemcpyAsync(x.p, x0, N * nroots * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    std::vector<double> ev;
    int it = 0;
    const double E_est = E[0];  // energy estimate for the shifted preconditioners (NaN: none)
    c.davidson(mode, block != 0, nroots, x.p, max_copies, tol, false, ev, it, E_est);
    SHCI_CUDA(cudaMemcpyAsync(x0, x.p, N * nroots * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SHCI_CUDA(cudaStreamSynchronize(c.stream));
    for (int r = 0; r < nroots; ++r) E[r] = ev[r];
    if (iters) *iters = it;
  });
}

int shci_run_input(shci_ctx* ctx, const char* input_path, const char* fcidump, int mode, int block, double* E,
                   int cap_roots, int* nroots) {
  return guarded(ctx, [&](Context& c) {
    if (!input_path) throw Error(SHCI_ERR_INVALID, "null input path");
    shci::Schedule s;
    shci::read_input(input_path, s);
    std::string dir = input_path;
    size_t slash = dir.find_last_of('/');
    dir = slash == std::string::npos ? std::string(".") : dir.substr(0, slash);
    s.baseDir = dir;
    std::string fd = fcidump ? std::string(fcidump)
                             : (s.integralFile.size() && s.integralFile[0] == '/' ? s.integralFile
                                                                                   : dir + "/" + s.integralFile);
    c.load_fcidump(fd);
    if (mode < 0) mode = s.mode >= 0 ? s.mode : SHCI_MODE_FP64;
    if (block < 0) block = s.block ? 1 : 0;
    if (s.precond >= 0) c.precond = s.precond;
    if (s.basis_max > 0) {
      c.basis_max = s.basis_max;
      c.basis_keep = s.basis_keep;
    }
    std::vector<double> ev;
    c.run(s, mode, block != 0, ev);
    for (int r = 0; s.writeBest > 0 && r < (int)ev.size(); ++r)
      c.write_best_dets(c.ci.p + (size_t)r * c.ndet, s.writeBest,
                        dir + (r == 0 ? std::string("/dets.bin") : "/dets_" + std::to_string(r) + ".bin"));
    if (nroots) *nroots = (int)ev.size();
    for (int r = 0; r < (int)ev.size() && r < cap_roots; ++r) E[r] = ev[r];
  });
}

int shci_pt_deterministic(shci_ctx* ctx, const double* ci, double E0, double eps2, double* e2) {
  return guarded(ctx, [&](Context& c) {
    if (!ci || !e2) throw Error(SHCI_ERR_INVALID, "null argument");
    c.require_dets();
    c.ptc.resize(c.ndet);
    SHCI_CUDA(cudaMemcpyAsync(c.ptc.p, ci, c.ndet * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    *e2 = c.perturb(c.ptc.p, E0, eps2);
  });
}

int shci_run_pt(shci_ctx* ctx, double eps2, double* E, int cap_roots, int* nroots) {
  return guarded(ctx, [&](Context& c) {
    if (c.Evar.empty() || c.nroots_run != (int)c.Evar.size())
      throw Error(SHCI_ERR_STATE, "no variational run to perturb (call shci_run_input first)");
    if (!(eps2 > 0.0)) eps2 = c.run_eps2;
    const shci::Schedule& s = c.run_sched;
    // the reference's choice of PT (SHCI/SHCI.cpp:707-760)
    if (s.stochastic && s.sampleN == -1)
      throw Error(SHCI_ERR_INVALID, "semistochastic PT needs sampleN (or `deterministic`)");
    if (s.stochastic && s.sampleN < 2) throw Error(SHCI_ERR_INVALID, "sampleN must be at least 2");
    if (nroots) *nroots = (int)c.Evar.size();
    for (int r = 0; r < (int)c.Evar.size(); ++r) {
      const double* cr = c.ci.p + (size_t)r * c.ndet;
      double e2 = 0.0;
      if (!s.stochastic)
        e2 = c.perturb(cr, c.Evar[r], eps2);
      else if (s.nPTiter != 0)
        e2 = c.perturb_stoch(cr, c.Evar[r], eps2, s.epsilon2Large, s.sampleN, s.nPTiter, s.targetError,
                             s.seed >= 0 ? (uint64_t)s.seed + (uint64_t)r : (uint64_t)0x5eedu + (uint64_t)r);
      if (E && r < cap_roots) E[r] = c.Evar[r] + e2;
    }
  });
}

int shci_pt_semistochastic(shci_ctx* ctx, const double* ci, double E0, double eps2, double eps2_large, int sample_n,
                           int max_iter, double target_error, uint64_t seed, double* e2, double* stddev,
                           int* iterations) {
  return guarded(ctx, [&](Context& c) {
    if (!ci || !e2) throw Error(SHCI_ERR_INVALID, "null argument");
    c.require_dets();
    c.ptc.resize(c.ndet);
    SHCI_CUDA(cudaMemcpyAsync(c.ptc.p, ci, c.ndet * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    *e2 = c.perturb_stoch(c.ptc.p, E0, eps2, eps2_large, sample_n, max_iter, target_error, seed);
    if (stddev) *stddev = c.pts_last.stddev;
    if (iterations) *iterations = c.pts_last.iterations;
  });
}

int shci_pt_error(shci_ctx* ctx, double* stddev, int* iterations, double* e_large) {
  return guarded(ctx, [&](Context& c) {
    if (stddev) *stddev = c.pts_last.stddev;
    if (iterations) *iterations = c.pts_last.iterations;
    if (e_large) *e_large = c.pts_last.e_large;
  });
}

int shci_write_best_dets(shci_ctx* ctx, int root, int num, const char* path) {
  return guarded(ctx, [&](Context& c) {
    if (!path) throw Error(SHCI_ERR_INVALID, "null path");
    if (c.Evar.empty() || c.nroots_run != (int)c.Evar.size())
      throw Error(SHCI_ERR_STATE, "no variational run (call shci_run_input first)");
    if (root < 0 || root >= c.nroots_run) throw Error(SHCI_ERR_INVALID, "root out of range");
    c.write_best_dets(c.ci.p + (size_t)root * c.ndet, num, path);
  });
}

int shci_ints_info(shci_ctx* ctx, int* norb, int* nelec, double* coreE) {
  return guarded(ctx, [&](Context& c) {
    c.require_ints();
    if (norb) *norb = c.hints.norb;
    if (nelec) *nelec = c.hints.nelec;
    if (coreE) *coreE = c.hints.coreE;
  });
}

int shci_rdm(shci_ctx* ctx, const double* ci, double* s2, double* s1) {
  return guarded(ctx, [&](Context& c) {
    if (!ci) throw Error(SHCI_ERR_INVALID, "null coefficients");
    c.require_dets();
    c.ptc.resize(c.ndet);
    SHCI_CUDA(cudaMemcpyAsync(c.ptc.p, ci, c.ndet * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    c.rdm(c.ptc.p, s2, s1);
  });
}

int shci_run_rdm(shci_ctx* ctx, int root, double* s2, double* s1) {
  return guarded(ctx, [&](Context& c) {
    if (c.Evar.empty() || c.nroots_run != (int)c.Evar.size())
      throw Error(SHCI_ERR_STATE, "no variational run (call shci_run_input first)");
    if (root < 0 || root >= c.nroots_run) throw Error(SHCI_ERR_INVALID, "root out of range");
    c.rdm(c.ci.p + (size_t)root * c.ndet, s2, s1);
  });
}

int shci_pt_stats(shci_ctx* ctx, int64_t* candidates, int64_t* unique, int* partitions, double* psi1_norm,
                  double* seconds) {
  return guarded(ctx, [&](Context& c) {
    if (candidates) *candidates = c.pt_last.candidates;
    if (unique) *unique = c.pt_last.unique;
    if (partitions) *partitions = c.pt_last.partitions;
    if (psi1_norm) *psi1_norm = c.pt_last.psi1_norm;
    if (seconds) *seconds = c.t_pt;
  });
}

int shci_set_pt_batch(shci_ctx* ctx, int64_t max_candidates) {
  return guarded(ctx, [&](Context& c) {
    if (max_candidates < 0) throw Error(SHCI_ERR_INVALID, "max_candidates must be >= 0");
    c.pt_max_cand = max_candidates;
  });
}

int shci_run_log(shci_ctx* ctx, int cap, int* niter, int64_t* ndets, double* energy, int* dav_iters,
                 double* seconds) {
  return guarded(ctx, [&](Context& c) {
    if (niter) *niter = (int)c.log.size();
    for (int i = 0; i < (int)c.log.size() && i < cap; ++i) {
      if (ndets) ndets[i] = c.log[i].ndets;
      if (energy) energy[i] = c.log[i].energy;
      if (dav_iters) dav_iters[i] = c.log[i].dav_iters;
      if (seconds) seconds[i] = c.log[i].seconds;
    }
  });
}

int shci_run_ci(shci_ctx* ctx, double* out, int64_t cap) {
  return guarded(ctx, [&](Context& c) {
    const size_t n = c.ndet * (size_t)c.nroots_run;
    if (cap < (int64_t)n) throw Error(SHCI_ERR_INVALID, "output buffer too small");
    SHCI_CUDA(cudaMemcpyAsync(out, c.ci.p, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SHCI_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int shci_run_timings(shci_ctx* ctx, double* t_select, double* t_ham, double* t_davidson, double* t_total,
                     int64_t* n_sigma, double* t_sigma) {
  return guarded(ctx, [&](Context& c) {
    if (t_select) *t_select = c.t_select;
    if (t_ham) *t_ham = c.t_ham;
    if (t_davidson) *t_davidson = c.t_dav;
    if (t_total) *t_total = c.t_total;
    if (n_sigma) *n_sigma = c.n_sigma;
    if (t_sigma) *t_sigma = c.t_sigma;
  });
}

int shci_set_preconditioner(shci_ctx* ctx, int mode) {
  return guarded(ctx, [&](Context& c) {
    if (mode < 0 || mode > 2) throw Error(SHCI_ERR_INVALID, "preconditioner must be 0 (diagonal), 1 (PT2) or 2 (MLP)");
    c.precond = mode;
    c.shift_ready = false;
  });
}

int shci_set_davidson_basis(shci_ctx* ctx, int max_basis, int keep) {
  return guarded(ctx, [&](Context& c) {
    if (max_basis == 0 && keep == 0) {
      c.basis_max = c.basis_keep = 0;
      return;
    }
    if (max_basis < 3 || max_basis > 16) throw Error(SHCI_ERR_INVALID, "max_basis must be 0 or in 3..16");
    if (keep < 1 || keep >= max_basis) throw Error(SHCI_ERR_INVALID, "keep must be in 1..max_basis-1");
    c.basis_max = max_basis;
    c.basis_keep = keep;
  });
}

int shci_set_davidson_graphs(shci_ctx* ctx, int on) {
  return guarded(ctx, [&](Context& c) {
    c.graphs_clear();
    c.use_graphs = on != 0;
  });
}

int shci_pt2_shift(shci_ctx* ctx, double E, double* out) {
  return guarded(ctx, [&](Context& c) {
    if (!c.whole_ham()) throw Error(SHCI_ERR_STATE, "no stored Hamiltonian of the whole space");
    c.ensure_diag();
    c.teacher.resize(c.ndet);
    shci::pt2_shift(c.H, c.diag.p, E, c.teacher.p, c.pt2inv, c.stream);
    SHCI_CUDA(cudaMemcpyAsync(out, c.teacher.p, c.ndet * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SHCI_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int shci_mlp_configure(shci_ctx* ctx, int steps, int batch, float lr, int64_t sample_rows) {
  return guarded(ctx, [&](Context& c) {
    if (steps < 0 || batch < 1 || !(lr > 0.f) || sample_rows < 1) throw Error(SHCI_ERR_INVALID, "bad MLP settings");
    c.mlp_steps = steps;
    c.mlp_batch = batch;
    c.mlp_lr = lr;
    c.mlp_sample = sample_rows;
  });
}

int shci_mlp_train(shci_ctx* ctx, double E, float* loss) {
  return guarded(ctx, [&](Context& c) {
    const double l = c.train_mlp(E);
    if (loss) *loss = (float)l;
  });
}

int shci_mlp_predict(shci_ctx* ctx, double E, double* out) {
  return guarded(ctx, [&](Context& c) {
    if (!c.mlp.trained && c.mlp.nparam == 0) throw Error(SHCI_ERR_STATE, "MLP not trained or loaded");
    c.ensure_diag();
    c.shift.resize(c.ndet);
    c.mlp.infer(c.dets.p, c.diag.p, c.ndet, E, c.shift.p, c.stream);
    SHCI_CUDA(cudaMemcpyAsync(out, c.shift.p, c.ndet * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SHCI_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int shci_mlp_params(shci_ctx* ctx, float* out, int cap, int* n, double* sigma) {
  return guarded(ctx, [&](Context& c) {
    c.require_ints();
    if (c.mlp.nspin != 2 * c.hints.norb) c.mlp.init(2 * c.hints.norb, 7, c.stream);
    if (n) *n = c.mlp.nparam;
    if (sigma) *sigma = c.mlp.sigma;
    if (out) {
      if (cap < c.mlp.nparam) throw Error(SHCI_ERR_INVALID, "output buffer too small");
      auto h = c.mlp.get_params(c.stream);
      std::memcpy(out, h.data(), h.size() * sizeof(float));
    }
  });
}

int shci_mlp_set_params(shci_ctx* ctx, const float* in, int n, double sigma) {
  return guarded(ctx, [&](Context& c) {
    c.require_ints();
    if (c.mlp.nspin != 2 * c.hints.norb) c.mlp.init(2 * c.hints.norb, 7, c.stream);
    c.mlp.set_params(std::vector<float>(in, in + n), c.stream);
    c.mlp.sigma = sigma;
    c.mlp.trained = true;
  });
}

int shci_mlp_gradient(shci_ctx* ctx, const int32_t* rows, const float* target, int B, double E, float* grad,
                      float* loss) {
  return guarded(ctx, [&](Context& c) {
    c.require_dets();
    c.ensure_diag();
    if (c.mlp.nspin != 2 * c.hints.norb) c.mlp.init(2 * c.hints.norb, 7, c.stream);
    for (int i = 0; i < B; ++i)
      if (rows[i] < 0 || (size_t)rows[i] >= c.ndet) throw Error(SHCI_ERR_INVALID, "row index out of range");
    c.tr_idx.resize(B);
    c.tr_tgt.resize(B);
    SHCI_CUDA(cudaMemcpyAsync(c.tr_idx.p, rows, B * sizeof(int32_t), cudaMemcpyHostToDevice, c.stream));
    SHCI_CUDA(cudaMemcpyAsync(c.tr_tgt.p, target, B * sizeof(float), cudaMemcpyHostToDevice, c.stream));
    const float l = c.mlp.gradient(c.dets.p, c.diag.p, c.tr_idx.p, c.tr_tgt.p, B, E, c.stream);
    if (loss) *loss = l;
    if (grad)
      SHCI_CUDA(cudaMemcpyAsync(grad, c.mlp.grad.p, c.mlp.nparam * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    SHCI_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int shci_run_stats(shci_ctx* ctx, int64_t* davidson_iters, double* t_mlp, float* mlp_loss) {
  return guarded(ctx, [&](Context& c) {
    if (davidson_iters) *davidson_iters = c.total_dav_iters;
    if (t_mlp) *t_mlp = c.t_mlp;
    if (mlp_loss) *mlp_loss = (float)c.last_loss;
  });
}

int shci_launch_count(shci_ctx* ctx, int64_t* n) {
  return guarded(ctx, [&](Context&) { *n = shci::g_launch_count.load(); });
}

}  // extern "C"
