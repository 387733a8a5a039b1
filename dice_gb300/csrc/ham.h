// Device data structures of the determinant space and the Hamiltonian.
#pragma once
#include "engine.h"

namespace shci {

// Plain-pointer view passed to kernels.
struct HelperView {
  size_t N;
  const uint64_t* astr;  // alpha string of each determinant
  const uint64_t* bstr;  // beta string of each determinant
  const uint32_t* aidx;  // determinant -> alpha group
  const uint32_t* bidx;  // determinant -> beta group
  const int64_t* aStart;  // alpha group g spans [aStart[g], aStart[g+1])
  const uint32_t* aDets;  // determinant indices grouped by alpha string (AlphaMajorToDet)
  const uint64_t* aGroupB;  // beta string of aDets[p] (AlphaMajorToBeta)
  const int64_t* bStart;
  const uint32_t* bDets;    // BetaMajorToDet
  const uint64_t* bGroupA;  // BetaMajorToAlpha
  const int64_t* aSingStart;  // SinglesFromAlpha as CSR over alpha groups
  const uint32_t* aSing;
  // the list of alpha group g holds its small groups (a few times n_beta
  // determinants at most) in [aSingStart[g], aSingMid[g]), then the large ones
  const int64_t* aSingMid;
  // partial-string index: one 16-byte entry per (determinant J, occupied
  // beta orbital b of J): {beta string of J without b (low, high word),
  // alpha group of J | b << 26, J}, sorted by (alpha group, partial string),
  // so that the entries of one key (alpha group, partial string) are a run
  const uint4* m1ent;
  // per alpha group g, an open-addressing table over the group's distinct
  // partial strings: m1dir[g] = first slot << 6 | log2(slots); a slot is
  // {first entry of the key's run, (run length - 1) << 26 | 26-bit
  // fingerprint of the partial string}, all bits set in an empty slot's first
  // word; every table is at most half full
  const uint2* m1tab;
  const uint64_t* m1dir;
};

// Alpha/beta string tables of one determinant space
// (HamHelpers2, SHCI/SHCImakeHamiltonian.h:44-82).
struct Helpers {
  size_t N = 0;
  int64_t NA = 0, NB = 0, nsing = 0;
  DevBuf<uint64_t> astr, bstr, ua, ub, aGroupB, bGroupA;
  DevBuf<uint32_t> aidx, bidx, aDets, bDets, aSing;
  DevBuf<int64_t> aStart, bStart, aSingStart, aSingMid;
  DevBuf<uint4> m1ent;
  DevBuf<uint2> m1tab;
  DevBuf<uint64_t> m1dir;
  int64_t nm1 = 0;
  void build(const Det2* dets, size_t n, int norb, Prims& pr, cudaStream_t s);
  HelperView view() const {
    return HelperView{N,         astr.p,      bstr.p,  aidx.p,  bidx.p,  aStart.p, aDets.p,
                      aGroupB.p, bStart.p,    bDets.p, bGroupA.p, aSingStart.p, aSing.p, aSingMid.p,
                      nm1 > 0 ? m1ent.p : nullptr, m1tab.p, m1dir.p};
  }
  size_t bytes() const {
    return astr.bytes() + bstr.bytes() + ua.bytes() + ub.bytes() + aGroupB.bytes() + bGroupA.bytes() +
           aidx.bytes() + bidx.bytes() + aDets.bytes() + bDets.bytes() + aSing.bytes() + aStart.bytes() +
           bStart.bytes() + aSingStart.bytes() + aSingMid.bytes() + m1ent.bytes() + m1tab.bytes() + m1dir.bytes();
  }
};

// Off-diagonal Hamiltonian as full-row CSR (both triangles); the diagonal is
// kept separately in FP64. Values are FP64 (v64) for the plain path, or an
// FP32 head (vhi) plus an FP32 tail (vlo = h - (double)vhi) for the mixed path,
// so that vhi + vlo reproduces the FP64 element to about 2^-48 relative.
//
// Rows and columns are in storage order: the determinants sorted by (alpha
// string, beta string). perm[i] is the index in the determinant array of the
// determinant at storage position i, spos its inverse. Consecutive rows are
// then determinants of one alpha string, whose connections largely coincide,
// and a row's same-alpha connections form one contiguous range of columns, so
// the x gathers of sigma fall on fewer 32-byte sectors and hit in L1 more
// often than in the selection order. Vectors outside the matrix (Davidson,
// the C-ABI) stay in the determinant array's order: the sigma kernels read
// the diagonal and write y through perm, and x is packed through perm.
struct Csr {
  size_t N = 0;
  int64_t nnz = 0;
  DevBuf<int64_t> rowptr;
  DevBuf<int32_t> col;
  DevBuf<double> v64;
  DevBuf<float> vhi, vlo;
  DevBuf<uint32_t> perm, spos;
  // Copy for the single-vector FP32 sigma with 16-bit column deltas: row r's
  // entries are [crow[r], crow[r+1]); the column of an entry is cbase[r] plus
  // the deltas of the row up to and including it (the first delta is 0).
  // Gaps of 65536 or more are bridged by zero-valued entries of delta 65535.
  // 6 bytes per entry instead of 8.
  DevBuf<int64_t> crow;
  DevBuf<int32_t> cbase;
  DevBuf<uint16_t> cdel;
  DevBuf<float> cval;
  int64_t cnnz = 0;
  bool cvalid = false;
  // Row block (build_ham_block): N local rows, the full rows of the
  // determinants [row0, row0 + N) of a space of nfull; perm[r] = determinant
  // of local row r, xpos[r] = its storage position, xperm = the whole storage
  // order through which x is packed. Columns are storage positions of the
  // whole space.
  bool block = false;
  size_t nfull = 0, row0 = 0;
  DevBuf<uint32_t> xpos, xperm;
  // storage position -> determinant over the whole space (what x is packed by)
  const uint32_t* pack_perm() const { return block ? xperm.p : perm.p; }
  // number of determinants x and y span
  size_t ncols() const { return block ? nfull : N; }
  void clear_block() {
    block = false;
    nfull = row0 = 0;
    xpos.release();
    xperm.release();
  }
  size_t bytes() const {
    return rowptr.bytes() + col.bytes() + v64.bytes() + vhi.bytes() + vlo.bytes() + perm.bytes() + spos.bytes() +
           crow.bytes() + cbase.bytes() + cdel.bytes() + cval.bytes() + xpos.bytes() + xperm.bytes();
  }
  void drop_compressed() {
    crow.release();
    cbase.release();
    cdel.release();
    cval.release();
    cnnz = 0;
    cvalid = false;
  }
};
// Builds the 16-bit-delta copy of a column-sorted FP32 (head) matrix.
void compress_csr(Csr& H, Prims& pr, cudaStream_t s);

// Builds H for the space described by hp, in storage order. When H already
// holds the first n_old determinants (same value arrays), only the rows of the
// determinants >= n_old and the new columns of the old rows are computed; the
// old rows are relabelled to the new storage order (a monotone map, so they
// stay sorted) and merged with their new columns. Otherwise all rows.
void build_ham_csr(const Helpers& hp, const Det2* dets, const IntsView& ints, Csr& H, bool want64, bool want32,
                   bool want_lo, size_t n_old, Prims& pr, cudaStream_t s);
// Builds only the full rows of the determinants [r0, r1) (see Csr::block).
void build_ham_block(const Helpers& hp, const Det2* dets, const IntsView& ints, Csr& H, bool want64, bool want32,
                     bool want_lo, size_t r0, size_t r1, Prims& pr, cudaStream_t s);
void compute_diag(const Det2* dets, size_t n, const IntsView& ints, double* diag, cudaStream_t s);
void sigma_direct(const Helpers& hp, const Det2* dets, const IntsView& ints, const double* diag, const double* x,
                  double* y, int k, cudaStream_t s);
// FP32 matrix-free sigma: x row-interleaved FP32 [N][k], y FP64 [N][k].
void sigma_direct32(const Helpers& hp, const Det2* dets, const IntsView& ints, const double* diag, const float* x,
                    double* y, int k, cudaStream_t s);

// ---- selection (kernels_select.cu) -----------------------------------------
struct HeatBathView {
  const float* sameVal;
  const int16_t* samePairs;
  const int64_t* sameStart;
  const float* oppVal;
  const int16_t* oppPairs;
  const int64_t* oppStart;
  const double* singles;  // (2n)x(2n)
};

constexpr int kMaxRestrict = 4;
struct SelectParams {
  int ncore = 0;
  int nact = 1000000;
  int nrestrict = 0;
  int rmin[kMaxRestrict];
  int rmax[kMaxRestrict];
  uint64_t rmask0[kMaxRestrict];  // spin-orbital masks, bits 0..63
  uint64_t rmask1[kMaxRestrict];  // bits 64..127
};

// Membership test in a DetHash (slots index into `dets`; linear probing).
__device__ __forceinline__ bool hash_contains(const uint32_t* __restrict__ slots, uint64_t mask,
                                              const Det2* __restrict__ dets, const Det2& x) {
  uint64_t h = det_hash(x) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    uint32_t s = slots[h];
    if (s == 0xffffffffu) return false;
    Det2 y = dets[s];
    if (det_eq(x, y)) return true;
    h = (h + 1) & mask;
  }
  return false;
}

// Whether spin orbital p belongs to restriction r.
__device__ __forceinline__ int in_mask(const SelectParams& sp, int r, int p) {
  return p < 64 ? (int)((sp.rmask0[r] >> p) & 1ull) : (int)((sp.rmask1[r] >> (p - 64)) & 1ull);
}

// Candidates from every parent, dropping those already present (hash set);
// returns the number of candidates written (may exceed cap: then nothing past
// cap is written and the caller retries with a larger buffer).
int64_t select_candidates(const Det2* dets, const double* cmax, size_t n, double eps1, const IntsView& ints,
                          const HeatBathView& hb, double maxEntry, const SelectParams& sp, const DetHash& present,
                          Det2* out, int64_t cap, int64_t* d_counter, cudaStream_t s);
// Time reversal (kernels_select.cu): cMax of the reference's symmetrized
// basis for every determinant (0 for the non-standard member of a pair), and
// the new determinants of a selection: the standard members of the
// candidates' pairs, sorted, unique and absent from the space, followed by
// the flipped partners of the open-shell ones, written to out (room for 2n);
// returns how many.
void trev_cmax(const Det2* dets, const double* ci, size_t ld, int nroots, size_t n, const int32_t* flip, double* out,
               cudaStream_t s);
size_t trev_new_dets(Det2* cand, size_t n, const DetHash& present, const Det2* dets, Det2* out, DevBuf<int64_t>& flag,
                     DevBuf<int64_t>& pos, Prims& pr, cudaStream_t s);
// Number of the n determinants q that the hash set `present` (over dets) holds.
int64_t count_present(const Det2* q, size_t n, const DetHash& present, const Det2* dets, int64_t* d_counter,
                      cudaStream_t s);

// ---- alpha <-> beta flip of the space (kernels_select.cu) -------------------
// flip[i] = index of the determinant with alpha and beta strings exchanged,
// sign[i] = (-1)^(number of doubly occupied orbitals of det i), the phase of
// the relabelling in the interleaved spin-orbital order. Returns false (and
// leaves the map unusable) when some flipped determinant is not in the space.
bool build_flip_map(const Det2* dets, size_t n, const DetHash& hash, int32_t* flip, int8_t* sign,
                    int64_t* d_missing, cudaStream_t s);
// parity p = <x|F|x> / <x|x> of one column (host result)
double flip_parity(const double* x, size_t n, const int32_t* flip, const int8_t* sign, DevBuf<double>& part,
                   cudaStream_t s);
// x <- (x + p F x) / 2 in place (p = +1 or -1), using tmp (n doubles)
void flip_project(double* x, size_t n, const int32_t* flip, const int8_t* sign, double p, double* tmp,
                  cudaStream_t s);

// ---- deterministic second-order perturbation theory (kernels_pt.cu) --------
struct PtResult {
  double e2 = 0.0;         // sum_a N_a^2 / (E0 - E_a)
  double psi1_norm = 0.0;  // sum_a (N_a / (E0 - E_a))^2
  int64_t candidates = 0;  // generated outside the variational space (before merging)
  int64_t unique = 0;      // distinct determinants a
  int partitions = 0;
};
struct PtWork {
  DevBuf<uint64_t> key0, key1;  // candidate determinants, word by word
  DevBuf<float4> ne;  // numerator and E_a - E0 of each candidate (float pairs)
  DevBuf<double2> n2p;  // semistochastic mode: both numerators in FP64
  DevBuf<double> part;
  DevBuf<uint32_t> perm;
  DevBuf<unsigned long long> next;  // parent queue, candidate counter
  DevBuf<double> coul, exch;        // dense (AI|JJ), (AJ|JI) of the integrals below
  DevBuf<float> coul32, exch32;     // and their FP32 roundings
  DevBuf<float2> coulff, exchff;    // and as float pairs
  const double* tables_of = nullptr;
  int tables_n = 0;
};
// E2 of the space `dets` (hash set `present` over it) with coefficients c
// (device, n) for threshold eps2: candidates with |H_ai c_i| criteria of the
// reference, numerators merged per determinant. E0 without the core energy.
// sp supplies the occupation restrictions (its ncore/nact are not applied).
// max_candidates > 0 caps one partition (default: from free device memory).
PtResult pt_deterministic(const Det2* dets, size_t n, const double* c, double E0, double eps2, const IntsView& ints,
                          const HeatBathView& hb, double maxEntry, const SelectParams& sp, const DetHash& present,
                          int64_t max_candidates, PtWork& w, Prims& pr, cudaStream_t s);

// ---- reduced density matrices (kernels_rdm.cu) ------------------------------
// Spatial 2-RDM (out[0, n^4): element (p n + q, r n + s) at (p n + q) n^2 + r n + s)
// and spatial 1-RDM (out[n^4, n^4 + n^2)) of the wavefunction c over the
// connection lists of the stored Hamiltonian H of the space `dets`.
void rdm_evaluate(const Det2* dets, const double* c, size_t N, const Csr& H, int n, DevBuf<unsigned long long>& fix,
                  DevBuf<double>& out, cudaStream_t s);

struct PtStochResult {
  double e2 = 0.0;       // mean of the iteration estimates
  double stddev = 0.0;   // standard error of the mean (1e4 before the fifth iteration)
  double e_large = 0.0;  // deterministic part at eps2L (0 when eps2L >= 999)
  int iterations = 0;
  int64_t candidates = 0;  // over all iterations
};
// Semistochastic PT2 (SHCIbasics::DoPerturbativeStochastic2SingleListDoubleEpsilon2AllTogether,
// SHCI/SHCIbasics.cpp:55-451): c on the device and on the host (the alias
// table and the draws are made on the host), E0 without the core energy.
PtStochResult pt_semistochastic(const Det2* dets, size_t n, const double* c_dev, const std::vector<double>& c_host,
                                double E0, double eps2, double eps2L, int nsample, int max_iter, double target,
                                uint64_t seed, const IntsView& ints, const HeatBathView& hb, double maxEntry,
                                const SelectParams& sp, const DetHash& present, PtWork& w, Prims& pr,
                                cudaStream_t s);

// ---- sigma and Davidson vector kernels (kernels_sigma.cu) -------------------
// Y[:, c] (column-major, leading dimension ldy) = diag .* X[:, c] + Hoff X[:, c]
// for c < k, where X is row-interleaved [N][kp] in the path's precision and in
// H's storage order (packed through H.perm); y and diag are in the
// determinant array's order.
void sigma_csr_mixed(const Csr& H, const double* diag, const float* x32, int kp, int k, double* y, size_t ldy,
                     cudaStream_t s);
void sigma_csr_f64(const Csr& H, const double* diag, const double* x64, int kp, int k, double* y, size_t ldy,
                   cudaStream_t s);
// Refinement sigma on the FP32 head + tail values in float-float arithmetic:
// xff is x split as (head, tail) float pairs, row-interleaved [N][kp]; the
// diagonal term is taken in FP64 from column-major xd (columns c0..c0+k-1).
void sigma_csr_ff(const Csr& H, const double* diag, const float* xff, int kp, const double* xd, size_t ldx, int c0,
                  int k, double* y, size_t ldy, cudaStream_t s);
// Sigma that allocates nothing: x (column-major, ldx) is packed into a fixed
// device array of kNoAllocPackBytes (16 MiB: N x k up to 4,194,304 in the
// mixed path, 2,097,152 in the FP64 path; k = 3 counts as 4) and the stored
// Hamiltonian's sigma kernel runs on it. Larger sizes are rejected.
constexpr size_t kNoAllocPackBytes = (size_t)16 << 20;
// scratch: the array's device address on the context's device, from
// noalloc_scratch_address() (looked up while the Hamiltonian is built).
void sigma_noalloc(const Csr& H, const double* diag, int mode_mixed, const double* x, size_t ldx, int k, double* y,
                   size_t ldy, void* scratch, cudaStream_t s);
void* noalloc_scratch_address();
// Pack columns [c0, c0+k) of column-major A (lda) into row-interleaved [N][kp]
// (zero padded) in FP32 or FP64; with perm (storage order of the stored
// Hamiltonian), packed row i holds row perm[i] of A.
void pack_f32(const double* A, size_t lda, int c0, int k, int kp, size_t N, float* out, cudaStream_t s,
              const uint32_t* perm = nullptr);
void pack_f64(const double* A, size_t lda, int c0, int k, int kp, size_t N, double* out, cudaStream_t s,
              const uint32_t* perm = nullptr);
// Columns split into (head, tail) float pairs, row-interleaved [N][kp] float2.
void pack_ff(const double* A, size_t lda, int c0, int k, int kp, size_t N, float* out, cudaStream_t s,
             const uint32_t* perm = nullptr);
// out row i = in row perm[i] of a row-interleaved array of `bytes_per_row`
// (4, 8, 16 or 32) bytes per row.
void gather_rows(const void* in, size_t bytes_per_row, const uint32_t* perm, size_t N, void* out, cudaStream_t s);
void unpack_f64(const double* in, int kp, int k, size_t N, double* A, size_t lda, int c0, cudaStream_t s);
// Tall-skinny products over column-major N x m blocks (deterministic order):
// G (ma x mb, column-major) = A^T B.
void ts_gram(const double* A, size_t lda, int ma, const double* B, size_t ldb, int mb, size_t N, double* G,
             DevBuf<double>& part, cudaStream_t s);
// Y = alpha * A Q + beta * Y, Q (m x k column-major, device).
void ts_gemm(const double* A, size_t lda, int m, const double* Q, int k, size_t N, double alpha, double beta,
             double* Y, size_t ldy, cudaStream_t s);
// c <- c / sqrt(g[0]) when sqrt(g[0]) > 1e-14 (g: device squared norm)
void scale_inv_norm(double* c, size_t N, const double* g, cudaStream_t s);
// R[:, c] = Y[:, c] - lam[c] X[:, c]
void residual(const double* X, const double* Y, const double* lam, int k, size_t N, size_t ld, double* R,
              cudaStream_t s);
// R[:, c] /= (lam[c] - diag) with the reference's 1e-12 guard
void precondition(const double* diag, const double* lam, int k, size_t N, double* R, size_t ld, cudaStream_t s);
// R[:, c] /= (lam[c] - diag - shift) where that is safe, else the plain denominator
void precondition_shift(const double* diag, const double* shift, const double* lam, int k, size_t N, double* R,
                        size_t ld, cudaStream_t s);
// A[:, c] *= scale[c]
void scale_cols(double* A, size_t ld, const double* scale, int k, size_t N, cudaStream_t s);

}  // namespace shci
