/*
 * libshci_gpu: C-ABI of the GB300 engine for the variational stage of
 * semistochastic heat-bath CI (the drop-in for Dice's SHCI variational loop).
 *
 * Conventions
 *   - Every entry point returns an int status (SHCI_OK = 0). On failure the
 *     message is available from shci_last_error(ctx). The reference has no
 *     error codes: it calls exit(0)/abort() (SHCI/integral.cpp:71-74,
 *     SHCI/Davidson.cpp:262-266, :305-308, SHCI/input.cpp:373-375).
 *   - Determinants are two uint64 words each (up to 64 spatial orbitals):
 *     spin-orbital p is bit p%64 of word p/64, alpha orbital k = spin-orbital
 *     2k, beta orbital k = 2k+1 (Dice's Determinant, SHCI/Determinants.h:247-602).
 *   - Vectors on the host are column-major: vector c of length N starts at
 *     x + c*N (Eigen MatrixXx columns in the reference).
 *   - Energies exclude the core energy unless stated (the reference zeroes
 *     coreE during the variational loop, SHCI/SHCIbasics.cpp:815-818).
 *   - A context owns one CUDA stream and all device buffers; calls on one
 *     context must not overlap (not thread-safe per context).
 */
#ifndef SHCI_GPU_H
#define SHCI_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct shci_ctx shci_ctx;

enum {
  SHCI_OK = 0,
  SHCI_ERR_INVALID = 1, /* bad argument or input file */
  SHCI_ERR_IO = 2,      /* file missing or unreadable */
  SHCI_ERR_CUDA = 3,    /* CUDA runtime error */
  SHCI_ERR_OOM = 4,     /* device allocation failed or exceeded the cap */
  SHCI_ERR_NOCONV = 5,  /* Davidson did not converge */
  SHCI_ERR_TIMEOUT = 6, /* a bounded device wait gave up */
  SHCI_ERR_STATE = 7    /* call out of order (e.g. sigma before ham_build) */
};

/* Sigma / Hamiltonian storage modes. */
enum {
  SHCI_MODE_FP64 = 0,   /* plain path: FP64 CSR values, FP64 sigma */
  SHCI_MODE_MIXED = 1,  /* FP32 CSR head + FP32 tail, FP32 sigma, FP64 refinement */
  SHCI_MODE_DIRECT = 2,       /* matrix-free: H_ij recomputed in every sigma (HmultDirect), FP64 */
  SHCI_MODE_DIRECT_MIXED = 3  /* matrix-free, FP32 elements and accumulation, then FP64 refinement */
};

/* Context. */
int shci_ctx_create(int device, shci_ctx** out);
int shci_ctx_destroy(shci_ctx* ctx);
const char* shci_last_error(shci_ctx* ctx);
/* The context's cudaStream_t, for callers that time or order work on it. */
void* shci_ctx_stream(shci_ctx* ctx);
/* Cap on the context's device allocations in bytes (0 = no cap). */
int shci_set_alloc_cap(shci_ctx* ctx, uint64_t bytes);

/* Integrals. Replaces readIntegrals (SHCI/integral.cpp:43-225) and the
 * heat-bath construction twoIntHeatBath::constructClass +
 * twoIntHeatBathSHM::constructClass (SHCI/integral.h:125-153,
 * SHCI/integral.cpp:228-389). Builds the heat-bath tables as well. */
int shci_read_fcidump(shci_ctx* ctx, const char* path, int* norb, int* nelec, double* coreE);
/* Header values of the integrals the context holds (after shci_read_fcidump
 * or shci_run_input); any pointer may be NULL. */
int shci_ints_info(shci_ctx* ctx, int* norb, int* nelec, double* coreE);

/* Host-only parsers (no context, no device): the same readers the context
 * calls, for drivers that validate their inputs before touching a GPU. On
 * failure the message is in shci_last_error(NULL).
 * shci_fcidump_info: readIntegrals' header and body checks
 * (SHCI/integral.cpp:43-225); *nnz_i2 receives the number of distinct
 * nonzero two-electron integrals (up to the 8-fold permutational symmetry). */
int shci_fcidump_info(const char* path, int* norb, int* nelec, double* coreE, int64_t* nnz_i2);
/* shci_input_info: readInput for the variational keys (SHCI/input.cpp:35-404).
 * eps1[cap_eps] receives the expanded eps1 schedule (one entry per variational
 * iteration), *n_eps its length; tols[3] = davidsonTol, davidsonTolLoose, dE;
 * ints[8] = nroots, ndet (nocc lines), ncore, nact, precision (-1 unset,
 * 0 fp64, 1 mixed), blockdavidson, precond (-1 unset, 0 plain, 1 pt2, 2 mlp),
 * davidsonBasis max (0 = the reference's subspace). Any pointer may be NULL. */
int shci_input_info(const char* path, double* eps1, int cap_eps, int* n_eps, double* tols, int* ints);
/* Heat-bath table sizes and contents (for parity checks). which: 1 = same
 * spin, 0 = opposite spin. Arrays may be NULL. starts has n(n+1)/2+1 entries,
 * pairs 2 per entry, singles (2n)^2. */
int shci_heatbath_export(shci_ctx* ctx, int which, int64_t* count, float* vals, int16_t* pairs, int64_t* starts,
                         double* singles);

/* Selection parameters (schedule fields ncore, nact, restrict/restrictv;
 * SHCI/input.h:35-194, SHCI/OccRestrictions.h:37-78). Each restriction is
 * (min, max, 64-bit mask of spatial orbitals). At most 4 restrictions. */
int shci_set_selection_params(shci_ctx* ctx, int ncore, int nact, int nrestrict, const int* rmin, const int* rmax,
                              const uint64_t* spatial_masks);

/* Determinant space. set replaces the space; get copies it out in index
 * order (new determinants are appended in sorted order, as the reference
 * does at SHCI/SHCIbasics.cpp:1059-1077). */
int shci_dets_set(shci_ctx* ctx, const uint64_t* dets, int64_t n);
int shci_dets_count(shci_ctx* ctx, int64_t* n);
int shci_dets_get(shci_ctx* ctx, uint64_t* out, int64_t cap);

/* Heat-bath selection. Replaces the parent loop over
 * SHCIgetdeterminants::getDeterminantsVariationalApprox
 * (SHCI/SHCIgetdeterminants.cpp:586-739, called at SHCI/SHCIbasics.cpp:969-982)
 * plus sort/unique and the append at SHCI/SHCIbasics.cpp:992-1077.
 * cmax: host array of |c| per current determinant (cMax,
 * SHCI/SHCIbasics.cpp:954-965). The new determinants are appended to the
 * space; *n_new returns how many. */
int shci_select(shci_ctx* ctx, const double* cmax, double eps1, int64_t* n_new);

/* Sharded selection, one rank's part. Replaces the rank's share of the parent
 * loop at SHCI/SHCIbasics.cpp:969-982 (parents i with i % world == rank)
 * followed by the rank-local sort/unique at :992-994; the reference then
 * merges the ranks' lists up a binary tree (:1002-1050), which the host
 * driver (dice_gb300/shard.py) replaces by a hash-partitioned exchange.
 * shci_select_candidates: the new determinants this rank's parents generate
 *   (absent from the space, sorted in the reference's order, unique), kept in
 *   the context; the space is not changed. *n_new = their count.
 * shci_candidates_get: copies them out (cap >= *n_new, 2 words each).
 * shci_dets_append: appends determinants to the space in the given order; they
 *   must be strictly increasing in the reference's order (Determinant::operator<,
 *   SHCI/Determinants.h:490-498), carry NELEC electrons and be absent from the
 *   space (SHCI_ERR_INVALID otherwise), as the reference appends the merged
 *   new determinants at SHCI/SHCIbasics.cpp:1059-1077. */
int shci_select_candidates(shci_ctx* ctx, const double* cmax, double eps1, int rank, int world, int64_t* n_new);
int shci_candidates_get(shci_ctx* ctx, uint64_t* out, int64_t cap);
int shci_dets_append(shci_ctx* ctx, const uint64_t* dets, int64_t n);

/* Hamiltonian. Replaces HamHelpers2::PopulateHelpers/MakeSHMHelpers and
 * SparseHam::makeFromHelper (SHCI/SHCImakeHamiltonian.cpp:290-408, :959-1147,
 * :486-715). mode: SHCI_MODE_*; MIXED also keeps the FP32 tail for FP64
 * refinement, DIRECT and DIRECT_MIXED build only the string tables.
 * *nnz = off-diagonal nonzeros, both triangles. */
int shci_ham_build(shci_ctx* ctx, int mode, int64_t* nnz);
/* One rank's row block of the stored Hamiltonian in the sharded path: the full
 * rows (every column) of the determinants [r0, r1), mode SHCI_MODE_FP64 or
 * SHCI_MODE_MIXED; *nnz = their off-diagonal entries. Replaces the rank's
 * share of SparseHam::makeFromHelper (SHCI/SHCImakeHamiltonian.cpp:486-715,
 * rows I % nprocs == rank there, a contiguous block here). A row's entries
 * and their order are those of the same row in the whole matrix.
 * shci_sigma / shci_sigma_device then write only the rows [r0, r1) of y and
 * leave the others untouched; x spans the whole space. shci_davidson,
 * shci_ham_export, the packed and allocation-free sigmas and the shifted
 * preconditioners need the whole matrix and return SHCI_ERR_STATE until
 * shci_ham_build is called again. */
int shci_ham_build_rows(shci_ctx* ctx, int mode, int64_t r0, int64_t r1, int64_t* nnz);
/* The stored off-diagonal CSR (full rows) in FP64; rowptr N+1, col/val nnz.
 * For MIXED, val = head + tail. */
int shci_ham_export(shci_ctx* ctx, int64_t* rowptr, int32_t* col, double* val);

/* Diagonal energies Determinant::Energy (SHCI/Determinants.cpp:252-300),
 * coreE excluded, into host out[N] (may be NULL to only compute them). */
int shci_diag(shci_ctx* ctx, double* out);

/* Sigma y = H x for k vectors (1 <= k <= 4), host buffers (column-major N x k).
 * Replaces Hmult2::operator() / HmultDirect::operator() (SHCI/Hmult.h:52,
 * :241). The reference's Hmult2 writes y (zero-initialised) and HmultDirect
 * accumulates into y; this call always overwrites y.
 * mode SHCI_MODE_MIXED computes in FP32; SHCI_MODE_FP64 in FP64 (FP64 values,
 * or head+tail when the matrix was built MIXED, then in float-float
 * arithmetic); SHCI_MODE_DIRECT matrix-free in FP64; SHCI_MODE_DIRECT_MIXED
 * matrix-free with FP32 elements and compensated FP32 accumulation. */
int shci_sigma(shci_ctx* ctx, int mode, const double* x, double* y, int k);
/* Same on device buffers of this context's device (column-major, leading
 * dimension ld), enqueued on the context stream without host synchronisation. */
int shci_sigma_device(shci_ctx* ctx, int mode, const double* x_dev, double* y_dev, int k, int64_t ld);

/* Sigma on vectors already in the engine's gather layout: x_packed is
 * row-interleaved N x kp (kp = 1, 2 or 4; k <= kp columns used), FP32 for
 * SHCI_MODE_MIXED and FP64 for SHCI_MODE_FP64, rows in the determinant order
 * of shci_dets_get; y_dev column-major (ld), same order. Two kernel launches
 * on the context stream, no synchronisation: the rows of x_packed gathered
 * into the stored matrix's storage order (sorted by alpha, then beta string;
 * a context buffer, allocated on first use), then the sigma kernel.
 * SHCI_MODE_FP64 needs a Hamiltonian built in FP64 mode (SHCI_ERR_STATE
 * otherwise: a mixed build's FP64 refinement sigma is shci_sigma_device).
 * Replaces the inner product loop of Hmult2::operator() (SHCI/Hmult.h:108-123). */
int shci_sigma_packed_device(shci_ctx* ctx, int mode, const void* x_packed, int kp, int k, double* y_dev,
                             int64_t ld);
/* Allocation-free variant of shci_sigma_device. It has no counterpart in the
 * reference. It is for callers that cannot allocate device memory while they
 * run: for example a host program whose own memory pool owns all of the GPU's
 * memory, or a time-critical loop that must not trigger the implicit device
 * synchronisation that cudaMalloc/cudaFree can cause. The context must have
 * been set up beforehand (shci_ham_build, which does allocate); this call
 * itself calls no cudaMalloc, cudaFree or allocating library routine.
 * The row-interleaved copy of x goes to one fixed 16 MiB device array
 * compiled into the library instead of a context buffer, which limits N x k
 * (k = 3 counts as 4) to 4,194,304 for SHCI_MODE_MIXED and 2,097,152 for
 * SHCI_MODE_FP64; larger sizes return SHCI_ERR_INVALID. The array is held by
 * every GPU that loads the library until the process exits. Its device
 * address is looked up (cudaGetSymbolAddress) by shci_ham_build on the
 * context's device, so this call does no set-up of its own; after a
 * cudaDeviceReset every context is gone and a new one must be built. All
 * calls share the array: calls that overlap on the GPU (other streams or
 * contexts at the same time) race on it. Null vectors return
 * SHCI_ERR_INVALID. Enqueued on the context stream, no host synchronisation.
 * SHCI_MODE_DIRECT is not supported. */
int shci_sigma_device_noalloc(shci_ctx* ctx, int mode, const double* x_dev, double* y_dev, int k, int64_t ld);
/* Bytes of the stored Hamiltonian (row pointers, columns, values) and of the
 * string tables, for memory and roofline accounting. */
int shci_ham_bytes(shci_ctx* ctx, int64_t* csr_bytes, int64_t* helper_bytes);
/* Algorithmic bytes one stored-matrix sigma call of k vectors
 * (shci_sigma_packed_device) streams in the given mode for the current layout
 * (matrix entries, row pointers, diagonal, x read once, y written once, the
 * storage-order permutation, and the gather of x into storage order): the
 * numerator of its roofline. No counterpart in the reference. */
int shci_sigma_bytes(shci_ctx* ctx, int mode, int k, int64_t* bytes);

/* Davidson. Replaces davidson / davidsonDirect (SHCI/Davidson.cpp:111-348,
 * :353-590) with the diagonal preconditioner (:85-106).
 * x0: host nroots x N column-major, initial guesses in, eigenvectors out.
 * mode: SHCI_MODE_FP64 (plain), SHCI_MODE_MIXED (FP32 sigma, then FP64
 * refinement of the Ritz pairs), SHCI_MODE_DIRECT, SHCI_MODE_DIRECT_MIXED
 * (FP32 matrix-free sigma, then FP64 matrix-free refinement).
 * block: 0 = one correction vector per iteration for the lowest unconverged
 * root (the reference's scheme), 1 = one per unconverged root in a single
 * k-vector sigma launch. max_copies: subspace size (reference: nroots+4).
 * E[nroots] receives eigenvalues (coreE excluded); *iters the iteration count.
 * On entry E[0] is an energy estimate used by the shifted preconditioners
 * (shci_set_preconditioner 1 or 2); NaN means none (diagonal preconditioner). */
int shci_davidson(shci_ctx* ctx, int mode, int block, int nroots, double* x0, int max_copies, double tol, double* E,
                  int* iters);

/* Whole variational stage from a Dice input file (replaces
 * SHCIbasics::DoVariational, SHCI/SHCIbasics.cpp:783-1378, driven as in
 * SHCI/SHCI.cpp:157-446). Reads input.dat and its FCIDUMP (relative paths
 * resolve against the input file's directory unless fcidump is given).
 * E[cap_roots] receives E_var per root with coreE added; *nroots the count.
 * Checkpoints as the reference keeps them (writeVariationalResult /
 * readVariationalResult, SHCI/SHCIbasics.cpp:871-943, 1224-1226, 1346-1352,
 * 1481-1590): with `io` (the default) the iteration, determinants,
 * coefficients and E0 are written after every iteration to
 * <prefix>/shci_gpu-variational.chk (this library's own binary layout; a
 * relative prefix resolves against the input file's directory); `restart`
 * resumes after the saved iteration, or returns the saved result when that
 * iteration already used the final eps1; `fullrestart` reruns the schedule
 * from the saved space. A missing or foreign checkpoint is SHCI_ERR_IO.
 * Treversal t = +-1 (time-reversal symmetry, SHCI/input.cpp:253-258;
 * ignored for an odd electron count as SHCI/SHCI.cpp:188-195 does; needs as
 * many alpha as beta electrons): the reference keeps the standard member of
 * every alpha <-> beta flipped pair and works in the basis
 * (D + t p(D) flip(D))/sqrt(2) (SHCI/Determinants.cpp:32-121,
 * SHCI/SHCImakeHamiltonian.cpp:411-483); here the space holds both members of
 * every pair (the form the reference unpacks to, SHCI/SHCIbasics.cpp:730-781),
 * selection runs from the standard member with the pair's coefficient
 * (SHCI/SHCIbasics.cpp:984-997) and every Davidson vector is kept in the
 * sector c(flip(D)) = t p(D) c(D): the same eigenvalues. The space, the
 * coefficients and the per-iteration determinant counts then count both
 * members of every pair. */
int shci_run_input(shci_ctx* ctx, const char* input_path, const char* fcidump, int mode, int block, double* E,
                   int cap_roots, int* nroots);
/* Per-iteration log of the last run: ndets, E (root 0, coreE added),
 * Davidson iterations and seconds since the start of the run. */
int shci_run_log(shci_ctx* ctx, int cap, int* niter, int64_t* ndets, double* energy, int* dav_iters, double* seconds);
/* Coefficient vectors of the last run's final space, host out (nroots x N). */
int shci_run_ci(shci_ctx* ctx, double* out, int64_t cap);

/* Deterministic second-order (Epstein-Nesbet) perturbation theory.
 * Replaces SHCIbasics::DoPerturbativeDeterministic (SHCI/SHCIbasics.cpp:453-728,
 * without its RDM branch) and its generator
 * SHCIgetdeterminants::getDeterminantsDeterministicPT
 * (SHCI/SHCIgetdeterminants.cpp:40-171), as selected by `deterministic` in
 * the input (SHCI/SHCI.cpp:707-721).
 * shci_pt_deterministic: E2 for the context's current space with coefficients
 *   ci (host, one per determinant, in the order of shci_dets_get), E0 the
 *   variational energy WITH coreE (as the reference passes it), threshold
 *   eps2 (>= 0). The caller adds E0 to get the PT energy. The selection
 *   restrictions of shci_set_selection_params apply; ncore/nact do not.
 * shci_run_pt: after shci_run_input, E[r] = E_var[r] + E2[r] for every root
 *   (what the reference writes to shci.e), eps2 <= 0 taking the input's
 *   epsilon2 (default 1e-8, SHCI/input.cpp:58). As the reference chooses
 *   (SHCI/SHCI.cpp:707-760): `deterministic` in the input gives the
 *   deterministic PT; otherwise the semistochastic PT with the input's
 *   sampleN, nPTiter (0: no PT, E = E_var), targetError, epsilon2Large and
 *   seed (+ root; without `seed` a fixed default instead of the clock), and an
 *   input without sampleN is an error, as in the reference.
 * shci_pt_stats: of the last PT call: candidates generated outside the
 *   variational space before merging, distinct determinants, hash partitions
 *   used, first-order norm sum_a (N_a / (E0 - E_a))^2, seconds.
 * shci_set_pt_batch: cap on the candidates held on the device at once
 *   (0 = from free memory). Larger candidate sets are split into hash
 *   partitions, as the reference splits them over MPI ranks; E2 agrees to
 *   rounding across partition counts. */
int shci_pt_deterministic(shci_ctx* ctx, const double* ci, double E0, double eps2, double* e2);
/* Semistochastic PT2. Replaces
 * SHCIbasics::DoPerturbativeStochastic2SingleListDoubleEpsilon2AllTogether
 * (SHCI/SHCIbasics.cpp:55-451) with its sampler
 * SHCIsampledeterminants::setUpAliasMethod / sample_N2_alias
 * (SHCI/SHCIsampledeterminants.cpp:64-190) and generator
 * getDeterminantsStochastic2Epsilon (SHCI/SHCIgetdeterminants.cpp:889-1045):
 * the deterministic part at eps2_large (skipped when >= 999, the reference's
 * default 1000), then iterations of sample_n alias draws with probability
 * |c_i| / sum |c| until the standard error of the mean (from the fifth
 * iteration on) is below target_error or max_iter iterations ran. *e2 = the
 * mean estimate (the caller adds E0), *stddev its standard error,
 * *iterations the count. The draws come from a 64-bit Mersenne twister seeded
 * with `seed` (the reference uses rand() seeded from the clock), so results
 * are reproducible for a given seed; the estimator is the reference's. */
int shci_pt_semistochastic(shci_ctx* ctx, const double* ci, double E0, double eps2, double eps2_large, int sample_n,
                           int max_iter, double target_error, uint64_t seed, double* e2, double* stddev,
                           int* iterations);
/* Error of the last semistochastic PT (zeros after a deterministic one):
 * standard error, iterations, deterministic part at eps2_large. */
int shci_pt_error(shci_ctx* ctx, double* stddev, int* iterations, double* e_large);
int shci_run_pt(shci_ctx* ctx, double eps2, double* E, int cap_roots, int* nroots);
int shci_pt_stats(shci_ctx* ctx, int64_t* candidates, int64_t* unique, int* partitions, double* psi1_norm,
                  double* seconds);
int shci_set_pt_batch(shci_ctx* ctx, int64_t max_candidates);

/* Spatial reduced density matrices of the variational wavefunction.
 * Replace SHCIrdm::EvaluateRDM (SHCI/SHCIrdm.cpp:863-993) and
 * SHCIrdm::EvaluateOneRDM (:996-1100) as DoVariational calls them for
 * DoRDM / DoOneRDM (SHCI/SHCIbasics.cpp:1236-1341), bra = ket.
 * shci_rdm: ci = host coefficients of the current space (order of
 *   shci_dets_get); s2 (NORB^4 doubles, may be NULL) receives s2RDM with
 *   element (p NORB + q, r NORB + s) at (p NORB + q) NORB^2 + r NORB + s, the
 *   reference's spatialRDM.i.i.txt values; s1 (NORB^2, may be NULL) the
 *   spatial 1-RDM, row-major (spatial1RDM.i.i.txt). The connection lists of
 *   the stored Hamiltonian are used (built in the mixed form when the
 *   current one is matrix-free or missing). Sums are kept in 64-bit fixed
 *   point (2^-58) with integer atomics: bitwise reproducible.
 * shci_run_rdm: the same for root `root` of the last shci_run_input. */
int shci_rdm(shci_ctx* ctx, const double* ci, double* s2, double* s1);
int shci_run_rdm(shci_ctx* ctx, int root, double* s2, double* s1);

/* writeBestDeterminants (SHCI/SHCI.cpp:465-506) for root `root` of the last
 * shci_run_input: the file the reference names dets.bin (dets_<root>.bin for
 * root > 0), for QMC codes: int num, int NORB, then for each of the num
 * largest |c| the coefficient times getParityForDiceToAlphaBeta
 * (SHCI/Determinants.cpp:691-706) as a double and NORB characters '0', 'a',
 * 'b', '2'. Ties in |c| keep index order. shci_run_input writes these files
 * into the input file's directory when the input sets writebestdeterminants. */
int shci_write_best_dets(shci_ctx* ctx, int root, int num, const char* path);

/* Stage timings of the last run in seconds: selection, Hamiltonian build,
 * Davidson, total; and the sigma calls/time spent inside Davidson. */
int shci_run_timings(shci_ctx* ctx, double* t_select, double* t_ham, double* t_davidson, double* t_total,
                     int64_t* n_sigma, double* t_sigma);

/* Davidson preconditioner (replaces precondition, SHCI/Davidson.cpp:85-106):
 * 0 = the reference's r_i / (theta - H_ii) (default);
 * 1 = denominator shifted by the second-order level shift
 *     s_i = sum_j H_ij^2 / (E - H_jj) of the stored Hamiltonian;
 * 2 = shift predicted by the learned MLP (no counterpart in the reference):
 *     in shci_run_input the network is trained after every loose Davidson
 *     solve on the (residual, correction) pairs that solve generated -- at
 *     iterations 2, 4, 8 and 16 the Ritz vector x_k and residual r_k of the
 *     lowest root; once converged to x_s, e = x_s / (x_s . x_k) - x_k is the
 *     correction that iteration needed, and s_i = -r_i/e_i - (H_ii - theta_k)
 *     the shift that would have produced it from r_i -- and used from the next
 *     solve on, in the stored and the matrix-free paths alike. The plain
 *     denominator is kept wherever a shift would flip its sign or shrink it
 *     below a fifth, and convergence is still judged on the unpreconditioned
 *     residual, so eigenvalues do not change. */
int shci_set_preconditioner(shci_ctx* ctx, int mode);
/* Davidson subspace size (no counterpart in the reference, whose subspace is
 * nroots+4 vectors collapsed to nroots+2 Ritz vectors, SHCI/SHCIbasics.cpp:1171,
 * SHCI/Davidson.cpp:325-345): at most max_basis (3..16) vectors, collapsed to
 * the keep lowest Ritz vectors. Used by shci_run_input for every solve;
 * (0, 0) restores the reference's rule. A larger subspace keeps more of the
 * Krylov space across restarts and needs fewer iterations to the same
 * tolerance; it changes no converged eigenvalue. */
int shci_set_davidson_basis(shci_ctx* ctx, int max_basis, int keep);
/* Davidson iterations as captured CUDA graphs (1, the default) or as the
 * same kernels launched one by one (0); results are identical. No
 * counterpart in the reference. */
int shci_set_davidson_graphs(shci_ctx* ctx, int on);
/* Second-order level shifts of the current space at energy E (host out[N]). */
int shci_pt2_shift(shci_ctx* ctx, double E, double* out);
/* MLP training settings: Adam steps per training call, minibatch, learning
 * rate, rows sampled from the space. */
int shci_mlp_configure(shci_ctx* ctx, int steps, int batch, float lr, int64_t sample_rows);
/* Train on the current space's second-order level shifts at energy E (a
 * regression target for tests and experiments; shci_run_input trains on
 * Davidson's own pairs instead); final minibatch loss. */
int shci_mlp_train(shci_ctx* ctx, double E, float* loss);
/* Predicted shifts for every determinant of the current space (host out[N]). */
int shci_mlp_predict(shci_ctx* ctx, double E, double* out);
/* FP32 master parameters (W1 128xF row-major, W2 128x128, b1, b2, w3, b3;
 * F = 2 NORB + 2) and the target scale; out may be NULL to query *n. */
int shci_mlp_params(shci_ctx* ctx, float* out, int cap, int* n, double* sigma);
int shci_mlp_set_params(shci_ctx* ctx, const float* in, int n, double sigma);
/* Mean squared error and its gradient (FP32, same layout as the parameters)
 * for the given rows of the current space and scaled targets. */
int shci_mlp_gradient(shci_ctx* ctx, const int32_t* rows, const float* target, int B, double E, float* grad,
                      float* loss);
/* Totals of the last shci_run_input: Davidson iterations, seconds spent
 * training the MLP, last training loss. */
int shci_run_stats(shci_ctx* ctx, int64_t* davidson_iters, double* t_mlp, float* mlp_loss);

/* Kernel launches issued by this context since creation (own kernels only). */
int shci_launch_count(shci_ctx* ctx, int64_t* n);

#ifdef __cplusplus
}
#endif
#endif
