/*
 * tnx -- C ABI of the GB300 (sm_103a) DMRG / tSDRG numerical core.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (as void*), returns a tnx_status code, and never throws. Buffers are owned
 * by the caller; workspace is passed in explicitly and its size is given by
 * the matching *_workspace_bytes query. The library allocates no device memory
 * on any of these paths. tnx_last_error() returns a thread-local message for the
 * last failing call on the calling thread.
 *
 * Tensor layouts (row-major, FP64 unless stated):
 *   MPS site tensor  A[chi_l][d][chi_r]            ('lpr', tnpy/matrix_product_state.py:45)
 *   MPO site tensor  W[dl][dr][d][d]  (l, r, ket, bra; boundary tensors carry a 1-sized dl / dr)
 *   environments     L[chi_l][dl][chi_l], R[chi_r][dr][chi_r]  (ket, mpo, bra; 1x1x1 ones on
 *                    the open ends)
 */
#ifndef TNX_H_
#define TNX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum tnx_status {
  TNX_OK = 0,
  TNX_ERR_INVALID_ARG = 1,   /* null pointer, non-positive size, bad enum   (reference: ValueError) */
  TNX_ERR_SHAPE = 2,         /* inconsistent or unsupported dimensions      (reference: ValueError) */
  TNX_ERR_WORKSPACE = 3,     /* workspace smaller than *_workspace_bytes    */
  TNX_ERR_NOT_CONVERGED = 4, /* iteration limit reached (result still written) */
  TNX_ERR_CUDA = 5,          /* a CUDA launch or copy failed                */
  TNX_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up          */
  TNX_ERR_UNSUPPORTED = 7    /* precision / size not built into this library */
};

enum tnx_precision {
  TNX_FP64 = 0,       /* plain FP64 contractions (FP64 pipe)                                */
  TNX_BF16X3 = 1,     /* mixed form: split-BF16 three-term matvec products on tcgen05 with FP32
                         accumulation for the Davidson iterations; environment updates, gauge
                         moves and the Davidson's anchor matvec FP64-class as in TNX_DF64     */
  TNX_DF64 = 2        /* FP64-class contractions: Ozaki-sliced FP64 GEMMs on tcgen05 where large
                         (~2^-52 per product relative to row/column maxima), double-FP32 on the
                         FP32 pipe otherwise (~2^-48 per product); double-FP32 QR panels       */
};

const char* tnx_status_string(int status);
const char* tnx_last_error(void);
int tnx_version(void);
/* 1 when the loaded library was built for sm_103a and a device of compute capability
 * 10.3 is current; 0 otherwise. */
int tnx_device_ok(void);

/* Number of kernels the library has launched in this process (all entry points). */
long long tnx_launch_count(void);
/* Time every launch of one kernel family with CUDA events on its stream until
 * tnx_profile_end, which synchronises and returns the launch count, the summed device
 * time and the summed algorithmic flops / bytes of those launches.
 * Families: 0 tcgen05 split-BF16 GEMM, 1 FP64 / double-FP32 SIMT GEMM, 2 Davidson vector
 * kernels, 3 QR panel, 4 dense eigensolver, 5 other, 6 Ozaki FP64-class GEMM (large products),
 * 7 Ozaki FP64-class GEMM (narrow products: a side of 128 or less, split K, batches). */
int tnx_profile_begin(int family);
int tnx_profile_end(int* launches, double* total_ms, double* flops, double* bytes);

/* ---- autotuner ---------------------------------------------------------------------------
 * Kernel variants are chosen per call site and shape by timing every candidate once on the
 * caller's stream (first call of that shape, outside stream capture, output-overwriting calls
 * only) and caching the fastest for the process: the double-FP32 GEMM tile (64 x 128 / 32 x 32),
 * the FP64-class GEMM engine (tcgen05 Ozaki / double-FP32 SIMT) and the split-BF16 tcgen05 GEMM
 * tile (128 x 256 / 128 x 128). On by default; TNX_AUTOTUNE=0 in the environment or
 * tnx_autotune_set(0) keeps the fixed size rules. tnx_autotune_report writes one line per cached
 * choice, "kind key0..key4 -> variant ms_0 .. ms_(n-1)" (kind 1 / 2 / 3 as listed; -1 ms for a
 * candidate that did not apply), and returns the bytes needed including the terminating zero.
 * A builder addition: the reference has no native kernels to tune. */
int tnx_autotune_set(int enable);
int tnx_autotune_clear(void);
int tnx_autotune_count(void);
size_t tnx_autotune_report(char* buf, size_t len);

/* ---- one-site effective Hamiltonian ------------------------------------------------
 * Replaces Environment.one_site_matvec (tnpy/matrix_product_state.py:411-440):
 *   y[a',s',c'] = sum L[a,w,a'] x[a,s,c] W[w,v,s,s'] R[c,v,c']
 * with L = 1x1x1 ones on site 0 and R = 1x1x1 ones on site n-1 (:425-430). */
size_t tnx_matvec1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                                   int64_t dr, int precision);
int tnx_matvec1(const double* L, const double* W, const double* R, const double* x, double* y,
                int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr, int precision,
                void* workspace, size_t workspace_bytes, void* stream);

/* FP64 one-site matvec (same contract as tnx_matvec1 with TNX_FP64) that allocates nothing and
 * takes no workspace: for callers that cannot allocate device memory where they call it
 * (inside a stream capture that must not allocate, allocator-less host bindings, processes
 * whose device memory is held by another framework's pool). Its two intermediates live in a
 * file-scope device array of 2 x TNX_NOALLOC_MAX_ELEMS doubles (32 MiB) that every device
 * loading the library keeps until exit. Limit: chi_l * d * chi_r * max(dl, dr) <=
 * TNX_NOALLOC_MAX_ELEMS (e.g. chi_l = chi_r = 448 with D = 5, d = 2); larger problems return
 * TNX_ERR_SHAPE. The first call on a device looks up the array's device address (do it before
 * any stream capture). All calls share the array: calls that overlap on the GPU race.
 * No counterpart in the reference. */
#define TNX_NOALLOC_MAX_ELEMS 2097152
int tnx_matvec1_noalloc(const double* L, const double* W, const double* R, const double* x,
                        double* y, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                        void* stream);

/* Dense effective Hamiltonian H[(a,s,c),(a',s',c')] (tnpy/matrix_product_state.py:372-409),
 * row = ket indices, column = bra indices; H has N = chi_l*d*chi_r rows. */
int tnx_full_matrix1(const double* L, const double* W, const double* R, double* H, int64_t chi_l,
                     int64_t d, int64_t chi_r, int64_t dl, int64_t dr, void* stream);

/* diag(H_eff)[a,s,c] = sum_{w,v} L[a,w,a] W[w,v,s,s] R[c,v,c] (Davidson preconditioner). */
int tnx_diag1(const double* L, const double* W, const double* R, double* diag, int64_t chi_l,
              int64_t d, int64_t chi_r, int64_t dl, int64_t dr, void* stream);

/* ---- environment update -------------------------------------------------------------
 * Replaces Environment.update_left / update_right (tnpy/matrix_product_state.py:296-336).
 * direction = +1: E_in = L_i [chi_l][dl][chi_l] -> E_out = L_{i+1} [chi_r][dr][chi_r]
 * direction = -1: E_in = R_i [chi_r][dr][chi_r] -> E_out = R_{i-1} [chi_l][dl][chi_l] */
size_t tnx_env_update_workspace_bytes(int direction, int64_t chi_l, int64_t d, int64_t chi_r,
                                      int64_t dl, int64_t dr, int precision);
int tnx_env_update(int direction, const double* E_in, const double* A, const double* W,
                   double* E_out, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                   int precision, void* workspace, size_t workspace_bytes, void* stream);

/* ---- lowest eigenpair of H_eff: block Davidson on the device --------------------------
 * Replaces linalg.eigshmv -> primme.eigsh(k=1, which='SA', tol) (tnpy/linalg.py:64-87) as
 * called by FiniteDMRG.one_site_solver (tnpy/finite_dmrg.py:97-111).
 * x: in = start vector (need not be normalised), out = unit Ritz vector.
 * Stops when ||H x - theta x|| <= tol * max(1, |theta|) (primme's residual criterion relative to
 * the operator scale), or after max_iter matvecs (TNX_ERR_NOT_CONVERGED, best Ritz pair still
 * written). precision selects the matvec; Rayleigh-Ritz is FP64. With TNX_BF16X3 a first phase
 * runs split-BF16 matvecs on FP32 vectors to a residual of ~3e-6 |theta|; an anchored phase
 * then continues from the Ritz vector x with one FP64-class product H x per anchor (exact
 * first row of the projected matrix, split-BF16 products for the corrections) until the
 * FP64-class residual is below max(tol, 2e-7) |theta|. */
size_t tnx_davidson1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                                     int64_t dr, int max_basis, int precision);
int tnx_davidson1(const double* L, const double* W, const double* R, double* x, int64_t chi_l,
                  int64_t d, int64_t chi_r, int64_t dl, int64_t dr, double tol, int max_iter,
                  int max_basis, int precision, double* eval_out, double* resid_out,
                  int* iters_out, void* workspace, size_t workspace_bytes, void* stream);
/* tnx_davidson1 with flags. TNX_DAV_START_ANCHORED (mixed precision only): x is expected to be
 * the answer already (the site converged in the previous sweep); the solve starts with the
 * FP64-class anchor product and skips the first split-BF16 phase, which would hand over after
 * its first product. The result and its certification are those of tnx_davidson1. */
#define TNX_DAV_START_ANCHORED 1
int tnx_davidson1_ex(const double* L, const double* W, const double* R, double* x, int64_t chi_l, int64_t d,
                     int64_t chi_r, int64_t dl, int64_t dr, double tol, int max_iter, int max_basis, int precision,
                     int flags, double* eval_out, double* resid_out, int* iters_out, void* workspace,
                     size_t workspace_bytes, void* stream);
/* Generalised problem A x = lambda B x, lowest lambda, for shift-invert DMRG
 * (ShiftInvertDMRG.one_site_solver -> primme.eigsh(A, M=B), tnpy/finite_dmrg.py:345-363): A is
 * the one-site H_eff of (L, W, R), B that of (L2, W2, R2) (environments of the MPO square,
 * bond dl2 / dr2), B positive definite. Davidson with a B-orthonormal basis (two classical
 * B-orthogonalisation passes, one B and one A product per expansion), correction
 * (diag A - lambda diag B)^-1 r; stops when ||A x - lambda B x|| <= tol max(1, |lambda|), or when
 * the residual has stagnated for 40 expansions below 1e-6 max(1, |lambda|) (the Ritz value is
 * then accurate to ~residual^2 / gap). x: in = start vector, out = Ritz vector with x^T B x = 1.
 * *iters_out = expansions. precision: TNX_FP64 native, TNX_DF64 / TNX_BF16X3 FP64-class products. */
size_t tnx_gdavidson1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                      int64_t dl2, int64_t dr2, int max_basis);
int tnx_gdavidson1(const double* L, const double* W, const double* R, const double* L2, const double* W2,
                   const double* R2, double* x, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                   int64_t dl2, int64_t dr2, double tol, int max_iter, int max_basis, int precision,
                   double* eval_out, double* resid_out, int* iters_out, void* workspace, size_t workspace_bytes,
                   void* stream);

/* One MPO tensor applied to one MPS tensor, out[(a,w)][k][(c,v)] = sum_b W[w][v][k][b] A[a][b][c]
 * (out: chi_l*dl x d x chi_r*dr): the site tensors of O|psi>, as ShiftInvertDMRG restores
 * psi = (H - eps) phi (tnpy/finite_dmrg.py:314-343). */
int tnx_mpo_apply_site(const double* A, const double* W, double* out, int64_t chi_l, int64_t d, int64_t chi_r,
                       int64_t dl, int64_t dr, void* stream);

/* Counters of the calling host thread's last tnx_davidson1 call: out[0] matvecs of the first
 * phase, out[1] matvecs of the anchored phase (TNX_BF16X3; 0 otherwise), out[2] FP64-class
 * anchor products, out[3] thick restarts. */
int tnx_davidson1_stats(int* out);

/* ---- dense symmetric eigensolver (batched, one CTA per matrix) ---------------------------
 * Replaces linalg.eigh (tnpy/linalg.py:42-61) and the np.linalg.eigh of
 * TreeTensorNetworkSDRG.block_eigen_solver (tnpy/tsdrg.py:569-592).
 * A: batch matrices, matrix b at A + offsets[b] (doubles), size sizes[b] (<= 1024), row-major,
 * symmetric; destroyed. evals: batch x keep, ascending; evecs: batch x (max_size x keep)
 * column j of matrix b = eigenvector j at evecs + b*max_size*keep, row-major [row][j].
 * A matrix smaller than keep writes only its own eigenpairs; rows >= size are left untouched. */
size_t tnx_eigh_batched_workspace_bytes(int batch, int max_size, int keep);
int tnx_eigh_batched(double* A, const int64_t* offsets, const int* sizes, int batch,
                     int max_size, int keep, double* evals, double* evecs, void* workspace,
                     size_t workspace_bytes, void* stream);
/* The same for matrices of at most 64 rows in double-FP32 arithmetic (FP64-class, ~2^-47):
 * matrix and rotations in shared memory, rotation angles from FP32 leading parts made exactly
 * orthogonal in double-FP32. A faster FP64-class form of the dense block spectra of tSDRG
 * (np.linalg.eigh at tnpy/tsdrg.py:584); no workspace. */
int tnx_eigh_batched_df64(double* A, const int64_t* offsets, const int* sizes, int batch, int max_size, int keep,
                          double* evals, double* evecs, void* stream);

/* ---- QR / SVD gauge move -----------------------------------------------------------------
 * Householder QR of a row-major m x n matrix (m >= n): Q (m x n, orthonormal columns),
 * R (n x n, upper triangular). Replaces linalg.qr (tnpy/linalg.py:26-39). */
size_t tnx_qr_workspace_bytes(int64_t m, int64_t n);
int tnx_qr(const double* M, int64_t m, int64_t n, double* Q, double* R, void* workspace,
           size_t workspace_bytes, void* stream);

/* Thin SVD of a row-major m x n matrix (m >= n) by one-sided Jacobi in FP64: S (n, descending),
 * U (m x n, row-major, may be null), VT (n x n, row-major, may be null; V is accumulated only
 * when VT is given). Replaces np.linalg.svd in linalg.svd (tnpy/linalg.py:9-23) and gives the
 * Schmidt values of the SVD gauge move (tnpy/matrix_product_state.py:200-223). The singular
 * values come from the matrix itself (absolute error ~eps * sigma_max, not the
 * ~sqrt(eps) * sigma_max of a Gram matrix). A column of U whose sigma is exactly zero is left
 * zero. *sweeps_out (may be null) = Jacobi sweeps run; TNX_ERR_NOT_CONVERGED after 40 sweeps
 * (results still written). */
size_t tnx_svd_workspace_bytes(int64_t m, int64_t n, int want_vt);
int tnx_svd(const double* A, int64_t m, int64_t n, double* S, double* U, double* VT, int* sweeps_out,
            void* workspace, size_t workspace_bytes, void* stream);

/* One-site gauge move of FiniteDMRG.sweep (tnpy/matrix_product_state.py:187-225,
 * :359-365), QR form: direction = +1: A_site (chi_l d x chi_r) = Q R, A_site <- Q,
 * A_next <- R A_next (A_next is chi_r x d x chi_r2). direction = -1: A_site^T = Q R,
 * A_site <- Q^T, A_prev <- A_prev R^T (A_prev is chi_l0 x d x chi_l). The neighbour is
 * rewritten in place; chi_other is its far bond. */
size_t tnx_gauge_move_workspace_bytes(int direction, int64_t chi_l, int64_t d, int64_t chi_r,
                                      int64_t chi_other);
int tnx_gauge_move(int direction, double* A_site, double* A_neighbour, int64_t chi_l,
                   int64_t d, int64_t chi_r, int64_t chi_other, int precision, void* workspace,
                   size_t workspace_bytes, void* stream);

/* ---- many chains in lockstep ------------------------------------------------------------
 * Independent chains of one shape (equal bonds, MPO bond and physical dimension) stacked with
 * a fixed stride between chains (sX etc., in doubles); every call spans all `batch` chains.
 * Replaces FiniteDMRG.run (tnpy/finite_dmrg.py:214-257) called once per chain: the one-site
 * matvec (:411-440 of matrix_product_state.py), dense H_eff (:372-409), environment update
 * (:296-336), the eigensolver (linalg.eigshmv, tnpy/linalg.py:64-87) and the gauge move
 * (:187-225), each for all chains at once. precision: TNX_FP64 native FP64 GEMMs, TNX_DF64 or
 * TNX_BF16X3 double-FP32 GEMMs (FP64-class results from the FP32 pipe). */
size_t tnx_batched_matvec1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                           int batch);
int tnx_batched_matvec1(const double* L, int64_t sL, const double* W, int64_t sW, const double* R, int64_t sR,
                        const double* x, int64_t sx, double* y, int64_t sy, int batch, int64_t chi_l, int64_t d,
                        int64_t chi_r, int64_t dl, int64_t dr, int precision, void* workspace,
                        size_t workspace_bytes, void* stream);
/* H[b] (n x n, n = chi_l d chi_r <= 4096) stored at H + b n^2 */
int tnx_batched_full_matrix1(const double* L, int64_t sL, const double* W, int64_t sW, const double* R, int64_t sR,
                             double* H, int batch, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                             void* stream);
size_t tnx_batched_env_update_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                              int batch);
int tnx_batched_env_update(int direction, const double* E_in, int64_t sE, const double* A, int64_t sA,
                           const double* W, int64_t sW, double* E_out, int64_t sO, int batch, int64_t chi_l, int64_t d,
                           int64_t chi_r, int64_t dl, int64_t dr, int precision, void* workspace,
                           size_t workspace_bytes, void* stream);
/* Davidson for every chain in the same launches, with a per-chain convergence mask: chain b
 * retires once ||H x - theta x|| <= tol max(1, |theta|) (or its correction vanishes against its
 * basis) and every vector kernel skips it from then on. X: in = start vectors, out = unit Ritz
 * vectors. evals_out / resid_out (device, batch doubles), active_out (device, batch ints, may
 * be null): 1 for chains still unconverged after max_iter expansions (TNX_ERR_NOT_CONVERGED),
 * *iters_out = expansions run. Once at most batch / 64 chains are still active, those get as many
 * more expansions as the batch had taken by then (at least 32) and stop with their current Ritz
 * pair, reported unconverged. One host read (the active count) every fourth expansion; restarts
 * keep two vectors per chain (the Ritz vector and the previous one, GD+1), and the products of
 * retired chains are skipped. */
size_t tnx_batched_davidson1_workspace_bytes(int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl, int64_t dr,
                                             int batch, int max_basis);
int tnx_batched_davidson1(const double* L, int64_t sL, const double* W, int64_t sW, const double* R, int64_t sR,
                          double* X, int64_t sX, int batch, int64_t chi_l, int64_t d, int64_t chi_r, int64_t dl,
                          int64_t dr, double tol, int max_iter, int max_basis, int precision, double* evals_out,
                          double* resid_out, int* iters_out, int* active_out, void* workspace,
                          size_t workspace_bytes, void* stream);
/* Gauge move of every chain (same contract as tnx_gauge_move): one Householder QR per chain in
 * shared memory (site matrix m x n with m n <= 12800, n <= 128), then the neighbours take R. */
size_t tnx_batched_gauge_move_workspace_bytes(int direction, int64_t chi_l, int64_t d, int64_t chi_r,
                                              int64_t chi_other, int batch);
int tnx_batched_gauge_move(int direction, double* A_site, int64_t sA, double* A_nb, int64_t sN, int batch,
                           int64_t chi_l, int64_t d, int64_t chi_r, int64_t chi_other, int precision, void* workspace,
                           size_t workspace_bytes, void* stream);

/* ---- tSDRG ----------------------------------------------------------------------------
 * Batched two-block Hamiltonians (TreeTensorNetworkSDRG.block_hamiltonian,
 * tnpy/tsdrg.py:607-631): item b multiplies W1_b[0,w] (x) W2_b[w,dr2-1] over the MPO bond w:
 *   H_b[(k1 k2),(b1 b2)] = sum_w W1_b[0,w,k1,b1] W2_b[w,dr2-1,k2,b2]
 * w1[b] -> [dl1][D][m1][m1], w2[b] -> [D][dr2][m2][m2] (device arrays of device pointers),
 * meta[4b..4b+3] = m1, m2, dl1, dr2; H_b is written row-major at h + h_off[b]. */
int tnx_tsdrg_block_hamiltonian(const double* const* w1, const double* const* w2, const int* meta,
                                int D, double* h, const int64_t* h_off, int batch, int max_m,
                                void* stream);
/* Batched spectrum projectors (TreeTensorNetworkSDRG.spectrum_projector, tnpy/tsdrg.py:633-669):
 *   out_b[l,r,i,j] = sum V_b[(k1 k2),i] W1_b[l,w,k1,b1] W2_b[w,r,k2,b2] V_b[(b1 b2),j]
 * v[b] -> [m1*m2][k] (the k kept eigenvectors as columns), out[b] -> [dl1][dr2][k][k],
 * meta[5b..5b+4] = m1, m2, dl1, dr2, k; node dimensions m1, m2, k <= 32. */
int tnx_tsdrg_project(const double* const* w1, const double* const* w2, const double* const* v,
                      const int* meta, int D, double* const* out, int batch, int max_m1,
                      int max_m2, int max_k, void* stream);

/* Lowest-keep eigenpairs of tSDRG block Hamiltonians H = sum_w W1_b[0,w] (x) W2_b[w,dr2-1]
 * (TreeTensorNetworkSDRG.block_eigen_solver, tnpy/tsdrg.py:569-592) without forming H:
 * Chebyshev-filtered subspace iteration on the Kronecker matvec (FP32 for TNX_DF64 /
 * TNX_BF16X3, FP64 for TNX_FP64) followed by an FP64 Rayleigh-Ritz refinement, one CTA per
 * block. meta[5b..5b+4] = m1, m2, dr2, k, p (node dimensions m1, m2 <= 32, k kept pairs,
 * p = subspace size with k <= p <= min(m1 m2, 48)); D <= 6; keep >= every k.
 * evals: batch x keep; evecs: batch x (max_m x keep) row-major, like tnx_eigh_batched;
 * iters (device, may be null): filter iterations per block, or a negative count for a block
 * whose wanted residuals did not reach the tolerance within the iteration limit (its pairs are
 * then approximate; callers re-solve such blocks densely). */
size_t tnx_tsdrg_block_eigh_workspace_bytes(int batch, int max_m, int keep, int precision);
int tnx_tsdrg_block_eigh(const double* const* w1, const double* const* w2, const int* meta, int D,
                         int batch, int max_m, int keep, int precision, double* evals,
                         double* evecs, int* iters, void* workspace, size_t workspace_bytes,
                         void* stream);

/* ---- exact diagonalisation --------------------------------------------------------------
 * Dense Hamiltonian of an MPO (FullHamiltonian, tnpy/operators.py:119-166): W is the MPO packed
 * as [n][D][D][d][d] (the uniform four-index tensors padded with zeros to bond D <= 32: site 0
 * uses row 0, site n-1 column 0); H (d^n x d^n, row-major, d^n <= 65536) gets
 * H[K][B] = e_0^T W_0[:,:,k_0,b_0] ... W_{n-1}[:,:,k_{n-1},b_{n-1}] e_0, with k_0 / b_0 the most
 * significant digits of the ket / bra strings K / B. */
int tnx_full_hamiltonian(const double* W, int n, int D, int d, double* H, void* stream);
/* H += c I with c = max_i sum_j |H_ij| + 1 written to *shift (device double), which makes a
 * symmetric H positive definite; undo = 1 subtracts the c already in *shift. With tnx_svd this
 * gives the full spectrum of ExactDiagonalization (tnpy/exact_diagonalization.py:10-60):
 * eigenvalues = singular values - c, eigenvectors = left singular vectors. */
int tnx_shift_to_spd(double* H, int64_t dim, double* shift, int undo, void* stream);

/* ---- generic helpers used by the host mirror ------------------------------------------ */
/* C[b] = alpha * op(A[b]) op(B[b]) + beta * C[b], row-major, FP64; trans_a / trans_b = 1
 * means A is stored K x M / B is stored N x K. */
int tnx_gemm_f64(int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                 const double* A, int64_t lda, int64_t stride_a, const double* B, int64_t ldb,
                 int64_t stride_b, double beta, double* C, int64_t ldc, int64_t stride_c,
                 int64_t batch, void* stream);

/* C = alpha * op(A) op(B) + beta * C in double-FP32 arithmetic (TNX_DF64), row-major. */
int tnx_gemm_df64(int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                  const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
                  int64_t ldc, void* stream);

/* C = alpha * op(A) op(B) + beta * C, row-major FP64, on the tcgen05 tensor cores by exact
 * integer slicing (Ozaki scheme): rows of op(A) / columns of op(B) scaled by powers of two and
 * cut into eight balanced base-128 digits held exactly in BF16, the 36 slice products with
 * s + t < 8 accumulated exactly in FP32 tensor memory over 480-long K chunks and summed in
 * double-FP32. Error ~2^-52 per product relative to max|row of op(A)| max|column of op(B)|.
 * Returns TNX_ERR_TIMEOUT if a bounded wait in the kernel expired (synchronises the stream). */
size_t tnx_gemm_oz_workspace_bytes(int64_t m, int64_t n, int64_t k);
int tnx_gemm_oz(int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                void* workspace, size_t workspace_bytes, void* stream);
/* The same product for `batch` operand sets at element strides sA, sB, sC (one launch; sets
 * with mask[b] == 0 are skipped, mask may be null) and with K split into `nsplit` ranges whose
 * partial products are added in range order (long-K products with small outputs: the QR's
 * V^T C). Backs the tensor-core form of the lockstep chains' products and the gauge move's
 * trailing updates. */
size_t tnx_gemm_oz_batched_workspace_bytes(int64_t m, int64_t n, int64_t k, int batch, int nsplit);
int tnx_gemm_oz_batched(int trans_a, int trans_b, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                        int64_t lda, int64_t sA, const double* B, int64_t ldb, int64_t sB, double beta, double* C,
                        int64_t ldc, int64_t sC, int batch, int nsplit, const int* mask, void* workspace,
                        size_t workspace_bytes, void* stream);

/* C (m x n, row-major FP64) = A (m x k) B^T (B is n x k), both row-major FP64, computed as
 * three BF16 tensor-core products (split-BF16) with FP32 accumulation. Test / building-block
 * entry point of the tcgen05 GEMM used by the mixed-precision matvec. */
size_t tnx_gemm_bf16x3_workspace_bytes(int64_t m, int64_t n, int64_t k);
int tnx_gemm_bf16x3(int64_t m, int64_t n, int64_t k, const double* A, const double* B, double* C,
                    void* workspace, size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TNX_H_ */
