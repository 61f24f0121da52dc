/*
 * C ABI of the GB300-native two-site DMRG hot path.
 *
 * Tensors are block-sparse with U(1)xU(1) (N, 2Sz) quantum numbers, the data
 * model of the reference's btas::QSDArray<N,fermion> = QSTArray<double,N,fermion>
 * (include/btas/QSPARSE/QSDArray.h:14-19, include/btas/QSPARSE/QSTArray.h:17-328):
 *   - per index: a list of sectors, each with a quantum number (p, 2Sz) and a dim;
 *   - a block with sector index (i_0..i_{N-1}) may be non-zero iff
 *     q_total == sum_k q[k][i_k]  (QSTArray.h:34-36);
 *   - blocks are identified by their row-major sparse tag
 *     (include/btas/SPARSE/STArray.h:338-348) and stored packed in ascending
 *     tag order in one device allocation, each block dense row-major.
 *
 * Every function returns an mpsxx_status; mpsxx_last_error() gives the message
 * of the last failure on the calling thread (the reference throws
 * std::runtime_error with the same texts, include/btas/common/btas.h:19-20).
 * Functions that take a context run on its stream and return after the work
 * has completed unless stated otherwise.
 */
#ifndef MPSXX_GB300_H
#define MPSXX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpsxx_context mpsxx_context;
typedef struct mpsxx_tensor mpsxx_tensor;

enum mpsxx_status {
  MPSXX_OK = 0,
  MPSXX_QSHAPE_MISMATCH = 1,
  MPSXX_ALLOC = 2,
  MPSXX_NO_CONVERGENCE = 3,
  MPSXX_DEVICE_TIMEOUT = 4,
  MPSXX_INVALID_ARGUMENT = 5,
  MPSXX_CUDA = 6,
  MPSXX_SOLVER = 7,
  MPSXX_INTERNAL = 8
};

enum mpsxx_trans { MPSXX_NOTRANS = 0, MPSXX_TRANS = 1 };

/* Library version (major*10000 + minor*100 + patch). */
int mpsxx_version(void);
/* Message of the last failure on this thread ("" if none). */
const char* mpsxx_last_error(void);

/* ---- context: one device, one stream ------------------------------------ */
/* stream may be NULL (the context creates its own non-blocking stream). */
int mpsxx_context_create(int device, void* stream, mpsxx_context** out);
int mpsxx_context_destroy(mpsxx_context* ctx);
int mpsxx_context_sync(mpsxx_context* ctx);
/* Precision of the bulk contractions of this context (no reference counterpart:
 * the reference computes in FP64 only).  MPSXX_FP64: every contraction in FP64.
 * MPSXX_SPLIT_TF32: H_eff*psi runs on the tensor cores with each FP64 operand
 * split into two TF32 numbers (3 products, FP32 accumulation within groups of
 * 1024 products, FP64 across groups); Davidson subspace algebra, the Rayleigh-Ritz
 * solve and residual norms stay FP64.  Every diagonalize call ends with a
 * refinement anchored on one FP64 H_eff*psi: the converged split vector's FP64
 * product fixes all subspace entries that involve it, and the remaining
 * corrections use the split operator (a second anchor only when that continuation
 * does not converge).  The returned value is that refined Ritz value; when the
 * split vector already meets the tolerance it is the FP64 Rayleigh quotient. */
enum mpsxx_precision { MPSXX_FP64 = 0, MPSXX_SPLIT_TF32 = 1, MPSXX_SPLIT_TF32_ALL = 2 };
int mpsxx_context_set_precision(mpsxx_context* ctx, int precision);
int mpsxx_context_get_precision(const mpsxx_context* ctx, int* precision);

/* Truncation tie window of canonicalize: singular values s with
 * s >= cutoff * (1 - tie_rtol) are kept together with the cutoff value (the
 * reference keeps s >= cutoff, include/btas/QSPARSE/QSTLAPACK.h:217-232), so that
 * symmetry-degenerate values that differ by rounding stay together.
 * tie_rtol < 0 restores the default, 1e-10. */
int mpsxx_context_set_truncation(mpsxx_context* ctx, double tie_rtol);

/* Split-precision diagonalize (MPSXX_SPLIT_TF32): the tensor-core Davidson runs until
 * |r|^2 < (residual_floor * E)^2, the resolution of the inexact operator; then up to
 * `rounds` continuations, each anchored by one FP64 H_eff*psi of the current vector,
 * bring |r|^2 under the caller's tolerance (src/diagonalize.hpp:337-437 with the FP64
 * operator).  Negative values restore the defaults, 1e-5 and 2 rounds.  No reference
 * counterpart: the reference has one (FP64) operator. */
int mpsxx_context_set_split_refinement(mpsxx_context* ctx, double residual_floor, int rounds);

/* Kernel launches issued, FP64-equivalent sigma FLOPs and sigma calls so far. */
int mpsxx_context_counters(const mpsxx_context* ctx, int64_t* launches, double* sigma_flops, int64_t* sigma_calls);

/* Phase timers of the bond step, in seconds.  enable = 1 starts accumulating (each
 * phase then ends with a stream synchronisation), 0 stops, -1 leaves the setting;
 * reset = 1 zeroes them after they are read.  Up to n timers are written to t, in
 * the order of MPSXX_PHASE_NAMES; *count receives the number of phases. */
#define MPSXX_PHASE_NAMES                                                                                    \
  "merge_plan", "merge_alloc", "merge_run", "wave_merge", "sigma_plan", "sigma", "davidson_rest", "svd_solve", \
      "svd_select", "svd_post", "renorm_plan", "renorm_run", "sigma_fp64", "batch_group", \
      "batch_plan", "svd_jacobi", "svd_gram"
int mpsxx_context_profile(mpsxx_context* ctx, int enable, int reset, double* t, int n, int* count);

/* The split-precision H_eff*psi plan of a bond is autotuned on first use: candidate
 * schedules (stage-2 split-K sized for a target number of tensor-core tiles; the L*psi
 * intermediate stored as hi|lo TF32 tiles or as FP32 tiles split on chip; for very
 * large intermediates the MPO index w processed in groups that fit a scratch budget)
 * are timed and the fastest is kept with the plan.  The last tuning's (budget bytes,
 * target tiles, FP32 intermediate (0/1), milliseconds) quadruples are written to out
 * (up to n values); *count receives the number of values. */
int mpsxx_context_tuning(const mpsxx_context* ctx, double* out, int n, int* count);
/* Fix the split-precision H_eff*psi schedule instead of autotuning it: the MPO index w
 * processed in groups whose packed L*psi intermediate fits w_budget_bytes (0 = all of
 * w at once), stage-2 split-K sized for target_tiles tensor-core tiles (0 = default),
 * the intermediate as FP32 tiles split on chip (fp32_intermediate = 1) or as hi|lo
 * tiles (0).  w_budget_bytes < 0 restores autotuning.  Cached plans are dropped. */
int mpsxx_context_set_sigma_schedule(mpsxx_context* ctx, int64_t w_budget_bytes, int target_tiles,
                                     int fp32_intermediate);
/* Storage of the merged operators for the split-precision H_eff*psi: pre-split hi|lo
 * TF32 tiles (fp32_operators = 0, the default) or FP32 tiles that the tensor-core
 * kernel splits into hi|lo in shared memory (1: half the packed bytes, for operators
 * that would not fit otherwise; slower, as the on-chip split of both operands costs
 * shared-memory bandwidth).  Either way x = hi + lo to ~2^-22 relative.  Applies to
 * plans made afterwards; cached plans are dropped. */
int mpsxx_context_set_sigma_operator_format(mpsxx_context* ctx, int fp32_operators);
/* Routing of canonicalize's per-block SVDs: blocks with min(m, n) <= jacobi_max_cols
 * (at most 128) go to the batched one-sided Jacobi kernel; of the rest, blocks whose
 * Gram matrix (rows for a forward step, columns backward) has dimension <=
 * gram_max_dim go to the batched symmetric eigensolver (one grouped launch sequence
 * for all of them); the remaining blocks take cuSOLVER gesvd (min(m, n) < 96) or
 * syevd on the Gram matrix, on concurrent solver lanes.  A negative value selects the
 * default (24; 256, for padded sizes shared by at least 6 blocks); 0 switches a route
 * off. */
int mpsxx_context_set_svd_routes(mpsxx_context* ctx, int jacobi_max_cols, int gram_max_dim);
/* Plans (H_eff*psi, diagonal, merged-operator, renormalisation) kept per kind before
 * the context empties a cache (default 512).  Plans are keyed by structural layouts,
 * so a converged sweep reuses the previous sweep's plans when they are still cached;
 * a batched scan of many chains needs room for all of one sweep's bonds. */
int mpsxx_context_set_plan_cache(mpsxx_context* ctx, int64_t max_plans);
/* Wait limit of the tensor-core kernels (one launch; <= 0: the default 20 s).  A kernel
 * that runs out drains its own bulk copies and MMAs, frees its tensor memory and
 * returns; the call reports MPSXX_DEVICE_TIMEOUT and the context stays usable. */
int mpsxx_context_set_device_timeout(mpsxx_context* ctx, int64_t timeout_ns);

/* ---- tensors ------------------------------------------------------------- */
/* Create a block-sparse tensor.  qn holds 2*sum(nsec) ints (p, 2Sz per sector,
 * index by index), dims holds sum(nsec) ints.  nblocks < 0 allocates every
 * allowed block of non-zero size (STArray.h:219-237); otherwise tags lists the
 * stored blocks in ascending order.  ctx == NULL gives a host-only descriptor
 * (no device storage) usable by the planner.  Device storage is zero-filled. */
int mpsxx_tensor_create(mpsxx_context* ctx, int rank, const int* q, const int* nsec, const int* qn, const int* dims,
                        int64_t nblocks, const int64_t* tags, mpsxx_tensor** out);
/* Same shape and block layout as `like`, zero-filled. */
int mpsxx_tensor_create_like(mpsxx_context* ctx, const mpsxx_tensor* like, mpsxx_tensor** out);
int mpsxx_tensor_destroy(mpsxx_tensor* t);
int mpsxx_tensor_info(const mpsxx_tensor* t, int* rank, int* q, int64_t* nblocks, int64_t* nnz);
/* nsec[rank], qn[2*sum nsec], dims[sum nsec] (caller-sized, see mpsxx_tensor_info). */
int mpsxx_tensor_shape(const mpsxx_tensor* t, int* nsec, int* qn, int* dims);
int mpsxx_tensor_blocks(const mpsxx_tensor* t, int64_t* tags, int64_t* offsets);
/* Host <-> device copies of all nnz elements (block-packed order). */
int mpsxx_tensor_upload(mpsxx_tensor* t, const double* host);
int mpsxx_tensor_download(const mpsxx_tensor* t, double* host);
int mpsxx_tensor_device_ptr(const mpsxx_tensor* t, double** out);

/* ---- planner (host only) --------------------------------------------------- */
/* Block-task enumeration of btas::Gemm (include/btas/QSPARSE/QSTBLAS.h:182-226,
 * include/btas/SPARSE/STBLAS.h:297-359) for c = op(a) op(b) with c of rank c_rank.
 * Call with c_tags == NULL to get ntasks/npairs; then with arrays of those sizes:
 * c_tags[ntasks], pair_ptr[ntasks+1], a_tags[npairs], b_tags[npairs] (original,
 * un-viewed tags), in the reference's enumeration order. */
int mpsxx_gemm_tasks(int transa, int transb, const mpsxx_tensor* a, const mpsxx_tensor* b, int c_rank,
                     int64_t* ntasks, int64_t* npairs, int64_t* c_tags, int64_t* pair_ptr, int64_t* a_tags,
                     int64_t* b_tags);

/* ---- hot path ------------------------------------------------------------- */
/* sgv += H_eff * wfn for merged two-site operators:
 * sgv[A,B] += sum_{w,A',B'} lopr[A,w,A'] wfn[A',B'] ropr[B,w,B']
 * Replaces mpsxx::compute_sigma_vector(lopr, ropr, wfn0, sgv0)
 * (src/compute_sigma_vector.hpp:85-96).  sgv must have wfn's block layout. */
int mpsxx_compute_sigma_vector(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                               const mpsxx_tensor* wfn, mpsxx_tensor* sgv);

/* The other rank overloads of mpsxx::compute_sigma_vector, with the reference's
 * allocate-or-accumulate output: *sgv == NULL -> the result is allocated; otherwise it
 * is added to *sgv, whose missing blocks are added (the handle then refers to the
 * grown tensor).  The H forms run as the merged product above on every allowed merged
 * block of wfn's sectors.
 * one-site, sgv[l,n,r] += sum lopr[l,w,l'] mpo[w,n,n',w'] wfn[l',n',r'] ropr[r,w',r']
 *   (src/compute_sigma_vector.hpp:9-22; used by the one-site Functor<3>); */
int mpsxx_compute_sigma_vector_onesite(mpsxx_context* ctx, const mpsxx_tensor* mpo, const mpsxx_tensor* lopr,
                                       const mpsxx_tensor* ropr, const mpsxx_tensor* wfn, mpsxx_tensor** sgv);
/* two-site four-index, sgv[l,n,n',r] += H_eff wfn with both site MPOs
 *   (src/compute_sigma_vector.hpp:53-70); */
int mpsxx_compute_sigma_vector_twosite(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                                       const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, const mpsxx_tensor* wfn,
                                       mpsxx_tensor** sgv);
/* overlap, sgv += lopr wfn ropr^T for two-index (S) block operators and wfn of 2, 3 or 4
 *   indices: Gemm(N, N, lopr, wfn) then Gemm(N, T, ., ropr)
 *   (src/compute_sigma_vector.hpp:24-35, 72-83, 98-109). */
int mpsxx_compute_sigma_vector_overlap(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                                       const mpsxx_tensor* wfn, mpsxx_tensor** sgv);

/* Work of the split-precision H_eff*psi plan for these operands (the plan is built if
 * needed; no device data is read): out[0..12] = useful FLOPs of stage 1 and 2, tile
 * FLOPs of stage 1 and 2 (128 x 128 tensor-core tiles, 64 on tails, K slices of 32, padding
 * included), K slices of stage 1 and 2, tiles of stage 1 and 2, packed bytes of lopr,
 * ropr, the L*psi intermediate and wfn, and the intermediate's element count;
 * out[13..18] = FLOPs of stage 1 and then stage 2 with only the rows (to 128), only
 * the columns (to 128) or only K (to 32) padded; out[19..20] = tile FLOPs of stage 1
 * and 2 with 64-row tails on the rows only (columns padded to 128); out[21..22] =
 * tiles of both stages on a 64-row and on a 64-column tail. */
int mpsxx_sigma_plan_stats(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                           const mpsxx_tensor* wfn, double* out, int n, int* count);

/* diag[A,B] += sum_w lopr[A,w,A] ropr[B,w,B] on diag's blocks.
 * Replaces mpsxx::compute_diagonal_elements(lopr, ropr, diag)
 * (src/compute_diagonal_elements.hpp:65-80). */
int mpsxx_compute_diagonal_elements(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                                    mpsxx_tensor* diag);

/* diag = the diagonal of H for one-site (src/compute_diagonal_elements.hpp:10-32,
 * diag[l,n,r] = sum lopr[l,w,l] mpo[w,n,n,w'] ropr[r,w',r]) and four-index two-site
 * wavefunctions (:35-62).  diag supplies the sectors and q; as the reference's
 * Copy(scr, diag, 1) (:31, :58), the values diag held are dropped and it holds every
 * block its quantum numbers allow (the handle then refers to the new tensor); blocks
 * no term reaches, which the reference leaves out, are stored as zeros.  The reference's operator-group sum (:84-100) is this call into a fresh
 * tensor per group followed by mpsxx_tensor_accumulate. */
int mpsxx_compute_diagonal_elements_onesite(mpsxx_context* ctx, const mpsxx_tensor* mpo, const mpsxx_tensor* lopr,
                                            const mpsxx_tensor* ropr, mpsxx_tensor* diag);
int mpsxx_compute_diagonal_elements_twosite(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                                            const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, mpsxx_tensor* diag);

/* opr1 = bra^T opr0 ket (forward) or bra opr0 ket^T (backward), allocated by the callee.
 * Replaces mpsxx::renormalize(forward, opr0, bra0, ket0, opr1) for merged operators
 * (src/renormalize.hpp:57-95). */
int mpsxx_renormalize(mpsxx_context* ctx, int forward, const mpsxx_tensor* opr0, const mpsxx_tensor* bra,
                      const mpsxx_tensor* ket, mpsxx_tensor** opr1);

/* renormalize with the site MPO, opr1 (+)= the new block operator (src/renormalize.hpp:10-32;
 * the one-site step and the initial state use it): forward,
 * opr1[a,w',a'] = sum bra*[l,n,a] opr0[l,w,l'] mpo[w,n,n',w'] ket[l',n',a'];
 * backward, opr1[a,w,a'] = sum bra*[a,n,r] opr0[r,w',r'] mpo[w,n,n',w'] ket[a',n',r'].
 * Allocate-or-accumulate output as for the compute_sigma_vector overloads. */
int mpsxx_renormalize_mpo(mpsxx_context* ctx, int forward, const mpsxx_tensor* mpo, const mpsxx_tensor* opr0,
                          const mpsxx_tensor* bra, const mpsxx_tensor* ket, mpsxx_tensor** opr1);
/* renormalize an overlap matrix (src/renormalize.hpp:35-54): forward
 * sov1 = (sov0^T bra*)^T ket over (l, n), backward sov1 = (bra* sov0) ket^T over (n, r). */
int mpsxx_renormalize_overlap(mpsxx_context* ctx, int forward, const mpsxx_tensor* sov0, const mpsxx_tensor* bra,
                              const mpsxx_tensor* ket, mpsxx_tensor** sov1);

/* Guess wavefunction of the next site, mpsxx::compute_guesswave
 * (src/compute_guesswave.hpp:11-38): forward (mps0 = L(i), wfn0 = C(i), mps1 = R(i+1))
 * wfn1 = (L(i)^+ C(i)) R(i+1); backward (mps0 = R(i+1), wfn0 = C(i+1), mps1 = L(i))
 * wfn1 = L(i) (C(i+1) R(i+1)^+).  Two Gemms; *wfn1 is allocated when NULL, else the
 * result is added to it (quantum numbers and shapes checked). */
int mpsxx_compute_guesswave(mpsxx_context* ctx, int forward, const mpsxx_tensor* mps0, const mpsxx_tensor* wfn0,
                            const mpsxx_tensor* mps1, mpsxx_tensor** wfn1);

/* Merged super-block operator of one MPO site and one block operator.
 * Replaces the per-group body of mpsxx::compute_merged_operator
 * (src/optimize.hpp:273-368).  mpo must have been uploaded from the host. */
int mpsxx_compute_merged_operator(mpsxx_context* ctx, int forward, const mpsxx_tensor* mpo,
                                  const mpsxx_tensor* opr, mpsxx_tensor** out);

/* Davidson lowest eigenpair of H_eff = (lopr, ropr) starting from wfnc (overwritten).
 * Replaces mpsxx::Davidson::diagonalize (src/diagonalize.hpp:310-449) for one root.
 * stats (may be NULL): [n_sigma, macro, micro, converged]. */
int mpsxx_diagonalize(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                      const mpsxx_tensor* diag, mpsxx_tensor* wfnc, double tol, double* energy, int* stats);

/* diagonalize with lower roots projected out (state-specific multi-root targeting,
 * the projected Functor of src/diagonalize.hpp:200-277): for every lower root j, S[j]
 * is its wavefunction and H[j] its H_eff product expressed in this bond's basis
 * (tensors with wfnc's block layout), E[j] its energy; the operator applied is
 * H c - S_j <H_j|c> - H_j <S_j|c> + E_j S_j <S_j|c>, and the start vector and the
 * result are orthogonalised against the S_j (at most 12 roots). */
int mpsxx_diagonalize_projected(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                                const mpsxx_tensor* diag, mpsxx_tensor* wfnc, double tol, int nproj,
                                const mpsxx_tensor* const* S, const mpsxx_tensor* const* H, const double* E,
                                double* energy, int* stats);

/* y += alpha x for tensors of the same sectors; every block of x must be stored in y
 * (btas::Axpy over the blocks of x, include/btas/SPARSE/STBLAS.h). */
int mpsxx_tensor_accumulate(mpsxx_context* ctx, double alpha, const mpsxx_tensor* x, mpsxx_tensor* y);

/* Truncated SVD of a merged wavefunction; forward: lmat = U, rmat = s V^T;
 * backward: lmat = U s, rmat = V^T.  Replaces mpsxx::canonicalize(forward, wfnc,
 * lmat, rmat, M, noise) (src/canonicalize.hpp:88-106).  With noise >= 1e-8 the SVD
 * runs on make_noise(wfnc, noise); wfnc itself is left unchanged (the reference
 * noises it in place and its callers do not read it afterwards). */
int mpsxx_canonicalize(mpsxx_context* ctx, int forward, const mpsxx_tensor* wfnc, int M, double noise,
                       mpsxx_tensor** lmat, mpsxx_tensor** rmat);

/* wfnc += noise * (array of the reference's noise sequence), in place; nothing when
 * noise < 1e-8.  Replaces mpsxx::make_noise(wfnc, noise) (src/canonicalize.hpp:11-24):
 * the array holds every allowed block whose sectors have a block in wfnc (blocks
 * wfnc lacks are added), and each of its blocks holds, row-major, the leading values
 * of the sequence of mpsxx_noise_sequence. */
int mpsxx_make_noise(mpsxx_context* ctx, mpsxx_tensor* wfnc, double noise);

/* Host only: the first n values make_noise draws (a default-seeded std::mt19937 through
 * std::uniform_real_distribution<double>(-1, 1), src/canonicalize.hpp:16-21). */
int mpsxx_noise_sequence(int64_t n, double* out);

/* One bond of the two-site sweep (src/optimize.hpp:495-651), single root and one
 * operator group: returns the Ritz value, the renormalised operator of the grown
 * block and the new site tensors.  stats (may be NULL, 12 doubles): n_sigma,
 * sigma FLOPs, t_merge, t_diag, t_davidson, t_svd, t_renorm, converged,
 * Davidson |r|^2, Ritz value before refinement, FP64 |r|^2 after refinement,
 * FP64 refinement applications (the last three are 0 in FP64 precision). */
int mpsxx_optimize_twosite_merged(mpsxx_context* ctx, int forward, const mpsxx_tensor* lmpo,
                                  const mpsxx_tensor* rmpo, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                                  const mpsxx_tensor* lwfn, const mpsxx_tensor* rwfn, double tole, int M,
                                  double noise, double* energy, mpsxx_tensor** env, mpsxx_tensor** new_lwfn,
                                  mpsxx_tensor** new_rwfn, double* stats);

/* optimize_twosite_merged for n independent bonds at once (e.g. the chains of a
 * parameter scan), arrays of n entries each.  The Davidson iterations of all bonds
 * run in lockstep: in split precision every H_eff*psi of the unconverged bonds is
 * one grouped tensor-core launch per stage (captured with its packing as a CUDA
 * graph) and the vector algebra is one batched launch per operation; the results
 * equal n separate mpsxx_optimize_twosite_merged calls up to rounding.  noise (may be
 * NULL: no noise) holds each bond's make_noise amplitude.  stats: 6 doubles per bond
 * (n_sigma, n_sigma_fp64, micro iterations, converged, |r|^2, energy before
 * refinement). */
int mpsxx_optimize_twosite_merged_batch(mpsxx_context* ctx, int n, const int* forward,
                                        const mpsxx_tensor* const* lmpo, const mpsxx_tensor* const* rmpo,
                                        const mpsxx_tensor* const* lopr, const mpsxx_tensor* const* ropr,
                                        const mpsxx_tensor* const* lwfn, const mpsxx_tensor* const* rwfn, double tole,
                                        const int* M, const double* noise, double* energy, mpsxx_tensor** env,
                                        mpsxx_tensor** new_lwfn, mpsxx_tensor** new_rwfn, double* stats);

/* Adjoint of the bond energy with respect to the MPO: for the normalised merged
 * two-site wavefunction psi[A,B] of the bond between lmpo and rmpo,
 * E = <psi| H_eff |psi>, and grad_l[b] = dE/d(block b of lmpo), grad_r likewise
 * (arrays of nnz(lmpo) and nnz(rmpo) doubles, block order; MPO blocks are 1x1x1x1).
 * dE/d(merged operator) is contracted on the tensor cores in split precision when
 * the context's precision is not MPSXX_FP64, then pulled back through the merged-
 * operator scatter by a deterministic adjoint kernel.  E is linear in each site
 * MPO, so sum_b W_l[b] grad_l[b] = E.  No reference counterpart (the reference has
 * no derivatives); it differentiates mpsxx::compute_merged_operator
 * (src/optimize.hpp:273-368) and compute_sigma_vector. */
int mpsxx_mpo_gradient(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                       const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, const mpsxx_tensor* psi, double* grad_l,
                       double* grad_r);

/* a[i, j, k, ...] -> out[(i, j), k, ...] and its inverse (QSTmerge / QSTexpand over
 * the leading two indices, include/btas/QSPARSE/QSTmerge.h:31-120,218-295) for the
 * one-site algorithm; a has 3 or more indices; `like` (3 indices) supplies the
 * unmerged sectors. */
int mpsxx_merge_rows(mpsxx_context* ctx, const mpsxx_tensor* a, mpsxx_tensor** out);
int mpsxx_expand_rows(mpsxx_context* ctx, const mpsxx_tensor* b, const mpsxx_tensor* like, mpsxx_tensor** out);

/* Merge the last two indices of a tensor of 3 or more indices in place of the
 * reference's QSTmerge(a, cols_info, b) (include/btas/QSPARSE/QSTmerge.h:85-140). */
int mpsxx_merge_cols(mpsxx_context* ctx, const mpsxx_tensor* a, mpsxx_tensor** out);

/* c = alpha * op(a) op(b) into a new tensor of rank c_rank whose blocks are the
 * enumerated task results (btas::Gemm into an empty array,
 * include/btas/QSPARSE/QSTBLAS.h:182-226). */
int mpsxx_gemm(mpsxx_context* ctx, int transa, int transb, double alpha, const mpsxx_tensor* a,
               const mpsxx_tensor* b, int c_rank, mpsxx_tensor** c);

/* Expand the last index of b into the last two indices of `like` (a 3-index
 * tensor whose trailing index shapes define the merge), the reference's
 * QSTexpand(b, cols_info, a) (include/btas/QSPARSE/QSTmerge.h:297-372). */
int mpsxx_expand_cols(mpsxx_context* ctx, const mpsxx_tensor* b, const mpsxx_tensor* like, mpsxx_tensor** out);

/* Merged two-site wavefunction psi[A,B] = merge(lwfn[l,n,m] rwfn[m,n',r]) with the
 * ket merge infos of the bond (src/optimize.hpp:536-557); every allowed block is stored. */
int mpsxx_merge_wavefunction(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                             const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, const mpsxx_tensor* lwfn,
                             const mpsxx_tensor* rwfn, mpsxx_tensor** psi);

/* Split merged lmat[A,m] / rmat[m,B] back into site tensors (QSTexpand of
 * src/optimize.hpp:611-612) with the same merge infos. */
int mpsxx_expand_wavefunction(mpsxx_context* ctx, const mpsxx_tensor* lmpo, const mpsxx_tensor* rmpo,
                              const mpsxx_tensor* lopr, const mpsxx_tensor* ropr, const mpsxx_tensor* lmat,
                              const mpsxx_tensor* rmat, mpsxx_tensor** lwfn, mpsxx_tensor** rwfn);

/* Measurement helper (no reference counterpart): average device time in seconds of
 * `reps` back-to-back sigma applications, bracketed by CUDA events on the
 * context's stream (sgv accumulates reps times). */
int mpsxx_sigma_device_time(mpsxx_context* ctx, const mpsxx_tensor* lopr, const mpsxx_tensor* ropr,
                            const mpsxx_tensor* wfn, mpsxx_tensor* sgv, int reps, double* seconds);

/* x /= ||x||_2 (btas::Normalize, include/btas/QSPARSE/QSTBLAS.h:239-243); norm may be NULL. */
int mpsxx_normalize(mpsxx_context* ctx, mpsxx_tensor* x, double* norm);

/* Allocation-free multi-dot; this entry point has no counterpart in the reference.
 * out[i*ny + j] = dot(X + i*stride, Y + j*stride) over n doubles (all device
 * pointers), 1 <= nx, ny <= 10: the Rayleigh-Ritz products of the Davidson solver.
 * It is for callers that cannot call cudaMalloc while they run — a host application
 * that has claimed the device memory for its own pool and hands plugins only its own
 * buffers, or a loop that cannot afford the device-wide synchronisation an
 * allocation may cause.  It needs no context and calls no allocator: its reduction
 * scratch is a fixed array of 304 x 100 doubles (243 KB) built into the library,
 * which every device that loads the library holds until the process exits.  The
 * first call on a device resolves the array's address for that device, so make it
 * before any stream capture.  All calls on a device share the array: calls whose
 * kernels overlap on the GPU race.  Larger requests (nx or ny > 10) are rejected
 * with MPSXX_INVALID_ARGUMENT.  The work is enqueued on `stream` (NULL: the default
 * stream) and the call returns without waiting for it. */
int mpsxx_multidot_noalloc(const double* X, int nx, const double* Y, int ny, int64_t n, int64_t stride,
                           double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MPSXX_GB300_H */
