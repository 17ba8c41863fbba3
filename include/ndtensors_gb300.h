/*
 * ndtensors_gb300.h -- C ABI of libndtensors_gb300.so, the GB300 (sm_103a)
 * implementation of the NDTensors contraction hot path.
 *
 * Conventions (identical to NDTensors):
 *   - tensors are column-major (first index fastest);
 *   - block numbers are 1-based (Julia `Block{N}`), block offsets are 0-based
 *     element offsets into one flat data vector (`BlockOffsets`);
 *   - labels follow ncon: a label shared by both inputs is contracted
 *     (NDTensors uses negative labels for those), output labels list the
 *     uncontracted labels in output order;
 *   - permutations are 1-based (Julia `permutedims(T, perm)`);
 *   - every function returns an nd_status; nd_last_error() gives the message.
 *     No entry point aborts, exits or traps the GPU.
 *
 * All data pointers are DEVICE pointers unless a parameter says "host".
 * Work is enqueued on the handle's stream; functions that return structure
 * to the host (plans, SVD kept dimensions) synchronise that stream.
 */
#ifndef NDTENSORS_GB300_H
#define NDTENSORS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t nd_status;
enum {
  ND_OK = 0,
  ND_ERR_ARG = 1,          /* invalid argument (labels, dims, perm, sizes)      */
  ND_ERR_OOM = 2,          /* device allocation failed                          */
  ND_ERR_NOCONV = 3,       /* an SVD did not converge within the sweep limit    */
  ND_ERR_TIMEOUT = 4,      /* a device-side wait ran past its iteration limit   */
  ND_ERR_CUDA = 5,         /* a CUDA runtime/driver call failed                 */
  ND_ERR_UNSUPPORTED = 6,  /* shape/feature outside what the library supports  */
  ND_ERR_NONFINITE = 7     /* split-precision GEMM met Inf/NaN input            */
};

/* GEMM arithmetic for contractions. */
enum {
  ND_PREC_FP64 = 0,    /* FP64 tensor-core (DMMA) GEMM: the plain drop-in          */
  ND_PREC_OZAKI = 1,   /* exact int8-range slices on tcgen05 BF16, FP64 result     */
  ND_PREC_BF16X3 = 2   /* 3xBF16 split, FP32 accumulate, FP64 result               */
};

#define ND_MAX_RANK 8

typedef struct nd_context *nd_handle;
typedef struct nd_bs_plan_s *nd_plan;

/* ---- context, memory, streams ------------------------------------------ */
/* Replaces the storage/stream management CUDA.jl gives NDTensorsCUDAExt
 * (NDTensors/ext/NDTensorsCUDAExt/NDTensorsCUDAExt.jl). */
nd_status nd_create(int32_t device, nd_handle *out);
nd_status nd_destroy(nd_handle h);
const char *nd_last_error(nd_handle h);
nd_status nd_set_stream(nd_handle h, void *cuda_stream);      /* NULL = legacy default stream */
nd_status nd_get_stream(nd_handle h, void **cuda_stream);
nd_status nd_sync(nd_handle h);
nd_status nd_alloc(nd_handle h, size_t bytes, void **dptr);
nd_status nd_free(nd_handle h, void *dptr);
nd_status nd_h2d(nd_handle h, void *dst, const void *host_src, size_t bytes);
nd_status nd_d2h(nd_handle h, void *host_dst, const void *src, size_t bytes);
nd_status nd_memset0(nd_handle h, void *dst, size_t bytes);
/* Poll limit of the library's device-side waits (mbarrier waits of the TMA and
 * tensor-core pipelines, grid barriers of the SVD).  A wait that runs past it
 * makes the call return ND_ERR_TIMEOUT instead of hanging; copies and MMAs
 * already issued are still waited for before a kernel exits, and the handle stays
 * usable.  0 restores the default (2^26 polls).  Synchronises the handle's stream.
 * No counterpart in the reference (its CPU path has no device waits). */
nd_status nd_set_spin_limit(nd_handle h, uint32_t polls);
/* FP64 Jacobi sweep limit of nd_bs_svd_f64 (default 60; negative restores it).  A
 * block that has not converged within it makes the SVD return ND_ERR_NOCONV, the
 * case where the reference's svd returns `nothing`
 * (NDTensors/src/linearalgebra/linearalgebra.jl:91-127). */
nd_status nd_set_svd_max_sweeps(nd_handle h, int32_t sweeps);
/* How the last blockwise SVD / eigen on this handle converged (diagnostics; no
 * counterpart in the reference, whose LAPACK calls report nothing of the kind).
 * ints (up to nints): [0] FP32 sweeps, [1] refinement steps, [2] FP64 sweeps,
 * [3] 1 if the sweeps ran on shared-memory panels, [4..] blocks still active at the
 * start of each FP64 sweep.  dbls (up to ndbls): the largest first-order rotation of
 * each refinement step, then the largest relative off-diagonal |w_i . w_j| /
 * (|w_i| |w_j|) rotated in each FP64 sweep, then the same for each FP32 sweep. */
nd_status nd_svd_last_info(nd_handle h, int32_t* ints, int32_t nints, double* dbls, int32_t ndbls);
/* Per-CTA timing of the persistent split-GEMM launches (diagnostics for the
 * longest-first tile schedule; no counterpart in the reference).  With timing on,
 * each split-GEMM launch records, per CTA, its start and end (%globaltimer, ns).
 * nd_cta_times_read synchronises and returns the last min(#launches, 8) launches in
 * order: times[k * 2048 + 2 * c + {0, 1}] for CTA c < nctas[k] of launch k. */
nd_status nd_set_cta_timing(nd_handle h, int32_t enable);
nd_status nd_cta_times_read(nd_handle h, uint64_t* times, int32_t* nctas, int32_t* nlaunch);
/* Output tile of the split-precision (Ozaki / 3xBF16) GEMM when the autotuner has no
 * entry for a contraction: 0 (default) = 128 x 64 tiles on single CTAs, 1 = 256 x 64
 * tiles on pairs of CTAs (tcgen05.mma.cta_group::2).  With tuning on, both are timed
 * and the faster is cached.  No counterpart in the reference. */
nd_status nd_set_split_tile(nd_handle h, int32_t shape);
/* Transposing permutes: 0 (default) = shared-memory tiles over dimension groups with
 * plain loads; 1 = TMA-staged tiles (cp.async.bulk.tensor) for shapes a 5-D tensor
 * map describes, the group tiles otherwise.  Both are bit-exact.  No counterpart in
 * the reference. */
nd_status nd_set_permute_path(nd_handle h, int32_t path);
/* Verify mode.  With on != 0, every contraction in a split precision (ND_PREC_OZAKI,
 * ND_PREC_BF16X3) through nd_contract_dense_f64, nd_bs_contract_f64 and
 * nd_bs_contract_adjoint_f64 is computed a second time with the FP64 kernels into
 * scratch memory, and the relative Frobenius distance of the two results,
 * ||R - R_fp64||_F / ||R_fp64||_F over every element the call writes (both cotangents
 * for the adjoint), is recorded; FP64 calls record 0.  A verified call synchronises the
 * stream and is refused (ND_ERR_ARG) during graph capture.  Switching the mode resets
 * the record.  No counterpart in the reference (its BLAS path has one precision). */
nd_status nd_set_verify(nd_handle h, int32_t on);
/* The relative error recorded by the last verified contraction; -1 before any, and when
 * the last verified call failed before its comparison. */
nd_status nd_verify_last(nd_handle h, double* rel_err);
/* Where nd_bs_plan_create builds plans: 0 (default) = on the host up to 4096 pairs,
 * else on the device; 1 = always on the device; 2 = on the host whenever the
 * contracted block numbers fit a 64-bit key.  Every placement gives the same plan.
 * No counterpart in the reference (its plan is host code). */
nd_status nd_set_plan_placement(nd_handle h, int32_t where);
/* Number of slice digits used by ND_PREC_OZAKI (3..6, default 5). */
nd_status nd_set_ozaki_slices(nd_handle h, int32_t slices);
/* Count of kernel launches this handle enqueued so far (diagnostics). */
nd_status nd_launch_count(nd_handle h, int64_t *count);
/* Kernel timing: when enabled, every library kernel launch is bracketed by CUDA
 * events on the handle's stream.  nd_profile_read synchronises, then reports per
 * kernel name (up to `cap` entries, names copied into `names` as 64-byte
 * NUL-terminated slots) the launch count and the summed device time in ms, and
 * clears the records. */
nd_status nd_profile_enable(nd_handle h, int32_t enable);
nd_status nd_profile_read(nd_handle h, int32_t cap, char *names, int64_t *counts, double *total_ms,
                          int32_t *n_out);

/* ---- dense permutation --------------------------------------------------
 * R = beta*R + alpha*permutedims(T, perm), with the reference's rules: beta == 0
 * overwrites R (NaN in R does not propagate), alpha == 0 keeps only beta*R.
 * Replaces permutedims!(::Exposed{<:Array}, ...) (NDTensors/src/array/permutedims.jl:5-24)
 * and the fused _contract_scalar_perm! (NDTensors/src/abstractarray/tensoralgebra/contract.jl:88-113);
 * GPU counterpart NDTensors/ext/NDTensorsCUDAExt/permutedims.jl:4-23. */
nd_status nd_permutedims_f64(nd_handle h, double *R, const double *T, int32_t rank,
                             const int64_t *dimsT /* host */, const int32_t *perm /* host, 1-based */,
                             double alpha, double beta);

/* ---- dense contraction --------------------------------------------------
 * R = alpha * contract(A, B) + beta * R.  Replaces
 * contract!(R::DenseTensor, labelsR, T1, labelsT1, T2, labelsT2, alpha, beta)
 * (NDTensors/src/dense/tensoralgebra/contract.jl:160-216), i.e. the cuTENSOR hook
 * NDTensors/ext/NDTensorscuTENSORExt/contract.jl:15-58 and the cuBLAS mul! of
 * NDTensors/ext/NDTensorsCUDAExt/mul.jl:7-47.  A one-element operand takes the
 * reference's scalar branch (contract.jl:100-150).  The call synchronises the
 * handle's stream before it returns. */
nd_status nd_contract_dense_f64(nd_handle h,
                                double *R, int32_t rankR, const int64_t *dimsR, const int32_t *labelsR,
                                const double *A, int32_t rankA, const int64_t *dimsA, const int32_t *labelsA,
                                const double *B, int32_t rankB, const int64_t *dimsB, const int32_t *labelsB,
                                double alpha, double beta, int32_t precision);

/* Same contraction as nd_contract_dense_f64 with ND_PREC_OZAKI, for callers that
 * cannot allocate device memory during the call (their memory belongs to another
 * allocator with a hard budget, or they cannot afford cudaMalloc's
 * synchronisation).  It allocates nothing: its scratch is a fixed 32 MiB device
 * array inside the library, held by every GPU that loads the library until exit.
 * Its address is looked up on the first call per device; make that first call
 * before any stream capture.  Each call uploads its descriptors from host memory
 * and synchronises the handle's stream before it returns, so calls made while
 * that stream is being captured are refused with ND_ERR_ARG.  Contractions
 * needing more scratch are rejected with ND_ERR_ARG.  All calls share the array,
 * so calls whose GPU work overlaps race.  No counterpart in the reference:
 * NDTensors always allocates its outputs and BLAS manages its own workspace. */
nd_status nd_contract_dense_ozaki_noalloc_f64(nd_handle h,
                                              double *R, int32_t rankR, const int64_t *dimsR, const int32_t *labelsR,
                                              const double *A, int32_t rankA, const int64_t *dimsA, const int32_t *labelsA,
                                              const double *B, int32_t rankB, const int64_t *dimsB, const int32_t *labelsB,
                                              double alpha, double beta);

/* ---- block-sparse structure ---------------------------------------------
 * A block-sparse operand: per-dimension block dims plus the ordered list of
 * nonzero blocks and their offsets (NDTensors BlockSparse + BlockOffsets,
 * NDTensors/src/blocksparse/blocksparse.jl:5-13, blockoffsets.jl:11). Host arrays. */
typedef struct {
  int32_t rank;
  const int32_t *nblocks;    /* [rank] number of blocks of each dimension                */
  const int64_t *blockdims;  /* concatenation over dimensions of the per-block dims      */
  int32_t nnzblocks;
  const int32_t *blocks;     /* [nnzblocks][rank] 1-based block numbers, row per block   */
  const int64_t *offsets;    /* [nnzblocks] 0-based element offsets                      */
} nd_bs_desc;

/* Build the contraction plan: the list of contracted block pairs in the
 * reference's sequential order (A-block major, B-block minor), the output block
 * list in first-appearance order and its offsets.  Bit-exact with
 * contract_blockoffsets(::Algorithm"sequential", ...)
 * (NDTensors/src/blocksparse/contract_sequential.jl:1-41,
 *  contract_utilities.jl:45-91, contract.jl:20-55).  Plans of up to 4096 pairs are
 * built on the host, larger ones by the device planner (see nd_set_plan_placement). */
nd_status nd_bs_plan_create(nd_handle h, const nd_bs_desc *A, const int32_t *labelsA,
                            const nd_bs_desc *B, const int32_t *labelsB,
                            int32_t rankR, const int32_t *labelsR, nd_plan *plan);
/* Sizes of the plan's outputs. */
nd_status nd_bs_plan_sizes(nd_plan plan, int32_t *npairs, int32_t *nnzblocksR, int64_t *nnzR);
/* Copy the plan to host arrays: blocksR [nnzblocksR][rankR] (1-based), offsetsR,
 * pairs [npairs][3] = (A block index, B block index, R block index), 0-based
 * positions in the respective block lists.  Any pointer may be NULL. */
nd_status nd_bs_plan_get(nd_plan plan, int32_t *blocksR, int64_t *offsetsR, int32_t *pairs);
nd_status nd_bs_plan_destroy(nd_plan plan);
/* Write the plan's output blocks at these element offsets (host, nnzblocksR entries)
 * instead of the reference's first-appearance offsets: the contraction then lands
 * directly in a caller's layout (e.g. an H_eff apply writing back into psi's block
 * order, which a Krylov solver needs).  The caller guarantees the blocks do not
 * overlap.  No counterpart in the reference (its result is always a fresh tensor). */
nd_status nd_bs_plan_set_output_offsets(nd_plan plan, const int64_t *offsetsR);

/* R = alpha * contract(A, B) executed as ONE grouped-GEMM launch over all
 * block pairs: pairs are grouped by output block, the first pair of a group
 * overwrites and the rest accumulate (NDTensors/src/blocksparse/contract_generic.jl:37-129,
 * with compute_alpha == 1, contract_utilities.jl:2-15). */
nd_status nd_bs_contract_f64(nd_handle h, nd_plan plan, double *R, const double *A,
                             const double *B, double alpha, int32_t precision);

/* R = alpha * contract(T, D) for a block-sparse T and a block-diagonal DiagBlockSparse D
 * (NDTensors/src/blocksparse/diagblocksparse.jl:601-696; per pair the diagonal
 * contraction of NDTensors/src/diag/tensoralgebra/contract.jl:103-214).  The plan is
 * built with nd_bs_plan_create from T and D's block structure (every D block has equal
 * block numbers); D's data is the diagonal of each of its blocks, block b's
 * min(block dims) values starting at diag_offsets[b] (host).  Output structure and
 * block order are the plan's; elements off the diagonal of D's indices are zero. */
nd_status nd_bs_contract_diag_f64(nd_handle h, nd_plan plan, double *R, const double *T, const double *Ddiag,
                                  const int64_t *diag_offsets, double alpha);

/* Pullback of R = contract(A, B) for the same plan (ext/ITensorsChainRulesCoreExt/itensor.jl:94-103):
 * Abar = Rbar * B (contract over B's free labels), Bbar = A * Rbar.  Both
 * contractions run in one grouped-GEMM launch.  Abar/Bbar have A's/B's structure. */
nd_status nd_bs_contract_adjoint_f64(nd_handle h, nd_plan plan, const double *Rbar,
                                     const double *A, const double *B,
                                     double *Abar, double *Bbar, int32_t precision);

/* Block-sparse permutedims: every block permuted; output block order = input
 * order, offsets recomputed by the caller's layout (offsetsR, host).
 * (NDTensors/src/blocksparse/blocksparsetensor.jl:834-881, blockoffsets.jl:103-111)
 * Blocks of 2^22 elements or more run through the tiled transposer one by one; all
 * smaller blocks in one batched launch.  Bit-exact; stream-ordered. */
nd_status nd_bs_permutedims_f64(nd_handle h, const nd_bs_desc *T, const double *Tdata,
                                const int32_t *perm, const int64_t *offsetsR, double *Rdata);

/* ---- block matrix factorizations ----------------------------------------
 * Blockwise SVD of a 2-index block matrix with truncation
 * (NDTensors/src/blocksparse/linearalgebra.jl:45-215, truncate.jl:23-107).
 * Blocks are dense column-major m_b x n_b at offsets[b] in A.  Outputs, for
 * the kept blocks in input order (dropped blocks removed):
 *   U: concatenation of m_b x k_b column-major blocks,
 *   S: concatenation of k_b values (descending within a block),
 *   V: concatenation of n_b x k_b column-major blocks,
 * where k_b = kept[b] (0 = dropped).  Caller sizes U/S/V for the untruncated
 * case (sum m_b*min, sum min, sum n_b*min).  spectrum (host, length >= sum min)
 * receives the truncated sorted s^2; *spectrum_len its length.  Pass maxdim or
 * cutoff < 0 to mean "nothing" (no truncation).  ND_ERR_NOCONV if a block
 * did not converge (the reference returns `nothing`). */
nd_status nd_bs_svd_f64(nd_handle h, int32_t nblocks, const int64_t *rows, const int64_t *cols,
                        const int64_t *offsets, const double *A,
                        double *U, double *S, double *V,
                        int32_t mindim, int32_t maxdim, double cutoff,
                        int32_t use_absolute_cutoff, int32_t use_relative_cutoff, int32_t min_blockdim,
                        int32_t *kept, double *spectrum, int32_t *spectrum_len,
                        double *truncerr, double *docut);

/* Blockwise SVD plan (no counterpart in the reference): the blockwise truncated SVD
 * of nd_bs_svd_f64 for fixed block dimensions (block b is rows[b] x cols[b]), with
 * every buffer and launch state built at creation (creation runs the SVD once on
 * zeros and synchronises), fixed sweep and refinement counts, and convergence, kept
 * dimensions, spectrum and truncation error left in DEVICE memory.  An execution only
 * enqueues work on the handle's stream, so it can be captured into a CUDA graph (for
 * example with the Krylov loop of a sweep step).  Outputs: U, S, V as nd_bs_svd_f64
 * (kept prefixes concatenated in block order; size them for the untruncated case),
 * kept[nblocks], spectrum[sum of min(rows, cols)] (the first *spectrum_len entries are
 * the truncated pooled s^2, descending), truncerr[1], status[1] = ND_OK or
 * ND_ERR_NOCONV (all device).  offsets: host, the blocks' offsets in A (a change is
 * uploaded, which is refused during capture).  Blocks taller than a shared-memory
 * panel (3200 rows in FP64) give ND_ERR_UNSUPPORTED at creation. */
typedef struct nd_svd_plan_s *nd_svd_plan;
nd_status nd_bs_svd_plan_create(nd_handle h, int32_t nblocks, const int64_t *rows, const int64_t *cols,
                                nd_svd_plan *plan);
nd_status nd_bs_svd_plan_exec(nd_svd_plan plan, const int64_t *offsets, const double *A, double *U, double *S,
                              double *V, int32_t mindim, int32_t maxdim, double cutoff, int32_t use_absolute_cutoff,
                              int32_t use_relative_cutoff, int32_t min_blockdim, int32_t *kept, double *spectrum,
                              int32_t *spectrum_len, double *truncerr, int32_t *status);
nd_status nd_bs_svd_plan_destroy(nd_svd_plan plan);

/* Blockwise eigendecomposition of a real symmetric block-diagonal matrix with
 * truncation (eigen(::Hermitian{<:BlockSparseMatrix}), NDTensors/src/blocksparse/
 * linearalgebra.jl:221-348; per block the dense Hermitian eigen sorted by |lambda|
 * descending, NDTensors/src/linearalgebra/linearalgebra.jl:162-213).  Block b is
 * dims[b] x dims[b] at offsets[b] in A.  Outputs for the kept blocks in input order:
 * D, the concatenated kept eigenvalues (|lambda| descending within a block), and V,
 * the concatenated dims[b] x kept[b] column-major eigenvector blocks; kept[b] = 0 for
 * a dropped block.  Size D and V for the untruncated case.  spectrum (host) receives
 * the truncated pooled |lambda| (sorted descending).  ND_ERR_NOCONV as nd_bs_svd_f64. */
nd_status nd_bs_eigen_f64(nd_handle h, int32_t nblocks, const int64_t *dims, const int64_t *offsets, const double *A,
                          double *D, double *V, int32_t mindim, int32_t maxdim, double cutoff,
                          int32_t use_absolute_cutoff, int32_t use_relative_cutoff, int32_t min_blockdim,
                          int32_t *kept, double *spectrum, int32_t *spectrum_len, double *truncerr, double *docut);

/* Blockwise QR (NDTensors/src/blocksparse/linearalgebra.jl:351-415, dense qr /
 * qr_positive NDTensors/src/linearalgebra/linearalgebra.jl:321-381).  Q blocks
 * m_b x k_b, R blocks k_b x n_b, k_b = min(m_b, n_b), concatenated in order.
 * Householder reflectors with LAPACK geqrf's signs (positive != 0: diag(R) >= 0), in
 * 16-column panels whose trailing updates and Q accumulation run on many CTAs per
 * block; FP64 throughout.  Stream-ordered: returns once the work is enqueued. */
nd_status nd_bs_qr_f64(nd_handle h, int32_t nblocks, const int64_t *rows, const int64_t *cols,
                       const int64_t *offsets, const double *A, double *Q, double *Rf,
                       int32_t positive);

/* truncate! on a device vector of descending weights (NDTensors/src/truncate.jl:23-107);
 * results to host.  *newlen = kept length. */
nd_status nd_truncate_f64(nd_handle h, const double *P, int32_t n, int32_t mindim, int32_t maxdim,
                          double cutoff, int32_t use_absolute_cutoff, int32_t use_relative_cutoff,
                          int32_t *newlen, double *truncerr, double *docut);

/* Strided block copies: for each entry, dst[dst_off + sum_k i_k*dst_strides[k]] =
 * src[src_off + sum_k i_k*src_strides[k]] over the box dims[0..rank).  This is the
 * data motion of the block-sparse combiner (permutedims_combine / uncombine,
 * NDTensors/src/blocksparse/blocksparsetensor.jl:537-638,693-791): the host
 * computes the combined block structure, the device gathers / scatters. */
typedef struct {
  int64_t src_off, dst_off;
  int32_t rank;
  int64_t dims[ND_MAX_RANK];
  int64_t src_strides[ND_MAX_RANK];
  int64_t dst_strides[ND_MAX_RANK];
} nd_block_copy;
nd_status nd_block_copy_f64(nd_handle h, int32_t n, const nd_block_copy *list /* host */, const double *src,
                            double *dst);
/* The same copies prepared once (the list converted and uploaded at creation), so that
 * a run only launches the kernel and can be captured into a CUDA graph. */
typedef struct nd_copy_plan_s *nd_copy_plan;
nd_status nd_block_copy_plan_create(nd_handle h, int32_t n, const nd_block_copy *list /* host */, nd_copy_plan *plan);
nd_status nd_block_copy_plan_run(nd_copy_plan plan, const double *src, double *dst);
nd_status nd_block_copy_plan_destroy(nd_copy_plan plan);

/* ---- vector-space operations (Krylov solvers) ---------------------------------
 * The VectorInterface methods the reference defines for ITensors
 * (ext/ITensorsVectorInterfaceExt/ITensorsVectorInterfaceExt.jl:5-84) on flat FP64
 * device vectors of length n, plus the two block forms of classical Gram-Schmidt
 * against k <= 32 basis vectors stored ldv apart.  Results and scalars are DEVICE
 * pointers and nothing synchronises, so a Krylov iteration built from these calls and
 * contractions can be captured into one CUDA graph (make one eager call per handle
 * before capturing: the first reduction allocates its fixed partial-sum buffer).
 * Reductions run in a fixed order: replays reproduce eager results bit for bit. */
nd_status nd_vec_inner_f64(nd_handle h, int64_t n, const double *x, const double *y, double *out);   /* inner(x, y)     */
nd_status nd_vec_norm_f64(nd_handle h, int64_t n, const double *x, double *out);                     /* norm(x)         */
/* y = alpha * x, times (invert = 0) or divided by (invert = 1) the device scalar *s when s != NULL:
 * scale(x, alpha) / scale!(y, x, alpha) */
nd_status nd_vec_scale_f64(nd_handle h, int64_t n, const double *x, double *y, double alpha, const double *s,
                           int32_t invert);
/* y = beta * y + alpha * x (beta == 0 overwrites y): add!(y, x, alpha, beta) */
nd_status nd_vec_add_f64(nd_handle h, int64_t n, const double *x, double *y, double alpha, double beta);
/* out[j] = inner(V_j, x), V_j = V + j * ldv, j < k */
nd_status nd_vec_dots_f64(nd_handle h, int64_t n, int32_t k, const double *V, int64_t ldv, const double *x,
                          double *out);
/* y += sign * sum_j coef[j] * V_j, j < k (coef a device array) */
nd_status nd_vec_update_f64(nd_handle h, int64_t n, int32_t k, const double *V, int64_t ldv, const double *coef,
                            double sign, double *y);
/* Lowest eigenpair of the k x k symmetric tridiagonal matrix (diagonal alpha[k],
 * off-diagonal beta[k - 1]; k <= 32), all device arrays: *value, and y[k] normalised
 * with its largest component positive.  The Krylov solver's small eigenproblem on the
 * device, so that a whole Lanczos solve can be one CUDA graph (the reference's solver,
 * KrylovKit, solves it on the host). */
nd_status nd_tridiag_lowest_f64(nd_handle h, int32_t k, const double *alpha, const double *beta, double *value,
                                double *y);

/* ---- autotuner -------------------------------------------------------------
 * Execution parameters of a contraction (today: the split-K target of the FP64
 * tile kernel and whether skinny block pairs, N <= 8 and K <= 32, run on the FP64
 * CUDA-core kernel or with the precision's tile kernel) are chosen per
 * block-size histogram: the key is the device's SM count, the precision, the
 * Ozaki slice count and the counts of block pairs per (log2 M, log2 N, log2 K)
 * bucket.  With tuning on, the first execution of a contraction whose key is
 * not cached times every candidate on the real operands (only when beta == 0,
 * never inside a capture) and caches the fastest; otherwise a cached choice is
 * used, else the defaults.  The cache persists as a text file.  No counterpart
 * in the reference (its tuning knobs are the BLAS/backend choice,
 * NDTensors/src/lib/BackendSelection/src/backend_types.jl:45-52). */
nd_status nd_tune_enable(nd_handle h, int32_t enable);
nd_status nd_tune_count(nd_handle h, int32_t *entries);
nd_status nd_tune_save(nd_handle h, const char *path);
nd_status nd_tune_load(nd_handle h, const char *path);   /* merges; ND_ERR_ARG on a malformed file */

/* ---- CUDA graphs ---------------------------------------------------------
 * Capture the handle's stream into a graph (a sweep step) and replay it. */
nd_status nd_graph_begin(nd_handle h);
nd_status nd_graph_end(nd_handle h, void **graph_exec);
nd_status nd_graph_launch(nd_handle h, void *graph_exec);
nd_status nd_graph_destroy(void *graph_exec);

#ifdef __cplusplus
}
#endif
#endif /* NDTENSORS_GB300_H */
