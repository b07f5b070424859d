/* mpsgb300 — C ABI of the GB300 block-sparse U(1) tensor library.
 *
 * The entry points replace the SymTensors / TensorNetAlgs functions of amiragha/mps on the
 * 2-site DMRG hot path.  Each declaration cites the reference routine it stands in for (paths
 * relative to the reference project root).  A Julia `ccall` binding and a Python ctypes binding
 * map these one to one.
 *
 * Conventions
 *   - Every function returns an int status: 0 = success, otherwise one of MPSG_ERR_*;
 *     mpsg_last_error() returns the message of the last failure on the calling thread.
 *   - Leg positions are 1-based and contraction index tuples are ncon-style (negative labels are
 *     contracted, positive labels give the output leg order), exactly as in the reference.
 *   - A leg space is passed as parallel arrays: `nsect[l]` charges for leg l, then the charges
 *     and dims of all legs concatenated, and `isdual[l]`.
 *   - Tensor data crosses the boundary as one flat float64 array: blocks in reference sector order
 *     (column-major sector order, last leg slowest, src/sector.jl:35-36), each block
 *     column-major, blocks concatenated (mpsg_tensor_sectors gives the offsets).
 *   - `precision` selects the block-GEMM arithmetic: 0 = FP64 (the plain drop-in);
 *     s >= 2 = split precision with s bf16 slices per operand, FP32 accumulation in tensor memory
 *     and an FP64 epilogue.
 *   - All work is ordered on the context's CUDA stream; calls that return host values
 *     synchronise that stream.
 */
#ifndef MPSGB300_H
#define MPSGB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPSG_OK 0
#define MPSG_ERR_ARGUMENT 1
#define MPSG_ERR_SPACE_MISMATCH 2   /* reference: SpaceMismatch / SectorMismatch / error() */
#define MPSG_ERR_CUDA 3
#define MPSG_ERR_NO_CONVERGENCE 4
#define MPSG_ERR_UNSUPPORTED 5
#define MPSG_ERR_TOLERANCE 6        /* reference: "largest singular value is smaller than tol" */

typedef struct mpsg_ctx mpsg_ctx;
typedef struct mpsg_tensor mpsg_tensor;

/* ---- library and context ---------------------------------------------------------------- */
int mpsg_version(void);
const char* mpsg_last_error(void);
/* Context = one device + one CUDA stream + plan caches.  No reference counterpart (the
 * reference is single-threaded host code, src/TensorNetAlgs.jl). */
int mpsg_ctx_create(int device, mpsg_ctx** out);
int mpsg_ctx_destroy(mpsg_ctx* ctx);
int mpsg_ctx_synchronize(mpsg_ctx* ctx);
/* Counters: kernels launched by this library and algorithmic block-GEMM flops issued. */
int mpsg_ctx_counters(mpsg_ctx* ctx, int64_t* kernel_launches, double* gemm_flops);
int mpsg_ctx_clear_caches(mpsg_ctx* ctx);
/* Debug library only (libmpsgb300_checked.so, built with MPSG_DEVICE_CHECKS): the copy kernel
 * recomputes every block offset it decodes by plain division, checks every address against its
 * task's span, and records a violation instead of making the access (no counterpart in the
 * reference, whose arrays are bounds-checked by Julia). Returns the violations since the last
 * reset and the first one as {kind (1 task lookup, 2 decode, 3 span), task, index, detail};
 * reset = 1 clears them. The normal library returns MPSG_ERR_UNSUPPORTED. */
int mpsg_device_checks(mpsg_ctx* ctx, int32_t reset, int64_t* violations, int64_t* first);
/* The context's cudaStream_t, so callers can order their own work (or events) with it. */
int mpsg_ctx_stream(mpsg_ctx* ctx, void** stream);
/* Per-kernel CUDA-event timing: when enabled, every launch of kernel class `kind`
 * (0 = block-permute copy, 1 = FP64 block GEMM, 2 = split-precision block GEMM,
 *  3 = split-precision operand packing, 4 = vector ops) is bracketed by events on the context
 * stream; mpsg_ctx_kernel_time synchronises and returns the summed milliseconds, launch
 * count and algorithmic flops (GEMM classes) since the last reset. */
int mpsg_ctx_set_timing(mpsg_ctx* ctx, int32_t enable);
int mpsg_ctx_kernel_time(mpsg_ctx* ctx, int32_t kind, double* total_ms, int64_t* launches,
                         double* flops);

/* ---- tensors (src/symtensor.jl:12-30; constructors :132-191) ----------------------------- */
/* Zero-filled tensor holding every allowed sector of (charge, space)  (fill, symtensor.jl:157). */
int mpsg_tensor_create(mpsg_ctx* ctx, int32_t charge, int32_t nlegs, const int32_t* nsect,
                       const int32_t* charges, const int64_t* dims, const int32_t* isdual,
                       mpsg_tensor** out);
int mpsg_tensor_free(mpsg_tensor* t);
int mpsg_tensor_rank(const mpsg_tensor* t, int32_t* nlegs);
int mpsg_tensor_charge(const mpsg_tensor* t, int32_t* charge);
int mpsg_tensor_numel(const mpsg_tensor* t, int64_t* nblocks, int64_t* nelem);
int mpsg_tensor_is_diagonal(const mpsg_tensor* t, int32_t* isdiag);
/* Leg space `leg` (1-based): call once with charges=dims=NULL to get nsect. */
int mpsg_tensor_space(const mpsg_tensor* t, int32_t leg, int32_t* nsect, int32_t* charges,
                      int64_t* dims, int32_t* isdual);
/* Sector labels [nblocks*nlegs], block sizes [nblocks*nlegs], offsets [nblocks] (any may be
 * NULL).  Order = SortedDict order of the reference (src/sorteddict.jl:39-45). */
int mpsg_tensor_sectors(const mpsg_tensor* t, int32_t* labels, int64_t* sizes, int64_t* offsets);
int mpsg_tensor_upload(mpsg_tensor* t, const double* host, int64_t nelem);
int mpsg_tensor_download(const mpsg_tensor* t, double* host, int64_t nelem);
/* Raw device pointer of the flat buffer (for callers that keep data resident). */
int mpsg_tensor_device_ptr(const mpsg_tensor* t, double** dptr);
int mpsg_tensor_copy(mpsg_ctx* ctx, const mpsg_tensor* t, mpsg_tensor** out);
/* ---- asynchronous host copies (src/dmrg_envio.jl:5-261 keeps environments in files and
 * moves them with @async tasks; here they move between HBM and pinned host memory on the
 * context's copy stream while the context stream computes) -------------------------------- */
typedef struct mpsg_copy mpsg_copy;
/* Page-locked host memory for nelem doubles (the copies below overlap compute only from it). */
int mpsg_host_alloc(int64_t nelem, double** host);
int mpsg_host_free(double* host);
/* Starts t -> host (download) or host -> t (upload) after the work queued so far on the
 * context stream; t must belong to ctx and nelem must equal its size. The copy holds t's device
 * memory until it completes, so t may be freed at once. host must stay valid until the copy
 * completes. Context-stream work that reads an uploaded t must come after mpsg_copy_wait. */
int mpsg_tensor_download_async(mpsg_ctx* ctx, const mpsg_tensor* t, double* host, int64_t nelem,
                               mpsg_copy** copy);
int mpsg_tensor_upload_async(mpsg_ctx* ctx, mpsg_tensor* t, const double* host, int64_t nelem,
                             mpsg_copy** copy);
/* Orders the context stream after the copy without waiting on the host. */
int mpsg_copy_wait(mpsg_ctx* ctx, mpsg_copy* copy);
/* *done = 1 once the copy has completed, else 0. */
int mpsg_copy_query(mpsg_copy* copy, int32_t* done);
/* Waits on the host until the copy has completed. */
int mpsg_copy_synchronize(mpsg_copy* copy);
/* Releases the handle (waiting on the host first if the copy is still running). */
int mpsg_copy_free(mpsg_copy* copy);
/* dual(A): negated charge, flipped leg flags, same blocks (symtensor.jl:201-212). */
int mpsg_dual(mpsg_ctx* ctx, const mpsg_tensor* a, mpsg_tensor** out);

/* ---- releg (src/symreleg.jl) -------------------------------------------------------------- */
int mpsg_permutelegs(mpsg_ctx* ctx, const mpsg_tensor* a, const int32_t* perm,
                     mpsg_tensor** out);                                   /* :34-51   */
int mpsg_fuselegs(mpsg_ctx* ctx, const mpsg_tensor* a, int32_t l, int32_t n, int32_t dual,
                  mpsg_tensor** out);                                      /* :79-146  */
int mpsg_splitleg(mpsg_ctx* ctx, const mpsg_tensor* a, int32_t l, int32_t nspaces,
                  const int32_t* nsect, const int32_t* charges, const int64_t* dims,
                  const int32_t* isdual, mpsg_tensor** out);               /* :160-214 */

/* ---- contraction (src/contract.jl) -------------------------------------------------------- */
int mpsg_symmatrix(mpsg_ctx* ctx, const mpsg_tensor* a, int32_t nrows, const int32_t* rows,
                   int32_t ncols, const int32_t* cols, mpsg_tensor** out); /* :112-171 */
int mpsg_matmul(mpsg_ctx* ctx, const mpsg_tensor* a, const mpsg_tensor* b, int32_t precision,
                mpsg_tensor** out);                                        /* :234-298 */
/* contract(A, idxA, B, idxB) (:11-47).  When every leg is contracted the result is the scalar in
 * *scalar and *out is set to NULL. */
int mpsg_contract(mpsg_ctx* ctx, const mpsg_tensor* a, const int32_t* idxa, const mpsg_tensor* b,
                  const int32_t* idxb, int32_t precision, mpsg_tensor** out, double* scalar);
/* contract for complex operands held as real and imaginary parts (a = ar + i sa ai, b = br +
 * i sb bi; ai or bi may be NULL for a real operand; sa, sb = +-1 fold a conjugation in): up to
 * four real contractions on one plan, combined in place, so c = cr + i ci (ci NULL when both
 * operands are real). A full contraction returns the complex number in scalar_re, scalar_im with
 * cr = ci = NULL. For the complex MPS of time evolution (src/tdvp.jl, whose @tensor contractions
 * this replaces). */
int mpsg_contract_complex(mpsg_ctx* ctx, const mpsg_tensor* ar, const mpsg_tensor* ai,
                          double sa, const int32_t* idxa, const mpsg_tensor* br,
                          const mpsg_tensor* bi, double sb, const int32_t* idxb,
                          int32_t precision, mpsg_tensor** cr, mpsg_tensor** ci,
                          double* scalar_re, double* scalar_im);
/* The same FP64 contraction into a caller-provided result, allocating no device memory (no
 * counterpart in the reference). For hosts that cannot let a library allocate during a call,
 * e.g. one that handed the GPU's memory to its own arena up front. `out` must already exist
 * with the result's charge and spaces (MPSG_ERR_SPACE_MISMATCH otherwise) and must not share
 * storage with a or b. Every temporary lives in one fixed 64 MiB device array that each GPU
 * loading the library holds until exit; a contraction needing more is rejected with
 * MPSG_ERR_UNSUPPORTED, a fully contracted (scalar) one too. The first call on a device looks
 * up that array's address: make it before any stream capture. Calls share the array, so calls
 * whose kernels overlap on the GPU (different streams or contexts of one device) race; calls
 * on one context are ordered. a, b and out must belong to ctx (MPSG_ERR_ARGUMENT otherwise).
 * Each call plans on the host, stages its task tables and waits for ctx's stream: in a loop it
 * costs that host work and one synchronisation per call, which mpsg_contract's cached plans do
 * not. Returns when the result is complete. */
int mpsg_contract_noalloc(mpsg_ctx* ctx, const mpsg_tensor* a, const int32_t* idxa,
                          const mpsg_tensor* b, const int32_t* idxb, mpsg_tensor* out);
/* Algorithmic flops of contract(A, idxA, B, idxB) as planned (sum of 2*M*N*K over sectors). */
int mpsg_contract_flops(mpsg_ctx* ctx, const mpsg_tensor* a, const int32_t* idxa,
                        const mpsg_tensor* b, const int32_t* idxb, double* flops);

/* ---- effective Hamiltonian and environments (src/apply.jl) -------------------------------- */
int mpsg_applymps2site(mpsg_ctx* ctx, const mpsg_tensor* v, const mpsg_tensor* envl,
                       const mpsg_tensor* envr, const mpsg_tensor* w1, const mpsg_tensor* w2,
                       int32_t precision, mpsg_tensor** out);              /* :93-105 */
/* _applymps2site from host arrays to a host array (no reference counterpart: the reference's
 * data lives on the host). hv, henvl, henvr, hw1, hw2 hold the flat data of v, envl, envr, w1,
 * w2 (each tensor's element count), which are overwritten with it; the result's flat data is
 * written to hout (v's element count) and, if out is not NULL, returned as a device tensor too.
 * The uploads run on a copy stream while the operator is prepared: each W fold starts once its
 * two inputs have arrived. Pinned host memory makes the copies asynchronous. Returns when hout
 * is complete. */
int mpsg_applymps2site_host(mpsg_ctx* ctx, mpsg_tensor* v, mpsg_tensor* envl, mpsg_tensor* envr,
                            mpsg_tensor* w1, mpsg_tensor* w2, const double* hv,
                            const double* henvl, const double* henvr, const double* hw1,
                            const double* hw2, int32_t precision, double* hout,
                            mpsg_tensor** out);
int mpsg_applymps2site_flops(mpsg_ctx* ctx, const mpsg_tensor* v, const mpsg_tensor* envl,
                             const mpsg_tensor* envr, const mpsg_tensor* w1,
                             const mpsg_tensor* w2, double* flops);
int mpsg_mpsupdateleft(mpsg_ctx* ctx, const mpsg_tensor* env, const mpsg_tensor* a,
                       const mpsg_tensor* w, int32_t precision, mpsg_tensor** out); /* :49-58 */
int mpsg_mpsupdateright(mpsg_ctx* ctx, const mpsg_tensor* env, const mpsg_tensor* a,
                        const mpsg_tensor* w, int32_t precision, mpsg_tensor** out); /* :17-25 */

/* ---- factorisations and the Krylov solver -------------------------------------------------- */
/* _svd_(A) on a rank-2 tensor (src/symtools.jl:1-35): per-sector thin SVD; S is returned as a
 * diagonal tensor (dense diagonal blocks, mpsg_tensor_is_diagonal = 1). */
int mpsg_svd(mpsg_ctx* ctx, const mpsg_tensor* a, mpsg_tensor** u, mpsg_tensor** s,
             mpsg_tensor** v);
/* svdtrunc(A; maxdim, tol) (src/mpsutils.jl:116-179): keeps the maxdim largest singular values
 * above the ABSOLUTE tol across all sectors, ties to the first sector (:89-112); tieband > 0
 * treats values within tieband*max as equal (0 = the reference rule). */
int mpsg_svdtrunc(mpsg_ctx* ctx, const mpsg_tensor* a, int64_t maxdim, double tol,
                  double tieband, mpsg_tensor** u, mpsg_tensor** s, mpsg_tensor** v);
/* svdtrunc by the density-matrix method (no counterpart in the reference; same truncation rule
 * and output spaces as mpsg_svdtrunc). Per sector, the FP64 eigen-decomposition of A A^T
 * (side 0: u orthonormal) or A^T A (side 1: v orthonormal) replaces the SVD; the other factor is
 * S^-1 times the projection of A, so u*s*v equals the projection of A on the kept singular
 * subspace. Singular values carry an absolute error of about eps * max(S)^2 / S. For sweeps,
 * which keep the orthonormal side as the new site tensor and absorb s*v (or u*s) into the next. */
int mpsg_svdtrunc_gram(mpsg_ctx* ctx, const mpsg_tensor* a, int64_t maxdim, double tol,
                       double tieband, int32_t side, mpsg_tensor** u, mpsg_tensor** s,
                       mpsg_tensor** v);
/* Complex _svd_ / svdtrunc for the complex MPS of time evolution (the reference factorises dense
 * complex site tensors in src/tdvp.jl:35,61,132,165,195 with LAPACK; here per sector). The matrix is
 * a_re + i a_im (same charge and spaces); the results are u = u_re + i u_im (isometric columns),
 * s (real, diagonal) and v = v_re + i v_im holding V^H, so that A = u s v per sector. truncate = 0
 * keeps every singular value (_svd_); otherwise the rule of mpsg_svdtrunc applies. */
int mpsg_svd_complex(mpsg_ctx* ctx, const mpsg_tensor* a_re, const mpsg_tensor* a_im,
                     int32_t truncate, int64_t maxdim, double tol, double tieband,
                     mpsg_tensor** u_re, mpsg_tensor** u_im, mpsg_tensor** s,
                     mpsg_tensor** v_re, mpsg_tensor** v_im);
/* truncatedsizes (src/mpsutils.jl:89-112) on host arrays: nsect sectors, lens[i] descending values
 * each, concatenated in `values`; writes the kept count per sector to ns. */
int mpsg_truncatedsizes(int32_t nsect, const int64_t* lens, const double* values, int64_t maxdim,
                        double tol, double tieband, int64_t* ns);
/* Symmetric eigen-decomposition of a small dense column-major n x n matrix (ascending). */
int mpsg_small_eigh(int32_t n, const double* a, double* evals, double* evecs);
/* eigsolve(v -> _applymps2site(v, envL, envR, W1, W2), x0, 1, :SR, ishermitian=true; tol,
 * krylovdim, maxiter) (src/dmrg.jl:77-82, KrylovKit Lanczos): lowest eigenpair.  Returns
 * MPSG_OK also when not converged after maxiter restarts (the reference only warns);
 * *converged reports it. */
int mpsg_eigsolve_heff2(mpsg_ctx* ctx, const mpsg_tensor* x0, const mpsg_tensor* envl,
                        const mpsg_tensor* envr, const mpsg_tensor* w1, const mpsg_tensor* w2,
                        int32_t krylovdim, int32_t maxiter, double tol, int32_t precision,
                        double* eigenvalue, mpsg_tensor** eigenvector, double* normres,
                        int32_t* numiter, int32_t* numops, int32_t* converged);

/* ---- structure-only planning (no device memory; usable on hosts without a GPU) ---------- */
/* A structure-only tensor carries charge, spaces and the sector table but no data; every
 * mpsg_plan_* call returns the structure the matching operation would produce, computed by the
 * same planner that drives the kernels.  Query them with mpsg_tensor_space/_sectors/_numel. */
int mpsg_meta_create(int32_t charge, int32_t nlegs, const int32_t* nsect, const int32_t* charges,
                     const int64_t* dims, const int32_t* isdual, mpsg_tensor** out);
int mpsg_plan_permutelegs(const mpsg_tensor* a, const int32_t* perm, mpsg_tensor** out);
int mpsg_plan_fuselegs(const mpsg_tensor* a, int32_t l, int32_t n, int32_t dual,
                       mpsg_tensor** out);
int mpsg_plan_splitleg(const mpsg_tensor* a, int32_t l, int32_t nspaces, const int32_t* nsect,
                       const int32_t* charges, const int64_t* dims, const int32_t* isdual,
                       mpsg_tensor** out);
int mpsg_plan_symmatrix(const mpsg_tensor* a, int32_t nrows, const int32_t* rows, int32_t ncols,
                        const int32_t* cols, mpsg_tensor** out);
int mpsg_plan_matmul(const mpsg_tensor* a, const mpsg_tensor* b, mpsg_tensor** out,
                     double* flops);
/* *out is NULL for a full contraction (scalar result). */
int mpsg_plan_contract(const mpsg_tensor* a, const int32_t* idxa, const mpsg_tensor* b,
                       const int32_t* idxb, mpsg_tensor** out, double* flops);
/* Sector GEMM shapes (M, N, K per GEMM, 3*count values) of contract(A, idxA, B, idxB); call
 * with mnk = NULL to get the count (diagnostics and tile tuning). */
int mpsg_plan_contract_gemms(const mpsg_tensor* a, const int32_t* idxa, const mpsg_tensor* b,
                             const int32_t* idxb, int64_t* count, int64_t* mnk);
/* Number of copy tasks and GEMM tasks the planner emits for contract (diagnostics). */
int mpsg_plan_contract_tasks(const mpsg_tensor* a, const int32_t* idxa, const mpsg_tensor* b,
                             const int32_t* idxb, int64_t* copy_tasks, int64_t* gemm_tasks);

/* ---- prepared two-site effective Hamiltonian ---------------------------------------------- */
/* The matvec closure v -> _applymps2site(v, envL, envR, W1, W2) of src/dmrg.jl:77 as an object
 * that is built once per bond and applied many times.  precision 0 runs the reference's four
 * FP64 contractions; precision S >= 2 folds W1 into envL and W2 into envR once and applies
 * H_eff as two split-precision tensor-core GEMMs whose constant operands are sliced once. */
typedef struct mpsg_heff mpsg_heff;
int mpsg_heff2_create(mpsg_ctx* ctx, const mpsg_tensor* v_like, const mpsg_tensor* envl,
                      const mpsg_tensor* envr, const mpsg_tensor* w1, const mpsg_tensor* w2,
                      int32_t precision, mpsg_heff** out);
int mpsg_heff2_apply(mpsg_ctx* ctx, mpsg_heff* op, const mpsg_tensor* v, mpsg_tensor** out);
/* Algorithmic flops of one application in the reference contraction order. */
int mpsg_heff2_flops(const mpsg_heff* op, double* flops);
/* Algorithmic bytes per application of a prepared split-precision operator: block-permute
 * copies (8 read + 8 written per element moved) and operand packing (exponent pass 8 read, slice
 * pass 8 read + 2 S written per element); 0 for precision 0. For HBM rooflines of those kernels. */
int mpsg_heff2_traffic(const mpsg_heff* op, double* copy_bytes, double* pack_bytes);
int mpsg_heff2_free(mpsg_heff* op);

/* ---- many independent chains at once (no counterpart in the reference, which runs one DMRG
 * chain per process: src/dmrg.jl:58-179) --------------------------------------------------- */
/* The two-site H_eff of n chains (any structures, one slice count `precision` = 2..7) prepared
 * together: every phase of an application (block copies, operand packing, the two sector-GEMM
 * stages) is one launch over all chains, the split GEMMs one persistent grouped launch each
 * over every chain's sector problems. Kernel tile shape and tile order come from the tuner
 * (mpsg_ctx_tuner; on unless MPSG_AUTOTUNE=0). With use_graph != 0 the application is captured
 * in a CUDA graph at its second use and replayed after that. The work runs on ctx's stream;
 * operands may belong to other contexts of the same device (one per chain) once their
 * producers have finished (synchronise those contexts first). */
typedef struct mpsg_heff_batch mpsg_heff_batch;
int mpsg_heff2_batch_create(mpsg_ctx* ctx, int32_t n, const mpsg_tensor* const* v_like,
                            const mpsg_tensor* const* envl, const mpsg_tensor* const* envr,
                            const mpsg_tensor* const* w1, const mpsg_tensor* const* w2,
                            int32_t precision, int32_t use_graph, mpsg_heff_batch** out);
/* One chain's share of a batch, prepared on that chain's own context (plans and the FP64 W
 * folds; no split-precision packing of its own): usable only in mpsg_heff2_batch_from. */
int mpsg_heff2_prepare(mpsg_ctx* ctx, const mpsg_tensor* v_like, const mpsg_tensor* envl,
                       const mpsg_tensor* envr, const mpsg_tensor* w1, const mpsg_tensor* w2,
                       int32_t precision, mpsg_heff** out);
/* The batch of n prepared operators (any contexts of ctx's device, all preparations finished,
 * e.g. their contexts synchronised): their host work is already done, so assembling the batch
 * on ctx is concatenation, one copy of the constant operands and one packing. The operators
 * may be freed once this returns. */
int mpsg_heff2_batch_from(mpsg_ctx* ctx, int32_t n, const mpsg_heff* const* ops,
                          int32_t use_graph, mpsg_heff_batch** out);
/* out[i] = H_eff_i(v[i]) for every chain, in one batched application. */
int mpsg_heff2_batch_apply(mpsg_heff_batch* b, const mpsg_tensor* const* v, mpsg_tensor** out);
/* mpsg_eigsolve_heff2 for every chain from x0[i] (at most 128 chains), the Lanczos recurrences
 * run in lock step: one batched application per Krylov step and a fixed number of launches
 * for all chains' vector updates. Outputs are arrays of n (normres .. converged may be NULL). */
int mpsg_heff2_batch_eigsolve(mpsg_heff_batch* b, const mpsg_tensor* const* x0, int32_t krylovdim,
                              int32_t maxiter, double tol, double* eigenvalues,
                              mpsg_tensor** eigenvectors, double* normres, int32_t* numiter,
                              int32_t* numops, int32_t* converged);
/* Reference 4-step flops of one batched application, kernels per graph replay (0 before the
 * graph exists), applications so far, and the tuned configuration tuning[4] = (N tile, tile
 * order) of the first and of the second GEMM stage (N tile 0 = the kernel's default). */
int mpsg_heff2_batch_info(const mpsg_heff_batch* b, double* ref_flops, int64_t* graph_kernels,
                          int64_t* applies, int32_t* tuning);
int mpsg_heff2_batch_free(mpsg_heff_batch* b);
/* Split-GEMM tuner of the context: enable = 1 / 0 switches tuning of single prepared operators
 * on / off (-1 leaves it); runs = shape classes timed so far, hits = choices served from the
 * context's table. */
int mpsg_ctx_tuner(mpsg_ctx* ctx, int32_t enable, int64_t* runs, int64_t* hits);
/* Fixes the split-GEMM configuration of plans built from now on in this context: N tile bn (64,
 * 128, or 0 = the kernel's default for the slice count; 128 falls back to the default where it
 * does not fit), tile order (0 = decreasing K, 1 = problem by problem) and split-K (1: the
 * longest tiles halved along K while there are fewer than two waves of tiles; exact mode);
 * bn < 0 returns to the tuner / defaults. For measurements and tests. */
int mpsg_ctx_set_split_tuning(mpsg_ctx* ctx, int32_t bn, int32_t order, int32_t splitk);
/* Host self-check of the tensor-core H_eff plans for these structures (any tensors, also
 * structure-only ones): every copy and GEMM window in bounds, every output element written
 * once, and the composed intermediate copy equal to the two-step copy. */
int mpsg_plan_heff2_check(const mpsg_tensor* v, const mpsg_tensor* envl, const mpsg_tensor* envr,
                          const mpsg_tensor* w1, const mpsg_tensor* w2);

/* ---- vector operations used by the Krylov solver (src/symtensor.jl:252-323) -------------- */
int mpsg_fill(mpsg_ctx* ctx, mpsg_tensor* a, double x);                          /* :166-171 */
int mpsg_rmul(mpsg_ctx* ctx, mpsg_tensor* a, double alpha);                      /* :280-285 */
int mpsg_mul(mpsg_ctx* ctx, mpsg_tensor* b, const mpsg_tensor* a, double alpha); /* :268-276 */
int mpsg_axpy(mpsg_ctx* ctx, double alpha, const mpsg_tensor* a, mpsg_tensor* b); /* :288-296 */
int mpsg_axpby(mpsg_ctx* ctx, double alpha, const mpsg_tensor* a, double beta,
               mpsg_tensor* b);                                                  /* :299-308 */
int mpsg_dot(mpsg_ctx* ctx, const mpsg_tensor* a, const mpsg_tensor* b, double* out); /* :314 */
/* n dot products in one call, one synchronisation: out[i] = dot(a[i], b[i]), each pair similar.
 * For Krylov bases, whose reorthogonalisation takes one dot per basis vector (KrylovKit's
 * orthogonalizers behind eigsolve / exponentiate, src/tdvp.jl:27 and dmrg.jl:77). */
int mpsg_dots(mpsg_ctx* ctx, int32_t n, const mpsg_tensor* const* a,
              const mpsg_tensor* const* b, double* out);
/* out <- sum_i c[i] * x[i] over n tensors similar to out, in one launch (out may be one of the
 * x[i]): the multi-term axpy of the same reorthogonalisations (symtensor.jl:288-308 applied
 * term by term in the reference). */
int mpsg_lincomb(mpsg_ctx* ctx, int32_t n, const double* c, const mpsg_tensor* const* x,
                 mpsg_tensor* out);
int mpsg_norm(mpsg_ctx* ctx, const mpsg_tensor* a, double* out);                 /* :321-323 */

#ifdef __cplusplus
}
#endif

#endif /* MPSGB300_H */
