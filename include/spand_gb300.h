/*
 * spand_gb300.h -- C ABI of the GB300 spaND factorization and solve.
 *
 * This is the drop-in boundary for the reference's Tree::partition / assemble /
 * factorize / solve (leopoldcambier/spaND_public include/tree.h) and its CG driver
 * (include/is.h).  Plain pointers and sizes only: column-major dense data, CSC sparse
 * matrices with 0-based sorted int32 row indices, FP64 vectors.  Every function
 * returns a spand_status; spand_last_error() returns the message of the last failure
 * on the calling thread.  No function aborts or traps.
 *
 * Threading: one spand_tree is used by one thread at a time (the reference Tree is not
 * re-entrant either: solve() mutates the cluster vectors, include/tree.h:192).
 */
#ifndef SPAND_GB300_H
#define SPAND_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SPAND_OK = 0,
    SPAND_ERR_ARG = 1,            /* invalid argument */
    SPAND_ERR_STATE = 2,          /* call out of order (e.g. solve before factorize) */
    SPAND_ERR_CUDA = 3,           /* CUDA runtime failure */
    SPAND_ERR_NOT_SPD = 4,        /* failed pivot: the reference throws "Error: Non-SPD Pivot" (LLT, src/tree.cpp:587-590)
                                     or "Error: Singular Pivot" (PLU, src/tree.cpp:624-628) */
    SPAND_ERR_UNSUPPORTED = 5,    /* configuration not implemented on the device path */
    SPAND_ERR_NO_CONVERGENCE = 6
} spand_status;

typedef struct spand_tree spand_tree;
typedef struct spand_forest spand_forest;

/* Message of the last failing call on this thread ("" if none). */
const char* spand_last_error(void);

/* Tree(int lvl)                                    -- include/tree.h:173, src/tree.cpp:113 */
int spand_tree_create(spand_tree** out, int nlevels);
/* ~Tree()                                                                              */
int spand_tree_destroy(spand_tree* t);

/* Setters                                          -- include/tree.h:133-147            */
int spand_tree_set_verb(spand_tree* t, int verb);                   /* set_verb          */
int spand_tree_set_use_geo(spand_tree* t, int geo);                 /* set_use_geo       */
int spand_tree_set_Xcoo(spand_tree* t, const double* X, int dim, int n); /* set_Xcoo: dim x n col-major */
int spand_tree_set_tol(spand_tree* t, double tol);                  /* set_tol           */
int spand_tree_set_skip(spand_tree* t, int skip);                   /* set_skip          */
/* ScalingKind {SVD=0, PLU=1, PLUQ=2, EVD=3, LLT=4, LDLT=5} (include/spaND.h:19)         */
int spand_tree_set_scaling_kind(spand_tree* t, int kind);           /* set_scaling_kind  */
/* SymmKind {SPD=0, SYM=1, GEN=2} (include/spaND.h:21)                                   */
int spand_tree_set_symm_kind(spand_tree* t, int kind);              /* set_symm_kind     */
/* PartKind {MND=0, RB=1} (include/spaND.h:20)                                           */
int spand_tree_set_part_kind(spand_tree* t, int kind);              /* set_part_kind     */
int spand_tree_set_use_sparsify(spand_tree* t, int use);            /* set_use_sparsify  */
/* set_preserve / set_phi                           -- include/tree.h:136-137
 * Keep the columns of phi (n x nphi, column-major, natural ordering; copied) in the range
 * of every sparsification: the preconditioner then reproduces them exactly.  SPD and SYM
 * kinds only (factorize returns SPAND_ERR_ARG otherwise, or when phi has not N rows).    */
int spand_tree_set_preserve(spand_tree* t, int preserve);
int spand_tree_set_phi(spand_tree* t, const double* phi, int n, int nphi);
/* No reference counterpart: factor storage and arithmetic in FP32 (1) or FP64 (0).      */
int spand_tree_set_fp32(spand_tree* t, int fp32);

/* std::vector<ClusterID> partition(SpMat&)         -- include/tree.h:176, src/tree.cpp:306-419
 * A: n x n pattern in CSC.  sepids (optional, 6*n ints): per dof in natural ordering
 * self.lvl self.sep l.lvl l.sep r.lvl r.sep. */
int spand_tree_partition(spand_tree* t, int n, const int* colptr, const int* rowval, int* sepids);

/* void partition_lorasp(SpMat&)                    -- include/tree.h:177, src/tree.cpp:421-503
 * LoRaSp ordering: geometric recursive bisection (coordinates required).  parts (optional,
 * n ints): the part of every dof, natural ordering.  Then spand_tree_assemble and
 * spand_tree_factorize_lorasp (SPD / LLT). */
int spand_tree_partition_lorasp(spand_tree* t, int n, const int* colptr, const int* rowval, int* parts);

/* void assemble(SpMat&)                            -- include/tree.h:182, src/tree.cpp:505-575
 * Also builds the symbolic plan of the factorization and uploads the blocks. */
int spand_tree_assemble(spand_tree* t, int n, const int* colptr, const int* rowval, const double* vals);
/* No counterpart in the reference: assemble() again with new values on the pattern of the
 * last spand_tree_assemble (vals: nnz doubles in that matrix's CSC order; device memory
 * when on_device != 0).  The symbolic plan and the device work lists are reused: one copy
 * of the values and two scatter kernels (blocks, CSR).  SPAND_ERR_STATE before the first
 * assemble, SPAND_ERR_ARG when nnz differs. */
int spand_tree_assemble_values(spand_tree* t, const double* vals, long long nnz, int on_device);

/* void factorize()                                 -- include/tree.h:186, src/tree.cpp:1447-1551 */
int spand_tree_factorize(spand_tree* t);
/* void factorize_lorasp()                          -- include/tree.h:187, src/tree.cpp:1553-1608 */
int spand_tree_factorize_lorasp(spand_tree* t);

/* void solve(Eigen::VectorXd&) const               -- include/tree.h:192, src/tree.cpp:1610-1635
 * x: host buffer n x nrhs (leading dimension ld >= n), natural ordering, in place. */
int spand_tree_solve(spand_tree* t, double* x, int nrhs, int ld);
/* Same on a device buffer; runs on the tree's stream and returns without synchronising. */
int spand_tree_solve_device(spand_tree* t, double* x_dev, int nrhs, int ld);
/* No counterpart in the reference.  spand_tree_solve_device that allocates nothing: the
 * per-cluster solve vectors and their scratch copy live in a fixed 16 MiB device array
 * inside the library (a file-scope static __device__ array, held by every GPU that loads
 * the library until the process exits) instead of memory the tree allocates on its first
 * solve.  For callers that cannot call cudaMalloc when they solve: code that must stay
 * within a device-memory budget fixed in advance, and frameworks whose own allocator owns
 * the GPU's memory and must not be bypassed.  Limit: 2 * x_len * nrhs * sizeof(factor
 * type) <= 16 MiB, where x_len is the sum of all cluster capacities (about 3N for a 3D
 * grid; one right-hand side of a 64^3 problem fits in either precision); a larger request
 * returns SPAND_ERR_ARG before anything is touched, and its message states x_len.  The
 * first call on a device looks up the array's device address (cudaGetSymbolAddress, with
 * the tree's device current); make that first call before any stream capture.  Runs on the
 * tree's stream and returns without synchronising.  All calls share the array, which keeps
 * the last call's contents: allocation-free solves that overlap on the GPU race. */
int spand_tree_solve_device_noalloc(spand_tree* t, double* x_dev, int nrhs, int ld);

/* int cg(const SpMat&, const VectorXd& rhs, VectorXd& x, const Tree&, int iters, double tol, bool verb)
 *                                                  -- include/is.h:12, src/is.cpp:39-121
 * The matrix is the one given to assemble().  b, x: host vectors (x holds the initial
 * guess).  iters_out: the reference's return value (i+1); relres_out: |r|/|b| of the
 * recurrence residual. */
int spand_cg(spand_tree* t, const double* b, double* x, int iters, double tol, int verb, int* iters_out,
             double* relres_out);
/* Same with device vectors. */
int spand_cg_device(spand_tree* t, const double* b_dev, double* x_dev, int iters, double tol, int* iters_out,
                    double* relres_out);
/* gmres(A, rhs, x, precond, iters, restart, tol, verb) (include/is.h:13, src/is.cpp:123-300):
 * restarted GMRES with Householder Arnoldi, left preconditioned by the tree, on the device.
 * b, x: host vectors (x holds the initial guess); iters_out: the iteration count the
 * reference returns; relres_out: |w_k| / |M^{-1} r_0|, the quantity of its stopping test. */
int spand_gmres(spand_tree* t, const double* b, double* x, int iters, int restart, double tol, int verb,
                int* iters_out, double* relres_out);
/* Same with device vectors. */
int spand_gmres_device(spand_tree* t, const double* b_dev, double* x_dev, int iters, int restart, double tol,
                       int* iters_out, double* relres_out);
/* No counterpart in the reference: flexible (right-preconditioned) restarted GMRES.  Its
 * recurrence residual is the true |b - A x| whatever precision the factor is stored in, so
 * an FP32 factor (spand_tree_set_fp32) reaches an FP64 tolerance; stops when
 * |b - A x| < tol |b|, relres_out = that ratio.  Host vectors, x holds the initial guess. */
int spand_fgmres(spand_tree* t, const double* b, double* x, int iters, int restart, double tol, int verb,
                 int* iters_out, double* relres_out);
/* ir(A, rhs, x, precond, iters, tol, verb) (include/is.h:14, src/is.cpp:12-37): iterative
 * refinement x += M^{-1}(b - A x) on the device; relres_out = |b - A x| / |b|. */
int spand_ir(spand_tree* t, const double* b, double* x, int iters, double tol, int verb, int* iters_out,
             double* relres_out);
/* No counterpart in the reference: the adjoint of x = A^{-1} b.  lambda_dev = A^{-T} g_dev
 * (g = dL/dx; A SPD, so the PCG of spand_cg_device with the same factor), then
 * grad_vals_dev[k] = -lambda[row_k] * x[col_k] for every stored entry k of the assembled
 * pattern, in its CSC order (dL/dvalues; dL/db = lambda).  x_dev: the solution of the
 * forward solve.  Device vectors; lambda_dev holds the initial guess. */
int spand_adjoint_device(spand_tree* t, const double* g_dev, const double* x_dev, double* lambda_dev,
                         double* grad_vals_dev, int iters, double tol, int* iters_out, double* relres_out);
/* No counterpart in the reference: cg on nrhs right-hand sides at once.  Each column is an
 * independent CG with the reference's stopping rule (|r| < tol |b|); the columns advance in
 * lockstep so that one multi-right-hand-side preconditioner application, one SpMV and three
 * dots per iteration serve them all, and a converged column stops changing.  b, x: host
 * n x nrhs with leading dimension ld (x holds the initial guess); iters_out[nrhs] and
 * relres_out[nrhs] receive each column's iteration count and recurrence residual. */
int spand_cg_multi(spand_tree* t, const double* b, double* x, int nrhs, int ld, int iters, double tol,
                   int* iters_out, double* relres_out);
/* Same on device buffers (n x nrhs, leading dimension n); runs on the tree's stream and
 * returns after the last column converged (one host read per iteration for the test). */
int spand_cg_multi_device(spand_tree* t, const double* b_dev, double* x_dev, int nrhs, int iters, double tol,
                          int* iters_out, double* relres_out);

/* No counterpart in the reference: many independent systems at once (e.g. a batch of
 * small problems).  spand_batch_factorize queues every tree's factorization on its own
 * stream before it waits for any; status_out[count] receives each tree's status (the call
 * returns the first failure's status and message).  spand_batch_cg runs tree k's cg on
 * host vectors b[k] -> x[k] (its own size, x[k] holds the initial guess) for all trees in
 * lockstep, one host wait per iteration for the whole batch. */
int spand_batch_factorize(spand_tree* const* trees, int count, int* status_out);
int spand_batch_cg(spand_tree* const* trees, int count, const double* const* b, double* const* x, int iters,
                   double tol, int* iters_out, double* relres_out);
/* Same on device vectors b_dev[k] -> x_dev[k] (FP64, the tree's size; x_dev[k] holds the
 * initial guess); every system runs on its tree's stream and the call returns when all have converged or stopped. */
int spand_batch_cg_device(spand_tree* const* trees, int count, const double* const* b_dev, double* const* x_dev,
                          int iters, double tol, int* iters_out, double* relres_out);

/* No counterpart in the reference: a forest factors many independent SPD systems as ONE
 * block-diagonal matrix.  Each system keeps the ordering and cluster hierarchy of its
 * (partitioned, assembled) tree; level l of the forest is level l of every system, so each
 * launch of the factorization and of the solve carries the work of all systems, and one
 * segmented CG (per-system scalars and stopping tests) serves all right-hand sides.  The
 * trees share tolerance, skip, precision and sparsification setting; they are copied and
 * may be destroyed afterwards.  Vectors are stacked: system k at rows [off[k], off[k+1])
 * in its natural ordering; values stacked at [nnz_off[k], nnz_off[k+1]) in the CSC order
 * of its tree's pattern. */
int spand_forest_create(spand_forest** f, spand_tree* const* trees, int count);
int spand_forest_destroy(spand_forest* f);
/* off, nnz_off: count + 1 entries each (either may be NULL) */
int spand_forest_offsets(spand_forest* f, long long* off, long long* nnz_off);
int spand_forest_assemble_values(spand_forest* f, const double* vals, long long nnz, int on_device);
/* SPAND_ERR_NOT_SPD when a pivot fails; *failed_system: that system (-1: none) */
int spand_forest_factorize(spand_forest* f, int* failed_system);
int spand_forest_solve_device(spand_forest* f, double* x_dev);
/* cg (src/is.cpp:39-121) on every system: b, x stacked host vectors (x: initial guess);
 * iters_out[count], relres_out[count] per system */
int spand_forest_cg(spand_forest* f, const double* b, double* x, int iters, double tol, int* iters_out,
                    double* relres_out);
int spand_forest_cg_device(spand_forest* f, const double* b_dev, double* x_dev, int iters, double tol,
                           int* iters_out, double* relres_out);
/* 5 ints per sparsified cluster: system, level, cluster order in its tree, rows, rank */
int spand_forest_num_ranks(spand_forest* f, int* n);
int spand_forest_get_ranks(spand_forest* f, int* out);
int spand_forest_launches(spand_forest* f, long long* n, int reset);
/* per-kernel-class device time (CUDA events around every launch while on), as for trees */
int spand_forest_set_profiling(spand_forest* f, int on);
int spand_forest_profile_count(spand_forest* f, int* n);
int spand_forest_profile_entry(spand_forest* f, int idx, char* name, long long* launches, double* ms);
int spand_forest_profile_reset(spand_forest* f);

/* Introspection (reference: get_N, get_assembly_perm, nnz, get_stop, print_log fields;
 * include/tree.h:150-165, src/tree.cpp:1645-1727) */
int spand_tree_get_N(spand_tree* t, int* n);
int spand_tree_get_perm(spand_tree* t, int* perm);
int spand_tree_nnz(spand_tree* t, long long* nnz);
int spand_tree_get_stop(spand_tree* t, int* stop);
/* 11 values per level: dofs_nd dofs_left_nd dofs_left_elim dofs_left_spars rank_before_sum
 * rank_after_sum rank_after_count ignored nbrs_sum nbrs_count fact_nnz */
int spand_tree_level_log(spand_tree* t, long long* out);
/* (level, cluster order, rows, rank) per sparsified cluster */
int spand_tree_num_ranks(spand_tree* t, int* n);
int spand_tree_get_ranks(spand_tree* t, int* out);
/* Operation list in recording order: kind level self nbr ns nn rows cols (8 ints each);
 * kind: 0 ScalingLLT 1 GemmSymmOut 2 GemmSymmIn 3 Orthogonal 4 Merge 5 Split
 *       6 GemmOut 7 GemmIn 8 ScalingPLUQ (GEN / PLU; its matrix: L_s strictly below the
 *       diagonal, U_s on and above it) 9 ScalingLDLT (SYM / LDLT; L_s in the lower triangle) */
int spand_tree_num_ops(spand_tree* t, int* n);
int spand_tree_get_ops(spand_tree* t, int* out);
int spand_tree_get_op_matrix(spand_tree* t, int idx, double* out);
int spand_tree_get_op_tau(spand_tree* t, int idx, double* out);
/* row permutation p (ns entries) of a ScalingPLUQ / ScalingLDLT op: x_s <- x_s[p] before
 * L_s^{-1} */
int spand_tree_get_op_perm(spand_tree* t, int idx, int* out);
/* sign(D) (ns entries) of a ScalingLDLT op (SYM / LDLT path) */
int spand_tree_get_op_signs(spand_tree* t, int idx, double* out);
/* seconds: partition, assemble, factorize */
int spand_tree_timings(spand_tree* t, double* out);
/* kernels launched by this tree since the last reset */
int spand_tree_launches(spand_tree* t, long long* n, int reset);
int spand_tree_device_bytes(spand_tree* t, long long* bytes);

/* No reference counterpart -- measurement hooks used by bench.py:
 * one factorize() + device CG on device arrays b_dev / x_dev, n x nrhs with leading
 * dimension n (x_dev is zeroed first; nrhs > 1: the columns' CGs in lockstep, as in
 * spand_cg_multi_device), timed with CUDA events on the tree's stream.  out[4]: factor ms,
 * CG ms, iterations and |r|/|b| of the recurrence residual (largest over the columns). */
int spand_tree_bench_step(spand_tree* t, const double* b_dev, double* x_dev, int nrhs, int iters, double tol,
                          double* out);
/* Bytes uploaded by assemble() for the block values (the factorization's device input). */
int spand_tree_assembled_bytes(spand_tree* t, long long* bytes);
/* Per-kernel-class device time (CUDA events around every launch while enabled). */
int spand_tree_set_profiling(spand_tree* t, int on);
int spand_tree_profile_count(spand_tree* t, int* n); /* collects pending records */
int spand_tree_profile_entry(spand_tree* t, int idx, char* name64, long long* launches, double* ms);
int spand_tree_profile_reset(spand_tree* t);
/* Algorithmic bytes and flops per kernel class: which = 0 one factorization, 1 one solve. */
int spand_tree_work_count(spand_tree* t, int which, int* n);
int spand_tree_work_entry(spand_tree* t, int which, int idx, char* name64, double* bytes, double* flops);
/* The QRCP launch of every sparsification wave, in launch order (after a factorization).
 * conf9: level, wave, matrices, row capacity of the largest, blocked rows per lane (0: the
 * unblocked kernel), CTAs per cluster, threads per CTA, dynamic shared memory bytes, rows
 * from which the trailing update is vectorised (INT_MAX: never).  ncand: configurations
 * the measuring factorization timed for the wave (0 where none was measured); conf5 of
 * candidate k: blocked rows per lane, CTAs per cluster, threads, shared memory, vectorised
 * rows, with its measured time in ms. */
int spand_tree_qrcp_wave_count(spand_tree* t, int* n);
int spand_tree_qrcp_wave(spand_tree* t, int idx, int* conf9, int* ncand);
int spand_tree_qrcp_wave_candidate(spand_tree* t, int idx, int k, int* conf5, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* SPAND_GB300_H */
