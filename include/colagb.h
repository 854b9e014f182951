/*
 * colagb.h -- C ABI of libcolagb, the sm_103a implementation of CoLA's
 * iterative Krylov hot path (CG for solve/inv, Lanczos for eig, stochastic
 * Lanczos quadrature for logdet/trace) and of the structured matvecs those
 * loops call.
 *
 * Conventions
 *   - Every pointer to array data is a DEVICE pointer unless the comment says
 *     "host".  Nothing here takes or returns a framework tensor type.
 *   - A block of k vectors of length n ("n x k") is row-major with a leading
 *     dimension ld >= k: element (i, c) lives at X[i * ld + c].  This is the
 *     layout of CoLA's (n,) / (n, k) right-hand sides (cola/linalg/inverse/cg.py:59-64).
 *   - Every entry point returns an int status: COLAGB_OK (0) or an error code;
 *     colagb_last_error() gives a human readable message for the calling thread.
 *   - Work is enqueued on the caller's stream.  Entry points that must make a
 *     host decision (the CG / Lanczos stop rules) synchronise that stream.
 *   - Temporary device memory is supplied by the caller through a workspace
 *     pointer whose size comes from the matching *_workspace_bytes query; the
 *     library itself never allocates device memory on these paths.
 */
#ifndef COLAGB_H
#define COLAGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define COLAGB_OK 0
#define COLAGB_ERR_INVALID 1      /* bad argument: shape, dtype, null pointer  (Python: ValueError) */
#define COLAGB_ERR_CUDA 2         /* CUDA runtime error                        (Python: RuntimeError) */
#define COLAGB_ERR_TIMEOUT 3      /* a bounded device wait gave up             (Python: RuntimeError) */
#define COLAGB_ERR_UNSUPPORTED 4  /* operator / dtype combination not handled   (Python: NotImplementedError) */
#define COLAGB_ERR_WORKSPACE 5    /* workspace smaller than the query returned  (Python: ValueError) */

/* ---- element types ------------------------------------------------------ */
#define COLAGB_F32 0
#define COLAGB_F64 1
#define COLAGB_BF16 2

/* ---- per-system solver status (colagb_cg_batched_*) --------------------- */
#define COLAGB_SYS_RUNNING 0
#define COLAGB_SYS_CONVERGED 1
#define COLAGB_SYS_MAX_ITERS 2
#define COLAGB_SYS_BREAKDOWN 3    /* <p, A p> <= 0: operator not SPD in working precision */
#define COLAGB_SYS_NAN 4
#define COLAGB_SYS_FALLBACK 5     /* learned preconditioner stalled; finished with Jacobi */

const char* colagb_last_error(void);
/* Library version and the sm architecture it was built for (e.g. 1003 = sm_103a). */
int colagb_version(int32_t* version, int32_t* arch);

/* ======================================================================== *
 *  Operator programs                                                       *
 *  A LinearOperator tree (cola/ops/operators.py) lowered to a flat array   *
 *  of nodes.  The handle keeps a copy of the node array; the device arrays *
 *  it points to stay owned by the caller and must outlive the handle.      *
 * ======================================================================== */
#define COLAGB_OP_DENSE 1      /* Dense(A)                 operators.py:12-28   */
#define COLAGB_OP_CSR 2        /* Sparse(data, row, col)   operators.py:48-81   */
#define COLAGB_OP_DIAG 3       /* Diagonal(d)              operators.py:323-339 */
#define COLAGB_OP_SCALAR 4     /* ScalarMul(c) = c * I     operators.py:84-101  */
#define COLAGB_OP_IDENTITY 5   /* Identity / I_like        operators.py:104-136 */
#define COLAGB_OP_SUM 6        /* Sum(*Ms)                 operators.py:168-196 */
#define COLAGB_OP_PRODUCT 7    /* Product(*Ms)             operators.py:139-165 */
#define COLAGB_OP_KRON 8       /* Kronecker(*Ms)           operators.py:199-228 */
#define COLAGB_OP_BLOCKDIAG 9  /* BlockDiag(*Ms, mult)     operators.py:278-320 */

typedef struct colagb_op_node {
  int32_t kind;            /* COLAGB_OP_* */
  int32_t dtype;           /* storage type of data (DENSE values, CSR values, DIAG entries) */
  int64_t rows, cols;
  const void* data;        /* DENSE: row-major matrix; CSR: values[nnz]; DIAG: diagonal[rows] */
  int64_t ld;              /* DENSE: row stride in elements (>= cols) */
  const int32_t* indptr;   /* CSR: rows + 1 row offsets */
  const int32_t* indices;  /* CSR: nnz column indices */
  int64_t nnz;             /* CSR */
  double scalar;           /* SCALAR: c */
  const int32_t* children; /* host: indices of child nodes in the node array */
  int32_t num_children;
  const int64_t* multiplicities; /* host, BLOCKDIAG: one per child, NULL = all 1 */
  int32_t precision;       /* KRON: arithmetic of the factor contractions, COLAGB_KRON_* below */
  int32_t reserved;
  const int32_t* perm;     /* CSR (square), or NULL: the matrix is stored symmetrically permuted,
                              stored row / column r being original row / column perm[r] (a
                              bandwidth-reducing order); products gather x through perm and write
                              y through it, so the node still means the original matrix */
} colagb_op_node;

/* Kronecker contraction arithmetic (FP32 compute type; FP64 operators always use FP64 arithmetic).
 * AUTO: tensor cores with the three-product BF16 split (BF16X3) for contractions of at least 2^26
 * multiply-adds whose factor is Dense with at least 256 columns, FP32 SIMT otherwise.
 * BF16: one BF16 product per term (FP32 accumulation).  BF16X3: hi = bf16(v), lo = bf16(v - hi);
 * hi.hi + hi.lo + lo.hi in FP32 (about 2^-16 relative per product).  FP32: FP32 SIMT only. */
#define COLAGB_KRON_AUTO 0
#define COLAGB_KRON_FP32 1
#define COLAGB_KRON_BF16 2
#define COLAGB_KRON_BF16X3 3

typedef struct colagb_op colagb_op; /* opaque */

/* Build a handle for the operator rooted at nodes[root]. */
int colagb_op_create(const colagb_op_node* nodes, int32_t num_nodes, int32_t root, colagb_op** out);
int colagb_op_free(colagb_op* op);
/* Shape and compute type (COLAGB_F32 or COLAGB_F64) of the vectors the operator acts on. */
int colagb_op_info(const colagb_op* op, int64_t* rows, int64_t* cols, int32_t* compute_dtype);

/* Y = alpha * (op @ X) + beta * Y, X: cols x k, Y: rows x k, vector type = compute_dtype.
 * Replaces LinearOperator.__matmul__ -> _matmat (cola/ops/operator_base.py:97-106). */
int colagb_matmat_workspace_bytes(const colagb_op* op, int64_t k, size_t* bytes);
int colagb_matmat(const colagb_op* op, const void* X, int64_t ldx, void* Y, int64_t ldy, int64_t k,
                  double alpha, double beta, void* workspace, size_t workspace_bytes, void* stream);

/* Gradients with respect to the operator's own arrays: for Y = op(theta) X and a cotangent G
 * (rows x k, compute type), node_grads[i] += alpha * d<G, op(theta) X>/d data_i for every node i whose
 * node_grads entry (a HOST array of num_nodes device pointers, NULL = skip) is set: Dense (rows x cols,
 * contiguous), Sparse (nnz values) and Diagonal (rows) leaves stored in the compute type, through Sum /
 * ScalarMul / Identity compositions.  Product, Kronecker and BlockDiag trees: COLAGB_ERR_UNSUPPORTED.
 * Replaces the autograd of _matmat that cg_bwd and slq_bwd rely on (cola/linalg/inverse/cg.py:72-86,
 * cola/linalg/tbd/slq.py:10-31). */
int colagb_matmat_vjp(const colagb_op* op, const void* X, int64_t ldx, const void* G, int64_t ldg, int64_t k,
                      double alpha, void* const* node_grads, void* stream);

/* ======================================================================== *
 *  Conjugate gradients                                                     *
 *  Replaces cg() / run_batched_cg() / take_cg_step()                       *
 *  (cola/linalg/inverse/cg.py:39-178) and the while_loop_winfo driver      *
 *  (cola/utils/torch_tqdm.py:7-71).  Semantics follow the reference: each  *
 *  column of B is normalised by its norm, r0 = B/|B| - A X0, the loop runs *
 *  while any column has |r| > tol*|r0| + tol and k < max_iters, alpha and  *
 *  beta use the 1e-40 safe division and are zeroed once |r| < 1e-40, and   *
 *  the solution is scaled back by |B|.                                     *
 * ======================================================================== */
typedef struct colagb_cg_params {
  double tol;            /* CG(tol=...) */
  int32_t max_iters;     /* CG(max_iters=...) */
  int32_t check_every;   /* host polls the device stop flag every this many iterations (0 = 16) */
  int32_t allow_fused;   /* 1: use the single-launch persistent kernel when the operator allows it */
  int32_t graph;         /* multi-launch loop: 0 = capture one block of check_every steps as a CUDA graph
                            and replay it (when max_iters >= 2 * check_every); 1 = plain launches */
  int64_t spin_limit;    /* grid-barrier spin bound of the persistent kernel (0 = default) */
} colagb_cg_params;

typedef struct colagb_cg_result {
  int32_t iterations;    /* k, the number of CG steps taken (state[1] of run_batched_cg) */
  int32_t fused;         /* 1 if the persistent single-launch kernel ran */
  int32_t status;        /* COLAGB_OK or COLAGB_ERR_TIMEOUT */
  int32_t graph;         /* 1 if the multi-launch loop ran as replays of a captured CUDA graph */
} colagb_cg_result;

/* P may be NULL (identity).  X holds x0 on entry and the solution on exit.
 * residual_history (device, compute dtype, max_iters + 1 entries, may be NULL) receives
 * mean_c |r_c| (normalised scale) after each step, index 0 = initial residual; this is the
 * quantity the reference's info['errors'] records. */
int colagb_cg_workspace_bytes(const colagb_op* A, const colagb_op* P, int64_t k, size_t* bytes);
int colagb_cg_solve(const colagb_op* A, const colagb_op* P, const void* B, int64_t ldb, void* X, int64_t ldx,
                    int64_t k, const colagb_cg_params* params, void* residual_history,
                    void* workspace, size_t workspace_bytes, colagb_cg_result* result, void* stream);

/* colagb_cg_solve for callers that cannot allocate device memory -- for example a host runtime
 * that hands out only its own fixed pool, or code running where cudaMalloc is not allowed.  It takes
 * no workspace: its scratch is one fixed 8 MiB device array inside this library (every GPU that loads
 * the library keeps it until the process exits).  Problems whose colagb_cg_workspace_bytes exceeds
 * 8 MiB (roughly n*k above 600,000 in FP32 or 300,000 in FP64) are rejected with COLAGB_ERR_INVALID.
 * The array's device address belongs to the CUDA context current on the calling thread (the
 * device's primary context for runtime-API callers; the caller's own context if it pushed one).  The
 * first call in each context looks that address up and caches it under the context's unique id, so
 * a new context (a pushed driver context, or the primary context re-created after cudaDeviceReset)
 * gets its own lookup; make the first call in a context before any stream capture.  All calls in a
 * context share the array: calls whose GPU work overlaps (other streams, other threads) race and
 * corrupt each other's results.  This entry point has no counterpart in the reference; otherwise it
 * behaves exactly like colagb_cg_solve. */
int colagb_cg_solve_noalloc(const colagb_op* A, const colagb_op* P, const void* B, int64_t ldb, void* X,
                            int64_t ldx, int64_t k, const colagb_cg_params* params, void* residual_history,
                            colagb_cg_result* result, void* stream);

/* ------------------------------------------------------------------------ *
 *  Batched independent SPD systems sharing one CSR sparsity pattern        *
 *  (a family of discretised operators: same mesh, different coefficients). *
 *  S systems, each n x n with nnz entries; values[s * nnz + j].            *
 *  Solved to a TRUE relative residual |b - A x| / |b| <= tol measured in   *
 *  FP64, by FP32 preconditioned CG with FP64 iterative refinement: the     *
 *  solution accumulates in FP64 and the residual is replaced by the FP64   *
 *  b - A x whenever the FP32 residual has dropped by inner_tol.            *
 *  The reference solves such systems one call at a time                    *
 *  (cola/linalg/inverse/inv.py:66-69 per system); here one persistent      *
 *  launch per refinement sweep advances all of them with per-system        *
 *  convergence masks.                                                      *
 * ------------------------------------------------------------------------ */
#define COLAGB_PREC_NONE 0
#define COLAGB_PREC_JACOBI 1   /* CG(P=Diagonal(1/diag(A))) */
#define COLAGB_PREC_FSAI 2     /* P = G^T G, G lower triangular on A's lower pattern */

typedef struct colagb_batched_csr {
  int64_t n, nnz, num_systems;
  const int32_t* indptr;   /* n + 1 */
  const int32_t* indices;  /* nnz, sorted within each row */
  const float* values;     /* num_systems * nnz */
  /* FSAI factor G (only for COLAGB_PREC_FSAI): lower pattern and its transpose */
  int64_t g_nnz;
  const int32_t* g_indptr;    /* n + 1 */
  const int32_t* g_indices;   /* g_nnz */
  const int32_t* gt_indptr;   /* n + 1, pattern of G^T */
  const int32_t* gt_indices;  /* g_nnz */
  const int32_t* gt_perm;     /* g_nnz: G^T entry e holds G value gt_perm[e] */
  const float* g_values;      /* num_systems * g_nnz */
  int32_t shared_values;      /* 1: every system uses values[0 .. nnz) (one matrix, many right-hand sides) */
  int32_t reserved;
} colagb_batched_csr;

#define COLAGB_IR_RELIABLE 0   /* FP64 residual replacement, the CG recurrence continues (default) */
#define COLAGB_IR_RESTART 1    /* classic refinement: each FP64 residual starts a fresh inner CG */

typedef struct colagb_ir_params {
  double tol;            /* target true relative residual (FP64), e.g. 1e-8 */
  double inner_tol;      /* FP32 residual reduction between two FP64 residual replacements */
  int32_t max_sweeps;    /* FP64 residual replacements per system */
  int32_t max_inner_iters; /* CG iterations per system */
  int32_t preconditioner;/* COLAGB_PREC_* */
  int32_t fallback;      /* 1: a system whose FSAI-PCG stalls continues with Jacobi */
  int64_t spin_limit;    /* grid-barrier spin bound (0 = default) */
  int32_t mode;          /* COLAGB_IR_RELIABLE or COLAGB_IR_RESTART */
  int32_t schedule;      /* COLAGB_SCHED_* */
  int32_t no_wait;       /* 1: the on-chip and cluster schedules return once the solve is enqueued
                            (per-system outputs valid when the stream gets there, result->sweeps
                            = -1); 0: wait and report the largest replacement count.  The grid
                            schedule always waits (it reads its barrier-timeout flag). */
  int32_t matvec;        /* COLAGB_MATVEC_*: storage of A in the inner FP32 CG's matvec */
  int32_t spare;         /* COLAGB_SPARE_*: the on-chip schedule's use of the SMs its clusters leave free */
} colagb_ir_params;

/* The on-chip schedule's clusters occupy 16 SMs each (7 clusters = 112 of 152 SMs at 224 KB of shared
 * memory per CTA).  AUTO: one 512-thread CTA on each remaining SM also solves whole systems, with the
 * same algorithm, stop rule and outputs, its vectors in global memory (L2 evict-first, so that the
 * clusters' diagonal slots stay in L2); it claims systems from the same counter while more than ~28
 * per resident cluster remain unclaimed, so that the clusters (that much faster per system) finish the
 * tail.  Which kernel solved a system depends on timing, so the FP32 rounding of its iterates (not its
 * stop rule) can differ between runs.  OFF (0, the zero-initialised value): clusters only, the same
 * bits run to run.  ONLY: every system on those CTAs (a test and measurement mode).  The Python layer's
 * solve_batched asks for AUTO unless told otherwise. */
#define COLAGB_SPARE_OFF 0
#define COLAGB_SPARE_AUTO 1
#define COLAGB_SPARE_ONLY 2

/* Inner matvec storage.  FP32: the CSR values as given.  BF16 (cluster schedules only; AUTO then
 * picks the cluster schedule): off-diagonal values rounded to BF16 and a separate FP32 diagonal
 * d'_i = a_ii - sum_j (bf16(a_ij) - a_ij), so that A' - A = -1/2 sum_ij delta_ij (e_i - e_j)(e_i - e_j)^T.
 * For a weighted-Laplacian-type operator (off-diagonals <= 0, diagonal >= the row's off-diagonal sum)
 * this keeps A' within 2^-9 of A in the energy norm: |x^T (A' - A) x| <= 2^-9 x^T A x, whatever the
 * condition number, so the FP64 residual replacements converge.  The FP64 residual b - A x always
 * uses the FP32 values.  6 bytes per nonzero + 4 per row instead of 8 per nonzero. */
#define COLAGB_MATVEC_FP32 0
#define COLAGB_MATVEC_BF16 1

#define COLAGB_SCHED_AUTO 0     /* on-chip when the pattern allows it, else a cluster per system */
#define COLAGB_SCHED_GRID 1     /* one cooperative grid advancing every system together */
#define COLAGB_SCHED_CLUSTER8 2 /* one 8-CTA thread-block cluster per system */
#define COLAGB_SCHED_CLUSTER16 3/* one 16-CTA cluster per system (non-portable cluster size) */
#define COLAGB_SCHED_ONCHIP 4   /* one cluster per system with p, r and the FP32 correction held in the
                                   cluster's shared memory and the matrix in diagonal storage; needs a
                                   pattern of <= 9 constant-offset diagonals (FSAI: a lower G of <= 5),
                                   n <= 262144.  AUTO takes it whenever those hold. */
#define COLAGB_SCHED_BLOCK 5    /* shared-values families (one matrix, many right-hand sides): all
                                   right-hand sides advance in lockstep as the columns of one (n, k)
                                   block, so each step reads the matrix once for all of them (the
                                   reference's own multi-column CG layout); one cooperative grid; no
                                   FSAI, FP32 matvec.  AUTO takes it for shared-values families of at
                                   least 4 right-hand sides with those options. */

/* Geometry of the on-chip schedule for systems of n rows whose diagonals reach `halo` rows off the
 * main diagonal: info[0] cluster size (0: n too large), info[1] rows per CTA, info[2] clusters that
 * can be resident at once on this device (systems in flight), info[3] shared memory per CTA. */
int colagb_onchip_schedule_info(int64_t n, int32_t halo, int32_t* info);

typedef struct colagb_ir_result {
  int32_t sweeps;              /* largest FP64 residual replacement count (-1 with no_wait) */
  int32_t total_inner_iters;   /* sum over sweeps of the max inner iterations */
  int32_t status;              /* COLAGB_OK or COLAGB_ERR_TIMEOUT */
  int32_t schedule;            /* the COLAGB_SCHED_* that ran (AUTO resolved) */
  int32_t companion_systems;   /* systems solved by the on-chip schedule's companion CTAs (0 without
                                  them, -1 with no_wait) */
} colagb_ir_result;

/* B: num_systems x n FP64 right-hand sides; X: num_systems x n FP64 solutions (out).
 * per_system_iters / per_system_status / relres (device, may be NULL): inner iterations summed
 * over sweeps, COLAGB_SYS_* and the final FP64 true relative residual of each system. */
int colagb_cg_batched_csr_workspace_bytes(const colagb_batched_csr* A, const colagb_ir_params* params,
                                          size_t* bytes);
int colagb_cg_batched_csr_solve(const colagb_batched_csr* A, const double* B, double* X,
                                const colagb_ir_params* params, int32_t* per_system_iters,
                                int32_t* per_system_status, double* relres, void* workspace,
                                size_t workspace_bytes, colagb_ir_result* result, void* stream);

/* ------------------------------------------------------------------------ *
 *  Batched independent dense SPD systems of uneven sizes (FP32 CG), one    *
 *  persistent launch.  Each system behaves exactly like its own call of    *
 *  cola.linalg.solve(PSD(Dense(A_s)), b_s, CG(tol, max_iters))             *
 *  (cg.py:94-154), with its own stop test.  A_s is sizes[s] x sizes[s]     *
 *  row-major at values + a_offsets[s]; b_s, x_s at B / X + v_offsets[s].   *
 *  sizes, a_offsets, v_offsets are device arrays; num_systems <= 1024.     *
 * ------------------------------------------------------------------------ */
int colagb_cg_dense_batched_workspace_bytes(int64_t num_systems, int64_t total_rows, size_t* bytes);
int colagb_cg_dense_batched_solve(int64_t num_systems, const int32_t* sizes, const int64_t* a_offsets,
                                  const int64_t* v_offsets, int64_t total_rows, const float* values, const float* B,
                                  float* X, double tol, int32_t max_iters, int32_t* per_system_iters,
                                  int32_t* per_system_status, void* workspace, size_t workspace_bytes, void* stream);
/* No reference counterpart (the reference's FP32 CG stops at its FP32 recursive residual): the FP64
 * residual R = B - A X of the same uneven batch (FP32 matrices, FP64 B, X, R) and |R_s|^2 per system
 * into rr (num_systems doubles) -- the outer step of iterative refinement around
 * colagb_cg_dense_batched_solve, which lets ill-conditioned systems reach a true residual that FP32
 * CG alone stagnates above. */
int colagb_dense_batched_residual64(int64_t num_systems, const int32_t* sizes, const int64_t* a_offsets,
                                    const int64_t* v_offsets, int64_t total_rows, const float* values, const double* B,
                                    const double* X, double* R, double* rr, void* stream);

/* ======================================================================== *
 *  Lanczos with full reorthogonalisation                                   *
 *  Replaces lanczos() / lanczos_fact() / do_double_gram()                  *
 *  (cola/linalg/decompositions/lanczos.py:185-296).  bs start vectors are  *
 *  run together (the probe block of LanczosUnary, unary.py:46-60).         *
 *  V0: n x bs start vectors.  basis: (max_iters + 2) x n x bs, slot j holds *
 *  the reference's V[..., j] (slot 0 stays zero).  diag: bs x max_iters and *
 *  subdiag: bs x (max_iters + 1), compute dtype, exactly the reference's    *
 *  `diag` / `subdiag` arrays.  *steps = the reference's final loop index i. *
 * ======================================================================== */
typedef struct colagb_lanczos_params {
  double tol;
  int32_t max_iters;
  int32_t check_every;   /* host polls the device stop flag every this many steps (0 = 8) */
} colagb_lanczos_params;

int colagb_lanczos_workspace_bytes(const colagb_op* A, int64_t bs, int32_t max_iters, size_t* bytes);
int colagb_lanczos(const colagb_op* A, const void* V0, int64_t ldv0, int64_t bs,
                   const colagb_lanczos_params* params, void* basis, void* diag, void* subdiag,
                   int32_t* steps, void* workspace, size_t workspace_bytes, void* stream);

/* Ritz combination: out (n x bs) = for each probe b: sum_j basis[j+1][:, b] * coef[b][j], j < m.
 * Forms Q @ w for the LanczosUnary quadrature (unary.py:58-59) and Ritz vectors. */
/* ------------------------------------------------------------------------ *
 *  Arnoldi decomposition of a square (non-symmetric) operator              *
 *  (cola/linalg/decompositions/arnoldi.py:166-201, 303-334): Q[0] = V0 /   *
 *  |V0|, each step w = A Q[idx] orthogonalised against Q[0..idx] (two      *
 *  classical Gram-Schmidt passes; the reference does one modified pass),   *
 *  H[:, idx] = the coefficients, H[idx+1, idx] = |w|, Q[idx+1] = w /       *
 *  max(|w|, tol/2); stops when idx = max_iters or every column's |w| <=    *
 *  tol * H[1, 0].  basis: (max_iters + 2) x n x bs slots, Q[j] in slot     *
 *  j + 1; H: bs x (max_iters + 1) x max_iters row-major; steps = idx.      *
 *  Workspace as for colagb_lanczos.                                        *
 * ------------------------------------------------------------------------ */
int colagb_arnoldi_workspace_bytes(const colagb_op* A, int64_t bs, int32_t max_iters, size_t* bytes);
int colagb_arnoldi(const colagb_op* A, const void* V0, int64_t ldv0, int64_t bs, const colagb_lanczos_params* params,
                   void* basis, void* H, int32_t* steps, void* workspace, size_t workspace_bytes, void* stream);

int colagb_basis_combine(const void* basis, int64_t n, int64_t bs, int32_t m, const void* coef, int64_t ldc,
                         void* out, int32_t dtype, void* stream);

/* ======================================================================== *
 *  Symmetric tridiagonal eigensolver (batched), implicit QL with Wilkinson *
 *  shifts, in FP64 or FP32.  Replaces xnp.eigh(T) in lanczos_eigs         *
 *  (lanczos.py:57), LanczosUnary (unary.py:52) and slq_fwd (tbd/slq.py:44),*
 *  which solve T in the precision of the recurrence that produced it.     *
 *  a: batch x m diagonal, b: batch x m off-diagonal (b[i] couples i, i+1;  *
 *  b[m-1] ignored).  evals: batch x m ascending (NaN last).  first_row:    *
 *  batch x m, row 0 of the eigenvector matrix (Gauss quadrature weights),  *
 *  may be NULL.  evecs: batch x m x m (row-major, column j = eigenvector   *
 *  j), may be NULL.  status: batch ints, 0 = converged, 1 = iteration      *
 *  limit hit.  Each matrix is scaled by a power of two before the sweeps   *
 *  (exact), so any finite input is handled without overflow.  FP32 with   *
 *  evecs: each eigenvalue is then replaced by the FP64 Rayleigh quotient  *
 *  of its eigenvector (rounded to FP32), removing the sweeps' rounding.   *
 * ======================================================================== */
/* With evecs, the rotations of the QL sweeps are recorded and replayed on the rows of the eigenvector
 * matrix by a second kernel; the record lives in a stream-ordered temporary (cudaMallocAsync /
 * cudaFreeAsync on `stream`) of batch * (6 m^2 + 64) * (2 s + 4) bytes (s = 8 or 4) -- the one entry
 * point that allocates device memory itself. */
int colagb_tridiag_eig_f64(const double* a, const double* b, int64_t m, int64_t batch, double* evals,
                           double* first_row, double* evecs, int32_t* status, void* stream);
int colagb_tridiag_eig_f32(const float* a, const float* b, int64_t m, int64_t batch, float* evals,
                           float* first_row, float* evecs, int32_t* status, void* stream);

/* ======================================================================== *
 *  Learned FSAI preconditioner for 5-point operators on an m x m grid     *
 *  (cells p = i*m + j; CSR columns sorted N = p-m, W = p-1, C, E, S).     *
 *  A convolutional network reads the operator's coefficients and outputs  *
 *  per-cell scalings o (S, 3, m, m) of the closed-form FSAI factor G on   *
 *  A's lower pattern {N, W, C}; the CG preconditioner is P = G^T G.  It   *
 *  plugs into the CG(P=...) hook of cola/linalg/inverse/cg.py:124, 150.   *
 *  No counterpart in the reference beyond that hook (its only shipped     *
 *  preconditioners are Nystrom, preconditioners.py:10-153).               *
 *  Grid fields are (S, C, m, m) float32.                                   *
 * ======================================================================== */
/* CSR values (S, nnz) -> stencil (S, 5, m, m) [N, W, C, E, S]; *err_flag set if a column is off-stencil */
int colagb_grid5_stencil(const int32_t* indptr, const int32_t* indices, const float* values, int64_t nnz, int64_t m,
                         int64_t S, float* stencil, int32_t* err_flag, void* stream);
/* network input features (S, 6, m, m) from the stencil */
int colagb_fsai_features(const float* stencil, int64_t m, int64_t S, float* feats, void* stream);
/* G stencil (S, 3, m, m) [N, W, C] from the stencil and the network output (NULL = closed-form FSAI) */
int colagb_fsai_assemble(const float* stencil, const float* net_out, int64_t m, int64_t S, float* g_stencil, void* stream);
/* G stencil -> CSR values (S, g_nnz) in the lower pattern order (for colagb_batched_csr.g_values) */
int colagb_fsai_compact(const float* g_stencil, const int32_t* g_indptr, int64_t m, int64_t S, int64_t g_nnz,
                        float* g_values, void* stream);
/* The preconditioner build in one pass: the CSR values (S, g_nnz) of the normalised learned factor
 * from the stencil and the network's parameters (n_params = 3635 floats in FsaiNet's flat layout:
 * per layer W (cout, cin, 3, 3) then b (cout), layers 6->16 ReLU, 16->16 ReLU, 16->3).  The same
 * values as colagb_fsai_features -> 3 x colagb_conv3x3_forward -> colagb_fsai_assemble ->
 * colagb_fsai_compact, without the intermediate fields.  tile_counter (device, one word, may be NULL):
 * scratch that lets the CTAs take 32 x 32 tiles in arrival order -- pass one when the build shares
 * the GPU with another kernel (e.g. the previous batch's solve on another stream). */
int colagb_fsai_net_build(const float* stencil, const float* params, int64_t n_params, int64_t m, int64_t S,
                          const int32_t* g_indptr, int64_t g_nnz, float* g_values, uint32_t* tile_counter,
                          void* stream);
/* closed-form FSAI straight to CSR values (colagb_fsai_assemble with NULL, then colagb_fsai_compact) */
int colagb_fsai_closed_build(const float* stencil, int64_t m, int64_t S, const int32_t* g_indptr, int64_t g_nnz,
                             float* g_values, void* stream);
/* 3x3 convolution (padding 1): out (B, cout, H, W) = bias + w * in (B, cin, H, W); cout in {16, 3} */
int colagb_conv3x3_forward(const float* in, int64_t B, int32_t cin, int32_t cout, int64_t H, int64_t W,
                           const float* weight, const float* bias, int32_t relu, float* out, void* stream);
/* backward of one conv layer: grad_wb = [dW (cout*cin*9) | db (cout)], grad_in (may be NULL; cin in {16, 6}).
 * act (may be NULL): the layer's forward output when it was ReLU'd (grad_out is masked by act > 0). */
int colagb_conv3x3_backward_scratch_bytes(int32_t cin, int32_t cout, size_t* bytes);
int colagb_conv3x3_backward(const float* grad_out, const float* act, const float* in, int64_t B, int32_t cin,
                            int32_t cout, int64_t H, int64_t W, const float* weight, float* grad_in, float* grad_wb,
                            float* scratch, size_t scratch_bytes, void* stream);
/* training loss l_s = ||G^T G r - e||_A^2 / ||e||_A^2 for pairs A e = r (S, m*m); loss_terms (3, S) FP64 =
 * [e^T r, v^T A v, v^T r] with v = G^T G r; grad_out (S, 3, m, m) = d(mean_s l_s)/d(net_out) (may be NULL).
 * scratch: 3 * S * m * m floats. */
int colagb_fsai_loss_grad(const float* stencil, const float* net_out, const float* g_stencil, const float* r,
                          const float* e, int64_t m, int64_t S, float* grad_out, double* loss_terms, float* scratch,
                          size_t scratch_bytes, void* stream);
/* Spectral training loss: for each pair (r = A e, e) the Rayleigh quotient R_s = |G r|^2 / e^T r of
 * P A (P = G^T G) in the A inner product; loss = sum_s weights[s] log R_s (weights: +1/#white-noise
 * pairs, -1/#smooth pairs -- a scale-free proxy of log cond(P A)).  loss_terms (device, 2 S doubles):
 * e^T r, |G r|^2.  grad_out (S, 3, m, m) as for colagb_fsai_loss_grad; scratch >= S m^2 floats. */
int colagb_fsai_rq_loss_grad(const float* stencil, const float* net_out, const float* g_stencil, const float* r,
                             const float* e, const float* weights, int64_t m, int64_t S, float* grad_out,
                             double* loss_terms, float* scratch, size_t scratch_bytes, void* stream);
/* Adam update of count parameters (bias-corrected, step >= 1) */
int colagb_adam_step(float* param, const float* grad, float* m1, float* m2, int64_t count, float lr, float beta1,
                     float beta2, float eps, int32_t step, void* stream);

/* ======================================================================== *
 *  Measurement                                                             *
 * ======================================================================== */
/* No counterpart in the reference: the roofline denominator for kernels whose operands L2 serves.
 * Streams `bytes` (16-byte aligned) of `buffer` `reps` times with 128-bit loads that bypass L1 and
 * reduces them; sink (device, 1 float) is written only for impossible data.  Time two launches with
 * different reps on the caller's stream: (bytes * reps difference) / time difference is the
 * L2 -> SM read bandwidth when the buffer fits in L2, the HBM read bandwidth when it does not. */
int colagb_read_bandwidth_probe(const void* buffer, size_t bytes, int32_t reps, void* sink, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* COLAGB_H */
