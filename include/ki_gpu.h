/*
 * ki_gpu.h -- C ABI of the GB300 recursive-skeletonization solver.
 *
 * Drop-in boundary for the reference's factor-and-solve path (kern_interp,
 * C++ namespace kern_interp).  Each entry point names the reference function
 * whose role it takes; all reference paths are relative to that project.
 *
 * Conventions
 *  - Plain C types only; matrices are column-major doubles with an explicit
 *    leading dimension, like the reference's ki_Mat (kern_interp/ki_mat.h:19-104).
 *  - Every function returns a ki_status; on failure ki_last_error() returns a
 *    message for the calling thread.  No function asserts or exits (the
 *    reference asserts on LAPACK failures, kern_interp/ki_mat.cpp:452-565).
 *  - A ki_factor owns its device memory and a CUDA stream.  Calls on one
 *    handle must not overlap; distinct handles are independent.
 */
#ifndef KI_GPU_H_
#define KI_GPU_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  KI_OK = 0,
  KI_ERR_ARG = 1,      /* invalid argument (sizes, NULL pointers, non-finite data) */
  KI_ERR_CUDA = 2,     /* CUDA runtime error or no usable GPU */
  KI_ERR_NUMERIC = 3,  /* singular pivot / non-finite value during factorization */
  KI_ERR_TIMEOUT = 4,  /* a bounded device wait gave up */
  KI_ERR_OOM = 5,      /* device allocation failed */
  KI_ERR_STATE = 6     /* call not valid for this handle (e.g. wrong problem kind) */
} ki_status;

/* Kernel::Pde (kern_interp/kernel/kernel.h:19-24).  LAPLACE and STOKES in 2D
 * and 3D; LAPLACE_NEUMANN (the interior Neumann problem's adjoint double
 * layer plus the rank-one weight term, kernel.cpp:44-54; domain targets take
 * the single layer) and GAUSS (exp(-|r|^2), 5 on the diagonal, three proxy
 * rings, kernel.cpp:55-60 and :661-672) in 2D with solution_dimension 1.
 * These two have no border: holes are ignored (initialize_U_mat gives them
 * an empty U, linear_solve.cpp:101-104), and their refinement residual is
 * the dense FP64 apply (the FMM serves 2D LAPLACE). */
typedef enum {
  KI_PDE_LAPLACE = 0,
  KI_PDE_LAPLACE_NEUMANN = 1,
  KI_PDE_GAUSS = 2,
  KI_PDE_STOKES = 3
} ki_pde;

typedef enum {
  KI_PRECISION_FP64 = 0,   /* plain form: every stage in FP64 (the reference's arithmetic) */
  KI_PRECISION_FP32 = 1    /* FP32 factorization (preconditioner for refinement); id_tol >= 5e-8 */
} ki_precision;

/*
 * Problem description: the data a reference Boundary carries
 * (kern_interp/boundaries/boundary.h:47-64) plus the tree/proxy parameters the
 * reference fixes as macros (MAX_LEAF_DOFS quadtree/quadtree.h:11,
 * NUM_PROXY_POINTS / RADIUS_RATIO kernel/kernel.h:13-14,
 * MIN_DOFS_TO_COMPRESS skel_factorization/skel_factorization.h:12) and the
 * SkelFactorization constructor's id_tol
 * (skel_factorization/skel_factorization.h:27).  Zero parameters take the
 * reference defaults (64, 128, 2.0, 64).
 */
typedef struct {
  int n_points;              /* boundary nodes */
  int domain_dimension;      /* d = 2 (curves) or 3 (surfaces) */
  int solution_dimension;    /* 1 (Laplace) or d (Stokes: 2 in 2D, 3 in 3D) */
  int pde;                   /* ki_pde */
  const double* points;      /* d*n_points, interleaved (x, y[, z]) */
  const double* normals;     /* d*n_points, interleaved (GAUSS: may be NULL, read as 0) */
  const double* weights;     /* n_points quadrature weights (GAUSS: may be NULL) */
  const double* curvatures;  /* n_points, may be NULL (treated as 0; unused in 3D) */
  int n_holes;               /* multiply connected: number of holes */
  const double* hole_centers;    /* d*n_holes */
  const int* hole_node_start;    /* first node of each hole */
  const int* hole_node_count;    /* nodes of each hole */
  int max_leaf_dofs;
  int num_proxy_points;
  double radius_ratio;
  int min_dofs_to_compress;
  double id_tol;
  int precision;             /* ki_precision */
  /* Learned rank predictor (no reference counterpart): a model blob of
   * ki_rank_model_floats() floats (see ki_rank_model_train) or NULL.  Used by
   * FP32 factorizations only: each box whose ID fits the shared-memory kernel
   * is compressed from a random sketch of l = min(n, 1.25 k^ + 8) rows, k^
   * the predicted rank; a sketch that does not reveal the rank within l
   * pivots is recompressed by the plain ID.  FP64 factorizations ignore it
   * (they keep the reference's deterministic ID). */
  const float* rank_model;
} ki_problem_desc;

typedef struct ki_factor ki_factor;

typedef struct {
  int n_dofs;           /* unknowns */
  int n_levels;         /* tree levels */
  int n_compressed;     /* boxes compressed */
  long n_redundant;     /* DOFs eliminated below the root */
  int n_root;           /* root skeleton size */
  int n_border;         /* bordered unknowns (holes x border columns) */
  double factor_seconds;
  long device_bytes;    /* device memory held by the factorization */
  int n_sketched;       /* boxes compressed from a sketch (learned rank) */
  int n_fallback;       /* sketches recompressed by the plain ID */
  int n_reused;         /* boxes whose factors ki_factor_update copied from the
                           previous factorization */
} ki_factor_info;

/*
 * Build the tree (QuadTree::initialize_tree, quadtree/quadtree.cpp:240-287)
 * and skeletonize (SkelFactorization::skeletonize,
 * skel_factorization/skel_factorization.cpp:173-551) on the current GPU.
 */
int ki_factor_create(const ki_problem_desc* desc, ki_factor** out);

/*
 * Re-factorize the handle for a perturbed boundary: QuadTree::perturb
 * (quadtree/quadtree.cpp:581-890) followed by SkelFactorization::skeletonize,
 * which skips the boxes perturb left compressed (skel_factorization/
 * skel_factorization.cpp:199-208).  desc describes the new boundary (the same
 * fields as for ki_factor_create).  The tree is rebuilt for the new points;
 * a box keeps its previous factors, copied on the device without an ID or
 * elimination, when the previous tree has a box at the same level and
 * centre, its DOFs and their data (coordinates, normals, weights,
 * curvatures, the 3D diagonal) are bitwise unchanged, its children were
 * kept, and its near-field neighbours are the same boxes with unchanged
 * DOFs.  Every other box, the top levels whose ID reads the whole level, the
 * root block and the border of a multiply connected problem are computed
 * afresh.  Points are identified by index, so the new boundary should list
 * its unmoved points at their old indices; a boundary of a different
 * size, kind, precision, parameter set or rank model is factorized from
 * scratch (info.n_reused = 0).  The result is a factorization of the new
 * problem like ki_factor_create's; its recomputed boxes may be launched in
 * other groupings than a fresh factorization's, so the two agree to rounding
 * and the ID tolerance, not bit for bit.  On failure the handle keeps its
 * previous factorization.  No solve on the handle may be in flight.
 */
int ki_factor_update(ki_factor* f, const ki_problem_desc* desc);

/* Release a factorization (QuadTree destructor). */
int ki_factor_destroy(ki_factor* f);

/* Factorization statistics. */
int ki_factor_get_info(const ki_factor* f, ki_factor_info* info);

/*
 * Apply the inverse to nrhs right-hand sides held in HOST memory:
 * SkelFactorization::solve (skel_factorization.cpp:595-778) for simply
 * connected problems, multiply_connected_solve (:781-1141, generalised to
 * every column) otherwise; linear_solve (linear_solve.cpp:202-227) is the
 * reference's wrapper over both.  b: n_dofs x nrhs (ldb), x: n_dofs x nrhs
 * (ldx), alpha: n_border x nrhs (ldalpha, may be NULL when n_border == 0).
 * x may alias b.
 */
int ki_solve(ki_factor* f, const double* b, int ldb, int nrhs, double* x, int ldx,
             double* alpha, int ldalpha);

/*
 * The same with DEVICE pointers; runs on `stream` (a cudaStream_t, NULL for
 * the handle's own stream) and returns without synchronizing.
 */
int ki_solve_device(ki_factor* f, const double* d_b, int ldb, int nrhs, double* d_x, int ldx,
                    double* d_alpha, int ldalpha, void* stream);

/*
 * ki_solve_device without any device allocation.  No counterpart in the
 * reference.  For callers that cannot allocate device memory while solving:
 * applications that reserve all device memory up front for their own
 * allocator and account for every byte, and latency-critical loops that
 * cannot absorb the implicit synchronization of cudaMalloc/cudaFree.
 * Same arguments, stream and results as ki_solve_device; its temporaries
 * come from one fixed 32 MiB device array that every GPU loading the
 * library holds until the process exits.  Limit: the DOF-major copy of the
 * right-hand sides plus the solve's temporaries must fit in those 32 MiB
 * (about n_dofs * nrhs * 8 bytes for simply connected problems, twice that
 * with holes); larger calls return KI_ERR_ARG with the size needed.
 * The first call on a device looks up the array's device address (with that
 * device current); make that first call before any stream capture.  All
 * calls share the array and it keeps the last call's contents (nothing in it
 * is read before being written): calls that overlap on the GPU -- on
 * different streams or handles at the same time -- race.
 */
int ki_solve_device_noalloc(ki_factor* f, const double* d_b, int ldb, int nrhs, double* d_x,
                            int ldx, double* d_alpha, int ldalpha, void* stream);

/*
 * y = K x with the dense FP64 Nystrom operator of the problem, x and y in
 * HOST memory (n_dofs x ncols): the reference's dense residual check
 * (solve_err, linear_solve.cpp:379-425, via Kernel::operator(),
 * kernel/kernel.cpp:304-360).  When the problem has holes the border term
 * U*alpha is added if alpha != NULL.  Cost O(n_dofs^2 * ncols).  3D Laplace
 * computes its entries and sums in FP32-pair arithmetic (~1e-13 relative
 * per entry; KI_DENSE3=fp64 keeps FP64).
 */
int ki_apply(ki_factor* f, const double* x, int ldx, int ncols, const double* alpha,
             int ldalpha, double* y, int ldy);

/*
 * The same product by a fast multipole method (2D Laplace problems only,
 * KI_ERR_STATE otherwise): uniform-depth quadtree, 24-term Laurent/Taylor
 * expansions of the Cauchy-sum form of the double layer, direct near field
 * with the exact Nystrom entries; relative error ~1e-12.  O(n_dofs * ncols)
 * work.  No reference counterpart (the reference's residual and forward
 * evaluation are dense, kern_interp/linear_solve.cpp:339-426,
 * kern_interp/kernel/kernel.cpp:799-825); it serves the residuals of
 * ki_solve_refined, whose dense O(n_dofs^2) product is out of reach at a
 * million unknowns.
 */
int ki_apply_fmm(ki_factor* f, const double* x, int ldx, int ncols, const double* alpha,
                 int ldalpha, double* y, int ldy);

/*
 * ki_apply_fmm with `order` expansion terms (0: 24; at most 32) and, with
 * fp32 != 0, FP32 arithmetic for the charges, expansions, translations and
 * near-field sums (the apply of refinement's residual updates; relative
 * error ~1e-6 at 12 terms).
 */
int ki_apply_fmm_ex(ki_factor* f, const double* x, int ldx, int ncols, const double* alpha,
                    int ldalpha, double* y, int ldy, int order, int fp32);

/*
 * The same restricted to the listed DOFs: y (nrows x ncols, ldy) = rows of
 * K x (+ U alpha).  Cost O(nrows * n_dofs * ncols): a sampled residual check
 * at sizes where the full dense product is out of reach.
 */
int ki_apply_rows(ki_factor* f, const int* rows, int nrows, const double* x, int ldx, int ncols,
                  const double* alpha, int ldalpha, double* y, int ldy);

/*
 * Solution at domain points: u = K_forward mu (+ U_forward alpha), HOST
 * buffers (Kernel::apply_forward, kernel/kernel.cpp:809-825, and the
 * U_forward term of schur_solve, linear_solve.cpp:241-249).
 * targets: 2*n_targets interleaved; out: (n_targets*solution_dimension) x ncols.
 */
int ki_eval_targets(ki_factor* f, const double* targets, int n_targets, const double* mu,
                    int ldmu, int ncols, const double* alpha, int ldalpha, double* out,
                    int ldout);

/* Outcome of a refined solve. */
typedef struct {
  int steps;          /* refinement corrections applied after the first solve */
  double residual0;   /* max over columns of ||[b;0] - A[x;alpha]|| / ||b|| after the first solve */
  double residual;    /* the same after the last correction: an upper bound, the updated
                         residual plus drift_bound (max over columns) */
  int updates;        /* corrections whose residual was updated (r -= A_low d) rather than
                         recomputed */
  double drift_bound; /* bound on the updated residuals' distance from the FP64 residual,
                         relative to ||b|| (max over columns; 0 without updates) */
} ki_refine_info;

/*
 * Solve to a relative residual `tol` by iterative refinement: x0 = M^-1 b
 * with the handle's factorization M (FP32 or FP64), then, while the
 * largest column residual ||[b;0] - A[x;alpha]|| / ||b|| of the FP64
 * operator A (the dense Nystrom matrix K, bordered by [U; Psi -I] when the
 * problem has holes) exceeds tol and fewer than max_steps corrections were
 * made, [x;alpha] += M^-1 r.  No reference counterpart: the reference
 * solves once with its FP64 factorization (linear_solve,
 * kern_interp/linear_solve.cpp:202-227) and checks the residual separately
 * (solve_err, :339-426).  HOST buffers as in ki_solve.  The residual's
 * operator product is the FMM of ki_apply_fmm for 2D Laplace problems with
 * at least 4096 unknowns (O(n_dofs * nrhs) per step), else the dense
 * product of ki_apply (O(n_dofs^2 * nrhs)); the environment variable
 * KI_RESIDUAL_APPLY=dense|fmm overrides the choice.  With the FMM, a
 * correction d whose residual change is small enough is followed by the
 * update r -= A_low d, A_low the FMM in FP32 arithmetic at 12 terms
 * (relative error eps_low = 1e-5 or better), instead of a new FP64 product:
 * the update is kept while the accumulated bound eps_low * sum over
 * updates of (||r_before|| + ||r_after||) / ||b|| (so that ||A d|| <=
 * ||r_before|| + ||r_after||) stays below tol / 20 per column -- it is
 * tried when eps_low ||r_before|| / ||b|| fits, and an update whose actual
 * bound does not fit is followed by the FP64 product after all; the
 * reported residual is the updated one plus that bound.
 * KI_REFINE_UPDATE=0 recomputes the FP64 residual after every correction.
 */
int ki_solve_refined(ki_factor* f, const double* b, int ldb, int nrhs, double* x, int ldx,
                     double* alpha, int ldalpha, double tol, int max_steps, ki_refine_info* info);

/*
 * The same on DEVICE buffers with leading dimensions n_dofs (b, x) and
 * n_border (alpha; required when the problem has holes), on `stream`
 * (NULL: the handle's stream); returns after the stream has finished.
 */
int ki_solve_refined_device(ki_factor* f, const double* d_b, int nrhs, double* d_x,
                            double* d_alpha, double tol, int max_steps, ki_refine_info* info,
                            void* stream);

/*
 * Per-stage device times (CUDA events on the handle's stream) as a JSON
 * string: {"factor": [{"stage", "launches", "ms", "flops", "bytes"}...],
 * "solve": [...]}; flops/bytes are the algorithmic counts of each stage.
 * No reference counterpart (the reference prints omp_get_wtime totals,
 * kern_interp/linear_solve.cpp:275-279).  Solves are recorded only after
 * ki_factor_set_profiling(f, 1).
 */
int ki_factor_get_profile(ki_factor* f, char* buf, int len);
int ki_factor_set_profiling(ki_factor* f, int on);

/*
 * FMA throughput of the current GPU's CUDA cores in GFLOP/s (FP64 and FP32),
 * measured with register-resident independent FMA chains.  No reference
 * counterpart: the compute denominators of the roofline figures.
 */
int ki_measure_fma_peak(double* fp64_gflops, double* fp32_gflops);

/*
 * Health check of the tensor-core path (no reference counterpart): runs the
 * machinery of the FP32 factorization's tensor-core ID sketch (tcgen05 TF32
 * MMAs from shared-memory operand tiles into TMEM accumulators, entries
 * split hi + lo) on fixed data on the current GPU and returns in
 * *max_rel_err its largest difference from the same product summed in FP64,
 * relative to the largest entry (about 1e-6 when the path works).
 */
int ki_tensor_core_check(double* max_rel_err);

/*
 * Learned rank predictor (no reference counterpart): a 12-64-64-1 MLP
 * (ReLU hidden layers, logistic output) mapping per-box features to the rank
 * fraction k/n of the box's interpolative decomposition, trained and
 * evaluated by the library's own FP32 CUDA kernels.  Feature rows are the
 * first 12 floats of the box log below.
 *
 * ki_rank_model_floats: size of a model blob (feature mean and scale,
 *   weights, biases).
 * ki_rank_model_train: full-batch Adam on the mean squared error over n
 *   samples (features: n x 12 row-major, ratios: n); the blob is initialized
 *   from the data (feature standardization) and `seed` (weights), trained for
 *   `epochs` steps of rate `lr`, and written to `model`; `loss` receives the
 *   final mean squared error.  Deterministic for given inputs.
 * ki_rank_model_predict: ratios (n) for n feature rows.
 * ki_rank_model_predict_bf16: the same as the FP32 factorizations infer them:
 *   BF16 operands on the tensor cores (tcgen05 MMAs, FP32 accumulation).
 * ki_rank_model_grad: the loss and its gradient with respect to the blob
 *   (the standardization entries get zero) -- for checking the kernels.
 * ki_factor_get_box_log: per ID box of the factorization, 15 floats: the 12
 *   features, the box's active DOFs n, its rank k (0: not compressed) and its
 *   level; at most max_rows rows are written, *rows receives the total.
 */
int ki_rank_model_floats(void);
int ki_rank_model_train(const float* features, const float* ratios, int n, int epochs, float lr,
                        unsigned seed, float* model, float* loss);
int ki_rank_model_predict(const float* model, const float* features, int n, float* ratios);
int ki_rank_model_predict_bf16(const float* model, const float* features, int n, float* ratios);
int ki_rank_model_grad(const float* model, const float* features, const float* ratios, int n,
                       float* grad, float* loss);
int ki_factor_get_box_log(const ki_factor* f, float* out, int max_rows, int* rows);

/*
 * The library allocates its device memory stream-ordered from a pool of its
 * own (one per device) that keeps freed memory for reuse, so repeated
 * factorizations and solves do not map fresh pages each time.  This returns
 * the memory the pool holds but no live factorization uses.  No reference
 * counterpart (the reference allocates host memory with new[]).
 */
int ki_trim_memory(void);

/*
 * Kernels the library has launched since it was loaded (every launch goes
 * through one counted helper).  No reference counterpart.
 */
long long ki_launch_count(void);

/*
 * Autotuner (no reference counterpart; the reference has nothing to tune):
 * per box-size bucket, the launch shape of the factorization's ID bins (fold
 * rows x threads), Schur bins (threads, Gauss-Jordan split) and solve sweeps
 * (threads) that runs fastest on the current GPU.
 *
 * ki_autotune: factorizes desc `repeats` times per candidate and knob (knob
 *   after knob, each later knob under the choices already made), with every
 *   launch group on one stream and timed by CUDA events, and, for the sweeps,
 *   solves nrhs right-hand sides; keeps per bucket the fastest candidate in
 *   the library's table (buckets it did not see keep theirs) and writes
 *   {"table": {...}, "ms": {"id:17": [ms per candidate], ...}} to out.
 * ki_tune_set: replaces the table with a flat JSON object {"id:17": 2, ...}
 *   (the "table" part of ki_autotune's output); {} restores the built-in
 *   heuristics.  KI_ERR_ARG on malformed input.
 * ki_tune_get: the current table as such a JSON object.
 * The table is process-wide; set it before factorizing.
 */
int ki_autotune(const ki_problem_desc* desc, int nrhs, int repeats, char* out, int len);
int ki_tune_set(const char* json);
int ki_tune_get(char* buf, int len);

/* Message of the last failure on the calling thread ("" if none). */
const char* ki_last_error(void);

/* Library version string. */
const char* ki_version(void);

#ifdef __cplusplus
}
#endif

#endif /* KI_GPU_H_ */
