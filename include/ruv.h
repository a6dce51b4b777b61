/* ruv.h — C ABI of the GB300 (sm_103a) LSCM solve path.
 *
 * Drop-in boundary for ResearchUV's CUDA solve (paths relative to the reference's crates/,
 * `researchuv-` prefix dropped):
 *   GpuSolver::global / GpuSolver::new      gpu/src/solver.rs:104-113, :122-201  -> ruv_ctx_create
 *   GpuSolver::cg_solve_precond            gpu/src/solver.rs:284-565            -> ruv_cg_solve
 *   GpuSolver::cg_solve                    gpu/src/solver.rs:274-277            -> ruv_cg_solve(PRECOND_NONE)
 *   GpuSolver::apply_ic0_for_test          gpu/src/solver.rs:205-270            -> ruv_apply_ic0
 *   Precond {None, Jacobi, Ic0, Ic0Color, Amg, AmgSa}  gpu/src/precond.rs:20-47 -> ruv_precond
 *   unfold_chart with SolverBackend::Gpu   unwrap/src/lscm.rs:471-506, :512-727 -> ruv_lscm_solve_batch
 *   weld + segment + border pass (the chart stages of pipeline::run)
 *                                          unwrap/src/pipeline.rs:146-150, lscm.rs:512-592
 *                                                                               -> ruv_prepare_mesh / ruv_prepare_patches
 *
 * Conventions: every entry returns a ruv_status (the reference's Option::None maps to any
 * non-OK status; the caller decides about a CPU fallback, the library never falls back).
 * Host buffers are caller-owned; device buffers are owned by the context and reused across
 * calls.  No exceptions cross the ABI.  A context is not thread-safe: use one per thread
 * (each holds its own CUDA stream) or serialise calls.
 */
#ifndef RUV_H
#define RUV_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RUV_ABI_VERSION 1

typedef enum ruv_status {
  RUV_OK = 0,
  RUV_ERR_NO_DEVICE = 1,     /* no CUDA device / wrong architecture            */
  RUV_ERR_BAD_INPUT = 2,     /* malformed sizes, indices or options            */
  RUV_ERR_OOM = 3,           /* device allocation failed                       */
  RUV_ERR_NOT_CONVERGED = 4, /* max_iter reached above tolerance (any chart)   */
  RUV_ERR_BREAKDOWN = 5,     /* |p.Ap| <= 1e-300, non-finite, or zero diagonal */
  RUV_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up             */
  RUV_ERR_LAUNCH = 7,        /* a CUDA launch / runtime call failed            */
  RUV_ERR_INTERNAL = 8
} ruv_status;

/* gpu/src/precond.rs:20-47 */
typedef enum ruv_precond {
  RUV_PRECOND_NONE = 0,
  RUV_PRECOND_JACOBI = 1,
  RUV_PRECOND_IC0 = 2,
  RUV_PRECOND_IC0_COLOR = 3,
  RUV_PRECOND_AMG = 4,
  RUV_PRECOND_AMG_SA = 5
} ruv_precond;

/* Arithmetic of the inner Krylov loop. */
typedef enum ruv_precision {
  RUV_PREC_FP64 = 0,  /* FP64 PCG throughout                                        */
  RUV_PREC_MIXED = 1  /* FP32 SpMV / preconditioner / CG, FP64 true residual r = b - Ax
                         and FP64 solution accumulation (reliable-update refinement)   */
} ruv_precision;

typedef struct ruv_ctx ruv_ctx;

int32_t ruv_abi_version(void);
const char* ruv_status_str(ruv_status s);

/* GpuSolver::new (gpu/src/solver.rs:122-201): device init, kernels resident (no JIT). */
ruv_status ruv_ctx_create(ruv_ctx** out, int32_t device);
void ruv_ctx_destroy(ruv_ctx* ctx);
/* Message of the last failing call on this context ("" if none). */
const char* ruv_last_error(const ruv_ctx* ctx);
/* Fault injection for tests of the out-of-memory paths (no counterpart in the reference,
 * whose DeviceMem::alloc failure is an Option::None, gpu/src/solver.rs:671-729): with
 * nth > 0 the nth device allocation this context makes from now on fails as if the device
 * were out of memory (no cudaMalloc is made; the call returns OOM), nth <= 0 turns it off.
 * The context stays usable after the failure. */
ruv_status ruv_debug_fail_alloc(ruv_ctx* ctx, int64_t nth);

/* GpuSolver::cg_solve_precond (gpu/src/solver.rs:284-565).
 * A: n x n SPD CSR (row_ptr[n+1], cols[nnz], vals[nnz]); b[n]; x_out[n] (written on OK).
 * Stops when ||r|| <= tol * ||b|| (tol absolute when ||b|| <= 1e-300), x0 = 0.
 * iters_out (may be NULL) receives the iteration count.  NOT_CONVERGED after max_iter;
 * BREAKDOWN on |p.Ap| <= 1e-300 or a non-finite iterate (solver.rs:505-508, :561-563);
 * BAD_INPUT on size mismatches (solver.rs:297-299) or a zero diagonal under Jacobi
 * (precond.rs:595-611). */
ruv_status ruv_cg_solve(ruv_ctx* ctx, int32_t n, const int32_t* row_ptr, const int32_t* cols,
                        const double* vals, const double* b, double* x_out, int64_t max_iter,
                        double tol, ruv_precond pc, int64_t* iters_out);

/* GpuSolver::apply_ic0_for_test (gpu/src/solver.rs:205-270): z = (L L^T)^-1 r with the
 * IC(0) factor of A (natural order, pivot floor 1e-12 |a_ii|, precond.rs:145-219). */
ruv_status ruv_apply_ic0(ruv_ctx* ctx, int32_t n, const int32_t* row_ptr, const int32_t* cols,
                         const double* vals, const double* r, double* z_out);

/* The IC(0) factor the preconditioner builds on the device, copied out for inspection: what
 * factor_ic0 returns to the reference's own tests (gpu/src/precond.rs:145-205; with
 * `colored`, of the colour-permuted matrix, precond.rs:49-123).  l_ptr[n+1] receives the row
 * offsets, l_cols / l_vals (capacity `cap`) the rows of L with the diagonal last, to_orig[n]
 * the position -> original row map (identity without colouring), *nnz_out the factor's
 * nonzeros, *levels_out the dependency-level count (the larger of the two sweeps),
 * *colours_out the colour count (0 without colouring).  BAD_INPUT when nnz exceeds cap
 * (counts are still written); BREAKDOWN where factor_ic0 returns None. */
/* One level of the aggregation AMG hierarchy the preconditioner builds for A (smoothed != 0:
 * AMG-SA, else plain aggregation), copied out for inspection: what the reference's own AMG
 * tests read from its hierarchy (gpu/src/amg.rs:800-942).  sizes[6] receives the level count,
 * whether this level's prolongator is smoothed, the level's rows, the next level's rows (0 on
 * the last level), and the nonzeros of the level operator and of its prolongator.  With
 * cap > 0 the arrays (capacity cap each, cap >= rows + 1) receive the level operator in FP64
 * CSR (a_ptr, a_cols, a_vals), the prolongator to the next level (p_ptr, p_cols, p_vals; rows
 * of this level, columns of the next) and the aggregate of each row (-1 on the last level).
 * BAD_INPUT for a level out of range or a capacity too small (sizes are still written). */
ruv_status ruv_amg_export(ruv_ctx* ctx, int32_t n, const int32_t* row_ptr, const int32_t* cols,
                          const double* vals, int32_t smoothed, int32_t level, int64_t cap, int64_t* sizes,
                          int64_t* a_ptr, int32_t* a_cols, double* a_vals, int64_t* p_ptr, int32_t* p_cols,
                          float* p_vals, int32_t* agg);

ruv_status ruv_ic0_export(ruv_ctx* ctx, int32_t n, const int32_t* row_ptr, const int32_t* cols,
                          const double* vals, int32_t colored, int64_t cap, int64_t* l_ptr,
                          int32_t* l_cols, double* l_vals, int32_t* to_orig, int64_t* nnz_out,
                          int32_t* levels_out, int32_t* colours_out);

/* Variant of ruv_cg_solve that allocates nothing, for callers that cannot call cudaMalloc:
 * code running inside a host application that owns all device memory through its own
 * allocator or memory pool (a renderer, a game engine, a plugin host with a fixed budget),
 * or code that must not trigger an allocation (and its implicit synchronisation) mid-frame.
 * It has no counterpart in the reference.
 *
 * The caller passes DEVICE pointers for the system (row_ptr[n+1], cols[nnz], vals[nnz]),
 * the right-hand side b[n] and the solution x[n]; the solver's own scratch (CG vectors,
 * inverse diagonal, partial sums, solver state) lives in one fixed array compiled into the
 * library, about 12.6 MB.  Each CUDA context that runs this entry holds its own copy of the
 * array until the context ends: CUDA loads the library's solver module into a context lazily,
 * on its first use there, and the array is reserved by the driver at that moment.  So the
 * FIRST call in each context (each device's primary context, or any context the caller
 * makes current) does allocate device memory through the driver and may synchronise: make
 * it at start-up, before any stream capture and outside the frame loop; later calls in that
 * context allocate nothing.  Every call resolves the array's address in the current
 * context.  Systems with n > RUV_NOALLOC_MAX_ROWS are rejected with BAD_INPUT.
 * PRECOND_NONE or _JACOBI.  Same stopping rule and statuses as ruv_cg_solve; work is
 * enqueued on `stream` (a cudaStream_t, NULL = the legacy default stream) and the call
 * returns after it finished.  All calls in a context share the one array, so calls that
 * overlap on the GPU (other threads or streams at the same time) race and must be
 * serialised by the caller.  An explanation of a non-OK status is written to msg
 * (msg_len bytes, may be NULL). */
#define RUV_NOALLOC_MAX_ROWS 262144
ruv_status ruv_cg_solve_noalloc(int32_t n, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                                const double* b, double* x, int64_t max_iter, double tol, ruv_precond pc,
                                int64_t* iters_out, void* stream, char* msg, int32_t msg_len);

/* ------------------------------------------------------------------ batched LSCM solve */

/* All charts of a mesh, packed.  Chart c owns packed vertices [vert_off[c], vert_off[c+1])
 * in chart-local order (ascending source id) and triangles [tri_off[c], tri_off[c+1]) whose
 * indices are chart-local.  This is the data unfold_chart consumes (lscm.rs:512-592):
 * positions, triangles in chart order, Dirichlet pins with their targets, and the
 * tangent-frame projection p2 that seeds the driver. */
typedef struct ruv_lscm_batch {
  int64_t n_charts;
  const int64_t* vert_off; /* n_charts + 1 */
  const int64_t* tri_off;  /* n_charts + 1 */
  const double* p3;        /* 3 * n_verts */
  const int32_t* tris;     /* 3 * n_tris (chart-local) */
  const uint8_t* pinned;   /* n_verts, 1 = pinned */
  const double* pin_uv;    /* 2 * n_verts, target of pinned vertices (others ignored) */
  const double* p2;        /* 2 * n_verts */
} ruv_lscm_batch;

/* UnfoldOptions (lscm.rs:76-101) plus the solver controls of gpu_solve (lscm.rs:471-506). */
typedef struct ruv_unfold_opts {
  double angle_mix;        /* #AngleDistanceMix, default 1.0 (mix_b = 1 - angle_mix)  */
  double mix_w;            /* slack weight, default 1.0 (must be > 0)                 */
  int32_t max_iter;        /* driver iterations, default 100                          */
  ruv_precond precond;     /* default JACOBI (lscm.rs:498)                            */
  ruv_precision precision; /* default MIXED                                           */
  double tol;              /* relative residual per chart, default 1e-12 (lscm.rs:501) */
  int64_t max_cg_iter;     /* default max(max_iter, 1024) * 16 (lscm.rs:501)         */
} ruv_unfold_opts;

void ruv_unfold_opts_default(ruv_unfold_opts* o);

/* Per-chart outcome (UnfoldResult, lscm.rs:105-116, plus solver statistics). */
typedef struct ruv_chart_stat {
  int32_t status;       /* ruv_status of this chart's solve                    */
  int32_t driver_iters; /* UnfoldResult::iters                                  */
  int32_t cg_iters;     /* Krylov iterations                                    */
  int32_t n_free;       /* free (unpinned) vertices; unknowns = 2 * n_free      */
  double rel_res;       /* final ||b - Ax|| / ||b|| in FP64                     */
  double err_accum;     /* UnfoldResult::err_accum                              */
} ruv_chart_stat;

/* One batched unfold of every chart: GPU assembly of the cotangent system with pins
 * eliminated, one batched PCG over the packed block-diagonal operator with per-chart
 * convergence, and the damped driver update.  uv_out: 2 * n_verts (chart-local order, as
 * UnfoldResult::uv).  stats: n_charts entries (may be NULL).  Returns the worst chart
 * status (OK when every chart converged). */
ruv_status ruv_lscm_solve_batch(ruv_ctx* ctx, const ruv_lscm_batch* in, const ruv_unfold_opts* opts,
                                double* uv_out, ruv_chart_stat* stats);

/* Device-resident variant of ruv_lscm_solve_batch, split in three: upload a batch into the
 * context, solve it (assembly + batched PCG + driver, results stay in device memory), and
 * download the UVs.  ruv_lscm_solve_batch is exactly these three calls. */
ruv_status ruv_lscm_upload(ruv_ctx* ctx, const ruv_lscm_batch* in);
ruv_status ruv_lscm_solve_resident(ruv_ctx* ctx, const ruv_unfold_opts* opts, ruv_chart_stat* stats);
ruv_status ruv_lscm_download_uv(ruv_ctx* ctx, double* uv_out);

/* unfold_chart with KeepMetric (lscm.rs:544-568, :642-676): the slack row becomes the area
 * row -- the conformal free block K bordered by the slack column flip * area_w (both rows of
 * a free vertex), the area gradient g(uv) and the corner area(uv) - target, rhs 2 * target.
 * The reference factors that matrix by its CPU LU every driver iteration (it is not
 * symmetric; lscm.rs:672-680).  Here only g and area change between iterations, so K is
 * solved once for two right-hand sides by the batched PCG (y_b = K^-1 b, y_u = K^-1 u) and
 * every iteration is the Schur complement aux = (2 target - g.y_b) / ((area - target) -
 * g.y_u), x = y_b - aux y_u, followed by the damped driver step.  target: per chart
 * (opts.target_area if > 0, else the chart's area3d, lscm.rs:568).  stats: status worst of
 * the two solves, cg_iters their sum. */
ruv_status ruv_lscm_solve_batch_keep_metric(ruv_ctx* ctx, const ruv_lscm_batch* in, const ruv_unfold_opts* opts,
                                            const double* target, double* uv_out, ruv_chart_stat* stats);

/* Differentiation (the forward / backward pair a torch.autograd.Function would wrap).
 * No counterpart in the reference's API: its unfold is not differentiable.
 *
 * ruv_lscm_forward: the forward solve, exactly ruv_lscm_solve_batch; the batch and the
 * solution stay on the context for the backward call.
 *
 * ruv_lscm_backward: given dL/duv (2 * n_verts, chart-local vertex order as uv_out), writes
 * dL/dp3 (3 * n_verts) of the last forward solve, the pins held at their targets.  The
 * assembly is recomputed; one adjoint solve A lam = dL/duv (free rows) runs with the same
 * operator, preconditioner and precision as `opts` asks; the reverse pass of the assembly
 * (edge coefficients, cotangents) maps lam to the positions.  stats (may be NULL) report the
 * adjoint solve per chart.  dL/duv of pinned vertices is ignored (their UVs are constants). */
ruv_status ruv_lscm_forward(ruv_ctx* ctx, const ruv_lscm_batch* in, const ruv_unfold_opts* opts,
                            double* uv_out, ruv_chart_stat* stats);
ruv_status ruv_lscm_backward(ruv_ctx* ctx, const ruv_unfold_opts* opts, const double* dl_duv,
                             double* dl_dp3, ruv_chart_stat* stats);

/* Distortion loss of a UV layout of the resident batch: per chart
 * sum_t area_t (s1/s2 - 1)^2, area_t the 3-D triangle area and s1 >= s2 the singular values
 * of the UV Jacobian as unwrap/src/metrics.rs:73-128 forms them (triangles that metric skips
 * add nothing).  loss_out: n_charts; dl_duv (2 * n_verts) and dl_dp3 (3 * n_verts) receive
 * its gradients when non-NULL. */
ruv_status ruv_distortion_loss(ruv_ctx* ctx, const double* uv, double* loss_out, double* dl_duv,
                               double* dl_dp3);

/* chart_distortion (unwrap/src/metrics.rs:73-141) of a UV layout of the resident batch: per
 * chart [conformal mean, conformal max, area-ratio mean, flips, folds] (metrics_out:
 * 5 * n_charts). */
ruv_status ruv_chart_distortion(ruv_ctx* ctx, const double* uv, double* metrics_out);

/* Device time (ms, CUDA events on the context stream) of the phases of the last
 * ruv_lscm_solve_resident: [0] assembly, [1] batched PCG, [2] driver update, [3] the
 * preconditioner set-up inside [1] (AMG hierarchy; 0 otherwise).
 * Returns the number of values written (<= n). */
int32_t ruv_last_timings(const ruv_ctx* ctx, double* ms, int32_t n);

/* rectangularize (unwrap/src/metrics.rs:147-227), the post-solve normalisation pipeline::run
 * applies to every chart (pipeline.rs:171-176), for every chart of the resident batch: the
 * chart rotated by the angle of the 72-step ladder whose border bounding box scores least,
 * normalised to [0,1]^2, its border points snapped onto the nearest side.  uv: 2 * n_verts;
 * border: n_verts flags (the chart's border set); rectified_out: 2 * n_verts; ext_out:
 * 2 * n_charts (the extents before normalisation).  Bit-identical to the reference on the
 * same host libm (the angle table is computed on the host). */
ruv_status ruv_rectangularize(ruv_ctx* ctx, const double* uv, const uint8_t* border,
                              double* rectified_out, double* ext_out);

/* Page-locked host memory (cudaHostAlloc) for a caller's input and output arrays: copies
 * between it and the device run at the link's full rate.  Freed with ruv_host_free. */
ruv_status ruv_host_alloc(ruv_ctx* ctx, int64_t bytes, void** out);
void ruv_host_free(void* p);

/* Self-test of the assembly's FP64 division and square root (computed on the integer and
 * FP32 pipes, bit-identical to the IEEE operations by design): n seeded inputs of class
 * `mode` (0-2: quotients -- moderate exponents, arbitrary bit patterns, near midpoints;
 * 3-5: square roots -- moderate exponents, arbitrary bit patterns, near perfect squares)
 * compared bit for bit with the hardware operations.  *mismatches = the count; first4 =
 * (a, b, got, want) of the first mismatch.  No reference counterpart: a diagnostic. */
ruv_status ruv_selftest_fp64(ruv_ctx* ctx, int mode, uint64_t seed, int64_t n, int64_t* mismatches, double* first4);

/* Number of kernels this context has enqueued so far (each node of a replayed CUDA graph
 * counts once per replay). */
int64_t ruv_kernel_launches(const ruv_ctx* ctx);

/* Kernel benchmark on the last assembled batch: `reps` launches of the batched SpMV kernel
 * (q = A p over every row, FP32 values when precision is MIXED, FP64 otherwise), rotating
 * between `n_buffers` vector sets so the timed launches read their vectors from HBM.
 * Writes the mean device time per launch (ms, CUDA events), the algorithmic bytes of one
 * launch (values + 32-bit columns + row pointers + p read once + q written) and the bytes
 * its streams actually hold (the same with 16-bit columns where the operator has them).
 * Any output may be NULL. */
ruv_status ruv_bench_spmv(ruv_ctx* ctx, ruv_precision precision, int32_t reps, int32_t n_buffers,
                          double* ms_per_launch, double* bytes_per_launch, double* stream_bytes_per_launch);

/* Autotuner: on the last assembled batch, time the batched SpMV together with the CG
 * iteration's other kernels over the same row tiles (update, dots, direction) for each
 * instantiated launch shape (lanes per row x rows in flight per sub-warp) and tile height
 * (rows per CTA), keep the fastest for this context's later solves, and report it
 * (ms_per_launch: that SpMV plus those three kernels).  Any output may be NULL. */
ruv_status ruv_autotune(ruv_ctx* ctx, ruv_precision precision, int32_t reps, int32_t* lanes_per_row,
                        int32_t* rows_in_flight, int32_t* tile_rows, double* ms_per_launch);

/* The SpMV form this context's solves use: *bulk_copy = 1 for the kernel that stages each
 * tile by bulk asynchronous copies, 0 for the CSR-vector kernel (the default; the autotuner
 * picks one; the environment variable RUV_SPMV_TMA=0/1 overrides both). */
ruv_status ruv_spmv_form(ruv_ctx* ctx, int32_t* bulk_copy);

/* ------------------------------------------------------------------ host chart stages */

typedef struct ruv_prepared ruv_prepared;

/* weld (weld.rs:19-57) + segment (segment.rs:130-331) of a raw triangle soup, then per
 * chart the tangent frame (lscm.rs:152-183) and the pins: border rectangle
 * (lscm.rs:280-413) or 4 anchors for closed charts (lscm.rs:210-247, :524-542). */
ruv_status ruv_prepare_mesh(const double* pos, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                            double weld_tol, double angle_min_deg, int32_t threads, ruv_prepared** out);
/* ruv_prepare_mesh with its data-parallel stages on the device of ctx: the weld (a device
 * hash table keeping the reference's first occurrence), the edge-face lists (a stable radix
 * sort of the edge keys), the face normals and dihedral cut flags (round-to-nearest FP64;
 * the acos test as a threshold on n1.n2 derived from the host libm) and the per-chart vertex
 * sets (a radix sort of (chart, vertex) keys).  The DFS component order, border loops,
 * frames and pins stay on the host.  The result equals ruv_prepare_mesh's bit for bit
 * (weld.rs:19-57, segment.rs:61-331, lscm.rs:152-413 as there). */
ruv_status ruv_prepare_mesh_gpu(ruv_ctx* ctx, const double* pos, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                                double weld_tol, double angle_min_deg, int32_t threads, ruv_prepared** out);

/* Seam cut of closed charts (seam.rs SeamCutOptions, :286-305) and distortion-driven
 * re-cutting of folding charts (recut.rs RecutOptions, :98-146), run after the segmentation
 * as pipeline::run does (pipeline.rs:149-167).  Both are off by default, as in the reference. */
typedef struct ruv_cut_opts {
  int32_t seam_enable;         /* open borderless charts along a seam tree, default 0     */
  int32_t seam_min_faces;      /* only charts with at least this many faces, default 8    */
  int32_t seam_branch_count;   /* branches beyond the geodesic-diameter trunk, default 1  */
  int32_t recut_enable;        /* re-cut charts that fold, default 0                       */
  int32_t recut_max_rounds;    /* controller rounds, default 6                             */
  int32_t recut_max_splits;    /* total new cut edges, default 48                          */
  double recut_fold_fraction;  /* re-cut when more triangles than this fraction fold, 0.02 */
  int32_t recut_max_charts;    /* stop when the chart count exceeds this, default 64      */
} ruv_cut_opts;

void ruv_cut_opts_default(ruv_cut_opts* o);

/* ruv_prepare_mesh followed by the seam cut and / or the re-cutting controller.  Every
 * controller round unfolds all charts in one batched solve on ctx (unfold: the options of
 * that solve; the reference unfolds chart by chart, recut.rs:71-79) and counts each chart's
 * winding-inconsistent triangles (metrics.rs:33-56); every folding chart gets its separating
 * cut (seam tree when closed, border-crossing chord when open, seam.rs:167-283) and the
 * charts are rebuilt over the grown cut set.  *added_out = the cut edges the controller added.
 * ctx may be NULL when re-cutting is off (the seam cut alone runs on the host). */
ruv_status ruv_prepare_mesh_cut(ruv_ctx* ctx, const double* pos, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                                double weld_tol, double angle_min_deg, const ruv_cut_opts* cut,
                                const ruv_unfold_opts* unfold, int32_t threads, ruv_prepared** out, int64_t* added_out);

/* Charts given directly (one chart per patch, no weld / segmentation): patch c owns
 * vertices [vert_off[c], vert_off[c+1]) and triangles [tri_off[c], tri_off[c+1]) with
 * patch-local indices.  Border loops are walked over each patch's boundary edges. */
ruv_status ruv_prepare_patches(int64_t n_patches, const int64_t* vert_off, const int64_t* tri_off,
                               const double* p3, const int32_t* tris, int32_t threads, ruv_prepared** out);
/* ruv_prepare_patches with its data-parallel stages on the device of ctx: the patch faces
 * and their checks, the edge-face lists (a stable radix sort of the edge keys), every
 * patch's faces in the reference's DFS pop order (segment.rs:150-175, one thread per patch),
 * face areas and chart areas, the centroid and covariance of each chart's vertices and the
 * projection on the chart's frame (lscm.rs:152-183), the boundary edges.  The border-loop
 * walk (segment.rs:227-331), the 3 x 3 eig3 of each frame (host libm) and the pins
 * (lscm.rs:187-413) run on the host per chart.  The result equals ruv_prepare_patches's bit
 * for bit. */
ruv_status ruv_prepare_patches_gpu(ruv_ctx* ctx, int64_t n_patches, const int64_t* vert_off, const int64_t* tri_off,
                                   const double* p3, const int32_t* tris, int32_t threads, ruv_prepared** out);
void ruv_prepared_free(ruv_prepared* p);
/* Read-only view of the prepared charts as the batched-solve input (valid while p lives). */
ruv_status ruv_prepared_batch(const ruv_prepared* p, ruv_lscm_batch* view);

/* Structure queries for parity checks.  `what` selects an int64 array:
 *   "chart.vert_off" (n_charts+1)  "chart.tri_off" (n_charts+1)  "chart.vertex_ids" (source id
 *   per packed vertex)  "chart.face_ids" (source face per packed triangle)  "chart.border_off"
 *   "chart.border"  "chart.loop_off" (per chart, into loop_seg)  "chart.loop_seg" (per loop,
 *   into loop_ids)  "chart.loop_ids"  "mesh.faces"  "chart.pinned"
 * or a double array: "chart.area3d"  "mesh.pos"  "chart.pin_uv"  "chart.p2"  "chart.p3".
 * Returns the element count (copies when out != NULL), or -1 for an unknown name. */
int64_t ruv_prepared_get_i64(const ruv_prepared* p, const char* what, int64_t* out);
int64_t ruv_prepared_get_f64(const ruv_prepared* p, const char* what, double* out);

/* Assembled system of one chart of the last ruv_lscm_solve_batch on ctx, exported as the
 * interleaved CSR the reference hands its GPU solver (Sparse::to_csr(2 nf), sparse.rs:69-84):
 * row_ptr[2nf+1], cols[nnz], vals[nnz], rhs[2nf].  Call with NULL buffers to get nnz and nf. */
ruv_status ruv_export_chart_system(ruv_ctx* ctx, int64_t chart, int64_t* nf_out, int64_t* nnz_out,
                                   int32_t* row_ptr, int32_t* cols, double* vals, double* rhs);

#ifdef __cplusplus
}
#endif

#endif /* RUV_H */
