// The packed block-diagonal operator the batched solver works on, and the stages that
// produce and consume it.
#pragma once

#include <memory>

#include "common.cuh"

namespace ruv {

// One SPD block per chart, rows packed chart after chart (chart c owns rows
// [chart_row[c], chart_row[c+1])).  For the LSCM path a row is a free vertex and the block is
// the scalar cotangent Laplacian L of the chart: the reference's interleaved system is
// A = L (x) I2 (u and v rows carry identical values), so the solver stores L once and
// carries (u, v) as one 2-wide right-hand side.  For the generic drop-in (ruv_cg_solve) a
// row is a scalar unknown and nrhs = 1.
struct DevSystem {
  int64_t n_charts = 0, n_rows = 0, nnz = 0;
  int nrhs = 2;
  int64_t* chart_row = nullptr;  // n_charts + 1 (device)
  std::vector<int64_t> h_chart_row;
  int32_t* row_ptr = nullptr;    // n_rows + 1
  int32_t* cols = nullptr;       // nnz (global row ids)
  double* vals = nullptr;        // nnz, FP64
  float* vals32 = nullptr;       // nnz, FP32 copy for the mixed-precision inner loop
  uint16_t* cols16 = nullptr;    // nnz: column - first row of the chart (every chart <= 65536 rows),
                                 // or column - row + 32768 (rowrel16: some chart is larger)
  int32_t* cbase = nullptr;      // n_charts: first row of each chart (chart-relative stream)
  bool rowrel16 = false;
  double* diag = nullptr;        // n_rows
  double* b = nullptr;           // nrhs * n_rows
  // the mixed solver's low FP32 halves of vals and FP64 row sums as double-float pairs, when
  // the assembly formed them (else the solver forms them)
  float* vals_lo = nullptr;      // nnz
  float2* rsum = nullptr;        // n_rows
};

// Solver controls and per-chart outcome.
struct SolveOpts {
  ruv_precond precond = RUV_PRECOND_JACOBI;
  ruv_precision precision = RUV_PREC_FP64;
  double tol = 1e-12;
  int64_t max_iter = 16384;
};

struct ChartResult {
  int32_t status;
  int32_t iters;
  int32_t refinements;
  double rel_res;
};

struct Ctx;

// A preconditioner applied as its own launch sequence between the CG's update and direction
// steps: z = M^-1 r for every chart whose CG is still running.  Set up from an assembled
// system on construction; bound once to the CG's r and z; apply() only enqueues launches
// (capturable in a CUDA graph) and returns how many.
struct SepPrecond {
  virtual ~SepPrecond() = default;
  virtual bool native_fp64() const = 0;  // applies in FP64 under the FP64 loop (else FP32 copies)
  virtual bool flexible() const = 0;     // varies between applications: flexible-CG beta
  virtual void bind(Ctx& ctx, void* r, void* z, bool fp64) = 0;
  virtual int apply(Ctx& ctx, const int32_t* done) = 0;
  // device flag set when an application gave up a bounded device-side wait (nullptr: none)
  virtual const int* error_flag() const { return nullptr; }
};

// Batched aggregation AMG (amg.cu): hierarchy built on the device, one V(1,1) cycle per apply.
struct AmgHierarchy;
AmgHierarchy* amg_setup(Ctx& ctx, const DevSystem& sys, bool smooth, std::string& info);
void amg_free(AmgHierarchy* H);
int amg_levels(const AmgHierarchy* H);
// One level of the hierarchy amg_setup builds for `sys`, copied to the host: its operator
// (FP64), and when a coarser level follows, the prolongator to it and the aggregate of each row.
struct AmgLevelHost {
  int n_levels = 0;
  bool smoothed = false;  // this level's prolongator is smoothed
  int64_t n = 0, nnz = 0, n_next = 0, pnnz = 0;
  std::vector<int32_t> rp, cols;
  std::vector<double> vals;
  std::vector<int64_t> poff;
  std::vector<int32_t> pc, agg;
  std::vector<float> pv;
};
void amg_export_level(Ctx& ctx, const DevSystem& sys, bool smooth, int level, AmgLevelHost& out);
void amg_bind(Ctx& ctx, AmgHierarchy* H, float* r0, float* z0);
int amg_apply(Ctx& ctx, AmgHierarchy* H, const int32_t* done);
std::unique_ptr<SepPrecond> make_amg(Ctx& ctx, const DevSystem& sys, bool smooth);

// Batched IC(0), natural or multi-colour ordering (ic0.cu): factor on the device, two
// level-scheduled triangular sweeps per apply.
std::unique_ptr<SepPrecond> make_ic0(Ctx& ctx, const DevSystem& sys, bool colored);
// One FP64 application z = (L L^T)^-1 r on device vectors (factor built and dropped).
void ic0_apply_once(Ctx& ctx, const DevSystem& sys, const double* d_r, double* d_z, int* fwd_levels);
void ic0_export(Ctx& ctx, const DevSystem& sys, bool colored, std::vector<int64_t>& ptr, std::vector<int32_t>& cols,
                std::vector<double>& vals, std::vector<int32_t>& to_orig, int& levels, int& colours);

// The 16-bit column stream of `sys` (cols16, cbase), built on the device.
void narrow_columns(Ctx& ctx, DevSystem& sys);
// The same for any chart-blocked CSR operator (an AMG level): chart-relative when every chart
// has at most 65536 rows, else row-relative (*rowrel); false (null pointers) when an entry of
// a row-relative operator lies more than 32767 rows from its row.
bool narrow_operator(Ctx& ctx, int64_t n, int64_t nnz, int64_t n_charts, const std::vector<int64_t>& h_chart_row,
                     const int64_t* chart_row, const int32_t* row_ptr, const int32_t* cols, const std::string& tag,
                     uint16_t** c16, int32_t** cbase, bool* rowrel);

// x (nrhs * n_rows, device) <- A^-1 b per chart.  Returns per-chart results (host).
std::vector<ChartResult> pcg_solve(Ctx& ctx, DevSystem& sys, double* x, const SolveOpts& o);

// Assembly of the LSCM systems of a batch on the device (see assemble.cu).
struct DevBatch {
  int64_t n_charts = 0, n_verts = 0, n_tris = 0;
  int64_t* vert_off = nullptr;  // n_charts + 1
  int64_t* tri_off = nullptr;
  double* p3 = nullptr;         // 3 * n_verts
  int32_t* tris = nullptr;      // 3 * n_tris, chart-local
  uint8_t* pinned = nullptr;
  double* pin_uv = nullptr;     // 2 * n_verts
  double* p2 = nullptr;         // 2 * n_verts
  // The one-call entry's split upload (n_parts > 0): triangles [part_tri[k], part_tri[k + 1])
  // and their charts' positions are still being copied on Ctx::side until part_ready[k]
  // (nullptr once on the device), the pin flags until pins_ready, the pin targets and frame
  // positions until rest_ready.  The assembly waits for each before its first use.
  static constexpr int kMaxParts = 16;
  int n_parts = 0;
  int64_t part_tri[kMaxParts + 1] = {};
  cudaEvent_t part_ready[kMaxParts] = {};
  cudaEvent_t pins_ready = nullptr;
  cudaEvent_t rest_ready = nullptr;
  // produced by assembly
  int64_t* row_of = nullptr;    // n_verts + 1: exclusive count of free vertices (row id if free)
  int32_t* row_vert = nullptr;  // n_rows: packed vertex of each row
  int32_t* tri_g = nullptr;     // 3 * n_tris: packed vertex ids
  double* cot = nullptr;        // 3 * n_tris: clamped corner cotangents (0 where skipped)
  int64_t* rec_off = nullptr;   // n_verts + 1: incidence records of each free vertex
  int2* rec = nullptr;          // (neighbour, corner) sorted per vertex
  double* coef = nullptr;       // edge coefficient at each neighbour's first record (-1: dropped)
  std::vector<int64_t> h_vert_off, h_tri_off;
};

void assemble_lscm(Ctx& ctx, DevBatch& bt, DevSystem& sys, double angle_mix);

// Adjoint of the LSCM solve (adjoint.cu): the batch's vertex-position gradient of a loss
// given its gradient with respect to the free rows' solution (g, 2 per row): lam = A^-1 g
// with the same operator and preconditioner, then the assembly's reverse pass.
void lscm_backward(Ctx& ctx, DevBatch& bt, const DevSystem& sys, const double* x, const double* g, const SolveOpts& o,
                   double* dp3, std::vector<ChartResult>& res);
// Per-triangle distortion loss sum_t area_t (s1/s2 - 1)^2 of a UV layout and its gradients
// (accumulated into duv / dp3 when non-null); loss per chart (host).
void distortion_loss(Ctx& ctx, const DevBatch& bt, const double* uv, double* duv, double* dp3,
                     std::vector<double>& loss);
// chart_distortion (unwrap/src/metrics.rs:73-141) per chart: conformal mean / max, area
// ratio mean, flips, folds.
void chart_metrics(Ctx& ctx, const DevBatch& bt, const double* uv, std::vector<double>& out5);
// rectangularize (unwrap/src/metrics.rs:147-227) per chart: q (2 * n_verts) in [0,1]^2 per
// chart, ext (2 * n_charts) the extents before normalisation; border: one flag per vertex.
void rectangularize(Ctx& ctx, const DevBatch& bt, const double* uv, const uint8_t* border, double* q, double* ext);
// Bitwise comparison of div_rn / sqrt_rn with the hardware operations on n seeded inputs of
// class `mode` (0-5, see assemble.cu); returns the mismatch count, first4 = (a, b, got, want)
// of the first mismatch.
int64_t fp64_selftest(Ctx& ctx, int mode, uint64_t seed, int64_t n, double* first4);

// Damped driver update (unfold_chart's loop, lscm.rs:570-719) on the device: writes uv
// (2 * n_verts) and per-chart driver iterations / err_accum.
void driver_update(Ctx& ctx, DevBatch& bt, const DevSystem& sys, const double* x, int max_iter, double* uv,
                   std::vector<int32_t>& iters, std::vector<double>& err_accum);
// KeepMetric (lscm.rs:544-568, :642-676): the slack column u (2 * n_rows) of the bordered
// system (d_flip: per chart, the sign of the UV area of p2), and the driver whose every iteration forms x = y_b - aux y_u from the current uv
// (y_b = K^-1 b, y_u = K^-1 u; d_target per chart).
void keep_metric_rhs(Ctx& ctx, DevBatch& bt, DevSystem& sys, const double* d_flip, double* u);
void driver_keep_metric(Ctx& ctx, DevBatch& bt, const DevSystem& sys, const double* yb, const double* yu,
                        const double* d_target, int max_iter, double* uv, std::vector<int32_t>& iters,
                        std::vector<double>& err_accum);

struct Ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  // a second stream for host-to-device copies that overlap the first assembly kernels, and
  // the events ordering it against `stream`
  cudaStream_t side = nullptr;
  cudaEvent_t ev_core = nullptr, ev_pins = nullptr, ev_rest = nullptr;
  cudaEvent_t ev_part[DevBatch::kMaxParts] = {};
  Workspace ws;
  PinnedHost pinned;
  std::string last_error;
  // the last batch's assembled system (for ruv_export_chart_system)
  DevSystem last_sys;
  bool have_last = false;
  int lanes_per_row = 0;   // SpMV sub-warp width (0 = from the row-length profile)
  int unroll = 0;          // SpMV rows in flight per sub-warp (0 = from the shape)
  int tile_rows = 1024;    // rows per CTA tile (the autotuner's pick on the disks and the height fields)
  // the bulk-copy SpMV (k_spmv_tma): 0 off (the default: on the 4096-disk step the CSR-vector
  // kernel's iteration ran faster), 1 on; the autotuner chooses it, RUV_SPMV_TMA=0/1 overrides
  int spmv_tma = 0;
  // the batch resident on the device (ruv_lscm_upload)
  DevBatch resident;
  bool have_batch = false;
  bool have_uv = false;
  double timings[4] = {0.0, 0.0, 0.0, 0.0};  // assembly, PCG, driver, preconditioner setup (in PCG)
  int64_t launches = 0;  // kernels enqueued by this context so far
};

// Standalone timing of the batched SpMV kernel on an assembled system (see ruv_bench_spmv).
double bench_spmv(Ctx& ctx, DevSystem& sys, bool mixed, int reps, int n_buffers, double* bytes,
                  double* stream_bytes);

struct TuneResult {
  int lpr, unroll, tile_rows, tma;
  double ms;
};
TuneResult autotune_spmv(Ctx& ctx, DevSystem& sys, bool mixed, int reps);

}  // namespace ruv
