// C ABI (include/ruv.h): the drop-in for the reference's GpuSolver boundary
// (gpu/src/solver.rs:104-565) and the batched unfold_chart solve (unwrap/src/lscm.rs:471-727).
// Every entry point catches internally and reports a ruv_status; no exception crosses.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>

#include "system.cuh"

using namespace ruv;

struct ruv_ctx {
  Ctx c;
};

struct ruv_prepared {
  Prepared p;
};

namespace {

ruv_status fail(ruv_ctx* ctx, ruv_status s, const std::string& msg) {
  if (ctx) ctx->c.last_error = msg;
  return s;
}

template <class F>
ruv_status guarded(ruv_ctx* ctx, F&& body) {
  struct CounterScope {
    explicit CounterScope(ruv_ctx* c) { g_launch_counter = c ? &c->c.launches : nullptr; }
    ~CounterScope() { g_launch_counter = nullptr; }
  } scope(ctx);
  try {
    if (ctx) {
      ctx->c.last_error.clear();
      cudaError_t e = cudaSetDevice(ctx->c.device);
      if (e != cudaSuccess) return fail(ctx, RUV_ERR_NO_DEVICE, cudaGetErrorString(e));
    }
    return body();
  } catch (const Error& e) {
    if (ctx) {
      // an error thrown while the stream was being captured leaves the capture open: close it
      // so that the context's stream stays usable for the next call
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(ctx->c.stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(ctx->c.stream, &g);
        if (g) cudaGraphDestroy(g);
      }
      cudaGetLastError();
      cudaStreamSynchronize(ctx->c.stream);
      cudaStreamSynchronize(ctx->c.side);
    }
    cudaGetLastError();
    return fail(ctx, e.status, e.msg);
  } catch (const std::bad_alloc&) {
    return fail(ctx, RUV_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(ctx, RUV_ERR_INTERNAL, e.what());
  } catch (...) {
    return fail(ctx, RUV_ERR_INTERNAL, "unknown error");
  }
}

// Copy through the SMs between device memory and a page-locked, mapped host buffer (read or
// written over its device mapping), 16 bytes per access with four loads in flight per thread
// (head and tail bytewise).
__global__ void k_h2d(const unsigned char* __restrict__ src, unsigned char* __restrict__ dst, size_t head,
                      size_t n16, size_t tail) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (size_t)gridDim.x * blockDim.x;
  if (tid < head) dst[tid] = src[tid];
  const uint4* s4 = reinterpret_cast<const uint4*>(src + head);
  uint4* d4 = reinterpret_cast<uint4*>(dst + head);
  size_t i = tid;
  for (; i + 3 * nth < n16; i += 4 * nth) {
    const uint4 a = s4[i], b = s4[i + nth], c = s4[i + 2 * nth], d = s4[i + 3 * nth];
    d4[i] = a;
    d4[i + nth] = b;
    d4[i + 2 * nth] = c;
    d4[i + 3 * nth] = d;
  }
  for (; i < n16; i += nth) d4[i] = s4[i];
  if (tid < tail) dst[head + 16 * n16 + tid] = src[head + 16 * n16 + tid];
}

// The copy kernel's grid: `knob` (RUV_H2D_GRID for host-to-device, RUV_D2H_GRID back) CTAs of
// 256 threads, default a quarter of the SMs.  Four 16-byte loads in flight per thread over 38
// CTAs (608 KB) already hold the host link's rate, and the SMs the copy leaves free keep the
// assembly kernels it overlaps at speed: on the 4096-disk one-call solve 38 CTAs ran 0.9 ms
// faster per call than one CTA per SM (152), 19 CTAs the same as 38; the copy back of the
// UVs took the same time with 38, 76 or 152 CTAs.
unsigned h2d_grid(size_t n16, const char* knob = "RUV_H2D_GRID") {
  const char* g = std::getenv(knob);
  int dev_id = 0, sms = 0;
  RUV_CUDA(cudaGetDevice(&dev_id));
  RUV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
  const int64_t want = g ? std::max(1, std::atoi(g)) : std::max(1, sms / 4);
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, div_up((int64_t)n16, 256)));
}

// RUV_H2D_KERNEL=0 (read on every copy): host copies through cudaMemcpyAsync only
bool copies_by_engines() {
  const char* e = std::getenv("RUV_H2D_KERNEL");
  return e && e[0] == '0';
}

// n bytes host -> device on stream st.  Where the host buffer is page-locked and mapped (and
// both ends share their offset from a 16-byte boundary) the copy is k_h2d; otherwise
// cudaMemcpyAsync.  On GB300 hosts copy-engine transfers of pinned memory ran at 211 GB/s but
// now and then many times slower right after heavy GPU work, while the SMs pulling the same
// mapped buffer held 211 GB/s in every repetition.  RUV_H2D_KERNEL=0: always cudaMemcpyAsync.
void h2d(Ctx& c, void* dev, const void* host, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return;
  const bool off = copies_by_engines();
  cudaPointerAttributes a{};
  const void* src = nullptr;
  if (!off) {
    if (cudaPointerGetAttributes(&a, host) == cudaSuccess) {
      if (a.type == cudaMemoryTypeHost && a.devicePointer) src = a.devicePointer;
    } else {
      cudaGetLastError();  // clear what the query left (the copy below reports its own errors)
    }
  }
  const uintptr_t sa = (uintptr_t)src, da = (uintptr_t)dev;
  if (!src || (sa & 15) != (da & 15)) {
    RUV_CUDA(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, st));
    return;
  }
  const size_t head = std::min<size_t>(bytes, (16 - (sa & 15)) & 15);
  const size_t n16 = (bytes - head) / 16, tail = bytes - head - 16 * n16;
  const unsigned grid = h2d_grid(n16);
  k_h2d<<<grid, 256, 0, st>>>(static_cast<const unsigned char*>(src), static_cast<unsigned char*>(dev), head, n16,
                              tail);
  count_launches(1);
  RUV_LAUNCH_CHECK();
}

// n bytes device -> host on stream st: the same choice as h2d (k_h2d writing through the
// host buffer's device mapping where it is page-locked and mapped, else cudaMemcpyAsync).
void d2h(Ctx& c, void* host, const void* dev, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return;
  const bool off = copies_by_engines();
  cudaPointerAttributes a{};
  void* dst = nullptr;
  if (!off) {
    if (cudaPointerGetAttributes(&a, host) == cudaSuccess) {
      if (a.type == cudaMemoryTypeHost && a.devicePointer) dst = a.devicePointer;
    } else {
      cudaGetLastError();
    }
  }
  const uintptr_t sa = (uintptr_t)dev, da = (uintptr_t)dst;
  if (!dst || (sa & 15) != (da & 15)) {
    RUV_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, st));
    return;
  }
  const size_t head = std::min<size_t>(bytes, (16 - (sa & 15)) & 15);
  const size_t n16 = (bytes - head) / 16, tail = bytes - head - 16 * n16;
  const unsigned grid = h2d_grid(n16, "RUV_D2H_GRID");
  k_h2d<<<grid, 256, 0, st>>>(static_cast<const unsigned char*>(dev), static_cast<unsigned char*>(dst), head, n16,
                              tail);
  count_launches(1);
  RUV_LAUNCH_CHECK();
}

template <class T>
T* upload(Ctx& c, const std::string& name, const T* host, int64_t n, cudaStream_t st = nullptr) {
  T* d = c.ws.get<T>(name, n);
  if (n > 0) h2d(c, d, host, sizeof(T) * n, st ? st : c.stream);
  return d;
}

int worst(int a, int b) {
  // NOT_CONVERGED < BREAKDOWN in severity; any non-OK beats OK
  if (a == RUV_OK) return b;
  if (b == RUV_OK) return a;
  return a > b ? a : b;
}

// the context's events of the split upload
std::vector<cudaEvent_t*> copy_events(Ctx& c) {
  std::vector<cudaEvent_t*> e{&c.ev_core, &c.ev_pins, &c.ev_rest};
  for (cudaEvent_t& p : c.ev_part) e.push_back(&p);
  return e;
}

// Orders the resident batch's side-stream copies that the assembly has not waited for yet
// before everything enqueued next on the main stream (a path that failed or returned before
// the assembly, or before its last wait).
void order_pending_copies(Ctx& c) {
  DevBatch& bt = c.resident;
  std::vector<cudaEvent_t*> pending{&bt.pins_ready, &bt.rest_ready};
  for (cudaEvent_t& p : bt.part_ready) pending.push_back(&p);
  for (cudaEvent_t* e : pending)
    if (*e) {
      cudaStreamWaitEvent(c.stream, *e, 0);
      *e = nullptr;
    }
}

}  // namespace

extern "C" {

int32_t ruv_abi_version(void) { return RUV_ABI_VERSION; }

const char* ruv_status_str(ruv_status s) {
  switch (s) {
    case RUV_OK: return "ok";
    case RUV_ERR_NO_DEVICE: return "no usable CUDA device";
    case RUV_ERR_BAD_INPUT: return "bad input";
    case RUV_ERR_OOM: return "out of device memory";
    case RUV_ERR_NOT_CONVERGED: return "not converged";
    case RUV_ERR_BREAKDOWN: return "breakdown";
    case RUV_ERR_TIMEOUT: return "device wait timed out";
    case RUV_ERR_LAUNCH: return "CUDA launch/runtime failure";
    default: return "internal error";
  }
}

ruv_status ruv_ctx_create(ruv_ctx** out, int32_t device) {
  if (!out) return RUV_ERR_BAD_INPUT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return RUV_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return RUV_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return RUV_ERR_NO_DEVICE;
  // the kernels are built for sm_103a only
  if (!(prop.major == 10 && prop.minor == 3)) return RUV_ERR_NO_DEVICE;
  std::unique_ptr<ruv_ctx> ctx(new (std::nothrow) ruv_ctx());
  if (!ctx) return RUV_ERR_OOM;
  ctx->c.device = device;
  ctx->c.sm_count = prop.multiProcessorCount;
  // launch-shape overrides for the tuner (RUV_LPR, RUV_UNROLL, RUV_TILE_ROWS)
  if (const char* e = std::getenv("RUV_LPR")) ctx->c.lanes_per_row = std::atoi(e);
  if (const char* e = std::getenv("RUV_UNROLL")) ctx->c.unroll = std::atoi(e);
  if (const char* e = std::getenv("RUV_TILE_ROWS")) ctx->c.tile_rows = std::max(32, std::atoi(e));
  if (cudaSetDevice(device) != cudaSuccess) return RUV_ERR_NO_DEVICE;
  if (cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking) != cudaSuccess) return RUV_ERR_LAUNCH;
  bool ok = cudaStreamCreateWithFlags(&ctx->c.side, cudaStreamNonBlocking) == cudaSuccess;
  for (cudaEvent_t* e : copy_events(ctx->c))
    ok = ok && cudaEventCreateWithFlags(e, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaStreamDestroy(ctx->c.stream);
    if (ctx->c.side) cudaStreamDestroy(ctx->c.side);
    for (cudaEvent_t* e : copy_events(ctx->c))
      if (*e) cudaEventDestroy(*e);
    return RUV_ERR_LAUNCH;
  }
  *out = ctx.release();
  return RUV_OK;
}

void ruv_ctx_destroy(ruv_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  cudaStreamSynchronize(ctx->c.side);
  ctx->c.ws.release();
  cudaStreamDestroy(ctx->c.stream);
  cudaStreamDestroy(ctx->c.side);
  for (cudaEvent_t* e : copy_events(ctx->c)) cudaEventDestroy(*e);
  delete ctx;
}

const char* ruv_last_error(const ruv_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : ""; }

ruv_status ruv_debug_fail_alloc(ruv_ctx* ctx, int64_t nth) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  ctx->c.ws.fail_countdown = nth > 0 ? nth : 0;
  return RUV_OK;
}

void ruv_unfold_opts_default(ruv_unfold_opts* o) {
  if (!o) return;
  o->angle_mix = 1.0;
  o->mix_w = 1.0;
  o->max_iter = 100;
  o->precond = RUV_PRECOND_JACOBI;
  o->precision = RUV_PREC_MIXED;
  o->tol = 1e-12;
  o->max_cg_iter = 1024 * 16;
}

// A host CSR system checked and uploaded as a one-chart DevSystem (nrhs = 1).  Returns a
// non-OK status (with the context's message set) for a malformed system (solver.rs:296-299).
static ruv_status host_system(ruv_ctx* ctx, int32_t n, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                              const double* b, DevSystem& sys, std::vector<double>& diag) {
  if (n <= 0 || !row_ptr || !cols || !vals || !b) return fail(ctx, RUV_ERR_BAD_INPUT, "empty system or null buffer");
  if (row_ptr[0] != 0) return fail(ctx, RUV_ERR_BAD_INPUT, "row_ptr[0] != 0");
  for (int32_t i = 0; i < n; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return fail(ctx, RUV_ERR_BAD_INPUT, "row_ptr not monotone");
  const int64_t nnz = row_ptr[n];
  diag.assign(n, 0.0);
  for (int32_t i = 0; i < n; ++i) {
    bool found = false;
    for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
      if (cols[k] < 0 || cols[k] >= n) return fail(ctx, RUV_ERR_BAD_INPUT, "column index out of range");
      if (cols[k] == i && !found) {  // CsrMatrix::row_get returns the first match
        diag[i] = vals[k];
        found = true;
      }
    }
  }
  Ctx& c = ctx->c;
  sys = DevSystem();
  sys.n_charts = 1;
  sys.n_rows = n;
  sys.nnz = nnz;
  sys.nrhs = 1;
  sys.h_chart_row = {0, (int64_t)n};
  sys.chart_row = upload(c, "cg.chart_row", sys.h_chart_row.data(), 2);
  sys.row_ptr = upload(c, "cg.row_ptr", row_ptr, (int64_t)n + 1);
  sys.cols = upload(c, "cg.cols", cols, nnz);
  sys.vals = upload(c, "cg.vals", vals, nnz);
  std::vector<float> v32(vals, vals + nnz);
  sys.vals32 = upload(c, "cg.vals32", v32.data(), nnz);
  sys.diag = upload(c, "cg.diag", diag.data(), n);
  sys.b = upload(c, "cg.b", b, n);
  return RUV_OK;
}

static bool known_precond(int pc) { return pc >= RUV_PRECOND_NONE && pc <= RUV_PRECOND_AMG_SA; }

ruv_status ruv_cg_solve(ruv_ctx* ctx, int32_t n, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                        const double* b, double* x_out, int64_t max_iter, double tol, ruv_precond pc,
                        int64_t* iters_out) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    if (!x_out) return fail(ctx, RUV_ERR_BAD_INPUT, "null output buffer");
    if (!known_precond(pc)) return fail(ctx, RUV_ERR_BAD_INPUT, "unknown preconditioner");
    Ctx& c = ctx->c;
    DevSystem sys;
    std::vector<double> diag;
    const ruv_status hs = host_system(ctx, n, row_ptr, cols, vals, b, sys, diag);
    if (hs != RUV_OK) return hs;
    if (pc == RUV_PRECOND_JACOBI)
      for (int32_t i = 0; i < n; ++i)
        if (std::fabs(diag[i]) < 1e-300) return fail(ctx, RUV_ERR_BAD_INPUT, "Jacobi: zero diagonal");
    double* x = c.ws.get<double>("cg.x", n);
    SolveOpts o;
    o.precond = pc;
    o.precision = RUV_PREC_FP64;
    o.tol = tol;
    o.max_iter = max_iter;
    auto res = pcg_solve(c, sys, x, o);
    if (iters_out) *iters_out = res[0].iters;
    if (res[0].status != RUV_OK) return fail(ctx, (ruv_status)res[0].status, "CG did not converge / broke down");
    RUV_CUDA(cudaMemcpyAsync(x_out, x, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    RUV_CUDA(cudaStreamSynchronize(c.stream));
    for (int32_t i = 0; i < n; ++i)
      if (!std::isfinite(x_out[i])) return fail(ctx, RUV_ERR_BREAKDOWN, "non-finite solution");  // solver.rs:561-563
    return RUV_OK;
  });
}

ruv_status ruv_apply_ic0(ruv_ctx* ctx, int32_t n, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                         const double* r, double* z_out) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    if (!z_out) return fail(ctx, RUV_ERR_BAD_INPUT, "null output buffer");
    Ctx& c = ctx->c;
    DevSystem sys;
    std::vector<double> diag;
    const ruv_status hs = host_system(ctx, n, row_ptr, cols, vals, r, sys, diag);  // b carries r
    if (hs != RUV_OK) return hs;
    double* z = c.ws.get<double>("ic0.z", n);
    ic0_apply_once(c, sys, sys.b, z, nullptr);
    RUV_CUDA(cudaMemcpyAsync(z_out, z, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    RUV_CUDA(cudaStreamSynchronize(c.stream));
    return RUV_OK;
  });
}

ruv_status ruv_ic0_export(ruv_ctx* ctx, int32_t n, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                          int32_t colored, int64_t cap, int64_t* l_ptr, int32_t* l_cols, double* l_vals,
                          int32_t* to_orig, int64_t* nnz_out, int32_t* levels_out, int32_t* colours_out) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    if (!l_ptr || !to_orig || !nnz_out || !levels_out || !colours_out || (cap > 0 && (!l_cols || !l_vals)))
      return fail(ctx, RUV_ERR_BAD_INPUT, "null output buffer");
    Ctx& c = ctx->c;
    DevSystem sys;
    std::vector<double> diag, zero(n > 0 ? n : 0, 0.0);
    const ruv_status hs = host_system(ctx, n, row_ptr, cols, vals, zero.data(), sys, diag);
    if (hs != RUV_OK) return hs;
    std::vector<int64_t> p;
    std::vector<int32_t> lc, perm;
    std::vector<double> lv;
    int levels = 0, colours = 0;
    ic0_export(c, sys, colored != 0, p, lc, lv, perm, levels, colours);
    *nnz_out = (int64_t)lc.size();
    *levels_out = levels;
    *colours_out = colours;
    std::copy(p.begin(), p.end(), l_ptr);
    std::copy(perm.begin(), perm.end(), to_orig);
    if ((int64_t)lc.size() > cap) return fail(ctx, RUV_ERR_BAD_INPUT, "factor larger than the output capacity");
    std::copy(lc.begin(), lc.end(), l_cols);
    std::copy(lv.begin(), lv.end(), l_vals);
    return RUV_OK;
  });
}

ruv_status ruv_amg_export(ruv_ctx* ctx, int32_t n, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                          int32_t smoothed, int32_t level, int64_t cap, int64_t* sizes, int64_t* a_ptr, int32_t* a_cols,
                          double* a_vals, int64_t* p_ptr, int32_t* p_cols, float* p_vals, int32_t* agg) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    if (!sizes || cap < 0) return fail(ctx, RUV_ERR_BAD_INPUT, "null sizes or negative capacity");
    if (cap > 0 && (!a_ptr || !a_cols || !a_vals || !p_ptr || !p_cols || !p_vals || !agg))
      return fail(ctx, RUV_ERR_BAD_INPUT, "null output buffer");
    Ctx& c = ctx->c;
    DevSystem sys;
    std::vector<double> diag, zero(n > 0 ? n : 0, 0.0);
    const ruv_status hs = host_system(ctx, n, row_ptr, cols, vals, zero.data(), sys, diag);
    if (hs != RUV_OK) return hs;
    AmgLevelHost h;
    amg_export_level(c, sys, smoothed != 0, level, h);
    sizes[0] = h.n_levels;
    sizes[1] = h.smoothed ? 1 : 0;
    sizes[2] = h.n;
    sizes[3] = h.n_next;
    sizes[4] = h.nnz;
    sizes[5] = h.pnnz;
    if (cap == 0) return RUV_OK;
    if (std::max({h.n + 1, h.nnz, h.pnnz}) > cap) return fail(ctx, RUV_ERR_BAD_INPUT, "level larger than the output capacity");
    for (int64_t i = 0; i <= h.n; ++i) a_ptr[i] = h.rp[i];
    std::copy(h.cols.begin(), h.cols.end(), a_cols);
    std::copy(h.vals.begin(), h.vals.end(), a_vals);
    if (h.n_next > 0) {
      std::copy(h.poff.begin(), h.poff.end(), p_ptr);
      std::copy(h.pc.begin(), h.pc.end(), p_cols);
      std::copy(h.pv.begin(), h.pv.end(), p_vals);
      std::copy(h.agg.begin(), h.agg.end(), agg);
    } else {
      std::fill(p_ptr, p_ptr + h.n + 1, 0);
      std::fill(agg, agg + h.n, -1);
    }
    return RUV_OK;
  });
}

namespace {
// The batch upload.  With `overlap` (the one-call solve) the triangles and positions go in
// parts split at chart boundaries (about equal triangle counts; RUV_UPLOAD_PARTS, default 8):
// the first part on the main stream, the others and then the arrays the assembly reads only
// after its cotangent pass (pin flags, pin targets, tangent-frame positions) on the side
// stream, under the kernels of the parts before them.  bt.part_ready, bt.pins_ready and
// bt.rest_ready order them before their first use.
ruv_status upload_batch(ruv_ctx* ctx, const ruv_lscm_batch* in, bool overlap);
}  // namespace

ruv_status ruv_lscm_upload(ruv_ctx* ctx, const ruv_lscm_batch* in) { return upload_batch(ctx, in, false); }

namespace {
ruv_status upload_batch(ruv_ctx* ctx, const ruv_lscm_batch* in, bool overlap) {
  if (!ctx || !in) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    const int64_t NC = in->n_charts;
    if (NC < 0 || !in->vert_off || !in->tri_off) return fail(ctx, RUV_ERR_BAD_INPUT, "null offsets");
    if (in->vert_off[0] != 0 || in->tri_off[0] != 0) return fail(ctx, RUV_ERR_BAD_INPUT, "offsets must start at 0");
    for (int64_t c = 0; c < NC; ++c)
      if (in->vert_off[c + 1] < in->vert_off[c] || in->tri_off[c + 1] < in->tri_off[c])
        return fail(ctx, RUV_ERR_BAD_INPUT, "offsets must be non-decreasing");
    const int64_t NV = in->vert_off[NC], NT = in->tri_off[NC];
    if ((NV > 0 && (!in->p3 || !in->pinned || !in->pin_uv || !in->p2)) || (NT > 0 && !in->tris))
      return fail(ctx, RUV_ERR_BAD_INPUT, "null array");
    Ctx& c = ctx->c;
    c.have_batch = false;
    c.have_uv = false;
    order_pending_copies(c);
    DevBatch& bt = c.resident;
    bt = DevBatch();
    bt.n_charts = NC;
    bt.n_verts = NV;
    bt.n_tris = NT;
    bt.h_vert_off.assign(in->vert_off, in->vert_off + NC + 1);
    bt.h_tri_off.assign(in->tri_off, in->tri_off + NC + 1);
    bt.vert_off = upload(c, "in.vert_off", in->vert_off, NC + 1);
    bt.tri_off = upload(c, "in.tri_off", in->tri_off, NC + 1);
    bt.p3 = c.ws.get<double>("in.p3", 3 * NV);
    bt.tris = c.ws.get<int32_t>("in.tris", 3 * NT);
    // part k: charts [cs[k], cs[k + 1]), cs[k] the first chart boundary at or past k / P of
    // the triangles
    const char* parts_env = std::getenv("RUV_UPLOAD_PARTS");
    const int env_parts = parts_env ? std::atoi(parts_env) : 8;
    const int P = overlap ? (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)env_parts, DevBatch::kMaxParts, NC}))
                          : 1;
    std::vector<int64_t> cs(P + 1, NC);
    cs[0] = 0;
    for (int k = 1; k < P; ++k)
      cs[k] = std::max(cs[k - 1], (int64_t)(std::lower_bound(in->tri_off, in->tri_off + NC + 1, NT * k / P) -
                                            in->tri_off));
    auto copy_part = [&](int k, cudaStream_t st) {
      const int64_t v0 = in->vert_off[cs[k]], v1 = in->vert_off[cs[k + 1]];
      const int64_t t0 = in->tri_off[cs[k]], t1 = in->tri_off[cs[k + 1]];
      if (v1 > v0) h2d(c, bt.p3 + 3 * v0, in->p3 + 3 * v0, sizeof(double) * 3 * (v1 - v0), st);
      if (t1 > t0) h2d(c, bt.tris + 3 * t0, in->tris + 3 * t0, sizeof(int32_t) * 3 * (t1 - t0), st);
    };
    copy_part(0, c.stream);
    cudaStream_t rest = c.stream;
    if (overlap) {  // after everything already on the main stream, then in parallel with it
      RUV_CUDA(cudaEventRecord(c.ev_core, c.stream));
      RUV_CUDA(cudaStreamWaitEvent(c.side, c.ev_core, 0));
      rest = c.side;
    }
    struct SideGuard {  // an exit before every side copy was enqueued: the main stream waits
      Ctx& c;
      bool on;
      ~SideGuard() {
        if (!on) return;
        cudaEventRecord(c.ev_rest, c.side);
        cudaStreamWaitEvent(c.stream, c.ev_rest, 0);
        c.resident.n_parts = 0;
        for (cudaEvent_t& e : c.resident.part_ready) e = nullptr;
        c.resident.pins_ready = c.resident.rest_ready = nullptr;
      }
    } guard{c, overlap};
    for (int k = 1; k < P; ++k) {
      copy_part(k, rest);
      RUV_CUDA(cudaEventRecord(c.ev_part[k], rest));
      bt.part_ready[k] = c.ev_part[k];
    }
    bt.pinned = upload(c, "in.pinned", in->pinned, NV, rest);
    if (overlap) {
      RUV_CUDA(cudaEventRecord(c.ev_pins, rest));
      bt.pins_ready = c.ev_pins;
    }
    bt.pin_uv = upload(c, "in.pin_uv", in->pin_uv, 2 * NV, rest);
    bt.p2 = upload(c, "in.p2", in->p2, 2 * NV, rest);
    if (overlap) {
      RUV_CUDA(cudaEventRecord(c.ev_rest, rest));
      bt.rest_ready = c.ev_rest;
      bt.n_parts = P;
      for (int k = 0; k <= P; ++k) bt.part_tri[k] = in->tri_off[cs[k]];
      guard.on = false;
    }
    c.have_batch = true;
    return RUV_OK;
  });
}
}  // namespace

ruv_status ruv_lscm_solve_resident(ruv_ctx* ctx, const ruv_unfold_opts* opts, ruv_chart_stat* stats) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    if (!c.have_batch) return fail(ctx, RUV_ERR_BAD_INPUT, "no batch uploaded on this context");
    ruv_unfold_opts o;
    ruv_unfold_opts_default(&o);
    if (opts) o = *opts;
    if (!(o.mix_w > 0.0)) return fail(ctx, RUV_ERR_BAD_INPUT, "mix_w must be > 0 (lscm.rs:479)");
    if (!known_precond(o.precond)) return fail(ctx, RUV_ERR_BAD_INPUT, "unknown preconditioner");
    DevBatch& bt = c.resident;
    const int64_t NC = bt.n_charts, NV = bt.n_verts;
    if (NC == 0) {
      c.have_uv = true;
      c.timings[0] = c.timings[1] = c.timings[2] = c.timings[3] = 0.0;
      return RUV_OK;
    }
    cudaEvent_t ev[4];
    for (auto& e : ev) RUV_CUDA(cudaEventCreate(&e));
    struct EvGuard {
      cudaEvent_t* e;
      ~EvGuard() {
        for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]);
      }
    } guard{ev};
    DevSystem& sys = c.last_sys;
    c.have_last = false;
    c.have_uv = false;
    RUV_CUDA(cudaEventRecord(ev[0], c.stream));
    assemble_lscm(c, bt, sys, o.angle_mix);
    c.have_last = true;
    RUV_CUDA(cudaEventRecord(ev[1], c.stream));
    double* x = c.ws.get<double>("lscm.x", 2 * sys.n_rows);
    SolveOpts so;
    so.precond = o.precond;
    so.precision = o.precision;
    so.tol = o.tol;
    so.max_iter = o.max_cg_iter > 0 ? o.max_cg_iter : 16384;
    auto res = pcg_solve(c, sys, x, so);
    RUV_CUDA(cudaEventRecord(ev[2], c.stream));
    double* uv = c.ws.get<double>("lscm.uv", 2 * NV);
    std::vector<int32_t> iters;
    std::vector<double> err_accum;
    driver_update(c, bt, sys, x, o.max_iter, uv, iters, err_accum);
    RUV_CUDA(cudaEventRecord(ev[3], c.stream));
    RUV_CUDA(cudaEventSynchronize(ev[3]));
    for (int k = 0; k < 3; ++k) {
      float ms = 0.f;
      RUV_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
      c.timings[k] = ms;
    }

    c.have_uv = true;
    int w = RUV_OK;
    for (int64_t k = 0; k < NC; ++k) {
      w = worst(w, res[k].status);
      if (stats) {
        stats[k].status = res[k].status;
        stats[k].driver_iters = iters[k];
        stats[k].cg_iters = res[k].iters;
        stats[k].n_free = (int32_t)(sys.h_chart_row[k + 1] - sys.h_chart_row[k]);
        stats[k].rel_res = res[k].rel_res;
        stats[k].err_accum = err_accum[k];
      }
    }
    if (w != RUV_OK) return fail(ctx, (ruv_status)w, "at least one chart did not converge");
    return RUV_OK;
  });
}

ruv_status ruv_lscm_download_uv(ruv_ctx* ctx, double* uv_out) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    if (!c.have_uv) return fail(ctx, RUV_ERR_BAD_INPUT, "no solved batch on this context");
    const int64_t NV = c.resident.n_verts;
    if (NV > 0 && !uv_out) return fail(ctx, RUV_ERR_BAD_INPUT, "null uv_out");
    double* uv = c.ws.get<double>("lscm.uv", 2 * NV);
    if (NV > 0) d2h(c, uv_out, uv, sizeof(double) * 2 * NV, c.stream);
    RUV_CUDA(cudaStreamSynchronize(c.stream));
    return RUV_OK;
  });
}

ruv_status ruv_lscm_solve_batch(ruv_ctx* ctx, const ruv_lscm_batch* in, const ruv_unfold_opts* opts, double* uv_out,
                                ruv_chart_stat* stats) {
  ruv_status s = upload_batch(ctx, in, true);
  if (s != RUV_OK) return s;
  ruv_status solved = RUV_OK;
  if (in->vert_off[in->n_charts] > 0 && !uv_out) solved = fail(ctx, RUV_ERR_BAD_INPUT, "null uv_out");
  else solved = ruv_lscm_solve_resident(ctx, opts, stats);
  order_pending_copies(ctx->c);  // (a path that returned before the assembly's waits)
  if (solved != RUV_OK && solved != RUV_ERR_NOT_CONVERGED && solved != RUV_ERR_BREAKDOWN) return solved;
  std::string msg = ctx->c.last_error;
  if (!ctx->c.have_uv) return solved;
  s = ruv_lscm_download_uv(ctx, uv_out);
  if (s != RUV_OK) return s;
  ctx->c.last_error = msg;
  return solved;
}

ruv_status ruv_lscm_solve_batch_keep_metric(ruv_ctx* ctx, const ruv_lscm_batch* in, const ruv_unfold_opts* opts,
                                            const double* target, double* uv_out, ruv_chart_stat* stats) {
  ruv_status up = ruv_lscm_upload(ctx, in);
  if (up != RUV_OK) return up;
  const int64_t NC = in->n_charts, NV = in->vert_off[NC];
  if ((NV > 0 && !uv_out) || (NC > 0 && !target)) return fail(ctx, RUV_ERR_BAD_INPUT, "null buffer");
  ruv_status solved = guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    ruv_unfold_opts o;
    ruv_unfold_opts_default(&o);
    if (opts) o = *opts;
    if (!known_precond(o.precond)) return fail(ctx, RUV_ERR_BAD_INPUT, "unknown preconditioner");
    DevBatch& bt = c.resident;
    c.have_uv = false;
    c.have_last = false;  // (no backward pass for KeepMetric)
    if (NC == 0) {
      c.have_uv = true;
      return RUV_OK;
    }
    DevSystem& sys = c.last_sys;
    assemble_lscm(c, bt, sys, o.angle_mix);
    const int64_t NR = sys.n_rows;
    double* u = c.ws.get<double>("km.u", 2 * std::max<int64_t>(NR, 1));
    std::vector<double> flip(NC);
    for (int64_t k = 0; k < NC; ++k)  // (host: the reference's summation order decides the sign)
      flip[k] = uv_signed_area(in->p2 + 2 * in->vert_off[k], in->tris + 3 * in->tri_off[k],
                               in->tri_off[k + 1] - in->tri_off[k]) >= 0.0 ? 1.0 : -1.0;
    keep_metric_rhs(c, bt, sys, upload(c, "km.flip", flip.data(), NC), u);
    double* yb = c.ws.get<double>("km.yb", 2 * std::max<int64_t>(NR, 1));
    double* yu = c.ws.get<double>("km.yu", 2 * std::max<int64_t>(NR, 1));
    SolveOpts so;
    so.precond = o.precond;
    so.precision = o.precision;
    so.tol = o.tol;
    so.max_iter = o.max_cg_iter > 0 ? o.max_cg_iter : 16384;
    auto r1 = pcg_solve(c, sys, yb, so);
    double* b_saved = sys.b;
    sys.b = u;
    auto r2 = pcg_solve(c, sys, yu, so);
    sys.b = b_saved;
    const double* d_target = upload(c, "km.target", target, NC);
    double* uv = c.ws.get<double>("lscm.uv", 2 * std::max<int64_t>(NV, 1));
    std::vector<int32_t> iters;
    std::vector<double> err_accum;
    driver_keep_metric(c, bt, sys, yb, yu, d_target, o.max_iter, uv, iters, err_accum);
    c.have_uv = true;
    int w = RUV_OK;
    for (int64_t k = 0; k < NC; ++k) {
      const int st = worst(r1[k].status, r2[k].status);
      w = worst(w, st);
      if (stats) {
        stats[k].status = st;
        stats[k].driver_iters = iters[k];
        stats[k].cg_iters = r1[k].iters + r2[k].iters;
        stats[k].n_free = (int32_t)(sys.h_chart_row[k + 1] - sys.h_chart_row[k]);
        stats[k].rel_res = std::max(r1[k].rel_res, r2[k].rel_res);
        stats[k].err_accum = err_accum[k];
      }
    }
    if (w != RUV_OK) return fail(ctx, (ruv_status)w, "at least one chart did not converge");
    return RUV_OK;
  });
  if (solved != RUV_OK && solved != RUV_ERR_NOT_CONVERGED && solved != RUV_ERR_BREAKDOWN) return solved;
  std::string msg = ctx->c.last_error;
  if (!ctx->c.have_uv) return solved;
  ruv_status s = ruv_lscm_download_uv(ctx, uv_out);
  if (s != RUV_OK) return s;
  ctx->c.last_error = msg;
  return solved;
}

ruv_status ruv_lscm_forward(ruv_ctx* ctx, const ruv_lscm_batch* in, const ruv_unfold_opts* opts, double* uv_out,
                            ruv_chart_stat* stats) {
  return ruv_lscm_solve_batch(ctx, in, opts, uv_out, stats);
}

ruv_status ruv_lscm_backward(ruv_ctx* ctx, const ruv_unfold_opts* opts, const double* dl_duv, double* dl_dp3,
                             ruv_chart_stat* stats) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    if (!c.have_uv || !c.have_batch) return fail(ctx, RUV_ERR_BAD_INPUT, "no forward solve on this context");
    DevBatch& bt = c.resident;
    const int64_t NV = bt.n_verts, NC = bt.n_charts;
    if (NV > 0 && (!dl_duv || !dl_dp3)) return fail(ctx, RUV_ERR_BAD_INPUT, "null gradient buffer");
    ruv_unfold_opts o;
    ruv_unfold_opts_default(&o);
    if (opts) o = *opts;
    if (!known_precond(o.precond)) return fail(ctx, RUV_ERR_BAD_INPUT, "unknown preconditioner");
    double* x = c.ws.get<double>("lscm.x", 1);  // the forward solution (rows), kept by the solve
    // the assembly is recomputed (same inputs, bit-identical operator)
    DevSystem sys;
    assemble_lscm(c, bt, sys, o.angle_mix);
    double* gv = upload(c, "adj.gv", dl_duv, 2 * NV);
    double* dp = c.ws.get<double>("adj.dp3", std::max<int64_t>(3 * NV, 1));
    SolveOpts so;
    so.precond = o.precond;
    so.precision = o.precision;
    so.tol = o.tol;
    so.max_iter = o.max_cg_iter > 0 ? o.max_cg_iter : 16384;
    std::vector<ChartResult> res;
    lscm_backward(c, bt, sys, x, gv, so, dp, res);
    if (NV > 0) RUV_CUDA(cudaMemcpyAsync(dl_dp3, dp, sizeof(double) * 3 * NV, cudaMemcpyDeviceToHost, c.stream));
    RUV_CUDA(cudaStreamSynchronize(c.stream));
    int w = RUV_OK;
    for (int64_t k = 0; k < NC; ++k) {
      w = worst(w, res[k].status);
      if (stats) {
        stats[k].status = res[k].status;
        stats[k].driver_iters = 0;
        stats[k].cg_iters = res[k].iters;
        stats[k].n_free = (int32_t)(sys.h_chart_row[k + 1] - sys.h_chart_row[k]);
        stats[k].rel_res = res[k].rel_res;
        stats[k].err_accum = 0.0;
      }
    }
    if (w != RUV_OK) return fail(ctx, (ruv_status)w, "adjoint solve: at least one chart did not converge");
    return RUV_OK;
  });
}

ruv_status ruv_distortion_loss(ruv_ctx* ctx, const double* uv, double* loss_out, double* dl_duv, double* dl_dp3) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    if (!c.have_batch) return fail(ctx, RUV_ERR_BAD_INPUT, "no batch uploaded on this context");
    const DevBatch& bt = c.resident;
    const int64_t NV = bt.n_verts, NC = bt.n_charts;
    if (NV > 0 && !uv) return fail(ctx, RUV_ERR_BAD_INPUT, "null uv");
    if (NC > 0 && !loss_out) return fail(ctx, RUV_ERR_BAD_INPUT, "null loss_out");
    const double* duv = upload(c, "dist.uv", uv, 2 * NV);
    double* g_uv = nullptr;
    double* g_p = nullptr;
    if (dl_duv) {
      g_uv = c.ws.get<double>("dist.guv", std::max<int64_t>(2 * NV, 1));
      RUV_CUDA(cudaMemsetAsync(g_uv, 0, sizeof(double) * std::max<int64_t>(2 * NV, 1), c.stream));
    }
    if (dl_dp3) {
      g_p = c.ws.get<double>("dist.gp", std::max<int64_t>(3 * NV, 1));
      RUV_CUDA(cudaMemsetAsync(g_p, 0, sizeof(double) * std::max<int64_t>(3 * NV, 1), c.stream));
    }
    std::vector<double> loss;
    distortion_loss(c, bt, duv, g_uv, g_p, loss);
    std::copy(loss.begin(), loss.end(), loss_out);
    if (g_uv && NV > 0) RUV_CUDA(cudaMemcpyAsync(dl_duv, g_uv, sizeof(double) * 2 * NV, cudaMemcpyDeviceToHost, c.stream));
    if (g_p && NV > 0) RUV_CUDA(cudaMemcpyAsync(dl_dp3, g_p, sizeof(double) * 3 * NV, cudaMemcpyDeviceToHost, c.stream));
    RUV_CUDA(cudaStreamSynchronize(c.stream));
    return RUV_OK;
  });
}

ruv_status ruv_chart_distortion(ruv_ctx* ctx, const double* uv, double* metrics_out) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    if (!c.have_batch) return fail(ctx, RUV_ERR_BAD_INPUT, "no batch uploaded on this context");
    const DevBatch& bt = c.resident;
    const int64_t NV = bt.n_verts, NC = bt.n_charts;
    if ((NV > 0 && !uv) || (NC > 0 && !metrics_out)) return fail(ctx, RUV_ERR_BAD_INPUT, "null buffer");
    const double* duv = upload(c, "met.uv", uv, 2 * NV);
    std::vector<double> out;
    chart_metrics(c, bt, duv, out);
    std::copy(out.begin(), out.end(), metrics_out);
    return RUV_OK;
  });
}

ruv_status ruv_rectangularize(ruv_ctx* ctx, const double* uv, const uint8_t* border, double* rectified_out,
                              double* ext_out) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    if (!c.have_batch) return fail(ctx, RUV_ERR_BAD_INPUT, "no batch uploaded on this context");
    const DevBatch& bt = c.resident;
    const int64_t NV = bt.n_verts, NC = bt.n_charts;
    if ((NV > 0 && (!uv || !border || !rectified_out)) || (NC > 0 && !ext_out))
      return fail(ctx, RUV_ERR_BAD_INPUT, "null buffer");
    const double* duv = upload(c, "rect.uv", uv, 2 * NV);
    const uint8_t* db = upload(c, "rect.border", border, NV);
    double* q = c.ws.get<double>("rect.q", std::max<int64_t>(2 * NV, 1));
    double* e = c.ws.get<double>("rect.ext", std::max<int64_t>(2 * NC, 1));
    rectangularize(c, bt, duv, db, q, e);
    if (NV > 0) RUV_CUDA(cudaMemcpyAsync(rectified_out, q, sizeof(double) * 2 * NV, cudaMemcpyDeviceToHost, c.stream));
    if (NC > 0) RUV_CUDA(cudaMemcpyAsync(ext_out, e, sizeof(double) * 2 * NC, cudaMemcpyDeviceToHost, c.stream));
    RUV_CUDA(cudaStreamSynchronize(c.stream));
    return RUV_OK;
  });
}

ruv_status ruv_selftest_fp64(ruv_ctx* ctx, int mode, uint64_t seed, int64_t n, int64_t* mismatches, double* first4) {
  if (!ctx || !mismatches || !first4 || mode < 0 || mode > 5 || n < 0) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    *mismatches = fp64_selftest(ctx->c, mode, seed, n, first4);
    return RUV_OK;
  });
}

ruv_status ruv_host_alloc(ruv_ctx* ctx, int64_t bytes, void** out) {
  if (!ctx || !out || bytes < 0) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    *out = nullptr;
    if (cudaHostAlloc(out, (size_t)(bytes > 0 ? bytes : 1), cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      *out = nullptr;
      return fail(ctx, RUV_ERR_OOM, "page-locked host allocation failed");
    }
    return RUV_OK;
  });
}

void ruv_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int64_t ruv_kernel_launches(const ruv_ctx* ctx) { return ctx ? ctx->c.launches : 0; }

int32_t ruv_last_timings(const ruv_ctx* ctx, double* ms, int32_t n) {
  if (!ctx || !ms) return 0;
  int32_t k = n < 4 ? n : 4;
  for (int32_t i = 0; i < k; ++i) ms[i] = ctx->c.timings[i];
  return k;
}

ruv_status ruv_bench_spmv(ruv_ctx* ctx, ruv_precision precision, int32_t reps, int32_t n_buffers, double* ms_per_launch,
                          double* bytes_per_launch, double* stream_bytes_per_launch) {
  if (!ctx || reps <= 0 || n_buffers <= 0) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    if (!c.have_last) return fail(ctx, RUV_ERR_BAD_INPUT, "no assembled batch on this context");
    double bytes = 0.0, stream = 0.0;
    double ms = bench_spmv(c, c.last_sys, precision == RUV_PREC_MIXED, reps, n_buffers, &bytes, &stream);
    if (ms_per_launch) *ms_per_launch = ms;
    if (bytes_per_launch) *bytes_per_launch = bytes;
    if (stream_bytes_per_launch) *stream_bytes_per_launch = stream;
    return RUV_OK;
  });
}

ruv_status ruv_spmv_form(ruv_ctx* ctx, int32_t* bulk_copy) {
  if (!ctx || !bulk_copy) return RUV_ERR_BAD_INPUT;
  const char* te = std::getenv("RUV_SPMV_TMA");
  *bulk_copy = te ? (te[0] == '1' ? 1 : 0) : ctx->c.spmv_tma;
  return RUV_OK;
}

ruv_status ruv_autotune(ruv_ctx* ctx, ruv_precision precision, int32_t reps, int32_t* lanes_per_row,
                        int32_t* rows_in_flight, int32_t* tile_rows, double* ms_per_launch) {
  if (!ctx || reps <= 0) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    if (!c.have_last) return fail(ctx, RUV_ERR_BAD_INPUT, "no assembled batch on this context");
    TuneResult t = autotune_spmv(c, c.last_sys, precision == RUV_PREC_MIXED, reps);
    if (lanes_per_row) *lanes_per_row = t.lpr;
    if (rows_in_flight) *rows_in_flight = t.unroll;
    if (tile_rows) *tile_rows = t.tile_rows;
    if (ms_per_launch) *ms_per_launch = t.ms;
    return RUV_OK;
  });
}

ruv_status ruv_export_chart_system(ruv_ctx* ctx, int64_t chart, int64_t* nf_out, int64_t* nnz_out, int32_t* row_ptr,
                                   int32_t* cols, double* vals, double* rhs) {
  if (!ctx) return RUV_ERR_BAD_INPUT;
  return guarded(ctx, [&]() -> ruv_status {
    Ctx& c = ctx->c;
    if (!c.have_last) return fail(ctx, RUV_ERR_BAD_INPUT, "no assembled batch on this context");
    DevSystem& sys = c.last_sys;
    if (chart < 0 || chart >= sys.n_charts) return fail(ctx, RUV_ERR_BAD_INPUT, "chart out of range");
    const int64_t r0 = sys.h_chart_row[chart], r1 = sys.h_chart_row[chart + 1], nf = r1 - r0;
    std::vector<int32_t> rp(nf + 1);
    RUV_CUDA(cudaMemcpyAsync(rp.data(), sys.row_ptr + r0, sizeof(int32_t) * (nf + 1), cudaMemcpyDeviceToHost, c.stream));
    RUV_CUDA(cudaStreamSynchronize(c.stream));
    const int64_t e0 = rp[0], ne = rp[nf] - rp[0];
    if (nf_out) *nf_out = nf;
    if (nnz_out) *nnz_out = 2 * ne;
    if (!row_ptr && !cols && !vals && !rhs) return RUV_OK;
    std::vector<int32_t> sc(ne);
    std::vector<double> sv(ne), sb(2 * nf);
    if (ne > 0) {
      RUV_CUDA(cudaMemcpyAsync(sc.data(), sys.cols + e0, sizeof(int32_t) * ne, cudaMemcpyDeviceToHost, c.stream));
      RUV_CUDA(cudaMemcpyAsync(sv.data(), sys.vals + e0, sizeof(double) * ne, cudaMemcpyDeviceToHost, c.stream));
    }
    if (nf > 0)
      RUV_CUDA(cudaMemcpyAsync(sb.data(), sys.b + 2 * r0, sizeof(double) * 2 * nf, cudaMemcpyDeviceToHost, c.stream));
    RUV_CUDA(cudaStreamSynchronize(c.stream));
    // A = L (x) I2: scalar row r -> interleaved rows 2r (u) and 2r + 1 (v)
    int64_t at = 0;
    if (row_ptr) row_ptr[0] = 0;
    for (int64_t r = 0; r < nf; ++r)
      for (int comp = 0; comp < 2; ++comp) {
        for (int64_t k = rp[r] - e0; k < rp[r + 1] - e0; ++k) {
          if (cols) cols[at] = (int32_t)(2 * (sc[k] - r0) + comp);
          if (vals) vals[at] = sv[k];
          ++at;
        }
        if (row_ptr) row_ptr[2 * r + comp + 1] = (int32_t)at;
      }
    if (rhs)
      for (int64_t i = 0; i < 2 * nf; ++i) rhs[i] = sb[i];
    return RUV_OK;
  });
}

// ------------------------------------------------------------------ host chart stages
ruv_status ruv_prepare_mesh(const double* pos, int64_t n_verts, const int32_t* faces, int64_t n_faces, double weld_tol,
                            double angle_min_deg, int32_t threads, ruv_prepared** out) {
  if (!out || n_verts < 0 || n_faces < 0 || (n_verts > 0 && !pos) || (n_faces > 0 && !faces)) return RUV_ERR_BAD_INPUT;
  if (n_verts >= (int64_t)INT32_MAX) return RUV_ERR_BAD_INPUT;
  *out = nullptr;
  try {
    std::unique_ptr<ruv_prepared> p(new ruv_prepared());
    std::string err;
    ruv_status s = prepare_mesh(pos, n_verts, faces, n_faces, weld_tol, angle_min_deg, threads, p->p, err);
    if (s != RUV_OK) return s;
    *out = p.release();
    return RUV_OK;
  } catch (const std::bad_alloc&) {
    return RUV_ERR_OOM;
  } catch (...) {
    return RUV_ERR_INTERNAL;
  }
}

ruv_status ruv_prepare_mesh_gpu(ruv_ctx* ctx, const double* pos, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                                double weld_tol, double angle_min_deg, int32_t threads, ruv_prepared** out) {
  if (!ctx || !out || n_verts < 0 || n_faces < 0 || (n_verts > 0 && !pos) || (n_faces > 0 && !faces))
    return RUV_ERR_BAD_INPUT;
  if (n_verts >= (int64_t)INT32_MAX || n_faces >= (int64_t)INT32_MAX / 3) return RUV_ERR_BAD_INPUT;
  *out = nullptr;
  return guarded(ctx, [&]() -> ruv_status {
    std::unique_ptr<ruv_prepared> p(new ruv_prepared());
    std::string err;
    ruv_status s = prepare_mesh_gpu(ctx->c, pos, n_verts, faces, n_faces, weld_tol, angle_min_deg, threads, p->p, err);
    if (s != RUV_OK) return fail(ctx, s, err.empty() ? "mesh preparation failed" : err);
    *out = p.release();
    return RUV_OK;
  });
}

void ruv_cut_opts_default(ruv_cut_opts* o) {
  if (!o) return;
  o->seam_enable = 0;
  o->seam_min_faces = 8;
  o->seam_branch_count = 1;
  o->recut_enable = 0;
  o->recut_max_rounds = 6;
  o->recut_max_splits = 48;
  o->recut_fold_fraction = 0.02;
  o->recut_max_charts = 64;
}

ruv_status ruv_prepare_mesh_cut(ruv_ctx* ctx, const double* pos, int64_t n_verts, const int32_t* faces, int64_t n_faces,
                                double weld_tol, double angle_min_deg, const ruv_cut_opts* cut,
                                const ruv_unfold_opts* unfold, int32_t threads, ruv_prepared** out, int64_t* added_out) {
  if (!out || n_verts < 0 || n_faces < 0 || (n_verts > 0 && !pos) || (n_faces > 0 && !faces))
    return RUV_ERR_BAD_INPUT;
  if (n_verts >= (int64_t)INT32_MAX) return RUV_ERR_BAD_INPUT;
  *out = nullptr;
  ruv_cut_opts co;
  ruv_cut_opts_default(&co);
  if (cut) co = *cut;
  if (!ctx && co.recut_enable) return RUV_ERR_BAD_INPUT;  // (the seam cut alone needs no device)
  ruv_unfold_opts uo;
  ruv_unfold_opts_default(&uo);
  if (unfold) uo = *unfold;
  CutOpts o;
  o.seam_enable = co.seam_enable != 0;
  o.seam_min_faces = co.seam_min_faces;
  o.seam_branch = co.seam_branch_count;
  o.recut_enable = co.recut_enable != 0;
  o.max_rounds = co.recut_max_rounds;
  o.max_splits = co.recut_max_splits;
  o.fold_fraction = co.recut_fold_fraction;
  o.max_charts = co.recut_max_charts;
  std::unique_ptr<ruv_prepared> p(new ruv_prepared());
  std::string err;
  // each controller round: every chart unfolded in one batched solve on the context
  UnfoldFn solve = [&](const Prepared& P, std::vector<double>& uv, std::string& e) -> bool {
    ruv_lscm_batch b;
    b.n_charts = (int64_t)P.vert_off.size() - 1;
    b.vert_off = P.vert_off.data();
    b.tri_off = P.tri_off.data();
    b.p3 = P.p3.data();
    b.tris = P.tris.data();
    b.pinned = P.pinned.data();
    b.pin_uv = P.pin_uv.data();
    b.p2 = P.p2.data();
    uv.assign(2 * std::max<int64_t>(P.vert_off.back(), 1), 0.0);
    ruv_status st = ruv_lscm_solve_batch(ctx, &b, &uo, uv.data(), nullptr);
    if (st != RUV_OK && st != RUV_ERR_NOT_CONVERGED && st != RUV_ERR_BREAKDOWN) {
      e = ctx->c.last_error;
      return false;
    }
    return true;
  };
  int64_t added = 0;
  ruv_status s;
  try {
    s = prepare_mesh_cut(pos, n_verts, faces, n_faces, weld_tol, angle_min_deg, threads, o, &solve, p->p, &added, err);
  } catch (const std::bad_alloc&) {
    return RUV_ERR_OOM;
  } catch (...) {
    return RUV_ERR_INTERNAL;
  }
  if (s != RUV_OK) return ctx ? fail(ctx, s, err.empty() ? "mesh preparation failed" : err) : s;
  if (added_out) *added_out = added;
  *out = p.release();
  return RUV_OK;
}

ruv_status ruv_prepare_patches(int64_t n_patches, const int64_t* vert_off, const int64_t* tri_off, const double* p3,
                               const int32_t* tris, int32_t threads, ruv_prepared** out) {
  if (!out || n_patches < 0 || !vert_off || !tri_off) return RUV_ERR_BAD_INPUT;
  if ((vert_off[n_patches] > 0 && !p3) || (tri_off[n_patches] > 0 && !tris)) return RUV_ERR_BAD_INPUT;
  if (vert_off[n_patches] >= (int64_t)INT32_MAX) return RUV_ERR_BAD_INPUT;
  *out = nullptr;
  try {
    std::unique_ptr<ruv_prepared> p(new ruv_prepared());
    std::string err;
    ruv_status s = prepare_patches(n_patches, vert_off, tri_off, p3, tris, threads, p->p, err);
    if (s != RUV_OK) return s;
    *out = p.release();
    return RUV_OK;
  } catch (const std::bad_alloc&) {
    return RUV_ERR_OOM;
  } catch (...) {
    return RUV_ERR_INTERNAL;
  }
}

ruv_status ruv_prepare_patches_gpu(ruv_ctx* ctx, int64_t n_patches, const int64_t* vert_off, const int64_t* tri_off,
                                   const double* p3, const int32_t* tris, int32_t threads, ruv_prepared** out) {
  if (!ctx || !out || n_patches < 0 || !vert_off || !tri_off) return RUV_ERR_BAD_INPUT;
  if ((vert_off[n_patches] > 0 && !p3) || (tri_off[n_patches] > 0 && !tris)) return RUV_ERR_BAD_INPUT;
  if (vert_off[n_patches] >= (int64_t)INT32_MAX || tri_off[n_patches] >= (int64_t)INT32_MAX / 3) return RUV_ERR_BAD_INPUT;
  *out = nullptr;
  return guarded(ctx, [&]() -> ruv_status {
    std::unique_ptr<ruv_prepared> p(new ruv_prepared());
    std::string err;
    ruv_status s = prepare_patches_gpu(ctx->c, n_patches, vert_off, tri_off, p3, tris, threads, p->p, err);
    if (s != RUV_OK) return fail(ctx, s, err.empty() ? "patch preparation failed" : err);
    *out = p.release();
    return RUV_OK;
  });
}

void ruv_prepared_free(ruv_prepared* p) { delete p; }

ruv_status ruv_prepared_batch(const ruv_prepared* p, ruv_lscm_batch* v) {
  if (!p || !v) return RUV_ERR_BAD_INPUT;
  const Prepared& P = p->p;
  v->n_charts = (int64_t)P.vert_off.size() - 1;
  v->vert_off = P.vert_off.data();
  v->tri_off = P.tri_off.data();
  v->p3 = P.p3.data();
  v->tris = P.tris.data();
  v->pinned = P.pinned.data();
  v->pin_uv = P.pin_uv.data();
  v->p2 = P.p2.data();
  return RUV_OK;
}

int64_t ruv_prepared_get_i64(const ruv_prepared* p, const char* what, int64_t* out) {
  if (!p || !what) return -1;
  const Prepared& P = p->p;
  std::string w(what);
  auto emit = [&](const auto& vec) -> int64_t {
    if (out)
      for (size_t i = 0; i < vec.size(); ++i) out[i] = (int64_t)vec[i];
    return (int64_t)vec.size();
  };
  if (w == "chart.vert_off") return emit(P.vert_off);
  if (w == "chart.tri_off") return emit(P.tri_off);
  if (w == "chart.vertex_ids") return emit(P.vertex_ids);
  if (w == "chart.face_ids") return emit(P.face_ids);
  if (w == "chart.tris") return emit(P.tris);
  if (w == "chart.border_off") return emit(P.border_off);
  if (w == "chart.border") return emit(P.border);
  if (w == "chart.loop_off") return emit(P.loop_off);
  if (w == "chart.loop_seg") return emit(P.loop_seg);
  if (w == "chart.loop_ids") return emit(P.loop_ids);
  if (w == "chart.pinned") return emit(P.pinned);
  if (w == "mesh.faces") return emit(P.mesh_faces);
  if (w == "mesh.n_cut_slots") {
    if (out) out[0] = P.n_cut_slots;
    return 1;
  }
  return -1;
}

int64_t ruv_prepared_get_f64(const ruv_prepared* p, const char* what, double* out) {
  if (!p || !what) return -1;
  const Prepared& P = p->p;
  std::string w(what);
  auto emit = [&](const std::vector<double>& vec) -> int64_t {
    if (out && !vec.empty()) std::memcpy(out, vec.data(), sizeof(double) * vec.size());
    return (int64_t)vec.size();
  };
  if (w == "chart.area3d") return emit(P.area3d);
  if (w == "mesh.pos") return emit(P.mesh_pos);
  if (w == "chart.pin_uv") return emit(P.pin_uv);
  if (w == "chart.p2") return emit(P.p2);
  if (w == "chart.p3") return emit(P.p3);
  return -1;
}

}  // extern "C"
