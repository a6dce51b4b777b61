// ORACLE HARNESS — test infrastructure only (a measuring stick; never the thing measured or
// shipped).  The reference's own single-system GPU solve, for the "plain single-chart FP64
// GPU PCG" baseline: the reference's CG kernels (gpu/src/kernels.cu:7-102, compiled from the
// reference's source to compute_80 PTX exactly as gpu/build.rs:41-49 does, JIT-loaded by the
// driver) driven by a C++ restatement of GpuSolver::cg_solve_precond (gpu/src/solver.rs:
// 284-565) for Precond::None and Precond::Jacobi (precond.rs:593-608): per-call device
// allocations and uploads (DeviceMem, solver.rs:671-729), 256-thread blocks over n rows on
// the legacy default stream, and every dot product as block partials summed on the host after
// a context synchronisation (dot_s, solver.rs:569-615).
//
// Built by oracle.build_ref_cg() with g++ against the CUDA driver API (cuda.h, -lcuda).
#include <cuda.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace {

constexpr unsigned kBlock = 256;  // gpu/src/solver.rs BLOCK

struct Ref {
  bool ready = false;
  CUcontext ctx = nullptr;
  CUmodule mod = nullptr;
  CUfunction fill0 = nullptr, spmv = nullptr, dot = nullptr, axpy = nullptr, xpay = nullptr, copy = nullptr,
             mul = nullptr;
  std::string err;
};
Ref g;

bool ok(CUresult r, const char* what) {
  if (r == CUDA_SUCCESS) return true;
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  g.err = std::string(what) + ": " + (s ? s : "?");
  return false;
}

// DeviceMem: every allocation of one solve, freed when the solve returns.
struct DeviceMem {
  std::vector<CUdeviceptr> bufs;
  ~DeviceMem() {
    for (CUdeviceptr p : bufs) cuMemFree(p);
  }
  CUdeviceptr alloc(size_t bytes) {
    CUdeviceptr p = 0;
    if (!ok(cuMemAlloc(&p, bytes > 0 ? bytes : 8), "cuMemAlloc")) return 0;
    bufs.push_back(p);
    return p;
  }
  CUdeviceptr upload(const void* host, size_t bytes) {
    CUdeviceptr p = alloc(bytes);
    if (p && bytes > 0 && !ok(cuMemcpyHtoD(p, host, bytes), "cuMemcpyHtoD")) return 0;
    return p;
  }
};

bool launch(CUfunction f, unsigned grid, void** params) {
  return ok(cuLaunchKernel(f, grid, 1, 1, kBlock, 1, 1, 0, nullptr, params, nullptr), "cuLaunchKernel");
}

// dot(a, b): block partials, a context synchronisation, the partials summed on the host.
bool dot_s(CUdeviceptr a, CUdeviceptr b, int n, CUdeviceptr& scratch, size_t& scratch_blocks, DeviceMem& mem,
           double& out) {
  const unsigned blocks = (unsigned)((n + kBlock - 1) / kBlock);
  if (scratch_blocks < blocks) {
    scratch = mem.alloc(sizeof(double) * blocks);
    if (!scratch) return false;
    scratch_blocks = blocks;
  }
  void* params[] = {&a, &b, &scratch, &n};
  if (!launch(g.dot, blocks, params) || !ok(cuCtxSynchronize(), "cuCtxSynchronize")) return false;
  std::vector<double> partials(blocks);
  if (!ok(cuMemcpyDtoH(partials.data(), scratch, sizeof(double) * blocks), "cuMemcpyDtoH")) return false;
  double s = 0.0;
  for (double v : partials) s += v;
  out = s;
  return true;
}

}  // namespace

extern "C" {

// GpuSolver::new: driver, primary context of device 0, the module from the PTX text.
int rcg_init(const char* ptx_path) {
  if (g.ready) return 0;
  std::FILE* f = std::fopen(ptx_path, "rb");
  if (!f) {
    g.err = std::string("cannot open ") + ptx_path;
    return 1;
  }
  std::string ptx;
  char buf[65536];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) ptx.append(buf, n);
  std::fclose(f);
  if (ptx.empty()) {
    g.err = "empty PTX";
    return 1;
  }
  CUdevice dev;
  if (!ok(cuInit(0), "cuInit") || !ok(cuDeviceGet(&dev, 0), "cuDeviceGet") ||
      !ok(cuDevicePrimaryCtxRetain(&g.ctx, dev), "cuDevicePrimaryCtxRetain") ||
      !ok(cuCtxSetCurrent(g.ctx), "cuCtxSetCurrent") || !ok(cuModuleLoadData(&g.mod, ptx.c_str()), "cuModuleLoadData"))
    return 1;
  struct {
    CUfunction* f;
    const char* name;
  } fs[] = {{&g.fill0, "fill0"}, {&g.spmv, "spmv"}, {&g.dot, "dot"},  {&g.axpy, "axpy"},
            {&g.xpay, "xpay"},   {&g.copy, "copy"}, {&g.mul, "mul"}};
  for (auto& e : fs)
    if (!ok(cuModuleGetFunction(e.f, g.mod, e.name), e.name)) return 1;
  g.ready = true;
  return 0;
}

const char* rcg_last_error(void) { return g.err.c_str(); }

// GpuSolver::cg_solve_precond for precond 0 (None) or 1 (Jacobi).  Returns 0 with x_out and
// iters_out written, 1 where the reference returns None.
int rcg_solve(int n, const int32_t* row_ptr, const int32_t* cols, const double* vals, const double* b, double* x_out,
              int64_t max_iter, double tol, int precond, int64_t* iters_out) {
  if (!g.ready || n <= 0 || row_ptr[0] != 0) return 1;
  if (!ok(cuCtxSetCurrent(g.ctx), "cuCtxSetCurrent")) return 1;
  const int64_t nnz = row_ptr[n];
  DeviceMem mem;
  CUdeviceptr d_vals = mem.upload(vals, sizeof(double) * nnz);
  CUdeviceptr d_cols = mem.upload(cols, sizeof(int32_t) * nnz);
  CUdeviceptr d_ptr = mem.upload(row_ptr, sizeof(int32_t) * (n + 1));
  CUdeviceptr d_b = mem.upload(b, sizeof(double) * n);
  CUdeviceptr d_x = mem.alloc(sizeof(double) * n);
  CUdeviceptr d_r = mem.upload(b, sizeof(double) * n);
  CUdeviceptr d_ap = mem.alloc(sizeof(double) * n);
  CUdeviceptr d_z = mem.alloc(sizeof(double) * n);
  CUdeviceptr d_p = mem.alloc(sizeof(double) * n);
  if (!d_vals || !d_cols || !d_ptr || !d_b || !d_x || !d_r || !d_ap || !d_z || !d_p) return 1;
  CUdeviceptr d_inv = 0;
  if (precond == 1) {  // upload_precond, Precond::Jacobi: 1 / a_ii of the first stored (i, i)
    std::vector<double> inv(n);
    for (int i = 0; i < n; ++i) {
      double d = 0.0;
      for (int32_t e = row_ptr[i]; e < row_ptr[i + 1]; ++e)
        if (cols[e] == i) {
          d = vals[e];
          break;
        }
      if (std::fabs(d) < 1e-300) return 1;
      inv[i] = 1.0 / d;
    }
    d_inv = mem.upload(inv.data(), sizeof(double) * n);
    if (!d_inv) return 1;
  }
  const unsigned grid = (unsigned)((n + kBlock - 1) / kBlock);
  CUdeviceptr scratch = 0;
  size_t scratch_blocks = 0;
  auto apply_precond = [&]() -> bool {
    if (precond == 1) {
      void* p[] = {&d_inv, &d_r, &d_z, &n};
      return launch(g.mul, grid, p);
    }
    void* p[] = {&d_z, &d_r, &n};
    return launch(g.copy, grid, p);
  };
  {
    void* p[] = {&d_x, &n};
    if (!launch(g.fill0, grid, p)) return 1;
  }
  double bb = 0.0, rsold = 0.0, rz = 0.0;
  if (!dot_s(d_b, d_b, n, scratch, scratch_blocks, mem, bb)) return 1;
  const double bnorm = std::sqrt(bb);
  const double tol_abs = bnorm <= 1e-300 ? tol : tol * bnorm;
  if (!dot_s(d_r, d_r, n, scratch, scratch_blocks, mem, rsold)) return 1;
  bool converged = std::sqrt(rsold) <= tol_abs;
  if (!apply_precond()) return 1;
  {
    void* p[] = {&d_p, &d_z, &n};
    if (!launch(g.copy, grid, p)) return 1;
  }
  if (precond == 0) rz = rsold;
  else if (!dot_s(d_r, d_z, n, scratch, scratch_blocks, mem, rz)) return 1;
  int64_t iters = 0;
  while (!converged && iters < max_iter) {
    ++iters;
    {
      void* p[] = {&d_vals, &d_cols, &d_ptr, &d_p, &d_ap, &n};
      if (!launch(g.spmv, grid, p)) return 1;
    }
    double pap = 0.0;
    if (!dot_s(d_p, d_ap, n, scratch, scratch_blocks, mem, pap)) return 1;
    if (std::fabs(pap) <= 1e-300 || !std::isfinite(pap)) return 1;  // breakdown
    double alpha = rz / pap, nalpha = -alpha;
    {
      void* p1[] = {&alpha, &d_p, &d_x, &n};
      void* p2[] = {&nalpha, &d_ap, &d_r, &n};
      if (!launch(g.axpy, grid, p1) || !launch(g.axpy, grid, p2)) return 1;
    }
    if (!dot_s(d_r, d_r, n, scratch, scratch_blocks, mem, rsold)) return 1;
    if (std::sqrt(rsold) <= tol_abs) {
      converged = true;
      break;
    }
    if (!apply_precond()) return 1;
    double rznew = 0.0;
    if (!dot_s(d_r, d_z, n, scratch, scratch_blocks, mem, rznew)) return 1;
    double beta = rznew / rz;
    {
      void* p[] = {&beta, &d_z, &d_p, &n};
      if (!launch(g.xpay, grid, p)) return 1;
    }
    rz = rznew;
  }
  if (!converged) return 1;
  if (!ok(cuMemcpyDtoH(x_out, d_x, sizeof(double) * n), "cuMemcpyDtoH")) return 1;
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(x_out[i])) return 1;
  if (iters_out) *iters_out = iters;
  return 0;
}

}  // extern "C"
