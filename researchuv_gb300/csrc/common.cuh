// Device-side building blocks shared by the LSCM kernels: status handling, the device
// workspace, warp/block reductions with a fixed (deterministic) combine order, and a
// device-wide exclusive scan.  Everything runs on the context's own stream.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "ruv_internal.h"

namespace ruv {

constexpr int kWarp = 32;
constexpr double kEpsDegenerate = 1.1754943508222875e-38;  // unwrap/src/lscm.rs:36

// ------------------------------------------------------------------ errors
struct Error {
  ruv_status status;
  std::string msg;
};

#define RUV_CUDA(call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      throw ::ruv::Error{e_ == cudaErrorMemoryAllocation ? RUV_ERR_OOM : RUV_ERR_LAUNCH,     \
                         std::string(#call) + ": " + cudaGetErrorString(e_)};               \
  } while (0)

#define RUV_LAUNCH_CHECK() RUV_CUDA(cudaGetLastError())

inline unsigned div_up(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// Kernel-launch accounting: the calling context points this at its counter for the duration
// of an API call; every launch site adds the kernels it enqueues (graph replays add their
// node count).
inline thread_local int64_t* g_launch_counter = nullptr;
inline void count_launches(int64_t n) {
  if (g_launch_counter) *g_launch_counter += n;
}

// ------------------------------------------------------------------ workspace
// Named device buffers owned by a context, grown on demand and reused across calls, so a
// steady stream of same-shaped solves allocates nothing after the first.
class Workspace {
 public:
  ~Workspace() { release(); }
  void* get(const std::string& name, size_t bytes) {
    auto& b = bufs_[name];
    if (b.bytes < bytes) {
      if (b.ptr) cudaFree(b.ptr);
      b.ptr = nullptr;
      b.bytes = 0;
      size_t want = bytes + bytes / 8 + 256;
      if (fail_countdown > 0 && --fail_countdown == 0)  // host-side fault injection (ruv_debug_fail_alloc)
        throw Error{RUV_ERR_OOM, "injected allocation failure: cudaMalloc(" + std::to_string(want) + ") for " + name};
      cudaError_t e = cudaMalloc(&b.ptr, want);
      if (e != cudaSuccess) {
        b.ptr = nullptr;
        cudaGetLastError();
        throw Error{RUV_ERR_OOM, "cudaMalloc(" + std::to_string(want) + ") for " + name + ": " +
                                     cudaGetErrorString(e)};
      }
      b.bytes = want;
    }
    return b.ptr;
  }
  template <class T>
  T* get(const std::string& name, int64_t count) {
    return static_cast<T*>(get(name, (size_t)(count > 0 ? count : 1) * sizeof(T)));
  }
  void release() {
    for (auto& kv : bufs_)
      if (kv.second.ptr) cudaFree(kv.second.ptr);
    bufs_.clear();
  }
  size_t bytes() const {
    size_t s = 0;
    for (auto& kv : bufs_) s += kv.second.bytes;
    return s;
  }
  // > 0: the fail_countdown-th device allocation from now on fails as if the device were out
  // of memory (no cudaMalloc is made); 0: off.
  int64_t fail_countdown = 0;

 private:
  struct Buf {
    void* ptr = nullptr;
    size_t bytes = 0;
  };
  std::map<std::string, Buf> bufs_;
};

// Pinned host staging (for the small per-iteration control reads).
class PinnedHost {
 public:
  ~PinnedHost() {
    if (p_) cudaFreeHost(p_);
  }
  void* get(size_t bytes) {
    if (bytes > n_) {
      if (p_) cudaFreeHost(p_);
      p_ = nullptr;
      n_ = 0;
      RUV_CUDA(cudaMallocHost(&p_, bytes));
      n_ = bytes;
    }
    return p_;
  }

 private:
  void* p_ = nullptr;
  size_t n_ = 0;
};

// ------------------------------------------------------------------ reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sum of up to NV values per thread; every thread gets the totals.  `sh` must hold
// NV * 32 values.  Fixed combine order => bitwise reproducible for a fixed launch shape.
// (GB300 runs FP64 at a small fraction of the FP32 rate: the per-element loops of the
// FP32 solver reduce in float and widen once per tile.)
// Column-index streams of a CSR operator: 32-bit global row ids, or 16-bit offsets (2 bytes
// less per non-zero in every pass that streams the operator) -- from the chart's first row when
// every chart of the operator has at most 65536 rows (ColsNarrow), or, when a chart is larger,
// from each row's own index minus 32768 where every entry lies within 32767 rows of its row
// (ColsRowRel: the natural orders of grids and of locally numbered meshes).  A tile never spans
// two charts.  Kernels take the stream kind as a template parameter NW (0 wide, 1 chart-
// relative, 2 row-relative), form a row's base once (row_base) and add one offset per entry.
struct ColsWide {
  const int32_t* c;
  __device__ __forceinline__ int32_t row_base(int64_t) const { return 0; }
  __device__ __forceinline__ int32_t operator()(int64_t e, int32_t) const { return c[e]; }
};
struct ColsNarrow {
  const uint16_t* c;
  int32_t base;
  __device__ __forceinline__ int32_t row_base(int64_t) const { return base; }
  __device__ __forceinline__ int32_t operator()(int64_t e, int32_t rb) const { return rb + (int32_t)c[e]; }
};
constexpr int32_t kRowRelBias = 32768;
struct ColsRowRel {
  const uint16_t* c;
  __device__ __forceinline__ int32_t row_base(int64_t i) const { return (int32_t)i - kRowRelBias; }
  __device__ __forceinline__ int32_t operator()(int64_t e, int32_t rb) const { return rb + (int32_t)c[e]; }
};
// the base of a row in a 16-bit stream of kind NW (1: the chart's first row cb, 2: the row's own)
template <int NW>
__device__ __forceinline__ int32_t narrow_row_base(int32_t cb, int64_t i) {
  return NW == 2 ? (int32_t)i - kRowRelBias : NW == 1 ? cb : 0;
}

template <int NV, class A>
__device__ __forceinline__ void block_sum_t(A (&v)[NV], A* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k * 32 + wid] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    A t = lane < nw ? sh[k * 32 + lane] : A(0);
    v[k] = warp_sum(t);
  }
  __syncthreads();
}

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k * 32 + wid] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double t = lane < nw ? sh[k * 32 + lane] : 0.0;
    v[k] = warp_sum(t);
  }
  __syncthreads();
}

// ------------------------------------------------------------------ bulk-copy staging
// A window of a global array staged into shared memory by cp.async.bulk: the element range
// [e0, e1) widened to 16-byte boundaries (the copy's alignment rule; callers allocate the
// slack the widened end may read).
struct Win {
  const char* src;   // 16-byte aligned start in global memory
  int64_t first;     // element index of the first staged element
  uint32_t bytes;    // multiple of 16
};
__device__ __forceinline__ Win stage_window(const void* base, int64_t e0, int64_t e1, int es) {
  const uint64_t b0 = (uint64_t)e0 * es, b1 = (uint64_t)e1 * es;
  const uint64_t a0 = b0 & ~(uint64_t)15, a1 = (b1 + 15) & ~(uint64_t)15;
  return Win{static_cast<const char*>(base) + a0, (int64_t)(a0 / es), (uint32_t)(a1 - a0)};
}
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  if (bytes == 0) return;
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, int64_t limit) {
  const uint32_t a = smem_addr(bar);
  for (int64_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}


// A tile's rows [beg, end) of a CSR operator staged into `stage` (dynamic shared memory, 16
// bytes of mbarrier first): its row pointers (int32), values (es_v bytes each) and columns
// (es_c bytes each).  Every thread of the CTA calls it.  The wait is bounded: past `limit`
// tries the CTA sets *err, waits once more (bounded) for its own copies and gets false.
struct StagedRows {
  const int32_t* rp;
  const unsigned char* v;
  const unsigned char* c;
  int64_t fr, fv, fc;  // first staged element of each window
};
__device__ __forceinline__ bool stage_rows(unsigned char* stage, const int32_t* rp, int64_t beg, int64_t end,
                                           const void* vals, int es_v, const void* cols, int es_c, int64_t limit,
                                           int* err, StagedRows& out) {
  const int64_t e0 = rp[beg], e1 = rp[end];
  const Win wr = stage_window(rp, beg, end + 1, 4);
  const Win wv = stage_window(vals, e0, e1, es_v);
  const Win wc = stage_window(cols, e0, e1, es_c);
  uint64_t* bar = reinterpret_cast<uint64_t*>(stage);
  unsigned char* sr = stage + 16;
  unsigned char* sv = sr + wr.bytes;
  unsigned char* sc = sv + wv.bytes;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(wr.bytes + wv.bytes + wc.bytes)
                 : "memory");
    bulk_g2s(sr, wr.src, wr.bytes, bar);
    bulk_g2s(sv, wv.src, wv.bytes, bar);
    bulk_g2s(sc, wc.src, wc.bytes, bar);
  }
  __syncthreads();
  // one decision for the whole CTA: a wait that ran out in any thread sends every thread out
  if (__syncthreads_or(!mbar_wait(bar, 0, limit))) {
    if (threadIdx.x == 0) atomicOr(err, 1);
    mbar_wait(bar, 0, limit);
    return false;
  }
  out = StagedRows{reinterpret_cast<const int32_t*>(sr), sv, sc, wr.first, wv.first, wc.first};
  return true;
}
// bytes of stage a tile of `rows` rows and `nnz` entries needs
inline size_t stage_bytes(int64_t rows, int64_t nnz, int es_v, int es_c) {
  auto up16 = [](int64_t b) { return (size_t)((b + 15) & ~(int64_t)15); };
  return 16 + up16(4 * (rows + 1) + 16) + up16((int64_t)es_v * nnz + 16) + up16((int64_t)es_c * nnz + 16);
}

// ------------------------------------------------------------------ scan
// Exclusive scan of int32 counts into int64 offsets (out has n + 1 entries; out[n] = total).
void exclusive_scan(const int32_t* in, int64_t* out, int64_t n, Workspace& ws, cudaStream_t s,
                    const std::string& tag);
// Same for uint8 flags.
void exclusive_scan_u8(const uint8_t* in, int64_t* out, int64_t n, Workspace& ws, cudaStream_t s,
                       const std::string& tag);

}  // namespace ruv
