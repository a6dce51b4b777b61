// Batched preconditioned conjugate gradients over the packed block-diagonal operator
// (every chart of a mesh in one launch sequence, each chart with its own scalars,
// convergence test and status) — the sm_103a replacement for the reference's host-driven
// single-system loop (gpu/src/solver.rs:284-565) and its kernels (gpu/src/kernels.cu:7-75).
//
// Work decomposition: rows are cut into tiles that never span two charts; one CTA owns a
// tile.  A tile-level kernel writes one partial per reduction; a chart-level kernel (one
// CTA per chart) combines its chart's partials in tile order, so every reduction is
// deterministic and no host round trip happens inside an iteration.  Charts that are done
// exit at the top of every kernel.  One iteration is captured once as a CUDA graph and
// replayed; the host reads the count of active charts every `kCheckEvery` iterations.
//
// SpMV: CSR-vector with `LPR` lanes per row (sub-warp per row, chosen from the row-length
// profile), coalesced 32-bit value/column loads across the lanes, (u, v) pairs moved as one
// 64-bit (FP32) / 128-bit (FP64) vector, shuffle reduction inside the sub-warp, and the
// p.q product fused into the same pass.
//
// Precision: RUV_PREC_FP64 runs the reference's recurrence in FP64.  RUV_PREC_MIXED runs
// the SpMV, preconditioner and CG recurrence in FP32 and keeps an extended-precision
// solution accumulator and true residual r = b - A x, recomputed per chart whenever the
// FP32 residual has dropped by `kDelta` (1000x) since the last true residual ("reliable
// updates"); convergence is decided on the true residual only.  The extended precision is
// double-float (a value is an unevaluated FP32 pair hi + lo, ~48 significant bits, FP32
// instructions only: GB300's FP64 pipe is a small fraction of its FP32 rate).  The true
// residual is formed as r_i = b_i - rs_i x_i - sum_j a_ij (x_j - x_i), rs_i the FP64 row
// sum: for a Laplacian with eliminated pins rs_i is zero away from the pins, so the
// products are of the small differences x_j - x_i rather than of x itself and the
// cancellation in b - A x costs no more than the FP64 product does.
#include "system.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>

namespace ruv {
namespace {

constexpr int kTileThreads = 256;
constexpr int kChartThreads = 128;
constexpr int kCheckEvery = 16;
// refresh after a 1000x drop of the FP32 residual: the FP32 recurrence then drifts from the
// true residual by about 1e-7 x 1e3 relative, far inside CG's tolerance of an inexact residual,
// and the solve needs fewer double-float refreshes (4096 disks, AMG-SA: the same iterations,
// PCG 92.2 -> 91.1 ms against 100x)
constexpr double kDelta = 0.001;
inline double refresh_delta() {
  const char* e = std::getenv("RUV_REFRESH_DELTA");
  return e ? std::atof(e) : kDelta;
}

enum : int32_t { kActive = 0, kDone = 1 };

struct ChartState {
  double rz;       // r.z of the current iterate
  double alpha;
  double beta;
  double tol_abs;  // tol * ||b|| (tol when ||b|| <= 1e-300), solver.rs:465-466
  double r_ref;    // ||r|| at the last true-residual (mixed)
  double rr;       // last ||r||^2 (FP64 true residual for mixed)
  double bnorm;
  int32_t iters;
  int32_t status;
  int32_t state;
  int32_t refresh;  // mixed: a true-residual refresh is due
  int32_t refinements;
  float alpha32;  // alpha / beta rounded once per chart for the FP32 tile kernels
  float beta32;
  float rscale;   // 1 / ||b|| as FP32 (1 when b = 0): FP32 sums of squares of r * rscale stay in range
};

template <class S, int NR>
struct V {
  S c[NR];
};
template <class S, int NR>
__device__ __forceinline__ V<S, NR> ldv(const S* p, int64_t i) {
  V<S, NR> r;
  if constexpr (NR == 2 && sizeof(S) == 8) {
    double2 t = reinterpret_cast<const double2*>(p)[i];
    r.c[0] = t.x;
    r.c[1] = t.y;
  } else if constexpr (NR == 2 && sizeof(S) == 4) {
    float2 t = reinterpret_cast<const float2*>(p)[i];
    r.c[0] = t.x;
    r.c[1] = t.y;
  } else {
    r.c[0] = p[i];
  }
  return r;
}
template <class S, int NR>
__device__ __forceinline__ void stv(S* p, int64_t i, const V<S, NR>& v) {
  if constexpr (NR == 2 && sizeof(S) == 8) {
    reinterpret_cast<double2*>(p)[i] = make_double2(v.c[0], v.c[1]);
  } else if constexpr (NR == 2 && sizeof(S) == 4) {
    reinterpret_cast<float2*>(p)[i] = make_float2(v.c[0], v.c[1]);
  } else {
    p[i] = v.c[0];
  }
}

// Double-float arithmetic: TwoSum (Knuth) and the FMA TwoProduct carry the rounding error
// of an FP32 add / multiply exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// (Sh, Sl) += (ah + al) * (dh + dl), dropping the al * dl term (2^-48 relative).
__device__ __forceinline__ void df_fma(float ah, float al, float dh, float dl, float& Sh, float& Sl) {
  const float p = ah * dh;
  const float t = fmaf(ah, dl, fmaf(al, dh, fmaf(ah, dh, -p)));
  float sh, se;
  two_sum(Sh, p, sh, se);
  Sh = sh;
  Sl += se + t;
}
// A row's double-float value: NR hi parts then NR lo parts (one 16- / 8-byte access).
template <int NR>
struct DF {
  float h[NR], l[NR];
};
template <int NR>
__device__ __forceinline__ DF<NR> lddf(const float* p, int64_t i) {
  DF<NR> r;
  if constexpr (NR == 2) {
    const float4 t = reinterpret_cast<const float4*>(p)[i];
    r.h[0] = t.x;
    r.h[1] = t.y;
    r.l[0] = t.z;
    r.l[1] = t.w;
  } else {
    const float2 t = reinterpret_cast<const float2*>(p)[i];
    r.h[0] = t.x;
    r.l[0] = t.y;
  }
  return r;
}
template <int NR>
__device__ __forceinline__ void stdf(float* p, int64_t i, const DF<NR>& v) {
  if constexpr (NR == 2) reinterpret_cast<float4*>(p)[i] = make_float4(v.h[0], v.h[1], v.l[0], v.l[1]);
  else reinterpret_cast<float2*>(p)[i] = make_float2(v.h[0], v.l[0]);
}
__device__ __forceinline__ void split_f64(double v, float& h, float& l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

struct Tiles {
  const int64_t* tab;      // [begin, end) pairs
  const int32_t* chart;    // chart of each tile
  const int64_t* chart_tile;
  int64_t n;
  // bulk-copy SpMV (k_spmv_tma): the largest tile's rows and nonzeros (0: not set up), the
  // flag a timed-out staging wait sets, and the wait's iteration limit
  int64_t max_rows = 0, max_nnz = 0;
  int* err = nullptr;
  int64_t spin_limit = 0;
};

// ---------------------------------------------------------------- tile kernels
// Accumulator type of the per-element loops: float in the FP32 solver (GB300's FP64 pipe is
// a small fraction of its FP32 rate, so FP64 appears only per tile and per chart), double in
// the FP64 solver.

// Inverse diagonal (Jacobi) once per solve: dinv in the solver's precision; zero diagonals
// are counted so the chart can report a breakdown (precond.rs:595-611).
template <class S>
__global__ void __launch_bounds__(kTileThreads) k_dinv(int64_t n, const double* __restrict__ diag, S* __restrict__ dinv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dinv[i] = diag[i] == 0.0 ? S(0) : S(1) / (S)diag[i];
}

// Initial state: x = 0, r = b, z = M^-1 r, p = z.  Partials (FP64, once per solve): b.b, r.z,
// #zero diagonals.
// Mixed precision also: the double-float solution xdf = 0 and right-hand side bdf = b.
template <class S, int NR>
__global__ void __launch_bounds__(kTileThreads) k_init(Tiles T, const double* __restrict__ b, const double* __restrict__ diag,
                                                       const S* __restrict__ dinv, int use_jacobi, double* __restrict__ x64,
                                                       S* __restrict__ xs, S* __restrict__ r, S* __restrict__ z,
                                                       S* __restrict__ p, double* __restrict__ part,
                                                       float* __restrict__ xdf, float* __restrict__ bdf) {
  __shared__ double sh[3 * 32];
  int64_t t = blockIdx.x;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int64_t i = T.tab[2 * t] + threadIdx.x; i < T.tab[2 * t + 1]; i += blockDim.x) {
    V<double, NR> bv = ldv<double, NR>(b, i);
    V<S, NR> rv, zv, zero;
    if (diag[i] == 0.0) acc[2] += 1.0;
    const S di = use_jacobi ? dinv[i] : S(1);
#pragma unroll
    for (int k = 0; k < NR; ++k) {
      rv.c[k] = (S)bv.c[k];
      zv.c[k] = rv.c[k] * di;
      zero.c[k] = (S)0;
      acc[0] += bv.c[k] * bv.c[k];
      acc[1] += (double)rv.c[k] * (double)zv.c[k];
    }
    V<double, NR> z64;
#pragma unroll
    for (int k = 0; k < NR; ++k) z64.c[k] = 0.0;
    stv<double, NR>(x64, i, z64);
    if (xs) stv<S, NR>(xs, i, zero);
    if (xdf) {
      DF<NR> xz, bd;
#pragma unroll
      for (int k = 0; k < NR; ++k) {
        xz.h[k] = xz.l[k] = 0.0f;
        split_f64(bv.c[k], bd.h[k], bd.l[k]);
      }
      stdf<NR>(xdf, i, xz);
      stdf<NR>(bdf, i, bd);
    }
    stv<S, NR>(r, i, rv);
    stv<S, NR>(z, i, zv);
    stv<S, NR>(p, i, zv);
  }
  block_sum<3>(acc, sh);
  if (threadIdx.x == 0) {
    part[3 * t] = acc[0];
    part[3 * t + 1] = acc[1];
    part[3 * t + 2] = acc[2];
  }
}

// The row loop of one SpMV tile (see k_spmv_pq); `col` maps an entry to its column.
template <class S, int NR, int LPR, int U, class Col>
__device__ __forceinline__ void spmv_pq_tile(int64_t beg, int64_t end, const int32_t* __restrict__ row_ptr, Col col,
                                             const S* __restrict__ vals, const S* __restrict__ p, S* __restrict__ q,
                                             S (&acc)[1]) {
  constexpr int K = (8 + LPR - 1) / LPR;
  const int sub = threadIdx.x % LPR;
  const int rpp = kTileThreads / LPR;
  for (int64_t base = beg; base < end; base += (int64_t)rpp * U) {
    int lo[U], hi[U];
    int32_t rb[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
      rb[u] = col.row_base(i);
      const bool valid = i < end;
      lo[u] = valid ? row_ptr[i] : 0;
      hi[u] = valid ? row_ptr[i + 1] : 0;
    }
    S av[U][K];
    int cv[U][K];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int e = lo[u] + sub + k * LPR;
        const bool in = e < hi[u];
        av[u][k] = in ? vals[e] : S(0);
        cv[u][k] = in ? col(e, rb[u]) : -1;
      }
    V<S, NR> s[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int c = 0; c < NR; ++c) s[u].c[c] = S(0);
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (cv[u][k] >= 0) {
          const V<S, NR> pv = ldv<S, NR>(p, cv[u][k]);
#pragma unroll
          for (int c = 0; c < NR; ++c) s[u].c[c] += av[u][k] * pv.c[c];
        }
      for (int e = lo[u] + sub + K * LPR; e < hi[u]; e += LPR) {  // rows longer than K * LPR
        const S a = vals[e];
        const V<S, NR> pv = ldv<S, NR>(p, col(e, rb[u]));
#pragma unroll
        for (int c = 0; c < NR; ++c) s[u].c[c] += a * pv.c[c];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < NR; ++c) s[u].c[c] += __shfl_xor_sync(0xffffffffu, s[u].c[c], o, LPR);
    if (sub == 0) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
        if (i < end) {
          stv<S, NR>(q, i, s[u]);
          const V<S, NR> pi = ldv<S, NR>(p, i);
#pragma unroll
          for (int c = 0; c < NR; ++c) acc[0] += pi.c[c] * s[u].c[c];
        }
      }
    }
  }
}

// q = A p on the tile's rows fused with the partial p.q.  CSR-vector: LPR lanes per row,
// each lane covering K = ceil(8 / LPR) entries in one unrolled sweep (rows of a mesh
// Laplacian hold <= 8 entries almost always; longer rows finish in a remainder loop), U rows
// per sub-warp in flight so a warp keeps U * K independent value/column loads and U * K
// gathers outstanding.  Block-uniform trip counts keep every lane in the shuffles.  NW: the
// column stream's kind (ColsWide, ColsNarrow, ColsRowRel).
template <class S, int NR, int LPR, int U, int NW>
__global__ void __launch_bounds__(kTileThreads) k_spmv_pq_k(Tiles T, const ChartState* __restrict__ st,
                                                            const int32_t* __restrict__ row_ptr,
                                                            const int32_t* __restrict__ cols,
                                                            const uint16_t* __restrict__ c16,
                                                            const int32_t* __restrict__ cbase, const S* __restrict__ vals,
                                                            const S* __restrict__ p, S* __restrict__ q,
                                                            double* __restrict__ part) {
  __shared__ S sh[32];
  const int64_t t = blockIdx.x;
  const int32_t ch = T.chart[t];
  if (st[ch].state != kActive) return;
  S acc[1] = {S(0)};
  const int64_t beg = T.tab[2 * t], end = T.tab[2 * t + 1];
  if constexpr (NW == 1) spmv_pq_tile<S, NR, LPR, U>(beg, end, row_ptr, ColsNarrow{c16, cbase[ch]}, vals, p, q, acc);
  else if constexpr (NW == 2) spmv_pq_tile<S, NR, LPR, U>(beg, end, row_ptr, ColsRowRel{c16}, vals, p, q, acc);
  else spmv_pq_tile<S, NR, LPR, U>(beg, end, row_ptr, ColsWide{cols}, vals, p, q, acc);
  block_sum_t<1, S>(acc, sh);
  if (threadIdx.x == 0) part[t] = (double)acc[0];
}

// ---------------------------------------------------------------- bulk-copy SpMV
// the largest tile's nonzeros and rows (for the bulk-copy SpMV's staging size)
__global__ void k_tile_max(Tiles T, const int32_t* __restrict__ row_ptr, unsigned long long* __restrict__ mx) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.n) return;
  const int64_t b = T.tab[2 * t], e = T.tab[2 * t + 1];
  atomicMax(mx, (unsigned long long)(row_ptr[e] - row_ptr[b]));
  atomicMax(mx + 1, (unsigned long long)(e - b));
}


// The same q = A p with the fused p.q as k_spmv_pq_k, but each CTA first stages its tile's
// row pointers, FP32 values and column stream into shared memory with 1-D bulk asynchronous
// copies (cp.async.bulk, completing on an mbarrier) and then runs the row loop from shared
// memory: the per-row chain of dependent global loads (row pointers, then values and
// columns, then the gathers of p) loses its first two links, and the copy engine keeps a
// whole tile of bytes in flight per CTA.  Windows are widened to 16-byte boundaries (the
// bulk copy's alignment rule); the workspace allocations carry the slack that the widened
// end may read.  The staging wait is bounded: past its iteration limit the CTA sets T.err,
// waits once more (bounded) for its own copies and returns.
// bytes of one tile's stage (row pointers, values, columns) for the largest tile
template <class S, int NW>
inline size_t spmv_stage_bytes(const Tiles& T) {
  auto up16 = [](int64_t b) { return (size_t)((b + 15) & ~(int64_t)15); };
  return up16(4 * (T.max_rows + 1) + 16) + up16((int64_t)sizeof(S) * T.max_nnz + 16) +
         up16((NW ? 2 : 4) * T.max_nnz + 16);
}
template <class S, int NW>
inline size_t spmv_tma_smem(const Tiles& T) {
  return 16 + spmv_stage_bytes<S, NW>(T);
}
constexpr size_t kSpmvTmaMaxSmem = 100 * 1024;  // two CTAs per SM at least

// One tile's windows and where they sit in a stage buffer.
struct SpmvWin {
  Win r, v, c;
};
template <class S, int NW>
__device__ __forceinline__ SpmvWin spmv_windows(const int32_t* row_ptr, const S* vals, const int32_t* cols,
                                                const uint16_t* c16, int64_t beg, int64_t end) {
  const int64_t e0 = row_ptr[beg], e1 = row_ptr[end];
  return SpmvWin{stage_window(row_ptr, beg, end + 1, 4), stage_window(vals, e0, e1, (int)sizeof(S)),
                 NW ? stage_window(c16, e0, e1, 2) : stage_window(cols, e0, e1, 4)};
}
// thread 0: arm `bar` for the tile's bytes and start its three copies into `buf`
__device__ __forceinline__ void spmv_issue(const SpmvWin& w, unsigned char* buf, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(w.r.bytes + w.v.bytes + w.c.bytes)
               : "memory");
  bulk_g2s(buf, w.r.src, w.r.bytes, bar);
  bulk_g2s(buf + w.r.bytes, w.v.src, w.v.bytes, bar);
  bulk_g2s(buf + w.r.bytes + w.v.bytes, w.c.src, w.c.bytes, bar);
}

// The row loop of spmv_pq_tile over a staged tile: row pointers, values and columns read from
// the stage buffer (the same arithmetic in the same order, so the same bits).
template <class S, int NR, int LPR, int U, int NW>
__device__ __forceinline__ void spmv_staged_tile(int64_t beg, int64_t end, const SpmvWin& w,
                                                 const unsigned char* buf, int32_t cb, const S* __restrict__ p,
                                                 S* __restrict__ q, S& acc) {
  const int32_t* rs = reinterpret_cast<const int32_t*>(buf);
  const S* vs = reinterpret_cast<const S*>(buf + w.r.bytes);
  const unsigned char* sc = buf + w.r.bytes + w.v.bytes;
  struct {
    const unsigned char* sc;
    int64_t first;
    int32_t cb;
    __device__ __forceinline__ int32_t row_base(int64_t i) const { return narrow_row_base<NW>(cb, i); }
    __device__ __forceinline__ int32_t operator()(int64_t e, int32_t rb) const {
      if constexpr (NW != 0) return rb + (int32_t)(reinterpret_cast<const uint16_t*>(sc)[e - first]);
      else return reinterpret_cast<const int32_t*>(sc)[e - first];
    }
  } col{sc, w.c.first, cb};
  constexpr int K = (8 + LPR - 1) / LPR;
  const int sub = threadIdx.x % LPR;
  const int rpp = kTileThreads / LPR;
  for (int64_t base = beg; base < end; base += (int64_t)rpp * U) {
    int lo[U], hi[U];
    int32_t rb[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
      rb[u] = col.row_base(i);
      const bool valid = i < end;
      lo[u] = valid ? rs[i - w.r.first] : 0;
      hi[u] = valid ? rs[i + 1 - w.r.first] : 0;
    }
    S av[U][K];
    int cv[U][K];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int e = lo[u] + sub + k * LPR;
        const bool in = e < hi[u];
        av[u][k] = in ? vs[e - w.v.first] : S(0);
        cv[u][k] = in ? col(e, rb[u]) : -1;
      }
    V<S, NR> sm[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int c = 0; c < NR; ++c) sm[u].c[c] = S(0);
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (cv[u][k] >= 0) {
          const V<S, NR> pv = ldv<S, NR>(p, cv[u][k]);
#pragma unroll
          for (int c = 0; c < NR; ++c) sm[u].c[c] += av[u][k] * pv.c[c];
        }
      for (int e = lo[u] + sub + K * LPR; e < hi[u]; e += LPR) {  // rows longer than K * LPR
        const S a = vs[e - w.v.first];
        const V<S, NR> pv = ldv<S, NR>(p, col(e, rb[u]));
#pragma unroll
        for (int c = 0; c < NR; ++c) sm[u].c[c] += a * pv.c[c];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < NR; ++c) sm[u].c[c] += __shfl_xor_sync(0xffffffffu, sm[u].c[c], o, LPR);
    if (sub == 0) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
        if (i < end) {
          stv<S, NR>(q, i, sm[u]);
          const V<S, NR> pi = ldv<S, NR>(p, i);
#pragma unroll
          for (int c = 0; c < NR; ++c) acc += pi.c[c] * sm[u].c[c];
        }
      }
    }
  }
}

template <class S, int NR, int LPR, int U, int NW>
__global__ void __launch_bounds__(kTileThreads) k_spmv_tma(Tiles T, const ChartState* __restrict__ st,
                                                           const int32_t* __restrict__ row_ptr,
                                                           const int32_t* __restrict__ cols,
                                                           const uint16_t* __restrict__ c16,
                                                           const int32_t* __restrict__ cbase, const S* __restrict__ vals,
                                                           const S* __restrict__ p, S* __restrict__ q,
                                                           double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char stage[];
  __shared__ S sh[32];
  const int64_t t = blockIdx.x;
  const int32_t ch = T.chart[t];
  if (st[ch].state != kActive) return;
  const int64_t beg = T.tab[2 * t], end = T.tab[2 * t + 1];
  const SpmvWin w = spmv_windows<S, NW>(row_ptr, vals, cols, c16, beg, end);
  uint64_t* bar = reinterpret_cast<uint64_t*>(stage);
  unsigned char* buf = stage + 16;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    spmv_issue(w, buf, bar);
  }
  __syncthreads();  // the barrier is initialised before anyone waits on it
  // one decision for the whole CTA: a wait that ran out in any thread sends every thread out
  if (__syncthreads_or(!mbar_wait(bar, 0, T.spin_limit))) {
    if (threadIdx.x == 0) atomicOr(T.err, 1);
    mbar_wait(bar, 0, T.spin_limit);  // (bounded) let this CTA's own copies land before it exits
    return;
  }
  S acc = S(0);
  spmv_staged_tile<S, NR, LPR, U, NW>(beg, end, w, buf, NW == 1 ? cbase[ch] : 0, p, q, acc);
  S accv[1] = {acc};
  block_sum_t<1, S>(accv, sh);
  if (threadIdx.x == 0) part[t] = (double)accv[0];
}

// One launch of the SpMV for a column stream of kind nw (0 wide, 1 chart-relative, 2 row-
// relative): the bulk-copy kernel when the context set it up (upload_tiles) and its stage fits,
// else the CSR-vector kernel.
template <class S, int NR, int LPR, int U, int NW>
void launch_spmv_nw(cudaStream_t s, unsigned grid, const Tiles& T, const ChartState* st, const int32_t* row_ptr,
                    const int32_t* cols, const uint16_t* c16, const int32_t* cbase, const S* vals, const S* p, S* q,
                    double* part) {
  if constexpr (std::is_same<S, float>::value && NR == 2) {
    const size_t sm = spmv_tma_smem<S, NW>(T);
    if (T.max_rows > 0 && sm <= kSpmvTmaMaxSmem) {
      k_spmv_tma<S, NR, LPR, U, NW><<<grid, kTileThreads, sm, s>>>(T, st, row_ptr, cols, c16, cbase, vals, p, q, part);
      return;
    }
  }
  k_spmv_pq_k<S, NR, LPR, U, NW><<<grid, kTileThreads, 0, s>>>(T, st, row_ptr, cols, c16, cbase, vals, p, q, part);
}
template <class S, int NR, int LPR, int U>
void launch_spmv(cudaStream_t s, unsigned grid, const Tiles& T, const ChartState* st, const DevSystem& sys,
                 const S* vals, const S* p, S* q, double* part) {
  if (sys.cols16 && sys.rowrel16)
    launch_spmv_nw<S, NR, LPR, U, 2>(s, grid, T, st, sys.row_ptr, sys.cols, sys.cols16, sys.cbase, vals, p, q, part);
  else if (sys.cols16)
    launch_spmv_nw<S, NR, LPR, U, 1>(s, grid, T, st, sys.row_ptr, sys.cols, sys.cols16, sys.cbase, vals, p, q, part);
  else
    launch_spmv_nw<S, NR, LPR, U, 0>(s, grid, T, st, sys.row_ptr, sys.cols, sys.cols16, sys.cbase, vals, p, q, part);
}

// Allows the bulk-copy kernels the dynamic shared memory they need (outside any capture).
template <class S, int NR, int LPR, int U>
void spmv_tma_attributes(const Tiles& T) {
  if constexpr (std::is_same<S, float>::value && NR == 2) {
    if (T.max_rows <= 0) return;
    RUV_CUDA(cudaFuncSetAttribute(k_spmv_tma<S, NR, LPR, U, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kSpmvTmaMaxSmem));
    RUV_CUDA(cudaFuncSetAttribute(k_spmv_tma<S, NR, LPR, U, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kSpmvTmaMaxSmem));
    RUV_CUDA(cudaFuncSetAttribute(k_spmv_tma<S, NR, LPR, U, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kSpmvTmaMaxSmem));
  }
}

// x += alpha p; r -= alpha q; z = M^-1 r.  Partials: r.r, r.z.  precond: 0 = none (z = r),
// 1 = Jacobi, 2 = applied separately afterwards (z is not written).
template <class S, int NR>
__global__ void __launch_bounds__(kTileThreads) k_update(Tiles T, const ChartState* __restrict__ st,
                                                         const S* __restrict__ dinv, int use_jacobi,
                                                         S* __restrict__ x, S* __restrict__ r, S* __restrict__ z,
                                                         const S* __restrict__ p, const S* __restrict__ q,
                                                         double* __restrict__ part) {
  __shared__ S sh[2 * 32];
  int64_t t = blockIdx.x;
  const ChartState& cs = st[T.chart[t]];
  if (cs.state != kActive) return;
  const S alpha = std::is_same<S, float>::value ? (S)cs.alpha32 : (S)cs.alpha;
  S acc[2] = {S(0), S(0)};
  for (int64_t i = T.tab[2 * t] + threadIdx.x; i < T.tab[2 * t + 1]; i += blockDim.x) {
    V<S, NR> xv = ldv<S, NR>(x, i), rv = ldv<S, NR>(r, i), pv = ldv<S, NR>(p, i), qv = ldv<S, NR>(q, i), zv;
    const S di = use_jacobi == 1 ? dinv[i] : S(1);
#pragma unroll
    for (int k = 0; k < NR; ++k) {
      xv.c[k] += alpha * pv.c[k];
      rv.c[k] -= alpha * qv.c[k];
      zv.c[k] = rv.c[k] * di;
      acc[0] += rv.c[k] * rv.c[k];
      acc[1] += rv.c[k] * zv.c[k];
    }
    stv<S, NR>(x, i, xv);
    stv<S, NR>(r, i, rv);
    if (use_jacobi != 2) stv<S, NR>(z, i, zv);
  }
  block_sum_t<2, S>(acc, sh);
  if (threadIdx.x == 0) {
    part[2 * t] = (double)acc[0];
    part[2 * t + 1] = (double)acc[1];
  }
}

// p = z + beta p
template <class S, int NR>
__global__ void __launch_bounds__(kTileThreads) k_direction(Tiles T, const ChartState* __restrict__ st,
                                                            const S* __restrict__ z, S* __restrict__ p) {
  int64_t t = blockIdx.x;
  const ChartState& cs = st[T.chart[t]];
  if (cs.state != kActive) return;
  const S beta = std::is_same<S, float>::value ? (S)cs.beta32 : (S)cs.beta;
  for (int64_t i = T.tab[2 * t] + threadIdx.x; i < T.tab[2 * t + 1]; i += blockDim.x) {
    V<S, NR> zv = ldv<S, NR>(z, i), pv = ldv<S, NR>(p, i);
#pragma unroll
    for (int k = 0; k < NR; ++k) pv.c[k] = zv.c[k] + beta * pv.c[k];
    stv<S, NR>(p, i, pv);
  }
}

// Mixed precision, once per solve: the low FP32 halves of the FP64 values (vals32 holds the
// high halves) and the FP64 row sums as double-float pairs.
__global__ void k_split_rows(int64_t n, const int32_t* __restrict__ row_ptr, const double* __restrict__ vals,
                             const float* __restrict__ vals32, float* __restrict__ vals_lo, float2* __restrict__ rsum) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = 0.0;
  for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
    const double v = vals[e];
    vals_lo[e] = (float)(v - (double)vals32[e]);
    acc += v;
  }
  float h, l;
  split_f64(acc, h, l);
  rsum[i] = make_float2(h, l);
}

// Mixed precision, refresh step 1 (charts that asked for a refresh, or every chart when
// `all`): fold the FP32 increment into the double-float solution, xs = 0.  A separate launch
// from the true residual, which reads the solution of neighbouring rows in other tiles.
// With `all` (end of the solve) the FP64 solution x64 = hi + lo is written too.
template <int NR>
__global__ void __launch_bounds__(kTileThreads) k_fold(Tiles T, const ChartState* __restrict__ st, int all,
                                                       float* __restrict__ xdf, float* __restrict__ xs,
                                                       double* __restrict__ x64) {
  int64_t t = blockIdx.x;
  const ChartState& cs = st[T.chart[t]];
  if (!all && (cs.state != kActive || !cs.refresh)) return;
  for (int64_t i = T.tab[2 * t] + threadIdx.x; i < T.tab[2 * t + 1]; i += blockDim.x) {
    DF<NR> xv = lddf<NR>(xdf, i);
    V<float, NR> dv = ldv<float, NR>(xs, i), zero;
#pragma unroll
    for (int k = 0; k < NR; ++k) {
      float sh, se;
      two_sum(xv.h[k], dv.c[k], sh, se);
      se += xv.l[k];
      xv.h[k] = sh + se;  // renormalise: |lo| <= ulp(hi) / 2
      xv.l[k] = se - (xv.h[k] - sh);
      zero.c[k] = 0.f;
    }
    stdf<NR>(xdf, i, xv);
    stv<float, NR>(xs, i, zero);
    if (all) {
      V<double, NR> x;
#pragma unroll
      for (int k = 0; k < NR; ++k) x.c[k] = (double)xv.h[k] + (double)xv.l[k];
      stv<double, NR>(x64, i, x);
    }
  }
}

// Mixed precision, refresh step 2: r = b - A x in double-float (see the file comment),
// r32 = r, z = M^-1 r (precond 0: z = r, 1: Jacobi, 2: applied separately, z not written).
// Partials: r.r and r.z, summed in FP32 over r * rscale and rescaled per tile.  The CSR-vector
// shape (LPR lanes, K = ceil(8 / LPR) slots, U rows in flight) is the tuned SpMV's.
template <int NR, int LPR, int U, int NW>
__global__ void __launch_bounds__(kTileThreads) k_true_residual(Tiles T, const ChartState* __restrict__ st,
                                                                const int32_t* __restrict__ row_ptr,
                                                                const int32_t* __restrict__ cols,
                                                                const uint16_t* __restrict__ c16,
                                                                const int32_t* __restrict__ cbase, const float* __restrict__ vh,
                                                                const float* __restrict__ vl, const float2* __restrict__ rsum,
                                                                const float* __restrict__ bdf, const float* __restrict__ dinv,
                                                                int precond, const float* __restrict__ xdf,
                                                                float* __restrict__ r, float* __restrict__ z,
                                                                double* __restrict__ part) {
  constexpr int K = (8 + LPR - 1) / LPR;
  __shared__ float sh[2 * 32];
  const int64_t t = blockIdx.x;
  const ChartState& cs = st[T.chart[t]];
  if (cs.state != kActive || !cs.refresh) return;
  const float rsc = cs.rscale;
  const int sub = threadIdx.x % LPR;
  const int rpp = kTileThreads / LPR;
  float acc[2] = {0.0f, 0.0f};
  const int64_t beg = T.tab[2 * t], end = T.tab[2 * t + 1];
  auto run = [&](auto col) {
  for (int64_t base = beg; base < end; base += (int64_t)rpp * U) {
    int lo[U], hi[U];
    int32_t rb[U];
    DF<NR> xi[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
      rb[u] = col.row_base(i);
      const bool valid = i < end;
      lo[u] = valid ? row_ptr[i] : 0;
      hi[u] = valid ? row_ptr[i + 1] : 0;
      xi[u] = lddf<NR>(xdf, valid ? i : beg);
    }
    float ah[U][K], al[U][K];
    int cv[U][K];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int e = lo[u] + sub + k * LPR;
        const bool in = e < hi[u];
        ah[u][k] = in ? vh[e] : 0.0f;
        al[u][k] = in ? vl[e] : 0.0f;
        cv[u][k] = in ? col(e, rb[u]) : -1;
      }
    float Sh[U][NR], Sl[U][NR];
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int c = 0; c < NR; ++c) Sh[u][c] = Sl[u][c] = 0.0f;
      auto entry = [&](float a_h, float a_l, int j) {
        const DF<NR> xj = lddf<NR>(xdf, j);
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          float dh, dl;
          two_sum(xj.h[c], -xi[u].h[c], dh, dl);
          dl += xj.l[c] - xi[u].l[c];
          df_fma(a_h, a_l, dh, dl, Sh[u][c], Sl[u][c]);
        }
      };
#pragma unroll
      for (int k = 0; k < K; ++k)
        if (cv[u][k] >= 0) entry(ah[u][k], al[u][k], cv[u][k]);
      for (int e = lo[u] + sub + K * LPR; e < hi[u]; e += LPR) entry(vh[e], vl[e], col(e, rb[u]));
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          const float oh = __shfl_xor_sync(0xffffffffu, Sh[u][c], o, LPR);
          const float ol = __shfl_xor_sync(0xffffffffu, Sl[u][c], o, LPR);
          float s2, e2;
          two_sum(Sh[u][c], oh, s2, e2);
          Sh[u][c] = s2;
          Sl[u][c] += ol + e2;
        }
      const int64_t i = base + threadIdx.x / LPR + (int64_t)u * rpp;
      if (sub == 0 && i < end) {
        const float2 rs = rsum[i];
        const DF<NR> bv = lddf<NR>(bdf, i);
        const float di = precond == 1 ? dinv[i] : 1.0f;
        V<float, NR> rv, zv;
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          // A x = rs * x_i + S
          float th = 0.0f, tl = 0.0f;
          df_fma(rs.x, rs.y, xi[u].h[c], xi[u].l[c], th, tl);
          float ah2, ae2;
          two_sum(th, Sh[u][c], ah2, ae2);
          const float axl = tl + Sl[u][c] + ae2;
          // r = b - A x
          float uh, ue;
          two_sum(bv.h[c], -ah2, uh, ue);
          ue += bv.l[c] - axl;
          rv.c[c] = uh + ue;
          zv.c[c] = rv.c[c] * di;
          const float rs_ = rv.c[c] * rsc;
          acc[0] += rs_ * rs_;
          acc[1] += rs_ * (zv.c[c] * rsc);
        }
        stv<float, NR>(r, i, rv);
        if (precond != 2) stv<float, NR>(z, i, zv);
      }
    }
  }
  };
  if constexpr (NW == 1) run(ColsNarrow{c16, cbase[T.chart[t]]});
  else if constexpr (NW == 2) run(ColsRowRel{c16});
  else run(ColsWide{cols});
  block_sum_t<2, float>(acc, sh);
  if (threadIdx.x == 0) {
    const double inv = 1.0 / ((double)rsc * (double)rsc);
    part[2 * t] = (double)acc[0] * inv;
    part[2 * t + 1] = (double)acc[1] * inv;
  }
}

// One launch of the true residual for the system's column stream kind.
template <int NR, int LPR, int U, class MX>
void launch_true_residual(cudaStream_t s, unsigned grid, const Tiles& T, const ChartState* st, const DevSystem& sys,
                          const MX& mx, const float* dinv32, int precond, float* r, float* z, double* part) {
#define RUV_TR(NWV)                                                                                                   \
  k_true_residual<NR, LPR, U, NWV><<<grid, kTileThreads, 0, s>>>(T, st, sys.row_ptr, sys.cols, sys.cols16, sys.cbase, \
                                                                sys.vals32, mx.vals_lo, mx.rsum, mx.bdf, dinv32,      \
                                                                precond, mx.xdf, r, z, part)
  if (sys.cols16 && sys.rowrel16) RUV_TR(2);
  else if (sys.cols16) RUV_TR(1);
  else RUV_TR(0);
#undef RUV_TR
}

// ---------------------------------------------------------------- chart kernels
template <int NV>
__device__ __forceinline__ void chart_reduce(const Tiles& T, int64_t c, const double* part, int stride, double (&v)[NV],
                                             double* sh) {
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = 0.0;
  for (int64_t t = T.chart_tile[c] + threadIdx.x; t < T.chart_tile[c + 1]; t += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += part[stride * t + k];
  block_sum<NV>(v, sh);
}

__global__ void __launch_bounds__(kChartThreads) k_chart_init(Tiles T, ChartState* __restrict__ st, const double* __restrict__ part,
                                                              double tol, int precond_none, int* __restrict__ n_active) {
  __shared__ double sh[3 * 32];
  int64_t c = blockIdx.x;
  double v[3];
  chart_reduce<3>(T, c, part, 3, v, sh);
  if (threadIdx.x != 0) return;
  ChartState s{};
  s.bnorm = sqrt(v[0]);
  s.tol_abs = s.bnorm <= 1e-300 ? tol : tol * s.bnorm;
  s.rscale = s.bnorm > 0.0 ? (float)fmin(fmax(1.0 / s.bnorm, 1e-30), 1e30) : 1.0f;
  s.rr = v[0];
  s.r_ref = s.bnorm;
  s.rz = precond_none ? v[0] : v[1];
  s.iters = 0;
  s.refinements = 0;
  s.refresh = 0;
  if (v[2] > 0.0 && !precond_none) {
    s.status = RUV_ERR_BREAKDOWN;  // Jacobi with a zero diagonal (precond.rs:595-611)
    s.state = kDone;
  } else if (sqrt(v[0]) <= s.tol_abs) {
    s.status = RUV_OK;
    s.state = kDone;
  } else {
    s.status = RUV_ERR_NOT_CONVERGED;
    s.state = kActive;
    atomicAdd(n_active, 1);
  }
  st[c] = s;
}

__global__ void __launch_bounds__(kChartThreads) k_chart_alpha(Tiles T, ChartState* __restrict__ st, const double* __restrict__ part,
                                                               int* __restrict__ n_active) {
  __shared__ double sh[32];
  int64_t c = blockIdx.x;
  if (st[c].state != kActive) return;
  double v[1];
  chart_reduce<1>(T, c, part, 1, v, sh);
  if (threadIdx.x != 0) return;
  ChartState& s = st[c];
  double pap = v[0];
  if (fabs(pap) <= 1e-300 || !isfinite(pap)) {  // solver.rs:505-508
    s.status = RUV_ERR_BREAKDOWN;
    s.state = kDone;
    atomicSub(n_active, 1);
    return;
  }
  s.alpha = s.rz / pap;
  s.alpha32 = (float)s.alpha;
}

// FP64 path: convergence on the recurrence residual (solver.rs:518-522), then beta.
__global__ void __launch_bounds__(kChartThreads) k_chart_beta(Tiles T, ChartState* __restrict__ st, const double* __restrict__ part,
                                                              int precond_none, int64_t max_iter, int* __restrict__ n_active) {
  __shared__ double sh[2 * 32];
  int64_t c = blockIdx.x;
  if (st[c].state != kActive) return;
  double v[2];
  chart_reduce<2>(T, c, part, 2, v, sh);
  if (threadIdx.x != 0) return;
  ChartState& s = st[c];
  s.iters += 1;
  s.rr = v[0];
  if (sqrt(v[0]) <= s.tol_abs) {
    s.status = RUV_OK;
    s.state = kDone;
    atomicSub(n_active, 1);
    return;
  }
  if (s.iters >= max_iter) {
    s.status = RUV_ERR_NOT_CONVERGED;
    s.state = kDone;
    atomicSub(n_active, 1);
    return;
  }
  double rznew = precond_none ? v[0] : v[1];
  s.beta = rznew / s.rz;
  s.beta32 = (float)s.beta;
  s.rz = rznew;
}

// Mixed path: the FP32 residual only schedules true-residual refreshes.
__global__ void __launch_bounds__(kChartThreads) k_chart_beta_mixed(Tiles T, ChartState* __restrict__ st,
                                                                    const double* __restrict__ part, int precond_none,
                                                                    int64_t max_iter, int* __restrict__ n_active,
                                                                    int separate_precond, double delta) {
  __shared__ double sh[2 * 32];
  int64_t c = blockIdx.x;
  if (st[c].state != kActive) return;
  double v[2];
  chart_reduce<2>(T, c, part, 2, v, sh);
  if (threadIdx.x != 0) return;
  ChartState& s = st[c];
  s.iters += 1;
  double rn = sqrt(v[0]);
  double rznew = precond_none ? v[0] : v[1];
  if (rn <= delta * s.r_ref || rn <= s.tol_abs || !isfinite(rn) || s.iters >= max_iter) {
    s.refresh = 1;  // beta is formed after the refresh, from the true residual
  } else {
    s.refresh = 0;
    if (!separate_precond) {  // (a separate preconditioner forms beta after its apply)
      s.beta = rznew / s.rz;
      s.beta32 = (float)s.beta;
      s.rz = rznew;
    }
  }
  (void)n_active;
}

__global__ void __launch_bounds__(kChartThreads) k_chart_after_refresh(Tiles T, ChartState* __restrict__ st,
                                                                       const double* __restrict__ part, int precond_none,
                                                                       int64_t max_iter, int* __restrict__ n_active,
                                                                       int separate_precond) {
  __shared__ double sh[2 * 32];
  int64_t c = blockIdx.x;
  if (st[c].state != kActive || !st[c].refresh) return;
  double v[2];
  chart_reduce<2>(T, c, part, 2, v, sh);
  if (threadIdx.x != 0) return;
  ChartState& s = st[c];
  s.refinements += 1;
  s.rr = v[0];
  double rn = sqrt(v[0]);
  if (rn <= s.tol_abs) {
    s.status = RUV_OK;
    s.state = kDone;
    atomicSub(n_active, 1);
    return;
  }
  if (!isfinite(rn)) {
    s.status = RUV_ERR_BREAKDOWN;
    s.state = kDone;
    atomicSub(n_active, 1);
    return;
  }
  if (s.iters >= max_iter) {
    s.status = RUV_ERR_NOT_CONVERGED;
    s.state = kDone;
    atomicSub(n_active, 1);
    return;
  }
  s.r_ref = rn;
  if (separate_precond) {
    s.refresh = 2;  // refreshed: the beta kernel uses the plain Fletcher-Reeves ratio
    return;
  }
  double rznew = precond_none ? v[0] : v[1];
  s.beta = rznew / s.rz;
  s.beta32 = (float)s.beta;
  s.rz = rznew;
  s.refresh = 0;
}

// ---------------------------------------------------------------- separate preconditioner
// (AMG) support: done mask, r.z / z.q partials, chart-level beta.
__global__ void k_mark_done(const ChartState* __restrict__ st, int64_t n, int32_t* __restrict__ done) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) done[c] = st[c].state != kActive ? 1 : 0;
}

template <class S, int NR>
__global__ void __launch_bounds__(kTileThreads) k_dots_rz(Tiles T, const ChartState* __restrict__ st, const S* __restrict__ r,
                                                          const S* __restrict__ z, const S* __restrict__ q,
                                                          double* __restrict__ part) {
  __shared__ S sh[2 * 32];
  int64_t t = blockIdx.x;
  if (st[T.chart[t]].state != kActive) return;
  S acc[2] = {S(0), S(0)};
  for (int64_t i = T.tab[2 * t] + threadIdx.x; i < T.tab[2 * t + 1]; i += blockDim.x) {
    const V<S, NR> rv = ldv<S, NR>(r, i), zv = ldv<S, NR>(z, i), qv = ldv<S, NR>(q, i);
#pragma unroll
    for (int k = 0; k < NR; ++k) {
      acc[0] += rv.c[k] * zv.c[k];
      acc[1] += zv.c[k] * qv.c[k];
    }
  }
  block_sum_t<2, S>(acc, sh);
  if (threadIdx.x == 0) {
    part[2 * t] = (double)acc[0];
    part[2 * t + 1] = (double)acc[1];
  }
}

template <class S, int NR>
__global__ void __launch_bounds__(kTileThreads) k_copy_dir(Tiles T, const ChartState* __restrict__ st, const S* __restrict__ z,
                                                           S* __restrict__ p) {
  int64_t t = blockIdx.x;
  if (st[T.chart[t]].state != kActive) return;
  for (int64_t i = T.tab[2 * t] + threadIdx.x; i < T.tab[2 * t + 1]; i += blockDim.x) stv<S, NR>(p, i, ldv<S, NR>(z, i));
}

// FP64 outer loop with a separate preconditioner: convergence on the recurrence residual
// (solver.rs:518-522); beta comes after the apply.
__global__ void __launch_bounds__(kChartThreads) k_chart_check64(Tiles T, ChartState* __restrict__ st,
                                                                 const double* __restrict__ part, int64_t max_iter,
                                                                 int* __restrict__ n_active) {
  __shared__ double sh[2 * 32];
  int64_t c = blockIdx.x;
  if (st[c].state != kActive) return;
  double v[2];
  chart_reduce<2>(T, c, part, 2, v, sh);
  if (threadIdx.x != 0) return;
  ChartState& s = st[c];
  s.iters += 1;
  s.rr = v[0];
  if (sqrt(v[0]) <= s.tol_abs) {
    s.status = RUV_OK;
    s.state = kDone;
    atomicSub(n_active, 1);
  } else if (!isfinite(v[0])) {
    s.status = RUV_ERR_BREAKDOWN;
    s.state = kDone;
    atomicSub(n_active, 1);
  } else if (s.iters >= max_iter) {
    s.status = RUV_ERR_NOT_CONVERGED;
    s.state = kDone;
    atomicSub(n_active, 1);
  }
}

// FP64 <-> FP32 copies of the preconditioner's input / output (FP64 outer loop).
template <class A, class Bt>
__global__ void k_convert(int64_t n, const A* __restrict__ in, Bt* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (Bt)in[i];
}

// After the first apply: rz = r.z.
__global__ void __launch_bounds__(kChartThreads) k_chart_rz0(Tiles T, ChartState* __restrict__ st, const double* __restrict__ part) {
  __shared__ double sh[2 * 32];
  int64_t c = blockIdx.x;
  if (st[c].state != kActive) return;
  double v[2];
  chart_reduce<2>(T, c, part, 2, v, sh);
  if (threadIdx.x == 0) st[c].rz = v[0];
}

// beta after a separate apply: flexible (Polak-Ribiere, as the reference's FCG for AMG,
// solver.rs:474-481, :526-539) using r_new - r_old = -alpha q, or Fletcher-Reeves right
// after a true-residual refresh (r jumped).
__global__ void __launch_bounds__(kChartThreads) k_chart_beta_pc(Tiles T, ChartState* __restrict__ st,
                                                                 const double* __restrict__ part, int flexible) {
  __shared__ double sh[2 * 32];
  int64_t c = blockIdx.x;
  if (st[c].state != kActive) return;
  double v[2];
  chart_reduce<2>(T, c, part, 2, v, sh);
  if (threadIdx.x != 0) return;
  ChartState& s = st[c];
  const double rznew = v[0];
  double beta = (flexible && s.refresh != 2) ? (-s.alpha * v[1]) / s.rz : rznew / s.rz;
  if (!isfinite(beta)) beta = 0.0;
  s.beta = beta;
  s.beta32 = (float)beta;
  s.rz = rznew;
  s.refresh = 0;
}

// ---------------------------------------------------------------- host driver
struct TileTable {
  std::vector<int64_t> tab, chart_tile;
  std::vector<int32_t> chart;
};

// Mixed precision's double-float state: solution and right-hand side (2 * NR floats per
// row), the low halves of the FP64 values and the FP64 row sums (k_split_rows, launched here).
struct MixedExtras {
  float* xdf = nullptr;
  float* bdf = nullptr;
  float* vals_lo = nullptr;
  float2* rsum = nullptr;
};

MixedExtras mixed_extras(Ctx& ctx, DevSystem& sys, int nr) {
  MixedExtras m;
  if (nr == 0) return m;
  const int64_t N = sys.n_rows;
  m.xdf = ctx.ws.get<float>("pcg.xdf", 2 * nr * N);
  m.bdf = ctx.ws.get<float>("pcg.bdf", 2 * nr * N);
  if (sys.vals_lo && sys.rsum) {  // formed by the assembly's fill pass
    m.vals_lo = sys.vals_lo;
    m.rsum = sys.rsum;
    return m;
  }
  m.vals_lo = ctx.ws.get<float>("pcg.vals_lo", sys.nnz);
  m.rsum = ctx.ws.get<float2>("pcg.rsum", N);
  if (N > 0) {
    k_split_rows<<<div_up(N, kTileThreads), kTileThreads, 0, ctx.stream>>>(N, sys.row_ptr, sys.vals, sys.vals32, m.vals_lo,
                                                                           m.rsum);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  return m;
}

template <class S, int NR, int LPR, int U>
void run_pcg(Ctx& ctx, DevSystem& sys, double* x64, const SolveOpts& o, Tiles T, ChartState* st, int* n_active,
             std::vector<ChartState>& out) {
  cudaStream_t s = ctx.stream;
  Workspace& ws = ctx.ws;
  const bool mixed = std::is_same<S, float>::value;
  const int64_t NR_ = sys.n_rows, NC = sys.n_charts, NTL = T.n;
  const int jac = o.precond == RUV_PRECOND_JACOBI ? 1 : 0;
  const int none = o.precond == RUV_PRECOND_NONE ? 1 : 0;
  S* xs = mixed ? ws.get<S>("pcg.xs", NR * NR_) : nullptr;
  S* r = ws.get<S>("pcg.r", NR * NR_);
  S* z = ws.get<S>("pcg.z", NR * NR_);
  S* p = ws.get<S>("pcg.p", NR * NR_);
  S* q = ws.get<S>("pcg.q", NR * NR_);
  S* dinv = ws.get<S>("pcg.dinv", NR_);
  float* dinv32 = mixed ? reinterpret_cast<float*>(dinv) : nullptr;
  double* part = ws.get<double>("pcg.part", 3 * NTL);
  const S* vals = mixed ? reinterpret_cast<const S*>(sys.vals32) : reinterpret_cast<const S*>(sys.vals);
  MixedExtras mx = mixed_extras(ctx, sys, mixed ? NR : 0);
  RUV_CUDA(cudaMemsetAsync(n_active, 0, sizeof(int), s));
  if (NR_ > 0) {
    k_dinv<S><<<div_up(NR_, kTileThreads), kTileThreads, 0, s>>>(NR_, sys.diag, dinv);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  if (NTL > 0) {
    k_init<S, NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, sys.b, sys.diag, dinv, jac, x64, xs, r, z, p, part, mx.xdf,
                                                         mx.bdf);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  k_chart_init<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, o.tol, none, n_active);
  count_launches(1);
  RUV_LAUNCH_CHECK();
  int* h_active = static_cast<int*>(ctx.pinned.get(3 * sizeof(int)));
  spmv_tma_attributes<S, NR, LPR, U>(T);
  RUV_CUDA(cudaMemcpyAsync(h_active, n_active, sizeof(int), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  if (*h_active > 0 && NTL > 0) {
    // capture kCheckEvery iterations as one graph, replay it
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    RUV_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int rep = 0; rep < kCheckEvery; ++rep) {
      launch_spmv<S, NR, LPR, U>(s, (unsigned)NTL, T, st, sys, vals, p, q, part);
      k_chart_alpha<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, n_active);
      k_update<S, NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, dinv, jac, mixed ? xs : reinterpret_cast<S*>(x64), r,
                                                             z, p, q, part);
      if (!mixed) {
        k_chart_beta<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, none, o.max_iter, n_active);
      } else {
        k_chart_beta_mixed<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, none, o.max_iter, n_active, 0,
                                                                  refresh_delta());
        k_fold<NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, 0, mx.xdf, reinterpret_cast<float*>(xs), x64);
        launch_true_residual<NR, LPR, U>(s, (unsigned)NTL, T, st, sys, mx, dinv32, jac, reinterpret_cast<float*>(r),
                                         reinterpret_cast<float*>(z), part);
        k_chart_after_refresh<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, none, o.max_iter, n_active, 0);
      }
      k_direction<S, NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, z, p);
    }
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess) throw Error{RUV_ERR_LAUNCH, std::string("graph capture: ") + cudaGetErrorString(ce)};
    ce = cudaGraphInstantiate(&exec, graph, 0);
    if (ce != cudaSuccess) {
      cudaGraphDestroy(graph);
      throw Error{RUV_ERR_LAUNCH, std::string("graph instantiate: ") + cudaGetErrorString(ce)};
    }
    int64_t launched = 0;
    try {
      while (launched < o.max_iter + kCheckEvery) {
        RUV_CUDA(cudaGraphLaunch(exec, s));
        count_launches((int64_t)kCheckEvery * (mixed ? 8 : 5));
        launched += kCheckEvery;
        RUV_CUDA(cudaMemcpyAsync(h_active, n_active, sizeof(int), cudaMemcpyDeviceToHost, s));
        if (T.err) RUV_CUDA(cudaMemcpyAsync(h_active + 2, T.err, sizeof(int), cudaMemcpyDeviceToHost, s));
        RUV_CUDA(cudaStreamSynchronize(s));
        if (T.err && h_active[2] != 0) {
          RUV_CUDA(cudaMemsetAsync(T.err, 0, sizeof(int), s));
          throw Error{RUV_ERR_TIMEOUT, "SpMV: a bounded wait for the staged tile ran out"};
        }
        if (*h_active <= 0) break;
      }
    } catch (...) {
      cudaGraphExecDestroy(exec);
      cudaGraphDestroy(graph);
      throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
  }
  if (mixed && NTL > 0) {
    // fold any FP32 increment still pending (charts that stopped between refreshes); x64 = xdf
    k_fold<NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, 1, mx.xdf, reinterpret_cast<float*>(xs), x64);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  out.resize(NC);
  RUV_CUDA(cudaMemcpyAsync(out.data(), st, sizeof(ChartState) * NC, cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
}

// Batched PCG with a separately applied preconditioner (AMG V-cycle, IC(0) sweeps): the
// mixed loop (FP32 recurrences, double-float true-residual refreshes) or the FP64 loop.
// A preconditioner that has no FP64 form gets FP32 copies of r and z under the FP64 loop.
template <class S, int NR, int LPR, int U>
void run_pcg_sep(Ctx& ctx, DevSystem& sys, double* x64, const SolveOpts& o, Tiles T, ChartState* st, int* n_active,
                 std::vector<ChartState>& out, SepPrecond& P) {
  constexpr bool mixed = std::is_same<S, float>::value;
  cudaStream_t s = ctx.stream;
  Workspace& ws = ctx.ws;
  const int64_t NR_ = sys.n_rows, NC = sys.n_charts, NTL = T.n;
  S* xs = mixed ? ws.get<S>("pcg.xs", NR * NR_) : nullptr;
  S* r = ws.get<S>("pcg.r", NR * NR_);
  S* z = ws.get<S>("pcg.z", NR * NR_);
  S* p = ws.get<S>("pcg.p", NR * NR_);
  S* q = ws.get<S>("pcg.q", NR * NR_);
  S* dinv = ws.get<S>("pcg.dinv", NR_);
  float* dinv32 = mixed ? reinterpret_cast<float*>(dinv) : nullptr;
  const bool copies = !mixed && !P.native_fp64();
  float* r32 = copies ? ws.get<float>("pcg.r32", NR * NR_) : reinterpret_cast<float*>(r);
  float* z32 = copies ? ws.get<float>("pcg.z32", NR * NR_) : reinterpret_cast<float*>(z);
  const S* vals = mixed ? reinterpret_cast<const S*>(sys.vals32) : reinterpret_cast<const S*>(sys.vals);
  S* xiter = mixed ? xs : reinterpret_cast<S*>(x64);
  double* part = ws.get<double>("pcg.part", 3 * NTL);
  double* part2 = ws.get<double>("pcg.part2", 2 * NTL);
  MixedExtras mx = mixed_extras(ctx, sys, mixed ? NR : 0);
  int32_t* done = ws.get<int32_t>("pcg.done", NC);
  if (copies) P.bind(ctx, r32, z32, false);
  else P.bind(ctx, r, z, !mixed);
  const int flex = P.flexible() ? 1 : 0;
  const unsigned gv = div_up(NR * NR_, 256);
  auto to32 = [&]() {
    if (copies) k_convert<S, float><<<gv, 256, 0, s>>>(NR * NR_, r, r32);
  };
  auto to64 = [&]() {
    if (copies) k_convert<float, S><<<gv, 256, 0, s>>>(NR * NR_, z32, z);
  };
  const int conv = copies ? 2 : 0;
  RUV_CUDA(cudaMemsetAsync(n_active, 0, sizeof(int), s));
  if (NR_ > 0) {
    k_dinv<S><<<div_up(NR_, kTileThreads), kTileThreads, 0, s>>>(NR_, sys.diag, dinv);
    count_launches(1);
  }
  if (NTL > 0) {
    k_init<S, NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, sys.b, sys.diag, dinv, 1, x64, xs, r, z, p, part, mx.xdf,
                                                         mx.bdf);
    count_launches(1);
  }
  k_chart_init<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, o.tol, 0, n_active);  // (rz replaced below)
  count_launches(1);
  RUV_LAUNCH_CHECK();
  int* h_active = static_cast<int*>(ctx.pinned.get(3 * sizeof(int)));
  spmv_tma_attributes<S, NR, LPR, U>(T);
  RUV_CUDA(cudaMemcpyAsync(h_active, n_active, sizeof(int), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  if (*h_active > 0 && NTL > 0) {
    // z0 = M^-1 r0, rz = r.z, p = z
    k_mark_done<<<div_up(NC, 256), 256, 0, s>>>(st, NC, done);
    to32();
    count_launches(1 + conv + P.apply(ctx, done));
    to64();
    k_dots_rz<S, NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, r, z, q, part2);
    k_chart_rz0<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part2);
    k_copy_dir<S, NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, z, p);
    count_launches(3);
    RUV_LAUNCH_CHECK();
    constexpr int kRep = 8;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int per_iter = 0;
    RUV_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int rep = 0; rep < kRep; ++rep) {
      int l = 0;
      launch_spmv<S, NR, LPR, U>(s, (unsigned)NTL, T, st, sys, vals, p, q, part);
      k_chart_alpha<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, n_active);
      k_update<S, NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, dinv, 2, xiter, r, z, p, q, part);
      if (mixed) {
        k_chart_beta_mixed<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, 1, o.max_iter, n_active, 1,
                                                                  refresh_delta());
        k_fold<NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, 0, mx.xdf, reinterpret_cast<float*>(xs), x64);
        launch_true_residual<NR, LPR, U>(s, (unsigned)NTL, T, st, sys, mx, dinv32, 2, reinterpret_cast<float*>(r),
                                         reinterpret_cast<float*>(z), part);
        k_chart_after_refresh<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, 1, o.max_iter, n_active, 1);
        l += 4;
      } else {
        k_chart_check64<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part, o.max_iter, n_active);
        l += 1;
      }
      k_mark_done<<<div_up(NC, 256), 256, 0, s>>>(st, NC, done);
      to32();
      l += 4 + conv;
      l += P.apply(ctx, done);
      to64();
      k_dots_rz<S, NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, r, z, q, part2);
      k_chart_beta_pc<<<(unsigned)NC, kChartThreads, 0, s>>>(T, st, part2, flex);
      k_direction<S, NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, z, p);
      l += 3;
      per_iter = l;
    }
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess) throw Error{RUV_ERR_LAUNCH, std::string("graph capture: ") + cudaGetErrorString(ce)};
    ce = cudaGraphInstantiate(&exec, graph, 0);
    if (ce != cudaSuccess) {
      cudaGraphDestroy(graph);
      throw Error{RUV_ERR_LAUNCH, std::string("graph instantiate: ") + cudaGetErrorString(ce)};
    }
    int64_t launched = 0;
    const int* perr = P.error_flag();
    try {
      while (launched < o.max_iter + kRep) {
        RUV_CUDA(cudaGraphLaunch(exec, s));
        count_launches((int64_t)kRep * per_iter);
        launched += kRep;
        RUV_CUDA(cudaMemcpyAsync(h_active, n_active, sizeof(int), cudaMemcpyDeviceToHost, s));
        if (perr) RUV_CUDA(cudaMemcpyAsync(h_active + 1, perr, sizeof(int), cudaMemcpyDeviceToHost, s));
        if (T.err) RUV_CUDA(cudaMemcpyAsync(h_active + 2, T.err, sizeof(int), cudaMemcpyDeviceToHost, s));
        RUV_CUDA(cudaStreamSynchronize(s));
        if (T.err && h_active[2] != 0) {
          RUV_CUDA(cudaMemsetAsync(T.err, 0, sizeof(int), s));
          throw Error{RUV_ERR_TIMEOUT, "SpMV: a bounded wait for the staged tile ran out"};
        }
        if (perr && h_active[1] != 0) {
          RUV_CUDA(cudaMemsetAsync(const_cast<int*>(perr), 0, sizeof(int), s));
          throw Error{RUV_ERR_TIMEOUT, "preconditioner: a bounded device-side wait ran out"};
        }
        if (*h_active <= 0) break;
      }
    } catch (...) {
      cudaGraphExecDestroy(exec);
      cudaGraphDestroy(graph);
      throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
  }
  if (mixed && NTL > 0) {
    k_fold<NR><<<(unsigned)NTL, kTileThreads, 0, s>>>(T, st, 1, mx.xdf, reinterpret_cast<float*>(xs), x64);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  out.resize(NC);
  RUV_CUDA(cudaMemcpyAsync(out.data(), st, sizeof(ChartState) * NC, cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
}

// The SpMV shape: lanes per row (LPR) and rows in flight per sub-warp (U).  Instantiated
// for the shapes the tuner explores; see pick_shape.
struct Shape {
  int lpr, unroll;
};

#define RUV_SHAPES(X) X(1, 2) X(2, 2) X(2, 4) X(4, 1) X(4, 2) X(4, 4) X(8, 1) X(8, 2) X(8, 4) X(16, 1) X(32, 1)

template <class S, int NR>
void dispatch_pcg(Shape sh, Ctx& ctx, DevSystem& sys, double* x64, const SolveOpts& o, Tiles T, ChartState* st,
                  int* n_active, std::vector<ChartState>& out) {
#define RUV_CASE(L, UU) \
  if (sh.lpr == L && sh.unroll == UU) return run_pcg<S, NR, L, UU>(ctx, sys, x64, o, T, st, n_active, out);
  RUV_SHAPES(RUV_CASE)
#undef RUV_CASE
  throw Error{RUV_ERR_BAD_INPUT, "unsupported SpMV shape"};
}

TileTable make_tiles(const std::vector<int64_t>& chart_row, int64_t tile_rows);

Tiles upload_tiles(Ctx& ctx, const DevSystem& sys, const std::string& tag) {
  cudaStream_t s = ctx.stream;
  TileTable TT = make_tiles(sys.h_chart_row, ctx.tile_rows);
  const int64_t NTL = (int64_t)TT.chart.size(), NC = sys.n_charts;
  int64_t* d_tab = ctx.ws.get<int64_t>(tag + ".tab", 2 * NTL);
  int32_t* d_chart = ctx.ws.get<int32_t>(tag + ".tchart", NTL);
  int64_t* d_ctile = ctx.ws.get<int64_t>(tag + ".ctile", NC + 1);
  if (NTL > 0) {
    RUV_CUDA(cudaMemcpyAsync(d_tab, TT.tab.data(), sizeof(int64_t) * 2 * NTL, cudaMemcpyHostToDevice, s));
    RUV_CUDA(cudaMemcpyAsync(d_chart, TT.chart.data(), sizeof(int32_t) * NTL, cudaMemcpyHostToDevice, s));
  }
  RUV_CUDA(cudaMemcpyAsync(d_ctile, TT.chart_tile.data(), sizeof(int64_t) * (NC + 1), cudaMemcpyHostToDevice, s));
  Tiles T{d_tab, d_chart, d_ctile, NTL};
  // the bulk-copy SpMV (when the context chose it, or RUV_SPMV_TMA=1 / =0 says so): its
  // staging size from the largest tile
  const char* te = std::getenv("RUV_SPMV_TMA");
  const bool tma = te ? te[0] == '1' : ctx.spmv_tma == 1;
  if (NTL > 0 && sys.row_ptr && tma) {
    unsigned long long* mx = ctx.ws.get<unsigned long long>(tag + ".tmax", 2);
    int* err = ctx.ws.get<int>(tag + ".terr", 1);
    RUV_CUDA(cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), s));
    RUV_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    k_tile_max<<<div_up(NTL, 256), 256, 0, s>>>(T, sys.row_ptr, mx);
    count_launches(1);
    unsigned long long h[2] = {0, 0};
    RUV_CUDA(cudaMemcpyAsync(h, mx, sizeof(h), cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaStreamSynchronize(s));
    T.max_nnz = (int64_t)h[0];
    T.max_rows = (int64_t)h[1];
    T.err = err;
    const char* le = std::getenv("RUV_SPIN_LIMIT");
    T.spin_limit = le ? std::max<int64_t>(1, std::atoll(le)) : (int64_t(1) << 22);
  }
  RUV_CUDA(cudaStreamSynchronize(s));  // the host tables go out of scope
  return T;
}

// SpMV shape: explicit (RUV_LPR / RUV_UNROLL via the context) or from the row-length
// profile: enough lanes to cover a typical row once, then as many rows in flight as keep
// 8 independent loads per lane.
// The launch shape without the autotuner: for mesh Laplacians (at most 8 entries per row) two
// lanes per row and two rows in flight, which the autotuner picked on every such operator
// measured (4096 disks, 1024^2 and 2048^2 height fields); wider sub-warps for denser rows.
Shape pick_shape(const Ctx& ctx, const DevSystem& sys) {
  double avg = sys.n_rows > 0 ? (double)sys.nnz / (double)sys.n_rows : 1.0;
  int lpr = ctx.lanes_per_row > 0 ? ctx.lanes_per_row : (avg <= 8 ? 2 : avg <= 12 ? 8 : avg <= 24 ? 16 : 32);
  int u = ctx.unroll > 0 ? ctx.unroll : (lpr <= 4 ? 2 : lpr == 8 ? 4 : 1);
  return Shape{lpr, u};
}

template <class S, int NR, int LPR, int U>
double time_spmv(Ctx& ctx, DevSystem& sys, Tiles T, int reps, int nbuf, bool iter) {
  cudaStream_t s = ctx.stream;
  spmv_tma_attributes<S, NR, LPR, U>(T);
  const int64_t N = sys.n_rows, NC = sys.n_charts;
  ChartState* st = ctx.ws.get<ChartState>("bench.state", NC);
  RUV_CUDA(cudaMemsetAsync(st, 0, sizeof(ChartState) * NC, s));  // every chart active
  double* part = ctx.ws.get<double>("bench.part", T.n);
  // iter: also the tile kernels of a CG iteration that run over the same tiles (update, dots,
  // direction), whose cost depends on the tile height as well
  S* xv = iter ? ctx.ws.get<S>("bench.x", NR * N) : nullptr;
  S* rv = iter ? ctx.ws.get<S>("bench.r", NR * N) : nullptr;
  double* part2 = iter ? ctx.ws.get<double>("bench.part2", 2 * T.n) : nullptr;
  if (iter) {
    RUV_CUDA(cudaMemsetAsync(xv, 0, sizeof(S) * NR * N, s));
    RUV_CUDA(cudaMemsetAsync(rv, 0, sizeof(S) * NR * N, s));
  }
  std::vector<S*> ps(nbuf), qs(nbuf);
  for (int k = 0; k < nbuf; ++k) {
    ps[k] = ctx.ws.get<S>("bench.p" + std::to_string(k), NR * N);
    qs[k] = ctx.ws.get<S>("bench.q" + std::to_string(k), NR * N);
    RUV_CUDA(cudaMemsetAsync(ps[k], 0, sizeof(S) * NR * N, s));
  }
  const S* vals = std::is_same<S, float>::value ? reinterpret_cast<const S*>(sys.vals32) : reinterpret_cast<const S*>(sys.vals);
  auto launch = [&](int k) {
    launch_spmv<S, NR, LPR, U>(s, (unsigned)T.n, T, st, sys, vals, ps[k % nbuf],
                               qs[k % nbuf], part);
    count_launches(1);
    if (iter && T.n > 0) {
      k_update<S, NR><<<(unsigned)T.n, kTileThreads, 0, s>>>(T, st, nullptr, 2, xv, rv, nullptr, ps[k % nbuf],
                                                             qs[k % nbuf], part2);
      k_dots_rz<S, NR><<<(unsigned)T.n, kTileThreads, 0, s>>>(T, st, rv, rv, qs[k % nbuf], part2);
      k_direction<S, NR><<<(unsigned)T.n, kTileThreads, 0, s>>>(T, st, rv, ps[k % nbuf]);
      count_launches(3);
    }
  };
  for (int k = 0; k < 3; ++k) launch(k);
  RUV_LAUNCH_CHECK();
  cudaEvent_t e0, e1;
  RUV_CUDA(cudaEventCreate(&e0));
  RUV_CUDA(cudaEventCreate(&e1));
  RUV_CUDA(cudaEventRecord(e0, s));
  for (int k = 0; k < reps; ++k) launch(k);
  RUV_CUDA(cudaEventRecord(e1, s));
  RUV_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  RUV_LAUNCH_CHECK();
  return (double)ms / reps;
}

template <class S, int NR>
void dispatch_pcg_sep(Shape sh, Ctx& ctx, DevSystem& sys, double* x64, const SolveOpts& o, Tiles T, ChartState* st,
                      int* n_active, std::vector<ChartState>& out, SepPrecond& P) {
#define RUV_CASE(L, UU) \
  if (sh.lpr == L && sh.unroll == UU) return run_pcg_sep<S, NR, L, UU>(ctx, sys, x64, o, T, st, n_active, out, P);
  RUV_SHAPES(RUV_CASE)
#undef RUV_CASE
  throw Error{RUV_ERR_BAD_INPUT, "unsupported SpMV shape"};
}

template <class S, int NR>
double dispatch_time(Shape sh, Ctx& ctx, DevSystem& sys, Tiles T, int reps, int nbuf, bool iter = false) {
#define RUV_CASE(L, UU) \
  if (sh.lpr == L && sh.unroll == UU) return time_spmv<S, NR, L, UU>(ctx, sys, T, reps, nbuf, iter);
  RUV_SHAPES(RUV_CASE)
#undef RUV_CASE
  throw Error{RUV_ERR_BAD_INPUT, "unsupported SpMV shape"};
}

TileTable make_tiles(const std::vector<int64_t>& chart_row, int64_t tile_rows) {
  TileTable T;
  int64_t nc = (int64_t)chart_row.size() - 1;
  T.chart_tile.assign(nc + 1, 0);
  for (int64_t c = 0; c < nc; ++c) {
    T.chart_tile[c] = (int64_t)T.chart.size();
    for (int64_t a = chart_row[c]; a < chart_row[c + 1]; a += tile_rows) {
      T.tab.push_back(a);
      T.tab.push_back(std::min(a + tile_rows, chart_row[c + 1]));
      T.chart.push_back((int32_t)c);
    }
  }
  T.chart_tile[nc] = (int64_t)T.chart.size();
  return T;
}

// 16-bit column stream, one thread per row: every entry as an offset from its chart's first
// row (all charts of at most 65536 rows), or with `rowrel` as an offset from its row's index
// minus 32768, *bad set where an entry lies more than 32767 rows from its row.
constexpr int64_t kNarrowRows = 65536;
__global__ void k_narrow_cols(int64_t n, const int64_t* __restrict__ chart_row, int64_t n_charts,
                              const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ cols, int rowrel,
                              uint16_t* __restrict__ c16, int* __restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (rowrel) {
    for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
      const int64_t d = (int64_t)cols[e] - i + kRowRelBias;
      if (d < 0 || d > 65535) {
        atomicOr(bad, 1);
        return;
      }
      c16[e] = (uint16_t)d;
    }
    return;
  }
  int64_t lo = 0, hi = n_charts;  // the chart of row i: largest c with chart_row[c] <= i
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (chart_row[mid] <= i) lo = mid; else hi = mid;
  }
  const int64_t r0 = chart_row[lo];
  for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) c16[e] = (uint16_t)(cols[e] - r0);
}
__global__ void k_chart_base(int64_t n_charts, const int64_t* __restrict__ chart_row, int32_t* __restrict__ cbase) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n_charts) cbase[c] = (int32_t)chart_row[c];
}

}  // namespace

// The 16-bit column stream of a chart-blocked CSR operator: chart-relative (cbase = each
// chart's first row) when every chart has at most 65536 rows, else row-relative (*rowrel,
// cbase null) when every entry lies within 32767 rows of its row.  Returns false and leaves
// the pointers null otherwise (the one case that reads a flag back: only operators with a
// chart above 65536 rows pay that synchronisation).  RUV_NARROW_COLS=chart: chart-relative
// streams only.
bool narrow_operator(Ctx& ctx, int64_t n, int64_t nnz, int64_t n_charts, const std::vector<int64_t>& h_chart_row,
                     const int64_t* chart_row, const int32_t* row_ptr, const int32_t* cols, const std::string& tag,
                     uint16_t** c16, int32_t** cbase, bool* rowrel) {
  *c16 = nullptr;
  *cbase = nullptr;
  *rowrel = false;
  bool large = false;
  for (int64_t c = 0; c < n_charts; ++c)
    if (h_chart_row[c + 1] - h_chart_row[c] > kNarrowRows) large = true;
  const char* env = std::getenv("RUV_NARROW_COLS");
  if (large && env && std::string(env) == "chart") return false;
  cudaStream_t s = ctx.stream;
  uint16_t* d16 = ctx.ws.get<uint16_t>(tag + ".c16", std::max<int64_t>(nnz, 1));
  int32_t* dbase = large ? nullptr : ctx.ws.get<int32_t>(tag + ".cbase", std::max<int64_t>(n_charts, 1));
  int* bad = ctx.ws.get<int>(tag + ".c16bad", 1);
  RUV_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
  if (n > 0) {
    k_narrow_cols<<<div_up(n, 256), 256, 0, s>>>(n, chart_row, n_charts, row_ptr, cols, large ? 1 : 0, d16, bad);
    count_launches(1);
  }
  if (!large && n_charts > 0) {
    k_chart_base<<<div_up(n_charts, 256), 256, 0, s>>>(n_charts, chart_row, dbase);
    count_launches(1);
  }
  RUV_LAUNCH_CHECK();
  if (large) {
    int h = 0;
    RUV_CUDA(cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaStreamSynchronize(s));
    if (h != 0) return false;
  }
  *c16 = d16;
  *cbase = dbase;
  *rowrel = large;
  return true;
}

// On unless RUV_NARROW_COLS=0: on the 4096-disk operator the 16-bit stream cuts the SpMV's
// bytes by 18% and its time by 13% (0.215 -> 0.187 ms); RUV_NARROW_COLS=chart keeps it to
// charts of at most 65536 rows (larger charts then make the whole operator 32-bit).
void narrow_columns(Ctx& ctx, DevSystem& sys) {
  const char* e = std::getenv("RUV_NARROW_COLS");
  if (e && e[0] == '0') {  // 32-bit columns only
    sys.cols16 = nullptr;
    sys.cbase = nullptr;
    sys.rowrel16 = false;
    return;
  }
  narrow_operator(ctx, sys.n_rows, sys.nnz, sys.n_charts, sys.h_chart_row, sys.chart_row, sys.row_ptr, sys.cols,
                  "sys", &sys.cols16, &sys.cbase, &sys.rowrel16);
}

double bench_spmv(Ctx& ctx, DevSystem& sys, bool mixed, int reps, int n_buffers, double* bytes,
                  double* stream_bytes) {
  narrow_columns(ctx, sys);
  Tiles T = upload_tiles(ctx, sys, "bench");
  const Shape sh = pick_shape(ctx, sys);
  const double N = (double)sys.n_rows, NNZ = (double)sys.nnz, nr = (double)sys.nrhs;
  const double vb = mixed ? 4.0 : 8.0;
  // column bytes per entry: 2 with the 16-bit stream (every chart has it then), 4 otherwise
  const double cb = sys.cols16 ? 2.0 : 4.0;
  // algorithmic bytes: values, 32-bit columns, row pointers, p read once, q written; the
  // stream bytes count the columns the kernel actually reads (16-bit where narrowed)
  if (bytes) *bytes = NNZ * (vb + 4.0) + (N + 1.0) * 4.0 + 2.0 * N * nr * vb;
  if (stream_bytes) *stream_bytes = NNZ * (vb + cb) + (N + 1.0) * 4.0 + 2.0 * N * nr * vb;
  if (T.n == 0) return 0.0;
  if (sys.nrhs == 2)
    return mixed ? dispatch_time<float, 2>(sh, ctx, sys, T, reps, n_buffers)
                 : dispatch_time<double, 2>(sh, ctx, sys, T, reps, n_buffers);
  return dispatch_time<double, 1>(sh, ctx, sys, T, reps, n_buffers);
}

// Autotuner: time the batched SpMV for every instantiated (lanes per row, rows in flight)
// shape, tile height and SpMV form (CSR-vector or bulk-copy staged) on the assembled operator,
// each with the update, dots and direction kernels of a CG iteration over the same tiles (the
// tile height sets their grid too); keep the fastest in the context.
TuneResult autotune_spmv(Ctx& ctx, DevSystem& sys, bool mixed, int reps) {
  narrow_columns(ctx, sys);
  TuneResult best{0, 0, 0, 0, 1e30};
  const int tiles[] = {128, 256, 512, 1024};
  const Shape shapes[] = {
#define RUV_SH(L, UU) Shape{L, UU},
      RUV_SHAPES(RUV_SH)
#undef RUV_SH
  };
  const int saved_tile = ctx.tile_rows, saved_tma = ctx.spmv_tma;
  // the bulk-copy kernel exists for the mixed solver's two-column SpMV only
  const int n_tma = mixed && sys.nrhs == 2 ? 2 : 1;
  for (int tr : tiles) {
    ctx.tile_rows = tr;
    for (int tma = 0; tma < n_tma; ++tma) {
      ctx.spmv_tma = tma;
      Tiles T = upload_tiles(ctx, sys, "tune");
      if (T.n == 0) break;
      for (const Shape& sh : shapes) {
        double ms = sys.nrhs == 2 ? (mixed ? dispatch_time<float, 2>(sh, ctx, sys, T, reps, 2, true)
                                           : dispatch_time<double, 2>(sh, ctx, sys, T, reps, 2, true))
                                  : dispatch_time<double, 1>(sh, ctx, sys, T, reps, 2, true);
        if (ms < best.ms) best = TuneResult{sh.lpr, sh.unroll, tr, tma, ms};
      }
    }
  }
  if (best.lpr > 0) {
    ctx.lanes_per_row = best.lpr;
    ctx.unroll = best.unroll;
    ctx.tile_rows = best.tile_rows;
    ctx.spmv_tma = best.tma;
  } else {
    ctx.tile_rows = saved_tile;
    ctx.spmv_tma = saved_tma;
  }
  return best;
}

std::vector<ChartResult> pcg_solve(Ctx& ctx, DevSystem& sys, double* x, const SolveOpts& o) {
  const bool sep = o.precond == RUV_PRECOND_AMG || o.precond == RUV_PRECOND_AMG_SA || o.precond == RUV_PRECOND_IC0 ||
                   o.precond == RUV_PRECOND_IC0_COLOR;
  if (o.precond != RUV_PRECOND_NONE && o.precond != RUV_PRECOND_JACOBI && !sep)
    throw Error{RUV_ERR_BAD_INPUT, "unknown preconditioner"};
  const int64_t NC = sys.n_charts;
  narrow_columns(ctx, sys);
  Tiles T = upload_tiles(ctx, sys, "pcg");
  ChartState* st = ctx.ws.get<ChartState>("pcg.state", NC);
  int* n_active = ctx.ws.get<int>("pcg.nactive", 1);
  const Shape sh = pick_shape(ctx, sys);
  std::vector<ChartState> out;
  const bool mixed = o.precision == RUV_PREC_MIXED;
  ctx.timings[3] = 0.0;
  if (sep) {
    // preconditioner set-up, timed on the stream
    cudaEvent_t e[2];
    RUV_CUDA(cudaEventCreate(&e[0]));
    RUV_CUDA(cudaEventCreate(&e[1]));
    struct EvGuard {
      cudaEvent_t* e;
      ~EvGuard() {
        cudaEventDestroy(e[0]);
        cudaEventDestroy(e[1]);
      }
    } guard{e};
    RUV_CUDA(cudaEventRecord(e[0], ctx.stream));
    std::unique_ptr<SepPrecond> P = (o.precond == RUV_PRECOND_AMG || o.precond == RUV_PRECOND_AMG_SA)
                                        ? make_amg(ctx, sys, o.precond == RUV_PRECOND_AMG_SA)
                                        : make_ic0(ctx, sys, o.precond == RUV_PRECOND_IC0_COLOR);
    RUV_CUDA(cudaEventRecord(e[1], ctx.stream));
    RUV_CUDA(cudaEventSynchronize(e[1]));
    float ms = 0.f;
    RUV_CUDA(cudaEventElapsedTime(&ms, e[0], e[1]));
    ctx.timings[3] = ms;
    if (sys.nrhs == 2) {
      if (mixed) dispatch_pcg_sep<float, 2>(sh, ctx, sys, x, o, T, st, n_active, out, *P);
      else dispatch_pcg_sep<double, 2>(sh, ctx, sys, x, o, T, st, n_active, out, *P);
    } else {
      if (mixed) dispatch_pcg_sep<float, 1>(sh, ctx, sys, x, o, T, st, n_active, out, *P);
      else dispatch_pcg_sep<double, 1>(sh, ctx, sys, x, o, T, st, n_active, out, *P);
    }
  } else if (sys.nrhs == 2) {
    if (mixed) dispatch_pcg<float, 2>(sh, ctx, sys, x, o, T, st, n_active, out);
    else dispatch_pcg<double, 2>(sh, ctx, sys, x, o, T, st, n_active, out);
  } else {
    // the generic drop-in (one scalar right-hand side) runs in FP64 as the reference does
    dispatch_pcg<double, 1>(sh, ctx, sys, x, o, T, st, n_active, out);
  }
  std::vector<ChartResult> res(NC);
  for (int64_t c = 0; c < NC; ++c) {
    const ChartState& cs = out[c];
    res[c].status = cs.status;
    res[c].iters = cs.iters;
    res[c].refinements = cs.refinements;
    res[c].rel_res = cs.bnorm > 1e-300 ? std::sqrt(cs.rr) / cs.bnorm : std::sqrt(cs.rr);
  }
  return res;
}


// ===================================================================== no-alloc CG
// A variant of the FP64 PCG behind ruv_cg_solve for callers that cannot allocate device
// memory: its scratch (the CG vectors, the inverse diagonal, tile partials, tile table and
// solver state) lives in one file-scope __device__ array of fixed size instead of the
// context workspace, the caller's device buffers hold the system and the solution, and
// the host loop issues plain launches (no CUDA graph, no pinned staging).
namespace {

constexpr int64_t kNoAllocMaxRows = RUV_NOALLOC_MAX_ROWS;
constexpr int kNoAllocTile = 256;
constexpr int64_t kNoAllocMaxTiles = (kNoAllocMaxRows + kNoAllocTile - 1) / kNoAllocTile;

struct NoAllocScratch {
  double r[kNoAllocMaxRows], z[kNoAllocMaxRows], p[kNoAllocMaxRows], q[kNoAllocMaxRows];
  double dinv[kNoAllocMaxRows], diag[kNoAllocMaxRows];
  double part[3 * kNoAllocMaxTiles];
  int64_t tab[2 * kNoAllocMaxTiles];
  int64_t chart_tile[2];
  int32_t tchart[kNoAllocMaxTiles];
  ChartState st;
  int32_t n_active;
  int32_t bad;
  int32_t nonfinite;
};

// The allocation-free solve's scratch (about 12.6 MB).  A __device__ array belongs to the
// module instance of this file, and every CUDA context that loads the module gets its own
// copy, mapped when the module loads (under CUDA's default lazy loading: the first launch or
// symbol query in that context) and held until the context ends.  Host code may not use the
// symbol's name as a device pointer; the entry point resolves the address in the current
// context on every call (a host-side lookup once the module is loaded), so a context other
// than the device's primary one, or a context created again after cudaDeviceReset, never
// sees an address of another context.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

__global__ void k_na_check_ptr(int32_t n, const int32_t* __restrict__ row_ptr, int32_t* __restrict__ bad) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && row_ptr[0] != 0) atomicExch(bad, 1);
  if (i < n && row_ptr[i + 1] < row_ptr[i]) atomicExch(bad, 1);
}

// Column check, diagonal extraction (first entry on the diagonal, as CsrMatrix::row_get)
// and the single-chart tile table.
__global__ void k_na_setup(int32_t n, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ cols,
                           const double* __restrict__ vals, NoAllocScratch* __restrict__ S) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    double d = 0.0;
    bool found = false;
    for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
      const int32_t c = cols[k];
      if (c < 0 || c >= n) atomicExch(&S->bad, 2);
      if (c == i && !found) {
        d = vals[k];
        found = true;
      }
    }
    S->diag[i] = d;
  }
  const int64_t n_tiles = (n + kNoAllocTile - 1) / kNoAllocTile;
  if (i < n_tiles) {
    S->tab[2 * i] = i * kNoAllocTile;
    S->tab[2 * i + 1] = min((int64_t)n, (i + 1) * kNoAllocTile);
    S->tchart[i] = 0;
  }
  if (i == 0) {
    S->chart_tile[0] = 0;
    S->chart_tile[1] = n_tiles;
  }
}

__global__ void k_na_nonfinite(int32_t n, const double* __restrict__ x, int32_t* __restrict__ flag) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !isfinite(x[i])) atomicExch(flag, 1);
}

void na_message(char* msg, int32_t len, const char* text) {
  if (msg && len > 0) {
    std::snprintf(msg, (size_t)len, "%s", text);
  }
}

template <int LPR, int U>
void na_iterations(cudaStream_t s, NoAllocScratch* S, Tiles T, const int32_t* row_ptr, const int32_t* cols,
                   const double* vals, double* x, int jac, int none, int64_t max_iter) {
  k_spmv_pq_k<double, 1, LPR, U, false><<<(unsigned)T.n, kTileThreads, 0, s>>>(T, &S->st, row_ptr, cols, nullptr, nullptr,
                                                                              vals, S->p, S->q, S->part);
  k_chart_alpha<<<1, kChartThreads, 0, s>>>(T, &S->st, S->part, &S->n_active);
  k_update<double, 1><<<(unsigned)T.n, kTileThreads, 0, s>>>(T, &S->st, S->dinv, jac, x, S->r, S->z, S->p, S->q, S->part);
  k_chart_beta<<<1, kChartThreads, 0, s>>>(T, &S->st, S->part, none, max_iter, &S->n_active);
  k_direction<double, 1><<<(unsigned)T.n, kTileThreads, 0, s>>>(T, &S->st, S->z, S->p);
}

}  // namespace
}  // namespace ruv

extern "C" ruv_status ruv_cg_solve_noalloc(int32_t n, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                                           const double* b, double* x, int64_t max_iter, double tol, ruv_precond pc,
                                           int64_t* iters_out, void* stream, char* msg, int32_t msg_len) {
  using namespace ruv;
  if (n <= 0 || !row_ptr || !cols || !vals || !b || !x) {
    na_message(msg, msg_len, "empty system or null device pointer");
    return RUV_ERR_BAD_INPUT;
  }
  if ((int64_t)n > kNoAllocMaxRows) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "n = %d exceeds the no-alloc scratch maximum of %lld rows (RUV_NOALLOC_MAX_ROWS)",
                  (int)n, (long long)kNoAllocMaxRows);
    na_message(msg, msg_len, buf);
    return RUV_ERR_BAD_INPUT;
  }
  if (pc != RUV_PRECOND_NONE && pc != RUV_PRECOND_JACOBI) {
    na_message(msg, msg_len, "the no-alloc solve supports PRECOND_NONE and PRECOND_JACOBI");
    return RUV_ERR_BAD_INPUT;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    na_message(msg, msg_len, "no current CUDA device");
    return RUV_ERR_NO_DEVICE;
  }
  // The scratch's address in the current context (see g_noalloc_scratch).
  NoAllocScratch* S = nullptr;
  {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      cudaGetLastError();
      na_message(msg, msg_len, "cudaGetSymbolAddress of the no-alloc scratch failed");
      return RUV_ERR_NO_DEVICE;
    }
    S = static_cast<NoAllocScratch*>(ptr);
  }
  auto launch_fail = [&](const char* what) {
    cudaGetLastError();
    na_message(msg, msg_len, what);
    return RUV_ERR_LAUNCH;
  };
  // flags that must start at zero on every call (the scratch keeps the last call's contents)
  if (cudaMemsetAsync(&S->n_active, 0, 3 * sizeof(int32_t), s) != cudaSuccess) return launch_fail("memset");
  const unsigned grid_n = div_up((int64_t)n + 1, 256);
  k_na_check_ptr<<<grid_n, 256, 0, s>>>(n, row_ptr, &S->bad);
  int32_t flags[3] = {0, 0, 0};
  if (cudaMemcpyAsync(flags, &S->n_active, sizeof(flags), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return launch_fail("row pointer check failed to run");
  if (flags[1]) {
    na_message(msg, msg_len, "row_ptr[0] != 0 or row_ptr not monotone");
    return RUV_ERR_BAD_INPUT;
  }
  k_na_setup<<<grid_n, 256, 0, s>>>(n, row_ptr, cols, vals, S);
  int32_t nnz = 0;
  if (cudaMemcpyAsync(flags, &S->n_active, sizeof(flags), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&nnz, row_ptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return launch_fail("set-up kernel failed");
  if (flags[1]) {
    na_message(msg, msg_len, "column index out of range");
    return RUV_ERR_BAD_INPUT;
  }
  const int jac = pc == RUV_PRECOND_JACOBI ? 1 : 0, none = pc == RUV_PRECOND_NONE ? 1 : 0;
  const int64_t n_tiles = (n + kNoAllocTile - 1) / kNoAllocTile;
  Tiles T{S->tab, S->tchart, S->chart_tile, n_tiles};
  k_dinv<double><<<div_up(n, kTileThreads), kTileThreads, 0, s>>>(n, S->diag, S->dinv);
  k_init<double, 1><<<(unsigned)n_tiles, kTileThreads, 0, s>>>(T, b, S->diag, S->dinv, jac, x, nullptr, S->r, S->z, S->p,
                                                               S->part, nullptr, nullptr);
  k_chart_init<<<1, kChartThreads, 0, s>>>(T, &S->st, S->part, tol, none, &S->n_active);
  const double avg = (double)nnz / (double)n;
  const int lpr = avg <= 5 ? 4 : avg <= 12 ? 8 : avg <= 24 ? 16 : 32;
  int64_t launched = 0;
  for (;;) {
    int32_t active = 0;
    if (cudaMemcpyAsync(&active, &S->n_active, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return launch_fail("CG iteration failed");
    if (active <= 0 || launched >= max_iter + kCheckEvery) break;
    for (int k = 0; k < kCheckEvery; ++k) {
      if (lpr == 4) na_iterations<4, 2>(s, S, T, row_ptr, cols, vals, x, jac, none, max_iter);
      else if (lpr == 8) na_iterations<8, 4>(s, S, T, row_ptr, cols, vals, x, jac, none, max_iter);
      else if (lpr == 16) na_iterations<16, 1>(s, S, T, row_ptr, cols, vals, x, jac, none, max_iter);
      else na_iterations<32, 1>(s, S, T, row_ptr, cols, vals, x, jac, none, max_iter);
    }
    if (cudaGetLastError() != cudaSuccess) return launch_fail("CG kernel launch failed");
    launched += kCheckEvery;
  }
  ChartState st;
  k_na_nonfinite<<<div_up(n, 256), 256, 0, s>>>(n, x, &S->nonfinite);
  if (cudaMemcpyAsync(&st, &S->st, sizeof(st), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(flags, &S->n_active, sizeof(flags), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return launch_fail("reading the solver state failed");
  if (iters_out) *iters_out = st.iters;
  if (st.status != RUV_OK) {
    na_message(msg, msg_len, st.status == RUV_ERR_NOT_CONVERGED ? "CG did not converge within max_iter" : "CG breakdown");
    return (ruv_status)st.status;
  }
  if (flags[2]) {
    na_message(msg, msg_len, "non-finite solution");
    return RUV_ERR_BREAKDOWN;
  }
  na_message(msg, msg_len, "");
  return RUV_OK;
}
