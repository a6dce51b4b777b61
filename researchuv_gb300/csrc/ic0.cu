// IC(0) preconditioner in natural or multi-colour ordering, set up and applied on the GPU:
// the sm_103a counterpart of gpu/src/precond.rs:49-123 (graph_coloring, color_permutation,
// permute_csr), :145-262 (factor_ic0, tri_levels, transpose_lower) and of the reference's
// per-level triangular-solve launches (gpu/src/solver.rs:205-270, :361-404).
//
// Batched: the factors of all charts live in one packed lower-triangular CSR (chart c keeps
// rows [chart_row[c], chart_row[c+1])).  Dependency levels are found per chart by one CTA
// with Kahn's layering (a row's level is 1 + the highest level among its dependencies, which
// is what tri_levels computes), and the factorization and both triangular sweeps walk those
// levels with one CTA per chart and a block barrier between levels: one launch per sweep for
// the whole batch instead of one launch per level.
//
// The factor equals the reference's host factor_ic0 bit for bit: the same ascending merge for
// L(i,k) = (A(i,k) - sum_{j<k} L(i,j) L(k,j)) / L(k,k), the same pivot floor
// 1e-12 * max(|a_ii|, 1e-30), FP64 with each operation rounded on its own (no FMA
// contraction).  The mixed-precision solver applies an FP32 copy of it.
//
// Large charts with many levels (natural ordering of a big grid-like chart: thousands of
// levels, ~1000 rows each) would leave one CTA per chart walking its levels serially.  There
// the factorization and both sweeps run sync-free over the whole GPU instead ("tickets"):
// rows are numbered in global level order, persistent warps take 32 consecutive numbers at a
// time from an atomic counter, and each thread waits on the done-flags of its row's
// dependencies (acquire loads) before computing the row and publishing it (release store).
// A row only waits on rows with smaller numbers, which were taken earlier by warps that are
// running, so the scheme needs no co-residency of the grid.  Every wait is bounded (a spin
// limit, RUV_SPIN_LIMIT iterations of a short sleep, about a second by default); a wait that
// runs out sets an error flag that ends every other wait at once, and the call reports
// RUV_ERR_TIMEOUT with the context still usable.  Each row's arithmetic is the same as in
// the per-chart path, so the results are bit-identical to it.
//
// Multi-colour ordering: the greedy colouring (smallest colour not taken by a lower-numbered
// neighbour, vertices in index order) depends on lower neighbours only, so it is computed on
// the same forward levels and equals the reference's sequential result.  The colour-major
// permutation (original index ascending within a colour, per chart) is a counting sort on
// the host; P A P^T is formed on the device and factored as above.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <memory>

#include "system.cuh"

namespace ruv {
namespace {

constexpr int kIcThreads = 256;

// ---------------------------------------------------------------- pattern of L and L^T
// lcnt[i] = strictly lower entries of row i + 1 (the diagonal); flags[0] |= 1 when row i
// has no diagonal entry or a zero one (factor_ic0 returns None, precond.rs:183-186).
__global__ void k_l_count(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                          const double* __restrict__ vals, int32_t* __restrict__ lcnt, int* __restrict__ flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = 1;
  bool diag = false;
  double a_ii = 0.0;
  for (int e = rp[i]; e < rp[i + 1]; ++e) {
    const int j = cols[e];
    if (j < i) ++c;
    if (j == i && !diag) {  // CsrMatrix::row_get: the first stored (i, i)
      diag = true;
      a_ii = vals[e];
    }
  }
  if (!(fabs(a_ii) >= 1e-300)) atomicOr(flags, 1);
  lcnt[i] = c;
}

// Row i of L: the strictly lower (column, value) pairs sorted by column, then (i, a_ii).
// Values start as A's and are overwritten by the factorization.  flags[0] |= 2 on a repeated
// column in the lower part (not supported: the reference's map would merge them).
__global__ void k_l_fill(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                         const double* __restrict__ vals, const int64_t* __restrict__ lptr, int32_t* __restrict__ lc,
                         double* __restrict__ lv, int* __restrict__ flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = lptr[i], end = lptr[i + 1];
  int64_t at = b;
  double a_ii = 0.0;
  bool diag = false;
  for (int e = rp[i]; e < rp[i + 1]; ++e) {
    const int j = cols[e];
    if (j < i) {
      // insertion by column (rows are short)
      int64_t k = at++;
      while (k > b && lc[k - 1] > j) {
        lc[k] = lc[k - 1];
        lv[k] = lv[k - 1];
        --k;
      }
      if (k > b && lc[k - 1] == j) atomicOr(flags, 2);
      lc[k] = j;
      lv[k] = vals[e];
    } else if (j == i && !diag) {
      diag = true;
      a_ii = vals[e];
    }
  }
  lc[end - 1] = (int32_t)i;
  lv[end - 1] = a_ii;
}

// Transpose pattern: tcnt[k] = #{i > k : L(i,k)} + 1.
__global__ void k_t_count(int64_t n, const int64_t* __restrict__ lptr, const int32_t* __restrict__ lc,
                          int32_t* __restrict__ tcnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t e = lptr[i]; e < lptr[i + 1] - 1; ++e) atomicAdd(&tcnt[lc[e]], 1);
  atomicAdd(&tcnt[i], 1);
}

// Scatter L's entries into L^T rows (src = position in L), then each row sorted by column
// with its diagonal last (transpose_lower, precond.rs:238-262).
__global__ void k_t_scatter(int64_t n, const int64_t* __restrict__ lptr, const int32_t* __restrict__ lc,
                            const int64_t* __restrict__ tptr, int32_t* __restrict__ cursor, int32_t* __restrict__ tc,
                            int64_t* __restrict__ tsrc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int64_t e = lptr[i]; e < lptr[i + 1]; ++e) {
    const int32_t k = e == lptr[i + 1] - 1 ? (int32_t)i : lc[e];  // the diagonal lands on its own row
    const int64_t at = tptr[k] + atomicAdd(&cursor[k], 1);
    tc[at] = (int32_t)i;
    tsrc[at] = e;
  }
}

__global__ void k_t_sort(int64_t n, const int64_t* __restrict__ tptr, int32_t* __restrict__ tc, int64_t* __restrict__ tsrc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t b = tptr[i], end = tptr[i + 1];
  for (int64_t k = b + 1; k < end; ++k) {
    const int32_t c = tc[k];
    const int64_t s = tsrc[k];
    int64_t j = k;
    // ascending, with column i (the diagonal) ordered after every other column
    auto key = [i](int32_t x) { return x == (int32_t)i ? INT32_MAX : x; };
    while (j > b && key(tc[j - 1]) > key(c)) {
      tc[j] = tc[j - 1];
      tsrc[j] = tsrc[j - 1];
      --j;
    }
    tc[j] = c;
    tsrc[j] = s;
  }
}

// ---------------------------------------------------------------- levels (one CTA per chart)
// Kahn's layering over the chart's rows: deps of row i are the off-diagonal entries of
// row i of D (D = L forward, L^T backward); the rows that depend on row k are the
// off-diagonal entries of row k of S (the other factor).  Rows of chart c are written level
// by level to rows[chart_row[c] ..]; level l of chart c starts at lev[chart_row[c] + c + l]
// (absolute position), n_lev[c] levels, lev[.. + n_lev[c]] = the chart's end.  flags |= 4 if
// some rows never became ready (cannot happen for a triangular factor).
__global__ void __launch_bounds__(kIcThreads) k_levels(const int64_t* __restrict__ chart_row, const int64_t* __restrict__ dptr,
                                                       const int64_t* __restrict__ sptr, const int32_t* __restrict__ sc,
                                                       int32_t* __restrict__ indeg, int32_t* __restrict__ rows,
                                                       int32_t* __restrict__ lev, int32_t* __restrict__ n_lev,
                                                       int* __restrict__ flags) {
  __shared__ int count;
  const int64_t c = blockIdx.x;
  const int64_t r0 = chart_row[c], r1 = chart_row[c + 1];
  int32_t* out = rows + r0;
  int32_t* lv = lev + r0 + c;
  if (threadIdx.x == 0) count = 0;
  __syncthreads();
  for (int64_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
    const int32_t d = (int32_t)(dptr[i + 1] - dptr[i] - 1);
    indeg[i] = d;
    if (d == 0) out[atomicAdd(&count, 1)] = (int32_t)i;
  }
  __syncthreads();
  int lo = 0, hi = count, nl = 0;
  const int total = (int)(r1 - r0);
  while (lo < hi) {
    if (threadIdx.x == 0) lv[nl] = (int32_t)(r0 + lo);
    ++nl;
    for (int idx = lo + threadIdx.x; idx < hi; idx += blockDim.x) {
      const int32_t k = out[idx];
      for (int64_t e = sptr[k]; e < sptr[k + 1] - 1; ++e) {
        const int32_t j = sc[e];
        if (atomicSub(&indeg[j], 1) == 1) out[atomicAdd(&count, 1)] = j;
      }
    }
    __syncthreads();
    lo = hi;
    hi = count;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    lv[nl] = (int32_t)r1;
    n_lev[c] = nl;
    if (hi != total) atomicOr(flags, 4);
  }
}

// ---------------------------------------------------------------- factorization (FP64)
// Per chart, level by level, one thread per row.  L(i,k) for the strictly lower entries in
// ascending k: s = A(i,k) minus L(i,j) L(k,j) over the common columns j < k (an ascending
// merge of row i's entries already computed and row k's finished row), divided by L(k,k);
// then L(i,i) = sqrt(max(A(i,i) - sum L(i,k)^2, floor)).  flags |= 8 when a pivot is below
// 1e-300 (factor_ic0 returns None, precond.rs:172-175).
__global__ void __launch_bounds__(kIcThreads) k_factor(const int64_t* __restrict__ chart_row, const int32_t* __restrict__ rows,
                                                       const int32_t* __restrict__ lev, const int32_t* __restrict__ n_lev,
                                                       const int64_t* __restrict__ lptr, const int32_t* __restrict__ lc,
                                                       double* lv, int* __restrict__ flags) {
  const int64_t c = blockIdx.x;
  const int32_t* lvl = lev + chart_row[c] + c;
  const int nl = n_lev[c];
  for (int l = 0; l < nl; ++l) {
    for (int idx = lvl[l] + threadIdx.x; idx < lvl[l + 1]; idx += blockDim.x) {
      const int32_t i = rows[idx];
      const int64_t b = lptr[i], d = lptr[i + 1] - 1;
      for (int64_t e = b; e < d; ++e) {
        const int32_t k = lc[e];
        double s = lv[e];
        const int64_t kb = lptr[k], kd = lptr[k + 1] - 1;
        int64_t q = kb;
        for (int64_t p = b; p < e; ++p) {  // row i's columns j < k, ascending
          const int32_t j = lc[p];
          while (q < kd && lc[q] < j) ++q;
          if (q < kd && lc[q] == j) s = __dsub_rn(s, __dmul_rn(lv[p], lv[q]));
        }
        const double l_kk = lv[kd];
        if (!(fabs(l_kk) >= 1e-300)) atomicOr(flags, 8);
        lv[e] = __ddiv_rn(s, l_kk);
      }
      const double a_ii = lv[d];
      double sum = a_ii;
      for (int64_t e = b; e < d; ++e) sum = __dsub_rn(sum, __dmul_rn(lv[e], lv[e]));
      const double fl = 1e-12 * fmax(fabs(a_ii), 1e-30);
      if (sum < fl) sum = fl;
      lv[d] = __dsqrt_rn(sum);
    }
    __syncthreads();
  }
}

__global__ void k_t_values(int64_t nnz, const int64_t* __restrict__ tsrc, const double* __restrict__ lv,
                           double* __restrict__ tv, float* __restrict__ tv32, float* __restrict__ lv32) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  const double v = lv[tsrc[e]];
  tv[e] = v;
  tv32[e] = (float)v;
  lv32[e] = (float)lv[e];
}

// Greedy colouring on the forward levels: colour(v) = the smallest colour not taken by a
// lower-numbered neighbour (graph_coloring, precond.rs:49-75).
__global__ void __launch_bounds__(kIcThreads) k_colour(const int64_t* __restrict__ chart_row, const int32_t* __restrict__ rows,
                                                       const int32_t* __restrict__ lev, const int32_t* __restrict__ n_lev,
                                                       const int64_t* __restrict__ lptr, const int32_t* __restrict__ lc,
                                                       int32_t* colour) {
  const int64_t c = blockIdx.x;
  const int32_t* lvl = lev + chart_row[c] + c;
  const int nl = n_lev[c];
  for (int l = 0; l < nl; ++l) {
    for (int idx = lvl[l] + threadIdx.x; idx < lvl[l + 1]; idx += blockDim.x) {
      const int32_t v = rows[idx];
      const int64_t b = lptr[v], d = lptr[v + 1] - 1;
      int k = 0;
      for (bool taken = true; taken; ) {
        taken = false;
        for (int64_t e = b; e < d; ++e)
          if (colour[lc[e]] == k) {
            taken = true;
            ++k;
            break;
          }
      }
      colour[v] = k;
    }
    __syncthreads();
  }
}

// P A P^T: row pos of the result is row to_orig[pos] with columns mapped through to_perm and
// sorted (permute_csr, precond.rs:103-123).
__global__ void k_perm_count(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ to_orig,
                             int32_t* __restrict__ cnt) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) cnt[p] = rp[to_orig[p] + 1] - rp[to_orig[p]];
}
__global__ void k_perm_fill(int64_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                            const double* __restrict__ vals, const int32_t* __restrict__ to_orig,
                            const int32_t* __restrict__ to_perm, const int32_t* __restrict__ prp, int32_t* __restrict__ pc,
                            double* __restrict__ pv) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int32_t o = to_orig[p];
  const int32_t b = prp[p];
  int32_t at = b;
  for (int e = rp[o]; e < rp[o + 1]; ++e) {
    const int32_t j = to_perm[cols[e]];
    int32_t k = at++;
    while (k > b && pc[k - 1] > j) {  // stable: equal columns keep their order
      pc[k] = pc[k - 1];
      pv[k] = pv[k - 1];
      --k;
    }
    pc[k] = j;
    pv[k] = vals[e];
  }
}

// ---------------------------------------------------------------- apply
template <class S, int NR>
struct Vec {
  S c[NR];
};
template <class S, int NR>
__device__ __forceinline__ Vec<S, NR> ldvec(const S* p, int64_t i) {
  Vec<S, NR> v;
#pragma unroll
  for (int k = 0; k < NR; ++k) v.c[k] = p[NR * i + k];
  return v;
}
template <class S, int NR>
__device__ __forceinline__ void stvec(S* p, int64_t i, const Vec<S, NR>& v) {
#pragma unroll
  for (int k = 0; k < NR; ++k) p[NR * i + k] = v.c[k];
}

// One triangular sweep per chart (charts marked done skip): for each level, every row of the
// level solves out[i] = (in[i] - sum_{off-diagonal e} v[e] out[col[e]]) / v[diagonal];
// forward with L, backward with L^T.  `out` is read and written in the same launch (no
// read-only path); the block barrier between levels publishes each level's results.
template <class S, int NR, int BT>
__global__ void __launch_bounds__(BT) k_sweep(const int64_t* __restrict__ chart_row, const int32_t* __restrict__ done,
                                                      const int32_t* __restrict__ rows, const int32_t* __restrict__ lev,
                                                      const int32_t* __restrict__ n_lev, const int64_t* __restrict__ ptr,
                                                      const int32_t* __restrict__ col, const S* __restrict__ val,
                                                      const S* __restrict__ in, S* out) {
  const int64_t c = blockIdx.x;
  if (done && done[c]) return;
  const int32_t* lvl = lev + chart_row[c] + c;
  const int nl = n_lev[c];
  for (int l = 0; l < nl; ++l) {
    for (int idx = lvl[l] + threadIdx.x; idx < lvl[l + 1]; idx += blockDim.x) {
      const int32_t i = rows[idx];
      const int64_t b = ptr[i], d = ptr[i + 1] - 1;
      Vec<S, NR> s = ldvec<S, NR>(in, i);
      for (int64_t e = b; e < d; ++e) {
        const S a = val[e];
        const Vec<S, NR> o = ldvec<S, NR>(out, col[e]);
#pragma unroll
        for (int k = 0; k < NR; ++k) s.c[k] -= a * o.c[k];
      }
      const S dg = val[d];
#pragma unroll
      for (int k = 0; k < NR; ++k) s.c[k] /= dg;
      stvec<S, NR>(out, i, s);
    }
    __syncthreads();
  }
}

// Global levels, for few and wide levels (a colour-ordered factor, a large chart): level l
// is the union of every chart's level l, solved by one grid-wide launch.
__global__ void __launch_bounds__(kIcThreads) k_row_level(const int64_t* __restrict__ chart_row,
                                                          const int32_t* __restrict__ rows, const int32_t* __restrict__ lev,
                                                          const int32_t* __restrict__ n_lev, int32_t* __restrict__ row_level,
                                                          int32_t* __restrict__ row_chart) {
  const int64_t c = blockIdx.x;
  const int32_t* lvl = lev + chart_row[c] + c;
  for (int l = 0; l < n_lev[c]; ++l)
    for (int idx = lvl[l] + threadIdx.x; idx < lvl[l + 1]; idx += blockDim.x) {
      row_level[rows[idx]] = l;
      row_chart[rows[idx]] = (int32_t)c;
    }
}
__global__ void k_level_hist(int64_t n, const int32_t* __restrict__ row_level, int32_t* __restrict__ hist) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&hist[row_level[i]], 1);
}
__global__ void k_level_scatter(int64_t n, const int32_t* __restrict__ row_level, int32_t* __restrict__ cursor,
                                int32_t* __restrict__ grows) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) grows[atomicAdd(&cursor[row_level[i]], 1)] = (int32_t)i;
}

// One global level: out[i] = (in[i] - sum v[e] out[col[e]]) / v[diagonal] for its rows.
template <class S, int NR>
__global__ void k_level_rows(const int32_t* __restrict__ lrows, int32_t count, const int32_t* __restrict__ row_chart,
                             const int32_t* __restrict__ done, const int64_t* __restrict__ ptr,
                             const int32_t* __restrict__ col, const S* __restrict__ val, const S* __restrict__ in, S* out) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int32_t i = lrows[t];
  if (done && done[row_chart[i]]) return;
  const int64_t b = ptr[i], d = ptr[i + 1] - 1;
  Vec<S, NR> s = ldvec<S, NR>(in, i);
  for (int64_t e = b; e < d; ++e) {
    const S a = val[e];
    const Vec<S, NR> o = ldvec<S, NR>(out, col[e]);
#pragma unroll
    for (int k = 0; k < NR; ++k) s.c[k] -= a * o.c[k];
  }
  const S dg = val[d];
#pragma unroll
  for (int k = 0; k < NR; ++k) s.c[k] /= dg;
  stvec<S, NR>(out, i, s);
}

// Colour permutation of the sweep's input / output: out[p] = in[to_orig[p]] (gather) or
// out[to_orig[p]] = in[p] (scatter).
template <class S, int NR, bool GATHER>
__global__ void k_permute(int64_t n, const int32_t* __restrict__ to_orig, const S* __restrict__ in, S* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int64_t o = to_orig[p];
  if (GATHER) stvec<S, NR>(out, p, ldvec<S, NR>(in, o));
  else stvec<S, NR>(out, o, ldvec<S, NR>(in, p));
}

// ---------------------------------------------------------------- sync-free (ticket) kernels
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Wait until flag == ep; false (and the error flag set) when the spin limit runs out or
// another wait has already failed.
__device__ __forceinline__ bool wait_ready(const int* flag, int ep, int* err, int64_t limit) {
  for (int64_t it = 0;; ++it) {
    if (ld_acquire(flag) == ep) return true;
    if (it >= limit || ld_relaxed(err) != 0) {
      atomicOr(err, 1);
      return false;
    }
    __nanosleep(64);
  }
}

// Per sweep: the next epoch (the value a finished row's flag takes) and a fresh ticket counter.
__global__ void k_ticket_begin(int* __restrict__ epoch, int* __restrict__ ticket) {
  *epoch += 1;
  *ticket = 0;
}

// 32 consecutive tickets for the calling warp; n or more when none are left.
__device__ __forceinline__ int64_t take_tickets(int* ticket) {
  int t0 = 0;
  if ((threadIdx.x & 31) == 0) t0 = atomicAdd(ticket, 32);
  return (int64_t)__shfl_sync(0xffffffffu, t0, 0);
}

// The factorization of k_factor over the rows in ticket order (forward dependencies).
__global__ void __launch_bounds__(kIcThreads) k_factor_ticket(const int32_t* __restrict__ order, int64_t n,
                                                              const int64_t* __restrict__ lptr, const int32_t* __restrict__ lc,
                                                              double* lv, int* __restrict__ ready, const int* __restrict__ epoch,
                                                              int* __restrict__ ticket, int* __restrict__ err, int64_t limit,
                                                              int* __restrict__ flags) {
  const int ep = *epoch;
  for (;;) {
    const int64_t t0 = take_tickets(ticket);
    if (t0 >= n) return;
    const int64_t t = t0 + (threadIdx.x & 31);
    if (t >= n) continue;
    const int32_t i = order[t];
    const int64_t b = lptr[i], d = lptr[i + 1] - 1;
    bool ok = true;
    for (int64_t e = b; e < d && ok; ++e) {
      const int32_t k = lc[e];
      if (!wait_ready(ready + k, ep, err, limit)) {
        ok = false;
        break;
      }
      double s = lv[e];
      const int64_t kb = lptr[k], kd = lptr[k + 1] - 1;
      int64_t q = kb;
      for (int64_t p = b; p < e; ++p) {
        const int32_t j = lc[p];
        while (q < kd && lc[q] < j) ++q;
        if (q < kd && lc[q] == j) s = __dsub_rn(s, __dmul_rn(lv[p], __ldcg(lv + q)));
      }
      const double l_kk = __ldcg(lv + kd);
      if (!(fabs(l_kk) >= 1e-300)) atomicOr(flags, 8);
      lv[e] = __ddiv_rn(s, l_kk);
    }
    if (!ok) continue;
    const double a_ii = lv[d];
    double sum = a_ii;
    for (int64_t e = b; e < d; ++e) sum = __dsub_rn(sum, __dmul_rn(lv[e], lv[e]));
    const double fl = 1e-12 * fmax(fabs(a_ii), 1e-30);
    if (sum < fl) sum = fl;
    lv[d] = __dsqrt_rn(sum);
    st_release(ready + i, ep);  // the row's entries are visible to every later acquire of its flag
  }
}

// One triangular sweep of k_sweep over the rows in ticket order (rows of charts marked done
// are skipped; their dependents are in the same chart).  The output is its own message: the
// sweep's output starts filled with all-one bits (a NaN that arithmetic never produces), a
// row's solved value replaces it, and a thread waiting on a dependency polls that value's
// components (aligned 4- or 8-byte words: each is read whole, old or new) until none holds
// the fill -- one load per component and no fences on either side.
template <class S>
struct Bits;
template <>
struct Bits<float> {
  using U = uint32_t;
  static __device__ __forceinline__ U load(const float* p) {
    U v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
  }
  static __device__ __forceinline__ void store(float* p, float x) {
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(__float_as_uint(x)) : "memory");
  }
  static __device__ __forceinline__ float value(U v) { return __uint_as_float(v); }
};
template <>
struct Bits<double> {
  using U = unsigned long long;
  static __device__ __forceinline__ U load(const double* p) {
    U v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
  }
  static __device__ __forceinline__ void store(double* p, double x) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(__double_as_longlong(x)) : "memory");
  }
  static __device__ __forceinline__ double value(U v) { return __longlong_as_double((long long)v); }
};

// A component of a solved row: spins (bounded, ending at once when another wait failed)
// until it no longer holds the fill.
template <class S>
__device__ __forceinline__ bool wait_value(const S* p, int* err, int64_t limit, S& out) {
  using B = Bits<S>;
  for (int64_t it = 0;; ++it) {
    const typename B::U v = B::load(p);
    if (v != (typename B::U)(~(typename B::U)0)) {
      out = B::value(v);
      return true;
    }
    if (it >= limit || ld_relaxed(err) != 0) {
      atomicOr(err, 1);
      return false;
    }
    if (it >= 32) __nanosleep(32);
  }
}

constexpr int kDeps = 4;  // dependencies a sweep row loads at once
// (a register cap instead of launch bounds: under __launch_bounds__(256) the FP32 two-column
// instance was held at 32 registers and spilled)

template <class S, int NR>
__global__ void __maxnreg__(48) k_sweep_ticket(const int32_t* __restrict__ order, int64_t n,
                                                             const int32_t* __restrict__ row_chart,
                                                             const int32_t* __restrict__ done, const int64_t* __restrict__ ptr,
                                                             const int32_t* __restrict__ col, const S* __restrict__ val,
                                                             const S* __restrict__ in, S* out, int* __restrict__ ticket,
                                                             int* __restrict__ err, int64_t limit) {
  for (;;) {
    const int64_t t0 = take_tickets(ticket);
    if (t0 >= n) return;
    const int64_t t = t0 + (threadIdx.x & 31);
    if (t >= n) continue;
    const int32_t i = order[t];
    if (done && done[row_chart[i]]) continue;
    const int64_t b = ptr[i], d = ptr[i + 1] - 1;
    Vec<S, NR> s = ldvec<S, NR>(in, i);
    bool ok = true;
    // The dependencies' components are loaded kDeps entries at a time, all loads in flight
    // together (one round trip to L2 instead of one per component); only those still holding
    // the fill are then waited on, and the row sums in entry order as before.
    for (int64_t e0 = b; e0 < d && ok; e0 += kDeps) {
      const int m = (int)(d - e0 < kDeps ? d - e0 : kDeps);
      typename Bits<S>::U raw[kDeps][NR];
      int32_t jj[kDeps];
#pragma unroll
      for (int q = 0; q < kDeps; ++q) {
        jj[q] = q < m ? col[e0 + q] : 0;
#pragma unroll
        for (int k = 0; k < NR; ++k) raw[q][k] = q < m ? Bits<S>::load(out + (int64_t)NR * jj[q] + k) : 0;
      }
#pragma unroll
      for (int q = 0; q < kDeps; ++q) {
        if (q < m && ok) {
          const S a = val[e0 + q];
#pragma unroll
          for (int k = 0; k < NR; ++k) {
            S o = Bits<S>::value(raw[q][k]);
            if (raw[q][k] == (typename Bits<S>::U)(~(typename Bits<S>::U)0) &&
                !wait_value<S>(out + (int64_t)NR * jj[q] + k, err, limit, o)) {
              ok = false;
              break;
            }
            s.c[k] -= a * o;
          }
        }
      }
    }
    if (!ok) continue;
    const S dg = val[d];
#pragma unroll
    for (int k = 0; k < NR; ++k) Bits<S>::store(out + (int64_t)NR * i + k, s.c[k] / dg);
  }
}

// a fresh ticket counter for a sweep
__global__ void k_ticket_reset(int* __restrict__ ticket) { *ticket = 0; }

// ---------------------------------------------------------------- host side
struct Factor {
  int64_t n = 0, nnz = 0;
  int64_t *lptr = nullptr, *tptr = nullptr, *tsrc = nullptr;
  int32_t *lc = nullptr, *tc = nullptr;
  double *lv = nullptr, *tv = nullptr;
  float *lv32 = nullptr, *tv32 = nullptr;
  int32_t *frows = nullptr, *flev = nullptr, *fnl = nullptr;
  int32_t *brows = nullptr, *blev = nullptr, *bnl = nullptr;
  int max_levels = 0;
  int64_t max_chart_rows = 0;
  // global levels (when chosen): rows by level, host offsets per level
  int32_t *fgrows = nullptr, *bgrows = nullptr, *row_chart = nullptr;
  std::vector<int32_t> foff, boff;
  // sync-free ticket kernels (when chosen): rows in global level order are fgrows / bgrows
  bool tickets = false;
  int* ready = nullptr;  // per row: the epoch of the sweep that finished it
  int* tick = nullptr;   // [0] epoch, [1] ticket counter, [2] error (a wait ran out)
  int64_t spin_limit = 0;
  unsigned ticket_grid = 0;
};

// Few, wide levels run as one launch per level over all charts; many levels on a large chart
// run sync-free over the whole GPU (tickets); otherwise one CTA per chart walks its own levels.
constexpr int kGlobalMaxLevels = 64;
constexpr int64_t kGlobalMinRows = 32768;
constexpr int kTicketMinLevels = 256;
// iterations of a ~64 ns sleep before a dependency wait gives up (about a second)
constexpr int64_t kSpinLimit = int64_t(1) << 24;

int64_t spin_limit() {
  const char* e = std::getenv("RUV_SPIN_LIMIT");
  return e ? std::max<int64_t>(1, std::atoll(e)) : kSpinLimit;
}

// Pattern, transpose and both level tables of the IC(0) factor of `sys` (values not yet
// factored).  Buffers are workspace entries under `tag`.
Factor factor_pattern(Ctx& ctx, const DevSystem& sys, const std::string& tag, int* flags) {
  cudaStream_t s = ctx.stream;
  Workspace& ws = ctx.ws;
  const int64_t N = sys.n_rows, NC = sys.n_charts;
  const unsigned g = div_up(std::max<int64_t>(N, 1), kIcThreads);
  Factor F;
  F.n = N;
  int32_t* cnt = ws.get<int32_t>(tag + ".cnt", std::max<int64_t>(N, 1));
  F.lptr = ws.get<int64_t>(tag + ".lptr", N + 1);
  if (N > 0) {
    k_l_count<<<g, kIcThreads, 0, s>>>(N, sys.row_ptr, sys.cols, sys.vals, cnt, flags);
    count_launches(1);
  }
  exclusive_scan(cnt, F.lptr, N, ws, s, tag + ".scan");
  int64_t nnz = 0;
  RUV_CUDA(cudaMemcpyAsync(&nnz, F.lptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  F.nnz = nnz;
  F.lc = ws.get<int32_t>(tag + ".lc", std::max<int64_t>(nnz, 1));
  F.lv = ws.get<double>(tag + ".lv", std::max<int64_t>(nnz, 1));
  F.tc = ws.get<int32_t>(tag + ".tc", std::max<int64_t>(nnz, 1));
  F.tsrc = ws.get<int64_t>(tag + ".tsrc", std::max<int64_t>(nnz, 1));
  F.tv = ws.get<double>(tag + ".tv", std::max<int64_t>(nnz, 1));
  F.lv32 = ws.get<float>(tag + ".lv32", std::max<int64_t>(nnz, 1));
  F.tv32 = ws.get<float>(tag + ".tv32", std::max<int64_t>(nnz, 1));
  F.tptr = ws.get<int64_t>(tag + ".tptr", N + 1);
  if (N > 0) {
    k_l_fill<<<g, kIcThreads, 0, s>>>(N, sys.row_ptr, sys.cols, sys.vals, F.lptr, F.lc, F.lv, flags);
    RUV_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * N, s));
    k_t_count<<<g, kIcThreads, 0, s>>>(N, F.lptr, F.lc, cnt);
    count_launches(2);
  }
  exclusive_scan(cnt, F.tptr, N, ws, s, tag + ".tscan");
  if (N > 0) {
    RUV_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * N, s));
    k_t_scatter<<<g, kIcThreads, 0, s>>>(N, F.lptr, F.lc, F.tptr, cnt, F.tc, F.tsrc);
    k_t_sort<<<g, kIcThreads, 0, s>>>(N, F.tptr, F.tc, F.tsrc);
    count_launches(2);
  }
  int32_t* indeg = ws.get<int32_t>(tag + ".indeg", std::max<int64_t>(N, 1));
  F.frows = ws.get<int32_t>(tag + ".frows", std::max<int64_t>(N, 1));
  F.brows = ws.get<int32_t>(tag + ".brows", std::max<int64_t>(N, 1));
  F.flev = ws.get<int32_t>(tag + ".flev", N + NC + 1);
  F.blev = ws.get<int32_t>(tag + ".blev", N + NC + 1);
  F.fnl = ws.get<int32_t>(tag + ".fnl", std::max<int64_t>(NC, 1));
  F.bnl = ws.get<int32_t>(tag + ".bnl", std::max<int64_t>(NC, 1));
  if (NC > 0) {
    k_levels<<<(unsigned)NC, kIcThreads, 0, s>>>(sys.chart_row, F.lptr, F.tptr, F.tc, indeg, F.frows, F.flev, F.fnl, flags);
    k_levels<<<(unsigned)NC, kIcThreads, 0, s>>>(sys.chart_row, F.tptr, F.lptr, F.lc, indeg, F.brows, F.blev, F.bnl, flags);
    count_launches(2);
    std::vector<int32_t> fl(NC), bl(NC);
    RUV_CUDA(cudaMemcpyAsync(fl.data(), F.fnl, sizeof(int32_t) * NC, cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaMemcpyAsync(bl.data(), F.bnl, sizeof(int32_t) * NC, cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaStreamSynchronize(s));
    for (int64_t c = 0; c < NC; ++c) {
      F.max_levels = std::max(F.max_levels, std::max(fl[c], bl[c]));
      F.max_chart_rows = std::max(F.max_chart_rows, sys.h_chart_row[c + 1] - sys.h_chart_row[c]);
    }
  }
  RUV_LAUNCH_CHECK();
  const char* te = std::getenv("RUV_IC0_TICKETS");
  F.tickets = te ? te[0] == '1' : (F.max_levels > kTicketMinLevels && F.max_chart_rows >= kGlobalMinRows);
  if (F.tickets || (F.max_levels > 0 && F.max_levels <= kGlobalMaxLevels && F.max_chart_rows >= kGlobalMinRows)) {
    int32_t* row_level = ws.get<int32_t>(tag + ".rlev", N);
    int32_t* hist = ws.get<int32_t>(tag + ".hist", F.max_levels);
    F.row_chart = ws.get<int32_t>(tag + ".rchart", N);
    F.fgrows = ws.get<int32_t>(tag + ".fgrows", N);
    F.bgrows = ws.get<int32_t>(tag + ".bgrows", N);
    const int32_t* rows_of[2] = {F.frows, F.brows};
    const int32_t* lev_of[2] = {F.flev, F.blev};
    const int32_t* nl_of[2] = {F.fnl, F.bnl};
    int32_t* grows_of[2] = {F.fgrows, F.bgrows};
    std::vector<int32_t>* off_of[2] = {&F.foff, &F.boff};
    for (int k = 0; k < 2; ++k) {
      k_row_level<<<(unsigned)NC, kIcThreads, 0, s>>>(sys.chart_row, rows_of[k], lev_of[k], nl_of[k], row_level, F.row_chart);
      RUV_CUDA(cudaMemsetAsync(hist, 0, sizeof(int32_t) * F.max_levels, s));
      k_level_hist<<<g, kIcThreads, 0, s>>>(N, row_level, hist);
      std::vector<int32_t> h(F.max_levels);
      RUV_CUDA(cudaMemcpyAsync(h.data(), hist, sizeof(int32_t) * F.max_levels, cudaMemcpyDeviceToHost, s));
      RUV_CUDA(cudaStreamSynchronize(s));
      std::vector<int32_t>& off = *off_of[k];
      off.assign(F.max_levels + 1, 0);
      for (int l = 0; l < F.max_levels; ++l) off[l + 1] = off[l] + h[l];
      RUV_CUDA(cudaMemcpyAsync(hist, off.data(), sizeof(int32_t) * F.max_levels, cudaMemcpyHostToDevice, s));
      k_level_scatter<<<g, kIcThreads, 0, s>>>(N, row_level, hist, grows_of[k]);
      RUV_CUDA(cudaStreamSynchronize(s));  // `off` is the host copy the cursor came from
      count_launches(3);
    }
    RUV_LAUNCH_CHECK();
  }
  if (F.tickets && N > 0) {
    F.ready = ws.get<int>(tag + ".ready", N);
    F.tick = ws.get<int>(tag + ".tick", 4);
    RUV_CUDA(cudaMemsetAsync(F.ready, 0, sizeof(int) * N, s));
    RUV_CUDA(cudaMemsetAsync(F.tick, 0, sizeof(int) * 4, s));
    F.spin_limit = spin_limit();
    // enough warps for a few levels in flight (the widest level's rows, 4 times over), at
    // least one CTA per SM, at most 8
    int32_t widest = 0;
    for (size_t l = 0; l + 1 < F.foff.size(); ++l) widest = std::max(widest, F.foff[l + 1] - F.foff[l]);
    for (size_t l = 0; l + 1 < F.boff.size(); ++l) widest = std::max(widest, F.boff[l + 1] - F.boff[l]);
    const int64_t want = div_up(4 * (int64_t)widest, kIcThreads);
    F.ticket_grid = (unsigned)std::min<int64_t>(8 * (int64_t)ctx.sm_count, std::max<int64_t>(ctx.sm_count, want));
  } else {
    F.tickets = false;
  }
  return F;
}

// Throws RUV_ERR_TIMEOUT when a ticket kernel's dependency wait ran out.
void check_ticket_error(Ctx& ctx, const Factor& F) {
  if (!F.tickets) return;
  int h = 0;
  RUV_CUDA(cudaMemcpyAsync(&h, F.tick + 2, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  RUV_CUDA(cudaStreamSynchronize(ctx.stream));
  if (h) {
    RUV_CUDA(cudaMemsetAsync(F.tick + 2, 0, sizeof(int), ctx.stream));
    throw Error{RUV_ERR_TIMEOUT, "IC(0): a dependency wait of the sync-free sweep ran out (RUV_SPIN_LIMIT)"};
  }
}

void factor_values(Ctx& ctx, const DevSystem& sys, Factor& F, int* flags) {
  cudaStream_t s = ctx.stream;
  if (F.tickets) {
    k_ticket_begin<<<1, 1, 0, s>>>(F.tick, F.tick + 1);
    k_factor_ticket<<<F.ticket_grid, kIcThreads, 0, s>>>(F.fgrows, F.n, F.lptr, F.lc, F.lv, F.ready, F.tick, F.tick + 1,
                                                           F.tick + 2, F.spin_limit, flags);
    count_launches(2);
    RUV_LAUNCH_CHECK();
    check_ticket_error(ctx, F);
  } else if (sys.n_charts > 0) {
    k_factor<<<(unsigned)sys.n_charts, kIcThreads, 0, s>>>(sys.chart_row, F.frows, F.flev, F.fnl, F.lptr, F.lc, F.lv, flags);
    count_launches(1);
  }
  if (F.nnz > 0) {
    k_t_values<<<div_up(F.nnz, 256), 256, 0, s>>>(F.nnz, F.tsrc, F.lv, F.tv, F.tv32, F.lv32);
    count_launches(1);
  }
  RUV_LAUNCH_CHECK();
}

void check_flags(Ctx& ctx, const int* flags) {
  int h = 0;
  RUV_CUDA(cudaMemcpyAsync(&h, flags, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  RUV_CUDA(cudaStreamSynchronize(ctx.stream));
  if (h & 1) throw Error{RUV_ERR_BREAKDOWN, "IC(0): a zero or missing diagonal entry"};
  if (h & 2) throw Error{RUV_ERR_BAD_INPUT, "IC(0): repeated column index in a row"};
  if (h & 4) throw Error{RUV_ERR_INTERNAL, "IC(0): dependency levels do not cover every row"};
  if (h & 8) throw Error{RUV_ERR_BREAKDOWN, "IC(0): a pivot below 1e-300"};
}

class Ic0Precond final : public SepPrecond {
 public:
  Ic0Precond(Ctx& ctx, const DevSystem& sys, bool colored) : n_(sys.n_rows), nc_(sys.n_charts), nrhs_(sys.nrhs) {
    cudaStream_t s = ctx.stream;
    Workspace& ws = ctx.ws;
    chart_row_ = sys.chart_row;
    int* flags = ws.get<int>("ic0.flags", 1);
    RUV_CUDA(cudaMemsetAsync(flags, 0, sizeof(int), s));
    DevSystem a = sys;
    if (colored) {
      // colouring on the original matrix's forward levels, permutation on the host
      Factor P0 = factor_pattern(ctx, sys, "ic0c", flags);
      int32_t* colour = ws.get<int32_t>("ic0c.colour", std::max<int64_t>(n_, 1));
      if (nc_ > 0) {
        k_colour<<<(unsigned)nc_, kIcThreads, 0, s>>>(sys.chart_row, P0.frows, P0.flev, P0.fnl, P0.lptr, P0.lc, colour);
        count_launches(1);
      }
      std::vector<int32_t> hc(n_), to_orig(n_), to_perm(n_);
      if (n_ > 0) RUV_CUDA(cudaMemcpyAsync(hc.data(), colour, sizeof(int32_t) * n_, cudaMemcpyDeviceToHost, s));
      RUV_CUDA(cudaStreamSynchronize(s));
      check_flags(ctx, flags);
      n_colours_ = 0;
      for (int64_t c = 0; c < nc_; ++c) {  // color_permutation per chart (precond.rs:77-101)
        const int64_t r0 = sys.h_chart_row[c], r1 = sys.h_chart_row[c + 1];
        int32_t m = 0;
        for (int64_t i = r0; i < r1; ++i) m = std::max(m, hc[i] + 1);
        n_colours_ = std::max(n_colours_, (int)m);
        std::vector<int64_t> start(m + 1, 0);
        for (int64_t i = r0; i < r1; ++i) start[hc[i] + 1] += 1;
        for (int32_t k = 1; k <= m; ++k) start[k] += start[k - 1];
        for (int64_t i = r0; i < r1; ++i) {
          const int64_t pos = r0 + start[hc[i]]++;
          to_perm[i] = (int32_t)pos;
          to_orig[pos] = (int32_t)i;
        }
      }
      to_orig_ = ws.get<int32_t>("ic0c.to_orig", std::max<int64_t>(n_, 1));
      int32_t* d_to_perm = ws.get<int32_t>("ic0c.to_perm", std::max<int64_t>(n_, 1));
      if (n_ > 0) {
        RUV_CUDA(cudaMemcpyAsync(to_orig_, to_orig.data(), sizeof(int32_t) * n_, cudaMemcpyHostToDevice, s));
        RUV_CUDA(cudaMemcpyAsync(d_to_perm, to_perm.data(), sizeof(int32_t) * n_, cudaMemcpyHostToDevice, s));
      }
      int32_t* cnt = ws.get<int32_t>("ic0c.pcnt", std::max<int64_t>(n_, 1));
      int64_t* prp64 = ws.get<int64_t>("ic0c.prp64", n_ + 1);
      int32_t* prp = ws.get<int32_t>("ic0c.prp", n_ + 1);
      int32_t* pc = ws.get<int32_t>("ic0c.pc", std::max<int64_t>(sys.nnz, 1));
      double* pv = ws.get<double>("ic0c.pv", std::max<int64_t>(sys.nnz, 1));
      const unsigned g = div_up(std::max<int64_t>(n_, 1), kIcThreads);
      if (n_ > 0) {
        k_perm_count<<<g, kIcThreads, 0, s>>>(n_, sys.row_ptr, to_orig_, cnt);
        count_launches(1);
      }
      exclusive_scan(cnt, prp64, n_, ws, s, "ic0c.pscan");
      std::vector<int64_t> h64(n_ + 1);
      RUV_CUDA(cudaMemcpyAsync(h64.data(), prp64, sizeof(int64_t) * (n_ + 1), cudaMemcpyDeviceToHost, s));
      RUV_CUDA(cudaStreamSynchronize(s));
      std::vector<int32_t> h32(h64.begin(), h64.end());
      RUV_CUDA(cudaMemcpyAsync(prp, h32.data(), sizeof(int32_t) * (n_ + 1), cudaMemcpyHostToDevice, s));
      if (n_ > 0) {
        k_perm_fill<<<g, kIcThreads, 0, s>>>(n_, sys.row_ptr, sys.cols, sys.vals, to_orig_, d_to_perm, prp, pc, pv);
        count_launches(1);
      }
      RUV_CUDA(cudaStreamSynchronize(s));  // the host tables above go out of scope
      a.row_ptr = prp;
      a.cols = pc;
      a.vals = pv;
      rp_ = ws.get<double>("ic0c.rp", std::max<int64_t>(nrhs_ * n_, 1));
      zp_ = ws.get<double>("ic0c.zp", std::max<int64_t>(nrhs_ * n_, 1));
    }
    F_ = factor_pattern(ctx, a, "ic0", flags);
    factor_values(ctx, a, F_, flags);
    check_flags(ctx, flags);
  }

  bool native_fp64() const override { return true; }
  bool flexible() const override { return false; }
  void bind(Ctx& ctx, void* r, void* z, bool fp64) override {
    r_ = r;
    z_ = z;
    fp64_ = fp64;
    y_ = ctx.ws.get<double>("ic0.y", std::max<int64_t>(nrhs_ * n_, 1));
  }
  int apply(Ctx& ctx, const int32_t* done) override {
    if (fp64_) return nrhs_ == 2 ? run<double, 2>(ctx, done) : run<double, 1>(ctx, done);
    return nrhs_ == 2 ? run<float, 2>(ctx, done) : run<float, 1>(ctx, done);
  }
  const int* error_flag() const override { return F_.tickets ? F_.tick + 2 : nullptr; }
  int levels() const { return F_.max_levels; }
  int colours() const { return n_colours_; }
  const Factor& factor() const { return F_; }
  const int32_t* to_orig() const { return to_orig_; }

 private:
  template <class S, int NR>
  int run(Ctx& ctx, const int32_t* done) {
    cudaStream_t s = ctx.stream;
    const bool f64 = std::is_same<S, double>::value;
    const S* lv = f64 ? reinterpret_cast<const S*>(F_.lv) : reinterpret_cast<const S*>(F_.lv32);
    const S* tv = f64 ? reinterpret_cast<const S*>(F_.tv) : reinterpret_cast<const S*>(F_.tv32);
    S* r = static_cast<S*>(r_);
    S* z = static_cast<S*>(z_);
    S* y = reinterpret_cast<S*>(y_);
    int launches = 0;
    const unsigned g = div_up(std::max<int64_t>(n_, 1), 256);
    S* rin = r;
    S* zout = z;
    if (to_orig_) {
      rin = reinterpret_cast<S*>(rp_);
      zout = reinterpret_cast<S*>(zp_);
      k_permute<S, NR, true><<<g, 256, 0, s>>>(n_, to_orig_, r, rin);
      ++launches;
    }
    if (F_.tickets) {
      const size_t bytes = sizeof(S) * NR * (size_t)n_;
      RUV_CUDA(cudaMemsetAsync(y, 0xff, bytes, s));  // the fill every output starts as (see k_sweep_ticket)
      k_ticket_reset<<<1, 1, 0, s>>>(F_.tick + 1);
      k_sweep_ticket<S, NR><<<F_.ticket_grid, kIcThreads, 0, s>>>(F_.fgrows, n_, F_.row_chart, done, F_.lptr, F_.lc, lv,
                                                                  rin, y, F_.tick + 1, F_.tick + 2, F_.spin_limit);
      RUV_CUDA(cudaMemsetAsync(zout, 0xff, bytes, s));
      k_ticket_reset<<<1, 1, 0, s>>>(F_.tick + 1);
      k_sweep_ticket<S, NR><<<F_.ticket_grid, kIcThreads, 0, s>>>(F_.bgrows, n_, F_.row_chart, done, F_.tptr, F_.tc, tv,
                                                                  y, zout, F_.tick + 1, F_.tick + 2, F_.spin_limit);
      launches += 4;
    } else if (F_.fgrows) {
      for (int l = 0; l + 1 < (int)F_.foff.size(); ++l) {
        const int32_t cnt = F_.foff[l + 1] - F_.foff[l];
        if (cnt == 0) continue;
        k_level_rows<S, NR><<<div_up(cnt, 256), 256, 0, s>>>(F_.fgrows + F_.foff[l], cnt, F_.row_chart, done, F_.lptr, F_.lc,
                                                             lv, rin, y);
        ++launches;
      }
      for (int l = 0; l + 1 < (int)F_.boff.size(); ++l) {
        const int32_t cnt = F_.boff[l + 1] - F_.boff[l];
        if (cnt == 0) continue;
        k_level_rows<S, NR><<<div_up(cnt, 256), 256, 0, s>>>(F_.bgrows + F_.boff[l], cnt, F_.row_chart, done, F_.tptr, F_.tc,
                                                             tv, y, zout);
        ++launches;
      }
    } else if (F_.max_chart_rows >= 65536) {  // a large chart: more rows per round of its CTA
      k_sweep<S, NR, 1024><<<(unsigned)nc_, 1024, 0, s>>>(chart_row_, done, F_.frows, F_.flev, F_.fnl, F_.lptr, F_.lc, lv,
                                                            rin, y);
      k_sweep<S, NR, 1024><<<(unsigned)nc_, 1024, 0, s>>>(chart_row_, done, F_.brows, F_.blev, F_.bnl, F_.tptr, F_.tc, tv,
                                                            y, zout);
      launches += 2;
    } else {
      k_sweep<S, NR, kIcThreads><<<(unsigned)nc_, kIcThreads, 0, s>>>(chart_row_, done, F_.frows, F_.flev, F_.fnl, F_.lptr,
                                                                      F_.lc, lv, rin, y);
      k_sweep<S, NR, kIcThreads><<<(unsigned)nc_, kIcThreads, 0, s>>>(chart_row_, done, F_.brows, F_.blev, F_.bnl, F_.tptr,
                                                                      F_.tc, tv, y, zout);
      launches += 2;
    }
    if (to_orig_) {
      k_permute<S, NR, false><<<g, 256, 0, s>>>(n_, to_orig_, zout, z);
      ++launches;
    }
    return launches;
  }

  int64_t n_, nc_;
  int nrhs_;
  const int64_t* chart_row_ = nullptr;
  Factor F_;
  int32_t* to_orig_ = nullptr;
  double *rp_ = nullptr, *zp_ = nullptr, *y_ = nullptr;
  void *r_ = nullptr, *z_ = nullptr;
  bool fp64_ = true;
  int n_colours_ = 0;
};

}  // namespace

std::unique_ptr<SepPrecond> make_ic0(Ctx& ctx, const DevSystem& sys, bool colored) {
  return std::unique_ptr<SepPrecond>(new Ic0Precond(ctx, sys, colored));
}

// Factor + one application z = (L L^T)^-1 r on a single system in FP64 (the reference's
// apply_ic0_for_test, gpu/src/solver.rs:205-270).  Also returns the level counts.
void ic0_apply_once(Ctx& ctx, const DevSystem& sys, const double* d_r, double* d_z, int* fwd_levels) {
  Ic0Precond P(ctx, sys, false);
  P.bind(ctx, const_cast<double*>(d_r), d_z, true);
  count_launches(P.apply(ctx, nullptr));
  RUV_LAUNCH_CHECK();
  RUV_CUDA(cudaStreamSynchronize(ctx.stream));
  check_ticket_error(ctx, P.factor());
  if (fwd_levels) *fwd_levels = P.levels();
}

// The factor of a one-chart system copied to the host (rows of L, diagonal last), with the
// colour permutation (position -> original row; identity without colouring) and the level
// and colour counts.
void ic0_export(Ctx& ctx, const DevSystem& sys, bool colored, std::vector<int64_t>& ptr, std::vector<int32_t>& cols,
                std::vector<double>& vals, std::vector<int32_t>& to_orig, int& levels, int& colours) {
  Ic0Precond P(ctx, sys, colored);
  const Factor& F = P.factor();
  cudaStream_t s = ctx.stream;
  ptr.resize(F.n + 1);
  cols.resize(F.nnz);
  vals.resize(F.nnz);
  to_orig.resize(F.n);
  RUV_CUDA(cudaMemcpyAsync(ptr.data(), F.lptr, sizeof(int64_t) * (F.n + 1), cudaMemcpyDeviceToHost, s));
  if (F.nnz > 0) {
    RUV_CUDA(cudaMemcpyAsync(cols.data(), F.lc, sizeof(int32_t) * F.nnz, cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaMemcpyAsync(vals.data(), F.lv, sizeof(double) * F.nnz, cudaMemcpyDeviceToHost, s));
  }
  if (P.to_orig() && F.n > 0)
    RUV_CUDA(cudaMemcpyAsync(to_orig.data(), P.to_orig(), sizeof(int32_t) * F.n, cudaMemcpyDeviceToHost, s));
  else
    for (int64_t i = 0; i < F.n; ++i) to_orig[i] = (int32_t)i;
  RUV_CUDA(cudaStreamSynchronize(s));
  levels = P.levels();
  colours = P.colours();
}

}  // namespace ruv
