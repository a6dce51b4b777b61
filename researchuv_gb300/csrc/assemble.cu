// GPU assembly of the per-chart LSCM systems with the pins eliminated, and the damped
// driver update — unfold_chart's numeric core (unwrap/src/lscm.rs:252-274 edge_weights,
// :594-676 assembly, :686-719 driver), for every chart of a batch at once.
//
// Layout: vertices and triangles of all charts are packed chart after chart.  A row is a
// free vertex; rows are numbered by an exclusive scan of the free flags, so each chart's
// rows are contiguous and ascend with the chart-local vertex id, exactly like the
// reference's free_pos map (lscm.rs:582-592).
//
// Bit-exactness: every floating operation is an explicit round-to-nearest operation
// (__dadd_rn, __dmul_rn, and division and square root by div_rn / sqrt_rn, which give the
// bits of __ddiv_rn / __dsqrt_rn off the FP64 pipe; never contracted into FMAs) in the
// reference's evaluation order, and every sum runs in the reference's order (edge weight:
// triangle order; diagonal and right-hand side: ascending neighbour id), so the CSR
// pattern, values and right-hand side are bit-identical to the reference's
// Sparse::to_csr(2 nf) (sparse.rs:69-84) of the same chart.
#include <cstdlib>
#include <functional>

#include "fp64rn.cuh"
#include "system.cuh"

namespace ruv {
namespace {

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return div_rn(a, b); }  // = __ddiv_rn

struct P3 {
  double x, y, z;
};
__device__ __forceinline__ P3 ld3(const double* p, int64_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
__device__ __forceinline__ P3 psub(P3 a, P3 b) { return {dsub(a.x, b.x), dsub(a.y, b.y), dsub(a.z, b.z)}; }
__device__ __forceinline__ double pdot(P3 a, P3 b) { return dadd(dadd(dmul(a.x, b.x), dmul(a.y, b.y)), dmul(a.z, b.z)); }
__device__ __forceinline__ double plen(P3 a) { return sqrt_rn(pdot(a, a)); }  // = __dsqrt_rn
__device__ __forceinline__ P3 pcross(P3 a, P3 b) {
  return {dsub(dmul(a.y, b.z), dmul(a.z, b.y)), dsub(dmul(a.z, b.x), dmul(a.x, b.z)), dsub(dmul(a.x, b.y), dmul(a.y, b.x))};
}
__device__ __forceinline__ P3 pneg(P3 a) {  // sign flips (integer pipe)
  constexpr long long kSign = (long long)0x8000000000000000ull;
  return {__longlong_as_double(__double_as_longlong(a.x) ^ kSign), __longlong_as_double(__double_as_longlong(a.y) ^ kSign),
          __longlong_as_double(__double_as_longlong(a.z) ^ kSign)};
}
__device__ __forceinline__ bool is_nan_bits(long long b) {
  return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}
// x <= c for a positive constant c, on the integer pipe: non-negative doubles order as their
// bit patterns, negative ones (and -0) read as negative integers, NaN compares false
__device__ __forceinline__ bool le_pos(double x, double c) {
  const long long b = __double_as_longlong(x);
  return !is_nan_bits(b) && b <= __double_as_longlong(c);
}
// Rust f64::max(x, 0.0) on the integer pipe: NaN -> 0, positive -> x, zeros and negatives -> +0
__device__ __forceinline__ double max0(double x) {
  const long long b = __double_as_longlong(x);
  return (!is_nan_bits(b) && b > 0) ? x : 0.0;
}
// x < 0.0 and x != 0.0 on the integer pipe (-0 is not below zero; NaN is unequal to zero)
__device__ __forceinline__ bool lt0(double x) {
  const long long b = __double_as_longlong(x);
  return b < 0 && (b & 0x7fffffffffffffffll) != 0 && !is_nan_bits(b);
}
__device__ __forceinline__ double dneg(double x) {  // -x (sign flip on the integer pipe)
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ bool ne0(double x) { return (__double_as_longlong(x) & 0x7fffffffffffffffll) != 0; }
// Rust f64::max(x, c) for a positive constant c, on the integer pipe
__device__ __forceinline__ double max_pos(double x, double c) {
  const long long b = __double_as_longlong(x);
  return (!is_nan_bits(b) && b > __double_as_longlong(c)) ? x : c;
}
// (float)x, round to nearest-even, on the integer pipe (double-to-float conversions run on the
// FP64 pipe); zeros, results outside float's normal range, infinities and NaNs go to the
// hardware conversion
__device__ __forceinline__ float f32_rn(double x) {
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  const int ef = (int)((u >> 52) & 0x7ff) - 1023 + 127;
  if (ef <= 0 || ef >= 255) return __double2float_rn(x);
  uint32_t mf = (uint32_t)((u >> 29) & 0x7fffffu);
  const uint64_t rest = u & ((1ull << 29) - 1), half = 1ull << 28;
  if (rest > half || (rest == half && (mf & 1u))) mf += 1;  // a carry moves into the exponent
  const uint32_t fb = ((uint32_t)ef << 23) + mf;
  if ((fb >> 23) >= 255u) return __double2float_rn(x);
  return __uint_as_float(fb | ((uint32_t)(u >> 32) & 0x80000000u));
}
__device__ __forceinline__ double rs_max(double a, double b) {  // Rust f64::max
  if (a != a) return b;
  if (b != b) return a;
  return a > b ? a : b;
}

__device__ __forceinline__ int64_t find_chart(const int64_t* off, int64_t n_charts, int64_t i) {
  int64_t lo = 0, hi = n_charts;  // largest c with off[c] <= i
  while (hi - lo > 1) {
    int64_t mid = (lo + hi) >> 1;
    if (off[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// chart-local triangle indices -> packed vertex ids (validated)
__global__ void k_globalize(const int32_t* __restrict__ tris, const int64_t* __restrict__ tri_off,
                            const int64_t* __restrict__ vert_off, int64_t n_charts, int64_t t_begin,
                            int64_t t_end, int32_t* __restrict__ tri_g, int* __restrict__ bad) {
  int64_t t = t_begin + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= t_end) return;
  int64_t c = find_chart(tri_off, n_charts, t);
  int64_t v0 = vert_off[c], nv = vert_off[c + 1] - v0;
  int32_t a = tris[3 * t], b = tris[3 * t + 1], d = tris[3 * t + 2];
  if (a < 0 || b < 0 || d < 0 || a >= nv || b >= nv || d >= nv || a == b || b == d || a == d) {
    atomicExch(bad, 1);
    a = b = d = 0;
  }
  tri_g[3 * t] = (int32_t)(v0 + a);
  tri_g[3 * t + 1] = (int32_t)(v0 + b);
  tri_g[3 * t + 2] = (int32_t)(v0 + d);
}

// Clamped cotangent at each triangle corner m (angle at t[m], opposite edge t[m+1]-t[m+2]),
// lscm.rs:256-268; 0.0 where the reference skips the corner (degenerate guard).  Also the
// squared length of each corner's opposite edge (sq).
__global__ void k_corner_cot(const double* __restrict__ p3, const int32_t* __restrict__ tri_g, int64_t t_begin,
                             int64_t t_end, double* __restrict__ cot, double* __restrict__ sq) {
  int64_t t = t_begin + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= t_end) return;
  int32_t v[3] = {tri_g[3 * t], tri_g[3 * t + 1], tri_g[3 * t + 2]};
  P3 p[3] = {ld3(p3, v[0]), ld3(p3, v[1]), ld3(p3, v[2])};
  // edge vectors e_k = p[k+1] - p[k] and their lengths, each once: the corner vectors are
  // e1 - o = p[m+2] - p[m] = -e_{m+2} (IEEE subtraction is antisymmetric: only the sign of an
  // exact zero can differ, which no step below turns into a different nonzero value, and the
  // clamp maps both zeros to +0) and e0 - o = e_m; the squares make the lengths of both
  // corners at an edge the same bits
  P3 e[3];
  double len[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    e[k] = psub(p[(k + 1) % 3], p[k]);
    const double d2 = pdot(e[k], e[k]);
    len[k] = sqrt_rn(d2);  // = plen(e[k])
    // the squared length of the edge opposite corner (k + 2) % 3, for the rows pass: the same
    // bits as |p_nb - p_v|^2 from either endpoint (a negated difference squares the same)
    sq[3 * t + (k + 2) % 3] = d2;
  }
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const P3 a1 = pneg(e[(m + 2) % 3]);  // e1 - o
    const P3 a2 = e[m];                  // e0 - o
    const double la = len[(m + 2) % 3], lb = len[m];
    double c = 0.0;
    if (!(le_pos(la, kEpsDegenerate) || le_pos(lb, kEpsDegenerate))) {
      const double lab = dmul(la, lb);
      const double sn = ddiv(plen(pcross(a1, a2)), lab);
      if (!le_pos(sn, kEpsDegenerate)) c = max0(ddiv(ddiv(pdot(a1, a2), lab), sn));
    }
    cot[3 * t + m] = c;
  }
}

__global__ void k_free_flags(const uint8_t* __restrict__ pinned, int64_t n, uint8_t* __restrict__ fr) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) fr[i] = pinned[i] ? 0 : 1;
}

__global__ void k_chart_rows(const int64_t* __restrict__ vert_off, const int64_t* __restrict__ row_of,
                             int64_t n_charts, int64_t* __restrict__ chart_row) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c <= n_charts) chart_row[c] = row_of[vert_off[c]];
}

// Two incidence records per (triangle, corner) for free vertices: (neighbour, corner index
// of the cotangent opposite that edge).
__global__ void k_count_records(const int32_t* __restrict__ tri_g, const uint8_t* __restrict__ pinned,
                                int64_t n_tris, int32_t* __restrict__ deg) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tris) return;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int32_t v = tri_g[3 * t + m];
    if (!pinned[v]) atomicAdd(&deg[v], 2);
  }
}

__global__ void k_scatter_records(const int32_t* __restrict__ tri_g, const uint8_t* __restrict__ pinned,
                                  int64_t n_tris, const int64_t* __restrict__ rec_off, int32_t* __restrict__ cursor,
                                  int2* __restrict__ rec) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tris) return;
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    int32_t v = tri_g[3 * t + m];
    if (pinned[v]) continue;
    int64_t at = rec_off[v] + atomicAdd(&cursor[v], 2);
    rec[at] = make_int2(tri_g[3 * t + (m + 1) % 3], (int32_t)(3 * t + (m + 2) % 3));
    rec[at + 1] = make_int2(tri_g[3 * t + (m + 2) % 3], (int32_t)(3 * t + (m + 1) % 3));
  }
}

__device__ __forceinline__ bool rec_less(int2 a, int2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }

// Ascending bitonic sorting network over 16 keys held in registers (every index is a
// compile-time constant once unrolled).  A record (neighbour, corner) packs into one 64-bit
// key, both fields non-negative, so the key order is rec_less; keys are distinct (a corner
// appears once), so the result equals the insertion sort's.
__device__ __forceinline__ void sort16(unsigned long long (&k)[16]) {
#pragma unroll
  for (int size = 2; size <= 16; size <<= 1)
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1)
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int l = i ^ stride;
        if (l > i) {
          const unsigned long long a = k[i], b = k[l];
          const bool sw = (i & size) == 0 ? b < a : a < b;
          k[i] = sw ? b : a;
          k[l] = sw ? a : b;
        }
      }
}

// One row (free vertex v).  MODE 0: sort the bucket, form each kept edge's coefficient
// c = w / max(|p_nb - p_v|^2, EPS) once (stored at the neighbour's first record; -1 marks a
// dropped edge) and count entries; MODE 1: fill from the stored coefficients.
template <int MODE, bool MIXB>
__global__ void k_rows(int64_t n_verts, const uint8_t* __restrict__ pinned, const int64_t* __restrict__ row_of,
                       const int64_t* __restrict__ rec_off, int2* __restrict__ rec, const double* __restrict__ cot,
                       const double* __restrict__ sq,
                       const double* __restrict__ p3, const double* __restrict__ p2, const double* __restrict__ pin_uv,
                       double mix_b, int32_t* __restrict__ row_len, const int64_t* __restrict__ row_ptr,
                       int32_t* __restrict__ cols, double* __restrict__ vals, float* __restrict__ vals32,
                       double* __restrict__ diag_out, double* __restrict__ b, int32_t* __restrict__ row_vert,
                       double* __restrict__ coef, float* __restrict__ vals_lo, float2* __restrict__ rsum) {
  int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_verts || pinned[v]) return;
  const int64_t r0 = rec_off[v], r1 = rec_off[v + 1];
  if (MODE == 0) {  // sort by (neighbour, corner) — buckets hold ~2x valence records
    constexpr int kLocal = 48;  // sorted in thread-local memory, written back once
    const int64_t nrec = r1 - r0;
    if (nrec <= 16) {  // the common case (valence <= 8): a sorting network in registers
      unsigned long long key[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int2 q = i < nrec ? rec[r0 + i] : make_int2(-1, -1);
        key[i] = i < nrec ? ((unsigned long long)(uint32_t)q.x << 32) | (uint32_t)q.y : ~0ull;
      }
      sort16(key);
#pragma unroll
      for (int i = 0; i < 16; ++i)
        if (i < nrec) rec[r0 + i] = make_int2((int32_t)(key[i] >> 32), (int32_t)(uint32_t)key[i]);
    } else if (nrec <= kLocal) {
      int2 b[kLocal];
      for (int64_t i = 0; i < nrec; ++i) {
        const int2 key = rec[r0 + i];
        int64_t j = i - 1;
        while (j >= 0 && rec_less(key, b[j])) {
          b[j + 1] = b[j];
          --j;
        }
        b[j + 1] = key;
      }
      for (int64_t i = 0; i < nrec; ++i) rec[r0 + i] = b[i];
    } else {  // a high-valence vertex: in place
      for (int64_t i = r0 + 1; i < r1; ++i) {
        int2 key = rec[i];
        int64_t j = i - 1;
        while (j >= r0 && rec_less(key, rec[j])) {
          rec[j + 1] = rec[j];
          --j;
        }
        rec[j + 1] = key;
      }
    }
  }
  const int64_t row = row_of[v];
  // the coefficient of the neighbour group starting at record i (its end returned in j)
  auto group = [&](int64_t i, int64_t& j) -> double {
    const int32_t nb = rec[i].x;
    j = i;
    if (MODE == 1) {
      while (j < r1 && rec[j].x == nb) ++j;
      return coef[i];
    }
    // w = 0 + cot_1 + cot_2 + ... in record order; every cotangent is +0 or positive, so the
    // first addition returns cot_1 itself
    double w = cot[rec[j].y];
    for (++j; j < r1 && rec[j].x == nb; ++j) w = dadd(w, cot[rec[j].y]);
    double c = -1.0;
    if (!le_pos(w, kEpsDegenerate)) c = ddiv(w, max_pos(sq[rec[i].y], kEpsDegenerate));  // lscm.rs:606
    coef[i] = c;
    return c;
  };
  // pass A (MODE 0): diagonal (sum of c over kept edges, ascending neighbour) and entry
  // count.  Every kept c is > 0, so a row has a diagonal entry iff that sum is nonzero, and
  // MODE 1 takes both from the stored diagonal instead of walking the records again.
  double dg = 0.0;
  bool has_diag = false;
  if (MODE == 0) {
    int32_t n_off = 0;
    for (int64_t i = r0; i < r1;) {
      int32_t nb = rec[i].x;
      int64_t j;
      const double c = group(i, j);
      i = j;
      if (lt0(c)) continue;  // dropped: w <= EPS
      if (ne0(c)) {  // Sparse::add skips zeros (sparse.rs:47-52)
        dg = dadd(dg, c);
        has_diag = true;
        if (!pinned[nb]) ++n_off;
      }
    }
    row_len[row] = n_off + (has_diag ? 1 : 0);
    diag_out[row] = dg;
    return;
  }
  dg = diag_out[row];
  has_diag = ne0(dg);
  // pass B: entries in column order (diagonal between the lower and upper neighbours) and
  // the right-hand side (pinned neighbours eliminated; mix_b pull term, lscm.rs:630-638)
  int64_t at = row_ptr[row];
  bool diag_done = !has_diag;
  // one entry, in storage order; with vals_lo / rsum also the mixed solver's low FP32 halves
  // and the FP64 row sum as a double-float pair (the rounding split_f64 does, so the same bits)
  double rs = 0.0;
  auto put = [&](int32_t col, double val) {
    cols[at] = col;
    vals[at] = val;
    const float h = f32_rn(val);
    vals32[at] = h;
    if (vals_lo) {
      vals_lo[at] = f32_rn(dsub(val, (double)h));
      rs = dadd(rs, val);
    }
    ++at;
  };
  double bu = 0.0, bv = 0.0;
  // MIXB false (mix_b == 0, the default angle_mix = 1): every pull term mix_b * c * d is a
  // signed zero and b starts at +0, so adding it changes no bit of b (x + (+-0) = x for
  // x != 0, +0 + (+-0) = +0, and b never becomes -0); those FP64 operations and the p2
  // gathers are skipped.  A pinned neighbour's term reduces to c * pin_uv exactly.
  const double p2u = MIXB ? p2[2 * v] : 0.0, p2v = MIXB ? p2[2 * v + 1] : 0.0;
  for (int64_t i = r0; i < r1;) {
    int32_t nb = rec[i].x;
    int64_t j;
    const double c = group(i, j);
    i = j;
    if (lt0(c)) continue;
    // dv as the reference forms it: d = p2[hi] - p2[lo], negated for the higher endpoint
    double du = 0.0, dw = 0.0, mc = 0.0;
    if (MIXB) {
      if (v < nb) {
        du = dsub(p2[2 * nb], p2u);
        dw = dsub(p2[2 * nb + 1], p2v);
      } else {
        du = dneg(dsub(p2u, p2[2 * nb]));
        dw = dneg(dsub(p2v, p2[2 * nb + 1]));
      }
      mc = dmul(mix_b, c);
    }
    if (!pinned[nb]) {
      if (MIXB) {
        bu = dadd(bu, dmul(mc, du));
        bv = dadd(bv, dmul(mc, dw));
      }
      if (ne0(c)) {
        if (!diag_done && nb > v) {
          put((int32_t)row, dg);
          diag_done = true;
        }
        put((int32_t)row_of[nb], dneg(c));
      }
    } else if (MIXB) {
      bu = dadd(bu, dadd(dmul(mc, du), dmul(c, pin_uv[2 * nb])));
      bv = dadd(bv, dadd(dmul(mc, dw), dmul(c, pin_uv[2 * nb + 1])));
    } else {
      bu = dadd(bu, dmul(c, pin_uv[2 * nb]));
      bv = dadd(bv, dmul(c, pin_uv[2 * nb + 1]));
    }
  }
  if (!diag_done) put((int32_t)row, dg);
  if (rsum) {
    const float h = f32_rn(rs);
    rsum[row] = make_float2(h, f32_rn(dsub(rs, (double)h)));
  }
  diag_out[row] = dg;
  b[2 * row] = bu;
  b[2 * row + 1] = bv;
  row_vert[row] = (int32_t)v;
}

__global__ void k_i64_to_i32(const int64_t* __restrict__ a, int64_t n, int32_t* __restrict__ o) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = (int32_t)a[i];
}

// ---------------------------------------------------------------- driver (lscm.rs:570-719)
struct DriverState {
  double step, prev_err, err_accum;
  int32_t iters, active, broke;
};

__global__ void k_driver_init(const double* __restrict__ p2, int64_t n, double* __restrict__ uv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 2 * n) uv[i] = p2[i];
}

__global__ void k_driver_state_init(DriverState* st, int64_t n_charts) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n_charts) st[c] = DriverState{1.0, __longlong_as_double(0x7ff0000000000000ll), 1.0, 0, 1, 0};
}

__device__ __forceinline__ void new_uv_of(int64_t v, const uint8_t* pinned, const double* pin_uv, const int64_t* row_of,
                                          const double* x, double& u, double& w) {
  if (pinned[v]) {
    u = pin_uv[2 * v];
    w = pin_uv[2 * v + 1];
  } else {
    int64_t r = row_of[v];
    u = x[2 * r];
    w = x[2 * r + 1];
  }
}

// per vertex-tile partial sums of |new_uv - uv|^2 and |uv|^2 for active charts
__global__ void k_driver_partials(const int64_t* __restrict__ tile_beg, const int32_t* __restrict__ tile_chart,
                                  int64_t n_tiles, const DriverState* __restrict__ st, const uint8_t* __restrict__ pinned,
                                  const double* __restrict__ pin_uv, const int64_t* __restrict__ row_of,
                                  const double* __restrict__ x, const double* __restrict__ uv,
                                  double* __restrict__ part) {
  __shared__ double sh[64];
  int64_t t = blockIdx.x;
  int c = tile_chart[t];
  if (!st[c].active) return;
  double s[2] = {0.0, 0.0};
  for (int64_t v = tile_beg[2 * t] + threadIdx.x; v < tile_beg[2 * t + 1]; v += blockDim.x) {
    double nu, nw;
    new_uv_of(v, pinned, pin_uv, row_of, x, nu, nw);
    double du = nu - uv[2 * v], dw = nw - uv[2 * v + 1];
    s[0] += du * du + dw * dw;
    s[1] += uv[2 * v] * uv[2 * v] + uv[2 * v + 1] * uv[2 * v + 1];
  }
  block_sum<2>(s, sh);
  if (threadIdx.x == 0) {
    part[2 * t] = s[0];
    part[2 * t + 1] = s[1];
  }
}

__global__ void k_driver_decide(const int64_t* __restrict__ chart_tile, int64_t n_charts, DriverState* __restrict__ st,
                                const double* __restrict__ part, int it, int max_iter, int* __restrict__ n_active) {
  __shared__ double sh[64];
  int64_t c = blockIdx.x;
  if (!st[c].active) return;
  double s[2] = {0.0, 0.0};
  for (int64_t t = chart_tile[c] + threadIdx.x; t < chart_tile[c + 1]; t += blockDim.x) {
    s[0] += part[2 * t];
    s[1] += part[2 * t + 1];
  }
  block_sum<2>(s, sh);
  if (threadIdx.x != 0) return;
  DriverState d = st[c];
  d.iters = it + 1;
  double err = sqrt(s[0]) / rs_max(sqrt(s[1]), 1e-30);
  double applied = err * d.step;
  if (d.prev_err > 1e-30 && err > 2.0 * d.prev_err)
    d.step = rs_max(d.step * 0.5, 0.05);
  else if (it > 3)
    d.step = fmin(d.step * 1.2, 1.0);
  if (applied < 1e-8 || (d.prev_err > 1e-30 && it != 0 && applied / d.prev_err <= 0.01)) {
    d.active = 0;  // converged / stagnation: uv stays as is
    d.broke = 1;
  } else {
    d.prev_err = applied;
    d.err_accum += err;
    if (max_iter * 10 < it || it + 1 >= max_iter) d.active = 2;  // apply this update, then stop
  }
  st[c] = d;
  if (d.active != 1) atomicSub(n_active, 1);
}

__global__ void k_driver_apply(const int64_t* __restrict__ tile_beg, const int32_t* __restrict__ tile_chart,
                               int64_t n_tiles, DriverState* __restrict__ st, const uint8_t* __restrict__ pinned,
                               const double* __restrict__ pin_uv, const int64_t* __restrict__ row_of,
                               const double* __restrict__ x, double* __restrict__ uv) {
  int64_t t = blockIdx.x;
  int c = tile_chart[t];
  int a = st[c].active;
  if (a == 0) return;
  double step = st[c].step;
  for (int64_t v = tile_beg[2 * t] + threadIdx.x; v < tile_beg[2 * t + 1]; v += blockDim.x) {
    double nu, nw;
    new_uv_of(v, pinned, pin_uv, row_of, x, nu, nw);
    double du = dsub(nu, uv[2 * v]), dw = dsub(nw, uv[2 * v + 1]);
    uv[2 * v] = dadd(uv[2 * v], dmul(du, step));
    uv[2 * v + 1] = dadd(uv[2 * v + 1], dmul(dw, step));
  }
}

__global__ void k_driver_retire(DriverState* st, int64_t n_charts) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n_charts && st[c].active == 2) st[c].active = 0;
}

}  // namespace

void assemble_lscm(Ctx& ctx, DevBatch& bt, DevSystem& sys, double angle_mix) {
  cudaStream_t s = ctx.stream;
  Workspace& ws = ctx.ws;
  const int64_t NV = bt.n_verts, NT = bt.n_tris, NC = bt.n_charts;
  const int B = 256;
  if (NT * 6 >= (int64_t)INT32_MAX || NV >= (int64_t)INT32_MAX)
    throw Error{RUV_ERR_BAD_INPUT, "batch too large for 32-bit record indices"};
  int* bad = ws.get<int>("asm.bad", 1);
  RUV_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
  int32_t* tri_g = ws.get<int32_t>("asm.tri_g", 3 * NT);
  double* cot = ws.get<double>("asm.cot", 3 * NT);
  double* sq = ws.get<double>("asm.sq", 3 * NT);
  bt.tri_g = tri_g;
  bt.cot = cot;
  // part by part, as a split upload delivers them (one part [0, NT) otherwise): each part's
  // triangles and positions may still be being copied on the side stream until its event
  const int n_parts = std::min(std::max(bt.n_parts, 1), DevBatch::kMaxParts);
  for (int part = 0; part < n_parts; ++part) {
    const int64_t t0 = bt.n_parts > 0 ? std::min(std::max<int64_t>(bt.part_tri[part], 0), NT) : 0;
    const int64_t t1 = bt.n_parts > 0 ? std::min(std::max<int64_t>(bt.part_tri[part + 1], 0), NT) : NT;
    if (bt.part_ready[part]) {
      RUV_CUDA(cudaStreamWaitEvent(s, bt.part_ready[part], 0));
      bt.part_ready[part] = nullptr;
    }
    if (t1 <= t0) continue;
    k_globalize<<<div_up(t1 - t0, B), B, 0, s>>>(bt.tris, bt.tri_off, bt.vert_off, NC, t0, t1, tri_g, bad);
    count_launches(1);
    RUV_LAUNCH_CHECK();
    k_corner_cot<<<div_up(t1 - t0, B), B, 0, s>>>(bt.p3, tri_g, t0, t1, cot, sq);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  // free-row numbering (the first use of the pin flags)
  if (bt.pins_ready) {
    RUV_CUDA(cudaStreamWaitEvent(s, bt.pins_ready, 0));
    bt.pins_ready = nullptr;
  }
  uint8_t* fr = ws.get<uint8_t>("asm.free", NV);
  bt.row_of = ws.get<int64_t>("asm.row_of", NV + 1);
  if (NV > 0) {
    k_free_flags<<<div_up(NV, B), B, 0, s>>>(bt.pinned, NV, fr);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  exclusive_scan_u8(fr, bt.row_of, NV, ws, s, "asm.rows");
  sys.chart_row = ws.get<int64_t>("sys.chart_row", NC + 1);
  k_chart_rows<<<div_up(NC + 1, B), B, 0, s>>>(bt.vert_off, bt.row_of, NC, sys.chart_row);
  count_launches(1);
  RUV_LAUNCH_CHECK();
  // incidence buckets
  int32_t* deg = ws.get<int32_t>("asm.deg", NV);
  RUV_CUDA(cudaMemsetAsync(deg, 0, sizeof(int32_t) * (NV > 0 ? NV : 1), s));
  if (NT > 0) {
    k_count_records<<<div_up(NT, B), B, 0, s>>>(tri_g, bt.pinned, NT, deg);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  int64_t* rec_off = ws.get<int64_t>("asm.rec_off", NV + 1);
  exclusive_scan(deg, rec_off, NV, ws, s, "asm.rec");
  // host reads: totals and per-chart row offsets (one small sync)
  int64_t* hp = static_cast<int64_t*>(ctx.pinned.get(sizeof(int64_t) * (NC + 4)));
  RUV_CUDA(cudaMemcpyAsync(hp, bt.row_of + NV, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaMemcpyAsync(hp + 1, rec_off + NV, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaMemcpyAsync(hp + 2, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  const int64_t NR = hp[0], NREC = hp[1];
  int bad_flag = (int)(reinterpret_cast<int*>(hp + 2)[0]);
  if (bad_flag) throw Error{RUV_ERR_BAD_INPUT, "triangle index out of range or repeated within a triangle"};
  int32_t* cursor = ws.get<int32_t>("asm.cursor", NV);
  RUV_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (NV > 0 ? NV : 1), s));
  int2* rec = ws.get<int2>("asm.rec", NREC);
  double* coef = ws.get<double>("asm.coef", NREC);
  bt.rec_off = rec_off;
  bt.rec = rec;
  bt.coef = coef;
  if (NT > 0) {
    k_scatter_records<<<div_up(NT, B), B, 0, s>>>(tri_g, bt.pinned, NT, rec_off, cursor, rec);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  const double mix_b = 1.0 - angle_mix;
  int32_t* row_len = ws.get<int32_t>("asm.row_len", NR);
  sys.diag = ws.get<double>("sys.diag", NR);  // written by the counting pass, read by the fill
  if (NV > 0) {
    k_rows<0, false><<<div_up(NV, 128), 128, 0, s>>>(NV, bt.pinned, bt.row_of, rec_off, rec, cot, sq, bt.p3, bt.p2, bt.pin_uv, mix_b,
                                             row_len, nullptr, nullptr, nullptr, nullptr, sys.diag, nullptr, nullptr,
                                             coef, nullptr, nullptr);
    count_launches(1);
  }
  RUV_LAUNCH_CHECK();
  int64_t* rp64 = ws.get<int64_t>("asm.rp64", NR + 1);
  exclusive_scan(row_len, rp64, NR, ws, s, "asm.rp");
  RUV_CUDA(cudaMemcpyAsync(hp + 3, rp64 + NR, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  const int64_t NNZ = hp[3];
  if (NNZ >= (int64_t)INT32_MAX) throw Error{RUV_ERR_BAD_INPUT, "operator too large for 32-bit CSR offsets"};
  sys.n_charts = NC;
  sys.n_rows = NR;
  sys.nnz = NNZ;
  sys.nrhs = 2;
  sys.row_ptr = ws.get<int32_t>("sys.row_ptr", NR + 1);
  sys.cols = ws.get<int32_t>("sys.cols", NNZ);
  sys.vals = ws.get<double>("sys.vals", NNZ);
  sys.vals32 = ws.get<float>("sys.vals32", NNZ);
  sys.b = ws.get<double>("sys.b", 2 * NR);
  // the mixed solver's split, formed by the fill (RUV_SPLIT_IN_FILL=0: by the solver instead)
  const char* split_env = std::getenv("RUV_SPLIT_IN_FILL");
  const bool split_in_fill = !(split_env && split_env[0] == '0');
  sys.vals_lo = split_in_fill ? ws.get<float>("asm.vals_lo", NNZ) : nullptr;
  sys.rsum = split_in_fill ? ws.get<float2>("asm.rsum", NR) : nullptr;
  bt.row_vert = ws.get<int32_t>("sys.row_vert", NR);
  k_i64_to_i32<<<div_up(NR + 1, B), B, 0, s>>>(rp64, NR + 1, sys.row_ptr);
  count_launches(1);
  RUV_LAUNCH_CHECK();
  // the fill: the first use of the pin targets and frame positions
  if (bt.rest_ready) {
    RUV_CUDA(cudaStreamWaitEvent(s, bt.rest_ready, 0));
    bt.rest_ready = nullptr;
  }
  if (NV > 0) {
    if (mix_b != 0.0)
      k_rows<1, true><<<div_up(NV, 128), 128, 0, s>>>(NV, bt.pinned, bt.row_of, rec_off, rec, cot, sq, bt.p3, bt.p2,
                                                      bt.pin_uv, mix_b, nullptr, rp64, sys.cols, sys.vals, sys.vals32,
                                                      sys.diag, sys.b, bt.row_vert, coef, sys.vals_lo, sys.rsum);
    else
      k_rows<1, false><<<div_up(NV, 128), 128, 0, s>>>(NV, bt.pinned, bt.row_of, rec_off, rec, cot, sq, bt.p3, bt.p2,
                                                       bt.pin_uv, mix_b, nullptr, rp64, sys.cols, sys.vals, sys.vals32,
                                                       sys.diag, sys.b, bt.row_vert, coef, sys.vals_lo, sys.rsum);
    count_launches(1);
  }
  RUV_LAUNCH_CHECK();
  sys.h_chart_row.resize(NC + 1);
  RUV_CUDA(cudaMemcpyAsync(sys.h_chart_row.data(), sys.chart_row, sizeof(int64_t) * (NC + 1), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
}

// Tiles over a packed per-chart range (vertices or rows): no tile spans two charts.
static void build_tiles(const std::vector<int64_t>& off, int64_t tile, std::vector<int64_t>& beg, std::vector<int32_t>& chart,
                        std::vector<int64_t>& chart_tile) {
  int64_t nc = (int64_t)off.size() - 1;
  beg.clear();
  chart.clear();
  chart_tile.assign(nc + 1, 0);
  for (int64_t c = 0; c < nc; ++c) {
    chart_tile[c] = (int64_t)chart.size();
    for (int64_t a = off[c]; a < off[c + 1]; a += tile) {
      beg.push_back(a);
      chart.push_back((int32_t)c);
    }
  }
  chart_tile[nc] = (int64_t)chart.size();
  beg.push_back(off[nc]);
}

namespace {
// Per-iteration hook of the driver loop: run before the iteration's partials with the
// iteration index, the per-chart driver states and the active-chart counter (KeepMetric
// forms that iteration's solution there).
using DriverHook = std::function<void(int, DriverState*, int*)>;
}  // namespace

static void driver_loop_dev(Ctx& ctx, DevBatch& bt, const DevSystem& sys, const double* x, int max_iter, double* uv,
                            std::vector<int32_t>& iters, std::vector<double>& err_accum, const DriverHook* hook);

void driver_update(Ctx& ctx, DevBatch& bt, const DevSystem& sys, const double* x, int max_iter, double* uv,
                   std::vector<int32_t>& iters, std::vector<double>& err_accum) {
  driver_loop_dev(ctx, bt, sys, x, max_iter, uv, iters, err_accum, nullptr);
}

static void driver_loop_dev(Ctx& ctx, DevBatch& bt, const DevSystem& sys, const double* x, int max_iter, double* uv,
                            std::vector<int32_t>& iters, std::vector<double>& err_accum, const DriverHook* hook) {
  cudaStream_t s = ctx.stream;
  Workspace& ws = ctx.ws;
  const int64_t NC = bt.n_charts, NV = bt.n_verts;
  if (max_iter <= 0) max_iter = 100;
  // vertex tiles of <= 2048 that never span two charts: table of [begin, end) pairs
  std::vector<int64_t> beg, chart_tile;
  std::vector<int32_t> tchart;
  build_tiles(bt.h_vert_off, 2048, beg, tchart, chart_tile);
  const int64_t NTL = (int64_t)tchart.size();
  std::vector<int64_t> tab(2 * NTL);
  for (int64_t t = 0; t < NTL; ++t) {
    tab[2 * t] = beg[t];
    tab[2 * t + 1] = std::min(beg[t] + 2048, bt.h_vert_off[tchart[t] + 1]);
  }
  int64_t* d_tab = ws.get<int64_t>("drv.tab", 2 * NTL);
  int32_t* d_tchart = ws.get<int32_t>("drv.tchart", NTL);
  int64_t* d_ctile = ws.get<int64_t>("drv.ctile", NC + 1);
  DriverState* st = ws.get<DriverState>("drv.state", NC);
  double* part = ws.get<double>("drv.part", 2 * NTL);
  int* n_active = ws.get<int>("drv.nactive", 1);
  RUV_CUDA(cudaMemcpyAsync(d_tab, tab.data(), sizeof(int64_t) * 2 * NTL, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_tchart, tchart.data(), sizeof(int32_t) * NTL, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_ctile, chart_tile.data(), sizeof(int64_t) * (NC + 1), cudaMemcpyHostToDevice, s));
  int h_nc = (int)NC;
  RUV_CUDA(cudaMemcpyAsync(n_active, &h_nc, sizeof(int), cudaMemcpyHostToDevice, s));
  if (NV > 0) {
    k_driver_init<<<div_up(2 * NV, 256), 256, 0, s>>>(bt.p2, NV, uv);
    count_launches(1);
  }
  k_driver_state_init<<<div_up(NC, 256), 256, 0, s>>>(st, NC);
  count_launches(1);
  RUV_LAUNCH_CHECK();
  int* h_active = static_cast<int*>(ctx.pinned.get(sizeof(int)));
  for (int it = 0; it < max_iter; ++it) {
    if (hook) (*hook)(it, st, n_active);
    if (NTL > 0) {
      k_driver_partials<<<(unsigned)NTL, 256, 0, s>>>(d_tab, d_tchart, NTL, st, bt.pinned, bt.pin_uv, bt.row_of, x, uv,
                                                      part);
      count_launches(1);
      RUV_LAUNCH_CHECK();
    }
    k_driver_decide<<<(unsigned)NC, 128, 0, s>>>(d_ctile, NC, st, part, it, max_iter, n_active);
    count_launches(1);
    RUV_LAUNCH_CHECK();
    if (NTL > 0) {
      k_driver_apply<<<(unsigned)NTL, 256, 0, s>>>(d_tab, d_tchart, NTL, st, bt.pinned, bt.pin_uv, bt.row_of, x, uv);
      count_launches(1);
      RUV_LAUNCH_CHECK();
    }
    k_driver_retire<<<div_up(NC, 256), 256, 0, s>>>(st, NC);
    count_launches(1);
    RUV_LAUNCH_CHECK();
    RUV_CUDA(cudaMemcpyAsync(h_active, n_active, sizeof(int), cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaStreamSynchronize(s));
    if (*h_active <= 0) break;
  }
  std::vector<DriverState> hs(NC);
  RUV_CUDA(cudaMemcpyAsync(hs.data(), st, sizeof(DriverState) * NC, cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  iters.resize(NC);
  err_accum.resize(NC);
  for (int64_t c = 0; c < NC; ++c) {
    iters[c] = hs[c].iters;
    err_accum[c] = hs[c].err_accum;
  }
}

namespace {
// ---------------------------------------------------------------- KeepMetric (lscm.rs:544-568, :642-676)
// The slack row of the system becomes the area row: with K the conformal free block, u the
// slack column (flip * normalised vertex area weight, both rows of a free vertex), g(uv) the
// area gradient and a(uv) the signed UV area,
//     [ K   u          ] [x  ]   [ b          ]
//     [ g^T a - target ] [aux] = [ 2 target   ].
// Only g and a change between driver iterations, so the SPD block is solved once for the two
// right-hand sides (y_b = K^-1 b, y_u = K^-1 u, the batched PCG) and every iteration is the
// Schur complement aux = (2 target - g.y_b) / ((a - target) - g.y_u), x = y_b - aux y_u.  The
// reference factors the bordered matrix every iteration (lscm.rs:672-680); a singular one
// ends its loop, which here is a zero area row (every free gradient component and a - target
// exactly zero) or a non-finite aux.

// Vertices (triangles) per KeepMetric tile, one per thread of a 256-thread CTA: the gradient
// is a few dozen FP64 operations per vertex, so a large chart wants many CTAs in flight.
constexpr int64_t kKmTile = 256;

// 3-D area per triangle (segment.rs:61-70)
__global__ void k_km_face_area(const double* __restrict__ p3, const int32_t* __restrict__ tri_g, int64_t nt,
                               double* __restrict__ A) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const P3 p0 = ld3(p3, tri_g[3 * t]), p1 = ld3(p3, tri_g[3 * t + 1]), p2 = ld3(p3, tri_g[3 * t + 2]);
  A[t] = dmul(0.5, plen(pcross(psub(p1, p0), psub(p2, p0))));
}

// Each triangle at a free vertex once, in the vertex's sorted record order: the record
// (t[m+1], corner m+2) of the pair that triangle t's corner m contributes.  Calls f(t, m).
template <class F>
__device__ __forceinline__ void km_vertex_tris(int64_t v, const int64_t* rec_off, const int2* rec,
                                               const int32_t* tri_g, F&& f) {
  for (int64_t r = rec_off[v]; r < rec_off[v + 1]; ++r) {
    const int2 q = rec[r];
    const int64_t t = q.y / 3;
    const int j = q.y - 3 * (int)t;
    if (q.x == tri_g[3 * t + (j + 2) % 3]) f(t, (j + 1) % 3);
  }
}

// area weight of every free vertex (the areas of its triangles)
__global__ void k_km_area_w(int64_t nv, const uint8_t* __restrict__ pinned, const int64_t* __restrict__ rec_off,
                            const int2* __restrict__ rec, const int32_t* __restrict__ tri_g,
                            const double* __restrict__ A, double* __restrict__ aw) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double w = 0.0;
  if (!pinned[v]) km_vertex_tris(v, rec_off, rec, tri_g, [&](int64_t t, int) { w = dadd(w, A[t]); });
  aw[v] = w;
}

// the signed-area term of a triangle (lscm.rs:120-129) from per-vertex (u, v) pairs
__device__ __forceinline__ double km_area_term(const double* uv, int32_t a, int32_t b, int32_t c) {
  const double x0 = uv[2 * a], y0 = uv[2 * a + 1], x1 = uv[2 * b], y1 = uv[2 * b + 1], x2 = uv[2 * c],
               y2 = uv[2 * c + 1];
  return dsub(dmul(dsub(x1, x0), dsub(y2, y0)), dmul(dsub(x2, x0), dsub(y1, y0)));
}

// per triangle tile: the sum of 3 A_t (the total of the vertex area weights)
__global__ void k_km_setup_part(const int64_t* __restrict__ ttab, const double* __restrict__ A,
                                double* __restrict__ part) {
  __shared__ double sh[64];
  const int64_t tl = blockIdx.x;
  double acc[2] = {0.0, 0.0};
  for (int64_t t = ttab[2 * tl] + threadIdx.x; t < ttab[2 * tl + 1]; t += blockDim.x) acc[0] += 3.0 * A[t];
  block_sum<2>(acc, sh);
  if (threadIdx.x == 0) {
    part[2 * tl] = acc[0];
    part[2 * tl + 1] = acc[1];
  }
}

__global__ void k_km_setup_chart(const int64_t* __restrict__ chart_ttile, const double* __restrict__ part,
                                 double* __restrict__ wsum) {
  __shared__ double sh[64];
  const int64_t c = blockIdx.x;
  double acc[2] = {0.0, 0.0};
  for (int64_t t = chart_ttile[c] + threadIdx.x; t < chart_ttile[c + 1]; t += blockDim.x) {
    acc[0] += part[2 * t];
    acc[1] += part[2 * t + 1];
  }
  block_sum<2>(acc, sh);
  if (threadIdx.x == 0) {
    wsum[c] = rs_max(acc[0], 1e-30);
  }
}

// slack column: flip * area_w / wsum on both rows of every free vertex
__global__ void k_km_u(const int64_t* __restrict__ tab, const int32_t* __restrict__ tchart,
                       const uint8_t* __restrict__ pinned, const int64_t* __restrict__ row_of,
                       const double* __restrict__ aw, const double* __restrict__ wsum, const double* __restrict__ flip,
                       double* __restrict__ u) {
  const int64_t tl = blockIdx.x;
  const int c = tchart[tl];
  for (int64_t v = tab[2 * tl] + threadIdx.x; v < tab[2 * tl + 1]; v += blockDim.x) {
    if (pinned[v]) continue;
    const int64_t r = row_of[v];
    const double w = flip[c] * ddiv(aw[v], wsum[c]);
    u[2 * r] = w;
    u[2 * r + 1] = w;
  }
}

// per triangle tile of an active chart: the sum of the area terms of uv
__global__ void k_km_area(const int64_t* __restrict__ ttab, const int32_t* __restrict__ ttchart,
                          const DriverState* __restrict__ st, const int32_t* __restrict__ tri_g,
                          const double* __restrict__ uv, double* __restrict__ part) {
  __shared__ double sh[32];
  const int64_t tl = blockIdx.x;
  if (!st[ttchart[tl]].active) return;
  double acc[1] = {0.0};
  for (int64_t t = ttab[2 * tl] + threadIdx.x; t < ttab[2 * tl + 1]; t += blockDim.x)
    acc[0] += km_area_term(uv, tri_g[3 * t], tri_g[3 * t + 1], tri_g[3 * t + 2]);
  block_sum<1>(acc, sh);
  if (threadIdx.x == 0) part[tl] = acc[0];
}

// per vertex tile of an active chart: the area gradient of every free vertex (lscm.rs:133-155,
// its triangles in record order) dotted with y_b and y_u, and the count of its nonzero
// components
__global__ void k_km_grad(const int64_t* __restrict__ tab, const int32_t* __restrict__ tchart,
                          const DriverState* __restrict__ st, const uint8_t* __restrict__ pinned,
                          const int64_t* __restrict__ row_of, const int64_t* __restrict__ rec_off,
                          const int2* __restrict__ rec, const int32_t* __restrict__ tri_g, const double* __restrict__ uv,
                          const double* __restrict__ yb, const double* __restrict__ yu, double* __restrict__ part) {
  __shared__ double sh[96];
  const int64_t tl = blockIdx.x;
  if (!st[tchart[tl]].active) return;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int64_t v = tab[2 * tl] + threadIdx.x; v < tab[2 * tl + 1]; v += blockDim.x) {
    if (pinned[v]) continue;
    double gu = 0.0, gv = 0.0;
    km_vertex_tris(v, rec_off, rec, tri_g, [&](int64_t t, int m) {
      const int32_t a = tri_g[3 * t], b = tri_g[3 * t + 1], c = tri_g[3 * t + 2];
      const double x0 = uv[2 * a], y0 = uv[2 * a + 1], x1 = uv[2 * b], y1 = uv[2 * b + 1], x2 = uv[2 * c],
                   y2 = uv[2 * c + 1];
      const double sgd = dmul(0.5, dadd(dadd(dmul(x0, dsub(y2, y1)), dmul(x1, dsub(y0, y2))), dmul(x2, dsub(y1, y0))));
      const double h = sgd > 0.0 ? 0.5 : -0.5;
      if (m == 0) {
        gu = dadd(gu, dmul(dsub(y2, y1), h));
        gv = dadd(gv, dmul(dsub(x1, x2), h));
      } else if (m == 1) {
        gu = dadd(gu, dmul(dsub(y0, y2), h));
        gv = dadd(gv, dmul(dsub(x2, x0), h));
      } else {
        gu = dadd(gu, dmul(dsub(y1, y0), h));
        gv = dadd(gv, dmul(dsub(x0, x1), h));
      }
    });
    const int64_t r = row_of[v];
    acc[0] += gu * yb[2 * r] + gv * yb[2 * r + 1];
    acc[1] += gu * yu[2 * r] + gv * yu[2 * r + 1];
    acc[2] += (gu != 0.0 ? 1.0 : 0.0) + (gv != 0.0 ? 1.0 : 0.0);
  }
  block_sum<3>(acc, sh);
  if (threadIdx.x == 0) {
    part[3 * tl] = acc[0];
    part[3 * tl + 1] = acc[1];
    part[3 * tl + 2] = acc[2];
  }
}

// per chart: aux of this iteration; a singular bordered system ends the chart's loop
__global__ void k_km_aux(const int64_t* __restrict__ chart_ttile, const int64_t* __restrict__ chart_vtile,
                         DriverState* __restrict__ st, const double* __restrict__ apart, const double* __restrict__ gpart,
                         const double* __restrict__ target, int it, double* __restrict__ aux, int* __restrict__ n_active) {
  __shared__ double sh[128];
  const int64_t c = blockIdx.x;
  if (!st[c].active) return;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t t = chart_ttile[c] + threadIdx.x; t < chart_ttile[c + 1]; t += blockDim.x) acc[0] += apart[t];
  for (int64_t t = chart_vtile[c] + threadIdx.x; t < chart_vtile[c + 1]; t += blockDim.x) {
    acc[1] += gpart[3 * t];
    acc[2] += gpart[3 * t + 1];
    acc[3] += gpart[3 * t + 2];
  }
  block_sum<4>(acc, sh);
  if (threadIdx.x != 0) return;
  const double area = 0.5 * acc[0], diag = area - target[c];
  const double a = (2.0 * target[c] - acc[1]) / (diag - acc[2]);
  if ((acc[3] == 0.0 && diag == 0.0) || !isfinite(a)) {
    st[c].active = 0;  // the reference's LU fails: the loop ends before this iteration's update
    st[c].iters = it + 1;
    atomicSub(n_active, 1);
    return;
  }
  aux[c] = a;
}

// x = y_b - aux y_u on the rows of active charts
__global__ void k_km_x(const int64_t* __restrict__ tab, const int32_t* __restrict__ tchart,
                       const DriverState* __restrict__ st, const uint8_t* __restrict__ pinned,
                       const int64_t* __restrict__ row_of, const double* __restrict__ yb, const double* __restrict__ yu,
                       const double* __restrict__ aux, double* __restrict__ x) {
  const int64_t tl = blockIdx.x;
  const int c = tchart[tl];
  if (!st[c].active) return;
  const double a = aux[c];
  for (int64_t v = tab[2 * tl] + threadIdx.x; v < tab[2 * tl + 1]; v += blockDim.x) {
    if (pinned[v]) continue;
    const int64_t r = row_of[v];
    x[2 * r] = yb[2 * r] - a * yu[2 * r];
    x[2 * r + 1] = yb[2 * r + 1] - a * yu[2 * r + 1];
  }
}
}  // namespace

// The slack column u of the KeepMetric system (2 * n_rows, device) after assemble_lscm.
void keep_metric_rhs(Ctx& ctx, DevBatch& bt, DevSystem& sys, const double* d_flip, double* u) {
  cudaStream_t s = ctx.stream;
  Workspace& ws = ctx.ws;
  const int64_t NV = bt.n_verts, NT = bt.n_tris, NC = bt.n_charts;
  if (sys.n_rows > 0) RUV_CUDA(cudaMemsetAsync(u, 0, sizeof(double) * 2 * sys.n_rows, s));
  if (NC == 0 || NT == 0) return;
  double* A = ws.get<double>("km.A", NT);
  double* aw = ws.get<double>("km.aw", NV);
  k_km_face_area<<<div_up(NT, 256), 256, 0, s>>>(bt.p3, bt.tri_g, NT, A);
  k_km_area_w<<<div_up(NV, 256), 256, 0, s>>>(NV, bt.pinned, bt.rec_off, bt.rec, bt.tri_g, A, aw);
  count_launches(2);
  std::vector<int64_t> tbeg, tctile, vbeg, vctile;
  std::vector<int32_t> tchart, vchart;
  build_tiles(bt.h_tri_off, kKmTile, tbeg, tchart, tctile);
  build_tiles(bt.h_vert_off, kKmTile, vbeg, vchart, vctile);
  const int64_t NTT = (int64_t)tchart.size(), NTL = (int64_t)vchart.size();
  std::vector<int64_t> ttab(2 * NTT), vtab(2 * NTL);
  for (int64_t t = 0; t < NTT; ++t) {
    ttab[2 * t] = tbeg[t];
    ttab[2 * t + 1] = std::min(tbeg[t] + kKmTile, bt.h_tri_off[tchart[t] + 1]);
  }
  for (int64_t t = 0; t < NTL; ++t) {
    vtab[2 * t] = vbeg[t];
    vtab[2 * t + 1] = std::min(vbeg[t] + kKmTile, bt.h_vert_off[vchart[t] + 1]);
  }
  int64_t* d_ttab = ws.get<int64_t>("km.ttab", std::max<int64_t>(2 * NTT, 1));
  int64_t* d_tct = ws.get<int64_t>("km.tctile", NC + 1);
  int64_t* d_vtab = ws.get<int64_t>("km.vtab", std::max<int64_t>(2 * NTL, 1));
  int32_t* d_vch = ws.get<int32_t>("km.vchart", std::max<int64_t>(NTL, 1));
  RUV_CUDA(cudaMemcpyAsync(d_ttab, ttab.data(), sizeof(int64_t) * 2 * NTT, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_tct, tctile.data(), sizeof(int64_t) * (NC + 1), cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_vtab, vtab.data(), sizeof(int64_t) * 2 * NTL, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_vch, vchart.data(), sizeof(int32_t) * NTL, cudaMemcpyHostToDevice, s));
  double* part = ws.get<double>("km.spart", 2 * std::max<int64_t>(NTT, 1));
  double* wsum = ws.get<double>("km.wsum", NC);
  if (NTT > 0) k_km_setup_part<<<(unsigned)NTT, 256, 0, s>>>(d_ttab, A, part);
  k_km_setup_chart<<<(unsigned)NC, 128, 0, s>>>(d_tct, part, wsum);
  if (NTL > 0) k_km_u<<<(unsigned)NTL, 256, 0, s>>>(d_vtab, d_vch, bt.pinned, bt.row_of, aw, wsum, d_flip, u);
  count_launches(3);
  RUV_LAUNCH_CHECK();
  (void)sys;
}

// The KeepMetric driver: every iteration forms x = y_b - aux y_u from the current uv, then
// takes the damped driver step (the same kernels as the default path).
void driver_keep_metric(Ctx& ctx, DevBatch& bt, const DevSystem& sys, const double* yb, const double* yu,
                        const double* d_target, int max_iter, double* uv, std::vector<int32_t>& iters,
                        std::vector<double>& err_accum) {
  cudaStream_t s = ctx.stream;
  Workspace& ws = ctx.ws;
  const int64_t NC = bt.n_charts;
  std::vector<int64_t> tbeg, tctile, vbeg, vctile;
  std::vector<int32_t> tchart, vchart;
  build_tiles(bt.h_tri_off, kKmTile, tbeg, tchart, tctile);
  build_tiles(bt.h_vert_off, kKmTile, vbeg, vchart, vctile);
  const int64_t NTT = (int64_t)tchart.size(), NTL = (int64_t)vchart.size();
  std::vector<int64_t> ttab(2 * NTT), vtab(2 * NTL);
  for (int64_t t = 0; t < NTT; ++t) {
    ttab[2 * t] = tbeg[t];
    ttab[2 * t + 1] = std::min(tbeg[t] + kKmTile, bt.h_tri_off[tchart[t] + 1]);
  }
  for (int64_t t = 0; t < NTL; ++t) {
    vtab[2 * t] = vbeg[t];
    vtab[2 * t + 1] = std::min(vbeg[t] + kKmTile, bt.h_vert_off[vchart[t] + 1]);
  }
  int64_t* d_ttab = ws.get<int64_t>("kmd.ttab", std::max<int64_t>(2 * NTT, 1));
  int32_t* d_tch = ws.get<int32_t>("kmd.tchart", std::max<int64_t>(NTT, 1));
  int64_t* d_tct = ws.get<int64_t>("kmd.tctile", NC + 1);
  int64_t* d_vtab = ws.get<int64_t>("kmd.vtab", std::max<int64_t>(2 * NTL, 1));
  int32_t* d_vch = ws.get<int32_t>("kmd.vchart", std::max<int64_t>(NTL, 1));
  int64_t* d_vct = ws.get<int64_t>("kmd.vctile", NC + 1);
  RUV_CUDA(cudaMemcpyAsync(d_ttab, ttab.data(), sizeof(int64_t) * 2 * NTT, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_tch, tchart.data(), sizeof(int32_t) * NTT, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_tct, tctile.data(), sizeof(int64_t) * (NC + 1), cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_vtab, vtab.data(), sizeof(int64_t) * 2 * NTL, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_vch, vchart.data(), sizeof(int32_t) * NTL, cudaMemcpyHostToDevice, s));
  RUV_CUDA(cudaMemcpyAsync(d_vct, vctile.data(), sizeof(int64_t) * (NC + 1), cudaMemcpyHostToDevice, s));
  double* apart = ws.get<double>("kmd.apart", std::max<int64_t>(NTT, 1));
  double* gpart = ws.get<double>("kmd.gpart", 3 * std::max<int64_t>(NTL, 1));
  double* aux = ws.get<double>("kmd.aux", std::max<int64_t>(NC, 1));
  double* x = ws.get<double>("kmd.x", 2 * std::max<int64_t>(sys.n_rows, 1));
  DriverHook hook = [&](int it, DriverState* st, int* n_active) {
    if (NTT > 0) k_km_area<<<(unsigned)NTT, 256, 0, s>>>(d_ttab, d_tch, st, bt.tri_g, uv, apart);
    if (NTL > 0)
      k_km_grad<<<(unsigned)NTL, 256, 0, s>>>(d_vtab, d_vch, st, bt.pinned, bt.row_of, bt.rec_off, bt.rec, bt.tri_g, uv,
                                              yb, yu, gpart);
    k_km_aux<<<(unsigned)NC, 128, 0, s>>>(d_tct, d_vct, st, apart, gpart, d_target, it, aux, n_active);
    if (NTL > 0) k_km_x<<<(unsigned)NTL, 256, 0, s>>>(d_vtab, d_vch, st, bt.pinned, bt.row_of, yb, yu, aux, x);
    count_launches(4);
    RUV_LAUNCH_CHECK();
  };
  driver_loop_dev(ctx, bt, sys, x, max_iter, uv, iters, err_accum, &hook);
}

namespace {
// ---------------------------------------------------------------- self-test of div_rn / sqrt_rn
// Seeded inputs (splitmix64 of seed + i), compared bit for bit with the hardware operations.
// mode 0: quotients of random significands, exponents within +-60 of 1, random signs;
// 1: quotients of arbitrary bit patterns (every class: zeros, subnormals, infinities, NaNs,
//    quotients leaving the normal range); 2: quotients near a midpoint (a = b q rounded, moved
//    by -2..2 ulps); 3: square roots, exponents within +-60; 4: square roots of arbitrary bit
//    patterns; 5: square roots near perfect squares (s^2 exact for s < 2^26, moved by -2..2
//    ulps, scaled by 4^k).
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double bits_d(uint64_t u) { return __longlong_as_double((long long)u); }
__device__ __forceinline__ uint64_t d_bits(double d) { return (uint64_t)__double_as_longlong(d); }

__global__ void k_fp64_selftest(int mode, uint64_t seed, int64_t n, unsigned long long* __restrict__ bad,
                                double* __restrict__ first) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t r0 = splitmix64(seed + 3 * (uint64_t)i), r1 = splitmix64(seed + 3 * (uint64_t)i + 1),
                 r2 = splitmix64(seed + 3 * (uint64_t)i + 2);
  double a = 0.0, b = 0.0, got, want;
  if (mode <= 2) {
    if (mode == 0) {
      a = bits_d((r0 & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(1023 - 60 + (int)(r2 % 121)) << 52));
      b = bits_d((r1 & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(1023 - 60 + (int)((r2 >> 8) % 121)) << 52));
    } else if (mode == 1) {
      a = bits_d(r0);
      b = bits_d(r1);
    } else {
      b = bits_d((r1 & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(1023 - 30 + (int)(r2 % 61)) << 52));
      const double q = bits_d((r0 & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(1023 - 30 + (int)((r2 >> 8) % 61)) << 52));
      a = bits_d(d_bits(__dmul_rn(b, q)) + (uint64_t)((int)((r2 >> 16) % 5) - 2));
    }
    got = div_rn(a, b);
    want = __ddiv_rn(a, b);
  } else {
    if (mode == 3) {
      a = bits_d((r0 & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(1023 - 60 + (int)(r2 % 121)) << 52));
    } else if (mode == 4) {
      a = bits_d(r0);
    } else {
      const double sq = (double)(r0 & ((1ull << 26) - 1)) + 1.0;
      const double x = __dmul_rn(sq, sq);  // exact
      const int k = (int)(r2 % 61) - 30;
      a = bits_d(d_bits(x) + (uint64_t)((int)((r2 >> 8) % 5) - 2)) * exp2((double)(2 * k));
    }
    got = sqrt_rn(a);
    want = __dsqrt_rn(a);
  }
  if (d_bits(got) != d_bits(want)) {
    if (atomicAdd(bad, 1ull) == 0ull) {
      first[0] = a;
      first[1] = b;
      first[2] = got;
      first[3] = want;
    }
  }
}

}  // namespace

int64_t fp64_selftest(Ctx& ctx, int mode, uint64_t seed, int64_t n, double* first4) {
  cudaStream_t s = ctx.stream;
  unsigned long long* bad = ctx.ws.get<unsigned long long>("selftest.bad", 1);
  double* first = ctx.ws.get<double>("selftest.first", 4);
  RUV_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s));
  RUV_CUDA(cudaMemsetAsync(first, 0, 4 * sizeof(double), s));
  if (n > 0) {
    k_fp64_selftest<<<div_up(n, 256), 256, 0, s>>>(mode, seed, n, bad, first);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  unsigned long long h = 0;
  RUV_CUDA(cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaMemcpyAsync(first4, first, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
  return (int64_t)h;
}

}  // namespace ruv
