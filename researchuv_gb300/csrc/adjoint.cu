// Differentiation of the batched LSCM unfold with respect to the 3-D vertex positions, and
// the distortion metrics of a UV layout (unwrap/src/metrics.rs:59-141).
//
// The differentiated map is the solve the reference runs (unwrap/src/lscm.rs:594-719) with
// the pins held at their targets: for every chart, A(p) uv = b(p), where A is the weighted
// Laplacian over free vertices with coefficients c_ij = w_ij / max(|p_j - p_i|^2, EPS),
// w_ij the sum of the clamped corner cotangents opposite edge ij, and b collects
// c_ij * pin_j over pinned neighbours.  For a loss with gradient g = dL/duv (free rows):
//   lam = A^-1 g                       (the same SPD operator and preconditioner)
//   dL/dc_ij = -(lam_i - lam_j) . (uv_i - uv_j)     (lam = 0 on pinned vertices)
//   dL/dw_ij = dL/dc_ij / max(d2, EPS);  dL/dd2 = -dL/dc_ij w_ij / d2^2 (when d2 > EPS)
//   dL/dcot  = dL/dw of the edge the corner faces (0 where the cotangent was clamped)
//   dcot / dp from cot = (a1 . a2) / |a1 x a2| at the corner.
// The assembly is recomputed in the backward pass (the reverse pass reads the recomputed
// cotangents, incidence records and edge coefficients, nothing stored by the forward solve).
// Position gradients are accumulated with FP64 atomics.
//
// The distortion loss sum_t area_t (s1/s2 - 1)^2 (area_t the 3-D area, s1 >= s2 the
// singular values of the UV Jacobian F = U P^-1 of metrics.rs:95-128, formed stably) is differentiated per
// triangle by forward-mode dual numbers (three seeds per pass, five passes for the 15
// coordinates of a triangle), FP64.  Triangles whose three vertices are all pinned are left
// out of the loss: their UVs are set by the pin rule, not by the solve, and the rule can
// place all three on one side of the border rectangle (the corner triangles of a grid chart),
// where s2 = 0 and the term is unbounded.
#include <cmath>

#include "system.cuh"

namespace ruv {
namespace {

constexpr int kAdjThreads = 256;

// ---------------------------------------------------------------- dual numbers
template <int N>
struct Dual {
  double v;
  double d[N];
};
template <int N>
__device__ __forceinline__ Dual<N> cst(double v) {
  Dual<N> r;
  r.v = v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = 0.0;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(double s, const Dual<N>& a) {
  Dual<N> r;
  r.v = s * a.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = s * a.d[k];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dsqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = sqrt(a.v);
  const double h = r.v > 0.0 ? 0.5 / r.v : 0.0;  // at 0: the one-sided slope is unbounded; taken as 0
#pragma unroll
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * h;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dmax(const Dual<N>& a, double c) {  // Rust f64::max(a, c), c finite
  return a.v > c ? a : cst<N>(c);
}

// The distortion term of one triangle (metrics.rs:95-128): 0.5 |n| (s1 / max(s2, 1e-30) - 1)^2,
// or a skip (degenerate normal or tangent-frame determinant; those triangles add nothing).
template <class T>
__device__ __forceinline__ bool tri_distortion(const T (&p)[9], const T (&u)[6], T& out) {
  const T e1x = p[3] - p[0], e1y = p[4] - p[1], e1z = p[5] - p[2];
  const T e2x = p[6] - p[0], e2y = p[7] - p[1], e2z = p[8] - p[2];
  const T nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
  const T ln = dsqrt(nx * nx + ny * ny + nz * nz);
  if (ln.v < 1e-30) return false;
  const T ux = nx / ln, uy = ny / ln, uz = nz / ln;
  const T l1 = dmax(dsqrt(e1x * e1x + e1y * e1y + e1z * e1z), 1e-30);
  const T t1x = e1x / l1, t1y = e1y / l1, t1z = e1z / l1;
  const T t2x = uy * t1z - uz * t1y, t2y = uz * t1x - ux * t1z, t2z = ux * t1y - uy * t1x;
  const T e1t1 = e1x * t1x + e1y * t1y + e1z * t1z;
  const T e2t1 = e2x * t1x + e2y * t1y + e2z * t1z;
  const T e1t2 = e1x * t2x + e1y * t2y + e1z * t2z;
  const T e2t2 = e2x * t2x + e2y * t2y + e2z * t2z;
  const T det = e1t1 * e2t2 - e2t1 * e1t2;
  if (fabs(det.v) < 1e-30) return false;
  const T i00 = e2t2 / det, i01 = -e2t1 / det, i10 = -e1t2 / det, i11 = e1t1 / det;
  const T d1u = u[2] - u[0], d1v = u[3] - u[1], d2u = u[4] - u[0], d2v = u[5] - u[1];
  const T f00 = d1u * i00 + d2u * i10, f01 = d1u * i01 + d2u * i11;
  const T f10 = d1v * i00 + d2v * i10, f11 = d1v * i01 + d2v * i11;
  // singular values of F: s1 = (|(f00 + f11, f10 - f01)| + |(f00 - f11, f10 + f01)|) / 2 and
  // s2 = |det F| / s1 -- the same values as svd2 (metrics.rs:59-70), formed without its
  // 0.5 tr - disc cancellation, which loses (s1/s2)^2 ulps on anisotropic triangles
  const T p0 = f00 + f11, p1 = f10 - f01, q0 = f00 - f11, q1 = f10 + f01;
  const T s1 = 0.5 * (dsqrt(p0 * p0 + p1 * p1) + dsqrt(q0 * q0 + q1 * q1));
  T dF = f00 * f11 - f01 * f10;
  if (dF.v < 0.0) dF = -dF;
  const T s2 = s1.v > 0.0 ? dF / s1 : cst<3>(0.0);
  const T r = s1 / dmax(s2, 1e-30) - cst<3>(1.0);
  out = 0.5 * (ln * (r * r));
  return true;
}

__device__ __forceinline__ int64_t chart_of(const int64_t* off, int64_t n, int64_t i) {
  int64_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (off[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// Loss per triangle (loss_t) and, with gradients wanted, d loss / d(p, uv) accumulated.
__global__ void __launch_bounds__(kAdjThreads) k_distortion(const int64_t* __restrict__ tri_off,
                                                            const int64_t* __restrict__ vert_off, int64_t n_charts,
                                                            int64_t n_tris, const int32_t* __restrict__ tris,
                                                            const uint8_t* __restrict__ pinned,
                                                            const double* __restrict__ p3, const double* __restrict__ uv,
                                                            double* __restrict__ loss_t, double* duv, double* dp3) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tris) return;
  const int64_t c = chart_of(tri_off, n_charts, t);
  const int64_t v0 = vert_off[c];
  int64_t v[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = v0 + tris[3 * t + k];
  if (pinned[v[0]] && pinned[v[1]] && pinned[v[2]]) {
    loss_t[t] = 0.0;
    return;
  }
  double pin[15];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int j = 0; j < 3; ++j) pin[3 * k + j] = p3[3 * v[k] + j];
    pin[9 + 2 * k] = uv[2 * v[k]];
    pin[10 + 2 * k] = uv[2 * v[k] + 1];
  }
  double val = 0.0;
  const bool grad = duv != nullptr || dp3 != nullptr;
  for (int pass = 0; pass < (grad ? 5 : 1); ++pass) {
    Dual<3> p[9], u[6];
#pragma unroll
    for (int q = 0; q < 15; ++q) {
      Dual<3> x = cst<3>(pin[q]);
#pragma unroll
      for (int k = 0; k < 3; ++k) x.d[k] = (grad && q == 3 * pass + k) ? 1.0 : 0.0;
      if (q < 9) p[q] = x;
      else u[q - 9] = x;
    }
    Dual<3> out;
    if (!tri_distortion(p, u, out)) break;
    val = out.v;
    if (!grad) break;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int q = 3 * pass + k;
      if (q < 9) {
        if (dp3) atomicAdd(&dp3[3 * v[q / 3] + q % 3], out.d[k]);
      } else if (duv) {
        atomicAdd(&duv[2 * v[(q - 9) / 2] + (q - 9) % 2], out.d[k]);
      }
    }
  }
  loss_t[t] = val;
}

// Per-chart sums of a per-triangle array (one CTA per chart, fixed order: deterministic).
__global__ void __launch_bounds__(kAdjThreads) k_chart_sum(const int64_t* __restrict__ tri_off, const double* __restrict__ a,
                                                           double* __restrict__ out) {
  __shared__ double sh[32];
  const int64_t c = blockIdx.x;
  double s[1] = {0.0};
  for (int64_t t = tri_off[c] + threadIdx.x; t < tri_off[c + 1]; t += blockDim.x) s[0] += a[t];
  block_sum<1>(s, sh);
  if (threadIdx.x == 0) out[c] = s[0];
}

// ---------------------------------------------------------------- metrics (metrics.rs:73-141)
// Every operation rounded on its own (no FMA contraction) in the reference's order, so each
// per-triangle value equals the reference's bit for bit; the per-chart sums run in triangle
// order.
__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double rmax(double a, double b) {  // Rust f64::max
  if (a != a) return b;
  if (b != b) return a;
  return a > b ? a : b;
}
__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return ad(ad(ml(a[0], b[0]), ml(a[1], b[1])), ml(a[2], b[2]));
}
__device__ __forceinline__ void cross3(const double* a, const double* b, double* o) {
  o[0] = sb(ml(a[1], b[2]), ml(a[2], b[1]));
  o[1] = sb(ml(a[2], b[0]), ml(a[0], b[2]));
  o[2] = sb(ml(a[0], b[1]), ml(a[1], b[0]));
}
__device__ __forceinline__ double tri_signed(double au, double av, double bu, double bv, double cu, double cv) {
  return sb(ml(sb(bu, au), sb(cv, av)), ml(sb(cu, au), sb(bv, av)));  // metrics.rs:32-35
}

// Per triangle: conformal ratio (or -1 when skipped), area ratio, flip flag, signed UV area.
__global__ void __launch_bounds__(kAdjThreads) k_tri_metrics(const int64_t* __restrict__ tri_off,
                                                             const int64_t* __restrict__ vert_off, int64_t n_charts,
                                                             int64_t n_tris, const int32_t* __restrict__ tris,
                                                             const double* __restrict__ p3, const double* __restrict__ uv,
                                                             double4* __restrict__ m) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tris) return;
  const int64_t c = chart_of(tri_off, n_charts, t);
  const int64_t v0 = vert_off[c];
  const int64_t a = v0 + tris[3 * t], b = v0 + tris[3 * t + 1], d = v0 + tris[3 * t + 2];
  double e1[3], e2[3], n[3];
  for (int k = 0; k < 3; ++k) {
    e1[k] = sb(p3[3 * b + k], p3[3 * a + k]);
    e2[k] = sb(p3[3 * d + k], p3[3 * a + k]);
  }
  cross3(e1, e2, n);
  const double ln = sqrt(dot3(n, n));
  const double sgn = tri_signed(uv[2 * a], uv[2 * a + 1], uv[2 * b], uv[2 * b + 1], uv[2 * d], uv[2 * d + 1]);
  double4 r = make_double4(-1.0, -1.0, 0.0, sgn);
  if (ln >= 1e-30) {
    double nu[3], t1[3], t2[3];
    const double l1 = rmax(sqrt(dot3(e1, e1)), 1e-30);
    for (int k = 0; k < 3; ++k) {
      nu[k] = dv(n[k], ln);
      t1[k] = dv(e1[k], l1);
    }
    cross3(nu, t1, t2);
    const double e1t1 = dot3(e1, t1), e2t1 = dot3(e2, t1), e1t2 = dot3(e1, t2), e2t2 = dot3(e2, t2);
    const double det = sb(ml(e1t1, e2t2), ml(e2t1, e1t2));
    if (fabs(det) < 1e-30) {
      r.z = 1.0;
    } else {
      const double i00 = dv(e2t2, det), i01 = dv(-e2t1, det), i10 = dv(-e1t2, det), i11 = dv(e1t1, det);
      const double d1u = sb(uv[2 * b], uv[2 * a]), d1v = sb(uv[2 * b + 1], uv[2 * a + 1]);
      const double d2u = sb(uv[2 * d], uv[2 * a]), d2v = sb(uv[2 * d + 1], uv[2 * a + 1]);
      const double f00 = ad(ml(d1u, i00), ml(d2u, i10)), f01 = ad(ml(d1u, i01), ml(d2u, i11));
      const double f10 = ad(ml(d1v, i00), ml(d2v, i10)), f11 = ad(ml(d1v, i01), ml(d2v, i11));
      const double aa = ad(ml(f00, f00), ml(f10, f10)), bb = ad(ml(f00, f01), ml(f10, f11));
      const double cc = ad(ml(f01, f01), ml(f11, f11));
      const double tr = ad(aa, cc), dd = ml(0.5, sb(aa, cc));
      const double disc = sqrt(rmax(ad(ml(dd, dd), ml(bb, bb)), 0.0));
      const double lam1 = ad(ml(0.5, tr), disc), lam2 = rmax(sb(ml(0.5, tr), disc), 0.0);
      const double s1 = sqrt(rmax(lam1, 0.0)), s2 = sqrt(lam2);
      r.x = dv(s1, rmax(s2, 1e-30));
      r.y = dv(ml(0.5, fabs(sb(ml(d1u, d2v), ml(d2u, d1v)))), ml(0.5, ln));
    }
  }
  m[t] = r;
}

// Per chart (one thread, triangle order): [conformal mean, conformal max, area ratio mean,
// flips, folds].
__global__ void k_chart_metrics(int64_t n_charts, const int64_t* __restrict__ tri_off, const double4* __restrict__ m,
                                double* __restrict__ out) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_charts) return;
  double cs = 0.0, cm = 0.0, as = 0.0, sg = 0.0;
  int64_t cnt = 0, flips = 0, folds = 0;
  for (int64_t t = tri_off[c]; t < tri_off[c + 1]; ++t) {
    const double4 r = m[t];
    if (r.x >= 0.0) {
      cs = ad(cs, r.x);
      cm = rmax(cm, r.x);
      as = ad(as, r.y);
      ++cnt;
    }
    flips += r.z != 0.0;
    sg = ad(sg, r.w);
  }
  const double dom = sg < 0.0 ? -1.0 : 1.0;
  for (int64_t t = tri_off[c]; t < tri_off[c + 1]; ++t) folds += ml(m[t].w, dom) <= 0.0;
  const double nd = (double)(cnt > 1 ? cnt : 1);
  out[5 * c] = dv(cs, nd);
  out[5 * c + 1] = cm;
  out[5 * c + 2] = dv(as, nd);
  out[5 * c + 3] = (double)flips;
  out[5 * c + 4] = (double)folds;
}

// ---------------------------------------------------------------- rectangularize (metrics.rs:147-227)
constexpr int kRectAngles = 72;
constexpr int kRectThreads = 256;

__device__ __forceinline__ void warp_minmax4(double (&v)[4]) {  // min, max, min, max
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v[0] = fmin(v[0], __shfl_xor_sync(0xffffffffu, v[0], o));
    v[1] = fmax(v[1], __shfl_xor_sync(0xffffffffu, v[1], o));
    v[2] = fmin(v[2], __shfl_xor_sync(0xffffffffu, v[2], o));
    v[3] = fmax(v[3], __shfl_xor_sync(0xffffffffu, v[3], o));
  }
}

// One CTA per chart.  The 72-angle ladder over the border points (each warp a set of
// angles; min / max are exact in any order), the first angle of least score kept, then the
// whole chart rotated, normalised to [0,1]^2 and its border points snapped to the nearest
// rectangle side.  The angle table (cos, sin) comes from the host's libm, as the reference's
// does; every product and sum is rounded on its own (no FMA), so the result is bit-identical.
__global__ void __launch_bounds__(kRectThreads) k_rectangularize(const int64_t* __restrict__ vert_off,
                                                                 const double* __restrict__ uv,
                                                                 const uint8_t* __restrict__ border,
                                                                 const double* __restrict__ cs, double* __restrict__ q,
                                                                 double* __restrict__ ext) {
  __shared__ double score[kRectAngles];
  __shared__ double red[4][kRectThreads / 32];
  __shared__ double rot[2];
  __shared__ int has_border;
  const int64_t c = blockIdx.x;
  const int64_t v0 = vert_off[c], v1 = vert_off[c + 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = kRectThreads / 32;
  if (v1 <= v0) return;
  if (threadIdx.x == 0) has_border = 0;
  __syncthreads();
  for (int64_t i = v0 + threadIdx.x; i < v1; i += blockDim.x)
    if (border[i]) has_border = 1;
  __syncthreads();
  double cth = 1.0, sth = 0.0;
  if (has_border) {
    for (int k = wid; k < kRectAngles; k += nw) {
      const double co = cs[2 * k], si = cs[2 * k + 1];
      double v[4] = {INFINITY, -INFINITY, INFINITY, -INFINITY};
      for (int64_t i = v0 + lane; i < v1; i += 32) {
        if (!border[i]) continue;
        const double pu = uv[2 * i], pv = uv[2 * i + 1];
        const double qu = ad(ml(co, pu), ml(si, pv));
        const double qv = ad(ml(-si, pu), ml(co, pv));
        v[0] = fmin(v[0], qu);
        v[1] = fmax(v[1], qu);
        v[2] = fmin(v[2], qv);
        v[3] = fmax(v[3], qv);
      }
      warp_minmax4(v);
      if (lane == 0) {
        const double e0 = sb(v[1], v[0]), e1 = sb(v[3], v[2]);
        score[k] = sqrt(ad(ml(e0, ad(e0, 1e-30)), ml(e1, ad(e1, 1e-30))));
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int best = 0;  // the first angle of least score (later ties do not replace it)
      for (int k = 1; k < kRectAngles; ++k)
        if (score[k] < score[best]) best = k;
      rot[0] = cs[2 * best];
      rot[1] = cs[2 * best + 1];
    }
    __syncthreads();
    cth = rot[0];
    sth = rot[1];
  }
  // rotate and take the bounding box
  double v[4] = {INFINITY, -INFINITY, INFINITY, -INFINITY};
  for (int64_t i = v0 + threadIdx.x; i < v1; i += blockDim.x) {
    const double pu = uv[2 * i], pv = uv[2 * i + 1];
    double qu = pu, qv = pv;
    if (has_border) {
      qu = ad(ml(cth, pu), ml(sth, pv));
      qv = ad(ml(-sth, pu), ml(cth, pv));
    }
    q[2 * i] = qu;
    q[2 * i + 1] = qv;
    v[0] = fmin(v[0], qu);
    v[1] = fmax(v[1], qu);
    v[2] = fmin(v[2], qv);
    v[3] = fmax(v[3], qv);
  }
  warp_minmax4(v);
  if (lane == 0)
    for (int k = 0; k < 4; ++k) red[k][wid] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    double m[4] = {red[0][0], red[1][0], red[2][0], red[3][0]};
    for (int w = 1; w < nw; ++w) {
      m[0] = fmin(m[0], red[0][w]);
      m[1] = fmax(m[1], red[1][w]);
      m[2] = fmin(m[2], red[2][w]);
      m[3] = fmax(m[3], red[3][w]);
    }
    red[0][0] = m[0];
    red[2][0] = m[2];
    red[1][0] = sb(m[1], m[0]);  // extents
    red[3][0] = sb(m[3], m[2]);
    ext[2 * c] = red[1][0];
    ext[2 * c + 1] = red[3][0];
  }
  __syncthreads();
  const double mu = red[0][0], mv = red[2][0], eu = rmax(red[1][0], 1e-30), ev = rmax(red[3][0], 1e-30);
  for (int64_t i = v0 + threadIdx.x; i < v1; i += blockDim.x) {
    double pu = dv(sb(q[2 * i], mu), eu), pv = dv(sb(q[2 * i + 1], mv), ev);
    if (has_border && border[i]) {  // verticalize: snap onto the nearest side
      const double dx = fmin(pu, sb(1.0, pu)), dy = fmin(pv, sb(1.0, pv));
      if (dx <= dy) pu = pu < 0.5 ? 0.0 : 1.0;
      else pv = pv < 0.5 ? 0.0 : 1.0;
    }
    q[2 * i] = pu;
    q[2 * i + 1] = pv;
  }
}

// ---------------------------------------------------------------- reverse pass of the assembly
// g (vertex-ordered, 2 per vertex) -> per free row.
__global__ void k_gather_rows(int64_t n_rows, const int32_t* __restrict__ row_vert, const double* __restrict__ gv,
                              double* __restrict__ grow) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  const int64_t v = row_vert[r];
  grow[2 * r] = gv[2 * v];
  grow[2 * r + 1] = gv[2 * v + 1];
}

// One free vertex v: for each kept edge (v, nb) that v owns (nb pinned, or v < nb), the
// coefficient's adjoint; its edge-length part goes to p_v and p_nb, its weight part to the
// corners facing the edge (corner_g).
__global__ void k_edge_adjoint(int64_t n_verts, const uint8_t* __restrict__ pinned, const int64_t* __restrict__ row_of,
                               const int64_t* __restrict__ rec_off, const int2* __restrict__ rec,
                               const double* __restrict__ coef, const double* __restrict__ cot,
                               const double* __restrict__ p3, const double* __restrict__ pin_uv,
                               const double* __restrict__ x, const double* __restrict__ lam, double* __restrict__ corner_g,
                               double* dp3) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_verts || pinned[v]) return;
  const int64_t r1 = rec_off[v + 1];
  const int64_t rv = row_of[v];
  const double xu = x[2 * rv], xv = x[2 * rv + 1], lu = lam[2 * rv], lv = lam[2 * rv + 1];
  for (int64_t i = rec_off[v]; i < r1;) {
    const int32_t nb = rec[i].x;
    int64_t j = i;
    double w = 0.0;
    for (; j < r1 && rec[j].x == nb; ++j) w += cot[rec[j].y];
    const double c = coef[i];
    const bool own = pinned[nb] || v < nb;
    if (own && c >= 0.0) {
      double nu, nv, mu = 0.0, mv = 0.0;
      if (pinned[nb]) {
        nu = pin_uv[2 * nb];
        nv = pin_uv[2 * nb + 1];
      } else {
        const int64_t rn = row_of[nb];
        nu = x[2 * rn];
        nv = x[2 * rn + 1];
        mu = lam[2 * rn];
        mv = lam[2 * rn + 1];
      }
      const double gc = -((lu - mu) * (xu - nu) + (lv - mv) * (xv - nv));
      const double dx = p3[3 * nb] - p3[3 * v], dy = p3[3 * nb + 1] - p3[3 * v + 1], dz = p3[3 * nb + 2] - p3[3 * v + 2];
      const double d2 = dx * dx + dy * dy + dz * dz;
      double gw;
      if (d2 > kEpsDegenerate) {
        gw = gc / d2;
        const double gd2 = -gc * w / (d2 * d2);
        atomicAdd(&dp3[3 * nb], 2.0 * gd2 * dx);
        atomicAdd(&dp3[3 * nb + 1], 2.0 * gd2 * dy);
        atomicAdd(&dp3[3 * nb + 2], 2.0 * gd2 * dz);
        atomicAdd(&dp3[3 * v], -2.0 * gd2 * dx);
        atomicAdd(&dp3[3 * v + 1], -2.0 * gd2 * dy);
        atomicAdd(&dp3[3 * v + 2], -2.0 * gd2 * dz);
      } else {
        gw = gc / kEpsDegenerate;
      }
      for (int64_t k = i; k < j; ++k) corner_g[rec[k].y] = gw;
    }
    i = j;
  }
}

// One triangle: the cotangent adjoint of each corner that was not clamped.
__global__ void k_cot_adjoint(int64_t n_tris, const int32_t* __restrict__ tri_g, const double* __restrict__ p3,
                              const double* __restrict__ cot, const double* __restrict__ corner_g, double* dp3) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tris) return;
  int64_t vi[3];
  double p[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vi[k] = tri_g[3 * t + k];
#pragma unroll
    for (int j = 0; j < 3; ++j) p[k][j] = p3[3 * vi[k] + j];
  }
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const double g = corner_g[3 * t + m];
    const double ct = cot[3 * t + m];
    if (g == 0.0 || !(ct > 0.0)) continue;
    const int o = m, e1 = (m + 2) % 3, e0 = (m + 1) % 3;
    double a1[3], a2[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      a1[j] = p[e1][j] - p[o][j];
      a2[j] = p[e0][j] - p[o][j];
    }
    const double n[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]};
    const double C = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(C > 0.0)) continue;
    const double nh[3] = {n[0] / C, n[1] / C, n[2] / C};
    // d cot / d a1 = (a2 - cot (a2 x nh)) / C;  d cot / d a2 = (a1 - cot (nh x a1)) / C
    const double a2n[3] = {a2[1] * nh[2] - a2[2] * nh[1], a2[2] * nh[0] - a2[0] * nh[2], a2[0] * nh[1] - a2[1] * nh[0]};
    const double na1[3] = {nh[1] * a1[2] - nh[2] * a1[1], nh[2] * a1[0] - nh[0] * a1[2], nh[0] * a1[1] - nh[1] * a1[0]};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double g1 = g * (a2[j] - ct * a2n[j]) / C;
      const double g2 = g * (a1[j] - ct * na1[j]) / C;
      atomicAdd(&dp3[3 * vi[e1] + j], g1);
      atomicAdd(&dp3[3 * vi[e0] + j], g2);
      atomicAdd(&dp3[3 * vi[o] + j], -(g1 + g2));
    }
  }
}

}  // namespace

void lscm_backward(Ctx& ctx, DevBatch& bt, const DevSystem& sys, const double* x, const double* g_vert,
                   const SolveOpts& o, double* dp3, std::vector<ChartResult>& res) {
  cudaStream_t s = ctx.stream;
  Workspace& ws = ctx.ws;
  const int64_t NR = sys.n_rows, NV = bt.n_verts, NT = bt.n_tris;
  double* grow = ws.get<double>("adj.g", std::max<int64_t>(2 * NR, 1));
  double* lam = ws.get<double>("adj.lam", std::max<int64_t>(2 * NR, 1));
  if (NR > 0) {
    k_gather_rows<<<div_up(NR, kAdjThreads), kAdjThreads, 0, s>>>(NR, bt.row_vert, g_vert, grow);
    count_launches(1);
    RUV_LAUNCH_CHECK();
  }
  DevSystem adj = sys;  // same operator, right-hand side g
  adj.b = grow;
  res = pcg_solve(ctx, adj, lam, o);
  double* corner_g = ws.get<double>("adj.corner_g", std::max<int64_t>(3 * NT, 1));
  RUV_CUDA(cudaMemsetAsync(corner_g, 0, sizeof(double) * std::max<int64_t>(3 * NT, 1), s));
  RUV_CUDA(cudaMemsetAsync(dp3, 0, sizeof(double) * std::max<int64_t>(3 * NV, 1), s));
  if (NV > 0) {
    k_edge_adjoint<<<div_up(NV, kAdjThreads), kAdjThreads, 0, s>>>(NV, bt.pinned, bt.row_of, bt.rec_off, bt.rec, bt.coef,
                                                                    bt.cot, bt.p3, bt.pin_uv, x, lam, corner_g, dp3);
    count_launches(1);
  }
  if (NT > 0) {
    k_cot_adjoint<<<div_up(NT, kAdjThreads), kAdjThreads, 0, s>>>(NT, bt.tri_g, bt.p3, bt.cot, corner_g, dp3);
    count_launches(1);
  }
  RUV_LAUNCH_CHECK();
}

void distortion_loss(Ctx& ctx, const DevBatch& bt, const double* uv, double* duv, double* dp3, std::vector<double>& loss) {
  cudaStream_t s = ctx.stream;
  const int64_t NT = bt.n_tris, NC = bt.n_charts;
  double* lt = ctx.ws.get<double>("dist.loss_t", std::max<int64_t>(NT, 1));
  double* lc = ctx.ws.get<double>("dist.loss_c", std::max<int64_t>(NC, 1));
  if (NT > 0) {
    k_distortion<<<div_up(NT, kAdjThreads), kAdjThreads, 0, s>>>(bt.tri_off, bt.vert_off, NC, NT, bt.tris, bt.pinned,
                                                                  bt.p3, uv, lt, duv, dp3);
    count_launches(1);
  }
  if (NC > 0) {
    k_chart_sum<<<(unsigned)NC, kAdjThreads, 0, s>>>(bt.tri_off, lt, lc);
    count_launches(1);
  }
  RUV_LAUNCH_CHECK();
  loss.resize(NC);
  if (NC > 0) RUV_CUDA(cudaMemcpyAsync(loss.data(), lc, sizeof(double) * NC, cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
}

void rectangularize(Ctx& ctx, const DevBatch& bt, const double* uv, const uint8_t* border, double* q, double* ext) {
  cudaStream_t s = ctx.stream;
  // the angle ladder of metrics.rs:166-171 with the host's libm (np.linspace(0, pi, 72))
  std::vector<double> h(2 * kRectAngles);
  for (int k = 0; k < kRectAngles; ++k) {
    const double ang = 3.141592653589793 * (double)k / (double)(kRectAngles - 1);
    h[2 * k] = std::cos(ang);
    h[2 * k + 1] = std::sin(ang);
  }
  double* cs = ctx.ws.get<double>("rect.cs", 2 * kRectAngles);
  RUV_CUDA(cudaMemcpyAsync(cs, h.data(), sizeof(double) * 2 * kRectAngles, cudaMemcpyHostToDevice, s));
  if (bt.n_charts > 0) {
    k_rectangularize<<<(unsigned)bt.n_charts, kRectThreads, 0, s>>>(bt.vert_off, uv, border, cs, q, ext);
    count_launches(1);
  }
  RUV_LAUNCH_CHECK();
  RUV_CUDA(cudaStreamSynchronize(s));  // `h` goes out of scope
}

void chart_metrics(Ctx& ctx, const DevBatch& bt, const double* uv, std::vector<double>& out5) {
  cudaStream_t s = ctx.stream;
  const int64_t NT = bt.n_tris, NC = bt.n_charts;
  double4* m = ctx.ws.get<double4>("met.tri", std::max<int64_t>(NT, 1));
  double* o = ctx.ws.get<double>("met.out", std::max<int64_t>(5 * NC, 1));
  if (NT > 0) {
    k_tri_metrics<<<div_up(NT, kAdjThreads), kAdjThreads, 0, s>>>(bt.tri_off, bt.vert_off, NC, NT, bt.tris, bt.p3, uv, m);
    count_launches(1);
  }
  if (NC > 0) {
    k_chart_metrics<<<div_up(NC, 64), 64, 0, s>>>(NC, bt.tri_off, m, o);
    count_launches(1);
  }
  RUV_LAUNCH_CHECK();
  out5.resize(5 * NC);
  if (NC > 0) RUV_CUDA(cudaMemcpyAsync(out5.data(), o, sizeof(double) * 5 * NC, cudaMemcpyDeviceToHost, s));
  RUV_CUDA(cudaStreamSynchronize(s));
}

}  // namespace ruv
