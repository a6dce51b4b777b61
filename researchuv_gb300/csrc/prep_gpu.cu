// Mesh preparation on the device: the data-parallel stages of prepare_mesh (weld.rs:19-57,
// segment.rs:73-137 and :177-196) with the results of the host path bit for bit.
//
// * weld: an open-addressing table keyed by the rounded coordinates; a slot is claimed by
//   the first vertex to reach it (its keys are recomputed from its position when compared,
//   so the table stores vertex ids only) and keeps the smallest vertex id of its key -- the
//   reference's first occurrence.  Welded ids number the first occurrences in index order;
//   collapsed faces are dropped by a compaction that keeps the face order.
// * edge-face lists: the key min*V + max of every face slot, a stable radix sort, and the
//   runs of equal keys: each slot's list is its run's faces, ascending (stable order).
// * normals and cut flags: the host's operation order with explicit round-to-nearest
//   operations; acos(n1.n2) > angle becomes n1.n2 < d* with d* from the host libm.
// * chart vertex sets: the key chart*V + vertex of every corner in chart face order, a
//   stable radix sort; the runs give each chart's sorted vertex ids and every corner's
//   chart-local index.
// The DFS order of the components, the border loops, frames, pins and packing stay on the
// host (sequential by definition: stack pops, walks, left-to-right sums).
#include <algorithm>
#include <climits>
#include <cmath>

#include "fp64rn.cuh"
#include "ruv_internal.h"
#include "system.cuh"

namespace ruv {
namespace {

// ---------------------------------------------------------------- stable LSD radix sort
// (key, value) pairs by the low `bits` bits of the 64-bit keys, 8 bits per pass.  Pass:
// per-tile digit counts, one exclusive scan over (digit, tile), then a scatter that ranks each
// item among the tile's equal digits in tile order (warp match + per-warp counts), so equal
// keys keep their input order.
constexpr int kRsThreads = 256, kRsItems = 8, kRsTile = kRsThreads * kRsItems;

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint64_t* __restrict__ keys, int64_t n, int shift,
                                                        int32_t* __restrict__ hist, int64_t ntiles) {
  __shared__ int32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsItems; ++r) {
    const int64_t i = base + (int64_t)r * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint64_t* __restrict__ kin,
                                                           const int32_t* __restrict__ vin, int64_t n, int shift,
                                                           const int64_t* __restrict__ off, int64_t ntiles,
                                                           uint64_t* __restrict__ kout, int32_t* __restrict__ vout) {
  constexpr int kWarps = kRsThreads / 32;
  __shared__ int64_t toff[256];
  __shared__ int32_t run[256];
  __shared__ int32_t wcnt[kWarps][256];
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  toff[t] = off[(int64_t)t * ntiles + blockIdx.x];
  run[t] = 0;
  for (int ww = 0; ww < kWarps; ++ww) wcnt[ww][t] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsItems; ++r) {
    const int64_t i = base + (int64_t)r * kRsThreads + t;
    const bool valid = i < n;
    const uint64_t k = valid ? kin[i] : 0ull;
    const int32_t v = valid ? vin[i] : 0;
    const int d = valid ? (int)((k >> shift) & 255u) : 256;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid && (__ffs(peers) - 1) == lane) wcnt[w][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      int rank = run[d] + __popc(peers & ((1u << lane) - 1u));
      for (int ww = 0; ww < w; ++ww) rank += wcnt[ww][d];
      const int64_t pos = toff[d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
    int tot = 0;
    for (int ww = 0; ww < kWarps; ++ww) {
      tot += wcnt[ww][t];
      wcnt[ww][t] = 0;
    }
    run[t] += tot;
    __syncthreads();
  }
}

int bits_for(uint64_t max_key) {
  int b = 0;
  while (b < 64 && (max_key >> b) != 0) ++b;
  return b;
}

// Sorts (keys, vals) by the low `bits` bits; returns the buffers holding the result (the
// inputs or the workspace pair).
std::pair<uint64_t*, int32_t*> radix_sort(Ctx& ctx, uint64_t* keys, int32_t* vals, int64_t n, int bits,
                                          const std::string& tag) {
  if (n <= 1 || bits <= 0) return {keys, vals};
  cudaStream_t s = ctx.stream;
  const int64_t ntiles = div_up(n, (int64_t)kRsTile);
  uint64_t* k2 = ctx.ws.get<uint64_t>(tag + ".k2", n);
  int32_t* v2 = ctx.ws.get<int32_t>(tag + ".v2", n);
  int32_t* hist = ctx.ws.get<int32_t>(tag + ".hist", 256 * ntiles);
  int64_t* off = ctx.ws.get<int64_t>(tag + ".off", 256 * ntiles + 1);
  for (int shift = 0; shift < bits; shift += 8) {
    k_rs_hist<<<(unsigned)ntiles, kRsThreads, 0, s>>>(keys, n, shift, hist, ntiles);
    exclusive_scan(hist, off, 256 * ntiles, ctx.ws, s, tag + ".scan");
    k_rs_scatter<<<(unsigned)ntiles, kRsThreads, 0, s>>>(keys, vals, n, shift, off, ntiles, k2, v2);
    count_launches(2);
    RUV_LAUNCH_CHECK();
    std::swap(keys, k2);
    std::swap(vals, v2);
  }
  return {keys, vals};
}

// ---------------------------------------------------------------- weld
__device__ __forceinline__ long long round_i64(double x) {  // (x).round() as i64, saturating
  const double r = round(x);
  if (r != r) return 0;
  if (r >= 9.2233720368547758e18) return LLONG_MAX;
  if (r <= -9.2233720368547758e18) return LLONG_MIN;
  return (long long)r;
}
struct Key3 {
  long long a, b, c;
};
__device__ __forceinline__ Key3 weld_key(const double* __restrict__ pos, int64_t i, double inv) {
  return {round_i64(__dmul_rn(pos[3 * i], inv)), round_i64(__dmul_rn(pos[3 * i + 1], inv)),
          round_i64(__dmul_rn(pos[3 * i + 2], inv))};
}
__device__ __forceinline__ uint64_t weld_hash(Key3 k) {
  uint64_t h = (uint64_t)k.a * 0xff51afd7ed558ccdull ^ ((uint64_t)k.b + 0x9e3779b97f4a7c15ull) * 0xc4ceb9fe1a85ec53ull ^
               ((uint64_t)k.c + 0x632be59bd9b4e019ull) * 0x94d049bb133111ebull;
  return h ^ (h >> 29);
}

// MODE 0: claim or find the slot of the key and lower its smallest id; MODE 1: canon[i] =
// the smallest id of the key.  Probing is bounded by the table size.
template <int MODE>
__global__ void k_weld(const double* __restrict__ pos, int64_t nv, double inv, int32_t* __restrict__ owner,
                       int32_t* __restrict__ minid, uint64_t cap, int32_t* __restrict__ canon, int* __restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const Key3 k = weld_key(pos, i, inv);
  uint64_t s = weld_hash(k) & (cap - 1);
  for (uint64_t probe = 0; probe < cap; ++probe) {
    int32_t o = reinterpret_cast<volatile int32_t*>(owner)[s];
    if (MODE == 0 && o < 0) {
      const int32_t old = atomicCAS(&owner[s], -1, (int32_t)i);
      o = old < 0 ? (int32_t)i : old;
    }
    if (o >= 0) {
      const Key3 ko = o == (int32_t)i ? k : weld_key(pos, o, inv);
      if (ko.a == k.a && ko.b == k.b && ko.c == k.c) {
        if (MODE == 0)
          atomicMin(&minid[s], (int32_t)i);
        else
          canon[i] = minid[s];
        return;
      }
    }
    s = (s + 1) & (cap - 1);
  }
  atomicExch(bad, 1);  // (a table of twice the vertex count cannot fill up)
}

__global__ void k_weld_first(const int32_t* __restrict__ canon, int64_t nv, uint8_t* __restrict__ first) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nv) first[i] = canon[i] == (int32_t)i ? 1 : 0;
}

__global__ void k_weld_compact(const double* __restrict__ pos, const int32_t* __restrict__ canon,
                               const int64_t* __restrict__ newid, int64_t nv, double* __restrict__ wpos,
                               int32_t* __restrict__ remap) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const int32_t c = canon[i];
  remap[i] = (int32_t)newid[c];
  if (c == (int32_t)i) {
    const int64_t j = newid[i];
    wpos[3 * j] = pos[3 * i];
    wpos[3 * j + 1] = pos[3 * i + 1];
    wpos[3 * j + 2] = pos[3 * i + 2];
  }
}

__global__ void k_face_keep(const int32_t* __restrict__ faces, const int32_t* __restrict__ remap, int64_t nf,
                            uint8_t* __restrict__ keep) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int32_t a = remap ? remap[faces[3 * f]] : faces[3 * f], b = remap ? remap[faces[3 * f + 1]] : faces[3 * f + 1],
                c = remap ? remap[faces[3 * f + 2]] : faces[3 * f + 2];
  // without welding every face is kept (the host path reports a repeated vertex as an error)
  keep[f] = (!remap || (a != b && b != c && a != c)) ? 1 : 0;
}

__global__ void k_face_compact(const int32_t* __restrict__ faces, const int32_t* __restrict__ remap,
                               const uint8_t* __restrict__ keep, const int64_t* __restrict__ at, int64_t nf,
                               int32_t* __restrict__ F) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf || !keep[f]) return;
  const int64_t j = at[f];
  for (int k = 0; k < 3; ++k) F[3 * j + k] = remap ? remap[faces[3 * f + k]] : faces[3 * f + k];
}

// ---------------------------------------------------------------- edge-face lists
__global__ void k_edge_keys(const int32_t* __restrict__ F, int64_t nf, uint64_t nv, uint64_t* __restrict__ keys,
                            int32_t* __restrict__ vals) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= 3 * nf) return;
  const int64_t f = s / 3;
  const int k = (int)(s - 3 * f);
  const uint32_t x = (uint32_t)F[3 * f + k], y = (uint32_t)F[3 * f + (k + 1) % 3];
  keys[s] = (uint64_t)min(x, y) * nv + max(x, y);
  vals[s] = (int32_t)s;
}

// run boundaries of the sorted keys: beg[j] = first position of j's run, cnt[slot] = run length
__global__ void k_run_start(const uint64_t* __restrict__ keys, int64_t n, uint8_t* __restrict__ start) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) start[j] = (j == 0 || keys[j] != keys[j - 1]) ? 1 : 0;
}

__global__ void k_run_bounds(const uint8_t* __restrict__ start, const int64_t* __restrict__ rid, int64_t n,
                             int64_t* __restrict__ rbeg) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n && start[j]) rbeg[rid[j]] = j;
  if (j == 0) rbeg[rid[n]] = n;  // (rid has n + 1 entries: the run count at the end)
}

__global__ void k_ef_count(const int32_t* __restrict__ vals, const int64_t* __restrict__ rid,
                           const int64_t* __restrict__ rbeg, int64_t n, int32_t* __restrict__ cnt) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t r = rid[j + 1] - 1;  // (inclusive run id: rid is the exclusive scan of starts)
  cnt[vals[j]] = (int32_t)(rbeg[r + 1] - rbeg[r]);
}

__global__ void k_ef_fill(const int32_t* __restrict__ vals, const int64_t* __restrict__ rid,
                          const int64_t* __restrict__ rbeg, const int64_t* __restrict__ ef_off, int64_t n,
                          int32_t* __restrict__ ef_faces) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t r = rid[j + 1] - 1;
  const int64_t o = ef_off[vals[j]];
  for (int64_t m = rbeg[r]; m < rbeg[r + 1]; ++m) ef_faces[o + (m - rbeg[r])] = vals[m] / 3;
}

// ---------------------------------------------------------------- normals and cuts
struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 ld3(const double* p, int64_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return {__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)}; }
__device__ __forceinline__ double vdot(V3 a, V3 b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 vcross(V3 a, V3 b) {
  return {__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)), __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
          __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
}

__global__ void k_normals(const double* __restrict__ wpos, const int32_t* __restrict__ F, int64_t nf,
                          double* __restrict__ nrm) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const V3 a = ld3(wpos, F[3 * f]), b = ld3(wpos, F[3 * f + 1]), c = ld3(wpos, F[3 * f + 2]);
  const V3 n = vcross(vsub(a, b), vsub(c, b));
  const double l = sqrt_rn(vdot(n, n));
  V3 u;
  if (l < 1e-30)
    u = {0.0, 0.0, 1.0};
  else
    u = {div_rn(n.x, l), div_rn(n.y, l), div_rn(n.z, l)};
  nrm[3 * f] = u.x;
  nrm[3 * f + 1] = u.y;
  nrm[3 * f + 2] = u.z;
}

__global__ void k_cuts(const int64_t* __restrict__ ef_off, const int32_t* __restrict__ ef_faces,
                       const double* __restrict__ nrm, int64_t nslots, double dstar, int cut_one, int cut_many,
                       uint8_t* __restrict__ cut) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  const int64_t o = ef_off[s], cnt = ef_off[s + 1] - o;
  uint8_t c;
  if (cnt == 1) {
    c = (uint8_t)cut_one;  // angle 0
  } else if (cnt == 2) {
    double d = vdot(ld3(nrm, ef_faces[o]), ld3(nrm, ef_faces[o + 1]));
    d = d < -1.0 ? -1.0 : (d > 1.0 ? 1.0 : d);
    c = d < dstar ? 1 : 0;
  } else {
    c = (uint8_t)cut_many;
  }
  cut[s] = c;
}

// ---------------------------------------------------------------- chart vertex sets
__global__ void k_corner_keys(const int64_t* __restrict__ cf_off, const int32_t* __restrict__ cf, int64_t nc,
                              const int32_t* __restrict__ F, uint64_t nv, int64_t ncorner, uint64_t* __restrict__ keys,
                              int32_t* __restrict__ vals) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ncorner) return;
  const int64_t q = j / 3;
  const int k = (int)(j - 3 * q);
  int64_t lo = 0, hi = nc;  // chart of face position q: largest c with cf_off[c] <= q
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (cf_off[mid] <= q) lo = mid; else hi = mid;
  }
  keys[j] = (uint64_t)lo * nv + (uint32_t)F[3 * (int64_t)cf[q] + k];
  vals[j] = (int32_t)j;
}

__global__ void k_chart_verts(const uint64_t* __restrict__ keys, const int32_t* __restrict__ vals,
                              const uint8_t* __restrict__ start, const int64_t* __restrict__ uid, int64_t n, uint64_t nv,
                              int32_t* __restrict__ verts, int64_t* __restrict__ vert_off) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n || !start[j]) return;
  const int64_t u = uid[j];
  verts[u] = (int32_t)(keys[j] % nv);
  const uint64_t c = keys[j] / nv;
  if (j == 0 || keys[j - 1] / nv != c) vert_off[c] = u;  // first vertex of chart c
}

__global__ void k_chart_local(const uint64_t* __restrict__ keys, const int32_t* __restrict__ vals,
                              const int64_t* __restrict__ uid, const int64_t* __restrict__ vert_off, int64_t n,
                              uint64_t nv, int32_t* __restrict__ tris) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t u = uid[j + 1] - 1;  // this key's unique index
  tris[vals[j]] = (int32_t)(u - vert_off[keys[j] / nv]);
}

// ---------------------------------------------------------------- patches (prepare_patches)
// The last c with off[c] <= t (off[0] = 0 <= t < off[n]): the patch of face or vertex t.
__device__ __forceinline__ int64_t patch_of(const int64_t* __restrict__ off, int64_t n, int64_t t) {
  int64_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) / 2;
    if (off[mid] <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Global faces from the patch-local triangles; bad |= 1 for an index outside its patch, 2 for
// a triangle with a repeated vertex; used[v] = 1 for every vertex a triangle uses.
__global__ void k_patch_faces(const int64_t* __restrict__ vo, const int64_t* __restrict__ to, int64_t np,
                              const int32_t* __restrict__ tris, int64_t nt, int32_t* __restrict__ F,
                              uint8_t* __restrict__ used, int* __restrict__ bad) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const int64_t c = patch_of(to, np, t);
  const int64_t v0 = vo[c], nvc = vo[c + 1] - v0;
  int32_t a[3];
  bool ok = true;
  for (int k = 0; k < 3; ++k) {
    a[k] = tris[3 * t + k];
    if (a[k] < 0 || a[k] >= nvc) ok = false;
  }
  if (!ok) {
    atomicOr(bad, 1);
    for (int k = 0; k < 3; ++k) F[3 * t + k] = 0;
    return;
  }
  if (a[0] == a[1] || a[1] == a[2] || a[0] == a[2]) atomicOr(bad, 2);
  for (int k = 0; k < 3; ++k) {
    F[3 * t + k] = (int32_t)(v0 + a[k]);
    used[v0 + a[k]] = 1;
  }
}

// Faces of each patch in the reference's DFS pop order (segment.rs:150-175: roots in face
// order, a stack, every edge's faces pushed in ascending order when unseen), one thread per
// patch; a patch of several components stays one chart, its components one after the other
// (as on the host); ncomp = the patch's components.  The stack never holds more than the patch's faces
// (a face is pushed once); bad |= 4 if a list leaves the patch (cannot happen: patches share
// no vertices).
__global__ void k_patch_dfs(int64_t np, const int64_t* __restrict__ to, const int64_t* __restrict__ ef_off,
                            const int32_t* __restrict__ ef_faces, uint8_t* __restrict__ seen, int32_t* __restrict__ stack,
                            int32_t* __restrict__ order, int32_t* __restrict__ ncomp, int* __restrict__ bad) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= np) return;
  const int64_t fb = to[c], fe = to[c + 1], n = fe - fb;
  int64_t out = fb, sp = 0;
  int32_t comps = 0;
  for (int64_t f0 = fb; f0 < fe; ++f0) {
    if (seen[f0]) continue;
    ++comps;
    seen[f0] = 1;
    stack[fb + sp++] = (int32_t)f0;
    while (sp > 0) {
      const int32_t f = stack[fb + --sp];
      order[out++] = f;
      for (int k = 0; k < 3; ++k) {
        const int64_t sl = 3 * (int64_t)f + k;
        for (int64_t q = ef_off[sl]; q < ef_off[sl + 1]; ++q) {
          const int32_t g = ef_faces[q];
          if (g < fb || g >= fe) {
            atomicOr(bad, 4);
            continue;
          }
          if (!seen[g]) {
            seen[g] = 1;
            if (sp < n) stack[fb + sp++] = g;
            else atomicOr(bad, 4);
          }
        }
      }
    }
  }
  ncomp[c] = comps;
}

// flags |= 1 when a vertex is used by no triangle
__global__ void k_patch_checks(const uint8_t* __restrict__ used, int64_t nv, int* __restrict__ flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nv && !used[i]) atomicOr(flags, 1);
}

__device__ __forceinline__ double dot3_rn(double ax, double ay, double az, double bx, double by, double bz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}

// Face areas 0.5 |e1 x e2| in the host's operation order (face_areas, segment.rs:61-70).
__global__ void k_face_area(const double* __restrict__ pos, const int32_t* __restrict__ F, int64_t nt,
                            double* __restrict__ area) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nt) return;
  const double* p0 = pos + 3 * (int64_t)F[3 * f];
  const double* p1 = pos + 3 * (int64_t)F[3 * f + 1];
  const double* p2 = pos + 3 * (int64_t)F[3 * f + 2];
  const double ax = __dsub_rn(p1[0], p0[0]), ay = __dsub_rn(p1[1], p0[1]), az = __dsub_rn(p1[2], p0[2]);
  const double bx = __dsub_rn(p2[0], p0[0]), by = __dsub_rn(p2[1], p0[1]), bz = __dsub_rn(p2[2], p0[2]);
  const double cx = __dsub_rn(__dmul_rn(ay, bz), __dmul_rn(az, by));
  const double cy = __dsub_rn(__dmul_rn(az, bx), __dmul_rn(ax, bz));
  const double cz = __dsub_rn(__dmul_rn(ax, by), __dmul_rn(ay, bx));
  area[f] = __dmul_rn(0.5, __dsqrt_rn(dot3_rn(cx, cy, cz, cx, cy, cz)));
}

// Per patch (one thread): the area summed in chart face order (segment.rs:212) and the
// centroid and covariance of its vertices in vertex order (pca_project, lscm.rs:152-170).
__global__ void k_patch_stats(int64_t np, const int64_t* __restrict__ vo, const int64_t* __restrict__ to,
                              const double* __restrict__ pos, const int32_t* __restrict__ order,
                              const double* __restrict__ farea, double* __restrict__ area3d, double* __restrict__ cov) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= np) return;
  double a = 0.0;
  for (int64_t k = to[c]; k < to[c + 1]; ++k) a = __dadd_rn(a, farea[order[k]]);
  area3d[c] = a;
  double* o = cov + 12 * c;
  const int64_t v0 = vo[c], n = vo[c + 1] - v0;
  double m[3] = {0.0, 0.0, 0.0}, cm[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (n > 0) {
    for (int64_t i = v0; i < v0 + n; ++i)
      for (int k = 0; k < 3; ++k) m[k] = __dadd_rn(m[k], pos[3 * i + k]);
    for (int k = 0; k < 3; ++k) m[k] = __ddiv_rn(m[k], (double)n);
    for (int64_t i = v0; i < v0 + n; ++i) {
      double e[3];
      for (int k = 0; k < 3; ++k) e[k] = __dsub_rn(pos[3 * i + k], m[k]);
      for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) cm[3 * r + q] = __dadd_rn(cm[3 * r + q], __dmul_rn(e[r], e[q]));
    }
  }
  for (int k = 0; k < 3; ++k) o[k] = m[k];
  for (int k = 0; k < 9; ++k) o[3 + k] = cm[k];
}

// boundary face slots (an edge carried by one face: segment.rs:198-209 with no cuts)
__global__ void k_border_flag(const int64_t* __restrict__ ef_off, int64_t ns, uint8_t* __restrict__ flag) {
  const int64_t sl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (sl < ns) flag[sl] = (ef_off[sl + 1] - ef_off[sl]) == 1 ? 1 : 0;
}
__global__ void k_border_keys(const int32_t* __restrict__ F, int64_t ns, const uint8_t* __restrict__ flag,
                              const int64_t* __restrict__ at, uint64_t* __restrict__ keys) {
  const int64_t sl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (sl >= ns || !flag[sl]) return;
  const int64_t f = sl / 3;
  const int k = (int)(sl % 3);
  const uint32_t x = (uint32_t)F[3 * f + k], y = (uint32_t)F[3 * f + (k + 1) % 3];
  const uint32_t a = min(x, y), b = max(x, y);
  keys[at[sl]] = ((uint64_t)a << 32) | b;
}
__global__ void k_border_off(const int64_t* __restrict__ to, int64_t np, const int64_t* __restrict__ at,
                             int64_t* __restrict__ boff) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c <= np) boff[c] = at[3 * to[c]];
}

// local triangles in chart (DFS) order
__global__ void k_tris_order(const int32_t* __restrict__ order, const int32_t* __restrict__ tris, int64_t nt,
                             const int64_t* __restrict__ to, int64_t np, int32_t* __restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt) return;
  const int64_t f = order[k];
  for (int j = 0; j < 3; ++j) out[3 * k + j] = tris[3 * f + j];
}

// p2 of every vertex on its chart's frame (centroid, e1, e2): the projection of pca_project
__global__ void k_patch_project(const int64_t* __restrict__ vo, int64_t np, const double* __restrict__ pos,
                                const double* __restrict__ frames, int64_t nv, double* __restrict__ p2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const double* fr = frames + 9 * patch_of(vo, np, i);
  const double dx = __dsub_rn(pos[3 * i], fr[0]), dy = __dsub_rn(pos[3 * i + 1], fr[1]),
               dz = __dsub_rn(pos[3 * i + 2], fr[2]);
  p2[2 * i] = dot3_rn(dx, dy, dz, fr[3], fr[4], fr[5]);
  p2[2 * i + 1] = dot3_rn(dx, dy, dz, fr[6], fr[7], fr[8]);
}

int64_t read_i64(Ctx& ctx, const int64_t* d);

// Edge-face lists of the faces F (3 nf vertex ids < nv) on the device: for every face slot,
// the faces carrying its edge in ascending order (ef_off: 3 nf + 1 offsets, ef_faces).
// Returns the number of list entries.
int64_t device_edge_faces(Ctx& ctx, const int32_t* F, int64_t nf, int64_t nv, int64_t*& ef_off, int32_t*& ef_faces) {
  cudaStream_t s = ctx.stream;
  constexpr int B = 256;
  const int64_t ns = 3 * nf;
  ef_off = ctx.ws.get<int64_t>("prep.ef_off", ns + 1);
  ef_faces = nullptr;
  if (ns <= 0) {
    RUV_CUDA(cudaMemsetAsync(ef_off, 0, sizeof(int64_t), s));
    return 0;
  }
  uint64_t* keys = ctx.ws.get<uint64_t>("prep.ekeys", ns);
  int32_t* vals = ctx.ws.get<int32_t>("prep.evals", ns);
  k_edge_keys<<<div_up(ns, B), B, 0, s>>>(F, nf, (uint64_t)nv, keys, vals);
  count_launches(1);
  const uint64_t maxk = (uint64_t)nv * (uint64_t)nv;
  auto sorted = radix_sort(ctx, keys, vals, ns, bits_for(maxk), "prep.esort");
  uint8_t* start = ctx.ws.get<uint8_t>("prep.estart", ns);
  int64_t* rid = ctx.ws.get<int64_t>("prep.erid", ns + 1);
  k_run_start<<<div_up(ns, B), B, 0, s>>>(sorted.first, ns, start);
  count_launches(1);
  exclusive_scan_u8(start, rid, ns, ctx.ws, s, "prep.erun");
  const int64_t nruns = read_i64(ctx, rid + ns);
  int64_t* rbeg = ctx.ws.get<int64_t>("prep.erbeg", nruns + 1);
  int32_t* cnt = ctx.ws.get<int32_t>("prep.ecnt", ns);
  k_run_bounds<<<div_up(ns, B), B, 0, s>>>(start, rid, ns, rbeg);
  // rid[j + 1] - 1 is j's run for j < ns - 1; the last position reads rid[ns] = the run count
  k_ef_count<<<div_up(ns, B), B, 0, s>>>(sorted.second, rid, rbeg, ns, cnt);
  count_launches(2);
  exclusive_scan(cnt, ef_off, ns, ctx.ws, s, "prep.efoff");
  const int64_t nef = read_i64(ctx, ef_off + ns);
  ef_faces = ctx.ws.get<int32_t>("prep.ef_faces", nef);
  k_ef_fill<<<div_up(ns, B), B, 0, s>>>(sorted.second, rid, rbeg, ef_off, ns, ef_faces);
  count_launches(1);
  return nef;
}

int64_t read_i64(Ctx& ctx, const int64_t* d) {
  int64_t h = 0;
  RUV_CUDA(cudaMemcpyAsync(&h, d, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx.stream));
  RUV_CUDA(cudaStreamSynchronize(ctx.stream));
  return h;
}

template <class T>
void download(Ctx& ctx, std::vector<T>& host, const T* dev, int64_t n) {
  host.resize(n);
  if (n > 0) RUV_CUDA(cudaMemcpyAsync(host.data(), dev, sizeof(T) * n, cudaMemcpyDeviceToHost, ctx.stream));
}

}  // namespace

ruv_status prepare_mesh_gpu(Ctx& ctx, const double* pos, int64_t nv, const int32_t* faces, int64_t nf, double weld_tol,
                            double angle_min_deg, int threads, Prepared& P, std::string& err) {
  cudaStream_t s = ctx.stream;
  constexpr int B = 256;
  for (int64_t i = 0; i < 3 * nf; ++i)
    if (faces[i] < 0 || faces[i] >= nv) {
      err = "face index out of range";
      return RUV_ERR_BAD_INPUT;
    }
  const double dstar = acos_cut_threshold(angle_min_deg);
  if (!(dstar == dstar)) return prepare_mesh(pos, nv, faces, nf, weld_tol, angle_min_deg, threads, P, err);
  const double th = angle_min_deg * (3.14159265358979323846 / 180.0);
  const int cut_one = 0.0 > th ? 1 : 0, cut_many = 3.14159265358979323846 > th ? 1 : 0;
  double* d_pos = ctx.ws.get<double>("prep.pos", 3 * std::max<int64_t>(nv, 1));
  int32_t* d_faces = ctx.ws.get<int32_t>("prep.faces", 3 * std::max<int64_t>(nf, 1));
  if (nv > 0) RUV_CUDA(cudaMemcpyAsync(d_pos, pos, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, s));
  if (nf > 0) RUV_CUDA(cudaMemcpyAsync(d_faces, faces, sizeof(int32_t) * 3 * nf, cudaMemcpyHostToDevice, s));
  int* bad = ctx.ws.get<int>("prep.bad", 1);
  RUV_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
  // ---- weld
  const double* d_wpos = d_pos;
  const int32_t* remap = nullptr;
  int64_t wnv = nv;
  if (weld_tol > 0.0 && nv > 0) {
    const double inv = 1.0 / weld_tol;
    uint64_t cap = 16;
    while (cap < (uint64_t)nv * 2 + 16) cap <<= 1;
    int32_t* owner = ctx.ws.get<int32_t>("prep.owner", (int64_t)cap);
    int32_t* minid = ctx.ws.get<int32_t>("prep.minid", (int64_t)cap);
    int32_t* canon = ctx.ws.get<int32_t>("prep.canon", nv);
    RUV_CUDA(cudaMemsetAsync(owner, 0xff, sizeof(int32_t) * cap, s));
    RUV_CUDA(cudaMemsetAsync(minid, 0x7f, sizeof(int32_t) * cap, s));
    k_weld<0><<<div_up(nv, B), B, 0, s>>>(d_pos, nv, inv, owner, minid, cap, canon, bad);
    k_weld<1><<<div_up(nv, B), B, 0, s>>>(d_pos, nv, inv, owner, minid, cap, canon, bad);
    uint8_t* first = ctx.ws.get<uint8_t>("prep.first", nv);
    k_weld_first<<<div_up(nv, B), B, 0, s>>>(canon, nv, first);
    count_launches(3);
    int64_t* newid = ctx.ws.get<int64_t>("prep.newid", nv + 1);
    exclusive_scan_u8(first, newid, nv, ctx.ws, s, "prep.weld");
    wnv = read_i64(ctx, newid + nv);
    double* wpos = ctx.ws.get<double>("prep.wpos", 3 * std::max<int64_t>(wnv, 1));
    int32_t* rm = ctx.ws.get<int32_t>("prep.remap", nv);
    k_weld_compact<<<div_up(nv, B), B, 0, s>>>(d_pos, canon, newid, nv, wpos, rm);
    count_launches(1);
    d_wpos = wpos;
    remap = rm;
  }
  uint8_t* keep = ctx.ws.get<uint8_t>("prep.keep", std::max<int64_t>(nf, 1));
  int64_t* fat = ctx.ws.get<int64_t>("prep.fat", nf + 1);
  if (nf > 0) {
    k_face_keep<<<div_up(nf, B), B, 0, s>>>(d_faces, remap, nf, keep);
    count_launches(1);
  }
  exclusive_scan_u8(keep, fat, nf, ctx.ws, s, "prep.keep");
  const int64_t wnf = read_i64(ctx, fat + nf);
  int32_t* F = ctx.ws.get<int32_t>("prep.F", 3 * std::max<int64_t>(wnf, 1));
  if (nf > 0) {
    k_face_compact<<<div_up(nf, B), B, 0, s>>>(d_faces, remap, keep, fat, nf, F);
    count_launches(1);
  }
  // ---- edge-face lists
  const int64_t ns = 3 * wnf;
  int64_t* ef_off = nullptr;
  int32_t* ef_faces = nullptr;
  const int64_t nef = device_edge_faces(ctx, F, wnf, wnv, ef_off, ef_faces);
  // ---- normals and cut flags
  uint8_t* cut = ctx.ws.get<uint8_t>("prep.cut", std::max<int64_t>(ns, 1));
  if (wnf > 0) {
    double* nrm = ctx.ws.get<double>("prep.nrm", 3 * wnf);
    k_normals<<<div_up(wnf, B), B, 0, s>>>(d_wpos, F, wnf, nrm);
    k_cuts<<<div_up(ns, B), B, 0, s>>>(ef_off, ef_faces, nrm, ns, dstar, cut_one, cut_many, cut);
    count_launches(2);
  }
  RUV_LAUNCH_CHECK();
  int h_bad = 0;
  RUV_CUDA(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  std::vector<double> h_wpos;
  std::vector<int32_t> h_F, h_ef_faces;
  std::vector<int64_t> h_ef_off;
  std::vector<uint8_t> h_cut;
  download(ctx, h_wpos, d_wpos, 3 * wnv);
  download(ctx, h_F, (const int32_t*)F, 3 * wnf);
  download(ctx, h_ef_off, (const int64_t*)ef_off, ns + 1);
  download(ctx, h_ef_faces, (const int32_t*)ef_faces, nef);
  download(ctx, h_cut, (const uint8_t*)cut, ns);
  RUV_CUDA(cudaStreamSynchronize(s));
  if (h_bad) {
    err = "weld table overflow";
    return RUV_ERR_INTERNAL;
  }
  // ---- chart vertex sets on the device, after the host's DFS order
  ChartSetsFn sets = [&](const std::vector<int64_t>& cf_off, const std::vector<int32_t>& cf, ChartSets& out,
                         std::string& e) -> bool {
    const int64_t nc = (int64_t)cf_off.size() - 1, nq = cf_off.back(), ncn = 3 * nq;
    out.vert_off.assign(nc + 1, 0);
    out.verts.clear();
    out.tris.assign(ncn, 0);
    if (nc <= 0 || ncn == 0) return true;
    int64_t* d_cf_off = ctx.ws.get<int64_t>("prep.cf_off", nc + 1);
    int32_t* d_cf = ctx.ws.get<int32_t>("prep.cf", nq);
    RUV_CUDA(cudaMemcpyAsync(d_cf_off, cf_off.data(), sizeof(int64_t) * (nc + 1), cudaMemcpyHostToDevice, s));
    RUV_CUDA(cudaMemcpyAsync(d_cf, cf.data(), sizeof(int32_t) * nq, cudaMemcpyHostToDevice, s));
    uint64_t* keys = ctx.ws.get<uint64_t>("prep.ckeys", ncn);
    int32_t* vals = ctx.ws.get<int32_t>("prep.cvals", ncn);
    k_corner_keys<<<div_up(ncn, B), B, 0, s>>>(d_cf_off, d_cf, nc, F, (uint64_t)wnv, ncn, keys, vals);
    count_launches(1);
    auto sorted = radix_sort(ctx, keys, vals, ncn, bits_for((uint64_t)nc * (uint64_t)wnv), "prep.csort");
    uint8_t* start = ctx.ws.get<uint8_t>("prep.cstart", ncn);
    int64_t* uid = ctx.ws.get<int64_t>("prep.cuid", ncn + 1);
    k_run_start<<<div_up(ncn, B), B, 0, s>>>(sorted.first, ncn, start);
    count_launches(1);
    exclusive_scan_u8(start, uid, ncn, ctx.ws, s, "prep.cuniq");
    const int64_t nu = read_i64(ctx, uid + ncn);
    int32_t* d_verts = ctx.ws.get<int32_t>("prep.cverts", nu);
    int64_t* d_voff = ctx.ws.get<int64_t>("prep.cvoff", nc + 1);
    RUV_CUDA(cudaMemcpyAsync(d_voff + nc, &nu, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    int32_t* d_tris = ctx.ws.get<int32_t>("prep.ctris", ncn);
    k_chart_verts<<<div_up(ncn, B), B, 0, s>>>(sorted.first, sorted.second, start, uid, ncn, (uint64_t)wnv, d_verts,
                                               d_voff);
    k_chart_local<<<div_up(ncn, B), B, 0, s>>>(sorted.first, sorted.second, uid, d_voff, ncn, (uint64_t)wnv, d_tris);
    count_launches(2);
    RUV_LAUNCH_CHECK();
    download(ctx, out.vert_off, (const int64_t*)d_voff, nc + 1);
    download(ctx, out.verts, (const int32_t*)d_verts, nu);
    download(ctx, out.tris, (const int32_t*)d_tris, ncn);
    RUV_CUDA(cudaStreamSynchronize(s));
    (void)e;
    return true;
  };
  return prepare_mesh_topology(std::move(h_wpos), std::move(h_F), std::move(h_ef_off), std::move(h_ef_faces),
                               std::move(h_cut), threads, &sets, P, err);
}

// prepare_patches with its data-parallel stages on the device of `ctx` (see
// prepare_patches_device): the same Prepared as the host path, bit for bit.
ruv_status prepare_patches_gpu(Ctx& ctx, int64_t np, const int64_t* vert_off, const int64_t* tri_off, const double* p3,
                               const int32_t* tris, int threads, Prepared& P, std::string& err) {
  cudaStream_t s = ctx.stream;
  constexpr int B = 256;
  int64_t* d_vo = nullptr;
  double* d_pos = nullptr;
  PatchDeviceFn dev = [&](PatchDevice& D, std::string& e) -> ruv_status {
    const int64_t NV = vert_off[np], NT = tri_off[np], ns = 3 * NT;
    d_vo = ctx.ws.get<int64_t>("pp.vo", np + 1);
    int64_t* d_to = ctx.ws.get<int64_t>("pp.to", np + 1);
    d_pos = ctx.ws.get<double>("pp.pos", 3 * std::max<int64_t>(NV, 1));
    int32_t* d_tris = ctx.ws.get<int32_t>("pp.tris", 3 * std::max<int64_t>(NT, 1));
    RUV_CUDA(cudaMemcpyAsync(d_vo, vert_off, sizeof(int64_t) * (np + 1), cudaMemcpyHostToDevice, s));
    RUV_CUDA(cudaMemcpyAsync(d_to, tri_off, sizeof(int64_t) * (np + 1), cudaMemcpyHostToDevice, s));
    if (NV > 0) RUV_CUDA(cudaMemcpyAsync(d_pos, p3, sizeof(double) * 3 * NV, cudaMemcpyHostToDevice, s));
    if (NT > 0) RUV_CUDA(cudaMemcpyAsync(d_tris, tris, sizeof(int32_t) * 3 * NT, cudaMemcpyHostToDevice, s));
    int32_t* F = ctx.ws.get<int32_t>("pp.F", 3 * std::max<int64_t>(NT, 1));
    uint8_t* used = ctx.ws.get<uint8_t>("pp.used", std::max<int64_t>(NV, 1));
    int* bad = ctx.ws.get<int>("pp.bad", 4);
    RUV_CUDA(cudaMemsetAsync(bad, 0, 4 * sizeof(int), s));
    if (NV > 0) RUV_CUDA(cudaMemsetAsync(used, 0, NV, s));
    if (NT > 0) {
      k_patch_faces<<<div_up(NT, B), B, 0, s>>>(d_vo, d_to, np, d_tris, NT, F, used, bad);
      count_launches(1);
    }
    int hb[4] = {0, 0, 0, 0};
    RUV_CUDA(cudaMemcpyAsync(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaStreamSynchronize(s));
    if (hb[0] & 1) {
      e = "patch triangle index out of range";
      return RUV_ERR_BAD_INPUT;
    }
    if (hb[0] & 2) {
      e = "degenerate patch triangle";
      return RUV_ERR_BAD_INPUT;
    }
    int64_t* ef_off = nullptr;
    int32_t* ef_faces = nullptr;
    device_edge_faces(ctx, F, NT, NV, ef_off, ef_faces);
    uint8_t* seen = ctx.ws.get<uint8_t>("pp.seen", std::max<int64_t>(NT, 1));
    int32_t* stack = ctx.ws.get<int32_t>("pp.stack", std::max<int64_t>(NT, 1));
    int32_t* order = ctx.ws.get<int32_t>("pp.order", std::max<int64_t>(NT, 1));
    int32_t* ncomp = ctx.ws.get<int32_t>("pp.ncomp", std::max<int64_t>(np, 1));
    if (NT > 0) RUV_CUDA(cudaMemsetAsync(seen, 0, NT, s));
    if (np > 0) {
      k_patch_dfs<<<div_up(np, 128), 128, 0, s>>>(np, d_to, ef_off, ef_faces, seen, stack, order, ncomp, bad);
      count_launches(1);
    }
    if (NV > 0) {
      k_patch_checks<<<div_up(NV, B), B, 0, s>>>(used, NV, bad + 1);
      count_launches(1);
    }
    RUV_CUDA(cudaMemcpyAsync(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost, s));
    RUV_CUDA(cudaStreamSynchronize(s));
    if (hb[0] & 4) {
      e = "patch edge lists leave their patch";
      return RUV_ERR_INTERNAL;
    }
    if (hb[1] & 1) {  // name the first patch with an unused vertex, as the host path does
      std::vector<uint8_t> hu;
      download(ctx, hu, (const uint8_t*)used, NV);
      RUV_CUDA(cudaStreamSynchronize(s));
      const int64_t v = (int64_t)(std::find(hu.begin(), hu.end(), (uint8_t)0) - hu.begin());
      const int64_t c = (int64_t)(std::upper_bound(vert_off, vert_off + np + 1, v) - vert_off) - 1;
      e = "patch " + std::to_string(c) + " has vertices no triangle uses";
      return RUV_ERR_BAD_INPUT;
    }
    double* farea = ctx.ws.get<double>("pp.farea", std::max<int64_t>(NT, 1));
    double* area3d = ctx.ws.get<double>("pp.area3d", std::max<int64_t>(np, 1));
    double* cov = ctx.ws.get<double>("pp.cov", 12 * std::max<int64_t>(np, 1));
    uint8_t* bflag = ctx.ws.get<uint8_t>("pp.bflag", std::max<int64_t>(ns, 1));
    int64_t* bat = ctx.ws.get<int64_t>("pp.bat", ns + 1);
    int64_t* boff = ctx.ws.get<int64_t>("pp.boff", np + 1);
    int32_t* tris_out = ctx.ws.get<int32_t>("pp.tris_out", 3 * std::max<int64_t>(NT, 1));
    if (NT > 0) {
      k_face_area<<<div_up(NT, B), B, 0, s>>>(d_pos, F, NT, farea);
      k_border_flag<<<div_up(ns, B), B, 0, s>>>(ef_off, ns, bflag);
      k_tris_order<<<div_up(NT, B), B, 0, s>>>(order, d_tris, NT, d_to, np, tris_out);
      count_launches(3);
    }
    if (np > 0) {
      k_patch_stats<<<div_up(np, 64), 64, 0, s>>>(np, d_vo, d_to, d_pos, order, farea, area3d, cov);
      count_launches(1);
    }
    exclusive_scan_u8(bflag, bat, ns, ctx.ws, s, "pp.bscan");
    const int64_t nb = read_i64(ctx, bat + ns);
    uint64_t* bkeys = ctx.ws.get<uint64_t>("pp.bkeys", std::max<int64_t>(nb, 1));
    if (ns > 0) {
      k_border_keys<<<div_up(ns, B), B, 0, s>>>(F, ns, bflag, bat, bkeys);
      count_launches(1);
    }
    k_border_off<<<div_up(np + 1, B), B, 0, s>>>(d_to, np, bat, boff);
    count_launches(1);
    RUV_LAUNCH_CHECK();
    download(ctx, D.order, (const int32_t*)order, NT);
    download(ctx, D.tris, (const int32_t*)tris_out, 3 * NT);
    download(ctx, D.area3d, (const double*)area3d, np);
    download(ctx, D.cov, (const double*)cov, 12 * np);
    download(ctx, D.boff, (const int64_t*)boff, np + 1);
    download(ctx, D.bkeys, (const uint64_t*)bkeys, nb);
    RUV_CUDA(cudaStreamSynchronize(s));
    return RUV_OK;
  };
  PatchProjectFn proj = [&](const std::vector<double>& frames, std::vector<double>& p2, std::string& e) -> ruv_status {
    (void)e;
    const int64_t NV = vert_off[np];
    double* d_fr = ctx.ws.get<double>("pp.frames", 9 * std::max<int64_t>(np, 1));
    double* d_p2 = ctx.ws.get<double>("pp.p2", 2 * std::max<int64_t>(NV, 1));
    if (np > 0) RUV_CUDA(cudaMemcpyAsync(d_fr, frames.data(), sizeof(double) * 9 * np, cudaMemcpyHostToDevice, s));
    if (NV > 0) {
      k_patch_project<<<div_up(NV, B), B, 0, s>>>(d_vo, np, d_pos, d_fr, NV, d_p2);
      count_launches(1);
      RUV_LAUNCH_CHECK();
      RUV_CUDA(cudaMemcpyAsync(p2.data(), d_p2, sizeof(double) * 2 * NV, cudaMemcpyDeviceToHost, s));
    }
    RUV_CUDA(cudaStreamSynchronize(s));
    return RUV_OK;
  };
  return prepare_patches_device(np, vert_off, tri_off, p3, tris, threads, dev, proj, P, err);
}

}  // namespace ruv
