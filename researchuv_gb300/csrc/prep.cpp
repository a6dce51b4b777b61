// Host chart stages of the LSCM path: weld, sharp-edge segmentation, border loops, tangent
// frames and Dirichlet pins — everything unfold_chart computes before it assembles
// (reference: unwrap/src/weld.rs:19-57, unwrap/src/segment.rs:61-331,
// unwrap/src/lscm.rs:152-247, :280-413, :512-592).
//
// These stages are O(V + F) integer/topology work with a little libm (acos, atan2, sin,
// cos) and stay on the host; they run on the calling thread plus a pool over charts.  The
// data structures are flat arrays (vertex->face CSR, sorted edge tables, per-chart scratch)
// instead of the reference's BTreeMaps, but every visit order that decides a result — DFS
// stack pops, ascending-neighbour walks, left-to-right floating sums — is the reference's,
// so the partition, loops, pins and frames are bit-identical on the same host libm.
// Compiled with -ffp-contract=off (no FMA contraction).

#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <chrono>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

#include "ruv_internal.h"

namespace ruv {
namespace {

constexpr double kPi = 3.14159265358979323846;

struct D3 {
  double x, y, z;
};
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator/(D3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double dot3(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm3(D3 a) { return std::sqrt(dot3(a, a)); }

inline double fmax_rs(double a, double b) {  // Rust f64::max
  if (a != a) return b;
  if (b != b) return a;
  return a > b ? a : b;
}
inline double fmin_rs(double a, double b) {  // Rust f64::min
  if (a != a) return b;
  if (b != b) return a;
  return a < b ? a : b;
}
inline int64_t total_order_key(double a) {  // Rust f64::total_cmp
  int64_t i;
  std::memcpy(&i, &a, 8);
  return i ^ (int64_t)(((uint64_t)(i >> 63)) >> 1);
}
inline int64_t round_to_i64(double x) {  // (x).round() as i64, saturating
  double r = std::round(x);
  if (r != r) return 0;
  if (r >= 9.2233720368547758e18) return INT64_MAX;
  if (r <= -9.2233720368547758e18) return INT64_MIN;
  return (int64_t)r;
}

template <class F>
void parallel_for(int64_t n, int threads, F&& body) {
  if (n <= 0) return;
  int nt = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
  nt = (int)std::min<int64_t>(nt, n);
  if (nt <= 1) {
    for (int64_t i = 0; i < n; ++i) body(i);
    return;
  }
  std::atomic<int64_t> next{0};
  std::vector<std::thread> pool;
  pool.reserve(nt);
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&] {
      for (;;) {
        int64_t i = next.fetch_add(1);
        if (i >= n) break;
        body(i);
      }
    });
  for (auto& th : pool) th.join();
}

// ------------------------------------------------------------------ weld (weld.rs:19-57)
// Open-addressing table on the rounded integer key; the first vertex with a key becomes
// the canonical id (the reference's HashMap-first-occurrence rule).
void weld(const double* pos, int64_t nv, const int32_t* faces, int64_t nf, double tol,
          std::vector<D3>& out_pos, std::vector<int32_t>& out_faces) {
  out_pos.clear();
  out_faces.clear();
  if (tol <= 0.0) {
    out_pos.resize(nv);
    for (int64_t i = 0; i < nv; ++i) out_pos[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    out_faces.assign(faces, faces + 3 * nf);
    return;
  }
  double inv = 1.0 / tol;
  uint64_t cap = 16;
  while (cap < (uint64_t)nv * 2 + 16) cap <<= 1;
  struct Slot {
    int64_t k[3];
    int32_t id;
  };
  std::vector<Slot> table(cap, Slot{{0, 0, 0}, -1});
  std::vector<int32_t> remap(nv);
  for (int64_t i = 0; i < nv; ++i) {
    int64_t k0 = round_to_i64(pos[3 * i] * inv), k1 = round_to_i64(pos[3 * i + 1] * inv),
            k2 = round_to_i64(pos[3 * i + 2] * inv);
    uint64_t h = (uint64_t)k0 * 0xff51afd7ed558ccdull ^ ((uint64_t)k1 + 0x9e3779b97f4a7c15ull) * 0xc4ceb9fe1a85ec53ull ^
                 ((uint64_t)k2 + 0x632be59bd9b4e019ull) * 0x94d049bb133111ebull;
    h ^= h >> 29;
    uint64_t s = h & (cap - 1);
    for (;;) {
      Slot& sl = table[s];
      if (sl.id < 0) {
        sl.k[0] = k0;
        sl.k[1] = k1;
        sl.k[2] = k2;
        sl.id = (int32_t)out_pos.size();
        out_pos.push_back({pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]});
        remap[i] = sl.id;
        break;
      }
      if (sl.k[0] == k0 && sl.k[1] == k1 && sl.k[2] == k2) {
        remap[i] = sl.id;
        break;
      }
      s = (s + 1) & (cap - 1);
    }
  }
  out_faces.reserve(3 * nf);
  for (int64_t f = 0; f < nf; ++f) {
    int32_t a = remap[faces[3 * f]], b = remap[faces[3 * f + 1]], c = remap[faces[3 * f + 2]];
    if (a != b && b != c && a != c) {
      out_faces.push_back(a);
      out_faces.push_back(b);
      out_faces.push_back(c);
    }
  }
}

// ------------------------------------------------------------------ face adjacency
// For every face slot (f, k) — edge (t[k], t[k+1]) — the list of faces carrying that edge in
// ascending face order (segment.rs:73-81 edge_faces), via a vertex->faces CSR.
struct EdgeFaces {
  std::vector<int64_t> off;  // 3F + 1
  std::vector<int32_t> faces;
};

void build_vertex_faces(int64_t nv, const std::vector<int32_t>& F, std::vector<int64_t>& vf_off,
                        std::vector<int32_t>& vf) {
  int64_t nf = (int64_t)F.size() / 3;
  vf_off.assign(nv + 1, 0);
  for (int64_t i = 0; i < 3 * nf; ++i) vf_off[F[i] + 1]++;
  for (int64_t v = 0; v < nv; ++v) vf_off[v + 1] += vf_off[v];
  vf.resize(3 * nf);
  std::vector<int64_t> cur(vf_off.begin(), vf_off.end() - 1);
  for (int64_t f = 0; f < nf; ++f)
    for (int k = 0; k < 3; ++k) vf[cur[F[3 * f + k]]++] = (int32_t)f;
  // a face with a repeated vertex cannot occur after weld; faces per vertex stay ascending
}

EdgeFaces build_edge_faces(int64_t nv, const std::vector<int32_t>& F, int threads) {
  int64_t nf = (int64_t)F.size() / 3;
  std::vector<int64_t> vf_off;
  std::vector<int32_t> vf;
  build_vertex_faces(nv, F, vf_off, vf);
  EdgeFaces ef;
  std::vector<int32_t> cnt(3 * nf);
  auto contains = [&](int32_t g, int32_t y) { return F[3 * g] == y || F[3 * g + 1] == y || F[3 * g + 2] == y; };
  parallel_for((nf + 4095) / 4096, threads, [&](int64_t blk) {
    int64_t f1 = std::min(nf, (blk + 1) * 4096);
    for (int64_t f = blk * 4096; f < f1; ++f)
      for (int k = 0; k < 3; ++k) {
        int32_t x = F[3 * f + k], y = F[3 * f + (k + 1) % 3];
        int32_t a = std::min(x, y), b = std::max(x, y);
        int32_t c = 0;
        for (int64_t q = vf_off[a]; q < vf_off[a + 1]; ++q)
          if (contains(vf[q], b)) ++c;
        cnt[3 * f + k] = c;
      }
  });
  ef.off.assign(3 * nf + 1, 0);
  for (int64_t i = 0; i < 3 * nf; ++i) ef.off[i + 1] = ef.off[i] + cnt[i];
  ef.faces.resize(ef.off[3 * nf]);
  parallel_for((nf + 4095) / 4096, threads, [&](int64_t blk) {
    int64_t f1 = std::min(nf, (blk + 1) * 4096);
    for (int64_t f = blk * 4096; f < f1; ++f)
      for (int k = 0; k < 3; ++k) {
        int32_t x = F[3 * f + k], y = F[3 * f + (k + 1) % 3];
        int32_t a = std::min(x, y), b = std::max(x, y);
        int64_t o = ef.off[3 * f + k];
        for (int64_t q = vf_off[a]; q < vf_off[a + 1]; ++q)
          if (contains(vf[q], b)) ef.faces[o++] = vf[q];
      }
  });
  (void)nv;
  return ef;
}

// ------------------------------------------------------------------ eig3 / tangent frame
// lscm_eig.rs:13-66 — cyclic-by-largest Jacobi rotations on the 3x3 covariance.
void jacobi_eig3(double a[3][3], double w[3], double v[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v[i][j] = i == j ? 1.0 : 0.0;
  for (int it = 0; it < 64; ++it) {
    int p = 0, q = 1;
    double off = std::fabs(a[0][1]);
    if (std::fabs(a[0][2]) > off) {
      off = std::fabs(a[0][2]);
      p = 0;
      q = 2;
    }
    if (std::fabs(a[1][2]) > off) {
      off = std::fabs(a[1][2]);
      p = 1;
      q = 2;
    }
    if (off <= 1e-300) break;
    double apq = a[p][q], app = a[p][p], aqq = a[q][q];
    double th = 0.5 * std::atan2(2.0 * apq, app - aqq);
    double c = std::cos(th), s = std::sin(th);
    int r = 3 - p - q;  // the one index that is neither p nor q
    double arp = c * a[r][p] + s * a[r][q];
    double arq = -s * a[r][p] + c * a[r][q];
    a[r][p] = a[p][r] = arp;
    a[r][q] = a[q][r] = arq;
    a[p][p] = c * c * app + 2.0 * s * c * apq + s * s * aqq;
    a[q][q] = s * s * app - 2.0 * s * c * apq + c * c * aqq;
    a[p][q] = a[q][p] = 0.0;
    for (int k = 0; k < 3; ++k) {
      double vp = v[p][k], vq = v[q][k];
      v[p][k] = c * vp - s * vq;
      v[q][k] = s * vp + c * vq;
    }
  }
  w[0] = a[0][0];
  w[1] = a[1][1];
  w[2] = a[2][2];
}

// lscm.rs:165-178 — the two dominant principal directions of a covariance matrix (eig3, then
// the eigenvalues in descending total order, ties in index order).
void frame_axes(double cm[3][3], D3& e1, D3& e2) {
  double w[3], v[3][3];
  jacobi_eig3(cm, w, v);
  int idx[3] = {0, 1, 2};
  std::stable_sort(idx, idx + 3, [&](int a, int b) { return total_order_key(w[b]) < total_order_key(w[a]); });
  e1 = D3{v[0][idx[0]], v[1][idx[0]], v[2][idx[0]]};
  e2 = D3{v[0][idx[1]], v[1][idx[1]], v[2][idx[1]]};
}

// lscm.rs:152-183 — projection on the two dominant principal directions.
template <class Get>
void pca_project(int64_t n, Get get, double* out_uv) {
  if (n == 0) return;
  D3 c{0.0, 0.0, 0.0};
  for (int64_t i = 0; i < n; ++i) c = c + get(i);
  c = c / (double)n;
  double cm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int64_t i = 0; i < n; ++i) {
    D3 d = get(i) - c;
    double e[3] = {d.x, d.y, d.z};
    for (int r = 0; r < 3; ++r)
      for (int s = 0; s < 3; ++s) cm[r][s] += e[r] * e[s];
  }
  D3 e1, e2;
  frame_axes(cm, e1, e2);
  for (int64_t i = 0; i < n; ++i) {
    D3 d = get(i) - c;
    out_uv[2 * i] = dot3(d, e1);
    out_uv[2 * i + 1] = dot3(d, e2);
  }
}

// lscm.rs:187-204 — clockwise perimeter point of a centred a x b rectangle.
inline void rect_point(double f, double a, double b, double* uv) {
  double per = 2.0 * (a + b);
  double t = std::fmod(f, 1.0) * per;
  if (t < a) {
    uv[0] = a / 2.0 - t;
    uv[1] = -b / 2.0;
    return;
  }
  t -= a;
  if (t < b) {
    uv[0] = -a / 2.0;
    uv[1] = -b / 2.0 + t;
    return;
  }
  t -= b;
  if (t < a) {
    uv[0] = -a / 2.0 + t;
    uv[1] = b / 2.0;
    return;
  }
  t -= a;
  uv[0] = a / 2.0;
  uv[1] = b / 2.0 - t;
}

// ------------------------------------------------------------------ one chart
struct ChartOut {
  std::vector<int32_t> faces;      // source face ids, chart order
  std::vector<int32_t> verts;      // sorted source vertex ids
  std::vector<int32_t> tris;       // local
  std::vector<int32_t> border;     // sorted source ids
  std::vector<int64_t> loop_len;   // per loop
  std::vector<int32_t> loop_ids;   // concatenated loops (source ids)
  double area3d = 0.0;
  std::vector<double> p3, p2, pin_uv;
  std::vector<uint8_t> pinned;
};

struct MeshView {
  const std::vector<D3>& pos;
  const std::vector<int32_t>& F;
  const EdgeFaces& ef;
  const std::vector<uint8_t>& cut;   // per face slot
  const std::vector<double>& farea;  // per face
};

inline bool slot_is_border(const MeshView& m, int64_t slot) {
  return m.cut[slot] || (m.ef.off[slot + 1] - m.ef.off[slot]) == 1;
}

// vertex set (segment.rs:177-196) and chart-local triangles
void chart_sets(const MeshView& m, ChartOut& ch) {
  const auto& F = m.F;
  ch.verts.clear();
  ch.verts.reserve(ch.faces.size() * 3);
  for (int32_t f : ch.faces)
    for (int k = 0; k < 3; ++k) ch.verts.push_back(F[3 * f + k]);
  std::sort(ch.verts.begin(), ch.verts.end());
  ch.verts.erase(std::unique(ch.verts.begin(), ch.verts.end()), ch.verts.end());
  ch.tris.resize(ch.faces.size() * 3);
  for (size_t t = 0; t < ch.faces.size(); ++t)
    for (int k = 0; k < 3; ++k)
      ch.tris[3 * t + k] =
          (int32_t)(std::lower_bound(ch.verts.begin(), ch.verts.end(), F[3 * ch.faces[t] + k]) - ch.verts.begin());
}

// The border vertices (sorted, unique) and boundary edges (key min << 32 | max, sorted, unique)
// of a chart from its border face slots' edges (x, y) in chart face order
// (segment.rs:198-209, :235-244).
void chart_border_set(ChartOut& ch, std::vector<uint64_t>& bedges) {
  ch.border.clear();
  for (uint64_t e : bedges) {
    ch.border.push_back((int32_t)(uint32_t)(e >> 32));
    ch.border.push_back((int32_t)(uint32_t)e);
  }
  std::sort(ch.border.begin(), ch.border.end());
  ch.border.erase(std::unique(ch.border.begin(), ch.border.end()), ch.border.end());
  std::sort(bedges.begin(), bedges.end());
  bedges.erase(std::unique(bedges.begin(), bedges.end()), bedges.end());
}

// border vertices and boundary edges of a chart, and its area (segment.rs:198-212)
void chart_border(const MeshView& m, ChartOut& ch, std::vector<uint64_t>& bedges) {
  const auto& F = m.F;
  bedges.clear();
  for (int32_t f : ch.faces)
    for (int k = 0; k < 3; ++k)
      if (slot_is_border(m, 3 * (int64_t)f + k)) {
        uint32_t x = (uint32_t)F[3 * f + k], y = (uint32_t)F[3 * f + (k + 1) % 3];
        uint32_t a = std::min(x, y), b = std::max(x, y);
        bedges.push_back(((uint64_t)a << 32) | b);
      }
  chart_border_set(ch, bedges);
  // area (segment.rs:212): sum in chart face order
  double area = 0.0;
  for (int32_t f : ch.faces) area += m.farea[f];
  ch.area3d = area;
}

// border loops: keep-going-straight walk (segment.rs:245-330) over the boundary edges;
// positions by source vertex id
void chart_loops(const D3* pos, ChartOut& ch, const std::vector<uint64_t>& bedges) {
  ch.loop_len.clear();
  ch.loop_ids.clear();
  if (!bedges.empty()) {
    // adjacency over boundary vertices; neighbour lists come out ascending because the
    // sorted edge list is scanned in order (segment.rs:249-255)
    std::vector<int32_t> bv(ch.border);  // every endpoint of a boundary edge is a border vertex
    auto bidx = [&](uint32_t v) { return (int64_t)(std::lower_bound(bv.begin(), bv.end(), (int32_t)v) - bv.begin()); };
    std::vector<int64_t> aoff(bv.size() + 1, 0);
    for (uint64_t e : bedges) {
      aoff[bidx((uint32_t)(e >> 32)) + 1]++;
      aoff[bidx((uint32_t)e) + 1]++;
    }
    for (size_t i = 0; i < bv.size(); ++i) aoff[i + 1] += aoff[i];
    std::vector<int32_t> adj(aoff.back());
    std::vector<int64_t> cur(aoff.begin(), aoff.end() - 1);
    for (uint64_t e : bedges) {
      uint32_t a = (uint32_t)(e >> 32), b = (uint32_t)e;
      adj[cur[bidx(a)]++] = (int32_t)b;
      adj[cur[bidx(b)]++] = (int32_t)a;
    }
    std::vector<uint8_t> used(bedges.size(), 0);
    auto eidx = [&](uint32_t x, uint32_t y) {
      uint32_t a = std::min(x, y), b = std::max(x, y);
      uint64_t key = ((uint64_t)a << 32) | b;
      return (int64_t)(std::lower_bound(bedges.begin(), bedges.end(), key) - bedges.begin());
    };
    std::vector<int32_t> walk, nxts;
    for (size_t si = 0; si < bv.size(); ++si) {
      uint32_t start = (uint32_t)bv[si];
      if (aoff[si + 1] == aoff[si]) continue;
      bool any_unused = false;
      for (int64_t q = aoff[si]; q < aoff[si + 1]; ++q)
        if (!used[eidx(start, (uint32_t)adj[q])]) any_unused = true;
      if (!any_unused) continue;
      walk.clear();
      walk.push_back((int32_t)start);
      uint32_t first = (uint32_t)adj[aoff[si]];  // smallest neighbour (lists are ascending)
      for (int64_t q = aoff[si]; q < aoff[si + 1]; ++q) first = std::min(first, (uint32_t)adj[q]);
      used[eidx(start, first)] = 1;
      uint32_t prev = start, now = first;
      walk.push_back((int32_t)now);
      for (;;) {
        int64_t ni = bidx(now);
        nxts.clear();
        for (int64_t q = aoff[ni]; q < aoff[ni + 1]; ++q) {
          uint32_t n = (uint32_t)adj[q];
          if (n != prev && !used[eidx(now, n)]) nxts.push_back((int32_t)n);
        }
        if (nxts.empty()) break;
        D3 din = pos[now] - pos[prev];
        double ln = norm3(din);
        uint32_t next = (uint32_t)nxts[0];
        if (!(ln < 1e-30)) {
          din = din / ln;
          bool have = false;
          double best = 0.0;
          for (int32_t n : nxts) {
            double d = dot3(pos[n] - pos[now], din);
            if (!have || !(d <= best)) {  // the first maximum wins (segment.rs:307-310)
              have = true;
              best = d;
              next = (uint32_t)n;
            }
          }
        }
        used[eidx(now, next)] = 1;
        prev = now;
        now = next;
        walk.push_back((int32_t)now);
        if (now == start) break;
      }
      if (walk.size() >= 4) {
        ch.loop_len.push_back((int64_t)walk.size());
        ch.loop_ids.insert(ch.loop_ids.end(), walk.begin(), walk.end());
      }
    }
  }
}

// positions and tangent frame of a chart (lscm.rs:513-516)
void chart_frame(const D3* pos, ChartOut& ch) {
  int64_t nv = (int64_t)ch.verts.size();
  ch.p3.resize(3 * nv);
  for (int64_t i = 0; i < nv; ++i) {
    D3 p = pos[ch.verts[i]];
    ch.p3[3 * i] = p.x;
    ch.p3[3 * i + 1] = p.y;
    ch.p3[3 * i + 2] = p.z;
  }
  ch.p2.resize(2 * nv);
  pca_project(nv, [&](int64_t i) { return pos[ch.verts[i]]; }, ch.p2.data());
}

// pins of a chart (lscm.rs:524-542): 4 anchors of a closed chart (needs ch.p3, ch.p2) or
// the border rectangle pass over its loops; positions by source vertex id
void chart_pins(const D3* pos, ChartOut& ch) {
  auto local = [&](int32_t v) -> int32_t {
    return (int32_t)(std::lower_bound(ch.verts.begin(), ch.verts.end(), v) - ch.verts.begin());
  };
  const int64_t nv = (int64_t)ch.verts.size();
  // pins (lscm.rs:524-542)
  ch.pinned.assign(nv, 0);
  ch.pin_uv.assign(2 * nv, 0.0);
  if (ch.loop_len.empty()) {
    // closed chart: 4 greedy farthest-point anchors pinned to their p2 (lscm.rs:210-247)
    std::vector<int64_t> chosen;
    if (nv <= 4) {
      for (int64_t i = 0; i < nv; ++i) chosen.push_back(i);
    } else {
      double min_x = std::numeric_limits<double>::max();
      for (int64_t i = 0; i < nv; ++i) min_x = fmin_rs(min_x, ch.p3[3 * i]);
      int64_t s0 = 0;
      for (int64_t i = 0; i < nv; ++i)
        if (ch.p3[3 * i] == min_x) {
          s0 = i;
          break;
        }
      chosen.push_back(s0);
      std::vector<double> dmin(nv, std::numeric_limits<double>::max());
      while (chosen.size() < 4) {
        int64_t c = chosen.back();
        D3 pc{ch.p3[3 * c], ch.p3[3 * c + 1], ch.p3[3 * c + 2]};
        for (int64_t i = 0; i < nv; ++i) {
          D3 pi{ch.p3[3 * i], ch.p3[3 * i + 1], ch.p3[3 * i + 2]};
          dmin[i] = fmin_rs(dmin[i], norm3(pi - pc));
        }
        int64_t best = 0;
        double bd = std::numeric_limits<double>::lowest();
        for (int64_t i = 0; i < nv; ++i) {
          bool taken = std::find(chosen.begin(), chosen.end(), i) != chosen.end();
          double d = taken ? -1.0 : dmin[i];
          if (d > bd) {
            bd = d;
            best = i;
          }
        }
        chosen.push_back(best);
      }
    }
    for (int64_t i : chosen) {
      ch.pinned[i] = 1;
      ch.pin_uv[2 * i] = ch.p2[2 * i];
      ch.pin_uv[2 * i + 1] = ch.p2[2 * i + 1];
    }
    return;
  }
  // border rectangle pass (lscm.rs:280-413); "last loop wins" for a vertex on two loops
  size_t nl = ch.loop_len.size();
  std::vector<int64_t> loff(nl + 1, 0);
  for (size_t l = 0; l < nl; ++l) loff[l + 1] = loff[l] + ch.loop_len[l];
  std::vector<std::vector<double>> fracs(nl);
  std::vector<double> perim(nl);
  for (size_t l = 0; l < nl; ++l) {
    const int32_t* L = ch.loop_ids.data() + loff[l];
    int64_t len = ch.loop_len[l];
    std::vector<double> seg(len > 0 ? len - 1 : 0);
    for (int64_t w = 0; w + 1 < len; ++w) seg[w] = norm3(pos[L[w + 1]] - pos[L[w]]);
    double total = 0.0;
    for (double s : seg) total += s;
    perim[l] = total;
    total = fmax_rs(total, 1e-30);
    auto& fr = fracs[l];
    fr.assign(1, 0.0);
    for (double s : seg) fr.push_back(fr.back() + s);
    for (double& x : fr) x /= total;
  }
  auto set_pin = [&](int32_t src, double u, double v) {
    int32_t li = local(src);
    ch.pinned[li] = 1;
    ch.pin_uv[2 * li] = u;
    ch.pin_uv[2 * li + 1] = v;
  };
  if (nl == 2) {
    double pm = fmax_rs(fmax_rs(0.0, perim[0]), perim[1]);
    if (std::fabs(perim[0] - perim[1]) <= 0.25 * pm) {
      // cylinder strip (lscm.rs:305-338)
      double w = 0.5 * (perim[0] + perim[1]);
      double h = ch.area3d / fmax_rs(w, 1e-30);
      auto strip_len = [&](size_t l) {
        const int32_t* L = ch.loop_ids.data() + loff[l];
        int64_t len = ch.loop_len[l];
        return (len > 1 && L[0] == L[len - 1]) ? len - 1 : len;
      };
      int64_t n0 = strip_len(0), n1 = strip_len(1);
      const int32_t* L0 = ch.loop_ids.data() + loff[0];
      const int32_t* L1 = ch.loop_ids.data() + loff[1];
      // pins is a map (later inserts overwrite): emulate by writing in reference order
      for (int64_t k = 0; k < n0; ++k) set_pin(L0[k], -w / 2.0 + w * fracs[0][k], h / 2.0);
      for (int64_t k1 = 0; k1 < n1; ++k1) {
        D3 p1 = pos[L1[k1]];
        int64_t best = 0;
        double bd = std::numeric_limits<double>::infinity();
        for (int64_t k0 = 0; k0 < n0; ++k0) {
          double d = norm3(pos[L0[k0]] - p1);
          if (d < bd) {
            bd = d;
            best = k0;
          }
        }
        set_pin(L1[k1], -w / 2.0 + w * fracs[0][best], -h / 2.0);
      }
      return;
    }
  }
  std::vector<double> sa(nl), sb(nl);
  if (nl == 1) {
    double p = perim[0], a = ch.area3d;
    if (p * p >= 16.0 * a) {
      double hs = p / 2.0;
      double d = std::sqrt(fmax_rs(hs * hs - 4.0 * a, 0.0));
      sa[0] = (hs + d) / 2.0;
      sb[0] = (hs - d) / 2.0;
    } else {
      sa[0] = sb[0] = std::sqrt(a);
    }
  } else {
    // multi-loop similarity scale (lscm.rs:351-384)
    D3 c{0.0, 0.0, 0.0};
    for (int32_t v : ch.verts) c = c + pos[v];
    c = c / (double)std::max<int64_t>(nv, 1);
    std::vector<double> dist(nl);
    for (size_t l = 0; l < nl; ++l) {
      double s = 0.0;
      for (int64_t k = 0; k < ch.loop_len[l]; ++k) s += norm3(pos[ch.loop_ids[loff[l] + k]] - c);
      dist[l] = s / (double)std::max<int64_t>(ch.loop_len[l], 1);
    }
    std::vector<size_t> order(nl);
    for (size_t l = 0; l < nl; ++l) order[l] = l;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return total_order_key(dist[a]) < total_order_key(dist[b]); });
    double denom = 0.0;
    for (size_t k = 0; k < nl; ++k) {
      double sign = ((nl - 1 - k) % 2 == 0) ? 1.0 : -1.0;
      denom += sign * perim[order[k]] * perim[order[k]];
    }
    double s = 4.0 * std::sqrt(ch.area3d / fmax_rs(std::fabs(denom), 1e-30));
    for (size_t l : order) sa[l] = sb[l] = s * perim[l] / 4.0;
  }
  std::vector<double> lp2;
  for (size_t l = 0; l < nl; ++l) {
    const int32_t* L = ch.loop_ids.data() + loff[l];
    int64_t len = ch.loop_len[l];
    bool closed = len > 1 && L[0] == L[len - 1];
    int64_t nverts = closed ? len - 1 : len;
    // winding of the 3-D walk in its own tangent frame (lscm.rs:394-406)
    lp2.assign(2 * len, 0.0);
    pca_project(len, [&](int64_t i) { return pos[L[i]]; }, lp2.data());
    double sa3 = 0.0;
    for (int64_t i = 0; i < len; ++i) {
      int64_t j = (i + 1) % len;
      sa3 += lp2[2 * i] * lp2[2 * j + 1] - lp2[2 * i + 1] * lp2[2 * j];
    }
    sa3 *= 0.5;
    for (int64_t k = 0; k < nverts; ++k) {
      double f = sa3 > 0.0 ? std::fmod(1.0 - fracs[l][k], 1.0) : fracs[l][k];
      double uv[2];
      rect_point(f, sa[l], sb[l], uv);
      set_pin(L[k], uv[0], uv[1]);
    }
  }
}

// everything after the vertex set: border, area, loops, frame, pins
void chart_finish(const MeshView& m, ChartOut& ch) {
  std::vector<uint64_t> bedges;
  chart_border(m, ch, bedges);
  chart_loops(m.pos.data(), ch, bedges);
  chart_frame(m.pos.data(), ch);
  chart_pins(m.pos.data(), ch);
}

void pack_charts(std::vector<ChartOut>& charts, Prepared& P) {
  int64_t nc = (int64_t)charts.size();
  P.vert_off.assign(nc + 1, 0);
  P.tri_off.assign(nc + 1, 0);
  P.border_off.assign(nc + 1, 0);
  P.loop_off.assign(nc + 1, 0);
  int64_t nloops = 0;
  for (int64_t c = 0; c < nc; ++c) {
    P.vert_off[c + 1] = P.vert_off[c] + (int64_t)charts[c].verts.size();
    P.tri_off[c + 1] = P.tri_off[c] + (int64_t)charts[c].faces.size();
    P.border_off[c + 1] = P.border_off[c] + (int64_t)charts[c].border.size();
    nloops += (int64_t)charts[c].loop_len.size();
    P.loop_off[c + 1] = nloops;
  }
  int64_t NV = P.vert_off[nc], NT = P.tri_off[nc];
  P.vertex_ids.resize(NV);
  P.face_ids.resize(NT);
  P.tris.resize(3 * NT);
  P.p3.resize(3 * NV);
  P.p2.resize(2 * NV);
  P.pin_uv.resize(2 * NV);
  P.pinned.resize(NV);
  P.border.resize(P.border_off[nc]);
  P.area3d.resize(nc);
  P.loop_seg.assign(nloops + 1, 0);
  {
    int64_t li = 0;
    for (int64_t c = 0; c < nc; ++c)
      for (int64_t len : charts[c].loop_len) {
        P.loop_seg[li + 1] = P.loop_seg[li] + len;
        ++li;
      }
  }
  P.loop_ids.resize(P.loop_seg[nloops]);
  parallel_for(nc, 0, [&](int64_t c) {
    ChartOut& ch = charts[c];
    int64_t v0 = P.vert_off[c], t0 = P.tri_off[c];
    std::copy(ch.verts.begin(), ch.verts.end(), P.vertex_ids.begin() + v0);
    std::copy(ch.faces.begin(), ch.faces.end(), P.face_ids.begin() + t0);
    std::copy(ch.tris.begin(), ch.tris.end(), P.tris.begin() + 3 * t0);
    std::copy(ch.p3.begin(), ch.p3.end(), P.p3.begin() + 3 * v0);
    std::copy(ch.p2.begin(), ch.p2.end(), P.p2.begin() + 2 * v0);
    std::copy(ch.pin_uv.begin(), ch.pin_uv.end(), P.pin_uv.begin() + 2 * v0);
    std::copy(ch.pinned.begin(), ch.pinned.end(), P.pinned.begin() + v0);
    std::copy(ch.border.begin(), ch.border.end(), P.border.begin() + P.border_off[c]);
    if (!ch.loop_ids.empty()) std::copy(ch.loop_ids.begin(), ch.loop_ids.end(), P.loop_ids.begin() + P.loop_seg[P.loop_off[c]]);
    P.area3d[c] = ch.area3d;
    ChartOut().faces.swap(ch.faces);  // release per-chart memory early
  });
}

std::vector<double> face_areas(const std::vector<D3>& pos, const std::vector<int32_t>& F, int threads) {
  int64_t nf = (int64_t)F.size() / 3;
  std::vector<double> a(nf);
  parallel_for((nf + 8191) / 8192, threads, [&](int64_t blk) {
    int64_t f1 = std::min(nf, (blk + 1) * 8192);
    for (int64_t f = blk * 8192; f < f1; ++f) {
      D3 e1 = pos[F[3 * f + 1]] - pos[F[3 * f]];
      D3 e2 = pos[F[3 * f + 2]] - pos[F[3 * f]];
      a[f] = 0.5 * norm3(cross(e1, e2));
    }
  });
  return a;
}

// ------------------------------------------------------------------ entry points
// Stage timings on stderr when RUV_PREP_TIMING is set.
struct StageClock {
  bool on = std::getenv("RUV_PREP_TIMING") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const char* what) {
    if (!on) return;
    auto n = std::chrono::steady_clock::now();
    std::fprintf(stderr, "prep %-22s %9.3f ms\n", what, std::chrono::duration<double, std::milli>(n - t).count());
    t = n;
  }
};

// face normals and the cut flag per face slot (segment.rs:85-137): an edge carried by one
// face is never cut, by two faces when acos(n1.n2) > angle, by more always
std::vector<uint8_t> cut_flags(const std::vector<D3>& wpos, const std::vector<int32_t>& F, const EdgeFaces& ef,
                               double angle_min_deg, int threads) {
  const int64_t wnf = (int64_t)F.size() / 3;
  std::vector<D3> nrm(wnf);
  parallel_for((wnf + 8191) / 8192, threads, [&](int64_t blk) {
    int64_t f1 = std::min(wnf, (blk + 1) * 8192);
    for (int64_t f = blk * 8192; f < f1; ++f) {
      D3 a = wpos[F[3 * f]], b = wpos[F[3 * f + 1]], c = wpos[F[3 * f + 2]];
      D3 n = cross(a - b, c - b);
      double l = norm3(n);
      nrm[f] = l < 1e-30 ? D3{0.0, 0.0, 1.0} : n / l;
    }
  });
  double th = angle_min_deg * (kPi / 180.0);
  std::vector<uint8_t> cut(3 * wnf, 0);
  parallel_for((wnf + 8191) / 8192, threads, [&](int64_t blk) {
    int64_t f1 = std::min(wnf, (blk + 1) * 8192);
    for (int64_t s = blk * 8192 * 3; s < f1 * 3; ++s) {
      int64_t cnt = ef.off[s + 1] - ef.off[s];
      double ang;
      if (cnt == 1)
        ang = 0.0;
      else if (cnt == 2) {
        double d = dot3(nrm[ef.faces[ef.off[s]]], nrm[ef.faces[ef.off[s] + 1]]);
        d = d < -1.0 ? -1.0 : (d > 1.0 ? 1.0 : d);
        ang = std::acos(d);
      } else
        ang = kPi;
      cut[s] = ang > th ? 1 : 0;
    }
  });
  return cut;
}

// face components over non-cut edges in the reference's DFS stack order (segment.rs:150-175)
std::vector<ChartOut> dfs_components(int64_t wnf, const std::vector<uint8_t>& cut, const EdgeFaces& ef) {
  std::vector<uint8_t> seen(wnf, 0);
  std::vector<ChartOut> charts;
  std::vector<int32_t> stack;
  for (int64_t f0 = 0; f0 < wnf; ++f0) {
    if (seen[f0]) continue;
    charts.emplace_back();
    auto& comp = charts.back().faces;
    stack.assign(1, (int32_t)f0);
    seen[f0] = 1;
    while (!stack.empty()) {
      int32_t f = stack.back();
      stack.pop_back();
      comp.push_back(f);
      for (int k = 0; k < 3; ++k) {
        int64_t s = 3 * (int64_t)f + k;
        if (cut[s]) continue;
        for (int64_t q = ef.off[s]; q < ef.off[s + 1]; ++q) {
          int32_t g = ef.faces[q];
          if (!seen[g]) {
            seen[g] = 1;
            stack.push_back(g);
          }
        }
      }
    }
  }
  return charts;
}

// DFS components, chart sets (from `sets`, or on the host), the per-chart finish and packing
ruv_status finish_mesh(std::vector<D3>& wpos, std::vector<int32_t>& F, EdgeFaces& ef, std::vector<uint8_t>& cut,
                       int threads, const ChartSetsFn* sets, StageClock& clk, Prepared& P, std::string& err) {
  const int64_t wnv = (int64_t)wpos.size(), wnf = (int64_t)F.size() / 3;
  P.mesh_pos.resize(3 * wnv);
  for (int64_t i = 0; i < wnv; ++i) {
    P.mesh_pos[3 * i] = wpos[i].x;
    P.mesh_pos[3 * i + 1] = wpos[i].y;
    P.mesh_pos[3 * i + 2] = wpos[i].z;
  }
  P.mesh_faces.assign(F.begin(), F.end());
  P.n_cut_slots = 0;
  for (uint8_t c : cut) P.n_cut_slots += c;
  std::vector<ChartOut> charts = dfs_components(wnf, cut, ef);
  clk.mark("components (DFS)");
  std::vector<double> farea = face_areas(wpos, F, threads);
  MeshView mv{wpos, F, ef, cut, farea};
  // biggest charts first for load balance; results land in their own slots
  std::vector<int64_t> order(charts.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int64_t)i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return charts[a].faces.size() > charts[b].faces.size(); });
  if (sets) {
    const int64_t nc = (int64_t)charts.size();
    std::vector<int64_t> cf_off(nc + 1, 0);
    for (int64_t c = 0; c < nc; ++c) cf_off[c + 1] = cf_off[c] + (int64_t)charts[c].faces.size();
    std::vector<int32_t> cf(cf_off[nc]);
    for (int64_t c = 0; c < nc; ++c) std::copy(charts[c].faces.begin(), charts[c].faces.end(), cf.begin() + cf_off[c]);
    ChartSets cs;
    if (!(*sets)(cf_off, cf, cs, err)) return RUV_ERR_INTERNAL;
    parallel_for(nc, threads, [&](int64_t c) {
      ChartOut& ch = charts[c];
      ch.verts.assign(cs.verts.begin() + cs.vert_off[c], cs.verts.begin() + cs.vert_off[c + 1]);
      ch.tris.assign(cs.tris.begin() + 3 * cf_off[c], cs.tris.begin() + 3 * cf_off[c + 1]);
    });
  } else {
    parallel_for((int64_t)charts.size(), threads, [&](int64_t i) { chart_sets(mv, charts[order[i]]); });
  }
  clk.mark("chart vertex sets");
  parallel_for((int64_t)charts.size(), threads, [&](int64_t i) { chart_finish(mv, charts[order[i]]); });
  clk.mark("chart finish");
  pack_charts(charts, P);
  clk.mark("pack");
  return RUV_OK;
}

}  // namespace

ruv_status prepare_mesh(const double* pos, int64_t nv, const int32_t* faces, int64_t nf, double weld_tol,
                        double angle_min_deg, int threads, Prepared& P, std::string& err) {
  for (int64_t i = 0; i < 3 * nf; ++i)
    if (faces[i] < 0 || faces[i] >= nv) {
      err = "face index out of range";
      return RUV_ERR_BAD_INPUT;
    }
  StageClock clk;
  std::vector<D3> wpos;
  std::vector<int32_t> F;
  weld(pos, nv, faces, nf, weld_tol, wpos, F);
  clk.mark("weld");
  int64_t wnf = (int64_t)F.size() / 3;
  for (int64_t f = 0; f < wnf; ++f)
    if (F[3 * f] == F[3 * f + 1] || F[3 * f + 1] == F[3 * f + 2] || F[3 * f] == F[3 * f + 2]) {
      err = "degenerate face with a repeated vertex";  // only possible without welding
      return RUV_ERR_BAD_INPUT;
    }
  EdgeFaces ef = build_edge_faces((int64_t)wpos.size(), F, threads);
  clk.mark("edge-faces");
  std::vector<uint8_t> cut = cut_flags(wpos, F, ef, angle_min_deg, threads);
  clk.mark("normals+cuts");
  return finish_mesh(wpos, F, ef, cut, threads, nullptr, clk, P, err);
}

ruv_status prepare_mesh_topology(std::vector<double>&& wpos3, std::vector<int32_t>&& F, std::vector<int64_t>&& ef_off,
                                 std::vector<int32_t>&& ef_faces, std::vector<uint8_t>&& cut, int threads,
                                 const ChartSetsFn* sets, Prepared& P, std::string& err) {
  StageClock clk;
  const int64_t wnf = (int64_t)F.size() / 3;
  for (int64_t f = 0; f < wnf; ++f)
    if (F[3 * f] == F[3 * f + 1] || F[3 * f + 1] == F[3 * f + 2] || F[3 * f] == F[3 * f + 2]) {
      err = "degenerate face with a repeated vertex";
      return RUV_ERR_BAD_INPUT;
    }
  std::vector<D3> wpos(wpos3.size() / 3);
  for (size_t i = 0; i < wpos.size(); ++i) wpos[i] = {wpos3[3 * i], wpos3[3 * i + 1], wpos3[3 * i + 2]};
  EdgeFaces ef;
  ef.off = std::move(ef_off);
  ef.faces = std::move(ef_faces);
  clk.mark("host copies");
  return finish_mesh(wpos, F, ef, cut, threads, sets, clk, P, err);
}

namespace {
// ------------------------------------------------------------------ seam cuts and re-cutting
// seam.rs:54-305, recut.rs:71-146 on one chart of a Prepared, in chart-local vertex indices
// (the chart's vertex ids are sorted, so local order is source-id order and every visit order
// and tie-break of the reference's id-keyed maps and sets is kept).
struct ChartRef {
  const int64_t* faces;
  int64_t nf;
  const int64_t* verts;
  int64_t nv;
  const int64_t* border;
  int64_t nb;
  bool borderless;
};

ChartRef chart_ref(const Prepared& P, int64_t c) {
  return {P.face_ids.data() + P.tri_off[c], P.tri_off[c + 1] - P.tri_off[c], P.vertex_ids.data() + P.vert_off[c],
          P.vert_off[c + 1] - P.vert_off[c], P.border.data() + P.border_off[c], P.border_off[c + 1] - P.border_off[c],
          P.loop_off[c + 1] == P.loop_off[c]};
}

int64_t local_id(const ChartRef& ch, int64_t v) { return std::lower_bound(ch.verts, ch.verts + ch.nv, v) - ch.verts; }

inline uint64_t ekey(uint64_t a, uint64_t b) { return a < b ? (a << 32) | b : (b << 32) | a; }

// undirected adjacency with 3-D lengths, edges ascending, each edge's two entries in that order
struct LocalAdj {
  std::vector<int64_t> off;
  std::vector<int32_t> to;
  std::vector<double> len;
};
LocalAdj local_adjacency(const std::vector<double>& pos, const std::vector<int32_t>& F, const ChartRef& ch) {
  std::vector<uint64_t> keys;
  keys.reserve(3 * ch.nf);
  for (int64_t q = 0; q < ch.nf; ++q) {
    const int64_t f = ch.faces[q];
    for (int k = 0; k < 3; ++k)
      keys.push_back(ekey((uint64_t)local_id(ch, F[3 * f + k]), (uint64_t)local_id(ch, F[3 * f + (k + 1) % 3])));
  }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  LocalAdj A;
  A.off.assign(ch.nv + 1, 0);
  for (uint64_t k : keys) {
    A.off[(k >> 32) + 1]++;
    A.off[(k & 0xffffffffu) + 1]++;
  }
  for (int64_t i = 0; i < ch.nv; ++i) A.off[i + 1] += A.off[i];
  A.to.resize(A.off[ch.nv]);
  A.len.resize(A.off[ch.nv]);
  std::vector<int64_t> cur(A.off.begin(), A.off.end() - 1);
  for (uint64_t k : keys) {
    const int64_t a = (int64_t)(k >> 32), b = (int64_t)(k & 0xffffffffu);
    const int64_t sa = ch.verts[a], sb = ch.verts[b];
    const D3 d = D3{pos[3 * sa], pos[3 * sa + 1], pos[3 * sa + 2]} - D3{pos[3 * sb], pos[3 * sb + 1], pos[3 * sb + 2]};
    const double l = norm3(d);
    A.to[cur[a]] = (int32_t)b;
    A.len[cur[a]++] = l;
    A.to[cur[b]] = (int32_t)a;
    A.len[cur[b]++] = l;
  }
  return A;
}

// multi-source Dijkstra: pops the smallest distance, ties the larger id; a relaxation must
// improve by more than 1e-12 (seam.rs:54-109).  Unreached vertices keep +inf.
void local_dijkstra(const LocalAdj& A, const std::vector<int32_t>& seeds, std::vector<double>& dist,
                    std::vector<int32_t>& prev) {
  const int64_t n = (int64_t)A.off.size() - 1;
  dist.assign(n, std::numeric_limits<double>::infinity());
  prev.assign(n, -1);
  struct Item {
    double d;
    int32_t v;
  };
  auto less = [](const Item& x, const Item& y) { return x.d > y.d || (x.d == y.d && x.v < y.v); };
  std::vector<Item> heap;
  for (int32_t s : seeds) {
    dist[s] = 0.0;
    heap.push_back({0.0, s});
    std::push_heap(heap.begin(), heap.end(), less);
  }
  while (!heap.empty()) {
    std::pop_heap(heap.begin(), heap.end(), less);
    const Item it = heap.back();
    heap.pop_back();
    if (dist[it.v] < it.d - 1e-12) continue;
    for (int64_t e = A.off[it.v]; e < A.off[it.v + 1]; ++e) {
      const int32_t w = A.to[e];
      const double nd = it.d + A.len[e];
      if (nd < dist[w] - 1e-12) {
        dist[w] = nd;
        prev[w] = it.v;
        heap.push_back({nd, w});
        std::push_heap(heap.begin(), heap.end(), less);
      }
    }
  }
}

// the reached vertex with the largest distance outside `skip`, the smallest id on ties
int32_t local_farthest(const std::vector<double>& dist, const std::vector<uint8_t>& skip) {
  int32_t best = -1;
  for (int32_t v = 0; v < (int32_t)dist.size(); ++v) {
    if (!std::isfinite(dist[v]) || skip[v]) continue;
    if (best < 0 || dist[v] > dist[best]) best = v;
  }
  return best;
}

std::vector<int32_t> local_path(const std::vector<int32_t>& prev, int32_t target) {
  std::vector<int32_t> path{target};
  for (int32_t cur = prev[target]; cur >= 0; cur = prev[cur]) path.push_back(cur);
  std::reverse(path.begin(), path.end());
  return path;
}

// the first minimum of pos.x over ids (ids ascending), seam.rs:177-187
int64_t min_x_of(const std::vector<double>& pos, const int64_t* ids, int64_t n) {
  int64_t best = 0;
  for (int64_t i = 1; i < n; ++i)
    if (pos[3 * ids[i]] < pos[3 * ids[best]]) best = i;
  return best;
}

// the seam tree's cut edges (seam.rs:167-231), as sorted source-id keys
std::vector<uint64_t> seam_edges(const std::vector<double>& pos, const std::vector<int32_t>& F, const ChartRef& ch,
                                 int64_t branch_count) {
  std::vector<uint64_t> out;
  if (ch.nf < 2 || ch.nv == 0) return out;
  const LocalAdj A = local_adjacency(pos, F, ch);
  std::vector<uint8_t> tree(ch.nv, 0);
  std::vector<double> dist;
  std::vector<int32_t> prev;
  local_dijkstra(A, {(int32_t)min_x_of(pos, ch.verts, ch.nv)}, dist, prev);
  const int32_t a = local_farthest(dist, tree);
  if (a < 0) return out;
  local_dijkstra(A, {a}, dist, prev);
  const int32_t b = local_farthest(dist, tree);
  if (b < 0 || a == b) return out;
  std::vector<std::vector<int32_t>> paths{local_path(prev, b)};
  for (int32_t v : paths[0]) tree[v] = 1;
  for (int64_t k = 0; k < branch_count; ++k) {
    std::vector<int32_t> seeds;
    for (int32_t v = 0; v < (int32_t)ch.nv; ++v)
      if (tree[v]) seeds.push_back(v);
    local_dijkstra(A, seeds, dist, prev);
    const int32_t f = local_farthest(dist, tree);
    if (f < 0) break;
    std::vector<int32_t> br = local_path(prev, f);
    if (br.size() < 2) break;
    for (int32_t v : br) tree[v] = 1;
    paths.push_back(std::move(br));
  }
  for (auto& pth : paths)
    for (size_t k = 0; k + 1 < pth.size(); ++k) out.push_back(ekey((uint64_t)ch.verts[pth[k]], (uint64_t)ch.verts[pth[k + 1]]));
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return out;
}

// the border-crossing chord's edges (seam.rs:246-283)
std::vector<uint64_t> chord_edges(const std::vector<double>& pos, const std::vector<int32_t>& F, const ChartRef& ch) {
  std::vector<uint64_t> out;
  if (ch.nb == 0 || ch.nf < 2) return out;
  const LocalAdj A = local_adjacency(pos, F, ch);
  const int64_t a_src = ch.border[min_x_of(pos, ch.border, ch.nb)];
  const int32_t a = (int32_t)local_id(ch, a_src);
  std::vector<double> dist;
  std::vector<int32_t> prev;
  local_dijkstra(A, {a}, dist, prev);
  int32_t best = -1;
  for (int64_t k = 0; k < ch.nb; ++k) {
    const int32_t v = (int32_t)local_id(ch, ch.border[k]);
    if (v == a || !std::isfinite(dist[v])) continue;
    if (best >= 0 && dist[v] < dist[best]) continue;
    if (best >= 0 && dist[v] == dist[best]) best = std::min(best, v);
    else best = v;
  }
  if (best < 0 || !(dist[best] > 1e-12)) return out;
  const std::vector<int32_t> pth = local_path(prev, best);
  for (size_t k = 0; k + 1 < pth.size(); ++k) out.push_back(ekey((uint64_t)ch.verts[pth[k]], (uint64_t)ch.verts[pth[k + 1]]));
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return out;
}

// triangles against the dominant winding (metrics.rs:33-56)
int64_t winding_flips(const double* uv, const int32_t* tris, int64_t nt) {
  if (nt == 0) return 0;
  auto ts = [&](int64_t t) {
    const double* u = uv + 2 * (int64_t)tris[3 * t];
    const double* v = uv + 2 * (int64_t)tris[3 * t + 1];
    const double* w = uv + 2 * (int64_t)tris[3 * t + 2];
    return (v[0] - u[0]) * (w[1] - u[1]) - (w[0] - u[0]) * (v[1] - u[1]);
  };
  double sum = 0.0;
  for (int64_t t = 0; t < nt; ++t) sum += ts(t);
  const double dom = sum < 0.0 ? -1.0 : 1.0;
  int64_t n = 0;
  for (int64_t t = 0; t < nt; ++t)
    if (ts(t) * dom <= 0.0) ++n;
  return n;
}
}  // namespace

ruv_status prepare_mesh_cut(const double* pos, int64_t nv, const int32_t* faces, int64_t nf, double weld_tol,
                            double angle_min_deg, int threads, const CutOpts& co, const UnfoldFn* unfold,
                            Prepared& P, int64_t* added_out, std::string& err) {
  *added_out = 0;
  for (int64_t i = 0; i < 3 * nf; ++i)
    if (faces[i] < 0 || faces[i] >= nv) {
      err = "face index out of range";
      return RUV_ERR_BAD_INPUT;
    }
  StageClock clk;
  std::vector<D3> wpos;
  std::vector<int32_t> F;
  weld(pos, nv, faces, nf, weld_tol, wpos, F);
  const int64_t wnf = (int64_t)F.size() / 3;
  for (int64_t f = 0; f < wnf; ++f)
    if (F[3 * f] == F[3 * f + 1] || F[3 * f + 1] == F[3 * f + 2] || F[3 * f] == F[3 * f + 2]) {
      err = "degenerate face with a repeated vertex";
      return RUV_ERR_BAD_INPUT;
    }
  EdgeFaces ef = build_edge_faces((int64_t)wpos.size(), F, threads);
  std::vector<uint8_t> cut = cut_flags(wpos, F, ef, angle_min_deg, threads);
  // the segmentation's cut set as sorted edge keys, and slot flags from a key set
  std::vector<uint64_t> cut0;
  for (int64_t sl = 0; sl < 3 * wnf; ++sl)
    if (cut[sl]) cut0.push_back(ekey((uint64_t)F[sl], (uint64_t)F[3 * (sl / 3) + (sl % 3 + 1) % 3]));
  std::sort(cut0.begin(), cut0.end());
  cut0.erase(std::unique(cut0.begin(), cut0.end()), cut0.end());
  auto flags_of = [&](const std::vector<uint64_t>& keys) {
    std::vector<uint8_t> fl(3 * wnf, 0);
    for (int64_t sl = 0; sl < 3 * wnf; ++sl)
      fl[sl] = std::binary_search(keys.begin(), keys.end(),
                                  ekey((uint64_t)F[sl], (uint64_t)F[3 * (sl / 3) + (sl % 3 + 1) % 3]))
                   ? 1
                   : 0;
    return fl;
  };
  auto rebuild = [&](const std::vector<uint64_t>& keys) -> ruv_status {
    std::vector<uint8_t> fl = flags_of(keys);
    Prepared Q;
    ruv_status st = finish_mesh(wpos, F, ef, fl, threads, nullptr, clk, Q, err);
    if (st == RUV_OK) P = std::move(Q);
    return st;
  };
  ruv_status st = finish_mesh(wpos, F, ef, cut, threads, nullptr, clk, P, err);
  if (st != RUV_OK) return st;
  // seam cut of the closed charts (seam.rs:286-305)
  if (co.seam_enable) {
    std::vector<uint64_t> all = cut0;
    for (int64_t c = 0; c + 1 < (int64_t)P.vert_off.size(); ++c) {
      const ChartRef ch = chart_ref(P, c);
      if (!ch.borderless || ch.nf < co.seam_min_faces) continue;
      for (uint64_t e : seam_edges(P.mesh_pos, P.mesh_faces, ch, co.seam_branch)) all.push_back(e);
    }
    std::sort(all.begin(), all.end());
    all.erase(std::unique(all.begin(), all.end()), all.end());
    if (all.size() != cut0.size() && (st = rebuild(all)) != RUV_OK) return st;
  }
  // re-cutting of folding charts (recut.rs:98-146), from the segmentation's cut set as the
  // reference's pipeline passes it (pipeline.rs:158)
  if (co.recut_enable) {
    if (!unfold) {
      err = "re-cutting needs an unfold";
      return RUV_ERR_BAD_INPUT;
    }
    std::vector<uint64_t> all = cut0;
    int64_t added = 0;
    for (int64_t round = 0; round < co.max_rounds; ++round) {
      if (added >= co.max_splits) break;
      std::vector<double> uv;
      if (!(*unfold)(P, uv, err)) return RUV_ERR_INTERNAL;
      const int64_t NC = (int64_t)P.vert_off.size() - 1;
      std::vector<int64_t> folds(NC);
      std::vector<int64_t> folding;
      for (int64_t c = 0; c < NC; ++c) {
        const int64_t nt = P.tri_off[c + 1] - P.tri_off[c];
        folds[c] = winding_flips(uv.data() + 2 * P.vert_off[c], P.tris.data() + 3 * P.tri_off[c], nt);
        if ((double)folds[c] / (double)std::max<int64_t>(nt, 1) > co.fold_fraction) folding.push_back(c);
      }
      if (folding.empty()) break;
      std::stable_sort(folding.begin(), folding.end(), [&](int64_t x, int64_t y) { return folds[x] > folds[y]; });
      bool grew = false;
      for (int64_t c : folding) {
        if (added >= co.max_splits) break;
        const ChartRef ch = chart_ref(P, c);
        const std::vector<uint64_t> e = ch.borderless
                                            ? seam_edges(P.mesh_pos, P.mesh_faces, ch, std::max<int64_t>(co.seam_branch, 1))
                                            : chord_edges(P.mesh_pos, P.mesh_faces, ch);
        for (uint64_t k : e) {
          auto it = std::lower_bound(all.begin(), all.end(), k);
          if (it == all.end() || *it != k) {
            all.insert(it, k);
            ++added;
            grew = true;
          }
        }
      }
      if (!grew) break;
      if ((st = rebuild(all)) != RUV_OK) return st;
      if ((int64_t)P.vert_off.size() - 1 > co.max_charts) break;
    }
    *added_out = added;
  }
  return RUV_OK;
}

double uv_signed_area(const double* uv, const int32_t* tris, int64_t nt) {  // lscm.rs:120-129
  double a = 0.0;
  for (int64_t t = 0; t < nt; ++t) {
    const double* p0 = uv + 2 * (int64_t)tris[3 * t];
    const double* p1 = uv + 2 * (int64_t)tris[3 * t + 1];
    const double* p2 = uv + 2 * (int64_t)tris[3 * t + 2];
    a += (p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]);
  }
  return a * 0.5;
}

double acos_cut_threshold(double angle_min_deg) {
  // acos(d) > th  <=>  d < d*: the smallest d in [-1, 1] with acos(d) <= th, by bisection over
  // the doubles in value order (acos is non-increasing); NaN when no such d exists or when
  // acos is not monotone near d* (callers then keep the host test)
  const double th = angle_min_deg * (kPi / 180.0);
  auto idx_of = [](double d) -> int64_t {  // order-preserving integer index of a double (-0 = +0)
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return (u >> 63) ? -(int64_t)(u & 0x7fffffffffffffffull) : (int64_t)u;
  };
  auto dbl_of = [](int64_t k) -> double {
    uint64_t u = k >= 0 ? (uint64_t)k : (0x8000000000000000ull | (uint64_t)(-k));
    double d;
    std::memcpy(&d, &u, 8);
    return d;
  };
  auto cutp = [&](double d) { return std::acos(d) > th; };
  int64_t lo = idx_of(-1.0), hi = idx_of(1.0);
  if (!cutp(dbl_of(lo))) return -1.0;                       // nothing is ever cut: d < -1 never holds
  if (cutp(dbl_of(hi))) return std::nextafter(1.0, 2.0);    // everything is cut
  while (hi - lo > 1) {  // invariant: cutp(lo), !cutp(hi)
    int64_t mid = lo + (hi - lo) / 2;
    if (cutp(dbl_of(mid))) lo = mid; else hi = mid;
  }
  for (int64_t k = 1; k <= 256; ++k)
    if ((lo - k >= idx_of(-1.0) && !cutp(dbl_of(lo - k))) || (hi + k <= idx_of(1.0) && cutp(dbl_of(hi + k))))
      return std::numeric_limits<double>::quiet_NaN();
  return dbl_of(hi);
}

ruv_status prepare_patches(int64_t np, const int64_t* vert_off, const int64_t* tri_off, const double* p3,
                           const int32_t* tris, int threads, Prepared& P, std::string& err) {
  if (np < 0 || vert_off[0] != 0 || tri_off[0] != 0) {
    err = "offsets must start at 0";
    return RUV_ERR_BAD_INPUT;
  }
  for (int64_t c = 0; c < np; ++c)
    if (vert_off[c + 1] < vert_off[c] || tri_off[c + 1] < tri_off[c]) {
      err = "offsets must be non-decreasing";
      return RUV_ERR_BAD_INPUT;
    }
  StageClock clk;
  int64_t NV = vert_off[np], NT = tri_off[np];
  std::vector<D3> pos(NV);
  for (int64_t i = 0; i < NV; ++i) pos[i] = {p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]};
  std::vector<int32_t> F(3 * NT);
  for (int64_t c = 0; c < np; ++c) {
    int64_t nvc = vert_off[c + 1] - vert_off[c];
    for (int64_t t = tri_off[c]; t < tri_off[c + 1]; ++t)
      for (int k = 0; k < 3; ++k) {
        int32_t v = tris[3 * t + k];
        if (v < 0 || v >= nvc) {
          err = "patch triangle index out of range";
          return RUV_ERR_BAD_INPUT;
        }
        F[3 * t + k] = (int32_t)(vert_off[c] + v);
      }
    for (int64_t t = tri_off[c]; t < tri_off[c + 1]; ++t)
      if (F[3 * t] == F[3 * t + 1] || F[3 * t + 1] == F[3 * t + 2] || F[3 * t] == F[3 * t + 2]) {
        err = "degenerate patch triangle";
        return RUV_ERR_BAD_INPUT;
      }
  }
  P.mesh_pos.assign(p3, p3 + 3 * NV);
  P.mesh_faces.assign(F.begin(), F.end());
  clk.mark("patch copy/validate");
  EdgeFaces ef = build_edge_faces(NV, F, threads);
  clk.mark("edge faces");
  std::vector<uint8_t> cut(3 * NT, 0);  // no segmentation: only mesh-boundary edges are border
  P.n_cut_slots = 0;
  // faces of each patch in the reference's DFS pop order (segment.rs:150-175), so a
  // connected patch gets exactly the chart the segmentation of that patch would produce
  std::vector<ChartOut> charts(np);
  std::vector<uint8_t> seen(NT, 0);
  parallel_for(np, threads, [&](int64_t c) {
    auto& comp = charts[c].faces;
    comp.reserve(tri_off[c + 1] - tri_off[c]);
    std::vector<int32_t> stack;
    for (int64_t f0 = tri_off[c]; f0 < tri_off[c + 1]; ++f0) {
      if (seen[f0]) continue;
      stack.assign(1, (int32_t)f0);
      seen[f0] = 1;
      while (!stack.empty()) {
        int32_t f = stack.back();
        stack.pop_back();
        comp.push_back(f);
        for (int k = 0; k < 3; ++k) {
          int64_t s = 3 * (int64_t)f + k;
          for (int64_t q = ef.off[s]; q < ef.off[s + 1]; ++q) {
            int32_t g = ef.faces[q];
            if (!seen[g]) {
              seen[g] = 1;
              stack.push_back(g);
            }
          }
        }
      }
    }
  });
  clk.mark("dfs");
  std::vector<double> farea = face_areas(pos, F, threads);
  clk.mark("face areas");
  MeshView mv{pos, F, ef, cut, farea};
  std::vector<int64_t> order(np);
  for (int64_t i = 0; i < np; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return charts[a].faces.size() > charts[b].faces.size(); });
  parallel_for(np, threads, [&](int64_t i) {
    chart_sets(mv, charts[order[i]]);
    chart_finish(mv, charts[order[i]]);
  });
  clk.mark("sets + finish");
  pack_charts(charts, P);
  clk.mark("pack");
  // a patch's vertices that no triangle uses would be dropped by the vertex set; require
  // every patch vertex to be used so the packed layout equals the caller's
  for (int64_t c = 0; c < np; ++c)
    if (P.vert_off[c + 1] - P.vert_off[c] != vert_off[c + 1] - vert_off[c]) {
      err = "patch " + std::to_string(c) + " has vertices no triangle uses";
      return RUV_ERR_BAD_INPUT;
    }
  return RUV_OK;
}

ruv_status prepare_patches_device(int64_t np, const int64_t* vert_off, const int64_t* tri_off, const double* p3,
                                  const int32_t* tris, int threads, const PatchDeviceFn& dev, const PatchProjectFn& proj,
                                  Prepared& P, std::string& err) {
  if (np < 0 || vert_off[0] != 0 || tri_off[0] != 0) {
    err = "offsets must start at 0";
    return RUV_ERR_BAD_INPUT;
  }
  for (int64_t c = 0; c < np; ++c)
    if (vert_off[c + 1] < vert_off[c] || tri_off[c + 1] < tri_off[c]) {
      err = "offsets must be non-decreasing";
      return RUV_ERR_BAD_INPUT;
    }
  StageClock clk;
  const int64_t NV = vert_off[np], NT = tri_off[np];
  PatchDevice D;
  ruv_status st = dev(D, err);
  if (st != RUV_OK) return st;
  clk.mark("device stages");
  const D3* pos = reinterpret_cast<const D3*>(p3);
  std::vector<ChartOut> charts(np);
  std::vector<double> frames(9 * np, 0.0);
  std::vector<int64_t> order(np);
  for (int64_t i = 0; i < np; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    return D.boff[a + 1] - D.boff[a] > D.boff[b + 1] - D.boff[b];
  });
  parallel_for(np, threads, [&](int64_t i) {
    const int64_t c = order[i];
    ChartOut& ch = charts[c];
    std::vector<uint64_t> bedges(D.bkeys.begin() + D.boff[c], D.bkeys.begin() + D.boff[c + 1]);
    chart_border_set(ch, bedges);
    ch.area3d = D.area3d[c];
    chart_loops(pos, ch, bedges);
    double cm[3][3];
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) cm[r][q] = D.cov[12 * c + 3 + 3 * r + q];
    D3 e1, e2;
    if (vert_off[c + 1] > vert_off[c]) frame_axes(cm, e1, e2);
    else e1 = e2 = D3{0.0, 0.0, 0.0};
    double* fr = frames.data() + 9 * c;
    fr[0] = D.cov[12 * c];
    fr[1] = D.cov[12 * c + 1];
    fr[2] = D.cov[12 * c + 2];
    fr[3] = e1.x;
    fr[4] = e1.y;
    fr[5] = e1.z;
    fr[6] = e2.x;
    fr[7] = e2.y;
    fr[8] = e2.z;
  });
  clk.mark("borders + loops + axes");
  P.p2.resize(2 * NV);
  st = proj(frames, P.p2, err);
  if (st != RUV_OK) return st;
  clk.mark("projection");
  // pins (the closed charts' anchors read the chart's p3 and p2)
  P.pinned.resize(NV);
  P.pin_uv.resize(2 * NV);
  parallel_for(np, threads, [&](int64_t i) {
    const int64_t c = order[i];
    ChartOut& ch = charts[c];
    const int64_t v0 = vert_off[c], nv = vert_off[c + 1] - v0;
    ch.verts.resize(nv);
    for (int64_t k = 0; k < nv; ++k) ch.verts[k] = (int32_t)(v0 + k);
    if (ch.loop_len.empty()) {
      ch.p3.assign(p3 + 3 * v0, p3 + 3 * (v0 + nv));
      ch.p2.assign(P.p2.begin() + 2 * v0, P.p2.begin() + 2 * (v0 + nv));
    }
    chart_pins(pos, ch);
    std::copy(ch.pinned.begin(), ch.pinned.end(), P.pinned.begin() + v0);
    std::copy(ch.pin_uv.begin(), ch.pin_uv.end(), P.pin_uv.begin() + 2 * v0);
    std::vector<int32_t>().swap(ch.verts);
    std::vector<uint8_t>().swap(ch.pinned);
    std::vector<double>().swap(ch.pin_uv);
  });
  clk.mark("pins");
  // packing: the charts are the patches, in order; their vertices the patch's, ascending
  P.mesh_pos.assign(p3, p3 + 3 * NV);
  P.p3 = P.mesh_pos;
  P.mesh_faces.resize(3 * NT);
  P.n_cut_slots = 0;
  P.vert_off.assign(vert_off, vert_off + np + 1);
  P.tri_off.assign(tri_off, tri_off + np + 1);
  P.vertex_ids.resize(NV);
  P.face_ids.resize(NT);
  P.tris = std::move(D.tris);
  P.area3d = std::move(D.area3d);
  parallel_for(np, threads, [&](int64_t c) {
    const int64_t v0 = vert_off[c];
    for (int64_t k = v0; k < vert_off[c + 1]; ++k) P.vertex_ids[k] = k;
    for (int64_t t = tri_off[c]; t < tri_off[c + 1]; ++t) P.face_ids[t] = D.order[t];
    for (int64_t t = 3 * tri_off[c]; t < 3 * tri_off[c + 1]; ++t) P.mesh_faces[t] = (int32_t)(v0 + tris[t]);
  });
  P.border_off.assign(np + 1, 0);
  P.loop_off.assign(np + 1, 0);
  int64_t nloops = 0;
  for (int64_t c = 0; c < np; ++c) {
    P.border_off[c + 1] = P.border_off[c] + (int64_t)charts[c].border.size();
    nloops += (int64_t)charts[c].loop_len.size();
    P.loop_off[c + 1] = nloops;
  }
  P.border.resize(P.border_off[np]);
  P.loop_seg.assign(nloops + 1, 0);
  {
    int64_t li = 0;
    for (int64_t c = 0; c < np; ++c)
      for (int64_t len : charts[c].loop_len) {
        P.loop_seg[li + 1] = P.loop_seg[li] + len;
        ++li;
      }
  }
  P.loop_ids.resize(P.loop_seg[nloops]);
  for (int64_t c = 0; c < np; ++c) {
    std::copy(charts[c].border.begin(), charts[c].border.end(), P.border.begin() + P.border_off[c]);
    if (!charts[c].loop_ids.empty())
      std::copy(charts[c].loop_ids.begin(), charts[c].loop_ids.end(), P.loop_ids.begin() + P.loop_seg[P.loop_off[c]]);
  }
  clk.mark("pack");
  return RUV_OK;
}

}  // namespace ruv
