// ORACLE — test infrastructure only. Never linked into, loaded by, or called from the
// product library (researchuv_gb300 / libruv). Only tests/, __graft_entry__.smoke() and
// bench.py's cpu_baseline / reference legs use it, and only to check or time against.
//
// A CPU restatement of ResearchUV's per-chart LSCM unfold path, written from the
// reference's Rust source semantics (paths relative to crates/, `researchuv-` dropped):
//   weld                 unwrap/src/weld.rs:19-57
//   segment / charts     unwrap/src/segment.rs:61-331
//   eig3                 unwrap/src/lscm_eig.rs:13-66
//   tangent_frame        unwrap/src/lscm.rs:152-183
//   rect_point           unwrap/src/lscm.rs:187-204
//   anchor_ids           unwrap/src/lscm.rs:210-247
//   edge_weights         unwrap/src/lscm.rs:252-274
//   border_targets       unwrap/src/lscm.rs:280-413
//   unfold_chart driver  unwrap/src/lscm.rs:512-727 (default path, and KeepMetric's area row
//                        lscm.rs:120-155, :544-568, :642-676 solved by the LU each iteration)
//   Sparse + LU          unwrap/src/sparse.rs:19-265
//   meshgen fixtures     unwrap/src/meshgen.rs:12-198
//   chart_distortion     unwrap/src/metrics.rs:41-141
//   vector arithmetic    math/src/vec.rs:100-124
//   rectangularize       unwrap/src/metrics.rs:147-227
//   IC(0) + colouring    gpu/src/precond.rs:49-123 (graph_coloring, color_permutation,
//                        permute_csr), :145-262 (factor_ic0, tri_levels, transpose_lower)
//   fixed-pin system     lscm.rs:594-676 with the pins given (the map the adjoint
//                        differentiates), its reverse pass and the metrics.rs:73-128
//                        distortion loss with its gradient (forward-mode duals, 15 seeds)
//
// Arithmetic follows the Rust evaluation order (left-to-right sums, no FMA contraction:
// compile with -ffp-contract=off) so that results are bit-identical to the reference on
// the same host libm.  Parity pinning: the reference (pure Rust) cannot be built in this
// environment, so this restatement is pinned against the known answers of the reference's
// own tests (unwrap/tests/parity.rs, unwrap/src/sparse.rs tests, lscm_eig.rs tests,
// meshgen.rs tests, segment.rs tests, weld.rs tests), transcribed with citations into
// tests/golden/reference_known_answers.json.
//
// Interface: a "bag" of named f64 / i64 arrays behind an opaque handle (ctypes-friendly).

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <queue>
#include <set>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

namespace {

// ---------------------------------------------------------------- vec.rs arithmetic
struct V3 {
  double x, y, z;
};
struct V2 {
  double u, v;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 divs(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross_v(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double len3(V3 a) { return std::sqrt(dot(a, a)); }
// Vec3::cross(a, b, c) = (a - b) x (c - b)   (math/src/vec.rs:100-102)
inline V3 cross3(V3 a, V3 b, V3 c) { return cross_v(sub(a, b), sub(c, b)); }
inline V2 sub2(V2 a, V2 b) { return {a.u - b.u, a.v - b.v}; }

// Rust f64::max / f64::min (NaN-ignoring maxNum/minNum).
inline double rmax(double a, double b) {
  if (std::isnan(a)) return b;
  if (std::isnan(b)) return a;
  return a > b ? a : b;
}
inline double rmin(double a, double b) {
  if (std::isnan(a)) return b;
  if (std::isnan(b)) return a;
  return a < b ? a : b;
}
// Rust f64::total_cmp as a strict-weak "less".
inline int64_t total_key(double a) {
  int64_t i;
  std::memcpy(&i, &a, 8);
  i ^= (int64_t)(((uint64_t)(i >> 63)) >> 1);
  return i;
}
// Rust `x as i64` (saturating, NaN -> 0).
inline int64_t sat_i64(double x) {
  if (std::isnan(x)) return 0;
  if (x >= 9.2233720368547758e18) return std::numeric_limits<int64_t>::max();
  if (x <= -9.2233720368547758e18) return std::numeric_limits<int64_t>::min();
  return (int64_t)x;
}

constexpr double EPS_DEGENERATE = 1.1754943508222875e-38;  // lscm.rs:36
constexpr double PI = 3.14159265358979323846;

// ---------------------------------------------------------------- meshes
struct Mesh {
  std::vector<V3> pos;
  std::vector<std::array<uint32_t, 3>> faces;
};

// weld.rs:19-57 — rounding-grid weld, first occurrence is canonical, collapsed faces dropped.
Mesh weld(const Mesh& in, double tol) {
  if (tol <= 0.0) return in;
  struct KeyHash {
    size_t operator()(const std::tuple<int64_t, int64_t, int64_t>& k) const {
      uint64_t h = (uint64_t)std::get<0>(k) * 0x9E3779B97F4A7C15ull;
      h ^= (uint64_t)std::get<1>(k) + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
      h ^= (uint64_t)std::get<2>(k) + 0x94D049BB133111EBull + (h << 6) + (h >> 2);
      return (size_t)h;
    }
  };
  double inv = 1.0 / tol;
  std::unordered_map<std::tuple<int64_t, int64_t, int64_t>, uint32_t, KeyHash> canon;
  canon.reserve(in.pos.size() * 2);
  std::vector<uint32_t> remap(in.pos.size());
  Mesh out;
  for (size_t i = 0; i < in.pos.size(); ++i) {
    V3 p = in.pos[i];
    auto key = std::make_tuple(sat_i64(std::round(p.x * inv)), sat_i64(std::round(p.y * inv)),
                               sat_i64(std::round(p.z * inv)));
    auto it = canon.find(key);
    uint32_t c;
    if (it == canon.end()) {
      c = (uint32_t)out.pos.size();
      canon.emplace(key, c);
      out.pos.push_back(p);
    } else {
      c = it->second;
    }
    remap[i] = c;
  }
  for (auto& f : in.faces) {
    std::array<uint32_t, 3> g{remap[f[0]], remap[f[1]], remap[f[2]]};
    if (g[0] != g[1] && g[1] != g[2] && g[0] != g[2]) out.faces.push_back(g);
  }
  return out;
}

// ---------------------------------------------------------------- segment.rs
using EdgeKey = std::pair<uint32_t, uint32_t>;
inline EdgeKey edge_key(uint32_t a, uint32_t b) { return a < b ? EdgeKey{a, b} : EdgeKey{b, a}; }

struct Chart {
  std::vector<size_t> face_ids;
  std::vector<uint32_t> vertex_ids;
  std::vector<std::array<uint32_t, 3>> tris;
  std::vector<uint32_t> border;
  std::vector<std::vector<uint32_t>> border_loops;
  double area3d = 0.0;
  long local_of(uint32_t v) const {
    auto it = std::lower_bound(vertex_ids.begin(), vertex_ids.end(), v);
    if (it != vertex_ids.end() && *it == v) return (long)(it - vertex_ids.begin());
    return -1;
  }
};

std::vector<double> face_areas3d(const Mesh& m) {  // segment.rs:61-70
  std::vector<double> a(m.faces.size());
  for (size_t f = 0; f < m.faces.size(); ++f) {
    V3 e1 = sub(m.pos[m.faces[f][1]], m.pos[m.faces[f][0]]);
    V3 e2 = sub(m.pos[m.faces[f][2]], m.pos[m.faces[f][0]]);
    a[f] = 0.5 * len3(cross_v(e1, e2));
  }
  return a;
}

std::map<EdgeKey, std::vector<size_t>> edge_faces(const Mesh& m) {  // segment.rs:73-81
  std::map<EdgeKey, std::vector<size_t>> ef;
  for (size_t fi = 0; fi < m.faces.size(); ++fi) {
    auto& f = m.faces[fi];
    uint32_t a = f[0], b = f[1], c = f[2];
    ef[edge_key(a, b)].push_back(fi);
    ef[edge_key(b, c)].push_back(fi);
    ef[edge_key(c, a)].push_back(fi);
  }
  return ef;
}

V3 face_normal_unit(const Mesh& m, size_t fi) {  // segment.rs:104-117
  auto& f = m.faces[fi];
  V3 n = cross3(m.pos[f[0]], m.pos[f[1]], m.pos[f[2]]);
  double l = len3(n);
  if (l < 1e-30) return {0.0, 0.0, 1.0};
  return divs(n, l);
}

std::vector<std::vector<uint32_t>> chart_border_loops(const Mesh& mesh,
                                                      const std::vector<size_t>& comp,
                                                      const std::set<EdgeKey>& cut,
                                                      const std::set<EdgeKey>& mbnd,
                                                      const std::map<uint32_t, uint32_t>& vid) {
  // segment.rs:227-331 — keep-going-straight boundary walk.
  std::set<EdgeKey> bnd_edges;
  for (size_t f : comp) {
    auto& t = mesh.faces[f];
    uint32_t pr[3][2] = {{t[0], t[1]}, {t[1], t[2]}, {t[2], t[0]}};
    for (auto& e : pr) {
      EdgeKey k = edge_key(e[0], e[1]);
      if (cut.count(k) || mbnd.count(k)) bnd_edges.insert(k);
    }
  }
  std::vector<std::vector<uint32_t>> loops;
  if (bnd_edges.empty()) return loops;
  std::map<uint32_t, std::vector<uint32_t>> adj;
  for (auto& e : bnd_edges) {
    if (vid.count(e.first) && vid.count(e.second)) {
      adj[e.first].push_back(e.second);
      adj[e.second].push_back(e.first);
    }
  }
  std::set<EdgeKey> used;
  std::vector<uint32_t> starts;
  for (auto& kv : adj) starts.push_back(kv.first);
  for (uint32_t start : starts) {
    bool has_unused = false;
    for (uint32_t n : adj[start])
      if (!used.count(edge_key(start, n))) {
        has_unused = true;
        break;
      }
    if (!has_unused) continue;
    std::vector<uint32_t> loop_v{start};
    uint32_t cur = start;
    std::vector<uint32_t> cands = adj[start];
    std::sort(cands.begin(), cands.end());
    if (cands.empty()) continue;
    uint32_t first = cands[0];
    used.insert(edge_key(cur, first));
    uint32_t prev = cur;
    cur = first;
    loop_v.push_back(cur);
    for (;;) {
      std::vector<uint32_t> nxts;
      auto it = adj.find(cur);
      if (it != adj.end())
        for (uint32_t n : it->second)
          if (n != prev && !used.count(edge_key(cur, n))) nxts.push_back(n);
      if (nxts.empty()) break;
      V3 d_in = sub(mesh.pos[cur], mesh.pos[prev]);
      double ln = len3(d_in);
      uint32_t next;
      if (ln < 1e-30) {
        next = nxts[0];
      } else {
        V3 din = divs(d_in, ln);
        bool have = false;
        double bd = 0.0;
        uint32_t bn = nxts[0];
        for (uint32_t n : nxts) {
          double dt = dot(sub(mesh.pos[n], mesh.pos[cur]), din);
          if (have && dt <= bd) continue;
          have = true;
          bd = dt;
          bn = n;
        }
        next = bn;
      }
      used.insert(edge_key(cur, next));
      prev = cur;
      cur = next;
      loop_v.push_back(cur);
      if (cur == start) break;
    }
    if (loop_v.size() >= 4) loops.push_back(std::move(loop_v));
  }
  return loops;
}

std::vector<Chart> build_charts(const Mesh& mesh, const std::set<EdgeKey>& cut);

// segment.rs:85-102 (dihedrals), :130-140 (segment); the charts by build_charts below
std::vector<Chart> segment(const Mesh& mesh, double angle_min_deg, size_t* n_cut_out,
                           std::set<EdgeKey>* cut_out = nullptr) {
  double th = angle_min_deg * (PI / 180.0);
  auto ef = edge_faces(mesh);
  std::set<EdgeKey> cut, mbnd;
  for (auto& kv : ef) {
    double ang;
    if (kv.second.size() == 1) {
      ang = 0.0;
      mbnd.insert(kv.first);
    } else if (kv.second.size() == 2) {
      V3 n1 = face_normal_unit(mesh, kv.second[0]);
      V3 n2 = face_normal_unit(mesh, kv.second[1]);
      double d = dot(n1, n2);
      if (d < -1.0) d = -1.0;
      if (d > 1.0) d = 1.0;
      ang = std::acos(d);
    } else {
      ang = PI;
    }
    if (ang > th) cut.insert(kv.first);
  }
  if (n_cut_out) *n_cut_out = cut.size();
  if (cut_out) *cut_out = cut;
  return build_charts(mesh, cut);
}

// segment.rs:143-223: face components over non-cut edges (DFS stack order), vertex sets,
// local triangles, border (cut or mesh-boundary edges), loops, area
std::vector<Chart> build_charts(const Mesh& mesh, const std::set<EdgeKey>& cut) {
  auto ef = edge_faces(mesh);
  std::set<EdgeKey> mbnd;
  for (auto& kv : ef)
    if (kv.second.size() == 1) mbnd.insert(kv.first);
  auto areas = face_areas3d(mesh);
  size_t nf = mesh.faces.size();
  std::vector<char> seen(nf, 0);
  std::vector<Chart> charts;
  for (size_t fi = 0; fi < nf; ++fi) {
    if (seen[fi]) continue;
    std::vector<size_t> stack{fi};
    seen[fi] = 1;
    std::vector<size_t> comp;
    while (!stack.empty()) {
      size_t f = stack.back();
      stack.pop_back();
      comp.push_back(f);
      auto& t = mesh.faces[f];
      uint32_t pr[3][2] = {{t[0], t[1]}, {t[1], t[2]}, {t[2], t[0]}};
      for (auto& e : pr) {
        EdgeKey k = edge_key(e[0], e[1]);
        if (cut.count(k)) continue;
        auto it = ef.find(k);
        if (it == ef.end()) continue;
        for (size_t g : it->second)
          if (!seen[g]) {
            seen[g] = 1;
            stack.push_back(g);
          }
      }
    }
    Chart ch;
    std::set<uint32_t> vset;
    for (size_t f : comp)
      for (uint32_t v : mesh.faces[f]) vset.insert(v);
    ch.vertex_ids.assign(vset.begin(), vset.end());
    std::map<uint32_t, uint32_t> vid;
    for (size_t i = 0; i < ch.vertex_ids.size(); ++i) vid[ch.vertex_ids[i]] = (uint32_t)i;
    for (size_t f : comp) {
      auto& t = mesh.faces[f];
      ch.tris.push_back({vid[t[0]], vid[t[1]], vid[t[2]]});
    }
    std::set<uint32_t> bnd;
    for (size_t f : comp) {
      auto& t = mesh.faces[f];
      uint32_t pr[3][2] = {{t[0], t[1]}, {t[1], t[2]}, {t[2], t[0]}};
      for (auto& e : pr) {
        EdgeKey k = edge_key(e[0], e[1]);
        if (cut.count(k) || mbnd.count(k)) {
          bnd.insert(e[0]);
          bnd.insert(e[1]);
        }
      }
    }
    ch.border.assign(bnd.begin(), bnd.end());
    ch.border_loops = chart_border_loops(mesh, comp, cut, mbnd, vid);
    double a = 0.0;
    for (size_t f : comp) a += areas[f];
    ch.area3d = a;
    ch.face_ids = std::move(comp);
    charts.push_back(std::move(ch));
  }
  return charts;
}

// ---------------------------------------------------------------- lscm_eig.rs:13-66
void eig3(const double m[3][3], double w[3], double v[3][3]) {
  double a[3][3];
  std::memcpy(a, m, sizeof(a));
  double vv[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int sweep = 0; sweep < 64; ++sweep) {
    int p = 0, q = 1;
    double max_off = std::fabs(a[0][1]);
    int pairs[2][2] = {{0, 2}, {1, 2}};
    for (auto& pq : pairs) {
      double x = std::fabs(a[pq[0]][pq[1]]);
      if (x > max_off) {
        max_off = x;
        p = pq[0];
        q = pq[1];
      }
    }
    if (max_off <= 1e-300) break;
    double apq = a[p][q], app = a[p][p], aqq = a[q][q];
    double theta = 0.5 * std::atan2(2.0 * apq, app - aqq);
    double c = std::cos(theta), s = std::sin(theta);
    for (int r = 0; r < 3; ++r) {
      if (r == p || r == q) continue;
      double ar_p = c * a[r][p] + s * a[r][q];
      double ar_q = -s * a[r][p] + c * a[r][q];
      a[r][p] = ar_p;
      a[p][r] = ar_p;
      a[r][q] = ar_q;
      a[q][r] = ar_q;
    }
    a[p][p] = c * c * app + 2.0 * s * c * apq + s * s * aqq;
    a[q][q] = s * s * app - 2.0 * s * c * apq + c * c * aqq;
    a[p][q] = 0.0;
    a[q][p] = 0.0;
    for (int k = 0; k < 3; ++k) {
      double vp = vv[p][k], vq = vv[q][k];
      vv[p][k] = c * vp - s * vq;
      vv[q][k] = s * vp + c * vq;
    }
  }
  w[0] = a[0][0];
  w[1] = a[1][1];
  w[2] = a[2][2];
  std::memcpy(v, vv, sizeof(vv));
}

// lscm.rs:152-183
std::vector<V2> tangent_frame(const std::vector<V3>& p3) {
  size_t n = p3.size();
  std::vector<V2> out;
  if (n == 0) return out;
  V3 c{0.0, 0.0, 0.0};
  for (auto& p : p3) c = add(c, p);
  c = divs(c, (double)n);
  std::vector<V3> d(n);
  for (size_t i = 0; i < n; ++i) d[i] = sub(p3[i], c);
  double cm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (auto& v : d) {
    double vi[3] = {v.x, v.y, v.z};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) cm[i][j] += vi[i] * vi[j];
  }
  double w[3], vv[3][3];
  eig3(cm, w, vv);
  int idx[3] = {0, 1, 2};
  std::stable_sort(idx, idx + 3, [&](int a, int b) { return total_key(w[b]) < total_key(w[a]); });
  V3 e1{vv[0][idx[0]], vv[1][idx[0]], vv[2][idx[0]]};
  V3 e2{vv[0][idx[1]], vv[1][idx[1]], vv[2][idx[1]]};
  out.resize(n);
  for (size_t i = 0; i < n; ++i) out[i] = {dot(d[i], e1), dot(d[i], e2)};
  return out;
}

// lscm.rs:187-204
V2 rect_point(double f, double a, double b) {
  double p2 = 2.0 * (a + b);
  double t = std::fmod(f, 1.0) * p2;
  double x0 = a / 2.0, y0 = -b / 2.0;
  if (t < a) return {x0 - t, y0};
  t -= a;
  if (t < b) return {-a / 2.0, y0 + t};
  t -= b;
  if (t < a) return {-a / 2.0 + t, b / 2.0};
  t -= a;
  return {a / 2.0, b / 2.0 - t};
}

// lscm.rs:210-247
std::vector<size_t> anchor_ids(const std::vector<V3>& p3, size_t n) {
  size_t n3 = p3.size();
  std::vector<size_t> chosen;
  if (n3 <= n) {
    for (size_t i = 0; i < n3; ++i) chosen.push_back(i);
    return chosen;
  }
  double min_x = std::numeric_limits<double>::max();
  for (auto& q : p3) min_x = rmin(min_x, q.x);
  size_t start = 0;
  for (size_t i = 0; i < n3; ++i)
    if (p3[i].x == min_x) {
      start = i;
      break;
    }
  chosen.push_back(start);
  while (chosen.size() < n) {
    std::vector<double> d(n3);
    for (size_t i = 0; i < n3; ++i) {
      double m = std::numeric_limits<double>::max();
      for (size_t c : chosen) m = rmin(m, len3(sub(p3[i], p3[c])));
      d[i] = m;
    }
    for (size_t c : chosen) d[c] = -1.0;
    size_t bi = 0;
    double bd = std::numeric_limits<double>::lowest();
    for (size_t i = 0; i < n3; ++i)
      if (d[i] > bd) {
        bi = i;
        bd = d[i];
      }
    chosen.push_back(bi);
  }
  std::sort(chosen.begin(), chosen.end());
  return chosen;
}

// lscm.rs:252-274
std::map<std::pair<size_t, size_t>, double> edge_weights(const std::vector<V3>& p3,
                                                         const std::vector<std::array<uint32_t, 3>>& tris) {
  std::map<std::pair<size_t, size_t>, double> ew;
  for (auto& t : tris) {
    size_t i = t[0], j = t[1], k = t[2];
    size_t cs[3][3] = {{i, j, k}, {j, k, i}, {k, i, j}};
    for (auto& c : cs) {
      size_t e0 = c[0], e1 = c[1], o = c[2];
      V3 a1 = sub(p3[e1], p3[o]);
      V3 a2 = sub(p3[e0], p3[o]);
      double la = len3(a1), lb = len3(a2);
      if (la <= EPS_DEGENERATE || lb <= EPS_DEGENERATE) continue;
      double s = len3(cross_v(a1, a2)) / (la * lb);
      if (s <= EPS_DEGENERATE) continue;
      double cot = rmax((dot(a1, a2) / (la * lb)) / s, 0.0);
      auto key = std::make_pair(std::min(e0, e1), std::max(e0, e1));
      auto it = ew.find(key);
      if (it == ew.end()) it = ew.emplace(key, 0.0).first;
      it->second += cot;
    }
  }
  return ew;
}

// lscm.rs:280-413
std::map<uint32_t, V2> border_targets(const Mesh& mesh, const Chart& chart,
                                      const std::vector<std::vector<uint32_t>>& loops) {
  double area3d = chart.area3d;
  std::vector<std::vector<double>> fracs;
  std::vector<double> perims;
  for (auto& l : loops) {
    std::vector<double> segs;
    for (size_t w = 0; w + 1 < l.size(); ++w) segs.push_back(len3(sub(mesh.pos[l[w + 1]], mesh.pos[l[w]])));
    double total = 0.0;
    for (double s : segs) total += s;
    total = rmax(total, 1e-30);
    std::vector<double> fr{0.0};
    for (double s : segs) fr.push_back(fr.back() + s);
    for (double& f : fr) f /= total;
    fracs.push_back(fr);
    double per = 0.0;
    for (double s : segs) per += s;
    perims.push_back(per);
  }
  size_t n = loops.size();
  std::map<uint32_t, V2> pins;
  if (n == 2) {
    double pm = 0.0;
    for (double p : perims) pm = rmax(pm, p);
    if (std::fabs(perims[0] - perims[1]) <= 0.25 * pm) {
      double w = 0.5 * (perims[0] + perims[1]);
      double h = area3d / rmax(w, 1e-30);
      auto strip = [](const std::vector<uint32_t>& l) {
        if (l.size() > 1 && l.front() == l.back()) return std::vector<uint32_t>(l.begin(), l.end() - 1);
        return l;
      };
      auto l0u = strip(loops[0]);
      auto l1u = strip(loops[1]);
      size_t f0n = std::min(l0u.size(), fracs[0].size());
      for (size_t k = 0; k < l0u.size(); ++k) pins[l0u[k]] = {-w / 2.0 + w * fracs[0][k], h / 2.0};
      (void)f0n;
      for (uint32_t v1 : l1u) {
        V3 p1 = mesh.pos[v1];
        size_t best = 0;
        double best_d = std::numeric_limits<double>::infinity();
        for (size_t k0 = 0; k0 < l0u.size(); ++k0) {
          double d = len3(sub(mesh.pos[l0u[k0]], p1));
          if (d < best_d) {
            best_d = d;
            best = k0;
          }
        }
        pins[v1] = {-w / 2.0 + w * fracs[0][best], -h / 2.0};
      }
      return pins;
    }
  }
  std::vector<std::pair<double, double>> sides;
  if (n == 1) {
    double p = perims[0], a = area3d;
    if (p * p >= 16.0 * a) {
      double s_ = p / 2.0;
      double d = std::sqrt(rmax(s_ * s_ - 4.0 * a, 0.0));
      sides.push_back({(s_ + d) / 2.0, (s_ - d) / 2.0});
    } else {
      double s = std::sqrt(a);
      sides.push_back({s, s});
    }
  } else {
    V3 c{0, 0, 0};
    size_t nv = chart.vertex_ids.size();
    for (uint32_t v : chart.vertex_ids) c = add(c, mesh.pos[v]);
    c = divs(c, (double)std::max<size_t>(nv, 1));
    std::vector<double> dists;
    for (auto& l : loops) {
      double s = 0.0;
      for (uint32_t v : l) s += len3(sub(mesh.pos[v], c));
      dists.push_back(s / (double)std::max<size_t>(l.size(), 1));
    }
    std::vector<size_t> order(n);
    for (size_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return total_key(dists[a]) < total_key(dists[b]); });
    double denom = 0.0;
    for (size_t k = 0; k < n; ++k) {
      double sign = ((n - 1 - k) % 2 == 0) ? 1.0 : -1.0;
      denom += sign * perims[order[k]] * perims[order[k]];
    }
    double s = 4.0 * std::sqrt(area3d / rmax(std::fabs(denom), 1e-30));
    sides.assign(n, {0.0, 0.0});
    for (size_t li : order) {
      double side = s * perims[li] / 4.0;
      sides[li] = {side, side};
    }
  }
  for (size_t li = 0; li < n; ++li) {
    auto& l = loops[li];
    double a = sides[li].first, b = sides[li].second;
    auto& fr = fracs[li];
    bool closed = l.size() > 1 && l.front() == l.back();
    size_t nverts = closed ? l.size() - 1 : l.size();
    std::vector<V3> lp;
    for (uint32_t v : l) lp.push_back(mesh.pos[v]);
    auto p2loop = tangent_frame(lp);
    double sa3 = 0.0;
    for (size_t i = 0; i < p2loop.size(); ++i) {
      size_t j = (i + 1) % p2loop.size();
      sa3 += p2loop[i].u * p2loop[j].v - p2loop[i].v * p2loop[j].u;
    }
    sa3 *= 0.5;
    for (size_t k = 0; k < nverts; ++k) {
      double f = sa3 > 0.0 ? std::fmod(1.0 - fr[k], 1.0) : fr[k];
      pins[l[k]] = rect_point(f, a, b);
    }
  }
  return pins;
}

// ---------------------------------------------------------------- sparse.rs:19-265
struct Sparse {
  size_t n;
  std::vector<std::map<size_t, double>> rows;
  explicit Sparse(size_t n_) : n(n_), rows(n_) {}
  void add(size_t r, size_t c, double v) {  // sparse.rs:47-52
    if (v != 0.0) rows[r][c] += v;
  }
};

struct LU {
  std::vector<size_t> perm;
  std::vector<std::pair<size_t, size_t>> swaps;
  std::map<std::pair<size_t, size_t>, double> lu;
};

// sparse.rs:91-95, :120-214. Same arithmetic and visit order as the reference; the scans
// over all rows / all of `lu` are replaced by indexed lookups that visit the same entries
// in the same (ascending) order.
LU factorize(const Sparse& S) {
  size_t n = S.n;
  LU F;
  F.perm.resize(n);
  for (size_t i = 0; i < n; ++i) F.perm[i] = i;
  std::stable_sort(F.perm.begin(), F.perm.end(), [&](size_t a, size_t b) {
    return std::make_pair(S.rows[a].size(), a) < std::make_pair(S.rows[b].size(), b);
  });
  std::vector<size_t> inv(n);
  for (size_t i = 0; i < n; ++i) inv[F.perm[i]] = i;
  std::vector<std::map<size_t, double>> a(n);
  std::vector<std::set<size_t>> colrows(n);  // rows r that hold a key at column c
  for (size_t i = 0; i < n; ++i)
    for (auto& kv : S.rows[F.perm[i]]) {
      a[i][inv[kv.first]] = kv.second;
      colrows[inv[kv.first]].insert(i);
    }
  for (size_t k = 0; k < n; ++k) {
    size_t piv = k;
    double piv_val = 0.0;
    for (auto it = colrows[k].lower_bound(k); it != colrows[k].end(); ++it) {
      size_t r = *it;
      auto f = a[r].find(k);
      double v = std::fabs(f == a[r].end() ? 0.0 : f->second);
      if (v > piv_val) {
        piv_val = v;
        piv = r;
      }
    }
    if (piv_val < 1e-300) continue;
    if (piv != k) {
      F.swaps.push_back({k, piv});
      for (auto& kv : a[k]) colrows[kv.first].erase(k);
      for (auto& kv : a[piv]) colrows[kv.first].erase(piv);
      std::swap(a[k], a[piv]);
      for (auto& kv : a[k]) colrows[kv.first].insert(k);
      for (auto& kv : a[piv]) colrows[kv.first].insert(piv);
      // swap the L history (entries with column < k) of rows k and piv
      std::vector<std::pair<std::pair<size_t, size_t>, double>> moved;
      for (size_t r : {k, piv}) {
        auto lo = F.lu.lower_bound({r, 0});
        auto hi = F.lu.lower_bound({r, k});
        for (auto it = lo; it != hi; ++it) moved.push_back(*it);
        F.lu.erase(lo, hi);
      }
      for (auto& mv : moved) {
        size_t r2 = mv.first.first == k ? piv : k;
        F.lu[{r2, mv.first.second}] = mv.second;
      }
    }
    double pivot;
    {
      auto f = a[k].find(k);
      pivot = f == a[k].end() ? 0.0 : f->second;
    }
    F.lu[{k, k}] = pivot;
    std::vector<std::pair<size_t, double>> u_part;
    for (auto it = a[k].upper_bound(k); it != a[k].end(); ++it) u_part.push_back(*it);
    for (auto& cv : u_part)
      if (cv.second != 0.0) F.lu[{k, cv.first}] = cv.second;
    std::vector<size_t> rlist;
    for (auto it = colrows[k].upper_bound(k); it != colrows[k].end(); ++it) rlist.push_back(*it);
    for (size_t r : rlist) {
      auto f = a[r].find(k);
      if (f == a[r].end() || f->second == 0.0) continue;
      double a_rk = f->second;
      double factor = a_rk / pivot;
      F.lu[{r, k}] = factor;
      f->second = 0.0;
      for (auto& cv : u_part) {
        size_t c = cv.first;
        double vk = cv.second;
        auto g = a[r].find(c);
        double cur = g == a[r].end() ? 0.0 : g->second;
        double nv = cur - factor * vk;
        if (nv == 0.0) {
          if (g != a[r].end()) {
            a[r].erase(g);
            colrows[c].erase(r);
          }
        } else {
          if (g != a[r].end())
            g->second = nv;
          else {
            a[r].emplace(c, nv);
            colrows[c].insert(r);
          }
        }
      }
    }
  }
  return F;
}

// sparse.rs:219-265. Returns false for a singular / non-finite solve.
bool lu_solve(const LU& F, size_t n, const std::vector<double>& b, std::vector<double>& xo) {
  std::vector<double> bp(n);
  for (size_t i = 0; i < n; ++i) bp[i] = b[F.perm[i]];
  for (auto& sw : F.swaps) std::swap(bp[sw.first], bp[sw.second]);
  std::vector<double> y(n, 0.0);
  for (size_t i = 0; i < n; ++i) {
    double s = bp[i];
    auto lo = F.lu.lower_bound({i, 0});
    auto hi = F.lu.lower_bound({i, i});
    for (auto it = lo; it != hi; ++it) s -= it->second * y[it->first.second];
    y[i] = s;
  }
  std::vector<double> x(n, 0.0);
  for (size_t ii = n; ii-- > 0;) {
    auto d = F.lu.find({ii, ii});
    double diag = d == F.lu.end() ? 0.0 : d->second;
    if (std::fabs(diag) < 1e-300) return false;
    double s = y[ii];
    auto lo = F.lu.upper_bound({ii, ii});
    auto hi = F.lu.lower_bound({ii + 1, 0});
    for (auto it = lo; it != hi; ++it) s -= it->second * x[it->first.second];
    x[ii] = s / diag;
  }
  for (double v : x)
    if (!std::isfinite(v)) return false;
  xo.assign(n, 0.0);
  for (size_t i = 0; i < n; ++i) xo[F.perm[i]] = x[i];
  return true;
}

// ---------------------------------------------------------------- bag of named arrays
struct Bag {
  std::map<std::string, std::vector<double>> f;
  std::map<std::string, std::vector<int64_t>> i;
  std::string err;
};

std::string key(int c, const char* name) { return "c" + std::to_string(c) + "." + name; }

// The per-chart system of the default unfold path (lscm.rs:512-676), as the interleaved
// CSR the GPU boundary receives (Sparse::to_csr(2 nf), sparse.rs:69-84) and the full
// Sparse for the CPU LU.
struct ChartSystem {
  std::vector<V2> p2;
  std::vector<size_t> pin_ids;
  std::vector<V2> pin_uv;
  std::vector<long> free_pos;
  std::vector<size_t> free_ids;
  size_t nfree = 0;
  Sparse M{0};
  std::vector<double> rhs;
};

ChartSystem build_system(const Mesh& mesh, const Chart& ch, double angle_mix, double mix_w) {
  ChartSystem S;
  std::vector<V3> p3;
  for (uint32_t v : ch.vertex_ids) p3.push_back(mesh.pos[v]);
  size_t nv = p3.size();
  S.p2 = tangent_frame(p3);
  std::map<uint32_t, V2> pin_source;
  if (ch.border_loops.empty()) {
    auto anchors = anchor_ids(p3, 4);
    for (size_t i : anchors) pin_source[ch.vertex_ids[i]] = S.p2[i];
  } else {
    pin_source = border_targets(mesh, ch, ch.border_loops);
  }
  for (auto& kv : pin_source) {
    long li = ch.local_of(kv.first);
    if (li >= 0 && std::find(S.pin_ids.begin(), S.pin_ids.end(), (size_t)li) == S.pin_ids.end()) {
      S.pin_ids.push_back((size_t)li);
      S.pin_uv.push_back(kv.second);
    }
  }
  auto ew = edge_weights(p3, ch.tris);
  std::vector<char> is_free(nv, 1);
  for (size_t pi : S.pin_ids) is_free[pi] = 0;
  std::map<size_t, V2> pin_lookup;
  for (size_t k = 0; k < S.pin_ids.size(); ++k) pin_lookup[S.pin_ids[k]] = S.pin_uv[k];
  S.free_pos.assign(nv, -1);
  for (size_t i = 0; i < nv; ++i)
    if (is_free[i]) {
      S.free_pos[i] = (long)S.free_ids.size();
      S.free_ids.push_back(i);
    }
  S.nfree = S.free_ids.size();
  size_t nvar = 2 * S.nfree + 1, aux = 2 * S.nfree;
  double mix_b = 1.0 - angle_mix;
  S.rhs.assign(nvar, 0.0);
  S.M = Sparse(nvar);
  const size_t NONE = (size_t)-1;
  for (auto& kv : ew) {
    size_t i = kv.first.first, j = kv.first.second;
    double w = kv.second;
    if (w <= EPS_DEGENERATE) continue;
    V3 d3 = sub(p3[j], p3[i]);
    double c = w / rmax(dot(d3, d3), EPS_DEGENERATE);
    V2 d = sub2(S.p2[j], S.p2[i]);
    struct Dir {
      size_t aa, bb;
      V2 dv;
    } dirs[2] = {{i, j, d}, {j, i, {-d.u, -d.v}}};
    for (auto& dr : dirs) {
      if (!is_free[dr.aa]) continue;
      size_t ra = 2 * (size_t)S.free_pos[dr.aa];
      size_t bbx = NONE, bby = NONE;
      if (is_free[dr.bb]) {
        bbx = 2 * (size_t)S.free_pos[dr.bb];
        bby = bbx + 1;
      }
      S.M.add(ra, ra, c);
      S.M.add(ra + 1, ra + 1, c);
      if (bbx != NONE) S.M.add(ra, bbx, -c);
      if (bby != NONE) S.M.add(ra + 1, bby, -c);
      if (is_free[dr.bb]) {
        S.rhs[ra] += mix_b * c * dr.dv.u;
        S.rhs[ra + 1] += mix_b * c * dr.dv.v;
      } else {
        V2 pin = pin_lookup[dr.bb];
        S.rhs[ra] += mix_b * c * dr.dv.u + c * pin.u;
        S.rhs[ra + 1] += mix_b * c * dr.dv.v + c * pin.v;
      }
    }
  }
  S.M.add(aux, aux, mix_w);
  S.rhs[aux] = mix_w;
  return S;
}

// Damped driver loop (lscm.rs:570-719). The default path's system does not change between
// iterations (assembly depends only on positions, the tangent frame and the pins), so a
// deterministic solver returns the same solution every iteration: the loop is a function
// of (p2, pinned targets, solution).
void driver_loop(const ChartSystem& S, const std::vector<double>& sol, int max_iter, std::vector<V2>& uv,
                 int64_t* iters_out, double* err_accum_out) {
  size_t nv = S.p2.size();
  uv = S.p2;
  std::vector<V2> new_uv(nv);
  double err_accum = 1.0, step = 1.0, prev_err = std::numeric_limits<double>::infinity();
  int64_t iters_done = 0;
  if (max_iter <= 0) max_iter = 100;
  for (int it = 0; it < max_iter; ++it) {
    iters_done = it + 1;
    new_uv = uv;
    for (size_t i : S.free_ids) {
      size_t pos = (size_t)S.free_pos[i];
      new_uv[i] = {sol[2 * pos], sol[2 * pos + 1]};
    }
    for (size_t k = 0; k < S.pin_ids.size(); ++k) new_uv[S.pin_ids[k]] = S.pin_uv[k];
    std::vector<V2> dv(nv);
    for (size_t i = 0; i < nv; ++i) dv[i] = sub2(new_uv[i], uv[i]);
    double ndv = 0.0, nuv = 0.0;
    for (auto& d : dv) ndv += d.u * d.u + d.v * d.v;
    for (auto& u : uv) nuv += u.u * u.u + u.v * u.v;
    double err = std::sqrt(ndv) / rmax(std::sqrt(nuv), 1e-30);
    double applied = err * step;
    if (prev_err > 1e-30 && err > 2.0 * prev_err)
      step = rmax(step * 0.5, 0.05);
    else if (it > 3)
      step = rmin(step * 1.2, 1.0);
    if (applied < 1e-8 || (prev_err > 1e-30 && it != 0 && applied / prev_err <= 0.01)) break;
    for (size_t i = 0; i < nv; ++i) uv[i] = {uv[i].u + dv[i].u * step, uv[i].v + dv[i].v * step};
    prev_err = applied;
    err_accum += err;
    if (max_iter * 10 < it) break;
  }
  *iters_out = iters_done;
  *err_accum_out = err_accum;
}

// KeepMetric's signed UV area and its gradient (lscm.rs:120-155, triangle order).
double compute_area(const std::vector<V2>& uv, const std::vector<std::array<uint32_t, 3>>& tris) {
  double a = 0.0;
  for (auto& t : tris) {
    V2 p0 = uv[t[0]], p1 = uv[t[1]], p2 = uv[t[2]];
    a += (p1.u - p0.u) * (p2.v - p0.v) - (p2.u - p0.u) * (p1.v - p0.v);
  }
  return a * 0.5;
}
std::vector<V2> compute_area_grad(const std::vector<V2>& uv, const std::vector<std::array<uint32_t, 3>>& tris,
                                  size_t nv) {
  std::vector<V2> g(nv, V2{0.0, 0.0});
  for (auto& t : tris) {
    double x0 = uv[t[0]].u, y0 = uv[t[0]].v, x1 = uv[t[1]].u, y1 = uv[t[1]].v, x2 = uv[t[2]].u, y2 = uv[t[2]].v;
    double sgd = 0.5 * (x0 * (y2 - y1) + x1 * (y0 - y2) + x2 * (y1 - y0));
    double sgn = sgd > 0.0 ? 1.0 : -1.0;
    g[t[0]].u += (y2 - y1) * 0.5 * sgn;
    g[t[0]].v += (x1 - x2) * 0.5 * sgn;
    g[t[1]].u += (y0 - y2) * 0.5 * sgn;
    g[t[1]].v += (x2 - x0) * 0.5 * sgn;
    g[t[2]].u += (y1 - y0) * 0.5 * sgn;
    g[t[2]].v += (x0 - x1) * 0.5 * sgn;
  }
  return g;
}

// The KeepMetric unfold (lscm.rs:544-727 with keep_metric): the conformal free block of
// build_system, bordered by the slack column flip * area_w (both rows of a free vertex), the
// area-gradient row g(uv) and the corner area(uv) - target, rhs[aux] = 2 target; a sparse LU
// of that system every driver iteration (the matrix changes with uv), then the damped
// driver step.  Returns false when an LU fails (the reference breaks out of the loop).
bool keep_metric_loop(const Mesh& mesh, const Chart& ch, const ChartSystem& S, int max_iter, double target_area,
                      std::vector<V2>& uv, int64_t* iters_out, double* err_accum_out) {
  size_t nv = S.p2.size(), nf2 = 2 * S.nfree, aux = nf2;
  auto areas = face_areas3d(mesh);
  std::vector<double> area_w(nv, 0.0);
  for (size_t t = 0; t < ch.tris.size(); ++t)
    for (uint32_t vv : ch.tris[t]) area_w[vv] += areas[ch.face_ids[t]];
  double wsum = 0.0;
  for (double w : area_w) wsum += w;
  wsum = rmax(wsum, 1e-30);
  for (double& w : area_w) w /= wsum;
  uv = S.p2;
  double flip = compute_area(uv, ch.tris) >= 0.0 ? 1.0 : -1.0;
  double target = target_area > 0.0 ? target_area : ch.area3d;
  double err_accum = 1.0, step = 1.0, prev_err = std::numeric_limits<double>::infinity();
  int64_t iters_done = 0;
  if (max_iter <= 0) max_iter = 100;
  bool ok = true;
  for (int it = 0; it < max_iter; ++it) {
    iters_done = it + 1;
    Sparse M(nf2 + 1);
    for (size_t r = 0; r < nf2; ++r)
      for (auto& kv : S.M.rows[r])
        if (kv.first < nf2) M.rows[r][kv.first] = kv.second;
    std::vector<double> rhs(S.rhs.begin(), S.rhs.begin() + nf2);
    rhs.push_back(2.0 * target);
    double area_now = compute_area(uv, ch.tris);
    auto g = compute_area_grad(uv, ch.tris, nv);
    for (size_t i = 0; i < nv; ++i)
      if (S.free_pos[i] >= 0) {
        size_t ri = 2 * (size_t)S.free_pos[i];
        M.add(ri, aux, flip * area_w[i]);
        M.add(ri + 1, aux, flip * area_w[i]);
        M.add(aux, ri, g[i].u);
        M.add(aux, ri + 1, g[i].v);
      }
    M.add(aux, aux, area_now - target);
    LU F = factorize(M);
    std::vector<double> sol;
    if (!lu_solve(F, M.n, rhs, sol)) {
      ok = false;
      break;
    }
    std::vector<V2> new_uv = uv;
    for (size_t i : S.free_ids) {
      size_t pos = (size_t)S.free_pos[i];
      new_uv[i] = {sol[2 * pos], sol[2 * pos + 1]};
    }
    for (size_t k = 0; k < S.pin_ids.size(); ++k) new_uv[S.pin_ids[k]] = S.pin_uv[k];
    std::vector<V2> dv(nv);
    for (size_t i = 0; i < nv; ++i) dv[i] = sub2(new_uv[i], uv[i]);
    double ndv = 0.0, nuv = 0.0;
    for (auto& d : dv) ndv += d.u * d.u + d.v * d.v;
    for (auto& u : uv) nuv += u.u * u.u + u.v * u.v;
    double err = std::sqrt(ndv) / rmax(std::sqrt(nuv), 1e-30);
    double applied = err * step;
    if (prev_err > 1e-30 && err > 2.0 * prev_err)
      step = rmax(step * 0.5, 0.05);
    else if (it > 3)
      step = rmin(step * 1.2, 1.0);
    if (applied < 1e-8 || (prev_err > 1e-30 && it != 0 && applied / prev_err <= 0.01)) break;
    for (size_t i = 0; i < nv; ++i) uv[i] = {uv[i].u + dv[i].u * step, uv[i].v + dv[i].v * step};
    prev_err = applied;
    err_accum += err;
    if (max_iter * 10 < it) break;
  }
  *iters_out = iters_done;
  *err_accum_out = err_accum;
  return ok;
}

// ---------------------------------------------------------------- seam.rs / recut.rs
// seam.rs:145-165: undirected adjacency over the chart's faces (edges ascending), 3-D lengths
std::map<uint32_t, std::vector<std::pair<uint32_t, double>>> chart_adjacency(const Mesh& mesh, const Chart& ch) {
  std::set<EdgeKey> edges;
  for (size_t fi : ch.face_ids) {
    auto& t = mesh.faces[fi];
    edges.insert(edge_key(t[0], t[1]));
    edges.insert(edge_key(t[1], t[2]));
    edges.insert(edge_key(t[2], t[0]));
  }
  std::map<uint32_t, std::vector<std::pair<uint32_t, double>>> adj;
  for (auto& e : edges) {
    double len = len3(sub(mesh.pos[e.first], mesh.pos[e.second]));
    adj[e.first].push_back({e.second, len});
    adj[e.second].push_back({e.first, len});
  }
  return adj;
}

// seam.rs:54-109: multi-source Dijkstra; the heap pops the smallest distance, ties the
// larger vertex id (HeapItem's ordering); relaxations need a 1e-12 improvement
void dijkstra(const std::map<uint32_t, std::vector<std::pair<uint32_t, double>>>& adj, const std::vector<uint32_t>& seeds,
              std::map<uint32_t, double>& dist, std::map<uint32_t, uint32_t>& prev) {
  struct Item {
    double d;
    uint32_t v;
  };
  auto less = [](const Item& x, const Item& y) { return x.d > y.d || (x.d == y.d && x.v < y.v); };
  std::priority_queue<Item, std::vector<Item>, decltype(less)> heap(less);
  dist.clear();
  prev.clear();
  for (uint32_t s : seeds) {
    dist[s] = 0.0;
    heap.push({0.0, s});
  }
  while (!heap.empty()) {
    Item it = heap.top();
    heap.pop();
    auto f = dist.find(it.v);
    if (f != dist.end() && f->second < it.d - 1e-12) continue;
    auto a = adj.find(it.v);
    if (a == adj.end()) continue;
    for (auto& wl : a->second) {
      double nd = it.d + wl.second;
      auto g = dist.find(wl.first);
      bool better = g == dist.end() ? true : nd < g->second - 1e-12;
      if (better) {
        dist[wl.first] = nd;
        prev[wl.first] = it.v;
        heap.push({nd, wl.first});
      }
    }
  }
}

// seam.rs:111-131
bool farthest_excluding(const std::map<uint32_t, double>& dist, const std::set<uint32_t>& skip, uint32_t* out) {
  bool have = false;
  uint32_t bv = 0;
  double bd = 0.0;
  for (auto& kv : dist) {
    if (!std::isfinite(kv.second) || skip.count(kv.first)) continue;
    if (!have || kv.second > bd || (kv.second == bd && kv.first < bv)) {
      have = true;
      bv = kv.first;
      bd = kv.second;
    }
  }
  *out = bv;
  return have;
}

std::vector<uint32_t> reconstruct(const std::map<uint32_t, uint32_t>& prev, uint32_t target) {  // seam.rs:133-143
  std::vector<uint32_t> path{target};
  uint32_t cur = target;
  for (auto p = prev.find(cur); p != prev.end(); p = prev.find(cur)) {
    path.push_back(p->second);
    cur = p->second;
  }
  std::reverse(path.begin(), path.end());
  return path;
}

// min over ids by (x, id): the first minimum (seam.rs:177-187, :253-262)
template <class It>
uint32_t min_x_vertex(const Mesh& mesh, It b, It e) {
  uint32_t best = *b;
  for (It i = b; i != e; ++i) {
    double px = mesh.pos[*i].x, pb = mesh.pos[best].x;
    if (px < pb || (!(px > pb) && !(px < pb) && *i < best)) best = *i;
  }
  return best;
}

std::vector<std::vector<uint32_t>> seam_paths(const Mesh& mesh, const Chart& ch, size_t branch_count) {  // seam.rs:167-220
  std::vector<std::vector<uint32_t>> paths;
  if (ch.face_ids.size() < 2 || ch.vertex_ids.empty()) return paths;
  auto adj = chart_adjacency(mesh, ch);
  uint32_t start = min_x_vertex(mesh, ch.vertex_ids.begin(), ch.vertex_ids.end());
  std::set<uint32_t> tree;
  std::map<uint32_t, double> dist0, dist1;
  std::map<uint32_t, uint32_t> prev0, prev;
  dijkstra(adj, {start}, dist0, prev0);
  uint32_t a, b;
  if (!farthest_excluding(dist0, tree, &a)) return paths;
  dijkstra(adj, {a}, dist1, prev);
  if (!farthest_excluding(dist1, tree, &b)) return paths;
  if (a == b) return paths;
  auto trunk = reconstruct(prev, b);
  tree.insert(trunk.begin(), trunk.end());
  paths.push_back(trunk);
  for (size_t k = 0; k < branch_count; ++k) {
    std::vector<uint32_t> seeds(tree.begin(), tree.end());
    std::map<uint32_t, double> dt;
    std::map<uint32_t, uint32_t> pt;
    dijkstra(adj, seeds, dt, pt);
    uint32_t f;
    if (!farthest_excluding(dt, tree, &f)) break;
    auto branch = reconstruct(pt, f);
    if (branch.size() < 2) break;
    tree.insert(branch.begin(), branch.end());
    paths.push_back(branch);
  }
  return paths;
}

std::set<EdgeKey> seam_cut_edges(const Mesh& mesh, const Chart& ch, size_t branch_count) {  // seam.rs:222-231
  std::set<EdgeKey> cut;
  for (auto& path : seam_paths(mesh, ch, branch_count))
    for (size_t k = 0; k + 1 < path.size(); ++k) cut.insert(edge_key(path[k], path[k + 1]));
  return cut;
}

std::vector<uint32_t> border_crossing_path(const Mesh& mesh, const Chart& ch) {  // seam.rs:246-283
  if (ch.border.empty() || ch.face_ids.size() < 2) return {};
  auto adj = chart_adjacency(mesh, ch);
  uint32_t a = min_x_vertex(mesh, ch.border.begin(), ch.border.end());
  std::map<uint32_t, double> dist;
  std::map<uint32_t, uint32_t> prev;
  dijkstra(adj, {a}, dist, prev);
  bool have = false;
  uint32_t bv = 0;
  double bd = 0.0;
  for (uint32_t v : ch.border) {
    if (v == a) continue;
    auto f = dist.find(v);
    if (f == dist.end() || !std::isfinite(f->second)) continue;
    double d = f->second;
    if (have && d < bd) continue;
    if (have && d == bd) {
      bv = std::min(bv, v);
    } else {
      have = true;
      bv = v;
      bd = d;
    }
  }
  if (have && bd > 1e-12) return reconstruct(prev, bv);
  return {};
}

// metrics.rs:33-56
size_t winding_flips(const std::vector<V2>& uv, const std::vector<std::array<uint32_t, 3>>& tris) {
  if (tris.empty()) return 0;
  auto ts = [&](const std::array<uint32_t, 3>& t) {
    V2 u = uv[t[0]], v = uv[t[1]], w = uv[t[2]];
    return (v.u - u.u) * (w.v - u.v) - (w.u - u.u) * (v.v - u.v);
  };
  double sum = 0.0;
  for (auto& t : tris) sum += ts(t);
  double dom = sum < 0.0 ? -1.0 : 1.0;
  size_t n = 0;
  for (auto& t : tris)
    if (ts(t) * dom <= 0.0) ++n;
  return n;
}

struct CutOptions {
  bool seam_enable = false;
  size_t seam_min_faces = 8, seam_branch = 1;
  bool recut_enable = false;
  size_t max_rounds = 6, max_splits = 48, max_charts = 64;
  double fold_fraction = 0.02;
};

// seam.rs:286-305
std::vector<Chart> cut_closed_charts(const Mesh& mesh, const std::vector<Chart>& charts, std::set<EdgeKey>& all,
                                     const CutOptions& o) {
  size_t before = all.size();
  for (auto& ch : charts) {
    if (!ch.border_loops.empty() || ch.face_ids.size() < o.seam_min_faces) continue;
    for (auto& e : seam_cut_edges(mesh, ch, o.seam_branch)) all.insert(e);
  }
  if (all.size() == before) return charts;
  return build_charts(mesh, all);
}

// recut.rs:98-146, with each round's unfolds by the reference LU path (unfold_chart with the
// default options: angle_mix 1, mix_w 1)
std::vector<Chart> recut_folding_charts(const Mesh& mesh, std::vector<Chart> charts, std::set<EdgeKey>& all,
                                        const CutOptions& o, int max_iter, size_t* added_out,
                                        std::vector<std::vector<size_t>>* folds_log) {
  size_t added = 0;
  for (size_t round = 0; round < o.max_rounds; ++round) {
    if (added >= o.max_splits) break;
    std::vector<size_t> folds(charts.size());
    for (size_t i = 0; i < charts.size(); ++i) {
      ChartSystem S = build_system(mesh, charts[i], 1.0, 1.0);
      LU Fc = factorize(S.M);
      std::vector<double> sol;
      std::vector<V2> uv = S.p2;
      if (lu_solve(Fc, S.M.n, S.rhs, sol)) {
        int64_t iters;
        double ea;
        driver_loop(S, sol, max_iter, uv, &iters, &ea);
      }
      folds[i] = winding_flips(uv, charts[i].tris);
    }
    if (folds_log) folds_log->push_back(folds);
    std::vector<size_t> folding;
    for (size_t i = 0; i < charts.size(); ++i)
      if ((double)folds[i] / (double)std::max<size_t>(charts[i].tris.size(), 1) > o.fold_fraction) folding.push_back(i);
    if (folding.empty()) break;
    std::stable_sort(folding.begin(), folding.end(), [&](size_t x, size_t y) { return folds[x] > folds[y]; });
    bool grew = false;
    for (size_t i : folding) {
      if (added >= o.max_splits) break;
      std::set<EdgeKey> cut;
      if (charts[i].border_loops.empty()) {
        cut = seam_cut_edges(mesh, charts[i], std::max<size_t>(o.seam_branch, 1));
      } else {
        auto path = border_crossing_path(mesh, charts[i]);
        for (size_t k = 0; k + 1 < path.size(); ++k) cut.insert(edge_key(path[k], path[k + 1]));
      }
      for (auto& e : cut)
        if (all.insert(e).second) {
          ++added;
          grew = true;
        }
    }
    if (!grew) break;
    charts = build_charts(mesh, all);
    if (charts.size() > o.max_charts) break;
  }
  *added_out = added;
  return charts;
}

// metrics.rs:59-70
void svd2(const double m[2][2], double* s1, double* s2) {
  double a = m[0][0] * m[0][0] + m[1][0] * m[1][0];
  double b = m[0][0] * m[0][1] + m[1][0] * m[1][1];
  double c = m[0][1] * m[0][1] + m[1][1] * m[1][1];
  double tr = a + c;
  double d = 0.5 * (a - c);
  double disc = std::sqrt(rmax(d * d + b * b, 0.0));
  double l1 = 0.5 * tr + disc;
  double l2 = rmax(0.5 * tr - disc, 0.0);
  *s1 = std::sqrt(rmax(l1, 0.0));
  *s2 = std::sqrt(l2);
}

// metrics.rs:73-141 (conformal / area ratio per triangle; folds per metrics.rs:41-56)
void chart_distortion(const Mesh& mesh, const Chart& ch, const std::vector<V2>& uv, double out[5]) {
  std::vector<double> conf, ar;
  int64_t flips = 0;
  for (size_t t = 0; t < ch.tris.size(); ++t) {
    auto& f = mesh.faces[ch.face_ids[t]];
    V3 a3 = mesh.pos[f[0]], b3 = mesh.pos[f[1]], c3 = mesh.pos[f[2]];
    V2 u0 = uv[ch.tris[t][0]], u1 = uv[ch.tris[t][1]], u2 = uv[ch.tris[t][2]];
    V3 e1 = sub(b3, a3), e2 = sub(c3, a3);
    V3 nrm = cross_v(e1, e2);
    double ln = len3(nrm);
    if (ln < 1e-30) continue;
    V3 n = divs(nrm, ln);
    V3 t1 = divs(e1, rmax(len3(e1), 1e-30));
    V3 t2 = cross_v(n, t1);
    double e1t1 = dot(e1, t1), e2t1 = dot(e2, t1), e1t2 = dot(e1, t2), e2t2 = dot(e2, t2);
    double det = e1t1 * e2t2 - e2t1 * e1t2;
    if (std::fabs(det) < 1e-30) {
      flips++;
      continue;
    }
    double i00 = e2t2 / det, i01 = -e2t1 / det, i10 = -e1t2 / det, i11 = e1t1 / det;
    V2 du1 = sub2(u1, u0), du2 = sub2(u2, u0);
    double F[2][2] = {{du1.u * i00 + du2.u * i10, du1.u * i01 + du2.u * i11},
                      {du1.v * i00 + du2.v * i10, du1.v * i01 + du2.v * i11}};
    double s1, s2;
    svd2(F, &s1, &s2);
    conf.push_back(s1 / rmax(s2, 1e-30));
    double uva = 0.5 * std::fabs(du1.u * du2.v - du2.u * du1.v);
    ar.push_back(uva / (0.5 * ln));
  }
  double cs = 0.0, cm = 0.0, as = 0.0;
  for (double x : conf) cs += x;
  for (double x : conf) cm = rmax(cm, x);
  for (double x : ar) as += x;
  // winding_flips (metrics.rs:41-56)
  int64_t folds = 0;
  if (!ch.tris.empty()) {
    auto sgn = [&](size_t t) {
      V2 a = uv[ch.tris[t][0]], b = uv[ch.tris[t][1]], c = uv[ch.tris[t][2]];
      return (b.u - a.u) * (c.v - a.v) - (c.u - a.u) * (b.v - a.v);
    };
    double sum = 0.0;
    for (size_t t = 0; t < ch.tris.size(); ++t) sum += sgn(t);
    double dom = sum < 0.0 ? -1.0 : 1.0;
    for (size_t t = 0; t < ch.tris.size(); ++t)
      if (sgn(t) * dom <= 0.0) folds++;
  }
  out[0] = cs / (double)std::max<size_t>(conf.size(), 1);
  out[1] = cm;
  out[2] = as / (double)std::max<size_t>(ar.size(), 1);
  out[3] = (double)flips;
  out[4] = (double)folds;
}


// ---------------------------------------------------------------- precond.rs IC(0)
struct Csr {
  int64_t n = 0;
  std::vector<int64_t> ptr, cols;
  std::vector<double> vals;
};

// factor_ic0 (gpu/src/precond.rs:145-205): IC(0) on the lower pattern, natural order, rows
// of L with the strictly lower entries ascending and the diagonal last; pivot floor
// 1e-12 * max(|a_ii|, 1e-30).  false where the reference returns None.
bool ic0_factor(const Csr& a, Csr& L) {
  const int64_t n = a.n;
  std::vector<std::map<int64_t, double>> rows(n);
  std::vector<double> diag(n, 0.0);
  L.n = n;
  L.ptr.assign(1, 0);
  L.cols.clear();
  L.vals.clear();
  for (int64_t i = 0; i < n; ++i) {
    std::vector<std::pair<int64_t, double>> low;
    for (int64_t e = a.ptr[i]; e < a.ptr[i + 1]; ++e)
      if (a.cols[e] < i) low.push_back({a.cols[e], a.vals[e]});
    std::sort(low.begin(), low.end(), [](const std::pair<int64_t, double>& x, const std::pair<int64_t, double>& y) {
      return x.first < y.first;
    });
    for (auto& kv : low) {
      const int64_t k = kv.first;
      double s_ = kv.second;
      for (auto it = rows[i].begin(); it != rows[i].end() && it->first < k; ++it) {
        auto f = rows[k].find(it->first);
        if (f != rows[k].end()) s_ -= it->second * f->second;
      }
      const double l_kk = diag[k];
      if (std::fabs(l_kk) < 1e-300) return false;
      rows[i][k] = s_ / l_kk;  // a repeated column overwrites, as BTreeMap::insert does
    }
    double a_ii = 0.0;  // row_get: the first stored (i, i)
    for (int64_t e = a.ptr[i]; e < a.ptr[i + 1]; ++e)
      if (a.cols[e] == i) {
        a_ii = a.vals[e];
        break;
      }
    if (std::fabs(a_ii) < 1e-300) return false;
    double sum = a_ii;
    for (auto& kv : rows[i]) sum -= kv.second * kv.second;
    const double floor_ = 1e-12 * std::max(std::fabs(a_ii), 1e-30);
    if (sum < floor_) sum = floor_;
    diag[i] = std::sqrt(sum);
    for (auto& kv : rows[i]) {
      L.cols.push_back(kv.first);
      L.vals.push_back(kv.second);
    }
    L.cols.push_back(i);
    L.vals.push_back(diag[i]);
    L.ptr.push_back((int64_t)L.cols.size());
  }
  return true;
}

// transpose_lower (precond.rs:238-262): rows of the transpose, ascending, diagonal last.
Csr transpose_lower(const Csr& L) {
  const int64_t n = L.n;
  std::vector<std::vector<std::pair<int64_t, double>>> t(n);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t e = L.ptr[i]; e < L.ptr[i + 1]; ++e) {
      const int64_t j = L.cols[e];
      t[j == i ? i : j].push_back({i, L.vals[e]});
    }
  Csr T;
  T.n = n;
  T.ptr.assign(1, 0);
  for (int64_t i = 0; i < n; ++i) {
    auto row = t[i];
    std::stable_sort(row.begin(), row.end(), [](const std::pair<int64_t, double>& x, const std::pair<int64_t, double>& y) {
      return x.first < y.first;
    });
    size_t d = 0;  // the first entry on the diagonal moves to the end
    while (d < row.size() && row[d].first != i) ++d;
    const std::pair<int64_t, double> dg = row[d];
    row.erase(row.begin() + (std::ptrdiff_t)d);
    for (auto& kv : row) {
      T.cols.push_back(kv.first);
      T.vals.push_back(kv.second);
    }
    T.cols.push_back(dg.first);
    T.vals.push_back(dg.second);
    T.ptr.push_back((int64_t)T.cols.size());
  }
  return T;
}

// tri_levels (precond.rs:214-236): level of each row of a diagonal-last factor.
std::vector<int64_t> tri_levels(const Csr& F, bool descending) {
  const int64_t n = F.n;
  std::vector<int64_t> level(n, 0);
  for (int64_t t = 0; t < n; ++t) {
    const int64_t i = descending ? n - 1 - t : t;
    int64_t lv = 0;
    for (int64_t e = F.ptr[i]; e < F.ptr[i + 1] - 1; ++e) lv = std::max(lv, level[F.cols[e]] + 1);
    level[i] = lv;
  }
  return level;
}

// graph_coloring (precond.rs:49-75): greedy, vertices in index order, smallest free colour.
std::vector<int64_t> graph_coloring(const Csr& a) {
  const int64_t n = a.n;
  std::vector<int64_t> color(n, -1);
  std::vector<int64_t> used;
  for (int64_t v = 0; v < n; ++v) {
    used.clear();
    for (int64_t e = a.ptr[v]; e < a.ptr[v + 1]; ++e) {
      const int64_t c = a.cols[e];
      if (c != v && color[c] >= 0) used.push_back(color[c]);
    }
    std::sort(used.begin(), used.end());
    used.erase(std::unique(used.begin(), used.end()), used.end());
    int64_t k = 0;
    for (int64_t c : used) {
      if (c == k) ++k;
      else break;
    }
    color[v] = k;
  }
  return color;
}

// color_permutation + permute_csr (precond.rs:77-123).
void color_permute(const Csr& a, const std::vector<int64_t>& color, std::vector<int64_t>& to_perm,
                   std::vector<int64_t>& to_orig, Csr& P) {
  const int64_t n = a.n;
  int64_t nc = 0;
  for (int64_t c : color) nc = std::max(nc, c + 1);
  std::vector<int64_t> cnt(nc + 1, 0);
  for (int64_t c : color) cnt[c + 1] += 1;
  for (int64_t k = 1; k <= nc; ++k) cnt[k] += cnt[k - 1];
  to_perm.assign(n, 0);
  to_orig.assign(n, 0);
  for (int64_t v = 0; v < n; ++v) {
    const int64_t pos = cnt[color[v]]++;
    to_perm[v] = pos;
    to_orig[pos] = v;
  }
  P.n = n;
  P.ptr.assign(1, 0);
  P.cols.clear();
  P.vals.clear();
  for (int64_t pos = 0; pos < n; ++pos) {
    const int64_t o = to_orig[pos];
    std::vector<std::pair<int64_t, double>> row;
    for (int64_t e = a.ptr[o]; e < a.ptr[o + 1]; ++e) row.push_back({to_perm[a.cols[e]], a.vals[e]});
    std::stable_sort(row.begin(), row.end(), [](const std::pair<int64_t, double>& x, const std::pair<int64_t, double>& y) {
      return x.first < y.first;
    });
    for (auto& kv : row) {
      P.cols.push_back(kv.first);
      P.vals.push_back(kv.second);
    }
    P.ptr.push_back((int64_t)P.cols.size());
  }
}


// ---------------------------------------------------------------- fixed-pin system + adjoint
// Forward-mode dual numbers (value + N partials), CPU.
template <int N>
struct Dn {
  double v = 0.0;
  std::array<double, N> d{};
  Dn() = default;
  Dn(double x) : v(x) {}
};
template <int N> Dn<N> operator+(const Dn<N>& a, const Dn<N>& b) { Dn<N> r(a.v + b.v); for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k]; return r; }
template <int N> Dn<N> operator-(const Dn<N>& a, const Dn<N>& b) { Dn<N> r(a.v - b.v); for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k]; return r; }
template <int N> Dn<N> operator-(const Dn<N>& a) { Dn<N> r(-a.v); for (int k = 0; k < N; ++k) r.d[k] = -a.d[k]; return r; }
template <int N> Dn<N> operator*(const Dn<N>& a, const Dn<N>& b) { Dn<N> r(a.v * b.v); for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r; }
template <int N> Dn<N> operator/(const Dn<N>& a, const Dn<N>& b) { Dn<N> r(a.v / b.v); for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v); return r; }
template <int N> Dn<N> dnsqrt(const Dn<N>& a) { Dn<N> r(std::sqrt(a.v)); for (int k = 0; k < N; ++k) r.d[k] = r.v > 0.0 ? a.d[k] / (2.0 * r.v) : 0.0; return r; }
template <int N> Dn<N> dnmax(const Dn<N>& a, double c) { return a.v > c ? a : Dn<N>(c); }

struct FixedSystem {
  size_t n = 0, nf = 0;
  std::vector<V3> p3;
  std::vector<std::array<uint32_t, 3>> tris;
  std::vector<char> pinned;
  std::vector<V2> pin_uv;
  std::vector<long> row_of;
  std::vector<std::map<size_t, double>> rows;  // scalar L over free vertices
  std::vector<double> b;                       // 2 nf
};

FixedSystem fixed_system(Bag* bg) {
  FixedSystem S;
  const auto& P = bg->f["p3"];
  const auto& T = bg->i["tris"];
  const auto& pin = bg->i["pinned"];
  const auto& pu = bg->f["pin_uv"];
  S.n = pin.size();
  for (size_t i = 0; i < S.n; ++i) {
    S.p3.push_back({P[3 * i], P[3 * i + 1], P[3 * i + 2]});
    S.pinned.push_back(pin[i] ? 1 : 0);
    S.pin_uv.push_back({pu[2 * i], pu[2 * i + 1]});
  }
  for (size_t t = 0; t + 2 < T.size(); t += 3) S.tris.push_back({(uint32_t)T[t], (uint32_t)T[t + 1], (uint32_t)T[t + 2]});
  S.row_of.assign(S.n, -1);
  for (size_t i = 0; i < S.n; ++i)
    if (!S.pinned[i]) S.row_of[i] = (long)S.nf++;
  S.rows.assign(S.nf, {});
  S.b.assign(2 * S.nf, 0.0);
  auto ew = edge_weights(S.p3, S.tris);
  for (auto& kv : ew) {  // lscm.rs:594-676 with mix_b = 0 (angle_mix = 1, the default)
    size_t i = kv.first.first, j = kv.first.second;
    double w = kv.second;
    if (w <= EPS_DEGENERATE) continue;
    V3 d3 = sub(S.p3[j], S.p3[i]);
    double c = w / rmax(dot(d3, d3), EPS_DEGENERATE);
    size_t ab[2][2] = {{i, j}, {j, i}};
    for (auto& e : ab) {
      if (S.pinned[e[0]]) continue;
      size_t r = (size_t)S.row_of[e[0]];
      if (c != 0.0) S.rows[r][r] += c;  // Sparse::add skips zeros
      if (!S.pinned[e[1]]) {
        if (c != 0.0) S.rows[r][(size_t)S.row_of[e[1]]] += -c;
      } else {
        S.b[2 * r] += c * S.pin_uv[e[1]].u;
        S.b[2 * r + 1] += c * S.pin_uv[e[1]].v;
      }
    }
  }
  return S;
}

// The distortion term of one triangle with the F of metrics.rs:95-128: 0.5 |n| (s1/s2 - 1)^2.
template <class T>
bool tri_distortion_cpu(const T (&p)[9], const T (&u)[6], T& out) {
  T e1x = p[3] - p[0], e1y = p[4] - p[1], e1z = p[5] - p[2];
  T e2x = p[6] - p[0], e2y = p[7] - p[1], e2z = p[8] - p[2];
  T nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
  T ln = dnsqrt(nx * nx + ny * ny + nz * nz);
  if (ln.v < 1e-30) return false;
  T ux = nx / ln, uy = ny / ln, uz = nz / ln;
  T l1 = dnmax(dnsqrt(e1x * e1x + e1y * e1y + e1z * e1z), 1e-30);
  T t1x = e1x / l1, t1y = e1y / l1, t1z = e1z / l1;
  T t2x = uy * t1z - uz * t1y, t2y = uz * t1x - ux * t1z, t2z = ux * t1y - uy * t1x;
  T e1t1 = e1x * t1x + e1y * t1y + e1z * t1z, e2t1 = e2x * t1x + e2y * t1y + e2z * t1z;
  T e1t2 = e1x * t2x + e1y * t2y + e1z * t2z, e2t2 = e2x * t2x + e2y * t2y + e2z * t2z;
  T det = e1t1 * e2t2 - e2t1 * e1t2;
  if (std::fabs(det.v) < 1e-30) return false;
  T i00 = e2t2 / det, i01 = -e2t1 / det, i10 = -e1t2 / det, i11 = e1t1 / det;
  T d1u = u[2] - u[0], d1v = u[3] - u[1], d2u = u[4] - u[0], d2v = u[5] - u[1];
  T f00 = d1u * i00 + d2u * i10, f01 = d1u * i01 + d2u * i11;
  T f10 = d1v * i00 + d2v * i10, f11 = d1v * i01 + d2v * i11;
  // singular values without svd2's 0.5 tr - disc cancellation: s1 = (|(f00 + f11, f10 - f01)|
  // + |(f00 - f11, f10 + f01)|) / 2, s2 = |det F| / s1
  T p0 = f00 + f11, p1 = f10 - f01, q0 = f00 - f11, q1 = f10 + f01;
  T s1 = T(0.5) * (dnsqrt(p0 * p0 + p1 * p1) + dnsqrt(q0 * q0 + q1 * q1));
  T dF = f00 * f11 - f01 * f10;
  if (dF.v < 0.0) dF = -dF;
  T s2 = s1.v > 0.0 ? dF / s1 : T(0.0);
  T r = s1 / dnmax(s2, 1e-30) - T(1.0);
  out = T(0.5) * ln * r * r;
  return true;
}

// Clamped corner cotangent as edge_weights forms it (lscm.rs:256-268); false where skipped.
template <class T>
bool corner_cot_cpu(const T (&o)[3], const T (&e1)[3], const T (&e0)[3], T& out) {
  T a1[3] = {e1[0] - o[0], e1[1] - o[1], e1[2] - o[2]};
  T a2[3] = {e0[0] - o[0], e0[1] - o[1], e0[2] - o[2]};
  T la = dnsqrt(a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2]);
  T lb = dnsqrt(a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2]);
  if (la.v <= EPS_DEGENERATE || lb.v <= EPS_DEGENERATE) return false;
  T cx = a1[1] * a2[2] - a1[2] * a2[1], cy = a1[2] * a2[0] - a1[0] * a2[2], cz = a1[0] * a2[1] - a1[1] * a2[0];
  T s_ = dnsqrt(cx * cx + cy * cy + cz * cz) / (la * lb);
  if (s_.v <= EPS_DEGENERATE) return false;
  T dt = a1[0] * a2[0] + a1[1] * a2[1] + a1[2] * a2[2];
  out = dnmax((dt / (la * lb)) / s_, 0.0);
  return true;
}

Csr bag_csr(Bag* b, const std::string& pre) {
  Csr a;
  a.ptr = b->i[pre + ".row_ptr"];
  a.cols = b->i[pre + ".cols"];
  a.vals = b->f[pre + ".vals"];
  a.n = (int64_t)a.ptr.size() - 1;
  return a;
}
void put_csr(Bag* b, const std::string& pre, const Csr& a) {
  b->i[pre + ".ptr"] = a.ptr;
  b->i[pre + ".cols"] = a.cols;
  b->f[pre + ".vals"] = a.vals;
}
}  // namespace

// ================================================================= extern "C" interface
extern "C" {

void* orc_bag_new() { return new Bag(); }
void orc_bag_free(void* h) { delete static_cast<Bag*>(h); }

int64_t orc_len(void* h, const char* name) {
  Bag* b = static_cast<Bag*>(h);
  auto f = b->f.find(name);
  if (f != b->f.end()) return (int64_t)f->second.size();
  auto i = b->i.find(name);
  if (i != b->i.end()) return (int64_t)i->second.size();
  return -1;
}
int orc_get_f64(void* h, const char* name, double* out) {
  Bag* b = static_cast<Bag*>(h);
  auto f = b->f.find(name);
  if (f == b->f.end()) return -1;
  std::memcpy(out, f->second.data(), f->second.size() * 8);
  return 0;
}
int orc_get_i64(void* h, const char* name, int64_t* out) {
  Bag* b = static_cast<Bag*>(h);
  auto i = b->i.find(name);
  if (i == b->i.end()) return -1;
  std::memcpy(out, i->second.data(), i->second.size() * 8);
  return 0;
}
void orc_put_f64(void* h, const char* name, const double* v, int64_t n) {
  static_cast<Bag*>(h)->f[name].assign(v, v + n);
}
void orc_put_i64(void* h, const char* name, const int64_t* v, int64_t n) {
  static_cast<Bag*>(h)->i[name].assign(v, v + n);
}

// meshgen.rs fixtures -> bag {"pos" (3*nv), "faces" (3*nf)}
void orc_meshgen(void* h, const char* name, int64_t n, double r_major, double r_minor, int64_t nu, int64_t nv_) {
  Bag* b = static_cast<Bag*>(h);
  std::vector<V3> p;
  std::vector<std::array<uint32_t, 3>> f;
  std::string nm(name);
  if (nm == "cube") {  // meshgen.rs:12-54
    int fd[6][4] = {{2, 0, 0, 1}, {2, 1, 0, 1}, {0, 0, 1, 2}, {0, 1, 1, 2}, {1, 0, 0, 2}, {1, 1, 0, 2}};
    for (auto& d : fd) {
      uint32_t base = (uint32_t)p.size();
      for (int64_t i = 0; i <= n; ++i)
        for (int64_t j = 0; j <= n; ++j) {
          double pt[3];
          for (int k = 0; k < 3; ++k) {
            if (k == d[0])
              pt[k] = (double)d[1];
            else if (k == d[2])
              pt[k] = (double)i / (double)n;
            else if (k == d[3])
              pt[k] = (double)j / (double)n;
            else
              pt[k] = 0.0;
          }
          p.push_back({pt[0], pt[1], pt[2]});
        }
      for (int64_t i = 0; i < n; ++i)
        for (int64_t j = 0; j < n; ++j) {
          uint32_t a = base + (uint32_t)i * ((uint32_t)n + 1) + (uint32_t)j;
          uint32_t bb = a + 1, c = a + ((uint32_t)n + 1), dd = c + 1;
          f.push_back({a, bb, dd});
          f.push_back({a, dd, c});
        }
    }
  } else if (nm == "sphere") {  // meshgen.rs:60-87 (nu x nv_)
    double du = 2.0 * PI / (double)(nu - 1);
    double dv = PI / (double)(nv_ - 1);
    for (int64_t j = 0; j < nv_; ++j) {
      double v = dv * (double)j;
      for (int64_t i = 0; i < nu; ++i) {
        double u = du * (double)i;
        p.push_back({std::sin(v) * std::cos(u), std::sin(v) * std::sin(u), std::cos(v)});
      }
    }
    for (int64_t i = 0; i < nu; ++i)
      for (int64_t j = 0; j < nv_ - 1; ++j) {
        uint32_t a = (uint32_t)(j * nu + i), bb = (uint32_t)(j * nu + (i + 1) % nu);
        uint32_t c = a + (uint32_t)nu, d = bb + (uint32_t)nu;
        f.push_back({a, c, d});
        f.push_back({a, d, bb});
      }
  } else if (nm == "torus" || nm == "annulus") {  // meshgen.rs:92-131
    for (int64_t j = 0; j < nv_; ++j) {
      double v = 2.0 * PI * (double)j / (double)nv_;
      for (int64_t i = 0; i < nu; ++i) {
        double u = 2.0 * PI * (double)i / (double)nu;
        double cr = r_major + r_minor * std::cos(v);
        p.push_back({cr * std::cos(u), cr * std::sin(u), r_minor * std::sin(v)});
      }
    }
    int64_t jc = nv_ / 2, k = 0;
    for (int64_t i = 0; i < nu; ++i)
      for (int64_t j = 0; j < nv_; ++j) {
        uint32_t a = (uint32_t)(j * nu + i), bb = (uint32_t)(j * nu + (i + 1) % nu);
        int64_t jn = (j + 1) % nv_;
        uint32_t c = (uint32_t)(jn * nu + i), d = (uint32_t)(jn * nu + (i + 1) % nu);
        bool keep = nm == "torus" || ((k / 2) % nv_ != jc);
        if (keep) f.push_back({a, bb, d});
        ++k;
        keep = nm == "torus" || ((k / 2) % nv_ != jc);
        if (keep) f.push_back({a, d, c});
        ++k;
      }
  } else if (nm == "grid") {  // meshgen.rs:135-155 (nu x nv_ quads)
    int64_t w = nu, hh = nv_;
    for (int64_t j = 0; j <= hh; ++j)
      for (int64_t i = 0; i <= w; ++i) p.push_back({(double)i, (double)j, 0.0});
    uint32_t stride = (uint32_t)(w + 1);
    for (int64_t j = 0; j < hh; ++j)
      for (int64_t i = 0; i < w; ++i) {
        uint32_t a = (uint32_t)j * stride + (uint32_t)i, bb = a + 1, c = a + stride, d = c + 1;
        f.push_back({a, bb, d});
        f.push_back({a, d, c});
      }
  } else if (nm == "cylinder") {  // meshgen.rs:160-182 (r = r_major, height = r_minor)
    double r = r_major, height = r_minor;
    for (int64_t j = 0; j <= nv_; ++j) {
      double z = height * (double)j / (double)std::max<int64_t>(nv_, 1);
      for (int64_t i = 0; i <= nu; ++i) {
        double t = 2.0 * PI * (double)i / (double)std::max<int64_t>(nu, 1);
        p.push_back({r * std::cos(t), r * std::sin(t), z});
      }
    }
    uint32_t stride = (uint32_t)(nu + 1);
    for (int64_t j = 0; j < nv_; ++j)
      for (int64_t i = 0; i < nu; ++i) {
        uint32_t a = (uint32_t)j * stride + (uint32_t)i, bb = a + 1, c = a + stride, d = c + 1;
        f.push_back({a, bb, d});
        f.push_back({a, d, c});
      }
  }
  auto& P = b->f["pos"];
  P.clear();
  for (auto& q : p) {
    P.push_back(q.x);
    P.push_back(q.y);
    P.push_back(q.z);
  }
  auto& F = b->i["faces"];
  F.clear();
  for (auto& t : f)
    for (uint32_t v : t) F.push_back(v);
}

// eig3 (lscm_eig.rs:13-66): m row-major 9 -> w[3], v[9] (v[i*3+k] = component i of vector k)
void orc_eig3(const double* m, double* w, double* v) {
  double mm[3][3], vv[3][3];
  for (int i = 0; i < 9; ++i) mm[i / 3][i % 3] = m[i];
  eig3(mm, w, vv);
  for (int i = 0; i < 9; ++i) v[i] = vv[i / 3][i % 3];
}

// Sparse::solve on COO triples (sparse.rs:47-52 add semantics, :219-265 solve).
int orc_sparse_solve(int64_t n, int64_t nnz, const int64_t* r, const int64_t* c, const double* v,
                     const double* b, double* x) {
  Sparse S((size_t)n);
  for (int64_t k = 0; k < nnz; ++k) S.add((size_t)r[k], (size_t)c[k], v[k]);
  LU F = factorize(S);
  std::vector<double> bb(b, b + n), xo;
  if (!lu_solve(F, (size_t)n, bb, xo)) return -1;
  std::memcpy(x, xo.data(), (size_t)n * 8);
  return 0;
}

// The unfold pipeline's chart stages for a raw triangle soup.
// in: bag with "pos" (3*nv), "faces" (3*nf).
// out (same bag): "mesh.pos", "mesh.faces", "n_charts", "n_cut", per chart c:
//   c.face_ids, c.vertex_ids, c.tris, c.border, c.loop_off, c.loop_ids, c.area3d,
//   c.p2 (2*nv), c.pin_ids (local), c.pin_uv (2*npins), c.free_pos (nv, -1 = pinned),
//   c.csr_ptr, c.csr_cols, c.csr_vals (interleaved, Sparse::to_csr(2 nf)), c.rhs (2nf+1)
//   and, when solve_limit >= 2nf+1: c.sol (LU solution), c.uv, c.iters, c.err_accum,
//   c.metrics (conformal mean/max, area ratio mean, flips, folds).
int orc_pipeline(void* h, double weld_tol, double angle_deg, double angle_mix, double mix_w,
                 int64_t solve_limit, int64_t max_iter) {
  Bag* b = static_cast<Bag*>(h);
  Mesh raw;
  auto& P = b->f["pos"];
  auto& F = b->i["faces"];
  for (size_t k = 0; k + 2 < P.size(); k += 3) raw.pos.push_back({P[k], P[k + 1], P[k + 2]});
  for (size_t k = 0; k + 2 < F.size(); k += 3)
    raw.faces.push_back({(uint32_t)F[k], (uint32_t)F[k + 1], (uint32_t)F[k + 2]});
  Mesh mesh = weld(raw, weld_tol);
  {
    auto& mp = b->f["mesh.pos"];
    mp.clear();
    for (auto& q : mesh.pos) {
      mp.push_back(q.x);
      mp.push_back(q.y);
      mp.push_back(q.z);
    }
    auto& mf = b->i["mesh.faces"];
    mf.clear();
    for (auto& t : mesh.faces)
      for (uint32_t v : t) mf.push_back(v);
  }
  size_t n_cut = 0;
  std::set<EdgeKey> cut0;
  auto charts = segment(mesh, angle_deg, &n_cut, &cut0);
  // pipeline.rs:149-167: optional seam cut of closed charts, then optional re-cutting of
  // folding charts (which starts again from the segmentation's cut set, as the reference does)
  CutOptions co;
  if (b->f.count("opt.seam") && b->f["opt.seam"].size() == 3 && b->f["opt.seam"][0] != 0.0) {
    co.seam_enable = true;
    co.seam_min_faces = (size_t)b->f["opt.seam"][1];
    co.seam_branch = (size_t)b->f["opt.seam"][2];
  }
  if (b->f.count("opt.seam_branch") && !b->f["opt.seam_branch"].empty())
    co.seam_branch = (size_t)b->f["opt.seam_branch"][0];
  if (b->f.count("opt.recut") && b->f["opt.recut"].size() == 5 && b->f["opt.recut"][0] != 0.0) {
    co.recut_enable = true;
    co.max_rounds = (size_t)b->f["opt.recut"][1];
    co.max_splits = (size_t)b->f["opt.recut"][2];
    co.fold_fraction = b->f["opt.recut"][3];
    co.max_charts = (size_t)b->f["opt.recut"][4];
  }
  if (co.seam_enable) {
    std::set<EdgeKey> all = cut0;
    charts = cut_closed_charts(mesh, charts, all, co);
  }
  if (co.recut_enable) {
    std::set<EdgeKey> all = cut0;
    size_t added = 0;
    std::vector<std::vector<size_t>> log;
    charts = recut_folding_charts(mesh, charts, all, co, (int)max_iter, &added, &log);
    b->i["recut.added"] = {(int64_t)added};
    auto& lf = b->i["recut.folds"];
    lf.clear();
    for (auto& r : log) {
      lf.push_back((int64_t)r.size());
      for (size_t x : r) lf.push_back((int64_t)x);
    }
  }
  b->i["n_charts"] = {(int64_t)charts.size()};
  b->i["n_cut"] = {(int64_t)n_cut};
  for (size_t ci = 0; ci < charts.size(); ++ci) {
    auto& ch = charts[ci];
    int c = (int)ci;
    auto& fi = b->i[key(c, "face_ids")];
    fi.assign(ch.face_ids.begin(), ch.face_ids.end());
    auto& vi = b->i[key(c, "vertex_ids")];
    vi.assign(ch.vertex_ids.begin(), ch.vertex_ids.end());
    auto& tr = b->i[key(c, "tris")];
    tr.clear();
    for (auto& t : ch.tris)
      for (uint32_t v : t) tr.push_back(v);
    auto& bd = b->i[key(c, "border")];
    bd.assign(ch.border.begin(), ch.border.end());
    auto& lo = b->i[key(c, "loop_off")];
    auto& li = b->i[key(c, "loop_ids")];
    lo = {0};
    li.clear();
    for (auto& l : ch.border_loops) {
      for (uint32_t v : l) li.push_back(v);
      lo.push_back((int64_t)li.size());
    }
    b->f[key(c, "area3d")] = {ch.area3d};
    ChartSystem S = build_system(mesh, ch, angle_mix, mix_w);
    auto& p2 = b->f[key(c, "p2")];
    p2.clear();
    for (auto& q : S.p2) {
      p2.push_back(q.u);
      p2.push_back(q.v);
    }
    auto& pid = b->i[key(c, "pin_ids")];
    pid.assign(S.pin_ids.begin(), S.pin_ids.end());
    auto& puv = b->f[key(c, "pin_uv")];
    puv.clear();
    for (auto& q : S.pin_uv) {
      puv.push_back(q.u);
      puv.push_back(q.v);
    }
    auto& fp = b->i[key(c, "free_pos")];
    fp.assign(S.free_pos.begin(), S.free_pos.end());
    // Sparse::to_csr(2 nf)  (sparse.rs:69-84)
    size_t limit = 2 * S.nfree;
    auto& cp = b->i[key(c, "csr_ptr")];
    auto& cc = b->i[key(c, "csr_cols")];
    auto& cv = b->f[key(c, "csr_vals")];
    cp = {0};
    cc.clear();
    cv.clear();
    for (size_t r = 0; r < limit; ++r) {
      for (auto& kv : S.M.rows[r])
        if (kv.first < limit) {
          cc.push_back((int64_t)kv.first);
          cv.push_back(kv.second);
        }
      cp.push_back((int64_t)cv.size());
    }
    b->f[key(c, "rhs")] = S.rhs;
    const bool keep_metric = b->f.count("opt.keep_metric") && !b->f["opt.keep_metric"].empty() &&
                             b->f["opt.keep_metric"][0] != 0.0;
    if (keep_metric && (int64_t)(2 * S.nfree + 1) <= solve_limit) {
      const double target_area = b->f.count("opt.target_area") ? b->f["opt.target_area"][0] : 0.0;
      std::vector<V2> uv;
      int64_t iters;
      double ea;
      keep_metric_loop(mesh, ch, S, (int)max_iter, target_area, uv, &iters, &ea);
      auto& u = b->f[key(c, "uv")];
      u.clear();
      for (auto& q : uv) {
        u.push_back(q.u);
        u.push_back(q.v);
      }
      b->i[key(c, "iters")] = {iters};
      b->f[key(c, "err_accum")] = {ea};
    } else if ((int64_t)(2 * S.nfree + 1) <= solve_limit) {
      LU Fc = factorize(S.M);
      std::vector<double> sol;
      bool ok = lu_solve(Fc, S.M.n, S.rhs, sol);
      if (ok) {
        b->f[key(c, "sol")] = sol;
        std::vector<V2> uv;
        int64_t iters;
        double ea;
        driver_loop(S, sol, (int)max_iter, uv, &iters, &ea);
        auto& u = b->f[key(c, "uv")];
        u.clear();
        for (auto& q : uv) {
          u.push_back(q.u);
          u.push_back(q.v);
        }
        b->i[key(c, "iters")] = {iters};
        b->f[key(c, "err_accum")] = {ea};
        double met[5];
        chart_distortion(mesh, ch, uv, met);
        b->f[key(c, "metrics")] = std::vector<double>(met, met + 5);
      } else {
        b->i[key(c, "iters")] = {0};
      }
    }
  }
  return 0;
}

// Driver loop with an externally supplied solution (e.g. a SuperLU solve of the exported
// CSR): in-bag c.sol must hold 2nf+1 values.  Writes c.uv, c.iters, c.err_accum, c.metrics.
int orc_driver_from_solution(void* h, int64_t chart, int64_t max_iter) {
  Bag* b = static_cast<Bag*>(h);
  int c = (int)chart;
  auto& p2 = b->f[key(c, "p2")];
  auto& pid = b->i[key(c, "pin_ids")];
  auto& puv = b->f[key(c, "pin_uv")];
  auto& fp = b->i[key(c, "free_pos")];
  auto& sol = b->f[key(c, "sol")];
  ChartSystem S;
  size_t nv = p2.size() / 2;
  for (size_t i = 0; i < nv; ++i) S.p2.push_back({p2[2 * i], p2[2 * i + 1]});
  for (size_t k = 0; k < pid.size(); ++k) {
    S.pin_ids.push_back((size_t)pid[k]);
    S.pin_uv.push_back({puv[2 * k], puv[2 * k + 1]});
  }
  S.free_pos.assign(fp.begin(), fp.end());
  for (size_t i = 0; i < nv; ++i)
    if (fp[i] >= 0) S.free_ids.push_back(i);
  S.nfree = S.free_ids.size();
  if (sol.size() < 2 * S.nfree) return -1;
  std::vector<V2> uv;
  int64_t iters;
  double ea;
  driver_loop(S, sol, (int)max_iter, uv, &iters, &ea);
  auto& u = b->f[key(c, "uv")];
  u.clear();
  for (auto& q : uv) {
    u.push_back(q.u);
    u.push_back(q.v);
  }
  b->i[key(c, "iters")] = {iters};
  b->f[key(c, "err_accum")] = {ea};
  return 0;
}

// chart_distortion on given UVs for chart c of the last orc_pipeline (needs mesh.* and c.*).
int orc_chart_metrics(void* h, int64_t chart, const double* uv, double* out5) {
  Bag* b = static_cast<Bag*>(h);
  int c = (int)chart;
  Mesh mesh;
  auto& mp = b->f["mesh.pos"];
  auto& mf = b->i["mesh.faces"];
  for (size_t k = 0; k + 2 < mp.size(); k += 3) mesh.pos.push_back({mp[k], mp[k + 1], mp[k + 2]});
  for (size_t k = 0; k + 2 < mf.size(); k += 3)
    mesh.faces.push_back({(uint32_t)mf[k], (uint32_t)mf[k + 1], (uint32_t)mf[k + 2]});
  Chart ch;
  auto& fi = b->i[key(c, "face_ids")];
  auto& tr = b->i[key(c, "tris")];
  ch.face_ids.assign(fi.begin(), fi.end());
  for (size_t k = 0; k + 2 < tr.size(); k += 3)
    ch.tris.push_back({(uint32_t)tr[k], (uint32_t)tr[k + 1], (uint32_t)tr[k + 2]});
  size_t nv = b->i[key(c, "vertex_ids")].size();
  std::vector<V2> u(nv);
  for (size_t i = 0; i < nv; ++i) u[i] = {uv[2 * i], uv[2 * i + 1]};
  chart_distortion(mesh, ch, u, out5);
  return 0;
}


// rectangularize (metrics.rs:147-227) of one chart: uv (2n), border flags (n) ->
// q (2n), ext (2).
void orc_rectangularize(int64_t n, const double* uv, const int64_t* border, double* q, double* ext) {
  std::vector<size_t> bnd;
  for (int64_t i = 0; i < n; ++i)
    if (border[i]) bnd.push_back((size_t)i);
  if (n == 0) return;
  if (bnd.empty()) {
    double mu = uv[0], mv = uv[1], xu = uv[0], xv = uv[1];
    for (int64_t i = 0; i < n; ++i) {
      mu = rmin(mu, uv[2 * i]);
      mv = rmin(mv, uv[2 * i + 1]);
      xu = rmax(xu, uv[2 * i]);
      xv = rmax(xv, uv[2 * i + 1]);
    }
    ext[0] = xu - mu;
    ext[1] = xv - mv;
    for (int64_t i = 0; i < n; ++i) {
      q[2 * i] = (uv[2 * i] - mu) / rmax(ext[0], 1e-30);
      q[2 * i + 1] = (uv[2 * i + 1] - mv) / rmax(ext[1], 1e-30);
    }
    return;
  }
  const int n_steps = 72;
  bool have = false;
  double bc = 1.0, bs_ = 0.0, bscore = 0.0;
  for (int k = 0; k < n_steps; ++k) {
    const double ang = 3.141592653589793 * (double)k / (double)(n_steps - 1);
    const double co = std::cos(ang), si = std::sin(ang);
    double mn = INFINITY, mx = -INFINITY, mnv = INFINITY, mxv = -INFINITY;
    for (size_t bi : bnd) {
      const double pu = uv[2 * bi], pv = uv[2 * bi + 1];
      const double qu = co * pu + si * pv;
      const double qv = -si * pu + co * pv;
      mn = rmin(mn, qu);
      mx = rmax(mx, qu);
      mnv = rmin(mnv, qv);
      mxv = rmax(mxv, qv);
    }
    const double e0 = mx - mn, e1 = mxv - mnv;
    const double score = std::sqrt(e0 * (e0 + 1e-30) + e1 * (e1 + 1e-30));
    if (!(have && score >= bscore)) {
      have = true;
      bc = co;
      bs_ = si;
      bscore = score;
    }
  }
  for (int64_t i = 0; i < n; ++i) {
    const double pu = uv[2 * i], pv = uv[2 * i + 1];
    q[2 * i] = bc * pu + bs_ * pv;
    q[2 * i + 1] = -bs_ * pu + bc * pv;
  }
  double mu = q[0], mv = q[1], xu = q[0], xv = q[1];
  for (int64_t i = 0; i < n; ++i) {
    mu = rmin(mu, q[2 * i]);
    mv = rmin(mv, q[2 * i + 1]);
    xu = rmax(xu, q[2 * i]);
    xv = rmax(xv, q[2 * i + 1]);
  }
  ext[0] = xu - mu;
  ext[1] = xv - mv;
  for (int64_t i = 0; i < n; ++i) {
    q[2 * i] = (q[2 * i] - mu) / rmax(ext[0], 1e-30);
    q[2 * i + 1] = (q[2 * i + 1] - mv) / rmax(ext[1], 1e-30);
  }
  for (size_t bi : bnd) {
    const double pu = q[2 * bi], pv = q[2 * bi + 1];
    const double dx = rmin(pu, 1.0 - pu), dy = rmin(pv, 1.0 - pv);
    if (dx <= dy) q[2 * bi] = pu < 0.5 ? 0.0 : 1.0;
    else q[2 * bi + 1] = pv < 0.5 ? 0.0 : 1.0;
  }
}

// IC(0) of bag {"a.row_ptr", "a.cols", "a.vals"} -> {"l.*", "lt.*" (ptr, cols, vals),
// "fwd.level", "bwd.level"}; with `colored`, of the colour-permuted matrix, adding
// {"color", "to_perm", "to_orig", "p.ptr", "p.cols", "p.vals"}.  0, or -1 where the
// reference's factor_ic0 returns None.
int orc_ic0(void* h, int colored) {
  Bag* b = static_cast<Bag*>(h);
  Csr a = bag_csr(b, "a");
  if (colored) {
    std::vector<int64_t> color = graph_coloring(a), tp, to;
    Csr P;
    color_permute(a, color, tp, to, P);
    b->i["color"] = color;
    b->i["to_perm"] = tp;
    b->i["to_orig"] = to;
    put_csr(b, "p", P);
    a = P;
  }
  Csr L;
  if (!ic0_factor(a, L)) return -1;
  Csr T = transpose_lower(L);
  put_csr(b, "l", L);
  put_csr(b, "lt", T);
  b->i["fwd.level"] = tri_levels(L, false);
  b->i["bwd.level"] = tri_levels(T, true);
  return 0;
}

// z = (L L^T)^-1 r with the factor in the bag (the reference test's host sweeps,
// precond.rs:932-950: forward over L, backward over L^T, diagonal read from each row).
void orc_ic0_apply(void* h, const double* r, double* z) {
  Bag* b = static_cast<Bag*>(h);
  const auto& lp = b->i["l.ptr"];
  const auto& lc = b->i["l.cols"];
  const auto& lv = b->f["l.vals"];
  const auto& tp = b->i["lt.ptr"];
  const auto& tc = b->i["lt.cols"];
  const auto& tv = b->f["lt.vals"];
  const int64_t n = (int64_t)lp.size() - 1;
  auto get = [](const std::vector<int64_t>& p, const std::vector<int64_t>& c, const std::vector<double>& v, int64_t i,
                int64_t j) {
    for (int64_t k = p[i]; k < p[i + 1]; ++k)
      if (c[k] == j) return v[k];
    return 0.0;
  };
  std::vector<double> y(n, 0.0);
  for (int64_t i = 0; i < n; ++i) {
    double s_ = r[i];
    for (int64_t k = lp[i]; k < lp[i + 1] - 1; ++k) s_ -= lv[k] * y[lc[k]];
    y[i] = s_ / get(lp, lc, lv, i, i);
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double s_ = y[i];
    for (int64_t k = tp[i]; k < tp[i + 1] - 1; ++k) s_ -= tv[k] * z[tc[k]];
    z[i] = s_ / get(tp, tc, tv, i, i);
  }
}

// Fixed-pin LSCM system of one chart: bag {"p3" (3n), "tris" (3T, local), "pinned" (n),
// "pin_uv" (2n)} -> {"row_of" (n, -1 pinned), "csr.ptr", "csr.cols", "csr.vals" (scalar L
// over free vertices, columns ascending), "b" (2 nf)}.
void orc_lscm_fixed(void* h) {
  Bag* b = static_cast<Bag*>(h);
  FixedSystem S = fixed_system(b);
  std::vector<int64_t> ptr(1, 0), cols, row_of(S.n);
  std::vector<double> vals;
  for (size_t r = 0; r < S.nf; ++r) {
    for (auto& kv : S.rows[r]) {
      cols.push_back((int64_t)kv.first);
      vals.push_back(kv.second);
    }
    ptr.push_back((int64_t)cols.size());
  }
  for (size_t i = 0; i < S.n; ++i) row_of[i] = S.row_of[i];
  b->i["row_of"] = row_of;
  b->i["csr.ptr"] = ptr;
  b->i["csr.cols"] = cols;
  b->f["csr.vals"] = vals;
  b->f["b"] = S.b;
}

// Distortion loss of a layout (uv: 2n, all vertices) with its gradients: per-triangle terms
// summed in triangle order into *loss; duv (2n) and dp3 (3n) receive the gradients.
// Triangles with all three vertices pinned are left out (their UVs come from the pin rule,
// which can make them collinear).  Also bag "loss_t" (per triangle, 0 where skipped).
void orc_distortion_loss(void* h, const double* uv, double* loss, double* duv, double* dp3) {
  Bag* b = static_cast<Bag*>(h);
  const auto& P = b->f["p3"];
  const auto& T = b->i["tris"];
  const auto& pin = b->i["pinned"];
  const size_t n = P.size() / 3, nt = T.size() / 3;
  std::fill(duv, duv + 2 * n, 0.0);
  std::fill(dp3, dp3 + 3 * n, 0.0);
  std::vector<double> lt(nt, 0.0);
  double total = 0.0;
  for (size_t t = 0; t < nt; ++t) {
    size_t v[3] = {(size_t)T[3 * t], (size_t)T[3 * t + 1], (size_t)T[3 * t + 2]};
    if (pin[v[0]] && pin[v[1]] && pin[v[2]]) continue;
    Dn<15> p[9], u[6];
    for (int k = 0; k < 3; ++k) {
      for (int j = 0; j < 3; ++j) {
        p[3 * k + j] = Dn<15>(P[3 * v[k] + j]);
        p[3 * k + j].d[3 * k + j] = 1.0;
      }
      for (int j = 0; j < 2; ++j) {
        u[2 * k + j] = Dn<15>(uv[2 * v[k] + j]);
        u[2 * k + j].d[9 + 2 * k + j] = 1.0;
      }
    }
    Dn<15> out;
    if (!tri_distortion_cpu(p, u, out)) continue;
    lt[t] = out.v;
    total += out.v;
    for (int k = 0; k < 3; ++k) {
      for (int j = 0; j < 3; ++j) dp3[3 * v[k] + j] += out.d[3 * k + j];
      for (int j = 0; j < 2; ++j) duv[2 * v[k] + j] += out.d[9 + 2 * k + j];
    }
  }
  b->f["loss_t"] = lt;
  *loss = total;
}

// Reverse pass of the fixed-pin assembly: given the solution x and the adjoint lam (2 nf
// each, free rows), dp3 (3n) = d(lam^T (b - A x)) / dp3, i.e. the position gradient of a
// loss whose uv-gradient produced lam.
void orc_lscm_adjoint_positions(void* h, const double* x, const double* lam, double* dp3) {
  Bag* b = static_cast<Bag*>(h);
  FixedSystem S = fixed_system(b);
  std::fill(dp3, dp3 + 3 * S.n, 0.0);
  auto ew = edge_weights(S.p3, S.tris);
  std::map<std::pair<size_t, size_t>, double> gw;  // dL/dw per edge
  for (auto& kv : ew) {
    size_t i = kv.first.first, j = kv.first.second;
    double w = kv.second;
    if (w <= EPS_DEGENERATE) continue;
    if (S.pinned[i] && S.pinned[j]) continue;
    auto uvl = [&](size_t v, double& u0, double& u1, double& l0, double& l1) {
      if (S.pinned[v]) {
        u0 = S.pin_uv[v].u;
        u1 = S.pin_uv[v].v;
        l0 = l1 = 0.0;
      } else {
        size_t r = (size_t)S.row_of[v];
        u0 = x[2 * r];
        u1 = x[2 * r + 1];
        l0 = lam[2 * r];
        l1 = lam[2 * r + 1];
      }
    };
    double ui0, ui1, li0, li1, uj0, uj1, lj0, lj1;
    uvl(i, ui0, ui1, li0, li1);
    uvl(j, uj0, uj1, lj0, lj1);
    const double gc = -((li0 - lj0) * (ui0 - uj0) + (li1 - lj1) * (ui1 - uj1));
    V3 d3 = sub(S.p3[j], S.p3[i]);
    const double d2 = dot(d3, d3);
    if (d2 > EPS_DEGENERATE) {
      gw[kv.first] = gc / d2;
      const double gd2 = -gc * w / (d2 * d2);
      const double g3[3] = {2.0 * gd2 * d3.x, 2.0 * gd2 * d3.y, 2.0 * gd2 * d3.z};
      for (int k = 0; k < 3; ++k) {
        dp3[3 * j + k] += g3[k];
        dp3[3 * i + k] -= g3[k];
      }
    } else {
      gw[kv.first] = gc / EPS_DEGENERATE;
    }
  }
  for (auto& t : S.tris) {  // cotangent partials by duals over the 9 coordinates
    size_t vs[3] = {t[0], t[1], t[2]};
    Dn<9> q[3][3];
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j) {
        q[k][j] = Dn<9>(S.p3[vs[k]].x * (j == 0) + S.p3[vs[k]].y * (j == 1) + S.p3[vs[k]].z * (j == 2));
        q[k][j].d[3 * k + j] = 1.0;
      }
    int cs[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};  // (e0, e1, o) as edge_weights walks them
    for (auto& c : cs) {
      size_t e0 = vs[c[0]], e1 = vs[c[1]];
      auto it = gw.find(std::make_pair(std::min(e0, e1), std::max(e0, e1)));
      if (it == gw.end() || it->second == 0.0) continue;
      Dn<9> ct;
      if (!corner_cot_cpu(q[c[2]], q[c[1]], q[c[0]], ct) || !(ct.v > 0.0)) continue;
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 3; ++j) dp3[3 * vs[k] + j] += it->second * ct.d[3 * k + j];
    }
  }
}
}  // extern "C"
