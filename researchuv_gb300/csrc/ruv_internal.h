// Internal declarations shared by the host chart stages (prep.cpp) and the CUDA side.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "../../include/ruv.h"

namespace ruv {

// Charts prepared on the host (the unfold_chart prologue for every chart of a mesh).
struct Prepared {
  std::vector<double> mesh_pos;      // welded mesh (3 * V)
  std::vector<int32_t> mesh_faces;   // welded mesh (3 * F)
  int64_t n_cut_slots = 0;           // face slots on a sharp (cut) edge
  std::vector<int64_t> vert_off, tri_off, border_off, loop_off, loop_seg;
  std::vector<int64_t> vertex_ids;   // source vertex per packed vertex
  std::vector<int64_t> face_ids;     // source face per packed triangle
  std::vector<int32_t> tris;         // chart-local
  std::vector<int64_t> border;       // per chart, sorted source ids
  std::vector<int64_t> loop_ids;     // source ids
  std::vector<double> area3d;
  std::vector<double> p3, p2, pin_uv;
  std::vector<uint8_t> pinned;
};

ruv_status prepare_mesh(const double* pos, int64_t nv, const int32_t* faces, int64_t nf, double weld_tol,
                        double angle_min_deg, int threads, Prepared& P, std::string& err);
ruv_status prepare_patches(int64_t np, const int64_t* vert_off, const int64_t* tri_off, const double* p3,
                           const int32_t* tris, int threads, Prepared& P, std::string& err);

// Per-chart vertex sets built elsewhere (on the device): chart c's sorted source vertex ids
// verts[vert_off[c], vert_off[c + 1]) and its chart-local triangles tris[3 cf_off[c], ...),
// in the chart's face order cf[cf_off[c], cf_off[c + 1]).
struct ChartSets {
  std::vector<int64_t> vert_off;
  std::vector<int32_t> verts;
  std::vector<int32_t> tris;
};
using ChartSetsFn = std::function<bool(const std::vector<int64_t>& cf_off, const std::vector<int32_t>& cf,
                                       ChartSets& out, std::string& err)>;

// prepare_mesh from a welded mesh (3 * V positions, 3 * F faces) with its edge-face lists
// (per face slot, the faces carrying the edge in ascending order) and cut flags: the DFS
// components, the chart vertex sets (from `sets` when given, else on the host), border
// loops, frames and pins, and the packing -- the host part of the device path.
ruv_status prepare_mesh_topology(std::vector<double>&& wpos3, std::vector<int32_t>&& F, std::vector<int64_t>&& ef_off,
                                 std::vector<int32_t>&& ef_faces, std::vector<uint8_t>&& cut, int threads,
                                 const ChartSetsFn* sets, Prepared& P, std::string& err);

// prepare_patches with its data-parallel stages on a device (prep_gpu.cu supplies the two
// callbacks): `dev` checks the patches and returns, for patches that are connected, every
// patch's faces in the reference's DFS pop order with its local triangles in that order, its
// area, the centroid and covariance of its vertices (tangent frame, lscm.rs:152-183) and
// its boundary edge keys; `proj` projects every vertex on its chart's frame (9 per chart:
// centroid, e1, e2).  The border loops, the eig3 of each frame and the pins run on the host
// (per chart, O(border)), then the packing.  The same Prepared as prepare_patches, bit for bit.
struct Ctx;
struct PatchDevice {
  std::vector<int32_t> order;    // tri_off[np]: source faces, DFS pop order per patch
  std::vector<int32_t> tris;     // 3 tri_off[np]: patch-local triangles in that order
  std::vector<double> area3d;    // np
  std::vector<double> cov;       // 12 np: centroid (3), covariance (3 x 3)
  std::vector<int64_t> boff;     // np + 1
  std::vector<uint64_t> bkeys;   // boundary edges (min << 32 | max, source ids), per patch
};
using PatchDeviceFn = std::function<ruv_status(PatchDevice& out, std::string& err)>;
using PatchProjectFn = std::function<ruv_status(const std::vector<double>& frames, std::vector<double>& p2,
                                                std::string& err)>;
ruv_status prepare_patches_device(int64_t np, const int64_t* vert_off, const int64_t* tri_off, const double* p3,
                                  const int32_t* tris, int threads, const PatchDeviceFn& dev, const PatchProjectFn& proj,
                                  Prepared& P, std::string& err);
ruv_status prepare_patches_gpu(Ctx& ctx, int64_t np, const int64_t* vert_off, const int64_t* tri_off, const double* p3,
                               const int32_t* tris, int threads, Prepared& P, std::string& err);

// Seam cut of closed charts (seam.rs SeamCutOptions) and re-cutting of folding charts
// (recut.rs RecutOptions) after the segmentation (pipeline.rs:149-167).
struct CutOpts {
  bool seam_enable = false;
  int64_t seam_min_faces = 8, seam_branch = 1;
  bool recut_enable = false;
  int64_t max_rounds = 6, max_splits = 48, max_charts = 64;
  double fold_fraction = 0.02;
};
// The unfold of every chart of a Prepared (2 * n_verts UVs, chart-local order).
using UnfoldFn = std::function<bool(const Prepared& P, std::vector<double>& uv, std::string& err)>;
ruv_status prepare_mesh_cut(const double* pos, int64_t nv, const int32_t* faces, int64_t nf, double weld_tol,
                            double angle_min_deg, int threads, const CutOpts& co, const UnfoldFn* unfold,
                            Prepared& P, int64_t* added_out, std::string& err);

// The dihedral test acos(n1.n2) > angle of segment.rs:130-137 as d < d*: d* from the host
// libm's acos (so both sides decide alike); NaN when acos is not monotone around d*.
double acos_cut_threshold(double angle_min_deg);

// compute_area (lscm.rs:120-129): the signed area of a chart's UVs, triangles in order (host,
// no FMA contraction) -- KeepMetric's orientation flip is its sign, a decision that must be
// the reference's even when the area is at rounding level
double uv_signed_area(const double* uv, const int32_t* tris, int64_t nt);

// prepare_mesh with the weld, edge-face lists, cut flags and chart vertex sets on the device
// of `ctx` (prep_gpu.cu): the same Prepared, bit for bit.
ruv_status prepare_mesh_gpu(Ctx& ctx, const double* pos, int64_t nv, const int32_t* faces, int64_t nf, double weld_tol,
                            double angle_min_deg, int threads, Prepared& P, std::string& err);

}  // namespace ruv
