// Internal declarations shared by the host chart stages (prep.cpp) and the CUDA side.
#pragma once

#include <cstdint>
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

}  // namespace ruv
