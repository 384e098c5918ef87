// The GPU part of the connectivity builder (mesh_build_gpu.cu), called by
// mcfd_build_faces_gpu in mesh_build.cpp.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace mcfd {

struct GpuPairs {
  std::vector<int64_t> inner_cells;  // [faces][2] holder (lower id), sharer, by (holder, side)
  std::vector<int32_t> inner_sides;  // [faces][2]
  std::vector<int64_t> lone_cells;   // free slots in (cell, side) order
  std::vector<int32_t> lone_sides;
};

// Pairs every (cell, local face) slot on the device.  slot_off [n_cells + 1]
// gives each cell's first slot (6 per hexahedron, 4 per tetrahedron).
// Returns 0, 1 for a CUDA or table error, 2 for a mesh error (text in err).
int gpu_pair_slots(int device, const int64_t *cell_nodes, int64_t stride, const int32_t *cell_type,
                   int64_t n_cells, const std::vector<int64_t> &slot_off, GpuPairs *out,
                   std::string *err);

}  // namespace mcfd
