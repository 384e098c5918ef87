// VTK local coordinates of the elements Writer<Part> writes
// (mesh/vtk.hpp:214-224, 310-330), in VTK's node order: Hexahedron27 in
// [-1, 1]^3 (corners, edge midpoints, face centres, centre) for Hex8 cells
// and Tetrahedron10 in units of 1/2 (corners, edge midpoints) for Tet4
// cells.  One copy per translation unit.
#pragma once

namespace mcfd {

static __constant__ signed char kVtkHex27[27][3] = {
    {-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
    {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1},
    {0, -1, -1},  {1, 0, -1},  {0, 1, -1}, {-1, 0, -1},
    {0, -1, 1},   {1, 0, 1},   {0, 1, 1},  {-1, 0, 1},
    {-1, -1, 0},  {1, -1, 0},  {1, 1, 0},  {-1, 1, 0},
    {-1, 0, 0},   {1, 0, 0},   {0, -1, 0}, {0, 1, 0},
    {0, 0, -1},   {0, 0, 1},   {0, 0, 0}};
static __constant__ signed char kVtkTet10Half[10][3] = {
    {2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {0, 0, 0}, {1, 1, 0},
    {0, 1, 1}, {1, 0, 1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

}  // namespace mcfd
