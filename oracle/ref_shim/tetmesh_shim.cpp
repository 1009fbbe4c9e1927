// C entry points over the reference's own mesh readers and vertex-neighbour builders:
// TetMesh (src/core/cuda/tetmesh.cu: TetMesh::read :251-376, need_neighbors :112-170) and
// TriMesh (src/core/aggmis/cuda/TriMesh_io.cu: TriMesh::read, PLY; TriMesh_connectivity.cu:
// need_neighbors), compiled from the reference sources by oracle/ref.mk into oracle/_ref/.
// Test infrastructure only: tests/test_reference_pins.py compares the mesh readers and the
// sparsity patterns of this repository with what the reference itself computes.
#include <cstdint>
#include <cstring>
#include <vector>

#include "TriMesh.h"
#include "tetmesh.h"

namespace {
TetMesh* g_mesh = nullptr;
TriMesh* g_tri = nullptr;

template <class NB>
int64_t flatten(const NB& neighbors, int32_t* offsets, int32_t* nbr) {
  int64_t total = 0;
  for (size_t i = 0; i < neighbors.size(); i++) {
    if (offsets) offsets[i] = (int32_t)total;
    for (int v : neighbors[i]) {
      if (nbr) nbr[total] = v;
      total++;
    }
  }
  if (offsets) offsets[neighbors.size()] = (int32_t)total;
  return total;
}
}  // namespace

extern "C" {

// Reads a TetGen .node/.ele pair with the reference reader and builds its vertex
// neighbours; returns 0 on success and the vertex and element counts.
int ref_tetmesh_read(const char* node, const char* ele, int64_t* nv, int64_t* ne) {
  delete g_mesh;
  g_mesh = TetMesh::read(node, ele, false);
  if (!g_mesh) return 1;
  g_mesh->need_neighbors();
  *nv = (int64_t)g_mesh->vertices.size();
  *ne = (int64_t)g_mesh->tets.size();
  return 0;
}

// Coordinates (nv x 3) and connectivity (ne x 4, as the reader stores it).
void ref_tetmesh_arrays(double* xyz, int32_t* tets) {
  for (size_t i = 0; i < g_mesh->vertices.size(); i++)
    for (int d = 0; d < 3; d++) xyz[3 * i + d] = g_mesh->vertices[i][d];
  for (size_t e = 0; e < g_mesh->tets.size(); e++)
    for (int a = 0; a < 4; a++) tets[4 * e + a] = g_mesh->tets[e][a];
}

// Neighbour lists in the order need_neighbors leaves them: offsets (nv + 1) when nbr is
// null, else the concatenated lists.  Returns the total count.
int64_t ref_tetmesh_neighbors(int32_t* offsets, int32_t* nbr) { return flatten(g_mesh->neighbors, offsets, nbr); }

void ref_tetmesh_free() {
  delete g_mesh;
  g_mesh = nullptr;
}

// A triangle mesh (PLY) with the reference reader and its vertex neighbours.
int ref_trimesh_read(const char* path, int64_t* nv, int64_t* nf) {
  delete g_tri;
  g_tri = TriMesh::read(path);
  if (!g_tri) return 1;
  g_tri->need_neighbors();
  *nv = (int64_t)g_tri->vertices.size();
  *nf = (int64_t)g_tri->faces.size();
  return 0;
}

// Coordinates (nv x 3, as the reader stores them) and faces (nf x 3).
void ref_trimesh_arrays(double* xyz, int32_t* faces) {
  for (size_t i = 0; i < g_tri->vertices.size(); i++)
    for (int d = 0; d < 3; d++) xyz[3 * i + d] = g_tri->vertices[i][d];
  for (size_t f = 0; f < g_tri->faces.size(); f++)
    for (int a = 0; a < 3; a++) faces[3 * f + a] = g_tri->faces[f][a];
}

int64_t ref_trimesh_neighbors(int32_t* offsets, int32_t* nbr) { return flatten(g_tri->neighbors, offsets, nbr); }
}
