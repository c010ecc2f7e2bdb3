// Mesh files to triangle arrays: the OFF, OBJ and PLY readers (Graphics/MeshCodecOff.hpp, MeshCodecObj.hpp,
// MeshCodecPly.hpp) building display meshes, whose faces are triangulated as DisplayMesh::addFace does (Graphics/DisplayMesh.cpp:249-320). Host code.
#pragma once

#include "common.cuh"

#include <string>
#include <vector>

namespace thea {

// A mesh group flattened into arrays in the reference's element order: submeshes in file order, each submesh's
// vertices in its builder order, each face's triangles in triangulation order.
struct MeshData {
  std::vector<float> vertices;                    // xyz of every vertex of every submesh
  std::vector<int32_t> vertex_source;             // file vertex index of each vertex (0-based)
  std::vector<int32_t> triangles;                 // three indices into `vertices` per triangle
  std::vector<int32_t> triangle_face;             // source face index of each triangle
  std::vector<int64_t> submesh_vertex_offsets{0};   // submesh s owns vertices [o[s], o[s+1])
  std::vector<int64_t> submesh_triangle_offsets{0}; // and triangles [o[s], o[s+1])
  int64_t num_faces = 0;                          // faces that produced at least one triangle
};

// Triangles of one face with vertex positions pos[0 .. n) (xyz), as DisplayMesh::addFace makes them: a triangle as it
// is, a quad by Polygon3::triangulateQuad, a larger polygon by Polygon3::triangulate. Appends local vertex indices
// (three per triangle, at most n - 2 triangles) to `tris` and returns the number of triangles (0: the face is skipped).
int triangulate_face(float const * pos, int n, std::vector<int32_t> & tris);

// Reads an OFF, OBJ or PLY file (ASCII or binary), chosen by the file extension as MeshGroup::load does. Throws Error
// (THEA_ERR_INVALID_ARGUMENT) where the reference's non-strict readers throw; faces they skip are skipped.
MeshData read_mesh_file(std::string const & path);

// The same readers on a file's bytes in memory (MeshGroup::read with an explicit codec): codec "obj", "off" or "ply".
MeshData read_mesh_buffer(void const * data, int64_t bytes, std::string const & codec);

}  // namespace thea
