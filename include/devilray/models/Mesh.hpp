// Mesh.hpp -- indexed triangle mesh (include/models/Mesh.hpp of the reference)
// and its Wavefront OBJ loader.
#pragma once

#include "Utils.hpp"

#include <cstdint>
#include <string>
#include <vector>

struct Vertex
{
    uint32_t pi;  // point index
    uint32_t ni;  // normal index
};

struct Triangle
{
    Vertex a, b, c;
};

struct Mesh
{
    std::vector<Vec3> points;
    std::vector<Vec3> normals;
    std::vector<Triangle> triangles;

    std::string name;
};

struct MeshBounds
{
    Vec3 center;
    float extent;
};

// Loads the OBJ subset of src/models/Mesh.cpp:117-186: `v`, `vn`, `o`,
// triangular `f` faces with 1-based `p`, `p/t`, `p//n` or `p/t/n` indices;
// `vt`, `s`, `mtllib` and comments are skipped. Throws std::runtime_error for a
// missing file, an unknown tag, a face with more than 3 vertices or an index
// out of range. A mesh without normals gets one zero normal.
Mesh loadMesh(const std::string &fileName);
// One flat normal per triangle, (A - B) x (A - C) normalised.
void generateCoarseNormals(Mesh &mesh);
// Centroid of the points and the largest distance from it.
MeshBounds calculateMeshBounds(const Mesh &mesh);
// Centres the mesh and scales it to unit extent.
void normalizeMeshSize(Mesh &mesh);
