// Mesh.cpp -- OBJ loading and mesh utilities (src/models/Mesh.cpp of the
// reference; same accepted grammar and error cases).
#include "models/Mesh.hpp"

#include <filesystem>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace {

// One face corner: p, p/t, p//n or p/t/n, 1-based; a missing normal index is 1.
Vertex parseCorner(const std::string &text)
{
    for (const char c : text)
        if (!(c == '/' || (c >= '0' && c <= '9')))
            throw std::runtime_error(std::string("unknown character in face corner: '") + c + "'");
    Vertex v{1, 1};
    size_t field = 0, start = 0;
    while (true) {
        const size_t slash = text.find('/', start);
        const std::string part = text.substr(start, slash == std::string::npos ? std::string::npos : slash - start);
        if (!part.empty() && field < 3) {
            const unsigned long idx = std::stoul(part);
            if (field == 0) v.pi = (uint32_t)idx;
            if (field == 2) v.ni = (uint32_t)idx;
        }
        ++field;
        if (slash == std::string::npos) break;
        start = slash + 1;
    }
    if (field > 3) throw std::runtime_error("face corner with " + std::to_string(field) + " indices");
    return v;
}

void toZeroBased(Mesh &m)
{
    if (m.normals.empty()) m.normals.push_back(Vec3{0, 0, 0});
    const uint32_t np = (uint32_t)m.points.size(), nn = (uint32_t)m.normals.size();
    for (size_t i = 0; i < m.triangles.size(); ++i) {
        Triangle &t = m.triangles[i];
        for (Vertex *v : {&t.a, &t.b, &t.c}) {
            if (v->pi == 0 || v->pi > np)
                throw std::runtime_error("triangle " + std::to_string(i) + ": point index " + std::to_string(v->pi) +
                                         " outside 1.." + std::to_string(np));
            if (v->ni == 0 || v->ni > nn)
                throw std::runtime_error("triangle " + std::to_string(i) + ": normal index " + std::to_string(v->ni) +
                                         " outside 1.." + std::to_string(nn));
            --v->pi;
            --v->ni;
        }
    }
}

}  // namespace

Mesh loadMesh(const std::string &fileName)
{
    if (!std::filesystem::exists(fileName)) throw std::runtime_error("File " + fileName + " does not exist");
    std::ifstream in(fileName);
    Mesh mesh;
    mesh.name = "Mesh";
    std::string line;
    while (std::getline(in, line)) {
        while (!line.empty() && (line.back() == ' ' || line.back() == '\t' || line.back() == '\r' || line.back() == '\n'))
            line.pop_back();
        std::istringstream ss(line);
        std::string tag;
        ss >> tag;
        if (tag.empty() || tag[0] == '#' || tag == "mtllib" || tag == "s" || tag == "vt") continue;
        if (tag == "v" || tag == "vn") {
            Vec3 q{};
            ss >> q.x >> q.y >> q.z;
            if (ss.fail()) throw std::runtime_error("Failed to parse: " + line);
            (tag == "v" ? mesh.points : mesh.normals).push_back(q);
            continue;
        }
        if (tag == "o") {
            ss >> mesh.name;
            continue;
        }
        if (tag == "f") {
            std::vector<Vertex> corners;
            std::string c;
            while (ss >> c) corners.push_back(parseCorner(c));
            if (corners.size() < 3) continue;
            if (corners.size() > 3)
                throw std::runtime_error("Triangulation not supported. Found face with " +
                                         std::to_string(corners.size()) + " vertices");
            mesh.triangles.push_back(Triangle{corners[0], corners[1], corners[2]});
            continue;
        }
        throw std::runtime_error("Unrecognized tag: " + tag);
    }
    toZeroBased(mesh);
    return mesh;
}

void generateCoarseNormals(Mesh &mesh)
{
    std::vector<Vec3> normals;
    normals.reserve(mesh.triangles.size());
    for (Triangle &t : mesh.triangles) {
        const Vec3 A = mesh.points[t.a.pi], B = mesh.points[t.b.pi], C = mesh.points[t.c.pi];
        const uint32_t idx = (uint32_t)normals.size();
        normals.push_back((A - B).cross(A - C).normalized());
        t.a.ni = t.b.ni = t.c.ni = idx;
    }
    mesh.normals = std::move(normals);
}

MeshBounds calculateMeshBounds(const Mesh &mesh)
{
    Vec3 sum{0, 0, 0};
    for (const Vec3 &p : mesh.points) sum += p;
    const Vec3 center = sum / static_cast<float>(mesh.points.size());
    float extent = 0;
    for (const Vec3 &p : mesh.points) extent = std::max(extent, (p - center).length());
    return MeshBounds{center, extent};
}

void normalizeMeshSize(Mesh &mesh)
{
    const MeshBounds b = calculateMeshBounds(mesh);
    for (Vec3 &p : mesh.points) p = (p - b.center) / b.extent;
}
