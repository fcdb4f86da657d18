// Cinder stand-ins that must be visible before any Xitils header is included.
// TEST INFRASTRUCTURE ONLY. Xitils names cinder::TriMesh in TriangleMesh.h
// (the mesh-loading overloads of setGeometry) and ci::Surface / ci::ColorA8u in
// RenderTarget.h (the 8-bit display mapping). The checker builds meshes through
// the raw-array setGeometry overload, so TriMesh only has to compile.
#pragma once
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include <glm/glm.hpp>

#define memcpy_s(dest, destsz, src, n) std::memcpy((dest), (src), (n))

namespace cinder {

struct ColorA8u { uint8_t r = 0, g = 0, b = 0, a = 0; };

struct Surface {
    int width = 0, height = 0;
    std::vector<ColorA8u> pixels;
    Surface() = default;
    Surface(int w, int h, bool /*alpha*/) : width(w), height(h), pixels((size_t)w * h) {}
    void setPixel(const glm::ivec2& p, const ColorA8u& c) { pixels[(size_t)p.y * width + p.x] = c; }
};

struct TriMesh {
    std::vector<glm::vec3> positions, normals, tangents, bitangents;
    std::vector<glm::vec2> texcoords;
    std::vector<uint32_t> indices;

    TriMesh* clone() const { return new TriMesh(*this); }
    size_t getNumVertices() const { return positions.size(); }
    size_t getNumTriangles() const { return indices.size() / 3; }
    template <int D> glm::vec3* getPositions() { return positions.data(); }
    std::vector<glm::vec3>& getNormals() { return normals; }
    bool hasTexCoords0() const { return !texcoords.empty(); }
    template <int D> glm::vec2* getTexCoords0() { return texcoords.data(); }
    std::vector<glm::vec3>& getTangents() { return tangents; }
    std::vector<glm::vec3>& getBitangents() { return bitangents; }
    std::vector<uint32_t>& getIndices() { return indices; }
    void recalculateTangents() { tangents.assign(positions.size(), glm::vec3()); }
    void recalculateBitangents() { bitangents.assign(positions.size(), glm::vec3()); }
    void recalculateNormals() { normals.assign(positions.size(), glm::vec3()); }
};

namespace app {}
namespace geom {}

}  // namespace cinder
namespace ci = cinder;
