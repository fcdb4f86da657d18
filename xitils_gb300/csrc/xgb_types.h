// Device data layout of a built scene (shared by host and device code).
//
// HBM layout, all arrays 16-byte aligned structure-of-arrays:
//   per mesh (BLAS): Node2[] (64 B/node), TriV[] (48 B/triangle, leaf order),
//     vertex attributes (float4 positions/normals/tangents/bitangents, float2 uv),
//     int32 indices, float4 geometric normal per triangle (object space).
//   per scene: Instance[] (mat, matInv, mesh, material), the top-level Node2[]
//     over instances, Material[], Texture[] descriptors, Light[] tables.
//   per render: path queues (2 x 64 B/path), hit records (32 B/path), shadow
//     queue (48 B/path), a control block of counters.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace xgb {

// Binary BVH node holding both children's boxes (one 64-byte line per visit).
// child >= 0: inner node index; child < 0: leaf, ~child = (first << 4) | (count - 1).
struct __align__(16) Node2 {
    float4 a;  // c0.lo.x c0.lo.y c0.lo.z c0.hi.x
    float4 b;  // c0.hi.y c0.hi.z c1.lo.x c1.lo.y
    float4 c;  // c1.lo.z c1.hi.x c1.hi.y c1.hi.z
    int4 d;    // child0 child1 - -
};
static_assert(sizeof(Node2) == 64, "Node2 size");

// Triangles per leaf of a binary mesh BVH. Measured on GB300 (leaf limit 2 / 3 / 4 / 6 / 8):
// terrain 1372 / 1362 / 1338 / 1284 / 1206 Mpaths/s, occluded room 26.9 / 26.8 / 26.1 / 24.6 /
// 22.9 -- a node test costs less than a triangle test.
constexpr int kLeafMax = 2;

// 8-wide mesh BVH node with 8-bit quantised child boxes (80 bytes, five 16-byte
// loads), after Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on
// GPUs Through Compressed Wide BVHs" (HPG 2017), with a layout of our own:
//   a: origin p.xyz, bits: exponent bytes ex | ey << 8 | ez << 16 | imask << 24
//      (child box plane = p + q * 2^(e - 127); imask bit s = slot s is an inner node)
//   b: childBase, triBase, meta[0..3], meta[4..7] (one byte per slot)
//   c: qlo.x[0..7], qlo.y[0..7];  d: qlo.z[0..7], qhi.x[0..7];  e: qhi.y[0..7], qhi.z[0..7]
// meta of an inner child: its index among the node's inner children (node
// childBase + meta); of a leaf child: count << 5 | offset, its 1..3 triangles
// at triBase + offset; 0 with the imask bit clear: an empty slot. Slots are
// filled so that for a ray whose direction has sign bits `oct`, visiting slot
// positions slot ^ oct in increasing order goes roughly front to back.
struct __align__(16) WNode {
    float4 a, b, c, d, e;
};
static_assert(sizeof(WNode) == 80, "WNode size");
constexpr int kWideLeafMax = 3;  // triangles per leaf child of a WNode

__host__ __device__ inline int leafEncode(int first, int count) { return ~((first << 4) | (count - 1)); }
__host__ __device__ inline int leafFirst(int code) { return (~code) >> 4; }
__host__ __device__ inline int leafCount(int code) { return ((~code) & 15) + 1; }

// Triangle vertices gathered in BVH leaf order: p0.xyz + original triangle index, p1, p2.
struct __align__(16) TriV {
    float4 p0;  // w = __int_as_float(original triangle index)
    float4 p1;
    float4 p2;
};

struct MeshDev {
    const Node2* nodes2;  // binary BVH (root at 0) when !wide
    const WNode* nodes;   // 8-wide BVH (root at 0) when wide
    int wide;
    const TriV* tris;
    const float4* pos;   // object-space positions (w = 0)
    const float2* uv;    // nullptr when absent
    const float4* nrm;   // nullptr when absent
    const float4* tan;   // nullptr when absent (then bit is nullptr too)
    const float4* bit;
    const int* idx;      // 3 per triangle
    const float4* gnrm;  // normalize(cross(p1-p0, p2-p0)) per triangle, FP64 cross (Vector.h:637-654)
    const float* triArea;  // TriangleIndexed::surfaceArea per triangle
    int nTris;
    int nVerts;
    int rootIsLeaf;  // 1 when the whole mesh is one leaf (no nodes): <= kLeafMax triangles (binary), <= kWideLeafMax (wide)
    int rootLeaf;    // leafEncode(0, nTris) of that leaf
    // Shell mapping (TriangleIndexedWithShellMapping, TriangleIndexed.h:220-256):
    // triangle t lies on layer t / shellFaces of shellLayers; shellLayers = 0
    // for an ordinary mesh.
    int shellLayers;
    int shellFaces;
    float shellScale;
    const float4* shellTexels;  // displacement texture (red channel used)
    int shellW, shellH, shellClamp, shellFilter;
};

struct __align__(16) Instance {
    float mat[16];     // object -> world, row-major m[r][c]
    float matInv[16];  // world -> object
    int mesh;
    int material;
    int lightIndex;    // index in the light table, -1 when not emissive
    int identity;      // 1 when mat and matInv are exactly the identity
};

enum MaterialKind : int {
    MAT_DIFFUSE = 0,
    MAT_METAL = 1,
    MAT_GLOSSY = 2,
    MAT_GLOSSY_HIGHLIGHT = 3,
    MAT_GLOSSY_CLAMPED = 4,
    MAT_EMISSION = 5,
    MAT_SPECULAR_REFLECTION = 6,
    MAT_SPECULAR_REFRACTION = 7,
    MAT_SPECULAR_FRESNEL = 8,
    MAT_MF_NORMALMAP = 9,
    MAT_MULTILOBE_SVBRDF = 10,  // base material + SVNDF (index in `tex`)
};

struct __align__(16) Material {
    int kind;
    int tex;        // albedo texture (Diffuse) or roughness texture (Metal), -1 none
    int normalmap;  // -1 none
    int base;       // facet material (MicrofacetNormalMapping), -1 none
    float3 albedo;  // albedo / f0 / power
    float roughness;
    float3 highlight;
    float sharpness;
    float sharpnessHL;
    float rate;
    float index;
    int flags;  // bit 0: Metal below-horizon fix (XGB_FIX_METAL_HORIZON)
};

struct TextureDev {
    const float4* texels;  // RGBA, row y = 0 first
    int w, h;
    int clamp;   // Texture::warpClamp
    int filter;  // Texture::filter
};

// SVNDF of a displacement map: per low texel 4 lobes as (mu.xyz, kappa) then the
// 4 weights, 5 float4 per texel, row-major [resV][resU].
constexpr int kSvndfLobes = 4;
struct SvndfDev {
    const float4* lobes;
    int resU, resV;
};

enum SkyKind : int { SKY_NONE = 0, SKY_UNIFORM = 1, SKY_PROBE = 2, SKY_LATLONG = 3 };

// One emissive object (Scene.h:17-22). Light triangle t of light L lives at
// triOffset[L] + t in the scene-wide light-triangle arrays.
struct LightDev {
    int instance;
    int mesh;
    int nTris;
    int triOffset;
};

constexpr int kDefaultMaxSteps = 1 << 22;
constexpr int kMaxStackLimit = 64;

struct SceneDev {
    const MeshDev* meshes;
    const Instance* instances;
    const Node2* tlas;
    int nInstances;
    int tlasRootIsLeaf;
    int blasLayout;  // every mesh binary (0), every mesh wide (1), or a mix (2)
    int fixes;       // opt-in quirk fixes of the render (XGB_FIX_DROP_NONFINITE = 2)
    int shell;       // 1 when some mesh is shell-mapped (its hits can be discarded during traversal)
    int nested;      // materials that evaluate another: bit 0 microfacet normal mapping, bit 1 MultiLobeSVBRDF
    int kinds;       // bit k: some material of the scene is of MaterialKind k
    // Device-side traversal bounds (xgb_scene_set_traversal_limits): a ray whose
    // traversal takes more than maxSteps loop steps sets error bit 4 and ends; a
    // push onto a stack already holding stackLimit entries sets error bit 1 and
    // ends the ray. Defaults: kDefaultMaxSteps and 64 (the stacks' size).
    int maxSteps;
    int stackLimit;
    const float4* instBox;  // per instance: world box lo (xyz), hi (xyz) as 2 float4
    const Material* materials;
    const TextureDev* textures;
    const SvndfDev* svndfs;
    const LightDev* lights;
    int nLights;
    // per light triangle (world data precomputed with the reference's arithmetic):
    const float4* lightNormal;  // world geometric normal (Object.h:99 asNormal of the triangle normal)
    const float* lightPdf;      // area pdf: 1/A / nTris / surfaceAreaScaling / nLights (Scene.h:40-55)
    // camera (Camera.h:45-55)
    float c2w[16];
    float tanHalfX;  // tanf(fov/2)
    float tanHalfY;  // tanf(fov/2 * aspect)
    // sky (SkySphere.h)
    int skyKind;
    int skyTex;
    float3 skyColor;
};

}  // namespace xgb
