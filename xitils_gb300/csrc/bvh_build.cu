// GPU construction of a per-mesh bounding-volume hierarchy (the reference
// builds its _BVH single-threaded on the CPU, AccelerationStructure.h:163-291;
// the tree shape affects speed only, never the image).
//
// Linear BVH after Karras, "Maximizing Parallelism in the Construction of
// BVHs, Octrees, and k-d Trees" (HPG 2012):
//   1. per triangle: bounds, centroid, FP64-cross geometric normal, area;
//   2. 30-bit Morton codes of the centroids, radix-sorted (CUB);
//   3. one thread per internal node finds its key range and split;
//   4. bounds propagate bottom-up (the second child to arrive merges);
//   5. subtrees of <= kLeafMax triangles collapse into leaves and each inner
//      node is written as a 64-byte Node2 holding both children's boxes;
//   6. triangle vertices are gathered into leaf order (48 B per triangle).
#include <cub/device/device_radix_sort.cuh>

#include "xgb_kernels.h"

namespace xgb {
namespace {

__device__ __forceinline__ unsigned int orderedBits(float f) {
    unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float orderedFloat(unsigned int u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
#else
    unsigned int v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    float f;
    memcpy(&f, &v, 4);
    return f;
#endif
}

// bounds[0..2] = min centroid, [3..5] = max centroid, [6..8] min vertex, [9..11] max vertex
__global__ void k_triPrep(const float4* __restrict__ pos, const int* __restrict__ idx, int n, float4* triLo,
                          float4* triHi, float4* cent, float4* gnrm, float* area, unsigned int* bounds) {
    __shared__ unsigned int sb[12];
    if (threadIdx.x < 12) sb[threadIdx.x] = (threadIdx.x % 6) < 3 ? 0xFFFFFFFFu : 0u;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float4 a = pos[idx[3 * i]], b = pos[idx[3 * i + 1]], c = pos[idx[3 * i + 2]];
        float4 lo = make_float4(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)), 0);
        float4 hi = make_float4(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)), 0);
        triLo[i] = lo;
        triHi[i] = hi;
        float4 ce = make_float4((lo.x + hi.x) * 0.5f, (lo.y + hi.y) * 0.5f, (lo.z + hi.z) * 0.5f, 0);
        cent[i] = ce;
        // TriangleIndexed.h:56-62 and :154: cross in FP64, then float normalize / length.
        double e1x = (double)__fsub_rn(b.x, a.x), e1y = (double)__fsub_rn(b.y, a.y), e1z = (double)__fsub_rn(b.z, a.z);
        double e2x = (double)__fsub_rn(c.x, a.x), e2y = (double)__fsub_rn(c.y, a.y), e2z = (double)__fsub_rn(c.z, a.z);
        float cx = (float)(e1y * e2z - e1z * e2y), cy = (float)(e1z * e2x - e1x * e2z), cz = (float)(e1x * e2y - e1y * e2x);
        float len2 = __fadd_rn(__fadd_rn(__fmul_rn(cx, cx), __fmul_rn(cy, cy)), __fadd_rn(__fmul_rn(cz, cz), 0.0f));
        float len = __fsqrt_rn(len2);
        float inv = __fdiv_rn(1.0f, len);
        gnrm[i] = make_float4(__fmul_rn(cx, inv), __fmul_rn(cy, inv), __fmul_rn(cz, inv), 0.0f);
        area[i] = __fdiv_rn(len, 2.0f);
        atomicMin(&sb[0], orderedBits(ce.x)); atomicMin(&sb[1], orderedBits(ce.y)); atomicMin(&sb[2], orderedBits(ce.z));
        atomicMax(&sb[3], orderedBits(ce.x)); atomicMax(&sb[4], orderedBits(ce.y)); atomicMax(&sb[5], orderedBits(ce.z));
        atomicMin(&sb[6], orderedBits(lo.x)); atomicMin(&sb[7], orderedBits(lo.y)); atomicMin(&sb[8], orderedBits(lo.z));
        atomicMax(&sb[9], orderedBits(hi.x)); atomicMax(&sb[10], orderedBits(hi.y)); atomicMax(&sb[11], orderedBits(hi.z));
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        if ((threadIdx.x % 6) < 3) atomicMin(&bounds[threadIdx.x], sb[threadIdx.x]);
        else atomicMax(&bounds[threadIdx.x], sb[threadIdx.x]);
    }
}

__device__ __forceinline__ unsigned int expandBits(unsigned int v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(const float4* __restrict__ cent, int n, const unsigned int* __restrict__ bounds,
                         unsigned int* keys, unsigned int* vals) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float lo[3], ext[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = orderedFloat(bounds[k]);
        ext[k] = orderedFloat(bounds[3 + k]) - lo[k];
    }
    float4 c = cent[i];
    float v[3] = {c.x, c.y, c.z};
    unsigned int q[3];
    for (int k = 0; k < 3; ++k) {
        float t = ext[k] > 0.0f ? (v[k] - lo[k]) / ext[k] : 0.5f;
        t = fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f);
        q[k] = (unsigned int)t;
    }
    keys[i] = (expandBits(q[0]) << 2) | (expandBits(q[1]) << 1) | expandBits(q[2]);
    vals[i] = (unsigned int)i;
}

__device__ __forceinline__ int delta(const unsigned int* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned int a = keys[i], b = keys[j];
    if (a == b) return 32 + __clz((unsigned int)(i ^ j));
    return __clz(a ^ b);
}

// Node numbering: internal nodes 0 .. n-2 (root 0), leaf k is node n-1+k.
__global__ void k_karras(const unsigned int* __restrict__ keys, int n, int* left, int* right, int* first, int* last,
                         int* parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    int lc = (lo == gamma) ? (n - 1 + gamma) : gamma;
    int rc = (hi == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
    left[i] = lc;
    right[i] = rc;
    first[i] = lo;
    last[i] = hi;
    parent[lc] = i;
    parent[rc] = i;
    if (i == 0) parent[0] = -1;
}

__global__ void k_leafBoxes(const unsigned int* __restrict__ vals, int n, const float4* __restrict__ triLo,
                            const float4* __restrict__ triHi, float4* nodeLo, float4* nodeHi) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    unsigned int t = vals[k];
    nodeLo[n - 1 + k] = triLo[t];
    nodeHi[n - 1 + k] = triHi[t];
}

__global__ void k_bottomUp(int n, const int* __restrict__ parent, const int* __restrict__ left,
                           const int* __restrict__ right, float4* nodeLo, float4* nodeHi, unsigned int* arrivals) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int node = parent[n - 1 + k];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&arrivals[node], 1u) == 0u) return;
        int a = left[node], b = right[node];
        float4 al = __ldcg(&nodeLo[a]), ah = __ldcg(&nodeHi[a]);
        float4 bl = __ldcg(&nodeLo[b]), bh = __ldcg(&nodeHi[b]);
        __stcg(&nodeLo[node], make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f));
        __stcg(&nodeHi[node], make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f));
        node = parent[node];
    }
}

__device__ __forceinline__ int childCode(int c, int n, const int* first, const int* last) {
    if (c >= n - 1) return leafEncode(c - (n - 1), 1);
    int cnt = last[c] - first[c] + 1;
    if (cnt <= kLeafMax) return leafEncode(first[c], cnt);
    return c;
}

__global__ void k_emit(int n, const int* __restrict__ left, const int* __restrict__ right,
                       const int* __restrict__ first, const int* __restrict__ last, const float4* __restrict__ nodeLo,
                       const float4* __restrict__ nodeHi, Node2* nodes) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int a = left[i], b = right[i];
    float4 al = nodeLo[a], ah = nodeHi[a], bl = nodeLo[b], bh = nodeHi[b];
    Node2 nd;
    nd.a = make_float4(al.x, al.y, al.z, ah.x);
    nd.b = make_float4(ah.y, ah.z, bl.x, bl.y);
    nd.c = make_float4(bl.z, bh.x, bh.y, bh.z);
    nd.d = make_int4(childCode(a, n, first, last), childCode(b, n, first, last), 0, 0);
    nodes[i] = nd;
}

__global__ void k_gather(const unsigned int* __restrict__ vals, int n, const float4* __restrict__ pos,
                         const int* __restrict__ idx, TriV* tris) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int t = (int)vals[k];
    float4 a = pos[idx[3 * t]], b = pos[idx[3 * t + 1]], c = pos[idx[3 * t + 2]];
    TriV tv;
    tv.p0 = make_float4(a.x, a.y, a.z, __int_as_float(t));
    tv.p1 = make_float4(b.x, b.y, b.z, 0.0f);
    tv.p2 = make_float4(c.x, c.y, c.z, 0.0f);
    tris[k] = tv;
}

struct DeviceScratch {
    void* p = nullptr;
    ~DeviceScratch() { if (p) cudaFree(p); }
};

}  // namespace

cudaError_t buildBlas(const BlasBuildInput& in, BlasBuildOutput* out, cudaStream_t stream) {
    const int n = in.nTris;
    if (n <= 0) return cudaErrorInvalidValue;
    const int B = 256;
    const int G = (n + B - 1) / B;
    cudaError_t e;
    // scratch layout
    size_t nNodes = (size_t)2 * n - 1;
    size_t sortTemp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, sortTemp, (unsigned int*)nullptr, (unsigned int*)nullptr,
                                    (unsigned int*)nullptr, (unsigned int*)nullptr, n, 0, 30, stream);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
    size_t oTriLo = take(sizeof(float4) * n), oTriHi = take(sizeof(float4) * n), oCent = take(sizeof(float4) * n);
    size_t oBounds = take(sizeof(unsigned int) * 12);
    size_t oKeys = take(4 * (size_t)n), oVals = take(4 * (size_t)n), oKeys2 = take(4 * (size_t)n), oVals2 = take(4 * (size_t)n);
    size_t oLeft = take(4 * (size_t)n), oRight = take(4 * (size_t)n), oFirst = take(4 * (size_t)n), oLast = take(4 * (size_t)n);
    size_t oParent = take(4 * nNodes), oArr = take(4 * (size_t)n);
    size_t oNLo = take(sizeof(float4) * nNodes), oNHi = take(sizeof(float4) * nNodes);
    size_t oSort = take(sortTemp);
    DeviceScratch scratch;
    if ((e = cudaMalloc(&scratch.p, off)) != cudaSuccess) return e;
    char* base = (char*)scratch.p;
    float4* triLo = (float4*)(base + oTriLo);
    float4* triHi = (float4*)(base + oTriHi);
    float4* cent = (float4*)(base + oCent);
    unsigned int* bounds = (unsigned int*)(base + oBounds);
    unsigned int *keys = (unsigned int*)(base + oKeys), *vals = (unsigned int*)(base + oVals);
    unsigned int *keys2 = (unsigned int*)(base + oKeys2), *vals2 = (unsigned int*)(base + oVals2);
    int *left = (int*)(base + oLeft), *right = (int*)(base + oRight), *first = (int*)(base + oFirst),
        *last = (int*)(base + oLast), *parent = (int*)(base + oParent);
    unsigned int* arrivals = (unsigned int*)(base + oArr);
    float4 *nodeLo = (float4*)(base + oNLo), *nodeHi = (float4*)(base + oNHi);

    unsigned int initBounds[12];
    for (int k = 0; k < 12; ++k) initBounds[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
    if ((e = cudaMemcpyAsync(bounds, initBounds, sizeof(initBounds), cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
    k_triPrep<<<G, B, 0, stream>>>(in.pos, in.idx, n, triLo, triHi, cent, out->gnrm, out->triArea, bounds);
    k_morton<<<G, B, 0, stream>>>(cent, n, bounds, keys, vals);
    if ((e = cub::DeviceRadixSort::SortPairs(base + oSort, sortTemp, keys, keys2, vals, vals2, n, 0, 30, stream)) != cudaSuccess)
        return e;
    if (n >= 2) {
        int Gi = (n - 1 + B - 1) / B;
        if ((e = cudaMemsetAsync(arrivals, 0, 4 * (size_t)n, stream)) != cudaSuccess) return e;
        k_karras<<<Gi, B, 0, stream>>>(keys2, n, left, right, first, last, parent);
        k_leafBoxes<<<G, B, 0, stream>>>(vals2, n, triLo, triHi, nodeLo, nodeHi);
        k_bottomUp<<<G, B, 0, stream>>>(n, parent, left, right, nodeLo, nodeHi, arrivals);
        k_emit<<<Gi, B, 0, stream>>>(n, left, right, first, last, nodeLo, nodeHi, out->nodes);
    }
    k_gather<<<G, B, 0, stream>>>(vals2, n, in.pos, in.idx, out->tris);
    unsigned int hb[12];
    if ((e = cudaMemcpyAsync(hb, bounds, sizeof(hb), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    for (int k = 0; k < 3; ++k) {
        out->boundsLo[k] = orderedFloat(hb[6 + k]);
        out->boundsHi[k] = orderedFloat(hb[9 + k]);
    }
    out->rootIsLeaf = n <= kLeafMax ? 1 : 0;
    out->rootLeaf = leafEncode(0, n <= kLeafMax ? n : 1);
    return cudaSuccess;
}

}  // namespace xgb
