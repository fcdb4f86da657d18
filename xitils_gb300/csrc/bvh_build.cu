// GPU construction of a per-mesh bounding-volume hierarchy (the reference
// builds its _BVH single-threaded on the CPU, AccelerationStructure.h:163-291;
// the tree shape affects speed only, never the image).
//
// Two builders share steps 1-2 and the output format:
//   1. per triangle: bounds, centroid, FP64-cross geometric normal, area;
//   2. 30-bit Morton codes of the centroids, radix-sorted (CUB);
// PLOC (default), Meister & Bittner, "Parallel Locally-Ordered Clustering for
// Bounding Volume Hierarchy Construction" (TVCG 2018): clusters start as the
// sorted triangles; every round each cluster finds the neighbour within
// kPlocRadius positions of the sorted order whose merged box has the smallest
// surface area, mutual nearest neighbours merge into a new node, and the
// cluster list is compacted in order, until one cluster is left. Merging by
// box area tracks SAH quality far more closely than Morton splits on scenes
// of overlapping or very unevenly sized triangles.
// LBVH, Karras, "Maximizing Parallelism in the Construction of BVHs, Octrees,
// and k-d Trees" (HPG 2012): one thread per internal node finds its key range
// and split; bounds propagate bottom-up (the second child to arrive merges).
// Output: subtrees of <= kLeafMax triangles collapse into leaves; each inner
// node is a 64-byte Node2 holding both children's boxes (root at index 0); the
// triangle vertices are gathered into leaf order (48 B per triangle).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

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

// ---- PLOC -------------------------------------------------------------------
// Node ids: leaf k (k-th triangle in Morton order) is k; internal nodes are
// n .. 2n-2 in creation order (the root is created last). Output Node2 index of
// internal node id is (2n-2) - id, so the root lands at 0.
constexpr int kPlocRadius = 16;
constexpr int kPlocBlock = 256;

__device__ __forceinline__ float halfArea(float4 lo, float4 hi) {
    float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_plocInit(const unsigned int* __restrict__ vals, int n, const float4* __restrict__ triLo,
                           const float4* __restrict__ triHi, float4* nodeLo, float4* nodeHi, int* clusters, int* count,
                           int* parent) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    unsigned int t = vals[k];
    nodeLo[k] = triLo[t];
    nodeHi[k] = triHi[t];
    clusters[k] = k;
    count[k] = 1;
    parent[k] = -1;
}

__global__ void __launch_bounds__(kPlocBlock) k_plocNearest(const int* __restrict__ clusters, int nc,
                                                            const float4* __restrict__ nodeLo,
                                                            const float4* __restrict__ nodeHi, int* nn) {
    __shared__ float4 sLo[kPlocBlock + 2 * kPlocRadius], sHi[kPlocBlock + 2 * kPlocRadius];
    const int b0 = blockIdx.x * kPlocBlock;
    for (int t = threadIdx.x; t < kPlocBlock + 2 * kPlocRadius; t += kPlocBlock) {
        int j = b0 - kPlocRadius + t;
        if (j >= 0 && j < nc) {
            int id = clusters[j];
            sLo[t] = nodeLo[id];
            sHi[t] = nodeHi[id];
        }
    }
    __syncthreads();
    const int i = b0 + threadIdx.x;
    if (i >= nc) return;
    const int si = threadIdx.x + kPlocRadius;
    const float4 lo = sLo[si], hi = sHi[si];
    float best = __int_as_float(0x7f800000);
    int bestJ = -1;
    const int jLo = max(0, i - kPlocRadius), jHi = min(nc - 1, i + kPlocRadius);
    for (int j = jLo; j <= jHi; ++j) {
        if (j == i) continue;
        const float4 l2 = sLo[j - b0 + kPlocRadius], h2 = sHi[j - b0 + kPlocRadius];
        float a = halfArea(make_float4(fminf(lo.x, l2.x), fminf(lo.y, l2.y), fminf(lo.z, l2.z), 0.f),
                           make_float4(fmaxf(hi.x, h2.x), fmaxf(hi.y, h2.y), fmaxf(hi.z, h2.z), 0.f));
        if (a < best || bestJ < 0) { best = a; bestJ = j; }  // ascending j: ties go to the lower index
    }
    nn[i] = bestJ;
}

__global__ void k_plocMerge(int* clusters, int nc, const int* __restrict__ nn, int n, float4* nodeLo, float4* nodeHi,
                            int* left, int* right, int* parent, int* count, int* counter, int* keep) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const int j = nn[i];
    const bool mutual = j >= 0 && nn[j] == i;
    if (mutual && i < j) {
        const int a = clusters[i], b = clusters[j];
        const int id = n + atomicAdd(counter, 1);
        const float4 al = nodeLo[a], ah = nodeHi[a], bl = nodeLo[b], bh = nodeHi[b];
        nodeLo[id] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.f);
        nodeHi[id] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.f);
        left[id - n] = a;
        right[id - n] = b;
        parent[a] = id;
        parent[b] = id;
        parent[id] = -1;
        count[id] = count[a] + count[b];
        clusters[i] = id;  // only this thread touches slot i; slot j is dropped by its own thread
        keep[i] = 1;
    } else {
        keep[i] = mutual ? 0 : 1;
    }
}

// Position of every node's first triangle in depth-first (left before right) order.
__global__ void k_dfsOffset(int nNodes, int n, const int* __restrict__ parent, const int* __restrict__ left,
                            const int* __restrict__ right, const int* __restrict__ count, int* dfs) {
    const int x0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (x0 >= nNodes) return;
    int off = 0, x = x0;
    for (int p = parent[x]; p >= 0; x = p, p = parent[x])
        if (right[p - n] == x) off += count[left[p - n]];
    dfs[x0] = off;
}

__device__ __forceinline__ int plocChild(int c, int n, const int* count, const int* dfs) {
    const int cnt = count[c];
    if (cnt <= kLeafMax) return leafEncode(dfs[c], cnt);
    return (2 * n - 2) - c;
}

__global__ void k_plocEmit(int n, const int* __restrict__ left, const int* __restrict__ right,
                           const int* __restrict__ count, const int* __restrict__ dfs, const float4* __restrict__ nodeLo,
                           const float4* __restrict__ nodeHi, Node2* nodes) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n - 1) return;
    const int id = n + k;
    const int a = left[k], b = right[k];
    const float4 al = nodeLo[a], ah = nodeHi[a], bl = nodeLo[b], bh = nodeHi[b];
    Node2 nd;
    nd.a = make_float4(al.x, al.y, al.z, ah.x);
    nd.b = make_float4(ah.y, ah.z, bl.x, bl.y);
    nd.c = make_float4(bl.z, bh.x, bh.y, bh.z);
    nd.d = make_int4(plocChild(a, n, count, dfs), plocChild(b, n, count, dfs), 0, 0);
    nodes[(2 * n - 2) - id] = nd;
}

__global__ void k_plocGather(const unsigned int* __restrict__ vals, int n, const int* __restrict__ dfs,
                             const float4* __restrict__ pos, const int* __restrict__ idx, TriV* tris) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int t = (int)vals[k];
    const float4 a = pos[idx[3 * t]], b = pos[idx[3 * t + 1]], c = pos[idx[3 * t + 2]];
    TriV tv;
    tv.p0 = make_float4(a.x, a.y, a.z, __int_as_float(t));
    tv.p1 = make_float4(b.x, b.y, b.z, 0.0f);
    tv.p2 = make_float4(c.x, c.y, c.z, 0.0f);
    tris[dfs[k]] = tv;
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
    // PLOC: second cluster list, nearest neighbours, keep flags, counts, DFS offsets, counters, select scratch
    const bool ploc = in.builder == kBuilderPloc;
    size_t selTemp = 0;
    if (ploc)
        cub::DeviceSelect::Flagged(nullptr, selTemp, (int*)nullptr, (int*)nullptr, (int*)nullptr, (int*)nullptr, n, stream);
    size_t oClB = ploc ? take(4 * (size_t)n) : 0, oNN = ploc ? take(4 * (size_t)n) : 0;
    size_t oKeep = ploc ? take(4 * (size_t)n) : 0, oCount = ploc ? take(4 * nNodes) : 0;
    size_t oDfs = ploc ? take(4 * nNodes) : 0, oCounters = ploc ? take(16) : 0;
    size_t oSel = ploc ? take(selTemp) : 0;
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
    if (ploc) {
        int* clA = (int*)(base + oKeys);  // the unsorted keys are free once sorted
        int* clB = (int*)(base + oClB);
        int* nn = (int*)(base + oNN);
        int* keep = (int*)(base + oKeep);
        int* count = (int*)(base + oCount);
        int* dfs = (int*)(base + oDfs);
        int* counters = (int*)(base + oCounters);  // [0] nodes created, [1] clusters selected
        if ((e = cudaMemsetAsync(counters, 0, 16, stream)) != cudaSuccess) return e;
        k_plocInit<<<G, B, 0, stream>>>(vals2, n, triLo, triHi, nodeLo, nodeHi, clA, count, parent);
        int nc = n;
        int* hostCount = nullptr;
        if ((e = cudaMallocHost((void**)&hostCount, 4)) != cudaSuccess) return e;
        for (int round = 0; nc > 1; ++round) {
            if (round > 4 * 1024) { cudaFreeHost(hostCount); return cudaErrorUnknown; }  // cannot happen: a round merges >= 1 pair
            const int Gc = (nc + kPlocBlock - 1) / kPlocBlock;
            k_plocNearest<<<Gc, kPlocBlock, 0, stream>>>(clA, nc, nodeLo, nodeHi, nn);
            k_plocMerge<<<Gc, kPlocBlock, 0, stream>>>(clA, nc, nn, n, nodeLo, nodeHi, left, right, parent, count,
                                                        counters, keep);
            size_t tb = selTemp;
            if ((e = cub::DeviceSelect::Flagged(base + oSel, tb, clA, keep, clB, counters + 1, nc, stream)) != cudaSuccess) break;
            if ((e = cudaMemcpyAsync(hostCount, counters + 1, 4, cudaMemcpyDeviceToHost, stream)) != cudaSuccess) break;
            if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) break;
            nc = *hostCount;
            std::swap(clA, clB);
        }
        cudaFreeHost(hostCount);
        if (e != cudaSuccess) return e;
        const int nAll = 2 * n - 1;
        k_dfsOffset<<<(nAll + B - 1) / B, B, 0, stream>>>(nAll, n, parent, left, right, count, dfs);
        if (n >= 2) k_plocEmit<<<(n - 1 + B - 1) / B, B, 0, stream>>>(n, left, right, count, dfs, nodeLo, nodeHi, out->nodes);
        k_plocGather<<<G, B, 0, stream>>>(vals2, n, dfs, in.pos, in.idx, out->tris);
    } else {
        if (n >= 2) {
            int Gi = (n - 1 + B - 1) / B;
            if ((e = cudaMemsetAsync(arrivals, 0, 4 * (size_t)n, stream)) != cudaSuccess) return e;
            k_karras<<<Gi, B, 0, stream>>>(keys2, n, left, right, first, last, parent);
            k_leafBoxes<<<G, B, 0, stream>>>(vals2, n, triLo, triHi, nodeLo, nodeHi);
            k_bottomUp<<<G, B, 0, stream>>>(n, parent, left, right, nodeLo, nodeHi, arrivals);
            k_emit<<<Gi, B, 0, stream>>>(n, left, right, first, last, nodeLo, nodeHi, out->nodes);
        }
        k_gather<<<G, B, 0, stream>>>(vals2, n, in.pos, in.idx, out->tris);
    }
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
