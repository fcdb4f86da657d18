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
// Output: the binary tree becomes an 8-wide compressed BVH (WNode, xgb_types.h),
// top down, one round per level: a wide node takes a binary node's two
// children and keeps opening the child of largest surface area until it has
// eight (subtrees of <= kWideLeafMax triangles may stay closed as leaf
// children), assigns them to slots by direction octant, quantises their boxes
// to 8 bits against its own box (rounded outwards), and gathers the leaf
// children's triangles next to each other (48 B per triangle).
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

// ---- LBVH -> the PLOC numbering used by the wide conversion ----------------------
// LBVH internal node i becomes n + i (root n), leaf n - 1 + k becomes k.
__global__ void k_lbvhUnify(int n, const int* __restrict__ left, const int* __restrict__ right,
                            const int* __restrict__ first, const int* __restrict__ last,
                            const float4* __restrict__ nodeLo, const float4* __restrict__ nodeHi, int* uLeft, int* uRight,
                            int* uCount, int* uStart, float4* uLo, float4* uHi) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= 2 * n - 1) return;
    if (x < n) {  // leaf x (LBVH id n - 1 + x)
        uCount[x] = 1;
        uStart[x] = x;
        uLo[x] = nodeLo[n - 1 + x];
        uHi[x] = nodeHi[n - 1 + x];
    } else {  // internal n + i (LBVH id i)
        const int i = x - n;
        auto map = [n](int c) { return c >= n - 1 ? c - (n - 1) : n + c; };
        uLeft[i] = map(left[i]);
        uRight[i] = map(right[i]);
        uCount[x] = last[i] - first[i] + 1;
        uStart[x] = first[i];
        uLo[x] = nodeLo[i];
        uHi[x] = nodeHi[i];
    }
}

// ---- binary -> 8-wide compressed BVH ------------------------------------------
struct WideItem {
    int bin;   // binary node id (PLOC numbering)
    int wide;  // WNode index it becomes
};

struct WideBuild {
    const int* left;   // [id - n] for internal ids
    const int* right;
    const int* count;  // triangles under each node
    const int* start;  // first triangle of each node in the binary-order triangle array
    const float4* lo;
    const float4* hi;
    const TriV* trisIn;  // binary (leaf) order
    int n;
    WNode* nodes;
    int nodeCap;
    TriV* trisOut;
    int* counters;  // [0] wide nodes used, [1] triangles placed, [2] items written, [3] error
};

__device__ __forceinline__ int wideExponent(float lo, float hi) {
    const float ext = __fsub_ru(hi, lo);
    if (!(ext > 0.0f)) return 1;  // flat axis: the smallest normal scale
    int x;
    frexpf(ext / 255.0f, &x);
    int e = x - 1;
    while (e < 127 && ldexpf(255.0f, e) < ext) ++e;
    while (e > -126 && ldexpf(255.0f, e - 1) >= ext) --e;
    return min(max(e, -126), 127) + 127;  // biased: 1 .. 254
}

__device__ __forceinline__ unsigned int quantLo(float c, float p, int eb) {
    double q = floor(((double)c - (double)p) * ldexp(1.0, 127 - eb)) - 1.0;  // one step outwards
    return (unsigned int)fmin(fmax(q, 0.0), 255.0);
}
__device__ __forceinline__ unsigned int quantHi(float c, float p, int eb) {
    double q = ceil(((double)c - (double)p) * ldexp(1.0, 127 - eb)) + 1.0;
    return (unsigned int)fmin(fmax(q, 0.0), 255.0);
}

__global__ void k_wideRound(WideBuild wb, const WideItem* in, int nIn, WideItem* out) {
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nIn) return;
    const int n = wb.n;
    const WideItem item = in[it];
    // children: open the largest-area inner child until there are eight
    int ch[8];
    int nch = 2;
    ch[0] = wb.left[item.bin - n];
    ch[1] = wb.right[item.bin - n];
    while (nch < 8) {
        int best = -1;
        float bestA = -1.0f;
        for (int j = 0; j < nch; ++j) {
            if (wb.count[ch[j]] < 2) continue;  // a single triangle cannot be opened
            float a = halfArea(wb.lo[ch[j]], wb.hi[ch[j]]);
            // subtrees too big for a leaf child must be opened or become wide nodes: prefer them on ties
            if (a > bestA || (a == bestA && wb.count[ch[j]] > kWideLeafMax)) { bestA = a; best = j; }
        }
        if (best < 0) break;
        const int c = ch[best];
        ch[best] = wb.left[c - n];
        ch[nch++] = wb.right[c - n];
    }
    // slot assignment: slot s takes the child furthest towards -dir(s), where bit k of
    // s set means a negative k component; greedy over the 8 x 8 costs
    const float4 plo = wb.lo[item.bin], phi = wb.hi[item.bin];
    const float cx = 0.5f * (plo.x + phi.x), cy = 0.5f * (plo.y + phi.y), cz = 0.5f * (plo.z + phi.z);
    int slotChild[8];
    for (int s = 0; s < 8; ++s) slotChild[s] = -1;
    unsigned int usedChild = 0, usedSlot = 0;
    for (int round = 0; round < nch; ++round) {
        float bestC = __int_as_float(0x7f800000);
        int bj = -1, bs = -1;
        for (int j = 0; j < nch; ++j) {
            if (usedChild >> j & 1) continue;
            const float4 l = wb.lo[ch[j]], h = wb.hi[ch[j]];
            const float dx = 0.5f * (l.x + h.x) - cx, dy = 0.5f * (l.y + h.y) - cy, dz = 0.5f * (l.z + h.z) - cz;
            for (int sl = 0; sl < 8; ++sl) {
                if (usedSlot >> sl & 1) continue;
                const float cost = ((sl & 1) ? -dx : dx) + ((sl & 2) ? -dy : dy) + ((sl & 4) ? -dz : dz);
                if (cost < bestC || bj < 0) { bestC = cost; bj = j; bs = sl; }
            }
        }
        usedChild |= 1u << bj;
        usedSlot |= 1u << bs;
        slotChild[bs] = ch[bj];
    }
    // allocation: inner children contiguous from childBase, leaf triangles from triBase
    int nInner = 0, nTri = 0;
    for (int s = 0; s < 8; ++s) {
        const int c = slotChild[s];
        if (c < 0) continue;
        if (wb.count[c] > kWideLeafMax) ++nInner;
        else nTri += wb.count[c];
    }
    const int childBase = nInner ? atomicAdd(&wb.counters[0], nInner) : 0;
    const int triBase = nTri ? atomicAdd(&wb.counters[1], nTri) : 0;
    if (childBase + nInner > wb.nodeCap || triBase + nTri > n) {
        atomicOr(&wb.counters[3], 1);
        return;
    }
    const int outBase = nInner ? atomicAdd(&wb.counters[2], nInner) : 0;
    // quantisation frame of this node
    const int ex = wideExponent(plo.x, phi.x), ey = wideExponent(plo.y, phi.y), ez = wideExponent(plo.z, phi.z);
    unsigned int imask = 0, meta[2] = {0, 0}, q[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    int kInner = 0, off = 0;
    for (int s = 0; s < 8; ++s) {
        const int c = slotChild[s];
        unsigned int mb = 0;
        const int w = s >> 2, sh = 8 * (s & 3);
        if (c >= 0) {
            const float4 l = wb.lo[c], h = wb.hi[c];
            q[0 + w] |= quantLo(l.x, plo.x, ex) << sh;
            q[2 + w] |= quantLo(l.y, plo.y, ey) << sh;
            q[4 + w] |= quantLo(l.z, plo.z, ez) << sh;
            q[6 + w] |= quantHi(h.x, plo.x, ex) << sh;
            q[8 + w] |= quantHi(h.y, plo.y, ey) << sh;
            q[10 + w] |= quantHi(h.z, plo.z, ez) << sh;
            const int cnt = wb.count[c];
            if (cnt > kWideLeafMax) {
                imask |= 1u << s;
                mb = (unsigned int)kInner;
                out[outBase + kInner] = WideItem{c, childBase + kInner};
                ++kInner;
            } else {
                mb = ((unsigned int)cnt << 5) | (unsigned int)off;
                for (int k = 0; k < cnt; ++k) wb.trisOut[triBase + off + k] = wb.trisIn[wb.start[c] + k];
                off += cnt;
            }
        } else {
            // empty slot: an inverted box that no slab test accepts
            q[0 + w] |= 255u << sh; q[2 + w] |= 255u << sh; q[4 + w] |= 255u << sh;
        }
        meta[w] |= mb << sh;
    }
    WNode nd;
    nd.a = make_float4(plo.x, plo.y, plo.z, __uint_as_float((unsigned)ex | ((unsigned)ey << 8) | ((unsigned)ez << 16) | (imask << 24)));
    nd.b = make_float4(__int_as_float(childBase), __int_as_float(triBase), __uint_as_float(meta[0]), __uint_as_float(meta[1]));
    nd.c = make_float4(__uint_as_float(q[0]), __uint_as_float(q[1]), __uint_as_float(q[2]), __uint_as_float(q[3]));
    nd.d = make_float4(__uint_as_float(q[4]), __uint_as_float(q[5]), __uint_as_float(q[6]), __uint_as_float(q[7]));
    nd.e = make_float4(__uint_as_float(q[8]), __uint_as_float(q[9]), __uint_as_float(q[10]), __uint_as_float(q[11]));
    wb.nodes[item.wide] = nd;
}

struct DeviceScratch {
    void* p = nullptr;
    ~DeviceScratch() { if (p) cudaFree(p); }
};

}  // namespace

cudaError_t buildBlas(const BlasBuildInput& in, BlasBuildOutput* out, cudaStream_t stream) {
    const int n = in.nTris;
    if (n <= 0) return cudaErrorInvalidValue;
    if (n >= (1 << 24)) return cudaErrorInvalidValue;  // node indices travel in 24 bits on the traversal stack
    out->nodes = nullptr;
    out->nodes2 = nullptr;
    out->nWide = 0;
    const bool wide = in.layout == kLayoutWide;
    out->wide = wide ? 1 : 0;
    const int B = 256;
    const int G = (n + B - 1) / B;
    cudaError_t e;
    // scratch layout
    const size_t nNodes = (size_t)2 * n - 1;
    size_t sortTemp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, sortTemp, (unsigned int*)nullptr, (unsigned int*)nullptr,
                                    (unsigned int*)nullptr, (unsigned int*)nullptr, n, 0, 30, stream);
    size_t selTemp = 0;
    cub::DeviceSelect::Flagged(nullptr, selTemp, (int*)nullptr, (int*)nullptr, (int*)nullptr, (int*)nullptr, n, stream);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
    const size_t oTriLo = take(sizeof(float4) * n), oTriHi = take(sizeof(float4) * n), oCent = take(sizeof(float4) * n);
    const size_t oBounds = take(sizeof(unsigned int) * 12);
    const size_t oKeys = take(4 * (size_t)n), oVals = take(4 * (size_t)n), oKeys2 = take(4 * (size_t)n),
                 oVals2 = take(4 * (size_t)n);
    const size_t oLeft = take(4 * (size_t)n), oRight = take(4 * (size_t)n), oFirst = take(4 * (size_t)n),
                 oLast = take(4 * (size_t)n);
    const size_t oParent = take(4 * nNodes), oArr = take(4 * (size_t)n);
    const size_t oNLo = take(sizeof(float4) * nNodes), oNHi = take(sizeof(float4) * nNodes);
    const size_t oSort = take(sortTemp);
    const size_t oClB = take(4 * (size_t)n), oNN = take(4 * (size_t)n), oKeep = take(4 * (size_t)n);
    const size_t oCount = take(4 * nNodes), oStart = take(4 * nNodes), oCounters = take(16), oSel = take(selTemp);
    // unified (PLOC-numbered) tree for the wide conversion: LBVH writes its own copy
    const size_t oULeft = take(4 * (size_t)n), oURight = take(4 * (size_t)n);
    const size_t oULo = take(sizeof(float4) * nNodes), oUHi = take(sizeof(float4) * nNodes);
    const size_t oTrisBin = take(sizeof(TriV) * n);
    const size_t oItemsA = take(sizeof(WideItem) * n), oItemsB = take(sizeof(WideItem) * n);
    const size_t oWide = take(sizeof(WNode) * n);  // upper bound: a wide node has >= 2 children
    const size_t oWCounters = take(16);
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
    int* count = (int*)(base + oCount);
    int* start = (int*)(base + oStart);
    TriV* trisBin = wide ? (TriV*)(base + oTrisBin) : out->tris;  // the binary layout gathers in place
    Node2* nodes2 = nullptr;
    if (!wide && n >= 2) {
        if ((e = cudaMalloc((void**)&nodes2, sizeof(Node2) * (size_t)(n - 1))) != cudaSuccess) return e;
        out->nodes2 = nodes2;  // the caller frees it, also on failure
    }
    int* hostCount = nullptr;
    if ((e = cudaMallocHost((void**)&hostCount, 16)) != cudaSuccess) return e;
    struct HostFree {
        int* p;
        ~HostFree() { cudaFreeHost(p); }
    } hostFree{hostCount};

    unsigned int initBounds[12];
    for (int k = 0; k < 12; ++k) initBounds[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
    if ((e = cudaMemcpyAsync(bounds, initBounds, sizeof(initBounds), cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
    k_triPrep<<<G, B, 0, stream>>>(in.pos, in.idx, n, triLo, triHi, cent, out->gnrm, out->triArea, bounds);
    k_morton<<<G, B, 0, stream>>>(cent, n, bounds, keys, vals);
    if ((e = cub::DeviceRadixSort::SortPairs(base + oSort, sortTemp, keys, keys2, vals, vals2, n, 0, 30, stream)) != cudaSuccess)
        return e;
    // binary tree in the PLOC numbering: left/right/count/start/boxes, root id, triangles in leaf order
    const int* uLeft = left;
    const int* uRight = right;
    const float4* uLo = nodeLo;
    const float4* uHi = nodeHi;
    int root = 2 * n - 2;
    if (in.builder == kBuilderPloc) {
        int* clA = (int*)(base + oKeys);  // the unsorted keys are free once sorted
        int* clB = (int*)(base + oClB);
        int* nn = (int*)(base + oNN);
        int* keep = (int*)(base + oKeep);
        int* counters = (int*)(base + oCounters);  // [0] nodes created, [1] clusters selected
        if ((e = cudaMemsetAsync(counters, 0, 16, stream)) != cudaSuccess) return e;
        k_plocInit<<<G, B, 0, stream>>>(vals2, n, triLo, triHi, nodeLo, nodeHi, clA, count, parent);
        int nc = n;
        for (int round = 0; nc > 1; ++round) {
            if (round > 4 * 1024) return cudaErrorUnknown;  // cannot happen: every round merges at least one pair
            const int Gc = (nc + kPlocBlock - 1) / kPlocBlock;
            k_plocNearest<<<Gc, kPlocBlock, 0, stream>>>(clA, nc, nodeLo, nodeHi, nn);
            k_plocMerge<<<Gc, kPlocBlock, 0, stream>>>(clA, nc, nn, n, nodeLo, nodeHi, left, right, parent, count,
                                                        counters, keep);
            size_t tb = selTemp;
            if ((e = cub::DeviceSelect::Flagged(base + oSel, tb, clA, keep, clB, counters + 1, nc, stream)) != cudaSuccess)
                return e;
            if ((e = cudaMemcpyAsync(hostCount, counters + 1, 4, cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
            if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
            nc = *hostCount;
            std::swap(clA, clB);
        }
        const int nAll = 2 * n - 1;
        k_dfsOffset<<<(nAll + B - 1) / B, B, 0, stream>>>(nAll, n, parent, left, right, count, start);
        if (!wide && n >= 2)
            k_plocEmit<<<(n - 1 + B - 1) / B, B, 0, stream>>>(n, left, right, count, start, nodeLo, nodeHi, nodes2);
        k_plocGather<<<G, B, 0, stream>>>(vals2, n, start, in.pos, in.idx, trisBin);
    } else {
        if (n >= 2) {
            const int Gi = (n - 1 + B - 1) / B;
            if ((e = cudaMemsetAsync(arrivals, 0, 4 * (size_t)n, stream)) != cudaSuccess) return e;
            k_karras<<<Gi, B, 0, stream>>>(keys2, n, left, right, first, last, parent);
            k_leafBoxes<<<G, B, 0, stream>>>(vals2, n, triLo, triHi, nodeLo, nodeHi);
            k_bottomUp<<<G, B, 0, stream>>>(n, parent, left, right, nodeLo, nodeHi, arrivals);
            if (!wide) k_emit<<<Gi, B, 0, stream>>>(n, left, right, first, last, nodeLo, nodeHi, nodes2);
            int* ul = (int*)(base + oULeft);
            int* ur = (int*)(base + oURight);
            float4* ulo = (float4*)(base + oULo);
            float4* uhi = (float4*)(base + oUHi);
            k_lbvhUnify<<<((int)nNodes + B - 1) / B, B, 0, stream>>>(n, left, right, first, last, nodeLo, nodeHi, ul, ur,
                                                                      count, start, ulo, uhi);
            uLeft = ul; uRight = ur; uLo = ulo; uHi = uhi;
            root = n;
        }
        k_gather<<<G, B, 0, stream>>>(vals2, n, in.pos, in.idx, trisBin);
    }
    // binary -> 8-wide, one round per wide level
    if (!wide) {
        // binary layout: done (Node2 nodes emitted, triangles gathered in leaf order)
    } else if (n <= kWideLeafMax) {
        if ((e = cudaMemcpyAsync(out->tris, trisBin, sizeof(TriV) * n, cudaMemcpyDeviceToDevice, stream)) != cudaSuccess)
            return e;
    } else {
        WideItem* itA = (WideItem*)(base + oItemsA);
        WideItem* itB = (WideItem*)(base + oItemsB);
        int* wc = (int*)(base + oWCounters);
        const int init[4] = {1, 0, 0, 0};  // the root takes wide node 0
        if ((e = cudaMemcpyAsync(wc, init, 16, cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
        const WideItem rootItem{root, 0};
        if ((e = cudaMemcpyAsync(itA, &rootItem, sizeof(WideItem), cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
        WideBuild wb{uLeft, uRight, count, start, uLo, uHi, trisBin, n, (WNode*)(base + oWide), n, out->tris, wc};
        int nIn = 1;
        for (int level = 0; nIn > 0; ++level) {
            if (level > 4096) return cudaErrorUnknown;  // cannot happen: every level goes one binary level deeper
            if ((e = cudaMemsetAsync(wc + 2, 0, 4, stream)) != cudaSuccess) return e;
            k_wideRound<<<(nIn + 127) / 128, 128, 0, stream>>>(wb, itA, nIn, itB);
            if ((e = cudaMemcpyAsync(hostCount, wc, 16, cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
            if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
            if (hostCount[3]) return cudaErrorUnknown;  // capacity check failed (cannot happen for a valid tree)
            nIn = hostCount[2];
            std::swap(itA, itB);
        }
        const int nWide = hostCount[0];
        if (hostCount[1] != n) return cudaErrorUnknown;  // every triangle lands in exactly one leaf child
        WNode* nodes = nullptr;
        if ((e = cudaMalloc((void**)&nodes, sizeof(WNode) * nWide)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(nodes, base + oWide, sizeof(WNode) * nWide, cudaMemcpyDeviceToDevice, stream)) != cudaSuccess) {
            cudaFree(nodes);
            return e;
        }
        out->nodes = nodes;
        out->nWide = nWide;
    }
    unsigned int hb[12];
    if ((e = cudaMemcpyAsync(hb, bounds, sizeof(hb), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    for (int k = 0; k < 3; ++k) {
        out->boundsLo[k] = orderedFloat(hb[6 + k]);
        out->boundsHi[k] = orderedFloat(hb[9 + k]);
    }
    const int rootMax = wide ? kWideLeafMax : kLeafMax;
    out->rootIsLeaf = n <= rootMax ? 1 : 0;
    out->rootLeaf = leafEncode(0, n <= rootMax ? n : 1);
    return cudaSuccess;
}

}  // namespace xgb
