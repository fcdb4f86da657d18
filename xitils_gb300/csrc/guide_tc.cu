// Inference of the guiding network on the fifth-generation tensor cores:
// tcgen05.mma with the accumulators in tensor memory (TMEM).
//
// A CTA holds kTcGroups warpgroups of 128 threads that share the staged weights;
// each warpgroup owns 128-row tiles on its own: thread t of the group builds
// row t's 64 features and writes them into the group's shared-memory A operand;
// the group's first thread issues the layer's four K = 16 steps
// (tcgen05.mma.cta_group::1.kind::f16, M = 128, BF16 operands from shared
// memory, FP32 accumulation in the group's 64 TMEM columns) and commits them to
// the group's mbarrier; after the wait, warp w of the group reads TMEM lanes
// 32 (w mod 4) .. + 31 (its rows) with tcgen05.ld, adds the bias, applies ReLU
// and overwrites the A operand with the next layer's input (the MMAs that read
// it have completed). The last layer's 48 accumulator columns go straight from
// TMEM to the thread that decodes its row's mixture. The weights (B operands,
// [N][64] row-major, K-major) are staged once per CTA. The groups synchronise
// with named barriers (id 1 + group), the CTA only around set-up and teardown.
//
// Operand layout (no swizzle, K-major): 8 x 8 BF16 core matrices of 128
// contiguous bytes; the core matrices of a row group are consecutive along K
// (leading-dimension byte offset 128), row groups of 8 follow each other every
// 1024 bytes (stride-dimension byte offset). A K = 16 step advances the operand
// start by two core matrices (256 bytes).
//
// The path kernel is latency-bound (the hit reconstruction before the first
// layer is a chain of dependent loads), so residency matters more than the
// matrix work: two groups per CTA and 63.5 KB of shared memory give three CTAs,
// 24 warps, per SM; the launch is a multiple of the resident CTAs and every
// group walks its tiles with a grid stride.
//
// Waits are bounded: an mbarrier wait that does not complete within its limit
// (GuideDevice::waitLimit polls, 2^22 unless a test lowers it)
// is voted on by the group, sets ERR_WAIT in the launch's error word (the render
// returns XGB_DEVICE_TIMEOUT), waits once more (bounded) for the group's MMAs in
// flight and leaves the group's loop; the CTA then frees its TMEM columns.
#include <cuda_bf16.h>

#include "guide.cuh"
#include "guide_kernels.h"
#include "materials.cuh"

namespace xgb {
namespace {

constexpr int kTcRows = 128;                   // rows per tile = TMEM lanes = threads per group
constexpr int kTcGroups = 2;                   // warpgroups per CTA
constexpr int kTcThreads = kTcRows * kTcGroups;
constexpr int kTcCols = 64 * kTcGroups;        // TMEM columns allocated: 64 FP32 accumulators per group
constexpr int kTcCtasPerSm = 3;                // launch = SMs x this x waves
constexpr int kTcWaves = 2;
constexpr int kTcWaitLimit = 1 << 22;  // polls of the wait for MMAs in flight after a timeout

struct __align__(1024) TcSmem {
    __nv_bfloat16 w[3][64 * 64];                   // layers 0-2 (B operands, core-matrix layout)
    __nv_bfloat16 w3[kGuideOutPad * 64];
    __nv_bfloat16 a[kTcGroups][kTcRows * 64];      // activations (A operands), one per group
    float bias[3 * 64 + kGuideOutPad];
    unsigned long long mbar[kTcGroups];
    unsigned int tmem;
};

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (r, k) of a K-major [rows][64] BF16 operand (see the header).
__device__ __forceinline__ uint32_t coreOffset(int r, int k) {
    return (uint32_t)((r >> 3) * 1024 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading-dimension byte offset
// (128), stride-dimension byte offset (1024), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t matDesc(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(1024u >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
template <int N>
__device__ __forceinline__ uint32_t instrDesc() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
}

__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Named barrier of one warpgroup (ids 1 and 2; 0 is __syncthreads). The ids are
// immediates so that the kernel reserves three barriers, not all sixteen.
static_assert(kTcGroups == 2, "one named barrier per warpgroup below");
__device__ __forceinline__ void groupSync(int group) {
    if (group == 0)
        asm volatile("bar.sync 1, %0;" ::"n"(kTcRows) : "memory");
    else
        asm volatile("bar.sync 2, %0;" ::"n"(kTcRows) : "memory");
}
// The same barrier, returning whether v holds for every thread of the group.
__device__ __forceinline__ bool groupAll(int group, bool v) {
    uint32_t r;
    if (group == 0)
        asm volatile(
            "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
            "bar.red.and.pred q, 1, %2, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
            : "=r"(r)
            : "r"((uint32_t)v), "n"(kTcRows)
            : "memory");
    else
        asm volatile(
            "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
            "bar.red.and.pred q, 2, %2, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
            : "=r"(r)
            : "r"((uint32_t)v), "n"(kTcRows)
            : "memory");
    return r != 0;
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// Bounded wait for the mbarrier phase of the given parity: at most `limit` polls.
__device__ __forceinline__ bool mbarWait(uint32_t mbar, uint32_t parity, int limit = kTcWaitLimit) {
    for (int it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmemWaitLoad() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t packBf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// Row r's 64 values as BF16 into an A operand.
__device__ __forceinline__ void storeRow(__nv_bfloat16* A, int r, const float* v) {
    char* base = reinterpret_cast<char*>(A);
#pragma unroll
    for (int g = 0; g < 8; ++g) {
        uint4 q;
        q.x = packBf16(v[8 * g], v[8 * g + 1]);
        q.y = packBf16(v[8 * g + 2], v[8 * g + 3]);
        q.z = packBf16(v[8 * g + 4], v[8 * g + 5]);
        q.w = packBf16(v[8 * g + 6], v[8 * g + 7]);
        *reinterpret_cast<uint4*>(base + coreOffset(r, 8 * g)) = q;
    }
}

// Per-CTA set-up: TMEM columns (warp 0), the groups' mbarriers, the weights and biases.
__device__ __forceinline__ void tcSetup(TcSmem& S, const GuideWeights& w) {
    const int tid = threadIdx.x;
    if (tid < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(&S.tmem)),
                     "r"((uint32_t)kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
#pragma unroll
        for (int g = 0; g < kTcGroups; ++g)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemAddr(&S.mbar[g])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int c = tid; c < 3 * 64 * 8; c += kTcThreads) {  // 16-byte chunks: layer, row, k group
        const int l = c / 512, rr = (c / 8) % 64, g = c % 8;
        const uint4 v = *reinterpret_cast<const uint4*>(w.W[l] + rr * 64 + 8 * g);
        *reinterpret_cast<uint4*>(reinterpret_cast<char*>(S.w[l]) + coreOffset(rr, 8 * g)) = v;
    }
    for (int c = tid; c < kGuideOutPad * 8; c += kTcThreads) {
        const int rr = c / 8, g = c % 8;
        const uint4 v = *reinterpret_cast<const uint4*>(w.W[3] + rr * 64 + 8 * g);
        *reinterpret_cast<uint4*>(reinterpret_cast<char*>(S.w3) + coreOffset(rr, 8 * g)) = v;
    }
    for (int c = tid; c < 3 * 64 + kGuideOutPad; c += kTcThreads)
        S.bias[c] = c < 192 ? w.bias[c / 64][c % 64] : w.bias[3][c - 192];
    tcFenceBefore();  // the allocated TMEM address in S.tmem
    __syncthreads();
    tcFenceAfter();
}

__device__ __forceinline__ void tcTeardown(TcSmem& S) {
    tcFenceBefore();
    __syncthreads();
    tcFenceAfter();
    if (threadIdx.x < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(S.tmem), "r"((uint32_t)kTcCols)
                     : "memory");
}

// One layer of one group: its A operand (written by every thread of the group
// before the call) times B^T into the group's TMEM columns, then row r's N
// outputs (+ bias) for the thread of row r. Returns false on a timed-out wait
// (the whole group agrees).
template <int N>
__device__ __forceinline__ bool tcLayer(TcSmem& S, int group, const __nv_bfloat16* B, uint32_t& parity,
                                        float (&out)[64], const float* bias, int waitLimit) {
    fenceProxyAsync();  // the operand stores become visible to the tensor cores
    tcFenceBefore();
    groupSync(group);
    tcFenceAfter();
    const uint32_t tmem = S.tmem + 64u * (uint32_t)group;
    const uint32_t mbar = smemAddr(&S.mbar[group]);
    if ((threadIdx.x & (kTcRows - 1)) == 0) {
        const uint32_t a0 = smemAddr(S.a[group]), b0 = smemAddr(B);
#pragma unroll
        for (int j = 0; j < 4; ++j) mma(tmem, matDesc(a0 + 256u * j), matDesc(b0 + 256u * j), instrDesc<N>(), j > 0);
        commit(mbar);
    }
    const bool done = mbarWait(mbar, parity, waitLimit);
    parity ^= 1u;
    if (!groupAll(group, done)) return false;
    tcFenceAfter();
    const uint32_t lane = (uint32_t)(threadIdx.x & 0x60) << 16;  // this warp's quarter of the TMEM lanes
#pragma unroll
    for (int c = 0; c < N / 16; ++c) {
        float v[16];
        tmemLoad16(tmem + lane + 16u * c, v);
        tmemWaitLoad();
#pragma unroll
        for (int k = 0; k < 16; ++k) out[16 * c + k] = v[k] + bias[16 * c + k];
    }
    return true;
}

// The four layers for the group's tile, whose features are in its A operand;
// row r's 40 outputs in y (the first kGuideOut of 48). Returns false on a
// timed-out wait.
__device__ __forceinline__ bool tcForward(TcSmem& S, int group, int r, uint32_t& parity, float (&y)[64],
                                          int waitLimit) {
    float h[64];
#pragma unroll
    for (int l = 0; l < 3; ++l) {
        if (!tcLayer<64>(S, group, S.w[l], parity, h, S.bias + 64 * l, waitLimit)) return false;
#pragma unroll
        for (int k = 0; k < 64; ++k) h[k] = fmaxf(h[k], 0.0f);
        storeRow(S.a[group], r, h);
    }
    return tcLayer<kGuideOutPad>(S, group, S.w3, parity, y, S.bias + 192, waitLimit);
}

// After a timed-out wait: the error bit, then a bounded second wait for the
// group's MMAs still in flight (parity has already been advanced past them).
__device__ __forceinline__ void tcAbort(TcSmem& S, int group, uint32_t parity, unsigned int* errors) {
    if ((threadIdx.x & (kTcRows - 1)) == 0) atomicOr(errors, ERR_WAIT);
    mbarWait(smemAddr(&S.mbar[group]), parity ^ 1u);
}

// Rows of feature vectors (xgb_guide_infer / xgb_guide_sample): X0 [rows][64]
// BF16, Y [rows][48] FP32.
__global__ void __launch_bounds__(kTcThreads, kTcCtasPerSm) k_inferRowsTc(const __nv_bfloat16* X0, int rows, GuideWeights w,
                                                            float* Y, unsigned int* errors, int waitLimit) {
    extern __shared__ unsigned char tcRaw[];
    TcSmem& S = *reinterpret_cast<TcSmem*>(tcRaw);
    tcSetup(S, w);
    uint32_t parity = 0;
    const int group = threadIdx.x / kTcRows, r = threadIdx.x & (kTcRows - 1);
    const int stride = gridDim.x * kTcGroups;
    for (int tile = blockIdx.x * kTcGroups + group; tile * kTcRows < rows; tile += stride) {
        const int i = tile * kTcRows + r;
        char* dst = reinterpret_cast<char*>(S.a[group]);
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const uint4 v = i < rows ? *reinterpret_cast<const uint4*>(X0 + (size_t)i * 64 + 8 * g) : make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4*>(dst + coreOffset(r, 8 * g)) = v;
        }
        float y[64];
        if (!tcForward(S, group, r, parity, y, waitLimit)) {
            tcAbort(S, group, parity, errors);
            break;
        }
        if (i < rows)
#pragma unroll
            for (int k = 0; k < kGuideOutPad; ++k) Y[(size_t)i * kGuideOutPad + k] = y[k];
    }
    tcTeardown(S);
}

// Per-path inference of the wavefront: each hit of the input queue gets its
// 8-lobe mixture (10 float4: the lobes' (mu, kappa), then the 8 weights).
__global__ void __launch_bounds__(kTcThreads, kTcCtasPerSm) k_inferPathsTc(SceneDev sc, GuideWeights w, GuideBounds gb, PathQueue q,
                                                             HitQueue h, Ctrl* ctrl, float4* mix, int waitLimit) {
    extern __shared__ unsigned char tcRaw[];
    TcSmem& S = *reinterpret_cast<TcSmem*>(tcRaw);
    const unsigned int n = ctrl->nActive;
    // CTAs without a tile (the short queues at the end of a render) leave before
    // allocating TMEM and staging the weights
    if (blockIdx.x * (unsigned int)(kTcGroups * kTcRows) >= n) return;
    tcSetup(S, w);
    uint32_t parity = 0;
    const int group = threadIdx.x / kTcRows, r = threadIdx.x & (kTcRows - 1);
    const unsigned int stride = gridDim.x * (unsigned int)(kTcGroups * kTcRows);
    for (unsigned int base = (blockIdx.x * kTcGroups + group) * (unsigned int)kTcRows; base < n; base += stride) {
        const unsigned int i = base + r;
        float f[64];
        bool valid = false;
        if (i < n) {
            const float4 hh = h.h[i];
            const int prim = __float_as_int(hh.w);
            if (prim >= 0) {
                const float4 d4 = q.d[i];
                const Surface s = makeSurface(sc, sc.instances[h.inst[i]], prim, hh.y, hh.z, V3(d4.x, d4.y, d4.z));
                const float pf[3] = {(s.p.x - gb.lo[0]) * gb.invExtent[0], (s.p.y - gb.lo[1]) * gb.invExtent[1],
                                     (s.p.z - gb.lo[2]) * gb.invExtent[2]};
                const float nf[3] = {s.sn.x, s.sn.y, s.sn.z}, wf[3] = {s.wo.x, s.wo.y, s.wo.z};
                guideFeatures(pf, nf, wf, f);
                valid = true;
            }
        }
        if (!valid)
#pragma unroll
            for (int k = 0; k < 64; ++k) f[k] = 0.0f;
        storeRow(S.a[group], r, f);
        float y[64];
        if (!tcForward(S, group, r, parity, y, waitLimit)) {
            tcAbort(S, group, parity, &ctrl->errors);
            break;
        }
        if (i < n) {
            VmfMixture mx;
            decodeMixture(y, mx);
            float4* o = mix + (size_t)i * 10;
#pragma unroll
            for (int j = 0; j < kGuideLobes; ++j)
                __stcs(o + j, make_float4(mx.lobe[j].mu.x, mx.lobe[j].mu.y, mx.lobe[j].mu.z, mx.lobe[j].kappa));
            __stcs(o + 8, make_float4(mx.lobe[0].alpha, mx.lobe[1].alpha, mx.lobe[2].alpha, mx.lobe[3].alpha));
            __stcs(o + 9, make_float4(mx.lobe[4].alpha, mx.lobe[5].alpha, mx.lobe[6].alpha, mx.lobe[7].alpha));
        }
    }
    tcTeardown(S);
}

int gLaunchCtas = 0;  // CTAs per launch of the inference kernels (set by guideTcPrepare)

}  // namespace

cudaError_t guideTcPrepare() {
    const int bytes = (int)sizeof(TcSmem);
    cudaError_t e = cudaFuncSetAttribute(k_inferRowsTc, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_inferPathsTc, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    int dev = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) gLaunchCtas = sms * kTcCtasPerSm * kTcWaves;
    return e;
}

void guideInferRows(const GuideDevice& g, const __nv_bfloat16* X0, int rowsPad, float* Y, cudaStream_t s) {
    const int groups = (rowsPad + kTcRows - 1) / kTcRows;
    int grid = (groups + kTcGroups - 1) / kTcGroups;
    if (gLaunchCtas > 0 && grid > gLaunchCtas) grid = gLaunchCtas;
    k_inferRowsTc<<<grid > 0 ? grid : 1, kTcThreads, sizeof(TcSmem), s>>>(
        X0, rowsPad, g.w, Y, reinterpret_cast<unsigned int*>(g.scratch.scalars + 2), g.waitLimit);
}

void guideInferPaths(const SceneDev& sc, const GuideDevice& g, GuideBounds gb, PathQueue q, HitQueue h, Ctrl* ctrl,
                     float4* mix, int grid, cudaStream_t s) {
    if (gLaunchCtas > 0) grid = gLaunchCtas;
    k_inferPathsTc<<<grid, kTcThreads, sizeof(TcSmem), s>>>(sc, g.w, gb, q, h, ctrl, mix, g.waitLimit);
}

}  // namespace xgb
