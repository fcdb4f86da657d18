// Guiding network kernels: BF16 tensor-core (mma.sync m16n8k16, FP32
// accumulation) inference and training of the 64-64-64-64-40 MLP, Adam, and
// the per-path inference pass of the wavefront.
//
// Layouts: activations are row-major bf16 [rows][64]; W_l is row-major bf16
// [out][in] (out padded to 48 for the last layer) and WT_l its transpose
// [in][out]. Fragment layouts follow the PTX ISA for mma.m16n8k16 .row.col:
//   A (16x16): a0 = (g, 2t..2t+1), a1 = (g+8, 2t..), a2 = (g, 2t+8..), a3 = (g+8, 2t+8..)
//   B (16x8):  b0 = (k 2t..2t+1, n g), b1 = (k 2t+8.., n g)
//   C (16x8):  c0,c1 = (g, 2t..2t+1), c2,c3 = (g+8, 2t..)
// with g = lane / 4, t = lane % 4. Every operand is read as 32-bit pairs of
// consecutive bf16, so A rows and B columns are stored contiguous along k.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "guide.cuh"
#include "guide_kernels.h"
#include "materials.cuh"

namespace xgb {
namespace {

__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// One dense layer for 16 rows held by a warp: out[16][N] = act(in[16][64] . W^T + b).
// in: row stride ldi (elements); W: [N][64]; out written as bf16 (ldo) or fp32 (ldf).
template <int N, bool RELU, bool OUT_F32>
__device__ __forceinline__ void warpLayer(const __nv_bfloat16* in, int ldi, const __nv_bfloat16* W, const float* bias,
                                          __nv_bfloat16* outb, int ldo, float* outf, int ldf) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a[4][4];
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        a[ks][0] = ld32(in + g * ldi + ks * 16 + 2 * t);
        a[ks][1] = ld32(in + (g + 8) * ldi + ks * 16 + 2 * t);
        a[ks][2] = ld32(in + g * ldi + ks * 16 + 2 * t + 8);
        a[ks][3] = ld32(in + (g + 8) * ldi + ks * 16 + 2 * t + 8);
    }
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        const __nv_bfloat16* wr = W + (nt * 8 + g) * 64;
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) mma16816(c, a[ks], ld32(wr + ks * 16 + 2 * t), ld32(wr + ks * 16 + 2 * t + 8));
        const int col = nt * 8 + 2 * t;
        float b0 = bias ? bias[col] : 0.f, b1 = bias ? bias[col + 1] : 0.f;
        float v0 = c[0] + b0, v1 = c[1] + b1, v2 = c[2] + b0, v3 = c[3] + b1;
        if (RELU) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); v2 = fmaxf(v2, 0.f); v3 = fmaxf(v3, 0.f); }
        if (OUT_F32) {
            outf[g * ldf + col] = v0; outf[g * ldf + col + 1] = v1;
            outf[(g + 8) * ldf + col] = v2; outf[(g + 8) * ldf + col + 1] = v3;
        } else {
            *reinterpret_cast<uint32_t*>(outb + g * ldo + col) = pack2(v0, v1);
            *reinterpret_cast<uint32_t*>(outb + (g + 8) * ldo + col) = pack2(v2, v3);
        }
    }
}

// --------------------------------------------------------------- training --
// Features of training records -> X0 (bf16 [rows][64]); rows >= n are zero.
__global__ void k_recordFeatures(const GuideRecord* rec, int n, int rowsPad, GuideBounds gb, __nv_bfloat16* X0,
                                 float4* dirw) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rowsPad) return;
    __nv_bfloat16* x = X0 + (size_t)r * 64;
    if (r >= n) {
        for (int i = 0; i < 64; ++i) x[i] = __float2bfloat16(0.f);
        dirw[r] = make_float4(0.f, 0.f, 1.f, 0.f);
        return;
    }
    GuideRecord g = rec[r];
    float p[3] = {(g.p.x - gb.lo[0]) * gb.invExtent[0], (g.p.y - gb.lo[1]) * gb.invExtent[1],
                  (g.p.z - gb.lo[2]) * gb.invExtent[2]};
    float nn[3] = {g.n.x, g.n.y, g.n.z}, wo[3] = {g.wo.x, g.wo.y, g.wo.z};
    for (int i = 0; i < 64; i += 2)
        *reinterpret_cast<uint32_t*>(x + i) = pack2(guideFeature(i, p, nn, wo), guideFeature(i + 1, p, nn, wo));
    float w = g.pdf > 0.f ? g.radiance / g.pdf : 0.f;
    dirw[r] = make_float4(g.wi.x, g.wi.y, g.wi.z, isfinite(w) ? w : 0.f);
}

// One layer over all rows: warps take 16-row slabs.
template <int N, bool RELU, bool OUT_F32>
__global__ void k_layerForward(const __nv_bfloat16* X, const __nv_bfloat16* W, const float* bias, int rows,
                               __nv_bfloat16* Yb, float* Yf) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int slabs = rows / 16;
    if (warp >= slabs) return;
    const size_t r0 = (size_t)warp * 16;
    warpLayer<N, RELU, OUT_F32>(X + r0 * 64, 64, W, bias, OUT_F32 ? nullptr : Yb + r0 * 64, 64,
                                OUT_F32 ? Yf + r0 * kGuideOutPad : nullptr, kGuideOutPad);
}

__global__ void k_weightSum(const float4* dirw, int n, float* sum) {
    float s = 0.f;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) s += dirw[r].w;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, s);
}

// Output-layer gradient of the normalised NLL: dY = d/dy [ -(w / mean w) log q ] / n.
__global__ void k_lossGrad(const float* Y, const float4* dirw, int n, int rowsPad, const float* wsum, __nv_bfloat16* dY,
                           float* lossSum) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    float loss = 0.f;
    if (r < rowsPad) {
        __nv_bfloat16* d = dY + (size_t)r * kGuideOutPad;
        if (r < n && *wsum > 0.f) {
            float4 dw = dirw[r];
            float w = dw.w / *wsum;  // weights normalised to sum to one over the batch
            float dy[kGuideOut];
            loss = mixtureNllGrad(Y + (size_t)r * kGuideOutPad, V3(dw.x, dw.y, dw.z), w, dy);
            for (int i = 0; i < kGuideOut; i += 2) *reinterpret_cast<uint32_t*>(d + i) = pack2(dy[i], dy[i + 1]);
        } else {
            for (int i = 0; i < kGuideOut; i += 2) *reinterpret_cast<uint32_t*>(d + i) = 0u;
        }
        for (int i = kGuideOut; i < kGuideOutPad; i += 2) *reinterpret_cast<uint32_t*>(d + i) = 0u;
    }
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_down_sync(0xFFFFFFFFu, loss, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(lossSum, loss);
}

// dX[r][i] = (sum_o dY[r][o] W[o][i]) * (Xact[r][i] > 0), K = KO (48 or 64); WT = W^T [64][KO].
template <int KO>
__global__ void k_layerBackwardData(const __nv_bfloat16* dY, const __nv_bfloat16* WT, const __nv_bfloat16* Xact,
                                    int rows, __nv_bfloat16* dX) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= rows / 16) return;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const size_t r0 = (size_t)warp * 16;
    const __nv_bfloat16* in = dY + r0 * KO;
    uint32_t a[KO / 16][4];
#pragma unroll
    for (int ks = 0; ks < KO / 16; ++ks) {
        a[ks][0] = ld32(in + g * KO + ks * 16 + 2 * t);
        a[ks][1] = ld32(in + (g + 8) * KO + ks * 16 + 2 * t);
        a[ks][2] = ld32(in + g * KO + ks * 16 + 2 * t + 8);
        a[ks][3] = ld32(in + (g + 8) * KO + ks * 16 + 2 * t + 8);
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        const __nv_bfloat16* wr = WT + (nt * 8 + g) * KO;
#pragma unroll
        for (int ks = 0; ks < KO / 16; ++ks) mma16816(c, a[ks], ld32(wr + ks * 16 + 2 * t), ld32(wr + ks * 16 + 2 * t + 8));
        const int col = nt * 8 + 2 * t;
        const __nv_bfloat16* xr0 = Xact + (r0 + g) * 64 + col;
        const __nv_bfloat16* xr1 = Xact + (r0 + g + 8) * 64 + col;
        float m0 = __bfloat162float(xr0[0]) > 0.f, m1 = __bfloat162float(xr0[1]) > 0.f;
        float m2 = __bfloat162float(xr1[0]) > 0.f, m3 = __bfloat162float(xr1[1]) > 0.f;
        *reinterpret_cast<uint32_t*>(dX + (r0 + g) * 64 + col) = pack2(c[0] * m0, c[1] * m1);
        *reinterpret_cast<uint32_t*>(dX + (r0 + g + 8) * 64 + col) = pack2(c[2] * m2, c[3] * m3);
    }
}

// dW[o][i] += sum_r dY[r][o] X[r][i], db[o] += sum_r dY[r][o]; NO = 48 or 64 output rows.
// A block takes a chunk of rows; each 16-row slab is staged transposed in shared memory.
constexpr int kWgRowsPerBlock = 512;
constexpr int kPadT = 18;  // shared row stride (bf16) of the transposed slabs

template <int NO>
__global__ void __launch_bounds__(128) k_layerBackwardWeight(const __nv_bfloat16* dY, const __nv_bfloat16* X, int rows,
                                                             float* dW, float* db) {
    __shared__ __align__(16) __nv_bfloat16 sY[NO * kPadT];
    __shared__ __align__(16) __nv_bfloat16 sX[64 * kPadT];
    __shared__ float sdb[NO];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    constexpr int TILES = (NO / 16) * 8;
    constexpr int PER_WARP = TILES / 4;
    float acc[PER_WARP][4];
#pragma unroll
    for (int k = 0; k < PER_WARP; ++k) acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = 0.f;
    if (threadIdx.x < NO) sdb[threadIdx.x] = 0.f;
    const int rBegin = blockIdx.x * kWgRowsPerBlock;
    const int rEnd = min(rows, rBegin + kWgRowsPerBlock);
    for (int r0 = rBegin; r0 < rEnd; r0 += 16) {
        __syncthreads();
        for (int e = threadIdx.x; e < 16 * NO; e += 128) {
            int r = e / NO, o = e % NO;
            sY[o * kPadT + r] = dY[(size_t)(r0 + r) * NO + o];
        }
        for (int e = threadIdx.x; e < 16 * 64; e += 128) {
            int r = e >> 6, i = e & 63;
            sX[i * kPadT + r] = X[(size_t)(r0 + r) * 64 + i];
        }
        __syncthreads();
        if (threadIdx.x < NO) {
            float s = 0.f;
            for (int r = 0; r < 16; ++r) s += __bfloat162float(sY[threadIdx.x * kPadT + r]);
            sdb[threadIdx.x] += s;
        }
#pragma unroll
        for (int k = 0; k < PER_WARP; ++k) {
            const int tile = warp * PER_WARP + k;
            const int mt = tile / 8, nt = tile % 8;
            uint32_t a[4];
            const __nv_bfloat16* ar = sY + (mt * 16) * kPadT;
            a[0] = ld32(ar + g * kPadT + 2 * t);
            a[1] = ld32(ar + (g + 8) * kPadT + 2 * t);
            a[2] = ld32(ar + g * kPadT + 2 * t + 8);
            a[3] = ld32(ar + (g + 8) * kPadT + 2 * t + 8);
            const __nv_bfloat16* br = sX + (nt * 8 + g) * kPadT;
            mma16816(acc[k], a, ld32(br + 2 * t), ld32(br + 2 * t + 8));
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < PER_WARP; ++k) {
        const int tile = warp * PER_WARP + k;
        const int mt = tile / 8, nt = tile % 8;
        const int o0 = mt * 16 + g, i0 = nt * 8 + 2 * t;
        atomicAdd(&dW[o0 * 64 + i0], acc[k][0]);
        atomicAdd(&dW[o0 * 64 + i0 + 1], acc[k][1]);
        atomicAdd(&dW[(o0 + 8) * 64 + i0], acc[k][2]);
        atomicAdd(&dW[(o0 + 8) * 64 + i0 + 1], acc[k][3]);
    }
    if (threadIdx.x < NO) atomicAdd(&db[threadIdx.x], sdb[threadIdx.x]);
}

// Adam on the fp32 master parameters; refreshes the bf16 copies W / WT.
__global__ void k_adam(float* params, const float* grads, float* m, float* v, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2, GuideWeights w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = grads[i];
    float mi = b1 * m[i] + (1.f - b1) * g;
    float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    float p = params[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    params[i] = p;
    guideStoreBf16(w, i, p);
}

// Gradient layout follows the parameters: dW rows are 64 wide; the last layer's
// gradient rows 40..47 (padding) are dropped when copied into the flat vector.
__global__ void k_gatherGrads(const float* dW0, const float* dW1, const float* dW2, const float* dW3, const float* db,
                              float* grads) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kGuideParams) return;
    float v;
    if (i < kGuideB0) v = dW0[i - kGuideW0];
    else if (i < kGuideW1) v = db[i - kGuideB0];
    else if (i < kGuideB1) v = dW1[i - kGuideW1];
    else if (i < kGuideW2) v = db[64 + i - kGuideB1];
    else if (i < kGuideB2) v = dW2[i - kGuideW2];
    else if (i < kGuideW3) v = db[128 + i - kGuideB2];
    else if (i < kGuideB3) v = dW3[i - kGuideW3];
    else v = db[192 + i - kGuideB3];
    grads[i] = v;
}

}  // namespace

__device__ void guideStoreBf16(const GuideWeights& w, int i, float p) {
    __nv_bfloat16 b = __float2bfloat16(p);
    if (i < kGuideB0) {
        int o = (i - kGuideW0) / 64, k = (i - kGuideW0) % 64;
        w.W[0][o * 64 + k] = b; w.WT[0][k * 64 + o] = b;
    } else if (i < kGuideW1) {
        w.bias[0][i - kGuideB0] = p;
    } else if (i < kGuideB1) {
        int o = (i - kGuideW1) / 64, k = (i - kGuideW1) % 64;
        w.W[1][o * 64 + k] = b; w.WT[1][k * 64 + o] = b;
    } else if (i < kGuideW2) {
        w.bias[1][i - kGuideB1] = p;
    } else if (i < kGuideB2) {
        int o = (i - kGuideW2) / 64, k = (i - kGuideW2) % 64;
        w.W[2][o * 64 + k] = b; w.WT[2][k * 64 + o] = b;
    } else if (i < kGuideW3) {
        w.bias[2][i - kGuideB2] = p;
    } else if (i < kGuideB3) {
        int o = (i - kGuideW3) / 64, k = (i - kGuideW3) % 64;
        w.W[3][o * 64 + k] = b; w.WT[3][k * kGuideOutPad + o] = b;
    } else {
        w.bias[3][i - kGuideB3] = p;
    }
}

namespace {
__global__ void k_refreshBf16(const float* params, GuideWeights w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kGuideParams) guideStoreBf16(w, i, params[i]);
}

// Fused inference for host-supplied feature rows (API / tests): X0 [rows][64] bf16 -> Y [rows][48] fp32.
__global__ void k_inferRows(const __nv_bfloat16* X0, int rows, GuideWeights w, float* Y) {
    __shared__ __align__(16) __nv_bfloat16 buf[4][2][16 * 72];
    const int warpInBlock = threadIdx.x >> 5;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= rows / 16) return;
    const size_t r0 = (size_t)warp * 16;
    __nv_bfloat16* s0 = buf[warpInBlock][0];
    __nv_bfloat16* s1 = buf[warpInBlock][1];
    warpLayer<64, true, false>(X0 + r0 * 64, 64, w.W[0], w.bias[0], s0, 72, nullptr, 0);
    __syncwarp();
    warpLayer<64, true, false>(s0, 72, w.W[1], w.bias[1], s1, 72, nullptr, 0);
    __syncwarp();
    warpLayer<64, true, false>(s1, 72, w.W[2], w.bias[2], s0, 72, nullptr, 0);
    __syncwarp();
    warpLayer<kGuideOutPad, false, true>(s0, 72, w.W[3], w.bias[3], nullptr, 0, Y + r0 * kGuideOutPad, kGuideOutPad);
}
}  // namespace

// ------------------------------------------------------------- host side --
void guideRefresh(const GuideDevice& g, cudaStream_t s) {
    k_refreshBf16<<<(kGuideParams + 255) / 256, 256, 0, s>>>(g.params, g.w);
}

void guideInferRows(const GuideDevice& g, const __nv_bfloat16* X0, int rowsPad, float* Y, cudaStream_t s) {
    int warps = rowsPad / 16;
    k_inferRows<<<(warps + 3) / 4, 128, 0, s>>>(X0, rowsPad, g.w, Y);
}

void guideTrainStep(GuideDevice& g, const GuideRecord* rec, int n, GuideBounds gb, float lr, cudaStream_t s) {
    n = std::min(n, g.maxRows);
    if (n <= 0) return;
    const int rows = (n + 63) & ~63;
    GuideScratch sc = g.scratch;
    k_recordFeatures<<<(rows + 127) / 128, 128, 0, s>>>(rec, n, rows, gb, sc.X[0], sc.dirw);
    const int wb = (rows / 16 + 3) / 4;
    k_layerForward<64, true, false><<<wb, 128, 0, s>>>(sc.X[0], g.w.W[0], g.w.bias[0], rows, sc.X[1], nullptr);
    k_layerForward<64, true, false><<<wb, 128, 0, s>>>(sc.X[1], g.w.W[1], g.w.bias[1], rows, sc.X[2], nullptr);
    k_layerForward<64, true, false><<<wb, 128, 0, s>>>(sc.X[2], g.w.W[2], g.w.bias[2], rows, sc.X[3], nullptr);
    k_layerForward<kGuideOutPad, false, true><<<wb, 128, 0, s>>>(sc.X[3], g.w.W[3], g.w.bias[3], rows, nullptr, sc.Y);
    cudaMemsetAsync(sc.scalars, 0, 4 * sizeof(float), s);
    k_weightSum<<<std::min(64, (rows + 255) / 256), 256, 0, s>>>(sc.dirw, rows, sc.scalars);
    k_lossGrad<<<(rows + 127) / 128, 128, 0, s>>>(sc.Y, sc.dirw, n, rows, sc.scalars, sc.dY3, sc.scalars + 1);
    k_layerBackwardData<kGuideOutPad><<<wb, 128, 0, s>>>(sc.dY3, g.w.WT[3], sc.X[3], rows, sc.dZ[2]);
    k_layerBackwardData<64><<<wb, 128, 0, s>>>(sc.dZ[2], g.w.WT[2], sc.X[2], rows, sc.dZ[1]);
    k_layerBackwardData<64><<<wb, 128, 0, s>>>(sc.dZ[1], g.w.WT[1], sc.X[1], rows, sc.dZ[0]);
    cudaMemsetAsync(sc.dW, 0, sizeof(float) * (3 * 64 * 64 + kGuideOutPad * 64 + 256), s);
    const int gw = (rows + kWgRowsPerBlock - 1) / kWgRowsPerBlock;
    float* dW0 = sc.dW;
    float* dW1 = dW0 + 64 * 64;
    float* dW2 = dW1 + 64 * 64;
    float* dW3 = dW2 + 64 * 64;
    float* db = dW3 + kGuideOutPad * 64;
    k_layerBackwardWeight<64><<<gw, 128, 0, s>>>(sc.dZ[0], sc.X[0], rows, dW0, db);
    k_layerBackwardWeight<64><<<gw, 128, 0, s>>>(sc.dZ[1], sc.X[1], rows, dW1, db + 64);
    k_layerBackwardWeight<64><<<gw, 128, 0, s>>>(sc.dZ[2], sc.X[2], rows, dW2, db + 128);
    k_layerBackwardWeight<kGuideOutPad><<<gw, 128, 0, s>>>(sc.dY3, sc.X[3], rows, dW3, db + 192);
    k_gatherGrads<<<(kGuideParams + 255) / 256, 256, 0, s>>>(dW0, dW1, dW2, dW3, db, g.grads);
    if (lr > 0.f) {
        g.step += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        float c1 = 1.f - std::pow(b1, (float)g.step), c2 = 1.f - std::pow(b2, (float)g.step);
        k_adam<<<(kGuideParams + 255) / 256, 256, 0, s>>>(g.params, g.grads, g.m, g.v, kGuideParams, lr, b1, b2, 1e-8f,
                                                         c1, c2, g.w);
    }
}

namespace {
// Credited wavefront records -> training pool; records that carry no radiance
// (zero weight in the loss) are left out.
__global__ void k_collect(const GuideRecord* rec, const unsigned int* nDev, int recCap, GuideRecord* pool,
                          unsigned int* poolCount, int poolCap) {
    const int n = min((int)*nDev, recCap);
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int r = base + threadIdx.x;
        GuideRecord g;
        bool keep = false;
        if (r < n) {
            g = rec[r];
            float w = g.pdf > 0.f ? g.radiance / g.pdf : 0.f;
            keep = w > 0.f && isfinite(w);
        }
        const unsigned int m = __ballot_sync(0xFFFFFFFFu, keep);
        const int lane = threadIdx.x & 31;
        unsigned int off = 0;
        if (lane == 0 && m) off = atomicAdd(poolCount, (unsigned int)__popc(m));
        off = __shfl_sync(0xFFFFFFFFu, off, 0) + __popc(m & ((1u << lane) - 1u));
        if (keep && off < (unsigned int)poolCap) pool[off] = g;
    }
}

__global__ void k_setCount(unsigned int* c, unsigned int v) { *c = v; }

// Incident radiance of each record once its path has finished: the path's
// contributions after the record's vertex, divided per channel by the
// throughput after that vertex; luminance, times the BSDF term for the
// product target. Records whose path never reached another vertex keep 0.
__global__ void k_finalize(GuideRecord* rec, const unsigned int* nDev, int cap, const float4* pathAcc, int product) {
    const int n = min((int)*nDev, cap);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const GuideRecord g = rec[r];
        float L = 0.0f;
        if (!isnan(g.snap.x)) {
            const float4 a = pathAcc[g.pid];
            float lr = g.thr.x > 0.0f ? (a.x - g.snap.x) / g.thr.x : 0.0f;
            float lg = g.thr.y > 0.0f ? (a.y - g.snap.y) / g.thr.y : 0.0f;
            float lb = g.thr.z > 0.0f ? (a.z - g.snap.z) / g.thr.z : 0.0f;
            L = fmaxf(0.0f, 0.2126f * lr + 0.7152f * lg + 0.0722f * lb);
            if (product) L *= g.fcos;
        }
        rec[r].radiance = isfinite(L) ? L : 0.0f;
    }
}
}  // namespace

void guideFinalizeRecords(GuideRecord* rec, const unsigned int* nDev, int cap, const float4* pathAcc, int product,
                          cudaStream_t s) {
    k_finalize<<<std::max(1, std::min(2048, (cap + 255) / 256)), 256, 0, s>>>(rec, nDev, cap, pathAcc, product);
}

void guideCollect(const GuideDevice& g, const GuideRecord* rec, const unsigned int* nDev, int recCap, cudaStream_t s) {
    k_collect<<<std::max(1, std::min(2048, (recCap + 255) / 256)), 256, 0, s>>>(rec, nDev, recCap, g.pool, g.poolCount,
                                                                               g.poolCap);
}

int guidePoolTrain(GuideDevice& g, unsigned int count, GuideBounds gb, float lr, int maxSteps, cudaStream_t s) {
    const unsigned int c = std::min(count, (unsigned int)g.poolCap);
    const int B = g.batch;
    const int steps = (int)std::min<unsigned int>(c / (unsigned int)B, (unsigned int)std::max(0, maxSteps));
    for (int j = 0; j < steps; ++j) guideTrainStep(g, g.pool + (size_t)j * B, B, gb, lr, s);
    unsigned int rest = c - (unsigned int)steps * (unsigned int)B;
    if (rest >= (unsigned int)B) rest = 0;  // step cap reached: drop the excess rather than train on stale records
    if (steps > 0 && rest > 0)  // rest < B <= steps * B: source and destination do not overlap
        cudaMemcpyAsync(g.pool, g.pool + (size_t)steps * B, sizeof(GuideRecord) * rest, cudaMemcpyDeviceToDevice, s);
    if (steps > 0 || count != rest) k_setCount<<<1, 1, 0, s>>>(g.poolCount, rest);
    return steps;
}

namespace {
__global__ void k_pointFeatures(const float* p, const float* n, const float* wo, int count, int rowsPad, GuideBounds gb,
                                __nv_bfloat16* X0) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rowsPad) return;
    __nv_bfloat16* x = X0 + (size_t)r * 64;
    if (r >= count) {
        for (int i = 0; i < 64; i += 2) *reinterpret_cast<uint32_t*>(x + i) = 0u;
        return;
    }
    float pp[3] = {(p[3 * r] - gb.lo[0]) * gb.invExtent[0], (p[3 * r + 1] - gb.lo[1]) * gb.invExtent[1],
                   (p[3 * r + 2] - gb.lo[2]) * gb.invExtent[2]};
    float nn[3] = {n[3 * r], n[3 * r + 1], n[3 * r + 2]}, ww[3] = {wo[3 * r], wo[3 * r + 1], wo[3 * r + 2]};
    for (int i = 0; i < 64; i += 2)
        *reinterpret_cast<uint32_t*>(x + i) = pack2(guideFeature(i, pp, nn, ww), guideFeature(i + 1, pp, nn, ww));
}

// Per-path inference: every hit of the input queue gets its 8-lobe mixture
// (10 float4: lobes' (mu, kappa) then the 8 weights). Warps take 16 paths; the
// two half-warps build the two halves of each feature row.
__global__ void __launch_bounds__(128) k_inferPaths(SceneDev sc, GuideWeights w, GuideBounds gb, PathQueue q, HitQueue h,
                                                    const Ctrl* ctrl, float4* mix) {
    __shared__ __align__(16) __nv_bfloat16 act[4][2][16 * 72];
    __shared__ float outY[4][16 * kGuideOutPad];
    const unsigned int n = ctrl->nActive;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned int warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned int nWarps = (gridDim.x * blockDim.x) >> 5;
    const int row = lane & 15, half = lane >> 4;
    for (unsigned int base = warpGlobal * 16u; base < n; base += nWarps * 16u) {
        const unsigned int i = base + row;
        float pf[3] = {0.f, 0.f, 0.f}, nf[3] = {0.f, 0.f, 0.f}, wf[3] = {0.f, 0.f, 0.f};
        bool valid = false;
        if (i < n) {
            float4 hh = h.h[i];
            int prim = __float_as_int(hh.w);
            if (prim >= 0) {
                float4 d4 = q.d[i];
                Surface s = makeSurface(sc, sc.instances[h.inst[i]], prim, hh.y, hh.z, V3(d4.x, d4.y, d4.z));
                pf[0] = (s.p.x - gb.lo[0]) * gb.invExtent[0];
                pf[1] = (s.p.y - gb.lo[1]) * gb.invExtent[1];
                pf[2] = (s.p.z - gb.lo[2]) * gb.invExtent[2];
                nf[0] = s.sn.x; nf[1] = s.sn.y; nf[2] = s.sn.z;
                wf[0] = s.wo.x; wf[1] = s.wo.y; wf[2] = s.wo.z;
                valid = true;
            }
        }
        __nv_bfloat16* x = act[wib][0] + row * 72;
        for (int k = half * 32; k < half * 32 + 32; k += 2)
            *reinterpret_cast<uint32_t*>(x + k) =
                valid ? pack2(guideFeature(k, pf, nf, wf), guideFeature(k + 1, pf, nf, wf)) : 0u;
        __syncwarp();
        warpLayer<64, true, false>(act[wib][0], 72, w.W[0], w.bias[0], act[wib][1], 72, nullptr, 0);
        __syncwarp();
        warpLayer<64, true, false>(act[wib][1], 72, w.W[1], w.bias[1], act[wib][0], 72, nullptr, 0);
        __syncwarp();
        warpLayer<64, true, false>(act[wib][0], 72, w.W[2], w.bias[2], act[wib][1], 72, nullptr, 0);
        __syncwarp();
        warpLayer<kGuideOutPad, false, true>(act[wib][1], 72, w.W[3], w.bias[3], nullptr, 0, outY[wib], kGuideOutPad);
        __syncwarp();
        if (half == 0 && i < n) {
            VmfMixture mx;
            decodeMixture(outY[wib] + row * kGuideOutPad, mx);
            float4* o = mix + (size_t)i * 10;
            for (int j = 0; j < kGuideLobes; ++j)
                o[j] = make_float4(mx.lobe[j].mu.x, mx.lobe[j].mu.y, mx.lobe[j].mu.z, mx.lobe[j].kappa);
            o[8] = make_float4(mx.lobe[0].alpha, mx.lobe[1].alpha, mx.lobe[2].alpha, mx.lobe[3].alpha);
            o[9] = make_float4(mx.lobe[4].alpha, mx.lobe[5].alpha, mx.lobe[6].alpha, mx.lobe[7].alpha);
        }
        __syncwarp();
    }
}
}  // namespace

namespace {
__global__ void k_sampleRows(const float* Y, int n, uint32_t seed, float* dirs, float* pdf) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    VmfMixture mx;
    decodeMixture(Y + (size_t)r * kGuideOutPad, mx);
    Pcg rng;
    rng.seed((uint32_t)r, 0u, seed);
    V3 d = mixtureSample(mx, rng);
    dirs[3 * r] = d.x; dirs[3 * r + 1] = d.y; dirs[3 * r + 2] = d.z;
    pdf[r] = mixturePdf(mx, d);
}
}  // namespace

void guideSampleRows(const float* Y, int n, uint32_t seed, float* dirs, float* pdf, cudaStream_t s) {
    k_sampleRows<<<(n + 127) / 128, 128, 0, s>>>(Y, n, seed, dirs, pdf);
}

void guideFeaturesFromPoints(const float* p, const float* n, const float* wo, int count, int rowsPad, GuideBounds gb,
                             __nv_bfloat16* X0, cudaStream_t s) {
    k_pointFeatures<<<(rowsPad + 127) / 128, 128, 0, s>>>(p, n, wo, count, rowsPad, gb, X0);
}

void guideInferPaths(const SceneDev& sc, const GuideDevice& g, GuideBounds gb, PathQueue q, HitQueue h, const Ctrl* ctrl,
                     float4* mix, int grid, cudaStream_t s) {
    k_inferPaths<<<grid, 128, 0, s>>>(sc, g.w, gb, q, h, ctrl, mix);
}

}  // namespace xgb
