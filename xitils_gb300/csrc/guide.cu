// Guiding network kernels: BF16 tensor-core (mma.sync m16n8k16, FP32
// accumulation) training of the 64-64-64-64-40 MLP (forward, backward and the
// weight gradients of a 64-row tile per warp group) and Adam. Inference, for
// host rows and for the wavefront's paths, is in guide_tc.cu (tcgen05, TMEM).
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
// --------------------------------------------------------------- training --
// One Adam step is two launches.
//   k_trainTiles: a CTA takes 64-row tiles of the batch (4 warps x 16 rows) and
//     runs the whole step for them out of shared memory -- features, forward
//     pass, mixture NLL gradient, backward pass, weight and bias gradients -- and
//     adds the tile's gradients into the CTA's own slot of a partial buffer.
//   k_reduceAdam: sums the slots of every parameter, normalises by the batch's
//     total sample weight and takes the Adam step (refreshing the bf16 copies).
// The loss is -sum_i (w_i / sum_j w_j) log q(wi_i) with w_i = radiance / pdf;
// rows enter with their raw weight and the slot sums are divided by sum_j w_j,
// which is the same gradient. Weight gradients dW = dZ^T X are tensor-core
// products over the tile's rows: both operands are read transposed from
// shared memory with ldmatrix.trans.
constexpr int kTileRows = 64;
constexpr int kLd = 72;   // shared row stride (bf16) of 64-wide rows (144 B: ldmatrix and fragment loads conflict-free)
constexpr int kLdO = 56;  // shared row stride (bf16) of 48-wide rows (112 B)
constexpr int kSlot = kGuideParams + 4;  // partial gradient of one CTA, then its weight sum and loss sum
constexpr int kMaxSlots = 256;

struct TrainSmem {
    __nv_bfloat16 W[3][64 * kLd];  // [out][in]
    __nv_bfloat16 W3[kGuideOutPad * kLd];
    __nv_bfloat16 WT[3][64 * kLd];  // [in][out]
    __nv_bfloat16 WT3[64 * kLdO];
    float bias[4][64];
    __nv_bfloat16 X[4][kTileRows * kLd];  // layer inputs
    __nv_bfloat16 dY[kTileRows * kLdO];   // output-layer gradient
    __nv_bfloat16 dZ[3][kTileRows * kLd];  // hidden pre-activation gradients (layers 0..2)
    float Y[kTileRows * kGuideOutPad];
    float4 dirw[kTileRows];
    float red[2][4];
};

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsmX4T(uint32_t (&r)[4], const __nv_bfloat16* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smemAddr(p)));
}

// out[16][N] = act(in[16][64] . W^T + b) for the warp's 16 rows; W [N][64] with row stride ldw.
template <int N, bool RELU, bool OUT_F32>
__device__ __forceinline__ void warpLayerS(const __nv_bfloat16* in, const __nv_bfloat16* W, const float* bias,
                                           __nv_bfloat16* outb, float* outf) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a[4][4];
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        a[ks][0] = ld32(in + g * kLd + ks * 16 + 2 * t);
        a[ks][1] = ld32(in + (g + 8) * kLd + ks * 16 + 2 * t);
        a[ks][2] = ld32(in + g * kLd + ks * 16 + 2 * t + 8);
        a[ks][3] = ld32(in + (g + 8) * kLd + ks * 16 + 2 * t + 8);
    }
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        const __nv_bfloat16* wr = W + (nt * 8 + g) * kLd;
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) mma16816(c, a[ks], ld32(wr + ks * 16 + 2 * t), ld32(wr + ks * 16 + 2 * t + 8));
        const int col = nt * 8 + 2 * t;
        float v0 = c[0] + bias[col], v1 = c[1] + bias[col + 1], v2 = c[2] + bias[col], v3 = c[3] + bias[col + 1];
        if (RELU) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); v2 = fmaxf(v2, 0.f); v3 = fmaxf(v3, 0.f); }
        if (OUT_F32) {
            outf[g * kGuideOutPad + col] = v0; outf[g * kGuideOutPad + col + 1] = v1;
            outf[(g + 8) * kGuideOutPad + col] = v2; outf[(g + 8) * kGuideOutPad + col + 1] = v3;
        } else {
            *reinterpret_cast<uint32_t*>(outb + g * kLd + col) = pack2(v0, v1);
            *reinterpret_cast<uint32_t*>(outb + (g + 8) * kLd + col) = pack2(v2, v3);
        }
    }
}

// dX[16][64] = (dZ[16][KO] . W) * (Xact > 0) for the warp's 16 rows; WT = W^T [64][KO] with row stride ldwt.
template <int KO>
__device__ __forceinline__ void warpBackData(const __nv_bfloat16* dZ, int ldz, const __nv_bfloat16* WT, int ldwt,
                                             const __nv_bfloat16* Xact, __nv_bfloat16* dX) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a[KO / 16][4];
#pragma unroll
    for (int ks = 0; ks < KO / 16; ++ks) {
        a[ks][0] = ld32(dZ + g * ldz + ks * 16 + 2 * t);
        a[ks][1] = ld32(dZ + (g + 8) * ldz + ks * 16 + 2 * t);
        a[ks][2] = ld32(dZ + g * ldz + ks * 16 + 2 * t + 8);
        a[ks][3] = ld32(dZ + (g + 8) * ldz + ks * 16 + 2 * t + 8);
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        const __nv_bfloat16* wr = WT + (nt * 8 + g) * ldwt;
#pragma unroll
        for (int ks = 0; ks < KO / 16; ++ks) mma16816(c, a[ks], ld32(wr + ks * 16 + 2 * t), ld32(wr + ks * 16 + 2 * t + 8));
        const int col = nt * 8 + 2 * t;
        const __nv_bfloat16* x0 = Xact + g * kLd + col;
        const __nv_bfloat16* x1 = Xact + (g + 8) * kLd + col;
        const float m0 = __bfloat162float(x0[0]) > 0.f, m1 = __bfloat162float(x0[1]) > 0.f;
        const float m2 = __bfloat162float(x1[0]) > 0.f, m3 = __bfloat162float(x1[1]) > 0.f;
        *reinterpret_cast<uint32_t*>(dX + g * kLd + col) = pack2(c[0] * m0, c[1] * m1);
        *reinterpret_cast<uint32_t*>(dX + (g + 8) * kLd + col) = pack2(c[2] * m2, c[3] * m3);
    }
}

// slot[wOff + o * 64 + i] (+)= sum over the tile's 64 rows of D[r][o] X[r][i], o < oValid.
// Work unit = one 16-row block of o times two 8-column blocks of i; D rows have stride ldd.
template <int O>
__device__ __forceinline__ void tileWeightGrad(const __nv_bfloat16* D, int ldd, const __nv_bfloat16* X, float* slot,
                                               int wOff, int oValid, bool first) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int q = lane >> 3, i8 = lane & 7;
    for (int u = warp; u < (O / 16) * 4; u += 4) {
        const int o0 = (u >> 2) * 16, c0 = (u & 3) * 16;
        float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int ks = 0; ks < kTileRows / 16; ++ks) {
            const int r0 = ks * 16;
            uint32_t a[4], b[4];
            // A = D^T (16 o x 16 r): matrices (r, o), (r, o + 8), (r + 8, o), (r + 8, o + 8)
            ldsmX4T(a, D + (r0 + i8 + ((q >> 1) << 3)) * ldd + o0 + ((q & 1) << 3));
            // B = X (16 r x 8 i), two i blocks: matrices (r, i), (r + 8, i), (r, i + 8), (r + 8, i + 8)
            ldsmX4T(b, X + (r0 + i8 + ((q & 1) << 3)) * kLd + c0 + ((q >> 1) << 3));
            mma16816(acc[0], a, b[0], b[1]);
            mma16816(acc[1], a, b[2], b[3]);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = c0 + h * 8 + 2 * t;
            const int oa = o0 + g, ob = o0 + g + 8;
            float* pa = slot + wOff + oa * 64 + i;
            float* pb = slot + wOff + ob * 64 + i;
            if (oa < oValid) {
                if (first) { pa[0] = acc[h][0]; pa[1] = acc[h][1]; } else { pa[0] += acc[h][0]; pa[1] += acc[h][1]; }
            }
            if (ob < oValid) {
                if (first) { pb[0] = acc[h][2]; pb[1] = acc[h][3]; } else { pb[0] += acc[h][2]; pb[1] += acc[h][3]; }
            }
        }
    }
}

__global__ void __launch_bounds__(128) k_trainTiles(const GuideRecord* rec, int n, int tiles, GuideBounds gb,
                                                    GuideWeights w, float* partial) {
    extern __shared__ __align__(128) unsigned char smemRaw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smemRaw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // weights and biases, once per CTA (rows of 128 B as 16-byte pieces)
    for (int e = tid; e < 3 * 64 * 8; e += 128) {
        const int l = e / 512, r = (e >> 3) & 63, c = e & 7;
        *reinterpret_cast<uint4*>(S.W[l] + r * kLd + 8 * c) = reinterpret_cast<const uint4*>(w.W[l] + r * 64)[c];
        *reinterpret_cast<uint4*>(S.WT[l] + r * kLd + 8 * c) = reinterpret_cast<const uint4*>(w.WT[l] + r * 64)[c];
    }
    for (int e = tid; e < kGuideOutPad * 8; e += 128) {
        const int r = e >> 3, c = e & 7;
        *reinterpret_cast<uint4*>(S.W3 + r * kLd + 8 * c) = reinterpret_cast<const uint4*>(w.W[3] + r * 64)[c];
    }
    for (int e = tid; e < 64 * 6; e += 128) {
        const int r = e / 6, c = e % 6;
        *reinterpret_cast<uint4*>(S.WT3 + r * kLdO + 8 * c) =
            reinterpret_cast<const uint4*>(w.WT[3] + r * kGuideOutPad)[c];
    }
    for (int e = tid; e < 4 * 64; e += 128) {
        const int l = e >> 6, o = e & 63;
        S.bias[l][o] = (l < 3 || o < kGuideOutPad) ? w.bias[l][o] : 0.f;
    }
    float* slot = partial + (size_t)blockIdx.x * kSlot;
    float wsum = 0.f, lsum = 0.f;
    bool first = true;
    const int r0 = warp * 16;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, first = false) {
        __syncthreads();  // weights staged / the previous tile's shared data consumed
        {   // features: two threads per row, 32 features each
            const int r = tid >> 1, half = tid & 1;
            const int gr = tile * kTileRows + r;
            __nv_bfloat16* x = S.X[0] + r * kLd + half * 32;
            if (gr < n) {
                const GuideRecord& gd = rec[gr];
                const float p[3] = {(gd.p.x - gb.lo[0]) * gb.invExtent[0], (gd.p.y - gb.lo[1]) * gb.invExtent[1],
                                    (gd.p.z - gb.lo[2]) * gb.invExtent[2]};
                const float nn[3] = {gd.n.x, gd.n.y, gd.n.z}, wo[3] = {gd.wo.x, gd.wo.y, gd.wo.z};
                float f[64];
                guideFeatures(p, nn, wo, f);
#pragma unroll
                for (int i = 0; i < 32; i += 2)
                    *reinterpret_cast<uint32_t*>(x + i) =
                        half ? pack2(f[32 + i], f[33 + i]) : pack2(f[i], f[i + 1]);
                if (half == 0) {
                    const float wgt = gd.pdf > 0.f ? gd.radiance / gd.pdf : 0.f;
                    S.dirw[r] = make_float4(gd.wi.x, gd.wi.y, gd.wi.z, isfinite(wgt) ? wgt : 0.f);
                }
            } else {
                for (int i = 0; i < 32; i += 2) *reinterpret_cast<uint32_t*>(x + i) = 0u;
                if (half == 0) S.dirw[r] = make_float4(0.f, 0.f, 1.f, 0.f);
            }
        }
        __syncthreads();
        // forward, each warp on its 16 rows
        warpLayerS<64, true, false>(S.X[0] + r0 * kLd, S.W[0], S.bias[0], S.X[1] + r0 * kLd, nullptr);
        __syncwarp();
        warpLayerS<64, true, false>(S.X[1] + r0 * kLd, S.W[1], S.bias[1], S.X[2] + r0 * kLd, nullptr);
        __syncwarp();
        warpLayerS<64, true, false>(S.X[2] + r0 * kLd, S.W[2], S.bias[2], S.X[3] + r0 * kLd, nullptr);
        __syncwarp();
        warpLayerS<kGuideOutPad, false, true>(S.X[3] + r0 * kLd, S.W3, S.bias[3], nullptr, S.Y + r0 * kGuideOutPad);
        __syncwarp();
        // output gradient of -w log q, one lane per row
        if (lane < 16) {
            const int r = r0 + lane;
            __nv_bfloat16* d = S.dY + r * kLdO;
            const float4 dw = S.dirw[r];
            if (dw.w > 0.f) {
                float dy[kGuideOut];
                lsum += mixtureNllGrad(S.Y + r * kGuideOutPad, V3(dw.x, dw.y, dw.z), dw.w, dy);
                wsum += dw.w;
                for (int i = 0; i < kGuideOut; i += 2) *reinterpret_cast<uint32_t*>(d + i) = pack2(dy[i], dy[i + 1]);
            } else {
                for (int i = 0; i < kGuideOut; i += 2) *reinterpret_cast<uint32_t*>(d + i) = 0u;
            }
            for (int i = kGuideOut; i < kGuideOutPad; i += 2) *reinterpret_cast<uint32_t*>(d + i) = 0u;
        }
        __syncwarp();
        // backward through the hidden layers
        warpBackData<kGuideOutPad>(S.dY + r0 * kLdO, kLdO, S.WT3, kLdO, S.X[3] + r0 * kLd, S.dZ[2] + r0 * kLd);
        __syncwarp();
        warpBackData<64>(S.dZ[2] + r0 * kLd, kLd, S.WT[2], kLd, S.X[2] + r0 * kLd, S.dZ[1] + r0 * kLd);
        __syncwarp();
        warpBackData<64>(S.dZ[1] + r0 * kLd, kLd, S.WT[1], kLd, S.X[1] + r0 * kLd, S.dZ[0] + r0 * kLd);
        __syncthreads();
        // weight gradients over all 64 rows of the tile
        tileWeightGrad<64>(S.dZ[0], kLd, S.X[0], slot, kGuideW0, 64, first);
        tileWeightGrad<64>(S.dZ[1], kLd, S.X[1], slot, kGuideW1, 64, first);
        tileWeightGrad<64>(S.dZ[2], kLd, S.X[2], slot, kGuideW2, 64, first);
        tileWeightGrad<kGuideOutPad>(S.dY, kLdO, S.X[3], slot, kGuideW3, kGuideOut, first);
        // bias gradients: 64 + 64 + 64 + 40 columns
        for (int c = tid; c < 192 + kGuideOut; c += 128) {
            const int l = c < 192 ? c >> 6 : 3, o = c < 192 ? c & 63 : c - 192;
            const __nv_bfloat16* D = l < 3 ? S.dZ[l] : S.dY;
            const int ld = l < 3 ? kLd : kLdO;
            float sum = 0.f;
            for (int r = 0; r < kTileRows; ++r) sum += __bfloat162float(D[r * ld + o]);
            const int off = (l == 0 ? kGuideB0 : l == 1 ? kGuideB1 : l == 2 ? kGuideB2 : kGuideB3) + o;
            slot[off] = first ? sum : slot[off] + sum;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        wsum += __shfl_down_sync(0xFFFFFFFFu, wsum, off);
        lsum += __shfl_down_sync(0xFFFFFFFFu, lsum, off);
    }
    if (lane == 0) { S.red[0][warp] = wsum; S.red[1][warp] = lsum; }
    __syncthreads();
    if (tid == 0) {
        slot[kGuideParams] = (S.red[0][0] + S.red[0][1]) + (S.red[0][2] + S.red[0][3]);
        slot[kGuideParams + 1] = (S.red[1][0] + S.red[1][1]) + (S.red[1][2] + S.red[1][3]);
    }
}

// Gradient = slot sum / total weight; Adam (lr > 0) on the fp32 master
// parameters with bias corrections c1, c2, refreshing the bf16 copies.
// scalars[0] = total weight, scalars[1] = loss.
__global__ void k_reduceAdam(const float* partial, int slots, float* grads, float* params, float* m, float* v,
                             float lr, float b1, float b2, float eps, float c1, float c2, GuideWeights w,
                             float* scalars) {
    __shared__ float tot[2];
    if (threadIdx.x < 32) {
        float ws = 0.f, ls = 0.f;
        for (int s = threadIdx.x; s < slots; s += 32) {
            ws += partial[(size_t)s * kSlot + kGuideParams];
            ls += partial[(size_t)s * kSlot + kGuideParams + 1];
        }
        for (int off = 16; off > 0; off >>= 1) {
            ws += __shfl_down_sync(0xFFFFFFFFu, ws, off);
            ls += __shfl_down_sync(0xFFFFFFFFu, ls, off);
        }
        if (threadIdx.x == 0) { tot[0] = ws; tot[1] = ls; }
    }
    __syncthreads();
    const float W = tot[0];
    const float inv = W > 0.f ? 1.f / W : 0.f;
    if (blockIdx.x == 0 && threadIdx.x == 0) { scalars[0] = W; scalars[1] = tot[1] * inv; }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kGuideParams) return;
    float sum = 0.f;
    for (int s = 0; s < slots; ++s) sum += partial[(size_t)s * kSlot + i];
    const float gr = sum * inv;
    grads[i] = gr;
    if (lr > 0.f) {
        const float mi = b1 * m[i] + (1.f - b1) * gr;
        const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        const float p = params[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        params[i] = p;
        guideStoreBf16(w, i, p);
    }
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

}  // namespace

// ------------------------------------------------------------- host side --
void guideRefresh(const GuideDevice& g, cudaStream_t s) {
    k_refreshBf16<<<(kGuideParams + 255) / 256, 256, 0, s>>>(g.params, g.w);
}

void guideTrainStep(GuideDevice& g, const GuideRecord* rec, int n, GuideBounds gb, float lr, cudaStream_t s) {
    n = std::min(n, g.maxRows);
    if (n <= 0) return;
    const int tiles = (n + kTileRows - 1) / kTileRows;
    const int slots = std::min(tiles, kMaxSlots);
    cudaFuncSetAttribute(k_trainTiles, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
    k_trainTiles<<<slots, 128, sizeof(TrainSmem), s>>>(rec, n, tiles, gb, g.w, g.scratch.partial);
    const float b1 = 0.9f, b2 = 0.999f;
    float c1 = 1.f, c2 = 1.f;
    if (lr > 0.f) {
        g.step += 1;
        c1 = 1.f - std::pow(b1, (float)g.step);
        c2 = 1.f - std::pow(b2, (float)g.step);
    }
    k_reduceAdam<<<(kGuideParams + 255) / 256, 256, 0, s>>>(g.scratch.partial, slots, g.grads, g.params, g.m, g.v, lr,
                                                            b1, b2, 1e-8f, c1, c2, g.w, g.scratch.scalars);
}

size_t guidePartialBytes() { return sizeof(float) * (size_t)kSlot * kMaxSlots; }

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
    float f[64];
    guideFeatures(pp, nn, ww, f);
#pragma unroll
    for (int i = 0; i < 64; i += 2) *reinterpret_cast<uint32_t*>(x + i) = pack2(f[i], f[i + 1]);
}

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

}  // namespace xgb
