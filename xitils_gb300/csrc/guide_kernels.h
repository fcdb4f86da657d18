// Device-side state of the guiding network and the launch wrappers of guide.cu.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "guide.cuh"
#include "xgb_kernels.h"

namespace xgb {

// bf16 copies used by the tensor-core kernels (refreshed from the fp32 master
// parameters after every Adam step). W[l] is [out][in] (W[3] padded to 48 rows
// of which 40..47 stay zero), WT[l] = W[l]^T ([64][48] for the last layer);
// bias[3] has 48 entries, 40..47 zero.
struct GuideWeights {
    __nv_bfloat16* W[4];
    __nv_bfloat16* WT[4];
    float* bias[4];
};

struct GuideScratch {
    __nv_bfloat16* X0;  // feature rows [rows][64] of the inference entry points
    float* Y;           // outputs [rows][48]
    float* partial;     // per-CTA partial gradients of a training step (guidePartialBytes())
    float* scalars;     // [0] total sample weight, [1] loss of the last training step,
                        // [2] (as unsigned int) ERR_WAIT of the tensor-memory row inference
};

struct GuideDevice {
    float* params;  // fp32 master parameters (kGuideParams)
    float* grads;
    float* m;
    float* v;
    GuideWeights w;
    GuideScratch scratch;
    int maxRows;  // training batch capacity (multiple of 64)
    int waitLimit;  // polls of a tensor-memory inference wait before it gives up (xgb_guide_set_wait_limit)
    int step;     // Adam step count
    // training pool filled by the wavefront (records with non-zero radiance)
    GuideRecord* pool;
    unsigned int* poolCount;  // may run past poolCap; readers clamp
    int poolCap;
    int batch;  // rows per Adam step taken from the pool
};

__device__ void guideStoreBf16(const GuideWeights& w, int i, float p);

void guideRefresh(const GuideDevice& g, cudaStream_t s);
// Network outputs Y [rowsPad][48] of feature rows X0 [rowsPad][64] (tcgen05 kernel of
// guide_tc.cu); a timed-out wait sets ERR_WAIT in the word at g.scratch.scalars + 2.
void guideInferRows(const GuideDevice& g, const __nv_bfloat16* X0, int rowsPad, float* Y, cudaStream_t s);
// Bytes of GuideScratch::partial.
size_t guidePartialBytes();
// One Adam step (lr > 0) or gradients only (lr == 0) on records [0, n) (at most maxRows).
void guideTrainStep(GuideDevice& g, const GuideRecord* rec, int n, GuideBounds gb, float lr, cudaStream_t s);
// Training targets of the records [0, min(*nDev, cap)) from the per-path accumulators.
void guideFinalizeRecords(GuideRecord* rec, const unsigned int* nDev, int cap, const float4* pathAcc, int product,
                          cudaStream_t s);
// Appends the records [0, min(*nDev, recCap)) that carry radiance to the training pool.
void guideCollect(const GuideDevice& g, const GuideRecord* rec, const unsigned int* nDev, int recCap, cudaStream_t s);
// Adam steps of g.batch rows over a pool that held `count` records (read by the
// host after a synchronisation), at most maxSteps; keeps a remainder smaller
// than a batch at the front for the next call.
// Returns the number of steps enqueued.
int guidePoolTrain(GuideDevice& g, unsigned int count, GuideBounds gb, float lr, int maxSteps, cudaStream_t s);
// Features of host-style inputs (p, n, wo arrays of float3) -> X0 rows.
void guideFeaturesFromPoints(const float* p, const float* n, const float* wo, int count, int rowsPad, GuideBounds gb,
                             __nv_bfloat16* X0, cudaStream_t s);
// Directions drawn from decoded output rows (Y [n][48]) and their mixture pdf.
void guideSampleRows(const float* Y, int n, uint32_t seed, float* dirs, float* pdf, cudaStream_t s);
// Per-path inference for the wavefront: mixture (10 float4 per path) for every hit in q[0, nActive);
// a timed-out wait of the tensor-memory kernel sets ERR_WAIT in ctrl->errors.
void guideInferPaths(const SceneDev& sc, const GuideDevice& g, GuideBounds gb, PathQueue q, HitQueue h, Ctrl* ctrl,
                     float4* mix, int grid, cudaStream_t s);
// Sets the dynamic shared-memory limit of the tensor-memory inference kernels
// and sizes their grid (once per process, on the current device).
cudaError_t guideTcPrepare();

}  // namespace xgb
