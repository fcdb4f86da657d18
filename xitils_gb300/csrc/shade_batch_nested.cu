// Shade kernel variant with both nested materials (mask 3) for the batches that
// contain any nested material (batches take neither guiding nor AOV planes); see
// shade.cuh. Compiled with -fmad=false.
#include "shade.cuh"

namespace xgb {

void launchShadeMask3Batch(const ManyJobs& jobs, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl,
                           int numSMs, cudaStream_t s) {
    launchShadeVariant<ManyJobs, 3, false>(jobs, in, h, out, sq, ctrl, numSMs, s);
}

}  // namespace xgb
