// Shade kernel variant with both nested materials (mask 3) for one scene; see
// shade.cuh. Compiled with -fmad=false.
#include "shade.cuh"

namespace xgb {

void launchShadeMask3(const OneJob& job, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl, int grid,
                      cudaStream_t s) {
    k_shade<OneJob, 3, true><<<grid, kShadeBlock, 0, s>>>(job, in, h, out, sq, ctrl);
}

}  // namespace xgb
