// Shade kernel variants for scenes with microfacet normal mapping (mask 1) or with
// MultiLobeSVBRDF (mask 2); see shade.cuh. Compiled with -fmad=false.
#include "shade.cuh"

namespace xgb {

void launchShadeMask1(const OneJob& job, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl, int grid,
                      cudaStream_t s) {
    k_shade<OneJob, 1, true><<<grid, kShadeBlock, 0, s>>>(job, in, h, out, sq, ctrl);
}

void launchShadeMask2(const OneJob& job, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl, int grid,
                      cudaStream_t s) {
    k_shade<OneJob, 2, true><<<grid, kShadeBlock, 0, s>>>(job, in, h, out, sq, ctrl);
}

}  // namespace xgb
