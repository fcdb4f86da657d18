// Shade kernel variants for scenes with microfacet normal mapping (mask 1) or with
// MultiLobeSVBRDF (mask 2); see shade.cuh. Compiled with -fmad=false.
#include "shade.cuh"

namespace xgb {

void launchShadeMask1(const OneJob& job, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl, int numSMs,
                      cudaStream_t s) {
    launchShadeVariant<OneJob, 1, true>(job, in, h, out, sq, ctrl, numSMs, s);
}

void launchShadeMask2(const OneJob& job, PathQueue in, HitQueue h, PathQueue out, ShadowQueue sq, Ctrl* ctrl, int numSMs,
                      cudaStream_t s) {
    launchShadeVariant<OneJob, 2, true>(job, in, h, out, sq, ctrl, numSMs, s);
}

}  // namespace xgb
