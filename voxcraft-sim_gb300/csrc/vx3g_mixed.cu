// Mixed-precision instantiation of the step passes: FP32 link math and force
// sums, FP64 position/orientation/momentum accumulation.
#include "vx3g_step.cuh"

namespace vx3g {

void launch_links_mixed(const Dev &d, cudaStream_t s) {
    if (d.nl) k_links<float><<<(d.nl + 255) / 256, 256, 0, s>>>(d);
}
void launch_voxels_mixed(const Dev &d, int parity, cudaStream_t s) {
    if (d.nv) k_voxels<float><<<(d.nv + 255) / 256, 256, 0, s>>>(d, parity);
}

}  // namespace vx3g
