// FP64 instantiation of the step passes (compiled with --fmad=false: every
// multiply and add rounds separately, as in the reference's arithmetic).
#include "vx3g_step.cuh"

namespace vx3g {

void launch_links_fp64(const Dev &d, cudaStream_t s) {
    if (d.nl) k_links<double><<<(d.nl + 255) / 256, 256, 0, s>>>(d);
}
void launch_voxels_fp64(const Dev &d, int parity, cudaStream_t s) {
    if (d.nv) k_voxels<double><<<(d.nv + 255) / 256, 256, 0, s>>>(d, parity);
}

}  // namespace vx3g
