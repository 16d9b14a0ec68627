// OpenPBR instances of the ReSTIR DI passes (shade_stage.cuh),
// in its own translation unit for the same reasons as shade_pbr.cu.
#include "shade_stage.cuh"

namespace rtgb {

void launch_restir_pbr(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters,
    const LaunchShape* shapes, cudaStream_t stream) {
    k_restir_ris<true><<<shapes[11].grid, shapes[11].block, 0, stream>>>(fp, scene, paths, counters);
    k_restir_vis<true><<<shapes[12].grid, shapes[12].block, 0, stream>>>(fp, scene, paths, counters);
    k_restir<true><<<shapes[8].grid, shapes[8].block, 0, stream>>>(fp, scene, paths, counters);
}

// shapes[8], [11], [12]: the final, RIS and visibility passes.
void query_restir_pbr_shapes(int sm_count, LaunchShape* shapes) {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_restir<true>, 128, 0);
    shapes[8] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_restir_ris<true>, 128, 0);
    shapes[11] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_restir_vis<true>, 128, 0);
    shapes[12] = LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
}

}  // namespace rtgb
