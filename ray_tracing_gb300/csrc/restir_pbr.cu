// OpenPBR instance of the ReSTIR DI kernel, k_restir<true> (shade_stage.cuh),
// in its own translation unit for the same reasons as shade_pbr.cu.
#include "shade_stage.cuh"

namespace rtgb {

void launch_restir_pbr(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, LaunchShape shape,
    cudaStream_t stream) {
    k_restir<true><<<shape.grid, 128, 0, stream>>>(fp, scene, paths, counters);
}

LaunchShape query_restir_pbr_shape(int sm_count) {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_restir<true>, 128, 0);
    return LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
}

}  // namespace rtgb
