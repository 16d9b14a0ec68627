// OpenPBR instance of the shade kernel, k_shade<true> (shade_stage.cuh), in its
// own translation unit so the large OpenPBR code compiles in parallel with the
// rest and never enters the legacy instances.
#include "shade_stage.cuh"

namespace rtgb {

// The OpenPBR shade stage is split: k_shade<true, true> (emission, next-event
// estimation, the random-walk step) queues the paths that scatter for
// k_scatter<true> (BSDF sampling, Russian roulette).
void launch_shade_pbr(const FrameParams* fp, DeviceScene scene, Paths paths, Counters* counters, int bounce,
    LaunchShape shape, LaunchShape scatter_shape, cudaStream_t stream) {
    k_shade<true, true><<<shape.grid, shape.block, 0, stream>>>(fp, scene, paths, counters, bounce);
    k_scatter<true><<<scatter_shape.grid, scatter_shape.block, 0, stream>>>(fp, scene, paths, counters, bounce);
}

LaunchShape query_shade_pbr_shape(int sm_count) {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_shade<true, true>, 128, 0);
    return LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
}

LaunchShape query_scatter_pbr_shape(int sm_count) {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_scatter<true>, 128, 0);
    return LaunchShape{sm_count * (blocks > 0 ? blocks : 1), 128};
}

}  // namespace rtgb
