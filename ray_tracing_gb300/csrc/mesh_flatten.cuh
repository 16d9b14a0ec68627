// Instanced meshes flattened into packed triangles on the device.
#pragma once

#include "device_common.cuh"

namespace rtgb {

// One prototype, its arrays concatenated with the other prototypes' in the
// device copy of the mesh set.
struct MeshProtoDev {
    long long point_offset;   // into points (3 doubles each)
    long long tri_offset;     // into corners / normals / texcoords / materials (per triangle)
    int tri_count;
    int has_normals;
    int has_texcoords;
};

// One instance; `out_offset` = its first triangle in the scene's triangle array.
struct MeshInstDev {
    long long out_offset;
    int prototype;
    int material;
    int flip;
    double world[12];
    double normal_matrix[9];
};

struct MeshSetDev {
    const double* points;
    const int* corners;        // 3 per triangle
    const double* normals;     // 9 per triangle (prototypes with normals)
    const double* texcoords;   // 6 per triangle (prototypes with texcoords)
    const int* materials;      // per triangle
    const MeshProtoDev* prototypes;
    const MeshInstDev* instances;
    int instance_count;
    long long first_out;       // instances[0].out_offset
    long long end_out;         // one past the last flattened triangle
};

// add_v2_mesh (realtime_scene_adapter.cpp:289-346) for every instance: points
// by the 3 x 4 world transform, normals by the transposed normal matrix and
// normalised, both in double precision and in the host lowering's order of
// operations, then rounded to float; texcoords rounded to float; corners 1
// and 2 swapped where the instance flips the winding. A normal whose length
// is not finite or at most 1e-12 sets *bad_normal.
cudaError_t launch_flatten_meshes(const MeshSetDev& set, rtgb_triangle* out, int* bad_normal, int sm_count,
    cudaStream_t stream);

// max over every primitive of the coordinate magnitudes the LBVH padding
// uses (|center| + |radius| per sphere axis, |origin| + |edge_u| + |edge_v|
// per quad axis, |p0|, |p1|, |p2| per triangle axis), NaN skipped, as float
// bits into *scale_bits (zeroed first); the same value as the host's running
// std::max over the primitives.
cudaError_t launch_scene_scale(const DeviceScene& d, unsigned* scale_bits, int sm_count, cudaStream_t stream);

}  // namespace rtgb
