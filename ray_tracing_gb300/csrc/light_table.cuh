// The emissive light table (power CDF) built on the device.
#pragma once

#include "device_common.cuh"

namespace rtgb {

// Inputs of the light table: the scene's primitives (device arrays), the
// emission luminance of each material (material_emission_luminance,
// packed_scene_preparation.cpp:227-251, evaluated once per material on the
// host) and the environment's weight (4 pi x background luminance).
struct LightSources {
    const rtgb_sphere* spheres;
    const rtgb_quad* quads;
    const rtgb_triangle* triangles;
    int sphere_count, quad_count, triangle_count;
    const float* material_lum;
    int material_count;
    float environment_weight;
};

// Outputs: lights and cdf hold up to primitives + 1 entries, guide kGuide + 1,
// the maps one entry per primitive (light index or -1); counts[0] = the light
// count, counts[1] = the environment light's index or -1 (device ints).
struct LightTable {
    PackedLight* lights;
    float* cdf;
    int* guide;
    int* sphere_light;
    int* quad_light;
    int* triangle_light;
    int* counts;
};

size_t light_table_scratch_bytes(long long primitives);

// build_light_distribution (packed_scene_preparation.cpp:265-302): every
// emissive primitive in scene order (spheres, quads, triangles), then the
// environment, weighted by area x emission luminance; selection pdf = weight /
// total and cdf = running sum of the pdfs in that order, in single precision
// and in the reference's order of additions, so the table is bit-identical to
// the sequential host construction. Stream-ordered; the counts are ready when
// the stream reaches them.
cudaError_t launch_light_table(const LightSources& src, const LightTable& out, void* scratch, cudaStream_t stream);

}  // namespace rtgb
