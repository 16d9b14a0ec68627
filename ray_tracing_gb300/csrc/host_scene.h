// The packed host scene behind the C ABI's opaque rtgb_host_scene: the arrays
// an rtgb_scene view points into. Filled by the builtin scene builders
// (host_scene.cpp), the SceneIR v2 adapter (scene_ir_adapter.cpp) and the
// scene file reader (rtgb_host_scene_load).
#pragma once

#include <array>
#include <string>
#include <vector>

#include "rtgb.h"

struct rtgb_host_scene {
    std::vector<rtgb_texture> textures;
    std::vector<float> texels;
    std::vector<rtgb_material> materials;
    std::vector<rtgb_sphere> spheres;
    std::vector<rtgb_quad> quads;
    std::vector<rtgb_triangle> triangles;
    std::vector<rtgb_medium> media;
    std::vector<rtgb_analytic_light> analytic;
    std::vector<rtgb_openpbr_material> openpbr;
    std::array<float, 3> background {0.0f, 0.0f, 0.0f};
};

namespace rtgb::scene::detail {
// An 8-bit PNG's texels appended to `texels` as RGB floats scaled by 1/255
// (scene_ir_adapter.cpp); false when no readable file is found.
bool load_png_texels(const std::string& path, int& width, int& height, std::vector<float>& texels);
}  // namespace rtgb::scene::detail

namespace rtgb::scene {
struct SceneMaterialConnection;
struct SceneTexture;
namespace detail {
// One OpenPBR texture connection bound to realtime texture `index`
// (scene_ir_adapter.cpp); throws for connections the core cannot read.
void bind_connection(rtgb_openpbr_material& out, const SceneMaterialConnection& c, const SceneTexture& tex, int index);
}  // namespace detail
}  // namespace rtgb::scene
