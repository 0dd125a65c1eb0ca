// wf_host_scene.h — the host-side scene behind wf_host_scene_* (generated
// workloads and scene files): flat arrays a wf_scene_desc points into.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/wf_api.h"

struct wf_host_scene {
    int32_t config = 0;  // generator config, -1 for a loaded file
    std::vector<float> px, py, pz;
    std::vector<int32_t> idx;
    std::vector<int32_t> mesh_off, mesh_cnt, mesh_mat;
    std::vector<wf_material> mats;
    std::vector<float> cu, cv;                    // per triangle corner (only with UVs)
    std::vector<uint8_t> has_uv;                  // per mesh
    std::vector<std::vector<uint8_t>> tex_data;   // texels of each texture, raw
    std::vector<wf_texture> textures;
    std::vector<float> env;                       // equirect RGB (width*height*3)
    int32_t env_w = 0, env_h = 0;
    float env_scale = 1.0f;
    float env_tint[3] = {1.0f, 1.0f, 1.0f};
    wf_directional_light dir{{0.0f, 0.0f, 0.0f}, {1.0f, 1.0f, 1.0f}, 0.0f};
    float look_from[3] = {0, 0, 0}, look_at[3] = {0, 0, -1}, up[3] = {0, 1, 0};
    float vfov = 40.0f;
};
