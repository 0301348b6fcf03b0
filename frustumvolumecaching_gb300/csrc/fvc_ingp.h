/*
 * fvc_ingp.h - instant-ngp snapshot (.ingp) reader used by the model loader.
 */
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace fvc_ingp {

/* what load_ingp_snapshot (src/loader.cu:146-230) reads from a snapshot */
struct Snapshot {
    int aabb_scale = 1;
    float aabb_min[3] = {0, 0, 0}, aabb_max[3] = {1, 1, 1};
    int n_levels = 16, n_features = 2, log2_hashmap_size = 19, base_resolution = 16;
    int base_neurons = 64, base_hidden = 1, head_neurons = 64, head_hidden = 2, sh_degree = 4;
    std::vector<uint16_t> params;        /* fp16: density MLP, color MLP, hash grid (the reference's set_params order) */
    std::vector<uint16_t> density_grid;  /* fp16 [cascade][128^3] in Morton order */
};

/* false with a message on a missing, corrupt or non-nerf snapshot */
bool read_snapshot(const std::string &file, Snapshot &out, std::string &err);

}  // namespace fvc_ingp
