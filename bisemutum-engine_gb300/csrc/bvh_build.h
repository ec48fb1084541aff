// bvh_build.h — host builder of the compressed 8-wide BVH (see bvh_build.cpp).
#pragma once
#include <string>
#include <vector>

#include "bsm_pt.h"
#include "bvh_layout.h"

namespace bsm {

struct BvhBuildResult {
    std::vector<CwNode> nodes;
    std::vector<CwTri> tris;
    uint32_t max_depth = 0;
    double sah_cost = 0.0;
    double build_ms = 0.0;
};

// positions: 3 floats per vertex; indices: 3 per triangle or NULL (soup).
bool build_cwbvh(const float* positions, const uint32_t* indices, uint32_t num_tris, const uint32_t* material_ids,
                 const bsm_bvh_opts* opts, BvhBuildResult& out, std::string& err);

}  // namespace bsm
