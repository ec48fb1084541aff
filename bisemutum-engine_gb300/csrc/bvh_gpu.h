// bvh_gpu.h — device build of the compressed 8-wide BVH (see bvh_gpu.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "bsm_pt.h"
#include "bvh_layout.h"

namespace bsm {

struct DeviceBvhResult {
    CwNode* nodes = nullptr;   // cudaMalloc'd by the build, num_nodes entries; owned by the caller afterwards
    CwTri* tris = nullptr;     // cudaMalloc'd by the build, num_tris entries
    uint32_t num_nodes = 0;
    uint32_t num_tris = 0;
    uint32_t max_depth = 0;
    double sah_cost = 0.0;     // SAH cost of the binary BVH before collapsing
    double build_ms = 0.0;     // wall time of the build, waits included
};

// Device scratch the build holds while it runs (bytes), for num_tris triangles.
uint64_t device_build_scratch_bytes(uint32_t num_tris);
// Output bytes (nodes upper bound + triangles) the build allocates.
uint64_t device_build_output_bytes(uint32_t num_tris);

// Builds the BVH of num_tris triangles whose data are DEVICE arrays: positions
// (3 floats per vertex, nv vertices), indices (3 per triangle, or null for a
// soup), per-triangle material ids (or null: 0) and per-material transparency
// (or null: 0) that leaf triangles carry for the any-hit rule.  Work runs on
// `st`; the call returns when the build is done.  On failure `err` says why and
// nothing is left allocated.
bool build_cwbvh_device(cudaStream_t st, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t num_tris,
                        const uint32_t* mat, const float* transparency, uint32_t num_materials,
                        const bsm_bvh_opts* opts, DeviceBvhResult& out, std::string& err);

}  // namespace bsm
