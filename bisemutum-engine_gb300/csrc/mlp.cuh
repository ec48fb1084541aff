// mlp.cuh — the radiance-cache network: input encoding and parameter layout,
// shared by the CUDA kernels (mlp_tc.cu, mlp.cu, train_paths.cu) and the host code.
//
// Network: 12 raw inputs -> 64 encoded features -> 4 hidden layers of 64 with
// ReLU -> 3 outputs (RGB radiance), no biases (a constant-1 feature feeds the
// first layer).  Weights are BF16 for the tensor cores with FP32 master copies
// for Adam; products accumulate in FP32.
//
// Raw inputs (12): position (3, normalised to the scene box), outgoing
// direction (2: theta/pi, phi/2pi + 1/2), normal (2, same mapping), roughness,
// albedo (3), path depth (bounce / 8).
// Encoding (64): for each of the 7 geometric inputs x and k = 0..3,
// sin(2^k pi x) and cos(2^k pi x) (56 features), then roughness, albedo rgb,
// depth, 1, 0, 0.
#pragma once
#include <stdint.h>

#include "pt_math.cuh"

namespace bsm {

constexpr int kMlpRaw = 12;
constexpr int kMlpIn = 64;
constexpr int kMlpHid = 64;
constexpr int kMlpOut = 3;
constexpr int kMlpOutPad = 8;      // output layer rows padded to an n8 tile
constexpr int kMlpHidden = 4;      // hidden layers
// parameters: W0..W3 [64 out][64 in], W4 [8 out][64 in] (rows 3..7 zero), row-major
constexpr int kMlpLayerParams = kMlpHid * kMlpIn;
constexpr int kMlpParams = kMlpHidden * kMlpLayerParams + kMlpOutPad * kMlpHid;  // 16896

// Position of parameter i (row i / 64, column i % 64 of the row-major [264][64]
// weight matrix) in the BF16 copies the tensor-core kernels read: each row is
// one 128-byte line whose 16-byte chunk c (columns 8c..8c+7) sits at chunk
// c ^ (row mod 8), the layout of the kernels' shared-memory tiles (128-byte
// swizzle), so that one bulk copy moves the weights into shared memory.
BSM_HD int mlp_tile_index(int i) {
    const int r = i >> 6, c = i & 63;
    return (r << 6) | ((((c >> 3) ^ (r & 7)) << 3) | (c & 7));
}

// Encoded feature f of a sample with raw inputs `raw`.
BSM_HD float mlp_feature(const float* raw, int f) {
    if (f < 56) {
        int d = f >> 3, k = (f & 7) >> 1;
        float s, c;
        sincos_turns(raw[d] * (float)(1 << k) * 0.5f, &s, &c);
        return (f & 1) ? c : s;
    }
    int r = f - 56;
    if (r < 5) return raw[7 + r];
    return r == 5 ? 1.0f : 0.0f;
}

// Raw inputs of a path vertex.
BSM_HD void mlp_raw_inputs(V3 p, V3 box_lo, V3 box_inv, V3 wo, V3 n, float roughness, V3 albedo, float depth,
                           float* raw) {
    raw[0] = (p.x - box_lo.x) * box_inv.x;
    raw[1] = (p.y - box_lo.y) * box_inv.y;
    raw[2] = (p.z - box_lo.z) * box_inv.z;
    float t, ph;
    t = atan2_det(sqrtf(wo.x * wo.x + wo.z * wo.z), wo.y) * BSM_INV_PI;
    ph = atan2_det(wo.z, wo.x) * (0.5f * BSM_INV_PI) + 0.5f;
    raw[3] = t; raw[4] = ph;
    t = atan2_det(sqrtf(n.x * n.x + n.z * n.z), n.y) * BSM_INV_PI;
    ph = atan2_det(n.z, n.x) * (0.5f * BSM_INV_PI) + 0.5f;
    raw[5] = t; raw[6] = ph;
    raw[7] = roughness;
    raw[8] = albedo.x; raw[9] = albedo.y; raw[10] = albedo.z;
    raw[11] = depth;
}

}  // namespace bsm
