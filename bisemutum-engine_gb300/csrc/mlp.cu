// mlp.cu — fused BF16 tensor-core kernels of the radiance cache.
//
// Per warp, a tile of 16 samples goes through the whole network with
// mma.sync.m16n8k16 (BF16 inputs, FP32 accumulation).  The accumulator
// fragment of two adjacent n8 tiles is exactly the A fragment of one k16 step
// of the next layer, so activations stay in registers from layer to layer
// (the fully fused scheme of Müller et al., "Real-time Neural Radiance
// Caching for Path Tracing", 2021).  Weights sit in shared memory with rows
// padded to 72 elements, so that ldmatrix's eight 16-byte rows fall in
// distinct banks.
//
// (Inference runs on the tcgen05 path of mlp_tc.cu; the training step stays
// on mma.sync, whose register fragments carry the activations through the
// backward pass.)
//
//   k_mlp_train   forward, relative-L2 loss gradient, backward through the
//                 layers, weight gradients dW_l = g_z^T a_{l-1} (also on the
//                 tensor cores: per block 64 samples at a time, each warp
//                 owning 16 rows of every layer's gradient in shared FP32,
//                 then one global vector atomic per 4 weights per block)
//   k_mlp_adam    Adam on the FP32 master weights, BF16 copies for the next pass
//
// The training step stays on mma.sync because its backward pass reuses the
// forward's register fragments and needs the activations and gradients
// transposed for the weight gradient: 16-sample tiles in registers and
// shared memory serve both, at 26 us per Adam step of ~13,000 vertices.
#include <cuda_bf16.h>
#include <atomic>
#include <cuda_runtime.h>

#include "mlp.cuh"
#include "pt_device.h"

namespace bsm {

constexpr int kLd = 72;                                   // padded row length (bf16 elements)
constexpr int kWSmem = (kMlpHidden * 64 + kMlpOutPad) * kLd;  // weight elements in shared memory

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }
__device__ __forceinline__ uint32_t pack_u16(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Loads the BF16 weights (global, row-major [out][64], 16-byte aligned) into
// padded shared rows, 16 bytes per load.
__device__ __forceinline__ void load_weights(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* sw) {
    const int rows = kMlpHidden * 64 + kMlpOutPad;
    const uint4* src = reinterpret_cast<const uint4*>(w);
#pragma unroll 4
    for (int i = threadIdx.x; i < rows * 8; i += blockDim.x) {
        int r = i >> 3, c = (i & 7) * 8;
        *reinterpret_cast<uint4*>(sw + r * kLd + c) = __ldg(src + i);
    }
}

// Four 8x8 BF16 matrices from shared memory (ldmatrix): lane L gives the
// address of row L & 7 of matrix L >> 3; register i of lane (g, t) receives
// elements (g, 2t) and (g, 2t + 1) of matrix i.
__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a)
                 : "memory");
}

// Four transposed 8x8 BF16 matrices from shared memory (ldmatrix .trans):
// lane L gives the address of row L & 7 of matrix L >> 3; register i of lane
// (g, t) receives elements (2t, g) and (2t + 1, g) of matrix i, which is the
// mma fragment layout of a matrix stored with its K dimension along the rows.
__device__ __forceinline__ void ldsm_x4_t(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a)
                 : "memory");
}

// Encoded input tile as A fragments: act[kk] covers features 16kk..16kk+15.
__device__ __forceinline__ void encode_tile(const float* raw_g, const float* raw_g8, uint32_t (&act)[4][4], int t) {
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        int f0 = 16 * kk + 2 * t, f1 = f0 + 8;
        act[kk][0] = pack_bf16(mlp_feature(raw_g, f0), mlp_feature(raw_g, f0 + 1));
        act[kk][1] = pack_bf16(mlp_feature(raw_g8, f0), mlp_feature(raw_g8, f0 + 1));
        act[kk][2] = pack_bf16(mlp_feature(raw_g, f1), mlp_feature(raw_g, f1 + 1));
        act[kk][3] = pack_bf16(mlp_feature(raw_g8, f1), mlp_feature(raw_g8, f1 + 1));
    }
}

// One hidden layer: out = relu(W act) as A fragments of the next layer.
// B[k=in][n=out] = W[out][in] lies in shared memory with K along the rows'
// length, so plain 8x8 matrix loads give the B fragments (matrices: k half
// (lane >> 3) & 1, n block of the pair (lane >> 4)).
__device__ __forceinline__ void hidden_layer(const __nv_bfloat16* sw, const uint32_t (&in)[4][4], uint32_t (&out)[4][4],
                                             int g, int t) {
    const int lane = threadIdx.x & 31, mi = lane >> 3, r = lane & 7;
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int jp = 0; jp < 4; ++jp) {
            uint32_t b0, b1, b2, b3;
            ldsm_x4(b0, b1, b2, b3, sw + (8 * (2 * jp + (mi >> 1)) + r) * kLd + 16 * kk + (mi & 1) * 8);
            mma16816(acc[2 * jp], in[kk], b0, b1);
            mma16816(acc[2 * jp + 1], in[kk], b2, b3);
        }
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        out[kk][0] = pack_bf16(fmaxf(acc[2 * kk][0], 0.0f), fmaxf(acc[2 * kk][1], 0.0f));
        out[kk][1] = pack_bf16(fmaxf(acc[2 * kk][2], 0.0f), fmaxf(acc[2 * kk][3], 0.0f));
        out[kk][2] = pack_bf16(fmaxf(acc[2 * kk + 1][0], 0.0f), fmaxf(acc[2 * kk + 1][1], 0.0f));
        out[kk][3] = pack_bf16(fmaxf(acc[2 * kk + 1][2], 0.0f), fmaxf(acc[2 * kk + 1][3], 0.0f));
    }
}

// Output layer (8 rows, 3 used): y fragment (row g: y[0], y[1] = channels 2t, 2t+1; row g+8: y[2], y[3]).
// One matrix load covers two k steps (matrices: k half (lane >> 3) & 1, k step of the pair (lane >> 4)).
__device__ __forceinline__ void output_layer(const __nv_bfloat16* sw4, const uint32_t (&in)[4][4], float (&y)[4],
                                             int g, int t) {
    const int lane = threadIdx.x & 31, mi = lane >> 3, r = lane & 7;
    y[0] = y[1] = y[2] = y[3] = 0.0f;
#pragma unroll
    for (int kp = 0; kp < 2; ++kp) {
        uint32_t b0, b1, b2, b3;
        ldsm_x4(b0, b1, b2, b3, sw4 + r * kLd + 16 * (2 * kp + (mi >> 1)) + (mi & 1) * 8);
        mma16816(y, in[2 * kp], b0, b1);
        mma16816(y, in[2 * kp + 1], b2, b3);
    }
}


// --------------------------------------------------------------- training ----
// Shared memory: weights | dW (fp32) | per warp: activations e,a0..a3 and
// gradients gz0..gz3, gy as bf16 [16][72] tiles.
constexpr int kTileElems = 16 * kLd;
constexpr size_t kTrainWarpBytes = 10 * kTileElems * 2;
constexpr size_t kTrainSmem = kWSmem * 2 + kMlpParams * 4 + 4 * kTrainWarpBytes;

__device__ __forceinline__ void store_act_tile(__nv_bfloat16* tile, const uint32_t (&act)[4][4], int g, int t) {
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        int c = 16 * kk + 2 * t;
        *reinterpret_cast<uint32_t*>(tile + g * kLd + c) = act[kk][0];
        *reinterpret_cast<uint32_t*>(tile + (g + 8) * kLd + c) = act[kk][1];
        *reinterpret_cast<uint32_t*>(tile + g * kLd + c + 8) = act[kk][2];
        *reinterpret_cast<uint32_t*>(tile + (g + 8) * kLd + c + 8) = act[kk][3];
    }
}

// g_a (C fragments over 64 columns) -> g_z = g_a * (a > 0), stored as bf16 and
// returned as A fragments for the next backward product.
__device__ __forceinline__ void relu_grad(const float (&ga)[8][4], const __nv_bfloat16* a_tile, __nv_bfloat16* gz_tile,
                                          uint32_t (&gz)[4][4], int g, int t) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        int c = 8 * j + 2 * t;
        uint32_t m0 = *reinterpret_cast<const uint32_t*>(a_tile + g * kLd + c);
        uint32_t m1 = *reinterpret_cast<const uint32_t*>(a_tile + (g + 8) * kLd + c);
        float v0 = bf16_lo(m0) > 0.0f ? ga[j][0] : 0.0f;
        float v1 = bf16_hi(m0) > 0.0f ? ga[j][1] : 0.0f;
        float v2 = bf16_lo(m1) > 0.0f ? ga[j][2] : 0.0f;
        float v3 = bf16_hi(m1) > 0.0f ? ga[j][3] : 0.0f;
        uint32_t p0 = pack_bf16(v0, v1), p1 = pack_bf16(v2, v3);
        *reinterpret_cast<uint32_t*>(gz_tile + g * kLd + c) = p0;
        *reinterpret_cast<uint32_t*>(gz_tile + (g + 8) * kLd + c) = p1;
        int kk = j >> 1;
        if ((j & 1) == 0) { gz[kk][0] = p0; gz[kk][1] = p1; }
        else { gz[kk][2] = p0; gz[kk][3] = p1; }
    }
}

// g_a = g_z W for a [64 out][64 in] weight block: B[k=out][n=in] = W[out][in]
// lies in shared memory with K along the rows, so transposed loads give the
// B fragments (matrices: k half (lane >> 3) & 1, n block of the pair (lane >> 4)).
__device__ __forceinline__ void backward_data(const __nv_bfloat16* sw, const uint32_t (&gz)[4][4], float (&ga)[8][4],
                                              int lane) {
    const int mi = lane >> 3, r = lane & 7;
#pragma unroll
    for (int j = 0; j < 8; ++j) ga[j][0] = ga[j][1] = ga[j][2] = ga[j][3] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int jp = 0; jp < 4; ++jp) {
            uint32_t b0, b1, b2, b3;
            ldsm_x4_t(b0, b1, b2, b3, sw + (16 * kk + (mi & 1) * 8 + r) * kLd + 8 * (2 * jp + (mi >> 1)));
            mma16816(ga[2 * jp], gz[kk], b0, b1);
            mma16816(ga[2 * jp + 1], gz[kk], b2, b3);
        }
}

// Rows [m0, m0 + 16) of dW[out][in] += sum over the block's 64 samples (the
// four warps' 16-sample tiles) of gz[s][out] * a[s][in], for one 64x64 layer.
// A[m=out][k=s] and B[k=s][n=in] are both stored [s][.]: transposed loads.
// The calling warp owns these rows, so the update is a plain read-add-write.
__device__ __forceinline__ void weight_grad_rows(const __nv_bfloat16* const (&gz_q)[4],
                                                 const __nv_bfloat16* const (&a_q)[4], float* dW, int m0, int lane) {
    const int mi = lane >> 3, r = lane & 7, g = lane >> 2, t = lane & 3;
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint32_t A[4];
        ldsm_x4_t(A[0], A[1], A[2], A[3], gz_q[q] + ((mi >> 1) * 8 + r) * kLd + m0 + (mi & 1) * 8);
#pragma unroll
        for (int jp = 0; jp < 4; ++jp) {
            uint32_t b0, b1, b2, b3;
            ldsm_x4_t(b0, b1, b2, b3, a_q[q] + ((mi & 1) * 8 + r) * kLd + 8 * (2 * jp + (mi >> 1)));
            mma16816(acc[2 * jp], A, b0, b1);
            mma16816(acc[2 * jp + 1], A, b2, b3);
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        float2* p0 = reinterpret_cast<float2*>(dW + (m0 + g) * 64 + 8 * j + 2 * t);
        float2* p1 = reinterpret_cast<float2*>(dW + (m0 + g + 8) * 64 + 8 * j + 2 * t);
        float2 v0 = *p0, v1 = *p1;
        *p0 = make_float2(v0.x + acc[j][0], v0.y + acc[j][1]);
        *p1 = make_float2(v1.x + acc[j][2], v1.y + acc[j][3]);
    }
}

// Output layer (8 rows): columns [16 jb, 16 jb + 16) of dW4[out][in] += sum over
// the block's 64 samples of gy[s][out] * a3[s][in]; rows 8..15 of the A tile are zero.
__device__ __forceinline__ void weight_grad_out(const __nv_bfloat16* const (&gy_q)[4],
                                                const __nv_bfloat16* const (&a_q)[4], float* dW4, int jb, int lane) {
    const int mi = lane >> 3, r = lane & 7, g = lane >> 2, t = lane & 3;
    float acc[2][4] = {{0.0f, 0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f, 0.0f}};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint32_t A[4];
        ldsm_x4_t(A[0], A[1], A[2], A[3], gy_q[q] + ((mi >> 1) * 8 + r) * kLd);  // matrices 1, 3 repeat 0, 2
        A[1] = 0u;
        A[3] = 0u;
        uint32_t b0, b1, b2, b3;
        ldsm_x4_t(b0, b1, b2, b3, a_q[q] + ((mi & 1) * 8 + r) * kLd + 8 * (2 * jb + (mi >> 1)));
        mma16816(acc[0], A, b0, b1);
        mma16816(acc[1], A, b2, b3);
    }
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) {
        float2* p = reinterpret_cast<float2*>(dW4 + g * 64 + 8 * (2 * jb + jj) + 2 * t);
        float2 v = *p;
        *p = make_float2(v.x + acc[jj][0], v.y + acc[jj][1]);
    }
}

// samples: as k_mlp_predict (targets in the 4th float4).  Accumulates the
// gradient of the mean relative L2 loss over `n` samples into dW_global and
// the loss into loss_out[0].  A block takes 64 samples at a time (one 16-row
// tile per warp); after forward and backward passes each warp reduces its own
// rows of every layer's weight gradient over all 64 samples on the tensor
// cores, into the block's FP32 copy, and the block adds that copy to
// dW_global once at the end.
__global__ void __launch_bounds__(128) k_mlp_train(const __nv_bfloat16* __restrict__ w, const float4* __restrict__ s,
                                                   uint32_t n, float* dW_global, float* loss_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    float* sdw = reinterpret_cast<float*>(smem_raw + kWSmem * 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    auto tile_of = [&](int wq, int i) {
        return reinterpret_cast<__nv_bfloat16*>(smem_raw + kWSmem * 2 + kMlpParams * 4 + wq * kTrainWarpBytes) +
               i * kTileElems;
    };
    __nv_bfloat16* act_t[5];  // e, a0, a1, a2, a3
    __nv_bfloat16* gz_t[5];   // gz0, gz1, gz2, gz3, gy
    for (int i = 0; i < 5; ++i) { act_t[i] = tile_of(warp, i); gz_t[i] = tile_of(warp, 5 + i); }
    load_weights(w, sw);
    for (int i = threadIdx.x; i < kMlpParams / 4; i += blockDim.x)
        reinterpret_cast<float4*>(sdw)[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    __syncthreads();
    const float inv = 1.0f / (3.0f * (float)n);
    float loss = 0.0f;
    const uint32_t groups = (n + 63) / 64;
    for (uint32_t grp = blockIdx.x; grp < groups; grp += gridDim.x) {   // uniform trip count within the block
        uint32_t r0 = (grp * 4 + warp) * 16 + g, r1 = r0 + 8;          // rows >= n: zero loss gradient
        float raw0[kMlpRaw], raw1[kMlpRaw];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float4 a = r0 < n ? s[4 * (size_t)r0 + k] : make_float4(0, 0, 0, 0);
            float4 b = r1 < n ? s[4 * (size_t)r1 + k] : make_float4(0, 0, 0, 0);
            raw0[4 * k] = a.x; raw0[4 * k + 1] = a.y; raw0[4 * k + 2] = a.z; raw0[4 * k + 3] = a.w;
            raw1[4 * k] = b.x; raw1[4 * k + 1] = b.y; raw1[4 * k + 2] = b.z; raw1[4 * k + 3] = b.w;
        }
        uint32_t act[4][4], tmp[4][4];
        encode_tile(raw0, raw1, act, t);
        store_act_tile(act_t[0], act, g, t);
        hidden_layer(sw + 0 * 64 * kLd, act, tmp, g, t);
        store_act_tile(act_t[1], tmp, g, t);
        hidden_layer(sw + 1 * 64 * kLd, tmp, act, g, t);
        store_act_tile(act_t[2], act, g, t);
        hidden_layer(sw + 2 * 64 * kLd, act, tmp, g, t);
        store_act_tile(act_t[3], tmp, g, t);
        hidden_layer(sw + 3 * 64 * kLd, tmp, act, g, t);
        store_act_tile(act_t[4], act, g, t);
        float y[4];
        output_layer(sw + 4 * 64 * kLd, act, y, g, t);
        // loss gradient (channels 2t, 2t+1 of rows g and g+8; channels >= 3 are padding)
        float gy[4];
        {
            float4 t0 = r0 < n ? s[4 * (size_t)r0 + 3] : make_float4(0, 0, 0, 0);
            float4 t1 = r1 < n ? s[4 * (size_t)r1 + 3] : make_float4(0, 0, 0, 0);
            float tg0[4] = {t0.x, t0.y, t0.z, 0.0f}, tg1[4] = {t1.x, t1.y, t1.z, 0.0f};
            for (int e = 0; e < 4; ++e) {
                int ch = 2 * t + (e & 1);
                bool row_ok = (e < 2) ? (r0 < n) : (r1 < n);
                float target = (e < 2) ? tg0[ch < 3 ? ch : 3] : tg1[ch < 3 ? ch : 3];
                float yy = y[e];
                float d = yy - target, den = yy * yy + 0.01f;
                bool ok = row_ok && ch < 3;
                loss += ok ? d * d / den * inv : 0.0f;
                gy[e] = ok ? 2.0f * d / den * inv : 0.0f;
            }
        }
        uint32_t gyp0 = pack_bf16(gy[0], gy[1]), gyp1 = pack_bf16(gy[2], gy[3]);
        {
            __nv_bfloat16* gyt = gz_t[4];
            int c = 2 * t;
            *reinterpret_cast<uint32_t*>(gyt + g * kLd + c) = gyp0;
            *reinterpret_cast<uint32_t*>(gyt + (g + 8) * kLd + c) = gyp1;
        }
        // g_a3 = gy W4 (K = 8 padded to 16): B[k=out][n=in] rows 0..7 of W4, four n blocks per transposed load
        float ga[8][4];
        uint32_t gz[4][4];
        {
            uint32_t A[4] = {gyp0, gyp1, 0u, 0u};
            const __nv_bfloat16* w4 = sw + 4 * 64 * kLd;
#pragma unroll
            for (int jq = 0; jq < 2; ++jq) {
                uint32_t b[4];
                ldsm_x4_t(b[0], b[1], b[2], b[3], w4 + (lane & 7) * kLd + 8 * (4 * jq + (lane >> 3)));
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    float* c = ga[4 * jq + i];
                    c[0] = c[1] = c[2] = c[3] = 0.0f;
                    mma16816(ga[4 * jq + i], A, b[i], 0u);
                }
            }
        }
        __syncwarp();
        relu_grad(ga, act_t[4], gz_t[3], gz, g, t);   // gz3
        backward_data(sw + 3 * 64 * kLd, gz, ga, lane);
        relu_grad(ga, act_t[3], gz_t[2], gz, g, t);   // gz2
        backward_data(sw + 2 * 64 * kLd, gz, ga, lane);
        relu_grad(ga, act_t[2], gz_t[1], gz, g, t);   // gz1
        backward_data(sw + 1 * 64 * kLd, gz, ga, lane);
        relu_grad(ga, act_t[1], gz_t[0], gz, g, t);   // gz0
        __syncthreads();                               // all four tiles of the group are in shared memory
        // weight gradients: dW_l = gz_l^T a_{l-1}; dW4 = gy^T a3.  Warp w: rows 16w..16w+15 of the
        // hidden layers, columns 16w..16w+15 of the output layer.
#pragma unroll 1
        for (int l = 0; l < 4; ++l) {
            const __nv_bfloat16* const gq[4] = {tile_of(0, 5 + l), tile_of(1, 5 + l), tile_of(2, 5 + l),
                                                tile_of(3, 5 + l)};
            const __nv_bfloat16* const aq[4] = {tile_of(0, l), tile_of(1, l), tile_of(2, l), tile_of(3, l)};
            weight_grad_rows(gq, aq, sdw + l * kMlpLayerParams, 16 * warp, lane);
        }
        {
            const __nv_bfloat16* const gq[4] = {tile_of(0, 9), tile_of(1, 9), tile_of(2, 9), tile_of(3, 9)};
            const __nv_bfloat16* const aq[4] = {tile_of(0, 4), tile_of(1, 4), tile_of(2, 4), tile_of(3, 4)};
            weight_grad_out(gq, aq, sdw + 4 * kMlpLayerParams, warp, lane);
        }
        __syncthreads();                               // tiles are rewritten by the next group
    }
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if (lane == 0) atomicAdd(loss_out, loss);
    for (int i = threadIdx.x; i < kMlpParams / 4; i += blockDim.x) {
        float4 v = reinterpret_cast<const float4*>(sdw)[i];
        if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f)
            atomicAdd(reinterpret_cast<float4*>(dW_global) + i, v);
    }
}

// Adam (Kingma and Ba 2015) on the fp32 master weights; writes the bf16 copy.
// With ema_decay > 0 it also keeps an exponential moving average of the
// weights (zero-started, so ema_corr = 1 / (1 - decay^steps) corrects its bias)
// and writes the corrected average's bf16 copy, which renders read.
__global__ void k_mlp_adam(float* __restrict__ wm, __nv_bfloat16* __restrict__ wb, const float* __restrict__ dW,
                           float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2, float eps,
                           float bc1, float bc2, float* __restrict__ ema, __nv_bfloat16* __restrict__ emab,
                           float ema_decay, float ema_corr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    float gr = dW[i];
    float mi = b1 * m[i] + (1.0f - b1) * gr;
    float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    float mh = mi / bc1, vh = vi / bc2;
    float wi = wm[i] - lr * mh / (sqrtf(vh) + eps);
    // padded output rows stay zero
    if (i >= kMlpHidden * kMlpLayerParams + kMlpOut * kMlpHid) wi = 0.0f;
    wm[i] = wi;
    wb[i] = __float2bfloat16_rn(wi);
    if (ema_decay > 0.0f) {
        float e = ema_decay * ema[i] + (1.0f - ema_decay) * wi;
        ema[i] = e;
        emab[i] = __float2bfloat16_rn(e * ema_corr);
    }
}

// ------------------------------------------------------------- launchers ----
// Per device (ordinal < 64): the opt-in shared-memory size is a per-device function attribute.
static std::atomic<uint64_t> g_mlp_attr{0};
static int g_mlp_grid[64] = {};

static cudaError_t mlp_setup(int device) {
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    if (!(g_mlp_attr.load() & (1ull << device))) {
        cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
        if (e != cudaSuccess) return e;
        g_mlp_attr.fetch_or(1ull << device);
    }
    if (!g_mlp_grid[device]) {
        int sms = 0;
        cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (e != cudaSuccess) return e;
        g_mlp_grid[device] = sms;
    }
    return cudaSuccess;
}

cudaError_t launch_mlp_train(int device, cudaStream_t st, const void* wb, const float4* samples, uint32_t n,
                             float* dW, float* loss) {
    cudaError_t e = mlp_setup(device);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    // 64 samples per block and step; as few blocks as keep the number of steps per block minimal
    uint32_t groups = (n + 63) / 64;
    const uint32_t sms = (uint32_t)g_mlp_grid[device];
    uint32_t per_block = (groups + sms - 1) / sms;
    uint32_t grid = (groups + per_block - 1) / per_block;
    k_mlp_train<<<grid, 128, kTrainSmem, st>>>((const __nv_bfloat16*)wb, samples, n, dW, loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(cudaStream_t st, float* wm, void* wb, const float* dW, float* m, float* v, float lr,
                            int step, float* ema, void* ema_b, float ema_decay, int ema_step) {
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
    float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
    float corr = ema_decay > 0.0f ? (float)(1.0 / (1.0 - std::pow((double)ema_decay, (double)ema_step))) : 1.0f;
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(wm, (__nv_bfloat16*)wb, dW, m, v, lr, b1, b2, eps, bc1, bc2,
                                                         ema, (__nv_bfloat16*)ema_b, ema_decay, corr);
    return cudaGetLastError();
}

}  // namespace bsm
