// mlp.cu — fused BF16 tensor-core kernels of the radiance cache.
//
// Per warp, a tile of 16 samples goes through the whole network with
// mma.sync.m16n8k16 (BF16 inputs, FP32 accumulation).  The accumulator
// fragment of two adjacent n8 tiles is exactly the A fragment of one k16 step
// of the next layer, so activations stay in registers from layer to layer
// (the fully fused scheme of Müller et al., "Real-time Neural Radiance
// Caching for Path Tracing", 2021).  Weights sit in shared memory with rows
// padded to 72 elements (conflict-free B-fragment loads).
//
//   k_mlp_infer   encode -> 5 layers -> radiance; adds throughput x max(y, 0)
//                 to the pixel accumulator of each cache query
//   k_mlp_predict same forward, writes y (tests, evaluation)
//   k_mlp_train   forward, relative-L2 loss gradient, backward through the
//                 layers, weight gradients dW_l = g_z^T a_{l-1} (also on the
//                 tensor cores, reduced in shared FP32, then one global atomic
//                 per weight per block)
//   k_mlp_adam    Adam on the FP32 master weights, BF16 copies for the next pass
//
// Plain mma.sync is the right instruction for 64-wide layers: a tcgen05 tile
// of 128 rows would leave most of the tensor memory and the pipeline idle at
// this width, and the whole frame's inference is ~69 GFLOP.
#include <cuda_bf16.h>
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

// Loads the BF16 weights (global, row-major [out][64]) into padded shared rows.
__device__ __forceinline__ void load_weights(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* sw) {
    const int rows = kMlpHidden * 64 + kMlpOutPad;
    for (int i = threadIdx.x; i < rows * 32; i += blockDim.x) {
        int r = i >> 5, c = (i & 31) * 2;
        *reinterpret_cast<uint32_t*>(sw + r * kLd + c) = *reinterpret_cast<const uint32_t*>(w + r * 64 + c);
    }
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
__device__ __forceinline__ void hidden_layer(const __nv_bfloat16* sw, const uint32_t (&in)[4][4], uint32_t (&out)[4][4],
                                             int g, int t) {
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const __nv_bfloat16* wr = sw + (8 * j + g) * kLd + 16 * kk + 2 * t;
            mma16816(acc[j], in[kk], *reinterpret_cast<const uint32_t*>(wr), *reinterpret_cast<const uint32_t*>(wr + 8));
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
__device__ __forceinline__ void output_layer(const __nv_bfloat16* sw4, const uint32_t (&in)[4][4], float (&y)[4],
                                             int g, int t) {
    y[0] = y[1] = y[2] = y[3] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        const __nv_bfloat16* wr = sw4 + g * kLd + 16 * kk + 2 * t;
        mma16816(y, in[kk], *reinterpret_cast<const uint32_t*>(wr), *reinterpret_cast<const uint32_t*>(wr + 8));
    }
}

__device__ __forceinline__ void forward(const __nv_bfloat16* sw, uint32_t (&act)[4][4], float (&y)[4], int g, int t) {
    uint32_t tmp[4][4];
    hidden_layer(sw + 0 * 64 * kLd, act, tmp, g, t);
    hidden_layer(sw + 1 * 64 * kLd, tmp, act, g, t);
    hidden_layer(sw + 2 * 64 * kLd, act, tmp, g, t);
    hidden_layer(sw + 3 * 64 * kLd, tmp, act, g, t);
    output_layer(sw + 4 * 64 * kLd, act, y, g, t);
}

// ------------------------------------------------------------- inference ----
// queries: 4 float4 per query: raw[0..3], raw[4..7], raw[8..11], (throughput rgb, accumulator index bits)
__global__ void __launch_bounds__(128) k_mlp_infer(const __nv_bfloat16* __restrict__ w, const float4* __restrict__ q,
                                                   const uint32_t* __restrict__ count, uint32_t capacity,
                                                   float4* accum) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    load_weights(w, sw);
    __syncthreads();
    const uint32_t n = min(*count, capacity);   // queries beyond the queue were dropped by the shade kernel
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < n; tile += warps) {
        uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
        float raw0[kMlpRaw], raw1[kMlpRaw];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float4 a = r0 < n ? q[4 * (size_t)r0 + k] : make_float4(0, 0, 0, 0);
            float4 b = r1 < n ? q[4 * (size_t)r1 + k] : make_float4(0, 0, 0, 0);
            raw0[4 * k] = a.x; raw0[4 * k + 1] = a.y; raw0[4 * k + 2] = a.z; raw0[4 * k + 3] = a.w;
            raw1[4 * k] = b.x; raw1[4 * k + 1] = b.y; raw1[4 * k + 2] = b.z; raw1[4 * k + 3] = b.w;
        }
        uint32_t act[4][4];
        encode_tile(raw0, raw1, act, t);
        float y[4];
        forward(sw, act, y, g, t);
        // lane t=0 holds channels 0,1 and gets channel 2 from lane t=1
        float y2a = __shfl_down_sync(0xffffffffu, y[0], 1);
        float y2b = __shfl_down_sync(0xffffffffu, y[2], 1);
        if (t == 0) {
            if (r0 < n) {
                float4 m = q[4 * (size_t)r0 + 3];
                float4 c = make_float4(m.x * fmaxf(y[0], 0.0f), m.y * fmaxf(y[1], 0.0f), m.z * fmaxf(y2a, 0.0f), 0.0f);
                atomicAdd(accum + __float_as_uint(m.w), c);
            }
            if (r1 < n) {
                float4 m = q[4 * (size_t)r1 + 3];
                float4 c = make_float4(m.x * fmaxf(y[2], 0.0f), m.y * fmaxf(y[3], 0.0f), m.z * fmaxf(y2b, 0.0f), 0.0f);
                atomicAdd(accum + __float_as_uint(m.w), c);
            }
        }
    }
}

// samples: 4 float4 per sample: raw[0..3], raw[4..7], raw[8..11], (target rgb, unused)
__global__ void __launch_bounds__(128) k_mlp_predict(const __nv_bfloat16* __restrict__ w,
                                                     const float4* __restrict__ s, uint32_t n, float* out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    load_weights(w, sw);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < n; tile += warps) {
        uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
        float raw0[kMlpRaw], raw1[kMlpRaw];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float4 a = r0 < n ? s[4 * (size_t)r0 + k] : make_float4(0, 0, 0, 0);
            float4 b = r1 < n ? s[4 * (size_t)r1 + k] : make_float4(0, 0, 0, 0);
            raw0[4 * k] = a.x; raw0[4 * k + 1] = a.y; raw0[4 * k + 2] = a.z; raw0[4 * k + 3] = a.w;
            raw1[4 * k] = b.x; raw1[4 * k + 1] = b.y; raw1[4 * k + 2] = b.z; raw1[4 * k + 3] = b.w;
        }
        uint32_t act[4][4];
        encode_tile(raw0, raw1, act, t);
        float y[4];
        forward(sw, act, y, g, t);
        int c0 = 2 * t;
        if (c0 < 3) {
            if (r0 < n) { out[3 * (size_t)r0 + c0] = y[0]; if (c0 + 1 < 3) out[3 * (size_t)r0 + c0 + 1] = y[1]; }
            if (r1 < n) { out[3 * (size_t)r1 + c0] = y[2]; if (c0 + 1 < 3) out[3 * (size_t)r1 + c0 + 1] = y[3]; }
        }
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

// g_a = g_z W for a [64 out][64 in] weight block (B[k=out][n=in] = W[out][in]).
__device__ __forceinline__ void backward_data(const __nv_bfloat16* sw, const uint32_t (&gz)[4][4], float (&ga)[8][4],
                                              int g, int t) {
    const uint16_t* w16 = reinterpret_cast<const uint16_t*>(sw);
#pragma unroll
    for (int j = 0; j < 8; ++j) ga[j][0] = ga[j][1] = ga[j][2] = ga[j][3] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            int k0 = 16 * kk + 2 * t, n = 8 * j + g;
            uint32_t b0 = pack_u16(w16[k0 * kLd + n], w16[(k0 + 1) * kLd + n]);
            uint32_t b1 = pack_u16(w16[(k0 + 8) * kLd + n], w16[(k0 + 9) * kLd + n]);
            mma16816(ga[j], gz[kk], b0, b1);
        }
}

// dW[out][in] += sum over the 16 samples of gz[s][out] * a[s][in]  (rows_out = 64 or 8)
__device__ __forceinline__ void weight_grad(const __nv_bfloat16* gz_tile, const __nv_bfloat16* a_tile, float* dW,
                                            int rows_out, int g, int t) {
    const uint16_t* gz16 = reinterpret_cast<const uint16_t*>(gz_tile);
    const uint16_t* a16 = reinterpret_cast<const uint16_t*>(a_tile);
    for (int m = 0; m < rows_out; m += 16) {
        uint32_t A[4];
        int o0 = m + g, o1 = m + g + 8, s0 = 2 * t;
        bool v1 = o1 < rows_out;
        A[0] = pack_u16(gz16[s0 * kLd + o0], gz16[(s0 + 1) * kLd + o0]);
        A[1] = v1 ? pack_u16(gz16[s0 * kLd + o1], gz16[(s0 + 1) * kLd + o1]) : 0u;
        A[2] = pack_u16(gz16[(s0 + 8) * kLd + o0], gz16[(s0 + 9) * kLd + o0]);
        A[3] = v1 ? pack_u16(gz16[(s0 + 8) * kLd + o1], gz16[(s0 + 9) * kLd + o1]) : 0u;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            int n = 8 * j + g;
            uint32_t b0 = pack_u16(a16[s0 * kLd + n], a16[(s0 + 1) * kLd + n]);
            uint32_t b1 = pack_u16(a16[(s0 + 8) * kLd + n], a16[(s0 + 9) * kLd + n]);
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            mma16816(c, A, b0, b1);
            int col = 8 * j + 2 * t;
            atomicAdd(dW + o0 * 64 + col, c[0]);
            atomicAdd(dW + o0 * 64 + col + 1, c[1]);
            if (v1) {
                atomicAdd(dW + o1 * 64 + col, c[2]);
                atomicAdd(dW + o1 * 64 + col + 1, c[3]);
            }
        }
    }
}

// samples: as k_mlp_predict (targets in the 4th float4).  Accumulates the
// gradient of the mean relative L2 loss over `n` samples into dW_global and
// the loss into loss_out[0].
__global__ void __launch_bounds__(128) k_mlp_train(const __nv_bfloat16* __restrict__ w, const float4* __restrict__ s,
                                                   uint32_t n, float* dW_global, float* loss_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    float* sdw = reinterpret_cast<float*>(smem_raw + kWSmem * 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __nv_bfloat16* wt = reinterpret_cast<__nv_bfloat16*>(smem_raw + kWSmem * 2 + kMlpParams * 4 + warp * kTrainWarpBytes);
    __nv_bfloat16* act_t[5];  // e, a0, a1, a2, a3
    __nv_bfloat16* gz_t[5];   // gz0, gz1, gz2, gz3, gy
    for (int i = 0; i < 5; ++i) { act_t[i] = wt + i * kTileElems; gz_t[i] = wt + (5 + i) * kTileElems; }
    load_weights(w, sw);
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) sdw[i] = 0.0f;
    __syncthreads();
    const float inv = 1.0f / (3.0f * (float)n);
    float loss = 0.0f;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + warp; tile * 16 < n; tile += warps) {
        uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
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
        // g_a3 = gy W4 (K = 8 padded to 16)
        float ga[8][4];
        uint32_t gz[4][4];
        {
            uint32_t A[4] = {gyp0, gyp1, 0u, 0u};
            const uint16_t* w16 = reinterpret_cast<const uint16_t*>(sw + 4 * 64 * kLd);
            for (int j = 0; j < 8; ++j) {
                ga[j][0] = ga[j][1] = ga[j][2] = ga[j][3] = 0.0f;
                int k0 = 2 * t, nn = 8 * j + g;
                uint32_t b0 = pack_u16(w16[k0 * kLd + nn], w16[(k0 + 1) * kLd + nn]);
                mma16816(ga[j], A, b0, 0u);
            }
        }
        __syncwarp();
        relu_grad(ga, act_t[4], gz_t[3], gz, g, t);   // gz3
        backward_data(sw + 3 * 64 * kLd, gz, ga, g, t);
        relu_grad(ga, act_t[3], gz_t[2], gz, g, t);   // gz2
        backward_data(sw + 2 * 64 * kLd, gz, ga, g, t);
        relu_grad(ga, act_t[2], gz_t[1], gz, g, t);   // gz1
        backward_data(sw + 1 * 64 * kLd, gz, ga, g, t);
        relu_grad(ga, act_t[1], gz_t[0], gz, g, t);   // gz0
        __syncwarp();
        // weight gradients: dW_l = gz_l^T a_{l-1}; dW4 = gy^T a3
        weight_grad(gz_t[0], act_t[0], sdw + 0 * kMlpLayerParams, 64, g, t);
        weight_grad(gz_t[1], act_t[1], sdw + 1 * kMlpLayerParams, 64, g, t);
        weight_grad(gz_t[2], act_t[2], sdw + 2 * kMlpLayerParams, 64, g, t);
        weight_grad(gz_t[3], act_t[3], sdw + 3 * kMlpLayerParams, 64, g, t);
        weight_grad(gz_t[4], act_t[4], sdw + 4 * kMlpLayerParams, kMlpOutPad, g, t);
        __syncwarp();
    }
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if (lane == 0) atomicAdd(loss_out, loss);
    __syncthreads();
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) {
        float v = sdw[i];
        if (v != 0.0f) atomicAdd(dW_global + i, v);
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
static int g_mlp_grid = 0;
static bool g_mlp_attr = false;

static cudaError_t mlp_setup(int device) {
    if (!g_mlp_attr) {
        cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
        if (e != cudaSuccess) return e;
        g_mlp_attr = true;
    }
    if (!g_mlp_grid) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        g_mlp_grid = sms;
    }
    return cudaSuccess;
}

cudaError_t launch_mlp_infer(int device, cudaStream_t st, const void* wb, const float4* queries, const uint32_t* count,
                             uint32_t capacity, float4* accum) {
    cudaError_t e = mlp_setup(device);
    if (e != cudaSuccess) return e;
    k_mlp_infer<<<g_mlp_grid * 4, 128, kWSmem * 2, st>>>((const __nv_bfloat16*)wb, queries, count, capacity, accum);
    return cudaGetLastError();
}

cudaError_t launch_mlp_predict(int device, cudaStream_t st, const void* wb, const float4* samples, uint32_t n,
                               float* out) {
    cudaError_t e = mlp_setup(device);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    k_mlp_predict<<<g_mlp_grid * 4, 128, kWSmem * 2, st>>>((const __nv_bfloat16*)wb, samples, n, out);
    return cudaGetLastError();
}

cudaError_t launch_mlp_train(int device, cudaStream_t st, const void* wb, const float4* samples, uint32_t n,
                             float* dW, float* loss) {
    cudaError_t e = mlp_setup(device);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    uint32_t tiles = (n + 15) / 16;
    uint32_t grid = (uint32_t)g_mlp_grid;
    if (tiles < grid * 4) grid = (tiles + 3) / 4;
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
