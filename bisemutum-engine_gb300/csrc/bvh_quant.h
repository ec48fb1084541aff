// bvh_quant.h — outward quantisation of one compressed-BVH node, shared by the
// host and the device TLAS refit.  Same rules as the host builder
// (bvh_build.cpp): per axis the smallest exponent e with 253 * 2^e >= the node
// extent, the frame origin one step below the node box, and every child box
// rounded outward by at least one step, each bound checked in double.
#pragma once
#include <math.h>
#include <stdint.h>

#include "bvh_layout.h"

#if defined(__CUDACC__)
#define BSM_QHD __host__ __device__ inline
#else
#define BSM_QHD static inline
#endif

namespace bsm {

BSM_QHD int quant_exponent_hd(float extent) {
    double ext = (double)extent > 1e-30 ? (double)extent : 1e-30;
    int e;
    frexp(ext / 253.0, &e);
    while (ldexp(253.0, e - 1) >= ext) --e;
    while (ldexp(253.0, e) < ext) ++e;
    int biased = e + 127;
    return biased < 1 ? 1 : (biased > 254 ? 254 : biased);
}

// Rewrites the frame (px..pz, ex..ez) and the child bytes of node `n` for the
// child boxes of the slots in `used`; returns the node box.  Topology fields
// (imask, tri_mask, child_base, tri_base) are kept.
BSM_QHD void tlas_quantise(CwNode& n, const float lo[8][3], const float hi[8][3], uint32_t used, float nlo[3],
                           float nhi[3]) {
    for (int k = 0; k < 3; ++k) { nlo[k] = INFINITY; nhi[k] = -INFINITY; }
    for (int s = 0; s < 8; ++s) {
        if (!(used & (1u << s))) continue;
        for (int k = 0; k < 3; ++k) {
            nlo[k] = fminf(nlo[k], lo[s][k]);
            nhi[k] = fmaxf(nhi[k], hi[s][k]);
        }
    }
    float org[3];
    int e[3];
    for (int k = 0; k < 3; ++k) {
        e[k] = quant_exponent_hd(nhi[k] - nlo[k]);
        double step = ldexp(1.0, e[k] - 127);
        float o = (float)((double)nlo[k] - step);
        while ((double)o > (double)nlo[k] - step) o = nextafterf(o, -INFINITY);
        org[k] = o;
    }
    n.px = org[0]; n.py = org[1]; n.pz = org[2];
    n.ex = (uint8_t)e[0]; n.ey = (uint8_t)e[1]; n.ez = (uint8_t)e[2];
    uint8_t* qlo[3] = {n.qlo_x, n.qlo_y, n.qlo_z};
    uint8_t* qhi[3] = {n.qhi_x, n.qhi_y, n.qhi_z};
    for (int s = 0; s < 8; ++s) {
        if (!(used & (1u << s))) continue;
        for (int k = 0; k < 3; ++k) {
            double sc = ldexp(1.0, e[k] - 127);
            double l = floor(((double)lo[s][k] - org[k]) / sc) - 1.0;
            double h = ceil(((double)hi[s][k] - org[k]) / sc) + 1.0;
            l = l < 0.0 ? 0.0 : (l > 255.0 ? 255.0 : l);
            h = h < 0.0 ? 0.0 : (h > 255.0 ? 255.0 : h);
            while (l > 0.0 && (double)org[k] + l * sc > (double)lo[s][k]) l -= 1.0;
            while (h < 255.0 && (double)org[k] + h * sc < (double)hi[s][k]) h += 1.0;
            qlo[k][s] = (uint8_t)l;
            qhi[k][s] = (uint8_t)h;
        }
    }
}

}  // namespace bsm
