// xprec.cuh -- double-FP32 ("ff") arithmetic: a value carried as an unevaluated
// sum hi + lo of two floats, with error-free products (fmaf) and compensated
// sums (Knuth two-sum).  About 48 significant bits at FP32 speed; used for
// the residuals of iterative refinement, where the device's FP64 rate (1/74
// of FP32) would dominate.
#pragma once
#include "common.cuh"

namespace gbla {

struct ff {
    float h, l;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// acc += a * (xh + xl) with an error-free product of a * xh
__device__ __forceinline__ void ff_fma(ff &acc, float a, float xh, float xl) {
    float p = a * xh;
    float pe = fmaf(a, xh, -p);
    float s, e;
    two_sum(acc.h, p, s, e);
    acc.h = s;
    acc.l += e + pe;
    acc.l = fmaf(a, xl, acc.l);
}

__device__ __forceinline__ void ff_add(ff &acc, float xh, float xl) {
    float s, e;
    two_sum(acc.h, xh, s, e);
    acc.h = s;
    acc.l += e + xl;
}

__device__ __forceinline__ ff ff_norm(ff a) {
    float s = a.h + a.l;
    float e = a.l - (s - a.h);
    return {s, e};
}

__device__ __forceinline__ ff ff_warp_sum(ff a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        float oh = shfl_xor(a.h, o), ol = shfl_xor(a.l, o);
        float s, e;
        two_sum(a.h, oh, s, e);
        a.h = s;
        a.l += ol + e;
    }
    return ff_norm(a);
}

}  // namespace gbla
