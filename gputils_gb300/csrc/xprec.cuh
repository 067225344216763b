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

// Reduce-scatter of 8 double-FP32 slots across the warp (9 exchanges instead
// of 8 full butterflies): on return every lane holds the warp-wide total of
// slot (lane >> 2) & 7, i.e. lanes 4 s .. 4 s + 3 hold slot s.
__device__ __forceinline__ ff ff_reduce_scatter8(const ff (&p)[8], int lane) {
    ff q[4];
    const bool b4 = lane & 16;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const ff mine = b4 ? p[i + 4] : p[i], other = b4 ? p[i] : p[i + 4];
        q[i] = mine;
        ff_add(q[i], shfl_xor(other.h, 16), shfl_xor(other.l, 16));
    }
    const bool b3 = lane & 8;
    ff r[2];
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const ff mine = b3 ? q[i + 2] : q[i], other = b3 ? q[i] : q[i + 2];
        r[i] = mine;
        ff_add(r[i], shfl_xor(other.h, 8), shfl_xor(other.l, 8));
    }
    const bool b2 = lane & 4;
    ff s = b2 ? r[1] : r[0];
    {
        const ff other = b2 ? r[0] : r[1];
        ff_add(s, shfl_xor(other.h, 4), shfl_xor(other.l, 4));
    }
#pragma unroll
    for (int o = 2; o > 0; o >>= 1) {
        const float oh = shfl_xor(s.h, o), ol = shfl_xor(s.l, o);
        ff_add(s, oh, ol);
    }
    return ff_norm(s);
}

}  // namespace gbla
