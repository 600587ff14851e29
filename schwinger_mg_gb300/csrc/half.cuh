// FP16 fine-field storage with one FP32 scale per site.
//
// An F16 field stores, for every site q, the nrhs two-spinors of its
// right-hand sides as __half2 pairs (re, im) in the layout of the FP32 field,
// [q][rhs][spin], divided by the site's scale: the largest |re| or |im| over
// all right-hand sides and spins of that site ("per-site block scaling").
// Values are in [-1, 1], so FP16's 11-bit mantissa holds every component to
// about 5e-4 of the site's largest one; all arithmetic is FP32.
//
// Writers need the site maximum over the right-hand sides before they can
// store: the kernels that write F16 fields give each site one group of
// `lanes` = nrhs threads of a warp (nrhs a power of two <= 32) and reduce the
// maximum with shuffles inside the group.
#pragma once
#include <cuda_fp16.h>

#include "smg_internal.h"

struct alignas(8) Spinor16 {
    __half2 s0, s1;
};

__device__ __forceinline__ Spinor<float> ld_spinor_h(const __half2* __restrict__ f, const float* __restrict__ scale,
                                                      int64_t q, int rhs, int nrhs) {
    const Spinor16 h = reinterpret_cast<const Spinor16*>(f)[q * nrhs + rhs];
    const float s = scale[q];
    const float2 a = __half22float2(h.s0), b = __half22float2(h.s1);
    Spinor<float> o;
    o.s0 = mk(a.x * s, a.y * s);
    o.s1 = mk(b.x * s, b.y * s);
    return o;
}

// The stored values of one two-spinor without the site scale (the caller folds the scale into a
// factor it multiplies by anyway)
__device__ __forceinline__ Spinor<float> ld_spinor_h_raw(const __half2* __restrict__ f, int64_t q, int rhs, int nrhs) {
    const Spinor16 h = reinterpret_cast<const Spinor16*>(f)[q * nrhs + rhs];
    const float2 a = __half22float2(h.s0), b = __half22float2(h.s1);
    Spinor<float> o;
    o.s0 = mk(a.x, a.y);
    o.s1 = mk(b.x, b.y);
    return o;
}

// Stores one two-spinor per thread.  The `lanes` threads of a site group (consecutive lanes of one
// warp with blockDim.x == lanes) cooperate on the site's scale; every thread of the warp must call
// this (the shuffles span the warp), and `valid` (uniform within a group) says whether to store.
__device__ __forceinline__ void st_spinor_h(__half2* __restrict__ f, float* __restrict__ scale, int64_t q, int rhs,
                                            int nrhs, int lanes, Spinor<float> v, bool valid) {
    float m = valid ? fmaxf(fmaxf(fabsf(v.s0.re), fabsf(v.s0.im)), fmaxf(fabsf(v.s1.re), fabsf(v.s1.im))) : 0.f;
    for (int o = lanes >> 1; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o, lanes));
    if (!valid) return;
    const float inv = m > 0.f ? __fdividef(1.0f, m) : 0.f;  // fast reciprocal: FP16 rounding dominates
    Spinor16 h;
    h.s0 = __floats2half2_rn(v.s0.re * inv, v.s0.im * inv);
    h.s1 = __floats2half2_rn(v.s1.re * inv, v.s1.im * inv);
    reinterpret_cast<Spinor16*>(f)[q * nrhs + rhs] = h;
    if ((threadIdx.x & (lanes - 1)) == 0) scale[q] = m;
}

// Largest of the warp's non-negative floats v in one redux.sync (the IEEE bit patterns of non-negative
// floats order as unsigned integers); a NaN among them gives NaN.
__device__ __forceinline__ float warp_max_nonneg(float v) {
    return __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(v)));
}

// Two spinors per thread (right-hand sides rhs and rhs + lanes of one site), same contract as above.
__device__ __forceinline__ void st_spinor2_h(__half2* __restrict__ f, float* __restrict__ scale, int64_t q, int rhs,
                                             int nrhs, int lanes, Spinor<float> v, Spinor<float> w, bool valid) {
    float m = 0.f;
    if (valid) {
        m = fmaxf(fmaxf(fabsf(v.s0.re), fabsf(v.s0.im)), fmaxf(fabsf(v.s1.re), fabsf(v.s1.im)));
        m = fmaxf(m, fmaxf(fmaxf(fabsf(w.s0.re), fabsf(w.s0.im)), fmaxf(fabsf(w.s1.re), fabsf(w.s1.im))));
    }
    for (int o = lanes >> 1; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o, lanes));
    if (!valid) return;
    const float inv = m > 0.f ? __fdividef(1.0f, m) : 0.f;  // fast reciprocal: FP16 rounding dominates
    Spinor16 h;
    h.s0 = __floats2half2_rn(v.s0.re * inv, v.s0.im * inv);
    h.s1 = __floats2half2_rn(v.s1.re * inv, v.s1.im * inv);
    reinterpret_cast<Spinor16*>(f)[q * nrhs + rhs] = h;
    h.s0 = __floats2half2_rn(w.s0.re * inv, w.s0.im * inv);
    h.s1 = __floats2half2_rn(w.s1.re * inv, w.s1.im * inv);
    reinterpret_cast<Spinor16*>(f)[q * nrhs + rhs + lanes] = h;
    if ((threadIdx.x & (lanes - 1)) == 0) scale[q] = m;
}

// NR spinors per thread (right-hand sides rhs + k * lanes, k < NR), same contract as above.
template <int NR>
__device__ __forceinline__ void st_spinorN_h(__half2* __restrict__ f, float* __restrict__ scale, int64_t q, int rhs,
                                             int nrhs, int lanes, const Spinor<float> (&v)[NR], bool valid) {
    float m = 0.f;
    if (valid) {
#pragma unroll
        for (int k = 0; k < NR; ++k)
            m = fmaxf(m, fmaxf(fmaxf(fabsf(v[k].s0.re), fabsf(v[k].s0.im)), fmaxf(fabsf(v[k].s1.re), fabsf(v[k].s1.im))));
    }
    for (int o = lanes >> 1; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o, lanes));
    if (!valid) return;
    const float inv = m > 0.f ? __fdividef(1.0f, m) : 0.f;  // fast reciprocal: FP16 rounding dominates
#pragma unroll
    for (int k = 0; k < NR; ++k) {
        Spinor16 h;
        h.s0 = __floats2half2_rn(v[k].s0.re * inv, v[k].s0.im * inv);
        h.s1 = __floats2half2_rn(v[k].s1.re * inv, v[k].s1.im * inv);
        reinterpret_cast<Spinor16*>(f)[q * nrhs + rhs + k * lanes] = h;
    }
    if ((threadIdx.x & (lanes - 1)) == 0) scale[q] = m;
}

// ---- pairs of adjacent right-hand sides: one 16-byte access per pair (2 two-spinors) and site.
// 2 NP two-spinors of right-hand sides rhs0 .. rhs0 + 2 NP - 1 of site q
template <int NP>
__device__ __forceinline__ void ld_pairs_h(const __half2* __restrict__ f, int64_t q, int rhs0, int nrhs,
                                           Spinor<float> (&o)[2 * NP]) {
    const uint4* p = reinterpret_cast<const uint4*>(f) + ((q * nrhs + rhs0) >> 1);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const uint4 v = __ldg(p + k);
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
        const float2 c = __half22float2(*reinterpret_cast<const __half2*>(&v.z));
        const float2 d = __half22float2(*reinterpret_cast<const __half2*>(&v.w));
        o[2 * k].s0 = mk(a.x, a.y);
        o[2 * k].s1 = mk(b.x, b.y);
        o[2 * k + 1].s0 = mk(c.x, c.y);
        o[2 * k + 1].s1 = mk(d.x, d.y);
    }
}

template <int NP>
__device__ __forceinline__ void ld_pairs_f(const cx<float>* __restrict__ f, int64_t q, int rhs0, int nrhs,
                                           Spinor<float> (&o)[2 * NP]) {
    const float4* p = reinterpret_cast<const float4*>(f) + (q * nrhs + rhs0);
#pragma unroll
    for (int k = 0; k < 2 * NP; ++k) {
        const float4 v = __ldg(p + k);
        o[k].s0 = mk(v.x, v.y);
        o[k].s1 = mk(v.z, v.w);
    }
}

__device__ __forceinline__ unsigned pack_h2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const unsigned*>(&h);
}

// Stores 2 NP two-spinors of one site as FP16 with the site's scale (largest |re| or |im| over all
// its right-hand sides, reduced over the site's `lanes` threads); every thread of the warp calls it.
template <int NP>
__device__ __forceinline__ void st_pairs_h(__half2* __restrict__ f, float* __restrict__ scale, int64_t q, int rhs0,
                                           int nrhs, int lanes, const Spinor<float> (&v)[2 * NP], bool valid) {
    float m = 0.f;
    if (valid) {
#pragma unroll
        for (int k = 0; k < 2 * NP; ++k)
            m = fmaxf(m, fmaxf(fmaxf(fabsf(v[k].s0.re), fabsf(v[k].s0.im)), fmaxf(fabsf(v[k].s1.re), fabsf(v[k].s1.im))));
    }
    for (int o = lanes >> 1; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o, lanes));
    if (!valid) return;
    const float inv = m > 0.f ? __fdividef(1.0f, m) : 0.f;  // fast reciprocal: FP16 rounding dominates
    uint4* p = reinterpret_cast<uint4*>(f) + ((q * nrhs + rhs0) >> 1);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const Spinor<float>& a = v[2 * k];
        const Spinor<float>& b = v[2 * k + 1];
        uint4 h;
        h.x = pack_h2(a.s0.re * inv, a.s0.im * inv);
        h.y = pack_h2(a.s1.re * inv, a.s1.im * inv);
        h.z = pack_h2(b.s0.re * inv, b.s0.im * inv);
        h.w = pack_h2(b.s1.re * inv, b.s1.im * inv);
        p[k] = h;
    }
    if ((threadIdx.x & (lanes - 1)) == 0) scale[q] = m;
}

// nrhs values whose sites can be written as F16 (one site per power-of-two lane group)
inline bool f16_nrhs_ok(int nrhs) { return nrhs >= 1 && nrhs <= 32 && (nrhs & (nrhs - 1)) == 0; }
