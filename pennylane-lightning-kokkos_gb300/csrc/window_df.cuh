// window_df.cuh — double-float building blocks of the complex128 register
// windows (window_dfs.cuh).
//
// Every amplitude is held as a double-float pair per component (CDF: re.hi +
// re.lo, im.hi + im.lo); each op's products are error-free FP32 products
// accumulated with two-sum (df.cuh), about 2^-45 relative error per op.
// Matrices arrive split on the host as float4 {re.hi, re.lo, im.hi, im.lo}.
// Generator inner products accumulate in double-float (DAcc).
#pragma once

#include "batch_engine.cuh"

namespace plk {

// (rh, rl, ih, il) += m * v, complex
__device__ __forceinline__ void cdf_mac(const float4 m, const CDF &v, float &rh, float &rl, float &ih, float &il) {
    df_mac(m.x, m.y, v.re.hi, v.re.lo, rh, rl);
    df_mac(-m.z, -m.w, v.im.hi, v.im.lo, rh, rl);
    df_mac(m.x, m.y, v.im.hi, v.im.lo, ih, il);
    df_mac(m.z, m.w, v.re.hi, v.re.lo, ih, il);
}

// An op's outputs are formed afresh from error-free products: hi is the
// rounded sum of the hi products and lo collects this op's rounding errors,
// so |lo| stays within a few ulps of hi without renormalising, and the next
// op's products (which take hi and lo as separate operands) lose nothing.
// Ops therefore return their (hi, lo) pairs as they are.

__device__ __forceinline__ CDF cdf_mul(const float4 e, const CDF &v) {
    float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
    df_first(e.x, e.y, v.re.hi, v.re.lo, rh, rl);
    df_mac(-e.z, -e.w, v.im.hi, v.im.lo, rh, rl);
    df_first(e.x, e.y, v.im.hi, v.im.lo, ih, il);
    df_mac(e.z, e.w, v.re.hi, v.re.lo, ih, il);
    return {{rh, rl}, {ih, il}};
}

// a * x + b * y for real double-floats a, b
__device__ __forceinline__ DF df_lin2(const DF &a, const DF &x, const DF &b, const DF &y) {
    float h, l;
    df_first(a.hi, a.lo, x.hi, x.lo, h, l);
    df_mac(b.hi, b.lo, y.hi, y.lo, h, l);
    return {h, l};
}

__device__ __forceinline__ DF df_neg(const DF &a) { return {-a.hi, -a.lo}; }

// acc += Im(conj(h) * i^q * x) (q in 0..3)
__device__ __forceinline__ void im_dot_phase_df(DAcc &acc, const CDF &h, const CDF &x, uint32_t q) {
    // q even: +-(h.re x.im - h.im x.re); q odd: +-(h.re x.re + h.im x.im)
    const bool neg = q >= 2;
    if (q & 1u) {
        if (neg) {
            acc.msub(h.re, x.re);
            acc.msub(h.im, x.im);
        } else {
            acc.mac(h.re, x.re);
            acc.mac(h.im, x.im);
        }
    } else {
        if (neg) {
            acc.msub(h.re, x.im);
            acc.mac(h.im, x.re);
        } else {
            acc.mac(h.re, x.im);
            acc.msub(h.im, x.re);
        }
    }
}

// generator entries are 0, +-1, +-i: the phase code of an entry (-1: zero)
__device__ __forceinline__ int gen_code(const float4 e) {
    if (e.x == 1.0f) return 0;
    if (e.z == 1.0f) return 1;
    if (e.x == -1.0f) return 2;
    if (e.z == -1.0f) return 3;
    return -1;
}

} // namespace plk
