// df.cuh — FP64-class arithmetic on the FP32 pipe ("double-float").
//
// This GB300 executes 1.06 TFLOP/s of FP64 FMA against 71.6 TFLOP/s of FP32
// FMA, so any FP64 instruction per amplitude caps a complex128 kernel at
// 0.53 T FP64 instructions/s, well below HBM bandwidth.  These helpers carry
// a value as an unevaluated sum hi + lo of two floats and use error-free
// transformations on the FP32 pipe: the exact product a*b = p + e with
// e = fma(a, b, -p) (Dekker/Kahan via FMA) and Knuth's two-sum for exact
// addition.  Relative error per operation is about 2^-45 (lo terms below
// 2^-48 are dropped), far inside the 1e-12 state tolerance of complex128.
//
// Conversions avoid the FP64 pipe: a double is split into hi (its top 24
// significant bits, truncated) and lo (the next 23 bits) with integer
// operations and one exact FP32 subtraction; a hi/lo pair becomes a double by
// assembling each float's double encoding with integer operations (the low
// part scaled by 2^24 first, exactly) and one FP64 add.  Values below about
// 2^-103 in magnitude lose their lo part, values below 2^-126 become zero;
// non-finite values are not supported on this path (the native-FP64 kernels
// handle them).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace plk {

struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF df_split(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned hw = (unsigned)(u >> 32), lw = (unsigned)u;
    const unsigned sign = hw & 0x80000000u;
    const int e = (int)((hw >> 20) & 0x7ffu); // biased binary exponent of x
    const int ef = e - 896;                    // same exponent, float bias
    const unsigned m_top = ((hw & 0xfffffu) << 3) | (lw >> 29); // mantissa bits 51..29
    const unsigned m_next = (lw >> 6) & 0x7fffffu;              // mantissa bits 28..6
    DF r;
    r.hi = (ef >= 1 && ef <= 254) ? __uint_as_float(sign | ((unsigned)ef << 23) | m_top) : 0.0f;
    const int el = ef - 23; // float exponent of the unit in the last place of hi
    if (el >= 1 && el <= 254) {
        // (1 + m_next/2^23) 2^E - 2^E = m_next 2^(E-23): exact in FP32
        const float F = __uint_as_float(((unsigned)el << 23) | m_next);
        const float G = __uint_as_float((unsigned)el << 23);
        r.lo = __uint_as_float(__float_as_uint(__fsub_rn(F, G)) | sign);
    } else {
        r.lo = 0.0f;
    }
    return r;
}

// The double with the value f * 2^-k of a normal float f (zero and denormal
// floats give 0), assembled with integer operations: no FP64-pipe conversion.
__device__ __forceinline__ double df_f2d(float f, unsigned k = 0) {
    const unsigned b = __float_as_uint(f);
    const unsigned ef = (b >> 23) & 0xffu;
    if (ef == 0) return 0.0;
    const unsigned m = b & 0x7fffffu;
    const unsigned hw = (b & 0x80000000u) | ((ef + 896u - k) << 20) | (m >> 3);
    return __hiloint2double((int)hw, (int)(m << 29));
}

// hi + lo as a double.  The low part is scaled by 2^24 first (exact: it is
// at most about an ulp of hi, so the product stays finite, and a denormal
// low part becomes a normal float), then assembled with its exponent
// lowered by 24: small amplitudes keep their relative accuracy without a
// branch.
__device__ __forceinline__ double df_join(float hi, float lo) {
    return __dadd_rn(df_f2d(hi), df_f2d(__fmul_rn(lo, 16777216.0f), 24u));
}

// (sh, sl) += a * b with a = ah + al, b = bh + bl; the accumulator is kept
// unnormalised (sl collects the rounding errors).
__device__ __forceinline__ void df_mac(float ah, float al, float bh, float bl, float &sh, float &sl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(t, e));
}

// (sh, sl) += a with a = ah + al
__device__ __forceinline__ void df_add(float ah, float al, float &sh, float &sl) {
    const float s = __fadd_rn(sh, ah);
    const float bb = __fsub_rn(s, sh);
    const float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(ah, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(t, al));
}

__device__ __forceinline__ double df_result(float sh, float sl) {
    const float s = __fadd_rn(sh, sl);
    const float l = __fsub_rn(sl, __fsub_rn(s, sh));
    return df_join(s, l);
}

// Host-side split of a coefficient (exact hi, rounded lo).
inline void df_split_host(double x, float &hi, float &lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

// ---- two lanes per instruction --------------------------------------------
// PTX .f32x2 arithmetic (sm_100 and later) runs two independent FP32
// operations in one instruction; each lane is rounded exactly as the scalar
// instruction.  A complex double-float accumulator is carried as two packed
// pairs, (re.hi, im.hi) and (re.lo, im.lo), so the real and imaginary
// chains of a complex multiply-add share instructions.  Lane 0 is the low
// 32 bits (the first float of mov.b64 {a, b}).
typedef unsigned long long f2x;

__device__ __forceinline__ f2x f2x_pack(float a, float b) {
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2x_unpack(f2x v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
// (b, a) from (a, b)
__device__ __forceinline__ f2x f2x_swap(f2x v) {
    float a, b;
    f2x_unpack(v, a, b);
    return f2x_pack(b, a);
}
__device__ __forceinline__ f2x f2x_add(f2x a, f2x b) {
    f2x r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2x_sub(f2x a, f2x b) {
    f2x r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2x_mul(f2x a, f2x b) {
    f2x r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2x_fma(f2x a, f2x b, f2x c) {
    f2x r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Packed df_mac: (sh, sl) += a * b in both lanes, a given as ah and the
// negated pair (nah, nal) = -(ah, al).  The error chain is carried negated,
// en = -e (round-to-nearest is symmetric, so en is exactly the negative of
// df_mac's e at every step, up to the sign of a zero), which needs no
// negation instructions; each lane's result is df_mac's bit for bit (a zero
// may differ in sign).
__device__ __forceinline__ void df_mac2(f2x ah, f2x nah, f2x nal, f2x bh, f2x bl, f2x &sh, f2x &sl) {
    const f2x p = f2x_mul(ah, bh);
    f2x en = f2x_fma(nah, bh, p);
    en = f2x_fma(nah, bl, en);
    en = f2x_fma(nal, bh, en);
    const f2x s = f2x_add(sh, p);
    const f2x bb = f2x_sub(s, sh);
    const f2x t = f2x_add(f2x_sub(sh, f2x_sub(s, bb)), f2x_sub(p, bb));
    sh = s;
    sl = f2x_add(sl, f2x_sub(t, en));
}

// Packed df_first: (sh, sl) = a * b (the low part as 0 - en: a zero low
// part may differ from df_first's in sign only)
__device__ __forceinline__ void df_first2(f2x ah, f2x nah, f2x nal, f2x bh, f2x bl, f2x &sh, f2x &sl) {
    sh = f2x_mul(ah, bh);
    f2x en = f2x_fma(nah, bh, sh);
    en = f2x_fma(nah, bl, en);
    en = f2x_fma(nal, bh, en);
    sl = f2x_sub(0ull, en);
}

// df_mac2 / df_first2 with the negation on the other factor: b given as bh
// and (nbh, nbl) = -(bh, bl), for a data-dependent a reused against
// several b (the same operations lane by lane: fma(a, -b, p) = fma(-a, b, p)).
__device__ __forceinline__ void df_mac2n(f2x ah, f2x al, f2x bh, f2x nbh, f2x nbl, f2x &sh, f2x &sl) {
    const f2x p = f2x_mul(ah, bh);
    f2x en = f2x_fma(ah, nbh, p);
    en = f2x_fma(ah, nbl, en);
    en = f2x_fma(al, nbh, en);
    const f2x s = f2x_add(sh, p);
    const f2x bb = f2x_sub(s, sh);
    const f2x t = f2x_add(f2x_sub(sh, f2x_sub(s, bb)), f2x_sub(p, bb));
    sh = s;
    sl = f2x_add(sl, f2x_sub(t, en));
}
__device__ __forceinline__ void df_first2n(f2x ah, f2x al, f2x bh, f2x nbh, f2x nbl, f2x &sh, f2x &sl) {
    sh = f2x_mul(ah, bh);
    f2x en = f2x_fma(ah, nbh, sh);
    en = f2x_fma(ah, nbl, en);
    en = f2x_fma(al, nbh, en);
    sl = f2x_sub(0ull, en);
}

// Complex double-float amplitude
struct CDF {
    DF re, im;
};

__device__ __forceinline__ CDF cdf_split(double2 v) { return {df_split(v.x), df_split(v.y)}; }
__device__ __forceinline__ CDF to_cdf(double2 v) { return cdf_split(v); }
__device__ __forceinline__ CDF to_cdf(float2 v) { return {{v.x, 0.0f}, {v.y, 0.0f}}; }

// (sh, sl) = a * b (first term of a sum)
__device__ __forceinline__ void df_first(float ah, float al, float bh, float bl, float &sh, float &sl) {
    sh = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -sh);
    e = __fmaf_rn(ah, bl, e);
    sl = __fmaf_rn(al, bh, e);
}

// Per-thread FP64-class accumulator on the FP32 pipe; converted to a double
// once, at the end of the thread's loop, for the FP64 block reduction.
struct DAcc {
    float h = 0.0f, l = 0.0f;
    __device__ __forceinline__ void mac(const DF &a, const DF &b) { df_mac(a.hi, a.lo, b.hi, b.lo, h, l); }
    __device__ __forceinline__ void msub(const DF &a, const DF &b) { df_mac(-a.hi, -a.lo, b.hi, b.lo, h, l); }
    __device__ __forceinline__ void add(const DF &a) { df_add(a.hi, a.lo, h, l); }
    __device__ __forceinline__ void sub(const DF &a) { df_add(-a.hi, -a.lo, h, l); }
    __device__ __forceinline__ double value() const { return df_result(h, l); }
    __device__ __forceinline__ DF normalized() const {
        const float s = __fadd_rn(h, l);
        return {s, __fsub_rn(l, __fsub_rn(s, h))};
    }
};

// |a|^2 as a double-float
__device__ __forceinline__ DF df_norm2(const CDF &a) {
    float h, l;
    df_first(a.re.hi, a.re.lo, a.re.hi, a.re.lo, h, l);
    df_mac(a.im.hi, a.im.lo, a.im.hi, a.im.lo, h, l);
    return {h, l};
}

} // namespace plk
