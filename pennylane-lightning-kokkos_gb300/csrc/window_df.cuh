// window_df.cuh — register-window ops for complex128 states on the FP32 pipe.
//
// The same op kinds as window_op in batch_engine.cuh, with every amplitude
// held as a double-float pair per component (CDF: re.hi + re.lo, im.hi +
// im.lo) for the whole window: a double2 is split once when it is loaded and
// joined once when it is stored, and each op's products are error-free FP32
// products accumulated with two-sum (df.cuh), about 2^-45 relative error per
// op.  Matrices arrive split on the host as float4 {re.hi, re.lo, im.hi,
// im.lo}.  Generator inner products accumulate in double-float (DAcc).
#pragma once

#include "batch_engine.cuh"

namespace plk {

__device__ __forceinline__ CDF cdf_zero() { return {{0.0f, 0.0f}, {0.0f, 0.0f}}; }

// (rh, rl, ih, il) += m * v, complex
__device__ __forceinline__ void cdf_mac(const float4 m, const CDF &v, float &rh, float &rl, float &ih, float &il) {
    df_mac(m.x, m.y, v.re.hi, v.re.lo, rh, rl);
    df_mac(-m.z, -m.w, v.im.hi, v.im.lo, rh, rl);
    df_mac(m.x, m.y, v.im.hi, v.im.lo, ih, il);
    df_mac(m.z, m.w, v.re.hi, v.re.lo, ih, il);
}

__device__ __forceinline__ DF df_norm(float h, float l) {
    const float s = __fadd_rn(h, l);
    return {s, __fsub_rn(l, __fsub_rn(s, h))};
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

// dense U (canonical D x D) on the register bits of (K, SEL)
template <int K, int SEL> __device__ __forceinline__ void dense_apply_df(CDF (&v)[kWinAmps], const float4 *__restrict__ U) {
    constexpr int D = 1 << K;
    constexpr int M = selmask<K, SEL>();
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & M) continue;
        CDF in[D];
#pragma unroll
        for (int m = 0; m < D; m++) in[m] = v[j | spread<K, SEL>(m)];
#pragma unroll
        for (int r = 0; r < D; r++) {
            float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
#pragma unroll
            for (int c = 0; c < D; c++) cdf_mac(U[r * D + c], in[c], rh, rl, ih, il);
            v[j | spread<K, SEL>(r)] = {{rh, rl}, {ih, il}};
        }
    }
}

// RX form [[c, i w], [i w, c]] and RY form [[c, -s], [s, c]] (real c, w, s)
template <int Q> __device__ __forceinline__ void rx_apply_df(CDF (&v)[kWinAmps], const float4 *__restrict__ U) {
    const DF c = {U[0].x, U[0].y}, w = {U[1].z, U[1].w};
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & (1 << Q)) continue;
        const CDF x = v[j], y = v[j | (1 << Q)];
        v[j] = {df_lin2(c, x.re, df_neg(w), y.im), df_lin2(c, x.im, w, y.re)};
        v[j | (1 << Q)] = {df_lin2(c, y.re, df_neg(w), x.im), df_lin2(c, y.im, w, x.re)};
    }
}
template <int Q> __device__ __forceinline__ void ry_apply_df(CDF (&v)[kWinAmps], const float4 *__restrict__ U) {
    const DF c = {U[0].x, U[0].y}, s = {U[2].x, U[2].y};
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & (1 << Q)) continue;
        const CDF x = v[j], y = v[j | (1 << Q)];
        v[j] = {df_lin2(c, x.re, df_neg(s), y.re), df_lin2(c, x.im, df_neg(s), y.im)};
        v[j | (1 << Q)] = {df_lin2(s, x.re, c, y.re), df_lin2(s, x.im, c, y.im)};
    }
}

// acc += Im <h | G v>: RX generator (Pauli X) or RY generator (Pauli Y)
template <int Q, bool ISY>
__device__ __forceinline__ void gen1_fixed_df(const CDF (&v)[kWinAmps], const CDF (&h)[kWinAmps], DAcc &a0, DAcc &a1) {
    int g = 0;
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & (1 << Q)) continue;
        DAcc &acc = (g++ & 1) ? a1 : a0;
        const CDF v0 = v[j], v1 = v[j | (1 << Q)], h0 = h[j], h1 = h[j | (1 << Q)];
        if (ISY) { // -Re(conj(h0) v1) + Re(conj(h1) v0)
            acc.msub(h0.re, v1.re);
            acc.msub(h0.im, v1.im);
            acc.mac(h1.re, v0.re);
            acc.mac(h1.im, v0.im);
        } else { // Im(conj(h0) v1) + Im(conj(h1) v0)
            acc.mac(h0.re, v1.im);
            acc.msub(h0.im, v1.re);
            acc.mac(h1.re, v0.im);
            acc.msub(h1.im, v0.re);
        }
    }
}

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

// one-wire generator given as a monomial pattern (EOp::bits)
template <int Q>
__device__ __forceinline__ void gen1_pattern_df(const CDF (&v)[kWinAmps], const CDF (&h)[kWinAmps], uint32_t pat,
                                                DAcc &a0, DAcc &a1) {
    int g = 0;
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & (1 << Q)) continue;
        DAcc &acc = (g++ & 1) ? a1 : a0;
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const uint32_t rp = (pat >> (4 * r)) & 15u;
            if (!(rp & 1u)) continue;
            const CDF x = (rp & 2u) ? v[j | (1 << Q)] : v[j];
            im_dot_phase_df(acc, h[j | (r << Q)], x, rp >> 2);
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

// acc += Im <h | G v> for a dense generator on the register bits of (K, SEL)
template <int K, int SEL>
__device__ __forceinline__ void dense_gen_dot_df(const CDF (&v)[kWinAmps], const CDF (&h)[kWinAmps],
                                                 const float4 *__restrict__ G, DAcc &acc) {
    constexpr int D = 1 << K;
    constexpr int M = selmask<K, SEL>();
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & M) continue;
#pragma unroll
        for (int r = 0; r < D; r++) {
#pragma unroll
            for (int c = 0; c < D; c++) {
                const int q = gen_code(G[r * D + c]);
                if (q >= 0) im_dot_phase_df(acc, h[j | spread<K, SEL>(r)], v[j | spread<K, SEL>(c)], (uint32_t)q);
            }
        }
    }
}

// three or four register bits: rare ops, runtime indices on a local copy
static __device__ __noinline__ void dense_apply_df_rt(CDF *v, const float4 *__restrict__ U, int K, uint32_t smask) {
    const int D = 1 << K;
    int sb[4];
    int n = 0;
    for (int b = 0; b < kWinBits; b++)
        if (smask >> b & 1) sb[n++] = b;
    CDF in[16];
    for (int j = 0; j < kWinAmps; j++) {
        if (j & smask) continue;
        for (int m = 0; m < D; m++) {
            int o = 0;
            for (int i = 0; i < K; i++)
                if (m >> i & 1) o |= 1 << sb[i];
            in[m] = v[j | o];
        }
        for (int r = 0; r < D; r++) {
            float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
            for (int c = 0; c < D; c++) cdf_mac(U[r * D + c], in[c], rh, rl, ih, il);
            int o = 0;
            for (int i = 0; i < K; i++)
                if (r >> i & 1) o |= 1 << sb[i];
            v[j | o] = {{rh, rl}, {ih, il}};
        }
    }
}

static __device__ __noinline__ void dense_gen_dot_df_rt(const CDF *v, const CDF *h, const float4 *__restrict__ G, int K,
                                                 uint32_t smask, DAcc &acc) {
    const int D = 1 << K;
    int sb[4];
    int n = 0;
    for (int b = 0; b < kWinBits; b++)
        if (smask >> b & 1) sb[n++] = b;
    for (int j = 0; j < kWinAmps; j++) {
        if (j & smask) continue;
        for (int r = 0; r < D; r++) {
            int orow = 0;
            for (int i = 0; i < K; i++)
                if (r >> i & 1) orow |= 1 << sb[i];
            for (int c = 0; c < D; c++) {
                const int q = gen_code(G[r * D + c]);
                if (q < 0) continue;
                int oc = 0;
                for (int i = 0; i < K; i++)
                    if (c >> i & 1) oc |= 1 << sb[i];
                im_dot_phase_df(acc, h[j | orow], v[j | oc], (uint32_t)q);
            }
        }
    }
}

// one-wire diagonal on register bit Q
template <int Q, bool BWD>
__device__ __forceinline__ void diag1_reg_df(CDF (&lv)[kWinAmps], CDF (&hv)[kWinAmps], float4 e0, float4 e1, float g0,
                                             float g1, bool tr, DAcc &a0, DAcc &a1) {
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        const bool one = (j >> Q) & 1;
        if (tr) {
            // g (real, 0 or +-1) Im(conj(h) v)
            const float gd = one ? g1 : g0;
            DAcc &acc = (j & 1) ? a1 : a0;
            if (gd != 0.0f) im_dot_phase_df(acc, hv[j], lv[j], gd > 0.0f ? 0u : 2u);
        }
        const float4 e = one ? e1 : e0;
        lv[j] = cdf_mul(e, lv[j]);
        if (BWD) hv[j] = cdf_mul(e, hv[j]);
    }
}

// SLIM: the window holds only one-wire dense ops, one-wire diagonals and
// CNOTs (checked on the host); the kernel then carries only those cases,
// which keeps its hot loop inside the instruction cache.
template <bool BWD, bool SLIM = false>
__device__ __forceinline__ void window_op_df(const EOp &op, CDF (&lv)[kWinAmps], CDF (&hv)[kWinAmps], uint32_t base,
                                             const uint32_t (&bb)[4], const float4 *__restrict__ mats, DAcc &acc,
                                             DAcc &acc1) {
    const bool tr = BWD && op.red != 0xff;
    if (SLIM && op.kind == EK_DENSE) {
        const float4 *U = mats + op.mat;
#define PLK_DF1S_CASE(S_)                                                                                             \
    case S_:                                                                                                           \
        if (tr) gen1_pattern_df<S_>(lv, hv, op.bits, acc, acc1);                                                       \
        dense_apply_df<1, S_>(lv, U);                                                                                  \
        if (BWD) dense_apply_df<1, S_>(hv, U);                                                                         \
        break;                                                                                                         \
    case 4 + S_:                                                                                                       \
        if (tr) gen1_fixed_df<S_, false>(lv, hv, acc, acc1);                                                           \
        rx_apply_df<S_>(lv, U);                                                                                        \
        if (BWD) rx_apply_df<S_>(hv, U);                                                                               \
        break;                                                                                                         \
    case 8 + S_:                                                                                                       \
        if (tr) gen1_fixed_df<S_, true>(lv, hv, acc, acc1);                                                            \
        ry_apply_df<S_>(lv, U);                                                                                        \
        if (BWD) ry_apply_df<S_>(hv, U);                                                                               \
        break;
        switch (op.sel) {
            PLK_DF1S_CASE(0) PLK_DF1S_CASE(1) PLK_DF1S_CASE(2) PLK_DF1S_CASE(3)
        default: break;
        }
#undef PLK_DF1S_CASE
    } else if (!SLIM && op.kind == EK_DENSE) {
        const float4 *U = mats + op.mat;
#define PLK_DF1_CASE(S_)                                                                                              \
    case 16 + S_:                                                                                                      \
        if (tr) gen1_pattern_df<S_>(lv, hv, op.bits, acc, acc1);                                                       \
        dense_apply_df<1, S_>(lv, U);                                                                                  \
        if (BWD) dense_apply_df<1, S_>(hv, U);                                                                         \
        break;                                                                                                         \
    case 16 + 4 + S_:                                                                                                  \
        if (tr) gen1_fixed_df<S_, false>(lv, hv, acc, acc1);                                                           \
        rx_apply_df<S_>(lv, U);                                                                                        \
        if (BWD) rx_apply_df<S_>(hv, U);                                                                               \
        break;                                                                                                         \
    case 16 + 8 + S_:                                                                                                  \
        if (tr) gen1_fixed_df<S_, true>(lv, hv, acc, acc1);                                                            \
        ry_apply_df<S_>(lv, U);                                                                                        \
        if (BWD) ry_apply_df<S_>(hv, U);                                                                               \
        break;
#define PLK_DF2_CASE(S_)                                                                                              \
    case 32 + S_:                                                                                                      \
        if (tr) dense_gen_dot_df<2, S_>(lv, hv, mats + op.gen, acc);                                                   \
        dense_apply_df<2, S_>(lv, U);                                                                                  \
        if (BWD) dense_apply_df<2, S_>(hv, U);                                                                         \
        break;
        switch (op.K * 16 + op.sel) {
            PLK_DF1_CASE(0) PLK_DF1_CASE(1) PLK_DF1_CASE(2) PLK_DF1_CASE(3)
            PLK_DF2_CASE(0) PLK_DF2_CASE(1) PLK_DF2_CASE(2) PLK_DF2_CASE(3) PLK_DF2_CASE(4) PLK_DF2_CASE(5)
        default: {
            const uint32_t smask = op.K == 4 ? 15u : (15u & ~(1u << op.sel));
            CDF tl[kWinAmps], th[kWinAmps];
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                tl[j] = lv[j];
                th[j] = hv[j];
            }
            if (tr) dense_gen_dot_df_rt(tl, th, mats + op.gen, op.K, smask, acc);
            dense_apply_df_rt(tl, U, op.K, smask);
            if (BWD) dense_apply_df_rt(th, U, op.K, smask);
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                lv[j] = tl[j];
                hv[j] = th[j];
            }
            break;
        }
        }
#undef PLK_DF1_CASE
#undef PLK_DF2_CASE
    } else if (op.kind == EK_CX) {
#define PLK_CX_CASE(C_, T_)                                                                                           \
    case C_ * 4 + T_:                                                                                                  \
        cx_apply<C_, T_>(lv);                                                                                          \
        if (BWD) cx_apply<C_, T_>(hv);                                                                                 \
        break;
        switch (op.sel) {
            PLK_CX_CASE(0, 1) PLK_CX_CASE(0, 2) PLK_CX_CASE(0, 3) PLK_CX_CASE(1, 0) PLK_CX_CASE(1, 2)
            PLK_CX_CASE(1, 3) PLK_CX_CASE(2, 0) PLK_CX_CASE(2, 1) PLK_CX_CASE(2, 3) PLK_CX_CASE(3, 0)
            PLK_CX_CASE(3, 1) PLK_CX_CASE(3, 2)
        default: break;
        }
#undef PLK_CX_CASE
    } else if (op.kind == EK_DIAG && op.K == 1) {
        const float4 e0 = mats[op.mat], e1 = mats[op.mat + 1];
        float g0 = 0.0f, g1 = 0.0f;
        if (tr) {
            g0 = mats[op.gen].x;
            g1 = mats[op.gen + 1].x;
        }
        switch (op.sel) {
        case 0: diag1_reg_df<0, BWD>(lv, hv, e0, e1, g0, g1, tr, acc, acc1); break;
        case 1: diag1_reg_df<1, BWD>(lv, hv, e0, e1, g0, g1, tr, acc, acc1); break;
        case 2: diag1_reg_df<2, BWD>(lv, hv, e0, e1, g0, g1, tr, acc, acc1); break;
        case 3: diag1_reg_df<3, BWD>(lv, hv, e0, e1, g0, g1, tr, acc, acc1); break;
        default: {
            const bool one = (base >> (op.bits & 31u)) & 1u;
            const float4 e = one ? e1 : e0;
            const float gd = one ? g1 : g0;
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                if (tr && gd != 0.0f) im_dot_phase_df((j & 1) ? acc1 : acc, hv[j], lv[j], gd > 0.0f ? 0u : 2u);
                lv[j] = cdf_mul(e, lv[j]);
                if (BWD) hv[j] = cdf_mul(e, hv[j]);
            }
        }
        }
    } else if (!SLIM) {
        const bool parity = op.kind == EK_PARITY;
#pragma unroll
        for (int j = 0; j < kWinAmps; j++) {
            const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                 ((j & 8) ? bb[3] : 0);
            const uint32_t g = parity ? (uint32_t)(__popc(idx & op.bits) & 1) : diag_index(idx, op.bits, op.K);
            const float4 e = mats[op.mat + g];
            if (tr) {
                // generator diagonal: MultiRZ (-1)^parity, otherwise real entries 0, +-1
                const float gd = parity ? (g ? -1.0f : 1.0f) : mats[op.gen + g].x;
                if (gd != 0.0f) im_dot_phase_df((j & 1) ? acc1 : acc, hv[j], lv[j], gd > 0.0f ? 0u : 2u);
            }
            lv[j] = cdf_mul(e, lv[j]);
            if (BWD) hv[j] = cdf_mul(e, hv[j]);
        }
    }
}

constexpr int kWinThreadsDf = 256;

// complex128 windows on the FP32 pipe (window_df.cuh).  Between windows of
// one sweep the states stay in double-float form in their own buffers (a
// {re.hi, re.lo, im.hi, im.lo} float4 has the size of a double2): the first
// window splits the doubles (in_df = 0), the last joins them back
// (out_df = 0), the ones between move raw pairs.
template <bool BWD, bool SLIM>
__global__ void __launch_bounds__(kWinThreadsDf, 1)
    k_state_window_df(double2 *lam, double2 *hl, int nq, const EWin *__restrict__ wins, int wi,
                      const EOp *__restrict__ ops, const float4 *__restrict__ mats, const ETrain *__restrict__ train,
                      double *__restrict__ bpart, int in_df, int out_df) {
    __shared__ float2 part[kMaxWinTrain * kWinThreadsDf];
    const EWin w = wins[wi];
    const int tid = threadIdx.x;
    if (BWD)
        for (int t = 0; t < w.ntrain; t++) part[t * kWinThreadsDf + tid] = make_float2(0.0f, 0.0f);
    const uint32_t nu = 1u << (nq - kWinBits);
    const uint32_t bb[4] = {1u << w.rb[0], 1u << w.rb[1], 1u << w.rb[2], 1u << w.rb[3]};
    const uint32_t tstep = gridDim.x * kWinThreadsDf;
    for (uint32_t u = blockIdx.x * kWinThreadsDf + tid; u < nu; u += tstep) {
        uint32_t base = u;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t lo = base & (bb[i] - 1);
            base = ((base ^ lo) << 1) | lo;
        }
        CDF lv[kWinAmps], hv[kWinAmps];
#pragma unroll
        for (int j = 0; j < kWinAmps; j++) {
            const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                 ((j & 8) ? bb[3] : 0);
            if (in_df) {
                const float4 a = reinterpret_cast<const float4 *>(lam)[idx];
                lv[j] = {{a.x, a.y}, {a.z, a.w}};
                if (BWD) {
                    const float4 b = reinterpret_cast<const float4 *>(hl)[idx];
                    hv[j] = {{b.x, b.y}, {b.z, b.w}};
                } else {
                    hv[j] = cdf_zero();
                }
            } else {
                lv[j] = cdf_split(lam[idx]);
                hv[j] = BWD ? cdf_split(hl[idx]) : cdf_zero();
            }
        }
        for (int k = 0; k < w.nops; k++) {
            const EOp op = ops[w.op0 + k];
            DAcc acc, acc1;
            if (BWD && op.red != 0xff) {
                const float2 p = part[op.red * kWinThreadsDf + tid];
                acc.h = p.x;
                acc.l = p.y;
            }
            window_op_df<BWD, SLIM>(op, lv, hv, base, bb, mats, acc, acc1);
            if (BWD && op.red != 0xff) {
                df_add(acc1.h, acc1.l, acc.h, acc.l);
                part[op.red * kWinThreadsDf + tid] = make_float2(acc.h, acc.l);
            }
        }
#pragma unroll
        for (int j = 0; j < kWinAmps; j++) {
            const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                 ((j & 8) ? bb[3] : 0);
            if (out_df) {
                reinterpret_cast<float4 *>(lam)[idx] = make_float4(lv[j].re.hi, lv[j].re.lo, lv[j].im.hi, lv[j].im.lo);
                if (BWD)
                    reinterpret_cast<float4 *>(hl)[idx] =
                        make_float4(hv[j].re.hi, hv[j].re.lo, hv[j].im.hi, hv[j].im.lo);
            } else {
                lam[idx] = make_double2(df_join(lv[j].re.hi, lv[j].re.lo), df_join(lv[j].im.hi, lv[j].im.lo));
                if (BWD)
                    hl[idx] = make_double2(df_join(hv[j].re.hi, hv[j].re.lo), df_join(hv[j].im.hi, hv[j].im.lo));
            }
        }
    }
    if (BWD && w.ntrain > 0) {
        __syncthreads();
        const int lane = tid & 31, warp = tid >> 5;
        for (int t = warp; t < w.ntrain; t += kWinThreadsDf / 32) {
            EAcc<float> acc;
#pragma unroll
            for (int i = 0; i < kWinThreadsDf / 32; i++) {
                const float2 p = part[t * kWinThreadsDf + i * 32 + lane];
                df_add(p.x, p.y, acc.h, acc.l);
            }
            const double sum = acc.warp_sum();
            if (lane == 0) {
                const ETrain tr = train[w.tr0 + t];
                bpart[(size_t)tr.slot * gridDim.x + blockIdx.x] = (double)tr.gscale * sum;
            }
        }
    }
}


} // namespace plk
