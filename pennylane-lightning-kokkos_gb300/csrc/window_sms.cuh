// window_sms.cuh — complex64 register windows over one state, amplitudes
// staged in shared memory.
//
// The complex64 counterpart of window_dfs.cuh: a thread's 16 amplitudes of
// lambda (and, going backwards, of H lambda) live in shared memory slots
// [j][thread] between ops, and each op kind is one compact loop whose
// register-bit positions are runtime values.  Register-resident windows with
// every op kind unrolled for every register bit (batch_engine.cuh, still used
// by the batch engine) stalled on instruction fetch here ("no instruction"
// 1.1 cycles per issue at 48 % issue activity, 24 qubits).  Arithmetic is FP32;
// generator inner products are formed in FP32 over two amplitude pairs (or
// four amplitudes) and accumulated in double-float (EAcc<float>).
#pragma once

#include "batch_engine.cuh"

namespace plk {

constexpr int kWinThreadsSms = 128;
constexpr int kSmsCtasBwd = 4, kSmsCtasFwd = 6;

// dynamic shared memory of one CTA: lambda slots, H lambda slots (backward),
// double-float partial sums of the window's `ntrain` trainable ops (backward)
__host__ __device__ constexpr size_t sms_smem_bytes(bool bwd, int ntrain = kMaxWinTrain) {
    return (size_t)kWinAmps * kWinThreadsSms * sizeof(float2) * (bwd ? 2 : 1) +
           (bwd ? (size_t)ntrain * kWinThreadsSms * sizeof(float2) : 0);
}

struct SmsSlots {
    float2 *L, *M; // [kWinAmps][kWinThreadsSms]
    int tid;
    __device__ __forceinline__ float2 ld(const float2 *A, int j) const { return A[j * kWinThreadsSms + tid]; }
    __device__ __forceinline__ void st(float2 *A, int j, float2 v) const { A[j * kWinThreadsSms + tid] = v; }
};

__device__ __forceinline__ int sms_ins0(int p, int b) { return ((p >> b) << (b + 1)) | (p & ((1 << b) - 1)); }

__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 c_fma(float2 a, float2 b, float2 c) {
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

// One pair (j0, j1) of a one-wire dense op; the pair's generator terms are
// added to the FP32 partial t.  FORM: 0 general (generator pattern), 1 RX, 2 RY.
template <bool BWD, int FORM>
__device__ __forceinline__ void sms_pair1(const SmsSlots &S, int j0, int j1, const float2 (&u)[4], bool tr,
                                          uint32_t pat, float &t) {
    const float2 x = S.ld(S.L, j0), y = S.ld(S.L, j1);
    float2 hx, hy;
    if (BWD) {
        hx = S.ld(S.M, j0);
        hy = S.ld(S.M, j1);
    }
    if (BWD && tr) {
        if (FORM == 2) { // Pauli Y: -Re(conj(h0) v1) + Re(conj(h1) v0)
            t = fmaf(-hx.x, y.x, t);
            t = fmaf(-hx.y, y.y, t);
            t = fmaf(hy.x, x.x, t);
            t = fmaf(hy.y, x.y, t);
        } else if (FORM == 1) { // Pauli X: Im(conj(h0) v1) + Im(conj(h1) v0)
            t = fmaf(hx.x, y.y, t);
            t = fmaf(-hx.y, y.x, t);
            t = fmaf(hy.x, x.y, t);
            t = fmaf(-hy.y, x.x, t);
        } else {
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const uint32_t rp = (pat >> (4 * r)) & 15u;
                if (!(rp & 1u)) continue;
                const uint32_t q = rp >> 2;
                const float sg = q >= 2 ? -1.0f : 1.0f;
                const float2 v = (rp & 2u) ? y : x, h = r ? hy : hx;
                // Im(conj(h) i^q v): q even -> +-(h.x v.y - h.y v.x); q odd -> +-(h.x v.x + h.y v.y)
                if (q & 1u) {
                    t = fmaf(sg * h.x, v.x, t);
                    t = fmaf(sg * h.y, v.y, t);
                } else {
                    t = fmaf(sg * h.x, v.y, t);
                    t = fmaf(-sg * h.y, v.x, t);
                }
            }
        }
    }
    if (FORM == 2) {
        const float c = u[0].x, s = u[2].x;
        S.st(S.L, j0, make_float2(c * x.x - s * y.x, c * x.y - s * y.y));
        S.st(S.L, j1, make_float2(s * x.x + c * y.x, s * x.y + c * y.y));
        if (BWD) {
            S.st(S.M, j0, make_float2(c * hx.x - s * hy.x, c * hx.y - s * hy.y));
            S.st(S.M, j1, make_float2(s * hx.x + c * hy.x, s * hx.y + c * hy.y));
        }
    } else if (FORM == 1) {
        const float c = u[0].x, w = u[1].y;
        S.st(S.L, j0, make_float2(c * x.x - w * y.y, c * x.y + w * y.x));
        S.st(S.L, j1, make_float2(c * y.x - w * x.y, c * y.y + w * x.x));
        if (BWD) {
            S.st(S.M, j0, make_float2(c * hx.x - w * hy.y, c * hx.y + w * hy.x));
            S.st(S.M, j1, make_float2(c * hy.x - w * hx.y, c * hy.y + w * hx.x));
        }
    } else {
        S.st(S.L, j0, c_fma(u[1], y, c_mul(u[0], x)));
        S.st(S.L, j1, c_fma(u[3], y, c_mul(u[2], x)));
        if (BWD) {
            S.st(S.M, j0, c_fma(u[1], hy, c_mul(u[0], hx)));
            S.st(S.M, j1, c_fma(u[3], hy, c_mul(u[2], hx)));
        }
    }
}

// One-wire dense op on register bit b: 8 pairs; the FP32 partial of every two
// pairs goes into a0 or a1 alternately (independent addition chains)
template <bool BWD, int FORM>
__device__ __forceinline__ void sms_op1(const SmsSlots &S, int b, const float2 *__restrict__ U, bool tr, uint32_t pat,
                                        EAcc<float> &a0, EAcc<float> &a1) {
    const float2 u[4] = {U[0], U[1], U[2], U[3]};
#pragma unroll 1
    for (int p = 0; p < kWinAmps / 2; p += 4) {
        float t = 0.0f;
        int j = sms_ins0(p, b);
        sms_pair1<BWD, FORM>(S, j, j | (1 << b), u, tr, pat, t);
        j = sms_ins0(p + 1, b);
        sms_pair1<BWD, FORM>(S, j, j | (1 << b), u, tr, pat, t);
        if (BWD && tr) a0.addf(t);
        t = 0.0f;
        j = sms_ins0(p + 2, b);
        sms_pair1<BWD, FORM>(S, j, j | (1 << b), u, tr, pat, t);
        j = sms_ins0(p + 3, b);
        sms_pair1<BWD, FORM>(S, j, j | (1 << b), u, tr, pat, t);
        if (BWD && tr) a1.addf(t);
    }
}

template <int K> __device__ __forceinline__ int sms_spread(int m, uint32_t rbits) {
    int o = 0;
#pragma unroll
    for (int i = 0; i < K; i++)
        if ((m >> i) & 1) o |= 1 << ((rbits >> (8 * i)) & 3u);
    return o;
}

// Dense op on K = 2, 3 or 4 register bits; the trainable generator is a dense
// matrix with entries 0, +-1, +-i, so G v is exact in FP32.
template <int K, bool BWD>
__device__ __noinline__ EAcc<float> sms_dense(SmsSlots S, uint32_t rbits, const float2 *__restrict__ U,
                                              const float2 *__restrict__ G, bool tr, EAcc<float> acc) {
    constexpr int D = 1 << K;
    const int gm = sms_spread<K>(D - 1, rbits);
#pragma unroll 1
    for (int g0 = 0; g0 < kWinAmps; g0++) {
        if (g0 & gm) continue;
        float2 in[D];
#pragma unroll
        for (int m = 0; m < D; m++) in[m] = S.ld(S.L, g0 | sms_spread<K>(m, rbits));
        if (BWD && tr) {
#pragma unroll 1
            for (int r = 0; r < D; r++) {
                float2 gv = make_float2(0.0f, 0.0f);
#pragma unroll
                for (int c = 0; c < D; c++) gv = c_fma(G[r * D + c], in[c], gv);
                acc.im_dot(S.ld(S.M, g0 | sms_spread<K>(r, rbits)), gv);
            }
        }
#pragma unroll 1
        for (int r = 0; r < D; r++) {
            float2 o = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int c = 0; c < D; c++) o = c_fma(U[r * D + c], in[c], o);
            S.st(S.L, g0 | sms_spread<K>(r, rbits), o);
        }
        if (BWD) {
#pragma unroll
            for (int m = 0; m < D; m++) in[m] = S.ld(S.M, g0 | sms_spread<K>(m, rbits));
#pragma unroll 1
            for (int r = 0; r < D; r++) {
                float2 o = make_float2(0.0f, 0.0f);
#pragma unroll
                for (int c = 0; c < D; c++) o = c_fma(U[r * D + c], in[c], o);
                S.st(S.M, g0 | sms_spread<K>(r, rbits), o);
            }
        }
    }
    return acc;
}

template <bool BWD> __device__ __forceinline__ void sms_cx(const SmsSlots &S, int c, int t) {
    const int lo = c < t ? c : t, hi = c < t ? t : c;
#pragma unroll 1
    for (int p = 0; p < kWinAmps / 4; p++) {
        const int j = sms_ins0(sms_ins0(p, lo), hi) | (1 << c), k = j | (1 << t);
        const float2 a = S.ld(S.L, j), b = S.ld(S.L, k);
        S.st(S.L, j, b);
        S.st(S.L, k, a);
        if (BWD) {
            const float2 x = S.ld(S.M, j), y = S.ld(S.M, k);
            S.st(S.M, j, y);
            S.st(S.M, k, x);
        }
    }
}

// Diagonal op: amplitude j gets phase e(j); a trainable op's real generator
// entry gd(j) (0, +-1) weights Im(conj(h_j) v_j).  MODE as in window_dfs.cuh:
// 0 one wire on register bit sel, 1 one wire on a fixed state bit, 2 several
// wires or MultiRZ (phase from each amplitude's full index).
template <bool BWD, int MODE>
__device__ __forceinline__ void sms_diag(const SmsSlots &S, const EOp &op, uint32_t base, const uint32_t (&bb)[4],
                                         const float2 *__restrict__ mats, bool tr, EAcc<float> &a0,
                                         EAcc<float> &a1) {
    float2 e0 = make_float2(0.0f, 0.0f), e1 = e0;
    float g0 = 0.0f, g1 = 0.0f;
    if (MODE < 2) {
        e0 = mats[op.mat];
        e1 = mats[op.mat + 1];
        if (tr) {
            g0 = mats[op.gen].x;
            g1 = mats[op.gen + 1].x;
        }
    }
    const bool fixed_one = MODE == 1 && ((base >> (op.bits & 31u)) & 1u);
    const bool parity = op.kind == EK_PARITY;
    const int b = op.sel & 3;
#pragma unroll 1
    for (int j8 = 0; j8 < kWinAmps; j8 += 8) {
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const int j0 = j8 + 4 * half;
        float t = 0.0f;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int j = j0 + q;
            float2 e;
            float gd;
            if (MODE == 2) {
                const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                     ((j & 8) ? bb[3] : 0);
                const uint32_t g = parity ? (uint32_t)(__popc(idx & op.bits) & 1) : diag_index(idx, op.bits, op.K);
                e = mats[op.mat + g];
                gd = tr ? (parity ? (g ? -1.0f : 1.0f) : mats[op.gen + g].x) : 0.0f;
            } else {
                const bool one = MODE == 1 ? fixed_one : (bool)((j >> b) & 1);
                e = one ? e1 : e0;
                gd = one ? g1 : g0;
            }
            const float2 x = S.ld(S.L, j);
            if (BWD) {
                const float2 h = S.ld(S.M, j);
                if (tr && gd != 0.0f) t = fmaf(gd, fmaf(h.x, x.y, -h.y * x.x), t);
                S.st(S.M, j, c_mul(h, e));
            }
            S.st(S.L, j, c_mul(x, e));
        }
        if (BWD && tr) (half ? a1 : a0).addf(t);
    }
    }
}

// Merged diagonal ops (EK_DIAGSET): one product phase per amplitude, and every
// trainable one-wire member's inner product a signed sum of the same
// c_j = Im(conj(h_j) v_j) (the phases cancel in conj(h_j) v_j).
template <bool BWD>
__device__ __forceinline__ void sms_diagset(const SmsSlots &S, const EOp &op, const float2 *__restrict__ mats,
                                            float2 *part) {
    const int nm = BWD ? op.K : 0;
    EAcc<float> a[4];
#pragma unroll
    for (int m = 0; m < 4; m++)
        if (m < nm) a[m].load(part[((op.gen >> (4 * m)) & 15) * kWinThreadsSms + S.tid]);
#pragma unroll 1
    for (int j0 = 0; j0 < kWinAmps; j0 += 4) {
        float t[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int j = j0 + q;
            const float2 e = mats[op.mat + j];
            const float2 x = S.ld(S.L, j);
            if (BWD) {
                const float2 h = S.ld(S.M, j);
                if (nm > 0) {
                    const float c = fmaf(h.x, x.y, -h.y * x.x);
#pragma unroll
                    for (int m = 0; m < 4; m++)
                        if (m < nm) {
                            const uint32_t mb = op.bits >> (8 * m);
                            const uint32_t code = ((j >> (mb & 3u)) & 1) ? (mb >> 4) & 3u : (mb >> 2) & 3u;
                            if (code) t[m] += code == 1u ? c : -c;
                        }
                }
                S.st(S.M, j, c_mul(h, e));
            }
            S.st(S.L, j, c_mul(x, e));
        }
#pragma unroll
        for (int m = 0; m < 4; m++)
            if (m < nm) a[m].addf(t[m]);
    }
#pragma unroll
    for (int m = 0; m < 4; m++)
        if (m < nm) part[((op.gen >> (4 * m)) & 15) * kWinThreadsSms + S.tid] = a[m].slot();
}

template <bool BWD>
__device__ __forceinline__ void sms_window_op(const SmsSlots &S, const EOp &op, uint32_t base, const uint32_t (&bb)[4],
                                              const float2 *__restrict__ mats, EAcc<float> &acc, EAcc<float> &acc1,
                                              float2 *part) {
    const bool tr = BWD && op.red != 0xff;
    if (op.kind == EK_DIAGSET) {
        sms_diagset<BWD>(S, op, mats, part);
    } else if (op.kind == EK_DENSE) {
        const float2 *U = mats + op.mat;
        if (op.K == 1) {
            const int b = op.sel & 3, form = op.sel >> 2;
            if (form == EF_RY) sms_op1<BWD, 2>(S, b, U, tr, op.bits, acc, acc1);
            else if (form == EF_RX) sms_op1<BWD, 1>(S, b, U, tr, op.bits, acc, acc1);
            else sms_op1<BWD, 0>(S, b, U, tr, op.bits, acc, acc1);
        } else {
            uint32_t rbits = 0x03020100u;
            if (op.K == 2) rbits = ((0x211000u >> (4 * op.sel)) & 15u) | (((0x332321u >> (4 * op.sel)) & 15u) << 8);
            else if (op.K == 3) rbits = op.sel == 0 ? 0x030201u : op.sel == 1 ? 0x030200u : op.sel == 2 ? 0x030100u
                                                                                                   : 0x020100u;
            const float2 *G = mats + (tr ? op.gen : 0);
            if (op.K == 2) acc = sms_dense<2, BWD>(S, rbits, U, G, tr, acc);
            else if (op.K == 3) acc = sms_dense<3, BWD>(S, rbits, U, G, tr, acc);
            else acc = sms_dense<4, BWD>(S, rbits, U, G, tr, acc);
        }
    } else if (op.kind == EK_CX) {
        sms_cx<BWD>(S, op.sel >> 2, op.sel & 3);
    } else if (op.kind == EK_DIAG && op.K == 1) {
        if (op.sel < 4) sms_diag<BWD, 0>(S, op, base, bb, mats, tr, acc, acc1);
        else sms_diag<BWD, 1>(S, op, base, bb, mats, tr, acc, acc1);
    } else {
        sms_diag<BWD, 2>(S, op, base, bb, mats, tr, acc, acc1);
    }
}

// One window over the whole state (grid-stride over the 2^(n-4) groups).
// With state bit 0 in the window, the pairs (j, j | 1) are adjacent in the
// state and move as one 16-byte access.
template <bool BWD>
__global__ void __launch_bounds__(kWinThreadsSms, BWD ? kSmsCtasBwd : kSmsCtasFwd)
    k_state_window_sms(float2 *lam, float2 *hl, int nq, const EWin *__restrict__ wins, int wi,
                       const EOp *__restrict__ ops, const float2 *__restrict__ mats,
                       const ETrain *__restrict__ train, double *__restrict__ bpart) {
    extern __shared__ __align__(16) unsigned char sms_smem[];
    const int tid = threadIdx.x;
    SmsSlots S;
    S.L = reinterpret_cast<float2 *>(sms_smem);
    S.M = S.L + kWinAmps * kWinThreadsSms;
    S.tid = tid;
    float2 *part = S.L + (BWD ? 2 : 1) * kWinAmps * kWinThreadsSms;
    const EWin w = wins[wi];
    if (BWD)
        for (int t = 0; t < w.ntrain; t++) part[t * kWinThreadsSms + tid] = make_float2(0.0f, 0.0f);
    const uint32_t nu = 1u << (nq - kWinBits);
    const uint32_t bb[4] = {1u << w.rb[0], 1u << w.rb[1], 1u << w.rb[2], 1u << w.rb[3]};
    const bool pairs = bb[0] == 1u;
    const uint32_t tstep = gridDim.x * kWinThreadsSms;
    for (uint32_t u = blockIdx.x * kWinThreadsSms + tid; u < nu; u += tstep) {
        uint32_t base = u;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t lo = base & (bb[i] - 1);
            base = ((base ^ lo) << 1) | lo;
        }
        if (pairs) {
#pragma unroll
            for (int j = 0; j < kWinAmps; j += 2) {
                const uint32_t idx = base | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) | ((j & 8) ? bb[3] : 0);
                const float4 a = __ldcs(reinterpret_cast<const float4 *>(lam + idx));
                S.st(S.L, j, make_float2(a.x, a.y));
                S.st(S.L, j + 1, make_float2(a.z, a.w));
                if (BWD) {
                    const float4 h = __ldcs(reinterpret_cast<const float4 *>(hl + idx));
                    S.st(S.M, j, make_float2(h.x, h.y));
                    S.st(S.M, j + 1, make_float2(h.z, h.w));
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                     ((j & 8) ? bb[3] : 0);
                S.st(S.L, j, __ldcs(lam + idx));
                if (BWD) S.st(S.M, j, __ldcs(hl + idx));
            }
        }
        for (int k = 0; k < w.nops; k++) {
            const EOp op = ops[w.op0 + k];
            EAcc<float> acc, acc1;
            if (BWD && op.red != 0xff) acc.load(part[op.red * kWinThreadsSms + tid]);
            sms_window_op<BWD>(S, op, base, bb, mats, acc, acc1, part);
            if (BWD && op.red != 0xff) {
                acc.merge(acc1);
                part[op.red * kWinThreadsSms + tid] = acc.slot();
            }
        }
        if (pairs) {
#pragma unroll
            for (int j = 0; j < kWinAmps; j += 2) {
                const uint32_t idx = base | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) | ((j & 8) ? bb[3] : 0);
                const float2 a = S.ld(S.L, j), b = S.ld(S.L, j + 1);
                __stcs(reinterpret_cast<float4 *>(lam + idx), make_float4(a.x, a.y, b.x, b.y));
                if (BWD) {
                    const float2 x = S.ld(S.M, j), y = S.ld(S.M, j + 1);
                    __stcs(reinterpret_cast<float4 *>(hl + idx), make_float4(x.x, x.y, y.x, y.y));
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                     ((j & 8) ? bb[3] : 0);
                __stcs(lam + idx, S.ld(S.L, j));
                if (BWD) __stcs(hl + idx, S.ld(S.M, j));
            }
        }
    }
    if (BWD && w.ntrain > 0) {
        __syncthreads();
        const int lane = tid & 31, warp = tid >> 5;
        for (int t = warp; t < w.ntrain; t += kWinThreadsSms / 32) {
            EAcc<float> acc;
#pragma unroll
            for (int i = 0; i < kWinThreadsSms / 32; i++) {
                EAcc<float> x;
                x.load(part[t * kWinThreadsSms + i * 32 + lane]);
                acc.merge(x);
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
