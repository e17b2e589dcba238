// window_dfs.cuh — complex128 register windows, amplitudes staged in shared
// memory.
//
// Same op model and arithmetic as window_df.cuh (double-float pairs on the
// FP32 pipe, error-free products, two-sum accumulation), but a thread's 16
// amplitudes of lambda (and of H lambda going backwards) live in shared
// memory between ops, in slots [j][thread] (a warp touches 512 consecutive
// bytes per slot: no bank conflicts), and each op kind is one compact loop
// whose register-bit positions are runtime values.  Fully unrolled per-bit
// variants of every op (window_df.cuh) made a kernel of several hundred KB
// whose backward window stalled mostly on instruction fetch (ncu: "no
// instruction" 4.1 cycles per issue, 1.05 instructions per cycle per SM, 255
// registers with spills); here the code a window runs fits the instruction
// cache, registers hold only the amplitudes of the group being updated, and
// two or three (backward) or four (forward) CTAs share an SM.
#pragma once

#include "window_df.cuh"

namespace plk {

constexpr int kWinThreadsDfs = 128;
constexpr int kDfsCtasBwd = 3, kDfsCtasFwd = 4;

// dynamic shared memory of one CTA: lambda slots, H lambda slots (backward),
// per-thread partial sums of the window's `ntrain` trainable ops (backward).
// A backward window with up to 8 trainable ops takes 72 KiB, so three CTAs
// share an SM; with more, two.
__host__ __device__ constexpr size_t dfs_smem_bytes(bool bwd, int ntrain = kMaxWinTrain) {
    return (size_t)kWinAmps * kWinThreadsDfs * sizeof(float4) * (bwd ? 2 : 1) +
           (bwd ? (size_t)ntrain * kWinThreadsDfs * sizeof(float2) : 0);
}

struct DfsSlots {
    float4 *L, *M; // [kWinAmps][kWinThreadsDfs]
    int tid;
    __device__ __forceinline__ CDF ld(const float4 *A, int j) const {
        const float4 a = A[j * kWinThreadsDfs + tid];
        return {{a.x, a.y}, {a.z, a.w}};
    }
    __device__ __forceinline__ void st(float4 *A, int j, const CDF &v) const {
        A[j * kWinThreadsDfs + tid] = make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo);
    }
};

// slot index with a zero bit inserted at position b
__device__ __forceinline__ int ins0(int p, int b) { return ((p >> b) << (b + 1)) | (p & ((1 << b) - 1)); }

// One pair (j0, j1) of a one-wire dense op.  FORM: 0 general matrix
// (trainable generator given as a monomial pattern), 1 RX form, 2 RY form.
template <bool BWD, int FORM>
__device__ __forceinline__ void dfs_pair1(const DfsSlots &S, int j0, int j1, const float4 (&u)[4], bool tr,
                                          uint32_t pat, DAcc &acc) {
    const DF c = {u[0].x, u[0].y}, w = {u[1].z, u[1].w}, s = {u[2].x, u[2].y};
    const CDF x = S.ld(S.L, j0), y = S.ld(S.L, j1);
    CDF hx, hy;
    if (BWD) {
        hx = S.ld(S.M, j0);
        hy = S.ld(S.M, j1);
    }
    if (BWD && tr) {
        if (FORM == 2) { // Pauli Y: -Re(conj(h0) v1) + Re(conj(h1) v0)
            acc.msub(hx.re, y.re);
            acc.msub(hx.im, y.im);
            acc.mac(hy.re, x.re);
            acc.mac(hy.im, x.im);
        } else if (FORM == 1) { // Pauli X: Im(conj(h0) v1) + Im(conj(h1) v0)
            acc.mac(hx.re, y.im);
            acc.msub(hx.im, y.re);
            acc.mac(hy.re, x.im);
            acc.msub(hy.im, x.re);
        } else {
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const uint32_t rp = (pat >> (4 * r)) & 15u;
                if (!(rp & 1u)) continue;
                im_dot_phase_df(acc, r ? hy : hx, (rp & 2u) ? y : x, rp >> 2);
            }
        }
    }
    if (FORM == 2) {
        S.st(S.L, j0, {df_lin2(c, x.re, df_neg(s), y.re), df_lin2(c, x.im, df_neg(s), y.im)});
        S.st(S.L, j1, {df_lin2(s, x.re, c, y.re), df_lin2(s, x.im, c, y.im)});
        if (BWD) {
            S.st(S.M, j0, {df_lin2(c, hx.re, df_neg(s), hy.re), df_lin2(c, hx.im, df_neg(s), hy.im)});
            S.st(S.M, j1, {df_lin2(s, hx.re, c, hy.re), df_lin2(s, hx.im, c, hy.im)});
        }
    } else if (FORM == 1) {
        S.st(S.L, j0, {df_lin2(c, x.re, df_neg(w), y.im), df_lin2(c, x.im, w, y.re)});
        S.st(S.L, j1, {df_lin2(c, y.re, df_neg(w), x.im), df_lin2(c, y.im, w, x.re)});
        if (BWD) {
            S.st(S.M, j0, {df_lin2(c, hx.re, df_neg(w), hy.im), df_lin2(c, hx.im, w, hy.re)});
            S.st(S.M, j1, {df_lin2(c, hy.re, df_neg(w), hx.im), df_lin2(c, hy.im, w, hx.re)});
        }
    } else {
        float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
        cdf_mac(u[0], x, rh, rl, ih, il);
        cdf_mac(u[1], y, rh, rl, ih, il);
        S.st(S.L, j0, {{rh, rl}, {ih, il}});
        rh = rl = ih = il = 0.0f;
        cdf_mac(u[2], x, rh, rl, ih, il);
        cdf_mac(u[3], y, rh, rl, ih, il);
        S.st(S.L, j1, {{rh, rl}, {ih, il}});
        if (BWD) {
            rh = rl = ih = il = 0.0f;
            cdf_mac(u[0], hx, rh, rl, ih, il);
            cdf_mac(u[1], hy, rh, rl, ih, il);
            S.st(S.M, j0, {{rh, rl}, {ih, il}});
            rh = rl = ih = il = 0.0f;
            cdf_mac(u[2], hx, rh, rl, ih, il);
            cdf_mac(u[3], hy, rh, rl, ih, il);
            S.st(S.M, j1, {{rh, rl}, {ih, il}});
        }
    }
}

// One-wire dense op on register bit b: 8 pairs, two per iteration (one per
// accumulator, for independent addition chains)
template <bool BWD, int FORM>
__device__ __forceinline__ void dfs_op1(const DfsSlots &S, int b, const float4 *__restrict__ U, bool tr, uint32_t pat,
                                        DAcc &a0, DAcc &a1) {
    const float4 u[4] = {U[0], U[1], U[2], U[3]};
#pragma unroll 1
    for (int p = 0; p < kWinAmps / 2; p += 2) {
        const int j0 = ins0(p, b), j1 = ins0(p + 1, b);
        dfs_pair1<BWD, FORM>(S, j0, j0 | (1 << b), u, tr, pat, a0);
        dfs_pair1<BWD, FORM>(S, j1, j1 | (1 << b), u, tr, pat, a1);
    }
}

// slot offset of local index m of a K-bit op whose register bits are packed
// one per byte in rbits (local bit i <-> register bit byte i)
template <int K> __device__ __forceinline__ int dfs_spread(int m, uint32_t rbits) {
    int o = 0;
#pragma unroll
    for (int i = 0; i < K; i++)
        if ((m >> i) & 1) o |= 1 << ((rbits >> (8 * i)) & 3u);
    return o;
}

// Dense op on K = 2, 3 or 4 register bits; the trainable generator is a dense
// matrix with entries 0, +-1, +-i.  Rows run as a loop (the inputs of a group
// sit in registers), which keeps the code of the 16 x 16 case small.
template <int K, bool BWD>
__device__ __noinline__ DAcc dfs_dense(DfsSlots S, uint32_t rbits, const float4 *__restrict__ U,
                                       const float4 *__restrict__ G, bool tr, DAcc acc) {
    constexpr int D = 1 << K;
    const int gm = dfs_spread<K>(D - 1, rbits);
#pragma unroll 1
    for (int g0 = 0; g0 < kWinAmps; g0++) {
        if (g0 & gm) continue;
        CDF in[D];
#pragma unroll
        for (int m = 0; m < D; m++) in[m] = S.ld(S.L, g0 | dfs_spread<K>(m, rbits));
        if (BWD && tr) {
#pragma unroll 1
            for (int r = 0; r < D; r++) {
                const CDF h = S.ld(S.M, g0 | dfs_spread<K>(r, rbits));
#pragma unroll
                for (int c = 0; c < D; c++) {
                    const int q = gen_code(G[r * D + c]);
                    if (q >= 0) im_dot_phase_df(acc, h, in[c], (uint32_t)q);
                }
            }
        }
#pragma unroll 1
        for (int r = 0; r < D; r++) {
            float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
#pragma unroll
            for (int c = 0; c < D; c++) cdf_mac(U[r * D + c], in[c], rh, rl, ih, il);
            S.st(S.L, g0 | dfs_spread<K>(r, rbits), {{rh, rl}, {ih, il}});
        }
        if (BWD) {
#pragma unroll
            for (int m = 0; m < D; m++) in[m] = S.ld(S.M, g0 | dfs_spread<K>(m, rbits));
#pragma unroll 1
            for (int r = 0; r < D; r++) {
                float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
#pragma unroll
                for (int c = 0; c < D; c++) cdf_mac(U[r * D + c], in[c], rh, rl, ih, il);
                S.st(S.M, g0 | dfs_spread<K>(r, rbits), {{rh, rl}, {ih, il}});
            }
        }
    }
    return acc;
}

// CNOT inside the window: swap the slots of the target pair where the control is set
template <bool BWD> __device__ __forceinline__ void dfs_cx(const DfsSlots &S, int c, int t) {
    const int lo = c < t ? c : t, hi = c < t ? t : c;
#pragma unroll 1
    for (int p = 0; p < kWinAmps / 4; p++) {
        const int j = ins0(ins0(p, lo), hi) | (1 << c), k = j | (1 << t);
        const float4 a = S.L[j * kWinThreadsDfs + S.tid], b = S.L[k * kWinThreadsDfs + S.tid];
        S.L[j * kWinThreadsDfs + S.tid] = b;
        S.L[k * kWinThreadsDfs + S.tid] = a;
        if (BWD) {
            const float4 x = S.M[j * kWinThreadsDfs + S.tid], y = S.M[k * kWinThreadsDfs + S.tid];
            S.M[j * kWinThreadsDfs + S.tid] = y;
            S.M[k * kWinThreadsDfs + S.tid] = x;
        }
    }
}

// One amplitude of a diagonal op: phase e, real generator entry gd (0, +-1)
template <bool BWD>
__device__ __forceinline__ void dfs_diag1(const DfsSlots &S, int j, const float4 &e, float gd, bool tr, DAcc &acc) {
    const CDF x = S.ld(S.L, j);
    if (BWD) {
        const CDF h = S.ld(S.M, j);
        if (tr && gd != 0.0f) im_dot_phase_df(acc, h, x, gd > 0.0f ? 0u : 2u);
        S.st(S.M, j, cdf_mul(e, h));
    }
    S.st(S.L, j, cdf_mul(e, x));
}

// Diagonal op: amplitude j gets phase e(j) (and, trainable, the real
// generator entry gd(j) in 0, +-1 enters Im <h | G v>).  MODE 0: one wire on
// register bit sel (phase by that bit of j); 1: one wire on a state bit
// outside the window (one phase for the whole group); 2: several wires or
// MultiRZ (phase looked up from each amplitude's full index).
template <bool BWD, int MODE>
__device__ __forceinline__ void dfs_diag(const DfsSlots &S, const EOp &op, uint32_t base, const uint32_t (&bb)[4],
                                         const float4 *__restrict__ mats, bool tr, DAcc &a0, DAcc &a1) {
    if (MODE < 2) {
        const float4 e0 = mats[op.mat], e1 = mats[op.mat + 1];
        const float g0 = tr ? mats[op.gen].x : 0.0f, g1 = tr ? mats[op.gen + 1].x : 0.0f;
        const int b = op.sel & 3;
        const bool fixed_one = MODE == 1 && ((base >> (op.bits & 31u)) & 1u);
#pragma unroll 1
        for (int j = 0; j < kWinAmps; j += 2) {
            const bool o0 = MODE == 1 ? fixed_one : (bool)((j >> b) & 1);
            const bool o1 = MODE == 1 ? fixed_one : (bool)(((j + 1) >> b) & 1);
            dfs_diag1<BWD>(S, j, o0 ? e1 : e0, o0 ? g1 : g0, tr, a0);
            dfs_diag1<BWD>(S, j + 1, o1 ? e1 : e0, o1 ? g1 : g0, tr, a1);
        }
    } else {
        const bool parity = op.kind == EK_PARITY;
#pragma unroll 1
        for (int j = 0; j < kWinAmps; j += 2) {
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int jj = j + q;
                const uint32_t idx = base | ((jj & 1) ? bb[0] : 0) | ((jj & 2) ? bb[1] : 0) | ((jj & 4) ? bb[2] : 0) |
                                     ((jj & 8) ? bb[3] : 0);
                const uint32_t g = parity ? (uint32_t)(__popc(idx & op.bits) & 1) : diag_index(idx, op.bits, op.K);
                const float gd = tr ? (parity ? (g ? -1.0f : 1.0f) : mats[op.gen + g].x) : 0.0f;
                dfs_diag1<BWD>(S, jj, mats[op.mat + g], gd, tr, q ? a1 : a0);
            }
        }
    }
}

// Merged diagonal ops (EK_DIAGSET): amplitude j gets the product phase
// mats[op.mat + j].  All members' generators are diagonal, and the phases
// cancel in conj(h_j) v_j, so every trainable member's inner product is a
// signed sum of the same c_j = Im(conj(h_j) v_j): one product per amplitude
// for all members, then one addition per member.
template <bool BWD>
__device__ __forceinline__ void dfs_diagset(const DfsSlots &S, const EOp &op, const float4 *__restrict__ mats,
                                            float2 *part) {
    const int nm = BWD ? op.K : 0;
    DAcc a[4];
#pragma unroll
    for (int m = 0; m < 4; m++)
        if (m < nm) {
            const float2 p = part[((op.gen >> (4 * m)) & 15) * kWinThreadsDfs + S.tid];
            a[m].h = p.x;
            a[m].l = p.y;
        }
#pragma unroll 2
    for (int j = 0; j < kWinAmps; j++) {
        const float4 e = mats[op.mat + j];
        const CDF x = S.ld(S.L, j);
        if (BWD) {
            const CDF h = S.ld(S.M, j);
            if (nm > 0) {
                float ch, cl; // Im(conj(h) x) = h.re x.im - h.im x.re
                df_first(h.re.hi, h.re.lo, x.im.hi, x.im.lo, ch, cl);
                df_mac(-h.im.hi, -h.im.lo, x.re.hi, x.re.lo, ch, cl);
#pragma unroll
                for (int m = 0; m < 4; m++)
                    if (m < nm) {
                        const uint32_t mb = op.bits >> (8 * m);
                        const uint32_t code = ((j >> (mb & 3u)) & 1) ? (mb >> 4) & 3u : (mb >> 2) & 3u;
                        if (code) a[m].add(code == 1u ? DF{ch, cl} : DF{-ch, -cl});
                    }
            }
            S.st(S.M, j, cdf_mul(e, h));
        }
        S.st(S.L, j, cdf_mul(e, x));
    }
#pragma unroll
    for (int m = 0; m < 4; m++)
        if (m < nm) part[((op.gen >> (4 * m)) & 15) * kWinThreadsDfs + S.tid] = make_float2(a[m].h, a[m].l);
}

template <bool BWD>
__device__ __forceinline__ void dfs_window_op(const DfsSlots &S, const EOp &op, uint32_t base, const uint32_t (&bb)[4],
                                              const float4 *__restrict__ mats, DAcc &acc, DAcc &acc1, float2 *part) {
    const bool tr = BWD && op.red != 0xff;
    if (op.kind == EK_DIAGSET) {
        dfs_diagset<BWD>(S, op, mats, part);
    } else if (op.kind == EK_DENSE) {
        const float4 *U = mats + op.mat;
        if (op.K == 1) {
            const int b = op.sel & 3, form = op.sel >> 2;
            if (form == EF_RY) dfs_op1<BWD, 2>(S, b, U, tr, op.bits, acc, acc1);
            else if (form == EF_RX) dfs_op1<BWD, 1>(S, b, U, tr, op.bits, acc, acc1);
            else dfs_op1<BWD, 0>(S, b, U, tr, op.bits, acc, acc1);
        } else {
            // register bits of the op, one per byte (K = 2: the pair sel
            // enumerates 01 02 03 12 13 23; K = 3: sel is the missing bit)
            uint32_t rbits = 0x03020100u;
            if (op.K == 2) rbits = ((0x211000u >> (4 * op.sel)) & 15u) | (((0x332321u >> (4 * op.sel)) & 15u) << 8);
            else if (op.K == 3) rbits = op.sel == 0 ? 0x030201u : op.sel == 1 ? 0x030200u : op.sel == 2 ? 0x030100u
                                                                                                   : 0x020100u;
            const float4 *G = mats + (tr ? op.gen : 0);
            if (op.K == 2) acc = dfs_dense<2, BWD>(S, rbits, U, G, tr, acc);
            else if (op.K == 3) acc = dfs_dense<3, BWD>(S, rbits, U, G, tr, acc);
            else acc = dfs_dense<4, BWD>(S, rbits, U, G, tr, acc);
        }
    } else if (op.kind == EK_CX) {
        dfs_cx<BWD>(S, op.sel >> 2, op.sel & 3);
    } else if (op.kind == EK_DIAG && op.K == 1) {
        if (op.sel < 4) dfs_diag<BWD, 0>(S, op, base, bb, mats, tr, acc, acc1);
        else dfs_diag<BWD, 1>(S, op, base, bb, mats, tr, acc, acc1);
    } else {
        dfs_diag<BWD, 2>(S, op, base, bb, mats, tr, acc, acc1);
    }
}

// One window over the whole state (grid-stride over the 2^(n-4) groups).
// in_df / out_df: the state buffers hold raw double-float pairs on entry /
// on exit (between the windows of one sweep) instead of doubles.
template <bool BWD>
__global__ void __launch_bounds__(kWinThreadsDfs, BWD ? kDfsCtasBwd : kDfsCtasFwd)
    k_state_window_dfs(double2 *lam, double2 *hl, int nq, const EWin *__restrict__ wins, int wi,
                       const EOp *__restrict__ ops, const float4 *__restrict__ mats,
                       const ETrain *__restrict__ train, double *__restrict__ bpart, int in_df, int out_df) {
    extern __shared__ __align__(16) unsigned char dfs_smem[];
    const int tid = threadIdx.x;
    DfsSlots S;
    S.L = reinterpret_cast<float4 *>(dfs_smem);
    S.M = S.L + kWinAmps * kWinThreadsDfs;
    S.tid = tid;
    float2 *part = reinterpret_cast<float2 *>(S.L + (BWD ? 2 : 1) * kWinAmps * kWinThreadsDfs);
    const EWin w = wins[wi];
    if (BWD)
        for (int t = 0; t < w.ntrain; t++) part[t * kWinThreadsDfs + tid] = make_float2(0.0f, 0.0f);
    const uint32_t nu = 1u << (nq - kWinBits);
    const uint32_t bb[4] = {1u << w.rb[0], 1u << w.rb[1], 1u << w.rb[2], 1u << w.rb[3]};
    const uint32_t tstep = gridDim.x * kWinThreadsDfs;
    for (uint32_t u = blockIdx.x * kWinThreadsDfs + tid; u < nu; u += tstep) {
        uint32_t base = u;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t lo = base & (bb[i] - 1);
            base = ((base ^ lo) << 1) | lo;
        }
#pragma unroll
        for (int j = 0; j < kWinAmps; j++) {
            const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                 ((j & 8) ? bb[3] : 0);
            if (in_df) {
                S.L[j * kWinThreadsDfs + tid] = reinterpret_cast<const float4 *>(lam)[idx];
                if (BWD) S.M[j * kWinThreadsDfs + tid] = reinterpret_cast<const float4 *>(hl)[idx];
            } else {
                S.st(S.L, j, cdf_split(lam[idx]));
                if (BWD) S.st(S.M, j, cdf_split(hl[idx]));
            }
        }
        for (int k = 0; k < w.nops; k++) {
            const EOp op = ops[w.op0 + k];
            DAcc acc, acc1;
            if (BWD && op.red != 0xff) {
                const float2 p = part[op.red * kWinThreadsDfs + tid];
                acc.h = p.x;
                acc.l = p.y;
            }
            dfs_window_op<BWD>(S, op, base, bb, mats, acc, acc1, part);
            if (BWD && op.red != 0xff) {
                df_add(acc1.h, acc1.l, acc.h, acc.l);
                part[op.red * kWinThreadsDfs + tid] = make_float2(acc.h, acc.l);
            }
        }
#pragma unroll
        for (int j = 0; j < kWinAmps; j++) {
            const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                 ((j & 8) ? bb[3] : 0);
            if (out_df) {
                reinterpret_cast<float4 *>(lam)[idx] = S.L[j * kWinThreadsDfs + tid];
                if (BWD) reinterpret_cast<float4 *>(hl)[idx] = S.M[j * kWinThreadsDfs + tid];
            } else {
                const CDF v = S.ld(S.L, j);
                lam[idx] = make_double2(df_join(v.re.hi, v.re.lo), df_join(v.im.hi, v.im.lo));
                if (BWD) {
                    const CDF h = S.ld(S.M, j);
                    hl[idx] = make_double2(df_join(h.re.hi, h.re.lo), df_join(h.im.hi, h.im.lo));
                }
            }
        }
    }
    if (BWD && w.ntrain > 0) {
        __syncthreads();
        const int lane = tid & 31, warp = tid >> 5;
        for (int t = warp; t < w.ntrain; t += kWinThreadsDfs / 32) {
            EAcc<float> acc;
#pragma unroll
            for (int i = 0; i < kWinThreadsDfs / 32; i++) {
                const float2 p = part[t * kWinThreadsDfs + i * 32 + lane];
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
