// adjoint_kernels.cuh — the fused backward-step kernel of the adjoint
// Jacobian (see adjoint.cu), shared by the translation units that instantiate
// it for different gate kinds (adjoint.cu, adjoint_kinds2.cu) so that they
// compile in parallel.
#pragma once

#include <type_traits>

#include "df.cuh"
#include "gate_ops.cuh"
#include "reduce.cuh"

namespace plk {


enum AdjKind : int {
    A_RX = 0, A_RY, A_RZ, A_PS, A_CRX, A_CRY, A_CRZ, A_CPS, A_IXX, A_IXY, A_IYY, A_IZZ,
    A_SE, A_SEM, A_SEP, A_DE, A_DEM, A_DEP, A_MRZ, A_NONE
};

template <int KIND> __host__ __device__ constexpr int adj_K() {
    return KIND <= A_PS ? 1 : (KIND <= A_SEP ? 2 : (KIND <= A_DEP ? 4 : 0));
}

// Local indices where the gate or the generator acts.  Outside this set the
// gate is the identity and G lambda vanishes, so neither the update nor the
// inner product needs those amplitudes.
template <int KIND> __host__ __device__ constexpr uint32_t adj_touch() {
    switch (KIND) {
    case A_RX: case A_RY: case A_RZ: return 0x3u;
    case A_PS: return 0x2u;
    case A_CRX: case A_CRY: case A_CRZ: return 0xCu;
    case A_CPS: return 0x8u;
    case A_IXX: case A_IYY: case A_IZZ: case A_SEM: case A_SEP: return 0xFu;
    case A_IXY: case A_SE: return 0x6u;
    case A_DE: return (1u << 3) | (1u << 12);
    case A_DEM: case A_DEP: return 0xFFFFu;
    default: return 0x1u;
    }
}

template <class T> struct AdjArgs {
    Masks mk;
    uint64_t ngroups;
    uint64_t off[16];
    uint64_t mrz_mask;
    T g[8];  // gate (U^dag) coefficients
    T e[2];  // phase on the other amplitudes (+/- excitation gates)
    float gh[8], gl[8], eh[2], el[2]; // the same, split for the FP32-pipe complex128 path
};

// U^dag on the touched amplitudes (coefficients planned for adjoint = !inverse)
template <int KIND, class V, class T> __device__ __forceinline__ void adj_gate(V *v, const AdjArgs<T> &a) {
    if constexpr (KIND == A_RX) pair_op<P_RX>(v[0], v[1], a.g);
    else if constexpr (KIND == A_RY) pair_op<P_RY>(v[0], v[1], a.g);
    else if constexpr (KIND == A_RZ) pair_op<P_DIAG>(v[0], v[1], a.g);
    else if constexpr (KIND == A_PS) pair_op<P_PHASE_Y>(v[0], v[1], a.g);
    else if constexpr (KIND == A_CRX) pair_op<P_RX>(v[2], v[3], a.g);
    else if constexpr (KIND == A_CRY) pair_op<P_RY>(v[2], v[3], a.g);
    else if constexpr (KIND == A_CRZ) pair_op<P_DIAG>(v[2], v[3], a.g);
    else if constexpr (KIND == A_CPS) pair_op<P_PHASE_Y>(v[2], v[3], a.g);
    else if constexpr (KIND == A_IXX) {
        V q[4] = {v[0], v[1], v[2], v[3]};
        quad_op<Q_IXX>(q, a.g);
        for (int i = 0; i < 4; i++) v[i] = q[i];
    } else if constexpr (KIND == A_IYY) {
        V q[4] = {v[0], v[1], v[2], v[3]};
        quad_op<Q_IYY>(q, a.g);
        for (int i = 0; i < 4; i++) v[i] = q[i];
    } else if constexpr (KIND == A_IZZ) {
        V q[4] = {v[0], v[1], v[2], v[3]};
        quad_op<Q_DIAG>(q, a.g);
        for (int i = 0; i < 4; i++) v[i] = q[i];
    } else if constexpr (KIND == A_IXY) pair_op<P_RX>(v[1], v[2], a.g);
    else if constexpr (KIND == A_SE) pair_op<P_RY>(v[1], v[2], a.g);
    else if constexpr (KIND == A_SEM || KIND == A_SEP) {
        pair_op<P_RY>(v[1], v[2], a.g);
        v[0] = cmul(v[0], mk<V>(a.e[0], a.e[1]));
        v[3] = cmul(v[3], mk<V>(a.e[0], a.e[1]));
    } else if constexpr (KIND == A_DE) pair_op<P_RY>(v[3], v[12], a.g);
    else if constexpr (KIND == A_DEM || KIND == A_DEP) {
        pair_op<P_RY>(v[3], v[12], a.g);
#pragma unroll
        for (int i = 0; i < 16; i++)
            if (i != 3 && i != 12) v[i] = cmul(v[i], mk<V>(a.e[0], a.e[1]));
    }
}

// U^dag for complex128 on the FP32 pipe (double-float, see df.cuh)
template <int KIND> __device__ __forceinline__ void adj_gate_df(double2 *v, const AdjArgs<double> &a) {
    if constexpr (KIND == A_RX) pair_op_df<P_RX>(v[0], v[1], a.gh, a.gl);
    else if constexpr (KIND == A_RY) pair_op_df<P_RY>(v[0], v[1], a.gh, a.gl);
    else if constexpr (KIND == A_RZ) pair_op_df<P_DIAG>(v[0], v[1], a.gh, a.gl);
    else if constexpr (KIND == A_PS) pair_op_df<P_PHASE_Y>(v[0], v[1], a.gh, a.gl);
    else if constexpr (KIND == A_CRX) pair_op_df<P_RX>(v[2], v[3], a.gh, a.gl);
    else if constexpr (KIND == A_CRY) pair_op_df<P_RY>(v[2], v[3], a.gh, a.gl);
    else if constexpr (KIND == A_CRZ) pair_op_df<P_DIAG>(v[2], v[3], a.gh, a.gl);
    else if constexpr (KIND == A_CPS) pair_op_df<P_PHASE_Y>(v[2], v[3], a.gh, a.gl);
    else if constexpr (KIND == A_IXX || KIND == A_IYY || KIND == A_IZZ) {
        double2 q[4] = {v[0], v[1], v[2], v[3]};
        if constexpr (KIND == A_IXX) quad_op_df<Q_IXX>(q, a.gh, a.gl);
        else if constexpr (KIND == A_IYY) quad_op_df<Q_IYY>(q, a.gh, a.gl);
        else quad_op_df<Q_DIAG>(q, a.gh, a.gl);
        for (int i = 0; i < 4; i++) v[i] = q[i];
    } else if constexpr (KIND == A_IXY) pair_op_df<P_RX>(v[1], v[2], a.gh, a.gl);
    else if constexpr (KIND == A_SE) pair_op_df<P_RY>(v[1], v[2], a.gh, a.gl);
    else if constexpr (KIND == A_SEM || KIND == A_SEP) {
        pair_op_df<P_RY>(v[1], v[2], a.gh, a.gl);
        v[0] = df_cmul(a.eh, a.el, cdf_split(v[0]));
        v[3] = df_cmul(a.eh, a.el, cdf_split(v[3]));
    } else if constexpr (KIND == A_DE) pair_op_df<P_RY>(v[3], v[12], a.gh, a.gl);
    else if constexpr (KIND == A_DEM || KIND == A_DEP) {
        pair_op_df<P_RY>(v[3], v[12], a.gh, a.gl);
#pragma unroll
        for (int i = 0; i < 16; i++)
            if (i != 3 && i != 12) v[i] = df_cmul(a.eh, a.el, cdf_split(v[i]));
    }
}

// generator G on a copy (GateFunctors.hpp:2172-3132 and Pauli gates)
template <int KIND, class V> __device__ __forceinline__ void adj_gen(V *v) {
    const V Z = mk<V>(0, 0);
    if constexpr (KIND == A_RX) {
        V t = v[0]; v[0] = v[1]; v[1] = t;
    } else if constexpr (KIND == A_RY) {
        V t = v[0]; v[0] = mk<V>(v[1].y, -v[1].x); v[1] = mk<V>(-t.y, t.x);
    } else if constexpr (KIND == A_RZ) {
        v[1] = cneg(v[1]);
    } else if constexpr (KIND == A_PS) {
        v[0] = Z;
    } else if constexpr (KIND == A_CRX) {
        V t = v[2]; v[2] = v[3]; v[3] = t;
    } else if constexpr (KIND == A_CRY) {
        V t = v[2]; v[2] = mk<V>(v[3].y, -v[3].x); v[3] = mk<V>(-t.y, t.x);
    } else if constexpr (KIND == A_CRZ) {
        v[3] = cneg(v[3]);
    } else if constexpr (KIND == A_CPS) {
        // v[3] unchanged; v[0..2] are zero (outside the touched set)
    } else if constexpr (KIND == A_IXX) {
        V t = v[0]; v[0] = v[3]; v[3] = t;
        t = v[1]; v[1] = v[2]; v[2] = t;
    } else if constexpr (KIND == A_IYY) {
        const V v00 = v[0];
        v[0] = cneg(v[3]); v[3] = cneg(v00);
        V t = v[1]; v[1] = v[2]; v[2] = t;
    } else if constexpr (KIND == A_IZZ) {
        v[1] = cneg(v[1]); v[2] = cneg(v[2]);
    } else if constexpr (KIND == A_IXY) {
        V t = v[1]; v[1] = v[2]; v[2] = t;
    } else if constexpr (KIND == A_SE || KIND == A_SEM || KIND == A_SEP) {
        V t = v[1];
        v[1] = mk<V>(v[2].y, -v[2].x); // -i * old v10
        v[2] = mk<V>(-t.y, t.x);       //  i * old v01
        if constexpr (KIND == A_SEP) { v[0] = cneg(v[0]); v[3] = cneg(v[3]); }
        if constexpr (KIND == A_SEM) { /* v[0], v[3] unchanged */ }
    } else if constexpr (KIND == A_DE || KIND == A_DEM) {
        V t = v[3];
        v[3] = mk<V>(v[12].y, -v[12].x); // -i * v1100
        v[12] = mk<V>(-t.y, t.x);        //  i * v0011
    } else if constexpr (KIND == A_DEP) {
        V t = v[3];
        v[3] = mk<V>(-v[12].y, v[12].x); //  i * v1100
        v[12] = mk<V>(t.y, -t.x);        // -i * v0011
    }
}

constexpr int kAdjObsPerLaunch = 8;

template <class T, int KIND, int NV, bool DFP>
__global__ void __launch_bounds__(kThreads)
    k_adj_fused(c2_t<T> *__restrict__ lam, c2_t<T> *const *__restrict__ hl, int nobs, int write_lambda,
                const AdjArgs<T> a, double *partials, double *result, unsigned *counter, double post_scale) {
    using V = c2_t<T>;
    constexpr int K = adj_K<KIND>();
    constexpr int D = 1 << K;
    constexpr uint32_t TOUCH = adj_touch<KIND>();
    DAcc dacc[NV]; // Im <H lambda_o | G lambda> per thread, on the FP32 pipe
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.ngroups; g += step) {
        uint64_t base;
        V lv[D];
        if constexpr (KIND == A_MRZ) {
            base = g;
            lv[0] = lam[g];
        } else {
            base = group_base<K>(g, a.mk);
#pragma unroll
            for (int i = 0; i < D; i++)
                if (TOUCH & (1u << i)) lv[i] = lam[base + a.off[i]];
        }
        // mu = G lambda: the generators only move, negate, zero or multiply by
        // +-i, so this copy is exact in either precision
        CDF mu[D];
        {
            V m[D];
#pragma unroll
            for (int i = 0; i < D; i++) m[i] = lv[i];
            if constexpr (KIND == A_MRZ) {
                if (__popcll(g & a.mrz_mask) & 1) m[0] = cneg(m[0]);
            } else {
                adj_gen<KIND>(m);
            }
#pragma unroll
            for (int i = 0; i < D; i++)
                if (TOUCH & (1u << i)) mu[i] = to_cdf(m[i]);
        }
#pragma unroll
        for (int o = 0; o < NV; o++) {
            if (o < nobs) {
                V hv[D];
                if constexpr (KIND == A_MRZ) {
                    hv[0] = hl[o][g];
                } else {
#pragma unroll
                    for (int i = 0; i < D; i++)
                        if (TOUCH & (1u << i)) hv[i] = hl[o][base + a.off[i]];
                }
#pragma unroll
                for (int i = 0; i < D; i++)
                    if (TOUCH & (1u << i)) {
                        const CDF h = to_cdf(hv[i]);
                        dacc[o].mac(h.re, mu[i].im);
                        dacc[o].msub(h.im, mu[i].re);
                    }
                if constexpr (KIND == A_MRZ) {
                    const int odd = __popcll(g & a.mrz_mask) & 1;
                    if constexpr (DFP) hl[o][g] = df_cmul(a.gh + 2 * odd, a.gl + 2 * odd, cdf_split(hv[0]));
                    else hl[o][g] = odd ? cmul(hv[0], mk<V>(a.g[2], a.g[3])) : cmul(hv[0], mk<V>(a.g[0], a.g[1]));
                } else {
                    if constexpr (DFP) adj_gate_df<KIND>(hv, a);
                    else adj_gate<KIND>(hv, a);
#pragma unroll
                    for (int i = 0; i < D; i++)
                        if (TOUCH & (1u << i)) hl[o][base + a.off[i]] = hv[i];
                }
            }
        }
        if (write_lambda) {
            if constexpr (KIND == A_MRZ) {
                const int odd = __popcll(g & a.mrz_mask) & 1;
                if constexpr (DFP) lam[g] = df_cmul(a.gh + 2 * odd, a.gl + 2 * odd, cdf_split(lv[0]));
                else lam[g] = odd ? cmul(lv[0], mk<V>(a.g[2], a.g[3])) : cmul(lv[0], mk<V>(a.g[0], a.g[1]));
            } else {
                if constexpr (DFP) adj_gate_df<KIND>(lv, a);
                else adj_gate<KIND>(lv, a);
#pragma unroll
                for (int i = 0; i < D; i++)
                    if (TOUCH & (1u << i)) lam[base + a.off[i]] = lv[i];
            }
        }
    }
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] = dacc[v].value();
    block_reduce_finish<NV>(acc, partials, result, counter, post_scale, nobs);
}

template <class T, int KIND, bool DFP>
void launch_fused_dfp(plk_state lam, int grid, c2_t<T> *const *d_hl, int nobs, int write_lambda,
                             const AdjArgs<T> &a, double *result, double post_scale) {
    auto &w = lam->ws;
    auto *lp = (c2_t<T> *)lam->data;
    if (nobs <= 1)
        k_adj_fused<T, KIND, 1, DFP><<<grid, kThreads, 0, lam->stream>>>(lp, d_hl, nobs, write_lambda, a, w.d_partials,
                                                                        result, w.d_counter, post_scale);
    else if (nobs <= 2)
        k_adj_fused<T, KIND, 2, DFP><<<grid, kThreads, 0, lam->stream>>>(lp, d_hl, nobs, write_lambda, a, w.d_partials,
                                                                        result, w.d_counter, post_scale);
    else if (nobs <= 4)
        k_adj_fused<T, KIND, 4, DFP><<<grid, kThreads, 0, lam->stream>>>(lp, d_hl, nobs, write_lambda, a, w.d_partials,
                                                                        result, w.d_counter, post_scale);
    else
        k_adj_fused<T, KIND, 8, DFP><<<grid, kThreads, 0, lam->stream>>>(lp, d_hl, nobs, write_lambda, a, w.d_partials,
                                                                        result, w.d_counter, post_scale);
}

template <class T, int KIND>
int launch_fused_kind(plk_state lam, c2_t<T> *const *d_hl, int nobs, int write_lambda, const AdjArgs<T> &a,
                             double *result, double post_scale) {
    const int grid = red_grid(lam, a.ngroups);
    if constexpr (std::is_same_v<T, double>) {
        if (c128_use_df()) launch_fused_dfp<T, KIND, true>(lam, grid, d_hl, nobs, write_lambda, a, result, post_scale);
        else launch_fused_dfp<T, KIND, false>(lam, grid, d_hl, nobs, write_lambda, a, result, post_scale);
    } else {
        launch_fused_dfp<T, KIND, false>(lam, grid, d_hl, nobs, write_lambda, a, result, post_scale);
    }
    PLK_CHECK_LAUNCH();
    return PLK_OK;
}


// gate kinds whose launchers are instantiated in adjoint_kinds2.cu (two-wire
// kinds) and adjoint_kinds3.cu (four-wire and parity kinds)
#define PLK_ADJ_KINDS2(X) X(A_IXX) X(A_IXY) X(A_IYY) X(A_IZZ) X(A_SE) X(A_SEM) X(A_SEP)
#define PLK_ADJ_KINDS3(X) X(A_DE) X(A_DEM) X(A_DEP) X(A_MRZ)

} // namespace plk
