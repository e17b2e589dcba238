// expval_diag.cuh — one-pass expectation values of PauliZ / Identity sets.
//
// Shared by the regular entry points (expval.cu) and the allocation-free one
// (noalloc.cu).
#pragma once

#include "df.cuh"
#include "reduce.cuh"

namespace plk {

// Diagonal observables in one pass: value v = sum_k |psi_k|^2 * sign_v(k) with
// sign_v(k) = (-1)^popcount(k & zmask_v) (Identity: zmask 0; PauliZ: one bit).
// A thread takes "quads" of amplitudes base + 32 j (j = 0..3, base with bits
// 5 and 6 clear), so each load instruction of a warp reads 32 consecutive
// amplitudes.  The four weights of a quad are combined once into the Walsh
// sums W[s] = sum_j (-1)^popcount(j & s) p_j; an observable then needs the
// parity of base & zmask and W[(zmask >> 5) & 3]: one add per observable per
// four amplitudes.  Loads of the next quads are issued before the current
// ones are evaluated.
template <class T> struct Quad {
    c2_t<T> v[4];
};

template <class T>
__device__ __forceinline__ void diag_load_quad(const c2_t<T> *__restrict__ sv, uint64_t n, uint64_t q, Quad<T> &d,
                                               uint64_t &base) {
    base = ((q >> 5) << 7) | (q & 31);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const uint64_t k = base + 32 * j;
        d.v[j] = k < n ? sv[k] : mk<c2_t<T>>(0, 0);
    }
}

// up to 16 Z masks, passed by value (no allocation or copy per call); the
// kernel reads them in place (__grid_constant__), with runtime indices
struct DiagMasks {
    uint64_t z[16];
};

template <class T, int NV>
__global__ void __launch_bounds__(kThreads)
    k_expval_diag(const c2_t<T> *__restrict__ sv, uint64_t n, const __grid_constant__ DiagMasks zmask, int nv,
                  double *partials, double *result, unsigned *counter) {
    constexpr int U = (sizeof(T) == 8 || NV >= 8) ? 1 : 2; // quads per batch (registers)
    __shared__ uint64_t zm[NV];
    __shared__ int zs[NV];
    for (int v = threadIdx.x; v < NV; v += blockDim.x) {
        const uint64_t z = v < nv ? zmask.z[v] : 0;
        zm[v] = z & ~(3ULL << 5);
        zs[v] = (int)((z >> 5) & 3);
    }
    __syncthreads();
    DAcc dacc[NV];
    const uint64_t nquads = ((n + 127) >> 7) << 5;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    Quad<T> cur[U];
    uint64_t cb[U];
    uint64_t q0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
    for (int u = 0; u < U; u++) diag_load_quad(sv, q0 + u * step < nquads ? n : 0, q0 + u * step, cur[u], cb[u]);
    for (; q0 < nquads; q0 += step * U) {
        Quad<T> nxt[U];
        uint64_t nb[U];
        const uint64_t q1 = q0 + step * U;
#pragma unroll
        for (int u = 0; u < U; u++) diag_load_quad(sv, q1 + u * step < nquads ? n : 0, q1 + u * step, nxt[u], nb[u]);
        if constexpr (sizeof(T) == 4) {
            // complex64: Walsh sums and signed partials in FP32, one
            // double-float add per observable per batch
            float t[NV];
#pragma unroll
            for (int w = 0; w < NV; w++) t[w] = 0.0f;
#pragma unroll
            for (int u = 0; u < U; u++) {
                float p[4];
#pragma unroll
                for (int j = 0; j < 4; j++) p[j] = fmaf(cur[u].v[j].x, cur[u].v[j].x, cur[u].v[j].y * cur[u].v[j].y);
                const float a = p[0] + p[1], b = p[0] - p[1], c = p[2] + p[3], d = p[2] - p[3];
                const float W0 = a + c, W1 = b + d, W2 = a - c, W3 = b - d;
#pragma unroll
                for (int w = 0; w < NV; w++) {
                    const int sel = zs[w];
                    const float val = sel == 0 ? W0 : (sel == 1 ? W1 : (sel == 2 ? W2 : W3));
                    t[w] += (__popcll(cb[u] & zm[w]) & 1) ? -val : val;
                }
            }
#pragma unroll
            for (int w = 0; w < NV; w++) dacc[w].add(DF{t[w], 0.0f});
        } else {
#pragma unroll
            for (int u = 0; u < U; u++) {
                DF p[4];
#pragma unroll
                for (int j = 0; j < 4; j++) p[j] = df_norm2(to_cdf(cur[u].v[j]));
                // Walsh sums in double-float
                float ah = p[0].hi, al = p[0].lo, bh = p[0].hi, bl = p[0].lo;
                df_add(p[1].hi, p[1].lo, ah, al);
                df_add(-p[1].hi, -p[1].lo, bh, bl);
                float ch = p[2].hi, cl = p[2].lo, dh = p[2].hi, dl = p[2].lo;
                df_add(p[3].hi, p[3].lo, ch, cl);
                df_add(-p[3].hi, -p[3].lo, dh, dl);
                float w0h = ah, w0l = al, w2h = ah, w2l = al, w1h = bh, w1l = bl, w3h = bh, w3l = bl;
                df_add(ch, cl, w0h, w0l);
                df_add(-ch, -cl, w2h, w2l);
                df_add(dh, dl, w1h, w1l);
                df_add(-dh, -dl, w3h, w3l);
#pragma unroll
                for (int w = 0; w < NV; w++) {
                    const int sel = zs[w];
                    float vh = sel == 0 ? w0h : (sel == 1 ? w1h : (sel == 2 ? w2h : w3h));
                    float vl = sel == 0 ? w0l : (sel == 1 ? w1l : (sel == 2 ? w2l : w3l));
                    if (__popcll(cb[u] & zm[w]) & 1) {
                        vh = -vh;
                        vl = -vl;
                    }
                    dacc[w].add(DF{vh, vl});
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            cur[u] = nxt[u];
            cb[u] = nb[u];
        }
    }
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] = dacc[v].value();
    block_reduce_finish<NV>(acc, partials, result, counter, 1.0, nv);
}

} // namespace plk
