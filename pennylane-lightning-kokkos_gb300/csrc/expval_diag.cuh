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

// ---------------------------------------------------------------------------
// Many single-wire PauliZ (and Identity) values in one pass, at a per-amplitude
// cost that does not grow with their number.
//
// <Z_b> = sum_k p_k (-1)^(bit b of k), p_k = |psi_k|^2.  A warp reads chunks of
// 32 * 2^M consecutive amplitudes: lane = index bits 0-4, step it = bits
// 5 .. 5+M-1, chunk number = the bits above.  Each lane sums its 2^M values
// as a binary tree whose level-l partial sums of odd blocks give
// S_l = sum over steps with bit l set, so the lane keeps, across chunks, its
// total and M sums S_l (about two additions per amplitude in all).  Then
//   lane bits (b < 5):      sum over lanes of (-1)^(bit b of lane) total;
//   step bits (5 <= b < 5+M): total - 2 S_(b-5);
//   chunk bits (b >= 5+M):  per chunk, the warp's chunk sum with the sign of
//                           the chunk's bit b, accumulated by the lane that
//                           owns the observable (lane v % 32);
//   Identity:               like a chunk bit that is never set.
// complex64 forms the tree in FP32 and accumulates chunk sums in
// double-float; complex128 works in double-float throughout.  Results are
// reduced in a fixed order (bitwise reproducible for a given grid).
struct ZBits {
    int8_t b[kMaxRedValues]; // state bit of value v, -1: Identity
};

template <class T> struct ZTree; // per-lane binary-tree sums of 2^M values

template <> struct ZTree<float> {
    __device__ __forceinline__ static DF p(float2 v) { return {fmaf(v.x, v.x, v.y * v.y), 0.0f}; }
    __device__ __forceinline__ static DF add(DF a, DF b) { return {a.hi + b.hi, 0.0f}; }
};
template <> struct ZTree<double> {
    __device__ __forceinline__ static DF p(double2 v) { return df_norm2(to_cdf(v)); }
    __device__ __forceinline__ static DF add(DF a, DF b) {
        df_add(b.hi, b.lo, a.hi, a.lo);
        return a;
    }
};

// Streaming loads issued in program order (asm volatile), so that a lane's
// loads of a chunk are all in flight before its first value is used.
__device__ __forceinline__ double2 ld_stream(const double2 *p) {
    double2 r;
    asm volatile("ld.global.nc.v2.f64 {%0, %1}, [%2];" : "=d"(r.x), "=d"(r.y) : "l"(p));
    return r;
}
__device__ __forceinline__ float2 ld_stream(const float2 *p) {
    float2 r;
    asm volatile("ld.global.nc.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "l"(p));
    return r;
}

template <class T, int M>
__global__ void __launch_bounds__(kThreads)
    k_expval_zbits(const c2_t<T> *__restrict__ sv, uint64_t n, const __grid_constant__ ZBits zb, int nv,
                   double *partials, double *result, unsigned *counter) {
    constexpr int STEPS = 1 << M;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int WPB = kThreads / 32;
    const uint64_t chunk_amps = (uint64_t)32 << M;
    const uint64_t nchunks = (n + chunk_amps - 1) / chunk_amps;
    const uint64_t wstep = (uint64_t)gridDim.x * WPB;
    // observables owned by this lane (chunk-bit and Identity values)
    const int b0 = lane < nv ? zb.b[lane] : -2, b1 = lane + 32 < nv ? zb.b[lane + 32] : -2;
    const bool own0 = b0 == -1 || b0 >= 5 + M, own1 = b1 == -1 || b1 >= 5 + M;
    DAcc tot, S[M], h0, h1;
    const bool whole = n >= chunk_amps; // every chunk lies inside the state
    for (uint64_t c = (uint64_t)blockIdx.x * WPB + warp; c < nchunks; c += wstep) {
        const uint64_t base = c * chunk_amps + lane;
        c2_t<T> v[STEPS];
        if (whole) {
            // all of the chunk's loads in flight before the first is used
#pragma unroll
            for (int i = 0; i < STEPS; i++) v[i] = ld_stream(sv + base + (uint64_t)i * 32);
        } else {
#pragma unroll
            for (int i = 0; i < STEPS; i++) {
                const uint64_t k = base + (uint64_t)i * 32;
                v[i] = k < n ? sv[k] : mk<c2_t<T>>(0, 0);
            }
        }
        // binary tree over the steps: pend[l] holds the open even block of level l
        DF pend[M + 1];
        DF Sc[M];
#pragma unroll
        for (int l = 0; l < M; l++) Sc[l] = {0.0f, 0.0f};
#pragma unroll
        for (int i = 0; i < STEPS; i++) {
            DF x = ZTree<T>::p(v[i]);
#pragma unroll
            for (int l = 0; l <= M; l++) {
                if (l == M || !((i >> l) & 1)) { // even block at level l (or the chunk total)
                    pend[l] = x;
                    break;
                }
                Sc[l] = ZTree<T>::add(Sc[l], x); // odd block: its sum counts toward S_l
                x = ZTree<T>::add(pend[l], x);
            }
        }
        const DF ct = pend[M]; // this lane's total over the chunk
        tot.add(ct);
#pragma unroll
        for (int l = 0; l < M; l++) S[l].add(Sc[l]);
        if (__any_sync(0xffffffffu, own0 || own1)) {
            // the warp's chunk sum, on every lane, in a fixed order
            float sh = ct.hi, sl = ct.lo;
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, sh, o);
                const float ol = __shfl_xor_sync(0xffffffffu, sl, o);
                df_add(oh, ol, sh, sl);
            }
            const uint64_t cb = c * chunk_amps;
            if (own0) {
                const bool neg = b0 >= 0 && ((cb >> b0) & 1);
                h0.add(neg ? DF{-sh, -sl} : DF{sh, sl});
            }
            if (own1) {
                const bool neg = b1 >= 0 && ((cb >> b1) & 1);
                h1.add(neg ? DF{-sh, -sl} : DF{sh, sl});
            }
        }
    }
    // per-warp values, then per-block partials, then the last block sums them
    __shared__ double sh[kMaxRedValues][WPB];
    __shared__ bool is_last;
    const double t = tot.value();
    double sv_l[M];
#pragma unroll
    for (int l = 0; l < M; l++) sv_l[l] = S[l].value();
    const double hv0 = h0.value(), hv1 = h1.value();
    for (int vi = 0; vi < nv; vi++) {
        const int b = zb.b[vi];
        double x;
        if (b == -1 || b >= 5 + M) {
            x = (vi < 32) ? (lane == vi ? hv0 : 0.0) : (lane == vi - 32 ? hv1 : 0.0);
        } else if (b < 5) {
            x = ((lane >> b) & 1) ? -t : t;
        } else {
            double s = sv_l[0];
#pragma unroll
            for (int l = 1; l < M; l++) s = (b - 5 == l) ? sv_l[l] : s;
            x = t - 2.0 * s;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) sh[vi][warp] = x;
    }
    __syncthreads();
    const int nblocks = gridDim.x;
    for (int vi = threadIdx.x; vi < nv; vi += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < WPB; w++) s += sh[vi][w];
        partials[(size_t)vi * nblocks + blockIdx.x] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = (atomicAdd(counter, 1u) == (unsigned)(nblocks - 1));
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    for (int vi = warp; vi < nv; vi += WPB) {
        double s = 0.0;
        for (int b = lane; b < nblocks; b += 32) s += __ldcg(partials + (size_t)vi * nblocks + b);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) result[vi] = s;
    }
    if (threadIdx.x == 0) *counter = 0u;
}

} // namespace plk
