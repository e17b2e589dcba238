// expval.cu — expectation values, inner products, sparse products.
//
// Replaces ExpValFunctors.hpp, MeasuresKokkos::getExpectationValue*
// (simulator/MeasuresKokkos.hpp:80-346) and the reductions / SpMV of
// util/LinearAlgebraKokkos.hpp.  All reductions accumulate with FP64-class
// precision (double-float on the FP32 pipe, FP64 across blocks; the
// reference accumulates in the state precision) and are deterministic.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "df.cuh"
#include "gate_ops.cuh"
#include "reduce.cuh"
#include "expval_diag.cuh"

namespace plk {

int plan_gate(int gate, int nw, bool inv, const double *prm, int np, GatePlan &p);
int apply_matrix_impl(plk_state s, const double *matrix, const int64_t *wires, int nw, bool adj);

int fetch_results(plk_state s, int nv, double *out) {
    PLK_CUDA(cudaMemcpyAsync(s->ws.h_result, s->ws.d_result, sizeof(double) * nv, cudaMemcpyDeviceToHost, s->stream));
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    std::memcpy(out, s->ws.h_result, sizeof(double) * nv);
    return PLK_OK;
}

// ------------------------------------------------------------------ kernels --
// Named one-wire observables (ExpValFunctors.hpp:30-153) on the pair
// (i0, i1 = i0 | 2^b): X: 2 Re(conj v0 v1); Y: 2 Im(conj v0 v1);
// H: (|v0|^2 - |v1|^2 + 2 Re(conj v0 v1)) / sqrt 2.
enum NamedObs : int { OBS_X = 0, OBS_Y = 1, OBS_H = 2 };

template <class T, int OBS>
__global__ void __launch_bounds__(kThreads)
    k_expval_pair(const c2_t<T> *__restrict__ sv, uint64_t ngroups, uint64_t mask_lo, uint64_t bit, double *partials,
                  double *result, unsigned *counter) {
    // per-thread sums on the FP32 pipe (double-float), FP64 across the block
    DAcc a2; // X: Re(conj v0 v1); Y: Im(conj v0 v1); H: |v0|^2 - |v1|^2 + 2 Re(conj v0 v1)
    constexpr int U = 2;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g0 < ngroups; g0 += step * U) {
        c2_t<T> va[U], vb[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint64_t g = g0 + u * step;
            const uint64_t i0 = ((g & ~mask_lo) << 1) | (g & mask_lo);
            va[u] = g < ngroups ? sv[i0] : mk<c2_t<T>>(0, 0);
            vb[u] = g < ngroups ? sv[i0 | bit] : mk<c2_t<T>>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const CDF a = to_cdf(va[u]), b = to_cdf(vb[u]);
            if (OBS == OBS_X) {
                a2.mac(a.re, b.re);
                a2.mac(a.im, b.im);
            } else if (OBS == OBS_Y) {
                a2.mac(a.re, b.im);
                a2.msub(a.im, b.re);
            } else {
                a2.mac(a.re, a.re);
                a2.mac(a.im, a.im);
                a2.msub(b.re, b.re);
                a2.msub(b.im, b.im);
                const DF ar2 = {2.0f * a.re.hi, 2.0f * a.re.lo}, ai2 = {2.0f * a.im.hi, 2.0f * a.im.lo};
                a2.mac(ar2, b.re);
                a2.mac(ai2, b.im);
            }
        }
    }
    double acc[1] = {OBS == OBS_H ? 0.70710678118654752440 * a2.value() : 2.0 * a2.value()};
    block_reduce_finish<1>(acc, partials, result, counter);
}


// Re<psi| M |psi> for a matrix on K = 1, 2 or 3 wires (ExpValFunctors.hpp:155-250;
// MeasuresKokkos.hpp:318-346 for K >= 3).  Re<v|M|v> = <v|H|v> with the
// Hermitian part H = (M + M^dag)/2, so each group of 2^K amplitudes adds
//   sum_r H_rr |v_r|^2 + sum_{r<c} (a_rc Re(conj(v_r) v_c) + b_rc Im(conj(v_r) v_c))
// with a_rc = 2 Re H_rc, b_rc = -2 Im H_rc: about half the products of
// forming M v.  complex128 groups are evaluated in double-float on the FP32
// pipe, complex64 groups in FP32 (partial per group, then double-float).
template <int K> struct HermArgs {
    static constexpr int D = 1 << K, P = D * (D - 1) / 2;
    Masks mk;
    uint64_t ngroups;
    uint64_t off[D];
    float dh[D], dl[D];         // H_rr
    float ah[P], al[P], bh[P], bl[P];
    // complex128 packed form (herm_group_df2): per diagonal entry (d, d) and
    // per pair (a, b), each as {hi, -hi, -lo}
    f2x pd[D][3], pab[P][3];
};

// <v|H|v> of one complex128 group, real and imaginary lanes packed (df.cuh):
// the pair term (x, y) = (Re, Im-like) of conj(w_r) w_c is one packed
// double-float, weighted by (a, b); |w_r|^2 as the lanes (re^2, im^2)
// weighted by (d, d).  pa collects both lanes.
template <int K>
__device__ __forceinline__ void herm_group_df2(const double2 (&v)[1 << K], const HermArgs<K> &a, f2x &ph, f2x &pl) {
    constexpr int D = 1 << K;
    f2x vh[D], vl[D], nvh[D], nvl[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
        const CDF c = cdf_split(v[i]);
        vh[i] = f2x_pack(c.re.hi, c.im.hi);
        vl[i] = f2x_pack(c.re.lo, c.im.lo);
        nvh[i] = f2x_pack(-c.re.hi, -c.im.hi);
        nvl[i] = f2x_pack(-c.re.lo, -c.im.lo);
    }
#pragma unroll
    for (int r = 0; r < D; r++) {
        f2x nh, nl; // (re^2, im^2)
        df_first2n(vh[r], vl[r], vh[r], nvh[r], nvl[r], nh, nl);
        df_mac2(a.pd[r][0], a.pd[r][1], a.pd[r][2], nh, nl, ph, pl);
        float rh, ih, rl, il;
        f2x_unpack(vh[r], rh, ih);
        f2x_unpack(vl[r], rl, il);
        const f2x arh = f2x_pack(rh, rh), arl = f2x_pack(rl, rl); // (w_r.re, w_r.re)
        const f2x brh = f2x_pack(ih, -ih), brl = f2x_pack(il, -il); // (w_r.im, -w_r.im)
#pragma unroll
        for (int c = r + 1; c < D; c++) {
            const int P = r * D - r * (r + 1) / 2 + (c - r - 1); // index of (r, c) among r < c pairs
            // x = w_r.re w_c.re + w_r.im w_c.im, y = w_r.re w_c.im - w_r.im w_c.re
            f2x xh, xl;
            df_first2n(arh, arl, vh[c], nvh[c], nvl[c], xh, xl);
            df_mac2n(brh, brl, f2x_swap(vh[c]), f2x_swap(nvh[c]), f2x_swap(nvl[c]), xh, xl);
            df_mac2(a.pab[P][0], a.pab[P][1], a.pab[P][2], xh, xl, ph, pl);
        }
    }
}

template <class T, int K>
__global__ void __launch_bounds__(kThreads)
    k_expval_herm(const c2_t<T> *__restrict__ sv, const HermArgs<K> a, double *partials, double *result,
                  unsigned *counter) {
    constexpr int D = 1 << K;
    constexpr int UG = K == 1 ? 4 : (K == 2 ? 2 : 1); // groups in flight per thread
    DAcc acc;
    f2x ph = 0ull, pl = 0ull; // complex128: packed lanes (herm_group_df2)
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g0 < a.ngroups; g0 += step * UG) {
        c2_t<T> v[UG][D];
#pragma unroll
        for (int u = 0; u < UG; u++) {
            const uint64_t g = g0 + u * step;
            const uint64_t base = group_base<K>(g < a.ngroups ? g : 0, a.mk);
#pragma unroll
            for (int i = 0; i < D; i++) v[u][i] = g < a.ngroups ? sv[base + a.off[i]] : mk<c2_t<T>>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < UG; u++) {
            if constexpr (sizeof(T) == 4) {
                float t = 0.0f;
#pragma unroll
                for (int r = 0; r < D; r++) t = fmaf(a.dh[r], fmaf(v[u][r].x, v[u][r].x, v[u][r].y * v[u][r].y), t);
                int p = 0;
#pragma unroll
                for (int r = 0; r < D; r++)
#pragma unroll
                    for (int c = r + 1; c < D; c++, p++) {
                        const float x = fmaf(v[u][r].x, v[u][c].x, v[u][r].y * v[u][c].y);
                        const float y = fmaf(v[u][r].x, v[u][c].y, -v[u][r].y * v[u][c].x);
                        t = fmaf(a.ah[p], x, fmaf(a.bh[p], y, t));
                    }
                acc.add(DF{t, 0.0f});
            } else {
                herm_group_df2<K>(v[u], a, ph, pl);
            }
        }
    }
    if constexpr (sizeof(T) == 8) {
        float h0, h1, l0, l1;
        f2x_unpack(ph, h0, h1);
        f2x_unpack(pl, l0, l1);
        df_add(h0, l0, acc.h, acc.l);
        df_add(h1, l1, acc.h, acc.l);
    }
    double r[1] = {acc.value()};
    block_reduce_finish<1>(r, partials, result, counter);
}

// <x|y> = sum conj(x_k) y_k -> (re, im)
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_inner(const c2_t<T> *__restrict__ x, const c2_t<T> *__restrict__ y, uint64_t n, double *partials, double *result,
            unsigned *counter) {
    DAcc re, im;
    constexpr int U = 2;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += step * U) {
        c2_t<T> xa[U], ya[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint64_t k = k0 + u * step;
            xa[u] = k < n ? x[k] : mk<c2_t<T>>(0, 0);
            ya[u] = k < n ? y[k] : mk<c2_t<T>>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const CDF a = to_cdf(xa[u]), b = to_cdf(ya[u]);
            re.mac(a.re, b.re);
            re.mac(a.im, b.im);
            im.mac(a.re, b.im);
            im.msub(a.im, b.re);
        }
    }
    double acc[2] = {re.value(), im.value()};
    block_reduce_finish<2>(acc, partials, result, counter);
}

// CSR <psi|A|psi> (getExpectationValueSparseFunctor ExpValFunctors.hpp:252-280)
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_expval_csr(const c2_t<T> *__restrict__ sv, int64_t nrows, const double2 *__restrict__ data,
                 const int64_t *__restrict__ idx, const int64_t *__restrict__ ptr, double *partials, double *result,
                 unsigned *counter) {
    double acc[1] = {0.0};
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += step) {
        double tr = 0.0, ti = 0.0;
        for (int64_t j = ptr[r]; j < ptr[r + 1]; j++) {
            const double2 d = data[j];
            const c2_t<T> v = sv[idx[j]];
            tr += d.x * v.x - d.y * v.y;
            ti += d.x * v.y + d.y * v.x;
        }
        const c2_t<T> a = sv[r];
        acc[0] += (double)a.x * tr + (double)a.y * ti;
    }
    block_reduce_finish<1>(acc, partials, result, counter);
}

// y = A x (SparseMV_KokkosFunctor LinearAlgebraKokkos.hpp:68-104)
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_spmv(c2_t<T> *__restrict__ y, const c2_t<T> *__restrict__ x, int64_t nrows, const double2 *__restrict__ data,
           const int64_t *__restrict__ idx, const int64_t *__restrict__ ptr) {
    const int64_t step = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += step) {
        double tr = 0.0, ti = 0.0;
        for (int64_t j = ptr[r]; j < ptr[r + 1]; j++) {
            const double2 d = data[j];
            const c2_t<T> v = x[idx[j]];
            tr += d.x * v.x - d.y * v.y;
            ti += d.x * v.y + d.y * v.x;
        }
        y[r] = mk<c2_t<T>>((T)tr, (T)ti);
    }
}

// ---------------------------------------------------------- Pauli words --
// A Pauli word P acts as P|k> = i^ny (-1)^popcount(k & z) |k ^ x>, with x the
// X/Y positions, z the Y/Z positions, ny the number of Y letters.  Terms that
// share x form one group; a group costs one pass over the state.
struct PauliTerm {
    uint64_t z;
    double cr, ci;           // c_j * i^ny
    float crh, crl, cih, cil; // the same, split for the FP32-pipe accumulation
};

struct PauliGroup {
    uint64_t x;
    int first, count;
};

static int build_pauli_groups(plk_state s, int nterms, const double *coeffs, const int64_t *offsets,
                              const int64_t *wires, const char *paulis, std::vector<PauliGroup> &groups,
                              std::vector<PauliTerm> &terms) {
    if (nterms < 0 || (nterms > 0 && (!coeffs || !offsets))) PLK_FAIL(PLK_ERR_INVALID_ARG, "bad Pauli-sum arguments");
    std::map<uint64_t, std::vector<PauliTerm>> by_x;
    for (int t = 0; t < nterms; t++) {
        uint64_t x = 0, z = 0;
        int ny = 0;
        const int64_t b = offsets[t], e = offsets[t + 1];
        if (e < b) PLK_FAIL(PLK_ERR_INVALID_ARG, "Pauli-sum offsets must be non-decreasing");
        for (int64_t j = b; j < e; j++) {
            if (wires[j] < 0 || wires[j] >= s->nq) PLK_FAIL(PLK_ERR_INVALID_ARG, "Pauli word wire out of range");
            const uint64_t bit = 1ULL << (s->nq - 1 - wires[j]);
            if ((x | z) & bit) PLK_FAIL(PLK_ERR_INVALID_ARG, "repeated wire in a Pauli word");
            switch (paulis[j]) {
            case 'I': break;
            case 'X': x |= bit; break;
            case 'Y': x |= bit; z |= bit; ny++; break;
            case 'Z': z |= bit; break;
            default: PLK_FAIL(PLK_ERR_INVALID_ARG, std::string("bad Pauli letter ") + paulis[j]);
            }
        }
        // c * i^ny
        double cr = coeffs[t], ci = 0.0;
        for (int k = 0; k < (ny & 3); k++) {
            const double nr = -ci, ni = cr;
            cr = nr;
            ci = ni;
        }
        PauliTerm pt{z, cr, ci, 0, 0, 0, 0};
        df_split_host(cr, pt.crh, pt.crl);
        df_split_host(ci, pt.cih, pt.cil);
        by_x[x].push_back(pt);
    }
    groups.clear();
    terms.clear();
    for (auto &kv : by_x) {
        PauliGroup g{kv.first, (int)terms.size(), (int)kv.second.size()};
        for (auto &t : kv.second) terms.push_back(t);
        groups.push_back(g);
    }
    return PLK_OK;
}

// <psi| sum_{t in group} c_t P_t |psi> for one x-group.  For x != 0 the pairs
// (m, m ^ x) with bit p (the top bit of x) clear are visited once:
//   conj(psi_m) psi_m' f(m') + conj(psi_m') psi_m f(m),
//   f(q) = sum_t c_t i^ny (-1)^popcount(q & z_t).
// contribution of the pair (m, mp = m ^ x) to <psi|sum c_t P_t|psi> (complex64:
// formed in FP32, returned for a double-float add)
__device__ __forceinline__ float pauli_pair_f32(float2 a, float2 b, uint64_t m, uint64_t mp,
                                                const PauliTerm *__restrict__ st, int nt) {
    float f1 = 0.0f, f2 = 0.0f;
    for (int t = 0; t < nt; t++) {
        const PauliTerm tt = st[t];
        const bool s1 = __popcll(mp & tt.z) & 1, s0 = __popcll(m & tt.z) & 1;
        if (s1 == s0) f1 += s0 ? -2.0f * tt.crh : 2.0f * tt.crh;
        else f2 += s0 ? -2.0f * tt.cih : 2.0f * tt.cih;
    }
    const float re = fmaf(a.x, b.x, a.y * b.y), im = fmaf(a.x, b.y, -a.y * b.x);
    return fmaf(re, f1, im * f2);
}

// complex128: the same in double-float, added to `total`
__device__ __forceinline__ void pauli_pair_df(double2 ra, double2 rb, uint64_t m, uint64_t mp,
                                              const PauliTerm *__restrict__ st, int nt, DAcc &total) {
    const CDF a = to_cdf(ra), b = to_cdf(rb);
    // F1 = Re f(m') + Re f(m), F2 = Im f(m) - Im f(m')
    DAcc f1, f2;
    for (int t = 0; t < nt; t++) {
        const PauliTerm tt = st[t];
        const bool s1 = __popcll(mp & tt.z) & 1, s0 = __popcll(m & tt.z) & 1;
        if (s1 == s0) {
            const DF c = {2.0f * tt.crh, 2.0f * tt.crl};
            if (s0) f1.sub(c);
            else f1.add(c);
        } else {
            const DF c = {2.0f * tt.cih, 2.0f * tt.cil};
            if (s0) f2.sub(c); // s0 set: -ci from f(m), s1 clear: +ci from -f(m')
            else f2.add(c);
        }
    }
    DAcc ab_re, ab_im; // conj(a) b
    ab_re.mac(a.re, b.re);
    ab_re.mac(a.im, b.im);
    ab_im.mac(a.re, b.im);
    ab_im.msub(a.im, b.re);
    total.mac(ab_re.normalized(), f1.normalized());
    total.mac(ab_im.normalized(), f2.normalized());
}

__device__ __forceinline__ float pauli_diag_f32(float2 a, uint64_t k, const PauliTerm *__restrict__ st, int nt) {
    float f = 0.0f;
    for (int t = 0; t < nt; t++) f += (__popcll(k & st[t].z) & 1) ? -st[t].crh : st[t].crh;
    return fmaf(a.x, a.x, a.y * a.y) * f;
}

__device__ __forceinline__ void pauli_diag_df(double2 ra, uint64_t k, const PauliTerm *__restrict__ st, int nt,
                                              DAcc &total) {
    const DF p = df_norm2(to_cdf(ra));
    DAcc f;
    for (int t = 0; t < nt; t++) {
        const DF c = {st[t].crh, st[t].crl};
        if (__popcll(k & st[t].z) & 1) f.sub(c);
        else f.add(c);
    }
    total.mac(p, f.normalized());
}

// <psi| sum_{t in group} c_t P_t |psi> for one x-group.  For x != 0 the pairs
// (m, m ^ x) with bit p (the top bit of x) clear are visited once:
//   conj(psi_m) psi_m' f(m') + conj(psi_m') psi_m f(m),
//   f(q) = sum_t c_t i^ny (-1)^popcount(q & z_t).
// Software-pipelined: the loads of the next kPauliBatch items are issued
// before the current batch is evaluated, so every thread keeps loads in
// flight while it computes.
constexpr int kPauliBatch = 4;

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_expval_pauli(const c2_t<T> *__restrict__ sv, uint64_t n, uint64_t x, uint64_t pmask_lo,
                   const PauliTerm *__restrict__ terms, int nt, double *partials, double *result, unsigned *counter) {
    using V = c2_t<T>;
    constexpr int U = sizeof(T) == 8 ? kPauliBatch / 2 : kPauliBatch;
    extern __shared__ PauliTerm sterm[];
    for (int i = threadIdx.x; i < nt; i += blockDim.x) sterm[i] = terms[i];
    __syncthreads();
    DAcc total;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t items = x == 0 ? n : (n >> 1);
    const V zero = mk<V>(0, 0);
    // One-term group with x != 0 (most Pauli words): the parities of m and
    // m ^ x under z differ exactly when x & z has odd parity, so only
    // Re(conj(a) b) (even) or only Im(conj(a) b) (odd) contributes, with
    // coefficient 2 cr or 2 ci signed by the parity of m & z.  complex128
    // forms that product of the pair in native FP64 (two FP64 instructions
    // per pair, inside the FP64 pipe's budget at HBM speed) and accumulates
    // it in double-float.
    const bool single = nt == 1 && x != 0;
    const uint64_t z1 = sterm[0].z;
    const bool px = single && (__popcll(x & z1) & 1);
    const float cf = px ? 2.0f * sterm[0].cih : 2.0f * sterm[0].crh;
    const DF cd = px ? DF{2.0f * sterm[0].cih, 2.0f * sterm[0].cil} : DF{2.0f * sterm[0].crh, 2.0f * sterm[0].crl};
    // item g -> (m, m ^ x); for x == 0, m = g
    auto first_of = [&](uint64_t g) { return x == 0 ? g : (((g & ~pmask_lo) << 1) | (g & pmask_lo)); };
    V a[U], b[U];
    uint64_t g0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
#pragma unroll
    for (int u = 0; u < U; u++) {
        const uint64_t g = g0 + u * step;
        const uint64_t m = first_of(g);
        a[u] = g < items ? sv[m] : zero;
        b[u] = (x != 0 && g < items) ? sv[m ^ x] : zero;
    }
    for (; g0 < items; g0 += step * U) {
        V na[U], nb[U];
        const uint64_t g1 = g0 + step * U;
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint64_t g = g1 + u * step;
            const uint64_t m = first_of(g);
            na[u] = g < items ? sv[m] : zero;
            nb[u] = (x != 0 && g < items) ? sv[m ^ x] : zero;
        }
        if (single) {
            // items past the end hold zero amplitudes: they add nothing.
            // px is uniform: one branch around the batch, so only the needed
            // product is formed (complex128: two FP64 instructions per pair)
            float t = 0.0f;
            V pa[U], pb[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                // Im(conj(a) b) = Re(conj(a) (-i b)): rotate b once when px
                pa[u] = a[u];
                pb[u] = px ? mk<V>(b[u].y, -b[u].x) : b[u];
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const uint64_t m = first_of(g0 + u * step);
                const bool neg = __popcll(m & z1) & 1;
                if constexpr (sizeof(T) == 4) {
                    const float v = fmaf(pa[u].x, pb[u].x, pa[u].y * pb[u].y);
                    t = fmaf(neg ? -cf : cf, v, t);
                } else {
                    const double v = fma(pa[u].x, pb[u].x, pa[u].y * pb[u].y);
                    total.mac(neg ? DF{-cd.hi, -cd.lo} : cd, df_split(v));
                }
            }
            if constexpr (sizeof(T) == 4) total.add(DF{t, 0.0f});
        } else {
#pragma unroll
            for (int u = 0; u < U; u++) {
                const uint64_t g = g0 + u * step;
                if (g >= items) break;
                const uint64_t m = first_of(g);
                if constexpr (sizeof(T) == 4) {
                    const float c = x == 0 ? pauli_diag_f32(a[u], m, sterm, nt)
                                           : pauli_pair_f32(a[u], b[u], m, m ^ x, sterm, nt);
                    total.add(DF{c, 0.0f});
                } else {
                    if (x == 0) pauli_diag_df(a[u], m, sterm, nt, total);
                    else pauli_pair_df(a[u], b[u], m, m ^ x, sterm, nt, total);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            a[u] = na[u];
            b[u] = nb[u];
        }
    }
    double acc[1] = {total.value()};
    block_reduce_finish<1>(acc, partials, result, counter);
}

// out_m (+)= sum_{groups g} sum_{t in g} c_t i^ny (-1)^popcount((m^x_g) & z_t) in_{m ^ x_g}
constexpr int kPauliGroupsPerPass = 32;
struct PauliPass {
    uint64_t x[kPauliGroupsPerPass];
    int first[kPauliGroupsPerPass];
    int count[kPauliGroupsPerPass];
    int ngroups;
    int accumulate;
};

// out[m] (+)= sum over groups g of f_g(src) in[src], src = m ^ x_g, with
// f_g(src) = sum_t c_t i^ny_t (-1)^popc(src & z_t).  complex64 states in FP32
// (the result is stored in FP32); complex128 on the FP32 pipe in
// double-float, rounded once to FP64.
// f_g(src) = sum over the group's terms of c_t i^ny (-1)^popc(src & z_t), as
// double-floats; a one-term group needs no accumulation
__device__ __forceinline__ void pauli_coef_df(const PauliTerm *__restrict__ tp, int first, int count, uint64_t src,
                                              DF &f_re, DF &f_im) {
    if (count == 1) {
        const PauliTerm &tt = tp[first];
        const bool neg = __popcll(src & tt.z) & 1;
        f_re = neg ? DF{-tt.crh, -tt.crl} : DF{tt.crh, tt.crl};
        f_im = neg ? DF{-tt.cih, -tt.cil} : DF{tt.cih, tt.cil};
        return;
    }
    DAcc fr, fi;
    for (int t = first; t < first + count; t++) {
        const PauliTerm &tt = tp[t];
        if (__popcll(src & tt.z) & 1) {
            fr.sub(DF{tt.crh, tt.crl});
            fi.sub(DF{tt.cih, tt.cil});
        } else {
            fr.add(DF{tt.crh, tt.crl});
            fi.add(DF{tt.cih, tt.cil});
        }
    }
    f_re = fr.normalized();
    f_im = fi.normalized();
}

// out[m] (+)= sum over groups g of f_g(src) in[src], src = m ^ x_g.  complex64
// states in FP32 (the result is stored in FP32); complex128 on the FP32 pipe
// in double-float.  The pass's terms sit in shared memory (tp = sterm, term
// indices relative to t_lo) when they fit, else are read from global memory.
// A block owns a tile of 2048 consecutive outputs (8 per thread, kept in
// registers) and walks the groups in order: for each group the block reads
// one contiguous source tile (the output tile with x's high bits flipped,
// permuted inside by x's low bits), with eight loads in flight per thread.
constexpr int kPauliPerThread = 8;
constexpr int kPauliTile = kThreads * kPauliPerThread;

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_apply_pauli(c2_t<T> *__restrict__ out, const c2_t<T> *__restrict__ in, uint64_t n,
                  const PauliTerm *__restrict__ terms, const PauliPass pass, int t_lo, int t_cnt, int terms_in_smem) {
    using V = c2_t<T>;
    constexpr int P = kPauliPerThread;
    extern __shared__ PauliTerm sterm[];
    if (terms_in_smem) {
        for (int i = threadIdx.x; i < t_cnt; i += blockDim.x) sterm[i] = terms[t_lo + i];
        __syncthreads();
    }
    const PauliTerm *tp = terms_in_smem ? sterm : terms + t_lo;
    const int ng = pass.ngroups;
    const uint64_t ntiles = (n + kPauliTile - 1) / kPauliTile;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t m0 = tile * kPauliTile + threadIdx.x;
        // accumulators: complex64 in FP32, complex128 in double-float
        float ar[P], ai[P];
        DAcc dr[P], di[P];
#pragma unroll
        for (int i = 0; i < P; i++) {
            const uint64_t m = m0 + (uint64_t)i * kThreads;
            const V o = (pass.accumulate && m < n) ? out[m] : mk<V>(0, 0);
            if constexpr (sizeof(T) == 4) {
                ar[i] = o.x;
                ai[i] = o.y;
            } else {
                const CDF oc = to_cdf(o);
                dr[i].add(oc.re);
                di[i].add(oc.im);
            }
        }
        for (int gi = 0; gi < ng; gi++) {
            const uint64_t x = pass.x[gi];
            // m0 has bits 8-10 clear, so source i is (m0 ^ x) ^ (i << 8)
            const uint64_t y = m0 ^ x;
            V v[P];
#pragma unroll
            for (int i = 0; i < P; i++) {
                const uint64_t m = m0 + (uint64_t)i * kThreads;
                v[i] = m < n ? in[y ^ ((uint64_t)i << 8)] : mk<V>(0, 0);
            }
            const int first = pass.first[gi] - t_lo, count = pass.count[gi];
            const bool one_term = count == 1 && ((tp[first].cih == 0.0f && tp[first].cil == 0.0f) ||
                                                 (tp[first].crh == 0.0f && tp[first].crl == 0.0f));
            if (one_term) {
                // one term: f = (-1)^popcount(src & z) c with c real or
                // imaginary; popcount(src & z) = popcount(y & z) + that of
                // (i << 8) & z
                const PauliTerm &tt = tp[first];
                const uint32_t zi = (uint32_t)(tt.z >> 8) & 7u;
                const bool py = __popcll(y & tt.z) & 1;
                const bool is_real = tt.cih == 0.0f && tt.cil == 0.0f;
#pragma unroll
                for (int i = 0; i < P; i++) {
                    const bool neg = py ^ (__popc((uint32_t)i & zi) & 1);
                    if constexpr (sizeof(T) == 4) {
                        const float c = is_real ? tt.crh : tt.cih;
                        const float cs = neg ? -c : c;
                        if (is_real) {
                            ar[i] = fmaf(cs, v[i].x, ar[i]);
                            ai[i] = fmaf(cs, v[i].y, ai[i]);
                        } else { // i c v: (-c v.y, c v.x)
                            ar[i] = fmaf(-cs, v[i].y, ar[i]);
                            ai[i] = fmaf(cs, v[i].x, ai[i]);
                        }
                    } else {
                        const CDF c = to_cdf(v[i]);
                        const DF k = is_real ? DF{tt.crh, tt.crl} : DF{tt.cih, tt.cil};
                        const DF ks = neg ? DF{-k.hi, -k.lo} : k;
                        if (is_real) {
                            dr[i].mac(ks, c.re);
                            di[i].mac(ks, c.im);
                        } else {
                            dr[i].msub(ks, c.im);
                            di[i].mac(ks, c.re);
                        }
                    }
                }
                continue;
            }
#pragma unroll
            for (int i = 0; i < P; i++) {
                const uint64_t src = (m0 + (uint64_t)i * kThreads) ^ x;
                if constexpr (sizeof(T) == 4) {
                    float fr = 0.0f, fi = 0.0f;
                    for (int t = first; t < first + count; t++) {
                        const bool neg = __popcll(src & tp[t].z) & 1;
                        fr += neg ? -tp[t].crh : tp[t].crh;
                        fi += neg ? -tp[t].cih : tp[t].cih;
                    }
                    ar[i] = fmaf(fr, v[i].x, fmaf(-fi, v[i].y, ar[i]));
                    ai[i] = fmaf(fr, v[i].y, fmaf(fi, v[i].x, ai[i]));
                } else {
                    const CDF c = to_cdf(v[i]);
                    DF f_re, f_im;
                    pauli_coef_df(tp, first, count, src, f_re, f_im);
                    dr[i].mac(f_re, c.re);
                    dr[i].msub(f_im, c.im);
                    di[i].mac(f_re, c.im);
                    di[i].mac(f_im, c.re);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < P; i++) {
            const uint64_t m = m0 + (uint64_t)i * kThreads;
            if (m >= n) continue;
            if constexpr (sizeof(T) == 4) out[m] = make_float2(ar[i], ai[i]);
            else out[m] = make_double2(dr[i].value(), di[i].value());
        }
    }
}

// --------------------------------------------------------------- helpers --
template <class T>
static int expval_named_impl(plk_state s, int gate, int64_t wire, double *out) {
    const int b = s->nq - 1 - (int)wire;
    const uint64_t bit = 1ULL << b, mask_lo = bit - 1;
    const uint64_t ng = s->length >> 1;
    const int grid = red_grid(s, ng);
    auto *sv = (const c2_t<T> *)s->data;
    auto &w = s->ws;
    switch (gate) {
    case PLK_GATE_PAULIX:
        k_expval_pair<T, OBS_X><<<grid, kThreads, 0, s->stream>>>(sv, ng, mask_lo, bit, w.d_partials, w.d_result, w.d_counter);
        break;
    case PLK_GATE_PAULIY:
        k_expval_pair<T, OBS_Y><<<grid, kThreads, 0, s->stream>>>(sv, ng, mask_lo, bit, w.d_partials, w.d_result, w.d_counter);
        break;
    case PLK_GATE_HADAMARD:
        k_expval_pair<T, OBS_H><<<grid, kThreads, 0, s->stream>>>(sv, ng, mask_lo, bit, w.d_partials, w.d_result, w.d_counter);
        break;
    default: PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "internal: bad named observable");
    }
    PLK_CHECK_LAUNCH();
    return fetch_results(s, 1, out);
}

template <class T, int NV> static void launch_diag(plk_state s, const DiagMasks &dm, int nv) {
    auto &w = s->ws;
    const int grid = red_grid_k(s, k_expval_diag<T, NV>, ((s->length + 127) >> 7) << 5);
    k_expval_diag<T, NV><<<grid, kThreads, 0, s->stream>>>((const c2_t<T> *)s->data, s->length, dm, nv, w.d_partials,
                                                          w.d_result, w.d_counter);
}

// Single-wire PauliZ / Identity values, up to kMaxRedValues per pass, at a
// per-amplitude cost independent of their number (k_expval_zbits).
template <class T> static int expval_zbits_impl(plk_state s, const std::vector<uint64_t> &zmasks, double *out) {
    constexpr int M = sizeof(T) == 4 ? 5 : 4; // steps per lane per chunk: 2^M
    const int total = (int)zmasks.size();
    auto &w = s->ws;
    const uint64_t chunks = (s->length + ((uint64_t)32 << M) - 1) / ((uint64_t)32 << M);
    // one warp per chunk: work items are the chunks' warps' threads
    const int grid = red_grid_k(s, k_expval_zbits<T, M>, chunks * 32);
    for (int start = 0; start < total; start += kMaxRedValues) {
        const int nv = std::min(kMaxRedValues, total - start);
        ZBits zb;
        for (int v = 0; v < nv; v++) {
            const uint64_t z = zmasks[start + v];
            zb.b[v] = z ? (int8_t)__builtin_ctzll(z) : (int8_t)-1;
        }
        k_expval_zbits<T, M><<<grid, kThreads, 0, s->stream>>>((const c2_t<T> *)s->data, s->length, zb, nv,
                                                               w.d_partials, w.d_result, w.d_counter);
        PLK_CHECK_LAUNCH();
        PLK_TRY(fetch_results(s, nv, out + start));
    }
    return PLK_OK;
}

// Diagonal (Identity / PauliZ) observables: single-wire masks through
// k_expval_zbits; masks of several bits up to 16 per pass (k_expval_diag).
template <class T> static int expval_diag_impl(plk_state s, const std::vector<uint64_t> &zmasks, double *out) {
    bool single = true;
    for (uint64_t z : zmasks) single = single && (z & (z - 1)) == 0;
    if (single) return expval_zbits_impl<T>(s, zmasks, out);
    const int total = (int)zmasks.size();
    for (int start = 0; start < total; start += 16) {
        const int nv = std::min(16, total - start);
        DiagMasks dm{};
        for (int v = 0; v < nv; v++) dm.z[v] = zmasks[start + v];
        if (nv == 1) launch_diag<T, 1>(s, dm, nv);
        else if (nv == 2) launch_diag<T, 2>(s, dm, nv);
        else if (nv <= 4) launch_diag<T, 4>(s, dm, nv);
        else if (nv <= 8) launch_diag<T, 8>(s, dm, nv);
        else launch_diag<T, 16>(s, dm, nv);
        PLK_CHECK_LAUNCH();
        PLK_TRY(fetch_results(s, nv, out + start));
    }
    return PLK_OK;
}

template <class T, int K>
static int expval_herm_impl(plk_state s, const double *matrix, const int64_t *wires, double *out) {
    constexpr int D = 1 << K;
    HermArgs<K> a;
    std::memset(&a, 0, sizeof(a));
    int rev[K], srt[K];
    for (int j = 0; j < K; j++) rev[j] = s->nq - 1 - (int)wires[j];
    std::copy(rev, rev + K, srt);
    std::sort(srt, srt + K);
    a.mk = make_masks(srt, K);
    a.ngroups = s->length >> K;
    for (int i = 0; i < D; i++)
        for (int j = 0; j < K; j++)
            if ((i >> (K - 1 - j)) & 1) a.off[i] |= 1ULL << rev[j];
    // Hermitian part H = (M + M^dag)/2 of the row-major complex matrix
    auto re = [&](int r, int c) { return matrix[2 * (r * D + c)]; };
    auto im = [&](int r, int c) { return matrix[2 * (r * D + c) + 1]; };
    for (int r = 0; r < D; r++) df_split_host(re(r, r), a.dh[r], a.dl[r]);
    int p = 0;
    for (int r = 0; r < D; r++)
        for (int c = r + 1; c < D; c++, p++) {
            const double hre = 0.5 * (re(r, c) + re(c, r)), him = 0.5 * (im(r, c) - im(c, r));
            df_split_host(2.0 * hre, a.ah[p], a.al[p]);
            df_split_host(-2.0 * him, a.bh[p], a.bl[p]);
        }
    // packed pairs {(x0, x1), -(x0, x1) hi, -(x0, x1) lo} for herm_group_df2
    auto bits = [](float f) {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        return (f2x)u;
    };
    auto pack = [&](float l0, float l1) { return bits(l0) | (bits(l1) << 32); };
    for (int r = 0; r < D; r++) {
        a.pd[r][0] = pack(a.dh[r], a.dh[r]);
        a.pd[r][1] = pack(-a.dh[r], -a.dh[r]);
        a.pd[r][2] = pack(-a.dl[r], -a.dl[r]);
    }
    for (int q = 0; q < p; q++) {
        a.pab[q][0] = pack(a.ah[q], a.bh[q]);
        a.pab[q][1] = pack(-a.ah[q], -a.bh[q]);
        a.pab[q][2] = pack(-a.al[q], -a.bl[q]);
    }
    const int grid = red_grid_k(s, k_expval_herm<T, K>, a.ngroups);
    auto &w = s->ws;
    k_expval_herm<T, K><<<grid, kThreads, 0, s->stream>>>((const c2_t<T> *)s->data, a, w.d_partials, w.d_result,
                                                          w.d_counter);
    PLK_CHECK_LAUNCH();
    return fetch_results(s, 1, out);
}

template <class T> static int expval_herm_any(plk_state s, const double *matrix, const int64_t *wires, int K,
                                              double *out) {
    switch (K) {
    case 1: return expval_herm_impl<T, 1>(s, matrix, wires, out);
    case 2: return expval_herm_impl<T, 2>(s, matrix, wires, out);
    default: return expval_herm_impl<T, 3>(s, matrix, wires, out);
    }
}

template <class T> static int inner_impl(plk_state x, plk_state y, double *re, double *im) {
    const int grid = red_grid_k(x, k_inner<T>, x->length);
    auto &w = x->ws;
    k_inner<T><<<grid, kThreads, 0, x->stream>>>((const c2_t<T> *)x->data, (const c2_t<T> *)y->data, x->length,
                                                 w.d_partials, w.d_result, w.d_counter);
    PLK_CHECK_LAUNCH();
    double r[2];
    PLK_TRY(fetch_results(x, 2, r));
    if (re) *re = r[0];
    if (im) *im = r[1];
    return PLK_OK;
}

struct CsrDev {
    double2 *data = nullptr;
    int64_t *idx = nullptr, *ptr = nullptr;
};

static int upload_csr(plk_state s, const double *data, const int64_t *indices, const int64_t *indptr, int64_t nrows,
                      int64_t nnz, CsrDev &c) {
    if (nrows < 0 || nnz < 0 || !indptr || (nnz > 0 && (!data || !indices)))
        PLK_FAIL(PLK_ERR_INVALID_ARG, "bad CSR arrays");
    if ((uint64_t)nrows != s->length) PLK_FAIL(PLK_ERR_INVALID_ARG, "CSR row count does not match the state size");
    if (indptr[0] != 0 || indptr[nrows] != nnz) PLK_FAIL(PLK_ERR_INVALID_ARG, "CSR indptr does not match nnz");
    for (int64_t r = 0; r < nrows; r++)
        if (indptr[r + 1] < indptr[r]) PLK_FAIL(PLK_ERR_INVALID_ARG, "CSR indptr must be non-decreasing");
    for (int64_t j = 0; j < nnz; j++)
        if (indices[j] < 0 || (uint64_t)indices[j] >= s->length) PLK_FAIL(PLK_ERR_INVALID_ARG, "CSR column index out of range");
    PLK_CUDA(cudaMallocAsync((void **)&c.data, sizeof(double2) * std::max<int64_t>(nnz, 1), s->stream));
    PLK_CUDA(cudaMallocAsync((void **)&c.idx, sizeof(int64_t) * std::max<int64_t>(nnz, 1), s->stream));
    PLK_CUDA(cudaMallocAsync((void **)&c.ptr, sizeof(int64_t) * (nrows + 1), s->stream));
    if (nnz > 0) {
        PLK_CUDA(cudaMemcpyAsync(c.data, data, sizeof(double2) * nnz, cudaMemcpyHostToDevice, s->stream));
        PLK_CUDA(cudaMemcpyAsync(c.idx, indices, sizeof(int64_t) * nnz, cudaMemcpyHostToDevice, s->stream));
    }
    PLK_CUDA(cudaMemcpyAsync(c.ptr, indptr, sizeof(int64_t) * (nrows + 1), cudaMemcpyHostToDevice, s->stream));
    return PLK_OK;
}

static int free_csr(plk_state s, CsrDev &c) {
    PLK_CUDA(cudaFreeAsync(c.data, s->stream));
    PLK_CUDA(cudaFreeAsync(c.idx, s->stream));
    PLK_CUDA(cudaFreeAsync(c.ptr, s->stream));
    return PLK_OK;
}

template <class T>
static int pauli_expval_impl(plk_state s, const std::vector<PauliGroup> &groups, const std::vector<PauliTerm> &terms,
                             double *out) {
    PoolBuf dt_buf(s->stream);
    PLK_TRY(pool_alloc(s->device, &dt_buf.p, sizeof(PauliTerm) * std::max<size_t>(terms.size(), 1), s->stream));
    PauliTerm *dt = dt_buf.as<PauliTerm>();
    PLK_CUDA(cudaMemcpyAsync(dt, terms.data(), sizeof(PauliTerm) * terms.size(), cudaMemcpyHostToDevice, s->stream));
    // each group's partial lands in d_result[gi % kMaxRedValues]; fetch in chunks
    double total = 0.0;
    auto &w = s->ws;
    std::vector<double> vals(groups.size());
    for (size_t gi = 0; gi < groups.size(); gi++) {
        const PauliGroup &g = groups[gi];
        uint64_t pmask_lo = 0;
        if (g.x) {
            const int p = 63 - __builtin_clzll(g.x);
            pmask_lo = (1ULL << p) - 1;
        }
        const size_t smem = sizeof(PauliTerm) * g.count;
        if (smem > 48 * 1024) PLK_FAIL(PLK_ERR_UNSUPPORTED, "too many Pauli terms share one X pattern");
        const int grid = red_grid_k(s, k_expval_pauli<T>, g.x ? s->length >> 1 : s->length, smem);
        k_expval_pauli<T><<<grid, kThreads, smem, s->stream>>>((const c2_t<T> *)s->data, s->length, g.x, pmask_lo,
                                                              dt + g.first, g.count, w.d_partials,
                                                              w.d_result + (gi % kMaxRedValues), w.d_counter);
        PLK_CHECK_LAUNCH();
        if (gi % kMaxRedValues == kMaxRedValues - 1 || gi + 1 == groups.size()) {
            const int nv = (int)(gi % kMaxRedValues) + 1;
            PLK_TRY(fetch_results(s, nv, vals.data() + (gi + 1 - nv)));
        }
    }
    for (double v : vals) total += v; // fixed (group) order
    *out = total;
    return PLK_OK;
}

template <class T>
static int pauli_apply_impl(plk_state outs, plk_state ins, const std::vector<PauliGroup> &groups,
                            const std::vector<PauliTerm> &terms) {
    cudaStream_t st = outs->stream;
    PoolBuf dt_buf(st);
    PLK_TRY(pool_alloc(outs->device, &dt_buf.p, sizeof(PauliTerm) * std::max<size_t>(terms.size(), 1), st));
    PauliTerm *dt = dt_buf.as<PauliTerm>();
    PLK_CUDA(cudaMemcpyAsync(dt, terms.data(), sizeof(PauliTerm) * terms.size(), cudaMemcpyHostToDevice, st));
    if (groups.empty()) PLK_CUDA(cudaMemsetAsync(outs->data, 0, outs->length * amp_bytes(outs->dtype), st));
    for (size_t g0 = 0; g0 < groups.size(); g0 += kPauliGroupsPerPass) {
        PauliPass pass;
        pass.ngroups = (int)std::min<size_t>(kPauliGroupsPerPass, groups.size() - g0);
        pass.accumulate = g0 > 0;
        for (int i = 0; i < pass.ngroups; i++) {
            pass.x[i] = groups[g0 + i].x;
            pass.first[i] = groups[g0 + i].first;
            pass.count[i] = groups[g0 + i].count;
        }
        const int t_lo = pass.first[0];
        const int t_cnt = pass.first[pass.ngroups - 1] + pass.count[pass.ngroups - 1] - t_lo;
        const size_t smem = sizeof(PauliTerm) * (size_t)t_cnt;
        const int in_smem = smem <= 48 * 1024 ? 1 : 0;
        // one resident wave of blocks, each walking its tiles in order
        int occ = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_apply_pauli<T>, kThreads, in_smem ? smem : 0) !=
                cudaSuccess ||
            occ < 1) {
            cudaGetLastError();
            occ = 1;
        }
        const int grid = (int)std::max<uint64_t>(
            1, std::min<uint64_t>((outs->length + kPauliTile - 1) / kPauliTile,
                                  (uint64_t)device_sm_count(outs->device) * occ));
        k_apply_pauli<T><<<grid, kThreads, in_smem ? smem : 0, st>>>((c2_t<T> *)outs->data, (const c2_t<T> *)ins->data,
                                                                     outs->length, dt, pass, t_lo, t_cnt, in_smem);
        PLK_CHECK_LAUNCH();
    }
    PLK_CUDA(cudaStreamSynchronize(st)); // host term vectors go away on return
    return PLK_OK;
}

} // namespace plk

using namespace plk;

extern "C" {

PLK_API int plk_expval_named(plk_state s, int32_t gate, const int64_t *wires, int32_t nw, double *out) {
    PLK_TRY(check_state(s));
    if (!out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    PLK_CUDA(cudaSetDevice(s->device));
    if (gate == PLK_GATE_IDENTITY) {
        std::vector<uint64_t> z{0};
        return s->dtype == PLK_C64 ? expval_diag_impl<float>(s, z, out) : expval_diag_impl<double>(s, z, out);
    }
    if (gate != PLK_GATE_PAULIX && gate != PLK_GATE_PAULIY && gate != PLK_GATE_PAULIZ && gate != PLK_GATE_HADAMARD)
        PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "named expectation values exist for Identity, PauliX, PauliY, PauliZ, Hadamard");
    if (nw != 1) PLK_FAIL(PLK_ERR_INVALID_ARG, "named observables act on one wire");
    PLK_TRY(check_wires(s, wires, nw));
    if (gate == PLK_GATE_PAULIZ) {
        std::vector<uint64_t> z{1ULL << (s->nq - 1 - wires[0])};
        return s->dtype == PLK_C64 ? expval_diag_impl<float>(s, z, out) : expval_diag_impl<double>(s, z, out);
    }
    return s->dtype == PLK_C64 ? expval_named_impl<float>(s, gate, wires[0], out)
                               : expval_named_impl<double>(s, gate, wires[0], out);
}

PLK_API int plk_expval_named_batch(plk_state s, int32_t count, const int32_t *gates, const int64_t *wires,
                                   double *out) {
    PLK_TRY(check_state(s));
    if (count < 0 || (count > 0 && (!gates || !wires || !out))) PLK_FAIL(PLK_ERR_INVALID_ARG, "bad batch arguments");
    PLK_CUDA(cudaSetDevice(s->device));
    // diagonal observables share one pass; the others take one pass each
    std::vector<uint64_t> z;
    std::vector<int> zpos;
    for (int i = 0; i < count; i++) {
        if (gates[i] == PLK_GATE_IDENTITY) {
            z.push_back(0);
            zpos.push_back(i);
        } else if (gates[i] == PLK_GATE_PAULIZ) {
            PLK_TRY(check_wires(s, wires + i, 1));
            z.push_back(1ULL << (s->nq - 1 - wires[i]));
            zpos.push_back(i);
        } else {
            PLK_TRY(plk_expval_named(s, gates[i], wires + i, 1, out + i));
        }
    }
    if (!z.empty()) {
        std::vector<double> zv(z.size());
        PLK_TRY(s->dtype == PLK_C64 ? expval_diag_impl<float>(s, z, zv.data()) : expval_diag_impl<double>(s, z, zv.data()));
        for (size_t j = 0; j < z.size(); j++) out[zpos[j]] = zv[j];
    }
    return PLK_OK;
}

PLK_API int plk_inner_product(plk_state x, plk_state y, double *re, double *im) {
    PLK_TRY(check_state(x));
    PLK_TRY(check_state(y));
    if (x->nq != y->nq || x->dtype != y->dtype) PLK_FAIL(PLK_ERR_INVALID_ARG, "states differ in size or precision");
    PLK_CUDA(cudaSetDevice(x->device));
    PLK_TRY(order_after(x, y));
    return x->dtype == PLK_C64 ? inner_impl<float>(x, y, re, im) : inner_impl<double>(x, y, re, im);
}

PLK_API int plk_expval_matrix(plk_state s, const double *matrix, const int64_t *wires, int32_t nw, double *out) {
    PLK_TRY(check_state(s));
    if (!matrix || !out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null argument");
    if (nw < 1) PLK_FAIL(PLK_ERR_INVALID_ARG, "matrix observable needs wires");
    PLK_TRY(check_wires(s, wires, nw));
    PLK_CUDA(cudaSetDevice(s->device));
    if (nw <= 3)
        return s->dtype == PLK_C64 ? expval_herm_any<float>(s, matrix, wires, nw, out)
                                   : expval_herm_any<double>(s, matrix, wires, nw, out);
    // k >= 4: copy, apply, Re<psi|M psi> (MeasuresKokkos.hpp:339-345)
    plk_state tmp = nullptr;
    PLK_TRY(plk_state_create(s->nq, s->dtype, s->device, &tmp));
    int st = plk_state_set_stream(tmp, s->stream);
    if (st == PLK_OK) st = plk_state_copy(tmp, s);
    if (st == PLK_OK) st = apply_matrix_impl(tmp, matrix, wires, nw, false);
    double re = 0.0;
    if (st == PLK_OK) st = plk_inner_product(s, tmp, &re, nullptr);
    plk_state_destroy(tmp);
    if (st == PLK_OK) *out = re;
    return st;
}

PLK_API int plk_expval_sparse(plk_state s, const double *data, const int64_t *indices, const int64_t *indptr,
                              int64_t nrows, int64_t nnz, double *out) {
    PLK_TRY(check_state(s));
    if (!out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    PLK_CUDA(cudaSetDevice(s->device));
    CsrDev c;
    PLK_TRY(upload_csr(s, data, indices, indptr, nrows, nnz, c));
    const int grid = red_grid(s, (uint64_t)nrows);
    auto &w = s->ws;
    if (s->dtype == PLK_C64)
        k_expval_csr<float><<<grid, kThreads, 0, s->stream>>>((const float2 *)s->data, nrows, c.data, c.idx, c.ptr,
                                                             w.d_partials, w.d_result, w.d_counter);
    else
        k_expval_csr<double><<<grid, kThreads, 0, s->stream>>>((const double2 *)s->data, nrows, c.data, c.idx, c.ptr,
                                                              w.d_partials, w.d_result, w.d_counter);
    PLK_CHECK_LAUNCH();
    PLK_TRY(free_csr(s, c));
    return fetch_results(s, 1, out);
}

PLK_API int plk_spmv(plk_state y, plk_state x, const double *data, const int64_t *indices, const int64_t *indptr,
                     int64_t nrows, int64_t nnz) {
    PLK_TRY(check_state(y));
    PLK_TRY(check_state(x));
    if (y == x) PLK_FAIL(PLK_ERR_INVALID_ARG, "SpMV needs distinct input and output states");
    if (x->nq != y->nq || x->dtype != y->dtype) PLK_FAIL(PLK_ERR_INVALID_ARG, "states differ in size or precision");
    PLK_CUDA(cudaSetDevice(y->device));
    PLK_TRY(order_after(y, x));
    CsrDev c;
    PLK_TRY(upload_csr(y, data, indices, indptr, nrows, nnz, c));
    const int grid = elem_grid(y, (uint64_t)nrows);
    if (y->dtype == PLK_C64)
        k_spmv<float><<<grid, kThreads, 0, y->stream>>>((float2 *)y->data, (const float2 *)x->data, nrows, c.data, c.idx,
                                                       c.ptr);
    else
        k_spmv<double><<<grid, kThreads, 0, y->stream>>>((double2 *)y->data, (const double2 *)x->data, nrows, c.data,
                                                        c.idx, c.ptr);
    PLK_CHECK_LAUNCH();
    PLK_TRY(free_csr(y, c));
    PLK_CUDA(cudaStreamSynchronize(y->stream));
    return PLK_OK;
}

PLK_API int plk_expval_pauli_sum(plk_state s, int32_t nterms, const double *coeffs, const int64_t *offsets,
                                 const int64_t *wires, const char *paulis, double *out) {
    PLK_TRY(check_state(s));
    if (!out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    PLK_CUDA(cudaSetDevice(s->device));
    std::vector<PauliGroup> groups;
    std::vector<PauliTerm> terms;
    PLK_TRY(build_pauli_groups(s, nterms, coeffs, offsets, wires, paulis, groups, terms));
    if (groups.empty()) {
        *out = 0.0;
        return PLK_OK;
    }
    return s->dtype == PLK_C64 ? pauli_expval_impl<float>(s, groups, terms, out)
                               : pauli_expval_impl<double>(s, groups, terms, out);
}

PLK_API int plk_apply_pauli_sum(plk_state out, plk_state in, int32_t nterms, const double *coeffs,
                                const int64_t *offsets, const int64_t *wires, const char *paulis) {
    PLK_TRY(check_state(out));
    PLK_TRY(check_state(in));
    if (out == in) PLK_FAIL(PLK_ERR_INVALID_ARG, "Pauli-sum application needs distinct input and output states");
    if (out->nq != in->nq || out->dtype != in->dtype) PLK_FAIL(PLK_ERR_INVALID_ARG, "states differ in size or precision");
    PLK_CUDA(cudaSetDevice(out->device));
    PLK_TRY(order_after(out, in));
    std::vector<PauliGroup> groups;
    std::vector<PauliTerm> terms;
    PLK_TRY(build_pauli_groups(in, nterms, coeffs, offsets, wires, paulis, groups, terms));
    return out->dtype == PLK_C64 ? pauli_apply_impl<float>(out, in, groups, terms)
                                 : pauli_apply_impl<double>(out, in, groups, terms);
}

} // extern "C"
