// expval.cu — expectation values, inner products, sparse products.
//
// Replaces ExpValFunctors.hpp, MeasuresKokkos::getExpectationValue*
// (simulator/MeasuresKokkos.hpp:80-346) and the reductions / SpMV of
// util/LinearAlgebraKokkos.hpp.  All reductions accumulate in FP64 (the
// reference accumulates in the state precision) and are deterministic.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "df.cuh"
#include "gate_ops.cuh"
#include "reduce.cuh"

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

// Diagonal observables in one pass: value v = sum_k |psi_k|^2 * sign_v(k) with
// sign_v(k) = (-1)^popcount(k & zmask_v) (Identity: zmask 0; PauliZ: one bit).
template <class T, int NV>
__global__ void __launch_bounds__(kThreads)
    k_expval_diag(const c2_t<T> *__restrict__ sv, uint64_t n, const uint64_t *__restrict__ zmask, int nv,
                  double *partials, double *result, unsigned *counter) {
    __shared__ uint64_t zm[NV];
    for (int v = threadIdx.x; v < NV; v += blockDim.x) zm[v] = v < nv ? zmask[v] : 0;
    __syncthreads();
    DAcc dacc[NV];
    constexpr int U = 4; // amplitudes in flight per thread
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += step * U) {
        c2_t<T> v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint64_t k = k0 + u * step;
            v[u] = k < n ? sv[k] : mk<c2_t<T>>(0, 0);
        }
        if constexpr (sizeof(T) == 4) {
            // complex64: the U amplitudes' signed |a|^2 summed in FP32, the
            // partial added in double-float (error of a partial ~2^-22 of
            // its size, below the state's own rounding)
            float t[NV];
#pragma unroll
            for (int w = 0; w < NV; w++) t[w] = 0.0f;
#pragma unroll
            for (int u = 0; u < U; u++) {
                const uint64_t k = k0 + u * step;
                const float p = fmaf(v[u].x, v[u].x, v[u].y * v[u].y);
#pragma unroll
                for (int w = 0; w < NV; w++) t[w] += (__popcll(k & zm[w]) & 1) ? -p : p;
            }
#pragma unroll
            for (int w = 0; w < NV; w++) dacc[w].add(DF{t[w], 0.0f});
        } else {
#pragma unroll
            for (int u = 0; u < U; u++) {
                const uint64_t k = k0 + u * step;
                const DF p = df_norm2(to_cdf(v[u]));
#pragma unroll
                for (int w = 0; w < NV; w++) {
                    if (__popcll(k & zm[w]) & 1) dacc[w].sub(p);
                    else dacc[w].add(p);
                }
            }
        }
    }
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] = dacc[v].value();
    block_reduce_finish<NV>(acc, partials, result, counter, 1.0, nv);
}

// <psi| M |psi> for a 1- or 2-wire matrix (ExpValFunctors.hpp:155-250).
template <class T, int K>
__global__ void __launch_bounds__(kThreads)
    k_expval_mat(const c2_t<T> *__restrict__ sv, Masks mk, uint64_t ngroups, const uint64_t off0, const uint64_t off1,
                 const uint64_t off2, const uint64_t off3, const double2 *__restrict__ mat, double *partials,
                 double *result, unsigned *counter) {
    constexpr int D = 1 << K;
    __shared__ double2 m[D * D];
    for (int i = threadIdx.x; i < D * D; i += blockDim.x) m[i] = mat[i];
    __syncthreads();
    const uint64_t off[4] = {off0, off1, off2, off3};
    double acc[1] = {0.0};
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += step) {
        const uint64_t base = group_base<K>(g, mk);
        double vr[D], vi[D];
#pragma unroll
        for (int i = 0; i < D; i++) {
            const c2_t<T> a = sv[base + off[i]];
            vr[i] = a.x;
            vi[i] = a.y;
        }
#pragma unroll
        for (int r = 0; r < D; r++) {
            double mr = 0.0, mi = 0.0;
#pragma unroll
            for (int c = 0; c < D; c++) {
                const double2 e = m[r * D + c];
                mr += e.x * vr[c] - e.y * vi[c];
                mi += e.x * vi[c] + e.y * vr[c];
            }
            acc[0] += vr[r] * mr + vi[r] * mi; // Re(conj(v_r) (M v)_r)
        }
    }
    block_reduce_finish<1>(acc, partials, result, counter);
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
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_expval_pauli(const c2_t<T> *__restrict__ sv, uint64_t n, uint64_t x, uint64_t pmask_lo,
                   const PauliTerm *__restrict__ terms, int nt, double *partials, double *result, unsigned *counter) {
    extern __shared__ PauliTerm sterm[];
    for (int i = threadIdx.x; i < nt; i += blockDim.x) sterm[i] = terms[i];
    __syncthreads();
    // coefficients of the group as double-floats (split once per thread)
    DAcc total;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    if constexpr (sizeof(T) == 4) {
        // complex64: each amplitude (pair)'s contribution formed in FP32,
        // accumulated in double-float
        if (x == 0) {
            for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += step) {
                const float2 a = sv[k];
                float f = 0.0f;
                for (int t = 0; t < nt; t++) f += (__popcll(k & sterm[t].z) & 1) ? -sterm[t].crh : sterm[t].crh;
                total.add(DF{fmaf(a.x, a.x, a.y * a.y) * f, 0.0f});
            }
        } else {
            const uint64_t half = n >> 1;
            for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < half; g += step) {
                const uint64_t m = ((g & ~pmask_lo) << 1) | (g & pmask_lo);
                const uint64_t mp = m ^ x;
                const float2 a = sv[m], b = sv[mp];
                float f1 = 0.0f, f2 = 0.0f;
                for (int t = 0; t < nt; t++) {
                    const PauliTerm tt = sterm[t];
                    const bool s1 = __popcll(mp & tt.z) & 1, s0 = __popcll(m & tt.z) & 1;
                    if (s1 == s0) f1 += s0 ? -2.0f * tt.crh : 2.0f * tt.crh;
                    else f2 += s0 ? -2.0f * tt.cih : 2.0f * tt.cih;
                }
                const float re = fmaf(a.x, b.x, a.y * b.y), im = fmaf(a.x, b.y, -a.y * b.x);
                total.add(DF{fmaf(re, f1, im * f2), 0.0f});
            }
        }
    } else if (x == 0) {
        for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += step) {
            const DF p = df_norm2(to_cdf(sv[k]));
            DAcc f;
            for (int t = 0; t < nt; t++) {
                const DF c = {sterm[t].crh, sterm[t].crl};
                if (__popcll(k & sterm[t].z) & 1) f.sub(c);
                else f.add(c);
            }
            total.mac(p, f.normalized());
        }
    } else {
        const uint64_t half = n >> 1;
        for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < half; g += step) {
            const uint64_t m = ((g & ~pmask_lo) << 1) | (g & pmask_lo);
            const uint64_t mp = m ^ x;
            const CDF a = to_cdf(sv[m]), b = to_cdf(sv[mp]);
            // F1 = Re f(m') + Re f(m), F2 = Im f(m) - Im f(m')
            DAcc f1, f2;
            for (int t = 0; t < nt; t++) {
                const PauliTerm tt = sterm[t];
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
    }
    double acc[1] = {total.value()};
    block_reduce_finish<1>(acc, partials, result, counter);
}

// out_m (+)= sum_{groups g} sum_{t in g} c_t i^ny (-1)^popcount((m^x_g) & z_t) in_{m ^ x_g}
constexpr int kPauliGroupsPerPass = 8;
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
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_apply_pauli(c2_t<T> *__restrict__ out, const c2_t<T> *__restrict__ in, uint64_t n,
                  const PauliTerm *__restrict__ terms, const PauliPass pass) {
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t m = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; m < n; m += step) {
        if constexpr (sizeof(T) == 4) {
            float ar = 0.0f, ai = 0.0f;
            if (pass.accumulate) {
                const float2 o = out[m];
                ar = o.x;
                ai = o.y;
            }
            for (int gi = 0; gi < pass.ngroups; gi++) {
                const uint64_t src = m ^ pass.x[gi];
                const float2 v = in[src];
                float fr = 0.0f, fi = 0.0f;
                for (int t = pass.first[gi]; t < pass.first[gi] + pass.count[gi]; t++) {
                    const PauliTerm tt = terms[t];
                    const bool neg = __popcll(src & tt.z) & 1;
                    fr += neg ? -tt.crh : tt.crh;
                    fi += neg ? -tt.cih : tt.cih;
                }
                ar = fmaf(fr, v.x, fmaf(-fi, v.y, ar));
                ai = fmaf(fr, v.y, fmaf(fi, v.x, ai));
            }
            out[m] = make_float2(ar, ai);
        } else {
            DAcc ar, ai;
            if (pass.accumulate) {
                const CDF o = to_cdf(out[m]);
                ar.add(o.re);
                ai.add(o.im);
            }
            for (int gi = 0; gi < pass.ngroups; gi++) {
                const uint64_t src = m ^ pass.x[gi];
                const CDF v = to_cdf(in[src]);
                DAcc fr, fi;
                for (int t = pass.first[gi]; t < pass.first[gi] + pass.count[gi]; t++) {
                    const PauliTerm tt = terms[t];
                    const bool neg = __popcll(src & tt.z) & 1;
                    if (neg) {
                        fr.sub(DF{tt.crh, tt.crl});
                        fi.sub(DF{tt.cih, tt.cil});
                    } else {
                        fr.add(DF{tt.crh, tt.crl});
                        fi.add(DF{tt.cih, tt.cil});
                    }
                }
                const DF f_re = fr.normalized(), f_im = fi.normalized();
                ar.mac(f_re, v.re);
                ar.msub(f_im, v.im);
                ai.mac(f_re, v.im);
                ai.mac(f_im, v.re);
            }
            out[m] = make_double2(ar.value(), ai.value());
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

template <class T, int NV> static void launch_diag(plk_state s, int grid, const uint64_t *dz, int nv) {
    auto &w = s->ws;
    k_expval_diag<T, NV><<<grid, kThreads, 0, s->stream>>>((const c2_t<T> *)s->data, s->length, dz, nv, w.d_partials,
                                                          w.d_result, w.d_counter);
}

// Diagonal (Identity / PauliZ) observables, up to 16 per pass.
template <class T> static int expval_diag_impl(plk_state s, const std::vector<uint64_t> &zmasks, double *out) {
    const int total = (int)zmasks.size();
    uint64_t *dz = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&dz, sizeof(uint64_t) * std::max(total, 1), s->stream));
    PLK_CUDA(cudaMemcpyAsync(dz, zmasks.data(), sizeof(uint64_t) * total, cudaMemcpyHostToDevice, s->stream));
    const int grid = red_grid(s, s->length);
    for (int start = 0; start < total; start += 16) {
        const int nv = std::min(16, total - start);
        if (nv == 1) launch_diag<T, 1>(s, grid, dz + start, nv);
        else if (nv == 2) launch_diag<T, 2>(s, grid, dz + start, nv);
        else if (nv <= 4) launch_diag<T, 4>(s, grid, dz + start, nv);
        else if (nv <= 8) launch_diag<T, 8>(s, grid, dz + start, nv);
        else launch_diag<T, 16>(s, grid, dz + start, nv);
        PLK_CHECK_LAUNCH();
        PLK_TRY(fetch_results(s, nv, out + start));
    }
    PLK_CUDA(cudaFreeAsync(dz, s->stream));
    return PLK_OK;
}

template <class T>
static int expval_mat12_impl(plk_state s, const double *matrix, const int64_t *wires, int K, double *out) {
    int rev[2], srt[2];
    for (int j = 0; j < K; j++) rev[j] = s->nq - 1 - (int)wires[j];
    std::copy(rev, rev + K, srt);
    std::sort(srt, srt + K);
    const Masks mk = make_masks(srt, K);
    uint64_t off[4] = {0, 0, 0, 0};
    for (int i = 0; i < (1 << K); i++)
        for (int j = 0; j < K; j++)
            if ((i >> (K - 1 - j)) & 1) off[i] |= 1ULL << rev[j];
    const int D = 1 << K;
    double2 *dm = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&dm, sizeof(double2) * D * D, s->stream));
    PLK_CUDA(cudaMemcpyAsync(dm, matrix, sizeof(double2) * D * D, cudaMemcpyHostToDevice, s->stream));
    const uint64_t ng = s->length >> K;
    const int grid = red_grid(s, ng);
    auto &w = s->ws;
    if (K == 1)
        k_expval_mat<T, 1><<<grid, kThreads, 0, s->stream>>>((const c2_t<T> *)s->data, mk, ng, off[0], off[1], 0, 0, dm,
                                                             w.d_partials, w.d_result, w.d_counter);
    else
        k_expval_mat<T, 2><<<grid, kThreads, 0, s->stream>>>((const c2_t<T> *)s->data, mk, ng, off[0], off[1], off[2],
                                                             off[3], dm, w.d_partials, w.d_result, w.d_counter);
    PLK_CHECK_LAUNCH();
    PLK_CUDA(cudaFreeAsync(dm, s->stream));
    return fetch_results(s, 1, out);
}

template <class T> static int inner_impl(plk_state x, plk_state y, double *re, double *im) {
    const int grid = red_grid(x, x->length);
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
    PauliTerm *dt = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&dt, sizeof(PauliTerm) * std::max<size_t>(terms.size(), 1), s->stream));
    PLK_CUDA(cudaMemcpyAsync(dt, terms.data(), sizeof(PauliTerm) * terms.size(), cudaMemcpyHostToDevice, s->stream));
    // each group's partial lands in d_result[gi % kMaxRedValues]; fetch in chunks
    double total = 0.0;
    const int grid = red_grid(s, s->length);
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
    PLK_CUDA(cudaFreeAsync(dt, s->stream));
    *out = total;
    return PLK_OK;
}

template <class T>
static int pauli_apply_impl(plk_state outs, plk_state ins, const std::vector<PauliGroup> &groups,
                            const std::vector<PauliTerm> &terms) {
    PauliTerm *dt = nullptr;
    cudaStream_t st = outs->stream;
    PLK_CUDA(cudaMallocAsync((void **)&dt, sizeof(PauliTerm) * std::max<size_t>(terms.size(), 1), st));
    PLK_CUDA(cudaMemcpyAsync(dt, terms.data(), sizeof(PauliTerm) * terms.size(), cudaMemcpyHostToDevice, st));
    const int grid = elem_grid(outs, outs->length);
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
        k_apply_pauli<T><<<grid, kThreads, 0, st>>>((c2_t<T> *)outs->data, (const c2_t<T> *)ins->data, outs->length, dt,
                                                    pass);
        PLK_CHECK_LAUNCH();
    }
    PLK_CUDA(cudaFreeAsync(dt, st));
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
    if (nw <= 2)
        return s->dtype == PLK_C64 ? expval_mat12_impl<float>(s, matrix, wires, nw, out)
                                   : expval_mat12_impl<double>(s, matrix, wires, nw, out);
    // k >= 3: copy, apply, Re<psi|M psi> (MeasuresKokkos.hpp:339-345)
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
