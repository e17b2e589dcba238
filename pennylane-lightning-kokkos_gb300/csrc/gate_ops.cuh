// gate_ops.cuh — local gate arithmetic on registers.
//
// Every named gate and generator of the reference reduces to one of a few
// local operations on the amplitudes of one group:
//   pair ops  act on two amplitudes (x, y) of a group (most gates touch only
//             a pair: X/CNOT/SWAP/CSWAP/Toffoli swap a pair, RX/CRX/IsingXY
//             rotate a pair, RY/CRY/SingleExcitation/DoubleExcitation mix a
//             pair with real coefficients, ...), optionally with a phase or a
//             zero applied to the other amplitudes of the group;
//   quad ops  act on the four amplitudes of a two-wire group (IsingXX,
//             IsingYY, IsingZZ, dense 4x4 matrices, two generators).
// The formulas keep the operation order of the reference functors
// (simulator/GateFunctors.hpp); FMA contraction is allowed.
#pragma once

#include <cstring>

#include "df.cuh"
#include "plk_internal.cuh"

namespace plk {

enum PairOp : int {
    P_SWAP = 0,   // x <-> y                                  (PauliX, CNOT, SWAP, CSWAP, Toffoli, CRX gen)
    P_Y,          // x' = -i y, y' = i x                        (PauliY, CY, CRY gen)
    P_H,          // Hadamard
    P_RX,         // x' = c x - i s y ... (RX/CRX/IsingXY form)  coef: c, s
    P_RY,         // x' = c x - s y, y' = s x + c y             coef: c, s
    P_MAT,        // general 2x2 complex                          coef: m00 m01 m10 m11 (re, im)
    P_DIAG,       // x *= e0, y *= e1                             coef: e0, e1 (re, im)
    P_PHASE_Y,    // y *= e (x untouched)                         coef: e (re, im)
    P_ZERO,       // x = y = 0
    P_GEN_SWAPI,  // x' = -i*sg*y, y' = i*sg*x                    coef: sg
    P_ZERO_Y,     // y = 0 (x untouched)                          (PhaseShift generator)
    P_NEG_Y,      // y = -y (exact)                               (PauliZ, CZ, RZ/CRZ generators)
    P_MULI_Y,     // y = i*sg*y (exact)                           coef: sg  (S, S^dag)
    P_NUM
};

enum QuadOp : int {
    Q_IXX = 0,   // coef: c, s
    Q_IYY,       // coef: c, s
    Q_DIAG,      // coef: e0..e3 (re, im)
    Q_MAT,       // coef: 16 complex, row-major
    Q_GEN_IXX,   // swap(00,11), swap(01,10)
    Q_GEN_IYY,   // 00' = -11, 11' = -00, swap(01,10)
    Q_NUM
};

// Extra amplitudes of a pair group that are multiplied by a phase or zeroed.
enum ExtraMode : int { X_NONE = 0, X_PHASE = 1, X_ZERO = 2 };

template <int OP> __host__ __device__ constexpr bool pair_touches_x() {
    return OP != P_PHASE_Y && OP != P_ZERO_Y && OP != P_NEG_Y && OP != P_MULI_Y;
}
// Ops whose complex128 arithmetic can run on the FP32 pipe (see df.cuh).
template <int OP> __host__ __device__ constexpr bool pair_has_df() {
    return OP == P_H || OP == P_RX || OP == P_RY || OP == P_MAT || OP == P_DIAG || OP == P_PHASE_Y;
}

template <int OP, class V, class T>
__host__ __device__ __forceinline__ void pair_op(V &x, V &y, const T *__restrict__ c) {
    if constexpr (OP == P_SWAP) {
        V t = x;
        x = y;
        y = t;
    } else if constexpr (OP == P_Y) {
        // pauliYFunctor: a0 = (v1.im, -v1.re), a1 = (-v0.im, v0.re)
        V t = x;
        x = mk<V>(y.y, -y.x);
        y = mk<V>(-t.y, t.x);
    } else if constexpr (OP == P_H) {
        const T r = (T)0.70710678118654752440;
        V t = x;
        x = mk<V>(r * t.x + r * y.x, r * t.y + r * y.y);
        y = mk<V>(r * t.x - r * y.x, r * t.y - r * y.y);
    } else if constexpr (OP == P_RX) {
        // rxFunctor: a0 = c v0 + (-v1.im s, v1.re s); a1 = (-v0.im s, v0.re s) + c v1
        const T cc = c[0], s = c[1];
        V t = x;
        x = mk<V>(cc * t.x - y.y * s, cc * t.y + y.x * s);
        y = mk<V>(cc * y.x - t.y * s, cc * y.y + t.x * s);
    } else if constexpr (OP == P_RY) {
        // ryFunctor: a0 = c v0 - s v1; a1 = s v0 + c v1
        const T cc = c[0], s = c[1];
        V t = x;
        x = mk<V>(cc * t.x - s * y.x, cc * t.y - s * y.y);
        y = mk<V>(s * t.x + cc * y.x, s * t.y + cc * y.y);
    } else if constexpr (OP == P_MAT) {
        const V m00 = mk<V>(c[0], c[1]), m01 = mk<V>(c[2], c[3]);
        const V m10 = mk<V>(c[4], c[5]), m11 = mk<V>(c[6], c[7]);
        V t = x;
        x = cadd(cmul(m00, t), cmul(m01, y));
        y = cadd(cmul(m10, t), cmul(m11, y));
    } else if constexpr (OP == P_DIAG) {
        x = cmul(x, mk<V>(c[0], c[1]));
        y = cmul(y, mk<V>(c[2], c[3]));
    } else if constexpr (OP == P_PHASE_Y) {
        y = cmul(y, mk<V>(c[0], c[1]));
    } else if constexpr (OP == P_ZERO) {
        x = mk<V>(0, 0);
        y = mk<V>(0, 0);
    } else if constexpr (OP == P_ZERO_Y) {
        y = mk<V>(0, 0);
    } else if constexpr (OP == P_NEG_Y) {
        y = cneg(y);
    } else if constexpr (OP == P_MULI_Y) {
        y = c[0] > 0 ? mul_i(y) : mul_mi(y);
    } else if constexpr (OP == P_GEN_SWAPI) {
        const T sg = c[0];
        V t = x;
        x = mk<V>(sg * y.y, -sg * y.x);   // -i*sg*y
        y = mk<V>(-sg * t.y, sg * t.x);   //  i*sg*x
    }
}

template <int OP, class V, class T>
__host__ __device__ __forceinline__ void quad_op(V (&v)[4], const T *__restrict__ c) {
    // v[0] = |00>, v[1] = |01> (target wire set), v[2] = |10> (control), v[3] = |11>
    if constexpr (OP == Q_IXX) {
        // isingXXFunctor
        const T cr = c[0], sj = c[1];
        const V v00 = v[0], v01 = v[1], v10 = v[2], v11 = v[3];
        v[0] = mk<V>(cr * v00.x + sj * v11.y, cr * v00.y - sj * v11.x);
        v[1] = mk<V>(cr * v01.x + sj * v10.y, cr * v01.y - sj * v10.x);
        v[2] = mk<V>(cr * v10.x + sj * v01.y, cr * v10.y - sj * v01.x);
        v[3] = mk<V>(cr * v11.x + sj * v00.y, cr * v11.y - sj * v00.x);
    } else if constexpr (OP == Q_IYY) {
        // isingYYFunctor
        const T cr = c[0], sj = c[1];
        const V v00 = v[0], v01 = v[1], v10 = v[2], v11 = v[3];
        v[0] = mk<V>(cr * v00.x - sj * v11.y, cr * v00.y + sj * v11.x);
        v[1] = mk<V>(cr * v01.x + sj * v10.y, cr * v01.y - sj * v10.x);
        v[2] = mk<V>(cr * v10.x + sj * v01.y, cr * v10.y - sj * v01.x);
        v[3] = mk<V>(cr * v11.x - sj * v00.y, cr * v11.y + sj * v00.x);
    } else if constexpr (OP == Q_DIAG) {
#pragma unroll
        for (int i = 0; i < 4; i++) v[i] = cmul(v[i], mk<V>(c[2 * i], c[2 * i + 1]));
    } else if constexpr (OP == Q_MAT) {
        V o[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            V acc = cmul(mk<V>(c[8 * r], c[8 * r + 1]), v[0]);
#pragma unroll
            for (int j = 1; j < 4; j++) acc = cadd(acc, cmul(mk<V>(c[8 * r + 2 * j], c[8 * r + 2 * j + 1]), v[j]));
            o[r] = acc;
        }
#pragma unroll
        for (int r = 0; r < 4; r++) v[r] = o[r];
    } else if constexpr (OP == Q_GEN_IXX) {
        V t = v[0];
        v[0] = v[3];
        v[3] = t;
        t = v[1];
        v[1] = v[2];
        v[2] = t;
    } else if constexpr (OP == Q_GEN_IYY) {
        const V v00 = v[0];
        v[0] = cneg(v[3]);
        v[3] = cneg(v00);
        V t = v[1];
        v[1] = v[2];
        v[2] = t;
    }
}

// ---------------------------------------------------------------------------
// complex128 versions on the FP32 pipe.  Coefficients arrive split on the host
// into hi (h) and lo (l) floats; every real output is a sum of at most eight
// products accumulated as a double-float and rounded once to FP64.
// ---------------------------------------------------------------------------
// c0*a0 + c1*a1 (real coefficients c in (h, l), real operands a as DF)
__device__ __forceinline__ double df_dot2(float c0h, float c0l, DF a0, float c1h, float c1l, DF a1) {
    float sh, sl;
    df_first(c0h, c0l, a0.hi, a0.lo, sh, sl);
    df_mac(c1h, c1l, a1.hi, a1.lo, sh, sl);
    return df_result(sh, sl);
}

// complex product e * v, e = (er, ei) in (h, l)
__device__ __forceinline__ double2 df_cmul(const float *eh, const float *el, const CDF &v) {
    double2 r;
    r.x = df_dot2(eh[0], el[0], v.re, -eh[1], -el[1], v.im);
    r.y = df_dot2(eh[0], el[0], v.im, eh[1], el[1], v.re);
    return r;
}

// sum_j m_j v_j for complex m (interleaved in h/l) and complex v
template <int N>
__device__ __forceinline__ double2 df_cdot(const float *mh, const float *ml, const CDF *v) {
    float rh, rl, ih, il;
    df_first(mh[0], ml[0], v[0].re.hi, v[0].re.lo, rh, rl);
    df_mac(-mh[1], -ml[1], v[0].im.hi, v[0].im.lo, rh, rl);
    df_first(mh[0], ml[0], v[0].im.hi, v[0].im.lo, ih, il);
    df_mac(mh[1], ml[1], v[0].re.hi, v[0].re.lo, ih, il);
#pragma unroll
    for (int j = 1; j < N; j++) {
        df_mac(mh[2 * j], ml[2 * j], v[j].re.hi, v[j].re.lo, rh, rl);
        df_mac(-mh[2 * j + 1], -ml[2 * j + 1], v[j].im.hi, v[j].im.lo, rh, rl);
        df_mac(mh[2 * j], ml[2 * j], v[j].im.hi, v[j].im.lo, ih, il);
        df_mac(mh[2 * j + 1], ml[2 * j + 1], v[j].re.hi, v[j].re.lo, ih, il);
    }
    return make_double2(df_result(rh, rl), df_result(ih, il));
}

template <int OP>
__device__ __forceinline__ void pair_op_df(double2 &x, double2 &y, const float *__restrict__ h,
                                           const float *__restrict__ l) {
    if constexpr (OP == P_PHASE_Y) {
        y = df_cmul(h, l, cdf_split(y));
    } else if constexpr (OP == P_DIAG) {
        x = df_cmul(h, l, cdf_split(x));
        y = df_cmul(h + 2, l + 2, cdf_split(y));
    } else {
        const CDF a = cdf_split(x), b = cdf_split(y);
        if constexpr (OP == P_H) {
            // h[0] = 1/sqrt(2)
            x = make_double2(df_dot2(h[0], l[0], a.re, h[0], l[0], b.re), df_dot2(h[0], l[0], a.im, h[0], l[0], b.im));
            y = make_double2(df_dot2(h[0], l[0], a.re, -h[0], -l[0], b.re),
                             df_dot2(h[0], l[0], a.im, -h[0], -l[0], b.im));
        } else if constexpr (OP == P_RX) {
            // x' = (c x.re - s y.im, c x.im + s y.re); y' = (c y.re - s x.im, c y.im + s x.re)
            x = make_double2(df_dot2(h[0], l[0], a.re, -h[1], -l[1], b.im), df_dot2(h[0], l[0], a.im, h[1], l[1], b.re));
            y = make_double2(df_dot2(h[0], l[0], b.re, -h[1], -l[1], a.im), df_dot2(h[0], l[0], b.im, h[1], l[1], a.re));
        } else if constexpr (OP == P_RY) {
            // x' = c x - s y; y' = s x + c y
            x = make_double2(df_dot2(h[0], l[0], a.re, -h[1], -l[1], b.re),
                             df_dot2(h[0], l[0], a.im, -h[1], -l[1], b.im));
            y = make_double2(df_dot2(h[1], l[1], a.re, h[0], l[0], b.re), df_dot2(h[1], l[1], a.im, h[0], l[0], b.im));
        } else if constexpr (OP == P_MAT) {
            const CDF v[2] = {a, b};
            x = df_cdot<2>(h, l, v);
            y = df_cdot<2>(h + 4, l + 4, v);
        }
    }
}

template <int OP>
__device__ __forceinline__ void quad_op_df(double2 (&v)[4], const float *__restrict__ h, const float *__restrict__ l) {
    if constexpr (OP == Q_DIAG) {
#pragma unroll
        for (int i = 0; i < 4; i++) v[i] = df_cmul(h + 2 * i, l + 2 * i, cdf_split(v[i]));
    } else {
        CDF a[4];
#pragma unroll
        for (int i = 0; i < 4; i++) a[i] = cdf_split(v[i]);
        static_assert(OP != Q_MAT, "the 4x4 matrix runs packed (quad_mat_df2)");
        if constexpr (OP == Q_IXX) {
            // (cr v.re + sj w.im, cr v.im - sj w.re) with w the flipped partner
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const CDF &w = a[3 - i];
                v[i] = make_double2(df_dot2(h[0], l[0], a[i].re, h[1], l[1], w.im),
                                    df_dot2(h[0], l[0], a[i].im, -h[1], -l[1], w.re));
            }
        } else if constexpr (OP == Q_IYY) {
            // 00, 11: (cr v.re - sj w.im, cr v.im + sj w.re); 01, 10: as IsingXX
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const CDF &w = a[3 - i];
                const float sg = (i == 0 || i == 3) ? -1.0f : 1.0f;
                v[i] = make_double2(df_dot2(h[0], l[0], a[i].re, sg * h[1], sg * l[1], w.im),
                                    df_dot2(h[0], l[0], a[i].im, -sg * h[1], -sg * l[1], w.re));
            }
        }
    }
}

template <int OP> __host__ __device__ constexpr bool quad_has_df() {
    return OP == Q_IXX || OP == Q_IYY || OP == Q_DIAG || OP == Q_MAT;
}

// Host-side description of one gate (or generator) application.
struct GatePlan {
    enum Family { F_NOOP = 0, F_PAIR, F_QUAD, F_MRZ, F_GEN_MRZ, F_DENSE };
    int family = F_NOOP;
    int op = 0;
    int K = 0;            // number of wires that define the group
    int a = 0, b = 1;     // local indices of the pair (pair family)
    int n_extra = 0;      // other local indices of the group (pair family)
    int extra_idx[16];
    int extra_mode = X_NONE;
    double coef[32];      // op coefficients (double; cast to the state precision)
    double extra_e[2];    // phase for X_PHASE
    double scale = 0;     // generator scale factor
};

// Device-side launch parameters derived from a plan and the wires.
template <class T> struct PairArgs {
    Masks mk;
    uint64_t ngroups;
    uint64_t offA, offB;
    int n_extra;
    int extra_mode;
    uint64_t off_extra[14];
    T coef[8];
    T e[2];
    float ch[8], cl[8]; // coefficients split for the FP32-pipe complex128 path
    float eh[2], el[2];
};

template <class T> struct QuadArgs {
    Masks mk;
    uint64_t ngroups;
    uint64_t off[4];
    T coef[32];
    float ch[32], cl[32];
    // complex128 4x4 matrix on the packed (re, im) double-float path: per
    // entry m = mr + i mi, the pairs (mr, mr) and (-mi, mi) (hi), and their
    // negations (hi and lo) -- see quad_mat_df2
    f2x pk[6][16];
};

// Fills QuadArgs::pk from the double-float split coefficients (ch, cl).
// The six packed words of one matrix entry m = (rh + rl) + i (ih + il):
// A = (mr, mr), its negation (hi, lo), B = (-mi, mi), its negation (hi, lo).
inline void pack_entry_host(float rh, float rl, float ih, float il, f2x (&w)[6]) {
    auto bits = [](float f) {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        return (f2x)u;
    };
    auto pack = [&](float lane0, float lane1) { return bits(lane0) | (bits(lane1) << 32); };
    w[0] = pack(rh, rh); // A term: (mr, mr) * (v.re, v.im)
    w[1] = pack(-rh, -rh);
    w[2] = pack(-rl, -rl);
    w[3] = pack(-ih, ih); // B term: (-mi, mi) * (v.im, v.re)
    w[4] = pack(ih, -ih);
    w[5] = pack(il, -il);
}

inline void quad_pack_host(const float *ch, const float *cl, f2x (&pk)[6][16]) {
    for (int e = 0; e < 16; e++) {
        f2x w[6];
        pack_entry_host(ch[2 * e], cl[2 * e], ch[2 * e + 1], cl[2 * e + 1], w);
        for (int q = 0; q < 6; q++) pk[q][e] = w[q];
    }
}

// The 4x4 complex128 matrix in double-float with the real and imaginary
// chains packed two lanes per instruction: lane by lane the same operations,
// in the same order, as df_cdot<4> would issue (each output's real part
// accumulates mr*v.re then -mi*v.im per column, its imaginary part mr*v.im
// then mi*v.re).
__device__ __forceinline__ void quad_mat_df2(double2 (&v)[4], const f2x (&pk)[6][16]) {
    f2x vh[4], vl[4], wh[4], wl[4]; // v = (re, im), w = (im, re)
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const CDF a = cdf_split(v[i]);
        vh[i] = f2x_pack(a.re.hi, a.im.hi);
        vl[i] = f2x_pack(a.re.lo, a.im.lo);
        wh[i] = f2x_pack(a.im.hi, a.re.hi);
        wl[i] = f2x_pack(a.im.lo, a.re.lo);
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
        f2x sh, sl;
        const int e0 = 4 * r;
        df_first2(pk[0][e0], pk[1][e0], pk[2][e0], vh[0], vl[0], sh, sl);
        df_mac2(pk[3][e0], pk[4][e0], pk[5][e0], wh[0], wl[0], sh, sl);
#pragma unroll
        for (int c = 1; c < 4; c++) {
            const int e = e0 + c;
            df_mac2(pk[0][e], pk[1][e], pk[2][e], vh[c], vl[c], sh, sl);
            df_mac2(pk[3][e], pk[4][e], pk[5][e], wh[c], wl[c], sh, sl);
        }
        float rh, ih, rl, il;
        f2x_unpack(sh, rh, ih);
        f2x_unpack(sl, rl, il);
        v[r] = make_double2(df_result(rh, rl), df_result(ih, il));
    }
}

} // namespace plk
