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

template <int OP> __host__ __device__ constexpr bool pair_touches_x() { return OP != P_PHASE_Y && OP != P_ZERO_Y; }

template <int OP, class V, class T>
__device__ __forceinline__ void pair_op(V &x, V &y, const T *__restrict__ c) {
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
    } else if constexpr (OP == P_GEN_SWAPI) {
        const T sg = c[0];
        V t = x;
        x = mk<V>(sg * y.y, -sg * y.x);   // -i*sg*y
        y = mk<V>(-sg * t.y, sg * t.x);   //  i*sg*x
    }
}

template <int OP, class V, class T>
__device__ __forceinline__ void quad_op(V (&v)[4], const T *__restrict__ c) {
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
};

template <class T> struct QuadArgs {
    Masks mk;
    uint64_t ngroups;
    uint64_t off[4];
    T coef[32];
};

} // namespace plk
