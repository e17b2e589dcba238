// batch_engine.cuh — device side of the batched-circuit engine.
//
// Many independent circuits (each with its own qubit count, gates, parameters
// and Pauli-sum observable) run forward, <H> and the adjoint gradient in one
// persistent launch.  Work is organised in register windows: a window fixes
// four state bits; every thread holds the 16 amplitudes that differ only in
// those bits (for lambda and, going backwards, for H lambda) and applies all
// consecutive ops that act inside the window in registers.  Diagonal ops
// (RZ, PhaseShift, CZ, CRZ, IsingZZ, MultiRZ, ...) need no window bits: their
// phase is looked up from each amplitude's full index.
//
// Placement of a circuit's two states:
//   shared memory  the whole circuit runs inside one CTA (n <= smem_bits);
//   global         states in a per-CTA global slot, worked on by one CTA or
//                  by a thread-block cluster of C CTAs; windows are separated
//                  by hardware cluster barriers (one CTA: __syncthreads) and
//                  global accesses bypass L1 (ld.global.cg / st.global.cg).
// Phase A of the kernel hands the cluster circuits to clusters, phase B the
// rest to single CTAs; both queues are ordered by decreasing cost.  There is
// no spin-wait anywhere: the only inter-CTA synchronisation is the cluster
// barrier, reached by every CTA of a cluster the same number of times.
//
// Reductions (expectation value, gradient inner products) use products that
// are exact on the FP32 pipe and double-float accumulation for complex64
// (FP64-class; see df.cuh), plain FP64 for complex128; per-warp partials go
// through shared memory in a fixed order, so results are bitwise
// reproducible for a given launch configuration.
#pragma once

#include <cooperative_groups.h>

#include "df.cuh"
#include "plk_internal.cuh"

namespace plk {

namespace cg = cooperative_groups;

constexpr int kWinBits = 4;      // state bits of a register window
constexpr int kWinAmps = 16;     // amplitudes per thread per state
constexpr int kMaxWinTrain = 16; // trainable ops per window (reduction slots)
constexpr int kMaxWinOps = 96;   // ops per window
constexpr int kMaxCluster = 8;

enum EKind : uint8_t {
    EK_DENSE = 1, // dense 2^K x 2^K matrix on K register bits (canonical order)
    EK_CX = 2,    // CNOT inside the window: a register permutation
    EK_DIAG = 3,  // diagonal gate on K <= 4 wires anywhere in the state
    EK_PARITY = 4, // MultiRZ: phase by parity of the state bits in a mask
    EK_DIAGSET = 5 // several diagonal ops on register bits merged into one 16-entry phase table
                   // (single-state windows only, not the batch engine): mat = the table; K = number of
                   // trainable one-wire members, member m in bits 8m.. of `bits` (register bit,
                   // generator codes of bit value 0 and 1: 0, 1 = +1, 2 = -1) and its reduction
                   // slot in bits 4m.. of `gen`
};

// forms of one-wire dense matrices
enum EForm : uint8_t { EF_GENERAL = 0, EF_RX = 1, EF_RY = 2 };

struct EOp {
    uint8_t kind;
    uint8_t sel;    // DENSE: register-bit selection (K = 1: bit + 4 * form); CX: control * 4 + target
    uint8_t K;      // wires of the op (DENSE, DIAG)
    uint8_t red;    // reduction slot within the window (trainable), 0xff otherwise
    int32_t mat;    // complex offset of U (forward) or U^dag (backward); DIAG/PARITY: phases
    int32_t gen;    // complex offset of the generator (trainable): DENSE matrix, DIAG diagonal
    uint32_t bits;  // DIAG: state bit of wires[j] in bits 5j..5j+4; PARITY: mask of state bits;
                    // DENSE K=1 trainable: generator pattern, 4 bits per row r:
                    // nonzero, column, phase i^q (2 bits)
};

struct EWin {
    uint8_t rb[4];   // state bits of register bits 0..3 (ascending)
    int32_t flags;   // bit 0: only one-wire dense ops, one-wire diagonals and CNOTs (slim)
    int32_t op0;     // ops [op0, op0 + nops)
    int32_t nops;
    int32_t tr0;     // trainable table [tr0, tr0 + ntrain)
    int32_t ntrain;
};

struct ETrain {
    int32_t slot;   // Jacobian slot within the circuit
    float gscale;   // -2 * generator scale * (inverse ? -1 : 1)
};

struct ETerm {
    uint32_t x, z;  // Pauli word: bit flips and sign bits (state bits)
    int32_t ny;     // number of Y letters
    float ch, cl;   // coefficient as a double-float
    double c;
};

enum EMode : int32_t { EM_SMEM = 0, EM_GLOBAL = 1 };

struct ECirc {
    int32_t nq;
    int32_t fw0, nfw;      // forward windows
    int32_t bw0, nbw;      // backward windows
    int32_t term0, nterms; // Pauli terms of the observable
    int32_t jac0, ntp;     // Jacobian slots [jac0, jac0 + ntp)
    int32_t id;            // index in the order circuits were added
};

template <class T> struct EngArgs {
    const ECirc *circ;
    const EWin *win;
    const EOp *ops;
    const ETrain *train;
    const ETerm *terms;
    const c2_t<T> *mats;
    const int32_t *order_cl; // circuits for clusters, by decreasing cost
    const int32_t *order_solo; // circuits for single CTAs, by decreasing cost
    int32_t n_cl, n_solo;
    unsigned *counters;      // [2], zero before the launch
    c2_t<T> *scratch;        // per-CTA slots of 2 * slot_amps amplitudes
    uint64_t slot_amps;
    double *expval;          // [num circuits]
    double *jac;             // [num Jacobian slots]
    double *jac_part;        // [num Jacobian slots][kMaxCluster]
    double *ev_part;         // [num circuits][kMaxCluster]
    int32_t smem_bits;
};

// ------------------------------------------------------------ accumulators --
template <class T> struct EAcc;

template <> struct EAcc<float> {
    using Slot = float2; // per-thread partial kept in shared memory between windows
    float h = 0.0f, l = 0.0f;
    __device__ __forceinline__ void load(const Slot &s) {
        h = s.x;
        l = s.y;
    }
    __device__ __forceinline__ Slot slot() const { return make_float2(h, l); }
    __device__ __forceinline__ void merge(const EAcc<float> &o) { df_add(o.h, o.l, h, l); }
    // += x (a float formed from a few products; two-sum into the pair)
    __device__ __forceinline__ void addf(float x) {
        const float s = __fadd_rn(h, x);
        const float bb = __fsub_rn(s, h);
        const float t = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(x, bb));
        h = s;
        l = __fadd_rn(l, t);
    }
    // += a * b, exact product
    __device__ __forceinline__ void mac(float a, float b) {
        const float p = __fmul_rn(a, b);
        const float e = __fmaf_rn(a, b, -p);
        const float s = __fadd_rn(h, p);
        const float bb = __fsub_rn(s, h);
        const float t = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
        h = s;
        l = __fadd_rn(l, __fadd_rn(t, e));
    }
    // += Im(conj(x) y)
    __device__ __forceinline__ void im_dot(float2 x, float2 y) {
        mac(x.x, y.y);
        mac(-x.y, y.x);
    }
    // += c * Re(conj(x) y), c = (ch + cl)
    __device__ __forceinline__ void re_dot_scaled(float ch, float cl, float2 x, float2 y) {
        float th = __fmul_rn(x.x, y.x);
        float tl = __fmaf_rn(x.x, y.x, -th);
        {
            const float p = __fmul_rn(x.y, y.y);
            const float e = __fmaf_rn(x.y, y.y, -p);
            const float s = __fadd_rn(th, p);
            const float bb = __fsub_rn(s, th);
            const float t = __fadd_rn(__fsub_rn(th, __fsub_rn(s, bb)), __fsub_rn(p, bb));
            th = s;
            tl = __fadd_rn(tl, __fadd_rn(t, e));
        }
        df_mac(ch, cl, th, tl, h, l);
    }
    // warp sum (every lane returns the sum)
    __device__ __forceinline__ double warp_sum() const {
        float sh = h, sl = l;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, sh, o);
            const float ol = __shfl_xor_sync(0xffffffffu, sl, o);
            df_add(oh, ol, sh, sl);
        }
        return df_result(sh, sl);
    }
};

template <> struct EAcc<double> {
    using Slot = double;
    double v = 0.0;
    __device__ __forceinline__ void load(const Slot &s) { v = s; }
    __device__ __forceinline__ Slot slot() const { return v; }
    __device__ __forceinline__ void merge(const EAcc<double> &o) { v += o.v; }
    __device__ __forceinline__ void mac(double a, double b) { v = fma(a, b, v); }
    __device__ __forceinline__ void addf(double x) { v += x; }
    __device__ __forceinline__ void im_dot(double2 x, double2 y) { v = fma(x.x, y.y, fma(-x.y, y.x, v)); }
    __device__ __forceinline__ void re_dot_scaled(float, float, double2, double2) {}
    __device__ __forceinline__ void re_dot_c(double c, double2 x, double2 y) { v = fma(c, x.x * y.x + x.y * y.y, v); }
    __device__ __forceinline__ double warp_sum() const {
        double s = v;
#pragma unroll
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        return s;
    }
};

// ------------------------------------------------------------ state access --
// Shared-memory states are XOR-swizzled so that the 32 lanes of a warp, which
// differ in non-window bits, spread over the banks (16 complex64 or 8
// complex128 amplitudes per 128-byte row).
template <class T> __device__ __forceinline__ uint32_t swz(uint32_t l) {
    if constexpr (sizeof(T) == 4) return l ^ ((l >> 4 ^ l >> 8 ^ l >> 12 ^ l >> 16) & 15u);
    else return l ^ ((l >> 3 ^ l >> 6 ^ l >> 9 ^ l >> 12 ^ l >> 15) & 7u);
}

// Global states are read and written at L2 (ld.global.cg / st.global.cg):
// the CTAs of a cluster share them, and L1 is not coherent across SMs.
template <class T, int MODE> __device__ __forceinline__ c2_t<T> eld(const c2_t<T> *p, uint32_t i) {
    if constexpr (MODE == EM_SMEM) return p[swz<T>(i)];
    else return __ldcg(p + i);
}
template <class T, int MODE> __device__ __forceinline__ void est(c2_t<T> *p, uint32_t i, c2_t<T> v) {
    if constexpr (MODE == EM_SMEM) p[swz<T>(i)] = v;
    else __stcg(p + i, v);
}

// ----------------------------------------------- register-bit selections --
// Dense ops act on K of the four register bits; sel enumerates the subsets
// (ascending bits): K=1: {q}; K=2: 01 02 03 12 13 23; K=3: sel = missing bit.
template <int K, int SEL> __host__ __device__ constexpr int rbit(int i) {
    if constexpr (K == 1) return SEL;
    else if constexpr (K == 2) {
        constexpr int a[6] = {0, 0, 0, 1, 1, 2}, b[6] = {1, 2, 3, 2, 3, 3};
        return i == 0 ? a[SEL] : b[SEL];
    } else if constexpr (K == 3) {
        return i < SEL ? i : i + 1;
    } else {
        return i;
    }
}
template <int K, int SEL> __host__ __device__ constexpr int selmask() {
    int m = 0;
    for (int i = 0; i < K; i++) m |= 1 << rbit<K, SEL>(i);
    return m;
}
template <int K, int SEL> __host__ __device__ constexpr int spread(int m) {
    int r = 0;
    for (int i = 0; i < K; i++)
        if ((m >> i) & 1) r |= 1 << rbit<K, SEL>(i);
    return r;
}

template <class V> __device__ __forceinline__ V cfma(V a, V b, V c) {
    return mk<V>(c.x + a.x * b.x - a.y * b.y, c.y + a.x * b.y + a.y * b.x);
}

// v <- U v on the register bits of (K, SEL); U canonical row-major D x D
template <int K, int SEL, class V> __device__ __forceinline__ void dense_apply(V (&v)[kWinAmps], const V *__restrict__ U) {
    constexpr int D = 1 << K;
    constexpr int M = selmask<K, SEL>();
    V u[D * D];
#pragma unroll
    for (int i = 0; i < D * D; i++) u[i] = U[i];
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & M) continue;
        V in[D];
#pragma unroll
        for (int m = 0; m < D; m++) in[m] = v[j | spread<K, SEL>(m)];
#pragma unroll
        for (int r = 0; r < D; r++) {
            V acc = mk<V>(0, 0);
#pragma unroll
            for (int c = 0; c < D; c++) acc = cfma(u[r * D + c], in[c], acc);
            v[j | spread<K, SEL>(r)] = acc;
        }
    }
}

// Ops on three or four register bits (Toffoli, CSWAP, DoubleExcitation, 3-4
// wire matrices) are rare; they run on a copy of the registers in local
// memory with runtime indices, which keeps the common paths small.
template <class V>
__device__ __noinline__ void dense_apply_rt(V *v, const V *__restrict__ U, int K, uint32_t smask) {
    const int D = 1 << K;
    int sb[4];
    int n = 0;
    for (int b = 0; b < kWinBits; b++)
        if (smask >> b & 1) sb[n++] = b;
    V in[16];
    for (int j = 0; j < kWinAmps; j++) {
        if (j & smask) continue;
        for (int m = 0; m < D; m++) {
            int o = 0;
            for (int i = 0; i < K; i++)
                if (m >> i & 1) o |= 1 << sb[i];
            in[m] = v[j | o];
        }
        for (int r = 0; r < D; r++) {
            V acc = mk<V>(0, 0);
            for (int c = 0; c < D; c++) acc = cfma(U[r * D + c], in[c], acc);
            int o = 0;
            for (int i = 0; i < K; i++)
                if (r >> i & 1) o |= 1 << sb[i];
            v[j | o] = acc;
        }
    }
}

// returns Im <h | G v> over the register groups (G monomial, exact products)
template <class T, class V>
__device__ __noinline__ void dense_gen_dot_rt(const V *v, const V *h, const V *__restrict__ G, int K, uint32_t smask,
                                              EAcc<T> &acc) {
    const int D = 1 << K;
    int sb[4];
    int n = 0;
    for (int b = 0; b < kWinBits; b++)
        if (smask >> b & 1) sb[n++] = b;
    for (int j = 0; j < kWinAmps; j++) {
        if (j & smask) continue;
        for (int r = 0; r < D; r++) {
            V g = mk<V>(0, 0);
            for (int c = 0; c < D; c++) {
                const V e = G[r * D + c];
                int o = 0;
                for (int i = 0; i < K; i++)
                    if (c >> i & 1) o |= 1 << sb[i];
                const V x = v[j | o];
                g = mk<V>(g.x + e.x * x.x - e.y * x.y, g.y + e.x * x.y + e.y * x.x);
            }
            int o = 0;
            for (int i = 0; i < K; i++)
                if (r >> i & 1) o |= 1 << sb[i];
            acc.im_dot(h[j | o], g);
        }
    }
}

// acc += Im <h | G v> on the register bits of (K, SEL); G canonical, monomial
// with entries in {0, +-1, +-i}, so G v is exact
template <int K, int SEL, class T, class V>
__device__ __forceinline__ void dense_gen_dot(const V (&v)[kWinAmps], const V (&h)[kWinAmps], const V *__restrict__ G,
                                              EAcc<T> &acc) {
    constexpr int D = 1 << K;
    constexpr int M = selmask<K, SEL>();
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & M) continue;
#pragma unroll
        for (int r = 0; r < D; r++) {
            V g = mk<V>(0, 0);
#pragma unroll
            for (int c = 0; c < D; c++) {
                const V e = G[r * D + c];
                const V x = v[j | spread<K, SEL>(c)];
                // entries are 0, +-1, +-i: the products and the sum are exact
                g = mk<V>(g.x + e.x * x.x - e.y * x.y, g.y + e.x * x.y + e.y * x.x);
            }
            acc.im_dot(h[j | spread<K, SEL>(r)], g);
        }
    }
}

// acc += Im <h | G v> for a one-wire generator on register bit Q given as a
// monomial pattern (see EOp::bits): row r takes i^q v[col] or nothing.  The
// contribution of two amplitude pairs (at most eight products) is formed in
// the state precision, then accumulated (double-float for complex64),
// alternately into a0 and a1 (two independent chains).
template <int Q, class T, class V>
__device__ __forceinline__ void gen1_dot(const V (&v)[kWinAmps], const V (&h)[kWinAmps], uint32_t pat, EAcc<T> &a0,
                                         EAcc<T> &a1) {
    // per row: value = s1 * (h.x * x.(q odd ? x : y)) + s2 * (h.y * x.(q odd ? y : x))
    T sa[2], sb[2];
    bool on[2], col[2], odd[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const uint32_t rp = (pat >> (4 * r)) & 15u;
        const uint32_t q = rp >> 2;
        on[r] = rp & 1u;
        col[r] = rp & 2u;
        odd[r] = q & 1u;
        const T sg = q >= 2 ? (T)-1 : (T)1;
        sa[r] = on[r] ? sg : (T)0;
        sb[r] = on[r] ? (odd[r] ? sg : -sg) : (T)0;
    }
    int g = 0;
    T t = 0;
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & (1 << Q)) continue;
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const V x = col[r] ? v[j | (1 << Q)] : v[j];
            const V hh = h[j | (r << Q)];
            // Im(conj(hh) i^q x): q even -> +-(hh.x x.y - hh.y x.x); q odd -> +-(hh.x x.x + hh.y x.y)
            t = fma(sa[r] * hh.x, odd[r] ? x.x : x.y, t);
            t = fma(sb[r] * hh.y, odd[r] ? x.y : x.x, t);
        }
        // two pairs (four amplitudes) per partial
        if (g & 1) {
            ((g >> 1) & 1 ? a1 : a0).addf(t);
            t = 0;
        }
        g++;
    }
}

// The same for the generators of RX (Pauli X) and RY (Pauli Y), with the
// pattern known at compile time:
//   X: Im(conj(h0) v1) + Im(conj(h1) v0)
//   Y: Im(conj(h0) (-i v1)) + Im(conj(h1) (i v0)) = -Re(conj(h0) v1) + Re(conj(h1) v0)
template <int Q, bool ISY, class T, class V>
__device__ __forceinline__ void gen1_fixed(const V (&v)[kWinAmps], const V (&h)[kWinAmps], EAcc<T> &a0, EAcc<T> &a1) {
    int g = 0;
    T t = 0;
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & (1 << Q)) continue;
        const V v0 = v[j], v1 = v[j | (1 << Q)], h0 = h[j], h1 = h[j | (1 << Q)];
        if (ISY) {
            t = fma(-h0.x, v1.x, t);
            t = fma(-h0.y, v1.y, t);
            t = fma(h1.x, v0.x, t);
            t = fma(h1.y, v0.y, t);
        } else {
            t = fma(h0.x, v1.y, t);
            t = fma(-h0.y, v1.x, t);
            t = fma(h1.x, v0.y, t);
            t = fma(-h1.y, v0.x, t);
        }
        if (g & 1) {
            ((g >> 1) & 1 ? a1 : a0).addf(t);
            t = 0;
        }
        g++;
    }
}

// One-wire diagonal on register bit Q: the phase (and generator entry) of
// every register amplitude is known at compile time.  Generator partials are
// formed over four amplitudes, then accumulated.
template <int Q, class T, bool BWD, class V>
__device__ __forceinline__ void diag1_reg(V (&lv)[kWinAmps], V (&hv)[kWinAmps], V e0, V e1, T g0, T g1, bool tr,
                                          EAcc<T> &a0, EAcc<T> &a1) {
    T t = 0;
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        const bool one = (j >> Q) & 1;
        if (tr) {
            const T gd = one ? g1 : g0;
            t = fma(gd * hv[j].x, lv[j].y, t);
            t = fma(-gd * hv[j].y, lv[j].x, t);
            if ((j & 3) == 3) {
                ((j >> 2) & 1 ? a1 : a0).addf(t);
                t = 0;
            }
        }
        const V e = one ? e1 : e0;
        lv[j] = cmul(lv[j], e);
        if (BWD) hv[j] = cmul(hv[j], e);
    }
}

// Structured one-wire matrices: RX form [[c, i w], [i w, c]] and RY form
// [[c, -s], [s, c]] (c, w, s real); both keep their form under U^dag.
template <int Q, class V> __device__ __forceinline__ void rx_apply(V (&v)[kWinAmps], const V *__restrict__ U) {
    const auto c = U[0].x, w = U[1].y;
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & (1 << Q)) continue;
        const V x = v[j], y = v[j | (1 << Q)];
        v[j] = mk<V>(c * x.x - w * y.y, c * x.y + w * y.x);
        v[j | (1 << Q)] = mk<V>(c * y.x - w * x.y, c * y.y + w * x.x);
    }
}
template <int Q, class V> __device__ __forceinline__ void ry_apply(V (&v)[kWinAmps], const V *__restrict__ U) {
    const auto c = U[0].x, s = U[2].x;
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (j & (1 << Q)) continue;
        const V x = v[j], y = v[j | (1 << Q)];
        v[j] = mk<V>(c * x.x - s * y.x, c * x.y - s * y.y);
        v[j | (1 << Q)] = mk<V>(s * x.x + c * y.x, s * x.y + c * y.y);
    }
}

template <int C, int TG, class V> __device__ __forceinline__ void cx_apply(V (&v)[kWinAmps]) {
#pragma unroll
    for (int j = 0; j < kWinAmps; j++) {
        if (((j >> C) & 1) && !((j >> TG) & 1)) {
            const V t = v[j];
            v[j] = v[j | (1 << TG)];
            v[j | (1 << TG)] = t;
        }
    }
}

// gate-local index of amplitude `idx` for a DIAG op (wire j -> bit K-1-j)
__device__ __forceinline__ uint32_t diag_index(uint32_t idx, uint32_t bits, int K) {
    uint32_t g = 0;
    for (int j = 0; j < K; j++) g = (g << 1) | ((idx >> ((bits >> (5 * j)) & 31u)) & 1u);
    return g;
}

// SLIM: only one-wire dense ops, one-wire diagonals and CNOTs (host-checked)
template <class T, bool BWD, bool SLIM = false>
__device__ __forceinline__ void window_op(const EOp &op, c2_t<T> (&lv)[kWinAmps], c2_t<T> (&hv)[kWinAmps], uint32_t base,
                                          const uint32_t (&bb)[4], const c2_t<T> *__restrict__ mats, EAcc<T> &acc,
                                          EAcc<T> &acc1) {
    using V = c2_t<T>;
    const bool tr = BWD && op.red != 0xff;
    if (SLIM && op.kind == EK_DENSE) {
        const V *U = mats + op.mat;
#define PLK_S1_CASE(S_)                                                                                               \
    case S_:                                                                                                           \
        if (tr) gen1_dot<S_, T>(lv, hv, op.bits, acc, acc1);                                                           \
        dense_apply<1, S_>(lv, U);                                                                                     \
        if (BWD) dense_apply<1, S_>(hv, U);                                                                            \
        break;                                                                                                         \
    case 4 + S_:                                                                                                       \
        if (tr) gen1_fixed<S_, false, T>(lv, hv, acc, acc1);                                                           \
        rx_apply<S_>(lv, U);                                                                                           \
        if (BWD) rx_apply<S_>(hv, U);                                                                                  \
        break;                                                                                                         \
    case 8 + S_:                                                                                                       \
        if (tr) gen1_fixed<S_, true, T>(lv, hv, acc, acc1);                                                            \
        ry_apply<S_>(lv, U);                                                                                           \
        if (BWD) ry_apply<S_>(hv, U);                                                                                  \
        break;
        switch (op.sel) {
            PLK_S1_CASE(0) PLK_S1_CASE(1) PLK_S1_CASE(2) PLK_S1_CASE(3)
        default: break;
        }
#undef PLK_S1_CASE
    } else if (!SLIM && op.kind == EK_DENSE) {
        const V *U = mats + op.mat;
#define PLK_DENSE1_CASE(S_)                                                                                           \
    case 16 + S_:                                                                                                      \
        if (tr) gen1_dot<S_, T>(lv, hv, op.bits, acc, acc1);                                                           \
        dense_apply<1, S_>(lv, U);                                                                                     \
        if (BWD) dense_apply<1, S_>(hv, U);                                                                            \
        break;                                                                                                         \
    case 16 + 4 + S_:                                                                                                  \
        if (tr) gen1_fixed<S_, false, T>(lv, hv, acc, acc1);                                                           \
        rx_apply<S_>(lv, U);                                                                                           \
        if (BWD) rx_apply<S_>(hv, U);                                                                                  \
        break;                                                                                                         \
    case 16 + 8 + S_:                                                                                                  \
        if (tr) gen1_fixed<S_, true, T>(lv, hv, acc, acc1);                                                            \
        ry_apply<S_>(lv, U);                                                                                           \
        if (BWD) ry_apply<S_>(hv, U);                                                                                  \
        break;
#define PLK_DENSE_CASE(K_, S_)                                                                                        \
    case K_ * 16 + S_:                                                                                                 \
        if (tr) dense_gen_dot<K_, S_, T>(lv, hv, mats + op.gen, acc);                                                  \
        dense_apply<K_, S_>(lv, U);                                                                                    \
        if (BWD) dense_apply<K_, S_>(hv, U);                                                                           \
        break;
        switch (op.K * 16 + op.sel) {
            PLK_DENSE1_CASE(0) PLK_DENSE1_CASE(1) PLK_DENSE1_CASE(2) PLK_DENSE1_CASE(3)
            PLK_DENSE_CASE(2, 0) PLK_DENSE_CASE(2, 1) PLK_DENSE_CASE(2, 2) PLK_DENSE_CASE(2, 3)
            PLK_DENSE_CASE(2, 4) PLK_DENSE_CASE(2, 5)
        default: {
            // K = 3, 4: sel = missing register bit (K = 3) or 0 (K = 4)
            // (copies keep lv / hv themselves in registers)
            const uint32_t smask = op.K == 4 ? 15u : (15u & ~(1u << op.sel));
            V tl[kWinAmps], th[kWinAmps];
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                tl[j] = lv[j];
                th[j] = hv[j];
            }
            if (tr) dense_gen_dot_rt<T>(tl, th, mats + op.gen, op.K, smask, acc);
            dense_apply_rt(tl, U, op.K, smask);
            if (BWD) dense_apply_rt(th, U, op.K, smask);
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                lv[j] = tl[j];
                hv[j] = th[j];
            }
            break;
        }
        }
#undef PLK_DENSE_CASE
#undef PLK_DENSE1_CASE
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
        // one-wire diagonal (RZ, PhaseShift, Z, S, T): two phases by one bit
        const V e0 = mats[op.mat], e1 = mats[op.mat + 1];
        T g0 = 0, g1 = 0;
        if (tr) {
            g0 = mats[op.gen].x;
            g1 = mats[op.gen + 1].x;
        }
        switch (op.sel) {
        case 0: diag1_reg<0, T, BWD>(lv, hv, e0, e1, g0, g1, tr, acc, acc1); break;
        case 1: diag1_reg<1, T, BWD>(lv, hv, e0, e1, g0, g1, tr, acc, acc1); break;
        case 2: diag1_reg<2, T, BWD>(lv, hv, e0, e1, g0, g1, tr, acc, acc1); break;
        case 3: diag1_reg<3, T, BWD>(lv, hv, e0, e1, g0, g1, tr, acc, acc1); break;
        default: {
            // the bit is one of the thread's fixed bits: one phase for all 16 amplitudes
            const bool one = (base >> (op.bits & 31u)) & 1u;
            const V e = one ? e1 : e0;
            const T gd = one ? g1 : g0;
            T t = 0;
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                if (tr) {
                    t = fma(gd * hv[j].x, lv[j].y, t);
                    t = fma(-gd * hv[j].y, lv[j].x, t);
                    if ((j & 3) == 3) {
                        ((j >> 2) & 1 ? acc1 : acc).addf(t);
                        t = 0;
                    }
                }
                lv[j] = cmul(lv[j], e);
                if (BWD) hv[j] = cmul(hv[j], e);
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
            const V e = mats[op.mat + g];
            if (tr) {
                // generator diagonal: MultiRZ (-1)^parity, otherwise real entries 0, +-1
                const T gd = parity ? (g ? (T)-1 : (T)1) : mats[op.gen + g].x;
                (j & 1 ? acc1 : acc).im_dot(hv[j], mk<V>(gd * lv[j].x, gd * lv[j].y));
            }
            lv[j] = cmul(lv[j], e);
            if (BWD) hv[j] = cmul(hv[j], e);
        }
    }
}

// One window over the work items u = t0, t0 + tstep, ... of a state: load the
// 16 amplitudes of lambda (and H lambda going backwards), apply the window's
// ops in registers, store them back; trainable ops add their per-thread
// inner-product partials to part[slot * NT + threadIdx.x].
template <class T, int NT, int MODE, bool BWD, bool SLIM = false>
__device__ __noinline__ void run_window(const EOp *__restrict__ ops, const c2_t<T> *__restrict__ mats, const EWin &w,
                                        int nq, c2_t<T> *lam, c2_t<T> *hl, uint32_t t0, uint32_t tstep,
                                        typename EAcc<T>::Slot *part) {
    using V = c2_t<T>;
    const int lane = threadIdx.x & 31;
    const uint32_t nu = 1u << (nq - kWinBits);
    const uint32_t bb[4] = {1u << w.rb[0], 1u << w.rb[1], 1u << w.rb[2], 1u << w.rb[3]};
    for (uint32_t u = t0; u - lane < nu; u += tstep) {
        const bool act = u < nu;
        uint32_t base = u;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t lo = base & (bb[i] - 1);
            base = ((base ^ lo) << 1) | lo;
        }
        V lv[kWinAmps], hv[kWinAmps];
        // complex64 in global memory with state bit 0 in the window: the
        // pairs (j, j | 1) are adjacent, one 16-byte access each
        const bool pairs = sizeof(T) == 4 && MODE == EM_GLOBAL && bb[0] == 1u;
        if (pairs) {
#pragma unroll
            for (int j = 0; j < kWinAmps; j += 2) {
                const uint32_t idx = base | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) | ((j & 8) ? bb[3] : 0);
                const float4 a = act ? __ldcg(reinterpret_cast<const float4 *>(lam + idx)) : make_float4(0, 0, 0, 0);
                lv[j] = mk<V>(a.x, a.y);
                lv[j + 1] = mk<V>(a.z, a.w);
                if (BWD) {
                    const float4 b = act ? __ldcg(reinterpret_cast<const float4 *>(hl + idx)) : make_float4(0, 0, 0, 0);
                    hv[j] = mk<V>(b.x, b.y);
                    hv[j + 1] = mk<V>(b.z, b.w);
                } else {
                    hv[j] = hv[j + 1] = mk<V>(0, 0);
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                     ((j & 8) ? bb[3] : 0);
                lv[j] = act ? eld<T, MODE>(lam, idx) : mk<V>(0, 0);
                if (BWD) hv[j] = act ? eld<T, MODE>(hl, idx) : mk<V>(0, 0);
                else hv[j] = mk<V>(0, 0);
            }
        }
        for (int k = 0; k < w.nops; k++) {
            const EOp op = ops[w.op0 + k];
            EAcc<T> acc, acc1;
            if (BWD && op.red != 0xff) acc.load(part[op.red * NT + threadIdx.x]);
            window_op<T, BWD, SLIM>(op, lv, hv, base, bb, mats, acc, acc1);
            if (BWD && op.red != 0xff) {
                acc.merge(acc1);
                part[op.red * NT + threadIdx.x] = acc.slot();
            }
        }
        if (act && pairs) {
#pragma unroll
            for (int j = 0; j < kWinAmps; j += 2) {
                const uint32_t idx = base | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) | ((j & 8) ? bb[3] : 0);
                __stcg(reinterpret_cast<float4 *>(lam + idx), make_float4(lv[j].x, lv[j].y, lv[j + 1].x, lv[j + 1].y));
                if (BWD)
                    __stcg(reinterpret_cast<float4 *>(hl + idx), make_float4(hv[j].x, hv[j].y, hv[j + 1].x, hv[j + 1].y));
            }
        } else if (act) {
#pragma unroll
            for (int j = 0; j < kWinAmps; j++) {
                const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                     ((j & 8) ? bb[3] : 0);
                est<T, MODE>(lam, idx, lv[j]);
                if (BWD) est<T, MODE>(hl, idx, hv[j]);
            }
        }
    }
}

} // namespace plk
