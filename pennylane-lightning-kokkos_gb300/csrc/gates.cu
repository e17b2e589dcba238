// gates.cu — gate, matrix and generator kernels.
//
// Replaces the gate functors of simulator/GateFunctors.hpp and their
// dispatch in simulator/StateVectorKokkos.hpp (applyOperation :585-676,
// applySingle/Two/MultiQubitOp :704-796, applyGateFunctor :807-824,
// applyMultiRZ :1222-1240, applyGenerator* :1275-1580).
//
// One kernel per local-operation shape instead of one functor per gate:
//   k_pair  — grid-stride over groups, loads only the two amplitudes the
//             gate changes (plus, for the +/- excitation gates and some
//             generators, the other amplitudes of the group), vectorised
//             float2/double2 loads;
//   k_quad  — the four amplitudes of a two-wire group;
//   k_mrz   — element-wise parity phase (MultiRZ and its generator;
//             k_mrz_df for complex128 in double-float);
//   k_dense_reg — 2^k x 2^k matrices for k = 3, 4: one group per thread in
//             registers, matrix in shared memory (complex128 in packed
//             double-float);
//   k_dense_df — complex128, k >= 5, in double-float;
//   k_dense — complex64 k >= 7 (5 and 6 run on the tensor cores,
//             dense_tc.cu) and complex128 k >= 3 in native-FP64 mode; group
//             vectors staged in shared memory, matrix in shared memory when
//             it fits.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "gate_ops.cuh"

namespace plk {

// ------------------------------------------------------------ gate table --
struct GateInfo {
    const char *name;
    int nwires; // -1: any
    int nparams;
};

static const GateInfo kGates[PLK_GATE_COUNT] = {
    {"Identity", -1, 0},
    {"PauliX", 1, 0}, {"PauliY", 1, 0}, {"PauliZ", 1, 0}, {"Hadamard", 1, 0},
    {"S", 1, 0}, {"T", 1, 0}, {"PhaseShift", 1, 1}, {"RX", 1, 1}, {"RY", 1, 1},
    {"RZ", 1, 1}, {"Rot", 1, 3},
    {"CNOT", 2, 0}, {"CY", 2, 0}, {"CZ", 2, 0}, {"SWAP", 2, 0},
    {"ControlledPhaseShift", 2, 1}, {"CRX", 2, 1}, {"CRY", 2, 1}, {"CRZ", 2, 1},
    {"CRot", 2, 3}, {"IsingXX", 2, 1}, {"IsingXY", 2, 1}, {"IsingYY", 2, 1},
    {"IsingZZ", 2, 1}, {"SingleExcitation", 2, 1},
    {"SingleExcitationMinus", 2, 1}, {"SingleExcitationPlus", 2, 1},
    {"DoubleExcitation", 4, 1}, {"DoubleExcitationMinus", 4, 1},
    {"DoubleExcitationPlus", 4, 1}, {"CSWAP", 3, 0}, {"Toffoli", 3, 0},
    {"MultiRZ", -1, 1},
    {"Matrix", -1, 0},
};

// Rot = RZ(omega) RY(theta) RZ(phi) (rotFunctor GateFunctors.hpp:3134-3160);
// the inverse negates and reverses the angles.
static void rot_matrix(const double *p, bool inv, double *m) {
    const double phi = inv ? -p[2] : p[0];
    const double theta = inv ? -p[1] : p[1];
    const double omega = inv ? -p[0] : p[2];
    const double c = std::cos(theta / 2), s = std::sin(theta / 2);
    const double pp = phi + omega, mm = phi - omega;
    m[0] = std::cos(pp / 2) * c;  m[1] = -std::sin(pp / 2) * c;   // e^{-i p/2} c
    m[2] = -std::cos(mm / 2) * s; m[3] = -std::sin(mm / 2) * s;   // -e^{i m/2} s
    m[4] = std::cos(mm / 2) * s;  m[5] = -std::sin(mm / 2) * s;   // e^{-i m/2} s
    m[6] = std::cos(pp / 2) * c;  m[7] = std::sin(pp / 2) * c;    // e^{i p/2} c
}

static void set_pair(GatePlan &p, int K, int op, int a, int b) {
    p.family = GatePlan::F_PAIR;
    p.K = K;
    p.op = op;
    p.a = a;
    p.b = b;
    p.n_extra = 0;
    p.extra_mode = X_NONE;
}

static void set_extras(GatePlan &p, int mode, double er = 0, double ei = 0) {
    const int dim = 1 << p.K;
    p.n_extra = 0;
    for (int i = 0; i < dim; i++)
        if (i != p.a && i != p.b) p.extra_idx[p.n_extra++] = i;
    p.extra_mode = mode;
    p.extra_e[0] = er;
    p.extra_e[1] = ei;
}

static void set_extras_list(GatePlan &p, int mode, std::initializer_list<int> idx) {
    p.n_extra = 0;
    for (int i : idx) p.extra_idx[p.n_extra++] = i;
    p.extra_mode = mode;
    p.extra_e[0] = p.extra_e[1] = 0;
}

// Plan of a named gate (GateFunctors.hpp functor constructors).
int window_apply_ops(plk_state s, const plk_op *ops, int nops, bool &handled);

int plan_gate(int gate, int nw, bool inv, const double *prm, int np, GatePlan &p) {
    if (gate < 0 || gate >= PLK_GATE_COUNT || gate == PLK_GATE_MATRIX)
        PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "unknown gate id " + std::to_string(gate));
    const GateInfo &gi = kGates[gate];
    if (gi.nwires > 0 && nw != gi.nwires)
        PLK_FAIL(PLK_ERR_INVALID_ARG, std::string(gi.name) + " acts on " + std::to_string(gi.nwires) + " wires, got " +
                                          std::to_string(nw));
    if (np < gi.nparams)
        PLK_FAIL(PLK_ERR_INVALID_ARG, std::string(gi.name) + " needs " + std::to_string(gi.nparams) + " parameter(s)");
    if (gate == PLK_GATE_MULTIRZ && nw < 1) PLK_FAIL(PLK_ERR_INVALID_ARG, "MultiRZ needs at least one wire");
    std::memset(p.coef, 0, sizeof(p.coef));
    const double th = np > 0 ? prm[0] : 0.0;
    const double ch = std::cos(th / 2), sh = std::sin(th / 2);
    switch (gate) {
    case PLK_GATE_IDENTITY: p.family = GatePlan::F_NOOP; return PLK_OK;
    case PLK_GATE_PAULIX: set_pair(p, 1, P_SWAP, 0, 1); break;
    case PLK_GATE_PAULIY: set_pair(p, 1, P_Y, 0, 1); break;
    case PLK_GATE_PAULIZ: set_pair(p, 1, P_NEG_Y, 0, 1); break;
    case PLK_GATE_HADAMARD: set_pair(p, 1, P_H, 0, 1); p.coef[0] = M_SQRT1_2; break;
    case PLK_GATE_S: set_pair(p, 1, P_MULI_Y, 0, 1); p.coef[0] = inv ? -1 : 1; break;
    case PLK_GATE_T:
        set_pair(p, 1, P_PHASE_Y, 0, 1);
        p.coef[0] = std::cos(M_PI / 4);
        p.coef[1] = inv ? -std::sin(M_PI / 4) : std::sin(M_PI / 4);
        break;
    case PLK_GATE_PHASESHIFT:
        set_pair(p, 1, P_PHASE_Y, 0, 1);
        p.coef[0] = std::cos(th);
        p.coef[1] = inv ? -std::sin(th) : std::sin(th);
        break;
    case PLK_GATE_RX: // rxFunctor: s = inverse ? sin(t/2) : sin(-t/2)
        set_pair(p, 1, P_RX, 0, 1);
        p.coef[0] = std::cos(th * 0.5);
        p.coef[1] = inv ? std::sin(th * 0.5) : std::sin(-th * 0.5);
        break;
    case PLK_GATE_RY: // ryFunctor: s = inverse ? -sin(t/2) : sin(t/2)
        set_pair(p, 1, P_RY, 0, 1);
        p.coef[0] = std::cos(th * 0.5);
        p.coef[1] = inv ? -std::sin(th * 0.5) : std::sin(th * 0.5);
        break;
    case PLK_GATE_RZ: // rzFunctor: (c, -s), (c, s); inverse conjugates
        set_pair(p, 1, P_DIAG, 0, 1);
        p.coef[0] = ch; p.coef[1] = inv ? sh : -sh;
        p.coef[2] = ch; p.coef[3] = inv ? -sh : sh;
        break;
    case PLK_GATE_ROT: set_pair(p, 1, P_MAT, 0, 1); rot_matrix(prm, inv, p.coef); break;
    // two-wire gates: local index bit 1 = wires[0] (control), bit 0 = wires[1]
    case PLK_GATE_CNOT: set_pair(p, 2, P_SWAP, 2, 3); break;
    case PLK_GATE_CY: set_pair(p, 2, P_Y, 2, 3); break;
    case PLK_GATE_CZ: set_pair(p, 2, P_NEG_Y, 2, 3); break;
    case PLK_GATE_SWAP: set_pair(p, 2, P_SWAP, 1, 2); break;
    case PLK_GATE_CONTROLLEDPHASESHIFT:
        set_pair(p, 2, P_PHASE_Y, 2, 3);
        p.coef[0] = std::cos(th);
        p.coef[1] = inv ? -std::sin(th) : std::sin(th);
        break;
    case PLK_GATE_CRX: // crxFunctor: js = inverse ? -sin : sin, same rotation as RX with s = -js
        set_pair(p, 2, P_RX, 2, 3);
        p.coef[0] = ch;
        p.coef[1] = inv ? sh : -sh;
        break;
    case PLK_GATE_CRY:
        set_pair(p, 2, P_RY, 2, 3);
        p.coef[0] = ch;
        p.coef[1] = inv ? -sh : sh;
        break;
    case PLK_GATE_CRZ:
        set_pair(p, 2, P_DIAG, 2, 3);
        p.coef[0] = ch; p.coef[1] = inv ? sh : -sh;
        p.coef[2] = ch; p.coef[3] = inv ? -sh : sh;
        break;
    case PLK_GATE_CROT: set_pair(p, 2, P_MAT, 2, 3); rot_matrix(prm, inv, p.coef); break;
    case PLK_GATE_ISINGXX:
        p.family = GatePlan::F_QUAD; p.K = 2; p.op = Q_IXX;
        p.coef[0] = ch; p.coef[1] = inv ? -sh : sh;
        break;
    case PLK_GATE_ISINGXY: // isingXYFunctor leaves |00>, |11>; rotates (01, 10) like RX with s = sj
        set_pair(p, 2, P_RX, 1, 2);
        p.coef[0] = ch; p.coef[1] = inv ? -sh : sh;
        break;
    case PLK_GATE_ISINGYY:
        p.family = GatePlan::F_QUAD; p.K = 2; p.op = Q_IYY;
        p.coef[0] = ch; p.coef[1] = inv ? -sh : sh;
        break;
    case PLK_GATE_ISINGZZ: {
        p.family = GatePlan::F_QUAD; p.K = 2; p.op = Q_DIAG;
        const double s0i = inv ? sh : -sh, s1i = inv ? -sh : sh;
        const double d[8] = {ch, s0i, ch, s1i, ch, s1i, ch, s0i};
        std::memcpy(p.coef, d, sizeof(d));
        break;
    }
    case PLK_GATE_SINGLEEXCITATION:
        set_pair(p, 2, P_RY, 1, 2);
        p.coef[0] = ch; p.coef[1] = inv ? -sh : sh;
        break;
    case PLK_GATE_SINGLEEXCITATIONMINUS:
    case PLK_GATE_SINGLEEXCITATIONPLUS: {
        set_pair(p, 2, P_RY, 1, 2);
        p.coef[0] = ch; p.coef[1] = inv ? -sh : sh;
        // SE-: e = inverse ? e^{i t/2} : e^{-i t/2};  SE+: the opposite
        const bool minus = gate == PLK_GATE_SINGLEEXCITATIONMINUS;
        const double si = (minus != inv) ? -sh : sh;
        set_extras(p, X_PHASE, ch, si);
        break;
    }
    case PLK_GATE_DOUBLEEXCITATION:
        set_pair(p, 4, P_RY, 3, 12);
        p.coef[0] = ch; p.coef[1] = inv ? -sh : sh;
        break;
    case PLK_GATE_DOUBLEEXCITATIONMINUS:
    case PLK_GATE_DOUBLEEXCITATIONPLUS: {
        set_pair(p, 4, P_RY, 3, 12);
        p.coef[0] = ch; p.coef[1] = inv ? -sh : sh;
        const bool minus = gate == PLK_GATE_DOUBLEEXCITATIONMINUS;
        const double si = (minus != inv) ? -sh : sh;
        set_extras(p, X_PHASE, ch, si);
        break;
    }
    case PLK_GATE_CSWAP: set_pair(p, 3, P_SWAP, 5, 6); break;
    case PLK_GATE_TOFFOLI: set_pair(p, 3, P_SWAP, 7, 6); break;
    case PLK_GATE_MULTIRZ:
        p.family = GatePlan::F_MRZ; p.K = nw;
        p.coef[0] = ch; p.coef[1] = inv ? sh : -sh; // shift_0 (even parity)
        p.coef[2] = ch; p.coef[3] = inv ? -sh : sh; // shift_1 (odd parity)
        break;
    default: PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "unknown gate id " + std::to_string(gate));
    }
    return PLK_OK;
}

// Plan of a generator (applyGenerator*, StateVectorKokkos.hpp:1275-1580 and
// the generator functors GateFunctors.hpp:2172-3132); the adjoint flag is
// ignored, as the reference's generator functors ignore it.
int plan_generator(int gate, int nw, GatePlan &p) {
    if (gate < 0 || gate >= PLK_GATE_COUNT) PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "unknown gate id");
    const GateInfo &gi = kGates[gate];
    if (gi.nwires > 0 && nw != gi.nwires)
        PLK_FAIL(PLK_ERR_INVALID_ARG, std::string(gi.name) + " acts on " + std::to_string(gi.nwires) + " wires");
    std::memset(p.coef, 0, sizeof(p.coef));
    p.scale = -0.5;
    switch (gate) {
    case PLK_GATE_RX: set_pair(p, 1, P_SWAP, 0, 1); break;
    case PLK_GATE_RY: set_pair(p, 1, P_Y, 0, 1); break;
    case PLK_GATE_RZ: set_pair(p, 1, P_NEG_Y, 0, 1); break;
    case PLK_GATE_PHASESHIFT: set_pair(p, 1, P_ZERO_Y, 1, 0); p.scale = 1.0; break;
    case PLK_GATE_CONTROLLEDPHASESHIFT:
        set_pair(p, 2, P_ZERO, 0, 1);
        set_extras_list(p, X_ZERO, {2});
        p.scale = 1.0;
        break;
    case PLK_GATE_CRX: set_pair(p, 2, P_SWAP, 2, 3); set_extras_list(p, X_ZERO, {0, 1}); break;
    case PLK_GATE_CRY: set_pair(p, 2, P_Y, 2, 3); set_extras_list(p, X_ZERO, {0, 1}); break;
    case PLK_GATE_CRZ:
        set_pair(p, 2, P_NEG_Y, 2, 3);
        set_extras_list(p, X_ZERO, {0, 1});
        break;
    case PLK_GATE_ISINGXX: p.family = GatePlan::F_QUAD; p.K = 2; p.op = Q_GEN_IXX; break;
    case PLK_GATE_ISINGXY:
        set_pair(p, 2, P_SWAP, 1, 2);
        set_extras_list(p, X_ZERO, {0, 3});
        p.scale = 0.5;
        break;
    case PLK_GATE_ISINGYY: p.family = GatePlan::F_QUAD; p.K = 2; p.op = Q_GEN_IYY; break;
    case PLK_GATE_ISINGZZ:
        set_pair(p, 2, P_DIAG, 1, 2);
        p.coef[0] = -1; p.coef[2] = -1;
        break;
    case PLK_GATE_SINGLEEXCITATION:
        set_pair(p, 2, P_GEN_SWAPI, 1, 2);
        p.coef[0] = 1;
        set_extras_list(p, X_ZERO, {0, 3});
        break;
    case PLK_GATE_SINGLEEXCITATIONMINUS: set_pair(p, 2, P_GEN_SWAPI, 1, 2); p.coef[0] = 1; break;
    case PLK_GATE_SINGLEEXCITATIONPLUS:
        set_pair(p, 2, P_GEN_SWAPI, 1, 2);
        p.coef[0] = 1;
        set_extras_list(p, X_PHASE, {0, 3});
        p.extra_e[0] = -1;
        p.extra_e[1] = 0;
        break;
    case PLK_GATE_DOUBLEEXCITATION:
        set_pair(p, 4, P_GEN_SWAPI, 3, 12);
        p.coef[0] = 1;
        set_extras(p, X_ZERO);
        break;
    case PLK_GATE_DOUBLEEXCITATIONMINUS: set_pair(p, 4, P_GEN_SWAPI, 3, 12); p.coef[0] = 1; break;
    case PLK_GATE_DOUBLEEXCITATIONPLUS:
        set_pair(p, 4, P_GEN_SWAPI, 3, 12);
        p.coef[0] = -1;
        p.scale = 0.5;
        break;
    case PLK_GATE_MULTIRZ:
        if (nw < 1) PLK_FAIL(PLK_ERR_INVALID_ARG, "MultiRZ needs at least one wire");
        p.family = GatePlan::F_GEN_MRZ;
        p.K = nw;
        break;
    default:
        PLK_FAIL(PLK_ERR_UNKNOWN_GATE, std::string("Generator does not exist for ") + gi.name);
    }
    return PLK_OK;
}

// Sorted bit positions, masks and local offsets of a wire list.
struct WireGeom {
    int K;
    int rev[kMaxDenseWires];
    int sorted[kMaxDenseWires];
    Masks mk;
    uint64_t local_off(int i) const { // local index bit (K-1-j) <-> wires[j]
        uint64_t o = 0;
        for (int j = 0; j < K; j++)
            if ((i >> (K - 1 - j)) & 1) o |= 1ULL << rev[j];
        return o;
    }
};

static void wire_geom(int nq, const int64_t *wires, int K, WireGeom &g) {
    g.K = K;
    for (int j = 0; j < K; j++) g.rev[j] = nq - 1 - (int)wires[j];
    std::copy(g.rev, g.rev + K, g.sorted);
    std::sort(g.sorted, g.sorted + K);
    g.mk = make_masks(g.sorted, K);
}

// ---------------------------------------------------------------- kernels --
constexpr int kUnroll = 2;

template <class T, int OP, int K, bool DFP>
__global__ void __launch_bounds__(kThreads) k_pair(c2_t<T> *__restrict__ sv, const PairArgs<T> a) {
    using V = c2_t<T>;
    constexpr bool TX = pair_touches_x<OP>();
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x * kUnroll;
    for (uint64_t g0 = (uint64_t)blockIdx.x * blockDim.x * kUnroll + threadIdx.x; g0 < a.ngroups; g0 += step) {
        uint64_t base[kUnroll];
        V x[kUnroll], y[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; u++) {
            const uint64_t g = g0 + (uint64_t)u * blockDim.x;
            base[u] = group_base<K>(g < a.ngroups ? g : 0, a.mk);
            if (g < a.ngroups) {
                if (TX) x[u] = sv[base[u] + a.offA];
                y[u] = sv[base[u] + a.offB];
            }
        }
#pragma unroll
        for (int u = 0; u < kUnroll; u++) {
            const uint64_t g = g0 + (uint64_t)u * blockDim.x;
            if (g < a.ngroups) {
                if constexpr (DFP) pair_op_df<OP>(x[u], y[u], a.ch, a.cl);
                else pair_op<OP>(x[u], y[u], a.coef);
                if (TX) sv[base[u] + a.offA] = x[u];
                sv[base[u] + a.offB] = y[u];
                for (int j = 0; j < a.n_extra; j++) {
                    V *p = sv + base[u] + a.off_extra[j];
                    if (a.extra_mode == X_PHASE) {
                        if constexpr (DFP) *p = df_cmul(a.eh, a.el, cdf_split(*p));
                        else *p = cmul(*p, mk<V>(a.e[0], a.e[1]));
                    } else {
                        *p = mk<V>(0, 0);
                    }
                }
            }
        }
    }
}

template <class T, int OP, bool DFP>
__global__ void __launch_bounds__(kThreads) k_quad(c2_t<T> *__restrict__ sv, const QuadArgs<T> a) {
    using V = c2_t<T>;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.ngroups; g += step) {
        const uint64_t base = group_base<2>(g, a.mk);
        V v[4];
#pragma unroll
        for (int i = 0; i < 4; i++) v[i] = sv[base + a.off[i]];
        if constexpr (DFP && OP == Q_MAT) quad_mat_df2(v, a.pk);
        else if constexpr (DFP) quad_op_df<OP>(v, a.ch, a.cl);
        else quad_op<OP>(v, a.coef);
#pragma unroll
        for (int i = 0; i < 4; i++) sv[base + a.off[i]] = v[i];
    }
}

// complex128 matrices on k >= 5 wires in double-float on the FP32 pipe: the
// native-FP64 k_dense spends 4 FP64 instructions per complex multiply-add
// (this GPU runs FP64 at about 1/64 of its FP32 rate).  The group vectors are
// split into double-float pairs once, when they are staged in shared memory;
// each thread forms one output row as a double-float complex dot product.
// The matrix is stored transposed, [column][row] (split on the host), so the
// threads of a warp (consecutive rows) read consecutive entries: no bank
// conflicts; in shared memory for k <= 6, through L1/L2 beyond.
constexpr int kSmemMatWiresDf = 6;

__global__ void __launch_bounds__(kThreads) k_dense_df(double2 *__restrict__ sv, const float4 *__restrict__ matT,
                                                       const uint64_t *__restrict__ off, Masks gm, int K,
                                                       uint64_t ngroups, int mat_in_smem) {
    extern __shared__ __align__(16) float4 dsm[];
    const int dim = 1 << K;
    float4 *smat = dsm;
    float4 *svec = dsm + (mat_in_smem ? dim * dim : 0);
    if (mat_in_smem)
        for (int i = threadIdx.x; i < dim * dim; i += blockDim.x) smat[i] = matT[i];
    const float4 *MT = mat_in_smem ? smat : matT;
    const int gpb = dim >= kThreads ? 1 : kThreads / dim;
    const int rows_per_thread = dim >= kThreads ? dim / kThreads : 1;
    for (uint64_t gb = (uint64_t)blockIdx.x * gpb; gb < ngroups; gb += (uint64_t)gridDim.x * gpb) {
        __syncthreads();
        for (int t = threadIdx.x; t < gpb * dim; t += blockDim.x) {
            const int gi = t / dim, r = t % dim;
            const uint64_t g = gb + gi;
            if (g < ngroups) {
                uint64_t base = g & gm.m[0];
                for (int j = 1; j <= K; j++) base |= (g << j) & gm.m[j];
                const CDF v = cdf_split(sv[base + off[r]]);
                svec[t] = make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo);
            }
        }
        __syncthreads();
        for (int rr = 0; rr < rows_per_thread; rr++) {
            const int t = threadIdx.x + rr * kThreads;
            const int gi = t / dim, r = t % dim;
            const uint64_t g = gb + gi;
            if (gi < gpb && g < ngroups) {
                const float4 *vec = svec + gi * dim;
                float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
#pragma unroll 4
                for (int j = 0; j < dim; j++) {
                    const float4 m = MT[(size_t)j * dim + r], v = vec[j];
                    df_mac(m.x, m.y, v.x, v.y, rh, rl);
                    df_mac(-m.z, -m.w, v.z, v.w, rh, rl);
                    df_mac(m.x, m.y, v.z, v.w, ih, il);
                    df_mac(m.z, m.w, v.x, v.y, ih, il);
                }
                uint64_t base = g & gm.m[0];
                for (int j = 1; j <= K; j++) base |= (g << j) & gm.m[j];
                sv[base + off[r]] = make_double2(df_result(rh, rl), df_result(ih, il));
            }
        }
    }
}

// MultiRZ: element-wise parity phase, four amplitudes in flight per thread
constexpr int kMrzUnroll = 4;

template <class T, bool GEN>
__global__ void __launch_bounds__(kThreads) k_mrz(c2_t<T> *__restrict__ sv, uint64_t n, uint64_t mask, T e0r, T e0i,
                                                   T e1r, T e1i) {
    using V = c2_t<T>;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += step * kMrzUnroll) {
        V v[kMrzUnroll];
#pragma unroll
        for (int u = 0; u < kMrzUnroll; u++)
            if (k0 + u * step < n) v[u] = sv[k0 + u * step];
#pragma unroll
        for (int u = 0; u < kMrzUnroll; u++) {
            const uint64_t k = k0 + u * step;
            if (k >= n) break;
            const bool odd = __popcll(k & mask) & 1;
            if (GEN) {
                if (odd) v[u] = cneg(v[u]);
            } else {
                v[u] = odd ? cmul(v[u], mk<V>(e1r, e1i)) : cmul(v[u], mk<V>(e0r, e0i));
            }
            sv[k] = v[u];
        }
    }
}

// complex128 MultiRZ with the phase products in double-float on the FP32
// pipe: eh/el hold e0 (even parity) then e1 (odd parity), split hi/lo
__global__ void __launch_bounds__(kThreads) k_mrz_df(double2 *__restrict__ sv, uint64_t n, uint64_t mask,
                                                      const float4 eh, const float4 el) {
    const float h0[2] = {eh.x, eh.y}, h1[2] = {eh.z, eh.w};
    const float l0[2] = {el.x, el.y}, l1[2] = {el.z, el.w};
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k0 < n; k0 += step * kMrzUnroll) {
        double2 v[kMrzUnroll];
#pragma unroll
        for (int u = 0; u < kMrzUnroll; u++)
            if (k0 + u * step < n) v[u] = sv[k0 + u * step];
#pragma unroll
        for (int u = 0; u < kMrzUnroll; u++) {
            const uint64_t k = k0 + u * step;
            if (k >= n) break;
            const bool odd = __popcll(k & mask) & 1;
            // select the phase first: one product per amplitude
            const float eh2[2] = {odd ? h1[0] : h0[0], odd ? h1[1] : h0[1]};
            const float el2[2] = {odd ? l1[0] : l0[0], odd ? l1[1] : l0[1]};
            sv[k] = df_cmul(eh2, el2, cdf_split(v[u]));
        }
    }
}

// Dense 2^K x 2^K matrix, K = 3 or 4: one thread per group, the group's
// amplitudes in registers, the matrix in shared memory (read as broadcasts).
// complex128 products run in double-float on the FP32 pipe (matrix split
// into hi/lo floats: re.hi, re.lo, im.hi, im.lo per entry).
template <int K> struct DenseRegArgs {
    Masks mk;
    uint64_t ngroups;
    uint64_t off[1 << K];
};

template <class T, int K>
__global__ void __launch_bounds__(kThreads)
    k_dense_reg(c2_t<T> *__restrict__ sv, const DenseRegArgs<K> a, const ulonglong2 *__restrict__ mat_pk,
                const float2 *__restrict__ mat_f) {
    constexpr int D = 1 << K;
    using V = c2_t<T>;
    // complex128: packed double-float (two lanes per instruction), per entry
    // three 16-byte words {A.h, A.nh}, {A.nl, B.h}, {B.nh, B.nl} with
    // A = (mr, mr), B = (-mi, mi) (pack_entry_host), passed as mat_pk
    constexpr bool PK = sizeof(T) == 8;
    __shared__ __align__(16) ulonglong2 mp[PK ? 3 * D * D : 1];
    __shared__ __align__(8) float2 m2[PK ? 1 : D * D];
    for (int i = threadIdx.x; i < (PK ? 3 : 1) * D * D; i += blockDim.x) {
        if constexpr (PK) mp[i] = mat_pk[i];
        else m2[i] = mat_f[i];
    }
    __syncthreads();
    // one group per thread and no loop: a grid-stride loop would let the
    // compiler hoist all D*D matrix reads out of it into registers
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < a.ngroups) {
        const uint64_t base = group_base<K>(g, a.mk);
        V v[D];
#pragma unroll
        for (int i = 0; i < D; i++) v[i] = sv[base + a.off[i]];
        if constexpr (PK) {
            f2x vh[D], vl[D], wh[D], wl[D]; // v = (re, im), w = (im, re)
#pragma unroll
            for (int i = 0; i < D; i++) {
                const CDF c = cdf_split(v[i]);
                vh[i] = f2x_pack(c.re.hi, c.im.hi);
                vl[i] = f2x_pack(c.re.lo, c.im.lo);
                wh[i] = f2x_pack(c.im.hi, c.re.hi);
                wl[i] = f2x_pack(c.im.lo, c.re.lo);
            }
#pragma unroll
            for (int r = 0; r < D; r++) {
                f2x sh, sl;
#pragma unroll
                for (int c = 0; c < D; c++) {
                    const ulonglong2 q0 = mp[3 * (r * D + c)], q1 = mp[3 * (r * D + c) + 1],
                                     q2 = mp[3 * (r * D + c) + 2];
                    if (c == 0) df_first2(q0.x, q0.y, q1.x, vh[0], vl[0], sh, sl);
                    else df_mac2(q0.x, q0.y, q1.x, vh[c], vl[c], sh, sl);
                    df_mac2(q1.y, q2.x, q2.y, wh[c], wl[c], sh, sl);
                }
                float rh, ih, rl, il;
                f2x_unpack(sh, rh, ih);
                f2x_unpack(sl, rl, il);
                sv[base + a.off[r]] = make_double2(df_result(rh, rl), df_result(ih, il));
            }
        } else {
#pragma unroll
            for (int r = 0; r < D; r++) {
                float re = 0.0f, im = 0.0f;
#pragma unroll
                for (int c = 0; c < D; c++) {
                    const float2 e = m2[r * D + c];
                    re = fmaf(e.x, v[c].x, fmaf(-e.y, v[c].y, re));
                    im = fmaf(e.x, v[c].y, fmaf(e.y, v[c].x, im));
                }
                sv[base + a.off[r]] = make_float2(re, im);
            }
        }
    }
}

// Dense 2^k x 2^k matrix, k >= 3.  Rows r of `ngrp` groups are handled by one
// thread each; the group vectors are staged in shared memory, the matrix sits
// in shared memory when it fits (k <= kSmemMatWires) and is read through L2
// otherwise.
constexpr int kSmemMatWires = 5;

template <class T>
__global__ void __launch_bounds__(kThreads) k_dense(c2_t<T> *__restrict__ sv, const c2_t<T> *__restrict__ mat,
                                                     const uint64_t *__restrict__ off, Masks gm, int K,
                                                     uint64_t ngroups, int mat_in_smem) {
    using V = c2_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int dim = 1 << K;
    V *smat = reinterpret_cast<V *>(smem_raw);
    V *svec = smat + (mat_in_smem ? dim * dim : 0);
    if (mat_in_smem)
        for (int i = threadIdx.x; i < dim * dim; i += blockDim.x) smat[i] = mat[i];
    const V *M = mat_in_smem ? smat : mat;
    const int gpb = dim >= kThreads ? 1 : kThreads / dim; // groups per block iteration
    const int rows_per_thread = dim >= kThreads ? dim / kThreads : 1;
    for (uint64_t gb = (uint64_t)blockIdx.x * gpb; gb < ngroups; gb += (uint64_t)gridDim.x * gpb) {
        __syncthreads();
        // stage group vectors
        for (int t = threadIdx.x; t < gpb * dim; t += blockDim.x) {
            const int gi = t / dim, r = t % dim;
            const uint64_t g = gb + gi;
            if (g < ngroups) {
                uint64_t base = g & gm.m[0];
                for (int j = 1; j <= K; j++) base |= (g << j) & gm.m[j];
                svec[t] = sv[base + off[r]];
            }
        }
        __syncthreads();
        for (int rr = 0; rr < rows_per_thread; rr++) {
            const int t = threadIdx.x + rr * kThreads;
            const int gi = t / dim, r = t % dim;
            const uint64_t g = gb + gi;
            if (gi < gpb && g < ngroups) {
                const V *vec = svec + gi * dim;
                const V *row = M + (size_t)r * dim;
                T ar = 0, ai = 0;
                for (int j = 0; j < dim; j++) {
                    const V m = row[j], v = vec[j];
                    ar += m.x * v.x - m.y * v.y;
                    ai += m.x * v.y + m.y * v.x;
                }
                uint64_t base = g & gm.m[0];
                for (int j = 1; j <= K; j++) base |= (g << j) & gm.m[j];
                sv[base + off[r]] = mk<V>(ar, ai);
            }
        }
    }
}

// ------------------------------------------------------------- launchers --
template <class T> static int gate_grid(plk_state s, uint64_t work, int unroll) {
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(s->device, &d));
    const uint64_t per_block = (uint64_t)kThreads * unroll;
    uint64_t want = (work + per_block - 1) / per_block;
    const uint64_t cap = (uint64_t)d->sm_count * (d->max_threads_per_sm / kThreads) * 8;
    return (int)std::max<uint64_t>(1, std::min(want, cap));
}

template <class T, int OP, bool DFP>
static void launch_pair_k(plk_state s, int K, int grid, const PairArgs<T> &a) {
    auto *sv = (c2_t<T> *)s->data;
    switch (K) {
    case 1: k_pair<T, OP, 1, DFP><<<grid, kThreads, 0, s->stream>>>(sv, a); break;
    case 2: k_pair<T, OP, 2, DFP><<<grid, kThreads, 0, s->stream>>>(sv, a); break;
    case 3: k_pair<T, OP, 3, DFP><<<grid, kThreads, 0, s->stream>>>(sv, a); break;
    default: k_pair<T, OP, 4, DFP><<<grid, kThreads, 0, s->stream>>>(sv, a); break;
    }
}

// complex128 gates with arithmetic run on the FP32 pipe unless the native
// FP64 path is requested (c128_use_df() == false)
template <class T, int OP>
static void launch_pair_op(plk_state s, int K, int grid, const PairArgs<T> &a) {
    if constexpr (std::is_same_v<T, double> && pair_has_df<OP>()) {
        if (c128_use_df()) {
            launch_pair_k<T, OP, true>(s, K, grid, a);
            return;
        }
    }
    launch_pair_k<T, OP, false>(s, K, grid, a);
}

template <class T> static int run_pair(plk_state s, const GatePlan &p, const WireGeom &g) {
    PairArgs<T> a;
    a.mk = g.mk;
    a.ngroups = s->length >> p.K;
    a.offA = g.local_off(p.a);
    a.offB = g.local_off(p.b);
    a.n_extra = p.n_extra;
    a.extra_mode = p.extra_mode;
    for (int j = 0; j < p.n_extra; j++) a.off_extra[j] = g.local_off(p.extra_idx[j]);
    for (int j = 0; j < 8; j++) {
        a.coef[j] = (T)p.coef[j];
        df_split_host(p.coef[j], a.ch[j], a.cl[j]);
    }
    a.e[0] = (T)p.extra_e[0];
    a.e[1] = (T)p.extra_e[1];
    df_split_host(p.extra_e[0], a.eh[0], a.el[0]);
    df_split_host(p.extra_e[1], a.eh[1], a.el[1]);
    const int grid = gate_grid<T>(s, a.ngroups, kUnroll);
    switch (p.op) {
    case P_SWAP: launch_pair_op<T, P_SWAP>(s, p.K, grid, a); break;
    case P_Y: launch_pair_op<T, P_Y>(s, p.K, grid, a); break;
    case P_H: launch_pair_op<T, P_H>(s, p.K, grid, a); break;
    case P_RX: launch_pair_op<T, P_RX>(s, p.K, grid, a); break;
    case P_RY: launch_pair_op<T, P_RY>(s, p.K, grid, a); break;
    case P_MAT: launch_pair_op<T, P_MAT>(s, p.K, grid, a); break;
    case P_DIAG: launch_pair_op<T, P_DIAG>(s, p.K, grid, a); break;
    case P_PHASE_Y: launch_pair_op<T, P_PHASE_Y>(s, p.K, grid, a); break;
    case P_ZERO: launch_pair_op<T, P_ZERO>(s, p.K, grid, a); break;
    case P_GEN_SWAPI: launch_pair_op<T, P_GEN_SWAPI>(s, p.K, grid, a); break;
    case P_ZERO_Y: launch_pair_op<T, P_ZERO_Y>(s, p.K, grid, a); break;
    case P_NEG_Y: launch_pair_op<T, P_NEG_Y>(s, p.K, grid, a); break;
    case P_MULI_Y: launch_pair_op<T, P_MULI_Y>(s, p.K, grid, a); break;
    default: PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "internal: bad pair op");
    }
    PLK_CHECK_LAUNCH();
    return PLK_OK;
}

template <class T, int OP> static void launch_quad_op(plk_state s, int grid, const QuadArgs<T> &a) {
    auto *sv = (c2_t<T> *)s->data;
    if constexpr (std::is_same_v<T, double> && quad_has_df<OP>()) {
        if (c128_use_df()) {
            k_quad<T, OP, true><<<grid, kThreads, 0, s->stream>>>(sv, a);
            return;
        }
    }
    k_quad<T, OP, false><<<grid, kThreads, 0, s->stream>>>(sv, a);
}

template <class T> static int run_quad(plk_state s, const GatePlan &p, const WireGeom &g) {
    QuadArgs<T> a;
    a.mk = g.mk;
    a.ngroups = s->length >> 2;
    for (int i = 0; i < 4; i++) a.off[i] = g.local_off(i);
    for (int j = 0; j < 32; j++) {
        a.coef[j] = (T)p.coef[j];
        df_split_host(p.coef[j], a.ch[j], a.cl[j]);
    }
    quad_pack_host(a.ch, a.cl, a.pk);
    const int grid = gate_grid<T>(s, a.ngroups, 1);
    switch (p.op) {
    case Q_IXX: launch_quad_op<T, Q_IXX>(s, grid, a); break;
    case Q_IYY: launch_quad_op<T, Q_IYY>(s, grid, a); break;
    case Q_DIAG: launch_quad_op<T, Q_DIAG>(s, grid, a); break;
    case Q_MAT: launch_quad_op<T, Q_MAT>(s, grid, a); break;
    case Q_GEN_IXX: launch_quad_op<T, Q_GEN_IXX>(s, grid, a); break;
    case Q_GEN_IYY: launch_quad_op<T, Q_GEN_IYY>(s, grid, a); break;
    default: PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "internal: bad quad op");
    }
    PLK_CHECK_LAUNCH();
    return PLK_OK;
}

int run_plan(plk_state s, const GatePlan &p, const int64_t *wires) {
    if (p.family == GatePlan::F_NOOP) return PLK_OK;
    WireGeom g;
    if (p.K > kMaxDenseWires && p.family != GatePlan::F_MRZ && p.family != GatePlan::F_GEN_MRZ)
        PLK_FAIL(PLK_ERR_UNSUPPORTED, "too many wires");
    if (p.family == GatePlan::F_MRZ || p.family == GatePlan::F_GEN_MRZ) {
        uint64_t mask = 0;
        for (int j = 0; j < p.K; j++) mask |= 1ULL << (s->nq - 1 - (int)wires[j]);
        const int grid = s->dtype == PLK_C64 ? gate_grid<float>(s, s->length, kMrzUnroll)
                                             : gate_grid<double>(s, s->length, kMrzUnroll);
        const bool gen = p.family == GatePlan::F_GEN_MRZ;
        if (s->dtype == PLK_C64) {
            if (gen) k_mrz<float, true><<<grid, kThreads, 0, s->stream>>>((float2 *)s->data, s->length, mask, 0, 0, 0, 0);
            else k_mrz<float, false><<<grid, kThreads, 0, s->stream>>>((float2 *)s->data, s->length, mask,
                                                                       (float)p.coef[0], (float)p.coef[1],
                                                                       (float)p.coef[2], (float)p.coef[3]);
        } else {
            if (gen) k_mrz<double, true><<<grid, kThreads, 0, s->stream>>>((double2 *)s->data, s->length, mask, 0, 0, 0, 0);
            else if (c128_use_df()) {
                float4 eh, el;
                df_split_host(p.coef[0], eh.x, el.x);
                df_split_host(p.coef[1], eh.y, el.y);
                df_split_host(p.coef[2], eh.z, el.z);
                df_split_host(p.coef[3], eh.w, el.w);
                k_mrz_df<<<grid, kThreads, 0, s->stream>>>((double2 *)s->data, s->length, mask, eh, el);
            } else
                k_mrz<double, false><<<grid, kThreads, 0, s->stream>>>((double2 *)s->data, s->length, mask, p.coef[0],
                                                                       p.coef[1], p.coef[2], p.coef[3]);
        }
        PLK_CHECK_LAUNCH();
        return PLK_OK;
    }
    wire_geom(s->nq, wires, p.K, g);
    if (p.family == GatePlan::F_PAIR)
        return s->dtype == PLK_C64 ? run_pair<float>(s, p, g) : run_pair<double>(s, p, g);
    if (p.family == GatePlan::F_QUAD)
        return s->dtype == PLK_C64 ? run_quad<float>(s, p, g) : run_quad<double>(s, p, g);
    PLK_FAIL(PLK_ERR_UNSUPPORTED, "internal: bad plan family");
}

template <class T, int K>
static int launch_dense_reg(plk_state s, const std::vector<c2_t<T>> &hm, const WireGeom &g) {
    constexpr int D = 1 << K;
    DenseRegArgs<K> a;
    a.mk = g.mk;
    a.ngroups = s->length >> K;
    for (int i = 0; i < D; i++) a.off[i] = g.local_off(i);
    constexpr bool PK = sizeof(T) == 8; // packed double-float (k_dense_reg)
    std::vector<float4> mdf(sizeof(T) == 8 ? D * D : 0);
    std::vector<float2> mf(sizeof(T) == 8 ? 0 : D * D);
    std::vector<f2x> mpk(PK ? 6 * D * D : 0);
    for (int i = 0; i < D * D; i++) {
        if constexpr (sizeof(T) == 8) {
            df_split_host(hm[i].x, mdf[i].x, mdf[i].y);
            df_split_host(hm[i].y, mdf[i].z, mdf[i].w);
        } else {
            mf[i] = make_float2((float)hm[i].x, (float)hm[i].y);
        }
    }
    if constexpr (PK) {
        // per entry {A.h, A.nh}, {A.nl, B.h}, {B.nh, B.nl}; A = (mr, mr), B = (-mi, mi)
        for (int i = 0; i < D * D; i++) {
            f2x w[6];
            pack_entry_host(mdf[i].x, mdf[i].y, mdf[i].z, mdf[i].w, w);
            std::copy(w, w + 6, mpk.begin() + 6 * i);
        }
    }
    const size_t bytes = PK ? sizeof(f2x) * mpk.size() : sizeof(T) == 8 ? sizeof(float4) * D * D : sizeof(float2) * D * D;
    void *d_mat = nullptr;
    PLK_TRY(pool_alloc(s->device, &d_mat, bytes, s->stream));
    const void *src = PK ? (const void *)mpk.data() : sizeof(T) == 8 ? (const void *)mdf.data() : (const void *)mf.data();
    cudaError_t e = cudaMemcpyAsync(d_mat, src, bytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) {
        const unsigned grid = (unsigned)((a.ngroups + kThreads - 1) / kThreads);
        k_dense_reg<T, K><<<grid, kThreads, 0, s->stream>>>((c2_t<T> *)s->data, a, (const ulonglong2 *)d_mat,
                                                            (const float2 *)d_mat);
        e = cudaGetLastError();
    }
    pool_free(d_mat, s->stream);
    // the host staging vectors are released on return: make the copy finish
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) PLK_FAIL(PLK_ERR_CUDA, std::string("dense matrix kernel: ") + cudaGetErrorString(e));
    return PLK_OK;
}

template <class T>
static int run_dense_reg(plk_state s, const std::vector<c2_t<T>> &hm, const WireGeom &g, int K) {
    return K == 3 ? launch_dense_reg<T, 3>(s, hm, g) : launch_dense_reg<T, 4>(s, hm, g);
}

// Dense matrix application (any k <= kMaxDenseWires).  `matrix` is complex128
// row-major on the host; the adjoint is applied as the conjugate transpose.
template <class T>
static int run_dense(plk_state s, const double *matrix, const int64_t *wires, int K, bool adj) {
    using V = c2_t<T>;
    const int dim = 1 << K;
    std::vector<V> hm((size_t)dim * dim);
    for (int r = 0; r < dim; r++)
        for (int c = 0; c < dim; c++) {
            const size_t src = adj ? ((size_t)c * dim + r) : ((size_t)r * dim + c);
            const double re = matrix[2 * src], im = adj ? -matrix[2 * src + 1] : matrix[2 * src + 1];
            hm[(size_t)r * dim + c] = mk<V>((T)re, (T)im);
        }
    WireGeom g;
    wire_geom(s->nq, wires, K, g);
    // 3 and 4 wires: one group per thread (complex128 in packed double-float;
    // native-FP64 mode takes the generic kernel below)
    if ((K == 3 || K == 4) && (sizeof(T) == 4 || c128_use_df())) return run_dense_reg<T>(s, hm, g, K);
    std::vector<uint64_t> hoff(dim);
    for (int i = 0; i < dim; i++) hoff[i] = g.local_off(i);
    // complex64 on 5 or 6 wires: tensor cores (dense_tc.cu)
    if constexpr (sizeof(T) == 4)
        if ((K == 5 || K == 6) && dense_tc_enabled())
            return launch_dense_tc(s, reinterpret_cast<const float2 *>(hm.data()), hoff.data(), g.mk, K);
    // complex128: double-float on the FP32 pipe unless native FP64 is requested
    if constexpr (sizeof(T) == 8)
        if (c128_use_df()) {
            std::vector<float4> mt((size_t)dim * dim);
            for (int r = 0; r < dim; r++)
                for (int c = 0; c < dim; c++) {
                    const V z = hm[(size_t)r * dim + c];
                    float4 &f = mt[(size_t)c * dim + r];
                    df_split_host(z.x, f.x, f.y);
                    df_split_host(z.y, f.z, f.w);
                }
            const size_t mbytes = mt.size() * sizeof(float4), obytes = hoff.size() * sizeof(uint64_t);
            char *buf = nullptr;
            PLK_TRY(pool_alloc(s->device, (void **)&buf, mbytes + obytes, s->stream));
            cudaError_t e = cudaMemcpyAsync(buf, mt.data(), mbytes, cudaMemcpyHostToDevice, s->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(buf + mbytes, hoff.data(), obytes, cudaMemcpyHostToDevice, s->stream);
            const uint64_t ngroups = s->length >> K;
            const int mat_smem = K <= kSmemMatWiresDf ? 1 : 0;
            const int gpb = dim >= kThreads ? 1 : kThreads / dim;
            const size_t smem = (mat_smem ? mbytes : 0) + (size_t)gpb * dim * sizeof(float4);
            DeviceCtx *d = nullptr;
            if (e == cudaSuccess && smem > 48 * 1024)
                e = cudaFuncSetAttribute(k_dense_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess && device_ctx(s->device, &d) == PLK_OK) {
                const uint64_t want = (ngroups + gpb - 1) / gpb;
                const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)d->sm_count * 8));
                k_dense_df<<<grid, kThreads, smem, s->stream>>>((double2 *)s->data, (const float4 *)buf,
                                                                 (const uint64_t *)(buf + mbytes), g.mk, K, ngroups,
                                                                 mat_smem);
                e = cudaGetLastError();
            }
            pool_free(buf, s->stream);
            // the host staging vectors are released on return: make the copies finish
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e != cudaSuccess) PLK_FAIL(PLK_ERR_CUDA, std::string("dense matrix kernel: ") + cudaGetErrorString(e));
            return PLK_OK;
        }
    void *d_mat = nullptr, *d_off = nullptr;
    PLK_CUDA(cudaMallocAsync(&d_mat, hm.size() * sizeof(V), s->stream));
    PLK_CUDA(cudaMallocAsync(&d_off, hoff.size() * sizeof(uint64_t), s->stream));
    PLK_CUDA(cudaMemcpyAsync(d_mat, hm.data(), hm.size() * sizeof(V), cudaMemcpyHostToDevice, s->stream));
    PLK_CUDA(cudaMemcpyAsync(d_off, hoff.data(), hoff.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, s->stream));
    const uint64_t ngroups = s->length >> K;
    const int mat_smem = K <= kSmemMatWires ? 1 : 0;
    const int gpb = dim >= kThreads ? 1 : kThreads / dim;
    const size_t smem = (mat_smem ? (size_t)dim * dim * sizeof(V) : 0) + (size_t)gpb * dim * sizeof(V);
    if (smem > 48 * 1024)
        PLK_CUDA(cudaFuncSetAttribute(k_dense<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(s->device, &d));
    const uint64_t want = (ngroups + gpb - 1) / gpb;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)d->sm_count * 8));
    k_dense<T><<<grid, kThreads, smem, s->stream>>>((V *)s->data, (const V *)d_mat, (const uint64_t *)d_off, g.mk, K,
                                                    ngroups, mat_smem);
    PLK_CHECK_LAUNCH();
    PLK_CUDA(cudaFreeAsync(d_mat, s->stream));
    PLK_CUDA(cudaFreeAsync(d_off, s->stream));
    // the host staging vectors are released on return: make the copies finish
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    return PLK_OK;
}

int apply_matrix_impl(plk_state s, const double *matrix, const int64_t *wires, int nw, bool adj) {
    if (!matrix) PLK_FAIL(PLK_ERR_INVALID_ARG, "null matrix");
    if (nw < 1) PLK_FAIL(PLK_ERR_INVALID_ARG, "matrix needs at least one wire");
    if (nw > kMaxDenseWires)
        PLK_FAIL(PLK_ERR_UNSUPPORTED, "dense matrices on more than " + std::to_string(kMaxDenseWires) + " wires");
    PLK_TRY(check_wires(s, wires, nw));
    if (nw <= 2) {
        GatePlan p;
        std::memset(p.coef, 0, sizeof(p.coef));
        const int dim = 1 << nw;
        for (int r = 0; r < dim; r++)
            for (int c = 0; c < dim; c++) {
                const int src = adj ? (c * dim + r) : (r * dim + c);
                p.coef[2 * (r * dim + c)] = matrix[2 * src];
                p.coef[2 * (r * dim + c) + 1] = adj ? -matrix[2 * src + 1] : matrix[2 * src + 1];
            }
        if (nw == 1) set_pair(p, 1, P_MAT, 0, 1);
        else {
            p.family = GatePlan::F_QUAD;
            p.K = 2;
            p.op = Q_MAT;
        }
        return run_plan(s, p, wires);
    }
    return s->dtype == PLK_C64 ? run_dense<float>(s, matrix, wires, nw, adj)
                               : run_dense<double>(s, matrix, wires, nw, adj);
}

int apply_gate_impl(plk_state s, int gate, const int64_t *wires, int nw, bool adj, const double *params, int np,
                    const double *matrix) {
    if (gate == PLK_GATE_MATRIX) return apply_matrix_impl(s, matrix, wires, nw, adj);
    GatePlan p;
    PLK_TRY(plan_gate(gate, nw, adj, params, np, p));
    if (p.family == GatePlan::F_NOOP) return PLK_OK;
    PLK_TRY(check_wires(s, wires, nw));
    return run_plan(s, p, wires);
}

} // namespace plk

using namespace plk;

extern "C" {

PLK_API int plk_gate_from_name(const char *name, int32_t *gate) {
    if (!name || !gate) PLK_FAIL(PLK_ERR_INVALID_ARG, "null argument");
    for (int i = 0; i < PLK_GATE_MATRIX; i++)
        if (std::strcmp(kGates[i].name, name) == 0) {
            *gate = i;
            return PLK_OK;
        }
    *gate = -1;
    PLK_FAIL(PLK_ERR_UNKNOWN_GATE, std::string("unknown gate name ") + name);
}

PLK_API int plk_gate_num_wires(int32_t gate) {
    if (gate < 0 || gate >= PLK_GATE_COUNT) return 0;
    return kGates[gate].nwires;
}

PLK_API int plk_gate_num_params(int32_t gate) {
    if (gate < 0 || gate >= PLK_GATE_COUNT) return 0;
    return kGates[gate].nparams;
}

PLK_API int plk_apply_gate(plk_state s, int32_t gate, const int64_t *wires, int32_t nw, int32_t adjoint,
                           const double *params, int32_t np) {
    PLK_TRY(check_state(s));
    PLK_CUDA(cudaSetDevice(s->device));
    if (gate == PLK_GATE_MATRIX) PLK_FAIL(PLK_ERR_INVALID_ARG, "use plk_apply_matrix for dense matrices");
    return apply_gate_impl(s, gate, wires, nw, adjoint != 0, params, np, nullptr);
}

PLK_API int plk_apply_matrix(plk_state s, const double *matrix, const int64_t *wires, int32_t nw, int32_t adjoint) {
    PLK_TRY(check_state(s));
    PLK_CUDA(cudaSetDevice(s->device));
    return apply_matrix_impl(s, matrix, wires, nw, adjoint != 0);
}

PLK_API int plk_apply_ops(plk_state s, const plk_op *ops, int32_t nops) {
    PLK_TRY(check_state(s));
    if (nops > 0 && !ops) PLK_FAIL(PLK_ERR_INVALID_ARG, "null ops");
    PLK_CUDA(cudaSetDevice(s->device));
    {
        bool handled = false;
        PLK_TRY(window_apply_ops(s, ops, nops, handled));
        if (handled) return PLK_OK;
    }
    for (int i = 0; i < nops; i++) {
        const plk_op &o = ops[i];
        int st = apply_gate_impl(s, o.gate, o.wires, o.num_wires, o.adjoint != 0, o.params, o.num_params, o.matrix);
        if (st != PLK_OK) {
            set_error("op " + std::to_string(i) + ": " + last_error());
            return st;
        }
    }
    return PLK_OK;
}

PLK_API int plk_apply_generator(plk_state s, int32_t gate, const int64_t *wires, int32_t nw, int32_t adjoint,
                                double *scale) {
    (void)adjoint;
    PLK_TRY(check_state(s));
    PLK_CUDA(cudaSetDevice(s->device));
    GatePlan p;
    PLK_TRY(plan_generator(gate, nw, p));
    PLK_TRY(check_wires(s, wires, nw));
    PLK_TRY(run_plan(s, p, wires));
    if (scale) *scale = p.scale;
    return PLK_OK;
}

} // extern "C"
