// window_host.cuh — host side of the register-window engine: dense gate
// matrices from the gate plans, their trigonometric fit in the parameter,
// expanded ops, and the compiler that packs an op sequence into 4-qubit
// register windows (used for batches and for single large states).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "batch_engine.cuh"
#include "gate_ops.cuh"

namespace plk {

int plan_gate(int gate, int nw, bool inv, const double *prm, int np, GatePlan &p);
int plan_generator(int gate, int nw, GatePlan &p);

// ------------------------------------------------------- dense gate plans --
// Applies a plan to the local amplitudes v[0 .. 2^K) (bit K-1-j <-> wires[j]).
inline void apply_plan_host(const GatePlan &p, int K, double2 *v) {
    const int D = 1 << K;
    switch (p.family) {
    case GatePlan::F_NOOP: return;
    case GatePlan::F_PAIR: {
        double2 &x = v[p.a], &y = v[p.b];
        switch (p.op) {
        case P_SWAP: pair_op<P_SWAP>(x, y, p.coef); break;
        case P_Y: pair_op<P_Y>(x, y, p.coef); break;
        case P_H: pair_op<P_H>(x, y, p.coef); break;
        case P_RX: pair_op<P_RX>(x, y, p.coef); break;
        case P_RY: pair_op<P_RY>(x, y, p.coef); break;
        case P_MAT: pair_op<P_MAT>(x, y, p.coef); break;
        case P_DIAG: pair_op<P_DIAG>(x, y, p.coef); break;
        case P_PHASE_Y: pair_op<P_PHASE_Y>(x, y, p.coef); break;
        case P_ZERO: pair_op<P_ZERO>(x, y, p.coef); break;
        case P_GEN_SWAPI: pair_op<P_GEN_SWAPI>(x, y, p.coef); break;
        case P_ZERO_Y: pair_op<P_ZERO_Y>(x, y, p.coef); break;
        case P_NEG_Y: pair_op<P_NEG_Y>(x, y, p.coef); break;
        case P_MULI_Y: pair_op<P_MULI_Y>(x, y, p.coef); break;
        default: break;
        }
        for (int i = 0; i < p.n_extra; i++) {
            double2 &e = v[p.extra_idx[i]];
            if (p.extra_mode == X_PHASE) e = cmul(e, mk<double2>(p.extra_e[0], p.extra_e[1]));
            else if (p.extra_mode == X_ZERO) e = mk<double2>(0, 0);
        }
        return;
    }
    case GatePlan::F_QUAD: {
        double2 q[4] = {v[0], v[1], v[2], v[3]};
        switch (p.op) {
        case Q_IXX: quad_op<Q_IXX>(q, p.coef); break;
        case Q_IYY: quad_op<Q_IYY>(q, p.coef); break;
        case Q_DIAG: quad_op<Q_DIAG>(q, p.coef); break;
        case Q_MAT: quad_op<Q_MAT>(q, p.coef); break;
        case Q_GEN_IXX: quad_op<Q_GEN_IXX>(q, p.coef); break;
        case Q_GEN_IYY: quad_op<Q_GEN_IYY>(q, p.coef); break;
        default: break;
        }
        for (int i = 0; i < 4; i++) v[i] = q[i];
        return;
    }
    case GatePlan::F_MRZ:
        for (int i = 0; i < D; i++) {
            const bool odd = __builtin_popcount((unsigned)i) & 1;
            v[i] = cmul(v[i], odd ? mk<double2>(p.coef[2], p.coef[3]) : mk<double2>(p.coef[0], p.coef[1]));
        }
        return;
    case GatePlan::F_GEN_MRZ:
        for (int i = 0; i < D; i++)
            if (__builtin_popcount((unsigned)i) & 1) v[i] = cneg(v[i]);
        return;
    default: return;
    }
}

inline void plan_dense(const GatePlan &p, int K, std::vector<double2> &M) {
    const int D = 1 << K;
    M.assign((size_t)D * D, mk<double2>(0, 0));
    std::vector<double2> v(D);
    for (int c = 0; c < D; c++) {
        std::fill(v.begin(), v.end(), mk<double2>(0, 0));
        v[c] = mk<double2>(1, 0);
        apply_plan_host(p, K, v.data());
        for (int r = 0; r < D; r++) M[(size_t)r * D + c] = v[r];
    }
}

inline int gate_dense(int gate, int K, bool inv, double theta, std::vector<double2> &M) {
    GatePlan p;
    const double prm[3] = {theta, 0.0, 0.0};
    PLK_TRY(plan_gate(gate, K, inv, prm, 3, p));
    plan_dense(p, p.family == GatePlan::F_NOOP ? K : (p.K > 0 ? p.K : K), M);
    return PLK_OK;
}

inline void trig5(double th, double *f) {
    f[0] = 1.0;
    f[1] = std::cos(th / 2);
    f[2] = std::sin(th / 2);
    f[3] = std::cos(th);
    f[4] = std::sin(th);
}

// Coefficient matrices A0..A4 of U(theta) (D*D complex each).
inline int fit_gate(int gate, int K, bool inv, int nparams, std::vector<double2> &A) {
    const int D = 1 << K;
    const size_t DD = (size_t)D * D;
    A.assign(5 * DD, mk<double2>(0, 0));
    std::vector<double2> U;
    if (nparams == 0) {
        PLK_TRY(gate_dense(gate, K, inv, 0.0, U));
        std::copy(U.begin(), U.end(), A.begin());
        return PLK_OK;
    }
    static const double th[5] = {0.37, 1.61, 2.83, 4.07, 5.51};
    double F[5][5];
    std::vector<std::vector<double2>> R(5);
    for (int k = 0; k < 5; k++) {
        trig5(th[k], F[k]);
        PLK_TRY(gate_dense(gate, K, inv, th[k], R[k]));
    }
    // Gaussian elimination with partial pivoting on F, applied to every entry
    int perm[5] = {0, 1, 2, 3, 4};
    for (int c = 0; c < 5; c++) {
        int piv = c;
        for (int r = c + 1; r < 5; r++)
            if (std::fabs(F[r][c]) > std::fabs(F[piv][c])) piv = r;
        if (piv != c) {
            for (int j = 0; j < 5; j++) std::swap(F[c][j], F[piv][j]);
            std::swap(R[c], R[piv]);
            std::swap(perm[c], perm[piv]);
        }
        for (int r = c + 1; r < 5; r++) {
            const double f = F[r][c] / F[c][c];
            for (int j = c; j < 5; j++) F[r][j] -= f * F[c][j];
            for (size_t e = 0; e < DD; e++) {
                R[r][e].x -= f * R[c][e].x;
                R[r][e].y -= f * R[c][e].y;
            }
        }
    }
    for (int i = 4; i >= 0; i--) {
        for (size_t e = 0; e < DD; e++) {
            double re = R[i][e].x, im = R[i][e].y;
            for (int j = i + 1; j < 5; j++) {
                re -= F[i][j] * A[j * DD + e].x;
                im -= F[i][j] * A[j * DD + e].y;
            }
            A[i * DD + e] = mk<double2>(re / F[i][i], im / F[i][i]);
        }
    }
    for (auto &z : A) {
        if (std::fabs(z.x) < 1e-15) z.x = 0.0;
        if (std::fabs(z.y) < 1e-15) z.y = 0.0;
    }
    // check the fit at angles it was not fitted on
    for (double t : {0.9, 3.3, -2.2}) {
        double f[5];
        trig5(t, f);
        PLK_TRY(gate_dense(gate, K, inv, t, U));
        for (size_t e = 0; e < DD; e++) {
            double re = 0, im = 0;
            for (int i = 0; i < 5; i++) {
                re += f[i] * A[i * DD + e].x;
                im += f[i] * A[i * DD + e].y;
            }
            if (std::fabs(re - U[e].x) > 1e-12 || std::fabs(im - U[e].y) > 1e-12)
                PLK_FAIL(PLK_ERR_UNSUPPORTED, "internal: gate matrix is not of degree one in theta/2");
        }
    }
    return PLK_OK;
}

// -------------------------------------------------------- host structures --
struct EPrep {
    int32_t basis; // complex offset of the 5 coefficient blocks
    int32_t pidx;  // flat parameter index, -1 for constant ops
    int32_t out;   // complex offset of the output in the matrix buffer
    uint8_t K, kind, conjT, pad;
    uint8_t perm[4]; // DENSE: canonical bit of wires[j]
};

struct XOp { // an op after expansion (Rot -> RZ RY RZ)
    int gate;
    int K;
    int wires[4];
    std::vector<int> mrz_wires; // MultiRZ
    bool inv;
    int pidx;   // flat parameter index in the batch, -1 if none
    int slot;   // Jacobian slot in the circuit, -1 if not trainable
    int kind;   // EK_*
    int basis;  // basis offset (complex)
    int user_matrix; // index into the batch's user matrices, -1 if none
    std::vector<double2> umat; // single states: the op's matrix (gate order, D x D; MultiRZ: its 2 x 2 diagonal)
};

inline bool is_diag_gate(int g) {
    switch (g) {
    case PLK_GATE_PAULIZ: case PLK_GATE_S: case PLK_GATE_T: case PLK_GATE_PHASESHIFT: case PLK_GATE_RZ:
    case PLK_GATE_CZ: case PLK_GATE_CONTROLLEDPHASESHIFT: case PLK_GATE_CRZ: case PLK_GATE_ISINGZZ:
        return true;
    default: return false;
    }
}


// ----------------------------------------------------------- compilation --
struct WinBuilder {
    int nq;
    bool bwd;
    std::vector<EWin> &wins;
    std::vector<EOp> &ops;
    std::vector<ETrain> &train;
    std::vector<EPrep> &prep;
    std::vector<double2> &gen;
    int64_t &n_mats;
    std::vector<double2> *hmats = nullptr; // when set: matrices from XOp::umat, written here (no EPrep)
    // merge runs of diagonal ops on register bits into EK_DIAGSET ops (needs
    // hmats; only the single-state window kernels implement the kind)
    bool fuse_diag = false;

    std::vector<const XOp *> cur;
    uint32_t wbits = 0; // state bits of the open window
    int ntrain = 0;

    static int popc(uint32_t x) { return __builtin_popcount(x); }

    uint32_t need(const XOp &o) const {
        if (o.kind == EK_DIAG || o.kind == EK_PARITY) return 0;
        uint32_t m = 0;
        for (int j = 0; j < o.K; j++) m |= 1u << (nq - 1 - o.wires[j]);
        return m;
    }

    int add(const XOp &o) {
        const uint32_t m = need(o);
        const bool tr = bwd && o.slot >= 0;
        if (!cur.empty() && (popc(wbits | m) > kWinBits || (int)cur.size() >= kMaxWinOps ||
                             (tr && ntrain >= kMaxWinTrain)))
            PLK_TRY(close());
        cur.push_back(&o);
        wbits |= m;
        if (tr) ntrain++;
        return PLK_OK;
    }

    bool fits(const XOp &o) const {
        const bool tr = bwd && o.slot >= 0;
        return popc(wbits | need(o)) <= kWinBits && (int)cur.size() < kMaxWinOps && !(tr && ntrain >= kMaxWinTrain);
    }

    // Packs `seq` (ops in application order) into windows, reordering ops
    // that commute: an op may move ahead of earlier ops that share none of
    // its wires (disjoint-wire ops commute, and so does the adjoint: a
    // commuting U_m leaves <U_m H lambda | G U_m lambda> unchanged).  The
    // schedule is a list schedule of the wire-dependency graph: the open
    // window first takes ready ops that add no window bits, then the
    // earliest ready op that still fits; when none fits it is closed.
    int add_scheduled(const std::vector<const XOp *> &seq) {
        const int n = (int)seq.size();
        std::vector<std::vector<int>> succ(n);
        std::vector<int> indeg(n, 0);
        std::vector<int> last(32, -1);
        for (int i = 0; i < n; i++) {
            const XOp &o = *seq[i];
            int ws[32];
            int nw = 0;
            if (o.kind == EK_PARITY)
                for (int w : o.mrz_wires) ws[nw++] = w;
            else
                for (int j = 0; j < o.K; j++) ws[nw++] = o.wires[j];
            for (int j = 0; j < nw; j++) {
                const int p = last[ws[j]];
                if (p >= 0 && (succ[p].empty() || succ[p].back() != i)) {
                    succ[p].push_back(i);
                    indeg[i]++;
                }
                last[ws[j]] = i;
            }
        }
        std::vector<int> ready; // kept sorted by original index
        for (int i = 0; i < n; i++)
            if (indeg[i] == 0) ready.push_back(i);
        int done = 0;
        while (done < n) {
            int pick = -1;
            for (size_t r = 0; r < ready.size() && pick < 0; r++) // free ops first
                if ((need(*seq[ready[r]]) & ~wbits) == 0 && fits(*seq[ready[r]])) pick = (int)r;
            for (size_t r = 0; r < ready.size() && pick < 0; r++)
                if (fits(*seq[ready[r]])) pick = (int)r;
            if (pick < 0) {
                PLK_TRY(close());
                continue;
            }
            const int i = ready[pick];
            ready.erase(ready.begin() + pick);
            PLK_TRY(add(*seq[i]));
            done++;
            for (int s2 : succ[i])
                if (--indeg[s2] == 0) ready.insert(std::lower_bound(ready.begin(), ready.end(), s2), s2);
        }
        return PLK_OK;
    }

    // ------------------------------------------------ diagonal-run fusion --
    static bool is_diagonal(const XOp &o) { return o.kind == EK_DIAG || o.kind == EK_PARITY; }

    uint32_t state_bits(const XOp &o) const {
        uint32_t m = 0;
        if (o.kind == EK_PARITY)
            for (int wv : o.mrz_wires) m |= 1u << (nq - 1 - wv);
        else
            for (int j = 0; j < o.K; j++) m |= 1u << (nq - 1 - o.wires[j]);
        return m;
    }

    // Diagonal ops commute with each other; any two ops on disjoint wires
    // commute.  Moving a diagonal op past an op it commutes with leaves every
    // adjoint inner product unchanged: both states get the same unit-modulus
    // phases, which cancel in <H lambda | G lambda> for a diagonal G, and a
    // disjoint op commutes with the other op's generator.
    bool commute(const XOp &a, const XOp &b) const {
        return (is_diagonal(a) && is_diagonal(b)) || (state_bits(a) & state_bits(b)) == 0;
    }

    // a diagonal op whose phases depend only on the window's register bits;
    // trainable ones only as one-wire members (their generator is a sign per
    // register-bit value)
    bool mergeable(const XOp &o, uint32_t w) const {
        if (!is_diagonal(o) || (state_bits(o) & ~w) != 0) return false;
        return !(bwd && o.slot >= 0) || (o.kind == EK_DIAG && o.K == 1);
    }

    // moves each diagonal op toward dir (-1: earlier, +1: later) past ops it
    // commutes with, until it meets another diagonal op or an op it does not
    // commute with; returns the order and the number of ops merging removes
    std::vector<const XOp *> bubble(int dir, uint32_t w, int &saved) const {
        std::vector<const XOp *> v = cur;
        const int n = (int)v.size();
        for (int t = 0; t < n; t++) {
            const int i = dir < 0 ? t : n - 1 - t;
            if (!is_diagonal(*v[i])) continue;
            int k = i;
            while (k + dir >= 0 && k + dir < n && !is_diagonal(*v[k + dir]) && commute(*v[k + dir], *v[k])) {
                std::swap(v[k + dir], v[k]);
                k += dir;
            }
        }
        saved = 0;
        for (int i = 0; i < n;) {
            int j = i, m = 0;
            while (j < n && is_diagonal(*v[j])) m += mergeable(*v[j++], w) ? 1 : 0;
            if (m >= 2) saved += m - 1;
            i = j > i ? j : i + 1;
        }
        return v;
    }

    int close() {
        if (cur.empty()) return PLK_OK;
        // pad with the highest unused state bits (low bits stay with the
        // threads, which keeps global accesses coalesced)
        uint32_t w = wbits;
        for (int bit = nq - 1; bit >= 0 && popc(w) < kWinBits; bit--) w |= 1u << bit;
        EWin win;
        int r = 0;
        int pos[32];
        for (int bit = 0; bit < nq; bit++)
            if (w >> bit & 1) {
                win.rb[r] = (uint8_t)bit;
                pos[bit] = r++;
            }
        win.flags = 1;
        for (const XOp *op : cur)
            if (!((op->kind == EK_DENSE && op->K == 1) || op->kind == EK_CX || (op->kind == EK_DIAG && op->K == 1)))
                win.flags = 0;
        // runs of diagonal ops on register bits become one phase table each
        std::vector<std::vector<const XOp *>> groups; // emitted units: one op, or a merged run
        if (fuse_diag && hmats) {
            int s_left = 0, s_right = 0;
            std::vector<const XOp *> vl = bubble(-1, w, s_left), vr = bubble(+1, w, s_right);
            const std::vector<const XOp *> &v = s_left >= s_right ? vl : vr;
            for (size_t i = 0; i < v.size();) {
                if (!is_diagonal(*v[i])) {
                    groups.push_back({v[i++]});
                    continue;
                }
                std::vector<const XOp *> merge, rest;
                while (i < v.size() && is_diagonal(*v[i])) (mergeable(*v[i], w) ? merge : rest).push_back(v[i++]);
                // at most four trainable members per merged op
                std::vector<const XOp *> g;
                int ntr = 0;
                for (const XOp *o : merge) {
                    const bool tr = bwd && o->slot >= 0;
                    if (tr && ntr == 4) {
                        groups.push_back(g);
                        g.clear();
                        ntr = 0;
                    }
                    g.push_back(o);
                    ntr += tr ? 1 : 0;
                }
                if (!g.empty()) groups.push_back(g);
                for (const XOp *o : rest) groups.push_back({o});
            }
        } else {
            for (const XOp *op : cur) groups.push_back({op});
        }
        win.op0 = (int)ops.size();
        win.nops = (int)groups.size();
        win.tr0 = (int)train.size();
        win.ntrain = 0;
        for (const auto &grp : groups) {
            if (grp.size() > 1) {
                PLK_TRY(emit_diagset(grp, pos, win));
                continue;
            }
            const XOp &o = *grp[0];
            EOp e;
            std::memset(&e, 0, sizeof(e));
            e.kind = (uint8_t)o.kind;
            e.K = (uint8_t)o.K;
            e.red = 0xff;
            e.mat = -1;
            e.gen = -1;
            const int D = 1 << o.K;
            uint8_t perm[4] = {0, 0, 0, 0};
            if (o.kind == EK_CX) {
                const int rc = pos[nq - 1 - o.wires[0]], rt = pos[nq - 1 - o.wires[1]];
                e.sel = (uint8_t)(rc * 4 + rt);
            } else if (o.kind == EK_DENSE) {
                int rr[4], srt[4];
                for (int j = 0; j < o.K; j++) srt[j] = rr[j] = pos[nq - 1 - o.wires[j]];
                std::sort(srt, srt + o.K);
                for (int j = 0; j < o.K; j++) perm[j] = (uint8_t)(std::find(srt, srt + o.K, rr[j]) - srt);
                if (o.K == 1) {
                    const int form = o.gate == PLK_GATE_RX ? EF_RX : (o.gate == PLK_GATE_RY ? EF_RY : EF_GENERAL);
                    e.sel = (uint8_t)(srt[0] + 4 * form);
                }
                else if (o.K == 2) {
                    static const int a[6] = {0, 0, 0, 1, 1, 2}, c[6] = {1, 2, 3, 2, 3, 3};
                    for (int s = 0; s < 6; s++)
                        if (a[s] == srt[0] && c[s] == srt[1]) e.sel = (uint8_t)s;
                } else if (o.K == 3) {
                    e.sel = (uint8_t)(6 - srt[0] - srt[1] - srt[2]);
                } else {
                    e.sel = 0;
                }
            } else if (o.kind == EK_DIAG) {
                uint32_t bits = 0;
                for (int j = 0; j < o.K; j++) bits |= (uint32_t)(nq - 1 - o.wires[j]) << (5 * j);
                e.bits = bits;
                // one wire: its register bit (0..3), or 4 when the bit is fixed per thread
                const int b0 = nq - 1 - o.wires[0];
                e.sel = (uint8_t)(o.K == 1 && ((w >> b0) & 1u) ? pos[b0] : 4);
            } else { // parity
                uint32_t mask = 0;
                for (int wv : o.mrz_wires) mask |= 1u << (nq - 1 - wv);
                e.bits = mask;
            }
            if (o.kind != EK_CX && hmats) {
                // canonical matrix (DENSE) or diagonal (DIAG, PARITY) from the op's own matrix
                const int Dm = o.kind == EK_PARITY ? 2 : D;
                e.mat = (int32_t)n_mats;
                if (o.kind == EK_DENSE) {
                    for (int r2 = 0; r2 < D; r2++)
                        for (int c2 = 0; c2 < D; c2++) {
                            int gr = 0, gc = 0;
                            for (int j = 0; j < o.K; j++) {
                                gr |= ((r2 >> perm[j]) & 1) << (o.K - 1 - j);
                                gc |= ((c2 >> perm[j]) & 1) << (o.K - 1 - j);
                            }
                            double2 z = bwd ? o.umat[(size_t)gc * D + gr] : o.umat[(size_t)gr * D + gc];
                            if (bwd) z.y = -z.y;
                            hmats->push_back(z);
                        }
                    n_mats += (int64_t)D * D;
                } else {
                    for (int i2 = 0; i2 < Dm; i2++) {
                        double2 z = o.umat[(size_t)i2 * Dm + i2];
                        if (bwd) z.y = -z.y;
                        hmats->push_back(z);
                    }
                    n_mats += Dm;
                }
            } else if (o.kind != EK_CX) {
                EPrep p;
                std::memset(&p, 0, sizeof(p));
                p.basis = o.basis;
                p.pidx = o.pidx;
                p.out = (int32_t)n_mats;
                p.K = (uint8_t)(o.kind == EK_PARITY ? 1 : o.K);
                p.kind = (uint8_t)o.kind;
                p.conjT = bwd ? 1 : 0;
                std::memcpy(p.perm, perm, 4);
                prep.push_back(p);
                e.mat = (int32_t)n_mats;
                n_mats += o.kind == EK_DENSE ? (int64_t)D * D : (o.kind == EK_DIAG ? D : 2);
            }
            if (bwd && o.slot >= 0) {
                // generator (constant): canonical dense block or diagonal
                GatePlan gp;
                PLK_TRY(plan_generator(o.gate, o.kind == EK_PARITY ? (int)o.mrz_wires.size() : o.K, gp));
                float gscale = (float)(-2.0 * gp.scale * (o.inv ? -1.0 : 1.0));
                if (o.kind != EK_PARITY) {
                    std::vector<double2> G;
                    plan_dense(gp, o.K, G);
                    e.gen = (int32_t)gen.size();
                    if (o.kind == EK_DENSE && o.K == 1) {
                        // monomial pattern (rows of G in canonical order = gate order for one wire)
                        uint32_t pat = 0;
                        for (int r2 = 0; r2 < 2; r2++)
                            for (int c2 = 0; c2 < 2; c2++) {
                                const double2 z = G[(size_t)r2 * 2 + c2];
                                if (z.x == 0.0 && z.y == 0.0) continue;
                                const int q = z.x == 1.0 ? 0 : z.y == 1.0 ? 1 : z.x == -1.0 ? 2 : z.y == -1.0 ? 3 : -1;
                                if (q < 0 || (pat >> (4 * r2) & 1u))
                                    PLK_FAIL(PLK_ERR_UNSUPPORTED, "internal: generator is not a signed permutation");
                                pat |= (uint32_t)(1 | (c2 << 1) | (q << 2)) << (4 * r2);
                            }
                        e.bits = pat;
                    }
                    if (o.kind == EK_DENSE) {
                        for (int r2 = 0; r2 < D; r2++)
                            for (int c2 = 0; c2 < D; c2++) {
                                int gr = 0, gc = 0;
                                for (int j = 0; j < o.K; j++) {
                                    gr |= ((r2 >> perm[j]) & 1) << (o.K - 1 - j);
                                    gc |= ((c2 >> perm[j]) & 1) << (o.K - 1 - j);
                                }
                                gen.push_back(G[(size_t)gr * D + gc]);
                            }
                    } else { // diagonal generator
                        for (int i = 0; i < D; i++) gen.push_back(G[(size_t)i * D + i]);
                    }
                }
                e.red = (uint8_t)win.ntrain;
                train.push_back(ETrain{o.slot, gscale});
                win.ntrain++;
            }
            ops.push_back(e);
        }
        wins.push_back(win);
        cur.clear();
        wbits = 0;
        ntrain = 0;
        return PLK_OK;
    }

    // One EK_DIAGSET op: the product of the group's diagonals as 16 phases
    // over the register index, and its trainable one-wire members.
    int emit_diagset(const std::vector<const XOp *> &grp, const int *pos, EWin &win) {
        EOp e;
        std::memset(&e, 0, sizeof(e));
        e.kind = EK_DIAGSET;
        e.red = 0xff;
        e.mat = (int32_t)n_mats;
        double2 ph[kWinAmps];
        for (int j = 0; j < kWinAmps; j++) ph[j] = mk<double2>(1.0, 0.0);
        int nm = 0;
        for (const XOp *op : grp) {
            const XOp &o = *op;
            for (int j = 0; j < kWinAmps; j++) {
                int li = 0, Dm = 2;
                if (o.kind == EK_PARITY) {
                    int par = 0;
                    for (int wv : o.mrz_wires) par ^= (j >> pos[nq - 1 - wv]) & 1;
                    li = par;
                } else {
                    Dm = 1 << o.K;
                    for (int q = 0; q < o.K; q++) li |= ((j >> pos[nq - 1 - o.wires[q]]) & 1) << (o.K - 1 - q);
                }
                double2 z = o.umat[(size_t)li * Dm + li];
                if (bwd) z.y = -z.y;
                ph[j] = cmul(ph[j], z);
            }
            if (bwd && o.slot >= 0) {
                GatePlan gp;
                PLK_TRY(plan_generator(o.gate, 1, gp));
                std::vector<double2> G;
                plan_dense(gp, 1, G);
                auto code = [](double2 z) -> uint32_t {
                    if (z.y != 0.0 || (z.x != 0.0 && z.x != 1.0 && z.x != -1.0)) return 3u; // not a real sign
                    return z.x == 0.0 ? 0u : (z.x > 0.0 ? 1u : 2u);
                };
                const uint32_t c0 = code(G[0]), c1 = code(G[3]);
                if (c0 == 3u || c1 == 3u) PLK_FAIL(PLK_ERR_UNSUPPORTED, "internal: diagonal generator is not real");
                const int rbit = pos[nq - 1 - o.wires[0]];
                e.bits |= ((uint32_t)rbit | (c0 << 2) | (c1 << 4)) << (8 * nm);
                e.gen |= (int32_t)win.ntrain << (4 * nm);
                train.push_back(ETrain{o.slot, (float)(-2.0 * gp.scale * (o.inv ? -1.0 : 1.0))});
                win.ntrain++;
                nm++;
            }
        }
        e.K = (uint8_t)nm;
        for (int j = 0; j < kWinAmps; j++) hmats->push_back(ph[j]);
        n_mats += kWinAmps;
        ops.push_back(e);
        return PLK_OK;
    }
};

} // namespace plk
