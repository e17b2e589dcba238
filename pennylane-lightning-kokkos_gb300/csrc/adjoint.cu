// adjoint.cu — adjoint-method Jacobian with a fused backward step.
//
// Restates AdjointJacobianKokkos::adjointJacobian
// (algorithms/AdjointDiffKokkos.hpp:404-478, apply_operations = false):
// walking the ops backwards, lambda <- U^dag lambda, and for a trainable op
//   jac[o][t] = -2 * scale * Im <H_lambda_o | G lambda_old>
// then H_lambda_o <- U^dag H_lambda_o.  The reference materialises
// mu = G lambda_old with a state copy, a generator sweep and one host-synced
// reduction per (op, observable): about (num_obs + 4) state sweeps per op.
// Here one kernel per trainable op reads lambda and every H_lambda_o once,
// applies the generator to a register copy, accumulates the imaginary inner
// products in FP64 (deterministic block reduction), applies U^dag to both and
// writes them back: 2 * (1 + num_obs) state passes per op, no host round trip
// until the Jacobian is complete.  Observables are processed in chunks of up
// to 8 per launch; lambda is written by the last chunk only.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "adjoint_kernels.cuh"

namespace plk {

int plan_gate(int gate, int nw, bool inv, const double *prm, int np, GatePlan &p);
int plan_generator(int gate, int nw, GatePlan &p);
int apply_gate_impl(plk_state s, int gate, const int64_t *wires, int nw, bool adj, const double *params, int np,
                    const double *matrix);
int window_adjoint(plk_state lam, plk_state *hls, int nobs, const plk_op *ops, int nops, const int64_t *tp, int ntp,
                   double *jac, bool &handled);

static int adj_kind(int gate) {
    switch (gate) {
    case PLK_GATE_RX: return A_RX;
    case PLK_GATE_RY: return A_RY;
    case PLK_GATE_RZ: return A_RZ;
    case PLK_GATE_PHASESHIFT: return A_PS;
    case PLK_GATE_CRX: return A_CRX;
    case PLK_GATE_CRY: return A_CRY;
    case PLK_GATE_CRZ: return A_CRZ;
    case PLK_GATE_CONTROLLEDPHASESHIFT: return A_CPS;
    case PLK_GATE_ISINGXX: return A_IXX;
    case PLK_GATE_ISINGXY: return A_IXY;
    case PLK_GATE_ISINGYY: return A_IYY;
    case PLK_GATE_ISINGZZ: return A_IZZ;
    case PLK_GATE_SINGLEEXCITATION: return A_SE;
    case PLK_GATE_SINGLEEXCITATIONMINUS: return A_SEM;
    case PLK_GATE_SINGLEEXCITATIONPLUS: return A_SEP;
    case PLK_GATE_DOUBLEEXCITATION: return A_DE;
    case PLK_GATE_DOUBLEEXCITATIONMINUS: return A_DEM;
    case PLK_GATE_DOUBLEEXCITATIONPLUS: return A_DEP;
    case PLK_GATE_MULTIRZ: return A_MRZ;
    default: return A_NONE;
    }
}

// launchers of the other kinds live in adjoint_kinds2.cu and adjoint_kinds3.cu
#define PLK_ADJ_EXTERN(K)                                                                                             \
    extern template int launch_fused_kind<float, K>(plk_state, c2_t<float> *const *, int, int, const AdjArgs<float> &,    \
                                                    double *, double);                                                 \
    extern template int launch_fused_kind<double, K>(plk_state, c2_t<double> *const *, int, int,                         \
                                                     const AdjArgs<double> &, double *, double);
PLK_ADJ_KINDS2(PLK_ADJ_EXTERN)
PLK_ADJ_KINDS3(PLK_ADJ_EXTERN)
#undef PLK_ADJ_EXTERN

template <class T>
static int launch_fused(int kind, plk_state lam, c2_t<T> *const *d_hl, int nobs, int write_lambda, const AdjArgs<T> &a,
                        double *result, double post_scale) {
#define PLK_ADJ_CASE(K)                                                                                                \
    case K: return launch_fused_kind<T, K>(lam, d_hl, nobs, write_lambda, a, result, post_scale);
    switch (kind) {
        PLK_ADJ_CASE(A_RX) PLK_ADJ_CASE(A_RY) PLK_ADJ_CASE(A_RZ) PLK_ADJ_CASE(A_PS) PLK_ADJ_CASE(A_CRX)
        PLK_ADJ_CASE(A_CRY) PLK_ADJ_CASE(A_CRZ) PLK_ADJ_CASE(A_CPS) PLK_ADJ_CASE(A_IXX) PLK_ADJ_CASE(A_IXY)
        PLK_ADJ_CASE(A_IYY) PLK_ADJ_CASE(A_IZZ) PLK_ADJ_CASE(A_SE) PLK_ADJ_CASE(A_SEM) PLK_ADJ_CASE(A_SEP)
        PLK_ADJ_CASE(A_DE) PLK_ADJ_CASE(A_DEM) PLK_ADJ_CASE(A_DEP) PLK_ADJ_CASE(A_MRZ)
    default: PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "internal: no fused adjoint kernel");
    }
#undef PLK_ADJ_CASE
}

// One trainable backward step for all observables.
template <class T>
static int fused_step(plk_state lam, c2_t<T> *const *d_hl, int nobs, const plk_op &op, double scale, double *d_jac_col) {
    const int kind = adj_kind(op.gate);
    if (kind == A_NONE) PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "no generator for this gate");
    GatePlan p;
    PLK_TRY(plan_gate(op.gate, op.num_wires, op.adjoint == 0, op.params, op.num_params, p)); // U^dag
    AdjArgs<T> a;
    std::memset(&a, 0, sizeof(a));
    for (int j = 0; j < 8; j++) {
        a.g[j] = (T)p.coef[j];
        df_split_host(p.coef[j], a.gh[j], a.gl[j]);
    }
    a.e[0] = (T)p.extra_e[0];
    a.e[1] = (T)p.extra_e[1];
    df_split_host(p.extra_e[0], a.eh[0], a.el[0]);
    df_split_host(p.extra_e[1], a.eh[1], a.el[1]);
    if (kind == A_MRZ) {
        a.ngroups = lam->length;
        for (int j = 0; j < op.num_wires; j++) a.mrz_mask |= 1ULL << (lam->nq - 1 - op.wires[j]);
    } else {
        const int K = op.num_wires;
        int rev[4], srt[4];
        for (int j = 0; j < K; j++) rev[j] = lam->nq - 1 - (int)op.wires[j];
        std::copy(rev, rev + K, srt);
        std::sort(srt, srt + K);
        a.mk = make_masks(srt, K);
        a.ngroups = lam->length >> K;
        for (int i = 0; i < (1 << K); i++) {
            uint64_t o = 0;
            for (int j = 0; j < K; j++)
                if ((i >> (K - 1 - j)) & 1) o |= 1ULL << rev[j];
            a.off[i] = o;
        }
    }
    if (nobs == 0) {
        // nothing to differentiate against: just advance lambda
        return apply_gate_impl(lam, op.gate, op.wires, op.num_wires, op.adjoint == 0, op.params, op.num_params, nullptr);
    }
    for (int o0 = 0; o0 < nobs; o0 += kAdjObsPerLaunch) {
        const int nv = std::min(kAdjObsPerLaunch, nobs - o0);
        const int last = (o0 + nv == nobs);
        PLK_TRY(launch_fused<T>(kind, lam, d_hl + o0, nv, last, a, d_jac_col + o0, -2.0 * scale));
    }
    return PLK_OK;
}

template <class T>
static int adjoint_impl(plk_state lam, plk_state *hl, int nobs, const plk_op *ops, int nops, const int64_t *tp,
                        int ntp, double *jac) {
    using V = c2_t<T>;
    // device pointer table of the H_lambda states
    std::vector<V *> hp(std::max(nobs, 1));
    for (int o = 0; o < nobs; o++) hp[o] = (V *)hl[o]->data;
    V **d_hl = nullptr;
    double *d_jac = nullptr; // [ntp][nobs]
    PLK_CUDA(cudaMallocAsync((void **)&d_hl, sizeof(V *) * hp.size(), lam->stream));
    PLK_CUDA(cudaMemcpyAsync(d_hl, hp.data(), sizeof(V *) * hp.size(), cudaMemcpyHostToDevice, lam->stream));
    PLK_CUDA(cudaMallocAsync((void **)&d_jac, sizeof(double) * std::max(1, ntp * nobs), lam->stream));
    PLK_CUDA(cudaMemsetAsync(d_jac, 0, sizeof(double) * std::max(1, ntp * nobs), lam->stream));

    int num_param_ops = 0;
    for (int i = 0; i < nops; i++)
        if (ops[i].num_params > 0) num_param_ops++;
    int tp_number = ntp - 1;
    long current_param_idx = num_param_ops - 1;
    int tp_it = ntp - 1;
    int st = PLK_OK;
    for (int i = nops - 1; i >= 0 && st == PLK_OK; i--) {
        const plk_op &op = ops[i];
        if (op.num_params > 1) {
            set_error("The operation is not supported using the adjoint differentiation method");
            st = PLK_ERR_INVALID_ARG;
            break;
        }
        if (tp_it < 0) break; // all trainable parameters done
        const bool trainable = op.num_params > 0 && current_param_idx == tp[tp_it];
        if (trainable) {
            GatePlan gp;
            st = plan_generator(op.gate, op.num_wires, gp);
            if (st != PLK_OK) break;
            const double scale = gp.scale * (op.adjoint ? -1.0 : 1.0);
            st = fused_step<T>(lam, d_hl, nobs, op, scale, d_jac + (size_t)tp_number * nobs);
            tp_number--;
            tp_it--;
        } else {
            const bool adj = op.adjoint == 0;
            st = apply_gate_impl(lam, op.gate, op.wires, op.num_wires, adj, op.params, op.num_params, op.matrix);
            for (int o = 0; o < nobs && st == PLK_OK; o++)
                st = apply_gate_impl(hl[o], op.gate, op.wires, op.num_wires, adj, op.params, op.num_params, op.matrix);
        }
        if (op.num_params > 0) current_param_idx--;
    }
    std::vector<double> hj((size_t)std::max(1, ntp * nobs));
    if (st == PLK_OK && ntp * nobs > 0) {
        PLK_CUDA(cudaMemcpyAsync(hj.data(), d_jac, sizeof(double) * ntp * nobs, cudaMemcpyDeviceToHost, lam->stream));
    }
    cudaFreeAsync(d_hl, lam->stream);
    cudaFreeAsync(d_jac, lam->stream);
    PLK_CUDA(cudaStreamSynchronize(lam->stream));
    if (st != PLK_OK) return st;
    for (int t = 0; t < ntp; t++)
        for (int o = 0; o < nobs; o++) jac[(size_t)o * ntp + t] = hj[(size_t)t * nobs + o];
    return PLK_OK;
}

} // namespace plk

using namespace plk;

extern "C" {

static int adjoint_checks(plk_state lambda, plk_state *hlambda, int32_t nobs, const plk_op *ops, int32_t nops,
                          const int64_t *trainable, int32_t ntp, double *jac) {
    PLK_TRY(check_state(lambda));
    if (ntp <= 0) PLK_FAIL(PLK_ERR_INVALID_ARG, "No trainable parameters provided.");
    if (!trainable || !jac || (nops > 0 && !ops) || nobs < 0 || (nobs > 0 && !hlambda))
        PLK_FAIL(PLK_ERR_INVALID_ARG, "null argument");
    for (int t = 1; t < ntp; t++)
        if (trainable[t] <= trainable[t - 1]) PLK_FAIL(PLK_ERR_INVALID_ARG, "trainable parameters must be sorted and unique");
    for (int o = 0; o < nobs; o++) {
        PLK_TRY(check_state(hlambda[o]));
        if (hlambda[o]->nq != lambda->nq || hlambda[o]->dtype != lambda->dtype)
            PLK_FAIL(PLK_ERR_INVALID_ARG, "observable states differ in size or precision");
        if (hlambda[o] == lambda) PLK_FAIL(PLK_ERR_INVALID_ARG, "lambda cannot be one of the observable states");
        for (int p = 0; p < o; p++)
            if (hlambda[p] == hlambda[o]) PLK_FAIL(PLK_ERR_INVALID_ARG, "repeated observable state");
    }
    for (int i = 0; i < nops; i++) {
        const plk_op &op = ops[i];
        if (op.gate < 0 || op.gate >= PLK_GATE_COUNT) PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "unknown gate in op list");
        PLK_TRY(check_wires(lambda, op.wires, op.num_wires));
    }
    return PLK_OK;
}

// Runs the sweep with `work` as lambda (overwritten) and the observable states
// moved onto its stream for the duration of the call.
static int adjoint_run(plk_state work, plk_state *hlambda, int32_t nobs, const plk_op *ops, int32_t nops,
                       const int64_t *trainable, int32_t ntp, double *jac) {
    std::vector<cudaStream_t> old_streams(nobs);
    int st = PLK_OK;
    for (int o = 0; o < nobs && st == PLK_OK; o++) {
        old_streams[o] = hlambda[o]->stream;
        st = plk_state_set_stream(hlambda[o], work->stream);
    }
    bool handled = false;
    if (st == PLK_OK) st = window_adjoint(work, hlambda, nobs, ops, nops, trainable, ntp, jac, handled);
    if (st == PLK_OK && !handled)
        st = work->dtype == PLK_C64 ? adjoint_impl<float>(work, hlambda, nobs, ops, nops, trainable, ntp, jac)
                                    : adjoint_impl<double>(work, hlambda, nobs, ops, nops, trainable, ntp, jac);
    const std::string err = st == PLK_OK ? std::string() : last_error();
    for (int o = 0; o < nobs; o++)
        if (old_streams[o]) plk_state_set_stream(hlambda[o], old_streams[o]);
    if (st != PLK_OK) set_error(err);
    return st;
}

PLK_API int plk_adjoint_jacobian(plk_state lambda, plk_state *hlambda, int32_t nobs, const plk_op *ops, int32_t nops,
                                 const int64_t *trainable, int32_t ntp, double *jac) {
    PLK_TRY(adjoint_checks(lambda, hlambda, nobs, ops, nops, trainable, ntp, jac));
    PLK_CUDA(cudaSetDevice(lambda->device));
    // work copy of lambda, on lambda's stream
    plk_state work = nullptr;
    PLK_TRY(plk_state_create(lambda->nq, lambda->dtype, lambda->device, &work));
    int st = plk_state_set_stream(work, lambda->stream);
    if (st == PLK_OK) st = plk_state_copy(work, lambda);
    if (st == PLK_OK) st = adjoint_run(work, hlambda, nobs, ops, nops, trainable, ntp, jac);
    const std::string err = st == PLK_OK ? std::string() : last_error();
    plk_state_destroy(work);
    if (st != PLK_OK) set_error(err);
    return st;
}

PLK_API int plk_adjoint_jacobian_inplace(plk_state lambda, plk_state *hlambda, int32_t nobs, const plk_op *ops,
                                         int32_t nops, const int64_t *trainable, int32_t ntp, double *jac) {
    PLK_TRY(adjoint_checks(lambda, hlambda, nobs, ops, nops, trainable, ntp, jac));
    PLK_CUDA(cudaSetDevice(lambda->device));
    return adjoint_run(lambda, hlambda, nobs, ops, nops, trainable, ntp, jac);
}

} // extern "C"
