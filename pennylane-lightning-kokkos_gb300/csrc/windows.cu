// windows.cu — register-window sweeps over one large state.
//
// The op-at-a-time paths read and write the whole state once per gate.  Here
// an op sequence is packed into 4-qubit register windows (the compiler of the
// batch engine, window_host.cuh) and each window is one kernel over the
// whole GPU: every thread loads the 16 amplitudes that differ in the window
// bits, applies all of the window's ops in registers and stores them once.
// A layer of RY, RZ on every wire plus a CNOT ladder needs about 0.6 state
// passes per wire instead of 3.
//
// Used (complex64; complex128 in double-float on the FP32 pipe, windows_df.cu,
// unless PLK_C128_ARITH=fp64) by
//   plk_apply_ops           (StateVectorKokkos::applyOperation over a tape,
//                            StateVectorKokkos.hpp:585-676), and
//   plk_adjoint_jacobian    with one observable (AdjointDiffKokkos.hpp:404-478):
//                            walking the ops backwards, each window applies
//                            U^dag to lambda and H lambda and accumulates
//                            -2 scale Im <H lambda | G lambda> per trainable op
//                            (double-float accumulation; per-block partials
//                            reduced in block order, so reruns are bitwise
//                            identical).
// Ops outside the window model (gates on more than four wires other than
// MultiRZ; for the adjoint, ops with more than one parameter, which the
// reference rejects) keep the op-at-a-time path.  plk_set_window_path(0)
// turns the window path off.
#include <atomic>
#include <vector>

#include <type_traits>

#include "window_host.cuh"

namespace plk {

namespace {
std::atomic<int> g_window_path{1};
} // namespace

// complex64 windows (windows_sms.cu: shared-memory staged, 128 threads per CTA)
int window_sms_grid(int sm_count, uint64_t groups, bool bwd);
void launch_window_sms(bool bwd, int grid, cudaStream_t st, float2 *lam, float2 *hl, int nq, const EWin *wins, int wi,
                       int ntrain, const EOp *ops, const float2 *mats, const ETrain *train, double *bpart);

// complex128 windows (windows_df.cu, windows_df_fwd.cu: shared-memory staged
// double-float kernels, 128 threads per CTA)
int window_df_grid(int sm_count, uint64_t groups, bool bwd);
void launch_window_df_bwd(int grid, cudaStream_t st, double2 *lam, double2 *hl, int nq, const EWin *wins, int wi,
                          int ntrain, const EOp *ops, const float4 *mats, const ETrain *train, double *bpart,
                          int in_df, int out_df);
void launch_window_df_fwd(int grid, cudaStream_t st, double2 *lam, double2 *hl, int nq, const EWin *wins, int wi,
                          const EOp *ops, const float4 *mats, const ETrain *train, double *bpart, int in_df,
                          int out_df);

// jac[s] = sum over blocks, in block order
__global__ void k_window_jac(const double *__restrict__ bpart, int nblocks, int ntp, double *__restrict__ jac) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ntp) return;
    double t = 0.0;
    for (int b = 0; b < nblocks; b++) t += bpart[(size_t)s * nblocks + b];
    jac[s] = t;
}

struct StateProgram {
    std::vector<EWin> wins;
    std::vector<EOp> ops;
    std::vector<ETrain> train;
    std::vector<EPrep> prep; // unused: matrices come from the ops themselves
    std::vector<double2> gen;
    std::vector<double2> mats;
    int64_t n_mats = 0;
};

// XOp of a reference op with its matrix U_op (gate order); false if the op
// does not fit the window model.
static int make_xop(const plk_op &op, int nq, XOp &x, bool &fits) {
    fits = true;
    x = XOp();
    x.gate = op.gate;
    x.inv = op.adjoint != 0;
    x.pidx = -1;
    x.slot = -1;
    x.basis = -1;
    x.user_matrix = -1;
    const int g = op.gate;
    if (g == PLK_GATE_MULTIRZ) {
        if (op.num_wires < 1 || op.num_wires > 32) {
            fits = false;
            return PLK_OK;
        }
        x.kind = EK_PARITY;
        x.K = 1;
        x.mrz_wires.assign(op.wires, op.wires + op.num_wires);
        GatePlan p;
        PLK_TRY(plan_gate(g, 1, x.inv, op.params, op.num_params, p));
        plan_dense(p, 1, x.umat);
        return PLK_OK;
    }
    if (op.num_wires > kWinBits || op.num_wires < 1) {
        fits = false;
        return PLK_OK;
    }
    x.K = op.num_wires;
    for (int j = 0; j < x.K; j++) x.wires[j] = (int)op.wires[j];
    if (g == PLK_GATE_MATRIX) {
        if (!op.matrix) PLK_FAIL(PLK_ERR_INVALID_ARG, "matrix op without a matrix");
        const int D = 1 << x.K;
        x.umat.resize((size_t)D * D);
        for (int r = 0; r < D; r++)
            for (int c = 0; c < D; c++) {
                // the op applies the matrix, or its conjugate transpose when adjoint
                const int src = x.inv ? c * D + r : r * D + c;
                x.umat[(size_t)r * D + c] = mk<double2>(op.matrix[2 * src], x.inv ? -op.matrix[2 * src + 1]
                                                                                  : op.matrix[2 * src + 1]);
            }
        x.kind = EK_DENSE;
        return PLK_OK;
    }
    GatePlan p;
    PLK_TRY(plan_gate(g, op.num_wires, x.inv, op.params, op.num_params, p));
    plan_dense(p, x.K, x.umat);
    x.kind = g == PLK_GATE_CNOT ? EK_CX : (is_diag_gate(g) ? EK_DIAG : EK_DENSE);
    return PLK_OK;
}

// Every index a window kernel will follow, checked on the host before the
// first launch: matrix and generator offsets inside the matrix buffer,
// register-bit selections, reduction slots below the window's trainable
// count, Jacobian slots below ntp.  A failed check is an internal error
// reported to the caller, never a launch.
static int validate_program(const StateProgram &P, const std::vector<EOp> &ops, int nq, size_t nmats, bool bwd,
                            int ntp) {
    auto bad = [](const std::string &what) {
        set_error("internal: window program check failed: " + what);
        return PLK_ERR_UNSUPPORTED;
    };
    for (size_t wi = 0; wi < P.wins.size(); wi++) {
        const EWin &w = P.wins[wi];
        if (w.op0 < 0 || w.nops < 0 || (size_t)w.op0 + w.nops > ops.size()) return bad("window op range");
        if (w.ntrain < 0 || w.ntrain > kMaxWinTrain || w.tr0 < 0 || (size_t)w.tr0 + w.ntrain > P.train.size())
            return bad("window trainable range");
        for (int i = 0; i < 4; i++)
            if (w.rb[i] >= nq || (i > 0 && w.rb[i] <= w.rb[i - 1])) return bad("window register bits");
        for (int t = 0; t < w.ntrain; t++)
            if (P.train[w.tr0 + t].slot < 0 || P.train[w.tr0 + t].slot >= std::max(1, ntp))
                return bad("Jacobian slot");
        for (int k = 0; k < w.nops; k++) {
            const EOp &o = ops[w.op0 + k];
            const bool tr = bwd && o.red != 0xff;
            if (o.red != 0xff && (!bwd || o.red >= w.ntrain)) return bad("reduction slot");
            auto in_mats = [&](int64_t off, int64_t len) { return off >= 0 && off + len <= (int64_t)nmats; };
            const int D = 1 << (o.K > 4 ? 4 : o.K);
            switch (o.kind) {
            case EK_DENSE:
                if (o.K < 1 || o.K > 4 || !in_mats(o.mat, (int64_t)D * D)) return bad("dense op matrix");
                if ((o.K == 1 && ((o.sel >> 2) > 2)) || (o.K == 2 && o.sel > 5) || (o.K == 3 && o.sel > 3))
                    return bad("dense op bits");
                if (tr && o.K > 1 && !in_mats(o.gen, (int64_t)D * D)) return bad("dense generator");
                break;
            case EK_CX:
                if ((o.sel >> 2) > 3 || (o.sel >> 2) == (o.sel & 3)) return bad("CNOT bits");
                break;
            case EK_DIAG:
                if (o.K < 1 || o.K > 4 || !in_mats(o.mat, D) || o.sel > 4) return bad("diagonal op");
                for (int j = 0; j < o.K; j++)
                    if (((o.bits >> (5 * j)) & 31u) >= (uint32_t)nq) return bad("diagonal op wire");
                if (tr && !in_mats(o.gen, D)) return bad("diagonal generator");
                break;
            case EK_PARITY:
                if (!in_mats(o.mat, 2) || (nq < 32 && (o.bits >> nq) != 0)) return bad("parity op");
                break;
            case EK_DIAGSET:
                if (o.K > 4 || !in_mats(o.mat, kWinAmps) || (o.K > 0 && !bwd)) return bad("merged diagonal");
                for (int m = 0; m < o.K; m++)
                    if (((o.gen >> (4 * m)) & 15) >= w.ntrain) return bad("merged diagonal member");
                break;
            default: return bad("op kind");
            }
        }
    }
    return PLK_OK;
}

template <class T>
// Runs a window program on `lam` (and `hl` going backwards) on lam's stream.
// Backward, the Jacobian row goes to jac_host (the call synchronizes), or,
// when d_jac_out is given, to that device row with nothing synchronized.
static int run_program(plk_state lam, plk_state hl, const StateProgram &P, bool bwd, int ntp, double *jac_host,
                       double *d_jac_out = nullptr) {
    using V = c2_t<T>;
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(lam->device, &d));
    cudaStream_t st = lam->stream;
    const uint64_t nu = lam->length >> kWinBits;
    const int grid = std::is_same<T, double>::value ? window_df_grid(d->sm_count, nu, bwd)
                                                     : window_sms_grid(d->sm_count, nu, bwd);
    // matrices: state precision for complex64, split double-floats for complex128
    using M = typename std::conditional<std::is_same<T, double>::value, float4, V>::type;
    std::vector<M> mats(P.mats.size() + P.gen.size());
    auto conv = [](double2 z) {
        if constexpr (std::is_same<T, double>::value) {
            float4 f;
            df_split_host(z.x, f.x, f.y);
            df_split_host(z.y, f.z, f.w);
            return f;
        } else {
            return mk<V>((T)z.x, (T)z.y);
        }
    };
    for (size_t i = 0; i < P.mats.size(); i++) mats[i] = conv(P.mats[i]);
    for (size_t i = 0; i < P.gen.size(); i++) mats[P.mats.size() + i] = conv(P.gen[i]);
    std::vector<EOp> ops = P.ops;
    for (auto &o : ops) // generators follow the matrices (EK_DIAGSET keeps reduction slots in gen)
        if (o.gen >= 0 && o.kind != EK_DIAGSET) o.gen += (int32_t)P.mats.size();
    PLK_TRY(validate_program(P, ops, lam->nq, mats.size(), bwd, ntp));
    const size_t b_w = P.wins.size() * sizeof(EWin), b_o = ops.size() * sizeof(EOp);
    const size_t b_t = std::max<size_t>(1, P.train.size()) * sizeof(ETrain), b_m = std::max<size_t>(1, mats.size()) * sizeof(M);
    const size_t b_p = bwd ? (size_t)std::max(1, ntp) * grid * sizeof(double) : 0;
    const size_t b_j = bwd ? (size_t)std::max(1, ntp) * sizeof(double) : 0;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t total = al(b_w) + al(b_o) + al(b_t) + al(b_m) + al(b_p) + al(b_j);
    char *buf = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&buf, total, st));
    char *p = buf;
    EWin *d_w = (EWin *)p;
    p += al(b_w);
    EOp *d_o = (EOp *)p;
    p += al(b_o);
    ETrain *d_t = (ETrain *)p;
    p += al(b_t);
    M *d_m = (M *)p;
    p += al(b_m);
    double *d_p = (double *)p;
    p += al(b_p);
    double *d_j = (double *)p;

    int rc = PLK_OK;
    auto cp = [&](void *dst, const void *src, size_t n) {
        if (rc == PLK_OK && n && cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, st) != cudaSuccess)
            rc = PLK_ERR_CUDA;
    };
    cp(d_w, P.wins.data(), b_w);
    cp(d_o, ops.data(), b_o);
    if (!P.train.empty()) cp(d_t, P.train.data(), P.train.size() * sizeof(ETrain));
    if (!mats.empty()) cp(d_m, mats.data(), mats.size() * sizeof(M));
    if (bwd && rc == PLK_OK && cudaMemsetAsync(d_p, 0, b_p, st) != cudaSuccess) rc = PLK_ERR_CUDA;

    V *lp = (V *)lam->data;
    V *hp = hl ? (V *)hl->data : nullptr;
    for (size_t wi = 0; wi < P.wins.size() && rc == PLK_OK; wi++) {
        if constexpr (std::is_same<T, double>::value) {
            const int in_df = wi > 0, out_df = wi + 1 < P.wins.size();
            if (bwd)
                launch_window_df_bwd(grid, st, lp, hp, lam->nq, d_w, (int)wi, P.wins[wi].ntrain, d_o, d_m, d_t, d_p,
                                     in_df, out_df);
            else
                launch_window_df_fwd(grid, st, lp, hp, lam->nq, d_w, (int)wi, d_o, d_m, d_t, d_p, in_df, out_df);
        } else {
            launch_window_sms(bwd, grid, st, reinterpret_cast<float2 *>(lp), reinterpret_cast<float2 *>(hp),
                              lam->nq, d_w, (int)wi, P.wins[wi].ntrain, d_o, reinterpret_cast<const float2 *>(d_m), d_t,
                              d_p);
        }
        if (cudaGetLastError() != cudaSuccess) rc = PLK_ERR_CUDA;
    }
    if (bwd && rc == PLK_OK && ntp > 0) {
        k_window_jac<<<(ntp + 255) / 256, 256, 0, st>>>(d_p, grid, ntp, d_jac_out ? d_jac_out : d_j);
        if (cudaGetLastError() != cudaSuccess) rc = PLK_ERR_CUDA;
        if (rc == PLK_OK && !d_jac_out &&
            cudaMemcpyAsync(jac_host, d_j, ntp * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = PLK_ERR_CUDA;
    }
    cudaFreeAsync(buf, st);
    if (rc != PLK_OK) PLK_FAIL(rc, std::string("window sweep failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (bwd && !d_jac_out) PLK_CUDA(cudaStreamSynchronize(st));
    return PLK_OK;
}

bool window_path_enabled() { return g_window_path.load() != 0; }

// Forward: the whole op list through windows (complex64).
int window_apply_ops(plk_state s, const plk_op *ops, int nops, bool &handled) {
    handled = false;
    if (!window_path_enabled() || (s->dtype != PLK_C64 && !c128_use_df()) || nops < 4 || s->nq < 6 || s->nq > 32)
        return PLK_OK;
    std::vector<XOp> xs;
    xs.reserve(nops * 3);
    for (int i = 0; i < nops; i++) {
        const plk_op &op = ops[i];
        if (op.gate < 0 || op.gate >= PLK_GATE_COUNT) return PLK_OK; // the per-op path reports it
        if (op.gate == PLK_GATE_IDENTITY) continue;
        if (check_wires(s, op.wires, op.num_wires) != PLK_OK) return PLK_OK;
        if (op.num_params < plk_gate_num_params(op.gate) || (op.num_params > 0 && !op.params)) return PLK_OK;
        XOp x;
        bool fits = false;
        if (make_xop(op, s->nq, x, fits) != PLK_OK) return PLK_OK;
        if (!fits) return PLK_OK;
        xs.push_back(std::move(x));
    }
    StateProgram P;
    WinBuilder wb{s->nq, false, P.wins, P.ops, P.train, P.prep, P.gen, P.n_mats};
    wb.hmats = &P.mats;
    wb.fuse_diag = true; // merged diagonal runs (the single-state window kernels of both precisions)
    std::vector<const XOp *> seq;
    for (const auto &x : xs) seq.push_back(&x);
    PLK_TRY(wb.add_scheduled(seq));
    PLK_TRY(wb.close());
    handled = true;
    return s->dtype == PLK_C64 ? run_program<float>(s, nullptr, P, false, 0, nullptr)
                               : run_program<double>(s, nullptr, P, false, 0, nullptr);
}

// Several observables on small states: the backward sweeps of different
// observables are independent, so up to kConcurrentObs of them run at once,
// each on its own stream with its own copy of lambda.  A window over a
// 20-qubit state has 65 536 amplitude groups against about 58 000 resident
// threads, so one sweep alone runs every launch in two rounds, the second
// nearly empty; concurrent sweeps fill those slots.  Jacobian rows go to one
// device array, read back once.  `handled` stays false (and nothing is left
// allocated) when the copies or streams cannot be had.
constexpr int kConcurrentObs = 4, kConcurrentObsMaxQubits = 22;

template <class T> static int run_program_t(plk_state l, plk_state hl, const StateProgram &P, int ntp, double *d_row) {
    return run_program<T>(l, hl, P, true, ntp, nullptr, d_row);
}

static int window_adjoint_concurrent(plk_state lam, plk_state *hls, int nobs, const StateProgram &P, int ntp,
                                     double *jac, bool &handled) {
    handled = false;
    const int S = std::min(nobs, kConcurrentObs);
    plk_state scratch[kConcurrentObs] = {};
    cudaStream_t streams[kConcurrentObs] = {};
    double *d_jac = nullptr;
    int made = 0, rc = PLK_OK;
    auto cleanup = [&]() {
        for (int i = 0; i < made; i++) {
            if (streams[i]) cudaStreamSynchronize(streams[i]);
            if (scratch[i]) plk_state_destroy(scratch[i]);
            if (streams[i]) cudaStreamDestroy(streams[i]);
        }
        if (d_jac) cudaFree(d_jac);
    };
    for (; made < S; made++) {
        if (plk_state_create(lam->nq, lam->dtype, lam->device, &scratch[made]) != PLK_OK ||
            cudaStreamCreateWithFlags(&streams[made], cudaStreamNonBlocking) != cudaSuccess ||
            plk_state_set_stream(scratch[made], streams[made]) != PLK_OK) {
            made++;
            cleanup();
            cudaGetLastError();
            set_error(std::string());
            return PLK_OK; // not handled: the sequential path takes it
        }
    }
    if (cudaMalloc((void **)&d_jac, sizeof(double) * (size_t)nobs * std::max(1, ntp)) != cudaSuccess) {
        d_jac = nullptr;
        cleanup();
        cudaGetLastError();
        set_error(std::string());
        return PLK_OK;
    }
    handled = true;
    // lambda and every H lambda are complete before the worker streams start
    if (cudaStreamSynchronize(lam->stream) != cudaSuccess) rc = PLK_ERR_CUDA;
    for (int o = 0; o < nobs && rc == PLK_OK; o++)
        if (cudaStreamSynchronize(hls[o]->stream) != cudaSuccess) rc = PLK_ERR_CUDA;
    for (int o = 0; o < nobs && rc == PLK_OK; o++) {
        const int w = o % S;
        rc = plk_state_copy(scratch[w], lam);
        if (rc == PLK_OK)
            rc = lam->dtype == PLK_C64 ? run_program_t<float>(scratch[w], hls[o], P, ntp, d_jac + (size_t)o * ntp)
                                       : run_program_t<double>(scratch[w], hls[o], P, ntp, d_jac + (size_t)o * ntp);
    }
    for (int i = 0; i < S && rc == PLK_OK; i++)
        if (cudaStreamSynchronize(streams[i]) != cudaSuccess) rc = PLK_ERR_CUDA;
    if (rc == PLK_OK && ntp > 0 &&
        cudaMemcpy(jac, d_jac, sizeof(double) * (size_t)nobs * ntp, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = PLK_ERR_CUDA;
    std::string err;
    if (rc != PLK_OK)
        err = !last_error().empty() ? last_error()
                                    : std::string("concurrent window sweeps failed: ") +
                                          cudaGetErrorString(cudaGetLastError());
    cleanup();
    if (rc != PLK_OK) set_error(err);
    return rc;
}

// Backward sweep of the adjoint Jacobian with one observable (complex64);
// `lam` is the working copy of the forward state (overwritten).
int window_adjoint(plk_state lam, plk_state *hls, int nobs, const plk_op *ops, int nops, const int64_t *tp, int ntp,
                   double *jac, bool &handled) {
    handled = false;
    if (!window_path_enabled() || (lam->dtype != PLK_C64 && !c128_use_df()) || lam->nq < 6 || lam->nq > 32 ||
        ntp <= 0)
        return PLK_OK;
    int num_param_ops = 0;
    for (int i = 0; i < nops; i++)
        if (ops[i].num_params > 0) num_param_ops++;
    // the reference's backward walk: ops in reverse until every trainable
    // parameter is done (AdjointDiffKokkos.hpp:436-470)
    std::vector<XOp> xs;
    long current_param_idx = num_param_ops - 1;
    int tp_it = ntp - 1;
    for (int i = nops - 1; i >= 0 && tp_it >= 0; i--) {
        const plk_op &op = ops[i];
        if (op.num_params > 1) return PLK_OK; // rejected by the reference; the per-op path reports it
        if (op.gate < 0 || op.gate >= PLK_GATE_COUNT) return PLK_OK;
        const bool trainable = op.num_params > 0 && current_param_idx == tp[tp_it];
        if (op.gate != PLK_GATE_IDENTITY) {
            XOp x;
            bool fits = false;
            if (make_xop(op, lam->nq, x, fits) != PLK_OK || !fits) return PLK_OK;
            if (trainable) {
                GatePlan gp;
                if (plan_generator(op.gate, op.num_wires, gp) != PLK_OK) return PLK_OK;
                x.slot = tp_it;
            }
            xs.push_back(std::move(x));
        } else if (trainable) {
            return PLK_OK;
        }
        if (trainable) tp_it--;
        if (op.num_params > 0) current_param_idx--;
    }
    StateProgram P;
    WinBuilder wb{lam->nq, true, P.wins, P.ops, P.train, P.prep, P.gen, P.n_mats};
    wb.hmats = &P.mats;
    wb.fuse_diag = true; // merged diagonal runs (the single-state window kernels of both precisions)
    std::vector<const XOp *> seq;
    for (const auto &x : xs) seq.push_back(&x);
    PLK_TRY(wb.add_scheduled(seq));
    PLK_TRY(wb.close());
    // Several observables: the program runs once per observable on a copy of
    // lambda (the last one on lambda itself): 4 state passes per window per
    // observable plus one copy, against 2 (1 + nobs) passes per op for the
    // op-at-a-time kernel that carries every H lambda along.
    if (nobs > 1 && (double)nobs * (4.0 * P.wins.size() + 2.0) > 2.0 * (1.0 + nobs) * xs.size()) return PLK_OK;
    if (nobs > 1 && lam->nq <= kConcurrentObsMaxQubits) {
        int rc = window_adjoint_concurrent(lam, hls, nobs, P, ntp, jac, handled);
        if (handled || rc != PLK_OK) return rc;
    }
    plk_state scratch = nullptr;
    if (nobs > 1) {
        if (plk_state_create(lam->nq, lam->dtype, lam->device, &scratch) != PLK_OK) {
            // no room for a copy of lambda: the op-at-a-time path needs none
            set_error(std::string());
            return PLK_OK;
        }
    }
    handled = true;
    int rc = PLK_OK;
    if (scratch) rc = plk_state_set_stream(scratch, lam->stream);
    std::vector<double> j(ntp, 0.0);
    for (int o = 0; o < nobs && rc == PLK_OK; o++) {
        plk_state l = lam;
        if (o + 1 < nobs) {
            rc = plk_state_copy(scratch, lam);
            l = scratch;
        }
        if (rc == PLK_OK)
            rc = lam->dtype == PLK_C64 ? run_program<float>(l, hls[o], P, true, ntp, j.data())
                                       : run_program<double>(l, hls[o], P, true, ntp, j.data());
        if (rc == PLK_OK)
            for (int t = 0; t < ntp; t++) jac[(size_t)o * ntp + t] = j[t];
    }
    const std::string err = rc == PLK_OK ? std::string() : last_error();
    if (scratch) plk_state_destroy(scratch);
    if (rc != PLK_OK) set_error(err);
    return rc;
}

} // namespace plk

extern "C" {

PLK_API int plk_set_window_path(int32_t enable) {
    plk::g_window_path.store(enable != 0);
    return PLK_OK;
}

PLK_API int plk_get_window_path(int32_t *enabled) {
    if (enabled) *enabled = plk::g_window_path.load();
    return PLK_OK;
}

} // extern "C"
