// batch.cu — batched circuits: forward pass, <H> and adjoint gradient of many
// independent circuits in one persistent launch (device side in
// batch_engine.cuh).
//
// The per-circuit work restates, for every circuit of the batch,
//   StateVectorKokkos::applyOperation over the tape (StateVectorKokkos.hpp:
//     585-676), the Hamiltonian expectation (ObservablesKokkos.hpp:484-494,
//     MeasuresKokkos.hpp:354-366) and
//   AdjointJacobianKokkos::adjointJacobian (AdjointDiffKokkos.hpp:404-478):
//     walking the ops backwards, jac[t] = -2 * scale * Im <H lambda | G lambda>
//     before lambda <- U^dag lambda and H lambda <- U^dag H lambda.
// The reference runs this one circuit at a time (the Python device loops over
// tapes); here a batch is compiled once into register windows and a CUDA
// graph replays [parameters H2D, matrix preparation, engine, results D2H].
//
// Gate matrices come from the same gate plans as the per-state kernels
// (plan_gate / plan_generator), expanded to dense matrices on the host.  A
// parametric gate's entries are trigonometric polynomials of degree one in
// theta/2, U(theta) = A0 + cos(theta/2) A1 + sin(theta/2) A2 + cos(theta) A3
// + sin(theta) A4; the five coefficient matrices are fitted once per gate
// from five angles (checked at two more), so the device rebuilds U from the
// parameter vector without gate-specific code.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "window_host.cuh"

namespace plk {

struct BatchConfig {
    int cluster = 8;        // CTAs per cluster for the largest circuits
    int threads = 256;      // threads per CTA
    int ctas_per_sm = 1;    // 1 or 2 (complex64): register budget 255 or 128 per thread
    int smem_bits = 13;     // circuits with at most this many qubits stay in shared memory
    int cluster_min_qubits = 17; // circuits with at least this many qubits go to clusters
};

struct LaunchPlan {
    int grid = 0;
    int cluster = 1;
    size_t smem = 0;
    std::vector<int32_t> order; // [order_cl..., order_solo...]
    int n_cl = 0, n_solo = 0;
    uint64_t slot_amps = 0;
    int max_global_nq = 0;
};

} // namespace plk

struct plk_batch_s {
    int dtype = PLK_C64;
    int device = 0;
    // circuits as added
    struct Circ {
        int nq;
        std::vector<plk::XOp> ops;
        int p0, np;        // flat parameter range
        int jac0, ntp;
        std::vector<plk::ETerm> terms;
    };
    std::vector<Circ> circs;
    std::vector<double> params; // flat initial parameters
    std::vector<std::vector<double2>> user_mats;
    std::map<int, int> basis_of;      // (gate * 2 + inv) -> basis offset
    std::vector<double2> basis;       // host copy of all coefficient blocks
    int njac = 0;
    plk::BatchConfig cfg;
    bool tuned = false;
    // compiled
    bool compiled = false;
    std::vector<plk::ECirc> h_circ;
    std::vector<plk::EWin> h_win;
    std::vector<plk::EOp> h_ops;
    std::vector<plk::ETrain> h_train;
    std::vector<plk::ETerm> h_terms;
    std::vector<plk::EPrep> h_prep;
    std::vector<double2> h_gen; // constant generator blocks (appended after the prepared matrices)
    int64_t n_mats = 0;         // prepared complex entries
    std::vector<double> cost;
    int max_nq = 0;
    // device
    void *d_circ = nullptr, *d_win = nullptr, *d_ops = nullptr, *d_train = nullptr, *d_terms = nullptr;
    void *d_prep = nullptr, *d_basis = nullptr, *d_mats = nullptr, *d_order = nullptr;
    double *d_params = nullptr, *d_expval = nullptr, *d_jac = nullptr, *d_jac_part = nullptr, *d_ev_part = nullptr;
    unsigned *d_counters = nullptr;
    void *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    double *h_params_pinned = nullptr, *h_out_pinned = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    bool use_graph = true;
    int graph_cfg_key = -1;
    plk::LaunchPlan lp;      // launch plan of the configuration lp_key
    int lp_key = -1;
    float last_ms = 0.0f;
    long long last_launches = 0;
};

namespace plk {

static int gate_nwires(int g);
static int gate_nparams(int g);

static int basis_for(plk_batch b, int gate, bool inv, int K, int &off) {
    const int key = gate * 2 + (inv ? 1 : 0);
    auto it = b->basis_of.find(key);
    if (it != b->basis_of.end()) {
        off = it->second;
        return PLK_OK;
    }
    std::vector<double2> A;
    const int Kb = gate == PLK_GATE_MULTIRZ ? 1 : K;
    PLK_TRY(fit_gate(gate, Kb, inv, gate_nparams(gate), A));
    off = (int)b->basis.size();
    b->basis.insert(b->basis.end(), A.begin(), A.end());
    b->basis_of[key] = off;
    return PLK_OK;
}

static void free_device(plk_batch b) {
    void **ptrs[] = {&b->d_circ, &b->d_win, &b->d_ops, &b->d_train, &b->d_terms, &b->d_prep, &b->d_basis,
                     &b->d_mats, &b->d_order, (void **)&b->d_params, (void **)&b->d_expval, (void **)&b->d_jac,
                     (void **)&b->d_jac_part, (void **)&b->d_ev_part, (void **)&b->d_counters, &b->d_scratch};
    for (void **p : ptrs) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    b->scratch_bytes = 0;
    if (b->h_params_pinned) cudaFreeHost(b->h_params_pinned);
    if (b->h_out_pinned) cudaFreeHost(b->h_out_pinned);
    b->h_params_pinned = b->h_out_pinned = nullptr;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_cfg_key = -1;
    b->lp_key = -1;
}

static int compile_batch(plk_batch b) {
    b->h_circ.clear();
    b->h_win.clear();
    b->h_ops.clear();
    b->h_train.clear();
    b->h_terms.clear();
    b->h_prep.clear();
    b->h_gen.clear();
    b->cost.clear();
    b->n_mats = 0;
    b->max_nq = 0;
    for (size_t ci = 0; ci < b->circs.size(); ci++) {
        auto &c = b->circs[ci];
        ECirc e;
        e.nq = c.nq;
        e.id = (int)ci;
        e.jac0 = c.jac0;
        e.ntp = c.ntp;
        e.term0 = (int)b->h_terms.size();
        e.nterms = (int)c.terms.size();
        b->h_terms.insert(b->h_terms.end(), c.terms.begin(), c.terms.end());
        for (int dir = 0; dir < 2; dir++) {
            const bool bwd = dir == 1;
            WinBuilder wb{c.nq, bwd, b->h_win, b->h_ops, b->h_train, b->h_prep, b->h_gen, b->n_mats};
            const int w0 = (int)b->h_win.size();
            const int n = (int)c.ops.size();
            std::vector<const XOp *> seq;
            if (!bwd) {
                for (int k = 0; k < n; k++) seq.push_back(&c.ops[k]);
            } else {
                // ops before the first trainable op do not change the Jacobian
                // (the reference loop ends there too, AdjointDiffKokkos.hpp:447)
                int first = n;
                for (int k = 0; k < n; k++)
                    if (c.ops[k].slot >= 0) {
                        first = k;
                        break;
                    }
                for (int k = n - 1; k >= first; k--) seq.push_back(&c.ops[k]);
            }
            PLK_TRY(wb.add_scheduled(seq));
            PLK_TRY(wb.close());
            if (!bwd) {
                e.fw0 = w0;
                e.nfw = (int)b->h_win.size() - w0;
            } else {
                e.bw0 = w0;
                e.nbw = (int)b->h_win.size() - w0;
            }
        }
        b->h_circ.push_back(e);
        double work = 0;
        for (int w = e.fw0; w < e.fw0 + e.nfw; w++) work += 4 + b->h_win[w].nops;
        for (int w = e.bw0; w < e.bw0 + e.nbw; w++) work += 2 * (4 + b->h_win[w].nops);
        work += 2 + e.nterms;
        b->cost.push_back(work * std::ldexp(1.0, c.nq));
        b->max_nq = std::max(b->max_nq, c.nq);
    }
    // generator blocks follow the prepared matrices in one buffer
    for (auto &o : b->h_ops)
        if (o.gen >= 0) o.gen += (int32_t)b->n_mats;
    b->compiled = true;
    return PLK_OK;
}

static int upload_vec(void **dptr, const void *src, size_t bytes, cudaStream_t st) {
    if (*dptr) cudaFree(*dptr);
    *dptr = nullptr;
    PLK_CUDA(cudaMalloc(dptr, std::max<size_t>(bytes, 16)));
    if (bytes) PLK_CUDA(cudaMemcpyAsync(*dptr, src, bytes, cudaMemcpyHostToDevice, st));
    return PLK_OK;
}

template <class T> static int upload_batch(plk_batch b) {
    using V = c2_t<T>;
    free_device(b);
    cudaStream_t st = b->stream;
    PLK_TRY(upload_vec(&b->d_circ, b->h_circ.data(), b->h_circ.size() * sizeof(ECirc), st));
    PLK_TRY(upload_vec(&b->d_win, b->h_win.data(), b->h_win.size() * sizeof(EWin), st));
    PLK_TRY(upload_vec(&b->d_ops, b->h_ops.data(), b->h_ops.size() * sizeof(EOp), st));
    PLK_TRY(upload_vec(&b->d_train, b->h_train.data(), b->h_train.size() * sizeof(ETrain), st));
    PLK_TRY(upload_vec(&b->d_terms, b->h_terms.data(), b->h_terms.size() * sizeof(ETerm), st));
    PLK_TRY(upload_vec(&b->d_prep, b->h_prep.data(), b->h_prep.size() * sizeof(EPrep), st));
    PLK_TRY(upload_vec(&b->d_basis, b->basis.data(), b->basis.size() * sizeof(double2), st));
    // matrices: prepared region then constant generators (cast to the state precision)
    const size_t nm = (size_t)b->n_mats + b->h_gen.size();
    std::vector<V> gen(b->h_gen.size());
    for (size_t i = 0; i < gen.size(); i++) gen[i] = mk<V>((T)b->h_gen[i].x, (T)b->h_gen[i].y);
    PLK_CUDA(cudaMalloc(&b->d_mats, std::max<size_t>(nm, 1) * sizeof(V)));
    if (!gen.empty())
        PLK_CUDA(cudaMemcpyAsync((V *)b->d_mats + b->n_mats, gen.data(), gen.size() * sizeof(V), cudaMemcpyHostToDevice,
                                 st));
    const size_t nc = b->circs.size();
    PLK_CUDA(cudaMalloc(&b->d_order, std::max<size_t>(nc, 1) * 2 * sizeof(int32_t)));
    PLK_CUDA(cudaMalloc(&b->d_params, std::max<size_t>(b->params.size(), 1) * sizeof(double)));
    PLK_CUDA(cudaMemcpyAsync(b->d_params, b->params.data(), b->params.size() * sizeof(double), cudaMemcpyHostToDevice,
                             st));
    PLK_CUDA(cudaMalloc(&b->d_expval, std::max<size_t>(nc, 1) * sizeof(double)));
    PLK_CUDA(cudaMalloc(&b->d_jac, std::max(b->njac, 1) * sizeof(double)));
    PLK_CUDA(cudaMalloc(&b->d_jac_part, std::max(b->njac, 1) * kMaxCluster * sizeof(double)));
    PLK_CUDA(cudaMalloc(&b->d_ev_part, std::max<size_t>(nc, 1) * kMaxCluster * sizeof(double)));
    PLK_CUDA(cudaMalloc(&b->d_counters, 4 * sizeof(unsigned)));
    PLK_CUDA(cudaMallocHost(&b->h_params_pinned, std::max<size_t>(b->params.size(), 1) * sizeof(double)));
    PLK_CUDA(cudaMallocHost(&b->h_out_pinned, (nc + b->njac + 1) * sizeof(double)));
    PLK_CUDA(cudaStreamSynchronize(st));
    return PLK_OK;
}

// ------------------------------------------------------------- kernels --
template <class T>
__global__ void k_batch_prepare(const EPrep *__restrict__ prep, int nprep, const double2 *__restrict__ basis,
                                const double *__restrict__ params, c2_t<T> *__restrict__ mats) {
    using V = c2_t<T>;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nprep) return;
    const EPrep p = prep[e];
    double f[5] = {1.0, 0.0, 0.0, 0.0, 0.0};
    if (p.pidx >= 0) {
        const double th = params[p.pidx];
        sincos(th * 0.5, &f[2], &f[1]);
        sincos(th, &f[4], &f[3]);
    }
    const int K = p.K, D = 1 << K;
    if (p.kind == EK_DENSE) {
        const int DD = D * D;
        for (int idx = 0; idx < DD; idx++) {
            const int r = idx / D, c = idx % D;
            int gr = 0, gc = 0;
            for (int j = 0; j < K; j++) {
                gr |= ((r >> p.perm[j]) & 1) << (K - 1 - j);
                gc |= ((c >> p.perm[j]) & 1) << (K - 1 - j);
            }
            const int src = p.conjT ? gc * D + gr : gr * D + gc;
            double re = 0.0, im = 0.0;
            for (int i = 0; i < 5; i++) {
                const double2 a = basis[p.basis + i * DD + src];
                re = fma(f[i], a.x, re);
                im = fma(f[i], a.y, im);
            }
            mats[p.out + idx] = mk<V>((T)re, (T)(p.conjT ? -im : im));
        }
    } else { // diagonal (DIAG: 2^K entries; PARITY: the 2 entries of MultiRZ on one wire)
        const int DD = D * D;
        for (int i2 = 0; i2 < D; i2++) {
            double re = 0.0, im = 0.0;
            for (int i = 0; i < 5; i++) {
                const double2 a = basis[p.basis + i * DD + i2 * D + i2];
                re = fma(f[i], a.x, re);
                im = fma(f[i], a.y, im);
            }
            mats[p.out + i2] = mk<V>((T)re, (T)(p.conjT ? -im : im));
        }
    }
}

// C > 1 only for global states shared by a cluster.  The cluster barrier
// arrives with release and waits with acquire semantics at cluster scope, so
// the window's global writes of every CTA are visible to the whole cluster
// after it (the accesses themselves bypass L1).
__device__ __forceinline__ void esync(int C) {
    if (C > 1) {
        asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
        asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
    } else {
        __syncthreads();
    }
}

// Per trainable op of the window: one warp sums the CTA's per-thread partials
// in a fixed order (and clears them for the next use of the buffer).
template <class T, int NT>
__device__ void finalize_window(const EngArgs<T> &a, const ECirc &ci, const EWin &w, typename EAcc<T>::Slot *part,
                                int rank, int C) {
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = warp; t < w.ntrain; t += NW) {
        EAcc<T> acc;
#pragma unroll
        for (int i = 0; i < NT / 32; i++) {
            auto &sl = part[t * NT + i * 32 + lane];
            EAcc<T> x;
            x.load(sl);
            acc.merge(x);
            sl = typename EAcc<T>::Slot{};
        }
        const double s = acc.warp_sum();
        if (lane == 0) {
            const ETrain tr = a.train[w.tr0 + t];
            const int js = ci.jac0 + tr.slot;
            if (C > 1) a.jac_part[(size_t)js * kMaxCluster + rank] = (double)tr.gscale * s;
            else a.jac[js] = (double)tr.gscale * s;
        }
    }
}

// H lambda and <lambda|H|lambda>; H = sum_w c_w P_w with
// <i|P|lambda> = i^ny (-1)^popc((i ^ x) & z) lambda[i ^ x]
template <class T, int NT, int MODE>
__device__ void h_pass(const EngArgs<T> &a, const ECirc &ci, c2_t<T> *lam, c2_t<T> *hl, uint32_t t0, uint32_t tstep,
                       double *misc, int rank, int C) {
    using V = c2_t<T>;
    constexpr int NW = NT / 32;
    const uint32_t N = 1u << ci.nq;
    EAcc<T> acc;
    constexpr int F = 4; // gathers issued together
    for (uint32_t i = t0; i < N; i += tstep) {
        const V li = eld<T, MODE>(lam, i);
        V hs = mk<V>(0, 0);
        for (int k0 = 0; k0 < ci.nterms; k0 += F) {
            // only the X masks are needed to issue the gathers; the rest of
            // each term is read (from L1) when it is used
            V v[F];
#pragma unroll
            for (int u = 0; u < F; u++)
                if (k0 + u < ci.nterms) v[u] = eld<T, MODE>(lam, i ^ a.terms[ci.term0 + k0 + u].x);
#pragma unroll
            for (int u = 0; u < F; u++) {
                if (k0 + u >= ci.nterms) break;
                const ETerm tm = a.terms[ci.term0 + k0 + u];
                const uint32_t j = i ^ tm.x;
                const int q = (tm.ny + 2 * (__popc(j & tm.z) & 1)) & 3;
                const V w = v[u];
                const V x = q == 0 ? w : (q == 1 ? mul_i(w) : (q == 2 ? cneg(w) : mul_mi(w)));
                const T c = (T)tm.c;
                hs = mk<V>(hs.x + c * x.x, hs.y + c * x.y);
                if constexpr (sizeof(T) == 4) acc.re_dot_scaled(tm.ch, tm.cl, li, x);
                else acc.re_dot_c(tm.c, li, x);
            }
        }
        est<T, MODE>(hl, i, hs);
    }
    const double s = acc.warp_sum();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) misc[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int wp = 0; wp < NW; wp++) t += misc[wp];
        if (C > 1) a.ev_part[(size_t)ci.id * kMaxCluster + rank] = t;
        else a.expval[ci.id] = t;
    }
}

template <class T, int NT, int MODE, int NBUF>
__device__ void run_circuit(const EngArgs<T> &a, int cid, int rank, int C, c2_t<T> *lam, c2_t<T> *hl,
                            typename EAcc<T>::Slot *part, double *misc) {
    using V = c2_t<T>;
    constexpr int NW = NT / 32;
    const ECirc ci = a.circ[cid];
    // state indices fit 32 bits (at most 30 qubits)
    const uint32_t N = 1u << ci.nq;
    const uint32_t t0 = (uint32_t)rank * NT + threadIdx.x, tstep = (uint32_t)C * NT;
    for (uint32_t i = t0; i < N; i += tstep) est<T, MODE>(lam, i, mk<V>(i == 0 ? (T)1 : (T)0, (T)0));
    esync(C);
    for (int k = 0; k < ci.nfw; k++) {
        const EWin w = a.win[ci.fw0 + k];
        if (w.flags & 1) run_window<T, NT, MODE, false, true>(a.ops, a.mats, w, ci.nq, lam, hl, t0, tstep, part);
        else run_window<T, NT, MODE, false, false>(a.ops, a.mats, w, ci.nq, lam, hl, t0, tstep, part);
        esync(C);
    }
    h_pass<T, NT, MODE>(a, ci, lam, hl, t0, tstep, misc, rank, C);
    esync(C);
    if (C > 1 && rank == 0 && threadIdx.x == 0) {
        double t = 0.0;
        for (int r = 0; r < C; r++) t += a.ev_part[(size_t)ci.id * kMaxCluster + r];
        a.expval[ci.id] = t;
    }
    for (int k = 0; k < ci.nbw; k++) {
        const EWin w = a.win[ci.bw0 + k];
        // two partial buffers: finalizing window k overlaps window k + 1;
        // one buffer: a barrier after finalizing
        typename EAcc<T>::Slot *rb = part + (NBUF == 2 ? (k & 1) : 0) * kMaxWinTrain * NT;
        if (w.flags & 1) run_window<T, NT, MODE, true, true>(a.ops, a.mats, w, ci.nq, lam, hl, t0, tstep, rb);
        else run_window<T, NT, MODE, true, false>(a.ops, a.mats, w, ci.nq, lam, hl, t0, tstep, rb);
        esync(C);
        finalize_window<T, NT>(a, ci, w, rb, rank, C);
        if (NBUF == 1) esync(C);
    }
    esync(C);
    if (C > 1 && rank == 0) {
        for (int s = threadIdx.x; s < ci.ntp; s += NT) {
            double t = 0.0;
            for (int r = 0; r < C; r++) t += a.jac_part[(size_t)(ci.jac0 + s) * kMaxCluster + r];
            a.jac[ci.jac0 + s] = t;
        }
    }
}

// MINB CTAs per SM: 1 (255 registers, two partial buffers, states of up to
// 13 qubits in shared memory for complex64) or 2 (128 registers, one buffer,
// up to 12 qubits)
template <class T, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_batch_engine(const EngArgs<T> a) {
    constexpr int NBUF = MINB == 1 ? 2 : 1;
    using V = c2_t<T>;
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) unsigned char esmem[];
    V *s_lam = (V *)esmem;
    V *s_hl = s_lam + (1u << a.smem_bits);
    using Slot = typename EAcc<T>::Slot;
    Slot *s_part = (Slot *)(s_hl + (1u << a.smem_bits)); // [2][kMaxWinTrain][NT]
    double *s_misc = (double *)(s_part + NBUF * kMaxWinTrain * NT);
    __shared__ int s_cur;
    for (int i = threadIdx.x; i < NBUF * kMaxWinTrain * NT; i += NT) s_part[i] = Slot{};
    __syncthreads();
    V *slot_cta = a.scratch ? a.scratch + (uint64_t)blockIdx.x * 2 * a.slot_amps : nullptr;
    if (a.n_cl > 0) {
        cg::cluster_group cl = cg::this_cluster();
        const int C = (int)cl.num_blocks();
        const int rank = (int)cl.block_rank();
        V *slot_cl = a.scratch + (uint64_t)(blockIdx.x - rank) * 2 * a.slot_amps;
        for (;;) {
            if (rank == 0 && threadIdx.x == 0) s_cur = (int)atomicAdd(&a.counters[0], 1u);
            cl.sync();
            const int c = *cl.map_shared_rank(&s_cur, 0);
            cl.sync();
            if (c >= a.n_cl) break;
            run_circuit<T, NT, EM_GLOBAL, NBUF>(a, a.order_cl[c], rank, C, slot_cl, slot_cl + a.slot_amps, s_part, s_misc);
        }
    }
    for (;;) {
        if (threadIdx.x == 0) s_cur = (int)atomicAdd(&a.counters[1], 1u);
        __syncthreads();
        const int c = s_cur;
        __syncthreads();
        if (c >= a.n_solo) break;
        const int cid = a.order_solo[c];
        if (a.circ[cid].nq <= a.smem_bits) run_circuit<T, NT, EM_SMEM, NBUF>(a, cid, 0, 1, s_lam, s_hl, s_part, s_misc);
        else run_circuit<T, NT, EM_GLOBAL, NBUF>(a, cid, 0, 1, slot_cta, slot_cta + a.slot_amps, s_part, s_misc);
    }
}

// ------------------------------------------------------------- launching --
template <class T, int NT, int MINB> static size_t engine_smem(int smem_bits) {
    return 2 * (sizeof(c2_t<T>) << smem_bits) + (MINB == 1 ? 2 : 1) * kMaxWinTrain * NT * sizeof(typename EAcc<T>::Slot) +
           (NT / 32 + 8) * sizeof(double);
}
template <class T, int MINB> static int max_smem_bits() { return sizeof(T) == 4 ? (MINB == 1 ? 13 : 12) : 12; }

template <class T, int NT, int MINB> static int plan_launch(plk_batch b, LaunchPlan &lp) {
    const BatchConfig &cfg = b->cfg;
    const int sb = std::min(cfg.smem_bits, max_smem_bits<T, MINB>());
    lp.smem = engine_smem<T, NT, MINB>(sb);
    auto kern = k_batch_engine<T, NT, MINB>;
    PLK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lp.smem));
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(b->device, &d));
    int per_sm = 0;
    PLK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, lp.smem));
    if (per_sm < 1) PLK_FAIL(PLK_ERR_UNSUPPORTED, "batch engine does not fit on an SM with this configuration");
    lp.cluster = std::max(1, std::min(cfg.cluster, kMaxCluster));
    // classify and order circuits (largest cost first)
    std::vector<int32_t> cl, solo;
    lp.max_global_nq = 0;
    for (size_t i = 0; i < b->h_circ.size(); i++) {
        const int nq = b->h_circ[i].nq;
        if (lp.cluster > 1 && nq > sb && nq >= cfg.cluster_min_qubits) cl.push_back((int32_t)i);
        else solo.push_back((int32_t)i);
        if (nq > sb) lp.max_global_nq = std::max(lp.max_global_nq, nq);
    }
    auto by_cost = [&](int32_t x, int32_t y) { return b->cost[x] > b->cost[y] || (b->cost[x] == b->cost[y] && x < y); };
    std::sort(cl.begin(), cl.end(), by_cost);
    std::sort(solo.begin(), solo.end(), by_cost);
    if (cl.empty()) lp.cluster = 1;
    lp.n_cl = (int)cl.size();
    lp.n_solo = (int)solo.size();
    lp.order = cl;
    lp.order.insert(lp.order.end(), solo.begin(), solo.end());
    if (lp.cluster > 1) {
        cudaLaunchConfig_t lc = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = lp.cluster;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        lc.gridDim = dim3(lp.cluster * d->sm_count);
        lc.blockDim = dim3(NT);
        lc.dynamicSmemBytes = lp.smem;
        lc.attrs = at;
        lc.numAttrs = 1;
        int ncl = 0;
        PLK_CUDA(cudaOccupancyMaxActiveClusters(&ncl, kern, &lc));
        if (ncl < 1) PLK_FAIL(PLK_ERR_UNSUPPORTED, "no cluster of this size fits the device");
        lp.grid = ncl * lp.cluster;
    } else {
        lp.grid = per_sm * d->sm_count;
    }
    lp.slot_amps = lp.max_global_nq > 0 ? (1ull << lp.max_global_nq) : 0;
    return PLK_OK;
}

template <class T, int NT, int MINB> static int launch_engine(plk_batch b, const LaunchPlan &lp, cudaStream_t st) {
    using V = c2_t<T>;
    EngArgs<T> a;
    a.circ = (const ECirc *)b->d_circ;
    a.win = (const EWin *)b->d_win;
    a.ops = (const EOp *)b->d_ops;
    a.train = (const ETrain *)b->d_train;
    a.terms = (const ETerm *)b->d_terms;
    a.mats = (const V *)b->d_mats;
    a.order_cl = (const int32_t *)b->d_order;
    a.order_solo = (const int32_t *)b->d_order + lp.n_cl;
    a.n_cl = lp.n_cl;
    a.n_solo = lp.n_solo;
    a.counters = b->d_counters;
    a.scratch = (V *)b->d_scratch;
    a.slot_amps = lp.slot_amps;
    a.expval = b->d_expval;
    a.jac = b->d_jac;
    a.jac_part = b->d_jac_part;
    a.ev_part = b->d_ev_part;
    a.smem_bits = std::min(b->cfg.smem_bits, max_smem_bits<T, MINB>());
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute at[1];
    lc.gridDim = dim3(lp.grid);
    lc.blockDim = dim3(NT);
    lc.dynamicSmemBytes = lp.smem;
    lc.stream = st;
    if (lp.cluster > 1) {
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = lp.cluster;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        lc.attrs = at;
        lc.numAttrs = 1;
    }
    PLK_CUDA(cudaLaunchKernelEx(&lc, k_batch_engine<T, NT, MINB>, a));
    return PLK_OK;
}

static int cfg_key(const BatchConfig &c) {
    return (((c.cluster * 4 + c.ctas_per_sm) * 1024 + c.threads) * 64 + c.smem_bits) * 64 + c.cluster_min_qubits;
}



template <class T> static int prepare_run(plk_batch b) {
    if (!b->compiled) {
        PLK_TRY(compile_batch(b));
        PLK_TRY(upload_batch<T>(b));
    }
    if (b->lp_key == cfg_key(b->cfg)) return PLK_OK;
    LaunchPlan &lp = b->lp;
    lp = LaunchPlan();
    if constexpr (sizeof(T) == 4) {
        if (b->cfg.ctas_per_sm == 2) PLK_TRY((plan_launch<T, 256, 2>(b, lp)));
        else PLK_TRY((plan_launch<T, 256, 1>(b, lp)));
    } else {
        PLK_TRY((plan_launch<T, 256, 1>(b, lp)));
    }
    // order and scratch for this configuration
    PLK_CUDA(cudaMemcpyAsync(b->d_order, lp.order.data(), lp.order.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                             b->stream));
    const size_t need = lp.slot_amps ? (size_t)lp.grid * 2 * lp.slot_amps * sizeof(c2_t<T>) : 0;
    if (need > b->scratch_bytes) {
        if (b->d_scratch) cudaFree(b->d_scratch);
        b->d_scratch = nullptr;
        b->scratch_bytes = 0;
        PLK_CUDA(cudaMalloc(&b->d_scratch, need));
        b->scratch_bytes = need;
    }
    PLK_CUDA(cudaStreamSynchronize(b->stream));
    b->lp_key = cfg_key(b->cfg);
    return PLK_OK;
}

// The stream work of one run: counters, matrices from parameters, engine.
template <class T> static int enqueue_run(plk_batch b, const double *d_params, cudaStream_t st) {
    const LaunchPlan &lp = b->lp;
    PLK_CUDA(cudaMemsetAsync(b->d_counters, 0, 4 * sizeof(unsigned), st));
    const int np = (int)b->h_prep.size();
    if (np > 0) {
        k_batch_prepare<T><<<(np + 255) / 256, 256, 0, st>>>((const EPrep *)b->d_prep, np, (const double2 *)b->d_basis,
                                                             d_params, (c2_t<T> *)b->d_mats);
        PLK_CHECK_LAUNCH();
    }
    if constexpr (sizeof(T) == 4) {
        if (b->cfg.ctas_per_sm == 2) PLK_TRY((launch_engine<T, 256, 2>(b, lp, st)));
        else PLK_TRY((launch_engine<T, 256, 1>(b, lp, st)));
    } else {
        PLK_TRY((launch_engine<T, 256, 1>(b, lp, st)));
    }
    return PLK_OK;
}

template <class T> static int run_host(plk_batch b, double *expval, double *jac) {
    PLK_TRY(prepare_run<T>(b));
    const size_t nc = b->circs.size();
    const size_t npar = b->params.size();
    cudaStream_t st = b->stream;
    std::memcpy(b->h_params_pinned, b->params.data(), npar * sizeof(double));
    if (b->use_graph && b->graph_cfg_key != cfg_key(b->cfg)) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t g = nullptr;
        PLK_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int rc = PLK_OK;
        if (npar && cudaMemcpyAsync(b->d_params, b->h_params_pinned, npar * sizeof(double), cudaMemcpyHostToDevice,
                                    st) != cudaSuccess)
            rc = PLK_ERR_CUDA;
        if (rc == PLK_OK) rc = enqueue_run<T>(b, b->d_params, st);
        if (rc == PLK_OK && cudaMemcpyAsync(b->h_out_pinned, b->d_expval, nc * sizeof(double), cudaMemcpyDeviceToHost,
                                            st) != cudaSuccess)
            rc = PLK_ERR_CUDA;
        if (rc == PLK_OK && b->njac &&
            cudaMemcpyAsync(b->h_out_pinned + nc, b->d_jac, b->njac * sizeof(double), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess)
            rc = PLK_ERR_CUDA;
        const cudaError_t ec = cudaStreamEndCapture(st, &g);
        if (rc != PLK_OK) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            PLK_FAIL(rc, "batch: graph capture failed: " + last_error());
        }
        PLK_CUDA(ec);
        const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        PLK_CUDA(ei);
        b->graph_cfg_key = cfg_key(b->cfg);
    }
    cudaEvent_t e0, e1;
    PLK_CUDA(cudaEventCreate(&e0));
    PLK_CUDA(cudaEventCreate(&e1));
    PLK_CUDA(cudaEventRecord(e0, st));
    if (b->use_graph) {
        PLK_CUDA(cudaGraphLaunch(b->graph, st));
    } else {
        if (npar)
            PLK_CUDA(cudaMemcpyAsync(b->d_params, b->h_params_pinned, npar * sizeof(double), cudaMemcpyHostToDevice, st));
        PLK_TRY(enqueue_run<T>(b, b->d_params, st));
        PLK_CUDA(cudaMemcpyAsync(b->h_out_pinned, b->d_expval, nc * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (b->njac)
            PLK_CUDA(cudaMemcpyAsync(b->h_out_pinned + nc, b->d_jac, b->njac * sizeof(double), cudaMemcpyDeviceToHost,
                                     st));
    }
    PLK_CUDA(cudaEventRecord(e1, st));
    PLK_CUDA(cudaStreamSynchronize(st));
    cudaEventElapsedTime(&b->last_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->last_launches = b->h_prep.empty() ? 1 : 2;
    if (expval) std::memcpy(expval, b->h_out_pinned, nc * sizeof(double));
    if (jac && b->njac) std::memcpy(jac, b->h_out_pinned + nc, b->njac * sizeof(double));
    return PLK_OK;
}

template <class T>
static int run_device(plk_batch b, const double *d_params, double *d_expval, double *d_jac, cudaStream_t st) {
    PLK_TRY(prepare_run<T>(b));
    PLK_TRY(enqueue_run<T>(b, d_params ? d_params : b->d_params, st));
    const size_t nc = b->circs.size();
    if (d_expval)
        PLK_CUDA(cudaMemcpyAsync(d_expval, b->d_expval, nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (d_jac && b->njac)
        PLK_CUDA(cudaMemcpyAsync(d_jac, b->d_jac, b->njac * sizeof(double), cudaMemcpyDeviceToDevice, st));
    return PLK_OK;
}

static int gate_nwires(int g) { return plk_gate_num_wires(g); }
static int gate_nparams(int g) { return plk_gate_num_params(g); }

static int add_circuit(plk_batch b, int nq, const plk_op *ops, int nops, const int64_t *trainable, int ntp,
                       int nterms, const double *coeffs, const int64_t *offsets, const int64_t *wires,
                       const char *letters, int64_t *index) {
    if (nq < kWinBits || nq > 30)
        PLK_FAIL(PLK_ERR_UNSUPPORTED, "batch circuits need 4 to 30 qubits, got " + std::to_string(nq));
    if (nops < 0 || (nops > 0 && !ops) || nterms < 0 || (nterms > 0 && (!coeffs || !offsets || !letters)))
        PLK_FAIL(PLK_ERR_INVALID_ARG, "null argument");
    plk_batch_s::Circ c;
    c.nq = nq;
    c.p0 = (int)b->params.size();
    std::vector<double> prm;
    auto check_w = [&](const int64_t *w, int k) -> int {
        if (k > 0 && !w) PLK_FAIL(PLK_ERR_INVALID_ARG, "null wires");
        for (int j = 0; j < k; j++) {
            if (w[j] < 0 || w[j] >= nq) PLK_FAIL(PLK_ERR_INVALID_ARG, "wire out of range");
            for (int i = 0; i < j; i++)
                if (w[i] == w[j]) PLK_FAIL(PLK_ERR_INVALID_ARG, "repeated wire");
        }
        return PLK_OK;
    };
    // expand
    std::vector<XOp> xs;
    for (int i = 0; i < nops; i++) {
        const plk_op &op = ops[i];
        if (op.gate < 0 || op.gate >= PLK_GATE_COUNT) PLK_FAIL(PLK_ERR_UNKNOWN_GATE, "unknown gate in op list");
        PLK_TRY(check_w(op.wires, op.num_wires));
        const int g = op.gate;
        const int gw = g == PLK_GATE_MATRIX ? op.num_wires : gate_nwires(g);
        if (gw > 0 && op.num_wires != gw)
            PLK_FAIL(PLK_ERR_INVALID_ARG, "gate acts on " + std::to_string(gw) + " wires, got " +
                                              std::to_string(op.num_wires));
        const int gp = g == PLK_GATE_MATRIX ? 0 : gate_nparams(g);
        if (op.num_params < gp || (gp > 0 && !op.params)) PLK_FAIL(PLK_ERR_INVALID_ARG, "missing gate parameters");
        const bool inv = op.adjoint != 0;
        auto base_op = [&](int gate, int K, const int64_t *w) {
            XOp x;
            x.gate = gate;
            x.K = K;
            for (int j = 0; j < 4; j++) x.wires[j] = j < K ? (int)w[j] : 0;
            x.inv = inv;
            x.pidx = -1;
            x.slot = -1;
            x.basis = -1;
            x.user_matrix = -1;
            x.kind = EK_DENSE;
            return x;
        };
        if (g == PLK_GATE_IDENTITY) continue;
        if (g == PLK_GATE_ROT || g == PLK_GATE_CROT) {
            const int K = g == PLK_GATE_ROT ? 1 : 2;
            const int gz = g == PLK_GATE_ROT ? PLK_GATE_RZ : PLK_GATE_CRZ;
            const int gy = g == PLK_GATE_ROT ? PLK_GATE_RY : PLK_GATE_CRY;
            // Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi); the inverse
            // applies RZ(-omega), RY(-theta), RZ(-phi)
            const int seq[3] = {gz, gy, gz};
            const int pi[3] = {inv ? 2 : 0, 1, inv ? 0 : 2};
            const int pbase = (int)prm.size();
            for (int k = 0; k < 3; k++) prm.push_back(op.params[k]);
            for (int k = 0; k < 3; k++) {
                XOp x = base_op(seq[k], K, op.wires);
                x.pidx = pbase + pi[k];
                x.kind = is_diag_gate(seq[k]) ? EK_DIAG : EK_DENSE;
                xs.push_back(x);
            }
            continue;
        }
        if (g == PLK_GATE_MULTIRZ) {
            if (op.num_wires < 1) PLK_FAIL(PLK_ERR_INVALID_ARG, "MultiRZ needs at least one wire");
            XOp x = base_op(g, 0, op.wires);
            x.mrz_wires.assign(op.wires, op.wires + op.num_wires);
            x.K = 1;
            x.kind = EK_PARITY;
            x.pidx = (int)prm.size();
            prm.push_back(op.params[0]);
            xs.push_back(x);
            continue;
        }
        if (op.num_wires > kWinBits)
            PLK_FAIL(PLK_ERR_UNSUPPORTED, "batch circuits support gates on at most 4 wires (and MultiRZ)");
        XOp x = base_op(g, op.num_wires, op.wires);
        if (g == PLK_GATE_MATRIX) {
            if (!op.matrix) PLK_FAIL(PLK_ERR_INVALID_ARG, "matrix op without a matrix");
            const int D = 1 << op.num_wires;
            std::vector<double2> A(5 * (size_t)D * D, mk<double2>(0, 0));
            for (int e = 0; e < D * D; e++) {
                const int r = e / D, cc = e % D;
                // adjoint: conjugate transpose
                const int src = inv ? cc * D + r : e;
                A[e] = mk<double2>(op.matrix[2 * src], inv ? -op.matrix[2 * src + 1] : op.matrix[2 * src + 1]);
            }
            x.user_matrix = (int)b->user_mats.size();
            b->user_mats.push_back(A);
            x.basis = (int)b->basis.size();
            b->basis.insert(b->basis.end(), A.begin(), A.end());
            xs.push_back(x);
            continue;
        }
        if (gp == 1) {
            x.pidx = (int)prm.size();
            prm.push_back(op.params[0]);
        }
        if (g == PLK_GATE_CNOT) x.kind = EK_CX;
        else if (is_diag_gate(g)) x.kind = EK_DIAG;
        xs.push_back(x);
    }
    c.np = (int)prm.size();
    // trainable parameters (flat indices of this circuit; all when null)
    std::vector<int64_t> tp;
    if (trainable) {
        for (int t = 0; t < ntp; t++) {
            if (trainable[t] < 0 || trainable[t] >= c.np) PLK_FAIL(PLK_ERR_INVALID_ARG, "trainable index out of range");
            if (t > 0 && trainable[t] <= trainable[t - 1])
                PLK_FAIL(PLK_ERR_INVALID_ARG, "trainable parameters must be sorted and unique");
            tp.push_back(trainable[t]);
        }
    } else {
        for (int t = 0; t < c.np; t++) tp.push_back(t);
    }
    std::vector<int> slot_of(c.np, -1);
    for (size_t t = 0; t < tp.size(); t++) slot_of[tp[t]] = (int)t;
    for (auto &x : xs) {
        if (x.pidx >= 0) {
            x.slot = slot_of[x.pidx];
            if (x.slot >= 0 && x.gate == PLK_GATE_MATRIX)
                PLK_FAIL(PLK_ERR_INVALID_ARG, "matrix ops have no parameter to differentiate");
            x.pidx += c.p0;
        }
        if (x.basis < 0) PLK_TRY(basis_for(b, x.gate, x.inv, x.K, x.basis));
    }
    c.ops = std::move(xs);
    c.ntp = (int)tp.size();
    c.jac0 = b->njac;
    // observable
    for (int t = 0; t < nterms; t++) {
        ETerm e;
        e.x = e.z = 0;
        e.ny = 0;
        e.c = coeffs[t];
        df_split_host(coeffs[t], e.ch, e.cl);
        const int64_t o0 = offsets[t], o1 = offsets[t + 1];
        if (o1 < o0) PLK_FAIL(PLK_ERR_INVALID_ARG, "Pauli word offsets must not decrease");
        for (int64_t k = o0; k < o1; k++) {
            const int64_t w = wires[k];
            if (w < 0 || w >= nq) PLK_FAIL(PLK_ERR_INVALID_ARG, "Pauli word wire out of range");
            const uint32_t bit = 1u << (nq - 1 - w);
            if ((e.x | e.z) & bit) PLK_FAIL(PLK_ERR_INVALID_ARG, "repeated wire in a Pauli word");
            switch (letters[k]) {
            case 'X': e.x |= bit; break;
            case 'Y': e.x |= bit; e.z |= bit; e.ny++; break;
            case 'Z': e.z |= bit; break;
            case 'I': break;
            default: PLK_FAIL(PLK_ERR_INVALID_ARG, std::string("unknown Pauli letter ") + letters[k]);
            }
        }
        c.terms.push_back(e);
    }
    b->params.insert(b->params.end(), prm.begin(), prm.end());
    b->njac += c.ntp;
    if (index) *index = (int64_t)b->circs.size();
    b->circs.push_back(std::move(c));
    b->compiled = false;
    free_device(b);
    return PLK_OK;
}

} // namespace plk

using namespace plk;

extern "C" {

PLK_API int plk_gate_matrix(int32_t gate, const double *params, int32_t num_params, int32_t adjoint, int32_t num_wires,
                            double *out) {
    if (!out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    if (gate == PLK_GATE_MATRIX) PLK_FAIL(PLK_ERR_INVALID_ARG, "Matrix has no named gate matrix");
    if (num_wires < 1 || num_wires > 12) PLK_FAIL(PLK_ERR_INVALID_ARG, "num_wires must be 1..12");
    GatePlan p;
    const double zero[3] = {0, 0, 0};
    PLK_TRY(plan_gate(gate, num_wires, adjoint != 0, params ? params : zero, params ? num_params : 3, p));
    std::vector<double2> M;
    plan_dense(p, num_wires, M);
    for (size_t i = 0; i < M.size(); i++) {
        out[2 * i] = M[i].x;
        out[2 * i + 1] = M[i].y;
    }
    return PLK_OK;
}

PLK_API int plk_batch_create(int32_t dtype, int32_t device, plk_batch *out) {
    if (!out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    *out = nullptr;
    if (dtype != PLK_C64 && dtype != PLK_C128) PLK_FAIL(PLK_ERR_INVALID_ARG, "dtype must be PLK_C64 or PLK_C128");
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(device, &d));
    PLK_CUDA(cudaSetDevice(device));
    plk_batch b = new plk_batch_s();
    b->dtype = dtype;
    b->device = device;
    b->cfg.smem_bits = dtype == PLK_C64 ? 13 : 12;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        cudaGetLastError();
        PLK_FAIL(PLK_ERR_CUDA, "cannot create a stream");
    }
    *out = b;
    return PLK_OK;
}

PLK_API int plk_batch_destroy(plk_batch b) {
    if (!b) return PLK_OK;
    cudaSetDevice(b->device);
    free_device(b);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return PLK_OK;
}

PLK_API int plk_batch_add(plk_batch b, int32_t num_qubits, const plk_op *ops, int32_t num_ops,
                          const int64_t *trainable, int32_t num_trainable, int32_t num_terms, const double *coeffs,
                          const int64_t *offsets, const int64_t *wires, const char *letters, int64_t *index) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    return add_circuit(b, num_qubits, ops, num_ops, trainable, num_trainable, num_terms, coeffs, offsets, wires,
                       letters, index);
}

PLK_API int plk_batch_info(plk_batch b, int64_t *num_circuits, int64_t *num_params, int64_t *num_jac) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (num_circuits) *num_circuits = (int64_t)b->circs.size();
    if (num_params) *num_params = (int64_t)b->params.size();
    if (num_jac) *num_jac = b->njac;
    return PLK_OK;
}

PLK_API int plk_batch_circuit_info(plk_batch b, int64_t circuit, int64_t *param_offset, int32_t *num_params,
                                   int64_t *jac_offset, int32_t *num_trainable) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (circuit < 0 || circuit >= (int64_t)b->circs.size()) PLK_FAIL(PLK_ERR_INVALID_ARG, "circuit index out of range");
    const auto &c = b->circs[circuit];
    if (param_offset) *param_offset = c.p0;
    if (num_params) *num_params = c.np;
    if (jac_offset) *jac_offset = c.jac0;
    if (num_trainable) *num_trainable = c.ntp;
    return PLK_OK;
}

PLK_API int plk_batch_set_params(plk_batch b, const double *params, int64_t count) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (count != (int64_t)b->params.size())
        PLK_FAIL(PLK_ERR_INVALID_ARG, "expected " + std::to_string(b->params.size()) + " parameters");
    if (count && !params) PLK_FAIL(PLK_ERR_INVALID_ARG, "null parameters");
    std::copy(params, params + count, b->params.begin());
    return PLK_OK;
}

PLK_API int plk_batch_set_config(plk_batch b, int32_t cluster, int32_t threads, int32_t smem_qubits,
                                 int32_t cluster_min_qubits) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8)
        PLK_FAIL(PLK_ERR_INVALID_ARG, "cluster must be 1, 2, 4 or 8");
    if (threads != 256) PLK_FAIL(PLK_ERR_INVALID_ARG, "threads must be 256");
    const int maxsb = b->dtype == PLK_C64 && b->cfg.ctas_per_sm == 1 ? 13 : 12;
    if (smem_qubits < kWinBits || smem_qubits > maxsb)
        PLK_FAIL(PLK_ERR_INVALID_ARG, "smem_qubits must be 4.." + std::to_string(maxsb));
    b->cfg.cluster = cluster;
    b->cfg.threads = threads;
    b->cfg.smem_bits = smem_qubits;
    b->cfg.cluster_min_qubits = cluster_min_qubits;
    return PLK_OK;
}

PLK_API int plk_batch_set_occupancy(plk_batch b, int32_t ctas_per_sm) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (ctas_per_sm != 1 && ctas_per_sm != 2) PLK_FAIL(PLK_ERR_INVALID_ARG, "ctas_per_sm must be 1 or 2");
    if (ctas_per_sm == 2 && b->dtype != PLK_C64) PLK_FAIL(PLK_ERR_UNSUPPORTED, "two CTAs per SM need complex64");
    b->cfg.ctas_per_sm = ctas_per_sm;
    b->cfg.smem_bits = std::min(b->cfg.smem_bits, ctas_per_sm == 2 ? 12 : 13);
    return PLK_OK;
}

PLK_API int plk_batch_get_occupancy(plk_batch b, int32_t *ctas_per_sm) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (ctas_per_sm) *ctas_per_sm = b->cfg.ctas_per_sm;
    return PLK_OK;
}

PLK_API int plk_batch_get_config(plk_batch b, int32_t *cluster, int32_t *threads, int32_t *smem_qubits,
                                 int32_t *cluster_min_qubits) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (cluster) *cluster = b->cfg.cluster;
    if (threads) *threads = b->cfg.threads;
    if (smem_qubits) *smem_qubits = b->cfg.smem_bits;
    if (cluster_min_qubits) *cluster_min_qubits = b->cfg.cluster_min_qubits;
    return PLK_OK;
}

PLK_API int plk_batch_set_graph(plk_batch b, int32_t use_graph) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    b->use_graph = use_graph != 0;
    return PLK_OK;
}

PLK_API int plk_batch_run(plk_batch b, double *expvals, double *jac) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (b->circs.empty()) PLK_FAIL(PLK_ERR_INVALID_ARG, "empty batch");
    PLK_CUDA(cudaSetDevice(b->device));
    return b->dtype == PLK_C64 ? run_host<float>(b, expvals, jac) : run_host<double>(b, expvals, jac);
}

PLK_API int plk_batch_run_device(plk_batch b, const double *d_params, double *d_expvals, double *d_jac, void *stream) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (b->circs.empty()) PLK_FAIL(PLK_ERR_INVALID_ARG, "empty batch");
    PLK_CUDA(cudaSetDevice(b->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
    return b->dtype == PLK_C64 ? run_device<float>(b, d_params, d_expvals, d_jac, st)
                               : run_device<double>(b, d_params, d_expvals, d_jac, st);
}

PLK_API int plk_batch_last_time(plk_batch b, double *ms, int64_t *launches) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (ms) *ms = b->last_ms;
    if (launches) *launches = b->last_launches;
    return PLK_OK;
}

// Autotuner: times every configuration of a small grid on this batch and
// keeps the fastest (median of `reps` graph replays after one warm-up).
PLK_API int plk_batch_tune(plk_batch b, int32_t reps, char *report, int32_t report_len) {
    if (!b) PLK_FAIL(PLK_ERR_INVALID_ARG, "null batch");
    if (b->circs.empty()) PLK_FAIL(PLK_ERR_INVALID_ARG, "empty batch");
    PLK_CUDA(cudaSetDevice(b->device));
    reps = std::max(1, reps);
    const BatchConfig saved = b->cfg;
    std::vector<BatchConfig> cands;
    int max_nq = 0;
    for (auto &c : b->circs) max_nq = std::max(max_nq, c.nq);
    for (int ctas : {1, 2}) {
        if (ctas == 2 && b->dtype != PLK_C64) continue;
        const int sb = b->dtype == PLK_C64 && ctas == 1 ? 13 : 12;
        for (int cl : {1, 2, 4, 8}) {
            for (int cmin : {sb + 1, sb + 3, sb + 5}) {
                if (cl == 1 && cmin != sb + 1) continue;
                if (cl > 1 && cmin > max_nq) continue;
                BatchConfig c;
                c.threads = 256;
                c.ctas_per_sm = ctas;
                c.cluster = cl;
                c.smem_bits = sb;
                c.cluster_min_qubits = cmin;
                cands.push_back(c);
            }
        }
    }
    std::string rep;
    double best = 1e300;
    BatchConfig best_cfg = saved;
    for (const auto &c : cands) {
        b->cfg = c;
        int st = plk_batch_run(b, nullptr, nullptr); // warm-up (and graph capture)
        if (st != PLK_OK) {
            rep += "ctas_per_sm=" + std::to_string(c.ctas_per_sm) + " cluster=" + std::to_string(c.cluster) +
                   " cluster_min=" + std::to_string(c.cluster_min_qubits) + " failed: " + last_error() + "\n";
            continue;
        }
        std::vector<double> t;
        for (int r = 0; r < reps; r++) {
            PLK_TRY(plk_batch_run(b, nullptr, nullptr));
            t.push_back(b->last_ms);
        }
        std::sort(t.begin(), t.end());
        const double med = t[t.size() / 2];
        char line[160];
        std::snprintf(line, sizeof(line), "ctas_per_sm=%d cluster=%d smem_qubits=%d cluster_min=%d: %.3f ms\n",
                      c.ctas_per_sm, c.cluster, c.smem_bits, c.cluster_min_qubits, med);
        rep += line;
        if (med < best) {
            best = med;
            best_cfg = c;
        }
    }
    b->cfg = best_cfg;
    b->tuned = true;
    if (report && report_len > 0) {
        std::strncpy(report, rep.c_str(), (size_t)report_len - 1);
        report[report_len - 1] = 0;
    }
    return PLK_OK;
}

} // extern "C"
