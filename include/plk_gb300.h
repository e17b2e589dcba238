/*
 * plk_gb300.h — C ABI of the GB300 state-vector core.
 *
 * A drop-in replacement for the device path under the LightningKokkos
 * plugin: the C++ host layer (state, measures, observables, adjoint
 * Jacobian) and the pybind11 module `lightning_kokkos_qubit_ops` call these
 * functions, which run hand-written sm_103a CUDA kernels.  Each declaration
 * names the reference entry point it replaces (paths relative to
 * pennylane_lightning_kokkos/src/).
 *
 * Conventions
 *   - A state holds 2^num_qubits amplitudes, complex64 (PLK_C64) or
 *     complex128 (PLK_C128), contiguous, wire 0 = most significant bit of the
 *     amplitude index (the reference's rev_wire = n - wire - 1).
 *   - Every function returns a plk_status; on failure plk_last_error()
 *     returns a message (thread-local) and the state is left unchanged
 *     unless stated otherwise.
 *   - Matrices are complex128, row-major, interleaved (re, im), whatever the
 *     state precision; a k-wire matrix has 4^k entries and wires[0] is the
 *     most significant bit of its row/column index.
 *   - Reductions (expectation values, inner products, Jacobian entries)
 *     accumulate in FP64 for both precisions and are deterministic: the same
 *     inputs on the same GPU give the same bits.
 *   - Host pointers may be pageable or pinned; device work for a state is
 *     issued on the state's stream (plk_state_set_stream).  Functions that
 *     return host values synchronize that stream.
 */
#ifndef PLK_GB300_H
#define PLK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLK_API __attribute__((visibility("default")))

typedef enum {
    PLK_OK = 0,
    PLK_ERR_INVALID_ARG = 1,  /* bad wires, sizes, names, parameters        */
    PLK_ERR_UNKNOWN_GATE = 2, /* name/id without a kernel (or generator)     */
    PLK_ERR_CUDA = 3,         /* a CUDA runtime call failed                 */
    PLK_ERR_OUT_OF_MEMORY = 4,
    PLK_ERR_UNSUPPORTED = 5,  /* valid request outside this build's limits  */
    PLK_ERR_NO_DEVICE = 6
} plk_status;

typedef enum { PLK_C64 = 0, PLK_C128 = 1 } plk_dtype;

/* Gate identifiers: the gate map of StateVectorKokkos.hpp:141-344 plus
 * Identity (a no-op, :589-590) and PLK_GATE_MATRIX (applyMultiQubitOp). */
typedef enum {
    PLK_GATE_IDENTITY = 0,
    PLK_GATE_PAULIX, PLK_GATE_PAULIY, PLK_GATE_PAULIZ, PLK_GATE_HADAMARD,
    PLK_GATE_S, PLK_GATE_T, PLK_GATE_PHASESHIFT, PLK_GATE_RX, PLK_GATE_RY,
    PLK_GATE_RZ, PLK_GATE_ROT,
    PLK_GATE_CNOT, PLK_GATE_CY, PLK_GATE_CZ, PLK_GATE_SWAP,
    PLK_GATE_CONTROLLEDPHASESHIFT, PLK_GATE_CRX, PLK_GATE_CRY, PLK_GATE_CRZ,
    PLK_GATE_CROT, PLK_GATE_ISINGXX, PLK_GATE_ISINGXY, PLK_GATE_ISINGYY,
    PLK_GATE_ISINGZZ, PLK_GATE_SINGLEEXCITATION,
    PLK_GATE_SINGLEEXCITATIONMINUS, PLK_GATE_SINGLEEXCITATIONPLUS,
    PLK_GATE_DOUBLEEXCITATION, PLK_GATE_DOUBLEEXCITATIONMINUS,
    PLK_GATE_DOUBLEEXCITATIONPLUS, PLK_GATE_CSWAP, PLK_GATE_TOFFOLI,
    PLK_GATE_MULTIRZ,
    PLK_GATE_MATRIX, /* dense 2^k x 2^k matrix in plk_op.matrix */
    PLK_GATE_COUNT
} plk_gate;

typedef struct plk_state_s *plk_state;

/* One operation of a circuit (the serialised tape of OpsData,
 * algorithms/AdjointDiffKokkos.hpp:17-173). */
typedef struct {
    int32_t gate;        /* plk_gate                                        */
    int32_t num_wires;
    int32_t adjoint;     /* apply the inverse gate                          */
    int32_t num_params;
    const int64_t *wires;
    const double *params;
    const double *matrix; /* PLK_GATE_MATRIX only: 4^num_wires complex128   */
} plk_op;

typedef struct {
    int device;
    int sm_count;
    int cc_major;
    int cc_minor;
    uint64_t total_mem;
    uint64_t free_mem;
    int clock_khz;
    int mem_clock_khz;
    int mem_bus_width;
    char name[128];
} plk_device_info;

/* ---- library ---------------------------------------------------------- */
/* Thread-local message of the last failure (never NULL). */
PLK_API const char *plk_last_error(void);
PLK_API int plk_version(void);
/* Replaces GetConfigInfo.hpp:64 getConfig / Kokkos::print_configuration
 * (bindings/Bindings.cpp:842-852) with a CUDA device description. */
PLK_API int plk_device_count(int *count);
PLK_API int plk_get_device_info(int device, plk_device_info *out);
/* Name -> plk_gate (the string keys of StateVectorKokkos.hpp:141-344). */
PLK_API int plk_gate_from_name(const char *name, int32_t *gate);
PLK_API int plk_gate_num_wires(int32_t gate);   /* -1: any number */
PLK_API int plk_gate_num_params(int32_t gate);

/* ---- state lifecycle (StateVectorKokkos.hpp:140-574, 1596-1636) ------- */
/* StateVectorKokkos(num_qubits): allocate and set |0...0> (InitView :46). */
PLK_API int plk_state_create(int num_qubits, int dtype, int device, plk_state *out);
/* Wrap caller-owned device memory (2^num_qubits amplitudes); the state does
 * not free it.  stream may be NULL (library stream of the device). */
PLK_API int plk_state_wrap(void *device_ptr, int num_qubits, int dtype, int device,
                           void *cuda_stream, plk_state *out);
PLK_API int plk_state_destroy(plk_state s);
PLK_API int plk_state_get(plk_state s, int *num_qubits, int *dtype, void **device_ptr);
PLK_API int plk_state_set_stream(plk_state s, void *cuda_stream);
PLK_API int plk_state_get_stream(plk_state s, void **cuda_stream);
PLK_API int plk_state_synchronize(plk_state s);
/* resetStateVector :508-512 */
PLK_API int plk_state_reset(plk_state s);
/* initZeros :483-485 */
PLK_API int plk_state_zero(plk_state s);
/* setBasisState :492-495 */
PLK_API int plk_state_set_basis(plk_state s, uint64_t index);
/* setStateVector :503-521: zero, then scatter values (host arrays, values in
 * the state precision, interleaved re/im). */
PLK_API int plk_state_set_values(plk_state s, const uint64_t *indices, const void *values,
                                 uint64_t count);
/* HostToDevice / DeviceToHost :1618-1628 (length in amplitudes, state
 * precision). */
PLK_API int plk_state_h2d(plk_state s, const void *host, uint64_t length);
PLK_API int plk_state_d2h(plk_state s, void *host, uint64_t length);
/* The same copies without the wait: queued on the state's stream after the
 * work already queued there, and returning at once.  The host buffer must
 * stay valid (and, for d2h, unread) until plk_state_synchronize; with pinned
 * host memory and a stream per state, one state's copies overlap another
 * state's gates. */
PLK_API int plk_state_h2d_async(plk_state s, const void *host, uint64_t length);
PLK_API int plk_state_d2h_async(plk_state s, void *host, uint64_t length);
/* DeviceToDevice / updateData :1596-1598, :1631-1633 */
PLK_API int plk_state_copy(plk_state dst, plk_state src);
/* axpy_Kokkos (util/LinearAlgebraKokkos.hpp:30-61): y += alpha * x */
PLK_API int plk_state_axpy(plk_state y, double alpha_re, double alpha_im, plk_state x);

/* ---- gates ------------------------------------------------------------ */
/* applyOperation :585-600 (named gate, adjoint flag, parameters). */
PLK_API int plk_apply_gate(plk_state s, int32_t gate, const int64_t *wires, int32_t num_wires,
                           int32_t adjoint, const double *params, int32_t num_params);
/* applyMultiQubitOp :757-796 (and single/two-qubit op :704-748). */
PLK_API int plk_apply_matrix(plk_state s, const double *matrix, const int64_t *wires,
                             int32_t num_wires, int32_t adjoint);
/* applyOperation(vector...) :640-676: a list of operations, in order. */
PLK_API int plk_apply_ops(plk_state s, const plk_op *ops, int32_t num_ops);
/* applyGenerator :687-695: apply the generator of `gate`, return its scale
 * factor (the value the reference's applyGenerator* returns). */
PLK_API int plk_apply_generator(plk_state s, int32_t gate, const int64_t *wires, int32_t num_wires,
                                int32_t adjoint, double *scale);

/* ---- expectation values and linear algebra --------------------------- */
/* getExpectationValue{Identity,PauliX,PauliY,PauliZ,Hadamard}
 * (simulator/MeasuresKokkos.hpp:167-271, ExpValFunctors.hpp:13-153);
 * gate must be one of IDENTITY, PAULIX, PAULIY, PAULIZ, HADAMARD. */
PLK_API int plk_expval_named(plk_state s, int32_t gate, const int64_t *wires, int32_t num_wires,
                             double *out);
/* Several named one-wire expectation values in one pass over the state
 * (count values; gates[i] on wires[i]). */
PLK_API int plk_expval_named_batch(plk_state s, int32_t count, const int32_t *gates,
                                   const int64_t *wires, double *out);
/* getExpectationValueMultiQubitOp :318-346 (1q/2q functors :155-250; k >= 3
 * matrices: Re<psi|M psi>). */
PLK_API int plk_expval_matrix(plk_state s, const double *matrix, const int64_t *wires,
                              int32_t num_wires, double *out);
/* getExpectationValue(data, indices, index_ptr) :111-135,
 * ExpValFunctors.hpp:252-280: CSR matrix (complex128 values). */
PLK_API int plk_expval_sparse(plk_state s, const double *data, const int64_t *indices,
                              const int64_t *indptr, int64_t num_rows, int64_t nnz, double *out);
/* Expectation value of a sum of Pauli words sum_j c_j P_j (the Hamiltonian
 * of NamedObs/TensorProdObs Pauli terms, ObservablesKokkos.hpp:296-402),
 * without materialising O|psi>.  Term j acts on
 * wires[offsets[j] .. offsets[j+1]) with letters paulis[offsets[j] ..]
 * ('I', 'X', 'Y', 'Z'). */
PLK_API int plk_expval_pauli_sum(plk_state s, int32_t num_terms, const double *coeffs,
                                 const int64_t *offsets, const int64_t *wires, const char *paulis,
                                 double *out);
/* out = sum_j c_j P_j in  (materialised Hamiltonian application; out != in) */
PLK_API int plk_apply_pauli_sum(plk_state out, plk_state in, int32_t num_terms, const double *coeffs,
                                const int64_t *offsets, const int64_t *wires, const char *paulis);
/* getRealOfComplexInnerProduct / getImagOfComplexInnerProduct
 * (LinearAlgebraKokkos.hpp:155-236): <x|y> = sum conj(x_k) y_k. */
PLK_API int plk_inner_product(plk_state x, plk_state y, double *re, double *im);
/* SparseMV_Kokkos (LinearAlgebraKokkos.hpp:68-148): y = A x (CSR). */
PLK_API int plk_spmv(plk_state y, plk_state x, const double *data, const int64_t *indices,
                     const int64_t *indptr, int64_t num_rows, int64_t nnz);

/* ---- probabilities and sampling -------------------------------------- */
/* probs() :389-408 (num_wires == 0) and probs(wires) :418-517: marginal
 * probabilities in the requested wire order, written to host `out`
 * (2^num_wires doubles). */
PLK_API int plk_probs(plk_state s, const int64_t *wires, int32_t num_wires, double *out);
/* getCDFFunctor (MeasuresFunctors.hpp:39-56): exclusive prefix sum of |psi|^2
 * in FP64, written to host `out` (2^n doubles). */
PLK_API int plk_cdf(plk_state s, double *out);
/* Sampler (MeasuresFunctors.hpp:86-119) with caller-supplied uniforms
 * (host, `shots` doubles in [0,1)); writes shots x n bits, MSB first. */
PLK_API int plk_sample_from_uniforms(plk_state s, const double *uniforms, uint64_t shots,
                                     int64_t *out_bits);
/* The same search over a caller-supplied CDF (host, `length` doubles):
 * identical indices for identical CDF and uniforms. */
PLK_API int plk_search_cdf(const double *cdf, uint64_t length, int32_t num_qubits,
                           const double *uniforms, uint64_t shots, int64_t *out_bits,
                           int device);
/* generate_samples :530-569: uniforms from a counter-based generator
 * (Philox-4x32-10) seeded by `seed`. */
PLK_API int plk_generate_samples(plk_state s, uint64_t shots, uint64_t seed, int64_t *out_bits);

/* ---- adjoint Jacobian ------------------------------------------------- */
/* AdjointJacobianKokkos::adjointJacobian (AdjointDiffKokkos.hpp:404-478),
 * apply_operations = false.  `lambda` is the forward-evolved state (not
 * modified); hlambda[i] = O_i|lambda> (overwritten).  Ops with more than one
 * parameter are rejected, StatePrep/BasisState are not representable here
 * (the host layer drops them).  jac is [num_obs][num_trainable] row-major;
 * trainable holds sorted indices into the parametric ops. */
PLK_API int plk_adjoint_jacobian(plk_state lambda, plk_state *hlambda, int32_t num_obs,
                                 const plk_op *ops, int32_t num_ops, const int64_t *trainable,
                                 int32_t num_trainable, double *jac);

/* The same sweep without the work copy of lambda: `lambda` is overwritten (it
 * ends as U_0^dag ... U_{n-1}^dag lambda).  Needs one state less, for callers
 * that regenerate lambda instead of keeping it (checkpointed re-forward). */
PLK_API int plk_adjoint_jacobian_inplace(plk_state lambda, plk_state *hlambda, int32_t num_obs,
                                         const plk_op *ops, int32_t num_ops, const int64_t *trainable,
                                         int32_t num_trainable, double *jac);

/* ---- allocation-free expectation values ------------------------------ */
/* No counterpart in the reference.  For callers that may not allocate device
 * memory — their device memory belongs to another allocator or to a fixed
 * budget, where cudaMalloc/cudaFree would bypass it and synchronize the
 * device: <PauliZ(wires[i])> (wires[i] = -1: the squared norm, i.e. Identity)
 * of a caller-owned device state of 2^num_qubits amplitudes, written to the
 * caller-owned device array `out` (count doubles) on `cuda_stream`, with no
 * plk_state and no allocation.  Its scratch is a fixed library array
 * (128.25 KiB per GPU, held until the process exits) shared by every call:
 * count is limited to 16 (larger counts are rejected), and calls that overlap
 * on the GPU race.  Runs on the current device; the first call on a device
 * sets the scratch address up and should come before any stream capture. */
PLK_API int plk_expval_pauliz_noalloc(const void *state, int32_t num_qubits, int32_t dtype, int32_t count,
                                      const int64_t *wires, double *out, void *cuda_stream);

/* ---- register-window path ----------------------------------------------- */
/* Op lists (plk_apply_ops) and adjoint Jacobians run as register-window
 * sweeps (about seven ops per state pass; complex128 in double-float on the
 * FP32 pipe; with several observables one backward sweep per observable on
 * a copy of lambda, when that moves fewer bytes) unless this is switched
 * off; results agree with the op-at-a-time path to rounding. */
PLK_API int plk_set_window_path(int32_t enable);
PLK_API int plk_get_window_path(int32_t *enabled);

/* ---- complex128 arithmetic ----------------------------------------------- */
/* How complex128 kernels compute (storage is complex128 either way; no
 * counterpart in the reference, whose Kokkos functors use native double).
 * PLK_ARITH_DOUBLE_FLOAT (default): each double is carried as an unevaluated
 * sum of two floats on the FP32 pipe (error-free products and sums, about
 * 2^-45 relative error per gate; values below about 2^-103 lose their low
 * part and below 2^-126 become zero), because this GPU's FP64 pipe is about
 * 1/64 of its FP32 rate.  PLK_ARITH_FP64: native IEEE double arithmetic (and
 * no register-window sweeps), slower for dense matrices and rotations.  The
 * environment variable PLK_C128_ARITH=fp64 selects the initial mode; the
 * setting applies to calls made after it. */
enum { PLK_ARITH_DOUBLE_FLOAT = 0, PLK_ARITH_FP64 = 1 };
PLK_API int plk_set_c128_arithmetic(int32_t mode);
PLK_API int plk_get_c128_arithmetic(int32_t *mode);

/* ---- tensor cores for dense complex64 matrices --------------------------- */
/* complex64 dense matrices on 5 or 6 wires (plk_apply_matrix,
 * applyMultiQubitOp, StateVectorKokkos.hpp:757-796) run on the tensor cores
 * (TF32 operands, three products per step for FP32 accuracy) unless this is
 * switched off; off, they run on the CUDA cores in FP32. */
PLK_API int plk_set_dense_tensor_cores(int32_t enable);
PLK_API int plk_get_dense_tensor_cores(int32_t *enabled);

/* ---- gate matrices ---------------------------------------------------- */
/* Dense matrix (row-major complex128 pairs, 4^num_wires of them; wires[0] is
 * the most significant bit of the row index) of a named gate, built from the
 * same gate plans as the state kernels.  The reference builds these on the
 * Python side (pennylane.operation.Operation.matrix, consumed by
 * StateVectorKokkos::applyMultiQubitOp, StateVectorKokkos.hpp:763-796). */
PLK_API int plk_gate_matrix(int32_t gate, const double *params, int32_t num_params, int32_t adjoint,
                            int32_t num_wires, double *out);

/* ---- batched circuits ------------------------------------------------- */
/* Many independent circuits (own qubit count 4..30, own gates and
 * parameters, own Pauli-sum observable) evaluated together: for every circuit
 * the forward pass from |0...0>, <H> and the adjoint gradient d<H>/dtheta of
 * its trainable parameters, in one persistent launch (replayed as a CUDA
 * graph).  Per circuit this is what the reference's device does one tape at
 * a time: apply the tape (StateVectorKokkos::applyOperation,
 * StateVectorKokkos.hpp:585-676), the Hamiltonian expectation
 * (ObservablesKokkos.hpp:484-494) and AdjointJacobianKokkos::adjointJacobian
 * (AdjointDiffKokkos.hpp:404-478).  Gates act on at most 4 wires (MultiRZ on
 * any number); Rot and CRot are decomposed into RZ RY RZ (CRZ CRY CRZ) and
 * each of their three parameters is differentiable.  Parameters of a circuit
 * form a flat list in op order; `trainable` lists sorted indices into it
 * (NULL: all).  The observable is packed as in plk_expval_pauli_sum. */
typedef struct plk_batch_s *plk_batch;
PLK_API int plk_batch_create(int32_t dtype, int32_t device, plk_batch *out);
PLK_API int plk_batch_destroy(plk_batch b);
PLK_API int plk_batch_add(plk_batch b, int32_t num_qubits, const plk_op *ops, int32_t num_ops,
                          const int64_t *trainable, int32_t num_trainable, int32_t num_terms,
                          const double *coeffs, const int64_t *offsets, const int64_t *wires,
                          const char *letters, int64_t *index);
/* totals: circuits, flat parameters, Jacobian entries (sum of trainables) */
PLK_API int plk_batch_info(plk_batch b, int64_t *num_circuits, int64_t *num_params, int64_t *num_jac);
PLK_API int plk_batch_circuit_info(plk_batch b, int64_t circuit, int64_t *param_offset, int32_t *num_params,
                                   int64_t *jac_offset, int32_t *num_trainable);
/* replaces all parameters (flat, circuits in the order they were added) */
PLK_API int plk_batch_set_params(plk_batch b, const double *params, int64_t count);
/* expvals: one per circuit; jac: flat, circuit c at its jac_offset, in the
 * order of its trainable list.  Either may be NULL.  Synchronous. */
PLK_API int plk_batch_run(plk_batch b, double *expvals, double *jac);
/* Device variant for callers that keep parameters and results on the GPU:
 * enqueues the run on cuda_stream (NULL: the batch's stream) without host
 * synchronisation or allocation after the first call of a configuration. */
PLK_API int plk_batch_run_device(plk_batch b, const double *d_params, double *d_expvals, double *d_jac,
                                 void *cuda_stream);
/* device time (CUDA events) and kernel launches of the last plk_batch_run */
PLK_API int plk_batch_last_time(plk_batch b, double *ms, int64_t *launches);
/* launch configuration: CTAs per cluster (1, 2, 4, 8), threads per CTA (256),
 * circuits of at most smem_qubits qubits run in shared memory, circuits of at
 * least cluster_min_qubits qubits are shared by a cluster */
PLK_API int plk_batch_set_config(plk_batch b, int32_t cluster, int32_t threads, int32_t smem_qubits,
                                 int32_t cluster_min_qubits);
PLK_API int plk_batch_get_config(plk_batch b, int32_t *cluster, int32_t *threads, int32_t *smem_qubits,
                                 int32_t *cluster_min_qubits);
/* CTAs per SM: 1 (255 registers per thread; complex64 circuits of up to 13
 * qubits in shared memory) or 2 (complex64 only; 128 registers, up to 12) */
PLK_API int plk_batch_set_occupancy(plk_batch b, int32_t ctas_per_sm);
PLK_API int plk_batch_get_occupancy(plk_batch b, int32_t *ctas_per_sm);
PLK_API int plk_batch_set_graph(plk_batch b, int32_t use_graph);
/* autotuner: times a grid of configurations on this batch (median of reps
 * runs each) and keeps the fastest; a text report goes to `report` */
PLK_API int plk_batch_tune(plk_batch b, int32_t reps, char *report, int32_t report_len);

#ifdef __cplusplus
}
#endif

#endif /* PLK_GB300_H */
