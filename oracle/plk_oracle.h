/*
 * plk_oracle.h — CPU oracle for the LightningKokkos state-vector hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain-C restatement of the
 * reference's Kokkos functors (pennylane_lightning_kokkos/src/simulator/
 * GateFunctors.hpp, ExpValFunctors.hpp, MeasuresFunctors.hpp,
 * MeasuresKokkos.hpp, src/util/LinearAlgebraKokkos.hpp and
 * src/algorithms/AdjointDiffKokkos.hpp).  It is the checker the GPU path is
 * compared against, and the timed CPU baseline; nothing in the product links
 * it or falls back to it.
 *
 * Conventions (same as the reference):
 *   - the state is complex<double>[2^nq], C order, wire 0 is the most
 *     significant bit of the amplitude index (rev_wire = nq - wire - 1);
 *   - gates are selected by their PennyLane name;
 *   - "inverse" selects the adjoint gate exactly as the functor's
 *     `bool inverse` template parameter does.
 */
#ifndef PLK_ORACLE_H
#define PLK_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double re;
    double im;
} orc_cplx;

/* Status codes. */
#define ORC_OK 0
#define ORC_UNKNOWN_GATE (-1)
#define ORC_BAD_ARGS (-2)

/* Number of OpenMP threads the oracle uses (0 = runtime default). */
void orc_set_num_threads(int n);
int orc_get_num_threads(void);

/* Named gate application (StateVectorKokkos::applyOperation). */
int orc_apply(orc_cplx *sv, int nq, const char *name, const int64_t *wires,
              int nw, int inverse, const double *params, int np);

/* Dense matrix application, row-major 2^k x 2^k (applyMultiQubitOp).
 * k = 1, 2 follow singleQubitOpFunctor / twoQubitOpFunctor; k >= 3 applies
 * the matrix on the requested wires (wires[0] = most significant bit of the
 * matrix index). */
int orc_apply_matrix(orc_cplx *sv, int nq, const orc_cplx *mat,
                     const int64_t *wires, int nw, int inverse);

/* The reference multiQubitOpFunctor's own index map (sequential bit swaps,
 * GateFunctors.hpp:232-252), kept to document where it departs from the
 * documented semantics. */
int orc_apply_matrix_refmap(orc_cplx *sv, int nq, const orc_cplx *mat,
                            const int64_t *wires, int nw, int inverse);

/* Generator application (StateVectorKokkos::applyGenerator); returns the
 * scale factor, *status receives ORC_OK or an error. */
double orc_apply_generator(orc_cplx *sv, int nq, const char *name,
                           const int64_t *wires, int nw, int adj, int *status);

/* Expectation values (MeasuresKokkos::getExpectationValue*). */
double orc_expval_named(const orc_cplx *sv, int nq, const char *name,
                        const int64_t *wires, int nw, int *status);
double orc_expval_matrix(const orc_cplx *sv, int nq, const orc_cplx *mat,
                         const int64_t *wires, int nw, int *status);
double orc_expval_sparse(const orc_cplx *sv, int64_t nrows,
                         const orc_cplx *data, const int64_t *indices,
                         const int64_t *indptr);

/* Linear algebra (LinearAlgebraKokkos.hpp). */
void orc_axpy(orc_cplx alpha, const orc_cplx *x, orc_cplx *y, size_t n);
void orc_spmv(const orc_cplx *x, orc_cplx *y, int64_t nrows,
              const orc_cplx *data, const int64_t *indices,
              const int64_t *indptr);
double orc_inner_re(const orc_cplx *x, const orc_cplx *y, size_t n);
double orc_inner_im(const orc_cplx *x, const orc_cplx *y, size_t n);

/* Measurements (MeasuresKokkos::probs / generate_samples). */
void orc_probs(const orc_cplx *sv, int nq, double *out);
int orc_probs_wires(const orc_cplx *sv, int nq, const int64_t *wires, int nw,
                    double *out);
void orc_cdf_exclusive(const double *probs, size_t n, double *cdf);
void orc_sample_from_uniforms(const double *cdf, size_t n, int nq,
                              const double *uniforms, size_t shots,
                              int64_t *out_bits);

/* Adjoint Jacobian backward sweep (AdjointJacobianKokkos::adjointJacobian
 * with apply_operations = false).  `lambda_state` is the forward-evolved
 * state (copied, not modified); `hlambda` holds nobs states O_i|lambda>
 * (modified in place).  Operations are flattened: op i has name names[i],
 * wires wires[wire_off[i] .. wire_off[i+1]), params
 * params[param_off[i] .. param_off[i+1]) and inverse flag inverses[i].
 * jac is [nobs][ntp], row-major. */
int orc_adjoint_jacobian(const orc_cplx *lambda_state, int nq,
                         orc_cplx *const *hlambda, int nobs, int nops,
                         const char *const *names, const int64_t *wires,
                         const int64_t *wire_off, const double *params,
                         const int64_t *param_off, const int32_t *inverses,
                         const int64_t *trainable, int ntp, double *jac);

#ifdef __cplusplus
}
#endif

#endif /* PLK_ORACLE_H */
