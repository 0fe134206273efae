/*
 * qf_oracle.h — CPU oracle for the GB300 state-vector engine.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of QuantumForge's
 * complex128 CPU simulator (the reference crate's `src/lib.rs`,
 * `src/gradients.rs`, `src/analytic.rs`, `src/qaoa_transfer.rs`,
 * `src/mps_qaoa.rs`). The CUDA engine's results are compared with it and it is
 * the timed CPU baseline; nothing in the product links it. Each function cites the
 * reference file:line it follows.
 *
 * Parity pin: the reference (Rust, crates.io dependencies) cannot be built in
 * this environment, so the oracle is pinned by the reference's own
 * known-answer tests (tests/gradients.rs, tests/quantum_core.rs,
 * tests/differential_anchors.rs, tests/proptest_quantum_core.rs,
 * tests/qaoa_transfer.rs, tests/maxcut_families.rs) ported to pytest, plus the
 * published splitmix64 output that `SmallRng::seeded` reproduces.
 *
 * Arithmetic: compiled with -ffp-contract=off so that, like Rust, no multiply
 * and add are fused; complex products are written out exactly as the
 * reference's `impl Mul for Complex64` (src/lib.rs:485-493).
 */
#ifndef QF_ORACLE_H
#define QF_ORACLE_H

#include <stdint.h>
#include "../include/qf.h"

#ifdef __cplusplus
extern "C" {
#endif

/* SmallRng (src/lib.rs:4881-4911). */
uint64_t qfo_rng_seeded(uint64_t seed);
uint64_t qfo_rng_next_u64(uint64_t *state);
double qfo_rng_next_f64(uint64_t *state);

/* Gate::matrix (src/lib.rs:2267-2333): out = m00.re, m00.im, m01..., m11.im */
int qfo_gate_matrix(int gate, double theta, double out[8]);

/* StateVector primitives on interleaved f64 amplitudes of length 2*2^n. */
int qfo_sv_zero(double *amps, uint32_t n);
int qfo_sv_apply(double *amps, uint32_t n, int gate, double theta, uint32_t target, int threads);
int qfo_sv_apply_cnot(double *amps, uint32_t n, uint32_t control, uint32_t target);
int qfo_sv_apply_cz(double *amps, uint32_t n, uint32_t first, uint32_t second);
int qfo_sv_apply_swap(double *amps, uint32_t n, uint32_t first, uint32_t second);
double qfo_sv_norm_sqr(const double *amps, uint32_t n);
void qfo_sv_probabilities(const double *amps, uint32_t n, double *out);
int qfo_sv_expectation(const double *amps, uint32_t n, int observable, uint32_t qubit, double *out);
int qfo_sv_measure(double *amps, uint32_t n, uint32_t qubit, uint64_t *rng_state, uint8_t *outcome);
int qfo_sv_normalize(double *amps, uint32_t n);
/* apply_channel_trajectory: `channel` is enum qf_channel, p the probability /
 * gamma / gamma_down, beta_delta the thermal channel's second parameter. */
int qfo_sv_channel_trajectory(double *amps, uint32_t n, int channel, double p, double beta_delta, uint32_t qubit,
                              uint64_t *rng_state);
int qfo_sv_expectation_pauli_sum(const double *amps, uint32_t n, const qf_pauli_term *terms,
                                 uint64_t n_terms, double out[2]);

/* Circuit::run / ParameterizedCircuit::run_with_shift on amps (in place). */
int qfo_run_ops(double *amps, uint32_t n, const qf_op *ops, uint64_t n_ops,
                const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                int64_t shift_op, double shift_delta, int threads);

/* Circuit::run_shots_impl, literal per-shot re-simulation (src/lib.rs:2842-2916). */
int qfo_run_shots_literal(const double *init_amps, uint32_t n, const qf_op *ops, uint64_t n_ops,
                          uint64_t shots, uint64_t seed, uint64_t *outcomes, uint32_t *width);
/* Circuit::run_shots_with_noise: the same with channel trajectories and the
 * initial state normalised (src/lib.rs:2829-2840, 1356-1506). */
int qfo_run_shots_noisy_literal(const double *init_amps, uint32_t n, const qf_op *ops, uint64_t n_ops,
                                uint64_t shots, uint64_t seed, uint64_t *outcomes, uint32_t *width);
/* Exact memoised form of the same for a unitary prefix followed by measures. */
int qfo_run_shots_tree(const double *init_amps, uint32_t n, const qf_op *ops, uint64_t n_ops,
                       uint64_t shots, uint64_t seed, uint64_t *outcomes, uint32_t *width, int threads);

/* DensityMatrix (src/lib.rs:1551-2235): row-major entries rho[row * 2^n + col],
 * interleaved f64 (2 * 4^n doubles). */
void qfo_dm_from_state(const double *amps, uint32_t n, double *rho);
void qfo_dm_maximally_mixed(uint32_t n, double *rho);
int qfo_dm_apply(double *rho, uint32_t n, int gate, double theta, uint32_t q);
int qfo_dm_apply_2q(double *rho, uint32_t n, int kind, uint32_t a, uint32_t b);  /* kind: QF_OP_CNOT/CZ/SWAP */
int qfo_dm_apply_channel(double *rho, uint32_t n, int channel, double p, double beta_delta, uint32_t q);
void qfo_dm_trace(const double *rho, uint32_t n, double out[2]);
double qfo_dm_purity(const double *rho, uint32_t n);
int qfo_dm_expectation(const double *rho, uint32_t n, int observable, uint32_t q, double *out);
int qfo_dm_probability_one(const double *rho, uint32_t n, uint32_t q, double *out);
int qfo_dm_measure(double *rho, uint32_t n, uint32_t q, uint64_t *rng_state, uint8_t *outcome);
int qfo_run_density(double *rho, uint32_t n, const qf_op *ops, uint64_t n_ops);

/* estimate_observable_shots (src/lib.rs:4806-4838): successes = outcome-0 count. */
int qfo_estimate_observable_shots(const double *amps, uint32_t n, int observable, uint32_t qubit, uint64_t shots,
                                  uint64_t seed, uint64_t *successes);

/* Gradients. `terms` is the observable (one term = SingleQubitObservable). */
int qfo_parameter_shift_gradient(uint32_t n, const qf_op *ops, uint64_t n_ops,
                                 const double *params, uint64_t n_params,
                                 const double *inputs, uint64_t n_inputs,
                                 const qf_pauli_term *terms, uint64_t n_terms, double *grad, int threads);
int qfo_finite_difference_gradient(uint32_t n, const qf_op *ops, uint64_t n_ops,
                                   const double *params, uint64_t n_params,
                                   const double *inputs, uint64_t n_inputs,
                                   const qf_pauli_term *terms, uint64_t n_terms, double step,
                                   double *grad, int threads);
/* The reference adjoint (stores every intermediate state). */
int qfo_adjoint_gradient_stored(uint32_t n, const qf_op *ops, uint64_t n_ops,
                                const double *params, uint64_t n_params,
                                const double *inputs, uint64_t n_inputs,
                                const qf_pauli_term *terms, uint64_t n_terms, double *grad);
/* Same gradient by uncomputing psi instead of storing it (O(2^n) memory). */
int qfo_adjoint_gradient_uncompute(uint32_t n, const qf_op *ops, uint64_t n_ops,
                                   const double *params, uint64_t n_params,
                                   const double *inputs, uint64_t n_inputs,
                                   const qf_pauli_term *terms, uint64_t n_terms,
                                   double *energy, double *grad, int threads);
int qfo_expectation(uint32_t n, const qf_op *ops, uint64_t n_ops,
                    const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                    const qf_pauli_term *terms, uint64_t n_terms, double *energy, int threads);

/* MaxCut helpers (src/qaoa_transfer.rs:199-218, src/mps_qaoa.rs:58-95). */
double qfo_maxcut_expectation(const double *amps, uint32_t n, const uint32_t *edges_uv,
                              const double *weights, uint64_t n_edges);
int qfo_random_3_regular(uint32_t n, uint64_t seed, uint32_t *edges_uv);

#ifdef __cplusplus
}
#endif
#endif
