/*
 * qf.h — C ABI of the GB300 state-vector engine for QuantumForge.
 *
 * This header is the drop-in boundary for QuantumForge's dense state-vector
 * path. Every entry point replaces one method of the reference's Rust API:
 * the CPU `StateVector` / `Circuit` / `ParameterizedCircuit` / `gradients`
 * path in `src/lib.rs` and `src/gradients.rs`, and the optional NVRTC backend
 * `cuda::CudaBackend` / `CudaDeviceState` in `src/cuda.rs`. The comment above
 * each declaration names the reference item it replaces (file:line in the
 * reference crate).
 *
 * Conventions (mirroring the reference):
 *   - Qubit q is bit q of the amplitude index; qubit 0 is the least
 *     significant bit (src/lib.rs:672-679).
 *   - Host amplitudes are interleaved (re, im) pairs of f64, the layout of the
 *     reference's `#[repr(C)] Complex64` (src/lib.rs:437-446).
 *   - Every call returns an `int` status: QF_OK (0) or one of the QF_ERR_*
 *     codes, which mirror the reference's `QuantumError` and `CudaError`
 *     variants (src/lib.rs:507-583, src/cuda.rs:3051-3078). Validation happens
 *     before any launch, as in src/cuda.rs:2256-2285. `qf_last_error()`
 *     returns a thread-local message for the last failing call on the thread.
 *   - Handles are opaque. The caller owns host buffers; the library owns
 *     device memory. A handle is used by one host thread at a time. Each
 *     context owns one CUDA stream; all work of a context is ordered on it.
 *   - Nothing in this header uses torch, C++ or CUDA types.
 */
#ifndef QF_H
#define QF_H

#include <stddef.h>
#include <stdint.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QF_ABI_VERSION 1

/* ---------------------------------------------------------------------------
 * Status codes. Mirror QuantumError (src/lib.rs:507-583) and CudaError
 * (src/cuda.rs:3051-3078).
 * ------------------------------------------------------------------------- */
enum qf_status {
    QF_OK = 0,
    QF_ERR_ZERO_QUBITS = 1,                       /* QuantumError::ZeroQubits */
    QF_ERR_MEMORY_BUDGET_EXCEEDED = 2,            /* QuantumError::MemoryBudgetExceeded */
    QF_ERR_SIMULATION_SIZE_OVERFLOW = 3,          /* QuantumError::SimulationSizeOverflow */
    QF_ERR_MEMORY_ALLOCATION_FAILED = 4,          /* QuantumError::MemoryAllocationFailed */
    QF_ERR_STATE_SIZE_NOT_POWER_OF_TWO = 5,       /* QuantumError::StateSizeNotPowerOfTwo */
    QF_ERR_QUBIT_OUT_OF_RANGE = 6,                /* QuantumError::QubitOutOfRange */
    QF_ERR_INVALID_QUBIT_PAIR = 7,                /* QuantumError::InvalidQubitPair */
    QF_ERR_INVALID_PROBABILITY = 8,               /* QuantumError::InvalidProbability */
    QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX = 9, /* QuantumError::OperationRequiresDensityMatrix */
    QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION = 10,/* QuantumError::OperationRequiresShotExecution */
    QF_ERR_INVALID_SHOT_COUNT = 11,               /* QuantumError::InvalidShotCount */
    QF_ERR_CLASSICAL_BIT_OUT_OF_RANGE = 12,       /* QuantumError::ClassicalBitOutOfRange */
    QF_ERR_INVALID_PARAMETER_COUNT = 13,          /* QuantumError::InvalidParameterCount */
    QF_ERR_INVALID_INPUT_COUNT = 14,              /* QuantumError::InvalidInputCount */
    QF_ERR_NON_FINITE_PARAMETER = 15,             /* QuantumError::NonFiniteParameter, CudaError::NonFiniteAngle */
    QF_ERR_INVALID_FINITE_DIFFERENCE_STEP = 16,   /* QuantumError::InvalidFiniteDifferenceStep */
    QF_ERR_UNSUPPORTED_OPERATION = 17,            /* QuantumError::UnsupportedOperation */
    QF_ERR_TIMEOUT = 18,                          /* QuantumError::Timeout */
    QF_ERR_CUDA = 19,                             /* CudaError::Driver */
    QF_ERR_INVALID_ARGUMENT = 20,                 /* null pointer, bad dtype/enum, length mismatch */
    QF_ERR_EMPTY_BATCH = 21,                      /* CudaError::EmptyBatch */
    QF_ERR_INCOMPATIBLE_BATCH = 22,               /* CudaError::IncompatibleBatch */
    QF_ERR_STATE_TOO_LARGE = 23,                  /* CudaError::StateTooLarge */
    QF_ERR_INCOMPATIBLE_DEVICE_STATE = 24         /* CudaError::IncompatibleDeviceState */
};

/* Gate codes, in the order of `enum Gate` (src/lib.rs:2239-2264). */
enum qf_gate {
    QF_GATE_I = 0, QF_GATE_X = 1, QF_GATE_Y = 2, QF_GATE_Z = 3, QF_GATE_H = 4,
    QF_GATE_S = 5, QF_GATE_SDG = 6, QF_GATE_T = 7, QF_GATE_TDG = 8,
    QF_GATE_RX = 9, QF_GATE_RY = 10, QF_GATE_RZ = 11
};

/* Single-qubit observables, in the order of `enum SingleQubitObservable`
 * (src/lib.rs:2930-2938). Rotation axes reuse X/Y/Z = 0/1/2
 * (`enum RotationAxis`, src/lib.rs:2919-2928). */
enum qf_pauli1 { QF_PAULI_X = 0, QF_PAULI_Y = 1, QF_PAULI_Z = 2 };

/* Operation kinds. One flat record covers both `CircuitOp`
 * (src/lib.rs:2386-2440) and `ParameterizedOp` (src/lib.rs:2942-3006). */
enum qf_op_kind {
    QF_OP_GATE = 0,       /* CircuitOp::SingleQubit / ParameterizedOp::Fixed: gate on q0 (theta for RX/RY/RZ) */
    QF_OP_CNOT = 1,       /* control q0, target q1 */
    QF_OP_CZ = 2,         /* first q0, second q1 */
    QF_OP_SWAP = 3,       /* first q0, second q1 */
    QF_OP_CHANNEL = 4,    /* noise channel `gate` (enum qf_channel) on q0, theta = probability / rate;
                             state-vector calls reject it like the reference; trajectories in
                             qf_run_shots_with_noise */
    QF_OP_MEASURE = 5,    /* measure q0 into classical bit `param` */
    QF_OP_COND = 6,       /* if classical bit `param` == flags&1 apply gate on q0 */
    QF_OP_ROTATION = 7,   /* ParameterizedOp::Rotation: axis in `gate` (QF_PAULI_*), q0, parameter index `param` */
    QF_OP_ENCODING = 8    /* ParameterizedOp::EncodingRotation: axis in `gate`, q0, input index `param` */
};

/* One circuit operation: 24 bytes, no padding ambiguity. */
typedef struct qf_op {
    uint8_t kind;    /* enum qf_op_kind */
    uint8_t gate;    /* enum qf_gate for GATE/COND, enum qf_pauli1 axis for ROTATION/ENCODING */
    uint16_t flags;  /* COND: required classical value (bit 0) */
    uint32_t q0;
    uint32_t q1;
    uint32_t param;  /* parameter / input / classical-bit index */
    double theta;    /* fixed angle of a GATE/COND with RX/RY/RZ */
} qf_op;

/* Noise channels (`enum NoiseChannel`, src/lib.rs:1561-1600), in the `gate`
 * field of a QF_OP_CHANNEL record: Depolarizing { probability = theta },
 * AmplitudeDamping { gamma = theta }, PhaseDamping { gamma = theta },
 * ThermalDamping { gamma_down = theta, beta_delta = qf_op_aux(op) }. */
enum qf_channel {
    QF_CHANNEL_DEPOLARIZING = 0,
    QF_CHANNEL_AMPLITUDE_DAMPING = 1,
    QF_CHANNEL_PHASE_DAMPING = 2,
    QF_CHANNEL_THERMAL_DAMPING = 3
};

/* A channel's second parameter: the double whose bits are
 * ((uint64_t)param << 32) | q1 (both unused by one-qubit channels). */
static inline double qf_op_aux(const qf_op *op) {
    const uint64_t bits = ((uint64_t)op->param << 32) | (uint64_t)op->q1;
    double v;
    memcpy(&v, &bits, sizeof v);
    return v;
}
static inline void qf_op_set_aux(qf_op *op, double v) {
    uint64_t bits;
    memcpy(&bits, &v, sizeof bits);
    op->q1 = (uint32_t)(bits & 0xFFFFFFFFu);
    op->param = (uint32_t)(bits >> 32);
}

/* One Pauli-string term c * P with P = (x-mask, z-mask): bit q set in both
 * masks is Y on qubit q, only in xmask is X, only in zmask is Z. The action
 * on a basis state follows PauliWord::apply_basis_index
 * (src/analytic.rs:2629-2650). */
typedef struct qf_pauli_term {
    uint64_t xmask;
    uint64_t zmask;
    double coeff_re;
    double coeff_im;
} qf_pauli_term;

/* Amplitude storage type on the device. */
enum qf_dtype {
    QF_C64 = 0,   /* complex64: f32 re/im; gate arithmetic in f32, reductions in f64 */
    QF_C128 = 1   /* complex128: f64 re/im, the reference's precision */
};

/* Execution strategy for a gate list. */
enum qf_exec_mode {
    QF_EXEC_AUTO = 0,     /* tile-fused passes with autotuned tile width */
    QF_EXEC_UNFUSED = 1,  /* one HBM sweep per gate (the reference's structure) */
    QF_EXEC_FUSED = 2     /* tile-fused passes with the widths given below */
};

/* qf_exec_opts.flags */
#define QF_EXEC_FLAG_SMEM_TILES 1  /* complex64: use the shared-memory tile kernel instead of register tiles */
#define QF_EXEC_FLAG_JIT 2         /* complex64: compile the plan's passes (NVRTC) even for small states */
#define QF_EXEC_FLAG_NO_JIT 4      /* complex64: never compile passes; interpret them */
#define QF_EXEC_FLAG_SHOTS_TREE 8  /* shots: always walk the branch tree of device states */
#define QF_EXEC_FLAG_SHOTS_TRAJECTORIES 16  /* shots: per-shot trajectories in shared memory whenever the state fits */
#define QF_EXEC_FLAG_PLAN_FIRST_COME 32  /* fused sweeps: fill each pass's tile in gate order (no look-ahead choice of
                                            its resident qubits) */
#define QF_EXEC_FLAG_BLOCKS_SIMT 64      /* block_qubits = 5, complex64: apply the blocks on the FP32 pipe (shared-memory
                                            interpreter) instead of the tensor cores */

typedef struct qf_exec_opts {
    int32_t mode;          /* enum qf_exec_mode */
    int32_t tile_qubits;   /* qubits resident per tile (0 = auto) */
    int32_t block_qubits;  /* dense fused-block width k: 0/1 = apply gates one by one (default); 2..5 = multiply the
                              gates of each tile pass into dense blocks of up to k qubits (f64 on the host) and apply
                              one 2^m x 2^m matrix per block. complex64: compiled register passes for k <= 4, the
                              tensor cores (tcgen05, 3xTF32) for k = 5; complex128: the shared-memory interpreter.
                              Every qubit a gate touches is then resident in the pass's tile. */
    int32_t flags;         /* QF_EXEC_FLAG_* */
} qf_exec_opts;

/* Gradient strategies, in the order of `enum GradientStrategy`
 * (src/gradients.rs:48-73). */
enum qf_gradient_strategy {
    QF_GRAD_PARAMETER_SHIFT = 0,
    QF_GRAD_ADJOINT = 1,
    QF_GRAD_BACKPROP = 2,
    QF_GRAD_FINITE_DIFFERENCE = 3,
    QF_GRAD_AUTO = 4
};

/* `GradientOptions` (src/gradients.rs:144-165) plus engine knobs. */
typedef struct qf_gradient_opts {
    int32_t strategy;              /* enum qf_gradient_strategy */
    int32_t dtype;                 /* enum qf_dtype of the device state */
    double finite_difference_step; /* default 1e-3 in the reference */
    uint64_t shots;                /* >0 makes AUTO select parameter shift */
    int32_t checkpoint_every;      /* adjoint: ops per checkpointed segment. The forward sweep stores
                                      psi at every segment start; the backward sweep restores it there
                                      instead of carrying the uncompute further (0 = pure uncompute). */
    int32_t reserved;
    qf_exec_opts exec;
} qf_gradient_opts;

/* `GradientEstimate` (src/gradients.rs:167-178). */
typedef struct qf_gradient_info {
    int32_t strategy;       /* the rule that ran (AUTO resolved) */
    int32_t reserved;
    uint64_t evaluations;   /* state-vector sweeps in the reference's accounting */
} qf_gradient_info;

typedef struct qf_ctx qf_ctx;  /* CudaBackend: device, stream, workspaces */
typedef struct qf_sv qf_sv;    /* CudaDeviceState: one resident state vector */
typedef struct qf_batch qf_batch;  /* CudaDeviceStateBatch: equal-width states in one allocation */
typedef struct qf_dm qf_dm;        /* CudaDeviceDensityMatrix: one resident density matrix */

/* ---------------------------------------------------------------------------
 * Errors and build information
 * ------------------------------------------------------------------------- */

/* Text of the last error on this thread (Display of QuantumError/CudaError,
 * src/lib.rs:585-664, src/cuda.rs:3079-3104). Never NULL. */
const char *qf_last_error(void);
/* Name of a status code, e.g. "QF_ERR_QUBIT_OUT_OF_RANGE". */
const char *qf_status_name(int status);
/* ABI version this library was built with (QF_ABI_VERSION). */
int qf_abi_version(void);

/* ---------------------------------------------------------------------------
 * Context — replaces CudaBackend::new (src/cuda.rs:556-790).
 * ------------------------------------------------------------------------- */
int qf_ctx_create(int device, qf_ctx **out);
int qf_ctx_destroy(qf_ctx *ctx);
/* CudaDeviceStateBatch::synchronize (src/cuda.rs:1792). */
int qf_ctx_synchronize(qf_ctx *ctx);
/* Raw stream handle (a cudaStream_t) of the context, for callers that order
 * their own work after the engine's. */
int qf_ctx_stream(qf_ctx *ctx, void **stream_out);

/* ---------------------------------------------------------------------------
 * Device state — replaces StateVector (src/lib.rs:928-1351) on the device and
 * CudaDeviceState (src/cuda.rs:521-528, 1285-1484).
 * ------------------------------------------------------------------------- */

/* StateVector::zero_with_memory_budget (src/lib.rs:940-966): |0...0> on
 * `qubits` qubits. `memory_budget_bytes` = 0 means no budget. */
int qf_sv_create(qf_ctx *ctx, uint32_t qubits, int dtype, uint64_t memory_budget_bytes, qf_sv **out);
int qf_sv_destroy(qf_sv *sv);
int qf_sv_qubits(const qf_sv *sv, uint32_t *qubits_out);
int qf_sv_dtype(const qf_sv *sv, int *dtype_out);
/* Raw device pointer to the amplitudes (interleaved, dtype-typed). */
int qf_sv_device_ptr(qf_sv *sv, void **ptr_out);
/* Reset to |0...0>. */
int qf_sv_set_zero(qf_sv *sv);
/* CudaBackend::upload (src/cuda.rs:844-868): host f64 interleaved amplitudes,
 * 2*2^qubits doubles; converted to the state's dtype on the device. */
int qf_sv_upload(qf_sv *sv, const double *amps, uint64_t n_doubles);
/* CudaDeviceState::download (src/cuda.rs:1459-1471): to host f64 interleaved. */
int qf_sv_download(qf_sv *sv, double *amps_out, uint64_t n_doubles);
/* Dtype-native host copies (f32 pairs for C64, f64 pairs for C128);
 * `bytes` must equal the state size. Host memory may be pinned. */
int qf_sv_upload_raw(qf_sv *sv, const void *host, uint64_t bytes);
int qf_sv_download_raw(qf_sv *sv, void *host_out, uint64_t bytes);
/* CudaDeviceStateBatch::copy_from_device (src/cuda.rs:1800-1817). */
int qf_sv_copy_from(qf_sv *dst, const qf_sv *src);

/* StateVector::apply (src/lib.rs:1017-1059), CudaDeviceState::apply_gate
 * (src/cuda.rs:1296-1325). */
int qf_sv_apply_gate(qf_sv *sv, int gate, double theta, uint32_t target);
/* StateVector::apply_cnot / apply_cz / apply_swap (src/lib.rs:1062-1122),
 * CudaDeviceState::apply_cnot/cz/swap (src/cuda.rs:1354-1384). */
int qf_sv_apply_cnot(qf_sv *sv, uint32_t control, uint32_t target);
int qf_sv_apply_cz(qf_sv *sv, uint32_t first, uint32_t second);
int qf_sv_apply_swap(qf_sv *sv, uint32_t first, uint32_t second);

/* Circuit::run (src/lib.rs:2786-2802) on a resident state, and
 * ParameterizedCircuit::run_with_inputs (src/lib.rs:3097-3106) when the list
 * holds ROTATION/ENCODING ops. `params`/`inputs` may be NULL when their
 * counts are 0. `opts` may be NULL (AUTO). MEASURE/COND are rejected with
 * QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION, CHANNEL with
 * QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX, as in the reference. */
int qf_sv_apply_ops(qf_sv *sv, const qf_op *ops, uint64_t n_ops,
                    const double *params, uint64_t n_params,
                    const double *inputs, uint64_t n_inputs,
                    const qf_exec_opts *opts);

/* StateVector::norm_sqr (src/lib.rs:998-1000), f64 accumulation. */
int qf_sv_norm_sqr(qf_sv *sv, double *out);
/* StateVector::probabilities (src/lib.rs:1144-1146): 2^qubits doubles to host. */
int qf_sv_probabilities(qf_sv *sv, double *out, uint64_t n_out);
/* StateVector::expectation_z (src/lib.rs:1149-1166) for every qubit in one
 * HBM pass: out[q] = <Z_q>, `n_out` == qubits. */
int qf_sv_expectation_z_all(qf_sv *sv, double *out, uint64_t n_out);
/* StateVector::expectation (src/lib.rs:1304-1318) for X/Y/Z on one qubit. */
int qf_sv_expectation(qf_sv *sv, int observable, uint32_t qubit, double *out);
/* <psi|H|psi> for H = sum_t c_t P_t (PauliSum::expectation_ket,
 * src/analytic.rs:2775). out[0] = Re, out[1] = Im. */
int qf_sv_expectation_pauli_sum(qf_sv *sv, const qf_pauli_term *terms, uint64_t n_terms, double *out);
/* StateVector::measure (src/lib.rs:1321-1351), CudaDeviceState::measure
 * (src/cuda.rs:1386-1457): draws one uniform from the SmallRng whose state is
 * *rng_state, collapses the state and returns the bit. */
int qf_sv_measure(qf_sv *sv, uint32_t qubit, uint64_t *rng_state, uint8_t *outcome);
/* StateVector::normalize (src/lib.rs:1005-1014): divide by sqrt(norm_sqr);
 * QF_ERR_INVALID_PROBABILITY for a zero or non-finite norm. */
int qf_sv_normalize(qf_sv *sv);
/* StateVector::apply_channel_trajectory (src/lib.rs:1356-1506) on a resident
 * state: `channel` is a QF_OP_CHANNEL record; one uniform is drawn from
 * *rng_state (advanced) and the selected Kraus branch applied and
 * renormalised. *branch_out (nullable): the branch taken (depolarizing: 0
 * none, 1 X, 2 Y, 3 Z; damping: 1 jump, 0 none; thermal: 1 down, 2 up, 0 stay). */
int qf_sv_apply_channel_trajectory(qf_sv *sv, const qf_op *channel, uint64_t *rng_state, int *branch_out);

/* ---------------------------------------------------------------------------
 * Whole-circuit calls with host buffers.
 * ------------------------------------------------------------------------- */

/* CudaBackend::run_circuit (src/cuda.rs:1050-1083): upload `init_amps`
 * (NULL = |0...0>), run, download into `out_amps` (NULL = no download). */
int qf_run_circuit(qf_ctx *ctx, uint32_t qubits, int dtype,
                   const qf_op *ops, uint64_t n_ops,
                   const double *init_amps, double *out_amps, uint64_t n_doubles,
                   const qf_exec_opts *opts);

/* Circuit::run_shots (src/lib.rs:2822-2916) with the reference's shot-major
 * SmallRng stream (one draw per Measure). Circuits whose measurements all
 * follow the last gate (the CLI `shots` form, src/bin/main.rs:574-602) are
 * sampled from the one pre-measurement state; mid-circuit measurements,
 * repeated measurements and ConditionalSingleQubit feed-forward (QF_OP_COND)
 * run as a tree of measurement branches, one device state per branch reached.
 * `outcomes` receives one packed classical register per shot (bit c =
 * classical bit c, width <= 64); NULL skips it. `n_ties` counts decisions with
 * |u - p_one| < tie_eps (outcomes that rounding could flip). Channels return
 * QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX as the reference's noiseless
 * run_shots does. */
int qf_run_shots(qf_ctx *ctx, uint32_t qubits, int dtype,
                 const qf_op *ops, uint64_t n_ops, const double *init_amps,
                 uint64_t shots, uint64_t seed, double tie_eps,
                 uint64_t *outcomes, uint32_t *classical_width, uint64_t *n_ties,
                 const qf_exec_opts *opts);

/* Circuit::run_shots_with_noise (src/lib.rs:2829-2840): run_shots with
 * channel trajectories (apply_channel_trajectory, src/lib.rs:1356-1506, one
 * draw per channel from the shot's stream) and the initial state normalized.
 * Same arguments and results as qf_run_shots. */
int qf_run_shots_with_noise(qf_ctx *ctx, uint32_t qubits, int dtype,
                             const qf_op *ops, uint64_t n_ops, const double *init_amps,
                             uint64_t shots, uint64_t seed, double tie_eps,
                             uint64_t *outcomes, uint32_t *classical_width, uint64_t *n_ties,
                             const qf_exec_opts *opts);

/* Sampling on a resident state: measure `qubit_order[j]` into classical bit
 * `classical_bits[j]` for j < m, for `shots` shots of the stream seeded by
 * `seed`. Same semantics and outputs as qf_run_shots. */
int qf_sv_sample(qf_sv *sv, const uint32_t *qubit_order, const uint32_t *classical_bits, uint32_t m,
                 uint64_t shots, uint64_t seed, double tie_eps,
                 uint64_t *outcomes, uint64_t *n_ties);

/* ---------------------------------------------------------------------------
 * State batches — replace CudaDeviceStateBatch (src/cuda.rs:529-540,
 * 1486-1992) and CudaBackend::upload_batch / run_circuit_batch
 * (src/cuda.rs:871-967). State b of a batch occupies amplitudes
 * [b * 2^qubits, (b + 1) * 2^qubits) of one device allocation; host buffers
 * hold the states back to back, f64 interleaved.
 * ------------------------------------------------------------------------- */

/* `batch_size` states |0...0> (0 -> QF_ERR_EMPTY_BATCH). */
int qf_batch_create(qf_ctx *ctx, uint32_t qubits, int dtype, uint64_t batch_size, qf_batch **out);
int qf_batch_destroy(qf_batch *batch);
int qf_batch_qubits(const qf_batch *batch, uint32_t *qubits_out);
int qf_batch_size(const qf_batch *batch, uint64_t *size_out);
/* upload_batch (src/cuda.rs:871-955): 2 * batch_size * 2^qubits doubles. */
int qf_batch_upload(qf_batch *batch, const double *amps, uint64_t n_doubles);
/* CudaDeviceStateBatch::download (src/cuda.rs:1973-1991). */
int qf_batch_download(qf_batch *batch, double *amps_out, uint64_t n_doubles);
/* CudaDeviceStateBatch::copy_from_device (src/cuda.rs:1797-1817). */
int qf_batch_copy_from(qf_batch *dst, const qf_batch *src);
/* CudaDeviceStateBatch::run_circuit / apply_gate / apply_cnot / apply_cz /
 * apply_swap (src/cuda.rs:1821-1969): the same unitary ops on every state;
 * channels -> QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX, measurements and
 * conditionals -> QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION. */
int qf_batch_apply_ops(qf_batch *batch, const qf_op *ops, uint64_t n_ops, const qf_exec_opts *opts);
/* CudaDeviceStateBatch::measure (src/cuda.rs:1497-1623): one uniform per
 * state in batch order from *rng_state (advanced), P(1) per state, outcome
 * u < P(1), kept amplitudes multiplied by 1/sqrt(P(outcome)); outcomes[b]
 * is 0 or 1. */
int qf_batch_measure(qf_batch *batch, uint32_t qubit, uint64_t *rng_state, uint8_t *outcomes);
/* CudaBackend::run_circuit_batch (src/cuda.rs:958-967): upload `batch_size`
 * states from `in_amps`, run the ops on each, download to `out_amps` (both
 * 2 * batch_size * 2^qubits doubles). */
int qf_run_circuit_batch(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                         const double *in_amps, uint64_t batch_size, double *out_amps, uint64_t n_doubles,
                         const qf_exec_opts *opts);

/* ---------------------------------------------------------------------------
 * Density matrices — replace DensityMatrix (src/lib.rs:1551-2235),
 * Circuit::run_density (src/lib.rs:2804-2818) and the CUDA density path
 * (CudaBackend::upload_density / run_density_circuit, CudaDeviceDensityMatrix,
 * src/cuda.rs:969-1045, 2007-2237). Entries are row-major rho[row * 2^n + col],
 * f64 interleaved on the host (2 * 4^qubits doubles).
 * ------------------------------------------------------------------------- */

/* |0...0><0...0| on `qubits` qubits (1..17; the entries take 16 * 4^qubits
 * bytes in complex128). */
int qf_dm_create(qf_ctx *ctx, uint32_t qubits, int dtype, qf_dm **out);
int qf_dm_destroy(qf_dm *dm);
int qf_dm_qubits(const qf_dm *dm, uint32_t *qubits_out);
/* upload_density (src/cuda.rs:969-1021) / CudaDeviceDensityMatrix::download. */
int qf_dm_upload(qf_dm *dm, const double *entries, uint64_t n_doubles);
int qf_dm_download(qf_dm *dm, double *entries_out, uint64_t n_doubles);
/* DensityMatrix::from_state (src/lib.rs:1641-1655) from a resident state of
 * the same width and dtype; maximally_mixed (src/lib.rs:1658-1700). */
int qf_dm_from_state(qf_dm *dm, const qf_sv *psi);
int qf_dm_set_maximally_mixed(qf_dm *dm);
/* Circuit::run_density (src/lib.rs:2804-2818) on the resident matrix: gates
 * (apply, src/lib.rs:2043-2054; apply_cnot/cz/swap :1983-2031) and channels
 * (apply_channel, :2056-2143); measurements and conditionals ->
 * QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION. The whole list is validated
 * before anything runs. */
int qf_dm_apply_ops(qf_dm *dm, const qf_op *ops, uint64_t n_ops, const qf_exec_opts *opts);
/* trace (src/lib.rs:1732-1736, out[0] re, out[1] im), purity (:1738-1741),
 * expectation / expectation_z (:1858-1904, observable = enum qf_pauli1),
 * probability_one (:1906-1920), diagonal probabilities (2^qubits values). */
int qf_dm_trace(qf_dm *dm, double out[2]);
int qf_dm_purity(qf_dm *dm, double *out);
int qf_dm_expectation(qf_dm *dm, int observable, uint32_t qubit, double *out);
int qf_dm_probability_one(qf_dm *dm, uint32_t qubit, double *out);
int qf_dm_probabilities(qf_dm *dm, double *out, uint64_t n_out);
/* DensityMatrix::measure (src/lib.rs:1922-1947), CudaDeviceDensityMatrix::measure. */
int qf_dm_measure(qf_dm *dm, uint32_t qubit, uint64_t *rng_state, uint8_t *outcome);
/* ParameterizedCircuit::expectation_density_with_inputs (src/lib.rs:3175-3186):
 * the parameterised op list (rotations, encodings, fixed gates, channels)
 * from |0...0><0...0| through the density matrix, then <P_q> for the
 * observable P = enum qf_pauli1 on `observable_qubit`. */
int qf_expectation_density(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                           const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                           int observable, uint32_t observable_qubit, const qf_exec_opts *opts, double *expectation);
/* parameter_shift_gradient_density_with_inputs (src/lib.rs:3235-3266): two
 * shifted density runs per rotation occurrence; `expectation` (nullable)
 * receives the unshifted value. */
int qf_parameter_shift_gradient_density(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                                        const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                                        int observable, uint32_t observable_qubit, const qf_exec_opts *opts,
                                        double *expectation, double *gradient);
/* CudaBackend::run_density_circuit (src/cuda.rs:1022-1045): upload, run, download. */
int qf_run_density_circuit(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                           const double *in_entries, double *out_entries, uint64_t n_doubles,
                           const qf_exec_opts *opts);

/* Finite-shot estimates (estimate_observable_shots, src/lib.rs:4806-4838):
 * the parameterised state prepared, the measured basis rotated, `shots`
 * single-qubit measurements of SmallRng::seeded(seed); *estimate = 2 p0 - 1
 * with p0 the outcome-0 fraction (*successes). Draws within tie_eps of P(1)
 * are counted in *n_ties.
 * ParameterizedCircuit::expectation_with_inputs_shots (src/lib.rs:3361-3382). */
int qf_expectation_shots(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                         const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                         int observable, uint32_t observable_qubit, uint64_t shots, uint64_t seed, double tie_eps,
                         const qf_exec_opts *opts, double *estimate, uint64_t *successes, uint64_t *n_ties);
/* parameter_shift_gradient_with_inputs_shots (src/lib.rs:3428-3479). */
int qf_parameter_shift_gradient_shots(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                                      const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                                      int observable, uint32_t observable_qubit, uint64_t shots, uint64_t seed,
                                      double tie_eps, const qf_exec_opts *opts, double *gradient, uint64_t *n_ties);

/* sample_expectation (src/lib.rs:4840-4850): `shots` Bernoulli draws of
 * SmallRng::seeded(seed) at P(+1) = clamp((1 + expectation) / 2, 0, 1);
 * *estimate = 2 (#positive) / shots - 1. Host arithmetic only; the density
 * shot estimates (src/lib.rs:3188-3320) apply it to the exact density-matrix
 * expectation. */
int qf_sample_expectation(double expectation, uint64_t shots, uint64_t seed, double *estimate, uint64_t *positive);
/* parameter_shift_gradient_density_with_inputs_shots (src/lib.rs:3268-3320):
 * every rotation occurrence k shifted by +-pi/2 on the density matrix, each
 * exact expectation passed through qf_sample_expectation with seeds
 * seed + 2k and seed + 2k + 1. */
int qf_parameter_shift_gradient_density_shots(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                                              const double *params, uint64_t n_params, const double *inputs,
                                              uint64_t n_inputs, int observable, uint32_t observable_qubit,
                                              uint64_t shots, uint64_t seed, const qf_exec_opts *opts, double *gradient);

/* ---------------------------------------------------------------------------
 * Circuit formats — OpenQASM 2.0 import (qasm::parse_qasm, src/qasm.rs:73),
 * QASM export (qasm_export::export_qasm / export_qasm_with_qubits,
 * src/qasm_export.rs), and the JSON form (Circuit::to_json / from_json,
 * src/serialize.rs:91-170). Ops come back as the qf_op records of the
 * circuit; pass ops_out = NULL to learn the count (*n_ops), text out = NULL
 * to learn the length (*len, without the terminating NUL). Parse errors are
 * QF_ERR_INVALID_ARGUMENT with the reference's message in qf_last_error
 * ("QASM error at line N: ..."; *error_line = N).
 * ------------------------------------------------------------------------- */
int qf_parse_qasm(const char *source, uint64_t len, qf_op *ops_out, uint64_t capacity, uint64_t *n_ops,
                  uint32_t *qubits, uint32_t *classical_bits, uint64_t *error_line);
int qf_circuit_from_json(const char *json, uint64_t len, qf_op *ops_out, uint64_t capacity, uint64_t *n_ops,
                         uint32_t *qubits, uint32_t *classical_bits);
int qf_circuit_to_json(const qf_op *ops, uint64_t n_ops, char *out, uint64_t capacity, uint64_t *len);
/* `qubits` < 0: the register spans the highest qubit used (export_qasm);
 * otherwise the declared register size (export_qasm_with_qubits, an error
 * when an op uses a qubit outside it). */
int qf_circuit_to_qasm(const qf_op *ops, uint64_t n_ops, int64_t qubits, char *out, uint64_t capacity, uint64_t *len);

/* ---------------------------------------------------------------------------
 * Gradients — ParameterizedCircuit::gradient_with_inputs
 * (src/gradients.rs:232-330), adjoint_gradient_with_inputs
 * (src/lib.rs:3564-3704), parameter_shift_gradient_with_inputs
 * (src/lib.rs:3516-3546), finite_difference_gradient_with_inputs
 * (src/gradients.rs:344-375), backprop_gradient_with_inputs
 * (src/gradients.rs:392-506).
 *
 * The observable is a Pauli sum; the reference's SingleQubitObservable is the
 * one-term case. `expectation` receives <H> (may be NULL), `gradient`
 * receives n_params values, `info` may be NULL.
 * ------------------------------------------------------------------------- */
int qf_gradient(qf_ctx *ctx, uint32_t qubits,
                const qf_op *ops, uint64_t n_ops,
                const double *params, uint64_t n_params,
                const double *inputs, uint64_t n_inputs,
                const qf_pauli_term *terms, uint64_t n_terms,
                const qf_gradient_opts *opts,
                double *expectation, double *gradient, qf_gradient_info *info);

/* <H> of the circuit's output state: ParameterizedCircuit::run_with_inputs
 * followed by the expectation (src/lib.rs:3097-3106, 3197-3226). */
int qf_expectation(qf_ctx *ctx, uint32_t qubits, int dtype,
                   const qf_op *ops, uint64_t n_ops,
                   const double *params, uint64_t n_params,
                   const double *inputs, uint64_t n_inputs,
                   const qf_pauli_term *terms, uint64_t n_terms,
                   const qf_exec_opts *opts, double *expectation);

/* ---------------------------------------------------------------------------
 * Batched QAOA MaxCut — replaces calling maxcut_qaoa_expectation
 * (src/qaoa_transfer.rs:221-236) per instance, and its central
 * finite-difference gradient (the `adagrad` optimiser, same file), for a batch
 * of instances of uneven qubit counts: one persistent launch computes every
 * instance's cost <C> (maxcut_expectation, src/qaoa_transfer.rs:199-218) and
 * its exact adjoint gradient for the circuit algorithms::qaoa_maxcut
 * (src/algorithms.rs:110-137) with unit edge weights. complex64 states,
 * f64 accumulation.
 * ------------------------------------------------------------------------- */
typedef struct qf_qaoa_instance {
    uint32_t qubits;       /* 2..30 */
    uint32_t edge_begin;   /* first (u, v) pair in edges_uv */
    uint32_t edge_count;   /* at most 96 */
    uint32_t tile_qubits;  /* 0 = from qf_qaoa_opts.tile_qubits[qubits] (autotuned) */
} qf_qaoa_instance;

typedef struct qf_qaoa_opts {
    int32_t use_graph;         /* capture the launch in a CUDA graph once per batch layout, then replay */
    int32_t tile_qubits[33];   /* per qubit count: up to 12 qubits the tile width of the one-CTA-per-instance
                                  kernel (0 = 10); above 12 qubits 0 = batched tile passes over every instance
                                  of that count (the default), 4..12 = one CTA per instance with tiles of that
                                  width instead */
} qf_qaoa_opts;

/* gammas/betas: n_inst x p (row = instance). cost_out: n_inst values;
 * grad_out: n_inst x 2p rows [dC/dγ_0..dC/dγ_{p-1}, dC/dβ_0..dC/dβ_{p-1}]. */
int qf_qaoa_maxcut_batch(qf_ctx *ctx, const qf_qaoa_instance *inst, uint64_t n_inst,
                         const uint32_t *edges_uv, uint64_t n_edges, uint32_t p,
                         const double *gammas, const double *betas,
                         double *cost_out, double *grad_out, const qf_qaoa_opts *opts);

/* ---------------------------------------------------------------------------
 * Plan inspection (host only, no device needed): the pass schedule the fused
 * executor would use for a gate list. `n_passes` = HBM sweeps of the state,
 * `n_gates` = gates after parameter binding. Used by tests and the autotuner.
 * ------------------------------------------------------------------------- */
int qf_plan_stats(uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                  const double *params, uint64_t n_params,
                  const double *inputs, uint64_t n_inputs,
                  const qf_exec_opts *opts, uint64_t *n_passes, uint64_t *n_gates);

/* What one adjoint gradient (qf_gradient with QF_GRAD_ADJOINT and these
 * options) launches, and its algorithmic HBM bytes: |0> written, forward
 * passes (read + write psi), the Pauli passes of lambda = H psi, backward
 * passes (psi and lambda read and written), checkpoint copies. Host only, no
 * GPU needed; the measurement helper behind the gradient's roofline fraction
 * (the reference's adjoint_gradient_with_inputs, src/lib.rs:3564-3704, stores
 * every intermediate state instead). */
typedef struct qf_adjoint_stats {
    uint64_t forward_passes;
    uint64_t backward_passes;
    uint64_t pauli_passes;
    uint64_t state_copies;
    double hbm_bytes;
} qf_adjoint_stats;
int qf_adjoint_plan_stats(uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                          const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                          const qf_pauli_term *terms, uint64_t n_terms, const qf_gradient_opts *opts,
                          qf_adjoint_stats *out);

/* SmallRng::next_u64 (src/lib.rs:4898-4905) advanced `steps` times, computed
 * by GF(2) matrix powers: the generator state from which the shot-major
 * stream of run_shots_impl (src/lib.rs:2874-2912) draws its `steps`-th value.
 * Host only; `state` is a SmallRng state (after SmallRng::seeded). */
uint64_t qf_rng_jump(uint64_t state, uint64_t steps);

/* ---------------------------------------------------------------------------
 * Allocation-free reduction. This entry point has no counterpart in the
 * reference; it serves callers that cannot let a library allocate device
 * memory: a host framework whose device memory all comes from its own pool
 * allocator, or a latency-bound loop where cudaMalloc/cudaFree (which
 * synchronise the device) are not acceptable.
 *
 * out[q] = <Z_q> for every qubit of the state at `d_amps` (caller-owned device
 * memory on `device`: 2^qubits complex64 or complex128 amplitudes,
 * interleaved, 8- or 16-byte aligned), the same values as
 * qf_sv_expectation_z_all. The library calls no cudaMalloc, cudaFree or other
 * allocating routine: its only scratch is a fixed array in the library's
 * device image (about 84 KB, held on every GPU that loads the library until
 * the process exits), which limits `qubits` to 1..40 (QF_ERR_STATE_TOO_LARGE
 * beyond). `stream` is a cudaStream_t of `device` (NULL = the legacy default
 * stream; a stream of another device is QF_ERR_INVALID_ARGUMENT); the call
 * returns after the result is on the host, with the calling thread's current
 * device as it was before the call. The first call on a device looks up the
 * scratch array's device address, so make it before any stream capture; the
 * address is kept for the life of the process, so do not call this entry
 * point again after destroying the device's primary context
 * (cudaDeviceReset). Every call reuses the same scratch, so calls that
 * overlap on the GPU race: serialise them.
 * ------------------------------------------------------------------------- */
int qf_expectation_z_all_noalloc(int device, const void *d_amps, uint32_t qubits, int dtype, void *stream,
                                 double *out, uint64_t n_out);

#ifdef __cplusplus
}
#endif
#endif /* QF_H */
