// qf_internal.h — internal declarations shared by the engine's translation
// units. Nothing here crosses the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <set>
#include <string>
#include <vector>

#include "../../include/qf.h"

struct qf_ctx {
    int device = 0;
    int sm_count = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    // Growable device workspaces owned by the context.
    void *ws_plan = nullptr;      size_t ws_plan_bytes = 0;      // pass descriptors + matrices
    void *ws_red = nullptr;       size_t ws_red_bytes = 0;       // reduction partials
    void *ws_tree = nullptr;      size_t ws_tree_bytes = 0;      // sampler marginal tree
    void *host_pinned = nullptr;  size_t host_pinned_bytes = 0;  // small pinned staging
    void *ws_stage = nullptr;     size_t ws_stage_bytes = 0;     // f64 <-> dtype conversion staging
    double *d_small = nullptr;    // 64 KiB device result area
    double *h_small = nullptr;    // 64 KiB pinned host mirror
    qf_sv *scratch_sv = nullptr;  // cached state for whole-circuit calls
    qf_sv *scratch_sv2 = nullptr; // cached second state (adjoint costate)
    std::set<qf_sv *> states;     // live states; orphaned (memory freed) when the context is destroyed
    std::vector<qf_sv *> ckpt_pool;  // adjoint checkpoint states kept for the next gradient (bounded bytes)
};
constexpr size_t kSmallBytes = 64 * 1024;

struct qf_sv {
    qf_ctx *ctx = nullptr;
    uint32_t n = 0;
    int dtype = QF_C64;
    uint64_t dim = 0;
    void *d = nullptr;  // 2^n complex amplitudes, interleaved
    size_t bytes() const { return dim * (dtype == QF_C64 ? 8u : 16u); }
};

// A batch of `size` states of `n` qubits: one state of n + ceil(log2 size)
// qubits whose top bits index the state (padding states stay zero), so the
// fused engine sweeps every state of the batch in the same passes.
struct qf_batch {
    qf_sv *sv = nullptr;
    uint32_t n = 0;
    uint64_t size = 0;
};

// A density matrix of n qubits: row-major rho[row * 2^n + col] held as one
// 2n-qubit vector (column qubit q = bit q, row qubit q = bit n + q).
struct qf_dm {
    qf_sv *sv = nullptr;
    uint32_t n = 0;
};

namespace qf {

// ---- errors -----------------------------------------------------------------
int fail(int status, const char *fmt, ...);
void clear_error();
int cuda_fail(cudaError_t e, const char *what);
#define QF_CUDA(expr)                                              \
    do {                                                           \
        cudaError_t qf_e_ = (expr);                                \
        if (qf_e_ != cudaSuccess) return qf::cuda_fail(qf_e_, #expr); \
    } while (0)
#define QF_TRY(expr)                 \
    do {                             \
        int qf_s_ = (expr);          \
        if (qf_s_ != QF_OK) return qf_s_; \
    } while (0)

// Opt a kernel into the largest dynamic shared memory the device allows
// (the opt-in limit minus the kernel's static shared memory); returns that
// dynamic limit in *dyn_limit.
template <typename F> int allow_max_dynamic_smem(F *func, const qf_ctx *ctx, size_t *dyn_limit) {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, func);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes");
    const size_t dyn = ctx->smem_optin > fa.sharedSizeBytes ? ctx->smem_optin - fa.sharedSizeBytes : 0;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(MaxDynamicSharedMemorySize)");
    *dyn_limit = dyn;
    return 0;
}

// Grow-only device workspace.
int ensure_device(void **ptr, size_t *bytes, size_t need);
int ensure_pinned(void **ptr, size_t *bytes, size_t need);

// ---- bound gates ------------------------------------------------------------
// A gate list with parameters resolved to matrices (host, f64).
// BK_OVL marks an adjoint overlap Im<lambda|P_q0 psi> in a backward pass:
// P = X/Y/Z from `axis`, op_index = the overlap slot.
// BK_BLOCK is a dense 2^nq x 2^nq block on qubits bq[0..nq-1] (ascending; bit
// i of the block's local index is qubit bq[i]) made by k-qubit fusion; its
// matrix is row-major complex at Plan::bmats[2 * boff ...].
enum BKind : uint8_t { BK_MAT1 = 0, BK_CNOT = 1, BK_CZ = 2, BK_SWAP = 3, BK_OVL = 4, BK_BLOCK = 5 };
constexpr int kMaxBlockQubits = 5;

struct BGate {
    uint8_t kind = BK_MAT1;
    uint8_t diag = 0;        // MAT1 only: m01 == m10 == 0
    uint8_t axis = 255;      // rotation occurrence: generator axis (QF_PAULI_*), else 255
    uint8_t varying = 0;     // matrix from a circuit parameter or an encoded input (changes between calls)
    uint32_t q0 = 0, q1 = 0;
    int64_t op_index = -1;   // index into the caller's op list
    int64_t param = -1;      // parameter index of a rotation occurrence
    double m[8] = {0};       // m00, m01, m10, m11 as (re, im)
    uint8_t nq = 0;          // BK_BLOCK: qubits of the block
    uint8_t bq[kMaxBlockQubits] = {0};
    uint32_t boff = 0;       // BK_BLOCK: complex offset of the matrix in Plan::bmats
};

// Gate::matrix (src/lib.rs:2267-2333) evaluated on the host in f64.
int gate_matrix(int gate, double theta, double m[8]);
bool matrix_is_diag(const double m[8]);
bool matrix_is_cheap(const double m[8]);

// Validate an op list for state-vector execution and bind it.
// `shift_op`/`shift` add `shift` to the angle of op `shift_op` (parameter shift).
int bind_ops(uint32_t n, const qf_op *ops, uint64_t n_ops, const double *params, uint64_t n_params,
             const double *inputs, uint64_t n_inputs, int64_t shift_op, double shift,
             std::vector<BGate> &out);
// The inverse of a bound gate (U^dagger).
BGate inverse_gate(const BGate &g);

// A unitary 2x2 whose entries are real (kind 1) or real on the diagonal and
// imaginary off it (kind 2) has |m00| = |m11| and |m01| = |m10|. Pulling the
// larger of m00, m01 (g) out of the gate leaves one unit coefficient per
// output: out0 = g (p0 + r0 q0), out1 = g (sigma p1 + r1 q1) with sigma = +-1
// and |r| <= 1 — half the multiplies of the plain form. ok = false for other
// matrices (general complex, non-unitary Kraus operators).
struct Factored {
    bool ok = false;
    int pivot = 0;        // 0: output 0 pivots on x (|m00| >= |m01|); 1: on y
    bool neg = false;     // sigma = -1
    bool imag_r = false;  // r0, r1 purely imaginary (kind 2), else real
    bool imag_g = false;  // g purely imaginary (kind 2 with pivot 1)
    std::complex<double> g, r0, r1;
};
Factored factor_unitary_2x2(const double m[8]);

// ---- tile-pass plans --------------------------------------------------------
enum TKind : uint8_t {
    T_MAT1 = 0,     // dense 2x2 on local bit b0
    T_DIAG1 = 1,    // diag(m00, m11) on local bit b0
    T_GPHASE = 2,   // diag(m00, m11) on non-local qubit g0: scalar per tile
    T_CNOT_LL = 3,  // control local b0, target local b1
    T_CNOT_GL = 4,  // control non-local g0, target local b1
    T_CZ_LL = 5,    // both local
    T_CZ_GL = 6,    // g0 non-local, b1 local
    T_CZ_GG = 7,    // both non-local
    T_SWAP_LL = 8,  // both local
    T_OVL_X = 9,    // adjoint overlap Im<lambda|X_b0 psi>, slot
    T_OVL_Y = 10,   // adjoint overlap Im<lambda|Y_b0 psi>
    T_OVL_ZL = 11,  // adjoint overlap Im<lambda|Z_b0 psi>, b0 local
    T_OVL_ZG = 12,  // adjoint overlap with Z on non-local g0
    T_MAT1F = 13,   // factored unitary on local bit b0: mats[mat] = (r0, r1, -, -); b1 bit 0 pivot, bit 1 sigma < 0,
                    // bit 2 r imaginary
    T_SCALE = 14,   // every amplitude times mats[mat].m00 (the factors pulled out by T_MAT1F)
    T_BLOCK = 15    // dense 2^b0 x 2^b0 block on local bits (g0 >> 5i) & 31, i < b0; matrix at complex offset
                    // `mat` of the plan's block matrices (row-major)
};

struct TileOp {
    uint8_t kind;
    uint8_t b0;
    uint8_t b1;
    uint8_t pad;
    uint32_t g0;
    uint32_t g1;
    uint32_t mat;   // matrix index (4 complex entries)
    int32_t slot;   // overlap slot
};
static_assert(sizeof(TileOp) == 20, "TileOp layout");

constexpr int kMaxLocal = 16;

// Kernel-side view of one pass: passed by value.
struct PassArgs {
    uint64_t nonlocal_mask;   // qubits not resident in the tile
    uint64_t n_tiles;
    uint32_t k;               // local qubits
    uint32_t low;             // local bits 0..low-1 are global qubits 0..low-1
    uint32_t n_ops;
    uint32_t n_mats;
    uint32_t slot_base;       // first overlap slot of this pass
    uint32_t n_slots;         // overlap slots in this pass
    uint8_t hi_q[kMaxLocal];  // global qubit of local bit low + r
};

struct Pass {
    PassArgs a;
    uint32_t op_begin = 0;    // into Plan::ops
    uint32_t mat_begin = 0;   // into Plan::mats (matrix index)
    uint64_t resident = 0;    // qubits resident in the tile
    std::vector<BGate> gates; // the pass's gates in order (after 1q merging, overlaps as BK_OVL), global qubits
    uint32_t n_blocks = 0;    // BK_BLOCK items among `gates`
    uint32_t max_block = 0;   // widest of them (qubits)
};

// ---- register-tiled passes (complex64) -------------------------------------
// A CTA of 32 << WB threads holds a 2^(9+WB)-amplitude tile: lane bits are
// qubits 0..4 (so every warp access is 256 contiguous bytes), each thread
// keeps 16 amplitudes in registers (4 register qubits) and the warp index
// spans WB more resident qubits. Gates on register qubits run in registers,
// on lane qubits through warp shuffles; a warp-qubit gate first exchanges
// register and warp qubits through shared memory (a remap). SWAPs among
// register/warp qubits relabel positions and move no data.
enum RsKind : uint8_t {
    RS_MREG = 0,    // dense 2x2 on register position p0
    RS_MLANE = 1,   // dense 2x2 on lane bit p0
    RS_DIAG = 2,    // diag(m00, m11) on bit descriptor p0
    RS_CNOT = 3,    // control descriptor p0, target descriptor p1 (lane or register)
    RS_CZ = 4,      // descriptors p0, p1
    RS_SWAP_LR = 5, // lane bit p0 <-> register position p1
    RS_SWAP_LL = 6, // lane bits p0 <-> p1
    RS_REMAP = 7    // a = old layout slots, b = new layout slots (3 bits per position)
};
// Bit descriptors: 0..4 lane bit, 8+r register position, 16+w warp position,
// 64+q qubit q outside the tile.
struct RsOp {
    uint8_t kind;
    uint8_t p0;
    uint8_t p1;
    uint8_t mk;    // matrix structure: 0 general, 1 real, 2 real diagonal + imaginary off-diagonal
    uint32_t a;
    uint32_t b;
    uint32_t mat;  // matrix index
};
static_assert(sizeof(RsOp) == 16, "RsOp layout");

struct RsPassArgs {
    uint64_t nonlocal_mask;
    uint64_t n_tiles;
    uint32_t n_ops;
    uint32_t n_mats;
    uint8_t load_q[8];   // qubit at register positions 0..3 then warp positions 0..WB-1, at load
    uint8_t store_q[8];  // the same at store (after relabels and remaps)
};

struct RsPass {
    RsPassArgs a;
    bool fallback = false;  // run this pass with the shared-memory tile kernel
    uint32_t op_begin = 0;
    uint32_t mat_begin = 0;
};

struct RsPlan {
    int wb = 3;
    std::vector<RsPass> passes;
    std::vector<RsOp> ops;
    std::vector<double> mats;
};

struct Plan {
    uint32_t n = 0;
    std::vector<Pass> passes;
    std::vector<TileOp> ops;
    std::vector<double> mats;        // 8 doubles per matrix
    std::vector<int64_t> slot_param; // overlap slot -> parameter index
    uint32_t n_slots = 0;
    std::vector<double> bmats;       // dense block matrices (interleaved complex), see BK_BLOCK
    uint32_t block_qubits = 0;       // fusion width the plan was made with (0: gates one by one)
};

struct PlanOpts {
    int tile_qubits = 12;   // k
    int low_qubits = 5;     // always-local contiguous low qubits
    bool merge_1q = true;   // multiply consecutive 1q gates on one qubit
    bool backward = false;  // adjoint reverse sweep: inverse gates + overlaps
    int max_items = 768;    // bound on ops per pass (shared-memory budget)
    bool search = true;     // choose each pass's resident qubits by look-ahead
    int block_qubits = 0;   // forward plans: fuse each pass's gates into dense blocks of up to this many
                            // qubits (2..5); every qubit a gate touches is then tile-resident
};

int plan_passes(uint32_t n, const std::vector<BGate> &gates, const PlanOpts &o, Plan &plan);
// Dense matrices of gates and fused blocks (host, f64, row-major, bit i of
// the local index = i-th qubit of the ascending list `qs`).
void dense_matrix(const BGate &g, const std::vector<double> &bmats, std::vector<uint32_t> &qs,
                  std::vector<std::complex<double>> &M);
std::vector<std::complex<double>> widen_matrix(const std::vector<uint32_t> &qs, const std::vector<std::complex<double>> &M,
                                               const std::vector<uint32_t> &nq);
void apply_gate_to_matrix(const std::vector<uint32_t> &qs, std::vector<std::complex<double>> &M, const BGate &g);
std::vector<uint32_t> qubits_of_mask(uint64_t m);
// Lower a forward plan to register-tiled passes; passes whose tile is not
// {qubits 0..4} plus 4 + wb more qubits are marked fallback.
int lower_rs(const Plan &plan, int wb, RsPlan &out);
// Default tile/low widths for a state.
void default_tiling(uint32_t n, int dtype, int requested_tile, int *tile, int *low);
void forward_tiling(uint32_t n, int dtype, int requested_tile, int flags, int *tile, int *low);

// ---- launchers (kernels in *.cu) ------------------------------------------
// Unfused single-gate sweeps.
int launch_gate1(qf_sv *sv, const BGate &g);
int launch_gate2(qf_sv *sv, const BGate &g);
// Upload a plan's ops+matrices into the context workspace and run every pass
// (register-tiled for complex64 where the tile fits, shared memory otherwise).
int run_plan(qf_sv *sv, const Plan &plan, int flags = 0);
int run_plan_smem(qf_sv *sv, const Plan &plan);
// Plans with dense blocks: the shared-memory block interpreter (any width,
// complex64 and complex128) and, for complex64 blocks of 5 qubits, the
// tensor-core pass (blockmma.cu).
int run_plan_blocks(qf_sv *sv, const Plan &plan);
bool mma_blocks_fit(const Plan &plan);
int run_plan_blocks_mma(qf_sv *sv, const Plan &plan);
int run_plan_rs(qf_sv *sv, const Plan &plan, int wb);
// Compiled register-tiled passes (jit.cpp); states of at least kJitMinQubits
// qubits use them by default.
constexpr uint32_t kJitMinQubits = 24;
bool jit_available();
int run_plan_jit(qf_sv *sv, const Plan &plan, int wb);
// Generate the plan's pass kernels and compile them with NVRTC without
// loading them (no GPU needed); for tests of the code generator. `dual`
// generates the backward (psi, lambda) kernels of an adjoint plan.
int jit_check_compile(const Plan &plan, int wb, std::string *source, std::string *err, bool dual = false);
// Backward adjoint passes on (psi, lambda); overlap partials per slot are
// accumulated into d_slot_sums (f64, plan.n_slots entries, not cleared here).
// Complex64 states use compiled dual passes (by default from kJitMinQubits
// qubits, or with QF_EXEC_FLAG_JIT; QF_EXEC_FLAG_SMEM_TILES forces the
// shared-memory kernel).
int run_plan_dual(qf_sv *psi, qf_sv *lambda, const Plan &plan, double *d_slot_sums, int flags = 0);
int run_plan_dual_smem(qf_sv *psi, qf_sv *lambda, const Plan &plan, double *d_slot_sums);
// Compiled backward passes; falls back to run_plan_dual_smem for plans the
// compiled layout does not cover.
int run_plan_jit_dual(qf_sv *psi, qf_sv *lambda, const Plan &plan, double *d_slot_sums);
// slot_sums[s] += sum over b < stride of partials[s * stride + b] (block order)
int reduce_slots(qf_ctx *ctx, const double *partials, uint32_t stride, uint32_t n_slots, double *d_slot_sums);

// Reductions (results to host unless noted).
int reduce_norm_sqr(qf_sv *sv, double *out);
int reduce_probabilities(qf_sv *sv, double *d_out);  // device output
int reduce_expect_z_all(qf_sv *sv, double *out);     // n values
int reduce_expect_1q(qf_sv *sv, int obs, uint32_t q, double *out);
int reduce_p_one(qf_sv *sv, uint32_t q, double *out);
int collapse(qf_sv *sv, uint32_t q, int outcome, double scale);
// Pauli sums: <psi|H|psi> (complex), and lambda = H psi with <psi|lambda>.
int pauli_expectation(qf_sv *sv, const qf_pauli_term *terms, uint64_t n_terms, double out[2]);
// lambda = H psi and <psi|H|psi>: into *energy after a stream synchronize, or,
// with d_energy, left in device memory (two doubles: real, imaginary part)
int pauli_apply(qf_sv *psi, qf_sv *lambda, const qf_pauli_term *terms, uint64_t n_terms, double *energy,
                double *d_energy = nullptr);
// ---- Pauli-sum passes (reduce.cu, compiled form in jit.cpp) --------------
struct PTerm {
    uint64_t z;
    double cre, cim;  // coefficient times i^{ny}
    uint64_t zo;      // z on the pass's non-resident qubits
    uint32_t zl;      // z on the resident qubits, in tile-local bits
    uint32_t q;       // bit r: parity of r & (zl >> 8) (the register part of a thread's amplitudes)
};
struct PGroup {
    uint64_t x;        // global x-mask
    uint32_t xl;       // the same mask in local tile bits
    uint32_t t_begin;  // into the pass's term array
    uint32_t t_count;
    uint32_t real;     // every coefficient of the group is real
    // Groups of many terms (the register-tiled pass) are evaluated from two
    // per-tile tables: their terms are ordered [z only on local bits 0..5 |
    // only on local bits 6.. | only off the tile | both halves], and
    // G(j) = TL[j & 63] + TH[j >> 6] + the terms spanning both halves.
    uint32_t tab;      // table slot, or kNoTable
    uint32_t n_lo, n_hi, n_const;
};
constexpr uint32_t kNoTable = 0xFFFFFFFFu;
constexpr uint32_t kTableTerms = 6;     // groups with at least this many terms get tables
constexpr uint32_t kTableEntries = 192;  // 64 (bits 0..5) + up to 128 (bits 6..12)
struct PPassArgs {
    uint64_t nonlocal_mask;
    uint64_t n_tiles;
    uint32_t k, low, n_groups, n_terms;
    uint32_t mode;  // 0 = expectation, 1 = write lambda, 2 = accumulate lambda
    uint32_t last;  // accumulate <psi|lambda> (mode 1/2)
    uint32_t n_tables;  // groups evaluated from per-tile tables (register-tiled pass)
    uint8_t hi_q[kMaxLocal];
};


// Compiled Pauli-sum passes (jit.cpp): complex64, every pass a 12-bit tile whose
// low five bits are qubits 0..4; pass p writes its partial sums to
// partials[p * slice_stride ...] (2 doubles per CTA, at most max_grid CTAs).
// *ran is false (and nothing launched) when a pass does not fit.
int run_pauli_jit(qf_sv *psi, qf_sv *lam, const std::vector<const PPassArgs *> &args,
                  const std::vector<const std::vector<PGroup> *> &groups, const std::vector<const std::vector<PTerm> *> &terms,
                  double *partials, uint32_t slice_stride, uint32_t max_grid, bool *ran);
// Launch counts of the Pauli-sum passes (host only): tile passes and sweeps of
// groups whose x-mask does not fit a tile.
int pauli_plan_stats(uint32_t n, int dtype, const qf_pauli_term *terms, uint64_t n_terms, uint64_t *tile_passes,
                     uint64_t *wide_passes);
// Fill/convert.
int fill_zero_state(qf_sv *sv);
int convert_from_f64(qf_sv *sv, const double *d_src);
int convert_to_f64(qf_sv *sv, double *d_dst);
// Batches: B states of 2^n amplitudes in one allocation (state b at b << n).
int batch_set_zero(qf_sv *sv, uint32_t n, uint64_t B);
// Measure qubit q of every state with uniforms[b]; outcomes to host; on an
// invalid probability nothing is collapsed.
int batch_measure(qf_sv *sv, uint32_t n, uint64_t B, uint32_t q, const double *uniforms, uint8_t *outcomes);
// Density matrices (density.cu). coef = (a, b, c, d, e, f) of
// v00' = a v00 + b v11, v11' = c v00 + d v11, v01' = e v01, v10' = f v10 on
// the bit pair (row n + q, column q).
int dm_channel(qf_sv *sv, uint32_t n, uint32_t q, const double coef[6]);
// `count` consecutive channels in one sweep; their bits plus the low five
// column bits must span at most 12 bits (2n >= 5).
int dm_channels_fused(qf_sv *sv, uint32_t n, const uint32_t *qs, const double (*coefs)[6], uint32_t count);
// mode 0 trace (out[0] re, out[1] im), 1 P(1) of q, 2 <Z_q>, 3 <X_q>, 4 <Y_q>.
int dm_diag_reduce(qf_sv *sv, uint32_t n, uint32_t q, int mode, double out[2]);
int dm_diagonal(qf_sv *sv, uint32_t n, double *d_out);
int dm_collapse(qf_sv *sv, uint32_t n, uint32_t q, int outcome, double prob);
int dm_from_state(qf_sv *dm, uint32_t n, const qf_sv *psi);
int dm_maximally_mixed(qf_sv *dm, uint32_t n);
// Per-shot trajectories in shared memory (trajectory.cu): whether 2^n
// amplitudes of the dtype fit one CTA, and the run itself from the initial
// device state; starts[s] = shot s's generator state at its first draw.
bool trajectories_fit(const qf_ctx *ctx, uint32_t n, int dtype);
int run_trajectories(qf_sv *init, const qf_op *ops, uint64_t n_ops, uint64_t shots, const uint64_t *starts, double tie_eps,
                     bool allow_noise, uint64_t *outcomes, uint64_t *n_ties);
// Sampler.
// start_states: optional per-shot generator states (host, `shots` entries)
// replacing the shot-major jump from `seed`.
int sample_shots(qf_sv *sv, const uint32_t *qubits, const uint32_t *cbits, uint32_t m, uint64_t shots,
                 uint64_t seed, double tie_eps, uint64_t *outcomes_host, uint64_t *n_ties,
                 const uint64_t *start_states = nullptr);


// SmallRng jump-ahead (host): state advanced by `steps` calls of next_u64.
uint64_t rng_jump(uint64_t state, uint64_t steps);
void rng_jump_matrices(uint64_t stride, uint64_t (*mats)[64], int count);
// A jump matrix (64 columns over GF(2)) applied to a generator state.
uint64_t rng_apply(const uint64_t cols[64], uint64_t state);

// Dispatcher for a bound gate list on a resident state.
int execute_gates(qf_sv *sv, const std::vector<BGate> &gates, const qf_exec_opts *opts);
// Planning options of a forward sweep (tile widths, look-ahead, block width).
int plan_opts_for(uint32_t n, int dtype, const qf_exec_opts *opts, PlanOpts &po);

}  // namespace qf
