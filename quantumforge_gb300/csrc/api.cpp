// api.cpp — the extern "C" boundary declared in include/qf.h. Validation and
// error texts follow the reference's QuantumError / CudaError
// (src/lib.rs:507-664, src/cuda.rs:3051-3104); all checks run before any
// launch, and the device state is left untouched when a call is rejected.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "qf_internal.h"

namespace qf {

static thread_local std::string g_last_error = "";

int fail(int status, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

void clear_error() { g_last_error.clear(); }

int cuda_fail(cudaError_t e, const char *what) {
    return fail(QF_ERR_CUDA, "CUDA error %d (%s): %s in %s", (int)e, cudaGetErrorName(e), cudaGetErrorString(e), what);
}

int ensure_device(void **ptr, size_t *bytes, size_t need) {
    if (*bytes >= need && *ptr) return QF_OK;
    if (*ptr) {
        cudaError_t e = cudaFree(*ptr);
        *ptr = nullptr;
        *bytes = 0;
        if (e != cudaSuccess) return cuda_fail(e, "cudaFree(workspace)");
    }
    size_t want = std::max<size_t>(need, 1 << 16);
    cudaError_t e = cudaMalloc(ptr, want);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        cudaGetLastError();
        return fail(QF_ERR_MEMORY_ALLOCATION_FAILED, "could not reserve %zu bytes of device workspace", want);
    }
    *bytes = want;
    return QF_OK;
}

int ensure_pinned(void **ptr, size_t *bytes, size_t need) {
    if (*bytes >= need && *ptr) return QF_OK;
    if (*ptr) cudaFreeHost(*ptr);
    *ptr = nullptr;
    *bytes = 0;
    if (cudaMallocHost(ptr, need) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return fail(QF_ERR_MEMORY_ALLOCATION_FAILED, "could not reserve %zu bytes of pinned host memory", need);
    }
    *bytes = need;
    return QF_OK;
}

}  // namespace qf

using namespace qf;

namespace {

int bind_device(qf_ctx *ctx) {
    QF_CUDA(cudaSetDevice(ctx->device));
    return QF_OK;
}

int check_sv(const qf_sv *sv) {
    if (!sv || !sv->ctx || !sv->d) return fail(QF_ERR_INVALID_ARGUMENT, "state handle is NULL or released");
    return QF_OK;
}

int check_dtype(int dtype) {
    if (dtype != QF_C64 && dtype != QF_C128) return fail(QF_ERR_INVALID_ARGUMENT, "unknown dtype %d", dtype);
    return QF_OK;
}

// StateVector::zero_with_memory_budget size checks (src/lib.rs:940-966).
int alloc_state(qf_ctx *ctx, uint32_t qubits, int dtype, uint64_t budget, qf_sv **out, bool fill = true) {
    QF_TRY(check_dtype(dtype));
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    if (qubits > 40) return fail(QF_ERR_SIMULATION_SIZE_OVERFLOW, "dense simulation size exceeds the supported addressable range");
    const uint64_t dim = 1ULL << qubits;
    const uint64_t bytes = dim * (dtype == QF_C64 ? 8ULL : 16ULL);
    if (budget && bytes > budget)
        return fail(QF_ERR_MEMORY_BUDGET_EXCEEDED, "dense state needs at least %llu bytes, exceeding the %llu-byte memory budget",
                    (unsigned long long)bytes, (unsigned long long)budget);
    qf_sv *sv = new qf_sv();
    sv->ctx = ctx;
    sv->n = qubits;
    sv->dtype = dtype;
    sv->dim = dim;
    cudaError_t e = cudaMalloc(&sv->d, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete sv;
        return fail(QF_ERR_MEMORY_ALLOCATION_FAILED, "could not reserve memory for the dense quantum state (%llu bytes)",
                    (unsigned long long)bytes);
    }
    int st = fill ? fill_zero_state(sv) : QF_OK;
    if (st) {
        cudaFree(sv->d);
        delete sv;
        return st;
    }
    ctx->states.insert(sv);
    *out = sv;
    return QF_OK;
}

void free_state(qf_sv *sv) {
    if (!sv) return;
    if (sv->ctx) sv->ctx->states.erase(sv);
    if (sv->d) cudaFree(sv->d);
    delete sv;
}

// Checkpoint states for the adjoint: reused across gradients of the same
// shape instead of a cudaMalloc (and the implicit synchronisation of its
// cudaFree) per segment per call; at most kCkptPoolBytes stay cached.
constexpr uint64_t kCkptPoolBytes = 16ULL << 30;

int take_checkpoint(qf_ctx *ctx, uint32_t n, int dtype, qf_sv **out) {
    for (size_t i = ctx->ckpt_pool.size(); i-- > 0;) {
        qf_sv *c = ctx->ckpt_pool[i];
        if (c->n == n && c->dtype == dtype) {
            ctx->ckpt_pool.erase(ctx->ckpt_pool.begin() + (ptrdiff_t)i);
            *out = c;
            return QF_OK;
        }
    }
    return alloc_state(ctx, n, dtype, 0, out, false);  // overwritten by the checkpoint copy
}

void release_checkpoint(qf_ctx *ctx, qf_sv *c) {
    uint64_t held = 0;
    for (qf_sv *x : ctx->ckpt_pool) held += x->bytes();
    if (held + c->bytes() <= kCkptPoolBytes) {
        ctx->ckpt_pool.push_back(c);
        return;
    }
    free_state(c);
}

// A cached context-owned state of the requested shape (whole-circuit calls).
int scratch_state(qf_ctx *ctx, qf_sv **slot, uint32_t n, int dtype, qf_sv **out) {
    if (*slot && ((*slot)->n != n || (*slot)->dtype != dtype)) {
        free_state(*slot);
        *slot = nullptr;
    }
    if (!*slot) QF_TRY(alloc_state(ctx, n, dtype, 0, slot));
    *out = *slot;
    return QF_OK;
}

uint64_t classical_bit_check(const qf_op *ops, uint64_t n_ops, int *status) {
    uint64_t width = 0;
    *status = QF_OK;
    for (uint64_t k = 0; k < n_ops; ++k)
        if (ops[k].kind == QF_OP_MEASURE || ops[k].kind == QF_OP_COND) {
            if (ops[k].param >= 4096) {
                *status = fail(QF_ERR_CLASSICAL_BIT_OUT_OF_RANGE, "classical bit index %u exceeds the supported maximum of 4095",
                               ops[k].param);
                return 0;
            }
            width = std::max<uint64_t>(width, (uint64_t)ops[k].param + 1);
        }
    return width;
}

uint64_t count_rotations(const qf_op *ops, uint64_t n_ops) {
    uint64_t c = 0;
    for (uint64_t k = 0; k < n_ops; ++k) c += ops[k].kind == QF_OP_ROTATION;
    return c;
}

bool has_channel(const qf_op *ops, uint64_t n_ops) {
    for (uint64_t k = 0; k < n_ops; ++k)
        if (ops[k].kind == QF_OP_CHANNEL) return true;
    return false;
}

int check_terms_real(const qf_pauli_term *terms, uint64_t n_terms) {
    if (n_terms && !terms) return fail(QF_ERR_INVALID_ARGUMENT, "terms is NULL");
    for (uint64_t t = 0; t < n_terms; ++t) {
        if (!std::isfinite(terms[t].coeff_re) || !std::isfinite(terms[t].coeff_im))
            return fail(QF_ERR_NON_FINITE_PARAMETER, "observable coefficients must be finite");
        if (terms[t].coeff_im != 0.0)
            return fail(QF_ERR_INVALID_ARGUMENT, "gradient observables must be Hermitian (real coefficients)");
    }
    return QF_OK;
}

// Forward circuit + expectation on the context's scratch state.
int forward_expectation(qf_ctx *ctx, uint32_t n, int dtype, const qf_op *ops, uint64_t n_ops, const double *params,
                        uint64_t n_params, const double *inputs, uint64_t n_inputs, int64_t shift_op, double shift,
                        const qf_pauli_term *terms, uint64_t n_terms, const qf_exec_opts *exec, double *e) {
    std::vector<BGate> gates;
    QF_TRY(bind_ops(n, ops, n_ops, params, n_params, inputs, n_inputs, shift_op, shift, gates));
    qf_sv *sv;
    QF_TRY(scratch_state(ctx, &ctx->scratch_sv, n, dtype, &sv));
    QF_TRY(fill_zero_state(sv));
    QF_TRY(execute_gates(sv, gates, exec));
    double out[2];
    QF_TRY(pauli_expectation(sv, terms, n_terms, out));
    *e = out[0];
    return QF_OK;
}

// Adjoint gradient on the device (the method of adjoint_gradient_with_inputs,
// src/lib.rs:3564-3704, with O(2^n) memory): forward psi with optional
// checkpoints at segment starts, lambda = H psi, then each segment backwards
// in tile passes that carry psi and lambda together, accumulate
// Im<lambda|P_k psi> per rotation occurrence in f64 and apply U_k^dagger to
// both. With checkpoints, psi is restored from the stored forward state at
// every segment boundary instead of carrying the uncompute drift further.
int adjoint_device(qf_ctx *ctx, uint32_t n, const std::vector<BGate> &gates, const qf_pauli_term *terms, uint64_t n_terms,
                   const qf_gradient_opts *o, uint64_t n_params, double *energy, double *grad) {
    const int dtype = o->dtype;
    const int every = std::max(0, o->checkpoint_every);
    // segment boundaries by op index in the bound list
    std::vector<size_t> seg_begin;
    if (every > 0) {
        for (size_t s = 0; s < gates.size(); s += (size_t)every) seg_begin.push_back(s);
    } else {
        seg_begin.push_back(0);
    }
    if (gates.empty()) seg_begin.assign(1, 0);
    const size_t n_seg = seg_begin.size();
    qf_sv *psi, *lam;
    QF_TRY(scratch_state(ctx, &ctx->scratch_sv, n, dtype, &psi));
    QF_TRY(scratch_state(ctx, &ctx->scratch_sv2, n, dtype, &lam));
    std::vector<qf_sv *> ckpt;  // ckpt[s] = psi at the start of segment s+1
    struct Guard {
        qf_ctx *ctx;
        std::vector<qf_sv *> *v;
        ~Guard() {
            for (qf_sv *s : *v) release_checkpoint(ctx, s);
        }
    } guard{ctx, &ckpt};
    PlanOpts po;
    default_tiling(n, dtype, o->exec.tile_qubits, &po.tile_qubits, &po.low_qubits);
    po.search = !(o->exec.flags & QF_EXEC_FLAG_PLAN_FIRST_COME);
    QF_TRY(fill_zero_state(psi));
    for (size_t s = 0; s < n_seg; ++s) {
        const size_t b = seg_begin[s], e = s + 1 < n_seg ? seg_begin[s + 1] : gates.size();
        std::vector<BGate> seg(gates.begin() + b, gates.begin() + e);
        Plan plan;
        po.backward = false;
        QF_TRY(plan_passes(n, seg, po, plan));
        QF_TRY(run_plan(psi, plan, o->exec.flags));
        if (s + 1 < n_seg) {
            qf_sv *c;
            QF_TRY(take_checkpoint(ctx, n, dtype, &c));
            ckpt.push_back(c);
            QF_CUDA(cudaMemcpyAsync(c->d, psi->d, psi->bytes(), cudaMemcpyDeviceToDevice, ctx->stream));
        }
    }
    // every backward segment is planned while the forward passes run (after
    // their launches), then run back to back: the overlap slots of all segments
    // land in one device buffer that is read once at the end
    std::vector<Plan> bplans(n_seg);
    std::vector<size_t> slot_off(n_seg, 0);
    size_t total_slots = 0;
    {
        PlanOpts bo = po;
        bo.backward = true;
        bo.merge_1q = true;
        // the dual passes (psi and lambda per tile) are bound by arithmetic, not
        // HBM: fewer, heavier passes from the look-ahead measured 3 % slower
        // on the 24-qubit VQE, so the backward sweep fills passes first-come
        bo.search = false;
        for (size_t s = n_seg; s-- > 0;) {
            const size_t b = seg_begin[s], e = s + 1 < n_seg ? seg_begin[s + 1] : gates.size();
            std::vector<BGate> seg(gates.begin() + b, gates.begin() + e);
            QF_TRY(plan_passes(n, seg, bo, bplans[s]));
            slot_off[s] = total_slots;
            total_slots += bplans[s].n_slots;
        }
    }
    // the slot sums and, behind them, the energy stay on the device until the
    // single synchronize at the end: the host prepares the backward passes
    // while lambda = H psi runs
    const size_t bytes = sizeof(double) * total_slots;
    QF_TRY(ensure_device(&ctx->ws_tree, &ctx->ws_tree_bytes, bytes + 2 * sizeof(double)));
    double *d_sums = static_cast<double *>(ctx->ws_tree);
    QF_TRY(pauli_apply(psi, lam, terms, n_terms, nullptr, d_sums + total_slots));
    if (total_slots) QF_CUDA(cudaMemsetAsync(d_sums, 0, bytes, ctx->stream));
    for (size_t s = n_seg; s-- > 0;) {
        QF_TRY(run_plan_dual(psi, lam, bplans[s], bplans[s].n_slots ? d_sums + slot_off[s] : nullptr, o->exec.flags));
        if (s > 0 && !ckpt.empty())
            QF_CUDA(cudaMemcpyAsync(psi->d, ckpt[s - 1]->d, psi->bytes(), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    std::vector<double> sums(total_slots + 2);
    QF_CUDA(cudaMemcpyAsync(sums.data(), d_sums, bytes + 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    if (energy) *energy = sums[total_slots];
    std::vector<double> g(n_params, 0.0);
    for (size_t s = n_seg; s-- > 0;)
        for (uint32_t k = 0; k < bplans[s].n_slots; ++k) g[(size_t)bplans[s].slot_param[k]] += sums[slot_off[s] + k];
    std::copy(g.begin(), g.end(), grad);
    return QF_OK;
}

// One uniform of SmallRng (src/lib.rs:4899-4911) from a shot's state.
inline double next_uniform(uint64_t *x) {
    uint64_t v = *x;
    v ^= v << 13;
    v ^= v >> 7;
    v ^= v << 17;
    *x = v;
    return (double)(v >> 11) * (1.0 / 9007199254740992.0);
}

inline bool valid_probability(double p) { return std::isfinite(p) && p >= 0.0 && p <= 1.0; }  // src/lib.rs:2229-2235

inline double clamp01(double x) { return std::min(1.0, std::max(0.0, x)); }

// SmallRng::seeded (src/lib.rs:4881-4897): splitmix64 of the seed, a zero
// state replaced by the golden-ratio constant.
inline uint64_t smallrng_seeded(uint64_t seed) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return z == 0 ? 0x9E3779B97F4A7C15ULL : z;
}

// Every shot's generator state at its first draw: shot s starts at draw s * d
// of SmallRng::seeded(seed) (src/lib.rs:4881-4897), d = measurements (and,
// with noise, channels) per shot — the reference's shot-major stream.
std::vector<uint64_t> shot_starts(const qf_op *ops, uint64_t n_ops, uint64_t shots, uint64_t seed, bool allow_noise) {
    uint64_t draws = 0;
    for (uint64_t k = 0; k < n_ops; ++k)
        draws += ops[k].kind == QF_OP_MEASURE || (allow_noise && ops[k].kind == QF_OP_CHANNEL);
    std::vector<uint64_t> st(shots);
    uint64_t x = smallrng_seeded(seed);
    if (draws <= 64) {  // step the stream
        for (uint64_t s = 0; s < shots; ++s) {
            st[s] = x;
            for (uint64_t k = 0; k < draws; ++k) next_uniform(&x);
        }
        return st;
    }
    uint64_t jump[1][64];  // T^draws: one matrix application per shot
    rng_jump_matrices(draws, jump, 1);
    for (uint64_t s = 0; s < shots; ++s) {
        st[s] = x;
        x = rng_apply(jump[0], x);
    }
    return st;
}

// StateVector::normalize (src/lib.rs:1005-1014): divide by sqrt(norm_sqr).
int normalize_state(qf_sv *sv) {
    double nrm;
    QF_TRY(reduce_norm_sqr(sv, &nrm));
    const double norm = std::sqrt(nrm);
    if (norm == 0.0 || !std::isfinite(norm)) return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", norm);
    return collapse(sv, 0, -1, norm);
}

BGate mat1(uint32_t q, double m00, double m01, double m10, double m11) {
    BGate g;
    g.kind = BK_MAT1;
    g.q0 = q;
    g.m[0] = m00;
    g.m[2] = m01;
    g.m[4] = m10;
    g.m[6] = m11;
    g.diag = matrix_is_diag(g.m);
    return g;
}

// Circuit::run_shots_impl (src/lib.rs:2842-2916) for circuits with
// mid-circuit measurements, repeated measurements, ConditionalSingleQubit
// feed-forward or (allow_noise) channel trajectories.
//
// Shots walk a tree: a node is one device state with its classical register
// and the shots that reached it. Unitary segments (with the conditionals that
// fire for the node's register) run through the fused engine once per node.
// At a measurement or a channel every shot of the node draws its own next
// uniform (shot s starts at draw s * draws-per-shot of SmallRng::seeded(seed),
// the reference's shot-major stream) and the shots split into children:
// measurement outcomes (collapse, src/lib.rs:1321-1351) or Kraus branches
// (apply_channel_trajectory, src/lib.rs:1356-1506; the branch matrix is
// queued in front of the child's next segment). The tree is walked depth
// first: a parent's state is shared by its children, copied for all but the
// last one, so at most one state per level of the current path is alive.
// The trailing measurements of distinct qubits use the prefix-tree sampler
// per leaf. Decisions equal the reference's except where a uniform lies
// within tie_eps of a threshold (counted); complex64 states take P(1)
// relative to their own norm.
int run_shots_branching(qf_ctx *ctx, uint32_t n, int dtype, const qf_op *ops, uint64_t n_ops, const double *init,
                        uint64_t shots, uint64_t seed, double tie_eps, bool allow_noise, uint64_t *outcomes,
                        uint64_t *n_ties, const qf_exec_opts *opts) {
    // terminal block: the trailing measurements of distinct qubits
    uint64_t T = n_ops, seen = 0;
    while (T > 0 && ops[T - 1].kind == QF_OP_MEASURE && !((seen >> ops[T - 1].q0) & 1ULL)) {
        seen |= 1ULL << ops[T - 1].q0;
        --T;
    }
    std::vector<uint64_t> st = shot_starts(ops, n_ops, shots, seed, allow_noise);
    // A state shared by the children of one node; the last child to start
    // takes it over, the others copy it.
    struct Shared {
        qf_sv *sv;
        int users;
    };
    struct Node {
        Shared *src;                 // parent state (nullptr: `own` is set)
        qf_sv *own;
        uint64_t k;                  // next op
        uint64_t reg;                // classical register
        std::vector<uint32_t> shots;
        std::vector<BGate> pre;      // Kraus branch matrix to apply first
        uint32_t mq;                 // measurement child: collapse q
        int out;                     //   outcome, or -1 for none
        double scale;                //   sqrt(probability)
    };
    std::vector<Node> stack;
    std::vector<Shared *> shared;
    std::vector<qf_sv *> spare;  // finished leaves' states, reused for copies
    qf_sv *cur = nullptr;
    struct Guard {
        std::vector<Shared *> *sh;
        std::vector<Node> *st;
        std::vector<qf_sv *> *spare;
        qf_sv **cur;
        ~Guard() {
            for (Shared *x : *sh) {
                if (x->sv) free_state(x->sv);
                delete x;
            }
            for (Node &nd : *st)
                if (nd.own) free_state(nd.own);
            for (qf_sv *x : *spare) free_state(x);
            if (*cur) free_state(*cur);
        }
    } guard{&shared, &stack, &spare, &cur};
    {
        Node root{};
        QF_TRY(alloc_state(ctx, n, dtype, 0, &root.own));
        stack.push_back(std::move(root));
        Node &r = stack.back();
        r.out = -1;
        r.shots.resize(shots);
        for (uint64_t s = 0; s < shots; ++s) r.shots[s] = (uint32_t)s;
        if (init) {
            QF_TRY(convert_from_f64(r.own, init));
            if (allow_noise) QF_TRY(normalize_state(r.own));
        } else {
            QF_TRY(fill_zero_state(r.own));
        }
    }
    std::vector<uint32_t> tq, tc;  // terminal block
    uint64_t tmask = 0;
    for (uint64_t k = T; k < n_ops; ++k) {
        tq.push_back(ops[k].q0);
        tc.push_back(ops[k].param);
        tmask |= 1ULL << ops[k].param;
    }
    uint64_t ties = 0;
    std::vector<qf_op> run;
    std::vector<BGate> gates;
    while (!stack.empty()) {
        Node nd = std::move(stack.back());
        stack.pop_back();
        // take or copy the state
        if (nd.own) {
            cur = nd.own;
            nd.own = nullptr;
        } else if (--nd.src->users == 0) {
            cur = nd.src->sv;
            nd.src->sv = nullptr;
        } else {
            if (!spare.empty()) {
                cur = spare.back();
                spare.pop_back();
            } else {
                QF_TRY(alloc_state(ctx, n, dtype, 0, &cur));
            }
            QF_CUDA(cudaMemcpyAsync(cur->d, nd.src->sv->d, cur->bytes(), cudaMemcpyDeviceToDevice, ctx->stream));
        }
        if (nd.out >= 0) QF_TRY(collapse(cur, nd.mq, nd.out, nd.scale));
        // the unitary segment up to the next branch point
        uint64_t k = nd.k;
        run.clear();
        for (; k < T; ++k) {
            const qf_op &o = ops[k];
            if (o.kind == QF_OP_MEASURE || (o.kind == QF_OP_CHANNEL && allow_noise)) break;
            if (o.kind == QF_OP_COND) {  // ConditionalSingleQubit: apply when classical[bit] == value
                if (((nd.reg >> o.param) & 1ULL) != (uint64_t)(o.flags & 1)) continue;
                qf_op g = o;
                g.kind = QF_OP_GATE;
                g.param = 0;
                g.flags = 0;
                run.push_back(g);
            } else {
                run.push_back(o);
            }
        }
        gates.clear();
        QF_TRY(bind_ops(n, run.data(), run.size(), nullptr, 0, nullptr, 0, -1, 0.0, gates));
        if (!nd.pre.empty()) gates.insert(gates.begin(), nd.pre.begin(), nd.pre.end());
        if (!gates.empty()) QF_TRY(execute_gates(cur, gates, opts));
        if (k >= T) {  // leaf: the terminal measurements, or the register as it stands
            if (!tq.empty()) {
                std::vector<uint64_t> starts(nd.shots.size()), out(nd.shots.size());
                for (size_t i = 0; i < nd.shots.size(); ++i) starts[i] = st[nd.shots[i]];
                uint64_t t = 0;
                QF_TRY(sample_shots(cur, tq.data(), tc.data(), (uint32_t)tq.size(), nd.shots.size(), seed, tie_eps,
                                    out.data(), &t, starts.data()));
                ties += t;
                if (outcomes)
                    for (size_t i = 0; i < nd.shots.size(); ++i) outcomes[nd.shots[i]] = (nd.reg & ~tmask) | out[i];
            } else if (outcomes) {
                for (uint32_t s : nd.shots) outcomes[s] = nd.reg;
            }
            spare.push_back(cur);
            cur = nullptr;
            continue;
        }
        // a branch point: split the node's shots into up to four children
        const qf_op &o = ops[k];
        const uint32_t q = o.q0;
        if (q >= n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", q, n);
        std::vector<uint32_t> go[4];
        BGate mats[4];
        bool has_mat[4] = {false, false, false, false};
        double child_norm[4] = {1.0, 1.0, 1.0, 1.0};  // checked for every child that gets shots
        bool check_norm = false;
        double prob[2] = {0.0, 0.0};
        if (o.kind == QF_OP_MEASURE) {
            double p1;
            QF_TRY(reduce_p_one(cur, q, &p1));
            if (dtype == QF_C64) {  // relative to the state's own norm, which f32 rounding moves off 1
                double nrm;
                QF_TRY(reduce_norm_sqr(cur, &nrm));
                if (nrm > 0.0) p1 /= nrm;
            }
            p1 = clamp01(p1);
            for (uint32_t s : nd.shots) {
                const double u = next_uniform(&st[s]);
                if (std::fabs(u - p1) < tie_eps) ++ties;
                go[u < p1 ? 1 : 0].push_back(s);
            }
            prob[0] = 1.0 - p1;
            prob[1] = p1;
            for (int c = 0; c < 2; ++c)
                if (!go[c].empty() && prob[c] <= 2.220446049250313e-16)
                    return fail(QF_ERR_INVALID_PROBABILITY, "measurement probability must be in [0, 1], got %g", prob[c]);
        } else if (o.gate == QF_CHANNEL_DEPOLARIZING) {
            const double p = o.theta;
            if (!valid_probability(p)) return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", p);
            for (uint32_t s : nd.shots) {
                const double u = next_uniform(&st[s]);
                int c = 0;
                if (u >= 1.0 - p && p > 0.0) {
                    const double b = std::floor((u - (1.0 - p)) * (3.0 / p));
                    c = 1 + (b >= 2.0 ? 2 : (int)b);  // X, Y, Z
                }
                go[c].push_back(s);
            }
            for (int c = 1; c < 4; ++c) {
                mats[c].kind = BK_MAT1;
                mats[c].q0 = q;
                QF_TRY(gate_matrix(c == 1 ? QF_GATE_X : c == 2 ? QF_GATE_Y : QF_GATE_Z, 0.0, mats[c].m));
                mats[c].diag = matrix_is_diag(mats[c].m);
                has_mat[c] = true;
            }
        } else if (o.gate == QF_CHANNEL_AMPLITUDE_DAMPING || o.gate == QF_CHANNEL_PHASE_DAMPING) {
            const double gamma = o.theta;
            if (!valid_probability(gamma))
                return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", gamma);
            double norm, p_one;
            QF_TRY(reduce_norm_sqr(cur, &norm));
            if (!std::isfinite(norm) || norm <= 2.220446049250313e-16)
                return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", norm);
            QF_TRY(reduce_p_one(cur, q, &p_one));
            const double jump_p = clamp01(gamma * p_one / norm);
            for (uint32_t s : nd.shots) {
                const double u = next_uniform(&st[s]);
                if (std::fabs(u - jump_p) < tie_eps) ++ties;
                go[u < jump_p ? 1 : 0].push_back(s);
            }
            child_norm[1] = gamma * p_one;
            child_norm[0] = norm - gamma * p_one;
            check_norm = true;
            const double inv1 = 1.0 / std::sqrt(child_norm[1]), inv0 = 1.0 / std::sqrt(child_norm[0]);
            const double s1 = std::sqrt(gamma) * inv1;
            mats[1] = o.gate == QF_CHANNEL_AMPLITUDE_DAMPING ? mat1(q, 0.0, s1, 0.0, 0.0) : mat1(q, 0.0, 0.0, 0.0, s1);
            mats[0] = mat1(q, inv0, 0.0, 0.0, std::sqrt(1.0 - gamma) * inv0);
            has_mat[0] = has_mat[1] = true;
        } else if (o.gate == QF_CHANNEL_THERMAL_DAMPING) {
            const double gd = o.theta, beta = qf_op_aux(&o);
            if (!valid_probability(gd)) return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", gd);
            if (!std::isfinite(beta) || beta < 0.0)
                return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", beta);
            const double gu = gd * std::exp(-beta);  // NoiseChannel::thermal_rates (src/lib.rs:1611-1626)
            double norm, p_one;
            QF_TRY(reduce_norm_sqr(cur, &norm));
            if (!std::isfinite(norm) || norm <= 2.220446049250313e-16)
                return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", norm);
            QF_TRY(reduce_p_one(cur, q, &p_one));
            const double p1 = clamp01(p_one / norm), p0 = 1.0 - p1;
            const double down = p1 * gd, up = p0 * gu;
            const double pd = p0 * (1.0 - gu), pe = p1 * (1.0 - gd);
            const double stay = pd + pe, du = down + up;
            for (uint32_t s : nd.shots) {
                const double u = next_uniform(&st[s]);
                if (std::fabs(u - down) < tie_eps || std::fabs(u - du) < tie_eps) ++ties;
                go[u < down ? 1 : (u < du ? 2 : 0)].push_back(s);
            }
            child_norm[1] = down;
            child_norm[2] = up;
            child_norm[0] = stay;
            check_norm = true;
            const double inv1 = 1.0 / std::sqrt(down), inv2 = 1.0 / std::sqrt(up), inv0 = 1.0 / std::sqrt(stay);
            mats[1] = mat1(q, 0.0, std::sqrt(gd) * inv1, 0.0, 0.0);
            mats[2] = mat1(q, 0.0, 0.0, std::sqrt(gu) * inv2, 0.0);
            mats[0] = mat1(q, std::sqrt(1.0 - gu) * inv0, 0.0, 0.0, std::sqrt(1.0 - gd) * inv0);
            has_mat[0] = has_mat[1] = has_mat[2] = true;
        } else {
            return fail(QF_ERR_INVALID_ARGUMENT, "unknown noise channel %u", (unsigned)o.gate);
        }
        if (check_norm)
            for (int c = 0; c < 4; ++c)
                if (!go[c].empty() && (!std::isfinite(child_norm[c]) || child_norm[c] <= 2.220446049250313e-16))
                    return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", child_norm[c]);
        int users = 0;
        for (int c = 0; c < 4; ++c) users += !go[c].empty();
        Shared *sh = new Shared{cur, users};
        shared.push_back(sh);
        cur = nullptr;
        // pushed in reverse so that child 0 runs first; the last to run takes the state
        for (int c = 3; c >= 0; --c) {
            if (go[c].empty()) continue;
            Node ch{};
            ch.src = sh;
            ch.k = k + 1;
            ch.reg = nd.reg;
            ch.shots = std::move(go[c]);
            ch.out = -1;
            if (o.kind == QF_OP_MEASURE) {
                ch.reg = (nd.reg & ~(1ULL << o.param)) | ((uint64_t)c << o.param);
                ch.mq = q;
                ch.out = c;
                ch.scale = std::sqrt(prob[c]);
            } else if (has_mat[c]) {
                ch.pre.push_back(mats[c]);
            }
            stack.push_back(std::move(ch));
        }
    }
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    if (n_ties) *n_ties = ties;
    return QF_OK;
}

// Circuit::run_shots / run_shots_with_noise (src/lib.rs:2822-2916): a
// unitary prefix then measurements of distinct qubits runs as one state and
// the prefix-tree sampler; anything else (feed-forward, a measurement
// followed by gates, a qubit measured twice, a channel trajectory) runs in
// the branching engine.
int run_shots_entry(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *init_amps,
                    uint64_t shots, uint64_t seed, double tie_eps, bool allow_noise, uint64_t *outcomes,
                    uint32_t *classical_width, uint64_t *n_ties, const qf_exec_opts *opts) {
    clear_error();
    if (!ctx) return fail(QF_ERR_INVALID_ARGUMENT, "context is NULL");
    QF_TRY(check_dtype(dtype));
    if (shots == 0) return fail(QF_ERR_INVALID_SHOT_COUNT, "shot count must be greater than zero");
    if (n_ops && !ops) return fail(QF_ERR_INVALID_ARGUMENT, "ops is NULL");
    int st;
    const uint64_t width = classical_bit_check(ops, n_ops, &st);
    if (st) return st;
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    uint64_t first = n_ops;
    for (uint64_t k = 0; k < n_ops; ++k)
        if (ops[k].kind == QF_OP_MEASURE) { first = k; break; }
    std::vector<uint32_t> mq, mc;
    bool branching = false;
    uint64_t measured = 0;
    for (uint64_t k = 0; k < n_ops; ++k) {
        if (ops[k].kind == QF_OP_CHANNEL) {
            if (!allow_noise)
                return fail(QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX, "this circuit operation requires density-matrix simulation");
            branching = true;
        }
        if (ops[k].kind == QF_OP_COND || (k > first && ops[k].kind != QF_OP_MEASURE)) branching = true;
        if (ops[k].kind == QF_OP_MEASURE || ops[k].kind == QF_OP_COND || ops[k].kind == QF_OP_CHANNEL) {
            if (ops[k].q0 >= qubits)
                return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", ops[k].q0, qubits);
        }
        if (ops[k].kind == QF_OP_MEASURE) {
            if ((measured >> ops[k].q0) & 1ULL) branching = true;
            measured |= 1ULL << ops[k].q0;
            mq.push_back(ops[k].q0);
            mc.push_back(ops[k].param);
        }
    }
    if (width > 64) return fail(QF_ERR_UNSUPPORTED_OPERATION, "classical registers wider than 64 bits are not packed");
    if (qubits > 63 && !mq.empty()) return fail(QF_ERR_UNSUPPORTED_OPERATION, "measurement masks cover at most 63 qubits");
    if (branching) {
        QF_TRY(bind_device(ctx));
        if (classical_width) *classical_width = (uint32_t)width;
        // Small states with channel trajectories (many distinct branches): one
        // CTA per shot in shared memory; otherwise the branch tree of device states.
        const int fl = opts ? opts->flags : 0;
        bool noisy = false;
        for (uint64_t k = 0; k < n_ops; ++k) noisy |= ops[k].kind == QF_OP_CHANNEL;
        const bool traj = trajectories_fit(ctx, qubits, dtype) && !(fl & QF_EXEC_FLAG_SHOTS_TREE) &&
                          ((fl & QF_EXEC_FLAG_SHOTS_TRAJECTORIES) || noisy);
        if (traj) {
            qf_sv *sv;
            QF_TRY(scratch_state(ctx, &ctx->scratch_sv, qubits, dtype, &sv));
            if (init_amps) {
                QF_TRY(convert_from_f64(sv, init_amps));
                if (allow_noise) QF_TRY(normalize_state(sv));
            } else {
                QF_TRY(fill_zero_state(sv));
            }
            const std::vector<uint64_t> st = shot_starts(ops, n_ops, shots, seed, allow_noise);
            return run_trajectories(sv, ops, n_ops, shots, st.data(), tie_eps, allow_noise, outcomes, n_ties);
        }
        return run_shots_branching(ctx, qubits, dtype, ops, n_ops, init_amps, shots, seed, tie_eps, allow_noise, outcomes,
                                   n_ties, opts);
    }
    std::vector<BGate> gates;
    QF_TRY(bind_ops(qubits, ops, first, nullptr, 0, nullptr, 0, -1, 0.0, gates));
    QF_TRY(bind_device(ctx));
    qf_sv *sv;
    QF_TRY(scratch_state(ctx, &ctx->scratch_sv, qubits, dtype, &sv));
    if (init_amps) {
        QF_TRY(convert_from_f64(sv, init_amps));
        if (allow_noise) QF_TRY(normalize_state(sv));
    } else {
        QF_TRY(fill_zero_state(sv));
    }
    QF_TRY(execute_gates(sv, gates, opts));
    if (classical_width) *classical_width = (uint32_t)width;
    return sample_shots(sv, mq.data(), mc.data(), (uint32_t)mq.size(), shots, seed, tie_eps, outcomes, n_ties);
}

}  // namespace

extern "C" {

const char *qf_last_error(void) { return g_last_error.c_str(); }

const char *qf_status_name(int status) {
    switch (status) {
    case QF_OK: return "QF_OK";
    case QF_ERR_ZERO_QUBITS: return "QF_ERR_ZERO_QUBITS";
    case QF_ERR_MEMORY_BUDGET_EXCEEDED: return "QF_ERR_MEMORY_BUDGET_EXCEEDED";
    case QF_ERR_SIMULATION_SIZE_OVERFLOW: return "QF_ERR_SIMULATION_SIZE_OVERFLOW";
    case QF_ERR_MEMORY_ALLOCATION_FAILED: return "QF_ERR_MEMORY_ALLOCATION_FAILED";
    case QF_ERR_STATE_SIZE_NOT_POWER_OF_TWO: return "QF_ERR_STATE_SIZE_NOT_POWER_OF_TWO";
    case QF_ERR_QUBIT_OUT_OF_RANGE: return "QF_ERR_QUBIT_OUT_OF_RANGE";
    case QF_ERR_INVALID_QUBIT_PAIR: return "QF_ERR_INVALID_QUBIT_PAIR";
    case QF_ERR_INVALID_PROBABILITY: return "QF_ERR_INVALID_PROBABILITY";
    case QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX: return "QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX";
    case QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION: return "QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION";
    case QF_ERR_INVALID_SHOT_COUNT: return "QF_ERR_INVALID_SHOT_COUNT";
    case QF_ERR_CLASSICAL_BIT_OUT_OF_RANGE: return "QF_ERR_CLASSICAL_BIT_OUT_OF_RANGE";
    case QF_ERR_INVALID_PARAMETER_COUNT: return "QF_ERR_INVALID_PARAMETER_COUNT";
    case QF_ERR_INVALID_INPUT_COUNT: return "QF_ERR_INVALID_INPUT_COUNT";
    case QF_ERR_NON_FINITE_PARAMETER: return "QF_ERR_NON_FINITE_PARAMETER";
    case QF_ERR_INVALID_FINITE_DIFFERENCE_STEP: return "QF_ERR_INVALID_FINITE_DIFFERENCE_STEP";
    case QF_ERR_UNSUPPORTED_OPERATION: return "QF_ERR_UNSUPPORTED_OPERATION";
    case QF_ERR_TIMEOUT: return "QF_ERR_TIMEOUT";
    case QF_ERR_CUDA: return "QF_ERR_CUDA";
    case QF_ERR_INVALID_ARGUMENT: return "QF_ERR_INVALID_ARGUMENT";
    case QF_ERR_EMPTY_BATCH: return "QF_ERR_EMPTY_BATCH";
    case QF_ERR_INCOMPATIBLE_BATCH: return "QF_ERR_INCOMPATIBLE_BATCH";
    case QF_ERR_STATE_TOO_LARGE: return "QF_ERR_STATE_TOO_LARGE";
    case QF_ERR_INCOMPATIBLE_DEVICE_STATE: return "QF_ERR_INCOMPATIBLE_DEVICE_STATE";
    default: return "QF_ERR_UNKNOWN";
    }
}

int qf_abi_version(void) { return QF_ABI_VERSION; }

int qf_ctx_create(int device, qf_ctx **out) {
    clear_error();
    if (!out) return fail(QF_ERR_INVALID_ARGUMENT, "out is NULL");
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= count) return fail(QF_ERR_CUDA, "CUDA device %d does not exist (%d visible)", device, count);
    QF_CUDA(cudaSetDevice(device));
    qf_ctx *ctx = new qf_ctx();
    ctx->device = device;
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    ctx->sm_count = v;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    ctx->smem_optin = (size_t)v;
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc(&ctx->d_small, kSmallBytes)) != cudaSuccess ||
        (e = cudaMallocHost(&ctx->h_small, kSmallBytes)) != cudaSuccess) {
        int st = cuda_fail(e, "qf_ctx_create");
        qf_ctx_destroy(ctx);
        return st;
    }
    *out = ctx;
    return QF_OK;
}

int qf_ctx_destroy(qf_ctx *ctx) {
    if (!ctx) return QF_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_state(ctx->scratch_sv);
    free_state(ctx->scratch_sv2);
    for (qf_sv *c : ctx->ckpt_pool) free_state(c);
    ctx->ckpt_pool.clear();
    // states the caller still holds: free their memory, keep the handle as an
    // orphan that qf_sv_destroy can release without the context
    for (qf_sv *sv : ctx->states) {
        if (sv->d) cudaFree(sv->d);
        sv->d = nullptr;
        sv->ctx = nullptr;
    }
    ctx->states.clear();
    if (ctx->ws_plan) cudaFree(ctx->ws_plan);
    if (ctx->ws_red) cudaFree(ctx->ws_red);
    if (ctx->ws_tree) cudaFree(ctx->ws_tree);
    if (ctx->ws_stage) cudaFree(ctx->ws_stage);
    if (ctx->d_small) cudaFree(ctx->d_small);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    if (ctx->host_pinned) cudaFreeHost(ctx->host_pinned);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return QF_OK;
}

int qf_ctx_synchronize(qf_ctx *ctx) {
    clear_error();
    if (!ctx) return fail(QF_ERR_INVALID_ARGUMENT, "context is NULL");
    QF_TRY(bind_device(ctx));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    return QF_OK;
}

int qf_ctx_stream(qf_ctx *ctx, void **stream_out) {
    if (!ctx || !stream_out) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    *stream_out = (void *)ctx->stream;
    return QF_OK;
}

int qf_sv_create(qf_ctx *ctx, uint32_t qubits, int dtype, uint64_t memory_budget_bytes, qf_sv **out) {
    clear_error();
    if (!ctx || !out) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    QF_TRY(bind_device(ctx));
    return alloc_state(ctx, qubits, dtype, memory_budget_bytes, out);
}

int qf_sv_destroy(qf_sv *sv) {
    if (!sv) return QF_OK;
    if (!sv->ctx) {  // orphaned by qf_ctx_destroy: memory already released
        delete sv;
        return QF_OK;
    }
    {
        cudaSetDevice(sv->ctx->device);
        cudaStreamSynchronize(sv->ctx->stream);
    }
    free_state(sv);
    return QF_OK;
}

int qf_sv_qubits(const qf_sv *sv, uint32_t *q) {
    QF_TRY(check_sv(sv));
    if (!q) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    *q = sv->n;
    return QF_OK;
}

int qf_sv_dtype(const qf_sv *sv, int *d) {
    QF_TRY(check_sv(sv));
    if (!d) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    *d = sv->dtype;
    return QF_OK;
}

int qf_sv_device_ptr(qf_sv *sv, void **p) {
    QF_TRY(check_sv(sv));
    if (!p) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    *p = sv->d;
    return QF_OK;
}

int qf_sv_set_zero(qf_sv *sv) {
    clear_error();
    QF_TRY(check_sv(sv));
    QF_TRY(bind_device(sv->ctx));
    return fill_zero_state(sv);
}

int qf_sv_upload(qf_sv *sv, const double *amps, uint64_t n_doubles) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!amps) return fail(QF_ERR_INVALID_ARGUMENT, "amplitudes are NULL");
    if (n_doubles != 2 * sv->dim)
        return fail(QF_ERR_STATE_SIZE_NOT_POWER_OF_TWO, "expected %llu doubles (2^%u complex amplitudes), got %llu",
                    (unsigned long long)(2 * sv->dim), sv->n, (unsigned long long)n_doubles);
    QF_TRY(bind_device(sv->ctx));
    QF_TRY(convert_from_f64(sv, amps));
    QF_CUDA(cudaStreamSynchronize(sv->ctx->stream));
    return QF_OK;
}

int qf_sv_download(qf_sv *sv, double *amps_out, uint64_t n_doubles) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!amps_out) return fail(QF_ERR_INVALID_ARGUMENT, "output is NULL");
    if (n_doubles != 2 * sv->dim)
        return fail(QF_ERR_INVALID_ARGUMENT, "expected %llu doubles, got %llu", (unsigned long long)(2 * sv->dim),
                    (unsigned long long)n_doubles);
    QF_TRY(bind_device(sv->ctx));
    return convert_to_f64(sv, amps_out);
}

int qf_sv_upload_raw(qf_sv *sv, const void *host, uint64_t bytes) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!host || bytes != sv->bytes()) return fail(QF_ERR_INVALID_ARGUMENT, "raw upload needs %zu bytes", sv->bytes());
    QF_TRY(bind_device(sv->ctx));
    QF_CUDA(cudaMemcpyAsync(sv->d, host, bytes, cudaMemcpyHostToDevice, sv->ctx->stream));
    QF_CUDA(cudaStreamSynchronize(sv->ctx->stream));
    return QF_OK;
}

int qf_sv_download_raw(qf_sv *sv, void *host_out, uint64_t bytes) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!host_out || bytes != sv->bytes()) return fail(QF_ERR_INVALID_ARGUMENT, "raw download needs %zu bytes", sv->bytes());
    QF_TRY(bind_device(sv->ctx));
    QF_CUDA(cudaMemcpyAsync(host_out, sv->d, bytes, cudaMemcpyDeviceToHost, sv->ctx->stream));
    QF_CUDA(cudaStreamSynchronize(sv->ctx->stream));
    return QF_OK;
}

int qf_sv_copy_from(qf_sv *dst, const qf_sv *src) {
    clear_error();
    QF_TRY(check_sv(dst));
    QF_TRY(check_sv(src));
    if (dst->n != src->n || dst->dtype != src->dtype || dst->ctx != src->ctx)
        return fail(QF_ERR_INCOMPATIBLE_DEVICE_STATE, "device states must share a backend and have equal dimensions");
    QF_TRY(bind_device(dst->ctx));
    QF_CUDA(cudaMemcpyAsync(dst->d, src->d, dst->bytes(), cudaMemcpyDeviceToDevice, dst->ctx->stream));
    return QF_OK;
}

int qf_sv_apply_gate(qf_sv *sv, int gate, double theta, uint32_t target) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (target >= sv->n)
        return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", target, sv->n);
    BGate g;
    QF_TRY(gate_matrix(gate, theta, g.m));
    g.kind = BK_MAT1;
    g.q0 = target;
    g.diag = matrix_is_diag(g.m);
    QF_TRY(bind_device(sv->ctx));
    return launch_gate1(sv, g);
}

static int apply_2q(qf_sv *sv, BKind kind, uint32_t a, uint32_t b) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (a >= sv->n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", a, sv->n);
    if (b >= sv->n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", b, sv->n);
    if (a == b) return fail(QF_ERR_INVALID_QUBIT_PAIR, "two-qubit operation requires distinct qubits, got %u and %u", a, b);
    BGate g;
    g.kind = kind;
    g.q0 = a;
    g.q1 = b;
    QF_TRY(bind_device(sv->ctx));
    return launch_gate2(sv, g);
}

int qf_sv_apply_cnot(qf_sv *sv, uint32_t c, uint32_t t) { return apply_2q(sv, BK_CNOT, c, t); }
int qf_sv_apply_cz(qf_sv *sv, uint32_t a, uint32_t b) { return apply_2q(sv, BK_CZ, a, b); }
int qf_sv_apply_swap(qf_sv *sv, uint32_t a, uint32_t b) { return apply_2q(sv, BK_SWAP, a, b); }

int qf_sv_apply_ops(qf_sv *sv, const qf_op *ops, uint64_t n_ops, const double *params, uint64_t n_params,
                    const double *inputs, uint64_t n_inputs, const qf_exec_opts *opts) {
    clear_error();
    QF_TRY(check_sv(sv));
    if ((n_params && !params) || (n_inputs && !inputs)) return fail(QF_ERR_INVALID_ARGUMENT, "parameter arrays are NULL");
    std::vector<BGate> gates;
    QF_TRY(bind_ops(sv->n, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, gates));
    QF_TRY(bind_device(sv->ctx));
    return execute_gates(sv, gates, opts);
}

int qf_sv_norm_sqr(qf_sv *sv, double *out) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!out) return fail(QF_ERR_INVALID_ARGUMENT, "output is NULL");
    QF_TRY(bind_device(sv->ctx));
    return reduce_norm_sqr(sv, out);
}

int qf_sv_probabilities(qf_sv *sv, double *out, uint64_t n_out) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!out || n_out != sv->dim) return fail(QF_ERR_INVALID_ARGUMENT, "probabilities need %llu outputs", (unsigned long long)sv->dim);
    QF_TRY(bind_device(sv->ctx));
    qf_ctx *ctx = sv->ctx;
    QF_TRY(ensure_device(&ctx->ws_stage, &ctx->ws_stage_bytes, sizeof(double) * sv->dim));
    QF_TRY(reduce_probabilities(sv, static_cast<double *>(ctx->ws_stage)));
    QF_CUDA(cudaMemcpyAsync(out, ctx->ws_stage, sizeof(double) * sv->dim, cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    return QF_OK;
}

int qf_sv_expectation_z_all(qf_sv *sv, double *out, uint64_t n_out) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!out || n_out != sv->n) return fail(QF_ERR_INVALID_ARGUMENT, "expectation_z_all needs %u outputs", sv->n);
    QF_TRY(bind_device(sv->ctx));
    return reduce_expect_z_all(sv, out);
}

int qf_sv_expectation(qf_sv *sv, int observable, uint32_t qubit, double *out) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!out) return fail(QF_ERR_INVALID_ARGUMENT, "output is NULL");
    if (observable < QF_PAULI_X || observable > QF_PAULI_Z) return fail(QF_ERR_INVALID_ARGUMENT, "unknown observable %d", observable);
    if (qubit >= sv->n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", qubit, sv->n);
    QF_TRY(bind_device(sv->ctx));
    return reduce_expect_1q(sv, observable, qubit, out);
}

int qf_sv_expectation_pauli_sum(qf_sv *sv, const qf_pauli_term *terms, uint64_t n_terms, double *out) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!out || (n_terms && !terms)) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    QF_TRY(bind_device(sv->ctx));
    return pauli_expectation(sv, terms, n_terms, out);
}

// StateVector::measure (src/lib.rs:1321-1351) with the uniform drawn on the
// host from the caller's SmallRng state, as CudaDeviceState::measure does.
int qf_sv_normalize(qf_sv *sv) {
    clear_error();
    QF_TRY(check_sv(sv));
    QF_TRY(bind_device(sv->ctx));
    QF_TRY(normalize_state(sv));
    QF_CUDA(cudaStreamSynchronize(sv->ctx->stream));
    return QF_OK;
}

int qf_sv_apply_channel_trajectory(qf_sv *sv, const qf_op *channel, uint64_t *rng_state, int *branch_out) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!channel || !rng_state) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    const qf_op &o = *channel;
    if (o.kind != QF_OP_CHANNEL) return fail(QF_ERR_INVALID_ARGUMENT, "operation is not a noise channel");
    const uint32_t q = o.q0;
    if (q >= sv->n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", q, sv->n);
    const double p = o.theta, eps = 2.220446049250313e-16;
    if (!valid_probability(p)) return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", p);
    double gu = 0.0;
    if (o.gate == QF_CHANNEL_THERMAL_DAMPING) {
        const double beta = qf_op_aux(&o);
        if (!std::isfinite(beta) || beta < 0.0) return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", beta);
        gu = p * std::exp(-beta);
    } else if (o.gate > QF_CHANNEL_THERMAL_DAMPING) {
        return fail(QF_ERR_INVALID_ARGUMENT, "unknown noise channel %u", (unsigned)o.gate);
    }
    QF_TRY(bind_device(sv->ctx));
    int branch = 0;
    BGate m;
    bool apply = true;
    if (o.gate == QF_CHANNEL_DEPOLARIZING) {
        const double u = next_uniform(rng_state);
        if (u >= 1.0 - p && p > 0.0) {
            const double b = std::floor((u - (1.0 - p)) * (3.0 / p));
            branch = 1 + (b >= 2.0 ? 2 : (int)b);
            m.kind = BK_MAT1;
            m.q0 = q;
            QF_TRY(gate_matrix(branch == 1 ? QF_GATE_X : branch == 2 ? QF_GATE_Y : QF_GATE_Z, 0.0, m.m));
            m.diag = matrix_is_diag(m.m);
        } else {
            apply = false;
        }
    } else {
        double norm, p_one;
        QF_TRY(reduce_norm_sqr(sv, &norm));
        if (!std::isfinite(norm) || norm <= eps) return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", norm);
        QF_TRY(reduce_p_one(sv, q, &p_one));
        double bn;
        if (o.gate != QF_CHANNEL_THERMAL_DAMPING) {
            const double jp = clamp01(p * p_one / norm);
            branch = next_uniform(rng_state) < jp ? 1 : 0;
            bn = branch ? p * p_one : norm - p * p_one;
            if (!std::isfinite(bn) || bn <= eps) return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", bn);
            const double inv = 1.0 / std::sqrt(bn);
            if (branch) m = o.gate == QF_CHANNEL_AMPLITUDE_DAMPING ? mat1(q, 0.0, std::sqrt(p) * inv, 0.0, 0.0)
                                                                    : mat1(q, 0.0, 0.0, 0.0, std::sqrt(p) * inv);
            else m = mat1(q, inv, 0.0, 0.0, std::sqrt(1.0 - p) * inv);
        } else {
            const double p1 = clamp01(p_one / norm), p0 = 1.0 - p1;
            const double down = p1 * p, up = p0 * gu, stay = p0 * (1.0 - gu) + p1 * (1.0 - p);
            const double u = next_uniform(rng_state);
            branch = u < down ? 1 : (u < down + up ? 2 : 0);
            bn = branch == 1 ? down : (branch == 2 ? up : stay);
            if (!std::isfinite(bn) || bn <= eps) return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", bn);
            const double inv = 1.0 / std::sqrt(bn);
            m = branch == 1 ? mat1(q, 0.0, std::sqrt(p) * inv, 0.0, 0.0)
                : branch == 2 ? mat1(q, 0.0, 0.0, std::sqrt(gu) * inv, 0.0)
                              : mat1(q, std::sqrt(1.0 - gu) * inv, 0.0, 0.0, std::sqrt(1.0 - p) * inv);
        }
    }
    if (apply) QF_TRY(launch_gate1(sv, m));
    QF_CUDA(cudaStreamSynchronize(sv->ctx->stream));
    if (branch_out) *branch_out = branch;
    return QF_OK;
}

int qf_sv_measure(qf_sv *sv, uint32_t qubit, uint64_t *rng_state, uint8_t *outcome) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (!rng_state || !outcome) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (qubit >= sv->n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", qubit, sv->n);
    QF_TRY(bind_device(sv->ctx));
    double p_one;
    QF_TRY(reduce_p_one(sv, qubit, &p_one));
    p_one = std::min(1.0, std::max(0.0, p_one));
    uint64_t x = *rng_state;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    *rng_state = x;
    const double u = (double)(x >> 11) * (1.0 / 9007199254740992.0);
    const uint8_t o = u < p_one ? 1 : 0;
    const double prob = o ? p_one : 1.0 - p_one;
    if (prob <= 2.220446049250313e-16)
        return fail(QF_ERR_INVALID_PROBABILITY, "measurement probability must be in [0, 1], got %g", prob);
    QF_TRY(collapse(sv, qubit, o, std::sqrt(prob)));
    *outcome = o;
    return QF_OK;
}

// ---- state batches (CudaDeviceStateBatch, src/cuda.rs:1486-1992) ------------
static int check_batch(const qf_batch *b) {
    if (!b || !b->sv || !b->sv->ctx || !b->sv->d) return fail(QF_ERR_INVALID_ARGUMENT, "batch handle is NULL or released");
    return QF_OK;
}

// The first size << n amplitudes of the batch allocation, as a state view for
// the f64 conversions.
static qf_sv batch_view(const qf_batch *b) {
    qf_sv v = *b->sv;
    v.dim = b->size << b->n;
    return v;
}

int qf_batch_create(qf_ctx *ctx, uint32_t qubits, int dtype, uint64_t batch_size, qf_batch **out) {
    clear_error();
    if (!ctx || !out) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    QF_TRY(check_dtype(dtype));
    if (batch_size == 0) return fail(QF_ERR_EMPTY_BATCH, "CUDA state batches must contain at least one state");
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    uint32_t extra = 0;
    while (extra < 63 && (1ULL << extra) < batch_size) ++extra;
    if ((uint64_t)qubits + extra > 40)
        return fail(QF_ERR_STATE_TOO_LARGE, "a batch of %llu states of %u qubits exceeds the supported device allocation",
                    (unsigned long long)batch_size, qubits);
    QF_TRY(bind_device(ctx));
    qf_sv *sv;
    QF_TRY(alloc_state(ctx, qubits + extra, dtype, 0, &sv));
    const int st = batch_set_zero(sv, qubits, batch_size);
    if (st) {
        free_state(sv);
        return st;
    }
    *out = new qf_batch{sv, qubits, batch_size};
    return QF_OK;
}

int qf_batch_destroy(qf_batch *batch) {
    if (!batch) return QF_OK;
    if (batch->sv) qf_sv_destroy(batch->sv);
    delete batch;
    return QF_OK;
}

int qf_batch_qubits(const qf_batch *batch, uint32_t *qubits_out) {
    QF_TRY(check_batch(batch));
    if (!qubits_out) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    *qubits_out = batch->n;
    return QF_OK;
}

int qf_batch_size(const qf_batch *batch, uint64_t *size_out) {
    QF_TRY(check_batch(batch));
    if (!size_out) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    *size_out = batch->size;
    return QF_OK;
}

int qf_batch_upload(qf_batch *batch, const double *amps, uint64_t n_doubles) {
    clear_error();
    QF_TRY(check_batch(batch));
    if (!amps) return fail(QF_ERR_INVALID_ARGUMENT, "amplitudes are NULL");
    qf_sv v = batch_view(batch);
    if (n_doubles != 2 * v.dim)
        return fail(QF_ERR_INCOMPATIBLE_BATCH, "expected %llu doubles (%llu states of 2^%u amplitudes), got %llu",
                    (unsigned long long)(2 * v.dim), (unsigned long long)batch->size, batch->n, (unsigned long long)n_doubles);
    QF_TRY(bind_device(v.ctx));
    QF_TRY(convert_from_f64(&v, amps));
    QF_CUDA(cudaStreamSynchronize(v.ctx->stream));
    return QF_OK;
}

int qf_batch_download(qf_batch *batch, double *amps_out, uint64_t n_doubles) {
    clear_error();
    QF_TRY(check_batch(batch));
    if (!amps_out) return fail(QF_ERR_INVALID_ARGUMENT, "output is NULL");
    qf_sv v = batch_view(batch);
    if (n_doubles != 2 * v.dim)
        return fail(QF_ERR_INVALID_ARGUMENT, "expected %llu doubles, got %llu", (unsigned long long)(2 * v.dim),
                    (unsigned long long)n_doubles);
    QF_TRY(bind_device(v.ctx));
    return convert_to_f64(&v, amps_out);
}

int qf_batch_copy_from(qf_batch *dst, const qf_batch *src) {
    clear_error();
    QF_TRY(check_batch(dst));
    QF_TRY(check_batch(src));
    if (dst->n != src->n || dst->size != src->size || dst->sv->dtype != src->sv->dtype || dst->sv->ctx != src->sv->ctx)
        return fail(QF_ERR_INCOMPATIBLE_DEVICE_STATE, "device states must share a backend and have equal dimensions");
    QF_TRY(bind_device(dst->sv->ctx));
    QF_CUDA(cudaMemcpyAsync(dst->sv->d, src->sv->d, dst->sv->bytes(), cudaMemcpyDeviceToDevice, dst->sv->ctx->stream));
    QF_CUDA(cudaStreamSynchronize(dst->sv->ctx->stream));
    return QF_OK;
}

int qf_batch_apply_ops(qf_batch *batch, const qf_op *ops, uint64_t n_ops, const qf_exec_opts *opts) {
    clear_error();
    QF_TRY(check_batch(batch));
    if (n_ops && !ops) return fail(QF_ERR_INVALID_ARGUMENT, "ops is NULL");
    std::vector<BGate> gates;
    QF_TRY(bind_ops(batch->n, ops, n_ops, nullptr, 0, nullptr, 0, -1, 0.0, gates));
    QF_TRY(bind_device(batch->sv->ctx));
    return execute_gates(batch->sv, gates, opts);
}

int qf_batch_measure(qf_batch *batch, uint32_t qubit, uint64_t *rng_state, uint8_t *outcomes) {
    clear_error();
    QF_TRY(check_batch(batch));
    if (!rng_state || !outcomes) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (qubit >= batch->n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", qubit, batch->n);
    std::vector<double> u(batch->size);
    for (uint64_t b = 0; b < batch->size; ++b) u[b] = next_uniform(rng_state);
    QF_TRY(bind_device(batch->sv->ctx));
    return batch_measure(batch->sv, batch->n, batch->size, qubit, u.data(), outcomes);
}

int qf_run_circuit_batch(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *in_amps,
                         uint64_t batch_size, double *out_amps, uint64_t n_doubles, const qf_exec_opts *opts) {
    clear_error();
    if (!ctx || !in_amps || !out_amps || (n_ops && !ops)) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (batch_size == 0) return fail(QF_ERR_EMPTY_BATCH, "CUDA state batches must contain at least one state");
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    if (qubits > 40 || batch_size > (1ULL << (40 - qubits)))
        return fail(QF_ERR_STATE_TOO_LARGE, "a batch of %llu states of %u qubits exceeds the supported device allocation",
                    (unsigned long long)batch_size, qubits);
    if (n_doubles != 2 * (batch_size << qubits))
        return fail(QF_ERR_INCOMPATIBLE_BATCH, "expected %llu doubles, got %llu",
                    (unsigned long long)(2 * (batch_size << qubits)), (unsigned long long)n_doubles);
    std::vector<BGate> gates;
    QF_TRY(bind_ops(qubits, ops, n_ops, nullptr, 0, nullptr, 0, -1, 0.0, gates));  // validated before any allocation
    qf_batch *b;
    QF_TRY(qf_batch_create(ctx, qubits, dtype, batch_size, &b));
    struct Release {
        qf_batch *b;
        ~Release() { qf_batch_destroy(b); }
    } release{b};
    qf_sv v = batch_view(b);
    QF_TRY(convert_from_f64(&v, in_amps));
    QF_TRY(execute_gates(b->sv, gates, opts));
    return convert_to_f64(&v, out_amps);
}

// ---- density matrices (DensityMatrix, src/lib.rs:1551-2235) ----------------
}  // extern "C"

namespace {

// One step of a density-matrix op list: a run of 2n-qubit gates for the fused
// engine, or one local channel.
struct DmStep {
    bool channel = false;
    std::vector<BGate> gates;
    uint32_t q = 0;
    double coef[6] = {0, 0, 0, 0, 0, 0};
};

int check_dm(const qf_dm *dm) {
    if (!dm || !dm->sv || !dm->sv->ctx || !dm->sv->d) return fail(QF_ERR_INVALID_ARGUMENT, "density handle is NULL or released");
    return QF_OK;
}

// U rho U^dagger on an n-qubit density matrix = U on row bit n + q and conj(U)
// on column bit q; CNOT/CZ/SWAP permute or sign both sides (apply_basis_permutation,
// src/lib.rs:2033-2041).
void lower_to_density(const BGate &g, uint32_t n, std::vector<BGate> &out) {
    BGate row = g, col = g;
    row.op_index = col.op_index = -1;
    row.param = col.param = -1;
    row.axis = col.axis = 255;
    row.q0 = g.q0 + n;
    if (g.kind == BK_MAT1) {
        for (int k = 0; k < 4; ++k) col.m[2 * k + 1] = -g.m[2 * k + 1];
    } else {
        row.q1 = g.q1 + n;
    }
    out.push_back(row);
    out.push_back(col);
}

// apply_channel (src/lib.rs:2056-2143) as the real superoperator of the
// channel on (row bit, column bit): populations mix, coherences scale.
int channel_coefficients(const qf_op &o, double coef[6]) {
    const double p = o.theta;
    auto bad = [](double v) { return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", v); };
    switch (o.gate) {
    case QF_CHANNEL_DEPOLARIZING: {  // (1-p) rho + p/3 (X rho X + Y rho Y + Z rho Z)
        if (!valid_probability(p)) return bad(p);
        const double t = p / 3.0;
        coef[0] = coef[3] = (1.0 - p) + t;
        coef[1] = coef[2] = t + t;
        coef[4] = coef[5] = (1.0 - p) - t;
        return QF_OK;
    }
    case QF_CHANNEL_AMPLITUDE_DAMPING:
        if (!valid_probability(p)) return bad(p);
        coef[0] = 1.0, coef[1] = p, coef[2] = 0.0, coef[3] = 1.0 - p;
        coef[4] = coef[5] = std::sqrt(1.0 - p);
        return QF_OK;
    case QF_CHANNEL_PHASE_DAMPING:
        if (!valid_probability(p)) return bad(p);
        coef[0] = 1.0, coef[1] = 0.0, coef[2] = 0.0, coef[3] = 1.0;
        coef[4] = coef[5] = std::sqrt(1.0 - p);
        return QF_OK;
    case QF_CHANNEL_THERMAL_DAMPING: {
        const double beta = qf_op_aux(&o);
        if (!valid_probability(p)) return bad(p);
        if (!std::isfinite(beta) || beta < 0.0) return bad(beta);
        const double gu = p * std::exp(-beta);  // NoiseChannel::thermal_rates (src/lib.rs:1611-1626)
        coef[0] = 1.0 - gu, coef[1] = p, coef[2] = gu, coef[3] = 1.0 - p;
        coef[4] = coef[5] = std::sqrt(1.0 - gu) * std::sqrt(1.0 - p);
        return QF_OK;
    }
    default:
        return fail(QF_ERR_INVALID_ARGUMENT, "unknown noise channel %u", (unsigned)o.gate);
    }
}

// Parameterised lists (rotations, encodings; ParameterizedCircuit::
// run_density_with_shift, src/lib.rs:4742-4806) bind their angles from
// params/inputs, with `shift` added to op `shift_op`.
int lower_density_ops(uint32_t n, const qf_op *ops, uint64_t n_ops, std::vector<DmStep> &steps, const double *params = nullptr,
                      uint64_t n_params = 0, const double *inputs = nullptr, uint64_t n_inputs = 0, int64_t shift_op = -1,
                      double shift = 0.0) {
    std::vector<qf_op> run;
    uint64_t run_start = 0;
    auto close_run = [&]() -> int {
        if (run.empty()) return QF_OK;
        std::vector<BGate> g;
        const int64_t local = shift_op >= (int64_t)run_start && shift_op < (int64_t)(run_start + run.size())
                                  ? shift_op - (int64_t)run_start
                                  : -1;
        QF_TRY(bind_ops(n, run.data(), run.size(), params, n_params, inputs, n_inputs, local, shift, g));
        DmStep st;
        for (const BGate &x : g) lower_to_density(x, n, st.gates);
        steps.push_back(std::move(st));
        run.clear();
        return QF_OK;
    };
    for (uint64_t k = 0; k < n_ops; ++k) {
        if (ops[k].kind != QF_OP_CHANNEL) {
            if (run.empty()) run_start = k;
            run.push_back(ops[k]);
            continue;
        }
        QF_TRY(close_run());
        if (ops[k].q0 >= n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", ops[k].q0, n);
        DmStep st;
        st.channel = true;
        st.q = ops[k].q0;
        QF_TRY(channel_coefficients(ops[k], st.coef));
        steps.push_back(std::move(st));
    }
    return close_run();
}

// Complex64: consecutive channels go through one fused sweep while their
// (row, column) bit pairs and the low five column bits fit a 12-bit tile (the
// single-channel kernel is HBM-bound there). Complex128 channels are bound by
// the FP64 pipe, which fusing does not relieve: one kernel per channel, as for
// a lone channel or a matrix under 3 qubits.
int run_density_steps(qf_sv *sv, uint32_t n, const std::vector<DmStep> &steps, const qf_exec_opts *opts) {
    // a run of consecutive channels cut into groups (in order) whose bit pairs
    // plus the low five column bits fit 12 tile bits, at most `cap` channels each
    auto group_run = [&](size_t b, size_t e, size_t cap) {
        std::vector<std::pair<size_t, size_t>> g;
        for (size_t i = b; i < e;) {
            uint64_t mask = 31;
            size_t j = i;
            while (j < e && j - i < cap) {
                const uint64_t m = mask | (1ULL << steps[j].q) | (1ULL << (n + steps[j].q));
                if (__builtin_popcountll(m) > 12) break;
                mask = m;
                ++j;
            }
            if (j == i) j = i + 1;
            g.emplace_back(i, j);
            i = j;
        }
        return g;
    };
    for (size_t i = 0; i < steps.size();) {
        if (!steps[i].channel) {
            QF_TRY(execute_gates(sv, steps[i].gates, opts));
            ++i;
            continue;
        }
        size_t e = i;
        while (e < steps.size() && steps[e].channel) ++e;
        if (n < 3 || sv->dtype != QF_C64) {
            for (; i < e; ++i) QF_TRY(dm_channel(sv, n, steps[i].q, steps[i].coef));
            continue;
        }
        // as many sweeps as the widest grouping needs, with the channels spread
        // evenly over them (for complex64 the sweeps apply two channels per
        // shared-memory round, so a sweep's time hardly depends on its count)
        auto groups = group_run(i, e, 12);
        const size_t cap = (e - i + groups.size() - 1) / groups.size();
        auto even = group_run(i, e, cap);
        if (even.size() <= groups.size()) groups.swap(even);
        for (const auto &gr : groups) {
            if (gr.second - gr.first >= 2) {
                std::vector<uint32_t> qs;
                std::vector<std::array<double, 6>> cf;
                for (size_t k = gr.first; k < gr.second; ++k) {
                    qs.push_back(steps[k].q);
                    std::array<double, 6> c;
                    std::copy(steps[k].coef, steps[k].coef + 6, c.begin());
                    cf.push_back(c);
                }
                QF_TRY(dm_channels_fused(sv, n, qs.data(), reinterpret_cast<const double(*)[6]>(cf.data()),
                                         (uint32_t)qs.size()));
            } else {
                QF_TRY(dm_channel(sv, n, steps[gr.first].q, steps[gr.first].coef));
            }
        }
        i = e;
    }
    return QF_OK;
}

int check_dm_qubits(uint32_t qubits) {
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    if (qubits > 17) return fail(QF_ERR_STATE_TOO_LARGE, "density matrices of %u qubits exceed the supported allocation", qubits);
    return QF_OK;
}

}  // namespace

extern "C" {

int qf_dm_create(qf_ctx *ctx, uint32_t qubits, int dtype, qf_dm **out) {
    clear_error();
    if (!ctx || !out) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    QF_TRY(check_dtype(dtype));
    QF_TRY(check_dm_qubits(qubits));
    QF_TRY(bind_device(ctx));
    qf_sv *sv;
    QF_TRY(alloc_state(ctx, 2 * qubits, dtype, 0, &sv));  // entry 0 = 1: |0...0><0...0|
    *out = new qf_dm{sv, qubits};
    return QF_OK;
}

int qf_dm_destroy(qf_dm *dm) {
    if (!dm) return QF_OK;
    if (dm->sv) qf_sv_destroy(dm->sv);
    delete dm;
    return QF_OK;
}

int qf_dm_qubits(const qf_dm *dm, uint32_t *qubits_out) {
    QF_TRY(check_dm(dm));
    if (!qubits_out) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    *qubits_out = dm->n;
    return QF_OK;
}

int qf_dm_upload(qf_dm *dm, const double *entries, uint64_t n_doubles) {
    clear_error();
    QF_TRY(check_dm(dm));
    if (!entries) return fail(QF_ERR_INVALID_ARGUMENT, "entries are NULL");
    if (n_doubles != 2 * dm->sv->dim)
        return fail(QF_ERR_STATE_TOO_LARGE, "expected %llu doubles (4^%u complex entries), got %llu",
                    (unsigned long long)(2 * dm->sv->dim), dm->n, (unsigned long long)n_doubles);
    QF_TRY(bind_device(dm->sv->ctx));
    QF_TRY(convert_from_f64(dm->sv, entries));
    QF_CUDA(cudaStreamSynchronize(dm->sv->ctx->stream));
    return QF_OK;
}

int qf_dm_download(qf_dm *dm, double *entries_out, uint64_t n_doubles) {
    clear_error();
    QF_TRY(check_dm(dm));
    if (!entries_out || n_doubles != 2 * dm->sv->dim)
        return fail(QF_ERR_INVALID_ARGUMENT, "download needs %llu doubles", (unsigned long long)(2 * dm->sv->dim));
    QF_TRY(bind_device(dm->sv->ctx));
    return convert_to_f64(dm->sv, entries_out);
}

int qf_dm_from_state(qf_dm *dm, const qf_sv *psi) {
    clear_error();
    QF_TRY(check_dm(dm));
    QF_TRY(check_sv(psi));
    if (psi->n != dm->n || psi->dtype != dm->sv->dtype || psi->ctx != dm->sv->ctx)
        return fail(QF_ERR_INCOMPATIBLE_DEVICE_STATE, "state and density matrix must share a backend, width and dtype");
    QF_TRY(bind_device(dm->sv->ctx));
    return dm_from_state(dm->sv, dm->n, psi);
}

int qf_dm_set_maximally_mixed(qf_dm *dm) {
    clear_error();
    QF_TRY(check_dm(dm));
    QF_TRY(bind_device(dm->sv->ctx));
    return dm_maximally_mixed(dm->sv, dm->n);
}

int qf_dm_apply_ops(qf_dm *dm, const qf_op *ops, uint64_t n_ops, const qf_exec_opts *opts) {
    clear_error();
    QF_TRY(check_dm(dm));
    if (n_ops && !ops) return fail(QF_ERR_INVALID_ARGUMENT, "ops is NULL");
    std::vector<DmStep> steps;
    QF_TRY(lower_density_ops(dm->n, ops, n_ops, steps));
    QF_TRY(bind_device(dm->sv->ctx));
    return run_density_steps(dm->sv, dm->n, steps, opts);
}

int qf_dm_trace(qf_dm *dm, double out[2]) {
    clear_error();
    QF_TRY(check_dm(dm));
    if (!out) return fail(QF_ERR_INVALID_ARGUMENT, "output is NULL");
    QF_TRY(bind_device(dm->sv->ctx));
    return dm_diag_reduce(dm->sv, dm->n, 0, 0, out);
}

int qf_dm_purity(qf_dm *dm, double *out) {
    clear_error();
    QF_TRY(check_dm(dm));
    if (!out) return fail(QF_ERR_INVALID_ARGUMENT, "output is NULL");
    QF_TRY(bind_device(dm->sv->ctx));
    return reduce_norm_sqr(dm->sv, out);  // sum |rho_ij|^2
}

int qf_dm_expectation(qf_dm *dm, int observable, uint32_t qubit, double *out) {
    clear_error();
    QF_TRY(check_dm(dm));
    if (!out) return fail(QF_ERR_INVALID_ARGUMENT, "output is NULL");
    if (qubit >= dm->n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", qubit, dm->n);
    const int mode = observable == QF_PAULI_Z ? 2 : observable == QF_PAULI_X ? 3 : observable == QF_PAULI_Y ? 4 : -1;
    if (mode < 0) return fail(QF_ERR_INVALID_ARGUMENT, "unknown observable %d", observable);
    QF_TRY(bind_device(dm->sv->ctx));
    double r[2];
    QF_TRY(dm_diag_reduce(dm->sv, dm->n, qubit, mode, r));
    *out = r[0];
    return QF_OK;
}

int qf_dm_probability_one(qf_dm *dm, uint32_t qubit, double *out) {
    clear_error();
    QF_TRY(check_dm(dm));
    if (!out) return fail(QF_ERR_INVALID_ARGUMENT, "output is NULL");
    if (qubit >= dm->n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", qubit, dm->n);
    QF_TRY(bind_device(dm->sv->ctx));
    double r[2];
    QF_TRY(dm_diag_reduce(dm->sv, dm->n, qubit, 1, r));
    *out = clamp01(r[0]);
    return QF_OK;
}

int qf_dm_probabilities(qf_dm *dm, double *out, uint64_t n_out) {
    clear_error();
    QF_TRY(check_dm(dm));
    const uint64_t D = 1ULL << dm->n;
    if (!out || n_out != D) return fail(QF_ERR_INVALID_ARGUMENT, "probabilities need %llu outputs", (unsigned long long)D);
    qf_ctx *ctx = dm->sv->ctx;
    QF_TRY(bind_device(ctx));
    QF_TRY(ensure_device(&ctx->ws_stage, &ctx->ws_stage_bytes, sizeof(double) * D));
    QF_TRY(dm_diagonal(dm->sv, dm->n, static_cast<double *>(ctx->ws_stage)));
    QF_CUDA(cudaMemcpyAsync(out, ctx->ws_stage, sizeof(double) * D, cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    return QF_OK;
}

int qf_dm_measure(qf_dm *dm, uint32_t qubit, uint64_t *rng_state, uint8_t *outcome) {
    clear_error();
    QF_TRY(check_dm(dm));
    if (!rng_state || !outcome) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (qubit >= dm->n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", qubit, dm->n);
    QF_TRY(bind_device(dm->sv->ctx));
    double r[2];
    QF_TRY(dm_diag_reduce(dm->sv, dm->n, qubit, 1, r));
    const double p_one = clamp01(r[0]);
    const uint8_t o = next_uniform(rng_state) < p_one ? 1 : 0;
    const double prob = o ? p_one : 1.0 - p_one;
    if (prob <= 2.220446049250313e-16)
        return fail(QF_ERR_INVALID_PROBABILITY, "measurement probability must be in [0, 1], got %g", prob);
    QF_TRY(dm_collapse(dm->sv, dm->n, qubit, o, prob));
    QF_CUDA(cudaStreamSynchronize(dm->sv->ctx->stream));
    *outcome = o;
    return QF_OK;
}

// ParameterizedCircuit::run_density_with_shift from |0...0><0...0| and the
// expectation of one Pauli on one qubit (expectation_density_with_inputs,
// src/lib.rs:3175-3186), on the context's scratch matrix.
static int density_expectation(qf_ctx *ctx, uint32_t n, int dtype, const qf_op *ops, uint64_t n_ops, const double *params,
                               uint64_t n_params, const double *inputs, uint64_t n_inputs, int64_t shift_op, double shift,
                               int mode, uint32_t q, const qf_exec_opts *opts, double *out) {
    std::vector<DmStep> steps;
    QF_TRY(lower_density_ops(n, ops, n_ops, steps, params, n_params, inputs, n_inputs, shift_op, shift));
    qf_sv *sv;
    QF_TRY(scratch_state(ctx, &ctx->scratch_sv, 2 * n, dtype, &sv));
    QF_TRY(fill_zero_state(sv));
    QF_TRY(run_density_steps(sv, n, steps, opts));
    double r[2];
    QF_TRY(dm_diag_reduce(sv, n, q, mode, r));
    *out = r[0];
    return QF_OK;
}

static int density_checks(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *params,
                          uint64_t n_params, const double *inputs, uint64_t n_inputs, int observable, uint32_t q, int *mode) {
    if (!ctx || (n_ops && !ops) || (n_params && !params) || (n_inputs && !inputs)) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    QF_TRY(check_dtype(dtype));
    QF_TRY(check_dm_qubits(qubits));
    for (uint64_t i = 0; i < n_params; ++i)
        if (!std::isfinite(params[i])) return fail(QF_ERR_NON_FINITE_PARAMETER, "parameter %llu is not finite", (unsigned long long)i);
    for (uint64_t i = 0; i < n_inputs; ++i)
        if (!std::isfinite(inputs[i])) return fail(QF_ERR_NON_FINITE_PARAMETER, "input %llu is not finite", (unsigned long long)i);
    if (q >= qubits) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", q, qubits);
    *mode = observable == QF_PAULI_Z ? 2 : observable == QF_PAULI_X ? 3 : observable == QF_PAULI_Y ? 4 : -1;
    if (*mode < 0) return fail(QF_ERR_INVALID_ARGUMENT, "unknown observable %d", observable);
    return QF_OK;
}

int qf_expectation_density(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *params,
                           uint64_t n_params, const double *inputs, uint64_t n_inputs, int observable, uint32_t observable_qubit,
                           const qf_exec_opts *opts, double *expectation) {
    clear_error();
    if (!expectation) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    int mode;
    QF_TRY(density_checks(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, observable, observable_qubit, &mode));
    QF_TRY(bind_device(ctx));
    return density_expectation(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, mode,
                               observable_qubit, opts, expectation);
}

// ParameterizedCircuit::parameter_shift_gradient_density_with_inputs
// (src/lib.rs:3235-3266): every rotation occurrence shifted by +-pi/2 through
// the density-matrix path, g[param] += (E+ - E-) / 2.
// Per rotation occurrence k: g[p_k] += (E(+pi/2 at k) - E(-pi/2 at k)) / 2 on
// the density matrix. With shots > 0 each E goes through sample_expectation
// with seed + 2k and seed + 2k + 1 (src/lib.rs:3268-3320).
static int density_shift_gradient(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                                  const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                                  int observable, uint32_t observable_qubit, const qf_exec_opts *opts, uint64_t shots,
                                  uint64_t seed, double *expectation, double *gradient) {
    clear_error();
    if (n_params && !gradient) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    int mode;
    QF_TRY(density_checks(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, observable, observable_qubit, &mode));
    QF_TRY(bind_device(ctx));
    std::vector<double> g(n_params, 0.0);
    double e;
    QF_TRY(density_expectation(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, mode,
                               observable_qubit, opts, &e));  // also validates the whole list before any shift runs
    const double shift = 1.5707963267948966;  // FRAC_PI_2
    for (uint64_t k = 0; k < n_ops; ++k) {
        if (ops[k].kind != QF_OP_ROTATION) continue;
        double plus, minus;
        QF_TRY(density_expectation(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, shift, mode,
                                   observable_qubit, opts, &plus));
        QF_TRY(density_expectation(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, -shift, mode,
                                   observable_qubit, opts, &minus));
        if (shots) {
            const uint64_t occ_seed = seed + 2 * k;
            QF_TRY(qf_sample_expectation(plus, shots, occ_seed, &plus, nullptr));
            QF_TRY(qf_sample_expectation(minus, shots, occ_seed + 1, &minus, nullptr));
        }
        g[ops[k].param] += 0.5 * (plus - minus);
    }
    if (expectation) *expectation = e;
    std::copy(g.begin(), g.end(), gradient);
    return QF_OK;
}

int qf_parameter_shift_gradient_density(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                                        const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                                        int observable, uint32_t observable_qubit, const qf_exec_opts *opts,
                                        double *expectation, double *gradient) {
    return density_shift_gradient(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, observable,
                                  observable_qubit, opts, 0, 0, expectation, gradient);
}

// ParameterizedCircuit::parameter_shift_gradient_density_with_inputs_shots (src/lib.rs:3268-3320).
int qf_parameter_shift_gradient_density_shots(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                                              const double *params, uint64_t n_params, const double *inputs,
                                              uint64_t n_inputs, int observable, uint32_t observable_qubit,
                                              uint64_t shots, uint64_t seed, const qf_exec_opts *opts, double *gradient) {
    clear_error();
    if (shots == 0) return fail(QF_ERR_INVALID_SHOT_COUNT, "shot count must be greater than zero");
    return density_shift_gradient(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, observable,
                                  observable_qubit, opts, shots, seed, nullptr, gradient);
}

int qf_run_density_circuit(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *in_entries,
                           double *out_entries, uint64_t n_doubles, const qf_exec_opts *opts) {
    clear_error();
    if (!ctx || !in_entries || !out_entries || (n_ops && !ops)) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    QF_TRY(check_dtype(dtype));
    QF_TRY(check_dm_qubits(qubits));
    if (n_doubles != 2 * (1ULL << (2 * qubits)))
        return fail(QF_ERR_STATE_TOO_LARGE, "expected %llu doubles (4^%u complex entries), got %llu",
                    (unsigned long long)(2 * (1ULL << (2 * qubits))), qubits, (unsigned long long)n_doubles);
    std::vector<DmStep> steps;
    QF_TRY(lower_density_ops(qubits, ops, n_ops, steps));
    QF_TRY(bind_device(ctx));
    qf_sv *sv;
    QF_TRY(scratch_state(ctx, &ctx->scratch_sv, 2 * qubits, dtype, &sv));
    QF_TRY(convert_from_f64(sv, in_entries));
    QF_TRY(run_density_steps(sv, qubits, steps, opts));
    return convert_to_f64(sv, out_entries);
}

int qf_run_circuit(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *init_amps,
                   double *out_amps, uint64_t n_doubles, const qf_exec_opts *opts) {
    clear_error();
    if (!ctx) return fail(QF_ERR_INVALID_ARGUMENT, "context is NULL");
    QF_TRY(check_dtype(dtype));
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    if (qubits > 40) return fail(QF_ERR_SIMULATION_SIZE_OVERFLOW, "dense simulation size exceeds the supported addressable range");
    if ((init_amps || out_amps) && n_doubles != (2ULL << qubits))
        return fail(QF_ERR_STATE_SIZE_NOT_POWER_OF_TWO, "expected %llu doubles", (unsigned long long)(2ULL << qubits));
    std::vector<BGate> gates;
    QF_TRY(bind_ops(qubits, ops, n_ops, nullptr, 0, nullptr, 0, -1, 0.0, gates));
    QF_TRY(bind_device(ctx));
    qf_sv *sv;
    QF_TRY(scratch_state(ctx, &ctx->scratch_sv, qubits, dtype, &sv));
    if (init_amps) QF_TRY(convert_from_f64(sv, init_amps));
    else QF_TRY(fill_zero_state(sv));
    QF_TRY(execute_gates(sv, gates, opts));
    if (out_amps) return convert_to_f64(sv, out_amps);
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    return QF_OK;
}

int qf_sv_sample(qf_sv *sv, const uint32_t *qubit_order, const uint32_t *classical_bits, uint32_t m, uint64_t shots,
                 uint64_t seed, double tie_eps, uint64_t *outcomes, uint64_t *n_ties) {
    clear_error();
    QF_TRY(check_sv(sv));
    if (shots == 0) return fail(QF_ERR_INVALID_SHOT_COUNT, "shot count must be greater than zero");
    if (m && (!qubit_order || !classical_bits)) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    for (uint32_t j = 0; j < m; ++j)
        if (classical_bits[j] >= 4096)
            return fail(QF_ERR_CLASSICAL_BIT_OUT_OF_RANGE, "classical bit index %u exceeds the supported maximum of 4095", classical_bits[j]);
    QF_TRY(bind_device(sv->ctx));
    return sample_shots(sv, qubit_order, classical_bits, m, shots, seed, tie_eps, outcomes, n_ties);
}

int qf_run_shots(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *init_amps,
                 uint64_t shots, uint64_t seed, double tie_eps, uint64_t *outcomes, uint32_t *classical_width,
                 uint64_t *n_ties, const qf_exec_opts *opts) {
    return run_shots_entry(ctx, qubits, dtype, ops, n_ops, init_amps, shots, seed, tie_eps, false, outcomes, classical_width,
                           n_ties, opts);
}

int qf_run_shots_with_noise(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                            const double *init_amps, uint64_t shots, uint64_t seed, double tie_eps, uint64_t *outcomes,
                            uint32_t *classical_width, uint64_t *n_ties, const qf_exec_opts *opts) {
    return run_shots_entry(ctx, qubits, dtype, ops, n_ops, init_amps, shots, seed, tie_eps, true, outcomes, classical_width,
                           n_ties, opts);
}

int qf_expectation(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *params,
                   uint64_t n_params, const double *inputs, uint64_t n_inputs, const qf_pauli_term *terms, uint64_t n_terms,
                   const qf_exec_opts *opts, double *expectation) {
    clear_error();
    if (!ctx || !expectation) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    QF_TRY(check_dtype(dtype));
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    if (n_terms && !terms) return fail(QF_ERR_INVALID_ARGUMENT, "terms is NULL");
    QF_TRY(bind_device(ctx));
    return forward_expectation(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, terms, n_terms,
                               opts, expectation);
}

// estimate_observable_shots (src/lib.rs:4806-4838) on the state the op list
// prepares (with `shift` on op `shift_op`): the measured basis rotated (X: H;
// Y: Rz(-pi/2) then H), P(1) of the qubit reduced once, then `shots` draws of
// SmallRng::seeded(seed) compared against it (each clone-and-measure of the
// reference draws one uniform against the same P(1)); *successes counts
// outcome 0. Draws within tie_eps of P(1) are counted.
static int shots_estimate(qf_ctx *ctx, uint32_t n, int dtype, const qf_op *ops, uint64_t n_ops, const double *params,
                          uint64_t n_params, const double *inputs, uint64_t n_inputs, int64_t shift_op, double shift,
                          int observable, uint32_t q, uint64_t shots, uint64_t seed, double tie_eps,
                          const qf_exec_opts *opts, uint64_t *successes, uint64_t *ties) {
    std::vector<BGate> gates;
    QF_TRY(bind_ops(n, ops, n_ops, params, n_params, inputs, n_inputs, shift_op, shift, gates));
    auto add = [&](int gate, double theta) -> int {
        BGate g;
        g.kind = BK_MAT1;
        g.q0 = q;
        QF_TRY(gate_matrix(gate, theta, g.m));
        g.diag = matrix_is_diag(g.m);
        gates.push_back(g);
        return QF_OK;
    };
    if (observable == QF_PAULI_X) QF_TRY(add(QF_GATE_H, 0.0));
    if (observable == QF_PAULI_Y) {
        QF_TRY(add(QF_GATE_RZ, -1.5707963267948966));
        QF_TRY(add(QF_GATE_H, 0.0));
    }
    qf_sv *sv;
    QF_TRY(scratch_state(ctx, &ctx->scratch_sv, n, dtype, &sv));
    QF_TRY(fill_zero_state(sv));
    QF_TRY(execute_gates(sv, gates, opts));
    double p1;
    QF_TRY(reduce_p_one(sv, q, &p1));
    p1 = clamp01(p1);
    uint64_t x = smallrng_seeded(seed), ok = 0, t = 0;
    for (uint64_t k = 0; k < shots; ++k) {
        const double u = next_uniform(&x);
        const int o = u < p1 ? 1 : 0;
        if (std::fabs(u - p1) < tie_eps) ++t;
        const double prob = o ? p1 : 1.0 - p1;
        if (prob <= 2.220446049250313e-16)
            return fail(QF_ERR_INVALID_PROBABILITY, "measurement probability must be in [0, 1], got %g", prob);
        ok += o == 0;
    }
    *successes = ok;
    if (ties) *ties += t;
    return QF_OK;
}

int qf_sample_expectation(double expectation, uint64_t shots, uint64_t seed, double *estimate, uint64_t *positive) {
    if (!estimate) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (shots == 0) return fail(QF_ERR_INVALID_SHOT_COUNT, "shot count must be greater than zero");
    const double p = clamp01((1.0 + expectation) * 0.5);
    uint64_t x = smallrng_seeded(seed), k = 0;
    for (uint64_t s = 0; s < shots; ++s) k += next_uniform(&x) < p;
    *estimate = (double)(2 * k) / (double)shots - 1.0;
    if (positive) *positive = k;
    return QF_OK;
}

static int shots_checks(qf_ctx *ctx, uint32_t qubits, int dtype, uint64_t n_ops, const qf_op *ops, const double *params,
                        uint64_t n_params, const double *inputs, uint64_t n_inputs, int observable, uint32_t q,
                        uint64_t shots) {
    if (!ctx || (n_ops && !ops) || (n_params && !params) || (n_inputs && !inputs)) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    QF_TRY(check_dtype(dtype));
    if (shots == 0) return fail(QF_ERR_INVALID_SHOT_COUNT, "shot count must be greater than zero");
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    if (q >= qubits) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", q, qubits);
    if (observable != QF_PAULI_X && observable != QF_PAULI_Y && observable != QF_PAULI_Z)
        return fail(QF_ERR_INVALID_ARGUMENT, "unknown observable %d", observable);
    return QF_OK;
}

// ParameterizedCircuit::expectation_with_inputs_shots (src/lib.rs:3361-3382).
int qf_expectation_shots(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *params,
                         uint64_t n_params, const double *inputs, uint64_t n_inputs, int observable, uint32_t observable_qubit,
                         uint64_t shots, uint64_t seed, double tie_eps, const qf_exec_opts *opts, double *estimate,
                         uint64_t *successes, uint64_t *n_ties) {
    clear_error();
    QF_TRY(shots_checks(ctx, qubits, dtype, n_ops, ops, params, n_params, inputs, n_inputs, observable, observable_qubit, shots));
    QF_TRY(bind_device(ctx));
    uint64_t ok = 0, t = 0;
    QF_TRY(shots_estimate(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, observable,
                          observable_qubit, shots, seed, tie_eps, opts, &ok, &t));
    if (estimate) *estimate = 2.0 * ((double)ok / (double)shots) - 1.0;
    if (successes) *successes = ok;
    if (n_ties) *n_ties = t;
    return QF_OK;
}

// ParameterizedCircuit::parameter_shift_gradient_with_inputs_shots
// (src/lib.rs:3428-3479): rotation occurrence k shifted by +-pi/2, each side
// estimated from `shots` draws, seeds seed + 2k and seed + 2k + 1.
int qf_parameter_shift_gradient_shots(qf_ctx *ctx, uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops,
                                      const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                                      int observable, uint32_t observable_qubit, uint64_t shots, uint64_t seed,
                                      double tie_eps, const qf_exec_opts *opts, double *gradient, uint64_t *n_ties) {
    clear_error();
    if (n_params && !gradient) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    QF_TRY(shots_checks(ctx, qubits, dtype, n_ops, ops, params, n_params, inputs, n_inputs, observable, observable_qubit, shots));
    {  // the whole list validated before any launch
        std::vector<BGate> g;
        QF_TRY(bind_ops(qubits, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, g));
    }
    QF_TRY(bind_device(ctx));
    std::vector<double> g(n_params, 0.0);
    uint64_t t = 0;
    const double shift = 1.5707963267948966;  // FRAC_PI_2
    for (uint64_t k = 0; k < n_ops; ++k) {
        if (ops[k].kind != QF_OP_ROTATION) continue;
        const uint64_t occ_seed = seed + k * 2;
        uint64_t okp, okm;
        QF_TRY(shots_estimate(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, shift, observable,
                              observable_qubit, shots, occ_seed, tie_eps, opts, &okp, &t));
        QF_TRY(shots_estimate(ctx, qubits, dtype, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, -shift, observable,
                              observable_qubit, shots, occ_seed + 1, tie_eps, opts, &okm, &t));
        const double plus = 2.0 * ((double)okp / (double)shots) - 1.0, minus = 2.0 * ((double)okm / (double)shots) - 1.0;
        g[ops[k].param] += 0.5 * (plus - minus);
    }
    std::copy(g.begin(), g.end(), gradient);
    if (n_ties) *n_ties = t;
    return QF_OK;
}

// ParameterizedCircuit::gradient_with_inputs (src/gradients.rs:232-330).
int qf_gradient(qf_ctx *ctx, uint32_t qubits, const qf_op *ops, uint64_t n_ops, const double *params, uint64_t n_params,
                const double *inputs, uint64_t n_inputs, const qf_pauli_term *terms, uint64_t n_terms,
                const qf_gradient_opts *opts, double *expectation, double *gradient, qf_gradient_info *info) {
    clear_error();
    if (!ctx || !opts || (n_params && !gradient)) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    if ((n_params && !params) || (n_inputs && !inputs)) return fail(QF_ERR_INVALID_ARGUMENT, "parameter arrays are NULL");
    QF_TRY(check_dtype(opts->dtype));
    QF_TRY(check_terms_real(terms, n_terms));
    const uint64_t occurrences = count_rotations(ops, n_ops);
    int strategy = opts->strategy;
    if (strategy == QF_GRAD_AUTO) {
        // GradientStrategy::select (src/gradients.rs:81-89)
        if (has_channel(ops, n_ops))
            return fail(QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX, "this circuit operation requires density-matrix simulation");
        strategy = opts->shots > 0 ? QF_GRAD_PARAMETER_SHIFT : QF_GRAD_ADJOINT;
    }
    if (strategy < QF_GRAD_PARAMETER_SHIFT || strategy > QF_GRAD_FINITE_DIFFERENCE)
        return fail(QF_ERR_INVALID_ARGUMENT, "unknown gradient strategy %d", opts->strategy);
    if (strategy == QF_GRAD_FINITE_DIFFERENCE &&
        (!std::isfinite(opts->finite_difference_step) || opts->finite_difference_step <= 0.0))
        return fail(QF_ERR_INVALID_FINITE_DIFFERENCE_STEP, "finite-difference step must be positive and finite, got %g",
                    opts->finite_difference_step);
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    // validate the whole list once (also rejects channels/measurements)
    std::vector<BGate> gates;
    QF_TRY(bind_ops(qubits, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, gates));
    {  // observable qubits in range
        const uint64_t valid = qubits >= 64 ? ~0ULL : ((1ULL << qubits) - 1);
        for (uint64_t t = 0; t < n_terms; ++t)
            if ((terms[t].xmask | terms[t].zmask) & ~valid)
                return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "observable acts outside %u qubits", qubits);
    }
    QF_TRY(bind_device(ctx));
    if (info) {
        info->strategy = strategy;
        info->reserved = 0;
        info->evaluations = (strategy == QF_GRAD_ADJOINT || strategy == QF_GRAD_BACKPROP) ? 2 : 2 * occurrences;
    }
    const qf_exec_opts *exec = &opts->exec;
    if (strategy == QF_GRAD_ADJOINT || strategy == QF_GRAD_BACKPROP)
        return adjoint_device(ctx, qubits, gates, terms, n_terms, opts, n_params, expectation, gradient);

    std::fill(gradient, gradient + n_params, 0.0);
    if (expectation)
        QF_TRY(forward_expectation(ctx, qubits, opts->dtype, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, terms,
                                   n_terms, exec, expectation));
    const bool shift_rule = strategy == QF_GRAD_PARAMETER_SHIFT;
    const double h = shift_rule ? 1.57079632679489661923 : opts->finite_difference_step;
    for (uint64_t k = 0; k < n_ops; ++k) {
        if (ops[k].kind != QF_OP_ROTATION) continue;
        double plus, minus;
        QF_TRY(forward_expectation(ctx, qubits, opts->dtype, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, h,
                                   terms, n_terms, exec, &plus));
        QF_TRY(forward_expectation(ctx, qubits, opts->dtype, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, -h,
                                   terms, n_terms, exec, &minus));
        // parameter_shift_gradient_with_inputs (src/lib.rs:3541) / FD (src/gradients.rs:369)
        gradient[ops[k].param] += shift_rule ? 0.5 * (plus - minus) : (plus - minus) / (2.0 * h);
    }
    return QF_OK;
}

uint64_t qf_rng_jump(uint64_t state, uint64_t steps) { return rng_jump(state, steps); }

int qf_adjoint_plan_stats(uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *params,
                          uint64_t n_params, const double *inputs, uint64_t n_inputs, const qf_pauli_term *terms,
                          uint64_t n_terms, const qf_gradient_opts *opts, qf_adjoint_stats *out) {
    clear_error();
    QF_TRY(check_dtype(dtype));
    if (!out || !opts) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    std::vector<BGate> gates;
    QF_TRY(bind_ops(qubits, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, gates));
    std::memset(out, 0, sizeof *out);
    // the planning of adjoint_device, without launches
    const int every = std::max(0, opts->checkpoint_every);
    std::vector<size_t> seg_begin;
    if (every > 0 && !gates.empty()) {
        for (size_t s = 0; s < gates.size(); s += (size_t)every) seg_begin.push_back(s);
    } else {
        seg_begin.push_back(0);
    }
    const size_t n_seg = seg_begin.size();
    PlanOpts po;
    default_tiling(qubits, dtype, opts->exec.tile_qubits, &po.tile_qubits, &po.low_qubits);
    po.search = !(opts->exec.flags & QF_EXEC_FLAG_PLAN_FIRST_COME);
    PlanOpts bo = po;
    bo.backward = true;
    bo.merge_1q = true;
    bo.search = false;
    for (size_t s = 0; s < n_seg; ++s) {
        const size_t b = seg_begin[s], e = s + 1 < n_seg ? seg_begin[s + 1] : gates.size();
        std::vector<BGate> seg(gates.begin() + b, gates.begin() + e);
        Plan fp, bp;
        QF_TRY(plan_passes(qubits, seg, po, fp));
        QF_TRY(plan_passes(qubits, seg, bo, bp));
        out->forward_passes += fp.passes.size();
        out->backward_passes += bp.passes.size();
    }
    uint64_t tiles = 0, wide = 0;
    QF_TRY(pauli_plan_stats(qubits, dtype, terms, n_terms, &tiles, &wide));
    out->pauli_passes = tiles + wide;
    out->state_copies = 2 * (n_seg - 1);  // checkpoints taken forward, restored backward
    // algorithmic bytes: |0> written; a forward pass reads and writes psi; the
    // first Pauli tile pass reads psi and writes lambda, later ones also read
    // lambda (as every wide group does); a separate <psi|lambda> follows wide
    // groups; a backward pass reads and writes psi and lambda; a copy reads
    // and writes one state
    const double N = (double)(1ULL << qubits) * (dtype == QF_C64 ? 8.0 : 16.0);
    double bytes = N + 2.0 * N * (double)out->forward_passes + 4.0 * N * (double)out->backward_passes +
                   2.0 * N * (double)out->state_copies;
    if (tiles) bytes += 2.0 * N + 3.0 * N * (double)(tiles - 1);
    bytes += 3.0 * N * (double)wide;
    if (wide && tiles == 0) bytes -= N;  // lambda is zeroed, not read, before the first wide sweep
    if (wide) bytes += 2.0 * N;
    out->hbm_bytes = bytes;
    return QF_OK;
}

int qf_plan_stats(uint32_t qubits, int dtype, const qf_op *ops, uint64_t n_ops, const double *params, uint64_t n_params,
                  const double *inputs, uint64_t n_inputs, const qf_exec_opts *opts, uint64_t *n_passes, uint64_t *n_gates) {
    clear_error();
    QF_TRY(check_dtype(dtype));
    if (!n_passes || !n_gates) return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    std::vector<BGate> gates;
    QF_TRY(bind_ops(qubits, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, gates));
    *n_gates = gates.size();
    if (opts && opts->mode == QF_EXEC_UNFUSED) {
        *n_passes = gates.size();
        return QF_OK;
    }
    PlanOpts po;
    QF_TRY(plan_opts_for(qubits, dtype, opts, po));
    Plan plan;
    QF_TRY(plan_passes(qubits, gates, po, plan));
    *n_passes = plan.passes.size();
    return QF_OK;
}

}  // extern "C"
