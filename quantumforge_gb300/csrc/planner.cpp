// planner.cpp — host side of the engine: gate binding, tile-pass planning and
// SmallRng jump-ahead. No device code; every function here also runs in the
// CPU-only test-suite through qf_plan_stats / qf_rng_jump.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <mutex>
#include <map>

#include "qf_internal.h"

namespace qf {

// Gate::matrix (src/lib.rs:2267-2333). Host f64 with the C library's cos/sin,
// as the reference's f64::cos/sin.
int gate_matrix(int gate, double theta, double m[8]) {
    const double s = 0.70710678118654752440;  // FRAC_1_SQRT_2
    std::memset(m, 0, sizeof(double) * 8);
    switch (gate) {
    case QF_GATE_I: m[0] = 1; m[6] = 1; return QF_OK;
    case QF_GATE_X: m[2] = 1; m[4] = 1; return QF_OK;
    case QF_GATE_Y: m[3] = -1; m[5] = 1; return QF_OK;
    case QF_GATE_Z: m[0] = 1; m[6] = -1; return QF_OK;
    case QF_GATE_H: m[0] = s; m[2] = s; m[4] = s; m[6] = -s; return QF_OK;
    case QF_GATE_S: m[0] = 1; m[7] = 1; return QF_OK;
    case QF_GATE_SDG: m[0] = 1; m[7] = -1; return QF_OK;
    case QF_GATE_T: m[0] = 1; m[6] = s; m[7] = s; return QF_OK;
    case QF_GATE_TDG: m[0] = 1; m[6] = s; m[7] = -s; return QF_OK;
    case QF_GATE_RX: {
        double c = std::cos(theta * 0.5), si = std::sin(theta * 0.5);
        m[0] = c; m[3] = -si; m[5] = -si; m[6] = c;
        return QF_OK;
    }
    case QF_GATE_RY: {
        double c = std::cos(theta * 0.5), si = std::sin(theta * 0.5);
        m[0] = c; m[2] = -si; m[4] = si; m[6] = c;
        return QF_OK;
    }
    case QF_GATE_RZ: {
        double half = theta * 0.5;
        m[0] = std::cos(half); m[1] = -std::sin(half);
        m[6] = std::cos(half); m[7] = std::sin(half);
        return QF_OK;
    }
    default:
        return fail(QF_ERR_INVALID_ARGUMENT, "unknown gate code %d", gate);
    }
}

bool matrix_is_diag(const double m[8]) { return m[2] == 0 && m[3] == 0 && m[4] == 0 && m[5] == 0; }
// all entries real, or real diagonal with an imaginary off-diagonal (RX type):
// the compiled passes' two cheap dense forms
bool matrix_is_cheap(const double m[8]) {
    if (m[1] == 0 && m[3] == 0 && m[5] == 0 && m[7] == 0) return true;
    return m[1] == 0 && m[7] == 0 && m[2] == 0 && m[4] == 0;
}

static int rotation_gate(int axis) {
    return axis == QF_PAULI_X ? QF_GATE_RX : axis == QF_PAULI_Y ? QF_GATE_RY : QF_GATE_RZ;
}

static int check_pair(uint32_t n, uint32_t a, uint32_t b) {
    if (a >= n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", a, n);
    if (b >= n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", b, n);
    if (a == b)
        return fail(QF_ERR_INVALID_QUBIT_PAIR, "two-qubit operation requires distinct qubits, got %u and %u", a, b);
    return QF_OK;
}

// Validation mirrors Circuit::run (src/lib.rs:2786-2802) and
// ParameterizedCircuit::run_with_shift (src/lib.rs:4677-4740), but is done for
// the whole list before any launch (src/cuda.rs:2256-2285).
int bind_ops(uint32_t n, const qf_op *ops, uint64_t n_ops, const double *params, uint64_t n_params,
             const double *inputs, uint64_t n_inputs, int64_t shift_op, double shift,
             std::vector<BGate> &out) {
    out.clear();
    out.reserve(n_ops);
    if (n_ops && !ops) return fail(QF_ERR_INVALID_ARGUMENT, "ops is NULL");
    for (uint64_t k = 0; k < n_inputs; ++k)
        if (!std::isfinite(inputs[k])) return fail(QF_ERR_NON_FINITE_PARAMETER, "circuit parameters must be finite");
    for (uint64_t k = 0; k < n_params; ++k)
        if (!std::isfinite(params[k])) return fail(QF_ERR_NON_FINITE_PARAMETER, "circuit parameters must be finite");
    for (uint64_t k = 0; k < n_ops; ++k) {
        const qf_op &op = ops[k];
        BGate g;
        g.op_index = (int64_t)k;
        switch (op.kind) {
        case QF_OP_GATE:
        case QF_OP_ROTATION:
        case QF_OP_ENCODING: {
            int gate;
            double theta;
            if (op.kind == QF_OP_GATE) {
                gate = op.gate;
                theta = op.theta;
            } else {
                if (op.gate > QF_PAULI_Z) return fail(QF_ERR_INVALID_ARGUMENT, "rotation axis %u is invalid", op.gate);
                gate = rotation_gate(op.gate);
                g.varying = 1;
                if (op.kind == QF_OP_ROTATION) {
                    if (op.param >= n_params)
                        return fail(QF_ERR_INVALID_PARAMETER_COUNT, "expected %llu circuit parameters, got %llu",
                                    (unsigned long long)n_params, (unsigned long long)op.param + 1);
                    theta = params[op.param];
                    g.axis = op.gate;
                    g.param = op.param;
                } else {
                    if (op.param >= n_inputs)
                        return fail(QF_ERR_INVALID_INPUT_COUNT, "expected %llu encoded inputs, got %llu",
                                    (unsigned long long)n_inputs, (unsigned long long)op.param + 1);
                    theta = inputs[op.param];
                }
            }
            if ((int64_t)k == shift_op) theta = theta + shift;
            if (op.q0 >= n)
                return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", op.q0, n);
            g.kind = BK_MAT1;
            g.q0 = op.q0;
            QF_TRY(gate_matrix(gate, theta, g.m));
            g.diag = matrix_is_diag(g.m);
            break;
        }
        case QF_OP_CNOT:
        case QF_OP_CZ:
        case QF_OP_SWAP:
            QF_TRY(check_pair(n, op.q0, op.q1));
            g.kind = op.kind == QF_OP_CNOT ? BK_CNOT : op.kind == QF_OP_CZ ? BK_CZ : BK_SWAP;
            g.q0 = op.q0;
            g.q1 = op.q1;
            break;
        case QF_OP_CHANNEL:
            return fail(QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX,
                        "this circuit operation requires density-matrix simulation");
        case QF_OP_MEASURE:
        case QF_OP_COND:
            return fail(QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION,
                        "measurement and classically conditioned circuit operations require shot execution");
        default:
            return fail(QF_ERR_INVALID_ARGUMENT, "unknown op kind %u at index %llu", op.kind, (unsigned long long)k);
        }
        out.push_back(g);
    }
    return QF_OK;
}

// U^dagger: conjugate transpose of the 2x2 (adjoint_gate, src/lib.rs:2363-2382,
// gives the same matrices); 2q gates are self-inverse.
BGate inverse_gate(const BGate &g) {
    BGate r = g;
    if (g.kind == BK_MAT1) {
        // (m00 m01; m10 m11)^dagger = (m00* m10*; m01* m11*)
        r.m[0] = g.m[0]; r.m[1] = -g.m[1];
        r.m[2] = g.m[4]; r.m[3] = -g.m[5];
        r.m[4] = g.m[2]; r.m[5] = -g.m[3];
        r.m[6] = g.m[6]; r.m[7] = -g.m[7];
    }
    return r;
}

Factored factor_unitary_2x2(const double md[8]) {
    Factored f;
    const std::complex<double> m[4] = {{md[0], md[1]}, {md[2], md[3]}, {md[4], md[5]}, {md[6], md[7]}};
    bool real = true;
    for (int k = 0; k < 4; ++k) real = real && m[k].imag() == 0.0;
    const bool xlike = !real && m[0].imag() == 0 && m[3].imag() == 0 && m[1].real() == 0 && m[2].real() == 0;
    if (!real && !xlike) return f;
    // unit rows: |g| >= 1/sqrt(2), which bounds the product of a pass's factors
    if (std::abs(std::norm(m[0]) + std::norm(m[1]) - 1.0) > 1e-9 || std::abs(std::norm(m[2]) + std::norm(m[3]) - 1.0) > 1e-9)
        return f;
    f.pivot = std::abs(m[0]) >= std::abs(m[1]) ? 0 : 1;
    const std::complex<double> g = f.pivot ? m[1] : m[0];
    const std::complex<double> h = f.pivot ? m[2] : m[3];
    if (!(std::abs(g) > 1e-150)) return f;
    const std::complex<double> sig = h / g;
    if (std::abs(sig.imag()) > 1e-12 || std::abs(std::abs(sig.real()) - 1.0) > 1e-12) return f;
    f.neg = sig.real() < 0.0;
    f.g = g;
    f.r0 = (f.pivot ? m[0] : m[1]) / g;
    f.r1 = (f.pivot ? m[3] : m[2]) / g;
    f.imag_r = xlike;
    f.imag_g = xlike && f.pivot == 1;
    f.ok = true;
    return f;
}

// c = a * b for 2x2 complex (row-major, interleaved).
static void mat_mul(const double a[8], const double b[8], double c[8]) {
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            double re = 0, im = 0;
            for (int t = 0; t < 2; ++t) {
                double ar = a[2 * (2 * i + t)], ai = a[2 * (2 * i + t) + 1];
                double br = b[2 * (2 * t + j)], bi = b[2 * (2 * t + j) + 1];
                re += ar * br - ai * bi;
                im += ar * bi + ai * br;
            }
            c[2 * (2 * i + j)] = re;
            c[2 * (2 * i + j) + 1] = im;
        }
}

void default_tiling(uint32_t n, int dtype, int requested_tile, int *tile, int *low) {
    int k = requested_tile > 0 ? requested_tile : (dtype == QF_C64 ? 12 : 11);
    if (k > kMaxLocal + 5) k = kMaxLocal + 5;
    int lo = dtype == QF_C64 ? 5 : 4;
    if ((int)n <= k) { k = (int)n; lo = (int)n; }
    if (lo > k) lo = k;
    *tile = k;
    *low = lo;
}

// Tiling of forward sweeps. Compiled passes also run on 13-qubit tiles when a
// caller asks for them (one CTA of 512 threads per SM: 18 % fewer passes on the
// 30-qubit circuit but 33 % slower passes, latency-bound), so the default stays
// at 12.
void forward_tiling(uint32_t n, int dtype, int requested_tile, int flags, int *tile, int *low) {
    (void)flags;
    default_tiling(n, dtype, requested_tile, tile, low);
}

namespace {
struct Item {
    BGate g;
    bool overlap = false;  // adjoint overlap marker for rotation g (axis in g.axis)
    uint64_t touch = 0;    // qubits this item reads or writes
    uint64_t need = 0;     // qubits that must be tile-resident
};

Item make_item(const BGate &g, bool overlap) {
    Item it;
    it.g = g;
    it.overlap = overlap;
    const uint64_t b0 = 1ULL << g.q0, b1 = 1ULL << g.q1;
    if (overlap) {
        it.touch = b0;
        it.need = g.axis == QF_PAULI_Z ? 0 : b0;
        return it;
    }
    switch (g.kind) {
    case BK_MAT1: it.touch = b0; it.need = g.diag ? 0 : b0; break;
    case BK_CNOT: it.touch = b0 | b1; it.need = b1; break;
    case BK_CZ: it.touch = b0 | b1; it.need = 0; break;
    default: it.touch = b0 | b1; it.need = b0 | b1; break;
    }
    return it;
}

int popc(uint64_t x) { return __builtin_popcountll(x); }
}  // namespace

// Greedy tile-pass planner. Walk the remaining items in circuit order; an item
// joins the current pass when none of its qubits is blocked by an item left
// behind and the qubits it needs resident still fit in the tile; otherwise its
// qubits become blocked, so no later item on those qubits may move ahead of
// it. Gates on different qubits commute, so the reordering is exact.
// Diagonal gates, CZ and a CNOT's control never need residency: within a tile
// their non-resident bits are constant and become per-tile scalars/conditions.
namespace {
// Items of `remaining` (in order) that one pass over resident set S runs: an
// item runs when none of its qubits is blocked and its needed qubits are in
// S; an item that cannot run blocks its qubits for everything after it.
int pass_closure(const std::vector<Item> &items, const std::vector<int> &remaining, uint64_t S, uint64_t all,
                 int max_items) {
    uint64_t blocked = 0;
    int cnt = 0;
    for (int idx : remaining) {
        if (blocked == all || cnt >= max_items) break;
        const Item &it = items[idx];
        if ((it.touch & blocked) || (it.need & ~S)) {
            blocked |= it.touch;
            continue;
        }
        ++cnt;
    }
    return cnt;
}

uint64_t choose_resident_greedy(const std::vector<Item> &items, const std::vector<int> &remaining, uint64_t base, int k,
                                uint32_t n, uint64_t all, int max_items);
// Items one pass runs when its resident set is completed greedily from S.
int rollout(const std::vector<Item> &items, const std::vector<int> &remaining, uint64_t S, int k, uint32_t n, uint64_t all,
            int max_items) {
    return pass_closure(items, remaining, choose_resident_greedy(items, remaining, S, k, n, all, max_items), all, max_items);
}
// Greedy completion: from `base`, add one qubit at a time, each time the one
// that lets the pass run the most items (lowest index on ties); stops when no
// single qubit adds an item (the first-come fill completes the set).
uint64_t choose_resident_greedy(const std::vector<Item> &items, const std::vector<int> &remaining, uint64_t base, int k,
                                uint32_t n, uint64_t all, int max_items) {
    uint64_t S = base;
    int cur = pass_closure(items, remaining, S, all, max_items);
    while (popc(S) < k) {
        // candidates: qubits some runnable-so-far frontier item needs
        uint64_t cand = 0, blocked = 0;
        for (int idx : remaining) {
            if (blocked == all) break;
            const Item &it = items[idx];
            if (it.touch & blocked) { blocked |= it.touch; continue; }
            if (it.need & ~S) {
                if (popc(it.need & ~S) == 1) cand |= it.need & ~S;
                blocked |= it.touch;
            }
        }
        int best = -1, best_cnt = cur;
        for (uint32_t q = 0; q < n; ++q) {
            if (!((cand >> q) & 1ULL)) continue;
            const int c = pass_closure(items, remaining, S | (1ULL << q), all, max_items);
            if (c > best_cnt) { best_cnt = c; best = (int)q; }
        }
        if (best < 0) break;
        S |= 1ULL << best;
        cur = best_cnt;
    }
    return S;
}

// Resident set of the next pass by rollouts: from `base`, add one qubit at a
// time, each time the one whose greedy completion lets the pass run the most
// items. Candidates are the qubits that frontier items (the first item on each
// qubit not yet blocked) still need, one or two of them (a SWAP needs both).
// On the 30-qubit depth-40 circuit this plans 47 passes where the plain greedy
// choice plans 52 (seven random circuits of 26-32 qubits: 285 against 323).
uint64_t choose_resident(const std::vector<Item> &items, const std::vector<int> &remaining, uint64_t base, int k,
                         uint32_t n, uint64_t all, int max_items) {
    uint64_t S = base;
    while (popc(S) < k) {
        uint64_t cand = 0, blocked = 0;
        for (int idx : remaining) {
            if (blocked == all) break;
            const Item &it = items[idx];
            if (it.touch & blocked) { blocked |= it.touch; continue; }
            if (it.need & ~S) {
                if (popc(it.need & ~S) <= 2) cand |= it.need & ~S;
                blocked |= it.touch;
            }
        }
        int best = -1, best_cnt = rollout(items, remaining, S, k, n, all, max_items);
        for (uint32_t q = 0; q < n; ++q) {
            if (!((cand >> q) & 1ULL)) continue;
            const int c = rollout(items, remaining, S | (1ULL << q), k, n, all, max_items);
            if (c > best_cnt) { best_cnt = c; best = (int)q; }
        }
        if (best < 0) break;
        S |= 1ULL << best;
    }
    return choose_resident_greedy(items, remaining, S, k, n, all, max_items);
}
}  // namespace

// ---- k-qubit dense-block fusion --------------------------------------------
// The reference applies every gate as its own sweep (StateVector::apply,
// src/lib.rs:1017-1059; kernel per gate in src/cuda.rs:114-128) and fuses
// nothing but same-axis rotation angles (src/optimizer.rs:767). Here the gates
// of one tile pass are multiplied into dense blocks of up to k qubits on the
// host in f64; the device then applies one 2^m x 2^m matrix per block.
using cd = std::complex<double>;

namespace {
struct FBlock {
    uint64_t mask = 0;
    std::vector<uint32_t> qs;  // ascending; bit i of the local index is qubit qs[i]
    std::vector<cd> M;         // row-major 2^m x 2^m
    int gates = 0;
    BGate first;               // the gate, when the block holds exactly one
    bool varying = false;
};

}  // namespace

std::vector<uint32_t> qubits_of_mask(uint64_t m) {
    std::vector<uint32_t> q;
    for (uint32_t b = 0; b < 64; ++b)
        if ((m >> b) & 1ULL) q.push_back(b);
    return q;
}
static int local_of(const std::vector<uint32_t> &qs, uint32_t q) {
    for (size_t i = 0; i < qs.size(); ++i)
        if (qs[i] == q) return (int)i;
    return -1;
}

// A matrix on ascending qubits `qs` widened to the ascending superset `nq`:
// M (x) identity on the added qubits.
std::vector<cd> widen_matrix(const std::vector<uint32_t> &qs, const std::vector<cd> &M, const std::vector<uint32_t> &nq) {
    const int m = (int)nq.size(), d = 1 << m, od = 1 << qs.size();
    std::vector<int> old(m);
    for (int i = 0; i < m; ++i) old[i] = local_of(qs, nq[i]);
    std::vector<cd> N((size_t)d * d, cd(0.0, 0.0));
    for (int r = 0; r < d; ++r)
        for (int c = 0; c < d; ++c) {
            uint32_t ro = 0, co = 0;
            bool ok = true;
            for (int i = 0; i < m && ok; ++i) {
                const int rb = (r >> i) & 1, cb = (c >> i) & 1;
                if (old[i] < 0) ok = rb == cb;
                else {
                    ro |= (uint32_t)rb << old[i];
                    co |= (uint32_t)cb << old[i];
                }
            }
            if (ok) N[(size_t)r * d + c] = M[(size_t)ro * od + co];
        }
    return N;
}

// v <- G v for one gate on local bits l0 (l1), the semantics of
// StateVector::apply / apply_cnot / apply_cz / apply_swap (src/lib.rs:1017-1122).
static void vec_apply(std::vector<cd> &v, int d, const BGate &g, int l0, int l1) {
    switch (g.kind) {
    case BK_MAT1: {
        const cd m00(g.m[0], g.m[1]), m01(g.m[2], g.m[3]), m10(g.m[4], g.m[5]), m11(g.m[6], g.m[7]);
        for (int i = 0; i < d; ++i)
            if (!((i >> l0) & 1)) {
                const int j = i | (1 << l0);
                const cd a = v[i], b = v[j];
                v[i] = m00 * a + m01 * b;
                v[j] = m10 * a + m11 * b;
            }
        break;
    }
    case BK_CNOT:
        for (int i = 0; i < d; ++i)
            if (((i >> l0) & 1) && !((i >> l1) & 1)) std::swap(v[i], v[i | (1 << l1)]);
        break;
    case BK_CZ:
        for (int i = 0; i < d; ++i)
            if (((i >> l0) & 1) && ((i >> l1) & 1)) v[i] = -v[i];
        break;
    default:  // SWAP
        for (int i = 0; i < d; ++i)
            if (((i >> l0) & 1) && !((i >> l1) & 1)) std::swap(v[i], v[(i & ~(1 << l0)) | (1 << l1)]);
        break;
    }
}

// M <- G M for a one- or two-qubit gate on qubits within `qs`: the gate
// applied to every column.
void apply_gate_to_matrix(const std::vector<uint32_t> &qs, std::vector<cd> &M, const BGate &g) {
    const int d = 1 << qs.size();
    const int l0 = local_of(qs, g.q0), l1 = g.kind == BK_MAT1 ? -1 : local_of(qs, g.q1);
    std::vector<cd> v(d);
    for (int c = 0; c < d; ++c) {
        for (int r = 0; r < d; ++r) v[r] = M[(size_t)r * d + c];
        vec_apply(v, d, g, l0, l1);
        for (int r = 0; r < d; ++r) M[(size_t)r * d + c] = v[r];
    }
}

// Dense matrix of a gate or a fused block over its qubits (ascending).
void dense_matrix(const BGate &g, const std::vector<double> &bmats, std::vector<uint32_t> &qs, std::vector<cd> &M) {
    if (g.kind == BK_BLOCK) {
        qs.assign(g.bq, g.bq + g.nq);
        const size_t dd = (size_t)1 << (2 * g.nq);
        M.resize(dd);
        for (size_t e = 0; e < dd; ++e) M[e] = cd(bmats[2 * (g.boff + e)], bmats[2 * (g.boff + e) + 1]);
        return;
    }
    qs.clear();
    qs.push_back(g.q0);
    if (g.kind != BK_MAT1) qs.push_back(g.q1);
    std::sort(qs.begin(), qs.end());
    const int d = 1 << qs.size();
    M.assign((size_t)d * d, cd(0.0, 0.0));
    for (int i = 0; i < d; ++i) M[(size_t)i * d + i] = 1.0;
    apply_gate_to_matrix(qs, M, g);
}

namespace {
// The tensor product of open blocks on disjoint qubits, over `nq` (their union).
std::vector<cd> kron_blocks(const std::vector<const FBlock *> &bs, const std::vector<uint32_t> &nq) {
    const int m = (int)nq.size(), d = 1 << m;
    std::vector<cd> P((size_t)d * d);
    std::vector<std::vector<int>> pos(bs.size());
    int covered = 0;
    for (size_t b = 0; b < bs.size(); ++b)
        for (uint32_t q : bs[b]->qs) {
            pos[b].push_back(local_of(nq, q));
            covered |= 1 << pos[b].back();
        }
    for (int r = 0; r < d; ++r)
        for (int c = 0; c < d; ++c) {
            if ((r ^ c) & ~covered) {  // qubits of nq outside every block: identity
                P[(size_t)r * d + c] = 0.0;
                continue;
            }
            cd v(1.0, 0.0);
            for (size_t b = 0; b < bs.size() && v != cd(0.0, 0.0); ++b) {
                uint32_t rb = 0, cb = 0;
                for (size_t i = 0; i < pos[b].size(); ++i) {
                    rb |= (uint32_t)((r >> pos[b][i]) & 1) << i;
                    cb |= (uint32_t)((c >> pos[b][i]) & 1) << i;
                }
                v *= bs[b]->M[(size_t)rb * (1u << pos[b].size()) + cb];
            }
            P[(size_t)r * d + c] = v;
        }
    return P;
}

// Greedy fusion of a pass's gates (in order) into blocks of at most k qubits.
// Open blocks act on disjoint qubits. A gate joins the open blocks it touches
// when their union with its qubits has at most k qubits; otherwise the widest
// of those blocks are closed (emitted) until the rest fits. Every block that
// touches a qubit is emitted after the blocks holding earlier gates on that
// qubit, so the emitted product equals the gate sequence.
std::vector<FBlock> fuse_gates(const std::vector<BGate> &gates, int k) {
    std::vector<FBlock> open, out;
    for (const BGate &g : gates) {
        const uint64_t gm = g.kind == BK_MAT1 ? (1ULL << g.q0) : ((1ULL << g.q0) | (1ULL << g.q1));
        std::vector<size_t> I;
        for (size_t j = 0; j < open.size(); ++j)
            if (open[j].mask & gm) I.push_back(j);
        auto width = [&]() {
            uint64_t u = gm;
            for (size_t j : I) u |= open[j].mask;
            return popc(u);
        };
        std::vector<size_t> closing;
        while (width() > k) {
            size_t wi = 0;
            for (size_t t = 1; t < I.size(); ++t)
                if (popc(open[I[t]].mask) > popc(open[I[wi]].mask)) wi = t;
            closing.push_back(I[wi]);
            I.erase(I.begin() + (long)wi);
        }
        FBlock nb;
        nb.mask = gm;
        for (size_t j : I) nb.mask |= open[j].mask;
        nb.qs = qubits_of_mask(nb.mask);
        std::vector<const FBlock *> parts;
        for (size_t j : I) {  // disjoint blocks commute: their tensor product (identity elsewhere)
            parts.push_back(&open[j]);
            nb.gates += open[j].gates;
            nb.varying = nb.varying || open[j].varying;
            if (open[j].gates == 1) nb.first = open[j].first;
        }
        nb.M = kron_blocks(parts, nb.qs);
        apply_gate_to_matrix(nb.qs, nb.M, g);
        if (nb.gates == 0) nb.first = g;
        ++nb.gates;
        nb.varying = nb.varying || g.varying;
        // emit the closed blocks, then replace the merged ones by the new block
        std::sort(closing.begin(), closing.end());
        for (size_t j : closing) out.push_back(open[j]);
        std::vector<size_t> gone = closing;
        gone.insert(gone.end(), I.begin(), I.end());
        std::sort(gone.begin(), gone.end());
        for (size_t t = gone.size(); t-- > 0;) open.erase(open.begin() + (long)gone[t]);
        open.push_back(std::move(nb));
    }
    for (FBlock &b : open) out.push_back(std::move(b));
    return out;
}
}  // namespace

namespace {
// A pass's choice: its resident qubits (before the lowest free qubits widen the
// tile) and the items it runs, in order.
struct PassChoice {
    uint64_t L;
    std::vector<int> sel;
};
std::string plan_key_of(uint32_t n, int k, int low, const PlanOpts &o, const std::vector<Item> &items) {
    std::string key;
    auto put = [&](uint64_t v, int bytes) {
        for (int b = 0; b < bytes; ++b) key.push_back((char)((v >> (8 * b)) & 0xFF));
    };
    put(n, 1);
    put((uint64_t)k, 1);
    put((uint64_t)low, 1);
    put(o.merge_1q | (o.backward << 1) | (o.search << 2), 1);
    put((uint64_t)o.max_items, 4);
    put((uint64_t)o.block_qubits, 1);
    put(items.size(), 4);
    for (const Item &it : items) {
        put(it.g.kind | (it.overlap << 3) | ((it.g.axis == QF_PAULI_Z) << 4), 1);
        put(it.g.q0, 1);
        put(it.g.q1, 1);
        put(it.need, 8);
    }
    return key;
}
struct PlanCache {
    std::mutex mu;
    std::map<std::string, std::vector<PassChoice>> entries;
};
PlanCache &plan_cache() {
    static PlanCache c;
    return c;
}
bool plan_cache_get(const std::string &key, std::vector<PassChoice> &out) {
    std::lock_guard<std::mutex> lk(plan_cache().mu);
    auto it = plan_cache().entries.find(key);
    if (it == plan_cache().entries.end()) return false;
    out = it->second;
    return true;
}
void plan_cache_put(const std::string &key, std::vector<PassChoice> &&v) {
    std::lock_guard<std::mutex> lk(plan_cache().mu);
    if (plan_cache().entries.size() >= 64) plan_cache().entries.clear();  // bound the host memory
    plan_cache().entries[key] = std::move(v);
}
}  // namespace

int plan_passes(uint32_t n, const std::vector<BGate> &gates, const PlanOpts &o, Plan &plan) {
    plan = Plan();
    plan.n = n;
    // at least 3 resident qubits: any two-qubit op plus qubit 0 (which keeps
    // complex64 tiles in 16-byte pairs) always fits
    const int k = std::min<int>(std::max(o.tile_qubits, 3), (int)n);
    const int low = std::min<int>(o.low_qubits, k);
    if (k - low > kMaxLocal) return fail(QF_ERR_INVALID_ARGUMENT, "tile of %d qubits over %d low qubits is too wide", k, low);
    const uint64_t all = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    const uint64_t low_mask = (low >= 64) ? ~0ULL : ((1ULL << low) - 1);

    const int kb = (!o.backward && o.block_qubits >= 2) ? std::min(o.block_qubits, kMaxBlockQubits) : 0;
    if (kb && kb > k) return fail(QF_ERR_INVALID_ARGUMENT, "blocks of %d qubits do not fit a %d-qubit tile", kb, k);
    plan.block_qubits = (uint32_t)kb;
    std::vector<Item> items;
    items.reserve(gates.size() * (o.backward ? 2 : 1));
    if (!o.backward) {
        for (const BGate &g : gates) {
            items.push_back(make_item(g, false));
            if (kb) items.back().need = items.back().touch;  // a dense block needs all its qubits in the tile
        }
    } else {
        for (size_t i = gates.size(); i-- > 0;) {
            if (gates[i].axis != 255) items.push_back(make_item(gates[i], true));
            items.push_back(make_item(inverse_gate(gates[i]), false));
        }
    }

    std::vector<int> remaining(items.size());
    for (size_t i = 0; i < items.size(); ++i) remaining[i] = (int)i;

    // The choice of every pass (resident qubits and items) depends only on the
    // list's structure: a list of the same gate kinds, qubits, diagonal flags
    // and overlaps (new angles, shifted parameters, another optimiser step)
    // replays the recorded choices instead of searching again.
    const std::string key = plan_key_of(n, k, low, o, items);
    std::vector<PassChoice> replay;
    const bool hit = plan_cache_get(key, replay);
    std::vector<PassChoice> record;
    size_t pass_i = 0;

    while (hit ? pass_i < replay.size() : !remaining.empty()) {
        uint64_t L;
        std::vector<Item> taken;
        std::vector<int> last_on(n, -1);  // index into taken of the last item touching q
        // merge consecutive 1q gates on one qubit into one matrix
        auto take = [&](const Item &it) {
            if (o.merge_1q && !it.overlap && it.g.kind == BK_MAT1) {
                int prev = last_on[it.g.q0];
                if (prev >= 0 && !taken[prev].overlap && taken[prev].g.kind == BK_MAT1) {
                    double c[8];
                    mat_mul(it.g.m, taken[prev].g.m, c);
                    // Gates from circuit parameters keep the plain matrix form (no
                    // factoring, so new angles never recompile): their product is
                    // merged only while it stays diagonal, real or RX-type. A
                    // general complex product (RZ after RY, RY after RX) costs 16
                    // FMAs per amplitude pair, the two apart a real rotation and a
                    // diagonal phase (deferred when its qubit is off the registers).
                    const bool varying = taken[prev].g.varying || it.g.varying;
                    if (!varying || matrix_is_diag(c) || matrix_is_cheap(c)) {
                        std::memcpy(taken[prev].g.m, c, sizeof c);
                        taken[prev].g.varying = varying;
                        taken[prev].g.diag = matrix_is_diag(c);
                        taken[prev].g.op_index = -1;
                        return;
                    }
                }
            }
            taken.push_back(it);
            const int ti = (int)taken.size() - 1;
            for (uint32_t q = 0; q < n; ++q)
                if ((it.touch >> q) & 1ULL) last_on[q] = ti;
        };
        if (hit) {
            L = replay[pass_i].L;
            for (int idx : replay[pass_i].sel) take(items[idx]);
            ++pass_i;
        } else {
            // The first remaining item must fit: shrink the always-resident low
            // block from the top until it does (qubit 0 stays resident, k >= 3).
            L = low_mask;
            const uint64_t first_need = items[remaining[0]].need;
            for (int b = low - 1; b >= 1 && popc(L | first_need) > k; --b) L &= ~(1ULL << b);
            if (o.search) L = choose_resident(items, remaining, L | first_need, k, n, all, o.max_items);
            uint64_t blocked = 0;
            std::vector<int> rest, sel;
            rest.reserve(remaining.size());
            for (size_t r = 0; r < remaining.size(); ++r) {
                const int idx = remaining[r];
                const Item &it = items[idx];
                if (blocked == all || taken.size() >= (size_t)o.max_items) { rest.push_back(idx); continue; }
                if (it.touch & blocked) { blocked |= it.touch; rest.push_back(idx); continue; }
                const uint64_t nl = L | it.need;
                if (popc(nl) > k) { blocked |= it.touch; rest.push_back(idx); continue; }
                L = nl;
                sel.push_back(idx);
                take(it);
            }
            if (taken.empty()) return fail(QF_ERR_INVALID_ARGUMENT, "planner made no progress");
            remaining.swap(rest);
            record.push_back(PassChoice{L, std::move(sel)});
        }
        uint32_t n_blocks = 0, max_block = 0;
        if (kb) {  // the pass's gates as dense blocks of up to kb qubits
            std::vector<BGate> seq;
            seq.reserve(taken.size());
            for (const Item &it : taken) seq.push_back(it.g);
            std::vector<Item> fused;
            for (FBlock &b : fuse_gates(seq, kb)) {
                if (b.gates == 1) {  // a lone gate keeps its own (cheaper) form
                    fused.push_back(make_item(b.first, false));
                } else if (b.qs.size() == 1) {  // a product of one-qubit gates
                    BGate g;
                    g.kind = BK_MAT1;
                    g.q0 = b.qs[0];
                    for (int e = 0; e < 4; ++e) {
                        g.m[2 * e] = b.M[e].real();
                        g.m[2 * e + 1] = b.M[e].imag();
                    }
                    g.diag = matrix_is_diag(g.m);
                    g.varying = b.varying;
                    fused.push_back(make_item(g, false));
                } else {
                    BGate g;
                    g.kind = BK_BLOCK;
                    g.nq = (uint8_t)b.qs.size();
                    for (size_t i = 0; i < b.qs.size(); ++i) g.bq[i] = (uint8_t)b.qs[i];
                    g.q0 = b.qs[0];
                    g.q1 = b.qs[1];
                    g.varying = b.varying;
                    g.boff = (uint32_t)(plan.bmats.size() / 2);
                    for (const cd &z : b.M) {
                        plan.bmats.push_back(z.real());
                        plan.bmats.push_back(z.imag());
                    }
                    Item it;
                    it.g = g;
                    it.touch = it.need = b.mask;
                    fused.push_back(it);
                    ++n_blocks;
                    max_block = std::max<uint32_t>(max_block, g.nq);
                }
            }
            taken.swap(fused);
        }

        // widen the tile with the lowest free qubits: longer contiguous runs
        for (uint32_t q = 0; q < n && popc(L) < k; ++q) L |= 1ULL << q;
        // lower to tile ops
        Pass p;
        uint32_t lo_eff = 0;
        while (lo_eff < n && ((L >> lo_eff) & 1ULL)) ++lo_eff;
        std::vector<int> local_bit(n, -1);
        for (uint32_t q = 0; q < lo_eff; ++q) local_bit[q] = (int)q;
        uint32_t r = 0;
        std::memset(p.a.hi_q, 0, sizeof p.a.hi_q);
        for (uint32_t q = lo_eff; q < n; ++q)
            if ((L >> q) & 1ULL) {
                if (r >= (uint32_t)kMaxLocal) return fail(QF_ERR_INVALID_ARGUMENT, "too many resident high qubits");
                p.a.hi_q[r] = (uint8_t)q;
                local_bit[q] = (int)(lo_eff + r);
                ++r;
            }
        p.a.k = lo_eff + r;
        p.a.low = lo_eff;
        if (lo_eff < 1 || p.a.k > 21) return fail(QF_ERR_INVALID_ARGUMENT, "invalid tile layout (low %u, k %u)", lo_eff, p.a.k);
        p.a.nonlocal_mask = all & ~L;
        p.a.n_tiles = 1ULL << (n - p.a.k);
        p.resident = L;
        p.n_blocks = n_blocks;
        p.max_block = max_block;
        p.op_begin = (uint32_t)plan.ops.size();
        p.mat_begin = (uint32_t)(plan.mats.size() / 8);
        p.a.slot_base = plan.n_slots;
        // factors pulled out of T_MAT1F gates (forward plans), applied by a
        // T_SCALE op at the end of the pass, or earlier once they get small
        std::complex<double> pscale(1.0, 0.0);
        bool any_factored = false;
        auto push_scale = [&]() {
            TileOp sc;
            std::memset(&sc, 0, sizeof sc);
            sc.slot = -1;
            sc.kind = T_SCALE;
            sc.mat = (uint32_t)(plan.mats.size() / 8) - p.mat_begin;
            const double e[8] = {pscale.real(), pscale.imag(), 0, 0, 0, 0, 0, 0};
            plan.mats.insert(plan.mats.end(), e, e + 8);
            plan.ops.push_back(sc);
            pscale = 1.0;
            any_factored = false;
        };
        for (const Item &it : taken) {
            TileOp t;
            std::memset(&t, 0, sizeof t);
            t.slot = -1;
            const BGate &g = it.g;
            const int lb0 = local_bit[g.q0];
            const int lb1 = g.kind == BK_MAT1 ? -1 : local_bit[g.q1];
            if (it.overlap) {
                t.slot = (int32_t)plan.n_slots++;
                plan.slot_param.push_back(g.param);
                if (g.axis == QF_PAULI_X) { t.kind = T_OVL_X; t.b0 = (uint8_t)lb0; }
                else if (g.axis == QF_PAULI_Y) { t.kind = T_OVL_Y; t.b0 = (uint8_t)lb0; }
                else if (lb0 >= 0) { t.kind = T_OVL_ZL; t.b0 = (uint8_t)lb0; }
                else { t.kind = T_OVL_ZG; t.g0 = g.q0; }
                plan.ops.push_back(t);
                BGate ov = g;
                ov.kind = BK_OVL;
                ov.op_index = t.slot;
                p.gates.push_back(ov);
                continue;
            }
            p.gates.push_back(g);
            switch (g.kind) {
            case BK_BLOCK: {
                t.kind = T_BLOCK;
                t.b0 = g.nq;
                for (int i = 0; i < g.nq; ++i) t.g0 |= (uint32_t)local_bit[g.bq[i]] << (5 * i);
                t.mat = g.boff;
                break;
            }
            case BK_MAT1: {
                const Factored f = (!g.diag && !o.backward) ? factor_unitary_2x2(g.m) : Factored();
                if (f.ok) {
                    if (std::abs(pscale) < 0x1p-40) push_scale();  // keep float32 tiles far from overflow
                    t.mat = (uint32_t)(plan.mats.size() / 8) - p.mat_begin;
                    const double e[8] = {f.r0.real(), f.r0.imag(), f.r1.real(), f.r1.imag(), 0, 0, 0, 0};
                    plan.mats.insert(plan.mats.end(), e, e + 8);
                    t.kind = T_MAT1F;
                    t.b0 = (uint8_t)lb0;
                    t.b1 = (uint8_t)(f.pivot | (f.neg ? 2 : 0) | (f.imag_r ? 4 : 0));
                    pscale *= f.g;
                    any_factored = true;
                    break;
                }
                t.mat = (uint32_t)(plan.mats.size() / 8) - p.mat_begin;
                plan.mats.insert(plan.mats.end(), g.m, g.m + 8);
                if (!g.diag) { t.kind = T_MAT1; t.b0 = (uint8_t)lb0; }
                else if (lb0 >= 0) { t.kind = T_DIAG1; t.b0 = (uint8_t)lb0; }
                else { t.kind = T_GPHASE; t.g0 = g.q0; }
                break;
            }
            case BK_CNOT:
                if (lb0 >= 0) { t.kind = T_CNOT_LL; t.b0 = (uint8_t)lb0; t.b1 = (uint8_t)lb1; }
                else { t.kind = T_CNOT_GL; t.g0 = g.q0; t.b1 = (uint8_t)lb1; }
                break;
            case BK_CZ:
                if (lb0 >= 0 && lb1 >= 0) { t.kind = T_CZ_LL; t.b0 = (uint8_t)lb0; t.b1 = (uint8_t)lb1; }
                else if (lb0 >= 0) { t.kind = T_CZ_GL; t.g0 = g.q1; t.b1 = (uint8_t)lb0; }
                else if (lb1 >= 0) { t.kind = T_CZ_GL; t.g0 = g.q0; t.b1 = (uint8_t)lb1; }
                else { t.kind = T_CZ_GG; t.g0 = g.q0; t.g1 = g.q1; }
                break;
            default:
                t.kind = T_SWAP_LL; t.b0 = (uint8_t)lb0; t.b1 = (uint8_t)lb1;
                break;
            }
            plan.ops.push_back(t);
        }
        if (any_factored) push_scale();
        p.a.n_ops = (uint32_t)plan.ops.size() - p.op_begin;
        p.a.n_mats = (uint32_t)(plan.mats.size() / 8) - p.mat_begin;
        p.a.n_slots = plan.n_slots - p.a.slot_base;
        plan.passes.push_back(p);
    }
    if (!hit) plan_cache_put(key, std::move(record));
    return QF_OK;
}

// ---- register-tiled lowering ----------------------------------------------
static uint8_t matrix_kind(const double m[8]) {
    if (m[1] == 0 && m[3] == 0 && m[5] == 0 && m[7] == 0) return 1;  // real
    if (m[1] == 0 && m[7] == 0 && m[2] == 0 && m[4] == 0) return 2;  // real diagonal, imaginary off-diagonal
    return 0;
}

int lower_rs(const Plan &plan, int wb, RsPlan &out) {
    out = RsPlan();
    out.wb = wb;
    const uint32_t n = plan.n;
    const int npos = 4 + wb;
    const int k = 5 + npos;
    for (const Pass &p : plan.passes) {
        RsPass rp;
        std::memset(&rp.a, 0, sizeof rp.a);
        rp.op_begin = (uint32_t)out.ops.size();
        rp.mat_begin = (uint32_t)(out.mats.size() / 8);
        if ((int)n < k || popc(p.resident) != k || (p.resident & 31ULL) != 31ULL) {
            rp.fallback = true;
            out.passes.push_back(rp);
            continue;
        }
        std::vector<uint32_t> freeq;
        for (uint32_t q = 5; q < n; ++q)
            if ((p.resident >> q) & 1ULL) freeq.push_back(q);
        int slot_of[64];
        for (int q = 0; q < 64; ++q) slot_of[q] = -1;
        for (size_t s = 0; s < freeq.size(); ++s) slot_of[freeq[s]] = (int)s;
        const std::vector<BGate> &G = p.gates;

        // the qubit a gate needs in a register position (-1: none)
        auto need_reg = [&](const BGate &g) -> int {
            if (g.kind == BK_MAT1) return (!g.diag && g.q0 >= 5) ? (int)g.q0 : -1;
            if (g.kind == BK_CNOT) return g.q1 >= 5 ? (int)g.q1 : -1;
            if (g.kind == BK_SWAP) {
                const bool f0 = g.q0 >= 5, f1 = g.q1 >= 5;
                if (f0 != f1) return f0 ? (int)g.q0 : (int)g.q1;
            }
            return -1;
        };
        uint32_t label[8];
        auto pos_of = [&](uint32_t q) -> int {
            for (int s = 0; s < npos; ++s)
                if (label[s] == q) return s;
            return -1;
        };
        // register set for the gates from `from` on: the next four distinct
        // qubits they need in registers, then free qubits already in registers
        auto relayout = [&](size_t from, bool have_current) {
            std::vector<uint32_t> regs;
            for (size_t i = from; i < G.size() && regs.size() < 4; ++i) {
                const int q = need_reg(G[i]);
                if (q >= 0 && std::find(regs.begin(), regs.end(), (uint32_t)q) == regs.end()) regs.push_back((uint32_t)q);
            }
            if (have_current)
                for (int s = 0; s < 4 && regs.size() < 4; ++s)
                    if (std::find(regs.begin(), regs.end(), label[s]) == regs.end()) regs.push_back(label[s]);
            for (uint32_t q : freeq)
                if (regs.size() < 4 && std::find(regs.begin(), regs.end(), q) == regs.end()) regs.push_back(q);
            uint32_t nl[8];
            for (int s = 0; s < 4; ++s) nl[s] = regs[s];
            int w = 4;
            for (uint32_t q : freeq)
                if (std::find(regs.begin(), regs.end(), q) == regs.end()) nl[w++] = q;
            std::memcpy(label, nl, sizeof nl);
        };
        auto pack = [&]() {
            uint32_t v = 0;
            for (int s = 0; s < npos; ++s) v |= (uint32_t)slot_of[label[s]] << (3 * s);
            return v;
        };
        auto desc = [&](uint32_t q) -> uint8_t {
            if (q < 5) return (uint8_t)q;
            const int s = pos_of(q);
            if (s >= 0) return (uint8_t)(s < 4 ? 8 + s : 16 + (s - 4));
            return (uint8_t)(64 + q);
        };
        auto add_mat = [&](const double *m) {
            out.mats.insert(out.mats.end(), m, m + 8);
            return (uint32_t)(out.mats.size() / 8 - 1) - rp.mat_begin;
        };
        relayout(0, false);
        for (int s = 0; s < npos; ++s) rp.a.load_q[s] = (uint8_t)label[s];
        for (size_t gi = 0; gi < G.size(); ++gi) {
            const BGate &g = G[gi];
            const int nq = need_reg(g);
            if (nq >= 0 && pos_of((uint32_t)nq) >= 4) {
                RsOp r{};
                r.kind = RS_REMAP;
                r.a = pack();
                relayout(gi, true);
                r.b = pack();
                out.ops.push_back(r);
            }
            RsOp r{};
            switch (g.kind) {
            case BK_MAT1:
                r.mat = add_mat(g.m);
                r.mk = matrix_kind(g.m);
                if (g.diag) { r.kind = RS_DIAG; r.p0 = desc(g.q0); }
                else if (g.q0 < 5) { r.kind = RS_MLANE; r.p0 = (uint8_t)g.q0; }
                else { r.kind = RS_MREG; r.p0 = (uint8_t)pos_of(g.q0); }
                out.ops.push_back(r);
                break;
            case BK_CNOT:
                r.kind = RS_CNOT;
                r.p0 = desc(g.q0);
                r.p1 = desc(g.q1);
                out.ops.push_back(r);
                break;
            case BK_CZ:
                r.kind = RS_CZ;
                r.p0 = desc(g.q0);
                r.p1 = desc(g.q1);
                out.ops.push_back(r);
                break;
            default: {  // SWAP
                const bool f0 = g.q0 >= 5, f1 = g.q1 >= 5;
                if (f0 && f1) {  // relabel: the positions now hold each other's qubit
                    const int a = pos_of(g.q0), b = pos_of(g.q1);
                    std::swap(label[a], label[b]);
                } else if (!f0 && !f1) {
                    r.kind = RS_SWAP_LL;
                    r.p0 = (uint8_t)g.q0;
                    r.p1 = (uint8_t)g.q1;
                    out.ops.push_back(r);
                } else {
                    r.kind = RS_SWAP_LR;
                    r.p0 = (uint8_t)(f0 ? g.q1 : g.q0);
                    r.p1 = (uint8_t)pos_of(f0 ? g.q0 : g.q1);
                    out.ops.push_back(r);
                }
                break;
            }
            }
        }
        for (int s = 0; s < npos; ++s) rp.a.store_q[s] = (uint8_t)label[s];
        rp.a.nonlocal_mask = p.a.nonlocal_mask;
        rp.a.n_tiles = p.a.n_tiles;
        rp.a.n_ops = (uint32_t)out.ops.size() - rp.op_begin;
        rp.a.n_mats = (uint32_t)(out.mats.size() / 8) - rp.mat_begin;
        out.passes.push_back(rp);
    }
    return QF_OK;
}

// ---- SmallRng jump-ahead --------------------------------------------------
// next_u64 (src/lib.rs:4898-4905) is linear over GF(2)^64: x -> T x. A 64x64
// bit matrix is stored as its 64 columns (the image of each basis vector).
static uint64_t xs_step(uint64_t x) {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return x;
}
static uint64_t mat_apply(const uint64_t *cols, uint64_t x) {
    uint64_t y = 0;
    while (x) {
        int c = __builtin_ctzll(x);
        y ^= cols[c];
        x &= x - 1;
    }
    return y;
}
static void mat_compose(const uint64_t *a, const uint64_t *b, uint64_t *out) {  // out = a . b
    uint64_t tmp[64];
    for (int c = 0; c < 64; ++c) tmp[c] = mat_apply(a, b[c]);
    std::memcpy(out, tmp, sizeof tmp);
}
static void mat_power(uint64_t steps, uint64_t *out) {
    uint64_t base[64], acc[64];
    for (int c = 0; c < 64; ++c) { base[c] = xs_step(1ULL << c); acc[c] = 1ULL << c; }
    while (steps) {
        if (steps & 1ULL) mat_compose(base, acc, acc);
        mat_compose(base, base, base);
        steps >>= 1;
    }
    std::memcpy(out, acc, sizeof acc);
}

uint64_t rng_jump(uint64_t state, uint64_t steps) {
    uint64_t m[64];
    mat_power(steps, m);
    return mat_apply(m, state);
}

uint64_t rng_apply(const uint64_t cols[64], uint64_t state) { return mat_apply(cols, state); }

// mats[j] = T^(stride * 2^j), j < count.
void rng_jump_matrices(uint64_t stride, uint64_t (*mats)[64], int count) {
    if (count <= 0) return;
    mat_power(stride, mats[0]);
    for (int j = 1; j < count; ++j) mat_compose(mats[j - 1], mats[j - 1], mats[j]);
}

}  // namespace qf
