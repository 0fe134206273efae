// jit.cpp — pass compiler for complex64 tile sweeps.
//
// Each pass of a forward plan (a run of gates on 12 resident qubits) becomes
// one straight-line CUDA kernel. A CTA of 256 threads handles a 4096-amplitude
// tile per loop iteration: the tile streams into shared memory one iteration
// ahead (16-byte cp.async, double buffered), is read into 16 registers per
// thread in a layout that assigns the 12 resident qubits to 5 lane bits, 4
// register bits and 3 warp bits, and every dense gate runs on a register
// qubit: when a gate's qubit is not in a register position the tile is
// re-read from shared memory in a new layout (a remap). Diagonal gates, CZ and
// CNOT controls read their qubit's bit wherever it lives; CNOTs inside the
// register positions are renames of the register variables and SWAPs of
// resident qubits are relabels, neither emits an instruction. Shared memory
// is XOR-swizzled on bits 1..3 so that warp accesses in any layout are
// (nearly) conflict-free while 16-byte chunks stay contiguous. The tile is
// stored straight from registers when the lanes hold qubits 0..4, otherwise
// through shared memory in coalesced 16-byte chunks.
//
// Matrices are read from __constant__ memory (real ones as packed f32x2
// pairs), so a structurally identical circuit with new angles reuses the
// compiled kernels; diagonal gates are applied as diag(1, m11/m00) and the
// product of the m00 factors once at the end of the plan (a global phase).
// Kernels are compiled with NVRTC (loaded with dlopen) for sm_103a, loaded
// with cudaLibraryLoadData and cached by source text.
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "qf_internal.h"

namespace qf {

namespace {

// ---- NVRTC through dlopen --------------------------------------------------
struct Nvrtc {
    decltype(&nvrtcCreateProgram) create = nullptr;
    decltype(&nvrtcCompileProgram) compile = nullptr;
    decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&nvrtcGetProgramLog) log = nullptr;
    decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&nvrtcGetCUBIN) cubin = nullptr;
    decltype(&nvrtcDestroyProgram) destroy = nullptr;
    decltype(&nvrtcGetErrorString) err = nullptr;
    bool ok = false;
    std::string why;
};

Nvrtc &nvrtc() {
    static Nvrtc n;
    static std::once_flag once;
    std::call_once(once, [] {
        const char *names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                               "/usr/local/cuda/lib64/libnvrtc.so"};
        void *h = nullptr;
        for (const char *nm : names)
            if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) {
            n.why = "libnvrtc.so could not be loaded";
            return;
        }
#define QF_SYM(field, name)                                          \
    n.field = reinterpret_cast<decltype(n.field)>(dlsym(h, name));   \
    if (!n.field) {                                                  \
        n.why = "libnvrtc lacks " name;                              \
        return;                                                      \
    }
        QF_SYM(create, "nvrtcCreateProgram");
        QF_SYM(compile, "nvrtcCompileProgram");
        QF_SYM(log_size, "nvrtcGetProgramLogSize");
        QF_SYM(log, "nvrtcGetProgramLog");
        QF_SYM(cubin_size, "nvrtcGetCUBINSize");
        QF_SYM(cubin, "nvrtcGetCUBIN");
        QF_SYM(destroy, "nvrtcDestroyProgram");
        QF_SYM(err, "nvrtcGetErrorString");
#undef QF_SYM
        n.ok = true;
    });
    return n;
}

// ---- code generation ---------------------------------------------------------
constexpr int kR = 16;        // amplitudes per thread
// A pass tile holds K = 12 or 13 resident qubits (forward passes may use 13,
// backward passes 12) in K positions: 0..4 lane bits, 5..8 register bits,
// 9..K-1 warp bits; 16 amplitudes per thread, so 2^(K-4) threads per CTA.
constexpr int kPosMax = 13;
constexpr int kChunks = 8;  // 16-byte chunks per thread per tile (2^K / 2 / 2^(K-4))
int tile_of(int K) { return 1 << K; }
int threads_of(int K) { return 1 << (K - 4); }
size_t dyn_smem_of(int K) { return 2u * (size_t)tile_of(K) * 8u; }  // two tile buffers of float2

// Shared-memory swizzle: tile index bits 4..12 are folded into bits 1..3
// (the bank bits of a 16-byte chunk) with the columns 1,2,4,3,6,5,7,1,2, so
// that the slots 1..12 reach every nonzero combination of bank bits and any
// four register slots leave a bank basis for the lanes. Bit 0 is never
// swizzled: 16-byte chunks stay whole.
constexpr uint32_t kSwzMask[3] = {0xE9u, 0x15Au, 0x74u};
uint32_t swz(uint32_t j) {
    const uint32_t h = (j >> 4) & 0x1FFu;
    uint32_t r = 0;
    for (int b = 0; b < 3; ++b) r |= (uint32_t)(__builtin_popcount(h & kSwzMask[b]) & 1) << b;
    return r;
}
uint32_t physj(uint32_t j) { return j ^ (swz(j) << 1); }
// bank vector (bits 0..3 of the swizzled index) contributed by slot s
uint32_t bank_vec(int s) { return physj(1u << s) & 15u; }

struct Gen {
    std::ostringstream s;
    int v[kR];                                 // logical register -> variable number
    std::vector<std::complex<double>> consts;  // 4 complex per matrix slot (float2 M[...])
    std::complex<double> gphase{1.0, 0.0};
    bool any_diag = false;
    // factors pulled out of the gates of the current forward pass (one
    // multiply per amplitude at the pass's end)
    std::complex<double> pscale{1.0, 0.0};
    bool pscale_imag = false;  // an odd number of imaginary factors
    bool any_scale = false;
    int n_factored = 0;  // factors in pscale: each |g| >= 1/sqrt(2), so 96 keep |pscale| >= 2^-48
    void reset_scale() {
        pscale = {1.0, 0.0};
        pscale_imag = false;
        any_scale = false;
        n_factored = 0;
    }
    int tmp = 0;

    std::string pfx = "r";  // register array: r = psi, l = lambda (backward passes)
    std::string R(int i) const { return pfx + std::to_string(v[i]); }
    std::string fresh(const char *stem) { return std::string(stem) + std::to_string(tmp++); }
    int slot(std::complex<double> a, std::complex<double> b, std::complex<double> c, std::complex<double> d) {
        consts.push_back(a);
        consts.push_back(b);
        consts.push_back(c);
        consts.push_back(d);
        return (int)consts.size() / 4 - 1;
    }
};

std::string Mref(int slot, int e) { return "M[" + std::to_string(4 * slot + e) + "]"; }

std::string hex64(uint64_t v) {
    std::ostringstream o;
    o << "0x" << std::hex << v << "ull";
    return o.str();
}

// deposit of the tile index `var` onto the outside qubits, as runs of shifts
std::string deposit_code(uint64_t mask, const std::string &var) {
    std::ostringstream o;
    o << "0ull";
    int consumed = 0;
    for (int q = 0; q < 64;) {
        if (!((mask >> q) & 1ULL)) {
            ++q;
            continue;
        }
        int e = q;
        while (e < 64 && ((mask >> e) & 1ULL)) ++e;
        const int len = e - q;
        o << " | (((" << var << " >> " << consumed << ") & " << hex64(len >= 64 ? ~0ULL : ((1ULL << len) - 1)) << ") << "
          << q << ")";
        consumed += len;
        q = e;
    }
    return o.str();
}

uint8_t matrix_kind_of(const std::complex<double> m[4]) {
    bool real = true;
    for (int k = 0; k < 4; ++k) real = real && m[k].imag() == 0.0;
    if (real) return 1;
    if (m[0].imag() == 0 && m[3].imag() == 0 && m[1].real() == 0 && m[2].real() == 0) return 2;
    return 0;
}

void emit_cmul_const(Gen &g, const std::string &R, int slot, int e) {
    const std::string f = Mref(slot, e);
    g.s << "{const float2 x=" << R << ";" << R << ".x=" << f << ".x*x.x-" << f << ".y*x.y;" << R << ".y=" << f
        << ".x*x.y+" << f << ".y*x.x;}\n";
}

// A dense 2x2 on the pair (A, B); real matrices use packed f32x2 FMA with
// splatted constants.
void emit_mat2(Gen &g, int slot, int mk, const std::string &A, const std::string &B) {
    const std::string m00 = Mref(slot, 0), m01 = Mref(slot, 1), m10 = Mref(slot, 2), m11 = Mref(slot, 3);
    auto &s = g.s;
    s << "{const float2 x=" << A << ",y=" << B << ";";
    if (mk == 1) {
        s << A << "=qf_ffma2(" << m01 << ",y,qf_fmul2(" << m00 << ",x));";
        s << B << "=qf_ffma2(" << m11 << ",y,qf_fmul2(" << m10 << ",x));";
    } else if (mk == 2) {
        s << A << ".x=" << m00 << ".x*x.x-" << m01 << ".y*y.y;" << A << ".y=" << m00 << ".x*x.y+" << m01 << ".y*y.x;";
        s << B << ".x=" << m11 << ".x*y.x-" << m10 << ".y*x.y;" << B << ".y=" << m11 << ".x*y.y+" << m10 << ".y*x.x;";
    } else {
        s << A << ".x=" << m00 << ".x*x.x-" << m00 << ".y*x.y+" << m01 << ".x*y.x-" << m01 << ".y*y.y;";
        s << A << ".y=" << m00 << ".x*x.y+" << m00 << ".y*x.x+" << m01 << ".x*y.y+" << m01 << ".y*y.x;";
        s << B << ".x=" << m10 << ".x*x.x-" << m10 << ".y*x.y+" << m11 << ".x*y.x-" << m11 << ".y*y.y;";
        s << B << ".y=" << m10 << ".x*x.y+" << m10 << ".y*x.x+" << m11 << ".x*y.y+" << m11 << ".y*y.x;";
    }
    s << "}\n";
}

// Gates factored as out0 = g (p0 + r0 q0), out1 = g (sigma p1 + r1 q1)
// (factor_unitary_2x2) take two packed FMAs per amplitude pair instead of four
// (real) or eight scalar FMAs (RX type). The factors g of a pass multiply into
// one scalar applied when the pass stores its tile. The pivot choice is part of
// a module's structure, so gates whose matrices come from circuit parameters
// or encoded inputs (they change between calls: training steps, shifted
// evaluations) keep the plain form and new angles never recompile. In the
// adjoint's dual passes psi and lambda carry the same factor G, so an overlap
// read mid-pass is scaled by |G|^2.
Factored factor_gate(const std::complex<double> m[4], int) {
    const double d[8] = {m[0].real(), m[0].imag(), m[1].real(), m[1].imag(),
                         m[2].real(), m[2].imag(), m[3].real(), m[3].imag()};
    return factor_unitary_2x2(d);
}
// the splatted constant of r: (r, r) when real, (-Im r, Im r) when imaginary
std::complex<double> factored_const(const Factored &f, std::complex<double> r) {
    return f.imag_r ? std::complex<double>(-r.imag(), r.imag()) : std::complex<double>(r.real(), r.real());
}
// structure code of a factored gate for the module cache key (0: plain form)
uint8_t factored_code(const Factored &f) {
    return f.ok ? (uint8_t)(1 + f.pivot + 2 * f.neg) : 0;
}
// Factors pulled out before the tile values are rescaled mid-pass: 96 of them
// keep the amplitudes below 2^48 times their size and the scale above 2^-48,
// far inside float32's range, however deep a pass is (a pass holds up to 768
// gates).
constexpr int kMaxFactors = 96;

int slot_factored(Gen &g, const Factored &f) {
    g.pscale *= f.g;
    ++g.n_factored;
    g.pscale_imag ^= f.imag_g;
    g.any_scale = true;
    return g.slot(factored_const(f, f.r0), factored_const(f, f.r1), 0.0, 0.0);
}
void emit_factored(Gen &g, int slot, const Factored &f, const std::string &A, const std::string &B) {
    const std::string k0 = Mref(slot, 0), k1 = Mref(slot, 1);
    auto S = [&](const char *v) { return f.imag_r ? std::string("make_float2(") + v + ".y," + v + ".x)" : std::string(v); };
    auto N = [&](const char *v) { return f.neg ? std::string("make_float2(-") + v + ".x,-" + v + ".y)" : std::string(v); };
    auto &s = g.s;
    s << "{const float2 x=" << A << ",y=" << B << ";";
    if (f.pivot == 0) {
        s << A << "=qf_ffma2(" << k0 << "," << S("y") << ",x);";
        s << B << "=qf_ffma2(" << k1 << "," << S("x") << "," << N("y") << ");";
    } else {
        s << A << "=qf_ffma2(" << k0 << "," << S("x") << ",y);";
        s << B << "=qf_ffma2(" << k1 << "," << S("y") << "," << N("x") << ");";
    }
    s << "}\n";
}

// the pass factor as a packed multiplier: (G, G) when real, (-Im G, Im G) when imaginary
std::complex<double> scale_const(const Gen &g) {
    return g.pscale_imag ? std::complex<double>(-g.pscale.imag(), g.pscale.imag())
                         : std::complex<double>(g.pscale.real(), g.pscale.real());
}

// A dense block's D x D matrix in the constant bank (row-major, from complex
// offset `boff` of the plan's block matrices); returns its first slot (entry
// (r, c) is M[4 * slot + r * D + c]).
int block_slots(Gen &g, const std::vector<double> &bm, uint32_t boff, int D) {
    const int first = (int)g.consts.size() / 4;
    for (int e = 0; e < D * D; ++e) g.consts.push_back({bm[2 * ((size_t)boff + e)], bm[2 * ((size_t)boff + e) + 1]});
    while (g.consts.size() % 4) g.consts.push_back(0.0);
    return first;
}

// One pass -> one kernel.
struct PassGen {
    Gen &g;
    const Pass &p;
    uint32_t n;
    int slot_of[64];
    uint32_t slot_q[kPosMax];
    uint32_t L[kPosMax];  // position -> qubit
    int K = 12;           // resident qubits (positions)
    int WB = 3;           // warp bits: K - 9

    bool dual;  // backward pass: psi (A, r*) and lambda (B, l*) with overlap slots
    const std::vector<double> *bmats = nullptr;  // the plan's dense block matrices (BK_BLOCK)

    PassGen(Gen &gen, const Pass &pass, uint32_t nq, bool dual_ = false, const std::vector<double> *bm = nullptr)
        : g(gen), p(pass), n(nq), dual(dual_), bmats(bm) {
        for (int q = 0; q < 64; ++q) slot_of[q] = -1;
        int s = 0;
        for (uint32_t q = 0; q < n; ++q)
            if ((p.resident >> q) & 1ULL) {
                slot_of[q] = s;
                slot_q[s++] = q;
            }
        K = s;
        WB = K - 9;
    }
    int pos_of(uint32_t q) const {
        for (int i = 0; i < K; ++i)
            if (L[i] == q) return i;
        return -1;
    }
    // bit descriptor of qubit q in the current layout
    uint8_t desc(uint32_t q) const {
        const int ps = pos_of(q);
        if (ps < 0) return (uint8_t)(64 + q);
        if (ps < 5) return (uint8_t)ps;
        if (ps < 9) return (uint8_t)(8 + ps - 5);
        return (uint8_t)(16 + ps - 9);
    }
    static bool is_reg(uint8_t d) { return d >= 8 && d < 16; }
    static std::string cbit(uint8_t d) {
        if (d < 8) return "((lane >> " + std::to_string(d) + ") & 1u)";
        if (d >= 16 && d < 64) return "((warp >> " + std::to_string(d - 16) + ") & 1u)";
        return "((unsigned)(tb >> " + std::to_string(d - 64) + ") & 1u)";
    }
    // ---- gate scheduling inside the pass ----
    // Gates commute unless they share a qubit on which one of them is not
    // diagonal (a diagonal 1q gate, both CZ qubits and a CNOT control are
    // diagonal on their qubit). A gate runs once every earlier gate it does
    // not commute with has run and, for a dense gate or a CNOT target, once
    // its qubit sits in a register position. Diagonal 1q gates wait for their
    // qubit to reach a register too (half the multiplies) unless only they
    // are left.
    std::vector<std::vector<int>> preds;
    std::vector<char> done;
    std::vector<int> order;  // gate indices in emission order
    bool failed = false;

    // An overlap Im<lambda|P_q psi> commutes with every gate that commutes
    // with P_q: it is diagonal on q for P = Z.
    static bool diag_on(const BGate &x, uint32_t q) {
        switch (x.kind) {
        case BK_MAT1: return x.diag != 0;
        case BK_CNOT: return q == x.q0;
        case BK_CZ: return true;
        case BK_OVL: return x.axis == QF_PAULI_Z;
        default: return false;  // SWAP, dense block
        }
    }
    static int arity(const BGate &x) {
        if (x.kind == BK_BLOCK) return x.nq;
        return (x.kind == BK_MAT1 || x.kind == BK_OVL) ? 1 : 2;
    }
    static uint32_t qubit(const BGate &x, int k) {
        if (x.kind == BK_BLOCK) return x.bq[k];
        return k ? x.q1 : x.q0;
    }
    static uint64_t block_mask(const BGate &x) {
        uint64_t m = 0;
        for (int i = 0; i < x.nq; ++i) m |= 1ULL << x.bq[i];
        return m;
    }
    void build_deps() {
        const auto &G = p.gates;
        preds.assign(G.size(), {});
        done.assign(G.size(), 0);
        for (size_t j = 0; j < G.size(); ++j)
            for (size_t i = 0; i < j; ++i) {
                bool conflict = false;
                for (int a = 0; a < arity(G[i]) && !conflict; ++a)
                    for (int b = 0; b < arity(G[j]) && !conflict; ++b) {
                        const uint32_t q = qubit(G[i], a);
                        if (q == qubit(G[j], b) && !(diag_on(G[i], q) && diag_on(G[j], q))) conflict = true;
                    }
                if (conflict) preds[j].push_back((int)i);
            }
    }
    bool ready(size_t j, const std::vector<char> &d) const {
        for (int i : preds[j])
            if (!d[i]) return false;
        return true;
    }
    static bool strict_need(const BGate &x) {
        return (x.kind == BK_MAT1 && !x.diag) || x.kind == BK_CNOT || (x.kind == BK_OVL && x.axis != QF_PAULI_Z) ||
               x.kind == BK_BLOCK;
    }
    bool runnable(const BGate &x, uint64_t regs, bool force_diag) const {
        if (x.kind == BK_BLOCK) {  // every qubit of a dense block in a register position
            const uint64_t bm = block_mask(x);
            return (regs & bm) == bm;
        }
        if (x.kind == BK_MAT1)  // a diagonal gate on a qubit outside the tile never reaches a register
            return ((regs >> x.q0) & 1ULL) || (x.diag && (force_diag || !((p.resident >> x.q0) & 1ULL)));
        if (x.kind == BK_CNOT) return (regs >> x.q1) & 1ULL;
        if (x.kind == BK_OVL) return x.axis == QF_PAULI_Z || ((regs >> x.q0) & 1ULL);
        return true;
    }
    // gates that would run with `regs` in register positions, from state `d`
    // (updated); SWAPs move register membership with the labels
    int simulate(uint64_t regs, std::vector<char> &d, bool force_diag, int *strict) const {
        const auto &G = p.gates;
        int count = 0, st = 0;
        for (bool progress = true; progress;) {
            progress = false;
            for (size_t j = 0; j < G.size(); ++j) {
                if (d[j] || !ready(j, d) || !runnable(G[j], regs, force_diag)) continue;
                d[j] = 1;
                ++count;
                st += strict_need(G[j]);
                if (G[j].kind == BK_SWAP) {
                    const uint64_t a = (regs >> G[j].q0) & 1ULL, b = (regs >> G[j].q1) & 1ULL;
                    if (a != b) regs ^= (1ULL << G[j].q0) | (1ULL << G[j].q1);
                }
                progress = true;
            }
        }
        if (strict) *strict = st;
        return count;
    }
    // register qubits for the next layout: greedily the qubits that let the
    // most dense gates (then gates) run
    std::vector<uint32_t> choose_regs() const {
        std::vector<uint32_t> best = greedy_regs({});
        bool any_block = false;
        for (size_t j = 0; j < p.gates.size(); ++j) any_block = any_block || (!done[j] && p.gates[j].kind == BK_BLOCK);
        if (!any_block) return best;
        // a dense block runs only with all its qubits in registers: try each
        // ready block's qubits as the start of the register set
        auto score = [&](const std::vector<uint32_t> &S, int *dn) {
            uint64_t m = 0;
            for (uint32_t q : S) m |= 1ULL << q;
            std::vector<char> d = done;
            return simulate(m, d, false, dn);
        };
        int bd = 0;
        int ba = score(best, &bd);
        for (size_t j = 0; j < p.gates.size(); ++j) {
            const BGate &x = p.gates[j];
            if (done[j] || x.kind != BK_BLOCK || !ready(j, done)) continue;
            std::vector<uint32_t> base(x.bq, x.bq + x.nq);
            std::vector<uint32_t> S = greedy_regs(base);
            int dn = 0;
            const int all = score(S, &dn);
            if (dn > bd || (dn == bd && all > ba)) {
                best = S;
                bd = dn;
                ba = all;
            }
        }
        return best;
    }
    // from `base`, add the qubit that lets the most dense gates (then gates)
    // run, until four register qubits are chosen or no qubit adds a gate
    std::vector<uint32_t> greedy_regs(std::vector<uint32_t> S) const {
        uint64_t mask = 0;
        for (uint32_t q : S) mask |= 1ULL << q;
        int best_dense = -1, best_all = -1;
        {
            std::vector<char> d = done;
            best_all = simulate(mask, d, false, &best_dense);
        }
        for (int k = (int)S.size(); k < 4; ++k) {
            int pick = -1, pd = best_dense, pa = best_all;
            for (int s = K - 1; s >= 0; --s) {  // ties keep qubits 0..4 for the lanes
                const uint32_t q = slot_q[s];
                if ((mask >> q) & 1ULL) continue;
                std::vector<char> d = done;
                int dn = 0;
                const int all = simulate(mask | (1ULL << q), d, false, &dn);
                if (dn > pd || (dn == pd && all > pa)) {
                    pick = (int)q;
                    pd = dn;
                    pa = all;
                }
            }
            if (pick < 0) break;
            S.push_back((uint32_t)pick);
            mask |= 1ULL << pick;
            best_dense = pd;
            best_all = pa;
        }
        return S;
    }
    uint64_t reg_mask() const {
        uint64_t m = 0;
        for (int i = 5; i < 9; ++i) m |= 1ULL << L[i];
        return m;
    }
    // layout with `want` (up to four qubits) in the register positions, lanes
    // chosen for conflict-free shared-memory access
    void relayout(const std::vector<uint32_t> &want) {
        std::vector<uint32_t> regs(want.begin(), want.begin() + std::min<size_t>(want.size(), 4));
        for (int s = K - 1; s >= 0 && regs.size() < 4; --s)  // prefer high slots: keep 0..4 for the lanes
            if (std::find(regs.begin(), regs.end(), slot_q[s]) == regs.end()) regs.push_back(slot_q[s]);
        std::vector<int> free_slots;
        for (int s = 0; s < K; ++s)
            if (std::find(regs.begin(), regs.end(), slot_q[s]) == regs.end()) free_slots.push_back(s);
        uint32_t nl[kPosMax];
        std::vector<bool> used(K, false);
        auto take = [&](int s) {
            used[s] = true;
            return slot_q[s];
        };
        bool natural = true;
        for (int s = 0; s < 5; ++s) natural = natural && std::find(free_slots.begin(), free_slots.end(), s) != free_slots.end();
        // qubit 0 in a register goes to register bit 0: register pairs are
        // then adjacent in shared memory and move as 16-byte accesses
        const auto q0 = std::find(regs.begin(), regs.end(), slot_q[0]);
        if (q0 != regs.end()) std::iter_swap(regs.begin(), q0);
        if (natural) {
            for (int ps = 0; ps < 5; ++ps) nl[ps] = take(ps);
        } else {
            // The lanes of one access phase take slots whose bank vectors are
            // independent: an 8-byte access has half-warp phases (lane bits
            // 0..3 must reach all four bank bits, so slot 0 goes first), a
            // 16-byte one quarter-warp phases (lane bits 0..2, bank bits 1..3).
            const int phase_lanes = q0 != regs.end() ? 3 : 4;
            std::vector<uint32_t> basis;
            auto reduce = [&](uint32_t v) {
                for (uint32_t b : basis) v = std::min(v, v ^ b);
                return v;
            };
            for (int c = 0; c < 4; ++c) {
                int pick = -1;
                if (c < phase_lanes)
                    for (int s : free_slots)
                        if (!used[s] && reduce(bank_vec(s))) {
                            pick = s;
                            break;
                        }
                if (pick < 0)
                    for (int s : free_slots)
                        if (!used[s]) {
                            pick = s;
                            break;
                        }
                if (const uint32_t r = reduce(bank_vec(pick))) basis.push_back(r);
                nl[c] = take(pick);
            }
            int pick = -1;
            for (int s : free_slots)
                if (!used[s]) {
                    pick = s;
                    break;
                }
            nl[4] = take(pick);
        }
        for (int r = 0; r < 4; ++r) nl[5 + r] = regs[r];
        int w = 9;
        for (int s : free_slots)
            if (!used[s]) {
                nl[w++] = take(s);
            }
        std::memcpy(L, nl, sizeof(uint32_t) * K);
    }
    // shared-memory index of the thread part (lane and warp bits), as code
    std::string thread_index() const {
        std::ostringstream o;
        o << "(0u";
        for (int ps = 0; ps < 5; ++ps) o << " | (((lane >> " << ps << ") & 1u) << " << slot_of[L[ps]] << ")";
        for (int w = 0; w < WB; ++w) o << " | (((warp >> " << w << ") & 1u) << " << slot_of[L[9 + w]] << ")";
        o << ")";
        return o.str();
    }
    uint32_t reg_index(int i) const {
        uint32_t j = 0;
        for (int r = 0; r < 4; ++r)
            if ((i >> r) & 1) j |= 1u << slot_of[L[5 + r]];
        return j;
    }
    // register bit holding qubit 0 (the registers i and i | 1 << bit are then
    // adjacent in shared memory), or -1
    int pair_bit() const {
        for (int r = 0; r < 4; ++r)
            if (L[5 + r] == slot_q[0]) return r;
        return -1;
    }
    // arrays: 0 = psi (registers r*, shared S, global A), 1 = lambda (l*, SL, B)
    int n_arrays() const { return dual ? 2 : 1; }
    static const char *reg_pfx(int a) { return a ? "l" : "r"; }
    static const char *smem_of(int a) { return a ? "SL" : "S"; }
    static const char *glob_of(int a) { return a ? "B" : "A"; }
    // read all registers from shared memory in the current layout
    void emit_read() {
        const std::string pt = g.fresh("pt");
        g.s << "const unsigned " << pt << " = qf_phys(" << thread_index() << ");\n";
        const int pb = pair_bit();
        for (int a = 0; a < n_arrays(); ++a) {
            g.pfx = reg_pfx(a);
            const char *S_ = smem_of(a);
            if (pb >= 0) {
                for (int i = 0; i < kR; ++i)
                    if (!((i >> pb) & 1))
                        g.s << "{const float4 t = *reinterpret_cast<const float4*>(" << S_ << " + (" << pt << " ^ "
                            << physj(reg_index(i)) << "u)); " << g.R(i) << " = make_float2(t.x, t.y); " << g.R(i | (1 << pb))
                            << " = make_float2(t.z, t.w);}\n";
            } else {
                for (int i = 0; i < kR; ++i)
                    g.s << g.R(i) << " = " << S_ << "[" << pt << " ^ " << physj(reg_index(i)) << "u];\n";
            }
        }
        g.pfx = "r";
    }
    void emit_write() {
        const std::string pt = g.fresh("pt");
        g.s << "const unsigned " << pt << " = qf_phys(" << thread_index() << ");\n";
        const int pb = pair_bit();
        for (int a = 0; a < n_arrays(); ++a) {
            g.pfx = reg_pfx(a);
            const char *S_ = smem_of(a);
            if (pb >= 0) {
                for (int i = 0; i < kR; ++i)
                    if (!((i >> pb) & 1)) {
                        const std::string A_ = g.R(i), B_ = g.R(i | (1 << pb));
                        g.s << "*reinterpret_cast<float4*>(" << S_ << " + (" << pt << " ^ " << physj(reg_index(i))
                            << "u)) = make_float4(" << A_ << ".x, " << A_ << ".y, " << B_ << ".x, " << B_ << ".y);\n";
                    }
            } else {
                for (int i = 0; i < kR; ++i)
                    g.s << S_ << "[" << pt << " ^ " << physj(reg_index(i)) << "u] = " << g.R(i) << ";\n";
            }
        }
        g.pfx = "r";
    }
    // Canonical shared index of 16-byte chunk k of thread tid: j = 2*tid +
    // (tile/8)*k, so bits 0..4 are qubits 0..4, bits 5..K-4 slots 5..K-4 (tid
    // bits 4..), bits K-3..K-1 the chunk index (the top three slots).
    uint32_t chunk_j(int k) const { return (uint32_t)(tile_of(K) / 8) * (uint32_t)k; }
    uint64_t chunk_k_bits(int k) const {
        uint64_t a = 0;
        for (int b = 0; b < 3; ++b)
            if ((k >> b) & 1) a |= 1ULL << slot_q[K - 3 + b];
        return a;
    }

    // slots of this pass held as f64 accumulators, one per lane and 32 slots
    static constexpr int kMaxAcc = 4;
    int n_acc() const { return ((int)p.a.n_slots + 31) / 32; }
    std::streamoff prefetch_mark = -1;  // backward passes: where the next tile's load is spliced in

    void emit_issue(const std::string &tq) {
        auto &s = g.s;
        for (int a = 0; a < n_arrays(); ++a)
            for (int k = 0; k < kChunks; ++k)
                s << "qf_cpa16(sbase + (" << (a ? std::to_string(tile_of(K)) + "u + " : std::string()) << "(pt2 ^ " << physj(chunk_j(k)) << "u)) * 8u, "
                  << glob_of(a) << " + (" << tq << " | toff | " << hex64(chunk_k_bits(k)) << "));\n";
    }

    void emit_kernel(int index, bool last_pass) {
        auto &s = g.s;
        for (int i = 0; i < kR; ++i) g.v[i] = i;
        g.reset_scale();
        const std::string dep_t = deposit_code(p.a.nonlocal_mask, "t");
        const std::string dep_t2 = deposit_code(p.a.nonlocal_mask, "t2");
        if (dual && n_acc() > kMaxAcc) {
            failed = true;
            return;
        }
        if (!dual)
            s << "extern \"C\" __global__ void __launch_bounds__(" << threads_of(K) << ", "
              << (K == 12 ? (p.max_block >= 2 ? 2 : 3) : 1) << ") p" << index
              << "(float2* __restrict__ A, unsigned long long nt) {\n";
        else
            s << "extern \"C\" __global__ void __launch_bounds__(" << threads_of(K) << ", 2) b" << index
              << "(float2* __restrict__ A, float2* __restrict__ B, unsigned long long nt, double* __restrict__ partials, "
                 "unsigned stride) {\n";
        s << "extern __shared__ __align__(16) float2 SB[];\n";
        s << "const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, tid = threadIdx.x;\n";
        s << "const unsigned sbase = (unsigned)__cvta_generic_to_shared(SB);\n";
        // canonical shared index j = 2*tid + 512*k: bits 0..4 = qubits 0..4,
        // bits 5..8 = slots 5..8 (from tid >> 4), bits 9..11 = slots 9..11 (k)
        s << "const unsigned long long toff = (unsigned long long)((2u * tid) & 31u)";
        for (int b = 0; b < K - 8; ++b) s << " | ((tid & " << (16u << b) << "u) ? (1ull << " << slot_q[5 + b] << ") : 0ull)";
        s << ";\n";
        s << "const unsigned pt2 = qf_phys(2u * tid);\n";
        auto issue = [&](const std::string &tq, const std::string &buf) {
            for (int k = 0; k < kChunks; ++k)
                s << "qf_cpa16(sbase + ((" << buf << ") * " << tile_of(K) << "u + (pt2 ^ " << physj(chunk_j(k)) << "u)) * 8u, A + (" << tq
                  << " | toff | " << hex64(chunk_k_bits(k)) << "));\n";
        };
        s << "unsigned long long t = blockIdx.x;\n";
        if (!dual) {
            s << "if (t < nt) {const unsigned long long tq = " << dep_t << ";\n";
            issue("tq", "0u");
            s << "}\nasm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n";
            s << "for (unsigned it = 0; t < nt; t += gridDim.x, ++it) {\n";
            s << "const unsigned cur = it & 1u;\n";
            s << "{const unsigned long long t2 = t + gridDim.x; if (t2 < nt) {const unsigned long long tq = " << dep_t2 << ";\n";
            issue("tq", "cur ^ 1u");
            s << "}}\nasm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n";
            s << "asm volatile(\"cp.async.wait_group 1;\\n\" ::: \"memory\");\n__syncthreads();\n";
            s << "float2* S = SB + cur * " << tile_of(K) << "u;\n";
        } else {
            // one psi + lambda buffer; the next tile streams in after the last
            // shared-memory read of the current one
            // overlap sums per lane as an unevaluated pair of floats (hi + lo,
            // every addition's rounding error carried in lo): the precision of
            // an f64 accumulator without the FP64 pipe, which GB300 runs at a
            // small fraction of its FP32 rate
            for (int a = 0; a < n_acc(); ++a) s << "float acc" << a << "h = 0.f, acc" << a << "l = 0.f;\n";
            s << "if (t < nt) {const unsigned long long tq = " << dep_t << ";\n";
            emit_issue("tq");
            s << "}\nasm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n";
            s << "for (; t < nt; t += gridDim.x) {\n";
            s << "asm volatile(\"cp.async.wait_group 0;\\n\" ::: \"memory\");\n__syncthreads();\n";
            s << "float2* S = SB;\nfloat2* SL = SB + " << tile_of(K) << "u;\n";
        }
        s << "const unsigned long long tb = " << dep_t << ";\n";
        s << "float2 tph = make_float2(1.f, 0.f);\n";  // deferred per-thread phase (psi and lambda alike)
        phase_pending = false;
        for (int a = 0; a < n_arrays(); ++a)
            for (int i = 0; i < kR; ++i) s << "float2 " << reg_pfx(a) << i << ";\n";
        build_deps();
        relayout(choose_regs());
        emit_read();
        s << "__syncthreads();\n";
        prefetch_mark = (std::streamoff)s.tellp();
        const auto &G = p.gates;
        size_t left = G.size();
        bool remapped = false;
        while (left) {
            bool progress = false;
            for (size_t j = 0; j < G.size() && left; ++j) {
                if (done[j] || is_zovl(G[j]) || !ready(j, done) || !runnable(G[j], reg_mask(), false)) continue;
                emit_gate(G[j]);
                order.push_back((int)j);
                done[j] = 1;
                --left;
                progress = true;
                j = (size_t)-1;  // rescan: the gate may have released earlier ones
            }
            if (progress) remapped = false;
            if (!left || progress) continue;
            if (dual) {  // nothing else runs: every ready Z-axis overlap at once
                std::vector<int> zs;
                for (size_t j = 0; j < G.size(); ++j)
                    if (!done[j] && is_zovl(G[j]) && ready(j, done)) zs.push_back((int)j);
                if (!zs.empty()) {
                    emit_overlap_group(zs);
                    for (int j : zs) {
                        order.push_back(j);
                        done[j] = 1;
                        --left;
                    }
                    remapped = false;
                    continue;
                }
            }
            bool dense_left = false;
            for (size_t j = 0; j < G.size(); ++j) dense_left = dense_left || (!done[j] && strict_need(G[j]));
            if (!dense_left || remapped) {  // only diagonal gates hold things up: run one where its qubit is
                bool ran = false;
                for (size_t j = 0; j < G.size(); ++j)
                    if (!done[j] && ready(j, done) && runnable(G[j], reg_mask(), true)) {
                        emit_gate(G[j]);
                        order.push_back((int)j);
                        done[j] = 1;
                        --left;
                        ran = true;
                        break;
                    }
                if (!ran) {  // cannot happen for a planned pass: every dense target is resident
                    failed = true;
                    return;
                }
                remapped = false;
                continue;
            }
            s << "{\n";  // remap: a new layout with the chosen qubits in register positions
            flush_phase();
            emit_write();
            s << "__syncthreads();\n";
            relayout(choose_regs());
            emit_read();
            s << "__syncthreads();\n}\n";
            prefetch_mark = (std::streamoff)s.tellp();
            remapped = true;
        }
        finish(last_pass, dep_t2);
    }

    // Im<lambda|P_q psi> over the thread's amplitudes (the adjoint term of
    // src/lib.rs:3648-3664, summed as the shared-memory kernel does), reduced
    // over the warp in f32 and added to the slot's f64 accumulator (held by
    // lane slot % 32).
    // Z-axis overlaps of a backward pass are held back until nothing else can
    // run, then evaluated together: Im<lambda|Z_q psi> commutes with every gate
    // still pending before it (none of them acts off-diagonal on q), and all of
    // them share the per-amplitude products w_i = Im(conj(l_i) r_i).
    bool is_zovl(const BGate &x) const { return dual && x.kind == BK_OVL && x.axis == QF_PAULI_Z; }
    static std::string tree_sum(const std::vector<std::string> &v, size_t b, size_t e) {
        if (e - b == 1) return v[b];
        const size_t m = b + (e - b) / 2;
        return "(" + tree_sum(v, b, m) + " + " + tree_sum(v, m, e) + ")";
    }
    void emit_overlap_group(const std::vector<int> &js) {
        auto &s = g.s;
        const auto &G = p.gates;
        s << "{\n";
        std::vector<std::string> w;
        for (int i = 0; i < kR; ++i) {
            const std::string l = "l" + std::to_string(g.v[i]), r = "r" + std::to_string(g.v[i]);
            s << "const float w" << i << " = " << l << ".x * " << r << ".y - " << l << ".y * " << r << ".x;\n";
            w.push_back("w" + std::to_string(i));
        }
        s << "const float wt = " << tree_sum(w, 0, w.size()) << ";\n";
        uint32_t rbits = 0;
        for (int j : js) {
            const uint8_t d = desc(G[j].q0);
            if (is_reg(d)) rbits |= 1u << (d - 8);
        }
        for (int rb = 0; rb < 4; ++rb) {  // sum over register bit rb clear minus bit set = 2 (clear) - total
            if (!((rbits >> rb) & 1u)) continue;
            std::vector<std::string> c;
            for (int i = 0; i < kR; ++i)
                if (!((i >> rb) & 1)) c.push_back(w[i]);
            s << "const float wz" << rb << " = 2.f * " << tree_sum(c, 0, c.size()) << " - wt;\n";
        }
        for (int j : js) {
            const BGate &x = G[j];
            const uint8_t d = desc(x.q0);
            s << "{float ov = ";
            if (is_reg(d)) s << "wz" << (d - 8) << ";\n";
            else s << "(" << cbit(d) << ") ? -wt : wt;\n";
            emit_overlap_sum(x);
            s << "}\n";
        }
        s << "}\n";
    }
    // the overlap value `ov` of x (psi and lambda scale by |G|^2), reduced over
    // the warp and added to the slot's float-pair accumulator
    void emit_overlap_sum(const BGate &x) {
        auto &s = g.s;
        const int ls = (int)x.op_index - (int)p.a.slot_base;
        // psi and lambda both wait for the deferred phase: <l|P|p> carries |tph|^2
        if (phase_pending) s << "ov *= tph.x * tph.x + tph.y * tph.y;\n";
        if (g.any_scale) {
            const int sl = g.slot(std::norm(g.pscale), 0.0, 0.0, 0.0);
            s << "ov *= " << Mref(sl, 0) << ".x;\n";
        }
        for (int o = 16; o >= 1; o >>= 1) s << "ov += __shfl_xor_sync(0xffffffffu, ov, " << o << ");\n";
        const std::string ah = "acc" + std::to_string(ls >> 5) + "h", al = "acc" + std::to_string(ls >> 5) + "l";
        s << "if (lane == " << (ls & 31) << "u) {const float sm = " << ah << " + ov, bb = sm - " << ah << "; " << al << " += ("
          << ah << " - (sm - bb)) + (ov - bb); " << ah << " = sm;}\n";
    }

    void emit_overlap(const BGate &x) {
        auto &s = g.s;
        auto R_ = [&](int i) { return "r" + std::to_string(g.v[i]); };
        auto L_ = [&](int i) { return "l" + std::to_string(g.v[i]); };
        s << "{float ov = 0.f;\n";
        const uint8_t d = desc(x.q0);
        if (x.axis == QF_PAULI_Z) {
            const int rb = is_reg(d) ? d - 8 : -1;
            for (int i = 0; i < kR; ++i) {
                const bool neg = rb >= 0 && ((i >> rb) & 1);
                s << "ov " << (neg ? "-" : "+") << "= " << L_(i) << ".x * " << R_(i) << ".y - " << L_(i) << ".y * " << R_(i)
                  << ".x;\n";
            }
            if (rb < 0) s << "if (" << cbit(d) << ") ov = -ov;\n";
        } else {
            const int rb = d - 8;
            const bool y = x.axis == QF_PAULI_Y;
            for (int i = 0; i < kR; ++i) {
                if ((i >> rb) & 1) continue;
                const int j = i | (1 << rb);
                const std::string l0 = L_(i), l1 = L_(j), p0 = R_(i), p1 = R_(j);
                if (!y)
                    s << "ov += (" << l0 << ".x * " << p1 << ".y - " << l0 << ".y * " << p1 << ".x) + (" << l1 << ".x * " << p0
                      << ".y - " << l1 << ".y * " << p0 << ".x);\n";
                else
                    s << "ov += -(" << l0 << ".x * " << p1 << ".x + " << l0 << ".y * " << p1 << ".y) + (" << l1 << ".x * " << p0
                      << ".x + " << l1 << ".y * " << p0 << ".y);\n";
            }
        }
        emit_overlap_sum(x);  // psi and lambda both carry the factor G pulled out so far
        s << "}\n";
    }

    void emit_gate(const BGate &x) {
        auto &s = g.s;
        switch (x.kind) {
        case BK_MAT1: {
            std::complex<double> m[4] = {{x.m[0], x.m[1]}, {x.m[2], x.m[3]}, {x.m[4], x.m[5]}, {x.m[6], x.m[7]}};
            if (x.diag) {  // diag(m00, m11) = m00 * diag(1, m11/m00)
                g.any_diag = true;
                g.gphase *= m[0];
                const std::complex<double> f = m[3] / m[0];
                const int sl = g.slot(f, 0.0, 0.0, f);
                const uint8_t d = desc(x.q0);
                for (int a = 0; a < n_arrays(); ++a) {
                    g.pfx = reg_pfx(a);
                    if (is_reg(d)) {
                        const int rb = d - 8;
                        for (int i = 0; i < kR; ++i)
                            if ((i >> rb) & 1) emit_cmul_const(g, g.R(i), sl, 0);
                    } else if (a == 0) {
                        // a lane, warp or outside-the-tile bit is constant over the thread's
                        // registers: the factor goes into the thread's deferred phase
                        // (applied once, before the next remap or the store; backward
                        // passes apply the same factor to psi and lambda)
                        s << "if (" << cbit(d) << ") ";
                        emit_cmul_const(g, "tph", sl, 0);
                        phase_pending = true;
                    }
                }
            } else {
                const int mk = matrix_kind_of(m);
                const Factored fg = x.varying ? Factored() : factor_gate(m, mk);
                if (fg.ok && g.n_factored >= kMaxFactors) emit_scale();
                int sl;
                if (fg.ok)
                    sl = slot_factored(g, fg);
                else if (mk == 1)  // splatted real entries for packed f32x2 arithmetic
                    sl = g.slot({m[0].real(), m[0].real()}, {m[1].real(), m[1].real()}, {m[2].real(), m[2].real()},
                                {m[3].real(), m[3].real()});
                else
                    sl = g.slot(m[0], m[1], m[2], m[3]);
                const int rb = pos_of(x.q0) - 5;
                for (int a = 0; a < n_arrays(); ++a) {
                    g.pfx = reg_pfx(a);
                    for (int i = 0; i < kR; ++i)
                        if (!((i >> rb) & 1)) {
                            if (fg.ok) emit_factored(g, sl, fg, g.R(i), g.R(i | (1 << rb)));
                            else emit_mat2(g, sl, mk, g.R(i), g.R(i | (1 << rb)));
                        }
                }
            }
            break;
        }
        case BK_CNOT: {
            const uint8_t dc = desc(x.q0);
            const int tb_ = pos_of(x.q1) - 5;
            if (is_reg(dc)) {  // rename only (the same for both arrays)
                const int cb = dc - 8;
                for (int i = 0; i < kR; ++i)
                    if (((i >> cb) & 1) && !((i >> tb_) & 1)) std::swap(g.v[i], g.v[i | (1 << tb_)]);
            } else {
                s << "if (" << cbit(dc) << ") {\n";
                for (int a = 0; a < n_arrays(); ++a) {
                    g.pfx = reg_pfx(a);
                    for (int i = 0; i < kR; ++i)
                        if (!((i >> tb_) & 1)) {
                            const std::string A_ = g.R(i), B_ = g.R(i | (1 << tb_));
                            s << "{const float2 x=" << A_ << "; " << A_ << "=" << B_ << "; " << B_ << "=x;}\n";
                        }
                }
                s << "}\n";
            }
            break;
        }
        case BK_CZ: {
            const uint8_t da = desc(x.q0), db = desc(x.q1);
            auto neg = [&](int i) { s << g.R(i) << ".x = -" << g.R(i) << ".x; " << g.R(i) << ".y = -" << g.R(i) << ".y;\n"; };
            for (int a = 0; a < n_arrays(); ++a) {
                g.pfx = reg_pfx(a);
                if (is_reg(da) && is_reg(db)) {
                    for (int i = 0; i < kR; ++i)
                        if (((i >> (da - 8)) & 1) && ((i >> (db - 8)) & 1)) neg(i);
                } else if (is_reg(da) || is_reg(db)) {
                    const int b = (is_reg(da) ? da : db) - 8;
                    s << "if (" << cbit(is_reg(da) ? db : da) << ") {\n";
                    for (int i = 0; i < kR; ++i)
                        if ((i >> b) & 1) neg(i);
                    s << "}\n";
                } else if (a == 0) {  // both bits constant over the thread's registers: the deferred phase
                    s << "if (" << cbit(da) << " & " << cbit(db) << ") {tph.x = -tph.x; tph.y = -tph.y;}\n";
                    phase_pending = true;
                }
            }
            break;
        }
        case BK_OVL: emit_overlap(x); break;
        case BK_BLOCK: emit_block(x); break;
        default: {  // SWAP of two resident qubits: relabel
            const int a = pos_of(x.q0), b = pos_of(x.q1);
            std::swap(L[a], L[b]);
            break;
        }
        }
        g.pfx = "r";
    }

    // A dense 2^m x 2^m block (m <= 4) whose qubits all sit in register
    // positions: for every setting of the other register bits, the thread's
    // 2^m amplitudes times the block's matrix (row-major in the constant
    // bank), four FMAs per complex multiply-add.
    void emit_block(const BGate &x) {
        auto &s = g.s;
        const int m = x.nq, D = 1 << m;
        int rb[kMaxBlockQubits];
        uint32_t bits = 0;
        for (int i = 0; i < m; ++i) {
            rb[i] = pos_of(x.bq[i]) - 5;
            bits |= 1u << rb[i];
        }
        const int base = block_slots(g, *bmats, x.boff, D);
        for (int i0 = 0; i0 < kR; ++i0) {
            if (i0 & (int)bits) continue;
            auto idx = [&](int c) {
                int r = i0;
                for (int i = 0; i < m; ++i)
                    if ((c >> i) & 1) r |= 1 << rb[i];
                return r;
            };
            s << "{";
            for (int c = 0; c < D; ++c) s << "const float2 x" << c << "=" << g.R(idx(c)) << ";";
            s << "\n";
            for (int r = 0; r < D; ++r) {
                std::ostringstream re, im;
                for (int c = 0; c < D; ++c) {
                    const std::string e = "M[" + std::to_string(4 * base + r * D + c) + "]";
                    re << (c ? "+" : "") << e << ".x*x" << c << ".x-" << e << ".y*x" << c << ".y";
                    im << (c ? "+" : "") << e << ".x*x" << c << ".y+" << e << ".y*x" << c << ".x";
                }
                s << g.R(idx(r)) << ".x=" << re.str() << ";" << g.R(idx(r)) << ".y=" << im.str() << ";\n";
            }
            s << "}\n";
        }
    }

    // the deferred per-thread phase of diagonal gates on lane, warp and
    // outside-the-tile bits, multiplied into the registers (forward passes)
    bool phase_pending = false;
    void flush_phase() {
        if (!phase_pending) return;
        auto &s = g.s;
        const std::string keep = g.pfx;
        for (int a = 0; a < n_arrays(); ++a) {
            g.pfx = reg_pfx(a);
            for (int i = 0; i < kR; ++i) {
                const std::string R = g.R(i);
                s << "{const float2 x=" << R << ";" << R << ".x=tph.x*x.x-tph.y*x.y;" << R << ".y=tph.x*x.y+tph.y*x.x;}\n";
            }
        }
        g.pfx = keep;
        s << "tph = make_float2(1.f, 0.f);\n";
        phase_pending = false;
    }

    // multiply the tile (psi and lambda alike) by the factors pulled out so
    // far, a real or an imaginary scalar, and start a new product
    void emit_scale() {
        auto &s = g.s;
        const int sl = g.slot(scale_const(g), 0.0, 0.0, 0.0);
        const std::string f = Mref(sl, 0);
        for (int a = 0; a < n_arrays(); ++a) {
            g.pfx = reg_pfx(a);
            for (int i = 0; i < kR; ++i) {
                const std::string R = g.R(i);
                if (g.pscale_imag) s << R << "=qf_fmul2(" << f << ",make_float2(" << R << ".y," << R << ".x));\n";
                else s << R << "=qf_fmul2(" << f << "," << R << ");\n";
            }
        }
        g.pfx = "r";
        g.reset_scale();
    }

    void finish(bool last_pass, const std::string &dep_t2) {
        auto &s = g.s;
        flush_phase();
        if (last_pass && g.any_diag) {  // the plan's global phase, once, at the very end (with this pass's factors)
            const int sl = g.slot(g.gphase * g.pscale, 0.0, 0.0, 0.0);
            for (int a = 0; a < n_arrays(); ++a) {
                g.pfx = reg_pfx(a);
                for (int i = 0; i < kR; ++i) emit_cmul_const(g, g.R(i), sl, 0);
            }
            g.pfx = "r";
        } else if (g.any_scale) {  // the factors pulled out of this pass's gates
            emit_scale();
        }
        const std::string prefetch = "{const unsigned long long t2 = t + gridDim.x; if (t2 < nt) {const unsigned long long tq = " +
                                     dep_t2 + ";\n";
        bool natural = true;
        for (int ps = 0; ps < 5; ++ps) natural = natural && L[ps] == (uint32_t)ps;
        if (natural) {  // lanes hold qubits 0..4: store straight from registers
            if (dual) {  // shared memory is free from the last read on: start the next tile there
                std::string txt = s.str();
                std::ostringstream keep;
                std::swap(keep, g.s);  // emit the copy code into a fresh stream
                emit_issue("tq");
                const std::string issue_code = g.s.str();
                std::swap(keep, g.s);
                txt.insert((size_t)prefetch_mark,
                           prefetch + issue_code + "}}\nasm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n");
                s.str("");
                s.clear();
                s << txt;
            }
            s << "const unsigned long long sw = 0ull";
            for (int w = 0; w < WB; ++w) s << " | ((warp & " << (1 << w) << "u) ? (1ull << " << L[9 + w] << ") : 0ull)";
            s << ";\n";
            for (int a = 0; a < n_arrays(); ++a) {
                g.pfx = reg_pfx(a);
                for (int i = 0; i < kR; ++i) {
                    uint64_t off = 0;
                    for (int r = 0; r < 4; ++r)
                        if ((i >> r) & 1) off |= 1ULL << L[5 + r];
                    s << glob_of(a) << "[(tb | lane | sw) | " << hex64(off) << "] = " << g.R(i) << ";\n";
                }
            }
            g.pfx = "r";
        } else {  // through shared memory, 16-byte coalesced stores
            emit_write();
            s << "__syncthreads();\n";
            for (int a = 0; a < n_arrays(); ++a)
                for (int k = 0; k < kChunks; ++k)
                    s << "*reinterpret_cast<float4*>(" << glob_of(a) << " + (tb | toff | " << hex64(chunk_k_bits(k))
                      << ")) = *reinterpret_cast<const float4*>(" << smem_of(a) << " + (pt2 ^ " << physj(chunk_j(k)) << "u));\n";
            s << "__syncthreads();\n";
            if (dual) {
                s << prefetch;
                emit_issue("tq");
                s << "}}\nasm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n";
            }
        }
        s << "}\n";  // tile loop
        if (dual) {  // per-CTA slot sums, warps in order
            s << "asm volatile(\"cp.async.wait_group 0;\\n\" ::: \"memory\");\n__syncthreads();\n";
            s << "double* RD = reinterpret_cast<double*>(SB);\n";
            for (int a = 0; a < n_acc(); ++a)
                s << "if (lane + " << 32 * a << "u < " << p.a.n_slots << "u) RD[(lane + " << 32 * a << "u) * 8u + warp] = (double)acc"
                  << a << "h + (double)acc" << a << "l;\n";
            s << "__syncthreads();\n";
            s << "for (unsigned k = tid; k < " << p.a.n_slots << "u; k += " << threads_of(K) << "u) {double v = 0.0;"
              << " for (unsigned w = 0; w < 8u; ++w) v += RD[k * 8u + w];"
              << " partials[(size_t)(" << p.a.slot_base << "u + k) * stride + blockIdx.x] = v;}\n";
        }
        s << "}\n";  // kernel
    }
};

struct JitModule {
    cudaLibrary_t lib = nullptr;
    std::vector<cudaKernel_t> kernels;
    void *consts = nullptr;
    size_t consts_bytes = 0;
};

struct JitCache {
    std::mutex mu;
    std::map<std::string, std::shared_ptr<JitModule>> mods;
};

JitCache &cache() {
    static JitCache c;
    return c;
}


const char *kPrelude =
    "__device__ __forceinline__ void qf_cpa16(unsigned s, const float2* g) {"
    " asm volatile(\"cp.async.cg.shared.global [%0], [%1], 16;\\n\" :: \"r\"(s), \"l\"(g) : \"memory\"); }\n"
    "__device__ __forceinline__ unsigned qf_phys(unsigned j) { const unsigned h = (j >> 4) & 0x1FFu;"
    " return j ^ ((__popc(h & 0xE9u) & 1u) << 1) ^ ((__popc(h & 0x15Au) & 1u) << 2) ^ ((__popc(h & 0x74u) & 1u) << 3); }\n"
    "__device__ __forceinline__ unsigned long long qf_pk(float2 v) { unsigned long long r;"
    " asm(\"mov.b64 %0, {%1, %2};\" : \"=l\"(r) : \"f\"(v.x), \"f\"(v.y)); return r; }\n"
    "__device__ __forceinline__ float2 qf_upk(unsigned long long r) { float2 v;"
    " asm(\"mov.b64 {%0, %1}, %2;\" : \"=f\"(v.x), \"=f\"(v.y) : \"l\"(r)); return v; }\n"
    "__device__ __forceinline__ float2 qf_ffma2(float2 a, float2 b, float2 c) { unsigned long long d;"
    " asm(\"fma.rn.f32x2 %0, %1, %2, %3;\" : \"=l\"(d) : \"l\"(qf_pk(a)), \"l\"(qf_pk(b)), \"l\"(qf_pk(c))); return qf_upk(d); }\n"
    "__device__ __forceinline__ float2 qf_fmul2(float2 a, float2 b) { unsigned long long d;"
    " asm(\"mul.rn.f32x2 %0, %1, %2;\" : \"=l\"(d) : \"l\"(qf_pk(a)), \"l\"(qf_pk(b))); return qf_upk(d); }\n";

const char *kNvrtcOpts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device", "-lineinfo"};

// kernels p0, p1, ... (forward passes) or b0, b1, ... (backward passes)
int compile_module(const std::string &src, int n_kernels, int device, JitModule &out, std::string &err, char prefix) {
    Nvrtc &nv = nvrtc();
    if (!nv.ok) {
        err = nv.why;
        return QF_ERR_UNSUPPORTED_OPERATION;
    }
    nvrtcProgram prog;
    if (nv.create(&prog, src.c_str(), "qf_pass.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        err = "nvrtcCreateProgram failed";
        return QF_ERR_CUDA;
    }
    nvrtcResult r = nv.compile(prog, 4, kNvrtcOpts);
    if (r != NVRTC_SUCCESS) {
        size_t ls = 0;
        nv.log_size(prog, &ls);
        std::string log(ls, '\0');
        nv.log(prog, &log[0]);
        err = std::string("NVRTC: ") + nv.err(r) + ": " + log.substr(0, 2000);
        nv.destroy(&prog);
        return QF_ERR_CUDA;
    }
    size_t cs = 0;
    nv.cubin_size(prog, &cs);
    std::vector<char> cubin(cs);
    nv.cubin(prog, cubin.data());
    nv.destroy(&prog);
    cudaError_t e = cudaLibraryLoadData(&out.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
        return QF_ERR_CUDA;
    }
    out.kernels.resize(n_kernels);
    for (int k = 0; k < n_kernels; ++k) {
        const std::string nm = std::string(1, prefix) + std::to_string(k);
        if ((e = cudaLibraryGetKernel(&out.kernels[k], out.lib, nm.c_str())) != cudaSuccess) {
            err = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(e);
            return QF_ERR_CUDA;
        }
        if ((e = cudaKernelSetAttributeForDevice(out.kernels[k], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)dyn_smem_of(kPosMax), device)) != cudaSuccess) {
            err = std::string("cudaKernelSetAttributeForDevice: ") + cudaGetErrorString(e);
            return QF_ERR_CUDA;
        }
    }
    if ((e = cudaLibraryGetGlobal(&out.consts, &out.consts_bytes, out.lib, "M")) != cudaSuccess) {
        err = std::string("cudaLibraryGetGlobal: ") + cudaGetErrorString(e);
        return QF_ERR_CUDA;
    }
    return QF_OK;
}

struct ModulePlan {
    char prefix = 'p';  // kernel names: p<k> forward, b<k> backward
    std::shared_ptr<const std::string> src;
    std::vector<float> consts;  // interleaved float2
    std::vector<int> pass_index;
};

// a pass the compiled kernels can run: 12 resident qubits including 0..4
// a pass the compiled kernels can run: 12 resident qubits (or 13 forward)
// including 0..4
bool pass_fits(const Pass &p, bool dual) {
    const int K = __builtin_popcountll(p.resident);
    return (K == 12 || (!dual && K == 13)) && (p.resident & 31ULL) == 31ULL;
}
int pass_k(const Pass &p) { return __builtin_popcountll(p.resident); }

// group passes into modules: at most 8 passes and 56 KB of constants each
// Everything of a plan that shapes its generated source: per pass the
// resident qubits and, per gate, kind, qubits, diagonal flag, matrix kind,
// overlap axis and slot. Matrix values only enter the constant banks.
std::string plan_key(const Plan &plan, bool dual) {
    std::string k;
    auto put = [&](uint64_t v, int bytes) {
        for (int b = 0; b < bytes; ++b) k.push_back((char)((v >> (8 * b)) & 0xFF));
    };
    put(plan.n, 1);
    put(dual, 1);
    put(plan.passes.size(), 4);
    for (const Pass &p : plan.passes) {
        put(p.resident, 8);
        put(p.gates.size(), 4);
        for (const BGate &x : p.gates) {
            uint8_t mk = 0;
            if (x.kind == BK_MAT1 && !x.diag) {
                const std::complex<double> m[4] = {{x.m[0], x.m[1]}, {x.m[2], x.m[3]}, {x.m[4], x.m[5]}, {x.m[6], x.m[7]}};
                mk = matrix_kind_of(m);
            }
            put(x.kind | (x.diag << 3) | (mk << 4), 1);
            if (x.kind == BK_MAT1 && !x.diag) {
                const std::complex<double> m[4] = {{x.m[0], x.m[1]}, {x.m[2], x.m[3]}, {x.m[4], x.m[5]}, {x.m[6], x.m[7]}};
                put(x.varying ? 0 : factored_code(factor_gate(m, mk)), 1);
            }
            put(x.q0, 1);
            put(x.q1, 1);
            if (x.kind == BK_BLOCK) {
                put(x.nq, 1);
                for (int i = 0; i < x.nq; ++i) put(x.bq[i], 1);
            }
            if (x.kind == BK_OVL) {
                put(x.axis, 1);
                put((uint64_t)x.op_index, 4);
            }
        }
    }
    return k;
}

// The constant banks of modules generated for `plan`, rebuilt from the gates
// in each pass's emission order exactly as emit_gate / finish allocate them.
void replay_consts(const Plan &plan, const std::vector<std::vector<int>> &orders, std::vector<ModulePlan> &mods) {
    Gen g;
    const size_t npass = plan.passes.size();
    for (ModulePlan &mp : mods) {
        g.consts.clear();
        for (int pi : mp.pass_index) {
            const Pass &p = plan.passes[pi];
            g.reset_scale();
            for (int j : orders[pi]) {
                const BGate &x = p.gates[j];
                if (x.kind == BK_OVL && g.any_scale) g.slot(std::norm(g.pscale), 0.0, 0.0, 0.0);
                if (x.kind == BK_BLOCK) block_slots(g, plan.bmats, x.boff, 1 << x.nq);
                if (x.kind != BK_MAT1) continue;
                const std::complex<double> m[4] = {{x.m[0], x.m[1]}, {x.m[2], x.m[3]}, {x.m[4], x.m[5]}, {x.m[6], x.m[7]}};
                if (x.diag) {
                    g.any_diag = true;
                    g.gphase *= m[0];
                    const std::complex<double> f = m[3] / m[0];
                    g.slot(f, 0.0, 0.0, f);
                } else {
                    const int mk = matrix_kind_of(m);
                    const Factored fg = x.varying ? Factored() : factor_gate(m, mk);
                    if (fg.ok && g.n_factored >= kMaxFactors) {
                        g.slot(scale_const(g), 0.0, 0.0, 0.0);
                        g.reset_scale();
                    }
                    if (fg.ok)
                        slot_factored(g, fg);
                    else if (mk == 1)
                        g.slot({m[0].real(), m[0].real()}, {m[1].real(), m[1].real()}, {m[2].real(), m[2].real()},
                               {m[3].real(), m[3].real()});
                    else
                        g.slot(m[0], m[1], m[2], m[3]);
                }
            }
            if ((size_t)pi + 1 == npass && g.any_diag) g.slot(g.gphase * g.pscale, 0.0, 0.0, 0.0);
            else if (g.any_scale) g.slot(scale_const(g), 0.0, 0.0, 0.0);
        }
        mp.consts.clear();
        mp.consts.reserve(g.consts.size() * 2);
        for (auto &c : g.consts) {
            mp.consts.push_back((float)c.real());
            mp.consts.push_back((float)c.imag());
        }
    }
}

struct GenEntry {
    std::vector<ModulePlan> mods;        // sources; constants refilled per use
    std::vector<std::vector<int>> orders;  // per pass: gate indices in emission order
};
struct GenCache {
    std::mutex mu;
    std::map<std::string, std::shared_ptr<const GenEntry>> entries;
};
GenCache &gen_cache() {
    static GenCache c;
    return c;
}

// Upper bound of the constant-bank bytes one pass adds.
size_t pass_const_bytes(const Pass &p) {
    size_t b = 64;
    for (const BGate &x : p.gates) {
        if (x.kind == BK_BLOCK) b += (size_t)8 << (2 * x.nq);
        else b += 2 * 32;  // a matrix (plus a possible mid-pass scale)
    }
    return b;
}

bool gen_modules_uncached(const Plan &plan, std::vector<ModulePlan> &mods, std::vector<std::vector<int>> &orders,
                          bool dual) {
    Gen g;
    const size_t npass = plan.passes.size();
    orders.assign(npass, {});
    size_t pi = 0;
    while (pi < npass) {
        ModulePlan mp;
        mp.prefix = dual ? 'b' : 'p';
        std::ostringstream body;
        g.consts.clear();
        int local = 0;
        while (pi < npass && local < 8 && (local == 0 || g.consts.size() * 8 + pass_const_bytes(plan.passes[pi]) < 60 * 1024)) {
            g.s.str("");
            g.s.clear();
            PassGen pg(g, plan.passes[pi], plan.n, dual, &plan.bmats);
            pg.emit_kernel(local, pi + 1 == npass);
            if (pg.failed) return false;
            body << g.s.str();
            orders[pi] = pg.order;
            mp.pass_index.push_back((int)pi);
            ++pi;
            ++local;
        }
        std::ostringstream head;
        head << "__constant__ float2 M[" << std::max<size_t>(1, g.consts.size()) << "];\n" << kPrelude;
        mp.src = std::make_shared<const std::string>(head.str() + body.str());
        mp.consts.reserve(g.consts.size() * 2);
        for (auto &c : g.consts) {
            mp.consts.push_back((float)c.real());
            mp.consts.push_back((float)c.imag());
        }
        mods.push_back(std::move(mp));
    }
    return true;
}

// Modules of a plan: generated once per structure, constants per call.
bool gen_modules(const Plan &plan, std::vector<ModulePlan> &mods, bool dual = false) {
    const std::string key = plan_key(plan, dual);
    std::shared_ptr<const GenEntry> hit;
    {
        std::lock_guard<std::mutex> lk(gen_cache().mu);
        auto it = gen_cache().entries.find(key);
        if (it != gen_cache().entries.end()) hit = it->second;
    }
    if (hit) {
        mods = hit->mods;
        replay_consts(plan, hit->orders, mods);
        return true;
    }
    auto e = std::make_shared<GenEntry>();
    if (!gen_modules_uncached(plan, e->mods, e->orders, dual)) return false;
    mods = e->mods;
    std::lock_guard<std::mutex> lk(gen_cache().mu);
    if (gen_cache().entries.size() > 256) gen_cache().entries.clear();  // bound the host memory of the cache
    gen_cache().entries[key] = e;
    return true;
}

}  // namespace

bool jit_available() { return nvrtc().ok; }

bool jit_plan_fits(const Plan &plan, bool dual = false) {
    if (plan.n < 12 || plan.passes.empty()) return false;
    for (const Pass &p : plan.passes)
        if (!pass_fits(p, dual) || pass_k(p) != pass_k(plan.passes[0])) return false;
    return true;
}

// Generated sources and an NVRTC compile without loading (needs no GPU).
int jit_check_compile(const Plan &plan, int, std::string *source, std::string *err, bool dual) {
    if (!jit_plan_fits(plan, dual)) return fail(QF_ERR_UNSUPPORTED_OPERATION, "plan has a pass outside the compiled layout");
    std::vector<ModulePlan> mods;
    if (!gen_modules(plan, mods, dual)) return fail(QF_ERR_UNSUPPORTED_OPERATION, "pass compiler could not schedule a pass");
    Nvrtc &nv = nvrtc();
    if (!nv.ok) return fail(QF_ERR_UNSUPPORTED_OPERATION, "%s", nv.why.c_str());
    for (auto &m : mods) {
        if (source) *source += *m.src;
        nvrtcProgram prog;
        nv.create(&prog, m.src->c_str(), "qf_pass.cu", 0, nullptr, nullptr);
        nvrtcResult r = nv.compile(prog, 3, kNvrtcOpts);
        if (r != NVRTC_SUCCESS) {
            size_t ls = 0;
            nv.log_size(prog, &ls);
            std::string log(ls, '\0');
            nv.log(prog, &log[0]);
            if (err) *err = log;
            nv.destroy(&prog);
            return QF_ERR_CUDA;
        }
        nv.destroy(&prog);
    }
    return QF_OK;
}

namespace {
// Compiled modules for `mods`, from the cache or compiled in parallel.
int fetch_modules(qf_ctx *ctx, const std::vector<ModulePlan> &mods, std::vector<std::shared_ptr<JitModule>> &handles) {
    handles.assign(mods.size(), nullptr);
    std::vector<size_t> todo;
    {
        std::lock_guard<std::mutex> lk(cache().mu);
        for (size_t m = 0; m < mods.size(); ++m) {
            auto it = cache().mods.find(*mods[m].src);
            if (it != cache().mods.end()) handles[m] = it->second;
            else todo.push_back(m);
        }
    }
    if (todo.empty()) return QF_OK;
    std::vector<int> st(todo.size(), QF_OK);
    std::vector<std::string> errs(todo.size());
    std::vector<std::shared_ptr<JitModule>> built(todo.size());
    std::vector<std::thread> th;
    const int dev = ctx->device;
    for (size_t k = 0; k < todo.size(); ++k) {
        built[k] = std::make_shared<JitModule>();
        th.emplace_back([&, k, dev] {
            cudaSetDevice(dev);
            st[k] = compile_module(*mods[todo[k]].src, (int)mods[todo[k]].pass_index.size(), dev, *built[k], errs[k],
                                   mods[todo[k]].prefix);
        });
    }
    for (auto &t : th) t.join();
    for (size_t k = 0; k < todo.size(); ++k)
        if (st[k]) return fail(st[k], "pass compiler: %s", errs[k].c_str());
    std::lock_guard<std::mutex> lk(cache().mu);
    for (size_t k = 0; k < todo.size(); ++k) {
        cache().mods[*mods[todo[k]].src] = built[k];
        handles[todo[k]] = built[k];
    }
    return QF_OK;
}

int upload_consts(qf_ctx *ctx, JitModule &jm, const ModulePlan &mp) {
    const size_t bytes = mp.consts.size() * sizeof(float);
    if (bytes > jm.consts_bytes) return fail(QF_ERR_CUDA, "pass compiler: constant bank size mismatch");
    if (bytes) QF_CUDA(cudaMemcpyAsync(jm.consts, mp.consts.data(), bytes, cudaMemcpyHostToDevice, ctx->stream));
    return QF_OK;
}

int grid_of(qf_ctx *ctx, cudaKernel_t k, int K, uint64_t n_tiles, uint64_t *grid) {
    int per_sm = 0;
    QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)k, threads_of(K), dyn_smem_of(K)));
    per_sm = std::min(std::max(per_sm, 1), 4);
    *grid = std::min<uint64_t>((uint64_t)per_sm * ctx->sm_count, n_tiles);
    return QF_OK;
}
}  // namespace

// Generate, compile (or fetch) and launch the plan's passes.
int run_plan_jit(qf_sv *sv, const Plan &plan, int) {
    const int wb = (int)plan.passes[0].a.k - 9;
    // interpreted when the plan does not fit the compiled layout
    if (!jit_plan_fits(plan)) return plan.block_qubits ? run_plan_blocks(sv, plan) : run_plan_rs(sv, plan, wb);
    qf_ctx *ctx = sv->ctx;
    std::vector<ModulePlan> mods;
    if (!gen_modules(plan, mods)) return plan.block_qubits ? run_plan_blocks(sv, plan) : run_plan_rs(sv, plan, wb);
    std::vector<std::shared_ptr<JitModule>> handles;
    QF_TRY(fetch_modules(ctx, mods, handles));
    for (size_t m = 0; m < mods.size(); ++m) {
        JitModule &jm = *handles[m];
        QF_TRY(upload_consts(ctx, jm, mods[m]));
        for (size_t k = 0; k < mods[m].pass_index.size(); ++k) {
            const Pass &p = plan.passes[mods[m].pass_index[k]];
            uint64_t grid;
            const int K = pass_k(p);
            QF_TRY(grid_of(ctx, jm.kernels[k], K, p.a.n_tiles, &grid));
            float2 *amps = static_cast<float2 *>(sv->d);
            unsigned long long nt = p.a.n_tiles;
            void *args[] = {&amps, &nt};
            QF_CUDA(cudaLaunchKernel((const void *)jm.kernels[k], dim3((unsigned)grid), dim3(threads_of(K)), args, dyn_smem_of(K),
                                     ctx->stream));
        }
    }
    return QF_OK;
}

// Backward adjoint passes: psi and lambda in registers, the overlap slots
// reduced per CTA into partials[slot * stride + block] and then summed in
// block order into d_slot_sums.
int run_plan_jit_dual(qf_sv *psi, qf_sv *lam, const Plan &plan, double *d_slot_sums) {
    if (!jit_plan_fits(plan, true)) return run_plan_dual_smem(psi, lam, plan, d_slot_sums);
    qf_ctx *ctx = psi->ctx;
    std::vector<ModulePlan> mods;
    if (!gen_modules(plan, mods, true)) return run_plan_dual_smem(psi, lam, plan, d_slot_sums);
    std::vector<std::shared_ptr<JitModule>> handles;
    QF_TRY(fetch_modules(ctx, mods, handles));
    const uint32_t stride = 4u * (uint32_t)std::max(1, ctx->sm_count);
    double *d_partials = nullptr;
    if (plan.n_slots) {
        const size_t bytes = sizeof(double) * (size_t)plan.n_slots * stride;
        QF_TRY(ensure_device(&ctx->ws_red, &ctx->ws_red_bytes, bytes));
        d_partials = static_cast<double *>(ctx->ws_red);
        QF_CUDA(cudaMemsetAsync(d_partials, 0, bytes, ctx->stream));
    }
    for (size_t m = 0; m < mods.size(); ++m) {
        JitModule &jm = *handles[m];
        QF_TRY(upload_consts(ctx, jm, mods[m]));
        for (size_t k = 0; k < mods[m].pass_index.size(); ++k) {
            const Pass &p = plan.passes[mods[m].pass_index[k]];
            uint64_t grid;
            const int K = pass_k(p);
            QF_TRY(grid_of(ctx, jm.kernels[k], K, p.a.n_tiles, &grid));
            float2 *a = static_cast<float2 *>(psi->d), *b = static_cast<float2 *>(lam->d);
            unsigned long long nt = p.a.n_tiles;
            double *parts = d_partials;
            unsigned str = stride;
            void *args[] = {&a, &b, &nt, &parts, &str};
            QF_CUDA(cudaLaunchKernel((const void *)jm.kernels[k], dim3((unsigned)grid), dim3(threads_of(K)), args, dyn_smem_of(K),
                                     ctx->stream));
        }
    }
    if (plan.n_slots && d_slot_sums) QF_TRY(reduce_slots(ctx, d_partials, stride, plan.n_slots, d_slot_sums));
    return QF_OK;
}


// ---- compiled Pauli-sum passes ----------------------------------------------
// A Pauli pass (terms grouped by x-mask, every x-bit of its groups resident in
// a 12-bit tile whose low five bits are qubits 0..4) as one generated kernel.
// Thread t holds the 16 amplitudes j = lane | i << 5 | warp << 9 (i < 16);
// the tile arrives by 16-byte cp.async one tile ahead. For a group of x-mask
// x, the partner of j is j ^ x: in the thread's own registers when x has only
// register bits, otherwise read from shared memory. The phase of term t at the
// source index splits into a per-thread bit (lane and warp bits of its z-mask,
// computed once per kernel), a per-tile bit (its z-mask off the tile), a
// compile-time bit (the x-mask's lane and warp bits) and the register bits:
// terms with the same register part of z add into one class sum per tile, and
// G_i = sum over classes of (-1)^parity((i ^ x_reg) & class) * sum (a
// Walsh-Hadamard transform when the classes are many). Coefficients live in the
// constant bank, so a Hamiltonian with new coefficients reuses its kernels.
namespace {

struct PauliPassDesc {
    const PPassArgs *a;
    const std::vector<PGroup> *groups;
    const std::vector<PTerm> *terms;
};

bool pauli_pass_fits(const PPassArgs &a) { return a.k == 12 && a.low >= 5 && a.n_terms > 0; }

void gen_pauli_kernel(std::ostringstream &s, const PauliPassDesc &d, int index, int coef_base) {
    const PPassArgs &a = *d.a;
    const uint32_t mode = a.mode;
    uint32_t qb[12];
    for (uint32_t b = 0; b < 12; ++b) qb[b] = b < a.low ? b : a.hi_q[b - a.low];
    auto bitq = [&](uint32_t b) { return hex64(1ULL << qb[b]); };
    s << "extern \"C\" __global__ void __launch_bounds__(256, 2) h" << index
      << "(const float2* __restrict__ P, float2* __restrict__ L, unsigned long long nt, double* __restrict__ partials) {\n";
    s << "extern __shared__ __align__(16) float2 SB[];\n";
    s << "__shared__ double red[32];\n";
    s << "const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, tid = threadIdx.x;\n";
    s << "const unsigned sbase = (unsigned)__cvta_generic_to_shared(SB);\n";
    s << "const unsigned jb = lane | (warp << 9);\n";
    s << "const unsigned long long ow = ((warp & 1u) ? " << bitq(9) << " : 0ull) | ((warp & 2u) ? " << bitq(10)
      << " : 0ull) | ((warp & 4u) ? " << bitq(11) << " : 0ull);\n";
    // cp.async chunk c = tid + 256 k holds tile indices 2c, 2c + 1
    s << "const unsigned long long toff = (unsigned long long)((2u * tid) & 31u)";
    for (int b = 0; b < 4; ++b) s << " | ((tid & " << (16u << b) << "u) ? " << bitq(5 + b) << " : 0ull)";
    s << ";\n";
    const std::string dep_t = deposit_code(a.nonlocal_mask, "t"), dep_t2 = deposit_code(a.nonlocal_mask, "t2");
    auto issue = [&](const std::string &tq, const std::string &buf) {
        for (int k = 0; k < 8; ++k) {
            uint64_t ck = 0;
            for (int b = 0; b < 3; ++b)
                if ((k >> b) & 1) ck |= 1ULL << qb[9 + b];
            s << "qf_cpa16(sbase + ((" << buf << ") * 4096u + 2u * tid + " << 512 * k << "u) * 8u, P + (" << tq
              << " | toff | " << hex64(ck) << "));\n";
        }
    };
    // per-thread parity bits of every term (lane and warp bits of its z-mask)
    const auto &T = *d.terms;
    const size_t nt_ = T.size();
    const int n_words = (int)((nt_ + 63) / 64);
    for (int w = 0; w < n_words; ++w) {
        s << "unsigned long long tpar" << w << " = 0ull";
        for (size_t t = 64 * (size_t)w; t < std::min(nt_, 64 * (size_t)w + 64); ++t) {
            const uint32_t zl = T[t].zl & 31u, zw = (T[t].zl >> 9) & 7u;
            if (zl || zw)
                s << " | ((unsigned long long)((__popc(lane & " << zl << "u) + __popc(warp & " << zw << "u)) & 1u) << "
                  << (t - 64 * w) << ")";
        }
        s << ";\n";
    }
    s << "double acc_re = 0.0, acc_im = 0.0;\n";
    s << "unsigned long long t = blockIdx.x;\n";
    s << "if (t < nt) {const unsigned long long tq = " << dep_t << ";\n";
    issue("tq", "0u");
    s << "}\nasm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n";
    s << "for (unsigned it = 0; t < nt; t += gridDim.x, ++it) {\n";
    s << "const unsigned cur = it & 1u;\n";
    s << "{const unsigned long long t2 = t + gridDim.x; if (t2 < nt) {const unsigned long long tq = " << dep_t2 << ";\n";
    issue("tq", "cur ^ 1u");
    s << "}}\nasm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n";
    s << "asm volatile(\"cp.async.wait_group 1;\\n\" ::: \"memory\");\n__syncthreads();\n";
    s << "const float2* S = SB + cur * 4096u;\n";
    s << "const unsigned long long base = " << dep_t << ";\n";
    if (mode != 0) s << "const unsigned long long gb = base | lane | ow;\n";
    for (int i = 0; i < 16; ++i) s << "const float2 r" << i << " = S[jb | " << (i << 5) << "u];\n";
    if (mode != 0)
        for (int i = 0; i < 16; ++i) s << "float2 l" << i << " = make_float2(0.f, 0.f);\n";
    else
        s << "float e_re = 0.f, e_im = 0.f;\n";
    int k = coef_base;
    for (const PGroup &G : *d.groups) {
        const uint32_t x = G.xl;
        const uint32_t xsrc = mode == 0 ? 0u : x;
        const uint32_t xr = (xsrc >> 5) & 15u;
        const bool real = G.real != 0;
        // class sums
        std::map<uint32_t, int> cls;
        for (uint32_t q = 0; q < G.t_count; ++q) cls.emplace((T[G.t_begin + q].zl >> 5) & 15u, (int)cls.size());
        s << "{\n";
        for (auto &c : cls) s << "float sr" << c.second << " = 0.f" << (real ? "" : std::string(", si") + std::to_string(c.second) + " = 0.f") << ";\n";
        for (uint32_t q = 0; q < G.t_count; ++q, ++k) {
            const PTerm &P = T[G.t_begin + q];
            const size_t ti = G.t_begin + q;
            const uint32_t zl = P.zl & 31u, zw = (P.zl >> 9) & 7u;
            const uint32_t cflip = (uint32_t)((__builtin_popcount((xsrc & 31u) & zl) + __builtin_popcount(((xsrc >> 9) & 7u) & zw)) & 1);
            std::ostringstream bit;
            bit << "(unsigned)((tpar" << ti / 64 << " >> " << ti % 64 << ") & 1ull)";
            if (P.zo) bit << " ^ (unsigned)(__popcll(base & " << hex64(P.zo) << ") & 1)";
            if (cflip) bit << " ^ 1u";
            const int c = cls[(P.zl >> 5) & 15u];
            s << "{const unsigned b = " << bit.str() << "; const float2 c = M[" << k << "]; sr" << c << " += b ? -c.x : c.x;";
            if (!real) s << " si" << c << " += b ? -c.y : c.y;";
            s << "}\n";
        }
        // G_i for every register index, then the multiply-add with the partner
        const bool fwht = cls.size() > 4;
        if (fwht) {  // W[c] for all 16 classes, then the butterflies: H[i] = sum_c (-1)^popc(i & c) W[c]
            for (int c = 0; c < 16; ++c) {
                auto it = cls.find((uint32_t)c);
                s << "float wr" << c << " = " << (it == cls.end() ? std::string("0.f") : "sr" + std::to_string(it->second)) << ";";
                if (!real) s << "float wi" << c << " = " << (it == cls.end() ? std::string("0.f") : "si" + std::to_string(it->second)) << ";";
            }
            s << "\n";
            for (int h = 1; h < 16; h <<= 1)
                for (int c = 0; c < 16; ++c)
                    if (!(c & h)) {
                        s << "{const float u = wr" << c << ", v = wr" << (c | h) << "; wr" << c << " = u + v; wr" << (c | h) << " = u - v;}";
                        if (!real)
                            s << "{const float u = wi" << c << ", v = wi" << (c | h) << "; wi" << c << " = u + v; wi" << (c | h) << " = u - v;}";
                    }
            s << "\n";
        }
        const bool in_regs = (x & 31u) == 0 && ((x >> 9) & 7u) == 0;
        for (int i = 0; i < 16; ++i) {
            const uint32_t isrc = (uint32_t)i ^ xr;
            std::ostringstream gr, gi;
            if (fwht) {
                gr << "wr" << isrc;
                gi << "wi" << isrc;
            } else {
                bool first = true;
                for (auto &c : cls) {
                    const bool neg = __builtin_popcount(isrc & c.first) & 1;
                    gr << (first ? (neg ? "-" : "") : (neg ? "-" : "+")) << "sr" << c.second;
                    gi << (first ? (neg ? "-" : "") : (neg ? "-" : "+")) << "si" << c.second;
                    first = false;
                }
            }
            std::string part;
            if (in_regs) part = "r" + std::to_string(i ^ (int)((x >> 5) & 15u));
            else part = "S[(jb | " + std::to_string(i << 5) + "u) ^ " + std::to_string(x) + "u]";
            s << "{const float g_r = " << gr.str() << ";";
            if (!real) s << "const float g_i = " << gi.str() << ";";
            s << "const float2 p = " << part << ";";
            if (mode != 0) {
                const std::string l = "l" + std::to_string(i);
                if (real) s << l << ".x = fmaf(g_r, p.x, " << l << ".x); " << l << ".y = fmaf(g_r, p.y, " << l << ".y);";
                else
                    s << l << ".x = fmaf(g_r, p.x, fmaf(-g_i, p.y, " << l << ".x)); " << l << ".y = fmaf(g_r, p.y, fmaf(g_i, p.x, "
                      << l << ".y));";
            } else {  // conj(psi_{j^x}) * G(j) * psi_j
                const std::string r = "r" + std::to_string(i);
                if (real) s << "const float tr = g_r * " << r << ".x, ti = g_r * " << r << ".y;";
                else s << "const float tr = g_r * " << r << ".x - g_i * " << r << ".y, ti = g_r * " << r << ".y + g_i * " << r << ".x;";
                s << "e_re = fmaf(p.x, tr, fmaf(p.y, ti, e_re)); e_im = fmaf(p.x, ti, fmaf(-p.y, tr, e_im));";
            }
            s << "}\n";
        }
        s << "}\n";
    }
    if (mode != 0) {
        s << "float e_re = 0.f, e_im = 0.f;\n";
        for (int i = 0; i < 16; ++i) {
            uint64_t off = 0;
            for (int b = 0; b < 4; ++b)
                if ((i >> b) & 1) off |= 1ULL << qb[5 + b];
            const std::string l = "l" + std::to_string(i), r = "r" + std::to_string(i);
            s << "{float2* q = L + (gb | " << hex64(off) << ");";
            if (mode == 2) s << "const float2 o = *q; " << l << ".x += o.x; " << l << ".y += o.y;";
            s << "*q = " << l << ";";
            if (a.last) s << "e_re = fmaf(" << r << ".x, " << l << ".x, fmaf(" << r << ".y, " << l << ".y, e_re)); e_im = fmaf(" << r
                          << ".x, " << l << ".y, fmaf(-" << r << ".y, " << l << ".x, e_im));";
            s << "}\n";
        }
    }
    s << "acc_re += (double)e_re; acc_im += (double)e_im;\n";
    s << "__syncthreads();\n}\n";  // tile loop
    s << "asm volatile(\"cp.async.wait_group 0;\\n\" ::: \"memory\");\n";
    s << "for (int o = 16; o > 0; o >>= 1) {acc_re += __shfl_xor_sync(0xffffffffu, acc_re, o); acc_im += __shfl_xor_sync(0xffffffffu, acc_im, o);}\n";
    s << "if (lane == 0) {red[warp] = acc_re; red[8 + warp] = acc_im;}\n__syncthreads();\n";
    s << "if (tid == 0) {double a = 0.0, b = 0.0; for (int w = 0; w < 8; ++w) {a += red[w]; b += red[8 + w];} partials[2 * blockIdx.x] = a; "
         "partials[2 * blockIdx.x + 1] = b;}\n";
    s << "}\n";
}

struct PauliModule {
    std::shared_ptr<JitModule> mod;
    std::vector<float> consts;
};

}  // namespace

int run_pauli_jit(qf_sv *psi, qf_sv *lam, const std::vector<const PPassArgs *> &args,
                  const std::vector<const std::vector<PGroup> *> &groups, const std::vector<const std::vector<PTerm> *> &terms,
                  double *partials, uint32_t slice_stride, uint32_t max_grid, bool *ran) {
    *ran = false;
    if (psi->dtype != QF_C64 || !jit_available() || args.empty()) return QF_OK;
    for (const PPassArgs *a : args)
        if (!pauli_pass_fits(*a)) return QF_OK;
    qf_ctx *ctx = psi->ctx;
    // source text (structure only) and constants (the coefficients)
    ModulePlan mp;
    mp.prefix = 'h';
    std::ostringstream body;
    std::vector<float> consts;
    for (size_t p = 0; p < args.size(); ++p) {
        PauliPassDesc d{args[p], groups[p], terms[p]};
        gen_pauli_kernel(body, d, (int)p, (int)(consts.size() / 2));
        for (const PGroup &G : *groups[p])
            for (uint32_t q = 0; q < G.t_count; ++q) {
                consts.push_back((float)(*terms[p])[G.t_begin + q].cre);
                consts.push_back((float)(*terms[p])[G.t_begin + q].cim);
            }
        mp.pass_index.push_back((int)p);
    }
    if (consts.size() * 4 > 60 * 1024) return QF_OK;  // the constant bank holds at most ~7500 terms
    std::ostringstream head;
    head << "__constant__ float2 M[" << std::max<size_t>(1, consts.size() / 2) << "];\n" << kPrelude;
    mp.src = std::make_shared<const std::string>(head.str() + body.str());
    mp.consts = consts;
    std::vector<ModulePlan> mods{mp};
    std::vector<std::shared_ptr<JitModule>> handles;
    QF_TRY(fetch_modules(ctx, mods, handles));
    JitModule &jm = *handles[0];
    QF_TRY(upload_consts(ctx, jm, mods[0]));
    for (size_t p = 0; p < args.size(); ++p) {
        const PPassArgs &a = *args[p];
        int per_sm = 0;
        QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)jm.kernels[p], 256, dyn_smem_of(12)));
        const uint64_t grid = std::min<uint64_t>(std::min<uint64_t>((uint64_t)std::max(per_sm, 1) * ctx->sm_count, max_grid),
                                                 a.n_tiles);
        const float2 *P = static_cast<const float2 *>(psi->d);
        float2 *Lp = lam ? static_cast<float2 *>(lam->d) : nullptr;
        unsigned long long nt = a.n_tiles;
        double *parts = partials + (size_t)slice_stride * p;
        void *kargs[] = {&P, &Lp, &nt, &parts};
        QF_CUDA(cudaLaunchKernel((const void *)jm.kernels[p], dim3((unsigned)grid), dim3(256), kargs, dyn_smem_of(12), ctx->stream));
    }
    *ran = true;
    return QF_OK;
}

}  // namespace qf
