// jit.cpp — pass compiler for complex64 register-tiled sweeps.
//
// A register-tiled plan (lower_rs) is turned into CUDA C with one kernel per
// pass: register positions, lane bits, layouts, remaps and the tile-address
// deposit are compile-time constants; CNOTs and SWAPs whose qubits are all in
// register positions become renames of the register variables and emit no
// code; matrix entries are read from __constant__ memory, so a structurally
// identical circuit with new angles reuses the compiled kernels. Diagonal
// gates are applied as diag(1, m11/m00) and the product of the m00 factors is
// applied once at the end of the plan (a global phase).
//
// Kernels are compiled with NVRTC (loaded with dlopen) for sm_103a, loaded
// with cudaLibraryLoadData and cached per context by source text.
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <complex>
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
constexpr int kR = 16;

struct Gen {
    std::ostringstream s;
    int v[kR];  // logical register -> variable number
    std::vector<std::complex<double>> consts;  // 4 complex per matrix slot (float2 M[...])
    std::complex<double> gphase{1.0, 0.0};
    bool any_diag = false;
    int wb = 3;
    bool prefetch = true;  // double-buffered cp.async tile loads

    std::string R(int i) const { return "r" + std::to_string(v[i]); }
    int slot(const std::complex<double> a, const std::complex<double> b, const std::complex<double> c,
             const std::complex<double> d) {
        consts.push_back(a);
        consts.push_back(b);
        consts.push_back(c);
        consts.push_back(d);
        return (int)consts.size() / 4 - 1;
    }
    // thread-constant bit expression of a descriptor (lane/warp/outside)
    static std::string cbit(uint8_t d) {
        if (d < 8) return "((lane >> " + std::to_string(d) + ") & 1u)";
        if (d >= 16 && d < 64) return "((warp >> " + std::to_string(d - 16) + ") & 1u)";
        return "((unsigned)(tb >> " + std::to_string(d - 64) + ") & 1u)";
    }
    static bool is_reg(uint8_t d) { return d >= 8 && d < 16; }
};

std::complex<double> cx(const double *m, int k) { return {m[2 * k], m[2 * k + 1]}; }

std::string Mref(int slot, int e) { return "M[" + std::to_string(4 * slot + e) + "]"; }

// deposit of the tile index t onto the outside qubits, as runs of shifts
std::string deposit_code(uint64_t mask) {
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
        o << " | (((t >> " << consumed << ") & 0x" << std::hex << ((len >= 64) ? ~0ULL : ((1ULL << len) - 1)) << std::dec
          << "ull) << " << q << ")";
        consumed += len;
        q = e;
    }
    return o.str();
}

std::string layout_offset(const uint8_t *qs, int i) {
    uint64_t off = 0;
    for (int b = 0; b < 4; ++b)
        if ((i >> b) & 1) off |= 1ULL << qs[b];
    std::ostringstream o;
    o << "0x" << std::hex << off << "ull";
    return o.str();
}

void emit_mat2(Gen &g, int slot, int mk, const std::string &A, const std::string &B) {
    const std::string m00 = Mref(slot, 0), m01 = Mref(slot, 1), m10 = Mref(slot, 2), m11 = Mref(slot, 3);
    auto &s = g.s;
    s << "{const float2 x=" << A << ",y=" << B << ";";
    if (mk == 1) {
        s << A << ".x=" << m00 << ".x*x.x+" << m01 << ".x*y.x;" << A << ".y=" << m00 << ".x*x.y+" << m01 << ".x*y.y;";
        s << B << ".x=" << m10 << ".x*x.x+" << m11 << ".x*y.x;" << B << ".y=" << m10 << ".x*x.y+" << m11 << ".x*y.y;";
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

void emit_cmul_const(Gen &g, const std::string &R, int slot, int e) {
    const std::string f = Mref(slot, e);
    g.s << "{const float2 x=" << R << ";" << R << ".x=" << f << ".x*x.x-" << f << ".y*x.y;" << R << ".y=" << f
        << ".x*x.y+" << f << ".y*x.x;}\n";
}

uint8_t matrix_kind_of(const std::complex<double> m[4]) {
    bool real = true;
    for (int k = 0; k < 4; ++k) real = real && m[k].imag() == 0.0;
    if (real) return 1;
    if (m[0].imag() == 0 && m[3].imag() == 0 && m[1].real() == 0 && m[2].real() == 0) return 2;
    return 0;
}

// one pass -> kernel body
void gen_pass(Gen &g, const RsPlan &rp, const RsPass &p, int index) {
    auto &s = g.s;
    const int wb = rp.wb;
    for (int i = 0; i < kR; ++i) g.v[i] = i;
    bool has_remap = false;
    for (uint32_t o = 0; o < p.a.n_ops; ++o) has_remap |= rp.ops[p.op_begin + o].kind == RS_REMAP;
    const int nt_threads = 32 << wb, tile = kR * nt_threads;
    s << "extern \"C\" __global__ void __launch_bounds__(" << nt_threads << ", " << (wb == 3 ? 2 : 1) << ") p" << index
      << "(float2* __restrict__ A, unsigned long long nt) {\n";
    s << "const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;\n";
    auto warp_off = [&](const uint8_t *qs) {
        std::ostringstream o;
        o << "0ull";
        for (int w = 0; w < wb; ++w) o << " | ((warp & " << (1 << w) << "u) ? (1ull << " << (int)qs[4 + w] << ") : 0ull)";
        return o.str();
    };
    s << "const unsigned long long lw = " << warp_off(p.a.load_q) << ", sw = " << warp_off(p.a.store_q) << ";\n";
    const std::string dep = deposit_code(p.a.nonlocal_mask);
    if (g.prefetch) {
        // Double-buffered asynchronous tile loads: tile t+1 streams into shared
        // memory (16-byte cp.async) while tile t is computed. Shared index j of
        // a tile: bits 0..4 = qubits 0..4, bits 5..8 = register positions,
        // bits 9.. = warp positions (load layout). Thread tid copies chunks
        // tid + nthreads*k (two amplitudes each).
        s << "extern __shared__ __align__(16) float2 SB[];\n";
        s << "const unsigned tid = threadIdx.x, sbase = (unsigned)__cvta_generic_to_shared(SB);\n";
        s << "const unsigned long long toff = (unsigned long long)((2u * tid) & 31u)";
        for (int b = 0; b < 4; ++b) s << " | ((tid & " << (16u << b) << "u) ? (1ull << " << (int)p.a.load_q[b] << ") : 0ull)";
        s << ";\n";
        const int chunks = tile / 2 / nt_threads;  // per thread
        auto issue = [&](const std::string &tq, const std::string &buf) {
            for (int k = 0; k < chunks; ++k) {
                uint64_t kk = 0;  // warp-position bits of chunk k (j >> 9 == k)
                for (int w = 0; w < wb; ++w)
                    if ((k >> w) & 1) kk |= 1ULL << p.a.load_q[4 + w];
                s << "qf_cpa16(sbase + ((" << buf << ") * " << tile << "u + 2u * (tid + " << nt_threads * k << "u)) * 8u, A + (" << tq
                  << " | toff | 0x" << std::hex << kk << std::dec << "ull));\n";
            }
        };
        s << "unsigned long long t = blockIdx.x;\n";
        s << "if (t < nt) {const unsigned long long tq = " << dep << ";\n";
        issue("tq", "0u");
        s << "}\nasm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n";
        s << "for (unsigned it = 0; t < nt; t += gridDim.x, ++it) {\n";
        s << "const unsigned cur = it & 1u;\n";
        // prefetch the CTA's next tile (the deposit expression reads `t`; substitute t2)
        s << "{const unsigned long long t2 = t + gridDim.x; if (t2 < nt) {const unsigned long long tq = ";
        {
            std::string d2 = dep;
            for (size_t pos = 0; (pos = d2.find("(t >>", pos)) != std::string::npos; pos += 6) d2.replace(pos, 5, "(t2 >>");
            s << d2 << ";\n";
        }
        issue("tq", "cur ^ 1u");
        s << "}}\nasm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\");\n";
        s << "asm volatile(\"cp.async.wait_group 1;\\n\" ::: \"memory\");\n__syncthreads();\n";
        s << "float2* S = SB + cur * " << tile << "u;\n";
        s << "const unsigned long long tb = " << dep << ";\n";
        for (int i = 0; i < kR; ++i) s << "float2 r" << i << " = S[lane | " << (i << 5) << "u | (warp << 9)];\n";
        s << "__syncthreads();\n";
    } else {
        if (has_remap) s << "__shared__ float2 S[" << tile << "];\n";
        s << "for (unsigned long long t = blockIdx.x; t < nt; t += gridDim.x) {\n";
        s << "const unsigned long long tb = " << dep << ";\n";
        s << "const unsigned long long b0 = tb | lane | lw;\n";
        for (int i = 0; i < kR; ++i) s << "float2 r" << i << " = A[b0 | " << layout_offset(p.a.load_q, i) << "];\n";
    }
    const double *mats = rp.mats.data() + 8 * (size_t)p.mat_begin;
    for (uint32_t o = 0; o < p.a.n_ops; ++o) {
        const RsOp &op = rp.ops[p.op_begin + o];
        std::complex<double> m[4];
        if (op.kind == RS_MREG || op.kind == RS_MLANE || op.kind == RS_DIAG)
            for (int k = 0; k < 4; ++k) m[k] = cx(mats + 8 * (size_t)op.mat, k);
        switch (op.kind) {
        case RS_MREG: {
            const int mk = matrix_kind_of(m);
            const int sl = g.slot(m[0], m[1], m[2], m[3]);
            for (int i = 0; i < kR; ++i)
                if (!(i & (1 << op.p0))) emit_mat2(g, sl, mk, g.R(i), g.R(i | (1 << op.p0)));
            break;
        }
        case RS_MLANE: {
            const int mk = matrix_kind_of(m);
            const int sl = g.slot(m[0], m[1], m[2], m[3]);
            const int b = op.p0;
            s << "{const unsigned hb = (lane >> " << b << ") & 1u; const float2 cs = hb ? " << Mref(sl, 3) << " : "
              << Mref(sl, 0) << ", co = hb ? " << Mref(sl, 2) << " : " << Mref(sl, 1) << ";\n";
            for (int i = 0; i < kR; ++i) {
                const std::string Ri = g.R(i);
                s << "{float2 q; q.x = __shfl_xor_sync(0xffffffffu, " << Ri << ".x, " << (1 << b) << "); q.y = __shfl_xor_sync(0xffffffffu, "
                  << Ri << ".y, " << (1 << b) << "); const float2 x=" << Ri << ";";
                if (mk == 1)
                    s << Ri << ".x=cs.x*x.x+co.x*q.x;" << Ri << ".y=cs.x*x.y+co.x*q.y;}\n";
                else
                    s << Ri << ".x=cs.x*x.x-cs.y*x.y+co.x*q.x-co.y*q.y;" << Ri << ".y=cs.x*x.y+cs.y*x.x+co.x*q.y+co.y*q.x;}\n";
            }
            s << "}\n";
            break;
        }
        case RS_DIAG: {
            // diag(m00, m11) = m00 * diag(1, m11/m00)
            g.any_diag = true;
            g.gphase *= m[0];
            const std::complex<double> f = m[3] / m[0];
            const int sl = g.slot(f, 0.0, 0.0, f);
            if (Gen::is_reg(op.p0)) {
                const int rb = op.p0 - 8;
                for (int i = 0; i < kR; ++i)
                    if ((i >> rb) & 1) emit_cmul_const(g, g.R(i), sl, 0);
            } else {
                s << "if (" << Gen::cbit(op.p0) << ") {\n";
                for (int i = 0; i < kR; ++i) emit_cmul_const(g, g.R(i), sl, 0);
                s << "}\n";
            }
            break;
        }
        case RS_CNOT: {
            const bool creg = Gen::is_reg(op.p0);
            if (Gen::is_reg(op.p1)) {
                const int tb = op.p1 - 8;
                if (creg) {  // rename only
                    const int cb = op.p0 - 8;
                    for (int i = 0; i < kR; ++i)
                        if (((i >> cb) & 1) && !((i >> tb) & 1)) std::swap(g.v[i], g.v[i | (1 << tb)]);
                } else {
                    s << "if (" << Gen::cbit(op.p0) << ") {\n";
                    for (int i = 0; i < kR; ++i)
                        if (!((i >> tb) & 1)) {
                            const std::string A = g.R(i), B = g.R(i | (1 << tb));
                            s << "{const float2 x=" << A << "; " << A << "=" << B << "; " << B << "=x;}\n";
                        }
                    s << "}\n";
                }
            } else {  // lane target
                const int b = op.p1;
                if (!creg) s << "{const unsigned cc = " << Gen::cbit(op.p0) << ";\n";
                for (int i = 0; i < kR; ++i) {
                    if (creg && !((i >> (op.p0 - 8)) & 1)) continue;
                    const std::string Ri = g.R(i);
                    s << "{float2 q; q.x = __shfl_xor_sync(0xffffffffu, " << Ri << ".x, " << (1 << b)
                      << "); q.y = __shfl_xor_sync(0xffffffffu, " << Ri << ".y, " << (1 << b) << ");";
                    if (creg) s << Ri << " = q;}\n";
                    else s << "if (cc) " << Ri << " = q;}\n";
                }
                if (!creg) s << "}\n";
            }
            break;
        }
        case RS_CZ: {
            const bool ra = Gen::is_reg(op.p0), rb = Gen::is_reg(op.p1);
            if (ra && rb) {
                const int a = op.p0 - 8, b = op.p1 - 8;
                for (int i = 0; i < kR; ++i)
                    if (((i >> a) & 1) && ((i >> b) & 1)) s << g.R(i) << ".x = -" << g.R(i) << ".x; " << g.R(i) << ".y = -" << g.R(i) << ".y;\n";
            } else if (ra || rb) {
                const int a = (ra ? op.p0 : op.p1) - 8;
                const uint8_t other = ra ? op.p1 : op.p0;
                s << "if (" << Gen::cbit(other) << ") {\n";
                for (int i = 0; i < kR; ++i)
                    if ((i >> a) & 1) s << g.R(i) << ".x = -" << g.R(i) << ".x; " << g.R(i) << ".y = -" << g.R(i) << ".y;\n";
                s << "}\n";
            } else {
                s << "if (" << Gen::cbit(op.p0) << " & " << Gen::cbit(op.p1) << ") {\n";
                for (int i = 0; i < kR; ++i) s << g.R(i) << ".x = -" << g.R(i) << ".x; " << g.R(i) << ".y = -" << g.R(i) << ".y;\n";
                s << "}\n";
            }
            break;
        }
        case RS_SWAP_LR: {
            const int a = op.p0, rb = op.p1;
            s << "{const unsigned la = (lane >> " << a << ") & 1u;\n";
            for (int i = 0; i < kR; ++i)
                if (!((i >> rb) & 1)) {
                    const std::string Ri = g.R(i), Rj = g.R(i | (1 << rb));
                    s << "{const float2 snd = la ? " << Ri << " : " << Rj << "; float2 q; q.x = __shfl_xor_sync(0xffffffffu, snd.x, "
                      << (1 << a) << "); q.y = __shfl_xor_sync(0xffffffffu, snd.y, " << (1 << a) << "); if (la) " << Ri
                      << " = q; else " << Rj << " = q;}\n";
                }
            s << "}\n";
            break;
        }
        case RS_SWAP_LL: {
            const int a = op.p0, b = op.p1;
            s << "{const unsigned ba = (lane >> " << a << ") & 1u, bb = (lane >> " << b << ") & 1u; const unsigned src = (lane & ~"
              << ((1u << a) | (1u << b)) << "u) | (ba << " << b << ") | (bb << " << a << ");\n";
            for (int i = 0; i < kR; ++i)
                s << g.R(i) << ".x = __shfl_sync(0xffffffffu, " << g.R(i) << ".x, src); " << g.R(i)
                  << ".y = __shfl_sync(0xffffffffu, " << g.R(i) << ".y, src);\n";
            s << "}\n";
            break;
        }
        default: {  // RS_REMAP
            auto slots = [&](uint32_t packed, int pos) { return (packed >> (3 * pos)) & 7u; };
            auto idx = [&](uint32_t packed, int i) {
                std::ostringstream o;
                uint32_t regbits = 0;
                for (int b = 0; b < 4; ++b)
                    if ((i >> b) & 1) regbits |= 1u << slots(packed, b);
                o << "lane + 32u * (" << regbits << "u";
                for (int w = 0; w < wb; ++w) o << " | ((warp & " << (1 << w) << "u) ? " << (1u << slots(packed, 4 + w)) << "u : 0u)";
                o << ")";
                return o.str();
            };
            for (int i = 0; i < kR; ++i) s << "S[" << idx(op.a, i) << "] = " << g.R(i) << ";\n";
            s << "__syncthreads();\n";
            for (int i = 0; i < kR; ++i) s << g.R(i) << " = S[" << idx(op.b, i) << "];\n";
            s << "__syncthreads();\n";
            break;
        }
        }
    }
    (void)index;
}

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

int compile_module(const std::string &src, int n_kernels, size_t dyn_smem, int device, JitModule &out, std::string &err) {
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
    const char *opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device", "-lineinfo"};
    nvrtcResult r = nv.compile(prog, 4, opts);
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
        const std::string nm = "p" + std::to_string(k);
        if ((e = cudaLibraryGetKernel(&out.kernels[k], out.lib, nm.c_str())) != cudaSuccess) {
            err = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(e);
            return QF_ERR_CUDA;
        }
    }
    if ((e = cudaLibraryGetGlobal(&out.consts, &out.consts_bytes, out.lib, "M")) != cudaSuccess) {
        err = std::string("cudaLibraryGetGlobal: ") + cudaGetErrorString(e);
        return QF_ERR_CUDA;
    }
    if (dyn_smem > 48 * 1024)
        for (int k = 0; k < n_kernels; ++k)
            if ((e = cudaKernelSetAttributeForDevice(out.kernels[k], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)dyn_smem, device)) != cudaSuccess) {
                err = std::string("cudaKernelSetAttributeForDevice: ") + cudaGetErrorString(e);
                return QF_ERR_CUDA;
            }
    return QF_OK;
}

struct ModulePlan {
    std::string src;
    std::vector<float> consts;  // interleaved float2
    std::vector<int> pass_index;
    size_t dyn_smem = 0;        // dynamic shared memory per CTA (prefetch buffers)
};

}  // namespace

bool jit_available() { return nvrtc().ok; }

// group passes into modules: at most 8 passes and 56 KB of constants each
static bool jit_prefetch_enabled() {
    const char *e = std::getenv("QF_JIT_PREFETCH");
    return !(e && e[0] == '0');
}

static void gen_modules(const RsPlan &rp, int wb, std::vector<ModulePlan> &mods) {
    Gen g;
    g.wb = wb;
    g.prefetch = jit_prefetch_enabled();
    const size_t npass = rp.passes.size();
    size_t pi = 0;
    while (pi < npass) {
        ModulePlan mp;
        std::ostringstream body;
        g.consts.clear();
        int local = 0;
        while (pi < npass && local < 8 && g.consts.size() * 8 < 56 * 1024) {
            g.s.str("");
            g.s.clear();
            gen_pass(g, rp, rp.passes[pi], local);
            if (pi + 1 == npass && g.any_diag) {  // the plan's global phase, once, at the very end
                const int sl = g.slot(g.gphase, 0.0, 0.0, 0.0);
                for (int i = 0; i < kR; ++i) emit_cmul_const(g, g.R(i), sl, 0);
            }
            // stores with the final register names
            for (int i = 0; i < kR; ++i)
                g.s << "A[(tb | lane | sw) | " << layout_offset(rp.passes[pi].a.store_q, i) << "] = " << g.R(i) << ";\n";
            g.s << "}\n}\n";
            body << g.s.str();
            mp.pass_index.push_back((int)pi);
            ++pi;
            ++local;
        }
        std::ostringstream head;
        head << "__constant__ float2 M[" << std::max<size_t>(1, g.consts.size()) << "];\n";
        head << "__device__ __forceinline__ void qf_cpa16(unsigned s, const float2* g) {"
                " asm volatile(\"cp.async.cg.shared.global [%0], [%1], 16;\\n\" :: \"r\"(s), \"l\"(g) : \"memory\"); }\n";
        mp.src = head.str() + body.str();
        mp.dyn_smem = g.prefetch ? 2u * kR * (32u << wb) * sizeof(float) * 2 : 0;
        mp.consts.reserve(g.consts.size() * 2);
        for (auto &c : g.consts) {
            mp.consts.push_back((float)c.real());
            mp.consts.push_back((float)c.imag());
        }
        mods.push_back(std::move(mp));
    }
}

// Generated sources and an NVRTC compile without loading (needs no GPU).
int jit_check_compile(const Plan &plan, int wb, std::string *source, std::string *err) {
    RsPlan rp;
    QF_TRY(lower_rs(plan, wb, rp));
    for (const RsPass &p : rp.passes)
        if (p.fallback) return fail(QF_ERR_UNSUPPORTED_OPERATION, "plan has a pass outside the register layout");
    std::vector<ModulePlan> mods;
    gen_modules(rp, wb, mods);
    Nvrtc &nv = nvrtc();
    if (!nv.ok) return fail(QF_ERR_UNSUPPORTED_OPERATION, "%s", nv.why.c_str());
    for (auto &m : mods) {
        if (source) *source += m.src;
        nvrtcProgram prog;
        nv.create(&prog, m.src.c_str(), "qf_pass.cu", 0, nullptr, nullptr);
        const char *opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device"};
        nvrtcResult r = nv.compile(prog, 3, opts);
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

// Generate, compile (or fetch) and launch the plan's passes.
int run_plan_jit(qf_sv *sv, const Plan &plan, int wb) {
    RsPlan rp;
    QF_TRY(lower_rs(plan, wb, rp));
    for (const RsPass &p : rp.passes)
        if (p.fallback) return run_plan_smem(sv, plan);
    qf_ctx *ctx = sv->ctx;
    std::vector<ModulePlan> mods;
    gen_modules(rp, wb, mods);
    // compile what is not cached (in parallel)
    std::vector<std::shared_ptr<JitModule>> handles(mods.size());
    std::vector<size_t> todo;
    {
        std::lock_guard<std::mutex> lk(cache().mu);
        for (size_t m = 0; m < mods.size(); ++m) {
            auto it = cache().mods.find(mods[m].src);
            if (it != cache().mods.end()) handles[m] = it->second;
            else todo.push_back(m);
        }
    }
    if (!todo.empty()) {
        std::vector<int> st(todo.size(), QF_OK);
        std::vector<std::string> errs(todo.size());
        std::vector<std::shared_ptr<JitModule>> built(todo.size());
        std::vector<std::thread> th;
        int dev = ctx->device;
        for (size_t k = 0; k < todo.size(); ++k) {
            built[k] = std::make_shared<JitModule>();
            th.emplace_back([&, k, dev] {
                cudaSetDevice(dev);
                st[k] = compile_module(mods[todo[k]].src, (int)mods[todo[k]].pass_index.size(), mods[todo[k]].dyn_smem, dev,
                                       *built[k], errs[k]);
            });
        }
        for (auto &t : th) t.join();
        for (size_t k = 0; k < todo.size(); ++k)
            if (st[k]) return fail(st[k], "pass compiler: %s", errs[k].c_str());
        std::lock_guard<std::mutex> lk(cache().mu);
        for (size_t k = 0; k < todo.size(); ++k) {
            cache().mods[mods[todo[k]].src] = built[k];
            handles[todo[k]] = built[k];
        }
    }
    // launch
    const int threads = 32 << wb;
    for (size_t m = 0; m < mods.size(); ++m) {
        JitModule &jm = *handles[m];
        const size_t bytes = mods[m].consts.size() * sizeof(float);
        if (bytes > jm.consts_bytes) return fail(QF_ERR_CUDA, "pass compiler: constant bank size mismatch");
        if (bytes) QF_CUDA(cudaMemcpyAsync(jm.consts, mods[m].consts.data(), bytes, cudaMemcpyHostToDevice, ctx->stream));
        for (size_t k = 0; k < mods[m].pass_index.size(); ++k) {
            const RsPass &p = rp.passes[mods[m].pass_index[k]];
            int per_sm = 0;
            const size_t dyn = mods[m].dyn_smem;
            QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)jm.kernels[k], threads, dyn));
            per_sm = std::max(per_sm, 1);
            const uint64_t grid = std::min<uint64_t>((uint64_t)per_sm * ctx->sm_count, p.a.n_tiles);
            float2 *amps = static_cast<float2 *>(sv->d);
            unsigned long long nt = p.a.n_tiles;
            void *args[] = {&amps, &nt};
            QF_CUDA(cudaLaunchKernel((const void *)jm.kernels[k], dim3((unsigned)grid), dim3(threads), args, dyn, ctx->stream));
        }
    }
    return QF_OK;
}

}  // namespace qf
