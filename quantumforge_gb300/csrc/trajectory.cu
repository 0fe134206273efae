// trajectory.cu — shots of small states as independent per-shot trajectories
// in shared memory (Circuit::run_shots_impl, src/lib.rs:2842-2916, with
// apply_channel_trajectory, src/lib.rs:1356-1506, and StateVector::measure,
// src/lib.rs:1321-1351).
//
// When 2^n amplitudes fit in one CTA's shared memory, every shot is simulated
// by one CTA exactly as the reference does it — the state cloned from the
// initial state, every op applied in order, measurements and channels drawing
// from the shot's own SmallRng position (shot s starts at draw s * d of the
// seeded stream, d = draws per shot) — but without leaving the SM: gates are
// in-place passes over shared memory, P(1) and norms are block reductions, and
// the classical register lives in registers. The grid is a persistent set of
// CTAs striding over shots. Decisions equal the reference's except where a
// uniform lies within tie_eps of a threshold (counted): the block reductions
// add in a different order than the reference's sequential sums, and the
// thresholds are formed with round-to-nearest double operations (no fused
// multiply-add), as the reference forms them.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "qf_device.cuh"
#include "qf_internal.h"

namespace qf {

namespace {

enum : uint8_t { T_GATE = 0, T_CNOT = 1, T_CZ = 2, T_SWAP = 3, T_MEASURE = 4, T_COND = 5, T_DEP = 6, T_AD = 7, T_PD = 8,
                 T_TH = 9, T_DIAG = 10, T_REAL = 11, T_X = 12, T_XLIKE = 13 };

// One op of a trajectory program. GATE/COND: m = the 2x2 matrix (re, im),
// mf the same in f32 for complex64 states; channels: m[0] = probability /
// gamma / gamma_down, m[1] = gamma_up, m[2] = sqrt(m[0]), m[3] = sqrt(1 - m[0]),
// m[4] = sqrt(m[1]), m[5] = sqrt(1 - m[1]).
struct TOp {
    uint8_t kind;
    uint8_t value;   // COND: required classical value
    uint16_t pad;
    uint32_t q0, q1, cbit;
    double m[8];
    float mf[8];
};

constexpr double kEps = 2.220446049250313e-16;

// Indices stay 32-bit: a state in shared memory has at most 2^15 amplitudes.
__device__ __forceinline__ uint32_t ins0(uint32_t x, uint32_t p) {
    return ((x >> p) << (p + 1)) | (x & ((1u << p) - 1u));
}

__device__ __forceinline__ double next_u(uint64_t &x) {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ double clamp01d(double x) { return fmin(1.0, fmax(0.0, x)); }

template <typename R> __device__ __forceinline__ R warp_sum_r(R v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// The per-shot decisions (uniform draw, thresholds, branch weights) are made
// by thread 0 alone in f64 with round-to-nearest operations and broadcast
// through shared memory: FP64 issues at a small fraction of FP32 on GB300, so
// the other 255 threads never touch it for a complex64 state.
template <typename R> struct Decision {
    int branch;  // measurement outcome / Kraus branch / Pauli index (-1: none)
    int fault;
    R s[4];      // scales, already in the state's precision (no per-thread f64 -> f32 conversion)
};

template <typename C>
__global__ void __launch_bounds__(256) k_trajectories(const C *__restrict__ init, uint32_t n, const TOp *__restrict__ ops,
                                                      uint32_t n_ops, uint64_t shots, const uint64_t *__restrict__ starts,
                                                      double tie_eps, int rel_norm, uint64_t *__restrict__ out,
                                                      unsigned long long *ties, int *err) {
    using R = typename Real<C>::T;
    constexpr bool kF32 = sizeof(R) == 4;
    extern __shared__ __align__(16) unsigned char traj_smem[];
    C *a = reinterpret_cast<C *>(traj_smem);
    __shared__ R wred[2][8];
    __shared__ Decision<R> dec;
    const uint32_t dim = 1u << n, half = dim >> 1, quarter = dim >> 2;
    const unsigned tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    for (uint64_t s = blockIdx.x; s < shots; s += gridDim.x) {
        for (uint32_t i = tid; i < dim; i += nt) a[i] = init[i];
        uint64_t rng = starts[s];  // used by thread 0
        uint64_t reg = 0;
        unsigned long long my_ties = 0;
        __syncthreads();
        for (uint32_t k = 0; k < n_ops; ++k) {
            const TOp &op = ops[k];
            const uint8_t kind = op.kind;
            const uint32_t q = op.q0;
            const uint32_t qm = 1u << q;
            if (kind == T_COND && ((reg >> op.cbit) & 1ULL) != (uint64_t)op.value) continue;
            if (kind == T_GATE || kind == T_COND || kind == T_DIAG || kind == T_REAL || kind == T_XLIKE) {
                C m00, m01, m10, m11;
                if (kF32) {
                    m00 = mk((R)op.mf[0], (R)op.mf[1]), m01 = mk((R)op.mf[2], (R)op.mf[3]);
                    m10 = mk((R)op.mf[4], (R)op.mf[5]), m11 = mk((R)op.mf[6], (R)op.mf[7]);
                } else {
                    m00 = mk((R)op.m[0], (R)op.m[1]), m01 = mk((R)op.m[2], (R)op.m[3]);
                    m10 = mk((R)op.m[4], (R)op.m[5]), m11 = mk((R)op.m[6], (R)op.m[7]);
                }
                if (kind == T_DIAG) {  // diag(m00, m11): Rz, S, T, Z and their adjoints
                    for (uint32_t i = tid; i < dim; i += nt) a[i] = cmul((i >> q) & 1u ? m11 : m00, a[i]);
                } else if (kind == T_REAL) {  // real 2x2: H, Ry
                    for (uint32_t p = tid; p < half; p += nt) {
                        const uint32_t i0 = ins0(p, q), i1 = i0 | qm;
                        const C a0 = a[i0], a1 = a[i1];
                        a[i0] = mk(m00.x * a0.x + m01.x * a1.x, m00.x * a0.y + m01.x * a1.y);
                        a[i1] = mk(m10.x * a0.x + m11.x * a1.x, m10.x * a0.y + m11.x * a1.y);
                    }
                } else if (kind == T_XLIKE) {  // real diagonal, imaginary off-diagonal: Rx
                    for (uint32_t p = tid; p < half; p += nt) {
                        const uint32_t i0 = ins0(p, q), i1 = i0 | qm;
                        const C a0 = a[i0], a1 = a[i1];
                        a[i0] = mk(m00.x * a0.x - m01.y * a1.y, m00.x * a0.y + m01.y * a1.x);
                        a[i1] = mk(m11.x * a1.x - m10.y * a0.y, m11.x * a1.y + m10.y * a0.x);
                    }
                } else {
                    for (uint32_t p = tid; p < half; p += nt) {
                        const uint32_t i0 = ins0(p, q), i1 = i0 | qm;
                        const C a0 = a[i0], a1 = a[i1];
                        a[i0] = cmac2(m00, a0, m01, a1);
                        a[i1] = cmac2(m10, a0, m11, a1);
                    }
                }
                __syncthreads();
                continue;
            }
            if (kind == T_X) {
                for (uint32_t p = tid; p < half; p += nt) {
                    const uint32_t i0 = ins0(p, q), i1 = i0 | qm;
                    const C a0 = a[i0];
                    a[i0] = a[i1];
                    a[i1] = a0;
                }
                __syncthreads();
                continue;
            }
            if (kind == T_CNOT || kind == T_CZ || kind == T_SWAP) {
                const uint32_t q1 = op.q1, lo = min(q, q1), hi = max(q, q1);
                const uint32_t m1 = 1u << q1;
                for (uint32_t p = tid; p < quarter; p += nt) {
                    const uint32_t b = ins0(ins0(p, lo), hi);
                    if (kind == T_CNOT) {  // control q, target q1
                        const C t = a[b | qm];
                        a[b | qm] = a[b | qm | m1];
                        a[b | qm | m1] = t;
                    } else if (kind == T_CZ) {
                        const C t = a[b | qm | m1];
                        a[b | qm | m1] = mk(-t.x, -t.y);
                    } else {
                        const C t = a[b | qm];
                        a[b | qm] = a[b | m1];
                        a[b | m1] = t;
                    }
                }
                __syncthreads();
                continue;
            }
            if (kind == T_DEP) {  // src/lib.rs:1369-1381: one draw, X/Y/Z with probability p/3 each
                if (tid == 0) {
                    const double pr = op.m[0];
                    const double u = next_u(rng);
                    const double keep = __dsub_rn(1.0, pr);
                    int g = -1;
                    if (u >= keep && pr > 0.0) {
                        const double b = floor(__dmul_rn(__dsub_rn(u, keep), __ddiv_rn(3.0, pr)));
                        g = b >= 2.0 ? 2 : (int)b;
                    }
                    dec.branch = g;
                }
                __syncthreads();
                const int g = dec.branch;
                if (g >= 0) {
                    for (uint32_t p = tid; p < half; p += nt) {
                        const uint32_t i0 = ins0(p, q), i1 = i0 | qm;
                        const C a0 = a[i0], a1 = a[i1];
                        if (g == 0) {  // X
                            a[i0] = a1;
                            a[i1] = a0;
                        } else if (g == 1) {  // Y: (a0, a1) -> (-i a1, i a0)
                            a[i0] = mk(a1.y, -a1.x);
                            a[i1] = mk(-a0.y, a0.x);
                        } else {  // Z
                            a[i1] = mk(-a1.x, -a1.y);
                        }
                    }
                }
                __syncthreads();
                continue;
            }
            // measurement and damping channels: P(1) and the norm, reduced
            // per thread and per warp in the state's precision
            {
                R xs = 0, ys = 0;
                for (uint32_t i = tid; i < dim; i += nt) {
                    const C v = a[i];
                    const R w = v.x * v.x + v.y * v.y;
                    ys += w;
                    if ((i >> q) & 1u) xs += w;
                }
                xs = warp_sum_r(xs);
                ys = warp_sum_r(ys);
                if (lane == 0) {
                    wred[0][warp] = xs;
                    wred[1][warp] = ys;
                }
            }
            __syncthreads();
            if (tid == 0) {
                double p_one = 0.0, norm = 0.0;
                for (unsigned w = 0; w < (nt >> 5); ++w) {
                    p_one += (double)wred[0][w];
                    norm += (double)wred[1][w];
                }
                Decision<R> d{-1, 0, {(R)0, (R)0, (R)0, (R)0}};
                if (kind == T_MEASURE) {  // StateVector::measure, src/lib.rs:1321-1351
                    double p = p_one;
                    if (rel_norm && norm > 0.0) p = __ddiv_rn(p_one, norm);
                    p = clamp01d(p);
                    const double u = next_u(rng);
                    d.branch = u < p ? 1 : 0;
                    if (fabs(u - p) < tie_eps) ++my_ties;
                    const double prob = d.branch ? p : __dsub_rn(1.0, p);
                    if (prob <= kEps) d.fault = 1;
                    else d.s[0] = (R)(1.0 / sqrt(prob));  // one rounding more than the reference's division
                } else if (kind == T_AD || kind == T_PD) {  // src/lib.rs:1383-1438
                    const double g = op.m[0];
                    if (!isfinite(norm) || norm <= kEps) {
                        d.fault = 1;
                    } else {
                        const double gp = __dmul_rn(g, p_one);
                        const double jp = clamp01d(__ddiv_rn(gp, norm));
                        const double u = next_u(rng);
                        d.branch = u < jp ? 1 : 0;
                        if (fabs(u - jp) < tie_eps) ++my_ties;
                        const double bn = d.branch ? gp : __dsub_rn(norm, gp);
                        if (!isfinite(bn) || bn <= kEps) {
                            d.fault = 1;
                        } else {
                            const double inv = 1.0 / sqrt(bn);
                            d.s[0] = (R)inv;
                            d.s[1] = (R)(op.m[2] * inv);  // jump
                            d.s[2] = (R)(op.m[3] * inv);  // no jump, excited part
                        }
                    }
                } else {  // T_TH, src/lib.rs:1440-1503
                    const double gd = op.m[0], gu = op.m[1];
                    if (!isfinite(norm) || norm <= kEps) {
                        d.fault = 1;
                    } else {
                        const double p1 = clamp01d(__ddiv_rn(p_one, norm)), p0 = __dsub_rn(1.0, p1);
                        const double down = __dmul_rn(p1, gd), up = __dmul_rn(p0, gu);
                        const double stay = __dadd_rn(__dmul_rn(p0, __dsub_rn(1.0, gu)), __dmul_rn(p1, __dsub_rn(1.0, gd)));
                        const double du = __dadd_rn(down, up);
                        const double u = next_u(rng);
                        d.branch = u < down ? 1 : (u < du ? 2 : 0);
                        if (fabs(u - down) < tie_eps || fabs(u - du) < tie_eps) ++my_ties;
                        const double bn = d.branch == 1 ? down : (d.branch == 2 ? up : stay);
                        if (!isfinite(bn) || bn <= kEps) {
                            d.fault = 1;
                        } else {
                            const double inv = 1.0 / sqrt(bn);
                            d.s[0] = (R)(op.m[2] * inv);  // down
                            d.s[1] = (R)(op.m[4] * inv);  // up
                            d.s[2] = (R)(op.m[5] * inv);  // stay, ground part
                            d.s[3] = (R)(op.m[3] * inv);  // stay, excited part
                        }
                    }
                }
                dec = d;
                if (d.fault) atomicExch(err, 1);
            }
            __syncthreads();
            if (dec.fault) return;  // uniform across the CTA
            const int br = dec.branch;
            if (kind == T_MEASURE) {
                const R inv = dec.s[0];
                for (uint32_t i = tid; i < dim; i += nt) {
                    const C v = a[i];
                    a[i] = ((int)((i >> q) & 1u) == br) ? mk(v.x * inv, v.y * inv) : mk((R)0, (R)0);
                }
                reg = (reg & ~(1ULL << op.cbit)) | ((uint64_t)br << op.cbit);
            } else if (kind == T_AD || kind == T_PD) {
                const R inv = dec.s[0], s_jump = dec.s[1], s_exc = dec.s[2];
                for (uint32_t p = tid; p < half; p += nt) {
                    const uint32_t i0 = ins0(p, q), i1 = i0 | qm;
                    const C a0 = a[i0], a1 = a[i1];
                    if (br) {
                        if (kind == T_AD) {
                            a[i0] = mk(a1.x * s_jump, a1.y * s_jump);
                            a[i1] = mk((R)0, (R)0);
                        } else {
                            a[i0] = mk((R)0, (R)0);
                            a[i1] = mk(a1.x * s_jump, a1.y * s_jump);
                        }
                    } else {
                        a[i0] = mk(a0.x * inv, a0.y * inv);
                        a[i1] = mk(a1.x * s_exc, a1.y * s_exc);
                    }
                }
            } else {
                const R s1 = dec.s[0], s2 = dec.s[1], s0g = dec.s[2], s0e = dec.s[3];
                for (uint32_t p = tid; p < half; p += nt) {
                    const uint32_t i0 = ins0(p, q), i1 = i0 | qm;
                    const C a0 = a[i0], a1 = a[i1];
                    if (br == 1) {
                        a[i0] = mk(a1.x * s1, a1.y * s1);
                        a[i1] = mk((R)0, (R)0);
                    } else if (br == 2) {
                        a[i1] = mk(a0.x * s2, a0.y * s2);
                        a[i0] = mk((R)0, (R)0);
                    } else {
                        a[i0] = mk(a0.x * s0g, a0.y * s0g);
                        a[i1] = mk(a1.x * s0e, a1.y * s0e);
                    }
                }
            }
            __syncthreads();
        }
        if (tid == 0) {
            out[s] = reg;
            if (my_ties) atomicAdd(ties, my_ties);
        }
        __syncthreads();
    }
}

template <typename C> int launch_trajectories(qf_sv *init, const TOp *d_ops, uint32_t n_ops, uint64_t shots,
                                              const uint64_t *d_starts, double tie_eps, uint64_t *d_out,
                                              unsigned long long *d_ties, int *d_err) {
    qf_ctx *ctx = init->ctx;
    const size_t bytes = init->bytes();
    QF_CUDA(cudaFuncSetAttribute(k_trajectories<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    int per_sm = 0;
    QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trajectories<C>, 256, bytes));
    per_sm = std::max(1, per_sm);
    const uint64_t grid = std::min<uint64_t>(shots, (uint64_t)ctx->sm_count * per_sm);
    k_trajectories<C><<<(unsigned)grid, 256, bytes, ctx->stream>>>(static_cast<const C *>(init->d), init->n, d_ops, n_ops,
                                                                  shots, d_starts, tie_eps, init->dtype == QF_C64 ? 1 : 0,
                                                                  d_out, d_ties, d_err);
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

}  // namespace

bool trajectories_fit(const qf_ctx *ctx, uint32_t n, int dtype) {
    if (n < 2 || n > 15) return false;
    const size_t bytes = (size_t(1) << n) * (dtype == QF_C64 ? 8u : 16u);
    return bytes + 2048 <= ctx->smem_optin;
}

int run_trajectories(qf_sv *init, const qf_op *ops, uint64_t n_ops, uint64_t shots, const uint64_t *starts, double tie_eps,
                     bool allow_noise, uint64_t *outcomes, uint64_t *n_ties) {
    qf_ctx *ctx = init->ctx;
    const uint32_t n = init->n;
    std::vector<TOp> prog;
    prog.reserve(n_ops);
    for (uint64_t k = 0; k < n_ops; ++k) {
        const qf_op &o = ops[k];
        TOp t{};
        t.q0 = o.q0;
        t.q1 = o.q1;
        switch (o.kind) {
        case QF_OP_GATE:
        case QF_OP_COND: {
            qf_op g = o;
            g.kind = QF_OP_GATE;
            g.param = 0;
            g.flags = 0;
            std::vector<BGate> b;
            QF_TRY(bind_ops(n, &g, 1, nullptr, 0, nullptr, 0, -1, 0.0, b));
            t.kind = o.kind == QF_OP_GATE ? T_GATE : T_COND;
            t.value = (uint8_t)(o.flags & 1);
            t.cbit = o.param;
            for (int j = 0; j < 8; ++j) {
                t.m[j] = b[0].m[j];
                t.mf[j] = (float)b[0].m[j];
            }
            if (t.kind == T_GATE) {  // structured matrices: fewer floating-point operations per pair
                const double *m = t.m;
                if (o.gate == QF_GATE_X) t.kind = T_X;
                else if (b[0].diag) t.kind = T_DIAG;
                else if (m[1] == 0.0 && m[3] == 0.0 && m[5] == 0.0 && m[7] == 0.0) t.kind = T_REAL;
                else if (m[1] == 0.0 && m[7] == 0.0 && m[2] == 0.0 && m[4] == 0.0) t.kind = T_XLIKE;
            }
            break;
        }
        case QF_OP_CNOT:
        case QF_OP_CZ:
        case QF_OP_SWAP: {
            std::vector<BGate> b;
            QF_TRY(bind_ops(n, &o, 1, nullptr, 0, nullptr, 0, -1, 0.0, b));
            t.kind = o.kind == QF_OP_CNOT ? T_CNOT : o.kind == QF_OP_CZ ? T_CZ : T_SWAP;
            break;
        }
        case QF_OP_MEASURE:
            if (o.q0 >= n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", o.q0, n);
            t.kind = T_MEASURE;
            t.cbit = o.param;
            break;
        case QF_OP_CHANNEL: {
            if (!allow_noise)
                return fail(QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX, "this circuit operation requires density-matrix simulation");
            if (o.q0 >= n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", o.q0, n);
            const double p = o.theta;
            if (!std::isfinite(p) || p < 0.0 || p > 1.0)
                return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", p);
            double gu = 0.0;
            if (o.gate == QF_CHANNEL_THERMAL_DAMPING) {
                const double beta = qf_op_aux(&o);
                if (!std::isfinite(beta) || beta < 0.0)
                    return fail(QF_ERR_INVALID_PROBABILITY, "probability must be in [0, 1], got %g", beta);
                gu = p * std::exp(-beta);  // NoiseChannel::thermal_rates (src/lib.rs:1611-1626)
            }
            switch (o.gate) {
            case QF_CHANNEL_DEPOLARIZING: t.kind = T_DEP; break;
            case QF_CHANNEL_AMPLITUDE_DAMPING: t.kind = T_AD; break;
            case QF_CHANNEL_PHASE_DAMPING: t.kind = T_PD; break;
            case QF_CHANNEL_THERMAL_DAMPING: t.kind = T_TH; break;
            default: return fail(QF_ERR_INVALID_ARGUMENT, "unknown noise channel %u", (unsigned)o.gate);
            }
            t.m[0] = p;
            t.m[1] = gu;
            t.m[2] = std::sqrt(p);
            t.m[3] = std::sqrt(1.0 - p);
            t.m[4] = std::sqrt(gu);
            t.m[5] = std::sqrt(1.0 - gu);
            break;
        }
        default:
            return fail(QF_ERR_INVALID_ARGUMENT, "operation kind %u is not valid in a shot circuit", (unsigned)o.kind);
        }
        prog.push_back(t);
    }
    // workspace: ops | starts | outcomes | ties + error
    const size_t ops_b = sizeof(TOp) * std::max<size_t>(prog.size(), 1);
    const size_t st_b = sizeof(uint64_t) * shots, out_b = sizeof(uint64_t) * shots;
    QF_TRY(ensure_device(&ctx->ws_tree, &ctx->ws_tree_bytes, ops_b + st_b + out_b + 16));
    unsigned char *w = static_cast<unsigned char *>(ctx->ws_tree);
    TOp *d_ops = reinterpret_cast<TOp *>(w);
    uint64_t *d_starts = reinterpret_cast<uint64_t *>(w + ops_b);
    uint64_t *d_out = reinterpret_cast<uint64_t *>(w + ops_b + st_b);
    unsigned long long *d_ties = reinterpret_cast<unsigned long long *>(w + ops_b + st_b + out_b);
    int *d_err = reinterpret_cast<int *>(d_ties + 1);
    if (!prog.empty()) QF_CUDA(cudaMemcpyAsync(d_ops, prog.data(), sizeof(TOp) * prog.size(), cudaMemcpyHostToDevice, ctx->stream));
    QF_CUDA(cudaMemcpyAsync(d_starts, starts, st_b, cudaMemcpyHostToDevice, ctx->stream));
    QF_CUDA(cudaMemsetAsync(d_ties, 0, 16, ctx->stream));
    if (init->dtype == QF_C64)
        QF_TRY(launch_trajectories<float2>(init, d_ops, (uint32_t)prog.size(), shots, d_starts, tie_eps, d_out, d_ties, d_err));
    else
        QF_TRY(launch_trajectories<double2>(init, d_ops, (uint32_t)prog.size(), shots, d_starts, tie_eps, d_out, d_ties, d_err));
    if (outcomes) QF_CUDA(cudaMemcpyAsync(outcomes, d_out, out_b, cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaMemcpyAsync(ctx->h_small, d_ties, 16, cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    unsigned long long t;
    int e;
    std::memcpy(&t, ctx->h_small, sizeof t);
    std::memcpy(&e, reinterpret_cast<unsigned char *>(ctx->h_small) + 8, sizeof e);
    if (e) return fail(QF_ERR_INVALID_PROBABILITY, "a shot selected a branch of probability <= f64::EPSILON");
    if (n_ties) *n_ties = t;
    return QF_OK;
}

}  // namespace qf
