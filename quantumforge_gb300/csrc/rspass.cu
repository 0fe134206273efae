// rspass.cu — register-tiled tile pass for complex64 states.
//
// One CTA of 32 << WB threads owns a tile of 2^(9+WB) amplitudes per loop
// iteration: lane l holds qubits 0..4 = l (every warp load/store is 256
// contiguous bytes), thread registers r[0..15] span 4 register qubits and the
// warp index spans WB qubits; the remaining qubits pick the tile. A pass of
// gates runs entirely on registers: register-qubit gates are straight-line
// register math, lane-qubit gates use warp shuffles, diagonal gates, CZ and
// CNOT controls read the qubit's bit wherever it lives, and SWAPs among
// register/warp qubits were folded into the layout on the host. Only a gate
// on a warp qubit needs shared memory: a remap writes the tile out and reads
// it back with different qubits in the register positions (32 consecutive
// float2 per warp access: no bank conflicts). HBM traffic is one read and one
// write of the state per pass.
#include <algorithm>

#include "qf_device.cuh"
#include "qf_internal.h"

namespace qf {

constexpr int kRsRegs = 16;

struct RsMat {
    float2 m00, m01, m10, m11;
};

// out0 = m00 a0 + m01 a1, out1 = m10 a0 + m11 a1 with the structure `mk`
__device__ __forceinline__ void mat2(const RsMat &M, int mk, float2 &a0, float2 &a1) {
    const float2 x = a0, y = a1;
    if (mk == 1) {  // real matrix (H, RY, merged real products)
        a0 = make_float2(M.m00.x * x.x + M.m01.x * y.x, M.m00.x * x.y + M.m01.x * y.y);
        a1 = make_float2(M.m10.x * x.x + M.m11.x * y.x, M.m10.x * x.y + M.m11.x * y.y);
    } else if (mk == 2) {  // real diagonal, imaginary off-diagonal (RX)
        a0 = make_float2(M.m00.x * x.x - M.m01.y * y.y, M.m00.x * x.y + M.m01.y * y.x);
        a1 = make_float2(M.m11.x * y.x - M.m10.y * x.y, M.m11.x * y.y + M.m10.y * x.x);
    } else {
        a0 = cmac2(M.m00, x, M.m01, y);
        a1 = cmac2(M.m10, x, M.m11, y);
    }
}

// self = c_self * self + c_other * other
__device__ __forceinline__ float2 mac_pair(float2 cs, float2 self, float2 co, float2 other, int mk) {
    if (mk == 1) return make_float2(cs.x * self.x + co.x * other.x, cs.x * self.y + co.x * other.y);
    return cmac2(cs, self, co, other);
}

template <int B> __device__ __forceinline__ void reg_mat(float2 (&r)[kRsRegs], const RsMat &M, int mk) {
#pragma unroll
    for (int i = 0; i < kRsRegs; ++i)
        if (!(i & (1 << B))) mat2(M, mk, r[i], r[i | (1 << B)]);
}

// bit of descriptor d for register i, given the thread-constant bits
struct BitSrc {
    int reg;    // register position, or -1
    int konst;  // value when not a register bit
};
__device__ __forceinline__ BitSrc bit_src(uint8_t d, uint32_t lane, uint32_t warp, uint64_t base) {
    BitSrc s;
    s.reg = -1;
    s.konst = 0;
    if (d < 8) s.konst = (lane >> d) & 1u;
    else if (d < 16) s.reg = d - 8;
    else if (d < 64) s.konst = (warp >> (d - 16)) & 1u;
    else s.konst = (int)((base >> (d - 64)) & 1ULL);
    return s;
}
__device__ __forceinline__ int bit_of(const BitSrc &s, int i) { return s.reg >= 0 ? (i >> s.reg) & 1 : s.konst; }

template <int B>
__device__ __forceinline__ void reg_cnot(float2 (&r)[kRsRegs], const BitSrc &c) {
#pragma unroll
    for (int i = 0; i < kRsRegs; ++i)
        if (!(i & (1 << B))) {
            const int j = i | (1 << B);
            if (bit_of(c, i)) {
                const float2 t = r[i];
                r[i] = r[j];
                r[j] = t;
            }
        }
}

template <int B>
__device__ __forceinline__ void reg_swap_lane(float2 (&r)[kRsRegs], uint32_t lane, int a) {
    const int la = (lane >> a) & 1;
#pragma unroll
    for (int i = 0; i < kRsRegs; ++i)
        if (!(i & (1 << B))) {
            const int j = i | (1 << B);
            // exchange amplitude (lane bit 1, reg bit 0) with (lane bit 0, reg bit 1)
            const float2 send = la ? r[i] : r[j];
            float2 recv;
            recv.x = __shfl_xor_sync(0xffffffffu, send.x, 1 << a);
            recv.y = __shfl_xor_sync(0xffffffffu, send.y, 1 << a);
            if (la) r[i] = recv;
            else r[j] = recv;
        }
}

__device__ __forceinline__ uint32_t layout_offset(uint32_t packed, int pos) { return (packed >> (3 * pos)) & 7u; }

template <int WB>
__global__ void __launch_bounds__(32 << WB, (WB == 3 ? 2 : 1))
    k_rs_pass(float2 *__restrict__ amps, const RsPassArgs pa, const RsOp *__restrict__ g_ops,
              const double *__restrict__ g_mats) {
    constexpr int NT = 32 << WB;
    extern __shared__ __align__(16) unsigned char smem[];
    float2 *buf = reinterpret_cast<float2 *>(smem);  // kRsRegs * NT amplitudes
    RsOp *ops = reinterpret_cast<RsOp *>(buf + kRsRegs * NT);
    RsMat *mats = reinterpret_cast<RsMat *>(ops + pa.n_ops);

    for (uint32_t o = threadIdx.x; o < pa.n_ops; o += NT) ops[o] = g_ops[o];
    for (uint32_t m = threadIdx.x; m < pa.n_mats; m += NT) {
        const double *s = g_mats + 8 * (size_t)m;
        mats[m].m00 = make_float2((float)s[0], (float)s[1]);
        mats[m].m01 = make_float2((float)s[2], (float)s[3]);
        mats[m].m10 = make_float2((float)s[4], (float)s[5]);
        mats[m].m11 = make_float2((float)s[6], (float)s[7]);
    }
    __syncthreads();

    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    // address bits of the register/warp positions at load and at store
    uint64_t lreg[4], sreg[4], lw = 0, sw = 0;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        lreg[s] = 1ULL << pa.load_q[s];
        sreg[s] = 1ULL << pa.store_q[s];
    }
#pragma unroll
    for (int w = 0; w < WB; ++w) {
        if ((warp >> w) & 1u) {
            lw |= 1ULL << pa.load_q[4 + w];
            sw |= 1ULL << pa.store_q[4 + w];
        }
    }
    // SWAP relabels can leave other qubits in the warp positions at the store
    // than at the load: a warp then stores into amplitudes another warp of the
    // CTA loads, so every warp must have loaded the tile before any stores
    bool cross_warp = false;
#pragma unroll
    for (int w = 0; w < WB; ++w) cross_warp |= pa.load_q[4 + w] != pa.store_q[4 + w];

    for (uint64_t t = blockIdx.x; t < pa.n_tiles; t += gridDim.x) {
        const uint64_t tb = deposit(t, pa.nonlocal_mask);
        float2 r[kRsRegs];
        {
            const uint64_t base = tb | lane | lw;
#pragma unroll
            for (int i = 0; i < kRsRegs; ++i) {
                const uint64_t off = ((i & 1) ? lreg[0] : 0) | ((i & 2) ? lreg[1] : 0) | ((i & 4) ? lreg[2] : 0) |
                                     ((i & 8) ? lreg[3] : 0);
                r[i] = amps[base | off];
            }
        }
        for (uint32_t o = 0; o < pa.n_ops; ++o) {
            const RsOp op = ops[o];
            switch (op.kind) {
            case RS_MREG: {
                const RsMat M = mats[op.mat];
                switch (op.p0) {
                case 0: reg_mat<0>(r, M, op.mk); break;
                case 1: reg_mat<1>(r, M, op.mk); break;
                case 2: reg_mat<2>(r, M, op.mk); break;
                default: reg_mat<3>(r, M, op.mk); break;
                }
                break;
            }
            case RS_MLANE: {
                const RsMat M = mats[op.mat];
                const int bit = (lane >> op.p0) & 1u;
                const float2 cs = bit ? M.m11 : M.m00, co = bit ? M.m10 : M.m01;
                const int mk = op.mk == 1 ? 1 : 0;
#pragma unroll
                for (int i = 0; i < kRsRegs; ++i) {
                    float2 p;
                    p.x = __shfl_xor_sync(0xffffffffu, r[i].x, 1 << op.p0);
                    p.y = __shfl_xor_sync(0xffffffffu, r[i].y, 1 << op.p0);
                    r[i] = mac_pair(cs, r[i], co, p, mk);
                }
                break;
            }
            case RS_DIAG: {
                const RsMat M = mats[op.mat];
                const BitSrc s = bit_src(op.p0, lane, warp, tb);
                const bool one0 = M.m00.x == 1.f && M.m00.y == 0.f;
                if (s.reg < 0) {
                    const float2 f = s.konst ? M.m11 : M.m00;
                    if (!(f.x == 1.f && f.y == 0.f))
#pragma unroll
                        for (int i = 0; i < kRsRegs; ++i) r[i] = cmul(r[i], f);
                } else if (one0) {
#pragma unroll
                    for (int i = 0; i < kRsRegs; ++i)
                        if ((i >> s.reg) & 1) r[i] = cmul(r[i], M.m11);
                } else {
#pragma unroll
                    for (int i = 0; i < kRsRegs; ++i) r[i] = cmul(r[i], ((i >> s.reg) & 1) ? M.m11 : M.m00);
                }
                break;
            }
            case RS_CNOT: {
                const BitSrc c = bit_src(op.p0, lane, warp, tb);
                if (op.p1 < 8) {  // lane target: exchange with the partner lane where the control is set
#pragma unroll
                    for (int i = 0; i < kRsRegs; ++i) {
                        float2 p;
                        p.x = __shfl_xor_sync(0xffffffffu, r[i].x, 1 << op.p1);
                        p.y = __shfl_xor_sync(0xffffffffu, r[i].y, 1 << op.p1);
                        if (bit_of(c, i)) r[i] = p;
                    }
                } else {
                    switch (op.p1 - 8) {
                    case 0: reg_cnot<0>(r, c); break;
                    case 1: reg_cnot<1>(r, c); break;
                    case 2: reg_cnot<2>(r, c); break;
                    default: reg_cnot<3>(r, c); break;
                    }
                }
                break;
            }
            case RS_CZ: {
                const BitSrc a = bit_src(op.p0, lane, warp, tb), b = bit_src(op.p1, lane, warp, tb);
#pragma unroll
                for (int i = 0; i < kRsRegs; ++i)
                    if (bit_of(a, i) & bit_of(b, i)) r[i] = cneg(r[i]);
                break;
            }
            case RS_SWAP_LR: {
                switch (op.p1) {
                case 0: reg_swap_lane<0>(r, lane, op.p0); break;
                case 1: reg_swap_lane<1>(r, lane, op.p0); break;
                case 2: reg_swap_lane<2>(r, lane, op.p0); break;
                default: reg_swap_lane<3>(r, lane, op.p0); break;
                }
                break;
            }
            case RS_SWAP_LL: {
                const uint32_t ba = (lane >> op.p0) & 1u, bb = (lane >> op.p1) & 1u;
                const uint32_t src = (lane & ~((1u << op.p0) | (1u << op.p1))) | (ba << op.p1) | (bb << op.p0);
#pragma unroll
                for (int i = 0; i < kRsRegs; ++i) {
                    r[i].x = __shfl_sync(0xffffffffu, r[i].x, src);
                    r[i].y = __shfl_sync(0xffffffffu, r[i].y, src);
                }
                break;
            }
            default: {  // RS_REMAP through shared memory: index = lane + 32 * (slot bits)
                uint32_t wo = 0, wn = 0;
#pragma unroll
                for (int w = 0; w < WB; ++w)
                    if ((warp >> w) & 1u) {
                        wo |= 1u << layout_offset(op.a, 4 + w);
                        wn |= 1u << layout_offset(op.b, 4 + w);
                    }
                uint32_t ro[4], rn[4];
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    ro[s] = 1u << layout_offset(op.a, s);
                    rn[s] = 1u << layout_offset(op.b, s);
                }
#pragma unroll
                for (int i = 0; i < kRsRegs; ++i) {
                    const uint32_t sl = wo | ((i & 1) ? ro[0] : 0) | ((i & 2) ? ro[1] : 0) | ((i & 4) ? ro[2] : 0) |
                                        ((i & 8) ? ro[3] : 0);
                    buf[lane + 32 * sl] = r[i];
                }
                __syncthreads();
#pragma unroll
                for (int i = 0; i < kRsRegs; ++i) {
                    const uint32_t sl = wn | ((i & 1) ? rn[0] : 0) | ((i & 2) ? rn[1] : 0) | ((i & 4) ? rn[2] : 0) |
                                        ((i & 8) ? rn[3] : 0);
                    r[i] = buf[lane + 32 * sl];
                }
                __syncthreads();
                break;
            }
            }
        }
        if (cross_warp) __syncthreads();
        {
            const uint64_t base = tb | lane | sw;
#pragma unroll
            for (int i = 0; i < kRsRegs; ++i) {
                const uint64_t off = ((i & 1) ? sreg[0] : 0) | ((i & 2) ? sreg[1] : 0) | ((i & 4) ? sreg[2] : 0) |
                                     ((i & 8) ? sreg[3] : 0);
                amps[base | off] = r[i];
            }
        }
    }
}

static size_t rs_smem(int wb, uint32_t n_ops, uint32_t n_mats) {
    return (size_t)kRsRegs * (32u << wb) * sizeof(float2) + n_ops * sizeof(RsOp) + n_mats * sizeof(RsMat);
}

template <int WB> static int rs_launch_all(qf_sv *sv, const RsPlan &rp, const Plan &plan) {
    qf_ctx *ctx = sv->ctx;
    static size_t dyn[64] = {0};
    if (!dyn[ctx->device & 63]) QF_TRY(allow_max_dynamic_smem(k_rs_pass<WB>, ctx, &dyn[ctx->device & 63]));
    const size_t ops_b = (rp.ops.size() * sizeof(RsOp) + 15) / 16 * 16;
    const size_t mats_b = rp.mats.size() * sizeof(double);
    QF_TRY(ensure_device(&ctx->ws_plan, &ctx->ws_plan_bytes, ops_b + mats_b + 16));
    unsigned char *d = static_cast<unsigned char *>(ctx->ws_plan);
    if (!rp.ops.empty())
        QF_CUDA(cudaMemcpyAsync(d, rp.ops.data(), rp.ops.size() * sizeof(RsOp), cudaMemcpyHostToDevice, ctx->stream));
    if (!rp.mats.empty())
        QF_CUDA(cudaMemcpyAsync(d + ops_b, rp.mats.data(), mats_b, cudaMemcpyHostToDevice, ctx->stream));
    const RsOp *d_ops = reinterpret_cast<const RsOp *>(d);
    const double *d_mats = reinterpret_cast<const double *>(d + ops_b);
    size_t max_smem = 0;
    for (const RsPass &p : rp.passes)
        if (!p.fallback) max_smem = std::max(max_smem, rs_smem(WB, p.a.n_ops, p.a.n_mats));
    if (max_smem > dyn[ctx->device & 63])
        return fail(QF_ERR_UNSUPPORTED_OPERATION, "register-tiled pass needs %zu bytes of shared memory", max_smem);
    int per_sm = 0;
    QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rs_pass<WB>, 32 << WB, max_smem));
    per_sm = std::max(per_sm, 1);
    const uint64_t grid = (uint64_t)per_sm * ctx->sm_count;
    for (size_t i = 0; i < rp.passes.size(); ++i) {
        const RsPass &p = rp.passes[i];
        const uint32_t g = (uint32_t)std::min<uint64_t>(grid, p.a.n_tiles);
        k_rs_pass<WB><<<g, 32 << WB, rs_smem(WB, p.a.n_ops, p.a.n_mats), ctx->stream>>>(
            static_cast<float2 *>(sv->d), p.a, d_ops + p.op_begin, d_mats + 8 * (size_t)p.mat_begin);
        QF_CUDA(cudaGetLastError());
    }
    return QF_OK;
}

int run_plan_rs(qf_sv *sv, const Plan &plan, int wb) {
    RsPlan rp;
    QF_TRY(lower_rs(plan, wb, rp));
    for (const RsPass &p : rp.passes)  // a pass that does not fit the register layout: whole plan in shared memory
        if (p.fallback) return run_plan_smem(sv, plan);
    if (wb == 3) return rs_launch_all<3>(sv, rp, plan);
    if (wb == 4) return rs_launch_all<4>(sv, rp, plan);
    return fail(QF_ERR_INVALID_ARGUMENT, "register-tiled passes take 3 or 4 warp qubits, got %d", wb);
}

}  // namespace qf
