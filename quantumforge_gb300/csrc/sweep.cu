// sweep.cu — gate-application kernels.
//
// Two execution forms replace the reference's per-gate NVRTC kernels
// (src/cuda.rs:79-128, launched once per gate with a cuCtxSynchronize):
//
//  * Unfused sweeps: one HBM pass per gate, 16-byte vector accesses, 64-bit
//    indices, 2^n/(2 or 4) work items in a grid-stride loop. This is the
//    reference's structure, kept as the unfused baseline and for the
//    single-gate API (CudaDeviceState::apply_gate, src/cuda.rs:1296-1325).
//  * Tile passes: a pass keeps k qubits resident. Each CTA gathers one 2^k
//    amplitude tile (contiguous runs of 2^low amplitudes, the other resident
//    qubits strided) into shared memory, applies every gate of the pass in
//    shared memory and writes the tile back: one HBM round trip for a whole
//    run of gates. Gates whose qubits are not resident but are diagonal (Rz,
//    S, T, Z, CZ) or only control a CNOT act as per-tile scalars/conditions.
//    The dual form carries psi and lambda together for the adjoint backward
//    sweep and accumulates the gradient overlaps in f64.
#include <algorithm>

#include "qf_device.cuh"
#include "qf_internal.h"

namespace qf {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// Unfused kernels
// ---------------------------------------------------------------------------

// Dense 2x2 on qubit 0, complex64: one float4 = one (a0, a1) pair.
__global__ void k_g1_c64_q0(float4 *__restrict__ a, uint64_t n_pairs, float2 m00, float2 m01, float2 m10,
                            float2 m11) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n_pairs;
         v += (uint64_t)gridDim.x * blockDim.x) {
        float4 x = a[v];
        const float2 a0 = make_float2(x.x, x.y), a1 = make_float2(x.z, x.w);
        const float2 r0 = cmac2(m00, a0, m01, a1), r1 = cmac2(m10, a0, m11, a1);
        a[v] = make_float4(r0.x, r0.y, r1.x, r1.y);
    }
}

// Dense 2x2 on qubit q >= 1, complex64: two adjacent pairs per thread.
__global__ void k_g1_c64_qhi(float2 *__restrict__ a, uint64_t n_items, uint32_t q, float2 m00, float2 m01,
                             float2 m10, float2 m11) {
    const uint64_t mask = 1ULL << q;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n_items;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i0 = insert0(v << 1, q);
        float4 *p0 = reinterpret_cast<float4 *>(a + i0);
        float4 *p1 = reinterpret_cast<float4 *>(a + (i0 | mask));
        const float4 x = *p0, y = *p1;
        const float2 a0 = make_float2(x.x, x.y), b0 = make_float2(x.z, x.w);
        const float2 a1 = make_float2(y.x, y.y), b1 = make_float2(y.z, y.w);
        const float2 r0 = cmac2(m00, a0, m01, a1), r1 = cmac2(m10, a0, m11, a1);
        const float2 s0 = cmac2(m00, b0, m01, b1), s1 = cmac2(m10, b0, m11, b1);
        *p0 = make_float4(r0.x, r0.y, s0.x, s0.y);
        *p1 = make_float4(r1.x, r1.y, s1.x, s1.y);
    }
}

// Dense 2x2, complex128: one pair per thread, 16-byte accesses.
__global__ void k_g1_c128(double2 *__restrict__ a, uint64_t n_pairs, uint32_t q, double2 m00, double2 m01,
                          double2 m10, double2 m11) {
    const uint64_t mask = 1ULL << q;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n_pairs;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i0 = insert0(p, q), i1 = i0 | mask;
        const double2 a0 = a[i0], a1 = a[i1];
        a[i0] = cmac2(m00, a0, m01, a1);
        a[i1] = cmac2(m10, a0, m11, a1);
    }
}

// Diagonal diag(d0, d1) on qubit q. When d0 == 1 only the bit-set half is
// touched (Z, S, T and friends move N*b bytes, not 2*N*b).
template <typename C>
__global__ void k_diag1(C *__restrict__ a, uint64_t dim, uint32_t q, C d0, C d1, int skip_zero_half) {
    const uint64_t mask = 1ULL << q;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if (skip_zero_half) {
        const uint64_t half = dim >> 1;
        for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < half; p += stride) {
            const uint64_t i = insert0(p, q) | mask;
            a[i] = cmul(a[i], d1);
        }
    } else {
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += stride)
            a[i] = cmul(a[i], (i & mask) ? d1 : d0);
    }
}

// CNOT / CZ / SWAP over the 2^(n-2) quads (StateVector::apply_cnot/cz/swap,
// src/lib.rs:1062-1122): exact moves and sign flips.
enum { OP2_CNOT = 0, OP2_CZ = 1, OP2_SWAP = 2 };
template <typename C>
__global__ void k_gate2(C *__restrict__ a, uint64_t n_quads, int op, uint32_t q0, uint32_t q1) {
    const uint32_t lo = q0 < q1 ? q0 : q1, hi = q0 < q1 ? q1 : q0;
    const uint64_t m0 = 1ULL << q0, m1 = 1ULL << q1;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n_quads;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = insert00(p, lo, hi);
        if (op == OP2_CNOT) {  // control q0, target q1
            const uint64_t i = b | m0, j = i | m1;
            const C t = a[i];
            a[i] = a[j];
            a[j] = t;
        } else if (op == OP2_CZ) {
            const uint64_t i = b | m0 | m1;
            a[i] = cneg(a[i]);
        } else {  // swap 01 <-> 10
            const uint64_t i = b | m1, j = b | m0;
            const C t = a[i];
            a[i] = a[j];
            a[j] = t;
        }
    }
}

// complex64 form with both qubits >= 1: two adjacent quads per thread.
__global__ void k_gate2_c64_vec(float2 *__restrict__ a, uint64_t n_items, int op, uint32_t q0, uint32_t q1) {
    const uint32_t lo = q0 < q1 ? q0 : q1, hi = q0 < q1 ? q1 : q0;
    const uint64_t m0 = 1ULL << q0, m1 = 1ULL << q1;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n_items;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = insert00(v << 1, lo, hi);
        if (op == OP2_CNOT) {
            float4 *pi = reinterpret_cast<float4 *>(a + (b | m0));
            float4 *pj = reinterpret_cast<float4 *>(a + (b | m0 | m1));
            const float4 x = *pi, y = *pj;
            *pi = y;
            *pj = x;
        } else if (op == OP2_CZ) {
            float4 *pi = reinterpret_cast<float4 *>(a + (b | m0 | m1));
            const float4 x = *pi;
            *pi = make_float4(-x.x, -x.y, -x.z, -x.w);
        } else {
            float4 *pi = reinterpret_cast<float4 *>(a + (b | m1));
            float4 *pj = reinterpret_cast<float4 *>(a + (b | m0));
            const float4 x = *pi, y = *pj;
            *pi = y;
            *pj = x;
        }
    }
}

static int grid_for(const qf_ctx *ctx, uint64_t items) {
    const uint64_t want = (items + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)std::max(1, ctx->sm_count) * 8;
    return (int)std::max<uint64_t>(1, std::min(want, cap));
}

template <typename C> static C to_c(const double *m);
template <> float2 to_c<float2>(const double *m) { return make_float2((float)m[0], (float)m[1]); }
template <> double2 to_c<double2>(const double *m) { return make_double2(m[0], m[1]); }

int launch_gate1(qf_sv *sv, const BGate &g) {
    qf_ctx *ctx = sv->ctx;
    const uint64_t dim = sv->dim;
    const bool one00 = g.m[0] == 1.0 && g.m[1] == 0.0;
    if (sv->dtype == QF_C64) {
        const float2 m00 = to_c<float2>(g.m), m01 = to_c<float2>(g.m + 2), m10 = to_c<float2>(g.m + 4),
                     m11 = to_c<float2>(g.m + 6);
        float2 *a = static_cast<float2 *>(sv->d);
        if (g.diag) {
            const int skip = one00 ? 1 : 0;
            const uint64_t items = skip ? dim / 2 : dim;
            k_diag1<float2><<<grid_for(ctx, items), kThreads, 0, ctx->stream>>>(a, dim, g.q0, m00, m11, skip);
        } else if (g.q0 == 0 || dim < 4) {
            if (g.q0 == 0) {
                k_g1_c64_q0<<<grid_for(ctx, dim / 2), kThreads, 0, ctx->stream>>>(reinterpret_cast<float4 *>(a),
                                                                                 dim / 2, m00, m01, m10, m11);
            } else {
                // dim == 2 cannot have q0 >= 1
                return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range", g.q0);
            }
        } else {
            k_g1_c64_qhi<<<grid_for(ctx, dim / 4), kThreads, 0, ctx->stream>>>(a, dim / 4, g.q0, m00, m01, m10, m11);
        }
    } else {
        const double2 m00 = to_c<double2>(g.m), m01 = to_c<double2>(g.m + 2), m10 = to_c<double2>(g.m + 4),
                      m11 = to_c<double2>(g.m + 6);
        double2 *a = static_cast<double2 *>(sv->d);
        if (g.diag) {
            const int skip = one00 ? 1 : 0;
            const uint64_t items = skip ? dim / 2 : dim;
            k_diag1<double2><<<grid_for(ctx, items), kThreads, 0, ctx->stream>>>(a, dim, g.q0, m00, m11, skip);
        } else {
            k_g1_c128<<<grid_for(ctx, dim / 2), kThreads, 0, ctx->stream>>>(a, dim / 2, g.q0, m00, m01, m10, m11);
        }
    }
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

int launch_gate2(qf_sv *sv, const BGate &g) {
    qf_ctx *ctx = sv->ctx;
    const int op = g.kind == BK_CNOT ? OP2_CNOT : g.kind == BK_CZ ? OP2_CZ : OP2_SWAP;
    const uint64_t quads = sv->dim / 4;
    if (sv->dtype == QF_C64) {
        float2 *a = static_cast<float2 *>(sv->d);
        if (g.q0 >= 1 && g.q1 >= 1 && quads >= 2)
            k_gate2_c64_vec<<<grid_for(ctx, quads / 2), kThreads, 0, ctx->stream>>>(a, quads / 2, op, g.q0, g.q1);
        else
            k_gate2<float2><<<grid_for(ctx, quads), kThreads, 0, ctx->stream>>>(a, quads, op, g.q0, g.q1);
    } else {
        k_gate2<double2><<<grid_for(ctx, quads), kThreads, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), quads,
                                                                          op, g.q0, g.q1);
    }
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

// ---------------------------------------------------------------------------
// Tile passes
// ---------------------------------------------------------------------------

struct TileSmem {
    uint32_t s0, s1, hi, ops, mats, acc, red, total;
};

__host__ __device__ inline uint32_t align_up(uint32_t x, uint32_t a) { return (x + a - 1) / a * a; }

__host__ __device__ inline TileSmem tile_smem(uint32_t k, uint32_t low, uint32_t n_ops, uint32_t n_mats,
                                              uint32_t n_slots, bool dual, uint32_t amp_bytes) {
    TileSmem L;
    uint32_t off = 0;
    const uint32_t tile = (1u << k) * amp_bytes;
    L.s0 = off;
    off += tile;
    L.s1 = off;
    if (dual) off += tile;
    L.hi = off;
    off += 8u << (k - low);
    L.ops = off;
    off = align_up(off + (uint32_t)sizeof(TileOp) * n_ops, 16);
    L.mats = off;
    off += 4 * amp_bytes * n_mats;
    off = align_up(off, 8);
    L.acc = off;
    off += 8 * n_slots;
    L.red = off;
    off += 8 * 32;
    L.total = align_up(off, 16);
    return L;
}

template <typename C>
__device__ __forceinline__ void tile_load(C *s, const C *__restrict__ g, uint64_t base, const uint64_t *hi_off,
                                          uint32_t T, uint32_t low) {
    const uint32_t lowmask = (1u << low) - 1;
    if (sizeof(C) == 8) {  // complex64: 2 amplitudes per 16-byte access (low >= 1)
        for (uint32_t v = threadIdx.x; v < (T >> 1); v += blockDim.x) {
            const uint32_t j = v << 1;
            const uint64_t gi = base | hi_off[j >> low] | (j & lowmask);
            *reinterpret_cast<float4 *>(s + j) = *reinterpret_cast<const float4 *>(g + gi);
        }
    } else {
        for (uint32_t j = threadIdx.x; j < T; j += blockDim.x) s[j] = g[base | hi_off[j >> low] | (j & lowmask)];
    }
}

template <typename C>
__device__ __forceinline__ void tile_store(const C *s, C *__restrict__ g, uint64_t base, const uint64_t *hi_off,
                                           uint32_t T, uint32_t low) {
    const uint32_t lowmask = (1u << low) - 1;
    if (sizeof(C) == 8) {
        for (uint32_t v = threadIdx.x; v < (T >> 1); v += blockDim.x) {
            const uint32_t j = v << 1;
            const uint64_t gi = base | hi_off[j >> low] | (j & lowmask);
            *reinterpret_cast<float4 *>(g + gi) = *reinterpret_cast<const float4 *>(s + j);
        }
    } else {
        for (uint32_t j = threadIdx.x; j < T; j += blockDim.x) g[base | hi_off[j >> low] | (j & lowmask)] = s[j];
    }
}

// A factored unitary (T_MAT1F): out0 = P + r0 Q, out1 = sigma Q + r1 P with
// (P, Q) = (x, y) for pivot 0 and (y, x) for pivot 1, r real or imaginary;
// the pass's factor comes with T_SCALE.
template <typename C, bool PIV, bool NEG, bool IM>
__device__ __forceinline__ void mat1f_pair(C *s, uint32_t i0, uint32_t i1, C r0, C r1) {
    const C x = s[i0], y = s[i1];
    const C P = PIV ? y : x, Q = PIV ? x : y;
    const C sq = NEG ? mk(-Q.x, -Q.y) : Q;
    if (IM) {  // r = i rho: r v = (-rho v.y, rho v.x)
        s[i0] = mk(P.x - r0.y * Q.y, P.y + r0.y * Q.x);
        s[i1] = mk(sq.x - r1.y * P.y, sq.y + r1.y * P.x);
    } else {
        s[i0] = mk(P.x + r0.x * Q.x, P.y + r0.x * Q.y);
        s[i1] = mk(sq.x + r1.x * P.x, sq.y + r1.x * P.y);
    }
}
template <typename C, bool DUAL, bool PIV, bool NEG, bool IM>
__device__ __forceinline__ void mat1f_tile(C *s0, C *s1, uint32_t b, C r0, C r1, uint32_t T) {
    for (uint32_t p = threadIdx.x; p < (T >> 1); p += blockDim.x) {
        const uint32_t i0 = insert0_32(p, b), i1 = i0 | (1u << b);
        mat1f_pair<C, PIV, NEG, IM>(s0, i0, i1, r0, r1);
        if (DUAL) mat1f_pair<C, PIV, NEG, IM>(s1, i0, i1, r0, r1);
    }
}

template <typename C, bool DUAL>
__device__ __forceinline__ void tile_apply(const TileOp &op, C *s0, C *s1, const C *mats, uint64_t base,
                                           uint32_t T) {
    const uint32_t tid = threadIdx.x, bd = blockDim.x;
    switch (op.kind) {
    case T_MAT1: {
        const C m00 = mats[4 * op.mat], m01 = mats[4 * op.mat + 1], m10 = mats[4 * op.mat + 2],
                m11 = mats[4 * op.mat + 3];
        const uint32_t b = op.b0, mb = 1u << b;
        // Complex128 passes run at the FP64 issue rate, so matrices whose
        // entries are all real (H, Ry) or real on the diagonal and imaginary
        // off it (Rx) take half the multiplies of a general 2x2.
        const bool real = m00.y == 0 && m01.y == 0 && m10.y == 0 && m11.y == 0;
        const bool xlike = !real && m00.y == 0 && m11.y == 0 && m01.x == 0 && m10.x == 0;
        if (sizeof(C) == 16 && real) {
            for (uint32_t p = tid; p < (T >> 1); p += bd) {
                const uint32_t i0 = insert0_32(p, b), i1 = i0 | mb;
                const C a0 = s0[i0], a1 = s0[i1];
                s0[i0] = mk(m00.x * a0.x + m01.x * a1.x, m00.x * a0.y + m01.x * a1.y);
                s0[i1] = mk(m10.x * a0.x + m11.x * a1.x, m10.x * a0.y + m11.x * a1.y);
                if (DUAL) {
                    const C c0 = s1[i0], c1 = s1[i1];
                    s1[i0] = mk(m00.x * c0.x + m01.x * c1.x, m00.x * c0.y + m01.x * c1.y);
                    s1[i1] = mk(m10.x * c0.x + m11.x * c1.x, m10.x * c0.y + m11.x * c1.y);
                }
            }
        } else if (sizeof(C) == 16 && xlike) {  // (m00, i u; i v, m11), all four real numbers
            const auto u = m01.y, v = m10.y;
            for (uint32_t p = tid; p < (T >> 1); p += bd) {
                const uint32_t i0 = insert0_32(p, b), i1 = i0 | mb;
                const C a0 = s0[i0], a1 = s0[i1];
                s0[i0] = mk(m00.x * a0.x - u * a1.y, m00.x * a0.y + u * a1.x);
                s0[i1] = mk(m11.x * a1.x - v * a0.y, m11.x * a1.y + v * a0.x);
                if (DUAL) {
                    const C c0 = s1[i0], c1 = s1[i1];
                    s1[i0] = mk(m00.x * c0.x - u * c1.y, m00.x * c0.y + u * c1.x);
                    s1[i1] = mk(m11.x * c1.x - v * c0.y, m11.x * c1.y + v * c0.x);
                }
            }
        } else {
            for (uint32_t p = tid; p < (T >> 1); p += bd) {
                const uint32_t i0 = insert0_32(p, b), i1 = i0 | mb;
                const C a0 = s0[i0], a1 = s0[i1];
                s0[i0] = cmac2(m00, a0, m01, a1);
                s0[i1] = cmac2(m10, a0, m11, a1);
                if (DUAL) {
                    const C c0 = s1[i0], c1 = s1[i1];
                    s1[i0] = cmac2(m00, c0, m01, c1);
                    s1[i1] = cmac2(m10, c0, m11, c1);
                }
            }
        }
        break;
    }
    case T_MAT1F: {
        const C r0 = mats[4 * op.mat], r1 = mats[4 * op.mat + 1];
        switch (op.b1 & 7u) {
        case 0: mat1f_tile<C, DUAL, false, false, false>(s0, s1, op.b0, r0, r1, T); break;
        case 1: mat1f_tile<C, DUAL, true, false, false>(s0, s1, op.b0, r0, r1, T); break;
        case 2: mat1f_tile<C, DUAL, false, true, false>(s0, s1, op.b0, r0, r1, T); break;
        case 3: mat1f_tile<C, DUAL, true, true, false>(s0, s1, op.b0, r0, r1, T); break;
        case 4: mat1f_tile<C, DUAL, false, false, true>(s0, s1, op.b0, r0, r1, T); break;
        case 5: mat1f_tile<C, DUAL, true, false, true>(s0, s1, op.b0, r0, r1, T); break;
        case 6: mat1f_tile<C, DUAL, false, true, true>(s0, s1, op.b0, r0, r1, T); break;
        default: mat1f_tile<C, DUAL, true, true, true>(s0, s1, op.b0, r0, r1, T); break;
        }
        break;
    }
    case T_SCALE: {
        const C f = mats[4 * op.mat];
        for (uint32_t i = threadIdx.x; i < T; i += blockDim.x) {
            s0[i] = cmul(s0[i], f);
            if (DUAL) s1[i] = cmul(s1[i], f);
        }
        break;
    }
    case T_DIAG1: {
        const C d0 = mats[4 * op.mat], d1 = mats[4 * op.mat + 3];
        const uint32_t b = op.b0;
        for (uint32_t i = tid; i < T; i += bd) {
            const C f = ((i >> b) & 1u) ? d1 : d0;
            s0[i] = cmul(s0[i], f);
            if (DUAL) s1[i] = cmul(s1[i], f);
        }
        break;
    }
    case T_GPHASE: {
        const C f = ((base >> op.g0) & 1ULL) ? mats[4 * op.mat + 3] : mats[4 * op.mat];
        if (!is_one(f))
            for (uint32_t i = tid; i < T; i += bd) {
                s0[i] = cmul(s0[i], f);
                if (DUAL) s1[i] = cmul(s1[i], f);
            }
        break;
    }
    case T_CNOT_LL: {
        const uint32_t lo = min(op.b0, op.b1), hi = max(op.b0, op.b1);
        const uint32_t mc = 1u << op.b0, mt = 1u << op.b1;
        for (uint32_t p = tid; p < (T >> 2); p += bd) {
            const uint32_t i = insert00_32(p, lo, hi) | mc, j = i | mt;
            C t = s0[i]; s0[i] = s0[j]; s0[j] = t;
            if (DUAL) { t = s1[i]; s1[i] = s1[j]; s1[j] = t; }
        }
        break;
    }
    case T_CNOT_GL: {
        if ((base >> op.g0) & 1ULL) {
            const uint32_t b = op.b1, mb = 1u << b;
            for (uint32_t p = tid; p < (T >> 1); p += bd) {
                const uint32_t i = insert0_32(p, b), j = i | mb;
                C t = s0[i]; s0[i] = s0[j]; s0[j] = t;
                if (DUAL) { t = s1[i]; s1[i] = s1[j]; s1[j] = t; }
            }
        }
        break;
    }
    case T_CZ_LL: {
        const uint32_t lo = min(op.b0, op.b1), hi = max(op.b0, op.b1);
        const uint32_t both = (1u << op.b0) | (1u << op.b1);
        for (uint32_t p = tid; p < (T >> 2); p += bd) {
            const uint32_t i = insert00_32(p, lo, hi) | both;
            s0[i] = cneg(s0[i]);
            if (DUAL) s1[i] = cneg(s1[i]);
        }
        break;
    }
    case T_CZ_GL: {
        if ((base >> op.g0) & 1ULL) {
            const uint32_t b = op.b1, mb = 1u << b;
            for (uint32_t p = tid; p < (T >> 1); p += bd) {
                const uint32_t i = insert0_32(p, b) | mb;
                s0[i] = cneg(s0[i]);
                if (DUAL) s1[i] = cneg(s1[i]);
            }
        }
        break;
    }
    case T_CZ_GG: {
        if (((base >> op.g0) & 1ULL) && ((base >> op.g1) & 1ULL))
            for (uint32_t i = tid; i < T; i += bd) {
                s0[i] = cneg(s0[i]);
                if (DUAL) s1[i] = cneg(s1[i]);
            }
        break;
    }
    case T_SWAP_LL: {
        const uint32_t lo = min(op.b0, op.b1), hi = max(op.b0, op.b1);
        const uint32_t m0 = 1u << op.b0, m1 = 1u << op.b1;
        for (uint32_t p = tid; p < (T >> 2); p += bd) {
            const uint32_t b = insert00_32(p, lo, hi), i = b | m1, j = b | m0;
            C t = s0[i]; s0[i] = s0[j]; s0[j] = t;
            if (DUAL) { t = s1[i]; s1[i] = s1[j]; s1[j] = t; }
        }
        break;
    }
    default:
        break;
    }
}

// sum_i Im(conj(lambda_i) (P psi)_i) over the tile for the overlap op; this is
// 2 Re <lambda|(-i/2) P psi>, the adjoint contribution of src/lib.rs:3648-3664.
template <typename C>
__device__ __forceinline__ double tile_overlap(const TileOp &op, const C *ps, const C *la, uint64_t base,
                                               uint32_t T) {
    using R = typename Real<C>::T;
    const uint32_t tid = threadIdx.x, bd = blockDim.x;
    R sum = 0;
    if (op.kind == T_OVL_X || op.kind == T_OVL_Y) {
        const uint32_t b = op.b0, mb = 1u << b;
        const bool y = op.kind == T_OVL_Y;
        for (uint32_t p = tid; p < (T >> 1); p += bd) {
            const uint32_t i0 = insert0_32(p, b), i1 = i0 | mb;
            const C l0 = la[i0], l1 = la[i1], p0 = ps[i0], p1 = ps[i1];
            if (!y) sum += (l0.x * p1.y - l0.y * p1.x) + (l1.x * p0.y - l1.y * p0.x);
            else sum += -(l0.x * p1.x + l0.y * p1.y) + (l1.x * p0.x + l1.y * p0.y);
        }
    } else if (op.kind == T_OVL_ZL) {
        const uint32_t b = op.b0;
        for (uint32_t i = tid; i < T; i += bd) {
            const C l = la[i], p = ps[i];
            const R v = l.x * p.y - l.y * p.x;
            sum += ((i >> b) & 1u) ? -v : v;
        }
    } else {
        for (uint32_t i = tid; i < T; i += bd) {
            const C l = la[i], p = ps[i];
            sum += l.x * p.y - l.y * p.x;
        }
        if ((base >> op.g0) & 1ULL) sum = -sum;
    }
    return (double)sum;
}

template <typename C, bool DUAL>
__global__ void __launch_bounds__(kThreads)
    k_tile_pass(C *__restrict__ psi, C *__restrict__ lam, const PassArgs pa, const TileOp *__restrict__ g_ops,
                const double *__restrict__ g_mats, double *__restrict__ partials, uint32_t partial_stride) {
    using R = typename Real<C>::T;
    extern __shared__ __align__(16) unsigned char smem[];
    const TileSmem L = tile_smem(pa.k, pa.low, pa.n_ops, pa.n_mats, pa.n_slots, DUAL, sizeof(C));
    C *s0 = reinterpret_cast<C *>(smem + L.s0);
    C *s1 = reinterpret_cast<C *>(smem + L.s1);
    uint64_t *hi_off = reinterpret_cast<uint64_t *>(smem + L.hi);
    TileOp *ops = reinterpret_cast<TileOp *>(smem + L.ops);
    C *mats = reinterpret_cast<C *>(smem + L.mats);
    double *acc = reinterpret_cast<double *>(smem + L.acc);
    double *red = reinterpret_cast<double *>(smem + L.red);

    const uint32_t T = 1u << pa.k, nhi = pa.k - pa.low;
    for (uint32_t h = threadIdx.x; h < (1u << nhi); h += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t r = 0; r < nhi; ++r)
            if ((h >> r) & 1u) off |= 1ULL << pa.hi_q[r];
        hi_off[h] = off;
    }
    for (uint32_t o = threadIdx.x; o < pa.n_ops; o += blockDim.x) ops[o] = g_ops[o];
    for (uint32_t e = threadIdx.x; e < 4 * pa.n_mats; e += blockDim.x)
        mats[e] = mk((R)g_mats[2 * e], (R)g_mats[2 * e + 1]);
    if (DUAL)
        for (uint32_t s = threadIdx.x; s < pa.n_slots; s += blockDim.x) acc[s] = 0.0;
    __syncthreads();

    for (uint64_t t = blockIdx.x; t < pa.n_tiles; t += gridDim.x) {
        const uint64_t base = deposit(t, pa.nonlocal_mask);
        tile_load(s0, psi, base, hi_off, T, pa.low);
        if (DUAL) tile_load(s1, lam, base, hi_off, T, pa.low);
        __syncthreads();
        for (uint32_t o = 0; o < pa.n_ops; ++o) {
            const TileOp op = ops[o];
            if (op.kind >= T_OVL_X && op.kind <= T_OVL_ZG) {
                if (DUAL) {
                    const double v = block_sum(tile_overlap(op, s0, s1, base, T), red);
                    if (threadIdx.x == 0) acc[op.slot - (int32_t)pa.slot_base] += v;
                }
            } else {
                tile_apply<C, DUAL>(op, s0, s1, mats, base, T);
            }
            __syncthreads();
        }
        tile_store(s0, psi, base, hi_off, T, pa.low);
        if (DUAL) tile_store(s1, lam, base, hi_off, T, pa.low);
        __syncthreads();
    }
    if (DUAL)
        for (uint32_t s = threadIdx.x; s < pa.n_slots; s += blockDim.x)
            partials[(size_t)(pa.slot_base + s) * partial_stride + blockIdx.x] = acc[s];
}

// ---------------------------------------------------------------------------
// Dense-block passes (k-qubit fusion, any width up to 5): the shared-memory
// interpreter. A T_BLOCK op multiplies every group of 2^m amplitudes (the
// tile indices that differ only in the block's m local bits) by the block's
// 2^m x 2^m matrix. Thread (group, part) holds the group's inputs in
// registers and computes outputs part, part + S, ... into the other tile
// buffer; the buffers then swap, so no output overwrites an input another
// thread still reads. S (a power of two up to 2^m) spreads small group counts
// over the CTA. Lanes of a warp share `part` and so read the same matrix
// entries (broadcast loads).
// ---------------------------------------------------------------------------
template <typename C, int M>
__device__ __forceinline__ void block_apply(const C *__restrict__ in, C *__restrict__ out, const TileOp &op,
                                            const C *__restrict__ bm, uint32_t T) {
    using R = typename Real<C>::T;
    constexpr int D = 1 << M;
    uint32_t bit[M];
#pragma unroll
    for (int i = 0; i < M; ++i) bit[i] = (op.g0 >> (5 * i)) & 31u;
    uint32_t off[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
        uint32_t o = 0;
#pragma unroll
        for (int i = 0; i < M; ++i)
            if ((c >> i) & 1) o |= 1u << bit[i];
        off[c] = o;
    }
    const uint32_t groups = T >> M;
    uint32_t S = 1;
    while (S < (uint32_t)D && groups * (S << 1) <= blockDim.x) S <<= 1;
    const uint32_t items = groups * S;
    const C *mx = bm + op.mat;
    for (uint32_t it = threadIdx.x; it < items; it += blockDim.x) {
        const uint32_t g = it % groups, part = it / groups;
        uint32_t base = g;  // insert a zero at every block bit, lowest first
        uint32_t sorted[M];
#pragma unroll
        for (int i = 0; i < M; ++i) sorted[i] = bit[i];
#pragma unroll
        for (int i = 0; i < M; ++i)
#pragma unroll
            for (int j = 0; j + 1 < M - i; ++j)
                if (sorted[j] > sorted[j + 1]) {
                    const uint32_t t = sorted[j];
                    sorted[j] = sorted[j + 1];
                    sorted[j + 1] = t;
                }
#pragma unroll
        for (int i = 0; i < M; ++i) base = insert0_32(base, sorted[i]);
        C x[D];
#pragma unroll
        for (int c = 0; c < D; ++c) x[c] = in[base | off[c]];
        for (uint32_t r = part; r < (uint32_t)D; r += S) {
            R yr = 0, yi = 0;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const C m = mx[r * D + c];
                yr += m.x * x[c].x - m.y * x[c].y;
                yi += m.x * x[c].y + m.y * x[c].x;
            }
            out[base | off[r]] = mk(yr, yi);
        }
    }
}

template <typename C>
__global__ void __launch_bounds__(kThreads)
    k_block_pass(C *__restrict__ psi, const PassArgs pa, const TileOp *__restrict__ g_ops,
                 const double *__restrict__ g_mats, const C *__restrict__ g_bmats) {
    using R = typename Real<C>::T;
    extern __shared__ __align__(16) unsigned char smem[];
    // the dual layout gives the second tile buffer
    const TileSmem L = tile_smem(pa.k, pa.low, pa.n_ops, pa.n_mats, 0, true, sizeof(C));
    C *buf[2] = {reinterpret_cast<C *>(smem + L.s0), reinterpret_cast<C *>(smem + L.s1)};
    uint64_t *hi_off = reinterpret_cast<uint64_t *>(smem + L.hi);
    TileOp *ops = reinterpret_cast<TileOp *>(smem + L.ops);
    C *mats = reinterpret_cast<C *>(smem + L.mats);

    const uint32_t T = 1u << pa.k, nhi = pa.k - pa.low;
    for (uint32_t h = threadIdx.x; h < (1u << nhi); h += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t r = 0; r < nhi; ++r)
            if ((h >> r) & 1u) off |= 1ULL << pa.hi_q[r];
        hi_off[h] = off;
    }
    for (uint32_t o = threadIdx.x; o < pa.n_ops; o += blockDim.x) ops[o] = g_ops[o];
    for (uint32_t e = threadIdx.x; e < 4 * pa.n_mats; e += blockDim.x)
        mats[e] = mk((R)g_mats[2 * e], (R)g_mats[2 * e + 1]);
    __syncthreads();

    for (uint64_t t = blockIdx.x; t < pa.n_tiles; t += gridDim.x) {
        const uint64_t base = deposit(t, pa.nonlocal_mask);
        int cur = 0;
        tile_load(buf[0], psi, base, hi_off, T, pa.low);
        __syncthreads();
        for (uint32_t o = 0; o < pa.n_ops; ++o) {
            const TileOp op = ops[o];
            if (op.kind == T_BLOCK) {
                switch (op.b0) {
                case 2: block_apply<C, 2>(buf[cur], buf[cur ^ 1], op, g_bmats, T); break;
                case 3: block_apply<C, 3>(buf[cur], buf[cur ^ 1], op, g_bmats, T); break;
                case 4: block_apply<C, 4>(buf[cur], buf[cur ^ 1], op, g_bmats, T); break;
                default: block_apply<C, 5>(buf[cur], buf[cur ^ 1], op, g_bmats, T); break;
                }
                cur ^= 1;
            } else {
                tile_apply<C, false>(op, buf[cur], nullptr, mats, base, T);
            }
            __syncthreads();
        }
        tile_store(buf[cur], psi, base, hi_off, T, pa.low);
        __syncthreads();
    }
}

template <typename C> static int launch_block_passes(qf_sv *sv, const Plan &plan) {
    qf_ctx *ctx = sv->ctx;
    static size_t dyn[64] = {0};
    const int dev = ctx->device & 63;
    if (!dyn[dev]) QF_TRY(allow_max_dynamic_smem(k_block_pass<C>, ctx, &dyn[dev]));
    // upload ops, 2x2 matrices (f64) and block matrices (in the state's precision)
    const size_t ops_bytes = align_up((uint32_t)(plan.ops.size() * sizeof(TileOp)), 16);
    const size_t mats_bytes = align_up((uint32_t)(plan.mats.size() * sizeof(double)), 16);
    const size_t n_bm = plan.bmats.size() / 2;
    std::vector<C> bm(n_bm);
    for (size_t i = 0; i < n_bm; ++i) bm[i] = to_c<C>(&plan.bmats[2 * i]);
    const size_t bm_bytes = n_bm * sizeof(C);
    QF_TRY(ensure_device(&ctx->ws_plan, &ctx->ws_plan_bytes, ops_bytes + mats_bytes + bm_bytes + 16));
    unsigned char *d_plan = static_cast<unsigned char *>(ctx->ws_plan);
    if (!plan.ops.empty())
        QF_CUDA(cudaMemcpyAsync(d_plan, plan.ops.data(), plan.ops.size() * sizeof(TileOp), cudaMemcpyHostToDevice,
                                ctx->stream));
    if (!plan.mats.empty())
        QF_CUDA(cudaMemcpyAsync(d_plan + ops_bytes, plan.mats.data(), plan.mats.size() * sizeof(double),
                                cudaMemcpyHostToDevice, ctx->stream));
    if (bm_bytes)
        QF_CUDA(cudaMemcpyAsync(d_plan + ops_bytes + mats_bytes, bm.data(), bm_bytes, cudaMemcpyHostToDevice, ctx->stream));
    const TileOp *d_ops = reinterpret_cast<const TileOp *>(d_plan);
    const double *d_mats = reinterpret_cast<const double *>(d_plan + ops_bytes);
    const C *d_bm = reinterpret_cast<const C *>(d_plan + ops_bytes + mats_bytes);
    uint32_t max_smem = 0;
    for (const Pass &p : plan.passes)
        max_smem = std::max(max_smem, tile_smem(p.a.k, p.a.low, p.a.n_ops, p.a.n_mats, 0, true, sizeof(C)).total);
    if (max_smem > dyn[dev])
        return fail(QF_ERR_UNSUPPORTED_OPERATION, "block pass needs %u bytes of shared memory (limit %zu)", max_smem,
                    dyn[dev]);
    int per_sm = 0;
    QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_block_pass<C>, kThreads, max_smem));
    const uint32_t grid = (uint32_t)std::max(per_sm, 1) * (uint32_t)ctx->sm_count;
    for (const Pass &p : plan.passes) {
        const TileSmem L = tile_smem(p.a.k, p.a.low, p.a.n_ops, p.a.n_mats, 0, true, sizeof(C));
        const uint32_t g = (uint32_t)std::min<uint64_t>(grid, p.a.n_tiles);
        k_block_pass<C><<<g, kThreads, L.total, ctx->stream>>>(static_cast<C *>(sv->d), p.a, d_ops + p.op_begin,
                                                               d_mats + 8 * (size_t)p.mat_begin, d_bm);
        QF_CUDA(cudaGetLastError());
    }
    return QF_OK;
}

int run_plan_blocks(qf_sv *sv, const Plan &plan) {
    if (plan.passes.empty()) return QF_OK;
    if (sv->dtype == QF_C64) return launch_block_passes<float2>(sv, plan);
    return launch_block_passes<double2>(sv, plan);
}

// slot_sums[s] += sum over blocks of partials[s * stride + b]: one warp per
// slot, lane l adding blocks l, l + 32, ... in order, then the warp's tree (the
// same order on every run). Launch with 256-thread blocks, 8 slots per block.
__global__ void k_reduce_slots(const double *__restrict__ partials, uint32_t stride, uint32_t n_slots,
                               double *__restrict__ slot_sums) {
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < n_slots; s += (gridDim.x * blockDim.x) >> 5) {
        double v = 0.0;
        for (uint32_t b = lane; b < stride; b += 32) v += partials[(size_t)s * stride + b];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) slot_sums[s] += v;
    }
}

template <typename C, bool DUAL> static int set_smem_attr(const qf_ctx *ctx, size_t *limit) {
    static size_t dyn[64] = {0};
    const int dev = ctx->device & 63;
    if (!dyn[dev]) QF_TRY(allow_max_dynamic_smem(k_tile_pass<C, DUAL>, ctx, &dyn[dev]));
    *limit = dyn[dev];
    return QF_OK;
}

template <typename C, bool DUAL>
static int launch_passes(qf_sv *psi, qf_sv *lam, const Plan &plan, double *d_slot_sums) {
    qf_ctx *ctx = psi->ctx;
    size_t smem_limit = 0;
    QF_TRY((set_smem_attr<C, DUAL>(ctx, &smem_limit)));
    // upload ops then matrices
    const size_t ops_bytes = align_up((uint32_t)(plan.ops.size() * sizeof(TileOp)), 16);
    const size_t mats_bytes = plan.mats.size() * sizeof(double);
    QF_TRY(ensure_device(&ctx->ws_plan, &ctx->ws_plan_bytes, ops_bytes + mats_bytes + 16));
    unsigned char *d_plan = static_cast<unsigned char *>(ctx->ws_plan);
    if (!plan.ops.empty())
        QF_CUDA(cudaMemcpyAsync(d_plan, plan.ops.data(), plan.ops.size() * sizeof(TileOp), cudaMemcpyHostToDevice,
                                ctx->stream));
    if (!plan.mats.empty())
        QF_CUDA(cudaMemcpyAsync(d_plan + ops_bytes, plan.mats.data(), mats_bytes, cudaMemcpyHostToDevice, ctx->stream));
    const TileOp *d_ops = reinterpret_cast<const TileOp *>(d_plan);
    const double *d_mats = reinterpret_cast<const double *>(d_plan + ops_bytes);

    // persistent grid: a fixed number of CTAs for every pass of the plan
    uint32_t max_smem = 0;
    for (const Pass &p : plan.passes) {
        const TileSmem L = tile_smem(p.a.k, p.a.low, p.a.n_ops, p.a.n_mats, p.a.n_slots, DUAL, sizeof(C));
        max_smem = std::max(max_smem, L.total);
    }
    if (max_smem > smem_limit)
        return fail(QF_ERR_UNSUPPORTED_OPERATION, "tile pass needs %u bytes of shared memory (limit %zu)", max_smem,
                    smem_limit);
    int per_sm = 0;
    QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_pass<C, DUAL>, kThreads, max_smem));
    per_sm = std::max(per_sm, 1);
    const uint32_t grid = (uint32_t)per_sm * (uint32_t)ctx->sm_count;

    double *d_partials = nullptr;
    if (DUAL && plan.n_slots) {
        QF_TRY(ensure_device(&ctx->ws_red, &ctx->ws_red_bytes, sizeof(double) * (size_t)plan.n_slots * grid));
        d_partials = static_cast<double *>(ctx->ws_red);
    }
    for (const Pass &p : plan.passes) {
        const TileSmem L = tile_smem(p.a.k, p.a.low, p.a.n_ops, p.a.n_mats, p.a.n_slots, DUAL, sizeof(C));
        const uint32_t g = DUAL ? grid : (uint32_t)std::min<uint64_t>(grid, p.a.n_tiles);
        k_tile_pass<C, DUAL><<<g, kThreads, L.total, ctx->stream>>>(
            static_cast<C *>(psi->d), lam ? static_cast<C *>(lam->d) : nullptr, p.a, d_ops + p.op_begin,
            d_mats + 8 * (size_t)p.mat_begin, d_partials, grid);
        QF_CUDA(cudaGetLastError());
    }
    if (DUAL && plan.n_slots) {
        k_reduce_slots<<<(plan.n_slots + 7) / 8, 256, 0, ctx->stream>>>(d_partials, grid, plan.n_slots, d_slot_sums);
        QF_CUDA(cudaGetLastError());
    }
    return QF_OK;
}

int run_plan_smem(qf_sv *sv, const Plan &plan) {
    if (plan.passes.empty()) return QF_OK;
    if (sv->dtype == QF_C64) return launch_passes<float2, false>(sv, nullptr, plan, nullptr);
    return launch_passes<double2, false>(sv, nullptr, plan, nullptr);
}

// complex64 plans with 12- or 13-qubit tiles run register-tiled; the rest
// (complex128, small states, QF_EXEC_FLAG_SMEM_TILES) in shared memory.
int run_plan(qf_sv *sv, const Plan &plan, int flags) {
    if (plan.passes.empty()) return QF_OK;
    if (plan.block_qubits) {  // dense k-qubit blocks
        if (sv->dtype == QF_C64 && !(flags & QF_EXEC_FLAG_SMEM_TILES)) {
            if (plan.block_qubits == 5 && !(flags & QF_EXEC_FLAG_BLOCKS_SIMT) && mma_blocks_fit(plan))
                return run_plan_blocks_mma(sv, plan);
            if (plan.block_qubits <= 4 && sv->n >= 12 && plan.passes[0].a.k == 12 && !(flags & QF_EXEC_FLAG_NO_JIT) &&
                ((flags & QF_EXEC_FLAG_JIT) || sv->n >= kJitMinQubits) && jit_available())
                return run_plan_jit(sv, plan, 3);
        }
        return run_plan_blocks(sv, plan);
    }
    if (sv->dtype == QF_C64 && !(flags & QF_EXEC_FLAG_SMEM_TILES) && sv->n >= 12) {
        const uint32_t k = plan.passes[0].a.k;
        // compiled passes for large states (the compile is amortised over many
        // sweeps of the state), interpreted register tiles otherwise
        const bool jit = (k == 12 || k == 13) && !(flags & QF_EXEC_FLAG_NO_JIT) &&
                         ((flags & QF_EXEC_FLAG_JIT) || sv->n >= kJitMinQubits) && jit_available();
        if (jit) return run_plan_jit(sv, plan, 3);
        if (k == 12 || k == 13) return run_plan_rs(sv, plan, (int)k - 9);
    }
    return run_plan_smem(sv, plan);
}

int run_plan_dual_smem(qf_sv *psi, qf_sv *lambda, const Plan &plan, double *d_slot_sums) {
    if (psi->dtype == QF_C64) return launch_passes<float2, true>(psi, lambda, plan, d_slot_sums);
    return launch_passes<double2, true>(psi, lambda, plan, d_slot_sums);
}

int run_plan_dual(qf_sv *psi, qf_sv *lambda, const Plan &plan, double *d_slot_sums, int flags) {
    if (plan.passes.empty()) return QF_OK;
    if (psi->dtype != lambda->dtype || psi->n != lambda->n)
        return fail(QF_ERR_INCOMPATIBLE_DEVICE_STATE, "device states must have equal dimensions and dtype");
    if (psi->dtype == QF_C64 && !(flags & QF_EXEC_FLAG_SMEM_TILES) && !(flags & QF_EXEC_FLAG_NO_JIT) &&
        ((flags & QF_EXEC_FLAG_JIT) || psi->n >= kJitMinQubits) && jit_available())
        return run_plan_jit_dual(psi, lambda, plan, d_slot_sums);
    return run_plan_dual_smem(psi, lambda, plan, d_slot_sums);
}

int reduce_slots(qf_ctx *ctx, const double *partials, uint32_t stride, uint32_t n_slots, double *d_slot_sums) {
    if (!n_slots) return QF_OK;
    k_reduce_slots<<<(n_slots + 7) / 8, 256, 0, ctx->stream>>>(partials, stride, n_slots, d_slot_sums);
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

// Bound gate list on a resident state: unfused sweeps or tile passes.
int execute_gates(qf_sv *sv, const std::vector<BGate> &gates, const qf_exec_opts *opts) {
    const int mode = opts ? opts->mode : QF_EXEC_AUTO;
    if (mode == QF_EXEC_UNFUSED) {
        for (const BGate &g : gates) {
            if (g.kind == BK_MAT1) QF_TRY(launch_gate1(sv, g));
            else QF_TRY(launch_gate2(sv, g));
        }
        return QF_OK;
    }
    if (mode != QF_EXEC_AUTO && mode != QF_EXEC_FUSED)
        return fail(QF_ERR_INVALID_ARGUMENT, "unknown execution mode %d", mode);
    PlanOpts po;
    QF_TRY(plan_opts_for(sv->n, sv->dtype, opts, po));
    Plan plan;
    QF_TRY(plan_passes(sv->n, gates, po, plan));
    return run_plan(sv, plan, opts ? opts->flags : 0);
}

// Forward-sweep planning options from a caller's qf_exec_opts.
int plan_opts_for(uint32_t n, int dtype, const qf_exec_opts *opts, PlanOpts &po) {
    forward_tiling(n, dtype, opts ? opts->tile_qubits : 0, opts ? opts->flags : 0, &po.tile_qubits, &po.low_qubits);
    po.search = !(opts && (opts->flags & QF_EXEC_FLAG_PLAN_FIRST_COME));
    const int kb = opts ? opts->block_qubits : 0;
    if (kb < 0 || kb > kMaxBlockQubits)
        return fail(QF_ERR_INVALID_ARGUMENT, "block_qubits must be 0..%d, got %d", kMaxBlockQubits, kb);
    po.block_qubits = kb >= 2 ? std::min<int>(kb, (int)n) : 0;
    if (po.block_qubits < 2) po.block_qubits = 0;
    return QF_OK;
}

}  // namespace qf
