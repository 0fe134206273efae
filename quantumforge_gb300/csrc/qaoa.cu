// qaoa.cu — batched QAOA MaxCut: cost and adjoint gradient for many
// instances of uneven qubit counts in one persistent launch.
//
// The circuit is algorithms::qaoa_maxcut (src/algorithms.rs:110-137): H on
// every qubit, then per layer CNOT(u,v)·Rz(2γw)·CNOT(u,v) for every edge and
// Rx(2β) on every qubit; the cost is maxcut_expectation
// (src/qaoa_transfer.rs:199-218). The edge gadgets multiply basis state x by
// exp(-iγ Σ_e w_e (1 - 2[x_u != x_v])) = exp(-iγ (W - 2 C(x))), so a cost
// layer is one phase per amplitude read from a table indexed by the cut value
// C(x) (unit weights) or computed from it. The mixer is exp(-iβ X) on every
// qubit.
//
// Each CTA takes instances from an atomic counter (no waiting on other CTAs)
// and runs the whole forward sweep, the costate λ = C ψ and the reverse sweep
// for its instance, with ψ, λ and a uint8 table of C(x) in a per-instance
// arena (L2/HBM). Gates run in shared-memory tiles of 2^k amplitudes (k per
// instance, autotuned per qubit count); inside a tile, mixer gates are applied
// four qubits at a time with 16 amplitudes per thread in registers. The
// gradient dE/dβ_l = 2 Im<λ|Σ_q X_q|ψ> and dE/dγ_l = 2 Im<λ|(W - 2C)|ψ> is
// accumulated in f64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "qf_device.cuh"
#include "qf_internal.h"

namespace qf {
namespace {

constexpr int kQThreads = 256;
constexpr int kQMaxTile = 12;  // 4096 amplitudes per tile (16 per thread)
constexpr int kQMaxP = 16;
constexpr int kQMaxEdges = 96;

struct QDesc {
    uint64_t psi;       // float2 offset of psi in the arena
    uint64_t lam;       // float2 offset of lambda
    uint64_t cost;      // byte offset of the C(x) table in the cost arena
    uint64_t ptab;      // batched instances: float2 offset of the per-layer phase tables
    uint64_t part;      // batched instances: double offset of the per-tile partial sums
    uint32_t n;
    uint32_t k;         // tile qubits
    uint32_t e_begin;
    uint32_t e_count;
    uint32_t out;       // output row (caller order)
    uint32_t pad;
};

struct QShared {
    float2 tp[1 << kQMaxTile];
    float2 tl[1 << kQMaxTile];
    float2 phase[kQMaxEdges + 1];  // exp(-iγ(W - 2c)) for the current layer
    uint32_t emask[kQMaxEdges];
    double red[32];
    double acc[2 * kQMaxP];
    double energy;
    uint32_t inst;
};

// Edge masks hold both endpoints as bits; instances have at most 24 qubits.
__device__ __forceinline__ uint32_t cut_value(uint32_t x, const uint32_t *emask, uint32_t ne) {
    uint32_t c = 0;
    for (uint32_t e = 0; e < ne; ++e) c += __popc(x & emask[e]) & 1u;
    return c;
}

// bit b < 4 of k = 4q + r as bytes r = 0..3 of a word (0 or 1 each)
__device__ __forceinline__ uint32_t cut_bit_bytes(uint32_t b, uint32_t q) {
    return b == 0 ? 0x01000100u : b == 1 ? 0x01010000u : ((q >> (b - 2)) & 1u) ? 0x01010101u : 0u;
}

// C(base | k) for k = 0..15, byte k & 3 of word k >> 2 (base has bits 0..3
// clear). An edge above bit 3 adds the constant parity of base; an edge from
// bit b < 4 to a bit w above adds bit b of k, or 1 minus it where bit w of
// base is set; an edge inside bits 0..3 adds a fixed byte pattern. Per k the
// sum is c + the D_b of the bits b set in k (D_b = edges at b with bit w clear
// minus those with it set), plus the pattern: one pass over the edges per 16
// amplitudes.
__device__ __forceinline__ uint4 cut16(uint32_t base, const uint32_t *emask, uint32_t ne) {
    uint32_t c = 0, dp = 0, dm = 0;
    uint32_t t2[4] = {0u, 0u, 0u, 0u};
    for (uint32_t e = 0; e < ne; ++e) {
        const uint32_t m = emask[e], lo = m & 15u;
        if (lo == 0) {
            c += __popc(base & m) & 1u;
        } else if (lo != m) {
            const uint32_t f = 1u << (8 * (__ffs(lo) - 1));
            if (base & m) {
                ++c;
                dm += f;
            } else {
                dp += f;
            }
        } else {
            const uint32_t u = __ffs(m) - 1, v = 31 - __clz(m);
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) t2[q] += cut_bit_bytes(u, q) ^ cut_bit_bytes(v, q);
        }
    }
    int d[4];
#pragma unroll
    for (uint32_t b = 0; b < 4; ++b) d[b] = (int)((dp >> (8 * b)) & 0xFFu) - (int)((dm >> (8 * b)) & 0xFFu);
    uint32_t w[4];
#pragma unroll
    for (uint32_t q = 0; q < 4; ++q) {
        const int h = (int)c + ((q & 1u) ? d[2] : 0) + ((q & 2u) ? d[3] : 0);
        w[q] = t2[q] + ((uint32_t)h | ((uint32_t)(h + d[0]) << 8) | ((uint32_t)(h + d[1]) << 16) |
                        ((uint32_t)(h + d[0] + d[1]) << 24));
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// Local tile index j <-> amplitude index for a tile whose qubits are the low
// `lo` qubits plus `hi` = high qubit list; tile t enumerates the rest.
struct TileMap {
    uint32_t k, lo;
    uint8_t hiq[kQMaxTile];
    uint64_t rest_mask;
};
__device__ __forceinline__ uint64_t tile_index(const TileMap &m, uint64_t base, uint32_t j) {
    uint64_t x = base | (j & ((1u << m.lo) - 1));
    const uint32_t h = j >> m.lo;
    for (uint32_t r = 0; r < m.k - m.lo; ++r)
        if ((h >> r) & 1u) x |= 1ULL << m.hiq[r];
    return x;
}

// exp(-iβX) on local bits b0..b0+nb-1 (nb <= 4) of the tile(s), 16 amplitudes
// per thread in registers. dual: both tiles; grad: accumulate 2 Im<λ|X_q|ψ>
// (before the gate) into *g.
template <bool DUAL, int NB>
__device__ void mixer_round_nb(float2 *tp, float2 *tl, uint32_t k, uint32_t b0, float c, float s, double *g) {
    const uint32_t T = 1u << k;
    const uint32_t groups = T >> NB;
    constexpr uint32_t cnt = 1u << NB;
    float gsum = 0.f;
    for (uint32_t grp = threadIdx.x; grp < groups; grp += blockDim.x) {
        // base: grp's bits spread around the NB bits at b0
        const uint32_t low = grp & ((1u << b0) - 1), high = grp >> b0;
        const uint32_t base = low | (high << (b0 + NB));
        float2 a[cnt], l[cnt];
#pragma unroll
        for (uint32_t i = 0; i < cnt; ++i) {
            a[i] = tp[base | (i << b0)];
            if (DUAL) l[i] = tl[base | (i << b0)];
        }
#pragma unroll
        for (uint32_t b = 0; b < (uint32_t)NB; ++b) {
#pragma unroll
            for (uint32_t i = 0; i < cnt; ++i) {
                if (i & (1u << b)) continue;
                const uint32_t j = i | (1u << b);
                if (DUAL) {  // Im(conj(l_i) a_j) + Im(conj(l_j) a_i) before the gate
                    gsum += (l[i].x * a[j].y - l[i].y * a[j].x) + (l[j].x * a[i].y - l[j].y * a[i].x);
                }
                // [c, -is; -is, c] (s = sin(angle/2) with the sign of the angle)
                const float2 x = a[i], y = a[j];
                a[i] = make_float2(c * x.x + s * y.y, c * x.y - s * y.x);
                a[j] = make_float2(c * y.x + s * x.y, c * y.y - s * x.x);
                if (DUAL) {
                    const float2 u = l[i], v = l[j];
                    l[i] = make_float2(c * u.x + s * v.y, c * u.y - s * v.x);
                    l[j] = make_float2(c * v.x + s * u.y, c * v.y - s * u.x);
                }
            }
        }
#pragma unroll
        for (uint32_t i = 0; i < cnt; ++i) {
            tp[base | (i << b0)] = a[i];
            if (DUAL) tl[base | (i << b0)] = l[i];
        }
    }
    if (DUAL && g) *g += (double)gsum;
}

template <bool DUAL>
__device__ void mixer_round(float2 *tp, float2 *tl, uint32_t k, uint32_t b0, uint32_t nb, float c, float s, double *g) {
    switch (nb) {
    case 1: mixer_round_nb<DUAL, 1>(tp, tl, k, b0, c, s, g); break;
    case 2: mixer_round_nb<DUAL, 2>(tp, tl, k, b0, c, s, g); break;
    case 3: mixer_round_nb<DUAL, 3>(tp, tl, k, b0, c, s, g); break;
    default: mixer_round_nb<DUAL, 4>(tp, tl, k, b0, c, s, g); break;
    }
}

__device__ __forceinline__ float2 cm(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmc(float2 a, float2 b) {  // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// one tile pass over an instance: load, [cost phase], mixer rounds on local
// bits [g0, g1), [gradients], store
template <bool DUAL>
__device__ void instance_pass(QShared &S, float2 *psi, float2 *lam, const uint8_t *cost, const TileMap &m, uint32_t n,
                              uint32_t g0, uint32_t g1, float c, float s, int cost_mode, float W, double *gb, double *gg) {
    const uint32_t T = 1u << m.k;
    const uint64_t ntiles = 1ULL << (n - m.k);
    double gcost = 0.0;
    for (uint64_t t = 0; t < ntiles; ++t) {
        const uint64_t base = deposit(t, m.rest_mask);
        for (uint32_t j = threadIdx.x; j < T; j += blockDim.x) {
            const uint64_t x = tile_index(m, base, j);
            float2 a = psi[x];
            float2 l = DUAL ? lam[x] : make_float2(0.f, 0.f);
            if (cost_mode == 1) {  // forward: multiply by the layer phase
                a = cm(a, S.phase[cost[x]]);
            }
            S.tp[j] = a;
            if (DUAL) S.tl[j] = l;
        }
        __syncthreads();
        double gb_local = 0.0;
        for (uint32_t b = g0; b < g1; b += 4) {
            mixer_round<DUAL>(S.tp, S.tl, m.k, b, min(4u, g1 - b), c, s, &gb_local);
            __syncthreads();
        }
        if (DUAL) *gb += gb_local;
        for (uint32_t j = threadIdx.x; j < T; j += blockDim.x) {
            const uint64_t x = tile_index(m, base, j);
            float2 a = S.tp[j];
            float2 l = DUAL ? S.tl[j] : make_float2(0.f, 0.f);
            if (cost_mode == 2) {  // reverse: gradient of the cost layer, then undo its phase
                const float gx = W - 2.f * (float)cost[x];
                gcost += (double)(gx * (l.x * a.y - l.y * a.x));
                a = cmc(a, S.phase[cost[x]]);
                l = cmc(l, S.phase[cost[x]]);
            }
            psi[x] = a;
            if (DUAL) lam[x] = l;
        }
        __syncthreads();
    }
    if (gg) *gg += gcost;
}

__device__ double block_total(double v, double *red) {
    v = block_sum(v, red);
    __syncthreads();
    return v;
}

__global__ void __launch_bounds__(kQThreads)
    k_qaoa_batch(const QDesc *__restrict__ desc, uint32_t n_inst, float2 *__restrict__ arena, uint8_t *__restrict__ costs,
                 const uint64_t *__restrict__ emasks, const double *__restrict__ gammas, const double *__restrict__ betas,
                 uint32_t p, double *__restrict__ out_cost, double *__restrict__ out_grad, unsigned *__restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    QShared &S = *reinterpret_cast<QShared *>(smem_raw);
    for (;;) {
        if (threadIdx.x == 0) S.inst = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t id = S.inst;
        __syncthreads();
        if (id >= n_inst) break;
        const QDesc D = desc[id];
        const uint32_t n = D.n, ne = D.e_count;
        float2 *psi = arena + D.psi, *lam = arena + D.lam;
        uint8_t *cost = costs + D.cost;
        for (uint32_t e = threadIdx.x; e < ne; e += blockDim.x) S.emask[e] = (uint32_t)emasks[D.e_begin + e];
        if (threadIdx.x < 2 * kQMaxP) S.acc[threadIdx.x] = 0.0;
        __syncthreads();
        const uint64_t dim = 1ULL << n;
        const float amp0 = (float)(1.0 / sqrt((double)dim));
        for (uint32_t x = threadIdx.x; x < (uint32_t)dim; x += blockDim.x) {  // H on every qubit of |0>; C(x)
            psi[x] = make_float2(amp0, 0.f);
            cost[x] = (uint8_t)cut_value(x, S.emask, ne);
        }
        __syncthreads();
        // tile maps: A = low k qubits (mixer on all of them); B = 3 low + the rest
        TileMap A, B;
        const uint32_t k = min(D.k, n);
        A.k = k;
        A.lo = k;
        A.rest_mask = (dim - 1) & ~((1ULL << k) - 1);
        const uint32_t rest = n - k;  // qubits k..n-1 for pass B
        const uint32_t blo = min(k - rest, 3u);
        B.k = blo + rest;
        B.lo = blo;
        for (uint32_t r = 0; r < rest; ++r) B.hiq[r] = (uint8_t)(k + r);
        B.rest_mask = (dim - 1) & ~(((1ULL << blo) - 1) | (((1ULL << rest) - 1) << k));
        const float W = (float)ne;
        // forward
        for (uint32_t l = 0; l < p; ++l) {
            const double gm = gammas[(size_t)D.out * p + l], bt = betas[(size_t)D.out * p + l];
            for (uint32_t c = threadIdx.x; c <= ne; c += blockDim.x) {
                const double ang = -gm * ((double)ne - 2.0 * (double)c);
                S.phase[c] = make_float2((float)cos(ang), (float)sin(ang));
            }
            __syncthreads();
            const float cc = (float)cos(bt), ss = (float)sin(bt);  // Rx(2β): cos β, sin β
            instance_pass<false>(S, psi, lam, cost, A, n, 0, k, cc, ss, 1, W, nullptr, nullptr);
            if (rest) instance_pass<false>(S, psi, lam, cost, B, n, blo, blo + rest, cc, ss, 0, W, nullptr, nullptr);
        }
        // energy and lambda = C psi
        double e_loc = 0.0;
        for (uint64_t x = threadIdx.x; x < dim; x += blockDim.x) {
            const float2 a = psi[x];
            const float cv = (float)cost[x];
            e_loc += (double)(cv * (a.x * a.x + a.y * a.y));
            lam[x] = make_float2(cv * a.x, cv * a.y);
        }
        const double energy = block_total(e_loc, S.red);
        __syncthreads();
        // reverse
        for (uint32_t l = p; l-- > 0;) {
            const double gm = gammas[(size_t)D.out * p + l], bt = betas[(size_t)D.out * p + l];
            for (uint32_t c = threadIdx.x; c <= ne; c += blockDim.x) {
                const double ang = -gm * ((double)ne - 2.0 * (double)c);
                S.phase[c] = make_float2((float)cos(ang), (float)sin(ang));
            }
            __syncthreads();
            const float cc = (float)cos(-bt), ss = (float)sin(-bt);  // inverse mixer
            double gb = 0.0, gg = 0.0;
            if (rest) instance_pass<true>(S, psi, lam, cost, B, n, blo, blo + rest, cc, ss, 0, W, &gb, nullptr);
            instance_pass<true>(S, psi, lam, cost, A, n, 0, k, cc, ss, 2, W, &gb, &gg);
            gb = block_total(gb, S.red);
            gg = block_total(gg, S.red);
            if (threadIdx.x == 0) {
                S.acc[l] = 2.0 * gg;      // dE/dγ_l
                S.acc[p + l] = 2.0 * gb;  // dE/dβ_l
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) out_cost[D.out] = energy;
        if (threadIdx.x < 2 * p) out_grad[(size_t)D.out * 2 * p + threadIdx.x] = S.acc[threadIdx.x];
        __syncthreads();
    }
}

// ---- batched passes for instances of 13..24 qubits ---------------------------
// All instances of one qubit count n are advanced together, one tile pass per
// launch over every (instance, tile) pair, so a pass streams at the rate of the
// whole GPU. Tiles hold 2^12 amplitudes: pass A the low 12 qubits (contiguous;
// cost phase and mixer on qubits 0..11), pass B the high n-12 qubits plus the
// low L = 24-n (mixer on qubits 12..n-1). A forward layer is A then B; the last
// B also writes lambda = C psi and the energy. A reverse layer undoes B then A
// on psi and lambda, with the dE/dbeta terms of both and the dE/dgamma term
// (after the mixer is undone) written per (instance, tile) and summed in tile
// order by k_qaoa_reduce.
constexpr int kQBTile = 12;
constexpr uint32_t kQBT = 1u << kQBTile;

struct QBArgs {
    uint32_t r0, m;  // descriptor rows [r0, r0 + m): one qubit count
    uint32_t n, L;   // qubits; low bits of a pass-B tile (24 - n)
    uint32_t p, layer;
    uint64_t tiles;  // tiles per instance: 2^(n-12)
    uint64_t chunk;  // items (instance, tile) per CTA, consecutive: CTA b takes [b chunk, (b + 1) chunk)
};

// part slots per tile: 0 energy, 1+l dE/dbeta (pass A), 1+p+l dE/dbeta
// (pass B), 1+2p+l dE/dgamma
__device__ __forceinline__ uint64_t qb_index(bool pass_b, uint32_t L, uint64_t t, uint32_t j) {
    if (!pass_b) return (t << kQBTile) | j;
    return (uint64_t)(j & ((1u << L) - 1)) | (t << L) | ((uint64_t)(j >> L) << kQBTile);
}

__device__ __forceinline__ void qb_cp16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
// Shared-memory position of tile amplitude j: bits 1..3 XOR bits 4..6, so
// that the mixer round on tile bits 0..3 (16-byte pair accesses, 8 lanes per
// phase) and the rounds on higher bits (8-byte accesses, 16 lanes per phase)
// are bank-conflict free; bit 0 is kept, so 16-byte pairs stay whole.
__device__ __forceinline__ uint32_t qb_phys(uint32_t j) { return j ^ (((j >> 4) & 7u) << 1); }
// a tile of 2^12 amplitudes into shared memory: 16-byte copies of amplitude
// pairs (pass B with L = 0 has no adjacent pair: plain loads)
__device__ __forceinline__ void qb_load(float2 *dst, const float2 *src, bool pass_b, uint32_t L, uint64_t t) {
    if (pass_b && L == 0) {
        for (uint32_t j = threadIdx.x; j < kQBT; j += blockDim.x) dst[qb_phys(j)] = src[qb_index(true, 0, t, j)];
        return;
    }
    for (uint32_t c = threadIdx.x; c < kQBT / 2; c += blockDim.x)
        qb_cp16(dst + qb_phys(2 * c), src + qb_index(pass_b, L, t, 2 * c));
}
// the cost bytes of a pass-A tile (contiguous)
__device__ __forceinline__ void qb_load_cost(uint8_t *dst, const uint8_t *src, uint64_t t) {
    for (uint32_t c = threadIdx.x; c < kQBT / 16; c += blockDim.x) qb_cp16(dst + 16 * c, src + (t << kQBTile) + 16 * c);
}

// C(x) for every amplitude of every instance of the class; per-layer phases
// exp(-i gamma (W - 2c)) and mixer (cos beta, sin beta) as the per-instance
// kernel computes them
__global__ void __launch_bounds__(kQThreads)
    k_qaoa_costs(const QBArgs a, const QDesc *__restrict__ desc, const uint64_t *__restrict__ emasks, uint8_t *__restrict__ costs) {
    __shared__ uint32_t em[kQMaxEdges];
    const uint64_t items = (uint64_t)a.m * a.tiles;
    for (uint64_t w = blockIdx.x; w < items; w += gridDim.x) {
        const uint32_t ci = (uint32_t)(w >> (a.n - kQBTile));
        const uint64_t t = (w & (a.tiles - 1));
        const QDesc D = desc[a.r0 + ci];
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < D.e_count; e += blockDim.x) em[e] = (uint32_t)emasks[D.e_begin + e];
        __syncthreads();
        uint8_t *cost = costs + D.cost + (t << kQBTile);  // 16-byte aligned: batched rows come first, 2^n >= 2^13 each
        for (uint32_t g = threadIdx.x; g < kQBT / 16; g += blockDim.x)
            *reinterpret_cast<uint4 *>(cost + 16 * g) = cut16((uint32_t)(t << kQBTile) | (g << 4), em, D.e_count);
    }
}

// Per (instance, layer) mixer constants of the batched passes. Each gate
// exp(-i beta X) is applied divided by a real factor F, which leaves four FMAs
// per amplitude pair: form C (|cos beta| >= |sin beta|) divides by cos beta
// (k = tan beta), form S by sin beta (k = cot beta); the inverse gate has -k
// and F' = cos beta or -sin beta. The factors a state picks up in a layer
// (F^n, or F'^n in reverse) are multiplied back where a pass already touches
// every amplitude (the next layer's cost phase, the last forward write, the
// inverse cost phase) and into the gradient sums as scalars.
struct QMix {
    float kf, kr;   // forward / inverse gate constant
    float f2;       // F^2
    float fn_f;     // F^n
    float fn_r;     // F'^n
    float f2_a0;    // F^(2(n-12)): a reverse pass A starts after the n-12 gates of pass B
    uint32_t form_c;
    uint32_t pad;
};

// Phase tables per (instance, layer): forward exp(-i gamma_l (W - 2c)) times
// the factor its input carries (2^(-n/2) in layer 0, F_{l-1}^n after), at
// ptab + l * span; the reverse table, times F'_l^n, at ptab + (p + l) * span.
__global__ void k_qaoa_tables(const QDesc *__restrict__ desc, uint32_t rows, const double *__restrict__ gammas,
                              const double *__restrict__ betas, uint32_t p, float2 *__restrict__ ptab, QMix *__restrict__ mtab) {
    const uint32_t span = kQMaxEdges + 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (uint64_t)rows * p * span;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r = (uint32_t)(i / ((uint64_t)p * span)), l = (uint32_t)((i / span) % p), c = (uint32_t)(i % span);
        const QDesc D = desc[r];
        const int n = (int)D.n;
        auto factor = [&](uint32_t layer, bool inverse) {  // F or F' of a layer's mixer
            const double bt = betas[(size_t)D.out * p + layer], cb = cos(bt), sb = sin(bt);
            return fabs(cb) >= fabs(sb) ? cb : (inverse ? -sb : sb);
        };
        if (c <= D.e_count) {
            const double gm = gammas[(size_t)D.out * p + l];
            const double ang = -gm * ((double)D.e_count - 2.0 * (double)c);
            const double hin = l == 0 ? 1.0 / sqrt((double)(1ULL << n)) : pow(factor(l - 1, false), n);
            const double hrev = pow(factor(l, true), n);
            const double ca = cos(ang), sa = sin(ang);
            ptab[D.ptab + (uint64_t)l * span + c] = make_float2((float)(hin * ca), (float)(hin * sa));
            ptab[D.ptab + (uint64_t)(p + l) * span + c] = make_float2((float)(hrev * ca), (float)(hrev * sa));
        }
        if (c == 0) {
            const double bt = betas[(size_t)D.out * p + l], cb = cos(bt), sb = sin(bt);
            const bool fc = fabs(cb) >= fabs(sb);
            const double f = fc ? cb : sb, k = fc ? sb / cb : cb / sb;
            QMix M;
            M.kf = (float)k;
            M.kr = (float)-k;
            M.f2 = (float)(f * f);
            M.fn_f = (float)pow(f, n);
            M.fn_r = (float)pow(fc ? cb : -sb, n);
            M.f2_a0 = (float)pow(f * f, n - kQBTile);
            M.form_c = fc ? 1u : 0u;
            M.pad = 0;
            mtab[(uint64_t)r * p + l] = M;
        }
    }
}

// Mixer windows of a batched pass: round k applies the mixer to the tile bits
// [b0, b0 + 4) selected by a mask, with the 16 amplitudes j = base | (i << b0)
// of each thread in registers. Pass A: b0 = 0, 4, 8 (all bits); pass B: b0 =
// 8, 4, 0 (top first) while the window holds a bit at or above L, the bits
// below L masked out. The round count is a template argument, so b0, the
// shared-memory offsets of the 16 amplitudes and the global offsets of pass A
// fold to constants.
__host__ __device__ constexpr int qb_rounds_b(uint32_t L) { return L <= 3 ? 3 : (L <= 7 ? 2 : 1); }
__device__ __forceinline__ uint32_t qb_mask(bool pass_b, uint32_t b0, uint32_t L) {
    if (!pass_b || L <= b0) return 0xFu;
    return L >= b0 + 4 ? 0u : (0xFu & ~((1u << (L - b0)) - 1u));
}
__device__ __forceinline__ uint32_t qb_base(uint32_t b0) {  // thread's group with the window bits cleared
    const uint32_t g = threadIdx.x;
    return (g & ((1u << b0) - 1)) | ((g >> b0) << (b0 + 4));
}
// v, opaque to the compiler: the addresses derived from it are formed where
// they are used instead of being hoisted out of the tile loop into registers
__device__ __forceinline__ uint32_t qb_opaque(uint32_t v) {
    uint32_t r;
    asm volatile("mov.b32 %0, %1;" : "=r"(r) : "r"(v));
    return r;
}
// the 16 amplitudes base | (i << b0), pb = qb_phys(base) (qb_phys is linear
// over XOR and the two parts have no common bit), and back
__device__ __forceinline__ void qb_read(const float2 *tile, uint32_t pb, uint32_t b0, float2 (&v)[16]) {
    if (b0 == 0) {
#pragma unroll
        for (uint32_t i = 0; i < 16; i += 2) {
            const float4 t = *reinterpret_cast<const float4 *>(tile + (pb ^ i));
            v[i] = make_float2(t.x, t.y);
            v[i + 1] = make_float2(t.z, t.w);
        }
    } else {
#pragma unroll
        for (uint32_t i = 0; i < 16; ++i) v[i] = tile[pb ^ qb_phys(i << b0)];
    }
}
__device__ __forceinline__ void qb_write(float2 *tile, uint32_t pb, uint32_t b0, const float2 (&v)[16]) {
    if (b0 == 0) {
#pragma unroll
        for (uint32_t i = 0; i < 16; i += 2)
            *reinterpret_cast<float4 *>(tile + (pb ^ i)) = make_float4(v[i].x, v[i].y, v[i + 1].x, v[i + 1].y);
    } else {
#pragma unroll
        for (uint32_t i = 0; i < 16; ++i) tile[pb ^ qb_phys(i << b0)] = v[i];
    }
}
// one scaled gate on the pair (x, y): form C (x - i k y, y - i k x), form S
// (k x - i y, k y - i x)
template <bool FORM_C>
__device__ __forceinline__ void qb_gate(float2 &x, float2 &y, float k) {
    float2 a, b;
    if (FORM_C) {
        a = make_float2(fmaf(k, y.y, x.x), fmaf(-k, y.x, x.y));
        b = make_float2(fmaf(k, x.y, y.x), fmaf(-k, x.x, y.y));
    } else {
        a = make_float2(fmaf(k, x.x, y.y), fmaf(k, x.y, -y.x));
        b = make_float2(fmaf(k, y.x, x.y), fmaf(k, y.y, -x.x));
    }
    x = a;
    y = b;
}
template <bool FORM_C>
__device__ __forceinline__ void qb_mix(float2 (&a)[16], uint32_t mask, float k) {
#pragma unroll
    for (uint32_t b = 0; b < 4; ++b) {
        if (!((mask >> b) & 1u)) continue;
#pragma unroll
        for (uint32_t i = 0; i < 16; ++i)
            if (!(i & (1u << b))) qb_gate<FORM_C>(a[i], a[i | (1u << b)], k);
    }
}
// sum over the window bits in mask of Im<l|X_b|a> on the thread's amplitudes
// (taken before the window's gates: they commute with every X_b, so the sum is
// the same at any point of the mixer)
__device__ __forceinline__ float qb_grad(const float2 (&a)[16], const float2 (&l)[16], uint32_t mask) {
    float g[2] = {0.f, 0.f}, h[2] = {0.f, 0.f};
#pragma unroll
    for (uint32_t b = 0; b < 4; ++b) {
        if (!((mask >> b) & 1u)) continue;
#pragma unroll
        for (uint32_t i = 0; i < 16; ++i) {
            if (i & (1u << b)) continue;
            const uint32_t j = i | (1u << b);
            g[b & 1] = fmaf(l[i].x, a[j].y, g[b & 1]);
            h[b & 1] = fmaf(l[i].y, a[j].x, h[b & 1]);
            g[b & 1] = fmaf(l[j].x, a[i].y, g[b & 1]);
            h[b & 1] = fmaf(l[j].y, a[i].x, h[b & 1]);
        }
    }
    return (g[0] - h[0]) + (g[1] - h[1]);
}
// block sum of a per-thread float: warps in float, warps' totals in double;
// valid in thread 0; red is free again on return
__device__ __forceinline__ double qb_block_sum(float v, double *red) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) s += red[w];
    __syncthreads();
    return s;
}
// the same for two values at once (one pair of barriers)
__device__ __forceinline__ void qb_block_sum2(float v, float u, double *red, double &sv, double &su) {
    v = warp_sum(v);
    u = warp_sum(u);
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = (double)v;
        red[16 + (threadIdx.x >> 5)] = (double)u;
    }
    __syncthreads();
    sv = su = 0.0;
    if (threadIdx.x == 0)
        for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) {
            sv += red[w];
            su += red[16 + w];
        }
    __syncthreads();
}
// the cp.async copies of item tile t of instance D (psi, lambda for dual
// passes, the cost bytes for pass A), one commit group
__device__ __forceinline__ void qb_issue(bool dual, bool pass_b, bool with_cost, const QBArgs &a, const QDesc &D,
                                         float2 *arena, const uint8_t *costs, uint64_t t, float2 *tp, float2 *tl,
                                         uint8_t *tc) {
    const bool load_psi = pass_b || dual || a.layer > 0;
    if (load_psi) qb_load(tp, arena + D.psi, pass_b, a.L, t);
    if (dual) qb_load(tl, arena + D.lam, pass_b, a.L, t);
    if (with_cost) qb_load_cost(tc, costs + D.cost, t);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// a phase table into shared memory (visible after the caller's next barrier)
__device__ __forceinline__ void qb_table(float2 *spt, const float2 *ph, uint32_t e_count) {
    for (uint32_t c = threadIdx.x; c <= e_count; c += blockDim.x) spt[c] = ph[c];
}// the element offsets of the last round's amplitudes base | (i << b0) in the
// state: pass A contiguous tiles, pass B through qb_index (a bit permutation,
// so the offset of i is the sum of those of its bits)
template <bool PASS_B>
__device__ __forceinline__ void qb_offsets(const QBArgs &a, uint64_t t, uint32_t base, uint32_t b0, uint64_t &x0,
                                           uint32_t (&off)[16]) {
    x0 = qb_index(PASS_B, a.L, t, base);
    uint32_t o[4];
#pragma unroll
    for (uint32_t b = 0; b < 4; ++b) o[b] = PASS_B ? (uint32_t)qb_index(true, a.L, 0, 1u << (b0 + b)) : (1u << (b0 + b));
#pragma unroll
    for (uint32_t i = 0; i < 16; ++i)
        off[i] = ((i & 1u) ? o[0] : 0u) + ((i & 2u) ? o[1] : 0u) + ((i & 4u) ? o[2] : 0u) + ((i & 8u) ? o[3] : 0u);
}

// Item order of the batched passes. Pass A: each CTA walks a run of
// consecutive items (the instance's descriptor stays in L1 and its phase table
// in shared memory across the run). Pass B: grid-stride, so the CTAs at work
// hold neighbouring tiles of one instance (a pass-B tile is 2^(12-L) runs of
// 2^L amplitudes, and neighbouring tiles' runs are adjacent in memory).
struct QItems {
    uint64_t w, end, step;
};
template <bool PASS_B>
__device__ __forceinline__ QItems qb_items(const QBArgs &a) {
    const uint64_t items = (uint64_t)a.m * a.tiles;
    if (PASS_B) return QItems{blockIdx.x, items, gridDim.x};
    const uint64_t w0 = blockIdx.x * a.chunk;
    return QItems{w0, min(items, w0 + a.chunk), 1};
}

// forward pass: [pass A: cost phase] + mixer; the last pass B of the last
// layer also writes lambda = C psi and the per-tile energy. Two tile buffers:
// the next item's copies are issued before the current item's rounds.
template <bool PASS_B, int NR>
__global__ void __launch_bounds__(kQThreads, 3)
    k_qaoa_fwd(const QBArgs a, const QDesc *__restrict__ desc, float2 *__restrict__ arena, const uint8_t *__restrict__ costs,
               const float2 *__restrict__ ptab, const QMix *__restrict__ mtab, double *__restrict__ part) {
    extern __shared__ __align__(16) float2 qb_tile[];  // two tiles, then two cost-byte tiles
    uint8_t *tcs = reinterpret_cast<uint8_t *>(qb_tile + 2 * kQBT);
    __shared__ double red[32];
    __shared__ float2 spt[kQMaxEdges + 1];  // the instance's phase table
    const QItems it = qb_items<PASS_B>(a);
    if (it.w >= it.end) return;
    const bool last = PASS_B && a.layer + 1 == a.p;
    // pass A keeps the run's descriptor and constants in registers and reloads
    // them (and the phase table) between instances; pass B reads them per item
    uint32_t ci = (uint32_t)(it.w >> (a.n - kQBTile));
    QDesc Dc = desc[a.r0 + ci];
    QMix Mc = mtab[(uint64_t)(a.r0 + ci) * a.p + a.layer];
    qb_issue(false, PASS_B, !PASS_B, a, Dc, arena, costs, (it.w & (a.tiles - 1)), qb_tile, nullptr, tcs);
    if (!PASS_B) qb_table(spt, ptab + Dc.ptab + (uint64_t)a.layer * (kQMaxEdges + 1), Dc.e_count);
    uint32_t cur = 0;
    for (uint64_t w = it.w; w < it.end; w += it.step, cur ^= 1u) {
        const uint64_t t = (w & (a.tiles - 1));
        if (PASS_B) ci = (uint32_t)(w >> (a.n - kQBTile));
        const QDesc D = PASS_B ? desc[a.r0 + ci] : Dc;
        const QMix M = PASS_B ? mtab[(uint64_t)(a.r0 + ci) * a.p + a.layer] : Mc;
        const uint64_t wn = w + it.step;
        const uint32_t cn = (uint32_t)(wn >> (a.n - kQBTile));
        QDesc Dn = D;
        if (wn < it.end) {
            if (cn != ci) Dn = desc[a.r0 + cn];
            qb_issue(false, PASS_B, !PASS_B, a, Dn, arena, costs, (wn & (a.tiles - 1)), qb_tile + ((cur ^ 1u) << kQBTile), nullptr,
                     tcs + ((cur ^ 1u) << kQBTile));
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();
        float2 *tile = qb_tile + (cur << kQBTile);
        const uint8_t *tc = tcs + (cur << kQBTile);
        float2 v[16];
        uint32_t base = 0, pb = 0, b0 = 0;
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            b0 = PASS_B ? 8u - 4u * (uint32_t)k : 4u * (uint32_t)k;
            base = qb_opaque(qb_base(b0));
            pb = qb_phys(base);
            const uint32_t mask = qb_mask(PASS_B, b0, a.L);
            if (!PASS_B && k == 0) {  // the cost phase on window 0..3 (layer 0: the table holds H|0> times the phase)
                if (a.layer > 0) qb_read(tile, pb, 0, v);
                const uint4 cb = *reinterpret_cast<const uint4 *>(tc + base);
                const uint32_t cw[4] = {cb.x, cb.y, cb.z, cb.w};
#pragma unroll
                for (uint32_t i = 0; i < 16; ++i) {
                    const float2 f = spt[(cw[i >> 2] >> (8 * (i & 3))) & 0xFFu];
                    v[i] = a.layer == 0 ? f : cm(v[i], f);
                }
            } else {
                qb_read(tile, pb, b0, v);
            }
            if (M.form_c) qb_mix<true>(v, mask, M.kf);
            else qb_mix<false>(v, mask, M.kf);
            if (k + 1 < NR) {
                qb_write(tile, pb, b0, v);
                __syncthreads();
            }
        }
        uint64_t x0;
        uint32_t off[16];
        qb_offsets<PASS_B>(a, t, base, b0, x0, off);
        float2 *psi = arena + D.psi + x0;
        if (!last) {
#pragma unroll
            for (uint32_t i = 0; i < 16; ++i) psi[off[i]] = v[i];
        } else {  // psi with the layer's factor F^n back in, lambda = C psi and <C>
            float2 *lam = arena + D.lam + x0;
            const uint8_t *cst = costs + D.cost + x0;
            float e = 0.f;
#pragma unroll
            for (uint32_t i = 0; i < 16; ++i) {
                const float2 u = make_float2(v[i].x * M.fn_f, v[i].y * M.fn_f);
                const float cv = (float)cst[off[i]];
                psi[off[i]] = u;
                lam[off[i]] = make_float2(cv * u.x, cv * u.y);
                e = fmaf(cv, fmaf(u.x, u.x, u.y * u.y), e);
            }
            const double et = qb_block_sum(e, red);
            if (threadIdx.x == 0) part[D.part + t] = et;
        }
        __syncthreads();  // every read of this tile buffer and of spt is done before they are refilled
        if (!PASS_B && wn < it.end && cn != ci) {
            ci = cn;
            Dc = Dn;
            Mc = mtab[(uint64_t)(a.r0 + ci) * a.p + a.layer];
            qb_table(spt, ptab + Dc.ptab + (uint64_t)a.layer * (kQMaxEdges + 1), Dc.e_count);
        }
    }
}

// reverse pass: the inverse mixer on psi and lambda with the dE/dbeta terms;
// pass A then the cost layer's dE/dgamma term and the inverse phase. One
// buffer per tile (psi and lambda): the next item's copies are issued after
// the last round's reads.
template <bool PASS_B, int NR>
__global__ void __launch_bounds__(kQThreads, 2)
    k_qaoa_rev(const QBArgs a, const QDesc *__restrict__ desc, float2 *__restrict__ arena, const uint8_t *__restrict__ costs,
               const float2 *__restrict__ ptab, const QMix *__restrict__ mtab, double *__restrict__ part) {
    extern __shared__ __align__(16) float2 qb_tile[];
    float2 *tp = qb_tile, *tl = qb_tile + kQBT;
    uint8_t *tc = reinterpret_cast<uint8_t *>(qb_tile + 2 * kQBT);
    __shared__ double red[32];
    __shared__ float2 spt[kQMaxEdges + 1];  // the instance's inverse phase table
    const QItems it = qb_items<PASS_B>(a);
    if (it.w >= it.end) return;
    uint32_t ci_tab = ~0u;
    {
        const QDesc D = desc[a.r0 + (uint32_t)(it.w >> (a.n - kQBTile))];
        qb_issue(true, PASS_B, !PASS_B, a, D, arena, costs, (it.w & (a.tiles - 1)), tp, tl, tc);
    }
    for (uint64_t w = it.w; w < it.end; w += it.step) {
        const uint32_t ci = (uint32_t)(w >> (a.n - kQBTile));
        const uint64_t t = (w & (a.tiles - 1));
        const QDesc D = desc[a.r0 + ci];
        const QMix M = mtab[(uint64_t)(a.r0 + ci) * a.p + a.layer];
        if (!PASS_B && ci != ci_tab) {  // the previous item's reads of spt ended before its block sums' barriers
            qb_table(spt, ptab + D.ptab + (uint64_t)(a.p + a.layer) * (kQMaxEdges + 1), D.e_count);
            ci_tab = ci;
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
        float2 v[16], l[16];
        uint32_t cw[4] = {0u, 0u, 0u, 0u};  // the last round's cost bytes, four per word
        float gb = 0.f;
        float sc = PASS_B ? 1.f : M.f2_a0;  // F'^(2m) after the m gates of this layer undone so far
        uint32_t base = 0, pb = 0, b0 = 0;
#pragma unroll
        for (int k = 0; k < NR; ++k) {
            b0 = PASS_B ? 8u - 4u * (uint32_t)k : 4u * (uint32_t)k;
            base = qb_opaque(qb_base(b0));
            pb = qb_phys(base);
            const uint32_t mask = qb_mask(PASS_B, b0, a.L);
            qb_read(tp, pb, b0, v);
            qb_read(tl, pb, b0, l);
            if (!PASS_B && k + 1 == NR)
#pragma unroll
                for (uint32_t i = 0; i < 16; ++i) cw[i >> 2] |= (uint32_t)tc[base | (i << b0)] << (8 * (i & 3));
            gb = fmaf(qb_grad(v, l, mask), sc, gb);
#pragma unroll
            for (uint32_t b = 0; b < 4; ++b)
                if ((mask >> b) & 1u) sc *= M.f2;
            if (M.form_c) {
                qb_mix<true>(v, mask, M.kr);
                qb_mix<true>(l, mask, M.kr);
            } else {
                qb_mix<false>(v, mask, M.kr);
                qb_mix<false>(l, mask, M.kr);
            }
            if (k + 1 < NR) {
                qb_write(tp, pb, b0, v);
                qb_write(tl, pb, b0, l);
                __syncthreads();
            }
        }
        __syncthreads();  // every read of the tile buffers is done: stream the next item in
        const uint64_t wn = w + it.step;
        if (wn < it.end) {
            const uint32_t cn = (uint32_t)(wn >> (a.n - kQBTile));
            qb_issue(true, PASS_B, !PASS_B, a, cn == ci ? D : desc[a.r0 + cn], arena, costs, (wn & (a.tiles - 1)), tp, tl, tc);
        }
        uint64_t x0;
        uint32_t off[16];
        qb_offsets<PASS_B>(a, t, base, b0, x0, off);
        float2 *psi = arena + D.psi + x0, *lam = arena + D.lam + x0;
        const float W = (float)D.e_count;
        float gg = 0.f;
#pragma unroll
        for (uint32_t i = 0; i < 16; ++i) {
            float2 pv = v[i], lv = l[i];
            if (!PASS_B) {  // the cost layer: its gradient term, then undo its phase (the table holds F'^n)
                const uint32_t cv = (cw[i >> 2] >> (8 * (i & 3))) & 0xFFu;
                const float2 f = spt[cv];
                gg = fmaf(W - 2.f * (float)cv, lv.x * pv.y - lv.y * pv.x, gg);
                pv = cmc(pv, f);
                lv = cmc(lv, f);
            }
            psi[off[i]] = pv;
            lam[off[i]] = lv;
        }
        if (PASS_B) {
            const double gbt = qb_block_sum(gb, red);
            if (threadIdx.x == 0) part[D.part + (uint64_t)(1 + a.p + a.layer) * a.tiles + t] = gbt;
        } else {
            double gbt, ggt;
            qb_block_sum2(gb, gg, red, gbt, ggt);
            if (threadIdx.x == 0) {
                part[D.part + (uint64_t)(1 + a.layer) * a.tiles + t] = gbt;
                part[D.part + (uint64_t)(1 + 2 * a.p + a.layer) * a.tiles + t] = ggt * (double)M.fn_r * (double)M.fn_r;
            }
        }
    }
}

// energy and gradients of the batched instances: per-tile partials in order
__global__ void k_qaoa_reduce(const QBArgs a, const QDesc *__restrict__ desc, const double *__restrict__ part,
                              double *__restrict__ out_cost, double *__restrict__ out_grad) {
    const uint32_t slots = 1 + 2 * a.p;  // energy, dE/dgamma_l, dE/dbeta_l
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (uint64_t)a.m * slots;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t ci = (uint32_t)(i / slots), sl = (uint32_t)(i % slots);
        const QDesc D = desc[a.r0 + ci];
        const double *P = part + D.part;
        double v = 0.0;
        if (sl == 0) {
            for (uint64_t t = 0; t < a.tiles; ++t) v += P[t];
            out_cost[D.out] = v;
        } else if (sl <= a.p) {  // dE/dgamma_l
            const uint32_t l = sl - 1;
            for (uint64_t t = 0; t < a.tiles; ++t) v += P[(uint64_t)(1 + 2 * a.p + l) * a.tiles + t];
            out_grad[(size_t)D.out * 2 * a.p + l] = 2.0 * v;
        } else {  // dE/dbeta_l: pass A then pass B terms
            const uint32_t l = sl - 1 - a.p;
            double vb = 0.0;
            for (uint64_t t = 0; t < a.tiles; ++t) v += P[(uint64_t)(1 + l) * a.tiles + t];
            for (uint64_t t = 0; t < a.tiles; ++t) vb += P[(uint64_t)(1 + a.p + l) * a.tiles + t];
            out_grad[(size_t)D.out * 2 * a.p + a.p + l] = 2.0 * (v + vb);
        }
    }
}

}  // namespace

struct QaoaGraph {
    cudaGraphExec_t exec = nullptr;
    uint64_t key = 0;
};

}  // namespace qf

using namespace qf;

extern "C" int qf_qaoa_maxcut_batch(qf_ctx *ctx, const qf_qaoa_instance *inst, uint64_t n_inst, const uint32_t *edges_uv,
                                    uint64_t n_edges, uint32_t p, const double *gammas, const double *betas,
                                    double *cost_out, double *grad_out, const qf_qaoa_opts *opts) {
    clear_error();
    if (!ctx || !inst || !edges_uv || !gammas || !betas || !cost_out || !grad_out)
        return fail(QF_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n_inst == 0) return fail(QF_ERR_EMPTY_BATCH, "a CUDA state batch cannot be empty");
    if (p == 0 || p > (uint32_t)kQMaxP) return fail(QF_ERR_INVALID_ARGUMENT, "QAOA depth must be 1..%d, got %u", kQMaxP, p);
    // validate instances, lay out the arenas (largest instances first)
    std::vector<QDesc> desc(n_inst);
    std::vector<uint64_t> masks(n_edges);
    std::vector<uint32_t> order(n_inst);
    for (uint64_t i = 0; i < n_inst; ++i) order[i] = (uint32_t)i;
    for (uint64_t i = 0; i < n_inst; ++i) {
        const qf_qaoa_instance &I = inst[i];
        if (I.qubits < 2 || I.qubits > 30) return fail(QF_ERR_INVALID_ARGUMENT, "instance %llu: qubits must be 2..30, got %u", (unsigned long long)i, I.qubits);
        if (I.edge_count > (uint32_t)kQMaxEdges) return fail(QF_ERR_INVALID_ARGUMENT, "instance %llu: at most %d edges", (unsigned long long)i, kQMaxEdges);
        if ((uint64_t)I.edge_begin + I.edge_count > n_edges) return fail(QF_ERR_INVALID_ARGUMENT, "instance %llu: edges out of range", (unsigned long long)i);
        for (uint32_t e = 0; e < I.edge_count; ++e) {
            const uint32_t u = edges_uv[2 * (I.edge_begin + e)], v = edges_uv[2 * (I.edge_begin + e) + 1];
            if (u >= I.qubits || v >= I.qubits) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "instance %llu: edge (%u, %u) outside %u qubits", (unsigned long long)i, u, v, I.qubits);
            if (u == v) return fail(QF_ERR_INVALID_QUBIT_PAIR, "instance %llu: self-loop on %u", (unsigned long long)i, u);
        }
    }
    for (uint64_t e = 0; e < n_edges; ++e) masks[e] = (1ULL << edges_uv[2 * e]) | (1ULL << edges_uv[2 * e + 1]);
    for (uint64_t i = 0; i < n_inst * p; ++i)
        if (!std::isfinite(gammas[i]) || !std::isfinite(betas[i])) return fail(QF_ERR_NON_FINITE_PARAMETER, "circuit parameters must be finite");
    // an instance above 12 qubits runs in the batched passes unless a tile
    // width is given for it (then one CTA per instance, like the small ones)
    auto tile_req = [&](const qf_qaoa_instance &I) -> int {
        return I.tile_qubits ? (int)I.tile_qubits : (opts && I.qubits <= 32 ? opts->tile_qubits[I.qubits] : 0);
    };
    auto batched = [&](const qf_qaoa_instance &I) { return I.qubits > (uint32_t)kQBTile && tile_req(I) == 0; };
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        const bool ba = batched(inst[a]), bb = batched(inst[b]);
        if (ba != bb) return ba;
        return inst[a].qubits > inst[b].qubits;
    });
    // rows [0, r_small): batched passes per qubit count (13..24 qubits); the
    // rest: one CTA per instance
    uint64_t amp_off = 0, cost_off = 0, ptab_off = 0, part_off = 0;
    uint32_t r_small = 0;
    for (uint64_t r = 0; r < n_inst; ++r) {
        const qf_qaoa_instance &I = inst[order[r]];
        QDesc &D = desc[r];
        std::memset(&D, 0, sizeof D);
        D.n = I.qubits;
        if (D.n > 24) return fail(QF_ERR_UNSUPPORTED_OPERATION, "batched QAOA supports up to 24 qubits, got %u", D.n);
        if (batched(I)) {
            r_small = (uint32_t)r + 1;
            D.k = kQBTile;
            D.ptab = ptab_off;
            ptab_off += 2ULL * p * (kQMaxEdges + 1);  // forward and reverse tables
            D.part = part_off;
            part_off += (uint64_t)(1 + 3 * p) << (D.n - kQBTile);
        } else {
            const int kt = tile_req(I) ? tile_req(I) : 10;
            D.k = (uint32_t)std::max(4, std::min(kQMaxTile, kt));
            if (D.n > D.k && D.n - D.k > D.k - 1) D.k = (D.n + 1) / 2 + 1;  // pass B needs n-k+1 <= k
            D.k = std::min<uint32_t>(D.k, (uint32_t)kQMaxTile);
        }
        D.e_begin = I.edge_begin;
        D.e_count = I.edge_count;
        D.out = order[r];
        D.pad = 0;
        D.psi = amp_off;
        amp_off += 1ULL << D.n;
        D.lam = amp_off;
        amp_off += 1ULL << D.n;
        D.cost = cost_off;
        cost_off += 1ULL << D.n;
    }
    QF_CUDA(cudaSetDevice(ctx->device));
    // device layout in the context's sampler workspace:
    // desc | masks | gammas | betas | out_cost | out_grad | counter | arena | costs
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t b_desc = al(sizeof(QDesc) * n_inst), b_mask = al(8 * std::max<uint64_t>(1, n_edges));
    const size_t b_par = al(8 * n_inst * p), b_cost = al(8 * n_inst), b_grad = al(16 * n_inst * p), b_cnt = 256;
    const size_t b_arena = al(8 * amp_off), b_costs = al(cost_off);
    const size_t b_ptab = al(8 * std::max<uint64_t>(1, ptab_off)), b_mtab = al(sizeof(QMix) * std::max<uint64_t>(1, (uint64_t)r_small * p));
    const size_t b_part = al(8 * std::max<uint64_t>(1, part_off));
    const size_t total = b_desc + b_mask + 2 * b_par + b_cost + b_grad + b_cnt + b_arena + b_costs + b_ptab + b_mtab + b_part;
    QF_TRY(ensure_device(&ctx->ws_tree, &ctx->ws_tree_bytes, total));
    unsigned char *w = static_cast<unsigned char *>(ctx->ws_tree);
    QDesc *d_desc = reinterpret_cast<QDesc *>(w);
    uint64_t *d_mask = reinterpret_cast<uint64_t *>(w + b_desc);
    double *d_gam = reinterpret_cast<double *>(w + b_desc + b_mask);
    double *d_bet = reinterpret_cast<double *>(w + b_desc + b_mask + b_par);
    double *d_cost = reinterpret_cast<double *>(w + b_desc + b_mask + 2 * b_par);
    double *d_grad = reinterpret_cast<double *>(w + b_desc + b_mask + 2 * b_par + b_cost);
    unsigned *d_cnt = reinterpret_cast<unsigned *>(w + b_desc + b_mask + 2 * b_par + b_cost + b_grad);
    float2 *d_arena = reinterpret_cast<float2 *>(w + b_desc + b_mask + 2 * b_par + b_cost + b_grad + b_cnt);
    uint8_t *d_costs = reinterpret_cast<uint8_t *>(w + b_desc + b_mask + 2 * b_par + b_cost + b_grad + b_cnt + b_arena);
    unsigned char *w2 = w + b_desc + b_mask + 2 * b_par + b_cost + b_grad + b_cnt + b_arena + b_costs;
    float2 *d_ptab = reinterpret_cast<float2 *>(w2);
    QMix *d_mtab = reinterpret_cast<QMix *>(w2 + b_ptab);
    double *d_part = reinterpret_cast<double *>(w2 + b_ptab + b_mtab);
    cudaStream_t st = ctx->stream;
    QF_CUDA(cudaMemcpyAsync(d_desc, desc.data(), sizeof(QDesc) * n_inst, cudaMemcpyHostToDevice, st));
    if (n_edges) QF_CUDA(cudaMemcpyAsync(d_mask, masks.data(), 8 * n_edges, cudaMemcpyHostToDevice, st));
    QF_CUDA(cudaMemcpyAsync(d_gam, gammas, 8 * n_inst * p, cudaMemcpyHostToDevice, st));
    QF_CUDA(cudaMemcpyAsync(d_bet, betas, 8 * n_inst * p, cudaMemcpyHostToDevice, st));
    static bool attr[64] = {false};
    static int pass_occ[64][8];
    const size_t smem = sizeof(QShared);
    // forward: two tiles + two cost-byte tiles; reverse: psi and lambda tiles + cost bytes
    const size_t smem_f = 2 * (sizeof(float2) * kQBT + kQBT), smem_r = 2 * sizeof(float2) * kQBT + kQBT;
    // passes: forward A, forward B with 1..3 rounds, reverse A, reverse B with 1..3 rounds
    using QPass = void (*)(QBArgs, const QDesc *, float2 *, const uint8_t *, const float2 *, const QMix *, double *);
    const QPass passes[8] = {k_qaoa_fwd<false, 3>, k_qaoa_fwd<true, 1>, k_qaoa_fwd<true, 2>, k_qaoa_fwd<true, 3>,
                             k_qaoa_rev<false, 3>, k_qaoa_rev<true, 1>, k_qaoa_rev<true, 2>, k_qaoa_rev<true, 3>};
    const int dev = ctx->device & 63;
    if (!attr[dev]) {
        QF_CUDA(cudaFuncSetAttribute(k_qaoa_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        for (int i = 0; i < 8; ++i) {
            const size_t sm_i = i < 4 ? smem_f : smem_r;
            QF_CUDA(cudaFuncSetAttribute(passes[i], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_i));
            QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pass_occ[dev][i], passes[i], kQThreads, sm_i));
        }
        attr[dev] = true;
    }
    const uint32_t n_small = (uint32_t)n_inst - r_small;
    int per_sm = 0;
    QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_qaoa_batch, kQThreads, smem));
    const uint32_t grid = (uint32_t)std::min<uint64_t>(std::max(1u, n_small), (uint64_t)std::max(1, per_sm) * ctx->sm_count);
    // one wave of resident CTAs, each on a run of consecutive items
    auto pass_grid = [&](int i, uint64_t items, uint64_t *chunk) {
        const uint64_t g = std::min<uint64_t>(items, (uint64_t)std::max(1, pass_occ[dev][i]) * ctx->sm_count);
        *chunk = (items + g - 1) / g;
        return (unsigned)((items + *chunk - 1) / *chunk);
    };
    auto enqueue = [&](cudaStream_t s) -> int {
        if (r_small) {
            k_qaoa_tables<<<(unsigned)std::min<uint64_t>(4096, ((uint64_t)r_small * p * (kQMaxEdges + 1) + 255) / 256), 256, 0, s>>>(
                d_desc, r_small, d_gam, d_bet, p, d_ptab, d_mtab);
            QF_CUDA(cudaGetLastError());
        }
        for (uint32_t r0 = 0; r0 < r_small;) {  // one launch sequence per qubit count
            uint32_t r1 = r0;
            while (r1 < r_small && desc[r1].n == desc[r0].n) ++r1;
            QBArgs A;
            A.r0 = r0;
            A.m = r1 - r0;
            A.n = desc[r0].n;
            A.L = 24 - A.n;
            A.p = p;
            A.tiles = 1ULL << (A.n - kQBTile);
            const uint64_t items = (uint64_t)A.m * A.tiles;
            const int rb = qb_rounds_b(A.L);  // pass B rounds: 3, 2 or 1
            uint64_t cfa, cfb, cra, crb;
            const unsigned gfa = pass_grid(0, items, &cfa), gfb = pass_grid(rb, items, &cfb);
            const unsigned gra = pass_grid(4, items, &cra), grb = pass_grid(4 + rb, items, &crb);
            A.layer = 0;
            A.chunk = 0;
            k_qaoa_costs<<<gfa, kQThreads, 0, s>>>(A, d_desc, d_mask, d_costs);
            for (uint32_t l = 0; l < p; ++l) {
                A.layer = l;
                A.chunk = cfa;
                passes[0]<<<gfa, kQThreads, smem_f, s>>>(A, d_desc, d_arena, d_costs, d_ptab, d_mtab, d_part);
                A.chunk = cfb;
                passes[rb]<<<gfb, kQThreads, smem_f, s>>>(A, d_desc, d_arena, d_costs, d_ptab, d_mtab, d_part);
            }
            for (uint32_t l = p; l-- > 0;) {
                A.layer = l;
                A.chunk = crb;
                passes[4 + rb]<<<grb, kQThreads, smem_r, s>>>(A, d_desc, d_arena, d_costs, d_ptab, d_mtab, d_part);
                A.chunk = cra;
                passes[4]<<<gra, kQThreads, smem_r, s>>>(A, d_desc, d_arena, d_costs, d_ptab, d_mtab, d_part);
            }
            k_qaoa_reduce<<<(unsigned)std::max<uint64_t>(1, ((uint64_t)A.m * (1 + 2 * p) + 127) / 128), 128, 0, s>>>(
                A, d_desc, d_part, d_cost, d_grad);
            QF_CUDA(cudaGetLastError());
            r0 = r1;
        }
        if (n_small) {
            QF_CUDA(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned), s));
            k_qaoa_batch<<<grid, kQThreads, smem, s>>>(d_desc + r_small, n_small, d_arena, d_costs, d_mask, d_gam, d_bet, p,
                                                       d_cost, d_grad, d_cnt);
            QF_CUDA(cudaGetLastError());
        }
        return QF_OK;
    };
    if (opts && opts->use_graph) {
        // capture the memset + persistent launch once per layout and replay it
        static thread_local cudaGraphExec_t exec = nullptr;
        static thread_local uint64_t key = 0;
        uint64_t k2 = 1469598103934665603ULL;  // FNV-1a over everything the captured launches depend on
        auto mix = [&](uint64_t v) {
            for (int b = 0; b < 8; ++b) k2 = (k2 ^ ((v >> (8 * b)) & 0xFF)) * 1099511628211ULL;
        };
        mix((uint64_t)(uintptr_t)w);
        mix(n_inst);
        mix(p);
        mix(amp_off);
        mix(grid);
        mix(r_small);
        for (uint32_t r = 0; r < r_small; ++r) mix(desc[r].n);
        if (!exec || key != k2) {
            if (exec) cudaGraphExecDestroy(exec);
            exec = nullptr;
            cudaGraph_t graph;
            QF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            const int est = enqueue(st);
            const cudaError_t ce = cudaStreamEndCapture(st, &graph);
            if (est) return est;
            if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
            const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ie != cudaSuccess) {
                exec = nullptr;
                return cuda_fail(ie, "cudaGraphInstantiate");
            }
            key = k2;
        }
        QF_CUDA(cudaGraphLaunch(exec, st));
    } else {
        QF_TRY(enqueue(st));
    }
    // results come back in caller order (d_cost/d_grad are indexed by D.out)
    QF_CUDA(cudaMemcpyAsync(cost_out, d_cost, 8 * n_inst, cudaMemcpyDeviceToHost, st));
    QF_CUDA(cudaMemcpyAsync(grad_out, d_grad, 16 * n_inst * p, cudaMemcpyDeviceToHost, st));
    QF_CUDA(cudaStreamSynchronize(st));
    return QF_OK;
}
