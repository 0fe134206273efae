// density.cu — density-matrix kernels (DensityMatrix, src/lib.rs:1551-2235;
// the reference's CUDA density path, src/cuda.rs:2007-2237).
//
// A density matrix of n qubits is stored row-major, rho[row * 2^n + col], as
// one 2n-qubit vector: column qubit q is index bit q, row qubit q is index bit
// n + q. Unitaries U rho U^dagger become U on bit n + q and conj(U) on bit q
// and run through the fused tile engine; the kernels here are the non-unitary
// pieces: local channels (a real superoperator on the bit pair (n + q, q)),
// diagonal reductions, measurement collapse and state preparation.
#include <algorithm>
#include <cmath>
#include <vector>

#include "qf_device.cuh"
#include "qf_internal.h"

namespace qf {

namespace {

// Insert a zero bit at position p of x.
__device__ __forceinline__ uint64_t insert0(uint64_t x, uint32_t p) {
    const uint64_t lo = x & ((1ULL << p) - 1);
    return ((x >> p) << (p + 1)) | lo;
}

// One local channel on qubit q: for each (row bit r, col bit c) group
//   v00' = a v00 + b v11,  v11' = c v00 + d v11,  v01' = e v01,  v10' = f v10
// (every channel of NoiseChannel has this form: populations mix, coherences scale).
// SHAPE 0: general; 1: a = 1, c = 0 (amplitude damping: 8 multiplies instead
// of 12, which matters because complex128 channels run close to the GB300's
// FP64 issue rate); 2: a = d = 1, b = c = 0 (phase damping: only the
// coherences are read and written). Arithmetic in the state's precision.
template <typename C, int SHAPE>
__global__ void k_dm_channel(C *__restrict__ v, uint32_t n, uint32_t q, uint64_t groups, double ca, double cb, double cc,
                             double cd, double ce, double cf) {
    using R = typename Real<C>::T;
    const uint64_t cm = 1ULL << q, rm = 1ULL << (n + q);
    const R a = (R)ca, b = (R)cb, c = (R)cc, d = (R)cd, e = (R)ce, f = (R)cf;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < groups; g += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i00 = insert0(insert0(g, q), n + q);
        const C x01 = v[i00 | cm], x10 = v[i00 | rm];
        if (SHAPE != 2) {
            const C x00 = v[i00], x11 = v[i00 | rm | cm];
            if (SHAPE == 1) {
                v[i00] = mk(x00.x + b * x11.x, x00.y + b * x11.y);
                v[i00 | rm | cm] = mk(d * x11.x, d * x11.y);
            } else {
                v[i00] = mk(a * x00.x + b * x11.x, a * x00.y + b * x11.y);
                v[i00 | rm | cm] = mk(c * x00.x + d * x11.x, c * x00.y + d * x11.y);
            }
        }
        v[i00 | cm] = mk(e * x01.x, e * x01.y);
        v[i00 | rm] = mk(f * x10.x, f * x10.y);
    }
}

// Diagonal / near-diagonal sums over rows r < 2^n:
// mode 0: Re and Im of rho[r][r] (trace); 1: Re rho[r][r] where bit q of r is
// set (P(1)); 2: (+/-) Re rho[r][r] by bit q (<Z_q>); 3: 2 Re rho[r][r|m] and
// 4: -2 Im rho[r][r|m] over r with bit q clear (<X_q>, <Y_q>).
template <typename C>
__global__ void k_dm_diag(const C *__restrict__ v, uint32_t n, uint32_t q, int mode, double *partials) {
    __shared__ double red[32];
    const uint64_t D = 1ULL << n, m = 1ULL << q;
    double s0 = 0.0, s1 = 0.0;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x) {
        if (mode <= 2) {
            const C x = v[(r << n) | r];
            if (mode == 0) {
                s0 += (double)x.x;
                s1 += (double)x.y;
            } else if (mode == 1) {
                if (r & m) s0 += (double)x.x;
            } else {
                s0 += (r & m) ? -(double)x.x : (double)x.x;
            }
        } else if (!(r & m)) {
            const C x = v[(r << n) | (r | m)];
            s0 += mode == 3 ? 2.0 * (double)x.x : -2.0 * (double)x.y;
        }
    }
    s0 = block_sum(s0, red);
    __syncthreads();
    s1 = block_sum(s1, red);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = s0;
        partials[2 * blockIdx.x + 1] = s1;
    }
}

// Re rho[r][r] for every row (DensityMatrix probabilities).
template <typename C>
__global__ void k_dm_diag_out(const C *__restrict__ v, uint32_t n, double *out) {
    const uint64_t D = 1ULL << n;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x)
        out[r] = (double)v[(r << n) | r].x;
}

// DensityMatrix::measure collapse (src/lib.rs:1937-1946): entries whose row or
// column bit differs from the outcome become 0, the rest are divided by P.
template <typename C>
__global__ void k_dm_collapse(C *__restrict__ v, uint32_t n, uint32_t q, int outcome, double prob) {
    using R = typename Real<C>::T;
    const uint64_t total = 1ULL << (2 * n);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const int rb = (int)((i >> (n + q)) & 1ULL), cb = (int)((i >> q) & 1ULL);
        if (rb != outcome || cb != outcome) {
            v[i] = mk((R)0, (R)0);
        } else {
            const C x = v[i];
            v[i] = mk((R)((double)x.x / prob), (R)((double)x.y / prob));
        }
    }
}

// DensityMatrix::from_state (src/lib.rs:1641-1655): rho[r][c] = a_r conj(a_c).
template <typename C>
__global__ void k_dm_outer(const C *__restrict__ a, uint32_t n, C *__restrict__ v) {
    using R = typename Real<C>::T;
    const uint64_t total = 1ULL << (2 * n), cmask = (1ULL << n) - 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const C x = a[i >> n], y = a[i & cmask];
        v[i] = mk((R)((double)x.x * (double)y.x + (double)x.y * (double)y.y),
                  (R)((double)x.y * (double)y.x - (double)x.x * (double)y.y));
    }
}

// I / 2^n (DensityMatrix::maximally_mixed, src/lib.rs:1668-1700).
template <typename C>
__global__ void k_dm_mixed(C *__restrict__ v, uint32_t n) {
    using R = typename Real<C>::T;
    const uint64_t total = 1ULL << (2 * n), cmask = (1ULL << n) - 1;
    const double d = 1.0 / (double)(1ULL << n);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x)
        v[i] = mk((R)((i >> n) == (i & cmask) ? d : 0.0), (R)0);
}

// Several local channels in one sweep: the matrix is walked in tiles of 2^k
// entries whose bits are the low five column bits (coalesced 32-entry runs)
// plus the (row, column) bit pairs of the channels; each CTA loads a tile to
// shared memory, applies the channels in order and stores it back.
constexpr int kMaxTileChannels = 12;
struct ChannelTile {
    uint32_t k;                       // tile bits
    uint32_t n_hi;                    // tile bits above the low five
    uint64_t outer_mask;              // bits enumerated by the tile index
    uint64_t hi_bits[kMaxTileChannels * 2];
    uint32_t n_ch;
    uint8_t lc[kMaxTileChannels], lr[kMaxTileChannels], shape[kMaxTileChannels];
    double coef[kMaxTileChannels][6];
    float coef_f[kMaxTileChannels][6];  // the same in f32: no f64 -> f32 conversion per tile for complex64
    // complex64 paired rounds (k = 12): per round its channels (0xFF: none),
    // the tile bits of the thread's eight index bits, the swizzled offsets of
    // its 16 entries and whether entries i, i + 1 share a 16-byte slot
    uint8_t rch[kMaxTileChannels / 2][2];
    uint8_t rpos[kMaxTileChannels / 2][8];
    uint16_t roff[kMaxTileChannels / 2][16];
    uint8_t rwide[kMaxTileChannels / 2];
    uint32_t n_rounds;
};

template <typename C>
__global__ void __launch_bounds__(256) k_dm_channel_tile(C *__restrict__ v, uint64_t n_tiles, const ChannelTile ct) {
    using R = typename Real<C>::T;
    extern __shared__ __align__(16) unsigned char dm_smem[];
    C *s = reinterpret_cast<C *>(dm_smem);
    uint64_t *hi_off = reinterpret_cast<uint64_t *>(dm_smem + (sizeof(C) << ct.k));
    const uint32_t T = 1u << ct.k;
    for (uint32_t h = threadIdx.x; h < (1u << ct.n_hi); h += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t r = 0; r < ct.n_hi; ++r)
            if ((h >> r) & 1u) off |= ct.hi_bits[r];
        hi_off[h] = off;
    }
    __syncthreads();
    for (uint64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const uint64_t base = deposit(t, ct.outer_mask);
        if (sizeof(C) == 8) {  // complex64: 16-byte accesses (2 amplitudes of a 32-amplitude run), all in flight
#pragma unroll 8
            for (uint32_t w = threadIdx.x; w < (T >> 1); w += blockDim.x) {
                const uint32_t j = w << 1;
                *reinterpret_cast<float4 *>(s + j) = *reinterpret_cast<const float4 *>(v + (base | hi_off[j >> 5] | (j & 31u)));
            }
        } else {
            for (uint32_t j = threadIdx.x; j < T; j += blockDim.x) s[j] = v[base | hi_off[j >> 5] | (j & 31u)];
        }
        __syncthreads();
        for (uint32_t c = 0; c < ct.n_ch; ++c) {
            const uint32_t lc = ct.lc[c], lr = ct.lr[c], lo = min(lc, lr), hi = max(lc, lr);
            const uint32_t cm = 1u << lc, rm = 1u << lr;
            R a, b, cc, d, e, f;
            if (sizeof(R) == 4) {
                a = (R)ct.coef_f[c][0], b = (R)ct.coef_f[c][1], cc = (R)ct.coef_f[c][2], d = (R)ct.coef_f[c][3];
                e = (R)ct.coef_f[c][4], f = (R)ct.coef_f[c][5];
            } else {
                a = (R)ct.coef[c][0], b = (R)ct.coef[c][1], cc = (R)ct.coef[c][2], d = (R)ct.coef[c][3];
                e = (R)ct.coef[c][4], f = (R)ct.coef[c][5];
            }
            const int shape = ct.shape[c];
            for (uint32_t g = threadIdx.x; g < (T >> 2); g += blockDim.x) {
                uint32_t i = g;
                i = ((i >> lo) << (lo + 1)) | (i & ((1u << lo) - 1u));
                i = ((i >> hi) << (hi + 1)) | (i & ((1u << hi) - 1u));
                const C x01 = s[i | cm], x10 = s[i | rm];
                if (shape != 2) {
                    const C x00 = s[i], x11 = s[i | rm | cm];
                    s[i] = mk(a * x00.x + b * x11.x, a * x00.y + b * x11.y);
                    s[i | rm | cm] = mk(cc * x00.x + d * x11.x, cc * x00.y + d * x11.y);
                }
                s[i | cm] = mk(e * x01.x, e * x01.y);
                s[i | rm] = mk(f * x10.x, f * x10.y);
            }
            __syncthreads();
        }
        if (sizeof(C) == 8) {
#pragma unroll 8
            for (uint32_t w = threadIdx.x; w < (T >> 1); w += blockDim.x) {
                const uint32_t j = w << 1;
                *reinterpret_cast<float4 *>(v + (base | hi_off[j >> 5] | (j & 31u))) = *reinterpret_cast<const float4 *>(s + j);
            }
        } else {
            for (uint32_t j = threadIdx.x; j < T; j += blockDim.x) v[base | hi_off[j >> 5] | (j & 31u)] = s[j];
        }
        __syncthreads();
    }
}

// Complex64 tiles of 12 bits, channels applied two per shared-memory round
// trip: in a round each thread holds the 16 entries base | (i over the bits
// lc, lr of its first channel and lc, lr of its second) in registers (a lone
// channel takes two other tile bits as bits 2, 3 of i). Tiles stream in by
// 16-byte cp.async into one of two buffers while the other is worked on (the
// next tile's copies are issued before the current tile's rounds). In shared
// memory entry j sits at dm_swz(j): bits 1..3 XOR bits 4..6, 7..9 and 10..11,
// bit 0 kept (a copied 16-byte pair stays whole). The host puts the lane bits
// of a round on tile bits whose bank-pair vectors dm_swz(1 << b) & 15 are
// independent (16 distinct bank pairs per half warp); a round holding tile bit
// 0 reads and writes its pairs as 16-byte words.
__host__ __device__ inline uint32_t dm_swz(uint32_t j) { return j ^ ((((j >> 4) ^ (j >> 7) ^ (j >> 10)) & 7u) << 1); }
template <bool GENERAL>
__device__ __forceinline__ void dm_quad(float2 &x00, float2 &x01, float2 &x10, float2 &x11, const float *k) {
    if (GENERAL) {
        const float2 p = x00, q = x11;
        x00 = make_float2(k[0] * p.x + k[1] * q.x, k[0] * p.y + k[1] * q.y);
        x11 = make_float2(k[2] * p.x + k[3] * q.x, k[2] * p.y + k[3] * q.y);
    }
    x01 = make_float2(k[4] * x01.x, k[4] * x01.y);
    x10 = make_float2(k[5] * x10.x, k[5] * x10.y);
}
// channel on bits (sel, sel << 1) of the 16-entry index: sel = 1 for bits 0, 1
// (quads over bits 2, 3), sel = 4 for bits 2, 3
template <uint32_t SEL>
__device__ __forceinline__ void dm_apply(float2 (&e)[16], int shape, const float *k) {
    constexpr uint32_t O = SEL == 1 ? 4u : 1u;  // step between the four quads
#pragma unroll
    for (uint32_t q = 0; q < 4; ++q) {
        const uint32_t b = q * O;
        if (shape == 2) dm_quad<false>(e[b], e[b | SEL], e[b | (SEL << 1)], e[b | (SEL * 3)], k);
        else dm_quad<true>(e[b], e[b | SEL], e[b | (SEL << 1)], e[b | (SEL * 3)], k);
    }
}
__device__ __forceinline__ void dm_cp16(float2 *dst, const float2 *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__global__ void __launch_bounds__(256, 3) k_dm_channel_pairs(float2 *__restrict__ v, uint64_t n_tiles, const ChannelTile ct) {
    extern __shared__ __align__(16) unsigned char dm_smem[];
    float2 *buf = reinterpret_cast<float2 *>(dm_smem);  // two tiles of 4096 entries
    uint64_t *hi_off = reinterpret_cast<uint64_t *>(dm_smem + 2 * (sizeof(float2) << 12));
    uint64_t *dep = hi_off + 128;  // the tile index's bits on outer_mask, per byte of the index
    for (uint32_t h = threadIdx.x; h < 128u; h += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t r = 0; r < ct.n_hi; ++r)
            if ((h >> r) & 1u) off |= ct.hi_bits[r];
        hi_off[h] = off;
    }
    for (uint32_t h = threadIdx.x; h < 3u * 256u; h += blockDim.x)
        dep[h] = deposit((uint64_t)(h & 255u) << (8 * (h >> 8)), ct.outer_mask);
    __syncthreads();
    // copy k of a thread holds the entries j, j + 1 for j = 2 (tid + 256 k)
    const uint32_t tid = threadIdx.x, j0 = tid << 1, slot0 = dm_swz(j0);
    auto tile_base = [&](uint64_t t) { return dep[t & 255u] | dep[256u + ((t >> 8) & 255u)] | dep[512u + ((t >> 16) & 255u)]; };
    auto issue = [&](uint64_t t, float2 *dst) {
        const float2 *src = v + (tile_base(t) | (j0 & 31u));
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k) dm_cp16(dst + (slot0 ^ dm_swz(512u * k)), src + hi_off[(tid >> 4) + 16 * k]);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    uint64_t t = blockIdx.x;
    uint32_t cur = 0;
    if (t < n_tiles) issue(t, buf);
    for (; t < n_tiles; t += gridDim.x, cur ^= 1u) {
        float2 *s = buf + (cur << 12);
        if (t + gridDim.x < n_tiles) {  // the other buffer's last reads ended before the previous tile's final barrier
            issue(t + gridDim.x, buf + ((cur ^ 1u) << 12));
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();
        for (uint32_t r = 0; r < ct.n_rounds; ++r) {
            const uint32_t c1 = ct.rch[r][0], c2 = ct.rch[r][1];
            uint32_t g = 0;
#pragma unroll
            for (uint32_t b = 0; b < 8; ++b) g |= ((tid >> b) & 1u) << ct.rpos[r][b];
            const uint32_t pb = dm_swz(g);
            float2 e[16];
            if (ct.rwide[r]) {
#pragma unroll
                for (uint32_t i = 0; i < 16; i += 2) {
                    const float4 x = *reinterpret_cast<const float4 *>(s + (pb ^ ct.roff[r][i]));
                    e[i] = make_float2(x.x, x.y);
                    e[i + 1] = make_float2(x.z, x.w);
                }
            } else {
#pragma unroll
                for (uint32_t i = 0; i < 16; ++i) e[i] = s[pb ^ ct.roff[r][i]];
            }
            dm_apply<1>(e, ct.shape[c1], ct.coef_f[c1]);
            if (c2 < ct.n_ch) dm_apply<4>(e, ct.shape[c2], ct.coef_f[c2]);
            if (ct.rwide[r]) {
#pragma unroll
                for (uint32_t i = 0; i < 16; i += 2)
                    *reinterpret_cast<float4 *>(s + (pb ^ ct.roff[r][i])) = make_float4(e[i].x, e[i].y, e[i + 1].x, e[i + 1].y);
            } else {
#pragma unroll
                for (uint32_t i = 0; i < 16; ++i) s[pb ^ ct.roff[r][i]] = e[i];
            }
            __syncthreads();
        }
        float2 *dst = v + (tile_base(t) | (j0 & 31u));
#pragma unroll
        for (uint32_t k = 0; k < 8; ++k)
            *reinterpret_cast<float4 *>(dst + hi_off[(tid >> 4) + 16 * k]) =
                *reinterpret_cast<const float4 *>(s + (slot0 ^ dm_swz(512u * k)));
        __syncthreads();
    }
}

int grid_for(const qf_ctx *ctx, uint64_t work) {
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((work + 255) / 256, (uint64_t)ctx->sm_count * 8));
}

}  // namespace

template <typename C, int SHAPE> void launch_channel(qf_sv *sv, uint32_t n, uint32_t q, const double *k) {
    qf_ctx *ctx = sv->ctx;
    const uint64_t groups = 1ULL << (2 * n - 2);
    k_dm_channel<C, SHAPE><<<grid_for(ctx, groups), 256, 0, ctx->stream>>>(static_cast<C *>(sv->d), n, q, groups, k[0], k[1],
                                                                           k[2], k[3], k[4], k[5]);
}

template <typename C> void launch_channel_shape(qf_sv *sv, uint32_t n, uint32_t q, const double *k) {
    if (k[0] == 1.0 && k[1] == 0.0 && k[2] == 0.0 && k[3] == 1.0) launch_channel<C, 2>(sv, n, q, k);
    else if (k[0] == 1.0 && k[2] == 0.0) launch_channel<C, 1>(sv, n, q, k);
    else launch_channel<C, 0>(sv, n, q, k);
}

int dm_channel(qf_sv *sv, uint32_t n, uint32_t q, const double coef[6]) {
    if (sv->dtype == QF_C64) launch_channel_shape<float2>(sv, n, q, coef);
    else launch_channel_shape<double2>(sv, n, q, coef);
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

int dm_channels_fused(qf_sv *sv, uint32_t n, const uint32_t *qs, const double (*coefs)[6], uint32_t count) {
    qf_ctx *ctx = sv->ctx;
    if (count == 0) return QF_OK;
    if (count > (uint32_t)kMaxTileChannels || 2 * n < 5) return fail(QF_ERR_INVALID_ARGUMENT, "channel group too large");
    // the kernel moves complex64 entries two at a time (16-byte accesses): the
    // tile's low five bits are column bits 0..4 and the matrix is 16-byte aligned
    if (reinterpret_cast<uintptr_t>(sv->d) % 16)
        return fail(QF_ERR_INVALID_ARGUMENT, "density matrix storage is not 16-byte aligned");
    uint64_t tile_mask = 31;  // the low five column bits
    for (uint32_t c = 0; c < count; ++c) tile_mask |= (1ULL << qs[c]) | (1ULL << (n + qs[c]));
    // widen to 12 tile bits with the lowest free bits: fewer, larger tiles
    // (per-tile index work and barriers amortised) and longer contiguous runs
    for (uint32_t b = 5; b < 2 * n && __builtin_popcountll(tile_mask) < 12; ++b) tile_mask |= 1ULL << b;
    ChannelTile ct{};
    ct.k = (uint32_t)__builtin_popcountll(tile_mask);
    if (ct.k > 12) return fail(QF_ERR_INVALID_ARGUMENT, "channel group needs %u tile bits", ct.k);
    ct.n_hi = ct.k - 5;
    const uint64_t all = (2 * n >= 64) ? ~0ULL : ((1ULL << (2 * n)) - 1);
    ct.outer_mask = all & ~tile_mask;
    uint32_t pos[64];
    uint32_t local = 0;
    for (uint32_t b = 0; b < 2 * n; ++b)
        if ((tile_mask >> b) & 1ULL) {
            pos[b] = local;
            if (local >= 5) ct.hi_bits[local - 5] = 1ULL << b;
            ++local;
        }
    ct.n_ch = count;
    for (uint32_t c = 0; c < count; ++c) {
        ct.lc[c] = (uint8_t)pos[qs[c]];
        ct.lr[c] = (uint8_t)pos[n + qs[c]];
        const double *k = coefs[c];
        ct.shape[c] = (k[0] == 1.0 && k[1] == 0.0 && k[2] == 0.0 && k[3] == 1.0) ? 2 : 0;
        for (int j = 0; j < 6; ++j) {
            ct.coef[c][j] = k[j];
            ct.coef_f[c][j] = (float)k[j];
        }
    }
    const uint64_t n_tiles = 1ULL << (2 * n - ct.k);
    const bool pairs = sv->dtype == QF_C64 && ct.k == 12 && 2 * n - ct.k <= 24;
    if (pairs) {
        // channels in pairs (they act on disjoint bits and commute); a channel
        // whose column bit is tile bit 0 goes first in its round, so the
        // round's entries i, i + 1 are 16-byte neighbours
        std::vector<uint32_t> order;
        for (uint32_t c = 0; c < count; ++c)
            if (ct.lc[c] == 0) order.push_back(c);
        for (uint32_t c = 0; c < count; ++c)
            if (ct.lc[c] != 0) order.push_back(c);
        ct.n_rounds = (count + 1) / 2;
        for (uint32_t r = 0; r < ct.n_rounds; ++r) {
            const uint32_t c1 = order[2 * r], c2 = 2 * r + 1 < count ? order[2 * r + 1] : 0xFFu;
            ct.rch[r][0] = (uint8_t)c1;
            ct.rch[r][1] = (uint8_t)c2;
            uint32_t P[4] = {ct.lc[c1], ct.lr[c1], 0, 0};
            if (c2 != 0xFFu) {
                P[2] = ct.lc[c2];
                P[3] = ct.lr[c2];
            } else {  // two filler bits, not tile bit 0 (it stays a lane bit)
                uint32_t f = 0;
                for (uint32_t b = 1; b < 12 && f < 2; ++b)
                    if (b != P[0] && b != P[1]) P[2 + f++] = b;
            }
            ct.rwide[r] = P[0] == 0 ? 1 : 0;
            // lane bits: free tile bits, taken in ascending order when their
            // bank-pair vector is independent of those taken (GF(2) basis by
            // leading bit), until four; then the rest in ascending order
            uint32_t taken = (1u << P[0]) | (1u << P[1]) | (1u << P[2]) | (1u << P[3]), nb = 0;
            uint32_t basis[4] = {0, 0, 0, 0};
            for (uint32_t b = 0; b < 12 && nb < 4; ++b) {
                if ((taken >> b) & 1u) continue;
                uint32_t x = dm_swz(1u << b) & 15u;
                for (int h = 3; h >= 0 && x; --h)
                    if ((x >> h) & 1u) {
                        if (!basis[h]) break;
                        x ^= basis[h];
                    }
                if (!x) continue;
                int h = 3;
                while (!((x >> h) & 1u)) --h;
                basis[h] = x;
                ct.rpos[r][nb++] = (uint8_t)b;
                taken |= 1u << b;
            }
            for (uint32_t b = 0; b < 12; ++b)
                if (!((taken >> b) & 1u)) {
                    ct.rpos[r][nb++] = (uint8_t)b;
                    taken |= 1u << b;
                }
            for (uint32_t i = 0; i < 16; ++i) {
                uint32_t off = 0;
                for (uint32_t b = 0; b < 4; ++b)
                    if ((i >> b) & 1u) off |= 1u << P[b];
                ct.roff[r][i] = (uint16_t)dm_swz(off);
            }
        }
    }
    const size_t smem = pairs ? 2 * sizeof(float2) * 4096 + sizeof(uint64_t) * (128 + 3 * 256)
                              : (sv->dtype == QF_C64 ? 8u : 16u) * (size_t(1) << ct.k) + sizeof(uint64_t) * (size_t(1) << ct.n_hi);
    // one wave of resident CTAs (a grid past the resident count leaves a tail
    // wave running on part of the GPU)
    auto grid_of = [&](const void *k, int *grid) -> int {
        int per_sm = 0;
        QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem));
        *grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(n_tiles, (uint64_t)std::max(per_sm, 1) * ctx->sm_count));
        return QF_OK;
    };
    int grid = 1;
    if (pairs) {
        QF_CUDA(cudaFuncSetAttribute(k_dm_channel_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        QF_TRY(grid_of((const void *)k_dm_channel_pairs, &grid));
        k_dm_channel_pairs<<<grid, 256, smem, ctx->stream>>>(static_cast<float2 *>(sv->d), n_tiles, ct);
    } else if (sv->dtype == QF_C64) {
        QF_CUDA(cudaFuncSetAttribute(k_dm_channel_tile<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        QF_TRY(grid_of((const void *)k_dm_channel_tile<float2>, &grid));
        k_dm_channel_tile<float2><<<grid, 256, smem, ctx->stream>>>(static_cast<float2 *>(sv->d), n_tiles, ct);
    } else {
        QF_CUDA(cudaFuncSetAttribute(k_dm_channel_tile<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        QF_TRY(grid_of((const void *)k_dm_channel_tile<double2>, &grid));
        k_dm_channel_tile<double2><<<grid, 256, smem, ctx->stream>>>(static_cast<double2 *>(sv->d), n_tiles, ct);
    }
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

int dm_diag_reduce(qf_sv *sv, uint32_t n, uint32_t q, int mode, double out[2]) {
    qf_ctx *ctx = sv->ctx;
    const uint64_t D = 1ULL << n;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((D + 255) / 256, (uint64_t)ctx->sm_count * 2));
    const size_t bytes = sizeof(double) * 2 * grid;
    QF_TRY(ensure_device(&ctx->ws_red, &ctx->ws_red_bytes, bytes));
    double *d_part = static_cast<double *>(ctx->ws_red);
    if (sv->dtype == QF_C64)
        k_dm_diag<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<const float2 *>(sv->d), n, q, mode, d_part);
    else
        k_dm_diag<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<const double2 *>(sv->d), n, q, mode, d_part);
    QF_CUDA(cudaGetLastError());
    std::vector<double> part(2 * (size_t)grid);
    QF_CUDA(cudaMemcpyAsync(part.data(), d_part, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    out[0] = out[1] = 0.0;
    for (int b = 0; b < grid; ++b) {
        out[0] += part[2 * (size_t)b];
        out[1] += part[2 * (size_t)b + 1];
    }
    return QF_OK;
}

int dm_diagonal(qf_sv *sv, uint32_t n, double *d_out) {
    qf_ctx *ctx = sv->ctx;
    const int grid = grid_for(ctx, 1ULL << n);
    if (sv->dtype == QF_C64) k_dm_diag_out<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<const float2 *>(sv->d), n, d_out);
    else k_dm_diag_out<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<const double2 *>(sv->d), n, d_out);
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

int dm_collapse(qf_sv *sv, uint32_t n, uint32_t q, int outcome, double prob) {
    qf_ctx *ctx = sv->ctx;
    const int grid = grid_for(ctx, sv->dim);
    if (sv->dtype == QF_C64) k_dm_collapse<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), n, q, outcome, prob);
    else k_dm_collapse<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), n, q, outcome, prob);
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

int dm_from_state(qf_sv *dm, uint32_t n, const qf_sv *psi) {
    qf_ctx *ctx = dm->ctx;
    const int grid = grid_for(ctx, dm->dim);
    if (dm->dtype == QF_C64)
        k_dm_outer<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<const float2 *>(psi->d), n, static_cast<float2 *>(dm->d));
    else
        k_dm_outer<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<const double2 *>(psi->d), n, static_cast<double2 *>(dm->d));
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

int dm_maximally_mixed(qf_sv *dm, uint32_t n) {
    qf_ctx *ctx = dm->ctx;
    const int grid = grid_for(ctx, dm->dim);
    if (dm->dtype == QF_C64) k_dm_mixed<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<float2 *>(dm->d), n);
    else k_dm_mixed<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<double2 *>(dm->d), n);
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

}  // namespace qf
