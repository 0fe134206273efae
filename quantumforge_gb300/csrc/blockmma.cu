// blockmma.cu — dense 5-qubit blocks on the tensor cores (tcgen05, 3xTF32).
//
// A plan made with block_qubits = 5 multiplies the gates of each 12-qubit
// tile pass into dense blocks of at most 5 qubits (planner.cpp). Here every
// block becomes a real contraction on the 5th-generation tensor cores: the
// 32 complex amplitudes of a group (the tile indices that differ only in the
// block's 5 bits) are one row of a 128 x 64 real matrix A (row = group, column
// k = 2 j + re/im of local amplitude j), the block's complex 32 x 32 matrix U
// is the real 64 x 64 matrix B with B[2j][2i] = B[2j+1][2i+1] = Re U_ij,
// B[2j+1][2i] = -Im U_ij, B[2j][2i+1] = Im U_ij, and D = A B holds the 128
// groups' outputs (interleaved re/im). One 4096-amplitude tile = 128 groups =
// one M = 128, N = 64, K = 64 product per block.
//
// Precision (complex64 state, FP32 results): A and B are split into a TF32
// head and a TF32 tail, both rounded to nearest (truncating either biased
// every block toward zero: 30-qubit error vs complex128 2e-8 instead of
// 1e-10), and D = Ah Bh + Al Bh + Ah Bl accumulates in FP32 in tensor memory
// (the dropped Al Bl term is below 2^-24 of the product). Each block is 24
// tcgen05.mma instructions of K = 8.
//
// Data path of one CTA (128 threads; thread r owns TMEM lane r = group row r):
//   * the tile streams into a 32 KB staging buffer (16-byte cp.async, one
//     tile ahead, two buffers), indexed by tile index with an XOR swizzle on
//     bits 1..3 (16-byte chunks stay whole);
//   * per block, each thread gathers its row (the block's 5 bits vary) from
//     staging, splits head and tail and writes them to tensor memory as the A
//     operand (tcgen05.st); thread 0 issues the 24 MMAs against the block's B
//     (head and tail, 32 KB, fetched with one cp.async.bulk into shared memory,
//     completion on an mbarrier) and commits them to a second mbarrier;
//   * every thread then reads its 64 outputs (tcgen05.ld) and scatters them
//     back into staging in the same row layout; the next block gathers rows
//     along its own bits (the relayout between blocks);
//   * the finished tile leaves staging in coalesced 16-byte stores.
// Rows are chosen so that the first four row bits reach distinct banks of the
// swizzled staging buffer (conflict-free 8-byte gathers and scatters).
//
// Every wait on an mbarrier is bounded (about two seconds of SM clock); a
// wait that gives up sets an error word that the host reads after the plan,
// the CTA stops issuing work, waits (bounded) for its copies in flight and
// frees its tensor memory before returning.
//
// The reference has no fused or tensor-core path: it applies each gate as its
// own sweep (StateVector::apply, src/lib.rs:1017-1059; one NVRTC kernel launch
// per gate in src/cuda.rs:114-128).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "qf_device.cuh"
#include "qf_internal.h"

namespace qf {
namespace {

constexpr int kMmaThreads = 128;
constexpr uint32_t kTileQ = 12;
constexpr uint32_t kTileAmps = 1u << kTileQ;
constexpr uint32_t kStageBytes = kTileAmps * 8;  // one staging buffer (float2 per amplitude)
constexpr uint32_t kMatFloats = 64 * 64;         // one real 64 x 64 operand
constexpr uint32_t kBlockMatBytes = 2 * kMatFloats * 4;  // head + tail
constexpr uint32_t kTmemCols = 256;
constexpr uint32_t kColD = 0, kColAh = 64, kColAl = 128;
// shared memory map (bytes)
constexpr uint32_t kSmStage0 = 0;
constexpr uint32_t kSmStage1 = kStageBytes;
constexpr uint32_t kSmB = 2 * kStageBytes;
constexpr uint32_t kSmHiOff = kSmB + kBlockMatBytes;    // 128 x u64
constexpr uint32_t kSmBars = kSmHiOff + 128 * 8;        // 2 mbarriers
constexpr uint32_t kSmTmem = kSmBars + 16;              // TMEM base address
constexpr uint32_t kSmFlag = kSmTmem + 4;               // abort flag
constexpr uint32_t kMaxPassBlocks = 64;                 // block descriptors kept in shared memory
constexpr uint32_t kSmDesc = kSmFlag + 12;              // kMaxPassBlocks x 16 bytes
constexpr uint32_t kSmBytes = (kSmDesc + kMaxPassBlocks * 16 + 127) / 128 * 128;

// Instruction descriptor of kind::tf32: D f32 (bits 4-5 = 1), A and B tf32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

struct MmaBlock {
    uint8_t jbit[5];  // tile bit of local amplitude bit i
    uint8_t mbit[7];  // tile bit of row bit r
    uint32_t pad;
};
static_assert(sizeof(MmaBlock) == 16, "MmaBlock layout");

struct MmaPassArgs {
    uint64_t nonlocal_mask;
    uint64_t n_tiles;
    uint32_t n_blocks;
    uint8_t hi_q[8];  // global qubit of tile bit 5 + r (r < 7)
};

// Staging swizzle: tile-index bits 4..11 folded onto bits 1..3.
__host__ __device__ inline uint32_t stage_phys(uint32_t t) {
    const uint32_t h = (t >> 4) & 0xFFu;
#ifdef __CUDA_ARCH__
    const uint32_t s = ((__popc(h & 0xE9u) & 1u) << 1) | ((__popc(h & 0x5Au) & 1u) << 2) | ((__popc(h & 0x74u) & 1u) << 3);
#else
    const uint32_t s = ((__builtin_popcount(h & 0xE9u) & 1u) << 1) | ((__builtin_popcount(h & 0x5Au) & 1u) << 2) |
                       ((__builtin_popcount(h & 0x74u) & 1u) << 3);
#endif
    return t ^ s;
}

// ---- PTX wrappers ----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase of `parity`: false after about two seconds.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try(bar, parity))
        if (clock64() - t0 > (4ll << 30)) return false;
    return true;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// f32 -> tf32, round to nearest (ties away from zero); low 13 bits zero.
__device__ __forceinline__ uint32_t tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// Shared-memory matrix descriptor, K-major without swizzle: 8-row core
// matrices of 16-byte rows; LBO = distance of core matrices along K, SBO =
// along M/N; bit 46 set (descriptor version of this architecture).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %3, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %4, p;\n}\n" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b_desc), "r"(accumulate), "r"(kIdesc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}

#define QF_R8(b) "r"(v[b + 0]), "r"(v[b + 1]), "r"(v[b + 2]), "r"(v[b + 3]), "r"(v[b + 4]), "r"(v[b + 5]), "r"(v[b + 6]), "r"(v[b + 7])
#define QF_W8(b) "=r"(v[b + 0]), "=r"(v[b + 1]), "=r"(v[b + 2]), "=r"(v[b + 3]), "=r"(v[b + 4]), "=r"(v[b + 5]), "=r"(v[b + 6]), "=r"(v[b + 7])
#define QF_LIST64(p)                                                                                                    \
    "{" p "1, " p "2, " p "3, " p "4, " p "5, " p "6, " p "7, " p "8, " p "9, " p "10, " p "11, " p "12, " p "13, " p "14, " \
    p "15, " p "16, " p "17, " p "18, " p "19, " p "20, " p "21, " p "22, " p "23, " p "24, " p "25, " p "26, " p "27, " p  \
    "28, " p "29, " p "30, " p "31, " p "32, " p "33, " p "34, " p "35, " p "36, " p "37, " p "38, " p "39, " p "40, " p    \
    "41, " p "42, " p "43, " p "44, " p "45, " p "46, " p "47, " p "48, " p "49, " p "50, " p "51, " p "52, " p "53, " p    \
    "54, " p "55, " p "56, " p "57, " p "58, " p "59, " p "60, " p "61, " p "62, " p "63, " p "64}"
#define QF_LIST64_0(p)                                                                                                  \
    "{" p "0, " p "1, " p "2, " p "3, " p "4, " p "5, " p "6, " p "7, " p "8, " p "9, " p "10, " p "11, " p "12, " p "13, " \
    p "14, " p "15, " p "16, " p "17, " p "18, " p "19, " p "20, " p "21, " p "22, " p "23, " p "24, " p "25, " p "26, " p  \
    "27, " p "28, " p "29, " p "30, " p "31, " p "32, " p "33, " p "34, " p "35, " p "36, " p "37, " p "38, " p "39, " p    \
    "40, " p "41, " p "42, " p "43, " p "44, " p "45, " p "46, " p "47, " p "48, " p "49, " p "50, " p "51, " p "52, " p    \
    "53, " p "54, " p "55, " p "56, " p "57, " p "58, " p "59, " p "60, " p "61, " p "62, " p "63}"

// 64 consecutive 32-bit columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_st64(uint32_t taddr, const uint32_t (&v)[64]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x64.b32 [%0], " QF_LIST64("%") ";\n" ::"r"(taddr), QF_R8(0), QF_R8(8),
                 QF_R8(16), QF_R8(24), QF_R8(32), QF_R8(40), QF_R8(48), QF_R8(56)
                 : "memory");
}
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&v)[64]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 " QF_LIST64_0("%") ", [%64];\n"
                 : QF_W8(0), QF_W8(8), QF_W8(16), QF_W8(24), QF_W8(32), QF_W8(40), QF_W8(48), QF_W8(56)
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

__global__ void __launch_bounds__(kMmaThreads, 2)
    k_mma_pass(float2 *__restrict__ A, const MmaPassArgs pa, const MmaBlock *__restrict__ blocks,
               const float *__restrict__ mats, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    float2 *stage[2] = {reinterpret_cast<float2 *>(sm + kSmStage0), reinterpret_cast<float2 *>(sm + kSmStage1)};
    uint64_t *hi_off = reinterpret_cast<uint64_t *>(sm + kSmHiOff);
    volatile uint32_t *tslot = reinterpret_cast<volatile uint32_t *>(sm + kSmTmem);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + kSmFlag);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t bar_b = smem_u32(sm + kSmBars), bar_m = smem_u32(sm + kSmBars + 8);
    const uint32_t sB = smem_u32(sm + kSmB);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(sm + kSmTmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(bar_b, 1);
        mbar_init(bar_m, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    for (uint32_t h = tid; h < 128; h += kMmaThreads) {
        uint64_t off = 0;
        for (uint32_t r = 0; r < 7; ++r)
            if ((h >> r) & 1u) off |= 1ULL << pa.hi_q[r];
        hi_off[h] = off;
    }
    MmaBlock *sblocks = reinterpret_cast<MmaBlock *>(sm + kSmDesc);
    for (uint32_t b = tid; b < pa.n_blocks; b += kMmaThreads) sblocks[b] = blocks[b];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t lane_base = (warp * 32u) << 16;  // this warp's TMEM lanes
    const uint32_t nb = pa.n_blocks;
    uint32_t ph_b = 0, ph_m = 0;
    bool b_pending = false;  // a B load is in flight (thread 0's view)
    bool ok = true;

    auto issue_tile = [&](uint64_t t, float2 *dst) {
        const uint64_t base = deposit(t, pa.nonlocal_mask);
        const uint32_t sdst = smem_u32(dst);
#pragma unroll 4
        for (uint32_t k = 0; k < kTileAmps / 2 / kMmaThreads; ++k) {
            const uint32_t ti = 2u * (tid + kMmaThreads * k);
            cp_async16(sdst + stage_phys(ti) * 8u, A + (base | hi_off[ti >> 5] | (ti & 31u)));
        }
    };
    auto issue_b = [&](uint32_t b) {  // thread 0
        mbar_expect_tx(bar_b, kBlockMatBytes);
        bulk_g2s(sB, mats + (size_t)b * 2 * kMatFloats, kBlockMatBytes, bar_b);
        b_pending = true;
    };

    uint64_t t = blockIdx.x;
    int cur = 0;
    if (t < pa.n_tiles) {
        issue_tile(t, stage[0]);
        if (tid == 0) issue_b(0);
    }
    cp_async_commit();
    for (; t < pa.n_tiles && ok; t += gridDim.x) {
        const uint64_t t2 = t + gridDim.x;
        if (t2 < pa.n_tiles) issue_tile(t2, stage[cur ^ 1]);
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();
        float2 *S = stage[cur];
        for (uint32_t b = 0; b < nb; ++b) {
            const MmaBlock blk = sblocks[b];
            // this thread's row (group) and the swizzled offsets of its 32 amplitudes
            uint32_t tm = 0;
#pragma unroll
            for (int i = 0; i < 7; ++i) tm |= ((tid >> i) & 1u) << blk.mbit[i];
            const uint32_t pm = stage_phys(tm);
            uint32_t q[5];
#pragma unroll
            for (int i = 0; i < 5; ++i) q[i] = stage_phys(1u << blk.jbit[i]);
            {
                uint32_t v[64];
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    uint32_t pj = pm;
#pragma unroll
                    for (int i = 0; i < 5; ++i)
                        if ((j >> i) & 1) pj ^= q[i];
                    const float2 x = S[pj];
                    v[2 * j] = __float_as_uint(x.x);
                    v[2 * j + 1] = __float_as_uint(x.y);
                }
                uint32_t lo[64];
#pragma unroll
                for (int e = 0; e < 64; ++e) {  // head and tail both rounded to nearest: unbiased
                    const float x = __uint_as_float(v[e]);
                    const uint32_t h = tf32_rna(x) & 0xFFFFE000u;
                    lo[e] = tf32_rna(x - __uint_as_float(h)) & 0xFFFFE000u;
                    v[e] = h;
                }
                tmem_st64(tmem + lane_base + kColAh, v);
                tmem_st64(tmem + lane_base + kColAl, lo);
                tmem_wait_st();
            }
            tc_fence_before();
            __syncthreads();
            if (tid == 0) {
                if (!mbar_wait(bar_b, ph_b)) {  // the block's matrix never arrived
                    atomicExch(err, 1);
                    *abort_flag = 1;
                    mbar_arrive(bar_m);  // release the others
                } else {
                    b_pending = false;
                    tc_fence_after();
                    const uint32_t d = tmem + kColD;
#pragma unroll
                    for (uint32_t s = 0; s < 8; ++s)
                        mma_tf32(d, tmem + kColAh + 8 * s, smem_desc(sB + 256 * s, 128, 2048), s > 0);
#pragma unroll
                    for (uint32_t s = 0; s < 8; ++s)
                        mma_tf32(d, tmem + kColAl + 8 * s, smem_desc(sB + 256 * s, 128, 2048), 1);
#pragma unroll
                    for (uint32_t s = 0; s < 8; ++s)
                        mma_tf32(d, tmem + kColAh + 8 * s, smem_desc(sB + 4 * kMatFloats + 256 * s, 128, 2048), 1);
                    mma_commit(bar_m);
                }
            }
            ph_b ^= 1u;
            int bad = tid == 0 && *abort_flag;
            if (!mbar_wait(bar_m, ph_m)) {
                atomicExch(err, 2);
                bad = 1;
            }
            ph_m ^= 1u;
            tc_fence_after();
            if (__syncthreads_or(bad)) {  // every thread leaves together
                ok = false;
                break;
            }
            // the MMAs are done with B: fetch the next block's (or the next tile's first)
            if (tid == 0 && (b + 1 < nb || t2 < pa.n_tiles)) issue_b(b + 1 < nb ? b + 1 : 0);
            {
                uint32_t v[64];
                tmem_ld64(tmem + lane_base + kColD, v);
                tmem_wait_ld();
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    uint32_t pj = pm;
#pragma unroll
                    for (int i = 0; i < 5; ++i)
                        if ((j >> i) & 1) pj ^= q[i];
                    S[pj] = make_float2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
                }
            }
            tc_fence_before();
            __syncthreads();
        }
        if (!ok) break;
        // the finished tile to global memory, 16-byte chunks
        {
            const uint64_t base = deposit(t, pa.nonlocal_mask);
#pragma unroll 4
            for (uint32_t k = 0; k < kTileAmps / 2 / kMmaThreads; ++k) {
                const uint32_t ti = 2u * (tid + kMmaThreads * k);
                *reinterpret_cast<float4 *>(A + (base | hi_off[ti >> 5] | (ti & 31u))) =
                    *reinterpret_cast<const float4 *>(S + stage_phys(ti));
            }
        }
        __syncthreads();
        cur ^= 1;
    }
    // leave nothing in flight: tile prefetches, a B load (bounded), then free TMEM
    cp_async_wait<0>();
    if (tid == 0 && b_pending && !mbar_wait(bar_b, ph_b)) atomicExch(err, 3);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// ---- host: lowering a block plan to 5-qubit tensor-core blocks -------------
using cd = std::complex<double>;

struct MmaPlan {
    std::vector<MmaPassArgs> passes;
    std::vector<uint32_t> block_begin;  // per pass, into blocks
    std::vector<MmaBlock> blocks;
    std::vector<float> mats;  // per block: head then tail, each the canonical 64 x 64 layout
};

uint32_t bank_vec(uint32_t s) { return stage_phys(1u << s) & 15u; }

// Row bits of a block: the four lane bits of each half warp first, chosen to
// reach independent bank vectors of the staging swizzle, then the rest.
void choose_rows(const uint8_t jbit[5], uint8_t mbit[7]) {
    std::vector<uint32_t> free_bits;
    for (uint32_t s = 0; s < kTileQ; ++s)
        if (std::find(jbit, jbit + 5, (uint8_t)s) == jbit + 5) free_bits.push_back(s);
    std::vector<uint32_t> basis, order;
    auto reduce = [&](uint32_t v) {
        for (uint32_t b : basis) v = std::min(v, v ^ b);
        return v;
    };
    std::vector<bool> used(free_bits.size(), false);
    for (int c = 0; c < 4; ++c) {
        int pick = -1;
        for (size_t i = 0; i < free_bits.size() && pick < 0; ++i)
            if (!used[i] && reduce(bank_vec(free_bits[i]))) pick = (int)i;
        if (pick < 0) break;
        used[pick] = true;
        basis.push_back(reduce(bank_vec(free_bits[pick])));
        order.push_back(free_bits[pick]);
    }
    for (size_t i = 0; i < free_bits.size(); ++i)
        if (!used[i]) order.push_back(free_bits[i]);
    for (int i = 0; i < 7; ++i) mbit[i] = (uint8_t)order[i];
}

// w rounded to TF32 (nearest, ties away from zero), as a float.
float tf32_rn(double w) {
    float f = (float)w;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    std::memcpy(&f, &u, 4);
    return f;
}

// The real 64 x 64 operand of a complex 32 x 32 block (row n = output
// component, column k = input component) in the canonical K-major layout
// without swizzle: byte (n / 8) * 2048 + (k / 4) * 128 + (n % 8) * 16 + (k % 4) * 4.
void pack_block(const std::vector<cd> &U, float *head, float *tail) {
    for (int n = 0; n < 64; ++n)
        for (int k = 0; k < 64; ++k) {
            const int i = n >> 1, j = k >> 1;
            const cd u = U[(size_t)i * 32 + j];
            double w;
            if ((n & 1) == 0) w = (k & 1) == 0 ? u.real() : -u.imag();
            else w = (k & 1) == 0 ? u.imag() : u.real();
            const size_t at = (size_t)(n >> 3) * 512 + (size_t)(k >> 2) * 32 + (size_t)(n & 7) * 4 + (size_t)(k & 3);
            head[at] = tf32_rn(w);
            tail[at] = tf32_rn(w - (double)head[at]);
        }
}

// Each pass's gates and blocks (in order) as 5-qubit blocks: consecutive
// items merge while their qubits fit in five; a block of fewer qubits is
// padded with high tile bits (identity there).
int lower_mma(const Plan &plan, MmaPlan &out) {
    out = MmaPlan();
    for (const Pass &p : plan.passes) {
        MmaPassArgs a;
        std::memset(&a, 0, sizeof a);
        a.nonlocal_mask = p.a.nonlocal_mask;
        a.n_tiles = p.a.n_tiles;
        int slot_of[64];
        std::vector<uint32_t> slot_q;
        for (uint32_t q = 0; q < plan.n; ++q)
            if ((p.resident >> q) & 1ULL) {
                slot_of[q] = (int)slot_q.size();
                slot_q.push_back(q);
            }
        for (int r = 0; r < 7; ++r) a.hi_q[r] = (uint8_t)slot_q[5 + r];  // tile bits 5..11
        out.block_begin.push_back((uint32_t)out.blocks.size());
        std::vector<uint32_t> cq;  // current block's qubits (ascending)
        std::vector<cd> cm;
        auto emit = [&]() {
            if (cq.empty()) return;
            std::vector<uint32_t> nq = cq;
            for (int s = (int)kTileQ - 1; s >= 0 && nq.size() < 5; --s)
                if (std::find(nq.begin(), nq.end(), slot_q[s]) == nq.end()) nq.push_back(slot_q[s]);
            std::sort(nq.begin(), nq.end());
            const std::vector<cd> U = nq.size() == cq.size() ? cm : widen_matrix(cq, cm, nq);
            MmaBlock mb;
            std::memset(&mb, 0, sizeof mb);
            for (int i = 0; i < 5; ++i) mb.jbit[i] = (uint8_t)slot_of[nq[i]];
            choose_rows(mb.jbit, mb.mbit);
            out.blocks.push_back(mb);
            const size_t at = out.mats.size();
            out.mats.resize(at + 2 * kMatFloats);
            pack_block(U, &out.mats[at], &out.mats[at + kMatFloats]);
            cq.clear();
            cm.clear();
        };
        for (const BGate &g : p.gates) {
            if (g.kind == BK_OVL) return fail(QF_ERR_UNSUPPORTED_OPERATION, "tensor-core passes run forward plans only");
            std::vector<uint32_t> gq;
            std::vector<cd> gm;
            if (g.kind == BK_BLOCK) {
                dense_matrix(g, plan.bmats, gq, gm);
            } else {
                gq.push_back(g.q0);
                if (g.kind != BK_MAT1) gq.push_back(g.q1);
                std::sort(gq.begin(), gq.end());
            }
            for (uint32_t q : gq)
                if (!((p.resident >> q) & 1ULL)) return fail(QF_ERR_UNSUPPORTED_OPERATION, "block qubit outside the tile");
            std::vector<uint32_t> un = cq;
            for (uint32_t q : gq)
                if (std::find(un.begin(), un.end(), q) == un.end()) un.push_back(q);
            std::sort(un.begin(), un.end());
            if (un.size() > 5) {
                emit();
                un = gq;
            }
            if (cq.empty()) {
                cq = un;
                const size_t d = (size_t)1 << cq.size();
                cm.assign(d * d, cd(0.0, 0.0));
                for (size_t i = 0; i < d; ++i) cm[i * d + i] = 1.0;
            } else if (un.size() != cq.size()) {
                cm = widen_matrix(cq, cm, un);
                cq = un;
            }
            if (g.kind == BK_BLOCK) {  // cm <- G cm (G widened to the block's qubits)
                const std::vector<cd> G = gq.size() == cq.size() ? gm : widen_matrix(gq, gm, cq);
                const size_t d = (size_t)1 << cq.size();
                std::vector<cd> P(d * d, cd(0.0, 0.0));
                for (size_t r = 0; r < d; ++r)
                    for (size_t t = 0; t < d; ++t) {
                        const cd w = G[r * d + t];
                        if (w == cd(0.0, 0.0)) continue;
                        for (size_t c = 0; c < d; ++c) P[r * d + c] += w * cm[t * d + c];
                    }
                cm.swap(P);
            } else {
                apply_gate_to_matrix(cq, cm, g);
            }
        }
        emit();
        a.n_blocks = (uint32_t)(out.blocks.size() - out.block_begin.back());
        if (a.n_blocks > kMaxPassBlocks)
            return fail(QF_ERR_UNSUPPORTED_OPERATION, "a pass of %u tensor-core blocks (at most %u)", a.n_blocks, kMaxPassBlocks);
        out.passes.push_back(a);
    }
    return QF_OK;
}

struct MmaCache {
    std::mutex mu;
    std::vector<uint8_t> key;  // the last plan's structure and matrices
    MmaPlan plan;
};
MmaCache &mma_cache() {
    static MmaCache c;
    return c;
}

// Everything that shapes the lowered blocks: passes' resident sets, gates
// (kind, qubits, 2x2 matrices) and the block matrices.
void mma_key(const Plan &plan, std::vector<uint8_t> &k) {
    auto put = [&](const void *p, size_t n) {
        const uint8_t *b = static_cast<const uint8_t *>(p);
        k.insert(k.end(), b, b + n);
    };
    put(&plan.n, sizeof plan.n);
    for (const Pass &p : plan.passes) {
        put(&p.resident, 8);
        put(&p.a.nonlocal_mask, 8);
        for (const BGate &g : p.gates) {
            put(&g.kind, 1);
            put(&g.q0, 4);
            put(&g.q1, 4);
            put(g.m, sizeof g.m);
            put(&g.nq, 1);
            put(g.bq, sizeof g.bq);
            put(&g.boff, 4);
        }
    }
    put(plan.bmats.data(), plan.bmats.size() * sizeof(double));
}

}  // namespace

// A block plan the tensor-core pass can run: blocks of 5 on 12-qubit tiles
// whose low five bits are qubits 0..4 (256-byte contiguous runs).
bool mma_blocks_fit(const Plan &plan) {
    if (plan.block_qubits != 5 || plan.n < kTileQ || plan.passes.empty()) return false;
    for (const Pass &p : plan.passes)
        if (p.a.k != kTileQ || p.a.low < 5 || (p.resident & 31ULL) != 31ULL) return false;
    return true;
}

int run_plan_blocks_mma(qf_sv *sv, const Plan &plan) {
    if (sv->dtype != QF_C64 || !mma_blocks_fit(plan)) return run_plan_blocks(sv, plan);
    qf_ctx *ctx = sv->ctx;
    static bool attr_set[64] = {false};
    const int dev = ctx->device & 63;
    if (!attr_set[dev]) {
        QF_CUDA(cudaFuncSetAttribute(k_mma_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmBytes));
        attr_set[dev] = true;
    }
    // lowered blocks: cached for the last plan (a circuit applied again and again)
    std::vector<uint8_t> key;
    mma_key(plan, key);
    MmaCache &mc = mma_cache();
    std::lock_guard<std::mutex> lk(mc.mu);
    if (key != mc.key) {
        QF_TRY(lower_mma(plan, mc.plan));
        mc.key.swap(key);
    }
    const MmaPlan &mp = mc.plan;
    const size_t blocks_bytes = (mp.blocks.size() * sizeof(MmaBlock) + 255) / 256 * 256;
    const size_t mats_bytes = mp.mats.size() * sizeof(float);
    QF_TRY(ensure_device(&ctx->ws_plan, &ctx->ws_plan_bytes, 256 + blocks_bytes + mats_bytes));
    unsigned char *d = static_cast<unsigned char *>(ctx->ws_plan);
    int *d_err = reinterpret_cast<int *>(d);
    MmaBlock *d_blocks = reinterpret_cast<MmaBlock *>(d + 256);
    float *d_mats = reinterpret_cast<float *>(d + 256 + blocks_bytes);
    QF_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
    if (!mp.blocks.empty())
        QF_CUDA(cudaMemcpyAsync(d_blocks, mp.blocks.data(), mp.blocks.size() * sizeof(MmaBlock), cudaMemcpyHostToDevice,
                                ctx->stream));
    if (mats_bytes) QF_CUDA(cudaMemcpyAsync(d_mats, mp.mats.data(), mats_bytes, cudaMemcpyHostToDevice, ctx->stream));
    // two CTAs per SM: together they hold all 512 TMEM columns, and one
    // CTA's gathers and scatters overlap the other's MMAs (the occupancy
    // query answered one here, although two fit by registers and shared
    // memory, as the launch's own occupancy limits show)
    int smem_sm = 0, regs_sm = 0;
    QF_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device));
    QF_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, ctx->device));
    cudaFuncAttributes fa;
    QF_CUDA(cudaFuncGetAttributes(&fa, k_mma_pass));
    const int regs_cta = ((fa.numRegs + 7) / 8) * 8 * kMmaThreads;
    int per_sm = std::min(smem_sm / (int)(kSmBytes + 1024), regs_sm / std::max(1, regs_cta));
    per_sm = std::min(std::max(per_sm, 1), 2);
    const uint64_t grid_max = (uint64_t)per_sm * (uint64_t)ctx->sm_count;
    for (size_t i = 0; i < mp.passes.size(); ++i) {
        const MmaPassArgs &a = mp.passes[i];
        if (!a.n_blocks) continue;
        const unsigned grid = (unsigned)std::min<uint64_t>(grid_max, a.n_tiles);
        k_mma_pass<<<grid, kMmaThreads, kSmBytes, ctx->stream>>>(static_cast<float2 *>(sv->d), a,
                                                                  d_blocks + mp.block_begin[i],
                                                                  d_mats + (size_t)mp.block_begin[i] * 2 * kMatFloats, d_err);
        QF_CUDA(cudaGetLastError());
    }
    int h_err = 0;
    QF_CUDA(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    if (h_err)
        return fail(QF_ERR_TIMEOUT, "tensor-core block pass gave up waiting (%s)",
                    h_err == 1 ? "block matrix copy" : h_err == 2 ? "MMA completion" : "copy in flight at exit");
    return QF_OK;
}

}  // namespace qf
