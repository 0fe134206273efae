// reduce.cu — reductions over a resident state: norm, probabilities, <Z_q>
// for every qubit in one pass, one-qubit X/Y/Z expectations, measurement
// probability and collapse, Pauli-sum expectations and lambda = H psi.
//
// Every sum is accumulated in f64 from the first block-level partial on;
// complex64 states form the per-thread partial over a short contiguous chunk
// (8-16 amplitudes) in f32 first. Two-stage reductions write one partial per
// block and sum the partials in block order, so results are deterministic.
#include <algorithm>
#include <cstring>
#include <map>

#include "qf_device.cuh"
#include "qf_internal.h"

namespace qf {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 512;  // power of two: the <Z> kernel reads index bits from the thread id

// Sum `n_vals` values per block over `n_blocks` blocks, in block order.
// out[v] = sum over blocks of partials[b * n_vals + v]: one block, every
// thread adds a fixed strided subset, then a block reduction (the same order
// on every run, so results are reproducible).
__global__ void k_final_sum(const double *__restrict__ partials, uint32_t n_blocks, uint32_t n_vals,
                            double *__restrict__ out) {
    __shared__ double red[32];
    for (uint32_t v = 0; v < n_vals; ++v) {
        double s = 0.0;
        for (uint32_t b = threadIdx.x; b < n_blocks; b += blockDim.x) s += partials[(size_t)b * n_vals + v];
        s = block_sum(s, red);
        if (threadIdx.x == 0) out[v] = s;
        __syncthreads();
    }
}

static int finish_sum(qf_ctx *ctx, const double *d_partials, uint32_t n_blocks, uint32_t n_vals, double *host_out) {
    k_final_sum<<<1, 256, 0, ctx->stream>>>(d_partials, n_blocks, n_vals, ctx->d_small);
    QF_CUDA(cudaGetLastError());
    QF_CUDA(cudaMemcpyAsync(ctx->h_small, ctx->d_small, sizeof(double) * n_vals, cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    std::copy(ctx->h_small, ctx->h_small + n_vals, host_out);
    return QF_OK;
}

static int partials_buffer(qf_ctx *ctx, size_t doubles, double **out) {
    QF_TRY(ensure_device(&ctx->ws_red, &ctx->ws_red_bytes, doubles * sizeof(double)));
    *out = static_cast<double *>(ctx->ws_red);
    return QF_OK;
}

template <typename C> __device__ __forceinline__ typename Real<C>::T nsq(C a) { return a.x * a.x + a.y * a.y; }

// ---- state fill / conversion ---------------------------------------------
template <typename C> __global__ void k_set_first_one(C *a) { a[0] = mk((typename Real<C>::T)1, (typename Real<C>::T)0); }

int fill_zero_state(qf_sv *sv) {
    QF_CUDA(cudaMemsetAsync(sv->d, 0, sv->bytes(), sv->ctx->stream));
    if (sv->dtype == QF_C64) k_set_first_one<float2><<<1, 1, 0, sv->ctx->stream>>>(static_cast<float2 *>(sv->d));
    else k_set_first_one<double2><<<1, 1, 0, sv->ctx->stream>>>(static_cast<double2 *>(sv->d));
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

__global__ void k_f64_to_c64(const double2 *__restrict__ src, float2 *__restrict__ dst, uint64_t count) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        const double2 v = src[i];
        dst[i] = make_float2((float)v.x, (float)v.y);
    }
}
__global__ void k_c64_to_f64(const float2 *__restrict__ src, double2 *__restrict__ dst, uint64_t count) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        const float2 v = src[i];
        dst[i] = make_double2((double)v.x, (double)v.y);
    }
}

// Device address of a page-locked host buffer (the kernels then read or write
// it directly over the host link, no staging), or nullptr for pageable memory.
static const void *pinned_device_ptr(const void *host) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return pa.type == cudaMemoryTypeHost ? pa.devicePointer : nullptr;
}

// Host f64 amplitudes -> device state: a conversion kernel reading a pinned
// host buffer directly, else chunks through a device staging buffer.
int convert_from_f64(qf_sv *sv, const double *host) {
    qf_ctx *ctx = sv->ctx;
    // the caller may reuse `host` once this returns: finish reading it first
    if (sv->dtype == QF_C128) {
        QF_CUDA(cudaMemcpyAsync(sv->d, host, sv->bytes(), cudaMemcpyHostToDevice, ctx->stream));
        QF_CUDA(cudaStreamSynchronize(ctx->stream));
        return QF_OK;
    }
    if (const void *dp = pinned_device_ptr(host)) {
        k_f64_to_c64<<<(unsigned)std::max(1, ctx->sm_count) * 8, 256, 0, ctx->stream>>>(static_cast<const double2 *>(dp),
                                                                                        static_cast<float2 *>(sv->d), sv->dim);
        QF_CUDA(cudaGetLastError());
        QF_CUDA(cudaStreamSynchronize(ctx->stream));
        return QF_OK;
    }
    const uint64_t chunk = std::min<uint64_t>(sv->dim, 1ULL << 24);  // amplitudes per chunk (256 MiB staging)
    QF_TRY(ensure_device(&ctx->ws_stage, &ctx->ws_stage_bytes, chunk * 16));
    for (uint64_t off = 0; off < sv->dim; off += chunk) {
        const uint64_t cnt = std::min(chunk, sv->dim - off);
        QF_CUDA(cudaMemcpyAsync(ctx->ws_stage, host + 2 * off, cnt * 16, cudaMemcpyHostToDevice, ctx->stream));
        k_f64_to_c64<<<std::max<uint64_t>(1, std::min<uint64_t>((cnt + 255) / 256, 4096)), 256, 0, ctx->stream>>>(
            static_cast<const double2 *>(ctx->ws_stage), static_cast<float2 *>(sv->d) + off, cnt);
        QF_CUDA(cudaGetLastError());
    }
    return QF_OK;
}

int convert_to_f64(qf_sv *sv, double *host) {
    qf_ctx *ctx = sv->ctx;
    if (sv->dtype == QF_C128) {
        QF_CUDA(cudaMemcpyAsync(host, sv->d, sv->bytes(), cudaMemcpyDeviceToHost, ctx->stream));
        QF_CUDA(cudaStreamSynchronize(ctx->stream));
        return QF_OK;
    }
    if (void *dp = const_cast<void *>(pinned_device_ptr(host))) {
        k_c64_to_f64<<<(unsigned)std::max(1, ctx->sm_count) * 8, 256, 0, ctx->stream>>>(static_cast<const float2 *>(sv->d),
                                                                                        static_cast<double2 *>(dp), sv->dim);
        QF_CUDA(cudaGetLastError());
        QF_CUDA(cudaStreamSynchronize(ctx->stream));
        return QF_OK;
    }
    const uint64_t chunk = std::min<uint64_t>(sv->dim, 1ULL << 24);
    QF_TRY(ensure_device(&ctx->ws_stage, &ctx->ws_stage_bytes, chunk * 16));
    for (uint64_t off = 0; off < sv->dim; off += chunk) {
        const uint64_t cnt = std::min(chunk, sv->dim - off);
        k_c64_to_f64<<<std::max<uint64_t>(1, std::min<uint64_t>((cnt + 255) / 256, 4096)), 256, 0, ctx->stream>>>(
            static_cast<const float2 *>(sv->d) + off, static_cast<double2 *>(ctx->ws_stage), cnt);
        QF_CUDA(cudaGetLastError());
        QF_CUDA(cudaMemcpyAsync(host + 2 * off, ctx->ws_stage, cnt * 16, cudaMemcpyDeviceToHost, ctx->stream));
    }
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    return QF_OK;
}

// ---- norm / probabilities --------------------------------------------------
template <typename C>
__global__ void k_norm(const C *__restrict__ a, uint64_t dim, double *__restrict__ partials) {
    __shared__ double red[32];
    double s = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x)
        s += (double)nsq(a[i]);
    s = block_sum(s, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

int reduce_norm_sqr(qf_sv *sv, double *out) {
    qf_ctx *ctx = sv->ctx;
    double *p;
    QF_TRY(partials_buffer(ctx, kRedBlocks, &p));
    if (sv->dtype == QF_C64) k_norm<float2><<<kRedBlocks, kRedThreads, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), sv->dim, p);
    else k_norm<double2><<<kRedBlocks, kRedThreads, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), sv->dim, p);
    QF_CUDA(cudaGetLastError());
    return finish_sum(ctx, p, kRedBlocks, 1, out);
}

// StateVector::probabilities (src/lib.rs:1144-1146): |a_i|^2 per index.
template <typename C>
__global__ void k_probs(const C *__restrict__ a, uint64_t dim, double *__restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x) {
        const C v = a[i];
        out[i] = (double)v.x * (double)v.x + (double)v.y * (double)v.y;
    }
}

int reduce_probabilities(qf_sv *sv, double *d_out) {
    qf_ctx *ctx = sv->ctx;
    const int grid = std::max(1, std::min<int>((int)((sv->dim + 255) / 256), ctx->sm_count * 8));
    if (sv->dtype == QF_C64) k_probs<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), sv->dim, d_out);
    else k_probs<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), sv->dim, d_out);
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

// ---- <Z_q> for every qubit in one HBM pass --------------------------------
// Each thread takes chunks of 2^CH contiguous amplitudes. Inside a chunk the
// per-bit sums of bits < CH are a small tree; bits CH..CH+S-1 (S = log2 of the
// total thread count) are fixed by the thread id; the higher bits are fixed
// per loop iteration and take the chunk total. partials[block][q] holds the
// sum of p over indices with bit q set; partials[block][n] the total.
template <typename C, int CH>
__global__ void __launch_bounds__(kRedThreads)
    k_expect_z_all(const C *__restrict__ a, uint32_t n, uint32_t s_log, double *__restrict__ partials) {
    using R = typename Real<C>::T;
    __shared__ double red[32];
    const uint64_t gtid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t stride = 1ULL << s_log;
    const uint64_t nchunks = 1ULL << (n - CH);
    double tot = 0.0, lowsum[CH], hisum[64];
#pragma unroll
    for (int b = 0; b < CH; ++b) lowsum[b] = 0.0;
    const uint32_t nhi = n > CH + s_log ? n - CH - s_log : 0;
    for (uint32_t r = 0; r < nhi; ++r) hisum[r] = 0.0;
    uint64_t it = 0;
    for (uint64_t c = gtid; c < nchunks; c += stride, ++it) {
        R p[1 << CH];
        const C *src = a + (c << CH);
#pragma unroll
        for (int j = 0; j < (1 << CH); ++j) p[j] = nsq(src[j]);
        R t = 0;
#pragma unroll
        for (int j = 0; j < (1 << CH); ++j) t += p[j];
        tot += (double)t;
#pragma unroll
        for (int b = 0; b < CH; ++b) {
            R s = 0;
#pragma unroll
            for (int j = 0; j < (1 << CH); ++j)
                if ((j >> b) & 1) s += p[j];
            lowsum[b] += (double)s;
        }
        for (uint32_t r = 0; r < nhi; ++r)
            if ((it >> r) & 1ULL) hisum[r] += (double)t;
    }
    for (uint32_t q = 0; q <= n; ++q) {
        double v;
        if (q == n) v = tot;
        else if (q < CH) v = lowsum[q];
        else if (q < CH + s_log) v = ((gtid >> (q - CH)) & 1ULL) ? tot : 0.0;
        else v = hisum[q - CH - s_log];
        v = block_sum(v, red);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * (n + 1) + q] = v;
    }
}

// Tiny states: one thread.
template <typename C>
__global__ void k_expect_z_small(const C *__restrict__ a, uint32_t n, double *__restrict__ partials) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[65];
    for (uint32_t q = 0; q <= n; ++q) s[q] = 0.0;
    for (uint64_t i = 0; i < (1ULL << n); ++i) {
        const double p = (double)a[i].x * (double)a[i].x + (double)a[i].y * (double)a[i].y;
        s[n] += p;
        for (uint32_t q = 0; q < n; ++q)
            if ((i >> q) & 1ULL) s[q] += p;
    }
    for (uint32_t q = 0; q <= n; ++q) partials[q] = s[q];
}

int reduce_expect_z_all(qf_sv *sv, double *out) {
    qf_ctx *ctx = sv->ctx;
    const uint32_t n = sv->n;
    double *p;
    QF_TRY(partials_buffer(ctx, (size_t)kRedBlocks * (n + 1), &p));
    uint32_t blocks = 1;
    const int ch = sv->dtype == QF_C64 ? 4 : 3;
    if ((int)n < ch + 5) {
        if (sv->dtype == QF_C64) k_expect_z_small<float2><<<1, 32, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), n, p);
        else k_expect_z_small<double2><<<1, 32, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), n, p);
    } else {
        // threads = min(kRedBlocks * kRedThreads, chunks), a power of two
        uint32_t s_log = 0;
        const uint32_t max_log = 17;  // log2(kRedBlocks * kRedThreads)
        s_log = std::min<uint32_t>(max_log, n - ch);
        const uint32_t threads_total = 1u << s_log;
        const uint32_t tpb = std::min<uint32_t>(kRedThreads, threads_total);
        blocks = threads_total / tpb;
        if (sv->dtype == QF_C64)
            k_expect_z_all<float2, 4><<<blocks, tpb, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), n, s_log, p);
        else
            k_expect_z_all<double2, 3><<<blocks, tpb, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), n, s_log, p);
    }
    QF_CUDA(cudaGetLastError());
    std::vector<double> sums(n + 1);
    QF_TRY(finish_sum(ctx, p, blocks, n + 1, sums.data()));
    for (uint32_t q = 0; q < n; ++q) out[q] = sums[n] - 2.0 * sums[q];
    return QF_OK;
}

// ---- one-qubit expectations, P(q = 1), collapse --------------------------
// mode 0: 2 sum Re(conj(a0) a1) (<X>), 1: 2 sum Im(conj(a0) a1) (<Y>),
// 2: sum |a0|^2 - |a1|^2 (<Z>), 3: sum |a1|^2 (P(q=1)); a0/a1 = bit clear/set.
template <typename C>
__global__ void k_pair_reduce(const C *__restrict__ a, uint64_t n_pairs, uint32_t q, int mode,
                              double *__restrict__ partials) {
    __shared__ double red[32];
    const uint64_t mask = 1ULL << q;
    double s = 0.0;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n_pairs; p += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i0 = insert0(p, q);
        const C a0 = a[i0], a1 = a[i0 | mask];
        double v;
        if (mode == 0) v = 2.0 * ((double)a0.x * a1.x + (double)a0.y * a1.y);
        else if (mode == 1) v = 2.0 * ((double)a0.x * a1.y - (double)a0.y * a1.x);
        else if (mode == 2) v = ((double)a0.x * a0.x + (double)a0.y * a0.y) - ((double)a1.x * a1.x + (double)a1.y * a1.y);
        else v = (double)a1.x * a1.x + (double)a1.y * a1.y;
        s += v;
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

static int pair_reduce(qf_sv *sv, uint32_t q, int mode, double *out) {
    qf_ctx *ctx = sv->ctx;
    double *p;
    QF_TRY(partials_buffer(ctx, kRedBlocks, &p));
    const uint64_t pairs = sv->dim / 2;
    const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(kRedBlocks, (pairs + 255) / 256));
    if (sv->dtype == QF_C64)
        k_pair_reduce<float2><<<blocks, kRedThreads, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), pairs, q, mode, p);
    else
        k_pair_reduce<double2><<<blocks, kRedThreads, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), pairs, q, mode, p);
    QF_CUDA(cudaGetLastError());
    return finish_sum(ctx, p, blocks, 1, out);
}

int reduce_expect_1q(qf_sv *sv, int obs, uint32_t q, double *out) {
    const int mode = obs == QF_PAULI_X ? 0 : obs == QF_PAULI_Y ? 1 : 2;
    return pair_reduce(sv, q, mode, out);
}

int reduce_p_one(qf_sv *sv, uint32_t q, double *out) { return pair_reduce(sv, q, 3, out); }

// Collapse after measure (src/lib.rs:1341-1350): amplitudes whose bit differs
// from the outcome become 0, the others are divided by `scale`. outcome < 0
// divides every amplitude (StateVector::normalize, src/lib.rs:1005-1014).
template <typename C>
__global__ void k_collapse(C *__restrict__ a, uint64_t dim, uint32_t q, int outcome, double scale) {
    using R = typename Real<C>::T;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x) {
        if (outcome >= 0 && (int)((i >> q) & 1ULL) != outcome) a[i] = mk((R)0, (R)0);
        else a[i] = mk((R)((double)a[i].x / scale), (R)((double)a[i].y / scale));
    }
}

int collapse(qf_sv *sv, uint32_t q, int outcome, double scale) {
    qf_ctx *ctx = sv->ctx;
    const int grid = std::max(1, std::min<int>((int)((sv->dim + 255) / 256), ctx->sm_count * 8));
    if (sv->dtype == QF_C64) k_collapse<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), sv->dim, q, outcome, scale);
    else k_collapse<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), sv->dim, q, outcome, scale);
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

// ---- batches of states --------------------------------------------------------
// A batch of B states of 2^n amplitudes is one allocation; state b starts at
// amplitude b << n (CudaDeviceStateBatch, src/cuda.rs:529-540).

// Every state |0...0>, the padding after the last state zero.
template <typename C>
__global__ void k_batch_zero(C *__restrict__ a, uint64_t total, uint32_t n, uint64_t B) {
    using R = typename Real<C>::T;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const bool one = (i & ((1ULL << n) - 1)) == 0 && (i >> n) < B;
        a[i] = mk((R)(one ? 1 : 0), (R)0);
    }
}

int batch_set_zero(qf_sv *sv, uint32_t n, uint64_t B) {
    qf_ctx *ctx = sv->ctx;
    const int grid = std::max(1, std::min<int>((int)((sv->dim + 255) / 256), ctx->sm_count * 8));
    if (sv->dtype == QF_C64) k_batch_zero<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), sv->dim, n, B);
    else k_batch_zero<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), sv->dim, n, B);
    QF_CUDA(cudaGetLastError());
    return QF_OK;
}

// P(1) of qubit q per state: block (b, c) sums chunk c of state b into
// partials[b * chunks + c]; k_batch_finish adds each state's chunks in order.
template <typename C>
__global__ void k_batch_p_one(const C *__restrict__ a, uint32_t n, uint32_t q, uint32_t chunk_log, double *partials) {
    __shared__ double red[32];
    const uint32_t chunks_log = n - chunk_log;
    const uint64_t b = blockIdx.x >> chunks_log, c = blockIdx.x & ((1ULL << chunks_log) - 1);
    const uint64_t base = (b << n) + (c << chunk_log), len = 1ULL << chunk_log;
    double s = 0.0;
    for (uint64_t j = threadIdx.x; j < len; j += blockDim.x) {
        const uint64_t i = base + j;
        if ((i >> q) & 1ULL) {
            const C v = a[i];
            s += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
        }
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void k_batch_finish(const double *__restrict__ partials, uint64_t B, uint32_t chunks, double *out) {
    const uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (b >= B) return;
    double s = 0.0;
    for (uint32_t c = 0; c < chunks; ++c) s += partials[b * chunks + c];
    out[b] = s;
}

// Collapse state b to outcome[b] on qubit q, multiplying the kept amplitudes
// by inv[b] (the batch collapse of src/cuda.rs:1582-1621).
template <typename C>
__global__ void k_batch_collapse(C *__restrict__ a, uint64_t total, uint32_t n, uint32_t q, const uint8_t *__restrict__ outcome,
                                 const double *__restrict__ inv) {
    using R = typename Real<C>::T;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = i >> n;
        if ((uint8_t)((i >> q) & 1ULL) != outcome[b]) {
            a[i] = mk((R)0, (R)0);
        } else {
            const C v = a[i];
            a[i] = mk((R)((double)v.x * inv[b]), (R)((double)v.y * inv[b]));
        }
    }
}

int batch_measure(qf_sv *sv, uint32_t n, uint64_t B, uint32_t q, const double *uniforms, uint8_t *outcomes) {
    qf_ctx *ctx = sv->ctx;
    const uint32_t chunk_log = std::min<uint32_t>(n, 13);  // 8192 amplitudes per block
    const uint64_t chunks = 1ULL << (n - chunk_log);
    const uint64_t blocks = B * chunks;
    if (blocks > 0x7FFFFFFFULL) return fail(QF_ERR_STATE_TOO_LARGE, "batch reduction grid exceeds the launch limit");
    const size_t part_b = sizeof(double) * blocks, p1_b = sizeof(double) * B, inv_b = sizeof(double) * B;
    QF_TRY(ensure_device(&ctx->ws_tree, &ctx->ws_tree_bytes, part_b + p1_b + inv_b + B + 16));
    unsigned char *w = static_cast<unsigned char *>(ctx->ws_tree);
    double *d_part = reinterpret_cast<double *>(w);
    double *d_p1 = reinterpret_cast<double *>(w + part_b);
    double *d_inv = reinterpret_cast<double *>(w + part_b + p1_b);
    uint8_t *d_out = w + part_b + p1_b + inv_b;
    if (sv->dtype == QF_C64)
        k_batch_p_one<float2><<<(unsigned)blocks, 256, 0, ctx->stream>>>(static_cast<const float2 *>(sv->d), n, q, chunk_log, d_part);
    else
        k_batch_p_one<double2><<<(unsigned)blocks, 256, 0, ctx->stream>>>(static_cast<const double2 *>(sv->d), n, q, chunk_log, d_part);
    QF_CUDA(cudaGetLastError());
    k_batch_finish<<<(unsigned)((B + 255) / 256), 256, 0, ctx->stream>>>(d_part, B, (uint32_t)chunks, d_p1);
    QF_CUDA(cudaGetLastError());
    std::vector<double> p1(B), inv(B);
    QF_CUDA(cudaMemcpyAsync(p1.data(), d_p1, p1_b, cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    for (uint64_t b = 0; b < B; ++b) {
        const double p = std::min(1.0, std::max(0.0, p1[b]));
        const uint8_t o = uniforms[b] < p ? 1 : 0;
        const double prob = o ? p : 1.0 - p;
        if (prob <= 2.220446049250313e-16)
            return fail(QF_ERR_INVALID_PROBABILITY, "measurement probability must be in [0, 1], got %g", prob);
        outcomes[b] = o;
        inv[b] = 1.0 / std::sqrt(prob);
    }
    QF_CUDA(cudaMemcpyAsync(d_out, outcomes, B, cudaMemcpyHostToDevice, ctx->stream));
    QF_CUDA(cudaMemcpyAsync(d_inv, inv.data(), inv_b, cudaMemcpyHostToDevice, ctx->stream));
    const uint64_t total = B << n;
    const int grid = std::max(1, std::min<int>((int)((total + 255) / 256), ctx->sm_count * 8));
    if (sv->dtype == QF_C64)
        k_batch_collapse<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), total, n, q, d_out, d_inv);
    else
        k_batch_collapse<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), total, n, q, d_out, d_inv);
    QF_CUDA(cudaGetLastError());
    QF_CUDA(cudaStreamSynchronize(ctx->stream));  // host outcome/inverse buffers are read by the copies
    return QF_OK;
}

// ---- Pauli sums --------------------------------------------------------------
// Terms are grouped by x-mask. For one group, G_x(i) = sum_t c_t * i^{ny_t} *
// (-1)^{popcount(i & z_t)} is the phase PauliWord::apply_basis_index gives
// basis state i (src/analytic.rs:2629-2650), so
//   <psi|H_x|psi> = sum_i conj(psi_{i^x}) G_x(i) psi_i,  (H_x psi)_j = G_x(j^x) psi_{j^x}.
// A pass keeps every x-bit of its groups tile-resident, so each partner
// amplitude is in shared memory.
// a term staged in shared memory with its coefficient in the state's real
// type: converted once per CTA, not once per amplitude
template <typename R>
struct PTermR {
    uint64_t z;
    R cre, cim;
};
template <typename R>
struct PTermT {
    uint64_t zo;
    uint32_t zl, q;
    R cre, cim;
};
template <typename C>
__global__ void __launch_bounds__(kRedThreads)
    k_pauli_pass(const C *__restrict__ psi, C *__restrict__ lam, const PPassArgs pa, const PGroup *__restrict__ g_groups,
                 const PTerm *__restrict__ g_terms, double *__restrict__ partials) {
    using R = typename Real<C>::T;
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t T = 1u << pa.k, nhi = pa.k - pa.low;
    C *s = reinterpret_cast<C *>(smem);
    uint64_t *hi_off = reinterpret_cast<uint64_t *>(smem + (size_t)T * sizeof(C));
    PGroup *groups = reinterpret_cast<PGroup *>(hi_off + (1u << nhi));
    PTermR<R> *terms = reinterpret_cast<PTermR<R> *>(groups + pa.n_groups);
    __shared__ double red[32];
    for (uint32_t h = threadIdx.x; h < (1u << nhi); h += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t r = 0; r < nhi; ++r)
            if ((h >> r) & 1u) off |= 1ULL << pa.hi_q[r];
        hi_off[h] = off;
    }
    for (uint32_t g = threadIdx.x; g < pa.n_groups; g += blockDim.x) groups[g] = g_groups[g];
    for (uint32_t t = threadIdx.x; t < pa.n_terms; t += blockDim.x)
        terms[t] = PTermR<R>{g_terms[t].z, (R)g_terms[t].cre, (R)g_terms[t].cim};
    __syncthreads();
    const uint32_t lowmask = (1u << pa.low) - 1;
    double acc_re = 0.0, acc_im = 0.0;
    for (uint64_t t = blockIdx.x; t < pa.n_tiles; t += gridDim.x) {
        const uint64_t base = deposit(t, pa.nonlocal_mask);
        for (uint32_t j = threadIdx.x; j < T; j += blockDim.x) s[j] = psi[base | hi_off[j >> pa.low] | (j & lowmask)];
        __syncthreads();
        R tile_re = 0, tile_im = 0;  // this thread's share of the tile, then one f64 add per tile
        for (uint32_t j = threadIdx.x; j < T; j += blockDim.x) {
            const uint64_t gi = base | hi_off[j >> pa.low] | (j & lowmask);
            R er = 0, ei = 0;
            for (uint32_t g = 0; g < pa.n_groups; ++g) {
                const PGroup G = groups[g];
                // phase evaluated at the source index of the matrix element
                const uint64_t src = pa.mode == 0 ? gi : (gi ^ G.x);
                R gr = 0, gim = 0;
                for (uint32_t q = 0; q < G.t_count; ++q) {
                    const PTermR<R> P = terms[G.t_begin + q];
                    if (__popcll(src & P.z) & 1) {
                        gr -= P.cre;
                        gim -= P.cim;
                    } else {
                        gr += P.cre;
                        gim += P.cim;
                    }
                }
                const C a = s[j ^ G.xl];
                if (pa.mode == 0) {
                    // conj(psi_{j^x}) * G * psi_j
                    const C b = s[j];
                    const R pr = gr * b.x - gim * b.y, pim = gr * b.y + gim * b.x;
                    er += a.x * pr + a.y * pim;
                    ei += a.x * pim - a.y * pr;
                } else {
                    er += gr * a.x - gim * a.y;
                    ei += gr * a.y + gim * a.x;
                }
            }
            if (pa.mode == 0) {
                tile_re += er;
                tile_im += ei;
            } else {
                if (pa.mode == 2) {
                    const C old = lam[gi];
                    er += old.x;
                    ei += old.y;
                }
                lam[gi] = mk(er, ei);
                if (pa.last) {
                    const C b = s[j];  // conj(psi_j) * lambda_j
                    tile_re += b.x * er + b.y * ei;
                    tile_im += b.x * ei - b.y * er;
                }
            }
        }
        acc_re += (double)tile_re;
        acc_im += (double)tile_im;
        __syncthreads();
    }
    acc_re = block_sum(acc_re, red);
    if (threadIdx.x == 0) partials[2 * blockIdx.x] = acc_re;
    acc_im = block_sum(acc_im, red);
    if (threadIdx.x == 0) partials[2 * blockIdx.x + 1] = acc_im;
}

// The same pass for tiles of 256 * NR amplitudes: thread tid owns the
// amplitudes j = tid + 256 r (r < NR), processed RC at a time. A term's sign
// at j (or j ^ x) is parity(tid & zl) ^ parity(tile base & zo) ^ parity(x & zl)
// ^ bit r of the precomputed q, so each term costs one select-add per
// amplitude and the NR sums are independent.
template <typename C, int NR, int RC>
__global__ void __launch_bounds__(kRedThreads)
    k_pauli_pass_r(const C *__restrict__ psi, C *__restrict__ lam, const PPassArgs pa, const PGroup *__restrict__ g_groups,
                   const PTerm *__restrict__ g_terms, double *__restrict__ partials) {
    using R = typename Real<C>::T;
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr uint32_t T = 256u * NR;
    const uint32_t nhi = pa.k - pa.low, tid = threadIdx.x;
    C *s = reinterpret_cast<C *>(smem);
    C *tabs = s + T;  // pa.n_tables x kTableEntries
    uint64_t *hi_off = reinterpret_cast<uint64_t *>(tabs + (size_t)pa.n_tables * kTableEntries);
    PGroup *groups = reinterpret_cast<PGroup *>(hi_off + (1u << nhi));
    PTermT<R> *terms = reinterpret_cast<PTermT<R> *>(groups + pa.n_groups);
    __shared__ double red[32];
    for (uint32_t h = tid; h < (1u << nhi); h += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t r = 0; r < nhi; ++r)
            if ((h >> r) & 1u) off |= 1ULL << pa.hi_q[r];
        hi_off[h] = off;
    }
    for (uint32_t g = tid; g < pa.n_groups; g += blockDim.x) groups[g] = g_groups[g];
    for (uint32_t t = tid; t < pa.n_terms; t += blockDim.x) {
        const PTerm P = g_terms[t];
        terms[t] = PTermT<R>{P.zo, P.zl, P.q, (R)P.cre, (R)P.cim};
    }
    __syncthreads();
    const uint32_t lowmask = (1u << pa.low) - 1;
    double acc_re = 0.0, acc_im = 0.0;
    for (uint64_t t = blockIdx.x; t < pa.n_tiles; t += gridDim.x) {
        const uint64_t base = deposit(t, pa.nonlocal_mask);
        for (uint32_t j = tid; j < T; j += blockDim.x) s[j] = psi[base | hi_off[j >> pa.low] | (j & lowmask)];
        // this tile's tables of the many-term groups: each coefficient signed
        // by the tile's own bits, then summed per 6-bit half of the local index
        for (uint32_t g = 0; g < pa.n_groups; ++g) {
            const PGroup G = groups[g];
            if (G.tab == kNoTable) continue;
            C *tb = tabs + (size_t)G.tab * kTableEntries;
            const uint32_t n_hi_entries = 1u << (pa.k - 6);
            for (uint32_t e = tid; e < 64u + n_hi_entries; e += blockDim.x) {
                R vr = 0, vi = 0;
                const bool lo = e < 64u;
                const uint32_t a = lo ? e : ((e - 64u) << 6);
                const uint32_t q0 = G.t_begin + (lo ? 0u : G.n_lo), q1 = G.t_begin + (lo ? G.n_lo : G.n_lo + G.n_hi + G.n_const);
                for (uint32_t q = q0; q < q1; ++q) {
                    const PTermT<R> P = terms[q];
                    const bool odd = (__popc(a & P.zl) + __popcll(base & P.zo)) & 1u;
                    vr += odd ? -P.cre : P.cre;
                    vi += odd ? -P.cim : P.cim;
                }
                tb[e] = mk(vr, vi);
            }
        }
        __syncthreads();
        R tile_re = 0, tile_im = 0;
#pragma unroll 1
        for (uint32_t rc = 0; rc < (uint32_t)NR; rc += RC) {
            R er[RC], ei[RC];
#pragma unroll
            for (int r = 0; r < RC; ++r) er[r] = ei[r] = 0;
            for (uint32_t g = 0; g < pa.n_groups; ++g) {
                const PGroup G = groups[g];
                const uint32_t xo = pa.mode == 0 ? 0u : G.xl;  // phase at the source index of the element
                R gr[RC], gim[RC];
                uint32_t q_first = 0;
                if (G.tab != kNoTable) {  // table lookups, then the terms spanning both halves
                    const C *tb = tabs + (size_t)G.tab * kTableEntries;
#pragma unroll
                    for (int r = 0; r < RC; ++r) {
                        const uint32_t src = (tid + 256u * (rc + r)) ^ xo;
                        const C lo = tb[src & 63u], hi = tb[64u + (src >> 6)];
                        gr[r] = lo.x + hi.x;
                        gim[r] = lo.y + hi.y;
                    }
                    q_first = G.n_lo + G.n_hi + G.n_const;
                } else {
#pragma unroll
                    for (int r = 0; r < RC; ++r) gr[r] = gim[r] = 0;
                }
                for (uint32_t q = q_first; q < G.t_count; ++q) {
                    const PTermT<R> P = terms[G.t_begin + q];
                    const uint32_t par = (__popc((tid ^ xo) & P.zl & 0xFFu) + __popc(xo & P.zl & ~0xFFu) + __popcll(base & P.zo)) & 1u;
                    const uint32_t m = (P.q >> rc) ^ (0u - par);
                    if (G.real) {
#pragma unroll
                        for (int r = 0; r < RC; ++r) gr[r] += ((m >> r) & 1u) ? -P.cre : P.cre;
                    } else {
#pragma unroll
                        for (int r = 0; r < RC; ++r) {
                            const bool odd = (m >> r) & 1u;
                            gr[r] += odd ? -P.cre : P.cre;
                            gim[r] += odd ? -P.cim : P.cim;
                        }
                    }
                }
#pragma unroll
                for (int r = 0; r < RC; ++r) {
                    const uint32_t j = tid + 256u * (rc + r);
                    const C a = s[j ^ G.xl];
                    if (pa.mode == 0) {  // conj(psi_{j^x}) * G * psi_j
                        const C b = s[j];
                        const R pr = gr[r] * b.x - gim[r] * b.y, pim = gr[r] * b.y + gim[r] * b.x;
                        er[r] += a.x * pr + a.y * pim;
                        ei[r] += a.x * pim - a.y * pr;
                    } else {
                        er[r] += gr[r] * a.x - gim[r] * a.y;
                        ei[r] += gr[r] * a.y + gim[r] * a.x;
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < RC; ++r) {
                const uint32_t j = tid + 256u * (rc + r);
                if (pa.mode == 0) {
                    tile_re += er[r];
                    tile_im += ei[r];
                } else {
                    const uint64_t gi = base | hi_off[j >> pa.low] | (j & lowmask);
                    R vr = er[r], vi = ei[r];
                    if (pa.mode == 2) {
                        const C old = lam[gi];
                        vr += old.x;
                        vi += old.y;
                    }
                    lam[gi] = mk(vr, vi);
                    if (pa.last) {
                        const C b = s[j];  // conj(psi_j) * lambda_j
                        tile_re += b.x * vr + b.y * vi;
                        tile_im += b.x * vi - b.y * vr;
                    }
                }
            }
        }
        acc_re += (double)tile_re;
        acc_im += (double)tile_im;
        __syncthreads();
    }
    acc_re = block_sum(acc_re, red);
    if (threadIdx.x == 0) partials[2 * blockIdx.x] = acc_re;
    acc_im = block_sum(acc_im, red);
    if (threadIdx.x == 0) partials[2 * blockIdx.x + 1] = acc_im;
}

// A group whose x-mask does not fit in one tile: one grid-stride sweep over
// the pairs (i, i ^ x) straight from global memory (coalesced runs on both
// sides of the pair). mode 0 accumulates <psi|H_x|psi>; mode 2 adds H_x psi
// into lambda.
template <typename C>
__global__ void k_pauli_wide(const C *__restrict__ psi, C *__restrict__ lam, uint64_t n_pairs, uint64_t x, uint32_t xb,
                             const PTerm *__restrict__ g_terms, uint32_t nt, uint32_t mode, double *__restrict__ partials) {
    using R = typename Real<C>::T;
    __shared__ double red[32];
    extern __shared__ __align__(16) unsigned char wsmem[];
    PTermR<R> *terms = reinterpret_cast<PTermR<R> *>(wsmem);
    for (uint32_t t = threadIdx.x; t < nt; t += blockDim.x)
        terms[t] = PTermR<R>{g_terms[t].z, (R)g_terms[t].cre, (R)g_terms[t].cim};
    __syncthreads();
    double acc_re = 0.0, acc_im = 0.0;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n_pairs; p += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = insert0(p, xb), j = i ^ x;
        R gir = 0, gii = 0, gjr = 0, gji = 0;
        for (uint32_t t = 0; t < nt; ++t) {
            const PTermR<R> P = terms[t];
            const R si = (__popcll(i & P.z) & 1) ? R(-1) : R(1);
            const R sj = (__popcll(j & P.z) & 1) ? R(-1) : R(1);
            gir += si * P.cre;
            gii += si * P.cim;
            gjr += sj * P.cre;
            gji += sj * P.cim;
        }
        const C ai = psi[i], aj = psi[j];
        // G_i a_i and G_j a_j
        const R pir = gir * ai.x - gii * ai.y, pii = gir * ai.y + gii * ai.x;
        const R pjr = gjr * aj.x - gji * aj.y, pji = gjr * aj.y + gji * aj.x;
        if (mode == 0) {
            // conj(a_j) G_i a_i + conj(a_i) G_j a_j
            acc_re += (double)(aj.x * pir + aj.y * pii) + (double)(ai.x * pjr + ai.y * pji);
            acc_im += (double)(aj.x * pii - aj.y * pir) + (double)(ai.x * pji - ai.y * pjr);
        } else {
            C lj = lam[j], li = lam[i];
            lj.x += pir;
            lj.y += pii;
            li.x += pjr;
            li.y += pji;
            lam[j] = lj;
            lam[i] = li;
        }
    }
    acc_re = block_sum(acc_re, red);
    if (threadIdx.x == 0) partials[2 * blockIdx.x] = acc_re;
    acc_im = block_sum(acc_im, red);
    if (threadIdx.x == 0) partials[2 * blockIdx.x + 1] = acc_im;
}

// sum_i conj(a_i) b_i
template <typename C>
__global__ void k_dot(const C *__restrict__ a, const C *__restrict__ b, uint64_t dim, double *__restrict__ partials) {
    __shared__ double red[32];
    double re = 0.0, im = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += (uint64_t)gridDim.x * blockDim.x) {
        const C u = a[i], v = b[i];
        re += (double)u.x * v.x + (double)u.y * v.y;
        im += (double)u.x * v.y - (double)u.y * v.x;
    }
    re = block_sum(re, red);
    if (threadIdx.x == 0) partials[2 * blockIdx.x] = re;
    im = block_sum(im, red);
    if (threadIdx.x == 0) partials[2 * blockIdx.x + 1] = im;
}

namespace {
struct PPassHost {
    PPassArgs a;
    std::vector<PGroup> groups;
    std::vector<PTerm> terms;
};
struct PWide {
    uint64_t x;
    std::vector<PTerm> terms;
};
struct PauliPlan {
    std::vector<PPassHost> tiles;
    std::vector<PWide> wide;
};

int plan_pauli(uint32_t n, int dtype, const qf_pauli_term *terms, uint64_t n_terms, PauliPlan &plan) {
    const uint64_t valid = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    std::map<uint64_t, std::vector<PTerm>> by_x;
    for (uint64_t t = 0; t < n_terms; ++t) {
        const qf_pauli_term &P = terms[t];
        if ((P.xmask | P.zmask) & ~valid)
            return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "Pauli term %llu acts outside %u qubits", (unsigned long long)t, n);
        const int ny = __builtin_popcountll(P.xmask & P.zmask) & 3;
        double re = P.coeff_re, im = P.coeff_im;
        for (int r = 0; r < ny; ++r) {  // multiply by i
            const double t2 = re;
            re = -im;
            im = t2;
        }
        by_x[P.xmask].push_back(PTerm{P.zmask, re, im, 0, 0, 0});
    }
    int k, low;
    default_tiling(n, dtype, 0, &k, &low);
    const uint64_t low_mask = (1ULL << low) - 1;
    std::vector<std::pair<uint64_t, std::vector<PTerm>>> groups;
    for (auto &kv : by_x) {
        if (__builtin_popcountll(low_mask | kv.first) > k) plan.wide.push_back(PWide{kv.first, kv.second});
        else groups.push_back(kv);
    }
    std::vector<bool> done(groups.size(), false);
    size_t left = groups.size();
    while (left) {
        uint64_t L = low_mask;
        std::vector<size_t> sel;
        for (size_t g = 0; g < groups.size(); ++g) {
            if (done[g]) continue;
            const uint64_t nl = L | groups[g].first;
            if (__builtin_popcountll(nl) <= k) {
                L = nl;
                sel.push_back(g);
            }
        }
        for (uint32_t q = 0; q < n && __builtin_popcountll(L) < k; ++q) L |= 1ULL << q;
        PPassHost P;
        std::memset(&P.a, 0, sizeof P.a);
        uint32_t lo_eff = 0;
        while (lo_eff < n && ((L >> lo_eff) & 1ULL)) ++lo_eff;
        std::vector<int> lbit(n, -1);
        for (uint32_t q = 0; q < lo_eff; ++q) lbit[q] = (int)q;
        uint32_t r = 0;
        for (uint32_t q = lo_eff; q < n; ++q)
            if ((L >> q) & 1ULL) {
                if (r >= (uint32_t)kMaxLocal) return fail(QF_ERR_UNSUPPORTED_OPERATION, "Pauli pass too wide");
                P.a.hi_q[r] = (uint8_t)q;
                lbit[q] = (int)(lo_eff + r++);
            }
        P.a.k = lo_eff + r;
        P.a.low = lo_eff;
        P.a.nonlocal_mask = valid & ~L;
        P.a.n_tiles = 1ULL << (n - P.a.k);
        for (size_t g : sel) {
            done[g] = true;
            --left;
            PGroup G;
            G.x = groups[g].first;
            G.xl = 0;
            for (uint32_t q = 0; q < n; ++q)
                if ((G.x >> q) & 1ULL) G.xl |= 1u << lbit[q];
            G.t_begin = (uint32_t)P.terms.size();
            G.t_count = (uint32_t)groups[g].second.size();
            G.real = 1;
            G.tab = kNoTable;
            G.n_lo = G.n_hi = G.n_const = 0;
            std::vector<PTerm> part[4];  // low half, high half, off the tile, both halves
            for (PTerm T : groups[g].second) {
                // the term's z on the resident qubits in tile bits, on the rest as is
                T.zo = T.z & P.a.nonlocal_mask;
                T.zl = 0;
                for (uint32_t q = 0; q < n; ++q)
                    if (((T.z >> q) & 1ULL) && lbit[q] >= 0) T.zl |= 1u << lbit[q];
                T.q = 0;
                const uint32_t nr = P.a.k > 8 ? 1u << (P.a.k - 8) : 1u;
                for (uint32_t r = 0; r < nr && r < 32; ++r) T.q |= (uint32_t)(__builtin_popcount(r & (T.zl >> 8)) & 1) << r;
                if (T.cim != 0.0) G.real = 0;
                const int kind = (T.zl & 63u) && (T.zl >> 6) ? 3 : (T.zl & 63u) ? 0 : (T.zl >> 6) ? 1 : 2;
                part[kind].push_back(T);
            }
            // the register-tiled pass (tiles of 2^9..2^13) evaluates a group of many
            // terms from two tables unless most of its terms span both halves
            if (P.a.k >= 9 && P.a.k <= 13 && G.t_count >= kTableTerms && part[3].size() * 2 < G.t_count) {
                G.tab = P.a.n_tables++;
                G.n_lo = (uint32_t)part[0].size();
                G.n_hi = (uint32_t)part[1].size();
                G.n_const = (uint32_t)part[2].size();
            }
            for (int kind = 0; kind < 4; ++kind)
                for (const PTerm &T : part[kind]) P.terms.push_back(T);
            P.groups.push_back(G);
        }
        P.a.n_groups = (uint32_t)P.groups.size();
        P.a.n_terms = (uint32_t)P.terms.size();
        plan.tiles.push_back(std::move(P));
    }
    return QF_OK;
}

// Expectation (apply == false): every launch adds its slice of partials.
// Apply: lambda = sum of the launches; the energy <psi|lambda> comes from the
// last tile pass, or from a separate dot product when wide groups follow.
// the register-blocked pass for a tile of 2^k = 256 * NR amplitudes
template <typename C>
struct PauliRKernel {
    using Fn = void (*)(const C *, C *, const PPassArgs, const PGroup *, const PTerm *, double *);
    static Fn get(uint32_t k) {
        switch (k) {
        case 9: return k_pauli_pass_r<C, 2, 2>;
        case 10: return k_pauli_pass_r<C, 4, 4>;
        case 11: return k_pauli_pass_r<C, 8, 8>;
        case 12: return k_pauli_pass_r<C, 16, 8>;
        case 13: return k_pauli_pass_r<C, 32, 8>;
        default: return nullptr;
        }
    }
};

template <typename C>
// The sums land in out[] after a stream synchronize, or, with d_out, in
// device memory (two doubles) with nothing waited for.
int run_pauli(qf_sv *psi, qf_sv *lam, PauliPlan &plan, bool apply, double out[2], double *d_out = nullptr) {
    qf_ctx *ctx = psi->ctx;
    using R = typename Real<C>::T;
    static size_t dyn_limit[64] = {0};
    if (!dyn_limit[ctx->device & 63]) {
        QF_TRY(allow_max_dynamic_smem(k_pauli_pass<C>, ctx, &dyn_limit[ctx->device & 63]));
        for (uint32_t k = 9; k <= 13; ++k) {
            size_t lim = 0;
            QF_TRY(allow_max_dynamic_smem(PauliRKernel<C>::get(k), ctx, &lim));
        }
    }
    size_t meta = 0;
    for (auto &P : plan.tiles) meta += P.groups.size() * sizeof(PGroup) + P.terms.size() * sizeof(PTerm) + 64;
    for (auto &W : plan.wide) meta += W.terms.size() * sizeof(PTerm) + 32;
    QF_TRY(ensure_device(&ctx->ws_plan, &ctx->ws_plan_bytes, meta));
    const uint32_t grid = (uint32_t)ctx->sm_count * 8;  // upper bound; tile passes use their occupancy
    const bool need_dot = apply && !plan.wide.empty();
    const size_t launches = plan.tiles.size() + plan.wide.size() + (need_dot ? 1 : 0);
    double *partials;
    QF_TRY(partials_buffer(ctx, (size_t)2 * grid * launches, &partials));
    QF_CUDA(cudaMemsetAsync(partials, 0, sizeof(double) * 2 * grid * launches, ctx->stream));
    unsigned char *dmeta = static_cast<unsigned char *>(ctx->ws_plan);
    size_t off = 0, slice = 0;
    if (apply && plan.tiles.empty()) QF_CUDA(cudaMemsetAsync(lam->d, 0, lam->bytes(), ctx->stream));
    for (size_t i = 0; i < plan.tiles.size(); ++i) {
        PPassHost &P = plan.tiles[i];
        P.a.mode = apply ? (i == 0 ? 1u : 2u) : 0u;
        P.a.last = (apply && !need_dot && i + 1 == plan.tiles.size()) ? 1u : 0u;
    }
    // complex64 tile passes: compiled kernels (one per pass) when every pass fits
    bool compiled = false;
    if (sizeof(C) == 8 && !plan.tiles.empty()) {
        std::vector<const PPassArgs *> pa;
        std::vector<const std::vector<PGroup> *> pg;
        std::vector<const std::vector<PTerm> *> pt;
        for (const PPassHost &P : plan.tiles) {
            pa.push_back(&P.a);
            pg.push_back(&P.groups);
            pt.push_back(&P.terms);
        }
        QF_TRY(run_pauli_jit(psi, lam, pa, pg, pt, partials, 2 * grid, grid, &compiled));
        if (compiled) slice += plan.tiles.size();
    }
    for (size_t i = 0; i < plan.tiles.size() && !compiled; ++i, ++slice) {
        PPassHost &P = plan.tiles[i];
        PGroup *dg = reinterpret_cast<PGroup *>(dmeta + off);
        QF_CUDA(cudaMemcpyAsync(dg, P.groups.data(), P.groups.size() * sizeof(PGroup), cudaMemcpyHostToDevice, ctx->stream));
        off += (P.groups.size() * sizeof(PGroup) + 15) / 16 * 16;
        PTerm *dt = reinterpret_cast<PTerm *>(dmeta + off);
        QF_CUDA(cudaMemcpyAsync(dt, P.terms.data(), P.terms.size() * sizeof(PTerm), cudaMemcpyHostToDevice, ctx->stream));
        off += (P.terms.size() * sizeof(PTerm) + 15) / 16 * 16;
        auto rk = PauliRKernel<C>::get(P.a.k);
        const size_t head = ((size_t)1 << P.a.k) * sizeof(C) + (size_t)P.a.n_tables * kTableEntries * sizeof(C) +
                            (8u << (P.a.k - P.a.low)) + P.groups.size() * sizeof(PGroup);
        const size_t smem = head + P.terms.size() * (rk ? sizeof(PTermT<R>) : sizeof(PTermR<R>));
        if (smem > dyn_limit[ctx->device & 63])
            return fail(QF_ERR_UNSUPPORTED_OPERATION, "Pauli pass needs too much shared memory");
        int per_sm = 0;
        if (rk) QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rk, kRedThreads, smem));
        else QF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pauli_pass<C>, kRedThreads, smem));
        const uint32_t g = (uint32_t)std::min<uint64_t>(std::min<uint64_t>(grid, (uint64_t)std::max(per_sm, 1) * ctx->sm_count),
                                                        P.a.n_tiles);
        if (rk)
            rk<<<g, kRedThreads, smem, ctx->stream>>>(static_cast<const C *>(psi->d), lam ? static_cast<C *>(lam->d) : nullptr,
                                                      P.a, dg, dt, partials + (size_t)2 * grid * slice);
        else
            k_pauli_pass<C><<<g, kRedThreads, smem, ctx->stream>>>(static_cast<const C *>(psi->d),
                                                                   lam ? static_cast<C *>(lam->d) : nullptr, P.a, dg, dt,
                                                                   partials + (size_t)2 * grid * slice);
        QF_CUDA(cudaGetLastError());
    }
    for (size_t w = 0; w < plan.wide.size(); ++w, ++slice) {
        PWide &Wg = plan.wide[w];
        PTerm *dt = reinterpret_cast<PTerm *>(dmeta + off);
        QF_CUDA(cudaMemcpyAsync(dt, Wg.terms.data(), Wg.terms.size() * sizeof(PTerm), cudaMemcpyHostToDevice, ctx->stream));
        off += (Wg.terms.size() * sizeof(PTerm) + 15) / 16 * 16;
        const uint32_t xb = (uint32_t)__builtin_ctzll(Wg.x);
        const uint64_t pairs = psi->dim / 2;
        const uint32_t g = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(grid, (pairs + kRedThreads - 1) / kRedThreads));
        const size_t wsm = Wg.terms.size() * sizeof(PTermR<typename Real<C>::T>);
        if (wsm > 48 * 1024) return fail(QF_ERR_UNSUPPORTED_OPERATION, "too many Pauli terms share one x-mask");
        k_pauli_wide<C><<<g, kRedThreads, wsm, ctx->stream>>>(static_cast<const C *>(psi->d),
                                                            lam ? static_cast<C *>(lam->d) : nullptr, pairs, Wg.x, xb, dt,
                                                            (uint32_t)Wg.terms.size(), apply ? 2u : 0u,
                                                            partials + (size_t)2 * grid * slice);
        QF_CUDA(cudaGetLastError());
    }
    if (need_dot) {
        k_dot<C><<<grid, kRedThreads, 0, ctx->stream>>>(static_cast<const C *>(psi->d), static_cast<const C *>(lam->d),
                                                        psi->dim, partials + (size_t)2 * grid * slice);
        QF_CUDA(cudaGetLastError());
        ++slice;
    }
    // expectation: every slice; apply: only the slice carrying <psi|lambda>
    const size_t first = apply ? slice - 1 : 0;
    const uint32_t nblk = (uint32_t)(grid * (slice - first));
    k_final_sum<<<1, 256, 0, ctx->stream>>>(partials + 2 * grid * first, nblk, 2, d_out ? d_out : ctx->d_small);
    QF_CUDA(cudaGetLastError());
    if (d_out) return QF_OK;
    QF_CUDA(cudaMemcpyAsync(ctx->h_small, ctx->d_small, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    out[0] = ctx->h_small[0];
    out[1] = ctx->h_small[1];
    return QF_OK;
}
}  // namespace

int pauli_plan_stats(uint32_t n, int dtype, const qf_pauli_term *terms, uint64_t n_terms, uint64_t *tile_passes,
                     uint64_t *wide_passes) {
    PauliPlan plan;
    if (n_terms) QF_TRY(plan_pauli(n, dtype, terms, n_terms, plan));
    *tile_passes = plan.tiles.size();
    *wide_passes = plan.wide.size();
    return QF_OK;
}

int pauli_expectation(qf_sv *sv, const qf_pauli_term *terms, uint64_t n_terms, double out[2]) {
    out[0] = out[1] = 0.0;
    if (n_terms == 0) return QF_OK;
    PauliPlan plan;
    QF_TRY(plan_pauli(sv->n, sv->dtype, terms, n_terms, plan));
    if (sv->dtype == QF_C64) return run_pauli<float2>(sv, nullptr, plan, false, out);
    return run_pauli<double2>(sv, nullptr, plan, false, out);
}

int pauli_apply(qf_sv *psi, qf_sv *lam, const qf_pauli_term *terms, uint64_t n_terms, double *energy, double *d_energy) {
    if (n_terms == 0) {
        QF_CUDA(cudaMemsetAsync(lam->d, 0, lam->bytes(), psi->ctx->stream));
        if (d_energy) QF_CUDA(cudaMemsetAsync(d_energy, 0, 2 * sizeof(double), psi->ctx->stream));
        if (energy) *energy = 0.0;
        return QF_OK;
    }
    PauliPlan plan;
    QF_TRY(plan_pauli(psi->n, psi->dtype, terms, n_terms, plan));
    double out[2] = {0.0, 0.0};
    if (psi->dtype == QF_C64) QF_TRY(run_pauli<float2>(psi, lam, plan, true, out, d_energy));
    else QF_TRY(run_pauli<double2>(psi, lam, plan, true, out, d_energy));
    if (energy && !d_energy) *energy = out[0];
    return QF_OK;
}

// ---- sampler -----------------------------------------------------------------
// Terminal measurements of qubits q_0..q_{m-1} (distinct). J_m[b] is the
// probability mass of the indices whose measured bits spell b (bit j = bit
// q_j); level k of the tree sums level k+1 over the outcome of q_k. A shot
// starts its SmallRng at draw s*m (the reference's shot-major order,
// src/lib.rs:2874-2912) via jump matrices and descends the tree:
// p_one = J_{k+1}(b | 1<<k) / D, D = product of the chosen branch
// probabilities, which is the reference's successive renormalisation
// (src/lib.rs:1329-1350) up to rounding; |u - p_one| < tie_eps is reported.
template <typename C>
__global__ void k_marginal(const C *__restrict__ a, uint32_t n, const uint32_t *__restrict__ mq, uint32_t m,
                           uint64_t rest_mask, double *__restrict__ leaf) {
    const uint64_t nb = 1ULL << m, nu = 1ULL << (n - m);
    for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; b < nb; b += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t idx = 0;
        for (uint32_t j = 0; j < m; ++j)
            if ((b >> j) & 1ULL) idx |= 1ULL << mq[j];
        double s = 0.0;
        for (uint64_t u = 0; u < nu; ++u) {
            const C v = a[idx | deposit(u, rest_mask)];
            s += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
        }
        leaf[b] = s;
    }
}

// level k (2^k entries at offset 2^k - 1) from level k+1
__global__ void k_tree_level(double *tree, uint32_t k) {
    const uint64_t cnt = 1ULL << k;
    double *dst = tree + (cnt - 1), *src = tree + (2 * cnt - 1);
    for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; b < cnt; b += (uint64_t)gridDim.x * blockDim.x)
        dst[b] = src[b] + src[b | cnt];
}

__device__ __forceinline__ uint64_t gf2_apply(const uint64_t *cols, uint64_t x) {
    uint64_t y = 0;
    while (x) {
        const int c = __ffsll((long long)x) - 1;
        y ^= cols[c];
        x &= x - 1;
    }
    return y;
}

__global__ void k_shots(const double *__restrict__ tree, uint32_t m, const uint32_t *__restrict__ cbits, uint64_t shots,
                        uint64_t seed_state, const uint64_t *__restrict__ jump, const uint64_t *__restrict__ starts,
                        int normalize, double tie_eps, uint64_t *__restrict__ outcomes, unsigned long long *__restrict__ ties,
                        int *__restrict__ err) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < shots; s += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t x = seed_state;
        if (starts) {  // the shot's generator state given (shots of one branch of a feed-forward circuit)
            x = starts[s];
        } else {
            for (int j = 0; j < 64; ++j)
                if ((s >> j) & 1ULL) x = gf2_apply(jump + 64 * j, x);
        }
        uint64_t b = 0, reg = 0;
        double D = normalize ? tree[0] : 1.0;  // complex64: probabilities relative to the state's own norm
        unsigned long long nt = 0;
        for (uint32_t k = 0; k < m; ++k) {
            const double J1 = tree[((1ULL << (k + 1)) - 1) + (b | (1ULL << k))];
            double p = J1 / D;
            if (p < 0.0) p = 0.0;
            if (p > 1.0) p = 1.0;
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            const double u = (double)(x >> 11) * (1.0 / 9007199254740992.0);
            const int o = u < p ? 1 : 0;
            if (fabs(u - p) < tie_eps) ++nt;
            const double prob = o ? p : 1.0 - p;
            if (prob <= 2.220446049250313e-16) {
                atomicOr(err, 1);
                break;
            }
            D *= prob;
            b |= (uint64_t)o << k;
            reg = (reg & ~(1ULL << cbits[k])) | ((uint64_t)o << cbits[k]);
        }
        outcomes[s] = reg;
        if (nt) atomicAdd(ties, nt);
    }
}

int sample_shots(qf_sv *sv, const uint32_t *qubits, const uint32_t *cbits, uint32_t m, uint64_t shots, uint64_t seed,
                 double tie_eps, uint64_t *outcomes_host, uint64_t *n_ties, const uint64_t *start_states) {
    qf_ctx *ctx = sv->ctx;
    const uint32_t n = sv->n;
    if (m > 30) return fail(QF_ERR_UNSUPPORTED_OPERATION, "at most 30 terminal measurements are supported, got %u", m);
    uint64_t seen = 0;
    for (uint32_t j = 0; j < m; ++j) {
        if (qubits[j] >= n) return fail(QF_ERR_QUBIT_OUT_OF_RANGE, "qubit index %u is out of range for %u qubits", qubits[j], n);
        if (cbits[j] >= 64) return fail(QF_ERR_UNSUPPORTED_OPERATION, "classical bit %u exceeds the packed 64-bit register", cbits[j]);
        if ((seen >> qubits[j]) & 1ULL)
            return fail(QF_ERR_UNSUPPORTED_OPERATION, "qubit %u is measured twice; repeated measurement needs the per-shot engine", qubits[j]);
        seen |= 1ULL << qubits[j];
    }
    if (m == 0) {  // no measurement: every shot reads an empty register
        if (outcomes_host) std::memset(outcomes_host, 0, sizeof(uint64_t) * shots);
        if (n_ties) *n_ties = 0;
        return QF_OK;
    }
    const uint64_t valid = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    const uint64_t rest = valid & ~seen;
    // workspace: tree (2^(m+1) doubles) | outcomes (shots u64) | jump (64*64 u64) | mq | cb | ties | err | starts
    const size_t tree_b = sizeof(double) * ((2ULL << m));
    const size_t out_b = sizeof(uint64_t) * shots;
    const size_t jump_b = sizeof(uint64_t) * 64 * 64;
    const size_t meta_b = 2 * sizeof(uint32_t) * 32 + 64;
    const size_t start_b = start_states ? sizeof(uint64_t) * shots : 0;
    QF_TRY(ensure_device(&ctx->ws_tree, &ctx->ws_tree_bytes, tree_b + out_b + jump_b + meta_b + start_b));
    unsigned char *w = static_cast<unsigned char *>(ctx->ws_tree);
    double *tree = reinterpret_cast<double *>(w);
    uint64_t *d_out = reinterpret_cast<uint64_t *>(w + tree_b);
    uint64_t *d_jump = reinterpret_cast<uint64_t *>(w + tree_b + out_b);
    uint32_t *d_mq = reinterpret_cast<uint32_t *>(w + tree_b + out_b + jump_b);
    uint32_t *d_cb = d_mq + 32;
    unsigned long long *d_ties = reinterpret_cast<unsigned long long *>(d_cb + 32);
    int *d_err = reinterpret_cast<int *>(d_ties + 1);
    uint64_t *d_starts = start_states ? reinterpret_cast<uint64_t *>(w + tree_b + out_b + jump_b + meta_b) : nullptr;
    if (d_starts) QF_CUDA(cudaMemcpyAsync(d_starts, start_states, start_b, cudaMemcpyHostToDevice, ctx->stream));

    static thread_local uint64_t jump[64][64];
    rng_jump_matrices(m, jump, 64);
    QF_CUDA(cudaMemcpyAsync(d_jump, jump, jump_b, cudaMemcpyHostToDevice, ctx->stream));
    if (m) {
        QF_CUDA(cudaMemcpyAsync(d_mq, qubits, sizeof(uint32_t) * m, cudaMemcpyHostToDevice, ctx->stream));
        QF_CUDA(cudaMemcpyAsync(d_cb, cbits, sizeof(uint32_t) * m, cudaMemcpyHostToDevice, ctx->stream));
    }
    QF_CUDA(cudaMemsetAsync(d_ties, 0, sizeof(unsigned long long) + sizeof(int) + 4, ctx->stream));
    // leaves at offset 2^m - 1
    double *leaf = tree + ((1ULL << m) - 1);
    const uint64_t nb = 1ULL << m;
    const int grid = std::max(1, std::min<int>((int)((nb + 255) / 256), ctx->sm_count * 8));
    if (sv->dtype == QF_C64)
        k_marginal<float2><<<grid, 256, 0, ctx->stream>>>(static_cast<float2 *>(sv->d), n, d_mq, m, rest, leaf);
    else
        k_marginal<double2><<<grid, 256, 0, ctx->stream>>>(static_cast<double2 *>(sv->d), n, d_mq, m, rest, leaf);
    QF_CUDA(cudaGetLastError());
    for (int k = (int)m - 1; k >= 0; --k) {
        const uint64_t cnt = 1ULL << k;
        k_tree_level<<<std::max(1, std::min<int>((int)((cnt + 255) / 256), ctx->sm_count * 8)), 256, 0, ctx->stream>>>(tree, (uint32_t)k);
        QF_CUDA(cudaGetLastError());
    }
    const uint64_t seed_state = [&] {
        uint64_t z = seed + 0x9E3779B97F4A7C15ULL;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        return z == 0 ? 0x9E3779B97F4A7C15ULL : z;
    }();
    const int sgrid = std::max(1, std::min<int>((int)((shots + 127) / 128), ctx->sm_count * 16));
    k_shots<<<sgrid, 128, 0, ctx->stream>>>(tree, m, d_cb, shots, seed_state, d_jump, d_starts, sv->dtype == QF_C64 ? 1 : 0,
                                            tie_eps, d_out, d_ties, d_err);
    QF_CUDA(cudaGetLastError());
    if (outcomes_host)
        QF_CUDA(cudaMemcpyAsync(outcomes_host, d_out, out_b, cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaMemcpyAsync(ctx->h_small, d_ties, 16, cudaMemcpyDeviceToHost, ctx->stream));
    QF_CUDA(cudaStreamSynchronize(ctx->stream));
    unsigned long long t;
    int e;
    std::memcpy(&t, ctx->h_small, sizeof t);
    std::memcpy(&e, reinterpret_cast<unsigned char *>(ctx->h_small) + 8, sizeof e);
    if (n_ties) *n_ties = t;
    if (e) return fail(QF_ERR_INVALID_PROBABILITY, "a shot selected a measurement branch of probability <= f64::EPSILON");
    return QF_OK;
}

}  // namespace qf
