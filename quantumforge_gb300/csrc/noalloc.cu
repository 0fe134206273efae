// noalloc.cu — <Z_q> for every qubit of a state held in caller-owned device
// memory, with no allocation by the library.
//
// Some callers cannot let a library call cudaMalloc: a host framework that
// owns all device memory through its own pool allocator, or a latency-bound
// loop in which cudaMalloc/cudaFree (which synchronise the device) are not
// acceptable. For them this file computes the same reduction as
// qf_sv_expectation_z_all from a raw device pointer, using as its only scratch
// a fixed file-scope __device__ array. Every GPU that loads this library holds
// that array (about 84 KB) until the process exits.
//
// Host code cannot use the array's name as a device address; the device
// address is looked up once per device with cudaGetSymbolAddress (with that
// device current) by the first call on the device, and passed to the
// kernels. That first call should therefore come before any stream capture.
// The address is cached for the life of the process: it belongs to the
// device's primary context, so a caller that destroys that context
// (cudaDeviceReset) must not call this entry point again in the same process.
// All calls share the array and every call overwrites the part it reads, so
// calls that overlap on the GPU (different streams, or different host
// threads) race and must be serialised by the caller. The calling thread's
// current device is the same after the call as before it.
#include <algorithm>
#include <mutex>

#include "qf_device.cuh"
#include "qf_internal.h"

namespace qf {
namespace {

constexpr uint32_t kNaMaxQubits = 40;
constexpr uint32_t kNaThreads = 256;
constexpr uint32_t kNaMaxBlocks = 256;
constexpr uint32_t kNaVals = kNaMaxQubits + 1;
// per-block partial sums (kNaMaxBlocks x kNaVals), then the final sums (kNaVals)
constexpr size_t kNaScratch = (size_t)kNaMaxBlocks * kNaVals + kNaVals;

static __device__ __align__(256) double g_na_scratch[kNaScratch];

std::mutex g_na_mu;
double *g_na_addr[64] = {nullptr};

// Device address of the scratch array on `device` (current), looked up once.
int na_scratch(int device, double **out) {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
        g_na_addr[device] = static_cast<double *>(p);
    }
    *out = g_na_addr[device];
    return QF_OK;
}

template <typename C> __device__ __forceinline__ double na_p(const C *a, uint64_t i) {
    const C v = a[i];
    return (double)v.x * (double)v.x + (double)v.y * (double)v.y;
}

// Chunks of 8 contiguous amplitudes per thread and iteration; per-bit sums of
// index bits 0..2 inside the chunk, bits 3..3+s_log-1 fixed by the thread id,
// higher bits fixed by the iteration. Writes partial[block][q] = sum of |a|^2
// over indices with bit q set, partial[block][n] = the total.
template <typename C>
__global__ void __launch_bounds__(kNaThreads) k_na_zsum(const C *__restrict__ a, uint32_t n, uint32_t s_log,
                                                        double *__restrict__ partial) {
    __shared__ double red[32];
    const uint64_t gtid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nchunks = 1ULL << (n - 3);
    double tot = 0.0, lo[3] = {0.0, 0.0, 0.0}, hi[kNaMaxQubits];
    const uint32_t nhi = n > 3 + s_log ? n - 3 - s_log : 0;
    for (uint32_t r = 0; r < nhi; ++r) hi[r] = 0.0;
    uint64_t it = 0;
    for (uint64_t c = gtid; c < nchunks; c += (1ULL << s_log), ++it) {
        double p[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) p[j] = na_p(a, (c << 3) + j);
        const double t = ((p[0] + p[1]) + (p[2] + p[3])) + ((p[4] + p[5]) + (p[6] + p[7]));
        tot += t;
        lo[0] += (p[1] + p[3]) + (p[5] + p[7]);
        lo[1] += (p[2] + p[3]) + (p[6] + p[7]);
        lo[2] += (p[4] + p[5]) + (p[6] + p[7]);
        for (uint32_t r = 0; r < nhi; ++r)
            if ((it >> r) & 1ULL) hi[r] += t;
    }
    for (uint32_t q = 0; q <= n; ++q) {
        double v;
        if (q == n) v = tot;
        else if (q < 3) v = lo[q];
        else if (q < 3 + s_log) v = ((gtid >> (q - 3)) & 1ULL) ? tot : 0.0;
        else v = hi[q - 3 - s_log];
        v = block_sum(v, red);
        if (threadIdx.x == 0) partial[(size_t)blockIdx.x * (n + 1) + q] = v;
    }
}

// States too small for 8-amplitude chunks over a full warp: one thread.
template <typename C>
__global__ void k_na_zsum_small(const C *__restrict__ a, uint32_t n, double *__restrict__ partial) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[kNaVals];
    for (uint32_t q = 0; q <= n; ++q) s[q] = 0.0;
    for (uint64_t i = 0; i < (1ULL << n); ++i) {
        const double p = na_p(a, i);
        s[n] += p;
        for (uint32_t q = 0; q < n; ++q)
            if ((i >> q) & 1ULL) s[q] += p;
    }
    for (uint32_t q = 0; q <= n; ++q) partial[q] = s[q];
}

// final[q] = sum over blocks of partial[block][q], in block order
__global__ void k_na_final(const double *__restrict__ partial, uint32_t blocks, uint32_t vals, double *__restrict__ final_) {
    for (uint32_t v = threadIdx.x; v < vals; v += blockDim.x) {
        double s = 0.0;
        for (uint32_t b = 0; b < blocks; ++b) s += partial[(size_t)b * vals + v];
        final_[v] = s;
    }
}

// Makes `device` current for the call and gives the caller's device back on
// every return path: the hosts this entry point serves manage their own
// current device.
struct DeviceGuard {
    int saved = -1;
    cudaError_t enter(int device) {
        cudaError_t e = cudaGetDevice(&saved);
        if (e != cudaSuccess) {
            saved = -1;
            return e;
        }
        return saved == device ? cudaSuccess : cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (saved >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != saved) cudaSetDevice(saved);
    }
};

template <typename C>
int na_launch(const C *a, uint32_t n, cudaStream_t stream, double *scratch, uint32_t *blocks_out) {
    uint32_t blocks = 1;
    if (n < 3 + 5) {
        k_na_zsum_small<C><<<1, 32, 0, stream>>>(a, n, scratch);
    } else {
        const uint32_t s_log = std::min<uint32_t>(16, n - 3);  // 2^16 = kNaMaxBlocks * kNaThreads threads at most
        const uint32_t threads_total = 1u << s_log;
        const uint32_t tpb = std::min<uint32_t>(kNaThreads, threads_total);
        blocks = threads_total / tpb;
        k_na_zsum<C><<<blocks, tpb, 0, stream>>>(a, n, s_log, scratch);
    }
    QF_CUDA(cudaGetLastError());
    *blocks_out = blocks;
    return QF_OK;
}

}  // namespace
}  // namespace qf

using namespace qf;

extern "C" int qf_expectation_z_all_noalloc(int device, const void *d_amps, uint32_t qubits, int dtype, void *stream,
                                            double *out, uint64_t n_out) {
    clear_error();
    if (dtype != QF_C64 && dtype != QF_C128) return fail(QF_ERR_INVALID_ARGUMENT, "unknown dtype %d", dtype);
    if (qubits == 0) return fail(QF_ERR_ZERO_QUBITS, "a state vector must contain at least one qubit");
    if (qubits > kNaMaxQubits)
        return fail(QF_ERR_STATE_TOO_LARGE,
                    "the allocation-free <Z> reduction takes at most %u qubits (its fixed scratch holds %u values per block), got %u",
                    kNaMaxQubits, kNaVals, qubits);
    if (!d_amps || !out) return fail(QF_ERR_INVALID_ARGUMENT, "amplitude or output pointer is NULL");
    if (n_out != qubits) return fail(QF_ERR_INVALID_ARGUMENT, "expected %u outputs, got %llu", qubits, (unsigned long long)n_out);
    const size_t align = dtype == QF_C64 ? 8 : 16;
    if (reinterpret_cast<uintptr_t>(d_amps) % align)
        return fail(QF_ERR_INVALID_ARGUMENT, "amplitudes must be %zu-byte aligned", align);
    if (device < 0 || device >= 64) return fail(QF_ERR_INVALID_ARGUMENT, "device %d is out of range", device);
    DeviceGuard guard;
    QF_CUDA(guard.enter(device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (s) {  // a stream of another device would fail later with a generic launch error
        int sdev = -1;
        QF_CUDA(cudaStreamGetDevice(s, &sdev));
        if (sdev != device)
            return fail(QF_ERR_INVALID_ARGUMENT, "the stream belongs to device %d, not to device %d", sdev, device);
    }
    double *scratch = nullptr;
    QF_TRY(na_scratch(device, &scratch));
    uint32_t blocks = 1;
    if (dtype == QF_C64) QF_TRY(na_launch(static_cast<const float2 *>(d_amps), qubits, s, scratch, &blocks));
    else QF_TRY(na_launch(static_cast<const double2 *>(d_amps), qubits, s, scratch, &blocks));
    double *final_ = scratch + (size_t)kNaMaxBlocks * kNaVals;
    k_na_final<<<1, 64, 0, s>>>(scratch, blocks, qubits + 1, final_);
    QF_CUDA(cudaGetLastError());
    double sums[kNaVals];
    QF_CUDA(cudaMemcpyAsync(sums, final_, sizeof(double) * (qubits + 1), cudaMemcpyDeviceToHost, s));
    QF_CUDA(cudaStreamSynchronize(s));
    for (uint32_t q = 0; q < qubits; ++q) out[q] = sums[qubits] - 2.0 * sums[q];
    return QF_OK;
}
