// qf_device.cuh — device helpers shared by the kernels: complex arithmetic on
// float2/double2, index bit manipulation and block reductions.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace qf {

template <typename C> struct Real;
template <> struct Real<float2> { using T = float; };
template <> struct Real<double2> { using T = double; };

__device__ __forceinline__ float2 mk(float re, float im) { return make_float2(re, im); }
__device__ __forceinline__ double2 mk(double re, double im) { return make_double2(re, im); }

template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) {
    C r;
    r.x = a.x + b.x;
    r.y = a.y + b.y;
    return r;
}
// m0 * a0 + m1 * a1
template <typename C> __device__ __forceinline__ C cmac2(C m0, C a0, C m1, C a1) {
    C r;
    r.x = m0.x * a0.x - m0.y * a0.y + m1.x * a1.x - m1.y * a1.y;
    r.y = m0.x * a0.y + m0.y * a0.x + m1.x * a1.y + m1.y * a1.x;
    return r;
}
template <typename C> __device__ __forceinline__ C cneg(C a) {
    C r;
    r.x = -a.x;
    r.y = -a.y;
    return r;
}
template <typename C> __device__ __forceinline__ bool is_one(C a) { return a.x == 1 && a.y == 0; }

// Insert a zero bit at position b of p.
__device__ __forceinline__ uint64_t insert0(uint64_t p, uint32_t b) {
    const uint64_t lowm = (1ULL << b) - 1;
    return ((p & ~lowm) << 1) | (p & lowm);
}
__device__ __forceinline__ uint32_t insert0_32(uint32_t p, uint32_t b) {
    const uint32_t lowm = (1u << b) - 1;
    return ((p & ~lowm) << 1) | (p & lowm);
}
// Insert zeros at positions lo < hi.
__device__ __forceinline__ uint64_t insert00(uint64_t p, uint32_t lo, uint32_t hi) {
    return insert0(insert0(p, lo), hi);
}
__device__ __forceinline__ uint32_t insert00_32(uint32_t p, uint32_t lo, uint32_t hi) {
    return insert0_32(insert0_32(p, lo), hi);
}
// Scatter the low bits of v onto the set bits of mask (bit-deposit).
__device__ __forceinline__ uint64_t deposit(uint64_t v, uint64_t mask) {
    uint64_t r = 0;
    while (mask && v) {
        const uint64_t lowest = mask & (~mask + 1);
        if (v & 1ULL) r |= lowest;
        v >>= 1;
        mask &= mask - 1;
    }
    return r;
}

// Sum over the block; result valid in thread 0. `scratch` holds one value per warp.
template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <typename T> __device__ __forceinline__ T block_sum(T v, T *scratch) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    T r = 0;
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        r = lane < nw ? scratch[lane] : T(0);
        r = warp_sum(r);
    }
    return r;
}

}  // namespace qf
