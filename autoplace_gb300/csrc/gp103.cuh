// Shared device helpers of the gp103 kernels (GB300, sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gp103.h"

// After every kernel launch (stream `s` in scope): the launch status, the library's launch count and, while a
// profile is open, an event on the stream named after the launching function.
#define GP103_CHECK_LAUNCH()                                   \
    do {                                                       \
        int e_ = gp103::after_launch(s, __func__);             \
        if (e_) return e_;                                     \
    } while (0)

namespace gp103 {

int after_launch(cudaStream_t s, const char* name);

constexpr double DENSITY_SCALE = 4294967296.0;     // fixed point of the density map: 2^32 per bin area
constexpr int SMS = 152;                           // GB300: 2 dies x 76 SMs

__host__ __device__ inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Grid for a grid-stride loop over n items: at most `per_sm` blocks per SM, at least one block.
inline int grid_for(long long n, int threads, int per_sm) {
    long long g = (n + threads - 1) / threads;
    long long cap = (long long)SMS * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// ----------------------------------------------------------------------------- deterministic float64 reductions
// Per-block partial sums in a fixed slot per block; the last block to finish adds the partials in block order.
// The result does not depend on which block finishes last: bit-identical on every run.
struct Reduce {
    double* partials;       // [K][max_blocks]
    unsigned int* counter;  // one counter, zero between uses (the last block resets it)
    double* out;            // [K]
};

template <int K>
__device__ __forceinline__ void warp_sum(double (&v)[K]) {
#pragma unroll
    for (int k = 0; k < K; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
}

// Block-wide sum (fixed tree); thread 0 gets the totals. Uses `sh` (>= K * 32 doubles of shared memory).
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* sh) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    warp_sum<K>(v);
    __syncthreads();
    if (l == 0)
#pragma unroll
        for (int k = 0; k < K; k++) sh[k * 32 + w] = v[k];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = l < nw ? sh[k * 32 + l] : 0.0;
        warp_sum<K>(v);
    }
}

// The blocks taking part are numbered bid = 0 .. nblk - 1 (a launch may hold several independent reductions).
template <int K>
__device__ __forceinline__ void grid_sum(double (&v)[K], const Reduce& r, int nblk, int bid) {
    __shared__ double sh[K * 32];
    __shared__ bool last;
    block_sum<K>(v, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) r.partials[(size_t)k * nblk + bid] = v[k];
        __threadfence();
        unsigned int t = atomicAdd(r.counter, 1u);
        last = (t == (unsigned int)nblk - 1);
    }
    __syncthreads();
    if (last) {
        __threadfence();
        double s[K];
#pragma unroll
        for (int k = 0; k < K; k++) s[k] = 0.0;
        for (int b = threadIdx.x; b < nblk; b += blockDim.x)
#pragma unroll
            for (int k = 0; k < K; k++) s[k] += __ldcg(r.partials + (size_t)k * nblk + b);
        block_sum<K>(s, sh);
        if (threadIdx.x == 0) {
#pragma unroll
            for (int k = 0; k < K; k++) r.out[k] = s[k];
            *r.counter = 0;
        }
    }
}

template <int K>
__device__ __forceinline__ void grid_sum(double (&v)[K], const Reduce& r) {
    grid_sum<K>(v, r, (int)gridDim.x, (int)blockIdx.x);
}

// ----------------------------------------------------------------------------- node span on a bin grid
// The float32 operation order of the reference's span / overlap (cpp_to_py/gp_cuda_kernel.cu:73-82): the density
// map built from it is the same integer map.
struct Span {
    float lo, hi;
    int b0, b1;
};
__device__ __forceinline__ Span span(float centre, float size, float inv_bin, int nb) {
    Span s;
    const float half = __fmul_rn(0.5f, size);
    s.lo = __fmul_rn(__fsub_rn(centre, half), inv_bin);
    s.hi = __fmul_rn(__fadd_rn(centre, half), inv_bin);
    s.b0 = max((int)floorf(s.lo), 0);
    s.b1 = min((int)floorf(s.hi), nb - 1);
    return s;
}
__device__ __forceinline__ float overlap(const Span& s, int b) {
    return fmaxf(__fsub_rn(fminf(s.hi, __fadd_rn((float)b, 1.f)), fmaxf(s.lo, (float)b)), 0.f);
}
// Fixed-point charge of one (node, bin) pair: trunc(float(wx * oy) * 2^32).
__device__ __forceinline__ unsigned long long charge(float wx, float oy) {
    return (unsigned long long)((double)__fmul_rn(wx, oy) * DENSITY_SCALE);
}

}  // namespace gp103
