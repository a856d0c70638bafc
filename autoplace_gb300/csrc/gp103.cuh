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
bool pdl_enabled();
long long tc_wait_ns();     // GP103_OPT_WAIT_MS, in ns: the limit of a tensor-core field wait
bool tc_test_stall();       // GP103_OPT_TEST_STALL_FIELD
int wa_long_share();        // GP103_OPT_WA_FUSED: percent of the fused WA launch's blocks on long nets (0: two launches)
int field_early();          // GP103_OPT_FIELD_EARLY: bit 0 constant operand before the wait, bit 1 early trigger

// Programmatic dependent launch: a kernel may be launched while the one before it on the stream is finishing; it
// waits here (at its very start, before touching any data) until that one has completed and its writes are
// visible. Without the launch attribute this is a no-op. A kernel signals, once its blocks are past their main
// work, that the next one may start launching.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Launch with the programmatic-serialization attribute (when enabled): successive kernels of a pass overlap their
// launch with the tail of the previous kernel; in a captured graph the edges become programmatic edges.
template <typename... KArgs, typename... Args>
cudaError_t launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

constexpr double DENSITY_SCALE = 4294967296.0;     // fixed point of the density map: 2^32 per bin area
constexpr int SMS = 152;                           // GB300: 2 dies x 76 SMs

__host__ __device__ inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// The blocks of `kernel` that are resident on the whole GPU at `threads` per block (its occupancy x the SMs): the
// grid of a grid-stride loop in which every block stays busy to the end, with no second wave, and which writes as
// few reduction partials as that allows. Callers keep it in a function-local static (one query per kernel).
template <typename K>
inline int resident_blocks(K kernel, int threads, size_t smem = 0) {
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess || per < 1) per = 1;
    return per * SMS;
}

// Field mode f16x3: the power-of-two exponent e that scales a chunk of largest magnitude mx into [2^14, 2^15)
// (float16 terms with room to spare), clamped to [-100, 100] so that every factor 2^(+-e - 14) stays a normal
// float32 (a chunk of zeros or of subnormals gets 100).
__device__ __forceinline__ int f16_chunk_exp(float mx) {
    const int be = (int)((__float_as_uint(mx) >> 23) & 0xFFu);
    const int e = be == 0 ? 100 : 14 - (be - 127);
    return min(max(e, -100), 100);
}

// x rounded to tf32 (10 mantissa bits, to nearest, ties away from zero), as a float32 with its low 13 bits zero: the
// first term of a tf32 split; x - tf32_round(x) is exact, and its own rounding is the second term.
__device__ __forceinline__ float tf32_round(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r & 0xffffe000u);
}

// Grid for a grid-stride loop over n items: at most `per_sm` blocks per SM, at least one block.
inline int grid_for(long long n, int threads, int per_sm) {
    long long g = (n + threads - 1) / threads;
    long long cap = (long long)SMS * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// ----------------------------------------------------------------------------- deterministic float64 reductions
// A producing kernel writes one partial sum per block, in a fixed slot per block (no atomics, no "last block"
// tail); the kernel that consumes the value adds the partials in block order with a whole block. The result does
// not depend on the scheduling of the blocks: bit-identical on every run.
constexpr int MAX_BLOCKS = 2048;
struct Reduce {
    double* partials;       // [K][MAX_BLOCKS]
    int* count;             // number of partials, written by block 0 of the producer
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

// Producer side: the blocks taking part are numbered bid = 0 .. nblk - 1 (<= MAX_BLOCKS; a launch may hold several
// independent reductions).
template <int K>
__device__ __forceinline__ void grid_sum(double (&v)[K], const Reduce& r, int nblk, int bid) {
    __shared__ double sh[K * 32];
    pdl_trigger();                          // the main work is done: the next kernel may start launching
    block_sum<K>(v, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) r.partials[(size_t)k * MAX_BLOCKS + bid] = v[k];
        if (bid == 0) *r.count = nblk;
    }
}

template <int K>
__device__ __forceinline__ void grid_sum(double (&v)[K], const Reduce& r) {
    grid_sum<K>(v, r, (int)gridDim.x, (int)blockIdx.x);
}

// Producer side for float32 per-thread partials (the hot kernels): a fixed float32 tree inside each warp, then the
// warp totals in float64 across the block, so a block spends 1 + log2(warps) float64 warp instructions per value
// (GB300's float64 rate is 1/64 of its float32 rate: a float64 tree over every lane costs more than the kernel's own
// arithmetic in the short kernels).
template <int K>
__device__ __forceinline__ void grid_sum(float (&v)[K], const Reduce& r, int nblk, int bid) {
    __shared__ float shf[K * 32];
    pdl_trigger();
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (l == 0)
#pragma unroll
        for (int k = 0; k < K; k++) shf[k * 32 + w] = v[k];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            double d = l < nw ? (double)shf[k * 32 + l] : 0.0;
            for (int o = 16; o > 0; o >>= 1)
                if (o < nw) d += __shfl_down_sync(0xffffffffu, d, o);
            if (l == 0) r.partials[(size_t)k * MAX_BLOCKS + bid] = d;
        }
        if (l == 0 && bid == 0) *r.count = nblk;
    }
}

template <int K>
__device__ __forceinline__ void grid_sum(float (&v)[K], const Reduce& r) {
    grid_sum<K>(v, r, (int)gridDim.x, (int)blockIdx.x);
}


// Consumer side (every thread of the block calls it): value k of a reduction, returned to every thread.
__device__ __forceinline__ double block_total(const Reduce& r, int k) {
    __shared__ double sh[32];
    __shared__ double total;
    const int n = *r.count;
    double v[1] = {0.0};
    const double* p = r.partials + (size_t)k * MAX_BLOCKS;
    const int T = blockDim.x;
    for (int b = threadIdx.x; b < n; b += 4 * T) {              // four loads in flight per step, added in order
        double x[4];
#pragma unroll
        for (int u = 0; u < 4; u++) x[u] = b + u * T < n ? p[b + u * T] : 0.0;
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (b + u * T < n) v[0] += x[u];
    }
    block_sum<1>(v, sh);
    if (threadIdx.x == 0) total = v[0];
    __syncthreads();
    const double t = total;
    __syncthreads();
    return t;
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
// trunc(f * 2^32) as a 64-bit integer, exactly what (unsigned long long)((double)f * 2^32) gives (the double holds
// f and the product exactly; the conversion truncates and saturates, NaN and negatives give 0), from the bits of f:
// f = m 2^(e - 150) with a 24-bit m, so f 2^32 = m 2^(e - 118). Integer work only (GB300's float64 rate is 1/64 of
// its float32 rate).
__device__ __forceinline__ unsigned long long fixed32(float f) {
    const unsigned int b = __float_as_uint(f);
    if (b & 0x80000000u) return 0ull;                              // negative (or -0, -NaN)
    const int e = (int)(b >> 23);
    if (e == 0xff) return (b & 0x7fffffu) ? 0ull : ~0ull;          // NaN -> 0, +inf saturates
    if (e == 0) return 0ull;                                       // zero / denormal: below 2^-32
    const unsigned long long m = (unsigned long long)((b & 0x7fffffu) | 0x800000u);
    const int sh = e - 118;
    if (sh >= 0) return sh > 40 ? ~0ull : (m << sh);
    return sh <= -24 ? 0ull : (m >> -sh);
}
// Fixed-point charge of one (node, bin) pair: trunc(float(wx * oy) * 2^32).
__device__ __forceinline__ unsigned long long charge(float wx, float oy) { return fixed32(__fmul_rn(wx, oy)); }

// (float)((double)q / 2^32) of a map entry. Below 2^53 the double is exact and one rounding to float is all there
// is: q 2^-32 rounded to nearest even, built here from q's bits on the integer pipes (64-bit integer conversions
// run on GB300's float64 pipe, at 1/64 of the float32 rate). The float is m 2^(e - 150) with the 24 leading bits
// of q as m; the bits shifted out decide the rounding (above half: up; exactly half: up to even). No float denormal
// can occur: the smallest non-zero value is 2^-32.
// m 2^(e2 - 32) rounded to float (nearest even), m < 2^54: the float is m' 2^(top - 23 - 32) with the 24 leading
// bits of m as m' (the bits shifted out decide the rounding: above half up, exactly half up to even).
__device__ __forceinline__ float round_to_float(unsigned long long m, int e2) {
    if (m == 0ull) return 0.f;
    const int msb = 63 - __clzll(m);
    unsigned int f;
    int top = msb;
    if (msb <= 23) {
        f = (unsigned int)m << (23 - msb);                 // exact
    } else {
        const int sh = msb - 23;
        f = (unsigned int)(m >> sh);
        const unsigned long long rest = m & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rest > half || (rest == half && (f & 1u))) {
            f += 1u;
            if (f == (1u << 24)) {                         // carried into a new leading bit
                f >>= 1;
                top += 1;
            }
        }
    }
    return __uint_as_float(((unsigned int)(top + e2 + 95) << 23) | (f & 0x7fffffu));
}

// (float)((double)q / 2^32) of a map entry, on the integer pipes (64-bit integer conversions run on GB300's float64
// pipe, at 1/64 of the float32 rate). Below 2^53 the double is exact and one rounding to float is all there is; above,
// q is first rounded to the 53 bits of a double (nearest even), then to float. No float denormal can occur: the
// smallest non-zero value is 2^-32.
__device__ __forceinline__ float unfixed32(unsigned long long q) {
    if (q < (1ull << 53)) return round_to_float(q, 0);
    const int sh = (63 - __clzll(q)) - 52;                 // 1 .. 11
    unsigned long long m = q >> sh;
    const unsigned long long rest = q & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    if (rest > half || (rest == half && (m & 1ull))) m += 1ull;   // may reach 2^53: still exact below
    return round_to_float(m, sh);
}

}  // namespace gp103
