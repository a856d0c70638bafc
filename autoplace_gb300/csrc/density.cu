// Density: fixed-point charge scatter, map post-processing and the field gather (GB300, sm_103a).
//
// Reference: cpp_to_py/gp_cuda_kernel.cu:67-153 (density_map_kernel, density_post_kernel, density_grad_kernel) and
// src/core/electronic_density_layer.py:96-149. The charge of a (node, bin) pair is the reference's float32 product
// truncated to 2^-32 bin areas and summed as 64-bit integers: the map is the same integers in any summation order.
// This file is built with -ftz=true, as the reference's kernels are (--use_fast_math), so that even denormal
// intermediates round the same way.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "gp103.cuh"
#include "kernels.cuh"

namespace gp103 {

// ----------------------------------------------------------------------------- scatter
// A block takes a chunk of SCAT_CHUNK consecutive nodes (in the spatial order when one is given), all movable or all
// fillers. If the bins its nodes touch fit in shared memory (bounding box <= SCAT_SMEM_BINS), the block sums its
// charges there and then adds every non-zero bin to the global map once; otherwise it adds each charge to the global
// map directly (64-bit atomics in L2).
constexpr int SCAT_THREADS = 384;
constexpr int SCAT_PER_THREAD = 2;
constexpr int SCAT_CHUNK = SCAT_THREADS * SCAT_PER_THREAD;   // 768 nodes (measured: 512 and 1024 nodes, and 256 x 3 or 128 x 6 threads x nodes, are slower)
static_assert((long long)SCAT_CHUNK << 17 < (1LL << 32), "the shared-memory charge words could wrap");
constexpr int SCAT_SMEM_BINS = 3072;      // 2 x 12 KB of 32-bit words
constexpr float TWO32 = 4294967296.f, TWO33 = 8589934592.f, TWO_M32 = 2.3283064365386963e-10f;

__device__ __forceinline__ void red_shared(unsigned int* a, unsigned int v) {
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"((unsigned int)__cvta_generic_to_shared(a)), "r"(v) : "memory");
}

// Where a block's charges go. A charge is v = float(wx * oy) * 2^32 (the scaling is exact), truncated to an integer
// q. In shared memory q < 2^33 is kept as two 32-bit sums: its low 16 bits in lo[b], the rest in hi[b], by adds
// whose old values nobody reads. A block adds at most SCAT_CHUNK charges to a bin (one per node), so neither word
// can wrap (SCAT_CHUNK x 2^17 < 2^32, checked below) and the bin's sum is hi * 2^16 + lo exactly. Larger charges (only
// from ratios above 1), infinities and NaNs take the exact 64-bit conversion and a global atomic.
struct Tally {
    unsigned int* lo;
    unsigned int* hi;
    unsigned long long* map;
    int nby, bx0, by0, H;
    bool local;

    __device__ __forceinline__ void add(int x, int y, float v) const {
        unsigned int q, top;
        if (v < TWO32) {
            q = __float2uint_rz(v);                                  // negatives and -inf clamp to 0
            top = 0u;
        } else if (v < TWO33) {
            q = __float2uint_rz(__fsub_rn(v, TWO32));                // exact: v is a multiple of 2^9 here
            top = 1u;
        } else {
            const unsigned long long Q = fixed32(__fmul_rn(v, TWO_M32));
            if (Q) atomicAdd(&map[(size_t)x * nby + y], Q);
            return;
        }
        if ((q | top) == 0u) return;
        if (local) {
            const int b = (x - bx0) * H + (y - by0);
            red_shared(lo + b, q & 0xffffu);
            red_shared(hi + b, (q >> 16) | (top << 16));
        } else {
            atomicAdd(&map[(size_t)x * nby + y], (unsigned long long)q | ((unsigned long long)top << 32));
        }
    }
};

// Overlaps of a span with its first three bins b0, b0 + 1, b0 + 2: overlap() with the bin edges formed by exact
// float additions ((float)(b0 + k) == (float)b0 + k below 2^24).
__device__ __forceinline__ void overlaps3(const Span& s, float (&o)[3]) {
    const float e0 = (float)s.b0, e1 = __fadd_rn(e0, 1.f), e2 = __fadd_rn(e0, 2.f), e3 = __fadd_rn(e0, 3.f);
    o[0] = fmaxf(__fsub_rn(fminf(s.hi, e1), fmaxf(s.lo, e0)), 0.f);
    o[1] = fmaxf(__fsub_rn(fminf(s.hi, e2), fmaxf(s.lo, e1)), 0.f);
    o[2] = fmaxf(__fsub_rn(fminf(s.hi, e3), fmaxf(s.lo, e2)), 0.f);
}

// The charges of one node. wx is scaled by 2^32 before the product: float(wx * oy) * 2^32 equals
// float(wx 2^32 * oy) whenever the former is a normal float, and both truncate to 0 below that.
// Fast case (every node whose smoothed size is under 2 bins, with a ratio up to 1): both spans have at most 3 bins
// and the largest product is below 2^32 (rounding is monotonic, so then every product is), so all 9 charges are
// plain 32-bit truncations added to shared memory, unrolled and predicated. Anything else takes Tally::add.
__device__ __forceinline__ void node_charges(const Tally& t, const Span& sx, const Span& sy, float ratio) {
    const int nx = sx.b1 - sx.b0, ny = sy.b1 - sy.b0;
    if (nx < 0 || ny < 0) return;
    if (nx <= 2 && ny <= 2) {
        float wx[3], oy[3];
        overlaps3(sx, wx);
        overlaps3(sy, oy);
#pragma unroll
        for (int a = 0; a < 3; a++) wx[a] = __fmul_rn(__fmul_rn(ratio, wx[a]), TWO32);
        const float vmax = __fmul_rn(fmaxf(fmaxf(wx[0], wx[1]), wx[2]), fmaxf(fmaxf(oy[0], oy[1]), oy[2]));
        if (t.local && vmax < TWO32) {
            const int base = (sx.b0 - t.bx0) * t.H + (sy.b0 - t.by0);
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int c = 0; c < 3; c++)
                    if (a <= nx && c <= ny) {
                        const unsigned int q = __float2uint_rz(__fmul_rn(wx[a], oy[c]));
                        const int b = base + a * t.H + c;
                        red_shared(t.lo + b, q & 0xffffu);
                        red_shared(t.hi + b, q >> 16);
                    }
            return;
        }
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int c = 0; c < 3; c++)
                if (a <= nx && c <= ny) t.add(sx.b0 + a, sy.b0 + c, __fmul_rn(wx[a], oy[c]));
        return;
    }
    for (int x = sx.b0; x <= sx.b1; x++) {
        const float wx = __fmul_rn(__fmul_rn(ratio, overlap(sx, x)), TWO32);
        for (int y = sy.b0; y <= sy.b1; y++) t.add(x, y, __fmul_rn(wx, overlap(sy, y)));
    }
}

__global__ void __launch_bounds__(SCAT_THREADS) scatter_kernel(const __grid_constant__ ScatterPair pair) {
    pdl_wait();
    __shared__ __align__(16) unsigned int tlo[SCAT_SMEM_BINS];
    __shared__ __align__(16) unsigned int thi[SCAT_SMEM_BINS];
    __shared__ int box[4];
    const bool second = (int)blockIdx.x >= pair.blocks0;
    const ScatterJob& j = second ? pair.j[1] : pair.j[0];
    const int bid = second ? (int)blockIdx.x - pair.blocks0 : (int)blockIdx.x;
    const float2* pos = pick(j.pos_a, j.pos_b, j.sel);
    const int cell_chunks = ceil_div(j.num_mov, SCAT_CHUNK);
    int first, last;
    unsigned long long* map;
    if (bid < cell_chunks) {
        first = bid * SCAT_CHUNK;
        last = min(first + SCAT_CHUNK, j.num_mov);
        map = j.map0;
    } else {
        first = j.num_mov + (bid - cell_chunks) * SCAT_CHUNK;
        last = min(first + SCAT_CHUNK, j.num_nodes);
        map = j.map1;
    }
    if (threadIdx.x == 0) { box[0] = INT_MAX; box[1] = INT_MIN; box[2] = INT_MAX; box[3] = INT_MIN; }
    Span sx[SCAT_PER_THREAD], sy[SCAT_PER_THREAD];
    float ratio[SCAT_PER_THREAD];
    int x0 = INT_MAX, x1 = INT_MIN, y0 = INT_MAX, y1 = INT_MIN;
#pragma unroll
    for (int k = 0; k < SCAT_PER_THREAD; k++) {
        const int at = first + k * SCAT_THREADS + threadIdx.x;
        sx[k].b0 = 1; sx[k].b1 = 0; sy[k].b0 = 1; sy[k].b1 = 0; ratio[k] = 0.f;
        if (at < last) {
            int i = at;
            if (j.order) {
                const int o = j.order[at];
                if ((unsigned)o < (unsigned)j.num_nodes) i = o;      // an order must be a permutation; never leave the arrays
            }
            const float2 p = pos[i], s = j.size[i];
            sx[k] = span(p.x, s.x, j.inv_bx, j.nbx);
            sy[k] = span(p.y, s.y, j.inv_by, j.nby);
            ratio[k] = j.ratio ? j.ratio[i] : 1.f;
            if (sx[k].b0 <= sx[k].b1 && sy[k].b0 <= sy[k].b1) {
                x0 = min(x0, sx[k].b0); x1 = max(x1, sx[k].b1);
                y0 = min(y0, sy[k].b0); y1 = max(y1, sy[k].b1);
            }
        }
    }
    x0 = __reduce_min_sync(0xffffffffu, x0); x1 = __reduce_max_sync(0xffffffffu, x1);
    y0 = __reduce_min_sync(0xffffffffu, y0); y1 = __reduce_max_sync(0xffffffffu, y1);
    __syncthreads();
    if ((threadIdx.x & 31) == 0 && x0 <= x1) {
        atomicMin(&box[0], x0); atomicMax(&box[1], x1); atomicMin(&box[2], y0); atomicMax(&box[3], y1);
    }
    __syncthreads();
    const int bx0 = box[0], bx1 = box[1], by0 = box[2], by1 = box[3];
    if (bx0 > bx1 || map == nullptr) return;                       // nothing to add (uniform over the block)
    const long long w = (long long)(bx1 - bx0 + 1), h = (long long)(by1 - by0 + 1);
    Tally t;
    t.lo = tlo; t.hi = thi; t.map = map; t.nby = j.nby; t.bx0 = bx0; t.by0 = by0; t.H = (int)h;
    t.local = w * h <= SCAT_SMEM_BINS;
    const int area = t.local ? (int)(w * h) : 0;
    const int quads = (area + 3) >> 2;
    for (int k = threadIdx.x; k < quads; k += SCAT_THREADS) {
        ((uint4*)tlo)[k] = make_uint4(0u, 0u, 0u, 0u);
        ((uint4*)thi)[k] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SCAT_PER_THREAD; k++) node_charges(t, sx[k], sy[k], ratio[k]);
    if (!t.local) return;
    __syncthreads();
    // row = b / H by a multiply: magic = ceil(2^32 / H) is exact for b * (magic * H - 2^32) < 2^32, here < 2^26
    const unsigned long long magic = ((1ull << 32) + (unsigned long long)(t.H - 1)) / (unsigned long long)t.H;
    for (int b = threadIdx.x; b < area; b += SCAT_THREADS) {
        const unsigned long long q = ((unsigned long long)thi[b] << 16) + tlo[b];
        if (q) {
            const int row = (int)(((unsigned long long)b * magic) >> 32);
            atomicAdd(&map[(size_t)(bx0 + row) * j.nby + (by0 + b - row * t.H)], q);
        }
    }
}

static int scatter_blocks(const ScatterJob& j) {
    return ceil_div(j.num_mov, SCAT_CHUNK) + ceil_div(j.num_nodes - j.num_mov, SCAT_CHUNK);
}

int launch_scatter(const ScatterJob* jobs, int njobs, cudaStream_t s) {
    ScatterPair p = {};
    p.j[0] = jobs[0];
    p.j[1] = njobs > 1 ? jobs[1] : jobs[0];
    p.njobs = njobs;
    p.blocks0 = scatter_blocks(jobs[0]);
    const int blocks = p.blocks0 + (njobs > 1 ? scatter_blocks(jobs[1]) : 0);
    if (blocks == 0) return GP103_OK;
    if (launch_k(scatter_kernel, dim3(blocks), dim3(SCAT_THREADS), 0, s, p) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// ----------------------------------------------------------------------------- spatial order
// Exclusive scan of the per-tile counts into the cursors (one block; at most ORDER_MAX_KEYS keys), counts zeroed
// for the next count.
__global__ void __launch_bounds__(1024) order_scan_kernel(OrderJob o) {
    __shared__ int warp_total[32];
    pdl_wait();
    const int keys = 2 * o.tiles_x * o.tiles_y, t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int a = 2 * t < keys ? o.counts[2 * t] : 0, b = 2 * t + 1 < keys ? o.counts[2 * t + 1] : 0;
    const int sum = a + b;
    int x = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warp_total[w] = x;
    __syncthreads();
    if (w == 0) {
        const int orig = lane < (int)(blockDim.x >> 5) ? warp_total[lane] : 0;
        int z = orig;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, z, off);
            if (lane >= off) z += y;
        }
        warp_total[lane] = z - orig;
    }
    __syncthreads();
    const int excl = x - sum + warp_total[w];
    if (2 * t < keys) {
        o.cursor[2 * t] = excl;
        o.counts[2 * t] = 0;
    }
    if (2 * t + 1 < keys) {
        o.cursor[2 * t + 1] = excl + a;
        o.counts[2 * t + 1] = 0;
    }
}

// Every node takes the next slot of its tile (one atomic per group of lanes with the same tile).
__global__ void __launch_bounds__(256) order_place_kernel(OrderJob o, const float2* pos_a, const float2* pos_b,
                                                          const int* sel) {
    pdl_wait();
    const float2* pos = pick(pos_a, pos_b, sel);
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < o.num_nodes; base += stride) {
        const int i = base + lane;
        const bool valid = i < o.num_nodes;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        const int key = order_key(o, pos[i], i);
        const unsigned grp = __match_any_sync(act, key);
        const int leader = __ffs(grp) - 1;
        int slot = 0;
        if (lane == leader) slot = atomicAdd(&o.cursor[key], __popc(grp));
        slot = __shfl_sync(grp, slot, leader);
        o.order[slot + __popc(grp & ((1u << lane) - 1u))] = i;
    }
}

int launch_order(const OrderJob& o, const float2* pos_a, const float2* pos_b, const int* sel, bool counted,
                 cudaStream_t s) {
    if (!counted || 2 * o.tiles_x * o.tiles_y > ORDER_MAX_KEYS) return GP103_ERR_ARG;
    if (launch_k(order_scan_kernel, dim3(1), dim3(1024), 0, s, o) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (launch_k(order_place_kernel, dim3(grid_for(o.num_nodes, 256, 8)), dim3(256), 0, s, o, pos_a, pos_b, sel) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// ----------------------------------------------------------------------------- post
// Reference layout: rho mirrored [2 nbx][2 nby] and over [nbx][nby] (density_post_kernel, gp_cuda_kernel.cu:130-139).
__global__ void post_mirror_kernel(const unsigned long long* map, const float* fixed, float target, int nbx, int nby,
                                   float* rho, float* over) {
    pdl_wait();
    const int nb = nbx * nby;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        const int bx = b / nby, by = b - bx * nby, w = 2 * nby, mx = 2 * nbx - 1 - bx, my = w - 1 - by;
        const float mov = __fadd_rn(unfixed32(map[b]), fixed[b]);
        const float r = __fadd_rn(mov, unfixed32(map[nb + b]));
        over[b] = fmaxf(__fsub_rn(mov, target), 0.f);
        rho[(size_t)bx * w + by] = r;
        rho[(size_t)bx * w + my] = r;
        rho[(size_t)mx * w + by] = r;
        rho[(size_t)mx * w + my] = r;
    }
}

int launch_post_mirror(const unsigned long long* map, const float* fixed, float target, int nbx, int nby, float* rho,
                       float* over, cudaStream_t s) {
    const int nb = nbx * nby;
    if (launch_k(post_mirror_kernel, dim3(grid_for(nb, 256, 8)), dim3(256), 0, s, map, fixed, target, nbx, nby, rho, over) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// Fused layout: the plain total density for the field (float32 plane, or the bf16 terms of its split) and the
// float64 sum of the density above the target; the map is zeroed behind the read for the next pass. Up to two
// grids per launch (force grid, overflow grid), each with its own reduction.
__device__ __forceinline__ void split_bf16(float r, int terms, __nv_bfloat16* t0, __nv_bfloat16* t1,
                                           __nv_bfloat16* t2, size_t at) {
    __nv_bfloat16 a = __float2bfloat16_rn(r);
    float rem = __fsub_rn(r, __bfloat162float(a));
    __nv_bfloat16 b = __float2bfloat16_rn(rem);
    t0[at] = a;
    t1[at] = b;
    if (terms > 2) t2[at] = __float2bfloat16_rn(__fsub_rn(rem, __bfloat162float(b)));
}

// f16x3 folded (j.fold, with exps and the filler plane; nby a multiple of 128): as the float16 path below, but the
// density goes out folded about the middle of y for the folded first transform of the field: s = rho(y) +
// rho(nby-1-y) and t = rho(y) - rho(nby-1-y) for y < nby/2, each [nbx][nby/2] as two float16 terms with a
// power-of-two scale per 64-value chunk of a row: planes s0, s1, t0, t1 of nbx * nby/2 values from j.t0 on; exponents
// of s at exps[(y / 64) * nbx + x], of t behind them. A thread takes the quad y .. y+3 of a row's lower half and its
// mirror nby-4-y .. nby-1-y (the mirror of y + k is the mirror quad's element 3 - k); a 64-value chunk is 16
// consecutive threads, half a warp (the loop keeps whole warps: nbx * nby / 8 is a multiple of 32).
__device__ __forceinline__ void post_fold(const PostJob& j, int bid, int nblk, float& ov) {
    const int nb = j.nbx * j.nby, hq = j.nby / 8, hy = j.nby / 2;
    const size_t hn = (size_t)j.nbx * hy;
    __half* out = (__half*)j.t0;
    ulonglong2* mov_map = (ulonglong2*)j.map;
    ulonglong2* fill = (ulonglong2*)(j.map + nb);
    for (int qp = bid * blockDim.x + threadIdx.x; qp < nb / 8; qp += nblk * blockDim.x) {
        const int x = qp / hq, y = 4 * (qp - x * hq);
        float r[2][4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int q = (x * j.nby + (h ? j.nby - 4 - y : y)) >> 2;      // the quad (of 4 bins)
            const ulonglong2 ma = mov_map[2 * q], mb = mov_map[2 * q + 1];
            const ulonglong2 fa = fill[2 * q], fb = fill[2 * q + 1];
            const float4 fx = *(const float4*)(j.fixed + 4 * q);
            float mov[4];
            mov[0] = __fadd_rn(unfixed32(ma.x), fx.x);
            mov[1] = __fadd_rn(unfixed32(ma.y), fx.y);
            mov[2] = __fadd_rn(unfixed32(mb.x), fx.z);
            mov[3] = __fadd_rn(unfixed32(mb.y), fx.w);
#pragma unroll
            for (int k = 0; k < 4; k++) ov += fmaxf(__fsub_rn(mov[k], j.target), 0.f);
            r[h][0] = __fadd_rn(mov[0], unfixed32(fa.x));
            r[h][1] = __fadd_rn(mov[1], unfixed32(fa.y));
            r[h][2] = __fadd_rn(mov[2], unfixed32(fb.x));
            r[h][3] = __fadd_rn(mov[3], unfixed32(fb.y));
            const ulonglong2 zero = make_ulonglong2(0ull, 0ull);
            mov_map[2 * q] = zero;
            mov_map[2 * q + 1] = zero;
            fill[2 * q] = zero;
            fill[2 * q + 1] = zero;
        }
        float sv[4], tv[4], ms = 0.f, mt = 0.f;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            sv[k] = __fadd_rn(__fsub_rn(r[0][k], j.shift), __fsub_rn(r[1][3 - k], j.shift));
            tv[k] = __fsub_rn(r[0][k], r[1][3 - k]);
            ms = fmaxf(ms, fabsf(sv[k]));
            mt = fmaxf(mt, fabsf(tv[k]));
        }
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            ms = fmaxf(ms, __shfl_xor_sync(0xffffffffu, ms, o));
            mt = fmaxf(mt, __shfl_xor_sync(0xffffffffu, mt, o));
        }
        const int es = f16_chunk_exp(ms), et = f16_chunk_exp(mt);
        const float scs = __int_as_float((127 + es) << 23), sct = __int_as_float((127 + et) << 23);
        __align__(8) __half h[4][4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float xs = sv[k] * scs, xt = tv[k] * sct;
            h[0][k] = __float2half_rn(xs);
            h[1][k] = __float2half_rn(__fsub_rn(xs, __half2float(h[0][k])));
            h[2][k] = __float2half_rn(xt);
            h[3][k] = __float2half_rn(__fsub_rn(xt, __half2float(h[2][k])));
        }
        const size_t at = (size_t)x * hy + y;
#pragma unroll
        for (int t = 0; t < 4; t++) *(uint2*)(out + t * hn + at) = *(const uint2*)h[t];
        if ((threadIdx.x & 15) == 0) {
            const size_t k = (size_t)(y >> 6) * j.nbx + x;
            j.exps[k] = (signed char)es;
            j.exps[(size_t)(hy >> 6) * j.nbx + k] = (signed char)et;
        }
    }
}

// EXACT: float64 per-thread partials of the overflow (the evaluators); a template argument, so that the hot path
// carries no float64 instruction at all (a runtime flag gets both sides if-converted).
template <bool EXACT>
__global__ void post_plain_kernel(const __grid_constant__ PostPair pair) {
    pdl_wait();
    const bool second = (int)blockIdx.x >= pair.blocks0;
    const PostJob& j = second ? pair.j[1] : pair.j[0];
    const int bid = second ? (int)blockIdx.x - pair.blocks0 : (int)blockIdx.x;
    const int nblk = second ? (int)gridDim.x - pair.blocks0 : pair.blocks0;
    const int nb = j.nbx * j.nby;
    float ov = 0.f;             // per-thread partial of the hot path (a few bins)
    double ovd = 0.0;           // the same in float64 for an exact evaluation (j.exact)
    if (!EXACT && j.fold) post_fold(j, bid, nblk, ov);
    // four bins per thread and iteration: 32-byte map loads / stores, 8-byte stores of each bf16 term plane (a bin
    // count that is a multiple of 4 keeps every plane aligned; any other takes the scalar loop below for every bin)
    const int quads = (nb & 3) || (!EXACT && j.fold) ? 0 : nb >> 2;
    for (int q = bid * blockDim.x + threadIdx.x; q < quads; q += nblk * blockDim.x) {
        const int b = 4 * q;
        const ulonglong2 m0a = ((const ulonglong2*)j.map)[2 * q], m0b = ((const ulonglong2*)j.map)[2 * q + 1];
        const float4 fx = *(const float4*)(j.fixed + b);
        float mov[4];
        mov[0] = __fadd_rn(unfixed32(m0a.x), fx.x);
        mov[1] = __fadd_rn(unfixed32(m0a.y), fx.y);
        mov[2] = __fadd_rn(unfixed32(m0b.x), fx.z);
        mov[3] = __fadd_rn(unfixed32(m0b.y), fx.w);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float o = fmaxf(__fsub_rn(mov[k], j.target), 0.f);
            if (EXACT) ovd += (double)o; else ov += o;
        }
        if (j.with_fill) {
            ulonglong2* fill = (ulonglong2*)(j.map + nb);
            const ulonglong2 m1a = fill[2 * q], m1b = fill[2 * q + 1];
            float r[4];
            r[0] = __fadd_rn(mov[0], unfixed32(m1a.x));
            r[1] = __fadd_rn(mov[1], unfixed32(m1a.y));
            r[2] = __fadd_rn(mov[2], unfixed32(m1b.x));
            r[3] = __fadd_rn(mov[3], unfixed32(m1b.y));
#pragma unroll
            for (int k = 0; k < 4; k++) r[k] = __fsub_rn(r[k], j.shift);
            if (j.dens) *(float4*)(j.dens + b) = make_float4(r[0], r[1], r[2], r[3]);
            if (j.tf0) {                                     // tf32 terms: the rounding and what it leaves
                float4 a, c;
                a.x = tf32_round(r[0]); a.y = tf32_round(r[1]); a.z = tf32_round(r[2]); a.w = tf32_round(r[3]);
                c.x = tf32_round(__fsub_rn(r[0], a.x)); c.y = tf32_round(__fsub_rn(r[1], a.y));
                c.z = tf32_round(__fsub_rn(r[2], a.z)); c.w = tf32_round(__fsub_rn(r[3], a.w));
                *(float4*)(j.tf0 + b) = a;
                *(float4*)(j.tf1 + b) = c;
            }
            if (j.exps) {
                // a 64-bin chunk of a row is 16 consecutive quads: half a warp (the loop keeps whole warps, since
                // quads is a multiple of 32 on the tensor-core grids); its scale from its largest magnitude
                float mx = fmaxf(fmaxf(fabsf(r[0]), fabsf(r[1])), fmaxf(fabsf(r[2]), fabsf(r[3])));
#pragma unroll
                for (int o = 8; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                const int e = f16_chunk_exp(mx);
                const float sc = __int_as_float((127 + e) << 23);
                __align__(8) __half h[2][4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const float x = r[k] * sc;
                    h[0][k] = __float2half_rn(x);
                    h[1][k] = __float2half_rn(__fsub_rn(x, __half2float(h[0][k])));
                }
                *(uint2*)(j.t0 + b) = *(const uint2*)h[0];
                *(uint2*)(j.t1 + b) = *(const uint2*)h[1];
                if ((threadIdx.x & 15) == 0) j.exps[(size_t)((b % j.nby) >> 6) * j.nbx + b / j.nby] = (signed char)e;
            } else if (j.t0) {
                __align__(8) __nv_bfloat16 t[3][4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    t[0][k] = __float2bfloat16_rn(r[k]);
                    const float rem = __fsub_rn(r[k], __bfloat162float(t[0][k]));
                    t[1][k] = __float2bfloat16_rn(rem);
                    t[2][k] = __float2bfloat16_rn(__fsub_rn(rem, __bfloat162float(t[1][k])));
                }
                *(uint2*)(j.t0 + b) = *(const uint2*)t[0];
                *(uint2*)(j.t1 + b) = *(const uint2*)t[1];
                if (j.terms > 2) *(uint2*)(j.t2 + b) = *(const uint2*)t[2];
            }
            fill[2 * q] = make_ulonglong2(0ull, 0ull);
            fill[2 * q + 1] = make_ulonglong2(0ull, 0ull);
        }
        ((ulonglong2*)j.map)[2 * q] = make_ulonglong2(0ull, 0ull);
        ((ulonglong2*)j.map)[2 * q + 1] = make_ulonglong2(0ull, 0ull);
    }
    for (int b = (nb & 3) ? bid * blockDim.x + threadIdx.x : nb; b < nb; b += nblk * blockDim.x) {
        const float mov = __fadd_rn(unfixed32(j.map[b]), j.fixed[b]);
        const float o = fmaxf(__fsub_rn(mov, j.target), 0.f);
        if (EXACT) ovd += (double)o; else ov += o;
        if (j.with_fill) {
            const float r = __fsub_rn(__fadd_rn(mov, unfixed32(j.map[nb + b])), j.shift);
            if (j.dens) j.dens[b] = r;
            if (j.t0) split_bf16(r, j.terms, j.t0, j.t1, j.t2, b);
            if (j.tf0) {
                const float a = tf32_round(r);
                j.tf0[b] = a;
                j.tf1[b] = tf32_round(__fsub_rn(r, a));
            }
            j.map[nb + b] = 0ull;
        }
        j.map[b] = 0ull;
    }
    if (EXACT) {
        double v[1] = {ovd};
        grid_sum<1>(v, j.red, nblk, bid);
    } else {
        float v[1] = {ov};
        grid_sum<1>(v, j.red, nblk, bid);
    }
}

int launch_post_plain(const PostJob* jobs, int njobs, cudaStream_t s) {
    PostPair p = {};
    p.j[0] = jobs[0];
    p.j[1] = njobs > 1 ? jobs[1] : jobs[0];
    p.njobs = njobs;
    p.blocks0 = grid_for((long long)jobs[0].nbx * jobs[0].nby / 4, 256, 8);
    const int blocks = p.blocks0 + (njobs > 1 ? grid_for((long long)jobs[1].nbx * jobs[1].nby / 4, 256, 8) : 0);
    const cudaError_t e = jobs[0].exact ? launch_k(post_plain_kernel<true>, dim3(blocks), dim3(256), 0, s, p)
                                        : launch_k(post_plain_kernel<false>, dim3(blocks), dim3(256), 0, s, p);
    if (e != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// ----------------------------------------------------------------------------- gather
// Reference semantics (density_grad_kernel): field = mirrored planes [2][2 nbx][2 nby], first quadrant read.
__global__ void gather_mirror_kernel(const float2* pos, const float2* size, const float* ratio, const float* field,
                                     const float2* wl_grad, const float* pins, const float* area, int num_nodes,
                                     int num_wl, const float* weight_p, const float* precond_p, float inv_bx,
                                     float inv_by, int nbx, int nby, float2* grad) {
    pdl_wait();
    const float weight = *weight_p, precond = *precond_p;
    const float* fy = field + (size_t)4 * nbx * nby;
    const int ld = 2 * nby;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num_nodes; i += gridDim.x * blockDim.x) {
        const float2 p = pos[i], sz = size[i];
        const Span sx = span(p.x, sz.x, inv_bx, nbx), sy = span(p.y, sz.y, inv_by, nby);
        const float r = ratio[i];
        float gx = 0.f, gy = 0.f;
        for (int x = sx.b0; x <= sx.b1; x++) {
            const float wx = __fmul_rn(r, overlap(sx, x));
            for (int y = sy.b0; y <= sy.b1; y++) {
                const float w = __fmul_rn(wx, overlap(sy, y));
                gx = fmaf(-w, field[(size_t)x * ld + y], gx);
                gy = fmaf(-w, fy[(size_t)x * ld + y], gy);
            }
        }
        gx *= weight;
        gy *= weight;
        if (i < num_wl) {
            const float2 wl = wl_grad[i];
            gx += wl.x;
            gy += wl.y;
        }
        const float scale = precond < 0.f ? 1.f : 1.f / fmaxf(pins[i] + precond * area[i], 1.f);
        grad[i] = make_float2(gx * scale, gy * scale);
    }
}

int launch_gather_mirror(const float* pos, const float* size, const float* ratio, const float* field,
                         const float* wl_grad, const float* pins, const float* area, int num_nodes, int num_wl,
                         const float* weight, const float* precond, float bx, float by, int nbx, int nby, float* grad,
                         cudaStream_t s) {
    if (num_nodes == 0) return GP103_OK;
    if (launch_k(gather_mirror_kernel, dim3(grid_for(num_nodes, 256, 8)), dim3(256), 0, s, (const float2*)pos, (const float2*)size, ratio, field, (const float2*)wl_grad, pins, area, num_nodes, num_wl,
        weight, precond, 1.f / bx, 1.f / by, nbx, nby, (float2*)grad) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// Fused gather: the field planes [nbx][nby]; the wirelength gradient of a cell summed here from its pins'
// gradients in the reference's order (cell CSR: contiguous when the pin gradients are stored in cell order, else
// through cell_pin); the new gradient, its squared distance to the previous one and its L1 norm over the cells
// reduced in float64.
// Every load a node needs is issued in two waves: its own data (position, size, ratio, pin range, pins, area,
// reference gradient), then the field values of its bins and its pins' gradients, all predicated and unrolled for
// the common shapes (spans of up to 3 bins per axis, up to GATHER_PINS pins), so that a thread waits for two
// memory latencies per node rather than one per bin and per pin.
constexpr int GATHER_PINS = 8;

__global__ void __launch_bounds__(256, 5) gather_kernel(GatherJob j) {      // 48 registers: 5 blocks per SM
    pdl_wait();
    if (j.npre > 0 && blockIdx.x == 0) {                 // the earlier kernels' totals, off the critical path
        for (int i = 0; i < j.npre; i++) {
            const double t = block_total(j.pre[i], j.pre_k[i]);
            if (threadIdx.x == 0) j.pre_out[i] = t;
        }
        return;
    }
    const int b0 = j.npre > 0 ? 1 : 0;                   // blocks b0 .. gridDim.x - 1 gather
    const int bid = (int)blockIdx.x - b0, nblk = (int)gridDim.x - b0;
    const float2* pos = pick(j.pos_a, j.pos_b, j.sel);
    float2* gout = pick_mut(j.gout_a, j.gout_b, j.sel);
    const float2* gref = j.gref_a ? pick_ref(j.gref_a, j.gref_b, j.sel) : nullptr;
    float weight = j.weight_p ? j.weight_p[0] : j.weight;
    float precond = j.precond_p ? j.precond_p[0] : j.precond;
    const bool density = j.ex != nullptr;
    float d2 = 0.f, l1 = 0.f;                  // per-thread partials (a few nodes); float32 warp trees, float64 across warps and blocks
    for (int i = bid * blockDim.x + threadIdx.x; i < j.num_nodes; i += nblk * blockDim.x) {
        // wave 1: the node's own data
        const bool cell = i < j.num_mov;
        const bool wl = j.with_wl && cell;
        float2 p = make_float2(0.f, 0.f), sz = make_float2(0.f, 0.f);
        float r = 0.f;
        if (density) {
            p = pos[i];
            sz = j.size[i];
            r = j.ratio[i];
        }
        int k0 = 0, k1 = 0;
        if (wl) {
            k0 = j.cell_start[i];
            k1 = j.cell_start[i + 1];
        }
        const float pins = j.pins[i];
        const float area = density && precond >= 0.f ? j.area[i] : 0.f;
        const float2 o = gref ? gref[i] : make_float2(0.f, 0.f);
        // wave 2: field values and pin gradients
        float gx = 0.f, gy = 0.f;
        if (density) {
            const Span sx = span(p.x, sz.x, j.inv_bx, j.nbx), sy = span(p.y, sz.y, j.inv_by, j.nby);
            const int nx = sx.b1 - sx.b0, ny = sy.b1 - sy.b0;
            if (nx >= 0 && ny >= 0 && nx <= 2 && ny <= 2) {
                float fx[3][3], fy[3][3];
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const bool in = a <= nx && c <= ny;
                        const size_t at = (size_t)(sx.b0 + a) * j.nby + (sy.b0 + c);
                        fx[a][c] = in ? j.ex[at] : 0.f;
                        fy[a][c] = in ? j.ey[at] : 0.f;
                    }
                float ox[3], oy[3];
                overlaps3(sx, ox);
                overlaps3(sy, oy);
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    if (a > nx) break;
                    const float wx = __fmul_rn(r, ox[a]);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        if (c > ny) break;
                        const float w = __fmul_rn(wx, oy[c]);
                        gx = fmaf(-w, fx[a][c], gx);
                        gy = fmaf(-w, fy[a][c], gy);
                    }
                }
            } else {
                for (int x = sx.b0; x <= sx.b1; x++) {
                    const float wx = __fmul_rn(r, overlap(sx, x));
                    const float* ex = j.ex + (size_t)x * j.nby;
                    const float* ey = j.ey + (size_t)x * j.nby;
                    for (int y = sy.b0; y <= sy.b1; y++) {
                        const float w = __fmul_rn(wx, overlap(sy, y));
                        gx = fmaf(-w, ex[y], gx);
                        gy = fmaf(-w, ey[y], gy);
                    }
                }
            }
            gx *= weight;
            gy *= weight;
        }
        float wx = 0.f, wy = 0.f;
        if (wl) {
            float2 q[GATHER_PINS];
#pragma unroll
            for (int t = 0; t < GATHER_PINS; t++)
                q[t] = k0 + t < k1 ? j.pin_grad[j.cell_pin ? j.cell_pin[k0 + t] : k0 + t] : make_float2(0.f, 0.f);
#pragma unroll
            for (int t = 0; t < GATHER_PINS; t++) {           // in cell_pin order, as the reference sums
                if (k0 + t >= k1) break;
                wx += q[t].x;
                wy += q[t].y;
            }
            for (int k = k0 + GATHER_PINS; k < k1; k++) {
                const float2 qq = j.pin_grad[j.cell_pin ? j.cell_pin[k] : k];
                wx += qq.x;
                wy += qq.y;
            }
        }
        float2 g;
        if (density) {
            gx += wx;
            gy += wy;
            const float scale = precond < 0.f ? 1.f : 1.f / fmaxf(pins + precond * area, 1.f);
            g = make_float2(gx * scale, gy * scale);
        } else if (cell) {                              // wirelength only: wl_grad / max(1, pins)
            const float pc = fmaxf(pins, 1.f);
            g = make_float2(wx / pc, wy / pc);
        } else {
            g = make_float2(0.f, 0.f);
        }
        gout[i] = g;
        if (gref) {
            const float dx = g.x - o.x, dy = g.y - o.y;
            d2 += dx * dx + dy * dy;
        }
        if (cell) l1 += fabsf(g.x) + fabsf(g.y);
    }
    float v[2] = {d2, l1};
    grid_sum<2>(v, j.red, nblk, bid);
}

int launch_gather(const GatherJob& j, cudaStream_t s) {
    static const int resident = resident_blocks(gather_kernel, 256);
    int grid = min(grid_for(j.num_nodes, 256, 8), resident);
    if (j.npre > 0) grid = max(grid, 2);                 // block 0 sums, the others gather
    if (launch_k(gather_kernel, dim3(grid), dim3(256), 0, s, j) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

}  // namespace gp103
