// Density: fixed-point charge scatter, map post-processing and the field gather (GB300, sm_103a).
//
// Reference: cpp_to_py/gp_cuda_kernel.cu:67-153 (density_map_kernel, density_post_kernel, density_grad_kernel) and
// src/core/electronic_density_layer.py:96-149. The charge of a (node, bin) pair is the reference's float32 product
// truncated to 2^-32 bin areas and summed as 64-bit integers: the map is the same integers in any summation order.
// This file is built with -ftz=true, as the reference's kernels are (--use_fast_math), so that even denormal
// intermediates round the same way.
#include <cuda_bf16.h>

#include "gp103.cuh"
#include "kernels.cuh"

namespace gp103 {

// ----------------------------------------------------------------------------- scatter
// A block takes a chunk of SCAT_CHUNK consecutive nodes, all movable or all fillers. If the bins its nodes touch fit
// in shared memory (bounding box <= SCAT_SMEM_BINS), the block sums its charges there and then adds every non-zero
// bin to the global map once; otherwise it adds each charge to the global map directly (64-bit atomics in L2).
// In shared memory a 64-bit sum is kept as two 32-bit words: a charge (at most 2^32) adds its low word to `lo` with
// a 32-bit atomic whose old value tells whether the word wrapped; the wrap and the charge's high bit go to `hi`.
// Exact (integer) in any order, with a single 32-bit atomic for most charges.
constexpr int SCAT_THREADS = 256;
constexpr int SCAT_PER_THREAD = 4;
constexpr int SCAT_CHUNK = SCAT_THREADS * SCAT_PER_THREAD;
constexpr int SCAT_SMEM_BINS = 6144;      // 2 x 24 KB of 32-bit words

__device__ __forceinline__ void add_shared(unsigned int* lo, unsigned int* hi, int b, unsigned long long q) {
    const unsigned int ql = (unsigned int)q;
    unsigned int qh = (unsigned int)(q >> 32);
    const unsigned int old = atomicAdd(lo + b, ql);
    if (old + ql < old) qh += 1u;
    if (qh) atomicAdd(hi + b, qh);
}

__global__ void __launch_bounds__(SCAT_THREADS) scatter_kernel(const __grid_constant__ ScatterPair pair) {
    pdl_wait();
    __shared__ unsigned int tlo[SCAT_SMEM_BINS], thi[SCAT_SMEM_BINS];
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
            const int i = j.order ? j.order[at] : at;
            float2 p = pos[i], s = j.size[i];
            sx[k] = span(p.x, s.x, j.inv_bx, j.nbx);
            sy[k] = span(p.y, s.y, j.inv_by, j.nby);
            ratio[k] = j.ratio[i];
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
    if (w * h <= SCAT_SMEM_BINS) {
        const int H = (int)h, area = (int)(w * h);
        for (int t = threadIdx.x; t < area; t += SCAT_THREADS) { tlo[t] = 0u; thi[t] = 0u; }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SCAT_PER_THREAD; k++) {
            for (int x = sx[k].b0; x <= sx[k].b1; x++) {
                const float wx = __fmul_rn(ratio[k], overlap(sx[k], x));
                const int row = (x - bx0) * H - by0;
                for (int y = sy[k].b0; y <= sy[k].b1; y++) {
                    const unsigned long long q = charge(wx, overlap(sy[k], y));
                    if (q) add_shared(tlo, thi, row + y, q);
                }
            }
        }
        __syncthreads();
        for (int t = threadIdx.x; t < area; t += SCAT_THREADS) {
            const unsigned long long q = ((unsigned long long)thi[t] << 32) | tlo[t];
            if (q) atomicAdd(&map[(size_t)(bx0 + t / H) * j.nby + (by0 + t % H)], q);
        }
    } else {
#pragma unroll
        for (int k = 0; k < SCAT_PER_THREAD; k++) {
            for (int x = sx[k].b0; x <= sx[k].b1; x++) {
                const float wx = __fmul_rn(ratio[k], overlap(sx[k], x));
                for (int y = sy[k].b0; y <= sy[k].b1; y++) {
                    const unsigned long long q = charge(wx, overlap(sy[k], y));
                    if (q) atomicAdd(&map[(size_t)x * j.nby + y], q);
                }
            }
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

__global__ void post_plain_kernel(const __grid_constant__ PostPair pair) {
    pdl_wait();
    const bool second = (int)blockIdx.x >= pair.blocks0;
    const PostJob& j = second ? pair.j[1] : pair.j[0];
    const int bid = second ? (int)blockIdx.x - pair.blocks0 : (int)blockIdx.x;
    const int nblk = second ? (int)gridDim.x - pair.blocks0 : pair.blocks0;
    const int nb = j.nbx * j.nby;
    float ov = 0.f;
    // four bins per thread and iteration: 32-byte map loads / stores, 8-byte stores of each bf16 term plane (a bin
    // count that is a multiple of 4 keeps every plane aligned; any other takes the scalar loop below for every bin)
    const int quads = (nb & 3) ? 0 : nb >> 2;
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
        for (int k = 0; k < 4; k++) ov += fmaxf(__fsub_rn(mov[k], j.target), 0.f);
        if (j.with_fill) {
            ulonglong2* fill = (ulonglong2*)(j.map + nb);
            const ulonglong2 m1a = fill[2 * q], m1b = fill[2 * q + 1];
            float r[4];
            r[0] = __fadd_rn(mov[0], unfixed32(m1a.x));
            r[1] = __fadd_rn(mov[1], unfixed32(m1a.y));
            r[2] = __fadd_rn(mov[2], unfixed32(m1b.x));
            r[3] = __fadd_rn(mov[3], unfixed32(m1b.y));
            if (j.dens) *(float4*)(j.dens + b) = make_float4(r[0], r[1], r[2], r[3]);
            if (j.t0) {
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
        ov += fmaxf(__fsub_rn(mov, j.target), 0.f);
        if (j.with_fill) {
            const float r = __fadd_rn(mov, unfixed32(j.map[nb + b]));
            if (j.dens) j.dens[b] = r;
            if (j.t0) split_bf16(r, j.terms, j.t0, j.t1, j.t2, b);
            j.map[nb + b] = 0ull;
        }
        j.map[b] = 0ull;
    }
    double v[1] = {ov};
    grid_sum<1>(v, j.red, nblk, bid);
}

int launch_post_plain(const PostJob* jobs, int njobs, cudaStream_t s) {
    PostPair p = {};
    p.j[0] = jobs[0];
    p.j[1] = njobs > 1 ? jobs[1] : jobs[0];
    p.njobs = njobs;
    p.blocks0 = grid_for((long long)jobs[0].nbx * jobs[0].nby / 4, 256, 8);
    const int blocks = p.blocks0 + (njobs > 1 ? grid_for((long long)jobs[1].nbx * jobs[1].nby / 4, 256, 8) : 0);
    if (launch_k(post_plain_kernel, dim3(blocks), dim3(256), 0, s, p) != cudaSuccess) return GP103_ERR_CUDA;
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
__global__ void __launch_bounds__(256) gather_kernel(GatherJob j) {
    pdl_wait();
    const float2* pos = pick(j.pos_a, j.pos_b, j.sel);
    float2* gout = pick_mut(j.gout_a, j.gout_b, j.sel);
    const float2* gref = j.gref_a ? pick_ref(j.gref_a, j.gref_b, j.sel) : nullptr;
    float weight = j.weight_p ? j.weight_p[0] : j.weight;
    float precond = j.precond_p ? j.precond_p[0] : j.precond;
    const bool density = j.ex != nullptr;
    float d2 = 0.f, l1 = 0.f;                  // per-thread partials (a few nodes); float64 above
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < j.num_nodes; i += gridDim.x * blockDim.x) {
        float gx = 0.f, gy = 0.f;
        if (density) {
            const float2 p = pos[i], sz = j.size[i];
            const Span sx = span(p.x, sz.x, j.inv_bx, j.nbx), sy = span(p.y, sz.y, j.inv_by, j.nby);
            const float r = j.ratio[i];
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
            gx *= weight;
            gy *= weight;
        }
        float wx = 0.f, wy = 0.f;
        if (j.with_wl && i < j.num_mov) {
            const int k0 = j.cell_start[i], k1 = j.cell_start[i + 1];
            for (int k = k0; k < k1; k++) {
                const float2 q = j.pin_grad[j.cell_pin ? j.cell_pin[k] : k];
                wx += q.x;
                wy += q.y;
            }
        }
        float2 g;
        if (density) {
            gx += wx;
            gy += wy;
            const float scale = precond < 0.f ? 1.f : 1.f / fmaxf(j.pins[i] + precond * j.area[i], 1.f);
            g = make_float2(gx * scale, gy * scale);
        } else if (i < j.num_mov) {                     // wirelength only: wl_grad / max(1, pins)
            const float pc = fmaxf(j.pins[i], 1.f);
            g = make_float2(wx / pc, wy / pc);
        } else {
            g = make_float2(0.f, 0.f);
        }
        gout[i] = g;
        if (gref) {
            const float2 o = gref[i];
            const float dx = g.x - o.x, dy = g.y - o.y;
            d2 += dx * dx + dy * dy;
        }
        if (i < j.num_mov) l1 += fabsf(g.x) + fabsf(g.y);
    }
    double v[2] = {d2, l1};
    grid_sum<2>(v, j.red);
}

int launch_gather(const GatherJob& j, cudaStream_t s) {
    if (launch_k(gather_kernel, dim3(grid_for(j.num_nodes, 256, 8)), dim3(256), 0, s, j) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

}  // namespace gp103
