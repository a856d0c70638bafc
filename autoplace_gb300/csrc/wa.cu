// Weighted-average wirelength: value, pin gradient and HPWL per net, gradient per cell (GB300, sm_103a).
//
// Reference: cpp_to_py/gp_cuda_kernel.cu:8-65 (wa_net_kernel, wa_cell_kernel) and the PyTorch form
// src/core/wa_wirelength_hpwl.py:72-94. Per net and axis: hi / lo, max-shifted sums
// sp = sum e^{(x - hi)/g}, xp = sum x e^{(x - hi)/g} / sp (and sn, xn with lo), WA = xp - xn, HPWL = hi - lo,
// pin gradient ep (1 + (x - xp)/g)/sp - en (1 - (x - xn)/g)/sn.
//
// Work items: a warp takes either 32 consecutive nets, one per lane (nets of up to WA_REG pins; a longer one met
// there is done by the whole warp in turn), or, for nets from `split` on, one long net with the whole warp (lane l
// takes pins l, l + 32, ...; max / min and sums by butterfly reductions). Pins stay in registers: one pass over
// memory. The fused path orders the nets at set-up (short ones by their first cell, long ones after `split`), so
// that warps do equal work and their gathers stay local; any order gives the same numbers. The pin gradient can go
// to a slot in cell order (the gather then reads each cell's pins contiguously). Exponentials use the hardware exp2
// path (__expf), as the reference does under --use_fast_math; the per-pin divisions by the sums are multiplications
// by their reciprocals (within an ulp of the reference's form).
#include "gp103.cuh"
#include "kernels.cuh"

namespace gp103 {

constexpr int WA_REG = 8;      // pins of a thread-per-net net kept in registers
constexpr int WA_WREG = 4;     // pins per lane of a warp-per-net net kept in registers (nets up to 128 pins)

__device__ __forceinline__ float2 pin_xy(const WaJob& j, const float2* pos, int p) {
    const int c = __ldg(j.pin_cell + p);
    const float2 o = __ldg(j.pin_off + p);
    const float2 q = c < j.num_mov ? pos[c] : make_float2(0.f, 0.f);
    return make_float2(q.x + o.x, q.y + o.y);
}

// Where pin p's gradient goes (loaded together with the pin, ahead of the arithmetic that needs the positions).
__device__ __forceinline__ int slot_of(const WaJob& j, int p) { return j.slot ? __ldg(j.slot + p) : p; }
__device__ __forceinline__ void put(const WaJob& j, int q, float gx, float gy) { j.pin_grad[q] = make_float2(gx, gy); }

// Butterfly reductions over aligned groups of L lanes (the whole warp takes part; each group gets its own value).
template <int L>
__device__ __forceinline__ float gmax(float v) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <int L>
__device__ __forceinline__ float gmin(float v) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <int L>
__device__ __forceinline__ float gsum(float v) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Running state of a net: per axis hi / lo and the sums sp, sn, xp, xn.
struct Net {
    float hx, lx, hy, ly;
    float spx, snx, xpx, xnx, spy, sny, xpy, xny;
    __device__ __forceinline__ void init() {
        hx = hy = -1e30f;
        lx = ly = 1e30f;
        spx = snx = xpx = xnx = spy = sny = xpy = xny = 0.f;
    }
    __device__ __forceinline__ void extent(float2 x) {
        hx = fmaxf(hx, x.x); lx = fminf(lx, x.x);
        hy = fmaxf(hy, x.y); ly = fminf(ly, x.y);
    }
    __device__ __forceinline__ void add(float2 x, float ig) {
        const float epx = __expf((x.x - hx) * ig), enx = __expf((lx - x.x) * ig);
        const float epy = __expf((x.y - hy) * ig), eny = __expf((ly - x.y) * ig);
        spx += epx; snx += enx; xpx += x.x * epx; xnx += x.x * enx;
        spy += epy; sny += eny; xpy += x.y * epy; xny += x.y * eny;
    }
};

// After the sums: the means and reciprocals the pin gradients need.
struct Coef {
    float xpx, xnx, xpy, xny, ipx, inx, ipy, iny;
    __device__ __forceinline__ void from(const Net& n) {
        xpx = n.xpx / n.spx; xnx = n.xnx / n.snx; xpy = n.xpy / n.spy; xny = n.xny / n.sny;
        ipx = 1.f / n.spx; inx = 1.f / n.snx; ipy = 1.f / n.spy; iny = 1.f / n.sny;
    }
    __device__ __forceinline__ float2 grad(const Net& n, float2 x, float ig) const {
        const float epx = __expf((x.x - n.hx) * ig), enx = __expf((n.lx - x.x) * ig);
        const float epy = __expf((x.y - n.hy) * ig), eny = __expf((n.ly - x.y) * ig);
        return make_float2(epx * (1.f + (x.x - xpx) * ig) * ipx - enx * (1.f - (x.x - xnx) * ig) * inx,
                           epy * (1.f + (x.y - xpy) * ig) * ipy - eny * (1.f - (x.y - xny) * ig) * iny);
    }
};

// A net of d <= R pins by one thread (R = d for the exact-degree forms).
template <int R>
__device__ __forceinline__ void net_thread(const WaJob& j, const float2* pos, float ig, int s, int d, float& wa,
                                           float& hp) {
    Net n;
    n.init();
    float2 x[R];
    int q[R];
#pragma unroll
    for (int k = 0; k < R; k++)
        if (k < d) {
            q[k] = slot_of(j, s + k);
            x[k] = pin_xy(j, pos, s + k);
            n.extent(x[k]);
        }
#pragma unroll
    for (int k = 0; k < R; k++)
        if (k < d) n.add(x[k], ig);
    Coef c;
    c.from(n);
#pragma unroll
    for (int k = 0; k < R; k++)
        if (k < d) {
            const float2 g = c.grad(n, x[k], ig);
            put(j, q[k], g.x, g.y);
        }
    wa = (c.xpx - c.xnx) + (c.xpy - c.xny);
    hp = (n.hx - n.lx) + (n.hy - n.ly);
}

// A longer net by a group of L lanes (every lane of the group ends with the net's values; `gl` = lane in the group).
// Up to L * WA_WREG pins stay in registers; longer nets take three passes over their pins (re-read, cached). The
// whole warp must call it together (the reductions are warp shuffles); d = 0 for a group with no net.
template <int L>
__device__ __forceinline__ void net_group(const WaJob& j, const float2* pos, float ig, int s, int d, int gl,
                                          float& wa, float& hp) {
    Net n;
    n.init();
    Coef c;
    if (__all_sync(0xffffffffu, d <= L * WA_WREG)) {
        float2 x[WA_WREG];
        int q[WA_WREG];
#pragma unroll
        for (int t = 0; t < WA_WREG; t++)
            if (gl + L * t < d) {
                q[t] = slot_of(j, s + gl + L * t);
                x[t] = pin_xy(j, pos, s + gl + L * t);
                n.extent(x[t]);
            }
        n.hx = gmax<L>(n.hx); n.lx = gmin<L>(n.lx); n.hy = gmax<L>(n.hy); n.ly = gmin<L>(n.ly);
#pragma unroll
        for (int t = 0; t < WA_WREG; t++)
            if (gl + L * t < d) n.add(x[t], ig);
        n.spx = gsum<L>(n.spx); n.snx = gsum<L>(n.snx); n.xpx = gsum<L>(n.xpx); n.xnx = gsum<L>(n.xnx);
        n.spy = gsum<L>(n.spy); n.sny = gsum<L>(n.sny); n.xpy = gsum<L>(n.xpy); n.xny = gsum<L>(n.xny);
        c.from(n);
#pragma unroll
        for (int t = 0; t < WA_WREG; t++)
            if (gl + L * t < d) {
                const float2 g = c.grad(n, x[t], ig);
                put(j, q[t], g.x, g.y);
            }
    } else {                                             // very long nets: three passes, pins re-read (cached)
        for (int p = gl; p < d; p += L) n.extent(pin_xy(j, pos, s + p));
        n.hx = gmax<L>(n.hx); n.lx = gmin<L>(n.lx); n.hy = gmax<L>(n.hy); n.ly = gmin<L>(n.ly);
        for (int p = gl; p < d; p += L) n.add(pin_xy(j, pos, s + p), ig);
        n.spx = gsum<L>(n.spx); n.snx = gsum<L>(n.snx); n.xpx = gsum<L>(n.xpx); n.xnx = gsum<L>(n.xnx);
        n.spy = gsum<L>(n.spy); n.sny = gsum<L>(n.sny); n.xpy = gsum<L>(n.xpy); n.xny = gsum<L>(n.xny);
        c.from(n);
        for (int p = gl; p < d; p += L) {
            const float2 g = c.grad(n, pin_xy(j, pos, s + p), ig);
            put(j, slot_of(j, s + p), g.x, g.y);
        }
    }
    wa = (c.xpx - c.xnx) + (c.xpy - c.xny);
    hp = (n.hx - n.lx) + (n.hy - n.ly);
}

__device__ __forceinline__ void net_warp(const WaJob& j, const float2* pos, float ig, int s, int d, int lane,
                                         float& wa, float& hp) {
    net_group<32>(j, pos, ig, s, d, lane, wa, hp);
}

// A 2-pin net by one thread. Per axis the two pins share one exponential: with hi / lo the larger / smaller
// coordinate, e = exp((lo - hi) / g) is ep of the low pin and en of the high pin, while ep of the high pin and en
// of the low pin are exp(0) = 1 (both 1 when the pins coincide) -- the values the general form computes, with one
// exponential instead of four per axis.
__device__ __forceinline__ void net_two(const WaJob& j, const float2* pos, float ig, int s, float& wa, float& hp) {
    const int qa = slot_of(j, s), qb = slot_of(j, s + 1);
    const float2 a = pin_xy(j, pos, s), b = pin_xy(j, pos, s + 1);
    float g[2][2], wsum = 0.f, hsum = 0.f;
#pragma unroll
    for (int ax = 0; ax < 2; ax++) {
        const float xa = ax ? a.y : a.x, xb = ax ? b.y : b.x;
        const float hi = fmaxf(xa, xb), lo = fminf(xa, xb);
        const float e = __expf((lo - hi) * ig);
        const float epa = xa == hi ? 1.f : e, epb = xb == hi ? 1.f : e;
        const float ena = xa == lo ? 1.f : e, enb = xb == lo ? 1.f : e;
        const float sp = epa + epb, sn = ena + enb;
        const float ip = __frcp_rn(sp), in = __frcp_rn(sn);
        const float xp = (xa * epa + xb * epb) * ip, xn = (xa * ena + xb * enb) * in;
        g[0][ax] = epa * (1.f + (xa - xp) * ig) * ip - ena * (1.f - (xa - xn) * ig) * in;
        g[1][ax] = epb * (1.f + (xb - xp) * ig) * ip - enb * (1.f - (xb - xn) * ig) * in;
        wsum += xp - xn;
        hsum += hi - lo;
    }
    put(j, qa, g[0][0], g[0][1]);
    put(j, qb, g[1][0], g[1][1]);
    wa = wsum;
    hp = hsum;
}

// A 2-pin net whose pins are s, s + 1 with s even (the 2-pin class of the ordered layout): cells, offsets and slots of
// both pins in one 8-, one 16- and one 8-byte load, all issued before the position gathers.
__device__ __forceinline__ void net_two_pair(const WaJob& j, const float2* pos, float ig, int s, float& wa,
                                             float& hp) {
    const int2 c = __ldg((const int2*)(j.pin_cell + s));
    const float4 o = __ldg((const float4*)(j.pin_off + s));
    const int2 q = j.slot ? __ldg((const int2*)(j.slot + s)) : make_int2(s, s + 1);
    const float2 pa = c.x < j.num_mov ? pos[c.x] : make_float2(0.f, 0.f);
    const float2 pb = c.y < j.num_mov ? pos[c.y] : make_float2(0.f, 0.f);
    const float2 a = make_float2(pa.x + o.x, pa.y + o.y), b = make_float2(pb.x + o.z, pb.y + o.w);
    float g[2][2], wsum = 0.f, hsum = 0.f;
#pragma unroll
    for (int ax = 0; ax < 2; ax++) {
        const float xa = ax ? a.y : a.x, xb = ax ? b.y : b.x;
        const float hi = fmaxf(xa, xb), lo = fminf(xa, xb);
        const float e = __expf((lo - hi) * ig);
        const float epa = xa == hi ? 1.f : e, epb = xb == hi ? 1.f : e;
        const float ena = xa == lo ? 1.f : e, enb = xb == lo ? 1.f : e;
        const float sp = epa + epb, sn = ena + enb;
        const float ip = __frcp_rn(sp), in = __frcp_rn(sn);
        const float xp = (xa * epa + xb * epb) * ip, xn = (xa * ena + xb * enb) * in;
        g[0][ax] = epa * (1.f + (xa - xp) * ig) * ip - ena * (1.f - (xa - xn) * ig) * in;
        g[1][ax] = epb * (1.f + (xb - xp) * ig) * ip - enb * (1.f - (xb - xn) * ig) * in;
        wsum += xp - xn;
        hsum += hi - lo;
    }
    put(j, q.x, g[0][0], g[0][1]);
    put(j, q.y, g[1][0], g[1][1]);
    wa = wsum;
    hp = hsum;
}

// Short nets, one per lane: 32 consecutive nets [0, split) per warp item. With the class layout (three > 0) the
// nets below `three` need no net_start: net i < two starts at pin 2 i, net i < three at 2 two + 3 (i - two). LONG: nets longer than WA_REG met there
// (any order) are done by the whole warp in turn; without it every net below split is short (the ordered layout).
// Blocks write float64 partials at bid0 + blockIdx.x of nblk.
template <bool LONG>
__device__ __forceinline__ void wa_short_body(const WaJob& j, int blk, int nb, float& wa_sum, float& hp_sum) {
    const float2* pos = pick(j.pos_a, j.pos_b, j.sel);
    const float ig = __frcp_rn(*j.gamma);
    const int lane = threadIdx.x & 31;
    const long long nwarps = (long long)nb * (blockDim.x >> 5);
    const long long chunks = (j.split + 31) / 32;
    for (long long it = (long long)blk * (blockDim.x >> 5) + (threadIdx.x >> 5); it < chunks; it += nwarps) {
        const int i = (int)(it * 32) + lane;
        const bool valid = i < j.split;
        int s = 0, d = 0;
        if (valid) {
            if (i < j.two) {
                s = 2 * i;
                d = 2;
            } else if (i < j.three) {
                s = 2 * j.two + 3 * (i - j.two);
                d = 3;
            } else {
                s = j.net_start[i];
                d = j.net_start[i + 1] - s;
            }
        }
        if (valid && d <= WA_REG) {
            float wa, hp;
            if (i < j.two) net_two_pair(j, pos, ig, s, wa, hp);
            else if (d == 2) net_two(j, pos, ig, s, wa, hp);
            else if (d == 3) net_thread<3>(j, pos, ig, s, d, wa, hp);
            else net_thread<WA_REG>(j, pos, ig, s, d, wa, hp);
            if (j.out) j.out[i] = make_float2(wa, hp);
            wa_sum += wa;
            hp_sum += hp;
        }
        if (LONG) {
            unsigned big = __ballot_sync(0xffffffffu, valid && d > WA_REG);
            while (big) {
                const int src = __ffs(big) - 1;
                big &= big - 1;
                const int bs = __shfl_sync(0xffffffffu, s, src), bd = __shfl_sync(0xffffffffu, d, src);
                float wa, hp;
                net_warp(j, pos, ig, bs, bd, lane, wa, hp);
                if (lane == src) {
                    if (j.out) j.out[i] = make_float2(wa, hp);
                    wa_sum += wa;
                    hp_sum += hp;
                }
            }
        }
    }
}

template <bool LONG>
__global__ void __launch_bounds__(256) wa_short_kernel(const __grid_constant__ WaJob j, int bid0, int nblk) {
    pdl_wait();
    float wa_sum = 0.f, hp_sum = 0.f;          // per-thread partials (a few nets); float32 warp trees, float64 across warps and blocks
    wa_short_body<LONG>(j, blockIdx.x, gridDim.x, wa_sum, hp_sum);
    if (j.red.partials) {
        float v[2] = {wa_sum, hp_sum};
        grid_sum<2>(v, j.red, nblk, bid0 + (int)blockIdx.x);
    }
}

// Long nets [split, num_nets), by degree class: [split, mid) (9 .. 16 pins) by groups of 4 lanes, eight nets per
// warp item; [mid, g8) (17 .. 32) by 8 lanes, four per item; [g8, g16) (33 .. 64) by 16 lanes, two per item; the
// rest one per warp. Every lane of a group holds at most WA_WREG pins.
template <int L>
__device__ __forceinline__ void group_item(const WaJob& j, const float2* pos, float ig, int first, int end, int item,
                                           int lane, float& wa_sum, float& hp_sum) {
    const int gl = lane & (L - 1), i = first + item * (32 / L) + lane / L;
    const bool valid = i < end;
    int s = 0, d = 0;
    if (valid) {
        s = j.net_start[i];
        d = j.net_start[i + 1] - s;
    }
    float wa, hp;
    net_group<L>(j, pos, ig, s, d, gl, wa, hp);
    if (valid && gl == 0) {
        if (j.out) j.out[i] = make_float2(wa, hp);
        wa_sum += wa;
        hp_sum += hp;
    }
}

__host__ __device__ inline int group_items(int first, int end, int lanes) {
    return (end - first + 32 / lanes - 1) / (32 / lanes);
}

__device__ __forceinline__ void wa_long_body(const WaJob& j, int blk, int nb, float& wa_sum, float& hp_sum) {
    const float2* pos = pick(j.pos_a, j.pos_b, j.sel);
    const float ig = __frcp_rn(*j.gamma);
    const int lane = threadIdx.x & 31;
    const int nwarps = nb * (blockDim.x >> 5);
    const int n4 = group_items(j.split, j.mid, 4), n8 = group_items(j.mid, j.g8, 8);
    const int n16 = group_items(j.g8, j.g16, 16);
    const int groups = n4 + n8 + n16;
    const int items = groups + (j.num_nets - j.g16);
    for (int it = blk * (blockDim.x >> 5) + (threadIdx.x >> 5); it < items; it += nwarps) {
        if (it < n4) {                                       // (every branch is uniform over the warp)
            group_item<4>(j, pos, ig, j.split, j.mid, it, lane, wa_sum, hp_sum);
        } else if (it < n4 + n8) {
            group_item<8>(j, pos, ig, j.mid, j.g8, it - n4, lane, wa_sum, hp_sum);
        } else if (it < groups) {
            group_item<16>(j, pos, ig, j.g8, j.g16, it - n4 - n8, lane, wa_sum, hp_sum);
        } else {
            const int i = j.g16 + (it - groups);
            const int s = j.net_start[i], d = j.net_start[i + 1] - s;
            float wa, hp;
            net_warp(j, pos, ig, s, d, lane, wa, hp);
            if (lane == 0) {
                if (j.out) j.out[i] = make_float2(wa, hp);
                wa_sum += wa;
                hp_sum += hp;
            }
        }
    }
}

__global__ void __launch_bounds__(256) wa_long_kernel(const __grid_constant__ WaJob j, int bid0, int nblk) {
    pdl_wait();
    float wa_sum = 0.f, hp_sum = 0.f;
    wa_long_body(j, blockIdx.x, gridDim.x, wa_sum, hp_sum);
    if (j.red.partials) {
        float v[2] = {wa_sum, hp_sum};
        grid_sum<2>(v, j.red, nblk, bid0 + (int)blockIdx.x);
    }
}

// Both halves in one launch (the ordered layout): blocks [0, nlong) take the long nets, the rest the short ones, so
// the two run side by side in one resident wave instead of one after the other (each with its own tail). Partials:
// block b writes slot b of nblk = gridDim.x.
__global__ void __launch_bounds__(256) wa_fused_kernel(const __grid_constant__ WaJob j, int nlong) {
    pdl_wait();
    float wa_sum = 0.f, hp_sum = 0.f;
    if ((int)blockIdx.x < nlong) wa_long_body(j, blockIdx.x, nlong, wa_sum, hp_sum);
    else wa_short_body<false>(j, blockIdx.x - nlong, gridDim.x - nlong, wa_sum, hp_sum);
    if (j.red.partials) {
        float v[2] = {wa_sum, hp_sum};
        grid_sum<2>(v, j.red, gridDim.x, (int)blockIdx.x);
    }
}

int launch_wa_net(const WaJob& j, cudaStream_t s) {
    const long long chunks = (j.split + 31) / 32;
    const long long longs = (long long)group_items(j.split, j.mid, 4) + group_items(j.mid, j.g8, 8) +
                            group_items(j.g8, j.g16, 16) + (j.num_nets - j.g16);          // warp items
    const bool inline_long = j.split == j.num_nets;     // any order: long nets where they are met
    static const int res_short = resident_blocks(wa_short_kernel<false>, 256);
    static const int res_long = resident_blocks(wa_long_kernel, 256);
    // the plan's share where it gives one, while the process option has the launch fused (0 there: two launches)
    const int pct = wa_long_share() > 0 && j.long_share > 0 ? j.long_share : wa_long_share();
    if (pct > 0 && !inline_long && chunks > 0 && longs > 0) {
        // one resident wave: pct % of its blocks on the long nets, the rest on the short ones
        static const int res = resident_blocks(wa_fused_kernel, 256);
        const int nlong = max(1, min((res * pct + 50) / 100, res - 1));
        if (launch_k(wa_fused_kernel, dim3(res), dim3(256), 0, s, j, nlong) != cudaSuccess) return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
        return GP103_OK;
    }
    const int g1 = chunks > 0 || longs == 0 ? min(grid_for(chunks * 32, 256, 8), res_short) : 0;
    const int g2 = longs > 0 ? min(grid_for(longs * 32, 256, 4), res_long) : 0;
    if (g1 > 0) {
        cudaError_t e = inline_long ? launch_k(wa_short_kernel<true>, dim3(g1), dim3(256), 0, s, j, 0, g1 + g2)
                                    : launch_k(wa_short_kernel<false>, dim3(g1), dim3(256), 0, s, j, 0, g1 + g2);
        if (e != cudaSuccess) return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    if (g2 > 0) {
        if (launch_k(wa_long_kernel, dim3(g2), dim3(256), 0, s, j, g1, g1 + g2) != cudaSuccess) return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    return GP103_OK;
}

// One thread per cell: its pins' gradients in cell_pin order (the reference's fixed order).
__global__ void wa_cell_kernel(const float2* pin_grad, const int* cell_start, const int* cell_pin, int num_mov,
                               float2* grad) {
    pdl_wait();
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < num_mov; c += gridDim.x * blockDim.x) {
        float gx = 0.f, gy = 0.f;
        for (int k = cell_start[c]; k < cell_start[c + 1]; k++) {
            const float2 q = pin_grad[cell_pin[k]];
            gx += q.x;
            gy += q.y;
        }
        grad[c] = make_float2(gx, gy);
    }
}

int launch_wa_cell(const float2* pin_grad, const int* cell_start, const int* cell_pin, int num_mov, float2* grad,
                   cudaStream_t s) {
    if (num_mov == 0) return GP103_OK;
    if (launch_k(wa_cell_kernel, dim3(grid_for(num_mov, 256, 8)), dim3(256), 0, s, pin_grad, cell_start, cell_pin, num_mov, grad) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

}  // namespace gp103
