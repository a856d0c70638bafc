// Weighted-average wirelength: value, pin gradient and HPWL per net, gradient per cell (GB300, sm_103a).
//
// Reference: cpp_to_py/gp_cuda_kernel.cu:8-65 (wa_net_kernel, wa_cell_kernel) and the PyTorch form
// src/core/wa_wirelength_hpwl.py:72-94. Per net and axis: hi / lo, max-shifted sums
// sp = sum e^{(x - hi)/g}, xp = sum x e^{(x - hi)/g} / sp (and sn, xn with lo), WA = xp - xn, HPWL = hi - lo,
// pin gradient ep (1 + (x - xp)/g)/sp - en (1 - (x - xn)/g)/sn.
//
// A thread per net up to WA_REG pins, a warp per longer net, pins held in registers (one pass over memory). With
// nets ordered by degree (what the fused path does at set-up) a warp's nets have equal degree and its loads are
// contiguous. Exponentials use the hardware exp2 path (__expf), as the reference does under --use_fast_math.
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

__device__ __forceinline__ float wmax(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float wmin(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float wsum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-axis sums of a net: sp, sn, xp (sum x ep), xn (sum x en).
struct Sums {
    float spx, snx, xpx, xnx, spy, sny, xpy, xny;
};

// A net of d <= WA_REG pins by one thread, pins in registers.
__device__ __forceinline__ void net_thread(const WaJob& j, const float2* pos, float ig, int s, int d, float& wa,
                                           float& hp) {
    float hx = -1e30f, lx = 1e30f, hy = -1e30f, ly = 1e30f;
    float2 x[WA_REG];
#pragma unroll
    for (int k = 0; k < WA_REG; k++)
        if (k < d) {
            x[k] = pin_xy(j, pos, s + k);
            hx = fmaxf(hx, x[k].x); lx = fminf(lx, x[k].x);
            hy = fmaxf(hy, x[k].y); ly = fminf(ly, x[k].y);
        }
    float epx[WA_REG], enx[WA_REG], epy[WA_REG], eny[WA_REG];
    Sums m = {};
#pragma unroll
    for (int k = 0; k < WA_REG; k++)
        if (k < d) {
            epx[k] = __expf((x[k].x - hx) * ig); enx[k] = __expf((lx - x[k].x) * ig);
            epy[k] = __expf((x[k].y - hy) * ig); eny[k] = __expf((ly - x[k].y) * ig);
            m.spx += epx[k]; m.snx += enx[k]; m.xpx += x[k].x * epx[k]; m.xnx += x[k].x * enx[k];
            m.spy += epy[k]; m.sny += eny[k]; m.xpy += x[k].y * epy[k]; m.xny += x[k].y * eny[k];
        }
    const float xpx = m.xpx / m.spx, xnx = m.xnx / m.snx, xpy = m.xpy / m.spy, xny = m.xny / m.sny;
#pragma unroll
    for (int k = 0; k < WA_REG; k++)
        if (k < d) {
            float gx = epx[k] * (1.f + (x[k].x - xpx) * ig) / m.spx - enx[k] * (1.f - (x[k].x - xnx) * ig) / m.snx;
            float gy = epy[k] * (1.f + (x[k].y - xpy) * ig) / m.spy - eny[k] * (1.f - (x[k].y - xny) * ig) / m.sny;
            j.pin_grad[s + k] = make_float2(gx, gy);
        }
    wa = (xpx - xnx) + (xpy - xny);
    hp = (hx - lx) + (hy - ly);
}

// A longer net by the whole warp: lane l takes pins l, l + 32, ...; max / min and sums by butterfly reductions
// (every lane ends with the net's values).
__device__ __forceinline__ void net_warp(const WaJob& j, const float2* pos, float ig, int s, int d, int lane,
                                         float& wa, float& hp) {
    float hx = -1e30f, lx = 1e30f, hy = -1e30f, ly = 1e30f;
    Sums m = {};
    if (d <= 32 * WA_WREG) {
        float2 x[WA_WREG];
#pragma unroll
        for (int t = 0; t < WA_WREG; t++) {
            const int p = lane + 32 * t;
            if (p < d) {
                x[t] = pin_xy(j, pos, s + p);
                hx = fmaxf(hx, x[t].x); lx = fminf(lx, x[t].x);
                hy = fmaxf(hy, x[t].y); ly = fminf(ly, x[t].y);
            }
        }
        hx = wmax(hx); lx = wmin(lx); hy = wmax(hy); ly = wmin(ly);
        float epx[WA_WREG], enx[WA_WREG], epy[WA_WREG], eny[WA_WREG];
#pragma unroll
        for (int t = 0; t < WA_WREG; t++)
            if (lane + 32 * t < d) {
                epx[t] = __expf((x[t].x - hx) * ig); enx[t] = __expf((lx - x[t].x) * ig);
                epy[t] = __expf((x[t].y - hy) * ig); eny[t] = __expf((ly - x[t].y) * ig);
                m.spx += epx[t]; m.snx += enx[t]; m.xpx += x[t].x * epx[t]; m.xnx += x[t].x * enx[t];
                m.spy += epy[t]; m.sny += eny[t]; m.xpy += x[t].y * epy[t]; m.xny += x[t].y * eny[t];
            }
        m.spx = wsum(m.spx); m.snx = wsum(m.snx); m.xpx = wsum(m.xpx); m.xnx = wsum(m.xnx);
        m.spy = wsum(m.spy); m.sny = wsum(m.sny); m.xpy = wsum(m.xpy); m.xny = wsum(m.xny);
        const float xpx = m.xpx / m.spx, xnx = m.xnx / m.snx, xpy = m.xpy / m.spy, xny = m.xny / m.sny;
#pragma unroll
        for (int t = 0; t < WA_WREG; t++)
            if (lane + 32 * t < d) {
                float gx = epx[t] * (1.f + (x[t].x - xpx) * ig) / m.spx - enx[t] * (1.f - (x[t].x - xnx) * ig) / m.snx;
                float gy = epy[t] * (1.f + (x[t].y - xpy) * ig) / m.spy - eny[t] * (1.f - (x[t].y - xny) * ig) / m.sny;
                j.pin_grad[s + lane + 32 * t] = make_float2(gx, gy);
            }
        wa = (xpx - xnx) + (xpy - xny);
        hp = (hx - lx) + (hy - ly);
        return;
    }
    for (int p = lane; p < d; p += 32) {                 // very long nets: three passes, pins re-read (cached)
        const float2 x = pin_xy(j, pos, s + p);
        hx = fmaxf(hx, x.x); lx = fminf(lx, x.x);
        hy = fmaxf(hy, x.y); ly = fminf(ly, x.y);
    }
    hx = wmax(hx); lx = wmin(lx); hy = wmax(hy); ly = wmin(ly);
    for (int p = lane; p < d; p += 32) {
        const float2 x = pin_xy(j, pos, s + p);
        const float epx = __expf((x.x - hx) * ig), enx = __expf((lx - x.x) * ig);
        const float epy = __expf((x.y - hy) * ig), eny = __expf((ly - x.y) * ig);
        m.spx += epx; m.snx += enx; m.xpx += x.x * epx; m.xnx += x.x * enx;
        m.spy += epy; m.sny += eny; m.xpy += x.y * epy; m.xny += x.y * eny;
    }
    m.spx = wsum(m.spx); m.snx = wsum(m.snx); m.xpx = wsum(m.xpx); m.xnx = wsum(m.xnx);
    m.spy = wsum(m.spy); m.sny = wsum(m.sny); m.xpy = wsum(m.xpy); m.xny = wsum(m.xny);
    const float xpx = m.xpx / m.spx, xnx = m.xnx / m.snx, xpy = m.xpy / m.spy, xny = m.xny / m.sny;
    for (int p = lane; p < d; p += 32) {
        const float2 x = pin_xy(j, pos, s + p);
        const float epx = __expf((x.x - hx) * ig), enx = __expf((lx - x.x) * ig);
        const float epy = __expf((x.y - hy) * ig), eny = __expf((ly - x.y) * ig);
        float gx = epx * (1.f + (x.x - xpx) * ig) / m.spx - enx * (1.f - (x.x - xnx) * ig) / m.snx;
        float gy = epy * (1.f + (x.y - xpy) * ig) / m.spy - eny * (1.f - (x.y - xny) * ig) / m.sny;
        j.pin_grad[s + p] = make_float2(gx, gy);
    }
    wa = (xpx - xnx) + (xpy - xny);
    hp = (hx - lx) + (hy - ly);
}

// A warp takes 32 consecutive nets: nets of up to WA_REG pins one per lane, then every longer one by the whole
// warp. Works for nets in any order; with nets sorted by degree (the fused path) the lanes of a warp do equal work.
__global__ void __launch_bounds__(256) wa_net_kernel(WaJob j) {
    const float2* pos = pick(j.pos_a, j.pos_b, j.sel);
    const float ig = __frcp_rn(*j.gamma);
    const int lane = threadIdx.x & 31;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    double wa_sum = 0.0, hp_sum = 0.0;
    for (long long c = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c * 32 < j.num_nets;
         c += nwarps) {
        const int i = (int)(c * 32) + lane;
        int s = 0, d = 0;
        if (i < j.num_nets) {
            s = j.net_start[i];
            d = j.net_start[i + 1] - s;
        }
        if (i < j.num_nets && d <= WA_REG) {
            float wa, hp;
            net_thread(j, pos, ig, s, d, wa, hp);
            if (j.out) j.out[i] = make_float2(wa, hp);
            wa_sum += (double)wa;
            hp_sum += (double)hp;
        }
        unsigned big = __ballot_sync(0xffffffffu, i < j.num_nets && d > WA_REG);
        while (big) {
            const int src = __ffs(big) - 1;
            big &= big - 1;
            const int bs = __shfl_sync(0xffffffffu, s, src), bd = __shfl_sync(0xffffffffu, d, src);
            float wa, hp;
            net_warp(j, pos, ig, bs, bd, lane, wa, hp);
            if (lane == src) {
                if (j.out) j.out[i] = make_float2(wa, hp);
                wa_sum += (double)wa;
                hp_sum += (double)hp;
            }
        }
    }
    if (j.red.out) {
        double v[2] = {wa_sum, hp_sum};
        grid_sum<2>(v, j.red);
    }
}

int launch_wa_net(const WaJob& j, cudaStream_t s) {
    wa_net_kernel<<<grid_for(j.num_nets, 256, 8), 256, 0, s>>>(j);
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// One thread per cell: its pins' gradients in cell_pin order (the reference's fixed order).
__global__ void wa_cell_kernel(const float2* pin_grad, const int* cell_start, const int* cell_pin, int num_mov,
                               float2* grad) {
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
    wa_cell_kernel<<<grid_for(num_mov, 256, 8), 256, 0, s>>>(pin_grad, cell_start, cell_pin, num_mov, grad);
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

}  // namespace gp103
