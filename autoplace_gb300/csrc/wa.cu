// Weighted-average wirelength: value, pin gradient and HPWL per net, gradient per cell (GB300, sm_103a).
//
// Reference: cpp_to_py/gp_cuda_kernel.cu:8-65 (wa_net_kernel, wa_cell_kernel) and the PyTorch form
// src/core/wa_wirelength_hpwl.py:72-94. Per net and axis: hi / lo, max-shifted sums
// sp = sum e^{(x - hi)/g}, xp = sum x e^{(x - hi)/g} / sp (and sn, xn with lo), WA = xp - xn, HPWL = hi - lo,
// pin gradient ep (1 + (x - xp)/g)/sp - en (1 - (x - xn)/g)/sn.
//
// One thread per net. Nets of up to WA_REG pins keep their pins in registers (one pass over memory); longer nets
// re-read their pins (cached) in three passes instead of storing coordinates in the gradient buffer. With nets
// ordered by degree (what the fused path does at set-up) a warp's nets have equal degree and its loads are
// contiguous. Exponentials use the hardware exp2 path (__expf), as the reference does under --use_fast_math.
#include "gp103.cuh"
#include "kernels.cuh"

namespace gp103 {

constexpr int WA_REG = 8;

__device__ __forceinline__ float2 pin_xy(const WaJob& j, const float2* pos, int p) {
    const int c = __ldg(j.pin_cell + p);
    const float2 o = __ldg(j.pin_off + p);
    const float2 q = c < j.num_mov ? pos[c] : make_float2(0.f, 0.f);
    return make_float2(q.x + o.x, q.y + o.y);
}

__global__ void __launch_bounds__(256) wa_net_kernel(WaJob j) {
    const float2* pos = pick(j.pos_a, j.pos_b, j.sel);
    const float ig = __frcp_rn(*j.gamma);
    double wa_sum = 0.0, hp_sum = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < j.num_nets; i += gridDim.x * blockDim.x) {
        const int s = j.net_start[i], d = j.net_start[i + 1] - s;
        float hx = -1e30f, lx = 1e30f, hy = -1e30f, ly = 1e30f;
        float spx = 0.f, snx = 0.f, xpx = 0.f, xnx = 0.f, spy = 0.f, sny = 0.f, xpy = 0.f, xny = 0.f;
        if (d <= WA_REG) {
            float2 x[WA_REG];
#pragma unroll
            for (int k = 0; k < WA_REG; k++)
                if (k < d) {
                    x[k] = pin_xy(j, pos, s + k);
                    hx = fmaxf(hx, x[k].x); lx = fminf(lx, x[k].x);
                    hy = fmaxf(hy, x[k].y); ly = fminf(ly, x[k].y);
                }
            float epx[WA_REG], enx[WA_REG], epy[WA_REG], eny[WA_REG];
#pragma unroll
            for (int k = 0; k < WA_REG; k++)
                if (k < d) {
                    epx[k] = __expf((x[k].x - hx) * ig); enx[k] = __expf((lx - x[k].x) * ig);
                    epy[k] = __expf((x[k].y - hy) * ig); eny[k] = __expf((ly - x[k].y) * ig);
                    spx += epx[k]; snx += enx[k]; xpx += x[k].x * epx[k]; xnx += x[k].x * enx[k];
                    spy += epy[k]; sny += eny[k]; xpy += x[k].y * epy[k]; xny += x[k].y * eny[k];
                }
            xpx /= spx; xnx /= snx; xpy /= spy; xny /= sny;
#pragma unroll
            for (int k = 0; k < WA_REG; k++)
                if (k < d) {
                    float gx = epx[k] * (1.f + (x[k].x - xpx) * ig) / spx - enx[k] * (1.f - (x[k].x - xnx) * ig) / snx;
                    float gy = epy[k] * (1.f + (x[k].y - xpy) * ig) / spy - eny[k] * (1.f - (x[k].y - xny) * ig) / sny;
                    j.pin_grad[s + k] = make_float2(gx, gy);
                }
        } else {
            for (int k = 0; k < d; k++) {
                const float2 x = pin_xy(j, pos, s + k);
                hx = fmaxf(hx, x.x); lx = fminf(lx, x.x);
                hy = fmaxf(hy, x.y); ly = fminf(ly, x.y);
            }
            for (int k = 0; k < d; k++) {
                const float2 x = pin_xy(j, pos, s + k);
                const float epx = __expf((x.x - hx) * ig), enx = __expf((lx - x.x) * ig);
                const float epy = __expf((x.y - hy) * ig), eny = __expf((ly - x.y) * ig);
                spx += epx; snx += enx; xpx += x.x * epx; xnx += x.x * enx;
                spy += epy; sny += eny; xpy += x.y * epy; xny += x.y * eny;
            }
            xpx /= spx; xnx /= snx; xpy /= spy; xny /= sny;
            for (int k = 0; k < d; k++) {
                const float2 x = pin_xy(j, pos, s + k);
                const float epx = __expf((x.x - hx) * ig), enx = __expf((lx - x.x) * ig);
                const float epy = __expf((x.y - hy) * ig), eny = __expf((ly - x.y) * ig);
                float gx = epx * (1.f + (x.x - xpx) * ig) / spx - enx * (1.f - (x.x - xnx) * ig) / snx;
                float gy = epy * (1.f + (x.y - xpy) * ig) / spy - eny * (1.f - (x.y - xny) * ig) / sny;
                j.pin_grad[s + k] = make_float2(gx, gy);
            }
        }
        const float wa = (xpx - xnx) + (xpy - xny), hp = (hx - lx) + (hy - ly);
        if (j.out) j.out[i] = make_float2(wa, hp);
        wa_sum += (double)wa;
        hp_sum += (double)hp;
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
