// The learned start: a message-passing network over the cluster graph that proposes the clusters' start positions
// (in place of the wirelength-only start, src/run_placement.py:48-65, and of the clusters' start positions,
// src/run_placement.py:98). The reference has no learned part; these kernels are this library's own.
//
// The graph is the cluster problem's netlist as the placer keeps it: pins grouped by net (net_start, pin_cell with
// K = a fixed pin) and by cluster (cell_start, cell_pin). A message-passing step averages twice: each net takes the
// mean of its movable pins' clusters, each cluster the mean of its pins' nets. Both are gathers over a CSR in a fixed
// order, and so are their transposes (the backward pass), so training is deterministic without atomics:
//   P2N   out[net]     = sum over the net's pins of w_p2n[k] h[cell(k)]       (w_p2n = 1 / movable pins of the net)
//   N2C   out[cell]    = sum over the cell's pins of w_n2c[k] m[net(k)]       (w_n2c = 1 / pins of the cell)
//   N2C^T out[net]     = sum over the net's pins of w_n2ct[k] d[cell(k)]      (w_n2ct = 1 / pins of cell(k))
//   P2N^T out[cell]    = sum over the cell's pins of w_p2nt[k] d[net(k)]      (w_p2nt = 1 / movable pins of net(k))
// Dense layers keep their weights in bf16 (an fp32 master copy lives with the optimiser) and accumulate in fp32.
// Weight gradients are per-block partial sums over rows, added in block order by a second kernel.
#include <cuda_bf16.h>

#include "gp103.cuh"
#include "kernels.cuh"
#include "step.cuh"

using namespace gp103;

#define REQUIRE(cond)                      \
    do {                                   \
        if (!(cond)) return GP103_ERR_ARG; \
    } while (0)

namespace {

constexpr int LW = 64;                     // hidden width (and the largest input / output width of a dense layer)
constexpr int WG_ROWS = 32;                // rows per shared-memory tile of the weight-gradient kernel
constexpr int WG_BLOCKS = 304;             // weight-gradient partials: 2 blocks per SM

__device__ __forceinline__ float bf(uint16_t u) { return __uint_as_float((uint32_t)u << 16); }

// ----------------------------------------------------------------------------- graph
__global__ void net_pins_kernel(const int* net_start, const int* pin_cell, int num_nets, int num_cells, int* pin_net,
                                float* mov_inv) {
    pdl_wait();
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < num_nets; e += gridDim.x * blockDim.x) {
        int mov = 0;
        for (int p = net_start[e]; p < net_start[e + 1]; p++) {
            pin_net[p] = e;
            mov += (unsigned)pin_cell[p] < (unsigned)num_cells;
        }
        mov_inv[e] = mov > 0 ? 1.f / (float)mov : 0.f;
    }
}

__global__ void graph_ops_kernel(const int* pin_cell, const int* cell_start, const int* cell_pin, const int* pin_net,
                                 const float* mov_inv, int num_cells, int num_pins, int* net_pin_cell, float* w_p2n,
                                 float* w_n2ct, int* cell_pin_net, float* w_n2c, float* w_p2nt) {
    pdl_wait();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < num_pins; k += gridDim.x * blockDim.x) {
        // net order: pin k of the net CSR
        const int c = pin_cell[k];
        const bool mov = (unsigned)c < (unsigned)num_cells;
        net_pin_cell[k] = mov ? c : -1;
        w_p2n[k] = mov_inv[pin_net[k]];
        w_n2ct[k] = mov ? 1.f / (float)max(cell_start[c + 1] - cell_start[c], 1) : 0.f;
    }
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < num_cells; c += gridDim.x * blockDim.x) {
        // cell order: the pins of cell c
        const int b = cell_start[c], e = cell_start[c + 1];
        const float inv = e > b ? 1.f / (float)(e - b) : 0.f;
        for (int k = b; k < e; k++) {
            const int p = cell_pin[k], net = pin_net[p];
            cell_pin_net[k] = net;
            w_n2c[k] = inv;
            w_p2nt[k] = mov_inv[net];
        }
    }
}

// out[s][0:W] (+)= sum over k in [seg[s], seg[s+1]) of w[k] src[idx[k]][0:W] (idx < 0: skipped; accumulate: added to
// what out holds); one warp per segment, the elements in order (deterministic), each lane two columns.
__global__ void __launch_bounds__(256) seg_gather_kernel(const int* seg, int num_seg, const int* idx, const float* w,
                                                         const float* src, int width, int accumulate, float* out) {
    pdl_wait();
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < num_seg; s += warps) {
        float a0 = 0.f, a1 = 0.f;
        const int b = seg[s], e = seg[s + 1];
        for (int k = b; k < e; k++) {
            const int r = idx[k];
            if (r < 0) continue;
            const float wk = w[k];
            const float* row = src + (size_t)r * width;
            if (lane < width) a0 = fmaf(wk, row[lane], a0);
            if (lane + 32 < width) a1 = fmaf(wk, row[lane + 32], a1);
        }
        float* o = out + (size_t)s * width;
        if (lane < width) o[lane] = accumulate ? o[lane] + a0 : a0;
        if (lane + 32 < width) o[lane + 32] = accumulate ? o[lane + 32] + a1 : a1;
    }
}

// ----------------------------------------------------------------------------- dense layers
// out[i][c] = act(b[c] + sum_j x[i][j] wx[j][c] + sum_j a[i][j] wa[j][c]), c < out_dim; one warp per row, lane c
// computes columns c and c + 32; weights as fp32 in shared memory (from their bf16 values).
__device__ __forceinline__ float act_fwd(float z, int act) {
    return act == 1 ? fmaxf(z, 0.f) : act == 2 ? 1.f / (1.f + __expf(-z)) : z;
}

__global__ void __launch_bounds__(256) dense_fwd_kernel(const float* x, int n, int in_x, const float* a, int in_a,
                                                        const uint16_t* wx, const uint16_t* wa, const float* bias,
                                                        int out_dim, int act, float* out) {
    __shared__ float swx[LW * LW], swa[LW * LW], sb[LW];
    pdl_wait();                                   // (the weights may come from the optimiser step just before)
    for (int i = threadIdx.x; i < in_x * out_dim; i += blockDim.x) swx[(i / out_dim) * LW + i % out_dim] = bf(wx[i]);
    for (int i = threadIdx.x; i < in_a * out_dim; i += blockDim.x) swa[(i / out_dim) * LW + i % out_dim] = bf(wa[i]);
    for (int i = threadIdx.x; i < out_dim; i += blockDim.x) sb[i] = bias[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warps = (gridDim.x * blockDim.x) >> 5;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        const float* xr = x + (size_t)r * in_x;
        const float x0 = lane < in_x ? xr[lane] : 0.f, x1 = lane + 32 < in_x ? xr[lane + 32] : 0.f;
        float a0v = 0.f, a1v = 0.f;
        if (in_a) {
            const float* ar = a + (size_t)r * in_a;
            a0v = lane < in_a ? ar[lane] : 0.f;
            a1v = lane + 32 < in_a ? ar[lane + 32] : 0.f;
        }
        const int c0 = lane, c1 = lane + 32;
        float z0 = c0 < out_dim ? sb[c0] : 0.f, z1 = c1 < out_dim ? sb[c1] : 0.f;
        for (int j = 0; j < in_x; j++) {
            const float xj = __shfl_sync(0xffffffffu, j < 32 ? x0 : x1, j & 31);
            z0 = fmaf(xj, swx[j * LW + c0], z0);
            z1 = fmaf(xj, swx[j * LW + c1], z1);
        }
        for (int j = 0; j < in_a; j++) {
            const float aj = __shfl_sync(0xffffffffu, j < 32 ? a0v : a1v, j & 31);
            z0 = fmaf(aj, swa[j * LW + c0], z0);
            z1 = fmaf(aj, swa[j * LW + c1], z1);
        }
        float* orow = out + (size_t)r * out_dim;
        if (c0 < out_dim) orow[c0] = act_fwd(z0, act);
        if (c1 < out_dim) orow[c1] = act_fwd(z1, act);
    }
}

// dz = dout * act'(out); dx[i][j] = sum_c dz[i][c] wx[j][c], da likewise with wa (either may be null).
__global__ void __launch_bounds__(256) dense_bwd_data_kernel(int n, int in_x, int in_a, const uint16_t* wx,
                                                             const uint16_t* wa, int out_dim, int act,
                                                             const float* out, const float* dout, float* dz,
                                                             float* dx, float* da) {
    __shared__ float swx[LW * LW], swa[LW * LW];     // transposed: [c][j]
    pdl_wait();
    for (int i = threadIdx.x; i < in_x * out_dim; i += blockDim.x) swx[(i % out_dim) * LW + i / out_dim] = bf(wx[i]);
    for (int i = threadIdx.x; i < in_a * out_dim; i += blockDim.x) swa[(i % out_dim) * LW + i / out_dim] = bf(wa[i]);
    __syncthreads();
    const int lane = threadIdx.x & 31, warps = (gridDim.x * blockDim.x) >> 5;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        const float* orow = out + (size_t)r * out_dim;
        const float* grow = dout + (size_t)r * out_dim;
        float d0 = 0.f, d1 = 0.f;
        const int c0 = lane, c1 = lane + 32;
        if (c0 < out_dim) {
            const float y = orow[c0], g = grow[c0];
            d0 = act == 1 ? (y > 0.f ? g : 0.f) : act == 2 ? g * y * (1.f - y) : g;
        }
        if (c1 < out_dim) {
            const float y = orow[c1], g = grow[c1];
            d1 = act == 1 ? (y > 0.f ? g : 0.f) : act == 2 ? g * y * (1.f - y) : g;
        }
        float* zrow = dz + (size_t)r * out_dim;
        if (c0 < out_dim) zrow[c0] = d0;
        if (c1 < out_dim) zrow[c1] = d1;
        if (dx) {
            float s0 = 0.f, s1 = 0.f;
            for (int c = 0; c < out_dim; c++) {
                const float dc = __shfl_sync(0xffffffffu, c < 32 ? d0 : d1, c & 31);
                s0 = fmaf(dc, swx[c * LW + lane], s0);
                s1 = fmaf(dc, swx[c * LW + lane + 32], s1);
            }
            float* xr = dx + (size_t)r * in_x;
            if (lane < in_x) xr[lane] = s0;
            if (lane + 32 < in_x) xr[lane + 32] = s1;
        }
        if (da) {
            float s0 = 0.f, s1 = 0.f;
            for (int c = 0; c < out_dim; c++) {
                const float dc = __shfl_sync(0xffffffffu, c < 32 ? d0 : d1, c & 31);
                s0 = fmaf(dc, swa[c * LW + lane], s0);
                s1 = fmaf(dc, swa[c * LW + lane + 32], s1);
            }
            float* ar = da + (size_t)r * in_a;
            if (lane < in_a) ar[lane] = s0;
            if (lane + 32 < in_a) ar[lane + 32] = s1;
        }
    }
}

// Partial weight gradients of one block (a contiguous range of rows): g[j][c] = sum_i v[i][j] dz[i][c] for v = x
// (j < in_x) and v = a (in_x <= j < in_x + in_a), then the bias sum_i dz[i][c]; rows staged in shared memory 32 at a
// time, thread t holding the (j, c) pairs t, t + 256, ... of the (in_x + in_a + 1) x out_dim outputs.
__global__ void __launch_bounds__(256) dense_bwd_weight_kernel(const float* x, int n, int in_x, const float* a,
                                                               int in_a, const float* dz, int out_dim,
                                                               float* partials) {
    __shared__ float sv[WG_ROWS][2 * LW + 1], sd[WG_ROWS][LW];
    pdl_wait();
    const int in = in_x + in_a + 1, total = in * out_dim;
    constexpr int PER = (2 * LW + 1) * LW / 256 + 1;
    float acc[PER];
#pragma unroll
    for (int q = 0; q < PER; q++) acc[q] = 0.f;
    const long long r0 = (long long)n * blockIdx.x / gridDim.x, r1 = (long long)n * (blockIdx.x + 1) / gridDim.x;
    for (long long t0 = r0; t0 < r1; t0 += WG_ROWS) {
        const int rows = (int)min((long long)WG_ROWS, r1 - t0);
        __syncthreads();
        for (int i = threadIdx.x; i < rows * in; i += blockDim.x) {
            const int rr = i / in, j = i - rr * in;
            const long long r = t0 + rr;
            sv[rr][j] = j < in_x ? x[r * in_x + j] : j < in_x + in_a ? a[r * in_a + (j - in_x)] : 1.f;
        }
        for (int i = threadIdx.x; i < rows * out_dim; i += blockDim.x) {
            const int rr = i / out_dim, c = i - rr * out_dim;
            sd[rr][c] = dz[(t0 + rr) * out_dim + c];
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const int o = threadIdx.x + q * 256;
            if (o < total) {
                const int j = o / out_dim, c = o - j * out_dim;
                float s = acc[q];
                for (int rr = 0; rr < rows; rr++) s = fmaf(sv[rr][j], sd[rr][c], s);
                acc[q] = s;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int o = threadIdx.x + q * 256;
        if (o < total) partials[(size_t)blockIdx.x * total + o] = acc[q];
    }
}

// The partials added in block order (double), -> gwx [in_x][out], gwa [in_a][out], gb [out].
__global__ void weight_reduce_kernel(const float* partials, int blocks, int in_x, int in_a, int out_dim, float* gwx,
                                     float* gwa, float* gb) {
    pdl_wait();
    const int total = (in_x + in_a + 1) * out_dim;
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < total; o += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < blocks; b++) s += partials[(size_t)b * total + o];
        const int j = o / out_dim, c = o - j * out_dim;
        if (j < in_x) gwx[j * out_dim + c] = (float)s;
        else if (j < in_x + in_a) gwa[(j - in_x) * out_dim + c] = (float)s;
        else gb[c] = (float)s;
    }
}

// ----------------------------------------------------------------------------- loss, optimiser
// loss = mean over rows of sum_d (y - t)^2 (float64 block partials); dy = 2 (y - t) / n.
__global__ void __launch_bounds__(256) mse_kernel(const float* y, const float* t, int n, int dim, float* dy,
                                                  Reduce red) {
    pdl_wait();
    const float inv = 2.f / (float)max(n, 1);
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)n * dim;
         i += (long long)gridDim.x * blockDim.x) {
        const float d = y[i] - t[i];
        dy[i] = inv * d;
        acc += (double)d * d;
    }
    double v[1] = {acc / (double)max(n, 1)};
    grid_sum<1>(v, red);
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, uint16_t* p16, int n, float lr, float b1,
                            float b2, float eps, float c1, float c2, float wd) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float step = lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        const float pi = p[i] - step - lr * wd * p[i];
        p[i] = pi;
        p16[i] = __bfloat16_as_ushort(__float2bfloat16_rn(pi));
    }
}

// ----------------------------------------------------------------------------- features
// Fixed pins of each net (a pin whose cell is >= num_cells sits at its offset): r[net] = (mean x / width, mean y /
// height, 1) when the net has one, else 0.
__global__ void net_anchor_kernel(const int* net_start, const int* pin_cell, const float2* pin_off, int num_nets,
                                  int num_cells, float inv_w, float inv_h, float* r) {
    pdl_wait();
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < num_nets; e += gridDim.x * blockDim.x) {
        float sx = 0.f, sy = 0.f;
        int k = 0;
        for (int p = net_start[e]; p < net_start[e + 1]; p++)
            if ((unsigned)pin_cell[p] >= (unsigned)num_cells) {
                sx += pin_off[p].x;
                sy += pin_off[p].y;
                k++;
            }
        r[3 * e] = k ? sx / k * inv_w : 0.f;
        r[3 * e + 1] = k ? sy / k * inv_h : 0.f;
        r[3 * e + 2] = k ? 1.f : 0.f;
    }
}

// One step of the anchor propagation: a cluster without an anchor whose neighbourhood mean z (x, y, weight) has
// weight takes the anchor z.xy / z.w at hop `hop`; state: anc [K][3] = (x, y, 1) or 0, hop [K] (-1: none).
__global__ void anchor_step_kernel(const float* z, int num_cells, int hop, float* anc, float* hops) {
    pdl_wait();
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < num_cells; c += gridDim.x * blockDim.x) {
        if (hops[c] >= 0.f) continue;
        const float w = z[3 * c + 2];
        if (w > 0.f) {
            anc[3 * c] = z[3 * c] / w;
            anc[3 * c + 1] = z[3 * c + 1] / w;
            anc[3 * c + 2] = 1.f;
            hops[c] = (float)hop;
        }
    }
}

// One Jacobi sweep of the harmonic coordinates: each net's mean position over all its pins (a movable pin at its
// cluster's current estimate h, a fixed pin where it is), r[net] = (x, y, 1) (0 for a net without pins).
__global__ void net_mean_kernel(const int* net_start, const int* pin_cell, const float2* pin_off, const float* h,
                                int num_nets, int num_cells, float inv_w, float inv_h, float* r) {
    pdl_wait();
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < num_nets; e += gridDim.x * blockDim.x) {
        float sx = 0.f, sy = 0.f;
        const int b = net_start[e], n = net_start[e + 1] - b;
        for (int p = b; p < b + n; p++) {
            const int c = pin_cell[p];
            if ((unsigned)c < (unsigned)num_cells) {
                sx += h[2 * c];
                sy += h[2 * c + 1];
            } else {
                sx += pin_off[p].x * inv_w;
                sy += pin_off[p].y * inv_h;
            }
        }
        r[3 * e] = n ? sx / n : 0.f;
        r[3 * e + 1] = n ? sy / n : 0.f;
        r[3 * e + 2] = n ? 1.f : 0.f;
    }
}

// The sweep's cluster side: h = z.xy / z.w (the mean over the cluster's nets; a cluster without nets keeps its h).
__global__ void harmonic_step_kernel(const float* z, int num_cells, float* h) {
    pdl_wait();
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < num_cells; c += gridDim.x * blockDim.x) {
        const float w = z[3 * c + 2];
        if (w > 0.f) {
            h[2 * c] = z[3 * c] / w;
            h[2 * c + 1] = z[3 * c + 1] / w;
        }
    }
}

// The sweeps start from the anchors (the region's centre for a cluster without one).
__global__ void harmonic_init_kernel(const float* anc, const float* hops, int num_cells, float* h) {
    pdl_wait();
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < num_cells; c += gridDim.x * blockDim.x) {
        const bool has = hops[c] >= 0.f;
        h[2 * c] = has ? anc[3 * c] : 0.5f;
        h[2 * c + 1] = has ? anc[3 * c + 1] : 0.5f;
    }
}

__global__ void fill_kernel(float* p, int n, float v) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

// Features of each cluster, F = 10: log(area / mean area), log(1 + nets) / 4, log(1 + member pins) / 4, anchor x,
// anchor y (fractions of the region; the centre when none), hop / max_hop (1 when none), 1 if anchored, the anchor's
// distance from the region's centre, the harmonic x and y.
__global__ void features_kernel(const float* area, double mean_area, const int* cell_start, const float* pin_count,
                                const float* anc, const float* hops, const float* harm, int num_cells, int max_hop,
                                float* feat) {
    pdl_wait();
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < num_cells; c += gridDim.x * blockDim.x) {
        const int nets = cell_start[c + 1] - cell_start[c];      // (the cluster problem: one pin per net and cluster)
        const bool has = hops[c] >= 0.f;
        const float ax = has ? anc[3 * c] : 0.5f, ay = has ? anc[3 * c + 1] : 0.5f;
        float* f = feat + (size_t)c * 10;
        f[0] = logf(fmaxf(area[c], 1e-30f) / (float)mean_area);
        f[1] = log1pf((float)nets) * 0.25f;
        f[2] = log1pf(pin_count ? pin_count[c] : (float)nets) * 0.25f;
        f[3] = ax;
        f[4] = ay;
        f[5] = has ? hops[c] / (float)max_hop : 1.f;
        f[6] = has ? 1.f : 0.f;
        f[7] = sqrtf((ax - 0.5f) * (ax - 0.5f) + (ay - 0.5f) * (ay - 0.5f));
        f[8] = harm[2 * c];
        f[9] = harm[2 * c + 1];
    }
}

}  // namespace

// ================================================================================================ C ABI
extern "C" size_t gp103_learn_graph_scratch(int num_nets, int num_pins) {
    return (size_t)num_pins * sizeof(int) + (size_t)num_nets * sizeof(float) + 256;
}

extern "C" int gp103_learn_graph(const int* net_start, const int* pin_cell, const int* cell_start, const int* cell_pin,
                                 int num_nets, int num_cells, int num_pins, void* scratch, size_t scratch_bytes,
                                 int* net_pin_cell, float* w_p2n, float* w_n2ct, int* cell_pin_net, float* w_n2c,
                                 float* w_p2nt, cudaStream_t s) {
    REQUIRE(num_nets >= 0 && num_cells >= 0 && num_pins >= 0 && net_start && cell_start);
    REQUIRE(num_pins == 0 || (pin_cell && cell_pin && net_pin_cell && w_p2n && w_n2ct && cell_pin_net && w_n2c &&
                              w_p2nt));
    REQUIRE(scratch && scratch_bytes >= gp103_learn_graph_scratch(num_nets, num_pins));
    int* pin_net = (int*)scratch;
    float* mov_inv = (float*)((char*)scratch + (((size_t)num_pins * sizeof(int) + 255) & ~(size_t)255));
    if (num_nets > 0) {
        if (launch_k(net_pins_kernel, dim3(grid_for(num_nets, 256, 8)), dim3(256), 0, s, net_start, pin_cell,
                     num_nets, num_cells, pin_net, mov_inv) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    const long long items = num_pins > num_cells ? num_pins : num_cells;
    if (items > 0) {
        if (launch_k(graph_ops_kernel, dim3(grid_for(items, 256, 8)), dim3(256), 0, s, pin_cell, cell_start, cell_pin,
                     (const int*)pin_net, (const float*)mov_inv, num_cells, num_pins, net_pin_cell, w_p2n, w_n2ct,
                     cell_pin_net, w_n2c, w_p2nt) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    return GP103_OK;
}

extern "C" int gp103_seg_gather(const int* seg_start, int num_seg, const int* idx, const float* w, const float* src,
                                int width, int accumulate, float* out, cudaStream_t s) {
    REQUIRE(num_seg >= 0 && width >= 1 && width <= LW && seg_start && out);
    if (num_seg == 0) return GP103_OK;
    REQUIRE(idx && w && src);
    if (launch_k(seg_gather_kernel, dim3(grid_for((long long)num_seg * 32, 256, 8)), dim3(256), 0, s, seg_start,
                 num_seg, idx, w, src, width, accumulate, out) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

extern "C" int gp103_dense_fwd(const float* x, int n, int in_x, const float* a, int in_a, const uint16_t* wx,
                               const uint16_t* wa, const float* bias, int out_dim, int act, float* out,
                               cudaStream_t s) {
    REQUIRE(n >= 0 && in_x >= 1 && in_x <= LW && in_a >= 0 && in_a <= LW && out_dim >= 1 && out_dim <= LW);
    REQUIRE(act >= 0 && act <= 2 && wx && bias && (in_a == 0 || wa));
    if (n == 0) return GP103_OK;
    REQUIRE(x && out && (in_a == 0 || a));
    if (launch_k(dense_fwd_kernel, dim3(grid_for((long long)n * 32, 256, 8)), dim3(256), 0, s, x, n, in_x, a, in_a,
                 wx, wa, bias, out_dim, act, out) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

extern "C" size_t gp103_dense_bwd_scratch(int in_x, int in_a, int out_dim) {
    return (size_t)WG_BLOCKS * (in_x + in_a + 1) * out_dim * sizeof(float);
}

extern "C" int gp103_dense_bwd(const float* x, int n, int in_x, const float* a, int in_a, const uint16_t* wx,
                               const uint16_t* wa, int out_dim, int act, const float* out, const float* dout,
                               float* dz, float* dx, float* da, void* scratch, size_t scratch_bytes, float* gwx,
                               float* gwa, float* gb, cudaStream_t s) {
    REQUIRE(n >= 0 && in_x >= 1 && in_x <= LW && in_a >= 0 && in_a <= LW && out_dim >= 1 && out_dim <= LW);
    REQUIRE(act >= 0 && act <= 2 && wx && (in_a == 0 || (wa && gwa)) && gwx && gb && scratch);
    REQUIRE(scratch_bytes >= gp103_dense_bwd_scratch(in_x, in_a, out_dim));
    REQUIRE(n == 0 || (x && out && dout && dz && (in_a == 0 || a)));
    if (n > 0) {
        if (launch_k(dense_bwd_data_kernel, dim3(grid_for((long long)n * 32, 256, 8)), dim3(256), 0, s, n, in_x,
                     in_a, wx, wa, out_dim, act, out, dout, dz, dx, in_a ? da : (float*)nullptr) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    const int blocks = n > 0 ? (n < WG_BLOCKS * WG_ROWS ? ceil_div(n, WG_ROWS) : WG_BLOCKS) : 1;
    if (launch_k(dense_bwd_weight_kernel, dim3(blocks), dim3(256), 0, s, x, n, in_x, a, in_a, (const float*)dz,
                 out_dim, (float*)scratch) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    const int total = (in_x + in_a + 1) * out_dim;
    if (launch_k(weight_reduce_kernel, dim3(ceil_div(total, 256)), dim3(256), 0, s, (const float*)scratch, blocks,
                 in_x, in_a, out_dim, gwx, gwa, gb) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

extern "C" int gp103_mse(const float* y, const float* t, int n, int dim, float* dy, double* loss, void* scratch,
                         cudaStream_t s) {
    REQUIRE(n >= 0 && dim >= 1 && loss && scratch && (n == 0 || (y && t && dy)));
    Reduce r;
    r.partials = (double*)scratch;
    r.count = (int*)((char*)scratch + sizeof(double) * MAX_BLOCKS);
    static int grid = 0;
    if (!grid) grid = resident_blocks(mse_kernel, 256);
    if (launch_k(mse_kernel, dim3(grid < MAX_BLOCKS ? grid : MAX_BLOCKS), dim3(256), 0, s, y, t, n, dim, dy, r) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    const int k0 = 0;
    return launch_totals(&r, &k0, 1, loss, s);
}

extern "C" int gp103_adam(float* param, const float* grad, float* m, float* v, uint16_t* param_bf16, int n, float lr,
                          float beta1, float beta2, float eps, int step, float weight_decay, cudaStream_t s) {
    REQUIRE(n >= 0 && step >= 1 && (n == 0 || (param && grad && m && v && param_bf16)));
    if (n == 0) return GP103_OK;
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    if (launch_k(adam_kernel, dim3(grid_for(n, 256, 4)), dim3(256), 0, s, param, grad, m, v, param_bf16, n, lr, beta1,
                 beta2, eps, c1, c2, weight_decay) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

extern "C" size_t gp103_learn_features_scratch(int num_nets, int num_cells) {
    return ((size_t)3 * num_nets * sizeof(float) + 255 & ~(size_t)255) +
           2 * ((size_t)3 * num_cells * sizeof(float) + 255 & ~(size_t)255) +
           ((size_t)num_cells * sizeof(float) + 255 & ~(size_t)255) +
           ((size_t)2 * num_cells * sizeof(float) + 255 & ~(size_t)255);
}

extern "C" int gp103_learn_features(const int* net_start, const int* pin_cell, const float* pin_off,
                                    const int* cell_start, int num_nets, int num_cells, int num_pins,
                                    const int* net_pin_cell, const float* w_p2n, const int* cell_pin_net,
                                    const float* w_n2c, const float* area, const float* pin_count, double mean_area,
                                    float width, float height, int max_hop, int sweeps, void* scratch,
                                    size_t scratch_bytes, float* feat, cudaStream_t s) {
    REQUIRE(num_nets >= 0 && num_cells >= 0 && num_pins >= 0 && max_hop >= 1 && sweeps >= 0 && width > 0.f &&
            height > 0.f);
    REQUIRE(net_start && cell_start && feat && scratch && mean_area > 0.0);
    REQUIRE(scratch_bytes >= gp103_learn_features_scratch(num_nets, num_cells));
    REQUIRE(num_pins == 0 || (pin_cell && pin_off && net_pin_cell && w_p2n && cell_pin_net && w_n2c));
    REQUIRE(num_cells == 0 || area);
    if (num_cells == 0) return GP103_OK;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    char* w = (char*)scratch;
    float* rnet = (float*)w;
    w += up((size_t)3 * num_nets * sizeof(float));
    float* anc = (float*)w;
    w += up((size_t)3 * num_cells * sizeof(float));
    float* z = (float*)w;
    w += up((size_t)3 * num_cells * sizeof(float));
    float* hops = (float*)w;
    w += up((size_t)num_cells * sizeof(float));
    float* harm = (float*)w;
    if (cudaMemsetAsync(anc, 0, sizeof(float) * 3 * num_cells, s) != cudaSuccess) return GP103_ERR_CUDA;
    if (launch_k(fill_kernel, dim3(grid_for(num_cells, 256, 8)), dim3(256), 0, s, hops, num_cells, -1.f) !=
        cudaSuccess)                                                 // no anchor yet
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (num_nets > 0) {
        if (launch_k(net_anchor_kernel, dim3(grid_for(num_nets, 256, 8)), dim3(256), 0, s, net_start, pin_cell,
                     (const float2*)pin_off, num_nets, num_cells, 1.f / width, 1.f / height, rnet) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    // hop 0: a cluster on a net with a fixed pin takes the mean of those nets' fixed pins (N2C of r with weights
    // 1 / pins: the weight channel says whether any such net exists)
    for (int hop = 0; hop <= max_hop; hop++) {
        int st;
        if (hop > 0) {
            // the anchored clusters' (x, y, 1) averaged over each net's movable pins
            if ((st = gp103_seg_gather(net_start, num_nets, net_pin_cell, w_p2n, anc, 3, 0, rnet, s))) return st;
        }
        // then over each cluster's nets (hop 0: the nets' fixed pins)
        if ((st = gp103_seg_gather(cell_start, num_cells, cell_pin_net, w_n2c, rnet, 3, 0, z, s))) return st;
        if (launch_k(anchor_step_kernel, dim3(grid_for(num_cells, 256, 8)), dim3(256), 0, s, (const float*)z,
                     num_cells, hop, anc, hops) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    // the harmonic coordinates: from the anchors, `sweeps` Jacobi sweeps of the mean over each cluster's nets
    const int gc = grid_for(num_cells, 256, 8), ge = grid_for(num_nets > 0 ? num_nets : 1, 256, 8);
    if (launch_k(harmonic_init_kernel, dim3(gc), dim3(256), 0, s, (const float*)anc, (const float*)hops, num_cells,
                 harm) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    for (int k = 0; k < sweeps && num_nets > 0; k++) {
        if (launch_k(net_mean_kernel, dim3(ge), dim3(256), 0, s, net_start, pin_cell, (const float2*)pin_off,
                     (const float*)harm, num_nets, num_cells, 1.f / width, 1.f / height, rnet) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
        int st;
        if ((st = gp103_seg_gather(cell_start, num_cells, cell_pin_net, w_n2c, rnet, 3, 0, z, s))) return st;
        if (launch_k(harmonic_step_kernel, dim3(gc), dim3(256), 0, s, (const float*)z, num_cells, harm) !=
            cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    if (launch_k(features_kernel, dim3(gc), dim3(256), 0, s, area, mean_area, cell_start, pin_count,
                 (const float*)anc, (const float*)hops, (const float*)harm, num_cells, max_hop, feat) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}
