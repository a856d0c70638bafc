// Nesterov / Barzilai-Borwein step, the run's control and the accepted-step selection (GB300, sm_103a).
//
// Reference: cpp_to_py/gp_cuda_kernel.cu:155-259 (nesterov_step_kernel, control_kernel, select_kernel) with the
// host rules they replay: src/nesterov_optimizer.py:34-53, src/param_scheduler.py:63-116, src/resolution.py:33-56.
// The fused path keeps two copies of (u, v, g) and an index of the current one in device memory: an accepted step
// flips the index instead of copying three arrays (select_kernel's copies).
#include <math.h>

#include "gp103.cuh"
#include "kernels.cuh"
#include "step.cuh"

namespace gp103 {

// ----------------------------------------------------------------------------- reference-layout kernels
__global__ void nesterov_step_kernel(const float* u, const float* v, const float* g, const float* lo, const float* hi,
                                     const float* alpha_p, const float* coef_p, int n, float* u_next, float* v_next) {
    pdl_wait();
    const float alpha = *alpha_p, coef = *coef_p;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float un = fmaf(-alpha, g[i], v[i]);
        u_next[i] = un;
        v_next[i] = fminf(fmaxf(fmaf(coef, un - u[i], un), lo[i]), hi[i]);
    }
}

int launch_nesterov_step(const float* u, const float* v, const float* g, const float* lo, const float* hi,
                         const float* alpha, const float* coef, int n, float* u_next, float* v_next, cudaStream_t s) {
    if (n == 0) return GP103_OK;
    if (launch_k(nesterov_step_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, u, v, g, lo, hi, alpha, coef, n, u_next, v_next) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// One pass of the control, float64, in the order of control_kernel (gp_cuda_kernel.cu:183-240). -> accepted.
__device__ __forceinline__ bool control_body(double* S, float* kp, const double* c, double moved, double turned,
                                             double hpwl, double ovf, double wa) {
    S[S_ACCEPT] = 0;
    S[S_IS_BEST] = 0;
    if (S[S_STOP] != 0) return false;
    if (!(isfinite(moved) && isfinite(turned) && isfinite(hpwl) && isfinite(ovf))) {
        S[S_STOP] = 3;
        return false;
    }
    const double alpha_next = turned > 0 ? moved / turned : S[S_ALPHA];
    S[S_ALPHA] = alpha_next;
    S[S_EVALS] += 1;
    S[S_ACCEPT] = 1;
    S[S_A] = (1 + sqrt(4 * S[S_A] * S[S_A] + 1)) / 2;
    double iter = S[S_ITER];
    S[S_MOTION] = moved / c[C_MOTION_UNIT];
    const double part = S[S_LAM] * c[C_TOTAL_AREA];
    S[S_WW] = part / (c[C_TOTAL_PINS] + part);
    const double mu = hpwl < S[S_HPWL_PREV] ? 1.05 * 0.98
                                             : 1.05 * fmax(pow(1.05, -S[S_MOTION] * c[C_PITCH] / S[S_GAM]), 0.95);
    S[S_HPWL_PREV] = hpwl;
    S[S_MU] = mu;
    S[S_LAM] *= mu;
    if (c[C_ACCURACY] != 0) {
        const double err = fmax(1e-6, 1 - wa / fmax(hpwl, 1e-12)), m = fmax(mu, 1 / mu);
        const double g = S[S_GAM] * fmin(m, fmax(1 / m, sqrt(fmax(ovf, 1e-3) / c[C_REFINE] / err)));
        S[S_GAM] = fmin(100 * c[C_BASE_GAMMA], fmax(0.01 * c[C_BASE_GAMMA], g));
    } else {
        S[S_GAM] = c[C_BASE_GAMMA] * pow(10.0, (ovf - 0.1) * 20 / 9 - 1);
    }
    S[S_ITER] = iter = iter + 1;
    double stop = 0, is_best = 0;
    if (!(hpwl < 1e30 && ovf < 1e30)) {
        stop = 3;
    } else {
        if (iter >= c[C_MIN_ITER] && ovf < c[C_STOP_OVF]) {
            S[S_SETTLED] += 1;
            is_best = hpwl < S[S_BEST_HPWL];
            S[S_BEST_HPWL] = fmin(hpwl, S[S_BEST_HPWL]);
            if (S[S_SETTLED] > c[C_SETTLE]) stop = 1;
        } else if (S[S_SETTLED] == 0) {
            is_best = ovf < S[S_BEST_OVF];
            if (ovf < S[S_BEST_OVF] * 0.999) S[S_IMPROVED] = iter;
            S[S_BEST_OVF] = fmin(ovf, S[S_BEST_OVF]);
        }
        if (stop == 0) {
            if ((is_best != 0 && S[S_SETTLED] > 0) || S[S_WW] < 0.95) S[S_IMPROVED] = iter;
            if (iter - S[S_IMPROVED] > c[C_STALL]) stop = 2;
        }
        if (stop == 0 && c[C_HANDOVER] > 0 && S[S_LAM] > 0 && S[S_GAM] <= c[C_HANDOVER]) stop = 5;
    }
    S[S_IS_BEST] = is_best;
    if (is_best != 0) {
        S[S_RES_HPWL] = hpwl;
        S[S_RES_OVF] = ovf;
        S[S_HAS_BEST] = 1;
    }
    S[S_LOOP_IT] += 1;
    if (stop == 0 && S[S_LOOP_IT] >= c[C_INNER]) stop = 4;
    S[S_STOP] = stop;
    if (S[S_HAS_BEST] == 0) {
        S[S_RES_HPWL] = hpwl;
        S[S_RES_OVF] = ovf;
    }
    const double a_next = (1 + sqrt(4 * S[S_A] * S[S_A] + 1)) / 2;
    kp[0] = (float)S[S_GAM];
    kp[1] = (float)S[S_LAM];
    kp[2] = (float)S[S_LAM];
    kp[3] = (float)alpha_next;
    kp[4] = (float)((S[S_A] - 1) / a_next);
    return true;
}

__global__ void control_kernel(double* S, float* kp, const double* c, const float* moved, const float* turned,
                               const float* hpwl, const float* ovf, const float* wa) {
    pdl_wait();
    control_body(S, kp, c, *moved, *turned, *hpwl, *ovf, *wa);
}

int launch_control(double* S, float* kp, const double* c, const float* moved, const float* turned, const float* hpwl,
                   const float* ovf, const float* wa, cudaStream_t s) {
    if (launch_k(control_kernel, dim3(1), dim3(1), 0, s, S, kp, c, moved, turned, hpwl, ovf, wa) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

__global__ void select_kernel(const double* S, float* u, float* v, float* g, const float* u_next, const float* v_next,
                              const float* g_next, float* best, int n) {
    pdl_wait();
    if (S[S_ACCEPT] == 0) return;
    const bool is_best = S[S_IS_BEST] != 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        u[i] = u_next[i];
        v[i] = v_next[i];
        g[i] = g_next[i];
        if (is_best) best[i] = v_next[i];
    }
}

int launch_select(const double* S, float* u, float* v, float* g, const float* u_next, const float* v_next,
                  const float* g_next, float* best, int n, cudaStream_t s) {
    if (n == 0) return GP103_OK;
    if (launch_k(select_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, S, u, v, g, u_next, v_next, g_next, best, n) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// ----------------------------------------------------------------------------- fused path
// u' = v - alpha g, v' = clamp(u' + coef (u' - u)) from the current buffers into the other ones, |v' - v|^2 in
// float64; the best placement of the previous pass (S[is_best]) is copied on the way, and the nodes of v' are
// counted per tile for the scatter's spatial order (shared-memory histogram, one global add per tile).
__global__ void __launch_bounds__(256) step_kernel(const __grid_constant__ StepJob j) {
    __shared__ int hist[ORDER_MAX_KEYS];
    pdl_wait();
    const bool counting = j.ord.counts != nullptr;
    const int keys = 2 * j.ord.tiles_x * j.ord.tiles_y;
    if (counting) {
        for (int k = threadIdx.x; k < keys; k += blockDim.x) hist[k] = 0;
        __syncthreads();
    }
    const int c = j.cur ? *j.cur : 0;
    const float2 *u = (const float2*)j.u[c], *v = (const float2*)j.v[c], *g = (const float2*)j.g[c];
    float2 *un_out = (float2*)j.u[1 - c], *vn_out = (float2*)j.v[1 - c];
    const float alpha = j.kp[3], coef = j.kp[4];
    const bool copy_best = j.best && j.S && j.S[S_IS_BEST] != 0;
    const float2 *lo = (const float2*)j.lo, *hi = (const float2*)j.hi;
    float d2 = 0.f;                            // per-thread partial (a few nodes); float32 warp tree, float64 across warps and blocks
    // two nodes (four coordinates) per iteration with 16-byte accesses when the node count is even
    const int quads = (j.n & 1) ? 0 : j.n >> 1;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < quads; q += gridDim.x * blockDim.x) {
        const float4 vi = ((const float4*)v)[q], gi = ((const float4*)g)[q], ui = ((const float4*)u)[q];
        const float4 l = ((const float4*)lo)[q], h = ((const float4*)hi)[q];
        float4 un, vn;
        un.x = fmaf(-alpha, gi.x, vi.x); un.y = fmaf(-alpha, gi.y, vi.y);
        un.z = fmaf(-alpha, gi.z, vi.z); un.w = fmaf(-alpha, gi.w, vi.w);
        vn.x = fminf(fmaxf(fmaf(coef, un.x - ui.x, un.x), l.x), h.x);
        vn.y = fminf(fmaxf(fmaf(coef, un.y - ui.y, un.y), l.y), h.y);
        vn.z = fminf(fmaxf(fmaf(coef, un.z - ui.z, un.z), l.z), h.z);
        vn.w = fminf(fmaxf(fmaf(coef, un.w - ui.w, un.w), l.w), h.w);
        ((float4*)un_out)[q] = un;
        ((float4*)vn_out)[q] = vn;
        if (copy_best) ((float4*)j.best)[q] = vi;
        const float dx = vn.x - vi.x, dy = vn.y - vi.y, dz = vn.z - vi.z, dw = vn.w - vi.w;
        d2 += (dx * dx + dy * dy) + (dz * dz + dw * dw);
        if (counting) {
            atomicAdd(&hist[order_key(j.ord, make_float2(vn.x, vn.y), 2 * q)], 1);
            atomicAdd(&hist[order_key(j.ord, make_float2(vn.z, vn.w), 2 * q + 1)], 1);
        }
    }
    for (int i = (j.n & 1) ? blockIdx.x * blockDim.x + threadIdx.x : j.n; i < j.n; i += gridDim.x * blockDim.x) {
        const float2 vi = v[i], gi = g[i], ui = u[i], l = lo[i], h = hi[i];
        const float ux = fmaf(-alpha, gi.x, vi.x), uy = fmaf(-alpha, gi.y, vi.y);
        const float vx = fminf(fmaxf(fmaf(coef, ux - ui.x, ux), l.x), h.x);
        const float vy = fminf(fmaxf(fmaf(coef, uy - ui.y, uy), l.y), h.y);
        un_out[i] = make_float2(ux, uy);
        vn_out[i] = make_float2(vx, vy);
        if (copy_best) ((float2*)j.best)[i] = vi;
        const float dx = vx - vi.x, dy = vy - vi.y;
        d2 += dx * dx + dy * dy;
        if (counting) atomicAdd(&hist[order_key(j.ord, make_float2(vx, vy), i)], 1);
    }
    if (counting) {
        __syncthreads();
        for (int k = threadIdx.x; k < keys; k += blockDim.x)
            if (hist[k]) atomicAdd(&j.ord.counts[k], hist[k]);
    }
    float r[1] = {d2};
    grid_sum<1>(r, j.red);
}

int launch_step(const StepJob& j, cudaStream_t s) {
    static const int resident = resident_blocks(step_kernel, 256);
    const int grid = min(grid_for(j.n, 256, 8), resident);
    if (launch_k(step_kernel, dim3(grid), dim3(256), 0, s, j) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// probe = clamp(v - step g, lo, hi); |probe - v|^2
__global__ void probe_kernel(const float2* v, const float2* g, const float2* lo, const float2* hi, float step,
                             const double* step_p, int n, float2* probe, Reduce red) {
    pdl_wait();
    if (step_p) step = __double2float_rn(*step_p);
    float d2 = 0.f;                            // per-thread partial (a few nodes); float32 warp tree, float64 across warps and blocks
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float2 vi = v[i], gi = g[i], l = lo[i], h = hi[i];
        const float px = fminf(fmaxf(fmaf(-step, gi.x, vi.x), l.x), h.x);
        const float py = fminf(fmaxf(fmaf(-step, gi.y, vi.y), l.y), h.y);
        probe[i] = make_float2(px, py);
        const float dx = px - vi.x, dy = py - vi.y;
        d2 += dx * dx + dy * dy;
    }
    float r[1] = {d2};
    grid_sum<1>(r, red);
}

int launch_probe(const float* v, const float* g, const float* lo, const float* hi, float step, int n, float* probe,
                 Reduce red, cudaStream_t s, const double* step_p) {
    if (launch_k(probe_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, (const float2*)v, (const float2*)g, (const float2*)lo,
                                                      (const float2*)hi, step, step_p, n, (float2*)probe, red) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// The density phase's control: one block adds the pass's float64 partial sums (in block order), then one thread
// runs the control; an accepted step flips the current buffers.
// pre: the totals the gather's block 0 summed (TOT_MOVED, TOT_WA, TOT_HPWL, TOT_OVF); the gather's own partials
// (the squared distance of the gradients) are summed here
__global__ void __launch_bounds__(256) control_fused_kernel(double* S, float* kp, const double* c, Reduce grad,
                                                            const double* pre, double ovf_scale, int* cur,
                                                            const int* ferr) {
    pdl_wait();
    __shared__ int failed;                                  // the field gave up a wait: this pass's field is stale
    if (threadIdx.x == 0) failed = ferr ? *(volatile const int*)ferr : 0;
    __syncthreads();
    if (failed) {
        if (threadIdx.x == 0) {
            S[S_ACCEPT] = 0;
            S[S_IS_BEST] = 0;
            if (S[S_STOP] == 0) S[S_STOP] = STOP_DEVICE_ERROR;
        }
        return;
    }
    // the state and the constants in registers first (one wave of loads): the control reads them one after another,
    // and through global memory every read after a write would wait a full memory latency
    double Sl[S_SIZE], cl[C_SIZE];
    float kpl[5];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < S_SIZE; i++) Sl[i] = S[i];
#pragma unroll
        for (int i = 0; i < C_SIZE; i++) cl[i] = c[i];
#pragma unroll
        for (int i = 0; i < 5; i++) kpl[i] = kp[i];
    }
    const double turned2 = block_total(grad, 0);
    if (threadIdx.x == 0) {
        const bool accepted = control_body(Sl, kpl, cl, sqrt(pre[TOT_MOVED]), sqrt(turned2), pre[TOT_HPWL],
                                           pre[TOT_OVF] * ovf_scale, pre[TOT_WA]);
#pragma unroll
        for (int i = 0; i < S_SIZE; i++) S[i] = Sl[i];
#pragma unroll
        for (int i = 0; i < 5; i++) kp[i] = kpl[i];
        if (accepted) *cur = 1 - *cur;
    }
}

int launch_control_fused(double* S, float* kp, const double* c, Reduce grad, const double* pre, double ovf_scale,
                         int* cur, const int* ferr, cudaStream_t s) {
    if (launch_k(control_fused_kernel, dim3(1), dim3(256), 0, s, S, kp, c, grad, pre, ovf_scale, cur, ferr) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// The wirelength-only start: NesterovOptimizer.step's step length and acceptance, ParamScheduler.start_step's end
// test (the WA fell by less than start_tol per iteration over the last 5), in float64.
__device__ void control_start_body(double* T, float* kp, double moved, double turned, double wa, double hpwl,
                                   int* cur) {
    T[GP103_T_ACCEPT] = 0;
    if (T[GP103_T_STOP] != 0 || T[GP103_T_DONE] != 0) return;
    if (!(isfinite(moved) && isfinite(turned) && isfinite(hpwl))) {
        T[GP103_T_STOP] = 3;
        return;
    }
    if (turned > 0) T[GP103_T_ALPHA] = moved / turned;
    const double a = T[GP103_T_A];
    T[GP103_T_A] = (1 + sqrt(4 * a * a + 1)) / 2;
    T[GP103_T_ACCEPT] = 1;
    *cur = 1 - *cur;
    T[GP103_T_EVALS] += 1;
    T[GP103_T_HPWL] = hpwl;
    T[GP103_T_WA] = wa;
    T[GP103_T_ITER] += 1;
    T[GP103_T_LOOP_IT] += 1;
    const int n = (int)T[GP103_T_NWA];
    T[GP103_T_RING + n % 6] = wa;
    T[GP103_T_NWA] = n + 1;
    const int window = 5;
    const bool done = (n + 1) > window && !(T[GP103_T_RING + (n + 1) % 6] - wa > T[GP103_T_START_TOL] * window * wa);
    if (done) T[GP103_T_DONE] = 1;
    else if (T[GP103_T_LOOP_IT] >= T[GP103_T_INNER]) T[GP103_T_STOP] = 4;
    const double an = T[GP103_T_A];
    kp[3] = (float)T[GP103_T_ALPHA];
    kp[4] = (float)((an - 1) / ((1 + sqrt(4 * an * an + 1)) / 2));
}

__global__ void __launch_bounds__(256) control_start_kernel(double* T, float* kp, Reduce grad, const double* pre,
                                                            int* cur, const int* ferr) {
    pdl_wait();
    __shared__ int failed;
    if (threadIdx.x == 0) failed = ferr ? *(volatile const int*)ferr : 0;
    __syncthreads();
    if (failed) {
        if (threadIdx.x == 0) {
            T[GP103_T_ACCEPT] = 0;
            if (T[GP103_T_STOP] == 0) T[GP103_T_STOP] = STOP_DEVICE_ERROR;
        }
        return;
    }
    const double turned2 = block_total(grad, 0);
    if (threadIdx.x == 0)
        control_start_body(T, kp, sqrt(pre[TOT_MOVED]), sqrt(turned2), pre[TOT_WA], pre[TOT_HPWL], cur);
}

int launch_control_start(double* T, float* kp, Reduce grad, const double* pre, int* cur, const int* ferr,
                         cudaStream_t s) {
    if (launch_k(control_start_kernel, dim3(1), dim3(256), 0, s, T, kp, grad, pre, cur, ferr) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

__global__ void finish_kernel(const double* S, const int* cur, float* const* v_unused, const float* v0, const float* v1,
                              float* best, int n) {
    pdl_wait();
    if (S[S_IS_BEST] == 0) return;
    const float* v = *cur ? v1 : v0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) best[i] = v[i];
}

int launch_finish(const double* S, const int* cur, const float* v0, const float* v1, float* best, int n,
                  cudaStream_t s) {
    if (n == 0) return GP103_OK;
    if (launch_k(finish_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, S, cur, nullptr, v0, v1, best, n) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// The set-up of a level's state before its first pass (the scalars of Placer.begin): kp = (gamma, lam, lam, 0, 0)
// and cur = 0 before the probes (the WA kernels read gamma from kp[0]).
__global__ void begin_kernel(float* kp, int* cur, double gamma, double lam) {
    pdl_wait();
    kp[0] = __double2float_rn(gamma);
    kp[1] = kp[2] = __double2float_rn(lam);
    kp[3] = kp[4] = 0.f;
    *cur = 0;
}

// *out = sqrt(*a) / sqrt(*b) in float64: the step length of a probe (src/nesterov_optimizer.py:56-63 and :15-32,
// estimate_initial_learning_rate and NesterovOptimizer.__init__), correctly rounded operations.
__global__ void sqrt_ratio_kernel(const double* a, const double* b, double* out) {
    pdl_wait();
    *out = __ddiv_rn(__dsqrt_rn(*a), __dsqrt_rn(*b));
}

__global__ void copy_kernel(const float* src, float* dst, int n) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

// The first phase's state after the probes, alpha = *alpha_p. A fresh run (lam <= 0): T of the wirelength-only start
// (alpha, a = 1, the start rule's tolerance and pass limit, the iteration counts; the rest 0) and kp = (gamma, 0, 0,
// alpha, 0). Resumed with the density term on (lam > 0): S of the density phase (lam, gamma, alpha, a = 1, iteration,
// last HPWL, mu 1, best HPWL and overflow +inf, loop count; the rest 0), kp = (gamma, lam, lam, alpha, 0) (the
// Nesterov coefficient of a = 1) and best = v.
__global__ void first_state_kernel(double* T, double* S, float* kp, float* best, const float* v, int n,
                                   const double* alpha_p, double gamma, double lam, double start_tol, double inner,
                                   double iter, double loop_it, double hpwl_prev) {
    pdl_wait();
    const double alpha = *alpha_p;
    const bool resumed = lam > 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (!resumed) {
            for (int i = 0; i < GP103_T_SIZE; i++) T[i] = 0.0;
            T[GP103_T_ALPHA] = alpha;
            T[GP103_T_A] = 1.0;
            T[GP103_T_START_TOL] = start_tol;
            T[GP103_T_INNER] = inner;
            T[GP103_T_ITER] = iter;
            T[GP103_T_LOOP_IT] = loop_it;
        } else {
            for (int i = 0; i < S_SIZE; i++) S[i] = 0.0;
            S[S_LAM] = lam;
            S[S_GAM] = gamma;
            S[S_ALPHA] = alpha;
            S[S_A] = 1.0;
            S[S_ITER] = iter;
            S[S_HPWL_PREV] = hpwl_prev;
            S[S_MU] = 1.0;
            S[S_BEST_HPWL] = S[S_BEST_OVF] = __longlong_as_double(0x7ff0000000000000LL);     // +inf
            S[S_LOOP_IT] = loop_it;
        }
        kp[0] = __double2float_rn(gamma);
        kp[1] = kp[2] = resumed ? __double2float_rn(lam) : 0.f;
        kp[3] = __double2float_rn(alpha);
        kp[4] = 0.f;
    }
    if (resumed)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) best[i] = v[i];
}

int launch_begin(float* kp, int* cur, double gamma, double lam, cudaStream_t s) {
    if (launch_k(begin_kernel, dim3(1), dim3(1), 0, s, kp, cur, gamma, lam) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

int launch_sqrt_ratio(const double* a, const double* b, double* out, cudaStream_t s) {
    if (launch_k(sqrt_ratio_kernel, dim3(1), dim3(1), 0, s, a, b, out) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

int launch_copy(const float* src, float* dst, int n, cudaStream_t s) {
    if (n == 0) return GP103_OK;
    if (launch_k(copy_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, src, dst, n) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

int launch_first_state(double* T, double* S, float* kp, float* best, const float* v, int n, const double* alpha_p,
                       double gamma, double lam, double start_tol, double inner, double iter, double loop_it,
                       double hpwl_prev, cudaStream_t s) {
    if (launch_k(first_state_kernel, dim3(grid_for(n > 0 ? n : 1, 256, 8)), dim3(256), 0, s, T, S, kp, best, v, n,
                 alpha_p, gamma, lam, start_tol, inner, iter, loop_it, hpwl_prev) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// The hand-over from the wirelength-only start to the density phase, on the device (src/run_placement.py:60-64 and
// the state set-up of src/gpu_loop.py:38-48). l1 = the L1 norm over the cells of the plain density gradient at v[cur];
// the density weight is density_weight x (total_pins / l1), the tension unit; S is the density phase's state
// (iteration, last HPWL, step length alpha and momentum a carried over from T), kp its float32 parameters with the
// Nesterov coefficient (a - 1) / ((1 + sqrt(4 a^2 + 1)) / 2), and best = v[cur]. Every float64 operation is a
// rounded IEEE operation in the order of the host's statement of the same rule, so the state is the same bits. When
// the start itself stopped the run (T[stop] != 0), only S[stop] is set: the density passes then do nothing.
__global__ void handover_kernel(const double* T, double* S, float* kp, const int* cur, const float* v0,
                                const float* v1, float* best, const double* l1, double total_pins,
                                double density_weight, double gamma, int n) {
    pdl_wait();
    const double stop = T[GP103_T_STOP];
    if (stop != 0.0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) S[S_STOP] = stop;
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double lam = __dmul_rn(density_weight, __ddiv_rn(total_pins, *l1));
        const double alpha = T[GP103_T_ALPHA], a = T[GP103_T_A];
        const double a_next = __ddiv_rn(__dadd_rn(1.0, __dsqrt_rn(__dadd_rn(__dmul_rn(__dmul_rn(4.0, a), a), 1.0))), 2.0);
        for (int i = 0; i < S_SIZE; i++) S[i] = 0.0;
        S[S_LAM] = lam;
        S[S_GAM] = gamma;
        S[S_ALPHA] = alpha;
        S[S_A] = a;
        S[S_ITER] = T[GP103_T_ITER];
        S[S_HPWL_PREV] = T[GP103_T_HPWL];
        S[S_MU] = 1.0;
        S[S_BEST_HPWL] = S[S_BEST_OVF] = __longlong_as_double(0x7ff0000000000000LL);     // +inf
        S[S_LOOP_IT] = T[GP103_T_LOOP_IT];
        kp[0] = __double2float_rn(gamma);
        kp[1] = kp[2] = __double2float_rn(lam);
        kp[3] = __double2float_rn(alpha);
        kp[4] = __double2float_rn(__ddiv_rn(__dsub_rn(a, 1.0), a_next));
    }
    const float* v = *cur ? v1 : v0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) best[i] = v[i];
}

int launch_handover(const double* T, double* S, float* kp, const int* cur, const float* v0, const float* v1,
                    float* best, const double* l1, double total_pins, double density_weight, double gamma, int n,
                    cudaStream_t s) {
    if (launch_k(handover_kernel, dim3(grid_for(n > 0 ? n : 1, 256, 8)), dim3(256), 0, s, T, S, kp, cur, v0, v1,
                 best, l1, total_pins, density_weight, gamma, n) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// out[i] = value k[i] of reduction r[i] (i < n <= 8): the scalars of an evaluation, for the host.
struct Totals {
    Reduce r[8];
    int k[8];
    double mul[8];
    int n;
};

__global__ void __launch_bounds__(256) totals_kernel(Totals t, double* out) {
    pdl_wait();
    for (int i = 0; i < t.n; i++) {
        const double v = block_total(t.r[i], t.k[i]);
        if (threadIdx.x == 0) out[i] = v * t.mul[i];
    }
}

int launch_totals(const Reduce* r, const int* k, int n, double* out, cudaStream_t s) {
    Totals t = {};
    for (int i = 0; i < n && i < 8; i++) {
        t.r[i] = r[i];
        t.k[i] = k[i];
        t.mul[i] = 1.0;
    }
    t.n = n < 8 ? n : 8;
    if (launch_k(totals_kernel, dim3(1), dim3(256), 0, s, t, out) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

int launch_scale_total(const Reduce& r, double mul, double* out, cudaStream_t s) {
    Totals t = {};
    t.r[0] = r;
    t.mul[0] = mul;
    t.n = 1;
    if (launch_k(totals_kernel, dim3(1), dim3(256), 0, s, t, out) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

}  // namespace gp103
