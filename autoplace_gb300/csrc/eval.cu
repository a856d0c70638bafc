// Exact evaluators of a placement in float64: the HPWL over every net and the overflow of the movable cells with
// their real sizes. They judge a run (final HPWL, overflow <= the stop value) and run once per level.
//
// Reference: Wirelength.hpwl (src/core/wa_wirelength_hpwl.py:66-70) and ElectronicDensityLayer.exact_overflow
// (src/core/electronic_density_layer.py:112-116), both float32 there.
#include "gp103.cuh"
#include "kernels.cuh"
#include "step.cuh"

using namespace gp103;

#define REQUIRE(cond)                      \
    do {                                   \
        if (!(cond)) return GP103_ERR_ARG; \
    } while (0)
#define TRY(call)                          \
    do {                                   \
        int st_ = (call);                  \
        if (st_) return st_;               \
    } while (0)

namespace {

// The reduction scratch of an evaluator: MAX_BLOCKS float64 partials, then the partial count.
Reduce scratch_reduce(void* scratch) {
    Reduce r;
    r.partials = (double*)scratch;
    r.count = (int*)((char*)scratch + sizeof(double) * MAX_BLOCKS);
    return r;
}

// One thread per net: pin position = pos[cell] + offset in float64 (a cell >= num_mov is a fixed pin: the offset
// alone), hi - lo on each axis; float64 block partials in block order.
__global__ void __launch_bounds__(256) hpwl_kernel(const float2* pos, const int* pin_cell, const float2* pin_off,
                                                   const int* net_start, int num_nets, int num_mov, Reduce red) {
    pdl_wait();
    double acc = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < num_nets; n += gridDim.x * blockDim.x) {
        const int b = net_start[n], e = net_start[n + 1];
        if (e <= b) continue;
        double xl = INFINITY, xh = -INFINITY, yl = INFINITY, yh = -INFINITY;
        for (int p = b; p < e; p++) {
            const int c = pin_cell[p];
            const float2 o = pin_off[p];
            double x = (double)o.x, y = (double)o.y;
            if ((unsigned)c < (unsigned)num_mov) {
                const float2 q = pos[c];
                x += (double)q.x;
                y += (double)q.y;
            }
            xl = fmin(xl, x); xh = fmax(xh, x);
            yl = fmin(yl, y); yh = fmax(yh, y);
        }
        acc += (xh - xl) + (yh - yl);
    }
    double v[1] = {acc};
    grid_sum<1>(v, red);
}

}  // namespace

extern "C" int gp103_hpwl(const float* pos, const int* pin_cell, const float* pin_off, const int* net_start,
                          int num_nets, int num_mov, void* scratch, double* out, cudaStream_t s) {
    REQUIRE(num_nets >= 0 && num_mov >= 0 && net_start && scratch && out);
    REQUIRE(num_nets == 0 || (pin_cell && pin_off && (pos || num_mov == 0)));
    const Reduce r = scratch_reduce(scratch);
    const int blocks = num_nets > 0 ? grid_for(num_nets, 256, 8) : 1;
    if (launch_k(hpwl_kernel, dim3(blocks), dim3(256), 0, s, (const float2*)pos, pin_cell,
                 (const float2*)pin_off, net_start, num_nets, num_mov, r) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    const int k0 = 0;
    return launch_totals(&r, &k0, 1, out, s);
}

extern "C" int gp103_exact_overflow(const float* pos, const float* size, int num_mov, float bx, float by, int nbx,
                                    int nby, const float* fixed, float target, double area_scale,
                                    unsigned long long* map, void* scratch, double* out, cudaStream_t stream) {
    REQUIRE(num_mov >= 0 && nbx > 0 && nby > 0 && bx > 0.f && by > 0.f);
    REQUIRE(fixed && map && scratch && out && (num_mov == 0 || (pos && size)));
    const Reduce r = scratch_reduce(scratch);
    if (num_mov > 0) {
        ScatterJob sj = {};
        sj.pos_a = sj.pos_b = (const float2*)pos;
        sj.size = (const float2*)size;
        sj.ratio = nullptr;                      // real sizes: every charge at full weight
        sj.num_nodes = sj.num_mov = num_mov;
        sj.inv_bx = 1.f / bx;
        sj.inv_by = 1.f / by;
        sj.nbx = nbx;
        sj.nby = nby;
        sj.map0 = map;
        TRY(launch_scatter(&sj, 1, stream));
    }
    PostJob pj = {};
    pj.map = map;
    pj.fixed = fixed;
    pj.target = target;
    pj.nbx = nbx;
    pj.nby = nby;
    pj.exact = 1;
    pj.red = r;
    TRY(launch_post_plain(&pj, 1, stream));
    TRY(launch_scale_total(r, area_scale, out, stream));
    return GP103_OK;
}
