// Job descriptions and launchers shared by the gp103 translation units.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "gp103.cuh"

namespace gp103 {

// Ping-pong selection: with sel = the device index of the current buffers, the evaluated point of a pass lives in
// the other buffer: pick(a, b, sel) = *sel ? a : b; pick_ref is the current one. sel == nullptr -> a.
template <typename T>
__device__ __forceinline__ const T* pick(const T* a, const T* b, const int* sel) {
    return sel == nullptr ? a : (*sel ? a : b);
}
template <typename T>
__device__ __forceinline__ T* pick_mut(T* a, T* b, const int* sel) {
    return sel == nullptr ? a : (*sel ? a : b);
}
template <typename T>
__device__ __forceinline__ const T* pick_ref(const T* a, const T* b, const int* sel) {
    return sel == nullptr ? a : (*sel ? b : a);
}

// Reduction slots of a plan's `red` buffer (float64): each has K <= 4 values, MAX_BLOCKS partials per value; the
// partial counts live in the plan's `counters`.
enum { R_WA = 0, R_OVF, R_JOVF, R_MOVED, R_GRAD, R_COUNT };
inline Reduce reduce_slot(double* red, unsigned int* counters, int slot) {
    Reduce r;
    r.partials = red + (size_t)slot * 4 * MAX_BLOCKS;
    r.count = (int*)(counters + slot);
    return r;
}
// behind the partials: totals summed ahead of the control (GatherJob::pre), TOT_* order
enum { TOT_MOVED = 0, TOT_WA, TOT_HPWL, TOT_OVF, TOT_COUNT };
constexpr size_t RED_TOTALS = (size_t)R_COUNT * 4 * MAX_BLOCKS;
constexpr size_t RED_DOUBLES = RED_TOTALS + 8;

struct WaJob {
    const float2* pos_a; const float2* pos_b; const int* sel;
    const int* pin_cell; const float2* pin_off; const int* net_start;
    int num_nets, num_mov;
    int split;              // nets [split, num_nets): one warp each; below: 32 per warp (num_nets: any order)
    int mid;                // nets [split, mid): 9 .. 16 pins, 4 lanes each (mid = split: none)
    int g8, g16;            // nets [mid, g8): 17 .. 32 pins, 8 lanes each; [g8, g16): 33 .. 64 pins, 16 lanes each
                            // (g8 = g16 = mid: none; the rest a warp each)
    int two, three;         // nets [0, two): 2 pins, [two, three): 3 pins, pins from 0 in net order (three = 0: none)
    const int* slot;        // pin p's gradient goes to pin_grad[slot[p]] (null: pin_grad[p])
    const float* gamma;
    float2* pin_grad;
    float2* out;            // per-net (WA, HPWL), may be null
    Reduce red;             // (WA, HPWL) totals; red.partials == nullptr: none
    int long_share;         // percent of the fused launch's blocks on the long nets (0: GP103_OPT_WA_FUSED)
};

struct ScatterJob {
    const float2* pos_a; const float2* pos_b; const int* sel;
    const float2* size; const float* ratio;     // ratio null: 1 for every node
    int num_nodes, num_mov;
    float inv_bx, inv_by;
    int nbx, nby;
    unsigned long long* map0;   // nodes < num_mov
    unsigned long long* map1;   // the rest (null: not added)
    const int* order;           // the nodes in this order (cells first, then fillers); null: index order
};

// Spatial order of the nodes for the scatter: a counting sort of the nodes by the tile (tile x tile bins of the
// force grid) their centre is in, cells before fillers. Blocks of the scatter then take nodes that are close on
// the grid, so their charges meet in shared memory. Any order gives the same map (integer sums); the order only
// decides how many charges reach the global map through atomics.
struct OrderJob {
    int* counts;                // [2 tiles], zero between uses
    int* cursor;                // [2 tiles]
    int* order;                 // [num_nodes]
    int tiles_x, tiles_y;
    float inv_tx, inv_ty;       // 1 / (tile edge in length units)
    int num_nodes, num_mov;
};
constexpr int ORDER_MAX_KEYS = 2048;

// Tiles in column-major order, every other column upwards (a snake), so that consecutive keys are adjacent tiles.
__device__ __forceinline__ int order_key(const OrderJob& o, float2 p, int i) {
    const int tx = min(max((int)(p.x * o.inv_tx), 0), o.tiles_x - 1);
    int ty = min(max((int)(p.y * o.inv_ty), 0), o.tiles_y - 1);
    if (tx & 1) ty = o.tiles_y - 1 - ty;
    return tx * o.tiles_y + ty + (i < o.num_mov ? 0 : o.tiles_x * o.tiles_y);
}

// One launch for up to two scatters (the force grid and the overflow grid read the same positions).
struct ScatterPair {
    ScatterJob j[2];
    int njobs;
    int blocks0;                // blocks of job 0; the rest are job 1's
};

struct PostJob {
    unsigned long long* map;    // [1 or 2][nbx][nby], zeroed behind the read
    const float* fixed;
    float target;
    int nbx, nby;
    int with_fill;              // map has the filler plane
    float* dens;                // plain density, may be null
    __nv_bfloat16 *t0, *t1, *t2;  // bf16 split terms of the density, may be null
    int terms;
    float *tf0, *tf1;           // tf32 split terms of the density (float32 planes), may be null
    signed char* exps;          // non-null: float16 terms (t0, t1 hold __half) of each 64-bin chunk of a row scaled by
                                // 2^e, e = exps[(y / 64) * nbx + x] (nby a multiple of 64)
    int fold;                   // with exps (nby a multiple of 128): the terms of the density folded about the middle
                                // of y (post_fold), for the folded first transform of the field
    int exact;                  // float64 per-thread partials of the sum (evaluators); 0: float32 (hot path)
    Reduce red;                 // sum of the density above the target
    float shift;                // subtracted from the density that goes to the field (dens / terms): the field of a
                                // density and of the density minus a constant are the same (only the zero frequency
                                // changes, and the field drops it); with the mean density, the transforms' rounding
                                // follows the density's variation instead of its mean
};

struct PostPair {
    PostJob j[2];
    int njobs;
    int blocks0;
};

struct GatherJob {
    const float2* pos_a; const float2* pos_b; const int* sel;
    const float2* size; const float* ratio; const float* pins; const float* area;
    int num_nodes, num_mov;
    float inv_bx, inv_by;
    int nbx, nby;
    const float* ex; const float* ey;      // null: no density term (wirelength-only gradient)
    const float* weight_p; const float* precond_p;   // device scalars, or null: the host values below
    float weight, precond;
    int with_wl;
    const float2* pin_grad; const int* cell_start; const int* cell_pin;   // cell_pin null: pin_grad in cell order
    float2* gout_a; float2* gout_b;
    const float2* gref_a; const float2* gref_b;     // null: no distance
    Reduce red;                 // (|g - gref|^2, L1 of g over the cells)
    // npre > 0: block 0 does no gathering: it sums the partials of earlier kernels, pre[i] value pre_k[i], in the
    // order block_total sums them (the order of every consumer), into pre_out[i], while the other blocks gather
    Reduce pre[4];
    int pre_k[4];
    int npre;
    double* pre_out;
};

// Exclusive scan of n ints (build.cu): out[i] = in[0] + ... + in[i - 1], *total = the whole sum (device int);
// tile_sum is SCAN_MAX_TILES ints of scratch; GP103_ERR_TOO_LARGE beyond SCAN_TILE * SCAN_MAX_TILES elements.
constexpr int SCAN_TILE = 4096;           // elements per block of the scans (256 threads x 16)
constexpr int SCAN_MAX_TILES = 4096;      // one block scans the tile sums: scans of up to 16.7M elements
int exclusive_scan(const int* in, int n, int* out, int* tile_sum, int* total, cudaStream_t s);

int launch_wa_net(const WaJob& j, cudaStream_t s);
int launch_wa_cell(const float2* pin_grad, const int* cell_start, const int* cell_pin, int num_mov, float2* grad,
                   cudaStream_t s);
int launch_scatter(const ScatterJob* jobs, int njobs, cudaStream_t s);
int launch_post_mirror(const unsigned long long* map, const float* fixed, float target, int nbx, int nby, float* rho,
                       float* over, cudaStream_t s);
int launch_post_plain(const PostJob* jobs, int njobs, cudaStream_t s);
int launch_gather_mirror(const float* pos, const float* size, const float* ratio, const float* field,
                         const float* wl_grad, const float* pins, const float* area, int num_nodes, int num_wl,
                         const float* weight, const float* precond, float bx, float by, int nbx, int nby, float* grad,
                         cudaStream_t s);
int launch_gather(const GatherJob& j, cudaStream_t s);
int launch_order(const OrderJob& o, const float2* pos_a, const float2* pos_b, const int* sel, bool counted,
                 cudaStream_t s);

}  // namespace gp103
