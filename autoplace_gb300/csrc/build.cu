// Device build of the WA kernels' net order (the per-run set-up of the fused path, GB300 sm_103a).
//
// Input: the optimised pin set as AutoPlace builds it (Wirelength._pin_set, src/core/wa_wirelength_hpwl.py:38-46):
// pins grouped by net (net_start, cell per pin with num_mov for a fixed pin, offsets) and the pins in cell order
// (cell_pin). Output: the same nets reordered for the WA kernels (short nets by class of degree 2 / 3 / 4-8, each
// class by the net's lowest cell, then the nets of 9-16 pins and the longer ones, likewise), their pins moved with them, and for every pin its position
// in cell order (pin_slot), where the WA kernels write its gradient. The order is exactly a stable sort of the nets
// by (class, lowest cell): a counting sort over the keys, ties put back in net order, so the result is the same
// on every run.
#include "gp103.cuh"
#include "kernels.cuh"

namespace gp103 {

constexpr int NO_SHORT = 8;               // nets of up to 8 pins are short (one thread each in the WA kernels)
constexpr int NO_MID = 16;                // nets of 9 .. 16 pins: 4 lanes each
constexpr int NO_G8 = 32;                 // 17 .. 32 pins: 8 lanes each
constexpr int NO_G16 = 64;                // 33 .. 64 pins: 16 lanes each; longer: a warp each
constexpr int NO_CLASSES = 7;
// SCAN_TILE, SCAN_MAX_TILES: kernels.cuh

__device__ __forceinline__ int net_class(int deg) {
    return deg == 2 ? 0 : deg == 3 ? 1 : deg <= NO_SHORT ? 2 : deg <= NO_MID ? 3 : deg <= NO_G8 ? 4 :
           deg <= NO_G16 ? 5 : 6;
}

// key of a net = class * (num_mov + 1) + lowest cell (a cell index in [0, num_mov]); count per key
__global__ void __launch_bounds__(256) net_key_kernel(const int* ns, const int* cell, int num_nets, int num_mov,
                                                      int* key, int* count) {
    pdl_wait();
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < num_nets; n += gridDim.x * blockDim.x) {
        const int b = ns[n], e = ns[n + 1];
        int first = INT_MAX;
        for (int p = b; p < e; p++) first = min(first, cell[p]);
        first = e > b ? min(max(first, 0), num_mov) : 0;
        const int k = net_class(e - b) * (num_mov + 1) + first;
        key[n] = k;
        atomicAdd(&count[k], 1);
    }
}

// ---- exclusive scan of int32 (three launches: tile sums, one-block scan of the sums, tiles with their offsets)
__device__ __forceinline__ int block_exclusive(int v, int* sh, int& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        const int s = lane < nw ? sh[lane] : 0;
        int z = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, z, o);
            if (lane >= o) z += y;
        }
        sh[lane] = z - s;
        if (lane == 31) sh[32] = z;
    }
    __syncthreads();
    total = sh[32];
    const int r = x - v + sh[w];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(256) scan_tiles_kernel(const int* in, int n, int* tile_sum) {
    pdl_wait();
    __shared__ int sh[33];
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * 16;
    int s = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) s += base + k < n ? in[base + k] : 0;
    int total;
    block_exclusive(s, sh, total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) scan_top_kernel(int* tile_sum, int tiles, int* total_out) {
    pdl_wait();
    __shared__ int sh[33];
    int v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int t = threadIdx.x * 4 + k;
        v[k] = t < tiles ? tile_sum[t] : 0;
        s += v[k];
    }
    int total;
    int run = block_exclusive(s, sh, total);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int t = threadIdx.x * 4 + k;
        if (t < tiles) tile_sum[t] = run;
        run += v[k];
    }
    if (threadIdx.x == 0 && total_out) *total_out = total;
}

__global__ void __launch_bounds__(256) scan_apply_kernel(const int* in, int n, const int* tile_off, int* out) {
    pdl_wait();
    __shared__ int sh[33];
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * 16;
    int v[16], s = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    int total;
    int run = block_exclusive(s, sh, total) + tile_off[blockIdx.x];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

// out[i] = sum of in[0..i) for i < n, *total = the sum of all (out may alias in); tile_sum: SCAN_MAX_TILES ints
int exclusive_scan(const int* in, int n, int* out, int* tile_sum, int* total, cudaStream_t s) {
    const int tiles = ceil_div(n, SCAN_TILE);
    if (tiles > SCAN_MAX_TILES) return GP103_ERR_TOO_LARGE;
    if (tiles == 0) return cudaMemsetAsync(total, 0, sizeof(int), s) == cudaSuccess ? GP103_OK : GP103_ERR_CUDA;
    if (launch_k(scan_tiles_kernel, dim3(tiles), dim3(256), 0, s, in, n, tile_sum) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (launch_k(scan_top_kernel, dim3(1), dim3(1024), 0, s, tile_sum, tiles, total) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (launch_k(scan_apply_kernel, dim3(tiles), dim3(256), 0, s, in, n, (const int*)tile_sum, out) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// every net takes a slot of its key (any order inside a key, fixed below)
__global__ void __launch_bounds__(256) net_place_kernel(const int* key, int num_nets, int* cursor, int* order) {
    pdl_wait();
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < num_nets; n += gridDim.x * blockDim.x)
        order[atomicAdd(&cursor[key[n]], 1)] = n;
}

// the nets of one key back in net order (insertion sort of the key's few slots); start = exclusive scan of counts
__global__ void __launch_bounds__(256) net_ties_kernel(const int* start, const int* count, int keys, int* order) {
    pdl_wait();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < keys; k += gridDim.x * blockDim.x) {
        const int c = count[k];
        if (c < 2) continue;
        int* o = order + start[k];
        for (int i = 1; i < c; i++) {
            const int v = o[i];
            int j = i - 1;
            while (j >= 0 && o[j] > v) {
                o[j + 1] = o[j];
                j--;
            }
            o[j + 1] = v;
        }
    }
}

__global__ void __launch_bounds__(256) net_degree_kernel(const int* ns, const int* order, int num_nets, int* deg) {
    pdl_wait();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < num_nets; r += gridDim.x * blockDim.x) {
        const int o = order[r];
        deg[r] = ns[o + 1] - ns[o];
    }
}

// pins of new net r = old net order[r], in their old order; newpos[old pin] = new position
__global__ void __launch_bounds__(256) net_pins_kernel(const int* ns, const int* order, const int* ns_out,
                                                       const int* cell, const float2* off, int num_nets,
                                                       int* cell_out, float2* off_out, int* newpos) {
    pdl_wait();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < num_nets; r += gridDim.x * blockDim.x) {
        const int o = order[r], b = ns[o], d = ns[o + 1] - b, q0 = ns_out[r];
        for (int j = 0; j < d; j++) {
            cell_out[q0 + j] = cell[b + j];
            off_out[q0 + j] = off[b + j];
            newpos[b + j] = q0 + j;
        }
    }
}

__global__ void __launch_bounds__(256) pin_slot_kernel(const int* cell_pin, const int* newpos, int num_pins,
                                                       int* slot) {
    pdl_wait();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < num_pins; k += gridDim.x * blockDim.x)
        slot[newpos[cell_pin[k]]] = k;
}

// split[0] = nets of up to 8 pins = start of the keys of class 3, split[1] = nets of up to 16 pins (class 4),
// split[2] = nets of 2 pins (class 0), split[3] = nets of up to 3 pins (class 1), split[4] = nets of up to 32 pins
// (class 5), split[5] = nets of up to 64 pins (class 6)
__global__ void net_split_kernel(const int* start, int stride, int num_nets, int keys, int* split) {
    pdl_wait();
    const int cls[6] = {3, 4, 1, 2, 5, 6};
    for (int c = 0; c < 6; c++) {
        const int k = cls[c] * stride;
        split[c] = k < keys ? start[k] : num_nets;
    }
}

struct NetOrderScratch {
    size_t key, count, start, cursor, order, deg, newpos, tile, total, bytes;
};

static NetOrderScratch net_order_scratch(long long num_nets, long long num_pins, long long num_mov) {
    NetOrderScratch s = {};
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t keys = (size_t)NO_CLASSES * (size_t)(num_mov + 1);
    size_t at = 0;
    s.key = at; at += al(sizeof(int) * (size_t)num_nets);
    s.count = at; at += al(sizeof(int) * keys);
    s.start = at; at += al(sizeof(int) * keys);
    s.cursor = at; at += al(sizeof(int) * keys);
    s.order = at; at += al(sizeof(int) * (size_t)num_nets);
    s.deg = at; at += al(sizeof(int) * (size_t)(num_nets + 1));
    s.newpos = at; at += al(sizeof(int) * (size_t)num_pins);
    s.tile = at; at += al(sizeof(int) * SCAN_MAX_TILES);
    s.total = at; at += al(sizeof(int) * 4);
    s.bytes = at;
    return s;
}

}  // namespace gp103

using namespace gp103;

extern "C" size_t gp103_net_order_scratch(int num_nets, int num_pins, int num_mov) {
    if (num_nets < 0 || num_pins < 0 || num_mov < 0) return 0;
    return net_order_scratch(num_nets, num_pins, num_mov).bytes;
}

extern "C" int gp103_net_order(const int* net_start, const int* pin_cell, const float* pin_off, const int* cell_pin,
                               int num_nets, int num_pins, int num_mov, void* scratch, size_t scratch_bytes,
                               int* net_start_out, int* pin_cell_out, float* pin_off_out, int* pin_slot,
                               int* split, cudaStream_t s) {
    if (num_nets < 0 || num_pins < 0 || num_mov < 0 || !net_start || !scratch || !net_start_out || !split)
        return GP103_ERR_ARG;
    if (num_pins > 0 && (!pin_cell || !pin_off || !cell_pin || !pin_cell_out || !pin_off_out || !pin_slot))
        return GP103_ERR_ARG;
    const long long keys = (long long)NO_CLASSES * ((long long)num_mov + 1);
    if (keys > (long long)SCAN_TILE * SCAN_MAX_TILES || num_nets + 1LL > (long long)SCAN_TILE * SCAN_MAX_TILES)
        return GP103_ERR_TOO_LARGE;
    const NetOrderScratch L = net_order_scratch(num_nets, num_pins, num_mov);
    if (scratch_bytes < L.bytes) return GP103_ERR_ARG;
    char* w = (char*)scratch;
    int *key = (int*)(w + L.key), *count = (int*)(w + L.count), *start = (int*)(w + L.start);
    int *order = (int*)(w + L.order), *deg = (int*)(w + L.deg), *newpos = (int*)(w + L.newpos);
    int *tile = (int*)(w + L.tile), *total = (int*)(w + L.total), *cursor = (int*)(w + L.cursor);
    const int K = (int)keys;
    if (cudaMemsetAsync(count, 0, sizeof(int) * (size_t)K, s) != cudaSuccess) return GP103_ERR_CUDA;
    const int gn = grid_for(num_nets > 0 ? num_nets : 1, 256, 8), gk = grid_for(K, 256, 8);
    const int gp = grid_for(num_pins > 0 ? num_pins : 1, 256, 8);
    if (num_nets > 0) {
        if (launch_k(net_key_kernel, dim3(gn), dim3(256), 0, s, net_start, pin_cell, num_nets, num_mov, key, count) !=
            cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    int st = exclusive_scan(count, K, start, tile, total, s);
    if (st) return st;
    if (cudaMemcpyAsync(cursor, start, sizeof(int) * (size_t)K, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return GP103_ERR_CUDA;
    if (num_nets > 0) {
        if (launch_k(net_place_kernel, dim3(gn), dim3(256), 0, s, (const int*)key, num_nets, cursor, order) !=
            cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
        if (launch_k(net_ties_kernel, dim3(gk), dim3(256), 0, s, (const int*)start, (const int*)count, K, order) !=
            cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
        if (launch_k(net_degree_kernel, dim3(gn), dim3(256), 0, s, net_start, (const int*)order, num_nets, deg) !=
            cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    if (cudaMemsetAsync(deg + num_nets, 0, sizeof(int), s) != cudaSuccess) return GP103_ERR_CUDA;
    if ((st = exclusive_scan(deg, num_nets + 1, net_start_out, tile, total + 1, s))) return st;
    if (num_nets > 0 && num_pins > 0) {
        if (launch_k(net_pins_kernel, dim3(gn), dim3(256), 0, s, net_start, (const int*)order,
                     (const int*)net_start_out, pin_cell, (const float2*)pin_off, num_nets, pin_cell_out,
                     (float2*)pin_off_out, newpos) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
        if (launch_k(pin_slot_kernel, dim3(gp), dim3(256), 0, s, cell_pin, (const int*)newpos, num_pins, pin_slot) !=
            cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    if (launch_k(net_split_kernel, dim3(1), dim3(1), 0, s, (const int*)start, num_mov + 1, num_nets, K,
                 split) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}
