// gp103_density_map_noalloc: the density map of gp103_density_map for callers that cannot allocate device memory.
//
// Some callers may not call cudaMalloc (or any allocating routine): a plugin that runs inside a host application
// whose device memory is owned by that application's own pool allocator, or a latency-critical loop that must not
// call cudaMalloc because it can synchronise the device. They can still pass their inputs and outputs, but not the
// 64-bit scratch map the density kernels accumulate into. This entry point keeps that scratch in a file-scope
// device array of fixed size instead, so it allocates nothing.
//
// Limits and behaviour:
//   * at most NOALLOC_MAX_BINS bins per map (nbx * nby <= 262,144, e.g. 512 x 512): the array is
//     2 x 262,144 x 8 bytes = 4 MiB, held on every GPU that loads the library until the process exits;
//     larger grids are rejected with GP103_ERR_TOO_LARGE before any work;
//   * the array's device address is looked up once per device (cudaGetSymbolAddress, with that device current) by
//     the first call on that device; make that first call before any stream capture. The address is kept for the
//     life of the process: after a cudaDeviceReset of a device it is stale (the reset destroys the context it
//     belongs to), so do not call this entry point on that device again in the same process;
//   * `stream` must belong to the current device (checked: GP103_ERR_ARG otherwise), whose array the call uses;
//   * every call shares the one array and leaves its contents behind: each call clears the part it uses before
//     adding to it, and calls whose work overlaps on the GPU (other streams, other host threads) race on it.
#include <mutex>

#include "gp103.cuh"
#include "kernels.cuh"

namespace {

constexpr int NOALLOC_MAX_BINS = 512 * 512;
constexpr int NOALLOC_MAX_DEVICES = 64;

// The scratch map [2][NOALLOC_MAX_BINS] (map 0: movable nodes, map 1: the rest). In host code this name is only a
// stand-in for the symbol: kernels get the device address looked up below.
static __device__ __align__(256) unsigned long long g_noalloc_map[2 * NOALLOC_MAX_BINS];

std::mutex g_noalloc_mu;
unsigned long long* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch map on the current device (looked up on the first call per device).
int noalloc_map(unsigned long long** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return GP103_ERR_CUDA;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return GP103_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_map) != cudaSuccess || p == nullptr) return GP103_ERR_CUDA;
        g_noalloc_ptr[dev] = (unsigned long long*)p;
    }
    *out = g_noalloc_ptr[dev];
    return GP103_OK;
}

}  // namespace

using namespace gp103;

extern "C" int gp103_density_map_noalloc(const float* pos, const float* size, const float* ratio, int num_nodes,
                                         int num_mov, float bx, float by, int nbx, int nby, const float* fixed,
                                         float target, float* rho, float* over, cudaStream_t stream) {
    if (!(num_nodes >= 0 && num_mov >= 0 && nbx > 0 && nby > 0 && fixed && rho && over)) return GP103_ERR_ARG;
    if (num_nodes > 0 && !(pos && size && ratio)) return GP103_ERR_ARG;
    if (!(bx > 0.f && by > 0.f)) return GP103_ERR_ARG;
    if ((long long)nbx * nby > NOALLOC_MAX_BINS) return GP103_ERR_TOO_LARGE;
    int cur = -1, sdev = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cudaStreamGetDevice(stream, &sdev) != cudaSuccess) return GP103_ERR_CUDA;
    if (sdev != cur) return GP103_ERR_ARG;                    // the array of another device than the stream's
    unsigned long long* map = nullptr;
    int st = noalloc_map(&map);
    if (st) return st;
    const size_t nb = (size_t)nbx * nby;
    // the map must start at zero: clear the two planes this grid uses (the array keeps the last call's sums)
    if (cudaMemsetAsync(map, 0, sizeof(unsigned long long) * 2 * nb, stream) != cudaSuccess) return GP103_ERR_CUDA;
    ScatterJob j = {};
    j.pos_a = j.pos_b = (const float2*)pos;
    j.size = (const float2*)size;
    j.ratio = ratio;
    j.num_nodes = num_nodes;
    j.num_mov = num_mov < num_nodes ? num_mov : num_nodes;
    j.inv_bx = 1.f / bx;
    j.inv_by = 1.f / by;
    j.nbx = nbx;
    j.nby = nby;
    j.map0 = map;
    j.map1 = map + nb;
    st = launch_scatter(&j, 1, stream);
    if (st) return st;
    return launch_post_mirror(map, fixed, target, nbx, nby, rho, over, stream);
}
