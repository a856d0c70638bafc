// Device build of a placement problem's per-pin and per-node arrays (GB300, sm_103a): what AutoPlace builds once
// per level with torch operations on the GPU before the first iteration.
//
// gp103_build_csr: the optimised pin set (Wirelength.__init__ net filter, src/core/wa_wirelength_hpwl.py:26-32, and
// Wirelength._pin_set, :38-46): nets of 2 .. ignore_degree pins renumbered in order, their pins in net order
// (net_start), the pins in cell order (cell_pin = a stable argsort of the pins' cells, cell_start), and the start of
// every net of the whole netlist (the exact HPWL's, :66-70). Every output is integer work or a copy, fixed by the
// input alone: the host build's arrays, bit for bit. Stability of the cell order: the pins of a cell are placed by
// atomics, then put back in pin order (an insertion sort per cell of up to 32 pins, a rank count by one block in
// shared memory up to 12,288 pins, an error beyond); the fixed pins (cell index num_mov) take their rank from a scan.
//
// gp103_smooth_nodes: the nodes as a density grid sees them (ElectronicDensityLayer.__init__,
// src/core/electronic_density_layer.py:36-58): smoothed size max(size, sqrt(2) bin) and density ratio real area /
// smoothed area in float64, rounded once to float32, the position bounds, and the preconditioner's area and pins.
#include "gp103.cuh"
#include "kernels.cuh"

namespace gp103 {

namespace {

constexpr int CSR_SMALL = 32;     // cells of up to this many pins are put back in order by one thread
constexpr int CSR_BIG = 12288;    // beyond: by one block, the cell's slots in shared memory (48 KB); more: an error

// the pins checked (pin_net ascending in [0, num_nets): bad |= 1; a cell in [0, num_mov]: bad |= 2) and counted per
// movable cell over every pin; count[3] += pins on movable cells
__global__ void __launch_bounds__(256) pin_check_kernel(const int* pin_net, const int* pin_cell, int P, int num_nets,
                                                        int num_mov, int* cell_pins, int* count) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        const int cur = pin_net[i];
        if (cur < 0 || cur >= num_nets || (i > 0 && pin_net[i - 1] > cur)) atomicOr(&count[2], 1);
        const int c = pin_cell[i];
        const bool mov = c >= 0 && c < num_mov;
        if (mov) atomicAdd(&cell_pins[c], 1);
        else if (c != num_mov) atomicOr(&count[2], 2);
        const unsigned b = __ballot_sync(__activemask(), mov);
        if (b && (threadIdx.x & 31) == __ffs(b) - 1) atomicAdd(&count[3], __popc(b));
    }
}

// all_start[k] = first pin of net k (searchsorted left over the sorted pin_net), k in [0, num_nets]: pin i starts the
// nets after its predecessor's up to its own. Nothing is written when the check failed (all_start stays zero: what
// follows stays in bounds, and the host raises).
__global__ void __launch_bounds__(256) net_bounds_kernel(const int* pin_net, int P, int num_nets, const int* count,
                                                         int* all_start) {
    pdl_wait();
    if (count[2] & 1) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= P; i += gridDim.x * blockDim.x) {
        const int prev = i == 0 ? -1 : pin_net[i - 1];
        const int cur = i == P ? num_nets : pin_net[i];
        for (int k = prev + 1; k <= cur; k++) all_start[k] = i;
    }
}

// keep[k] = net k is optimised (2 <= degree <= ignore_degree), kdeg[k] = its degree if kept, else 0
__global__ void __launch_bounds__(256) net_keep_kernel(const int* all_start, int num_nets, int ignore_degree,
                                                       int* keep, int* kdeg) {
    pdl_wait();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < num_nets; k += gridDim.x * blockDim.x) {
        const int d = all_start[k + 1] - all_start[k];
        const bool use = d >= 2 && d <= ignore_degree;
        keep[k] = use;
        kdeg[k] = use ? d : 0;
    }
}

// net_start[new id of k] = first optimised pin of k; net_start[num_opt] = the optimised pins (k == num_nets)
__global__ void __launch_bounds__(256) net_emit_kernel(const int* keep, const int* new_id, const int* ostart,
                                                       const int* totals, int num_nets, int* net_start) {
    pdl_wait();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= num_nets; k += gridDim.x * blockDim.x) {
        if (k == num_nets) net_start[totals[0]] = totals[1];
        else if (keep[k]) net_start[new_id[k]] = ostart[k];
    }
}

// the optimised pins in net order (cell, offset) and their count per cell (index num_mov: the fixed pins)
__global__ void __launch_bounds__(256) pin_copy_kernel(const int* pin_net, const int* pin_cell, const float2* pin_off,
                                                       int P, int num_nets, int num_mov, const int* all_start,
                                                       const int* kdeg, const int* ostart, int* cell32, float2* off,
                                                       int* ccount) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        const int k = pin_net[i];
        if (k < 0 || k >= num_nets) continue;
        const int d = kdeg[k], j = i - all_start[k];
        if (j < 0 || j >= d) continue;
        const int q = ostart[k] + j, c = pin_cell[i];
        if (q >= P) continue;                  // (only with an unsorted pin_net, which the host rejects)
        cell32[q] = c;
        off[q] = pin_off[i];
        if (c >= 0 && c <= num_mov) atomicAdd(&ccount[c], 1);
    }
}

// every optimised pin of a movable cell takes a slot of its cell (any order, fixed below); fixed[q] = pin q is fixed
__global__ void __launch_bounds__(256) cell_place_kernel(const int* cell32, const int* totals, int P, int num_mov,
                                                         int* cursor, int* cell_pin, int* fixed) {
    pdl_wait();
    const int n = min(totals[1], P);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int c = cell32[q];
        fixed[q] = c == num_mov;
        if (c >= 0 && c < num_mov) {
            const int t = atomicAdd(&cursor[c], 1);
            if (t < P) cell_pin[t] = q;
        }
    }
}

// the fixed pins after the movable ones, in pin order (rank = exclusive scan of `fixed`)
__global__ void __launch_bounds__(256) fixed_place_kernel(const int* fixed, const int* rank, const int* totals, int P,
                                                          const int* cell_start, int num_mov, int* cell_pin) {
    pdl_wait();
    const int n = min(totals[1], P), base = cell_start[num_mov];
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int t = base + rank[q];
        if (fixed[q] && t < P) cell_pin[t] = q;
    }
}

// the pins of a cell back in pin order: insertion sort up to CSR_SMALL pins, longer cells listed for a block each
// (bad |= 4 for a cell beyond CSR_BIG pins, left unsorted: the host raises)
__global__ void __launch_bounds__(256) cell_ties_kernel(const int* cell_start, int num_mov, int* cell_pin, int* big,
                                                        int* nbig, int* bad) {
    pdl_wait();
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < num_mov; c += gridDim.x * blockDim.x) {
        const int b = cell_start[c], n = cell_start[c + 1] - b;
        if (n < 2) continue;
        if (n > CSR_SMALL) {
            if (n > CSR_BIG) atomicOr(bad, 4);
            else big[atomicAdd(nbig, 1)] = c;
            continue;
        }
        int* o = cell_pin + b;
        for (int i = 1; i < n; i++) {
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

// a cell of many pins (one block): its slots copied to shared memory, each pin's place = the number of the cell's
// pins of a lower index (the pins of a cell are distinct)
__global__ void __launch_bounds__(256) cell_ties_big_kernel(const int* big, const int* nbig, const int* cell_start,
                                                            int* cell_pin) {
    pdl_wait();
    __shared__ int seg[CSR_BIG];
    const int nb = *nbig;
    for (int w = blockIdx.x; w < nb; w += gridDim.x) {
        const int c = big[w], b = cell_start[c], n = min(cell_start[c + 1] - b, CSR_BIG);
        for (int i = threadIdx.x; i < n; i += blockDim.x) seg[i] = cell_pin[b + i];
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int v = seg[i];
            int r = 0;
            for (int k = 0; k < n; k++) r += seg[k] < v;
            cell_pin[b + r] = v;
        }
        __syncthreads();
    }
}

struct CsrScratch {
    size_t keep, kdeg, new_id, ostart, ccount, cursor, fixed, rank, big, tile, totals, bytes;
};

CsrScratch csr_scratch(long long P, long long num_nets, long long num_mov) {
    CsrScratch s = {};
    auto al = [](long long x) { return (size_t)((x + 255) & ~255LL); };
    size_t at = 0;
    s.keep = at; at += al(4 * (num_nets + 1));
    s.kdeg = at; at += al(4 * (num_nets + 1));
    s.new_id = at; at += al(4 * (num_nets + 1));
    s.ostart = at; at += al(4 * (num_nets + 1));
    s.ccount = at; at += al(4 * (num_mov + 2));
    s.cursor = at; at += al(4 * (num_mov + 2));
    s.fixed = at; at += al(4 * (P + 1));
    s.rank = at; at += al(4 * (P + 1));
    s.big = at; at += al(4 * (num_mov + 1));
    s.tile = at; at += al(4 * (long long)SCAN_MAX_TILES);
    s.totals = at; at += al(4 * 8);
    s.bytes = at;
    return s;
}

// ---- smoothed nodes
__global__ void __launch_bounds__(256) smooth_kernel(const double2* size, int n, int num_mov, double minx,
                                                     double miny, float width, float height, float2* size_s,
                                                     float* ratio, float2* lo, float2* hi, float* area,
                                                     const int* cell_pins, float* pins) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double2 r = size[i];
        const double sx = fmax(r.x, minx), sy = fmax(r.y, miny);
        const double real = __dmul_rn(r.x, r.y);
        const float2 s = make_float2(__double2float_rn(sx), __double2float_rn(sy));
        size_s[i] = s;
        ratio[i] = __double2float_rn(__ddiv_rn(real, __dmul_rn(sx, sy)));
        const float2 l = make_float2(s.x * 0.5f, s.y * 0.5f);
        if (lo) lo[i] = l;
        if (hi) hi[i] = make_float2(__fsub_rn(width, l.x), __fsub_rn(height, l.y));
        if (area) area[i] = __double2float_rn(real);
        if (pins) pins[i] = i < num_mov && cell_pins ? (float)cell_pins[i] : 0.f;
    }
}

}  // namespace

}  // namespace gp103

using namespace gp103;

extern "C" size_t gp103_build_csr_scratch(int num_pins, int num_nets, int num_mov) {
    if (num_pins < 0 || num_nets < 0 || num_mov < 0) return 0;
    return csr_scratch(num_pins, num_nets, num_mov).bytes;
}

#define GP103_LAUNCH(...)                                   \
    do {                                                    \
        if (launch_k(__VA_ARGS__) != cudaSuccess) return GP103_ERR_CUDA; \
        GP103_CHECK_LAUNCH();                               \
    } while (0)

extern "C" int gp103_build_csr(const int* pin_cell, const float* pin_off, const int* pin_net, int num_pins,
                               int num_nets, int num_mov, int ignore_degree, void* scratch, size_t scratch_bytes,
                               int* net_start, int* cell32, float* off, int* cell_start, int* cell_pin,
                               int* all_net_start, int* cell_pins, int* counts, cudaStream_t s) {
    const int P = num_pins;
    if (P < 0 || num_nets < 0 || num_mov < 0 || !scratch || !net_start || !cell_start || !all_net_start ||
        !counts || (num_mov > 0 && !cell_pins))
        return GP103_ERR_ARG;
    if (P > 0 && (!pin_cell || !pin_off || !pin_net || !cell32 || !off || !cell_pin)) return GP103_ERR_ARG;
    const long long lim = (long long)SCAN_TILE * SCAN_MAX_TILES;
    if (P + 1LL > lim || num_nets + 1LL > lim || num_mov + 1LL > lim) return GP103_ERR_TOO_LARGE;
    const CsrScratch L = csr_scratch(P, num_nets, num_mov);
    if (scratch_bytes < L.bytes) return GP103_ERR_ARG;
    char* w = (char*)scratch;
    int *keep = (int*)(w + L.keep), *kdeg = (int*)(w + L.kdeg), *new_id = (int*)(w + L.new_id);
    int *ostart = (int*)(w + L.ostart), *ccount = (int*)(w + L.ccount), *cursor = (int*)(w + L.cursor);
    int *fixed = (int*)(w + L.fixed), *rank = (int*)(w + L.rank), *big = (int*)(w + L.big);
    int *tile = (int*)(w + L.tile), *totals = (int*)(w + L.totals);
    // totals: [0] optimised nets, [1] optimised pins, [2] pins counted per cell, [3] fixed pins, [4] big cells
    if (cudaMemsetAsync(totals, 0, 32, s) != cudaSuccess || cudaMemsetAsync(counts, 0, 4 * sizeof(int), s) ||
        cudaMemsetAsync(all_net_start, 0, sizeof(int) * ((size_t)num_nets + 1), s) ||
        cudaMemsetAsync(ccount, 0, sizeof(int) * ((size_t)num_mov + 1), s) ||
        cudaMemsetAsync(fixed, 0, sizeof(int) * ((size_t)P + 1), s) ||
        (num_mov > 0 && cudaMemsetAsync(cell_pins, 0, sizeof(int) * (size_t)num_mov, s)))
        return GP103_ERR_CUDA;
    const int gp = grid_for(P + 1, 256, 8), gn = grid_for(num_nets + 1, 256, 8), gc = grid_for(num_mov + 1, 256, 8);
    if (P > 0)
        GP103_LAUNCH(pin_check_kernel, dim3(gp), dim3(256), 0, s, pin_net, pin_cell, P, num_nets, num_mov, cell_pins,
                     counts);
    GP103_LAUNCH(net_bounds_kernel, dim3(gp), dim3(256), 0, s, pin_net, P, num_nets, (const int*)counts,
                 all_net_start);
    if (num_nets > 0)
        GP103_LAUNCH(net_keep_kernel, dim3(gn), dim3(256), 0, s, (const int*)all_net_start, num_nets, ignore_degree,
                     keep, kdeg);
    int st;
    if ((st = exclusive_scan(keep, num_nets, new_id, tile, totals + 0, s))) return st;
    if ((st = exclusive_scan(kdeg, num_nets, ostart, tile, totals + 1, s))) return st;
    GP103_LAUNCH(net_emit_kernel, dim3(gn), dim3(256), 0, s, (const int*)keep, (const int*)new_id,
                 (const int*)ostart, (const int*)totals, num_nets, net_start);
    if (P > 0)
        GP103_LAUNCH(pin_copy_kernel, dim3(gp), dim3(256), 0, s, pin_net, pin_cell, (const float2*)pin_off, P,
                     num_nets, num_mov, (const int*)all_net_start, (const int*)kdeg, (const int*)ostart, cell32,
                     (float2*)off, ccount);
    if ((st = exclusive_scan(ccount, num_mov + 1, cell_start, tile, totals + 2, s))) return st;
    if (cudaMemcpyAsync(cursor, cell_start, sizeof(int) * ((size_t)num_mov + 1), cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    if (P > 0) {
        GP103_LAUNCH(cell_place_kernel, dim3(gp), dim3(256), 0, s, (const int*)cell32, (const int*)totals, P,
                     num_mov, cursor, cell_pin, fixed);
        if ((st = exclusive_scan(fixed, P, rank, tile, totals + 3, s))) return st;
        GP103_LAUNCH(fixed_place_kernel, dim3(gp), dim3(256), 0, s, (const int*)fixed, (const int*)rank,
                     (const int*)totals, P, (const int*)cell_start, num_mov, cell_pin);
        if (num_mov > 0) {
            GP103_LAUNCH(cell_ties_kernel, dim3(gc), dim3(256), 0, s, (const int*)cell_start, num_mov, cell_pin, big,
                         totals + 4, counts + 2);
            GP103_LAUNCH(cell_ties_big_kernel, dim3(SMS * 4), dim3(256), 0, s, (const int*)big,
                         (const int*)(totals + 4), (const int*)cell_start, cell_pin);
        }
    }
    // counts = (optimised nets, optimised pins, errors, pins on movable cells)
    if (cudaMemcpyAsync(counts, totals, 2 * sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return GP103_ERR_CUDA;
    return GP103_OK;
}

extern "C" int gp103_smooth_nodes(const double* size, int n, int num_mov, double min_x, double min_y, float width,
                                  float height, float* size_s, float* ratio, float* lo, float* hi, float* area,
                                  const int* cell_pins, float* pins, cudaStream_t s) {
    if (n < 0 || num_mov < 0 || num_mov > n) return GP103_ERR_ARG;
    if (n == 0) return GP103_OK;
    if (!size || !size_s || !ratio || (pins && num_mov > 0 && !cell_pins)) return GP103_ERR_ARG;
    GP103_LAUNCH(smooth_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, (const double2*)size, n, num_mov, min_x,
                 min_y, width, height, (float2*)size_s, ratio, (float2*)lo, (float2*)hi, area, cell_pins, pins);
    return GP103_OK;
}

// ----------------------------------------------------------------------------- fixed fraction of the bins
// The share of each bin under a fixed object (PlaceData.fixed_fraction, src/database.py:103-134, in the form it takes
// when the rows cover the whole region and the fixed rectangles do not overlap, as in the synthetic netlists): per
// bin, the overlap area of every rectangle in rectangle order, over the bin area, clipped to [0, 1]. float64, the
// host statement's operations in its order (no contraction into fused multiply-adds): the same bits.
namespace gp103 {
__global__ void macro_fraction_kernel(const double* rects, int count, double bx, double by, int nbx, int nby,
                                      double* out) {
    gp103::pdl_wait();
    const double area = __dmul_rn(bx, by);
    for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < (long long)nbx * nby;
         b += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(b / nby), j = (int)(b - (long long)i * nby);
        const double x0 = __dmul_rn((double)i, bx), x1 = __dmul_rn((double)(i + 1), bx);
        const double y0 = __dmul_rn((double)j, by), y1 = __dmul_rn((double)(j + 1), by);
        double cover = 0.0;
        for (int m = 0; m < count; m++) {
            const double* r = rects + 4 * m;
            const double ox = fmax(__dsub_rn(fmin(x1, r[2]), fmax(x0, r[0])), 0.0);
            const double oy = fmax(__dsub_rn(fmin(y1, r[3]), fmax(y0, r[1])), 0.0);
            cover = __dadd_rn(cover, __dmul_rn(ox, oy));
        }
        out[b] = fmin(fmax(__ddiv_rn(cover, area), 0.0), 1.0);
    }
}
}  // namespace gp103

extern "C" int gp103_macro_fraction(const double* rects, int count, double width, double height, int nbx, int nby,
                                    double* fraction, cudaStream_t s) {
    if (count < 0 || nbx <= 0 || nby <= 0 || !(width > 0.0) || !(height > 0.0) || !fraction || (count > 0 && !rects))
        return GP103_ERR_ARG;
    const double bx = width / nbx, by = height / nby;
    if (gp103::launch_k(macro_fraction_kernel, dim3(gp103::grid_for((long long)nbx * nby, 256, 8)), dim3(256), 0, s,
                        rects, count, bx, by, nbx, nby, fraction) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}
