// Clustering of the cells by rounds of star matching (GB300, sm_103a): the first step of AutoPlace's two-level
// placement, on the device.
//
// Reference: src/cluster.py:38-85 (cluster_cells). Pair edges: every net of at most max_degree pins gives each
// ordered pair of distinct movable cells 420 // (degree - 1), summed per pair. A round: the non-head clusters pick
// the head with the largest w / (area_i + area_j) (first edge on ties), a head keeps its per_head best (lower index
// first on ties), clusters are renumbered in order, areas and edges summed. Every sum is an integer and every choice
// has a fixed tie rule, so the result does not depend on the order atomics place things in: it is the reference's,
// bit for bit. The head draws of a round come from the host (the reference draws them from a seeded CPU generator).
#include "gp103.cuh"
#include "kernels.cuh"

namespace gp103 {

namespace {

// ---------------------------------------------------------------------------------------------- COO -> CSR
// rows: row index of each entry; result: per row, its columns ascending, equal columns merged (weights summed).
struct CsrTemp {
    int* count;    // [rows + 1]
    int* cursor;   // [rows + 1]
    int* merged;   // [rows + 1]
    int* tmp_j;    // [max entries]
    int* tmp_w;    // [max entries]
    int* tile;     // [SCAN_MAX_TILES]
    int* total;    // [4]
    int* long_rows;  // [rows]: the rows merged by a warp each
    int* nlong;      // [1]: their number
};

// (entries beyond cap were never written, rows out of range never produced: both guarded all the same)
__global__ void __launch_bounds__(256) coo_count_kernel(const int* ci, const int* num, int cap, int rows, int* count) {
    pdl_wait();
    const int m = min(*num, cap);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x)
        if ((unsigned)ci[e] < (unsigned)rows) atomicAdd(&count[ci[e]], 1);
}

__global__ void __launch_bounds__(256) coo_place_kernel(const int* ci, const int* cj, const int* cw, const int* num,
                                                        int cap, int rows, int* cursor, int* tj, int* tw) {
    pdl_wait();
    const int m = min(*num, cap);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x) {
        if ((unsigned)ci[e] >= (unsigned)rows) continue;
        const int at = atomicAdd(&cursor[ci[e]], 1);
        tj[at] = cj[e];
        tw[at] = cw[e];
    }
}

// A warp's appends to one list: lane l appends k_l entries; -> the position of the lane's first one (one atomic per
// warp; every lane of the warp must call it). The order of the entries in the list is arbitrary either way: the
// CSR build sorts each row and sums the weights of equal columns (integers).
__device__ __forceinline__ int warp_append(int* m, int k) {
    const int lane = threadIdx.x & 31;
    int incl = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(m, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + incl - k;
}

// A row's entries sorted by column, equal columns merged (weights summed) to the front of the row. Rows of up to
// ROW_SHORT entries: a thread per row (insertion sort); longer ones: a warp per row (bitonic sort of (column, weight)
// keys in shared memory, then the runs of equal columns summed); beyond ROW_WARP_MAX entries (rare): lane 0 by
// insertion sort. Integer sums in any order: every form gives the same row.
__device__ int serial_merge_row(int b, int e, int* tj, int* tw) {
    for (int k = b + 1; k < e; k++) {
        const int j = tj[k], w = tw[k];
        int q = k - 1;
        while (q >= b && tj[q] > j) {
            tj[q + 1] = tj[q];
            tw[q + 1] = tw[q];
            q--;
        }
        tj[q + 1] = j;
        tw[q + 1] = w;
    }
    int out = b;
    for (int k = b; k < e; k++) {
        if (out > b && tj[out - 1] == tj[k]) {
            tw[out - 1] += tw[k];
        } else {
            tj[out] = tj[k];
            tw[out] = tw[k];
            out++;
        }
    }
    return out - b;
}

__device__ __forceinline__ int warp_id_global() { return (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); }
__device__ __forceinline__ int warps_in_grid() { return (int)(((size_t)gridDim.x * blockDim.x) >> 5); }

// Rows of up to ROW_SHORT entries: a thread per row; longer ones go to a list (warp-aggregated appends) for
// row_merge_long_kernel.
constexpr int ROW_SHORT = 32;

__global__ void __launch_bounds__(256) row_merge_kernel(const int* start, int rows, int* tj, int* tw, int* merged,
                                                        int* long_rows, int* nlong) {
    pdl_wait();
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x; base < rows; base += stride) {          // warp-uniform trip count
        const int r = base + threadIdx.x;
        bool is_long = false;
        if (r < rows) {
            const int b = start[r], e = start[r + 1];
            if (e - b <= ROW_SHORT) merged[r] = serial_merge_row(b, e, tj, tw);
            else is_long = true;
        }
        const int at = warp_append(nlong, is_long ? 1 : 0);
        if (is_long) long_rows[at] = r;
    }
}

// the listed long rows, a warp per row: keys (column << 32 | weight) sorted ascending, padded to a power of two
constexpr int ROW_WARP_MAX = 512;

__global__ void __launch_bounds__(256) row_merge_long_kernel(const int* start, const int* long_rows, const int* nlong,
                                                             int* tj, int* tw, int* merged) {
    pdl_wait();
    __shared__ unsigned long long keys[8][ROW_WARP_MAX];
    const int lane = threadIdx.x & 31, count = *nlong;
    unsigned long long* sk = keys[threadIdx.x >> 5];
    for (int q = warp_id_global(); q < count; q += warps_in_grid()) {
        const int r = long_rows[q];
        const int b = start[r], k = start[r + 1] - b;
        int m = 0;
        if (k > ROW_WARP_MAX) {
            if (lane == 0) m = serial_merge_row(b, b + k, tj, tw);
            m = __shfl_sync(0xffffffffu, m, 0);
        } else {
            int n = 64;
            while (n < k) n <<= 1;
            for (int i = lane; i < n; i += 32)
                sk[i] = i < k ? ((unsigned long long)(unsigned)tj[b + i] << 32) | (unsigned)tw[b + i] : ~0ull;
            __syncwarp();
            for (int size = 2; size <= n; size <<= 1)
                for (int stride = size >> 1; stride > 0; stride >>= 1) {
                    for (int t = lane; t < n / 2; t += 32) {
                        const int i = 2 * t - (t & (stride - 1)), j = i + stride;
                        const unsigned long long x = sk[i], y = sk[j];
                        if ((x > y) == ((i & size) == 0)) {
                            sk[i] = y;
                            sk[j] = x;
                        }
                    }
                    __syncwarp();
                }
            // runs of equal columns: each run's first entry writes the run's sum at its rank among the runs
            for (int c = 0; c < k; c += 32) {
                const int i = c + lane;
                const unsigned col = i < k ? (unsigned)(sk[i] >> 32) : 0u;
                const bool first = i < k && (i == 0 || (unsigned)(sk[i - 1] >> 32) != col);
                const unsigned fb = __ballot_sync(0xffffffffu, first);
                if (first) {
                    int sum = 0;
                    for (int j = i; j < k && (unsigned)(sk[j] >> 32) == col; j++) sum += (int)(unsigned)sk[j];
                    const int at = m + __popc(fb & ((1u << lane) - 1u));
                    tj[b + at] = (int)col;
                    tw[b + at] = sum;
                }
                m += __popc(fb);
            }
        }
        __syncwarp();
        if (lane == 0) merged[r] = m;
    }
}

// the merged front of every row to its place in the CSR, one warp per row (coalesced copies)
__global__ void __launch_bounds__(256) row_compact_kernel(const int* start, const int* row_start, int rows,
                                                          const int* tj, const int* tw, int* col, int* w) {
    pdl_wait();
    const int lane = threadIdx.x & 31;
    for (int r = warp_id_global(); r < rows; r += warps_in_grid()) {
        const int b = start[r], o = row_start[r], k = row_start[r + 1] - o;
        for (int t = lane; t < k; t += 32) {
            col[o + t] = tj[b + t];
            w[o + t] = tw[b + t];
        }
    }
}

// entries (ci, cj, cw) [*num, at most cap] -> CSR (row_start [rows + 1], col, w); *nnz = merged entries
int coo_to_csr(const int* ci, const int* cj, const int* cw, const int* num, int cap, int rows, const CsrTemp& t,
               int* row_start, int* col, int* w, int* nnz, cudaStream_t s) {
    if (cudaMemsetAsync(t.count, 0, sizeof(int) * (size_t)(rows + 1), s) != cudaSuccess) return GP103_ERR_CUDA;
    const int ge = grid_for(cap > 0 ? cap : 1, 256, 8);
    if (launch_k(coo_count_kernel, dim3(ge), dim3(256), 0, s, ci, num, cap, rows, t.count) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    int st;
    if ((st = exclusive_scan(t.count, rows + 1, t.cursor, t.tile, t.total, s))) return st;
    // cursor now holds the row starts; keep a copy (placement advances cursor)
    if (cudaMemcpyAsync(t.merged, t.cursor, sizeof(int) * (size_t)(rows + 1), cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    if (launch_k(coo_place_kernel, dim3(ge), dim3(256), 0, s, ci, cj, cw, num, cap, rows, t.cursor, t.tmp_j,
                 t.tmp_w) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    // t.merged = row starts; merged counts go to t.count (short rows by a thread each, long ones by a warp each)
    const int gr = grid_for(rows > 0 ? rows : 1, 256, 8), gw = grid_for(rows > 0 ? 32LL * rows : 1, 256, 8);
    if (cudaMemsetAsync(t.nlong, 0, sizeof(int), s) != cudaSuccess) return GP103_ERR_CUDA;
    if (launch_k(row_merge_kernel, dim3(gr), dim3(256), 0, s, (const int*)t.merged, rows, t.tmp_j, t.tmp_w, t.count,
                 t.long_rows, t.nlong) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (launch_k(row_merge_long_kernel, dim3(gw), dim3(256), 0, s, (const int*)t.merged, (const int*)t.long_rows,
                 (const int*)t.nlong, t.tmp_j, t.tmp_w, t.count) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (cudaMemsetAsync(t.count + rows, 0, sizeof(int), s) != cudaSuccess) return GP103_ERR_CUDA;
    if ((st = exclusive_scan(t.count, rows + 1, row_start, t.tile, nnz, s))) return st;
    if (launch_k(row_compact_kernel, dim3(gw), dim3(256), 0, s, (const int*)t.merged, (const int*)row_start, rows,
                 (const int*)t.tmp_j, (const int*)t.tmp_w, col, w) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// ---------------------------------------------------------------------------------------------- pair edges
__global__ void __launch_bounds__(256) net_degree_count_kernel(const int* pin_net, int num_pins, int num_nets,
                                                               int* deg) {
    pdl_wait();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < num_pins; p += gridDim.x * blockDim.x) {
        const int net = pin_net[p];
        if ((unsigned)net < (unsigned)num_nets) atomicAdd(&deg[net], 1);
    }
}

// pins k apart in the pin list (k < max_degree) of one net of at most max_degree pins: both ordered pairs (a thread per
// pin counts its pairs, then the warp appends them with one atomic)
__device__ __forceinline__ bool pair_ok(const int* pin_cell, const int* pin_net, int num_pins, int n, int p, int k,
                                        int net, int a, int& b) {
    if (p + k >= num_pins || pin_net[p + k] != net) return false;
    b = pin_cell[p + k];
    return !(a < 0 || b < 0 || a >= n || b >= n || a == b);
}

__global__ void __launch_bounds__(256) pair_emit_kernel(const int* pin_cell, const int* pin_net, int num_pins,
                                                        int num_nets, int n, int max_degree, const int* deg, int cap,
                                                        int* num, int* ci, int* cj, int* cw) {
    pdl_wait();
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x; base < num_pins; base += stride) {     // warp-uniform trip count
        const int p = base + threadIdx.x;
        int net = -1, d = 0, a = -1, cnt = 0;
        if (p < num_pins) {
            net = pin_net[p];
            if ((unsigned)net < (unsigned)num_nets) {
                d = deg[net];
                a = pin_cell[p];
            }
        }
        const bool live = d >= 2 && d <= max_degree;
        if (live)
            for (int k = 1; k < max_degree; k++) {
                int b;
                if (p + k >= num_pins || pin_net[p + k] != net) break;
                if (pair_ok(pin_cell, pin_net, num_pins, n, p, k, net, a, b)) cnt++;
            }
        int at = warp_append(num, 2 * cnt);
        if (live) {
            const int wgt = 420 / (d - 1);
            for (int k = 1; k < max_degree; k++) {
                int b;
                if (p + k >= num_pins || pin_net[p + k] != net) break;
                if (!pair_ok(pin_cell, pin_net, num_pins, n, p, k, net, a, b)) continue;
                if (at + 1 < cap) {
                    ci[at] = a; cj[at] = b; cw[at] = wgt;
                    ci[at + 1] = b; cj[at + 1] = a; cw[at + 1] = wgt;
                }
                at += 2;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------- a round
// per non-head cluster: the head of the largest score, the first one (first edge of the row) on ties
__global__ void __launch_bounds__(256) best_head_kernel(const int* row_start, const int* col, const int* w, int num,
                                                        const long long* area, const unsigned char* head,
                                                        long long cap, long long big, int* best_to, double* best) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x) {
        int to = -1;
        double sc = 0.0;
        if (!head[i] && area[i] < big) {
            for (int e = row_start[i]; e < row_start[i + 1]; e++) {
                const int j = col[e];
                if (!head[j] || area[j] >= big) continue;
                const long long total = area[i] + area[j];
                if (total > cap) continue;
                const double s = (double)w[e] / (double)total;
                if (to < 0 || s > sc) {
                    to = j;
                    sc = s;
                }
            }
        }
        best_to[i] = to;
        best[i] = sc;
    }
}

__global__ void __launch_bounds__(256) cand_count_kernel(const int* best_to, int num, int* count, int* parent) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x) {
        parent[i] = i;
        if (best_to[i] >= 0) atomicAdd(&count[best_to[i]], 1);
    }
}

__global__ void __launch_bounds__(256) cand_place_kernel(const int* best_to, int num, int* cursor, int* list) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x)
        if (best_to[i] >= 0) list[atomicAdd(&cursor[best_to[i]], 1)] = i;
}

// per head: its per_head best tails (score descending, lower tail first on ties) join it
__global__ void __launch_bounds__(256) take_kernel(const int* start, const int* list, const double* best, int num,
                                                   int per_head, int* parent) {
    pdl_wait();
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < num; h += gridDim.x * blockDim.x) {
        const int b = start[h], e = start[h + 1];
        double last_s = 0.0;
        int last_t = -1;
        for (int k = 0; k < per_head && k < e - b; k++) {
            // the best candidate below (last_s, last_t) in the order (score desc, tail asc)
            int pick = -1;
            double ps = 0.0;
            for (int q = b; q < e; q++) {
                const int t = list[q];
                const double s = best[t];
                const bool below = last_t < 0 || s < last_s || (s == last_s && t > last_t);
                if (!below) continue;
                if (pick < 0 || s > ps || (s == ps && t < pick)) {
                    pick = t;
                    ps = s;
                }
            }
            if (pick < 0) break;
            parent[pick] = h;
            last_s = ps;
            last_t = pick;
        }
    }
}

__global__ void __launch_bounds__(256) kept_flag_kernel(const int* parent, int num, int* flag) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x) flag[i] = parent[i] == i;
}

// new index of every cluster (its parent's rank among the kept ones), summed areas
__global__ void __launch_bounds__(256) renumber_kernel(const int* parent, const int* rank, int num,
                                                       const long long* area, int* new_index, long long* area_out) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x) {
        const int k = rank[parent[i]];
        new_index[i] = k;
        atomicAdd((unsigned long long*)&area_out[k], (unsigned long long)area[i]);
    }
}

// the edges between the new clusters (a cluster's own edges dropped), as entries for coo_to_csr (a thread per old
// cluster counts its kept edges, then the warp appends them with one atomic)
__global__ void __launch_bounds__(256) edge_relabel_kernel(const int* row_start, const int* col, const int* w, int num,
                                                           const int* new_index, int cap, int* m, int* ci, int* cj,
                                                           int* cw) {
    pdl_wait();
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x; base < num; base += stride) {           // warp-uniform trip count
        const int i = base + threadIdx.x;
        int a = -1, b0 = 0, b1 = 0, cnt = 0;
        if (i < num) {
            a = new_index[i];
            b0 = row_start[i];
            b1 = row_start[i + 1];
            for (int e = b0; e < b1; e++) cnt += new_index[col[e]] != a;
        }
        int at = warp_append(m, cnt);
        for (int e = b0; e < b1; e++) {
            const int b = new_index[col[e]];
            if (a == b) continue;
            if (at < cap) {
                ci[at] = a;
                cj[at] = b;
                cw[at] = w[e];
            }
            at++;
        }
    }
}

// ---------------------------------------------------------------------------------------------- cluster problem
// A pin of the cluster problem: its cluster (num for a fixed pin); kept if its cluster has one cell or the pin is
// fixed (then with its offset), or if it is the first pin of its net on its (merged) cluster (then at the centre).
__global__ void __launch_bounds__(256) coarse_keep_kernel(const int* pin_cell, const int* pin_net, int num_pins, int n,
                                                          const int* cid, int num, const unsigned char* single,
                                                          int* owner, int* keep) {
    pdl_wait();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < num_pins; p += gridDim.x * blockDim.x) {
        const int c = pin_cell[p];
        const int o = (c >= 0 && c < n) ? cid[c] : num;
        owner[p] = o;
        const bool fixed_off = o >= num || single[o];
        bool first = true;
        if (!fixed_off) {
            const int net = pin_net[p];
            for (int q = p - 1; q >= 0 && pin_net[q] == net; q--) {
                const int cq = pin_cell[q];
                if (((cq >= 0 && cq < n) ? cid[cq] : num) == o) {
                    first = false;
                    break;
                }
            }
        }
        keep[p] = fixed_off || first;
    }
}

__global__ void __launch_bounds__(256) coarse_write_kernel(const float2* pin_off, const int* pin_net, int num_pins,
                                                           int num, const unsigned char* single, const int* owner,
                                                           const int* keep, const int* at, int* out_cell,
                                                           float2* out_off, int* out_net) {
    pdl_wait();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < num_pins; p += gridDim.x * blockDim.x) {
        if (!keep[p]) continue;
        const int o = owner[p], k = at[p];
        out_cell[k] = o;
        out_off[k] = (o >= num || single[o]) ? pin_off[p] : make_float2(0.f, 0.f);
        out_net[k] = pin_net[p];
    }
}

// cells at a point of their cluster's square: cpos[cid] + (r - 0.5) (csize[cid] - size, clamped at 0), in float32
// with the reference's operation order (no contraction into fused multiply-adds)
__global__ void __launch_bounds__(256) expand_kernel(const float2* cpos, const int* cid, const float2* csize,
                                                     const float2* size, const float2* r, int n, float2* pos) {
    pdl_wait();
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int k = cid[c];
        const float2 cs = csize[k], s = size[c], q = cpos[k], u = r[c];
        const float rx = fmaxf(__fsub_rn(cs.x, s.x), 0.f), ry = fmaxf(__fsub_rn(cs.y, s.y), 0.f);
        pos[c] = make_float2(__fadd_rn(q.x, __fmul_rn(__fsub_rn(u.x, 0.5f), rx)),
                             __fadd_rn(q.y, __fmul_rn(__fsub_rn(u.y, 0.5f), ry)));
    }
}

__global__ void relabel_kernel(int* cid, int n, const int* new_index) {
    pdl_wait();
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) cid[c] = new_index[cid[c]];
}

// ---------------------------------------------------------------------------------------------- scratch
struct ClusterScratch {
    size_t count, cursor, merged, tmp_j, tmp_w, coo_i, coo_j, coo_w, deg, best_to, best, list, parent, tile, total,
        bytes;
};

ClusterScratch cluster_scratch(long long n, long long num_nets, long long max_edges) {
    ClusterScratch c = {};
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t rows = (size_t)n + 1, e = (size_t)(max_edges > 0 ? max_edges : 1);
    size_t at = 0;
    c.count = at; at += al(4 * rows);
    c.cursor = at; at += al(4 * rows);
    c.merged = at; at += al(4 * rows);
    c.tmp_j = at; at += al(4 * e);
    c.tmp_w = at; at += al(4 * e);
    c.coo_i = at; at += al(4 * e);
    c.coo_j = at; at += al(4 * e);
    c.coo_w = at; at += al(4 * e);
    c.deg = at; at += al(4 * (size_t)(num_nets > 0 ? num_nets : 1));
    c.best_to = at; at += al(4 * rows);
    c.best = at; at += al(8 * rows);
    c.list = at; at += al(4 * rows);
    c.parent = at; at += al(4 * rows);
    c.tile = at; at += al(4 * (size_t)SCAN_MAX_TILES);
    c.total = at; at += al(4 * 8);
    c.bytes = at;
    return c;
}

CsrTemp csr_temp(char* base, const ClusterScratch& L) {
    CsrTemp t;
    t.count = (int*)(base + L.count);
    t.cursor = (int*)(base + L.cursor);
    t.merged = (int*)(base + L.merged);
    t.tmp_j = (int*)(base + L.tmp_j);
    t.tmp_w = (int*)(base + L.tmp_w);
    t.tile = (int*)(base + L.tile);
    t.total = (int*)(base + L.total) + 4;
    // (the candidate list of a round is consumed before the round's CSR build)
    t.long_rows = (int*)(base + L.list);
    t.nlong = (int*)(base + L.total) + 2;
    return t;
}

// The clusters' members: counts per cluster (integer atomics: the same counts in any order).
__global__ void member_count_kernel(const int* cid, int n, int* count) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) atomicAdd(&count[cid[i]], 1);
}

// Per cluster: single = one member; the size of a merged cluster is the square of its summed area (areas in 1/1024 of
// a site area): float32(sqrt(area / 1024)) from float64, each side.
__global__ void cluster_square_kernel(const int* count, const long long* carea, int num, unsigned char* single,
                                      float2* csize) {
    pdl_wait();
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < num; c += gridDim.x * blockDim.x) {
        const bool one = count[c] == 1;
        single[c] = one ? 1 : 0;
        if (!one) {
            const float side = (float)__dsqrt_rn(__ddiv_rn((double)carea[c], 1024.0));
            csize[c] = make_float2(side, side);
        }
    }
}

// A one-cell cluster keeps its cell's size (its only member writes it).
__global__ void single_size_kernel(const int* cid, int n, const unsigned char* single, const float2* size,
                                   float2* csize) {
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = cid[i];
        if (single[c]) csize[c] = size[i];
    }
}

// ----------------------------------------------------------------------------- seeded draws
// The float32 stream of torch.rand(count, generator=torch.Generator().manual_seed(seed)) on the CPU, which the
// reference's clustering and expand draw from: the MT19937 generator (Matsumoto and Nishimura, 1998) with its
// standard initialisation from the seed's low 32 bits, each tempered 32-bit output x giving (x mod 2^24) 2^-24.
// One block of 624 threads, one state word each. A twist of the state runs in three parallel phases: words
// [0, 227) read only words of the old state, [227, 454) also the first phase's new words (i + 397 - 624), and
// [454, 624) the second phase's (and word 0, new, for word 623); each phase reads, waits, then writes. Then every
// thread tempers its word and writes one value.
constexpr int MT_N = 624, MT_M = 397;
constexpr unsigned MT_UPPER = 0x80000000u, MT_LOWER = 0x7fffffffu, MT_A = 0x9908b0dfu;

__device__ __forceinline__ unsigned mt_word(unsigned cur, unsigned next, unsigned far) {
    const unsigned y = (cur & MT_UPPER) | (next & MT_LOWER);
    return far ^ (y >> 1) ^ ((y & 1u) ? MT_A : 0u);
}

__global__ void __launch_bounds__(MT_N) mt_uniform_kernel(unsigned long long seed, long long count, float* out) {
    __shared__ unsigned mt[MT_N];
    pdl_wait();
    const int i = threadIdx.x;
    if (i == 0) {
        unsigned v = (unsigned)(seed & 0xffffffffull);
        mt[0] = v;
        for (int k = 1; k < MT_N; k++) {
            v = 1812433253u * (v ^ (v >> 30)) + (unsigned)k;
            mt[k] = v;
        }
    }
    __syncthreads();
    const bool a = i < MT_N - MT_M, b = i >= MT_N - MT_M && i < 2 * (MT_N - MT_M), c = i >= 2 * (MT_N - MT_M);
    for (long long base = 0; base < count; base += MT_N) {
        unsigned w = 0u;
        if (a) w = mt_word(mt[i], mt[i + 1], mt[i + MT_M]);
        __syncthreads();
        if (a) mt[i] = w;
        __syncthreads();
        if (b) w = mt_word(mt[i], mt[i + 1], mt[i + MT_M - MT_N]);
        __syncthreads();
        if (b) mt[i] = w;
        __syncthreads();
        if (c) w = mt_word(mt[i], mt[(i + 1) % MT_N], mt[i + MT_M - MT_N]);
        __syncthreads();
        if (c) mt[i] = w;
        __syncthreads();
        unsigned y = mt[i];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        if (base + i < count) out[base + i] = (float)(y & 0xffffffu) * 5.9604644775390625e-8f;   // 2^-24
    }
}

}  // namespace
}  // namespace gp103

using namespace gp103;

extern "C" int gp103_seeded_uniform(unsigned long long seed, long long count, float* out, cudaStream_t s) {
    if (count < 0 || (count > 0 && !out)) return GP103_ERR_ARG;
    if (count == 0) return GP103_OK;
    if (launch_k(mt_uniform_kernel, dim3(1), dim3(MT_N), 0, s, seed, count, out) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

extern "C" int gp103_cluster_members(const int* cid, int n, int num, const long long* carea, const float* size,
                                     int* count, unsigned char* single, float* csize, cudaStream_t s) {
    if (n < 0 || num < 0 || (n > 0 && (!cid || !size)) || (num > 0 && (!carea || !count || !single || !csize)))
        return GP103_ERR_ARG;
    if (num == 0) return GP103_OK;
    if (cudaMemsetAsync(count, 0, sizeof(int) * (size_t)num, s) != cudaSuccess) return GP103_ERR_CUDA;
    if (n > 0) {
        if (launch_k(member_count_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, cid, n, count) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    if (launch_k(cluster_square_kernel, dim3(grid_for(num, 256, 8)), dim3(256), 0, s, (const int*)count, carea, num,
                 single, (float2*)csize) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (n > 0) {
        if (launch_k(single_size_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, cid, n,
                     (const unsigned char*)single, (const float2*)size, (float2*)csize) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    return GP103_OK;
}

extern "C" size_t gp103_cluster_scratch(int n, int num_nets, int max_edges) {
    if (n < 0 || num_nets < 0 || max_edges < 0) return 0;
    return cluster_scratch(n, num_nets, max_edges).bytes;
}

extern "C" int gp103_cluster_edges(const int* pin_cell, const int* pin_net, int num_pins, int num_nets, int n,
                                   int max_degree, int max_edges, void* scratch, size_t scratch_bytes,
                                   int* row_start, int* col, int* w, int* counts, cudaStream_t s) {
    if (num_pins < 0 || num_nets < 0 || n < 0 || max_degree < 2 || max_edges < 0 || !scratch || !row_start ||
        !counts)
        return GP103_ERR_ARG;
    if (num_pins > 0 && (!pin_cell || !pin_net)) return GP103_ERR_ARG;
    if (max_edges > 0 && (!col || !w)) return GP103_ERR_ARG;
    if (n + 1LL > (long long)SCAN_TILE * SCAN_MAX_TILES) return GP103_ERR_TOO_LARGE;
    const ClusterScratch L = cluster_scratch(n, num_nets, max_edges);
    if (scratch_bytes < L.bytes) return GP103_ERR_ARG;
    char* base = (char*)scratch;
    int* deg = (int*)(base + L.deg);
    int *ci = (int*)(base + L.coo_i), *cj = (int*)(base + L.coo_j), *cw = (int*)(base + L.coo_w);
    int* m = (int*)(base + L.total);                              // entries appended (device)
    if (cudaMemsetAsync(deg, 0, sizeof(int) * (size_t)(num_nets > 0 ? num_nets : 1), s) != cudaSuccess ||
        cudaMemsetAsync(m, 0, sizeof(int), s) != cudaSuccess)
        return GP103_ERR_CUDA;
    const int gp = grid_for(num_pins > 0 ? num_pins : 1, 256, 8);
    if (num_pins > 0) {
        if (launch_k(net_degree_count_kernel, dim3(gp), dim3(256), 0, s, pin_net, num_pins, num_nets, deg) !=
            cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
        if (launch_k(pair_emit_kernel, dim3(gp), dim3(256), 0, s, pin_cell, pin_net, num_pins, num_nets, n,
                     max_degree, (const int*)deg, max_edges, m, ci, cj, cw) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    // counts[1] = entries appended (more than max_edges: the caller's bound was too small, the edges are not valid)
    if (cudaMemcpyAsync(counts + 1, m, sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess) return GP103_ERR_CUDA;
    return coo_to_csr(ci, cj, cw, m, max_edges, n, csr_temp(base, L), row_start, col, w, counts, s);
}

extern "C" int gp103_cluster_round(const int* row_start, const int* col, const int* w, int num, int max_edges,
                                   const long long* area, const unsigned char* head, long long cap, long long big,
                                   int per_head, void* scratch, size_t scratch_bytes, int* new_index,
                                   long long* area_out, int* row_out, int* col_out, int* w_out, int* counts,
                                   cudaStream_t s) {
    if (num < 1 || max_edges < 0 || per_head < 1 || !row_start || !area || !head || !scratch || !new_index ||
        !area_out || !row_out || !counts)
        return GP103_ERR_ARG;
    if (max_edges > 0 && (!col || !w || !col_out || !w_out)) return GP103_ERR_ARG;
    const ClusterScratch L = cluster_scratch(num, 0, max_edges);
    if (scratch_bytes < L.bytes) return GP103_ERR_ARG;
    char* base = (char*)scratch;
    const CsrTemp t = csr_temp(base, L);
    int* best_to = (int*)(base + L.best_to);
    double* best = (double*)(base + L.best);
    int* list = (int*)(base + L.list);
    int* parent = (int*)(base + L.parent);
    int *ci = (int*)(base + L.coo_i), *cj = (int*)(base + L.coo_j), *cw = (int*)(base + L.coo_w);
    int* m = (int*)(base + L.total);
    const int g = grid_for(num, 256, 8);
    int st;
    if (launch_k(best_head_kernel, dim3(g), dim3(256), 0, s, row_start, col, w, num, area, head, cap, big, best_to,
                 best) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    // candidates grouped by head: counts, starts (in t.merged), placement
    if (cudaMemsetAsync(t.count, 0, sizeof(int) * (size_t)(num + 1), s) != cudaSuccess) return GP103_ERR_CUDA;
    if (launch_k(cand_count_kernel, dim3(g), dim3(256), 0, s, (const int*)best_to, num, t.count, parent) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if ((st = exclusive_scan(t.count, num + 1, t.merged, t.tile, t.total, s))) return st;
    if (cudaMemcpyAsync(t.cursor, t.merged, sizeof(int) * (size_t)(num + 1), cudaMemcpyDeviceToDevice, s) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    if (launch_k(cand_place_kernel, dim3(g), dim3(256), 0, s, (const int*)best_to, num, t.cursor, list) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (launch_k(take_kernel, dim3(g), dim3(256), 0, s, (const int*)t.merged, (const int*)list, (const double*)best,
                 num, per_head, parent) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    // kept clusters (their own parent), ranked: counts[0] = the new number of clusters
    if (launch_k(kept_flag_kernel, dim3(g), dim3(256), 0, s, (const int*)parent, num, t.count) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (cudaMemsetAsync(t.count + num, 0, sizeof(int), s) != cudaSuccess) return GP103_ERR_CUDA;
    if ((st = exclusive_scan(t.count, num + 1, t.cursor, t.tile, counts, s))) return st;
    if (cudaMemsetAsync(area_out, 0, sizeof(long long) * (size_t)num, s) != cudaSuccess) return GP103_ERR_CUDA;
    if (launch_k(renumber_kernel, dim3(g), dim3(256), 0, s, (const int*)parent, (const int*)t.cursor, num, area,
                 new_index, area_out) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    // the new edges: relabelled, internal ones dropped, merged (rows: at most num)
    if (cudaMemsetAsync(m, 0, sizeof(int), s) != cudaSuccess) return GP103_ERR_CUDA;
    if (launch_k(edge_relabel_kernel, dim3(g), dim3(256), 0, s, row_start, col, w, num, (const int*)new_index,
                 max_edges, m, ci, cj, cw) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return coo_to_csr(ci, cj, cw, m, max_edges, num, t, row_out, col_out, w_out, counts + 1, s);
}

extern "C" int gp103_cluster_relabel(int* cid, int n, const int* new_index, cudaStream_t s) {
    if (n < 0 || (n > 0 && (!cid || !new_index))) return GP103_ERR_ARG;
    if (n == 0) return GP103_OK;
    if (launch_k(relabel_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, cid, n, new_index) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

extern "C" size_t gp103_coarse_pins_scratch(int num_pins) {
    if (num_pins < 0) return 0;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    return 3 * al(4 * ((size_t)num_pins + 1)) + al(4 * (size_t)SCAN_MAX_TILES) + al(64);
}

extern "C" int gp103_coarse_pins(const int* pin_cell, const float* pin_off, const int* pin_net, int num_pins, int n,
                                 const int* cid, int num, const unsigned char* single, void* scratch,
                                 size_t scratch_bytes, int* out_cell, float* out_off, int* out_net, int* count,
                                 cudaStream_t s) {
    if (num_pins < 0 || n < 0 || num < 0 || !scratch || !count) return GP103_ERR_ARG;
    if (num_pins > 0 && (!pin_cell || !pin_off || !pin_net || !out_cell || !out_off || !out_net)) return GP103_ERR_ARG;
    if (n > 0 && (!cid || !single)) return GP103_ERR_ARG;
    if (num_pins + 1LL > (long long)SCAN_TILE * SCAN_MAX_TILES) return GP103_ERR_TOO_LARGE;
    if (scratch_bytes < gp103_coarse_pins_scratch(num_pins)) return GP103_ERR_ARG;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    char* base = (char*)scratch;
    const size_t seg = al(4 * ((size_t)num_pins + 1));
    int *owner = (int*)base, *keep = (int*)(base + seg), *at = (int*)(base + 2 * seg);
    int* tile = (int*)(base + 3 * seg);
    if (num_pins == 0) return cudaMemsetAsync(count, 0, sizeof(int), s) == cudaSuccess ? GP103_OK : GP103_ERR_CUDA;
    const int g = grid_for(num_pins, 256, 8);
    if (launch_k(coarse_keep_kernel, dim3(g), dim3(256), 0, s, pin_cell, pin_net, num_pins, n, cid, num, single, owner,
                 keep) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (cudaMemsetAsync(keep + num_pins, 0, sizeof(int), s) != cudaSuccess) return GP103_ERR_CUDA;
    int st;
    if ((st = exclusive_scan(keep, num_pins + 1, at, tile, count, s))) return st;
    if (launch_k(coarse_write_kernel, dim3(g), dim3(256), 0, s, (const float2*)pin_off, pin_net, num_pins, num, single,
                 (const int*)owner, (const int*)keep, (const int*)at, out_cell, (float2*)out_off, out_net) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

extern "C" int gp103_expand(const float* cpos, const int* cid, const float* csize, const float* size,
                            const float* draws, int n, float* pos, cudaStream_t s) {
    if (n < 0 || (n > 0 && (!cpos || !cid || !csize || !size || !draws || !pos))) return GP103_ERR_ARG;
    if (n == 0) return GP103_OK;
    if (launch_k(expand_kernel, dim3(grid_for(n, 256, 8)), dim3(256), 0, s, (const float2*)cpos, cid,
                 (const float2*)csize, (const float2*)size, (const float2*)draws, n, (float2*)pos) != cudaSuccess)
        return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}
