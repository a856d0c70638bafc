/* ORACLE — test infrastructure only. Not part of the product: only tests/ and the CPU legs of bench.py (the CPU
 * baseline and the reference arm) load this library.
 *
 * Multi-threaded (OpenMP) forms of the oracle's per-iteration operators, so that a whole level of the reference's
 * CPU iteration (its `--gpu -1` path) runs to the stop on a large netlist in minutes on the host cores:
 *   oracle_wa_mt            WA wirelength and cell gradients (src/core/wa_wirelength_hpwl.py:83-94) in float32, the
 *                           arithmetic of gp_oracle.wa_forward(dtype=float32): per net and axis max / min, max-shifted
 *                           exponent sums in pin order, per-pin gradient; each cell's sum over its pins in pin order
 *                           (float64, then float32)
 *   oracle_density_map_mt   the fixed-point map of oracle_density_map: per-thread integer maps, then their sum (integer
 *                           sums: the same map in any order)
 *   oracle_density_grad_mt  oracle_density_grad, nodes split over the threads (each node independent: the same bits)
 * Without OpenMP the pragmas are ignored and every routine runs on one thread, with the same results.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void oracle_density_map(const float* pos, const float* size, const float* ratio, int num_nodes, int num_mov,
                        float bx, float by, int nbx, int nby, uint64_t* map);
void oracle_density_grad(const float* pos, const float* size, const float* ratio, const double* fx, const double* fy,
                         int ld, const float* wl_grad, int num_wl, const float* pins, const float* area, int num_nodes,
                         double weight, double precond, float bx, float by, int nbx, int nby, double* grad);

int oracle_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* pos [>= num_mov, 2] float32; pins grouped by net (net_start [num_nets + 1]); a pin whose cell is >= num_mov sits
 * at its offset (a fixed pin). Writes pin_grad [P, 2] (float32), grad [num_mov, 2] (float32, each cell's pins summed
 * in float64 in cell_pin order), net_out [num_nets, 2] = (WA, HPWL) in float32; returns the totals (WA, HPWL) in
 * float64 through totals[2]. */
void oracle_wa_mt(const float* pos, const int* cell32, const float* off, const int* net_start, int num_nets,
                  int num_mov, float gamma, const int* cell_start, const int* cell_pin, float* pin_grad, float* grad,
                  float* net_out, double* totals) {
    double wa_total = 0, hpwl_total = 0;
#pragma omp parallel for schedule(dynamic, 2048) reduction(+ : wa_total, hpwl_total)
    for (int e = 0; e < num_nets; e++) {
        const int p0 = net_start[e], p1 = net_start[e + 1];
        float net_wa = 0.f, net_hpwl = 0.f;
        for (int a = 0; a < 2; a++) {
            float hi = -INFINITY, lo = INFINITY;
            for (int p = p0; p < p1; p++) {
                const int c = cell32[p];
                const float x = (c < num_mov ? pos[2 * c + a] : 0.f) + off[2 * p + a];
                hi = x > hi ? x : hi;
                lo = x < lo ? x : lo;
            }
            float sp = 0.f, sn = 0.f, xsp = 0.f, xsn = 0.f;
            for (int p = p0; p < p1; p++) {
                const int c = cell32[p];
                const float x = (c < num_mov ? pos[2 * c + a] : 0.f) + off[2 * p + a];
                const float ep = expf((x - hi) / gamma), en = expf((lo - x) / gamma);
                sp += ep;
                sn += en;
                xsp += x * ep;
                xsn += x * en;
            }
            const float xp = xsp / sp, xn = xsn / sn;
            for (int p = p0; p < p1; p++) {
                const int c = cell32[p];
                const float x = (c < num_mov ? pos[2 * c + a] : 0.f) + off[2 * p + a];
                const float ep = expf((x - hi) / gamma), en = expf((lo - x) / gamma);
                pin_grad[2 * p + a] = ep * (1.f + (x - xp) / gamma) / sp - en * (1.f - (x - xn) / gamma) / sn;
            }
            net_wa += xp - xn;
            net_hpwl += hi - lo;
        }
        net_out[2 * e] = net_wa;
        net_out[2 * e + 1] = net_hpwl;
        wa_total += net_wa;
        hpwl_total += net_hpwl;
    }
#pragma omp parallel for schedule(static)
    for (int c = 0; c < num_mov; c++) {
        double gx = 0, gy = 0;
        for (int k = cell_start[c]; k < cell_start[c + 1]; k++) {
            const int p = cell_pin[k];
            gx += pin_grad[2 * p];
            gy += pin_grad[2 * p + 1];
        }
        grad[2 * c] = (float)gx;
        grad[2 * c + 1] = (float)gy;
    }
    totals[0] = wa_total;
    totals[1] = hpwl_total;
}

/* The map of oracle_density_map (the caller zeroes map [2][nbx][nby]); scratch: threads x 2 nbx nby uint64 (or NULL:
 * allocated here). */
void oracle_density_map_mt(const float* pos, const float* size, const float* ratio, int num_nodes, int num_mov,
                           float bx, float by, int nbx, int nby, uint64_t* map) {
    const size_t plane = (size_t)2 * nbx * nby;
    int threads = oracle_threads(0);
    if (threads <= 1 || num_nodes < 4096) {
        oracle_density_map(pos, size, ratio, num_nodes, num_mov, bx, by, nbx, nby, map);
        return;
    }
    uint64_t* priv = (uint64_t*)calloc((size_t)threads * plane, sizeof(uint64_t));
    if (!priv) {
        oracle_density_map(pos, size, ratio, num_nodes, num_mov, bx, by, nbx, nby, map);
        return;
    }
#pragma omp parallel num_threads(threads)
    {
        int t = 0, nt = 1;
#ifdef _OPENMP
        t = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        const long long lo = (long long)num_nodes * t / nt, hi = (long long)num_nodes * (t + 1) / nt;
        /* the nodes [lo, hi) into this thread's own map: the movable ones into plane 0, the rest into plane 1 */
        const int mov_hi = (int)(hi < num_mov ? hi : num_mov);
        uint64_t* m = priv + (size_t)t * plane;
        if (lo < mov_hi)
            oracle_density_map(pos + 2 * lo, size + 2 * lo, ratio + lo, (int)(mov_hi - lo), (int)(mov_hi - lo), bx,
                               by, nbx, nby, m);
        const long long f0 = lo > num_mov ? lo : num_mov;
        if (f0 < hi)
            oracle_density_map(pos + 2 * f0, size + 2 * f0, ratio + f0, (int)(hi - f0), 0, bx, by, nbx, nby, m);
#pragma omp barrier
#pragma omp for schedule(static)
        for (long long b = 0; b < (long long)plane; b++) {
            uint64_t s = map[b];
            for (int k = 0; k < nt; k++) s += priv[(size_t)k * plane + b];
            map[b] = s;
        }
    }
    free(priv);
}

void oracle_density_grad_mt(const float* pos, const float* size, const float* ratio, const double* fx,
                            const double* fy, int ld, const float* wl_grad, int num_wl, const float* pins,
                            const float* area, int num_nodes, double weight, double precond, float bx, float by,
                            int nbx, int nby, double* grad) {
    const int chunk = 8192;
    const int parts = (num_nodes + chunk - 1) / chunk;
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < parts; k++) {
        const int i0 = k * chunk, n = num_nodes - i0 < chunk ? num_nodes - i0 : chunk;
        const int nwl = num_wl - i0 < 0 ? 0 : (num_wl - i0 < n ? num_wl - i0 : n);
        oracle_density_grad(pos + 2 * i0, size + 2 * i0, ratio + i0, fx, fy, ld, wl_grad ? wl_grad + 2 * i0 : NULL,
                            nwl, pins + i0, area + i0, n, weight, precond, bx, by, nbx, nby, grad + 2 * i0);
    }
}
