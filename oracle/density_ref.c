/* ORACLE — test infrastructure only. Not part of the product: only tests/, the smoke check and the CPU baseline of
 * bench.py load this library, as the checker.
 *
 * CPU restatement of AutoPlace's density kernels (cpp_to_py/gp_cuda_kernel.cu), in the same float32 operation
 * order, so that the fixed-point density map is the same integer map, bit for bit:
 *   span / overlap        gp_cuda_kernel.cu:73-82
 *   density_map_kernel    gp_cuda_kernel.cu:84-95   (u64 sum of trunc(float(ratio*ox*oy) * 2^32))
 *   density_post_kernel   gp_cuda_kernel.cu:130-139 (mirrored total density, density above the target)
 *   density_grad_kernel   gp_cuda_kernel.cu:102-125 (here in float64: the oracle of the gather)
 * The reference is built with --use_fast_math, which flushes float32 denormals to zero: ftz() does the same after
 * every float32 operation. Float-to-integer conversions follow the GPU's (saturating, NaN -> 0): f2i(), f2u64().
 * Built with -ffp-contract=off so that no multiply-add is fused behind our back (x86 and Arm give the same bits).
 */
#include <math.h>
#include <stdint.h>
#include <float.h>
#include <limits.h>
#include <string.h>

#define DENSITY_SCALE 4294967296.0

static inline float ftz(float x) { return (fabsf(x) < FLT_MIN) ? copysignf(0.0f, x) : x; }
static inline float fmul(float a, float b) { return ftz(ftz(a) * ftz(b)); }
static inline float fadd(float a, float b) { return ftz(ftz(a) + ftz(b)); }
static inline float fsub(float a, float b) { return ftz(ftz(a) - ftz(b)); }
/* fminf / fmaxf: the non-NaN operand wins, as min.f32 / max.f32 on the GPU */
static inline float fmn(float a, float b) { return ftz(fminf(ftz(a), ftz(b))); }
static inline float fmx(float a, float b) { return ftz(fmaxf(ftz(a), ftz(b))); }

static inline int f2i(float x) {                       /* cvt.rzi.s32.f32 of an already floored value */
    if (isnan(x)) return 0;
    if (x >= 2147483648.0f) return INT_MAX;
    if (x <= -2147483648.0f) return INT_MIN;
    return (int)x;
}
static inline uint64_t f2u64(double x) {               /* cvt.rzi.u64.f64 */
    if (isnan(x) || x <= 0.0) return 0;
    if (x >= 18446744073709551616.0) return UINT64_MAX;
    return (uint64_t)x;
}

typedef struct { float lo, hi; int b0, b1; } Span;

static inline Span span(float centre, float size, float inv_bin, int nb) {
    Span s;
    float half = fmul(0.5f, size);
    s.lo = fmul(fsub(centre, half), inv_bin);
    s.hi = fmul(fadd(centre, half), inv_bin);
    int f0 = f2i(ftz(floorf(s.lo))), f1 = f2i(ftz(floorf(s.hi)));
    s.b0 = f0 > 0 ? f0 : 0;
    s.b1 = f1 < nb - 1 ? f1 : nb - 1;
    return s;
}

static inline float overlap(const Span* s, int b) {
    return fmx(fsub(fmn(s->hi, (float)b + 1.f), fmx(s->lo, (float)b)), 0.f);
}

/* Accumulates into map [2][nbx][nby] (map 0: nodes below num_mov, map 1: the rest). The caller zeroes it. */
void oracle_density_map(const float* pos, const float* size, const float* ratio, int num_nodes, int num_mov,
                        float bx, float by, int nbx, int nby, uint64_t* map) {
    float inv_bx = 1.f / bx, inv_by = 1.f / by;
    for (int i = 0; i < num_nodes; i++) {
        Span sx = span(pos[2 * i], size[2 * i], inv_bx, nbx), sy = span(pos[2 * i + 1], size[2 * i + 1], inv_by, nby);
        uint64_t* m = map + (i < num_mov ? 0 : (size_t)nbx * nby);
        for (int x = sx.b0; x <= sx.b1; x++) {
            float wx = fmul(ratio[i], overlap(&sx, x));
            for (int y = sy.b0; y <= sy.b1; y++)
                m[(size_t)x * nby + y] += f2u64((double)fmul(wx, overlap(&sy, y)) * DENSITY_SCALE);
        }
    }
}

/* rho [2 nbx][2 nby] (may be NULL), over [nbx][nby] (may be NULL); returns the sum of `over` in float64. */
double oracle_density_post(const uint64_t* map, const float* fixed, float target, int nbx, int nby, float* rho,
                           float* over) {
    size_t nb = (size_t)nbx * nby;
    double total = 0;
    int w = 2 * nby;
    for (int bx = 0; bx < nbx; bx++)
        for (int by = 0; by < nby; by++) {
            size_t b = (size_t)bx * nby + by;
            float mov = fadd((float)((double)map[b] / DENSITY_SCALE), fixed[b]);
            float r = fadd(mov, (float)((double)map[nb + b] / DENSITY_SCALE));
            float o = fmx(fsub(mov, target), 0.f);
            total += o;
            if (over) over[b] = o;
            if (rho) {
                int mx = 2 * nbx - 1 - bx, my = w - 1 - by;
                rho[(size_t)bx * w + by] = r; rho[(size_t)bx * w + my] = r;
                rho[(size_t)mx * w + by] = r; rho[(size_t)mx * w + my] = r;
            }
        }
    return total;
}

/* Gradient of every node from a field given as two planes (x, y) with row stride `ld` (2 nby for the mirrored
 * layout of the reference, nby for a plain [nbx][nby] field); float64 accumulation. */
void oracle_density_grad(const float* pos, const float* size, const float* ratio, const double* fx, const double* fy,
                         int ld, const float* wl_grad, int num_wl, const float* pins, const float* area, int num_nodes,
                         double weight, double precond, float bx, float by, int nbx, int nby, double* grad) {
    float inv_bx = 1.f / bx, inv_by = 1.f / by;
    for (int i = 0; i < num_nodes; i++) {
        Span sx = span(pos[2 * i], size[2 * i], inv_bx, nbx), sy = span(pos[2 * i + 1], size[2 * i + 1], inv_by, nby);
        double gx = 0, gy = 0;
        for (int x = sx.b0; x <= sx.b1; x++) {
            double wx = (double)ratio[i] * (double)overlap(&sx, x);
            for (int y = sy.b0; y <= sy.b1; y++) {
                double w = wx * (double)overlap(&sy, y);
                gx -= w * fx[(size_t)x * ld + y];
                gy -= w * fy[(size_t)x * ld + y];
            }
        }
        gx *= weight; gy *= weight;
        if (i < num_wl) { gx += wl_grad[2 * i]; gy += wl_grad[2 * i + 1]; }
        double scale = precond < 0 ? 1.0 : 1.0 / fmax((double)pins[i] + precond * (double)area[i], 1.0);
        grad[2 * i] = gx * scale;
        grad[2 * i + 1] = gy * scale;
    }
}
