// The field of the density map: Poisson's equation with zero normal field at the region boundary, solved by
// cosine / sine transforms written as GEMMs (GB300, sm_103a).
//
// Reference: src/core/electronic_density_layer.py:70-77,133 solves it by an FFT of the map mirrored to
// [2 nbx, 2 nby] (operator to_field: -i k / |k|^2 / bin_x, DC and Nyquist derivative zeroed) and reads the first
// quadrant. On the first quadrant that is exactly (frequencies p, q = 0 .. n - 1, C = cosine, S = sine matrices,
// C[p][u] = cos(pi p (2u + 1) / 2n)):
//     coefficients   K  = Cx A Cy^T
//     Ex = Sx^T (K * Wx) Cy,   Wx[p][q] = 2 / (nbx nby) * w_q * kx_p * inv[p][q]
//     Ey = Cx^T (K * Wy) Sy,   Wy[p][q] = 2 / (nbx nby) * w_p * ky_q * inv[p][q]
// with kx_p = pi p / (nbx bin_x), ky_q = pi q / (nby bin_y), inv = 1 / (kx^2 + ky^2) / bin_x (0 at p = q = 0), and
// w_0 = 1, w_q = 2 otherwise (the mirrored frequencies folded onto 0 .. n - 1).
//
// Six GEMMs, each D[M][N] = sum_k A[M][K] B[N][K] with both operands K-major; an epilogue writes each product in the
// layout its consumer reads (transposed where the next GEMM needs it as its B operand):
//   1  Tt[q][u]  = (A . Cy^T)^T            A = density [nbx][nby], B = Cy  [nby][nby]
//   2  K[p][q]   = Cx . T  -> Kx = K * Wx, Ky = K * Wy           A = Cx [nbx][nbx], B = Tt [nby][nbx]
//   3a Pt[n][p]  = (Kx . Cy)^T                                    A = Kx, B = CyT [nby][nby] (CyT[n][q] = Cy[q][n])
//   3b Ex[m][n]  = Sx^T . P                                       A = SxT [nbx][nbx], B = Pt
//   4a Qt[n][p]  = (Ky . Sy)^T                                    A = Ky, B = SyT [nby][nby]
//   4b Ey[m][n]  = Cx^T . Q                                       A = CxT [nbx][nbx], B = Qt
// With f16x3 on grids of multiples of 256 the tensor-core form folds the transforms (FieldLayout::fold): half the
// products, the frequencies in the folded order (even ones first), which the constants below follow.
// This file has the constants and the float32 CUDA-core GEMM (any grid); field_tc.cu has the tensor-core form.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <math.h>

#include "field.cuh"
#include "gp103.cuh"

namespace gp103 {

// ----------------------------------------------------------------------------- constants
// Matrices in float64 from exact integer argument reduction (cospi / sinpi of (p (2u + 1) mod 4n) / 2n).
__device__ __forceinline__ double trig(int kind, int p, int u, int n) {
    const long long r = ((long long)p * (2 * u + 1)) % (4LL * n);
    const double t = (double)r / (2.0 * n);
    return kind == 0 ? cospi(t) : sinpi(t);
}

// what: 0 = C[p][u], 1 = S[p][u], 2 = C^T[m][p] = C[p][m], 3 = S^T[m][p] = S[p][m]; f16 = 1: two float16 terms of
// the value times 2^F16_CONST instead of three bf16 terms; f16 = 2: two tf32 terms as float32 planes (t0, t1 point
// at float planes)
// The frequency of position c in the folded order of the coefficients (f16x3): the even frequencies 0, 2, .. first,
// then the odd ones 1, 3, ..
__device__ __forceinline__ int folded_freq(int c, int n) { return c < n / 2 ? 2 * c : 2 * (c - n / 2) + 1; }

// fold = 1 / 2: the (n/2) x (n/2) matrix of the even / odd frequencies of C over the lower half of the positions,
// F[r][u] = C[2r (+1)][u], u < n/2 (the forward transform of a folded input, below); pcols (what 2, 3): the
// frequency index of the transposed matrix in the folded order, T[m][c] = C[folded_freq(c)][m]
__global__ void trig_matrix_kernel(int what, int n, float* f32, __nv_bfloat16* t0, __nv_bfloat16* t1,
                                   __nv_bfloat16* t2, size_t plane, int f16, int fold, int pcols) {
    pdl_wait();
    const int m = fold ? n / 2 : n;                      // the matrix is m x m
    const size_t total = (size_t)m * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e / m), col = (int)(e % m);
        const int kind = what & 1;
        double v;
        if (fold) v = trig(0, 2 * r + fold - 1, col, n);
        else if (what < 2) v = trig(kind, r, col, n);
        else v = trig(kind, pcols ? folded_freq(col, n) : col, r, n);
        if (f32) f32[e] = (float)v;
        if (t0 && f16 == 2) {
            const float a = tf32_round((float)v);
            ((float*)t0)[e] = a;
            ((float*)t1)[e] = tf32_round((float)(v - (double)a));
        } else if (t0 && f16) {
            const double w = ldexp(v, F16_CONST);
            const __half a = __double2half(w);
            const __half b = __double2half(w - (double)__half2float(a));
            ((__half*)t0)[e] = a;
            ((__half*)t1)[e] = b;
        } else if (t0) {     // three bf16 terms of the float64 value
            const __nv_bfloat16 a = __double2bfloat16(v);
            const double r1 = v - (double)__bfloat162float(a);
            const __nv_bfloat16 b = __double2bfloat16(r1);
            const double r2 = r1 - (double)__bfloat162float(b);
            t0[e] = a;
            t1[e] = b;
            t2[e] = __double2bfloat16(r2);
        }
        (void)plane;
    }
}

__global__ void weight_kernel(int nbx, int nby, double bx, double by, float* wx, float* wy) {
    pdl_wait();
    const size_t total = (size_t)nbx * nby;
    const double pi = 3.14159265358979323846;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int p = (int)(e / nby), q = (int)(e % nby);
        const double kx = pi * p / (nbx * bx), ky = pi * q / (nby * by), k2 = kx * kx + ky * ky;
        const double inv = k2 > 0 ? 1.0 / k2 / bx : 0.0;
        const double scale = 2.0 / ((double)nbx * nby);
        wx[e] = (float)(scale * (q == 0 ? 1.0 : 2.0) * kx * inv);
        wy[e] = (float)(scale * (p == 0 ? 1.0 : 2.0) * ky * inv);
    }
}

// The separable parts of the weights, for epilogues that form them on the fly: per row p (kx^2, s kx / bin_x, w_p)
// and per column q (ky^2, s ky / bin_x, w_q), s = 2 / (nbx nby); Wx = (s kx / bin_x) w_q / (kx^2 + ky^2).
// (perm: entry c for the frequency folded_freq(c), the column order of the folded coefficients)
__global__ void weight_table_kernel(int n, int nbx, int nby, double bin, double bx, float4* tab, int perm) {
    pdl_wait();
    const double pi = 3.14159265358979323846;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int p = perm ? folded_freq(c, n) : c;
        const double k = pi * p / (n * bin), s = 2.0 / ((double)nbx * nby);
        tab[c] = make_float4((float)(k * k), (float)(s * k / bx), p == 0 ? 1.f : 2.f, 0.f);
    }
}

FieldLayout field_layout(int nbx, int nby, int mode) {
    FieldLayout L = {};
    L.nbx = nbx;
    L.nby = nby;
    L.mode = mode;
    L.fold = mode == GP103_FIELD_F16X3 && nbx % 256 == 0 && nby % 256 == 0;   // halves of whole 128-row tiles
    const size_t xx = (size_t)nbx * nbx, yy = (size_t)nby * nby, xy = (size_t)nbx * nby;
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o += (bytes + 1023) & ~(size_t)1023; return at; };
    // constants: the 6 operand matrices (float32 or 3 bf16 terms) and the two weight planes (float32)
    // bytes per element (all terms): float32; 3 x 16 bits (the 16-bit modes use 2 or 3 of them); tf32x3: 2 x 32 bits
    const size_t es = mode == GP103_FIELD_FP32 ? 4 : mode == GP103_FIELD_TF32X3 ? 8 : 3 * 2;
    L.c_cx = take(xx * es); L.c_cy = take(yy * es); L.c_cyt = take(yy * es);
    L.c_sxt = take(xx * es); L.c_syt = take(yy * es); L.c_cxt = take(xx * es);
    L.c_wx = take(xy * 4); L.c_wy = take(xy * 4);
    L.c_wrow = take((size_t)nbx * 16); L.c_wcol = take((size_t)nby * 16);
    L.const_bytes = o;
    o = 0;
    L.w_a = take(xy * es); L.w_tt = take(xy * es); L.w_kx = take(xy * es); L.w_ky = take(xy * es);
    L.w_pt = take(xy * es); L.w_qt = take(xy * es);
    L.w_err = take(1024);                                   // error flag of the tensor-core waits (int, zeroed)
    const size_t ex = mode == GP103_FIELD_F16X3 ? xy / 64 : 0;   // one byte per row and 64-wide chunk
    L.e_a = take(ex); L.e_tt = take(ex); L.e_kx = take(ex); L.e_ky = take(ex); L.e_pt = take(ex); L.e_qt = take(ex);
    L.work_bytes = o;
    return L;
}

int field_constants(const FieldLayout& L, void* cbuf, cudaStream_t s) {
    char* c = (char*)cbuf;
    const bool fp32 = L.mode == GP103_FIELD_FP32;
    // folded (f16x3): Cx and Cy as their even- and odd-frequency halves over the lower half of the positions (two
    // 2-term matrices of (n/2)^2 each, one after the other), the transposed matrices with their frequency columns in
    // the folded order
    const int fold = L.fold ? 1 : 0;
    const size_t half_cx = (size_t)(L.nbx / 2) * (L.nbx / 2) * 2 * 2;       // bytes of one folded half (2 terms)
    const size_t half_cy = (size_t)(L.nby / 2) * (L.nby / 2) * 2 * 2;
    struct M { int what, n; size_t off; int fold, pcols; } mats[8] = {
        {0, L.nbx, L.c_cx, fold, 0}, {0, L.nbx, L.c_cx + half_cx, 2, 0}, {0, L.nby, L.c_cy, fold, 0},
        {0, L.nby, L.c_cy + half_cy, 2, 0}, {2, L.nby, L.c_cyt, 0, fold}, {3, L.nbx, L.c_sxt, 0, fold},
        {3, L.nby, L.c_syt, 0, fold}, {2, L.nbx, L.c_cxt, 0, fold}};
    for (auto& m : mats) {
        if (m.fold == 2 && !fold) continue;                  // the odd half exists only in the folded layout
        const size_t plane = m.fold ? (size_t)(m.n / 2) * (m.n / 2) : (size_t)m.n * m.n;
        float* f = fp32 ? (float*)(c + m.off) : nullptr;
        __nv_bfloat16* t0 = fp32 ? nullptr : (__nv_bfloat16*)(c + m.off);
        const bool tf = L.mode == GP103_FIELD_TF32X3;            // two float32 planes
        __nv_bfloat16* t1 = !t0 ? nullptr : tf ? (__nv_bfloat16*)((float*)t0 + plane) : t0 + plane;
        __nv_bfloat16* t2 = !t0 || tf ? nullptr : t0 + 2 * plane;
        if (launch_k(trig_matrix_kernel, dim3(grid_for(plane, 256, 8)), dim3(256), 0, s, m.what, m.n, f, t0, t1, t2, plane,
                     tf ? 2 : (int)(L.mode == GP103_FIELD_F16X3), m.fold, m.pcols) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
    }
    if (launch_k(weight_kernel, dim3(grid_for((size_t)L.nbx * L.nby, 256, 8)), dim3(256), 0, s, L.nbx, L.nby, L.bx, L.by,
                                                                            (float*)(c + L.c_wx), (float*)(c + L.c_wy)) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (launch_k(weight_table_kernel, dim3(grid_for(L.nbx, 256, 8)), dim3(256), 0, s, L.nbx, L.nbx, L.nby, L.bx, L.bx,
                                                                 (float4*)(c + L.c_wrow), fold) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    if (launch_k(weight_table_kernel, dim3(grid_for(L.nby, 256, 8)), dim3(256), 0, s, L.nby, L.nbx, L.nby, L.by, L.bx,
                                                                 (float4*)(c + L.c_wcol), fold) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// ----------------------------------------------------------------------------- float32 CUDA-core GEMM
// 64 x 64 output tile per block, 256 threads x (4 x 4) outputs, k-tiles of 16 staged in shared memory. Each k-tile's
// 16 products are summed apart and then added to the output's running sum (two-level summation: the rounding error
// grows with K / 16 + 16 terms instead of K).
constexpr int SG_BM = 64, SG_BN = 64, SG_BK = 16;

__global__ void __launch_bounds__(256) sgemm_kernel(SGemm g) {
    pdl_wait();
    __shared__ float As[SG_BK][SG_BM + 4];
    __shared__ float Bs[SG_BK][SG_BN + 4];
    const int m0 = blockIdx.y * SG_BM, n0 = blockIdx.x * SG_BN;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < g.K; k0 += SG_BK) {
        for (int t = threadIdx.x; t < SG_BM * SG_BK; t += 256) {
            const int r = t / SG_BK, kk = t % SG_BK;
            const int m = m0 + r, n = n0 + r, k = k0 + kk;
            As[kk][r] = (m < g.M && k < g.K) ? g.A[(size_t)m * g.K + k] : 0.f;
            Bs[kk][r] = (n < g.N && k < g.K) ? g.B[(size_t)n * g.K + k] : 0.f;
        }
        __syncthreads();
        float part[4][4] = {};
#pragma unroll
        for (int kk = 0; kk < SG_BK; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) { a[i] = As[kk][ty * 4 + i]; b[i] = Bs[kk][tx * 4 + i]; }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int jj = 0; jj < 4; jj++) part[i][jj] = fmaf(a[i], b[jj], part[i][jj]);
        }
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int jj = 0; jj < 4; jj++) acc[i][jj] += part[i][jj];
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int jj = 0; jj < 4; jj++) {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + jj;
            if (m >= g.M || n >= g.N) continue;
            const float v = acc[i][jj];
            switch (g.epi) {
                case EPI_PLAIN: g.out0[(size_t)m * g.N + n] = v; break;
                case EPI_TRANS: g.out0[(size_t)n * g.M + m] = v; break;
                case EPI_WEIGHT2:
                    g.out0[(size_t)m * g.N + n] = v * g.w0[(size_t)m * g.N + n];
                    g.out1[(size_t)m * g.N + n] = v * g.w1[(size_t)m * g.N + n];
                    break;
            }
        }
}

int launch_sgemm(const SGemm& g, cudaStream_t s) {
    dim3 grid(ceil_div(g.N, SG_BN), ceil_div(g.M, SG_BM));
    if (launch_k(sgemm_kernel, dim3(grid), dim3(256), 0, s, g) != cudaSuccess) return GP103_ERR_CUDA;
    GP103_CHECK_LAUNCH();
    return GP103_OK;
}

// A caller's density less the plan's shift, into the work buffer's density plane (the field of the same map).
__global__ void shift_density_kernel(const float* d, size_t n, float shift, float* out) {
    pdl_wait();
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        out[e] = __fsub_rn(d[e], shift);
}

int field_fp32(const FieldLayout& L, const void* cbuf, void* wbuf, const float* density, float* ex, float* ey,
               cudaStream_t s) {
    const char* c = (const char*)cbuf;
    char* w = (char*)wbuf;
    const int X = L.nbx, Y = L.nby;
    auto F = [&](const char* base, size_t off) { return (const float*)(base + off); };
    auto W = [&](size_t off) { return (float*)(w + off); };
    if (density && L.shift != 0.f) {            // (the fused path's post kernel writes the shifted plane itself)
        if (launch_k(shift_density_kernel, dim3(grid_for((size_t)X * Y, 256, 8)), dim3(256), 0, s, density,
                     (size_t)X * Y, L.shift, W(L.w_a)) != cudaSuccess)
            return GP103_ERR_CUDA;
        GP103_CHECK_LAUNCH();
        density = nullptr;
    }
    const float* a = density ? density : W(L.w_a);
    int st;
    SGemm g1 = {X, Y, Y, a, F(c, L.c_cy), EPI_TRANS, W(L.w_tt), nullptr, nullptr, nullptr};
    if ((st = launch_sgemm(g1, s))) return st;
    SGemm g2 = {X, Y, X, F(c, L.c_cx), W(L.w_tt), EPI_WEIGHT2, W(L.w_kx), W(L.w_ky), F(c, L.c_wx), F(c, L.c_wy)};
    if ((st = launch_sgemm(g2, s))) return st;
    SGemm g3a = {X, Y, Y, W(L.w_kx), F(c, L.c_cyt), EPI_TRANS, W(L.w_pt), nullptr, nullptr, nullptr};
    if ((st = launch_sgemm(g3a, s))) return st;
    SGemm g3b = {X, Y, X, F(c, L.c_sxt), W(L.w_pt), EPI_PLAIN, ex, nullptr, nullptr, nullptr};
    if ((st = launch_sgemm(g3b, s))) return st;
    SGemm g4a = {X, Y, Y, W(L.w_ky), F(c, L.c_syt), EPI_TRANS, W(L.w_qt), nullptr, nullptr, nullptr};
    if ((st = launch_sgemm(g4a, s))) return st;
    SGemm g4b = {X, Y, X, F(c, L.c_cxt), W(L.w_qt), EPI_PLAIN, ey, nullptr, nullptr, nullptr};
    return launch_sgemm(g4b, s);
}

}  // namespace gp103
