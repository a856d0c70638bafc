// Field (Poisson solve) declarations: buffer layout of the constants and the work planes, GEMM descriptions.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace gp103 {

// Byte offsets inside the plan's field_const / field_work buffers. Every operand is either one float32 plane
// (GP103_FIELD_FP32) or up to three 16-bit planes back to back (tensor-core modes: bf16x6 three bf16 terms, bf16x3
// two of them, f16x3 two float16 terms). In f16x3 every data operand also has a power-of-two scale per row and
// 64-wide chunk of K: x_e[kb][n] = e, the terms hold x * 2^e (the constant matrices are scaled by 2^F16_CONST).
// fold (f16x3, nbx and nby multiples of 256): both forward transforms take their input folded about its middle and
// give the even and odd frequencies separately (C[p][n-1-u] = (-1)^p C[p][u]): half the products of each. The first
// (along y) takes the density folded about the middle of y, s = a(y) + a(nby-1-y) and d = a(y) - a(nby-1-y) for
// y < nby/2; its epilogue folds its output about the middle of x for the second. Both frequencies then run in the
// folded order (even ones first, then odd), which the constants that meet them follow.
struct FieldLayout {
    int nbx, nby, mode;
    bool fold;
    double bx, by;
    float shift;                // subtracted from a float32 density before the transforms (the same field)
    size_t c_cx, c_cy, c_cyt, c_sxt, c_syt, c_cxt, c_wx, c_wy, c_wrow, c_wcol, const_bytes;
    size_t w_a, w_tt, w_kx, w_ky, w_pt, w_qt, w_err;
    size_t e_a, e_tt, e_kx, e_ky, e_pt, e_qt, work_bytes;     // f16x3 chunk exponents (signed char)
};

constexpr int F16_CONST = 14;     // f16x3: the cosine / sine matrices (|c| <= 1) are stored times 2^14
constexpr int F16_TOP = 14;       // f16x3: a chunk of data is scaled so that its largest magnitude is in [2^14, 2^15)
constexpr int F16_EMAX = 100;     // f16x3: chunk exponents are clamped to [-100, 100] (all factors stay normal)

// PLAIN: float32 [M][N]; TRANS: float32 [N][M] (CUDA-core GEMM); WEIGHT2: the two weighted products of the field;
// SPLIT: the 16-bit terms of the product, [terms][M][N] (tensor-core GEMM); FOLD (f16x3): the product's columns in
// mirrored pairs (B rows n and N-1-n), the float16 terms of their sums and of their differences, [terms][M][N/2] each;
// MSPLIT / MPLAIN (f16x3): an inverse transform over a depth in the folded frequency order, rows m < M_out/2 computed
// as E (the even frequencies, the first half of K) and O (the odd ones): row m = E + O, row M_out-1-m = msign (E - O),
// out as SPLIT / PLAIN
enum { EPI_PLAIN = 0, EPI_TRANS = 1, EPI_WEIGHT2 = 2, EPI_SPLIT = 3, EPI_FOLD = 4, EPI_MSPLIT = 5, EPI_MPLAIN = 6 };

struct SGemm {
    int M, N, K;
    const float* A;     // [M][K]
    const float* B;     // [N][K]
    int epi;
    float* out0; float* out1;
    const float* w0; const float* w1;
};

FieldLayout field_layout(int nbx, int nby, int mode);
int field_constants(const FieldLayout& L, void* cbuf, cudaStream_t s);
int launch_sgemm(const SGemm& g, cudaStream_t s);
int field_fp32(const FieldLayout& L, const void* cbuf, void* wbuf, const float* density, float* ex, float* ey,
               cudaStream_t s);
// Tensor-core field: the density's bf16 terms are in the work buffer (w_a) unless `density` is given.
int field_tc(const FieldLayout& L, const void* cbuf, void* wbuf, const float* density, float* ex, float* ey,
             cudaStream_t s);
bool field_tc_supported(int nbx, int nby);

}  // namespace gp103
