// Field (Poisson solve) declarations: buffer layout of the constants and the work planes, GEMM descriptions.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace gp103 {

// Byte offsets inside the plan's field_const / field_work buffers. Every operand is either one float32 plane
// (GP103_FIELD_FP32) or three bf16 planes back to back (tensor-core modes; the bf16x3 mode reads two of them).
struct FieldLayout {
    int nbx, nby, mode;
    double bx, by;
    size_t c_cx, c_cy, c_cyt, c_sxt, c_syt, c_cxt, c_wx, c_wy, c_wrow, c_wcol, const_bytes;
    size_t w_a, w_tt, w_kx, w_ky, w_pt, w_qt, w_err, work_bytes;
};

// PLAIN: float32 [M][N]; TRANS: float32 [N][M] (CUDA-core GEMM); WEIGHT2: the two weighted products of the field;
// SPLIT: the three bf16 terms of the product, [3][M][N] (tensor-core GEMM)
enum { EPI_PLAIN = 0, EPI_TRANS = 1, EPI_WEIGHT2 = 2, EPI_SPLIT = 3 };

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
