// Step / control declarations (state layout of the reference's control kernel).
#pragma once
#include "gp103.cuh"
#include "kernels.cuh"

namespace gp103 {

// State S [21]: the order of FIELDS in src/gpu_loop.py:19-22 (and of the enum of control_kernel).
enum {
    S_LAM, S_GAM, S_ALPHA, S_A, S_ITER, S_HPWL_PREV, S_MOTION, S_WW, S_MU, S_SETTLED, S_BEST_HPWL, S_BEST_OVF,
    S_IS_BEST, S_IMPROVED, S_STOP, S_ACCEPT, S_LOOP_IT, S_EVALS, S_RES_HPWL, S_RES_OVF, S_HAS_BEST, S_SIZE
};
// Constants c [13]: the order of src/gpu_loop.py:50-53.
enum {
    C_BASE_GAMMA, C_MOTION_UNIT, C_TOTAL_PINS, C_TOTAL_AREA, C_PITCH, C_MIN_ITER, C_STOP_OVF, C_SETTLE, C_STALL,
    C_INNER, C_REFINE, C_ACCURACY, C_HANDOVER, C_SIZE
};

struct StepJob {
    float* u[2]; float* v[2]; float* g[2];
    const int* cur;             // null: buffers 0 are current
    const float* lo; const float* hi;
    const float* kp;            // kp[3] = alpha, kp[4] = coef
    const double* S;            // S[is_best] of the previous pass: copy v[cur] to best (null: never)
    float* best;
    int n;                      // nodes
    Reduce red;                 // |v' - v|^2
    OrderJob ord;               // counts of the spatial order of v' (ord.counts null: none)
};

int launch_nesterov_step(const float* u, const float* v, const float* g, const float* lo, const float* hi,
                         const float* alpha, const float* coef, int n, float* u_next, float* v_next, cudaStream_t s);
int launch_control(double* S, float* kp, const double* c, const float* moved, const float* turned, const float* hpwl,
                   const float* ovf, const float* wa, cudaStream_t s);
int launch_select(const double* S, float* u, float* v, float* g, const float* u_next, const float* v_next,
                  const float* g_next, float* best, int n, cudaStream_t s);
int launch_step(const StepJob& j, cudaStream_t s);
// step_p (device, or null): the step as a float64 written by an earlier kernel, instead of `step`
int launch_probe(const float* v, const float* g, const float* lo, const float* hi, float step, int n, float* probe,
                 Reduce red, cudaStream_t s, const double* step_p = nullptr);
// The scalars of a level's set-up (begin_kernel, sqrt_ratio_kernel, first_state_kernel) and a device copy.
int launch_begin(float* kp, int* cur, double gamma, double lam, cudaStream_t s);
int launch_sqrt_ratio(const double* a, const double* b, double* out, cudaStream_t s);
int launch_copy(const float* src, float* dst, int n, cudaStream_t s);
int launch_first_state(double* T, double* S, float* kp, float* best, const float* v, int n, const double* alpha_p,
                       double gamma, double lam, double start_tol, double inner, double iter, double loop_it,
                       double hpwl_prev, cudaStream_t s);
// ferr: the tensor-core field's device error flag (or null): when set, the control stops the run with reason
// STOP_DEVICE_ERROR and changes nothing else.
constexpr int STOP_DEVICE_ERROR = 6;
int launch_control_fused(double* S, float* kp, const double* c, Reduce grad, const double* pre, double ovf_scale,
                         int* cur, const int* ferr, cudaStream_t s);
int launch_control_start(double* T, float* kp, Reduce grad, const double* pre, int* cur, const int* ferr,
                         cudaStream_t s);
int launch_finish(const double* S, const int* cur, const float* v0, const float* v1, float* best, int n,
                  cudaStream_t s);
// The start-to-density hand-over of the state (handover_kernel); l1: the device L1 norm of the tension unit.
int launch_handover(const double* T, double* S, float* kp, const int* cur, const float* v0, const float* v1,
                    float* best, const double* l1, double total_pins, double density_weight, double gamma, int n,
                    cudaStream_t s);
int launch_totals(const Reduce* r, const int* k, int n, double* out, cudaStream_t s);
// out[0] = value 0 of r times mul
int launch_scale_total(const Reduce& r, double mul, double* out, cudaStream_t s);

}  // namespace gp103
