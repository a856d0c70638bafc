/* gp103: GB300-native (sm_103a) electrostatic global-placement iteration behind a C ABI.
 *
 * Drop-in boundary for AutoPlace's `gp_cuda` operator module. Every entry point takes raw device pointers, sizes
 * and a CUDA stream, launches on that stream only (never the legacy default stream), allocates nothing, and returns
 * a status: 0 = ok, > 0 = GP103_ERR_* (bad argument, or the CUDA error of a launch). Float arrays of shape [n, 2]
 * are row-major (x, y) pairs, as in the reference. Device scalars (gamma, weights, step sizes) are read inside the
 * kernels: no host synchronisation.
 *
 * Part 1 mirrors the six host launchers of the reference (cpp_to_py/gp_cuda_kernel.cu) that its pybind11 module
 * (cpp_to_py/gp_cuda.cpp:78-85) exposes to Python; part 2 is the fused iteration this library runs itself.
 */
#ifndef GP103_H
#define GP103_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GP103_OK = 0,
    GP103_ERR_ARG = 1,       /* a size or pointer the kernels cannot take */
    GP103_ERR_CUDA = 2,      /* a launch failed (cudaGetLastError) */
    GP103_ERR_SHAPE = 3,     /* a grid the tensor-core field does not support */
    GP103_ERR_TOO_LARGE = 4  /* a size beyond a fixed limit of the library: the grid of gp103_density_map_noalloc
                              * (nbx * nby <= 262,144 bins), the 16,777,215 pins, nets or cells of the device
                              * problem build and of the net order */
};

/* Library version and the status text of an error code. */
int gp103_version(void);
const char* gp103_status_string(int status);

/* Process-wide options, read when a kernel is launched (a CUDA graph keeps the values of its capture).
 * GP103_OPT_PDL (default 1): launch with programmatic dependent launch, so that each kernel of a pass is launched
 *   while the previous one finishes (and graph edges become programmatic edges); 0 = plain stream order.
 * GP103_OPT_WAIT_MS (default 2000, 1 .. 60000): how long a wait of the tensor-core field (a TMA stage, an MMA, an
 *   accumulator) may take before the kernel gives it up: it then records the failure in the plan's device error
 *   flag (gp103_device_error), waits (at most 2 s) for its own copies and MMAs already in flight, frees its tensor
 *   memory and returns; later waits of the same launch give up at once, and no output is stored.
 * GP103_OPT_TEST_STALL_FIELD (default 0): a test hook. 1 = the field's TMA producer issues no load, so that every
 *   wait of the tensor-core field runs out (after GP103_OPT_WAIT_MS) with nothing in flight; it exists to test how
 *   a failure reaches the caller without faulting the GPU.
 * GP103_OPT_WA_FUSED (default 55, 0 .. 99): 0 = the WA kernels of a pass as two launches (short nets, then long
 *   ones); p > 0 = one launch of one resident wave, p % of its blocks on the long nets and the rest on the short
 *   ones, so that the two halves run side by side (every net's arithmetic is unchanged; the WA and HPWL totals are
 *   summed from other block partials). Measured at 1.2M cells: 0.0854 ms per pass in two launches, 0.0778 at 55.
 * GP103_OPT_FIELD_EARLY (default 3, bits): how a tensor-core field GEMM overlaps the kernel before it (with
 *   GP103_OPT_PDL). Bit 0: the constant operand (a cosine or sine matrix, written once by the field's set-up) of the
 *   first pipeline stages is loaded before the wait for the previous kernel; bit 1: the GEMMs that another GEMM
 *   follows let it launch as soon as their accumulation is done, so that its set-up and constant loads run beside
 *   their epilogue. The results are the same bits either way. */
enum { GP103_OPT_PDL = 0, GP103_OPT_WAIT_MS = 1, GP103_OPT_TEST_STALL_FIELD = 2, GP103_OPT_WA_FUSED = 3,
       GP103_OPT_FIELD_EARLY = 4 };
int gp103_set_option(int option, int value);

/* Kernel launches issued through this library so far (a launch captured into a CUDA graph counts once). */
unsigned long long gp103_launch_count(void);

/* Launch profile (single host thread): after gp103_profile_begin(stream), every launch records an event on its
 * stream; gp103_profile_end waits for the last one and writes each launch's duration (ms, event to event, so a
 * launch's time includes any gap before it) and the name of its launcher. Returns the number of launches profiled
 * (at most GP103_PROFILE_MAX), negative on a CUDA error. */
#define GP103_PROFILE_MAX 512
int gp103_profile_begin(cudaStream_t stream);
int gp103_profile_end(float* ms, const char** names, int max);

/* ------------------------------------------------------------------------------------------------ part 1
 * gp_cuda.wa (cpp_to_py/gp_cuda.cpp:31-38; launcher wa_wirelength, gp_cuda_kernel.cu:59-65).
 * Weighted-average wirelength of the nets [0, num_nets) grouped by net_start, gamma read from device memory.
 * pin_grad [P, 2] is scratch (P = net_start[num_nets]); out [num_nets, 2] = per-net (WA, HPWL); grad [num_mov, 2] =
 * per-cell sum of its pins' gradients in cell_pin order (cell_start [num_mov + 1]). A pin whose cell is >= num_mov
 * is fixed: its offset is its position. */
int gp103_wa(const float* pos, const int* pin_cell, const float* pin_off, const int* net_start, const int* cell_start,
             const int* cell_pin, int num_nets, int num_mov, const float* gamma, float* pin_grad, float* out,
             float* grad, cudaStream_t stream);

/* gp_cuda.density_map (gp_cuda.cpp:41-48; launcher density_map, gp_cuda_kernel.cu:141-146).
 * Fixed-point (2^32 per bin area) charge of nodes [0, num_nodes) into map [2, nbx, nby] (map 0: nodes < num_mov,
 * map 1: the rest; zeroed here first, it is scratch), then rho [2 nbx, 2 nby] = total density mirrored in both
 * axes and over [nbx, nby] = max(movable + fixed - target, 0). The map is the reference's integer map, bit for bit. */
int gp103_density_map(const float* pos, const float* size, const float* ratio, int num_nodes, int num_mov, float bx,
                      float by, int nbx, int nby, unsigned long long* map, const float* fixed, float target,
                      float* rho, float* over, cudaStream_t stream);

/* No counterpart in the reference. The density map of gp103_density_map (same results, bit for bit) for callers
 * that cannot allocate device memory: e.g. a plugin inside a host application whose device memory belongs to that
 * application's own pool, or a latency-critical loop that must not call cudaMalloc (it can synchronise the
 * device). Instead of a caller-provided map it uses a fixed 4 MiB device array inside this library, so grids are
 * limited to nbx * nby <= 262,144 bins (GP103_ERR_TOO_LARGE beyond, before any work). It allocates nothing: no
 * cudaMalloc, cudaFree or allocating library call. The first call on a device looks up the array's address
 * (make it before any stream capture); every call clears the part of the array it uses, all calls share the array,
 * and calls whose work overlaps on the GPU race on it. `stream` must belong to the current device (GP103_ERR_ARG
 * otherwise). The address stays cached for the process: after cudaDeviceReset of a device, do not call this entry
 * point on that device again. */
int gp103_density_map_noalloc(const float* pos, const float* size, const float* ratio, int num_nodes, int num_mov,
                              float bx, float by, int nbx, int nby, const float* fixed, float target, float* rho,
                              float* over, cudaStream_t stream);

/* gp_cuda.nesterov_step (gp_cuda.cpp:51-56; launcher nesterov_step, gp_cuda_kernel.cu:167-170).
 * n floats: u_next = v - alpha g; v_next = clamp(u_next + coef (u_next - u), lo, hi); alpha, coef on the device. */
int gp103_nesterov_step(const float* u, const float* v, const float* g, const float* lo, const float* hi,
                        const float* alpha, const float* coef, int n, float* u_next, float* v_next,
                        cudaStream_t stream);

/* gp_cuda.density_grad (gp_cuda.cpp:59-65; launcher density_grad, gp_cuda_kernel.cu:148-153).
 * grad[i] = (wl_grad[i] (i < num_wl) + weight * -(charge x field)) / max(1, pins[i] + precond area[i]) (precond < 0:
 * no division). field = two planes (x, y) of the mirrored map, each [2 nbx, 2 nby]; weight, precond on the device. */
int gp103_density_grad(const float* pos, const float* size, const float* ratio, const float* field,
                       const float* wl_grad, const float* pins, const float* area, int num_nodes, int num_wl,
                       const float* weight, const float* precond, float bx, float by, int nbx, int nby, float* grad,
                       cudaStream_t stream);

/* gp_cuda.control (gp_cuda.cpp:69-71; launcher control, gp_cuda_kernel.cu:251-254).
 * One pass of the run's control in float64: S [21] (layout FIELDS of src/gpu_loop.py:19-22) and kp [5] (gamma,
 * density weight, density weight of the preconditioner, alpha, coef) updated in place; c [13] constants (order of
 * src/gpu_loop.py:50-53); moved / turned / hpwl / ovf / wa are float32 device scalars of the pass. */
int gp103_control(double* S, float* kp, const double* c, const float* moved, const float* turned, const float* hpwl,
                  const float* ovf, const float* wa, cudaStream_t stream);

/* gp_cuda.select (gp_cuda.cpp:74-76; launcher select_step, gp_cuda_kernel.cu:256-259).
 * n floats: if S[accept]: u, v, g <- next; if S[is_best]: best <- v_next. */
int gp103_select(const double* S, float* u, float* v, float* g, const float* u_next, const float* v_next,
                 const float* g_next, float* best, int n, cudaStream_t stream);

/* ------------------------------------------------------------------------------------------------ part 2
 * The fused iteration. The caller owns all memory: it fills a gp103_plan with device pointers (sizes from
 * gp103_plan_sizes) and captures gp103_pass calls in a CUDA graph if it wants one. */

/* Field precision of the Poisson solve. */
enum {
    GP103_FIELD_FP32 = 0,     /* cosine / sine transforms as float32 CUDA-core GEMMs (any grid) */
    GP103_FIELD_BF16X3 = 1,   /* tensor cores (tcgen05), bf16 operands split in 2 terms, 3 products, fp32 accumulation */
    GP103_FIELD_BF16X6 = 2,   /* tensor cores, bf16 operands split in 3 terms, 6 products (error ~1e-7 of the max) */
    GP103_FIELD_F16X3 = 3,    /* tensor cores, float16 operands split in 2 terms, 3 products, each row's 64-wide chunk
                               * of K scaled by its own power of two (error ~1e-7 of the max, half the products) */
    GP103_FIELD_TF32X3 = 4    /* tensor cores (tcgen05 kind::tf32), float32 operands split in 2 tf32 terms (each the
                               * value rounded to 10 mantissa bits, then the rest), 3 products, fp32 accumulation */
};

/* Phases of gp103_pass. */
enum {
    GP103_PHASE_START = 0,    /* wirelength-only start (density weight 0), src/run_placement.py:60-65 */
    GP103_PHASE_DENSITY = 1,  /* the device loop of src/gpu_loop.py:58-68 */
    GP103_PASS_SORT = 0x100,  /* or-ed to GP103_PHASE_DENSITY: refresh plan->order from this pass's positions */
    GP103_PASS_JOIN_FIELD = 0x200 /* or-ed, gp103_pass_split only: `stream` waits for the WA kernels before the field
                                   * instead of before the gather (the WA kernels share the GPU with the density map
                                   * only; the field has all of it) */
};

/* Layout of the start-phase state T [32] (float64): what NesterovOptimizer (alpha, a) and
 * ParamScheduler.start_step (src/param_scheduler.py:42-48) keep during the wirelength-only start. */
enum {
    GP103_T_ALPHA = 0, GP103_T_A = 1, GP103_T_ITER = 2, GP103_T_LOOP_IT = 3, GP103_T_DONE = 4, GP103_T_STOP = 5,
    GP103_T_ACCEPT = 6, GP103_T_HPWL = 7, GP103_T_WA = 8, GP103_T_EVALS = 9, GP103_T_NWA = 10,
    GP103_T_START_TOL = 11, GP103_T_INNER = 12, GP103_T_RING = 16 /* 6 slots: the last WA values */,
    GP103_T_SIZE = 32
};

typedef struct {
    /* sizes */
    int num_nodes, num_mov, num_nets, num_pins;
    int nbx, nby;             /* force grid */
    int jnbx, jnby;           /* overflow grid; 0 = the force grid measures the overflow */
    int field_mode;           /* GP103_FIELD_* */
    /* netlist, grouped by net (nets in any order) and by cell (cell_pin = positions in the pin arrays) */
    const int* pin_cell; const float* pin_off; const int* net_start; const int* cell_start; const int* cell_pin;
    /* nodes */
    const float* size; const float* ratio; const float* pins; const float* area; const float* lo; const float* hi;
    float bx, by, target;
    const float* fixed;       /* [nbx, nby] */
    double ovf_scale;         /* bin area / movable area of the overflow grid */
    /* overflow grid (when jnbx > 0): smoothed sizes of the cells on it */
    const float* jsize; const float* jratio; const float* jfixed; float jbx, jby; double jovf_scale;
    /* field constants (gp103_field_constants fills them) and the field planes */
    void* field_const;        /* gp103_plan_sizes(...).field_const bytes */
    void* field_work;         /* gp103_plan_sizes(...).field_work bytes */
    float* ex; float* ey;     /* [nbx, nby] */
    /* optimiser state: ping-pong buffers, *cur = the current one; best placement */
    float* u[2]; float* v[2]; float* g[2]; float* best; int* cur;
    double* S;                /* [21] density phase (layout of the reference) */
    double* T;                /* [GP103_T_SIZE] start phase */
    float* kp;                /* [5] */
    const double* c;          /* [13] constants of the density phase */
    /* scratch */
    float* pin_grad;          /* [num_pins, 2] */
    unsigned long long* map;  /* [2, nbx, nby], zero between passes */
    unsigned long long* jmap; /* [jnbx, jnby], zero between passes */
    double* red;              /* gp103_plan_sizes(...).red doubles */
    unsigned int* counters;   /* 16, zero */
    /* layout of the pin gradients: when pin_slot is given, the gradient of pin p is stored at pin_slot[p], the
     * position of p in cell order (cell_start ranges), and cell_pin is not read */
    const int* pin_slot;
    int net_split;            /* nets [net_split, num_nets) are long: one warp each (num_nets: any order) */
    /* spatial order of the nodes for the scatter (optional; all three or none): order [num_nodes], a permutation
     * of 0..num_nodes-1 (fill it with 0, 1, ... before the first pass; density passes with GP103_PASS_SORT refresh
     * it, the others only read it), order_counts [2048] (zero), order_cursor [2048]. Any permutation gives the same
     * density map; a recent spatial one gives a faster scatter. */
    int* order; int* order_counts; int* order_cursor;
    /* nets [net_split, net_mid) have 9 to 16 pins: four lanes each, eight nets per warp (net_mid = 0: none, every
     * long net takes a warp) */
    int net_mid;
    /* nets [0, net_two) have 2 pins and nets [net_two, net_three) 3 pins, their pins from 0 on in net order (the
     * order gp103_net_order makes): their first pins follow from the net index, net_start is not read for them.
     * net_three = 0: not known, net_start is read for every net. */
    int net_two; int net_three;
    /* subtracted from the density before the field's transforms (0: nothing). The field is the same either way: a
     * constant changes only the zero-frequency coefficient, which the field drops. Set it to the grid's mean density
     * (node area / bin area + the fixed map, over the bins: the charge is conserved while the nodes stay inside the
     * region), so that the transforms' rounding follows the density's variation, not its mean -- on a spread
     * placement, where the density is near its mean everywhere, the error against float64 falls by that ratio. */
    float field_shift;
    /* nets [net_mid, net_g8) have 17 to 32 pins (eight lanes each, four nets per warp), [net_g8, net_g16) 33 to 64
     * (sixteen lanes each, two per warp), the rest a warp each (net_g16 = 0: every net from net_mid on a warp) */
    int net_g8; int net_g16;
    /* the share (percent, 1 .. 99) of the fused WA launch's blocks that take the long nets (net_split on) in this
     * plan's passes; 0: the process option GP103_OPT_WA_FUSED's (which, at 0, makes every plan's WA two launches).
     * The best share follows the share of the pins on long nets: measured at 1.2M cells (38 % of the pins on nets of
     * 9 pins or more) 50-55, on its 272k clusters (53 %) 60-65. */
    int wa_long_share;
} gp103_plan;

typedef struct {
    size_t field_const;       /* bytes */
    size_t field_work;        /* bytes */
    size_t red;               /* doubles */
} gp103_sizes;

/* Byte offsets of gp103_plan's fields in declaration order (arrays count once), for bindings that lay the struct
 * out themselves; returns the number of fields, writes at most n offsets and then sizeof(gp103_plan) if room. */
int gp103_plan_offsets(size_t* out, int n);

/* Sizes of the plan's buffers for a force grid nbx x nby and a field mode; GP103_ERR_SHAPE if the mode does not
 * support the grid (tensor-core modes: nbx and nby multiples of 128). */
int gp103_plan_sizes(int nbx, int nby, int field_mode, gp103_sizes* out);

/* Fill plan->field_const (cosine / sine matrices, in the operand layout of the mode). Once per grid. */
int gp103_field_constants(const gp103_plan* plan, cudaStream_t stream);

/* One iteration of the phase (all kernels, on `stream`). The scalar results of the pass stay on the device; the
 * reductions behind them are float64 and bit-reproducible. */
int gp103_pass(const gp103_plan* plan, int phase, cudaStream_t stream);

/* The gradient of the objective at pos ([num_nodes, 2]) into g_out, with the density weight `weight` (0: the
 * wirelength-only gradient, the density map and field are not computed) and preconditioner weight `precond`
 * (< 0: none), both host values; -1 for wl_scale skips the wirelength term (the plain density gradient of
 * tension_unit). Writes out3 = (sum of squares of g_out - g_ref or 0 if g_ref is NULL, WA, HPWL, overflow,
 * L1 norm of g_out over the cells) as 5 doubles. gamma is read from plan->kp[0]. */
int gp103_eval(const gp103_plan* plan, const float* pos, float* g_out, const float* g_ref, double weight,
               double precond, int with_wl, double* out5, cudaStream_t stream);

/* probe = clamp(v - step * g, lo, hi) for the whole node set; out[0] = sum of squares of probe - v. */
int gp103_probe(const gp103_plan* plan, const float* v, const float* g, double step, float* probe, double* out1,
                cudaStream_t stream);

/* The field of a plain density map a [nbx, nby] (float32) into ex, ey [nbx, nby] with the plan's field mode. */
int gp103_field(const gp103_plan* plan, const float* density, float* ex, float* ey, cudaStream_t stream);

/* gp103_pass with two streams (density passes; a wirelength-only pass runs on `stream` alone): the WA kernels run on
 * `side`, which waits for the step (event `fork`, recorded on `stream`), while `stream` runs the spatial sort, the
 * density map and the field; `stream` waits for them (event `join`, recorded on `side`) before the gather. The two
 * halves of a pass share the GPU; the results are those of gp103_pass. Captured in a CUDA graph, the events become
 * the graph's fork and join. fork, join: two distinct events (gp103_event_create), side != stream. */
int gp103_pass_split(const gp103_plan* plan, int phase_flags, cudaStream_t stream, cudaStream_t side, void* fork,
                     void* join);
/* An event for gp103_pass_split (cudaEventDisableTiming), and its release. */
int gp103_event_create(void** event);
int gp103_event_destroy(void* event);

/* The scalars of a level's set-up (gp103_begin). */
typedef struct {
    double lr;                /* the first probe's step (--lr) */
    double gamma;             /* WA smoothing */
    double lam;               /* density weight: <= 0 a fresh run (the wirelength-only start follows), > 0 resumed */
    double start_tol;         /* the start phase's rule: relative WA decrease per pass ... */
    double inner_iter;        /* ... and its limit of passes (fresh runs) */
    double iter;              /* the scheduler's iteration count */
    double loop_it;           /* the level's first loop iteration */
    double hpwl_prev;         /* resumed: the last HPWL */
} gp103_begin_args;

/* A level's set-up before its first pass, queued on `stream` with no host synchronisation: the two probe steps of the
 * step length (estimate_initial_learning_rate and NesterovOptimizer.__init__, src/nesterov_optimizer.py:56-63 and :15-32; four
 * gradient evaluations at v[0], the start positions, and two probes of v[0] along g[0]) and the first phase's state.
 * kp = (gamma, lam, lam, 0, 0) and *cur = 0 first; the gradients with the density weight lam and preconditioner
 * weight lam when lam > 0 (else the wirelength-only gradient); u[0] = v[0]; the step length into scal8[7] (the first
 * probe's into scal8[6]; scal8: 8 device doubles, scratch too), tmp0 and tmp1 [num_nodes, 2] scratch. Then for a
 * fresh run T = the wirelength-only start's state and kp = (gamma, 0, 0, alpha, 0); resumed, S = the density phase's
 * state (lam, gamma, alpha, a = 1, iter, hpwl_prev, mu 1, best HPWL and overflow +inf, loop_it), kp = (gamma, lam,
 * lam, alpha, 0) and best = v[0]. Float64 scalars by correctly rounded operations, the same bits as on the host. */
int gp103_begin(const gp103_plan* plan, const gp103_begin_args* args, float* tmp0, float* tmp1, double* scal8,
                cudaStream_t stream);

/* The hand-over from the wirelength-only start to the density phase, queued on `stream` with no host
 * synchronisation (src/run_placement.py:60-64 with the state set-up of src/gpu_loop.py:38-48): the plain density
 * gradient at v[*cur] (gp103_eval's kernels with weight 1, precond -1, no wirelength term; into g_tmp
 * [num_nodes, 2], its 5 totals into out5, device doubles), then on the device the first density weight
 * lam = density_weight x (total_pins / out5[4]) (the tension unit), S = the density phase's state (lam, gamma, the
 * step length, momentum, iteration, last HPWL and loop count of T; mu 1; best HPWL and overflow +inf; the rest 0),
 * kp = (gamma, lam, lam, alpha, Nesterov coefficient) in float32 and best = v[*cur]. If the start phase stopped the
 * run (T[GP103_T_STOP] != 0), only S[14] = T[GP103_T_STOP] is written, and density passes change nothing. */
int gp103_start_to_density(const gp103_plan* plan, double density_weight, double total_pins, double gamma,
                           float* g_tmp, double* out5, cudaStream_t stream);

/* After the last pass: copy the pending best placement (S[is_best] of the last control) from v[*cur]. */
int gp103_finish(const gp103_plan* plan, cudaStream_t stream);

/* The plan's device error flag: 0, or the wait of the tensor-core field that ran out first (1 = a TMA stage's
 * slot, 2 = an accumulator's buffer, 3 = a TMA stage's data, 4 = an accumulator's result). The flag is set by the
 * field's kernels (the outputs of that launch are not written), cleared by gp103_field_constants and, with
 * clear != 0, here. The control kernel of every pass reads it: a set flag stops the run with stop reason 6 (S[14]
 * in the density phase, T[GP103_T_STOP] in the start phase). Copies the flag to *code after the work queued on
 * `stream` (a host synchronisation of the stream). Always 0 in field mode GP103_FIELD_FP32 (no bounded waits). */
int gp103_device_error(const gp103_plan* plan, int clear, int* code, cudaStream_t stream);

/* Set-up of the fused path on the device: the nets of the optimised pin set (Wirelength._pin_set,
 * src/core/wa_wirelength_hpwl.py:38-46; net_start [num_nets + 1], pin_cell [num_pins] with num_mov for a fixed pin,
 * pin_off [num_pins, 2], cell_pin [num_pins] = the pins in cell order) reordered for the WA kernels: a stable sort
 * of the nets by (class, lowest cell), classes 2 pins / 3 pins / 4-8 / 9-16 / 17-32 / 33-64 pins / longer, pins
 * moving with their nets.
 * Writes net_start_out, pin_cell_out, pin_off_out (the plan's net_start, pin_cell, pin_off), pin_slot (each new
 * pin's position in cell order: the plan's pin_slot) and split (device int [6]: the plan's net_split, net_mid,
 * net_two, net_three, net_g8 and net_g16 = numbers of nets of up to 8, up to 16, 2, up to 3, up to 32 and up to 64
 * pins). scratch: gp103_net_order_scratch(...) bytes. No counterpart in the reference, whose kernel reads the nets
 * in their original order. GP103_ERR_TOO_LARGE beyond 7 (num_mov + 1) > 16,777,216. */
size_t gp103_net_order_scratch(int num_nets, int num_pins, int num_mov);
int gp103_net_order(const int* net_start, const int* pin_cell, const float* pin_off, const int* cell_pin,
                    int num_nets, int num_pins, int num_mov, void* scratch, size_t scratch_bytes,
                    int* net_start_out, int* pin_cell_out, float* pin_off_out, int* pin_slot, int* split,
                    cudaStream_t stream);

/* Clustering of the cells (src/cluster.py:38-85, cluster_cells), the first step of the two-level placement: rounds
 * of star matching on the pair edges of the small nets. Integer weights and areas, fixed tie rules: the clusters are
 * the reference's, bit for bit. Scratch: gp103_cluster_scratch(n, num_nets, max_edges) bytes, max_edges >= the
 * number of ordered pin pairs of the nets of 2 .. max_degree pins (sum of d (d - 1)).
 *
 * gp103_cluster_edges: the pair edges of the pins (pin_cell [num_pins] with n for a fixed pin, pin_net sorted by
 * net, nets < num_nets) as a CSR over the n cells: row_start [n + 1], col / w [max_edges], columns ascending per row,
 * w = the summed 420 / (degree - 1). counts (device int [2]): [0] = edges, [1] = ordered pairs found (above
 * max_edges: the bound was too small and the edges are not valid).
 *
 * gp103_cluster_round: one round on `num` clusters (their edges in CSR, areas int64, head [num] = 1 for the heads of
 * the round, drawn by the caller): writes new_index [num] (each cluster's index among the kept ones), area_out
 * [num] (the first counts[0] valid), the new edges row_out [num + 1] / col_out / w_out (counts[1] of them) and
 * counts (device int [2]) = (clusters kept, edges). counts[0] == num: nothing merged (the reference stops there).
 *
 * gp103_cluster_relabel: cid[c] = new_index[cid[c]] for the n cells after a round that merged. */
size_t gp103_cluster_scratch(int n, int num_nets, int max_edges);
int gp103_cluster_edges(const int* pin_cell, const int* pin_net, int num_pins, int num_nets, int n, int max_degree,
                        int max_edges, void* scratch, size_t scratch_bytes, int* row_start, int* col, int* w,
                        int* counts, cudaStream_t stream);
int gp103_cluster_round(const int* row_start, const int* col, const int* w, int num, int max_edges,
                        const long long* area, const unsigned char* head, long long cap, long long big, int per_head,
                        void* scratch, size_t scratch_bytes, int* new_index, long long* area_out, int* row_out,
                        int* col_out, int* w_out, int* counts, cudaStream_t stream);
int gp103_cluster_relabel(int* cid, int n, const int* new_index, cudaStream_t stream);

/* The clusters of cluster_cells' result (cid [n] in 0..num-1, carea [num] int64 in 1/1024 of a site area): count
 * [num] (scratch, zeroed here) the members of each, single [num] = 1 for a cluster of one cell, csize [num, 2] float32
 * = the cell's own size for a one-cell cluster, else float32(sqrt(carea / 1024)) on both sides (coarse_problem,
 * src/cluster.py:102-107: a merged cluster is the square of its summed area). size [n, 2]: the cells' sizes. */
int gp103_cluster_members(const int* cid, int n, int num, const long long* carea, const float* size, int* count,
                          unsigned char* single, float* csize, cudaStream_t stream);

/* The pins of the cluster problem (coarse_problem, src/cluster.py:88-130): every pin of every net (pin_cell with n
 * for a fixed pin, pin_off [num_pins, 2], pin_net sorted by net) mapped to its cluster (cid [n]; num for a fixed
 * pin); a pin on a one-cell cluster (single [num] = 1) or a fixed pin is kept with its offset, otherwise only the first
 * pin of its net on its cluster is kept, at the cluster's centre. Writes the kept pins in order (out_cell, out_off,
 * out_net) and their number to count (device int). Scratch: gp103_coarse_pins_scratch(num_pins) bytes. */
size_t gp103_coarse_pins_scratch(int num_pins);
int gp103_coarse_pins(const int* pin_cell, const float* pin_off, const int* pin_net, int num_pins, int n, const int* cid,
                      int num, const unsigned char* single, void* scratch, size_t scratch_bytes, int* out_cell,
                      float* out_off, int* out_net, int* count, cudaStream_t stream);

/* expand (src/cluster.py:133-144): pos[c] = cpos[cid[c]] + (draws[c] - 0.5) max(csize[cid[c]] - size[c], 0) for the n
 * cells, float32 in the reference's operation order; draws [n, 2] are the caller's uniform draws (the reference's
 * seeded CPU generator). The fillers' positions are the caller's to copy. */
int gp103_expand(const float* cpos, const int* cid, const float* csize, const float* size, const float* draws, int n,
                 float* pos, cudaStream_t stream);

/* The seeded draws of the clustering's heads (src/cluster.py:62, a share of 0.5) and of expand (src/cluster.py:142),
 * on the device: out[0 .. count) = the float32 values of torch.rand(count, generator=torch.Generator().manual_seed(
 * seed)) on the CPU, the same bits (the generator's MT19937 stream, each 32-bit output x giving (x mod 2^24) 2^-24;
 * consecutive torch.rand calls on one generator continue this one stream). One block; count any size. */
int gp103_seeded_uniform(unsigned long long seed, long long count, float* out, cudaStream_t stream);

/* Problem build on the device: the arrays AutoPlace builds once per level before the first iteration.
 *
 * gp103_build_csr: the optimised pin set (Wirelength.__init__ net filter and Wirelength._pin_set,
 * src/core/wa_wirelength_hpwl.py:26-46) from the netlist's pins sorted by net (pin_cell [num_pins] with num_mov for a
 * fixed pin, pin_off [num_pins, 2], pin_net [num_pins] ascending, nets < num_nets): nets of 2 .. ignore_degree pins
 * renumbered in order; net_start [num_nets + 1] (the first num_opt + 1 written), cell32 / off [num_pins] (the first
 * num_opt_pins written), cell_start [num_mov + 1], cell_pin [num_pins] (a stable argsort of cell32), all_net_start
 * [num_nets + 1] (every net's first pin, for the exact HPWL), cell_pins [num_mov] (pins per movable cell over every
 * pin). counts (device int [4]) = (num_opt, num_opt_pins, error bits: 1 = pin_net unsorted or out of range, 2 = a
 * cell out of [0, num_mov], pins on movable cells). Integer work and copies: the host build's arrays, bit for bit.
 * scratch: gp103_build_csr_scratch(...) bytes. GP103_ERR_TOO_LARGE beyond 16,777,215 pins, nets or cells. */
size_t gp103_build_csr_scratch(int num_pins, int num_nets, int num_mov);
int gp103_build_csr(const int* pin_cell, const float* pin_off, const int* pin_net, int num_pins, int num_nets,
                    int num_mov, int ignore_degree, void* scratch, size_t scratch_bytes, int* net_start, int* cell32,
                    float* off, int* cell_start, int* cell_pin, int* all_net_start, int* cell_pins, int* counts,
                    cudaStream_t stream);

/* gp103_smooth_nodes: the n nodes (size [n, 2] float64) as one density grid sees them (ElectronicDensityLayer
 * smoothing, src/core/electronic_density_layer.py:36-58): size_s = float32(max(size, (min_x, min_y))) with min =
 * sqrt(2) x the bin, ratio = float32(real area / smoothed area) in float64, lo = size_s / 2 and hi = (width, height) -
 * lo in float32 (lo, hi may be NULL); area = float32(real area) and pins = float32(cell_pins[i]) for the num_mov cells,
 * 0 for the rest (each may be NULL). */
int gp103_smooth_nodes(const double* size, int n, int num_mov, double min_x, double min_y, float width, float height,
                       float* size_s, float* ratio, float* lo, float* hi, float* area, const int* cell_pins,
                       float* pins, cudaStream_t stream);

/* The fixed share of every bin of an nbx x nby grid over a width x height region (PlaceData.fixed_fraction,
 * src/database.py:103-134, in the form it takes when the rows cover the region and the fixed rectangles -- rects
 * [count][4] = (x0, y0, x1, y1), float64 -- do not overlap): per bin the rectangles' overlap area, in rectangle order,
 * over the bin area, clipped to [0, 1]; fraction [nbx][nby] float64. The same bits as the host statement (numpy:
 * the per-rectangle outer products of the x and y overlaps, summed in order). */
int gp103_macro_fraction(const double* rects, int count, double width, double height, int nbx, int nby,
                         double* fraction, cudaStream_t stream);

/* ------------------------------------------------------------------------------------------------ part 3
 * Exact evaluators in float64 (the exact HPWL and overflow of a placement). `scratch` is GP103_EVAL_SCRATCH_BYTES of
 * device memory; *out is written by the device (read it after synchronising the stream). */
#define GP103_EVAL_SCRATCH_BYTES 16640

/* HPWL over every net (Wirelength.hpwl, src/core/wa_wirelength_hpwl.py:66-70): pin position pos[pin_cell] +
 * pin_off (pin_off alone for pin_cell >= num_mov: a fixed pin), per net max - min on each axis, all in float64.
 * Nets in net_start order [num_nets + 1]; empty nets add 0. */
int gp103_hpwl(const float* pos, const int* pin_cell, const float* pin_off, const int* net_start, int num_nets,
               int num_mov, void* scratch, double* out, cudaStream_t stream);

/* Overflow of the movable cells with their real sizes (ElectronicDensityLayer.exact_overflow,
 * src/core/electronic_density_layer.py:112-116): fixed-point map of the cells at ratio 1 on an nbx x nby grid of
 * bins bx x by, out = sum over bins of max(map + fixed - target, 0) in float64, times area_scale (bin area /
 * movable area). map: u64 [nbx, nby], zero on entry, zero again on return. */
int gp103_exact_overflow(const float* pos, const float* size, int num_mov, float bx, float by, int nbx, int nby,
                         const float* fixed, float target, double area_scale, unsigned long long* map,
                         void* scratch, double* out, cudaStream_t stream);

/* ------------------------------------------------------------------------------------------------ part 4
 * The learned start (no counterpart in the reference, whose clusters start at the seeded start positions,
 * src/run_placement.py:98, and run the wirelength-only start, src/run_placement.py:48-65): a message-passing network
 * over the cluster graph proposes the clusters' start positions. The graph is a netlist in the fused path's form:
 * pins grouped by net (net_start [num_nets + 1], pin_cell [num_pins], a cell >= num_cells being a fixed pin at its
 * pin_off) and by cell (cell_start [num_cells + 1], cell_pin [num_pins]). Deterministic: gathers in fixed order, no
 * atomics. Dense layers take bf16 weights (row-major [in][out]) and accumulate in fp32; widths <= 64. */

/* The weights of the graph's four gathers, each [num_pins]: net order (P2N and its transpose): net_pin_cell (the
 * pin's cell, -1 for a fixed pin), w_p2n = 1 / the net's movable pins, w_n2ct = 1 / the pins of the pin's cell; cell
 * order (N2C and its transpose): cell_pin_net (the pin's net), w_n2c = 1 / the cell's pins, w_p2nt = 1 / the movable
 * pins of the pin's net. scratch: gp103_learn_graph_scratch(num_nets, num_pins) bytes. */
size_t gp103_learn_graph_scratch(int num_nets, int num_pins);
int gp103_learn_graph(const int* net_start, const int* pin_cell, const int* cell_start, const int* cell_pin,
                      int num_nets, int num_cells, int num_pins, void* scratch, size_t scratch_bytes,
                      int* net_pin_cell, float* w_p2n, float* w_n2ct, int* cell_pin_net, float* w_n2c, float* w_p2nt,
                      cudaStream_t stream);

/* out[s][0:width] (+)= sum over k in [seg_start[s], seg_start[s + 1]) of w[k] * src[idx[k]][0:width], in k order
 * (idx[k] < 0: skipped; accumulate != 0: added to out). width 1 .. 64. */
int gp103_seg_gather(const int* seg_start, int num_seg, const int* idx, const float* w, const float* src, int width,
                     int accumulate, float* out, cudaStream_t stream);

/* out[i][c] = act(bias[c] + sum_j x[i][j] wx[j][c] + sum_j a[i][j] wa[j][c]) for n rows, c < out_dim; act 0 = none,
 * 1 = relu, 2 = sigmoid; in_a = 0: no second input. Weights bf16 (uint16 bit patterns), bias fp32. */
int gp103_dense_fwd(const float* x, int n, int in_x, const float* a, int in_a, const uint16_t* wx, const uint16_t* wa,
                    const float* bias, int out_dim, int act, float* out, cudaStream_t stream);

/* The backward of gp103_dense_fwd given its output `out` and the gradient dout: dz = dout * act'(out) [n][out_dim];
 * dx = dz wx^T, da = dz wa^T (either may be NULL); weight gradients gwx [in_x][out_dim], gwa, gbias (fp32, the rows'
 * sum in a fixed order: per-block partials in `scratch`, gp103_dense_bwd_scratch bytes, added in block order). */
size_t gp103_dense_bwd_scratch(int in_x, int in_a, int out_dim);
int gp103_dense_bwd(const float* x, int n, int in_x, const float* a, int in_a, const uint16_t* wx, const uint16_t* wa,
                    int out_dim, int act, const float* out, const float* dout, float* dz, float* dx, float* da,
                    void* scratch, size_t scratch_bytes, float* gwx, float* gwa, float* gbias, cudaStream_t stream);

/* Mean squared error: loss[0] = mean over the n rows of sum_d (y - t)^2 (float64, device), dy = 2 (y - t) / n.
 * scratch: GP103_EVAL_SCRATCH_BYTES. */
int gp103_mse(const float* y, const float* t, int n, int dim, float* dy, double* loss, void* scratch,
              cudaStream_t stream);

/* One Adam step (bias-corrected, decoupled weight decay) on fp32 parameters, also writing their bf16 copy. */
int gp103_adam(float* param, const float* grad, float* m, float* v, uint16_t* param_bf16, int n, float lr, float beta1,
               float beta2, float eps, int step, float weight_decay, cudaStream_t stream);

/* The 10 input features of every cell of the graph [num_cells][10]: log(area / mean_area), log(1 + nets) / 4,
 * log(1 + pin_count) / 4 (pin_count NULL: the cell's pins), the anchor (x / width, y / height: at hop 0 the mean of
 * the fixed pins on the cell's nets, then, hop by hop up to max_hop, the mean over each net's anchored cells averaged
 * over the cell's nets; the centre when none), hop / max_hop (1 when none), 1 if anchored, the anchor's distance from
 * the centre, and the harmonic coordinates: from the anchors, `sweeps` Jacobi sweeps in which every cell takes the
 * mean over its nets of each net's mean pin position (fixed pins held where they are). The gather weights come from
 * gp103_learn_graph. scratch: gp103_learn_features_scratch bytes. */
size_t gp103_learn_features_scratch(int num_nets, int num_cells);
int gp103_learn_features(const int* net_start, const int* pin_cell, const float* pin_off, const int* cell_start,
                         int num_nets, int num_cells, int num_pins, const int* net_pin_cell, const float* w_p2n,
                         const int* cell_pin_net, const float* w_n2c, const float* area, const float* pin_count,
                         double mean_area, float width, float height, int max_hop, int sweeps, void* scratch,
                         size_t scratch_bytes, float* feat, cudaStream_t stream);

/* ------------------------------------------------------------------------------------------------ part 5
 * Batches of independent placement instances in one CUDA graph (no counterpart in the reference, which runs one
 * design per process and polls the host every 16 passes, src/gpu_loop.py:58-70). Each instance is a conditional WHILE
 * node of the graph: its body is `passes` passes of the instance's plan (the first one refreshing the spatial order
 * when sort_first, density phase) and a condition kernel that ends the loop once the instance's control stops it
 * (S[14] != 0 in the density phase; T[GP103_T_DONE] or T[GP103_T_STOP] in the start phase) or after max_loops bodies.
 * The instances are separate branches, so the GPU runs them side by side. *loops (device int, zero it before each
 * launch) counts an instance's bodies; *stop_ns (device) receives the device time (ns) at which its loop ended.
 * gp103_batch_add captures the passes on `capture` (a stream of the plan's device, not the legacy default stream);
 * the plans and their buffers must outlive the batch. gp103_batch_launch instantiates the graph on its first call and
 * launches it on `stream`, after writing the device time to *t0_ns (when not NULL). An add that fails after its
 * argument checks may leave part of an instance in the graph: gp103_batch_launch then refuses the batch
 * (GP103_ERR_ARG), and the caller destroys it. */
int gp103_batch_create(void** batch);
int gp103_batch_add(void* batch, const gp103_plan* plan, int phase, int passes, int sort_first, int max_loops,
                    int* loops, unsigned long long* stop_ns, cudaStream_t capture);
/* A whole placement of one instance in the batch's graph: when `begin` is not NULL, an IF node that runs gp103_begin
 * once (begin, tmp0, tmp1, scal8 as there; the start positions must be in v[0] when the graph is launched); then the
 * start phase's WHILE node (start_passes per body, at most max_start_loops bodies), an IF node that runs
 * gp103_start_to_density once (density_weight, total_pins, gamma; tmp0 as g_tmp, scal8 as out5), and the density
 * phase's WHILE node (density_passes per body, the first refreshing the spatial order, at most max_density_loops
 * bodies). loops[0], stop_ns[0] belong to the start loop, loops[1], stop_ns[1] to the density loop. No host step
 * from the set-up to the stop. */
int gp103_batch_add_run(void* batch, const gp103_plan* plan, const gp103_begin_args* begin, int start_passes,
                        int density_passes, int max_start_loops, int max_density_loops, double density_weight,
                        double total_pins, double gamma, float* tmp0, float* tmp1, double* scal8, int* loops,
                        unsigned long long* stop_ns, cudaStream_t capture);
int gp103_batch_launch(void* batch, unsigned long long* t0_ns, cudaStream_t stream);
int gp103_batch_destroy(void* batch);

#ifdef __cplusplus
}
#endif
#endif
