// The C ABI of libgp103 (include/gp103.h): argument checks and launch order; no allocation, no host sync.
#include <string.h>

#include "field.cuh"
#include "gp103.cuh"
#include "kernels.cuh"
#include "step.cuh"

using namespace gp103;

#define REQUIRE(cond)                    \
    do {                                 \
        if (!(cond)) return GP103_ERR_ARG; \
    } while (0)
#define TRY(call)                        \
    do {                                 \
        int st_ = (call);                \
        if (st_) return st_;             \
    } while (0)

// ------------------------------------------------------------------------------------------------ options
static int g_pdl = 1;
static int g_wait_ms = 2000;
static int g_stall = 0;
static int g_wa_share = 55;
static int g_field_early = 3;
bool gp103::pdl_enabled() { return g_pdl != 0; }
int gp103::field_early() { return g_field_early; }
long long gp103::tc_wait_ns() { return (long long)g_wait_ms * 1000000LL; }
bool gp103::tc_test_stall() { return g_stall != 0; }
int gp103::wa_long_share() { return g_wa_share; }

extern "C" int gp103_set_option(int option, int value) {
    switch (option) {
        case GP103_OPT_PDL: g_pdl = value != 0; return GP103_OK;
        case GP103_OPT_WAIT_MS:
            REQUIRE(value >= 1 && value <= 60000);
            g_wait_ms = value;
            return GP103_OK;
        case GP103_OPT_TEST_STALL_FIELD: g_stall = value != 0; return GP103_OK;
        case GP103_OPT_WA_FUSED:
            REQUIRE(value >= 0 && value <= 99);
            g_wa_share = value;
            return GP103_OK;
        case GP103_OPT_FIELD_EARLY:
            REQUIRE(value >= 0 && value <= 3);
            g_field_early = value;
            return GP103_OK;
        default: return GP103_ERR_ARG;
    }
}

// ------------------------------------------------------------------------------------------------ launch accounting
static unsigned long long g_launches = 0;
static struct {
    cudaEvent_t ev[GP103_PROFILE_MAX + 1];
    const char* name[GP103_PROFILE_MAX + 1];
    int n, open;
} g_prof;

int gp103::after_launch(cudaStream_t s, const char* name) {
    if (cudaGetLastError() != cudaSuccess) return GP103_ERR_CUDA;
    __atomic_add_fetch(&g_launches, 1ull, __ATOMIC_RELAXED);
    if (g_prof.open && g_prof.n <= GP103_PROFILE_MAX) {
        if (cudaEventRecord(g_prof.ev[g_prof.n], s) != cudaSuccess) return GP103_ERR_CUDA;
        g_prof.name[g_prof.n++] = name;
    }
    return GP103_OK;
}

extern "C" unsigned long long gp103_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

extern "C" int gp103_profile_begin(cudaStream_t s) {
    REQUIRE(!g_prof.open);
    for (int i = 0; i <= GP103_PROFILE_MAX; i++)
        if (!g_prof.ev[i] && cudaEventCreate(&g_prof.ev[i]) != cudaSuccess) return GP103_ERR_CUDA;
    if (cudaEventRecord(g_prof.ev[0], s) != cudaSuccess) return GP103_ERR_CUDA;
    g_prof.name[0] = "begin";
    g_prof.n = 1;
    g_prof.open = 1;
    return GP103_OK;
}

extern "C" int gp103_profile_end(float* ms, const char** names, int max) {
    REQUIRE(g_prof.open);
    g_prof.open = 0;
    if (cudaEventSynchronize(g_prof.ev[g_prof.n - 1]) != cudaSuccess) return -GP103_ERR_CUDA;
    int k = 0;
    for (int i = 1; i < g_prof.n && k < max; i++, k++) {
        if (cudaEventElapsedTime(&ms[k], g_prof.ev[i - 1], g_prof.ev[i]) != cudaSuccess) return -GP103_ERR_CUDA;
        names[k] = g_prof.name[i];
    }
    return k;
}

extern "C" int gp103_version(void) { return 1; }

extern "C" const char* gp103_status_string(int status) {
    switch (status) {
        case GP103_OK: return "ok";
        case GP103_ERR_ARG: return "invalid argument (null pointer, negative size or empty grid)";
        case GP103_ERR_CUDA: return "a CUDA launch failed";
        case GP103_ERR_SHAPE: return "grid not supported by the tensor-core field (multiples of 128 bins per side)";
        case GP103_ERR_TOO_LARGE:
            return "size beyond a fixed limit (gp103_density_map_noalloc: nbx * nby <= 262144 bins; device problem "
                   "build and net order: <= 16,777,215 pins, nets or cells)";
        default: return "unknown status";
    }
}

// ------------------------------------------------------------------------------------------------ part 1
extern "C" int gp103_wa(const float* pos, const int* pin_cell, const float* pin_off, const int* net_start,
                        const int* cell_start, const int* cell_pin, int num_nets, int num_mov, const float* gamma,
                        float* pin_grad, float* out, float* grad, cudaStream_t stream) {
    REQUIRE(num_nets >= 0 && num_mov >= 0 && net_start && gamma && cell_start);
    // an optimised net has >= 2 pins: no nets <=> no pins (the pin arrays may then be empty / null)
    REQUIRE(num_nets == 0 || (pin_cell && pin_off && pin_grad && out && pos && cell_pin));
    REQUIRE(num_mov == 0 || grad);
    if (num_nets > 0) {
        WaJob j = {};
        j.pos_a = j.pos_b = (const float2*)pos;
        j.pin_cell = pin_cell;
        j.pin_off = (const float2*)pin_off;
        j.net_start = net_start;
        j.num_nets = num_nets;
        j.num_mov = num_mov;
        j.split = num_nets;
        j.mid = j.g8 = j.g16 = num_nets;
        j.gamma = gamma;
        j.pin_grad = (float2*)pin_grad;
        j.out = (float2*)out;
        TRY(launch_wa_net(j, stream));
    }
    return launch_wa_cell((const float2*)pin_grad, cell_start, cell_pin, num_mov, (float2*)grad, stream);
}

extern "C" int gp103_density_map(const float* pos, const float* size, const float* ratio, int num_nodes, int num_mov,
                                 float bx, float by, int nbx, int nby, unsigned long long* map, const float* fixed,
                                 float target, float* rho, float* over, cudaStream_t stream) {
    REQUIRE(num_nodes >= 0 && num_mov >= 0 && nbx > 0 && nby > 0 && map && fixed && rho && over);
    REQUIRE(num_nodes == 0 || (pos && size && ratio));
    REQUIRE(bx > 0.f && by > 0.f);
    const int mov = num_mov < num_nodes ? num_mov : num_nodes;
    if (cudaMemsetAsync(map, 0, sizeof(unsigned long long) * 2 * (size_t)nbx * nby, stream) != cudaSuccess)
        return GP103_ERR_CUDA;
    ScatterJob j = {};
    j.pos_a = j.pos_b = (const float2*)pos;
    j.size = (const float2*)size;
    j.ratio = ratio;
    j.num_nodes = num_nodes;
    j.num_mov = mov;
    j.inv_bx = 1.f / bx;
    j.inv_by = 1.f / by;
    j.nbx = nbx;
    j.nby = nby;
    j.map0 = map;
    j.map1 = map + (size_t)nbx * nby;
    TRY(launch_scatter(&j, 1, stream));
    return launch_post_mirror(map, fixed, target, nbx, nby, rho, over, stream);
}

extern "C" int gp103_nesterov_step(const float* u, const float* v, const float* g, const float* lo, const float* hi,
                                   const float* alpha, const float* coef, int n, float* u_next, float* v_next,
                                   cudaStream_t stream) {
    REQUIRE(n >= 0 && alpha && coef);
    REQUIRE(n == 0 || (u && v && g && lo && hi && u_next && v_next));
    return launch_nesterov_step(u, v, g, lo, hi, alpha, coef, n, u_next, v_next, stream);
}

extern "C" int gp103_density_grad(const float* pos, const float* size, const float* ratio, const float* field,
                                  const float* wl_grad, const float* pins, const float* area, int num_nodes,
                                  int num_wl, const float* weight, const float* precond, float bx, float by, int nbx,
                                  int nby, float* grad, cudaStream_t stream) {
    REQUIRE(num_nodes >= 0 && num_wl >= 0 && nbx > 0 && nby > 0 && weight && precond && bx > 0.f && by > 0.f);
    REQUIRE(num_nodes == 0 || (pos && size && ratio && field && pins && area && grad));
    REQUIRE(num_wl == 0 || wl_grad);
    return launch_gather_mirror(pos, size, ratio, field, wl_grad, pins, area, num_nodes, num_wl, weight, precond, bx,
                                by, nbx, nby, grad, stream);
}

extern "C" int gp103_control(double* S, float* kp, const double* c, const float* moved, const float* turned,
                             const float* hpwl, const float* ovf, const float* wa, cudaStream_t stream) {
    REQUIRE(S && kp && c && moved && turned && hpwl && ovf && wa);
    return launch_control(S, kp, c, moved, turned, hpwl, ovf, wa, stream);
}

extern "C" int gp103_select(const double* S, float* u, float* v, float* g, const float* u_next, const float* v_next,
                            const float* g_next, float* best, int n, cudaStream_t stream) {
    REQUIRE(S && n >= 0);
    REQUIRE(n == 0 || (u && v && g && u_next && v_next && g_next && best));
    return launch_select(S, u, v, g, u_next, v_next, g_next, best, n, stream);
}

// ------------------------------------------------------------------------------------------------ part 2
static FieldLayout layout_of(const gp103_plan* p) {
    FieldLayout L = field_layout(p->nbx, p->nby, p->field_mode);
    L.bx = p->bx;
    L.by = p->by;
    L.shift = p->field_shift;
    return L;
}

extern "C" int gp103_plan_offsets(size_t* out, int n) {
#define OFF(f) offsetof(gp103_plan, f)
    const size_t off[] = {
        OFF(num_nodes), OFF(num_mov), OFF(num_nets), OFF(num_pins), OFF(nbx), OFF(nby), OFF(jnbx), OFF(jnby),
        OFF(field_mode), OFF(pin_cell), OFF(pin_off), OFF(net_start), OFF(cell_start), OFF(cell_pin), OFF(size),
        OFF(ratio), OFF(pins), OFF(area), OFF(lo), OFF(hi), OFF(bx), OFF(by), OFF(target), OFF(fixed),
        OFF(ovf_scale), OFF(jsize), OFF(jratio), OFF(jfixed), OFF(jbx), OFF(jby), OFF(jovf_scale), OFF(field_const),
        OFF(field_work), OFF(ex), OFF(ey), OFF(u), OFF(v), OFF(g), OFF(best), OFF(cur), OFF(S), OFF(T), OFF(kp),
        OFF(c), OFF(pin_grad), OFF(map), OFF(jmap), OFF(red), OFF(counters), OFF(pin_slot), OFF(net_split),
        OFF(order), OFF(order_counts), OFF(order_cursor), OFF(net_mid), OFF(net_two), OFF(net_three),
        OFF(field_shift), OFF(net_g8), OFF(net_g16), OFF(wa_long_share)};
#undef OFF
    const int count = (int)(sizeof(off) / sizeof(off[0]));
    for (int i = 0; i < count && i < n; i++) out[i] = off[i];
    if (n > count) out[count] = sizeof(gp103_plan);
    return count;
}

extern "C" int gp103_plan_sizes(int nbx, int nby, int field_mode, gp103_sizes* out) {
    REQUIRE(out && nbx > 0 && nby > 0);
    REQUIRE(field_mode == GP103_FIELD_FP32 || field_mode == GP103_FIELD_BF16X3 || field_mode == GP103_FIELD_BF16X6 ||
            field_mode == GP103_FIELD_F16X3 || field_mode == GP103_FIELD_TF32X3);
    if (field_mode != GP103_FIELD_FP32 && !field_tc_supported(nbx, nby)) return GP103_ERR_SHAPE;
    FieldLayout L = field_layout(nbx, nby, field_mode);
    out->field_const = L.const_bytes;
    out->field_work = L.work_bytes;
    out->red = RED_DOUBLES;
    return GP103_OK;
}

static int check_plan(const gp103_plan* p) {
    REQUIRE(p && p->num_nodes >= 0 && p->num_mov >= 0 && p->num_mov <= p->num_nodes && p->num_nets >= 0);
    REQUIRE(p->nbx > 0 && p->nby > 0 && p->bx > 0.f && p->by > 0.f);
    REQUIRE(p->field_mode >= GP103_FIELD_FP32 && p->field_mode <= GP103_FIELD_TF32X3);
    REQUIRE(p->field_const && p->field_work && p->ex && p->ey && p->red && p->counters && p->map && p->kp);
    REQUIRE(p->jnbx == 0 || (p->jnby > 0 && p->jmap && p->jsize && p->jratio && p->jfixed));
    REQUIRE(p->net_split >= 0 && p->net_split <= p->num_nets);
    REQUIRE(p->net_mid == 0 || (p->net_mid >= p->net_split && p->net_mid <= p->num_nets));
    REQUIRE(p->net_g16 == 0 || (p->net_mid > 0 && p->net_g8 >= p->net_mid && p->net_g16 >= p->net_g8 &&
                                p->net_g16 <= p->num_nets));
    REQUIRE(p->net_three == 0 || (p->net_two >= 0 && p->net_two <= p->net_three && p->net_three <= p->net_split &&
                                  2LL * p->net_two + 3LL * (p->net_three - p->net_two) <= (long long)p->num_pins));
    REQUIRE(p->pin_slot || p->cell_pin || p->num_pins == 0);
    REQUIRE(p->wa_long_share >= 0 && p->wa_long_share <= 99);
    REQUIRE((p->order == nullptr) == (p->order_counts == nullptr) && (p->order == nullptr) == (p->order_cursor == nullptr));
    if (p->field_mode != GP103_FIELD_FP32 && !field_tc_supported(p->nbx, p->nby)) return GP103_ERR_SHAPE;
    return GP103_OK;
}

// The device error flag of the tensor-core field's waits (inside the field work buffer), or null (fp32 field).
static int* field_error_flag(const gp103_plan* p) {
    if (p->field_mode == GP103_FIELD_FP32) return nullptr;
    return (int*)((char*)p->field_work + layout_of(p).w_err);
}

extern "C" int gp103_field_constants(const gp103_plan* plan, cudaStream_t stream) {
    TRY(check_plan(plan));
    if (int* f = field_error_flag(plan))
        if (cudaMemsetAsync(f, 0, sizeof(int), stream) != cudaSuccess) return GP103_ERR_CUDA;
    return field_constants(layout_of(plan), plan->field_const, stream);
}

extern "C" int gp103_device_error(const gp103_plan* plan, int clear, int* code, cudaStream_t stream) {
    TRY(check_plan(plan));
    REQUIRE(code);
    *code = 0;
    int* f = field_error_flag(plan);
    if (!f) return GP103_OK;
    if (cudaMemcpyAsync(code, f, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess) return GP103_ERR_CUDA;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return GP103_ERR_CUDA;
    if (clear && *code != 0 && cudaMemsetAsync(f, 0, sizeof(int), stream) != cudaSuccess) return GP103_ERR_CUDA;
    return GP103_OK;
}

static int run_field(const gp103_plan* p, const float* density, cudaStream_t s) {
    const FieldLayout L = layout_of(p);
    if (p->field_mode == GP103_FIELD_FP32) return field_fp32(L, p->field_const, p->field_work, density, p->ex, p->ey, s);
    return field_tc(L, p->field_const, p->field_work, density, p->ex, p->ey, s);
}

extern "C" int gp103_field(const gp103_plan* plan, const float* density, float* ex, float* ey, cudaStream_t stream) {
    TRY(check_plan(plan));
    REQUIRE(density && ex && ey);
    gp103_plan q = *plan;
    q.ex = ex;
    q.ey = ey;
    return run_field(&q, density, stream);
}

// Density map(s) at the chosen positions, post-processing, field: the force grid's plain density goes straight into
// the field's first operand (float32 plane or bf16 terms).
// The spatial order of the scatter: tiles of T x T force-grid bins, T = max(32, ceil(max(nbx, nby) / 32)), so
// that there are at most 32 x 32 tiles per node class.
static OrderJob order_job(const gp103_plan* p) {
    OrderJob o = {};
    const int nmax = p->nbx > p->nby ? p->nbx : p->nby;
    int T = (nmax + 31) / 32;
    if (T < 32) T = 32;
    o.counts = p->order_counts;
    o.cursor = p->order_cursor;
    o.order = p->order;
    o.tiles_x = (p->nbx + T - 1) / T;
    o.tiles_y = (p->nby + T - 1) / T;
    o.inv_tx = 1.f / (T * p->bx);
    o.inv_ty = 1.f / (T * p->by);
    o.num_nodes = p->num_nodes;
    o.num_mov = p->num_mov;
    return o;
}

static int density_and_field(const gp103_plan* p, const float* pos_a, const float* pos_b, const int* sel,
                             const int* order, cudaStream_t s, const WaJob* wa = nullptr,
                             cudaEvent_t before_field = nullptr) {
    const size_t nb = (size_t)p->nbx * p->nby;
    ScatterJob sj = {};
    sj.pos_a = (const float2*)pos_a;
    sj.pos_b = (const float2*)pos_b;
    sj.sel = sel;
    sj.size = (const float2*)p->size;
    sj.ratio = p->ratio;
    sj.num_nodes = p->num_nodes;
    sj.num_mov = p->num_mov;
    sj.inv_bx = 1.f / p->bx;
    sj.inv_by = 1.f / p->by;
    sj.nbx = p->nbx;
    sj.nby = p->nby;
    sj.map0 = p->map;
    sj.map1 = p->map + nb;
    sj.order = order;
    ScatterJob jobs[2] = {sj, sj};
    if (p->jnbx > 0) {
        ScatterJob& jj = jobs[1];
        jj.size = (const float2*)p->jsize;
        jj.ratio = p->jratio;
        jj.num_nodes = p->num_mov;
        jj.inv_bx = 1.f / p->jbx;
        jj.inv_by = 1.f / p->jby;
        jj.nbx = p->jnbx;
        jj.nby = p->jnby;
        jj.map0 = p->jmap;
        jj.map1 = nullptr;
    }
    TRY(launch_scatter(jobs, p->jnbx > 0 ? 2 : 1, s));
    const FieldLayout L = layout_of(p);
    PostJob pj = {};
    pj.map = p->map;
    pj.fixed = p->fixed;
    pj.target = p->target;
    pj.nbx = p->nbx;
    pj.nby = p->nby;
    pj.with_fill = 1;
    pj.shift = p->field_shift;
    if (p->field_mode == GP103_FIELD_FP32) {
        pj.dens = (float*)((char*)p->field_work + L.w_a);
    } else if (p->field_mode == GP103_FIELD_TF32X3) {
        pj.tf0 = (float*)((char*)p->field_work + L.w_a);
        pj.tf1 = pj.tf0 + nb;
    } else {
        __nv_bfloat16* t = (__nv_bfloat16*)((char*)p->field_work + L.w_a);
        pj.t0 = t;
        pj.t1 = t + nb;
        pj.t2 = t + 2 * nb;
        pj.terms = 3;
        if (p->field_mode == GP103_FIELD_F16X3) {
            pj.terms = 2;
            pj.exps = (signed char*)((char*)p->field_work + L.e_a);
            pj.fold = L.fold ? 1 : 0;
        }
    }
    pj.red = reduce_slot(p->red, p->counters, R_OVF);
    PostJob posts[2] = {pj, pj};
    if (p->jnbx > 0) {
        PostJob& jp = posts[1];
        jp = PostJob{};
        jp.map = p->jmap;
        jp.fixed = p->jfixed;
        jp.target = p->target;
        jp.nbx = p->jnbx;
        jp.nby = p->jnby;
        jp.red = reduce_slot(p->red, p->counters, R_JOVF);
    }
    TRY(launch_post_plain(posts, p->jnbx > 0 ? 2 : 1, s));
    if (wa) TRY(launch_wa_net(*wa, s));                     // (see run_pass)
    if (before_field && cudaStreamWaitEvent(s, before_field, 0) != cudaSuccess) return GP103_ERR_CUDA;
    return run_field(p, nullptr, s);
}

static GatherJob gather_job(const gp103_plan* p) {
    GatherJob g = {};
    g.size = (const float2*)p->size;
    g.ratio = p->ratio;
    g.pins = p->pins;
    g.area = p->area;
    g.num_nodes = p->num_nodes;
    g.num_mov = p->num_mov;
    g.inv_bx = 1.f / p->bx;
    g.inv_by = 1.f / p->by;
    g.nbx = p->nbx;
    g.nby = p->nby;
    g.pin_grad = (const float2*)p->pin_grad;
    g.cell_start = p->cell_start;
    g.cell_pin = p->pin_slot ? nullptr : p->cell_pin;
    g.red = reduce_slot(p->red, p->counters, R_GRAD);
    return g;
}

static WaJob wa_job(const gp103_plan* p) {
    WaJob w = {};
    w.pin_cell = p->pin_cell;
    w.pin_off = (const float2*)p->pin_off;
    w.net_start = p->net_start;
    w.num_nets = p->num_nets;
    w.num_mov = p->num_mov;
    w.split = p->net_split;
    w.mid = p->net_mid > 0 ? p->net_mid : p->net_split;
    w.g8 = p->net_g16 > 0 ? p->net_g8 : w.mid;
    w.g16 = p->net_g16 > 0 ? p->net_g16 : w.mid;
    w.two = p->net_three > 0 ? p->net_two : 0;
    w.three = p->net_three;
    w.slot = p->pin_slot;
    w.gamma = p->kp;
    w.pin_grad = (float2*)p->pin_grad;
    w.red = reduce_slot(p->red, p->counters, R_WA);
    w.long_share = p->wa_long_share;
    return w;
}

extern "C" int gp103_event_create(void** event) {
    REQUIRE(event);
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return GP103_ERR_CUDA;
    *event = (void*)e;
    return GP103_OK;
}

extern "C" int gp103_event_destroy(void* event) {
    REQUIRE(event);
    return cudaEventDestroy((cudaEvent_t)event) == cudaSuccess ? GP103_OK : GP103_ERR_CUDA;
}

static int run_pass(const gp103_plan* plan, int phase_flags, cudaStream_t stream, cudaStream_t side,
                    cudaEvent_t fork, cudaEvent_t join);

extern "C" int gp103_pass(const gp103_plan* plan, int phase_flags, cudaStream_t stream) {
    return run_pass(plan, phase_flags, stream, nullptr, nullptr, nullptr);
}

extern "C" int gp103_pass_split(const gp103_plan* plan, int phase_flags, cudaStream_t stream, cudaStream_t side,
                                void* fork, void* join) {
    REQUIRE(side != stream && fork && join && fork != join);
    return run_pass(plan, phase_flags, stream, side, (cudaEvent_t)fork, (cudaEvent_t)join);
}

// One pass. With a side stream (density passes): the WA kernels run there, between a fork after the step and a
// join before the gather, while `stream` runs the sort, the density map and the field; the results are the same.
static int run_pass(const gp103_plan* plan, int phase_flags, cudaStream_t stream, cudaStream_t side,
                    cudaEvent_t fork, cudaEvent_t join) {
    TRY(check_plan(plan));
    const gp103_plan* p = plan;
    const int phase = phase_flags & ~(GP103_PASS_SORT | GP103_PASS_JOIN_FIELD);
    const bool sort = (phase_flags & GP103_PASS_SORT) != 0;
    const bool join_field = (phase_flags & GP103_PASS_JOIN_FIELD) != 0;
    REQUIRE(phase == GP103_PHASE_START || phase == GP103_PHASE_DENSITY);
    REQUIRE(!sort || (phase == GP103_PHASE_DENSITY && p->order != nullptr));
    REQUIRE(p->u[0] && p->u[1] && p->v[0] && p->v[1] && p->g[0] && p->g[1] && p->cur && p->lo && p->hi);
    REQUIRE(phase == GP103_PHASE_START ? p->T != nullptr : (p->S && p->c && p->best));
    StepJob sj = {};
    for (int k = 0; k < 2; k++) { sj.u[k] = p->u[k]; sj.v[k] = p->v[k]; sj.g[k] = p->g[k]; }
    sj.cur = p->cur;
    sj.lo = p->lo;
    sj.hi = p->hi;
    sj.kp = p->kp;
    sj.S = phase == GP103_PHASE_DENSITY ? p->S : nullptr;
    sj.best = phase == GP103_PHASE_DENSITY ? p->best : nullptr;
    sj.n = p->num_nodes;
    sj.red = reduce_slot(p->red, p->counters, R_MOVED);
    const bool ordered = phase == GP103_PHASE_DENSITY && p->order != nullptr;
    if (sort) sj.ord = order_job(p);
    TRY(launch_step(sj, stream));
    const bool split = side != nullptr && phase == GP103_PHASE_DENSITY;
    if (split) {
        if (cudaEventRecord(fork, stream) != cudaSuccess || cudaStreamWaitEvent(side, fork, 0) != cudaSuccess)
            return GP103_ERR_CUDA;
    }
    if (sort) TRY(launch_order(sj.ord, (const float2*)p->v[0], (const float2*)p->v[1], p->cur, true, stream));

    WaJob w = wa_job(p);
    w.pos_a = (const float2*)p->v[0];
    w.pos_b = (const float2*)p->v[1];
    w.sel = p->cur;
    // density passes in one stream: the WA kernels go between the density map and the field, so that the gather
    // reads their pin gradients (42 MB at 1.2M cells) from L2 behind only the field's small working set, and the
    // field planes it reads are the last thing written; nothing between depends on them
    const bool wa_late = phase == GP103_PHASE_DENSITY && !split;
    if (!wa_late) TRY(launch_wa_net(w, split ? side : stream));
    if (split && cudaEventRecord(join, side) != cudaSuccess) return GP103_ERR_CUDA;

    GatherJob g = gather_job(p);
    g.pos_a = (const float2*)p->v[0];
    g.pos_b = (const float2*)p->v[1];
    g.sel = p->cur;
    g.gout_a = (float2*)p->g[0];
    g.gout_b = (float2*)p->g[1];
    g.gref_a = (const float2*)p->g[0];
    g.gref_b = (const float2*)p->g[1];
    g.with_wl = 1;
    const Reduce r_moved = reduce_slot(p->red, p->counters, R_MOVED);
    const Reduce r_grad = reduce_slot(p->red, p->counters, R_GRAD);
    const Reduce r_wa = reduce_slot(p->red, p->counters, R_WA);
    // the step's, the WA kernels' and the post kernel's totals: summed by the gather's block 0 (TOT_* order)
    double* pre = p->red + RED_TOTALS;
    g.pre[TOT_MOVED] = r_moved; g.pre_k[TOT_MOVED] = 0;
    g.pre[TOT_WA] = r_wa; g.pre_k[TOT_WA] = 0;
    g.pre[TOT_HPWL] = r_wa; g.pre_k[TOT_HPWL] = 1;
    g.npre = 3;
    g.pre_out = pre;
    if (phase == GP103_PHASE_START) {
        TRY(launch_gather(g, stream));
        return launch_control_start(p->T, p->kp, r_grad, pre, p->cur, field_error_flag(p), stream);
    }
    TRY(density_and_field(p, p->v[0], p->v[1], p->cur, ordered ? p->order : nullptr, stream, wa_late ? &w : nullptr,
                          split && join_field ? join : nullptr));
    if (split && !join_field && cudaStreamWaitEvent(stream, join, 0) != cudaSuccess) return GP103_ERR_CUDA;
    g.ex = p->ex;
    g.ey = p->ey;
    g.weight_p = p->kp + 1;
    g.precond_p = p->kp + 2;
    g.pre[TOT_OVF] = reduce_slot(p->red, p->counters, p->jnbx > 0 ? R_JOVF : R_OVF);
    g.pre_k[TOT_OVF] = 0;
    g.npre = 4;
    TRY(launch_gather(g, stream));
    const double scale = p->jnbx > 0 ? p->jovf_scale : p->ovf_scale;
    return launch_control_fused(p->S, p->kp, p->c, r_grad, pre, scale, p->cur, field_error_flag(p), stream);
}

extern "C" int gp103_eval(const gp103_plan* plan, const float* pos, float* g_out, const float* g_ref, double weight,
                          double precond, int with_wl, double* out5, cudaStream_t stream) {
    TRY(check_plan(plan));
    const gp103_plan* p = plan;
    REQUIRE(pos && g_out && out5);
    if (with_wl) {
        WaJob w = wa_job(p);
        w.pos_a = w.pos_b = (const float2*)pos;
        TRY(launch_wa_net(w, stream));
    }
    GatherJob g = gather_job(p);
    g.pos_a = g.pos_b = (const float2*)pos;
    g.gout_a = g.gout_b = (float2*)g_out;
    g.gref_a = g.gref_b = (const float2*)g_ref;
    g.with_wl = with_wl;
    if (weight != 0.0) {
        TRY(density_and_field(p, pos, pos, nullptr, nullptr, stream));
        g.ex = p->ex;
        g.ey = p->ey;
        g.weight = (float)weight;
        g.precond = (float)precond;
    }
    TRY(launch_gather(g, stream));
    const Reduce r_wa = reduce_slot(p->red, p->counters, R_WA);
    const Reduce r_grad = reduce_slot(p->red, p->counters, R_GRAD);
    const Reduce ovf = reduce_slot(p->red, p->counters, p->jnbx > 0 ? R_JOVF : R_OVF);
    // out5 = (|g - g_ref|^2, WA, HPWL, overflow sum, L1 of g over the cells)
    const Reduce rs[5] = {r_grad, r_wa, r_wa, ovf, r_grad};
    const int ks[5] = {0, 0, 1, 0, 1};
    return launch_totals(rs, ks, 5, out5, stream);
}

extern "C" int gp103_probe(const gp103_plan* plan, const float* v, const float* g, double step, float* probe,
                           double* out1, cudaStream_t stream) {
    TRY(check_plan(plan));
    REQUIRE(v && g && probe && out1 && plan->lo && plan->hi);
    Reduce r = reduce_slot(plan->red, plan->counters, R_MOVED);
    TRY(launch_probe(v, g, plan->lo, plan->hi, (float)step, plan->num_nodes, probe, r, stream));
    const int k0 = 0;
    return launch_totals(&r, &k0, 1, out1, stream);
}

extern "C" int gp103_begin(const gp103_plan* plan, const gp103_begin_args* a, float* tmp0, float* tmp1,
                           double* scal8, cudaStream_t stream) {
    TRY(check_plan(plan));
    const gp103_plan* p = plan;
    REQUIRE(a && tmp0 && tmp1 && scal8 && p->T && p->S && p->kp && p->cur && p->best && p->v[0] && p->u[0] &&
            p->g[0] && p->lo && p->hi);
    const float* v = p->v[0];
    float* g = p->g[0];
    const double w = a->lam > 0 ? a->lam : 0.0, pc = a->lam > 0 ? a->lam : -1.0;
    const Reduce r = reduce_slot(p->red, p->counters, R_MOVED);
    const int k0 = 0;
    TRY(launch_begin(p->kp, p->cur, a->gamma, a->lam, stream));
    // estimate_initial_learning_rate: the gradient at v, a probe step of lr, the gradient there; the step length
    // sqrt(|probe - v|^2) / sqrt(|g(probe) - g|^2) into scal8[6]
    TRY(gp103_eval(p, v, g, nullptr, w, pc, 1, scal8, stream));
    TRY(launch_probe(v, g, p->lo, p->hi, (float)a->lr, p->num_nodes, tmp0, r, stream));
    TRY(launch_totals(&r, &k0, 1, scal8 + 5, stream));
    TRY(gp103_eval(p, tmp0, tmp1, g, w, pc, 1, scal8, stream));
    TRY(launch_sqrt_ratio(scal8 + 5, scal8, scal8 + 6, stream));
    // NesterovOptimizer.__init__: the gradient at v again, u = v, the probe with that step length; alpha into scal8[7]
    TRY(gp103_eval(p, v, g, nullptr, w, pc, 1, scal8, stream));
    TRY(launch_copy(v, p->u[0], 2 * p->num_nodes, stream));
    TRY(launch_probe(v, g, p->lo, p->hi, 0.f, p->num_nodes, tmp0, r, stream, scal8 + 6));
    TRY(launch_totals(&r, &k0, 1, scal8 + 5, stream));
    TRY(gp103_eval(p, tmp0, tmp1, g, w, pc, 1, scal8, stream));
    TRY(launch_sqrt_ratio(scal8 + 5, scal8, scal8 + 7, stream));
    return launch_first_state(p->T, p->S, p->kp, p->best, v, 2 * p->num_nodes, scal8 + 7, a->gamma, a->lam,
                              a->start_tol, a->inner_iter, a->iter, a->loop_it, a->hpwl_prev, stream);
}

extern "C" int gp103_start_to_density(const gp103_plan* plan, double density_weight, double total_pins,
                                      double gamma, float* g_tmp, double* out5, cudaStream_t stream) {
    TRY(check_plan(plan));
    const gp103_plan* p = plan;
    REQUIRE(g_tmp && out5 && p->T && p->S && p->kp && p->cur && p->best && p->v[0] && p->v[1]);
    // the plain density gradient at v[*cur] (weight 1, no preconditioner, no wirelength term): gp103_eval's kernels
    // with the positions picked on the device (pick(a, b, sel) = *sel ? a : b, so a = v[1], b = v[0])
    TRY(density_and_field(p, p->v[1], p->v[0], p->cur, nullptr, stream));
    GatherJob g = gather_job(p);
    g.pos_a = (const float2*)p->v[1];
    g.pos_b = (const float2*)p->v[0];
    g.sel = p->cur;
    g.gout_a = g.gout_b = (float2*)g_tmp;
    g.with_wl = 0;
    g.ex = p->ex;
    g.ey = p->ey;
    g.weight = 1.f;
    g.precond = -1.f;
    TRY(launch_gather(g, stream));
    const Reduce r_wa = reduce_slot(p->red, p->counters, R_WA);
    const Reduce r_grad = reduce_slot(p->red, p->counters, R_GRAD);
    const Reduce ovf = reduce_slot(p->red, p->counters, p->jnbx > 0 ? R_JOVF : R_OVF);
    const Reduce rs[5] = {r_grad, r_wa, r_wa, ovf, r_grad};
    const int ks[5] = {0, 0, 1, 0, 1};
    TRY(launch_totals(rs, ks, 5, out5, stream));
    return launch_handover(p->T, p->S, p->kp, p->cur, p->v[0], p->v[1], p->best, out5 + 4, total_pins,
                           density_weight, gamma, 2 * p->num_nodes, stream);
}

extern "C" int gp103_finish(const gp103_plan* plan, cudaStream_t stream) {
    REQUIRE(plan && plan->S && plan->cur && plan->v[0] && plan->v[1] && plan->best);
    return launch_finish(plan->S, plan->cur, plan->v[0], plan->v[1], plan->best, 2 * plan->num_nodes, stream);
}
