// Batches of placement instances in one CUDA graph: one conditional WHILE node per instance, its body a few passes of
// that instance's plan and a condition kernel. The instances are independent branches of the graph, so the GPU runs
// them side by side; each one loops on the device until its own control stops it, with no host poll between passes.
// The reference runs one design per process and polls the host every 16 passes (src/gpu_loop.py:58-70); this
// batching has no counterpart there.
//
// The condition kernel ends an instance's loop when its state says stop (the density phase's S[stop], or the start
// phase's T[done] / T[stop]) or after max_loops bodies (a hard limit, so that no loop can run forever), and records
// the device time (globaltimer, ns) of the end.
#include <new>
#include <vector>

#include "gp103.cuh"
#include "step.cuh"

using namespace gp103;

#define TRY(call)                \
    do {                         \
        int st_ = (call);        \
        if (st_) return st_;     \
    } while (0)

namespace {

struct Batch {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int count = 0;
    bool broken = false;        // an add failed after it changed the graph: the graph holds a partial instance
};

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void batch_cond_kernel(cudaGraphConditionalHandle h, const double* state, int stop_at, int done_at,
                                  int* loops, int max_loops, unsigned long long* stop_ns) {
    pdl_wait();
    const int l = *loops + 1;
    *loops = l;
    const bool stop = state[stop_at] != 0.0 || (done_at >= 0 && state[done_at] != 0.0) || l >= max_loops;
    if (stop) *stop_ns = now_ns();
    cudaGraphSetConditional(h, stop ? 0u : 1u);
}

__global__ void batch_clock_kernel(unsigned long long* t) { *t = now_ns(); }

}  // namespace

extern "C" int gp103_batch_create(void** batch) {
    if (!batch) return GP103_ERR_ARG;
    Batch* b = new (std::nothrow) Batch();
    if (!b) return GP103_ERR_ARG;
    if (cudaGraphCreate(&b->graph, 0) != cudaSuccess) {
        delete b;
        return GP103_ERR_CUDA;
    }
    *batch = b;
    return GP103_OK;
}

extern "C" int gp103_batch_destroy(void* batch) {
    Batch* b = (Batch*)batch;
    if (!b) return GP103_ERR_ARG;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    delete b;
    return GP103_OK;
}

// A conditional node of type `type` after the nodes deps[0..ndeps), its handle set to `value` at every launch of the
// graph (a WHILE node whose condition kernel clears it, or an IF node that runs its body once). -> its body graph.
static int add_conditional(Batch* b, cudaGraphConditionalNodeType type, unsigned int value,
                           const cudaGraphNode_t* deps, size_t ndeps, cudaGraphConditionalHandle* h,
                           cudaGraphNode_t* node, cudaGraph_t* body) {
    if (cudaGraphConditionalHandleCreate(h, b->graph, value, cudaGraphCondAssignDefault) != cudaSuccess)
        return GP103_ERR_CUDA;
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = *h;
    p.conditional.type = type;
    p.conditional.size = 1;
    if (cudaGraphAddNode(node, b->graph, deps, nullptr, ndeps, &p) != cudaSuccess) return GP103_ERR_CUDA;
    *body = p.conditional.phGraph_out[0];
    return GP103_OK;
}

// The loop of one phase of one instance after deps: `passes` passes and the condition kernel per body.
static int add_loop(Batch* b, const gp103_plan* plan, int phase, int passes, int sort_first, int max_loops,
                    int* loops, unsigned long long* stop_ns, const cudaGraphNode_t* deps, size_t ndeps,
                    cudaStream_t capture, cudaGraphNode_t* node) {
    cudaGraphConditionalHandle h;
    cudaGraph_t body;
    TRY(add_conditional(b, cudaGraphCondTypeWhile, 1, deps, ndeps, &h, node, &body));
    if (cudaStreamBeginCaptureToGraph(capture, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    int st = GP103_OK;
    for (int k = 0; k < passes && !st; k++) {
        const int flags = phase | (phase == GP103_PHASE_DENSITY && sort_first && k == 0 ? GP103_PASS_SORT : 0);
        st = gp103_pass(plan, flags, capture);
    }
    const double* state = phase == GP103_PHASE_START ? plan->T : plan->S;
    const int stop_at = phase == GP103_PHASE_START ? (int)GP103_T_STOP : (int)S_STOP;
    const int done_at = phase == GP103_PHASE_START ? GP103_T_DONE : -1;
    if (!st && launch_k(batch_cond_kernel, dim3(1), dim3(1), 0, capture, h, state, stop_at, done_at, loops, max_loops,
                        stop_ns) != cudaSuccess)
        st = GP103_ERR_CUDA;
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(capture, &out);      // (ends the capture whatever happened above)
    if (st) return st;
    return e == cudaSuccess ? GP103_OK : GP103_ERR_CUDA;
}

extern "C" int gp103_batch_add(void* batch, const gp103_plan* plan, int phase, int passes, int sort_first,
                               int max_loops, int* loops, unsigned long long* stop_ns, cudaStream_t capture) {
    Batch* b = (Batch*)batch;
    if (!b || !plan || !loops || !stop_ns || passes < 1 || max_loops < 1 || b->exec) return GP103_ERR_ARG;
    if (phase != GP103_PHASE_START && phase != GP103_PHASE_DENSITY) return GP103_ERR_ARG;
    if (phase == GP103_PHASE_START ? !plan->T : !plan->S) return GP103_ERR_ARG;
    cudaGraphNode_t node;
    const int st = add_loop(b, plan, phase, passes, sort_first, max_loops, loops, stop_ns, nullptr, 0, capture, &node);
    if (st) {
        b->broken = true;
        return st;
    }
    b->count++;
    return GP103_OK;
}

// An IF node after deps[0..ndeps) whose body (run once per launch) is what `queue` puts on the capture stream.
template <typename F>
static int add_once(Batch* b, const cudaGraphNode_t* deps, size_t ndeps, cudaStream_t capture, cudaGraphNode_t* node,
                    F queue) {
    cudaGraphConditionalHandle h;
    cudaGraph_t body;
    TRY(add_conditional(b, cudaGraphCondTypeIf, 1, deps, ndeps, &h, node, &body));
    if (cudaStreamBeginCaptureToGraph(capture, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) !=
        cudaSuccess)
        return GP103_ERR_CUDA;
    const int st = queue();
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(capture, &out);      // (ends the capture whatever happened above)
    if (st) return st;
    return e == cudaSuccess ? GP103_OK : GP103_ERR_CUDA;
}

extern "C" int gp103_batch_add_run(void* batch, const gp103_plan* plan, const gp103_begin_args* begin,
                                   int start_passes, int density_passes, int max_start_loops, int max_density_loops,
                                   double density_weight, double total_pins, double gamma, float* tmp0, float* tmp1,
                                   double* scal8, int* loops, unsigned long long* stop_ns, cudaStream_t capture) {
    Batch* b = (Batch*)batch;
    if (!b || !plan || !plan->T || !plan->S || !tmp0 || !scal8 || !loops || !stop_ns || start_passes < 1 ||
        density_passes < 1 || max_start_loops < 1 || max_density_loops < 1 || b->exec || (begin && !tmp1))
        return GP103_ERR_ARG;
    cudaGraphNode_t set_up, start, hand, density;
    const gp103_begin_args args = begin ? *begin : gp103_begin_args{};
    int st = GP103_OK;
    if (begin)
        st = add_once(b, nullptr, 0, capture, &set_up,
                      [&] { return gp103_begin(plan, &args, tmp0, tmp1, scal8, capture); });
    if (!st)
        st = add_loop(b, plan, GP103_PHASE_START, start_passes, 0, max_start_loops, loops, stop_ns,
                      begin ? &set_up : nullptr, begin ? 1 : 0, capture, &start);
    if (!st)
        st = add_once(b, &start, 1, capture, &hand, [&] {
            return gp103_start_to_density(plan, density_weight, total_pins, gamma, tmp0, scal8, capture);
        });
    if (!st)
        st = add_loop(b, plan, GP103_PHASE_DENSITY, density_passes, 1, max_density_loops, loops + 1, stop_ns + 1,
                      &hand, 1, capture, &density);
    if (st) {
        b->broken = true;
        return st;
    }
    b->count++;
    return GP103_OK;
}

extern "C" int gp103_batch_launch(void* batch, unsigned long long* t0_ns, cudaStream_t stream) {
    Batch* b = (Batch*)batch;
    if (!b || b->count == 0 || b->broken) return GP103_ERR_ARG;
    if (!b->exec && cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) return GP103_ERR_CUDA;
    if (t0_ns) {
        batch_clock_kernel<<<1, 1, 0, stream>>>(t0_ns);
        if (cudaGetLastError() != cudaSuccess) return GP103_ERR_CUDA;
    }
    if (cudaGraphLaunch(b->exec, stream) != cudaSuccess) return GP103_ERR_CUDA;
    return GP103_OK;
}
