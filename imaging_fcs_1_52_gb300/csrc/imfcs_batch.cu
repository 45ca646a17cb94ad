// imfcs_batch.cu -- several jobs over one stack as one CUDA graph.
//
// The plugin correlates one (binning, cross-correlation offset) per JNI call
// and repeats the call per binning for the diffusion law
// (Imaging_FCS_1_52.java:11146-11166).  A batch holds one plan per job and
// runs all of them from one graph launch:
//
//   lanes     the jobs are spread over L concurrent branches of the graph;
//             the jobs of a lane run one after another on one scratch arena
//             sized for the largest of them (the per-execution buffers of a
//             plan are dead between executions), so device memory grows
//             with L, not with the number of jobs;
//   graph     the whole launch sequence -- every job's trace, bleach,
//             streaming, blocking, correlator, GLS and fit kernels, the LM
//             counters' memsets -- is captured once and replayed; a new
//             stack pointer, new outputs or a new lane assignment re-captures
//             and updates the executable graph in place;
//   autotune  every job's correlator tile is timed on the real data, every
//             job is timed alone, and lane counts 1..max are timed with the
//             jobs assigned longest-first to the least-loaded lane.
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "imfcs_gb300.h"
#include "imfcs_host.h"

using namespace imfcs;

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) { set_error(cuda_msg(_e, #call)); return 1; } \
    } while (0)

struct imfcs_batch {
    std::vector<imfcs_plan *> plans;
    std::vector<size_t> need;          // scratch bytes per job
    std::vector<double> cost;          // estimated or measured time per job
    std::vector<float> job_ms;         // measured (autotune), 0 before
    std::vector<int> lane_of;          // lane per job
    int lanes = 0;
    std::vector<void *> arena;         // per lane
    std::vector<size_t> arena_bytes;
    std::vector<cudaStream_t> lane_stream;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
    cudaStream_t cap = nullptr;        // capture origin
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const uint16_t *g_stack = nullptr; // what the graph was captured with
    std::vector<imfcs_outputs> g_outs;
    bool dirty = true;
    int launches = 0;
    ~imfcs_batch()
    {
        if (cap) cudaStreamSynchronize(cap);
        for (auto st : lane_stream) cudaStreamSynchronize(st);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (auto p : plans) imfcs_plan_destroy(p);
        for (auto a : arena)
            if (a) cudaFree(a);
        for (auto ev : join) cudaEventDestroy(ev);
        for (auto st : lane_stream) cudaStreamDestroy(st);
        if (fork) cudaEventDestroy(fork);
        if (cap) cudaStreamDestroy(cap);
    }
};

// Lanes 0..nl-1 by longest cost first onto the least-loaded lane; arenas
// sized for each lane's largest job (re-allocated only when too small; lanes
// beyond nl are released).
static int batch_assign(imfcs_batch *b, int nl)
{
    const int n = (int)b->plans.size();
    nl = std::max(1, std::min(nl, n));
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->cost[x] > b->cost[y]; });
    std::vector<double> load(nl, 0.0);
    std::vector<size_t> want(nl, 0);
    for (int j : order) {
        int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        b->lane_of[j] = l;
        load[l] += b->cost[j];
        want[l] = std::max(want[l], b->need[j]);
    }
    // release arenas that are too small or not used, then allocate
    for (size_t l = 0; l < b->arena.size(); l++) {
        const bool keep = (int)l < nl && b->arena_bytes[l] >= want[l];
        if (!keep && b->arena[l]) {
            CK(cudaFree(b->arena[l]));
            b->arena[l] = nullptr;
            b->arena_bytes[l] = 0;
        }
    }
    if ((int)b->arena.size() < nl) {
        b->arena.resize(nl, nullptr);
        b->arena_bytes.resize(nl, 0);
    }
    while ((int)b->lane_stream.size() < nl) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        b->lane_stream.push_back(st);
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        b->join.push_back(ev);
    }
    for (int l = 0; l < nl; l++) {
        if (b->arena[l]) continue;
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, want[l]);
        if (e != cudaSuccess) {
            set_error(cuda_msg(e, "batch scratch arena"));
            return 1;
        }
        b->arena[l] = p;
        b->arena_bytes[l] = want[l];
    }
    b->lanes = nl;
    b->dirty = true;
    return 0;
}

static bool same_outs(const imfcs_batch *b, const imfcs_outputs *outs)
{
    for (size_t j = 0; j < b->g_outs.size(); j++)
        if (memcmp(&b->g_outs[j], &outs[j], sizeof(imfcs_outputs)) != 0) return false;
    return true;
}

// Captures the batch's launch sequence into b->graph and instantiates (or
// updates) b->exec.
static int batch_capture(imfcs_batch *b, const uint16_t *stack, const imfcs_outputs *outs)
{
    const int n = (int)b->plans.size();
    if (b->exec && !b->dirty && stack == b->g_stack && same_outs(b, outs)) return 0;
    CK(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed));
    int rc = 0;
    int launches = 0;
    cudaError_t e = cudaEventRecord(b->fork, b->cap);
    for (int l = 0; l < b->lanes && e == cudaSuccess; l++) e = cudaStreamWaitEvent(b->lane_stream[l], b->fork, 0);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "batch fork")); rc = 1; }
    for (int l = 0; l < b->lanes && !rc; l++)
        for (int j = 0; j < n && !rc; j++) {
            if (b->lane_of[j] != l) continue;
            plan_bind_scratch(b->plans[j], b->arena[l]);
            if (plan_execute_any(b->plans[j], stack, &outs[j], b->lane_stream[l])) rc = 1;
            else launches += imfcs_plan_kernel_launches(b->plans[j]);
        }
    // every forked lane joins the origin before the capture ends
    for (int l = 0; l < b->lanes; l++) {
        cudaError_t e2 = cudaEventRecord(b->join[l], b->lane_stream[l]);
        if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(b->cap, b->join[l], 0);
        if (e2 != cudaSuccess && !rc) { set_error(cuda_msg(e2, "batch join")); rc = 1; }
    }
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->cap, &g);
    if (e != cudaSuccess && !rc) { set_error(cuda_msg(e, "batch graph capture")); rc = 1; }
    if (rc) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return 1;
    }
    if (b->exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(b->exec, g, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
    }
    if (!b->exec) {
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            cudaGraphDestroy(g);
            set_error(cuda_msg(e, "batch graph instantiation"));
            return 1;
        }
    }
    if (b->graph) cudaGraphDestroy(b->graph);
    b->graph = g;
    b->g_stack = stack;
    b->g_outs.assign(outs, outs + n);
    b->dirty = false;
    b->launches = launches;
    return 0;
}

extern "C" int imfcs_batch_create(const imfcs_config *jobs, int n_jobs, int lanes, imfcs_batch **out)
{
    if (!out) { set_error("null batch pointer"); return 1; }
    *out = nullptr;
    if (!jobs || n_jobs < 1) { set_error("a batch needs at least one job"); return 1; }
    for (int i = 1; i < n_jobs; i++) {
        const imfcs_config &a = jobs[0], &c = jobs[i];
        if (c.width != a.width || c.height != a.height || c.frames != a.frames || c.first != a.first ||
            c.num != a.num) {
            set_error("batch jobs must read the same stack (width, height, frames, first, num)");
            return 1;
        }
    }
    imfcs_batch *b = new imfcs_batch();
    b->plans.assign(n_jobs, nullptr);
    b->need.assign(n_jobs, 0);
    b->cost.assign(n_jobs, 0.0);
    b->job_ms.assign(n_jobs, 0.f);
    b->lane_of.assign(n_jobs, 0);
    for (int i = 0; i < n_jobs; i++) {
        if (plan_create_ex(&jobs[i], 0, jobs[i].width, jobs[i].height, false, &b->plans[i], true)) {
            std::string m = "batch job " + std::to_string(i) + ": " + imfcs_get_last_error();
            delete b;
            set_error(m);
            return 1;
        }
        b->need[i] = plan_scratch_need(b->plans[i]);
        // first estimate: the traces' sample count (measured by the autotuner)
        const Job &j = plan_job(b->plans[i]);
        b->cost[i] = (double)j.ntrace * j.num * (jobs[i].gls ? 1.5 : 1.0);
    }
    cudaError_t e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        set_error(cuda_msg(e, "batch streams"));
        delete b;
        return 1;
    }
    if (batch_assign(b, lanes < 1 ? 1 : lanes)) {
        std::string m = imfcs_get_last_error();
        delete b;
        set_error(m);
        return 1;
    }
    *out = b;
    return 0;
}

extern "C" int imfcs_batch_destroy(imfcs_batch *b)
{
    delete b;
    return 0;
}

extern "C" int imfcs_batch_execute(imfcs_batch *b, const uint16_t *dev_stack, const imfcs_outputs *outs,
                                   void *stream)
{
    if (!b || !dev_stack || !outs) { set_error("null argument"); return 1; }
    if (batch_capture(b, dev_stack, outs)) return 1;
    CK(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
    return 0;
}

extern "C" int imfcs_batch_synchronize(imfcs_batch *b, void *stream)
{
    if (!b) { set_error("null batch"); return 1; }
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    for (size_t j = 0; j < b->plans.size(); j++) {
        int derr = 0;
        CK(cudaMemcpy(&derr, plan_dev_err(b->plans[j]), sizeof(int), cudaMemcpyDeviceToHost));
        if (derr) {
            set_error("batch job " + std::to_string(j) + ": a device-side wait timed out (TMA staging)");
            return 1;
        }
    }
    return 0;
}

extern "C" int imfcs_batch_autotune(imfcs_batch *b, const uint16_t *dev_stack, const imfcs_outputs *outs,
                                    void *stream, int max_lanes, float *lane_ms)
{
    if (!b || !dev_stack || !outs) { set_error("null argument"); return 1; }
    cudaStream_t s = (cudaStream_t)stream;
    const int n = (int)b->plans.size();
    max_lanes = std::max(1, std::min(max_lanes, n));
    for (int l = 0; l < max_lanes && lane_ms; l++) lane_ms[l] = 0.f;
    // every job alone on one arena: its correlator tile, then its time
    std::vector<double> save = b->cost;
    for (int j = 0; j < n; j++) b->cost[j] = 1.0;
    if (batch_assign(b, 1)) return 1;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int rc = 0;
    for (int j = 0; j < n && !rc; j++) {
        plan_bind_scratch(b->plans[j], b->arena[0]);
        if (imfcs_plan_autotune(b->plans[j], dev_stack, &outs[j], stream, nullptr, 0, nullptr)) { rc = 1; break; }
        float best = 0.f;
        for (int r = 0; r < 2 && !rc; r++) {
            float t = 0.f;
            cudaError_t e = cudaEventRecord(e0, s);
            if (e == cudaSuccess && plan_execute_any(b->plans[j], dev_stack, &outs[j], s)) { rc = 1; break; }
            if (e == cudaSuccess) e = cudaEventRecord(e1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
            if (e != cudaSuccess) { set_error(cuda_msg(e, "batch autotune timing")); rc = 1; break; }
            best = r == 0 ? t : std::min(best, t);
        }
        b->job_ms[j] = best;
    }
    if (rc) {
        b->cost = save;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return 1;
    }
    for (int j = 0; j < n; j++) b->cost[j] = b->job_ms[j];
    // lane counts
    int best_l = 1;
    float best_t = 0.f;
    for (int nl = 1; nl <= max_lanes && !rc; nl++) {
        if (batch_assign(b, nl)) {
            cudaGetLastError();
            break;   // arenas no longer fit: more lanes will not either
        }
        float t[2] = {0.f, 0.f};
        if (imfcs_batch_execute(b, dev_stack, outs, stream)) { rc = 1; break; }
        for (int r = 0; r < 2 && !rc; r++) {
            cudaError_t e = cudaEventRecord(e0, s);
            if (e == cudaSuccess && imfcs_batch_execute(b, dev_stack, outs, stream)) { rc = 1; break; }
            if (e == cudaSuccess) e = cudaEventRecord(e1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t[r], e0, e1);
            if (e != cudaSuccess) { set_error(cuda_msg(e, "batch autotune timing")); rc = 1; }
        }
        if (rc) break;
        const float tm = std::min(t[0], t[1]);
        if (lane_ms) lane_ms[nl - 1] = tm;
        if (nl == 1 || tm < best_t) { best_t = tm; best_l = nl; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return 1;
    return batch_assign(b, best_l);
}

extern "C" int imfcs_batch_job_info(const imfcs_batch *b, int job, int *npix, int *chanum, int *lane, int *cta,
                                    int *seg_extra, int *tail_extra, float *ms)
{
    if (!b || job < 0 || job >= (int)b->plans.size()) { set_error("invalid batch job"); return 1; }
    const Job &j = plan_job(b->plans[job]);
    if (npix) *npix = j.npix;
    if (chanum) *chanum = j.chanum;
    if (lane) *lane = b->lane_of[job];
    int c = 64, x = 0, tx = 0;
    imfcs_plan_get_corr_tile(b->plans[job], &c, &x, &tx);
    if (cta) *cta = c;
    if (seg_extra) *seg_extra = x;
    if (tail_extra) *tail_extra = tx;
    if (ms) *ms = b->job_ms[job];
    return 0;
}

extern "C" int imfcs_batch_lanes(const imfcs_batch *b) { return b ? b->lanes : -1; }

extern "C" size_t imfcs_batch_scratch_bytes(const imfcs_batch *b)
{
    if (!b) return 0;
    size_t t = 0;
    for (size_t l = 0; l < b->arena_bytes.size(); l++) t += b->arena_bytes[l];
    for (auto p : b->plans) t += imfcs_plan_scratch_bytes(p);
    return t;
}

extern "C" int imfcs_batch_kernel_launches(const imfcs_batch *b) { return b ? b->launches : -1; }
