// lumrad_batch.cpp — many resident worlds updated by one launch of the pass kernels.
//
// The reference updates one world per frame with one dispatch (internal_render.cpp:1204-1206),
// time-slicing its probes to stay within a frame budget.  A batch instead gathers many worlds
// (contexts) of different sizes, update lists and ray counts into one task space: every world's
// 32-ray subgroups are tasks of the same persistent march kernel and finalize kernel, so small
// worlds no longer leave most of the GPU idle.  One pass of the whole batch is captured once into
// a CUDA graph and replayed:
//   H2D copy of the world table (pinned, double-buffered: per-run seeds and ping-pong sides)
//   -> prep kernel (each world's next volume = its prev, counters cleared)
//   -> rounds of march + finalize over all tasks.
// The scheduling knobs of the march queue (guided divisor, chunk cap, CTAs per SM) are chosen by
// lumrad_batch_autotune, which times candidate settings on the batch itself.

#include "lumrad_world.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace lumrad {
namespace {

struct BatchWorld {
    Context* ctx = nullptr;
    short4* d_req = nullptr;
    int n = 0;
    LumRadPassParams p{};
    bool set = false;
};

struct Batch {
    int device = 0;
    int precision = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_end = nullptr;
    cudaEvent_t ev_done[2] = {nullptr, nullptr};
    bool run_pending[2] = {false, false};
    std::vector<BatchWorld> worlds;
    WorldPass* h_table[2] = {nullptr, nullptr};   // pinned
    WorldPass* d_table[2] = {nullptr, nullptr};
    long long n_tasks = 0;
    unsigned long long* d_queue = nullptr;
    int* d_error = nullptr;
    RayResult* d_ray_res = nullptr;
    size_t ray_cap = 0;
    Tuning tuning;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    bool dirty = true;
    long long runs = 0;
    bool have_run = false;

    void release_graphs() {
        for (auto& e : exec) {
            if (e) cudaGraphExecDestroy(e);
            e = nullptr;
        }
    }
};

Batch* as_batch(LumRadBatch b) { return reinterpret_cast<Batch*>(b); }

int wait_runs(Batch* b) {
    for (int k = 0; k < 2; k++)
        if (b->run_pending[k]) {
            LUMRAD_TRY(cudaEventSynchronize(b->ev_done[k]));
            b->run_pending[k] = false;
        }
    return LUMRAD_OK;
}

// World table, task offsets (each world starts at a multiple of 8 tasks so a probe's subgroups
// share a finalize CTA), buffers, and the two graphs.
int build(Batch* b) {
    NvtxRange range("lumrad batch build");
    int rc = wait_runs(b);
    if (rc) return rc;
    const int nw = (int)b->worlds.size();
    long long begin = 0;
    for (int i = 0; i < nw; i++) {
        BatchWorld& bw = b->worlds[i];
        if (!bw.set) return fail(LUMRAD_ESTATE, "every world of a batch needs lumrad_batch_set_requests");
        WorldPass w;
        if ((rc = bw.ctx->world.fill_pass(bw.d_req, bw.n, bw.p, b->stream, &w))) return rc;
        w.task_begin = begin;
        begin += (w.n_tasks + kWarps - 1) / kWarps * kWarps;
        b->h_table[0][i] = w;
        b->h_table[1][i] = w;
    }
    if (begin >= (1LL << 31)) return fail(LUMRAD_EINVAL, "batch has too many subgroups (>= 2^31)");
    b->n_tasks = begin;
    const size_t need = (size_t)std::min<long long>(std::max<long long>(begin, 1), kBatchRoundTasks) * kTaskRays;
    if (need > b->ray_cap) {
        cudaFree(b->d_ray_res);
        b->d_ray_res = nullptr;
        b->ray_cap = 0;
        LUMRAD_TRY(cudaMalloc(&b->d_ray_res, need * sizeof(RayResult)));
        b->ray_cap = need;
    }
    b->release_graphs();
    for (int k = 0; k < 2; k++) {
        LaunchArgs la;
        std::memset(&la, 0, sizeof la);
        la.worlds = b->d_table[k];
        la.n_worlds = nw;
        la.n_tasks = b->n_tasks;
        la.queue = b->d_queue;
        la.error = b->d_error;
        la.ray_res = b->d_ray_res;
        la.round_tasks = kBatchRoundTasks;
        la.in_cta = combines_in_cta(b->h_table[k], nw) ? 1 : 0;
        la.guided_div = b->tuning.guided_div;
        la.max_chunk = b->tuning.max_chunk;
        la.march_ctas = b->tuning.march_ctas;
        LUMRAD_TRY(cudaStreamSynchronize(b->stream));
        cudaGraph_t graph = nullptr;
        LUMRAD_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaMemcpyAsync(b->d_table[k], b->h_table[k], nw * sizeof(WorldPass), cudaMemcpyHostToDevice,
                                        b->stream);
        if (e == cudaSuccess) e = launch_prep(b->d_table[k], nw, b->precision, b->stream);
        if (e == cudaSuccess) e = launch_radiance(la, b->precision, false, b->num_sms, b->stream);
        const cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return fail(LUMRAD_EDEVICE, std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        e = cudaGraphInstantiate(&b->exec[k], graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(LUMRAD_EDEVICE, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    b->dirty = false;
    return LUMRAD_OK;
}

int check_batch_error(Batch* b) {
    int e = 0;
    LUMRAD_TRY(cudaMemcpyAsync(&e, b->d_error, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    LUMRAD_TRY(cudaStreamSynchronize(b->stream));
    if (e != 0) {
        cudaMemsetAsync(b->d_error, 0, sizeof(int), b->stream);
        cudaMemsetAsync(b->d_queue, 0, kQueueWords * sizeof(unsigned long long), b->stream);
        cudaStreamSynchronize(b->stream);
        return fail(LUMRAD_EDEVICE, "radiance kernel reported an error (code " + std::to_string(e) + ")");
    }
    return LUMRAD_OK;
}

int run_graph(Batch* b, int time_seed) {
    NvtxRange range("lumrad batch run");
    int rc;
    if (b->dirty && (rc = build(b))) return rc;
    const int k = (int)(b->runs & 1);
    if (b->run_pending[k]) {   // the table of run - 2 may still be in flight
        LUMRAD_TRY(cudaEventSynchronize(b->ev_done[k]));
        b->run_pending[k] = false;
    }
    WorldPass* t = b->h_table[k];
    for (size_t i = 0; i < b->worlds.size(); i++) {
        DeviceWorld& dw = b->worlds[i].ctx->world;
        t[i].prev = dw.d_rad[dw.cur];
        t[i].next = dw.d_rad[1 - dw.cur];
        t[i].seed = (uint32_t)time_seed;
    }
    LUMRAD_TRY(cudaEventRecord(b->ev_start, b->stream));
    LUMRAD_TRY(cudaGraphLaunch(b->exec[k], b->stream));
    LUMRAD_TRY(cudaEventRecord(b->ev_end, b->stream));
    LUMRAD_TRY(cudaEventRecord(b->ev_done[k], b->stream));
    b->run_pending[k] = true;
    for (auto& bw : b->worlds) {
        DeviceWorld& dw = bw.ctx->world;
        dw.cur = 1 - dw.cur;
        dw.hits_recorded = false;
        bw.ctx->have_pass = true;
        bw.ctx->last_count_on_device = false;   // this pass's list length is known on the host
        bw.ctx->last.probes = (uint64_t)(bw.n / bw.p.size);
        bw.ctx->last.rays = bw.ctx->last.probes * (uint64_t)bw.p.rays_per_probe;
    }
    b->runs++;
    b->have_run = true;
    return LUMRAD_OK;
}

}  // namespace
}  // namespace lumrad

using namespace lumrad;

extern "C" {

int lumrad_batch_create(LumRadContext const* worlds, int n_worlds, LumRadBatch* out) {
    if (!worlds || !out || n_worlds < 1) return fail(LUMRAD_EINVAL, "bad argument");
    *out = nullptr;
    Context* c0 = as_ctx(worlds[0]);
    if (!c0) return fail(LUMRAD_EINVAL, "null context");
    for (int i = 0; i < n_worlds; i++) {
        Context* c = as_ctx(worlds[i]);
        if (!c) return fail(LUMRAD_EINVAL, "null context");
        if (int rc = check_unowned(c)) return rc;
        if (c->device != c0->device) return fail(LUMRAD_EINVAL, "the worlds of a batch must share one device");
        if (c->world.precision != c0->world.precision) return fail(LUMRAD_EINVAL, "the worlds of a batch must share one precision");
        for (int j = 0; j < i; j++)
            if (worlds[j] == worlds[i]) return fail(LUMRAD_EINVAL, "a context appears twice in the batch");
    }
    Batch* b = new Batch();
    b->device = c0->device;
    b->precision = c0->world.precision;
    b->num_sms = c0->num_sms;
    auto attempt = [&]() -> int {
        LUMRAD_TRY(cudaSetDevice(b->device));
        for (int i = 0; i < n_worlds; i++) LUMRAD_TRY(cudaStreamSynchronize(as_ctx(worlds[i])->stream));
        LUMRAD_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        LUMRAD_TRY(cudaEventCreate(&b->ev_start));
        LUMRAD_TRY(cudaEventCreate(&b->ev_end));
        for (auto& e : b->ev_done) LUMRAD_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (int k = 0; k < 2; k++) {
            LUMRAD_TRY(cudaMallocHost(&b->h_table[k], n_worlds * sizeof(WorldPass)));
            LUMRAD_TRY(cudaMalloc(&b->d_table[k], n_worlds * sizeof(WorldPass)));
        }
        LUMRAD_TRY(cudaMalloc(&b->d_queue, kQueueWords * sizeof(unsigned long long)));
        LUMRAD_TRY(cudaMalloc(&b->d_error, sizeof(int)));
        LUMRAD_TRY(cudaMemsetAsync(b->d_queue, 0, kQueueWords * sizeof(unsigned long long), b->stream));
        LUMRAD_TRY(cudaMemsetAsync(b->d_error, 0, sizeof(int), b->stream));
        LUMRAD_TRY(cudaStreamSynchronize(b->stream));
        return LUMRAD_OK;
    };
    b->worlds.resize(n_worlds);
    for (int i = 0; i < n_worlds; i++) b->worlds[i].ctx = as_ctx(worlds[i]);
    const int rc = attempt();
    if (rc) {
        const std::string msg = g_error;
        lumrad_batch_destroy(b);
        return fail(rc, msg);
    }
    *out = b;
    return LUMRAD_OK;
}

void lumrad_batch_destroy(LumRadBatch batch) {
    Batch* b = as_batch(batch);
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    b->release_graphs();
    for (auto& bw : b->worlds) cudaFree(bw.d_req);
    for (int k = 0; k < 2; k++) {
        if (b->h_table[k]) cudaFreeHost(b->h_table[k]);
        cudaFree(b->d_table[k]);
        if (b->ev_done[k]) cudaEventDestroy(b->ev_done[k]);
    }
    cudaFree(b->d_queue);
    cudaFree(b->d_error);
    cudaFree(b->d_ray_res);
    if (b->ev_start) cudaEventDestroy(b->ev_start);
    if (b->ev_end) cudaEventDestroy(b->ev_end);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int lumrad_batch_set_requests(LumRadBatch batch, int world, const int16_t* requests, int n, const LumRadPassParams* p) {
    Batch* b = as_batch(batch);
    if (!b || world < 0 || world >= (int)b->worlds.size()) return fail(LUMRAD_EINVAL, "bad batch or world index");
    if (n < 0 || (n > 0 && !requests)) return fail(LUMRAD_EINVAL, "bad request list");
    int rc = check_params(p);
    if (rc) return rc;
    if (p->size < 1) return fail(LUMRAD_EINVAL, "size must be >= 1 in a batch");
    if (p->record_hits) return fail(LUMRAD_EINVAL, "hit records need lumrad_radiance_pass");
    LUMRAD_TRY(cudaSetDevice(b->device));
    if ((rc = wait_runs(b))) return rc;
    BatchWorld& bw = b->worlds[world];
    cudaFree(bw.d_req);
    bw.d_req = nullptr;
    bw.n = 0;
    LUMRAD_TRY(cudaMalloc(&bw.d_req, std::max(n, 1) * sizeof(short4)));
    if (n > 0) LUMRAD_TRY(cudaMemcpyAsync(bw.d_req, requests, (size_t)n * sizeof(short4), cudaMemcpyHostToDevice, b->stream));
    LUMRAD_TRY(cudaStreamSynchronize(b->stream));
    bw.n = n;
    bw.p = *p;
    bw.set = true;
    b->dirty = true;
    return LUMRAD_OK;
}

int lumrad_batch_run(LumRadBatch batch, int time_seed) {
    Batch* b = as_batch(batch);
    if (!b) return fail(LUMRAD_EINVAL, "null batch");
    LUMRAD_TRY(cudaSetDevice(b->device));
    return run_graph(b, time_seed);
}

int lumrad_batch_run_per_world(LumRadBatch batch, int time_seed) {
    Batch* b = as_batch(batch);
    if (!b) return fail(LUMRAD_EINVAL, "null batch");
    LUMRAD_TRY(cudaSetDevice(b->device));
    int rc = wait_runs(b);
    if (rc) return rc;
    LUMRAD_TRY(cudaStreamSynchronize(b->stream));
    LUMRAD_TRY(cudaEventRecord(b->ev_start, b->stream));
    for (auto& bw : b->worlds) {
        if (!bw.set) return fail(LUMRAD_ESTATE, "every world of a batch needs lumrad_batch_set_requests");
        LumRadPassParams p = bw.p;
        p.time_seed = time_seed;
        if ((rc = bw.ctx->run_pass(bw.d_req, bw.n, &p))) return rc;
        LUMRAD_TRY(cudaStreamSynchronize(bw.ctx->stream));
    }
    LUMRAD_TRY(cudaEventRecord(b->ev_end, b->stream));
    b->have_run = true;
    return LUMRAD_OK;
}

int lumrad_batch_synchronize(LumRadBatch batch) {
    Batch* b = as_batch(batch);
    if (!b) return fail(LUMRAD_EINVAL, "null batch");
    LUMRAD_TRY(cudaSetDevice(b->device));
    int rc = wait_runs(b);
    if (rc) return rc;
    return check_batch_error(b);
}

int lumrad_batch_last_ms(LumRadBatch batch, float* ms) {
    Batch* b = as_batch(batch);
    if (!b || !ms) return fail(LUMRAD_EINVAL, "null argument");
    if (!b->have_run) return fail(LUMRAD_ESTATE, "the batch has not run");
    LUMRAD_TRY(cudaSetDevice(b->device));
    LUMRAD_TRY(cudaEventSynchronize(b->ev_end));
    LUMRAD_TRY(cudaEventElapsedTime(ms, b->ev_start, b->ev_end));
    return LUMRAD_OK;
}

int lumrad_batch_set_tuning(LumRadBatch batch, const LumRadTuning* t) {
    Batch* b = as_batch(batch);
    if (!b || !t) return fail(LUMRAD_EINVAL, "null argument");
    if (t->guided_div < 0 || t->max_chunk < 0 || t->march_ctas < 0) return fail(LUMRAD_EINVAL, "negative tuning value");
    // a claimed chunk carries its task count in 12 bits (the march kernel's queue words)
    if (t->max_chunk > LUMRAD_MAX_CHUNK) return fail(LUMRAD_EINVAL, "max_chunk above LUMRAD_MAX_CHUNK");
    b->tuning.guided_div = t->guided_div;
    b->tuning.max_chunk = t->max_chunk;
    b->tuning.march_ctas = t->march_ctas;
    b->dirty = true;
    return LUMRAD_OK;
}

int lumrad_batch_autotune(LumRadBatch batch, int repeats, LumRadTuning* best) {
    Batch* b = as_batch(batch);
    if (!b || !best) return fail(LUMRAD_EINVAL, "null argument");
    if (repeats < 1) repeats = 3;
    LUMRAD_TRY(cudaSetDevice(b->device));
    int rc = wait_runs(b);
    if (rc) return rc;
    // tuning runs real passes: keep each world's volume and put it back afterwards
    std::vector<void*> saved(b->worlds.size(), nullptr);
    auto restore = [&]() {
        for (size_t i = 0; i < b->worlds.size(); i++) {
            if (!saved[i]) continue;
            DeviceWorld& dw = b->worlds[i].ctx->world;
            cudaMemcpyAsync(dw.d_rad[dw.cur], saved[i], dw.W * dw.rad_stride, cudaMemcpyDeviceToDevice, b->stream);
        }
        cudaStreamSynchronize(b->stream);
        for (void* p : saved) cudaFree(p);
    };
    for (size_t i = 0; i < b->worlds.size(); i++) {
        DeviceWorld& dw = b->worlds[i].ctx->world;
        if (cudaMalloc(&saved[i], dw.W * dw.rad_stride) != cudaSuccess) {
            restore();
            return fail(LUMRAD_ENOMEM, "no memory to keep the volumes while tuning");
        }
        cudaMemcpyAsync(saved[i], dw.d_rad[dw.cur], dw.W * dw.rad_stride, cudaMemcpyDeviceToDevice, b->stream);
    }
    const int divs[] = {1, 2, 4};
    const int caps[] = {4, 8, 16, 32};
    const int ctas[] = {0, 2, 3};
    LumRadTuning top{2, 16, 0, 1e30f};
    for (int d : divs)
        for (int c : caps)
            for (int m : ctas) {
                b->tuning = Tuning{d, c, m};
                b->dirty = true;
                float total = 0.0f;
                for (int r = 0; r <= repeats; r++) {
                    if ((rc = run_graph(b, r))) { restore(); return rc; }
                    float ms = 0.0f;
                    LUMRAD_TRY(cudaEventSynchronize(b->ev_end));
                    LUMRAD_TRY(cudaEventElapsedTime(&ms, b->ev_start, b->ev_end));
                    if (r > 0) total += ms;   // the first run warms up
                }
                const float avg = total / repeats;
                if (avg < top.pass_ms) top = LumRadTuning{d, c, m, avg};
            }
    b->tuning = Tuning{top.guided_div, top.max_chunk, top.march_ctas};
    b->dirty = true;
    if ((rc = wait_runs(b))) { restore(); return rc; }
    restore();
    if ((rc = check_batch_error(b))) return rc;
    *best = top;
    return LUMRAD_OK;
}

int lumrad_batch_stats(LumRadBatch batch, LumRadPassStats* out) {
    Batch* b = as_batch(batch);
    if (!b || !out) return fail(LUMRAD_EINVAL, "null argument");
    if (!b->have_run) return fail(LUMRAD_ESTATE, "the batch has not run");
    int rc = lumrad_batch_synchronize(batch);
    if (rc) return rc;
    LumRadPassStats s{};
    for (auto& bw : b->worlds) {
        unsigned long long h[2];
        LUMRAD_TRY(cudaMemcpy(h, bw.ctx->world.d_stats, sizeof h, cudaMemcpyDeviceToHost));
        s.probes += (uint64_t)(bw.n / bw.p.size);
        s.rays += (uint64_t)(bw.n / bw.p.size) * (uint64_t)bw.p.rays_per_probe;
        s.steps += h[0];
        s.hits += h[1];
    }
    LUMRAD_TRY(cudaEventElapsedTime(&s.gpu_ms, b->ev_start, b->ev_end));
    *out = s;
    return LUMRAD_OK;
}

}  // extern "C"
