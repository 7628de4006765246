// lumrad_serve.cpp — relight server: continuous batching of edit + relight requests over
// resident worlds.
//
// In the reference an edit (lum_set_world_block, crenderer.h) changes the grid, and the next
// frame's update_radiance (internal_render.cpp:1129-1214) re-lists every probe near non-air
// blocks, time-sliced over frames.  The server instead relights only the probes near each edit
// and serves many worlds at once:
//
//   host, per launch   take the oldest due request of each idle world (submission order) while
//                      its device bytes fit the HBM budget; per request, dedupe its edits (last
//                      edit of a block wins), update the host grid and compact ids, and list the
//                      probes within `radius` of the edits; pack the world table, the edit
//                      records and the lists into one pinned buffer
//   device, per launch one H2D copy -> edit kernel (grid + compact grid) -> prep kernel (next =
//                      prev) -> rounds of march + finalize over all worlds' tasks; the error word
//                      is read back and a host callback stamps the completion time
//
// Up to max_inflight launches run at once on their own streams.  A world is in at most one
// launch at a time (it is "busy" until its launch retires), so a world's requests run in order
// and every result equals the result of the same requests run alone.

#include "lumrad_world.h"
#include "lumrad_devloop.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>
#include <vector>

namespace lumrad {

// Probes within Chebyshev distance r of the edits, appended to `out` in x-fastest scan order.
// One bit per block: each (y, z) row of X blocks is ceil(X/64) words.  The edit bits are dilated
// along x by word shifts, along y and z by ORs of 2r+1 rows / planes, and the set bits are
// emitted in scan order.  a and b are scratch (resized here).
void dirty_probes(int X, int Y, int Z, const LumRadEdit* e, int n, int r, std::vector<uint64_t>& a,
                  std::vector<uint64_t>& b, std::vector<short4>& out) {
    const size_t wpr = ((size_t)X + 63) / 64;          // words per row
    const size_t rows = (size_t)Y * Z;
    const size_t words = rows * wpr;
    const size_t plane = (size_t)Y * wpr;
    a.assign(words, 0);
    b.assign(words, 0);
    for (int k = 0; k < n; k++) {
        const size_t row = (size_t)e[k].y + (size_t)Y * e[k].z;
        a[row * wpr + (size_t)e[k].x / 64] |= 1ull << (e[k].x % 64);
    }
    const uint64_t last = (X % 64) ? (1ull << (X % 64)) - 1 : ~0ull;   // valid bits of a row's last word
    // x: b = a | a shifted by 1..r either way, within each row
    for (size_t row = 0; row < rows; row++) {
        const uint64_t* in = a.data() + row * wpr;
        uint64_t* o = b.data() + row * wpr;
        for (size_t w = 0; w < wpr; w++) {
            uint64_t v = in[w];
            for (int s = 1; s <= r; s++) {
                v |= in[w] << s | in[w] >> s;
                if (w > 0) v |= in[w - 1] >> (64 - s);
                if (w + 1 < wpr) v |= in[w + 1] << (64 - s);
            }
            o[w] = v;
        }
        o[wpr - 1] &= last;
    }
    // y: a = OR of b rows [y-r, y+r] within each plane
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++) {
            uint64_t* o = a.data() + (size_t)z * plane + (size_t)y * wpr;
            for (size_t w = 0; w < wpr; w++) o[w] = 0;
            for (int yy = std::max(y - r, 0); yy <= std::min(y + r, Y - 1); yy++) {
                const uint64_t* in = b.data() + (size_t)z * plane + (size_t)yy * wpr;
                for (size_t w = 0; w < wpr; w++) o[w] |= in[w];
            }
        }
    // z: b = OR of a planes [z-r, z+r]
    for (int z = 0; z < Z; z++) {
        uint64_t* o = b.data() + (size_t)z * plane;
        for (size_t w = 0; w < plane; w++) o[w] = 0;
        for (int zz = std::max(z - r, 0); zz <= std::min(z + r, Z - 1); zz++) {
            const uint64_t* in = a.data() + (size_t)zz * plane;
            for (size_t w = 0; w < plane; w++) o[w] |= in[w];
        }
    }
    size_t count = 0;
    for (size_t w = 0; w < words; w++) count += (size_t)__builtin_popcountll(b[w]);
    const size_t base = out.size();
    out.resize(base + count);
    short4* p = out.data() + base;
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++) {
            const uint64_t* row = b.data() + (size_t)z * plane + (size_t)y * wpr;
            for (size_t w = 0; w < wpr; w++)
                for (uint64_t bits = row[w]; bits; bits &= bits - 1) {
                    p->x = (short)((int)(w * 64) + __builtin_ctzll(bits));
                    p->y = (short)y;
                    p->z = (short)z;
                    p->w = 0;
                    p++;
                }
        }
}

namespace {

double clock_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct SRequest {
    long long id = 0;
    int world = 0;
    double arrival = 0.0;
    LumRadPassParams p{};
    std::vector<LumRadEdit> edits;
};

struct SWorld {
    Context* ctx = nullptr;
    size_t bytes = 0;
    bool busy = false;
    double last_use = 0.0;        // server clock of its last launch (eviction order)
    int last_slot = -1;
    std::deque<SRequest> fifo;
    std::vector<int32_t> stamp;   // dedupe of a request's edits
    int32_t gen = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_done = nullptr;
    uint8_t* h_pack = nullptr;
    size_t h_cap = 0;
    std::vector<uint8_t*> h_old;  // outgrown pinned packs, freed with the server (freeing pinned
                                  // memory synchronises the device, which would stall every launch)
    uint8_t* d_pack = nullptr;
    size_t d_cap = 0;
    unsigned long long* d_queue = nullptr;
    int* d_error = nullptr;
    int* h_error = nullptr;       // pinned
    RayResult* d_ray_res = nullptr;
    bool busy = false;
    std::vector<SRequest> reqs;
    std::vector<int> probes;
    double start = 0.0;
    std::atomic<double> done{0.0};
    size_t reserved = 0;
};

void CUDART_CB slot_done(void* p) { static_cast<Slot*>(p)->done.store(clock_s(), std::memory_order_release); }

struct Server {
    LumRadServerSettings s{};
    int num_sms = 0;
    double t0 = 0.0;
    std::vector<SWorld> worlds;
    std::vector<std::unique_ptr<Slot>> slots;
    std::deque<LumRadCompletion> done;
    long long next_id = 0;
    long long pending = 0;
    size_t resident = 0, fixed = 0, inflight = 0;
    LumRadServerStats st{};
    Tuning tuning;
    // the device-resident request loop (settings.device_loop), or null
    struct DevLoopHost* dl = nullptr;
    // per-launch host scratch
    std::vector<EditRecord> erec;
    std::vector<short4> lists;
    std::vector<uint64_t> bits_a, bits_b;
    std::vector<int> kept;

    double now() const { return clock_s() - t0; }
    size_t budget() const { return s.hbm_budget_bytes > 0 ? (size_t)s.hbm_budget_bytes : (size_t)-1; }

    // device bytes a request needs while its launch runs (upper bound, before its list is built)
    size_t request_bytes(const SRequest& r) const {
        const DeviceWorld& dw = worlds[r.world].ctx->world;
        const size_t side = 2 * (size_t)s.radius + 1;
        const size_t probes = std::min(dw.W, r.edits.size() * side * side * side);
        return sizeof(WorldPass) + r.edits.size() * sizeof(EditRecord) + probes * sizeof(short4) + 512;
    }
};

Server* as_server(LumRadServer h) { return reinterpret_cast<Server*>(h); }

int grow_pinned(uint8_t** p, size_t* cap, size_t need, std::vector<uint8_t*>& old) {
    if (need <= *cap) return LUMRAD_OK;
    const size_t c = std::max(need, *cap * 2);
    uint8_t* q = nullptr;
    LUMRAD_TRY(cudaMallocHost(&q, c));
    if (*p) old.push_back(*p);
    *p = q;
    *cap = c;
    return LUMRAD_OK;
}

int retire(Server* sv) {
    for (size_t k = 0; k < sv->slots.size(); k++) {
        Slot& sl = *sv->slots[k];
        if (!sl.busy) continue;
        const cudaError_t q = cudaEventQuery(sl.ev_done);
        if (q == cudaErrorNotReady) continue;
        LUMRAD_TRY(q);
        const int err = *sl.h_error;
        if (err) {   // a warp's scheduler gave up: reset the slot's counters
            LUMRAD_TRY(cudaMemsetAsync(sl.d_queue, 0, kQueueWords * sizeof(unsigned long long), sl.stream));
            LUMRAD_TRY(cudaMemsetAsync(sl.d_error, 0, sizeof(int), sl.stream));
            for (auto& r : sl.reqs) {
                DeviceWorld& dw = sv->worlds[r.world].ctx->world;
                LUMRAD_TRY(cudaMemsetAsync(dw.d_probe_count, 0, dw.count_cap * sizeof(int), sl.stream));
            }
            LUMRAD_TRY(cudaStreamSynchronize(sl.stream));
        }
        const double t_done = sl.done.load(std::memory_order_acquire) - sv->t0;
        for (size_t j = 0; j < sl.reqs.size(); j++) {
            const SRequest& r = sl.reqs[j];
            LumRadCompletion c{};
            c.request = r.id;
            c.world = r.world;
            c.status = err ? LUMRAD_EDEVICE : LUMRAD_OK;
            c.probes = sl.probes[j];
            c.rays_per_probe = r.p.rays_per_probe;
            c.arrival_s = r.arrival;
            c.start_s = sl.start;
            c.done_s = t_done;
            sv->done.push_back(c);
            sv->worlds[r.world].busy = false;
            sv->st.requests++;
            sv->st.probes += (unsigned long long)sl.probes[j];
            sv->st.rays += (unsigned long long)sl.probes[j] * (unsigned long long)r.p.rays_per_probe;
        }
        sv->pending -= (long long)sl.reqs.size();
        sv->inflight -= sl.reserved;
        sl.reserved = 0;
        sl.reqs.clear();
        sl.busy = false;
    }
    return LUMRAD_OK;
}

void complete_now(Server* sv, const SRequest& r, int status) {
    LumRadCompletion c{};
    c.request = r.id;
    c.world = r.world;
    c.status = status;
    c.rays_per_probe = r.p.rays_per_probe;
    c.arrival_s = r.arrival;
    c.start_s = c.done_s = sv->now();
    sv->done.push_back(c);
    sv->pending--;
}

// Per-pass buffers of a world at their size for 256 rays, so the serving loop never reallocates them.
int prepare_world(DeviceWorld& dw, cudaStream_t stream) {
    int rc = dw.ensure_scratch(dw.W, 256, stream);
    if (rc) return rc;
    for (int R : {32, 64, 128, 256}) {
        const float4* d = nullptr;
        if ((rc = dw.ensure_dirs(R, stream, &d))) return rc;
    }
    return LUMRAD_OK;
}

// Evicts idle resident worlds, least recently used first and never one marked in `keep`, until
// `need` more device bytes fit the budget beside the resident worlds and the launches in flight.
// An evicted world keeps its grid, palette, materials and volume on the host.
int make_room(Server* sv, size_t need, const std::vector<char>& keep, bool* fits) {
    *fits = true;
    const size_t budget = sv->budget();
    if (budget == (size_t)-1) return LUMRAD_OK;
    while (sv->resident + sv->fixed + sv->inflight + need > budget) {
        int victim = -1;
        for (size_t w = 0; w < sv->worlds.size(); w++) {
            const SWorld& sw = sv->worlds[w];
            if (sw.ctx->world.evicted || sw.busy || keep[w]) continue;
            if (victim < 0 || sw.last_use < sv->worlds[victim].last_use) victim = (int)w;
        }
        if (victim < 0) {
            *fits = false;
            return LUMRAD_OK;
        }
        SWorld& v = sv->worlds[victim];
        int rc = v.ctx->world.evict(v.ctx->stream);
        if (rc) return rc;
        sv->resident -= v.bytes;
        sv->st.evictions++;
    }
    return LUMRAD_OK;
}

int readmit_world(Server* sv, SWorld& sw) {
    DeviceWorld& dw = sw.ctx->world;
    int rc = dw.readmit(sw.ctx->stream);
    if (rc) return rc;
    if ((rc = prepare_world(dw, sw.ctx->stream))) return rc;
    sw.bytes = dw.footprint();
    sv->resident += sw.bytes;
    sv->st.readmissions++;
    return LUMRAD_OK;
}

// Forms and enqueues one launch on slot `k`; *started = false if no request was due and fit.
// With `free_slots` launch slots idle, a launch takes at most 1/free_slots of the due requests,
// so under load several launches run at once and a finished one frees its worlds while the
// others still keep the GPU busy.
int launch(Server* sv, int k, int free_slots, bool* started) {
    NvtxRange range("lumrad server launch");
    *started = false;
    Slot& sl = *sv->slots[k];
    const double now = sv->now();
    const size_t budget = sv->budget();
    // candidates: the front request of each idle world, oldest submission first; a front request
    // past the queueing bound is shed (not run) and the world's next one considered
    std::vector<int> cand;
    const double bound = sv->s.max_queue_ms > 0.0f ? 1e-3 * sv->s.max_queue_ms : -1.0;
    for (size_t w = 0; w < sv->worlds.size(); w++) {
        SWorld& sw = sv->worlds[w];
        if (sw.busy) continue;
        while (bound >= 0.0 && !sw.fifo.empty() && now - sw.fifo.front().arrival > bound) {
            complete_now(sv, sw.fifo.front(), LUMRAD_ETIMEOUT);
            sw.fifo.pop_front();
            sv->st.shed++;
        }
        if (!sw.fifo.empty() && sw.fifo.front().arrival <= now) cand.push_back((int)w);
    }
    if (cand.empty()) return LUMRAD_OK;
    std::sort(cand.begin(), cand.end(),
              [&](int a, int b) { return sv->worlds[a].fifo.front().id < sv->worlds[b].fifo.front().id; });
    sl.reqs.clear();
    size_t bytes = 0;
    int cap = (int)((cand.size() + (size_t)free_slots - 1) / (size_t)free_slots);
    if (sv->s.max_requests_per_launch > 0) cap = std::min(cap, sv->s.max_requests_per_launch);
    std::vector<char> keep(sv->worlds.size(), 0);
    int rc;
    for (int w : cand) {
        SWorld& sw = sv->worlds[w];
        const bool resident = !sw.ctx->world.evicted;
        const size_t req = sv->request_bytes(sw.fifo.front());
        // can never fit: not even with every other world evicted and nothing in flight
        if (budget != (size_t)-1 && sv->fixed + sw.bytes + req > budget) {
            complete_now(sv, sw.fifo.front(), LUMRAD_ENOMEM);
            sw.fifo.pop_front();
            continue;
        }
        keep[w] = 1;
        bool fits = true;
        if ((rc = make_room(sv, bytes + req + (resident ? 0 : sw.bytes), keep, &fits))) return rc;
        if (!fits) {   // waits for launches in flight to retire
            keep[w] = 0;
            continue;
        }
        if (!resident && (rc = readmit_world(sv, sw))) return rc;
        bytes += req;
        sw.last_use = now;
        sl.reqs.push_back(std::move(sw.fifo.front()));
        sw.fifo.pop_front();
        if ((int)sl.reqs.size() >= cap) break;
    }
    const int nl = (int)sl.reqs.size();
    if (nl == 0) return LUMRAD_OK;

    // host side of each request: edits, then its dirty-probe list
    sv->erec.clear();
    sv->lists.clear();
    std::vector<size_t> list_off(nl);
    sl.probes.assign(nl, 0);
    for (int j = 0; j < nl; j++) {
        SRequest& r = sl.reqs[j];
        SWorld& sw = sv->worlds[r.world];
        DeviceWorld& dw = sw.ctx->world;
        if (++sw.gen == 0x7fffffff) {
            std::fill(sw.stamp.begin(), sw.stamp.end(), 0);
            sw.gen = 1;
        }
        sv->kept.clear();
        for (int e = (int)r.edits.size() - 1; e >= 0; e--) {   // the last edit of a block wins
            const LumRadEdit& ed = r.edits[e];
            const size_t idx = (size_t)ed.x + (size_t)dw.X * ((size_t)ed.y + (size_t)dw.Y * ed.z);
            if (sw.stamp[idx] == sw.gen) continue;
            sw.stamp[idx] = sw.gen;
            sv->kept.push_back(e);
        }
        const size_t e0 = sv->erec.size();
        bool rebuild = false;
        for (int e : sv->kept) {
            const LumRadEdit& ed = r.edits[e];
            const size_t idx = (size_t)ed.x + (size_t)dw.X * ((size_t)ed.y + (size_t)dw.Y * ed.z);
            dw.h_grid[idx] = ed.block;
            bool assigned = false;
            const int c = dw.compact_of(ed.block, &assigned);
            if (c < 0) {
                rebuild = true;
                continue;
            }
            if (assigned) {   // a block id new to this world: upload its occupancy mask and slot
                LUMRAD_TRY(cudaMemcpyAsync(dw.d_cbits + (size_t)c * 128, dw.h_cbits.data() + (size_t)c * 128,
                                           128 * sizeof(uint32_t), cudaMemcpyHostToDevice, sl.stream));
                LUMRAD_TRY(cudaMemcpyAsync(dw.d_cslot + c, dw.h_cslot.data() + c, sizeof(int), cudaMemcpyHostToDevice,
                                           sl.stream));
            }
            sv->erec.push_back(EditRecord{j, (int)idx, (int)ed.block, c});
        }
        if (rebuild) {   // more than 256 distinct ids: rebuild with a uint16 compact grid
            sv->erec.resize(e0);
            dw.grid_dirty = true;
            if ((rc = dw.sync_inputs(sw.ctx->stream))) return rc;
        }
        list_off[j] = sv->lists.size();
        dirty_probes(dw.X, dw.Y, dw.Z, r.edits.data(), (int)r.edits.size(), sv->s.radius, sv->bits_a, sv->bits_b,
                     sv->lists);
        sl.probes[j] = (int)(sv->lists.size() - list_off[j]);
    }

    // one pinned pack: world table | edit records | lists
    const size_t off_e = align_up((size_t)nl * sizeof(WorldPass), 256);
    const size_t off_l = align_up(off_e + sv->erec.size() * sizeof(EditRecord), 256);
    const size_t total = off_l + sv->lists.size() * sizeof(short4);
    if ((rc = grow_pinned(&sl.h_pack, &sl.h_cap, total, sl.h_old))) return rc;
    if (total > sl.d_cap) {
        const size_t c = std::max(total, sl.d_cap * 2);
        if (sl.d_pack) LUMRAD_TRY(cudaFreeAsync(sl.d_pack, sl.stream));
        sl.d_pack = nullptr;
        sl.d_cap = 0;
        LUMRAD_TRY(cudaMallocAsync(reinterpret_cast<void**>(&sl.d_pack), c, sl.stream));
        sl.d_cap = c;
    }
    WorldPass* table = reinterpret_cast<WorldPass*>(sl.h_pack);
    const WorldPass* d_table = reinterpret_cast<const WorldPass*>(sl.d_pack);
    const short4* d_lists = reinterpret_cast<const short4*>(sl.d_pack + off_l);
    long long begin = 0;
    for (int j = 0; j < nl; j++) {
        SRequest& r = sl.reqs[j];
        DeviceWorld& dw = sv->worlds[r.world].ctx->world;
        LumRadPassParams p = r.p;
        p.size = 1;
        p.shift = 0;
        p.record_hits = 0;
        WorldPass w;
        if ((rc = dw.fill_pass(d_lists + list_off[j], sl.probes[j], p, sl.stream, &w))) return rc;
        w.task_begin = begin;
        begin += (w.n_tasks + kWarps - 1) / kWarps * kWarps;
        table[j] = w;
    }
    if (!sv->erec.empty()) std::memcpy(sl.h_pack + off_e, sv->erec.data(), sv->erec.size() * sizeof(EditRecord));
    if (!sv->lists.empty()) std::memcpy(sl.h_pack + off_l, sv->lists.data(), sv->lists.size() * sizeof(short4));

    LUMRAD_TRY(cudaMemcpyAsync(sl.d_pack, sl.h_pack, total, cudaMemcpyHostToDevice, sl.stream));
    LUMRAD_TRY(launch_apply_edits(d_table, reinterpret_cast<const EditRecord*>(sl.d_pack + off_e),
                                  (int)sv->erec.size(), sl.stream));
    LUMRAD_TRY(launch_prep(d_table, nl, sv->s.precision, sl.stream));
    LaunchArgs la;
    std::memset(&la, 0, sizeof la);
    la.worlds = d_table;
    la.n_worlds = nl;
    la.n_tasks = begin;
    la.queue = sl.d_queue;
    la.error = sl.d_error;
    la.ray_res = sl.d_ray_res;
    la.in_cta = combines_in_cta(table, nl) ? 1 : 0;
    la.guided_div = sv->tuning.guided_div;
    la.max_chunk = sv->tuning.max_chunk;
    la.march_ctas = sv->tuning.march_ctas;
    LUMRAD_TRY(launch_radiance(la, sv->s.precision, false, sv->num_sms, sl.stream));
    LUMRAD_TRY(cudaMemcpyAsync(sl.h_error, sl.d_error, sizeof(int), cudaMemcpyDeviceToHost, sl.stream));
    LUMRAD_TRY(cudaLaunchHostFunc(sl.stream, slot_done, &sl));
    LUMRAD_TRY(cudaEventRecord(sl.ev_done, sl.stream));

    for (int j = 0; j < nl; j++) {
        SWorld& sw = sv->worlds[sl.reqs[j].world];
        sw.busy = true;
        sw.last_slot = k;
        sw.ctx->world.cur = 1 - sw.ctx->world.cur;
        sw.ctx->have_pass = true;
        sw.ctx->last_count_on_device = false;
    }
    sl.busy = true;
    sl.start = now;
    sl.reserved = bytes;
    sv->inflight += bytes;
    sv->st.launches++;
    sv->st.max_requests_in_launch = std::max(sv->st.max_requests_in_launch, nl);
    sv->st.peak_inflight_bytes = std::max(sv->st.peak_inflight_bytes, (double)sv->inflight);
    sv->st.peak_device_bytes =
        std::max(sv->st.peak_device_bytes, (double)(sv->resident + sv->fixed + sv->inflight));
    *started = true;
    return LUMRAD_OK;
}

int devloop_progress(Server* sv);

int progress(Server* sv) {
    if (sv->dl) return devloop_progress(sv);
    int rc = retire(sv);
    if (rc) return rc;
    int free_slots = 0;
    for (auto& sl : sv->slots) free_slots += sl->busy ? 0 : 1;
    for (size_t k = 0; k < sv->slots.size() && free_slots > 0; k++) {
        if (sv->slots[k]->busy) continue;
        bool started = false;
        if ((rc = launch(sv, (int)k, free_slots, &started))) return rc;
        if (!started) break;
        free_slots--;
    }
    return LUMRAD_OK;
}

// ---------------------------------------------------------------- device-resident loop
// The host side of the loop of radiance_serve.cu: requests wait here in submission order until
// due, then are copied into a page-locked ring (their edits into an edit arena) and the ring's
// head is published; the GPU's completion records are read back from another ring.  The host
// makes no CUDA call per request: it starts a loop's graph again only when that loop has ended
// (no request within poll_ms) and a published request waits.  Worlds are split over kDevLanes
// independent loops (world w in lane w % kDevLanes), each with its own rings, stream, graph and
// ray buffer, so one lane's small kernels and its pass's drain overlap the other's pass; a world's
// requests stay in one lane, in order.
constexpr int kDevLanes = 2;

struct DevLane {
    struct Published {
        long long id;
        int world, rays;
        double arrival, start;
    };
    DevRequest* ring = nullptr;          // page-locked, mapped (host pointers; the device's below)
    LumRadEdit* edits = nullptr;
    DevCompletion* done = nullptr;
    long long* ctl = nullptr;            // [0] head, [1] tail (taken by the loop), [2] done head, [3] stop
    DevRequest* d_ring = nullptr;
    LumRadEdit* d_edits = nullptr;
    DevCompletion* d_done = nullptr;
    long long* d_ctl = nullptr;
    long long head = 0, done_read = 0, edit_head = 0, edit_tail = 0;
    // published, not yet completed, by id (the loop completes a request in the iteration that runs
    // it, and holds back a request whose world is already in that iteration's batch); and the ids
    // in publish order with each one's arena position after its edits (the arena is freed up to
    // the oldest request not completed)
    std::unordered_map<long long, Published> published;
    std::deque<std::pair<long long, long long>> pub_order;
    DevLoop* d_loop = nullptr;
    int* d_chunk_count = nullptr;
    int* d_chunk_off = nullptr;
    long long chunk_cap = 0, chunks_total = 0;
    int* d_error = nullptr;
    unsigned long long* d_queue = nullptr;
    RayResult* d_ray_res = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_end = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool running = false;
};

struct DevLoopHost {
    long long ring_cap = 1 << 16, edit_cap = 1 << 22;
    long long max_tasks = 1 << 20;       // per lane and iteration
    DevLane lanes[kDevLanes];
    std::deque<SRequest> queue;          // submitted, not yet published
    std::vector<int> outstanding;        // per world: published, not completed
    DevWorld* d_worlds = nullptr;
    std::vector<void*> bufs;             // per-world device buffers of the loop
    double offset_s = 0.0;               // host clock = %globaltimer * 1e-9 - offset_s
    unsigned long long* h_timer = nullptr;
};

template <class T>
int host_mapped(T** h, T** d, size_t n) {
    LUMRAD_TRY(cudaHostAlloc(reinterpret_cast<void**>(h), n * sizeof(T), cudaHostAllocMapped));
    std::memset(static_cast<void*>(*h), 0, n * sizeof(T));
    LUMRAD_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(d), *h, 0));
    return LUMRAD_OK;
}

volatile long long& ctl_word(DevLane& ln, int k) { return reinterpret_cast<volatile long long*>(ln.ctl)[k]; }

int devloop_lane_create(Server* sv, DevLoopHost& dl, DevLane& ln) {
    int rc;
    if ((rc = host_mapped(&ln.ring, &ln.d_ring, (size_t)dl.ring_cap))) return rc;
    if ((rc = host_mapped(&ln.edits, &ln.d_edits, (size_t)dl.edit_cap))) return rc;
    if ((rc = host_mapped(&ln.done, &ln.d_done, (size_t)dl.ring_cap))) return rc;
    if ((rc = host_mapped(&ln.ctl, &ln.d_ctl, 8))) return rc;
    LUMRAD_TRY(cudaStreamCreateWithFlags(&ln.stream, cudaStreamNonBlocking));
    LUMRAD_TRY(cudaEventCreateWithFlags(&ln.ev_end, cudaEventDisableTiming));
    LUMRAD_TRY(cudaMalloc(&ln.d_loop, sizeof(DevLoop)));
    LUMRAD_TRY(cudaMalloc(&ln.d_error, sizeof(int)));
    LUMRAD_TRY(cudaMalloc(&ln.d_queue, kQueueWords * sizeof(unsigned long long)));
    LUMRAD_TRY(cudaMalloc(&ln.d_ray_res, (size_t)dl.max_tasks * kTaskRays * sizeof(RayResult)));
    LUMRAD_TRY(cudaMemsetAsync(ln.d_error, 0, sizeof(int), ln.stream));
    LUMRAD_TRY(cudaMemsetAsync(ln.d_queue, 0, kQueueWords * sizeof(unsigned long long), ln.stream));
    std::unique_ptr<DevLoop> h(new DevLoop());
    std::memset(static_cast<void*>(h.get()), 0, sizeof(DevLoop));
    h->ring = ln.d_ring;
    h->ring_cap = dl.ring_cap;
    h->head = ln.d_ctl;
    h->tail_host = ln.d_ctl + 1;
    h->edits = ln.d_edits;
    h->edit_cap = dl.edit_cap;
    h->done = ln.d_done;
    h->done_head = ln.d_ctl + 2;
    h->stop = reinterpret_cast<const int*>(ln.d_ctl + 3);
    h->worlds = dl.d_worlds;
    h->poll_ns = (unsigned long long)((sv->s.poll_ms > 0.0f ? sv->s.poll_ms : 2.0f) * 1e6);
    h->max_tasks = dl.max_tasks;
    h->radius = sv->s.radius;
    h->error = ln.d_error;
    h->queue = ln.d_queue;
    h->iteration = 1;
    LUMRAD_TRY(cudaMemcpyAsync(ln.d_loop, h.get(), sizeof(DevLoop), cudaMemcpyHostToDevice, ln.stream));
    LUMRAD_TRY(cudaStreamSynchronize(ln.stream));

    // the graph: one WHILE node whose body is one iteration of the loop
    LUMRAD_TRY(cudaGraphCreate(&ln.graph, 0));
    cudaGraphConditionalHandle cond;
    LUMRAD_TRY(cudaGraphConditionalHandleCreate(&cond, ln.graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    LUMRAD_TRY(cudaGraphAddNode(&node, ln.graph, nullptr, nullptr, 0, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    DevLoopLaunch a;
    std::memset(static_cast<void*>(&a), 0, sizeof a);
    char* base = reinterpret_cast<char*>(ln.d_loop);
    a.table = reinterpret_cast<const WorldPass*>(base + offsetof(DevLoop, table));
    a.n_table = reinterpret_cast<const int*>(base + offsetof(DevLoop, n_table));
    a.precision = sv->s.precision;
    a.num_sms = sv->num_sms;
    LaunchArgs& la = a.pass;
    la.worlds = a.table;
    la.n_worlds = kDevBatch;
    la.dev_n_worlds = a.n_table;
    la.dev_total = reinterpret_cast<const long long*>(base + offsetof(DevLoop, total_tasks));
    la.n_tasks = dl.max_tasks;
    la.queue = ln.d_queue;
    la.error = ln.d_error;
    la.ray_res = ln.d_ray_res;
    la.in_cta = 1;
    LUMRAD_TRY(cudaStreamBeginCaptureToGraph(ln.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const cudaError_t ce = capture_devloop_body(ln.d_loop, a, cond, ln.stream);
    const cudaError_t ee = cudaStreamEndCapture(ln.stream, &body);
    LUMRAD_TRY(ce);
    LUMRAD_TRY(ee);
    LUMRAD_TRY(cudaGraphInstantiate(&ln.exec, ln.graph, 0));
    sv->fixed += (size_t)dl.max_tasks * kTaskRays * sizeof(RayResult) + sizeof(DevLoop);
    return LUMRAD_OK;
}

int devloop_create(Server* sv) {
    DevLoopHost* dl = new DevLoopHost();
    sv->dl = dl;
    int rc;
    LUMRAD_TRY(cudaMalloc(&dl->d_worlds, kDevMaxWorlds * sizeof(DevWorld)));
    sv->fixed += kDevMaxWorlds * sizeof(DevWorld);
    for (DevLane& ln : dl->lanes)
        if ((rc = devloop_lane_create(sv, *dl, ln))) return rc;
    // the device clock against the host's: the read with the shortest round trip
    unsigned long long* d_timer = nullptr;
    if ((rc = host_mapped(&dl->h_timer, &d_timer, 1))) return rc;
    double best = 1e9;
    for (int i = 0; i < 20; i++) {
        const double t0 = clock_s();
        LUMRAD_TRY(launch_read_globaltimer(d_timer, dl->lanes[0].stream));
        LUMRAD_TRY(cudaStreamSynchronize(dl->lanes[0].stream));
        const double t1 = clock_s();
        if (t1 - t0 < best) {
            best = t1 - t0;
            dl->offset_s = (double)*reinterpret_cast<volatile unsigned long long*>(dl->h_timer) * 1e-9 - 0.5 * (t0 + t1);
        }
    }
    return LUMRAD_OK;
}

// Ends a lane's loop (it stops at its next admit) and waits for it; the flag is cleared again.
int devloop_halt(DevLane& ln) {
    if (!ln.running) return LUMRAD_OK;
    ctl_word(ln, 3) = 1;
    const cudaError_t e = cudaStreamSynchronize(ln.stream);
    ctl_word(ln, 3) = 0;
    ln.running = false;
    LUMRAD_TRY(e);
    return LUMRAD_OK;
}

int devloop_add_world(Server* sv, Context* c, int id, size_t* bytes) {
    DevLoopHost& dl = *sv->dl;
    DevLane& ln = dl.lanes[id % kDevLanes];
    DeviceWorld& dw = c->world;
    if (id >= kDevMaxWorlds) return fail(LUMRAD_EINVAL, "the device loop holds at most 1024 worlds");
    if (dw.n_slots > 192) return fail(LUMRAD_EINVAL, "the device loop needs max_block_types <= 192");
    if ((long long)dw.W > dl.max_tasks) return fail(LUMRAD_EINVAL, "world too large for the device loop (2^20 blocks)");
    if (dw.cgrid_wide) return fail(LUMRAD_EINVAL, "the device loop needs at most 256 distinct block ids");
    int rc = devloop_halt(ln);
    if (rc) return rc;
    // every id with a palette slot, and the shared empty id, gets its compact id now: the loop's
    // edits then only look ids up
    bool assigned = false;
    for (int b = -63; b < dw.n_slots; b++)
        if (b != 0 && dw.compact_of((int16_t)b, &assigned) < 0) return fail(LUMRAD_EINVAL, "too many block ids");
    if (dw.compact_of((int16_t)-64, &assigned) < 0) return fail(LUMRAD_EINVAL, "too many block ids");
    LUMRAD_TRY(cudaMemcpyAsync(dw.d_cbits, dw.h_cbits.data(), dw.h_cbits.size() * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, c->stream));
    LUMRAD_TRY(cudaMemcpyAsync(dw.d_cslot, dw.h_cslot.data(), dw.h_cslot.size() * sizeof(int), cudaMemcpyHostToDevice,
                               c->stream));
    std::vector<int16_t> cmap((size_t)dw.n_slots + 64);
    for (int b = -64; b < dw.n_slots; b++) cmap[(size_t)(b + 64)] = (int16_t)dw.id_to_c[(uint16_t)(int16_t)b];
    int16_t* d_cmap = nullptr;
    uint8_t* d_mask = nullptr;
    unsigned long long* d_stamp = nullptr;
    short4* d_list = nullptr;
    LUMRAD_TRY(cudaMalloc(&d_cmap, cmap.size() * sizeof(int16_t)));
    dl.bufs.push_back(d_cmap);
    LUMRAD_TRY(cudaMalloc(&d_mask, dw.W));
    dl.bufs.push_back(d_mask);
    LUMRAD_TRY(cudaMalloc(&d_stamp, dw.W * sizeof(unsigned long long)));
    dl.bufs.push_back(d_stamp);
    LUMRAD_TRY(cudaMalloc(&d_list, dw.W * sizeof(short4)));
    dl.bufs.push_back(d_list);
    LUMRAD_TRY(cudaMemcpyAsync(d_cmap, cmap.data(), cmap.size() * sizeof(int16_t), cudaMemcpyHostToDevice, c->stream));
    LUMRAD_TRY(cudaMemsetAsync(d_mask, 0, dw.W, c->stream));
    LUMRAD_TRY(cudaMemsetAsync(d_stamp, 0, dw.W * sizeof(unsigned long long), c->stream));
    DevWorld w;
    std::memset(static_cast<void*>(&w), 0, sizeof w);
    LumRadPassParams p{64, 128.0f, 0.1f, 0, 1, 0, 0};
    if ((rc = dw.fill_pass(nullptr, 0, p, c->stream, &w.pass))) return rc;
    const int rs[4] = {32, 64, 128, 256};
    for (int k = 0; k < 4; k++) {
        const float4* d = nullptr;
        if ((rc = dw.ensure_dirs(rs[k], c->stream, &d))) return rc;
        w.dirs[k] = d;
    }
    w.cmap = d_cmap;
    w.n_cmap = (int)cmap.size();
    w.empty_c = dw.id_to_c[(uint16_t)(int16_t)-64];
    w.mask = d_mask;
    w.stamp = d_stamp;
    w.list = d_list;
    w.rad[0] = dw.d_rad[0];
    w.rad[1] = dw.d_rad[1];
    w.cur = dw.cur;
    LUMRAD_TRY(cudaMemcpyAsync(dl.d_worlds + id, &w, sizeof w, cudaMemcpyHostToDevice, c->stream));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    // the lane's chunk arrays: room for its worlds' chunks (a batch holds each world at most once)
    ln.chunks_total += ((long long)dw.W + kDevChunk - 1) / kDevChunk;
    if (ln.chunks_total > ln.chunk_cap) {
        const long long cap = std::max(ln.chunks_total, 2 * ln.chunk_cap);
        cudaFree(ln.d_chunk_count);
        cudaFree(ln.d_chunk_off);
        ln.d_chunk_count = ln.d_chunk_off = nullptr;
        LUMRAD_TRY(cudaMalloc(&ln.d_chunk_count, cap * sizeof(int)));
        LUMRAD_TRY(cudaMalloc(&ln.d_chunk_off, cap * sizeof(int)));
        ln.chunk_cap = cap;
        int* ptrs[2] = {ln.d_chunk_count, ln.d_chunk_off};
        LUMRAD_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(ln.d_loop) + offsetof(DevLoop, chunk_count), ptrs,
                                   sizeof ptrs, cudaMemcpyHostToDevice, ln.stream));
        LUMRAD_TRY(cudaStreamSynchronize(ln.stream));
    }
    dl.outstanding.resize((size_t)id + 1, 0);
    *bytes = dw.W * (1 + sizeof(unsigned long long) + sizeof(short4)) + cmap.size() * sizeof(int16_t);
    return LUMRAD_OK;
}

int devloop_progress(Server* sv) {
    DevLoopHost& dl = *sv->dl;
    // completions the GPU wrote
    for (DevLane& ln : dl.lanes) {
        const long long dh = ctl_word(ln, 2);
        std::atomic_thread_fence(std::memory_order_acquire);
        for (; ln.done_read < dh; ln.done_read++) {
            const DevCompletion& c = ln.done[ln.done_read % dl.ring_cap];
            const auto it = ln.published.find(c.id);
            if (it == ln.published.end()) return fail(LUMRAD_EDEVICE, "the device loop completed an unknown request");
            const DevLane::Published pr = it->second;
            ln.published.erase(it);
            LumRadCompletion o{};
            o.request = pr.id;
            o.world = pr.world;
            o.status = c.status;
            o.probes = c.probes;
            o.rays_per_probe = pr.rays;
            o.arrival_s = pr.arrival;
            o.start_s = pr.start;
            o.done_s = (double)c.t_done_ns * 1e-9 - dl.offset_s - sv->t0;
            sv->done.push_back(o);
            sv->pending--;
            dl.outstanding[pr.world]--;
            sv->st.requests++;
            sv->st.probes += (unsigned long long)c.probes;
            sv->st.rays += (unsigned long long)c.probes * (unsigned long long)pr.rays;
        }
        while (!ln.pub_order.empty() && !ln.published.count(ln.pub_order.front().first)) {
            ln.edit_tail = ln.pub_order.front().second;
            ln.pub_order.pop_front();
        }
    }
    // due requests into their lanes' rings, in submission order.  With a queueing bound a lane
    // holds at most two iterations' requests published (the rest wait here, where a request past
    // the bound is shed rather than published)
    const double now = sv->now();
    const double bound = sv->s.max_queue_ms > 0.0f ? 1e-3 * sv->s.max_queue_ms : -1.0;
    const long long window = bound >= 0.0 ? 2LL * kDevBatch : dl.ring_cap;
    bool published[kDevLanes] = {};
    while (!dl.queue.empty()) {
        SRequest& r = dl.queue.front();
        if (r.arrival > now) break;
        if (bound >= 0.0 && now - r.arrival > bound) {
            complete_now(sv, r, LUMRAD_ETIMEOUT);
            dl.queue.pop_front();
            sv->st.shed++;
            continue;
        }
        DevLane& ln = dl.lanes[r.world % kDevLanes];
        const long long ne = (long long)r.edits.size();
        if (ln.head - ln.done_read >= std::min(window, dl.ring_cap) || ne > dl.edit_cap - (ln.edit_head - ln.edit_tail))
            break;
        for (long long k = 0; k < ne; k++) ln.edits[(ln.edit_head + k) % dl.edit_cap] = r.edits[(size_t)k];
        DevRequest& q = ln.ring[ln.head % dl.ring_cap];
        q.id = r.id;
        q.edit_off = ln.edit_head % dl.edit_cap;
        q.world = r.world;
        q.n_edits = (int)ne;
        q.rays = r.p.rays_per_probe;
        q.time_seed = r.p.time_seed;
        q.max_dist = r.p.max_dist;
        q.blend = r.p.blend;
        ln.edit_head += ne;
        ln.pub_order.emplace_back(r.id, ln.edit_head);
        ln.published.emplace(r.id, DevLane::Published{r.id, r.world, r.p.rays_per_probe, r.arrival, now});
        dl.outstanding[r.world]++;
        ln.head++;
        published[r.world % kDevLanes] = true;
        dl.queue.pop_front();
    }
    for (int l = 0; l < kDevLanes; l++) {
        DevLane& ln = dl.lanes[l];
        if (published[l]) {
            std::atomic_thread_fence(std::memory_order_release);   // the entries before the head
            ctl_word(ln, 0) = ln.head;
        }
        // the loop ended (no request within poll_ms): start it again if a published request waits
        if (ln.running) {
            const cudaError_t q = cudaEventQuery(ln.ev_end);
            if (q == cudaSuccess) ln.running = false;
            else if (q != cudaErrorNotReady) LUMRAD_TRY(q);
        }
        if (!ln.running && ln.head > ln.done_read) {
            LUMRAD_TRY(cudaGraphLaunch(ln.exec, ln.stream));
            LUMRAD_TRY(cudaEventRecord(ln.ev_end, ln.stream));
            ln.running = true;
            sv->st.launches++;
        }
    }
    return LUMRAD_OK;
}

void devloop_destroy(Server* sv) {
    DevLoopHost* dl = sv->dl;
    if (!dl) return;
    for (DevLane& ln : dl->lanes)
        if (ln.ctl) {
            ctl_word(ln, 3) = 1;
            if (ln.stream) cudaStreamSynchronize(ln.stream);
        }
    // the worlds go back to their contexts as the loop left them: volume side and grid
    for (size_t w = 0; w < sv->worlds.size() && dl->d_worlds && w < dl->outstanding.size(); w++) {
        DeviceWorld& dw = sv->worlds[w].ctx->world;
        int cur = dw.cur;
        if (cudaMemcpy(&cur, &dl->d_worlds[w].cur, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess) dw.cur = cur;
        if (cudaMemcpy(dw.h_grid.data(), dw.d_grid, dw.W * sizeof(int16_t), cudaMemcpyDeviceToHost) == cudaSuccess)
            dw.grid_dirty = true;
    }
    for (DevLane& ln : dl->lanes) {
        if (ln.exec) cudaGraphExecDestroy(ln.exec);
        if (ln.graph) cudaGraphDestroy(ln.graph);
        cudaFree(ln.d_chunk_count);
        cudaFree(ln.d_chunk_off);
        cudaFree(ln.d_ray_res);
        cudaFree(ln.d_queue);
        cudaFree(ln.d_error);
        cudaFree(ln.d_loop);
        if (ln.ring) cudaFreeHost(ln.ring);
        if (ln.edits) cudaFreeHost(ln.edits);
        if (ln.done) cudaFreeHost(ln.done);
        if (ln.ctl) cudaFreeHost(ln.ctl);
        if (ln.ev_end) cudaEventDestroy(ln.ev_end);
        if (ln.stream) cudaStreamDestroy(ln.stream);
    }
    for (void* p : dl->bufs) cudaFree(p);
    cudaFree(dl->d_worlds);
    if (dl->h_timer) cudaFreeHost(dl->h_timer);
    delete dl;
    sv->dl = nullptr;
}

void destroy_server(Server* sv) {
    cudaSetDevice(sv->s.device);
    devloop_destroy(sv);
    for (auto& slp : sv->slots) {
        Slot& sl = *slp;
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.d_pack) cudaFreeAsync(sl.d_pack, sl.stream);
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.h_pack) cudaFreeHost(sl.h_pack);
        for (uint8_t* p : sl.h_old) cudaFreeHost(p);
        if (sl.h_error) cudaFreeHost(sl.h_error);
        cudaFree(sl.d_queue);
        cudaFree(sl.d_error);
        cudaFree(sl.d_ray_res);
        if (sl.ev_done) cudaEventDestroy(sl.ev_done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    for (auto& w : sv->worlds) {   // contexts go back to their callers resident and usable
        if (w.ctx->world.evicted) w.ctx->world.readmit(w.ctx->stream);
        w.ctx->owner = nullptr;
    }
    delete sv;
}

}  // namespace
}  // namespace lumrad

using namespace lumrad;

extern "C" {

int lumrad_dirty_probes(const int* world_size, const LumRadEdit* edits, int n_edits, int radius, int16_t* out,
                        int cap, int* n) {
    if (!world_size || !n || (n_edits > 0 && !edits) || (cap > 0 && !out) || n_edits < 0)
        return fail(LUMRAD_EINVAL, "bad argument");
    const int X = world_size[0], Y = world_size[1], Z = world_size[2];
    if (X < 1 || Y < 1 || Z < 1 || X > 2047 || Y > 2047 || Z > 2047) return fail(LUMRAD_EINVAL, "bad world size");
    if (radius < 0 || radius > 15) return fail(LUMRAD_EINVAL, "radius must be in [0, 15]");
    for (int k = 0; k < n_edits; k++)
        if (edits[k].x < 0 || edits[k].y < 0 || edits[k].z < 0 || edits[k].x >= X || edits[k].y >= Y || edits[k].z >= Z)
            return fail(LUMRAD_EINVAL, "edit outside the world");
    std::vector<uint64_t> a, b;
    std::vector<short4> list;
    dirty_probes(X, Y, Z, edits, n_edits, radius, a, b, list);
    const int total = (int)list.size();
    if (cap > 0) std::memcpy(out, list.data(), (size_t)std::min(total, cap) * sizeof(short4));
    *n = total;
    return LUMRAD_OK;
}

int lumrad_server_create(const LumRadServerSettings* s, LumRadServer* out) {
    if (!s || !out) return fail(LUMRAD_EINVAL, "null argument");
    *out = nullptr;
    if (s->precision < 0 || s->precision > LUMRAD_PRECISION_RGB10A2) return fail(LUMRAD_EINVAL, "unknown precision");
    if (s->max_inflight < 0 || s->max_inflight > 8) return fail(LUMRAD_EINVAL, "max_inflight must be in [0, 8]");
    if (s->radius < 0 || s->radius > 15) return fail(LUMRAD_EINVAL, "radius must be in [0, 15]");
    if (s->hbm_budget_bytes < 0 || s->max_requests_per_launch < 0) return fail(LUMRAD_EINVAL, "negative limit");
    if (s->device_loop != 0 && s->device_loop != 1) return fail(LUMRAD_EINVAL, "device_loop must be 0 or 1");
    if (!(s->poll_ms >= 0.0f && s->poll_ms <= 1000.0f)) return fail(LUMRAD_EINVAL, "poll_ms must be in [0, 1000]");
    if (!(s->max_queue_ms >= 0.0f && s->max_queue_ms <= 3.6e6f)) return fail(LUMRAD_EINVAL, "max_queue_ms must be in [0, 3.6e6]");
    Server* sv = new Server();
    sv->s = *s;
    if (sv->s.max_inflight == 0) sv->s.max_inflight = 4;
    sv->t0 = clock_s();
    auto attempt = [&]() -> int {
        LUMRAD_TRY(cudaSetDevice(s->device));
        LUMRAD_TRY(cudaDeviceGetAttribute(&sv->num_sms, cudaDevAttrMultiProcessorCount, s->device));
        if (s->device_loop) {
            int rc = devloop_create(sv);
            if (rc) return rc;
            if (sv->fixed > sv->budget()) return fail(LUMRAD_ENOMEM, "the loop's buffers alone exceed the HBM budget");
            return LUMRAD_OK;
        }
        const size_t rays = (size_t)kChunkTasks * kTaskRays;
        for (int k = 0; k < sv->s.max_inflight; k++) {
            sv->slots.emplace_back(new Slot());
            Slot& sl = *sv->slots.back();
            LUMRAD_TRY(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking));
            LUMRAD_TRY(cudaEventCreateWithFlags(&sl.ev_done, cudaEventDisableTiming));
            LUMRAD_TRY(cudaMalloc(&sl.d_queue, kQueueWords * sizeof(unsigned long long)));
            LUMRAD_TRY(cudaMalloc(&sl.d_error, sizeof(int)));
            LUMRAD_TRY(cudaMallocHost(&sl.h_error, sizeof(int)));
            *sl.h_error = 0;
            LUMRAD_TRY(cudaMemsetAsync(sl.d_queue, 0, kQueueWords * sizeof(unsigned long long), sl.stream));
            LUMRAD_TRY(cudaMemsetAsync(sl.d_error, 0, sizeof(int), sl.stream));
            LUMRAD_TRY(cudaMalloc(&sl.d_ray_res, rays * sizeof(RayResult)));
            // request packs sized up front so the serving loop rarely grows them
            const size_t pack = (size_t)16 << 20;
            LUMRAD_TRY(cudaMallocHost(&sl.h_pack, pack));
            sl.h_cap = pack;
            LUMRAD_TRY(cudaMallocAsync(reinterpret_cast<void**>(&sl.d_pack), pack, sl.stream));
            sl.d_cap = pack;
            LUMRAD_TRY(cudaStreamSynchronize(sl.stream));
            sv->fixed += rays * sizeof(RayResult) + pack + 2 * sizeof(unsigned long long) + sizeof(int);
        }
        if (sv->fixed > sv->budget()) return fail(LUMRAD_ENOMEM, "the launch buffers alone exceed the HBM budget");
        return LUMRAD_OK;
    };
    const int rc = attempt();
    if (rc) {
        const std::string msg = g_error;
        destroy_server(sv);
        return fail(rc, msg);
    }
    sv->st.launch_bytes = (double)sv->fixed;
    *out = sv;
    return LUMRAD_OK;
}

void lumrad_server_destroy(LumRadServer server) {
    Server* sv = as_server(server);
    if (sv) destroy_server(sv);
}

int lumrad_server_add_world(LumRadServer server, LumRadContext world, int* id) {
    Server* sv = as_server(server);
    Context* c = as_ctx(world);
    if (!sv || !c || !id) return fail(LUMRAD_EINVAL, "null argument");
    if (c->device != sv->s.device) return fail(LUMRAD_EINVAL, "the world is on another device");
    if (c->world.precision != sv->s.precision) return fail(LUMRAD_EINVAL, "the world has another precision");
    if (c->owner) return fail(LUMRAD_ESTATE, "the world already belongs to a server");
    LUMRAD_TRY(cudaSetDevice(sv->s.device));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    DeviceWorld& dw = c->world;
    if (!dw.h_cur.empty()) dw.grid_dirty = true;   // a blockified frame is dropped: edits apply to the loaded world
    int rc = dw.sync_inputs(c->stream);
    if (rc) return rc;
    if ((rc = prepare_world(dw, c->stream))) return rc;
    size_t bytes = dw.footprint();
    if (sv->dl) {   // the device loop keeps every world resident
        size_t extra = 0;
        if (sv->resident + sv->fixed + bytes > sv->budget())
            return fail(LUMRAD_ENOMEM, "the world does not fit the HBM budget (the device loop does not evict)");
        if ((rc = devloop_add_world(sv, c, (int)sv->worlds.size(), &extra))) return rc;
        bytes += extra;
    } else {
        if (sv->fixed + bytes > sv->budget()) return fail(LUMRAD_ENOMEM, "the world does not fit the HBM budget");
        bool fits = true;
        if ((rc = make_room(sv, bytes, std::vector<char>(sv->worlds.size(), 0), &fits))) return rc;
        if (!fits) return fail(LUMRAD_ENOMEM, "the world does not fit the HBM budget beside the busy worlds");
    }
    SWorld w;
    w.ctx = c;
    w.bytes = bytes;
    w.stamp.assign(dw.W, 0);
    sv->worlds.push_back(std::move(w));
    sv->resident += bytes;
    sv->st.peak_device_bytes = std::max(sv->st.peak_device_bytes, (double)(sv->resident + sv->fixed + sv->inflight));
    sv->st.resident_bytes = (double)sv->resident;
    c->owner = sv;
    *id = (int)sv->worlds.size() - 1;
    return LUMRAD_OK;
}

int lumrad_server_submit(LumRadServer server, int world, const LumRadEdit* edits, int n_edits,
                         const LumRadPassParams* params, double arrival_s, long long* request) {
    Server* sv = as_server(server);
    if (!sv || !request || (n_edits > 0 && !edits) || n_edits < 0) return fail(LUMRAD_EINVAL, "bad argument");
    if (world < 0 || world >= (int)sv->worlds.size()) return fail(LUMRAD_EINVAL, "unknown world");
    int rc = check_params(params);
    if (rc) return rc;
    const DeviceWorld& dw = sv->worlds[world].ctx->world;
    for (int k = 0; k < n_edits; k++)
        if (edits[k].x < 0 || edits[k].y < 0 || edits[k].z < 0 || edits[k].x >= dw.X || edits[k].y >= dw.Y ||
            edits[k].z >= dw.Z)
            return fail(LUMRAD_EINVAL, "edit outside the world");
    if (sv->dl) {
        const int R = params->rays_per_probe;
        if (R != 32 && R != 64 && R != 128 && R != 256)
            return fail(LUMRAD_EINVAL, "the device loop runs 32, 64, 128 or 256 rays per probe");
        if ((long long)dw.W * (R / 32) > sv->dl->max_tasks)
            return fail(LUMRAD_EINVAL, "the world's probes x R/32 exceed the device loop's 2^20 tasks");
        if (n_edits > sv->dl->edit_cap) return fail(LUMRAD_EINVAL, "too many edits for the device loop's arena");
    }
    SRequest r;
    r.id = sv->next_id++;
    r.world = world;
    r.arrival = arrival_s < 0.0 ? sv->now() : arrival_s;
    r.p = *params;
    r.edits.assign(edits, edits + n_edits);
    if (sv->dl) sv->dl->queue.push_back(std::move(r));
    else sv->worlds[world].fifo.push_back(std::move(r));
    sv->pending++;
    *request = sv->next_id - 1;
    return LUMRAD_OK;
}

int lumrad_server_progress(LumRadServer server) {
    Server* sv = as_server(server);
    if (!sv) return fail(LUMRAD_EINVAL, "null server");
    LUMRAD_TRY(cudaSetDevice(sv->s.device));
    return progress(sv);
}

int lumrad_server_run(LumRadServer server, double timeout_s) {
    Server* sv = as_server(server);
    if (!sv) return fail(LUMRAD_EINVAL, "null server");
    LUMRAD_TRY(cudaSetDevice(sv->s.device));
    const double deadline = clock_s() + timeout_s;
    while (sv->pending > 0) {
        int rc = progress(sv);
        if (rc) return rc;
        if (clock_s() > deadline) return fail(LUMRAD_ETIMEOUT, "requests still pending at the timeout");
        std::this_thread::yield();
    }
    return LUMRAD_OK;
}

int lumrad_server_cancel(LumRadServer server, long long request, int* cancelled) {
    Server* sv = as_server(server);
    if (!sv || !cancelled) return fail(LUMRAD_EINVAL, "null argument");
    *cancelled = 0;
    if (sv->dl) {   // only requests not yet published into the ring
        auto& q = sv->dl->queue;
        for (auto it = q.begin(); it != q.end(); ++it)
            if (it->id == request) {
                complete_now(sv, *it, LUMRAD_ECANCELED);
                q.erase(it);
                *cancelled = 1;
                return LUMRAD_OK;
            }
        return LUMRAD_OK;
    }
    for (auto& sw : sv->worlds)
        for (auto it = sw.fifo.begin(); it != sw.fifo.end(); ++it)
            if (it->id == request) {
                complete_now(sv, *it, LUMRAD_ECANCELED);
                sw.fifo.erase(it);
                *cancelled = 1;
                return LUMRAD_OK;
            }
    return LUMRAD_OK;
}

int lumrad_server_poll(LumRadServer server, LumRadCompletion* out, int cap, int* n) {
    Server* sv = as_server(server);
    if (!sv || !n || (cap > 0 && !out)) return fail(LUMRAD_EINVAL, "bad argument");
    int k = 0;
    while (k < cap && !sv->done.empty()) {
        out[k++] = sv->done.front();
        sv->done.pop_front();
    }
    *n = k;
    return LUMRAD_OK;
}

double lumrad_server_now(LumRadServer server) {
    Server* sv = as_server(server);
    return sv ? sv->now() : 0.0;
}

int lumrad_server_get_radiance(LumRadServer server, int world, float* rgb) {
    Server* sv = as_server(server);
    if (!sv || !rgb) return fail(LUMRAD_EINVAL, "null argument");
    if (world < 0 || world >= (int)sv->worlds.size()) return fail(LUMRAD_EINVAL, "unknown world");
    LUMRAD_TRY(cudaSetDevice(sv->s.device));
    SWorld& w = sv->worlds[world];
    if (sv->dl) {   // after the world's published requests; its volume side is the loop's
        DevLoopHost& dl = *sv->dl;
        const double deadline = clock_s() + 60.0;
        while (dl.outstanding[world] > 0) {
            int rc = progress(sv);
            if (rc) return rc;
            if (clock_s() > deadline) return fail(LUMRAD_ETIMEOUT, "the world's requests did not complete");
            std::this_thread::yield();
        }
        int cur = 0;
        LUMRAD_TRY(cudaMemcpyAsync(&cur, &dl.d_worlds[world].cur, sizeof(int), cudaMemcpyDeviceToHost, w.ctx->stream));
        LUMRAD_TRY(cudaStreamSynchronize(w.ctx->stream));
        w.ctx->world.cur = cur;
        return lumrad_get_radiance(w.ctx, rgb);
    }
    if (w.busy) {
        LUMRAD_TRY(cudaEventSynchronize(sv->slots[w.last_slot]->ev_done));
        int rc = retire(sv);
        if (rc) return rc;
    }
    const DeviceWorld& dw = w.ctx->world;
    if (dw.evicted) {   // the volume kept on the host
        for (size_t i = 0; i < dw.W; i++)
            for (int k = 0; k < 3; k++) {
                float v;
                if (dw.precision == LUMRAD_PRECISION_FP32) {
                    std::memcpy(&v, dw.h_rad_saved.data() + 16 * i + 4 * k, 4);
                } else if (dw.precision == LUMRAD_PRECISION_RGB10A2) {
                    uint32_t word;
                    std::memcpy(&word, dw.h_rad_saved.data() + 4 * i, 4);
                    v = unorm10_decode_host((word >> (10 * k)) & 1023u);
                } else {
                    uint16_t bits;
                    std::memcpy(&bits, dw.h_rad_saved.data() + 8 * i + 2 * k, 2);
                    if (dw.precision == LUMRAD_PRECISION_FP16) {
                        __half_raw r;
                        r.x = bits;
                        v = __half2float(__half(r));
                    } else {
                        const uint32_t u = (uint32_t)bits << 16;
                        std::memcpy(&v, &u, 4);
                    }
                }
                rgb[3 * i + k] = v;
            }
        return LUMRAD_OK;
    }
    return lumrad_get_radiance(w.ctx, rgb);
}

int lumrad_server_stats(LumRadServer server, LumRadServerStats* out) {
    Server* sv = as_server(server);
    if (!sv || !out) return fail(LUMRAD_EINVAL, "null argument");
    sv->st.resident_bytes = (double)sv->resident;
    *out = sv->st;
    return LUMRAD_OK;
}

}  // extern "C"
