// lumrad_host.cpp — the C ABI of include/lumrad.h: contexts, resident device data, passes.
//
// One context = one world resident on one GPU plus a stream, events and pinned staging for
// update lists.  It replaces the radiance part of LumInternal::LumInternalRenderer: the
// resources of createImages (src/renderer/src/internal_render.cpp:107-209), the uploads of
// updateBlockPalette / updateMaterialPalette (load_stuff.cpp:36-111) and exec_copies' world
// upload (internal_render.cpp:1460-1475), and update_radiance itself (internal_render.cpp:1129-1214).
//
// Device layout of a world (all resident between passes):
//   grid      int16  X*Y*Z            block ids, x-fastest
//   cgrid     uint8 / uint16 X*Y*Z    compact ids (0 = air), rebuilt when the grid or palette changes
//   cbits     uint32 128 per compact id   voxel occupancy of each compact id
//   pal       uint8  slots*4096       voxel values, voxel (x,y,z) at x + 16y + 256z
//   mats      float4 256              (r, g, b, emission)
//   rad[2]    float4 or 4x16-bit per probe   previous / next radiance (ping-pong)
//   scratch   float4 per (probe, subgroup); probe_count int per probe (zero between passes)

#include "lumrad_world.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace lumrad {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

// Spherical-Fibonacci directions of radiance.comp:293-306 with n = R.  The float arithmetic
// follows the shader; cos/sin are evaluated in double and rounded to float.
void fibonacci_table(int n, float* xyz) {
    const float pi = 3.1415926535897932384626433832795f;
    const float golden = std::sqrt(5.0f) * 0.5f + 0.5f;
    for (int i = 0; i < n; i++) {
        const float fi = (float)i;
        const float a = fi * (golden - 1.0f);
        const float phi = 2.0f * pi * (a - std::floor(a));
        const float cos_t = 1.0f - (2.0f * fi + 1.0f) * (1.0f / (float)n);
        float s2 = 1.0f - cos_t * cos_t;
        s2 = s2 < 0.0f ? 0.0f : s2;
        s2 = 1.0f < s2 ? 1.0f : s2;
        const float sin_t = std::sqrt(s2);
        xyz[3 * i] = (float)std::cos((double)phi) * sin_t;
        xyz[3 * i + 1] = (float)std::sin((double)phi) * sin_t;
        xyz[3 * i + 2] = cos_t;
    }
}

static float unorm_clamp(float v) { return v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f; }
static float exact_inverse(int v) { return (v > 0 && (v & (v - 1)) == 0) ? 1.0f / (float)v : 0.0f; }

// ---------------------------------------------------------------- DeviceWorld
int DeviceWorld::init(int X_, int Y_, int Z_, int slots, int precision_, cudaStream_t stream) {
    X = X_; Y = Y_; Z = Z_;
    W = (size_t)X * Y * Z;
    n_slots = slots;
    precision = precision_;
    rad_stride = radiance_stride(precision);
    h_grid.assign(W, 0);
    h_pal.assign((size_t)n_slots * 4096, 0);
    h_pal_dev.assign((size_t)n_slots * 4096, 0);
    h_mats.assign(LUMRAD_MATERIALS, LumRadMaterial{});
    h_mats_dev.assign(LUMRAD_MATERIALS, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    LUMRAD_TRY(cudaMalloc(&d_grid, W * sizeof(int16_t)));
    LUMRAD_TRY(cudaMalloc(&d_cgrid, W * sizeof(uint16_t)));
    LUMRAD_TRY(cudaMalloc(&d_pal, h_pal.size()));
    LUMRAD_TRY(cudaMalloc(&d_mats, LUMRAD_MATERIALS * sizeof(float4)));
    LUMRAD_TRY(cudaMalloc(&d_stats, 2 * sizeof(unsigned long long)));
    for (int i = 0; i < 2; i++) {
        LUMRAD_TRY(cudaMalloc(&d_rad[i], W * rad_stride));
        LUMRAD_TRY(cudaMemsetAsync(d_rad[i], 0, W * rad_stride, stream));
    }
    LUMRAD_TRY(cudaMemsetAsync(d_grid, 0, W * sizeof(int16_t), stream));
    LUMRAD_TRY(cudaMemsetAsync(d_pal, 0, h_pal.size(), stream));
    LUMRAD_TRY(cudaMemsetAsync(d_mats, 0, LUMRAD_MATERIALS * sizeof(float4), stream));
    LUMRAD_TRY(cudaMemsetAsync(d_stats, 0, 2 * sizeof(unsigned long long), stream));
    grid_dirty = false;
    compact_dirty = true;
    return LUMRAD_OK;
}

void DeviceWorld::release() {
    cudaFree(d_grid); cudaFree(d_cgrid); cudaFree(d_cbits); cudaFree(d_cslot); cudaFree(d_pal); cudaFree(d_mats);
    cudaFree(d_rad[0]); cudaFree(d_rad[1]); cudaFree(d_scratch); cudaFree(d_probe_count); cudaFree(d_stats);
    cudaFree(d_hits);
    for (auto& kv : d_dirs) cudaFree(kv.second);
    d_dirs.clear();
    d_grid = nullptr; d_cgrid = nullptr; d_cbits = nullptr; d_cslot = nullptr; d_pal = nullptr; d_mats = nullptr;
    d_rad[0] = d_rad[1] = nullptr; d_scratch = nullptr; d_probe_count = nullptr; d_stats = nullptr; d_hits = nullptr;
}

int DeviceWorld::evict(cudaStream_t stream) {
    if (evicted) return LUMRAD_OK;
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    h_rad_saved.resize(W * rad_stride);
    LUMRAD_TRY(cudaMemcpy(h_rad_saved.data(), d_rad[cur], W * rad_stride, cudaMemcpyDeviceToHost));
    release();
    cbits_cap = scratch_cap = count_cap = hits_cap = hits_n = 0;
    hits_recorded = false;
    evicted = true;
    return LUMRAD_OK;
}

int DeviceWorld::readmit(cudaStream_t stream) {
    if (!evicted) return LUMRAD_OK;
    LUMRAD_TRY(cudaMalloc(&d_grid, W * sizeof(int16_t)));
    LUMRAD_TRY(cudaMalloc(&d_cgrid, W * sizeof(uint16_t)));
    LUMRAD_TRY(cudaMalloc(&d_pal, h_pal_dev.size()));
    LUMRAD_TRY(cudaMalloc(&d_mats, LUMRAD_MATERIALS * sizeof(float4)));
    LUMRAD_TRY(cudaMalloc(&d_stats, 2 * sizeof(unsigned long long)));
    for (int i = 0; i < 2; i++) LUMRAD_TRY(cudaMalloc(&d_rad[i], W * rad_stride));
    LUMRAD_TRY(cudaMemcpyAsync(d_grid, h_grid.data(), W * sizeof(int16_t), cudaMemcpyHostToDevice, stream));
    LUMRAD_TRY(cudaMemcpyAsync(d_pal, h_pal_dev.data(), h_pal_dev.size(), cudaMemcpyHostToDevice, stream));
    pal_dirty_end = n_slots;
    LUMRAD_TRY(cudaMemcpyAsync(d_mats, h_mats_dev.data(), LUMRAD_MATERIALS * sizeof(float4), cudaMemcpyHostToDevice,
                               stream));
    LUMRAD_TRY(cudaMemsetAsync(d_stats, 0, 2 * sizeof(unsigned long long), stream));
    LUMRAD_TRY(cudaMemcpyAsync(d_rad[cur], h_rad_saved.data(), W * rad_stride, cudaMemcpyHostToDevice, stream));
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    std::vector<uint8_t>().swap(h_rad_saved);
    evicted = false;
    grid_dirty = false;
    compact_dirty = true;   // compact ids and masks built again from the host grid and palette
    return sync_inputs(stream);
}

// Renumbers the block ids present in the grid into compact ids (0 stays 0; every id whose palette
// slot is absent shares one all-empty compact id) and builds each compact id's occupancy mask
// from the palette as uploaded.  Ids that appear later (edits) get the next free compact id
// through compact_of.
void DeviceWorld::build_compact(const int16_t* g, bool host_bits) {
    id_to_c.assign(65536, -1);
    reps.clear();
    empty_c = -1;
    id_to_c[0] = 0;
    reps.push_back(0);
    n_compact = 1;
    h_cbits.assign(128, 0u);
    skip_host_bits = !host_bits;
    for (int k = 0; k < 4096 && n_slots > 0 && host_bits; k++)   // block 0 reads palette slot 0 like any other id
        if (h_pal_dev[k]) h_cbits[k >> 5] |= 1u << (k & 31);
    h_cslot.assign(1, n_slots > 0 ? 0 : -1);
    cgrid_wide = false;
    bool assigned = false;
    for (size_t i = 0; i < W; i++) {
        if (id_to_c[(uint16_t)g[i]] >= 0) continue;
        if (compact_of(g[i], &assigned) < 0) cgrid_wide = true;   // > 256 ids: uint16
    }
    h_cgrid.resize(W * (cgrid_wide ? 2 : 1));
    for (size_t i = 0; i < W; i++) {
        const int32_t c = id_to_c[(uint16_t)g[i]];
        if (cgrid_wide) reinterpret_cast<uint16_t*>(h_cgrid.data())[i] = (uint16_t)c;
        else h_cgrid[i] = (uint8_t)c;
    }
    skip_host_bits = false;
}

int DeviceWorld::compact_of(int16_t b, bool* assigned) {
    *assigned = false;
    int32_t& c = id_to_c[(uint16_t)b];
    if (c >= 0) return c;
    const int slot = b >= 0 ? b : b + 64;
    const bool has_slot = b >= -63 && slot < n_slots;
    if (!has_slot && empty_c >= 0) return c = empty_c;
    // past 256 ids a uint8 compact grid overflows; the id is assigned anyway (a rebuild with a
    // uint16 grid numbers the ids in the same order)
    const bool overflow = !cgrid_wide && n_compact >= 256;
    if (!has_slot) empty_c = n_compact;
    c = n_compact++;
    reps.push_back(has_slot ? b : kEmptyRep);
    h_cslot.push_back(has_slot ? slot : -1);
    h_cbits.resize((size_t)n_compact * 128, 0u);
    if (has_slot && !skip_host_bits) {
        const uint8_t* v = h_pal_dev.data() + (size_t)slot * 4096;
        uint32_t* bits = h_cbits.data() + (size_t)c * 128;
        for (int k = 0; k < 4096; k++)
            if (v[k]) bits[k >> 5] |= 1u << (k & 31);
    }
    *assigned = true;
    return overflow ? -1 : c;
}

size_t DeviceWorld::footprint() const {
    size_t b = W * sizeof(int16_t) + W * sizeof(uint16_t) + cbits_cap * (128 * sizeof(uint32_t) + sizeof(int)) + h_pal.size() +
               LUMRAD_MATERIALS * sizeof(float4) + 2 * W * rad_stride + scratch_cap * sizeof(float4) +
               count_cap * sizeof(int) + 2 * sizeof(unsigned long long) + hits_cap * sizeof(LumRadHit);
    for (auto& kv : d_dirs) b += (size_t)kv.first * sizeof(float4);
    return b;
}

int DeviceWorld::sync_inputs(cudaStream_t stream) {
    // a changed origin world or palette replaces the blockified frame (the next blockify rebuilds it)
    if (!h_cur.empty() && (grid_dirty || compact_dirty)) {
        h_cur.clear();
        grid_dirty = true;
    }
    if (grid_dirty || compact_dirty) uploads++;
    if (grid_dirty) {
        LUMRAD_TRY(cudaMemcpyAsync(d_grid, h_grid.data(), W * sizeof(int16_t), cudaMemcpyHostToDevice, stream));
        grid_dirty = false;
        compact_dirty = true;
    }
    if (compact_dirty) {
        build_compact();
        // room for every id that has a palette slot (-63..-1, 1..n_slots-1), air and the empty id,
        // so ids that edits bring in later never reallocate
        const size_t cap = std::max<size_t>((size_t)n_compact, (size_t)n_slots + 64);
        if (cap > cbits_cap) {
            cudaFree(d_cbits);
            cudaFree(d_cslot);
            d_cbits = nullptr;
            d_cslot = nullptr;
            cbits_cap = 0;
            LUMRAD_TRY(cudaMalloc(&d_cbits, cap * 128 * sizeof(uint32_t)));
            LUMRAD_TRY(cudaMalloc(&d_cslot, cap * sizeof(int)));
            cbits_cap = cap;
        }
        LUMRAD_TRY(cudaMemcpyAsync(d_cgrid, h_cgrid.data(), h_cgrid.size(), cudaMemcpyHostToDevice, stream));
        LUMRAD_TRY(cudaMemcpyAsync(d_cbits, h_cbits.data(), h_cbits.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                   stream));
        LUMRAD_TRY(cudaMemcpyAsync(d_cslot, h_cslot.data(), h_cslot.size() * sizeof(int), cudaMemcpyHostToDevice, stream));
        LUMRAD_TRY(cudaStreamSynchronize(stream));   // host vectors may be rebuilt by the next call
        compact_dirty = false;
    }
    return LUMRAD_OK;
}

int DeviceWorld::ensure_dirs(int R, cudaStream_t stream, const float4** out) {
    auto it = d_dirs.find(R);
    if (it != d_dirs.end()) {
        *out = it->second;
        return LUMRAD_OK;
    }
    std::vector<float> xyz(3 * (size_t)R);
    fibonacci_table(R, xyz.data());
    std::vector<float4> t(R);
    for (int i = 0; i < R; i++) t[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
    float4* d = nullptr;
    uploads++;
    LUMRAD_TRY(cudaMalloc(&d, sizeof(float4) * R));
    LUMRAD_TRY(cudaMemcpyAsync(d, t.data(), sizeof(float4) * R, cudaMemcpyHostToDevice, stream));
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    d_dirs[R] = d;
    *out = d;
    return LUMRAD_OK;
}

int DeviceWorld::ensure_scratch(size_t groups, int R, cudaStream_t stream) {
    const size_t nsub = (size_t)(R / 32);
    if (groups * nsub > scratch_cap) {
        cudaFree(d_scratch);
        d_scratch = nullptr;
        scratch_cap = 0;
        const size_t cap = std::max<size_t>(groups * nsub, 1024);
        uploads++;
        LUMRAD_TRY(cudaMalloc(&d_scratch, cap * sizeof(float4)));
        scratch_cap = cap;
    }
    if (groups > count_cap) {
        cudaFree(d_probe_count);
        d_probe_count = nullptr;
        count_cap = 0;
        const size_t cap = std::max<size_t>(groups, 1024);
        uploads++;
        LUMRAD_TRY(cudaMalloc(&d_probe_count, cap * sizeof(int)));
        // zeroed in order on the pass's stream (a plain memset runs on the default stream, which
        // a non-blocking stream does not wait for)
        LUMRAD_TRY(cudaMemsetAsync(d_probe_count, 0, cap * sizeof(int), stream));
        count_cap = cap;
    }
    return LUMRAD_OK;
}

int DeviceWorld::ensure_hits(size_t n) {
    if (n <= hits_cap) return LUMRAD_OK;
    cudaFree(d_hits);
    d_hits = nullptr;
    hits_cap = 0;
    LUMRAD_TRY(cudaMalloc(&d_hits, std::max<size_t>(n, 1) * sizeof(LumRadHit)));
    hits_cap = std::max<size_t>(n, 1);
    return LUMRAD_OK;
}

// Fills the kernel's view of one pass over `d_req` (n requests) with parameters `p`
// (size >= 1) reading rad[cur] and writing rad[1-cur], and the pass's start: next starts as a copy
// of prev (probes not in the list keep their value) and the counters are cleared, both by the
// first march launch.
int DeviceWorld::prepare_pass(const short4* d_req, int n, const LumRadPassParams& p, cudaStream_t stream,
                              LaunchArgs* la) {
    int rc = fill_pass(d_req, n, p, stream, &la->single);
    if (rc) return rc;
    la->copy_src = d_rad[cur];
    la->copy_dst = d_rad[1 - cur];
    la->copy_bytes = (long long)(W * rad_stride);
    la->clear_stats = d_stats;
    return LUMRAD_OK;
}

// The kernels' descriptor of a pass (inputs synced to the device, buffers sized); no copies.
int DeviceWorld::fill_pass(const short4* d_req, int n, const LumRadPassParams& p, cudaStream_t stream,
                           WorldPass* out) {
    int rc = sync_inputs(stream);
    if (rc) return rc;
    const float4* dirs = nullptr;
    if ((rc = ensure_dirs(p.rays_per_probe, stream, &dirs))) return rc;
    const int R = p.rays_per_probe;
    const int groups = n / p.size;
    if ((long long)groups * (R / 32) >= (1LL << 31)) return fail(LUMRAD_EINVAL, "pass has too many subgroups (>= 2^31)");
    if ((rc = ensure_scratch((size_t)std::max(groups, 1), R, stream))) return rc;
    if (p.record_hits && (rc = ensure_hits((size_t)groups * R))) return rc;
    WorldPass& w = *out;
    std::memset(&w, 0, sizeof w);
    w.X = X; w.Y = Y; w.Z = Z;
    w.cgrid_wide = cgrid_wide ? 1 : 0;
    w.cgrid = d_cgrid;
    w.cbits = d_cbits;
    w.cslot = d_cslot;
    w.grid = d_grid;
    w.pal = d_pal;
    w.n_slots = n_slots;
    w.n_compact = n_compact;
    w.mats = d_mats;
    w.prev = d_rad[cur];
    w.next = d_rad[1 - cur];
    w.req = d_req;
    w.n_groups = groups;
    w.size = p.size;
    w.shift = p.shift;
    w.R = R;
    w.max_dist = p.max_dist;
    w.max_steps = (int)(2.0f * p.max_dist) + 2;
    w.alpha = p.blend;
    w.one_minus_alpha = 1.0f - p.blend;
    w.seed = (uint32_t)p.time_seed;
    w.inv_dim[0] = exact_inverse(X);
    w.inv_dim[1] = exact_inverse(Y);
    w.inv_dim[2] = exact_inverse(Z);
    w.inv_nsub = exact_inverse(R / 32);
    w.dirs = dirs;
    w.hits = p.record_hits ? d_hits : nullptr;
    w.scratch = d_scratch;
    w.probe_count = d_probe_count;
    w.stats = d_stats;
    w.task_begin = 0;
    w.n_tasks = (long long)groups * (R / 32);
    hits_recorded = p.record_hits != 0;
    hits_n = p.record_hits ? (size_t)groups * R : 0;
    return LUMRAD_OK;
}

// ---------------------------------------------------------------- Context
int Context::ensure_req_capacity(size_t n) {
    if (n <= req_cap) return LUMRAD_OK;
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    cudaFree(d_req);
    d_req = nullptr;
    req_cap = 0;
    const size_t cap = std::max<size_t>(n, 1024);
    LUMRAD_TRY(cudaMalloc(&d_req, cap * sizeof(short4)));
    req_cap = cap;
    return LUMRAD_OK;
}

int Context::ensure_rays(long long n_tasks, long long cap_tasks) {
    const size_t need = (size_t)std::min<long long>(std::max<long long>(n_tasks, 1), cap_tasks) * kTaskRays;
    if (need <= ray_cap) return LUMRAD_OK;
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    cudaFree(d_ray_res);
    cudaFree(d_ray_res2);
    cudaFree(d_ray_blk);
    d_ray_res = d_ray_res2 = nullptr;
    d_ray_blk = nullptr;
    ray_cap = 0;
    pass_mark = -1;   // the buffers are new: no launch overlaps the synchronised one
    LUMRAD_TRY(cudaMalloc(&d_ray_res, need * sizeof(RayResult)));
    LUMRAD_TRY(cudaMalloc(&d_ray_res2, need * sizeof(RayResult)));
    LUMRAD_TRY(cudaMalloc(&d_ray_blk, need * sizeof(int)));
    ray_cap = need;
    return LUMRAD_OK;
}

int Context::stage_requests(const int16_t* req, size_t n) {
    int rc = ensure_req_capacity(n);
    if (rc) return rc;
    if (n == 0) return LUMRAD_OK;
    if (req_copy_pending) {
        LUMRAD_TRY(cudaEventSynchronize(ev_req));
        req_copy_pending = false;
    }
    if (n > h_req_cap) {
        if (h_req_pinned) cudaFreeHost(h_req_pinned);
        h_req_pinned = nullptr;
        h_req_cap = 0;
        const size_t cap = std::max<size_t>(n, 1024);
        LUMRAD_TRY(cudaMallocHost(&h_req_pinned, cap * 4 * sizeof(int16_t)));
        h_req_cap = cap;
    }
    std::memcpy(h_req_pinned, req, n * 4 * sizeof(int16_t));
    world.uploads++;
    LUMRAD_TRY(cudaMemcpyAsync(d_req, h_req_pinned, n * sizeof(short4), cudaMemcpyHostToDevice, stream));
    LUMRAD_TRY(cudaEventRecord(ev_req, stream));
    req_copy_pending = true;
    return LUMRAD_OK;
}

int Context::check_error() {
    if (!have_pass) return LUMRAD_OK;
    LUMRAD_TRY(cudaMemcpyAsync(h_err, d_error, sizeof(int), cudaMemcpyDeviceToHost, stream));
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    return handle_error(*h_err);
}

int Context::handle_error(int e) {
    if (e != 0) {
        cudaMemsetAsync(d_error, 0, sizeof(int), stream);
        if (d_pass_mask) cudaMemsetAsync(d_pass_mask, 0, (size_t)world.W * sizeof(uint32_t), stream);
        if (d_pass_mask2) cudaMemsetAsync(d_pass_mask2, 0, (size_t)world.W * sizeof(uint32_t), stream);
        cudaMemsetAsync(d_queue, 0, kQueueWords * sizeof(unsigned long long), stream);
        cudaMemsetAsync(world.d_probe_count, 0, world.count_cap * sizeof(int), stream);
        cudaStreamSynchronize(stream);
        return fail(LUMRAD_EDEVICE, std::string(e & 1 ? "radiance kernel scheduler stopped making progress" :
                                                "finalize kernel without the cross-CTA combine got a probe spanning CTAs") +
                                        " (code " + std::to_string(e) + ")");
    }
    return LUMRAD_OK;
}

int Context::run_pass(const short4* d_reqs, int n, const LumRadPassParams* p_in, const int* dev_count) {
    NvtxRange range("lumrad radiance pass");
    if (int rc = check_unowned(this)) return rc;
    LumRadPassParams p = *p_in;
    if (p.size == 0) {
        // adaptive slicing of update_radiance (internal_render.cpp:1190-1203)
        if (last_ms < 1.8f) magic_size--;
        else if (last_ms > 2.2f) magic_size++;
        magic_size = std::min(std::max(magic_size, 1), 10);
        p.size = magic_size;
        p.shift = frame % magic_size;
        p.time_seed = frame;
    }
    frame++;
    LaunchArgs la;
    std::memset(&la, 0, sizeof la);
    int rc = world.prepare_pass(d_reqs, n, p, stream, &la);
    if (rc) return rc;
    la.worlds = nullptr;
    la.n_worlds = 1;
    la.n_tasks = la.single.n_tasks;
    la.queue = d_queue;
    la.error = d_error;
    if ((rc = ensure_rays(la.n_tasks))) return rc;
    // the march may start in the previous pass's finalize tail: see pass_mark (the list must not
    // come from a kernel, the hits use the one record buffer)
    const bool dependent = !p.record_hits && !dev_count && pass_mark == api_calls - 1 && uploads_mark == world.uploads;
    la.ray_res = ray_side ? d_ray_res2 : d_ray_res;
    ray_side ^= 1;
    la.ray_blk = d_ray_blk;
    la.dev_count = dev_count;
    la.force_lean = test_lean_finalize ? 1 : 0;
    last_count_on_device = dev_count != nullptr;
    if (dev_count) {
        if (!d_last_count) LUMRAD_TRY(cudaMalloc(&d_last_count, sizeof(int)));
        la.count_src = dev_count;   // copied by the march launch
        la.count_dst = d_last_count;
        last_size = p.size;
        last_R = p.rays_per_probe;
    }
    const int slot = (int)(n_passes % kRing);
    la.time_start = la.time_end = d_ptime + 2 * slot;
    timed[slot] = la.n_tasks > 0;
    LUMRAD_TRY(launch_radiance(la, world.precision, p.record_hits != 0, num_sms, stream, dependent));
    // the next pass call may start in this pass's finalize tail: only when its last operation is
    // that finalize launch (not the copies of an empty pass) and it has no hit records
    pass_mark = p.record_hits || la.n_tasks <= 0 ? -1 : api_calls;
    uploads_mark = world.uploads;
    last_slot = slot;
    last_slot_passes = 1;
    n_passes++;
    world.cur = 1 - world.cur;
    have_pass = true;
    last.probes = (uint64_t)la.single.n_groups;
    last.rays = (uint64_t)la.single.n_groups * la.single.R;
    return LUMRAD_OK;
}

int Context::read_times() {
    LUMRAD_TRY(cudaMemcpyAsync(h_ptime, d_ptime, 2 * kRing * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream));
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    return LUMRAD_OK;
}

float Context::slot_ms(int slot) const {
    const unsigned long long t0 = h_ptime[2 * slot], t1 = h_ptime[2 * slot + 1];
    return timed[slot] && t1 > t0 ? (float)((double)(t1 - t0) * 1e-6) : 0.0f;
}

int Context::ensure_pass_table(int n) {
    if (n <= ptab_cap) return LUMRAD_OK;
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    for (int h = 0; h < 2; h++) {
        if (h_ptab[h]) cudaFreeHost(h_ptab[h]);
        h_ptab[h] = nullptr;
    }
    cudaFree(d_ptab);
    d_ptab = nullptr;
    ptab_cap = 0;
    const int cap = std::max(n, 16);
    for (int h = 0; h < 2; h++) LUMRAD_TRY(cudaMallocHost(&h_ptab[h], cap * sizeof(WorldPass)));
    LUMRAD_TRY(cudaMalloc(&d_ptab, cap * sizeof(WorldPass)));
    ptab_cap = cap;
    return LUMRAD_OK;
}

// The passes' marches do not read the radiance volume, so consecutive passes whose tasks fit
// kMultiTasks share one march launch (one queue drain instead of one per pass); each pass's
// finalize then runs in order, reading the volume its predecessor wrote.  A pass larger than
// kMultiTasks runs alone in rounds, as lumrad_radiance_pass runs it.  Results are those of n
// single passes, bit for bit; counters and the kernel-time entry cover all n.
int Context::run_passes(const short4* const* reqs, const int* ns, const LumRadPassParams* ps, int n) {
    NvtxRange range("lumrad radiance passes");
    if (int rc = check_unowned(this)) return rc;
    if (n <= 0) return LUMRAD_OK;
    int rc = world.sync_inputs(stream);
    if (rc) return rc;
    if (!d_pass_mask) {   // zero between calls (the last finalize of each group clears its mask)
        world.uploads++;   // the zeroing below precedes the march: no launch may overlap it
        LUMRAD_TRY(cudaMalloc(&d_pass_mask, (size_t)world.W * sizeof(uint32_t)));
        LUMRAD_TRY(cudaMalloc(&d_pass_mask2, (size_t)world.W * sizeof(uint32_t)));
        LUMRAD_TRY(cudaMemsetAsync(d_pass_mask, 0, (size_t)world.W * sizeof(uint32_t), stream));
        LUMRAD_TRY(cudaMemsetAsync(d_pass_mask2, 0, (size_t)world.W * sizeof(uint32_t), stream));
    }
    const int slot = (int)(n_passes % kRing);
    timed[slot] = false;
    bool first = true;   // the first launch clears the counters and starts the kernel time
    bool ends_in_finalize = false;   // the call's last operation is a finalize launch
    // (the march here follows the pass table's copy, so it never starts in the previous pass's
    // finalize tail; the ray buffer and the pass mask still alternate, for the pass call after it)
    bool dependent = false;
    const int side = ray_side;   // this call's ray buffer (the previous pass's finalize reads the other)
    ray_side ^= 1;
    const size_t vol_bytes = (size_t)world.W * world.rad_stride;
    uint64_t probes = 0, rays = 0;
    auto aligned_tasks = [&](int i) -> long long {
        const long long t = (long long)(ns[i] / ps[i].size) * (ps[i].rays_per_probe / 32);
        return (t + kWarps - 1) / kWarps * kWarps;
    };
    int i = 0;
    while (i < n) {
        if (aligned_tasks(i) > kMultiTasks) {
            // one pass in rounds of kChunkTasks
            LaunchArgs la;
            std::memset(&la, 0, sizeof la);
            if ((rc = world.fill_pass(reqs[i], ns[i], ps[i], stream, &la.single))) return rc;
            la.copy_src = la.single.prev;   // next starts as a copy of prev: by the march launch
            la.copy_dst = la.single.next;
            la.copy_bytes = (long long)vol_bytes;
            if (first) la.clear_stats = world.d_stats;
            if (first) la.time_start = d_ptime + 2 * slot;
            la.time_end = d_ptime + 2 * slot;
            timed[slot] = timed[slot] || la.n_tasks > 0;
            first = false;
            la.n_worlds = 1;
            la.n_tasks = la.single.n_tasks;
            la.queue = d_queue;
            la.error = d_error;
            if ((rc = ensure_rays(la.n_tasks))) return rc;
            la.ray_res = side ? d_ray_res2 : d_ray_res;
            la.ray_blk = d_ray_blk;
            LUMRAD_TRY(launch_radiance(la, world.precision, false, num_sms, stream, dependent));
            dependent = false;
            ends_in_finalize = la.n_tasks > 0;
            probes += (uint64_t)la.single.n_groups;
            rays += (uint64_t)la.single.n_groups * la.single.R;
            world.cur = 1 - world.cur;
            i++;
            continue;
        }
        // the longest run of passes from i whose tasks fit one march launch
        int j = i;
        long long total = 0;
        while (j < n && j - i < kMultiPasses && aligned_tasks(j) <= kMultiTasks - total) total += aligned_tasks(j++);
        const int k = j - i;
        if ((rc = ensure_pass_table(k))) return rc;
        WorldPass* tab = h_ptab[ptab_half];
        if (ev_ptab[ptab_half]) LUMRAD_TRY(cudaEventSynchronize(ev_ptab[ptab_half]));   // its last copy is done
        // a failure before the group's launch leaves the volume as the previous group left it
        const int cur0 = world.cur;
        auto undo = [&](int code) {
            world.cur = cur0;
            return code;
        };
        long long begin = 0;
        for (int q = 0; q < k; q++) {
            if ((rc = world.fill_pass(reqs[i + q], ns[i + q], ps[i + q], stream, &tab[q]))) return undo(rc);
            tab[q].task_begin = begin;
            begin += aligned_tasks(i + q);
            probes += (uint64_t)tab[q].n_groups;
            rays += (uint64_t)tab[q].n_groups * tab[q].R;
            world.cur = 1 - world.cur;   // the next pass reads what this one writes
        }
        for (int q = 0; q < k; q++) {    // buffers fill_pass may have grown on a later pass
            tab[q].scratch = world.d_scratch;
            tab[q].probe_count = world.d_probe_count;
            tab[q].stats = world.d_stats;
        }
        if ((rc = ensure_rays(total, kMultiTasks))) return undo(rc);
        cudaError_t e = cudaMemcpyAsync(d_ptab, tab, k * sizeof(WorldPass), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess && !ev_ptab[ptab_half]) e = cudaEventCreateWithFlags(&ev_ptab[ptab_half], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(ev_ptab[ptab_half], stream);
        if (e != cudaSuccess) return undo(fail(LUMRAD_EDEVICE, std::string("pass table copy: ") + cudaGetErrorString(e)));
        ptab_half ^= 1;
        LaunchArgs la;
        std::memset(&la, 0, sizeof la);
        la.worlds = d_ptab;
        la.n_worlds = k;
        la.n_tasks = total;
        la.queue = d_queue;
        la.error = d_error;
        la.ray_res = side ? d_ray_res2 : d_ray_res;
        la.ray_blk = d_ray_blk;
        la.pass_mask = side ? d_pass_mask2 : d_pass_mask;
        if (first) la.clear_stats = world.d_stats;
        if (first) la.time_start = d_ptime + 2 * slot;
        la.time_end = d_ptime + 2 * slot;
        timed[slot] = timed[slot] || total > 0;
        first = false;
        LUMRAD_TRY(launch_passes(la, tab, k, vol_bytes, world.precision, num_sms, stream, dependent));
        dependent = false;
        ends_in_finalize = total > 0;
        i = j;
    }
    pass_mark = ends_in_finalize ? api_calls : -1;
    uploads_mark = world.uploads;
    last_slot = slot;
    last_slot_passes = n;
    n_passes++;
    frame += n;
    have_pass = true;
    world.hits_recorded = false;
    world.hits_n = 0;
    last.probes = probes;
    last.rays = rays;
    last_count_on_device = false;
    return LUMRAD_OK;
}

int Context::ensure_list_scratch() {
    const long long W = (long long)world.W;
    if (!list.bits) {
        LUMRAD_TRY(cudaMalloc(&list.bits, list_scratch_words(W) * sizeof(uint32_t)));
        LUMRAD_TRY(cudaMalloc(&list.cta_counts, list_scratch_ctas(W) * sizeof(int)));
        LUMRAD_TRY(cudaMalloc(&list.cta_offsets, list_scratch_ctas(W) * sizeof(int)));
        LUMRAD_TRY(cudaMalloc(&list.listed, sizeof(int)));
        LUMRAD_TRY(cudaMalloc(&d_list_count, sizeof(int)));
        LUMRAD_TRY(cudaMallocHost(&h_list_count, sizeof(int)));
    }
    return LUMRAD_OK;
}

int Context::build_list_device(bool consume, int* n) {
    NvtxRange range("lumrad update list");
    int rc = world.sync_inputs(stream);
    if (rc) return rc;
    const long long W = (long long)world.W;
    if ((rc = ensure_list_scratch())) return rc;
    const size_t ns = specials.size() / 4;
    if ((rc = ensure_req_capacity((size_t)W + ns))) return rc;
    if (ns > specials_cap) {
        LUMRAD_TRY(cudaStreamSynchronize(stream));
        cudaFree(d_specials);
        d_specials = nullptr;
        specials_cap = 0;
        LUMRAD_TRY(cudaMalloc(&d_specials, std::max<size_t>(ns, 256) * sizeof(short4)));
        specials_cap = std::max<size_t>(ns, 256);
    }
    if (ns) LUMRAD_TRY(cudaMemcpyAsync(d_specials, specials.data(), ns * sizeof(short4), cudaMemcpyHostToDevice, stream));
    LUMRAD_TRY(launch_update_list(world.d_grid, world.X, world.Y, world.Z, d_specials, (int)ns, list, d_req,
                                  d_list_count, stream));
    if (consume) specials.clear();
    if (!n) return LUMRAD_OK;   // the length stays on the device
    LUMRAD_TRY(cudaMemcpyAsync(h_list_count, d_list_count, sizeof(int), cudaMemcpyDeviceToHost, stream));
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    *n = *h_list_count;
    return LUMRAD_OK;
}

// shift_radiance (internal_render.cpp:1218-1335) into the other ping-pong volume.  The reference
// skips the copy when |shift.x| >= world_size.x and leaves larger y/z shifts undefined (a negative
// copy extent); here any axis with |shift| >= its size leaves the volume unchanged.
int Context::shift_volume(int dx, int dy, int dz) {
    if (dx == 0 && dy == 0 && dz == 0) return LUMRAD_OK;
    NvtxRange range("lumrad shift radiance");
    if (std::abs(dx) >= world.X || std::abs(dy) >= world.Y || std::abs(dz) >= world.Z) return LUMRAD_OK;
    LUMRAD_TRY(launch_shift_radiance(world.d_rad[world.cur], world.d_rad[1 - world.cur], world.X, world.Y, world.Z, dx,
                                     dy, dz, world.precision, stream));
    world.cur = 1 - world.cur;
    return LUMRAD_OK;
}

void Context::release() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    world.release();
    cudaFree(d_req);
    cudaFree(d_queue);
    cudaFree(d_error);
    cudaFree(d_ray_res);
    cudaFree(d_ray_res2);
    cudaFree(d_ray_blk);
    for (int h = 0; h < 2; h++) {
        if (h_ptab[h]) cudaFreeHost(h_ptab[h]);
        if (ev_ptab[h]) cudaEventDestroy(ev_ptab[h]);
    }
    cudaFree(d_ptab);
    for (auto& kv : resident) cudaFree(kv.second.ptr);
    if (h_req_pinned) cudaFreeHost(h_req_pinned);
    cudaFree(list.bits);
    cudaFree(list.cta_counts);
    cudaFree(list.cta_offsets);
    cudaFree(list.listed);
    cudaFree(d_specials);
    cudaFree(d_list_count);
    if (h_list_count) cudaFreeHost(h_list_count);
    cudaFree(d_dirty_mask);
    cudaFree(d_edits);
    cudaFree(d_gather);
    cudaFree(d_rgb);
    if (h_rgb) cudaFreeHost(h_rgb);
    for (auto& m : models) cudaFree(m.d_vox);
    models.clear();
    cudaFree(d_map_owner);
    if (h_blk) cudaFreeHost(h_blk);
    cudaFree(d_last_count);
    cudaFree(d_pass_mask);
    cudaFree(d_pass_mask2);
    cudaFree(d_blk_copies);
    if (h_err) cudaFreeHost(h_err);
    if (ev_req) cudaEventDestroy(ev_req);
    cudaFree(d_ptime);
    if (h_ptime) cudaFreeHost(h_ptime);
    if (stream) cudaStreamDestroy(stream);
}

Context* as_ctx(LumRadContext c) {
    Context* x = reinterpret_cast<Context*>(c);
    if (x) x->api_calls++;
    return x;
}

int check_unowned(const Context* c) {
    return c->owner ? fail(LUMRAD_ESTATE, "the context belongs to a server; use the server's calls") : LUMRAD_OK;
}

int check_params(const LumRadPassParams* p) {
    if (!p) return fail(LUMRAD_EINVAL, "params is null");
    if (p->rays_per_probe < 32 || p->rays_per_probe > 1024 || p->rays_per_probe % 32 != 0)
        return fail(LUMRAD_EINVAL, "rays_per_probe must be a multiple of 32 in [32, 1024]");
    if (!(p->max_dist > 0.0f) || p->max_dist > 16384.0f) return fail(LUMRAD_EINVAL, "max_dist must be in (0, 16384]");
    if (!(p->blend >= 0.0f && p->blend <= 1.0f)) return fail(LUMRAD_EINVAL, "blend must be in [0, 1]");
    if (p->size < 0 || p->size > (1 << 20)) return fail(LUMRAD_EINVAL, "size out of range");
    if (p->size > 0 && (p->shift < 0 || p->shift >= p->size)) return fail(LUMRAD_EINVAL, "shift must be in [0, size)");
    return LUMRAD_OK;
}

}  // namespace lumrad

using namespace lumrad;

extern "C" {

const char* lumrad_last_error(void) { return g_error.c_str(); }

int lumrad_create(const LumRadSettings* s, LumRadContext* out) {
    if (!s || !out) return fail(LUMRAD_EINVAL, "null argument");
    *out = nullptr;
    for (int i = 0; i < 3; i++)
        if (s->world_size[i] < 1 || s->world_size[i] > 2047)
            return fail(LUMRAD_EINVAL, "world_size must be in [1, 2047] per axis");
    const uint64_t W = (uint64_t)s->world_size[0] * s->world_size[1] * s->world_size[2];
    if (W >= (1ull << 31)) return fail(LUMRAD_EINVAL, "world has too many blocks (>= 2^31)");
    if (s->max_block_types < 1 || s->max_block_types > LUMRAD_MAX_BLOCK_SLOTS)
        return fail(LUMRAD_EINVAL, "max_block_types must be in [1, 4096]");
    if (s->precision < 0 || s->precision > LUMRAD_PRECISION_RGB10A2) return fail(LUMRAD_EINVAL, "unknown precision");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(LUMRAD_EDEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (s->device < 0 || s->device >= ndev) return fail(LUMRAD_EINVAL, "device ordinal out of range");

    Context* c = new Context();
    c->device = s->device;
    auto attempt = [&]() -> int {
        LUMRAD_TRY(cudaSetDevice(c->device));
        LUMRAD_TRY(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device));
        LUMRAD_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        LUMRAD_TRY(cudaMallocHost(&c->h_err, sizeof(int)));
        *c->h_err = 0;
        LUMRAD_TRY(cudaEventCreateWithFlags(&c->ev_req, cudaEventDisableTiming));
        LUMRAD_TRY(cudaMalloc(&c->d_ptime, 2 * Context::kRing * sizeof(unsigned long long)));
        LUMRAD_TRY(cudaMallocHost(&c->h_ptime, 2 * Context::kRing * sizeof(unsigned long long)));
        LUMRAD_TRY(cudaMemsetAsync(c->d_ptime, 0, 2 * Context::kRing * sizeof(unsigned long long), c->stream));
        LUMRAD_TRY(cudaMalloc(&c->d_queue, kQueueWords * sizeof(unsigned long long)));
        LUMRAD_TRY(cudaMalloc(&c->d_error, sizeof(int)));
        LUMRAD_TRY(cudaMemsetAsync(c->d_queue, 0, kQueueWords * sizeof(unsigned long long), c->stream));
        LUMRAD_TRY(cudaMemsetAsync(c->d_error, 0, sizeof(int), c->stream));
        int rc = c->world.init(s->world_size[0], s->world_size[1], s->world_size[2], s->max_block_types,
                               s->precision, c->stream);
        if (rc) return rc;
        LUMRAD_TRY(cudaStreamSynchronize(c->stream));
        return LUMRAD_OK;
    };
    const int rc = attempt();
    if (rc) {
        const std::string msg = g_error;
        c->release();
        delete c;
        return fail(rc, msg);
    }
    *out = c;
    return LUMRAD_OK;
}

void lumrad_destroy(LumRadContext ctx) {
    Context* c = as_ctx(ctx);
    if (!c) return;
    c->release();
    delete c;
}

int lumrad_synchronize(LumRadContext ctx) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    LUMRAD_TRY(cudaSetDevice(c->device));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    return c->check_error();
}

int lumrad_load_world(LumRadContext ctx, const int16_t* blocks) {
    Context* c = as_ctx(ctx);
    if (!c || !blocks) return fail(LUMRAD_EINVAL, "null argument");
    if (int rc = check_unowned(c)) return rc;
    std::memcpy(c->world.h_grid.data(), blocks, c->world.W * sizeof(int16_t));
    c->world.grid_dirty = true;
    LUMRAD_TRY(cudaSetDevice(c->device));
    return c->world.sync_inputs(c->stream);
}

int lumrad_set_world_block(LumRadContext ctx, int x, int y, int z, int16_t block) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    if (int rc = check_unowned(c)) return rc;
    DeviceWorld& w = c->world;
    if (x < 0 || y < 0 || z < 0 || x >= w.X || y >= w.Y || z >= w.Z)
        return fail(LUMRAD_EINVAL, "block coordinate out of the world");
    w.h_grid[(size_t)x + (size_t)w.X * ((size_t)y + (size_t)w.Y * z)] = block;
    w.grid_dirty = true;   // uploaded before the next pass, as exec_copies does every frame
    return LUMRAD_OK;
}

int lumrad_get_world_block(LumRadContext ctx, int x, int y, int z, int16_t* block) {
    Context* c = as_ctx(ctx);
    if (!c || !block) return fail(LUMRAD_EINVAL, "null argument");
    const DeviceWorld& w = c->world;
    if (x < 0 || y < 0 || z < 0 || x >= w.X || y >= w.Y || z >= w.Z)
        return fail(LUMRAD_EINVAL, "block coordinate out of the world");
    *block = w.h_grid[(size_t)x + (size_t)w.X * ((size_t)y + (size_t)w.Y * z)];
    return LUMRAD_OK;
}

int lumrad_load_block(LumRadContext ctx, int16_t block, const uint8_t* voxels) {
    Context* c = as_ctx(ctx);
    if (!c || !voxels) return fail(LUMRAD_EINVAL, "null argument");
    DeviceWorld& w = c->world;
    if (block < 0 || block >= w.n_slots) return fail(LUMRAD_EINVAL, "block id outside the palette slots");
    // BlockVoxels[x][y][z] (z fastest) -> x-fastest slot, as updateBlockPalette repacks it
    uint8_t* dst = w.h_pal.data() + (size_t)block * 4096;
    for (int x = 0; x < 16; x++)
        for (int y = 0; y < 16; y++)
            for (int z = 0; z < 16; z++) dst[x + 16 * y + 256 * z] = voxels[(x * 16 + y) * 16 + z];
    return LUMRAD_OK;
}

int lumrad_upload_block_palette(LumRadContext ctx) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    if (int rc = check_unowned(c)) return rc;
    DeviceWorld& w = c->world;
    LUMRAD_TRY(cudaSetDevice(c->device));
    w.h_pal_dev = w.h_pal;
    LUMRAD_TRY(cudaMemcpyAsync(w.d_pal, w.h_pal_dev.data(), w.h_pal_dev.size(), cudaMemcpyHostToDevice, c->stream));
    w.pal_dirty_end = w.n_slots;
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    w.compact_dirty = true;
    return LUMRAD_OK;
}

int lumrad_load_materials(LumRadContext ctx, const LumRadMaterial* materials) {
    Context* c = as_ctx(ctx);
    if (!c || !materials) return fail(LUMRAD_EINVAL, "null argument");
    std::memcpy(c->world.h_mats.data(), materials, LUMRAD_MATERIALS * sizeof(LumRadMaterial));
    return LUMRAD_OK;
}

int lumrad_upload_material_palette(LumRadContext ctx) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    if (int rc = check_unowned(c)) return rc;
    LUMRAD_TRY(cudaSetDevice(c->device));
    std::vector<float4>& m = c->world.h_mats_dev;
    const auto& hm = c->world.h_mats;
    for (int i = 0; i < LUMRAD_MATERIALS; i++) m[i] = make_float4(hm[i].color[0], hm[i].color[1], hm[i].color[2], hm[i].emmit);
    LUMRAD_TRY(cudaMemcpyAsync(c->world.d_mats, m.data(), m.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    return LUMRAD_OK;
}

// Whether [p, p + bytes) lies in page-locked host memory (cudaMallocHost / cudaHostRegister).
static bool host_pinned(const void* p, size_t bytes) {
    if (bytes == 0) return false;
    for (const void* q : {p, static_cast<const void*>(static_cast<const char*>(p) + bytes - 1)}) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost) return false;
    }
    return true;
}

int lumrad_get_radiance(LumRadContext ctx, float* rgb) {
    Context* c = as_ctx(ctx);
    if (!c || !rgb) return fail(LUMRAD_EINVAL, "null argument");
    LUMRAD_TRY(cudaSetDevice(c->device));
    DeviceWorld& w = c->world;
    const size_t bytes = w.W * 3 * sizeof(float);
    // packed to RGB floats on the device (FP16/BF16 widened exactly); one copy, straight into the
    // caller's array when it is page-locked, else through the context's pinned buffer
    const bool direct = host_pinned(rgb, bytes);
    if (!c->d_rgb) LUMRAD_TRY(cudaMalloc(&c->d_rgb, bytes));
    if (!direct && !c->h_rgb) LUMRAD_TRY(cudaMallocHost(&c->h_rgb, bytes));
    LUMRAD_TRY(launch_pack_rgb(w.d_rad[w.cur], w.precision, (long long)w.W, c->d_rgb, c->stream));
    LUMRAD_TRY(cudaMemcpyAsync(direct ? rgb : c->h_rgb, c->d_rgb, bytes, cudaMemcpyDeviceToHost, c->stream));
    LUMRAD_TRY(cudaMemcpyAsync(c->h_err, c->d_error, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));   // one wait for the volume and the error word
    if (!direct) std::memcpy(rgb, c->h_rgb, bytes);
    return c->have_pass ? c->handle_error(*c->h_err) : LUMRAD_OK;
}

int lumrad_set_radiance(LumRadContext ctx, const float* rgb) {
    Context* c = as_ctx(ctx);
    if (!c || !rgb) return fail(LUMRAD_EINVAL, "null argument");
    if (int rc = check_unowned(c)) return rc;
    LUMRAD_TRY(cudaSetDevice(c->device));
    DeviceWorld& w = c->world;
    if (w.precision == LUMRAD_PRECISION_FP32) {
        std::vector<float4> h(w.W);
        for (size_t i = 0; i < w.W; i++)
            h[i] = make_float4(unorm_clamp(rgb[3 * i]), unorm_clamp(rgb[3 * i + 1]), unorm_clamp(rgb[3 * i + 2]), 1.0f);
        LUMRAD_TRY(cudaMemcpyAsync(w.d_rad[w.cur], h.data(), w.W * 16, cudaMemcpyHostToDevice, c->stream));
        LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    } else if (w.precision == LUMRAD_PRECISION_RGB10A2) {
        std::vector<uint32_t> h(w.W);
        for (size_t i = 0; i < w.W; i++)
            h[i] = rgb10a2_pack_host(unorm_clamp(rgb[3 * i]), unorm_clamp(rgb[3 * i + 1]), unorm_clamp(rgb[3 * i + 2]));
        LUMRAD_TRY(cudaMemcpyAsync(w.d_rad[w.cur], h.data(), w.W * 4, cudaMemcpyHostToDevice, c->stream));
        LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    } else {
        std::vector<uint16_t> h(w.W * 4);
        for (size_t i = 0; i < w.W; i++)
            for (int k = 0; k < 4; k++) {
                const float v = k < 3 ? unorm_clamp(rgb[3 * i + k]) : 1.0f;
                if (w.precision == LUMRAD_PRECISION_FP16) h[4 * i + k] = __half_raw(__float2half_rn(v)).x;
                else h[4 * i + k] = __nv_bfloat16_raw(__float2bfloat16_rn(v)).x;
            }
        LUMRAD_TRY(cudaMemcpyAsync(w.d_rad[w.cur], h.data(), w.W * 8, cudaMemcpyHostToDevice, c->stream));
        LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    }
    return LUMRAD_OK;
}

int lumrad_request_update(LumRadContext ctx, int x, int y, int z) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    const DeviceWorld& w = c->world;
    if (x < 0 || y < 0 || z < 0 || x >= w.X || y >= w.Y || z >= w.Z) return fail(LUMRAD_EINVAL, "request outside the world");
    c->specials.insert(c->specials.end(), {(int16_t)x, (int16_t)y, (int16_t)z, 0});
    return LUMRAD_OK;
}

int lumrad_build_update_list(LumRadContext ctx, int16_t* out, int cap, int* n) {
    Context* c = as_ctx(ctx);
    if (!c || !n || (cap > 0 && !out)) return fail(LUMRAD_EINVAL, "null argument");
    if (int rc = check_unowned(c)) return rc;
    LUMRAD_TRY(cudaSetDevice(c->device));
    int total = 0;
    int rc = c->build_list_device(false, &total);   // building the list alone keeps the queue
    if (rc) return rc;
    if (cap > 0 && total > 0) {
        LUMRAD_TRY(cudaMemcpyAsync(out, c->d_req, (size_t)std::min(total, cap) * sizeof(short4), cudaMemcpyDeviceToHost,
                                   c->stream));
        LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    }
    *n = total;
    return LUMRAD_OK;
}

int lumrad_build_dirty_list(LumRadContext ctx, const LumRadEdit* edits, int n_edits, int radius, int16_t* out, int cap,
                            int* n) {
    Context* c = as_ctx(ctx);
    if (!c || !n || n_edits < 0 || (n_edits > 0 && !edits) || (cap > 0 && !out)) return fail(LUMRAD_EINVAL, "bad argument");
    if (radius < 0 || radius > 15) return fail(LUMRAD_EINVAL, "radius must be in [0, 15]");
    const DeviceWorld& w = c->world;
    for (int k = 0; k < n_edits; k++)
        if (edits[k].x < 0 || edits[k].y < 0 || edits[k].z < 0 || edits[k].x >= w.X || edits[k].y >= w.Y || edits[k].z >= w.Z)
            return fail(LUMRAD_EINVAL, "edit outside the world");
    LUMRAD_TRY(cudaSetDevice(c->device));
    int rc = c->ensure_list_scratch();
    if (rc) return rc;
    if ((rc = c->ensure_req_capacity(w.W))) return rc;
    if (!c->d_dirty_mask) LUMRAD_TRY(cudaMalloc(&c->d_dirty_mask, 2 * w.W));
    if ((size_t)n_edits > c->edits_cap) {
        LUMRAD_TRY(cudaStreamSynchronize(c->stream));
        cudaFree(c->d_edits);
        c->d_edits = nullptr;
        c->edits_cap = 0;
        LUMRAD_TRY(cudaMalloc(&c->d_edits, std::max<size_t>(n_edits, 256) * sizeof(short4)));
        c->edits_cap = std::max<size_t>(n_edits, 256);
    }
    if (n_edits > 0)
        LUMRAD_TRY(cudaMemcpyAsync(c->d_edits, edits, (size_t)n_edits * sizeof(short4), cudaMemcpyHostToDevice, c->stream));
    LUMRAD_TRY(launch_dirty_list(c->d_edits, n_edits, w.X, w.Y, w.Z, radius, c->d_dirty_mask, c->d_dirty_mask + w.W,
                                 c->list, c->d_req, c->d_list_count, c->stream));
    LUMRAD_TRY(cudaMemcpyAsync(c->h_list_count, c->d_list_count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    const int total = *c->h_list_count;
    if (cap > 0 && total > 0) {
        LUMRAD_TRY(cudaMemcpyAsync(out, c->d_req, (size_t)std::min(total, cap) * sizeof(short4), cudaMemcpyDeviceToHost,
                                   c->stream));
        LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    }
    *n = total;
    return LUMRAD_OK;
}

int lumrad_update_radiance(LumRadContext ctx, const LumRadPassParams* params) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    int rc = check_params(params);
    if (rc) return rc;
    LUMRAD_TRY(cudaSetDevice(c->device));
    if (params->size == 0 && c->have_pass) {
        if (c->test_pass_ms >= 0.0f) {
            c->last_ms = c->test_pass_ms;
        } else {
            if ((rc = c->read_times())) return rc;
            c->last_ms = c->slot_ms(c->last_slot);
            c->last_ms /= (float)c->last_slot_passes;   // a frame's pass time after a several-pass call
        }
    }
    if ((rc = check_unowned(c))) return rc;
    // a frame of Renderer::submitFrame: shift_radiance, then update_radiance (renderer.cpp:436-438)
    if ((rc = c->shift_volume(c->shift[0], c->shift[1], c->shift[2]))) return rc;
    if (params->record_hits) {   // hit records are sized by the list's length: wait for it
        int n = 0;
        if ((rc = c->build_list_device(true, &n))) return rc;
        return c->run_pass(c->d_req, n, params);
    }
    // the pass is launched for the longest list (every block plus the queued specials) and reads
    // the list's length on the device: the call does not wait for the GPU
    const long long longest = (long long)c->world.W + (long long)(c->specials.size() / 4);
    if (longest >= (1LL << 31)) return fail(LUMRAD_EINVAL, "update list too long");
    if ((rc = c->build_list_device(true, nullptr))) return rc;
    return c->run_pass(c->d_req, (int)longest, params, c->d_list_count);
}

int lumrad_shift_radiance(LumRadContext ctx, int dx, int dy, int dz) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    if (int rc = check_unowned(c)) return rc;
    LUMRAD_TRY(cudaSetDevice(c->device));
    return c->shift_volume(dx, dy, dz);
}

int lumrad_set_radiance_shift(LumRadContext ctx, int dx, int dy, int dz) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    c->shift[0] = dx;
    c->shift[1] = dy;
    c->shift[2] = dz;
    return LUMRAD_OK;
}

int lumrad_get_radiance_shift(LumRadContext ctx, int* shift) {
    Context* c = as_ctx(ctx);
    if (!c || !shift) return fail(LUMRAD_EINVAL, "null argument");
    for (int i = 0; i < 3; i++) shift[i] = c->shift[i];
    return LUMRAD_OK;
}

int lumrad_gather_radiance_device(LumRadContext ctx, const float* d_points, int n, float* d_rgb) {
    Context* c = as_ctx(ctx);
    if (!c || n < 0 || (n > 0 && (!d_points || !d_rgb))) return fail(LUMRAD_EINVAL, "bad argument");
    LUMRAD_TRY(cudaSetDevice(c->device));
    const DeviceWorld& w = c->world;
    LUMRAD_TRY(launch_gather(w.d_rad[w.cur], w.X, w.Y, w.Z, w.precision, d_points, n, d_rgb, c->stream));
    return LUMRAD_OK;
}

int lumrad_gather_radiance(LumRadContext ctx, const float* points, int n, float* rgb) {
    Context* c = as_ctx(ctx);
    if (!c || n < 0 || (n > 0 && (!points || !rgb))) return fail(LUMRAD_EINVAL, "bad argument");
    if (n == 0) return LUMRAD_OK;
    LUMRAD_TRY(cudaSetDevice(c->device));
    if ((size_t)n > c->gather_cap) {
        LUMRAD_TRY(cudaStreamSynchronize(c->stream));
        cudaFree(c->d_gather);
        c->d_gather = nullptr;
        c->gather_cap = 0;
        LUMRAD_TRY(cudaMalloc(&c->d_gather, (size_t)n * 9 * sizeof(float)));
        c->gather_cap = (size_t)n;
    }
    float* d_pts = c->d_gather;
    float* d_out = c->d_gather + (size_t)n * 6;
    LUMRAD_TRY(cudaMemcpyAsync(d_pts, points, (size_t)n * 6 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    int rc = lumrad_gather_radiance_device(ctx, d_pts, n, d_out);
    if (rc) return rc;
    LUMRAD_TRY(cudaMemcpyAsync(rgb, d_out, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    return LUMRAD_OK;
}

int lumrad_radiance_pass(LumRadContext ctx, const int16_t* requests, int n, const LumRadPassParams* params) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    if (n < 0 || (n > 0 && !requests)) return fail(LUMRAD_EINVAL, "bad request list");
    int rc = check_params(params);
    if (rc) return rc;
    if (params->size == 0) return fail(LUMRAD_EINVAL, "size 0 (adaptive) is only valid for lumrad_update_radiance");
    LUMRAD_TRY(cudaSetDevice(c->device));
    if ((rc = c->stage_requests(requests, (size_t)n))) return rc;
    return c->run_pass(c->d_req, n, params);
}

int lumrad_radiance_pass_i8(LumRadContext ctx, const int8_t* requests, int n, const LumRadPassParams* params) {
    if (n < 0 || (n > 0 && !requests)) return fail(LUMRAD_EINVAL, "bad request list");
    std::vector<int16_t> wide((size_t)n * 4);
    for (size_t i = 0; i < wide.size(); i++) wide[i] = requests[i];   // i8vec4 -> ivec4, sign-extended
    return lumrad_radiance_pass(ctx, wide.data(), n, params);
}

int lumrad_upload_requests(LumRadContext ctx, int slot, const int16_t* requests, int n) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    if (n < 0 || (n > 0 && !requests) || slot < 0) return fail(LUMRAD_EINVAL, "bad request list");
    LUMRAD_TRY(cudaSetDevice(c->device));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    auto& r = c->resident[slot];
    cudaFree(r.ptr);
    r.ptr = nullptr;
    r.n = 0;
    LUMRAD_TRY(cudaMalloc(&r.ptr, std::max(n, 1) * sizeof(short4)));
    if (n > 0) LUMRAD_TRY(cudaMemcpyAsync(r.ptr, requests, (size_t)n * sizeof(short4), cudaMemcpyHostToDevice, c->stream));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    r.n = n;
    return LUMRAD_OK;
}

int lumrad_radiance_pass_resident(LumRadContext ctx, int slot, const LumRadPassParams* params) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    auto it = c->resident.find(slot);
    if (it == c->resident.end()) return fail(LUMRAD_EINVAL, "no request list uploaded in this slot");
    int rc = check_params(params);
    if (rc) return rc;
    if (params->size == 0) return fail(LUMRAD_EINVAL, "size 0 (adaptive) is only valid for lumrad_update_radiance");
    LUMRAD_TRY(cudaSetDevice(c->device));
    return c->run_pass(it->second.ptr, it->second.n, params);
}

static int check_pass_list(const LumRadPassParams* params, int n) {
    if (n < 0 || (n > 0 && !params)) return fail(LUMRAD_EINVAL, "bad pass list");
    for (int i = 0; i < n; i++) {
        int rc = check_params(&params[i]);
        if (rc) return rc;
        if (params[i].size == 0) return fail(LUMRAD_EINVAL, "size 0 (adaptive) is only valid for lumrad_update_radiance");
        if (params[i].record_hits) return fail(LUMRAD_EINVAL, "hit records need lumrad_radiance_pass");
    }
    return LUMRAD_OK;
}

int lumrad_radiance_passes(LumRadContext ctx, const int16_t* const* requests, const int* counts,
                           const LumRadPassParams* params, int n) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    int rc = check_pass_list(params, n);
    if (rc) return rc;
    if (n > 0 && (!requests || !counts)) return fail(LUMRAD_EINVAL, "bad request lists");
    size_t total = 0;
    for (int i = 0; i < n; i++) {
        if (counts[i] < 0 || (counts[i] > 0 && !requests[i])) return fail(LUMRAD_EINVAL, "bad request list");
        total += (size_t)counts[i];
    }
    if (n == 0) return LUMRAD_OK;
    LUMRAD_TRY(cudaSetDevice(c->device));
    if ((rc = check_unowned(c))) return rc;
    if ((rc = c->ensure_req_capacity(total))) return rc;
    if (c->req_copy_pending) {
        LUMRAD_TRY(cudaEventSynchronize(c->ev_req));
        c->req_copy_pending = false;
    }
    std::vector<const short4*> reqs((size_t)n);
    // Page-locked lists and an idle stream: DMA straight from the caller's arrays (one copy per
    // run of adjacent lists), launch, and return once the copies (not the passes) are done.
    const cudaError_t idle = cudaStreamQuery(c->stream);
    if (idle == cudaErrorNotReady) cudaGetLastError();   // a busy stream is no error for later checks
    bool direct = total > 0 && idle == cudaSuccess;
    // runs of adjacent lists (each run one copy, its page-locking checked once)
    struct Run { const int16_t* src; size_t first, count; };
    std::vector<Run> runs;
    if (direct) {
        size_t off = 0;
        int i = 0;
        while (i < n && direct) {
            if (counts[i] == 0) { reqs[i++] = c->d_req + off; continue; }
            const Run r0{requests[i], off, 0};
            int j = i;
            while (j < n && (counts[j] == 0 || requests[j] == r0.src + (off - r0.first) * 4)) {
                reqs[j] = c->d_req + off;
                off += (size_t)counts[j++];
            }
            runs.push_back(Run{r0.src, r0.first, off - r0.first});
            direct = host_pinned(r0.src, (off - r0.first) * 4 * sizeof(int16_t));
            i = j;
        }
    }
    if (direct) {
        for (const Run& r : runs) {
            const cudaError_t e = cudaMemcpyAsync(c->d_req + r.first, r.src, r.count * sizeof(short4),
                                                  cudaMemcpyHostToDevice, c->stream);
            if (e != cudaSuccess) {
                cudaStreamSynchronize(c->stream);   // no copy may still read the caller's arrays
                return fail(LUMRAD_EDEVICE, std::string("request copy: ") + cudaGetErrorString(e));
            }
        }
        if (cudaEventRecord(c->ev_req, c->stream) != cudaSuccess) {
            cudaStreamSynchronize(c->stream);
            return fail(LUMRAD_EDEVICE, "request copy: event record failed");
        }
        rc = c->run_passes(reqs.data(), counts, params, n);
        LUMRAD_TRY(cudaEventSynchronize(c->ev_req));
        return rc;
    }
    // else every list through one pinned buffer and one copy
    if (total > c->h_req_cap) {
        if (c->h_req_pinned) cudaFreeHost(c->h_req_pinned);
        c->h_req_pinned = nullptr;
        c->h_req_cap = 0;
        const size_t cap = std::max<size_t>(total, 1024);
        LUMRAD_TRY(cudaMallocHost(&c->h_req_pinned, cap * 4 * sizeof(int16_t)));
        c->h_req_cap = cap;
    }
    size_t off = 0;
    for (int i = 0; i < n; i++) {
        if (counts[i] > 0) std::memcpy(c->h_req_pinned + off * 4, requests[i], (size_t)counts[i] * 4 * sizeof(int16_t));
        reqs[i] = c->d_req + off;
        off += (size_t)counts[i];
    }
    if (total > 0) {
        LUMRAD_TRY(cudaMemcpyAsync(c->d_req, c->h_req_pinned, total * sizeof(short4), cudaMemcpyHostToDevice, c->stream));
        LUMRAD_TRY(cudaEventRecord(c->ev_req, c->stream));
        c->req_copy_pending = true;
    }
    return c->run_passes(reqs.data(), counts, params, n);
}

int lumrad_radiance_passes_resident(LumRadContext ctx, const int* slots, const LumRadPassParams* params, int n) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    int rc = check_pass_list(params, n);
    if (rc) return rc;
    if (n > 0 && !slots) return fail(LUMRAD_EINVAL, "bad slot list");
    std::vector<const short4*> reqs((size_t)n);
    std::vector<int> counts((size_t)n);
    for (int i = 0; i < n; i++) {
        auto it = c->resident.find(slots[i]);
        if (it == c->resident.end()) return fail(LUMRAD_EINVAL, "no request list uploaded in this slot");
        reqs[i] = it->second.ptr;
        counts[i] = it->second.n;
    }
    if (n == 0) return LUMRAD_OK;
    LUMRAD_TRY(cudaSetDevice(c->device));
    return c->run_passes(reqs.data(), counts.data(), params, n);
}

int lumrad_get_hits(LumRadContext ctx, LumRadHit* out, size_t cap, size_t* n) {
    Context* c = as_ctx(ctx);
    if (!c || !n || (cap > 0 && !out)) return fail(LUMRAD_EINVAL, "null argument");
    if (!c->have_pass || !c->world.hits_recorded) {
        *n = 0;
        return fail(LUMRAD_ESTATE, "the last pass did not record hits");
    }
    LUMRAD_TRY(cudaSetDevice(c->device));
    const size_t k = std::min(cap, c->world.hits_n);
    if (k > 0) LUMRAD_TRY(cudaMemcpyAsync(out, c->world.d_hits, k * sizeof(LumRadHit), cudaMemcpyDeviceToHost, c->stream));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    *n = c->world.hits_n;
    return c->check_error();
}

int lumrad_get_pass_stats(LumRadContext ctx, LumRadPassStats* out) {
    Context* c = as_ctx(ctx);
    if (!c || !out) return fail(LUMRAD_EINVAL, "null argument");
    if (!c->have_pass) return fail(LUMRAD_ESTATE, "no pass has run");
    LUMRAD_TRY(cudaSetDevice(c->device));
    unsigned long long h[2];
    int count = 0;
    LUMRAD_TRY(cudaMemcpyAsync(h, c->world.d_stats, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    if (c->last_count_on_device)
        LUMRAD_TRY(cudaMemcpyAsync(&count, c->d_last_count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    if (int rc = c->read_times()) return rc;
    const float ms = c->slot_ms(c->last_slot);
    *out = c->last;
    if (c->last_count_on_device) {
        out->probes = (uint64_t)(count / c->last_size);
        out->rays = out->probes * (uint64_t)c->last_R;
    }
    out->steps = h[0];
    out->hits = h[1];
    out->gpu_ms = ms;
    return c->check_error();
}

int lumrad_test_hook(LumRadContext ctx, int hook, double value) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    switch (hook) {
        case LUMRAD_TEST_LEAN_FINALIZE: c->test_lean_finalize = value != 0.0; return LUMRAD_OK;
        case LUMRAD_TEST_PASS_MS: c->test_pass_ms = value >= 0.0 ? (float)value : -1.0f; return LUMRAD_OK;
        default: return fail(LUMRAD_EINVAL, "unknown test hook");
    }
}

int lumrad_get_stream(LumRadContext ctx, void** stream) {
    Context* c = as_ctx(ctx);
    if (!c || !stream) return fail(LUMRAD_EINVAL, "null argument");
    *stream = (void*)c->stream;
    return LUMRAD_OK;
}

int lumrad_get_kernel_times(LumRadContext ctx, float* ms, int cap, int* n) {
    Context* c = as_ctx(ctx);
    if (!c || !n || (cap > 0 && !ms)) return fail(LUMRAD_EINVAL, "null argument");
    LUMRAD_TRY(cudaSetDevice(c->device));
    if (int rc = c->read_times()) return rc;
    const long long avail = std::min<long long>(c->n_passes, Context::kRing);
    const int k = (int)std::min<long long>(avail, std::max(cap, 0));
    for (int i = 0; i < k; i++) {
        const long long pass = c->n_passes - k + i;
        ms[i] = c->slot_ms((int)(pass % Context::kRing));
    }
    *n = k;
    return c->check_error();
}

int lumrad_direction_table(int rays_per_probe, float* xyz) {
    if (rays_per_probe < 1 || rays_per_probe > 1024 || !xyz) return fail(LUMRAD_EINVAL, "bad argument");
    fibonacci_table(rays_per_probe, xyz);
    return LUMRAD_OK;
}

}  // extern "C"
