// lumrad_host.cpp — the C ABI of include/lumrad.h: contexts, resident device data, passes.
//
// One context = one world resident on one GPU (grid, palettes, materials, two radiance volumes
// for ping-pong) plus a stream, events and pinned staging for update lists.  It replaces the
// radiance part of LumInternal::LumInternalRenderer: the resources of createImages
// (src/renderer/src/internal_render.cpp:107-209), the uploads of updateBlockPalette /
// updateMaterialPalette (load_stuff.cpp:36-111) and exec_copies' world upload
// (internal_render.cpp:1460-1475), and update_radiance itself (internal_render.cpp:1129-1214).

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "lumrad_internal.h"

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

#define LUMRAD_CUDA(expr)                                                                  \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return fail(LUMRAD_EDEVICE, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

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

float unorm_clamp(float v) { return v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f; }

struct Context {
    int X = 0, Y = 0, Z = 0;
    size_t W = 0;
    int n_slots = 0;
    int precision = 0;
    int device = 0;
    int num_sms = 0;
    size_t rad_stride = 16;   // bytes per probe

    std::vector<int16_t> h_grid;
    std::vector<uint8_t> h_pal;          // n_slots * 4096, device layout
    std::vector<LumRadMaterial> h_mats;  // 256
    std::vector<int16_t> specials;       // queued (x,y,z,w)
    bool grid_dirty = true;
    bool slot0_empty = true;

    int16_t* d_grid = nullptr;
    uint8_t* d_pal = nullptr;
    float4* d_mats = nullptr;
    void* d_rad[2] = {nullptr, nullptr};
    int cur = 0;
    short4* d_req = nullptr;
    size_t req_cap = 0;
    int16_t* h_req_pinned = nullptr;
    size_t h_req_cap = 0;
    std::map<int, float4*> d_dirs;
    struct Resident { short4* ptr = nullptr; int n = 0; };
    std::map<int, Resident> resident;
    LumRadHit* d_hits = nullptr;
    size_t hits_cap = 0, hits_n = 0;
    bool hits_recorded = false;          // the last pass ran with record_hits = 1
    unsigned long long* d_counters = nullptr;

    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_end = nullptr, ev_req = nullptr;
    static constexpr int kRing = 64;      // kernel-time history
    cudaEvent_t ring0[kRing] = {}, ring1[kRing] = {};
    long long n_passes = 0;
    bool have_pass = false;
    bool req_copy_pending = false;
    LumRadPassStats last{};

    // adaptive time slicing state (internal_render.cpp:1190-1203)
    int frame = 0;
    int magic_size = 1;
    float last_ms = 0.0f;
};

Context* as_ctx(LumRadContext c) { return reinterpret_cast<Context*>(c); }

int set_device(Context* c) {
    LUMRAD_CUDA(cudaSetDevice(c->device));
    return LUMRAD_OK;
}

int ensure_dirs(Context* c, int R, const float4** out) {
    auto it = c->d_dirs.find(R);
    if (it != c->d_dirs.end()) {
        *out = it->second;
        return LUMRAD_OK;
    }
    std::vector<float> xyz(3 * (size_t)R);
    fibonacci_table(R, xyz.data());
    std::vector<float4> t(R);
    for (int i = 0; i < R; i++) t[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
    float4* d = nullptr;
    LUMRAD_CUDA(cudaMalloc(&d, sizeof(float4) * R));
    LUMRAD_CUDA(cudaMemcpyAsync(d, t.data(), sizeof(float4) * R, cudaMemcpyHostToDevice, c->stream));
    LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    c->d_dirs[R] = d;
    *out = d;
    return LUMRAD_OK;
}

int upload_grid(Context* c) {
    if (!c->grid_dirty) return LUMRAD_OK;
    LUMRAD_CUDA(cudaMemcpyAsync(c->d_grid, c->h_grid.data(), c->W * sizeof(int16_t),
                                cudaMemcpyHostToDevice, c->stream));
    LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    c->grid_dirty = false;
    return LUMRAD_OK;
}

int check_params(const Context* c, const LumRadPassParams* p) {
    if (!p) return fail(LUMRAD_EINVAL, "params is null");
    if (p->rays_per_probe < 32 || p->rays_per_probe > 1024 || p->rays_per_probe % 32 != 0)
        return fail(LUMRAD_EINVAL, "rays_per_probe must be a multiple of 32 in [32, 1024]");
    if (!(p->max_dist > 0.0f) || p->max_dist > 16384.0f)
        return fail(LUMRAD_EINVAL, "max_dist must be in (0, 16384]");
    if (!(p->blend >= 0.0f && p->blend <= 1.0f)) return fail(LUMRAD_EINVAL, "blend must be in [0, 1]");
    if (p->size < 0 || p->size > (1 << 20)) return fail(LUMRAD_EINVAL, "size out of range");
    if (p->size > 0 && (p->shift < 0 || p->shift >= p->size))
        return fail(LUMRAD_EINVAL, "shift must be in [0, size)");
    (void)c;
    return LUMRAD_OK;
}

int ensure_req_capacity(Context* c, size_t n) {
    if (n <= c->req_cap) return LUMRAD_OK;
    if (c->d_req) cudaFree(c->d_req);
    c->d_req = nullptr;
    size_t cap = std::max<size_t>(n, 1024);
    LUMRAD_CUDA(cudaMalloc(&c->d_req, cap * sizeof(short4)));
    c->req_cap = cap;
    return LUMRAD_OK;
}

// Copies n requests (x,y,z,w int16) into the device list through pinned staging.
int stage_requests(Context* c, const int16_t* req, size_t n) {
    int rc = ensure_req_capacity(c, n);
    if (rc) return rc;
    if (n == 0) return LUMRAD_OK;
    if (c->req_copy_pending) {
        LUMRAD_CUDA(cudaEventSynchronize(c->ev_req));
        c->req_copy_pending = false;
    }
    if (n > c->h_req_cap) {
        if (c->h_req_pinned) cudaFreeHost(c->h_req_pinned);
        c->h_req_pinned = nullptr;
        size_t cap = std::max<size_t>(n, 1024);
        LUMRAD_CUDA(cudaMallocHost(&c->h_req_pinned, cap * 4 * sizeof(int16_t)));
        c->h_req_cap = cap;
    }
    std::memcpy(c->h_req_pinned, req, n * 4 * sizeof(int16_t));
    LUMRAD_CUDA(cudaMemcpyAsync(c->d_req, c->h_req_pinned, n * sizeof(short4), cudaMemcpyHostToDevice,
                                c->stream));
    LUMRAD_CUDA(cudaEventRecord(c->ev_req, c->stream));
    c->req_copy_pending = true;
    return LUMRAD_OK;
}

// One pass over `n` requests already on the device at `d_req`.
int run_pass(Context* c, const short4* d_req, int n, const LumRadPassParams* p_in) {
    LumRadPassParams p = *p_in;
    if (p.size == 0) {
        // adaptive slicing of update_radiance (internal_render.cpp:1190-1203)
        if (c->last_ms < 1.8f) c->magic_size--;
        else if (c->last_ms > 2.2f) c->magic_size++;
        c->magic_size = std::min(std::max(c->magic_size, 1), 10);
        p.size = c->magic_size;
        p.shift = c->frame % c->magic_size;
        p.time_seed = c->frame;
    }
    c->frame++;
    int rc = upload_grid(c);
    if (rc) return rc;
    const float4* dirs = nullptr;
    rc = ensure_dirs(c, p.rays_per_probe, &dirs);
    if (rc) return rc;
    const int groups = n / p.size;
    const int R = p.rays_per_probe;
    if (p.record_hits) {
        const size_t need = (size_t)groups * R;
        if (need > c->hits_cap) {
            if (c->d_hits) cudaFree(c->d_hits);
            c->d_hits = nullptr;
            c->hits_cap = 0;
            LUMRAD_CUDA(cudaMalloc(&c->d_hits, std::max<size_t>(need, 1) * sizeof(LumRadHit)));
            c->hits_cap = std::max<size_t>(need, 1);
        }
        c->hits_n = need;
        c->hits_recorded = true;
    } else {
        c->hits_n = 0;
        c->hits_recorded = false;
    }
    const int src = c->cur, dst = 1 - c->cur;
    LUMRAD_CUDA(cudaMemcpyAsync(c->d_rad[dst], c->d_rad[src], c->W * c->rad_stride,
                                cudaMemcpyDeviceToDevice, c->stream));
    LUMRAD_CUDA(cudaMemsetAsync(c->d_counters, 0, 2 * sizeof(unsigned long long), c->stream));

    lumrad::PassArgs a{};
    a.w.X = c->X; a.w.Y = c->Y; a.w.Z = c->Z;
    a.w.n_slots = c->n_slots;
    a.w.slot0_empty = c->slot0_empty ? 1 : 0;
    a.w.grid = c->d_grid;
    a.w.pal = c->d_pal;
    a.w.mats = c->d_mats;
    a.prev = c->d_rad[src];
    a.next = c->d_rad[dst];
    a.req = d_req;
    a.n_groups = groups;
    a.size = p.size;
    a.shift = p.shift;
    a.R = R;
    a.probes_per_unit = R <= lumrad::kPool ? lumrad::kPool / R : 1;
    a.max_dist = p.max_dist;
    a.max_steps = (int)(2.0f * p.max_dist) + 2;
    a.alpha = p.blend;
    a.one_minus_alpha = 1.0f - p.blend;
    a.seed = (uint32_t)p.time_seed;
    a.dirs = dirs;
    a.hits = p.record_hits ? c->d_hits : nullptr;
    a.counters = c->d_counters;

    const int slot = (int)(c->n_passes % Context::kRing);
    LUMRAD_CUDA(cudaEventRecord(c->ev_start, c->stream));
    LUMRAD_CUDA(cudaEventRecord(c->ring0[slot], c->stream));
    LUMRAD_CUDA(lumrad::launch_radiance_pass(a, c->precision, p.record_hits != 0, true, c->num_sms,
                                             c->stream));
    LUMRAD_CUDA(cudaEventRecord(c->ring1[slot], c->stream));
    LUMRAD_CUDA(cudaEventRecord(c->ev_end, c->stream));
    c->n_passes++;
    c->cur = dst;
    c->have_pass = true;
    c->last.probes = (uint64_t)groups;
    c->last.rays = (uint64_t)groups * R;
    return LUMRAD_OK;
}

}  // namespace

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
    if (s->precision < 0 || s->precision > 2) return fail(LUMRAD_EINVAL, "unknown precision");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(LUMRAD_EDEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (s->device < 0 || s->device >= ndev) return fail(LUMRAD_EINVAL, "device ordinal out of range");

    Context* c = new Context();
    c->X = s->world_size[0]; c->Y = s->world_size[1]; c->Z = s->world_size[2];
    c->W = (size_t)W;
    c->n_slots = s->max_block_types;
    c->precision = s->precision;
    c->device = s->device;
    c->rad_stride = s->precision == LUMRAD_PRECISION_FP32 ? 16 : 8;
    c->h_grid.assign(c->W, 0);
    c->h_pal.assign((size_t)c->n_slots * 4096, 0);
    c->h_mats.assign(LUMRAD_MATERIALS, LumRadMaterial{});
    auto cleanup = [&](int rc) {
        lumrad_destroy(c);
        return rc;
    };
    int rc = set_device(c);
    if (rc) return cleanup(rc);
#define CREATE_CUDA(expr)                                                                      \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return cleanup(fail(e_ == cudaErrorMemoryAllocation ? LUMRAD_ENOMEM : LUMRAD_EDEVICE, \
                                std::string(#expr) + ": " + cudaGetErrorString(e_)));          \
    } while (0)
    CREATE_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device));
    CREATE_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CREATE_CUDA(cudaEventCreate(&c->ev_start));
    CREATE_CUDA(cudaEventCreate(&c->ev_end));
    CREATE_CUDA(cudaEventCreateWithFlags(&c->ev_req, cudaEventDisableTiming));
    for (int i = 0; i < Context::kRing; i++) {
        CREATE_CUDA(cudaEventCreate(&c->ring0[i]));
        CREATE_CUDA(cudaEventCreate(&c->ring1[i]));
    }
    CREATE_CUDA(cudaMalloc(&c->d_grid, c->W * sizeof(int16_t)));
    CREATE_CUDA(cudaMalloc(&c->d_pal, c->h_pal.size()));
    CREATE_CUDA(cudaMalloc(&c->d_mats, LUMRAD_MATERIALS * sizeof(float4)));
    for (int i = 0; i < 2; i++) {
        CREATE_CUDA(cudaMalloc(&c->d_rad[i], c->W * c->rad_stride));
        CREATE_CUDA(cudaMemsetAsync(c->d_rad[i], 0, c->W * c->rad_stride, c->stream));
    }
    CREATE_CUDA(cudaMalloc(&c->d_counters, 2 * sizeof(unsigned long long)));
    CREATE_CUDA(cudaMemsetAsync(c->d_grid, 0, c->W * sizeof(int16_t), c->stream));
    CREATE_CUDA(cudaMemsetAsync(c->d_pal, 0, c->h_pal.size(), c->stream));
    CREATE_CUDA(cudaMemsetAsync(c->d_mats, 0, LUMRAD_MATERIALS * sizeof(float4), c->stream));
    CREATE_CUDA(cudaStreamSynchronize(c->stream));
#undef CREATE_CUDA
    c->grid_dirty = false;
    *out = c;
    return LUMRAD_OK;
}

void lumrad_destroy(LumRadContext ctx) {
    Context* c = as_ctx(ctx);
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->d_grid);
    cudaFree(c->d_pal);
    cudaFree(c->d_mats);
    cudaFree(c->d_rad[0]);
    cudaFree(c->d_rad[1]);
    cudaFree(c->d_req);
    cudaFree(c->d_hits);
    cudaFree(c->d_counters);
    for (auto& kv : c->d_dirs) cudaFree(kv.second);
    for (auto& kv : c->resident) cudaFree(kv.second.ptr);
    if (c->h_req_pinned) cudaFreeHost(c->h_req_pinned);
    if (c->ev_start) cudaEventDestroy(c->ev_start);
    if (c->ev_end) cudaEventDestroy(c->ev_end);
    if (c->ev_req) cudaEventDestroy(c->ev_req);
    for (int i = 0; i < Context::kRing; i++) {
        if (c->ring0[i]) cudaEventDestroy(c->ring0[i]);
        if (c->ring1[i]) cudaEventDestroy(c->ring1[i]);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int lumrad_synchronize(LumRadContext ctx) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    LUMRAD_CUDA(cudaSetDevice(c->device));
    LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    return LUMRAD_OK;
}

int lumrad_load_world(LumRadContext ctx, const int16_t* blocks) {
    Context* c = as_ctx(ctx);
    if (!c || !blocks) return fail(LUMRAD_EINVAL, "null argument");
    std::memcpy(c->h_grid.data(), blocks, c->W * sizeof(int16_t));
    c->grid_dirty = true;
    int rc = set_device(c);
    if (rc) return rc;
    return upload_grid(c);
}

int lumrad_set_world_block(LumRadContext ctx, int x, int y, int z, int16_t block) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    if (x < 0 || y < 0 || z < 0 || x >= c->X || y >= c->Y || z >= c->Z)
        return fail(LUMRAD_EINVAL, "block coordinate out of the world");
    c->h_grid[(size_t)x + (size_t)c->X * ((size_t)y + (size_t)c->Y * z)] = block;
    c->grid_dirty = true;   // uploaded before the next pass, as exec_copies does every frame
    return LUMRAD_OK;
}

int lumrad_get_world_block(LumRadContext ctx, int x, int y, int z, int16_t* block) {
    Context* c = as_ctx(ctx);
    if (!c || !block) return fail(LUMRAD_EINVAL, "null argument");
    if (x < 0 || y < 0 || z < 0 || x >= c->X || y >= c->Y || z >= c->Z)
        return fail(LUMRAD_EINVAL, "block coordinate out of the world");
    *block = c->h_grid[(size_t)x + (size_t)c->X * ((size_t)y + (size_t)c->Y * z)];
    return LUMRAD_OK;
}

int lumrad_load_block(LumRadContext ctx, int16_t block, const uint8_t* voxels) {
    Context* c = as_ctx(ctx);
    if (!c || !voxels) return fail(LUMRAD_EINVAL, "null argument");
    if (block < 0 || block >= c->n_slots) return fail(LUMRAD_EINVAL, "block id outside the palette slots");
    // BlockVoxels[x][y][z] (z fastest) -> x-fastest slot, as updateBlockPalette repacks it
    uint8_t* dst = c->h_pal.data() + (size_t)block * 4096;
    for (int x = 0; x < 16; x++)
        for (int y = 0; y < 16; y++)
            for (int z = 0; z < 16; z++) dst[x + 16 * y + 256 * z] = voxels[(x * 16 + y) * 16 + z];
    return LUMRAD_OK;
}

int lumrad_upload_block_palette(LumRadContext ctx) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    int rc = set_device(c);
    if (rc) return rc;
    c->slot0_empty = std::all_of(c->h_pal.begin(), c->h_pal.begin() + 4096, [](uint8_t v) { return v == 0; });
    LUMRAD_CUDA(cudaMemcpyAsync(c->d_pal, c->h_pal.data(), c->h_pal.size(), cudaMemcpyHostToDevice, c->stream));
    LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    return LUMRAD_OK;
}

int lumrad_load_materials(LumRadContext ctx, const LumRadMaterial* materials) {
    Context* c = as_ctx(ctx);
    if (!c || !materials) return fail(LUMRAD_EINVAL, "null argument");
    std::memcpy(c->h_mats.data(), materials, LUMRAD_MATERIALS * sizeof(LumRadMaterial));
    return LUMRAD_OK;
}

int lumrad_upload_material_palette(LumRadContext ctx) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    int rc = set_device(c);
    if (rc) return rc;
    std::vector<float4> m(LUMRAD_MATERIALS);
    for (int i = 0; i < LUMRAD_MATERIALS; i++)
        m[i] = make_float4(c->h_mats[i].color[0], c->h_mats[i].color[1], c->h_mats[i].color[2], c->h_mats[i].emmit);
    LUMRAD_CUDA(cudaMemcpyAsync(c->d_mats, m.data(), m.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
    LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    return LUMRAD_OK;
}

int lumrad_get_radiance(LumRadContext ctx, float* rgb) {
    Context* c = as_ctx(ctx);
    if (!c || !rgb) return fail(LUMRAD_EINVAL, "null argument");
    int rc = set_device(c);
    if (rc) return rc;
    if (c->precision == LUMRAD_PRECISION_FP32) {
        std::vector<float4> h(c->W);
        LUMRAD_CUDA(cudaMemcpyAsync(h.data(), c->d_rad[c->cur], c->W * 16, cudaMemcpyDeviceToHost, c->stream));
        LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
        for (size_t i = 0; i < c->W; i++) {
            rgb[3 * i] = h[i].x; rgb[3 * i + 1] = h[i].y; rgb[3 * i + 2] = h[i].z;
        }
    } else {
        std::vector<uint16_t> h(c->W * 4);
        LUMRAD_CUDA(cudaMemcpyAsync(h.data(), c->d_rad[c->cur], c->W * 8, cudaMemcpyDeviceToHost, c->stream));
        LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
        for (size_t i = 0; i < c->W; i++)
            for (int k = 0; k < 3; k++) {
                uint16_t bits = h[4 * i + k];
                float v;
                if (c->precision == LUMRAD_PRECISION_FP16) {
                    __half_raw r; r.x = bits;
                    v = __half2float(__half(r));
                } else {
                    uint32_t u = (uint32_t)bits << 16;
                    std::memcpy(&v, &u, 4);
                }
                rgb[3 * i + k] = v;
            }
    }
    return LUMRAD_OK;
}

int lumrad_set_radiance(LumRadContext ctx, const float* rgb) {
    Context* c = as_ctx(ctx);
    if (!c || !rgb) return fail(LUMRAD_EINVAL, "null argument");
    int rc = set_device(c);
    if (rc) return rc;
    if (c->precision == LUMRAD_PRECISION_FP32) {
        std::vector<float4> h(c->W);
        for (size_t i = 0; i < c->W; i++)
            h[i] = make_float4(unorm_clamp(rgb[3 * i]), unorm_clamp(rgb[3 * i + 1]), unorm_clamp(rgb[3 * i + 2]), 1.0f);
        LUMRAD_CUDA(cudaMemcpyAsync(c->d_rad[c->cur], h.data(), c->W * 16, cudaMemcpyHostToDevice, c->stream));
        LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    } else {
        std::vector<uint16_t> h(c->W * 4);
        for (size_t i = 0; i < c->W; i++)
            for (int k = 0; k < 4; k++) {
                float v = k < 3 ? unorm_clamp(rgb[3 * i + k]) : 1.0f;
                uint16_t bits;
                if (c->precision == LUMRAD_PRECISION_FP16) {
                    __half_raw r = __half_raw(__float2half_rn(v));
                    bits = r.x;
                } else {
                    __nv_bfloat16_raw r = __nv_bfloat16_raw(__float2bfloat16_rn(v));
                    bits = r.x;
                }
                h[4 * i + k] = bits;
            }
        LUMRAD_CUDA(cudaMemcpyAsync(c->d_rad[c->cur], h.data(), c->W * 8, cudaMemcpyHostToDevice, c->stream));
        LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    }
    return LUMRAD_OK;
}

int lumrad_request_update(LumRadContext ctx, int x, int y, int z) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    if (x < 0 || y < 0 || z < 0 || x >= c->X || y >= c->Y || z >= c->Z)
        return fail(LUMRAD_EINVAL, "request outside the world");
    c->specials.insert(c->specials.end(), {(int16_t)x, (int16_t)y, (int16_t)z, 0});
    return LUMRAD_OK;
}

// The 27-neighbour rule of update_radiance (internal_render.cpp:1142-1161) plus specials
// (:1164-1168).  Specials are consumed, as the reference clears them.
static int build_list(Context* c, std::vector<int16_t>& out) {
    const int X = c->X, Y = c->Y, Z = c->Z;
    std::vector<uint8_t> set(c->W, 0);
    out.clear();
    const int16_t* g = c->h_grid.data();
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                int sum = 0;
                for (int dz = -1; dz <= 1; dz++) {
                    const int tz = std::min(std::max(z + dz, 0), Z - 1);
                    for (int dy = -1; dy <= 1; dy++) {
                        const int ty = std::min(std::max(y + dy, 0), Y - 1);
                        const int16_t* row = g + (size_t)X * ((size_t)ty + (size_t)Y * tz);
                        for (int dx = -1; dx <= 1; dx++) sum += row[std::min(std::max(x + dx, 0), X - 1)];
                    }
                }
                if (sum > 0) {
                    out.insert(out.end(), {(int16_t)x, (int16_t)y, (int16_t)z, 0});
                    set[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * z)] = 1;
                }
            }
    for (size_t i = 0; i + 3 < c->specials.size(); i += 4) {
        const int16_t* u = &c->specials[i];
        if (!set[(size_t)u[0] + (size_t)X * ((size_t)u[1] + (size_t)Y * u[2])]) out.insert(out.end(), u, u + 4);
    }
    c->specials.clear();
    return LUMRAD_OK;
}

int lumrad_build_update_list(LumRadContext ctx, int16_t* out, int cap, int* n) {
    Context* c = as_ctx(ctx);
    if (!c || !n || (cap > 0 && !out)) return fail(LUMRAD_EINVAL, "null argument");
    std::vector<int16_t> specials = c->specials;   // building the list alone keeps the queue
    std::vector<int16_t> list;
    build_list(c, list);
    c->specials = specials;
    const int total = (int)(list.size() / 4);
    std::memcpy(out, list.data(), (size_t)std::min(total, std::max(cap, 0)) * 4 * sizeof(int16_t));
    *n = total;
    return LUMRAD_OK;
}

int lumrad_update_radiance(LumRadContext ctx, const LumRadPassParams* params) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    int rc = check_params(c, params);
    if (rc) return rc;
    if ((rc = set_device(c))) return rc;
    if (params->size == 0 && c->have_pass) {
        LUMRAD_CUDA(cudaEventSynchronize(c->ev_end));
        LUMRAD_CUDA(cudaEventElapsedTime(&c->last_ms, c->ev_start, c->ev_end));
    }
    std::vector<int16_t> list;
    build_list(c, list);
    const size_t n = list.size() / 4;
    if ((rc = stage_requests(c, list.data(), n))) return rc;
    return run_pass(c, c->d_req, (int)n, params);
}

int lumrad_radiance_pass(LumRadContext ctx, const int16_t* requests, int n, const LumRadPassParams* params) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    if (n < 0 || (n > 0 && !requests)) return fail(LUMRAD_EINVAL, "bad request list");
    int rc = check_params(c, params);
    if (rc) return rc;
    if (params->size == 0) return fail(LUMRAD_EINVAL, "size 0 (adaptive) is only valid for lumrad_update_radiance");
    if ((rc = set_device(c))) return rc;
    if ((rc = stage_requests(c, requests, (size_t)n))) return rc;
    return run_pass(c, c->d_req, n, params);
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
    int rc = set_device(c);
    if (rc) return rc;
    auto& r = c->resident[slot];
    if (r.ptr) cudaFree(r.ptr);
    r.ptr = nullptr;
    r.n = 0;
    LUMRAD_CUDA(cudaMalloc(&r.ptr, std::max(n, 1) * sizeof(short4)));
    if (n > 0)
        LUMRAD_CUDA(cudaMemcpyAsync(r.ptr, requests, (size_t)n * sizeof(short4), cudaMemcpyHostToDevice, c->stream));
    LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    r.n = n;
    return LUMRAD_OK;
}

int lumrad_radiance_pass_resident(LumRadContext ctx, int slot, const LumRadPassParams* params) {
    Context* c = as_ctx(ctx);
    if (!c) return fail(LUMRAD_EINVAL, "null context");
    auto it = c->resident.find(slot);
    if (it == c->resident.end()) return fail(LUMRAD_EINVAL, "no request list uploaded in this slot");
    int rc = check_params(c, params);
    if (rc) return rc;
    if (params->size == 0) return fail(LUMRAD_EINVAL, "size 0 (adaptive) is only valid for lumrad_update_radiance");
    if ((rc = set_device(c))) return rc;
    return run_pass(c, it->second.ptr, it->second.n, params);
}

int lumrad_get_hits(LumRadContext ctx, LumRadHit* out, size_t cap, size_t* n) {
    Context* c = as_ctx(ctx);
    if (!c || !n || (cap > 0 && !out)) return fail(LUMRAD_EINVAL, "null argument");
    if (!c->have_pass || !c->hits_recorded) {
        *n = 0;
        return fail(LUMRAD_ESTATE, "the last pass did not record hits");
    }
    int rc = set_device(c);
    if (rc) return rc;
    const size_t k = std::min(cap, c->hits_n);
    if (k > 0)
        LUMRAD_CUDA(cudaMemcpyAsync(out, c->d_hits, k * sizeof(LumRadHit), cudaMemcpyDeviceToHost, c->stream));
    LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    *n = c->hits_n;
    return LUMRAD_OK;
}

int lumrad_get_pass_stats(LumRadContext ctx, LumRadPassStats* out) {
    Context* c = as_ctx(ctx);
    if (!c || !out) return fail(LUMRAD_EINVAL, "null argument");
    if (!c->have_pass) return fail(LUMRAD_ESTATE, "no pass has run");
    int rc = set_device(c);
    if (rc) return rc;
    unsigned long long h[2];
    LUMRAD_CUDA(cudaMemcpyAsync(h, c->d_counters, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    float ms = 0.0f;
    LUMRAD_CUDA(cudaEventElapsedTime(&ms, c->ev_start, c->ev_end));
    *out = c->last;
    out->steps = h[0];
    out->hits = h[1];
    out->gpu_ms = ms;
    return LUMRAD_OK;
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
    int rc = set_device(c);
    if (rc) return rc;
    LUMRAD_CUDA(cudaStreamSynchronize(c->stream));
    const long long avail = std::min<long long>(c->n_passes, Context::kRing);
    const int k = (int)std::min<long long>(avail, std::max(cap, 0));
    for (int i = 0; i < k; i++) {
        const long long pass = c->n_passes - k + i;
        const int slot = (int)(pass % Context::kRing);
        LUMRAD_CUDA(cudaEventElapsedTime(&ms[i], c->ring0[slot], c->ring1[slot]));
    }
    *n = k;
    return LUMRAD_OK;
}

int lumrad_direction_table(int rays_per_probe, float* xyz) {
    if (rays_per_probe < 1 || rays_per_probe > 1024 || !xyz) return fail(LUMRAD_EINVAL, "bad argument");
    fibonacci_table(rays_per_probe, xyz);
    return LUMRAD_OK;
}

}  // extern "C"
