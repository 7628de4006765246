// lumrad_world.h — host-side state of a resident world and of a C-ABI context.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "lumrad_internal.h"

namespace lumrad {

// An NVTX range around a host call, shown on profiler timelines (no cost without a tool attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Host side of the A2B10G10R10_UNORM format (the device side: StoreRGB10A2): a clamped value's
// code is the round-to-nearest-even of v * 1023 in FP32; a code reads back as code / 1023.
inline uint32_t unorm10_encode_host(float v) { return (uint32_t)std::nearbyint(v * 1023.0f); }
inline float unorm10_decode_host(uint32_t q) { return (float)q / 1023.0f; }
inline uint32_t rgb10a2_pack_host(float r, float g, float b) {
    return unorm10_encode_host(r) | (unorm10_encode_host(g) << 10) | (unorm10_encode_host(b) << 20) | (3u << 30);
}
// Bytes per probe of a radiance volume stored at `precision`.
inline size_t radiance_stride(int precision) {
    return precision == LUMRAD_PRECISION_FP32 ? 16 : precision == LUMRAD_PRECISION_RGB10A2 ? 4 : 8;
}

extern thread_local std::string g_error;
int fail(int code, const std::string& msg);
void fibonacci_table(int n, float* xyz);

#define LUMRAD_TRY(expr)                                                                            \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return ::lumrad::fail(e_ == cudaErrorMemoryAllocation ? LUMRAD_ENOMEM : LUMRAD_EDEVICE, \
                                  std::string(#expr) + ": " + cudaGetErrorString(e_));              \
    } while (0)

// One world resident on the device (grid, compact copy, palettes, materials, radiance x2) and the
// per-pass buffers that grow on demand (scratch, counters, hit records, direction tables).
struct DeviceWorld {
    int X = 0, Y = 0, Z = 0;
    size_t W = 0;
    int n_slots = 0;
    int precision = 0;
    size_t rad_stride = 16;

    std::vector<int16_t> h_grid;          // the world as the caller set it
    std::vector<uint8_t> h_pal;           // staged palette (lumrad_load_block)
    std::vector<uint8_t> h_pal_dev;       // palette as uploaded
    std::vector<LumRadMaterial> h_mats;
    std::vector<float4> h_mats_dev;       // materials as uploaded
    std::vector<uint8_t> h_cgrid;         // compact ids (uint8 or uint16)
    std::vector<uint32_t> h_cbits;
    std::vector<int> h_cslot;             // palette slot of each compact id (-1: none)
    bool grid_dirty = true;
    bool compact_dirty = true;
    int n_compact = 0;
    bool cgrid_wide = false;
    std::vector<int32_t> id_to_c;         // block id (as uint16) -> compact id, -1 if not assigned
    std::vector<int> reps;                // block id of each compact id (kEmptyRep: no voxels)
    int empty_c = -1;                     // the shared compact id of ids without a palette slot
    static constexpr int kEmptyRep = -100000;

    int16_t* d_grid = nullptr;
    void* d_cgrid = nullptr;
    long long uploads = 0;                // stream operations that changed inputs of a pass (copies)
    uint32_t* d_cbits = nullptr;
    int* d_cslot = nullptr;               // cbits_cap entries
    size_t cbits_cap = 0;
    uint8_t* d_pal = nullptr;
    float4* d_mats = nullptr;
    void* d_rad[2] = {nullptr, nullptr};
    int cur = 0;                          // rad[cur] holds the current volume
    float4* d_scratch = nullptr;
    size_t scratch_cap = 0;
    int* d_probe_count = nullptr;
    size_t count_cap = 0;
    unsigned long long* d_stats = nullptr;
    LumRadHit* d_hits = nullptr;
    size_t hits_cap = 0, hits_n = 0;
    bool hits_recorded = false;
    std::map<int, float4*> d_dirs;
    // blockify: the frame's grid with temporary blocks (empty when not blockified)
    std::vector<int16_t> h_cur;
    // one past the highest palette slot that may hold non-zero voxels on the device (blockify
    // clears the temporary slots up to here); every slot after a palette upload
    int pal_dirty_end = 1 << 30;
    bool skip_host_bits = false;          // inside build_compact(g, false)
    // eviction: the device buffers released, the volume kept here (raw storage, W * rad_stride)
    bool evicted = false;
    std::vector<uint8_t> h_rad_saved;

    int init(int X, int Y, int Z, int slots, int precision, cudaStream_t stream);
    void release();
    // Releases every device buffer of the world, keeping its grid, palette, materials and volume
    // on the host; readmit allocates and uploads them again (then the world is as it was).
    int evict(cudaStream_t stream);
    int readmit(cudaStream_t stream);
    void build_compact() { build_compact(h_grid.data()); }
    // compact ids of grid g (W ids); host_bits: also the occupancy masks from the host palette
    // (blockify computes them on the device from the palette it maps into)
    void build_compact(const int16_t* g, bool host_bits = true);
    // Compact id of block id b, assigning the next free one (and its occupancy mask in h_cbits)
    // if b has none yet; -1 if that needs a wider compact grid (a full rebuild).
    int compact_of(int16_t b, bool* assigned);
    // Device bytes this world holds.
    size_t footprint() const;
    int sync_inputs(cudaStream_t stream);
    int ensure_dirs(int R, cudaStream_t stream, const float4** out);
    int ensure_scratch(size_t groups, int R, cudaStream_t stream);
    int ensure_hits(size_t n);
    int prepare_pass(const short4* d_req, int n, const LumRadPassParams& p, cudaStream_t stream, LaunchArgs* la);
    int fill_pass(const short4* d_req, int n, const LumRadPassParams& p, cudaStream_t stream, WorldPass* out);
};

// A LumRadContext: one world plus its stream, events and request staging.
struct Context {
    static constexpr int kRing = 64;      // kernel-time history
    DeviceWorld world;
    int device = 0;
    int num_sms = 0;
    void* owner = nullptr;                // the server this context is registered with, if any
    std::vector<int16_t> specials;        // queued (x,y,z,w)
    short4* d_req = nullptr;
    size_t req_cap = 0;
    int16_t* h_req_pinned = nullptr;
    size_t h_req_cap = 0;
    struct Resident { short4* ptr = nullptr; int n = 0; };
    std::map<int, Resident> resident;
    unsigned long long* d_queue = nullptr;
    int* d_error = nullptr;
    // rays of one march/finalize round (up to kChunkTasks * 32 rays), or of one march launch over
    // several passes (up to kMultiTasks * 32)
    RayResult* d_ray_res = nullptr;
    RayResult* d_ray_res2 = nullptr;           // the other ray buffer (consecutive passes alternate)
    int* d_ray_blk = nullptr;
    size_t ray_cap = 0;
    int ray_side = 0;
    // a pass call's first march may start in the previous pass's finalize tail (a programmatic
    // dependent launch) when the call right before it on this context was a pass call whose last
    // launch is that finalize: api_calls counts entry points, pass_mark is api_calls after a pass
    // call's launches (-1 after one with hit records), and no upload happened since (world.uploads)
    long long api_calls = 0;
    long long pass_mark = -1;
    long long uploads_mark = -1;

    cudaStream_t stream = nullptr;
    cudaEvent_t ev_req = nullptr;
    // each pass's (or several-pass call's) kernel time: start and end %globaltimer words written by
    // its kernels (LaunchArgs::time_start / time_end), kRing entries; timed[slot]: kernels ran
    unsigned long long* d_ptime = nullptr;
    unsigned long long* h_ptime = nullptr;   // page-locked copy
    bool timed[kRing] = {};
    // the kernel times of the ring's entries, read back once the stream is idle (waits for it)
    int read_times();
    float slot_ms(int slot) const;
    int last_slot = 0;                    // ring entry of the last pass (or several-pass call)
    int last_slot_passes = 1;             // passes that entry covers
    int* h_err = nullptr;                 // pinned copy of the error word
    long long n_passes = 0;
    bool have_pass = false;
    bool req_copy_pending = false;
    LumRadPassStats last{};
    // the last pass ran over a device-built list: its probe count is read back when asked for
    // (d_last_count, copied from the list's length in stream order), in groups of last_size
    bool last_count_on_device = false;
    int* d_last_count = nullptr;
    int last_size = 1, last_R = 0;
    // several-pass calls: one word per probe, bit i set while pass i of a march launch lists it
    // (zero between calls)
    uint32_t* d_pass_mask = nullptr;
    uint32_t* d_pass_mask2 = nullptr;       // the other call's (consecutive calls alternate, as the rays)

    // adaptive time slicing state (internal_render.cpp:1190-1203)
    int frame = 0;
    int magic_size = 1;
    float last_ms = 0.0f;
    // test hooks (lumrad_test_hook): the lean finalize kernel on every pass; a fixed previous-pass
    // time for adaptive slicing (< 0: measured)
    bool test_lean_finalize = false;
    float test_pass_ms = -1.0f;
    // radiance shift applied before each lumrad_update_radiance (Renderer::stored_radiance_shift)
    int shift[3] = {0, 0, 0};
    // voxel models for blockify / map (InternalMeshModel::voxels)
    struct Model { int sx = 0, sy = 0, sz = 0; uint8_t* d_vox = nullptr; };
    std::vector<Model> models;
    unsigned long long* d_map_owner = nullptr;   // one word per voxel of the temporary palette slots
    size_t map_owner_cap = 0;
    // blockify staging, page-locked so the frame's uploads do not block the host: the working
    // grid (W int16), compact grid (W uint16 at most), compact slots (n_slots + 128 ints) and
    // palette copies (n_slots int2); and the copies' device buffer
    uint8_t* h_blk = nullptr;
    int2* d_blk_copies = nullptr;
    // device update-list builder
    ListScratch list{};
    short4* d_specials = nullptr;
    size_t specials_cap = 0;
    int* d_list_count = nullptr;
    int* h_list_count = nullptr;          // pinned
    uint8_t* d_dirty_mask = nullptr;      // 2 W bytes: the dirty-probe dilation's ping-pong masks
    short4* d_edits = nullptr;
    size_t edits_cap = 0;
    // volume read-back: packed RGB on the device, pinned staging on the host
    float* d_rgb = nullptr;
    float* h_rgb = nullptr;
    // gather staging (host-buffer calls)
    float* d_gather = nullptr;
    size_t gather_cap = 0;                // points
    // pass tables of lumrad_radiance_passes*: two pinned halves (one may still be copying) and
    // the device table (stream order keeps a copy behind the launches that read the last one)
    WorldPass* h_ptab[2] = {nullptr, nullptr};
    WorldPass* d_ptab = nullptr;
    int ptab_cap = 0;
    int ptab_half = 0;
    cudaEvent_t ev_ptab[2] = {nullptr, nullptr};

    int ensure_req_capacity(size_t n);
    int ensure_rays(long long n_tasks, long long cap_tasks = kChunkTasks);
    int stage_requests(const int16_t* req, size_t n);
    // One pass over n requests at d_req.  With dev_count, n is the longest the list can be and
    // the pass covers the first *dev_count requests (a list built on the device, not waited for).
    int run_pass(const short4* d_req, int n, const LumRadPassParams* p, const int* dev_count = nullptr);
    // n passes in order (requests reqs[i], ns[i] of them, params ps[i], all validated, size >= 1,
    // no hit records): marches of consecutive passes share launches
    int run_passes(const short4* const* reqs, const int* ns, const LumRadPassParams* ps, int n);
    int ensure_pass_table(int n);
    int check_error();
    int handle_error(int e);              // resets the launch counters after a reported error
    // Builds update_radiance's list on the device into d_req; *n = its length (waited for; with
    // a null n the length stays in d_list_count).  The queued specials are consumed when `consume`
    // is set.
    int build_list_device(bool consume, int* n);
    int ensure_list_scratch();
    int shift_volume(int dx, int dy, int dz);
    void release();
};

Context* as_ctx(LumRadContext c);
// LUMRAD_ESTATE if a server owns the context (its grid and passes are the server's).
int check_unowned(const Context* c);
int check_params(const LumRadPassParams* p);

}  // namespace lumrad
