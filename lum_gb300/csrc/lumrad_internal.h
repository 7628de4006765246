// lumrad_internal.h — device-side argument blocks shared by the host runtime and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "lumrad.h"

namespace lumrad {

// Warps per CTA of the pass kernels.
constexpr int kWarps = 8;
// Warps (one task each) per finalize CTA; a divisor of kWarps, since worlds of a batch start at
// multiples of kWarps tasks
constexpr int kFinWarps = 8;
static_assert(kWarps % kFinWarps == 0, "finalize CTAs must not straddle worlds");
// A task is one 32-ray subgroup of one probe (the unit radiance.comp sums with subgroupAdd).
constexpr int kTaskRays = 32;
// Tasks per march/finalize round: the per-ray buffer between the two kernels holds this many
// tasks' rays (32 B per ray: 268 MB).  Fewer, larger rounds shorten the march kernel's tails
// (measured: 2^18 tasks 13% faster than 2^16 on many small worlds).
constexpr int kChunkTasks = 1 << 18;
// Words of a launch's task queue: [0] next march task, [1] march warps finished; zero between
// launches (the march's last warp resets them)
constexpr int kQueueWords = 2;
// Round size of batches: their task spaces are large, and two rounds of 2^20 tasks beat seven of
// 2^18 by 2% on 256 mixed worlds (fewer queue drains; measured with 8-byte ray results)
constexpr int kBatchRoundTasks = 1 << 20;
// Passes of one march launch over several passes of a context (bits of a pass-mask word)
constexpr int kMultiPasses = 32;
// Tasks of one march launch over several passes of a context (their rays, 32 B each, are kept
// until the passes' finalize launches: 2^19 tasks = 537 MB)
constexpr int kMultiTasks = 1 << 19;

// A marched ray as the march leaves it for the finalize (32 B, two 16-byte words): the coarse
// fraction's bits and the info word (bits 0-15 coarse steps, 16-23 coarse voxel (records only),
// 24 hit, 25 stopped by the step bound), then the ray's origin and direction as the march set them
// up.  The finalize reads the ray back instead of setting it up again: against 8-byte results and
// a second set-up, the march +2.8% (four times the bytes stored) and each finalize -8.5%; the
// 8-pass step -3.0%, a single pass -2.4%, a batch -1.9% (bit-identical).
struct __align__(16) RayResult {
    uint32_t frac, info;
    float ox, oy;
    float oz, dx, dy, dz;
};
static_assert(sizeof(RayResult) == 32, "two 16-byte words");

// One world's pass as the kernels see it (all pointers are device pointers).
//
// The coarse march and the refine DDA only ask "is this block air" and "is this voxel solid",
// so they read a compact copy of the world: every distinct block id is renumbered (0 stays 0)
// into uint8 (or uint16) compact ids, and each compact id has a 4096-bit voxel occupancy mask
// (voxel (x,y,z) -> bit x + 16y + 256z).  Voxel values (material ids) and the original block ids
// are read from the int16 grid and the uint8 palette only where a value is needed.
struct WorldPass {
    int X, Y, Z;                 // blocks per axis
    int cgrid_wide;              // 0: uint8 compact ids, 1: uint16
    const void* cgrid;           // X*Y*Z compact ids, x-fastest
    const uint32_t* cbits;       // 128 words per compact id
    const int* cslot;            // palette slot of each compact id (-1: none), or null: read the grid
    const int16_t* grid;         // X*Y*Z block ids
    const uint8_t* pal;          // n_slots * 4096 voxels, voxel (x,y,z) at x + 16y + 256z
    int n_slots;
    int n_compact;               // compact ids in cbits (0: unknown)
    const float4* mats;          // 256 x (r, g, b, emission)
    const void* prev;            // radiance read
    void* next;                  // radiance written (holds a copy of prev before the pass)
    const short4* req;           // update list (x, y, z, w)
    int n_groups, size, shift;   // workgroup g updates request g*size + shift
    int R;                       // rays per probe, multiple of 32
    float max_dist;
    int max_steps;               // 2*max_dist + 2
    float alpha, one_minus_alpha;
    uint32_t seed;               // time seed
    float inv_dim[3];            // 1/X, 1/Y, 1/Z where that is exact (power of two), else 0
    float inv_nsub;              // 1/(R/32) where exact, else 0
    const float4* dirs;          // R spherical-Fibonacci directions
    LumRadHit* hits;             // per-ray records, or nullptr
    float4* scratch;             // n_groups * R/32 subgroup means (used when R > 32)
    int* probe_count;            // n_groups finished-subgroup counters, zero between launches
    unsigned long long* stats;   // [0] lookups, [1] hits (accumulated)
    long long task_begin;        // first task of this world in the launch
    long long n_tasks;           // n_groups * R/32
};

struct LaunchArgs {
    WorldPass single;            // the one world, passed by value, when `worlds` is null
    const WorldPass* worlds;     // device table of n_worlds worlds (a batch), or null
    int n_worlds;
    int total_warps;             // warps of the march grid (set by the launcher)
    int chunk_begin, chunk_end;  // tasks of this march/finalize round (set by the launcher)
    long long n_tasks;           // tasks of all worlds
    unsigned long long* queue;   // kQueueWords words (see kQueueWords); zero between launches
    int* error;                  // set non-zero if a warp's scheduler stops making progress
    RayResult* ray_res;          // per ray of the round
    int* ray_blk;                // per ray of the round: block id at the last coarse step (records)
    int ray_origin;              // task whose rays start ray_res (the march launch's chunk_begin)
    int round_tasks;             // tasks per march/finalize round (0: kChunkTasks); ray_res holds one round
    int in_cta;                  // table launches: 1 if combines_in_cta holds for every world (the lean
                                 // finalize kernel), 0 for the general one
    int force_lean;              // test hook: the lean finalize kernel even where a probe's subgroups span
                                 // CTAs; the kernel then stores nothing for them and sets error bit 2
    // single-world launches sized for the longest possible list: the list's length on the device
    // (its tasks are (count / size) * R/32; the kernels leave the rest alone), or null
    const int* dev_count;
    // table launches sized on the device (the device-resident serving loop): the tasks of all worlds
    // and the number of worlds in the table, read by the kernels; null otherwise
    const long long* dev_total;
    const int* dev_n_worlds;
    // single-world passes: after marching, the march kernel copies copy_bytes (a multiple of 4) from
    // copy_src to copy_dst (next starts as a copy of prev: probes not in the list keep their value),
    // clears the two counters at clear_stats and copies *count_src to *count_dst; null: nothing.
    // (One launch instead of three copies and a memset before it; after the marching, so that a
    // march launched in the previous pass's finalize tail touches them only once that has ended.)
    const void* copy_src;
    void* copy_dst;
    long long copy_bytes;
    unsigned long long* clear_stats;
    const int* count_src;
    int* count_dst;
    // several passes of one context (launch_passes): one word per probe, bit i set while pass i of
    // the launch lists the probe.  The march kernel sets the bits (after marching); the finalize kernel of pass
    // mask_bit copies every probe whose bit is clear from copy_src (prev) to copy_dst (next) in
    // fin_copy extra CTAs after its fin_ctas task CTAs (no copy launch between the passes), and
    // with mask_clear (the last pass) zeroes the words for the next launch.  Null: not used.
    uint32_t* pass_mask;
    int mask_bit, mask_clear, fin_ctas, fin_copy;
    // the kernel time of a pass (or several-pass call) as two %globaltimer words: the march launch
    // that starts it writes [0] = its start and [1] = 0, each finalize CTA raises [1] to its end;
    // null: not timed.  (Timestamps written by the kernels, not events between the launches, which
    // would keep the next pass's march from starting in the previous finalize's tail.)
    unsigned long long* time_start;
    unsigned long long* time_end;
    // scheduling (0 = the kernel's defaults, 2 and 32): a warp claims remaining / (guided_div *
    // warps) tasks at a time, clamped to [1, max_chunk]; the march grid has march_ctas CTAs per SM
    // (capped by occupancy)
    int guided_div, max_chunk, march_ctas;
};

// Whether every probe of these worlds combines its subgroup means inside one finalize CTA: R/32
// divides kFinWarps and the world's tasks start at a multiple of kFinWarps.
inline bool combines_in_cta(const WorldPass* w, int n) {
    for (int i = 0; i < n; i++) {
        const int nsub = w[i].R / 32;
        if (nsub > 1 && (kFinWarps % nsub != 0 || w[i].task_begin % kFinWarps != 0)) return false;
    }
    return true;
}

// Tunable scheduling of a multi-world launch (see LaunchArgs): batches start from these and
// autotune; servers use them as they are.
struct Tuning {
    int guided_div = 2;
    int max_chunk = 16;
    int march_ctas = 0;
};

// Runs one pass over the worlds of `args` (descriptors already on the device when n_worlds > 1)
// on `stream`: for each round of up to kChunkTasks tasks, the march kernel then the finalize
// kernel.  Returns a CUDA error code.
// dependent: the stream's previous kernel is the previous pass's finalize launch and this pass's
// rays go to the other ray buffer; the first march launch then starts in that launch's tail (its
// pass-start work waits for it to end).  No hit records.
cudaError_t launch_radiance(const LaunchArgs& args, int precision, bool record, int num_sms,
                            cudaStream_t stream, bool dependent = false);

// Several passes of one context (table `args.worlds`, pass i's tasks from worlds[i].task_begin,
// n_tasks <= kMultiTasks in all, n_passes <= kMultiPasses): one march launch over every pass's
// tasks that also marks each pass's probes in `args.pass_mask` (one zeroed word per probe); then,
// pass by pass, the finalize kernel over its tasks, whose extra CTAs copy the probes the pass does
// not list from its prev volume to its next (`vol_bytes` each).  `h_tab` is the host copy of the
// table.  No hit records.
cudaError_t launch_passes(const LaunchArgs& args, const WorldPass* h_tab, int n_passes, size_t vol_bytes,
                          int precision, int num_sms, cudaStream_t stream, bool dependent = false);

// Start of a multi-world pass: copies every world's prev volume into its next volume and clears
// its counters (descriptors already on the device).
// dev_n (optional): the number of worlds in the table, read on the device (n_worlds: its capacity).
cudaError_t launch_prep(const WorldPass* d_worlds, int n_worlds, int precision, cudaStream_t stream,
                        const int* dev_n = nullptr);

// Device scratch of the update-list builder for a world of W blocks: ceil(W/32) flag words,
// ceil(W/256) CTA counts and offsets, and the count of rule-listed blocks.
struct ListScratch {
    uint32_t* bits;
    int* cta_counts;
    int* cta_offsets;
    int* listed;
};
size_t list_scratch_words(long long W);
size_t list_scratch_ctas(long long W);

// update_radiance's list (internal_render.cpp:1142-1168) built on the device from the int16
// grid: rule-listed blocks in scan order, then the specials not already listed, in order.
// out holds W + n_specials entries; *count (device) receives the list length.
cudaError_t launch_update_list(const int16_t* grid, int X, int Y, int Z, const short4* specials, int n_specials,
                               const ListScratch& scratch, short4* out, int* count, cudaStream_t stream);

// Probes within Chebyshev distance `radius` of the edited blocks (edits as (x, y, z, block), all
// inside the world), in scan order, into out (W entries); *count (device) receives the length.
// mask_a and mask_b are W bytes of scratch each.
cudaError_t launch_dirty_list(const short4* edits, int n_edits, int X, int Y, int Z, int radius, uint8_t* mask_a,
                              uint8_t* mask_b, const ListScratch& scratch, short4* out, int* count,
                              cudaStream_t stream);

// shift_radiance (internal_render.cpp:1218-1335) from src into dst: dst(p) = src(p + shift)
// where p + shift is inside the world, src(p) elsewhere.
cudaError_t launch_shift_radiance(const void* src, void* dst, int X, int Y, int Z, int sx, int sy, int sz,
                                  int precision, cudaStream_t stream);

// diffuse.frag's 8-probe gather (sample_radiance(position, normal), :36-90) of n points
// (x, y, z, nx, ny, nz in voxel units) from a radiance volume; out: n x 3 floats.
cudaError_t launch_gather(const void* rad, int X, int Y, int Z, int precision, const float* pts, int n, float* out,
                          cudaStream_t stream);

// The volume rad (W probes, storage `precision`) as W*3 packed floats.
cudaError_t launch_pack_rgb(const void* rad, int precision, long long W, float* out, cudaStream_t stream);

// One mesh of map.comp: column-major inverse transform (float), the dispatch origin in world
// voxels (pco.shift) and the dispatch size in voxels (a multiple of 4 per axis).
struct MapArgs {
    float inv[16];
    int shift[3];
    int dims[3];
};
// exec_copies' static-to-temporary block copies: (src slot, dst slot) pairs.
cudaError_t launch_palette_copies(uint8_t* pal, const int2* copies, int n, cudaStream_t stream);
// map.comp for mesh `mesh` (model voxels x-fastest, mx*my*mz bytes): each write is claimed in
// owner (one 64-bit word per voxel of the palette slots from static_blocks up, zero at the start
// of a frame); launch_map_resolve then writes the winners into those slots.
cudaError_t launch_map(const int16_t* grid, int X, int Y, int Z, int n_slots, int static_blocks, const uint8_t* model,
                       int mx, int my, int mz, const MapArgs& a, int mesh, unsigned long long* owner,
                       cudaStream_t stream);
cudaError_t launch_map_resolve(uint8_t* pal_tmp, const unsigned long long* owner, size_t n, cudaStream_t stream);
// Occupancy masks (128 words per compact id) from the device palette; slot_of[c] = -1: empty.
cudaError_t launch_compact_bits(const uint8_t* pal, const int* slot_of, int n_compact, uint32_t* cbits,
                                cudaStream_t stream);

// One block edit of a served world: worlds[world].grid[index] = block and its compact id.
struct EditRecord {
    int world;                   // index into the launch's world table
    int index;                   // x + X*(y + Y*z)
    int block;                   // new block id (int16 range)
    int compact;                 // its compact id
};

// Writes n edits (each block at most once per launch) into the grids and compact grids of the
// worlds of `d_worlds`.
cudaError_t launch_apply_edits(const WorldPass* d_worlds, const EditRecord* d_edits, int n, cudaStream_t stream);

}  // namespace lumrad
