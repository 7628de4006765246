/*
 * lumrad.h — C ABI of the GB300 radiance-field update (Lum's per-block radiance pass).
 *
 * One context holds one world resident in device memory: the int16 block grid, the 16^3 uint8
 * block palettes, the 256-entry material table and the radiance volume (one probe per block).
 * A pass traces R rays per listed probe through the two-level voxel grid and blends the mean
 * into the probe, exactly as Lum's shaders/radiance.comp does (see "Semantics" below).
 *
 * Conventions (modelled on Lum's C99 API, src/renderer/api/crenderer.h:19-114):
 *   - opaque handles (typedef void*), like `LumRenderer` (crenderer.h:20);
 *   - every call returns a status: 0 = LUMRAD_OK, negative = error; nothing aborts;
 *   - the caller owns every array it passes; arrays are copied before the call returns;
 *   - a context is not thread-safe (Lum's renderer is single-threaded too); different
 *     contexts may be used from different host threads;
 *   - grids and radiance volumes are x-fastest: index = x + X*(y + Y*z)
 *     (table3d, src/renderer/src/internal_render.hpp:136-143).
 *
 * Semantics that differ from the Vulkan pass, by design (each one is a definition where the
 * shader's behaviour is undefined or a data race):
 *   - out-of-range texel fetches return 0 (robust-access semantics);
 *   - a pass reads the previous volume and writes a new one (ping-pong): the shader binds the
 *     same image for read and write (internal_render.cpp:240-241), which races;
 *   - radiance is stored as FP32 (or FP16/BF16) RGB clamped to [0,1] — the clamp of the
 *     A2B10G10R10_UNORM image, without its 10-bit quantisation — or, with
 *     LUMRAD_PRECISION_RGB10A2, in that format itself (round to nearest even);
 *   - world size and rays per probe are runtime values (consts.glsl:1, radiance.comp:37);
 *   - the trilinear radiance fetch uses exact FP32 weights (hardware uses 8-bit weights);
 *   - the subgroup sum is a fixed xor-butterfly order; the coarse march stops after
 *     2*max_dist+2 steps, a bound a finite ray never reaches (a NaN fraction would otherwise
 *     loop forever in the shader).
 */
#ifndef LUMRAD_H
#define LUMRAD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define LUMRAD_OK        0
#define LUMRAD_EINVAL   -1  /* bad argument (null pointer, size out of range, bad id) */
#define LUMRAD_ENOMEM   -2  /* device or host allocation failed, or HBM budget exceeded */
#define LUMRAD_EDEVICE  -3  /* CUDA error; the message is kept by lumrad_last_error() */
#define LUMRAD_ETIMEOUT -4  /* a bounded wait ran out */
#define LUMRAD_ESTATE   -5  /* call not valid in the current state (e.g. no hits recorded) */
#define LUMRAD_ECANCELED -6 /* a server request cancelled before it ran */

/* ---- constants (src/renderer/src/internal_types.hpp:13-25) -------------------------------- */
#define LUMRAD_BLOCK_SIZE          16     /* BLOCK_SIZE */
#define LUMRAD_MATERIALS           256    /* MATERIAL_PALETTE_SIZE */
#define LUMRAD_MAX_BLOCK_SLOTS     4096   /* BLOCK_PALETTE_SIZE_X * BLOCK_PALETTE_SIZE_Y */
#define LUMRAD_SPECIAL_BLOCK       32767  /* SPECIAL_BLOCK */

#define LUMRAD_PRECISION_FP32 0
#define LUMRAD_PRECISION_FP16 1
#define LUMRAD_PRECISION_BF16 2
/* The reference's own volume format, A2B10G10R10_UNORM_PACK32 (radiance.comp:20-21,
 * internal_render.cpp:128-135), 4 B per probe: each channel clamped to [0,1] and stored as the
 * round-to-nearest-even of v * 1023 in FP32 (alpha bits = 3); read back as code / 1023 rounded
 * once to FP32.  With it the drop-in's volume is the reference's, format included. */
#define LUMRAD_PRECISION_RGB10A2 3

typedef void* LumRadContext;

/* World settings; replaces the radiance-relevant part of LumSettings (crenderer.h:28-39). */
typedef struct {
    int world_size[3];      /* blocks per axis, each 1..2047 (LumSettings.world_size) */
    int max_block_types;    /* palette slots kept on the device, 1..4096
                               (LumSettings.static_block_palette_size) */
    int precision;          /* LUMRAD_PRECISION_*: radiance storage type; math is FP32 */
    int device;             /* CUDA device ordinal */
} LumRadSettings;

/* One material; identical layout to LumInternal::Material (internal_types.hpp:26-30),
 * uploaded as the 6x256 R32_SFLOAT image by updateMaterialPalette (load_stuff.cpp:89-111). */
typedef struct {
    float color[4];         /* rgb albedo + alpha (alpha unused by the pass) */
    float emmit;            /* emission */
    float rough;            /* roughness (unused by the pass) */
} LumRadMaterial;

/* Per-pass parameters; replaces radiance.comp's push constants (radiance.comp:30-35),
 * RAYS_PER_PROBE (:37), REACTIVNESS (:28) and max_dist (:193). */
typedef struct {
    int   rays_per_probe;   /* R: multiple of 32, 32..1024 (reference: 64) */
    float max_dist;         /* coarse-march length limit in voxels, (0, 16384] (reference: 128) */
    float blend;            /* temporal blend factor in [0,1] (reference REACTIVNESS: 0.01) */
    int   time_seed;        /* pco.timeSeed: the frame index in the reference */
    int   size;             /* pco.size (magicSize): process requests shift, shift+size, ...;
                               0 = adaptive time slicing as update_radiance does */
    int   shift;            /* pco.sihft: first request, 0 <= shift < size */
    int   record_hits;      /* 1 = keep one LumRadHit per traced ray for lumrad_get_hits */
} LumRadPassParams;

/* One traced ray, recorded when LumRadPassParams.record_hits = 1.  Layout is fixed (24 B). */
typedef struct {
    int32_t  voxel[3];      /* hit: voxel where the refine DDA stopped; miss: 0 */
    int16_t  block;         /* block id read at the last coarse-march position */
    uint8_t  voxel_id;      /* hit: palette value of that voxel (the material index) */
    uint8_t  flags;         /* LUMRAD_HIT_* bits */
    uint16_t coarse_steps;  /* coarse-march iterations (one grid+palette lookup each) */
    uint8_t  refine_steps;  /* refine-DDA iterations, 0..5 */
    uint8_t  coarse_voxel;  /* palette value that ended the coarse march (0 on a miss) */
    float    fraction;      /* hit: refine distance; miss: final coarse distance */
} LumRadHit;

#define LUMRAD_HIT_HIT      0x01  /* CastRay_fast returned true */
#define LUMRAD_HIT_STEP_X   0x02  /* last refine step moved along x (normal = -sign(dir.x)) */
#define LUMRAD_HIT_STEP_Y   0x04
#define LUMRAD_HIT_STEP_Z   0x08
#define LUMRAD_HIT_CAPPED   0x10  /* stopped by the 2*max_dist+2 step bound */

/* Counters of the last pass (exact; identical on every implementation of the pass). */
typedef struct {
    uint64_t probes;        /* probes updated */
    uint64_t rays;          /* rays traced */
    uint64_t steps;         /* grid+palette lookups: coarse steps + refine lookups */
    uint64_t hits;          /* rays that hit a voxel */
    float    gpu_ms;        /* device time of the pass's kernels (timestamps they write) */
} LumRadPassStats;

/* ---- context lifetime (lum_create_instance / lum_init / lum_destroy_instance) ------------- */
int  lumrad_create(const LumRadSettings* settings, LumRadContext* out);
void lumrad_destroy(LumRadContext ctx);
const char* lumrad_last_error(void);          /* last error message of this host thread */
int  lumrad_synchronize(LumRadContext ctx);    /* lum_wait_idle (crenderer.h:108) */

/* ---- inputs ------------------------------------------------------------------------------- */
/* lum_load_world (crenderer.h:72): X*Y*Z int16 ids, x-fastest. */
int  lumrad_load_world(LumRadContext ctx, const int16_t* blocks);
/* lum_set_world_block / lum_get_world_block (crenderer.h:75-76). */
int  lumrad_set_world_block(LumRadContext ctx, int x, int y, int z, int16_t block);
int  lumrad_get_world_block(LumRadContext ctx, int x, int y, int z, int16_t* block);
/* lum_load_block (crenderer.h:78): 4096 voxels as BlockVoxels[x][y][z] (z fastest). */
int  lumrad_load_block(LumRadContext ctx, int16_t block, const uint8_t* voxels);
/* lum_upload_block_palette_to_gpu (crenderer.h:81). */
int  lumrad_upload_block_palette(LumRadContext ctx);
/* 256 materials (Lum's material palette) and lum_upload_material_palette_to_gpu (crenderer.h:82). */
int  lumrad_load_materials(LumRadContext ctx, const LumRadMaterial* materials);
int  lumrad_upload_material_palette(LumRadContext ctx);

/* ---- radiance volume ---------------------------------------------------------------------- */
/* X*Y*Z*3 floats (rgb), x-fastest.  set clamps to [0,1] like a UNORM upload. */
int  lumrad_get_radiance(LumRadContext ctx, float* rgb);
int  lumrad_set_radiance(LumRadContext ctx, const float* rgb);

/* ---- the pass ----------------------------------------------------------------------------- */
/* Update list of LumInternalRenderer::update_radiance (internal_render.cpp:1142-1168):
 * blocks whose clamped 3x3x3 neighbourhood sums to > 0 (scan order), then the queued special
 * requests whose block is not already listed (request order).  Built on the device from the
 * resident grid.  Writes up to `cap` entries of (x,y,z,w) into out; *n = full list length;
 * the special queue is kept. */
int  lumrad_build_update_list(LumRadContext ctx, int16_t* out, int cap, int* n);
/* Queue one special request (specialRadianceUpdates, internal_render.cpp:1164-1168). */
int  lumrad_request_update(LumRadContext ctx, int x, int y, int z);

/* The drop-in for one frame's radiance work in Renderer::submitFrame (renderer.cpp:436-438):
 * shift_radiance by the stored shift, then LumInternalRenderer::update_radiance()
 * (internal_render.cpp:1129-1214): builds the update list on the device (consuming the special
 * requests) and runs one pass.  With params->size == 0 the time slicing adapts as the reference
 * does (magicSize in [1,10], 1.8-2.2 ms target) and time_seed/shift follow the context's frame
 * counter.  The call does not wait for the GPU: the pass is launched for the longest possible list
 * and its kernels read the list's length on the device (only hit records, sized by the length,
 * and adaptive slicing, which reads the previous pass's time, wait for the device). */
int  lumrad_update_radiance(LumRadContext ctx, const LumRadPassParams* params);

/* shift_radiance (internal_render.cpp:1218-1335), applied now: the volume becomes
 * new(p) = old(p + shift) where p + shift lies inside the world, old(p) elsewhere.  A shift
 * with |shift| >= the world's size on any axis leaves the volume unchanged (the reference
 * returns early for x and leaves y/z undefined). */
int  lumrad_shift_radiance(LumRadContext ctx, int dx, int dy, int dz);
/* Renderer::setStoredRadianceShift / getStoredRadianceShift (renderer.cpp:604-609): the shift
 * lumrad_update_radiance applies before each pass (it stays set until changed). */
int  lumrad_set_radiance_shift(LumRadContext ctx, int dx, int dy, int dz);
int  lumrad_get_radiance_shift(LumRadContext ctx, int* shift3);

/* The radiance consumer's 8-probe gather, diffuse.frag:36-90 (sample_radiance(position,
 * normal)): for each point (x, y, z, nx, ny, nz; position in voxel units, normal as given),
 * trilinear weights of the 8 surrounding probes times clamp(dot(dir_to_probe, normal), 0.1, 1),
 * each weight at least 1e-7, probe values clamped to [0, 2] (probes past the volume read 0);
 * rgb = sum(w * probe) / sum(w).  points: n*6 floats, rgb: n*3 floats. */
int  lumrad_gather_radiance(LumRadContext ctx, const float* points, int n, float* rgb);
/* The same on device pointers, enqueued on the context's stream (see lumrad_get_stream). */
int  lumrad_gather_radiance_device(LumRadContext ctx, const float* d_points, int n, float* d_rgb);

/* One pass over an explicit update list of n entries (x,y,z,w) — the body of
 * radiance.comp:361-413 dispatched over n/size workgroups.  int16 coordinates. */
int  lumrad_radiance_pass(LumRadContext ctx, const int16_t* requests, int n,
                          const LumRadPassParams* params);
/* Same with the reference's i8vec4 request encoding (internal_render.hpp:410). */
int  lumrad_radiance_pass_i8(LumRadContext ctx, const int8_t* requests, int n,
                             const LumRadPassParams* params);

/* Resident request lists: upload once, run passes without host traffic. */
int  lumrad_upload_requests(LumRadContext ctx, int slot, const int16_t* requests, int n);
int  lumrad_radiance_pass_resident(LumRadContext ctx, int slot, const LumRadPassParams* params);

/* n passes in order, with results equal bit for bit to n lumrad_radiance_pass calls over the same
 * lists (requests[i] holds counts[i] entries) — successive frames' update_radiance passes
 * (internal_render.cpp:1129-1214) in one call.  The traversal does not read the radiance volume,
 * so the marches of consecutive passes share one launch (their rays wait in device memory) and
 * each pass's shading/blend then runs in order on its predecessor's volume.  Every params[i]
 * needs size >= 1 and record_hits 0.  Afterwards lumrad_get_pass_stats sums probes, rays, steps
 * and hits over the n passes (gpu_ms: the whole call), lumrad_get_kernel_times has one entry for
 * the whole call, and adaptive slicing (size 0 in lumrad_update_radiance) takes the call's time
 * per pass as the last frame's.  Page-locked lists are copied straight from the caller's arrays
 * when the context's stream is idle (the call returns once they are copied). */
int  lumrad_radiance_passes(LumRadContext ctx, const int16_t* const* requests, const int* counts,
                            const LumRadPassParams* params, int n);
/* The same over resident lists (slots[i] for pass i). */
int  lumrad_radiance_passes_resident(LumRadContext ctx, const int* slots, const LumRadPassParams* params,
                                     int n);

/* Hit records of the last pass run with record_hits = 1: n_groups*R entries in dispatch
 * order (entry g*R + r = ray r of workgroup g).  *n = number available. */
int  lumrad_get_hits(LumRadContext ctx, LumRadHit* out, size_t cap, size_t* n);
/* Counters and device time of the last pass (synchronises). */
int  lumrad_get_pass_stats(LumRadContext ctx, LumRadPassStats* out);

/* The CUDA stream (cudaStream_t) every call of this context enqueues on, for callers that
 * order their own work or time passes with their own events on it. */
int  lumrad_get_stream(LumRadContext ctx, void** stream);
/* Device times (ms) of the last min(cap, 64) passes, oldest first; *n = number written.  Each is
 * the span from the start of the pass's first kernel to the end of its last, from %globaltimer
 * timestamps those kernels write (0 for a pass without kernels).  A one-pass call over a resident
 * list (lumrad_radiance_pass_resident) right after another pass call on the context (no other call
 * between them, no upload) starts its march while the previous pass's last kernel finishes, so
 * consecutive spans may overlap.  Synchronises. */
int  lumrad_get_kernel_times(LumRadContext ctx, float* ms, int cap, int* n);

/* ---- producers: voxel models blockified into the world (blockify + map) ---------------------
 * Each frame the reference turns its animated voxel models into temporary palette blocks
 * (Renderer::submitFrame, renderer.cpp:428-455): start_blockify / blockify_mesh / end_blockify
 * (internal_render.cpp:977-1070), exec_copies (:1375-1476) and map_mesh + shaders/map.comp
 * (:1484-1520).  lumrad_blockify does one frame of that: from the loaded (origin) world, every
 * block under a mesh's AABB whose id is below static_blocks gets the next temporary slot
 * (static_blocks, static_blocks+1, ... in mesh order, z-y-x within a mesh) holding a copy of the
 * static block's voxels; slots from static_blocks up are cleared first; then each mesh's non-zero
 * voxels are written into the temporary blocks through the inverse of its transform.  Passes
 * after the call read the blockified world and palette; the origin world is kept, and the next
 * lumrad_blockify (or any change of the origin world or palette) starts from it again.
 * LUMRAD_ENOMEM if the temporary slots would pass max_block_types (the world is left as it was).
 * Meshes are processed in the given order, so a later mesh's voxels win where meshes overlap
 * (the reference sorts them by camera distance, renderer.cpp:407-414).  The reference's map.comp
 * hard-codes 15 static blocks (its default static_block_palette_size); here it is the argument. */
typedef struct {
    float rot[4];           /* rotation quaternion x, y, z, w (glm::quat, MeshTransform.rot) */
    float shift[3];         /* translation in voxels (MeshTransform.shift) */
} LumRadMeshTransform;

/* A voxel model (InternalMeshModel::voxels): sx*sy*sz uint8 material ids, x-fastest (the .vox
 * model layout, load_stuff.cpp:376-385).  *model receives its index. */
int  lumrad_load_model(LumRadContext ctx, const uint8_t* voxels, int sx, int sy, int sz, int* model);
int  lumrad_blockify(LumRadContext ctx, int static_blocks, const int* models,
                     const LumRadMeshTransform* transforms, int n_meshes);
/* The grid the next pass reads (blockified, or the origin world), X*Y*Z int16 x-fastest. */
int  lumrad_get_world(LumRadContext ctx, int16_t* blocks);
/* The device palette as the next pass reads it: max_block_types * 4096 uint8, slot-major,
 * voxel (x,y,z) at x + 16y + 256z. */
int  lumrad_get_block_palette(LumRadContext ctx, uint8_t* voxels);

/* ---- batches: many worlds, one launch ------------------------------------------------------
 * The reference updates one world per frame with one dispatch and time-slices its probes
 * (internal_render.cpp:1190-1206).  A batch updates many resident worlds (contexts on one device,
 * one precision) of any sizes, list lengths and ray counts in one launch of the pass kernels,
 * captured once into a CUDA graph and replayed per run.  While a context belongs to a batch, run
 * its passes through the batch; call lumrad_batch_synchronize before reading its volume. */
typedef void* LumRadBatch;

/* Scheduling of the march queue: a warp claims remaining/(guided_div*warps) tasks at a time,
 * at most max_chunk (0 = the default; at most LUMRAD_MAX_CHUNK, else LUMRAD_EINVAL); march_ctas
 * CTAs per SM (0 = as many as fit).  pass_ms: autotune's timing. */
#define LUMRAD_MAX_CHUNK 4095
typedef struct {
    int   guided_div;
    int   max_chunk;
    int   march_ctas;
    float pass_ms;
} LumRadTuning;

int  lumrad_batch_create(LumRadContext const* worlds, int n_worlds, LumRadBatch* out);
void lumrad_batch_destroy(LumRadBatch batch);
/* World `world`'s update list (x,y,z,w int16) and parameters (size >= 1, no hit records). */
int  lumrad_batch_set_requests(LumRadBatch batch, int world, const int16_t* requests, int n,
                               const LumRadPassParams* params);
/* One pass of every world in one graph replay; time_seed replaces each world's seed. */
int  lumrad_batch_run(LumRadBatch batch, int time_seed);
/* The same pass as one launch per world on each context's stream, waiting for each: the plain
 * one-launch-per-world path, for comparison. */
int  lumrad_batch_run_per_world(LumRadBatch batch, int time_seed);
int  lumrad_batch_synchronize(LumRadBatch batch);
/* Device time of the last lumrad_batch_run (wall time of the last lumrad_batch_run_per_world). */
int  lumrad_batch_last_ms(LumRadBatch batch, float* ms);
int  lumrad_batch_set_tuning(LumRadBatch batch, const LumRadTuning* tuning);
/* Times every candidate setting (repeats runs each, after one warm-up run) on this batch, keeps
 * the fastest and returns it.  Runs real passes; the volumes are restored afterwards. */
int  lumrad_batch_autotune(LumRadBatch batch, int repeats, LumRadTuning* best);
/* Counters of the last run summed over the worlds. */
int  lumrad_batch_stats(LumRadBatch batch, LumRadPassStats* out);

/* ---- serving: relight requests over resident worlds ----------------------------------------
 * The reference relights after edits by re-listing every probe near non-air blocks each frame
 * (update_radiance, internal_render.cpp:1129-1214, after lum_set_world_block edits the grid).
 * A server keeps many worlds (contexts on one device, one precision) resident and serves relight
 * requests: a request edits blocks of one world and then runs one radiance pass over the probes
 * within Chebyshev distance `radius` (settings) of its edits, in x-fastest scan order, with the
 * request's own parameters (size 1; time_seed is the request's).  Requests are continuously
 * batched: each launch takes, in submission order, the oldest due request of every world that
 * has no request on the GPU, while its device bytes fit the HBM budget, and runs them all as one
 * multi-world pass; up to `max_inflight` launches run at once on their own streams, so requests
 * that arrive while others run are admitted as soon as a launch slot and memory are free.
 * A world's requests run one after another in submission order, so each result is the same
 * whether the request runs alone or among others.  Nothing runs until lumrad_server_progress
 * or lumrad_server_run is called.  A context registered with a server belongs to it until the
 * server is destroyed: read its volume with lumrad_server_get_radiance.
 * Under the HBM budget the server evicts idle worlds, least recently used first, when a world
 * or a request does not fit: an evicted world's device buffers are released and its grid,
 * palette, materials and volume kept on the host; it is uploaded again when a request for it
 * comes due.  Results do not depend on evictions.
 * With device_loop = 1 the request loop runs on the GPU instead: lumrad_server_progress only
 * publishes due requests (in submission order) into a ring in page-locked memory and reads the
 * completions the GPU writes back; one CUDA graph with a conditional WHILE node polls the ring
 * (a bounded wait of poll_ms), takes the oldest requests of distinct worlds, applies their
 * edits, derives the dirty probes, runs the pass over all of them and writes completions, and
 * ends when no request came within poll_ms (the host starts it again when one is published).
 * Results are the same as the host loop's.  Limits of that mode: every world stays resident
 * (no eviction; each must fit the budget when added), a world has at most 192 block types
 * (max_block_types), its probes times R/32 are at most 2^20, and R is 32, 64, 128 or 256. */
typedef void* LumRadServer;

typedef struct {
    int    device;
    int    precision;             /* LUMRAD_PRECISION_*; every world must match */
    double hbm_budget_bytes;      /* device bytes for resident worlds plus launches (0 = no limit) */
    int    max_inflight;          /* launches on the GPU at once, 1..8 (0 = 4: on 64 mixed worlds
                                     4 slots served 30% more than 2, 6 no more than 4) */
    int    max_requests_per_launch;   /* 0 = no limit */
    int    radius;                /* dirty-probe radius around each edit, in blocks (0..15) */
    int    device_loop;           /* 1 = the request loop runs on the device (see below) */
    float  poll_ms;               /* device loop: how long it waits for a request before it ends
                                     (the host starts it again on the next request); 0 = 2 ms */
    float  max_queue_ms;          /* queueing bound (0 = none): a request that has waited longer
                                     than this since its arrival when its turn comes is not run; it
                                     completes with LUMRAD_ETIMEOUT and its edits are not applied.
                                     Under overload this sheds load instead of letting every
                                     request's latency grow.  Host loop: checked at admission.
                                     Device loop: the host keeps at most two iterations' requests
                                     published per lane and checks when it publishes. */
} LumRadServerSettings;

typedef struct { int16_t x, y, z, block; } LumRadEdit;

typedef struct {
    long long request;            /* id given by lumrad_server_submit */
    int    world;
    int    status;                /* LUMRAD_OK, LUMRAD_ENOMEM (never fits the budget), LUMRAD_ECANCELED,
                                     LUMRAD_ETIMEOUT (waited past max_queue_ms; not run),
                                     LUMRAD_EDEVICE */
    int    probes;                /* probes relit */
    int    rays_per_probe;
    double arrival_s;             /* server clock (lumrad_server_now) */
    double start_s;               /* its launch was enqueued */
    double done_s;                /* its launch finished on the GPU */
} LumRadCompletion;

typedef struct {
    long long launches;
    long long requests;           /* completed */
    unsigned long long probes, rays;
    double resident_bytes;        /* registered worlds */
    double launch_bytes;          /* fixed per-slot buffers */
    double peak_inflight_bytes;   /* largest admitted request bytes on the GPU at once */
    int    max_requests_in_launch;
    long long evictions;          /* worlds evicted to make room */
    long long readmissions;       /* evicted worlds uploaded again */
    double peak_device_bytes;     /* largest resident + launch buffers + in flight, ever */
    long long shed;               /* requests not run: waited past max_queue_ms */
} LumRadServerStats;

int  lumrad_server_create(const LumRadServerSettings* settings, LumRadServer* out);
void lumrad_server_destroy(LumRadServer server);
/* Registers a loaded context; LUMRAD_ENOMEM if its device bytes do not fit the budget. */
int  lumrad_server_add_world(LumRadServer server, LumRadContext world, int* id);
/* Queues a request (edits in order; the last edit of a block wins).  arrival_s: when it becomes
 * due on the server clock (< 0: now). */
int  lumrad_server_submit(LumRadServer server, int world, const LumRadEdit* edits, int n_edits,
                          const LumRadPassParams* params, double arrival_s, long long* request);
/* Retires finished launches and starts new ones; never waits for the GPU. */
int  lumrad_server_progress(LumRadServer server);
/* Calls lumrad_server_progress until every queued request has completed, or timeout_s passes
 * (LUMRAD_ETIMEOUT). */
int  lumrad_server_run(LumRadServer server, double timeout_s);
/* Cancels a request that has not been launched yet (*cancelled = 1; it completes with
 * LUMRAD_ECANCELED); a running, finished or unknown request is left alone (*cancelled = 0). */
int  lumrad_server_cancel(LumRadServer server, long long request, int* cancelled);
/* Takes up to cap completions (oldest first). */
int  lumrad_server_poll(LumRadServer server, LumRadCompletion* out, int cap, int* n);
double lumrad_server_now(LumRadServer server);
/* The world's volume after its last completed request (waits for its launch), W*3 floats. */
int  lumrad_server_get_radiance(LumRadServer server, int world, float* rgb);
int  lumrad_server_stats(LumRadServer server, LumRadServerStats* out);
/* The same list built on the device of a context, for its world (the request list of a relight
 * request made on the GPU: edit mask, separable dilation, scan-order compaction).  Writes up to
 * cap entries; *n = full length. */
int  lumrad_build_dirty_list(LumRadContext ctx, const LumRadEdit* edits, int n_edits, int radius, int16_t* out,
                             int cap, int* n);
/* Probes within Chebyshev distance radius of the edits of a world of world_size blocks, as
 * (x, y, z, 0) int16 in x-fastest scan order: the request list a relight request runs.  Host
 * only; cap 0 returns the count in *n. */
int  lumrad_dirty_probes(const int* world_size, const LumRadEdit* edits, int n_edits, int radius,
                         int16_t* out, int cap, int* n);

/* ---- no-allocation pass (no counterpart in the reference) -----------------------------------
 * One pass like lumrad_radiance_pass, for callers that may not allocate device memory while
 * they run: engines that reserve their whole device-memory budget up front and forbid later
 * allocations (an allocation can synchronise the device mid-frame), or hosts whose allocator
 * owns the device heap.  The call allocates nothing; the caller passes device pointers to the
 * inputs and the output, and every working buffer lives in one fixed array (about 7 MiB)
 * compiled into this library, which each GPU that loads the library keeps until exit.
 *   world_size  blocks per axis; X*Y*Z <= LUMRAD_NOALLOC_MAX_BLOCKS, else LUMRAD_EINVAL
 *   d_grid      X*Y*Z int16 block ids (x-fastest)
 *   d_palette   n_slots * 4096 uint8 voxels, voxel (x,y,z) at x + 16y + 256z
 *   d_materials 256 * 4 floats: r, g, b, emission
 *   d_requests  n * 4 int16 (x, y, z, w)
 *   d_prev      X*Y*Z * 4 floats (rgb + pad), read;  d_next: same layout, written; the two must
 *               not overlap (LUMRAD_EINVAL)
 *   params      rays_per_probe 32, 64, 128 or 256; size >= 1; record_hits 0
 *   stream      a cudaStream_t (NULL = default stream); the pass is enqueued, not awaited
 * The first call on a device looks up the array's device address and uploads the direction
 * tables into it (a synchronous copy); make that first call before capturing a stream into a
 * CUDA graph.  All calls share the array: calls that overlap on the GPU (different streams, or
 * threads) race and give wrong results.  The call returns before the GPU runs the pass, so it
 * cannot report a device-side failure itself: the kernels record one in an error word in the
 * array, which lumrad_radiance_pass_noalloc_status reads. */
#define LUMRAD_NOALLOC_MAX_BLOCKS (1 << 19)
int  lumrad_radiance_pass_noalloc(const int* world_size, const int16_t* d_grid, const uint8_t* d_palette,
                                  int n_slots, const float* d_materials, const int16_t* d_requests, int n,
                                  const float* d_prev, float* d_next, const LumRadPassParams* params,
                                  void* stream);
/* Waits for `stream`, then reads and clears the no-allocation passes' error word of the current
 * device (allocates nothing): LUMRAD_OK with *device_error = 0 if every such pass since the last
 * status call completed; else LUMRAD_EDEVICE with the word's bits in *device_error (1: the march
 * kernel's scheduler stopped making progress; the outputs of those passes are incomplete). */
int  lumrad_radiance_pass_noalloc_status(void* stream, int* device_error);

/* ---- test hooks (host-side fault injection for this library's own tests) ------------------
 * Not for production use; no counterpart in the reference.  Each hook changes only what the host
 * launches or reads for later calls on ctx; nothing faults or waits on the GPU.
 *   LUMRAD_TEST_LEAN_FINALIZE  value != 0: later passes launch the finalize kernel variant without
 *       the cross-CTA combine even when a probe's subgroups span CTAs (R/32 not dividing 8, e.g.
 *       R = 96).  That kernel stores nothing for such probes and sets its error word, so the next
 *       call that checks it (lumrad_synchronize, lumrad_get_radiance, lumrad_get_pass_stats)
 *       returns LUMRAD_EDEVICE and the context stays usable.  value 0: normal launches again.
 *   LUMRAD_TEST_PASS_MS  value >= 0: lumrad_update_radiance's adaptive slicing (size 0) takes
 *       value as the previous pass's device time in ms instead of measuring it (the reference's
 *       timestamp query, internal_render.cpp:1190-1203); value < 0: measured again. */
#define LUMRAD_TEST_LEAN_FINALIZE 1
#define LUMRAD_TEST_PASS_MS       2
int  lumrad_test_hook(LumRadContext ctx, int hook, double value);

/* Direction table used for rays_per_probe = R (sphericalFibonacci, radiance.comp:293-314):
 * R*3 floats.  cos/sin are evaluated in double and rounded to float. */
int  lumrad_direction_table(int rays_per_probe, float* xyz);

#ifdef __cplusplus
}
#endif

#endif /* LUMRAD_H */
