// lumrad_devloop.h — state of the relight server's device-resident request loop, shared by the
// host runtime (lumrad_serve.cpp) and the loop's kernels (radiance_serve.cu).
#pragma once
#include "lumrad_internal.h"

namespace lumrad {

constexpr int kDevBatch = 64;          // requests (of distinct worlds) per loop iteration
constexpr int kDevMaxWorlds = 1024;    // worlds a device-loop server can hold
constexpr int kDevChunk = 1024;        // cells per chunk of the dirty-list scan
constexpr int kDevDefer = 256;         // requests taken from the ring and held for a later iteration

// One request in the host-written ring (page-locked, read by the loop's admit kernel).
struct DevRequest {
    long long id;
    long long edit_off;                // first edit in the edit arena (wraps at its capacity)
    int world, n_edits, rays, time_seed;
    float max_dist, blend;
    int pad[2];
};

// One completion in the device-written ring (page-locked, read by the host).
struct DevCompletion {
    long long id;
    unsigned long long t_done_ns;      // %globaltimer when the request's pass finished
    int status, probes;
};

// A registered world as the loop sees it (device memory).
struct DevWorld {
    WorldPass pass;                    // the world's pointers, sizes and counters (pass fields filled per batch)
    const float4* dirs[4];             // direction tables for R = 32, 64, 128, 256
    const int16_t* cmap;               // compact id of block id b at cmap[b + 64], -64 <= b < n_cmap - 64
    int n_cmap, empty_c;               // ids outside that range: empty_c (all voxels empty)
    uint8_t* mask;                     // W bytes: probes marked dirty (zero between iterations)
    unsigned long long* stamp;         // W words: (iteration << 32 | edit index) of a block's winning edit
    short4* list;                      // W entries: the dirty list of the world's request in a batch
    void* rad[2];
    int cur, pad;                      // rad[cur] holds the current volume
};

// The loop's state (device memory); ring, arena and control words point into page-locked memory.
struct DevLoop {
    const DevRequest* ring;
    long long ring_cap;
    const long long* head;             // requests published by the host
    volatile long long* tail_host;     // ring entries taken (run or held back; the slots may be reused)
    const LumRadEdit* edits;
    long long edit_cap;
    DevCompletion* done;               // completion ring (ring_cap entries)
    volatile long long* done_head;     // completions written
    const int* stop;                   // set by the host: the loop ends at its next admit
    DevWorld* worlds;
    unsigned long long poll_ns;        // how long admit waits for a request before the loop ends
    long long max_tasks;               // tasks per iteration (the ray buffer)
    int radius;
    int pad0;
    int* error;                        // the pass kernels' error word
    unsigned long long* queue;         // the march kernel's task queue
    int* chunk_count;                  // per chunk of the batch's worlds (capacity: every world's chunks)
    int* chunk_off;
    // requests taken from the ring whose world already had a request in that iteration's batch,
    // oldest first; the next iteration's admit takes from them before the ring
    DevRequest deferred[kDevDefer];
    int n_deferred, pad2;
    // per iteration
    long long tail;                    // next ring entry to admit
    unsigned long long iteration;      // starts at 1
    int n_batch, n_table, idle, pad1;
    long long total_tasks;
    DevRequest batch[kDevBatch];
    long long edit_base[kDevBatch + 1];
    long long chunk_base[kDevBatch + 1];
    int probes[kDevBatch];
    WorldPass table[kDevBatch];
};

struct DevLoopLaunch {
    LaunchArgs pass;                   // the table pass (worlds = the loop's table, sized on the device)
    const WorldPass* table;
    const int* n_table;
    int precision;
    int num_sms;
};

// Enqueues one iteration of the loop on `stream` (captured into the WHILE node's body graph);
// the admit kernel sets `cond` to 0 when it found no request within poll_ns.
cudaError_t capture_devloop_body(DevLoop* d_loop, const DevLoopLaunch& a, cudaGraphConditionalHandle cond,
                                 cudaStream_t stream);

// March + finalize over a table built on the device (args.dev_total / dev_n_worlds set, one round
// of at most args.n_tasks tasks, every world with R/32 dividing 8): the march grid at the
// occupancy limit and a persistent finalize grid.
cudaError_t launch_table_pass(const LaunchArgs& args, int precision, int num_sms, cudaStream_t stream);

// %globaltimer read on the device into *out (page-locked); for the host's clock calibration.
cudaError_t launch_read_globaltimer(unsigned long long* out, cudaStream_t stream);

}  // namespace lumrad
