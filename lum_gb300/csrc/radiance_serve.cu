// radiance_serve.cu — the device-resident request loop of the relight server.
//
// One iteration of the loop, every kernel on one stream and captured once into the body of a
// CUDA graph WHILE node (the loop runs on the device; the host only publishes requests into a
// ring in page-locked memory and reads completions from another):
//
//   admit       one warp polls the ring's head (a bounded wait: it gives up after poll_ns and
//               ends the loop); takes the requests from the tail in order while their worlds
//               are distinct and their tasks fit the iteration's ray buffer; sets the loop's
//               condition
//   edits       per edit of the batch: an atomicMax stamp (the last edit of a block in its
//               request wins) and the byte marks of the probes within `radius` of it
//   apply       the winning edits into the int16 grid and the compact grid
//   count       per 1024-cell chunk of each batch world: the marked probes
//   table       one CTA: a scan of the chunk counts per world and the batch's pass table (task
//               offsets 8-aligned, the lists' lengths, the ping-pong sides, the seeds)
//   list        the marked probes in x-fastest scan order into each world's list; marks cleared
//   prep        next = prev per batch world, counters cleared
//   march/finalize over the table (kernels of radiance_pass.cu, sized by the device's counts)
//   complete    per request: the world's volume flipped, a completion record (status, probes,
//               %globaltimer) written to the host ring, the ring's tail published
//
// Requests of one world run one after another (a batch holds a world at most once), so each
// result equals the same requests served by the host loop or run alone.

#include "radiance_device.cuh"
#include "lumrad_devloop.h"

namespace lumrad {
namespace {

constexpr int kLoopCta = 256;


__device__ __forceinline__ long long load_acquire_sys(const long long* p) {
    long long v;
    asm volatile("ld.acquire.sys.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int load_relaxed_sys(const int* p) {
    int v;
    asm volatile("ld.relaxed.sys.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// entry j of the batch whose prefix range [base[j], base[j+1]) holds i
__device__ __forceinline__ int batch_of(const long long* base, int n, long long i) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// The iteration's batch: requests of distinct worlds, oldest first, from the held-back requests
// and then the ring.  A request whose world already has one in the batch is held back (not a
// reason to stop: the batch goes on with other worlds' requests, as the host loop's launches do),
// and one past the ray buffer's task bound ends the batch.  One warp: ring entries (page-locked
// host memory) are fetched 32 at a time into shared memory; lane 0 forms the batch.
__global__ void admit_kernel(DevLoop* L, cudaGraphConditionalHandle cond) {
    __shared__ unsigned seen[kDevMaxWorlds / 32];
    __shared__ DevRequest s_buf[32];
    const int lane = threadIdx.x;
    for (int i = lane; i < kDevMaxWorlds / 32; i += blockDim.x) seen[i] = 0;
    const long long tail = L->tail;
    const int n_def = L->n_deferred;
    long long head = 0;
    int stop = 0;
    if (lane == 0) {
        head = load_acquire_sys(L->head);
        const unsigned long long t0 = globaltimer_ns();
        stop = load_relaxed_sys(L->stop);
        // a bounded wait for the host's next request (the loop ends when it runs out)
        while (n_def == 0 && head == tail && !stop && globaltimer_ns() - t0 < L->poll_ns) {
            __nanosleep(256);
            head = load_acquire_sys(L->head);
            stop = load_relaxed_sys(L->stop);
        }
    }
    head = __shfl_sync(kFull, head, 0);
    stop = __shfl_sync(kFull, stop, 0);
    if (lane != 0) (void)load_acquire_sys(L->head);   // each lane's ring reads ordered after the host's publish
    __syncwarp();
    int n = 0, m = 0;
    long long tasks = 0, edits = 0, chunks = 0;
    bool full = stop != 0;
    // lane 0: 0 = taken into the batch, 1 = held back (world already in the batch), 2 = batch full
    auto take = [&](const DevRequest& r) -> int {
        const unsigned bit = 1u << (r.world & 31);
        if (seen[r.world >> 5] & bit) return 1;
        if (n == kDevBatch) return 2;
        const DevWorld& w = L->worlds[r.world];
        const long long W = (long long)w.pass.X * w.pass.Y * w.pass.Z;
        const long long side = 2LL * L->radius + 1;
        const long long bound = (min(W, (long long)r.n_edits * side * side * side) * (r.rays >> 5) + 7) / 8 * 8;
        if (n > 0 && tasks + bound > L->max_tasks) return 2;
        seen[r.world >> 5] |= bit;
        L->batch[n] = r;
        tasks += bound;
        edits += r.n_edits;
        chunks += (W + kDevChunk - 1) / kDevChunk;
        n++;
        L->edit_base[n] = edits;
        L->chunk_base[n] = chunks;
        return 0;
    };
    if (lane == 0) {
        L->edit_base[0] = 0;
        L->chunk_base[0] = 0;
        // held-back requests first (compacted in place, order kept)
        for (int i = 0; i < n_def; i++) {
            const DevRequest r = L->deferred[i];
            const int v = full ? 2 : take(r);
            if (v == 2) full = true;
            if (v != 0) L->deferred[m++] = r;
        }
    }
    full = __shfl_sync(kFull, full ? 1 : 0, 0) != 0;
    m = __shfl_sync(kFull, m, 0);
    // then the ring, 32 entries at a time
    long long k = 0;
    while (!full && tail + k < head && m < kDevDefer) {
        const int avail = (int)min(32LL, head - (tail + k));
        if (lane < avail) s_buf[lane] = L->ring[(tail + k + lane) % L->ring_cap];
        __syncwarp();
        if (lane == 0) {
            for (int j = 0; j < avail && m < kDevDefer; j++) {
                const int v = take(s_buf[j]);
                if (v == 2) {
                    full = true;
                    break;
                }
                if (v == 1) L->deferred[m++] = s_buf[j];
                k++;
            }
        }
        full = __shfl_sync(kFull, full ? 1 : 0, 0) != 0;
        m = __shfl_sync(kFull, m, 0);
        k = __shfl_sync(kFull, k, 0);
        __syncwarp();
    }
    if (lane != 0) return;
    L->n_deferred = m;
    L->tail = tail + k;
    L->n_batch = n;
    L->n_table = n;
    L->total_tasks = 0;
    L->idle = (n == 0);
    // the taken ring slots may be reused by the host
    __threadfence_system();
    *L->tail_host = tail + k;
    // go on while there is work; a stop ends the loop at once (held-back requests stay for the
    // next launch)
    cudaGraphSetConditional(cond, (n > 0 || m > 0) && !stop ? 1u : 0u);
}

// per edit: the winning-edit stamp and the dirty marks around it
__global__ void edits_kernel(DevLoop* L) {
    const int n = L->n_batch;
    if (n == 0) return;
    const long long total = L->edit_base[n];
    const unsigned long long it = L->iteration;
    const int r = L->radius;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int j = batch_of(L->edit_base, n, e);
        const DevRequest& q = L->batch[j];
        const long long k = e - L->edit_base[j];
        const LumRadEdit ed = L->edits[(q.edit_off + k) % L->edit_cap];
        const DevWorld& w = L->worlds[q.world];
        const int X = w.pass.X, Y = w.pass.Y, Z = w.pass.Z;
        const long long idx = ed.x + (long long)X * (ed.y + (long long)Y * ed.z);
        atomicMax(w.stamp + idx, (it << 32) | (unsigned long long)k);
        for (int z = max(ed.z - r, 0); z <= min(ed.z + r, Z - 1); z++)
            for (int y = max(ed.y - r, 0); y <= min(ed.y + r, Y - 1); y++)
                for (int x = max(ed.x - r, 0); x <= min(ed.x + r, X - 1); x++)
                    w.mask[x + (long long)X * (y + (long long)Y * z)] = 1;
    }
}

__global__ void apply_kernel(DevLoop* L) {
    const int n = L->n_batch;
    if (n == 0) return;
    const long long total = L->edit_base[n];
    const unsigned long long it = L->iteration;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int j = batch_of(L->edit_base, n, e);
        const DevRequest& q = L->batch[j];
        const long long k = e - L->edit_base[j];
        const LumRadEdit ed = L->edits[(q.edit_off + k) % L->edit_cap];
        const DevWorld& w = L->worlds[q.world];
        const long long idx = ed.x + (long long)w.pass.X * (ed.y + (long long)w.pass.Y * ed.z);
        if (w.stamp[idx] != ((it << 32) | (unsigned long long)k)) continue;   // a later edit of the block wins
        const int b = ed.block;
        const int c = (b >= -64 && b < w.n_cmap - 64) ? (int)w.cmap[b + 64] : w.empty_c;
        const_cast<int16_t*>(w.pass.grid)[idx] = (int16_t)b;
        static_cast<uint8_t*>(const_cast<void*>(w.pass.cgrid))[idx] = (uint8_t)c;
    }
}

// marked probes per chunk of kDevChunk cells (kLoopCta threads x 4 cells)
__global__ void count_kernel(DevLoop* L) {
    __shared__ int s_sum[kLoopCta / 32];
    const int n = L->n_batch;
    if (n == 0) return;
    const long long total = L->chunk_base[n];
    for (long long c = blockIdx.x; c < total; c += gridDim.x) {
        const int j = batch_of(L->chunk_base, n, c);
        const DevWorld& w = L->worlds[L->batch[j].world];
        const long long W = (long long)w.pass.X * w.pass.Y * w.pass.Z;
        const long long cell0 = (c - L->chunk_base[j]) * kDevChunk + 4LL * threadIdx.x;
        int cnt = 0;
        for (int i = 0; i < 4; i++) cnt += (cell0 + i < W && w.mask[cell0 + i]) ? 1 : 0;
        cnt = __reduce_add_sync(kFull, cnt);
        if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = cnt;
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int i = 0; i < kLoopCta / 32; i++) t += s_sum[i];
            L->chunk_count[c] = t;
        }
        __syncthreads();
    }
}

// one CTA: chunk offsets per world, list lengths, and the batch's pass table
__global__ void table_kernel(DevLoop* L) {
    __shared__ long long s_off[kDevBatch + 1];
    const int n = L->n_batch;
    if (n == 0) return;
    // each batch world's chunks scanned by one warp, in order
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int j = warp; j < n; j += blockDim.x / 32) {
        const long long c0 = L->chunk_base[j], c1 = L->chunk_base[j + 1];
        int run = 0;
        for (long long c = c0; c < c1; c += 32) {
            const int v = c + lane < c1 ? L->chunk_count[c + lane] : 0;
            int incl = v;
            for (int d = 1; d < 32; d <<= 1) {
                const int u = __shfl_up_sync(kFull, incl, d);
                if (lane >= d) incl += u;
            }
            if (c + lane < c1) L->chunk_off[c + lane] = run + incl - v;
            run += __shfl_sync(kFull, incl, 31);
        }
        if (lane == 0) L->probes[j] = run;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long begin = 0;
        for (int j = 0; j < n; j++) {
            s_off[j] = begin;
            begin += ((long long)L->probes[j] * (L->batch[j].rays >> 5) + kWarps - 1) / kWarps * kWarps;
        }
        s_off[n] = begin;
        L->total_tasks = begin;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const DevRequest& q = L->batch[j];
        const DevWorld& dw = L->worlds[q.world];
        WorldPass w = dw.pass;
        const int R = q.rays;
        w.prev = dw.rad[dw.cur];
        w.next = dw.rad[1 - dw.cur];
        w.req = dw.list;
        w.n_groups = L->probes[j];
        w.size = 1;
        w.shift = 0;
        w.R = R;
        w.max_dist = q.max_dist;
        w.max_steps = (int)(2.0f * q.max_dist) + 2;
        w.alpha = q.blend;
        w.one_minus_alpha = 1.0f - q.blend;
        w.seed = (uint32_t)q.time_seed;
        w.inv_nsub = R == 32 ? 1.0f : R == 64 ? 0.5f : R == 128 ? 0.25f : 0.125f;
        w.dirs = dw.dirs[R == 32 ? 0 : R == 64 ? 1 : R == 128 ? 2 : 3];
        w.task_begin = s_off[j];
        w.n_tasks = (long long)w.n_groups * (R >> 5);
        L->table[j] = w;
    }
}

// the marked probes into each world's list in scan order; marks cleared
__global__ void list_kernel(DevLoop* L) {
    __shared__ int s_warp[kLoopCta / 32];
    const int n = L->n_batch;
    if (n == 0) return;
    const long long total = L->chunk_base[n];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (long long c = blockIdx.x; c < total; c += gridDim.x) {
        const int j = batch_of(L->chunk_base, n, c);
        const DevWorld& w = L->worlds[L->batch[j].world];
        const int X = w.pass.X, Y = w.pass.Y;
        const long long W = (long long)X * Y * w.pass.Z;
        const long long cell0 = (c - L->chunk_base[j]) * kDevChunk + 4LL * threadIdx.x;
        bool m[4];
        int cnt = 0;
        for (int i = 0; i < 4; i++) {
            m[i] = cell0 + i < W && w.mask[cell0 + i];
            cnt += m[i] ? 1 : 0;
        }
        int incl = cnt;
        for (int d = 1; d < 32; d <<= 1) {
            const int u = __shfl_up_sync(kFull, incl, d);
            if (lane >= d) incl += u;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        int before = 0;
        for (int i = 0; i < warp; i++) before += s_warp[i];
        int pos = L->chunk_off[c] + before + incl - cnt;
        for (int i = 0; i < 4; i++) {
            if (!m[i]) continue;
            const long long cell = cell0 + i;
            const int x = (int)(cell % X), y = (int)((cell / X) % Y), z = (int)(cell / ((long long)X * Y));
            w.list[pos++] = make_short4((short)x, (short)y, (short)z, 0);
            w.mask[cell] = 0;
        }
        __syncthreads();
    }
}

__global__ void complete_kernel(DevLoop* L) {
    const int n = L->n_batch;
    if (threadIdx.x != 0 || n == 0) return;
    const int err = *L->error;
    const unsigned long long t = globaltimer_ns();
    const long long d0 = *L->done_head;
    for (int j = 0; j < n; j++) {
        const DevRequest& q = L->batch[j];
        DevWorld& w = L->worlds[q.world];
        w.cur = 1 - w.cur;
        DevCompletion& c = L->done[(d0 + j) % L->ring_cap];
        c.id = q.id;
        c.status = err ? LUMRAD_EDEVICE : LUMRAD_OK;
        c.probes = L->probes[j];
        c.t_done_ns = t;
    }
    if (err) {   // a stalled scheduler: counters back to zero for the next iteration
        *L->error = 0;
        L->queue[0] = 0;
        L->queue[1] = 0;
    }
    L->iteration++;
    __threadfence_system();
    *L->done_head = d0 + n;
    __threadfence_system();
}

__global__ void read_globaltimer_kernel(unsigned long long* out) {
    *reinterpret_cast<volatile unsigned long long*>(out) = globaltimer_ns();
    __threadfence_system();
}

}  // namespace

cudaError_t launch_read_globaltimer(unsigned long long* out, cudaStream_t stream) {
    read_globaltimer_kernel<<<1, 1, 0, stream>>>(out);
    return cudaGetLastError();
}

cudaError_t capture_devloop_body(DevLoop* d_loop, const DevLoopLaunch& a, cudaGraphConditionalHandle cond,
                                 cudaStream_t stream) {
    const int grid = a.num_sms * 4;
    admit_kernel<<<1, 32, 0, stream>>>(d_loop, cond);
    edits_kernel<<<grid, kLoopCta, 0, stream>>>(d_loop);
    apply_kernel<<<grid, kLoopCta, 0, stream>>>(d_loop);
    count_kernel<<<grid, kLoopCta, 0, stream>>>(d_loop);
    table_kernel<<<1, 1024, 0, stream>>>(d_loop);
    list_kernel<<<grid, kLoopCta, 0, stream>>>(d_loop);
    cudaError_t e = launch_prep(a.table, kDevBatch, a.precision, stream, a.n_table);
    if (e != cudaSuccess) return e;
    if ((e = launch_table_pass(a.pass, a.precision, a.num_sms, stream)) != cudaSuccess) return e;
    complete_kernel<<<1, 32, 0, stream>>>(d_loop);
    return cudaGetLastError();
}

}  // namespace lumrad
