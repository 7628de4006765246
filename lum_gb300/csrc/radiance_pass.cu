// radiance_pass.cu — sm_103a kernels of the per-block radiance update.
//
// Restates shaders/radiance.comp (main :361-413, trace_ray :316-346, CastRay_fast :183-291) as two
// kernels per round of up to kChunkTasks tasks (a task = one 32-ray subgroup of one probe):
//
//   march_kernel     persistent warps take tasks from a queue in guided chunks (large early,
//                    single tasks at the end; through a shared-memory block per CTA when the
//                    launch has few tasks per warp).  A warp sets up a task's 32 rays in lock step
//                    (hash seeds, direction, origin, 1/direction) into a 32-ray ring in shared
//                    memory.  Its lanes march in a flat loop, two coarse steps per iteration; a
//                    lane whose ray ends writes its RayResult (fraction, info, origin, direction)
//                    and takes the next ray in ring order.  The ring is set up again as soon as its rays are handed out, so lanes
//                    never wait for each other.
//   finalize_kernel  one warp per task, eight consecutive tasks per CTA, in lock step: the ray
//                    read back, refine DDA, material, trilinear fetch of the previous radiance,
//                    shading, xor-butterfly sum.  When R/32 divides 8 a probe's subgroups share a
//                    CTA and their means are summed in order from shared memory (a lean
//                    instantiation, 8 CTAs per SM, 6 in the device loop's persistent form, when every
//                    probe of the launch does); otherwise through global scratch and a per-probe
//                    counter.  Lookup and hit counters are summed per CTA.
//
// Several passes of one context (launch_passes): one march launch over all their tasks (the
// traversal does not read the radiance volume), then each pass's finalize in order, each launched
// as a programmatic dependent of the one before (its volume-free work runs in that one's tail).
// The pass start (next = prev, counters cleared) runs inside the launches, not as copies between
// them; a one-pass call right after another pass call starts its march in the previous
// finalize's tail.
//
// Exactness: see radiance_device.cuh.  Memory: both kernels test voxels through the compact
// world (uint8 ids + occupancy bits, L1-resident; staged in shared memory by the march of a launch
// over one world that fits); between the kernels each ray keeps its 32 B RayResult: 268 MB for a
// single pass's round of 2^18 tasks, up to 537 MB for several passes, 1.07 GB for a batch's round
// of 2^20.

#include "radiance_device.cuh"
#include "lumrad_devloop.h"

#include <type_traits>

namespace lumrad {
namespace {

// ---------------------------------------------------------------- march kernel
// A ray is regular when each reciprocal of its direction is at most 2^100 in magnitude: no zero
// component (only an exact cancellation in the set-up gives one, or one of a tiny magnitude).
// Such a ray's march never meets a NaN or an infinity: its positions stay below 2^21 in
// magnitude, its block corners within 32 of them, and its fraction grows by at least 0.5 - 2^-8
// per step.  Hence, for it:
//   (a) GLSL's min/max (y < x ? y : x) equal the hardware's min/max: they differ only on NaN and
//       on the sign of a zero, and the skip's 0.01 floor maps both zeros alike;
//   (b) a position lies outside [0, 16*size) exactly when it lies outside the grid lookup's
//       range (-16, 16*size) or is negative (no position is -0: no origin is, and a sum is -0
//       only if both terms are), so the exit test is the lookup's range test and the sign bits;
//   (c) the 2*max_dist+2 step bound is never reached: the fraction passes max_dist first;
//   (d) the grid lookup can take the block index and the range test from trunc(p/16) in FP32
//       (solid_at_tbp), which the empty-block skip needs anyway.
// A warp whose rays are all regular marches with those forms (fewer compares and selects on the
// integer/compare pipe, the one that limits this kernel); any other warp with the exact forms of
// the general case.  Both give the same bits for a regular ray.
__device__ __forceinline__ bool regular_ray(float ivx, float ivy, float ivz) {
    const float lim = 1.2676506002282294e30f;   // 2^100
    return fabsf(ivx) <= lim && fabsf(ivy) <= lim && fabsf(ivz) <= lim;
}

// STAGE: one CTA of kStageWarps warps per SM, with the launch's compact world (compact grid and
// occupancy masks, every world of the launch the same) copied into shared memory at the start;
// lookups are then 32-bit-addressed shared loads (fewer address instructions, lower latency than
// the L1-resident form: 8% off the demo step's march).  Used where the world fits beside the rays'
// rings and parking space (98 KB of the 227 KB per CTA: a 64x64x16 world of 34 block types takes
// 81 KB, and compact worlds up to ~125 KB fit); other launches (batches, servers, larger worlds,
// hit records) read the world from global memory through L1.
constexpr int kStageWarps = 32;
// Queue defaults (LaunchArgs guided_div / max_chunk = 0): the CTA queue's divisor and the chunk
// cap; the per-warp queue divides by kWarpQueueDiv
constexpr int kQueueDiv = 2;
constexpr int kQueueCap = 32;
static_assert(LUMRAD_MAX_CHUNK < (1 << 12) && kQueueCap <= LUMRAD_MAX_CHUNK, "a chunk's count fits 12 bits");
constexpr int kWarpQueueDiv = 1;
// launches with fewer tasks than this per warp claim through the CTA queue (march_kernel's CTAQ)
constexpr int kCtaQueueTasksPerWarp = 32;
// Rays a warp keeps set up in its shared-memory ring (a multiple of 32, a power of two): each slot
// holds origin + ray index, direction, 1/direction + regular flag; a task (32 rays) is set up
// whenever a ring's worth minus one task has been handed out.  One task: its 32 rays wait in the
// ring while the lanes march the previous 32 (A/B on the demo step, bit-identical: 64-ray rings
// 3.3% slower on a single pass and equal on 8 passes, 128-ray rings 11-12% slower: their shared
// memory costs a CTA per SM).
constexpr int kRingRays = kTaskRays;
static_assert((kRingRays & (kRingRays - 1)) == 0 && kRingRays >= kTaskRays, "ring of whole tasks, a power of two");
constexpr size_t kStageRingBytes = (size_t)kStageWarps * 3 * (kRingRays + kTaskRays) * sizeof(float4);

// Tasks are claimed in two levels.  A CTA takes guided blocks from the launch's queue word
// (remaining / (div * CTAs), clamped to [1, cap * warps per CTA]) into a shared-memory block word
// (start << 32 | length << 20 | next); its warps take guided chunks of that block (its remainder /
// warps per CTA, clamped to [1, cap]) with a shared-memory atomic, and the warp that finds it
// empty fetches the next block under a shared lock.  The global word sees one claim per CTA block
// instead of one per warp chunk (same-address atomics serialise), and warps balance at single
// tasks at the end of a launch.
struct CtaQueue {
    unsigned long long blk;
    int lock, done;
};

// One claim from the CTA's block: start << 12 | count of a guided chunk (its remainder / WPC,
// clamped to [1, cap]; / (2 * WPC) measured 0.4% slower on a single pass, a CTA divisor of 3
// instead of 2 3% slower), or -2 when the block looked empty or ran out.
template <int WPC>
__device__ __forceinline__ long long claim_from_block(int cap, CtaQueue* q) {
    const unsigned long long b = *reinterpret_cast<volatile unsigned long long*>(&q->blk);
    const int next = (int)(b & 0xFFFFFull), len = (int)((b >> 20) & 0xFFFull);
    if (next >= len) return -2;
    const int k = max(1, min(cap, (len - next) / WPC));
    const unsigned long long o = atomicAdd(&q->blk, (unsigned long long)k);
    const int n2 = (int)(o & 0xFFFFFull), l2 = (int)((o >> 20) & 0xFFFull);
    return n2 < l2 ? ((long long)(o >> 32) + n2) << 12 | min(k, l2 - n2) : -2;
}

// The slow path (lane 0 of a warp that found the block empty): fetch the next block under the
// CTA's lock, or claim from a block another warp fetched meanwhile.  Returns a chunk as
// claim_from_block does, or -1 when the launch's tasks are exhausted.  Not inlined: the march loop
// keeps its registers (a call per block, not per chunk).
template <int WPC>
__device__ __noinline__ long long refill_block(const LaunchArgs& la, int n_round, CtaQueue* q) {
    const int div = la.guided_div > 0 ? la.guided_div : kQueueDiv;
    const int cap = la.max_chunk > 0 ? la.max_chunk : kQueueCap;
    const long long ctas = max(1, la.total_warps / WPC);
    for (int it = 0; it < (1 << 22); it++) {
        const long long c = claim_from_block<WPC>(cap, q);
        if (c != -2) return c;
        if (*reinterpret_cast<volatile int*>(&q->done)) return -1;
        if (atomicCAS(&q->lock, 0, 1) == 0) {
            const unsigned long long b = *reinterpret_cast<volatile unsigned long long*>(&q->blk);
            if ((b & 0xFFFFFull) < ((b >> 20) & 0xFFFull)) {   // another warp filled it since
                atomicExch(&q->lock, 0);
                continue;
            }
            const long long rem = (long long)n_round - (long long)*reinterpret_cast<volatile unsigned long long*>(la.queue);
            const long long cta_cap = min(4095LL, (long long)cap * WPC);
            const long long kk = rem / ((long long)div * ctas);
            const long long k = kk < 1 ? 1 : (kk > cta_cap ? cta_cap : kk);
            const unsigned long long start = atomicAdd(la.queue, (unsigned long long)k);
            if ((long long)start >= (long long)n_round) {
                *reinterpret_cast<volatile int*>(&q->done) = 1;
                __threadfence_block();
                atomicExch(&q->lock, 0);
                return -1;
            }
            const long long len = min(k, (long long)n_round - (long long)start);
            const long long own = max(1LL, min((long long)cap, len / (long long)WPC));
            atomicExch(&q->blk, (start << 32) | ((unsigned long long)len << 20) | (unsigned long long)own);
            atomicExch(&q->lock, 0);
            return ((long long)start << 12) | own;
        }
        __nanosleep(64);
    }
    atomicOr(la.error, 1);   // the lock holder never finished (it waits for nothing: cannot happen)
    return -1;
}

template <bool RECORD, bool STAGE = false, bool CTAQ = false>
__global__ void __launch_bounds__(STAGE ? kStageWarps * 32 : kWarps * 32, STAGE ? 1 : 4)
march_kernel(const __grid_constant__ LaunchArgs la) {
    if (la.time_start && blockIdx.x == 0 && threadIdx.x == 0) {   // the pass's kernel-time start
        la.time_start[0] = globaltimer_ns();
        la.time_start[1] = 0;
    }
    if (la.pass_mask) {   // several passes: mark each pass's probes (this call's mask: the previous
                          // call's last finalize clears the other)
        const long long stride = (long long)gridDim.x * blockDim.x;
        for (int i = 0; i < la.n_worlds; i++) {
            const WorldPass& w = la.worlds[i];
            for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < w.n_groups; g += stride) {
                const short4 q = __ldg(w.req + (g * w.size + w.shift));
                if (q.x < 0 || q.y < 0 || q.z < 0 || q.x >= w.X || q.y >= w.Y || q.z >= w.Z) continue;
                atomicOr(la.pass_mask + (q.x + (long long)w.X * (q.y + (long long)w.Y * q.z)), 1u << i);
            }
        }
    }
    float4 (*s_ray)[3][kRingRays];    // set-up rays: origin, direction, (1/direction, regular)
    float4 (*s_park)[3][kTaskRays];   // in-flight ray state while the warp sets up
    const uint8_t* s_cg = nullptr;
    const uint16_t* s_rows = nullptr;
    if constexpr (STAGE) {
        extern __shared__ __align__(16) unsigned char s_dyn[];
        s_ray = reinterpret_cast<float4 (*)[3][kRingRays]>(s_dyn);
        s_park = reinterpret_cast<float4 (*)[3][kTaskRays]>(s_dyn + (size_t)kStageWarps * 3 * kRingRays * sizeof(float4));
        unsigned char* wb = s_dyn + kStageRingBytes;
        const WorldPass& w0 = la.worlds ? la.worlds[0] : la.single;
        const int cg_bytes = w0.X * w0.Y * w0.Z * (w0.cgrid_wide ? 2 : 1);
        const int cg_pad = (cg_bytes + 15) & ~15;
        const int cb_bytes = w0.n_compact * 512;
        const uint8_t* gcg = reinterpret_cast<const uint8_t*>(w0.cgrid);
        for (int i = threadIdx.x; i < cg_bytes / 16; i += blockDim.x)
            reinterpret_cast<uint4*>(wb)[i] = __ldg(reinterpret_cast<const uint4*>(gcg) + i);
        for (int i = (cg_bytes & ~15) + (int)threadIdx.x; i < cg_bytes; i += blockDim.x) wb[i] = __ldg(gcg + i);
        for (int i = threadIdx.x; i < cb_bytes / 16; i += blockDim.x)
            reinterpret_cast<uint4*>(wb + cg_pad)[i] = __ldg(reinterpret_cast<const uint4*>(w0.cbits) + i);
        __syncthreads();
        s_cg = wb;
        s_rows = reinterpret_cast<const uint16_t*>(wb + cg_pad);
    } else {
        __shared__ float4 a_ray[kWarps][3][kRingRays];
        __shared__ float4 a_park[kWarps][3][kTaskRays];
        s_ray = a_ray;
        s_park = a_park;
    }

    __shared__ CtaQueue s_q;
    if (threadIdx.x == 0) {
        s_q.blk = 0;
        s_q.lock = 0;
        s_q.done = 0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    float4* so = s_ray[wib][0];
    float4* sd = s_ray[wib][1];
    float4* si = s_ray[wib][2];
    const unsigned lt_mask = (1u << lane) - 1u;
    int n_round = la.chunk_end - la.chunk_begin;
    if (la.dev_count) {   // a list built on the device: its own length bounds the round
        const long long real = (long long)(__ldcg(la.dev_count) / la.single.size) * (la.single.R >> 5);
        n_round = (int)max(0LL, min((long long)n_round, real - la.chunk_begin));
    }
    if (la.dev_total)     // a table built on the device: its task count bounds the round
        n_round = (int)max(0LL, min((long long)n_round, __ldcg(la.dev_total) - la.chunk_begin));

    // current world (warp-uniform)
    const WorldPass* wp = &la.single;
    MarchView mv{0, 0, 0, 0, nullptr, nullptr};
    float wx = 0.0f, wy = 0.0f, wz = 0.0f, max_dist = 0.0f;
    int max_steps = 0;
    int w_begin = 0, w_end = 0;
    // FIFO ring: ray q of the issue order lives in ring slot q mod kRingRays; `loaded` rays have
    // been set up, `issued` handed out
    int issued = 0, loaded = 0;
    int tb = 0, te = 0;          // grabbed task chunk [tb, te)
    bool exhausted = false;
    int pending = -1;            // grabbed task of another world, waiting for the lanes to drain

    // lane ray state
    int my = -1;                 // round-relative index of the lane's ray, -1 if idle
    float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0, ivx = 0, ivy = 0, ivz = 0, cx = 0, cy = 0, cz = 0, frac = 0;
    int steps = 0;
    bool reg = true;             // the lane's ray is regular (see regular_ray)

    // Tasks are claimed in two levels.  A CTA takes guided blocks from the launch's queue word
    // (remaining / (div * CTAs), clamped to [1, cap * warps per CTA]) into a shared-memory block;
    // its warps take single tasks from that block with a shared-memory atomic, and the warp that
    // finds it empty fetches the next block under a shared lock.  The global word sees one claim
    // per CTA block instead of one per warp chunk, and warps balance at single tasks.
    // Claims: CTAQ, through the CTA's block (claim_from_block, refill_block; launches with few tasks
    // per warp, such as a single pass: the warps balance at single tasks); else straight from the
    // launch's queue word in guided chunks of remaining / (div * warps), clamped to [1, cap]
    // (several passes, batches: large chunks, few claims).  Two instantiations: the CTA queue's code costs the
    // other form's march loop registers (2.5% on an 8-pass launch when only branched around).
    auto next_task = [&]() -> int {
        if (pending >= 0) return pending;
        if (tb >= te) {
            if (exhausted) return -1;
            long long c = 0;
            if (lane == 0) {
                const int cap = la.max_chunk > 0 ? la.max_chunk : kQueueCap;
                if (CTAQ) {
                    constexpr int kWpc = STAGE ? kStageWarps : kWarps;
                    c = claim_from_block<kWpc>(cap, &s_q);
                    if (c == -2) c = refill_block<kWpc>(la, n_round, &s_q);
                } else {
                    const unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(la.queue);
                    const long long kk = ((long long)n_round - (long long)cur) /
                                         ((long long)(la.guided_div > 0 ? la.guided_div : kWarpQueueDiv) * la.total_warps);
                    const long long k = kk < 1 ? 1 : (kk > cap ? cap : kk);
                    const unsigned long long start = atomicAdd(la.queue, (unsigned long long)k);
                    c = (long long)start >= (long long)n_round ? -1 : (long long)(start << 12) | min(k, (long long)n_round - (long long)start);
                }
            }
            c = __shfl_sync(kFull, c, 0);
            if (c < 0) {
                exhausted = true;
                return -1;
            }
            tb = la.chunk_begin + (int)(c >> 12);
            te = tb + (int)(c & 0xFFF);
        }
        return tb;
    };
    auto corner = [&]() {
        cx = dx > 0.0f ? 16.0f : 0.0f;
        cy = dy > 0.0f ? 16.0f : 0.0f;
        cz = dz > 0.0f ? 16.0f : 0.0f;
    };
    // hand the next rays in ring order to the lanes in `need`
    auto assign = [&](unsigned need) {
        const int avail = loaded - issued;
        const int rank = __popc(need & lt_mask);
        if (((need >> lane) & 1u) && rank < avail) {
            const int q = issued + rank;
            const int slot = q & (kRingRays - 1);
            const float4 o4 = so[slot], d4 = sd[slot], i4 = si[slot];
            my = __float_as_int(o4.w);   // the ray's round-relative index, stored with its origin
            ox = o4.x; oy = o4.y; oz = o4.z;
            dx = d4.x; dy = d4.y; dz = d4.z;
            ivx = i4.x; ivy = i4.y; ivz = i4.z;
            reg = i4.w != 0.0f;
            corner();
            frac = 0.0f;
            steps = 0;
        }
        issued += min(avail, __popc(need));
    };
    auto more_tasks = [&]() { return pending < 0 && !(exhausted && tb >= te); };

    // The coarse march (CastRay_fast, radiance.comp:198-244) of the lanes' rays, two coarse steps
    // per iteration (a lane whose ray ends in the first takes no second: the warp's vote and
    // hand-out run once per two steps), until the ring has room for a task while tasks may remain,
    // or no lane has a ray; a FAST loop also ends when a lane takes a ray that is not regular.
    auto march = [&](auto fast_tag, auto wide_tag) {
        constexpr bool FAST = decltype(fast_tag)::value;
        constexpr bool WIDE = decltype(wide_tag)::value;
        const uint8_t* cgp = STAGE ? s_cg : mv.cgrid;
        const uint16_t* rowp = STAGE ? s_rows : reinterpret_cast<const uint16_t*>(mv.cbits);
        while (true) {
            bool fin = false;
#pragma unroll
            for (int u = 0; u < 2; u++) {   // (3 or 4 steps per iteration measured 0.2-0.7% slower)
                // Straight-line: every lane runs the step (an idle lane's stale ray reads only
                // in-range cells and its results are dropped) and the empty-block skip
                // (radiance.comp:215-226) is formed for every lane and selected where the block is
                // air: no divergent branch per step (3% fewer instructions than branching).  The
                // block's low corner (ix/16)*16 with ix = trunc(px) is trunc(px/16)*16, formed in
                // FP32 (exact: px/16 and the product by 16 are exact, |px| < 2^21; a NaN px gives
                // a NaN skip either way).
                const bool act = my >= 0;
                const float f1 = fadd(frac, 0.5f);
                const int st = steps + 1;
                const float px = fadd(ox, fmul(dx, f1));
                const float py = fadd(oy, fmul(dy, f1));
                const float pz = fadd(oz, fmul(dz, f1));
                const int ix = f2i(px), iy = f2i(py), iz = f2i(pz);
                const float tbx = truncf(fmul(px, 0.0625f)), tby = truncf(fmul(py, 0.0625f)), tbz = truncf(fmul(pz, 0.0625f));
                int cid;
                bool in_range = true;
                const bool solid =
                    FAST ? solid_at_tbp<WIDE, STAGE>(cgp, rowp, mv.X, mv.Y, mv.Z, tbx, tby, tbz, ix, iy, iz, cid, in_range)
                         : solid_at_p<WIDE, STAGE>(cgp, rowp, mv.X, mv.Y, mv.Z, ix, iy, iz, cid);
                // tb*16 is exact (tb = trunc(p/16), an integer of at most |p|/16)
                const float bx = fadd_exact_mul(cx, tbx, 16.0f);
                const float by = fadd_exact_mul(cy, tby, 16.0f);
                const float bz = fadd_exact_mul(cz, tbz, 16.0f);
                const float tx = fadd(fmul(bx, ivx), fmul(-px, ivx));
                const float ty = fadd(fmul(by, ivy), fmul(-py, ivy));
                const float tz = fadd(fmul(bz, ivz), fmul(-pz, ivz));
                const float sk = FAST ? fmaxf(fminf(tx, fminf(ty, tz)), 0.01f) : gmax(gmin(tx, gmin(ty, tz)), 0.01f);
                const float f2 = cid == 0 ? fadd(f1, sk) : f1;
                bool out;
                // a regular ray's position is outside [0, 16*size) on an axis exactly when it is
                // outside the lookup's range (-16, 16*size) or negative (no position is -0): one
                // test of the three sign bits beside the lookup's own range test
                if (FAST)
                    out = !in_range || (int)(__float_as_uint(px) | __float_as_uint(py) | __float_as_uint(pz)) < 0 ||
                          f2 >= max_dist;
                else
                    out = px < 0.0f || py < 0.0f || pz < 0.0f || px >= wx || py >= wy || pz >= wz || f2 >= max_dist;
                const bool capped = !FAST && st >= max_steps;
                frac = f2;
                steps = st;
                const bool f = act && (solid || out || capped);
                if (f) {
                    uint32_t info = (uint32_t)st | (solid ? (1u << 24) : (out ? 0u : (1u << 25)));
                    if (RECORD) {
                        int blk;
                        const int v = voxel_value(*wp, ix, iy, iz, blk);
                        if (solid) info |= (uint32_t)v << 16;
                        la.ray_blk[my] = blk;
                    }
                    uint4* rr = reinterpret_cast<uint4*>(la.ray_res + my);   // RayResult
                    __stcg(rr, make_uint4(__float_as_uint(f2), info, __float_as_uint(ox), __float_as_uint(oy)));
                    __stcg(rr + 1, make_uint4(__float_as_uint(oz), __float_as_uint(dx), __float_as_uint(dy),
                                              __float_as_uint(dz)));
                    my = -1;
                    fin = true;
                }
            }
            const unsigned fm = __ballot_sync(kFull, fin);
            if (fm) {
                assign(fm);
                if (!__any_sync(kFull, my >= 0) || (loaded - issued <= kRingRays - kTaskRays && more_tasks())) break;
                if (FAST && !__all_sync(kFull, reg || my < 0)) break;
            }
        }
    };

    while (true) {
        // 1. set up tasks into the ring's free room (32 slots free once their rays are handed out)
        const bool refill = loaded - issued <= kRingRays - kTaskRays && (pending >= 0 || more_tasks());
        if (refill && my >= 0) {   // park: the setup needs the registers
            s_park[wib][0][lane] = make_float4(ox, oy, oz, frac);
            s_park[wib][1][lane] = make_float4(dx, dy, dz, __int_as_float(steps));
            s_park[wib][2][lane] = make_float4(ivx, ivy, ivz, reg ? 1.0f : 0.0f);
        }
        bool loaded_now = false;
        while (refill && loaded - issued <= kRingRays - kTaskRays) {
            const int t = next_task();
            if (t < 0) break;
            if (t < w_begin || t >= w_end) {
                const WorldPass* wq = la.worlds ? la.worlds + world_of(la, t) : &la.single;
                if (t >= (int)(wq->task_begin + wq->n_tasks)) {   // alignment gap between worlds
                    if (pending == t) pending = -1; else tb++;
                    continue;
                }
                // another world: drain this one first, unless it is another pass over the same
                // compact world with the same bound (passes of one context), whose rays march alike
                const bool alike = reinterpret_cast<const uint8_t*>(wq->cgrid) == mv.cgrid &&
                                   wq->max_dist == max_dist;
                if (!alike && (__any_sync(kFull, my >= 0) || loaded > issued)) {
                    if (pending != t) tb++;
                    pending = t;
                    break;
                }
                wp = wq;
                mv = march_view(*wp);
                wx = fmul((float)mv.X, 16.0f); wy = fmul((float)mv.Y, 16.0f); wz = fmul((float)mv.Z, 16.0f);
                max_dist = wp->max_dist;
                max_steps = wp->max_steps;
                w_begin = (int)wp->task_begin;
                w_end = (int)(wp->task_begin + wp->n_tasks);
            }
            if (pending == t) pending = -1; else tb++;
            // lane i builds ray i of the task (subgroup k of workgroup g)
            const int t_local = t - w_begin;
            const int nsub = wp->R >> 5;
            const int g = div_nsub(t_local, nsub);
            float3 o, d;
            setup_ray(*wp, g, (t_local - g * nsub) * kTaskRays + lane, o, d);
            const int slot = (loaded & (kRingRays - 1)) + lane;
            const float4 o4 = make_float4(o.x, o.y, o.z, __int_as_float((t - la.chunk_begin) * kTaskRays + lane));
            const float4 d4 = make_float4(d.x, d.y, d.z, 0.0f);
            so[slot] = o4;
            sd[slot] = d4;
            const float rx = __frcp_rn(d.x), ry = __frcp_rn(d.y), rz = __frcp_rn(d.z);
            si[slot] = make_float4(rx, ry, rz, regular_ray(rx, ry, rz) ? 1.0f : 0.0f);
            loaded += kTaskRays;
            loaded_now = true;
        }
        __syncwarp();
        if (refill && my >= 0) {
            const float4 a = s_park[wib][0][lane], b = s_park[wib][1][lane], c = s_park[wib][2][lane];
            ox = a.x; oy = a.y; oz = a.z; frac = a.w;
            dx = b.x; dy = b.y; dz = b.z; steps = __float_as_int(b.w);
            ivx = c.x; ivy = c.y; ivz = c.z; reg = c.w != 0.0f;
            corner();
        }
        // 2. idle lanes take rays
        assign(__ballot_sync(kFull, my < 0));
        if (!__any_sync(kFull, my >= 0)) {
            // nothing in flight and nothing set up: no task was left (a task of another world
            // would have been set up above, the lanes being drained)
            if ((pending >= 0 || loaded_now) && lane == 0) atomicOr(la.error, 1);
            break;
        }
        // 3. march
        const bool fast = __all_sync(kFull, reg || my < 0);
        if (mv.wide) {
            if (fast) march(std::true_type{}, std::true_type{});
            else march(std::false_type{}, std::true_type{});
        } else {
            if (fast) march(std::true_type{}, std::false_type{});
            else march(std::false_type{}, std::false_type{});
        }
    }


    // The pass's start (see LaunchArgs), after the marching: a launch dependent on the previous
    // pass's finalize marches in that launch's tail and waits here for it to end before touching
    // what that launch reads or writes (the volumes, the counters)
    if (la.copy_dst || la.clear_stats || la.count_dst) {
        grid_dependency_wait();
        const long long stride = (long long)gridDim.x * blockDim.x;
        const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        if (la.copy_dst) {   // next starts as a copy of prev
            const long long n16 = la.copy_bytes >> 4;
            const uint4* s16 = reinterpret_cast<const uint4*>(la.copy_src);
            uint4* d16 = reinterpret_cast<uint4*>(la.copy_dst);
            for (long long i = tid; i < n16; i += stride) d16[i] = __ldcs(s16 + i);
            const long long n4 = la.copy_bytes >> 2;
            for (long long i = n16 * 4 + tid; i < n4; i += stride)
                reinterpret_cast<unsigned*>(la.copy_dst)[i] = reinterpret_cast<const unsigned*>(la.copy_src)[i];
        }
        if (tid < 2 && la.clear_stats) la.clear_stats[tid] = 0;
        if (tid == 0 && la.count_dst) *la.count_dst = __ldcg(la.count_src);
    }

    // the last warp to finish resets the queue for the next launch
    if (lane == 0) {
        const unsigned long long e = atomicAdd(la.queue + 1, 1ull);
        if (e == (unsigned long long)la.total_warps - 1) {
            la.queue[0] = 0;
            la.queue[1] = 0;
        }
    }
}

// ---------------------------------------------------------------- finalize kernel
// IN_CTA: every probe of the launch combines inside one CTA (R/32 divides kFinWarps); the kernel
// then has no global-memory combine, which costs the general kernel 8 registers and spills.  The
// kernel waits on its lookup chain, so occupancy pays: the lean forms run 8 CTAs per SM at 32
// registers (the world-table form: 52 B of spills, the 256-world batch 2.8% faster than at 6 CTAs
// and 40 registers; at 4 CTAs it was slower again: five 4-6% faster, six 1% faster), the
// device loop's persistent form 6 (its spills at 32 registers would be 208 B).
// One 8-task group (one CTA's work) of the finalize kernel.  SINGLE: the launch covers one world
// (a single pass, or one pass of a several-pass call), read from the kernel's parameters, whose
// fields are operands from the constant bank; else the world table's entry for the group through
// a generic pointer, whose fields the compiler keeps in registers.  SINGLE took the lean kernel
// from 40 registers and 24 B of spills to 40 registers and none (the 8-pass step 5.6% faster, a
// single pass 2.8%), and then fits 8 CTAs per SM at 32 registers with 32 B of spills: 1.9% faster
// again on the 8-pass step, 0.9% on a single pass (launch 48.8 against 51.0 us).
template <class Store, bool RECORD, bool IN_CTA, bool SINGLE>
__device__ __forceinline__ void finalize_group(const LaunchArgs& la, int group, float4* s_mean, int* s_count,
                                               unsigned (*s_stat)[2]) {
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    if (threadIdx.x < kFinWarps) {
        s_count[threadIdx.x] = 0;
        s_stat[threadIdx.x][0] = 0;
        s_stat[threadIdx.x][1] = 0;
    }
    __syncthreads();
    const int t0 = la.chunk_begin + group * kFinWarps;   // worlds start at multiples of 8
    const int t = t0 + w;
    const WorldPass* wp = SINGLE ? &la.single : la.worlds ? la.worlds + world_of(la, t0) : &la.single;
    const int t_local = t - (int)wp->task_begin;
    bool valid = t < la.chunk_end && t_local < wp->n_tasks;
    if (la.dev_count)   // a list built on the device (single world): its own length bounds the tasks
        valid = valid && t_local < (__ldcg(la.dev_count) / wp->size) * (wp->R >> 5);
    const int nsub = wp->R >> 5;
    const int g = div_nsub(max(t_local, 0), nsub);
    const int k = t_local - g * nsub;
    // a probe's subgroups share this CTA when R/32 divides 8 (task_begin is a multiple of 8)
    const bool local = nsub > 1 && (kFinWarps % nsub) == 0 && (wp->task_begin % kFinWarps) == 0;
    float3 v = make_float3(0.0f, 0.0f, 0.0f);
    if (valid) {
        const long long idx = (long long)(t - la.ray_origin) * kTaskRays + lane;
        const uint4* rr = reinterpret_cast<const uint4*>(la.ray_res + idx);   // RayResult
        const uint4 r0 = __ldcg(rr), r1 = __ldcg(rr + 1);
        const uint2 res = make_uint2(r0.x, r0.y);
        const int blk = RECORD ? __ldcg(la.ray_blk + idx) : 0;
        const float3 o = make_float3(__uint_as_float(r0.z), __uint_as_float(r0.w), __uint_as_float(r1.x));
        const float3 d = make_float3(__uint_as_float(r1.y), __uint_as_float(r1.z), __uint_as_float(r1.w));
        uint32_t lookups;
        float3 L, u;
        float4 m;
        const MarchView mv = march_view(*wp);
        const float fc = __uint_as_float(res.x);
        const long long gr = (long long)t_local * kTaskRays + lane;
        const bool hit = mv.wide ? finalize_ray<RECORD, true>(*wp, mv, o, d, fc, res.y, blk, gr, lookups, L, u, m)
                                 : finalize_ray<RECORD, false>(*wp, mv, o, d, fc, res.y, blk, gr, lookups, L, u, m);
        grid_dependency_wait();   // from here on the volumes: the previous pass's launch has finished
        if (hit) L = shade_hit<Store>(*wp, u, m);
        L = butterfly_sum(L);
        v = make_float3(fmul(L.x, 0.03125f), fmul(L.y, 0.03125f), fmul(L.z, 0.03125f));   // /32
        // counters: lookups and hits of this task, summed per CTA below
        const unsigned a = __reduce_add_sync(kFull, lookups);
        const unsigned h = __popc(__ballot_sync(kFull, (res.y >> 24) & 1u));
        if (lane == 0) {
            s_stat[w][0] = a;
            s_stat[w][1] = h;
            if (nsub == 1) {
                store_probe<Store>(*wp, g, make_float3(fadd(0.0f, v.x), fadd(0.0f, v.y), fadd(0.0f, v.z)));
            } else if (!local) {
                if (IN_CTA) atomicOr(la.error, 2);   // launched with the wrong kernel: reported, never stored
                else subgroup_done<Store>(*wp, g, k, v);
            } else {
                // the last of the probe's subgroups in this CTA sums their means in subgroup
                // order (radiance.comp:401-407)
                volatile float* vm = reinterpret_cast<volatile float*>(s_mean);
                vm[4 * w] = v.x;
                vm[4 * w + 1] = v.y;
                vm[4 * w + 2] = v.z;
                __threadfence_block();
                if (atomicAdd(&s_count[w - k], 1) == nsub - 1) {
                    __threadfence_block();
                    float3 acc = make_float3(0.0f, 0.0f, 0.0f);
                    for (int j = w - k; j < w - k + nsub; j++) {
                        const float sx = vm[4 * j], sy = vm[4 * j + 1], sz = vm[4 * j + 2];
                        acc = make_float3(fadd(acc.x, sx), fadd(acc.y, sy), fadd(acc.z, sz));
                    }
                    const float fn = (float)nsub;
                    acc = make_float3(fdiv_by(acc.x, fn, wp->inv_nsub), fdiv_by(acc.y, fn, wp->inv_nsub),
                                      fdiv_by(acc.z, fn, wp->inv_nsub));
                    store_probe<Store>(*wp, g, acc);
                }
            }
        }
    }
    // the CTA's counters in one atomic each: one world per CTA; same-address atomics from every
    // task serialise at one L2 slice and held warps at exit (measured 5% of the pass)
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a = 0, h = 0;
        for (int j = 0; j < kFinWarps; j++) {
            a += s_stat[j][0];
            h += s_stat[j][1];
        }
        if (a) atomicAdd(wp->stats, a);
        if (h) atomicAdd(wp->stats + 1, h);
        if (la.time_end) atomicMax(la.time_end + 1, globaltimer_ns());
    }
}

// PERSIST (launches sized on the device): a fixed grid walks the 8-task groups of the device's
// task count; otherwise one CTA per group.
template <class Store, bool RECORD, bool IN_CTA, bool PERSIST = false, bool SINGLE = false>
__global__ void __launch_bounds__(kFinWarps * 32, IN_CTA ? (PERSIST ? 6 : 8) : 4)
finalize_kernel(const __grid_constant__ LaunchArgs la) {
    grid_launch_dependents();   // the next pass's launch may start its volume-free part
    if (la.pass_mask && (int)blockIdx.x >= la.fin_ctas) {   // copy role (see LaunchArgs)
        grid_dependency_wait();
        using T = typename Store::T;
        const T* src = reinterpret_cast<const T*>(la.copy_src);
        T* dst = reinterpret_cast<T*>(la.copy_dst);
        const long long n = la.copy_bytes / (long long)sizeof(T);
        const long long stride = (long long)(gridDim.x - la.fin_ctas) * blockDim.x;
        for (long long p = (long long)(blockIdx.x - la.fin_ctas) * blockDim.x + threadIdx.x; p < n; p += stride) {
            const uint32_t m = la.pass_mask[p];
            if (!((m >> la.mask_bit) & 1u)) dst[p] = __ldcs(src + p);
            if (la.mask_clear && m) la.pass_mask[p] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0 && la.time_end) atomicMax(la.time_end + 1, globaltimer_ns());
        return;
    }
    __shared__ float4 s_mean[kFinWarps];
    __shared__ int s_count[kFinWarps];
    __shared__ unsigned s_stat[kFinWarps][2];
    if (!PERSIST) {
        finalize_group<Store, RECORD, IN_CTA, SINGLE>(la, (int)blockIdx.x, s_mean, s_count, s_stat);
        return;
    }
    const long long total = la.dev_total ? __ldcg(la.dev_total) : (long long)la.chunk_end;
    const int groups = (int)((min(total, (long long)la.chunk_end) - la.chunk_begin + kFinWarps - 1) / kFinWarps);
    for (int g = (int)blockIdx.x; g < groups; g += (int)gridDim.x) {
        finalize_group<Store, RECORD, IN_CTA, false>(la, g, s_mean, s_count, s_stat);
        __syncthreads();   // thread 0 has read the counters before the next group clears them
    }
}

// CTAs of a march launch: the occupancy limit (or ctas_per_sm) on every SM, but no more warps
// than the largest round has tasks (a small world's launch would otherwise start hundreds of
// CTAs that find the queue empty)
int march_grid(bool record, int num_sms, long long round_tasks, int ctas_per_sm = 0) {
    int per_sm = 0;
    const cudaError_t e = record
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_kernel<true>, kWarps * 32, 0)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_kernel<false>, kWarps * 32, 0);
    if (e != cudaSuccess || per_sm < 1) per_sm = 1;
    if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
    const long long needed = (std::max(round_tasks, 1LL) + kWarps - 1) / kWarps;
    return (int)std::min<long long>((long long)num_sms * per_sm, needed);
}

// Whether a launch over these worlds (all with the same compact world) can stage it in shared
// memory, and the dynamic shared bytes it then takes (0 if not).  The kernel's opt-in limit is set
// once per device.
size_t stage_bytes(const WorldPass& w) {
    static int max_optin[64];
    static bool ready[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (!ready[dev]) {
        int v = 0;
        cudaFuncAttributes fa{}, fq{};
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, march_kernel<false, true>) != cudaSuccess ||
            cudaFuncGetAttributes(&fq, march_kernel<false, true, true>) != cudaSuccess)
            v = 0;
        // the kernels' static shared words (the CTA queue's block in one form)
        v = std::max(0, v - (int)std::max(fa.sharedSizeBytes, fq.sharedSizeBytes));
        if (v > 0 && (cudaFuncSetAttribute(march_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, v) !=
                          cudaSuccess ||
                      cudaFuncSetAttribute(march_kernel<false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           v) != cudaSuccess))
            v = 0;
        max_optin[dev] = v;
        ready[dev] = true;
    }
    if (w.n_compact <= 0) return 0;
    const size_t cg = ((size_t)w.X * w.Y * w.Z * (w.cgrid_wide ? 2 : 1) + 15) & ~(size_t)15;
    const size_t bytes = kStageRingBytes + cg + (size_t)w.n_compact * 512;
    return bytes <= (size_t)max_optin[dev] ? bytes : 0;
}

// A launch of `kern`; dependent: as a programmatic dependent of the stream's previous kernel (it
// may start once every CTA of that kernel has called grid_launch_dependents; its reads and writes of
// that kernel's data wait in grid_dependency_wait).
cudaError_t launch_k(void (*kern)(LaunchArgs), int blocks, int threads, size_t smem, cudaStream_t stream, bool dependent,
                     const LaunchArgs& args) {
    if (!dependent) {
        kern<<<blocks, threads, smem, stream>>>(args);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args);
}

// The march launch of a round (no hit records): staged when the world fits shared memory; the
// CTA queue when the round has few tasks per warp.  dependent: see launch_k (the previous kernel
// is the previous pass's finalize; the march writes the other ray buffer).
void launch_march(LaunchArgs args, const WorldPass& w, long long round_tasks, int num_sms, cudaStream_t stream,
                  bool dependent = false) {
    const size_t smem = stage_bytes(w);
    if (smem > 0) {
        const int blocks = (int)std::min<long long>(num_sms, (std::max(round_tasks, 1LL) + kStageWarps - 1) / kStageWarps);
        args.total_warps = blocks * kStageWarps;
        const bool q = round_tasks < (long long)kCtaQueueTasksPerWarp * args.total_warps;
        launch_k(q ? march_kernel<false, true, true> : march_kernel<false, true>, blocks, kStageWarps * 32, smem, stream,
                 dependent, args);
    } else {
        const int blocks = march_grid(false, num_sms, round_tasks, args.march_ctas);
        args.total_warps = blocks * kWarps;
        const bool q = round_tasks < (long long)kCtaQueueTasksPerWarp * args.total_warps;
        launch_k(q ? march_kernel<false, false, true> : march_kernel<false>, blocks, kWarps * 32, 0, stream, dependent,
                 args);
    }
}

// overlap: launched as a programmatic dependent of the stream's previous kernel (a finalize launch
// of the previous pass), whose CTAs let it start early (griddepcontrol.launch_dependents); its
// volume reads and writes wait for that kernel's end (griddepcontrol.wait).  single: every task of
// the launch belongs to args.single.
template <class Store, bool RECORD>
void launch_finalize(const LaunchArgs& args, int n, bool in_cta, cudaStream_t stream, bool overlap, bool single) {
    const int blocks = (n + kFinWarps - 1) / kFinWarps + (args.pass_mask ? args.fin_copy : 0);
    if (blocks <= 0) return;
    auto k = single ? (in_cta ? finalize_kernel<Store, RECORD, true, false, true> : finalize_kernel<Store, RECORD, false, false, true>)
                    : (in_cta ? finalize_kernel<Store, RECORD, true> : finalize_kernel<Store, RECORD, false>);
    launch_k(k, blocks, kFinWarps * 32, 0, stream, overlap, args);
}

template <class Store, bool RECORD>
cudaError_t launch_t(const LaunchArgs& a, int num_sms, cudaStream_t stream, bool dependent) {
    const long long round = a.round_tasks > 0 ? a.round_tasks : kChunkTasks;
    const int blocks = march_grid(RECORD, num_sms, std::min(a.n_tasks, round), a.march_ctas);
    LaunchArgs args = a;
    args.total_warps = blocks * kWarps;
    for (long long c0 = 0; c0 < a.n_tasks; c0 += round) {
        args.chunk_begin = (int)c0;
        args.chunk_end = (int)min(c0 + round, a.n_tasks);
        args.ray_origin = args.chunk_begin;
        const int n = args.chunk_end - args.chunk_begin;
        if (RECORD) march_kernel<RECORD><<<blocks, kWarps * 32, 0, stream>>>(args);
        else launch_march(args, a.single, std::min(a.n_tasks, round), num_sms, stream, dependent && c0 == 0);
        args.copy_dst = nullptr;   // the pass's start: in the first round's march only
        args.clear_stats = nullptr;
        args.count_dst = nullptr;
        args.time_start = nullptr;
        const bool lean = a.force_lean || (a.worlds ? a.in_cta != 0 : combines_in_cta(&a.single, 1));
        launch_finalize<Store, RECORD>(args, n, lean, stream, false, a.worlds == nullptr);
    }
    return cudaGetLastError();
}

template <class Store>
cudaError_t passes_t(const LaunchArgs& a, const WorldPass* h_tab, int n_passes, size_t vol_bytes, int num_sms,
                     cudaStream_t stream, bool dependent) {
    const int blocks = march_grid(false, num_sms, a.n_tasks, a.march_ctas);
    LaunchArgs args = a;
    args.total_warps = blocks * kWarps;
    args.chunk_begin = 0;
    args.chunk_end = (int)a.n_tasks;
    args.ray_origin = 0;
    if (a.n_tasks > 0) {
        launch_march(args, h_tab[0], a.n_tasks, num_sms, stream, dependent);
    } else {   // every pass empty: plain copies
        for (int i = 0; i < n_passes; i++) {
            cudaError_t e = cudaMemcpyAsync(h_tab[i].next, h_tab[i].prev, vol_bytes, cudaMemcpyDeviceToDevice, stream);
            if (e != cudaSuccess) return e;
        }
        if (a.clear_stats) return cudaMemsetAsync(a.clear_stats, 0, 2 * sizeof(unsigned long long), stream);
        return cudaSuccess;
    }
    args.clear_stats = nullptr;
    args.time_start = nullptr;
    const bool in_cta = combines_in_cta(h_tab, n_passes);
    const long long probes = (long long)(vol_bytes / sizeof(typename Store::T));
    const int copy_ctas = (int)std::max<long long>(1, std::min<long long>((probes + 1023) / 1024, 2LL * num_sms));
    for (int i = 0; i < n_passes; i++) {
        const WorldPass& w = h_tab[i];
        args.chunk_begin = (int)w.task_begin;
        args.chunk_end = (int)(w.task_begin + w.n_tasks);
        const int n = args.chunk_end - args.chunk_begin;
        args.copy_src = w.prev;
        args.copy_dst = w.next;
        args.copy_bytes = (long long)vol_bytes;
        args.mask_bit = i;
        args.mask_clear = i == n_passes - 1;
        args.fin_ctas = (n + kFinWarps - 1) / kFinWarps;
        args.fin_copy = copy_ctas;
        args.single = w;   // the launch's tasks are pass i's
        // from the second pass on, the launch overlaps the previous pass's tail: its refine and
        // materials read no volume (the first pass's rays come from the march launch before it)
        launch_finalize<Store, false>(args, n, in_cta, stream, i > 0, true);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_passes(const LaunchArgs& args, const WorldPass* h_tab, int n_passes, size_t vol_bytes,
                          int precision, int num_sms, cudaStream_t stream, bool dependent) {
    if (args.n_tasks > kMultiTasks || n_passes > kMultiPasses || !args.pass_mask) return cudaErrorInvalidValue;
    switch (precision) {
        case LUMRAD_PRECISION_FP16: return passes_t<StoreF16>(args, h_tab, n_passes, vol_bytes, num_sms, stream, dependent);
        case LUMRAD_PRECISION_BF16:
            return passes_t<StoreBF16>(args, h_tab, n_passes, vol_bytes, num_sms, stream, dependent);
        case LUMRAD_PRECISION_RGB10A2:
            return passes_t<StoreRGB10A2>(args, h_tab, n_passes, vol_bytes, num_sms, stream, dependent);
        default: return passes_t<StoreF32>(args, h_tab, n_passes, vol_bytes, num_sms, stream, dependent);
    }
}

cudaError_t launch_table_pass(const LaunchArgs& a, int precision, int num_sms, cudaStream_t stream) {
    const int blocks = march_grid(false, num_sms, a.n_tasks, a.march_ctas);
    LaunchArgs args = a;
    args.total_warps = blocks * kWarps;
    args.chunk_begin = 0;
    args.chunk_end = (int)a.n_tasks;
    args.ray_origin = 0;
    // the CTA queue: the host cannot see the task count, and the device loop's iterations are
    // mostly small (p50 5-8% lower at 2,000-10,000 requests/s than the per-warp queue; 2% less
    // throughput saturated, where the host loop is the faster one anyway)
    march_kernel<false, false, true><<<blocks, kWarps * 32, 0, stream>>>(args);
    const int fin = num_sms * 6;   // the persistent finalize's occupancy (6 CTAs per SM)
    switch (precision) {
        case LUMRAD_PRECISION_FP16: finalize_kernel<StoreF16, false, true, true><<<fin, kFinWarps * 32, 0, stream>>>(args); break;
        case LUMRAD_PRECISION_BF16: finalize_kernel<StoreBF16, false, true, true><<<fin, kFinWarps * 32, 0, stream>>>(args); break;
        case LUMRAD_PRECISION_RGB10A2:
            finalize_kernel<StoreRGB10A2, false, true, true><<<fin, kFinWarps * 32, 0, stream>>>(args);
            break;
        default: finalize_kernel<StoreF32, false, true, true><<<fin, kFinWarps * 32, 0, stream>>>(args);
    }
    return cudaGetLastError();
}

cudaError_t launch_radiance(const LaunchArgs& args, int precision, bool record, int num_sms, cudaStream_t stream,
                            bool dependent) {
    if (args.n_tasks <= 0) {   // no march launch: the pass's start as copies
        cudaError_t e = cudaSuccess;
        if (args.copy_dst && args.copy_bytes > 0)
            e = cudaMemcpyAsync(args.copy_dst, args.copy_src, (size_t)args.copy_bytes, cudaMemcpyDeviceToDevice, stream);
        if (e == cudaSuccess && args.clear_stats)
            e = cudaMemsetAsync(args.clear_stats, 0, 2 * sizeof(unsigned long long), stream);
        if (e == cudaSuccess && args.count_dst)
            e = cudaMemcpyAsync(args.count_dst, args.count_src, sizeof(int), cudaMemcpyDeviceToDevice, stream);
        return e;
    }
    switch (precision) {
        case LUMRAD_PRECISION_FP16:
            return record ? launch_t<StoreF16, true>(args, num_sms, stream, false) : launch_t<StoreF16, false>(args, num_sms, stream, dependent);
        case LUMRAD_PRECISION_BF16:
            return record ? launch_t<StoreBF16, true>(args, num_sms, stream, false) : launch_t<StoreBF16, false>(args, num_sms, stream, dependent);
        case LUMRAD_PRECISION_RGB10A2:
            return record ? launch_t<StoreRGB10A2, true>(args, num_sms, stream, false)
                          : launch_t<StoreRGB10A2, false>(args, num_sms, stream, dependent);
        default:
            return record ? launch_t<StoreF32, true>(args, num_sms, stream, false) : launch_t<StoreF32, false>(args, num_sms, stream, dependent);
    }
}

}  // namespace lumrad

namespace lumrad {
namespace {

// Start of a batched pass: each world's next volume becomes a copy of its previous one (probes
// not in its list keep their value) and its counters are cleared.  blockIdx.y = world.
template <typename V>
__global__ void prep_kernel(const WorldPass* __restrict__ worlds, const int* dev_n) {
    if (dev_n && (int)blockIdx.y >= __ldcg(dev_n)) return;   // a table built on the device
    const WorldPass& w = worlds[blockIdx.y];
    const long long n = (long long)w.X * w.Y * w.Z;
    const V* src = reinterpret_cast<const V*>(w.prev);
    V* dst = reinterpret_cast<V*>(w.next);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
    if (blockIdx.x == 0 && threadIdx.x < 2) w.stats[threadIdx.x] = 0;
}

}  // namespace

cudaError_t launch_prep(const WorldPass* d_worlds, int n_worlds, int precision, cudaStream_t stream, const int* dev_n) {
    if (n_worlds <= 0) return cudaSuccess;
    const dim3 grid(32, n_worlds);
    if (precision == LUMRAD_PRECISION_FP32) prep_kernel<uint4><<<grid, 256, 0, stream>>>(d_worlds, dev_n);
    else if (precision == LUMRAD_PRECISION_RGB10A2) prep_kernel<unsigned><<<grid, 256, 0, stream>>>(d_worlds, dev_n);
    else prep_kernel<uint2><<<grid, 256, 0, stream>>>(d_worlds, dev_n);
    return cudaGetLastError();
}

namespace {

__global__ void apply_edits_kernel(const WorldPass* __restrict__ worlds, const EditRecord* __restrict__ edits, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const EditRecord e = edits[i];
    const WorldPass& w = worlds[e.world];
    const_cast<int16_t*>(w.grid)[e.index] = (int16_t)e.block;
    if (w.cgrid_wide) static_cast<uint16_t*>(const_cast<void*>(w.cgrid))[e.index] = (uint16_t)e.compact;
    else static_cast<uint8_t*>(const_cast<void*>(w.cgrid))[e.index] = (uint8_t)e.compact;
}

}  // namespace

cudaError_t launch_apply_edits(const WorldPass* d_worlds, const EditRecord* d_edits, int n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    apply_edits_kernel<<<(n + 255) / 256, 256, 0, stream>>>(d_worlds, d_edits, n);
    return cudaGetLastError();
}

}  // namespace lumrad

// ================================================================ no-allocation entry point
//
// lumrad_radiance_pass_noalloc runs the same two kernels as a context's pass, but every working
// buffer lives in one fixed array compiled into this library (g_noalloc_scratch below), so the
// call itself never allocates device memory.  It exists for callers that may not allocate while
// they run a frame: engines that reserve their whole device-memory budget at start-up and forbid
// allocation afterwards (an allocation can synchronise the device and stall the frame), and hosts
// whose own allocator owns the device heap.  Such a caller owns the inputs and outputs and passes
// them as device pointers; the array holds the rest: the compact copy of the world, the rays of
// one round, the direction table and the queue.
//
// Limits: worlds of at most LUMRAD_NOALLOC_MAX_BLOCKS blocks, 32/64/128/256 rays per probe (a
// probe's subgroups then combine inside one CTA, so no per-probe scratch is needed), FP32
// radiance, no hit records.  Rounds of kNoAllocRoundTasks tasks.

#include "lumrad_world.h"
#include <mutex>

namespace lumrad {
namespace {

constexpr int kNoAllocMaxBlocks = LUMRAD_NOALLOC_MAX_BLOCKS;
constexpr int kNoAllocRoundTasks = 4096;
constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }
// byte offsets of the parts of the array
constexpr size_t kNaCgrid = 0;                                                        // uint16 per block
constexpr size_t kNaCbits = align256(kNaCgrid + 2 * (size_t)kNoAllocMaxBlocks);      // 512 B per compact id
constexpr size_t kNaRayRes = align256(kNaCbits + (size_t)(LUMRAD_MAX_BLOCK_SLOTS + 2) * 512);
// the direction tables for R = 32, 64, 128, 256 back to back (480 entries), uploaded once per device
constexpr size_t kNaDirs = align256(kNaRayRes + (size_t)kNoAllocRoundTasks * kTaskRays * sizeof(RayResult));
constexpr int kNaDirEntries = 32 + 64 + 128 + 256;
constexpr size_t kNaQueue = align256(kNaDirs + kNaDirEntries * sizeof(float4));
constexpr size_t kNaError = kNaQueue + kQueueWords * sizeof(unsigned long long);
constexpr size_t kNaStats = align256(kNaError + sizeof(int));
constexpr size_t kNaBytes = align256(kNaStats + 2 * sizeof(unsigned long long));
static_assert(kNaBytes <= (8u << 20), "no-allocation scratch must stay under 8 MiB");

}  // namespace
}  // namespace lumrad

// The scratch array: one per GPU that loads this library, held until the process exits.  In host
// code `g_noalloc_scratch` only names the symbol; its device address comes from
// cudaGetSymbolAddress (done once per device, below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[lumrad::kNaBytes];

namespace lumrad {
namespace {

// Compact ids for the no-allocation form: 0 for block id 0 (palette slot 0), 1 + slot for a
// non-zero id with a palette slot, n_slots + 1 (all empty) for any other id.
__global__ void noalloc_compact_grid(const int16_t* __restrict__ grid, int W, int n_slots, uint16_t* __restrict__ cgrid) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < W; i += gridDim.x * blockDim.x) {
        const int b = grid[i];
        const int slot = b < 0 ? b + 64 : b;
        const bool has = b >= -63 && slot < n_slots;
        cgrid[i] = (uint16_t)(b == 0 ? 0 : (has ? slot + 1 : n_slots + 1));
    }
}

// Occupancy words: entry 0 = slot 0, entry 1 + s = slot s, entry n_slots + 1 = empty.
__global__ void noalloc_compact_bits(const uint8_t* __restrict__ pal, int n_slots, uint32_t* __restrict__ bits) {
    const int n_words = (n_slots + 2) * 128;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_words; i += gridDim.x * blockDim.x) {
        const int e = i >> 7, word = i & 127;
        const int slot = e == 0 ? 0 : e - 1;
        uint32_t v = 0;
        if (e <= n_slots) {
            const uint8_t* p = pal + (size_t)slot * 4096 + word * 32;
            for (int b = 0; b < 32; b++) v |= (p[b] != 0 ? 1u : 0u) << b;
        }
        bits[i] = v;
    }
}

struct NoAllocDevice {
    bool ready = false;
    unsigned char* base = nullptr;   // device address of g_noalloc_scratch on this device
    int num_sms = 0;
};
std::mutex g_noalloc_mutex;
NoAllocDevice g_noalloc_dev[64];

// Offset (entries) of the direction table for R rays in the array's table area.
int noalloc_dir_offset(int R) { return R == 32 ? 0 : R == 64 ? 32 : R == 128 ? 96 : 224; }

// The array's device address on the current device, set up on the first call there: the address
// lookup, the SM count and the four direction tables (one synchronous upload, before any pass of
// this device can read them).  Sets *out to null on failure (and returns the status).
int noalloc_device(NoAllocDevice** out) {
    *out = nullptr;
    int dev = 0;
    LUMRAD_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(LUMRAD_EINVAL, "device ordinal beyond 63");
    NoAllocDevice* nd = &g_noalloc_dev[dev];
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!nd->ready) {
        void* addr = nullptr;
        LUMRAD_TRY(cudaGetSymbolAddress(&addr, g_noalloc_scratch));
        LUMRAD_TRY(cudaDeviceGetAttribute(&nd->num_sms, cudaDevAttrMultiProcessorCount, dev));
        float4 tab[kNaDirEntries];
        float xyz[3 * 256];
        for (int R = 32; R <= 256; R *= 2) {
            fibonacci_table(R, xyz);
            for (int i = 0; i < R; i++)
                tab[noalloc_dir_offset(R) + i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
        }
        unsigned char* base = static_cast<unsigned char*>(addr);
        LUMRAD_TRY(cudaMemcpy(base + kNaDirs, tab, sizeof tab, cudaMemcpyHostToDevice));
        nd->base = base;
        nd->ready = true;
    }
    *out = nd;
    return LUMRAD_OK;
}

}  // namespace
}  // namespace lumrad

using namespace lumrad;

extern "C" int lumrad_radiance_pass_noalloc(const int* world_size, const int16_t* d_grid, const uint8_t* d_palette,
                                            int n_slots, const float* d_materials, const int16_t* d_requests, int n,
                                            const float* d_prev, float* d_next, const LumRadPassParams* p,
                                            void* stream_handle) {
    if (!world_size || !d_grid || !d_palette || !d_materials || !d_prev || !d_next || !p || (n > 0 && !d_requests))
        return fail(LUMRAD_EINVAL, "null argument");
    int rc = check_params(p);
    if (rc) return rc;
    if (p->size < 1) return fail(LUMRAD_EINVAL, "size must be >= 1 (no adaptive slicing here)");
    if (p->record_hits) return fail(LUMRAD_EINVAL, "hit records need lumrad_radiance_pass");
    const int R = p->rays_per_probe;
    if (R != 32 && R != 64 && R != 128 && R != 256) return fail(LUMRAD_EINVAL, "rays_per_probe must be 32, 64, 128 or 256");
    for (int i = 0; i < 3; i++)
        if (world_size[i] < 1 || world_size[i] > 2047) return fail(LUMRAD_EINVAL, "world_size must be in [1, 2047] per axis");
    const long long W = (long long)world_size[0] * world_size[1] * world_size[2];
    if (W > kNoAllocMaxBlocks) return fail(LUMRAD_EINVAL, "world larger than LUMRAD_NOALLOC_MAX_BLOCKS blocks");
    {   // the pass reads prev while it writes next: the two volumes must not share bytes
        const uintptr_t a = reinterpret_cast<uintptr_t>(d_prev), b = reinterpret_cast<uintptr_t>(d_next);
        const uintptr_t bytes = (uintptr_t)W * sizeof(float4);
        if (a < b + bytes && b < a + bytes) return fail(LUMRAD_EINVAL, "d_prev and d_next overlap");
    }
    if (n_slots < 1 || n_slots > LUMRAD_MAX_BLOCK_SLOTS) return fail(LUMRAD_EINVAL, "n_slots must be in [1, 4096]");
    if (n < 0) return fail(LUMRAD_EINVAL, "negative request count");
    const long long groups = n / p->size;
    const long long n_tasks = groups * (R / 32);
    if (n_tasks >= (1LL << 31)) return fail(LUMRAD_EINVAL, "pass has too many subgroups (>= 2^31)");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_handle);

    // set-up, once per device (the first call there; make that call before capturing a stream
    // into a graph): the array's device address and the direction tables
    NoAllocDevice* nd = nullptr;
    if ((rc = noalloc_device(&nd))) return rc;
    unsigned char* base = nd->base;
    uint16_t* cgrid = reinterpret_cast<uint16_t*>(base + kNaCgrid);
    uint32_t* cbits = reinterpret_cast<uint32_t*>(base + kNaCbits);
    const float4* dirs = reinterpret_cast<const float4*>(base + kNaDirs) + noalloc_dir_offset(R);
    unsigned long long* queue = reinterpret_cast<unsigned long long*>(base + kNaQueue);
    int* error = reinterpret_cast<int*>(base + kNaError);
    unsigned long long* stats = reinterpret_cast<unsigned long long*>(base + kNaStats);

    // what must start at zero (the error word is kept until lumrad_radiance_pass_noalloc_status
    // reads it), and this call's inputs derived into the array
    LUMRAD_TRY(cudaMemsetAsync(queue, 0, kQueueWords * sizeof(unsigned long long), stream));
    LUMRAD_TRY(cudaMemsetAsync(stats, 0, 2 * sizeof(unsigned long long), stream));
    noalloc_compact_grid<<<256, 256, 0, stream>>>(d_grid, (int)W, n_slots, cgrid);
    noalloc_compact_bits<<<256, 256, 0, stream>>>(d_palette, n_slots, cbits);
    LUMRAD_TRY(cudaGetLastError());
    // probes outside the list keep their value
    LUMRAD_TRY(cudaMemcpyAsync(d_next, d_prev, (size_t)W * sizeof(float4), cudaMemcpyDeviceToDevice, stream));
    if (n_tasks == 0) return LUMRAD_OK;

    LaunchArgs la;
    std::memset(&la, 0, sizeof la);
    WorldPass& w = la.single;
    w.X = world_size[0]; w.Y = world_size[1]; w.Z = world_size[2];
    w.cgrid_wide = 1;
    w.cgrid = cgrid;
    w.cbits = cbits;
    w.grid = d_grid;
    w.pal = d_palette;
    w.n_slots = n_slots;
    w.mats = reinterpret_cast<const float4*>(d_materials);
    w.prev = d_prev;
    w.next = d_next;
    w.req = reinterpret_cast<const short4*>(d_requests);
    w.n_groups = (int)groups;
    w.size = p->size;
    w.shift = p->shift;
    w.R = R;
    w.max_dist = p->max_dist;
    w.max_steps = (int)(2.0f * p->max_dist) + 2;
    w.alpha = p->blend;
    w.one_minus_alpha = 1.0f - p->blend;
    w.seed = (uint32_t)p->time_seed;
    for (int i = 0; i < 3; i++) {
        const int v = world_size[i];
        w.inv_dim[i] = (v & (v - 1)) == 0 ? 1.0f / (float)v : 0.0f;
    }
    w.inv_nsub = 1.0f / (float)(R / 32);
    w.dirs = dirs;
    w.stats = stats;
    w.task_begin = 0;
    w.n_tasks = n_tasks;
    la.n_worlds = 1;
    la.n_tasks = n_tasks;
    la.queue = queue;
    la.error = error;
    la.ray_res = reinterpret_cast<RayResult*>(base + kNaRayRes);
    const int blocks = march_grid(false, nd->num_sms, std::min<long long>(n_tasks, kNoAllocRoundTasks));
    la.total_warps = blocks * kWarps;
    for (long long c0 = 0; c0 < n_tasks; c0 += kNoAllocRoundTasks) {
        la.chunk_begin = (int)c0;
        la.chunk_end = (int)std::min(c0 + (long long)kNoAllocRoundTasks, n_tasks);
        la.ray_origin = la.chunk_begin;
        const int tasks = la.chunk_end - la.chunk_begin;
        if (tasks < kCtaQueueTasksPerWarp * la.total_warps) march_kernel<false, false, true><<<blocks, kWarps * 32, 0, stream>>>(la);
        else march_kernel<false><<<blocks, kWarps * 32, 0, stream>>>(la);
        finalize_kernel<StoreF32, false, true, false, true><<<(tasks + kFinWarps - 1) / kFinWarps, kFinWarps * 32, 0, stream>>>(la);
    }
    LUMRAD_TRY(cudaGetLastError());
    return LUMRAD_OK;
}

extern "C" int lumrad_radiance_pass_noalloc_status(void* stream_handle, int* device_error) {
    if (!device_error) return fail(LUMRAD_EINVAL, "null argument");
    *device_error = 0;
    NoAllocDevice* nd = nullptr;
    if (int rc = noalloc_device(&nd)) return rc;
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_handle);
    int* error = reinterpret_cast<int*>(nd->base + kNaError);
    int word = 0;
    LUMRAD_TRY(cudaMemcpyAsync(&word, error, sizeof(int), cudaMemcpyDeviceToHost, stream));
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    if (word == 0) return LUMRAD_OK;
    LUMRAD_TRY(cudaMemsetAsync(error, 0, sizeof(int), stream));
    LUMRAD_TRY(cudaStreamSynchronize(stream));
    *device_error = word;
    return fail(LUMRAD_EDEVICE, "a no-allocation pass since the last status call did not complete (radiance "
                                "kernel scheduler stopped making progress, code " + std::to_string(word) + ")");
}
