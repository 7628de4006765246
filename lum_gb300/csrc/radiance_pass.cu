// radiance_pass.cu — sm_103a kernels of the per-block radiance update.
//
// Restates shaders/radiance.comp (main :361-413, trace_ray :316-346, CastRay_fast :183-291) as two
// kernels per round of up to kChunkTasks tasks (a task = one 32-ray subgroup of one probe):
//
//   march_kernel     persistent warps take tasks from a queue in guided chunks (large early,
//                    single tasks at the end).  A warp sets up a task's 32 rays in lock step
//                    (hash seeds, direction, origin, 1/direction) into one half of a 64-ray ring in
//                    shared memory and writes them to the round's ray buffer.  Its lanes march
//                    in a flat loop, one coarse step per iteration; a lane whose ray ends writes
//                    (fraction, info) and takes the next ray in ring order.  A half is set up again
//                    as soon as its rays are handed out, so lanes never wait for each other.
//   finalize_kernel  one warp per task, eight consecutive tasks per CTA, in lock step: refine
//                    DDA, material, trilinear fetch of the previous radiance, shading,
//                    xor-butterfly sum.  When R/32 divides 8 a probe's subgroups share a CTA and
//                    their means are summed in order from shared memory; otherwise through
//                    global scratch and a per-probe counter.
//
// Exactness: see radiance_device.cuh.  Memory: both kernels test voxels through the compact
// world (uint8 ids + occupancy bits, L1-resident); the ray buffers between the kernels
// (40 B per ray) stay in L2.

#include "radiance_device.cuh"

namespace lumrad {
namespace {

// ---------------------------------------------------------------- march kernel
template <bool RECORD>
__global__ void __launch_bounds__(kWarps * 32, 4)
march_kernel(const __grid_constant__ LaunchArgs la) {
    constexpr int kRingRays = 2 * kTaskRays;
    __shared__ float4 s_ray[kWarps][3][kRingRays];    // set-up rays: origin, direction, 1/direction
    __shared__ float4 s_park[kWarps][3][kTaskRays];   // in-flight ray state while the warp sets up

    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    float4* so = s_ray[wib][0];
    float4* sd = s_ray[wib][1];
    float4* si = s_ray[wib][2];
    const unsigned lt_mask = (1u << lane) - 1u;
    const int n_round = la.chunk_end - la.chunk_begin;

    // current world (warp-uniform)
    const WorldPass* wp = &la.single;
    MarchView mv{0, 0, 0, 0, nullptr, nullptr};
    float wx = 0.0f, wy = 0.0f, wz = 0.0f, max_dist = 0.0f;
    int max_steps = 0;
    int w_begin = 0, w_end = 0;
    // FIFO ring: ray q of the issue order lives in ring slot q & 63; `loaded` rays have been set
    // up, `issued` handed out; half h holds the task whose first round-relative ray is base[h]
    int issued = 0, loaded = 0, base0 = 0, base1 = 0;
    int tb = 0, te = 0;          // grabbed task chunk [tb, te)
    bool exhausted = false;
    int pending = -1;            // grabbed task of another world, waiting for the lanes to drain

    // lane ray state
    int my = -1;                 // round-relative index of the lane's ray, -1 if idle
    float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0, ivx = 0, ivy = 0, ivz = 0, cx = 0, cy = 0, cz = 0, frac = 0;
    int steps = 0;

    // Tasks are claimed in guided chunks: remaining / (2 * warps), clamped to [1, 16].  (Claiming
    // the next chunk ahead of time hides the atomic's latency but holds work back from idle
    // warps at the end; measured slower.)
    auto next_task = [&]() -> int {
        if (pending >= 0) return pending;
        if (tb >= te) {
            if (exhausted) return -1;
            unsigned long long start = 0, k = 1;
            if (lane == 0) {
                const unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(la.queue);
                const long long rem = (long long)n_round - (long long)cur;
                const long long kk = rem / (2LL * la.total_warps);
                k = (unsigned long long)(kk < 1 ? 1 : (kk > 16 ? 16 : kk));
                start = atomicAdd(la.queue, k);
            }
            start = __shfl_sync(kFull, start, 0);
            k = __shfl_sync(kFull, k, 0);
            if ((long long)start >= (long long)n_round) {
                exhausted = true;
                return -1;
            }
            tb = la.chunk_begin + (int)start;
            te = la.chunk_begin + (int)min((long long)(start + k), (long long)n_round);
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
            my = ((q & kTaskRays) ? base1 : base0) + (q & (kTaskRays - 1));
            const float4 o4 = so[slot], d4 = sd[slot], i4 = si[slot];
            ox = o4.x; oy = o4.y; oz = o4.z;
            dx = d4.x; dy = d4.y; dz = d4.z;
            ivx = i4.x; ivy = i4.y; ivz = i4.z;
            corner();
            frac = 0.0f;
            steps = 0;
        }
        issued += min(avail, __popc(need));
    };
    auto more_tasks = [&]() { return pending < 0 && !(exhausted && tb >= te); };

    while (true) {
        // 1. set up tasks into free ring halves (a half is free once its rays are handed out)
        const bool refill = loaded - issued <= kTaskRays && (pending >= 0 || more_tasks());
        if (refill && my >= 0) {   // park: the setup needs the registers
            s_park[wib][0][lane] = make_float4(ox, oy, oz, frac);
            s_park[wib][1][lane] = make_float4(dx, dy, dz, __int_as_float(steps));
            s_park[wib][2][lane] = make_float4(ivx, ivy, ivz, 0.0f);
        }
        bool loaded_now = false;
        while (refill && loaded - issued <= kTaskRays) {
            const int t = next_task();
            if (t < 0) break;
            if (t < w_begin || t >= w_end) {
                const WorldPass* wq = la.n_worlds == 1 ? &la.single : la.worlds + world_of(la, t);
                if (t >= (int)(wq->task_begin + wq->n_tasks)) {   // alignment gap between worlds
                    if (pending == t) pending = -1; else tb++;
                    continue;
                }
                if (__any_sync(kFull, my >= 0) || loaded > issued) {
                    if (pending != t) tb++;   // another world: drain this one first
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
            const int g = t_local / nsub;
            float3 o, d;
            setup_ray(*wp, g, (t_local - g * nsub) * kTaskRays + lane, o, d);
            const int base = (t - la.chunk_begin) * kTaskRays;
            const int slot = (loaded & kTaskRays) + lane;
            const float4 o4 = make_float4(o.x, o.y, o.z, 0.0f), d4 = make_float4(d.x, d.y, d.z, 0.0f);
            so[slot] = o4;
            sd[slot] = d4;
            si[slot] = make_float4(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z), 0.0f);
            __stcg(la.ray_od + 2 * ((long long)base + lane), o4);
            __stcg(la.ray_od + 2 * ((long long)base + lane) + 1, d4);
            if (loaded & kTaskRays) base1 = base; else base0 = base;
            loaded += kTaskRays;
            loaded_now = true;
        }
        __syncwarp();
        if (refill && my >= 0) {
            const float4 a = s_park[wib][0][lane], b = s_park[wib][1][lane], c = s_park[wib][2][lane];
            ox = a.x; oy = a.y; oz = a.z; frac = a.w;
            dx = b.x; dy = b.y; dz = b.z; steps = __float_as_int(b.w);
            ivx = c.x; ivy = c.y; ivz = c.z;
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
        // 3. march; leave to set up more when a ring half is free and tasks may remain
        while (true) {
            bool fin = false;
            if (my >= 0) {
                frac = fadd(frac, 0.5f);
                steps++;
                const float px = fadd(ox, fmul(dx, frac));
                const float py = fadd(oy, fmul(dy, frac));
                const float pz = fadd(oz, fmul(dz, frac));
                const int ix = f2i(px), iy = f2i(py), iz = f2i(pz);
                int cid;
                const bool solid = solid_at(mv, ix, iy, iz, cid);
                if (cid == 0) {
                    // empty block: skip to its far corner (radiance.comp:215-226)
                    const float bx = fadd((float)((ix / 16) * 16), cx);
                    const float by = fadd((float)((iy / 16) * 16), cy);
                    const float bz = fadd((float)((iz / 16) * 16), cz);
                    const float tx = fadd(fmul(bx, ivx), fmul(-px, ivx));
                    const float ty = fadd(fmul(by, ivy), fmul(-py, ivy));
                    const float tz = fadd(fmul(bz, ivz), fmul(-pz, ivz));
                    frac = fadd(frac, gmax(gmin(tx, gmin(ty, tz)), 0.01f));
                }
                uint32_t info = 0;
                if (solid) {
                    fin = true;
                    info = (uint32_t)steps | (1u << 24);
                } else if (px < 0.0f || py < 0.0f || pz < 0.0f || px >= wx || py >= wy || pz >= wz || frac >= max_dist) {
                    fin = true;
                    info = (uint32_t)steps;
                } else if (steps >= max_steps) {
                    fin = true;
                    info = (uint32_t)steps | (1u << 25);
                }
                if (fin) {
                    if (RECORD) {
                        int blk;
                        const int v = voxel_value(*wp, ix, iy, iz, blk);
                        if (solid) info |= (uint32_t)v << 16;
                        la.ray_blk[my] = blk;
                    }
                    __stcg(la.ray_res + my, make_uint2(__float_as_uint(frac), info));
                    my = -1;
                }
            }
            const unsigned fm = __ballot_sync(kFull, fin);
            if (fm) {
                assign(fm);
                if (!__any_sync(kFull, my >= 0) || (loaded - issued <= kTaskRays && more_tasks())) break;
            }
        }
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
template <class Store, bool RECORD>
__global__ void __launch_bounds__(kWarps * 32, 4)
finalize_kernel(const __grid_constant__ LaunchArgs la) {
    __shared__ float4 s_mean[kWarps];
    __shared__ int s_count[kWarps];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    if (threadIdx.x < kWarps) s_count[threadIdx.x] = 0;
    __syncthreads();
    const int t0 = la.chunk_begin + (int)blockIdx.x * kWarps;   // worlds start at multiples of 8
    const int t = t0 + w;
    const WorldPass* wp = la.n_worlds == 1 ? &la.single : la.worlds + world_of(la, t0);
    const int t_local = t - (int)wp->task_begin;
    const bool valid = t < la.chunk_end && t_local < wp->n_tasks;
    const int nsub = wp->R >> 5;
    const int g = t_local / nsub;
    const int k = t_local - g * nsub;
    // a probe's subgroups share this CTA when R/32 divides 8 (task_begin is a multiple of 8)
    const bool local = nsub > 1 && (kWarps % nsub) == 0 && (wp->task_begin % kWarps) == 0;
    float3 v = make_float3(0.0f, 0.0f, 0.0f);
    if (valid) {
        const long long idx = (long long)(t - la.chunk_begin) * kTaskRays + lane;
        const float4 o4 = __ldcg(la.ray_od + 2 * idx), d4 = __ldcg(la.ray_od + 2 * idx + 1);
        const uint2 res = __ldcg(la.ray_res + idx);
        const int blk = RECORD ? __ldcg(la.ray_blk + idx) : 0;
        uint32_t lookups;
        float3 L = finalize_ray<Store, RECORD>(*wp, march_view(*wp), make_float3(o4.x, o4.y, o4.z),
                                               make_float3(d4.x, d4.y, d4.z), __uint_as_float(res.x), res.y, blk,
                                               (long long)t_local * kTaskRays + lane, lookups);
        L = butterfly_sum(L);
        v = make_float3(fmul(L.x, 0.03125f), fmul(L.y, 0.03125f), fmul(L.z, 0.03125f));   // /32
        // counters: lookups and hits of this task
        unsigned a = lookups, h = (res.y >> 24) & 1u;
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) {
            a += __shfl_xor_sync(kFull, a, m);
            h += __shfl_xor_sync(kFull, h, m);
        }
        if (lane == 0) {
            atomicAdd(wp->stats, (unsigned long long)a);
            atomicAdd(wp->stats + 1, (unsigned long long)h);
            if (!local) {
                subgroup_done<Store>(*wp, g, k, v);
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
}

int march_grid(bool record, int num_sms) {
    int per_sm = 0;
    const cudaError_t e = record
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_kernel<true>, kWarps * 32, 0)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_kernel<false>, kWarps * 32, 0);
    if (e != cudaSuccess || per_sm < 1) per_sm = 1;
    return num_sms * per_sm;
}

template <class Store, bool RECORD>
cudaError_t launch_t(const LaunchArgs& a, int num_sms, cudaStream_t stream) {
    const int blocks = march_grid(RECORD, num_sms);
    LaunchArgs args = a;
    args.total_warps = blocks * kWarps;
    for (long long c0 = 0; c0 < a.n_tasks; c0 += kChunkTasks) {
        args.chunk_begin = (int)c0;
        args.chunk_end = (int)min(c0 + (long long)kChunkTasks, a.n_tasks);
        const int n = args.chunk_end - args.chunk_begin;
        march_kernel<RECORD><<<blocks, kWarps * 32, 0, stream>>>(args);
        finalize_kernel<Store, RECORD><<<(n + kWarps - 1) / kWarps, kWarps * 32, 0, stream>>>(args);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_radiance(const LaunchArgs& args, int precision, bool record, int num_sms, cudaStream_t stream) {
    if (args.n_tasks <= 0) return cudaSuccess;
    switch (precision) {
        case LUMRAD_PRECISION_FP16:
            return record ? launch_t<StoreF16, true>(args, num_sms, stream) : launch_t<StoreF16, false>(args, num_sms, stream);
        case LUMRAD_PRECISION_BF16:
            return record ? launch_t<StoreBF16, true>(args, num_sms, stream) : launch_t<StoreBF16, false>(args, num_sms, stream);
        default:
            return record ? launch_t<StoreF32, true>(args, num_sms, stream) : launch_t<StoreF32, false>(args, num_sms, stream);
    }
}

}  // namespace lumrad
