// lumrad_internal.h — device-side argument blocks shared by the host runtime and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/lumrad.h"

namespace lumrad {

// Rays per warp pool: a warp sets up, marches and reduces this many rays at a time.
constexpr int kPool = 128;
// Warps per CTA of the pass kernel.
constexpr int kWarps = 8;
// Shared memory per warp: origin, direction, 1/direction (float4 each) + fraction + info.
constexpr int kSmemPerWarp = kPool * (3 * 16 + 4 + 4);

// One resident world as the kernels see it (all pointers are device pointers).
struct WorldView {
    int X, Y, Z;              // blocks per axis
    int n_slots;              // palette slots present on the device
    int slot0_empty;          // 1 if palette slot 0 is all zero (lets air steps skip a load)
    const int16_t* grid;      // X*Y*Z block ids, x-fastest
    const uint8_t* pal;       // n_slots * 4096 voxels: voxel (x,y,z) at x + 16*y + 256*z
    const float4* mats;       // 256 x (r, g, b, emission)
};

// One pass over one world.
struct PassArgs {
    WorldView w;
    const void* prev;         // radiance volume read (storage type per precision)
    void* next;               // radiance volume written (a copy of prev before the pass)
    const short4* req;        // update list (x, y, z, w)
    int n_groups;             // workgroups: n_requests / size
    int size, shift;          // request r of group g is g*size + shift
    int R;                    // rays per probe (multiple of 32)
    int probes_per_unit;      // probes per warp work unit: kPool/R (>=1)
    float max_dist;
    int max_steps;            // 2*max_dist + 2
    float alpha, one_minus_alpha;
    uint32_t seed;            // time seed
    const float4* dirs;       // R spherical-Fibonacci directions
    LumRadHit* hits;          // per-ray records or nullptr
    unsigned long long* counters;  // [0] steps, [1] hits, or nullptr
};

// Launches one pass on `stream`; returns a CUDA error code.
cudaError_t launch_radiance_pass(const PassArgs& args, int precision, bool record, bool stats,
                                 int num_sms, cudaStream_t stream);

}  // namespace lumrad
