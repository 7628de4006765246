// radiance_aux.cu — the device work either side of the radiance pass:
//
//   update list   the probes update_radiance relights each frame (internal_render.cpp:1142-1168):
//                 every block whose clamped 3x3x3 neighbourhood has a positive id sum, in scan
//                 order, then each special request whose block is not already listed, in request
//                 order.  Four launches: flag (one bit per block, ballot) + per-CTA counts, a
//                 single-CTA scan of the counts, an order-preserving write, and the specials.
//   scroll        shift_radiance (internal_render.cpp:1218-1335): new(p) = old(p + shift) where
//                 p + shift is inside the world, old(p) elsewhere; one pass into the other
//                 ping-pong volume.
//   gather        the 8-probe consumer read of diffuse.frag:36-90 (sample_radiance(position,
//                 normal)): trilinear weights times a clamped directional weight over the 8
//                 surrounding probes, probe values clamped to [0, 2].
//
// All FP32 arithmetic is written out in the shader's order with round-to-nearest intrinsics (no
// contraction), so results are reproducible bit for bit.

#include "radiance_device.cuh"

#include <algorithm>

namespace lumrad {
namespace {

constexpr int kListCta = 256;      // blocks per CTA of the list kernels (8 warps)
constexpr int kScanCta = 1024;

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__global__ void __launch_bounds__(kListCta)
list_flags_kernel(const int16_t* __restrict__ grid, int X, int Y, int Z, long long W, uint32_t* __restrict__ bits,
                  int* __restrict__ cta_counts) {
    __shared__ int s_cnt[kListCta / 32];
    const long long i = (long long)blockIdx.x * kListCta + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool flag = false;
    if (i < W) {
        const int x = (int)(i % X);
        const long long q = i / X;
        const int y = (int)(q % Y);
        const int z = (int)(q / Y);
        int sum = 0;   // sum of the 27 clamped neighbours' ids (internal_render.cpp:1147-1156)
        for (int dz = -1; dz <= 1; dz++) {
            const int tz = clampi(z + dz, 0, Z - 1);
            for (int dy = -1; dy <= 1; dy++) {
                const int ty = clampi(y + dy, 0, Y - 1);
                const int16_t* row = grid + (size_t)X * ((size_t)ty + (size_t)Y * tz);
                for (int dx = -1; dx <= 1; dx++) sum += __ldg(row + clampi(x + dx, 0, X - 1));
            }
        }
        flag = sum > 0;
    }
    const unsigned b = __ballot_sync(kFull, flag);
    const long long word = i >> 5;
    if (lane == 0) {
        if (word < (W + 31) / 32) bits[word] = b;
        s_cnt[warp] = __popc(b);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int c = 0;
        for (int w = 0; w < kListCta / 32; w++) c += s_cnt[w];
        cta_counts[blockIdx.x] = c;
    }
}

// Exclusive scan of `v` over the CTA (kScanCta threads); returns the CTA total through *total.
__device__ __forceinline__ int cta_exclusive_scan(int v, int* s_warp, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += t;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    const int excl = x - v + (warp > 0 ? s_warp[warp - 1] : 0);
    *total = s_warp[31];
    __syncthreads();   // s_warp is reused by the next call
    return excl;
}

__global__ void __launch_bounds__(kScanCta)
list_scan_kernel(const int* __restrict__ counts, int n, int* __restrict__ offsets, int* __restrict__ total) {
    __shared__ int s_warp[32];
    int carry = 0;
    for (int base = 0; base < n; base += kScanCta) {
        const int i = base + threadIdx.x;
        const int v = i < n ? counts[i] : 0;
        int chunk = 0;
        const int excl = cta_exclusive_scan(v, s_warp, &chunk);
        if (i < n) offsets[i] = carry + excl;
        carry += chunk;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kListCta)
list_write_kernel(const uint32_t* __restrict__ bits, const int* __restrict__ offsets, int X, int Y, long long W,
                  short4* __restrict__ out) {
    __shared__ int s_pre[kListCta / 32];
    const long long words = (W + 31) / 32;
    if (threadIdx.x < kListCta / 32) {
        const long long wi = (long long)blockIdx.x * (kListCta / 32) + threadIdx.x;
        s_pre[threadIdx.x] = wi < words ? __popc(bits[wi]) : 0;
    }
    __syncthreads();
    const long long i = (long long)blockIdx.x * kListCta + threadIdx.x;
    if (i >= W) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t b = bits[i >> 5];
    if (!((b >> lane) & 1u)) return;
    int pos = offsets[blockIdx.x] + __popc(b & ((1u << lane) - 1u));
    for (int w = 0; w < warp; w++) pos += s_pre[w];
    const int x = (int)(i % X);
    const long long q = i / X;
    out[pos] = make_short4((short)x, (short)(q % Y), (short)(q / Y), 0);
}

// Dirty probes of block edits (Chebyshev distance <= r): a byte mask of the edited blocks, dilated
// along x, then y, then z; the last pass writes one bit per block and the CTA counts, as
// list_flags_kernel does, so list_scan_kernel and list_write_kernel emit the list in scan order.
__global__ void dirty_mark_kernel(const short4* __restrict__ edits, int n, int X, int Y, uint8_t* __restrict__ mask) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const short4 e = edits[k];
    mask[(size_t)e.x + (size_t)X * ((size_t)e.y + (size_t)Y * e.z)] = 1;
}

// one axis of the dilation: out[i] = OR of in over [-r, r] steps of `stride` along an axis of n
__global__ void dirty_dilate_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, int X, int Y, int Z,
                                    int axis, int r, long long W) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < W; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % X);
        const long long q = i / X;
        const int y = (int)(q % Y), z = (int)(q / Y);
        const int c = axis == 0 ? x : (axis == 1 ? y : z);
        const int n = axis == 0 ? X : (axis == 1 ? Y : Z);
        const long long stride = axis == 0 ? 1 : (axis == 1 ? (long long)X : (long long)X * Y);
        uint8_t v = 0;
        for (int d = max(c - r, 0); d <= min(c + r, n - 1); d++) v |= __ldg(in + i + (long long)(d - c) * stride);
        out[i] = v;
    }
}

__global__ void __launch_bounds__(kListCta)
dirty_flags_kernel(const uint8_t* __restrict__ in, int X, int Y, int Z, int r, long long W, uint32_t* __restrict__ bits,
                   int* __restrict__ cta_counts) {
    __shared__ int s_cnt[kListCta / 32];
    const long long i = (long long)blockIdx.x * kListCta + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool flag = false;
    if (i < W) {   // the z pass of the dilation
        const long long XY = (long long)X * Y;
        const int z = (int)(i / XY);
        for (int d = max(z - r, 0); d <= min(z + r, Z - 1) && !flag; d++) flag = __ldg(in + i + (long long)(d - z) * XY) != 0;
    }
    const unsigned b = __ballot_sync(kFull, flag);
    const long long word = i >> 5;
    if (lane == 0) {
        if (word < (W + 31) / 32) bits[word] = b;
        s_cnt[warp] = __popc(b);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int c = 0;
        for (int w = 0; w < kListCta / 32; w++) c += s_cnt[w];
        cta_counts[blockIdx.x] = c;
    }
}

// Specials in request order, each unless its block is already listed (duplicates are kept, as
// in the reference: `set` only marks rule-listed blocks).
__global__ void __launch_bounds__(kScanCta)
list_specials_kernel(const short4* __restrict__ sp, int ns, const uint32_t* __restrict__ bits, int X, int Y,
                     const int* __restrict__ listed, short4* __restrict__ out, int* __restrict__ count) {
    __shared__ int s_warp[32];
    int carry = *listed;
    for (int base = 0; base < ns; base += kScanCta) {
        const int i = base + threadIdx.x;
        int keep = 0;
        short4 s = make_short4(0, 0, 0, 0);
        if (i < ns) {
            s = sp[i];
            const long long idx = (long long)s.x + (long long)X * ((long long)s.y + (long long)Y * s.z);
            keep = ((bits[idx >> 5] >> (idx & 31)) & 1u) ? 0 : 1;
        }
        int chunk = 0;
        const int excl = cta_exclusive_scan(keep, s_warp, &chunk);
        if (keep) out[carry + excl] = s;
        carry += chunk;
    }
    if (threadIdx.x == 0) *count = carry;
}

template <typename V>
__global__ void shift_kernel(const V* __restrict__ src, V* __restrict__ dst, int X, int Y, int Z, int sx, int sy,
                             int sz, long long W) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < W; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % X);
        const long long q = i / X;
        const int y = (int)(q % Y), z = (int)(q / Y);
        const int qx = x + sx, qy = y + sy, qz = z + sz;
        const bool inside = qx >= 0 && qx < X && qy >= 0 && qy < Y && qz >= 0 && qz < Z;
        dst[i] = inside ? src[(size_t)qx + (size_t)X * ((size_t)qy + (size_t)Y * qz)] : src[i];
    }
}

// sample_probe (diffuse.frag:25-33): texelFetch at the clamped probe (outside the volume reads 0,
// the robust-access definition), clamped to [0, 2].
template <class Store>
__device__ __forceinline__ float3 gather_probe(const typename Store::T* rad, int X, int Y, int Z, int px, int py,
                                               int pz) {
    px = clampi(px, 0, X);
    py = clampi(py, 0, Y);
    pz = clampi(pz, 0, Z);
    float3 v = make_float3(0.0f, 0.0f, 0.0f);
    if (px < X && py < Y && pz < Z) v = Store::load(rad, (int)((size_t)px + (size_t)X * ((size_t)py + (size_t)Y * pz)));
    return make_float3(gmin(gmax(v.x, 0.0f), 2.0f), gmin(gmax(v.y, 0.0f), 2.0f), gmin(gmax(v.z, 0.0f), 2.0f));
}

template <class Store>
__global__ void gather_kernel(const typename Store::T* __restrict__ rad, int X, int Y, int Z,
                              const float* __restrict__ pts, int n, float* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float* q = pts + 6 * (size_t)k;
    const float px = q[0], py = q[1], pz = q[2], nx = q[3], ny = q[4], nz = q[5];
    // zero probe: clamp(ivec3(floor(position - 8.0)) / 16, 0, world_size)   (:42)
    const int zx = clampi(f2i(floorf(fsub(px, 8.0f))) / 16, 0, X);
    const int zy = clampi(f2i(floorf(fsub(py, 8.0f))) / 16, 0, Y);
    const int zz = clampi(f2i(floorf(fsub(pz, 8.0f))) / 16, 0, Z);
    const float cx = fadd(fmul((float)zx, 16.0f), 8.0f);   // (:43)
    const float cy = fadd(fmul((float)zy, 16.0f), 8.0f);
    const float cz = fadd(fmul((float)zz, 16.0f), 8.0f);
    // alpha = clamp((position - zero_probe_pos) / 16, 0, 1)   (:45); x/16 == x*0.0625 exactly
    const float ax = gmin(gmax(fmul(fsub(px, cx), 0.0625f), 0.0f), 1.0f);
    const float ay = gmin(gmax(fmul(fsub(py, cy), 0.0625f), 0.0f), 1.0f);
    const float az = gmin(gmax(fmul(fsub(pz, cz), 0.0625f), 0.0f), 1.0f);
    float tw = 0.0f, tr = 0.0f, tg = 0.0f, tb = 0.0f;
#pragma unroll 1
    for (int i = 0; i < 8; i++) {
        const int ox = i & 1, oy = (i >> 1) & 1, oz = (i >> 2) & 1;   // (:50)
        const float fx = (float)ox, fy = (float)oy, fz = (float)oz;
        const float3 ptp = make_float3(fsub(fadd(cx, fmul(fx, 16.0f)), px), fsub(fadd(cy, fmul(fy, 16.0f)), py),
                                       fsub(fadd(cz, fmul(fz, 16.0f)), pz));   // (:55-57)
        const float3 dir = normalize3(ptp);   // (:58)
        // mix(1 - alpha, alpha, offset) = (1-alpha)*(1-offset) + alpha*offset   (:60)
        const float tx = fadd(fmul(fsub(1.0f, ax), fsub(1.0f, fx)), fmul(ax, fx));
        const float ty = fadd(fmul(fsub(1.0f, ay), fsub(1.0f, fy)), fmul(ay, fy));
        const float tz = fadd(fmul(fsub(1.0f, az), fsub(1.0f, fz)), fmul(az, fz));
        float w = fmul(fmul(tx, ty), tz);   // (:61)
        const float d = fadd(fadd(fmul(dir.x, nx), fmul(dir.y, ny)), fmul(dir.z, nz));
        w = fmul(w, gmin(gmax(d, 0.1f), 1.0f));   // (:70-74)
        const float3 c = gather_probe<Store>(rad, X, Y, Z, zx + ox, zy + oy, zz + oz);   // (:81)
        w = gmax(1e-7f, w);   // (:84)
        tw = fadd(tw, w);
        tr = fadd(tr, fmul(w, c.x));
        tg = fadd(tg, fmul(w, c.y));
        tb = fadd(tb, fmul(w, c.z));
    }
    out[3 * (size_t)k] = fdiv(tr, tw);   // (:89)
    out[3 * (size_t)k + 1] = fdiv(tg, tw);
    out[3 * (size_t)k + 2] = fdiv(tb, tw);
}

// exec_copies' block copies (internal_render.cpp:1446-1451): palette slot dst = slot src, one CTA
// of 256 threads x 16 bytes per copy.
__global__ void __launch_bounds__(256) palette_copy_kernel(uint8_t* __restrict__ pal, const int2* __restrict__ copies) {
    const int2 c = copies[blockIdx.x];
    const uint4* src = reinterpret_cast<const uint4*>(pal + (size_t)c.x * 4096);
    uint4* dst = reinterpret_cast<uint4*>(pal + (size_t)c.y * 4096);
    dst[threadIdx.x] = src[threadIdx.x];
}

// map.comp:33-67 for one mesh.  Invocation g covers world voxel g + 0.5 + shift; the model voxel is
// inverse_trans * (world_voxel, 1) truncated; a non-zero model voxel goes to the temporary block
// (id >= static_blocks) that holds the world voxel.  Truncation sends world voxels in (-1, 1) to
// coordinate 0 and those in [-15, -1] onto block 0's far side, so several invocations can target
// one palette voxel (the reference races there).  Writes are resolved as if the invocations ran
// one after another in linear order (x fastest) and the meshes in order: each invocation
// atomicMax-es (mesh, invocation, value) into the target's 64-bit owner word; a resolve pass
// writes the winning values.
__global__ void map_kernel(const int16_t* __restrict__ grid, int X, int Y, int Z, int n_slots, int static_blocks,
                           const uint8_t* __restrict__ model, int mx, int my, int mz, MapArgs a,
                           unsigned long long* __restrict__ owner, unsigned long long mesh_key) {
    const int gx = blockIdx.x * blockDim.x + threadIdx.x;
    const int gy = blockIdx.y * blockDim.y + threadIdx.y;
    const int gz = blockIdx.z * blockDim.z + threadIdx.z;
    if (gx >= a.dims[0] || gy >= a.dims[1] || gz >= a.dims[2]) return;
    // world_voxel = vec3(g) / 1.0 + vec3(0.5) + vec3(shift)   (:37-40)
    const float wx = fadd(fadd((float)gx, 0.5f), (float)a.shift[0]);
    const float wy = fadd(fadd((float)gy, 0.5f), (float)a.shift[1]);
    const float wz = fadd(fadd((float)gz, 0.5f), (float)a.shift[2]);
    const int ix = f2i(wx), iy = f2i(wy), iz = f2i(wz);   // (:41)
    // model_voxel = (inverse_trans * vec4(world_voxel, 1)).xyz, columns summed in order   (:47-48)
    const float* m = a.inv;   // column-major m[4*col + row]
    const float vx = fadd(fadd(fadd(fmul(m[0], wx), fmul(m[4], wy)), fmul(m[8], wz)), m[12]);
    const float vy = fadd(fadd(fadd(fmul(m[1], wx), fmul(m[5], wy)), fmul(m[9], wz)), m[13]);
    const float vz = fadd(fadd(fadd(fmul(m[2], wx), fmul(m[6], wy)), fmul(m[10], wz)), m[14]);
    const int px = f2i(vx), py = f2i(vy), pz = f2i(vz);
    // target block = iworld / 16 (OpSDiv); out of range reads block 0   (:50-52)
    const int bx = ix / 16, by = iy / 16, bz = iz / 16;
    int id = 0;
    if (bx >= 0 && by >= 0 && bz >= 0 && bx < X && by < Y && bz < Z)
        id = grid[(size_t)bx + (size_t)X * ((size_t)by + (size_t)Y * bz)];
    if (id < static_blocks || id >= n_slots) return;   // (:59); the palette ends at its last slot
    int v = 0;
    if (px >= 0 && py >= 0 && pz >= 0 && px < mx && py < my && pz < mz)
        v = model[(size_t)px + (size_t)mx * ((size_t)py + (size_t)my * pz)];   // (:60)
    if (v == 0) return;
    const unsigned long long lin =
        (unsigned long long)gx + (unsigned long long)a.dims[0] * ((unsigned long long)gy + (unsigned long long)a.dims[1] * gz);
    const size_t t = ((size_t)(id - static_blocks) << 12) | (smod(iz, 16) << 8) | (smod(iy, 16) << 4) | smod(ix, 16);
    atomicMax(owner + t, mesh_key | (lin << 8) | (unsigned long long)v);   // (:54,62)
}

__global__ void map_resolve_kernel(uint8_t* __restrict__ pal_tmp, const unsigned long long* __restrict__ owner,
                                   size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long o = owner[i];
        if (o) pal_tmp[i] = (uint8_t)(o & 0xffu);
    }
}

// Occupancy masks of compact ids from the device palette: CTA c, thread w -> word w of id c.
__global__ void __launch_bounds__(128) compact_bits_kernel(const uint8_t* __restrict__ pal, const int* __restrict__ slot_of,
                                                           uint32_t* __restrict__ cbits) {
    const int c = blockIdx.x, w = threadIdx.x;
    const int slot = slot_of[c];
    uint32_t bits = 0;
    if (slot >= 0) {
        const uint4* p = reinterpret_cast<const uint4*>(pal + (size_t)slot * 4096 + 32 * w);
        const uint4 a = p[0], b = p[1];
        const uint32_t words[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int k = 0; k < 32; k++)
            if ((words[k >> 2] >> (8 * (k & 3))) & 0xffu) bits |= 1u << k;
    }
    cbits[(size_t)c * 128 + w] = bits;
}

// A radiance volume as packed RGB floats (the storage type decoded exactly).
template <class Store>
__global__ void pack_rgb_kernel(const typename Store::T* __restrict__ rad, float* __restrict__ out, long long W) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < W; i += (long long)gridDim.x * blockDim.x) {
        const float3 v = Store::load(rad, (int)i);
        out[3 * i] = v.x;
        out[3 * i + 1] = v.y;
        out[3 * i + 2] = v.z;
    }
}

}  // namespace

cudaError_t launch_pack_rgb(const void* rad, int precision, long long W, float* out, cudaStream_t stream) {
    const int blocks = (int)std::min<long long>((W + 255) / 256, 152LL * 8);
    switch (precision) {
        case LUMRAD_PRECISION_FP16:
            pack_rgb_kernel<StoreF16><<<blocks, 256, 0, stream>>>(static_cast<const uint2*>(rad), out, W);
            break;
        case LUMRAD_PRECISION_BF16:
            pack_rgb_kernel<StoreBF16><<<blocks, 256, 0, stream>>>(static_cast<const uint2*>(rad), out, W);
            break;
        case LUMRAD_PRECISION_RGB10A2:
            pack_rgb_kernel<StoreRGB10A2><<<blocks, 256, 0, stream>>>(static_cast<const unsigned*>(rad), out, W);
            break;
        default:
            pack_rgb_kernel<StoreF32><<<blocks, 256, 0, stream>>>(static_cast<const float4*>(rad), out, W);
    }
    return cudaGetLastError();
}

cudaError_t launch_palette_copies(uint8_t* pal, const int2* copies, int n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    palette_copy_kernel<<<n, 256, 0, stream>>>(pal, copies);
    return cudaGetLastError();
}

cudaError_t launch_map(const int16_t* grid, int X, int Y, int Z, int n_slots, int static_blocks, const uint8_t* model,
                       int mx, int my, int mz, const MapArgs& a, int mesh, unsigned long long* owner,
                       cudaStream_t stream) {
    if (a.dims[0] <= 0 || a.dims[1] <= 0 || a.dims[2] <= 0) return cudaSuccess;
    const dim3 block(4, 4, 4);   // local_size 4x4x4 (:32)
    const dim3 grid_dim((a.dims[0] + 3) / 4, (a.dims[1] + 3) / 4, (a.dims[2] + 3) / 4);
    map_kernel<<<grid_dim, block, 0, stream>>>(grid, X, Y, Z, n_slots, static_blocks, model, mx, my, mz, a, owner,
                                               (unsigned long long)(mesh + 1) << 40);
    return cudaGetLastError();
}

cudaError_t launch_map_resolve(uint8_t* pal_tmp, const unsigned long long* owner, size_t n, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    map_resolve_kernel<<<blocks, 256, 0, stream>>>(pal_tmp, owner, n);
    return cudaGetLastError();
}

cudaError_t launch_compact_bits(const uint8_t* pal, const int* slot_of, int n_compact, uint32_t* cbits,
                                cudaStream_t stream) {
    if (n_compact <= 0) return cudaSuccess;
    compact_bits_kernel<<<n_compact, 128, 0, stream>>>(pal, slot_of, cbits);
    return cudaGetLastError();
}

cudaError_t launch_update_list(const int16_t* grid, int X, int Y, int Z, const short4* specials, int n_specials,
                               const ListScratch& s, short4* out, int* count, cudaStream_t stream) {
    const long long W = (long long)X * Y * Z;
    const int ctas = (int)((W + kListCta - 1) / kListCta);
    list_flags_kernel<<<ctas, kListCta, 0, stream>>>(grid, X, Y, Z, W, s.bits, s.cta_counts);
    list_scan_kernel<<<1, kScanCta, 0, stream>>>(s.cta_counts, ctas, s.cta_offsets, s.listed);
    list_write_kernel<<<ctas, kListCta, 0, stream>>>(s.bits, s.cta_offsets, X, Y, W, out);
    list_specials_kernel<<<1, kScanCta, 0, stream>>>(specials, n_specials, s.bits, X, Y, s.listed, out, count);
    return cudaGetLastError();
}

cudaError_t launch_dirty_list(const short4* edits, int n_edits, int X, int Y, int Z, int radius, uint8_t* mask_a,
                              uint8_t* mask_b, const ListScratch& s, short4* out, int* count, cudaStream_t stream) {
    const long long W = (long long)X * Y * Z;
    const int ctas = (int)((W + kListCta - 1) / kListCta);
    const int blocks = (int)std::min<long long>((W + 255) / 256, 152LL * 16);
    cudaError_t e = cudaMemsetAsync(mask_a, 0, (size_t)W, stream);
    if (e != cudaSuccess) return e;
    if (n_edits > 0) dirty_mark_kernel<<<(n_edits + 255) / 256, 256, 0, stream>>>(edits, n_edits, X, Y, mask_a);
    dirty_dilate_kernel<<<blocks, 256, 0, stream>>>(mask_a, mask_b, X, Y, Z, 0, radius, W);
    dirty_dilate_kernel<<<blocks, 256, 0, stream>>>(mask_b, mask_a, X, Y, Z, 1, radius, W);
    dirty_flags_kernel<<<ctas, kListCta, 0, stream>>>(mask_a, X, Y, Z, radius, W, s.bits, s.cta_counts);
    list_scan_kernel<<<1, kScanCta, 0, stream>>>(s.cta_counts, ctas, s.cta_offsets, count);
    list_write_kernel<<<ctas, kListCta, 0, stream>>>(s.bits, s.cta_offsets, X, Y, W, out);
    return cudaGetLastError();
}

size_t list_scratch_words(long long W) { return (size_t)((W + 31) / 32); }
size_t list_scratch_ctas(long long W) { return (size_t)((W + kListCta - 1) / kListCta); }

cudaError_t launch_shift_radiance(const void* src, void* dst, int X, int Y, int Z, int sx, int sy, int sz,
                                  int precision, cudaStream_t stream) {
    const long long W = (long long)X * Y * Z;
    const int blocks = (int)std::min<long long>((W + 255) / 256, 152LL * 16);
    if (precision == LUMRAD_PRECISION_FP32)
        shift_kernel<uint4><<<blocks, 256, 0, stream>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), X, Y,
                                                        Z, sx, sy, sz, W);
    else if (precision == LUMRAD_PRECISION_RGB10A2)
        shift_kernel<unsigned><<<blocks, 256, 0, stream>>>(static_cast<const unsigned*>(src), static_cast<unsigned*>(dst),
                                                           X, Y, Z, sx, sy, sz, W);
    else
        shift_kernel<uint2><<<blocks, 256, 0, stream>>>(static_cast<const uint2*>(src), static_cast<uint2*>(dst), X, Y,
                                                        Z, sx, sy, sz, W);
    return cudaGetLastError();
}

cudaError_t launch_gather(const void* rad, int X, int Y, int Z, int precision, const float* pts, int n, float* out,
                          cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int blocks = (n + 255) / 256;
    switch (precision) {
        case LUMRAD_PRECISION_FP16:
            gather_kernel<StoreF16><<<blocks, 256, 0, stream>>>(static_cast<const uint2*>(rad), X, Y, Z, pts, n, out);
            break;
        case LUMRAD_PRECISION_BF16:
            gather_kernel<StoreBF16><<<blocks, 256, 0, stream>>>(static_cast<const uint2*>(rad), X, Y, Z, pts, n, out);
            break;
        case LUMRAD_PRECISION_RGB10A2:
            gather_kernel<StoreRGB10A2><<<blocks, 256, 0, stream>>>(static_cast<const unsigned*>(rad), X, Y, Z, pts, n,
                                                                    out);
            break;
        default:
            gather_kernel<StoreF32><<<blocks, 256, 0, stream>>>(static_cast<const float4*>(rad), X, Y, Z, pts, n, out);
    }
    return cudaGetLastError();
}

}  // namespace lumrad
