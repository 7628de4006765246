// radiance_device.cuh — device helpers of the radiance pass shared by its kernels: exact FP32
// arithmetic, radiance storage types, voxel lookups, ray setup, refine + shading, the subgroup
// reduction and the probe store.  Restates shaders/radiance.comp (line numbers cited inline).
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <cuda/atomic>
#include "lumrad_internal.h"

namespace lumrad {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
// c + a*b rounded once, for a product a*b that is exact in FP32 (a power-of-two scale of a value
// that stays normal, or a product by 0 or 1): then fadd(c, fmul(a, b)) rounds only the sum, the
// same value (a zero product takes the sign rules of the addition either way), in one instruction
// instead of two.
__device__ __forceinline__ float fadd_exact_mul(float c, float a, float b) { return __fmaf_rn(a, b, c); }
// x / d where `inv` is 1/d if that is exact (d a power of two), else 0
__device__ __forceinline__ float fdiv_by(float x, float d, float inv) { return inv != 0.0f ? fmul(x, inv) : fdiv(x, d); }
// GLSL min/max definitions: identical NaN and signed-zero behaviour everywhere.
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
// float -> int toward zero; PTX cvt.rzi saturates and maps NaN to 0.
__device__ __forceinline__ int f2i(float f) { return __float2int_rz(f); }

// The GPU's nanosecond clock (%globaltimer), the same on every SM.
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Programmatic dependent launch: a kernel launched as a dependent of the stream's previous one
// starts once every CTA of that one has called grid_launch_dependents, and grid_dependency_wait
// returns when that kernel has finished and its writes are visible (at once for a plain launch).
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
// SPIR-V OpSMod for a positive divisor.
__device__ __forceinline__ int smod(int a, int b) {
    int r = a % b;
    return (r < 0) ? r + b : r;
}
// Hit records report every NaN as the canonical quiet NaN 0x7FC00000.
__device__ __forceinline__ float canon_nan(float f) { return f == f ? f : __int_as_float(0x7FC00000); }

// ---------------------------------------------------------------- radiance storage types
struct StoreF32 {
    typedef float4 T;
    static __device__ __forceinline__ float3 load(const T* p, int i) {
        float4 v = __ldg(p + i);
        return make_float3(v.x, v.y, v.z);
    }
    static __device__ __forceinline__ void store(T* p, int i, float3 v) { p[i] = make_float4(v.x, v.y, v.z, 1.0f); }
};
struct StoreF16 {
    typedef uint2 T;   // (r,g) (b,1) as two half2
    static __device__ __forceinline__ float3 load(const T* p, int i) {
        uint2 v = __ldg(p + i);
        __half2 a = *reinterpret_cast<__half2*>(&v.x);
        __half2 b = *reinterpret_cast<__half2*>(&v.y);
        return make_float3(__low2float(a), __high2float(a), __low2float(b));
    }
    static __device__ __forceinline__ void store(T* p, int i, float3 v) {
        __half2 a = __floats2half2_rn(v.x, v.y);
        __half2 b = __floats2half2_rn(v.z, 1.0f);
        uint2 o;
        o.x = *reinterpret_cast<unsigned*>(&a);
        o.y = *reinterpret_cast<unsigned*>(&b);
        p[i] = o;
    }
};
struct StoreBF16 {
    typedef uint2 T;
    static __device__ __forceinline__ float3 load(const T* p, int i) {
        uint2 v = __ldg(p + i);
        __nv_bfloat162 a = *reinterpret_cast<__nv_bfloat162*>(&v.x);
        __nv_bfloat162 b = *reinterpret_cast<__nv_bfloat162*>(&v.y);
        return make_float3(__low2float(a), __high2float(a), __low2float(b));
    }
    static __device__ __forceinline__ void store(T* p, int i, float3 v) {
        __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
        __nv_bfloat162 b = __floats2bfloat162_rn(v.z, 1.0f);
        uint2 o;
        o.x = *reinterpret_cast<unsigned*>(&a);
        o.y = *reinterpret_cast<unsigned*>(&b);
        p[i] = o;
    }
};

// The reference's own volume format, A2B10G10R10_UNORM_PACK32 (radiance.comp:20-21,
// internal_render.cpp:128-135): R in bits 0-9, G 10-19, B 20-29, alpha 30-31 (stored as 3).
// Store: clamp to [0,1] (NaN -> 0; the caller has clamped), code = round-to-nearest-even of
// v * 1023 in FP32.  Load: code / 1023 rounded once to FP32, as r0 = code * RN(1/1023) and one
// FMA correction step (exact for every one of the 1024 codes; a test checks them all).
__device__ __forceinline__ unsigned unorm10_encode(float v) { return __float2uint_rn(fmul(v, 1023.0f)); }
__device__ __forceinline__ float unorm10_decode(unsigned q) {
    const float c = __uint_as_float(0x3a802008u);   // RN(1/1023)
    const float qf = (float)q;                      // exact: q < 1024
    const float r0 = fmul(qf, c);
    const float e = __fmaf_rn(-r0, 1023.0f, qf);    // q - r0 * 1023, exact
    return __fmaf_rn(e, c, r0);
}
struct StoreRGB10A2 {
    typedef unsigned T;
    static __device__ __forceinline__ float3 load(const T* p, int i) {
        const unsigned v = __ldg(p + i);
        return make_float3(unorm10_decode(v & 1023u), unorm10_decode((v >> 10) & 1023u), unorm10_decode((v >> 20) & 1023u));
    }
    static __device__ __forceinline__ void store(T* p, int i, float3 v) {
        p[i] = unorm10_encode(v.x) | (unorm10_encode(v.y) << 10) | (unorm10_encode(v.z) << 20) | (3u << 30);
    }
};

// ---------------------------------------------------------------- voxel lookups
// GetVoxel (radiance.comp:121-143) on integer voxel coordinates.  Block coordinate = ix/16
// truncated (OpSDiv); voxel in block = ix mod 16 floored (OpSMod) = ix & 15.  The grid fetch is
// in range iff -15 <= ix < 16*X, and then ix/16 == max(ix,0) >> 4; out of range reads block 0.
__device__ __forceinline__ bool grid_index(int X, int Y, int Z, int ix, int iy, int iz, int& idx) {
    const bool in = (unsigned)ix + 15u < (unsigned)(16 * X + 15) && (unsigned)iy + 15u < (unsigned)(16 * Y + 15) &&
                    (unsigned)iz + 15u < (unsigned)(16 * Z + 15);
    idx = (max(ix, 0) >> 4) + X * ((max(iy, 0) >> 4) + Y * (max(iz, 0) >> 4));
    return in;
}

// What the march and refine tests read of the current world (kept in registers).
struct MarchView {
    int X, Y, Z;
    int wide;                     // compact ids are uint16
    const uint8_t* cgrid;
    const uint32_t* cbits;
};

__device__ __forceinline__ MarchView march_view(const WorldPass& w) {
    return MarchView{w.X, w.Y, w.Z, w.cgrid_wide, reinterpret_cast<const uint8_t*>(w.cgrid), w.cbits};
}

// Compact lookup: compact id of the block (0 iff block id 0) and whether the voxel is solid (the
// mask's bit x + 16y + 256z, read as the 16-bit row (y, z) of its little-endian words: fewer index
// operations than the 32-bit word holding two rows), with the compact id's width known at
// compile time (WIDE: uint16 ids, else uint8), on the compact grid `cg` and the masks' 16-bit rows
// `rows`, in global memory (read through the read-only path) or, SMEM, staged in shared memory.
template <bool WIDE, bool SMEM>
__device__ __forceinline__ bool solid_at_p(const uint8_t* cg, const uint16_t* rows, int X, int Y, int Z, int ix,
                                           int iy, int iz, int& cid) {
    int idx;
    int c = 0;
    if (grid_index(X, Y, Z, ix, iy, iz, idx)) {
        if (SMEM) c = WIDE ? (int)reinterpret_cast<const uint16_t*>(cg)[idx] : (int)cg[idx];
        else c = WIDE ? (int)__ldg(reinterpret_cast<const uint16_t*>(cg) + idx) : (int)__ldg(cg + idx);
    }
    cid = c;
    const int r = (c << 8) | ((iz & 15) << 4) | (iy & 15);
    const unsigned row = SMEM ? (unsigned)rows[r] : (unsigned)__ldg(rows + r);
    return (row >> (ix & 15)) & 1u;
}
template <bool WIDE>
__device__ __forceinline__ bool solid_at_w(const MarchView& m, int ix, int iy, int iz, int& cid) {
    return solid_at_p<WIDE, false>(m.cgrid, reinterpret_cast<const uint16_t*>(m.cbits), m.X, m.Y, m.Z, ix, iy, iz, cid);
}

// solid_at_w for a regular ray's position (finite, |p| < 2^21), from tb = trunc(p/16) per axis
// (FP32, exact): trunc(p)/16 truncated is trunc(p/16), and -15 <= trunc(p) < 16*size holds exactly
// when 0 <= trunc(p/16) < size (p in (-16, 0) gives -0, block 0 like OpSDiv).  The block index is
// the float's integer through the bits of 1.5*2^23 + tb (an add; -0 becomes +0), and the range test
// one unsigned compare per axis; `in` reports it (the grid's range: -16 < p < 16*size per axis).
template <bool WIDE, bool SMEM>
__device__ __forceinline__ bool solid_at_tbp(const uint8_t* cg, const uint16_t* rows, int X, int Y, int Z, float tbx,
                                             float tby, float tbz, int ix, int iy, int iz, int& cid, bool& in) {
    const int bx = __float_as_int(fadd(tbx, 12582912.0f)) - 0x4B400000;
    const int by = __float_as_int(fadd(tby, 12582912.0f)) - 0x4B400000;
    const int bz = __float_as_int(fadd(tbz, 12582912.0f)) - 0x4B400000;
    int c = 0;
    in = (unsigned)bx < (unsigned)X && (unsigned)by < (unsigned)Y && (unsigned)bz < (unsigned)Z;
    if (in) {
        const int idx = bx + X * (by + Y * bz);
        if (SMEM) c = WIDE ? (int)reinterpret_cast<const uint16_t*>(cg)[idx] : (int)cg[idx];
        else c = WIDE ? (int)__ldg(reinterpret_cast<const uint16_t*>(cg) + idx) : (int)__ldg(cg + idx);
    }
    cid = c;
    const int r = (c << 8) | ((iz & 15) << 4) | (iy & 15);
    const unsigned row = SMEM ? (unsigned)rows[r] : (unsigned)__ldg(rows + r);
    return (row >> (ix & 15)) & 1u;
}

// Original lookup (voxel value and block id): block id b addresses palette slot
// (b mod 64) + 64*(b/64) (voxel_in_palette :105-110 on the 64x64-slot image): slot b for
// b >= 0, slot b+64 for -63 <= b < 0, nothing past the loaded slots.
__device__ __forceinline__ int voxel_value(const WorldPass& w, int ix, int iy, int iz, int& block) {
    int idx;
    int b = 0;
    if (grid_index(w.X, w.Y, w.Z, ix, iy, iz, idx)) b = __ldg(w.grid + idx);
    block = b;
    const int slot = b < 0 ? b + 64 : b;
    if (b < -63 || slot >= w.n_slots) return 0;
    return __ldg(w.pal + ((slot << 12) | ((iz & 15) << 8) | ((iy & 15) << 4) | (ix & 15)));
}

// t / nsub for t >= 0 (nsub = R/32: a power of two for the usual ray counts, a shift then)
__device__ __forceinline__ int div_nsub(int t, int nsub) {
    return (nsub & (nsub - 1)) == 0 ? t >> (__ffs(nsub) - 1) : t / nsub;
}

// ---------------------------------------------------------------- ray setup (:362-381)
__device__ __forceinline__ float3 hash33(uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t k = 1103515245u;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const uint32_t nx = ((x >> 8) ^ y) * k;
        const uint32_t ny = ((y >> 8) ^ z) * k;
        const uint32_t nz = ((z >> 8) ^ x) * k;
        x = nx; y = ny; z = nz;
    }
    const float s = 2.3283064365386963e-10f;   // 1/float(0xffffffffu) = 2^-32
    return make_float3(fmul(__uint2float_rn(x), s), fmul(__uint2float_rn(y), s), fmul(__uint2float_rn(z), s));
}

__device__ __forceinline__ float3 normalize3(float3 v) {
    const float dd = fadd(fadd(fmul(v.x, v.x), fmul(v.y, v.y)), fmul(v.z, v.z));
    const float s = __frcp_rn(__fsqrt_rn(dd));   // 1/x rounded once: the reciprocal rounded once
    return make_float3(fmul(v.x, s), fmul(v.y, s), fmul(v.z, s));
}

// Ray r of workgroup g: origin and direction.  The seed's x is the global invocation id g*R + r
// (radiance.comp:370), in uint32 arithmetic like gl_GlobalInvocationID.
__device__ __forceinline__ void setup_ray(const WorldPass& w, int g, int r, float3& o, float3& d) {
    const short4 q = __ldg(w.req + ((long long)g * w.size + w.shift));
    uint32_t sx = (uint32_t)g * (uint32_t)w.R + (uint32_t)r + w.seed;
    const uint32_t sy = w.seed, sz = w.seed;
    // block centre q*16 + 8 (q an int16: the product is exact)
    const float3 c = make_float3(fadd_exact_mul(8.0f, (float)q.x, 16.0f), fadd_exact_mul(8.0f, (float)q.y, 16.0f),
                                 fadd_exact_mul(8.0f, (float)q.z, 16.0f));
    const float4 f = __ldg(w.dirs + r);
    const float3 r1 = hash33(sx, sy, sz);
    sx++;
    // 0.1*((r - 0.5)*2) as 0.2*(r - 0.5): the doubling is exact (|r - 0.5| >= 2^-32 or 0) and the
    // float 0.2f is exactly twice the float 0.1f, so both round the same real product
    const float3 j = make_float3(fmul(0.2f, fsub(r1.x, 0.5f)), fmul(0.2f, fsub(r1.y, 0.5f)), fmul(0.2f, fsub(r1.z, 0.5f)));
    d = normalize3(make_float3(fadd(f.x, j.x), fadd(f.y, j.y), fadd(f.z, j.z)));
    o = make_float3(fadd(c.x, fmul(d.x, 6.0f)), fadd(c.y, fmul(d.y, 6.0f)), fadd(c.z, fmul(d.z, 6.0f)));
    const float3 r2 = hash33(sx, sy, sz);
    o = make_float3(fadd_exact_mul(o.x, fsub(r2.x, 0.5f), 2.0f), fadd_exact_mul(o.y, fsub(r2.y, 0.5f), 2.0f),
                    fadd_exact_mul(o.z, fsub(r2.z, 0.5f), 2.0f));
    if (r & 1) d = make_float3(-d.x, -d.y, -d.z);
}

// ---------------------------------------------------------------- finalize (:246-291, :316-354)
template <class Store>
__device__ __forceinline__ float3 sample_trilinear(const WorldPass& w, float ux, float uy, float uz) {
    const typename Store::T* rad = reinterpret_cast<const typename Store::T*>(w.prev);
    const int X = w.X, Y = w.Y, Z = w.Z;
    const float u[3] = {fsub(fmul(ux, (float)X), 0.5f), fsub(fmul(uy, (float)Y), 0.5f), fsub(fmul(uz, (float)Z), 0.5f)};
    const int n[3] = {X, Y, Z};
    int i0[3], i1[3];
    float t[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float fl = floorf(u[c]);
        t[c] = fsub(u[c], fl);
        int ii = f2i(fl);
        if ((unsigned)ii >= (unsigned)n[c]) ii = smod(ii, n[c]);   // REPEAT wrap; in range needs none
        i0[c] = ii;
        i1[c] = (ii + 1 == n[c]) ? 0 : ii + 1;
    }
    auto tex = [&](int x, int y, int z) { return Store::load(rad, x + X * (y + Y * z)); };
    auto lerp = [](float3 p, float3 q, float s) {
        const float r = fsub(1.0f, s);
        return make_float3(fadd(fmul(p.x, r), fmul(q.x, s)), fadd(fmul(p.y, r), fmul(q.y, s)),
                           fadd(fmul(p.z, r), fmul(q.z, s)));
    };
    const float3 c00 = lerp(tex(i0[0], i0[1], i0[2]), tex(i1[0], i0[1], i0[2]), t[0]);
    const float3 c10 = lerp(tex(i0[0], i1[1], i0[2]), tex(i1[0], i1[1], i0[2]), t[0]);
    const float3 c01 = lerp(tex(i0[0], i0[1], i1[2]), tex(i1[0], i0[1], i1[2]), t[0]);
    const float3 c11 = lerp(tex(i0[0], i1[1], i1[2]), tex(i1[0], i1[1], i1[2]), t[0]);
    return lerp(lerp(c00, c10, t[1]), lerp(c01, c11, t[1]), t[2]);
}

// info word of a marched ray: bits 0-15 coarse steps, 16-23 coarse voxel (records only),
// 24 hit, 25 stopped by the step bound.
//
// A marched ray's shading in two parts: finalize_ray (refine, material, hit point; the sky for a
// miss) reads no radiance volume; shade_hit (the trilinear taps of the previous volume) does.  A
// pass's finalize launch may run the first part while the previous pass still writes the volume.
// Returns whether the ray hit; a miss's light is in `light`, a hit's tap coordinates in u and its
// material in m.  WIDE: the compact ids' width (the caller branches on it once per warp: 3% of the
// finalize's instructions against testing it at every lookup).
template <bool RECORD, bool WIDE>
__device__ __forceinline__ bool finalize_ray(const WorldPass& w, const MarchView& mv, float3 o, float3 d,
                                             float coarse_frac, uint32_t info, int block, long long gr,
                                             uint32_t& lookups, float3& light, float3& u, float4& m) {
    const bool hit = (info >> 24) & 1u;
    const int coarse_steps = info & 0xffff;
    lookups = coarse_steps;
    LumRadHit rec;
    if (RECORD) {
        rec.voxel[0] = rec.voxel[1] = rec.voxel[2] = 0;
        rec.block = (int16_t)block;
        rec.voxel_id = 0;
        rec.flags = (hit ? LUMRAD_HIT_HIT : 0) | (((info >> 25) & 1u) ? LUMRAD_HIT_CAPPED : 0);
        rec.coarse_steps = (uint16_t)coarse_steps;
        rec.refine_steps = 0;
        rec.coarse_voxel = (uint8_t)((info >> 16) & 0xff);
        rec.fraction = canon_nan(coarse_frac);
    }
    if (hit) {
        // refine DDA (radiance.comp:246-288)
        const float back = fsub(coarse_frac, 1.5f);
        const float bhx = fadd(o.x, fmul(d.x, back));
        const float bhy = fadd(o.y, fmul(d.y, back));
        const float bhz = fadd(o.z, fmul(d.z, back));
        const int stx = d.x > 0.0f ? 1 : -1, sty = d.y > 0.0f ? 1 : -1, stz = d.z > 0.0f ? 1 : -1;
        const float ivx = __frcp_rn(d.x), ivy = __frcp_rn(d.y), ivz = __frcp_rn(d.z);
        const float c1x = fdiv(fsub(floorf(bhx), bhx), d.x);
        const float c1y = fdiv(fsub(floorf(bhy), bhy), d.y);
        const float c1z = fdiv(fsub(floorf(bhz), bhz), d.z);
        float tmx = gmax(c1x, fadd(c1x, ivx));
        float tmy = gmax(c1y, fadd(c1y, ivy));
        float tmz = gmax(c1z, fadd(c1z, ivz));
        const float tdx = fabsf(ivx), tdy = fabsf(ivy), tdz = fabsf(ivz);   // 1/|d| == |1/d|
        int vx = f2i(bhx), vy = f2i(bhy), vz = f2i(bhz);
        int cid;
        bool solid = solid_at_w<WIDE>(mv, vx, vy, vz, cid);
        float fsx = 0.0f, fsy = 0.0f, fsz = 0.0f;
        int it = 0;
        while (it < 5 && !solid) {
            const bool bx = (tmx <= tmy) && (tmx <= tmz);
            const bool by = (tmx >= tmy) && (tmy <= tmz);
            const bool bz = (tmz <= tmx) && (tmz <= tmy);
            fsx = bx ? 1.0f : 0.0f; fsy = by ? 1.0f : 0.0f; fsz = bz ? 1.0f : 0.0f;
            vx += bx ? stx : 0; vy += by ? sty : 0; vz += bz ? stz : 0;
            tmx = fadd_exact_mul(tmx, tdx, fsx);   // fs is 0 or 1 (inf * 0 is NaN either way)
            tmy = fadd_exact_mul(tmy, tdy, fsy);
            tmz = fadd_exact_mul(tmz, tdz, fsz);
            solid = solid_at_w<WIDE>(mv, vx, vy, vz, cid);
            it++;
        }
        lookups += 1 + it;
        int blk = 0;
        int cur = 0;
        if (solid) {
            if (!RECORD && w.cslot) {
                // the hit block's palette slot through its compact id (one dependent load less
                // than reading the int16 grid; same slot: a compact id stands for one block id)
                const int slot = __ldg(w.cslot + cid);
                cur = slot >= 0 ? __ldg(w.pal + ((slot << 12) | ((vz & 15) << 8) | ((vy & 15) << 4) | (vx & 15))) : 0;
            } else {
                cur = voxel_value(w, vx, vy, vz, blk);
            }
        }
        const float nx = -fmul((float)stx, fsx), ny = -fmul((float)sty, fsy), nz = -fmul((float)stz, fsz);
        const float fr = fadd_exact_mul(fadd_exact_mul(fmul(fsub(tmx, tdx), fsx), fsub(tmy, tdy), fsy), fsub(tmz, tdz), fsz);
        // material (GetMat :145-157) and sample_radiance (:161-166); /16 == *0.0625 exactly
        m = __ldg(w.mats + cur);
        const float hx = fadd(o.x, fmul(fr, d.x));
        const float hy = fadd(o.y, fmul(fr, d.y));
        const float hz = fadd(o.z, fmul(fr, d.z));
        const float bpx = fmul(fadd_exact_mul(hx, nx, 16.0f), 0.0625f);   // n is 0 or +-1
        const float bpy = fmul(fadd_exact_mul(hy, ny, 16.0f), 0.0625f);
        const float bpz = fmul(fadd_exact_mul(hz, nz, 16.0f), 0.0625f);
        u = make_float3(fdiv_by(fadd(bpx, 0.5f), (float)w.X, w.inv_dim[0]), fdiv_by(fadd(bpy, 0.5f), (float)w.Y, w.inv_dim[1]),
                        fdiv_by(fadd(bpz, 0.5f), (float)w.Z, w.inv_dim[2]));
        if (RECORD) {
            rec.voxel[0] = vx; rec.voxel[1] = vy; rec.voxel[2] = vz;
            rec.voxel_id = (uint8_t)cur;
            rec.refine_steps = (uint8_t)it;
            rec.flags |= (fsx != 0.0f ? LUMRAD_HIT_STEP_X : 0) | (fsy != 0.0f ? LUMRAD_HIT_STEP_Y : 0) |
                         (fsz != 0.0f ? LUMRAD_HIT_STEP_Z : 0);
            rec.fraction = canon_nan(fr);
        }
    } else {
        // sky and sun (radiance.comp:334-343).  Constants, each the FP32 round-to-nearest result
        // of the shader's expression (normalize3 above on (0.5, 0.5, -0.9), then the products):
        //   globalLightDir = (kGl, kGl, kGlz);  0.9*3 = kSun, 0.6*3 = kSunB;  0.1*(0.53, 0.81, 0.92)
        constexpr unsigned kGl = 0x3edfab13u, kGlz = 0xbf494d2au, kSun = 0x402cccccu, kSunB = 0x3fe66667u;
        constexpr unsigned kSkyR = 0x3d591687u, kSkyG = 0x3da5e354u, kSkyB = 0x3dbc6a7fu;
        const float gl = __uint_as_float(kGl);
        const float g = -fadd(fadd(fmul(d.x, gl), fmul(d.y, gl)), fmul(d.z, __uint_as_float(kGlz)));
        light = make_float3(0.0f, 0.0f, 0.0f);
        if (g > 0.95f) {
            light.x = fadd(light.x, fmul(g, __uint_as_float(kSun)));
            light.y = fadd(light.y, fmul(g, __uint_as_float(kSun)));
            light.z = fadd(light.z, fmul(g, __uint_as_float(kSunB)));
        }
        light.x = fadd(light.x, __uint_as_float(kSkyR));
        light.y = fadd(light.y, __uint_as_float(kSkyG));
        light.z = fadd(light.z, __uint_as_float(kSkyB));
    }
    if (RECORD) w.hits[gr] = rec;
    return hit;
}

// The hit's light (radiance.comp:331-333): the previous volume's trilinear sample at u
// (sample_radiance :161-166) times the material colour, plus colour times emission.
template <class Store>
__device__ __forceinline__ float3 shade_hit(const WorldPass& w, float3 u, float4 m) {
    const float3 L = sample_trilinear<Store>(w, u.x, u.y, u.z);
    return make_float3(fadd(0.0f, fadd(fmul(L.x, m.x), fmul(m.x, m.w))), fadd(0.0f, fadd(fmul(L.y, m.y), fmul(m.y, m.w))),
                       fadd(0.0f, fadd(fmul(L.z, m.z), fmul(m.z, m.w))));
}

__device__ __forceinline__ float3 butterfly_sum(float3 v) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        v.x = fadd(v.x, __shfl_xor_sync(kFull, v.x, m));
        v.y = fadd(v.y, __shfl_xor_sync(kFull, v.y, m));
        v.z = fadd(v.z, __shfl_xor_sync(kFull, v.z, m));
    }
    return v;
}

__device__ __forceinline__ float clamp01(float v) { return v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f; }

// store_probe (radiance.comp:349-354): blend the clamped old value with the mean, store clamped.
template <class Store>
__device__ __forceinline__ void store_probe(const WorldPass& w, int g, float3 acc) {
    const short4 q = __ldg(w.req + ((long long)g * w.size + w.shift));
    if (q.x < 0 || q.y < 0 || q.z < 0 || q.x >= w.X || q.y >= w.Y || q.z >= w.Z) return;
    const int idx = q.x + w.X * (q.y + w.Y * q.z);
    float3 old = Store::load(reinterpret_cast<const typename Store::T*>(w.prev), idx);
    old.x = old.x < 0.0f ? 0.0f : old.x; old.x = 1.0f < old.x ? 1.0f : old.x;
    old.y = old.y < 0.0f ? 0.0f : old.y; old.y = 1.0f < old.y ? 1.0f : old.y;
    old.z = old.z < 0.0f ? 0.0f : old.z; old.z = 1.0f < old.z ? 1.0f : old.z;
    const float3 nv = make_float3(clamp01(fadd(fmul(old.x, w.one_minus_alpha), fmul(acc.x, w.alpha))),
                                  clamp01(fadd(fmul(old.y, w.one_minus_alpha), fmul(acc.y, w.alpha))),
                                  clamp01(fadd(fmul(old.z, w.one_minus_alpha), fmul(acc.z, w.alpha))));
    Store::store(reinterpret_cast<typename Store::T*>(w.next), idx, nv);
}

// Subgroup mean V = sum/32 of subgroup k of workgroup g (R > 32) is done, and the probe's
// subgroups span CTAs: V goes to scratch and the last of the probe's R/32 subgroups sums them in
// order (radiance.comp:401-407), divides by R/32 and stores.  Lane 0 only.
template <class Store>
__device__ __forceinline__ void subgroup_done(const WorldPass& w, int g, int k, float3 v) {
    const int nsub = w.R >> 5;
    float4* slots = w.scratch + (long long)g * nsub;
    __stcg(slots + k, make_float4(v.x, v.y, v.z, 0.0f));
    // acq_rel at device scope: our mean is visible before the count, and the last subgroup
    // sees every other subgroup's mean
    cuda::atomic_ref<int, cuda::thread_scope_device> count(w.probe_count[g]);
    const int prior = count.fetch_add(1, cuda::memory_order_acq_rel);
    if (prior != nsub - 1) return;
    float3 acc = make_float3(0.0f, 0.0f, 0.0f);
    for (int j = 0; j < nsub; j++) {
        const float4 s = __ldcg(slots + j);
        acc = make_float3(fadd(acc.x, s.x), fadd(acc.y, s.y), fadd(acc.z, s.z));
    }
    const float fn = (float)nsub;
    acc = make_float3(fdiv_by(acc.x, fn, w.inv_nsub), fdiv_by(acc.y, fn, w.inv_nsub), fdiv_by(acc.z, fn, w.inv_nsub));
    store_probe<Store>(w, g, acc);
    count.store(0, cuda::memory_order_relaxed);   // ready for the next launch
}

__device__ __forceinline__ int world_of(const LaunchArgs& la, int t) {
    const int n = la.dev_n_worlds ? *la.dev_n_worlds : la.n_worlds;
    if (n <= 1) return 0;
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (la.worlds[mid].task_begin <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

}  // namespace
}  // namespace lumrad
