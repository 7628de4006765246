// radiance_pass.cu — sm_103a kernels of the per-block radiance update.
//
// Restates shaders/radiance.comp (main :361-413, trace_ray :316-346, CastRay_fast :183-291,
// GetVoxel :121-143, sample_radiance :161-166, store_probe :349-354, hash33 :51-66) for one
// warp per work unit instead of one 64-invocation workgroup per probe:
//
//   setup    all 32 lanes build the rays of a pool (kPool rays, in lock step) into shared memory;
//   march    a flat loop in which every lane advances its ray one coarse step per iteration and,
//            when the ray ends, records (fraction, voxel) and takes the next ray of the pool —
//            long and short rays share the warp without waiting for one another;
//   finalize in lock step again: refine DDA, material, trilinear radiance fetch, shading; then
//            the 32 lanes of each subgroup reduce by xor-butterfly and the last subgroup of a
//            probe blends and stores it.
//
// All float arithmetic uses round-to-nearest intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn,
// __fsqrt_rn), which the compiler never fuses into FMA, in the order the shader evaluates it,
// so hit records are bit-exact and radiance bit-identical to the FP32 CPU restatement.

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include "lumrad_internal.h"

namespace lumrad {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
// GLSL min/max definitions (y < x ? y : x, x < y ? y : x): identical NaN and signed-zero
// behaviour on every implementation.
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
// float -> int toward zero; PTX cvt.rzi saturates and maps NaN to 0.
__device__ __forceinline__ int f2i(float f) { return __float2int_rz(f); }
// SPIR-V OpSMod (sign of the divisor) for a positive divisor.
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
    static __device__ __forceinline__ void store(T* p, int i, float3 v) {
        p[i] = make_float4(v.x, v.y, v.z, 1.0f);
    }
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

// ---------------------------------------------------------------- voxel lookup
// GetVoxel + voxel_in_palette (radiance.comp:97-143) on integer voxel coordinates.
// Block coordinate = ix/16 truncated (OpSDiv); voxel in block = ix mod 16 floored (OpSMod,
// i.e. ix & 15).  The grid fetch is in range iff -15 <= ix < 16*X, and then ix/16 == max(ix,0)>>4.
// Block id b addresses palette slot (b mod 64) + 64*(b/64): slot b for b >= 0, slot b+64 for
// -63 <= b < 0, nothing (0) otherwise or past the loaded slots.
__device__ __forceinline__ int fetch_voxel(const WorldView& w, int ix, int iy, int iz, int& block) {
    int b = 0;
    if ((unsigned)ix + 15u < (unsigned)(16 * w.X + 15) &&
        (unsigned)iy + 15u < (unsigned)(16 * w.Y + 15) &&
        (unsigned)iz + 15u < (unsigned)(16 * w.Z + 15)) {
        int bx = max(ix, 0) >> 4, by = max(iy, 0) >> 4, bz = max(iz, 0) >> 4;
        b = __ldg(w.grid + (bx + w.X * (by + w.Y * bz)));
    }
    block = b;
    int v = 0;
    int slot = b < 0 ? b + 64 : b;
    if (b >= -63 && slot < w.n_slots && !(b == 0 && w.slot0_empty))
        v = __ldg(w.pal + ((slot << 12) | ((iz & 15) << 8) | ((iy & 15) << 4) | (ix & 15)));
    return v;
}

// ---------------------------------------------------------------- ray setup (:362-381)
__device__ __forceinline__ float3 hash33(uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t k = 1103515245u;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        uint32_t nx = ((x >> 8) ^ y) * k;
        uint32_t ny = ((y >> 8) ^ z) * k;
        uint32_t nz = ((z >> 8) ^ x) * k;
        x = nx; y = ny; z = nz;
    }
    const float s = 2.3283064365386963e-10f;   // 1/float(0xffffffffu) = 2^-32
    return make_float3(fmul(__uint2float_rn(x), s), fmul(__uint2float_rn(y), s),
                       fmul(__uint2float_rn(z), s));
}

__device__ __forceinline__ float3 normalize3(float3 v) {
    float dd = fadd(fadd(fmul(v.x, v.x), fmul(v.y, v.y)), fmul(v.z, v.z));
    float s = fdiv(1.0f, __fsqrt_rn(dd));
    return make_float3(fmul(v.x, s), fmul(v.y, s), fmul(v.z, s));
}

// Ray `gr` = g*R + r of the dispatch: origin, direction and 1/direction.
__device__ __forceinline__ void setup_ray(const PassArgs& a, long long gr, float4& o4, float4& d4,
                                          float4& inv4) {
    const int g = (int)(gr / a.R);
    const int r = (int)(gr - (long long)g * a.R);
    const short4 q = __ldg(a.req + ((long long)g * a.size + a.shift));
    uint32_t sx = (uint32_t)gr + a.seed, sy = a.seed, sz = a.seed;
    float3 c = make_float3(fadd(fmul((float)q.x, 16.0f), 8.0f), fadd(fmul((float)q.y, 16.0f), 8.0f),
                           fadd(fmul((float)q.z, 16.0f), 8.0f));
    const float4 f = __ldg(a.dirs + r);
    float3 r1 = hash33(sx, sy, sz);
    sx++;
    float3 j = make_float3(fmul(0.1f, fmul(fsub(r1.x, 0.5f), 2.0f)), fmul(0.1f, fmul(fsub(r1.y, 0.5f), 2.0f)),
                           fmul(0.1f, fmul(fsub(r1.z, 0.5f), 2.0f)));
    float3 d = normalize3(make_float3(fadd(f.x, j.x), fadd(f.y, j.y), fadd(f.z, j.z)));
    float3 o = make_float3(fadd(c.x, fmul(d.x, 6.0f)), fadd(c.y, fmul(d.y, 6.0f)), fadd(c.z, fmul(d.z, 6.0f)));
    float3 r2 = hash33(sx, sy, sz);
    o = make_float3(fadd(o.x, fmul(fsub(r2.x, 0.5f), 2.0f)), fadd(o.y, fmul(fsub(r2.y, 0.5f), 2.0f)),
                    fadd(o.z, fmul(fsub(r2.z, 0.5f), 2.0f)));
    if (r & 1) d = make_float3(-d.x, -d.y, -d.z);
    o4 = make_float4(o.x, o.y, o.z, 0.0f);
    d4 = make_float4(d.x, d.y, d.z, 0.0f);
    inv4 = make_float4(fdiv(1.0f, d.x), fdiv(1.0f, d.y), fdiv(1.0f, d.z), 0.0f);
}

// ---------------------------------------------------------------- coarse march (:198-244)
// info word: bits 0-15 coarse steps, 16-23 coarse voxel, 24 hit, 25 step bound reached.
template <bool RECORD>
__device__ __forceinline__ void march_pool(const WorldView& w, float4* so, const float4* sd,
                                           const float4* sinv, float* sfrac, uint32_t* sinfo,
                                           int n, float max_dist, int max_steps, int lane) {
    const float wx = fmul((float)w.X, 16.0f), wy = fmul((float)w.Y, 16.0f), wz = fmul((float)w.Z, 16.0f);
    int my = lane;
    float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0, ix_ = 0, iy_ = 0, iz_ = 0;
    float cx = 0, cy = 0, cz = 0, frac = 0.0f;
    int steps = 0;
    bool active = my < n;
    auto load = [&](int i) {
        float4 o = so[i], d = sd[i], v = sinv[i];
        ox = o.x; oy = o.y; oz = o.z;
        dx = d.x; dy = d.y; dz = d.z;
        ix_ = v.x; iy_ = v.y; iz_ = v.z;
        cx = dx > 0.0f ? 16.0f : 0.0f;
        cy = dy > 0.0f ? 16.0f : 0.0f;
        cz = dz > 0.0f ? 16.0f : 0.0f;
        frac = 0.0f;
        steps = 0;
    };
    if (active) load(my);
    int next_ray = 32;
    int done = 0;
    while (done < n) {
        bool fin = false;
        uint32_t info = 0;
        int block = 0;
        if (active) {
            frac = fadd(frac, 0.5f);
            steps++;
            const float px = fadd(ox, fmul(dx, frac));
            const float py = fadd(oy, fmul(dy, frac));
            const float pz = fadd(oz, fmul(dz, frac));
            const int ix = f2i(px), iy = f2i(py), iz = f2i(pz);
            const int vox = fetch_voxel(w, ix, iy, iz, block);
            if (block == 0) {
                const float bx = fadd((float)((ix / 16) * 16), cx);
                const float by = fadd((float)((iy / 16) * 16), cy);
                const float bz = fadd((float)((iz / 16) * 16), cz);
                const float tx = fadd(fmul(bx, ix_), fmul(-px, ix_));
                const float ty = fadd(fmul(by, iy_), fmul(-py, iy_));
                const float tz = fadd(fmul(bz, iz_), fmul(-pz, iz_));
                float f = gmin(tx, gmin(ty, tz));
                f = gmax(f, 0.01f);
                frac = fadd(frac, f);
            }
            if (vox != 0) {
                fin = true;
                info = (uint32_t)steps | ((uint32_t)vox << 16) | (1u << 24);
            } else if (px < 0.0f || py < 0.0f || pz < 0.0f || px >= wx || py >= wy || pz >= wz ||
                       frac >= max_dist) {
                fin = true;
                info = (uint32_t)steps;
            } else if (steps >= max_steps) {
                fin = true;
                info = (uint32_t)steps | (1u << 25);
            }
        }
        const unsigned fm = __ballot_sync(kFull, fin);
        if (fm) {
            if (fin) {
                sfrac[my] = frac;
                sinfo[my] = info;
                if (RECORD) so[my].w = __int_as_float(block);   // block id kept for the record
                const int rank = __popc(fm & ((1u << lane) - 1u));
                my = next_ray + rank;
                active = my < n;
                if (active) load(my);
            }
            next_ray += __popc(fm);
            done += __popc(fm);
        }
    }
}

// ---------------------------------------------------------------- finalize (:246-291, :316-346)
template <class Store>
__device__ __forceinline__ float3 sample_trilinear(const PassArgs& a, float ux, float uy, float uz) {
    const WorldView& w = a.w;
    const typename Store::T* rad = reinterpret_cast<const typename Store::T*>(a.prev);
    const float u[3] = {fsub(fmul(ux, (float)w.X), 0.5f), fsub(fmul(uy, (float)w.Y), 0.5f),
                        fsub(fmul(uz, (float)w.Z), 0.5f)};
    const int n[3] = {w.X, w.Y, w.Z};
    int i0[3], i1[3];
    float t[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float fl = floorf(u[c]);
        t[c] = fsub(u[c], fl);
        const int ii = smod(f2i(fl), n[c]);
        i0[c] = ii;
        i1[c] = (ii + 1 == n[c]) ? 0 : ii + 1;
    }
    auto tex = [&](int x, int y, int z) { return Store::load(rad, x + w.X * (y + w.Y * z)); };
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

template <class Store, bool RECORD>
__device__ __forceinline__ float3 finalize_ray(const PassArgs& a, float4 o4, float4 d4, float4 inv4,
                                               float coarse_frac, uint32_t info, int block,
                                               long long gr, uint32_t& lookups) {
    const WorldView& w = a.w;
    const bool hit = (info >> 24) & 1u;
    const int coarse_steps = info & 0xffff;
    lookups = coarse_steps;
    float3 light;
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
        const float bhx = fadd(o4.x, fmul(d4.x, fsub(coarse_frac, 1.5f)));
        const float bhy = fadd(o4.y, fmul(d4.y, fsub(coarse_frac, 1.5f)));
        const float bhz = fadd(o4.z, fmul(d4.z, fsub(coarse_frac, 1.5f)));
        const int stx = d4.x > 0.0f ? 1 : -1, sty = d4.y > 0.0f ? 1 : -1, stz = d4.z > 0.0f ? 1 : -1;
        const float c1x = fdiv(fsub(floorf(bhx), bhx), d4.x);
        const float c1y = fdiv(fsub(floorf(bhy), bhy), d4.y);
        const float c1z = fdiv(fsub(floorf(bhz), bhz), d4.z);
        float tmx = gmax(c1x, fadd(c1x, inv4.x));
        float tmy = gmax(c1y, fadd(c1y, inv4.y));
        float tmz = gmax(c1z, fadd(c1z, inv4.z));
        const float tdx = fabsf(inv4.x), tdy = fabsf(inv4.y), tdz = fabsf(inv4.z);
        int vx = f2i(bhx), vy = f2i(bhy), vz = f2i(bhz);
        int blk;
        int cur = fetch_voxel(w, vx, vy, vz, blk);
        float fsx = 0.0f, fsy = 0.0f, fsz = 0.0f;
        int it = 0;
        while (it < 5 && cur == 0) {
            const bool bx = (tmx <= tmy) && (tmx <= tmz);
            const bool by = (tmx >= tmy) && (tmy <= tmz);
            const bool bz = (tmz <= tmx) && (tmz <= tmy);
            fsx = bx ? 1.0f : 0.0f; fsy = by ? 1.0f : 0.0f; fsz = bz ? 1.0f : 0.0f;
            vx += bx ? stx : 0; vy += by ? sty : 0; vz += bz ? stz : 0;
            tmx = fadd(tmx, fmul(tdx, fsx));
            tmy = fadd(tmy, fmul(tdy, fsy));
            tmz = fadd(tmz, fmul(tdz, fsz));
            cur = fetch_voxel(w, vx, vy, vz, blk);
            it++;
        }
        lookups += 1 + it;
        const float nx = -fmul((float)stx, fsx), ny = -fmul((float)sty, fsy), nz = -fmul((float)stz, fsz);
        const float fr = fadd(fadd(fmul(fsub(tmx, tdx), fsx), fmul(fsub(tmy, tdy), fsy)),
                              fmul(fsub(tmz, tdz), fsz));
        // material (GetMat :145-157) and sample_radiance (:161-166)
        const float4 m = __ldg(a.w.mats + cur);
        const float hx = fadd(o4.x, fmul(fr, d4.x));
        const float hy = fadd(o4.y, fmul(fr, d4.y));
        const float hz = fadd(o4.z, fmul(fr, d4.z));
        const float bpx = fdiv(fadd(hx, fmul(nx, 16.0f)), 16.0f);
        const float bpy = fdiv(fadd(hy, fmul(ny, 16.0f)), 16.0f);
        const float bpz = fdiv(fadd(hz, fmul(nz, 16.0f)), 16.0f);
        const float3 L = sample_trilinear<Store>(a, fdiv(fadd(bpx, 0.5f), (float)w.X),
                                                 fdiv(fadd(bpy, 0.5f), (float)w.Y),
                                                 fdiv(fadd(bpz, 0.5f), (float)w.Z));
        light = make_float3(fadd(0.0f, fadd(fmul(L.x, m.x), fmul(m.x, m.w))),
                            fadd(0.0f, fadd(fmul(L.y, m.y), fmul(m.y, m.w))),
                            fadd(0.0f, fadd(fmul(L.z, m.z), fmul(m.z, m.w))));
        if (RECORD) {
            rec.voxel[0] = vx; rec.voxel[1] = vy; rec.voxel[2] = vz;
            rec.voxel_id = (uint8_t)cur;
            rec.refine_steps = (uint8_t)it;
            rec.flags |= (fsx != 0.0f ? LUMRAD_HIT_STEP_X : 0) | (fsy != 0.0f ? LUMRAD_HIT_STEP_Y : 0) |
                         (fsz != 0.0f ? LUMRAD_HIT_STEP_Z : 0);
            rec.fraction = canon_nan(fr);
        }
    } else {
        // sky and sun (radiance.comp:334-343); globalLightDir = normalize(0.5, 0.5, -0.9)
        const float3 gl = normalize3(make_float3(0.5f, 0.5f, -0.9f));
        const float g = -fadd(fadd(fmul(d4.x, gl.x), fmul(d4.y, gl.y)), fmul(d4.z, gl.z));
        light = make_float3(0.0f, 0.0f, 0.0f);
        if (g > 0.95f) {
            light.x = fadd(light.x, fmul(g, fmul(0.9f, 3.0f)));
            light.y = fadd(light.y, fmul(g, fmul(0.9f, 3.0f)));
            light.z = fadd(light.z, fmul(g, fmul(0.6f, 3.0f)));
        }
        light.x = fadd(light.x, fmul(0.53f, 0.1f));
        light.y = fadd(light.y, fmul(0.81f, 0.1f));
        light.z = fadd(light.z, fmul(0.92f, 0.1f));
    }
    if (RECORD) a.hits[gr] = rec;
    return light;
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

// store_probe (radiance.comp:349-354)
template <class Store>
__device__ __forceinline__ void store_probe(const PassArgs& a, int g, float3 acc) {
    const short4 q = __ldg(a.req + ((long long)g * a.size + a.shift));
    const WorldView& w = a.w;
    if (q.x < 0 || q.y < 0 || q.z < 0 || q.x >= w.X || q.y >= w.Y || q.z >= w.Z) return;
    const int idx = q.x + w.X * (q.y + w.Y * q.z);
    float3 old = Store::load(reinterpret_cast<const typename Store::T*>(a.prev), idx);
    old.x = old.x < 0.0f ? 0.0f : old.x; old.x = 1.0f < old.x ? 1.0f : old.x;
    old.y = old.y < 0.0f ? 0.0f : old.y; old.y = 1.0f < old.y ? 1.0f : old.y;
    old.z = old.z < 0.0f ? 0.0f : old.z; old.z = 1.0f < old.z ? 1.0f : old.z;
    float3 nv = make_float3(fadd(fmul(old.x, a.one_minus_alpha), fmul(acc.x, a.alpha)),
                            fadd(fmul(old.y, a.one_minus_alpha), fmul(acc.y, a.alpha)),
                            fadd(fmul(old.z, a.one_minus_alpha), fmul(acc.z, a.alpha)));
    nv = make_float3(clamp01(nv.x), clamp01(nv.y), clamp01(nv.z));
    Store::store(reinterpret_cast<typename Store::T*>(a.next), idx, nv);
}

template <class Store, bool RECORD, bool STATS>
__global__ void __launch_bounds__(kWarps * 32)
radiance_pass_kernel(const __grid_constant__ PassArgs a) {
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    float4* so = smem + (size_t)wib * (kSmemPerWarp / 16);
    float4* sd = so + kPool;
    float4* sinv = sd + kPool;
    float* sfrac = reinterpret_cast<float*>(sinv + kPool);
    uint32_t* sinfo = reinterpret_cast<uint32_t*>(sfrac + kPool);

    const int R = a.R;
    const int B = a.probes_per_unit;
    const long long n_units = ((long long)a.n_groups + B - 1) / B;
    const long long gwarp = (long long)blockIdx.x * kWarps + wib;
    const long long nwarps = (long long)gridDim.x * kWarps;
    unsigned long long my_lookups = 0, my_hits = 0;

    for (long long u = gwarp; u < n_units; u += nwarps) {
        const long long g0 = u * B;
        const long long g1 = min(g0 + B, (long long)a.n_groups);
        const long long ray_end = g1 * R;
        float3 acc = make_float3(0.0f, 0.0f, 0.0f);
        for (long long c0 = g0 * R; c0 < ray_end; c0 += kPool) {
            const int n = (int)min((long long)kPool, ray_end - c0);
            for (int i = lane; i < n; i += 32) setup_ray(a, c0 + i, so[i], sd[i], sinv[i]);
            __syncwarp();
            march_pool<RECORD>(a.w, so, sd, sinv, sfrac, sinfo, n, a.max_dist, a.max_steps, lane);
            __syncwarp();
            for (int s = 0; s < n; s += 32) {
                const int i = s + lane;
                const long long gr = c0 + i;
                const int block = RECORD ? __float_as_int(so[i].w) : 0;
                uint32_t lk;
                float3 L = finalize_ray<Store, RECORD>(a, so[i], sd[i], sinv[i], sfrac[i], sinfo[i],
                                                       block, gr, lk);
                if (STATS) {
                    my_lookups += lk;
                    my_hits += (sinfo[i] >> 24) & 1u;
                }
                L = butterfly_sum(L);
                acc.x = fadd(acc.x, fdiv(L.x, 32.0f));
                acc.y = fadd(acc.y, fdiv(L.y, 32.0f));
                acc.z = fadd(acc.z, fdiv(L.z, 32.0f));
                const long long g = (c0 + s) / R;
                const int r_last = (int)((c0 + s) - g * R) + 32;
                if (r_last == R) {
                    const float nsub = (float)(R / 32);
                    acc = make_float3(fdiv(acc.x, nsub), fdiv(acc.y, nsub), fdiv(acc.z, nsub));
                    if (lane == 0) store_probe<Store>(a, (int)g, acc);
                    acc = make_float3(0.0f, 0.0f, 0.0f);
                }
            }
            __syncwarp();
        }
    }
    if (STATS) {
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) {
            my_lookups += __shfl_xor_sync(kFull, my_lookups, m);
            my_hits += __shfl_xor_sync(kFull, my_hits, m);
        }
        if (lane == 0 && (my_lookups | my_hits)) {
            atomicAdd(a.counters, my_lookups);
            atomicAdd(a.counters + 1, my_hits);
        }
    }
}

template <class Store, bool RECORD, bool STATS>
cudaError_t launch_t(const PassArgs& args, int num_sms, cudaStream_t stream) {
    auto kern = radiance_pass_kernel<Store, RECORD, STATS>;
    const int smem = kWarps * kSmemPerWarp;
    static bool configured = false;   // attribute set once per instantiation
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    const long long units = ((long long)args.n_groups + args.probes_per_unit - 1) / args.probes_per_unit;
    const long long warps_needed = units;
    long long blocks = (warps_needed + kWarps - 1) / kWarps;
    const long long cap = (long long)num_sms * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) return cudaSuccess;
    kern<<<(unsigned)blocks, kWarps * 32, smem, stream>>>(args);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_radiance_pass(const PassArgs& args, int precision, bool record, bool stats,
                                 int num_sms, cudaStream_t stream) {
    if (args.n_groups <= 0) return cudaSuccess;
#define LUMRAD_DISPATCH(STORE)                                                           \
    if (record) return stats ? launch_t<STORE, true, true>(args, num_sms, stream)        \
                             : launch_t<STORE, true, false>(args, num_sms, stream);      \
    return stats ? launch_t<STORE, false, true>(args, num_sms, stream)                   \
                 : launch_t<STORE, false, false>(args, num_sms, stream);
    switch (precision) {
        case LUMRAD_PRECISION_FP16: { LUMRAD_DISPATCH(StoreF16) }
        case LUMRAD_PRECISION_BF16: { LUMRAD_DISPATCH(StoreBF16) }
        default: { LUMRAD_DISPATCH(StoreF32) }
    }
#undef LUMRAD_DISPATCH
}

}  // namespace lumrad
