// radiance_oracle.cpp — TEST INFRASTRUCTURE, not product code.
//
// A scalar CPU restatement of Lum's radiance pass (shaders/radiance.comp) and of the update-list
// rule of LumInternalRenderer::update_radiance (src/renderer/src/internal_render.cpp:1142-1168).
// Only the tests, the smoke check and the benchmark's CPU-baseline leg load this library, and
// only as the checker / the timed CPU baseline; the product path never calls it.
//
// Parity: pinned against the reference shader itself, compiled as C++ from its own source by
// oracle/build_ref.py (see tests/test_oracle_ref.py), at the shader's own constants
// (64 rays, max_dist 128) on synthetic worlds and on the reference's demo scene.
//
// Every float operation below is written out in the order the shader evaluates it and is built
// with -ffp-contract=off (no FMA contraction), so results are reproducible bit for bit.
// Integer '/' is SPIR-V OpSDiv (truncation) and '%' is OpSMod (sign of the divisor): that is
// how glslang lowers GLSL's signed integer division and remainder.
//
// The template parameter T is the radiance scalar: float reproduces the FP32 pass; double is the
// FP64 oracle, which keeps the traversal (ray setup, march, refine, sample coordinates) in FP32
// and only does shading, trilinear weighting, the reduction and the blend in double.

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <limits>
#include <utility>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
typedef struct {
    int X, Y, Z;               // blocks per axis
    const int16_t* grid;       // X*Y*Z ids, x-fastest
    const uint8_t* palette;    // n_slots * 4096 voxels, voxel (x,y,z) at x + 16*y + 256*z
    int n_slots;
    const float* materials;    // 256 * 6 floats (LumInternal::Material)
} OracleWorld;

typedef struct {
    int rays;                  // rays per probe (multiple of 32)
    float max_dist;
    float blend;
    int time_seed;
    int size;                  // magicSize
    int shift;
    int unorm10;               // 1: store as A2B10G10R10_UNORM (each channel rounded to code/1023)
} OracleParams;

typedef struct {               // same 24-byte layout as LumRadHit in include/lumrad.h
    int32_t voxel[3];
    int16_t block;
    uint8_t voxel_id;
    uint8_t flags;
    uint16_t coarse_steps;
    uint8_t refine_steps;
    uint8_t coarse_voxel;
    float fraction;
} OracleHit;

typedef struct {
    uint64_t probes, rays, steps, hits;
} OracleStats;
}

namespace {

// ---------------------------------------------------------------- small float3 helpers
struct V3 { float x, y, z; };
inline V3 v3(float a) { return {a, a, a}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

// GLSL min/max: min(x,y) = y < x ? y : x ; max(x,y) = x < y ? y : x (GLSL 4.50 §8.3)
inline float gmin(float x, float y) { return y < x ? y : x; }
inline float gmax(float x, float y) { return x < y ? y : x; }
// normalize(v) = v * (1 / sqrt(dot(v,v))), dot summed x, y, z in order
inline V3 normalize3(V3 v) {
    float s = 1.0f / std::sqrt(dot3(v, v));
    return v * s;
}

// float -> int, truncating toward zero; NaN -> 0; saturating (PTX cvt.rzi.s32.f32 semantics)
inline int f2i(float f) {
    if (!(f == f)) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int)f;
}
// SPIR-V OpSMod: result has the sign of the divisor
inline int smod(int a, int b) {
    int r = a % b;
    if (r != 0 && ((r < 0) != (b < 0))) r += b;
    return r;
}

// ---------------------------------------------------------------- world lookups
struct World {
    int X, Y, Z;
    const int16_t* grid;
    const uint8_t* pal;
    int n_slots;
    const float* mats;
};

// texelFetch(blocks, p) (radiance.comp:97-103); out of range -> 0
inline int fetch_block(const World& w, int bx, int by, int bz) {
    if (bx < 0 || by < 0 || bz < 0 || bx >= w.X || by >= w.Y || bz >= w.Z) return 0;
    return (int)w.grid[(size_t)bx + (size_t)w.X * ((size_t)by + (size_t)w.Y * (size_t)bz)];
}
// texelFetch(blockPalette, p) on the 1024x1024x16 palette image (internal_render.cpp:137-145):
// slot (px/16, py/16) = id (id%64, id/64), voxel (px%16, py%16, pz).  Out of range -> 0.
inline int fetch_palette(const World& w, int px, int py, int pz) {
    if (px < 0 || py < 0 || pz < 0 || px >= 1024 || py >= 1024 || pz >= 16) return 0;
    int slot = (py / 16) * 64 + (px / 16);
    if (slot >= w.n_slots) return 0;
    return w.pal[(size_t)slot * 4096 + (size_t)(px % 16) + 16 * (py % 16) + 256 * pz];
}

struct VoxBlock { int voxel, block; };
// GetVoxel + voxel_in_palette (radiance.comp:105-143)
inline VoxBlock get_voxel(const World& w, V3 pos) {
    int ix = f2i(pos.x), iy = f2i(pos.y), iz = f2i(pos.z);
    int bx = ix / 16, by = iy / 16, bz = iz / 16;
    int rx = smod(ix, 16), ry = smod(iy, 16), rz = smod(iz, 16);
    int block = fetch_block(w, bx, by, bz);
    int px = rx + 16 * smod(block, 64);
    int py = ry + 16 * (block / 64);
    int vox = fetch_palette(w, px, py, rz);
    return {vox, block};
}

// ---------------------------------------------------------------- RNG (radiance.comp:51-66)
struct U3 { uint32_t x, y, z; };
const uint32_t HASH_K = 1103515245u;
inline V3 hash33(U3 v) {
    for (int i = 0; i < 3; i++) {
        U3 n;
        n.x = ((v.x >> 8) ^ v.y) * HASH_K;
        n.y = ((v.y >> 8) ^ v.z) * HASH_K;
        n.z = ((v.z >> 8) ^ v.x) * HASH_K;
        v = n;
    }
    const float s = 1.0f / 4294967296.0f;   // 1.0/float(0xffffffffu), float(0xffffffffu) = 2^32
    return {(float)v.x * s, (float)v.y * s, (float)v.z * s};
}

// ---------------------------------------------------------------- directions (:293-314)
const float PI_F = 3.1415926535897932384626433832795f;
V3 spherical_fibonacci(int i, int n) {
    const float phi_golden = std::sqrt(5.0f) * 0.5f + 0.5f;
    float fi = (float)i;
    float a = fi * (phi_golden - 1.0f);
    float frac = a - std::floor(a);
    float phi = 2.0f * PI_F * frac;
    float cos_t = 1.0f - (2.0f * fi + 1.0f) * (1.0f / (float)n);
    float s2 = 1.0f - cos_t * cos_t;
    s2 = gmin(gmax(s2, 0.0f), 1.0f);
    float sin_t = std::sqrt(s2);
    float c = (float)std::cos((double)phi);
    float s = (float)std::sin((double)phi);
    return {c * sin_t, s * sin_t, cos_t};
}

// ---------------------------------------------------------------- trace (:183-291, :316-346)
struct CastResult {
    bool hit;
    bool capped;
    float fraction;       // coarse distance at exit
    int coarse_steps;
    int coarse_voxel;
    int block;
};

// CastRay_fast coarse loop (radiance.comp:198-244)
inline CastResult coarse_march(const World& w, V3 o, V3 d, float max_dist, int max_steps) {
    V3 inv = V3{1.0f, 1.0f, 1.0f} / d;
    V3 corner = {d.x > 0.0f ? 16.0f : 0.0f, d.y > 0.0f ? 16.0f : 0.0f, d.z > 0.0f ? 16.0f : 0.0f};
    const V3 wmax = {(float)w.X * 16.0f, (float)w.Y * 16.0f, (float)w.Z * 16.0f};
    CastResult r{};
    float fraction = 0.0f;
    int steps = 0;
    while (true) {
        fraction += 0.5f;
        steps++;
        V3 pos = o + d * fraction;
        VoxBlock vb = get_voxel(w, pos);
        if (vb.block == 0) {
            int ix = f2i(pos.x), iy = f2i(pos.y), iz = f2i(pos.z);
            V3 box = {(float)((ix / 16) * 16), (float)((iy / 16) * 16), (float)((iz / 16) * 16)};
            box = box + corner;
            V3 temp = (-pos) * inv;
            V3 bc = box * inv + temp;
            float f = gmin(bc.x, gmin(bc.y, bc.z));
            f = gmax(f, 0.01f);
            fraction += f;
        }
        r.block = vb.block;
        if (vb.voxel != 0) {
            r.hit = true;
            r.coarse_voxel = vb.voxel;
            break;
        }
        if (pos.x < 0.0f || pos.y < 0.0f || pos.z < 0.0f ||
            pos.x >= wmax.x || pos.y >= wmax.y || pos.z >= wmax.z) break;
        if (fraction >= max_dist) break;
        if (steps >= max_steps) { r.capped = true; break; }
    }
    r.fraction = fraction;
    r.coarse_steps = steps;
    return r;
}

struct RefineResult {
    int vx, vy, vz;
    int voxel_id;
    int iters;
    int sx, sy, sz;       // final step flags (0/1)
    V3 normal;
    float fraction;
};

// refine DDA after a coarse hit (radiance.comp:246-288)
inline RefineResult refine(const World& w, V3 o, V3 d, float coarse_fraction) {
    RefineResult r{};
    V3 before = o + d * (coarse_fraction - 1.5f);
    int stx = d.x > 0.0f ? 1 : -1, sty = d.y > 0.0f ? 1 : -1, stz = d.z > 0.0f ? 1 : -1;
    V3 fl = {std::floor(before.x), std::floor(before.y), std::floor(before.z)};
    V3 inv = V3{1.0f, 1.0f, 1.0f} / d;
    V3 c1 = (fl - before) / d;
    V3 c2 = c1 + inv;
    V3 tmax = {gmax(c1.x, c2.x), gmax(c1.y, c2.y), gmax(c1.z, c2.z)};
    V3 tdelta = {std::fabs(inv.x), std::fabs(inv.y), std::fabs(inv.z)};  // 1/|d| == |1/d|
    int vx = f2i(before.x), vy = f2i(before.y), vz = f2i(before.z);
    int cur = get_voxel(w, V3{(float)vx, (float)vy, (float)vz}).voxel;
    float fsx = 0.0f, fsy = 0.0f, fsz = 0.0f;
    int it = 0;
    while ((it++ <= 4) && (cur == 0)) {
        int bx = (tmax.x <= tmax.y) && (tmax.x <= tmax.z);
        int by = (tmax.x >= tmax.y) && (tmax.y <= tmax.z);
        int bz = (tmax.z <= tmax.x) && (tmax.z <= tmax.y);
        fsx = (float)bx; fsy = (float)by; fsz = (float)bz;
        vx += stx * bx; vy += sty * by; vz += stz * bz;
        tmax = tmax + tdelta * V3{fsx, fsy, fsz};
        cur = get_voxel(w, V3{(float)vx, (float)vy, (float)vz}).voxel;
        r.iters++;
    }
    V3 fs = {fsx, fsy, fsz};
    r.normal = -(V3{(float)stx, (float)sty, (float)stz} * fs);
    V3 tfinal = tmax - tdelta;
    r.fraction = dot3(tfinal, fs);
    r.vx = vx; r.vy = vy; r.vz = vz;
    r.voxel_id = cur;
    r.sx = fsx != 0.0f; r.sy = fsy != 0.0f; r.sz = fsz != 0.0f;
    return r;
}

// Hit records report every NaN as the canonical quiet NaN, so records compare bytewise across
// machines whose NaN payloads differ.
inline float canon(float f) {
    if (f == f) return f;
    uint32_t u = 0x7FC00000u;
    float q;
    std::memcpy(&q, &u, 4);
    return q;
}

template <typename T> struct C3 { T x, y, z; };

// textureLod(radianceCache2read, (p+0.5)/world_size) with LINEAR filtering and REPEAT addressing
// (setup.cpp:75-81): texel coordinate u*size-0.5, exact weights, wrapped indices.
template <typename T>
C3<T> sample_trilinear(const World& w, const T* rad, V3 uvw) {
    const int n[3] = {w.X, w.Y, w.Z};
    float u[3] = {uvw.x * (float)w.X - 0.5f, uvw.y * (float)w.Y - 0.5f, uvw.z * (float)w.Z - 0.5f};
    int i0[3], i1[3];
    T a[3];
    for (int c = 0; c < 3; c++) {
        float fl = std::floor(u[c]);
        float fr = u[c] - fl;
        int ii = f2i(fl);
        i0[c] = smod(ii, n[c]);
        i1[c] = smod(smod(ii, n[c]) + 1, n[c]);
        a[c] = (T)fr;
    }
    auto tex = [&](int x, int y, int z) -> C3<T> {
        size_t idx = ((size_t)x + (size_t)w.X * ((size_t)y + (size_t)w.Y * (size_t)z)) * 3;
        return {rad[idx], rad[idx + 1], rad[idx + 2]};
    };
    auto lerp = [](C3<T> p, C3<T> q, T t) -> C3<T> {
        T s = (T)1 - t;
        return {p.x * s + q.x * t, p.y * s + q.y * t, p.z * s + q.z * t};
    };
    C3<T> c00 = lerp(tex(i0[0], i0[1], i0[2]), tex(i1[0], i0[1], i0[2]), a[0]);
    C3<T> c10 = lerp(tex(i0[0], i1[1], i0[2]), tex(i1[0], i1[1], i0[2]), a[0]);
    C3<T> c01 = lerp(tex(i0[0], i0[1], i1[2]), tex(i1[0], i0[1], i1[2]), a[0]);
    C3<T> c11 = lerp(tex(i0[0], i1[1], i1[2]), tex(i1[0], i1[1], i1[2]), a[0]);
    C3<T> c0 = lerp(c00, c10, a[1]);
    C3<T> c1 = lerp(c01, c11, a[1]);
    return lerp(c0, c1, a[2]);
}

struct RayOut {
    CastResult cast;
    RefineResult ref;
};

// trace_ray (radiance.comp:316-346)
template <typename T>
C3<T> trace(const World& w, const T* prev, V3 o, V3 d, float max_dist, int max_steps, RayOut* out) {
    CastResult c = coarse_march(w, o, d, max_dist, max_steps);
    out->cast = c;
    C3<T> light;
    if (c.hit) {
        RefineResult rf = refine(w, o, d, c.fraction);
        out->ref = rf;
        const float* m = w.mats + 6 * (size_t)rf.voxel_id;   // GetMat (radiance.comp:145-157)
        V3 hitpos = o + rf.fraction * d;
        V3 bp = (hitpos + rf.normal * 16.0f) / v3(16.0f);     // sample_radiance (:161-166)
        V3 uvw = (bp + v3(0.5f)) / V3{(float)w.X, (float)w.Y, (float)w.Z};
        C3<T> L = sample_trilinear<T>(w, prev, uvw);
        T cr = (T)m[0], cg = (T)m[1], cb = (T)m[2], e = (T)m[4];
        light.x = (T)0 + (L.x * cr + cr * e);
        light.y = (T)0 + (L.y * cg + cg * e);
        light.z = (T)0 + (L.z * cb + cb * e);
    } else {
        out->ref = RefineResult{};
        V3 gl = normalize3(V3{0.5f, 0.5f, -0.9f});
        float g = -dot3(d, gl);
        light = {(T)0, (T)0, (T)0};
        if (g > 0.95f) {
            T tg = (T)g;
            light.x = light.x + tg * ((T)0.9f * (T)3.0f);
            light.y = light.y + tg * ((T)0.9f * (T)3.0f);
            light.z = light.z + tg * ((T)0.6f * (T)3.0f);
        }
        light.x = light.x + ((T)0.53f * (T)0.1f);
        light.y = light.y + ((T)0.81f * (T)0.1f);
        light.z = light.z + ((T)0.92f * (T)0.1f);
    }
    return light;
}

template <typename T> inline T clamp01(T v) { return v > (T)0 ? (v < (T)1 ? v : (T)1) : (T)0; }

template <typename T>
int run_pass(const OracleWorld* ow, const int16_t* req, int n_req, const OracleParams* p,
             const T* prev, T* next, OracleHit* hits, OracleStats* stats, T* ray_light_out, int threads) {
    if (!ow || !p || !prev || !next || (n_req > 0 && !req)) return -1;
    if (p->rays < 32 || p->rays % 32 != 0 || p->size < 1 || p->shift < 0 || p->shift >= p->size)
        return -1;
    World w{ow->X, ow->Y, ow->Z, ow->grid, ow->palette, ow->n_slots, ow->materials};
    const size_t W = (size_t)w.X * w.Y * w.Z;
    std::memcpy(next, prev, W * 3 * sizeof(T));   // probes not in the list keep their value
    const int R = p->rays;
    const int groups = n_req / p->size;
    const int max_steps = (int)(2.0f * p->max_dist) + 2;
    std::vector<V3> dirs(R);
    for (int i = 0; i < R; i++) dirs[i] = spherical_fibonacci(i, R);
    uint64_t tot_steps = 0, tot_hits = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : tot_steps, tot_hits)
#endif
    for (int g = 0; g < groups; g++) {
        const int req_num = g * p->size + p->shift;
        const int px = req[4 * req_num], py = req[4 * req_num + 1], pz = req[4 * req_num + 2];
        std::vector<C3<T>> ray_light(R);
        for (int r = 0; r < R; r++) {
            uint32_t gid = (uint32_t)g * (uint32_t)R + (uint32_t)r;
            U3 rs = {gid + (uint32_t)p->time_seed, 0u + (uint32_t)p->time_seed, (uint32_t)p->time_seed};
            V3 center = V3{(float)px * 16.0f, (float)py * 16.0f, (float)pz * 16.0f} + v3(8.0f);
            V3 r1 = hash33(rs); rs.x++;
            V3 jit = 0.1f * ((r1 - v3(0.5f)) * 2.0f);
            V3 d = normalize3(dirs[r] + jit);
            V3 o = center + d * 6.0f;
            V3 r2 = hash33(rs); rs.x++;
            o = o + (r2 - v3(0.5f)) * 2.0f;
            if (r % 2 != 0) d = -d;
            RayOut ro;
            ray_light[r] = trace<T>(w, prev, o, d, p->max_dist, max_steps, &ro);
            if (ray_light_out) {
                T* lo = ray_light_out + 3 * ((size_t)g * R + r);
                lo[0] = ray_light[r].x; lo[1] = ray_light[r].y; lo[2] = ray_light[r].z;
            }
            const CastResult& c = ro.cast;
            tot_steps += (uint64_t)c.coarse_steps + (c.hit ? 1u + (uint64_t)ro.ref.iters : 0u);
            tot_hits += c.hit ? 1u : 0u;
            if (hits) {
                OracleHit& h = hits[(size_t)g * R + r];
                std::memset(&h, 0, sizeof h);
                h.block = (int16_t)c.block;
                h.coarse_steps = (uint16_t)c.coarse_steps;
                h.coarse_voxel = (uint8_t)c.coarse_voxel;
                h.flags = (c.hit ? 0x01 : 0) | (c.capped ? 0x10 : 0);
                if (c.hit) {
                    h.voxel[0] = ro.ref.vx; h.voxel[1] = ro.ref.vy; h.voxel[2] = ro.ref.vz;
                    h.voxel_id = (uint8_t)ro.ref.voxel_id;
                    h.refine_steps = (uint8_t)ro.ref.iters;
                    h.flags |= (ro.ref.sx ? 0x02 : 0) | (ro.ref.sy ? 0x04 : 0) | (ro.ref.sz ? 0x08 : 0);
                    h.fraction = canon(ro.ref.fraction);
                } else {
                    h.fraction = canon(c.fraction);
                }
            }
        }
        // subgroupAdd over each 32-ray subgroup in xor-butterfly order, /32, then the mean of
        // the subgroup values summed in subgroup order (radiance.comp:386-408)
        C3<T> acc = {(T)0, (T)0, (T)0};
        for (int k = 0; k < R / 32; k++) {
            C3<T> v[32];
            for (int l = 0; l < 32; l++) v[l] = ray_light[32 * k + l];
            for (int m = 16; m >= 1; m >>= 1)
                for (int l = 0; l < m; l++) {
                    v[l].x = v[l].x + v[l + m].x;
                    v[l].y = v[l].y + v[l + m].y;
                    v[l].z = v[l].z + v[l + m].z;
                }
            acc.x = acc.x + v[0].x / (T)32;
            acc.y = acc.y + v[0].y / (T)32;
            acc.z = acc.z + v[0].z / (T)32;
        }
        const T nsub = (T)(R / 32);
        acc.x = acc.x / nsub; acc.y = acc.y / nsub; acc.z = acc.z / nsub;
        // store_probe (radiance.comp:349-354): clamp old, mix, UNORM clamp on store
        if (px < 0 || py < 0 || pz < 0 || px >= w.X || py >= w.Y || pz >= w.Z) continue;
        size_t pi = ((size_t)px + (size_t)w.X * ((size_t)py + (size_t)w.Y * (size_t)pz)) * 3;
        const T a = (T)p->blend;
        const T one_minus_a = (T)(1.0f - p->blend);
        T accv[3] = {acc.x, acc.y, acc.z};
        for (int c = 0; c < 3; c++) {
            T old = prev[pi + c];
            old = old < (T)0 ? (T)0 : old;              // clamp(old, 0, 1) = min(max(x,0),1)
            old = (T)1 < old ? (T)1 : old;
            T nv = old * one_minus_a + accv[c] * a;     // mix(x,y,a) = x*(1-a) + y*a
            nv = clamp01(nv);
            // imageStore into the rgb10_a2 image: code = round to nearest even of v*1023, read
            // back as code/1023
            if (p->unorm10) nv = std::nearbyint(nv * (T)1023) / (T)1023;
            next[pi + c] = nv;
        }
    }
    if (stats) {
        stats->probes = (uint64_t)groups;
        stats->rays = (uint64_t)groups * R;
        stats->steps = tot_steps;
        stats->hits = tot_hits;
    }
    return 0;
}

}  // namespace

extern "C" {

int oracle_pass_f32(const OracleWorld* w, const int16_t* req, int n, const OracleParams* p,
                    const float* prev, float* next, OracleHit* hits, OracleStats* stats, float* ray_light,
                    int threads) {
    return run_pass<float>(w, req, n, p, prev, next, hits, stats, ray_light, threads);
}

int oracle_pass_f64(const OracleWorld* w, const int16_t* req, int n, const OracleParams* p,
                    const double* prev, double* next, OracleHit* hits, OracleStats* stats, double* ray_light,
                    int threads) {
    return run_pass<double>(w, req, n, p, prev, next, hits, stats, ray_light, threads);
}

// hash33 of one seed (known-answer tests)
void oracle_hash33(uint32_t x, uint32_t y, uint32_t z, float* out3) {
    V3 r = hash33(U3{x, y, z});
    out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
}

int oracle_direction_table(int n, float* xyz) {
    if (n < 1 || !xyz) return -1;
    for (int i = 0; i < n; i++) {
        V3 d = spherical_fibonacci(i, n);
        xyz[3 * i] = d.x; xyz[3 * i + 1] = d.y; xyz[3 * i + 2] = d.z;
    }
    return 0;
}

// One ray traced from an explicit origin and direction (hand-built known-answer cases).
int oracle_trace_ray(const OracleWorld* ow, const float* prev, const float* o3, const float* d3,
                     float max_dist, float* light3, OracleHit* hit) {
    World w{ow->X, ow->Y, ow->Z, ow->grid, ow->palette, ow->n_slots, ow->materials};
    RayOut ro;
    int max_steps = (int)(2.0f * max_dist) + 2;
    C3<float> L = trace<float>(w, prev, V3{o3[0], o3[1], o3[2]}, V3{d3[0], d3[1], d3[2]},
                               max_dist, max_steps, &ro);
    light3[0] = L.x; light3[1] = L.y; light3[2] = L.z;
    if (hit) {
        std::memset(hit, 0, sizeof *hit);
        hit->block = (int16_t)ro.cast.block;
        hit->coarse_steps = (uint16_t)ro.cast.coarse_steps;
        hit->coarse_voxel = (uint8_t)ro.cast.coarse_voxel;
        hit->flags = (ro.cast.hit ? 1 : 0) | (ro.cast.capped ? 0x10 : 0);
        if (ro.cast.hit) {
            hit->voxel[0] = ro.ref.vx; hit->voxel[1] = ro.ref.vy; hit->voxel[2] = ro.ref.vz;
            hit->voxel_id = (uint8_t)ro.ref.voxel_id;
            hit->refine_steps = (uint8_t)ro.ref.iters;
            hit->flags |= (ro.ref.sx ? 2 : 0) | (ro.ref.sy ? 4 : 0) | (ro.ref.sz ? 8 : 0);
            hit->fraction = canon(ro.ref.fraction);
        } else {
            hit->fraction = canon(ro.cast.fraction);
        }
    }
    return 0;
}

// shift_radiance (internal_render.cpp:1218-1335): the two image copies amount to
// new(p) = old(p + shift) for p in the destination box [dst, dst + world - |shift|), where
// dst = shift >= 0 ? 0 : -shift per axis, and old(p) elsewhere.  The reference returns early
// only for |shift.x| >= world.x; a larger y or z shift gives it a negative extent, which is
// defined here as no change.  vol: W*3 floats, updated in place.
int oracle_shift(int X, int Y, int Z, float* vol, int sx, int sy, int sz) {
    if (std::abs(sx) >= X || std::abs(sy) >= Y || std::abs(sz) >= Z) return 0;
    const int off[3] = {sx, sy, sz}, size[3] = {X, Y, Z};
    int src[3], dst[3], ext[3];
    for (int a = 0; a < 3; a++) {
        src[a] = off[a] >= 0 ? off[a] : 0;     // process_axis (:1234-1251)
        dst[a] = off[a] >= 0 ? 0 : -off[a];
        ext[a] = size[a] - std::abs(off[a]);   // intersection_size (:1268)
    }
    std::vector<float> tmp((size_t)ext[0] * ext[1] * ext[2] * 3);
    for (int z = 0; z < ext[2]; z++)           // copy to temp (:1299-1301)
        for (int y = 0; y < ext[1]; y++)
            for (int x = 0; x < ext[0]; x++)
                for (int c = 0; c < 3; c++)
                    tmp[(((size_t)z * ext[1] + y) * ext[0] + x) * 3 + c] =
                        vol[(((size_t)(z + src[2]) * Y + (y + src[1])) * X + (x + src[0])) * 3 + c];
    for (int z = 0; z < ext[2]; z++)           // copy back at dst (:1312-1316)
        for (int y = 0; y < ext[1]; y++)
            for (int x = 0; x < ext[0]; x++)
                for (int c = 0; c < 3; c++)
                    vol[(((size_t)(z + dst[2]) * Y + (y + dst[1])) * X + (x + dst[0])) * 3 + c] =
                        tmp[(((size_t)z * ext[1] + y) * ext[0] + x) * 3 + c];
    return 0;
}

// The radiance consumer's gather, diffuse.frag:24-90 (sample_probe + sample_radiance(position,
// normal)) at n points (x, y, z, nx, ny, nz) of a W*3 float volume; out: n*3 floats.
// texelFetch past the volume reads 0 (the probe index is clamped to [0, world_size], one past
// the last probe).  ivec3(floor(...)) converts like f2i; '/' on ints is OpSDiv (truncation).
int oracle_gather(int X, int Y, int Z, const float* vol, const float* pts, int n, float* out) {
    auto clampi = [](int v, int lo, int hi) { return std::min(std::max(v, lo), hi); };
    auto probe = [&](int px, int py, int pz) -> V3 {   // sample_probe (:25-33)
        px = clampi(px, 0, X); py = clampi(py, 0, Y); pz = clampi(pz, 0, Z);
        V3 v{0.0f, 0.0f, 0.0f};
        if (px < X && py < Y && pz < Z) {
            const float* t = vol + (((size_t)pz * Y + py) * X + px) * 3;
            v = V3{t[0], t[1], t[2]};
        }
        return V3{gmin(gmax(v.x, 0.0f), 2.0f), gmin(gmax(v.y, 0.0f), 2.0f), gmin(gmax(v.z, 0.0f), 2.0f)};
    };
    for (int k = 0; k < n; k++) {
        const float* q = pts + 6 * (size_t)k;
        const V3 pos{q[0], q[1], q[2]}, nrm{q[3], q[4], q[5]};
        const int zx = clampi(f2i(std::floor(pos.x - 8.0f)) / 16, 0, X);   // (:42)
        const int zy = clampi(f2i(std::floor(pos.y - 8.0f)) / 16, 0, Y);
        const int zz = clampi(f2i(std::floor(pos.z - 8.0f)) / 16, 0, Z);
        const V3 zp{(float)zx * 16.0f + 8.0f, (float)zy * 16.0f + 8.0f, (float)zz * 16.0f + 8.0f};   // (:43)
        const V3 d = (pos - zp) * 0.0625f;   // (pos - zero_probe_pos) / 16.0, exact as * 1/16
        const V3 alpha{gmin(gmax(d.x, 0.0f), 1.0f), gmin(gmax(d.y, 0.0f), 1.0f), gmin(gmax(d.z, 0.0f), 1.0f)};
        float tw = 0.0f;
        V3 tc{0.0f, 0.0f, 0.0f};
        for (int i = 0; i < 8; i++) {
            const int ox = i & 1, oy = (i >> 1) & 1, oz = (i >> 2) & 1;   // (:50)
            const V3 off{(float)ox, (float)oy, (float)oz};
            const V3 pp = zp + off * 16.0f;   // (:55)
            const V3 dir = normalize3(pp - pos);   // (:57-58)
            const V3 one{1.0f, 1.0f, 1.0f};
            const V3 tri = (one - alpha) * (one - off) + alpha * off;   // mix(1-alpha, alpha, offset) (:60)
            float w = (tri.x * tri.y) * tri.z;   // (:61)
            w = w * gmin(gmax(dot3(dir, nrm), 0.1f), 1.0f);   // (:70-74)
            const V3 c = probe(zx + ox, zy + oy, zz + oz);   // (:81)
            w = gmax(1e-7f, w);   // (:84)
            tw = tw + w;
            tc = tc + V3{w * c.x, w * c.y, w * c.z};
        }
        out[3 * (size_t)k] = tc.x / tw;   // (:89)
        out[3 * (size_t)k + 1] = tc.y / tw;
        out[3 * (size_t)k + 2] = tc.z / tw;
    }
    return 0;
}

// One frame of the model producers: start_blockify / blockify_mesh (internal_render.cpp:977-1070),
// exec_copies' palette part (:1375-1451) and map_mesh + shaders/map.comp (:1484-1520, map.comp:33-67).
// grid: W ids, updated in place to the blockified world; pal: n_slots*4096 voxels, updated in place.
// models: voxel arrays x-fastest with sizes msize[3*i..]; rot: 4 floats (x,y,z,w) and shift: 3 floats
// per mesh.  Returns -2 when the temporary slots run past n_slots (nothing changed), 0 otherwise.
// Definitions where the reference is undefined: a negative static id gets an empty temporary block;
// map invocations that target one palette voxel (truncation aliases world voxels near and below 0
// into block 0) run one after another in linear order, x fastest, and the meshes in order; glm's
// inverse of [R|s] is [R^T | -R^T s] in double.
int oracle_blockify(int X, int Y, int Z, int16_t* grid, uint8_t* pal, int n_slots, int static_blocks,
                    const uint8_t* const* models, const int* msize, const float* rot, const float* shift, int n) {
    struct Box { float mn[3], mx[3]; };
    auto rotation = [](const float* q, float r[3][3]) {   // glm::mat3_cast, r[col][row]
        const float x = q[0], y = q[1], z = q[2], w = q[3];
        r[0][0] = 1.0f - 2.0f * (y * y + z * z); r[0][1] = 2.0f * (x * y + w * z); r[0][2] = 2.0f * (x * z - w * y);
        r[1][0] = 2.0f * (x * y - w * z); r[1][1] = 1.0f - 2.0f * (x * x + z * z); r[1][2] = 2.0f * (y * z + w * x);
        r[2][0] = 2.0f * (x * z + w * y); r[2][1] = 2.0f * (y * z - w * x); r[2][2] = 1.0f - 2.0f * (x * x + y * y);
    };
    auto aabb = [](const float r[3][3], const float* t, const int* size) {   // get_shift (:988-1012)
        const float b[3] = {(float)(size[0] - 1), (float)(size[1] - 1), (float)(size[2] - 1)};
        Box box;
        for (int a = 0; a < 3; a++) { box.mn[a] = std::numeric_limits<float>::max(); box.mx[a] = std::numeric_limits<float>::lowest(); }
        for (int k = 0; k < 8; k++) {
            // the corner order of get_shift: 0, y, yz, z, x, xy, xyz, xz
            static const int sel[8][3] = {{0,0,0},{0,1,0},{0,1,1},{0,0,1},{1,0,0},{1,1,0},{1,1,1},{1,0,1}};
            const float c[3] = {sel[k][0] ? b[0] : 0.0f, sel[k][1] ? b[1] : 0.0f, sel[k][2] ? b[2] : 0.0f};
            for (int a = 0; a < 3; a++) {
                // glm dmat4 * dvec4: (m0*v0 + m1*v1) + (m2*v2 + m3*v3), in double
                const double p = ((double)r[0][a] * (double)c[0] + (double)r[1][a] * (double)c[1]) +
                                 ((double)r[2][a] * (double)c[2] + (double)t[a] * 1.0);
                const float f = (float)p;
                box.mn[a] = gmin(box.mn[a], f);
                box.mx[a] = gmax(box.mx[a], f);
            }
        }
        return box;
    };
    const size_t W = (size_t)X * Y * Z;
    std::vector<int16_t> cur(grid, grid + W);
    std::vector<std::pair<int, int>> copies;
    int counter = static_blocks;
    const int ws[3] = {X, Y, Z};
    for (int i = 0; i < n; i++) {
        float r[3][3];
        rotation(rot + 4 * i, r);
        const Box box = aabb(r, shift + 3 * i, msize + 3 * i);
        int lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(std::max(((int)box.mn[a] - 1) / 16, 0), ws[a] - 1);
            hi[a] = std::min(std::max(((int)box.mx[a] + 1) / 16, 0), ws[a] - 1);
        }
        for (int z = lo[2]; z <= hi[2]; z++)
            for (int y = lo[1]; y <= hi[1]; y++)
                for (int x = lo[0]; x <= hi[0]; x++) {
                    int16_t& b = cur[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * z)];
                    if (b < static_blocks) {
                        if (counter >= n_slots || counter > 32767) return -2;
                        if (b > 0) copies.push_back({b, counter});
                        b = (int16_t)counter++;
                    }
                }
    }
    std::memcpy(grid, cur.data(), W * sizeof(int16_t));
    std::memset(pal + (size_t)static_blocks * 4096, 0, (size_t)(n_slots - static_blocks) * 4096);
    for (auto& cp : copies) std::memcpy(pal + (size_t)cp.second * 4096, pal + (size_t)cp.first * 4096, 4096);
    for (int i = 0; i < n; i++) {
        float r[3][3];
        rotation(rot + 4 * i, r);
        const float* t = shift + 3 * i;
        const int* size = msize + 3 * i;
        const Box box = aabb(r, t, size);
        int org[3], dims[3];
        for (int a = 0; a < 3; a++) {
            org[a] = (int)std::floor(box.mn[a]);
            dims[a] = ((int)std::ceil(box.mx[a]) - org[a] + 3) / 4 * 4;
        }
        float inv[3][4];   // rows of [R^T | -R^T t]
        for (int row = 0; row < 3; row++) {
            for (int col = 0; col < 3; col++) inv[row][col] = r[row][col];
            inv[row][3] = (float)(-(((double)r[row][0] * t[0] + (double)r[row][1] * t[1]) + (double)r[row][2] * t[2]));
        }
        for (int gz = 0; gz < dims[2]; gz++)
                for (int gy = 0; gy < dims[1]; gy++)
                    for (int gx = 0; gx < dims[0]; gx++) {
                        const float wv[3] = {((float)gx + 0.5f) + (float)org[0], ((float)gy + 0.5f) + (float)org[1],
                                             ((float)gz + 0.5f) + (float)org[2]};
                        int iw[3], im[3];
                        for (int a = 0; a < 3; a++) {
                            iw[a] = f2i(wv[a]);
                            const float mv = ((inv[a][0] * wv[0] + inv[a][1] * wv[1]) + inv[a][2] * wv[2]) + inv[a][3];
                            im[a] = f2i(mv);
                        }
                        const int bx = iw[0] / 16, by = iw[1] / 16, bz = iw[2] / 16;
                        int id = 0;
                        if (bx >= 0 && by >= 0 && bz >= 0 && bx < X && by < Y && bz < Z)
                            id = cur[(size_t)bx + (size_t)X * ((size_t)by + (size_t)Y * bz)];
                        if (id < static_blocks) continue;
                        int v = 0;
                        if (im[0] >= 0 && im[1] >= 0 && im[2] >= 0 && im[0] < size[0] && im[1] < size[1] && im[2] < size[2])
                            v = models[i][(size_t)im[0] + (size_t)size[0] * ((size_t)im[1] + (size_t)size[1] * im[2])];
                        if (v == 0 || id >= n_slots) continue;
                        pal[(size_t)id * 4096 + smod(iw[0], 16) + 16 * smod(iw[1], 16) + 256 * smod(iw[2], 16)] = (uint8_t)v;
                    }
    }
    return 0;
}

// Update-list rule of update_radiance (internal_render.cpp:1142-1168): every block whose
// clamped 3x3x3 neighbourhood sums to > 0 in z,y,x scan order, then each special request
// that the rule did not already list (specials are not de-duplicated among themselves).
int oracle_update_list(const OracleWorld* ow, const int16_t* specials, int n_specials,
                       int16_t* out, int cap, int* n_out) {
    const int X = ow->X, Y = ow->Y, Z = ow->Z;
    std::vector<uint8_t> set((size_t)X * Y * Z, 0);
    int n = 0;
    auto push = [&](int x, int y, int z, int wv) {
        if (n < cap) {
            out[4 * n] = (int16_t)x; out[4 * n + 1] = (int16_t)y;
            out[4 * n + 2] = (int16_t)z; out[4 * n + 3] = (int16_t)wv;
        }
        n++;
    };
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++)
            for (int x = 0; x < X; x++) {
                int sum = 0;
                for (int dz = -1; dz <= 1; dz++)
                    for (int dy = -1; dy <= 1; dy++)
                        for (int dx = -1; dx <= 1; dx++) {
                            int tx = std::min(std::max(x + dx, 0), X - 1);
                            int ty = std::min(std::max(y + dy, 0), Y - 1);
                            int tz = std::min(std::max(z + dz, 0), Z - 1);
                            sum += ow->grid[(size_t)tx + (size_t)X * ((size_t)ty + (size_t)Y * tz)];
                        }
                if (sum > 0) {
                    push(x, y, z, 0);
                    set[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * z)] = 1;
                }
            }
    for (int i = 0; i < n_specials; i++) {
        int x = specials[4 * i], y = specials[4 * i + 1], z = specials[4 * i + 2];
        if (x < 0 || y < 0 || z < 0 || x >= X || y >= Y || z >= Z) return -1;
        if (!set[(size_t)x + (size_t)X * ((size_t)y + (size_t)Y * z)])
            push(x, y, z, specials[4 * i + 3]);
    }
    *n_out = n;
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
