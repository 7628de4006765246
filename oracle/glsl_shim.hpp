// glsl_shim.hpp — TEST INFRASTRUCTURE.  The GLSL 4.50 types, operators and built-ins that
// shaders/radiance.comp uses, as C++, so oracle/build_ref.py can compile the reference shader's
// own source on the CPU.  Compiled with -fsingle-precision-constant (GLSL literals are float)
// and -ffp-contract=off.
//
// Definitions where GLSL leaves the result implementation-defined or undefined (each one is the
// same definition the CPU oracle and the CUDA kernels use):
//   - float -> int truncates toward zero, saturates, NaN -> 0;
//   - int '%' is SPIR-V OpSMod (sign of the divisor), int '/' truncates (OpSDiv);
//   - min(x,y) = y < x ? y : x; max(x,y) = x < y ? y : x; clamp = min(max(x,lo),hi);
//   - normalize(v) = v * (1/sqrt(dot(v,v))), dot summed x, y, z in order;
//   - mix(x,y,a) = x*(1-a) + y*a;
//   - cos/sin evaluated in double and rounded to float;
//   - texel fetches out of range return 0;
//   - textureLod on the radiance volume: LINEAR + REPEAT, texel coordinate u*size-0.5, exact
//     FP32 weights, lerp in x, then y, then z;
//   - imageStore to the rgb10_a2 volume clamps to [0,1] (NaN -> 0); with the 10-bit storage
//     switched on (lumref_set_unorm10) it also rounds each channel to the format's code,
//     round-to-nearest-even of v*1023, and keeps code/1023 (the value a later fetch returns);
//   - subgroupAdd sums the 32 lanes in xor-butterfly order (16, 8, 4, 2, 1).
#pragma once

#include <cmath>
#include <csetjmp>
#include <cstdint>
#include <cstring>
#include <initializer_list>

namespace lumref {

typedef unsigned int uint;

// ---------------------------------------------------------------- swizzle proxies
template <class V, class S, int N, int A, int B> struct Swz2 {
    S v[N];
    operator V() const { return V(v[A], v[B]); }
};
template <class V, class S, int N, int A, int B, int C> struct Swz3 {
    S v[N];
    operator V() const { return V(v[A], v[B], v[C]); }
};

struct ivec2;
struct ivec3;
struct uvec3;
struct vec3;

struct bvec3 {
    bool x, y, z;
    bvec3() { x = y = z = false; }
    explicit bvec3(bool a) { x = y = z = a; }
    bvec3(bool a, bool b, bool c) { x = a; y = b; z = c; }
};

struct vec2 {
    union {
        struct { float x, y; };
        Swz2<vec2, float, 2, 0, 1> xy;
    };
    vec2() { x = y = 0.0f; }
    explicit vec2(float a) { x = y = a; }
    vec2(float a, float b) { x = a; y = b; }
};

struct ivec2 {
    int x, y;
    ivec2() { x = y = 0; }
    ivec2(int a, int b) { x = a; y = b; }
};

struct ivec3 {
    union {
        struct { int x, y, z; };
        Swz2<ivec2, int, 3, 0, 1> xy;
    };
    ivec3() { x = y = z = 0; }
    explicit ivec3(int a) { x = y = z = a; }
    ivec3(int a, int b, int c) { x = a; y = b; z = c; }
    explicit ivec3(const vec3& v);
    explicit ivec3(const bvec3& b) { x = b.x; y = b.y; z = b.z; }
    explicit ivec3(const uvec3& u);
    ivec3& operator+=(const ivec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
};

struct uvec3 {
    union {
        struct { uint x, y, z; };
        Swz3<uvec3, uint, 3, 1, 2, 0> yzx;
        Swz3<uvec3, uint, 3, 0, 1, 2> xyz;
    };
    uvec3() { x = y = z = 0u; }
    uvec3(uint a, uint b, uint c) { x = a; y = b; z = c; }
    uvec3(const ivec2& a, int b) { x = (uint)a.x; y = (uint)a.y; z = (uint)b; }
};

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
    };
    vec3() { x = y = z = 0.0f; }
    explicit vec3(float a) { x = y = z = a; }
    vec3(float a, float b, float c) { x = a; y = b; z = c; }
    vec3(const ivec3& v) { x = (float)v.x; y = (float)v.y; z = (float)v.z; }   // GLSL implicit int->float
    explicit vec3(const uvec3& v) { x = (float)v.x; y = (float)v.y; z = (float)v.z; }
    explicit vec3(const bvec3& v) { x = v.x ? 1.0f : 0.0f; y = v.y ? 1.0f : 0.0f; z = v.z ? 1.0f : 0.0f; }
    explicit vec3(const vec2& a, float b) { x = a.x; y = a.y; z = b; }
    explicit vec3(const vec2& a, const vec2& b) { x = a.x; y = a.y; z = b.x; }
    vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3& operator/=(float s) { x = x / s; y = y / s; z = z / s; return *this; }
};

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        Swz3<vec3, float, 4, 0, 1, 2> xyz;
        Swz3<vec3, float, 4, 0, 1, 2> rgb;
    };
    vec4() { x = y = z = w = 0.0f; }
    vec4(float a, float b, float c, float d) { x = a; y = b; z = c; w = d; }
    vec4(const vec3& v, float d) { x = v.x; y = v.y; z = v.z; w = d; }
};

struct ivec4 {
    union {
        struct { int x, y, z, w; };
        struct { int r, g, b, a; };
    };
    ivec4() { x = y = z = w = 0; }
};

struct uvec4 {
    union {
        struct { uint x, y, z, w; };
        struct { uint r, g, b, a; };
    };
    uvec4() { x = y = z = w = 0u; }
};

struct i8vec4 {
    union {
        struct { int8_t x, y, z, w; };
        Swz3<ivec3, int8_t, 4, 0, 1, 2> xyz;
    };
};

// float -> int: toward zero, saturating, NaN -> 0
inline int f2i(float f) {
    if (!(f == f)) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int)f;
}
inline ivec3::ivec3(const vec3& v) { x = f2i(v.x); y = f2i(v.y); z = f2i(v.z); }
inline ivec3::ivec3(const uvec3& u) { x = (int)u.x; y = (int)u.y; z = (int)u.z; }

// ---------------------------------------------------------------- operators
inline vec2 operator*(vec2 a, vec2 b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator-(float s, vec2 a) { return vec2(s - a.x, s - a.y); }
inline vec2 sqrt(vec2 a) { return vec2(std::sqrt(a.x), std::sqrt(a.y)); }

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator+(vec3 a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(vec3 a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(float s, vec3 a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(ivec3 a, vec3 b) { return vec3(a) * b; }

inline ivec2 operator+(ivec2 a, int s) { return ivec2(a.x + s, a.y + s); }
inline ivec3 operator+(ivec3 a, ivec3 b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator+(ivec3 a, int s) { return ivec3(a.x + s, a.y + s, a.z + s); }
inline ivec3 operator*(ivec3 a, ivec3 b) { return ivec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline ivec3 operator*(ivec3 a, int s) { return ivec3(a.x * s, a.y * s, a.z * s); }
inline ivec3 operator*(int s, ivec3 a) { return ivec3(s * a.x, s * a.y, s * a.z); }
inline ivec3 operator/(ivec3 a, int s) { return ivec3(a.x / s, a.y / s, a.z / s); }   // OpSDiv
inline int smod(int a, int b) {
    int r = a % b;
    if (r != 0 && ((r < 0) != (b < 0))) r += b;
    return r;
}
inline ivec3 operator%(ivec3 a, int s) { return ivec3(smod(a.x, s), smod(a.y, s), smod(a.z, s)); }  // OpSMod

// An int specialization constant.  C++ gives `int % int` truncated semantics; GLSL's signed `%`
// is OpSMod, so integer constants carry this type and `int % constant` follows SPIR-V.
struct glsl_int {
    int v;
    glsl_int(int x) : v(x) {}
    operator int() const { return v; }
};
inline int operator%(int a, glsl_int b) { return smod(a, b.v); }
inline int operator/(int a, glsl_int b) { return a / b.v; }

inline uvec3 operator>>(uvec3 a, uint s) { return uvec3(a.x >> s, a.y >> s, a.z >> s); }
inline uvec3 operator^(uvec3 a, uvec3 b) { return uvec3(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z); }
inline uvec3 operator*(uvec3 a, uint s) { return uvec3(a.x * s, a.y * s, a.z * s); }

// ---------------------------------------------------------------- built-ins
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline int min(int x, int y) { return y < x ? y : x; }
inline int max(int x, int y) { return x < y ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline float clamp(float x, int lo, int hi) { return clamp(x, (float)lo, (float)hi); }   // genType, float, float
inline vec3 clamp(vec3 v, float lo, float hi) { return vec3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi)); }
inline float floor(float x) { return std::floor(x); }
inline vec3 floor(vec3 v) { return vec3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline float abs(float x) { return std::fabs(x); }
inline vec3 abs(vec3 v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float cos(float x) { return (float)std::cos((double)x); }
inline float sin(float x) { return (float)std::sin((double)x); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 normalize(vec3 v) { return v * (1.0f / std::sqrt(dot(v, v))); }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline vec3 mix(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }
inline bvec3 greaterThan(vec3 a, vec3 b) { return bvec3(a.x > b.x, a.y > b.y, a.z > b.z); }
inline bvec3 lessThan(vec3 a, vec3 b) { return bvec3(a.x < b.x, a.y < b.y, a.z < b.z); }
inline bvec3 greaterThanEqual(vec3 a, vec3 b) { return bvec3(a.x >= b.x, a.y >= b.y, a.z >= b.z); }
inline bool any(bvec3 b) { return b.x || b.y || b.z; }

// ---------------------------------------------------------------- resources
// An invocation is suspended at a subgroup operation or a barrier, or abandoned when its march
// exceeds the fetch budget (only a NaN fraction can), by a longjmp back to the harness (every frame
// it skips is trivially destructible).
constexpr int kSuspend = 1, kRunaway = 2;
inline std::jmp_buf g_jump;

struct ShimState {
    long long block_fetches = 0;
    long long fetch_limit = 0;
    ivec3 last_block;
    ivec3 last_palette;
    bool unorm10 = false;      // imageStore rounds to the 10-bit UNORM codes
};
inline ShimState g_shim;

struct isampler3D { const int16_t* data = nullptr; int X = 0, Y = 0, Z = 0; };
struct usampler3D { const uint8_t* pal = nullptr; int n_slots = 0; };     // 1024x1024x16 image view
struct sampler2D { const float* mats = nullptr; };                         // 6 x 256
struct sampler3D { const float* rgb = nullptr; int X = 0, Y = 0, Z = 0; };
struct image3D { float* rgb = nullptr; int X = 0, Y = 0, Z = 0; };

inline ivec4 texelFetch(const isampler3D& s, ivec3 p, int) {
    if (++g_shim.block_fetches > g_shim.fetch_limit) std::longjmp(g_jump, kRunaway);
    g_shim.last_block = p;
    ivec4 r;
    if (p.x >= 0 && p.y >= 0 && p.z >= 0 && p.x < s.X && p.y < s.Y && p.z < s.Z)
        r.x = s.data[(size_t)p.x + (size_t)s.X * ((size_t)p.y + (size_t)s.Y * (size_t)p.z)];
    return r;
}
inline uvec4 texelFetch(const usampler3D& s, ivec3 p, int) {
    g_shim.last_palette = p;
    uvec4 r;
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= 1024 || p.y >= 1024 || p.z >= 16) return r;
    const int slot = (p.y / 16) * 64 + p.x / 16;
    if (slot >= s.n_slots) return r;
    r.x = s.pal[(size_t)slot * 4096 + (size_t)(p.x % 16) + 16 * (p.y % 16) + 256 * p.z];
    return r;
}
inline vec4 texelFetch(const sampler2D& s, ivec2 p, int) {
    vec4 r;
    if (p.x < 0 || p.y < 0 || p.x >= 6 || p.y >= 256) return r;
    r.x = s.mats[6 * (size_t)p.y + p.x];
    return r;
}
inline vec4 texelFetch(const sampler3D& s, ivec3 p, int) {
    vec4 r;
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= s.X || p.y >= s.Y || p.z >= s.Z) return r;
    const float* t = s.rgb + 3 * ((size_t)p.x + (size_t)s.X * ((size_t)p.y + (size_t)s.Y * (size_t)p.z));
    return vec4(t[0], t[1], t[2], 1.0f);
}
inline vec4 textureLod(const sampler3D& s, vec3 uvw, float) {
    const int n[3] = {s.X, s.Y, s.Z};
    const float u[3] = {uvw.x * (float)s.X - 0.5f, uvw.y * (float)s.Y - 0.5f, uvw.z * (float)s.Z - 0.5f};
    int i0[3], i1[3];
    float a[3];
    for (int c = 0; c < 3; c++) {
        const float fl = std::floor(u[c]);
        a[c] = u[c] - fl;
        i0[c] = smod(f2i(fl), n[c]);
        i1[c] = smod(i0[c] + 1, n[c]);
    }
    auto tex = [&](int x, int y, int z) {
        const float* t = s.rgb + 3 * ((size_t)x + (size_t)s.X * ((size_t)y + (size_t)s.Y * (size_t)z));
        return vec3(t[0], t[1], t[2]);
    };
    auto lerp = [](vec3 p, vec3 q, float t) {
        const float k = 1.0f - t;
        return vec3(p.x * k + q.x * t, p.y * k + q.y * t, p.z * k + q.z * t);
    };
    const vec3 c00 = lerp(tex(i0[0], i0[1], i0[2]), tex(i1[0], i0[1], i0[2]), a[0]);
    const vec3 c10 = lerp(tex(i0[0], i1[1], i0[2]), tex(i1[0], i1[1], i0[2]), a[0]);
    const vec3 c01 = lerp(tex(i0[0], i0[1], i1[2]), tex(i1[0], i0[1], i1[2]), a[0]);
    const vec3 c11 = lerp(tex(i0[0], i1[1], i1[2]), tex(i1[0], i1[1], i1[2]), a[0]);
    const vec3 c = lerp(lerp(c00, c10, a[1]), lerp(c01, c11, a[1]), a[2]);
    return vec4(c, 1.0f);
}
inline float unorm(float v) { return v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f; }
inline void imageStore(const image3D& im, ivec3 p, vec4 v) {
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= im.X || p.y >= im.Y || p.z >= im.Z) return;
    float* t = im.rgb + 3 * ((size_t)p.x + (size_t)im.X * ((size_t)p.y + (size_t)im.Y * (size_t)p.z));
    t[0] = unorm(v.x); t[1] = unorm(v.y); t[2] = unorm(v.z);
    if (g_shim.unorm10)
        for (int c = 0; c < 3; c++) t[c] = std::nearbyint(t[c] * 1023.0f) / 1023.0f;
}

// ---------------------------------------------------------------- compute built-ins
// One workgroup runs as: (1) every invocation up to subgroupAdd, whose argument is collected;
// (2) the elected invocation of each subgroup up to barrier(), after writing shared memory;
// (3) the elected invocations again, past the barrier.  Re-running an invocation repeats the
// same deterministic work (the shader reseeds its RNG at the start of main).
enum Phase { kCollect, kToBarrier, kPastBarrier };
struct Invocation {
    Phase phase = kCollect;
    int lane = 0;
    vec3 collected[1024];
    vec3 sums[32];
};
inline Invocation g_inv;
inline uvec3 gl_GlobalInvocationID;
inline int gl_SubgroupSize = 32;
inline int gl_SubgroupID = 0;

inline vec3 subgroupAdd(vec3 v) {
    if (g_inv.phase == kCollect) {
        g_inv.collected[gl_SubgroupID * 32 + g_inv.lane] = v;
        std::longjmp(g_jump, kSuspend);
    }
    return g_inv.sums[gl_SubgroupID];
}
inline bool subgroupElect() { return g_inv.lane == 0; }
inline void barrier() {
    if (g_inv.phase == kToBarrier) std::longjmp(g_jump, kSuspend);
}

}  // namespace lumref
