/*
 * glsl_compat.h — just enough of GLSL 4.60 to compile the reference's
 * clustered-forward compute shaders, its frustum-culling compute shader and
 * the clustered lookup and direct lighting of its fragment shader as C++ on
 * the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build.py rewrites
 * HelloVulkan/Shaders/ClusteredForward/AABBGenerator.comp, LightCulling.comp,
 * HelloVulkan/Shaders/FrustumCulling.comp and the lookup and lighting
 * statements of ClusteredForward/Scene.frag (with Radiance.glsl and
 * PBR/PBRHeader.glsl) mechanically (interface blocks -> globals, float
 * literals -> float, swizzles -> calls) into oracle/_ref/, includes this
 * header in front of them, and builds a library that runs the shaders' own
 * code one invocation at a time.  Running the workgroups serially in index
 * order makes LightCulling's atomicAdd hand out offsets in cluster order, so
 * the outputs are directly comparable with the oracle and the CUDA path.
 *
 * Semantics are GLSL's, with its implementation-defined parts pinned the same
 * way as include/cf_pinned_math.h: mat4 * vec4 and dot summed left to right
 * with no FMA (build with -ffp-contract=off), pow = cf_pow_pinned,
 * log2 = cf_log2_pinned, sqrt correctly rounded, normalize(v) = v / length(v)
 * with length(v) = sqrt(dot(v, v)), min/max/clamp/mix by their GLSL
 * definitions.
 */
#ifndef CF_GLSL_COMPAT_H
#define CF_GLSL_COMPAT_H

#include <cstdint>
#include <cstdlib>

#include "cf_pinned_math.h"

namespace glsl {

typedef uint32_t uint;

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    vec2(float a, float b) : x(a), y(b) {}
};

struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](uint i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](uint i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec4 {
    float x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec3 xyz() const { return vec3(x, y, z); }
    float& operator[](uint i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](uint i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

/* Column-major: c[col]. */
struct mat4 {
    vec4 c[4];
};

struct uvec3 {
    uint x, y, z;
    uvec3() : x(0), y(0), z(0) {}
    /* GLSL's uvec3(a, b, c) converts each argument: float -> uint truncates. */
    template <class A, class B, class Cc>
    uvec3(A a, B b, Cc c) : x(uint(a)), y(uint(b)), z(uint(c)) {}
};

inline vec4 operator*(const mat4& m, const vec4& v)
{
    vec4 r;
    r.x = ((m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z) + m.c[3].x * v.w;
    r.y = ((m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z) + m.c[3].y * v.w;
    r.z = ((m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z) + m.c[3].z * v.w;
    r.w = ((m.c[0].w * v.x + m.c[1].w * v.y) + m.c[2].w * v.z) + m.c[3].w * v.w;
    return r;
}
inline vec4 operator/(const vec4& a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator-(float s, const vec3& a) { return vec3(s - a.x, s - a.y, s - a.z); }
inline vec3& operator+=(vec3& a, const vec3& b) { a = a + b; return a; }
inline vec3& operator*=(vec3& a, float s) { a = a * s; return a; }

/* dot: products summed x, y, z (, w) left to right. */
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(const vec4& a, const vec4& b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline float sqrt(float x) { return cf_fsqrt(x); }
inline float length(const vec3& v) { return cf_fsqrt(dot(v, v)); }
inline vec3 normalize(const vec3& v) { return v / length(v); }
inline float log2(float x) { return cf_log2_pinned(x); }

inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float pow(float x, float y) { return cf_pow_pinned(x, y); }
/* clamp(x, lo, hi) = min(max(x, lo), hi); mix(x, y, a) = x * (1 - a) + y * a. */
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }

/* Shader storage array with GLSL's .length().  An index past the end aborts
 * (the compute shaders never make one), unless `robust` is set: then it reads
 * a zero record, as Vulkan's robustBufferAccess2 defines out-of-bounds reads
 * (the fragment shader's lookup of a fragment beyond the last depth slice). */
template <class T>
struct Buffer {
    T* data = nullptr;
    uint n = 0;
    bool robust = false;
    T& operator[](uint i)
    {
        if (i >= n) {
            if (!robust) std::abort();
            static thread_local T zero;
            zero = T();
            return zero;
        }
        return data[i];
    }
    int length() const { return int(n); }
};

inline uint atomicAdd(uint& mem, uint v) { return __atomic_fetch_add(&mem, v, __ATOMIC_RELAXED); }

extern thread_local uvec3 gl_WorkGroupID;
extern thread_local uvec3 gl_NumWorkGroups;
extern thread_local uvec3 gl_GlobalInvocationID;
extern thread_local vec4 gl_FragCoord;

}  // namespace glsl

#endif /* CF_GLSL_COMPAT_H */
