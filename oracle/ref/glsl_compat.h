// glsl_compat.h — the subset of GLSL 4.60 that WaterCube's compute shaders use, as C++, so that
// the shaders under assets/ compile unchanged (after make_ref.py strips their layout
// qualifiers) into a host library. TEST INFRASTRUCTURE ONLY (it builds the parity reference).
//
// This header deliberately includes no standard header: libstdc++'s <cmath> would bring
// double-precision pow/sqrt overloads into scope and change the shaders' float arithmetic.
// Built-in semantics (identical to the ones stated at the top of oracle/wc_oracle.cpp):
//   length(v) = sqrt(fma(z,z,fma(y,y,x*x))); pow = powf; IEEE '/', sqrt; min/max/clamp as the
//   GLSL spec words them; ivec3(vec3) truncates with NaN -> 0 and saturation; v.length() == 3;
//   atomicAdd is a relaxed fetch-add (serial dispatch order makes Sort's ranks stable).
#ifndef WC_GLSL_COMPAT_H
#define WC_GLSL_COMPAT_H

namespace glsl {

typedef unsigned int uint;

struct bvec3 {
    bool x, y, z;
};

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
    int length() const { return 3; }  // GLSL: number of components
    vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3& operator-=(const vec3& o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
    vec3& operator*=(float s) { x = x * s; y = y * s; z = z * s; return *this; }
};

inline int f2i(float f) {
    if (!(f == f)) return 0;
    if (f >= 2147483648.0f) return 2147483647;
    if (f <= -2147483648.0f) return (-2147483647 - 1);
    return (int)f;
}

struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    explicit ivec3(int s) : x(s), y(s), z(s) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x(f2i(v.x)), y(f2i(v.y)), z(f2i(v.z)) {}
};

struct uvec3 {
    uint x, y, z;
    uvec3() : x(0), y(0), z(0) {}
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }

inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline float max(int x, float y) { return max((float)x, y); }
inline float max(float x, int y) { return max(x, (float)y); }
inline int min(int x, int y) { return y < x ? y : x; }
inline int max(int x, int y) { return x < y ? y : x; }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 clamp(const vec3& v, const vec3& lo, const vec3& hi) { return min(max(v, lo), hi); }
inline ivec3 clamp(const ivec3& v, const ivec3& lo, const ivec3& hi) {
    return ivec3(min(max(v.x, lo.x), hi.x), min(max(v.y, lo.y), hi.y), min(max(v.z, lo.z), hi.z));
}

inline float pow(float x, float y) { return __builtin_powf(x, y); }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float length(const vec3& v) { return __builtin_sqrtf(__builtin_fmaf(v.z, v.z, __builtin_fmaf(v.y, v.y, v.x * v.x))); }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

inline bvec3 lessThan(const ivec3& a, const ivec3& b) { return bvec3{a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bvec3 greaterThanEqual(const ivec3& a, const ivec3& b) { return bvec3{a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bool any(const bvec3& b) { return b.x || b.y || b.z; }

inline uint atomicAdd(uint& mem, uint v) { return __atomic_fetch_add(&mem, v, __ATOMIC_RELAXED); }

}  // namespace glsl

// The invocation id of the running shader instance; one per host thread.
extern thread_local glsl::uvec3 gl_GlobalInvocationID;

#endif
