// ORACLE PIN — test infrastructure only.  A small GLSL 4.60 subset in C++ so
// that the reference's own shader sources (data/shaders/*.glsl, *.rgen,
// *.rchit, *.rmiss, blur.comp) compile unchanged in substance as C++ after
// the mechanical rewrite of oracle/glsl_ref/translate.py.  Nothing here is
// product code.  The ray-tracing built-ins are driven by oracle/glsl_ref/
// harness.cpp, which plays the role of the Vulkan pipeline.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

namespace glsl {

typedef uint32_t uint;

struct vec2; struct vec3; struct vec4; struct ivec2; struct ivec3; struct uvec2; struct uvec3;
template <class T, int K> struct VecOf;
template <> struct VecOf<float, 2> { using type = vec2; };
template <> struct VecOf<float, 3> { using type = vec3; };
template <> struct VecOf<float, 4> { using type = vec4; };
template <> struct VecOf<int, 2> { using type = ivec2; };
template <> struct VecOf<int, 3> { using type = ivec3; };
template <> struct VecOf<uint, 2> { using type = uvec2; };
template <> struct VecOf<uint, 3> { using type = uvec3; };

// swizzle proxy: N components of type T viewed through indices I...
template <class T, int N, int... I> struct Sw {
    T e[N];
    using V = typename VecOf<T, sizeof...(I)>::type;
    operator V() const { return V(e[I]...); }
    Sw& operator=(const V& o) {
        int k = 0;
        ((e[I] = o[k++]), ...);
        return *this;
    }
};

#define GLSL_VEC_COMMON(NAME, T, N)                                                  \
    T& operator[](int i) { return e[i]; }                                            \
    T operator[](int i) const { return e[i]; }

struct vec2 {
    union {
        struct { float x, y; };
        float e[2];
    };
    vec2() : x(0), y(0) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2(float a, const vec2& b) : x(a), y(b.x) {}  // GLSL consumes components in order
    explicit vec2(const uvec2& u);
    GLSL_VEC_COMMON(vec2, float, 2)
};
struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        float e[3];
        Sw<float, 3, 0, 1, 2> xyz;
        Sw<float, 3, 0, 1, 2> rgb;
        Sw<float, 3, 0, 1> xy;
    };
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    GLSL_VEC_COMMON(vec3, float, 3)
};
struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        float e[4];
        Sw<float, 4, 0, 1, 2> xyz;
        Sw<float, 4, 0, 1, 2> rgb;
        Sw<float, 4, 0, 1> xy;
        Sw<float, 4, 0, 1> rg;
    };
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    GLSL_VEC_COMMON(vec4, float, 4)
};
struct ivec2 {
    union {
        struct { int x, y; };
        int e[2];
    };
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}
    explicit ivec2(const uvec2& u);
    GLSL_VEC_COMMON(ivec2, int, 2)
};
struct ivec3 {
    union {
        struct { int x, y, z; };
        int e[3];
    };
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    GLSL_VEC_COMMON(ivec3, int, 3)
};
struct uvec2 {
    union {
        struct { uint x, y; };
        uint e[2];
    };
    uvec2() : x(0), y(0) {}
    uvec2(uint a, uint b) : x(a), y(b) {}
    GLSL_VEC_COMMON(uvec2, uint, 2)
};
struct uvec3 {
    union {
        struct { uint x, y, z; };
        uint e[3];
        Sw<uint, 3, 0, 1> xy;
    };
    uvec3() : x(0), y(0), z(0) {}
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    GLSL_VEC_COMMON(uvec3, uint, 3)
};
inline vec2::vec2(const uvec2& u) : x((float)u.x), y((float)u.y) {}
inline ivec2::ivec2(const uvec2& u) : x((int)u.x), y((int)u.y) {}

// ---- arithmetic (non-template so swizzle proxies convert implicitly) ----
#define GLSL_BINOPS(V, N)                                                                    \
    inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] + b.e[i]; return r; } \
    inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] - b.e[i]; return r; } \
    inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] * b.e[i]; return r; } \
    inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] / b.e[i]; return r; } \
    inline V operator+(const V& a, float s) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] + s; return r; }        \
    inline V operator-(const V& a, float s) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] - s; return r; }        \
    inline V operator*(const V& a, float s) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] * s; return r; }        \
    inline V operator/(const V& a, float s) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] / s; return r; }        \
    inline V operator+(float s, const V& a) { V r; for (int i = 0; i < N; i++) r.e[i] = s + a.e[i]; return r; }        \
    inline V operator-(float s, const V& a) { V r; for (int i = 0; i < N; i++) r.e[i] = s - a.e[i]; return r; }        \
    inline V operator*(float s, const V& a) { V r; for (int i = 0; i < N; i++) r.e[i] = s * a.e[i]; return r; }        \
    inline V operator-(const V& a) { V r; for (int i = 0; i < N; i++) r.e[i] = -a.e[i]; return r; }                     \
    inline V& operator+=(V& a, const V& b) { a = a + b; return a; }                                                     \
    inline V& operator*=(V& a, const V& b) { a = a * b; return a; }                                                     \
    inline V& operator*=(V& a, float s) { a = a * s; return a; }                                                        \
    inline V& operator/=(V& a, float s) { a = a / s; return a; }                                                        \
    inline bool operator==(const V& a, const V& b) { for (int i = 0; i < N; i++) if (a.e[i] != b.e[i]) return false; return true; } \
    inline float dot(const V& a, const V& b) { float s = a.e[0] * b.e[0]; for (int i = 1; i < N; i++) s = s + a.e[i] * b.e[i]; return s; } \
    inline float length(const V& a) { return std::sqrt(dot(a, a)); }                                                   \
    inline V normalize(const V& a) { return a / length(a); }                                                            \
    inline V min(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.e[i] = b.e[i] < a.e[i] ? b.e[i] : a.e[i]; return r; } \
    inline V max(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] < b.e[i] ? b.e[i] : a.e[i]; return r; } \
    inline V min(const V& a, float b) { V r; for (int i = 0; i < N; i++) r.e[i] = b < a.e[i] ? b : a.e[i]; return r; } \
    inline V max(const V& a, float b) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] < b ? b : a.e[i]; return r; } \
    inline V mix(const V& a, const V& b, float t) { V r; for (int i = 0; i < N; i++) r.e[i] = a.e[i] * (1.0f - t) + b.e[i] * t; return r; } \
    inline V pow(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r.e[i] = std::pow(a.e[i], b.e[i]); return r; }

GLSL_BINOPS(vec2, 2)
GLSL_BINOPS(vec3, 3)
GLSL_BINOPS(vec4, 4)

// ---- scalar built-ins (GLSL 4.60 §8) ----
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline float pow(float a, float b) { return std::pow(a, b); }
inline float sqrt(float a) { return std::sqrt(a); }
inline float cos(float a) { return std::cos(a); }
inline float sin(float a) { return std::sin(a); }
inline float abs(float a) { return std::fabs(a); }
inline float atan(float y, float x) { return std::atan2(y, x); }
inline float asin(float a) { return std::asin(a); }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline vec3 reflect(const vec3& I, const vec3& N) { return I - 2.0f * dot(N, I) * N; }
inline vec3 refract(const vec3& I, const vec3& N, float eta) {
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return vec3(0.0f);
    return eta * I - (eta * d + std::sqrt(k)) * N;
}

// ---- matrices (column-major, m[c] is column c) ----
struct mat3 {
    vec3 c[3];
    mat3() {}
    explicit mat3(const struct mat4& m);
};
struct mat4 {
    vec4 c[4];
    mat4() {}
};
inline mat3::mat3(const mat4& m) {
    for (int i = 0; i < 3; i++) c[i] = vec3(m.c[i].x, m.c[i].y, m.c[i].z);
}
inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 r;
    for (int i = 0; i < 4; i++) {
        float s = m.c[0].e[i] * v.x;
        s = s + m.c[1].e[i] * v.y;
        s = s + m.c[2].e[i] * v.z;
        s = s + m.c[3].e[i] * v.w;
        r.e[i] = s;
    }
    return r;
}
inline vec3 operator*(const mat3& m, const vec3& v) {
    vec3 r;
    for (int i = 0; i < 3; i++) {
        float s = m.c[0].e[i] * v.x;
        s = s + m.c[1].e[i] * v.y;
        s = s + m.c[2].e[i] * v.z;
        r.e[i] = s;
    }
    return r;
}
inline mat4 transpose(const mat4& m) {
    mat4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.c[i].e[j] = m.c[j].e[i];
    return r;
}
mat4 inverse(const mat4& m);  // harness.cpp (double-precision cofactors, rounded to float)

// ---- resources ----
template <class T> struct RuntimeArray {
    T* data = nullptr;
    int n = 0;
    T& operator[](int i) { return data[i]; }
    int length() const { return n; }
};
template <class T> struct Array {
    std::vector<T> v;
    T& operator[](int i) { return v[i]; }
};
struct sampler2D {
    const float* texels = nullptr;  // rgba float per texel
    int w = 0, h = 0;
    bool repeat = false;
};
vec4 texture(const sampler2D& s, const vec2& uv);
struct image2D {
    void* data = nullptr;
    int w = 0, h = 0;
    bool unorm8 = true;  // R8/RGBA8 storage (first channel kept), else float
    bool bgra8 = false;  // with unorm8: four channels stored as bytes B, G, R, A (a B8G8R8A8 image)
};
vec4 imageLoad(const image2D& im, const ivec2& p);
void imageStore(image2D& im, const ivec2& p, const vec4& v);

struct accelerationStructureEXT {};
constexpr uint gl_RayFlagsOpaqueEXT = 1u;
constexpr uint gl_RayFlagsTerminateOnFirstHitEXT = 4u;
constexpr uint gl_RayFlagsSkipClosestHitShaderEXT = 8u;
void traceRayEXT(const accelerationStructureEXT&, uint flags, uint mask, uint sbt_offset, uint sbt_stride,
                 uint miss_index, const vec3& origin, float tmin, const vec3& dir, float tmax, int payload);

// built-in inputs, set by the harness before each shader invocation
extern uvec3 gl_LaunchIDEXT, gl_LaunchSizeEXT, gl_GlobalInvocationID;
extern vec3 gl_WorldRayOriginEXT, gl_WorldRayDirectionEXT;
extern float gl_HitTEXT;
extern int gl_PrimitiveID, gl_InstanceCustomIndexEXT;

// payload registry: each shader namespace registers its payload variables
struct PayloadTable {
    void* ptr[4] = {};
    size_t size[4] = {};
    void* in_ptr = nullptr;
    size_t in_size = 0;
};
struct PayloadReg {
    PayloadReg(PayloadTable& t, int loc, void* p, size_t n) { t.ptr[loc] = p; t.size[loc] = n; }
};
struct PayloadInReg {
    PayloadInReg(PayloadTable& t, void* p, size_t n) { t.in_ptr = p; t.in_size = n; }
};

}  // namespace glsl
