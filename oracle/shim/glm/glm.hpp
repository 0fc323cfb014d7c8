// Minimal, project-written stand-in for the few glm types and operations that the
// reference's CPU solver sources use (component-wise vec arithmetic, length2, max).
// This is test infrastructure for building the reference's own CPU path headless;
// it is not part of the product. Only what those sources reference is provided.
//
// Semantics follow the published glm conventions that matter for the hot path:
//  * vecN components are plain floats, value-initialised to zero;
//  * binary operators act component-wise, scalar operands broadcast;
//  * vec4(v3, w) packs a vec3 and a scalar.
#ifndef NBODY_SHIM_GLM_HPP
#define NBODY_SHIM_GLM_HPP

#include <cmath>
#include <cstdint>

namespace glm {

struct vec2 {
    float x = 0.f, y = 0.f;
    vec2() = default;
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    float &operator[](int i) { return (&x)[i]; }
    const float &operator[](int i) const { return (&x)[i]; }
};

struct vec3 {
    float x = 0.f, y = 0.f, z = 0.f;
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float &operator[](int i) { return (&x)[i]; }
    const float &operator[](int i) const { return (&x)[i]; }
};

struct alignas(16) vec4 {
    float x = 0.f, y = 0.f, z = 0.f, w = 0.f;
    vec4() = default;
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3 &v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float &operator[](int i) { return (&x)[i]; }
    const float &operator[](int i) const { return (&x)[i]; }

    vec4 &operator+=(const vec4 &o) { x += o.x; y += o.y; z += o.z; w += o.w; return *this; }
    vec4 &operator-=(const vec4 &o) { x -= o.x; y -= o.y; z -= o.z; w -= o.w; return *this; }
    vec4 &operator*=(float s) { x *= s; y *= s; z *= s; w *= s; return *this; }
    vec4 &operator/=(float s) { x /= s; y /= s; z /= s; w /= s; return *this; }
};

inline vec4 operator+(const vec4 &a, const vec4 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline vec4 operator-(const vec4 &a, const vec4 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
inline vec4 operator*(const vec4 &a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
inline vec4 operator*(float s, const vec4 &a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }
inline vec4 operator*(const vec4 &a, const vec4 &b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
inline vec4 operator/(const vec4 &a, float s) { return {a.x / s, a.y / s, a.z / s, a.w / s}; }

inline vec3 operator+(const vec3 &a, const vec3 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(const vec3 &a, const vec3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(const vec3 &a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline vec3 operator*(float s, const vec3 &a) { return {s * a.x, s * a.y, s * a.z}; }
inline vec3 operator/(const vec3 &a, float s) { return {a.x / s, a.y / s, a.z / s}; }

struct ivec2 { int x = 0, y = 0; ivec2() = default; ivec2(int a, int b) : x(a), y(b) {} };
struct uvec2 { unsigned x = 0, y = 0; uvec2() = default; uvec2(unsigned a, unsigned b) : x(a), y(b) {} };

// Column-major square matrices: declared only so that shader-uniform setter
// prototypes in the reference headers compile; no arithmetic is needed.
struct mat2 { vec2 c[2]; vec2 &operator[](int i) { return c[i]; } const vec2 &operator[](int i) const { return c[i]; } };
struct mat3 { vec3 c[3]; vec3 &operator[](int i) { return c[i]; } const vec3 &operator[](int i) const { return c[i]; } };
struct mat4 { vec4 c[4]; vec4 &operator[](int i) { return c[i]; } const vec4 &operator[](int i) const { return c[i]; } };

inline float max(float a, float b) { return a < b ? b : a; }
inline float dot(const vec3 &a, const vec3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(const vec3 &v) { return std::sqrt(dot(v, v)); }
inline float distance(const vec3 &a, const vec3 &b) { return length(a - b); }
inline vec3 normalize(const vec3 &v) { return v * (1.0f / length(v)); }
inline vec3 cross(const vec3 &a, const vec3 &b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
inline float min(float a, float b) { return b < a ? b : a; }

}  // namespace glm

#endif
