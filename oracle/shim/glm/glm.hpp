// Minimal stand-in for the glm subset that the reference's chunk-extraction
// translation units use (vec3 / ivec3 arithmetic, dot, cross, length,
// normalize, isnan).  Test infrastructure only: it exists so that the
// reference's own DMCChunk / MeshProcessor / ImplicitSampler sources can be
// compiled unmodified as the pinning oracle.
//
// Semantics chosen (glm itself is not vendored by the reference, so no version
// is pinned):
//   * component-wise IEEE single-precision operators, division is a true
//     division per component (vec / scalar divides each component);
//   * dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z;
//   * normalize(v) = v * (1 / sqrt(dot(v, v)));
//   * cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y);
//   * default constructors zero-initialise (the reference relies on
//     uninitialised members in a few places; zero is the defined choice).
#pragma once
#include <cmath>
#include <cstdint>

namespace glm {

struct vec3 {
  float x, y, z;
  inline vec3() : x(0.f), y(0.f), z(0.f) {}
  inline explicit vec3(float s) : x(s), y(s), z(s) {}
  inline vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  template <class T> inline vec3(const T& o) : x((float)o.x), y((float)o.y), z((float)o.z) {}
  inline float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  inline const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  inline vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
  inline vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  inline vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
  inline vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};

struct ivec3 {
  int x, y, z;
  inline ivec3() : x(0), y(0), z(0) {}
  inline explicit ivec3(int s) : x(s), y(s), z(s) {}
  inline ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
  inline int& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  inline const int& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  inline ivec3& operator+=(const ivec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
};

struct vec2 { float x, y; inline vec2() : x(0.f), y(0.f) {} inline vec2(float a, float b) : x(a), y(b) {} };
struct vec4 {
  float x, y, z, w;
  inline vec4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
  inline vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator+(float s, const vec3& a) { return vec3(s + a.x, s + a.y, s + a.z); }
inline bool operator==(const vec3& a, const vec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(const vec3& a, const vec3& b) { return !(a == b); }

inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator-(const ivec3& a, const ivec3& b) { return ivec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline ivec3 operator*(const ivec3& a, int s) { return ivec3(a.x * s, a.y * s, a.z * s); }
inline bool operator==(const ivec3& a, const ivec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

inline float dot(const vec3& a, const vec3& b) {
  float t0 = a.x * b.x, t1 = a.y * b.y, t2 = a.z * b.z;
  return (t0 + t1) + t2;
}
inline vec3 cross(const vec3& a, const vec3& b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float distance(const vec3& a, const vec3& b) { return length(b - a); }
inline vec3 normalize(const vec3& v) { float inv = 1.0f / std::sqrt(dot(v, v)); return v * inv; }
template <class T> inline bool isnan(T v) { return std::isnan(v); }
inline vec3 floor(const vec3& v) { return vec3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline vec3 abs(const vec3& v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)); }

}  // namespace glm
