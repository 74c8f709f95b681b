// ORACLE — test infrastructure only. A small GLSL execution environment in C++ with every floating-point
// type in FP64, so that the reference's shader sources (assets/shaders/*.glsl, *.rgen, *.rchit, *.rmiss,
// *.comp) compile and run on the CPU as the reference implementation of the DDGI probe update.
//
// Vector types carry GLSL swizzles as proxy members; every builtin is a non-template overload, so swizzle
// proxies convert implicitly wherever a vector is expected, as in GLSL. `float` is mapped to double by
// the stage translation units (ref_shaders.cpp). Texture sampling is exact FP64 bilinear with REPEAT
// addressing (the sampler the probe pass binds, PipelineUtil.h:98-112); the hardware's fixed-point
// filter weights are not modelled.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

namespace glsl {

typedef unsigned int uint;

template <class Out, class T, int N, int... I>
struct Swz;

#define GLSL_SWZ2(T, N, name, a, b) Swz<vec<T, 2>, T, N, a, b> name;
#define GLSL_SWZ3(T, N, name, a, b, c) Swz<vec<T, 3>, T, N, a, b, c> name;

template <class T, int N>
struct vec;

template <class T>
struct vec<T, 2> {
  union {
    struct { T x, y; };
    struct { T r, g; };
    T e[2];
    GLSL_SWZ2(T, 2, yx, 1, 0)
    GLSL_SWZ2(T, 2, xy, 0, 1)
  };
  vec() : x(0), y(0) {}
  explicit vec(T s) : x(s), y(s) {}
  vec(T a, T b) : x(a), y(b) {}
  template <class U>
  vec(const vec<U, 2>& o) : x(T(o.x)), y(T(o.y)) {}
  template <class U, int M, int... I, class = std::enable_if_t<!std::is_same<U, T>::value>>
  explicit vec(const Swz<vec<U, 2>, U, M, I...>& s) : vec(vec<U, 2>(s)) {}
  template <class U>
  explicit vec(const vec<U, 3>& o) : x(T(o.x)), y(T(o.y)) {}
  template <class U>
  explicit vec(const vec<U, 4>& o) : x(T(o.x)), y(T(o.y)) {}
  vec(const vec& o) { std::memcpy(e, o.e, sizeof(e)); }
  vec& operator=(const vec& o) { std::memcpy(e, o.e, sizeof(e)); return *this; }
  T& operator[](int i) { return e[i]; }
  T operator[](int i) const { return e[i]; }
};

template <class T>
struct vec<T, 3> {
  union {
    struct { T x, y, z; };
    struct { T r, g, b; };
    T e[3];
    GLSL_SWZ2(T, 3, xy, 0, 1)
    GLSL_SWZ2(T, 3, rg, 0, 1)
    GLSL_SWZ2(T, 3, yx, 1, 0)
    GLSL_SWZ2(T, 3, yz, 1, 2)
    GLSL_SWZ2(T, 3, gb, 1, 2)
    GLSL_SWZ2(T, 3, xz, 0, 2)
    GLSL_SWZ3(T, 3, xyz, 0, 1, 2)
    GLSL_SWZ3(T, 3, rgb, 0, 1, 2)
  };
  vec() : x(0), y(0), z(0) {}
  explicit vec(T s) : x(s), y(s), z(s) {}
  vec(T a, T b, T c) : x(a), y(b), z(c) {}
  vec(const vec<T, 2>& a, T c) : x(a.x), y(a.y), z(c) {}
  vec(T a, const vec<T, 2>& b) : x(a), y(b.x), z(b.y) {}
  template <class U>
  vec(const vec<U, 3>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
  template <class U, int M, int... I, class = std::enable_if_t<!std::is_same<U, T>::value>>
  explicit vec(const Swz<vec<U, 3>, U, M, I...>& s) : vec(vec<U, 3>(s)) {}
  template <class U>
  explicit vec(const vec<U, 4>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
  vec(const vec& o) { std::memcpy(e, o.e, sizeof(e)); }
  vec& operator=(const vec& o) { std::memcpy(e, o.e, sizeof(e)); return *this; }
  T& operator[](int i) { return e[i]; }
  T operator[](int i) const { return e[i]; }
};

template <class T>
struct vec<T, 4> {
  union {
    struct { T x, y, z, w; };
    struct { T r, g, b, a; };
    T e[4];
    GLSL_SWZ2(T, 4, xy, 0, 1)
    GLSL_SWZ2(T, 4, rg, 0, 1)
    GLSL_SWZ2(T, 4, zw, 2, 3)
    GLSL_SWZ2(T, 4, yz, 1, 2)
    GLSL_SWZ2(T, 4, gb, 1, 2)
    GLSL_SWZ2(T, 4, xz, 0, 2)
    GLSL_SWZ3(T, 4, xyz, 0, 1, 2)
    GLSL_SWZ3(T, 4, rgb, 0, 1, 2)
    GLSL_SWZ3(T, 4, yzw, 1, 2, 3)
  };
  vec() : x(0), y(0), z(0), w(0) {}
  explicit vec(T s) : x(s), y(s), z(s), w(s) {}
  vec(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
  vec(const vec<T, 3>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec(const vec<T, 2>& v, T c, T d) : x(v.x), y(v.y), z(c), w(d) {}
  vec(const vec<T, 2>& v, const vec<T, 2>& u) : x(v.x), y(v.y), z(u.x), w(u.y) {}
  vec(T a, const vec<T, 3>& v) : x(a), y(v.x), z(v.y), w(v.z) {}
  template <class U>
  vec(const vec<U, 4>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
  vec(const vec& o) { std::memcpy(e, o.e, sizeof(e)); }
  vec& operator=(const vec& o) { std::memcpy(e, o.e, sizeof(e)); return *this; }
  T& operator[](int i) { return e[i]; }
  T operator[](int i) const { return e[i]; }
};

// Swizzle proxy: shares the parent's storage, converts to and assigns from the swizzled vector type.
template <class Out, class T, int N, int... I>
struct Swz {
  T e[N];
  operator Out() const { return Out(e[I]...); }
  Swz& operator=(const Out& o) {
    int k = 0;
    for (int idx : {I...}) e[idx] = o.e[k++];
    return *this;
  }
  Swz& operator/=(T s) {
    for (int idx : {I...}) e[idx] /= s;
    return *this;
  }
  Swz& operator*=(T s) {
    for (int idx : {I...}) e[idx] *= s;
    return *this;
  }
  Swz& operator+=(const Out& o) {
    int k = 0;
    for (int idx : {I...}) e[idx] += o.e[k++];
    return *this;
  }
  Out operator()() const { return Out(*this); }
};

typedef vec<double, 2> dvec2;
typedef vec<double, 3> dvec3;
typedef vec<double, 4> dvec4;
typedef vec<int, 2> ivec2;
typedef vec<int, 3> ivec3;
typedef vec<int, 4> ivec4;
typedef vec<uint, 2> uvec2;
typedef vec<uint, 3> uvec3;
typedef vec<uint, 4> uvec4;
typedef vec<bool, 3> bvec3;

// ---- component-wise operators (non-template: swizzle proxies convert implicitly) -----------------------
#define GLSL_BINOPS(V, S, N)                                                                      \
  inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] + b.e[i]; return r; } \
  inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] - b.e[i]; return r; } \
  inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] * b.e[i]; return r; } \
  inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] / b.e[i]; return r; } \
  inline V operator+(const V& a, S s) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] + s; return r; }             \
  inline V operator-(const V& a, S s) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] - s; return r; }             \
  inline V operator*(const V& a, S s) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] * s; return r; }             \
  inline V operator/(const V& a, S s) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] / s; return r; }             \
  inline V operator+(S s, const V& a) { V r; for (int i = 0; i < N; ++i) r.e[i] = s + a.e[i]; return r; }             \
  inline V operator-(S s, const V& a) { V r; for (int i = 0; i < N; ++i) r.e[i] = s - a.e[i]; return r; }             \
  inline V operator*(S s, const V& a) { V r; for (int i = 0; i < N; ++i) r.e[i] = s * a.e[i]; return r; }             \
  inline V operator/(S s, const V& a) { V r; for (int i = 0; i < N; ++i) r.e[i] = s / a.e[i]; return r; }             \
  inline V operator-(const V& a) { V r; for (int i = 0; i < N; ++i) r.e[i] = -a.e[i]; return r; }                      \
  inline V& operator+=(V& a, const V& b) { a = a + b; return a; }                                                       \
  inline V& operator-=(V& a, const V& b) { a = a - b; return a; }                                                       \
  inline V& operator*=(V& a, const V& b) { a = a * b; return a; }                                                       \
  inline V& operator/=(V& a, const V& b) { a = a / b; return a; }                                                       \
  inline V& operator+=(V& a, S s) { a = a + s; return a; }                                                              \
  inline V& operator-=(V& a, S s) { a = a - s; return a; }                                                              \
  inline V& operator*=(V& a, S s) { a = a * s; return a; }                                                              \
  inline V& operator/=(V& a, S s) { a = a / s; return a; }                                                              \
  inline bool operator==(const V& a, const V& b) { for (int i = 0; i < N; ++i) if (a.e[i] != b.e[i]) return false; return true; } \
  inline bool operator!=(const V& a, const V& b) { return !(a == b); }

GLSL_BINOPS(dvec2, double, 2)
GLSL_BINOPS(dvec3, double, 3)
GLSL_BINOPS(dvec4, double, 4)
GLSL_BINOPS(ivec2, int, 2)
GLSL_BINOPS(ivec3, int, 3)
GLSL_BINOPS(ivec4, int, 4)
GLSL_BINOPS(uvec2, uint, 2)
GLSL_BINOPS(uvec3, uint, 3)

// ---- matrices (column-major, GLSL conventions) --------------------------------------------------------
struct mat3;
// mat4x3: 4 columns of 3 rows (gl_ObjectToWorldEXT / gl_WorldToObjectEXT)
struct mat4x3 {
  dvec3 c[4];
  dvec3& operator[](int i) { return c[i]; }
  const dvec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
  dvec4 c[4];
  mat4() {}
  explicit mat4(double d) { for (int i = 0; i < 4; ++i) { c[i] = dvec4(0.0); c[i].e[i] = d; } }
  dvec4& operator[](int i) { return c[i]; }
  const dvec4& operator[](int i) const { return c[i]; }
};
struct mat3 {
  dvec3 c[3];
  mat3() {}
  explicit mat3(double d) { for (int i = 0; i < 3; ++i) { c[i] = dvec3(0.0); c[i].e[i] = d; } }
  mat3(double a0, double a1, double a2, double b0, double b1, double b2, double d0, double d1, double d2) {
    c[0] = dvec3(a0, a1, a2); c[1] = dvec3(b0, b1, b2); c[2] = dvec3(d0, d1, d2);
  }
  mat3(const dvec3& a, const dvec3& b, const dvec3& d) { c[0] = a; c[1] = b; c[2] = d; }
  explicit mat3(const mat4& m) { for (int i = 0; i < 3; ++i) c[i] = dvec3(m.c[i].x, m.c[i].y, m.c[i].z); }
  explicit mat3(const mat4x3& m) { for (int i = 0; i < 3; ++i) c[i] = m.c[i]; }
  dvec3& operator[](int i) { return c[i]; }
  const dvec3& operator[](int i) const { return c[i]; }
};
inline dvec3 operator*(const mat3& m, const dvec3& v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z; }
inline dvec4 operator*(const mat4& m, const dvec4& v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3] * v.w; }
inline mat4 operator*(const mat4& a, const mat4& b) {
  mat4 r;
  for (int i = 0; i < 4; ++i) r.c[i] = a * b.c[i];
  return r;
}
inline dvec3 operator*(const mat4x3& m, const dvec4& v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3] * v.w; }
inline double dot(const dvec3& a, const dvec3& b);
inline dvec4 operator*(const dvec3& v, const mat4x3& m) {  // row vector times matrix
  return dvec4(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2]), dot(v, m.c[3]));
}
inline dvec3 operator*(const dvec3& v, const mat3& m) { return dvec3(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2])); }

// ---- builtins -------------------------------------------------------------------------------------------
#define GLSL_MAP1(fn, expr)                                                                    \
  inline double fn(double x) { return expr; }                                                 \
  inline dvec2 fn(const dvec2& v) { return dvec2(fn(v.x), fn(v.y)); }                          \
  inline dvec3 fn(const dvec3& v) { return dvec3(fn(v.x), fn(v.y), fn(v.z)); }                 \
  inline dvec4 fn(const dvec4& v) { return dvec4(fn(v.x), fn(v.y), fn(v.z), fn(v.w)); }

GLSL_MAP1(abs, std::fabs(x))
GLSL_MAP1(floor, std::floor(x))
GLSL_MAP1(fract, x - std::floor(x))
GLSL_MAP1(sqrt, std::sqrt(x))
GLSL_MAP1(sin, std::sin(x))
GLSL_MAP1(cos, std::cos(x))
GLSL_MAP1(acos, std::acos(x))
GLSL_MAP1(exp, std::exp(x))
GLSL_MAP1(log, std::log(x))
inline int abs(int x) { return x < 0 ? -x : x; }
inline ivec2 abs(const ivec2& v) { return ivec2(abs(v.x), abs(v.y)); }

#define GLSL_MAP2(fn, expr)                                                                                   \
  inline double fn(double x, double y) { return expr; }                                                      \
  inline dvec2 fn(const dvec2& a, const dvec2& b) { return dvec2(fn(a.x, b.x), fn(a.y, b.y)); }               \
  inline dvec3 fn(const dvec3& a, const dvec3& b) { return dvec3(fn(a.x, b.x), fn(a.y, b.y), fn(a.z, b.z)); } \
  inline dvec4 fn(const dvec4& a, const dvec4& b) {                                                          \
    return dvec4(fn(a.x, b.x), fn(a.y, b.y), fn(a.z, b.z), fn(a.w, b.w));                                     \
  }                                                                                                          \
  inline dvec2 fn(const dvec2& a, double b) { return fn(a, dvec2(b)); }                                      \
  inline dvec3 fn(const dvec3& a, double b) { return fn(a, dvec3(b)); }                                      \
  inline dvec4 fn(const dvec4& a, double b) { return fn(a, dvec4(b)); }

GLSL_MAP2(pow, std::pow(x, y))
GLSL_MAP2(max, (x < y ? y : x))
GLSL_MAP2(min, (y < x ? y : x))
GLSL_MAP2(mod, x - y * std::floor(x / y))
inline int max(int a, int b) { return a < b ? b : a; }
inline int min(int a, int b) { return b < a ? b : a; }
inline uint max(uint a, uint b) { return a < b ? b : a; }
inline uint min(uint a, uint b) { return b < a ? b : a; }
inline double pow(double x, int y) { return std::pow(x, (double)y); }
inline dvec3 pow(const dvec3& a, const ivec3& b) { return pow(a, dvec3(b)); }  // GLSL implicit int -> float

inline double clamp(double x, double lo, double hi) { return min(max(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline dvec2 clamp(const dvec2& v, double lo, double hi) { return dvec2(clamp(v.x, lo, hi), clamp(v.y, lo, hi)); }
inline dvec3 clamp(const dvec3& v, double lo, double hi) {
  return dvec3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi));
}
inline dvec3 clamp(const dvec3& v, const dvec3& lo, const dvec3& hi) {
  return dvec3(clamp(v.x, lo.x, hi.x), clamp(v.y, lo.y, hi.y), clamp(v.z, lo.z, hi.z));
}
inline dvec4 clamp(const dvec4& v, double lo, double hi) {
  return dvec4(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi), clamp(v.w, lo, hi));
}

inline double mix(double a, double b, double t) { return a * (1.0 - t) + b * t; }
inline dvec2 mix(const dvec2& a, const dvec2& b, double t) { return a * (1.0 - t) + b * t; }
inline dvec3 mix(const dvec3& a, const dvec3& b, double t) { return a * (1.0 - t) + b * t; }
inline dvec4 mix(const dvec4& a, const dvec4& b, double t) { return a * (1.0 - t) + b * t; }
inline dvec3 mix(const dvec3& a, const dvec3& b, const dvec3& t) { return a * (1.0 - t) + b * t; }
inline dvec3 mix(const dvec3& a, const dvec3& b, const ivec3& t) { return mix(a, b, dvec3(t)); }
inline dvec3 mix(const dvec3& a, const dvec3& b, const bvec3& t) {
  return dvec3(t.x ? b.x : a.x, t.y ? b.y : a.y, t.z ? b.z : a.z);
}
inline bvec3 lessThan(const dvec3& a, const dvec3& b) { return bvec3(a.x < b.x, a.y < b.y, a.z < b.z); }

inline double dot(double a, double b) { return a * b; }
inline double dot(const dvec2& a, const dvec2& b) { return a.x * b.x + a.y * b.y; }
inline double dot(const dvec3& a, const dvec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double dot(const dvec4& a, const dvec4& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline double length(const dvec2& v) { return std::sqrt(dot(v, v)); }
inline double length(const dvec3& v) { return std::sqrt(dot(v, v)); }
inline double distance(const dvec3& a, const dvec3& b) { return length(a - b); }
inline dvec2 normalize(const dvec2& v) { return v / length(v); }
inline dvec3 normalize(const dvec3& v) { return v / length(v); }
inline dvec3 cross(const dvec3& a, const dvec3& b) {
  return dvec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline dvec3 reflect(const dvec3& I, const dvec3& N) { return I - 2.0 * dot(N, I) * N; }

inline int bitfieldExtract(int v, int offset, int bits) {
  return bits == 0 ? 0 : (int)(((uint)v >> offset) & ((bits == 32) ? 0xffffffffu : ((1u << bits) - 1u)));
}
inline uint bitfieldExtract(uint v, int offset, int bits) {
  return bits == 0 ? 0u : ((v >> offset) & ((bits == 32) ? 0xffffffffu : ((1u << bits) - 1u)));
}
inline uint bitfieldInsert(uint base, uint ins, int offset, int bits) {
  uint mask = ((bits == 32) ? 0xffffffffu : ((1u << bits) - 1u)) << offset;
  return (base & ~mask) | ((ins << offset) & mask);
}
template <class T>
inline T nonuniformEXT(T v) { return v; }

// ---- images and samplers ------------------------------------------------------------------------------
struct image2D {
  double* data = nullptr;  // RGBA doubles, row-major
  int w = 0, h = 0;
};
struct sampler2D {
  const double* data = nullptr;  // RGBA doubles, row-major
  int w = 0, h = 0;
  bool clampToEdge = false;      // CLAMP_TO_EDGE addressing instead of REPEAT
};
// cube maps appear only in code the compared stages never execute (the deferred pass's point-light shadows)
struct samplerCube {};
inline dvec4 texture(const samplerCube&, const dvec3&) { return dvec4(0.0); }
struct accelerationStructureEXT {};

inline dvec4 imageLoad(const image2D& im, const ivec2& p) {
  if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return dvec4(0.0);  // outside: not modelled
  const double* t = im.data + 4 * ((size_t)p.y * im.w + p.x);
  return dvec4(t[0], t[1], t[2], t[3]);
}
inline void imageStore(image2D& im, const ivec2& p, const dvec4& v) {
  if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return;
  double* t = im.data + 4 * ((size_t)p.y * im.w + p.x);
  t[0] = v.x; t[1] = v.y; t[2] = v.z; t[3] = v.w;
}
inline ivec2 textureSize(const sampler2D& s, int) { return ivec2(s.w, s.h); }
// LINEAR filter, REPEAT (or CLAMP_TO_EDGE) addressing, texel centres at (i + 0.5) / size
inline dvec4 texture(const sampler2D& s, const dvec2& uv) {
  if (!s.data) return dvec4(0.0);
  double tx = uv.x * s.w - 0.5, ty = uv.y * s.h - 0.5;
  double fx0 = std::floor(tx), fy0 = std::floor(ty);
  double fx = tx - fx0, fy = ty - fy0;
  long long x0 = (long long)fx0, y0 = (long long)fy0;
  const bool clampEdge = s.clampToEdge;
  auto wrap = [clampEdge](long long v, int m) {
    if (clampEdge) return (int)(v < 0 ? 0 : (v >= m ? m - 1 : v));
    long long r = v % m;
    return (int)(r < 0 ? r + m : r);
  };
  int xs[2] = {wrap(x0, s.w), wrap(x0 + 1, s.w)}, ys[2] = {wrap(y0, s.h), wrap(y0 + 1, s.h)};
  double wx[2] = {1.0 - fx, fx}, wy[2] = {1.0 - fy, fy};
  dvec4 r(0.0);
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const double* t = s.data + 4 * ((size_t)ys[b] * s.w + xs[a]);
      r += dvec4(t[0], t[1], t[2], t[3]) * (wx[a] * wy[b]);
    }
  return r;
}
inline dvec4 textureLod(const sampler2D& s, const dvec2& uv, double) { return texture(s, uv); }

// ---- ray-tracing builtins (set by the harness before each stage runs) ---------------------------------
constexpr uint gl_RayFlagsOpaqueEXT = 1u;
constexpr uint gl_RayFlagsTerminateOnFirstHitEXT = 4u;
constexpr uint gl_RayFlagsSkipClosestHitShaderEXT = 8u;
extern thread_local uvec3 gl_LaunchIDEXT;
extern thread_local uvec3 gl_GlobalInvocationID;
extern thread_local int gl_InstanceCustomIndexEXT;
extern thread_local int gl_PrimitiveID;
extern thread_local mat4x3 gl_ObjectToWorldEXT;
extern thread_local mat4x3 gl_WorldToObjectEXT;
extern thread_local dvec3 gl_WorldRayOriginEXT;

}  // namespace glsl
