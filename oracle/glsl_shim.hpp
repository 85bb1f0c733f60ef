// GLSL-subset shim that lets the reference's fragment- and compute-shader
// bodies compile as C++ (evaluated in double precision).  Test
// infrastructure: used only by oracle/build_ref.py to run the reference's own
// shader text on the CPU.
//
// Compute passes (//!COMPUTE) get uvec3 / ivec2, the gl_* invocation ids,
// `shared` arrays, barrier() and imageStore (see `Compute` below); the
// recipe runs each workgroup's invocations one after another in phases.
//
// Covers what the root .hook files use: vec2/vec3/vec4 with .x .y .z .w
// members plus .xyz() / .wzyx() (the recipe rewrites those two swizzles
// into calls), mat4x3 with column indexing, componentwise arithmetic, and
// the built-ins mix, clamp, max, floor, fract, mod, atan(y, x), sqrt,
// inversesqrt, log2, exp, abs, dot, matrixCompMult, intBitsToFloat.
// Texture access (HOOKED_texOff, NAME_texOff, HOOKED_tex, texture()) is
// provided by the generated per-pass code on top of `Tex` below.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace glsl {

typedef double real;

struct vec2;
struct vec3;
struct vec4;

// integer vectors of the compute passes
struct uvec3 {
  unsigned x = 0, y = 0, z = 0;
};
struct ivec2 {
  int x, y;
  ivec2() : x(0), y(0) {}
  explicit ivec2(int s) : x(s), y(s) {}
  ivec2(int a, int b) : x(a), y(b) {}
  explicit ivec2(const uvec3& u) : x((int)u.x), y((int)u.y) {}
  explicit ivec2(const vec2& v);  // truncation, as GLSL's int()
};
inline ivec2 operator*(const ivec2& a, const ivec2& b) { return ivec2(a.x * b.x, a.y * b.y); }
inline ivec2 operator*(const ivec2& a, int s) { return ivec2(a.x * s, a.y * s); }
inline ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator-(const ivec2& a, const ivec2& b) { return ivec2(a.x - b.x, a.y - b.y); }
inline ivec2 operator+(const ivec2& a, int s) { return ivec2(a.x + s, a.y + s); }
inline ivec2 operator-(const ivec2& a, int s) { return ivec2(a.x - s, a.y - s); }

#define GLSL_VEC_OPS(V, N)                                                       \
  real& operator[](int i) { return (&x)[i]; }                                    \
  real operator[](int i) const { return (&x)[i]; }                               \
  V& operator+=(const V& o) { for (int i = 0; i < N; i++) (*this)[i] += o[i]; return *this; } \
  V& operator-=(const V& o) { for (int i = 0; i < N; i++) (*this)[i] -= o[i]; return *this; } \
  V& operator*=(const V& o) { for (int i = 0; i < N; i++) (*this)[i] *= o[i]; return *this; } \
  V& operator/=(const V& o) { for (int i = 0; i < N; i++) (*this)[i] /= o[i]; return *this; } \
  V& operator*=(real s) { for (int i = 0; i < N; i++) (*this)[i] *= s; return *this; }       \
  V& operator/=(real s) { for (int i = 0; i < N; i++) (*this)[i] /= s; return *this; }       \
  V operator-() const { V r = *this; for (int i = 0; i < N; i++) r[i] = -r[i]; return r; }

struct vec2 {
  real x, y;
  vec2() : x(0), y(0) {}
  explicit vec2(real s) : x(s), y(s) {}
  vec2(real a, real b) : x(a), y(b) {}
  explicit vec2(const ivec2& v) : x(v.x), y(v.y) {}
  GLSL_VEC_OPS(vec2, 2)
};
inline ivec2::ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}

struct vec3 {
  real x, y, z;
  vec3() : x(0), y(0), z(0) {}
  explicit vec3(real s) : x(s), y(s), z(s) {}
  vec3(real a, real b, real c) : x(a), y(b), z(c) {}
  GLSL_VEC_OPS(vec3, 3)
};

struct vec4 {
  real x, y, z, w;
  vec4() : x(0), y(0), z(0), w(0) {}
  explicit vec4(real s) : x(s), y(s), z(s), w(s) {}
  vec4(real a, real b, real c, real d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3& v, real d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec3 xyz() const { return vec3(x, y, z); }
  vec4 wzyx() const { return vec4(w, z, y, x); }
  GLSL_VEC_OPS(vec4, 4)
};

#define GLSL_BINOPS(V, N)                                                              \
  inline V operator+(V a, const V& b) { return a += b; }                               \
  inline V operator-(V a, const V& b) { return a -= b; }                               \
  inline V operator*(V a, const V& b) { return a *= b; }                               \
  inline V operator/(V a, const V& b) { return a /= b; }                               \
  inline V operator+(V a, real s) { for (int i = 0; i < N; i++) a[i] += s; return a; } \
  inline V operator-(V a, real s) { for (int i = 0; i < N; i++) a[i] -= s; return a; } \
  inline V operator*(V a, real s) { return a *= s; }                                   \
  inline V operator/(V a, real s) { return a /= s; }                                   \
  inline V operator+(real s, V a) { for (int i = 0; i < N; i++) a[i] = s + a[i]; return a; } \
  inline V operator-(real s, V a) { for (int i = 0; i < N; i++) a[i] = s - a[i]; return a; } \
  inline V operator*(real s, V a) { for (int i = 0; i < N; i++) a[i] = s * a[i]; return a; } \
  inline V operator/(real s, V a) { for (int i = 0; i < N; i++) a[i] = s / a[i]; return a; } \
  inline V max(V a, const V& b) { for (int i = 0; i < N; i++) a[i] = std::fmax(a[i], b[i]); return a; } \
  inline V min(V a, const V& b) { for (int i = 0; i < N; i++) a[i] = std::fmin(a[i], b[i]); return a; } \
  inline V clamp(V a, real lo, real hi) { for (int i = 0; i < N; i++) a[i] = std::fmin(std::fmax(a[i], lo), hi); return a; } \
  inline V clamp(V a, const V& lo, const V& hi) { for (int i = 0; i < N; i++) a[i] = std::fmin(std::fmax(a[i], lo[i]), hi[i]); return a; } \
  inline V mix(const V& a, const V& b, real t) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * (1.0 - t) + b[i] * t; return r; } \
  inline V mix(const V& a, const V& b, const V& t) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * (1.0 - t[i]) + b[i] * t[i]; return r; } \
  inline V floor(V a) { for (int i = 0; i < N; i++) a[i] = std::floor(a[i]); return a; } \
  inline V fract(V a) { for (int i = 0; i < N; i++) a[i] = a[i] - std::floor(a[i]); return a; } \
  inline real dot(const V& a, const V& b) { real s = 0; for (int i = 0; i < N; i++) s += a[i] * b[i]; return s; }

GLSL_BINOPS(vec2, 2)
GLSL_BINOPS(vec3, 3)
GLSL_BINOPS(vec4, 4)

struct mat4x3 {
  vec3 c[4];
  mat4x3() {}
  explicit mat4x3(real s) {  // s on the diagonal, as GLSL's scalar matrix constructor
    for (int i = 0; i < 3; i++) c[i][i] = s;
  }
  mat4x3(const vec3& a, const vec3& b, const vec3& d, const vec3& e) { c[0] = a; c[1] = b; c[2] = d; c[3] = e; }
  vec3& operator[](int i) { return c[i]; }
  const vec3& operator[](int i) const { return c[i]; }
  mat4x3& operator+=(const mat4x3& o) {
    for (int i = 0; i < 4; i++) c[i] += o.c[i];
    return *this;
  }
};
inline mat4x3 operator+(mat4x3 a, const mat4x3& b) { return a += b; }
// column vector times row vector: column i = col * row[i]
inline mat4x3 outerProduct(const vec3& col, const vec4& row) {
  mat4x3 r;
  for (int i = 0; i < 4; i++) r.c[i] = col * row[i];
  return r;
}
inline mat4x3 matrixCompMult(const mat4x3& a, const mat4x3& b) {
  mat4x3 r;
  for (int i = 0; i < 4; i++) r.c[i] = a.c[i] * b.c[i];
  return r;
}

inline real mix(real a, real b, real t) { return a * (1.0 - t) + b * t; }
inline real mix(real a, real b, bool sel) { return sel ? b : a; }
inline real clamp(real a, real lo, real hi) { return std::fmin(std::fmax(a, lo), hi); }
inline real max(real a, real b) { return std::fmax(a, b); }
inline real min(real a, real b) { return std::fmin(a, b); }
inline real floor(real a) { return std::floor(a); }
inline real fract(real a) { return a - std::floor(a); }
inline real mod(real a, real b) { return a - b * std::floor(a / b); }
inline real atan(real y, real x) { return std::atan2(y, x); }
inline real sqrt(real a) { return std::sqrt(a); }
inline real inversesqrt(real a) { return 1.0 / std::sqrt(a); }
inline real log2(real a) { return std::log2(a); }
inline real exp(real a) { return std::exp(a); }
inline real abs(real a) { return std::fabs(a); }
inline float intBitsToFloat(int32_t i) { float f; std::memcpy(&f, &i, 4); return f; }

// ---------------------------------------------------------------- textures
struct Tex {
  int w = 0, h = 0;
  bool linear = false;
  std::vector<vec4> px;  // row-major, x fastest
  vec4 at(int x, int y) const {
    x = x < 0 ? 0 : (x >= w ? w - 1 : x);
    y = y < 0 ? 0 : (y >= h ? h - 1 : y);
    return px[(size_t)y * w + x];
  }
  // normalised coordinates; NEAREST picks floor(uv*size), LINEAR blends
  // the four texels around uv*size - 0.5 (clamp-to-edge)
  vec4 sample(const vec2& uv) const {
    if (!linear) return at((int)std::floor(uv.x * w), (int)std::floor(uv.y * h));
    real tx = uv.x * w - 0.5, ty = uv.y * h - 0.5;
    int x0 = (int)std::floor(tx), y0 = (int)std::floor(ty);
    real fx = tx - x0, fy = ty - y0;
    return (at(x0, y0) * (1 - fx) + at(x0 + 1, y0) * fx) * (1 - fy) +
           (at(x0, y0 + 1) * (1 - fx) + at(x0 + 1, y0 + 1) * fx) * fy;
  }
};

// state of the pixel being shaded
struct Frag {
  vec2 pos;   // HOOKED_pos (normalised)
  vec2 size;  // HOOKED_size
};

inline vec4 tex_off(const Tex& t, const Frag& f, const vec2& off) {
  return t.sample(vec2(f.pos.x + off.x / t.w, f.pos.y + off.y / t.h));
}

// ---------------------------------------------------------- compute passes
// Invocation state of a compute pass.  A workgroup runs in phases: in phase
// k every invocation executes hook() from the start until it reaches its
// (k+1)-th barrier(), where it returns; the last phase runs every invocation
// to the end.  So all shared-memory writes before barrier k+1 of every
// invocation happen before any read after it -- what barrier() guarantees on
// a GPU -- provided that re-running the earlier segments rewrites the same
// values (true of the cooperative tile loads these shaders do before their
// barrier).
struct Compute {
  uvec3 wg_id, local_id, global_id, wg_size;
  unsigned local_index = 0;
  Tex* out = nullptr;  // out_image
  int bar = 0, phase = 0;
  void store(int x, int y, const vec4& v) {
    if (x >= 0 && y >= 0 && x < out->w && y < out->h) out->px[(size_t)y * out->w + x] = v;
  }
};

// WIDTH/HEIGHT/WHEN reverse-Polish evaluator
double rpn(const char* expr, const std::map<std::string, double>& env);

}  // namespace glsl
