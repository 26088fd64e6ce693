// glsl_shim.hpp -- just enough of GLSL 4.40 in C++ to compile the reference's
// shader sources (res/*.glsl of jaafersheriff/Cloud-Renderer) unchanged, so
// that the oracle can be checked against the reference's own shader code.
//
// TEST INFRASTRUCTURE ONLY (built into oracle/_ref/ by oracle/build_ref.py).
//
// Semantics follow the GLSL 4.40 specification: float is IEEE binary32 and
// every operation rounds once (the recipe compiles with -ffp-contract=off);
// normalize(x) = x / length(x); int operands of mixed expressions convert to
// float.  Texture sampling follows the OpenGL 4.4 specification, section 8.14
// (LINEAR / LINEAR_MIPMAP_LINEAR filtering, CLAMP_TO_EDGE wrapping), which is
// how the reference configures its volume (CloudVolume.cpp:17-23).
// Storage qualifiers (in/out/uniform/flat/layout) expand to nothing so that
// shader interface variables become plain globals of the namespace the build
// recipe wraps each shader in.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace glsl {

// ---- swizzle proxies (a few fixed patterns, as used by the shaders) -------
struct vec2;
struct vec3;
struct vec4;

template <int A, int B>
struct swz2 {
    float e[2];
    operator vec2() const;
};
template <int A, int B, int C>
struct swz3 {
    float e[3];
    operator vec3() const;
    swz3& operator+=(const vec3& o);
    swz3& operator*=(float s);
};

struct vec2 {
    union {
        struct { float x, y; };
        struct { float r, g; };
        struct { float s, t; };
    };
    vec2() : x(0), y(0) {}
    explicit vec2(float v) : x(v), y(v) {}
    vec2(float a, float b) : x(a), y(b) {}
    float& operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
};

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        swz2<0, 1> xy;
    };
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float v) : x(v), y(v), z(v) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
    vec3& operator=(const vec3& o) {
        x = o.x; y = o.y; z = o.z;
        return *this;
    }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        swz2<0, 1> xy;
        swz3<0, 1, 2> xyz;
        swz3<0, 1, 2> rgb;
    };
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float v) : x(v), y(v), z(v), w(v) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    vec4& operator=(const vec4& o) {
        x = o.x; y = o.y; z = o.z; w = o.w;
        return *this;
    }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

template <int A, int B>
swz2<A, B>::operator vec2() const { return vec2(e[A], e[B]); }
template <int A, int B, int C>
swz3<A, B, C>::operator vec3() const { return vec3(e[A], e[B], e[C]); }
template <int A, int B, int C>
swz3<A, B, C>& swz3<A, B, C>::operator+=(const vec3& o) {
    e[A] = e[A] + o.x; e[B] = e[B] + o.y; e[C] = e[C] + o.z;
    return *this;
}
template <int A, int B, int C>
swz3<A, B, C>& swz3<A, B, C>::operator*=(float s) {
    e[A] = e[A] * s; e[B] = e[B] * s; e[C] = e[C] * s;
    return *this;
}

struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}  // truncation
};
struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x((int)v.x), y((int)v.y), z((int)v.z) {}
};
struct ivec4 {
    int x, y, z, w;
    ivec4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {}
};

// ---- component-wise arithmetic ---------------------------------------------
#define GLSL_V2(OP)                                                                   \
    inline vec2 operator OP(const vec2& a, const vec2& b) { return vec2(a.x OP b.x, a.y OP b.y); } \
    inline vec2 operator OP(const vec2& a, float s) { return vec2(a.x OP s, a.y OP s); }         \
    inline vec2 operator OP(float s, const vec2& a) { return vec2(s OP a.x, s OP a.y); }
#define GLSL_V3(OP)                                                                   \
    inline vec3 operator OP(const vec3& a, const vec3& b) {                           \
        return vec3(a.x OP b.x, a.y OP b.y, a.z OP b.z);                              \
    }                                                                                 \
    inline vec3 operator OP(const vec3& a, float s) { return vec3(a.x OP s, a.y OP s, a.z OP s); } \
    inline vec3 operator OP(float s, const vec3& a) { return vec3(s OP a.x, s OP a.y, s OP a.z); }
#define GLSL_V4(OP)                                                                   \
    inline vec4 operator OP(const vec4& a, const vec4& b) {                           \
        return vec4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w);                  \
    }                                                                                 \
    inline vec4 operator OP(const vec4& a, float s) {                                 \
        return vec4(a.x OP s, a.y OP s, a.z OP s, a.w OP s);                          \
    }                                                                                 \
    inline vec4 operator OP(float s, const vec4& a) {                                 \
        return vec4(s OP a.x, s OP a.y, s OP a.z, s OP a.w);                          \
    }
GLSL_V2(+) GLSL_V2(-) GLSL_V2(*) GLSL_V2(/)
GLSL_V3(+) GLSL_V3(-) GLSL_V3(*) GLSL_V3(/)
GLSL_V4(+) GLSL_V4(-) GLSL_V4(*) GLSL_V4(/)
#undef GLSL_V2
#undef GLSL_V3
#undef GLSL_V4
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3& operator+=(vec3& a, const vec3& b) { return a = a + b; }
inline vec3& operator-=(vec3& a, const vec3& b) { return a = a - b; }
inline vec3& operator*=(vec3& a, float s) { return a = a * s; }
inline vec3& operator/=(vec3& a, float s) { return a = a / s; }
inline vec4& operator+=(vec4& a, const vec4& b) { return a = a + b; }
inline vec4& operator*=(vec4& a, float s) { return a = a * s; }

// ---- matrices (column-major: m[c] is column c) -------------------------------
struct mat3 {
    vec3 c[3];
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    mat4() {}
    explicit mat4(float d) {
        for (int i = 0; i < 4; ++i) c[i] = vec4(0.f);
        c[0].x = c[1].y = c[2].z = c[3].w = d;
    }
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline mat3 make_mat3(const mat4& m) {
    mat3 r;
    for (int i = 0; i < 3; ++i) r.c[i] = vec3(m.c[i].x, m.c[i].y, m.c[i].z);
    return r;
}
inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 r;
    for (int row = 0; row < 4; ++row)
        r[row] = ((m.c[0][row] * v.x + m.c[1][row] * v.y) + m.c[2][row] * v.z) + m.c[3][row] * v.w;
    return r;
}
// row vector times matrix: r[c] = dot(v, column c)
inline vec4 operator*(const vec4& v, const mat4& m) {
    vec4 r;
    for (int col = 0; col < 4; ++col)
        r[col] = ((v.x * m.c[col].x + v.y * m.c[col].y) + v.z * m.c[col].z) + v.w * m.c[col].w;
    return r;
}
inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r;
    for (int col = 0; col < 4; ++col) r.c[col] = a * b.c[col];
    return r;
}
inline vec3 operator*(const mat3& m, const vec3& v) {
    vec3 r;
    for (int row = 0; row < 3; ++row)
        r[row] = (m.c[0][row] * v.x + m.c[1][row] * v.y) + m.c[2][row] * v.z;
    return r;
}
inline mat4 transpose(const mat4& m) {
    mat4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) r.c[i][j] = m.c[j][i];
    return r;
}
// inverse by cofactor expansion: inv(r, c) = C(c, r) / det, with the
// cofactor C(i, j) = (-1)^(i+j) * minor(i, j) and det expanded along row 0
inline mat4 inverse(const mat4& m) {
    auto A = [&](int row, int col) { return m.c[col][row]; };
    auto cofactor = [&](int i, int j) {
        int rs[3], cs[3], nr = 0, nc = 0;
        for (int k = 0; k < 4; ++k) {
            if (k != i) rs[nr++] = k;
            if (k != j) cs[nc++] = k;
        }
        float d = A(rs[0], cs[0]) * (A(rs[1], cs[1]) * A(rs[2], cs[2]) - A(rs[1], cs[2]) * A(rs[2], cs[1])) -
                  A(rs[0], cs[1]) * (A(rs[1], cs[0]) * A(rs[2], cs[2]) - A(rs[1], cs[2]) * A(rs[2], cs[0])) +
                  A(rs[0], cs[2]) * (A(rs[1], cs[0]) * A(rs[2], cs[1]) - A(rs[1], cs[1]) * A(rs[2], cs[0]));
        return ((i + j) & 1) ? -d : d;
    };
    float det = 0.f;
    for (int k = 0; k < 4; ++k) det = det + A(0, k) * cofactor(0, k);
    mat4 r;
    for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 4; ++col) r.c[col][row] = cofactor(col, row) / det;
    return r;
}

// ---- built-in functions --------------------------------------------------------
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec2& v) { return std::sqrt(dot(v, v)); }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline vec3 normalize(const vec3& v) {
    float l = length(v);
    return vec3(v.x / l, v.y / l, v.z / l);
}
inline float sqrt(float x) { return std::sqrt(x); }
inline float tan(float x) { return std::tan(x); }
inline float log2(float x) { return std::log2(x); }
inline float abs(float x) { return std::fabs(x); }
inline float floor(float x) { return std::floor(x); }
template <class A, class B>
inline auto max(A a, B b) -> decltype(a + b) {
    return (decltype(a + b))a < (decltype(a + b))b ? (decltype(a + b))b : (decltype(a + b))a;
}
template <class A, class B>
inline auto min(A a, B b) -> decltype(a + b) {
    return (decltype(a + b))b < (decltype(a + b))a ? (decltype(a + b))b : (decltype(a + b))a;
}
template <class A, class B, class C>
inline float clamp(A x, B lo, C hi) {
    return min(max((float)x, (float)lo), (float)hi);
}

// ---- images ---------------------------------------------------------------------
// image3D: binary marks of an r8 volume, one byte per voxel; stores outside
// the image are ignored (OpenGL 4.4, 8.26: out-of-range image stores have no
// effect).
struct image3D {
    uint8_t* data = nullptr;
    int w = 0, h = 0, d = 0;
};
inline void imageStore(image3D img, ivec3 p, const vec4& v) {
    if (!img.data || p.x < 0 || p.y < 0 || p.z < 0 || p.x >= img.w || p.y >= img.h || p.z >= img.d)
        return;
    float r = v.x < 0.f ? 0.f : (v.x > 1.f ? 1.f : v.x);  // r8 unorm
    img.data[((size_t)p.z * img.h + p.y) * img.w + p.x] = (uint8_t)std::lround(r * 255.f);
}
struct image2D {
    const float* data = nullptr;  // rgba32f
    int w = 0, h = 0;
};
inline vec4 imageLoad(image2D img, ivec2 p) {
    if (!img.data || p.x < 0 || p.y < 0 || p.x >= img.w || p.y >= img.h) return vec4(0.f);
    const float* t = img.data + ((size_t)p.y * img.w + p.x) * 4;
    return vec4(t[0], t[1], t[2], t[3]);
}

// ---- 3D textures -------------------------------------------------------------------
// Mip chain of 1 channel (level l is dims[l]^3, x fastest, read as .r with
// g = b = 0, a = 1) or of 4 interleaved channels (RGBA), CLAMP_TO_EDGE or
// REPEAT wrapping (8.14.2).
struct sampler3D {
    const float* data = nullptr;
    const int* dims = nullptr;
    const long* offs = nullptr;
    int levels = 0;
    int channels = 1;
    bool repeat = false;
};
inline int wrap_index(const sampler3D& s, int i, int n) {
    if (s.repeat) return ((i % n) + n) % n;
    return i < 0 ? 0 : (i >= n ? n - 1 : i);
}
inline float texel(const sampler3D& s, int l, int i, int j, int k, int ch) {
    const int n = s.dims[l];
    i = wrap_index(s, i, n);
    j = wrap_index(s, j, n);
    k = wrap_index(s, k, n);
    return s.data[(s.offs[l] + ((long)k * n + j) * n + i) * s.channels + ch];
}
// LINEAR filter of one level at normalised coordinates (8.14.2, eq. 8.9-8.11)
inline float linear_level(const sampler3D& s, int l, const vec3& P, int ch) {
    const float n = (float)s.dims[l];
    const float u = P.x * n, v = P.y * n, w = P.z * n;
    const float uf = u - 0.5f, vf = v - 0.5f, wf = w - 0.5f;
    const int i0 = (int)std::floor(uf), j0 = (int)std::floor(vf), k0 = (int)std::floor(wf);
    const float a = uf - std::floor(uf), b = vf - std::floor(vf), c = wf - std::floor(wf);
    float t[2][2][2];
    for (int dk = 0; dk < 2; ++dk)
        for (int dj = 0; dj < 2; ++dj)
            for (int di = 0; di < 2; ++di)
                t[dk][dj][di] = texel(s, l, i0 + di, j0 + dj, k0 + dk, ch);
    float r = 0.f;
    for (int dk = 0; dk < 2; ++dk)
        for (int dj = 0; dj < 2; ++dj)
            for (int di = 0; di < 2; ++di) {
                float wgt = (di ? a : 1.f - a) * (dj ? b : 1.f - b) * (dk ? c : 1.f - c);
                r = r + wgt * t[dk][dj][di];
            }
    return r;
}
// textureLod with MIN_FILTER LINEAR_MIPMAP_LINEAR, MAG_FILTER LINEAR
// (8.14.1-8.14.3): lambda <= 0 magnifies from the base level; otherwise
// levels d1 = floor(lambda) and d1 + 1 (clamped to the last level q) blend by
// frac(lambda), and lambda >= q reads level q alone.
inline float lod_channel(const sampler3D& s, const vec3& P, float lod, int ch) {
    const int q = s.levels - 1;
    if (!(lod > 0.f)) return linear_level(s, 0, P, ch);
    if (lod >= (float)q) return linear_level(s, q, P, ch);
    const int d1 = (int)std::floor(lod);
    const float f = lod - std::floor(lod);
    const float t1 = linear_level(s, d1, P, ch), t2 = linear_level(s, d1 + 1, P, ch);
    return (1.f - f) * t1 + f * t2;
}
inline vec4 textureLod(const sampler3D& s, const vec3& P, float lod) {
    if (s.channels == 1) return vec4(lod_channel(s, P, lod, 0), 0.f, 0.f, 1.f);
    return vec4(lod_channel(s, P, lod, 0), lod_channel(s, P, lod, 1), lod_channel(s, P, lod, 2),
                lod_channel(s, P, lod, 3));
}
inline vec4 texture(const sampler3D& s, const vec3& P) {
    if (!s.data) return vec4(0.f);
    return textureLod(s, P, 0.f);
}

// Set by `discard` (see the macro below); the driver clears it before each
// fragment.
inline bool g_discarded = false;

}  // namespace glsl

// Storage and layout qualifiers carry no meaning for the CPU build.
#define in
#define out
#define inout
#define flat
#define uniform
#define layout(...)
#define discard { ::glsl::g_discarded = true; return; }
// GLSL's matrix-narrowing constructor mat3(m4)
#define mat3(m) glsl::make_mat3(m)
