// cl_shim.h -- just enough of OpenCL C's vector types and built-ins, in C++,
// to compile the reference's own .cl functions on the host (oracle/_ref).
//
// TEST INFRASTRUCTURE ONLY.  oracle/ref_shim/cl_to_cpp.py rewrites OpenCL C's
// vector literals `(floatN)(a, b, ...)` into C++ constructor calls; with that,
// the reference's noise, QEF, cuckoo, field and octree code compiles unchanged
// against this header.  The built-ins follow the same floating-point conventions as the
// oracle restatement (oracle/lvn_oracle.cpp): dot() is an fma chain
// fma(a.z, b.z, fma(a.y, b.y, a.x * b.x)), mix(a, b, t) = fma(b - a, t, a),
// rsqrt(x) = 1 / sqrt(x), normalize(v) = v / sqrt(dot(v, v)) (zero stays
// zero).  Image reads follow the OpenCL specification's nearest-filter,
// repeat-addressing rule with normalised coordinates on an RGBA8 UNORM
// image: i = floor((u - floor(u)) * width), wrapped once, texel / 255.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace clshim {

template <int N>
struct VecStore {
    float v[N];
};

// read / write view of components (A, B[, C]) of an N-float vector
template <int N, int A, int B>
struct Sw2;
template <int N, int A, int B, int C>
struct Sw3;

}  // namespace clshim

struct float2;
struct float3;
struct float4;

namespace clshim {
template <int N, int A, int B>
struct Sw2 {
    float v[N];
    inline operator float2() const;
    inline Sw2& operator=(const float2& o);
    inline Sw2& operator=(const Sw2& o);
};
template <int N, int A, int B, int C>
struct Sw3 {
    float v[N];
    inline operator float3() const;
    inline Sw3& operator=(const float3& o);
    inline Sw3& operator=(const Sw3& o);
};
}  // namespace clshim

#define CLSHIM_SW2(N)                                                                                    \
    clshim::Sw2<N, 0, 0> xx;                                                                             \
    clshim::Sw2<N, 0, 1> xy;                                                                             \
    clshim::Sw2<N, 1, 0> yx;                                                                             \
    clshim::Sw2<N, 1, 1> yy;
#define CLSHIM_SW2_3(N)                                                                                  \
    clshim::Sw2<N, 0, 2> xz;                                                                             \
    clshim::Sw2<N, 2, 0> zx;                                                                             \
    clshim::Sw2<N, 1, 2> yz;                                                                             \
    clshim::Sw2<N, 2, 1> zy;                                                                             \
    clshim::Sw2<N, 2, 2> zz;                                                                             \
    clshim::Sw3<N, 0, 1, 2> xyz;                                                                         \
    clshim::Sw3<N, 1, 2, 0> yzx;                                                                         \
    clshim::Sw3<N, 2, 0, 1> zxy;

struct float2 {
    union {
        struct {
            float x, y;
        };
        float v[2];
        CLSHIM_SW2(2)
    };
    float2() : x(0.f), y(0.f) {}
    explicit float2(float s) : x(s), y(s) {}
    float2(float a, float b) : x(a), y(b) {}
    float2(const float2& o) : x(o.x), y(o.y) {}
    float2& operator=(const float2& o) {
        x = o.x;
        y = o.y;
        return *this;
    }
};

struct float3 {
    union {
        struct {
            float x, y, z;
        };
        float v[3];
        CLSHIM_SW2(3)
        CLSHIM_SW2_3(3)
    };
    float3() : x(0.f), y(0.f), z(0.f) {}
    explicit float3(float s) : x(s), y(s), z(s) {}
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
    float3(const float3& o) : x(o.x), y(o.y), z(o.z) {}
    float3& operator=(const float3& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        return *this;
    }
};

struct float4 {
    union {
        struct {
            float x, y, z, w;
        };
        float v[4];
        CLSHIM_SW2(4)
        CLSHIM_SW2_3(4)
    };
    float4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
    explicit float4(float s) : x(s), y(s), z(s), w(s) {}
    float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    float4(const float3& a, float d) : x(a.x), y(a.y), z(a.z), w(d) {}
    float4(const float4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    float4& operator=(const float4& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        w = o.w;
        return *this;
    }
};

namespace clshim {
template <int N, int A, int B>
Sw2<N, A, B>::operator float2() const { return float2(v[A], v[B]); }
template <int N, int A, int B>
Sw2<N, A, B>& Sw2<N, A, B>::operator=(const float2& o) {
    const float a = o.x, b = o.y;
    v[A] = a;
    v[B] = b;
    return *this;
}
template <int N, int A, int B>
Sw2<N, A, B>& Sw2<N, A, B>::operator=(const Sw2& o) { return *this = (float2)o; }
template <int N, int A, int B, int C>
Sw3<N, A, B, C>::operator float3() const { return float3(v[A], v[B], v[C]); }
template <int N, int A, int B, int C>
Sw3<N, A, B, C>& Sw3<N, A, B, C>::operator=(const Sw3& o) { return *this = (float3)o; }
template <int N, int A, int B, int C>
Sw3<N, A, B, C>& Sw3<N, A, B, C>::operator=(const float3& o) {
    const float a = o.x, b = o.y, c = o.z;
    v[A] = a;
    v[B] = b;
    v[C] = c;
    return *this;
}
}  // namespace clshim

// ---- arithmetic: component-wise, with scalar broadcast ---------------------
#define CLSHIM_OPS(T, N)                                                                                 \
    inline T operator+(T a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] + b.v[i]; return a; } \
    inline T operator-(T a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] - b.v[i]; return a; } \
    inline T operator*(T a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] * b.v[i]; return a; } \
    inline T operator/(T a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] / b.v[i]; return a; } \
    inline T operator+(T a, float s) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] + s; return a; }       \
    inline T operator-(T a, float s) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] - s; return a; }       \
    inline T operator*(T a, float s) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] * s; return a; }       \
    inline T operator/(T a, float s) { for (int i = 0; i < N; i++) a.v[i] = a.v[i] / s; return a; }       \
    inline T operator+(float s, T a) { for (int i = 0; i < N; i++) a.v[i] = s + a.v[i]; return a; }       \
    inline T operator-(float s, T a) { for (int i = 0; i < N; i++) a.v[i] = s - a.v[i]; return a; }       \
    inline T operator*(float s, T a) { for (int i = 0; i < N; i++) a.v[i] = s * a.v[i]; return a; }       \
    inline T operator-(T a) { for (int i = 0; i < N; i++) a.v[i] = -a.v[i]; return a; }                   \
    inline T& operator+=(T& a, const T& b) { a = a + b; return a; }                                        \
    inline T& operator-=(T& a, const T& b) { a = a - b; return a; }                                        \
    inline T& operator*=(T& a, const T& b) { a = a * b; return a; }                                        \
    inline T& operator+=(T& a, float s) { a = a + s; return a; }                                           \
    inline T& operator-=(T& a, float s) { a = a - s; return a; }                                           \
    inline T& operator*=(T& a, float s) { a = a * s; return a; }                                           \
    inline T& operator/=(T& a, float s) { a = a / s; return a; }                                           \
    inline T floor(T a) { for (int i = 0; i < N; i++) a.v[i] = std::floor(a.v[i]); return a; }            \
    inline T fabs(T a) { for (int i = 0; i < N; i++) a.v[i] = std::fabs(a.v[i]); return a; }              \
    inline T clamp(T a, float lo, float hi) {                                                              \
        for (int i = 0; i < N; i++) a.v[i] = std::fmin(std::fmax(a.v[i], lo), hi);                         \
        return a;                                                                                          \
    }                                                                                                      \
    inline T step(const T& edge, T x) { for (int i = 0; i < N; i++) x.v[i] = x.v[i] < edge.v[i] ? 0.f : 1.f; return x; } \
    inline T max(T a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = std::fmax(a.v[i], b.v[i]); return a; } \
    inline T min(T a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = std::fmin(a.v[i], b.v[i]); return a; } \
    inline T fmod(T a, const T& b) { for (int i = 0; i < N; i++) a.v[i] = std::fmod(a.v[i], b.v[i]); return a; } \
    inline T sign(T a) {                                                                                   \
        for (int i = 0; i < N; i++) a.v[i] = a.v[i] > 0.f ? 1.f : a.v[i] < 0.f ? -1.f : 0.f;               \
        return a;                                                                                          \
    }                                                                                                      \
    inline T mix(const T& a, const T& b, float t) {                                                        \
        T r;                                                                                               \
        for (int i = 0; i < N; i++) r.v[i] = std::fmaf(b.v[i] - a.v[i], t, a.v[i]);                       \
        return r;                                                                                          \
    }
CLSHIM_OPS(float2, 2)
CLSHIM_OPS(float3, 3)
CLSHIM_OPS(float4, 4)

inline float dot(const float2& a, const float2& b) { return std::fmaf(a.y, b.y, a.x * b.x); }
inline float dot(const float3& a, const float3& b) { return std::fmaf(a.z, b.z, std::fmaf(a.y, b.y, a.x * b.x)); }
inline float dot(const float4& a, const float4& b) {
    return std::fmaf(a.w, b.w, std::fmaf(a.z, b.z, std::fmaf(a.y, b.y, a.x * b.x)));
}
template <typename T>
inline float length(const T& a) { return std::sqrt(dot(a, a)); }
template <typename T>
inline T normalize(const T& a) {
    const float l = std::sqrt(dot(a, a));
    return l > 0.f ? a / l : a;
}

inline float step(float edge, float x) { return x < edge ? 0.f : 1.f; }
inline float clamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline float mix(float a, float b, float t) { return std::fmaf(b - a, t, a); }
inline float rsqrt(float x) { return 1.f / std::sqrt(x); }
inline float sign(float x) { return x > 0.f ? 1.f : x < 0.f ? -1.f : 0.f; }
inline float radians(float d) { return d * (3.14159265358979f / 180.f); }
inline float fabs(float x) { return std::fabs(x); }
inline float floor(float x) { return std::floor(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }

// ---- images: the permutation lookup image (RGBA8 UNORM, 256 x 256) ---------
struct clshim_image2d {
    const uint8_t* texels;  // row-major, 4 bytes per texel
    int width, height;
};
typedef const clshim_image2d* image2d_t;
typedef int sampler_t;
#define CLK_FILTER_NEAREST 1
#define CLK_ADDRESS_REPEAT 2
#define CLK_NORMALIZED_COORDS_TRUE 4

// nearest filter, repeat addressing, normalised coordinates (the OpenCL
// specification's rule for CLK_ADDRESS_REPEAT with CLK_FILTER_NEAREST)
inline int clshim_repeat(float s, int w) {
    const float u = (s - std::floor(s)) * (float)w;
    int i = (int)std::floor(u);
    if (i > w - 1) i -= w;
    return i;
}
inline float4 read_imagef(image2d_t img, sampler_t, const float2& coord) {
    const int i = clshim_repeat(coord.x, img->width), j = clshim_repeat(coord.y, img->height);
    const uint8_t* t = img->texels + 4 * ((size_t)j * img->width + i);
    return float4(t[0] / 255.f, t[1] / 255.f, t[2] / 255.f, t[3] / 255.f);
}

// ---- integer vectors and the kernel built-ins the reference's kernels use ---
struct int4 {
    int x, y, z, w;
    int4() : x(0), y(0), z(0), w(0) {}
    int4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {}
};
inline int4 operator+(int4 a, const int4& b) { return int4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline int4 operator-(int4 a, const int4& b) { return int4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline int4 operator*(int s, const int4& a) { return int4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline int4& operator+=(int4& a, const int4& b) { a = a + b; return a; }
inline int4& operator/=(int4& a, int s) {
    a.x /= s;
    a.y /= s;
    a.z /= s;
    a.w /= s;
    return a;
}
inline float4 convert_float4(const int4& a) { return float4((float)a.x, (float)a.y, (float)a.z, (float)a.w); }
// uint and ulong (unsigned int, 64-bit unsigned long) come from glibc's <sys/types.h>
#include <sys/types.h>
inline int clz(uint n) { return n ? __builtin_clz(n) : 32; }

// A kernel runs as a loop over its global ids on one host thread; the
// reference's 64-bit atomics are then plain read-modify-writes.
extern thread_local int clshim_gid[3];
inline int get_global_id(int d) { return clshim_gid[d]; }
inline ulong atom_xchg(ulong* p, ulong v) {
    const ulong o = *p;
    *p = v;
    return o;
}
inline ulong atom_cmpxchg(ulong* p, ulong cmp, ulong v) {
    const ulong o = *p;
    if (o == cmp) *p = v;
    return o;
}

// ---- OpenCL C qualifiers ----------------------------------------------------
#define read_only
#define write_only
#define __read_only
#define __constant static const
#define __global
#define __private
#define global
#define kernel
