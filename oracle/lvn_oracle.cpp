// lvn_oracle.cpp -- CPU restatement of the leven chunk-meshing path.
//
// TEST INFRASTRUCTURE ONLY (see lvn_oracle.h).  Plain sequential C++17,
// compiled with -O2 -ffp-contract=off and no fast-math, so that every
// floating-point operation is the IEEE single-precision operation written
// here.  Fused multiply-adds appear only where this file calls std::fmaf;
// the CUDA product path performs the same operations in the same order.
//
// Floating-point conventions of this restatement (the reference was compiled
// with -cl-fast-relaxed-math, leven/src/compute.cpp:258, so its own bits are
// implementation-defined; these rules fix one admissible choice):
//   * dot(a,b) = fma(a.z,b.z, fma(a.y,b.y, a.x*b.x))   (2D: fma(a.y,b.y,a.x*b.x))
//   * a += b*c in fBm / octave accumulation loops = fma(b, c, a)
//   * mix(a,b,t) = fma(b-a, t, a)
//   * snoise3's `0.6 - dot` (a double literal in simplex.cl:243) is single
//     precision here; snoise2's `0.5 - dot` is exact either way.
//   * pow(frequency, -1) in RidgedMultiFractal (noise.cl:73) = 1.f / frequency
//   * normalize(v) = v / sqrt(dot(v,v)); a zero vector stays zero.
//   * rsqrt in givens_coeffs_sym (qef.cl:40) = 1.f / sqrtf(x); the double
//     expressions of svd_rotateq_xy (`2.0 * c * s * a`, qef.cl:52) and
//     svd_invdet (`1.0 / x`, qef.cl:108) are evaluated in single precision.
//   * Image reads (simplex.cl:59, nearest + repeat + normalised coordinates)
//     resolve an integer lattice coordinate i to texel (i & 255); the 3D
//     second lookup uses u = A/255, which selects column A for A < 255 and
//     column 0 for A == 255 (u == 1.0 wraps to 0).
#include "lvn_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <climits>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace {

constexpr int MATERIAL_NONE = 200;   // leven/src/volume_materials.h:7
constexpr int MATERIAL_AIR = 201;    // leven/src/volume_materials.h:8
constexpr int LEAF_SIZE_SCALE = 4;   // leven/src/volume_constants.h:7-8

// ---------------------------------------------------------------------------
// Permutation lookup image: compute_density_field.cpp:28-125
// ---------------------------------------------------------------------------

// Ken Perlin's reference permutation (public domain).
const int kPerlin[256] = {
    151, 160, 137, 91,  90,  15,  131, 13,  201, 95,  96,  53,  194, 233, 7,   225,
    140, 36,  103, 30,  69,  142, 8,   99,  37,  240, 21,  10,  23,  190, 6,   148,
    247, 120, 234, 75,  0,   26,  197, 62,  94,  252, 219, 203, 117, 35,  11,  32,
    57,  177, 33,  88,  237, 149, 56,  87,  174, 20,  125, 136, 171, 168, 68,  175,
    74,  165, 71,  134, 139, 48,  27,  166, 77,  146, 158, 231, 83,  111, 229, 122,
    60,  211, 133, 230, 220, 105, 92,  41,  55,  46,  245, 40,  244, 102, 143, 54,
    65,  25,  63,  161, 1,   216, 80,  73,  209, 76,  132, 187, 208, 89,  18,  169,
    200, 196, 135, 130, 116, 188, 159, 86,  164, 100, 109, 198, 173, 186, 3,   64,
    52,  217, 226, 250, 124, 123, 5,   202, 38,  147, 118, 126, 255, 82,  85,  212,
    207, 206, 59,  227, 47,  16,  58,  17,  182, 189, 28,  42,  223, 183, 170, 213,
    119, 248, 152, 2,   44,  154, 163, 70,  221, 153, 101, 155, 167, 43,  172, 9,
    129, 22,  39,  253, 19,  98,  108, 110, 79,  113, 224, 232, 178, 185, 112, 104,
    218, 246, 97,  228, 251, 34,  242, 193, 238, 210, 144, 12,  191, 179, 162, 241,
    81,  51,  145, 235, 249, 14,  239, 107, 49,  192, 214, 31,  181, 199, 106, 157,
    184, 84,  204, 176, 115, 121, 50,  45,  127, 4,   150, 254, 138, 236, 205, 93,
    222, 114, 67,  29,  24,  72,  243, 141, 128, 195, 78,  66,  215, 61,  156, 180,
};

// Perlin's 16 gradient directions (compute_density_field.cpp:60-63).
const int kGrad3[16][3] = {{0, 1, 1},  {0, 1, -1},  {0, -1, 1}, {0, -1, -1},
                           {1, 0, 1},  {1, 0, -1},  {-1, 0, 1}, {-1, 0, -1},
                           {1, 1, 0},  {1, -1, 0},  {-1, 1, 0}, {-1, -1, 0},
                           {1, 0, -1}, {-1, 0, -1}, {0, -1, 1}, {0, 1, 1}};

// The reference's `int perm[512]` literal (compute_density_field.cpp:28-52)
// holds 506 values: Perlin's 256, then the same list without its first six
// entries; aggregate initialisation zero-fills the last six.
std::array<int, 512> reference_perm512() {
    std::array<int, 512> p{};
    for (int i = 0; i < 256; i++) p[i] = kPerlin[i];
    for (int k = 0; k < 250; k++) p[256 + k] = kPerlin[6 + k];
    for (int i = 506; i < 512; i++) p[i] = 0;
    return p;
}

// Jenkins one-at-a-time over the four little-endian bytes of the key
// (compute_density_field.cpp:68-86).
uint32_t noise_hash(int x, int y, int seed) {
    const uint32_t key = (uint32_t)(((uint32_t)x << 24) | ((uint32_t)y << 16)) ^ (uint32_t)seed;
    uint32_t hash = 0;
    for (int i = 0; i < 4; i++) {
        hash += (key >> (8 * i)) & 0xffu;
        hash += (hash << 10);
        hash ^= (hash >> 6);
    }
    hash += (hash << 3);
    hash ^= (hash >> 11);
    hash += (hash << 15);
    return hash;
}

struct PermLut {
    uint8_t v[65536];   // alpha channel: shuffled permutation value per texel
    float g[16][3];     // RGB channel as read_imagef returns it: (b/255)*4-1
};

PermLut g_lut;
bool g_lut_ready = false;

// CreateNoisePermutationLookupImage (compute_density_field.cpp:90-125)
void build_lut(int seed, PermLut* L) {
    std::array<int, 512> shuffled = reference_perm512();
    std::shuffle(shuffled.begin(), shuffled.end(), std::default_random_engine(seed));
    for (int i = 0; i < 256; i++) {
        for (int j = 0; j < 256; j++) {
            const uint8_t value = (uint8_t)shuffled[noise_hash(i, j, seed) & 0x1ff];
            L->v[i * 256 + j] = value;  // row i (v coordinate), column j (u)
        }
    }
    for (int k = 0; k < 16; k++) {
        for (int c = 0; c < 3; c++) {
            const unsigned char b = (unsigned char)(kGrad3[k][c] * 64 + 64);
            L->g[k][c] = ((float)b / 255.0f) * 4.0f - 1.0f;
        }
    }
}

inline int texel(int row, int col) { return ((row & 255) << 8) | (col & 255); }
// u = A/255 as a normalised coordinate: column A, except A == 255 -> 1.0 -> 0
inline int alpha_column(int a) { return a == 255 ? 0 : a; }

// ---------------------------------------------------------------------------
// Operation counting.  The density and edge arithmetic below is written once
// for a scalar R: float for the restatement, Counted to count its FP32
// operations (the FLOP figures of the roofline): add, sub, mul, div, sqrt
// and floor count 1, an fma counts 2 (its two source operations);
// comparisons, min / max, abs and negation are free.  A Counted run takes
// every simplex corner and every normalisation, as the branch-free kernels
// execute them; the values it computes are not used.
// ---------------------------------------------------------------------------

struct Counted {
    float v = 0.f;
    static thread_local uint64_t ops;
    Counted() = default;
    Counted(float f) : v(f) {}  // literals and constants: free
    explicit operator int() const { return (int)v; }
};
thread_local uint64_t Counted::ops = 0;
inline Counted operator+(Counted a, Counted b) { ++Counted::ops; return Counted(a.v + b.v); }
inline Counted operator-(Counted a, Counted b) { ++Counted::ops; return Counted(a.v - b.v); }
inline Counted operator*(Counted a, Counted b) { ++Counted::ops; return Counted(a.v * b.v); }
inline Counted operator/(Counted a, Counted b) { ++Counted::ops; return Counted(a.v / b.v); }
inline Counted operator-(Counted a) { return Counted(-a.v); }
inline Counted& operator+=(Counted& a, Counted b) { return a = a + b; }
inline bool operator<(Counted a, Counted b) { return a.v < b.v; }
inline bool operator>(Counted a, Counted b) { return a.v > b.v; }
inline bool operator<=(Counted a, Counted b) { return a.v <= b.v; }
inline bool operator>=(Counted a, Counted b) { return a.v >= b.v; }
inline bool operator==(Counted a, Counted b) { return a.v == b.v; }
inline bool operator!=(Counted a, Counted b) { return a.v != b.v; }

template <class R> constexpr bool kCounting = false;
template <> constexpr bool kCounting<Counted> = true;

inline float r_fma(float a, float b, float c) { return std::fmaf(a, b, c); }
inline Counted r_fma(Counted a, Counted b, Counted c) {
    Counted::ops += 2;
    return Counted(std::fmaf(a.v, b.v, c.v));
}
inline float r_floor(float x) { return std::floor(x); }
inline Counted r_floor(Counted x) { ++Counted::ops; return Counted(std::floor(x.v)); }
inline float r_sqrt(float x) { return std::sqrt(x); }
inline Counted r_sqrt(Counted x) { ++Counted::ops; return Counted(std::sqrt(x.v)); }
inline float r_abs(float x) { return std::fabs(x); }
inline Counted r_abs(Counted x) { return Counted(std::fabs(x.v)); }
template <class R> inline R r_clamp01(R x) { return x < R(0.f) ? R(0.f) : (x > R(1.f) ? R(1.f) : x); }

// ---------------------------------------------------------------------------
// Simplex noise: simplex.cl:158-289 (Gustavson, public domain)
// ---------------------------------------------------------------------------

template <class R> inline R dot2_t(R ax, R ay, R bx, R by) { return r_fma(ay, by, ax * bx); }
template <class R> inline R dot3_t(R ax, R ay, R az, R bx, R by, R bz) { return r_fma(az, bz, r_fma(ay, by, ax * bx)); }
inline float dot2(float ax, float ay, float bx, float by) { return dot2_t<float>(ax, ay, bx, by); }
inline float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return dot3_t<float>(ax, ay, az, bx, by, bz);
}

const float F2 = 0.366025403784f;
const float G2 = 0.211324865405f;
const float F3 = 0.333333333333f;
const float G3 = 0.166666666667f;

template <class R>
R snoise2_t(R px, R py, const PermLut& L) {
    const float c2 = 1.f - 2.f * G2;
    const R s = (px + py) * R(F2);
    const R pix = r_floor(px + s);
    const R piy = r_floor(py + s);
    const R t = (pix + piy) * R(G2);
    const R x0 = px - (pix - t);
    const R y0 = py - (piy - t);
    const int ix = (int)pix, iy = (int)piy;
    const int o1x = x0 > y0 ? 1 : 0;
    const int o1y = 1 - o1x;

    R n0 = 0.f, n1 = 0.f, n2 = 0.f;
    {
        const float* g = L.g[L.v[texel(iy, ix)] & 15];
        R t0 = R(0.5f) - dot2_t<R>(x0, y0, x0, y0);
        if (kCounting<R> || !(t0 < R(0.f))) { t0 = t0 * t0; n0 = (t0 * t0) * dot2_t<R>(g[0], g[1], x0, y0); }
    }
    const R x1 = (x0 - R((float)o1x)) + R(G2), y1 = (y0 - R((float)o1y)) + R(G2);
    {
        const float* g = L.g[L.v[texel(iy + o1y, ix + o1x)] & 15];
        R t1 = R(0.5f) - dot2_t<R>(x1, y1, x1, y1);
        if (kCounting<R> || !(t1 < R(0.f))) { t1 = t1 * t1; n1 = (t1 * t1) * dot2_t<R>(g[0], g[1], x1, y1); }
    }
    const R x2 = x0 - R(c2), y2 = y0 - R(c2);
    {
        const float* g = L.g[L.v[texel(iy + 1, ix + 1)] & 15];
        R t2 = R(0.5f) - dot2_t<R>(x2, y2, x2, y2);
        if (kCounting<R> || !(t2 < R(0.f))) { t2 = t2 * t2; n2 = (t2 * t2) * dot2_t<R>(g[0], g[1], x2, y2); }
    }
    return R(70.f) * ((n0 + n1) + n2);
}

template <class R>
R snoise3_t(R px, R py, R pz, const PermLut& L) {
    const float c2 = 2.f * G3;
    const float c3 = 1.f - 3.f * G3;
    const R s = ((px + py) + pz) * R(F3);
    const R pix = r_floor(px + s);
    const R piy = r_floor(py + s);
    const R piz = r_floor(pz + s);
    const R t = ((pix + piy) + piz) * R(G3);
    const R x0 = px - (pix - t);
    const R y0 = py - (piy - t);
    const R z0 = pz - (piz - t);
    const int ix = (int)pix, iy = (int)piy, iz = (int)piz;

    // simplex() (simplex.cl:133-156): rank the components of Pf0
    const int isx_y = x0 >= y0 ? 1 : 0;  // step(P.y, P.x)
    const int isx_z = x0 >= z0 ? 1 : 0;  // step(P.z, P.x)
    const int isy_z = y0 >= z0 ? 1 : 0;  // step(P.z, P.y)
    const int off_x = isx_y + isx_z;
    const int off_y = (1 - isx_y) + isy_z;
    const int off_z = (1 - isx_z) + (1 - isy_z);
    const int o2x = std::min(std::max(off_x, 0), 1), o2y = std::min(std::max(off_y, 0), 1),
              o2z = std::min(std::max(off_z, 0), 1);
    const int o1x = std::min(std::max(off_x - 1, 0), 1), o1y = std::min(std::max(off_y - 1, 0), 1),
              o1z = std::min(std::max(off_z - 1, 0), 1);

    auto corner = [&](int dx, int dy, int dz, R x, R y, R z) -> R {
        const int a = L.v[texel(iy + dy, ix + dx)];
        const float* g = L.g[L.v[texel(iz + dz, alpha_column(a))] & 15];
        R tt = R(0.6f) - dot3_t<R>(x, y, z, x, y, z);
        if (!kCounting<R> && tt < R(0.f)) return R(0.f);
        tt = tt * tt;
        return (tt * tt) * dot3_t<R>(g[0], g[1], g[2], x, y, z);
    };

    const R n0 = corner(0, 0, 0, x0, y0, z0);
    const R x1 = (x0 - R((float)o1x)) + R(G3), y1 = (y0 - R((float)o1y)) + R(G3), z1 = (z0 - R((float)o1z)) + R(G3);
    const R n1 = corner(o1x, o1y, o1z, x1, y1, z1);
    const R x2 = (x0 - R((float)o2x)) + R(c2), y2 = (y0 - R((float)o2y)) + R(c2), z2 = (z0 - R((float)o2z)) + R(c2);
    const R n2 = corner(o2x, o2y, o2z, x2, y2, z2);
    const R x3 = x0 - R(c3), y3 = y0 - R(c3), z3 = z0 - R(c3);
    const R n3 = corner(1, 1, 1, x3, y3, z3);
    return R(32.f) * (((n0 + n1) + n2) + n3);
}

inline float snoise2(float px, float py, const PermLut& L) { return snoise2_t<float>(px, py, L); }
inline float snoise3(float px, float py, float pz, const PermLut& L) { return snoise3_t<float>(px, py, pz, L); }

// ---------------------------------------------------------------------------
// Fractals and density: noise.cl:8-81, 205-268
// ---------------------------------------------------------------------------

// BasicFractal (noise.cl:8-36); NOISE_SCALE == 1
template <class R>
R basic_fractal_t(int octaves, R frequency, R lacunarity, R persistence, R x, R y, const PermLut& L) {
    R px = x * R(1.f), py = y * R(1.f);
    R noise = 0.f, amplitude = 1.f;
    px = px * frequency;
    py = py * frequency;
    for (int i = 0; i < octaves; i++) {
        noise = r_fma(snoise2_t<R>(px, py, L), amplitude, noise);
        px = px * lacunarity;
        py = py * lacunarity;
        amplitude = amplitude * persistence;
    }
    return noise;
}

// 3D analogue of BasicFractal for the cave term of the caves density mode
template <class R>
R basic_fractal3_t(int octaves, R frequency, R lacunarity, R persistence, R x, R y, R z, const PermLut& L) {
    R px = x * frequency, py = y * frequency, pz = z * frequency;
    R noise = 0.f, amplitude = 1.f;
    for (int i = 0; i < octaves; i++) {
        noise = r_fma(snoise3_t<R>(px, py, pz, L), amplitude, noise);
        px = px * lacunarity;
        py = py * lacunarity;
        pz = pz * lacunarity;
        amplitude = amplitude * persistence;
    }
    return noise;
}

// RidgedMultiFractal (noise.cl:42-81) with RIDGED_MULTI_H == 1
template <class R>
R ridged_multi_fractal_t(int octaves, R lacunarity, R gain, R offset, R x, R y, const PermLut& L) {
    R px = x * R(1.f), py = y * R(1.f);
    R signal = snoise2_t<R>(px, py, L);
    signal = r_abs(signal);
    signal = offset - signal;
    signal = signal * signal;
    R noise = signal;
    R weight = 1.f;
    R frequency = 1.f;
    for (int i = 0; i < octaves; i++) {
        px = px * lacunarity;
        py = py * lacunarity;
        weight = signal * gain;
        weight = r_clamp01(weight);
        signal = snoise2_t<R>(px, py, L);
        signal = r_abs(signal);
        signal = offset - signal;
        signal = signal * weight;
        const R exponent = R(1.f) / frequency;
        frequency = frequency * lacunarity;
        noise = r_fma(signal, exponent, noise);
    }
    noise = noise * R(1.f / (float)octaves);
    return noise;
}

// Terrain (noise.cl:205-223)
template <class R>
R terrain_t(R x, R z, const PermLut& L) {
    const R px = x * R(1.f / 2000.f);
    const R pz = z * R(1.f / 2000.f);
    R ridged = R(0.8f) * ridged_multi_fractal_t<R>(7, 2.114352f, 1.5241f, 1.f, px, pz, L);
    ridged = r_clamp01(ridged);
    R billow = R(0.6f) * basic_fractal_t<R>(4, 0.24f, 1.8754f, 0.433f, R(-4.33f) * px, R(7.98f) * pz, L);
    billow = r_fma(R(0.5f), billow, R(0.5f));
    R b2 = R(0.6f) * basic_fractal_t<R>(2, 0.63f, 2.2f, 0.15f, px, pz, L);
    b2 = r_fma(b2, R(0.5f), R(0.5f));
    return r_fma(billow, ridged, b2);
}

// the height term h(x, z) of a heightfield mode (density = y - amp2 h [+ caves])
template <class R>
R height_t(const orc_density& d, R x, R z, const PermLut& L) {
    return basic_fractal_t<R>(d.octaves2, d.freq2, d.lacunarity2, d.gain2, x, z, L);
}

// DensityFunc (noise.cl:225-268) and the two heightfield modes
template <class R>
R density_t(const orc_density& d, R x, R y, R z, const PermLut& L) {
    switch (d.mode) {
        case 0:
            return r_fma(R(-900.f), terrain_t<R>(x, z, L), y);  // MAX_TERRAIN_HEIGHT = 900
        case 1: {
            const R h = height_t<R>(d, x, z, L);
            return r_fma(-R(d.amp2), h, y);
        }
        default: {
            const R h = height_t<R>(d, x, z, L);
            const R base = r_fma(-R(d.amp2), h, y);
            const R c = basic_fractal3_t<R>(d.octaves3, d.freq3, d.lacunarity3, d.gain3, x, y, z, L);
            return r_fma(R(d.amp3), c, base);
        }
    }
}

inline float basic_fractal(int octaves, float frequency, float lacunarity, float persistence, float x, float y,
                           const PermLut& L) {
    return basic_fractal_t<float>(octaves, frequency, lacunarity, persistence, x, y, L);
}
inline float density(const orc_density& d, float x, float y, float z, const PermLut& L) {
    return density_t<float>(d, x, y, z, L);
}

// ---------------------------------------------------------------------------
// Chunk geometry (compute.cpp:245-282)
// ---------------------------------------------------------------------------

struct Dims {
    int vpc;      // VOXELS_PER_CHUNK
    int hdim;     // HERMITE_INDEX_SIZE = vpc + 1
    int fdim;     // FIELD_DIM = vpc + 2
    int shift;    // VOXEL_INDEX_SHIFT = log2(vpc) + 1
    int mask;     // VOXEL_INDEX_MASK
    int depth;    // MAX_OCTREE_DEPTH = log2(vpc)
    explicit Dims(int v) : vpc(v), hdim(v + 1), fdim(v + 2) {
        int l = 0;
        while ((1 << l) < v) l++;
        depth = l;
        shift = l + 1;
        mask = (1 << shift) - 1;
    }
    int field_index(int x, int y, int z) const { return x + y * fdim + z * fdim * fdim; }
    int field_size() const { return fdim * fdim * fdim; }
};

const int kChildMinOffsets[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 0}, {0, 1, 1},
                                    {1, 0, 0}, {1, 0, 1}, {1, 1, 0}, {1, 1, 1}};  // shared_constants.cl:11-22
const int kEdgeMap[12][2] = {{0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 2}, {1, 3},
                             {4, 6}, {5, 7}, {0, 1}, {2, 3}, {4, 5}, {6, 7}};  // shared_constants.cl:4-9
const int kEdgeNodeOffsets[3][4][3] = {  // octree.cl:376-381
    {{0, 0, 0}, {0, 0, 1}, {0, 1, 0}, {0, 1, 1}},
    {{0, 0, 0}, {1, 0, 0}, {0, 0, 1}, {1, 0, 1}},
    {{0, 0, 0}, {0, 1, 0}, {1, 0, 0}, {1, 1, 0}}};
const int kAxisOffset[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

struct F4 {
    float x, y, z, w;
};

// ---------------------------------------------------------------------------
// FindNextPrime: primes.cpp:9-58
// ---------------------------------------------------------------------------

bool is_prime(int x) {
    int o = 4;
    int i = 5;
    while (true) {
        const int q = x / i;
        if (q < i) return true;
        if (x == q * i) return false;
        o ^= 6;
        i += o;
    }
}

int find_next_prime(int n) {
    if (n <= 2) return 2;
    if (n == 3) return 3;
    if (n <= 5) return 5;
    const int k = n / 6;
    int i = n - 6 * k;
    const int o = i < 2 ? 1 : 5;
    int x = 6 * k + o;
    for (i = (3 + o) / 2; !is_prime(x); x += i) i ^= 6;
    return x;
}

// ---------------------------------------------------------------------------
// Cuckoo hash: cuckoo.cl:1-105, compute_cuckoo.cpp:46-139, compute_cuckoo.h:6-10
// ---------------------------------------------------------------------------

constexpr uint64_t CUCKOO_EMPTY = ~0ull;
constexpr int CUCKOO_STASH_HASH_INDEX = 4;
constexpr int CUCKOO_HASH_FN_COUNT = 5;
constexpr int CUCKOO_STASH_SIZE = 101;
constexpr int CUCKOO_MAX_ITERATIONS = 32;
constexpr uint32_t CUCKOO_MIN_TABLE_SIZE = 2048u;

// Cuckoo_Hash (cuckoo.cl:18-24): the product a*key wraps at 32 bits
inline uint32_t cuckoo_hash(int which, uint32_t key, uint32_t a, uint32_t b, uint32_t prime) {
    const uint64_t p = 4294967291ull;
    const uint64_t h = (uint32_t)(a * key);
    const uint64_t mod = which < CUCKOO_STASH_HASH_INDEX ? prime : (uint64_t)CUCKOO_STASH_SIZE;
    return (uint32_t)(((h + b) % p) % mod);
}

struct Cuckoo {
    uint32_t prime = 0;
    std::vector<uint64_t> table;
    uint64_t stash[CUCKOO_STASH_SIZE];
    uint32_t params[CUCKOO_HASH_FN_COUNT * 2];
    bool stash_used = false;

    // one pass of Cuckoo_InsertKeys (cuckoo.cl:26-71) executed key by key;
    // the stash slot is the stash hash mod STASH_SIZE (the reference passes
    // whichHash 0 there, which indexes the 101-entry stash modulo the table
    // prime -- an out-of-bounds write; the intent is restated).
    bool insert_all(const uint32_t* keys, int n, bool* used_stash) {
        bool ok = true;
        *used_stash = false;
        for (int index = 0; index < n; index++) {
            uint32_t key = keys[index];
            uint64_t entry = ((uint64_t)(uint32_t)index << 32) | key;
            uint32_t h = cuckoo_hash(0, key, params[0], params[1], prime);
            bool done = false;
            for (int i = 0; i < CUCKOO_MAX_ITERATIONS; i++) {
                std::swap(table[h], entry);
                if (entry == CUCKOO_EMPTY) { done = true; break; }
                key = (uint32_t)(entry & 0xffffffffu);
                const uint32_t h0 = cuckoo_hash(0, key, params[0], params[1], prime);
                const uint32_t h1 = cuckoo_hash(1, key, params[2], params[3], prime);
                const uint32_t h2 = cuckoo_hash(2, key, params[4], params[5], prime);
                const uint32_t h3 = cuckoo_hash(3, key, params[6], params[7], prime);
                if (h == h0) h = h1;
                else if (h == h1) h = h2;
                else if (h == h2) h = h3;
                else if (h == h3) h = h0;
            }
            if (done) continue;
            *used_stash = true;
            key = (uint32_t)(entry & 0xffffffffu);
            const uint32_t hs = cuckoo_hash(CUCKOO_STASH_HASH_INDEX, key, params[8], params[9], prime);
            if (stash[hs] == CUCKOO_EMPTY) stash[hs] = entry;
            else ok = false;
        }
        return ok;
    }

    // Cuckoo_Find (cuckoo.cl:73-104) with the stash probe reading the stash
    // (the reference reads data[h] there).
    uint32_t find(uint32_t key) const {
        for (int i = 0; i < CUCKOO_STASH_HASH_INDEX; i++) {
            const uint32_t h = cuckoo_hash(i, key, params[2 * i], params[2 * i + 1], prime);
            const uint64_t e = table[h];
            if ((uint32_t)(e & 0xffffffffu) == key) return (uint32_t)(e >> 32);
        }
        if (stash_used) {
            const uint32_t h = cuckoo_hash(CUCKOO_STASH_HASH_INDEX, key, params[8], params[9], prime);
            const uint64_t e = stash[h];
            if ((uint32_t)(e & 0xffffffffu) == key) return (uint32_t)(e >> 32);
        }
        return ~0u;
    }
};

// Cuckoo_InitialiseTable + Cuckoo_InsertKeys host loop (compute_cuckoo.cpp:49-139):
// a fresh parameter set is drawn until every key inserts.
void cuckoo_build(Cuckoo* c, const uint32_t* keys, int n, std::mt19937& gen, int* retries) {
    std::uniform_int_distribution<uint32_t> dist(1u << 15, 1u << 30);
    c->prime = (uint32_t)find_next_prime((int)std::max(CUCKOO_MIN_TABLE_SIZE, (uint32_t)n * 2u));
    int attempts = 0;
    for (;;) {
        for (int i = 0; i < CUCKOO_HASH_FN_COUNT * 2; i++) c->params[i] = dist(gen);
        c->table.assign(c->prime, CUCKOO_EMPTY);
        for (int i = 0; i < CUCKOO_STASH_SIZE; i++) c->stash[i] = CUCKOO_EMPTY;
        bool used = false;
        const bool ok = c->insert_all(keys, n, &used);
        if (ok) {
            c->stash_used = used;
            break;
        }
        attempts++;
    }
    if (retries) *retries = attempts;
}

// ---------------------------------------------------------------------------
// RemoveDuplicates: compute.cpp:450-543, duplicate.cl:4-114
// ---------------------------------------------------------------------------

// MurmurHash (duplicate.cl:4-28); the seed argument is unused by the reference
inline uint32_t murmur(uint32_t value) {
    const uint32_t c1 = 0xcc9e2d51u, c2 = 0x1b873593u;
    uint32_t hash = value;
    hash *= c1;
    hash = (hash << 15) | (hash >> 17);
    hash *= c2;
    hash ^= value;
    hash = ((hash << 13) | (hash >> 19)) * 5u + 0xe6546b64u;
    hash ^= (hash >> 16);
    hash *= 0x85ebca6bu;
    hash ^= (hash >> 13);
    hash *= 0xc2b2ae35u;
    hash ^= (hash >> 16);
    return hash;
}

// The reference's racy `table[hash] = id` (MapSequenceIndices) is restated
// as a sequential loop, i.e. the highest sequence index wins a slot.
std::vector<int32_t> remove_duplicates(const std::vector<int32_t>& input) {
    std::vector<int32_t> result;
    const int n0 = (int)input.size();
    if (n0 == 0) return result;
    const uint32_t prime = (uint32_t)find_next_prime(n0 * 2);
    std::vector<int32_t> table(prime);
    std::vector<int32_t> sequence = input;
    while (!sequence.empty()) {
        std::fill(table.begin(), table.end(), -1);
        for (int id = 0; id < (int)sequence.size(); id++) table[murmur((uint32_t)sequence[id]) % prime] = id;
        std::vector<int32_t> winners;
        for (uint32_t s = 0; s < prime; s++)
            if (table[s] != -1) winners.push_back(sequence[table[s]]);
        result.insert(result.end(), winners.begin(), winners.end());
        for (int32_t w : winners) table[murmur((uint32_t)w) % prime] = w;
        std::vector<int32_t> losers;
        for (int32_t v : sequence)
            if (table[murmur((uint32_t)v) % prime] != v) losers.push_back(v);
        if (losers.empty()) break;
        sequence.swap(losers);
    }
    return result;
}

// ---------------------------------------------------------------------------
// CSG brushes: apply_csg_operation.cl:42-175, hg_sdf.glsl fBox / pR
// ---------------------------------------------------------------------------

struct Brush {
    orc_csg_op op;
    float c, s;  // cos / sin of rotate_y, evaluated once in double on the host
};

inline float length3(float x, float y, float z) { return std::sqrt(dot3(x, y, z, x, y, z)); }

// Density_Cuboid (apply_csg_operation.cl:49-68): pR rotation then fBox
float density_cuboid(float wx, float wy, float wz, const Brush& b) {
    const float lx = wx - b.op.origin[0], ly = wy - b.op.origin[1], lz = wz - b.op.origin[2];
    // pR(p.xz, a): p = cos(a)*p + sin(a)*(p.y, -p.x)   (hg_sdf.glsl:460-463)
    const float rx = std::fmaf(b.s, lz, b.c * lx);
    const float rz = std::fmaf(b.s, -lx, b.c * lz);
    // fBox (hg_sdf.glsl:218-221)
    const float dx = std::fabs(rx) - b.op.dimensions[0];
    const float dy = std::fabs(ly) - b.op.dimensions[1];
    const float dz = std::fabs(rz) - b.op.dimensions[2];
    const float outside = length3(std::max(dx, 0.f), std::max(dy, 0.f), std::max(dz, 0.f));
    const float inside = std::max(std::max(std::min(dx, 0.f), std::min(dy, 0.f)), std::min(dz, 0.f));
    return outside + inside;
}

// Density_Sphere (apply_csg_operation.cl:42-45)
float density_sphere(float wx, float wy, float wz, const Brush& b) {
    return length3(wx - b.op.origin[0], wy - b.op.origin[1], wz - b.op.origin[2]) - b.op.dimensions[0];
}

// BrushDensity (apply_csg_operation.cl:72-81)
inline float brush_density(float x, float y, float z, const Brush& b) {
    return b.op.brush == 0 ? density_cuboid(x, y, z, b) : density_sphere(x, y, z, b);
}

// BrushMaterial (apply_csg_operation.cl:114-140)
int brush_material(float x, float y, float z, const std::vector<Brush>& ops, int material) {
    int m = material;
    for (const Brush& b : ops)
        if (brush_density(x, y, z, b) <= 0.f) m = b.op.type == 0 ? b.op.material : MATERIAL_AIR;
    return m;
}

inline void normalize3(float& x, float& y, float& z) {
    const float len = std::sqrt(dot3(x, y, z, x, y, z));
    if (len == 0.f) { x = y = z = 0.f; return; }
    x = x / len;
    y = y / len;
    z = z / len;
}

// BrushZeroCrossing (apply_csg_operation.cl:86-110)
float brush_zero_crossing(const F4& p0, const F4& p1, const std::vector<Brush>& ops) {
    float min_density = FLT_MAX;
    float crossing = 0.f;
    for (float t = 0.f; t <= 1.f; t += (1.f / 16.f)) {
        const float px = std::fmaf(p1.x - p0.x, t, p0.x);
        const float py = std::fmaf(p1.y - p0.y, t, p0.y);
        const float pz = std::fmaf(p1.z - p0.z, t, p0.z);
        for (const Brush& b : ops) {
            const float d = std::fabs(brush_density(px, py, pz, b));
            if (d < min_density) { crossing = t; min_density = d; }
        }
    }
    return crossing;
}

// BrushNormal (apply_csg_operation.cl:144-175)
void brush_normal(float px, float py, float pz, const std::vector<Brush>& ops, float n[3]) {
    n[0] = n[1] = n[2] = 0.f;
    const float h = 0.001f;
    for (const Brush& b : ops) {
        if (brush_density(px, py, pz, b) > 0.f) continue;
        float gx = brush_density(px + h, py, pz, b) - brush_density(px - h, py, pz, b);
        float gy = brush_density(px, py + h, pz, b) - brush_density(px, py - h, pz, b);
        float gz = brush_density(px, py, pz + h, b) - brush_density(px, py, pz - h, b);
        normalize3(gx, gy, gz);
        const float flip = b.op.type == 0 ? 1.f : -1.f;
        n[0] = flip * gx;
        n[1] = flip * gy;
        n[2] = flip * gz;
    }
}

// ---------------------------------------------------------------------------
// QEF: qef.cl:1-305
// ---------------------------------------------------------------------------

struct QEF {
    float ata[6];
    float pad[2];
    F4 atb;
    F4 masspoint;
};
static_assert(sizeof(QEF) == 64, "QEFData layout (qef.cl:7-14): 8 floats + 2 float4");

inline float dot4(const F4& a, const F4& b) {
    return std::fmaf(a.w, b.w, std::fmaf(a.z, b.z, std::fmaf(a.y, b.y, a.x * b.x)));
}

// qef_add_point (qef.cl:170-191)
void qef_add_point(QEF& q, const F4& n, const F4& p) {
    q.ata[0] += n.x * n.x;
    q.ata[1] += n.x * n.y;
    q.ata[2] += n.x * n.z;
    q.ata[3] += n.y * n.y;
    q.ata[4] += n.y * n.z;
    q.ata[5] += n.z * n.z;
    const float b = dot4(p, n);
    q.atb.x += n.x * b;
    q.atb.y += n.y * b;
    q.atb.z += n.z * b;
    q.masspoint.x += p.x;
    q.masspoint.y += p.y;
    q.masspoint.z += p.z;
    q.masspoint.w += 1.f;
}

typedef float Mat3[3][3];

// givens_coeffs_sym (qef.cl:31-42)
void givens_coeffs_sym(float a_pp, float a_pq, float a_qq, float* c, float* s) {
    if (a_pq == 0.f) { *c = 1.f; *s = 0.f; return; }
    const float tau = (a_qq - a_pp) / (2.f * a_pq);
    const float stt = std::sqrt(1.f + tau * tau);
    const float tn = 1.f / ((tau >= 0.f) ? (tau + stt) : (tau - stt));
    *c = 1.f / std::sqrt(1.f + tn * tn);
    *s = tn * (*c);
}

inline void svd_rotate_xy(float& x, float& y, float c, float s) {
    const float u = x, v = y;
    x = c * u - s * v;
    y = s * u + c * v;
}

inline void svd_rotateq_xy(float& x, float& y, float a, float c, float s) {
    const float cc = c * c, ss = s * s;
    const float mx = 2.f * c * s * a;
    const float u = x, v = y;
    x = cc * u - mx + ss * v;
    y = ss * u + mx + cc * v;
}

// svd_rotate (qef.cl:58-86)
void svd_rotate(Mat3 vtav, Mat3 v, int a, int b) {
    if (vtav[a][b] == 0.f) return;
    float c, s;
    givens_coeffs_sym(vtav[a][a], vtav[a][b], vtav[b][b], &c, &s);
    float x = vtav[a][a], y = vtav[b][b];
    svd_rotateq_xy(x, y, vtav[a][b], c, s);
    vtav[a][a] = x;
    vtav[b][b] = y;
    x = vtav[0][3 - b];
    y = vtav[1 - a][2];
    svd_rotate_xy(x, y, c, s);
    vtav[0][3 - b] = x;
    vtav[1 - a][2] = y;
    vtav[a][b] = 0.f;
    for (int r = 0; r < 3; r++) {
        x = v[r][a];
        y = v[r][b];
        svd_rotate_xy(x, y, c, s);
        v[r][a] = x;
        v[r][b] = y;
    }
}

inline float svd_invdet(float x, float tol) {
    return (std::fabs(x) < tol || std::fabs(1.f / x) < tol) ? 0.f : (1.f / x);
}

// qef_solve (qef.cl:239-256) via svd_solve_ATA_ATb (qef.cl:127-144), 10 sweeps
F4 qef_solve(QEF q) {
    const float w = std::max(q.masspoint.w, 1.f);
    q.masspoint.x /= w;
    q.masspoint.y /= w;
    q.masspoint.z /= w;
    q.masspoint.w /= w;
    const float* A = q.ata;
    const F4 mp = q.masspoint;
    // svd_vmul_sym (qef.cl:146-152)
    F4 amp;
    amp.x = dot4(F4{A[0], A[1], A[2], 0.f}, mp);
    amp.y = A[1] * mp.x + A[3] * mp.y + A[4] * mp.z;
    amp.z = A[2] * mp.x + A[4] * mp.y + A[5] * mp.z;
    amp.w = 0.f;
    amp.x = q.atb.x - amp.x;
    amp.y = q.atb.y - amp.y;
    amp.z = q.atb.z - amp.z;
    amp.w = q.atb.w - amp.w;

    Mat3 V = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}};
    Mat3 vtav = {{A[0], A[1], A[2]}, {0.f, A[3], A[4]}, {0.f, 0.f, A[5]}};
    for (int i = 0; i < 10; i++) {
        svd_rotate(vtav, V, 0, 1);
        svd_rotate(vtav, V, 0, 2);
        svd_rotate(vtav, V, 1, 2);
    }
    const float d0 = svd_invdet(vtav[0][0], 0.1f);
    const float d1 = svd_invdet(vtav[1][1], 0.1f);
    const float d2 = svd_invdet(vtav[2][2], 0.1f);
    Mat3 o;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            o[r][c] = V[r][0] * d0 * V[c][0] + V[r][1] * d1 * V[c][1] + V[r][2] * d2 * V[c][2];
    F4 x;
    x.x = dot4(F4{o[0][0], o[0][1], o[0][2], 0.f}, amp);
    x.y = dot4(F4{o[1][0], o[1][1], o[1][2], 0.f}, amp);
    x.z = dot4(F4{o[2][0], o[2][1], o[2][2], 0.f}, amp);
    x.w = 0.f;
    x.x += mp.x;
    x.y += mp.y;
    x.z += mp.z;
    x.w += mp.w;
    return x;
}

// FP64 restatement of the same leaf solve, for stating the FP32 solve's
// error: qef_add_point (qef.cl:170-191) accumulated in double from the same
// crossing points and normals, then qef_solve (qef.cl:239-256) with its
// Jacobi sweeps (qef.cl:23-105), the pseudo-inverse truncation at 0.1
// (svd_invdet, qef.cl:107-111) and the mass-point bias, all in double.  Ten
// sweeps as qef.cl:16; in double they converge a 3x3 symmetric matrix fully.
struct QEF64 {
    double ata[6] = {0, 0, 0, 0, 0, 0};
    double atb[3] = {0, 0, 0};
    double mp[4] = {0, 0, 0, 0};
};

void qef64_add_point(QEF64& q, const double n[3], const double p[3]) {
    q.ata[0] += n[0] * n[0];
    q.ata[1] += n[0] * n[1];
    q.ata[2] += n[0] * n[2];
    q.ata[3] += n[1] * n[1];
    q.ata[4] += n[1] * n[2];
    q.ata[5] += n[2] * n[2];
    const double b = p[0] * n[0] + p[1] * n[1] + p[2] * n[2];
    for (int i = 0; i < 3; i++) q.atb[i] += n[i] * b;
    for (int i = 0; i < 3; i++) q.mp[i] += p[i];
    q.mp[3] += 1.0;
}

void svd64_rotate(double vtav[3][3], double v[3][3], int a, int b) {
    if (vtav[a][b] == 0.0) return;
    // givens_coeffs_sym (qef.cl:31-42)
    const double tau = (vtav[b][b] - vtav[a][a]) / (2.0 * vtav[a][b]);
    const double stt = std::sqrt(1.0 + tau * tau);
    const double tn = 1.0 / (tau >= 0.0 ? tau + stt : tau - stt);
    const double c = 1.0 / std::sqrt(1.0 + tn * tn), s = tn * c;
    // svd_rotateq_xy / svd_rotate_xy (qef.cl:44-56), on the same entries as svd_rotate
    const double cc = c * c, ss = s * s, mx = 2.0 * c * s * vtav[a][b];
    const double u = vtav[a][a], w = vtav[b][b];
    vtav[a][a] = cc * u - mx + ss * w;
    vtav[b][b] = ss * u + mx + cc * w;
    const double x = vtav[0][3 - b], y = vtav[1 - a][2];
    vtav[0][3 - b] = c * x - s * y;
    vtav[1 - a][2] = s * x + c * y;
    vtav[a][b] = 0.0;
    for (int r = 0; r < 3; r++) {
        const double p = v[r][a], q = v[r][b];
        v[r][a] = c * p - s * q;
        v[r][b] = s * p + c * q;
    }
}

inline double svd64_invdet(double x, double tol) {
    return (std::fabs(x) < tol || std::fabs(1.0 / x) < tol) ? 0.0 : 1.0 / x;
}

void qef64_solve(QEF64 q, double out[3]) {
    const double w = std::max(q.mp[3], 1.0);
    const double mp[3] = {q.mp[0] / w, q.mp[1] / w, q.mp[2] / w};
    const double* A = q.ata;
    const double amp[3] = {q.atb[0] - (A[0] * mp[0] + A[1] * mp[1] + A[2] * mp[2]),
                           q.atb[1] - (A[1] * mp[0] + A[3] * mp[1] + A[4] * mp[2]),
                           q.atb[2] - (A[2] * mp[0] + A[4] * mp[1] + A[5] * mp[2])};
    double V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double vtav[3][3] = {{A[0], A[1], A[2]}, {0, A[3], A[4]}, {0, 0, A[5]}};
    for (int i = 0; i < 10; i++) {
        svd64_rotate(vtav, V, 0, 1);
        svd64_rotate(vtav, V, 0, 2);
        svd64_rotate(vtav, V, 1, 2);
    }
    const double d[3] = {svd64_invdet(vtav[0][0], 0.1), svd64_invdet(vtav[1][1], 0.1), svd64_invdet(vtav[2][2], 0.1)};
    for (int r = 0; r < 3; r++) {
        double x = 0.0;
        for (int c = 0; c < 3; c++) {
            const double o = V[r][0] * d[0] * V[c][0] + V[r][1] * d[1] * V[c][1] + V[r][2] * d[2] * V[c][2];
            x += o * amp[c];
        }
        out[r] = x + mp[r];
    }
}

// ---------------------------------------------------------------------------
// Octree codes: octree.cl:3-72
// ---------------------------------------------------------------------------

uint32_t code_for_position(int x, int y, int z, int depth_max) {
    uint32_t code = 1;
    for (int depth = depth_max - 1; depth >= 0; depth--) {
        const uint32_t c = (uint32_t)((((x >> depth) & 1) << 2) | (((y >> depth) & 1) << 1) | ((z >> depth) & 1));
        code = (code << 3) | c;
    }
    return code;
}

void position_for_code(uint32_t code, int depth_max, int p[3]) {
    int msb = 0;
    for (uint32_t c = code; c; c >>= 1) msb++;
    const int node_depth = msb / 3;
    p[0] = p[1] = p[2] = 0;
    for (int i = depth_max - node_depth; i < depth_max; i++) {
        const uint32_t c = code & 7u;
        code >>= 3;
        p[0] |= (int)((c >> 2) & 1u) << i;
        p[1] |= (int)((c >> 1) & 1u) << i;
        p[2] |= (int)(c & 1u) << i;
    }
}

// FindDominantMaterial (octree.cl:96-138)
int dominant_material(const int m[8]) {
    int data[8];
    for (int i = 0; i < 8; i++) data[i] = m[i];
    for (int i = 1; i < 8; i++) {
        const int tmp = data[i];
        int j = i;
        for (; j >= 1 && tmp < data[j - 1]; j--) data[j] = data[j - 1];
        data[j] = tmp;
    }
    int current = data[0], count = 1, max_count = 0, max_material = 0;
    for (int i = 1; i < 8; i++) {
        const int v = data[i];
        if (v == MATERIAL_AIR || v == MATERIAL_NONE) continue;
        if (current != v) {
            if (count > max_count) { max_count = count; max_material = current; }
            current = v;
            count = 1;
        } else {
            count++;
        }
    }
    if (count > max_count) max_material = current;
    return max_material;
}

// ColourForMinLeafSize (clipmap.cpp:329-353)
void colour_for_min_leaf_size(int s, float c[3]) {
    switch (s) {
        case 1: c[0] = 0.3f; c[1] = 0.1f; c[2] = 0.f; break;
        case 2: c[0] = 0.f; c[1] = 0.f; c[2] = 0.5f; break;
        case 4: c[0] = 0.f; c[1] = 0.5f; c[2] = 0.5f; break;
        case 8: c[0] = 0.5f; c[1] = 0.f; c[2] = 0.5f; break;
        case 16: c[0] = 0.f; c[1] = 0.5f; c[2] = 0.f; break;
        default: c[0] = 0.5f; c[1] = 0.f; c[2] = 0.f; break;
    }
}

// ---------------------------------------------------------------------------
// The per-chunk pipeline
// ---------------------------------------------------------------------------

struct Chunk {
    std::vector<int32_t> materials;
    std::vector<int32_t> plain_edge_keys;
    std::vector<int32_t> edge_keys;
    std::vector<F4> edge_info;
    std::vector<int32_t> created_keys;
    std::vector<uint32_t> node_codes;
    std::vector<int32_t> node_edges;
    std::vector<int32_t> node_materials;
    std::vector<QEF> qefs;
    std::vector<F4> positions, normals;
    std::vector<double> positions64;  // 4 doubles per leaf: the FP64 solve, world units
    std::vector<int32_t> triangles;  // 3 ints per triangle
    std::vector<float> vertices;     // 12 floats per MeshVertex
    std::vector<int32_t> seams;      // 12 x 4-byte words per SeamNodeInfo
    int mesh_vertex_count = 0;
    // the chunk's arguments, for the simplification pass
    int vpc = 0, scale = 0, size = 0;
    int min[3] = {0, 0, 0};
    // bottom-up octree simplification (orc_chunk_simplify)
    std::vector<float> simp_vertices;
    std::vector<int32_t> simp_triangles;
    std::vector<int32_t> simp_reps;  // per voxel: anchor | level << 20
    int simp_vertex_count = 0;
};

inline int edge_key(const Dims& D, int x, int y, int z, int axis) {
    return ((x | (y << D.shift) | (z << (2 * D.shift))) << 2) | axis;
}
inline void decode_edge(const Dims& D, int key, int p[3], int* axis) {
    *axis = key & 3;
    const int h = key >> 2;
    p[0] = h & D.mask;
    p[1] = (h >> D.shift) & D.mask;
    p[2] = (h >> (2 * D.shift)) & D.mask;
}

// normalize(v) = v / sqrt(dot(v, v)); a zero vector stays zero
template <class R>
inline void normalize3_t(R& x, R& y, R& z) {
    const R len = r_sqrt(dot3_t<R>(x, y, z, x, y, z));
    if (!kCounting<R> && len == R(0.f)) { x = y = z = R(0.f); return; }
    x = x / len;
    y = y / len;
    z = z / len;
}

// FindEdgeIntersectionInfo (density_field.cl:96-151); crossing_mode 1
// replaces the 17-sample search by linear interpolation of the end densities.
template <class R>
void edge_info_density_t(const Dims& D, const orc_density& dn, const PermLut& L, int key, const int off[3], int scale,
                         int crossing_mode, R out[4]) {
    int lp[3], axis;
    decode_edge(D, key, lp, &axis);
    const int wx = scale * lp[0] + off[0], wy = scale * lp[1] + off[1], wz = scale * lp[2] + off[2];
    const R p0x = (float)wx, p0y = (float)wy, p0z = (float)wz;
    const R p1x = (float)(wx + scale * kAxisOffset[axis][0]), p1y = (float)(wy + scale * kAxisOffset[axis][1]),
            p1z = (float)(wz + scale * kAxisOffset[axis][2]);
    const R ex = p1x - p0x, ey = p1y - p0y, ez = p1z - p0z;  // the edge vector, once
    R t = 0.f;
    if (crossing_mode == 0) {
        R min_value = FLT_MAX;
        R current = 0.f;
        for (int i = 0; i <= 16; i++) {
            const R px = r_fma(ex, current, p0x);
            const R py = r_fma(ey, current, p0y);
            const R pz = r_fma(ez, current, p0z);
            const R d = r_abs(density_t<R>(dn, px, py, pz, L));
            if (d < min_value) { t = current; min_value = d; }
            current += R(0.0625f);
        }
    } else {
        const R d0 = density_t<R>(dn, p0x, p0y, p0z, L);
        const R d1 = density_t<R>(dn, p1x, p1y, p1z, L);
        const R den = d0 - d1;
        t = den != R(0.f) ? d0 / den : R(0.5f);
        t = r_clamp01(t);
    }
    const R px = r_fma(ex, t, p0x);
    const R py = r_fma(ey, t, p0y);
    const R pz = r_fma(ez, t, p0z);
    const R h = 0.001f;
    R nx = density_t<R>(dn, px + h, py, pz, L) - density_t<R>(dn, px - h, py, pz, L);
    R ny = density_t<R>(dn, px, py + h, pz, L) - density_t<R>(dn, px, py - h, pz, L);
    R nz = density_t<R>(dn, px, py, pz + h, L) - density_t<R>(dn, px, py, pz - h, L);
    normalize3_t<R>(nx, ny, nz);
    out[0] = nx;
    out[1] = ny;
    out[2] = nz;
    out[3] = t;
}

F4 edge_info_density(const Dims& D, const orc_density& dn, const PermLut& L, int key, const int off[3],
                     int scale, int crossing_mode) {
    float o[4];
    edge_info_density_t<float>(D, dn, L, key, off, scale, crossing_mode, o);
    return F4{o[0], o[1], o[2], o[3]};
}

// CSG FindEdgeIntersectionInfo (apply_csg_operation.cl:443-477)
F4 edge_info_brush(const Dims& D, int key, const int off[3], int scale, const std::vector<Brush>& ops) {
    int lp[3], axis;
    decode_edge(D, key, lp, &axis);
    const int wx = scale * lp[0] + off[0], wy = scale * lp[1] + off[1], wz = scale * lp[2] + off[2];
    const F4 p0{(float)wx, (float)wy, (float)wz, 0.f};
    const F4 p1{(float)(wx + scale * kAxisOffset[axis][0]), (float)(wy + scale * kAxisOffset[axis][1]),
                (float)(wz + scale * kAxisOffset[axis][2]), 0.f};
    const float t = brush_zero_crossing(p0, p1, ops);
    const float px = std::fmaf(p1.x - p0.x, t, p0.x);
    const float py = std::fmaf(p1.y - p0.y, t, p0.y);
    const float pz = std::fmaf(p1.z - p0.z, t, p0.z);
    float n[3];
    brush_normal(px, py, pz, ops, n);
    return F4{n[0], n[1], n[2], t};
}

std::vector<Brush> make_brushes(const orc_csg_op* ops, int n) {
    std::vector<Brush> out;
    for (int i = 0; i < n; i++) {
        Brush b;
        b.op = ops[i];
        b.c = (float)std::cos((double)ops[i].rotate_y);
        b.s = (float)std::sin((double)ops[i].rotate_y);
        out.push_back(b);
    }
    return out;
}

// ApplyCSGOperations (compute_csg.cpp:11-219)
void apply_csg(const Dims& D, Chunk& ch, const std::vector<Brush>& ops, const int off[3], int scale) {
    if (ops.empty()) return;
    const int F = D.field_size();
    // CSG_HermiteIndices + scan + CompactPoints + UpdateFieldMaterials
    std::vector<int> updated_points;  // field linear indices, ascending
    std::vector<int32_t> new_materials = ch.materials;
    for (int z = 0; z < D.fdim; z++)
        for (int y = 0; y < D.fdim; y++)
            for (int x = 0; x < D.fdim; x++) {
                const int idx = D.field_index(x, y, z);
                const int old = ch.materials[idx];
                const int m = brush_material((float)(off[0] + scale * x), (float)(off[1] + scale * y),
                                             (float)(off[2] + scale * z), ops, old);
                if (m != old) {
                    updated_points.push_back(idx);
                    new_materials[idx] = m;
                }
            }
    if (updated_points.empty()) return;
    ch.materials = new_materials;

    // FindUpdatedEdges + RemoveInvalidIndices + CompactIndexArray
    std::vector<int32_t> generated;
    for (int idx : updated_points) {
        const int x = idx % D.fdim, y = (idx / D.fdim) % D.fdim, z = idx / (D.fdim * D.fdim);
        const int base = (x | (y << D.shift) | (z << (2 * D.shift))) << 2;
        generated.push_back(base | 0);
        generated.push_back(base | 1);
        generated.push_back(base | 2);
        if (x > 0) generated.push_back(edge_key(D, x - 1, y, z, 0));
        if (y > 0) generated.push_back(edge_key(D, x, y - 1, z, 1));
        if (z > 0) generated.push_back(edge_key(D, x, y, z - 1, 2));
    }
    const std::vector<int32_t> invalidated = remove_duplicates(generated);

    // FilterValidEdges (with the PARANOID guard, apply_csg_operation.cl:363-365)
    std::vector<int32_t> created;
    for (int32_t e : invalidated) {
        int p[3], axis;
        decode_edge(D, e, p, &axis);
        const int i0 = D.field_index(p[0], p[1], p[2]);
        const int i1 = D.field_index(p[0] + kAxisOffset[axis][0], p[1] + kAxisOffset[axis][1],
                                     p[2] + kAxisOffset[axis][2]);
        const int m0 = i0 < F ? ch.materials[i0] : MATERIAL_AIR;
        const int m1 = i1 < F ? ch.materials[i1] : MATERIAL_AIR;
        const bool sign_change = (m0 == MATERIAL_AIR && m1 != MATERIAL_AIR) || (m1 == MATERIAL_AIR && m0 != MATERIAL_AIR);
        if (sign_change && e != -1) created.push_back(e);
    }

    // PruneFieldEdges + CompactFieldEdges.  When every field edge is pruned
    // the reference keeps the unpruned list (compute_csg.cpp:156); the
    // restatement replaces it by the empty list.
    if (!invalidated.empty() && !ch.edge_keys.empty()) {
        std::unordered_set<int32_t> inv(invalidated.begin(), invalidated.end());
        std::vector<int32_t> keys;
        std::vector<F4> info;
        for (size_t i = 0; i < ch.edge_keys.size(); i++) {
            if (inv.count(ch.edge_keys[i])) continue;
            keys.push_back(ch.edge_keys[i]);
            info.push_back(ch.edge_info[i]);
        }
        ch.edge_keys.swap(keys);
        ch.edge_info.swap(info);
    }

    // CSG FindEdgeIntersectionInfo for the created edges, appended
    for (int32_t e : created) {
        ch.edge_keys.push_back(e);
        ch.edge_info.push_back(edge_info_brush(D, e, off, scale, ops));
    }
    ch.created_keys.insert(ch.created_keys.end(), created.begin(), created.end());
}

int run_chunk(Chunk& ch, const orc_density& dn, const orc_chunk_args& a, const PermLut& L) {
    const Dims D(a.voxels_per_chunk);
    ch = Chunk();
    const int scale = a.size / (D.vpc * LEAF_SIZE_SCALE);
    if (scale <= 0) return -1;
    ch.vpc = D.vpc;
    ch.scale = scale;
    ch.size = a.size;
    for (int i = 0; i < 3; i++) ch.min[i] = a.min[i];
    const int off[3] = {a.min[0] / LEAF_SIZE_SCALE, a.min[1] / LEAF_SIZE_SCALE, a.min[2] / LEAF_SIZE_SCALE};

    // GenerateDefaultField (density_field.cl:11-37)
    const int F = D.field_size();
    ch.materials.assign(F, 0);
    for (int z = 0; z < D.fdim; z++)
        for (int y = 0; y < D.fdim; y++)
            for (int x = 0; x < D.fdim; x++) {
                const float d = density(dn, (float)(x * scale + off[0]), (float)(y * scale + off[1]),
                                        (float)(z * scale + off[2]), L);
                ch.materials[D.field_index(x, y, z)] = d < 0.f ? a.default_material : MATERIAL_AIR;
            }

    // FindFieldEdges + ExclusiveScan + CompactEdges (density_field.cl:41-92)
    for (int z = 0; z < D.hdim; z++)
        for (int y = 0; y < D.hdim; y++)
            for (int x = 0; x < D.hdim; x++) {
                const int c0 = ch.materials[D.field_index(x, y, z)];
                for (int i = 0; i < 3; i++) {
                    const int ce = ch.materials[D.field_index(x + kAxisOffset[i][0], y + kAxisOffset[i][1],
                                                              z + kAxisOffset[i][2])];
                    const bool sc = (c0 != MATERIAL_AIR && ce == MATERIAL_AIR) || (c0 == MATERIAL_AIR && ce != MATERIAL_AIR);
                    if (sc) ch.edge_keys.push_back(edge_key(D, x, y, z, i));
                }
            }
    ch.plain_edge_keys = ch.edge_keys;
    for (int32_t k : ch.edge_keys) ch.edge_info.push_back(edge_info_density(D, dn, L, k, off, scale, a.crossing_mode));

    // stored CSG operations replayed as one batch (compute_density_field.cpp:255-271)
    if (a.num_ops > 0) apply_csg(D, ch, make_brushes(a.ops, a.num_ops), off, scale);

    if (ch.edge_keys.empty()) return 0;

    // FindActiveVoxels + CompactVoxels (octree.cl:142-223)
    for (int z = 0; z < D.vpc; z++)
        for (int y = 0; y < D.vpc; y++)
            for (int x = 0; x < D.vpc; x++) {
                int cm[8];
                int corners = 0;
                for (int i = 0; i < 8; i++) {
                    cm[i] = ch.materials[D.field_index(x + kChildMinOffsets[i][0], y + kChildMinOffsets[i][1],
                                                       z + kChildMinOffsets[i][2])];
                    corners |= (cm[i] == MATERIAL_AIR ? 0 : 1) << i;
                }
                if (corners == 0 || corners == 255) continue;
                int edges = 0;
                for (int i = 0; i < 12; i++) {
                    const int s0 = (corners >> kEdgeMap[i][0]) & 1, s1 = (corners >> kEdgeMap[i][1]) & 1;
                    edges |= (s0 != s1 ? 1 : 0) << i;
                }
                ch.node_codes.push_back(code_for_position(x, y, z, D.depth));
                ch.node_edges.push_back(edges);
                ch.node_materials.push_back((dominant_material(cm) << 8) | corners);
            }
    const int V = (int)ch.node_codes.size();
    if (V == 0) return 0;

    std::mt19937 gen(a.hash_seed);

    // edge hash + CreateLeafNodes (octree.cl:236-312)
    Cuckoo edge_hash;
    cuckoo_build(&edge_hash, reinterpret_cast<const uint32_t*>(ch.edge_keys.data()), (int)ch.edge_keys.size(), gen,
                 nullptr);
    ch.qefs.resize(V);
    ch.normals.resize(V);
    ch.positions.resize(V);
    ch.positions64.assign(4 * (size_t)V, 0.0);
    for (int v = 0; v < V; v++) {
        int pos[3];
        position_for_code(ch.node_codes[v], D.depth, pos);
        const int edge_list = ch.node_edges[v];
        F4 ep[12], en[12];
        QEF64 q64;
        int count = 0;
        for (int i = 0; i < 12; i++) {
            if (!((edge_list >> i) & 1)) continue;
            const int e0 = kEdgeMap[i][0], e1 = kEdgeMap[i][1];
            const F4 p0{(float)pos[0] + (float)kChildMinOffsets[e0][0], (float)pos[1] + (float)kChildMinOffsets[e0][1],
                        (float)pos[2] + (float)kChildMinOffsets[e0][2], 0.f};
            const F4 p1{(float)pos[0] + (float)kChildMinOffsets[e1][0], (float)pos[1] + (float)kChildMinOffsets[e1][1],
                        (float)pos[2] + (float)kChildMinOffsets[e1][2], 0.f};
            const int axis = i / 4;
            const int key = edge_key(D, pos[0] + kChildMinOffsets[e0][0], pos[1] + kChildMinOffsets[e0][1],
                                     pos[2] + kChildMinOffsets[e0][2], axis);
            const uint32_t di = edge_hash.find((uint32_t)key);
            if (di == ~0u) continue;
            const F4 e = ch.edge_info[di];
            const float fs = (float)scale;
            ep[count] = F4{fs * std::fmaf(p1.x - p0.x, e.w, p0.x), fs * std::fmaf(p1.y - p0.y, e.w, p0.y),
                           fs * std::fmaf(p1.z - p0.z, e.w, p0.z), fs * std::fmaf(p1.w - p0.w, e.w, p0.w)};
            en[count] = F4{e.x, e.y, e.z, 0.f};
            {
                const double t = e.w, sd = scale;
                const double pd[3] = {sd * (p0.x + (p1.x - p0.x) * t), sd * (p0.y + (p1.y - p0.y) * t),
                                      sd * (p0.z + (p1.z - p0.z) * t)};
                const double nd[3] = {e.x, e.y, e.z};
                qef64_add_point(q64, nd, pd);
            }
            count++;
        }
        // qef_create_from_points (qef.cl:283-303)
        QEF q;
        std::memset(&q, 0, sizeof(q));
        for (int i = 0; i < count; i++) qef_add_point(q, en[i], ep[i]);
        q.masspoint.x /= q.masspoint.w;
        q.masspoint.y /= q.masspoint.w;
        q.masspoint.z /= q.masspoint.w;
        q.masspoint.w /= q.masspoint.w;
        ch.qefs[v] = q;
        F4 n{0.f, 0.f, 0.f, 0.f};
        for (int i = 0; i < count; i++) {
            n.x += en[i].x;
            n.y += en[i].y;
            n.z += en[i].z;
            n.w += 1.f;
        }
        n.x /= n.w;
        n.y /= n.w;
        n.z /= n.w;
        n.w = 0.f;
        ch.normals[v] = n;
        // SolveQEFs (octree.cl:316-331)
        F4 x = qef_solve(q);
        x.x = std::fmaf(x.x, (float)LEAF_SIZE_SCALE, (float)a.min[0]);
        x.y = std::fmaf(x.y, (float)LEAF_SIZE_SCALE, (float)a.min[1]);
        x.z = std::fmaf(x.z, (float)LEAF_SIZE_SCALE, (float)a.min[2]);
        x.w = 1.f;
        ch.positions[v] = x;
        double x64[3];
        qef64_solve(q64, x64);
        for (int i = 0; i < 3; i++) ch.positions64[4 * (size_t)v + i] = x64[i] * LEAF_SIZE_SCALE + a.min[i];
        ch.positions64[4 * (size_t)v + 3] = count;
    }

    // node hash (compute_octree.cpp:143-144) + GenerateMesh (octree.cl:385-442)
    Cuckoo node_hash;
    cuckoo_build(&node_hash, ch.node_codes.data(), V, gen, nullptr);
    for (int v = 0; v < V; v++) {
        int pos[3];
        position_for_code(ch.node_codes[v], D.depth, pos);
        for (int axis = 0; axis < 3; axis++) {
            const int aa = pos[(axis + 1) % 3], bb = pos[(axis + 2) % 3];
            if (aa == D.vpc - 1 || bb == D.vpc - 1) continue;
            int idx[4];
            idx[0] = v;
            bool all = true;
            for (int n = 1; n < 4; n++) {
                const uint32_t c = code_for_position(pos[0] + kEdgeNodeOffsets[axis][n][0],
                                                     pos[1] + kEdgeNodeOffsets[axis][n][1],
                                                     pos[2] + kEdgeNodeOffsets[axis][n][2], D.depth);
                const uint32_t f = node_hash.find(c);
                idx[n] = (int)f;
                if (f == ~0u) all = false;
            }
            if (!all) continue;
            // ProcessEdge (octree.cl:335-372)
            const int edge = axis * 4 + 3;
            const int corners = ch.node_materials[v] & 0xff;
            const int m1 = (corners >> kEdgeMap[edge][0]) & 1, m2 = (corners >> kEdgeMap[edge][1]) & 1;
            if (m1 == m2) continue;
            static const int kWinding[2][6] = {{0, 1, 3, 0, 3, 2}, {0, 3, 1, 0, 2, 3}};
            const int flip = m1 != 0 ? 1 : 0;
            for (int k = 0; k < 6; k++) ch.triangles.push_back(idx[kWinding[flip][k]]);
        }
    }

    // GenerateMeshVertexBuffer (octree.cl:475-487); the vertex count is
    // exported only when triangles exist (compute_octree.cpp:227-232, 331-337)
    float col[3];
    colour_for_min_leaf_size(a.size / 256, col);  // CLIPMAP_LEAF_SIZE (volume_constants.h:15)
    const int T = (int)ch.triangles.size() / 3;
    ch.mesh_vertex_count = T > 0 ? V : 0;
    ch.vertices.resize((size_t)V * 12);
    for (int v = 0; v < V; v++) {
        float* o = &ch.vertices[(size_t)v * 12];
        o[0] = ch.positions[v].x; o[1] = ch.positions[v].y; o[2] = ch.positions[v].z; o[3] = ch.positions[v].w;
        o[4] = ch.normals[v].x; o[5] = ch.normals[v].y; o[6] = ch.normals[v].z; o[7] = ch.normals[v].w;
        o[8] = col[0]; o[9] = col[1]; o[10] = col[2]; o[11] = (float)(ch.node_materials[v] >> 8);
    }

    // FindSeamNodes + ExtractSeamNodeInfo (octree.cl:506-551)
    for (int v = 0; v < V; v++) {
        int pos[3];
        position_for_code(ch.node_codes[v], D.depth, pos);
        bool seam = false;
        for (int i = 0; i < 3; i++) seam = seam || pos[i] == 0 || pos[i] == D.vpc - 1;
        if (!seam) continue;
        int32_t rec[12];
        rec[0] = pos[0]; rec[1] = pos[1]; rec[2] = pos[2]; rec[3] = ch.node_materials[v];
        std::memcpy(&rec[4], &ch.positions[v], 16);
        std::memcpy(&rec[8], &ch.normals[v], 16);
        ch.seams.insert(ch.seams.end(), rec, rec + 12);
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Bottom-up octree simplification (not in the reference).  Classic dual
// contouring collapse (Ju et al. 2002, section 4) over the chunk's leaf
// octree, with the reference's QEF solver (qef_solve, qef.cl:239-256):
//
//   * every node keeps its QEF in its own frame: origin at the node's min
//     corner, unit = one voxel, so that the error is well conditioned at every
//     LOD.  Next to ATA and ATb (qef.cl:7-14) it carries btb = sum (n.p)^2, the
//     point count w, the mass-point sum and the normal sum;
//   * a leaf's QEF holds its edge crossings (the ones CreateLeafNodes uses,
//     octree.cl:236-312), in edge order, as qef_add_point does (qef.cl:170-191);
//   * a node at level k (2^k voxels) sums its children's QEFs in child order
//     (CHILD_MIN_OFFSETS, shared_constants.cl:11-22), each moved from the child's
//     frame by d = child origin - node origin: ATb += ATA d, btb += 2 d.ATb +
//     d.ATA d, mass point += w d;
//   * it is solved with qef_solve (the mass point is the running sum over w,
//     which qef_solve divides out); if the solution leaves the node's cube the
//     mass point is used; the error is the QEF's value there,
//     E(x) = x.ATA x - 2 x.ATb + btb;
//   * a node collapses when E <= threshold, every child that exists collapsed
//     (leaves count as collapsed) and no child is a seam voxel (a voxel on the
//     chunk's faces, FindSeamNodes octree.cl:506-520), so the seams that the
//     neighbouring chunks stitch against are unchanged.
//
// The mesh is classic DC contouring of the collapsed octree expressed over the
// leaf quads of GenerateMesh (octree.cl:385-442): each leaf voxel stands for
// its highest collapsed ancestor (its representative); a quad is kept only on
// the first sign change along its minimal edge (the edge of the smallest of its
// four representatives) when that edge's end points differ in sign, its two
// triangles are remapped to the representatives' vertices and triangles with a
// repeated vertex are dropped.  Vertices are the representatives, ordered by
// their first voxel in the leaf order.
// ---------------------------------------------------------------------------

struct SQef {
    float ata[6];
    float btb, w;
    float atb[3];
    float mp[3];
    float ns[3];
    float pad;
};

void sqef_zero(SQef& q) { std::memset(&q, 0, sizeof(q)); }

// a leaf's QEF in its voxel frame from its crossings (p in [0,1]^3, n)
void sqef_add_point(SQef& q, float px, float py, float pz, float nx, float ny, float nz) {
    q.ata[0] += nx * nx;
    q.ata[1] += nx * ny;
    q.ata[2] += nx * nz;
    q.ata[3] += ny * ny;
    q.ata[4] += ny * nz;
    q.ata[5] += nz * nz;
    const float b = dot3(px, py, pz, nx, ny, nz);
    q.atb[0] += nx * b;
    q.atb[1] += ny * b;
    q.atb[2] += nz * b;
    q.btb = std::fmaf(b, b, q.btb);
    q.mp[0] += px;
    q.mp[1] += py;
    q.mp[2] += pz;
    q.w += 1.f;
    q.ns[0] += nx;
    q.ns[1] += ny;
    q.ns[2] += nz;
}

// q += child moved by d (child origin - node origin, voxels)
void sqef_merge(SQef& q, const SQef& c, float dx, float dy, float dz) {
    const float* A = c.ata;
    const float adx = dot3(A[0], A[1], A[2], dx, dy, dz);
    const float ady = dot3(A[1], A[3], A[4], dx, dy, dz);
    const float adz = dot3(A[2], A[4], A[5], dx, dy, dz);
    for (int i = 0; i < 6; i++) q.ata[i] += A[i];
    q.atb[0] += c.atb[0] + adx;
    q.atb[1] += c.atb[1] + ady;
    q.atb[2] += c.atb[2] + adz;
    q.btb += c.btb + std::fmaf(2.f, dot3(dx, dy, dz, c.atb[0], c.atb[1], c.atb[2]), dot3(dx, dy, dz, adx, ady, adz));
    q.mp[0] += std::fmaf(c.w, dx, c.mp[0]);
    q.mp[1] += std::fmaf(c.w, dy, c.mp[1]);
    q.mp[2] += std::fmaf(c.w, dz, c.mp[2]);
    q.w += c.w;
    q.ns[0] += c.ns[0];
    q.ns[1] += c.ns[1];
    q.ns[2] += c.ns[2];
}

float sqef_error(const SQef& q, float x, float y, float z) {
    const float* A = q.ata;
    const float ax = dot3(A[0], A[1], A[2], x, y, z);
    const float ay = dot3(A[1], A[3], A[4], x, y, z);
    const float az = dot3(A[2], A[4], A[5], x, y, z);
    return std::fmaf(-2.f, dot3(x, y, z, q.atb[0], q.atb[1], q.atb[2]), dot3(x, y, z, ax, ay, az)) + q.btb;
}

// solve a node's QEF (node size s voxels): position in the node frame and error
float sqef_solve(const SQef& q, float s, float out[3]) {
    QEF r;
    std::memset(&r, 0, sizeof(r));
    for (int i = 0; i < 6; i++) r.ata[i] = q.ata[i];
    r.atb = F4{q.atb[0], q.atb[1], q.atb[2], 0.f};
    r.masspoint = F4{q.mp[0], q.mp[1], q.mp[2], q.w};
    F4 x = qef_solve(r);
    if (!(x.x >= 0.f && x.x <= s && x.y >= 0.f && x.y <= s && x.z >= 0.f && x.z <= s)) {
        x.x = q.mp[0] / q.w;
        x.y = q.mp[1] / q.w;
        x.z = q.mp[2] / q.w;
    }
    out[0] = x.x;
    out[1] = x.y;
    out[2] = x.z;
    return sqef_error(q, x.x, x.y, x.z);
}

struct SNode {
    int collapsed = 0;
    int anchor = 0;
    int material = 0;
    float pos[3] = {0.f, 0.f, 0.f};  // world
    SQef q;
};

int simplify_chunk(Chunk& ch, float threshold) {
    ch.simp_vertices.clear();
    ch.simp_triangles.clear();
    ch.simp_reps.clear();
    ch.simp_vertex_count = 0;
    const int V = (int)ch.node_codes.size();
    if (ch.vpc == 0 || V == 0) return 0;
    const Dims D(ch.vpc);
    const int L = D.depth;
    const float fs = (float)ch.scale;

    // leaf QEFs from the same crossings the leaves were solved with
    std::unordered_map<int32_t, int> edge_index;
    for (size_t i = 0; i < ch.edge_keys.size(); i++) edge_index.emplace(ch.edge_keys[i], (int)i);
    std::vector<SQef> leaf(V);
    std::vector<std::array<int, 3>> vpos(V);
    std::unordered_map<int, int> voxel_at;  // packed position -> voxel
    auto pack = [](int x, int y, int z) { return x | (y << 8) | (z << 16); };
    for (int v = 0; v < V; v++) {
        int pos[3];
        position_for_code(ch.node_codes[v], D.depth, pos);
        vpos[v] = {pos[0], pos[1], pos[2]};
        voxel_at[pack(pos[0], pos[1], pos[2])] = v;
        sqef_zero(leaf[v]);
        for (int i = 0; i < 12; i++) {
            if (!((ch.node_edges[v] >> i) & 1)) continue;
            const int e0 = kEdgeMap[i][0], e1 = kEdgeMap[i][1];
            const int key = edge_key(D, pos[0] + kChildMinOffsets[e0][0], pos[1] + kChildMinOffsets[e0][1],
                                     pos[2] + kChildMinOffsets[e0][2], i / 4);
            auto it = edge_index.find(key);
            if (it == edge_index.end()) continue;
            const F4 e = ch.edge_info[it->second];
            float p[3];
            for (int a = 0; a < 3; a++) {
                const float o0 = (float)kChildMinOffsets[e0][a], o1 = (float)kChildMinOffsets[e1][a];
                p[a] = std::fmaf(o1 - o0, e.w, o0);
            }
            sqef_add_point(leaf[v], p[0], p[1], p[2], e.x, e.y, e.z);
        }
    }
    auto is_seam = [&](int v) {
        for (int a = 0; a < 3; a++)
            if (vpos[v][a] == 0 || vpos[v][a] == D.vpc - 1) return true;
        return false;
    };

    // levels 1..L
    std::vector<std::map<int, SNode>> lv(L + 1);
    for (int k = 1; k <= L; k++) {
        std::map<int, SNode>& cur = lv[k];
        for (int v = 0; v < V; v++) cur[pack(vpos[v][0] >> k, vpos[v][1] >> k, vpos[v][2] >> k)];
        const int h = 1 << (k - 1);
        for (auto& kv : cur) {
            const int px = kv.first & 255, py = (kv.first >> 8) & 255, pz = kv.first >> 16;
            SNode& n = kv.second;
            bool blocked = false;
            SQef q;
            sqef_zero(q);
            int mats[8];
            int anchor = INT32_MAX;
            for (int i = 0; i < 8; i++) {
                const int cx = 2 * px + kChildMinOffsets[i][0], cy = 2 * py + kChildMinOffsets[i][1],
                          cz = 2 * pz + kChildMinOffsets[i][2];
                mats[i] = MATERIAL_NONE;
                const SQef* cq = nullptr;
                if (k == 1) {
                    auto it = voxel_at.find(pack(cx, cy, cz));
                    if (it == voxel_at.end()) continue;
                    if (is_seam(it->second)) { blocked = true; continue; }
                    cq = &leaf[it->second];
                    mats[i] = ch.node_materials[it->second] >> 8;
                    anchor = std::min(anchor, it->second);
                } else {
                    auto it = lv[k - 1].find(pack(cx, cy, cz));
                    if (it == lv[k - 1].end()) continue;
                    if (!it->second.collapsed) { blocked = true; continue; }
                    cq = &it->second.q;
                    mats[i] = it->second.material;
                    anchor = std::min(anchor, it->second.anchor);
                }
                sqef_merge(q, *cq, (float)(kChildMinOffsets[i][0] * h), (float)(kChildMinOffsets[i][1] * h),
                           (float)(kChildMinOffsets[i][2] * h));
            }
            if (blocked) continue;
            float x[3];
            const float err = sqef_solve(q, (float)(2 * h), x);
            if (!(err <= threshold)) continue;
            n.collapsed = 1;
            n.anchor = anchor;
            n.material = dominant_material(mats);
            n.q = q;
            const int org[3] = {px << k, py << k, pz << k};
            for (int a = 0; a < 3; a++)
                n.pos[a] = std::fmaf(fs * ((float)org[a] + x[a]), (float)LEAF_SIZE_SCALE, (float)ch.min[a]);
        }
    }

    // representatives: the highest collapsed ancestor
    std::vector<int> rep_level(V, 0), rep_anchor(V);
    std::vector<const SNode*> rep_node(V, nullptr);
    ch.simp_reps.resize(V);
    for (int v = 0; v < V; v++) {
        rep_anchor[v] = v;
        for (int k = 1; k <= L; k++) {
            const SNode& n = lv[k].at(pack(vpos[v][0] >> k, vpos[v][1] >> k, vpos[v][2] >> k));
            if (!n.collapsed) break;
            rep_level[v] = k;
            rep_anchor[v] = n.anchor;
            rep_node[v] = &n;
        }
        ch.simp_reps[v] = rep_anchor[v] | (rep_level[v] << 20);
    }

    // triangles over the leaf quads (GenerateMesh, octree.cl:385-442)
    std::vector<int> tri_local;  // anchors, remapped below
    auto solid = [&](int x, int y, int z) { return ch.materials[D.field_index(x, y, z)] != MATERIAL_AIR; };
    for (int v = 0; v < V; v++) {
        const int* pos = vpos[v].data();
        for (int axis = 0; axis < 3; axis++) {
            const int aa = pos[(axis + 1) % 3], bb = pos[(axis + 2) % 3];
            if (aa == D.vpc - 1 || bb == D.vpc - 1) continue;
            int idx[4];
            idx[0] = v;
            bool all = true;
            for (int n = 1; n < 4; n++) {
                auto it = voxel_at.find(pack(pos[0] + kEdgeNodeOffsets[axis][n][0], pos[1] + kEdgeNodeOffsets[axis][n][1],
                                             pos[2] + kEdgeNodeOffsets[axis][n][2]));
                if (it == voxel_at.end()) { all = false; break; }
                idx[n] = it->second;
            }
            if (!all) continue;
            const int edge = axis * 4 + 3;
            const int corners = ch.node_materials[v] & 0xff;
            const int m1 = (corners >> kEdgeMap[edge][0]) & 1, m2 = (corners >> kEdgeMap[edge][1]) & 1;
            if (m1 == m2) continue;
            int minlev = L + 1;
            for (int n = 0; n < 4; n++) minlev = std::min(minlev, rep_level[idx[n]]);
            if (minlev > 0) {
                // the minimal edge: along `axis` through the edge's other two coordinates
                const int len = 1 << minlev;
                int p0[3] = {pos[0], pos[1], pos[2]};
                p0[(axis + 1) % 3] += 1;
                p0[(axis + 2) % 3] += 1;
                const int s0 = pos[axis] & ~(len - 1);
                auto sign_at = [&](int t) {
                    int q[3] = {p0[0], p0[1], p0[2]};
                    q[axis] = t;
                    return solid(q[0], q[1], q[2]);
                };
                const bool first = sign_at(s0);
                bool keep = first != sign_at(s0 + len);
                for (int t = s0 + 1; keep && t <= pos[axis]; t++) keep = sign_at(t) == first;
                if (!keep) continue;
            }
            static const int kWinding[2][6] = {{0, 1, 3, 0, 3, 2}, {0, 3, 1, 0, 2, 3}};
            const int flip = m1 != 0 ? 1 : 0;
            for (int t = 0; t < 2; t++) {
                const int a0 = rep_anchor[idx[kWinding[flip][3 * t]]];
                const int a1 = rep_anchor[idx[kWinding[flip][3 * t + 1]]];
                const int a2 = rep_anchor[idx[kWinding[flip][3 * t + 2]]];
                if (a0 == a1 || a1 == a2 || a0 == a2) continue;
                tri_local.push_back(a0);
                tri_local.push_back(a1);
                tri_local.push_back(a2);
            }
        }
    }

    // vertices: one per representative, in the order of their anchors
    std::vector<int> new_index(V, -1);
    float col[3];
    colour_for_min_leaf_size(ch.size / 256, col);
    int nv = 0;
    for (int v = 0; v < V; v++) {
        if (rep_anchor[v] != v) continue;
        new_index[v] = nv++;
        float o[12];
        if (rep_level[v] == 0) {
            std::memcpy(o, &ch.vertices[(size_t)v * 12], sizeof(o));
        } else {
            const SNode& n = *rep_node[v];
            o[0] = n.pos[0]; o[1] = n.pos[1]; o[2] = n.pos[2]; o[3] = 1.f;
            o[4] = n.q.ns[0] / n.q.w; o[5] = n.q.ns[1] / n.q.w; o[6] = n.q.ns[2] / n.q.w; o[7] = 0.f;
            o[8] = col[0]; o[9] = col[1]; o[10] = col[2]; o[11] = (float)n.material;
        }
        ch.simp_vertices.insert(ch.simp_vertices.end(), o, o + 12);
    }
    for (int a : tri_local) ch.simp_triangles.push_back(new_index[a]);
    ch.simp_vertex_count = ch.simp_triangles.empty() ? 0 : nv;
    return 0;
}

template <typename T>
int copy_out(const std::vector<T>& v, void* out, int64_t cap) {
    const int64_t bytes = (int64_t)(v.size() * sizeof(T));
    if (out == nullptr || cap < bytes) return -2;
    if (bytes) std::memcpy(out, v.data(), (size_t)bytes);
    return (int)v.size();
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

int orc_set_seed(int32_t seed) {
    build_lut(seed, &g_lut);
    g_lut_ready = true;
    return 0;
}

void orc_perm_lut(uint8_t* out) { std::memcpy(out, g_lut.v, sizeof(g_lut.v)); }

void orc_perm_image_rgba(uint8_t* out) {
    // the pixels CreateNoisePermutationLookupImage uploads (compute_density_field.cpp:104-114)
    for (int t = 0; t < 65536; t++) {
        const int v = g_lut.v[t];
        for (int c = 0; c < 3; c++) out[4 * t + c] = (uint8_t)(kGrad3[v & 0x0f][c] * 64 + 64);
        out[4 * t + 3] = (uint8_t)v;
    }
}

float orc_density_at(const orc_density* d, float x, float y, float z) { return density(*d, x, y, z, g_lut); }
float orc_snoise2(float x, float y) { return snoise2(x, y, g_lut); }
float orc_snoise3(float x, float y, float z) { return snoise3(x, y, z, g_lut); }

int orc_flop_counts(const orc_density* d, int64_t* out) {
    if (!d || !out) return -1;
    Counted::ops = 0;
    if (d->mode != 0) (void)height_t<Counted>(*d, 37.25f, -81.5f, g_lut);
    out[0] = (int64_t)Counted::ops;
    Counted::ops = 0;
    (void)density_t<Counted>(*d, 37.25f, 12.75f, -81.5f, g_lut);
    out[1] = (int64_t)Counted::ops - out[0];
    const Dims D(64);
    const int off[3] = {0, 0, 0};
    for (int axis = 0; axis < 3; axis++) {
        Counted o[4];
        Counted::ops = 0;
        edge_info_density_t<Counted>(D, *d, g_lut, edge_key(D, 5, 6, 7, axis), off, 1, 0, o);
        out[2 + axis] = (int64_t)Counted::ops;
    }
    return 0;
}
int orc_find_next_prime(int32_t n) { return find_next_prime(n); }

float orc_qef_solve_points(const float* positions, const float* normals, int32_t count, float* out) {
    // qef_create_from_points (qef.cl:283-303), then qef_solve (qef.cl:239-256)
    QEF q;
    std::memset(&q, 0, sizeof(q));
    for (int i = 0; i < count && i < 12; i++)
        qef_add_point(q, F4{normals[4 * i], normals[4 * i + 1], normals[4 * i + 2], normals[4 * i + 3]},
                      F4{positions[4 * i], positions[4 * i + 1], positions[4 * i + 2], positions[4 * i + 3]});
    q.masspoint.x /= q.masspoint.w;
    q.masspoint.y /= q.masspoint.w;
    q.masspoint.z /= q.masspoint.w;
    q.masspoint.w /= q.masspoint.w;
    const F4 x = qef_solve(q);
    out[0] = x.x;
    out[1] = x.y;
    out[2] = x.z;
    out[3] = x.w;
    return 0.f;
}

void* orc_chunk_new(void) { return new Chunk(); }
void orc_chunk_free(void* h) { delete static_cast<Chunk*>(h); }

int orc_chunk_run(void* h, const orc_density* d, const orc_chunk_args* a) {
    if (!g_lut_ready) return -3;
    const int v = a->voxels_per_chunk;
    if (v < 8 || v > 64 || (v & (v - 1))) return -1;
    return run_chunk(*static_cast<Chunk*>(h), *d, *a, g_lut);
}

int orc_chunk_simplify(void* h, float threshold) {
    Chunk& c = *static_cast<Chunk*>(h);
    if (threshold < 0.f) return -1;
    return simplify_chunk(c, threshold);
}

int orc_chunk_count(void* hp, int what) {
    const Chunk& c = *static_cast<Chunk*>(hp);
    switch (what) {
        case ORC_MATERIALS: return (int)c.materials.size();
        case ORC_EDGE_KEYS: case ORC_EDGE_INFO: return (int)c.edge_keys.size();
        case ORC_NODE_CODES: case ORC_NODE_EDGES: case ORC_NODE_MATERIALS: case ORC_VERTICES: case ORC_QEFS:
            return (int)c.node_codes.size();
        case ORC_TRIANGLES: return (int)c.triangles.size() / 3;
        case ORC_SEAMS: return (int)c.seams.size() / 12;
        case ORC_PLAIN_EDGE_KEYS: return (int)c.plain_edge_keys.size();
        case ORC_MESH_VERTEX_COUNT: return c.mesh_vertex_count;
        case ORC_CREATED_EDGE_KEYS: return (int)c.created_keys.size();
        case ORC_SIMP_VERTICES: return (int)c.simp_vertices.size() / 12;
        case ORC_SIMP_TRIANGLES: return (int)c.simp_triangles.size() / 3;
        case ORC_SIMP_VERTEX_COUNT: return c.simp_vertex_count;
        case ORC_SIMP_REPS: return (int)c.simp_reps.size();
        case ORC_POSITIONS_F64: return (int)c.positions64.size() / 4;
        default: return -1;
    }
}

int orc_chunk_get(void* hp, int what, void* out, int64_t cap) {
    const Chunk& c = *static_cast<Chunk*>(hp);
    switch (what) {
        case ORC_MATERIALS: return copy_out(c.materials, out, cap);
        case ORC_EDGE_KEYS: return copy_out(c.edge_keys, out, cap);
        case ORC_EDGE_INFO: return copy_out(c.edge_info, out, cap);
        case ORC_NODE_CODES: return copy_out(c.node_codes, out, cap);
        case ORC_NODE_EDGES: return copy_out(c.node_edges, out, cap);
        case ORC_NODE_MATERIALS: return copy_out(c.node_materials, out, cap);
        case ORC_VERTICES: return copy_out(c.vertices, out, cap) < 0 ? -2 : (int)c.node_codes.size();
        case ORC_TRIANGLES: return copy_out(c.triangles, out, cap) < 0 ? -2 : (int)c.triangles.size() / 3;
        case ORC_SEAMS: return copy_out(c.seams, out, cap) < 0 ? -2 : (int)c.seams.size() / 12;
        case ORC_PLAIN_EDGE_KEYS: return copy_out(c.plain_edge_keys, out, cap);
        case ORC_QEFS: return copy_out(c.qefs, out, cap);
        case ORC_CREATED_EDGE_KEYS: return copy_out(c.created_keys, out, cap);
        case ORC_SIMP_VERTICES: return copy_out(c.simp_vertices, out, cap) < 0 ? -2 : (int)c.simp_vertices.size() / 12;
        case ORC_SIMP_TRIANGLES: return copy_out(c.simp_triangles, out, cap) < 0 ? -2 : (int)c.simp_triangles.size() / 3;
        case ORC_SIMP_REPS: return copy_out(c.simp_reps, out, cap);
        case ORC_POSITIONS_F64: return copy_out(c.positions64, out, cap) < 0 ? -2 : (int)c.positions64.size() / 4;
        default: return -1;
    }
}

struct orc_cuckoo {
    Cuckoo c;
};

orc_cuckoo* orc_cuckoo_build(const uint32_t* keys, int32_t n, uint32_t seed, int32_t* retries) {
    auto* h = new orc_cuckoo();
    std::mt19937 gen(seed);
    int r = 0;
    cuckoo_build(&h->c, keys, n, gen, &r);
    if (retries) *retries = r;
    return h;
}

int orc_cuckoo_find(const orc_cuckoo* c, uint32_t key, uint32_t* value) {
    const uint32_t v = c->c.find(key);
    if (value) *value = v;
    return v != ~0u ? 1 : 0;
}

int orc_cuckoo_prime(const orc_cuckoo* c) { return (int)c->c.prime; }
void orc_cuckoo_free(orc_cuckoo* c) { delete c; }

int orc_remove_duplicates(const int32_t* in, int32_t n, int32_t* out) {
    std::vector<int32_t> v(in, in + n);
    const std::vector<int32_t> r = remove_duplicates(v);
    std::memcpy(out, r.data(), r.size() * sizeof(int32_t));
    return (int)r.size();
}

void orc_csg_op_bounds(const orc_csg_op* op, int32_t out_min[3], int32_t out_max[3]) {
    // CalcCSGOperationBounds (clipmap.cpp:1638-1643): CSG_OFFSET = 0.5,
    // CSG_BOUNDS_FUDGE = 2; ivec3(float) truncates toward zero
    for (int i = 0; i < 3; i++) {
        const int half = (int)(op->dimensions[i] * (float)LEAF_SIZE_SCALE) + 2;
        const int origin = (int)((op->origin[i] - 0.5f) * (float)LEAF_SIZE_SCALE);
        out_min[i] = origin - half;
        out_max[i] = origin + half;
    }
}

int orc_aabb_overlaps(const int32_t amin[3], const int32_t amax[3], const int32_t bmin[3], const int32_t bmax[3]) {
    return !(amax[0] < bmin[0] || amax[1] < bmin[1] || amax[2] < bmin[2] || amin[0] > bmax[0] ||
             amin[1] > bmax[1] || amin[2] > bmax[2]);
}

// ---- clipmap chunk lists ------------------------------------------------------

}  // extern "C"

namespace clipmap {
constexpr int kLeaf = 256;                  // CLIPMAP_LEAF_SIZE (volume_constants.h:15)
constexpr int kLodMax = kLeaf * (1 << 5);   // LOD_MAX_NODE_SIZE (clipmap.cpp:31)
const float kActive[6] = {0.f, kLeaf * 1.5f, kLeaf * 3.5f, kLeaf * 5.5f, kLeaf * 7.5f, kLeaf * 13.5f};  // clipmap.cpp:33-41

struct Out {
    int32_t* out4;
    int32_t cap;
    int32_t n = 0;
    void push(const int32_t mn[3], int32_t size) {
        if (n < cap) {
            out4[4 * n] = mn[0];
            out4[4 * n + 1] = mn[1];
            out4[4 * n + 2] = mn[2];
            out4[4 * n + 3] = size;
        }
        n++;
    }
};

// DistanceToNode (clipmap.cpp:1056-1064), float arithmetic
float distance_to_node(const int32_t mn[3], int32_t size, const float cam[3]) {
    float d[3];
    for (int a = 0; a < 3; a++) {
        const float lo = (float)mn[a], hi = (float)(mn[a] + size);
        d[a] = std::max(std::max(lo - cam[a], 0.f), cam[a] - hi);
    }
    return std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

void child_min(const int32_t mn[3], int32_t half, int i, int32_t c[3]) {
    // CHILD_MIN_OFFSETS order: x << 2 | y << 1 | z
    c[0] = mn[0] + ((i >> 2) & 1) * half;
    c[1] = mn[1] + ((i >> 1) & 1) * half;
    c[2] = mn[2] + (i & 1) * half;
}

// SelectActiveClipmapNodes (clipmap.cpp:1084-1128)
void select(const int32_t mn[3], int32_t size, bool parent_active, const float cam[3], Out& o) {
    bool active = false;
    if (!parent_active && size <= kLodMax) {
        int lod = 0;
        while ((kLeaf << lod) < size) lod++;  // log2(size / CLIPMAP_LEAF_SIZE)
        if (distance_to_node(mn, size, cam) >= kActive[lod]) {
            o.push(mn, size);
            active = true;
        }
    }
    if (size == kLeaf || parent_active || active) return;  // nothing below is selected
    const int32_t half = size / 2;
    for (int i = 0; i < 8; i++) {
        int32_t c[3];
        child_min(mn, half, i, c);
        select(c, half, false, cam, o);
    }
}

bool overlaps(const int32_t mn[3], int32_t size, const int32_t bmin[3], const int32_t bmax[3]) {
    const int32_t nmax[3] = {mn[0] + size, mn[1] + size, mn[2] + size};
    return orc_aabb_overlaps(bmin, bmax, mn, nmax) != 0;
}

// FindNodesInsideAABB (clipmap.cpp:1571-1597) generalised to a set of boxes:
// a node is visited when it overlaps any of them.  With one box this is the
// reference's recursion; with several, a node overlapping box j has every
// ancestor overlapping box j, so the union of the per-box walks is exactly
// the nodes this walk lists.
void inside(const int32_t mn[3], int32_t size, const std::vector<int32_t>& boxes, Out& o) {
    bool any = false;
    for (size_t b = 0; b < boxes.size(); b += 6)
        if (overlaps(mn, size, &boxes[b], &boxes[b + 3])) {
            any = true;
            break;
        }
    if (!any) return;
    if (size > kLeaf) {
        const int32_t half = size / 2;
        for (int i = 0; i < 8; i++) {
            int32_t c[3];
            child_min(mn, half, i, c);
            inside(c, half, boxes, o);
        }
    }
    if (size <= kLodMax) o.push(mn, size);
}

bool valid_root(int32_t root_size) { return root_size >= kLeaf && (root_size & (root_size - 1)) == 0; }
}  // namespace clipmap

// ---- seam octree and contouring -------------------------------------------------
//
// GenerateClipmapSeamMesh (clipmap.cpp:573-610) restated as the reference runs
// it: the active nodes around a host (FindNode / FindActiveNodes, clipmap.cpp:
// 982-1013, 1449-1479) give their seam nodes (GenerateMeshDataForNode,
// clipmap.cpp:398-418) to SelectSeamNodes / FilterSeamNode (clipmap.cpp:
// 508-570); Octree_ConstructUpwards (octree.cpp:31-148) builds a pointer
// octree from them and Octree_GenerateMesh (octree.cpp:197-551) numbers its
// leaves and contours it.

namespace seam {

constexpr int kLeafChunk = 256;  // CLIPMAP_LEAF_SIZE (volume_constants.h:15)

// the dual-contouring tables of contour_constants.h (the standard tables of
// the method; the recursion's order depends on them)
const int kEdgeVMap[12][2] = {{0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 2}, {1, 3},
                              {4, 6}, {5, 7}, {0, 1}, {2, 3}, {4, 5}, {6, 7}};
const int kCellProcFaceMask[12][3] = {{0, 4, 0}, {1, 5, 0}, {2, 6, 0}, {3, 7, 0}, {0, 2, 1}, {4, 6, 1},
                                      {1, 3, 1}, {5, 7, 1}, {0, 1, 2}, {2, 3, 2}, {4, 5, 2}, {6, 7, 2}};
const int kCellProcEdgeMask[6][5] = {{0, 1, 2, 3, 0}, {4, 5, 6, 7, 0}, {0, 4, 1, 5, 1},
                                     {2, 6, 3, 7, 1}, {0, 2, 4, 6, 2}, {1, 3, 5, 7, 2}};
const int kFaceProcFaceMask[3][4][3] = {{{4, 0, 0}, {5, 1, 0}, {6, 2, 0}, {7, 3, 0}},
                                        {{2, 0, 1}, {6, 4, 1}, {3, 1, 1}, {7, 5, 1}},
                                        {{1, 0, 2}, {3, 2, 2}, {5, 4, 2}, {7, 6, 2}}};
const int kFaceProcEdgeMask[3][4][6] = {{{1, 4, 0, 5, 1, 1}, {1, 6, 2, 7, 3, 1}, {0, 4, 6, 0, 2, 2}, {0, 5, 7, 1, 3, 2}},
                                        {{0, 2, 3, 0, 1, 0}, {0, 6, 7, 4, 5, 0}, {1, 2, 0, 6, 4, 2}, {1, 3, 1, 7, 5, 2}},
                                        {{1, 1, 0, 3, 2, 0}, {1, 5, 4, 7, 6, 0}, {0, 1, 5, 0, 4, 1}, {0, 3, 7, 2, 6, 1}}};
const int kEdgeProcEdgeMask[3][2][5] = {{{3, 2, 1, 0, 0}, {7, 6, 5, 4, 0}},
                                        {{5, 1, 4, 0, 1}, {7, 3, 6, 2, 1}},
                                        {{6, 4, 2, 0, 2}, {7, 5, 3, 1, 2}}};
const int kProcessEdgeMask[3][4] = {{3, 2, 1, 0}, {7, 5, 6, 4}, {11, 10, 9, 8}};

inline void child_offset(int i, int o[3]) {  // CHILD_MIN_OFFSETS (x << 2 | y << 1 | z)
    o[0] = (i >> 2) & 1;
    o[1] = (i >> 1) & 1;
    o[2] = i & 1;
}

struct Node {
    bool leaf = false;
    int32_t min[3] = {0, 0, 0};
    int32_t size = 0;
    Node* child[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    float position[3] = {0, 0, 0}, normal[3] = {0, 0, 0};
    int32_t material_info = 0;
    int32_t index = -1;
};

struct Mesh {
    std::vector<float> vertices;    // 12 floats each (MeshVertex)
    std::vector<int32_t> triangles;  // 3 each
};

bool same3(const int32_t a[3], const int32_t b[3]) { return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }

// ConstructParents (octree.cpp:31-86); `pool` owns the new nodes
std::vector<Node*> construct_parents(std::vector<Node*>& nodes, int parent_size, const int32_t root_min[3],
                                     std::vector<std::unique_ptr<Node>>& pool) {
    std::unordered_map<uint64_t, Node*> parents;
    std::vector<Node*> order;
    for (Node* n : nodes) {
        int32_t ppos[3];
        for (int a = 0; a < 3; a++) ppos[a] = n->min[a] - ((n->min[a] - root_min[a]) % parent_size);
        const uint64_t key = (uint64_t)(uint32_t)(ppos[0] - root_min[0]) |
                             ((uint64_t)(uint32_t)(ppos[1] - root_min[1]) << 20) |
                             ((uint64_t)(uint32_t)(ppos[2] - root_min[2]) << 40);  // HashOctreeMin (octree.cpp:24-27)
        Node* p;
        auto it = parents.find(key);
        if (it == parents.end()) {
            pool.emplace_back(new Node());
            p = pool.back().get();
            for (int a = 0; a < 3; a++) p->min[a] = ppos[a];
            p->size = parent_size;
            parents.emplace(key, p);
            order.push_back(p);
        } else {
            p = it->second;
        }
        for (int i = 0; i < 8; i++) {
            int o[3];
            child_offset(i, o);
            const int32_t cpos[3] = {ppos[0] + (parent_size / 2) * o[0], ppos[1] + (parent_size / 2) * o[1],
                                     ppos[2] + (parent_size / 2) * o[2]};
            if (same3(cpos, n->min)) {
                p->child[i] = n;
                break;
            }
        }
    }
    return order;
}

// Octree_ConstructUpwards (octree.cpp:90-148)
Node* construct_upwards(std::vector<Node*> nodes, const int32_t root_min[3], int root_size,
                        std::vector<std::unique_ptr<Node>>& pool) {
    if (nodes.empty()) return nullptr;
    std::stable_sort(nodes.begin(), nodes.end(), [](const Node* a, const Node* b) { return a->size < b->size; });
    while (nodes.front()->size != nodes.back()->size) {
        auto it = nodes.begin();
        const int size = (*it)->size;
        do {
            ++it;
        } while ((*it)->size == size);
        std::vector<Node*> run(nodes.begin(), it);
        std::vector<Node*> next = construct_parents(run, size * 2, root_min, pool);
        next.insert(next.end(), it, nodes.end());
        nodes.swap(next);
    }
    for (int parent = nodes.front()->size * 2; parent <= root_size; parent *= 2)
        nodes = construct_parents(nodes, parent, root_min, pool);
    return nodes.size() == 1 ? nodes.front() : nullptr;
}

// GenerateVertexIndices (octree.cpp:197-232)
void vertex_indices(Node* n, const float colour[3], Mesh& m) {
    if (!n) return;
    bool has_children = false;
    for (int i = 0; i < 8; i++) has_children |= n->child[i] != nullptr;
    if (has_children) {
        for (int i = 0; i < 8; i++) vertex_indices(n->child[i], colour, m);
        return;
    }
    n->index = (int32_t)(m.vertices.size() / 12);
    const float v[12] = {n->position[0], n->position[1], n->position[2], 0.f,
                         n->normal[0],   n->normal[1],   n->normal[2],   0.f,
                         colour[0],      colour[1],      colour[2],      (float)(n->material_info >> 8)};
    m.vertices.insert(m.vertices.end(), v, v + 12);
}

void chunk_min(const int32_t p[3], int32_t out[3]) {  // ChunkMinForPosition (volume.cpp:30-34)
    const unsigned mask = ~(unsigned)(kLeafChunk - 1);
    for (int a = 0; a < 3; a++) out[a] = (int32_t)((unsigned)p[a] & mask);
}

// ContourProcessEdge (octree.cpp:236-282)
void process_edge(Node* node[4], int dir, Mesh& m) {
    int min_size = INT_MAX, min_index = 0, indices[4] = {-1, -1, -1, -1};
    bool flip = false, sign_change[4] = {false, false, false, false};
    for (int i = 0; i < 4; i++) {
        if (node[i]->leaf) {
            const int edge = kProcessEdgeMask[dir][i];
            const int c0 = kEdgeVMap[edge][0], c1 = kEdgeVMap[edge][1];
            const int corners = node[i]->material_info & 0xff;
            const int m0 = (corners >> c0) & 1, m1 = (corners >> c1) & 1;
            if (node[i]->size < min_size) {
                min_size = node[i]->size;
                min_index = i;
                flip = m1 != 1;
            }
            indices[i] = node[i]->index;
            sign_change[i] = (m0 && !m1) || (!m0 && m1);
        }
    }
    if (!sign_change[min_index]) return;
    const int t[2][3] = {{indices[0], indices[1], indices[3]}, {indices[0], indices[3], indices[2]}};
    const int tf[2][3] = {{indices[0], indices[3], indices[1]}, {indices[0], indices[2], indices[3]}};
    for (int k = 0; k < 2; k++) m.triangles.insert(m.triangles.end(), flip ? tf[k] : t[k], (flip ? tf[k] : t[k]) + 3);
}

// ContourEdgeProc (octree.cpp:286-347)
void edge_proc(Node* node[4], int dir, Mesh& m) {
    if (!node[0] || !node[1] || !node[2] || !node[3]) return;
    int32_t c0[3];
    chunk_min(node[0]->min, c0);
    bool one_chunk = true;
    for (int i = 1; i < 4; i++) {
        int32_t ci[3];
        chunk_min(node[i]->min, ci);
        one_chunk &= same3(ci, c0);
    }
    if (one_chunk) return;  // only edges straddling chunks are contoured
    const bool branch[4] = {!node[0]->leaf, !node[1]->leaf, !node[2]->leaf, !node[3]->leaf};
    if (!branch[0] && !branch[1] && !branch[2] && !branch[3]) {
        process_edge(node, dir, m);
        return;
    }
    for (int i = 0; i < 2; i++) {
        Node* e[4];
        for (int j = 0; j < 4; j++) e[j] = branch[j] ? node[j]->child[kEdgeProcEdgeMask[dir][i][j]] : node[j];
        edge_proc(e, kEdgeProcEdgeMask[dir][i][4], m);
    }
}

// ContourFaceProc (octree.cpp:351-432)
void face_proc(Node* node[2], int dir, Mesh& m) {
    if (!node[0] || !node[1]) return;
    int32_t a[3], b[3];
    chunk_min(node[0]->min, a);
    chunk_min(node[1]->min, b);
    if (same3(a, b)) return;
    const bool branch[2] = {!node[0]->leaf, !node[1]->leaf};
    if (!branch[0] && !branch[1]) return;
    for (int i = 0; i < 4; i++) {
        Node* f[2];
        for (int j = 0; j < 2; j++) f[j] = branch[j] ? node[j]->child[kFaceProcFaceMask[dir][i][j]] : node[j];
        face_proc(f, kFaceProcFaceMask[dir][i][2], m);
    }
    const int orders[2][4] = {{0, 0, 1, 1}, {0, 1, 0, 1}};
    for (int i = 0; i < 4; i++) {
        const int* order = orders[kFaceProcEdgeMask[dir][i][0]];
        Node* e[4];
        for (int j = 0; j < 4; j++)
            e[j] = branch[order[j]] ? node[order[j]]->child[kFaceProcEdgeMask[dir][i][1 + j]] : node[order[j]];
        edge_proc(e, kFaceProcEdgeMask[dir][i][5], m);
    }
}

// ContourCellProc (octree.cpp:436-474)
void cell_proc(Node* n, Mesh& m) {
    if (!n || n->leaf) return;
    for (int i = 0; i < 8; i++) cell_proc(n->child[i], m);
    for (int i = 0; i < 12; i++) {
        Node* f[2] = {n->child[kCellProcFaceMask[i][0]], n->child[kCellProcFaceMask[i][1]]};
        face_proc(f, kCellProcFaceMask[i][2], m);
    }
    for (int i = 0; i < 6; i++) {
        Node* e[4];
        for (int j = 0; j < 4; j++) e[j] = n->child[kCellProcEdgeMask[i][j]];
        edge_proc(e, kCellProcEdgeMask[i][4], m);
    }
}

// FilterSeamNode (clipmap.cpp:508-538)
bool filter_seam_node(int child, const int32_t bounds[3], const int32_t mn[3], const int32_t mx[3]) {
    switch (child) {
        case 0: return mx[0] == bounds[0] || mx[1] == bounds[1] || mx[2] == bounds[2];
        case 1: return mn[2] == bounds[2];
        case 2: return mn[1] == bounds[1];
        case 3: return mn[1] == bounds[1] || mn[2] == bounds[2];
        case 4: return mn[0] == bounds[0];
        case 5: return mn[0] == bounds[0] || mn[2] == bounds[2];
        case 6: return mn[0] == bounds[0] || mn[1] == bounds[1];
        case 7: return same3(mn, bounds);
    }
    return false;
}

bool inside(const int32_t mn[3], int32_t size, const int32_t p[3]) {  // AABB::pointIsInside (aabb.h:37-43)
    for (int a = 0; a < 3; a++)
        if (!(p[a] >= mn[a] && p[a] < mn[a] + size)) return false;
    return true;
}

struct Clipmap {
    int32_t root_min[3];
    int32_t root_size;
    std::map<std::array<int32_t, 4>, int> active;  // (min, size) -> chunk index

    // FindNode (clipmap.cpp:982-1006) over the complete octree
    bool find_node(const int32_t mn[3], int32_t size, const int32_t nmin[3], int32_t nsize) const {
        if (nsize == size && same3(nmin, mn)) return true;
        if (!inside(nmin, nsize, mn) || nsize <= kLeafChunk) return false;
        for (int i = 0; i < 8; i++) {
            int o[3];
            child_offset(i, o);
            const int32_t c[3] = {nmin[0] + o[0] * nsize / 2, nmin[1] + o[1] * nsize / 2, nmin[2] + o[2] * nsize / 2};
            if (find_node(mn, size, c, nsize / 2)) return true;
        }
        return false;
    }
    // FindActiveNodes (clipmap.cpp:1449-1472)
    void find_active(const int32_t nmin[3], int32_t nsize, const int32_t rmin[3], int32_t rsize,
                     std::vector<int>& out) const {
        if (inside(nmin, nsize, rmin) || inside(rmin, rsize, nmin)) {
            auto it = active.find({nmin[0], nmin[1], nmin[2], nsize});
            if (it != active.end()) {
                out.push_back(it->second);
            } else if (nsize > kLeafChunk) {
                for (int i = 0; i < 8; i++) {
                    int o[3];
                    child_offset(i, o);
                    const int32_t c[3] = {nmin[0] + o[0] * nsize / 2, nmin[1] + o[1] * nsize / 2,
                                          nmin[2] + o[2] * nsize / 2};
                    find_active(c, nsize / 2, rmin, rsize, out);
                }
            }
        }
    }
};

struct Input {
    const int32_t* chunks4;
    const int32_t* seam_offsets;
    const int32_t* seams;  // SeamNodeInfo, 12 words each
    int vpc;
    float colour[3];
};

// GenerateClipmapSeamMesh (clipmap.cpp:573-610) for the host chunk `h`
Mesh seam_mesh(const Clipmap& cm, const Input& in, int h) {
    const int32_t* host = in.chunks4 + 4 * h;
    const int32_t hsize = host[3];
    std::vector<std::unique_ptr<Node>> pool;
    std::vector<Node*> nodes;
    for (int i = 0; i < 8; i++) {
        int o[3];
        child_offset(i, o);
        const int32_t nmin[3] = {host[0] + o[0] * hsize, host[1] + o[1] * hsize, host[2] + o[2] * hsize};
        if (!cm.find_node(nmin, hsize, cm.root_min, cm.root_size)) continue;
        std::vector<int> act;
        cm.find_active(cm.root_min, cm.root_size, nmin, hsize, act);
        for (int c : act) {
            // SelectSeamNodes (clipmap.cpp:542-570) over the seam nodes GenerateMeshDataForNode made
            const int32_t* ch = in.chunks4 + 4 * c;
            const int32_t bounds[3] = {host[0] + hsize, host[1] + hsize, host[2] + hsize};
            const int size = ch[3] / (in.vpc * LEAF_SIZE_SCALE);
            const int node_size = ch[3] / in.vpc;
            for (int k = in.seam_offsets[c]; k < in.seam_offsets[c + 1]; k++) {
                const int32_t* s = in.seams + 12 * (size_t)k;
                const int32_t mn[3] = {s[0] * node_size + ch[0], s[1] * node_size + ch[1], s[2] * node_size + ch[2]};
                const int32_t mx[3] = {mn[0] + size * LEAF_SIZE_SCALE, mn[1] + size * LEAF_SIZE_SCALE,
                                       mn[2] + size * LEAF_SIZE_SCALE};
                if (!filter_seam_node(i, bounds, mn, mx) || !inside(host, 2 * hsize, mn)) continue;
                pool.emplace_back(new Node());
                Node* n = pool.back().get();
                n->leaf = true;
                for (int a = 0; a < 3; a++) n->min[a] = mn[a];
                n->size = node_size;
                float f[8];
                std::memcpy(f, s + 4, sizeof(f));
                for (int a = 0; a < 3; a++) {
                    n->position[a] = f[a];
                    n->normal[a] = f[4 + a];
                }
                n->material_info = s[3];
                nodes.push_back(n);
            }
        }
    }
    Mesh m;
    Node* root = construct_upwards(nodes, host, 2 * hsize, pool);
    if (!root) return m;
    vertex_indices(root, in.colour, m);
    cell_proc(root, m);
    if (m.triangles.empty()) m.vertices.clear();  // Octree_GenerateMesh returns no mesh (octree.cpp:536-540)
    return m;
}

}  // namespace seam

// ---- edge-collapse mesh simplification ------------------------------------------
//
// ngMeshSimplifier (ng_mesh_simplify.cpp:441-540) with its QEF
// (qef_simd.h:93-530) restated in scalar float arithmetic, lane by lane as the
// SSE code computes it.  One deliberate difference: givens_coeffs_sym's
// c = _mm_rsqrt_ps(1 + tan^2) (qef_simd.h:209), an approximation whose result
// differs between x86 implementations, is 1 / sqrt(1 + tan^2) correctly
// rounded here.  The random edge subsets come from std::mt19937 and
// std::uniform_int_distribution as the reference calls them (libstdc++'s
// distribution; an MSVC build of the reference draws differently).

namespace collapse {

struct Opt {
    float edge_fraction;
    int32_t max_iterations;
    float target_percentage;
    float max_error;
    float max_edge_size;
    float min_angle_cosine;
};
struct MV {  // MeshVertex
    float p[4], n[4], c[4];
};

float dot4(const float a[4], const float b[4]) {  // vec4_dot (qef_simd.h:101-109)
    float m[4];
    for (int i = 0; i < 4; i++) m[i] = a[i] * b[i];
    return (m[0] + m[1]) + (m[3] + m[2]);
}
void mul_m4(const float a[4], const float B[4][4], float r[4]) {  // vec4_mul_m4x4 (qef_simd.h:114-121)
    for (int j = 0; j < 4; j++) {
        float t = a[0] * B[0][j];
        t = t + a[1] * B[1][j];
        t = t + a[2] * B[2][j];
        t = t + a[3] * B[3][j];
        r[j] = t;
    }
}

void givens(const float vt[4][4], float c[3], float s[3]) {  // givens_coeffs_sym (qef_simd.h:163-224)
    const float pp[3] = {vt[0][0], vt[0][0], vt[1][1]};
    const float pq[3] = {vt[0][1], vt[0][2], vt[1][2]};
    const float qq[3] = {vt[1][1], vt[2][2], vt[2][2]};
    for (int k = 0; k < 3; k++) {
        const float tau = (qq[k] - pp[k]) / (pq[k] * 2.f);
        const float stt = std::sqrt(tau * tau + 1.f);
        const float tan = 1.f / (tau >= 0.f ? tau + stt : tau - stt);
        const float ck = 1.f / std::sqrt(1.f + tan * tan);
        const float sk = tan * ck;
        c[k] = pq[k] == 0.f ? 1.f : ck;
        s[k] = pq[k] == 0.f ? 0.f : sk;
    }
}

void rotateq_xy(float vt[4][4], const float c[3], const float s[3]) {  // qef_simd.h:228-277, as written
    const float u[3] = {vt[0][0], vt[0][0], vt[1][1]};
    const float v[3] = {vt[1][1], vt[2][2], vt[2][2]};
    const float a[3] = {vt[0][1], vt[0][2], vt[1][2]};
    float x[3], y[3];
    for (int k = 0; k < 3; k++) {
        const float cc = c[k] * c[k], ss = s[k] * s[k];
        const float mx = ((2.f * c[k]) * s[k]) * a[k];
        const float x0 = cc * u[k];
        x[k] = (x0 - mx) + ss * v[k];
        y[k] = (x0 + mx) + (cc + v[k]);
    }
    vt[0][0] = x[0];
    vt[0][0] = x[1];
    vt[1][1] = x[2];
    vt[0][1] = y[0];
    vt[0][2] = y[1];
    vt[1][2] = y[2];
}

void svd_rotate(float vt[4][4], float V[4][4], float c, float s, int a, int b) {  // qef_simd.h:281-322
    if (vt[a][b] == 0.f) return;
    const float u[4] = {V[0][a], V[1][a], V[2][a], vt[0][3 - b]};
    const float v[4] = {V[0][b], V[1][b], V[2][b], vt[1 - a][2]};
    float x[4], y[4];
    for (int k = 0; k < 4; k++) {
        x[k] = c * u[k] - s * v[k];
        y[k] = s * u[k] + c * v[k];
    }
    for (int i = 0; i < 3; i++) V[i][a] = x[i];
    vt[0][3 - b] = x[3];
    for (int i = 0; i < 3; i++) V[i][b] = y[i];
    vt[1 - a][2] = y[3];
    vt[a][b] = 0.f;
}

// qef_solve_from_points over two (position, normal) pairs (qef_simd.h:403-480)
float qef2(const MV& v0, const MV& v1, float out[4]) {
    float ATA[4][4] = {}, ATb[4] = {}, acc[4] = {};
    const MV* vs[2] = {&v0, &v1};
    for (const MV* v : vs) {
        const float* n = v->n;
        for (int r = 0; r < 3; r++)
            for (int j = 0; j < 4; j++) ATA[r][j] = ATA[r][j] + n[r] * n[j];
        const float d = dot4(v->p, n);
        for (int j = 0; j < 3; j++) ATb[j] = ATb[j] + d * n[j];
        ATb[3] = ATb[3] + 0.f * n[3];
        for (int j = 0; j < 4; j++) acc[j] = acc[j] + v->p[j];
    }
    float mass[4];
    for (int j = 0; j < 4; j++) mass[j] = acc[j] / acc[3];
    float p[4];
    mul_m4(mass, ATA, p);
    for (int j = 0; j < 4; j++) p[j] = ATb[j] - p[j];
    // svd_solve_ATA_ATb (qef_simd.h:384-399)
    float V[4][4] = {{1.f, 0.f, 0.f, 0.f}, {0.f, 1.f, 0.f, 0.f}, {0.f, 0.f, 1.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    float vt[4][4];
    std::memcpy(vt, ATA, sizeof(vt));
    for (int sweep = 0; sweep < 5; sweep++) {
        float c[3], s[3];
        givens(vt, c, s);
        rotateq_xy(vt, c, s);
        svd_rotate(vt, V, c[0], s[0], 0, 1);
        svd_rotate(vt, V, c[1], s[1], 0, 2);
        svd_rotate(vt, V, c[2], s[2], 1, 2);
    }
    const float sigma[4] = {vt[0][0], vt[1][1], vt[2][2], 0.f};
    float inv[4];
    for (int j = 0; j < 4; j++) {  // svd_invdet (qef_simd.h:354-365)
        const float ox = 1.f / sigma[j];
        const float ax = std::fabs(sigma[j]), aox = std::fabs(ox);
        const float mn = ax < aox ? ax : aox;
        inv[j] = mn >= 0.1f ? ox : 0.f;
    }
    float O[4][4];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 4; j++) O[i][j] = V[i][j] * inv[j];
    for (int j = 0; j < 4; j++) O[3][j] = 0.f;
    for (int i = 0; i < 4; i++) {
        float row[4];
        mul_m4(O[i], V, row);
        std::memcpy(O[i], row, sizeof(row));
    }
    float x[4];
    mul_m4(p, O, x);
    float t[4];
    mul_m4(x, ATA, t);
    for (int j = 0; j < 4; j++) t[j] = ATb[j] - t[j];
    const float error = dot4(t, t);
    for (int j = 0; j < 4; j++) out[j] = x[j] + mass[j];
    return error;
}

struct Edge {
    uint32_t mn, mx;
    uint64_t idx() const { return (uint64_t)mn | ((uint64_t)mx << 32); }  // the union's idx_ (little endian)
};

// ngMeshSimplifier (ng_mesh_simplify.cpp:441-540); returns the simplified mesh
void simplify(std::vector<MV>& verts, std::vector<std::array<int32_t, 3>>& tris, const float offset[4],
              const Opt& o) {
    if (tris.size() < 100 || verts.size() < 100) return;
    std::vector<MV> vs = verts;
    for (MV& v : vs)
        for (int j = 0; j < 4; j++) v.p[j] = v.p[j] - offset[j];
    std::vector<std::array<int32_t, 3>> ts = tris;
    // BuildCandidateEdges (ng_mesh_simplify.cpp:122-177)
    std::vector<Edge> edges;
    for (const auto& t : ts) {
        edges.push_back({(uint32_t)std::min(t[0], t[1]), (uint32_t)std::max(t[0], t[1])});
        edges.push_back({(uint32_t)std::min(t[1], t[2]), (uint32_t)std::max(t[1], t[2])});
        edges.push_back({(uint32_t)std::min(t[0], t[2]), (uint32_t)std::max(t[0], t[2])});
    }
    std::sort(edges.begin(), edges.end(), [](const Edge& a, const Edge& b) { return a.idx() < b.idx(); });
    std::vector<Edge> filtered;
    std::vector<char> boundary(vs.size(), 0);
    Edge prev = edges[0];
    int count = 1;
    for (size_t i = 1; i < edges.size(); i++) {  // the last run is never examined, as in the reference
        const Edge cur = edges[i];
        if (cur.idx() != prev.idx()) {
            if (count == 1)
                boundary[prev.mn] = boundary[prev.mx] = 1;
            else
                filtered.push_back(prev);
            count = 1;
        } else {
            count++;
        }
        prev = cur;
    }
    edges.clear();
    for (const Edge& e : filtered)
        if (!boundary[e.mn] && !boundary[e.mx]) edges.push_back(e);
    std::vector<int> degree(vs.size(), 0);
    for (const auto& t : ts)
        for (int k = 0; k < 3; k++) degree[t[k]]++;
    const int target = (int)((float)ts.size() * o.target_percentage);
    std::vector<float> cpos(4 * edges.size()), cnrm(4 * edges.size());
    int iterations = 0;
    while ((int)ts.size() > target && iterations++ < o.max_iterations) {
        std::vector<int> edge_id(vs.size(), -1), coll_target(vs.size(), -1);
        std::vector<int> valid;
        // FindValidCollapses (ng_mesh_simplify.cpp:181-278)
        std::mt19937 prng;
        prng.seed(42);
        const int num_random = (int)((float)edges.size() * o.edge_fraction);
        std::uniform_int_distribution<int> dist(0, (int)(edges.size() - 1));
        std::vector<int> random(num_random);
        for (int i = 0; i < num_random; i++) random[i] = dist(prng);
        std::sort(random.begin(), random.end());
        std::vector<float> min_cost(vs.size(), FLT_MAX);
        int valid_count = 0;
        for (int i : random) {
            const Edge& e = edges[i];
            const MV& a = vs[e.mn];
            const MV& b = vs[e.mx];
            if (dot4(a.n, b.n) < o.min_angle_cosine) continue;
            float d[4];
            for (int j = 0; j < 4; j++) d[j] = b.p[j] - a.p[j];
            if (dot4(d, d) > o.max_edge_size * o.max_edge_size) continue;
            if ((double)std::fabs(a.c[3] - b.c[3]) > 1e-3) continue;
            const int deg = degree[e.mn] + degree[e.mx];
            if (deg > 16) continue;  // COLLAPSE_MAX_DEGREE
            float pos[4];
            float error = qef2(a, b, pos);
            if (error > 0.f) error = 1.f / error;
            const int penalty = std::max(0, deg - 10);
            error += (float)penalty * (o.max_error * 0.1f);
            if (error > o.max_error) continue;
            valid.push_back(i);
            for (int j = 0; j < 4; j++) cnrm[4 * i + j] = (a.n[j] - b.n[j]) * 0.5f;
            cpos[4 * i] = pos[0];
            cpos[4 * i + 1] = pos[1];
            cpos[4 * i + 2] = pos[2];
            cpos[4 * i + 3] = 1.f;
            if (error < min_cost[e.mn]) {
                min_cost[e.mn] = error;
                edge_id[e.mn] = i;
            }
            if (error < min_cost[e.mx]) {
                min_cost[e.mx] = error;
                edge_id[e.mx] = i;
            }
            valid_count++;
        }
        if (valid_count == 0) break;
        // CollapseEdges (ng_mesh_simplify.cpp:282-306)
        for (int i : valid) {
            const Edge& e = edges[i];
            if (edge_id[e.mn] == i && edge_id[e.mx] == i) {
                coll_target[e.mx] = (int)e.mn;
                std::memcpy(vs[e.mn].p, &cpos[4 * i], 16);
                std::memcpy(vs[e.mn].n, &cnrm[4 * i], 16);
            }
        }
        // RemoveTriangles (ng_mesh_simplify.cpp:310-352)
        std::fill(degree.begin(), degree.end(), 0);
        std::vector<std::array<int32_t, 3>> kept;
        for (auto t : ts) {
            for (int k = 0; k < 3; k++)
                if (coll_target[t[k]] != -1) t[k] = coll_target[t[k]];
            if (t[0] == t[1] || t[0] == t[2] || t[1] == t[2]) continue;
            for (int k = 0; k < 3; k++) degree[t[k]]++;
            kept.push_back(t);
        }
        ts.swap(kept);
        // RemoveEdges (ng_mesh_simplify.cpp:356-380)
        std::vector<Edge> ek;
        for (Edge e : edges) {
            if (coll_target[e.mn] != -1) e.mn = (uint32_t)coll_target[e.mn];
            if (coll_target[e.mx] != -1) e.mx = (uint32_t)coll_target[e.mx];
            if (e.mn != e.mx) ek.push_back(e);
        }
        edges.swap(ek);
    }
    // CompactVertices (ng_mesh_simplify.cpp:384-421) and the offset added back
    std::vector<char> used(vs.size(), 0);
    for (const auto& t : ts)
        for (int k = 0; k < 3; k++) used[t[k]] = 1;
    std::vector<int> remap(vs.size(), -1);
    std::vector<MV> out;
    for (size_t i = 0; i < vs.size(); i++)
        if (used[i]) {
            remap[i] = (int)out.size();
            out.push_back(vs[i]);
        }
    for (auto& t : ts)
        for (int k = 0; k < 3; k++) t[k] = remap[t[k]];
    for (MV& v : out)
        for (int j = 0; j < 4; j++) v.p[j] = v.p[j] + offset[j];
    verts.swap(out);
    tris.swap(ts);
}

}  // namespace collapse

extern "C" {

int orc_clipmap_select(const float cam[3], const int32_t root_min[3], int32_t root_size, int32_t* out4, int32_t cap) {
    if (!clipmap::valid_root(root_size)) return -1;
    clipmap::Out o{out4, cap};
    clipmap::select(root_min, root_size, false, cam, o);
    return o.n;
}

int orc_clipmap_nodes_in_aabb(const int32_t bmin[3], const int32_t bmax[3], const int32_t root_min[3],
                              int32_t root_size, int32_t* out4, int32_t cap) {
    if (!clipmap::valid_root(root_size)) return -1;
    std::vector<int32_t> boxes = {bmin[0], bmin[1], bmin[2], bmax[0], bmax[1], bmax[2]};
    clipmap::Out o{out4, cap};
    clipmap::inside(root_min, root_size, boxes, o);
    return o.n;
}

int orc_clipmap_touched(const orc_csg_op* ops, int32_t n, const int32_t root_min[3], int32_t root_size,
                        int32_t* out4, int32_t cap) {
    if (!clipmap::valid_root(root_size)) return -1;
    std::vector<int32_t> boxes(6 * (size_t)std::max(n, 0));
    for (int i = 0; i < n; i++) orc_csg_op_bounds(&ops[i], &boxes[6 * i], &boxes[6 * i + 3]);
    clipmap::Out o{out4, cap};
    if (n > 0) clipmap::inside(root_min, root_size, boxes, o);
    return o.n;
}

int orc_seam_generate(const int32_t* chunks4, const int32_t* seam_offsets, int32_t num_chunks, const int32_t* seams,
                      int32_t vpc, const int32_t root_min[3], int32_t root_size, const int32_t* hosts,
                      int32_t num_hosts, const float colour[3], float* vertices, int64_t vertex_cap,
                      int32_t* triangles, int64_t triangle_cap, int32_t* host_counts, int32_t threads) {
    if (num_chunks < 0 || num_hosts < 0 || vpc <= 0) return -1;
    seam::Clipmap cm;
    for (int a = 0; a < 3; a++) cm.root_min[a] = root_min[a];
    cm.root_size = root_size;
    for (int c = 0; c < num_chunks; c++)
        cm.active[{chunks4[4 * c], chunks4[4 * c + 1], chunks4[4 * c + 2], chunks4[4 * c + 3]}] = c;
    seam::Input in{chunks4, seam_offsets, seams, vpc, {colour[0], colour[1], colour[2]}};
    std::vector<seam::Mesh> meshes(num_hosts);
    if (threads < 1) threads = 1;
    std::atomic<int> next{0};
    auto worker = [&]() {
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= num_hosts) break;
            meshes[i] = seam::seam_mesh(cm, in, hosts[i]);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    int64_t nv = 0, nt = 0;
    for (int i = 0; i < num_hosts; i++) {
        host_counts[2 * i] = (int32_t)(meshes[i].vertices.size() / 12);
        host_counts[2 * i + 1] = (int32_t)(meshes[i].triangles.size() / 3);
        nv += host_counts[2 * i];
        nt += host_counts[2 * i + 1];
    }
    if (nv > vertex_cap || nt > triangle_cap) return -2;
    int64_t ov = 0, ot = 0;
    for (int i = 0; i < num_hosts; i++) {
        if (vertices) std::memcpy(vertices + 12 * ov, meshes[i].vertices.data(), meshes[i].vertices.size() * 4);
        if (triangles) std::memcpy(triangles + 3 * ot, meshes[i].triangles.data(), meshes[i].triangles.size() * 4);
        ov += host_counts[2 * i];
        ot += host_counts[2 * i + 1];
    }
    return 0;
}

int orc_mesh_collapse(const float* vertices, int32_t nv, const int32_t* triangles, int32_t nt, const float offset[4],
                      const float options[6], float* out_vertices, int32_t* out_nv, int32_t* out_triangles,
                      int32_t* out_nt) {
    collapse::Opt o{options[0], (int32_t)options[1], options[2], options[3], options[4], options[5]};
    std::vector<collapse::MV> vs(nv);
    std::memcpy(vs.data(), vertices, sizeof(collapse::MV) * nv);
    std::vector<std::array<int32_t, 3>> ts(nt);
    std::memcpy(ts.data(), triangles, 12 * (size_t)nt);
    collapse::simplify(vs, ts, offset, o);
    std::memcpy(out_vertices, vs.data(), sizeof(collapse::MV) * vs.size());
    std::memcpy(out_triangles, ts.data(), 12 * ts.size());
    *out_nv = (int32_t)vs.size();
    *out_nt = (int32_t)ts.size();
    return 0;
}

int orc_uniform_draws(int32_t hi, int32_t n, int32_t* out) {
    // the draws FindValidCollapses makes (ng_mesh_simplify.cpp:194-205)
    std::mt19937 prng;
    prng.seed(42);
    std::uniform_int_distribution<int> dist(0, hi);
    for (int i = 0; i < n; i++) out[i] = dist(prng);
    return 0;
}

int64_t orc_mesh_collapse_many(const float* vertices, const int32_t* triangles, const int32_t* ranges, int32_t n,
                               const float* offsets, const float* options, int32_t threads) {
    if (threads < 1) threads = 1;
    std::atomic<int> next{0};
    std::atomic<int64_t> total{0};
    auto worker = [&]() {
        std::vector<float> ov;
        std::vector<int32_t> ot;
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n) break;
            const int32_t* r = ranges + 4 * i;  // vertex offset, vertices, triangle offset, triangles
            ov.resize(12 * (size_t)std::max(r[1], 1));
            ot.resize(3 * (size_t)std::max(r[3], 1));
            int32_t nv = 0, nt = 0;
            orc_mesh_collapse(vertices + 12 * (size_t)r[0], r[1], triangles + 3 * (size_t)r[2], r[3], offsets + 4 * i,
                              options + 6 * i, ov.data(), &nv, ot.data(), &nt);
            total += nt;
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    return total.load();
}

int64_t orc_clipmap_select_many(const float* cams, int32_t n, const int32_t root_min[3], int32_t root_size,
                                int32_t threads) {
    if (!clipmap::valid_root(root_size) || n < 0) return -1;
    if (threads < 1) threads = 1;
    std::atomic<int> next{0};
    std::atomic<int64_t> total{0};
    auto worker = [&]() {
        std::vector<int32_t> buf(4 * 8192);
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n) break;
            clipmap::Out o{buf.data(), 8192};
            clipmap::select(root_min, root_size, false, cams + 3 * (size_t)i, o);
            total += o.n;
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    return total.load();
}

int64_t orc_mesh_chunks(const orc_density* d, const orc_chunk_args* chunks, int32_t n, int32_t threads) {
    return orc_mesh_chunks_simplified(d, chunks, n, threads, -1.f);
}

int64_t orc_mesh_chunks_simplified(const orc_density* d, const orc_chunk_args* chunks, int32_t n, int32_t threads,
                                   float threshold) {
    if (!g_lut_ready || n <= 0) return -1;
    if (threads < 1) threads = 1;
    std::atomic<int> next{0};
    std::atomic<int64_t> total{0};
    auto worker = [&]() {
        Chunk ch;
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n) break;
            if (run_chunk(ch, *d, chunks[i], g_lut) != 0) continue;
            if (threshold >= 0.f) {
                simplify_chunk(ch, threshold);
                total += (int64_t)ch.simp_vertex_count + (int64_t)ch.simp_triangles.size() / 3;
            } else {
                total += (int64_t)ch.mesh_vertex_count + (int64_t)ch.triangles.size() / 3;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    return total.load();
}

}  // extern "C"
