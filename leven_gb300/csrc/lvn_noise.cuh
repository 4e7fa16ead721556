// lvn_noise.cuh -- device simplex noise, fractals, terrain densities and CSG
// brushes for the chunk-meshing path.
//
// Semantics follow the reference's OpenCL (leven/cl/simplex.cl, noise.cl,
// apply_csg_operation.cl, hg_sdf.glsl fBox/pR).  The library is compiled with
// -fmad=false: a multiply-add is fused only where this file calls fmaf, so the
// result of every density evaluation is a fixed sequence of IEEE single
// precision operations:
//   * dot(a,b) = fma(a.z,b.z, fma(a.y,b.y, a.x*b.x))  (2D drops the z term)
//   * octave accumulation `noise += s * amplitude` = fma(s, amplitude, noise)
//   * mix(a,b,t) = fma(b-a, t, a)
//   * the image sampler (nearest, repeat, normalised coordinates) resolves an
//     integer lattice coordinate i to texel i & 255; the 3D second lookup
//     uses u = A/255, i.e. column A for A < 255 and column 0 for A == 255
//   * snoise3's falloff constant 0.6 is single precision
//   * pow(frequency, -1) in the ridged fractal is 1.f / frequency
#pragma once
#include <cstdint>
#include <cfloat>

#include "lvn_types.h"

namespace lvn {

__device__ __forceinline__ int texel(int row, int col) { return ((row & 255) << 8) | (col & 255); }
__device__ __forceinline__ int alpha_column(int a) { return a == 255 ? 0 : a; }

// The gradient table as the noise code reads it from shared memory (64
// floats, 16-byte aligned), staged from the 16 x float4 table `grad` by the
// block's first 64 threads: the 16 (x, y) pairs in bytes 0-127, then the 16
// (z, 0) pairs in bytes 128-255.  A texel's second-table byte (alpha & 15) * 8
// addresses both halves.  Across a warp an (x, y) load touches each of the 32
// banks at most once per half-warp and a z load 16 distinct banks, so neither
// conflicts; one float4 load from a 256-byte table conflicts wherever entries
// k and k + 8 meet in one quarter-warp.
__device__ __forceinline__ void stage_gradients(float* sg, const float* grad) {
    const int t = threadIdx.x;
    if (t < 64) {
        const int k = t >> 2, c = t & 3;
        sg[(c < 2 ? 0 : 30) + 2 * k + c] = grad[t];
    }
}

__device__ __forceinline__ float dot2(float ax, float ay, float bx, float by) { return fmaf(ay, by, ax * bx); }
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return fmaf(az, bz, fmaf(ay, by, ax * bx));
}

// Two-lane single precision arithmetic (the f32x2 forms of add, sub, mul and
// fma, sm_100 and later): each lane is the IEEE round-to-nearest result of the
// scalar operation on that lane, so two independent evaluations step through
// one instruction together and give the scalar code's bits.
// One exception: the code generator fuses a two-lane product that feeds a
// two-lane add or sub into one two-lane fma, even with -fmad=false and an
// explicit .rn (measured on GB300: every such mismatch equals the fused
// result).  So a product whose only use is an add or sub is taken in scalar
// (mul2s below): scalar products with a rounding mode are never fused.
__device__ __forceinline__ float2 v2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 mul2s(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
__device__ __forceinline__ float2 floor2(float2 a) { return make_float2(floorf(a.x), floorf(a.y)); }
__device__ __forceinline__ float2 max02(float2 a) { return make_float2(fmaxf(a.x, 0.f), fmaxf(a.y, 0.f)); }

// kSharedTables: the kernel staged the two lookup tables in shared memory
// (plain loads); otherwise they are read from global memory through the
// read-only path.
template <bool kSharedTables>
struct NoiseT {
    const uint8_t* __restrict__ t3;   // the two simplex lookup tables (kT3Row x kT3Row texels each)
    const float* __restrict__ g;      // 16 x 4 gradient table, staged in shared memory

    __device__ __forceinline__ int tab(int i) const {
        if (kSharedTables) return t3[i];
        return __ldg(t3 + i);
    }

    // the 2D gradient of texel b of the padded tables (row * kT3Row + column):
    // the second table holds (alpha & 15) * 8, the byte offset of its (x, y)
    // pair in the staged gradient table (stage_gradients)
    __device__ __forceinline__ float2 grad2(int b) const {
        const int kb = tab(kT3Second + b);
        return *reinterpret_cast<const float2*>(reinterpret_cast<const char*>(g) + kb);
    }

    // snoise2 (simplex.cl:158-216).  The three corners' texels are (iy, ix),
    // (iy, ix+1) or (iy+1, ix) by the x0 > y0 test, and (iy+1, ix+1), read
    // from the padded table without a wrap.
    __device__ __forceinline__ float snoise2(float px, float py) const {
        const float F2 = 0.366025403784f;
        const float G2 = 0.211324865405f;
        const float C2 = 1.f - 2.f * G2;
        const float s = (px + py) * F2;
        const float pix = floorf(px + s);
        const float piy = floorf(py + s);
        const float t = (pix + piy) * G2;
        const float x0 = px - (pix - t);
        const float y0 = py - (piy - t);
        const bool xgt = x0 > y0;
        const int b = ((int)piy & 255) * kT3Row + ((int)pix & 255);

        // A corner outside the kernel radius (t < 0) contributes 0.  Clamping
        // t to 0 instead of branching gives 0 * dot = +-0 there, and a signed
        // zero term leaves every sum below unchanged: the fractals accumulate
        // with fma(s, amplitude, acc) and the ridged one takes |s| first.
        const float2 ga = grad2(b), gb = grad2(b + (xgt ? 1 : kT3Row)), gc = grad2(b + kT3Row + 1);
        float t0 = fmaxf(0.5f - dot2(x0, y0, x0, y0), 0.f);
        t0 = t0 * t0;
        const float n0 = (t0 * t0) * dot2(ga.x, ga.y, x0, y0);
        const float x1 = (x0 - (xgt ? 1.f : 0.f)) + G2, y1 = (y0 - (xgt ? 0.f : 1.f)) + G2;
        float t1 = fmaxf(0.5f - dot2(x1, y1, x1, y1), 0.f);
        t1 = t1 * t1;
        const float n1 = (t1 * t1) * dot2(gb.x, gb.y, x1, y1);
        const float x2 = x0 - C2, y2 = y0 - C2;
        float t2 = fmaxf(0.5f - dot2(x2, y2, x2, y2), 0.f);
        t2 = t2 * t2;
        const float n2 = (t2 * t2) * dot2(gc.x, gc.y, x2, y2);
        return 70.f * ((n0 + n1) + n2);
    }

    // snoise2 at two points, one per lane, in the operation order of snoise2
    __device__ __forceinline__ float2 snoise2x2(float2 px, float2 py) const {
        const float F2 = 0.366025403784f;
        const float G2 = 0.211324865405f;
        const float C2 = 1.f - 2.f * G2;
        const float2 s = mul2s(add2(px, py), v2(F2));
        const float2 pix = floor2(add2(px, s));
        const float2 piy = floor2(add2(py, s));
        const float2 t = mul2s(add2(pix, piy), v2(G2));
        const float2 x0 = sub2(px, sub2(pix, t));
        const float2 y0 = sub2(py, sub2(piy, t));
        const bool xg0 = x0.x > y0.x, xg1 = x0.y > y0.y;
        const int ba = ((int)piy.x & 255) * kT3Row + ((int)pix.x & 255);
        const int bb = ((int)piy.y & 255) * kT3Row + ((int)pix.y & 255);
        const float2 ga0 = grad2(ba), gb0 = grad2(ba + (xg0 ? 1 : kT3Row)), gc0 = grad2(ba + kT3Row + 1);
        const float2 ga1 = grad2(bb), gb1 = grad2(bb + (xg1 ? 1 : kT3Row)), gc1 = grad2(bb + kT3Row + 1);

        float2 t0 = max02(sub2(v2(0.5f), fma2(y0, y0, mul2(x0, x0))));
        t0 = mul2(t0, t0);
        const float2 n0 = mul2s(mul2(t0, t0), make_float2(dot2(ga0.x, ga0.y, x0.x, y0.x), dot2(ga1.x, ga1.y, x0.y, y0.y)));
        const float2 x1 = add2(sub2(x0, make_float2(xg0 ? 1.f : 0.f, xg1 ? 1.f : 0.f)), v2(G2));
        const float2 y1 = add2(sub2(y0, make_float2(xg0 ? 0.f : 1.f, xg1 ? 0.f : 1.f)), v2(G2));
        float2 t1 = max02(sub2(v2(0.5f), fma2(y1, y1, mul2(x1, x1))));
        t1 = mul2(t1, t1);
        const float2 n1 = mul2s(mul2(t1, t1), make_float2(dot2(gb0.x, gb0.y, x1.x, y1.x), dot2(gb1.x, gb1.y, x1.y, y1.y)));
        const float2 x2 = sub2(x0, v2(C2)), y2 = sub2(y0, v2(C2));
        float2 t2 = max02(sub2(v2(0.5f), fma2(y2, y2, mul2(x2, x2))));
        t2 = mul2(t2, t2);
        const float2 n2 = mul2s(mul2(t2, t2), make_float2(dot2(gc0.x, gc0.y, x2.x, y2.x), dot2(gc1.x, gc1.y, x2.y, y2.y)));
        return mul2(v2(70.f), add2(add2(n0, n1), n2));
    }

    // the gradient of one snoise3 corner: the texel (iy, ix)'s alpha picks the
    // column of the texel in row iz whose alpha & 15 is the gradient index.
    // b1 = the first table's index of (iy, ix), b2 = the second table's row
    // offset of iz (rows and columns in [0, 256], so a corner adds its 0/1
    // steps without a wrap).
    __device__ __forceinline__ float4 grad3(int b1, int b2) const {
        const int a = tab(b1);
        const int kb = tab(kT3Second + b2 + a);
        // the (x, y) pair and, 128 bytes on, z (stage_gradients): two
        // conflict-free shared loads
        const char* e = reinterpret_cast<const char*>(g) + kb;
        const float2 xy = *reinterpret_cast<const float2*>(e);
        return make_float4(xy.x, xy.y, *reinterpret_cast<const float*>(e + 128), 0.f);
    }

    // one corner of snoise3 with its gradient
    __device__ __forceinline__ float corner3(float4 gk, float x, float y, float z) const {
        float tt = fmaxf(0.6f - dot3(x, y, z, x, y, z), 0.f);  // clamped as in snoise2
        tt = tt * tt;
        return (tt * tt) * dot3(gk.x, gk.y, gk.z, x, y, z);
    }

    // snoise3 (simplex.cl:218-289) with simplex() ranking (simplex.cl:133-156)
    __device__ __forceinline__ float snoise3(float px, float py, float pz) const {
        const float F3 = 0.333333333333f;
        const float G3 = 0.166666666667f;
        const float C2 = 2.f * G3;
        const float C3 = 1.f - 3.f * G3;
        const float s = ((px + py) + pz) * F3;
        const float pix = floorf(px + s);
        const float piy = floorf(py + s);
        const float piz = floorf(pz + s);
        const float t = ((pix + piy) + piz) * G3;
        const float x0 = px - (pix - t);
        const float y0 = py - (piy - t);
        const float z0 = pz - (piz - t);
        const int b1 = ((int)piy & 255) * kT3Row + ((int)pix & 255), b2 = ((int)piz & 255) * kT3Row;
        // simplex() ranks each axis by its two comparisons (rank 0..2): the
        // second corner steps the axes of rank 2, the third those of rank >= 1,
        // i.e. clamp(rank - 1, 0, 1) = both comparisons, clamp(rank, 0, 1) = either
        const bool xy = x0 >= y0, xz = x0 >= z0, yz = y0 >= z0;
        const bool o1x = xy && xz, o1y = !xy && yz, o1z = !xz && !yz;
        const bool o2x = xy || xz, o2y = !xy || yz, o2z = !xz || !yz;
        const float n0 = corner3(grad3(b1, b2), x0, y0, z0);
        const float n1 = corner3(grad3(b1 + (o1y ? kT3Row : 0) + o1x, b2 + (o1z ? kT3Row : 0)),
                                 (x0 - (o1x ? 1.f : 0.f)) + G3, (y0 - (o1y ? 1.f : 0.f)) + G3, (z0 - (o1z ? 1.f : 0.f)) + G3);
        const float n2 = corner3(grad3(b1 + (o2y ? kT3Row : 0) + o2x, b2 + (o2z ? kT3Row : 0)),
                                 (x0 - (o2x ? 1.f : 0.f)) + C2, (y0 - (o2y ? 1.f : 0.f)) + C2, (z0 - (o2z ? 1.f : 0.f)) + C2);
        const float n3 = corner3(grad3(b1 + kT3Row + 1, b2 + kT3Row), x0 - C3, y0 - C3, z0 - C3);
        return 32.f * (((n0 + n1) + n2) + n3);
    }

    // one snoise3 corner at two points, one per lane (corner3's operations)
    __device__ __forceinline__ float2 corner3x2(float4 ga, float4 gb, float2 x, float2 y, float2 z) const {
        float2 tt = max02(sub2(v2(0.6f), fma2(z, z, fma2(y, y, mul2(x, x)))));
        tt = mul2(tt, tt);
        return mul2s(mul2(tt, tt), make_float2(dot3(ga.x, ga.y, ga.z, x.x, y.x, z.x), dot3(gb.x, gb.y, gb.z, x.y, y.y, z.y)));
    }

    // snoise3 at two points, one per lane, in the operation order of snoise3
    __device__ __forceinline__ float2 snoise3x2(float2 px, float2 py, float2 pz) const {
        const float F3 = 0.333333333333f;
        const float G3 = 0.166666666667f;
        const float C2 = 2.f * G3;
        const float C3 = 1.f - 3.f * G3;
        const float2 s = mul2s(add2(add2(px, py), pz), v2(F3));
        const float2 pix = floor2(add2(px, s));
        const float2 piy = floor2(add2(py, s));
        const float2 piz = floor2(add2(pz, s));
        const float2 t = mul2s(add2(add2(pix, piy), piz), v2(G3));
        const float2 x0 = sub2(px, sub2(pix, t));
        const float2 y0 = sub2(py, sub2(piy, t));
        const float2 z0 = sub2(pz, sub2(piz, t));
        const int b1a = ((int)piy.x & 255) * kT3Row + ((int)pix.x & 255), b2a = ((int)piz.x & 255) * kT3Row;
        const int b1b = ((int)piy.y & 255) * kT3Row + ((int)pix.y & 255), b2b = ((int)piz.y & 255) * kT3Row;
        // simplex() (simplex.cl:74-100) in exact 0 / 1 float arithmetic, both
        // lanes at once: with fxy = (x0 >= y0) etc., the axis of rank 2 steps
        // first (o1 = the product of its two comparisons) and the axes of rank
        // >= 1 step second (o2 = a + b - ab, their "or").  The texel offsets of
        // those corners are the same 0 / 1 values times the row stride, exact in
        // float and converted once per lane.
        auto ge = [](float a, float b) { return a >= b ? 1.f : 0.f; };
        const float2 fxy = make_float2(ge(x0.x, y0.x), ge(x0.y, y0.y));
        const float2 fxz = make_float2(ge(x0.x, z0.x), ge(x0.y, z0.y));
        const float2 fyz = make_float2(ge(y0.x, z0.x), ge(y0.y, z0.y));
        const float2 nxy = sub2(v2(1.f), fxy), nxz = sub2(v2(1.f), fxz), nyz = sub2(v2(1.f), fyz);
        const float2 o1x = mul2(fxy, fxz), o2x = sub2(add2(fxy, fxz), o1x);
        const float2 o1y = mul2(nxy, fyz), o2y = sub2(add2(nxy, fyz), o1y);
        const float2 o1z = mul2(nxz, nyz), o2z = sub2(add2(nxz, nyz), o1z);
        const float R = (float)kT3Row;
        const float2 r1 = fma2(o1y, v2(R), o1x), r2 = fma2(o2y, v2(R), o2x);
        const float2 s1 = mul2(o1z, v2(R)), s2 = mul2(o2z, v2(R));
        const float2 n0 = corner3x2(grad3(b1a, b2a), grad3(b1b, b2b), x0, y0, z0);
        const float2 n1 = corner3x2(grad3(b1a + (int)r1.x, b2a + (int)s1.x), grad3(b1b + (int)r1.y, b2b + (int)s1.y),
                                    add2(sub2(x0, o1x), v2(G3)), add2(sub2(y0, o1y), v2(G3)),
                                    add2(sub2(z0, o1z), v2(G3)));
        const float2 n2 = corner3x2(grad3(b1a + (int)r2.x, b2a + (int)s2.x), grad3(b1b + (int)r2.y, b2b + (int)s2.y),
                                    add2(sub2(x0, o2x), v2(C2)), add2(sub2(y0, o2y), v2(C2)),
                                    add2(sub2(z0, o2z), v2(C2)));
        const float2 n3 = corner3x2(grad3(b1a + kT3Row + 1, b2a + kT3Row), grad3(b1b + kT3Row + 1, b2b + kT3Row),
                                    sub2(x0, v2(C3)), sub2(y0, v2(C3)), sub2(z0, v2(C3)));
        return mul2(v2(32.f), add2(add2(add2(n0, n1), n2), n3));
    }

    // BasicFractal (noise.cl:8-36), NOISE_SCALE == 1, two octaves a step:
    // octaves i and i + 1 are the two lanes of one paired evaluation.  The
    // coordinates, amplitudes and the accumulation keep the scalar order,
    // octave by octave.  The loop is fully unrolled for the common 8-octave
    // case.
    template <int OCT>
    __device__ __forceinline__ float fbm2_fixed(float frequency, float lacunarity, float persistence, float x,
                                                float y) const {
        float px = x * 1.f, py = y * 1.f;
        float noise = 0.f, amplitude = 1.f;
        px = px * frequency;
        py = py * frequency;
#pragma unroll
        for (int i = 0; i + 1 < OCT; i += 2) {
            const float qx = px * lacunarity, qy = py * lacunarity;
            const float2 n = snoise2x2(make_float2(px, qx), make_float2(py, qy));
            noise = fmaf(n.x, amplitude, noise);
            amplitude = amplitude * persistence;
            noise = fmaf(n.y, amplitude, noise);
            amplitude = amplitude * persistence;
            px = qx * lacunarity;
            py = qy * lacunarity;
        }
        if (OCT & 1) noise = fmaf(snoise2(px, py), amplitude, noise);
        return noise;
    }
    __device__ __forceinline__ float fbm2(int octaves, float frequency, float lacunarity, float persistence, float x,
                                          float y) const {
        if (octaves == 8) return fbm2_fixed<8>(frequency, lacunarity, persistence, x, y);
        float px = x * 1.f, py = y * 1.f;
        float noise = 0.f, amplitude = 1.f;
        px = px * frequency;
        py = py * frequency;
        int i = 0;
        for (; i + 1 < octaves; i += 2) {
            const float qx = px * lacunarity, qy = py * lacunarity;
            const float2 n = snoise2x2(make_float2(px, qx), make_float2(py, qy));
            noise = fmaf(n.x, amplitude, noise);
            amplitude = amplitude * persistence;
            noise = fmaf(n.y, amplitude, noise);
            amplitude = amplitude * persistence;
            px = qx * lacunarity;
            py = qy * lacunarity;
        }
        if (i < octaves) noise = fmaf(snoise2(px, py), amplitude, noise);
        return noise;
    }

    // 3D analogue of BasicFractal (the cave term), two octaves a step as fbm2
    __device__ __forceinline__ float fbm3(int octaves, float frequency, float lacunarity, float persistence, float x,
                                          float y, float z) const {
        float px = x * frequency, py = y * frequency, pz = z * frequency;
        float noise = 0.f, amplitude = 1.f;
        int i = 0;
        for (; i + 1 < octaves; i += 2) {
            const float qx = px * lacunarity, qy = py * lacunarity, qz = pz * lacunarity;
            const float2 n = snoise3x2(make_float2(px, qx), make_float2(py, qy), make_float2(pz, qz));
            noise = fmaf(n.x, amplitude, noise);
            amplitude = amplitude * persistence;
            noise = fmaf(n.y, amplitude, noise);
            amplitude = amplitude * persistence;
            px = qx * lacunarity;
            py = qy * lacunarity;
            pz = qz * lacunarity;
        }
        if (i < octaves) noise = fmaf(snoise3(px, py, pz), amplitude, noise);
        return noise;
    }

    // Step s of fbm3: octaves 2s and 2s + 1 (the last one alone when
    // `octaves` is odd) added to `noise`, at the coordinates and amplitude the
    // full loop reaches there (the same products, in the same order), so that
    // steps 0, 1, ... chained give fbm3's value bit for bit.
    __device__ __forceinline__ float fbm3_step(int s, int octaves, float frequency, float lacunarity,
                                               float persistence, float x, float y, float z, float noise) const {
        if (2 * s >= octaves) return noise;
        float px = x * frequency, py = y * frequency, pz = z * frequency;
        float amplitude = 1.f;
        for (int i = 0; i < s; i++) {
            px = (px * lacunarity) * lacunarity;
            py = (py * lacunarity) * lacunarity;
            pz = (pz * lacunarity) * lacunarity;
            amplitude = (amplitude * persistence) * persistence;
        }
        if (2 * s + 1 < octaves) {
            const float qx = px * lacunarity, qy = py * lacunarity, qz = pz * lacunarity;
            const float2 n = snoise3x2(make_float2(px, qx), make_float2(py, qy), make_float2(pz, qz));
            noise = fmaf(n.x, amplitude, noise);
            amplitude = amplitude * persistence;
            return fmaf(n.y, amplitude, noise);
        }
        return fmaf(snoise3(px, py, pz), amplitude, noise);
    }

    // RidgedMultiFractal (noise.cl:42-81), RIDGED_MULTI_H == 1
    __device__ __forceinline__ float ridged(int octaves, float lacunarity, float gain, float offset, float x,
                                            float y) const {
        float px = x * 1.f, py = y * 1.f;
        float signal = snoise2(px, py);
        signal = fabsf(signal);
        signal = offset - signal;
        signal = signal * signal;
        float noise = signal;
        float weight = 1.f;
        float frequency = 1.f;
        for (int i = 0; i < octaves; i++) {
            px = px * lacunarity;
            py = py * lacunarity;
            weight = signal * gain;
            weight = fminf(fmaxf(weight, 0.f), 1.f);
            signal = snoise2(px, py);
            signal = fabsf(signal);
            signal = offset - signal;
            signal = signal * weight;
            const float exponent = 1.f / frequency;
            frequency = frequency * lacunarity;
            noise = fmaf(signal, exponent, noise);
        }
        noise = noise * (1.f / (float)octaves);
        return noise;
    }

    // Terrain (noise.cl:205-223)
    __device__ __forceinline__ float terrain(float x, float z) const {
        const float px = x * (1.f / 2000.f);
        const float pz = z * (1.f / 2000.f);
        float r = 0.8f * ridged(7, 2.114352f, 1.5241f, 1.f, px, pz);
        r = fminf(fmaxf(r, 0.f), 1.f);
        float billow = 0.6f * fbm2(4, 0.24f, 1.8754f, 0.433f, -4.33f * px, 7.98f * pz);
        billow = fmaf(0.5f, billow, 0.5f);
        float b2 = 0.6f * fbm2(2, 0.63f, 2.2f, 0.15f, px, pz);
        b2 = fmaf(b2, 0.5f, 0.5f);
        return fmaf(billow, r, b2);
    }

    // The height term h(x,z) of a heightfield density d = y - amp*h (+ caves)
    __device__ __forceinline__ float height(const DensityParams& d, float x, float z) const {
        if (d.mode == LVN_DENSITY_REFERENCE) return terrain(x, z);
        return fbm2(d.octaves2, d.freq2, d.lacunarity2, d.gain2, x, z);
    }
    __device__ __forceinline__ float height_amp(const DensityParams& d) const {
        return d.mode == LVN_DENSITY_REFERENCE ? 900.f : d.amp2;  // MAX_TERRAIN_HEIGHT
    }
    // density from a precomputed height term: DensityFunc (noise.cl:225-268)
    __device__ __forceinline__ float density_h(const DensityParams& d, float h, float x, float y, float z) const {
        const float base = fmaf(-height_amp(d), h, y);
        if (d.mode != LVN_DENSITY_CAVES) return base;
        return fmaf(d.amp3, fbm3(d.octaves3, d.freq3, d.lacunarity3, d.gain3, x, y, z), base);
    }
    __device__ __forceinline__ float density(const DensityParams& d, float x, float y, float z) const {
        return density_h(d, height(d, x, z), x, y, z);
    }
};
using Noise = NoiseT<false>;

// ---------------------------------------------------------------------------
// CSG brushes: apply_csg_operation.cl:42-175, hg_sdf.glsl fBox (218-221), pR (460-463)
// ---------------------------------------------------------------------------

__device__ __forceinline__ float length3(float x, float y, float z) { return sqrtf(dot3(x, y, z, x, y, z)); }

__device__ __forceinline__ float brush_density(const Brush& b, float wx, float wy, float wz) {
    const float lx = wx - b.origin[0], ly = wy - b.origin[1], lz = wz - b.origin[2];
    if (b.brush != 0) return length3(lx, ly, lz) - b.dimensions[0];  // Density_Sphere
    const float rx = fmaf(b.sin_y, lz, b.cos_y * lx);                 // pR(p.xz, rotateY)
    const float rz = fmaf(b.sin_y, -lx, b.cos_y * lz);
    const float dx = fabsf(rx) - b.dimensions[0];
    const float dy = fabsf(ly) - b.dimensions[1];
    const float dz = fabsf(rz) - b.dimensions[2];
    const float outside = length3(fmaxf(dx, 0.f), fmaxf(dy, 0.f), fmaxf(dz, 0.f));
    const float inside = fmaxf(fmaxf(fminf(dx, 0.f), fminf(dy, 0.f)), fminf(dz, 0.f));
    return outside + inside;
}

__device__ __forceinline__ void normalize3(float& x, float& y, float& z) {
    const float len = sqrtf(dot3(x, y, z, x, y, z));
    if (len == 0.f) { x = y = z = 0.f; return; }
    x = x / len;
    y = y / len;
    z = z / len;
}

}  // namespace lvn
