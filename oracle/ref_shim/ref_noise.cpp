// ref_noise.cpp -- the reference's own noise code (leven/cl/simplex.cl,
// noise.cl), compiled on the host through cl_shim.h, behind C entry points.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref where
// the reference tree is present, and used only by tests to pin the oracle's
// restatement (oracle/lvn_oracle.cpp) against the reference source.
//
// The reference built its programs with -cl-fast-relaxed-math
// (compute.cpp:258), which lets a compiler fuse a multiply into an add, or
// not.  The restatement fixes one choice, and this harness compiles the
// reference's code under the same one: simplex.cl with no fusion outside
// dot() (this file is compiled with -ffp-contract=off), noise.cl with fusion
// (a multiply whose one use is an add becomes an fma: the octave sums, the
// terrain's remaps and its final y - 900 noise).  -fsingle-precision-constant
// makes double literals such as snoise3's 0.6 single precision, as on a device
// without doubles.
#include "cl_shim.h"

#define constant static const
#define MAX_TERRAIN_HEIGHT 900  // compute.cpp:254

#include "cl/simplex.cl"

#pragma GCC optimize("fp-contract=fast")
#include "cl/noise.cl"

namespace {
clshim_image2d g_perm = {nullptr, 256, 256};
uint8_t g_texels[256 * 256 * 4];
}  // namespace

extern "C" {

// the permutation lookup image: 256 x 256 RGBA8 texels, row-major
void ref_set_perm_image(const uint8_t* rgba) {
    std::memcpy(g_texels, rgba, sizeof(g_texels));
    g_perm.texels = g_texels;
}

float ref_snoise2(float x, float y) { return snoise2(float2(x, y), &g_perm); }
float ref_snoise3(float x, float y, float z) { return snoise3(float3(x, y, z), &g_perm); }

float ref_basic_fractal(int octaves, float frequency, float lacunarity, float persistence, float x, float y) {
    return BasicFractal(&g_perm, octaves, frequency, lacunarity, persistence, float2(x, y));
}

float ref_ridged_multi_fractal(int octaves, float lacunarity, float gain, float offset, float x, float y) {
    return RidgedMultiFractal(&g_perm, octaves, lacunarity, gain, offset, float2(x, y));
}

float ref_terrain(float x, float z) { return Terrain(float4(x, 0.f, z, 0.f), &g_perm); }

float ref_density_func(float x, float y, float z) { return DensityFunc(float4(x, y, z, 0.f), &g_perm); }

// The configured heightfield: y - amplitude * BasicFractal(octaves, frequency,
// lacunarity, persistence, (x, z)), the reference's fractal with the
// benchmark's parameters in place of Terrain's.
float ref_fbm_height_density(int octaves, float frequency, float lacunarity, float persistence, float amplitude,
                             float x, float y, float z) {
    const float h = BasicFractal(&g_perm, octaves, frequency, lacunarity, persistence, float2(x, z));
    return y - amplitude * h;
}

}
