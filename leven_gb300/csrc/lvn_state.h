// lvn_state.h -- read-only access to liblvn's global compute state for
// translation units other than lvn_api.cu (defined at the end of lvn_api.cu).
#pragma once
#include <cstdint>

#include "lvn_types.h"

namespace lvn {

struct GlobalView {
    bool initialised;
    int device;            // the CUDA device lvn_init ran on; every table below lives there
    int num_sms;
    int32_t default_material;
    const uint8_t* perm;   // device permutation image (65536 B)
    const uint8_t* perm_t3;   // device: the two simplex lookup tables (kT3Row x kT3Row texels each)
    const float* grad;     // device gradient table (16 x 4)
    DensityParams density;
};

GlobalView global_view();
// The stored operations whose AABB overlaps [min, min + size], in store
// order, written to out[0..cap); returns their count, or -1 when more than cap.
int stored_ops_for_chunk(const int32_t min[3], int32_t size, Brush* out, int cap);
// Draws one cuckoo parameter set (10 words) from the shared generator.
void draw_hash_params(uint32_t* p);
// 1 while injected degenerate draws also apply to the device-side table
// repair (BatchPtrs::hash_fault), 0 in normal use.
int device_hash_fault();
// ColourForMinLeafSize (clipmap.cpp:329-353)
void lod_colour_for(int min_leaf_size, float c[3]);
// The batch fields derived from the density and the default material: the
// cave band (|y - amp2 h| above it, the cave term cannot change the density's
// sign; 0 without a 3D term), the bounds rem[s] on |amp3 * (fbm3's octaves 2s
// and up)| for s = 0..kCaveSteps (0 where no octave is left), and the dominant
// material of 8 corners of which n hold the default material and the rest AIR,
// for n = 0..8.
void density_fields(const DensityParams& d, int32_t default_material, float* band, float* rem,
                    int32_t dom_by_solid[9]);
// Field-index box holding every point the operations can change.
void csg_box_for(const Brush* ops, int n, const int32_t off[3], int scale, int fd, int32_t lo[3], int32_t hi[3]);

}  // namespace lvn
