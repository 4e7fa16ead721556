// lvn_types.h -- plain structs shared by the host orchestration and the
// device kernels of liblvn.  No CUDA or torch types; includable from C++.
#pragma once
#include <cstdint>

#include "../../include/lvn.h"

namespace lvn {

constexpr int MATERIAL_NONE = 200;  // leven/src/volume_materials.h:7
constexpr int MATERIAL_AIR = 201;   // leven/src/volume_materials.h:8

#ifdef __CUDACC__
#define LVN_HD __host__ __device__
#else
#define LVN_HD
#endif

// FindDominantMaterial (octree.cl:96-138): the most frequent material of a
// voxel's 8 corners after sorting them, AIR and NONE not counted as a run's
// continuation, the first of equal counts kept.
LVN_HD inline int dominant_material(int (&m)[8]) {
#pragma unroll
    for (int i = 1; i < 8; i++) {
        const int tmp = m[i];
        int j = i;
        for (; j >= 1 && tmp < m[j - 1]; j--) m[j] = m[j - 1];
        m[j] = tmp;
    }
    int current = m[0], count = 1, max_count = 0, max_material = 0;
#pragma unroll
    for (int i = 1; i < 8; i++) {
        const int v = m[i];
        if (v == MATERIAL_AIR || v == MATERIAL_NONE) continue;
        if (current != v) {
            if (count > max_count) {
                max_count = count;
                max_material = current;
            }
            current = v;
            count = 1;
        } else {
            count++;
        }
    }
    if (count > max_count) max_material = current;
    return max_material;
}
constexpr int LEAF_SIZE_SCALE = 4;  // leven/src/volume_constants.h:7-8
constexpr int CLIPMAP_LEAF_SIZE = 256;  // volume_constants.h:15

// cuckoo constants (leven/src/compute_cuckoo.h:6-10)
constexpr uint64_t CUCKOO_EMPTY = ~0ull;
constexpr int CUCKOO_STASH_HASH_INDEX = 4;
constexpr int CUCKOO_HASH_FN_COUNT = 5;
constexpr int CUCKOO_STASH_SIZE = 101;
constexpr int CUCKOO_MAX_ITERATIONS = 32;
constexpr uint32_t CUCKOO_MIN_TABLE_SIZE = 2048u;  // compute_cuckoo.cpp:15

// fbm3 runs two octaves a step; the field kernel decides a point's sign after
// each step when the octaves left cannot change it (bounds for at most
// 2 kCaveSteps octaves)
constexpr int kCaveSteps = 16;


typedef lvn_density_params DensityParams;

// The simplex noise permutation lookups as two byte tables of 257 x 257
// texels: row r, column c holds texel (r & 255, c & 255), so a corner's +x, +y
// or +z neighbour needs no wrap.  The first table holds snoise3's first
// lookup's result (the alpha read as a column, 255 as 0).  The second, from
// byte kT3Second, holds a texel's gradient as a byte offset ((alpha & 15) * 8)
// into the gradient table as the kernels stage it in shared memory (the 16
// (x, y) pairs, then the 16 z components at the same 8-byte stride):
// snoise3's second lookup and snoise2's three corners read it.
constexpr int kT3Row = 257;
constexpr int kT3Second = 66064;  // 257 * 257 rounded up to 16 bytes
constexpr int kT3Bytes = 2 * kT3Second;

// A CSG operation as the kernels read it (48 B): the reference's
// CSGOperationInfo plus cos/sin of rotate_y evaluated once on the host.
struct Brush {
    float origin[3];
    int32_t type;
    float dimensions[3];
    int32_t brush;
    float cos_y, sin_y;
    int32_t material;
    int32_t pad;
};
static_assert(sizeof(Brush) == 48, "Brush layout");

// Per-chunk descriptor uploaded with each batch (host -> device).
struct ChunkDesc {
    int32_t off[3];      // density-space origin = min / LEAF_SIZE_SCALE
    int32_t scale;       // sampleScale
    int32_t min[3];      // world min
    int32_t size;        // world size
    float colour[3];     // ColourForMinLeafSize(size / 256)
    int32_t op_begin;    // into the batch brush array
    int32_t op_count;
    int32_t csg_lo[3];   // field-index box that holds every point the operations can change
    int32_t csg_hi[3];
    int32_t pad[3];
    uint32_t edge_params[CUCKOO_HASH_FN_COUNT * 2];
    uint32_t node_params[CUCKOO_HASH_FN_COUNT * 2];
};

// Per-chunk counters and offsets produced on the device.
struct ChunkState {
    int32_t plain_edges;     // plain edges kept (not touched by CSG)
    int32_t created_edges;   // CSG-created edges
    int32_t edge_off;        // first edge in the batch edge pool
    int32_t num_edges;
    int32_t nodes;           // active voxels
    int32_t node_off;
    int32_t quads;
    int32_t quad_off;
    int32_t seams;
    int32_t seam_off;
    uint32_t edge_prime;
    int32_t edge_table_off;  // slots; the stash follows the table
    uint32_t node_prime;
    int32_t node_table_off;
    int32_t edge_stash_used;
    int32_t node_stash_used;
    int32_t edge_insert_failed;
    int32_t node_insert_failed;
    int32_t kept_edges;      // edges kept from a cached field (cached-field CSG)
    int32_t edges_xz;        // new plain edges along x or z
    int32_t edges_y;         // new plain edges along y
    int32_t wl_xz_off;       // chunk's first entry in each hermite work-list segment
    int32_t wl_y_off;
    int32_t wl_c_off;
    uint32_t edge_magic;     // floor((2^32 - 1) / edge_prime), for the table modulo
    uint32_t node_magic;
    int32_t simp_verts;      // simplified mesh: vertices, first vertex, triangles, first triangle
    int32_t simp_vert_off;
    int32_t simp_tris;
    int32_t simp_tri_off;
    int32_t pad[2];
};
static_assert(sizeof(ChunkState) == 128, "ChunkState layout");

// Batch-wide totals and status (device).
struct BatchState {
    int32_t total_edges;
    int32_t total_nodes;
    int32_t total_quads;
    int32_t total_seams;
    int64_t total_edge_slots;
    int64_t total_node_slots;
    int32_t overflow;        // bitmask of pools that ran out of capacity
    int32_t status;          // device-side internal status (0 = ok)
    int32_t total_xz;        // hermite work-list segment sizes
    int32_t total_y;
    int32_t total_created;
    int32_t total_simp_verts;  // simplified mesh totals
    int32_t total_simp_tris;
    int32_t pad[1];
};

// Octree simplification: a node's QEF in its own frame (origin at the node's
// min corner, unit = one voxel).  ATA and ATb as in QEFData (qef.cl:7-14),
// plus btb = sum (n.p)^2, the point count, the mass-point sum and the normal sum.
struct SimpQef {
    float ata[6];
    float btb, w;
    float atb[3];
    float mp[3];
    float ns[3];
    float pad[3];
};
static_assert(sizeof(SimpQef) == 80, "SimpQef layout");

// One octree node above the leaves (level k >= 1) of the simplification.
struct SimpNode {
    int32_t chunk;
    int32_t pos;        // x | y << 8 | z << 16 in units of the node size
    int32_t collapsed;  // 1 when the node replaces its subtree
    int32_t anchor;     // first leaf voxel (chunk-local index) below the node
    float wpos[3];      // world position of the collapsed node's vertex
    int32_t material;
    SimpQef q;
};
static_assert(sizeof(SimpNode) == 112, "SimpNode layout");

enum OverflowBits : int32_t {
    OVF_EDGES = 1,
    OVF_NODES = 2,
    OVF_QUADS = 4,
    OVF_SEAMS = 8,
    OVF_EDGE_SLOTS = 16,
    OVF_NODE_SLOTS = 32,
};

}  // namespace lvn
