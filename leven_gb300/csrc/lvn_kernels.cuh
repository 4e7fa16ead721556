// lvn_kernels.cuh -- device pointers of one batch and the launcher interface
// of the chunk-meshing kernels (implemented in lvn_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "lvn_types.h"

namespace lvn {

// Every device buffer a batch touches.  Pools are chunk-major: chunk c's
// edges, nodes, quads and seams are contiguous and in the reference's
// compaction order, at offsets recorded in ChunkState.
struct BatchPtrs {
    int n;                       // chunks in the batch
    int vpc;                     // voxels per chunk
    int crossing_mode;           // 0 = 17-sample search, 1 = linear
    int plain_class;             // 1: plain field edges are generated (fresh fields)
    int derive_mats;             // 1: fresh fields: byte materials exist only inside a chunk's CSG box,
                                 //    elsewhere they are the default material or AIR by the solid bits
    int need_mats;               // 1: the field kernel writes every byte material (cached fields)
    int num_sms;
    int hash_fault;              // 1: a table repair draws degenerate parameters too (host fault injection)
    int hermite_form;            // LVN_OPT_HERMITE_FORM: 0 by batch size, 1 shared-memory tables, 2 global
    DensityParams density;
    float cave_band;             // |y - amp2 h| above this: the cave term cannot change the density's sign
    float cave_rem[kCaveSteps + 1];  // cave_rem[s]: bound on |amp3 * octaves 2s.. of fbm3| (0 past the last)
    float4* host_vertices;       // non-null: k_leaf also writes each vertex to this pinned host array
    int64_t host_vertex_cap;     //   (16-byte aligned), of this many vertices
    int4* host_seams;            // non-null: the seam pass of k_mesh_scatter also writes this pinned array
    int64_t host_seam_cap;       //   (16-byte aligned), of this many seam nodes
    int32_t default_material;
    int32_t dom_by_solid[9];     // dominant material of 8 corners, n of them the default material, the rest AIR

    const ChunkDesc* desc;       // [n]
    ChunkState* cs;              // [n]
    BatchState* bs;              // [1]
    const Brush* brushes;        // per-chunk op lists, flattened

    const uint8_t* perm;         // 65536 B permutation image (alpha channel)
    const uint8_t* perm_t3;      // the two simplex lookup tables, kT3Row x kT3Row texels each (lvn_types.h)
    const float* grad;           // 16 x 4 gradient table

    uint8_t* mats;               // [n][F] field materials, index x + FD*y + FD*FD*z
    uint4* planes;               // [n][3][FD*FD] bit rows: plain solid, final air, changed
    int4* edge_tiles;            // [n][NBE] (plain x/z, plain y, created) counts, then in-chunk offsets
    int* vox_tiles;              // [n][NBV]

    int32_t* edge_keys;          // [ecap]
    int32_t* edge_chunk;         // [ecap]
    float4* edge_info;           // [ecap]
    int32_t* edge_work;          // [ecap] hermite work list: plain x/z, plain y, created segments
    int64_t ecap;

    uint32_t* node_codes;        // [vcap]
    int32_t* node_info;          // [vcap] edges << 16 | material << 8 | corners
    int32_t* node_chunk;         // [vcap]
    int64_t vcap;

    unsigned long long* edge_slots;  // [edge_slot_cap]
    int64_t edge_slot_cap;
    unsigned long long* node_slots;  // [node_slot_cap]
    int64_t node_slot_cap;

    int4* quad_scratch;          // [3 * vcap] (n1, n2, n3, flags) per (node, axis)
    int2* node_tile_counts;      // [node tile cap] (quads, seams) per node tile, then offsets
    int* chunk_tile_off;         // [n + 1] first node tile of each chunk
    int64_t node_tile_cap;

    lvn_mesh_vertex* vertices;   // [vertex_cap]
    int64_t vertex_cap;
    lvn_mesh_triangle* triangles;// [triangle_cap]
    int64_t triangle_cap;
    lvn_seam_node* seams;        // [seam_cap]
    int64_t seam_cap;

    // bottom-up octree simplification (simp_on = 1): the leaves are written to
    // leaf_out, the simplified mesh to vertices / triangles
    int simp_on;
    float simp_threshold;        // collapse when the QEF error (voxel^2) is at most this
    lvn_mesh_vertex* leaf_out;   // [vcap]
    SimpQef* leaf_qef;           // [vcap]
    int* simp_grid;              // [n][simp_grid_cells(vpc)] node entry per level cell, -1 = none
    SimpNode* simp_nodes;        // level k's entries start at simp_level_off[k]
    int64_t simp_level_off[8];
    int* simp_count;             // [8] entries per level
    int* simp_rep;               // [vcap] representative: anchor | level << 20
    int* simp_entry;             // [vcap] the representative's node (-1 = the leaf itself)
    int* simp_newidx;            // [vcap] output vertex of an anchor leaf
    uint8_t* simp_mask;          // [vcap] kept triangles, bit 2 * axis + t
    int2* simp_tile_counts;      // [node tile cap] (vertices, triangles) per node tile, then offsets

    // learned-surrogate meshing (s_on = 1): chunks with sslot[c] >= 0 take their
    // field from sdens[sslot[c]][F] instead of the plain density
    int s_on;
    const float* sdens;
    const int* sslot;            // [n]
    float4* probe_pts;           // [n][512] probe positions
    float* probe_plain;          // [n][512] plain density at the probes
    const float* probe_s;        // [n][512] surrogate density at the probes
    int* gate_ok;                // [n] 1 when every probe is within `gate`
    float gate;

    // the height term of a heightfield density per field column (x + FD z) of
    // each chunk, written by the field kernels; null: hermite evaluates it
    float* hmap;                 // [n][FD * FD]

    // k_mesh_scatter writes triangles (scatter_what 1), seams (2) or both (0);
    // k_leaf and the vertex export take slice `slice` of `nslices` equal leaf
    // ranges (nslices <= 1: all of them)
    int scatter_what;
    int slice, nslices;

    // launch shapes chosen by the autotuner: CTAs per SM of each stage's
    // persistent grid (0 = the built-in default)
    int grid_per_sm[24];

    // cached-field CSG: the field's current edge list (chunk 0 only)
    const int32_t* prev_keys;
    const float4* prev_info;
    int prev_count;
};

constexpr int kRowTile = 256;       // field / voxel rows per CTA in the dense stages
constexpr int kTilePoints = 2048;
constexpr int kNodeTile = 256;      // sparse node tile per CTA iteration

inline int field_dim(int vpc) { return vpc + 2; }
inline int field_size(int vpc) { return (vpc + 2) * (vpc + 2) * (vpc + 2); }
inline int field_rows(int vpc) { return (vpc + 2) * (vpc + 2); }
inline int edge_tiles_per_chunk(int vpc) { return (field_rows(vpc) + kRowTile - 1) / kRowTile; }
inline int vox_tiles_per_chunk(int vpc) { return (vpc * vpc + kRowTile - 1) / kRowTile; }
inline int octree_depth(int vpc) { return vpc == 8 ? 3 : vpc == 16 ? 4 : vpc == 32 ? 5 : 6; }
// cells of the level grids 1..depth of one chunk: sum (vpc >> k)^3
inline int64_t simp_grid_cells(int vpc) {
    int64_t s = 0;
    for (int k = 1; k <= octree_depth(vpc); k++) s += (int64_t)(vpc >> k) * (vpc >> k) * (vpc >> k);
    return s;
}

// Stage identifiers for profiling (order of execution).
enum Stage {
    ST_FIELD = 0,
    ST_CSG,
    ST_EDGE_COUNT,
    ST_EDGE_PLAN,
    ST_EDGE_SCATTER,
    ST_HERMITE,
    ST_VOX_COUNT,
    ST_VOX_PLAN,
    ST_VOX_SCATTER,
    ST_PRIMES,
    ST_HASH_FILL,
    ST_EDGE_INSERT,
    ST_LEAF,
    ST_NODE_INSERT,
    ST_MESH_COUNT,
    ST_MESH_PLAN,
    ST_MESH_SCATTER,
    ST_SIMPLIFY,
    ST_COUNT
};
static_assert(ST_COUNT <= 24, "BatchPtrs::grid_per_sm holds one entry per stage");
// the stages whose kernels run on a persistent grid, tunable by CTAs per SM
inline bool stage_has_persistent_grid(int st) {
    return st == ST_HERMITE || st == ST_HASH_FILL || st == ST_EDGE_INSERT || st == ST_LEAF || st == ST_NODE_INSERT ||
           st == ST_MESH_COUNT || st == ST_MESH_SCATTER || st == ST_SIMPLIFY;
}
const char* stage_name(int s);

// Launchers: each enqueues one kernel of the pipeline on `stream`.
cudaError_t launch_reset(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_field(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_csg(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_prune_edges(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_edge_count(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_edge_plan(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_edge_scatter(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_hermite(const BatchPtrs& b, cudaStream_t stream);
cudaError_t set_kernel_attributes();  // once per device, at initialisation
cudaError_t launch_vox_count(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_vox_plan(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_vox_scatter(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_primes(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_hash_fill(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_edge_insert(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_leaf(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_node_insert(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_mesh_count(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_mesh_plan(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_mesh_scatter(const BatchPtrs& b, cudaStream_t stream);
// surrogate probes: 512 field points per chunk with their plain density, and
// the gate that compares them with the surrogate's
constexpr int kProbes = 512;
cudaError_t launch_probe(const BatchPtrs& b, cudaStream_t stream);
cudaError_t launch_gate(const BatchPtrs& b, cudaStream_t stream);
// copy one output pool (which: 0 vertices, 1 triangles, 2 seams) to the
// caller's array; dst must be device-addressable (device or pinned host memory)
cudaError_t launch_export(const BatchPtrs& b, int which, void* dst, int64_t capacity, cudaStream_t stream);
// the whole simplification pass (level grids reset, levels, map, plan, scatter)
cudaError_t launch_simplify(const BatchPtrs& b, cudaStream_t stream);

// Measurement pass over the last batch's leaves: the FP32 solve k_leaf runs
// against an FP64 solve of the same crossings.  stats (zeroed by the caller):
// [0] max distance in voxels (double bits), [1] sum (double), [2] leaves,
// [3] leaves farther than 1e-3 voxel.
cudaError_t launch_leaf_qef_check(const BatchPtrs& b, unsigned long long* stats, cudaStream_t stream);

// Test hook: the meshing stages' cuckoo insert and find over an arbitrary key
// list.  table holds prime + CUCKOO_STASH_SIZE slots; status[0] = a key went
// to the stash, status[1] = an insert failed.  reference_find probes the main
// table at the stash index instead of the stash, as Cuckoo_Find does
// (cuckoo.cl:93-101).
struct CuckooParams {
    uint32_t p[CUCKOO_HASH_FN_COUNT * 2];
};
cudaError_t launch_debug_cuckoo(const uint32_t* keys, int n, unsigned long long* table, uint32_t prime,
                                CuckooParams params, int* status, int reference_find, uint32_t* values,
                                cudaStream_t stream);

}  // namespace lvn
