/*
 * lvn_oracle.h -- C ABI of the CPU oracle for the leven chunk-meshing path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * entry point and the bench's CPU-baseline leg load it.  The product library
 * (leven_gb300/csrc) never includes, links or calls anything in oracle/.
 *
 * The oracle is a plain, sequential C++17 restatement of the reference's
 * OpenCL kernels (the .cl files under leven/cl) and their host orchestration
 * (leven/src/compute*.cpp).  Every function in lvn_oracle.cpp cites the
 * reference file:line it follows.  Parity is pinned only where the reference
 * ships known answers (cuckoo fixtures, RemoveDuplicates, FindNextPrime);
 * field / edge / QEF / mesh results are the restatement's own and are pinned
 * by nothing in the reference ("parity unpinned" for those stages).
 */
#ifndef LVN_ORACLE_H
#define LVN_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* byte-identical to CSGOperationInfo (leven/src/compute.h:16-24), 48 B */
typedef struct orc_csg_op {
    int32_t type;        /* 0 = add (union), 1 = subtract */
    int32_t brush;       /* 0 = cuboid, 1 = sphere */
    int32_t material;
    float   rotate_y;
    float   origin[4];
    float   dimensions[4];
} orc_csg_op;

/* density selector; mode 0 = reference Terrain (noise.cl:205-268),
 * 1 = 2D fBm heightfield, 2 = 2D fBm heightfield + 3D fBm caves */
typedef struct orc_density {
    int32_t mode;
    int32_t octaves2;
    float   freq2, lacunarity2, gain2, amp2;
    int32_t octaves3;
    float   freq3, lacunarity3, gain3, amp3;
} orc_density;

typedef struct orc_chunk_args {
    int32_t min[3];          /* world units (1 voxel = 4 at LOD0) */
    int32_t size;            /* world units; sampleScale = size / (vpc*4) */
    int32_t voxels_per_chunk;/* power of two, 8..64 */
    int32_t default_material;
    int32_t crossing_mode;   /* 0 = 17-sample search (reference), 1 = linear */
    int32_t num_ops;
    const orc_csg_op* ops;   /* applied as ONE batch after the plain edges */
    uint32_t hash_seed;      /* seeds the hash-parameter generator */
} orc_chunk_args;

/* what orc_chunk_get / orc_chunk_count fetch */
enum {
    ORC_MATERIALS = 0,      /* int32[F]   final field materials             */
    ORC_EDGE_KEYS = 1,      /* int32[E]   field edge keys (final list order) */
    ORC_EDGE_INFO = 2,      /* float4[E]  (normal.xyz, t)                    */
    ORC_NODE_CODES = 3,     /* uint32[V]  leaf codes, linear voxel order     */
    ORC_NODE_EDGES = 4,     /* int32[V]   12-bit edge masks                  */
    ORC_NODE_MATERIALS = 5, /* int32[V]   material<<8 | corners              */
    ORC_VERTICES = 6,       /* MeshVertex[V]  (48 B)                         */
    ORC_TRIANGLES = 7,      /* int32[3 * 2T]                                 */
    ORC_SEAMS = 8,          /* SeamNodeInfo[S] (48 B)                        */
    ORC_PLAIN_EDGE_KEYS = 9,/* int32[E0]  edges before CSG                   */
    ORC_QEFS = 10,          /* QEFData[V] (64 B)                             */
    ORC_MESH_VERTEX_COUNT = 11, /* reported vertex count (0 when no tris)     */
    ORC_CREATED_EDGE_KEYS = 12, /* int32[]   CSG-created edge keys           */
    ORC_SIMP_VERTICES = 13, /* MeshVertex[]  simplified mesh (orc_chunk_simplify) */
    ORC_SIMP_TRIANGLES = 14,/* int32[3 * T'] simplified triangles            */
    ORC_SIMP_VERTEX_COUNT = 15, /* reported simplified vertex count          */
    ORC_SIMP_REPS = 16,     /* int32[V] representative anchor | level << 20  */
    ORC_POSITIONS_F64 = 17, /* double[4 * V] leaf vertex solved in FP64 (world units, count) */
    ORC_NUM_WHAT = 18
};

int   orc_set_seed(int32_t seed);
void  orc_perm_lut(uint8_t* out65536);
/* the RGBA8 permutation image (256 x 256 x 4 bytes, row-major): RGB the
 * gradient bytes, A the permutation value */
void  orc_perm_image_rgba(uint8_t* out);
float orc_density_at(const orc_density* d, float x, float y, float z);
float orc_snoise2(float x, float y);
float orc_snoise3(float x, float y, float z);
/* FP32 operation counts of the restated arithmetic (add, sub, mul, div,
 * sqrt, floor 1; fma 2; compares, min / max, abs free; every simplex corner
 * taken): out[0] the height term of a heightfield mode (0 for the reference
 * terrain), out[1] the rest of one density sample, out[2..4] the whole
 * FindEdgeIntersectionInfo of an x, y and z edge (17-sample search, 23
 * density samples, each with its own height term) */
int   orc_flop_counts(const orc_density* d, int64_t* out);
int   orc_find_next_prime(int32_t n);
/* qef_create_from_points + qef_solve (qef.cl:239-303) over `count` (<= 12)
 * points and normals (4 floats each); out[4] = the solved position */
float orc_qef_solve_points(const float* positions, const float* normals, int32_t count, float* out);

void* orc_chunk_new(void);
void  orc_chunk_free(void* h);
int   orc_chunk_run(void* h, const orc_density* d, const orc_chunk_args* a);
int   orc_chunk_count(void* h, int what);
int   orc_chunk_get(void* h, int what, void* out, int64_t cap_bytes);
/* bottom-up octree simplification of a chunk that orc_chunk_run meshed
 * (threshold = QEF error bound in voxel^2; not in the reference) */
int   orc_chunk_simplify(void* h, float threshold);

/* cuckoo restatement (cuckoo.cl + compute_cuckoo.cpp), sequential insert */
typedef struct orc_cuckoo orc_cuckoo;
orc_cuckoo* orc_cuckoo_build(const uint32_t* keys, int32_t n, uint32_t seed, int32_t* retries);
int      orc_cuckoo_find(const orc_cuckoo* c, uint32_t key, uint32_t* value);
int      orc_cuckoo_prime(const orc_cuckoo* c);
void     orc_cuckoo_free(orc_cuckoo* c);

/* RemoveDuplicates restatement (compute.cpp:450-543, duplicate.cl) */
int orc_remove_duplicates(const int32_t* in, int32_t n, int32_t* out);

/* CSG op AABB (clipmap.cpp:1638-1643) and overlap (aabb.h:26-35) */
void orc_csg_op_bounds(const orc_csg_op* op, int32_t out_min[3], int32_t out_max[3]);
int  orc_aabb_overlaps(const int32_t amin[3], const int32_t amax[3],
                       const int32_t bmin[3], const int32_t bmax[3]);

/* Clipmap chunk lists over a complete octree (root_min, root_size; every node
 * subdivided down to 256-unit leaves, ConstructChildren clipmap.cpp:715-735).
 * Nodes are written as (min x, y, z, size) int32 quadruples, at most cap of
 * them; the return value is the full count.
 * orc_clipmap_select: SelectActiveClipmapNodes (clipmap.cpp:1084-1128) for one
 * camera, in its recursion's pre-order.
 * orc_clipmap_nodes_in_aabb: FindNodesInsideAABB (clipmap.cpp:1571-1597) for
 * one box, in its recursion's post-order.
 * orc_clipmap_touched: the touch set of processCSGOperationsImpl
 * (clipmap.cpp:1661-1669), the union over the operations' bounds, each node
 * once, in the octree's post-order. */
int orc_clipmap_select(const float cam[3], const int32_t root_min[3], int32_t root_size, int32_t* out4, int32_t cap);
int orc_clipmap_nodes_in_aabb(const int32_t bmin[3], const int32_t bmax[3], const int32_t root_min[3],
                              int32_t root_size, int32_t* out4, int32_t cap);
int orc_clipmap_touched(const orc_csg_op* ops, int32_t n, const int32_t root_min[3], int32_t root_size,
                        int32_t* out4, int32_t cap);
/* CPU baseline: orc_clipmap_select for n cameras on `threads` host threads;
 * returns the total node count */
int64_t orc_clipmap_select_many(const float* cams, int32_t n, const int32_t root_min[3], int32_t root_size,
                                int32_t threads);

/* GenerateClipmapSeamMesh (clipmap.cpp:573-610) for each host: the active
 * clipmap nodes are chunks4 (min xyz, size), chunk c's seam nodes (SeamNodeInfo,
 * 12 words) seams[seam_offsets[c] .. seam_offsets[c + 1]); hosts index chunks.
 * Writes the hosts' meshes back to back (MeshVertex, 12 floats; triangles, 3
 * int32 host-local indices) and per host (vertices, triangles) into
 * host_counts; a host without triangles has no mesh (0, 0).  Returns 0, -2
 * when the capacities are too small (host_counts set), -1 on bad arguments. */
int orc_seam_generate(const int32_t* chunks4, const int32_t* seam_offsets, int32_t num_chunks, const int32_t* seams,
                      int32_t vpc, const int32_t root_min[3], int32_t root_size, const int32_t* hosts,
                      int32_t num_hosts, const float colour[3], float* vertices, int64_t vertex_cap,
                      int32_t* triangles, int64_t triangle_cap, int32_t* host_counts, int32_t threads);

/* ngMeshSimplifier (ng_mesh_simplify.cpp:441-540) on one mesh: vertices
 * (MeshVertex, 12 floats) and triangles (3 int32), worldSpaceOffset (4 floats),
 * options = MeshSimplificationOptions {edgeFraction, maxIterations,
 * targetPercentage, maxError, maxEdgeSize, minAngleCosine} as 6 floats.  The
 * outputs hold at most nv vertices and nt triangles. */
int orc_mesh_collapse(const float* vertices, int32_t nv, const int32_t* triangles, int32_t nt, const float offset[4],
                      const float options[6], float* out_vertices, int32_t* out_nv, int32_t* out_triangles,
                      int32_t* out_nt);
/* n draws of std::uniform_int_distribution<int>(0, hi) from std::mt19937
 * seeded 42, as FindValidCollapses makes them */
int orc_uniform_draws(int32_t hi, int32_t n, int32_t* out);
/* CPU baseline: orc_mesh_collapse over n meshes on `threads` host threads;
 * ranges = 4 per mesh (vertex offset, vertices, triangle offset, triangles),
 * offsets 4 and options 6 floats per mesh; returns the total triangles left */
int64_t orc_mesh_collapse_many(const float* vertices, const int32_t* triangles, const int32_t* ranges, int32_t n,
                               const float* offsets, const float* options, int32_t threads);

/* CPU baseline: mesh n chunks (each a fresh field with its ops) on `threads`
 * host threads; returns total vertices + triangles for sanity */
int64_t orc_mesh_chunks(const orc_density* d, const orc_chunk_args* chunks, int32_t n,
                        int32_t threads);
/* the same followed by orc_chunk_simplify(threshold) of each chunk (threshold < 0: none) */
int64_t orc_mesh_chunks_simplified(const orc_density* d, const orc_chunk_args* chunks, int32_t n,
                                   int32_t threads, float threshold);

#ifdef __cplusplus
}
#endif
#endif
