/*
 * lvn.h -- C ABI of the GB300-native chunk-meshing library (liblvn.so).
 *
 * Drop-in replacement for the OpenCL compute layer of the leven voxel engine
 * (leven/src/compute.h:35-77).  Every entry point below names the reference
 * interface it replaces.  Conventions carried over from the reference:
 *   - int return: 0 on success, a negative code on failure (compute.h:12);
 *   - chunk `min` and `size` are world units, 1 voxel = 4 world units at
 *     LOD0; the density-space offset is min / 4 and sampleScale is
 *     size / (voxels_per_chunk * 4) (compute.cpp:569-577);
 *   - not thread-safe: global state (noise seed, stored CSG operations) is
 *     shared, and one mesh-generation context is driven from one thread
 *     (compute.cpp:168-191).
 * Struct layouts are byte-identical to the reference's CSGOperationInfo,
 * MeshVertex, MeshTriangle and SeamNodeInfo.
 *
 * No torch or CUDA types appear in the signatures; a CUDA stream is passed as
 * an opaque pointer.
 */
#ifndef LVN_H
#define LVN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes (negative, like the reference's CL codes) ------------- */
#define LVN_OK                  0
#define LVN_ERR_NO_DEVICE      (-1)     /* CL_DEVICE_NOT_FOUND analogue          */
#define LVN_ERR_OUT_OF_MEMORY  (-5)     /* CL_OUT_OF_RESOURCES analogue          */
#define LVN_ERR_INVALID        (-30)    /* CL_INVALID_VALUE analogue             */
#define LVN_ERR_CAPACITY       (-100)   /* caller buffer too small; counts set   */
#define LVN_ERR_NOT_INITIALISED (-101)
#define LVN_ERR_HASH           (-102)   /* cuckoo insert failed after retries    */
#define LVN_ERR_DEVICE_STATUS  (-103)   /* a kernel reported an internal limit   */
#define LVN_ERR_CUDA           (-99999) /* LVN_CL_ERROR (compute.h:12) analogue  */

/* ---- density selector (new; the reference hard-codes Terrain) ---------- */
#define LVN_DENSITY_REFERENCE 0   /* Terrain: ridged x billow + fBm (noise.cl:205-268) */
#define LVN_DENSITY_FBM2D     1   /* y - amp2 * fBm2D(xz)                              */
#define LVN_DENSITY_CAVES     2   /* y - amp2 * fBm2D(xz) + amp3 * fBm3D(xyz)           */

#define LVN_MEMORY_HOST   0
#define LVN_MEMORY_DEVICE 1

/* mesh-generation options (lvn_meshgen_set_option) */
#define LVN_OPT_CROSSING_MODE 1   /* 0 = 17-sample search (reference), 1 = linear     */
#define LVN_OPT_CACHE         2   /* 1 = keep density-field / octree caches (default) */
#define LVN_OPT_PROFILE       3   /* 1 = record per-stage CUDA events                 */
#define LVN_OPT_GRAPHS        4   /* 1 = run batches as one captured CUDA graph (default) */
#define LVN_OPT_HOST_WRITES   5   /* pinned host outputs: 1 = written by the kernels over the
                                     host link as they are made (default); 0 = meshed into
                                     device pools, then moved by the copy engine, which leaves
                                     the SMs to another context's batch in flight */
#define LVN_OPT_COMPUTE_ORDER 6   /* 1 = the context's batches join a device-wide order: a
                                      batch's kernels start after the kernels of the previous
                                      ordered batch (any context) have ended; its copy-engine
                                      transfers stay outside the order, so they overlap the next
                                      batch's kernels (default 0) */
#define LVN_OPT_HERMITE_FORM  7   /* new: the hermite kernel's form.  0 = by batch size (default):
                                      batches of 256 chunks and more with the caves density, of
                                      2048 and more with the others, stage the noise lookup tables
                                      in shared memory (one 1024-thread CTA per SM), smaller ones
                                      read them from global memory; 1 = shared-memory tables
                                      for every batch; 2 = global tables for every batch.  The
                                      results are the same bits in every form */

/* CSGOperationInfo (leven/src/compute.h:16-24; apply_csg_operation.cl:5-14), 48 B */
typedef struct lvn_csg_op {
    int32_t type;          /* 0 = add (union), 1 = subtract           */
    int32_t brush_shape;   /* RenderShape: 0 = cube, 1 = sphere       */
    int32_t material;      /* 0..255                                  */
    float   rotate_y;      /* radians, cube brushes                   */
    float   origin[4];     /* density units                           */
    float   dimensions[4]; /* half extents (cube) / radius in [0]     */
} lvn_csg_op;

/* MeshVertex (leven/src/render_types.h:24-38), 48 B */
typedef struct lvn_mesh_vertex {
    float position[4];
    float normal[4];
    float colour[4];       /* rgb = LOD colour, a = dominant material */
} lvn_mesh_vertex;

/* MeshTriangle (leven/src/render_types.h:42-58), 12 B, chunk-local indices */
typedef struct lvn_mesh_triangle {
    int32_t indices[3];
} lvn_mesh_triangle;

/* SeamNodeInfo (leven/src/compute.h:26-31), 48 B */
typedef struct lvn_seam_node {
    int32_t localspace_min[4]; /* voxel xyz, w = material << 8 | corners */
    float   position[4];
    float   normal[4];
} lvn_seam_node;

/* density parameters (new) */
typedef struct lvn_density_params {
    int32_t mode;          /* LVN_DENSITY_*                             */
    int32_t octaves2;      /* 2D fBm: octaves, base frequency (1/voxel), */
    float   freq2;         /*   lacunarity, gain, amplitude (voxels)     */
    float   lacunarity2;
    float   gain2;
    float   amp2;
    int32_t octaves3;      /* 3D cave fBm, same parameters               */
    float   freq3;
    float   lacunarity3;
    float   gain3;
    float   amp3;
} lvn_density_params;

/* Output of one generateChunkMesh call.  The caller owns the arrays (host or
 * device memory per `memory`) and sets the capacities; the callee fills the
 * counts.  When an array is too small nothing is written to it,
 * LVN_ERR_CAPACITY is returned and the counts give the required sizes.  The
 * reference's fixed MeshBuffer arrays (render_types.h:62-90) become these
 * caller-sized arrays; the 14,336-vertex cap is lifted. */
typedef struct lvn_mesh_out {
    int32_t            memory;
    lvn_mesh_vertex*   vertices;
    int32_t            vertex_capacity;
    int32_t            num_vertices;
    lvn_mesh_triangle* triangles;
    int32_t            triangle_capacity;
    int32_t            num_triangles;
    lvn_seam_node*     seams;
    int32_t            seam_capacity;
    int32_t            num_seams;
} lvn_mesh_out;

/* one chunk of a batch: world-space min and size (as generateChunkMesh) */
typedef struct lvn_chunk_desc {
    int32_t min[3];
    int32_t size;
} lvn_chunk_desc;

/* per-chunk result of a batch; offsets index the batch arrays */
typedef struct lvn_chunk_result {
    int32_t vertex_offset;
    int32_t num_vertices;     /* 0 when the chunk has no triangles (compute_octree.cpp:227-232) */
    int32_t triangle_offset;
    int32_t num_triangles;
    int32_t seam_offset;
    int32_t num_seams;
    int32_t num_edges;        /* active field edges after CSG */
    int32_t num_nodes;        /* active voxels (leaf nodes)   */
} lvn_chunk_result;

typedef struct lvn_batch_out {
    int32_t            memory;          /* LVN_MEMORY_HOST / LVN_MEMORY_DEVICE */
    lvn_mesh_vertex*   vertices;
    int64_t            vertex_capacity;
    int64_t            total_vertices;  /* vertex slots used (all leaves)      */
    lvn_mesh_triangle* triangles;
    int64_t            triangle_capacity;
    int64_t            total_triangles;
    lvn_seam_node*     seams;
    int64_t            seam_capacity;
    int64_t            total_seams;
    lvn_chunk_result*  chunks;          /* host array, one entry per chunk     */
} lvn_batch_out;

typedef struct lvn_meshgen lvn_meshgen;

/* ---- global compute state --------------------------------------------- */

/* Compute_Initialise (compute.h:35; compute.cpp:195-232): selects device 0,
 * builds the noise permutation image for `noise_seed`. */
int lvn_initialise(int32_t noise_seed, uint32_t default_material, int32_t num_csg_brushes);
/* Compute_Shutdown (compute.h:36; compute.cpp:236-239) */
int lvn_shutdown(void);
/* Compute_SetNoiseSeed (compute.h:38; compute_density_field.cpp:129-134) */
int lvn_set_noise_seed(int32_t noise_seed);
/* Compute_StoreCSGOperation (compute.h:39; compute_density_field.cpp:312-317);
 * aabb_min/aabb_max are the AABB fields of the reference's AABB (aabb.h:168-259) */
int lvn_store_csg_operation(const lvn_csg_op* op, const int32_t aabb_min[3], const int32_t aabb_max[3]);
/* Compute_ClearCSGOperations (compute.h:40; compute_density_field.cpp:321-326) */
int lvn_clear_csg_operations(void);
/* CalcCSGOperationBounds (clipmap.cpp:1638-1643): the AABB the engine stores
 * with an operation */
int lvn_csg_operation_bounds(const lvn_csg_op* op, int32_t aabb_min[3], int32_t aabb_max[3]);
/* new: density function selector (the reference's DensityFunc, noise.cl:225-268,
 * is mode LVN_DENSITY_REFERENCE) */
int lvn_set_density(const lvn_density_params* params);
/* GetCLErrorString (compute.h:81) */
const char* lvn_error_string(int32_t code);

/* ---- mesh-generation context (class Compute_MeshGenContext, compute.h:46-77) */

/* Compute_MeshGenContext::create (compute.h:50; compute.cpp:605-610,
 * 245-312); NULL on failure.  voxels_per_chunk: 8, 16, 32 or 64. */
lvn_meshgen* lvn_meshgen_create(int32_t voxels_per_chunk);
void         lvn_meshgen_destroy(lvn_meshgen* ctx);
/* Compute_MeshGenContext::voxelsPerChunk (compute.h:52; compute.cpp:612-615) */
int lvn_meshgen_voxels_per_chunk(const lvn_meshgen* ctx);
/* Compute_MeshGenContext::applyCSGOperations (compute.h:54-57; compute_csg.cpp:224-242) */
int lvn_meshgen_apply_csg_operations(lvn_meshgen* ctx, const lvn_csg_op* ops, int32_t num_ops,
                                     const int32_t min[3], int32_t size);
/* Compute_MeshGenContext::freeChunkOctree (compute.h:59-61; compute_octree.cpp:379-387) */
int lvn_meshgen_free_chunk_octree(lvn_meshgen* ctx, const int32_t min[3], int32_t size);
/* Compute_MeshGenContext::isChunkEmpty (compute.h:63-66; compute_density_field.cpp:278-299).
 * *is_empty = 1 when the chunk's field has no active edge (the reference
 * returns the inverse, numEdges > 0; that call site is unreachable). */
int lvn_meshgen_is_chunk_empty(lvn_meshgen* ctx, const int32_t min[3], int32_t size, int32_t* is_empty);
/* Compute_MeshGenContext::generateChunkMesh (compute.h:68-72; compute_octree.cpp:351-375) */
int lvn_meshgen_generate_chunk_mesh(lvn_meshgen* ctx, const int32_t min[3], int32_t size, lvn_mesh_out* out);

/* new: mesh `num_chunks` chunks in one batched pass on the GPU.  Each chunk is
 * generated exactly as generateChunkMesh would on a cold cache (fresh field,
 * stored CSG operations whose AABB overlaps the chunk replayed in store
 * order); the caches are neither read nor written. */
int lvn_meshgen_generate_chunks(lvn_meshgen* ctx, const lvn_chunk_desc* chunks, int32_t num_chunks,
                                lvn_batch_out* out);

/* New: lvn_meshgen_generate_chunks without waiting.  The call copies `chunks`
 * and returns once the batch is handed to a host thread of the context's own,
 * which runs the synchronous call; lvn_meshgen_wait(ctx) joins it and returns
 * its result code, after which `out` holds the totals and per-chunk results.
 * `out` and the arrays it points to must stay valid and untouched until then.
 * One batch is in flight per context (a second call before the wait returns
 * LVN_ERR_INVALID); two contexts, each with its own stream, keep two batches
 * in flight, so that one batch's transfer to host arrays overlaps the next
 * one's kernels.  A context must not be used by other calls between the two.
 * lvn_meshgen_wait returns LVN_OK when nothing is in flight; destroying a
 * context waits for its batch. */
int lvn_meshgen_generate_chunks_async(lvn_meshgen* ctx, const lvn_chunk_desc* chunks, int32_t n, lvn_batch_out* out);
int lvn_meshgen_wait(lvn_meshgen* ctx);

/* new: execution control */
int   lvn_meshgen_set_stream(lvn_meshgen* ctx, void* cuda_stream);
void* lvn_meshgen_get_stream(lvn_meshgen* ctx);
int   lvn_meshgen_set_option(lvn_meshgen* ctx, int32_t option, int32_t value);
/* per-stage device times (ms) accumulated while LVN_OPT_PROFILE is on;
 * returns the number of stages, names via lvn_meshgen_stage_name */
int         lvn_meshgen_stage_times(lvn_meshgen* ctx, float* ms, int32_t* launches, int32_t capacity);
const char* lvn_meshgen_stage_name(int32_t stage);
int         lvn_meshgen_reset_stage_times(lvn_meshgen* ctx);

/* new (not in the reference): bottom-up octree simplification of every mesh
 * this context makes from now on.  Classic dual contouring collapse (Ju et al.
 * 2002): an octree node replaces its subtree when all of its children did
 * (leaves count, voxels on the chunk's faces never collapse, so seams are
 * unchanged) and the QEF error of its summed crossings, solved with the
 * reference's qef_solve (qef.cl:239-256), is at most `threshold` (voxel^2,
 * the chunk's own voxel as unit).  The mesh is re-expressed over the collapsed
 * nodes; lvn_chunk_result and the totals then describe the simplified mesh.
 * threshold < 0 turns it off (the default). */
int lvn_meshgen_set_simplify(lvn_meshgen* ctx, float threshold);

/* new: launch-shape autotuner.  Runs the batch `chunks` (as
 * lvn_meshgen_generate_chunks would, outputs discarded) with each stage's
 * persistent grid at 2, 4, 8, 16 and 32 CTAs per SM, and keeps the fastest
 * shape of every stage for later batches with the same density mode,
 * crossing mode, simplification setting and power-of-two batch size, on
 * every context of the process (tune once, then keep batches in flight on
 * several contexts that all run the tuned shapes).  The
 * hermite stage, which a batch runs beside the voxel / hash / quad stages, is
 * then tuned again by the time of the whole batch.  The chosen CTAs per SM,
 * indexed by stage (0 = built-in default), go to
 * grid_per_sm[0 .. lvn_meshgen_stage_times' count) when it is not NULL. */
int lvn_meshgen_autotune(lvn_meshgen* ctx, const lvn_chunk_desc* chunks, int32_t num_chunks, int32_t* grid_per_sm);

/* new: intermediate buffers of chunk `chunk` of the last batch, for
 * stage-level parity checks (what = LVN_DEBUG_*).  Returns the element count,
 * or LVN_ERR_CAPACITY when cap_bytes is too small. */
#define LVN_DEBUG_MATERIALS    0  /* uint8[F]   final field materials           */
#define LVN_DEBUG_EDGE_KEYS    1  /* int32[E]   edge keys, final list order     */
#define LVN_DEBUG_EDGE_INFO    2  /* float4[E]  (normal.xyz, t)                 */
#define LVN_DEBUG_NODE_CODES   3  /* uint32[V]                                  */
#define LVN_DEBUG_NODE_INFO    4  /* int32[V]   edges << 16 | material << 8 | corners */
#define LVN_DEBUG_EDGE_TABLE   5  /* uint64[prime] edge cuckoo table            */
#define LVN_DEBUG_EDGE_STASH   6  /* uint64[101]                                */
#define LVN_DEBUG_NODE_TABLE   7  /* uint64[prime] node cuckoo table            */
#define LVN_DEBUG_NODE_STASH   8  /* uint64[101]                                */
#define LVN_DEBUG_PLAIN_EDGES  9  /* int32       number of plain (non-CSG) edges */
#define LVN_DEBUG_SIMP_REPS   10  /* int32[V]   simplification: representative of each leaf,
                                     first leaf below it | octree level << 20   */
int64_t lvn_meshgen_debug_fetch(lvn_meshgen* ctx, int32_t what, int32_t chunk, void* host, int64_t cap_bytes);

/* New: the error of the FP32 leaf solve (qef_solve, qef.cl:239-256) against
 * an FP64 solve of the same crossings and normals, over every leaf of the
 * context's last fresh batch (not simplified leaves' parents): out[0] max and
 * out[1] mean distance in voxels of the leaf's chunk, out[2] leaves, out[3]
 * leaves farther than 1e-3 voxel.  A measurement pass on the GPU;
 * LVN_ERR_INVALID before any fresh batch. */
int lvn_meshgen_qef_fp64_error(lvn_meshgen* ctx, double out[4]);

/* Test hook (new).  The device cuckoo table the meshing stages build, over an
 * arbitrary list of n distinct keys with value = key index: Cuckoo_InsertKeys
 * (cuckoo.cl:26-71) under Cuckoo_InsertKeys' host retry loop
 * (compute_cuckoo.cpp:76-139, here bounded to 16 parameter draws), then
 * Cuckoo_Find (cuckoo.cl:73-104) of every key into values[n] (~0 = not found).
 * prime 0 sizes the table as Cuckoo_InitialiseTable does
 * (compute_cuckoo.cpp:49-73: FindNextPrime(max(2048, 2n))); another value
 * forces that table size, so that a small one sends keys to the 101-entry
 * stash.  flags LVN_CUCKOO_REFERENCE_FIND looks keys up as the reference's
 * Cuckoo_Find is written, whose stash probe reads data[h] instead of
 * stash[h] (cuckoo.cl:93-101), so stashed keys are not found.  table_out
 * (optional, prime + 101 entries) receives the table then the stash.  info:
 * prime, stash used, parameter draws, insert failed.  Returns LVN_ERR_HASH
 * when every draw failed. */
#define LVN_CUCKOO_REFERENCE_FIND 1
int lvn_debug_cuckoo(const uint32_t* keys, int32_t n, uint32_t prime, int32_t flags, uint32_t* values,
                     uint64_t* table_out, int64_t table_capacity, int32_t info[4]);

/* Test hook (new): host-side fault injection, for the failure paths of the
 * meshing calls.  LVN_FAULT_DEVICE_ALLOC makes the next `count` device
 * allocations fail as cudaMalloc's out-of-memory does (the call returns
 * LVN_ERR_OUT_OF_MEMORY); LVN_FAULT_HASH_FAMILY makes the next `count` cuckoo
 * parameter draws a degenerate family under which no table holds three keys,
 * and the batch's device-side table repair degenerate as well (the call
 * returns LVN_ERR_HASH after its bounded retries, where the reference's loop
 * at compute_cuckoo.cpp:86-132 retries without bound);
 * LVN_FAULT_HASH_FAMILY_HOST makes the next `count` host draws degenerate
 * but leaves the device-side repair its own parameters, so that a batch
 * meshes only through that repair; LVN_FAULT_NONE clears them all.  No GPU
 * fault is involved. */
#define LVN_FAULT_NONE              0
#define LVN_FAULT_DEVICE_ALLOC      1
#define LVN_FAULT_HASH_FAMILY       2
#define LVN_FAULT_HASH_FAMILY_HOST  3
int lvn_debug_inject_fault(int32_t what, int32_t count);

/* No counterpart in the reference.  Meshes one chunk exactly as
 * lvn_meshgen_generate_chunk_mesh does with caching off, but allocates no
 * memory: for engine threads that cannot call cudaMalloc / cudaFree (a
 * frame-locked render or streaming thread, where cudaFree would synchronise
 * the device; engines that reserve all GPU memory at start-up).  The caller
 * passes the chunk and its output arrays (host or device per out->memory);
 * the stored CSG operations and the noise seed come from the global state as
 * usual.  All intermediate buffers live in one static device array of
 * LVN_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until
 * exit; the first call looks up that array's device address
 * (cudaGetSymbolAddress).  The call runs on the device lvn_init ran on and
 * returns LVN_ERR_INVALID when another device is current.  It reads its
 * counters back and synchronises cuda_stream before returning.  Chunks beyond
 * the LVN_NOALLOC_MAX_* limits are rejected with LVN_ERR_CAPACITY.  Calls
 * share the array, from every host thread: two calls in flight on the GPU at
 * the same time (different streams or threads) race; serialise them.
 * cuda_stream may be NULL (the legacy default stream). */
#define LVN_NOALLOC_SCRATCH_BYTES        (12 * 1024 * 1024)
#define LVN_NOALLOC_MAX_VOXELS_PER_CHUNK 64
#define LVN_NOALLOC_MAX_EDGES            65536   /* active field edges after CSG */
#define LVN_NOALLOC_MAX_NODES            32768   /* leaves (active voxels)       */
#define LVN_NOALLOC_MAX_CSG_OPS          64      /* stored operations per chunk  */
int lvn_generate_chunk_mesh_noalloc(const int32_t min[3], int32_t size, int32_t voxels_per_chunk, lvn_mesh_out* out,
                                    void* cuda_stream);

/* ---- learned density surrogate (new; not in the reference) ------------
 * An MLP from a density-space position to the density: 16 frequencies per
 * axis of sin / cos Fourier features over the domain (96 inputs), 4 hidden
 * layers of 128 with SiLU, a linear output; 62,081 parameters.  BF16 weights
 * and activations with FP32 accumulation on the tensor cores (tcgen05), FP32
 * master weights and Adam (beta 0.9 / 0.999, eps 1e-8).  All functions return
 * LVN_OK or a negative error code unless noted. */
typedef struct lvn_surrogate lvn_surrogate;

/* a surrogate over [domain_min, domain_max] (density units), weights drawn
 * as PyTorch's Linear does from `seed`; NULL on failure */
lvn_surrogate* lvn_surrogate_create(const float domain_min[3], const float domain_max[3], uint64_t seed);
void    lvn_surrogate_destroy(lvn_surrogate* s);
int32_t lvn_surrogate_num_params(void);
/* parameters as one float array: W0[128][96] b0[128] W1[128][128] b1 W2 b2 W3 b3 w4[128] b4 */
int     lvn_surrogate_set_params(lvn_surrogate* s, const float* params, int64_t n);
int     lvn_surrogate_get_params(lvn_surrogate* s, float* params, int64_t capacity);
/* generate the training pool: n samples (x, y, z, plain density) of the
 * density set by lvn_set_density, 70% within 4 voxels of the zero set (the
 * heightfield surface, or with caves up to eight tries within the cave band
 * of it for |density| <= 4) and 30% uniform in the domain; copied to
 * host_out when not NULL */
int     lvn_surrogate_sample(lvn_surrogate* s, int64_t n, uint64_t seed, float* host_out);
/* `steps` Adam steps on consecutive batches of the pool; losses[steps] (MSE
 * of density / 8) when not NULL.  batch is a multiple of 128. */
int     lvn_surrogate_train(lvn_surrogate* s, int32_t steps, int32_t batch, float lr, float* losses);
/* one forward + backward on n host samples (x, y, z, target), n a multiple of
 * 128: the gradient of the loss into grad[lvn_surrogate_num_params()] */
int     lvn_surrogate_grad(lvn_surrogate* s, const float* samples, int32_t n, float* grad, float* loss);
/* densities of n points (x, y, z, unused) in `memory` (LVN_MEMORY_HOST or
 * LVN_MEMORY_DEVICE).  Above and below the domain's y range the density is
 * extrapolated with unit slope from the range's edge. */
int     lvn_surrogate_eval(lvn_surrogate* s, const float* points, int64_t n, float* density, int32_t memory);
/* densities of `count` lattices of dim^3 points in device memory: lattice l
 * is lattices[4l .. 4l+3] = (x0, y0, z0, step), points x0 + step (i, j, k)
 * with i fastest; density[l dim^3 + i + dim (j + dim k)] (device) */
int     lvn_surrogate_eval_lattices(lvn_surrogate* s, const float* lattices, int32_t count, int32_t dim,
                                    float* density);
int     lvn_surrogate_domain(const lvn_surrogate* s, float domain_min[3], float domain_max[3]);
void*   lvn_surrogate_get_stream(lvn_surrogate* s);

/* the density set by lvn_set_density (2D fBm, or 2D fBm + caves) at n points
 * (x, y, z, unused; host) in double precision with the exact simplex
 * constants, into density[n] (host): the FP64 reference the FP32 density and
 * the surrogate are measured against */
int     lvn_density_f64(const float* points, int64_t n, double* density);

/* Mesh with the surrogate: every fresh chunk of this context is probed at
 * 8 x 8 x 8 of its field points; when the chunk's field lies inside the
 * domain in x and z and the surrogate is within `gate` voxels of the chunk
 * (gate x the chunk's voxel size in density units) of the plain density at
 * every probe, the chunk's field is the surrogate's (signs from its
 * densities, crossings by linear interpolation, normals from central
 * differences of its field), else the plain path (fallback).  NULL turns it
 * off.  The surrogate must outlive its use by this context. */
int lvn_meshgen_set_surrogate(lvn_meshgen* ctx, lvn_surrogate* s, float gate);
/* chunks of the last batch that used the surrogate; use[c] = 1 / 0 when not NULL */
int lvn_meshgen_surrogate_chunks(lvn_meshgen* ctx, int32_t* use, int32_t capacity);

/* ---- clipmap chunk lists (class Clipmap, clipmap.h / clipmap.cpp) ----------
 * Over a complete clipmap octree: root_min, root_size (a power of two, at
 * least 256 = CLIPMAP_LEAF_SIZE and at most 16 LOD_MAX_NODE_SIZE nodes per
 * axis) with every node subdivided down to CLIPMAP_LEAF_SIZE, as
 * Clipmap::constructTree / ConstructChildren (clipmap.cpp:715-735, 797-818)
 * build it.  Nodes are written as chunk descriptors (min, size), ready for
 * lvn_meshgen_generate_chunks.  One query lists at most LVN_CLIPMAP_MAX_NODES
 * nodes and opens at most LVN_CLIPMAP_MAX_OPEN nodes per level; beyond that the
 * call returns LVN_ERR_DEVICE_STATUS.  The calls share scratch on the first
 * device they run on and serialise each other. */
#define LVN_CLIPMAP_MAX_NODES 8192
#define LVN_CLIPMAP_MAX_OPEN  4096

/* SelectActiveClipmapNodes (clipmap.cpp:1084-1128, DistanceToNode 1056-1064)
 * for num_cameras cameras (x, y, z each) in one launch: camera q's nodes in
 * the reference's recursion order (pre-order over CHILD_MIN_OFFSETS), the
 * cameras' lists back to back in out; counts[q] = camera q's node count.
 * When the lists do not fit `capacity`, LVN_ERR_CAPACITY (counts set). */
int lvn_clipmap_select(const float* cameras, int32_t num_cameras, const int32_t root_min[3], int32_t root_size,
                       lvn_chunk_desc* out, int32_t capacity, int32_t* counts);
/* The same on device buffers, enqueued on cuda_stream (NULL: the legacy
 * default stream) with no host synchronisation: d_cameras[3 num_cameras],
 * camera q's list at d_out[q stride ..] (its first `stride` nodes), its count
 * in d_counts[q] (-1: an internal limit was exceeded).  Calls on different
 * streams share the scratch: order them. */
int lvn_clipmap_select_device(const float* d_cameras, int32_t num_cameras, const int32_t root_min[3],
                              int32_t root_size, lvn_chunk_desc* d_out, int32_t stride, int32_t* d_counts,
                              void* cuda_stream);
/* The nodes a batch of CSG operations touches (processCSGOperationsImpl,
 * clipmap.cpp:1661-1669): every node no larger than LOD_MAX_NODE_SIZE whose
 * box overlaps an operation's CalcCSGOperationBounds (FindNodesInsideAABB,
 * clipmap.cpp:1571-1597), each once, in the recursion's post-order. */
int lvn_clipmap_touched(const lvn_csg_op* ops, int32_t num_ops, const int32_t root_min[3], int32_t root_size,
                        lvn_chunk_desc* out, int32_t capacity, int32_t* count);

/* ---- seam meshes (GenerateClipmapSeamMesh, clipmap.cpp:573-610) -----------
 * The clipmap's active nodes are `chunks` (disjoint, inside the complete
 * octree root_min / root_size, as above; overlapping or repeated chunks are
 * LVN_ERR_INVALID); chunk c's seam nodes, as
 * lvn_meshgen_generate_chunks returns them (SeamNodeInfo), are
 * seams[seam_offsets[c] .. seam_offsets[c + 1]) (seam_offsets[0] = 0; seams in
 * host or device memory per seams_memory).  For each host (an index into
 * chunks) the seam nodes of the host and of the active nodes next to it are
 * gathered (FindNode / FindActiveNodes / SelectSeamNodes / FilterSeamNode,
 * clipmap.cpp:508-570, 982-1013, 1449-1479), built into an octree
 * (Octree_ConstructUpwards, octree.cpp:90-148) and contoured
 * (Octree_GenerateMesh, octree.cpp:197-551): every leaf becomes a vertex
 * (position, normal, rgb = colour, a = material) in the octree's depth-first
 * order and the quads of edges straddling chunks become triangles of
 * host-local indices, in the recursion's order.  out->chunks[h] gives host h's
 * offsets and counts (num_nodes = its seam leaves); a host without triangles
 * has no mesh (no vertices).  Limits per host: LVN_SEAM_MAX_LEAVES leaves
 * (else LVN_ERR_DEVICE_STATUS) and 2 x host size at most 4096 x the smallest
 * leaf gathered (else LVN_ERR_INVALID).  Calls share scratch on the first
 * device they run on and serialise each other. */
#define LVN_SEAM_MAX_LEAVES 32768
int lvn_seam_generate(const lvn_chunk_desc* chunks, const int32_t* seam_offsets, int32_t num_chunks,
                      const lvn_seam_node* seams, int32_t seams_memory, int32_t voxels_per_chunk,
                      const int32_t root_min[3], int32_t root_size, const int32_t* hosts, int32_t num_hosts,
                      const float colour[3], lvn_batch_out* out);

/* ---- edge-collapse mesh simplification (ngMeshSimplifier) -----------------
 * MeshSimplificationOptions (ng_mesh_simplify.h:8-31); the clipmap scales
 * max_error and max_edge_size by the node's leaf size (clipmap.cpp:456-462). */
typedef struct lvn_simplify_options {
    float   edge_fraction;      /* candidate edges drawn per iteration        */
    int32_t max_iterations;
    float   target_percentage;  /* stop at this fraction of the triangles     */
    float   max_error;          /* 1 / QEF error, plus the degree penalty     */
    float   max_edge_size;
    float   min_angle_cosine;
} lvn_simplify_options;
/* the header's defaults: 0.125, 10, 0.05, 5, 2.5, 0.8 */
void lvn_simplify_options_default(lvn_simplify_options* options);
/* ngMeshSimplifier (ng_mesh_simplify.cpp:441-540) for num_meshes meshes in
 * one launch.  Mesh m is vertices[meshes[m].vertex_offset ..
 * + num_vertices) with triangles[triangle_offset .. + num_triangles)
 * (indices local to the mesh), worldSpaceOffset offsets[4m .. 4m + 3] and
 * options[m]; inputs and outputs in host or device memory per `memory`.  The
 * simplified mesh is written at the same offsets of out_vertices /
 * out_triangles (which may be the inputs) and meshes[m]'s counts are updated;
 * the rest of each mesh's input range holds unspecified values afterwards.
 * Meshes under 100 triangles or vertices are copied unchanged, as in the
 * reference.  The QEF's approximate _mm_rsqrt_ps (qef_simd.h:209) is an exact
 * 1 / sqrt here; the random candidate edges follow std::mt19937(42) with
 * libstdc++'s uniform_int_distribution. */
int lvn_mesh_simplify(const lvn_mesh_vertex* vertices, const lvn_mesh_triangle* triangles, int32_t memory,
                      lvn_chunk_result* meshes, int32_t num_meshes, const float* offsets,
                      const lvn_simplify_options* options, lvn_mesh_vertex* out_vertices,
                      lvn_mesh_triangle* out_triangles);

/* ---- device-resident render meshes (headless GL upload) --------------------
 * The engine uploads a MeshBuffer into GL buffers from a fixed pool of render
 * meshes (Render_AllocRenderMesh / RenderMesh::uploadData,
 * render_mesh.cpp:9-30, 94-138).  GL is not part of this library: a pool here
 * is one vertex arena and one triangle arena in device memory, allocated at
 * creation, that meshes take ranges of (first fit, freed ranges coalesce).
 * A renderer reads a mesh through its handle. */
typedef struct lvn_render_pool lvn_render_pool;
typedef struct lvn_render_mesh_view {
    const lvn_mesh_vertex*   vertices;   /* device */
    int32_t                  num_vertices;
    const lvn_mesh_triangle* triangles;  /* device, mesh-local indices */
    int32_t                  num_triangles;
    float                    position[3];
} lvn_render_mesh_view;
/* NULL on failure (bad sizes, out of device memory) */
lvn_render_pool* lvn_render_pool_create(int64_t vertex_capacity, int64_t triangle_capacity, int32_t max_meshes);
void lvn_render_pool_destroy(lvn_render_pool* pool);
/* Render_AllocRenderMesh(tag, buffer, position): a mesh without triangles
 * gets no render mesh (*handle = -1, LVN_OK); LVN_ERR_CAPACITY when the
 * arenas or handles are exhausted. */
int lvn_render_mesh_upload(lvn_render_pool* pool, const lvn_mesh_vertex* vertices, int32_t num_vertices,
                           const lvn_mesh_triangle* triangles, int32_t num_triangles, int32_t memory,
                           const float position[3], int32_t* handle);
/* every chunk of a batch left in device memory (batch->memory =
 * LVN_MEMORY_DEVICE) in one gather launch: handles[c] (-1 for chunks
 * without triangles); positions[3c..] as the engine passes them (may be
 * NULL).  All or nothing: on LVN_ERR_CAPACITY no mesh is taken. */
int lvn_render_meshes_from_batch(lvn_render_pool* pool, const lvn_batch_out* batch, int32_t num_chunks,
                                 const float* positions, int32_t* handles);
int lvn_render_mesh_get(lvn_render_pool* pool, int32_t handle, lvn_render_mesh_view* out);
/* a mesh's data to host arrays of at least its counts (tests, file dumps) */
int lvn_render_mesh_download(lvn_render_pool* pool, int32_t handle, lvn_mesh_vertex* vertices,
                             lvn_mesh_triangle* triangles);
int lvn_render_mesh_free(lvn_render_pool* pool, int32_t handle);
int lvn_render_pool_usage(lvn_render_pool* pool, int64_t* vertices_used, int64_t* triangles_used, int32_t* meshes);

#ifdef __cplusplus
}
#endif
#endif /* LVN_H */
