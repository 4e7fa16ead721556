// lvn_noalloc.cu -- lvn_generate_chunk_mesh_noalloc: one chunk meshed with
// no memory allocation at all.
//
// Who needs it: an engine thread that cannot call cudaMalloc / cudaFree.
// cudaFree synchronises the whole device and cudaMalloc can stall on the
// driver's allocator, which a frame-locked render or streaming thread cannot
// afford; and engines that budget GPU memory up front forbid allocation after
// start-up.  Such callers pass their own input and output memory and get the
// same mesh as lvn_meshgen_generate_chunk_mesh with caching off.  The call
// reads its counters back and synchronises its stream before it returns.
//
// Every buffer the pipeline needs between its kernels (field corners, edge
// list, cuckoo tables, leaf and quad lists, output staging) lives in one
// file-scope device array of LVN_NOALLOC_SCRATCH_BYTES, held by every GPU
// that loads the library until the process exits.  Its fixed capacities
// (LVN_NOALLOC_MAX_*) bound the chunks it accepts; larger ones are rejected
// with LVN_ERR_CAPACITY.  All calls, from every host thread, share the array
// and each call rewrites what it reads, so calls must not overlap on the GPU:
// two calls in flight at once (different streams or host threads) race on it.
// The call runs on the device lvn_init ran on (the permutation tables live
// there); with another device current it returns LVN_ERR_INVALID.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <cstring>

#include "lvn_kernels.cuh"
#include "lvn_state.h"

namespace {

using namespace lvn;

constexpr int kMaxVpc = LVN_NOALLOC_MAX_VOXELS_PER_CHUNK;
constexpr int64_t kMaxEdges = LVN_NOALLOC_MAX_EDGES;
constexpr int64_t kMaxNodes = LVN_NOALLOC_MAX_NODES;
constexpr int kMaxOps = LVN_NOALLOC_MAX_CSG_OPS;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kF = (size_t)(kMaxVpc + 2) * (kMaxVpc + 2) * (kMaxVpc + 2);
constexpr size_t kNbe = ((size_t)(kMaxVpc + 2) * (kMaxVpc + 2) + kRowTile - 1) / kRowTile;
constexpr size_t kNbv = ((size_t)kMaxVpc * kMaxVpc + kRowTile - 1) / kRowTile;
constexpr int64_t kEdgeSlots = 2 * kMaxEdges + CUCKOO_MIN_TABLE_SIZE + CUCKOO_STASH_SIZE + 512;
constexpr int64_t kNodeSlots = 2 * kMaxNodes + CUCKOO_MIN_TABLE_SIZE + CUCKOO_STASH_SIZE + 512;
constexpr int64_t kNodeTiles = kMaxNodes / kNodeTile + 2;

// byte offsets of the pools inside the scratch array
constexpr size_t OFF_DESC = 0;
constexpr size_t OFF_CS = OFF_DESC + align256(sizeof(ChunkDesc));
constexpr size_t OFF_BS = OFF_CS + align256(sizeof(ChunkState));
constexpr size_t OFF_BRUSH = OFF_BS + align256(sizeof(BatchState));
constexpr size_t kRows = (size_t)(kMaxVpc + 2) * (kMaxVpc + 2);
constexpr size_t OFF_MATS = OFF_BRUSH + align256(sizeof(Brush) * kMaxOps);
constexpr size_t OFF_PLANES = OFF_MATS + align256(kF);
constexpr size_t OFF_ETILES = OFF_PLANES + align256(16 * 3 * kRows);
constexpr size_t OFF_VTILES = OFF_ETILES + align256(16 * kNbe);
constexpr size_t OFF_CTILE = OFF_VTILES + align256(4 * kNbv);
constexpr size_t OFF_EKEYS = OFF_CTILE + align256(4 * 2);
constexpr size_t OFF_ECHUNK = OFF_EKEYS + align256(4 * kMaxEdges);
constexpr size_t OFF_EINFO = OFF_ECHUNK + align256(4 * kMaxEdges);
constexpr size_t OFF_EWORK = OFF_EINFO + align256(16 * kMaxEdges);
constexpr size_t OFF_NCODES = OFF_EWORK + align256(4 * kMaxEdges);
constexpr size_t OFF_NINFO = OFF_NCODES + align256(4 * kMaxNodes);
constexpr size_t OFF_NCHUNK = OFF_NINFO + align256(4 * kMaxNodes);
constexpr size_t OFF_ESLOTS = OFF_NCHUNK + align256(4 * kMaxNodes);
constexpr size_t OFF_NSLOTS = OFF_ESLOTS + align256(8 * kEdgeSlots);
constexpr size_t OFF_QUADS = OFF_NSLOTS + align256(8 * kNodeSlots);
constexpr size_t OFF_NTILES = OFF_QUADS + align256(16 * 3 * kMaxNodes);
constexpr size_t OFF_VERTS = OFF_NTILES + align256(8 * kNodeTiles);
constexpr size_t OFF_TRIS = OFF_VERTS + align256(sizeof(lvn_mesh_vertex) * kMaxNodes);
constexpr size_t OFF_SEAMS = OFF_TRIS + align256(sizeof(lvn_mesh_triangle) * 6 * kMaxNodes);
constexpr size_t OFF_END = OFF_SEAMS + align256(sizeof(lvn_seam_node) * kMaxNodes);
static_assert(OFF_END <= (size_t)LVN_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds LVN_NOALLOC_SCRATCH_BYTES");

// The scratch array.  Host code may not use its name as an address: the
// device address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[LVN_NOALLOC_SCRATCH_BYTES];

// The scratch array's device address, looked up on the first call (with the
// init device current) and kept for the device it was looked up on; the
// lookup is under a lock, so that threads whose first calls meet do not race
// on it (the calls themselves must still not overlap, as they share the array).
int g_scratch_dev = -1;
unsigned char* g_scratch_ptr = nullptr;
std::mutex g_scratch_mutex;

int scratch_for_init_device(int init_device, unsigned char** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return LVN_ERR_NO_DEVICE;
    if (dev != init_device) {
        std::fprintf(stderr, "liblvn: noalloc: device %d is current, but lvn_init ran on device %d\n", dev,
                     init_device);
        return LVN_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_dev != dev || !g_scratch_ptr) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "liblvn: cudaGetSymbolAddress(noalloc scratch) failed: %s\n", cudaGetErrorString(e));
            return LVN_ERR_CUDA;
        }
        g_scratch_ptr = static_cast<unsigned char*>(p);
        g_scratch_dev = dev;
    }
    *out = g_scratch_ptr;
    return LVN_OK;
}

#define NA_CK(call)                                                                            \
    do {                                                                                       \
        const cudaError_t e__ = (call);                                                        \
        if (e__ != cudaSuccess) {                                                              \
            std::fprintf(stderr, "liblvn: %s failed: %s\n", #call, cudaGetErrorString(e__));  \
            return LVN_ERR_CUDA;                                                               \
        }                                                                                      \
    } while (0)

}  // namespace

extern "C" int lvn_generate_chunk_mesh_noalloc(const int32_t min[3], int32_t size, int32_t voxels_per_chunk,
                                               lvn_mesh_out* out, void* cuda_stream) {
    const GlobalView gv = global_view();
    if (!gv.initialised) return LVN_ERR_NOT_INITIALISED;
    if (!min || !out) return LVN_ERR_INVALID;
    const int vpc = voxels_per_chunk;
    if (vpc != 8 && vpc != 16 && vpc != 32 && vpc != 64) return LVN_ERR_INVALID;
    if (vpc > kMaxVpc) return LVN_ERR_CAPACITY;
    if (size <= 0 || size % (vpc * LEAF_SIZE_SCALE) != 0) return LVN_ERR_INVALID;
    cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);

    unsigned char* base = nullptr;
    int rc = scratch_for_init_device(gv.device, &base);
    if (rc) return rc;

    // chunk descriptor and its stored operations, on the stack
    ChunkDesc desc;
    std::memset(&desc, 0, sizeof(desc));
    for (int i = 0; i < 3; i++) {
        desc.off[i] = min[i] / LEAF_SIZE_SCALE;
        desc.min[i] = min[i];
    }
    desc.scale = size / (vpc * LEAF_SIZE_SCALE);
    desc.size = size;
    lod_colour_for(size / CLIPMAP_LEAF_SIZE, desc.colour);
    Brush brushes[kMaxOps];
    const int nops = stored_ops_for_chunk(min, size, brushes, kMaxOps);
    if (nops < 0) {
        std::fprintf(stderr, "liblvn: noalloc: more than %d stored CSG operations overlap the chunk\n", kMaxOps);
        return LVN_ERR_CAPACITY;
    }
    desc.op_begin = 0;
    desc.op_count = nops;
    csg_box_for(brushes, nops, desc.off, desc.scale, vpc + 2, desc.csg_lo, desc.csg_hi);

    BatchPtrs b;
    std::memset(&b, 0, sizeof(b));
    b.n = 1;
    b.hash_fault = device_hash_fault();
    b.vpc = vpc;
    b.crossing_mode = 0;
    b.plain_class = 1;
    b.derive_mats = 1;
    b.num_sms = gv.num_sms;
    b.density = gv.density;
    b.default_material = gv.default_material;
    density_fields(gv.density, gv.default_material, &b.cave_band, b.cave_rem, b.dom_by_solid);
    b.perm = gv.perm;
    b.perm_t3 = gv.perm_t3;
    b.grad = gv.grad;
    b.desc = reinterpret_cast<ChunkDesc*>(base + OFF_DESC);
    b.cs = reinterpret_cast<ChunkState*>(base + OFF_CS);
    b.bs = reinterpret_cast<BatchState*>(base + OFF_BS);
    b.brushes = reinterpret_cast<Brush*>(base + OFF_BRUSH);
    b.mats = reinterpret_cast<uint8_t*>(base + OFF_MATS);
    b.planes = reinterpret_cast<uint4*>(base + OFF_PLANES);
    b.edge_tiles = reinterpret_cast<int4*>(base + OFF_ETILES);
    b.vox_tiles = reinterpret_cast<int*>(base + OFF_VTILES);
    b.chunk_tile_off = reinterpret_cast<int*>(base + OFF_CTILE);
    b.edge_keys = reinterpret_cast<int32_t*>(base + OFF_EKEYS);
    b.edge_chunk = reinterpret_cast<int32_t*>(base + OFF_ECHUNK);
    b.edge_info = reinterpret_cast<float4*>(base + OFF_EINFO);
    b.edge_work = reinterpret_cast<int32_t*>(base + OFF_EWORK);
    b.ecap = kMaxEdges;
    b.node_codes = reinterpret_cast<uint32_t*>(base + OFF_NCODES);
    b.node_info = reinterpret_cast<int32_t*>(base + OFF_NINFO);
    b.node_chunk = reinterpret_cast<int32_t*>(base + OFF_NCHUNK);
    b.vcap = kMaxNodes;
    b.edge_slots = reinterpret_cast<unsigned long long*>(base + OFF_ESLOTS);
    b.edge_slot_cap = kEdgeSlots;
    b.node_slots = reinterpret_cast<unsigned long long*>(base + OFF_NSLOTS);
    b.node_slot_cap = kNodeSlots;
    b.quad_scratch = reinterpret_cast<int4*>(base + OFF_QUADS);
    b.node_tile_counts = reinterpret_cast<int2*>(base + OFF_NTILES);
    b.node_tile_cap = kNodeTiles;
    b.vertices = reinterpret_cast<lvn_mesh_vertex*>(base + OFF_VERTS);
    b.vertex_cap = kMaxNodes;
    b.triangles = reinterpret_cast<lvn_mesh_triangle*>(base + OFF_TRIS);
    b.triangle_cap = 6 * kMaxNodes;
    b.seams = reinterpret_cast<lvn_seam_node*>(base + OFF_SEAMS);
    b.seam_cap = kMaxNodes;

    ChunkState cs;
    BatchState bs;
    constexpr int kMaxHashAttempts = 16;
    int attempt = 0;
    for (;; attempt++) {
        if (attempt == kMaxHashAttempts) return LVN_ERR_HASH;
        draw_hash_params(desc.edge_params);
        draw_hash_params(desc.node_params);
        // pageable host sources: the driver stages them, nothing is allocated here
        NA_CK(cudaMemcpyAsync(base + OFF_DESC, &desc, sizeof(desc), cudaMemcpyHostToDevice, stream));
        if (nops) NA_CK(cudaMemcpyAsync(base + OFF_BRUSH, brushes, sizeof(Brush) * nops, cudaMemcpyHostToDevice, stream));
        // the reset kernel clears the per-chunk counters; every other pool is
        // written before it is read within this call
        NA_CK(launch_reset(b, stream));
        NA_CK(launch_field(b, stream));
        if (nops) NA_CK(launch_csg(b, stream));
        NA_CK(launch_edge_count(b, stream));
        NA_CK(launch_edge_plan(b, stream));
        NA_CK(launch_edge_scatter(b, stream));
        NA_CK(launch_hermite(b, stream));
        NA_CK(launch_vox_count(b, stream));
        NA_CK(launch_vox_plan(b, stream));
        NA_CK(launch_vox_scatter(b, stream));
        NA_CK(launch_primes(b, stream));
        NA_CK(launch_hash_fill(b, stream));
        NA_CK(launch_edge_insert(b, stream));
        NA_CK(launch_leaf(b, stream));
        NA_CK(launch_node_insert(b, stream));
        NA_CK(launch_mesh_count(b, stream));
        NA_CK(launch_mesh_plan(b, stream));
        NA_CK(launch_mesh_scatter(b, stream));
        NA_CK(cudaMemcpyAsync(&cs, base + OFF_CS, sizeof(cs), cudaMemcpyDeviceToHost, stream));
        NA_CK(cudaMemcpyAsync(&bs, base + OFF_BS, sizeof(bs), cudaMemcpyDeviceToHost, stream));
        NA_CK(cudaStreamSynchronize(stream));
        if (bs.overflow) {
            std::fprintf(stderr,
                         "liblvn: noalloc: chunk exceeds the static scratch (edges %d of %lld, leaves %d of %lld)\n",
                         bs.total_edges, (long long)kMaxEdges, bs.total_nodes, (long long)kMaxNodes);
            return LVN_ERR_CAPACITY;
        }
        if (!cs.edge_insert_failed && !cs.node_insert_failed) break;
    }

    out->num_vertices = cs.quads > 0 ? cs.nodes : 0;
    out->num_triangles = 2 * cs.quads;
    out->num_seams = cs.seams;
    if (out->num_vertices > out->vertex_capacity || out->num_triangles > out->triangle_capacity ||
        out->num_seams > out->seam_capacity)
        return LVN_ERR_CAPACITY;
    const cudaMemcpyKind kind = out->memory == LVN_MEMORY_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (out->num_vertices)
        NA_CK(cudaMemcpyAsync(out->vertices, base + OFF_VERTS, sizeof(lvn_mesh_vertex) * out->num_vertices, kind, stream));
    if (out->num_triangles)
        NA_CK(cudaMemcpyAsync(out->triangles, base + OFF_TRIS, sizeof(lvn_mesh_triangle) * out->num_triangles, kind,
                              stream));
    if (out->num_seams)
        NA_CK(cudaMemcpyAsync(out->seams, base + OFF_SEAMS, sizeof(lvn_seam_node) * out->num_seams, kind, stream));
    NA_CK(cudaStreamSynchronize(stream));
    return LVN_OK;
}
