// lvn_api.cu -- host orchestration and the C ABI of liblvn (include/lvn.h).
//
// Replaces the reference's OpenCL host layer (leven/src/compute.cpp,
// compute_density_field.cpp, compute_octree.cpp, compute_csg.cpp,
// compute_cuckoo.cpp).  One CUDA stream per mesh-generation context; a batch
// of chunks is enqueued as a fixed sequence of kernels with no host round
// trip, then one small device-to-host read returns the per-chunk counts.
// Device pools grow on demand and are reused across calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <thread>
#include <tuple>
#include <vector>

#include "lvn_kernels.cuh"
#include "lvn_state.h"

using namespace lvn;

namespace {

#define LVN_CK(call)                                                                 \
    do {                                                                             \
        cudaError_t err__ = (call);                                                  \
        if (err__ != cudaSuccess) {                                                  \
            std::fprintf(stderr, "liblvn: %s failed: %s\n", #call, cudaGetErrorString(err__)); \
            return err__ == cudaErrorMemoryAllocation ? LVN_ERR_OUT_OF_MEMORY : LVN_ERR_CUDA; \
        }                                                                            \
    } while (0)

// ---------------------------------------------------------------------------
// buffers
// ---------------------------------------------------------------------------

// Host-side fault injection (lvn_debug_inject_fault): how many of the next
// device allocations fail, and how many of the next hash-parameter draws
// return a degenerate family.  Test hooks; both stay 0 in normal use.
int g_fault_device_alloc = 0;
int g_fault_hash_family = 0;
bool g_fault_hash_host_only = false;  // the degenerate draws spare the device-side repair

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (g_fault_device_alloc > 0) {  // an injected allocation failure
            g_fault_device_alloc--;
            return cudaErrorMemoryAllocation;
        }
        const size_t alloc = std::max<size_t>(need, 256);
        cudaError_t e = cudaMalloc(&p, alloc);
        if (e == cudaSuccess) bytes = alloc;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

struct HostBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        const size_t alloc = std::max<size_t>(need, 256);
        cudaError_t e = cudaMallocHost(&p, alloc);
        if (e == cudaSuccess) bytes = alloc;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

// ---------------------------------------------------------------------------
// global compute state (compute.cpp:168-232, compute_density_field.cpp:23-24)
// ---------------------------------------------------------------------------

struct StoredOp {
    lvn_csg_op op;
    int32_t lo[3], hi[3];
};

struct Global {
    bool initialised = false;
    int device = 0;
    int num_sms = 0;
    int32_t default_material = 0;
    int32_t seed = 0;
    DevBuf perm, perm_t3, grad;
    DensityParams density{LVN_DENSITY_REFERENCE, 8, 1.f / 256.f, 2.f, 0.5f, 48.f, 6, 1.f / 64.f, 2.f, 0.5f, 12.f};
    std::vector<StoredOp> ops;
    std::mt19937 hash_gen;  // default-seeded, drawn in call order (compute_cuckoo.cpp:46-47)
} g;

// Ken Perlin's reference permutation (public domain).
const uint8_t kPerlin[256] = {
    151, 160, 137, 91,  90,  15,  131, 13,  201, 95,  96,  53,  194, 233, 7,   225, 140, 36,  103, 30,  69,  142,
    8,   99,  37,  240, 21,  10,  23,  190, 6,   148, 247, 120, 234, 75,  0,   26,  197, 62,  94,  252, 219, 203,
    117, 35,  11,  32,  57,  177, 33,  88,  237, 149, 56,  87,  174, 20,  125, 136, 171, 168, 68,  175, 74,  165,
    71,  134, 139, 48,  27,  166, 77,  146, 158, 231, 83,  111, 229, 122, 60,  211, 133, 230, 220, 105, 92,  41,
    55,  46,  245, 40,  244, 102, 143, 54,  65,  25,  63,  161, 1,   216, 80,  73,  209, 76,  132, 187, 208, 89,
    18,  169, 200, 196, 135, 130, 116, 188, 159, 86,  164, 100, 109, 198, 173, 186, 3,   64,  52,  217, 226, 250,
    124, 123, 5,   202, 38,  147, 118, 126, 255, 82,  85,  212, 207, 206, 59,  227, 47,  16,  58,  17,  182, 189,
    28,  42,  223, 183, 170, 213, 119, 248, 152, 2,   44,  154, 163, 70,  221, 153, 101, 155, 167, 43,  172, 9,
    129, 22,  39,  253, 19,  98,  108, 110, 79,  113, 224, 232, 178, 185, 112, 104, 218, 246, 97,  228, 251, 34,
    242, 193, 238, 210, 144, 12,  191, 179, 162, 241, 81,  51,  145, 235, 249, 14,  239, 107, 49,  192, 214, 31,
    181, 199, 106, 157, 184, 84,  204, 176, 115, 121, 50,  45,  127, 4,   150, 254, 138, 236, 205, 93,  222, 114,
    67,  29,  24,  72,  243, 141, 128, 195, 78,  66,  215, 61,  156, 180};

// gradient directions (compute_density_field.cpp:60-63)
const int8_t kGrad3[16][3] = {{0, 1, 1},  {0, 1, -1},  {0, -1, 1}, {0, -1, -1}, {1, 0, 1},  {1, 0, -1},
                              {-1, 0, 1}, {-1, 0, -1}, {1, 1, 0},  {1, -1, 0},  {-1, 1, 0}, {-1, -1, 0},
                              {1, 0, -1}, {-1, 0, -1}, {0, -1, 1}, {0, 1, 1}};

// Jenkins one-at-a-time over the key's little-endian bytes (compute_density_field.cpp:68-86)
uint32_t noise_hash(int x, int y, int seed) {
    const uint32_t key = (((uint32_t)x << 24) | ((uint32_t)y << 16)) ^ (uint32_t)seed;
    uint32_t h = 0;
    for (int i = 0; i < 4; i++) {
        h += (key >> (8 * i)) & 0xffu;
        h += h << 10;
        h ^= h >> 6;
    }
    h += h << 3;
    h ^= h >> 11;
    h += h << 15;
    return h;
}

// CreateNoisePermutationLookupImage (compute_density_field.cpp:90-125): the
// 512-entry literal there holds Perlin's 256 values, then the same list
// without its first six, then six zeros; it is shuffled with the seeded
// default engine and sampled per texel by the Jenkins hash.
int upload_perm(int seed) {
    std::array<int, 512> perm{};
    for (int i = 0; i < 256; i++) perm[i] = kPerlin[i];
    for (int k = 0; k < 250; k++) perm[256 + k] = kPerlin[6 + k];
    std::shuffle(perm.begin(), perm.end(), std::default_random_engine(seed));
    std::vector<uint8_t> v(65536);
    for (int i = 0; i < 256; i++)
        for (int j = 0; j < 256; j++) v[i * 256 + j] = (uint8_t)perm[noise_hash(i, j, seed) & 0x1ff];
    // RGB as read_imagef returns UNORM8: (b / 255) * 4 - 1
    float grad[64];
    for (int k = 0; k < 16; k++) {
        for (int c = 0; c < 3; c++) {
            const unsigned char b = (unsigned char)(kGrad3[k][c] * 64 + 64);
            grad[4 * k + c] = ((float)b / 255.0f) * 4.0f - 1.0f;
        }
        grad[4 * k + 3] = 0.f;
    }
    LVN_CK(g.perm.ensure(65536));
    // the simplex lookup tables (kT3Row x kT3Row texels each, see lvn_types.h)
    std::vector<uint8_t> t3(kT3Bytes, 0);
    for (int r = 0; r < kT3Row; r++)
        for (int c = 0; c < kT3Row; c++) {
            const uint8_t a = v[(r & 255) * 256 + (c & 255)];
            t3[r * kT3Row + c] = a == 255 ? 0 : a;
            t3[kT3Second + r * kT3Row + c] = (uint8_t)((a & 15) * 8);
        }
    LVN_CK(g.perm_t3.ensure(kT3Bytes));
    LVN_CK(cudaMemcpy(g.perm_t3.p, t3.data(), kT3Bytes, cudaMemcpyHostToDevice));
    LVN_CK(g.grad.ensure(sizeof(grad)));
    LVN_CK(cudaMemcpy(g.perm.p, v.data(), 65536, cudaMemcpyHostToDevice));
    LVN_CK(cudaMemcpy(g.grad.p, grad, sizeof(grad), cudaMemcpyHostToDevice));
    g.seed = seed;
    return LVN_OK;
}

// CalcCSGOperationBounds (clipmap.cpp:1638-1643): CSG_OFFSET 0.5, fudge 2,
// ivec3(float) truncation
void op_bounds(const lvn_csg_op& op, int32_t lo[3], int32_t hi[3]) {
    for (int i = 0; i < 3; i++) {
        const int half = (int)(op.dimensions[i] * (float)LEAF_SIZE_SCALE) + 2;
        const int origin = (int)((op.origin[i] - 0.5f) * (float)LEAF_SIZE_SCALE);
        lo[i] = origin - half;
        hi[i] = origin + half;
    }
}

// AABB::overlaps (aabb.h:26-35), inclusive bounds
bool overlaps(const int32_t alo[3], const int32_t ahi[3], const int32_t blo[3], const int32_t bhi[3]) {
    return !(ahi[0] < blo[0] || ahi[1] < blo[1] || ahi[2] < blo[2] || alo[0] > bhi[0] || alo[1] > bhi[1] ||
             alo[2] > bhi[2]);
}

Brush make_brush(const lvn_csg_op& op) {
    Brush b;
    for (int i = 0; i < 3; i++) {
        b.origin[i] = op.origin[i];
        b.dimensions[i] = op.dimensions[i];
    }
    b.type = op.type;
    b.brush = op.brush_shape;
    b.cos_y = (float)std::cos((double)op.rotate_y);
    b.sin_y = (float)std::sin((double)op.rotate_y);
    b.material = op.material;
    b.pad = 0;
    return b;
}

// Field-index box holding every point the operations can change: a sphere's
// points with d <= 0 lie within its radius, a cube's (rotated about y) within
// sqrt(hx^2 + hz^2) in x/z and hy in y; one density unit of margin.
void csg_box(const Brush* ops, int n, const int32_t off[3], int scale, int fd, int32_t lo[3], int32_t hi[3]) {
    for (int i = 0; i < 3; i++) {
        lo[i] = fd;
        hi[i] = -1;
    }
    for (int k = 0; k < n; k++) {
        const Brush& b = ops[k];
        double ext[3];
        if (b.brush != 0) {
            ext[0] = ext[1] = ext[2] = std::fabs((double)b.dimensions[0]);
        } else {
            const double r = std::sqrt((double)b.dimensions[0] * b.dimensions[0] + (double)b.dimensions[2] * b.dimensions[2]);
            ext[0] = ext[2] = r;
            ext[1] = std::fabs((double)b.dimensions[1]);
        }
        for (int i = 0; i < 3; i++) {
            const double l = ((double)b.origin[i] - ext[i] - 1.0 - off[i]) / scale;
            const double h = ((double)b.origin[i] + ext[i] + 1.0 - off[i]) / scale;
            int li = 0, hi_ = fd - 1;
            if (std::isfinite(l) && std::isfinite(h)) {
                li = (int)std::max(0.0, std::min((double)fd - 1, std::floor(l)));
                hi_ = (int)std::max(0.0, std::min((double)fd - 1, std::ceil(h)));
                if (h < 0.0 || l > fd - 1) { li = fd; hi_ = -1; }  // entirely outside the field
            }
            lo[i] = std::min(lo[i], li);
            hi[i] = std::max(hi[i], hi_);
        }
    }
}

bool valid_op(const lvn_csg_op& op) {
    return (op.type == 0 || op.type == 1) && (op.brush_shape == 0 || op.brush_shape == 1) && op.material >= 0 &&
           op.material <= 255;
}

// ColourForMinLeafSize (clipmap.cpp:329-353)
void lod_colour(int s, float c[3]) {
    switch (s) {
        case 1: c[0] = 0.3f; c[1] = 0.1f; c[2] = 0.f; break;
        case 2: c[0] = 0.f; c[1] = 0.f; c[2] = 0.5f; break;
        case 4: c[0] = 0.f; c[1] = 0.5f; c[2] = 0.5f; break;
        case 8: c[0] = 0.5f; c[1] = 0.f; c[2] = 0.5f; break;
        case 16: c[0] = 0.f; c[1] = 0.5f; c[2] = 0.f; break;
        default: c[0] = 0.5f; c[1] = 0.f; c[2] = 0.f; break;
    }
}

// the shared parameter generator; contexts running batches on their own host
// threads (lvn_meshgen_generate_chunks_async) draw from it concurrently
std::mutex g_hash_gen_mutex;

void draw_params(uint32_t* p) {
    std::lock_guard<std::mutex> lock(g_hash_gen_mutex);
    std::uniform_int_distribution<uint32_t> dist(1u << 15, 1u << 30);
    for (int i = 0; i < CUCKOO_HASH_FN_COUNT * 2; i++) p[i] = dist(g.hash_gen);
    if (g_fault_hash_family > 0) {
        // injected: a = 0 and one b for every function, so all keys share one
        // slot and one stash entry and a third key cannot be inserted
        g_fault_hash_family--;
        for (int i = 0; i < CUCKOO_HASH_FN_COUNT * 2; i++) p[i] = (i & 1) ? 1u << 15 : 0u;
    }
}

// FindNextPrime (primes.cpp:32-58) on the host
int host_next_prime(int n) {
    auto is_prime = [](int x) {
        int o = 4, i = 5;
        for (;;) {
            const int q = x / i;
            if (q < i) return true;
            if (x == q * i) return false;
            o ^= 6;
            i += o;
        }
    };
    if (n <= 5) return n <= 2 ? 2 : n == 3 ? 3 : 5;
    const int k = n / 6;
    int i = n - 6 * k;
    const int o = i < 2 ? 1 : 5;
    int x = 6 * k + o;
    for (i = (3 + o) / 2; !is_prime(x); x += i) i ^= 6;
    return x;
}

}  // namespace

// ---------------------------------------------------------------------------
// mesh-generation context
// ---------------------------------------------------------------------------

typedef std::tuple<int32_t, int32_t, int32_t, int32_t> ChunkKey;

struct FieldEntry {  // GPUDensityField (compute_local.h:28-37)
    DevBuf mats, planes;
    DevBuf keys, info;
    int32_t num_edges = 0;
    int32_t last_op = 0;
};

struct OctreeEntry {  // the mesh a cached GPUOctree (compute_local.h:43-49) regenerates
    std::vector<lvn_mesh_vertex> vertices;
    std::vector<lvn_mesh_triangle> triangles;
    std::vector<lvn_seam_node> seams;
    int32_t num_vertices = 0;
};

struct lvn_meshgen {
    int vpc = 64;
    // a batch in flight on a host thread of its own (lvn_meshgen_generate_chunks_async)
    std::thread async_thread;
    bool async_active = false;
    bool host_writes = true;  // LVN_OPT_HOST_WRITES
    int hermite_form = 0;     // LVN_OPT_HERMITE_FORM
    bool compute_order = false;  // LVN_OPT_COMPUTE_ORDER
    cudaEvent_t ev_order = nullptr;  // recorded after this context's last ordered batch's kernels
    int async_rc = 0;
    std::vector<lvn_chunk_desc> async_chunks;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int crossing_mode = 0;
    bool cache = true;
    bool profile = false;
    float simp_threshold = -1.f;  // bottom-up octree simplification; < 0 = off
    lvn_surrogate* surrogate = nullptr;  // learned density for the chunks that pass its probe gate
    float surrogate_gate = 0.5f;
    std::vector<int32_t> last_suse;

    // pools
    DevBuf desc, cs, bs, brushes, mats, planes, edge_tiles, vox_tiles, hmap;
    DevBuf edge_keys, edge_chunk, edge_info, edge_work, node_codes, node_info, node_chunk;
    DevBuf edge_slots, node_slots, quad_scratch, node_tile_counts, chunk_tile_off;
    DevBuf vertices, triangles, seams;
    // octree simplification
    DevBuf leaf_vertices, leaf_qef, simp_grid, simp_nodes, simp_count, simp_rep, simp_entry, simp_newidx, simp_mask,
        simp_tile_counts;
    int64_t simp_vcap = 0, simp_grid_chunks = 0, simp_node_cap = 0, simp_tile_cap = 0;
    // surrogate meshing
    DevBuf probe_pts, probe_plain, probe_s, gate_ok, sslot, sdens, lattices;
    HostBuf h_gate, h_sslot, h_lattices;
    HostBuf h_desc, h_brushes, h_cs, h_bs;
    int64_t ecap = 0, vcap = 0, eslot_cap = 0, nslot_cap = 0, ntile_cap = 0;
    int64_t vert_cap = 0, tri_cap = 0, seam_cap = 0;
    int chunk_cap = 0;

    // last batch, for debug fetch
    int last_n = 0;
    bool last_fresh = true;
    std::vector<ChunkState> last_cs;
    std::vector<ChunkDesc> last_desc;

    // batch graph: the whole fresh-batch sequence captured once per key
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<uintptr_t> graph_key;
    bool use_graphs = true;

    // export of pinned host outputs: a side stream and its events
    cudaStream_t side = nullptr;
    cudaEvent_t ev_leaf = nullptr, ev_side = nullptr;
    // the fresh-batch DAG: hermite on `aux` beside the voxel, hash and quad
    // stages, with a grid of dag_hermite_per_sm CTAs per SM (0 = its tuned shape)
    cudaStream_t aux = nullptr, aux2 = nullptr;  // hermite; the quad chain
    cudaEvent_t ev_fork = nullptr, ev_herm = nullptr, ev_hash = nullptr, ev_mesh = nullptr;
    int dag_hermite_per_sm = 0;

    // the shapes an autotuning in progress on this context is trying (CTAs
    // per SM per stage, and hermite's inside the batch DAG); the results are
    // published process-wide (g_tunes) when the tuning ends
    bool tuning = false;
    std::map<std::array<int, 4>, std::array<int, ST_COUNT>> tunes;
    std::map<std::array<int, 4>, int> dag_tunes;

    // profiling
    cudaEvent_t ev[ST_COUNT + 1] = {};
    double stage_ms[ST_COUNT] = {};
    int stage_launches[ST_COUNT] = {};

    std::map<ChunkKey, FieldEntry> fields;
    std::map<ChunkKey, OctreeEntry> octrees;
};

namespace {

struct Capacity {
    int64_t ecap, vcap;
};

// Entries of the simplification's level lists: level k holds at most one
// entry per voxel and per level-k cell of each chunk.  `off` receives each
// level's first entry.
int64_t simp_node_capacity(int vpc, int n, int64_t vcap, int64_t* off) {
    int64_t total = 0;
    for (int k = 0; k < 8; k++) {
        if (off) off[k] = total;
        if (k == 0 || k > octree_depth(vpc)) continue;
        const int64_t cells = (int64_t)n * (vpc >> k) * (vpc >> k) * (vpc >> k);
        total += std::min(vcap, cells);
    }
    return total;
}

// Size every pool for `n` chunks with at least the given edge / node capacity.
int ensure_pools(lvn_meshgen* m, int n, Capacity want) {
    const int F = field_size(m->vpc);
    const int C = m->vpc * m->vpc * m->vpc;
    const int64_t ecap = std::max<int64_t>(want.ecap, 1024);
    const int64_t vcap = std::max<int64_t>(want.vcap, 1024);
    LVN_CK(m->desc.ensure(sizeof(ChunkDesc) * n));
    LVN_CK(m->cs.ensure(sizeof(ChunkState) * n));
    LVN_CK(m->bs.ensure(sizeof(BatchState)));
    LVN_CK(m->mats.ensure((size_t)F * n));
    LVN_CK(m->planes.ensure(sizeof(uint4) * 3 * (size_t)field_rows(m->vpc) * n));
    LVN_CK(m->hmap.ensure(sizeof(float) * (size_t)field_rows(m->vpc) * n));
    LVN_CK(m->edge_tiles.ensure(sizeof(int4) * (size_t)edge_tiles_per_chunk(m->vpc) * n));
    LVN_CK(m->vox_tiles.ensure(sizeof(int) * (size_t)vox_tiles_per_chunk(m->vpc) * n));
    LVN_CK(m->chunk_tile_off.ensure(sizeof(int) * (size_t)(n + 1)));
    LVN_CK(m->h_desc.ensure(sizeof(ChunkDesc) * n));
    LVN_CK(m->h_cs.ensure(sizeof(ChunkState) * n));
    LVN_CK(m->h_bs.ensure(sizeof(BatchState)));
    if (ecap > m->ecap) {
        LVN_CK(m->edge_keys.ensure(sizeof(int32_t) * ecap));
        LVN_CK(m->edge_chunk.ensure(sizeof(int32_t) * ecap));
        LVN_CK(m->edge_info.ensure(sizeof(float4) * ecap));
        LVN_CK(m->edge_work.ensure(sizeof(int32_t) * ecap));
        m->ecap = ecap;
    }
    const int64_t eslots = 2 * m->ecap + (int64_t)n * (CUCKOO_MIN_TABLE_SIZE + CUCKOO_STASH_SIZE + 512);
    if (eslots > m->eslot_cap) {
        LVN_CK(m->edge_slots.ensure(sizeof(unsigned long long) * eslots));
        m->eslot_cap = eslots;
    }
    if (vcap > m->vcap) {
        LVN_CK(m->node_codes.ensure(sizeof(uint32_t) * vcap));
        LVN_CK(m->node_info.ensure(sizeof(int32_t) * vcap));
        LVN_CK(m->node_chunk.ensure(sizeof(int32_t) * vcap));
        LVN_CK(m->quad_scratch.ensure(sizeof(int4) * 3 * vcap));
        LVN_CK(m->vertices.ensure(sizeof(lvn_mesh_vertex) * vcap));
        LVN_CK(m->triangles.ensure(sizeof(lvn_mesh_triangle) * 6 * vcap));
        LVN_CK(m->seams.ensure(sizeof(lvn_seam_node) * vcap));
        m->vcap = vcap;
        m->vert_cap = vcap;
        m->tri_cap = 6 * vcap;
        m->seam_cap = vcap;
    }
    const int64_t nslots = 2 * m->vcap + (int64_t)n * (CUCKOO_MIN_TABLE_SIZE + CUCKOO_STASH_SIZE + 512);
    if (nslots > m->nslot_cap) {
        LVN_CK(m->node_slots.ensure(sizeof(unsigned long long) * nslots));
        m->nslot_cap = nslots;
    }
    const int64_t ntiles = m->vcap / kNodeTile + n + 1;
    if (ntiles > m->ntile_cap) {
        LVN_CK(m->node_tile_counts.ensure(sizeof(int2) * ntiles));
        m->ntile_cap = ntiles;
    }
    (void)C;
    if (m->simp_threshold >= 0.f) {
        if (m->vcap > m->simp_vcap) {
            LVN_CK(m->leaf_vertices.ensure(sizeof(lvn_mesh_vertex) * m->vcap));
            LVN_CK(m->leaf_qef.ensure(sizeof(SimpQef) * m->vcap));
            LVN_CK(m->simp_rep.ensure(sizeof(int) * m->vcap));
            LVN_CK(m->simp_entry.ensure(sizeof(int) * m->vcap));
            LVN_CK(m->simp_newidx.ensure(sizeof(int) * m->vcap));
            LVN_CK(m->simp_mask.ensure(m->vcap));
            m->simp_vcap = m->vcap;
        }
        if (n > m->simp_grid_chunks) {
            LVN_CK(m->simp_grid.ensure(sizeof(int) * (size_t)n * (size_t)simp_grid_cells(m->vpc)));
            m->simp_grid_chunks = n;
        }
        const int64_t nodes = simp_node_capacity(m->vpc, n, m->vcap, nullptr);
        if (nodes > m->simp_node_cap) {
            LVN_CK(m->simp_nodes.ensure(sizeof(SimpNode) * nodes));
            m->simp_node_cap = nodes;
        }
        LVN_CK(m->simp_count.ensure(sizeof(int) * 8));
        if (m->ntile_cap > m->simp_tile_cap) {
            LVN_CK(m->simp_tile_counts.ensure(sizeof(int2) * m->ntile_cap));
            m->simp_tile_cap = m->ntile_cap;
        }
    }
    m->chunk_cap = std::max(m->chunk_cap, n);
    return LVN_OK;
}

Capacity default_capacity(const lvn_meshgen* m, int n) {
    const int F = field_size(m->vpc);
    const int C = m->vpc * m->vpc * m->vpc;
    // per-chunk averages sized for surface chunks; one chunk's worst case always fits
    return Capacity{(int64_t)n * (int64_t)std::min(3 * F, 48 * 1024) + 3 * (int64_t)F,
                    (int64_t)n * (int64_t)std::min(C, 24 * 1024) + (int64_t)C};
}

// Autotuned launch shapes, keyed by density mode, crossing mode,
// simplification on/off and log2(batch size), shared by every context of the
// process: the best shapes are a property of the device and the kind of
// batch, and contexts that keep batches in flight side by side should run
// them alike.
struct Tuned {
    std::array<int, ST_COUNT> shape;  // CTAs per SM per stage (0 = built-in)
    int dag_hermite;                  // hermite's CTAs per SM inside the batch DAG
};
std::mutex g_tune_mutex;
std::map<std::array<int, 4>, Tuned> g_tunes;

// The shapes for batches of kind `key` on context m: those its own tuning
// is trying, else the published ones.  False when there are none.
bool stage_shapes(const lvn_meshgen* m, const std::array<int, 4>& key, std::array<int, ST_COUNT>* shape,
                  int* dag_hermite) {
    if (m->tuning) {
        const auto t = m->tunes.find(key);
        const auto d = m->dag_tunes.find(key);
        if (shape && t != m->tunes.end()) *shape = t->second;
        if (dag_hermite) *dag_hermite = d != m->dag_tunes.end() ? d->second : 0;
        return t != m->tunes.end();
    }
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    const auto t = g_tunes.find(key);
    if (t == g_tunes.end()) {
        if (dag_hermite) *dag_hermite = 0;
        return false;
    }
    if (shape) *shape = t->second.shape;
    if (dag_hermite) *dag_hermite = t->second.dag_hermite;
    return true;
}

std::array<int, 4> tune_key(const lvn_meshgen* m, int n) {
    int bucket = 0;
    while ((2 << bucket) <= n) bucket++;
    return {g.density.mode, m->crossing_mode, m->simp_threshold >= 0.f ? 1 : 0, bucket};
}

BatchPtrs make_ptrs(lvn_meshgen* m, int n) {
    BatchPtrs b;
    std::memset(&b, 0, sizeof(b));
    std::array<int, ST_COUNT> shape{};
    if (stage_shapes(m, tune_key(m, n), &shape, nullptr))
        for (int st = 0; st < ST_COUNT; st++) b.grid_per_sm[st] = shape[st];
    b.n = n;
    b.vpc = m->vpc;
    b.crossing_mode = m->crossing_mode;
    b.plain_class = 1;
    b.derive_mats = 1;
    b.need_mats = 0;
    b.num_sms = g.num_sms;
    b.hash_fault = device_hash_fault();
    b.hermite_form = m->hermite_form;
    b.density = g.density;
    b.default_material = g.default_material;
    density_fields(g.density, g.default_material, &b.cave_band, b.cave_rem, b.dom_by_solid);
    b.desc = m->desc.as<ChunkDesc>();
    b.cs = m->cs.as<ChunkState>();
    b.bs = m->bs.as<BatchState>();
    b.brushes = m->brushes.as<Brush>();
    b.perm = g.perm.as<uint8_t>();
    b.perm_t3 = g.perm_t3.as<uint8_t>();
    b.grad = g.grad.as<float>();
    b.mats = m->mats.as<uint8_t>();
    b.planes = m->planes.as<uint4>();
    b.hmap = m->hmap.as<float>();
    b.edge_tiles = m->edge_tiles.as<int4>();
    b.vox_tiles = m->vox_tiles.as<int>();
    b.edge_keys = m->edge_keys.as<int32_t>();
    b.edge_chunk = m->edge_chunk.as<int32_t>();
    b.edge_info = m->edge_info.as<float4>();
    b.edge_work = m->edge_work.as<int32_t>();
    b.ecap = m->ecap;
    b.node_codes = m->node_codes.as<uint32_t>();
    b.node_info = m->node_info.as<int32_t>();
    b.node_chunk = m->node_chunk.as<int32_t>();
    b.vcap = m->vcap;
    b.edge_slots = m->edge_slots.as<unsigned long long>();
    b.edge_slot_cap = m->eslot_cap;
    b.node_slots = m->node_slots.as<unsigned long long>();
    b.node_slot_cap = m->nslot_cap;
    b.quad_scratch = m->quad_scratch.as<int4>();
    b.node_tile_counts = m->node_tile_counts.as<int2>();
    b.chunk_tile_off = m->chunk_tile_off.as<int>();
    b.node_tile_cap = m->ntile_cap;
    b.vertices = m->vertices.as<lvn_mesh_vertex>();
    b.vertex_cap = m->vert_cap;
    b.triangles = m->triangles.as<lvn_mesh_triangle>();
    b.triangle_cap = m->tri_cap;
    b.seams = m->seams.as<lvn_seam_node>();
    b.seam_cap = m->seam_cap;
    if (m->simp_threshold >= 0.f) {
        b.simp_on = 1;
        b.simp_threshold = m->simp_threshold;
        b.leaf_out = m->leaf_vertices.as<lvn_mesh_vertex>();
        b.leaf_qef = m->leaf_qef.as<SimpQef>();
        b.simp_grid = m->simp_grid.as<int>();
        b.simp_nodes = m->simp_nodes.as<SimpNode>();
        simp_node_capacity(m->vpc, n, m->vcap, b.simp_level_off);
        b.simp_count = m->simp_count.as<int>();
        b.simp_rep = m->simp_rep.as<int>();
        b.simp_entry = m->simp_entry.as<int>();
        b.simp_newidx = m->simp_newidx.as<int>();
        b.simp_mask = m->simp_mask.as<uint8_t>();
        b.simp_tile_counts = m->simp_tile_counts.as<int2>();
    }
    return b;
}

typedef cudaError_t (*Launcher)(const BatchPtrs&, cudaStream_t);

int stage(lvn_meshgen* m, int st, Launcher fn, const BatchPtrs& b) {
    if (m->profile) LVN_CK(cudaEventRecord(m->ev[st], m->stream));
    LVN_CK(fn(b, m->stream));
    if (m->profile) {
        LVN_CK(cudaEventRecord(m->ev[ST_COUNT], m->stream));
        LVN_CK(cudaEventSynchronize(m->ev[ST_COUNT]));
        float ms = 0.f;
        LVN_CK(cudaEventElapsedTime(&ms, m->ev[st], m->ev[ST_COUNT]));
        m->stage_ms[st] += ms;
        m->stage_launches[st] += 1;
    }
    return LVN_OK;
}

#define LVN_STAGE(ST, FN)                        \
    do {                                         \
        const int rc__ = stage(m, ST, FN, b);    \
        if (rc__ != LVN_OK) return rc__;         \
    } while (0)

// Field, CSG and edge stages for fresh fields (LoadDensityField on a cache
// miss followed by the replay of stored operations).
int enqueue_field_stages(lvn_meshgen* m, const BatchPtrs& b, bool any_ops) {
    LVN_CK(launch_reset(b, m->stream));
    LVN_STAGE(ST_FIELD, launch_field);
    if (any_ops) LVN_STAGE(ST_CSG, launch_csg);
    LVN_STAGE(ST_EDGE_COUNT, launch_edge_count);
    LVN_STAGE(ST_EDGE_PLAN, launch_edge_plan);
    LVN_STAGE(ST_EDGE_SCATTER, launch_edge_scatter);
    LVN_STAGE(ST_HERMITE, launch_hermite);
    return LVN_OK;
}

// ConstructOctreeFromField + GenerateMeshFromOctree + GatherSeamNodesFromOctree,
// then the octree simplification when it is on, one stage at a time.
int enqueue_octree_stages(lvn_meshgen* m, const BatchPtrs& b) {
    LVN_STAGE(ST_VOX_COUNT, launch_vox_count);
    LVN_STAGE(ST_VOX_PLAN, launch_vox_plan);
    LVN_STAGE(ST_VOX_SCATTER, launch_vox_scatter);
    LVN_STAGE(ST_PRIMES, launch_primes);
    LVN_STAGE(ST_HASH_FILL, launch_hash_fill);
    LVN_STAGE(ST_EDGE_INSERT, launch_edge_insert);
    LVN_STAGE(ST_LEAF, launch_leaf);
    LVN_STAGE(ST_NODE_INSERT, launch_node_insert);
    LVN_STAGE(ST_MESH_COUNT, launch_mesh_count);
    LVN_STAGE(ST_MESH_PLAN, launch_mesh_plan);
    LVN_STAGE(ST_MESH_SCATTER, launch_mesh_scatter);
    if (b.simp_on) LVN_STAGE(ST_SIMPLIFY, launch_simplify);
    return LVN_OK;
}

// Caller arrays the export kernels write directly (pinned host memory).
struct DirectOut {
    void* dst[3];
    int64_t cap[3];
};

// All three outputs, in order, on one stream.
int enqueue_exports(lvn_meshgen* m, const BatchPtrs& b, const DirectOut* direct, cudaStream_t s) {
    for (int which = 0; which < 3; which++) LVN_CK(launch_export(b, which, direct->dst[which], direct->cap[which], s));
    return LVN_OK;
}

constexpr int kLeafSlices = 4;  // leaf / vertex-export pipeline depth for pinned host outputs

// The fresh-batch DAG (one graph when captured):
//   field, CSG, edges                                           (stream)
//   -> hermite                                                   (aux)
//   || voxels, primes, hash-table fill                           (stream)
//      -> leaf-hash insert, quads, triangles                     (aux2)
//         [pinned outputs: triangles exported on aux2]
//      || edge-hash insert, join hermite, leaves                 (stream)
//         [pinned outputs: the leaves write their vertices to the host
//          array as they are made; an unaligned array instead gets the
//          leaves in slices, each exported on the side stream while the
//          next is computed]
//   -> join -> seams, simplification, exports' join              (stream)
// No branch reads what another writes before their join: the chain beside
// hermite reads edge keys, not edge information; the quad chain reads leaf
// codes and corners, not leaf vertices.  The FP32-bound hermite overlaps the
// latency-bound hash stages (its grid is sized by the autotuner for this), the
// leaves overlap the quad stages, and the exports over C2C (about 190 GB/s)
// start as soon as their data exists.
int enqueue_fresh_dag(lvn_meshgen* m, const BatchPtrs& b, bool any_ops, const DirectOut* direct) {
    cudaStream_t s0 = m->stream;
    LVN_CK(launch_reset(b, s0));
    LVN_CK(launch_field(b, s0));
    if (any_ops) LVN_CK(launch_csg(b, s0));
    LVN_CK(launch_edge_count(b, s0));
    LVN_CK(launch_edge_plan(b, s0));
    LVN_CK(launch_edge_scatter(b, s0));
    LVN_CK(cudaEventRecord(m->ev_fork, s0));
    LVN_CK(cudaStreamWaitEvent(m->aux, m->ev_fork, 0));
    BatchPtrs bh = b;
    if (m->dag_hermite_per_sm > 0) bh.grid_per_sm[ST_HERMITE] = m->dag_hermite_per_sm;
    LVN_CK(launch_hermite(bh, m->aux));
    LVN_CK(cudaEventRecord(m->ev_herm, m->aux));
    LVN_CK(launch_vox_count(b, s0));
    LVN_CK(launch_vox_plan(b, s0));
    LVN_CK(launch_vox_scatter(b, s0));
    LVN_CK(launch_primes(b, s0));
    LVN_CK(launch_hash_fill(b, s0));
    const bool simp = b.simp_on != 0;
    const bool pipelined = direct && !simp;
    // the quad chain
    LVN_CK(cudaEventRecord(m->ev_hash, s0));
    LVN_CK(cudaStreamWaitEvent(m->aux2, m->ev_hash, 0));
    LVN_CK(launch_node_insert(b, m->aux2));
    LVN_CK(launch_mesh_count(b, m->aux2));
    LVN_CK(launch_mesh_plan(b, m->aux2));
    if (!simp) {
        BatchPtrs bt = b;
        bt.scatter_what = 1;  // triangles now, seams once the leaves exist
        LVN_CK(launch_mesh_scatter(bt, m->aux2));
        if (pipelined) LVN_CK(launch_export(b, 1, direct->dst[1], direct->cap[1], m->aux2));
    }
    LVN_CK(cudaEventRecord(m->ev_mesh, m->aux2));
    // the leaves
    LVN_CK(launch_edge_insert(b, s0));
    LVN_CK(cudaStreamWaitEvent(s0, m->ev_herm, 0));
    // pinned host vertices: k_leaf writes them itself when the array is
    // 16-byte aligned; otherwise the leaves run in slices, each exported on
    // the side stream while the next is computed
    const bool fused = pipelined && (reinterpret_cast<uintptr_t>(direct->dst[0]) & 15) == 0;
    const int slices = pipelined && !fused ? kLeafSlices : 1;
    for (int sl = 0; sl < slices; sl++) {
        BatchPtrs bl = b;
        bl.slice = sl;
        bl.nslices = slices;
        if (fused) {
            bl.host_vertices = static_cast<float4*>(direct->dst[0]);
            bl.host_vertex_cap = direct->cap[0];
        }
        LVN_CK(launch_leaf(bl, s0));
        if (pipelined && !fused) {
            LVN_CK(cudaEventRecord(m->ev_leaf, s0));
            LVN_CK(cudaStreamWaitEvent(m->side, m->ev_leaf, 0));
            LVN_CK(launch_export(bl, 0, direct->dst[0], direct->cap[0], m->side));
        }
    }
    LVN_CK(cudaStreamWaitEvent(s0, m->ev_mesh, 0));
    BatchPtrs bs = b;
    bs.scatter_what = simp ? 0 : 2;
    // pinned host seams, 16-byte aligned: the seam pass writes them itself
    const bool fused_seams = pipelined && (reinterpret_cast<uintptr_t>(direct->dst[2]) & 15) == 0;
    if (fused_seams) {
        bs.host_seams = static_cast<int4*>(direct->dst[2]);
        bs.host_seam_cap = direct->cap[2];
    }
    LVN_CK(launch_mesh_scatter(bs, s0));
    if (simp) LVN_CK(launch_simplify(b, s0));
    if (direct) {
        if (simp) {
            const int rc = enqueue_exports(m, b, direct, s0);
            if (rc) return rc;
        } else {
            if (!fused_seams) LVN_CK(launch_export(b, 2, direct->dst[2], direct->cap[2], s0));
            if (!fused) {  // the side stream joined the DAG only for the sliced exports
                LVN_CK(cudaEventRecord(m->ev_side, m->side));
                LVN_CK(cudaStreamWaitEvent(s0, m->ev_side, 0));
            }
        }
    }
    return LVN_OK;
}

// Device addresses of caller arrays that are pinned (or registered) host
// memory, or of device memory; false when any array is pageable.
bool direct_addresses(const lvn_batch_out* out, DirectOut* d) {
    void* src[3] = {out->vertices, out->triangles, out->seams};
    const int64_t cap[3] = {out->vertex_capacity, out->triangle_capacity, out->seam_capacity};
    for (int i = 0; i < 3; i++) {
        d->cap[i] = cap[i];
        d->dst[i] = nullptr;
        if (!src[i]) {
            if (cap[i] > 0) return false;
            continue;
        }
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, src[i]) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost && a.type != cudaMemoryTypeDevice) return false;
        if (!a.devicePointer) return false;
        d->dst[i] = a.devicePointer;
    }
    return true;
}

int enqueue_state_readback(lvn_meshgen* m, int n) {
    LVN_CK(cudaMemcpyAsync(m->h_cs.p, m->cs.p, sizeof(ChunkState) * n, cudaMemcpyDeviceToHost, m->stream));
    LVN_CK(cudaMemcpyAsync(m->h_bs.p, m->bs.p, sizeof(BatchState), cudaMemcpyDeviceToHost, m->stream));
    return LVN_OK;
}

int finish_states(lvn_meshgen* m, int n) {
    LVN_CK(cudaStreamSynchronize(m->stream));
    m->last_n = n;
    m->last_cs.assign(m->h_cs.as<ChunkState>(), m->h_cs.as<ChunkState>() + n);
    return LVN_OK;
}

int read_states(lvn_meshgen* m, int n) {
    int rc = enqueue_state_readback(m, n);
    if (rc) return rc;
    return finish_states(m, n);
}

// Build the chunk descriptors of a batch of fresh chunks: density offset and
// sample scale (compute_density_field.cpp:146-149), LOD colour, the stored
// operations whose AABB overlaps the chunk (compute_density_field.cpp:255-265),
// and cuckoo parameters for its two tables.
int build_descs(lvn_meshgen* m, const lvn_chunk_desc* chunks, int n, std::vector<ChunkDesc>& descs,
                std::vector<Brush>& brushes, bool with_stored_ops) {
    descs.resize(n);
    brushes.clear();
    for (int c = 0; c < n; c++) {
        const lvn_chunk_desc& in = chunks[c];
        const int scale = in.size / (m->vpc * LEAF_SIZE_SCALE);
        if (scale <= 0 || in.size % (m->vpc * LEAF_SIZE_SCALE) != 0) return LVN_ERR_INVALID;
        ChunkDesc& d = descs[c];
        std::memset(&d, 0, sizeof(d));
        for (int i = 0; i < 3; i++) {
            d.off[i] = in.min[i] / LEAF_SIZE_SCALE;
            d.min[i] = in.min[i];
        }
        d.scale = scale;
        d.size = in.size;
        lod_colour(in.size / CLIPMAP_LEAF_SIZE, d.colour);
        d.op_begin = (int32_t)brushes.size();
        if (with_stored_ops) {
            const int32_t lo[3] = {in.min[0], in.min[1], in.min[2]};
            const int32_t hi[3] = {in.min[0] + in.size, in.min[1] + in.size, in.min[2] + in.size};
            for (const StoredOp& s : g.ops)
                if (overlaps(lo, hi, s.lo, s.hi)) brushes.push_back(make_brush(s.op));
        }
        d.op_count = (int32_t)brushes.size() - d.op_begin;
        csg_box(brushes.data() + d.op_begin, d.op_count, d.off, scale, m->vpc + 2, d.csg_lo, d.csg_hi);
        draw_params(d.edge_params);
        draw_params(d.node_params);
    }
    return LVN_OK;
}

// Host staging of a batch's descriptors and operations (pinned buffers).
int stage_inputs(lvn_meshgen* m, const std::vector<ChunkDesc>& descs, const std::vector<Brush>& brushes) {
    std::memcpy(m->h_desc.p, descs.data(), sizeof(ChunkDesc) * descs.size());
    const size_t nb = std::max<size_t>(brushes.size(), 1);
    LVN_CK(m->h_brushes.ensure(sizeof(Brush) * nb));
    LVN_CK(m->brushes.ensure(sizeof(Brush) * nb));
    if (!brushes.empty()) std::memcpy(m->h_brushes.p, brushes.data(), sizeof(Brush) * brushes.size());
    return LVN_OK;
}

// The copies of the staged inputs to the device (captured into batch graphs).
int enqueue_inputs(lvn_meshgen* m, int n, size_t n_brushes) {
    LVN_CK(cudaMemcpyAsync(m->desc.p, m->h_desc.p, sizeof(ChunkDesc) * n, cudaMemcpyHostToDevice, m->stream));
    if (n_brushes)
        LVN_CK(cudaMemcpyAsync(m->brushes.p, m->h_brushes.p, sizeof(Brush) * n_brushes, cudaMemcpyHostToDevice,
                               m->stream));
    return LVN_OK;
}

int upload(lvn_meshgen* m, const std::vector<ChunkDesc>& descs, const std::vector<Brush>& brushes) {
    int rc = stage_inputs(m, descs, brushes);
    if (rc) return rc;
    return enqueue_inputs(m, (int)descs.size(), brushes.size());
}

// Redraw cuckoo parameters for chunks whose insert failed (the reference
// retries with fresh parameters, compute_cuckoo.cpp:89-132).
bool redraw_failed(lvn_meshgen* m, std::vector<ChunkDesc>& descs) {
    bool any = false;
    const ChunkState* cs = m->h_cs.as<ChunkState>();
    for (size_t c = 0; c < descs.size(); c++) {
        if (cs[c].edge_insert_failed) { draw_params(descs[c].edge_params); any = true; }
        if (cs[c].node_insert_failed) { draw_params(descs[c].node_params); any = true; }
    }
    return any;
}

constexpr int kMaxHashRetries = 16;

// Learned-surrogate prologue of a fresh batch: probe every chunk, gate it,
// and evaluate the surrogate on the field lattices of the chunks that passed.
// Fills b's surrogate fields; the stages then read sdens for those chunks.
int surrogate_prologue(lvn_meshgen* m, const std::vector<ChunkDesc>& descs, size_t n_brushes, BatchPtrs& b) {
    const int n = (int)descs.size();
    const int FD = m->vpc + 2;
    const size_t F = (size_t)field_size(m->vpc);
    LVN_CK(m->probe_pts.ensure(sizeof(float4) * kProbes * n));
    LVN_CK(m->probe_plain.ensure(sizeof(float) * kProbes * n));
    LVN_CK(m->probe_s.ensure(sizeof(float) * kProbes * n));
    LVN_CK(m->gate_ok.ensure(sizeof(int) * n));
    LVN_CK(m->sslot.ensure(sizeof(int) * n));
    LVN_CK(m->h_gate.ensure(sizeof(int) * n));
    LVN_CK(m->h_sslot.ensure(sizeof(int) * n));
    b.s_on = 1;
    b.probe_pts = m->probe_pts.as<float4>();
    b.probe_plain = m->probe_plain.as<float>();
    b.probe_s = m->probe_s.as<float>();
    b.gate_ok = m->gate_ok.as<int>();
    b.gate = m->surrogate_gate;
    int rc = enqueue_inputs(m, n, n_brushes);
    if (rc) return rc;
    LVN_CK(launch_probe(b, m->stream));
    LVN_CK(cudaStreamSynchronize(m->stream));
    if ((rc = lvn_surrogate_eval(m->surrogate, m->probe_pts.as<float>(), (int64_t)kProbes * n, m->probe_s.as<float>(),
                                 LVN_MEMORY_DEVICE)))
        return rc;
    LVN_CK(launch_gate(b, m->stream));
    LVN_CK(cudaMemcpyAsync(m->h_gate.p, m->gate_ok.p, sizeof(int) * n, cudaMemcpyDeviceToHost, m->stream));
    LVN_CK(cudaStreamSynchronize(m->stream));
    float lo[3], hi[3];
    if ((rc = lvn_surrogate_domain(m->surrogate, lo, hi))) return rc;
    int32_t* slot = m->h_sslot.as<int32_t>();
    std::vector<float> lat;
    int k = 0;
    for (int c = 0; c < n; c++) {
        const ChunkDesc& d = descs[c];
        // x and z must lie in the domain; above and below its y range the
        // surrogate extrapolates (k_mlp_infer)
        bool inside = m->h_gate.as<int32_t>()[c] != 0;
        for (int a = 0; a < 3 && inside; a += 2)
            inside = (float)d.off[a] >= lo[a] && (float)(d.off[a] + d.scale * (FD - 1)) <= hi[a];
        slot[c] = inside ? k++ : -1;
        if (inside) lat.insert(lat.end(), {(float)d.off[0], (float)d.off[1], (float)d.off[2], (float)d.scale});
    }
    m->last_suse.assign(n, 0);
    for (int c = 0; c < n; c++) m->last_suse[c] = slot[c] >= 0;
    LVN_CK(cudaMemcpyAsync(m->sslot.p, slot, sizeof(int) * n, cudaMemcpyHostToDevice, m->stream));
    b.sslot = m->sslot.as<int>();
    if (k > 0) {
        LVN_CK(m->sdens.ensure(sizeof(float) * F * k));
        LVN_CK(m->lattices.ensure(sizeof(float) * lat.size()));
        LVN_CK(m->h_lattices.ensure(sizeof(float) * lat.size()));
        std::memcpy(m->h_lattices.p, lat.data(), sizeof(float) * lat.size());
        LVN_CK(cudaMemcpyAsync(m->lattices.p, m->h_lattices.p, sizeof(float) * lat.size(), cudaMemcpyHostToDevice,
                               m->stream));
        LVN_CK(cudaStreamSynchronize(m->stream));
        if ((rc = lvn_surrogate_eval_lattices(m->surrogate, m->lattices.as<float>(), k, FD, m->sdens.as<float>())))
            return rc;
        b.sdens = m->sdens.as<float>();
    }
    LVN_CK(cudaStreamSynchronize(m->stream));
    return LVN_OK;
}

// LVN_OPT_COMPUTE_ORDER: the ordered contexts' batches run their kernels one
// batch after another.  A batch's stream waits for the event recorded after
// the previous ordered batch's kernels (any context); the copy-engine
// transfers a batch enqueues after its kernels are not covered by that event,
// so they overlap the next batch's kernels instead of competing with them for
// SMs and L2.  The mutex makes "wait for the last, then become the last" one
// step across host threads.
std::mutex g_order_mutex;
cudaEvent_t g_order_last = nullptr;
const lvn_meshgen* g_order_owner = nullptr;

int order_begin(lvn_meshgen* m, std::unique_lock<std::mutex>& lock) {
    if (!m->compute_order) return LVN_OK;
    lock = std::unique_lock<std::mutex>(g_order_mutex);
    if (g_order_last && g_order_owner != m) LVN_CK(cudaStreamWaitEvent(m->stream, g_order_last, 0));
    return LVN_OK;
}

int order_end(lvn_meshgen* m) {  // the caller holds the lock order_begin took
    if (!m->compute_order) return LVN_OK;
    if (!m->ev_order) LVN_CK(cudaEventCreateWithFlags(&m->ev_order, cudaEventDisableTiming));
    LVN_CK(cudaEventRecord(m->ev_order, m->stream));
    g_order_last = m->ev_order;
    g_order_owner = m;
    return LVN_OK;
}

// Run fresh chunks end to end into the internal pools (or the caller's device
// buffers when `dev_out` is given).  Grows the pools and reruns once when a
// pool overflowed; retries the hash with new parameters when an insert failed.
int run_fresh_batch(lvn_meshgen* m, std::vector<ChunkDesc>& descs, const std::vector<Brush>& brushes,
                    const lvn_batch_out* dev_out, const DirectOut* direct = nullptr) {
    const int n = (int)descs.size();
    Capacity cap = default_capacity(m, n);
    cap.ecap = std::max(cap.ecap, m->ecap);
    cap.vcap = std::max(cap.vcap, m->vcap);
    int dag_hermite = 0;
    stage_shapes(m, tune_key(m, n), nullptr, &dag_hermite);
    m->dag_hermite_per_sm = dag_hermite;
    for (int attempt = 0; attempt < kMaxHashRetries + 2; attempt++) {
        int rc = ensure_pools(m, n, cap);
        if (rc) return rc;
        rc = stage_inputs(m, descs, brushes);
        if (rc) return rc;
        BatchPtrs b = make_ptrs(m, n);
        if (dev_out) {
            b.vertices = dev_out->vertices;
            b.vertex_cap = dev_out->vertex_capacity;
            b.triangles = dev_out->triangles;
            b.triangle_cap = dev_out->triangle_capacity;
            b.seams = dev_out->seams;
            b.seam_cap = dev_out->seam_capacity;
        }
        if (m->surrogate) {
            rc = surrogate_prologue(m, descs, brushes.size(), b);
            if (rc) return rc;
        }
        if (!m->aux) {
            LVN_CK(cudaStreamCreateWithFlags(&m->aux, cudaStreamNonBlocking));
            LVN_CK(cudaStreamCreateWithFlags(&m->aux2, cudaStreamNonBlocking));
            LVN_CK(cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming));
            LVN_CK(cudaEventCreateWithFlags(&m->ev_herm, cudaEventDisableTiming));
            LVN_CK(cudaEventCreateWithFlags(&m->ev_hash, cudaEventDisableTiming));
            LVN_CK(cudaEventCreateWithFlags(&m->ev_mesh, cudaEventDisableTiming));
        }
        auto enqueue_all = [&]() -> int {
            int r = enqueue_inputs(m, n, brushes.size());
            if (m->profile) {  // one stage at a time, each timed
                if (!r) r = enqueue_field_stages(m, b, !brushes.empty());
                if (!r) r = enqueue_octree_stages(m, b);
                if (!r && direct) r = enqueue_exports(m, b, direct, m->stream);
            } else if (!r) {
                r = enqueue_fresh_dag(m, b, !brushes.empty(), direct);
            }
            if (!r) r = enqueue_state_readback(m, n);
            return r;
        };
        if (m->use_graphs && !m->profile && !m->surrogate) {
            // N3: the batch is one graph launch; re-captured only when a
            // buffer, a capacity or the shape of the batch changes
            std::vector<uintptr_t> key = {(uintptr_t)n, (uintptr_t)brushes.size(), (uintptr_t)m->crossing_mode,
                                          (uintptr_t)g.density.mode, (uintptr_t)b.vertices, (uintptr_t)b.vertex_cap,
                                          (uintptr_t)b.triangles, (uintptr_t)b.triangle_cap, (uintptr_t)b.seams,
                                          (uintptr_t)b.seam_cap, (uintptr_t)b.ecap, (uintptr_t)b.vcap,
                                          (uintptr_t)b.edge_slot_cap, (uintptr_t)b.node_slot_cap,
                                          (uintptr_t)b.node_tile_cap, (uintptr_t)m->desc.p, (uintptr_t)m->brushes.p,
                                          (uintptr_t)m->mats.p, (uintptr_t)m->edge_keys.p, (uintptr_t)m->node_codes.p,
                                          (uintptr_t)m->edge_slots.p, (uintptr_t)m->node_slots.p,
                                          (uintptr_t)m->h_desc.p, (uintptr_t)m->h_brushes.p, (uintptr_t)m->h_cs.p,
                                          (uintptr_t)g.perm.p, (uintptr_t)(direct ? direct->dst[0] : nullptr),
                                          (uintptr_t)(direct ? direct->dst[1] : nullptr),
                                          (uintptr_t)(direct ? direct->dst[2] : nullptr),
                                          (uintptr_t)(direct ? direct->cap[0] : 0), (uintptr_t)(direct ? direct->cap[1] : 0),
                                          (uintptr_t)(direct ? direct->cap[2] : 0), (uintptr_t)g.default_material,
                                          (uintptr_t)b.simp_on, (uintptr_t)m->leaf_vertices.p, (uintptr_t)m->simp_nodes.p,
                                          (uintptr_t)m->simp_grid.p, (uintptr_t)m->simp_rep.p,
                                          (uintptr_t)m->simp_tile_counts.p};
            uint32_t thr_bits;
            std::memcpy(&thr_bits, &m->simp_threshold, 4);
            key.push_back(thr_bits);
            for (int st = 0; st < ST_COUNT; st++) key.push_back((uintptr_t)b.grid_per_sm[st]);
            key.push_back((uintptr_t)m->dag_hermite_per_sm);
            key.push_back((uintptr_t)b.hash_fault);
            key.push_back((uintptr_t)b.hermite_form);
            const uint32_t* dk = reinterpret_cast<const uint32_t*>(&g.density);
            for (size_t i = 0; i < sizeof(g.density) / 4; i++) key.push_back(dk[i]);
            if (!m->graph_exec || key != m->graph_key) {
                if (m->graph_exec) {
                    cudaGraphExecDestroy(m->graph_exec);
                    m->graph_exec = nullptr;
                }
                cudaGraph_t graph = nullptr;
                LVN_CK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
                const int r = enqueue_all();
                const cudaError_t ce = cudaStreamEndCapture(m->stream, &graph);
                if (r) {
                    if (graph) cudaGraphDestroy(graph);
                    return r;
                }
                LVN_CK(ce);
                const cudaError_t ie = cudaGraphInstantiate(&m->graph_exec, graph, 0);
                cudaGraphDestroy(graph);
                LVN_CK(ie);
                m->graph_key = key;
            }
            std::unique_lock<std::mutex> order;
            if ((rc = order_begin(m, order))) return rc;
            LVN_CK(cudaGraphLaunch(m->graph_exec, m->stream));
            if ((rc = order_end(m))) return rc;
        } else {
            std::unique_lock<std::mutex> order;
            if ((rc = order_begin(m, order))) return rc;
            rc = enqueue_all();
            if (!rc) rc = order_end(m);
            if (rc) return rc;
        }
        rc = finish_states(m, n);
        if (rc) return rc;
        m->last_fresh = true;
        m->last_desc = descs;
        const BatchState& bs = *m->h_bs.as<BatchState>();
        if (direct && bs.status) return LVN_ERR_CAPACITY;  // a caller array was too small
        if (bs.overflow) {
            const bool user_short = dev_out && ((bs.overflow & (OVF_QUADS | OVF_SEAMS)) ||
                                                ((bs.overflow & OVF_NODES) && bs.total_nodes > b.vertex_cap &&
                                                 bs.total_nodes <= b.vcap));
            if (user_short) return LVN_ERR_CAPACITY;
            // grow to the sizes this run reported and try again
            cap.ecap = std::max<int64_t>(cap.ecap, (int64_t)bs.total_edges + 1024);
            if (bs.overflow & OVF_EDGE_SLOTS) cap.ecap = std::max<int64_t>(cap.ecap, bs.total_edge_slots);
            if (bs.overflow & (OVF_NODES | OVF_NODE_SLOTS | OVF_QUADS | OVF_SEAMS))
                cap.vcap = std::max<int64_t>(cap.vcap * 2, (int64_t)bs.total_nodes + 1024);
            if (bs.overflow & OVF_EDGES) cap.ecap = std::max<int64_t>(cap.ecap * 2, (int64_t)bs.total_edges + 1024);
            continue;
        }
        if (redraw_failed(m, descs)) continue;
        return LVN_OK;
    }
    return LVN_ERR_HASH;
}

void fill_results(lvn_meshgen* m, int n, lvn_chunk_result* r) {
    const ChunkState* cs = m->h_cs.as<ChunkState>();
    const bool simp = m->simp_threshold >= 0.f;
    for (int c = 0; c < n; c++) {
        if (simp) {
            r[c].vertex_offset = cs[c].simp_vert_off;
            r[c].num_vertices = cs[c].simp_tris > 0 ? cs[c].simp_verts : 0;
            r[c].triangle_offset = cs[c].simp_tri_off;
            r[c].num_triangles = cs[c].simp_tris;
        } else {
            r[c].vertex_offset = cs[c].node_off;
            r[c].num_vertices = cs[c].quads > 0 ? cs[c].nodes : 0;
            r[c].triangle_offset = 2 * cs[c].quad_off;
            r[c].num_triangles = 2 * cs[c].quads;
        }
        r[c].seam_offset = cs[c].seam_off;
        r[c].num_seams = cs[c].seams;
        r[c].num_edges = cs[c].num_edges;
        r[c].num_nodes = cs[c].nodes;
    }
}

int copy_out(lvn_meshgen* m, void* dst, const void* src, size_t bytes, int memory) {
    if (bytes == 0) return LVN_OK;
    LVN_CK(cudaMemcpyAsync(dst, src, bytes, memory == LVN_MEMORY_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                           m->stream));
    return LVN_OK;
}

// ---- cached single-chunk path ---------------------------------------------

ChunkKey key_of(const int32_t min[3], int32_t size) { return ChunkKey(min[0], min[1], min[2], size); }

int one_desc(lvn_meshgen* m, const int32_t min[3], int32_t size, std::vector<ChunkDesc>& descs) {
    lvn_chunk_desc cd;
    for (int i = 0; i < 3; i++) cd.min[i] = min[i];
    cd.size = size;
    std::vector<Brush> none;
    return build_descs(m, &cd, 1, descs, none, false);
}

// Copy the pool state of chunk 0 (corners + edge list) into a field entry.
int save_field(lvn_meshgen* m, FieldEntry& f) {
    const ChunkState& cs = m->last_cs[0];
    const size_t F = (size_t)field_size(m->vpc);
    const size_t PB = sizeof(uint4) * 3 * (size_t)field_rows(m->vpc);
    LVN_CK(f.mats.ensure(F));
    LVN_CK(f.planes.ensure(PB));
    LVN_CK(cudaMemcpyAsync(f.mats.p, m->mats.p, F, cudaMemcpyDeviceToDevice, m->stream));
    LVN_CK(cudaMemcpyAsync(f.planes.p, m->planes.p, PB, cudaMemcpyDeviceToDevice, m->stream));
    f.num_edges = cs.num_edges;
    LVN_CK(f.keys.ensure(sizeof(int32_t) * std::max(1, cs.num_edges)));
    LVN_CK(f.info.ensure(sizeof(float4) * std::max(1, cs.num_edges)));
    LVN_CK(cudaMemcpyAsync(f.keys.p, m->edge_keys.p, sizeof(int32_t) * cs.num_edges, cudaMemcpyDeviceToDevice,
                           m->stream));
    LVN_CK(cudaMemcpyAsync(f.info.p, m->edge_info.p, sizeof(float4) * cs.num_edges, cudaMemcpyDeviceToDevice,
                           m->stream));
    LVN_CK(cudaStreamSynchronize(m->stream));
    return LVN_OK;
}

// GenerateDefaultDensityField + FindDefaultEdges (compute_density_field.cpp:138-231)
int generate_field(lvn_meshgen* m, const int32_t min[3], int32_t size, FieldEntry& f) {
    std::vector<ChunkDesc> descs;
    int rc = one_desc(m, min, size, descs);
    if (rc) return rc;
    Capacity cap = default_capacity(m, 1);
    cap.ecap = std::max(cap.ecap, m->ecap);
    cap.vcap = std::max(cap.vcap, m->vcap);
    if ((rc = ensure_pools(m, 1, cap))) return rc;
    std::vector<Brush> none;
    if ((rc = upload(m, descs, none))) return rc;
    BatchPtrs b = make_ptrs(m, 1);
    b.need_mats = 1;  // a cached field keeps every byte material
    b.derive_mats = 0;
    if ((rc = enqueue_field_stages(m, b, false))) return rc;
    if ((rc = read_states(m, 1))) return rc;
    m->last_fresh = false;
    if (m->h_bs.as<BatchState>()->overflow) return LVN_ERR_DEVICE_STATUS;
    f.last_op = 0;
    return save_field(m, f);
}

// ApplyCSGOperations on a cached field (compute_csg.cpp:11-219)
int apply_csg_to_field(lvn_meshgen* m, const int32_t min[3], int32_t size, FieldEntry& f,
                       const std::vector<lvn_csg_op>& ops) {
    if (ops.empty()) return LVN_OK;
    std::vector<ChunkDesc> descs;
    int rc = one_desc(m, min, size, descs);
    if (rc) return rc;
    std::vector<Brush> brushes;
    for (const lvn_csg_op& op : ops) brushes.push_back(make_brush(op));
    descs[0].op_begin = 0;
    descs[0].op_count = (int32_t)brushes.size();
    csg_box(brushes.data(), descs[0].op_count, descs[0].off, descs[0].scale, m->vpc + 2, descs[0].csg_lo,
            descs[0].csg_hi);
    Capacity cap = default_capacity(m, 1);
    cap.ecap = std::max<int64_t>(std::max(cap.ecap, m->ecap), (int64_t)f.num_edges + 3 * field_size(m->vpc));
    cap.vcap = std::max(cap.vcap, m->vcap);
    if ((rc = ensure_pools(m, 1, cap))) return rc;
    if ((rc = upload(m, descs, brushes))) return rc;
    const size_t F = (size_t)field_size(m->vpc);
    const size_t R = (size_t)field_rows(m->vpc);
    LVN_CK(cudaMemcpyAsync(m->mats.p, f.mats.p, F, cudaMemcpyDeviceToDevice, m->stream));
    LVN_CK(cudaMemcpyAsync(m->planes.p, f.planes.p, sizeof(uint4) * 2 * R, cudaMemcpyDeviceToDevice, m->stream));
    // no corner is changed by this batch until the CSG kernel says so
    LVN_CK(cudaMemsetAsync(m->planes.as<uint4>() + 2 * R, 0, sizeof(uint4) * R, m->stream));
    BatchPtrs b = make_ptrs(m, 1);
    b.plain_class = 0;
    b.need_mats = 1;
    b.derive_mats = 0;
    b.hmap = nullptr;  // no field kernel runs here: nothing to share
    b.prev_keys = f.keys.as<int32_t>();
    b.prev_info = f.info.as<float4>();
    b.prev_count = f.num_edges;
    LVN_CK(launch_reset(b, m->stream));
    if ((rc = stage(m, ST_CSG, launch_csg, b))) return rc;
    LVN_CK(launch_prune_edges(b, m->stream));
    if ((rc = stage(m, ST_EDGE_COUNT, launch_edge_count, b))) return rc;
    if ((rc = stage(m, ST_EDGE_PLAN, launch_edge_plan, b))) return rc;
    if ((rc = stage(m, ST_EDGE_SCATTER, launch_edge_scatter, b))) return rc;
    if ((rc = stage(m, ST_HERMITE, launch_hermite, b))) return rc;
    if ((rc = read_states(m, 1))) return rc;
    m->last_fresh = false;
    if (m->h_bs.as<BatchState>()->overflow) return LVN_ERR_DEVICE_STATUS;
    return save_field(m, f);
}

// LoadDensityField (compute_density_field.cpp:235-274)
int load_field(lvn_meshgen* m, const int32_t min[3], int32_t size, FieldEntry** out) {
    const ChunkKey k = key_of(min, size);
    auto it = m->fields.find(k);
    FieldEntry* f;
    if (it != m->fields.end()) {
        f = &it->second;
    } else {
        FieldEntry fresh;
        int rc = generate_field(m, min, size, fresh);
        if (rc) {
            fresh.mats.release();
            fresh.planes.release();
            fresh.keys.release();
            fresh.info.release();
            return rc;
        }
        f = &m->fields.emplace(k, std::move(fresh)).first->second;
    }
    const int32_t lo[3] = {min[0], min[1], min[2]};
    const int32_t hi[3] = {min[0] + size, min[1] + size, min[2] + size};
    std::vector<lvn_csg_op> replay;
    for (size_t i = (size_t)std::max(0, f->last_op); i < g.ops.size(); i++)
        if (overlaps(lo, hi, g.ops[i].lo, g.ops[i].hi)) replay.push_back(g.ops[i].op);
    f->last_op = (int32_t)g.ops.size();
    *out = f;
    if (!replay.empty()) return apply_csg_to_field(m, min, size, *f, replay);
    return LVN_OK;
}

// ConstructOctreeFromField + mesh + seams for one cached field
int mesh_from_field(lvn_meshgen* m, const int32_t min[3], int32_t size, FieldEntry& f) {
    std::vector<ChunkDesc> descs;
    int rc = one_desc(m, min, size, descs);
    if (rc) return rc;
    std::vector<Brush> none;
    Capacity cap = default_capacity(m, 1);
    cap.ecap = std::max<int64_t>(std::max(cap.ecap, m->ecap), (int64_t)f.num_edges + 1024);
    cap.vcap = std::max(cap.vcap, m->vcap);
    for (int attempt = 0; attempt < kMaxHashRetries; attempt++) {
        if ((rc = ensure_pools(m, 1, cap))) return rc;
        if ((rc = upload(m, descs, none))) return rc;
        const size_t F = (size_t)field_size(m->vpc);
        LVN_CK(cudaMemcpyAsync(m->mats.p, f.mats.p, F, cudaMemcpyDeviceToDevice, m->stream));
        LVN_CK(cudaMemcpyAsync(m->planes.p, f.planes.p, sizeof(uint4) * 3 * (size_t)field_rows(m->vpc),
                               cudaMemcpyDeviceToDevice, m->stream));
        LVN_CK(cudaMemcpyAsync(m->edge_keys.p, f.keys.p, sizeof(int32_t) * f.num_edges, cudaMemcpyDeviceToDevice,
                               m->stream));
        LVN_CK(cudaMemcpyAsync(m->edge_info.p, f.info.p, sizeof(float4) * f.num_edges, cudaMemcpyDeviceToDevice,
                               m->stream));
        LVN_CK(cudaMemsetAsync(m->edge_chunk.p, 0, sizeof(int32_t) * std::max(1, f.num_edges), m->stream));
        ChunkState cs;
        std::memset(&cs, 0, sizeof(cs));
        cs.plain_edges = f.num_edges;
        cs.num_edges = f.num_edges;
        cs.edge_prime = 0;
        if (f.num_edges > 0) {
            // FindNextPrime on the host for the cached path
            cs.edge_prime = (uint32_t)host_next_prime(std::max((int)CUCKOO_MIN_TABLE_SIZE, f.num_edges * 2));
        }
        BatchState bs;
        std::memset(&bs, 0, sizeof(bs));
        bs.total_edges = f.num_edges;
        bs.total_edge_slots = cs.edge_prime ? cs.edge_prime + CUCKOO_STASH_SIZE : 0;
        if (bs.total_edge_slots > m->eslot_cap) {
            cap.ecap = std::max<int64_t>(cap.ecap, bs.total_edge_slots);
            continue;
        }
        std::memcpy(m->h_cs.p, &cs, sizeof(cs));
        std::memcpy(m->h_bs.p, &bs, sizeof(bs));
        LVN_CK(cudaMemcpyAsync(m->cs.p, m->h_cs.p, sizeof(cs), cudaMemcpyHostToDevice, m->stream));
        LVN_CK(cudaMemcpyAsync(m->bs.p, m->h_bs.p, sizeof(bs), cudaMemcpyHostToDevice, m->stream));
        BatchPtrs b = make_ptrs(m, 1);
        b.derive_mats = 0;  // the cached field may hold CSG materials
        if ((rc = enqueue_octree_stages(m, b))) return rc;
        if ((rc = read_states(m, 1))) return rc;
        m->last_fresh = false;
        const BatchState& hb = *m->h_bs.as<BatchState>();
        if (hb.overflow) {
            cap.vcap = std::max<int64_t>(cap.vcap * 2, (int64_t)hb.total_nodes + 1024);
            continue;
        }
        if (redraw_failed(m, descs)) continue;
        return LVN_OK;
    }
    return LVN_ERR_HASH;
}

int export_chunk(lvn_meshgen* m, const OctreeEntry& o, lvn_mesh_out* out) {
    out->num_vertices = o.num_vertices;
    out->num_triangles = (int32_t)o.triangles.size();
    out->num_seams = (int32_t)o.seams.size();
    if (out->num_vertices > out->vertex_capacity || out->num_triangles > out->triangle_capacity ||
        out->num_seams > out->seam_capacity)
        return LVN_ERR_CAPACITY;
    const cudaMemcpyKind kind = out->memory == LVN_MEMORY_DEVICE ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
    if (out->num_vertices)
        LVN_CK(cudaMemcpy(out->vertices, o.vertices.data(), sizeof(lvn_mesh_vertex) * out->num_vertices, kind));
    if (out->num_triangles)
        LVN_CK(cudaMemcpy(out->triangles, o.triangles.data(), sizeof(lvn_mesh_triangle) * out->num_triangles, kind));
    if (out->num_seams) LVN_CK(cudaMemcpy(out->seams, o.seams.data(), sizeof(lvn_seam_node) * out->num_seams, kind));
    return LVN_OK;
}

// Pull chunk 0's mesh out of the pools into host vectors.
int pull_chunk(lvn_meshgen* m, OctreeEntry& o) {
    const ChunkState& cs = m->last_cs[0];
    const bool simp = m->simp_threshold >= 0.f;
    const int ntri = simp ? cs.simp_tris : 2 * cs.quads;
    o.num_vertices = ntri > 0 ? (simp ? cs.simp_verts : cs.nodes) : 0;
    o.vertices.resize(o.num_vertices);
    o.triangles.resize((size_t)ntri);
    o.seams.resize(cs.seams);
    if (o.num_vertices)
        LVN_CK(cudaMemcpyAsync(o.vertices.data(),
                               m->vertices.as<lvn_mesh_vertex>() + (simp ? cs.simp_vert_off : cs.node_off),
                               sizeof(lvn_mesh_vertex) * o.num_vertices, cudaMemcpyDeviceToHost, m->stream));
    if (ntri)
        LVN_CK(cudaMemcpyAsync(o.triangles.data(),
                               m->triangles.as<lvn_mesh_triangle>() + (simp ? (size_t)cs.simp_tri_off : 2 * (size_t)cs.quad_off),
                               sizeof(lvn_mesh_triangle) * o.triangles.size(), cudaMemcpyDeviceToHost, m->stream));
    if (cs.seams)
        LVN_CK(cudaMemcpyAsync(o.seams.data(), m->seams.as<lvn_seam_node>() + cs.seam_off,
                               sizeof(lvn_seam_node) * cs.seams, cudaMemcpyDeviceToHost, m->stream));
    LVN_CK(cudaStreamSynchronize(m->stream));
    return LVN_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

int lvn_initialise(int32_t noise_seed, uint32_t default_material, int32_t num_csg_brushes) {
    (void)num_csg_brushes;  // the brush set is fixed: cube and sphere (apply_csg_operation.cl:76-78)
    if (default_material > 255) return LVN_ERR_INVALID;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return LVN_ERR_NO_DEVICE;
    LVN_CK(cudaGetDevice(&g.device));
    LVN_CK(cudaDeviceGetAttribute(&g.num_sms, cudaDevAttrMultiProcessorCount, g.device));
    LVN_CK(set_kernel_attributes());
    g.default_material = (int32_t)default_material;
    g.hash_gen = std::mt19937();
    const int rc = upload_perm(noise_seed);
    if (rc) return rc;
    g.initialised = true;
    return LVN_OK;
}

int lvn_shutdown(void) {
    g.perm.release();
    g.perm_t3.release();
    g.grad.release();
    g.ops.clear();
    g.initialised = false;
    return LVN_OK;
}

int lvn_set_noise_seed(int32_t noise_seed) {
    if (!g.initialised) return LVN_ERR_NOT_INITIALISED;
    return upload_perm(noise_seed);
}

int lvn_store_csg_operation(const lvn_csg_op* op, const int32_t aabb_min[3], const int32_t aabb_max[3]) {
    if (!op || !aabb_min || !aabb_max || !valid_op(*op)) return LVN_ERR_INVALID;
    StoredOp s;
    s.op = *op;
    for (int i = 0; i < 3; i++) {
        s.lo[i] = aabb_min[i];
        s.hi[i] = aabb_max[i];
    }
    g.ops.push_back(s);
    return LVN_OK;
}

int lvn_clear_csg_operations(void) {
    g.ops.clear();
    return LVN_OK;
}

int lvn_csg_operation_bounds(const lvn_csg_op* op, int32_t aabb_min[3], int32_t aabb_max[3]) {
    if (!op || !aabb_min || !aabb_max) return LVN_ERR_INVALID;
    op_bounds(*op, aabb_min, aabb_max);
    return LVN_OK;
}

int lvn_set_density(const lvn_density_params* p) {
    if (!p || p->mode < LVN_DENSITY_REFERENCE || p->mode > LVN_DENSITY_CAVES || p->octaves2 < 0 || p->octaves2 > 32 ||
        p->octaves3 < 0 || p->octaves3 > 32)
        return LVN_ERR_INVALID;
    g.density = *p;
    return LVN_OK;
}

const char* lvn_error_string(int32_t code) {
    switch (code) {
        case LVN_OK: return "LVN_OK";
        case LVN_ERR_NO_DEVICE: return "LVN_ERR_NO_DEVICE";
        case LVN_ERR_OUT_OF_MEMORY: return "LVN_ERR_OUT_OF_MEMORY";
        case LVN_ERR_INVALID: return "LVN_ERR_INVALID";
        case LVN_ERR_CAPACITY: return "LVN_ERR_CAPACITY";
        case LVN_ERR_NOT_INITIALISED: return "LVN_ERR_NOT_INITIALISED";
        case LVN_ERR_HASH: return "LVN_ERR_HASH";
        case LVN_ERR_DEVICE_STATUS: return "LVN_ERR_DEVICE_STATUS";
        case LVN_ERR_CUDA: return "LVN_ERR_CUDA";
        default: return "unknown liblvn error code";
    }
}

lvn_meshgen* lvn_meshgen_create(int32_t voxels_per_chunk) {
    if (!g.initialised) return nullptr;
    if (voxels_per_chunk != 8 && voxels_per_chunk != 16 && voxels_per_chunk != 32 && voxels_per_chunk != 64)
        return nullptr;
    lvn_meshgen* m = new lvn_meshgen();
    m->vpc = voxels_per_chunk;
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete m;
        return nullptr;
    }
    m->own_stream = true;
    for (int i = 0; i <= ST_COUNT; i++) cudaEventCreate(&m->ev[i]);
    return m;
}

void lvn_meshgen_destroy(lvn_meshgen* m) {
    if (!m) return;
    lvn_meshgen_wait(m);
    cudaStreamSynchronize(m->stream);
    {
        std::lock_guard<std::mutex> lock(g_order_mutex);
        if (g_order_owner == m) {
            g_order_last = nullptr;
            g_order_owner = nullptr;
        }
    }
    if (m->ev_order) cudaEventDestroy(m->ev_order);
    DevBuf* bufs[] = {&m->desc,       &m->cs,         &m->bs,         &m->brushes,      &m->mats,  &m->planes, &m->hmap,
                      &m->edge_tiles, &m->vox_tiles,  &m->edge_keys,  &m->edge_chunk,   &m->edge_info, &m->edge_work,
                      &m->node_codes, &m->node_info,  &m->node_chunk, &m->edge_slots,   &m->node_slots,
                      &m->quad_scratch, &m->node_tile_counts, &m->chunk_tile_off, &m->vertices, &m->triangles,
                      &m->seams, &m->leaf_vertices, &m->leaf_qef, &m->simp_grid, &m->simp_nodes, &m->simp_count,
                      &m->simp_rep, &m->simp_entry, &m->simp_newidx, &m->simp_mask, &m->simp_tile_counts,
                      &m->probe_pts, &m->probe_plain, &m->probe_s, &m->gate_ok, &m->sslot, &m->sdens, &m->lattices};
    for (DevBuf* b : bufs) b->release();
    m->h_desc.release();
    m->h_brushes.release();
    m->h_cs.release();
    m->h_bs.release();
    m->h_gate.release();
    m->h_sslot.release();
    m->h_lattices.release();
    for (auto& kv : m->fields) {
        kv.second.mats.release();
        kv.second.planes.release();
        kv.second.keys.release();
        kv.second.info.release();
    }
    for (int i = 0; i <= ST_COUNT; i++)
        if (m->ev[i]) cudaEventDestroy(m->ev[i]);
    if (m->graph_exec) cudaGraphExecDestroy(m->graph_exec);
    if (m->ev_fork) cudaEventDestroy(m->ev_fork);
    if (m->ev_hash) cudaEventDestroy(m->ev_hash);
    if (m->ev_mesh) cudaEventDestroy(m->ev_mesh);
    if (m->aux2) cudaStreamDestroy(m->aux2);
    if (m->ev_leaf) cudaEventDestroy(m->ev_leaf);
    if (m->ev_side) cudaEventDestroy(m->ev_side);
    if (m->side) cudaStreamDestroy(m->side);
    if (m->ev_herm) cudaEventDestroy(m->ev_herm);
    if (m->aux) cudaStreamDestroy(m->aux);
    if (m->own_stream) cudaStreamDestroy(m->stream);
    delete m;
}

int lvn_meshgen_voxels_per_chunk(const lvn_meshgen* m) { return m ? m->vpc : 0; }

int lvn_meshgen_set_stream(lvn_meshgen* m, void* stream) {
    if (!m) return LVN_ERR_INVALID;
    LVN_CK(cudaStreamSynchronize(m->stream));
    if (m->own_stream) cudaStreamDestroy(m->stream);
    m->stream = static_cast<cudaStream_t>(stream);
    m->own_stream = false;
    return LVN_OK;
}

void* lvn_meshgen_get_stream(lvn_meshgen* m) { return m ? (void*)m->stream : nullptr; }

int lvn_meshgen_set_option(lvn_meshgen* m, int32_t option, int32_t value) {
    if (!m) return LVN_ERR_INVALID;
    switch (option) {
        case LVN_OPT_CROSSING_MODE:
            if (value != 0 && value != 1) return LVN_ERR_INVALID;
            m->crossing_mode = value;
            return LVN_OK;
        case LVN_OPT_CACHE: m->cache = value != 0; return LVN_OK;
        case LVN_OPT_PROFILE: m->profile = value != 0; return LVN_OK;
        case LVN_OPT_GRAPHS: m->use_graphs = value != 0; return LVN_OK;
        case LVN_OPT_HOST_WRITES: m->host_writes = value != 0; return LVN_OK;
        case LVN_OPT_COMPUTE_ORDER: m->compute_order = value != 0; return LVN_OK;
        case LVN_OPT_HERMITE_FORM:
            if (value < 0 || value > 2) return LVN_ERR_INVALID;
            m->hermite_form = value;
            return LVN_OK;
        default: return LVN_ERR_INVALID;
    }
}

int lvn_meshgen_stage_times(lvn_meshgen* m, float* ms, int32_t* launches, int32_t capacity) {
    if (!m) return LVN_ERR_INVALID;
    for (int i = 0; i < ST_COUNT && i < capacity; i++) {
        if (ms) ms[i] = (float)m->stage_ms[i];
        if (launches) launches[i] = m->stage_launches[i];
    }
    return ST_COUNT;
}

const char* lvn_meshgen_stage_name(int32_t s) { return stage_name(s); }

// N3 autotuner: times the batch's persistent-grid stages at 2..32 CTAs per SM
// and keeps each stage's fastest shape for batches of this kind.
int lvn_meshgen_autotune(lvn_meshgen* m, const lvn_chunk_desc* chunks, int32_t n, int32_t* grid_per_sm) {
    if (!g.initialised) return LVN_ERR_NOT_INITIALISED;
    if (!m || n <= 0 || !chunks || n > 65535) return LVN_ERR_INVALID;
    std::vector<ChunkDesc> descs;
    std::vector<Brush> brushes;
    int rc = build_descs(m, chunks, n, descs, brushes, true);
    if (rc) return rc;
    const auto key = tune_key(m, n);
    const bool profile = m->profile;
    double saved_ms[ST_COUNT];
    int saved_launches[ST_COUNT];
    std::memcpy(saved_ms, m->stage_ms, sizeof(saved_ms));
    std::memcpy(saved_launches, m->stage_launches, sizeof(saved_launches));
    m->profile = true;
    m->tuning = true;
    m->tunes.clear();
    m->dag_tunes.clear();
    static const int kCandidates[] = {2, 4, 8, 16, 32};
    constexpr int kCand = sizeof(kCandidates) / sizeof(kCandidates[0]);
    constexpr int kRounds = 3;
    auto shape_of = [](int cand) {
        std::array<int, ST_COUNT> shape{};
        for (int st = 0; st < ST_COUNT; st++) shape[st] = stage_has_persistent_grid(st) ? cand : 0;
        return shape;
    };
    // Warm-up runs size the pools and bring the SM clock up before anything is
    // timed.  The candidates are then timed in turn, round after round, and
    // each keeps its fastest run: a clock ramp or a cache warming up during the
    // tuning spreads over every candidate instead of favouring the last ones.
    m->tunes[key] = shape_of(kCandidates[0]);
    for (int rep = 0; rep < 3 && rc == LVN_OK; rep++) rc = run_fresh_batch(m, descs, brushes, nullptr);
    std::array<std::array<double, ST_COUNT>, kCand> ms;
    for (auto& a : ms) a.fill(1e30);
    for (int round = 0; round < kRounds && rc == LVN_OK; round++) {
        for (int k = 0; k < kCand && rc == LVN_OK; k++) {
            m->tunes[key] = shape_of(kCandidates[k]);
            for (int st = 0; st < ST_COUNT; st++) m->stage_ms[st] = 0.0, m->stage_launches[st] = 0;
            rc = run_fresh_batch(m, descs, brushes, nullptr);
            for (int st = 0; st < ST_COUNT; st++)
                if (m->stage_launches[st]) ms[k][st] = std::min(ms[k][st], m->stage_ms[st]);
        }
    }
    std::array<double, ST_COUNT> best_ms;
    std::array<int, ST_COUNT> best{};
    best_ms.fill(1e30);
    for (int k = 0; k < kCand && rc == LVN_OK; k++)
        for (int st = 0; st < ST_COUNT; st++)
            if (stage_has_persistent_grid(st) && ms[k][st] < best_ms[st]) {
                best_ms[st] = ms[k][st];
                best[st] = kCandidates[k];
            }
    m->profile = profile;
    std::memcpy(m->stage_ms, saved_ms, sizeof(saved_ms));
    std::memcpy(m->stage_launches, saved_launches, sizeof(saved_launches));
    if (rc) {
        m->tuning = false;
        return rc;
    }
    m->tunes[key] = best;
    // hermite shares the GPU with the voxel / hash / quad chain in the batch
    // DAG: its grid is chosen by the time of the whole batch graph.  A change
    // of shape re-captures the graph, so each candidate's first run in a round
    // (the capture) is not timed; candidates again take turns, round by round.
    std::array<double, kCand> total;
    total.fill(1e30);
    for (int round = 0; round < kRounds && rc == LVN_OK; round++) {
        for (int k = 0; k < kCand && rc == LVN_OK; k++) {
            m->dag_tunes[key] = kCandidates[k];
            rc = run_fresh_batch(m, descs, brushes, nullptr);
            if (rc) break;
            const auto t0 = std::chrono::steady_clock::now();
            rc = run_fresh_batch(m, descs, brushes, nullptr);
            const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            total[k] = std::min(total[k], dt);
        }
    }
    double best_total = 1e30;
    int best_h = 0;
    for (int k = 0; k < kCand && rc == LVN_OK; k++)
        if (total[k] < best_total) {
            best_total = total[k];
            best_h = kCandidates[k];
        }
    m->tuning = false;
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tunes[key] = Tuned{best, best_h};
    }
    if (grid_per_sm) {
        for (int st = 0; st < ST_COUNT; st++) grid_per_sm[st] = best[st];
        grid_per_sm[ST_HERMITE] = best_h;  // the shape used in batches
    }
    return LVN_OK;
}

int lvn_meshgen_set_surrogate(lvn_meshgen* m, lvn_surrogate* s, float gate) {
    if (!m || !(gate >= 0.f)) return LVN_ERR_INVALID;
    LVN_CK(cudaStreamSynchronize(m->stream));
    m->surrogate = s;
    m->surrogate_gate = gate;
    m->octrees.clear();
    m->fields.clear();
    return LVN_OK;
}

int lvn_meshgen_surrogate_chunks(lvn_meshgen* m, int32_t* use, int32_t capacity) {
    if (!m) return LVN_ERR_INVALID;
    int count = 0;
    for (size_t c = 0; c < m->last_suse.size(); c++) {
        if (use && (int32_t)c < capacity) use[c] = m->last_suse[c];
        count += m->last_suse[c];
    }
    return count;
}

int lvn_meshgen_set_simplify(lvn_meshgen* m, float threshold) {
    if (!m || threshold != threshold) return LVN_ERR_INVALID;
    LVN_CK(cudaStreamSynchronize(m->stream));
    m->simp_threshold = threshold < 0.f ? -1.f : threshold;
    m->octrees.clear();  // cached meshes were made with the previous setting
    return LVN_OK;
}

int lvn_meshgen_reset_stage_times(lvn_meshgen* m) {
    if (!m) return LVN_ERR_INVALID;
    for (int i = 0; i < ST_COUNT; i++) {
        m->stage_ms[i] = 0.0;
        m->stage_launches[i] = 0;
    }
    return LVN_OK;
}

int lvn_meshgen_generate_chunks(lvn_meshgen* m, const lvn_chunk_desc* chunks, int32_t n, lvn_batch_out* out) {
    if (!g.initialised) return LVN_ERR_NOT_INITIALISED;
    if (!m || !out || n < 0 || (n > 0 && !chunks)) return LVN_ERR_INVALID;
    if (n > 65535) return LVN_ERR_INVALID;
    if (n == 0) {
        out->total_vertices = out->total_triangles = out->total_seams = 0;
        return LVN_OK;
    }
    std::vector<ChunkDesc> descs;
    std::vector<Brush> brushes;
    int rc = build_descs(m, chunks, n, descs, brushes, true);
    if (rc) return rc;
    const bool dev = out->memory == LVN_MEMORY_DEVICE;
    DirectOut direct;
    const bool use_direct = !dev && m->host_writes && direct_addresses(out, &direct);
    if (use_direct && !m->side) {
        // exports take free SM slots ahead of the compute kernels they overlap
        int lo = 0, hi = 0;
        LVN_CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        LVN_CK(cudaStreamCreateWithPriority(&m->side, cudaStreamNonBlocking, hi));
        LVN_CK(cudaEventCreateWithFlags(&m->ev_leaf, cudaEventDisableTiming));
        LVN_CK(cudaEventCreateWithFlags(&m->ev_side, cudaEventDisableTiming));
    }
    rc = run_fresh_batch(m, descs, brushes, dev ? out : nullptr, use_direct ? &direct : nullptr);
    out->total_vertices = out->total_triangles = out->total_seams = 0;
    if (m->h_bs.p) {  // absent when the first pool allocation failed
        const BatchState& bs = *m->h_bs.as<BatchState>();
        const bool simp = m->simp_threshold >= 0.f;
        out->total_vertices = simp ? bs.total_simp_verts : bs.total_nodes;
        out->total_triangles = simp ? bs.total_simp_tris : 2 * (int64_t)bs.total_quads;
        out->total_seams = bs.total_seams;
    }
    if (rc) return rc;
    if (out->chunks) fill_results(m, n, out->chunks);
    if (!dev && !use_direct) {
        if (out->total_vertices > out->vertex_capacity || out->total_triangles > out->triangle_capacity ||
            out->total_seams > out->seam_capacity)
            return LVN_ERR_CAPACITY;
        if ((rc = copy_out(m, out->vertices, m->vertices.p, sizeof(lvn_mesh_vertex) * out->total_vertices, 0))) return rc;
        if ((rc = copy_out(m, out->triangles, m->triangles.p, sizeof(lvn_mesh_triangle) * out->total_triangles, 0)))
            return rc;
        if ((rc = copy_out(m, out->seams, m->seams.p, sizeof(lvn_seam_node) * out->total_seams, 0))) return rc;
        LVN_CK(cudaStreamSynchronize(m->stream));
    }
    return LVN_OK;
}

int lvn_meshgen_generate_chunks_async(lvn_meshgen* m, const lvn_chunk_desc* chunks, int32_t n, lvn_batch_out* out) {
    if (!g.initialised) return LVN_ERR_NOT_INITIALISED;
    if (!m || !out || n < 0 || (n > 0 && !chunks) || n > 65535) return LVN_ERR_INVALID;
    if (m->async_active) return LVN_ERR_INVALID;  // one batch in flight per context
    m->async_chunks.assign(chunks, chunks + n);
    m->async_active = true;
    m->async_rc = LVN_OK;
    const int device = g.device;
    m->async_thread = std::thread([m, out, device]() {
        if (cudaSetDevice(device) != cudaSuccess) {
            m->async_rc = LVN_ERR_CUDA;
            return;
        }
        m->async_rc = lvn_meshgen_generate_chunks(m, m->async_chunks.data(), (int32_t)m->async_chunks.size(), out);
    });
    return LVN_OK;
}

int lvn_meshgen_wait(lvn_meshgen* m) {
    if (!m) return LVN_ERR_INVALID;
    if (!m->async_active) return LVN_OK;
    m->async_thread.join();
    m->async_active = false;
    return m->async_rc;
}

int lvn_meshgen_generate_chunk_mesh(lvn_meshgen* m, const int32_t min[3], int32_t size, lvn_mesh_out* out) {
    if (!g.initialised) return LVN_ERR_NOT_INITIALISED;
    if (!m || !min || !out) return LVN_ERR_INVALID;
    if (size <= 0 || size % (m->vpc * LEAF_SIZE_SCALE) != 0) return LVN_ERR_INVALID;
    if (!m->cache) {
        // cold path: one fresh chunk with the stored operations replayed
        lvn_chunk_desc cd;
        for (int i = 0; i < 3; i++) cd.min[i] = min[i];
        cd.size = size;
        std::vector<ChunkDesc> descs;
        std::vector<Brush> brushes;
        int rc = build_descs(m, &cd, 1, descs, brushes, true);
        if (rc) return rc;
        if ((rc = run_fresh_batch(m, descs, brushes, nullptr))) return rc;
        OctreeEntry o;
        if ((rc = pull_chunk(m, o))) return rc;
        return export_chunk(m, o, out);
    }
    // LoadOctree (compute_octree.cpp:154-181)
    const ChunkKey k = key_of(min, size);
    auto it = m->octrees.find(k);
    if (it == m->octrees.end()) {
        FieldEntry* f = nullptr;
        int rc = load_field(m, min, size, &f);
        if (rc) return rc;
        f = &m->fields[k];
        OctreeEntry o;
        if (f->num_edges > 0) {
            if ((rc = mesh_from_field(m, min, size, *f))) return rc;
            if ((rc = pull_chunk(m, o))) return rc;
        }
        it = m->octrees.emplace(k, std::move(o)).first;
    }
    return export_chunk(m, it->second, out);
}

int lvn_meshgen_apply_csg_operations(lvn_meshgen* m, const lvn_csg_op* ops, int32_t num_ops, const int32_t min[3],
                                     int32_t size) {
    if (!g.initialised) return LVN_ERR_NOT_INITIALISED;
    if (!m || !min || num_ops < 0 || (num_ops > 0 && !ops)) return LVN_ERR_INVALID;
    if (size <= 0 || size % (m->vpc * LEAF_SIZE_SCALE) != 0) return LVN_ERR_INVALID;
    for (int i = 0; i < num_ops; i++)
        if (!valid_op(ops[i])) return LVN_ERR_INVALID;
    FieldEntry* f = nullptr;
    int rc = load_field(m, min, size, &f);
    if (rc) return rc;
    f = &m->fields[key_of(min, size)];
    std::vector<lvn_csg_op> v(ops, ops + num_ops);
    if ((rc = apply_csg_to_field(m, min, size, *f, v))) return rc;
    f->last_op += num_ops;  // compute_csg.cpp:237
    return LVN_OK;
}

int lvn_meshgen_free_chunk_octree(lvn_meshgen* m, const int32_t min[3], int32_t size) {
    if (!m || !min) return LVN_ERR_INVALID;
    m->octrees.erase(key_of(min, size));
    return LVN_OK;
}

int lvn_meshgen_is_chunk_empty(lvn_meshgen* m, const int32_t min[3], int32_t size, int32_t* is_empty) {
    if (!g.initialised) return LVN_ERR_NOT_INITIALISED;
    if (!m || !min || !is_empty) return LVN_ERR_INVALID;
    if (size <= 0 || size % (m->vpc * LEAF_SIZE_SCALE) != 0) return LVN_ERR_INVALID;
    const ChunkKey k = key_of(min, size);
    auto it = m->fields.find(k);
    if (it == m->fields.end()) {
        FieldEntry fresh;
        const int rc = generate_field(m, min, size, fresh);
        if (rc) return rc;
        it = m->fields.emplace(k, std::move(fresh)).first;
    }
    *is_empty = it->second.num_edges == 0 ? 1 : 0;
    return LVN_OK;
}

int64_t lvn_meshgen_debug_fetch(lvn_meshgen* m, int32_t what, int32_t chunk, void* host, int64_t cap) {
    if (!m || chunk < 0 || chunk >= m->last_n) return LVN_ERR_INVALID;
    const ChunkState& cs = m->last_cs[chunk];
    const size_t F = (size_t)field_size(m->vpc);
    const void* src = nullptr;
    int64_t count = 0, elem = 0;
    std::vector<uint8_t> mats;
    switch (what) {
        case LVN_DEBUG_MATERIALS: {
            if (cap < (int64_t)F) return LVN_ERR_CAPACITY;
            uint8_t* out = static_cast<uint8_t*>(host);
            if (cudaMemcpy(out, m->mats.as<uint8_t>() + F * chunk, F, cudaMemcpyDeviceToHost) != cudaSuccess)
                return LVN_ERR_CUDA;
            if (m->last_fresh && chunk < (int)m->last_desc.size()) {
                // fresh fields hold byte materials only inside the CSG box; the
                // rest are the default material or AIR by the final-air bits
                const int fd = m->vpc + 2;
                const size_t R = (size_t)fd * fd;
                std::vector<uint4> air(R);
                if (cudaMemcpy(air.data(), m->planes.as<uint4>() + (3 * (size_t)chunk + 1) * R, R * sizeof(uint4),
                               cudaMemcpyDeviceToHost) != cudaSuccess)
                    return LVN_ERR_CUDA;
                const ChunkDesc& d = m->last_desc[chunk];
                for (int z = 0; z < fd; z++)
                    for (int y = 0; y < fd; y++)
                        for (int x = 0; x < fd; x++) {
                            const bool in_box = d.op_count > 0 && x >= d.csg_lo[0] && x <= d.csg_hi[0] &&
                                                y >= d.csg_lo[1] && y <= d.csg_hi[1] && z >= d.csg_lo[2] &&
                                                z <= d.csg_hi[2];
                            if (in_box) continue;
                            const uint4 r = air[y + fd * z];
                            const unsigned w = x < 32 ? r.x : x < 64 ? r.y : r.z;
                            const bool is_air = (w >> (x & 31)) & 1u;
                            out[x + fd * y + (size_t)fd * fd * z] = is_air ? MATERIAL_AIR : (uint8_t)g.default_material;
                        }
            }
            return (int64_t)F;
        }
        case LVN_DEBUG_EDGE_KEYS: src = m->edge_keys.as<int32_t>() + cs.edge_off; count = cs.num_edges; elem = 4; break;
        case LVN_DEBUG_EDGE_INFO: src = m->edge_info.as<float4>() + cs.edge_off; count = cs.num_edges; elem = 16; break;
        case LVN_DEBUG_NODE_CODES: src = m->node_codes.as<uint32_t>() + cs.node_off; count = cs.nodes; elem = 4; break;
        case LVN_DEBUG_NODE_INFO: src = m->node_info.as<int32_t>() + cs.node_off; count = cs.nodes; elem = 4; break;
        case LVN_DEBUG_EDGE_TABLE:
            src = m->edge_slots.as<unsigned long long>() + cs.edge_table_off; count = cs.edge_prime; elem = 8; break;
        case LVN_DEBUG_EDGE_STASH:
            src = m->edge_slots.as<unsigned long long>() + cs.edge_table_off + cs.edge_prime;
            count = cs.edge_prime ? CUCKOO_STASH_SIZE : 0; elem = 8; break;
        case LVN_DEBUG_NODE_TABLE:
            src = m->node_slots.as<unsigned long long>() + cs.node_table_off; count = cs.node_prime; elem = 8; break;
        case LVN_DEBUG_NODE_STASH:
            src = m->node_slots.as<unsigned long long>() + cs.node_table_off + cs.node_prime;
            count = cs.node_prime ? CUCKOO_STASH_SIZE : 0; elem = 8; break;
        case LVN_DEBUG_PLAIN_EDGES: return cs.plain_edges;
        case LVN_DEBUG_SIMP_REPS:
            if (m->simp_threshold < 0.f) return LVN_ERR_INVALID;
            src = m->simp_rep.as<int>() + cs.node_off;
            count = cs.nodes; elem = 4; break;
        default: return LVN_ERR_INVALID;
    }
    if (count * elem > cap) return LVN_ERR_CAPACITY;
    if (count && cudaMemcpy(host, src, count * elem, cudaMemcpyDeviceToHost) != cudaSuccess) return LVN_ERR_CUDA;
    return count;
}

int lvn_meshgen_qef_fp64_error(lvn_meshgen* m, double out[4]) {
    if (!m || !out) return LVN_ERR_INVALID;
    if (!m->last_fresh || m->last_n <= 0) return LVN_ERR_INVALID;
    BatchPtrs b = make_ptrs(m, m->last_n);
    DevBuf stats;
    LVN_CK(stats.ensure(sizeof(unsigned long long) * 4));
    LVN_CK(cudaMemsetAsync(stats.p, 0, sizeof(unsigned long long) * 4, m->stream));
    LVN_CK(launch_leaf_qef_check(b, stats.as<unsigned long long>(), m->stream));
    unsigned long long h[4];
    const cudaError_t e = cudaMemcpyAsync(h, stats.p, sizeof(h), cudaMemcpyDeviceToHost, m->stream);
    const cudaError_t e2 = e == cudaSuccess ? cudaStreamSynchronize(m->stream) : e;
    stats.release();
    LVN_CK(e2);
    double mx, sum;
    std::memcpy(&mx, &h[0], 8);
    std::memcpy(&sum, &h[1], 8);
    out[0] = mx;
    out[1] = h[2] ? sum / (double)h[2] : 0.0;
    out[2] = (double)h[2];
    out[3] = (double)h[3];
    return LVN_OK;
}

int lvn_debug_inject_fault(int32_t what, int32_t count) {
    if (count < 0) return LVN_ERR_INVALID;
    switch (what) {
        case LVN_FAULT_NONE:
            g_fault_device_alloc = 0;
            g_fault_hash_family = 0;
            g_fault_hash_host_only = false;
            return LVN_OK;
        case LVN_FAULT_DEVICE_ALLOC: g_fault_device_alloc = count; return LVN_OK;
        case LVN_FAULT_HASH_FAMILY:
            g_fault_hash_family = count;
            g_fault_hash_host_only = false;
            return LVN_OK;
        case LVN_FAULT_HASH_FAMILY_HOST:
            g_fault_hash_family = count;
            g_fault_hash_host_only = true;
            return LVN_OK;
        default: return LVN_ERR_INVALID;
    }
}

int lvn_debug_cuckoo(const uint32_t* keys, int32_t n, uint32_t prime, int32_t flags, uint32_t* values,
                     uint64_t* table_out, int64_t table_capacity, int32_t info[4]) {
    if (!g.initialised) return LVN_ERR_NOT_INITIALISED;
    if (!keys || !values || !info || n <= 0 || (flags & ~LVN_CUCKOO_REFERENCE_FIND)) return LVN_ERR_INVALID;
    if (prime == 0) prime = (uint32_t)host_next_prime(std::max((int)CUCKOO_MIN_TABLE_SIZE, 2 * n));
    if (prime < 2 || prime > (1u << 30)) return LVN_ERR_INVALID;
    const int64_t slots = (int64_t)prime + CUCKOO_STASH_SIZE;
    if (table_out && table_capacity < slots) return LVN_ERR_CAPACITY;
    DevBuf d_keys, d_table, d_status, d_values;
    LVN_CK(d_keys.ensure(sizeof(uint32_t) * n));
    LVN_CK(d_table.ensure(sizeof(unsigned long long) * slots));
    LVN_CK(d_status.ensure(sizeof(int) * 2));
    LVN_CK(d_values.ensure(sizeof(uint32_t) * n));
    struct Release {
        DevBuf* b[4];
        ~Release() { for (DevBuf* x : b) x->release(); }
    } release{{&d_keys, &d_table, &d_status, &d_values}};
    LVN_CK(cudaMemcpy(d_keys.p, keys, sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    cudaStream_t stream = nullptr;  // the legacy default stream: a test hook
    int status[2] = {0, 0};
    int attempt = 0;
    CuckooParams cp;
    for (; attempt < kMaxHashRetries; attempt++) {
        draw_params(cp.p);  // Cuckoo_InitialiseTable's parameters (compute_cuckoo.cpp:62-67)
        LVN_CK(cudaMemsetAsync(d_status.p, 0, sizeof(int) * 2, stream));
        LVN_CK(launch_debug_cuckoo(d_keys.as<uint32_t>(), n, d_table.as<unsigned long long>(), prime, cp,
                                   d_status.as<int>(), (flags & LVN_CUCKOO_REFERENCE_FIND) ? 1 : 0,
                                   d_values.as<uint32_t>(), stream));
        LVN_CK(cudaMemcpyAsync(status, d_status.p, sizeof(status), cudaMemcpyDeviceToHost, stream));
        LVN_CK(cudaStreamSynchronize(stream));
        if (!status[1]) break;
    }
    info[0] = (int32_t)prime;
    info[1] = status[0];
    info[2] = std::min(attempt + 1, kMaxHashRetries);
    info[3] = status[1];
    if (status[1]) return LVN_ERR_HASH;
    LVN_CK(cudaMemcpy(values, d_values.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    if (table_out) LVN_CK(cudaMemcpy(table_out, d_table.p, sizeof(uint64_t) * slots, cudaMemcpyDeviceToHost));
    return LVN_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// read-only state access for other translation units (lvn_state.h)
// ---------------------------------------------------------------------------

#include "lvn_state.h"

namespace lvn {

// A bound on |amp3 * fbm3| as the kernels compute it, for the cave density
// (0 for the heightfield densities, which have no 3D term).
// |snoise3| <= 1.2972: each of a point's four simplex corners adds at most
// (0.6 - r^2)^4 r |g| to the sum before the factor 32, with |g| <= 1.42532 for
// the gradient table; the corners are among the lattice points within
// sqrt(0.6) of the point, and the largest sum of (0.6 - r^2)^4 r over those
// lattice points, over a 200^3 grid of one skewed cell, is 0.025074, plus
// 0.003367 for the grid spacing (6 lattice points in range, each changing by at
// most 0.6^4 per unit of distance).  32 * 1.42532 * 0.028441 = 1.2972.  fbm3
// sums the octaves scaled by amplitudes 1, gain3, gain3^2, ...; the 0.1% on
// top covers single-precision rounding of those sums and products.
static float cave_band(const DensityParams& d) {
    if (d.mode != LVN_DENSITY_CAVES) return 0.f;
    double sum = 0.0;
    float a = 1.f;
    for (int i = 0; i < d.octaves3; i++) {
        sum += std::fabs((double)a);
        a = a * d.gain3;
    }
    const double band = std::fabs((double)d.amp3) * 1.2972 * sum * 1.001;
    if (!(band < 1e30)) return INFINITY;  // non-finite parameters: every point is evaluated
    return std::nextafter((float)band, INFINITY);
}

// rem[s] = the same bound over fbm3's octaves 2s and up only (the octaves the
// field kernel has not evaluated after s steps of two), plus 4e-3 for the
// rounding of the partial sums the kernel compares against it; 0 once no
// octave is left.
static void cave_remainders(const DensityParams& d, float* rem) {
    for (int s = 0; s <= kCaveSteps; s++) rem[s] = 0.f;
    if (d.mode != LVN_DENSITY_CAVES) return;
    float a = 1.f;
    std::vector<double> amp;
    for (int i = 0; i < d.octaves3; i++) {
        amp.push_back(std::fabs((double)a));
        a = a * d.gain3;
    }
    for (int s = 0; s <= kCaveSteps; s++) {
        double sum = 0.0;
        for (size_t i = 2 * (size_t)s; i < amp.size(); i++) sum += amp[i];
        if (sum == 0.0) break;
        const double r = std::fabs((double)d.amp3) * 1.2972 * sum * 1.001 + 4e-3;
        rem[s] = r < 1e30 ? std::nextafter((float)r, INFINITY) : INFINITY;
    }
}

void density_fields(const DensityParams& d, int32_t default_material, float* band, float* rem,
                    int32_t dom_by_solid[9]) {
    *band = cave_band(d);
    cave_remainders(d, rem);
    for (int n = 0; n <= 8; n++) {
        int mats[8];
        for (int i = 0; i < 8; i++) mats[i] = i < n ? default_material : MATERIAL_AIR;
        dom_by_solid[n] = dominant_material(mats);
    }
}

GlobalView global_view() {
    GlobalView v;
    v.initialised = g.initialised;
    v.device = g.device;
    v.num_sms = g.num_sms;
    v.default_material = g.default_material;
    v.perm = g.perm.as<uint8_t>();
    v.perm_t3 = g.perm_t3.as<uint8_t>();
    v.grad = g.grad.as<float>();
    v.density = g.density;
    return v;
}

int stored_ops_for_chunk(const int32_t min[3], int32_t size, Brush* out, int cap) {
    const int32_t lo[3] = {min[0], min[1], min[2]};
    const int32_t hi[3] = {min[0] + size, min[1] + size, min[2] + size};
    int n = 0;
    for (const StoredOp& s : g.ops) {
        if (!overlaps(lo, hi, s.lo, s.hi)) continue;
        if (n >= cap) return -1;
        out[n++] = make_brush(s.op);
    }
    return n;
}

void draw_hash_params(uint32_t* p) { draw_params(p); }
int device_hash_fault() { return g_fault_hash_family > 0 && !g_fault_hash_host_only ? 1 : 0; }

void lod_colour_for(int s, float c[3]) { lod_colour(s, c); }

void csg_box_for(const Brush* ops, int n, const int32_t off[3], int scale, int fd, int32_t lo[3], int32_t hi[3]) {
    csg_box(ops, n, off, scale, fd, lo, hi);
}

}  // namespace lvn
