// lvn_clipmap.cu -- the clipmap's chunk lists made on the GPU: the active
// nodes a camera selects (SelectActiveClipmapNodes, leven/src/clipmap.cpp:
// 1084-1128) and the nodes a batch of CSG operations touches
// (processCSGOperationsImpl / FindNodesInsideAABB, clipmap.cpp:1571-1607,
// 1647-1673), over a complete clipmap octree whose leaves are
// CLIPMAP_LEAF_SIZE nodes (ConstructChildren, clipmap.cpp:715-735).  The lists
// feed lvn_meshgen_generate_chunks and lvn_meshgen_apply_csg_operations.
//
// One CTA walks one query (a camera, or the whole operation set) level by
// level from the largest renderable nodes (LOD_MAX_NODE_SIZE, clipmap.cpp:31):
// each pass takes the level's open nodes, lists the ones it decides and opens
// the children still to visit, so only the nodes the reference's recursion
// reaches are examined.  The listed nodes are then sorted in shared memory
// into the recursion's order (pre-order for the selection, post-order for the
// touch set) by a key built from their leaf-grid position.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/lvn.h"
#include "lvn_types.h"

namespace lvn {
namespace {

constexpr int kNumLods = 6;                                           // clipmap.cpp:28
constexpr int kLodMaxNodeSize = CLIPMAP_LEAF_SIZE << (kNumLods - 1);  // clipmap.cpp:31
__constant__ float kLodActiveDistances[kNumLods] = {                  // clipmap.cpp:33-41
    0.f,
    CLIPMAP_LEAF_SIZE * 1.5f,
    CLIPMAP_LEAF_SIZE * 3.5f,
    CLIPMAP_LEAF_SIZE * 5.5f,
    CLIPMAP_LEAF_SIZE * 7.5f,
    CLIPMAP_LEAF_SIZE * 13.5f,
};
constexpr int kMaxNodes = LVN_CLIPMAP_MAX_NODES;  // listed nodes per query
constexpr int kMaxOpen = LVN_CLIPMAP_MAX_OPEN;    // open nodes per level and query
constexpr int kIndexBits = 13;                    // sort entry: key << 13 | list index
static_assert(kMaxNodes <= (1 << kIndexBits), "list index bits");
constexpr int kWalkThreads = 256;
constexpr int kSlotNodes = 2 * kMaxOpen + kMaxNodes;  // scratch per CTA: two open lists + the listed nodes
constexpr int kHostStride = 1024;                     // first-pass list length per camera, host-buffer form
constexpr int kMaxBoxes = 4096;                       // operations per touch-set call
constexpr int kWarpList = 1024;  // selection by one warp per camera: listed nodes
constexpr int kWarpOpen = 512;   // and open nodes per level; beyond either the CTA walk redoes the camera
constexpr int kWarpsPerCta = 8;
constexpr int kRedo = -2;        // count of a camera the warp walk left to the CTA walk

struct Node {
    int32_t min[3];
    int32_t size;
};
static_assert(sizeof(Node) == sizeof(lvn_chunk_desc), "a node is written out as a chunk descriptor");

struct Tree {
    int32_t root_min[3];
    int32_t root_size;
    int depth;     // log2(root_size / CLIPMAP_LEAF_SIZE)
    int top_size;  // min(root_size, LOD_MAX_NODE_SIZE)
    int top_lod;   // log2(top_size / CLIPMAP_LEAF_SIZE)
    int per;       // root_size / top_size: top-level nodes per axis
};

// DistanceToNode (clipmap.cpp:1056-1064): float corners, float camera, each
// operation rounded on its own
__device__ __forceinline__ float distance_to_node(const Node& n, const float cam[3]) {
    float d[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float lo = (float)n.min[a], hi = (float)(n.min[a] + n.size);
        d[a] = fmaxf(fmaxf(__fsub_rn(lo, cam[a]), 0.f), __fsub_rn(cam[a], hi));
    }
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])));
}

// AABB::overlaps (aabb.h:26-35) of any operation bound and the node's box
__device__ __forceinline__ bool touches(const Node& n, const int32_t* box, int num_boxes) {
    for (int i = 0; i < num_boxes; i++) {
        const int32_t* b = box + 6 * i;
        const bool apart = b[3] < n.min[0] || b[4] < n.min[1] || b[5] < n.min[2] || b[0] > n.min[0] + n.size ||
                           b[1] > n.min[1] + n.size || b[2] > n.min[2] + n.size;
        if (!apart) return true;
    }
    return false;
}

// The recursion's order as a key.  Children are visited in CHILD_MIN_OFFSETS
// order (x << 2 | y << 1 | z), so the recursion meets leaves in the Morton
// order of their leaf-grid positions (x the most significant bit of each
// triple).  Pre-order: a node comes at its first leaf; post-order: at its last
// leaf, after its descendants, so the size is the tie-break (smaller first).
// The selection never lists a node and its descendant, so the tie-break only
// orders the touch set.
__device__ __forceinline__ unsigned long long order_key(const Node& n, const Tree& t, int lod, bool post) {
    int p[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int first = (n.min[a] - t.root_min[a]) / CLIPMAP_LEAF_SIZE;
        p[a] = post ? first + (n.size / CLIPMAP_LEAF_SIZE) - 1 : first;
    }
    unsigned long long code = 0;
    for (int bit = t.depth - 1; bit >= 0; bit--)
        code = (code << 3) | (unsigned long long)((((p[0] >> bit) & 1) << 2) | (((p[1] >> bit) & 1) << 1) |
                                                  ((p[2] >> bit) & 1));
    return (code << 3) | (unsigned long long)lod;
}

// One CTA per query.  cams == nullptr: the touch set of the num_boxes bounds
// (one query); else query q selects for camera cams[3q..3q+2].  Query q's
// sorted list goes to out[q * stride ...] (at most stride entries) and its
// length to counts[q]: -1 when it exceeded an internal limit.
__global__ void __launch_bounds__(kWalkThreads) k_clipmap_walk(Tree t, const float* __restrict__ cams, int num_queries,
                                                               const int32_t* __restrict__ boxes, int num_boxes,
                                                               Node* __restrict__ scratch, lvn_chunk_desc* out,
                                                               int stride, int32_t* counts, int redo_only) {
    extern __shared__ unsigned long long sk[];  // [kMaxNodes] sort entries
    __shared__ int s_open[2], s_listed, s_over;
    const bool post = cams == nullptr;
    Node* const open = scratch + (size_t)blockIdx.x * kSlotNodes;  // open list c at open + c * kMaxOpen
    Node* const listed = open + 2 * kMaxOpen;
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int q = blockIdx.x; q < num_queries; q += gridDim.x) {
        if (redo_only && counts[q] != kRedo) continue;  // the warp walk answered this camera
        float cam[3] = {0.f, 0.f, 0.f};
        if (!post)
            for (int a = 0; a < 3; a++) cam[a] = cams[3 * q + a];
        if (tid == 0) {
            s_open[0] = s_open[1] = 0;
            s_listed = s_over = 0;
        }
        __syncthreads();
        // the top level: every node of the largest renderable size (the host
        // keeps per^3 <= kMaxOpen)
        const int ntop = t.per * t.per * t.per;
        for (int i = tid; i < ntop; i += nth) {
            Node nd;
            nd.min[0] = t.root_min[0] + (i / (t.per * t.per)) * t.top_size;
            nd.min[1] = t.root_min[1] + ((i / t.per) % t.per) * t.top_size;
            nd.min[2] = t.root_min[2] + (i % t.per) * t.top_size;
            nd.size = t.top_size;
            if (post && !touches(nd, boxes, num_boxes)) continue;
            open[atomicAdd(&s_open[0], 1)] = nd;
        }
        __syncthreads();
        int cur = 0;
        for (int lod = t.top_lod; lod >= 0; lod--) {
            const int n = min(s_open[cur], kMaxOpen);
            for (int i = tid; i < n; i += nth) {
                const Node nd = open[cur * kMaxOpen + i];
                bool list, expand;
                if (post) {  // FindNodesInsideAABB: every overlapping node, and its overlapping children
                    list = true;
                    expand = lod > 0;
                } else {  // SelectActiveClipmapNodes: listed at its LOD's distance, else its children are visited
                    list = distance_to_node(nd, cam) >= kLodActiveDistances[lod];
                    expand = !list && lod > 0;
                }
                if (list) {
                    const int slot = atomicAdd(&s_listed, 1);
                    if (slot < kMaxNodes) {
                        listed[slot] = nd;
                        sk[slot] = (order_key(nd, t, lod, post) << kIndexBits) | (unsigned long long)slot;
                    }
                }
                if (expand) {
                    const int h = nd.size >> 1;
                    for (int c = 0; c < 8; c++) {
                        Node ch;
                        ch.min[0] = nd.min[0] + ((c >> 2) & 1) * h;
                        ch.min[1] = nd.min[1] + ((c >> 1) & 1) * h;
                        ch.min[2] = nd.min[2] + (c & 1) * h;
                        ch.size = h;
                        if (post && !touches(ch, boxes, num_boxes)) continue;
                        const int slot = atomicAdd(&s_open[cur ^ 1], 1);
                        if (slot < kMaxOpen)
                            open[(cur ^ 1) * kMaxOpen + slot] = ch;
                        else
                            s_over = 1;
                    }
                }
            }
            __syncthreads();
            if (tid == 0) s_open[cur] = 0;
            __syncthreads();
            cur ^= 1;
        }
        const int total = s_listed;
        const bool over = s_over || total > kMaxNodes;
        if (!over) {
            int p2 = 1;
            while (p2 < total) p2 <<= 1;
            for (int i = total + tid; i < p2; i += nth) sk[i] = ~0ull;
            __syncthreads();
            // bitonic sort of the p2 entries (distinct: the list index is in the low bits)
            for (int k = 2; k <= p2; k <<= 1) {
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int i = tid; i < p2; i += nth) {
                        const int l = i ^ j;
                        if (l > i) {
                            const unsigned long long a = sk[i], b = sk[l];
                            if (((i & k) == 0) == (a > b)) {
                                sk[i] = b;
                                sk[l] = a;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            const int nout = min(total, stride);
            for (int i = tid; i < nout; i += nth) {
                const Node nd = listed[sk[i] & ((1ull << kIndexBits) - 1)];
                lvn_chunk_desc d;
                for (int a = 0; a < 3; a++) d.min[a] = nd.min[a];
                d.size = nd.size;
                out[(size_t)q * stride + i] = d;
            }
        }
        if (tid == 0) counts[q] = over ? -1 : total;
        __syncthreads();  // the shared counters and entries are reused by the next query
    }
}

// Selection with one warp per camera (warp-synchronous: ballots, shuffles and
// __syncwarp, no CTA barriers).  Open nodes are packed leaf-grid positions
// (10 bits an axis) and LOD; a listed node is kept only as its sort key, which
// identifies it (first leaf and LOD).  A camera that lists more than
// kWarpList nodes or opens more than kWarpOpen in a level gets kRedo.
__device__ __forceinline__ uint64_t pack_open(const int32_t p[3], int lod) {
    return ((uint64_t)p[0] << 23) | ((uint64_t)p[1] << 13) | ((uint64_t)p[2] << 3) | (uint64_t)lod;
}

__global__ void __launch_bounds__(kWarpsPerCta * 32) k_clipmap_select_warp(Tree t, const float* __restrict__ cams,
                                                                          int num_queries, uint64_t* scratch,
                                                                          lvn_chunk_desc* out, int stride,
                                                                          int32_t* counts) {
    extern __shared__ unsigned long long wkeys[];  // [kWarpsPerCta][kWarpList]
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1;
    unsigned long long* keys = wkeys + wib * kWarpList;
    const int wslot = blockIdx.x * kWarpsPerCta + wib;
    uint64_t* open = scratch + (size_t)wslot * 2 * kWarpOpen;  // list c at open + c * kWarpOpen
    const int leaf = CLIPMAP_LEAF_SIZE;
    for (int q = wslot; q < num_queries; q += gridDim.x * kWarpsPerCta) {
        const float cam[3] = {cams[3 * q], cams[3 * q + 1], cams[3 * q + 2]};
        const int per = t.per, ntop = per * per * per, top_units = t.top_size / leaf;
        for (int i = lane; i < ntop; i += 32) {  // the host keeps ntop <= kWarpOpen for this walk
            const int32_t p[3] = {(i / (per * per)) * top_units, ((i / per) % per) * top_units, (i % per) * top_units};
            open[i] = pack_open(p, t.top_lod);
        }
        __syncwarp();
        int cur = 0, n = ntop, listed = 0;
        bool over = false;
        for (int lod = t.top_lod; lod >= 0; lod--) {
            int next = 0;
            for (int base = 0; base < n; base += 32) {
                const int i = base + lane;
                Node nd;
                bool list = false, expand = false;
                if (i < n) {
                    const uint64_t o = open[cur * kWarpOpen + i];
                    const int32_t p[3] = {(int32_t)((o >> 23) & 1023), (int32_t)((o >> 13) & 1023),
                                          (int32_t)((o >> 3) & 1023)};
                    for (int a = 0; a < 3; a++) nd.min[a] = t.root_min[a] + p[a] * leaf;
                    nd.size = leaf << lod;
                    list = distance_to_node(nd, cam) >= kLodActiveDistances[lod];
                    expand = !list && lod > 0;
                }
                const unsigned bl = __ballot_sync(0xffffffffu, list);
                if (list) {
                    const int pos = listed + __popc(bl & below);
                    if (pos < kWarpList) keys[pos] = order_key(nd, t, lod, false);
                }
                listed += __popc(bl);
                const unsigned be = __ballot_sync(0xffffffffu, expand);
                if (expand) {
                    const int pos = next + 8 * __popc(be & below);
                    const int32_t h = (nd.size >> 1) / leaf;
                    int32_t p[3];
                    for (int a = 0; a < 3; a++) p[a] = (nd.min[a] - t.root_min[a]) / leaf;
                    for (int c = 0; c < 8; c++) {
                        const int32_t cp[3] = {p[0] + ((c >> 2) & 1) * h, p[1] + ((c >> 1) & 1) * h, p[2] + (c & 1) * h};
                        if (pos + c < kWarpOpen) open[(cur ^ 1) * kWarpOpen + pos + c] = pack_open(cp, lod - 1);
                    }
                }
                next += 8 * __popc(be);
            }
            __syncwarp();
            over |= next > kWarpOpen;
            n = min(next, kWarpOpen);
            cur ^= 1;
        }
        over |= listed > kWarpList;
        if (!over) {
            // bitonic network over any n (mirrored first step), warp-synchronous
            for (int k = 2; k < 2 * listed; k <<= 1) {
                for (int j = k >> 1; j > 0; j >>= 1) {
                    const int mask = j == (k >> 1) ? k - 1 : j;
                    for (int i = lane; i < listed; i += 32) {
                        const int l = i ^ mask;
                        if (l > i && l < listed) {
                            const unsigned long long a = keys[i], b = keys[l];
                            if (a > b) {
                                keys[i] = b;
                                keys[l] = a;
                            }
                        }
                    }
                    __syncwarp();
                }
            }
            const int nout = min(listed, stride);
            for (int i = lane; i < nout; i += 32) {
                const unsigned long long key = keys[i];
                const int lod = (int)(key & 7);
                const unsigned long long code = key >> 3;
                int32_t p[3] = {0, 0, 0};
                for (int bit = t.depth - 1; bit >= 0; bit--) {
                    const int tr = (int)((code >> (3 * bit)) & 7);
                    p[0] = (p[0] << 1) | ((tr >> 2) & 1);
                    p[1] = (p[1] << 1) | ((tr >> 1) & 1);
                    p[2] = (p[2] << 1) | (tr & 1);
                }
                lvn_chunk_desc d;
                for (int a = 0; a < 3; a++) d.min[a] = t.root_min[a] + p[a] * leaf;
                d.size = leaf << lod;
                out[(size_t)q * stride + i] = d;
            }
        }
        if (lane == 0) counts[q] = over ? kRedo : listed;
        __syncwarp();
    }
}

// Packs the host form's lists back to back: list q (counts[q] nodes) goes to
// packed[place[2q]] from the first pass (stride kHostStride) or, when
// place[2q + 1] >= 0, from that row of the second pass (stride kMaxNodes).
__global__ void k_clipmap_pack(const lvn_chunk_desc* __restrict__ wide, const lvn_chunk_desc* __restrict__ wide_big,
                               const int32_t* __restrict__ counts, const int32_t* __restrict__ place,
                               lvn_chunk_desc* __restrict__ packed) {
    const int q = blockIdx.x;
    const int n = counts[q], off = place[2 * q], big = place[2 * q + 1];
    const lvn_chunk_desc* src = big >= 0 ? wide_big + (size_t)big * kMaxNodes : wide + (size_t)q * kHostStride;
    for (int i = threadIdx.x; i < n; i += blockDim.x) packed[(size_t)off + i] = src[i];
}

// A device (or pinned host) array that grows on demand; growing waits for the
// work in flight on the device.
template <class T, bool Host = false>
struct Grow {
    T* p = nullptr;
    size_t cap = 0;
    cudaError_t fit(size_t need) {
        if (need <= cap) return cudaSuccess;
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return e;
        need = std::max(need, 2 * cap);
        if (p) Host ? cudaFreeHost(p) : cudaFree(p);
        p = nullptr;
        cap = 0;
        e = Host ? cudaMallocHost(&p, sizeof(T) * need) : cudaMalloc(&p, sizeof(T) * need);
        if (e == cudaSuccess) cap = need;
        return e;
    }
};

// Scratch shared by the calls, which its mutex serialises (the device form's
// kernels also by the caller's stream order, see lvn.h).
struct Work {
    std::mutex mu;
    int device = -1;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    Node* scratch = nullptr;
    int scratch_ctas = 0;
    Grow<float> dcams, dcams_big;                  // cameras of the two passes
    Grow<int32_t> dcounts, dcounts_big, dplace;    // counts; (offset, second-pass row) per camera
    Grow<lvn_chunk_desc> wide, wide_big, packed;   // pass outputs (stride kHostStride / kMaxNodes), packed lists
    Grow<int32_t, true> hcounts, hplace;           // pinned
    int32_t* dboxes = nullptr;                     // kMaxBoxes x 6
    Grow<uint64_t> wscratch;                       // the warp walk's open lists
};
Work& work() {
    static Work w;
    return w;
}

int cuda_rc(cudaError_t e) {
    if (e == cudaSuccess) return LVN_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? LVN_ERR_OUT_OF_MEMORY : LVN_ERR_CUDA;
}

#define CM_TRY(x)                        \
    do {                                 \
        const int rc__ = cuda_rc(x);     \
        if (rc__ != LVN_OK) return rc__; \
    } while (0)

// root_min / root_size describe a complete octree down to CLIPMAP_LEAF_SIZE nodes
int make_tree(const int32_t root_min[3], int32_t root_size, Tree* t) {
    if (!root_min || root_size < CLIPMAP_LEAF_SIZE || (root_size & (root_size - 1))) return LVN_ERR_INVALID;
    for (int a = 0; a < 3; a++) {
        if ((int64_t)root_min[a] + root_size > INT32_MAX) return LVN_ERR_INVALID;
        t->root_min[a] = root_min[a];
    }
    t->root_size = root_size;
    t->depth = 0;
    while ((CLIPMAP_LEAF_SIZE << t->depth) < root_size) t->depth++;
    t->top_size = std::min(root_size, kLodMaxNodeSize);
    t->top_lod = 0;
    while ((CLIPMAP_LEAF_SIZE << t->top_lod) < t->top_size) t->top_lod++;
    t->per = root_size / t->top_size;
    if (t->per > 16 || t->per * t->per * t->per > kMaxOpen) return LVN_ERR_INVALID;  // top level fits one open list
    return LVN_OK;
}

// The walk's grid: one CTA per query, at most two per SM (each holds 64 KB of
// sort entries); the CTAs loop over further queries.
int walk_ctas(const Work& w, int num_queries) { return std::max(1, std::min(num_queries, 2 * w.num_sms)); }

int ensure_work(Work& w, int num_queries) {
    int dev = 0;
    CM_TRY(cudaGetDevice(&dev));
    if (w.device != dev) {
        if (w.device >= 0) return LVN_ERR_INVALID;  // the scratch lives on the first device used
        CM_TRY(cudaDeviceGetAttribute(&w.num_sms, cudaDevAttrMultiProcessorCount, dev));
        CM_TRY(cudaFuncSetAttribute(k_clipmap_walk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(unsigned long long) * kMaxNodes)));
        CM_TRY(cudaFuncSetAttribute(k_clipmap_select_warp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(unsigned long long) * kWarpList * kWarpsPerCta)));
        CM_TRY(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
        CM_TRY(cudaMalloc(&w.dboxes, sizeof(int32_t) * 6 * kMaxBoxes));
        w.device = dev;
    }
    const int ctas = walk_ctas(w, num_queries);
    if (ctas > w.scratch_ctas) {
        if (w.scratch) {
            CM_TRY(cudaDeviceSynchronize());
            CM_TRY(cudaFree(w.scratch));
            w.scratch = nullptr;
            w.scratch_ctas = 0;
        }
        CM_TRY(cudaMalloc(&w.scratch, sizeof(Node) * (size_t)kSlotNodes * ctas));
        w.scratch_ctas = ctas;
    }
    return LVN_OK;
}

void launch_walk(const Work& w, const Tree& t, const float* dcams, int num_queries, const int32_t* dboxes,
                 int num_boxes, lvn_chunk_desc* out, int stride, int32_t* counts, cudaStream_t s, int redo_only = 0) {
    const int ctas = std::min(walk_ctas(w, num_queries), w.scratch_ctas);
    k_clipmap_walk<<<ctas, kWalkThreads, sizeof(unsigned long long) * kMaxNodes, s>>>(
        t, dcams, num_queries, dboxes, num_boxes, w.scratch, out, stride, counts, redo_only);
}

// Selection for cameras: the warp walk where the top level fits it, then the
// CTA walk for the cameras it left (on the same stream).
int launch_select(Work& w, const Tree& t, const float* dcams, int num_queries, lvn_chunk_desc* out, int stride,
                  int32_t* counts, cudaStream_t s) {
    if (t.per * t.per * t.per > kWarpOpen) {
        launch_walk(w, t, dcams, num_queries, nullptr, 0, out, stride, counts, s);
        return cuda_rc(cudaGetLastError());
    }
    const int ctas = std::max(1, std::min((num_queries + kWarpsPerCta - 1) / kWarpsPerCta, 3 * w.num_sms));
    CM_TRY(w.wscratch.fit((size_t)ctas * kWarpsPerCta * 2 * kWarpOpen));
    k_clipmap_select_warp<<<ctas, kWarpsPerCta * 32, sizeof(unsigned long long) * kWarpList * kWarpsPerCta, s>>>(
        t, dcams, num_queries, w.wscratch.p, out, stride, counts);
    CM_TRY(cudaGetLastError());
    launch_walk(w, t, dcams, num_queries, nullptr, 0, out, stride, counts, s, 1);
    return cuda_rc(cudaGetLastError());
}

}  // namespace
}  // namespace lvn

using namespace lvn;

extern "C" {

int lvn_clipmap_select(const float* cameras, int32_t num_cameras, const int32_t root_min[3], int32_t root_size,
                       lvn_chunk_desc* out, int32_t capacity, int32_t* counts) {
    if (num_cameras < 0 || (num_cameras > 0 && (!cameras || !counts)) || capacity < 0 || (capacity > 0 && !out))
        return LVN_ERR_INVALID;
    Tree t;
    int rc = make_tree(root_min, root_size, &t);
    if (rc) return rc;
    if (num_cameras == 0) return LVN_OK;
    const size_t n = (size_t)num_cameras;
    Work& w = work();
    std::lock_guard<std::mutex> lock(w.mu);
    rc = ensure_work(w, num_cameras);
    if (rc) return rc;
    CM_TRY(w.dcams.fit(3 * n));
    CM_TRY(w.dcounts.fit(n));
    CM_TRY(w.dplace.fit(2 * n));
    CM_TRY(w.wide.fit(n * kHostStride));
    CM_TRY(w.hcounts.fit(n));
    CM_TRY(w.hplace.fit(2 * n));
    // first pass: every camera, lists cut at kHostStride nodes
    CM_TRY(cudaMemcpyAsync(w.dcams.p, cameras, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, w.stream));
    rc = launch_select(w, t, w.dcams.p, num_cameras, w.wide.p, kHostStride, w.dcounts.p, w.stream);
    if (rc) return rc;
    CM_TRY(cudaMemcpyAsync(w.hcounts.p, w.dcounts.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, w.stream));
    CM_TRY(cudaStreamSynchronize(w.stream));
    int64_t total = 0;
    bool limit = false;
    std::vector<float> big_cams;
    for (size_t q = 0; q < n; q++) {
        const int c = w.hcounts.p[q];
        counts[q] = c;
        w.hplace.p[2 * q] = (int32_t)std::min<int64_t>(total, INT32_MAX);
        w.hplace.p[2 * q + 1] = -1;
        if (c < 0) {
            limit = true;
            continue;
        }
        if (c > kHostStride) {
            w.hplace.p[2 * q + 1] = (int32_t)(big_cams.size() / 3);
            big_cams.insert(big_cams.end(), cameras + 3 * q, cameras + 3 * q + 3);
        }
        total += c;
    }
    if (limit) return LVN_ERR_DEVICE_STATUS;
    if (total > capacity) return LVN_ERR_CAPACITY;
    if (total == 0) return LVN_OK;
    // second pass: the cameras whose lists were cut, at the full length
    const size_t nbig = big_cams.size() / 3;
    if (nbig) {
        CM_TRY(w.dcams_big.fit(3 * nbig));
        CM_TRY(w.dcounts_big.fit(nbig));
        CM_TRY(w.wide_big.fit(nbig * kMaxNodes));
        CM_TRY(cudaMemcpyAsync(w.dcams_big.p, big_cams.data(), sizeof(float) * 3 * nbig, cudaMemcpyHostToDevice,
                               w.stream));
        launch_walk(w, t, w.dcams_big.p, (int)nbig, nullptr, 0, w.wide_big.p, kMaxNodes, w.dcounts_big.p, w.stream);
        CM_TRY(cudaGetLastError());
    }
    CM_TRY(w.packed.fit((size_t)total));
    CM_TRY(cudaMemcpyAsync(w.dplace.p, w.hplace.p, sizeof(int32_t) * 2 * n, cudaMemcpyHostToDevice, w.stream));
    k_clipmap_pack<<<num_cameras, 128, 0, w.stream>>>(w.wide.p, w.wide_big.p, w.dcounts.p, w.dplace.p, w.packed.p);
    CM_TRY(cudaGetLastError());
    CM_TRY(cudaMemcpyAsync(out, w.packed.p, sizeof(lvn_chunk_desc) * (size_t)total, cudaMemcpyDeviceToHost, w.stream));
    CM_TRY(cudaStreamSynchronize(w.stream));
    return LVN_OK;
}

int lvn_clipmap_select_device(const float* d_cameras, int32_t num_cameras, const int32_t root_min[3],
                              int32_t root_size, lvn_chunk_desc* d_out, int32_t stride, int32_t* d_counts,
                              void* cuda_stream) {
    if (num_cameras < 0 || (num_cameras > 0 && (!d_cameras || !d_out || !d_counts)) || stride < 0)
        return LVN_ERR_INVALID;
    Tree t;
    int rc = make_tree(root_min, root_size, &t);
    if (rc) return rc;
    if (num_cameras == 0) return LVN_OK;
    Work& w = work();
    std::lock_guard<std::mutex> lock(w.mu);
    rc = ensure_work(w, num_cameras);
    if (rc) return rc;
    return launch_select(w, t, d_cameras, num_cameras, d_out, stride, d_counts, (cudaStream_t)cuda_stream);
}

int lvn_clipmap_touched(const lvn_csg_op* ops, int32_t num_ops, const int32_t root_min[3], int32_t root_size,
                        lvn_chunk_desc* out, int32_t capacity, int32_t* count) {
    if (!count || num_ops < 0 || num_ops > kMaxBoxes || (num_ops > 0 && !ops) || capacity < 0 ||
        (capacity > 0 && !out))
        return LVN_ERR_INVALID;
    Tree t;
    int rc = make_tree(root_min, root_size, &t);
    if (rc) return rc;
    *count = 0;
    if (num_ops == 0) return LVN_OK;
    std::vector<int32_t> boxes(6 * (size_t)num_ops);
    for (int i = 0; i < num_ops; i++) {
        rc = lvn_csg_operation_bounds(&ops[i], &boxes[6 * i], &boxes[6 * i + 3]);
        if (rc) return rc;
    }
    Work& w = work();
    std::lock_guard<std::mutex> lock(w.mu);
    rc = ensure_work(w, 1);
    if (rc) return rc;
    CM_TRY(w.wide_big.fit(kMaxNodes));
    CM_TRY(w.dcounts.fit(1));
    CM_TRY(w.hcounts.fit(1));
    CM_TRY(cudaMemcpyAsync(w.dboxes, boxes.data(), sizeof(int32_t) * boxes.size(), cudaMemcpyHostToDevice, w.stream));
    launch_walk(w, t, nullptr, 1, w.dboxes, num_ops, w.wide_big.p, kMaxNodes, w.dcounts.p, w.stream);
    CM_TRY(cudaGetLastError());
    CM_TRY(cudaMemcpyAsync(w.hcounts.p, w.dcounts.p, sizeof(int32_t), cudaMemcpyDeviceToHost, w.stream));
    CM_TRY(cudaStreamSynchronize(w.stream));
    const int n = w.hcounts.p[0];
    if (n < 0) return LVN_ERR_DEVICE_STATUS;
    *count = n;
    if (n > capacity) return LVN_ERR_CAPACITY;
    if (n) {
        CM_TRY(cudaMemcpyAsync(out, w.wide_big.p, sizeof(lvn_chunk_desc) * n, cudaMemcpyDeviceToHost, w.stream));
        CM_TRY(cudaStreamSynchronize(w.stream));
    }
    return LVN_OK;
}

}  // extern "C"
