// lvn_seam.cu -- the clipmap's seam meshes on the GPU: GenerateClipmapSeamMesh
// (leven/src/clipmap.cpp:573-610) for a batch of host chunks.  The reference
// gathers the seam nodes of a host and of the active nodes next to it
// (SelectSeamNodes / FilterSeamNode, clipmap.cpp:508-570), builds a pointer
// octree from them (Octree_ConstructUpwards, octree.cpp:90-148), numbers its
// leaves depth first (GenerateVertexIndices, octree.cpp:197-232) and contours
// it recursively (ContourCellProc / ContourFaceProc / ContourEdgeProc /
// ContourProcessEdge, octree.cpp:236-474) on the CPU.
//
// Here the neighbour search, which walks the clipmap's node tree, stays on the
// host; everything that touches seam nodes runs on the device, one CTA per
// host, without building the tree:
//   * the depth-first leaf order is the Morton order of the leaves' minimum
//     corners (children are visited x << 2 | y << 1 | z), so the leaves are
//     sorted by Morton key (in shared memory when they fit, else in global
//     memory, which the L2 holds) and numbered by rank;
//   * the recursion emits one quad per final edge segment: an edge of the
//     smallest of the four leaves around it, all four present, not all four
//     in one CLIPMAP_LEAF_SIZE block (the straddle test of ContourEdgeProc /
//     ContourFaceProc prunes exactly those), with a sign change on that
//     leaf's edge.  Each leaf tests its 12 edges; the other three leaves come
//     from binary searches of the sorted keys.  This runs over blocks of 256
//     leaves, so a large host spreads over many CTAs;
//   * the recursion's order is restored by a key spelling the path the
//     recursion takes to the segment (cell: child 0-7, face 8-19, edge 20-25
//     in 5 bits; face: sub-face 0-3, edge 4-7 in 3 bits; edge: half in 1 bit),
//     by which the quads are sorted.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/lvn.h"
#include "lvn_types.h"

namespace lvn {
namespace {

constexpr int kMaxLeaves = LVN_SEAM_MAX_LEAVES;  // per host
constexpr int kSlotBits = 15;                    // leaf sort entry: (morton << 4 | size log2) << 15 | slot
constexpr int kRankBits = 15;                    // quad payload: 4 ranks of 15 bits, flip at bit 60
static_assert(kMaxLeaves <= (1 << kRankBits) && kMaxLeaves <= (1 << kSlotBits), "rank bits");
constexpr int kMaxLevels = 12;    // log2(2 host size / smallest leaf): path keys of 5 bits per level fit 64 bits
constexpr int kSortLeaves = 28672;  // hosts with more leaves sort them in global memory
constexpr int kSmemLeaves = 8192;   // hosts with more leaves search them in global memory
constexpr int kSmemQuads = 14336;   // hosts with more quads sort them in global memory
constexpr int kQuadBlock = 256;     // leaves per CTA of the quad enumeration (hosts up to kSmemLeaves)
constexpr int kBigQuadBlock = 512;  // leaves per CTA of the quad enumeration (larger hosts)
constexpr size_t kLeafSmem = (size_t)kSortLeaves * 8;
constexpr size_t kQuadSmem = (size_t)kSmemLeaves * 8;
constexpr size_t kBigQuadSmem = (size_t)kSortLeaves * 8;
constexpr size_t kSortSmem = (size_t)kSmemQuads * 16;
constexpr int kSmallLeaves = 2048;  // leaf sorts up to this size run several CTAs per SM
constexpr int kBucketBits = 6;      // leaves of larger hosts are sorted in 64 Morton-prefix buckets
constexpr int kBuckets = 1 << kBucketBits;
constexpr int kSmallQuads = 2048;   // as do quad sorts up to this size
constexpr size_t kSmallLeafSmem = (size_t)kSmallLeaves * 8;
constexpr size_t kSmallSortSmem = (size_t)kSmallQuads * 16;

// the dual-contouring tables of contour_constants.h, as the reference's
// recursion uses them (its output order depends on them)
__constant__ int8_t cEdgeVMap[12][2] = {{0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 2}, {1, 3},
                                        {4, 6}, {5, 7}, {0, 1}, {2, 3}, {4, 5}, {6, 7}};
__constant__ int8_t cCellProcFaceMask[12][3] = {{0, 4, 0}, {1, 5, 0}, {2, 6, 0}, {3, 7, 0}, {0, 2, 1}, {4, 6, 1},
                                                {1, 3, 1}, {5, 7, 1}, {0, 1, 2}, {2, 3, 2}, {4, 5, 2}, {6, 7, 2}};
__constant__ int8_t cCellProcEdgeMask[6][5] = {{0, 1, 2, 3, 0}, {4, 5, 6, 7, 0}, {0, 4, 1, 5, 1},
                                               {2, 6, 3, 7, 1}, {0, 2, 4, 6, 2}, {1, 3, 5, 7, 2}};
__constant__ int8_t cFaceProcFaceMask[3][4][3] = {{{4, 0, 0}, {5, 1, 0}, {6, 2, 0}, {7, 3, 0}},
                                                  {{2, 0, 1}, {6, 4, 1}, {3, 1, 1}, {7, 5, 1}},
                                                  {{1, 0, 2}, {3, 2, 2}, {5, 4, 2}, {7, 6, 2}}};
__constant__ int8_t cFaceProcEdgeMask[3][4][6] = {
    {{1, 4, 0, 5, 1, 1}, {1, 6, 2, 7, 3, 1}, {0, 4, 6, 0, 2, 2}, {0, 5, 7, 1, 3, 2}},
    {{0, 2, 3, 0, 1, 0}, {0, 6, 7, 4, 5, 0}, {1, 2, 0, 6, 4, 2}, {1, 3, 1, 7, 5, 2}},
    {{1, 1, 0, 3, 2, 0}, {1, 5, 4, 7, 6, 0}, {0, 1, 5, 0, 4, 1}, {0, 3, 7, 2, 6, 1}}};
__constant__ int8_t cProcessEdgeMask[3][4] = {{3, 2, 1, 0}, {7, 5, 6, 4}, {11, 10, 9, 8}};

__device__ __forceinline__ int cbit(int child, int axis) { return (child >> (2 - axis)) & 1; }


struct SeamHost {
    int32_t min[3];
    int32_t size;
    int32_t unit;        // smallest leaf size among the gathered chunks
    int32_t lev;         // log2(2 size / unit)
    int32_t pair_begin;  // gathered (chunk, neighbour mask) pairs
    int32_t pair_end;
    int64_t sel_off;     // the host's selected seam nodes (room for every node of its pairs)
    int64_t leaf_off;    // the host's leaves in the leaf arrays
    int64_t quad_off;    // the host's quads (12 per leaf at most) in the quad arrays
};

struct SeamArgs {
    const SeamHost* hosts;
    const int4* pairs;            // (chunk, mask of neighbour indices 0-7, host, -)
    const int4* chunks;           // (min xyz, size)
    const int32_t* seam_offsets;  // [num_chunks + 1]
    const lvn_seam_node* seams;
    int vpc;
    int32_t* counts;    // leaves per host
    int32_t* qcounts;   // quads per host
    uint64_t* sel;      // selected leaves' sort entries, per host at sel_off, by bucket
    uint32_t* slots;    // their seam indices, by the slot in the entry
    int32_t* bcount;    // leaves per (host, Morton-prefix bucket)
    const int32_t* bstart;  // the bucket's first slot in the host's region
    int32_t* cursor;    // next slot in the bucket
    const int4* lsort;  // leaf sorts: (host, first slot, count, -)
    uint64_t* ent;      // sorted leaf entries
    uint32_t* leaves;   // seam index per rank
    uint64_t* qkey;     // quad path keys
    uint64_t* qval;     // quad payloads (sorted by key after the sort kernel)
    const int2* items;  // quad enumeration: (host, first leaf)
    // emit
    const int64_t* vout_off;
    const int64_t* tout_off;
    lvn_mesh_vertex* vout;
    lvn_mesh_triangle* tout;
    float colour[3];
};

// FilterSeamNode (clipmap.cpp:508-538)
__device__ __forceinline__ bool filter_seam_node(int child, const int32_t b[3], const int32_t mn[3],
                                                 const int32_t mx[3]) {
    switch (child) {
        case 0: return mx[0] == b[0] || mx[1] == b[1] || mx[2] == b[2];
        case 1: return mn[2] == b[2];
        case 2: return mn[1] == b[1];
        case 3: return mn[1] == b[1] || mn[2] == b[2];
        case 4: return mn[0] == b[0];
        case 5: return mn[0] == b[0] || mn[2] == b[2];
        case 6: return mn[0] == b[0] || mn[1] == b[1];
        default: return mn[0] == b[0] && mn[1] == b[1] && mn[2] == b[2];
    }
}

// SelectSeamNodes (clipmap.cpp:542-570): is seam node k of `chunk` one of the
// host's, for any of the neighbour indices in `mask`?  A chunk reached through
// several neighbour indices is tested once with all of them (the reference
// may list such a node twice; the octree it builds holds it once).
__device__ __forceinline__ bool seam_selected(const SeamHost& h, int4 chunk, int mask, const lvn_seam_node& s,
                                              int vpc, int32_t mn[3]) {
    const int node_size = chunk.w / vpc;
    const int extent = (chunk.w / (vpc * 4)) * 4;  // size * LEAF_SIZE_SCALE (clipmap.cpp:553-560)
    mn[0] = s.localspace_min[0] * node_size + chunk.x;
    mn[1] = s.localspace_min[1] * node_size + chunk.y;
    mn[2] = s.localspace_min[2] * node_size + chunk.z;
    for (int a = 0; a < 3; a++)
        if (mn[a] < h.min[a] || mn[a] >= h.min[a] + 2 * h.size) return false;  // AABB::pointIsInside
    const int32_t b[3] = {h.min[0] + h.size, h.min[1] + h.size, h.min[2] + h.size};
    const int32_t mx[3] = {mn[0] + extent, mn[1] + extent, mn[2] + extent};
    for (int i = 0; i < 8; i++)
        if (((mask >> i) & 1) && filter_seam_node(i, b, mn, mx)) return true;
    return false;
}

// bit interleaving by shifts and masks (bit i of v to bit 3i), and back
__device__ __forceinline__ uint64_t part1by2(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}

__device__ __forceinline__ uint32_t compact1by2(uint64_t v) {
    v &= 0x1249249249249249ull;
    v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
    v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
    v = (v ^ (v >> 8)) & 0x1f0000ff0000ffull;
    v = (v ^ (v >> 16)) & 0x1f00000000ffffull;
    v = (v ^ (v >> 32)) & 0x1fffffull;
    return (uint32_t)v;
}

// Morton code of a host-relative position in units of 1 << unit_log: x in
// the highest bit of each triple, as the octree's children are numbered
__device__ __forceinline__ uint64_t morton(const int32_t rel[3], int unit_log, int lev) {
    (void)lev;
    return (part1by2((uint32_t)rel[0] >> unit_log) << 2) | (part1by2((uint32_t)rel[1] >> unit_log) << 1) |
           part1by2((uint32_t)rel[2] >> unit_log);
}

__device__ __forceinline__ void unmorton(uint64_t code, int lev, int unit_log, int32_t rel[3]) {
    (void)lev;
    rel[0] = (int32_t)(compact1by2(code >> 2) << unit_log);
    rel[1] = (int32_t)(compact1by2(code >> 1) << unit_log);
    rel[2] = (int32_t)(compact1by2(code) << unit_log);
}

// SelectSeamNodes for every (host, gathered chunk) pair.  The counting pass
// (Place = false) counts the selected seam nodes per host and per bucket of
// the top kBucketBits bits of their host-relative Morton code (units of the
// host's smallest leaf); the placing pass writes each one's sort entry
// ((morton << 4 | size log2) << 15 | slot) and seam index at a slot of its
// bucket, so that each host's region holds its buckets in Morton order.
template <bool Place>
__global__ void __launch_bounds__(128) k_seam_select(SeamArgs A) {
    const int4 pr = A.pairs[blockIdx.x];
    const SeamHost h = A.hosts[pr.z];
    const int4 ch = A.chunks[pr.x];
    int unit_log = 0;
    while ((1 << unit_log) < h.unit) unit_log++;
    int size_log = 0;
    while ((h.unit << size_log) < ch.w / A.vpc) size_log++;
    const int s0 = A.seam_offsets[pr.x], s1 = A.seam_offsets[pr.x + 1];
    const int lane = threadIdx.x & 31;
    const int shift = 3 * h.lev - kBucketBits;  // lev >= 4: 2 host size / smallest leaf >= 16
    for (int base = s0; base < s1; base += blockDim.x) {
        const int k = base + threadIdx.x;
        int32_t mn[3];
        const bool take = k < s1 && seam_selected(h, ch, pr.y, A.seams[k], A.vpc, mn);
        if (!Place) {
            const unsigned ballot = __ballot_sync(0xffffffffu, take);
            if (lane == 0 && ballot) atomicAdd(&A.counts[pr.z], __popc(ballot));
        }
        if (!take) continue;
        const int32_t rel[3] = {mn[0] - h.min[0], mn[1] - h.min[1], mn[2] - h.min[2]};
        const uint64_t code = morton(rel, unit_log, h.lev);
        const int b = pr.z * kBuckets + (int)(code >> shift);
        if (!Place) {
            atomicAdd(&A.bcount[b], 1);
            continue;
        }
        const int slot = A.bstart[b] + atomicAdd(&A.cursor[b], 1);
        if (slot >= kMaxLeaves) continue;  // the host reported the count; nothing past its region is written
        A.sel[h.sel_off + slot] = ((code << 4 | (uint64_t)size_log) << kSlotBits) | (uint64_t)slot;
        A.slots[h.sel_off + slot] = (uint32_t)k;
    }
}

// Ascending sort of n entries in place (a bitonic network whose first step of
// each merge compares mirrored positions, so every comparator is ascending and
// entries past n never move: any n, no padding), keys with an optional payload.
template <bool Pair>
__device__ void block_sort(uint64_t* key, uint64_t* val, int n) {
    for (int k = 2; k < 2 * n; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int mask = j == (k >> 1) ? k - 1 : j;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int l = i ^ mask;
                if (l > i && l < n) {
                    const uint64_t a = key[i], b = key[l];
                    if (a > b) {
                        key[i] = b;
                        key[l] = a;
                        if (Pair) {
                            const uint64_t t = val[i];
                            val[i] = val[l];
                            val[l] = t;
                        }
                    }
                }
            }
            __syncthreads();
        }
    }
}

struct LeafView {
    const uint64_t* ent;  // sorted entries
    int n;
    int lev, unit_log;
    int32_t root;  // 2 host size
};

__device__ __forceinline__ uint64_t ent_code(uint64_t e) { return e >> (kSlotBits + 4); }
__device__ __forceinline__ int ent_size_log(uint64_t e) { return (int)((e >> kSlotBits) & 15); }

// The leaf covering the region (min rel, size 1 << size_log units): its rank,
// -1 when nothing is there (a null child in the reference's tree), -2 when the
// region is subdivided (smaller leaves inside).
__device__ int find_leaf(const LeafView& v, const int32_t rel[3], int size_log) {
    for (int a = 0; a < 3; a++)
        if (rel[a] < 0 || rel[a] >= v.root) return -1;
    const uint64_t k = morton(rel, v.unit_log, v.lev);
    const uint64_t vol = 1ull << (3 * size_log);
    int lo = 0, hi = v.n;  // first entry with code >= k
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ent_code(v.ent[mid]) < k)
            lo = mid + 1;
        else
            hi = mid;
    }
    if (lo < v.n && ent_code(v.ent[lo]) < k + vol) {
        if (ent_code(v.ent[lo]) == k && ent_size_log(v.ent[lo]) >= size_log) return lo;
        return -2;
    }
    if (lo > 0) {  // a larger leaf before it in Morton order may contain the region
        const uint64_t e = v.ent[lo - 1];
        const int sl = ent_size_log(e);
        if (sl > size_log && (k >> (3 * sl)) == (ent_code(e) >> (3 * sl))) return lo - 1;
    }
    return -1;
}

__device__ __forceinline__ int log2_units(int32_t size, int32_t unit) {
    int l = 0;
    while ((unit << l) < size) l++;
    return l;
}

// The path of the reference's recursion (ContourCellProc from the seam
// octree's root) to the final segment along `dir` at line coordinates line[]
// (host-relative), starting at t0 along dir, `len` long.
__device__ uint64_t path_key(int32_t root, int dir, const int32_t line[3], int32_t t0, int32_t len) {
    uint64_t key = 0;
    int nbits = 0;
    auto put = [&](int digit, int width) {
        nbits += width;
        key |= (uint64_t)digit << (64 - nbits);
    };
    const int a1 = dir == 0 ? 1 : 0, a2 = dir == 2 ? 1 : 2;
    int32_t m[3] = {0, 0, 0};
    int32_t S = root;
    int32_t e0 = 0, es = 0;  // edge state: start along dir, length
    for (;;) {  // cell
        const int32_t h = S >> 1;
        const int32_t mid[3] = {m[0] + h, m[1] + h, m[2] + h};
        const bool on1 = line[a1] == mid[a1], on2 = line[a2] == mid[a2];
        const int hd = t0 >= mid[dir];
        if (!on1 && !on2) {
            int c = hd << (2 - dir);
            c |= (line[a1] > mid[a1]) << (2 - a1);
            c |= (line[a2] > mid[a2]) << (2 - a2);
            put(c, 5);
            for (int a = 0; a < 3; a++) m[a] += cbit(c, a) * h;
            S = h;
            continue;
        }
        if (on1 && on2) {
            int e = 0;
            for (int i = 0; i < 6; i++)
                if (cCellProcEdgeMask[i][4] == dir && cbit(cCellProcEdgeMask[i][0], dir) == hd) e = i;
            put(20 + e, 5);
            e0 = m[dir] + hd * h;
            es = h;
            break;
        }
        const int a = on1 ? a1 : a2, b = on1 ? a2 : a1;
        const int bs = line[b] > mid[b];
        const int c0 = (bs << (2 - b)) | (hd << (2 - dir)), c1 = c0 | (1 << (2 - a));
        int f = 0;
        for (int i = 0; i < 12; i++)
            if (cCellProcFaceMask[i][0] == c0 && cCellProcFaceMask[i][1] == c1) f = i;
        put(8 + f, 5);
        int32_t fb = m[b] + bs * h, fd = m[dir] + hd * h, fs = h;
        for (;;) {  // face, plane perpendicular to a
            const int32_t hh = fs >> 1;
            const int fhd = t0 >= fd + hh;
            if (line[b] != fb + hh) {
                const int fbs = line[b] > fb + hh;
                int i4 = 0;
                for (int i = 0; i < 4; i++) {
                    const int c = cFaceProcFaceMask[a][i][1];
                    if (cbit(c, b) == fbs && cbit(c, dir) == fhd) i4 = i;
                }
                put(i4, 3);
                fb += fbs * hh;
                fd += fhd * hh;
                fs = hh;
                continue;
            }
            int i4 = 0;
            for (int i = 0; i < 4; i++)
                if (cFaceProcEdgeMask[a][i][5] == dir && cbit(cFaceProcEdgeMask[a][i][1], dir) == fhd) i4 = i;
            put(4 + i4, 3);
            e0 = fd + fhd * hh;
            es = hh;
            break;
        }
        break;
    }
    while (es > len) {  // edge: halves along dir
        const int32_t eh = es >> 1;
        const int hf = t0 >= e0 + eh;
        put(hf, 1);
        e0 += hf * eh;
        es = eh;
    }
    return key;
}

// Leaf sort lsort[blockIdx.x] = (host, first, count): the host's slots
// [first, first + count) sorted (in shared memory when they fit `cap`) to
// A.ent and A.leaves at the same positions of the host's leaf range.  A
// small host is one sort; a larger one a sort per Morton-prefix bucket, which
// together order the whole host.
__global__ void __launch_bounds__(1024) k_seam_leaves(SeamArgs A, int cap) {
    extern __shared__ uint64_t smem[];
    const int4 it = A.lsort[blockIdx.x];
    const SeamHost h = A.hosts[it.x];
    const int n = it.z;
    uint64_t* ent = A.sel + h.sel_off + it.y;
    if (n <= cap) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) smem[i] = ent[i];
        __syncthreads();
        ent = smem;
    }
    block_sort<false>(ent, nullptr, n);
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        const uint64_t e = ent[r];
        A.ent[h.leaf_off + it.y + r] = e;
        A.leaves[h.leaf_off + it.y + r] = A.slots[h.sel_off + (e & ((1u << kSlotBits) - 1))];
    }
}

// The quads of the leaves [first, first + block) of one host, unsorted,
// with their recursion path keys.  The host's sorted entries are copied to
// shared memory when they fit `cap`, else searched in global memory.
__global__ void __launch_bounds__(1024) k_seam_quads(SeamArgs A, int block, int cap) {
    extern __shared__ uint64_t smem[];
    const int2 it = A.items[blockIdx.x];
    const SeamHost h = A.hosts[it.x];
    const int n = A.counts[it.x];
    const uint64_t* ent = A.ent + h.leaf_off;
    if (n <= cap) {  // binary searches in shared memory
        for (int i = threadIdx.x; i < n; i += blockDim.x) smem[i] = ent[i];
        __syncthreads();
        ent = smem;
    }
    const int unit_log = log2_units(h.unit, 1);
    LeafView v;
    v.ent = ent;
    v.n = n;
    v.lev = h.lev;
    v.unit_log = unit_log;
    v.root = 2 * h.size;
    const int r_end = min(n, it.y + block);
    for (int item = it.y * 12 + threadIdx.x; item < r_end * 12; item += blockDim.x) {
        const int r = item / 12, e = item - 12 * r;
        const uint64_t me = ent[r];
        const int corners = A.seams[A.leaves[h.leaf_off + r]].localspace_min[3] & 0xff;
        const int c0 = cEdgeVMap[e][0], c1 = cEdgeVMap[e][1];
        const int m0 = (corners >> c0) & 1, m1 = (corners >> c1) & 1;
        if (m0 == m1) continue;  // no sign change on the edge of the smallest leaf: no quad
        const int dir = e >> 2;
        int j = 0;
        for (int q = 0; q < 4; q++)
            if (cProcessEdgeMask[dir][q] == e) j = q;
        const int sl = ent_size_log(me);
        const int32_t s = h.unit << sl;
        int32_t lmin[3];
        unmorton(ent_code(me), h.lev, unit_log, lmin);
        int32_t line[3];
        for (int a = 0; a < 3; a++) line[a] = lmin[a] + cbit(c0, a) * s;
        // the four leaves around the edge, in the order ContourEdgeProc passes
        // them (the children of cellProcEdgeMask's first entry along dir)
        int rank[4];
        bool ok = true;
        for (int q = 0; q < 4 && ok; q++) {
            if (q == j) {
                rank[q] = r;
                continue;
            }
            const int child = cCellProcEdgeMask[2 * dir][q];
            int32_t rel[3];
            for (int a = 0; a < 3; a++) rel[a] = a == dir ? lmin[a] : line[a] - s + cbit(child, a) * s;
            rank[q] = find_leaf(v, rel, sl);
            ok = rank[q] >= 0;
        }
        if (!ok) continue;
        int min_index = 0, min_log = 64;  // ContourProcessEdge: the first of the smallest leaves
        for (int q = 0; q < 4; q++) {
            const int lq = ent_size_log(ent[rank[q]]);
            if (lq < min_log) {
                min_log = lq;
                min_index = q;
            }
        }
        if (min_index != j) continue;  // that leaf's edge is this segment: it emits the quad
        // the straddle test: not all four leaves in one CLIPMAP_LEAF_SIZE block
        bool one_block = true;
        int32_t b0[3];
        for (int q = 0; q < 4; q++) {
            int32_t rel[3];
            unmorton(ent_code(ent[rank[q]]), h.lev, unit_log, rel);
            for (int a = 0; a < 3; a++) {
                const int32_t blk = (int32_t)((uint32_t)(rel[a] + h.min[a]) & ~(uint32_t)(CLIPMAP_LEAF_SIZE - 1));
                if (q == 0)
                    b0[a] = blk;
                else
                    one_block &= blk == b0[a];
            }
        }
        if (one_block) continue;
        const int qi = atomicAdd(&A.qcounts[it.x], 1);  // < 12 n: every leaf edge emits at most once
        A.qkey[h.quad_off + qi] = path_key(2 * h.size, dir, line, lmin[dir], s);
        A.qval[h.quad_off + qi] = (uint64_t)rank[0] | ((uint64_t)rank[1] << kRankBits) |
                                  ((uint64_t)rank[2] << (2 * kRankBits)) | ((uint64_t)rank[3] << (3 * kRankBits)) |
                                  ((uint64_t)(m1 != 1) << (4 * kRankBits));
    }
}

// The quads of host list[blockIdx.x] in the recursion's order: payloads
// sorted in place, in shared memory when they fit `cap`.  With `only_above`,
// hosts with at most that many quads are left to the other size class.
__global__ void __launch_bounds__(1024) k_seam_qsort(SeamArgs A, const int32_t* list, int cap, int only_above) {
    extern __shared__ uint64_t smem[];
    const int hi = list[blockIdx.x];
    const SeamHost h = A.hosts[hi];
    const int nq = A.qcounts[hi];
    if (nq <= only_above || (only_above < 0 && nq > kSmallQuads)) return;
    uint64_t* key = A.qkey + h.quad_off;
    uint64_t* val = A.qval + h.quad_off;
    if (nq <= cap) {
        uint64_t* sk = smem;
        uint64_t* sv = smem + cap;
        for (int i = threadIdx.x; i < nq; i += blockDim.x) {
            sk[i] = key[i];
            sv[i] = val[i];
        }
        __syncthreads();
        block_sort<true>(sk, sv, nq);
        for (int i = threadIdx.x; i < nq; i += blockDim.x) val[i] = sv[i];
    } else {
        block_sort<true>(key, val, nq);
    }
}

// vertices (hosts with triangles only) and triangles, back to back by host;
// blockIdx.y splits a host's ranges over gridDim.y CTAs
__global__ void __launch_bounds__(256) k_seam_emit(SeamArgs A) {
    const SeamHost h = A.hosts[blockIdx.x];
    const int nq = A.qcounts[blockIdx.x];
    if (nq <= 0) return;
    const int n = A.counts[blockIdx.x];
    const int64_t vo = A.vout_off[blockIdx.x], to = A.tout_off[blockIdx.x];
    const int t0 = blockIdx.y * blockDim.x + threadIdx.x, step = gridDim.y * blockDim.x;
    for (int r = t0; r < n; r += step) {
        const lvn_seam_node s = A.seams[A.leaves[h.leaf_off + r]];
        lvn_mesh_vertex v;
        for (int a = 0; a < 3; a++) {
            v.position[a] = s.position[a];
            v.normal[a] = s.normal[a];
            v.colour[a] = A.colour[a];
        }
        v.position[3] = 0.f;
        v.normal[3] = 0.f;
        v.colour[3] = (float)(s.localspace_min[3] >> 8);
        A.vout[vo + r] = v;
    }
    const uint64_t mask = (1ull << kRankBits) - 1;
    for (int i = t0; i < nq; i += step) {
        const uint64_t q = A.qval[h.quad_off + i];
        const int i0 = (int)(q & mask), i1 = (int)((q >> kRankBits) & mask), i2 = (int)((q >> (2 * kRankBits)) & mask),
                  i3 = (int)((q >> (3 * kRankBits)) & mask);
        const bool flip = (q >> (4 * kRankBits)) & 1;
        lvn_mesh_triangle t0, t1;
        if (!flip) {
            t0 = {{i0, i1, i3}};
            t1 = {{i0, i3, i2}};
        } else {
            t0 = {{i0, i3, i1}};
            t1 = {{i0, i2, i3}};
        }
        A.tout[to + 2 * i] = t0;
        A.tout[to + 2 * i + 1] = t1;
    }
}

// ---- host side -----------------------------------------------------------

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

struct SeamWork {
    std::mutex mu;
    int device = -1;
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_fork2 = nullptr, ev_join2 = nullptr;
    Grow<SeamHost> hosts;
    Grow<int4> pairs;
    Grow<int4> chunks;
    Grow<int32_t> seam_offsets, counts, qcounts;
    Grow<lvn_seam_node> seams;
    Grow<uint64_t> sel, ent, qkey, qval;
    Grow<uint32_t> slots, leaves;
    Grow<int2> items;
    Grow<int32_t> lists, bcount, bstart, cursor;
    Grow<int4> lsort;
    Grow<int32_t, true> hbuckets;  // pinned
    Grow<int64_t> offs;  // vertex offsets, triangle offsets
    Grow<lvn_mesh_vertex> vstage;
    Grow<lvn_mesh_triangle> tstage;
    Grow<int32_t, true> hcounts;  // pinned: counts, qcounts
};
SeamWork& seam_work() {
    static SeamWork w;
    return w;
}

int cuda_rc(cudaError_t e) {
    if (e == cudaSuccess) return LVN_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? LVN_ERR_OUT_OF_MEMORY : LVN_ERR_CUDA;
}

#define SM_TRY(x)                        \
    do {                                 \
        const int rc__ = cuda_rc(x);     \
        if (rc__ != LVN_OK) return rc__; \
    } while (0)

// Open-addressing hash table of 64-bit keys (linear probing, never full).
class FlatTable {
   public:
    void reserve(size_t n) {
        size_t cap = 16;
        while (cap < 4 * n) cap <<= 1;
        keys_.assign(cap, kEmpty);
        vals_.assign(cap, -1);
        mask_ = cap - 1;
    }
    // inserts (key, val) unless key is present; returns false when it was
    bool insert(uint64_t key, int32_t val) {
        for (size_t i = slot(key);; i = (i + 1) & mask_) {
            if (keys_[i] == key) return false;
            if (keys_[i] == kEmpty) {
                keys_[i] = key;
                vals_[i] = val;
                return true;
            }
        }
    }
    int32_t find(uint64_t key) const {  // -1 when absent
        for (size_t i = slot(key);; i = (i + 1) & mask_) {
            if (keys_[i] == key) return vals_[i];
            if (keys_[i] == kEmpty) return -1;
        }
    }

   private:
    static constexpr uint64_t kEmpty = ~0ull;
    size_t slot(uint64_t key) const { return (size_t)((key * 0x9e3779b97f4a7c15ull) >> 20) & mask_; }
    std::vector<uint64_t> keys_;
    std::vector<int32_t> vals_;
    size_t mask_ = 0;
};

// The clipmap's active nodes (the chunks) and the nodes above them;
// FindNode / FindActiveNodes (clipmap.cpp:982-1013, 1449-1479) over the
// complete octree rooted at (root_min, root_size).  A node is keyed by its
// root-relative position in CLIPMAP_LEAF_SIZE units (19 bits per axis: roots
// up to 2^27) and log2(size / CLIPMAP_LEAF_SIZE).
struct ActiveSet {
    int32_t root_min[3];
    int32_t root_size;
    FlatTable active;  // -> chunk index
    FlatTable above;   // nodes with an active node below them (value unused)

    uint64_t key(const int32_t mn[3], int32_t size) const {
        int lg = 0;
        while ((CLIPMAP_LEAF_SIZE << lg) < size) lg++;
        uint64_t k = 0;
        for (int a = 0; a < 3; a++) k = (k << 19) | (uint64_t)(((int64_t)mn[a] - root_min[a]) / CLIPMAP_LEAF_SIZE);
        return (k << 5) | (uint64_t)lg;
    }
    bool in_root(const int32_t mn[3], int32_t size) const {
        for (int a = 0; a < 3; a++) {
            const int64_t rel = (int64_t)mn[a] - root_min[a];
            if (rel < 0 || rel + size > root_size || rel % size) return false;
        }
        return true;
    }
    // the active nodes FindActiveNodes lists for the node (mn, size)
    void find_active(const int32_t mn[3], int32_t size, std::vector<int>& out) const {
        // an active node containing mn (the node itself or above it)
        for (int32_t s = size; s <= root_size; s *= 2) {
            int32_t a[3];
            for (int k = 0; k < 3; k++) a[k] = root_min[k] + (int32_t)(((int64_t)mn[k] - root_min[k]) / s * s);
            const int32_t c = active.find(key(a, s));
            if (c >= 0) {
                out.push_back(c);
                return;
            }
        }
        descend(mn, size, out);
    }
    void descend(const int32_t mn[3], int32_t size, std::vector<int>& out) const {
        if (size <= CLIPMAP_LEAF_SIZE || above.find(key(mn, size)) < 0) return;
        const int32_t h = size / 2;
        for (int i = 0; i < 8; i++) {
            const int32_t c[3] = {mn[0] + ((i >> 2) & 1) * h, mn[1] + ((i >> 1) & 1) * h, mn[2] + (i & 1) * h};
            const int32_t ci = active.find(key(c, h));
            if (ci >= 0)
                out.push_back(ci);
            else
                descend(c, h, out);
        }
    }
};

}  // namespace
}  // namespace lvn

using namespace lvn;

extern "C" {

int lvn_seam_generate(const lvn_chunk_desc* chunks, const int32_t* seam_offsets, int32_t num_chunks,
                      const lvn_seam_node* seams, int32_t seams_memory, int32_t voxels_per_chunk,
                      const int32_t root_min[3], int32_t root_size, const int32_t* hosts, int32_t num_hosts,
                      const float colour[3], lvn_batch_out* out) {
    if (!out || !root_min || !colour || num_chunks < 0 || num_hosts < 0 || (num_chunks > 0 && (!chunks || !seam_offsets)) ||
        (num_hosts > 0 && !hosts) || voxels_per_chunk < 8 || voxels_per_chunk > 64 ||
        (voxels_per_chunk & (voxels_per_chunk - 1)) || (seams_memory != LVN_MEMORY_HOST && seams_memory != LVN_MEMORY_DEVICE) ||
        (out->memory != LVN_MEMORY_HOST && out->memory != LVN_MEMORY_DEVICE) || (num_hosts > 0 && !out->chunks))
        return LVN_ERR_INVALID;
    if (root_size < CLIPMAP_LEAF_SIZE || (root_size & (root_size - 1))) return LVN_ERR_INVALID;
    const int vpc = voxels_per_chunk;
    if (root_size > (1 << 27)) return LVN_ERR_INVALID;
    ActiveSet act;
    for (int a = 0; a < 3; a++) act.root_min[a] = root_min[a];
    act.root_size = root_size;
    act.active.reserve((size_t)num_chunks);
    act.above.reserve((size_t)num_chunks * 4 + 16);
    for (int c = 0; c < num_chunks; c++) {
        const lvn_chunk_desc& d = chunks[c];
        if (d.size < CLIPMAP_LEAF_SIZE || (d.size & (d.size - 1)) || !act.in_root(d.min, d.size) ||
            seam_offsets[c + 1] < seam_offsets[c])
            return LVN_ERR_INVALID;
        if (!act.active.insert(act.key(d.min, d.size), c)) return LVN_ERR_INVALID;  // listed twice
    }
    for (int c = 0; c < num_chunks; c++) {
        const lvn_chunk_desc& d = chunks[c];
        for (int32_t s = d.size * 2; s <= root_size; s *= 2) {
            int32_t a[3];
            for (int k = 0; k < 3; k++) a[k] = root_min[k] + (int32_t)(((int64_t)d.min[k] - root_min[k]) / s * s);
            // the clipmap's active nodes never overlap: an active node above an active node is an error
            if (act.active.find(act.key(a, s)) >= 0) return LVN_ERR_INVALID;
            if (!act.above.insert(act.key(a, s), 0)) break;
        }
    }
    const int64_t num_seams = num_chunks ? seam_offsets[num_chunks] : 0;
    if (seam_offsets && num_chunks && seam_offsets[0] != 0) return LVN_ERR_INVALID;
    // the gathered (chunk, neighbour mask) pairs of every host
    std::vector<SeamHost> hv(num_hosts);
    std::vector<int4> pairs;
    for (int hi = 0; hi < num_hosts; hi++) {
        if (hosts[hi] < 0 || hosts[hi] >= num_chunks) return LVN_ERR_INVALID;
        const lvn_chunk_desc& d = chunks[hosts[hi]];
        SeamHost& h = hv[hi];
        for (int a = 0; a < 3; a++) h.min[a] = d.min[a];
        h.size = d.size;
        h.pair_begin = (int32_t)pairs.size();
        std::vector<std::pair<int, int>> found;  // (chunk, neighbour index)
        for (int i = 0; i < 8; i++) {
            const int32_t nmin[3] = {d.min[0] + ((i >> 2) & 1) * d.size, d.min[1] + ((i >> 1) & 1) * d.size,
                                     d.min[2] + (i & 1) * d.size};
            if (!act.in_root(nmin, d.size)) continue;  // Clipmap::findNode finds no node there
            std::vector<int> cs;
            act.find_active(nmin, d.size, cs);
            for (int c : cs) found.push_back({c, i});
        }
        std::sort(found.begin(), found.end());
        int unit = d.size / vpc;
        for (size_t k = 0; k < found.size();) {
            int mask = 0;
            const int c = found[k].first;
            for (; k < found.size() && found[k].first == c; k++) mask |= 1 << found[k].second;
            pairs.push_back(make_int4(c, mask, hi, 0));
            unit = std::min(unit, chunks[c].size / vpc);
        }
        h.pair_end = (int32_t)pairs.size();
        h.unit = unit;
        h.lev = 0;
        while ((unit << h.lev) < 2 * d.size) h.lev++;
        if (h.lev > kMaxLevels) return LVN_ERR_INVALID;
    }
    SeamWork& w = seam_work();
    std::lock_guard<std::mutex> lock(w.mu);
    int dev = 0;
    SM_TRY(cudaGetDevice(&dev));
    if (w.device != dev) {
        if (w.device >= 0) return LVN_ERR_INVALID;  // the scratch lives on the first device used
        SM_TRY(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
        SM_TRY(cudaStreamCreateWithFlags(&w.side, cudaStreamNonBlocking));
        SM_TRY(cudaEventCreateWithFlags(&w.ev_fork, cudaEventDisableTiming));
        SM_TRY(cudaEventCreateWithFlags(&w.ev_join, cudaEventDisableTiming));
        SM_TRY(cudaEventCreateWithFlags(&w.ev_fork2, cudaEventDisableTiming));
        SM_TRY(cudaEventCreateWithFlags(&w.ev_join2, cudaEventDisableTiming));
        SM_TRY(cudaFuncSetAttribute(k_seam_leaves, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLeafSmem));
        SM_TRY(cudaFuncSetAttribute(k_seam_quads, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBigQuadSmem));
        SM_TRY(cudaFuncSetAttribute(k_seam_qsort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSortSmem));
        w.device = dev;
    }
    if (num_hosts == 0) {
        out->total_vertices = out->total_triangles = out->total_seams = 0;
        return LVN_OK;
    }
    const size_t nh = (size_t)num_hosts;
    SM_TRY(w.hosts.fit(nh));
    SM_TRY(w.pairs.fit(std::max<size_t>(pairs.size(), 1)));
    int64_t sel_total = 0;
    for (size_t i = 0; i < nh; i++) {
        hv[i].sel_off = sel_total;
        for (int p = hv[i].pair_begin; p < hv[i].pair_end; p++)
            sel_total += seam_offsets[pairs[p].x + 1] - seam_offsets[pairs[p].x];
    }
    SM_TRY(w.sel.fit(std::max<int64_t>(sel_total, 1)));
    SM_TRY(w.slots.fit(std::max<int64_t>(sel_total, 1)));
    SM_TRY(w.chunks.fit(std::max(num_chunks, 1)));
    SM_TRY(w.seam_offsets.fit((size_t)num_chunks + 1));
    SM_TRY(w.counts.fit(nh));
    SM_TRY(w.qcounts.fit(nh));
    SM_TRY(w.offs.fit(2 * nh));
    SM_TRY(w.hcounts.fit(2 * nh));
    std::vector<int4> c4(std::max(num_chunks, 1));
    for (int c = 0; c < num_chunks; c++)
        c4[c] = make_int4(chunks[c].min[0], chunks[c].min[1], chunks[c].min[2], chunks[c].size);
    cudaStream_t st = w.stream;
    SM_TRY(cudaMemcpyAsync(w.pairs.p, pairs.data(), sizeof(int4) * pairs.size(), cudaMemcpyHostToDevice, st));
    SM_TRY(cudaMemcpyAsync(w.chunks.p, c4.data(), sizeof(int4) * num_chunks, cudaMemcpyHostToDevice, st));
    SM_TRY(cudaMemcpyAsync(w.seam_offsets.p, seam_offsets, sizeof(int32_t) * (num_chunks + 1), cudaMemcpyHostToDevice,
                           st));
    const lvn_seam_node* dseams = seams;
    if (seams_memory == LVN_MEMORY_HOST && num_seams > 0) {
        SM_TRY(w.seams.fit((size_t)num_seams));
        SM_TRY(cudaMemcpyAsync(w.seams.p, seams, sizeof(lvn_seam_node) * num_seams, cudaMemcpyHostToDevice, st));
        dseams = w.seams.p;
    }
    SeamArgs A;
    std::memset(&A, 0, sizeof(A));
    A.hosts = w.hosts.p;
    A.pairs = w.pairs.p;
    A.chunks = w.chunks.p;
    A.seam_offsets = w.seam_offsets.p;
    A.seams = dseams;
    A.vpc = vpc;
    A.counts = w.counts.p;
    A.qcounts = w.qcounts.p;
    for (int a = 0; a < 3; a++) A.colour[a] = colour[a];
    A.sel = w.sel.p;
    A.slots = w.slots.p;
    const size_t nb = nh * kBuckets;
    SM_TRY(w.bcount.fit(nb));
    SM_TRY(w.bstart.fit(nb));
    SM_TRY(w.cursor.fit(nb));
    SM_TRY(w.hbuckets.fit(nb));
    A.bcount = w.bcount.p;
    A.bstart = w.bstart.p;
    A.cursor = w.cursor.p;
    // 1: the selected seam nodes of every host, counted by bucket
    SM_TRY(cudaMemcpyAsync(w.hosts.p, hv.data(), sizeof(SeamHost) * nh, cudaMemcpyHostToDevice, st));
    SM_TRY(cudaMemsetAsync(w.counts.p, 0, sizeof(int32_t) * nh, st));
    SM_TRY(cudaMemsetAsync(w.bcount.p, 0, sizeof(int32_t) * nb, st));
    SM_TRY(cudaMemsetAsync(w.cursor.p, 0, sizeof(int32_t) * nb, st));
    if (!pairs.empty()) {
        k_seam_select<false><<<(int)pairs.size(), 128, 0, st>>>(A);
        SM_TRY(cudaGetLastError());
    }
    SM_TRY(cudaMemcpyAsync(w.hcounts.p, w.counts.p, sizeof(int32_t) * nh, cudaMemcpyDeviceToHost, st));
    SM_TRY(cudaMemcpyAsync(w.hbuckets.p, w.bcount.p, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, st));
    SM_TRY(cudaStreamSynchronize(st));
    // bucket starts, and the leaf sorts: one per small host, one per non-empty bucket of a larger one
    std::vector<int32_t> bstart(nb);
    std::vector<int4> small_sorts, big_sorts;
    for (size_t i = 0; i < nh; i++) {
        int run = 0;
        for (int b = 0; b < kBuckets; b++) {
            bstart[i * kBuckets + b] = run;
            run += w.hbuckets.p[i * kBuckets + b];
        }
        const int n = w.hcounts.p[i];
        if (n == 0) continue;
        if (n <= kSmallLeaves) {
            small_sorts.push_back(make_int4((int)i, 0, n, 0));
            continue;
        }
        for (int b = 0; b < kBuckets; b++) {
            const int c = w.hbuckets.p[i * kBuckets + b];
            if (c) (c <= kSmallLeaves ? small_sorts : big_sorts).push_back(make_int4((int)i, bstart[i * kBuckets + b], c, 0));
        }
    }
    SM_TRY(cudaMemcpyAsync(w.bstart.p, bstart.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice, st));
    if (!pairs.empty()) {
        k_seam_select<true><<<(int)pairs.size(), 128, 0, st>>>(A);
        SM_TRY(cudaGetLastError());
    }
    int64_t leaf_total = 0, quad_total = 0;
    bool limit = false;
    std::vector<int2> items, big_items;  // (host, first leaf) of the quad enumeration's CTAs
    for (size_t i = 0; i < nh; i++) {
        const int n = w.hcounts.p[i];
        limit |= n > kMaxLeaves;
        hv[i].leaf_off = leaf_total;
        hv[i].quad_off = quad_total;
        leaf_total += n;
        quad_total += 12 * (int64_t)n;
        if (n <= kSmemLeaves)
            for (int r = 0; r < n; r += kQuadBlock) items.push_back(make_int2((int)i, r));
        else
            for (int r = 0; r < n; r += kBigQuadBlock) big_items.push_back(make_int2((int)i, r));
    }
    if (limit) return LVN_ERR_DEVICE_STATUS;
    // 2: sorted leaves, quads, quads in order
    SM_TRY(w.ent.fit(std::max<int64_t>(leaf_total, 1)));
    SM_TRY(w.leaves.fit(std::max<int64_t>(leaf_total, 1)));
    SM_TRY(w.qkey.fit(std::max<int64_t>(quad_total, 1)));
    SM_TRY(w.qval.fit(std::max<int64_t>(quad_total, 1)));
    SM_TRY(w.items.fit(std::max<size_t>(items.size() + big_items.size(), 1)));
    SM_TRY(w.lists.fit(nh));
    std::vector<int32_t> lists(nh);
    for (size_t i = 0; i < nh; i++) lists[i] = (int32_t)i;
    SM_TRY(cudaMemcpyAsync(w.lists.p, lists.data(), sizeof(int32_t) * nh, cudaMemcpyHostToDevice, st));
    const size_t n_sorts = small_sorts.size() + big_sorts.size();
    SM_TRY(w.lsort.fit(std::max<size_t>(n_sorts, 1)));
    std::vector<int4> sorts(small_sorts);
    sorts.insert(sorts.end(), big_sorts.begin(), big_sorts.end());
    SM_TRY(cudaMemcpyAsync(w.lsort.p, sorts.data(), sizeof(int4) * n_sorts, cudaMemcpyHostToDevice, st));
    items.insert(items.end(), big_items.begin(), big_items.end());
    const int n_small = (int)(items.size() - big_items.size());
    A.ent = w.ent.p;
    A.leaves = w.leaves.p;
    A.qkey = w.qkey.p;
    A.qval = w.qval.p;
    A.items = w.items.p;
    SM_TRY(cudaMemcpyAsync(w.hosts.p, hv.data(), sizeof(SeamHost) * nh, cudaMemcpyHostToDevice, st));
    SM_TRY(cudaMemcpyAsync(w.items.p, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, st));
    SM_TRY(cudaMemsetAsync(w.qcounts.p, 0, sizeof(int32_t) * nh, st));
    // the large hosts' sorts and enumeration beside the small hosts', on the second stream
    SM_TRY(cudaEventRecord(w.ev_fork, st));
    SM_TRY(cudaStreamWaitEvent(w.side, w.ev_fork, 0));
    if (!big_sorts.empty()) {
        SeamArgs B = A;
        B.lsort = w.lsort.p + small_sorts.size();
        k_seam_leaves<<<(int)big_sorts.size(), 1024, kLeafSmem, w.side>>>(B, kSortLeaves);
        SM_TRY(cudaGetLastError());
    }
    if (!small_sorts.empty()) {
        A.lsort = w.lsort.p;
        k_seam_leaves<<<(int)small_sorts.size(), 256, kSmallLeafSmem, st>>>(A, kSmallLeaves);
        SM_TRY(cudaGetLastError());
    }
    SM_TRY(cudaEventRecord(w.ev_fork2, st));
    SM_TRY(cudaStreamWaitEvent(w.side, w.ev_fork2, 0));  // the enumeration reads every host's sorted leaves
    if (!big_items.empty()) {
        SeamArgs B = A;
        B.items = w.items.p + n_small;
        k_seam_quads<<<(int)big_items.size(), 1024, kBigQuadSmem, w.side>>>(B, kBigQuadBlock, kSortLeaves);
        SM_TRY(cudaGetLastError());
        SM_TRY(cudaEventRecord(w.ev_join, w.side));
    }
    if (n_small) {
        k_seam_quads<<<n_small, 256, kQuadSmem, st>>>(A, kQuadBlock, kSmemLeaves);
        SM_TRY(cudaGetLastError());
    }
    if (!big_items.empty()) SM_TRY(cudaStreamWaitEvent(st, w.ev_join, 0));
    SM_TRY(cudaEventRecord(w.ev_join, st));
    SM_TRY(cudaStreamWaitEvent(w.side, w.ev_join, 0));
    // quad sorts: up to kSmallQuads quads in the small class, the rest (any host) on the side stream
    k_seam_qsort<<<num_hosts, 256, kSmallSortSmem, st>>>(A, w.lists.p, kSmallQuads, -1);
    SM_TRY(cudaGetLastError());
    k_seam_qsort<<<num_hosts, 1024, kSortSmem, w.side>>>(A, w.lists.p, kSmemQuads, kSmallQuads);
    SM_TRY(cudaGetLastError());
    SM_TRY(cudaEventRecord(w.ev_join2, w.side));
    SM_TRY(cudaStreamWaitEvent(st, w.ev_join2, 0));
    SM_TRY(cudaMemcpyAsync(w.hcounts.p + nh, w.qcounts.p, sizeof(int32_t) * nh, cudaMemcpyDeviceToHost, st));
    SM_TRY(cudaStreamSynchronize(st));
    // 3: output layout: hosts with triangles, back to back
    std::vector<int64_t> offs(2 * nh);
    int64_t tv = 0, tt = 0;
    for (size_t i = 0; i < nh; i++) {
        const int nq = w.hcounts.p[nh + i];
        const int nv = nq > 0 ? w.hcounts.p[i] : 0;
        lvn_chunk_result& r = out->chunks[i];
        std::memset(&r, 0, sizeof(r));
        r.vertex_offset = (int32_t)tv;
        r.num_vertices = nv;
        r.triangle_offset = (int32_t)tt;
        r.num_triangles = 2 * nq;
        r.num_nodes = w.hcounts.p[i];
        offs[i] = tv;
        offs[nh + i] = tt;
        tv += nv;
        tt += 2 * nq;
    }
    out->total_vertices = tv;
    out->total_triangles = tt;
    out->total_seams = 0;
    if (tv > out->vertex_capacity || tt > out->triangle_capacity) return LVN_ERR_CAPACITY;
    if (tt == 0) return LVN_OK;
    if ((tv && !out->vertices) || (tt && !out->triangles)) return LVN_ERR_INVALID;
    SM_TRY(cudaMemcpyAsync(w.offs.p, offs.data(), sizeof(int64_t) * 2 * nh, cudaMemcpyHostToDevice, st));
    A.vout_off = w.offs.p;
    A.tout_off = w.offs.p + nh;
    if (out->memory == LVN_MEMORY_DEVICE) {
        A.vout = out->vertices;
        A.tout = out->triangles;
    } else {
        SM_TRY(w.vstage.fit((size_t)tv));
        SM_TRY(w.tstage.fit((size_t)tt));
        A.vout = w.vstage.p;
        A.tout = w.tstage.p;
    }
    k_seam_emit<<<dim3(num_hosts, 16), 256, 0, st>>>(A);
    SM_TRY(cudaGetLastError());
    if (out->memory == LVN_MEMORY_HOST) {
        SM_TRY(cudaMemcpyAsync(out->vertices, w.vstage.p, sizeof(lvn_mesh_vertex) * tv, cudaMemcpyDeviceToHost, st));
        SM_TRY(cudaMemcpyAsync(out->triangles, w.tstage.p, sizeof(lvn_mesh_triangle) * tt, cudaMemcpyDeviceToHost, st));
    }
    SM_TRY(cudaStreamSynchronize(st));
    return LVN_OK;
}

}  // extern "C"
