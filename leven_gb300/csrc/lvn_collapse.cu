// lvn_collapse.cu -- the engine's edge-collapse mesh simplification on the
// GPU: ngMeshSimplifier (leven/src/ng_mesh_simplify.cpp:441-540), which the
// clipmap runs on every chunk mesh after meshing (clipmap.cpp:453-461), for a
// batch of meshes in one launch, one CTA per mesh.
//
// The reference is already a data-parallel algorithm written sequentially:
// each iteration draws a random eighth of the candidate edges, every drawn
// edge that passes the angle / length / material / degree tests and whose
// collapse error (1 / QEF error of its two end points, qef_simd.h) is small
// enough claims both end points, and an edge that holds both claims collapses.
// Here each phase is a parallel pass over the CTA:
//   * the candidate edges are put in the reference's sort order (the union's
//     idx_ = min | max << 32) by a counting sort on max and an insertion sort
//     of each vertex's few entries by min, then reduced to the interior edges
//     by run-length tests;
//   * the draws are the reference's std::mt19937(42) stream (reseeded each
//     iteration) passed through libstdc++'s uniform_int_distribution (Lemire's
//     method: a raw value is rejected when the low half of raw * range falls
//     below (2^32 - range) mod range), from a table the host fills once;
//   * a vertex's claim is the minimum of (error, edge index) over the drawn
//     edges, one 64-bit atomicMin on (orderable error bits << 32 | index),
//     which is what the reference's in-order strict-less updates select;
//   * triangle, edge and vertex removals are order-preserving block scans.
// The QEF is qef_simd.h's lane arithmetic in scalar form with one difference:
// _mm_rsqrt_ps (an approximation that differs between x86 implementations)
// becomes a correctly rounded 1 / sqrt.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <random>
#include <vector>

#include "../../include/lvn.h"

namespace lvn {
namespace {

constexpr int kThreads = 512;    // two CTAs (meshes) per SM
constexpr int kBigThreads = 1024;  // meshes above kBigTriangles: one CTA per SM, on a second stream
constexpr int kBigTriangles = 12000;
constexpr int kSortCap = 12288;  // u64 draws sorted in shared memory (96 KB); more sort in global memory
constexpr size_t kSmem = (size_t)kSortCap * 8;
constexpr int kMaxDegree = 16;  // COLLAPSE_MAX_DEGREE (ng_mesh_simplify.cpp:17)

struct MV {  // MeshVertex
    float p[4], n[4], c[4];
};
static_assert(sizeof(MV) == sizeof(lvn_mesh_vertex), "MeshVertex");

struct MeshJob {
    int32_t v_off, nv, t_off, nt;  // input (and output) ranges
    float offset[4];               // worldSpaceOffset
    lvn_simplify_options opt;
    int64_t s_v, s_t, s_e, s_r;    // scratch offsets: vertices, triangles, edges, draws
};

struct Scratch {
    MV* verts;            // working vertices
    int3* tris;           // triangles (compacted in place)
    uint64_t* edges;      // edges, min | max << 32 (compacted in place)
    uint8_t* eflag;       // candidate edge kept (setup)
    float4* cpos;         // collapse position per draw
    float4* cnrm;         // collapse normal per draw
    int32_t* degree;      // triangles per vertex
    uint64_t* claim;      // (orderable error << 32 | edge) per vertex
    int32_t* target;      // collapse target per vertex
    int32_t* flag;        // boundary / used marks per vertex
    uint64_t* draws;      // drawn edge indices
    uint8_t* valid;       // drawn edge passed the tests
};

// ---- qef_simd.h in scalar lanes -------------------------------------------

__device__ __forceinline__ float dot4(const float a[4], const float b[4]) {
    float m[4];
    for (int i = 0; i < 4; i++) m[i] = a[i] * b[i];
    return (m[0] + m[1]) + (m[3] + m[2]);
}

__device__ __forceinline__ void mul_m4(const float a[4], const float B[4][4], float r[4]) {
    for (int j = 0; j < 4; j++) {
        float t = a[0] * B[0][j];
        t = t + a[1] * B[1][j];
        t = t + a[2] * B[2][j];
        t = t + a[3] * B[3][j];
        r[j] = t;
    }
}

__device__ __noinline__ float qef2(const MV& v0, const MV& v1, float out[4]) {
    float ATA[4][4], ATb[4], acc[4];
    for (int r = 0; r < 4; r++) {
        ATb[r] = 0.f;
        acc[r] = 0.f;
        for (int j = 0; j < 4; j++) ATA[r][j] = 0.f;
    }
    const MV* vs[2] = {&v0, &v1};
    for (int q = 0; q < 2; q++) {
        const float* n = vs[q]->n;
        for (int r = 0; r < 3; r++)
            for (int j = 0; j < 4; j++) ATA[r][j] = ATA[r][j] + n[r] * n[j];
        const float d = dot4(vs[q]->p, n);
        for (int j = 0; j < 3; j++) ATb[j] = ATb[j] + d * n[j];
        ATb[3] = ATb[3] + 0.f * n[3];
        for (int j = 0; j < 4; j++) acc[j] = acc[j] + vs[q]->p[j];
    }
    float mass[4];
    for (int j = 0; j < 4; j++) mass[j] = acc[j] / acc[3];
    float p[4];
    mul_m4(mass, ATA, p);
    for (int j = 0; j < 4; j++) p[j] = ATb[j] - p[j];
    float V[4][4] = {{1.f, 0.f, 0.f, 0.f}, {0.f, 1.f, 0.f, 0.f}, {0.f, 0.f, 1.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    float vt[4][4];
    for (int r = 0; r < 4; r++)
        for (int j = 0; j < 4; j++) vt[r][j] = ATA[r][j];
    for (int sweep = 0; sweep < 5; sweep++) {  // SVD_NUM_SWEEPS
        // givens_coeffs_sym
        const float pp[3] = {vt[0][0], vt[0][0], vt[1][1]};
        const float pq[3] = {vt[0][1], vt[0][2], vt[1][2]};
        const float qq[3] = {vt[1][1], vt[2][2], vt[2][2]};
        float c[3], s[3];
        for (int k = 0; k < 3; k++) {
            const float tau = (qq[k] - pp[k]) / (pq[k] * 2.f);
            const float stt = sqrtf(tau * tau + 1.f);
            const float tan = 1.f / (tau >= 0.f ? tau + stt : tau - stt);
            const float ck = 1.f / sqrtf(1.f + tan * tan);
            const float sk = tan * ck;
            c[k] = pq[k] == 0.f ? 1.f : ck;
            s[k] = pq[k] == 0.f ? 0.f : sk;
        }
        // rotateq_xy, as the reference writes it
        {
            const float u[3] = {vt[0][0], vt[0][0], vt[1][1]};
            const float v[3] = {vt[1][1], vt[2][2], vt[2][2]};
            const float a[3] = {vt[0][1], vt[0][2], vt[1][2]};
            float x[3], y[3];
            for (int k = 0; k < 3; k++) {
                const float cc = c[k] * c[k], ss = s[k] * s[k];
                const float mx = ((2.f * c[k]) * s[k]) * a[k];
                const float x0 = cc * u[k];
                x[k] = (x0 - mx) + ss * v[k];
                y[k] = (x0 + mx) + (cc + v[k]);
            }
            vt[0][0] = x[0];
            vt[0][0] = x[1];
            vt[1][1] = x[2];
            vt[0][1] = y[0];
            vt[0][2] = y[1];
            vt[1][2] = y[2];
        }
        // svd_rotate for (0,1), (0,2), (1,2)
        const int ra[3] = {0, 0, 1}, rb[3] = {1, 2, 2};
        for (int k = 0; k < 3; k++) {
            const int a = ra[k], b = rb[k];
            if (vt[a][b] == 0.f) continue;
            const float u[4] = {V[0][a], V[1][a], V[2][a], vt[0][3 - b]};
            const float v[4] = {V[0][b], V[1][b], V[2][b], vt[1 - a][2]};
            float x[4], y[4];
            for (int q = 0; q < 4; q++) {
                x[q] = c[k] * u[q] - s[k] * v[q];
                y[q] = s[k] * u[q] + c[k] * v[q];
            }
            for (int i = 0; i < 3; i++) V[i][a] = x[i];
            vt[0][3 - b] = x[3];
            for (int i = 0; i < 3; i++) V[i][b] = y[i];
            vt[1 - a][2] = y[3];
            vt[a][b] = 0.f;
        }
    }
    const float sigma[4] = {vt[0][0], vt[1][1], vt[2][2], 0.f};
    float inv[4];
    for (int j = 0; j < 4; j++) {  // svd_invdet
        const float ox = 1.f / sigma[j];
        const float ax = fabsf(sigma[j]), aox = fabsf(ox);
        const float mn = ax < aox ? ax : aox;
        inv[j] = mn >= 0.1f ? ox : 0.f;
    }
    float O[4][4];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 4; j++) O[i][j] = V[i][j] * inv[j];
    for (int j = 0; j < 4; j++) O[3][j] = 0.f;
    for (int i = 0; i < 4; i++) {
        float row[4];
        mul_m4(O[i], V, row);
        for (int j = 0; j < 4; j++) O[i][j] = row[j];
    }
    float x[4];
    mul_m4(p, O, x);
    float t[4];
    mul_m4(x, ATA, t);
    for (int j = 0; j < 4; j++) t[j] = ATb[j] - t[j];
    const float error = dot4(t, t);
    for (int j = 0; j < 4; j++) out[j] = x[j] + mass[j];
    return error;
}

// ---- block helpers ----------------------------------------------------------

// Ascending in-place sort of n u64 entries (mirrored-step bitonic network: any
// n, entries past n never move).
__device__ void block_sort(uint64_t* key, int n) {
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
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Exclusive scan of the per-warp counts in s_warp (warp 0, by shuffles); the
// total to *s_total.  Call between barriers.
__device__ __forceinline__ void scan_warp_counts(int* s_warp, int* s_total) {
    const int lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    if (threadIdx.x < 32) {
        const int c = lane < nwarps ? s_warp[lane] : 0;
        int inc = c;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane < nwarps) s_warp[lane] = inc - c;
        if (lane == 31) *s_total = inc;
    }
}

// Order-preserving compaction of [0, n): keep(i) -> emit(i, rank); returns the count.
template <class Keep, class Emit>
__device__ int block_compact(int n, Keep keep, Emit emit, int* s_warp, int* s_total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int base = 0;
    for (int start = 0; start < n; start += blockDim.x) {
        const int i = start + threadIdx.x;
        const bool k = i < n && keep(i);
        const unsigned ballot = __ballot_sync(0xffffffffu, k);
        if (lane == 0) s_warp[warp] = __popc(ballot);
        __syncthreads();
        scan_warp_counts(s_warp, s_total);
        __syncthreads();
        if (k) emit(i, base + s_warp[warp] + __popc(ballot & ((1u << lane) - 1)));
        base += *s_total;
        __syncthreads();
    }
    return base;
}

__device__ __forceinline__ uint32_t orderable(float e) {
    const uint32_t b = __float_as_uint(e);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Order-preserving compaction with four consecutive items per thread and the
// kept value computed once: test(i, &v) -> keep, emit(rank, v).  Returns the count.
template <class T, class Test, class Emit>
__device__ int block_compact4(int n, Test test, Emit emit, int* s_warp, int* s_total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int base = 0;
    for (int start = 0; start < n; start += 4 * blockDim.x) {
        const int i0 = start + 4 * threadIdx.x;
        T v[4];
        bool k[4];
        int c = 0;
        for (int q = 0; q < 4; q++) {
            k[q] = i0 + q < n && test(i0 + q, &v[q]);
            c += k[q];
        }
        int inc = c;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        scan_warp_counts(s_warp, s_total);
        __syncthreads();
        int r = base + s_warp[warp] + inc - c;
        for (int q = 0; q < 4; q++)
            if (k[q]) emit(r++, v[q]);
        base += *s_total;
        __syncthreads();
    }
    return base;
}

// ---- the simplifier ---------------------------------------------------------

template <int Threads>
__global__ void __launch_bounds__(Threads, 1024 / Threads)
    k_mesh_collapse(const MeshJob* __restrict__ jobs, const int32_t* __restrict__ order, const lvn_mesh_vertex* in_v,
                    const lvn_mesh_triangle* in_t, lvn_mesh_vertex* out_v, lvn_mesh_triangle* out_t, int32_t* counts,
                    Scratch S, const uint32_t* __restrict__ raw, int raw_len) {
    extern __shared__ uint64_t smem[];
    __shared__ int s_warp[32], s_total, s_count, s_flag;
    const int jid = order[blockIdx.x];
    const MeshJob J = jobs[jid];
    const int tid = threadIdx.x, nth = blockDim.x;
    const lvn_simplify_options& o = J.opt;
    if (J.nt < 100 || J.nv < 100) {  // left as generated (ng_mesh_simplify.cpp:445-448)
        for (int i = tid; i < J.nv; i += nth) out_v[J.v_off + i] = in_v[J.v_off + i];
        for (int i = tid; i < J.nt; i += nth) out_t[J.t_off + i] = in_t[J.t_off + i];
        if (tid == 0) {
            counts[2 * jid] = J.nv;
            counts[2 * jid + 1] = J.nt;
        }
        return;
    }
    MV* vs = S.verts + J.s_v;
    int3* T = S.tris + J.s_t;
    uint64_t* E = S.edges + J.s_e;
    uint8_t* eflag = S.eflag + J.s_e;
    float4* cpos = S.cpos + J.s_r;
    float4* cnrm = S.cnrm + J.s_r;
    int32_t* degree = S.degree + J.s_v;
    uint64_t* claim = S.claim + J.s_v;
    int32_t* target = S.target + J.s_v;
    int32_t* flag = S.flag + J.s_v;
    uint64_t* draws = S.draws + J.s_r;
    uint8_t* valid = S.valid + J.s_r;
    const int nv = J.nv;
    for (int i = tid; i < nv; i += nth) {
        MV v;
        const lvn_mesh_vertex src = in_v[J.v_off + i];
        for (int j = 0; j < 4; j++) {
            v.p[j] = src.position[j] - J.offset[j];
            v.n[j] = src.normal[j];
            v.c[j] = src.colour[j];
        }
        vs[i] = v;
        degree[i] = 0;
        flag[i] = 0;
    }
    __syncthreads();
    // BuildCandidateEdges (ng_mesh_simplify.cpp:122-177).  The edges are sorted
    // by the union's idx_ = min | max << 32: a counting sort on max (bucket
    // sizes from target[], then a scan), then each bucket's few entries by min.
    const int ne0 = 3 * J.nt;
    uint64_t* ekeys = E;
    for (int i = tid; i < nv; i += nth) target[i] = 0;
    __syncthreads();
    for (int t = tid; t < J.nt; t += nth) {
        const lvn_mesh_triangle tr = in_t[J.t_off + t];
        const int a = tr.indices[0], b = tr.indices[1], c = tr.indices[2];
        T[t] = make_int3(a, b, c);
        atomicAdd(&degree[a], 1);
        atomicAdd(&degree[b], 1);
        atomicAdd(&degree[c], 1);
        atomicAdd(&target[max(a, b)], 1);
        atomicAdd(&target[max(b, c)], 1);
        atomicAdd(&target[max(a, c)], 1);
    }
    __syncthreads();
    {  // exclusive scan of the bucket sizes: bucket starts to claim[], cursors to target[]
        int base = 0;
        for (int start = 0; start < nv; start += nth) {
            const int i = start + tid;
            const int c = i < nv ? target[i] : 0;
            int inc = c;
            const int lane = tid & 31, warp = tid >> 5;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += t;
            }
            if (lane == 31) s_warp[warp] = inc;
            __syncthreads();
            scan_warp_counts(s_warp, &s_total);
            __syncthreads();
            if (i < nv) {
                claim[i] = (uint64_t)(base + s_warp[warp] + inc - c);  // bucket start
                target[i] = base + s_warp[warp] + inc - c;              // cursor
            }
            base += s_total;
            __syncthreads();
        }
    }
    for (int t = tid; t < J.nt; t += nth) {
        const int3 x = T[t];
        const int pa[3][2] = {{x.x, x.y}, {x.y, x.z}, {x.x, x.z}};
        for (int k = 0; k < 3; k++) {
            const uint32_t lo = (uint32_t)min(pa[k][0], pa[k][1]), hi = (uint32_t)max(pa[k][0], pa[k][1]);
            ekeys[atomicAdd(&target[hi], 1)] = (uint64_t)lo | ((uint64_t)hi << 32);
        }
    }
    __syncthreads();
    for (int v = tid; v < nv; v += nth) {  // insertion sort of bucket v by min
        const int b0 = (int)claim[v], b1 = target[v];
        for (int i = b0 + 1; i < b1; i++) {
            const uint64_t k = ekeys[i];
            int j = i - 1;
            while (j >= b0 && ekeys[j] > k) {
                ekeys[j + 1] = ekeys[j];
                j--;
            }
            ekeys[j + 1] = k;
        }
    }
    __syncthreads();
    const uint64_t last = ekeys[ne0 - 1];  // the final run is never examined (ng_mesh_simplify.cpp:143-164)
    for (int i = tid; i < ne0; i += nth) {
        const uint64_t k = ekeys[i];
        if (k == last || (i > 0 && ekeys[i - 1] == k)) continue;
        if (ekeys[i + 1] != k) {  // a single-use edge: its end points are on the boundary
            flag[(uint32_t)k] = 1;
            flag[(uint32_t)(k >> 32)] = 1;
        }
    }
    __syncthreads();
    for (int i = tid; i < ne0; i += nth) {  // an interior run's first entry, away from the boundary
        const uint64_t k = ekeys[i];
        eflag[i] = k != last && (i == 0 || ekeys[i - 1] != k) && ekeys[i + 1] == k && !flag[(uint32_t)k] &&
                   !flag[(uint32_t)(k >> 32)];
    }
    __syncthreads();
    int ne = block_compact4<uint64_t>(
        ne0,
        [&](int i, uint64_t* out) {
            *out = ekeys[i];
            return eflag[i] != 0;
        },
        [&](int r, uint64_t e) { E[r] = e; }, s_warp, &s_total);
    int nt = J.nt;
    const int target_tris = (int)((float)J.nt * o.target_percentage);
    int iterations = 0;
    while (nt > target_tris && iterations++ < o.max_iterations) {
        for (int i = tid; i < nv; i += nth) {
            claim[i] = ~0ull;
            target[i] = -1;
        }
        // the draws: uniform_int_distribution<int>(0, ne - 1) over mt19937(42)
        const int num_random = (int)((float)ne * o.edge_fraction);
        const uint32_t range = (uint32_t)ne;
        const uint32_t threshold = range ? (uint32_t)(0u - range) % range : 0u;
        if (tid == 0) s_flag = 0;
        __syncthreads();
        int got = 0;
        for (int start = 0; got < num_random; start += nth) {
            if (start >= raw_len) {
                if (tid == 0) s_flag = 1;  // the host sizes the table; never expected
                break;
            }
            const int k = start + tid;
            uint64_t prod = 0;
            bool acc = false;
            if (k < raw_len) {
                prod = (uint64_t)raw[k] * range;
                acc = (uint32_t)prod >= threshold;
            }
            const int lane = tid & 31, warp = tid >> 5;
            const unsigned ballot = __ballot_sync(0xffffffffu, acc);
            if (lane == 0) s_warp[warp] = __popc(ballot);
            __syncthreads();
            scan_warp_counts(s_warp, &s_total);
            __syncthreads();
            const int r = got + s_warp[warp] + __popc(ballot & ((1u << lane) - 1));
            if (acc && r < num_random) draws[r] = prod >> 32;
            got += s_total;
            __syncthreads();
        }
        uint64_t* dk = num_random <= kSortCap ? smem : draws;
        if (dk == smem)
            for (int i = tid; i < num_random; i += nth) smem[i] = draws[i];
        __syncthreads();
        block_sort(dk, num_random);
        // FindValidCollapses (ng_mesh_simplify.cpp:181-278)
        if (tid == 0) s_count = 0;
        __syncthreads();
        int my_valid = 0;
        for (int j = tid; j < num_random; j += nth) {
            const int i = (int)dk[j];
            valid[j] = 0;
            const uint64_t e = E[i];
            const uint32_t emn = (uint32_t)e, emx = (uint32_t)(e >> 32);
            const MV a = vs[emn], b = vs[emx];
            if (dot4(a.n, b.n) < o.min_angle_cosine) continue;
            float d[4];
            for (int q = 0; q < 4; q++) d[q] = b.p[q] - a.p[q];
            if (dot4(d, d) > o.max_edge_size * o.max_edge_size) continue;
            if ((double)fabsf(a.c[3] - b.c[3]) > 1e-3) continue;
            const int deg = degree[emn] + degree[emx];
            if (deg > kMaxDegree) continue;
            float pos[4];
            float error = qef2(a, b, pos);
            if (error > 0.f) error = 1.f / error;
            error += (float)max(0, deg - 10) * (o.max_error * 0.1f);
            if (error > o.max_error) continue;
            valid[j] = 1;
            my_valid++;
            cnrm[j] = make_float4((a.n[0] - b.n[0]) * 0.5f, (a.n[1] - b.n[1]) * 0.5f, (a.n[2] - b.n[2]) * 0.5f,
                                  (a.n[3] - b.n[3]) * 0.5f);
            cpos[j] = make_float4(pos[0], pos[1], pos[2], 1.f);
            if (error < FLT_MAX) {
                const uint64_t key = ((uint64_t)orderable(error) << 32) | (uint32_t)i;
                atomicMin((unsigned long long*)&claim[emn], (unsigned long long)key);
                atomicMin((unsigned long long*)&claim[emx], (unsigned long long)key);
            }
        }
        for (int off = 16; off > 0; off >>= 1) my_valid += __shfl_xor_sync(0xffffffffu, my_valid, off);
        if ((tid & 31) == 0 && my_valid) atomicAdd(&s_count, my_valid);
        __syncthreads();
        if (s_count == 0) break;
        // CollapseEdges (ng_mesh_simplify.cpp:282-306)
        for (int j = tid; j < num_random; j += nth) {
            if (!valid[j]) continue;
            const int i = (int)dk[j];
            const uint64_t e = E[i];
            const uint32_t emn = (uint32_t)e, emx = (uint32_t)(e >> 32);
            if ((uint32_t)claim[emn] == (uint32_t)i && (uint32_t)claim[emx] == (uint32_t)i &&
                claim[emn] != ~0ull && claim[emx] != ~0ull) {
                target[emx] = (int)emn;
                const float4 cp = cpos[j], cn = cnrm[j];
                vs[emn].p[0] = cp.x;
                vs[emn].p[1] = cp.y;
                vs[emn].p[2] = cp.z;
                vs[emn].p[3] = cp.w;
                vs[emn].n[0] = cn.x;
                vs[emn].n[1] = cn.y;
                vs[emn].n[2] = cn.z;
                vs[emn].n[3] = cn.w;
            }
        }
        for (int i = tid; i < nv; i += nth) degree[i] = 0;
        __syncthreads();
        // RemoveTriangles (ng_mesh_simplify.cpp:310-352)
        nt = block_compact4<int3>(
            nt,
            [&](int t, int3* out) {
                int3 x = T[t];
                int m = target[x.x];
                if (m != -1) x.x = m;
                m = target[x.y];
                if (m != -1) x.y = m;
                m = target[x.z];
                if (m != -1) x.z = m;
                *out = x;
                return !(x.x == x.y || x.x == x.z || x.y == x.z);
            },
            [&](int r, const int3& x) {
                T[r] = x;  // in place: r <= t, and a chunk's reads precede its writes
                atomicAdd(&degree[x.x], 1);
                atomicAdd(&degree[x.y], 1);
                atomicAdd(&degree[x.z], 1);
            },
            s_warp, &s_total);
        // RemoveEdges (ng_mesh_simplify.cpp:356-380)
        auto remap = [&](uint64_t e) {
            uint32_t emn = (uint32_t)e, emx = (uint32_t)(e >> 32);
            if (target[emn] != -1) emn = (uint32_t)target[emn];
            if (target[emx] != -1) emx = (uint32_t)target[emx];
            return (uint64_t)emn | ((uint64_t)emx << 32);
        };
        ne = block_compact4<uint64_t>(
            ne,
            [&](int i, uint64_t* out) {
                const uint64_t e = remap(E[i]);
                *out = e;
                return (uint32_t)e != (uint32_t)(e >> 32);
            },
            [&](int r, uint64_t e) { E[r] = e; }, s_warp, &s_total);
        __syncthreads();
    }
    // CompactVertices (ng_mesh_simplify.cpp:384-421) and the offset added back
    for (int i = tid; i < nv; i += nth) flag[i] = 0;
    __syncthreads();
    for (int t = tid; t < nt; t += nth) {
        const int3 x = T[t];
        flag[x.x] = 1;
        flag[x.y] = 1;
        flag[x.z] = 1;
    }
    __syncthreads();
    const int nv_out = block_compact(
        nv, [&](int i) { return flag[i] != 0; },
        [&](int i, int r) {
            target[i] = r;
            const MV v = vs[i];
            lvn_mesh_vertex w;
            for (int j = 0; j < 4; j++) {
                w.position[j] = v.p[j] + J.offset[j];
                w.normal[j] = v.n[j];
                w.colour[j] = v.c[j];
            }
            out_v[J.v_off + r] = w;
        },
        s_warp, &s_total);
    __syncthreads();
    for (int t = tid; t < nt; t += nth) {
        const int3 x = T[t];
        lvn_mesh_triangle w;
        w.indices[0] = target[x.x];
        w.indices[1] = target[x.y];
        w.indices[2] = target[x.z];
        out_t[J.t_off + t] = w;
    }
    if (tid == 0) {
        counts[2 * jid] = s_flag ? -1 : nv_out;
        counts[2 * jid + 1] = nt;
    }
}

// ---- host side -----------------------------------------------------------------

template <class T>
struct Grow {
    T* p = nullptr;
    size_t cap = 0;
    cudaError_t fit(size_t need) {
        if (need <= cap) return cudaSuccess;
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return e;
        need = std::max(need, 2 * cap);
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        e = cudaMalloc(&p, sizeof(T) * need);
        if (e == cudaSuccess) cap = need;
        return e;
    }
};

struct CollapseWork {
    std::mutex mu;
    int device = -1;
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    Grow<MeshJob> jobs;
    Grow<int32_t> order;
    Grow<MV> verts;
    Grow<int3> tris;
    Grow<uint64_t> edges, claim, draws;
    Grow<uint8_t> eflag;
    Grow<float4> cpos, cnrm;
    Grow<int32_t> degree, target, flag, counts;
    Grow<uint8_t> valid;
    Grow<uint32_t> raw;
    Grow<lvn_mesh_vertex> vin, vout;
    Grow<lvn_mesh_triangle> tin, tout;
    size_t raw_len = 0;
    std::vector<int32_t> hcounts;
};
CollapseWork& collapse_work() {
    static CollapseWork w;
    return w;
}

int cuda_rc(cudaError_t e) {
    if (e == cudaSuccess) return LVN_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? LVN_ERR_OUT_OF_MEMORY : LVN_ERR_CUDA;
}

#define CL_TRY(x)                        \
    do {                                 \
        const int rc__ = cuda_rc(x);     \
        if (rc__ != LVN_OK) return rc__; \
    } while (0)

}  // namespace
}  // namespace lvn

using namespace lvn;

extern "C" {

void lvn_simplify_options_default(lvn_simplify_options* o) {
    if (!o) return;
    o->edge_fraction = 0.125f;  // MeshSimplificationOptions (ng_mesh_simplify.h:8-31)
    o->max_iterations = 10;
    o->target_percentage = 0.05f;
    o->max_error = 5.f;
    o->max_edge_size = 2.5f;
    o->min_angle_cosine = 0.8f;
}

int lvn_mesh_simplify(const lvn_mesh_vertex* vertices, const lvn_mesh_triangle* triangles, int32_t memory,
                      lvn_chunk_result* meshes, int32_t num_meshes, const float* offsets,
                      const lvn_simplify_options* options, lvn_mesh_vertex* out_vertices,
                      lvn_mesh_triangle* out_triangles) {
    if (num_meshes < 0 || (num_meshes > 0 && (!meshes || !offsets || !options || !vertices || !triangles ||
                                              !out_vertices || !out_triangles)) ||
        (memory != LVN_MEMORY_HOST && memory != LVN_MEMORY_DEVICE))
        return LVN_ERR_INVALID;
    if (num_meshes == 0) return LVN_OK;
    std::vector<MeshJob> jobs(num_meshes);
    int64_t sv = 0, st = 0, se = 0, sr = 0, vmax = 0, tmax = 0;
    int max_draws = 0;
    for (int m = 0; m < num_meshes; m++) {
        const lvn_chunk_result& r = meshes[m];
        const lvn_simplify_options& o = options[m];
        if (r.num_vertices < 0 || r.num_triangles < 0 || r.vertex_offset < 0 || r.triangle_offset < 0 ||
            o.edge_fraction < 0.f || o.edge_fraction > 1.f || o.max_iterations < 0)
            return LVN_ERR_INVALID;
        MeshJob& J = jobs[m];
        J.v_off = r.vertex_offset;
        J.nv = r.num_vertices;
        J.t_off = r.triangle_offset;
        J.nt = r.num_triangles;
        for (int j = 0; j < 4; j++) J.offset[j] = offsets[4 * m + j];
        J.opt = o;
        J.s_v = sv;
        J.s_t = st;
        J.s_e = se;
        J.s_r = sr;
        sv += J.nv;
        st += J.nt;
        se += 3 * (int64_t)J.nt;
        const int draws = (int)((float)(3 * J.nt) * o.edge_fraction) + 1;
        sr += draws;
        max_draws = std::max(max_draws, draws);
        vmax = std::max<int64_t>(vmax, (int64_t)J.v_off + J.nv);
        tmax = std::max<int64_t>(tmax, (int64_t)J.t_off + J.nt);
    }
    CollapseWork& w = collapse_work();
    std::lock_guard<std::mutex> lock(w.mu);
    int dev = 0;
    CL_TRY(cudaGetDevice(&dev));
    if (w.device != dev) {
        if (w.device >= 0) return LVN_ERR_INVALID;  // the scratch lives on the first device used
        CL_TRY(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
        CL_TRY(cudaStreamCreateWithFlags(&w.side, cudaStreamNonBlocking));
        CL_TRY(cudaEventCreateWithFlags(&w.fork, cudaEventDisableTiming));
        CL_TRY(cudaEventCreateWithFlags(&w.join, cudaEventDisableTiming));
        CL_TRY(cudaFuncSetAttribute(k_mesh_collapse<kThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmem));
        CL_TRY(cudaFuncSetAttribute(k_mesh_collapse<kBigThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmem));
        w.device = dev;
    }
    cudaStream_t s = w.stream;
    // the raw mt19937(42) stream, long enough for the largest draw count
    // with room for the rare rejections
    const size_t need_raw = (size_t)max_draws + 4096;
    if (w.raw_len < need_raw) {
        std::vector<uint32_t> raw(need_raw);
        std::mt19937 gen;
        gen.seed(42);
        for (size_t i = 0; i < need_raw; i++) raw[i] = (uint32_t)gen();
        CL_TRY(w.raw.fit(need_raw));
        CL_TRY(cudaMemcpy(w.raw.p, raw.data(), sizeof(uint32_t) * need_raw, cudaMemcpyHostToDevice));
        w.raw_len = need_raw;
    }
    CL_TRY(w.jobs.fit(num_meshes));
    CL_TRY(w.verts.fit(std::max<int64_t>(sv, 1)));
    CL_TRY(w.degree.fit(std::max<int64_t>(sv, 1)));
    CL_TRY(w.claim.fit(std::max<int64_t>(sv, 1)));
    CL_TRY(w.target.fit(std::max<int64_t>(sv, 1)));
    CL_TRY(w.flag.fit(std::max<int64_t>(sv, 1)));
    CL_TRY(w.tris.fit(std::max<int64_t>(st, 1)));
    CL_TRY(w.edges.fit(std::max<int64_t>(se, 1)));
    CL_TRY(w.eflag.fit(std::max<int64_t>(se, 1)));
    CL_TRY(w.cpos.fit(std::max<int64_t>(sr, 1)));
    CL_TRY(w.cnrm.fit(std::max<int64_t>(sr, 1)));
    CL_TRY(w.draws.fit(std::max<int64_t>(sr, 1)));
    CL_TRY(w.valid.fit(std::max<int64_t>(sr, 1)));
    CL_TRY(w.counts.fit(2 * (size_t)num_meshes));
    CL_TRY(cudaMemcpyAsync(w.jobs.p, jobs.data(), sizeof(MeshJob) * num_meshes, cudaMemcpyHostToDevice, s));
    const lvn_mesh_vertex* dv = vertices;
    const lvn_mesh_triangle* dt = triangles;
    lvn_mesh_vertex* ov = out_vertices;
    lvn_mesh_triangle* ot = out_triangles;
    if (memory == LVN_MEMORY_HOST) {
        CL_TRY(w.vin.fit(std::max<int64_t>(vmax, 1)));
        CL_TRY(w.tin.fit(std::max<int64_t>(tmax, 1)));
        CL_TRY(w.vout.fit(std::max<int64_t>(vmax, 1)));
        CL_TRY(w.tout.fit(std::max<int64_t>(tmax, 1)));
        CL_TRY(cudaMemcpyAsync(w.vin.p, vertices, sizeof(lvn_mesh_vertex) * vmax, cudaMemcpyHostToDevice, s));
        CL_TRY(cudaMemcpyAsync(w.tin.p, triangles, sizeof(lvn_mesh_triangle) * tmax, cudaMemcpyHostToDevice, s));
        dv = w.vin.p;
        dt = w.tin.p;
        ov = w.vout.p;
        ot = w.tout.p;
    }
    Scratch S;
    S.verts = w.verts.p;
    S.tris = w.tris.p;
    S.edges = w.edges.p;
    S.eflag = w.eflag.p;
    S.cpos = w.cpos.p;
    S.cnrm = w.cnrm.p;
    S.degree = w.degree.p;
    S.claim = w.claim.p;
    S.target = w.target.p;
    S.flag = w.flag.p;
    S.draws = w.draws.p;
    S.valid = w.valid.p;
    // large meshes with twice the threads on a second stream, beside the rest
    std::vector<int32_t> order;
    for (int m = 0; m < num_meshes; m++)
        if (jobs[m].nt > kBigTriangles) order.push_back(m);
    const int n_big = (int)order.size();
    for (int m = 0; m < num_meshes; m++)
        if (jobs[m].nt <= kBigTriangles) order.push_back(m);
    CL_TRY(w.order.fit(num_meshes));
    CL_TRY(cudaMemcpyAsync(w.order.p, order.data(), sizeof(int32_t) * num_meshes, cudaMemcpyHostToDevice, s));
    if (n_big) {
        CL_TRY(cudaEventRecord(w.fork, s));
        CL_TRY(cudaStreamWaitEvent(w.side, w.fork, 0));
        k_mesh_collapse<kBigThreads><<<n_big, kBigThreads, kSmem, w.side>>>(
            w.jobs.p, w.order.p, dv, dt, ov, ot, w.counts.p, S, w.raw.p, (int)w.raw_len);
        CL_TRY(cudaGetLastError());
        CL_TRY(cudaEventRecord(w.join, w.side));
    }
    if (num_meshes > n_big)
        k_mesh_collapse<kThreads><<<num_meshes - n_big, kThreads, kSmem, s>>>(
            w.jobs.p, w.order.p + n_big, dv, dt, ov, ot, w.counts.p, S, w.raw.p, (int)w.raw_len);
    if (n_big) CL_TRY(cudaStreamWaitEvent(s, w.join, 0));
    CL_TRY(cudaGetLastError());
    w.hcounts.resize(2 * (size_t)num_meshes);
    CL_TRY(cudaMemcpyAsync(w.hcounts.data(), w.counts.p, sizeof(int32_t) * 2 * num_meshes, cudaMemcpyDeviceToHost, s));
    CL_TRY(cudaStreamSynchronize(s));
    for (int m = 0; m < num_meshes; m++) {
        if (w.hcounts[2 * m] < 0) return LVN_ERR_DEVICE_STATUS;
        meshes[m].num_vertices = w.hcounts[2 * m];
        meshes[m].num_triangles = w.hcounts[2 * m + 1];
    }
    if (memory == LVN_MEMORY_HOST) {
        // the meshes' input ranges, merged where they touch: one copy per run
        auto copy_runs = [&](bool verts) -> int {
            std::vector<std::pair<int64_t, int64_t>> r;
            for (const MeshJob& J : jobs)
                if (verts ? J.nv : J.nt) r.push_back(verts ? std::make_pair((int64_t)J.v_off, (int64_t)J.v_off + J.nv)
                                                           : std::make_pair((int64_t)J.t_off, (int64_t)J.t_off + J.nt));
            std::sort(r.begin(), r.end());
            for (size_t i = 0; i < r.size();) {
                int64_t a = r[i].first, b = r[i].second;
                for (i++; i < r.size() && r[i].first <= b; i++) b = std::max(b, r[i].second);
                const cudaError_t e =
                    verts ? cudaMemcpyAsync(out_vertices + a, ov + a, sizeof(lvn_mesh_vertex) * (b - a),
                                            cudaMemcpyDeviceToHost, s)
                          : cudaMemcpyAsync(out_triangles + a, ot + a, sizeof(lvn_mesh_triangle) * (b - a),
                                            cudaMemcpyDeviceToHost, s);
                if (e != cudaSuccess) return cuda_rc(e);
            }
            return LVN_OK;
        };
        int rc = copy_runs(true);
        if (rc == LVN_OK) rc = copy_runs(false);
        if (rc) return rc;
        CL_TRY(cudaStreamSynchronize(s));
    }
    return LVN_OK;
}

}  // extern "C"
