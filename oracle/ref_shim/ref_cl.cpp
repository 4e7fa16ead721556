// ref_cl.cpp -- the reference's own OpenCL C code for the chunk-meshing path
// (leven/cl/shared_constants.cl, simplex.cl, noise.cl with hg_sdf.glsl,
// qef.cl, cuckoo.cl, density_field.cl, octree.cl), compiled on the host
// through cl_shim.h, behind C entry points: single functions (noise, QEF) and
// a whole chunk run kernel by kernel (ref_mesh_chunk).
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref where
// the reference tree is present, and used only by tests to pin the oracle's
// restatement (oracle/lvn_oracle.cpp) against the reference source.
//
// The reference built its programs with -cl-fast-relaxed-math
// (compute.cpp:258), which lets a compiler fuse a multiply into an add, or
// not.  The restatement fixes one choice, and this harness compiles the
// reference's code under the same one: noise.cl with fusion (a multiply whose
// one use is an add becomes an fma: the octave sums, the terrain's remaps and
// its final y - 900 noise), every other file without fusion outside dot()
// and mix() (this file is compiled with -ffp-contract=off; a GCC optimize
// pragma switches noise.cl's functions to fusion).  -fsingle-precision-constant
// makes double literals (snoise3's 0.6, qef.cl's 2.0 and 1.0) single
// precision, as on a device without doubles.
#include "cl_shim.h"

#include <random>
#include <vector>

#include "primes.h"

thread_local int clshim_gid[3];

// the program's -D definitions for 64^3 chunks (compute.cpp:248-278)
#define VOXELS_PER_CHUNK 64
#define LEAF_SIZE_SCALE 4
#define FIELD_DIM 66
#define HERMITE_INDEX_SIZE 65
#define VOXEL_INDEX_SHIFT 7
#define VOXEL_INDEX_MASK 127
#define MAX_TERRAIN_HEIGHT 900
#define MATERIAL_AIR 201
#define MATERIAL_NONE 200
#define FIND_EDGE_INFO_STEPS 16
#define FIND_EDGE_INFO_INCREMENT 0.0625
#define MAX_OCTREE_DEPTH 6
#define CUCKOO_EMPTY_VALUE 18446744073709551615ull
#define CUCKOO_STASH_HASH_INDEX 4
#define CUCKOO_HASH_FN_COUNT 5
#define CUCKOO_STASH_SIZE 101
#define CUCKOO_MAX_ITERATIONS 32
#define constant static const

// ApplyCSGOperations through the reference's CSG kernels (ref_csg.cpp)
int ref_csg_apply(const int32_t off[3], int scale, const void* ops, int num_ops, int32_t* materials,
                  std::vector<int>& edge_keys, std::vector<float4>& edge_info);

namespace refmesh {
#include "cl/shared_constants.cl"
#include "cl/simplex.cl"
#include "cl/qef.cl"
#include "cl/cuckoo.cl"

#pragma GCC push_options
#pragma GCC optimize("fp-contract=fast")
#include "cl/noise.cl"

// The density the field kernels evaluate: the reference's DensityFunc (mode
// 0), or the benchmark's heightfield y - 48 BasicFractal(8, 1/256, 2, 0.5,
// xz) (mode 1), plus 12 times a 6-octave 3D fBm at 1/64 (mode 2).  The 3D fBm
// is not in the reference; it is BasicFractal's loop over the reference's
// snoise3.
int g_mode = 0;
clshim_image2d g_perm = {nullptr, 256, 256};
uint8_t g_texels[256 * 256 * 4];

float caves_fbm3(float3 p) {
    float noise = 0.f, amplitude = 1.f;
    p *= (1.f / 64.f);
    for (int i = 0; i < 6; i++) {
        noise += snoise3(p, &g_perm) * amplitude;
        p *= 2.f;
        amplitude *= 0.5f;
    }
    return noise;
}

float HarnessDensity(const float4 position, image2d_t permTexture) {
    if (g_mode == 0) return DensityFunc(position, permTexture);
    const float h = BasicFractal(permTexture, 8, 1.f / 256.f, 2.f, 0.5f, float2(position.x, position.z));
    const float base = position.y - 48.f * h;
    if (g_mode == 1) return base;
    return base + 12.f * caves_fbm3(float3(position.x, position.y, position.z));
}

#pragma GCC pop_options

#define DensityFunc HarnessDensity
#include "cl/density_field.cl"
#undef DensityFunc
#include "cl/octree.cl"
}  // namespace refmesh

namespace {
using namespace refmesh;

// Cuckoo_InitialiseTable + the host insert loop (compute_cuckoo.cpp:49-139):
// parameters from the generator until every key inserts.  The stash holds
// `prime` entries: the insert kernel indexes it with a hash taken modulo the
// table size (cuckoo.cl:66-68), past the reference's 101 entries.
struct HostCuckoo {
    uint prime = 0;
    std::vector<ulong> table, stash;
    uint params[CUCKOO_HASH_FN_COUNT * 2];
    int stash_used = 0;
    int stash_past_101 = 0;

    void build(const uint* keys, int n, std::mt19937& gen) {
        std::uniform_int_distribution<uint32_t> dist(1u << 15, 1u << 30);
        prime = (uint)FindNextPrime(std::max(2048, 2 * n));
        std::vector<int> inserted(n), used(n);
        for (;;) {
            for (int i = 0; i < CUCKOO_HASH_FN_COUNT * 2; i++) params[i] = dist(gen);
            table.assign(prime, CUCKOO_EMPTY_VALUE);
            stash.assign(std::max<uint>(prime, CUCKOO_STASH_SIZE), CUCKOO_EMPTY_VALUE);
            for (int i = 0; i < n; i++) {
                clshim_gid[0] = i;
                Cuckoo_InsertKeys(const_cast<uint*>(keys), table.data(), stash.data(), prime, params, inserted.data(),
                                  used.data());
            }
            bool ok = true;
            stash_used = 0;
            for (int i = 0; i < n; i++) {
                ok = ok && inserted[i];
                stash_used |= used[i];
            }
            if (ok) break;
        }
        for (size_t h = CUCKOO_STASH_SIZE; h < stash.size(); h++) stash_past_101 |= stash[h] != CUCKOO_EMPTY_VALUE;
    }
};

template <typename F>
void run_1d(int n, F f) {
    for (int i = 0; i < n; i++) {
        clshim_gid[0] = i;
        f();
    }
}
template <typename F>
void run_3d(int nx, int ny, int nz, F f) {
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                clshim_gid[0] = x;
                clshim_gid[1] = y;
                clshim_gid[2] = z;
                f();
            }
}

}  // namespace

extern "C" {

// the permutation lookup image: 256 x 256 RGBA8 texels, row-major
void ref_set_perm_image(const uint8_t* rgba) {
    std::memcpy(g_texels, rgba, sizeof(g_texels));
    g_perm.texels = g_texels;
}

float ref_snoise2(float x, float y) { return snoise2(float2(x, y), &g_perm); }
float ref_snoise3(float x, float y, float z) { return snoise3(float3(x, y, z), &g_perm); }

float ref_basic_fractal(int octaves, float frequency, float lacunarity, float persistence, float x, float y) {
    return BasicFractal(&g_perm, octaves, frequency, lacunarity, persistence, float2(x, y));
}

float ref_ridged_multi_fractal(int octaves, float lacunarity, float gain, float offset, float x, float y) {
    return RidgedMultiFractal(&g_perm, octaves, lacunarity, gain, offset, float2(x, y));
}

float ref_terrain(float x, float z) { return Terrain(float4(x, 0.f, z, 0.f), &g_perm); }

float ref_density_func(float x, float y, float z) { return DensityFunc(float4(x, y, z, 0.f), &g_perm); }

// the field kernels' density (see HarnessDensity) for mode 0, 1 or 2
float ref_harness_density(int mode, float x, float y, float z) {
    g_mode = mode;
    return HarnessDensity(float4(x, y, z, 0.f), &g_perm);
}

// qef_create_from_points (qef.cl:283-303) over `count` points and normals
// (x, y, z, w each), then qef_solve (qef.cl:239-256).  out: the solved
// position (x, y, z, w); returns qef_solve's error.
float ref_qef_solve_points(const float* positions, const float* normals, int count, float* out) {
    float4 p[12], n[12];
    for (int i = 0; i < count && i < 12; i++) {
        p[i] = float4(positions[4 * i], positions[4 * i + 1], positions[4 * i + 2], positions[4 * i + 3]);
        n[i] = float4(normals[4 * i], normals[4 * i + 1], normals[4 * i + 2], normals[4 * i + 3]);
    }
    QEFData q;
    qef_create_from_points(p, n, (size_t)(count < 12 ? count : 12), &q);
    float4 x = {0.f, 0.f, 0.f, 0.f};
    const float err = qef_solve(&q, &x);
    out[0] = x.x;
    out[1] = x.y;
    out[2] = x.z;
    out[3] = x.w;
    return err;
}

// One 64^3 chunk through the reference's kernels in the order
// generateChunkMesh runs them (compute_density_field.cpp:138-274,
// compute_octree.cpp:108-347): GenerateDefaultField, FindFieldEdges,
// compaction, FindEdgeIntersectionInfo, the stored CSG operations
// (`num_ops` CSGOperation records, 48 bytes each, through ref_csg.cpp's
// ApplyCSGOperations), FindActiveVoxels, compaction, the edge
// table, CreateLeafNodes, SolveQEFs, the node table, GenerateMesh, compaction,
// GenerateMeshVertexBuffer, FindSeamNodes, ExtractSeamNodeInfo.  Scans and
// compactions are sequential here (stable, in index order).  Hash parameters
// come from std::mt19937(hash_seed), edges first.  colour is the chunk's LOD
// colour (ColourForMinLeafSize).
// Outputs: materials[66^3]; edge keys and info; vertices (12 floats each);
// triangle indices; seam records (12 words each).  counts[0..5] = edges,
// leaves, triangle indices, seams, stash used (edge | node << 1), stash
// entries past the reference's 101.  Returns 0, -1 when an output array is
// too small (counts are set), -2 when CSG pruned every field edge (there the
// reference keeps the unpruned list, compute_csg.cpp:156).
int ref_mesh_chunk(const int32_t min[3], int32_t size, int32_t mode, uint32_t hash_seed, const float colour[3],
                   const void* ops, int32_t num_ops, int32_t* materials, int32_t* edge_keys, float* edge_info,
                   int64_t edge_cap, float* vertices, int32_t* triangles, int32_t* seams, int64_t node_cap,
                   int32_t counts[6]) {
    g_mode = mode;
    const int vpc = VOXELS_PER_CHUNK, fd = FIELD_DIM, hd = HERMITE_INDEX_SIZE;
    const int scale = size / (vpc * LEAF_SIZE_SCALE);
    const int4 offset(min[0] / LEAF_SIZE_SCALE, min[1] / LEAF_SIZE_SCALE, min[2] / LEAF_SIZE_SCALE, 0);
    for (int i = 0; i < 6; i++) counts[i] = 0;

    run_3d(fd, fd, fd, [&] { GenerateDefaultField(&g_perm, offset, scale, 0, materials); });
    std::vector<int> occ(3 * hd * hd * hd), idx(3 * hd * hd * hd);
    run_3d(hd, hd, hd, [&] { FindFieldEdges(offset, materials, occ.data(), idx.data()); });
    std::vector<int> edges;
    for (size_t i = 0; i < occ.size(); i++)
        if (occ[i]) edges.push_back(idx[i]);
    std::vector<float4> info(edges.size());
    run_1d((int)edges.size(), [&] { FindEdgeIntersectionInfo(&g_perm, offset, scale, edges.data(), info.data()); });
    // the stored operations replayed as one batch (compute_density_field.cpp:255-271)
    if (num_ops > 0) {
        const int32_t off[3] = {offset.x, offset.y, offset.z};
        if (ref_csg_apply(off, scale, ops, num_ops, materials, edges, info) < 0) return -2;
    }
    const int E = (int)edges.size();
    counts[0] = E;
    if (E > edge_cap) return -1;
    for (int i = 0; i < E; i++) {
        edge_keys[i] = edges[i];
        std::memcpy(edge_info + 4 * i, &info[i], 16);
    }
    if (E == 0) return 0;

    const int C3 = vpc * vpc * vpc;
    std::vector<int> vocc(C3), vedge(C3), vpos(C3), vmat(C3);
    run_3d(vpc, vpc, vpc, [&] { FindActiveVoxels(materials, vocc.data(), vedge.data(), vpos.data(), vmat.data()); });
    std::vector<uint> codes;
    std::vector<int> edge_lists, node_mats;
    for (int i = 0; i < C3; i++)
        if (vocc[i]) {
            codes.push_back((uint)vpos[i]);
            edge_lists.push_back(vedge[i]);
            node_mats.push_back(vmat[i]);
        }
    const int V = (int)codes.size();
    counts[1] = V;
    if (V > node_cap) return -1;
    if (V == 0) return 0;

    std::mt19937 gen(hash_seed);
    HostCuckoo eh;
    eh.build(reinterpret_cast<const uint*>(edges.data()), E, gen);
    std::vector<float4> normals(V), positions(V);
    std::vector<QEFData> qefs(V);
    std::vector<int> vpos_c(codes.begin(), codes.end());
    run_1d(V, [&] {
        CreateLeafNodes(scale, vpos_c.data(), edge_lists.data(), info.data(), normals.data(), qefs.data(),
                        eh.table.data(), eh.stash.data(), eh.prime, eh.params, eh.stash_used);
    });
    const float4 world(min[0], min[1], min[2], 0.f);
    run_1d(V, [&] { SolveQEFs(world, qefs.data(), positions.data()); });

    HostCuckoo nh;
    nh.build(codes.data(), V, gen);
    std::vector<int> valid(3 * V), index_buffer(18 * V);
    run_1d(V, [&] {
        GenerateMesh(codes.data(), node_mats.data(), index_buffer.data(), valid.data(), nh.table.data(),
                     nh.stash.data(), nh.prime, nh.params, nh.stash_used);
    });
    int T = 0;
    for (int i = 0; i < 3 * V; i++)
        if (valid[i])
            for (int k = 0; k < 6; k++) triangles[T++] = index_buffer[6 * i + k];
    counts[2] = T;

    std::vector<MeshVertex> mv(V);
    const float4 col(colour[0], colour[1], colour[2], 0.f);
    run_1d(V, [&] { GenerateMeshVertexBuffer(positions.data(), normals.data(), node_mats.data(), col, mv.data()); });
    for (int v = 0; v < V; v++) std::memcpy(vertices + 12 * (size_t)v, &mv[v], 48);

    std::vector<int> is_seam(V);
    run_1d(V, [&] { FindSeamNodes(codes.data(), is_seam.data()); });
    std::vector<int> scan(V);
    int S = 0;
    for (int v = 0; v < V; v++) {
        scan[v] = S;
        S += is_seam[v];
    }
    std::vector<SeamNodeInfo> sinfo(std::max(S, 1));
    run_1d(V, [&] {
        ExtractSeamNodeInfo(is_seam.data(), scan.data(), codes.data(), node_mats.data(), positions.data(),
                            normals.data(), sinfo.data());
    });
    for (int s = 0; s < S; s++) std::memcpy(seams + 12 * (size_t)s, &sinfo[s], 48);
    counts[3] = S;
    counts[4] = eh.stash_used | (nh.stash_used << 1);
    counts[5] = eh.stash_past_101 | nh.stash_past_101;
    return 0;
}

}
