// ref_csg.cpp -- the reference's own CSG kernels (leven/cl/apply_csg_operation.cl
// with hg_sdf.glsl, and duplicate.cl), compiled on the host through
// cl_shim.h, driven by a host loop that restates ApplyCSGOperations
// (compute_csg.cpp:11-219) and RemoveDuplicates (compute.cpp:450-543).
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref, see ref_cl.cpp).  This file is a
// translation unit of its own: apply_csg_operation.cl and noise.cl both
// include hg_sdf.glsl, and the reference builds them into separate programs.
// Compiled with -ffp-contract=off; apply_csg_operation.cl's functions are
// compiled with fusion (the restatement fuses pR's rotation), duplicate.cl's
// are integer code.
#include "cl_shim.h"

#include <vector>

#include "primes.h"

#define VOXELS_PER_CHUNK 64
#define FIELD_DIM 66
#define VOXEL_INDEX_SHIFT 7
#define VOXEL_INDEX_MASK 127
#define MATERIAL_AIR 201
#define MATERIAL_NONE 200
#define NUM_CSG_BRUSHES 2
#define FIELD_BUFFER_SIZE (FIELD_DIM * FIELD_DIM * FIELD_DIM)
// FilterValidEdges reads the far end of an edge on the field's +x/+y/+z face
// past the field (FindUpdatedEdges makes those edges for updated points on the
// face); the source's PARANOID branch reads AIR there (apply_csg_operation.cl:
// 361-368), the restatement's choice, where the plain build reads out of bounds
#define PARANOID
#define constant static const

namespace refcsg {
#include "cl/shared_constants.cl"
#include "cl/duplicate.cl"
#pragma GCC push_options
#pragma GCC optimize("fp-contract=fast")
#include "cl/apply_csg_operation.cl"
#pragma GCC pop_options
}  // namespace refcsg

namespace {

using namespace refcsg;

template <typename F>
void run_1d(int n, F f) {
    for (int i = 0; i < n; i++) {
        clshim_gid[0] = i;
        f();
    }
}

// stable compaction of `values` where valid != 0 (ExclusiveScan + the
// compaction kernels, sequential)
std::vector<int> compact(const std::vector<int>& values, const std::vector<int>& valid) {
    std::vector<int> out;
    for (size_t i = 0; i < values.size(); i++)
        if (valid[i]) out.push_back(values[i]);
    return out;
}

// RemoveDuplicates (compute.cpp:450-543): rounds of MapSequenceIndices,
// ExtractWinners, MapSequenceValues and ExtractLosers until no losers remain
std::vector<int> remove_duplicates(const std::vector<int>& input) {
    std::vector<int> result;
    if (input.empty()) return result;
    std::vector<int> sequence = input;
    const int prime = FindNextPrime((int)input.size() * 2);
    std::vector<int> table(prime), winners_valid(prime), winners(prime);
    int xor_value = (int)0xdecb7a37;
    int num = (int)sequence.size();
    while (num > 0) {
        std::fill(table.begin(), table.end(), -1);
        run_1d(num, [&] { MapSequenceIndices(sequence.data(), table.data(), prime, xor_value); });
        run_1d(prime, [&] { ExtractWinners(table.data(), sequence.data(), winners_valid.data(), winners.data()); });
        const std::vector<int> cw = compact(winners, winners_valid);
        result.insert(result.end(), cw.begin(), cw.end());
        std::vector<int> cwv(cw);
        run_1d((int)cw.size(), [&] { MapSequenceValues(cwv.data(), table.data(), prime, xor_value); });
        std::vector<int> losers_valid(num), losers(num);
        run_1d(num, [&] {
            ExtractLosers(sequence.data(), table.data(), losers_valid.data(), losers.data(), prime, xor_value);
        });
        sequence = compact(losers, losers_valid);
        if (sequence.empty()) break;
        num = (int)sequence.size();
        xor_value = (int)((unsigned)xor_value * (unsigned)prime);
        xor_value ^= (int)0xe93fbc48;
    }
    return result;
}

}  // namespace

// ApplyCSGOperations on one 64^3 field: materials[66^3] updated in place; the
// field's edge list (keys, info) pruned and extended with the created edges.
// Returns -1 when every field edge is invalidated and none survives the
// prune: there the reference keeps the unpruned list (compute_csg.cpp:156),
// which the harness does not reproduce.
int ref_csg_apply(const int32_t off[3], int scale, const void* ops_bytes, int num_ops, int32_t* materials,
                  std::vector<int>& edge_keys, std::vector<float4>& edge_info) {
    const CSGOperation* ops = static_cast<const CSGOperation*>(ops_bytes);
    const int fd = FIELD_DIM, F = fd * fd * fd;
    const int4 offset(off[0], off[1], off[2], 0);
    std::vector<int> updated(F), new_mats(F);
    std::vector<int4> points(F);
    for (int z = 0; z < fd; z++)
        for (int y = 0; y < fd; y++)
            for (int x = 0; x < fd; x++) {
                clshim_gid[0] = x;
                clshim_gid[1] = y;
                clshim_gid[2] = z;
                CSG_HermiteIndices(offset, num_ops, ops, scale, materials, updated.data(), points.data(),
                                   new_mats.data());
            }
    std::vector<int4> cpoints;
    std::vector<int> cmats;
    for (int i = 0; i < F; i++)
        if (updated[i]) {
            cpoints.push_back(points[i]);
            cmats.push_back(new_mats[i]);
        }
    const int nup = (int)cpoints.size();
    if (nup == 0) return 0;
    run_1d(nup, [&] { UpdateFieldMaterials(cpoints.data(), cmats.data(), materials); });

    std::vector<int> generated(6 * nup), gvalid(6 * nup);
    run_1d(nup, [&] { FindUpdatedEdges(cpoints.data(), generated.data()); });
    run_1d(6 * nup, [&] { RemoveInvalidIndices(generated.data(), gvalid.data()); });
    std::vector<int> invalidated = remove_duplicates(compact(generated, gvalid));
    const int ninv = (int)invalidated.size();
    std::vector<int> valid(ninv);
    run_1d(ninv, [&] { FilterValidEdges(invalidated.data(), materials, valid.data()); });
    std::vector<int> created = compact(invalidated, valid);

    if (ninv > 0 && !edge_keys.empty()) {
        const int ne = (int)edge_keys.size();
        std::vector<int> keep(ne);
        run_1d(ne, [&] { PruneFieldEdges(edge_keys.data(), invalidated.data(), ninv, keep.data()); });
        std::vector<int> pk;
        std::vector<float4> pi;
        for (int i = 0; i < ne; i++)
            if (keep[i]) {
                pk.push_back(edge_keys[i]);
                pi.push_back(edge_info[i]);
            }
        if (pk.empty()) return -1;
        edge_keys = pk;
        edge_info = pi;
    }
    if (!created.empty()) {
        std::vector<float4> cinfo(created.size());
        run_1d((int)created.size(),
               [&] { FindEdgeIntersectionInfo(offset, num_ops, ops, scale, created.data(), cinfo.data()); });
        edge_keys.insert(edge_keys.end(), created.begin(), created.end());
        edge_info.insert(edge_info.end(), cinfo.begin(), cinfo.end());
    }
    return (int)created.size();
}
