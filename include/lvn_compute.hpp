// lvn_compute.hpp -- header-only C++ facade over include/lvn.h with the
// reference engine's compute interface (leven/src/compute.h:35-77), so that
// the engine's call sites (clipmap.cpp:378, 651, 757, 1689-1718; main.cpp:419,
// 587, 599) compile against liblvn with their types swapped for these.
//
// Differences from the reference, all deliberate:
//   * MeshBuffer's fixed arrays (render_types.h:70-90) become std::vectors
//     sized by the callee;
//   * isChunkEmpty reports true when the chunk has no active edge (the
//     reference returns numEdges > 0, compute_density_field.cpp:285,296);
//   * glm types are replaced by plain int[3] / std::array.
#ifndef LVN_COMPUTE_HPP
#define LVN_COMPUTE_HPP

#include <array>
#include <vector>

#include "lvn.h"

typedef lvn_csg_op CSGOperationInfo;
typedef lvn_seam_node SeamNodeInfo;
typedef lvn_mesh_vertex MeshVertex;
typedef lvn_mesh_triangle MeshTriangle;

struct LvnMeshBuffer {
    std::vector<MeshVertex> vertices;
    std::vector<MeshTriangle> triangles;
    int numVertices = 0;
    int numTriangles = 0;
};

inline int Compute_Initialise(int noiseSeed, unsigned int defaultMaterial, int numCSGBrushes) {
    return lvn_initialise(noiseSeed, defaultMaterial, numCSGBrushes);
}
inline int Compute_Shutdown() { return lvn_shutdown(); }
inline int Compute_SetNoiseSeed(int noiseSeed) { return lvn_set_noise_seed(noiseSeed); }
inline int Compute_StoreCSGOperation(const CSGOperationInfo& op, const std::array<int, 3>& aabbMin,
                                     const std::array<int, 3>& aabbMax) {
    return lvn_store_csg_operation(&op, aabbMin.data(), aabbMax.data());
}
inline int Compute_ClearCSGOperations() { return lvn_clear_csg_operations(); }
inline const char* GetCLErrorString(int error) { return lvn_error_string(error); }

class Compute_MeshGenContext {
public:
    static Compute_MeshGenContext* create(int voxelsPerChunk) {
        lvn_meshgen* h = lvn_meshgen_create(voxelsPerChunk);
        if (!h) return nullptr;
        return new Compute_MeshGenContext(h);
    }
    ~Compute_MeshGenContext() { lvn_meshgen_destroy(ctx_); }

    int voxelsPerChunk() const { return lvn_meshgen_voxels_per_chunk(ctx_); }

    int applyCSGOperations(const std::vector<CSGOperationInfo>& opInfo, const std::array<int, 3>& clipmapNodeMin,
                           int clipmapNodeSize) {
        return lvn_meshgen_apply_csg_operations(ctx_, opInfo.data(), (int)opInfo.size(), clipmapNodeMin.data(),
                                                clipmapNodeSize);
    }

    int freeChunkOctree(const std::array<int, 3>& min, int size) {
        return lvn_meshgen_free_chunk_octree(ctx_, min.data(), size);
    }

    int isChunkEmpty(const std::array<int, 3>& min, int size, bool& isEmpty) {
        int32_t e = 0;
        const int rc = lvn_meshgen_is_chunk_empty(ctx_, min.data(), size, &e);
        isEmpty = e != 0;
        return rc;
    }

    int generateChunkMesh(const std::array<int, 3>& min, int clipmapNodeSize, LvnMeshBuffer* meshBuffer,
                          std::vector<SeamNodeInfo>& seamNodeBuffer) {
        int cap = 1 << 14;
        for (;;) {
            meshBuffer->vertices.resize(cap);
            meshBuffer->triangles.resize(2 * (size_t)cap);
            seamNodeBuffer.resize(cap);
            lvn_mesh_out out = {LVN_MEMORY_HOST, meshBuffer->vertices.data(), cap, 0,
                                meshBuffer->triangles.data(), 2 * cap, 0, seamNodeBuffer.data(), cap, 0};
            const int rc = lvn_meshgen_generate_chunk_mesh(ctx_, min.data(), clipmapNodeSize, &out);
            if (rc == LVN_ERR_CAPACITY) {
                int need = out.num_vertices;
                if (out.num_triangles / 2 > need) need = out.num_triangles / 2;
                if (out.num_seams > need) need = out.num_seams;
                cap = 2 * need;
                continue;
            }
            if (rc) return rc;
            meshBuffer->numVertices = out.num_vertices;
            meshBuffer->numTriangles = out.num_triangles;
            meshBuffer->vertices.resize(out.num_vertices);
            meshBuffer->triangles.resize(out.num_triangles);
            seamNodeBuffer.resize(out.num_seams);
            return LVN_OK;
        }
    }

    lvn_meshgen* handle() { return ctx_; }

private:
    explicit Compute_MeshGenContext(lvn_meshgen* h) : ctx_(h) {}
    lvn_meshgen* ctx_;
};

// ngMeshSimplifier (ng_mesh_simplify.cpp:441-540) for one mesh buffer in host
// memory, in place; `options` as MeshSimplificationOptions.  Batches of meshes
// go to lvn_mesh_simplify directly.
inline void ngMeshSimplifier(LvnMeshBuffer* mesh, const std::array<float, 4>& worldSpaceOffset,
                             const lvn_simplify_options& options) {
    if (!mesh || mesh->numTriangles == 0) return;
    lvn_chunk_result r = {0, mesh->numVertices, 0, mesh->numTriangles, 0, 0, 0, 0};
    if (lvn_mesh_simplify(mesh->vertices.data(), mesh->triangles.data(), LVN_MEMORY_HOST, &r, 1,
                          worldSpaceOffset.data(), &options, mesh->vertices.data(), mesh->triangles.data()) != LVN_OK)
        return;
    mesh->numVertices = r.num_vertices;
    mesh->numTriangles = r.num_triangles;
    mesh->vertices.resize(r.num_vertices);
    mesh->triangles.resize(r.num_triangles);
}

// SelectActiveClipmapNodes (clipmap.cpp:1084-1128) for one camera over the
// complete clipmap octree (rootMin, rootSize): the nodes' (min, size).
inline int SelectActiveClipmapNodes(const std::array<float, 3>& cameraPosition, const std::array<int, 3>& rootMin,
                                    int rootSize, std::vector<lvn_chunk_desc>& selectedNodes) {
    int32_t count = 0;
    selectedNodes.resize(1024);
    int rc = lvn_clipmap_select(cameraPosition.data(), 1, rootMin.data(), rootSize, selectedNodes.data(),
                                (int32_t)selectedNodes.size(), &count);
    if (rc == LVN_ERR_CAPACITY) {
        selectedNodes.resize(count);
        rc = lvn_clipmap_select(cameraPosition.data(), 1, rootMin.data(), rootSize, selectedNodes.data(), count,
                                &count);
    }
    selectedNodes.resize(rc == LVN_OK ? count : 0);
    return rc;
}

#endif  // LVN_COMPUTE_HPP
