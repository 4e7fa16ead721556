// lvn_render.cu -- device-resident render meshes: the headless stand-in for
// the engine's GL upload of a MeshBuffer (Render_AllocRenderMesh /
// RenderMesh::uploadData, leven/src/render_mesh.cpp:94-138; its pool of
// MAX_RENDER_MESH meshes, render_mesh.cpp:9-30).
//
// A pool is one vertex arena and one index arena in HBM, allocated once.
// Meshes take first-fit ranges of them (a host-side free list with
// coalescing), so uploading allocates no device memory.  A whole batch's
// chunk meshes, left in device memory by lvn_meshgen_generate_chunks, move
// into their ranges in one gather launch.  A renderer reads a mesh through
// its handle: device pointers to MeshVertex and MeshTriangle data, counts,
// and the position the engine passes with it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/lvn.h"

namespace lvn {
namespace {

// first-fit allocator over [0, capacity) with coalescing free ranges
class RangeAllocator {
   public:
    explicit RangeAllocator(int64_t capacity) : capacity_(capacity) {
        if (capacity > 0) free_[0] = capacity;
    }
    int64_t alloc(int64_t n) {
        if (n <= 0) return 0;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                const int64_t off = it->first, len = it->second;
                free_.erase(it);
                if (len > n) free_[off + n] = len - n;
                used_ += n;
                return off;
            }
        }
        return -1;
    }
    void release(int64_t off, int64_t n) {
        if (n <= 0) return;
        used_ -= n;
        auto next = free_.lower_bound(off);
        int64_t start = off, len = n;
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                start = prev->first;
                len += prev->second;
                free_.erase(prev);
            }
        }
        if (next != free_.end() && off + n == next->first) {
            len += next->second;
            free_.erase(next);
        }
        free_[start] = len;
    }
    int64_t used() const { return used_; }

   private:
    int64_t capacity_;
    int64_t used_ = 0;
    std::map<int64_t, int64_t> free_;  // offset -> length
};

struct Mesh {
    bool live = false;
    int64_t v_off = 0, t_off = 0;
    int32_t nv = 0, nt = 0;
    float position[3] = {0.f, 0.f, 0.f};
};

struct CopyJob {  // one chunk mesh of a batch into its pool ranges
    int64_t src_v, src_t, dst_v, dst_t;
    int32_t nv, nt;
};

__global__ void k_render_gather(const CopyJob* __restrict__ jobs, const lvn_mesh_vertex* __restrict__ src_v,
                                const lvn_mesh_triangle* __restrict__ src_t, lvn_mesh_vertex* __restrict__ dst_v,
                                lvn_mesh_triangle* __restrict__ dst_t) {
    const CopyJob J = jobs[blockIdx.x];
    // 16-byte words: a MeshVertex is 3, a MeshTriangle 3 / 4
    const float4* sv = reinterpret_cast<const float4*>(src_v + J.src_v);
    float4* dv = reinterpret_cast<float4*>(dst_v + J.dst_v);
    for (int i = threadIdx.x; i < 3 * J.nv; i += blockDim.x) dv[i] = sv[i];
    const int32_t* st = reinterpret_cast<const int32_t*>(src_t + J.src_t);
    int32_t* dt = reinterpret_cast<int32_t*>(dst_t + J.dst_t);
    for (int i = threadIdx.x; i < 3 * J.nt; i += blockDim.x) dt[i] = st[i];
}

int cuda_rc(cudaError_t e) {
    if (e == cudaSuccess) return LVN_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? LVN_ERR_OUT_OF_MEMORY : LVN_ERR_CUDA;
}

#define RP_TRY(x)                        \
    do {                                 \
        const int rc__ = cuda_rc(x);     \
        if (rc__ != LVN_OK) return rc__; \
    } while (0)

}  // namespace
}  // namespace lvn

using namespace lvn;

struct lvn_render_pool {
    std::mutex mu;
    lvn_mesh_vertex* vertices = nullptr;
    lvn_mesh_triangle* triangles = nullptr;
    RangeAllocator valloc{0}, talloc{0};
    std::vector<Mesh> meshes;
    std::vector<int32_t> free_handles;
    cudaStream_t stream = nullptr;
    CopyJob* jobs = nullptr;
    int32_t jobs_cap = 0;
};

namespace {

// a mesh's ranges, or an error (capacity) with nothing taken
int take(lvn_render_pool* p, int32_t nv, int32_t nt, const float position[3], int32_t* handle) {
    if (p->free_handles.empty()) return LVN_ERR_CAPACITY;
    const int64_t vo = p->valloc.alloc(nv);
    if (vo < 0) return LVN_ERR_CAPACITY;
    const int64_t to = p->talloc.alloc(nt);
    if (to < 0) {
        p->valloc.release(vo, nv);
        return LVN_ERR_CAPACITY;
    }
    const int32_t h = p->free_handles.back();
    p->free_handles.pop_back();
    Mesh& m = p->meshes[h];
    m.live = true;
    m.v_off = vo;
    m.t_off = to;
    m.nv = nv;
    m.nt = nt;
    for (int a = 0; a < 3; a++) m.position[a] = position ? position[a] : 0.f;
    *handle = h;
    return LVN_OK;
}

void give_back(lvn_render_pool* p, int32_t h) {
    Mesh& m = p->meshes[h];
    p->valloc.release(m.v_off, m.nv);
    p->talloc.release(m.t_off, m.nt);
    m = Mesh();
    p->free_handles.push_back(h);
}

}  // namespace

extern "C" {

lvn_render_pool* lvn_render_pool_create(int64_t vertex_capacity, int64_t triangle_capacity, int32_t max_meshes) {
    if (vertex_capacity <= 0 || triangle_capacity <= 0 || max_meshes <= 0) return nullptr;
    lvn_render_pool* p = new lvn_render_pool();
    if (cudaMalloc(&p->vertices, sizeof(lvn_mesh_vertex) * vertex_capacity) != cudaSuccess ||
        cudaMalloc(&p->triangles, sizeof(lvn_mesh_triangle) * triangle_capacity) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(p->vertices);
        cudaFree(p->triangles);
        delete p;
        return nullptr;
    }
    p->valloc = RangeAllocator(vertex_capacity);
    p->talloc = RangeAllocator(triangle_capacity);
    p->meshes.resize(max_meshes);
    for (int32_t h = max_meshes - 1; h >= 0; h--) p->free_handles.push_back(h);
    return p;
}

void lvn_render_pool_destroy(lvn_render_pool* p) {
    if (!p) return;
    cudaStreamSynchronize(p->stream);
    cudaFree(p->vertices);
    cudaFree(p->triangles);
    cudaFree(p->jobs);
    cudaStreamDestroy(p->stream);
    delete p;
}

int lvn_render_mesh_upload(lvn_render_pool* p, const lvn_mesh_vertex* vertices, int32_t num_vertices,
                           const lvn_mesh_triangle* triangles, int32_t num_triangles, int32_t memory,
                           const float position[3], int32_t* handle) {
    if (!p || !handle || num_vertices < 0 || num_triangles < 0 ||
        (memory != LVN_MEMORY_HOST && memory != LVN_MEMORY_DEVICE))
        return LVN_ERR_INVALID;
    *handle = -1;
    if (num_triangles == 0) return LVN_OK;  // no render mesh (render_mesh.cpp:117-120)
    if (!vertices || !triangles || num_vertices == 0) return LVN_ERR_INVALID;
    std::lock_guard<std::mutex> lock(p->mu);
    int32_t h = -1;
    int rc = take(p, num_vertices, num_triangles, position, &h);
    if (rc) return rc;
    const Mesh& m = p->meshes[h];
    const cudaMemcpyKind kind = memory == LVN_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpyAsync(p->vertices + m.v_off, vertices, sizeof(lvn_mesh_vertex) * num_vertices, kind,
                                    p->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->triangles + m.t_off, triangles, sizeof(lvn_mesh_triangle) * num_triangles, kind,
                            p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) {
        give_back(p, h);
        return cuda_rc(e);
    }
    *handle = h;
    return LVN_OK;
}

int lvn_render_meshes_from_batch(lvn_render_pool* p, const lvn_batch_out* batch, int32_t num_chunks,
                                 const float* positions, int32_t* handles) {
    if (!p || !batch || !handles || num_chunks < 0 || (num_chunks > 0 && !batch->chunks) ||
        batch->memory != LVN_MEMORY_DEVICE)
        return LVN_ERR_INVALID;
    std::lock_guard<std::mutex> lock(p->mu);
    std::vector<CopyJob> jobs;
    std::vector<int32_t> taken;
    for (int32_t c = 0; c < num_chunks; c++) {
        handles[c] = -1;
        const lvn_chunk_result& r = batch->chunks[c];
        if (r.num_triangles == 0) continue;  // no render mesh
        int32_t h = -1;
        const int rc = take(p, r.num_vertices, r.num_triangles, positions ? positions + 3 * c : nullptr, &h);
        if (rc) {  // all or nothing
            for (int32_t t : taken) give_back(p, t);
            for (int32_t k = 0; k < num_chunks; k++) handles[k] = -1;
            return rc;
        }
        taken.push_back(h);
        handles[c] = h;
        const Mesh& m = p->meshes[h];
        jobs.push_back({r.vertex_offset, r.triangle_offset, m.v_off, m.t_off, r.num_vertices, r.num_triangles});
    }
    if (jobs.empty()) return LVN_OK;
    cudaError_t e = cudaSuccess;
    if ((int32_t)jobs.size() > p->jobs_cap) {
        cudaFree(p->jobs);
        p->jobs = nullptr;
        p->jobs_cap = 0;
        e = cudaMalloc(&p->jobs, sizeof(CopyJob) * jobs.size());
        if (e == cudaSuccess) p->jobs_cap = (int32_t)jobs.size();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->jobs, jobs.data(), sizeof(CopyJob) * jobs.size(), cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) {
        k_render_gather<<<(int)jobs.size(), 256, 0, p->stream>>>(p->jobs, batch->vertices, batch->triangles,
                                                                  p->vertices, p->triangles);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) {
        for (int32_t t : taken) give_back(p, t);
        for (int32_t k = 0; k < num_chunks; k++) handles[k] = -1;
        return cuda_rc(e);
    }
    return LVN_OK;
}

int lvn_render_mesh_get(lvn_render_pool* p, int32_t handle, lvn_render_mesh_view* out) {
    if (!p || !out) return LVN_ERR_INVALID;
    std::lock_guard<std::mutex> lock(p->mu);
    if (handle < 0 || handle >= (int32_t)p->meshes.size() || !p->meshes[handle].live) return LVN_ERR_INVALID;
    const Mesh& m = p->meshes[handle];
    out->vertices = p->vertices + m.v_off;
    out->num_vertices = m.nv;
    out->triangles = p->triangles + m.t_off;
    out->num_triangles = m.nt;
    for (int a = 0; a < 3; a++) out->position[a] = m.position[a];
    return LVN_OK;
}

int lvn_render_mesh_download(lvn_render_pool* p, int32_t handle, lvn_mesh_vertex* vertices,
                             lvn_mesh_triangle* triangles) {
    if (!p || !vertices || !triangles) return LVN_ERR_INVALID;
    std::lock_guard<std::mutex> lock(p->mu);
    if (handle < 0 || handle >= (int32_t)p->meshes.size() || !p->meshes[handle].live) return LVN_ERR_INVALID;
    const Mesh& m = p->meshes[handle];
    RP_TRY(cudaMemcpyAsync(vertices, p->vertices + m.v_off, sizeof(lvn_mesh_vertex) * m.nv, cudaMemcpyDeviceToHost,
                           p->stream));
    RP_TRY(cudaMemcpyAsync(triangles, p->triangles + m.t_off, sizeof(lvn_mesh_triangle) * m.nt,
                           cudaMemcpyDeviceToHost, p->stream));
    RP_TRY(cudaStreamSynchronize(p->stream));
    return LVN_OK;
}

int lvn_render_mesh_free(lvn_render_pool* p, int32_t handle) {
    if (!p) return LVN_ERR_INVALID;
    std::lock_guard<std::mutex> lock(p->mu);
    if (handle < 0 || handle >= (int32_t)p->meshes.size() || !p->meshes[handle].live) return LVN_ERR_INVALID;
    give_back(p, handle);
    return LVN_OK;
}

int lvn_render_pool_usage(lvn_render_pool* p, int64_t* vertices_used, int64_t* triangles_used, int32_t* meshes) {
    if (!p) return LVN_ERR_INVALID;
    std::lock_guard<std::mutex> lock(p->mu);
    if (vertices_used) *vertices_used = p->valloc.used();
    if (triangles_used) *triangles_used = p->talloc.used();
    if (meshes) *meshes = (int32_t)(p->meshes.size() - p->free_handles.size());
    return LVN_OK;
}

}  // extern "C"
