"""Python binding of liblvn, the GB300-native chunk-meshing library.

Mirrors the reference engine's compute interface (leven/src/compute.h:35-77):
module functions for the global state (initialise, set_noise_seed,
store_csg_operation, clear_csg_operations) and `MeshGen` for the
Compute_MeshGenContext methods (apply_csg_operations, free_chunk_octree,
is_chunk_empty, generate_chunk_mesh), plus the batched `generate_chunks`.
Errors surface as `LvnError` carrying the library's negative code.

The compute path is liblvn.so only: if the library is missing this module
raises on first use; nothing falls back to a CPU implementation.
"""
import ctypes as C
import pathlib

import numpy as np

_PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = _PKG / "liblvn.so"

LVN_OK = 0
LVN_ERR_NO_DEVICE = -1
LVN_ERR_OUT_OF_MEMORY = -5
LVN_ERR_INVALID = -30
LVN_ERR_CAPACITY = -100
LVN_ERR_NOT_INITIALISED = -101
LVN_ERR_HASH = -102
LVN_ERR_DEVICE_STATUS = -103
LVN_ERR_CUDA = -99999
LVN_MEMORY_HOST = 0
LVN_MEMORY_DEVICE = 1
LVN_DENSITY_REFERENCE, LVN_DENSITY_FBM2D, LVN_DENSITY_CAVES = 0, 1, 2
LVN_OPT_CROSSING_MODE, LVN_OPT_CACHE, LVN_OPT_PROFILE, LVN_OPT_GRAPHS, LVN_OPT_HOST_WRITES = 1, 2, 3, 4, 5
LVN_OPT_COMPUTE_ORDER, LVN_OPT_HERMITE_FORM = 6, 7
(DEBUG_MATERIALS, DEBUG_EDGE_KEYS, DEBUG_EDGE_INFO, DEBUG_NODE_CODES, DEBUG_NODE_INFO, DEBUG_EDGE_TABLE,
 DEBUG_EDGE_STASH, DEBUG_NODE_TABLE, DEBUG_NODE_STASH, DEBUG_PLAIN_EDGES, DEBUG_SIMP_REPS) = range(11)


class LvnError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        super().__init__(f"{what}: {error_string(code)} ({code})")


class CsgOp(C.Structure):
    """CSGOperationInfo (leven/src/compute.h:16-24)."""
    _fields_ = [("type", C.c_int32), ("brush_shape", C.c_int32), ("material", C.c_int32),
                ("rotate_y", C.c_float), ("origin", C.c_float * 4), ("dimensions", C.c_float * 4)]


class DensityParams(C.Structure):
    _fields_ = [("mode", C.c_int32), ("octaves2", C.c_int32), ("freq2", C.c_float), ("lacunarity2", C.c_float),
                ("gain2", C.c_float), ("amp2", C.c_float), ("octaves3", C.c_int32), ("freq3", C.c_float),
                ("lacunarity3", C.c_float), ("gain3", C.c_float), ("amp3", C.c_float)]


class MeshOut(C.Structure):
    _fields_ = [("memory", C.c_int32), ("vertices", C.c_void_p), ("vertex_capacity", C.c_int32),
                ("num_vertices", C.c_int32), ("triangles", C.c_void_p), ("triangle_capacity", C.c_int32),
                ("num_triangles", C.c_int32), ("seams", C.c_void_p), ("seam_capacity", C.c_int32),
                ("num_seams", C.c_int32)]


class ChunkDesc(C.Structure):
    _fields_ = [("min", C.c_int32 * 3), ("size", C.c_int32)]


class ChunkResult(C.Structure):
    _fields_ = [("vertex_offset", C.c_int32), ("num_vertices", C.c_int32), ("triangle_offset", C.c_int32),
                ("num_triangles", C.c_int32), ("seam_offset", C.c_int32), ("num_seams", C.c_int32),
                ("num_edges", C.c_int32), ("num_nodes", C.c_int32)]


class SimplifyOptions(C.Structure):
    _fields_ = [("edge_fraction", C.c_float), ("max_iterations", C.c_int32), ("target_percentage", C.c_float),
                ("max_error", C.c_float), ("max_edge_size", C.c_float), ("min_angle_cosine", C.c_float)]


class RenderMeshView(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("num_vertices", C.c_int32), ("triangles", C.c_void_p),
                ("num_triangles", C.c_int32), ("position", C.c_float * 3)]


class BatchOut(C.Structure):
    _fields_ = [("memory", C.c_int32), ("vertices", C.c_void_p), ("vertex_capacity", C.c_int64),
                ("total_vertices", C.c_int64), ("triangles", C.c_void_p), ("triangle_capacity", C.c_int64),
                ("total_triangles", C.c_int64), ("seams", C.c_void_p), ("seam_capacity", C.c_int64),
                ("total_seams", C.c_int64), ("chunks", C.POINTER(ChunkResult))]


# every symbol include/lvn.h declares
EXPORTS = [
    "lvn_initialise", "lvn_shutdown", "lvn_set_noise_seed", "lvn_store_csg_operation", "lvn_clear_csg_operations",
    "lvn_csg_operation_bounds", "lvn_set_density", "lvn_error_string", "lvn_meshgen_create", "lvn_meshgen_destroy",
    "lvn_meshgen_voxels_per_chunk", "lvn_meshgen_apply_csg_operations", "lvn_meshgen_free_chunk_octree",
    "lvn_meshgen_is_chunk_empty", "lvn_meshgen_generate_chunk_mesh", "lvn_meshgen_generate_chunks",
    "lvn_meshgen_set_stream", "lvn_meshgen_get_stream", "lvn_meshgen_set_option", "lvn_meshgen_stage_times",
    "lvn_meshgen_stage_name", "lvn_meshgen_reset_stage_times", "lvn_meshgen_set_simplify",
    "lvn_meshgen_autotune", "lvn_meshgen_debug_fetch", "lvn_generate_chunk_mesh_noalloc",
    "lvn_surrogate_create", "lvn_surrogate_destroy", "lvn_surrogate_num_params", "lvn_surrogate_set_params",
    "lvn_surrogate_get_params", "lvn_surrogate_sample", "lvn_surrogate_train", "lvn_surrogate_grad",
    "lvn_surrogate_eval", "lvn_surrogate_eval_lattices", "lvn_surrogate_domain", "lvn_surrogate_get_stream",
    "lvn_meshgen_set_surrogate", "lvn_meshgen_surrogate_chunks", "lvn_density_f64",
    "lvn_clipmap_select", "lvn_clipmap_select_device", "lvn_clipmap_touched", "lvn_seam_generate",
    "lvn_simplify_options_default", "lvn_mesh_simplify", "lvn_render_pool_create", "lvn_render_pool_destroy",
    "lvn_render_mesh_upload", "lvn_render_meshes_from_batch", "lvn_render_mesh_get", "lvn_render_mesh_download",
    "lvn_render_mesh_free",
    "lvn_render_pool_usage", "lvn_meshgen_qef_fp64_error", "lvn_debug_cuckoo", "lvn_debug_inject_fault",
    "lvn_meshgen_generate_chunks_async", "lvn_meshgen_wait",
]

_lib = None


def lib():
    """Loads liblvn.so (built in-tree by leven_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(str(LIB_PATH))
    i32p = C.POINTER(C.c_int32)
    L.lvn_initialise.argtypes = [C.c_int32, C.c_uint32, C.c_int32]
    L.lvn_set_noise_seed.argtypes = [C.c_int32]
    L.lvn_store_csg_operation.argtypes = [C.POINTER(CsgOp), i32p, i32p]
    L.lvn_csg_operation_bounds.argtypes = [C.POINTER(CsgOp), i32p, i32p]
    L.lvn_set_density.argtypes = [C.POINTER(DensityParams)]
    L.lvn_error_string.argtypes = [C.c_int32]
    L.lvn_error_string.restype = C.c_char_p
    L.lvn_meshgen_create.argtypes = [C.c_int32]
    L.lvn_meshgen_create.restype = C.c_void_p
    L.lvn_meshgen_destroy.argtypes = [C.c_void_p]
    L.lvn_meshgen_destroy.restype = None
    L.lvn_meshgen_voxels_per_chunk.argtypes = [C.c_void_p]
    L.lvn_meshgen_apply_csg_operations.argtypes = [C.c_void_p, C.POINTER(CsgOp), C.c_int32, i32p, C.c_int32]
    L.lvn_meshgen_free_chunk_octree.argtypes = [C.c_void_p, i32p, C.c_int32]
    L.lvn_meshgen_is_chunk_empty.argtypes = [C.c_void_p, i32p, C.c_int32, i32p]
    L.lvn_meshgen_generate_chunk_mesh.argtypes = [C.c_void_p, i32p, C.c_int32, C.POINTER(MeshOut)]
    L.lvn_meshgen_generate_chunks.argtypes = [C.c_void_p, C.POINTER(ChunkDesc), C.c_int32, C.POINTER(BatchOut)]
    L.lvn_meshgen_generate_chunks_async.argtypes = [C.c_void_p, C.POINTER(ChunkDesc), C.c_int32, C.POINTER(BatchOut)]
    L.lvn_meshgen_wait.argtypes = [C.c_void_p]
    L.lvn_meshgen_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    L.lvn_meshgen_get_stream.argtypes = [C.c_void_p]
    L.lvn_meshgen_get_stream.restype = C.c_void_p
    L.lvn_meshgen_set_option.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    L.lvn_meshgen_stage_times.argtypes = [C.c_void_p, C.POINTER(C.c_float), i32p, C.c_int32]
    L.lvn_meshgen_stage_name.argtypes = [C.c_int32]
    L.lvn_meshgen_stage_name.restype = C.c_char_p
    L.lvn_meshgen_reset_stage_times.argtypes = [C.c_void_p]
    L.lvn_meshgen_set_simplify.argtypes = [C.c_void_p, C.c_float]
    L.lvn_meshgen_autotune.argtypes = [C.c_void_p, C.POINTER(ChunkDesc), C.c_int32, i32p]
    f32p = C.POINTER(C.c_float)
    L.lvn_surrogate_create.argtypes = [C.c_float * 3, C.c_float * 3, C.c_uint64]
    L.lvn_surrogate_create.restype = C.c_void_p
    L.lvn_surrogate_destroy.argtypes = [C.c_void_p]
    L.lvn_surrogate_destroy.restype = None
    L.lvn_surrogate_set_params.argtypes = [C.c_void_p, f32p, C.c_int64]
    L.lvn_surrogate_get_params.argtypes = [C.c_void_p, f32p, C.c_int64]
    L.lvn_surrogate_sample.argtypes = [C.c_void_p, C.c_int64, C.c_uint64, C.c_void_p]
    L.lvn_surrogate_train.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_void_p]
    L.lvn_surrogate_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, f32p]
    L.lvn_surrogate_eval.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32]
    L.lvn_surrogate_get_stream.argtypes = [C.c_void_p]
    L.lvn_surrogate_eval_lattices.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
    L.lvn_surrogate_domain.argtypes = [C.c_void_p, C.c_float * 3, C.c_float * 3]
    L.lvn_meshgen_set_surrogate.argtypes = [C.c_void_p, C.c_void_p, C.c_float]
    L.lvn_meshgen_surrogate_chunks.argtypes = [C.c_void_p, i32p, C.c_int32]
    L.lvn_density_f64.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
    L.lvn_clipmap_select.argtypes = [C.c_void_p, C.c_int32, i32p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]
    L.lvn_clipmap_select_device.argtypes = [C.c_void_p, C.c_int32, i32p, C.c_int32, C.c_void_p, C.c_int32,
                                            C.c_void_p, C.c_void_p]
    L.lvn_clipmap_touched.argtypes = [C.POINTER(CsgOp), C.c_int32, i32p, C.c_int32, C.c_void_p, C.c_int32, i32p]
    L.lvn_simplify_options_default.argtypes = [C.POINTER(SimplifyOptions)]
    L.lvn_simplify_options_default.restype = None
    L.lvn_mesh_simplify.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(ChunkResult), C.c_int32, C.c_void_p,
                                    C.POINTER(SimplifyOptions), C.c_void_p, C.c_void_p]
    L.lvn_render_pool_create.argtypes = [C.c_int64, C.c_int64, C.c_int32]
    L.lvn_render_pool_create.restype = C.c_void_p
    L.lvn_render_pool_destroy.argtypes = [C.c_void_p]
    L.lvn_render_pool_destroy.restype = None
    L.lvn_render_mesh_upload.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32,
                                         C.c_void_p, i32p]
    L.lvn_render_meshes_from_batch.argtypes = [C.c_void_p, C.POINTER(BatchOut), C.c_int32, C.c_void_p, C.c_void_p]
    L.lvn_render_mesh_get.argtypes = [C.c_void_p, C.c_int32, C.POINTER(RenderMeshView)]
    L.lvn_render_mesh_download.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    L.lvn_render_mesh_free.argtypes = [C.c_void_p, C.c_int32]
    L.lvn_render_pool_usage.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), i32p]
    L.lvn_seam_generate.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, i32p,
                                    C.c_int32, C.c_void_p, C.c_int32, C.c_float * 3, C.POINTER(BatchOut)]
    L.lvn_surrogate_get_stream.restype = C.c_void_p
    L.lvn_meshgen_debug_fetch.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int64]
    L.lvn_meshgen_debug_fetch.restype = C.c_int64
    L.lvn_generate_chunk_mesh_noalloc.argtypes = [i32p, C.c_int32, C.c_int32, C.POINTER(MeshOut), C.c_void_p]
    L.lvn_debug_cuckoo.argtypes = [C.c_void_p, C.c_int32, C.c_uint32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64,
                                   i32p]
    L.lvn_debug_inject_fault.argtypes = [C.c_int32, C.c_int32]
    L.lvn_meshgen_qef_fp64_error.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    _lib = L
    return L


def error_string(code):
    try:
        return lib().lvn_error_string(code).decode()
    except ImportError:
        return "liblvn unavailable"


def _check(rc, what):
    if rc < 0:
        raise LvnError(rc, what)
    return rc


def _ivec3(v):
    return (C.c_int32 * 3)(*[int(x) for x in v])


def make_op(type_, brush_shape, material, origin, dimensions, rotate_y=0.0):
    op = CsgOp()
    op.type, op.brush_shape, op.material, op.rotate_y = type_, brush_shape, material, rotate_y
    op.origin = (C.c_float * 4)(origin[0], origin[1], origin[2], 0.0)
    op.dimensions = (C.c_float * 4)(dimensions[0], dimensions[1], dimensions[2], 0.0)
    return op


def initialise(noise_seed, default_material=0, num_csg_brushes=2):
    """Compute_Initialise (compute.h:35)."""
    return _check(lib().lvn_initialise(noise_seed, default_material, num_csg_brushes), "lvn_initialise")


def shutdown():
    return _check(lib().lvn_shutdown(), "lvn_shutdown")


def set_noise_seed(seed):
    return _check(lib().lvn_set_noise_seed(seed), "lvn_set_noise_seed")


def set_density(mode=LVN_DENSITY_REFERENCE, octaves2=8, freq2=1.0 / 256, lacunarity2=2.0, gain2=0.5, amp2=48.0,
                octaves3=6, freq3=1.0 / 64, lacunarity3=2.0, gain3=0.5, amp3=12.0):
    p = DensityParams(mode, octaves2, freq2, lacunarity2, gain2, amp2, octaves3, freq3, lacunarity3, gain3, amp3)
    return _check(lib().lvn_set_density(C.byref(p)), "lvn_set_density")


def csg_operation_bounds(op):
    lo, hi = (C.c_int32 * 3)(), (C.c_int32 * 3)()
    _check(lib().lvn_csg_operation_bounds(C.byref(op), lo, hi), "lvn_csg_operation_bounds")
    return list(lo), list(hi)


LVN_CLIPMAP_MAX_NODES = 8192


def clipmap_select(cameras, root_min, root_size):
    """SelectActiveClipmapNodes (clipmap.cpp:1084-1128) for every camera of
    `cameras` (n x 3) over the complete octree (root_min, root_size), in one
    launch.  Returns one (count, 4) int32 array (min x, y, z, size) per camera,
    in the reference's recursion order."""
    cams = np.ascontiguousarray(np.asarray(cameras, dtype=np.float32).reshape(-1, 3))
    n = cams.shape[0]
    counts = np.zeros(max(n, 1), np.int32)
    cap = max(1024, 640 * n)
    for _ in range(2):
        out = np.zeros((cap, 4), np.int32)
        rc = lib().lvn_clipmap_select(cams.ctypes.data, n, _ivec3(root_min), int(root_size), out.ctypes.data, cap,
                                      counts.ctypes.data)
        if rc != LVN_ERR_CAPACITY:
            break
        cap = int(counts[:n].sum())
    _check(rc, "lvn_clipmap_select")
    offs = np.concatenate([[0], np.cumsum(counts[:n])])
    return [out[offs[i]:offs[i + 1]] for i in range(n)]


def clipmap_select_device(d_cameras, root_min, root_size, d_out, stride, d_counts, stream=None):
    """The device form: torch tensors d_cameras (n, 3) f32, d_out (n * stride, 4)
    i32, d_counts (n,) i32, all on the GPU; enqueued on `stream` (a
    torch.cuda.Stream, default the current stream), no host synchronisation."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    n = d_cameras.shape[0]
    return _check(lib().lvn_clipmap_select_device(d_cameras.data_ptr(), n, _ivec3(root_min), int(root_size),
                                                  d_out.data_ptr(), int(stride), d_counts.data_ptr(),
                                                  C.c_void_p(s.cuda_stream)), "lvn_clipmap_select_device")


def seam_generate(chunks, seam_offsets, seams, voxels_per_chunk, root_min, root_size, hosts,
                  colour=(1.0, 1.0, 1.0)):
    """GenerateClipmapSeamMesh (clipmap.cpp:573-610) for every host in `hosts`
    (indices into `chunks`, the clipmap's active nodes as (min_xyz, size)).
    `seams`: (S, 12) int32 SeamNodeInfo rows (host) or a torch int32 CUDA
    tensor of the same shape; chunk c's rows are seams[seam_offsets[c] ..
    seam_offsets[c + 1]).  Returns (vertices (V, 12) f32, triangles (T, 3)
    i32, results (H, 8) i32 as lvn_chunk_result)."""
    n = len(chunks)
    descs = (ChunkDesc * max(1, n))()
    for i, (mn, size) in enumerate(chunks):
        descs[i] = ChunkDesc((C.c_int32 * 3)(*[int(v) for v in mn]), int(size))
    offs = np.ascontiguousarray(np.asarray(seam_offsets, np.int32))
    hs = np.ascontiguousarray(np.asarray(hosts, np.int32))
    if isinstance(seams, np.ndarray):
        sp = np.ascontiguousarray(seams.astype(np.int32, copy=False))
        ptr, mem = sp.ctypes.data, LVN_MEMORY_HOST
    else:
        ptr, mem = seams.data_ptr(), LVN_MEMORY_DEVICE
    results = (ChunkResult * max(1, len(hs)))()
    cap_v, cap_t = 1 << 16, 1 << 17
    while True:
        v = np.zeros((cap_v, 12), np.float32)
        t = np.zeros((cap_t, 3), np.int32)
        bo = BatchOut(LVN_MEMORY_HOST, v.ctypes.data, cap_v, 0, t.ctypes.data, cap_t, 0, None, 0, 0,
                      C.cast(results, C.POINTER(ChunkResult)))
        rc = lib().lvn_seam_generate(descs, offs.ctypes.data, n, ptr, mem, int(voxels_per_chunk), _ivec3(root_min),
                                     int(root_size), hs.ctypes.data, len(hs), (C.c_float * 3)(*colour), C.byref(bo))
        if rc == LVN_ERR_CAPACITY:
            cap_v, cap_t = max(cap_v, int(bo.total_vertices)), max(cap_t, int(bo.total_triangles))
            continue
        _check(rc, "lvn_seam_generate")
        res = np.ctypeslib.as_array(C.cast(results, C.POINTER(C.c_int32)), shape=(max(1, len(hs)), 8))[:len(hs)]
        return v[:bo.total_vertices].copy(), t[:bo.total_triangles].copy(), res.copy()


def engine_simplify_options(size, max_error=5.0, max_edge_len=2.5, min_cos=0.7):
    """The options ConstructClipmapNodeData passes for a node of `size`
    (clipmap.cpp:456-462, with the engine's Options defaults, options.h:14-16)."""
    o = SimplifyOptions()
    lib().lvn_simplify_options_default(C.byref(o))
    leaf = 4.0 * (size / 256)
    o.max_error, o.max_edge_size, o.min_angle_cosine = max_error * leaf, max_edge_len * leaf, min_cos
    return o


def node_offset(mn, size):
    """worldSpaceOffset of a clipmap node: vec4(vec3(min) + vec3(size / 2.f), 0) (clipmap.cpp:455)."""
    return [float(np.float32(mn[a]) + np.float32(size / 2.0)) for a in range(3)] + [0.0]


def mesh_simplify(vertices, triangles, ranges, offsets, options):
    """ngMeshSimplifier (ng_mesh_simplify.cpp:441-540) for every mesh of a
    batch in one launch.  vertices (V, 12) f32 and triangles (T, 3) i32 as
    host arrays, or CUDA tensors (simplified in place); ranges (M, 4) =
    (vertex offset, vertices, triangle offset, triangles); offsets (M, 4);
    options: one SimplifyOptions per mesh.  Returns (vertices, triangles,
    ranges) with the simplified meshes at the same offsets."""
    r = np.ascontiguousarray(np.asarray(ranges, np.int32).reshape(-1, 4))
    m = len(r)
    res = (ChunkResult * max(1, m))()
    for i in range(m):
        res[i].vertex_offset, res[i].num_vertices, res[i].triangle_offset, res[i].num_triangles = (int(x) for x in r[i])
    offs = np.ascontiguousarray(np.asarray(offsets, np.float32).reshape(-1, 4))
    opts = (SimplifyOptions * max(1, m))(*options)
    if isinstance(vertices, np.ndarray):
        v = np.ascontiguousarray(vertices, np.float32)
        t = np.ascontiguousarray(triangles, np.int32)
        ov, ot = v.copy(), t.copy()
        _check(lib().lvn_mesh_simplify(v.ctypes.data, t.ctypes.data, LVN_MEMORY_HOST, res, m, offs.ctypes.data, opts,
                                       ov.ctypes.data, ot.ctypes.data), "lvn_mesh_simplify")
    else:
        ov, ot = vertices, triangles
        _check(lib().lvn_mesh_simplify(vertices.data_ptr(), triangles.data_ptr(), LVN_MEMORY_DEVICE, res, m,
                                       offs.ctypes.data, opts, vertices.data_ptr(), triangles.data_ptr()),
               "lvn_mesh_simplify")
    out = np.ctypeslib.as_array(C.cast(res, C.POINTER(C.c_int32)), shape=(max(1, m), 8))[:m, :4].copy()
    return ov, ot, out


class RenderPool:
    """Device-resident render meshes (the headless stand-in for the engine's
    GL upload, render_mesh.cpp:94-138): one vertex and one triangle arena."""

    def __init__(self, vertex_capacity, triangle_capacity, max_meshes=8192):
        self._h = lib().lvn_render_pool_create(int(vertex_capacity), int(triangle_capacity), int(max_meshes))
        if not self._h:
            raise LvnError(LVN_ERR_OUT_OF_MEMORY, "lvn_render_pool_create")

    def close(self):
        if self._h:
            lib().lvn_render_pool_destroy(self._h)
            self._h = None

    def upload(self, vertices, triangles, position=(0.0, 0.0, 0.0)):
        """Host arrays (V, 12) f32 / (T, 3) i32 -> handle (-1: no triangles)."""
        v = np.ascontiguousarray(vertices, np.float32)
        t = np.ascontiguousarray(triangles, np.int32)
        h = C.c_int32(-1)
        pos = np.asarray(position, np.float32)
        _check(lib().lvn_render_mesh_upload(self._h, v.ctypes.data, len(v), t.ctypes.data, len(t), LVN_MEMORY_HOST,
                                            pos.ctypes.data, C.byref(h)), "lvn_render_mesh_upload")
        return h.value

    def from_batch(self, batch_out, n, positions=None):
        handles = np.full(max(1, n), -1, np.int32)
        pos = None if positions is None else np.ascontiguousarray(positions, np.float32)
        _check(lib().lvn_render_meshes_from_batch(self._h, C.byref(batch_out), n,
                                                  None if pos is None else pos.ctypes.data, handles.ctypes.data),
               "lvn_render_meshes_from_batch")
        return handles[:n]

    def view(self, handle):
        v = RenderMeshView()
        _check(lib().lvn_render_mesh_get(self._h, int(handle), C.byref(v)), "lvn_render_mesh_get")
        return v

    def download(self, handle):
        """The mesh's (vertices (V, 12), triangles (T, 3)) as host arrays."""
        v = self.view(handle)
        vs = np.zeros((max(1, v.num_vertices), 12), np.float32)
        ts = np.zeros((max(1, v.num_triangles), 3), np.int32)
        _check(lib().lvn_render_mesh_download(self._h, int(handle), vs.ctypes.data, ts.ctypes.data),
               "lvn_render_mesh_download")
        return vs[:v.num_vertices], ts[:v.num_triangles]

    def free(self, handle):
        return _check(lib().lvn_render_mesh_free(self._h, int(handle)), "lvn_render_mesh_free")

    def usage(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int32()
        _check(lib().lvn_render_pool_usage(self._h, C.byref(a), C.byref(b), C.byref(c)), "lvn_render_pool_usage")
        return a.value, b.value, c.value


def clipmap_touched(ops, root_min, root_size):
    """The clipmap nodes a batch of CSG operations touches (processCSGOperationsImpl,
    clipmap.cpp:1661-1669), each once, in the recursion's post-order: (count, 4) int32."""
    arr = (CsgOp * max(len(ops), 1))(*ops)
    cap = 4096
    count = C.c_int32(0)
    for _ in range(2):
        out = np.zeros((cap, 4), np.int32)
        rc = lib().lvn_clipmap_touched(arr, len(ops), _ivec3(root_min), int(root_size), out.ctypes.data, cap,
                                       C.byref(count))
        if rc != LVN_ERR_CAPACITY:
            break
        cap = count.value
    _check(rc, "lvn_clipmap_touched")
    return out[:count.value]


def store_csg_operation(op, aabb=None):
    """Compute_StoreCSGOperation (compute.h:39); the AABB defaults to the
    engine's CalcCSGOperationBounds."""
    lo, hi = aabb if aabb is not None else csg_operation_bounds(op)
    return _check(lib().lvn_store_csg_operation(C.byref(op), _ivec3(lo), _ivec3(hi)), "lvn_store_csg_operation")


def clear_csg_operations():
    return _check(lib().lvn_clear_csg_operations(), "lvn_clear_csg_operations")


class Mesh:
    """Host copy of one chunk's generateChunkMesh output."""

    def __init__(self, vertices, triangles, seams):
        self.vertices = vertices    # float32 (V, 12): position, normal, colour
        self.triangles = triangles  # int32 (T, 3)
        self.seams = seams          # int32 (S, 12): localspaceMin (4 int), position, normal (as float bits)


class MeshGen:
    """Compute_MeshGenContext (compute.h:46-77) over liblvn."""

    def __init__(self, voxels_per_chunk=64):
        self._h = lib().lvn_meshgen_create(voxels_per_chunk)
        if not self._h:
            raise LvnError(-1, "lvn_meshgen_create")
        self.voxels_per_chunk = voxels_per_chunk

    def close(self):
        if getattr(self, "_h", None):
            lib().lvn_meshgen_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_option(self, option, value):
        return _check(lib().lvn_meshgen_set_option(self._h, option, value), "lvn_meshgen_set_option")

    def set_simplify(self, threshold):
        """Bottom-up octree simplification with QEF-error bound `threshold`
        (voxel^2); a negative threshold turns it off."""
        return _check(lib().lvn_meshgen_set_simplify(self._h, threshold), "lvn_meshgen_set_simplify")

    def autotune(self, chunks):
        """Tune the persistent-grid shapes for batches like `chunks`; returns
        {stage name: CTAs per SM} for the stages it chose."""
        n = len(chunks)
        descs = (ChunkDesc * max(1, n))()
        for i, (mn, size) in enumerate(chunks):
            descs[i] = ChunkDesc((C.c_int32 * 3)(*mn), size)
        out = (C.c_int32 * 32)()
        _check(lib().lvn_meshgen_autotune(self._h, descs, n, out), "lvn_meshgen_autotune")
        names = self.stage_times()
        return {name: out[i] for i, name in enumerate(names) if out[i] > 0}

    def set_surrogate(self, surrogate, gate=0.5):
        """Mesh fresh chunks with a learned surrogate where its probe gate
        passes (None = plain only)."""
        self._surrogate = surrogate  # kept alive while the context uses it
        h = surrogate._h if surrogate is not None else None
        return _check(lib().lvn_meshgen_set_surrogate(self._h, h, gate), "lvn_meshgen_set_surrogate")

    def surrogate_chunks(self, n):
        use = (C.c_int32 * max(1, n))()
        k = lib().lvn_meshgen_surrogate_chunks(self._h, use, n)
        _check(min(k, 0), "lvn_meshgen_surrogate_chunks")
        return np.array(use[:n], np.int32)

    def stream(self):
        return lib().lvn_meshgen_get_stream(self._h)

    def set_stream(self, ptr):
        return _check(lib().lvn_meshgen_set_stream(self._h, ptr), "lvn_meshgen_set_stream")

    def apply_csg_operations(self, ops, min_xyz, size):
        arr = (CsgOp * max(1, len(ops)))(*ops)
        return _check(lib().lvn_meshgen_apply_csg_operations(self._h, arr, len(ops), _ivec3(min_xyz), size),
                      "lvn_meshgen_apply_csg_operations")

    def free_chunk_octree(self, min_xyz, size):
        return _check(lib().lvn_meshgen_free_chunk_octree(self._h, _ivec3(min_xyz), size),
                      "lvn_meshgen_free_chunk_octree")

    def is_chunk_empty(self, min_xyz, size):
        out = C.c_int32(0)
        _check(lib().lvn_meshgen_is_chunk_empty(self._h, _ivec3(min_xyz), size, C.byref(out)),
               "lvn_meshgen_is_chunk_empty")
        return bool(out.value)

    def generate_chunk_mesh(self, min_xyz, size, capacity=1 << 16):
        while True:
            v = np.zeros((capacity, 12), np.float32)
            t = np.zeros((2 * capacity, 3), np.int32)
            s = np.zeros((capacity, 12), np.int32)
            out = MeshOut(LVN_MEMORY_HOST, v.ctypes.data, capacity, 0, t.ctypes.data, 2 * capacity, 0,
                          s.ctypes.data, capacity, 0)
            rc = lib().lvn_meshgen_generate_chunk_mesh(self._h, _ivec3(min_xyz), size, C.byref(out))
            if rc == LVN_ERR_CAPACITY:
                capacity = max(out.num_vertices, out.num_triangles, out.num_seams, capacity) * 2
                continue
            _check(rc, "lvn_meshgen_generate_chunk_mesh")
            return Mesh(v[:out.num_vertices].copy(), t[:out.num_triangles].copy(), s[:out.num_seams].copy())

    def generate_chunks(self, chunks, out=None):
        """Batched generation.  `chunks`: iterable of (min_xyz, size).  Returns
        (vertices, triangles, seams, results) as host arrays, results being a
        numpy structured array of lvn_chunk_result."""
        n = len(chunks)
        descs = (ChunkDesc * max(1, n))()
        for i, (mn, size) in enumerate(chunks):
            descs[i] = ChunkDesc((C.c_int32 * 3)(*mn), size)
        results = (ChunkResult * max(1, n))()
        cap = 1 << 20
        while True:
            v = np.zeros((cap, 12), np.float32)
            t = np.zeros((2 * cap, 3), np.int32)
            s = np.zeros((cap, 12), np.int32)
            bo = BatchOut(LVN_MEMORY_HOST, v.ctypes.data, cap, 0, t.ctypes.data, 2 * cap, 0, s.ctypes.data, cap, 0,
                          C.cast(results, C.POINTER(ChunkResult)))
            rc = lib().lvn_meshgen_generate_chunks(self._h, descs, n, C.byref(bo))
            if rc == LVN_ERR_CAPACITY:
                cap = int(max(bo.total_vertices, bo.total_triangles, bo.total_seams, cap) * 2)
                continue
            _check(rc, "lvn_meshgen_generate_chunks")
            res = np.ctypeslib.as_array(C.cast(results, C.POINTER(C.c_int32)), shape=(max(1, n), 8))[:n].copy()
            return (v[:bo.total_vertices].copy(), t[:bo.total_triangles].copy(), s[:bo.total_seams].copy(), res)

    def generate_chunks_raw(self, descs, n, batch_out):
        """Direct C-ABI call with caller-prepared ctypes structures."""
        return lib().lvn_meshgen_generate_chunks(self._h, descs, n, C.byref(batch_out))

    def generate_chunks_async_raw(self, descs, n, batch_out):
        """lvn_meshgen_generate_chunks_async: returns at once; batch_out and its
        arrays must stay alive and untouched until wait()."""
        return lib().lvn_meshgen_generate_chunks_async(self._h, descs, n, C.byref(batch_out))

    def wait(self):
        """lvn_meshgen_wait: the result code of the batch in flight (0 when none)."""
        return lib().lvn_meshgen_wait(self._h)

    def qef_fp64_error(self):
        """(max, mean, leaves, leaves beyond 1e-3): the FP32 leaf solve's
        distance in voxels from an FP64 solve of the same crossings, over the
        last fresh batch's leaves."""
        out = (C.c_double * 4)()
        _check(lib().lvn_meshgen_qef_fp64_error(self._h, out), "lvn_meshgen_qef_fp64_error")
        return float(out[0]), float(out[1]), int(out[2]), int(out[3])

    def debug_fetch(self, what, chunk, dtype, width=1, max_elems=1 << 22):
        buf = np.zeros(max_elems * width, dtype=dtype)
        n = lib().lvn_meshgen_debug_fetch(self._h, what, chunk, buf.ctypes.data, buf.nbytes)
        _check(int(n), "lvn_meshgen_debug_fetch")
        if what == DEBUG_PLAIN_EDGES:
            return int(n)
        out = buf[: n * width]
        return out.reshape(n, width) if width > 1 else out

    def stage_times(self):
        ms = (C.c_float * 32)()
        launches = (C.c_int32 * 32)()
        n = lib().lvn_meshgen_stage_times(self._h, ms, launches, 32)
        return {lib().lvn_meshgen_stage_name(i).decode(): (ms[i], launches[i]) for i in range(n)}

    def reset_stage_times(self):
        return lib().lvn_meshgen_reset_stage_times(self._h)


class Surrogate:
    """Learned density surrogate (lvn_surrogate_*): Fourier features -> 4 x
    [128, SiLU] -> 1, trained and evaluated with the library's tensor-core
    kernels."""

    def __init__(self, domain_min, domain_max, seed=1):
        self._h = lib().lvn_surrogate_create((C.c_float * 3)(*domain_min), (C.c_float * 3)(*domain_max), seed)
        if not self._h:
            raise LvnError(LVN_ERR_INVALID, "lvn_surrogate_create")
        self.domain_min, self.domain_max = tuple(domain_min), tuple(domain_max)

    def close(self):
        if self._h:
            lib().lvn_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @staticmethod
    def num_params():
        return lib().lvn_surrogate_num_params()

    def params(self):
        out = np.zeros(self.num_params(), np.float32)
        n = lib().lvn_surrogate_get_params(self._h, out.ctypes.data_as(C.POINTER(C.c_float)), out.size)
        _check(min(n, 0), "lvn_surrogate_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _check(lib().lvn_surrogate_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size),
               "lvn_surrogate_set_params")

    def sample(self, n, seed=1, fetch=False):
        out = np.zeros((n, 4), np.float32) if fetch else None
        _check(lib().lvn_surrogate_sample(self._h, n, seed, out.ctypes.data if fetch else None), "lvn_surrogate_sample")
        return out

    def train(self, steps, batch=65536, lr=1e-3):
        losses = np.zeros(max(steps, 1), np.float32)
        _check(lib().lvn_surrogate_train(self._h, steps, batch, lr, losses.ctypes.data), "lvn_surrogate_train")
        return losses[:steps]

    def grad(self, samples):
        samples = np.ascontiguousarray(samples, np.float32)
        g = np.zeros(self.num_params(), np.float32)
        loss = C.c_float()
        _check(lib().lvn_surrogate_grad(self._h, samples.ctypes.data, samples.shape[0], g.ctypes.data, C.byref(loss)),
               "lvn_surrogate_grad")
        return g, loss.value

    def eval(self, points):
        pts = np.zeros((len(points), 4), np.float32)
        pts[:, :3] = np.asarray(points, np.float32)[:, :3]
        out = np.zeros(len(points), np.float32)
        _check(lib().lvn_surrogate_eval(self._h, pts.ctypes.data, pts.shape[0], out.ctypes.data, LVN_MEMORY_HOST),
               "lvn_surrogate_eval")
        return out


LVN_CUCKOO_REFERENCE_FIND = 1
LVN_FAULT_NONE, LVN_FAULT_DEVICE_ALLOC, LVN_FAULT_HASH_FAMILY, LVN_FAULT_HASH_FAMILY_HOST = 0, 1, 2, 3


def debug_cuckoo(keys, prime=0, reference_find=False, with_table=False):
    """The device cuckoo table of the meshing stages over `keys` (distinct
    uint32, value = index): returns (values found per key, ~0 = missing,
    info = (prime, stash used, parameter draws, insert failed), table + stash
    or None)."""
    k = np.ascontiguousarray(keys, np.uint32)
    vals = np.zeros(max(k.size, 1), np.uint32)
    info = (C.c_int32 * 4)()
    p = prime or 0
    slots = 0
    if with_table:
        if not p:
            p = next_prime(max(2048, 2 * k.size))
        slots = p + 101
    table = np.zeros(max(slots, 1), np.uint64)
    rc = lib().lvn_debug_cuckoo(k.ctypes.data, k.size, p, LVN_CUCKOO_REFERENCE_FIND if reference_find else 0,
                                vals.ctypes.data, table.ctypes.data if with_table else None, slots, info)
    _check(rc, "lvn_debug_cuckoo")
    return vals[:k.size], tuple(info), (table if with_table else None)


def next_prime(n):
    """FindNextPrime (primes.cpp:32-58): the smallest prime >= n."""
    x = max(n, 2)
    while any(x % d == 0 for d in range(2, int(x ** 0.5) + 1)):
        x += 1
    return x


def inject_fault(what, count=1):
    """Host-side fault injection for the failure paths (test hook)."""
    _check(lib().lvn_debug_inject_fault(what, count), "lvn_debug_inject_fault")


def density_f64(points):
    """The current density at points (N x 3+) in double precision (GPU)."""
    pts = np.zeros((len(points), 4), np.float32)
    pts[:, :3] = np.asarray(points, np.float32)[:, :3]
    out = np.zeros(len(points), np.float64)
    _check(lib().lvn_density_f64(pts.ctypes.data, pts.shape[0], out.ctypes.data), "lvn_density_f64")
    return out
