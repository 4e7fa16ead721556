"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

The oracle is the checker: tests, the smoke entry point and the bench's CPU
baseline load it; the product never does.
"""
import ctypes as C
import pathlib
import subprocess

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[1]
ORACLE_SO = ROOT / "oracle" / "_build" / "liboracle.so"
REF_SO = ROOT / "oracle" / "_ref" / "libref.so"

(ORC_MATERIALS, ORC_EDGE_KEYS, ORC_EDGE_INFO, ORC_NODE_CODES, ORC_NODE_EDGES, ORC_NODE_MATERIALS,
 ORC_VERTICES, ORC_TRIANGLES, ORC_SEAMS, ORC_PLAIN_EDGE_KEYS, ORC_QEFS, ORC_MESH_VERTEX_COUNT,
 ORC_CREATED_EDGE_KEYS, ORC_SIMP_VERTICES, ORC_SIMP_TRIANGLES, ORC_SIMP_VERTEX_COUNT, ORC_SIMP_REPS,
 ORC_POSITIONS_F64) = range(18)


class CsgOp(C.Structure):
    _fields_ = [("type", C.c_int32), ("brush", C.c_int32), ("material", C.c_int32),
                ("rotate_y", C.c_float), ("origin", C.c_float * 4), ("dimensions", C.c_float * 4)]


class Density(C.Structure):
    _fields_ = [("mode", C.c_int32), ("octaves2", C.c_int32), ("freq2", C.c_float),
                ("lacunarity2", C.c_float), ("gain2", C.c_float), ("amp2", C.c_float),
                ("octaves3", C.c_int32), ("freq3", C.c_float), ("lacunarity3", C.c_float),
                ("gain3", C.c_float), ("amp3", C.c_float)]


class ChunkArgs(C.Structure):
    _fields_ = [("min", C.c_int32 * 3), ("size", C.c_int32), ("voxels_per_chunk", C.c_int32),
                ("default_material", C.c_int32), ("crossing_mode", C.c_int32), ("num_ops", C.c_int32),
                ("ops", C.POINTER(CsgOp)), ("hash_seed", C.c_uint32)]


def build():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "all"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not ORACLE_SO.exists():
            build()
        L = C.CDLL(str(ORACLE_SO))
        L.orc_set_seed.argtypes = [C.c_int32]
        L.orc_perm_lut.argtypes = [C.c_void_p]
        L.orc_density_at.argtypes = [C.POINTER(Density), C.c_float, C.c_float, C.c_float]
        L.orc_density_at.restype = C.c_float
        L.orc_snoise2.argtypes = [C.c_float, C.c_float]
        L.orc_snoise2.restype = C.c_float
        L.orc_snoise3.argtypes = [C.c_float, C.c_float, C.c_float]
        L.orc_snoise3.restype = C.c_float
        L.orc_find_next_prime.argtypes = [C.c_int32]
        L.orc_flop_counts.argtypes = [C.POINTER(Density), C.c_void_p]
        L.orc_chunk_new.restype = C.c_void_p
        L.orc_chunk_free.argtypes = [C.c_void_p]
        L.orc_chunk_run.argtypes = [C.c_void_p, C.POINTER(Density), C.POINTER(ChunkArgs)]
        L.orc_chunk_count.argtypes = [C.c_void_p, C.c_int]
        L.orc_chunk_get.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int64]
        L.orc_chunk_simplify.argtypes = [C.c_void_p, C.c_float]
        L.orc_cuckoo_build.argtypes = [C.c_void_p, C.c_int32, C.c_uint32, C.POINTER(C.c_int32)]
        L.orc_cuckoo_build.restype = C.c_void_p
        L.orc_cuckoo_find.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)]
        L.orc_cuckoo_prime.argtypes = [C.c_void_p]
        L.orc_cuckoo_free.argtypes = [C.c_void_p]
        L.orc_remove_duplicates.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.orc_csg_op_bounds.argtypes = [C.POINTER(CsgOp), C.c_int32 * 3, C.c_int32 * 3]
        L.orc_aabb_overlaps.argtypes = [C.c_int32 * 3] * 4
        L.orc_mesh_chunks.argtypes = [C.POINTER(Density), C.POINTER(ChunkArgs), C.c_int32, C.c_int32]
        L.orc_mesh_chunks.restype = C.c_int64
        L.orc_mesh_chunks_simplified.argtypes = [C.POINTER(Density), C.POINTER(ChunkArgs), C.c_int32, C.c_int32,
                                                 C.c_float]
        L.orc_mesh_chunks_simplified.restype = C.c_int64
        L.orc_clipmap_select.argtypes = [C.c_float * 3, C.c_int32 * 3, C.c_int32, C.c_void_p, C.c_int32]
        L.orc_clipmap_nodes_in_aabb.argtypes = [C.c_int32 * 3, C.c_int32 * 3, C.c_int32 * 3, C.c_int32, C.c_void_p,
                                                C.c_int32]
        L.orc_clipmap_touched.argtypes = [C.POINTER(CsgOp), C.c_int32, C.c_int32 * 3, C.c_int32, C.c_void_p,
                                          C.c_int32]
        L.orc_clipmap_select_many.argtypes = [C.c_void_p, C.c_int32, C.c_int32 * 3, C.c_int32, C.c_int32]
        L.orc_clipmap_select_many.restype = C.c_int64
        L.orc_mesh_collapse.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.POINTER(C.c_int32), C.c_void_p, C.POINTER(C.c_int32)]
        L.orc_mesh_collapse_many.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                             C.c_int32]
        L.orc_mesh_collapse_many.restype = C.c_int64
        L.orc_uniform_draws.argtypes = [C.c_int32, C.c_int32, C.c_void_p]
        L.orc_perm_image_rgba.argtypes = [C.c_void_p]
        L.orc_perm_image_rgba.restype = None
        L.orc_qef_solve_points.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
        L.orc_qef_solve_points.restype = C.c_float
        L.orc_seam_generate.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32 * 3,
                                        C.c_int32, C.c_void_p, C.c_int32, C.c_float * 3, C.c_void_p, C.c_int64,
                                        C.c_void_p, C.c_int64, C.c_void_p, C.c_int32]
        _lib = L
    return _lib


def density(mode=1, octaves2=8, freq2=1.0 / 256.0, lac2=2.0, gain2=0.5, amp2=48.0,
            octaves3=6, freq3=1.0 / 64.0, lac3=2.0, gain3=0.5, amp3=12.0):
    return Density(mode, octaves2, freq2, lac2, gain2, amp2, octaves3, freq3, lac3, gain3, amp3)


def make_ops(ops):
    """ops: list of (type, brush, material, rotate_y, origin[3], dims[3])."""
    arr = (CsgOp * max(1, len(ops)))()
    for i, (t, b, m, r, o, d) in enumerate(ops):
        arr[i] = CsgOp(t, b, m, r, (C.c_float * 4)(o[0], o[1], o[2], 0.0), (C.c_float * 4)(d[0], d[1], d[2], 0.0))
    return arr


class OracleChunk:
    """Runs the oracle pipeline for one chunk and exposes every stage."""

    def __init__(self, dens, min_xyz, size, vpc=64, default_material=0, crossing_mode=0, ops=(), hash_seed=5489):
        L = lib()
        self._h = L.orc_chunk_new()
        self._ops = make_ops(list(ops))
        a = ChunkArgs((C.c_int32 * 3)(*min_xyz), size, vpc, default_material, crossing_mode, len(ops),
                      C.cast(self._ops, C.POINTER(CsgOp)), hash_seed)
        self.scale = size // (vpc * 4)
        rc = L.orc_chunk_run(self._h, C.byref(dens), C.byref(a))
        if rc != 0:
            raise RuntimeError(f"orc_chunk_run failed: {rc}")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_chunk_free(self._h)
            self._h = None

    def count(self, what):
        return lib().orc_chunk_count(self._h, what)

    def get(self, what, dtype, width=1):
        n = self.count(what if what != ORC_VERTICES else ORC_NODE_CODES)
        if what == ORC_TRIANGLES:
            n = self.count(ORC_TRIANGLES)
        out = np.zeros((max(n, 1), width), dtype=dtype)
        got = lib().orc_chunk_get(self._h, what, out.ctypes.data, out.nbytes)
        if got < 0:
            raise RuntimeError(f"orc_chunk_get({what}) failed: {got}")
        out = out[:n]
        return out[:, 0] if width == 1 else out

    # convenience accessors
    def materials(self):
        return self.get(ORC_MATERIALS, np.int32)

    def edge_keys(self):
        return self.get(ORC_EDGE_KEYS, np.int32)

    def plain_edge_keys(self):
        return self.get(ORC_PLAIN_EDGE_KEYS, np.int32)

    def created_edge_keys(self):
        return self.get(ORC_CREATED_EDGE_KEYS, np.int32)

    def edge_info(self):
        return self.get(ORC_EDGE_INFO, np.float32, 4)

    def node_codes(self):
        return self.get(ORC_NODE_CODES, np.uint32)

    def node_edges(self):
        return self.get(ORC_NODE_EDGES, np.int32)

    def node_materials(self):
        return self.get(ORC_NODE_MATERIALS, np.int32)

    def vertices(self):
        return self.get(ORC_VERTICES, np.float32, 12)

    def triangles(self):
        return self.get(ORC_TRIANGLES, np.int32, 3)

    def seams(self):
        return self.get(ORC_SEAMS, np.int32, 12)

    def qefs(self):
        return self.get(ORC_QEFS, np.float32, 16)

    def mesh_vertex_count(self):
        return self.count(ORC_MESH_VERTEX_COUNT)

    def positions_f64(self):
        """(V, 4) float64: each leaf's vertex solved in FP64 from the same
        crossings and normals (world units), and its crossing count."""
        return self.get(ORC_POSITIONS_F64, np.float64, 4)

    def qef_fp64_error_voxels(self, vertices=None):
        """|x_fp32 - x_fp64| per leaf in this chunk's voxels (Euclidean), for
        the FP32 vertices given (default: the oracle's own, which the GPU's
        equal bit for bit) against the FP64 solve."""
        v = self.vertices() if vertices is None else vertices
        p64 = self.positions_f64()
        voxel = 4.0 * self.scale
        return np.sqrt(((v[:, :3].astype(np.float64) - p64[:, :3]) ** 2).sum(1)) / voxel

    # bottom-up octree simplification
    def simplify(self, threshold):
        rc = lib().orc_chunk_simplify(self._h, threshold)
        if rc != 0:
            raise RuntimeError(f"orc_chunk_simplify failed: {rc}")
        return self

    def simp_vertices(self):
        return self.get(ORC_SIMP_VERTICES, np.float32, 12)

    def simp_triangles(self):
        return self.get(ORC_SIMP_TRIANGLES, np.int32, 3)

    def simp_reps(self):
        return self.get(ORC_SIMP_REPS, np.int32)

    def simp_vertex_count(self):
        return self.count(ORC_SIMP_VERTEX_COUNT)


def set_seed(seed):
    lib().orc_set_seed(seed)


def perm_lut():
    out = np.zeros(65536, dtype=np.uint8)
    lib().orc_perm_lut(out.ctypes.data)
    return out


def perm_image_rgba():
    """The RGBA8 permutation image (256 x 256 x 4 bytes) of the current seed."""
    out = np.zeros(256 * 256 * 4, dtype=np.uint8)
    lib().orc_perm_image_rgba(out.ctypes.data)
    return out


_ref = None


def ref_lib():
    """oracle/_ref/libref.so (the reference's own code), or None when it was
    not built (no reference tree)."""
    global _ref
    if _ref is None and REF_SO.exists():
        _ref = C.CDLL(str(REF_SO))
    return _ref


def find_next_prime(n):
    return lib().orc_find_next_prime(n)


def remove_duplicates(values):
    v = np.ascontiguousarray(values, dtype=np.int32)
    out = np.zeros(max(1, v.size), dtype=np.int32)
    n = lib().orc_remove_duplicates(v.ctypes.data, v.size, out.ctypes.data)
    return out[:n]


def op_bounds(op_tuple):
    ops = make_ops([op_tuple])
    lo = (C.c_int32 * 3)()
    hi = (C.c_int32 * 3)()
    lib().orc_csg_op_bounds(ops, lo, hi)
    return list(lo), list(hi)


def _i3(v):
    return (C.c_int32 * 3)(*[int(x) for x in v])


def _nodes(fn, *args):
    cap = 4096
    while True:
        out = np.zeros((cap, 4), np.int32)
        n = fn(*args, out.ctypes.data, cap)
        if n < 0:
            raise ValueError("invalid clipmap root")
        if n <= cap:
            return out[:n]
        cap = n


def clipmap_select(cam, root_min, root_size):
    """SelectActiveClipmapNodes for one camera: (count, 4) int32 in pre-order."""
    return _nodes(lib().orc_clipmap_select, (C.c_float * 3)(*[float(x) for x in cam]), _i3(root_min), int(root_size))


def clipmap_nodes_in_aabb(bmin, bmax, root_min, root_size):
    """FindNodesInsideAABB for one box: (count, 4) int32 in post-order."""
    return _nodes(lib().orc_clipmap_nodes_in_aabb, _i3(bmin), _i3(bmax), _i3(root_min), int(root_size))


def clipmap_touched(op_tuples, root_min, root_size):
    """The CSG touch set of the operations: (count, 4) int32 in post-order."""
    ops = make_ops(op_tuples)
    return _nodes(lib().orc_clipmap_touched, ops, len(op_tuples), _i3(root_min), int(root_size))


def clipmap_select_many(cams, root_min, root_size, threads):
    c = np.ascontiguousarray(np.asarray(cams, np.float32).reshape(-1, 3))
    return lib().orc_clipmap_select_many(c.ctypes.data, c.shape[0], _i3(root_min), int(root_size), int(threads))


def seam_generate(chunks, seam_offsets, seams, vpc, root_min, root_size, hosts, colour=(1.0, 1.0, 1.0), threads=1):
    """GenerateClipmapSeamMesh restated: (vertices (V, 12) f32, triangles (T, 3)
    i32, counts (H, 2) = (vertices, triangles) per host), hosts back to back."""
    c4 = np.ascontiguousarray(np.array([[*mn, s] for mn, s in chunks], np.int32).reshape(-1, 4))
    offs = np.ascontiguousarray(np.asarray(seam_offsets, np.int32))
    sm = np.ascontiguousarray(np.asarray(seams, np.int32).reshape(-1, 12))
    hs = np.ascontiguousarray(np.asarray(hosts, np.int32))
    counts = np.zeros((max(1, len(hs)), 2), np.int32)
    cap_v, cap_t = 1 << 14, 1 << 15
    while True:
        v = np.zeros((cap_v, 12), np.float32)
        t = np.zeros((cap_t, 3), np.int32)
        rc = lib().orc_seam_generate(c4.ctypes.data, offs.ctypes.data, len(c4), sm.ctypes.data, int(vpc), _i3(root_min),
                                     int(root_size), hs.ctypes.data, len(hs), (C.c_float * 3)(*colour), v.ctypes.data,
                                     cap_v, t.ctypes.data, cap_t, counts.ctypes.data, int(threads))
        if rc == -2:
            cap_v, cap_t = int(counts[:, 0].sum()), int(counts[:, 1].sum())
            continue
        assert rc == 0, rc
        nv, nt = int(counts[:len(hs), 0].sum()), int(counts[:len(hs), 1].sum())
        return v[:nv], t[:nt], counts[:len(hs)]


def simplify_options(size, max_error=5.0, max_edge_len=2.5, min_cos=0.7):
    """The options ConstructClipmapNodeData passes for a node of `size`
    (clipmap.cpp:456-462, Options defaults options.h:14-16) as the 6 floats
    orc_mesh_collapse takes."""
    leaf = 4.0 * (size / 256)
    return np.array([0.125, 10, 0.05, max_error * leaf, max_edge_len * leaf, min_cos], np.float32)


def node_offset(mn, size):
    """worldSpaceOffset = vec4(vec3(min) + vec3(size / 2.f), 0) (clipmap.cpp:455)."""
    return np.array([np.float32(mn[0]) + np.float32(size / 2.0), np.float32(mn[1]) + np.float32(size / 2.0),
                     np.float32(mn[2]) + np.float32(size / 2.0), 0.0], np.float32)


def mesh_collapse(vertices, triangles, offset, options):
    """ngMeshSimplifier restated, one mesh: (vertices (V', 12), triangles (T', 3))."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 12)
    t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    ov = np.zeros((max(1, len(v)), 12), np.float32)
    ot = np.zeros((max(1, len(t)), 3), np.int32)
    a, b = C.c_int32(), C.c_int32()
    off = np.ascontiguousarray(offset, np.float32)
    opt = np.ascontiguousarray(options, np.float32)
    lib().orc_mesh_collapse(v.ctypes.data, len(v), t.ctypes.data, len(t), off.ctypes.data, opt.ctypes.data,
                            ov.ctypes.data, C.byref(a), ot.ctypes.data, C.byref(b))
    return ov[:a.value], ot[:b.value]


def uniform_draws(hi, n):
    out = np.zeros(max(1, n), np.int32)
    lib().orc_uniform_draws(int(hi), int(n), out.ctypes.data)
    return out[:n]


def flop_counts(d):
    """The oracle's FP32 operation counts for density d: (height term, rest of
    a density sample, x edge, y edge, z edge), see orc_flop_counts."""
    out = (C.c_int64 * 5)()
    assert lib().orc_flop_counts(C.byref(d), out) == 0
    return tuple(int(v) for v in out)
