"""lvn_generate_chunk_mesh_noalloc: the chunk mesher for callers that cannot
allocate memory.

An engine's render or streaming thread that must never block cannot call
cudaMalloc / cudaFree (cudaFree synchronises the device), and engines that
reserve all GPU memory at start-up forbid allocation afterwards.  This entry
point takes the caller's output arrays and keeps every intermediate buffer in
one static device array, so it allocates nothing.  Its output must equal
lvn_meshgen_generate_chunk_mesh's (caching off) for the same chunk.

Two calls run back to back on different chunks, so that anything the first
call leaves in the shared scratch and the second fails to overwrite or clear
would show up as a difference.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import leven_gb300 as lvn_mod
from leven_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def noalloc_mesh(lvn, mn, size, vpc, capacity=1 << 16):
    v = np.zeros((capacity, 12), np.float32)
    t = np.zeros((2 * capacity, 3), np.int32)
    s = np.zeros((capacity, 12), np.int32)
    out = lvn.MeshOut(lvn.LVN_MEMORY_HOST, v.ctypes.data, capacity, 0, t.ctypes.data, 2 * capacity, 0,
                      s.ctypes.data, capacity, 0)
    rc = lvn.lib().lvn_generate_chunk_mesh_noalloc((C.c_int32 * 3)(*mn), size, vpc, C.byref(out), None)
    assert rc == 0, lvn.error_string(rc)
    return v[:out.num_vertices], t[:out.num_triangles], s[:out.num_seams]


def test_noalloc_matches_generate_chunk_mesh(lvn_gpu):
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    wl = W.tiled_csg(4, 2, 4, n_ops=24, seed=7)
    lvn.clear_csg_operations()
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions))
    nops = [len(W.ops_for_chunk(wl.ops, mn, s)) for mn, s in wl.chunks]
    first = max(range(len(wl.chunks)), key=lambda c: nops[c])          # most CSG operations
    second = min(range(len(wl.chunks)), key=lambda c: nops[c])         # fewest
    mg = lvn.MeshGen(64)
    try:
        mg.set_option(lvn.LVN_OPT_CACHE, 0)
        for c in (first, second):
            mn, size = wl.chunks[c]
            ref = mg.generate_chunk_mesh(mn, size)
            v, t, s = noalloc_mesh(lvn, mn, size, 64)
            assert v.shape == ref.vertices.shape and t.shape == ref.triangles.shape and s.shape == ref.seams.shape
            # same tolerance as the parity tests: 1e-4 voxel on positions and normals, integers exact
            assert np.abs(v[:, :3] - ref.vertices[:, :3]).max(initial=0) <= 4e-4
            assert np.abs(v[:, 4:7] - ref.vertices[:, 4:7]).max(initial=0) <= 1e-4
            assert np.array_equal(v[:, 8:], ref.vertices[:, 8:])
            assert np.array_equal(t, ref.triangles)
            assert np.array_equal(s[:, :4], ref.seams[:, :4])
            assert np.abs(s[:, 4:].view(np.float32) - ref.seams[:, 4:].view(np.float32)).max(initial=0) <= 4e-4
    finally:
        mg.close()
        lvn.clear_csg_operations()


def test_noalloc_caves_density(lvn_gpu):
    """The caves density (a 3D term): the field kernel's cave band and the
    batch fields derived from the density are set on this path too."""
    lvn = lvn_gpu
    lvn.set_density(**W.CAVES)
    lvn.clear_csg_operations()
    mg = lvn.MeshGen(64)
    try:
        mg.set_option(lvn.LVN_OPT_CACHE, 0)
        for mn, size in (((0, 0, 0), 256), ((1024, -1024, 0), 1024)):
            ref = mg.generate_chunk_mesh(mn, size)
            v, t, s = noalloc_mesh(lvn, mn, size, 64)
            assert ref.vertices.shape[0] > 0
            assert v.shape == ref.vertices.shape and t.shape == ref.triangles.shape and s.shape == ref.seams.shape
            assert np.array_equal(v.view(np.int32), ref.vertices.view(np.int32))
            assert np.array_equal(t, ref.triangles)
            assert np.array_equal(s, ref.seams)
    finally:
        mg.close()
        lvn.set_density(**W.FBM2D)


def test_noalloc_rejects_out_of_range(lvn_gpu):
    lvn = lvn_gpu
    out = lvn_mod.MeshOut()
    mn = (C.c_int32 * 3)(0, 0, 0)
    assert lvn.lib().lvn_generate_chunk_mesh_noalloc(mn, 256, 12, C.byref(out), None) == -30
    assert lvn.lib().lvn_generate_chunk_mesh_noalloc(mn, 100, 64, C.byref(out), None) == -30
    # outputs smaller than the mesh: capacity error with the counts set
    lvn.set_density(**W.FBM2D)
    lvn.clear_csg_operations()
    v = np.zeros((4, 12), np.float32)
    t = np.zeros((4, 3), np.int32)
    s = np.zeros((4, 12), np.int32)
    small = lvn.MeshOut(lvn.LVN_MEMORY_HOST, v.ctypes.data, 4, 0, t.ctypes.data, 4, 0, s.ctypes.data, 4, 0)
    rc = lvn.lib().lvn_generate_chunk_mesh_noalloc((C.c_int32 * 3)(0, 128, 0), 256, 64, C.byref(small), None)
    assert rc == lvn.LVN_ERR_CAPACITY and small.num_vertices > 4
