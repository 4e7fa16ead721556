"""Parity of the CUDA octree simplification (through the C ABI) with the
oracle's restatement: representatives, vertices and triangles bit for bit.

The simplification is not in the reference, so the oracle is the only
authority here ("parity unpinned" against the reference); its own arithmetic
is checked in float64 by test_oracle_simplify.py.
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O
from leven_gb300 import workloads as W
from test_gpu_parity import density_args, oracle_density

pytestmark = pytest.mark.gpu


def compare_simplified(lvn, g, chunk, verts, tris, seams, ref):
    reps = g.debug_fetch(lvn.DEBUG_SIMP_REPS, chunk, np.int32)
    assert np.array_equal(reps, ref.simp_reps()), "representatives"
    nv = ref.simp_vertex_count()
    assert verts.shape[0] == nv, "simplified vertex count"
    assert np.array_equal(verts.view(np.int32), ref.simp_vertices()[:nv].view(np.int32)), "simplified vertices"
    assert np.array_equal(tris, ref.simp_triangles()), "simplified triangles"
    assert np.array_equal(seams, ref.seams()), "seams are unchanged by simplification"


@pytest.mark.parametrize("mode,mn,vpc", [(1, (0, 128, 0), 64), (2, (0, 0, 0), 64), (2, (128, 0, 256), 32),
                                         (1, (0, 0, 0), 16)])
@pytest.mark.parametrize("thr", [0.0, 0.05, 1.0, 1e9])
def test_simplify_chunk(lvn_gpu, mode, mn, vpc, thr):
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    lvn.set_density(**density_args(mode))
    g = lvn.MeshGen(vpc)
    try:
        g.set_option(lvn.LVN_OPT_CACHE, 0)
        g.set_simplify(thr)
        m = g.generate_chunk_mesh(mn, 4 * vpc)
        O.set_seed(1)
        ref = O.OracleChunk(oracle_density(mode), mn, 4 * vpc, vpc=vpc).simplify(thr)
        assert ref.count(O.ORC_NODE_CODES) > 0
        compare_simplified(lvn, g, 0, m.vertices, m.triangles, m.seams, ref)
    finally:
        g.close()


def test_simplify_clipmap_batch(lvn_gpu):
    """48 chunks of the LOD 0-4 clipmap caves workload (nearest first, then
    the coarsest) in one batch at the 0.05 threshold."""
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    lvn.set_density(**W.CAVES)
    wl = W.clipmap_caves()
    chunks = wl.chunks[:32] + sorted(wl.chunks, key=lambda c: -c[1])[:16]
    g = lvn.MeshGen(64)
    try:
        g.set_simplify(0.05)
        V, T, S, res = g.generate_chunks(chunks)
        O.set_seed(1)
        checked = 0
        for c, (mn, size) in enumerate(chunks):
            ref = O.OracleChunk(oracle_density(2), mn, size, vpc=64)
            r = res[c]
            assert r[7] == ref.count(O.ORC_NODE_CODES)
            if r[7] == 0:
                continue
            ref.simplify(0.05)
            compare_simplified(lvn, g, c, V[r[0]:r[0] + r[1]], T[r[2]:r[2] + r[3]], S[r[4]:r[4] + r[5]], ref)
            checked += 1
        assert checked > 20
    finally:
        g.close()


def test_simplify_csg_batch(lvn_gpu):
    """Tiled chunks with seeded CSG operations, simplified at threshold 1."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    wl = W.tiled_csg(2, 2, 2, n_ops=16, seed=3)
    lvn.clear_csg_operations()
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions))
    g = lvn.MeshGen(64)
    try:
        g.set_simplify(1.0)
        V, T, S, res = g.generate_chunks(wl.chunks)
        O.set_seed(1)
        for c, (mn, size) in enumerate(wl.chunks):
            ops = [op.as_tuple() for op in W.ops_for_chunk(wl.ops, mn, size)]
            ref = O.OracleChunk(oracle_density(1), mn, size, vpc=64, ops=ops)
            r = res[c]
            if r[7] == 0:
                continue
            ref.simplify(1.0)
            compare_simplified(lvn, g, c, V[r[0]:r[0] + r[1]], T[r[2]:r[2] + r[3]], S[r[4]:r[4] + r[5]], ref)
    finally:
        lvn.clear_csg_operations()
        g.close()


def test_simplify_off_and_outputs(lvn_gpu):
    """Turning simplification off restores the plain mesh; pinned host and
    device outputs equal the pageable result; the cached path simplifies too."""
    torch = pytest.importorskip("torch")
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    lvn.set_density(**W.FBM2D)
    chunks = [((256 * i, 0, 256 * j), 256) for i in range(3) for j in range(2)]
    g = lvn.MeshGen(64)
    try:
        V0, T0, S0, _ = g.generate_chunks(chunks)
        g.set_simplify(0.5)
        V1, T1, S1, res = g.generate_chunks(chunks)
        assert V1.shape[0] < V0.shape[0] and T1.shape[0] < T0.shape[0]
        assert np.array_equal(S1, S0)
        n = len(chunks)
        descs = (lvn.ChunkDesc * n)(*[lvn.ChunkDesc((C.c_int32 * 3)(*mn), s) for mn, s in chunks])
        results = (lvn.ChunkResult * n)()
        hv = torch.zeros(V1.size, dtype=torch.float32).pin_memory()
        ht = torch.zeros(T1.size, dtype=torch.int32).pin_memory()
        hs = torch.zeros(S1.size, dtype=torch.int32).pin_memory()
        bo = lvn.BatchOut(lvn.LVN_MEMORY_HOST, hv.data_ptr(), V1.shape[0], 0, ht.data_ptr(), T1.shape[0], 0,
                          hs.data_ptr(), S1.shape[0], 0, C.cast(results, C.POINTER(lvn.ChunkResult)))
        assert g.generate_chunks_raw(descs, n, bo) == 0
        assert np.array_equal(hv.numpy().reshape(-1, 12).view(np.int32), V1.view(np.int32))
        assert np.array_equal(ht.numpy().reshape(-1, 3), T1)
        assert np.array_equal(hs.numpy().reshape(-1, 12), S1)
        dv = torch.zeros(V1.size, dtype=torch.float32, device="cuda")
        dt = torch.zeros(T1.size, dtype=torch.int32, device="cuda")
        ds = torch.zeros(S1.size, dtype=torch.int32, device="cuda")
        bd = lvn.BatchOut(lvn.LVN_MEMORY_DEVICE, dv.data_ptr(), V1.shape[0], 0, dt.data_ptr(), T1.shape[0], 0,
                          ds.data_ptr(), S1.shape[0], 0, C.cast(results, C.POINTER(lvn.ChunkResult)))
        assert g.generate_chunks_raw(descs, n, bd) == 0
        torch.cuda.synchronize()
        assert np.array_equal(dv.cpu().numpy().reshape(-1, 12).view(np.int32), V1.view(np.int32))
        assert np.array_equal(dt.cpu().numpy().reshape(-1, 3), T1)
        # the cached single-chunk path gives each chunk's slice of the batch
        for c, (mn, size) in enumerate(chunks):
            m = g.generate_chunk_mesh(mn, size)
            r = res[c]
            assert np.array_equal(m.vertices.view(np.int32), V1[r[0]:r[0] + r[1]].view(np.int32))
            assert np.array_equal(m.triangles, T1[r[2]:r[2] + r[3]])
        g.set_simplify(-1.0)
        V2, T2, S2, _ = g.generate_chunks(chunks)
        assert np.array_equal(V2.view(np.int32), V0.view(np.int32))
        assert np.array_equal(T2, T0) and np.array_equal(S2, S0)
    finally:
        g.close()


def test_autotune_keeps_results(lvn_gpu):
    """The launch-shape autotuner picks a persistent grid per stage; batches
    run with the tuned shapes give the same meshes."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    wl = W.tiled_csg(2, 2, 2, n_ops=8, seed=11)
    lvn.clear_csg_operations()
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions))
    g = lvn.MeshGen(64)
    try:
        V0, T0, S0, _ = g.generate_chunks(wl.chunks)
        chosen = g.autotune(wl.chunks)
        assert set(chosen) >= {"hermite", "leaf", "mesh_count"}
        assert all(v in (2, 4, 8, 16, 32) for v in chosen.values())
        V1, T1, S1, _ = g.generate_chunks(wl.chunks)
        assert np.array_equal(V1.view(np.int32), V0.view(np.int32))
        assert np.array_equal(T1, T0) and np.array_equal(S1, S0)
    finally:
        lvn.clear_csg_operations()
        g.close()
