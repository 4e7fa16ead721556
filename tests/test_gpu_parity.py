"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Bar: bit-exact for every integer / topology output (materials, edge keys
and their order, leaf codes, edge masks, dominant materials, triangle
indices, seam nodes' integer fields, cuckoo key->value contents); vertex
positions and normals within 1e-4 voxel (the kernels in fact reproduce the
oracle's floating-point sequence bit for bit, which these tests also check
where it holds by construction).
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O
from leven_gb300 import workloads as W

pytestmark = pytest.mark.gpu

AIR = 201


def density_args(mode):
    return W.FBM2D if mode == 1 else W.CAVES if mode == 2 else dict(mode=0)


def oracle_density(mode):
    d = density_args(mode)
    return O.density(**{k: v for k, v in d.items() if k != "lacunarity2" and k != "lacunarity3"},
                     lac2=d.get("lacunarity2", 2.0), lac3=d.get("lacunarity3", 2.0))


def surface_min(mode, vpc):
    # chunks that intersect each density's surface
    if mode == 0:
        return (0, 2368, 0) if vpc == 16 else (0, 2304, 0)
    return (0, 128, 0)


def compare_stages(lvn, mg, chunk, ref, vpc, scale, created_as_set=False):
    mats = mg.debug_fetch(lvn.DEBUG_MATERIALS, chunk, np.uint8)
    assert np.array_equal(mats, ref.materials().astype(np.uint8)), "field materials"
    keys = mg.debug_fetch(lvn.DEBUG_EDGE_KEYS, chunk, np.int32)
    info = mg.debug_fetch(lvn.DEBUG_EDGE_INFO, chunk, np.float32, 4)
    rkeys, rinfo = ref.edge_keys(), ref.edge_info()
    assert keys.size == rkeys.size, "edge count"
    if created_as_set:
        # the reference orders CSG-created edges by a racy hash-based dedupe
        # (duplicate.cl:40-51): kept edges in order, created edges as a set
        ncreated = ref.count(O.ORC_CREATED_EDGE_KEYS)
        nk = keys.size - ncreated
        assert np.array_equal(keys[:nk], rkeys[:nk]), "kept edge order"
        assert set(keys[nk:].tolist()) == set(rkeys[nk:].tolist()), "created edge set"
        order = np.argsort(keys)
        rorder = np.argsort(rkeys)
        assert np.array_equal(keys[order], rkeys[rorder])
        assert np.array_equal(info[order].view(np.int32), rinfo[rorder].view(np.int32)), "edge hermite data"
    else:
        assert np.array_equal(keys, rkeys), "edge keys / compaction order"
        assert np.array_equal(info.view(np.int32), rinfo.view(np.int32)), "edge hermite data"
    codes = mg.debug_fetch(lvn.DEBUG_NODE_CODES, chunk, np.uint32)
    assert np.array_equal(codes, ref.node_codes()), "leaf codes / order"
    ninfo = mg.debug_fetch(lvn.DEBUG_NODE_INFO, chunk, np.int32)
    assert np.array_equal(ninfo, (ref.node_edges() << 16) | ref.node_materials()), "edge masks / materials"


def compare_mesh(vertices, triangles, seams, ref, scale):
    nv = ref.mesh_vertex_count()
    assert vertices.shape[0] == nv
    rv = ref.vertices()[:nv]
    tol = 1e-4 * 4 * scale  # 1e-4 voxel in world units
    if nv:
        assert np.abs(vertices[:, :3] - rv[:, :3]).max() <= tol, "vertex positions"
        assert np.abs(vertices[:, 4:7] - rv[:, 4:7]).max() <= 1e-4, "vertex normals"
        assert np.array_equal(vertices[:, 8:], rv[:, 8:]), "vertex colour / material"
    assert np.array_equal(triangles, ref.triangles()), "triangle indices"
    rs = ref.seams()
    assert seams.shape == rs.shape, "seam count"
    if rs.size:
        assert np.array_equal(seams[:, :4], rs[:, :4]), "seam localspaceMin + material"
        assert np.abs(seams[:, 4:].view(np.float32) - rs[:, 4:].view(np.float32)).max() <= tol


@pytest.fixture
def mg(lvn_gpu):
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    g = lvn.MeshGen(64)
    g.set_option(lvn.LVN_OPT_CACHE, 0)
    yield g
    g.close()


@pytest.mark.parametrize("mode", [1, 0, 2])
@pytest.mark.parametrize("vpc", [16, 32, 64])
@pytest.mark.parametrize("crossing", [0, 1])
def test_single_chunk(lvn_gpu, mode, vpc, crossing):
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    lvn.set_density(**density_args(mode))
    g = lvn.MeshGen(vpc)
    try:
        g.set_option(lvn.LVN_OPT_CACHE, 0)
        g.set_option(lvn.LVN_OPT_CROSSING_MODE, crossing)
        mn, size = surface_min(mode, vpc), 4 * vpc
        mesh = g.generate_chunk_mesh(mn, size)
        O.set_seed(1)
        ref = O.OracleChunk(oracle_density(mode), mn, size, vpc=vpc, crossing_mode=crossing)
        assert ref.count(O.ORC_EDGE_KEYS) > 0
        compare_stages(lvn, g, 0, ref, vpc, 1)
        compare_mesh(mesh.vertices, mesh.triangles, mesh.seams, ref, 1)
        # the kernels reproduce the oracle's arithmetic exactly
        assert np.array_equal(mesh.vertices.view(np.int32), ref.vertices()[:ref.mesh_vertex_count()].view(np.int32))
    finally:
        g.close()


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("mn,size", [((-512, 0, 768), 256), ((-1024, -256, -2048), 1024)])
def test_negative_coordinates(lvn_gpu, mode, mn, size):
    """Chunks whose field starts at negative density-space coordinates (every
    index computation is signed)."""
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    lvn.set_density(**density_args(mode))
    g = lvn.MeshGen(64)
    try:
        g.set_option(lvn.LVN_OPT_CACHE, 0)
        mesh = g.generate_chunk_mesh(mn, size)
        O.set_seed(1)
        ref = O.OracleChunk(oracle_density(mode), mn, size, vpc=64)
        scale = size // 256
        if ref.count(O.ORC_EDGE_KEYS):
            compare_stages(lvn, g, 0, ref, 64, scale)
        compare_mesh(mesh.vertices, mesh.triangles, mesh.seams, ref, scale)
    finally:
        g.close()


def table_entries(table):
    t = table[table != np.uint64(0xFFFFFFFFFFFFFFFF)]
    return set(zip((t & np.uint64(0xFFFFFFFF)).astype(np.int64).tolist(), (t >> np.uint64(32)).astype(np.int64).tolist()))


def test_hash_contents(lvn_gpu, mg):
    """Cuckoo tables hold exactly {(key, index)} for the edge and leaf key sets
    (cuckoo.cl:26-71); lookups are exercised by the mesh parity tests."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    mg.generate_chunk_mesh((0, 128, 0), 256)
    keys = mg.debug_fetch(lvn.DEBUG_EDGE_KEYS, 0, np.int32)
    codes = mg.debug_fetch(lvn.DEBUG_NODE_CODES, 0, np.uint32)
    et = mg.debug_fetch(lvn.DEBUG_EDGE_TABLE, 0, np.uint64)
    es = mg.debug_fetch(lvn.DEBUG_EDGE_STASH, 0, np.uint64)
    nt = mg.debug_fetch(lvn.DEBUG_NODE_TABLE, 0, np.uint64)
    ns = mg.debug_fetch(lvn.DEBUG_NODE_STASH, 0, np.uint64)
    assert et.size == O.find_next_prime(max(2048, 2 * keys.size))
    assert nt.size == O.find_next_prime(max(2048, 2 * codes.size))
    assert es.size == 101 and ns.size == 101
    assert table_entries(np.concatenate([et, es])) == set(zip(keys.tolist(), range(keys.size)))
    assert table_entries(np.concatenate([nt, ns])) == set(zip(codes.astype(np.int64).tolist(), range(codes.size)))


def run_batch_vs_oracle(lvn, g, wl, sample=None):
    lvn.clear_csg_operations()
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions,
                                            op.rotate_y))
    V, T, S, res = g.generate_chunks(wl.chunks)
    O.set_seed(wl.noise_seed)
    idx = range(len(wl.chunks)) if sample is None else sample
    checked = 0
    for c in idx:
        mn, size = wl.chunks[c]
        ops = [op.as_tuple() for op in W.ops_for_chunk(wl.ops, mn, size)]
        ref = O.OracleChunk(oracle_density(wl.density["mode"]), mn, size, vpc=g.voxels_per_chunk, ops=ops)
        r = res[c]
        assert r[6] == ref.count(O.ORC_EDGE_KEYS) and r[7] == ref.count(O.ORC_NODE_CODES)
        if r[6]:
            compare_stages(lvn, g, c, ref, g.voxels_per_chunk, size // (4 * g.voxels_per_chunk),
                           created_as_set=len(ops) > 0)
        verts = V[r[0]:r[0] + r[1]]
        tris = T[r[2]:r[2] + r[3]]
        seams = S[r[4]:r[4] + r[5]]
        compare_mesh(verts, tris, seams, ref, size // (4 * g.voxels_per_chunk))
        checked += 1
    lvn.clear_csg_operations()
    return res, checked


def test_csg_batch(lvn_gpu, mg):
    """4 x 2 x 4 LOD0 chunks, 24 seeded CSG operations: every chunk matches
    the oracle (edge lists after CSG compared as kept-in-order + created set)."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    wl = W.tiled_csg(4, 2, 4, n_ops=24, seed=7)
    res, checked = run_batch_vs_oracle(lvn, mg, wl)
    assert checked == 32
    assert res[:, 3].sum() > 0


def test_tiled_csg_128_sampled(lvn_gpu, mg):
    """The full 128-chunk, 32-operation tiled workload; 12 chunks (those with
    the most operations first) are checked stage by stage against the oracle,
    the rest through size-independent properties."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    wl = W.tiled_csg()
    nops = [len(W.ops_for_chunk(wl.ops, mn, s)) for mn, s in wl.chunks]
    sample = sorted(range(len(wl.chunks)), key=lambda c: -nops[c])[:12]
    res, checked = run_batch_vs_oracle(lvn, mg, wl, sample)
    assert checked == 12
    # properties over every chunk: triangle indices address the chunk's vertices
    V, T, S, res = mg.generate_chunks(wl.chunks)
    for r in res:
        tris = T[r[2]:r[2] + r[3]]
        if tris.size:
            assert tris.min() >= 0 and tris.max() < r[1]
    assert np.isfinite(V[:, :8]).all()


def test_batch_equals_single(lvn_gpu, mg):
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    chunks = [((256 * i, 0, 0), 256) for i in range(3)] + [((0, 0, 512), 512), ((0, 4096, 0), 256)]
    V, T, S, res = mg.generate_chunks(chunks)
    for c, (mn, size) in enumerate(chunks):
        m = mg.generate_chunk_mesh(mn, size)
        r = res[c]
        assert np.array_equal(m.vertices.view(np.int32), V[r[0]:r[0] + r[1]].view(np.int32))
        assert np.array_equal(m.triangles, T[r[2]:r[2] + r[3]])
        assert np.array_equal(m.seams, S[r[4]:r[4] + r[5]])


def test_lod_chunk(lvn_gpu, mg):
    """A LOD2 chunk (sampleScale 4) matches the oracle."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    mn, size = (1024, -512, 0), 1024
    m = mg.generate_chunk_mesh(mn, size)
    O.set_seed(1)
    ref = O.OracleChunk(oracle_density(1), mn, size, vpc=64)
    assert ref.count(O.ORC_EDGE_KEYS) > 0
    compare_stages(lvn_gpu, mg, 0, ref, 64, 4)
    compare_mesh(m.vertices, m.triangles, m.seams, ref, 4)


def test_cave_field_band(lvn_gpu, mg):
    """The caves density over chunks from deep underground to open air, LOD0
    and LOD2.  The field kernel takes a point's material from y - amp2 h
    alone where the cave term cannot change its sign, and evaluates the cave
    fBm only inside that band.  Every chunk matches the oracle, and the batch
    holds chunks wholly below and wholly above the band."""
    lvn = lvn_gpu
    lvn.set_density(**W.CAVES)
    chunks = [((256 * (k % 3), y, 256 * k), 256) for k, y in enumerate((-768, -512, -256, 0, 256, 512))]
    chunks += [((1024 * k, y, 0), 1024) for k, y in enumerate((-2048, -1024, 0))]
    V, T, S, res = mg.generate_chunks(chunks)
    O.set_seed(1)
    solid = air = 0
    for c, (mn, size) in enumerate(chunks):
        ref = O.OracleChunk(oracle_density(2), mn, size, vpc=64)
        scale = size // 256
        compare_stages(lvn, mg, c, ref, 64, scale)
        r = res[c]
        compare_mesh(V[r[0]:r[0] + r[1]], T[r[2]:r[2] + r[3]], S[r[4]:r[4] + r[5]], ref, scale)
        mats = ref.materials()
        solid += bool((mats != AIR).all())
        air += bool((mats == AIR).all())
    assert solid >= 1 and air >= 1, (solid, air)


@pytest.mark.parametrize("amp3", [0.0, -12.0, 300.0])
def test_cave_field_band_edges(lvn_gpu, mg, amp3):
    """The field kernel's band rows at their limits: no cave term (a band of
    width 0, only points with y - amp2 h == 0 evaluated), a negative cave
    amplitude (the band uses |amp3|), and a band wider than the chunks (every
    row of every column evaluated).  Materials and meshes match the oracle."""
    lvn = lvn_gpu
    dens = dict(W.CAVES, amp3=amp3)
    lvn.set_density(**dens)
    chunks = [((0, -256, 0), 256), ((256, 0, 0), 256), ((0, -1024, 1024), 1024)]
    V, T, S, res = mg.generate_chunks(chunks)
    O.set_seed(1)
    od = O.density(**{k: v for k, v in dens.items() if k not in ("lacunarity2", "lacunarity3")},
                   lac2=dens["lacunarity2"], lac3=dens["lacunarity3"])
    for c, (mn, size) in enumerate(chunks):
        ref = O.OracleChunk(od, mn, size, vpc=64)
        scale = size // 256
        compare_stages(lvn, mg, c, ref, 64, scale)
        r = res[c]
        compare_mesh(V[r[0]:r[0] + r[1]], T[r[2]:r[2] + r[3]], S[r[4]:r[4] + r[5]], ref, scale)
    lvn.set_density(**W.CAVES)


def test_empty_chunks(lvn_gpu, mg):
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    for mn in ((0, 40960, 0), (0, -40960, 0)):
        m = mg.generate_chunk_mesh(mn, 256)
        assert m.vertices.shape[0] == 0 and m.triangles.shape[0] == 0 and m.seams.shape[0] == 0
        assert mg.is_chunk_empty(mn, 256)
    assert not mg.is_chunk_empty((0, 128, 0), 256)


def test_determinism(lvn_gpu, mg):
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    wl = W.tiled_csg(3, 2, 3, n_ops=16, seed=3)
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions))
    a = mg.generate_chunks(wl.chunks)
    b = mg.generate_chunks(wl.chunks)
    lvn.clear_csg_operations()
    for x, y in zip(a, b):
        assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))


def test_capacity_error(lvn_gpu, mg):
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    v = np.zeros((4, 12), np.float32)
    t = np.zeros((4, 3), np.int32)
    s = np.zeros((4, 12), np.int32)
    out = lvn.MeshOut(lvn.LVN_MEMORY_HOST, v.ctypes.data, 4, 0, t.ctypes.data, 4, 0, s.ctypes.data, 4, 0)
    mn = (C.c_int32 * 3)(0, 128, 0)
    rc = lvn.lib().lvn_meshgen_generate_chunk_mesh(mg.handle, mn, 256, C.byref(out))
    assert rc == lvn.LVN_ERR_CAPACITY
    O.set_seed(1)
    ref = O.OracleChunk(oracle_density(1), (0, 128, 0), 256, vpc=64)
    assert out.num_vertices == ref.mesh_vertex_count() and out.num_triangles == ref.count(O.ORC_TRIANGLES)


def test_invalid_arguments(lvn_gpu, mg):
    lvn = lvn_gpu
    mn = (C.c_int32 * 3)(0, 0, 0)
    out = lvn.MeshOut()
    assert lvn.lib().lvn_meshgen_generate_chunk_mesh(mg.handle, mn, 100, C.byref(out)) == -30
    bad = lvn.make_op(3, 0, 1, (0, 0, 0), (1, 1, 1))
    assert lvn.lib().lvn_meshgen_apply_csg_operations(mg.handle, C.byref(bad), 1, mn, 256) == -30
    assert lvn.lib().lvn_meshgen_create(12) is None


def test_cached_apply_then_generate(lvn_gpu):
    """applyCSGOperations on a cached field, then generateChunkMesh
    (compute_csg.cpp:224-242, compute_octree.cpp:351-375) equals the oracle
    applying the same operations as one batch."""
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    lvn.set_density(**W.FBM2D)
    g = lvn.MeshGen(32)
    try:
        mn, size = (0, 128, 0), 128
        ops = [W.Op(1, 1, AIR, (10.0, 38.0, 12.0), (6.0, 6.0, 6.0)), W.Op(0, 0, 1, (20.0, 44.0, 20.0), (4.0, 3.0, 5.0))]
        g.apply_csg_operations([lvn.make_op(o.type, o.brush_shape, o.material, o.origin, o.dimensions) for o in ops],
                               mn, size)
        m = g.generate_chunk_mesh(mn, size)
        O.set_seed(1)
        ref = O.OracleChunk(oracle_density(1), mn, size, vpc=32, ops=[o.as_tuple() for o in ops])
        assert ref.count(O.ORC_CREATED_EDGE_KEYS) > 0
        compare_mesh(m.vertices, m.triangles, m.seams, ref, 1)
        # cache hit: the same mesh again without recomputation
        m2 = g.generate_chunk_mesh(mn, size)
        assert np.array_equal(m.vertices.view(np.int32), m2.vertices.view(np.int32))
    finally:
        g.close()


def test_stored_ops_replayed_on_load(lvn_gpu):
    """LoadDensityField replays stored operations overlapping a fresh field
    (compute_density_field.cpp:255-271); the cached and uncached paths agree."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    wl = W.tiled_csg(2, 2, 2, n_ops=10, seed=11)
    lvn.clear_csg_operations()
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions))
    cached, cold = lvn.MeshGen(64), lvn.MeshGen(64)
    try:
        cold.set_option(lvn.LVN_OPT_CACHE, 0)
        for mn, size in wl.chunks:
            a = cached.generate_chunk_mesh(mn, size)
            b = cold.generate_chunk_mesh(mn, size)
            assert np.array_equal(a.vertices.view(np.int32), b.vertices.view(np.int32))
            assert np.array_equal(a.triangles, b.triangles)
            assert np.array_equal(a.seams, b.seams)
    finally:
        cached.close()
        cold.close()
        lvn.clear_csg_operations()


def test_two_csg_batches_on_cached_field(lvn_gpu):
    """Two applyCSGOperations calls on one cached field: materials, edge-key
    set and triangles equal a single batch of both (hermite data of edges
    touched only by the first batch keeps that batch's brush crossing, as
    in the reference)."""
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    lvn.set_density(**W.FBM2D)
    g = lvn.MeshGen(32)
    try:
        mn, size = (0, 128, 0), 128
        a = W.Op(1, 1, AIR, (8.0, 38.0, 8.0), (5.0, 5.0, 5.0))
        b = W.Op(0, 0, 1, (24.0, 40.0, 22.0), (3.0, 4.0, 3.0))
        g.apply_csg_operations([lvn.make_op(a.type, a.brush_shape, a.material, a.origin, a.dimensions)], mn, size)
        g.apply_csg_operations([lvn.make_op(b.type, b.brush_shape, b.material, b.origin, b.dimensions)], mn, size)
        m = g.generate_chunk_mesh(mn, size)
        O.set_seed(1)
        ref = O.OracleChunk(oracle_density(1), mn, size, vpc=32, ops=[a.as_tuple(), b.as_tuple()])
        keys = g.debug_fetch(lvn.DEBUG_EDGE_KEYS, 0, np.int32)
        assert set(keys.tolist()) == set(ref.edge_keys().tolist())
        assert np.array_equal(m.triangles, ref.triangles())
        assert m.vertices.shape[0] == ref.mesh_vertex_count()
    finally:
        g.close()


def test_pinned_host_outputs(lvn_gpu, mg):
    """Pinned host arrays are written by export kernels over the C2C link; the
    result equals the pageable path byte for byte, and an array that is too
    small is reported as a capacity error."""
    torch = pytest.importorskip("torch")
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    wl = W.tiled_csg(2, 2, 2, n_ops=8, seed=5)
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions))
    V, T, S, res = mg.generate_chunks(wl.chunks)      # pageable numpy arrays
    n = len(wl.chunks)
    descs = (lvn.ChunkDesc * n)(*[lvn.ChunkDesc((C.c_int32 * 3)(*mn), s) for mn, s in wl.chunks])
    results = (lvn.ChunkResult * n)()
    cap_v, cap_t, cap_s = V.shape[0] + 7, T.shape[0] + 5, S.shape[0] + 3
    hv = torch.zeros(cap_v * 12, dtype=torch.float32).pin_memory()
    ht = torch.zeros(cap_t * 3, dtype=torch.int32).pin_memory()
    hs = torch.zeros(cap_s * 12, dtype=torch.int32).pin_memory()
    bo = lvn.BatchOut(lvn.LVN_MEMORY_HOST, hv.data_ptr(), cap_v, 0, ht.data_ptr(), cap_t, 0, hs.data_ptr(), cap_s, 0,
                      C.cast(results, C.POINTER(lvn.ChunkResult)))
    assert mg.generate_chunks_raw(descs, n, bo) == 0
    assert (bo.total_vertices, bo.total_triangles, bo.total_seams) == (V.shape[0], T.shape[0], S.shape[0])
    assert np.array_equal(hv.numpy().reshape(-1, 12)[:V.shape[0]].view(np.int32), V.view(np.int32))
    assert np.array_equal(ht.numpy().reshape(-1, 3)[:T.shape[0]], T)
    assert np.array_equal(hs.numpy().reshape(-1, 12)[:S.shape[0]], S)
    # an array too small is flagged and left unwritten past its capacity
    # (sentinels fill the host arrays beyond the capacity each call is given)
    sentinel = -0x5A5A5A5B
    ht.fill_(sentinel)
    small = lvn.BatchOut(lvn.LVN_MEMORY_HOST, hv.data_ptr(), cap_v, 0, ht.data_ptr(), 10, 0, hs.data_ptr(), cap_s, 0,
                         C.cast(results, C.POINTER(lvn.ChunkResult)))
    assert mg.generate_chunks_raw(descs, n, small) == lvn.LVN_ERR_CAPACITY
    assert small.total_triangles == T.shape[0]
    assert (ht.numpy()[3 * 10:] == sentinel).all(), "triangles written past the capacity"
    # a vertex array too small: the leaves, which write it themselves, flag it
    hv.view(torch.int32).fill_(sentinel)
    small_v = lvn.BatchOut(lvn.LVN_MEMORY_HOST, hv.data_ptr(), V.shape[0] - 1, 0, ht.data_ptr(), cap_t, 0,
                           hs.data_ptr(), cap_s, 0, C.cast(results, C.POINTER(lvn.ChunkResult)))
    assert mg.generate_chunks_raw(descs, n, small_v) == lvn.LVN_ERR_CAPACITY
    assert (hv.view(torch.int32).numpy()[12 * (V.shape[0] - 1):] == sentinel).all(), "vertices written past the capacity"
    # a vertex array that is not 16-byte aligned takes the sliced export path
    hv.zero_()
    odd = lvn.BatchOut(lvn.LVN_MEMORY_HOST, hv.data_ptr() + 4, cap_v - 1, 0, ht.data_ptr(), cap_t, 0,
                       hs.data_ptr(), cap_s, 0, C.cast(results, C.POINTER(lvn.ChunkResult)))
    assert mg.generate_chunks_raw(descs, n, odd) == 0
    got = hv.numpy()[1:1 + 12 * V.shape[0]].reshape(-1, 12)
    assert np.array_equal(got.view(np.int32), V.view(np.int32))
    # the same for the seams, which the seam pass writes itself when aligned
    hs.fill_(sentinel)
    small_s = lvn.BatchOut(lvn.LVN_MEMORY_HOST, hv.data_ptr(), cap_v, 0, ht.data_ptr(), cap_t, 0, hs.data_ptr(),
                           S.shape[0] - 1, 0, C.cast(results, C.POINTER(lvn.ChunkResult)))
    assert mg.generate_chunks_raw(descs, n, small_s) == lvn.LVN_ERR_CAPACITY
    assert (hs.numpy()[12 * (S.shape[0] - 1):] == sentinel).all(), "seams written past the capacity"
    hs.zero_()
    odd_s = lvn.BatchOut(lvn.LVN_MEMORY_HOST, hv.data_ptr(), cap_v, 0, ht.data_ptr(), cap_t, 0, hs.data_ptr() + 4,
                         cap_s - 1, 0, C.cast(results, C.POINTER(lvn.ChunkResult)))
    assert mg.generate_chunks_raw(descs, n, odd_s) == 0
    assert np.array_equal(hs.numpy()[1:1 + 12 * S.shape[0]].reshape(-1, 12), S)
    lvn.clear_csg_operations()


def test_graph_and_stream_paths_agree(lvn_gpu):
    """A batch replayed from its captured CUDA graph equals the same batch
    enqueued kernel by kernel, and a re-capture follows a change of shape."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    wl = W.tiled_csg(3, 2, 3, n_ops=12, seed=9)
    lvn.clear_csg_operations()
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions))
    a, b = lvn.MeshGen(64), lvn.MeshGen(64)
    try:
        b.set_option(lvn.LVN_OPT_GRAPHS, 0)
        for chunks in (wl.chunks, wl.chunks[:7], wl.chunks):
            ra = a.generate_chunks(chunks)
            rb = b.generate_chunks(chunks)
            for x, y in zip(ra, rb):
                assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))
    finally:
        a.close()
        b.close()
        lvn.clear_csg_operations()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_hermite_forms_agree(lvn_gpu, mode):
    """LVN_OPT_HERMITE_FORM: the hermite kernel with its noise lookup tables in
    shared memory (the form large batches take by default) and the one
    reading them from global memory give the same bits on the same batch, and
    the shared-memory form matches the oracle on chunks with CSG operations."""
    lvn = lvn_gpu
    lvn.set_density(**density_args(mode))
    lvn.clear_csg_operations()
    sx, sy, sz = surface_min(mode, 64)
    chunks = [((sx + 256 * i, sy, sz + 256 * k), 256) for i in range(3) for k in range(2)]
    chunks.append(((sx, sy - 256, sz), 512))
    gens = [lvn.MeshGen(64) for _ in range(3)]
    try:
        outs = []
        for form, g in enumerate(gens):
            g.set_option(lvn.LVN_OPT_CACHE, 0)
            g.set_option(lvn.LVN_OPT_HERMITE_FORM, form)
            outs.append(g.generate_chunks(chunks))
        assert outs[0][3][:, 3].sum() > 0
        for other in outs[1:]:
            for x, y in zip(outs[0], other):
                assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))
        with pytest.raises(lvn.LvnError):
            gens[0].set_option(lvn.LVN_OPT_HERMITE_FORM, 3)
        if mode == 2:
            wl = W.tiled_csg(2, 2, 2, n_ops=8, seed=5)
            wl = W.Workload(wl.name, wl.chunks, wl.ops, W.CAVES)
            res, checked = run_batch_vs_oracle(lvn, gens[1], wl)
            assert checked == 8 and res[:, 3].sum() > 0
    finally:
        for g in gens:
            g.close()
        lvn.clear_csg_operations()
