"""The oracle pinned against the reference's own OpenCL code.

oracle/Makefile compiles the reference's leven/cl/simplex.cl, noise.cl (with
hg_sdf.glsl) and qef.cl as C++ on the host through oracle/ref_shim/cl_shim.h,
straight from the reference tree (its vector literals rewritten into
constructor calls in a git-ignored build copy), into oracle/_ref/libref.so.
These tests run that code and the oracle's restatement on the same inputs and
require identical bits: simplex noise in 2D and 3D, the reference's terrain
density (DensityFunc with Terrain, RidgedMultiFractal and BasicFractal), the
benchmark's fBm heightfield built from the reference's BasicFractal, and the
QEF solve (qef_create_from_points + qef_solve).

The reference built these with -cl-fast-relaxed-math, so its own bits are
one of several admissible results.  The harness compiles simplex.cl and
qef.cl without fusing multiply-adds outside dot(), and noise.cl with fusion
(a multiply whose one use is an add), which is the restatement's convention;
the match is therefore exact, and any misread of the algorithm (a constant,
a corner, a lookup, the sampler's wrap, a sweep) would show as a mismatch.

The permutation image itself (CreateNoisePermutationLookupImage) lives in host
code that needs an OpenCL runtime to compile; the harness is given the
oracle's image.  Without the reference tree the harness is absent and these
tests skip.
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O


@pytest.fixture(scope="module")
def ref():
    lib = O.ref_lib()
    if lib is None or not hasattr(lib, "ref_snoise2"):
        pytest.skip("reference harness not built (no reference tree here)")
    for f in ("ref_snoise2", "ref_snoise3", "ref_basic_fractal", "ref_ridged_multi_fractal", "ref_terrain",
              "ref_density_func", "ref_harness_density", "ref_qef_solve_points"):
        getattr(lib, f).restype = C.c_float
    lib.ref_set_perm_image.argtypes = [C.c_void_p]
    lib.ref_snoise2.argtypes = [C.c_float] * 2
    lib.ref_snoise3.argtypes = [C.c_float] * 3
    lib.ref_terrain.argtypes = [C.c_float] * 2
    lib.ref_density_func.argtypes = [C.c_float] * 3
    lib.ref_ridged_multi_fractal.argtypes = [C.c_int] + [C.c_float] * 5
    lib.ref_basic_fractal.argtypes = [C.c_int] + [C.c_float] * 5
    lib.ref_harness_density.argtypes = [C.c_int] + [C.c_float] * 3
    lib.ref_qef_solve_points.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    O.set_seed(1)
    image = O.perm_image_rgba()  # held while the harness copies it
    lib.ref_set_perm_image(image.ctypes.data)
    return lib


def points(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, (n, 3)).astype(np.float32)


def test_snoise2_bits(ref):
    L = O.lib()
    pts = points(20000, -3000.0, 3000.0, 1)
    pts[:2000] *= np.float32(1.0 / 256.0)  # the fBm's base-octave scale
    for p in pts:
        x, y = float(p[0]), float(p[1])
        a, b = np.float32(ref.ref_snoise2(x, y)), np.float32(L.orc_snoise2(x, y))
        assert a.view(np.int32) == b.view(np.int32), (x, y, a, b)


def test_snoise3_bits(ref):
    L = O.lib()
    pts = points(20000, -3000.0, 3000.0, 2)
    pts[:2000] *= np.float32(1.0 / 64.0)
    for p in pts:
        a, b = np.float32(ref.ref_snoise3(*map(float, p))), np.float32(L.orc_snoise3(*map(float, p)))
        assert a.view(np.int32) == b.view(np.int32), (p, a, b)


def test_reference_terrain_density_bits(ref):
    """DensityFunc (noise.cl:225-268): y - 900 Terrain(x, z), with the
    reference's RidgedMultiFractal and BasicFractal."""
    L = O.lib()
    dens = O.density(mode=0)
    for p in points(5000, -20000.0, 20000.0, 3):
        a = np.float32(ref.ref_density_func(*map(float, p)))
        b = np.float32(L.orc_density_at(C.byref(dens), *map(float, p)))
        assert a.view(np.int32) == b.view(np.int32), (p, a, b)


@pytest.mark.parametrize("mode", [1, 2])
def test_benchmark_density_bits(ref, mode):
    """The benchmark's heightfield, y - 48 BasicFractal(8, 1/256, 2, 0.5, xz)
    from the reference's BasicFractal (mode 1), plus 12 times a 6-octave 3D
    fBm at 1/64 over the reference's snoise3 (mode 2), against the oracle's
    density modes."""
    L = O.lib()
    dens = O.density(mode=mode)
    for p in points(5000, -4096.0, 4096.0, 4):
        p[1] *= np.float32(1.0 / 32.0)
        a = np.float32(ref.ref_harness_density(mode, *map(float, p)))
        b = np.float32(L.orc_density_at(C.byref(dens), *map(float, p)))
        assert a.view(np.int32) == b.view(np.int32), (p, a, b)


def test_qef_solve_bits(ref):
    """qef_create_from_points + qef_solve (qef.cl:239-303) on 1-12 random
    crossings with unit normals, as a leaf gathers them."""
    L = O.lib()
    L.orc_qef_solve_points.restype = C.c_float
    L.orc_qef_solve_points.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    rng = np.random.default_rng(5)
    for _ in range(20000):
        n = int(rng.integers(1, 13))
        pos = np.zeros((12, 4), np.float32)
        nor = np.zeros((12, 4), np.float32)
        pos[:n, :3] = rng.uniform(0.0, 1.0, (n, 3)) * rng.choice([1.0, 4.0, 32.0])
        v = rng.normal(size=(n, 3))
        nor[:n, :3] = v / np.linalg.norm(v, axis=1, keepdims=True)
        a = np.zeros(4, np.float32)
        b = np.zeros(4, np.float32)
        ref.ref_qef_solve_points(pos.ctypes.data, nor.ctypes.data, n, a.ctypes.data)
        L.orc_qef_solve_points(pos.ctypes.data, nor.ctypes.data, n, b.ctypes.data)
        assert np.array_equal(a[:3].view(np.int32), b[:3].view(np.int32)), (n, a, b)


def ref_chunk(ref, mode, mn, size, colour, ops=()):
    ref.ref_mesh_chunk.argtypes = [C.c_int32 * 3, C.c_int32, C.c_int32, C.c_uint32, C.c_float * 3, C.c_void_p,
                                   C.c_int32] + [C.c_void_p] * 3 + [C.c_int64] + [C.c_void_p] * 3 + \
        [C.c_int64, C.c_int32 * 6]
    op_array = O.make_ops(list(ops))
    F = 66 ** 3
    ecap, ncap = 3 * 65 ** 3, 64 ** 3
    mats = np.zeros(F, np.int32)
    keys = np.zeros(ecap, np.int32)
    info = np.zeros((ecap, 4), np.float32)
    verts = np.zeros((ncap, 12), np.float32)
    tris = np.zeros(18 * ncap, np.int32)
    seams = np.zeros((ncap, 12), np.int32)
    counts = (C.c_int32 * 6)()
    rc = ref.ref_mesh_chunk((C.c_int32 * 3)(*mn), size, mode, 5489, (C.c_float * 3)(*colour),
                            C.cast(op_array, C.c_void_p), len(ops), mats.ctypes.data,
                            keys.ctypes.data, info.ctypes.data, ecap, verts.ctypes.data, tris.ctypes.data,
                            seams.ctypes.data, ncap, counts)
    assert rc == 0
    E, V, T, S, stash, past = counts
    return dict(materials=mats, keys=keys[:E], info=info[:E], vertices=verts[:V], triangles=tris[:T].reshape(-1, 3),
                seams=seams[:S], stash=stash, past=past)


@pytest.mark.parametrize("mode,mn,size", [(1, (0, 128, 0), 256), (1, (-512, 0, 768), 256), (2, (0, 0, 0), 256),
                                          (2, (1024, -1024, 0), 1024), (0, (0, 2304, 0), 256),
                                          (1, (-2048, -2048, 4096), 4096)])
def test_whole_chunk_through_the_reference_kernels(ref, mode, mn, size):
    """A chunk meshed by the reference's own kernels (GenerateDefaultField,
    FindFieldEdges, FindEdgeIntersectionInfo, FindActiveVoxels,
    Cuckoo_InsertKeys, CreateLeafNodes, SolveQEFs, GenerateMesh,
    GenerateMeshVertexBuffer, FindSeamNodes, ExtractSeamNodeInfo; the scans and
    compactions sequential) equals the oracle's chunk bit for bit: materials,
    edge keys and order, hermite data, vertices, triangles, seams.  Mode 0 is
    the reference's DensityFunc; modes 1 and 2 are the benchmark's densities in
    its place."""
    O.set_seed(1)
    image = O.perm_image_rgba()
    ref.ref_set_perm_image(image.ctypes.data)
    och = O.OracleChunk(O.density(mode=mode), mn, size, vpc=64)
    colour = och.vertices()[0, 8:11] if och.count(O.ORC_NODE_CODES) else np.zeros(3, np.float32)
    got = ref_chunk(ref, mode, mn, size, [float(c) for c in colour])
    assert np.array_equal(got["materials"], och.materials()), "field materials"
    assert np.array_equal(got["keys"], och.edge_keys()), "edge keys / compaction order"
    assert np.array_equal(got["info"].view(np.int32), och.edge_info().view(np.int32)), "hermite data"
    assert got["stash"] == 0 and got["past"] == 0  # the reference's stash lookup misses stashed keys
    assert got["keys"].size > 0 and got["vertices"].shape[0] > 0
    assert np.array_equal(got["vertices"].view(np.int32), och.vertices().view(np.int32)), "vertices"
    assert np.array_equal(got["triangles"], och.triangles()), "triangle indices"
    assert np.array_equal(got["seams"], och.seams()), "seam nodes"


def test_csg_chunks_through_the_reference_kernels(ref):
    """Chunks of the tiled CSG workload with the stored operations replayed
    through the reference's CSG kernels (CSG_HermiteIndices,
    UpdateFieldMaterials, FindUpdatedEdges, RemoveInvalidIndices, the
    RemoveDuplicates rounds of duplicate.cl, FilterValidEdges, PruneFieldEdges,
    the CSG FindEdgeIntersectionInfo) under ApplyCSGOperations' host flow: the
    field materials, the kept edges in order, the created edges as a set (the
    reference orders them by a racy dedupe, duplicate.cl:40-51), every edge's
    hermite data by key, and the vertices, triangles and seams all equal the
    oracle's bit for bit."""
    from leven_gb300 import workloads as W

    O.set_seed(1)
    image = O.perm_image_rgba()
    ref.ref_set_perm_image(image.ctypes.data)
    wl = W.tiled_csg()
    by_ops = sorted(range(len(wl.chunks)), key=lambda c: -len(W.ops_for_chunk(wl.ops, *wl.chunks[c])))
    checked = 0
    for c in by_ops[:10]:
        mn, size = wl.chunks[c]
        ops = [op.as_tuple() for op in W.ops_for_chunk(wl.ops, mn, size)]
        och = O.OracleChunk(O.density(mode=1), mn, size, vpc=64, ops=ops)
        colour = och.vertices()[0, 8:11] if och.count(O.ORC_NODE_CODES) else np.zeros(3, np.float32)
        got = ref_chunk(ref, 1, mn, size, [float(v) for v in colour], ops)
        assert np.array_equal(got["materials"], och.materials()), "materials after CSG"
        keys, okeys = got["keys"], och.edge_keys()
        ncreated = och.count(O.ORC_CREATED_EDGE_KEYS)
        nk = okeys.size - ncreated
        assert keys.size == okeys.size and np.array_equal(keys[:nk], okeys[:nk]), "kept edges"
        assert set(keys[nk:].tolist()) == set(okeys[nk:].tolist()), "created edges"
        a, b = np.argsort(keys), np.argsort(okeys)
        assert np.array_equal(got["info"][a].view(np.int32), och.edge_info()[b].view(np.int32)), "hermite by key"
        assert got["stash"] == 0
        assert np.array_equal(got["vertices"].view(np.int32), och.vertices().view(np.int32)), "vertices"
        assert np.array_equal(got["triangles"], och.triangles()), "triangles"
        assert np.array_equal(got["seams"], och.seams()), "seams"
        checked += ncreated > 0
    assert checked >= 5
