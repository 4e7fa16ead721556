"""Parity on the full workloads the benchmark times, every chunk against the
oracle (or, for the 4096-chunk sweep, a large subset), stage by stage:

- the tiled CSG workload: 128 LOD0 chunks, 32 stored operations;
- the clipmap caves set: 1024 chunks over LODs 0-4, plain and with the octree
  simplification at 0.05;
- the clipmap sweep: 4096 chunks over LODs 0-5 with caves and 64 stored
  operations; every chunk an operation touches plus every 12th other chunk.

Each chunk's edge keys (kept in order, CSG-created as a set), hermite data
(bits), leaf codes, edge masks and materials, vertices (bits), triangles and
seams are compared.  The leaves' FP32 vertices are also held against the
oracle's FP64 solve of the same crossings, and against the library's own FP64
check (lvn_meshgen_qef_fp64_error): mean within 1e-4 voxel, at most one leaf
in 10^4 farther than 1e-3 voxel, none farther than one voxel.  The far leaves
are those with a singular value of ATA at the pseudo-inverse threshold (0.1),
kept in one precision and truncated in the other.

The oracle runs on host threads (its ctypes calls release the GIL).
"""
import collections
import concurrent.futures as cf
import os

import numpy as np
import pytest

import oracle_lib as O
from leven_gb300 import workloads as W
from test_gpu_parity import compare_mesh, compare_stages, oracle_density
from test_gpu_simplify import compare_simplified

pytestmark = pytest.mark.gpu

QEF_FP64_MEAN = 1e-4     # voxel
QEF_FP64_FAR = 1e-3      # voxel; at most QEF_FP64_FAR_RATE of the leaves beyond it
QEF_FP64_FAR_RATE = 1e-4
QEF_FP64_MAX = 1.0       # voxel


def oracle_chunks(wl, idx, simplify=None, window=64):
    """(c, OracleChunk) for the chunks in idx, in order, computed on host
    threads with at most `window` finished chunks held."""
    dens = oracle_density(wl.density["mode"])

    def run(c):
        mn, size = wl.chunks[c]
        ops = [op.as_tuple() for op in W.ops_for_chunk(wl.ops, mn, size)]
        ref = O.OracleChunk(dens, mn, size, vpc=wl.voxels_per_chunk, ops=ops)
        if simplify is not None and ref.count(O.ORC_NODE_CODES) > 0:
            ref.simplify(simplify)
        return c, ref, len(ops)

    O.set_seed(wl.noise_seed)
    idx = list(idx)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        pending = collections.deque()
        it = iter(idx)
        for c in it:
            pending.append(ex.submit(run, c))
            if len(pending) >= window:
                break
        while pending:
            yield pending.popleft().result()
            nxt = next(it, None)
            if nxt is not None:
                pending.append(ex.submit(run, nxt))


def store_ops(lvn, wl):
    lvn.clear_csg_operations()
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions,
                                            op.rotate_y))


def check_workload(lvn, wl, idx=None, simplify=None):
    lvn.set_density(**wl.density)
    store_ops(lvn, wl)
    g = lvn.MeshGen(wl.voxels_per_chunk)
    try:
        g.set_option(lvn.LVN_OPT_CACHE, 0)
        if simplify is not None:
            g.set_simplify(simplify)
        V, T, S, res = g.generate_chunks(wl.chunks)
        idx = range(len(wl.chunks)) if idx is None else idx
        if simplify is None:
            gmax, gmean, gleaves, gfar = g.qef_fp64_error()
            assert gleaves == int(res[:, 7].sum())
            assert gmean <= QEF_FP64_MEAN and gmax <= QEF_FP64_MAX and gfar <= QEF_FP64_FAR_RATE * gleaves, \
                (gmax, gmean, gfar, gleaves)
        checked = with_ops = 0
        errs = []
        for c, ref, nops in oracle_chunks(wl, idx, simplify):
            mn, size = wl.chunks[c]
            scale = size // (4 * wl.voxels_per_chunk)
            r = res[c]
            assert r[6] == ref.count(O.ORC_EDGE_KEYS) and r[7] == ref.count(O.ORC_NODE_CODES), f"chunk {c} counts"
            if r[6]:
                compare_stages(lvn, g, c, ref, wl.voxels_per_chunk, scale, created_as_set=nops > 0)
            verts, tris, seams = V[r[0]:r[0] + r[1]], T[r[2]:r[2] + r[3]], S[r[4]:r[4] + r[5]]
            if simplify is not None:
                if r[7]:
                    compare_simplified(lvn, g, c, verts, tris, seams, ref)
            else:
                compare_mesh(verts, tris, seams, ref, scale)
                nv = ref.mesh_vertex_count()
                assert np.array_equal(verts.view(np.int32), ref.vertices()[:nv].view(np.int32)), f"chunk {c} vertex bits"
                if nv:
                    errs.append(ref.qef_fp64_error_voxels(verts))
            checked += 1
            with_ops += nops > 0
        if errs:
            e = np.concatenate(errs)
            assert e.mean() <= QEF_FP64_MEAN and e.max() <= QEF_FP64_MAX, (e.mean(), e.max())
            assert (e > QEF_FP64_FAR).sum() <= QEF_FP64_FAR_RATE * e.size + 1, (e > QEF_FP64_FAR).sum()
        return res, checked, with_ops
    finally:
        g.close()
        lvn.clear_csg_operations()


def test_tiled_csg_128_every_chunk(lvn_gpu):
    wl = W.tiled_csg()
    res, checked, with_ops = check_workload(lvn_gpu, wl)
    assert checked == 128 and with_ops > 0 and res[:, 3].sum() > 0


def test_clipmap_caves_1024_every_chunk(lvn_gpu):
    wl = W.clipmap_caves()
    res, checked, _ = check_workload(lvn_gpu, wl)
    assert checked == 1024 and (res[:, 7] == 0).any() and res[:, 7].max() > 10000


def test_clipmap_caves_1024_simplified_every_chunk(lvn_gpu):
    wl = W.clipmap_caves()
    res, checked, _ = check_workload(lvn_gpu, wl, simplify=0.05)
    assert checked == 1024


def test_clipmap_sweep_4096_subset(lvn_gpu):
    """Every chunk a stored operation touches, and every 12th other chunk of
    the 4096 (over 500 chunks, all six LODs)."""
    wl = W.clipmap_sweep()
    touched = [c for c, (mn, s) in enumerate(wl.chunks) if W.ops_for_chunk(wl.ops, mn, s)]
    idx = sorted(set(touched) | set(range(0, len(wl.chunks), 12)))
    res, checked, with_ops = check_workload(lvn_gpu, wl, idx)
    assert checked == len(idx) >= 500 and with_ops == len(touched) > 100
    assert {wl.chunks[c][1] for c in idx} == {256 << k for k in range(6)}
    assert res[:, 3].sum() > 0
