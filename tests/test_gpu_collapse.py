"""Parity of the GPU edge-collapse simplification (lvn_mesh_simplify, through
the C ABI) with the oracle's restatement of ngMeshSimplifier: every mesh's
vertices bit for bit and its triangles in order."""
import numpy as np
import pytest

import oracle_lib as O

pytestmark = pytest.mark.gpu


def batch(lvn, chunks, mode, vpc=64):
    lvn.clear_csg_operations()
    lvn.set_density(mode=mode)
    g = lvn.MeshGen(vpc)
    try:
        v, t, _, res = g.generate_chunks(chunks)
    finally:
        g.close()
    return v, t, res


def check(lvn, chunks, v, t, res, device=False):
    ranges = res[:, :4].copy()
    offsets = [lvn.node_offset(mn, size) for mn, size in chunks]
    opts = [lvn.engine_simplify_options(size) for _, size in chunks]
    if device:
        import torch

        dv = torch.from_numpy(v.copy()).cuda()
        dt = torch.from_numpy(t.copy()).cuda()
        _, _, out = lvn.mesh_simplify(dv, dt, ranges, offsets, opts)
        sv, st = dv.cpu().numpy(), dt.cpu().numpy()
    else:
        sv, st, out = lvn.mesh_simplify(v, t, ranges, offsets, opts)
    simplified = 0
    for m, (mn, size) in enumerate(chunks):
        vo, nv, to, nt = ranges[m]
        rv, rt = O.mesh_collapse(v[vo:vo + nv], t[to:to + nt], O.node_offset(mn, size), O.simplify_options(size))
        assert out[m, 1] == len(rv) and out[m, 3] == len(rt), (m, out[m], len(rv), len(rt))
        assert np.array_equal(sv[vo:vo + len(rv)].view(np.int32), rv.view(np.int32)), f"vertices of mesh {m}"
        assert np.array_equal(st[to:to + len(rt)], rt), f"triangles of mesh {m}"
        simplified += len(rt) < nt
    return simplified


def test_simplify_tiled_terrain(lvn_gpu):
    lvn = lvn_gpu
    chunks = [((x * 256, 128 * (x % 2), z * 256), 256) for x in range(4) for z in range(3)]
    v, t, res = batch(lvn, chunks, lvn.LVN_DENSITY_FBM2D)
    assert check(lvn, chunks, v, t, res) >= 6


def test_simplify_caves_mixed_sizes_device_in_place(lvn_gpu):
    lvn = lvn_gpu
    chunks = [((0, 0, 0), 256), ((256, -256, 0), 256), ((0, -512, 512), 512), ((1024, -1024, 0), 1024),
              ((-512, 0, -512), 512)]
    v, t, res = batch(lvn, chunks, lvn.LVN_DENSITY_CAVES)
    assert check(lvn, chunks, v, t, res, device=True) >= 3


def test_simplify_small_meshes_and_vpc(lvn_gpu):
    """vpc 16 and 8 chunks (fewer than 100 triangles are left as generated)."""
    lvn = lvn_gpu
    chunks = [((x * 256, 0, 0), 256) for x in range(6)]
    for vpc in (16, 8):
        v, t, res = batch(lvn, chunks, lvn.LVN_DENSITY_FBM2D, vpc=vpc)
        check(lvn, chunks, v, t, res)


def test_simplify_errors(lvn_gpu):
    lvn = lvn_gpu
    bad = lvn.engine_simplify_options(256)
    bad.edge_fraction = 2.0
    with pytest.raises(lvn.LvnError):
        lvn.mesh_simplify(np.zeros((1, 12), np.float32), np.zeros((1, 3), np.int32), [[0, 1, 0, 1]],
                          [[0, 0, 0, 0]], [bad])
