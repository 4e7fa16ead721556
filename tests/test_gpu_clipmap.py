"""Parity of the GPU clipmap chunk lists (through the C ABI) with the oracle:
the selected nodes of every camera and the CSG touch set, node for node and in
the reference's recursion order."""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as O
from test_oracle_clipmap import ROOT_MIN, ROOT_SIZE, edge_cameras, random_ops

pytestmark = pytest.mark.gpu


def cameras(seed, n, spread=20000.0):
    rng = np.random.default_rng(seed)
    cams = [rng.uniform(-spread, spread, 3).astype(np.float32) for _ in range(n // 2)]
    return np.array(cams + edge_cameras(rng, n - n // 2), np.float32)


@pytest.mark.parametrize("root_min,root_size", [(ROOT_MIN, ROOT_SIZE), ((0, -4096, 512), 8192), ((-256, 0, 0), 256),
                                                ((-65536, -65536, -65536), 1 << 17)])
def test_select_batch(lvn_gpu, root_min, root_size):
    """600 cameras (random, on the leaf lattice, at exact active distances) in
    one call.  The 2^17 root lists 4096 or more nodes per camera, past the
    first pass's 1024-node stride: those cameras take the second pass."""
    lvn = lvn_gpu
    cams = cameras(root_size, 600, spread=1.2 * root_size)
    got = lvn.clipmap_select(cams, root_min, root_size)
    assert len(got) == len(cams)
    for q, cam in enumerate(cams):
        ref = O.clipmap_select(cam, root_min, root_size)
        assert np.array_equal(got[q], ref), (q, cam)


def test_select_device_form(lvn_gpu):
    """The device form on torch buffers: lists truncated at the stride, full
    counts reported, nothing synchronised by the call."""
    import torch

    lvn = lvn_gpu
    cams = cameras(5, 1000)
    stride = 300
    d_cams = torch.from_numpy(cams).cuda()
    d_out = torch.full((len(cams) * stride, 4), -7, dtype=torch.int32, device="cuda")
    d_counts = torch.zeros(len(cams), dtype=torch.int32, device="cuda")
    lvn.clipmap_select_device(d_cams, ROOT_MIN, ROOT_SIZE, d_out, stride, d_counts)
    torch.cuda.synchronize()
    out = d_out.cpu().numpy().reshape(len(cams), stride, 4)
    counts = d_counts.cpu().numpy()
    for q, cam in enumerate(cams):
        ref = O.clipmap_select(cam, ROOT_MIN, ROOT_SIZE)
        assert counts[q] == len(ref)
        k = min(stride, len(ref))
        assert np.array_equal(out[q, :k], ref[:k])
        assert (out[q, k:] == -7).all()


@pytest.mark.parametrize("n_ops,spread,rmax", [(1, 900.0, 40.0), (8, 900.0, 40.0), (32, 3000.0, 200.0),
                                               (200, 3000.0, 20.0)])
def test_touched(lvn_gpu, n_ops, spread, rmax):
    lvn = lvn_gpu
    rng = np.random.default_rng(100 + n_ops)
    ops = random_ops(rng, n_ops, spread, rmax)
    got = lvn.clipmap_touched([lvn.make_op(t, b, m, o, d, r) for t, b, m, r, o, d in ops], ROOT_MIN, ROOT_SIZE)
    ref = O.clipmap_touched(ops, ROOT_MIN, ROOT_SIZE)
    assert len(ref) > 0
    assert np.array_equal(got, ref)


def test_limits_and_errors(lvn_gpu):
    lvn = lvn_gpu
    L = lvn.lib()
    cam = np.zeros(3, np.float32)
    out = np.zeros((8, 4), np.int32)
    counts = np.zeros(1, np.int32)
    # not a power of two, below the leaf size, more than 16 top-level nodes per axis
    for rs in (3000, 128, 1 << 18):
        assert L.lvn_clipmap_select(cam.ctypes.data, 1, lvn._ivec3(ROOT_MIN), rs, out.ctypes.data, 8,
                                    counts.ctypes.data) == lvn.LVN_ERR_INVALID
    # capacity: the count is reported
    rc = L.lvn_clipmap_select(cam.ctypes.data, 1, lvn._ivec3(ROOT_MIN), ROOT_SIZE, out.ctypes.data, 8,
                              counts.ctypes.data)
    assert rc == lvn.LVN_ERR_CAPACITY and counts[0] == len(O.clipmap_select(cam, ROOT_MIN, ROOT_SIZE))
    # an operation covering the whole root touches more nodes than one query lists
    huge = lvn.make_op(0, 0, 1, (0.0, 0.0, 0.0), (5000.0, 5000.0, 5000.0))
    count = C.c_int32(0)
    rc = L.lvn_clipmap_touched(C.byref(huge), 1, lvn._ivec3(ROOT_MIN), ROOT_SIZE, out.ctypes.data, 8,
                               C.byref(count))
    assert rc == lvn.LVN_ERR_DEVICE_STATUS
    # no operations, no cameras
    assert len(lvn.clipmap_touched([], ROOT_MIN, ROOT_SIZE)) == 0
    assert lvn.clipmap_select(np.zeros((0, 3), np.float32), ROOT_MIN, ROOT_SIZE) == []


def test_selection_feeds_the_batch(lvn_gpu):
    """The selected nodes of LOD <= 1 near a camera mesh through
    generate_chunks as the reference's chunk descriptors."""
    lvn = lvn_gpu
    lvn.clear_csg_operations()
    lvn.set_density(mode=lvn.LVN_DENSITY_FBM2D)
    nodes = lvn.clipmap_select(np.array([[100.0, 20.0, -300.0]], np.float32), ROOT_MIN, ROOT_SIZE)[0]
    near = nodes[(nodes[:, 3] <= 512) & (nodes[:, 1] <= 0) & (nodes[:, 1] + nodes[:, 3] >= 0)][:24]  # at the surface
    assert len(near) >= 8
    g = lvn.MeshGen(64)
    try:
        verts, tris, seams, res = g.generate_chunks([(tuple(int(v) for v in n[:3]), int(n[3])) for n in near])
        assert res.shape[0] == len(near)
        assert verts.shape[0] > 0 and tris.shape[0] > 0
    finally:
        g.close()
