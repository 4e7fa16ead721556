"""Parity of the GPU seam meshes (lvn_seam_generate, through the C ABI) with
the oracle's restatement of GenerateClipmapSeamMesh: per host, the vertices
bit for bit in the octree's order and the triangles in the recursion's order."""
import numpy as np
import pytest

import oracle_lib as O
from test_oracle_seam import ROOT_MIN, ROOT_SIZE, SCENES, scene

pytestmark = pytest.mark.gpu


def compare(lvn, chunks, offs, seams, vpc, root_min, root_size, hosts, colour=(0.25, 0.5, 0.75), device=False):
    if device:
        import torch

        seams_in = torch.from_numpy(np.ascontiguousarray(seams)).cuda()
    else:
        seams_in = seams
    v, t, res = lvn.seam_generate(chunks, offs, seams_in, vpc, root_min, root_size, hosts, colour)
    rv, rt, counts = O.seam_generate(chunks, offs, seams, vpc, root_min, root_size, hosts, colour)
    assert np.array_equal(res[:, 1], counts[:, 0]), "vertices per host"
    assert np.array_equal(res[:, 3], counts[:, 1]), "triangles per host"
    assert np.array_equal(v.view(np.int32), rv.view(np.int32)), "vertices"
    assert np.array_equal(t, rt), "triangles"
    assert np.array_equal(res[:, 0], np.concatenate([[0], np.cumsum(counts[:-1, 0])]))
    return int(counts[:, 1].sum())


@pytest.mark.parametrize("cam,mode,vpc", SCENES)
def test_seams_oracle_meshed_scene(lvn_gpu, cam, mode, vpc):
    chunks, offs, seams = scene(cam, mode=mode, vpc=vpc)
    hosts = list(range(len(chunks)))
    assert compare(lvn_gpu, chunks, offs, seams, vpc, ROOT_MIN, ROOT_SIZE, hosts) > 0


def test_seams_device_input_and_host_subset(lvn_gpu):
    chunks, offs, seams = scene(SCENES[1][0], mode=SCENES[1][1], vpc=SCENES[1][2])
    hosts = list(range(len(chunks)))[::-3]
    assert compare(lvn_gpu, chunks, offs, seams, SCENES[1][2], ROOT_MIN, ROOT_SIZE, hosts, device=True) > 0


def test_seams_of_gpu_meshed_clipmap(lvn_gpu):
    """64^3 chunks of the LOD 0-4 caves clipmap meshed by the batch path; their
    seam nodes feed both the GPU seams and the oracle."""
    from leven_gb300 import workloads as W

    lvn = lvn_gpu
    lvn.clear_csg_operations()
    lvn.set_density(**W.CAVES)
    cam = (300.0, 10.0, -200.0)
    rmin, rsize = W.CLIPMAP_ROOT_MIN, W.CLIPMAP_ROOT_SIZE
    nodes = lvn.clipmap_select(np.array([cam], np.float32), rmin, rsize)[0]
    nodes = nodes[nodes[:, 3] <= 4096]
    near = np.argsort(np.abs(nodes[:, :3] + nodes[:, 3:4] // 2 - np.array(cam)).max(1))[:160]
    chunks = [(tuple(int(x) for x in nodes[i, :3]), int(nodes[i, 3])) for i in sorted(near)]
    g = lvn.MeshGen(64)
    try:
        _, _, s, res = g.generate_chunks(chunks)
    finally:
        g.close()
    rows = np.concatenate([s[o:o + n] for o, n in zip(res[:, 4], res[:, 5])]).astype(np.int32)
    offs = np.concatenate([[0], np.cumsum(res[:, 5])]).astype(np.int32)
    assert compare(lvn, chunks, offs, rows, 64, rmin, rsize, list(range(len(chunks)))) > 0


def test_seams_errors(lvn_gpu):
    lvn = lvn_gpu
    chunks = [((0, 0, 0), 256)]
    offs = np.array([0, 0], np.int32)
    seams = np.zeros((0, 12), np.int32)
    v, t, res = lvn.seam_generate(chunks, offs, seams, 16, (-1024, -1024, -1024), 2048, [0])
    assert len(v) == 0 and len(t) == 0 and res[0, 1] == 0
    with pytest.raises(lvn.LvnError):
        lvn.seam_generate(chunks, offs, seams, 16, (-1024, -1024, -1024), 2048, [3])  # host out of range
    with pytest.raises(lvn.LvnError):
        lvn.seam_generate([((0, 0, 0), 384)], offs, seams, 16, (-1024, -1024, -1024), 2048, [0])  # not a node size
    two = np.array([0, 0, 0], np.int32)
    with pytest.raises(lvn.LvnError):  # overlapping active nodes
        lvn.seam_generate([((0, 0, 0), 256), ((0, 0, 0), 512)], two, seams, 16, (-1024, -1024, -1024), 2048, [0])
    with pytest.raises(lvn.LvnError):  # a chunk listed twice
        lvn.seam_generate([((0, 0, 0), 256), ((0, 0, 0), 256)], two, seams, 16, (-1024, -1024, -1024), 2048, [0])
