"""The seam meshes (GenerateClipmapSeamMesh, clipmap.cpp:573-610) on the CPU.

The oracle restates the reference literally: a pointer octree built upwards
from the gathered seam nodes (octree.cpp:31-148), numbered depth first and
contoured by the cell / face / edge recursion (octree.cpp:197-474).  The GPU
kernels use a different formulation (Morton-ordered leaves, one quad per final
edge segment, the recursion's order restored from its path); tests/seam_model.py
models that formulation in Python and is checked here against the oracle on
mixed-LOD clipmap scenes.  The reference ships no seam fixtures and octree.cpp
does not compile without the engine ("parity unpinned" against the reference
itself).
"""
import numpy as np
import pytest

import oracle_lib as O
import seam_model as SM

ROOT_MIN = (-2048, -2048, -2048)
ROOT_SIZE = 4096
VPC = 16


def scene(cam, root_min=ROOT_MIN, root_size=ROOT_SIZE, vpc=VPC, mode=1, ops=()):
    """The chunks a camera selects in a small clipmap, meshed by the oracle:
    (chunks, seam offsets, seam rows (S, 12) int32)."""
    O.set_seed(1)
    dens = O.density(mode=mode)
    nodes = O.clipmap_select(np.array(cam, np.float32), root_min, root_size)
    chunks, offs, rows = [], [0], []
    for x, y, z, s in nodes:
        ch = O.OracleChunk(dens, (int(x), int(y), int(z)), int(s), vpc=vpc, ops=ops)
        seams = ch.seams().reshape(-1, 12)
        chunks.append(((int(x), int(y), int(z)), int(s)))
        rows.append(seams)
        offs.append(offs[-1] + len(seams))
    return chunks, np.array(offs, np.int32), np.concatenate(rows).astype(np.int32)


@pytest.fixture(scope="module")
def mixed():
    return scene((100.0, 20.0, -300.0))


def test_scene_has_mixed_lods_and_seams(mixed):
    chunks, offs, seams = mixed
    assert len({s for _, s in chunks}) >= 3
    assert offs[-1] > 1000


def test_oracle_seams_valid(mixed):
    chunks, offs, seams = mixed
    hosts = list(range(len(chunks)))
    v, t, counts = O.seam_generate(chunks, offs, seams, VPC, ROOT_MIN, ROOT_SIZE, hosts)
    assert counts[:, 1].sum() > 0
    off = 0
    for nv, nt in counts:
        tri = t[off:off + nt] if nt else np.zeros((0, 3), np.int32)
        assert (nt == 0) == (nv == 0)
        if nt:
            assert tri.min() >= 0 and tri.max() < nv
        off += nt
    # a host's seam mesh does not depend on the other hosts in the call
    v1, t1, c1 = O.seam_generate(chunks, offs, seams, VPC, ROOT_MIN, ROOT_SIZE, hosts[::-1], threads=4)
    assert np.array_equal(c1[::-1], counts)


SCENES = [((100.0, 20.0, -300.0), 1, VPC), ((-700.0, 60.0, 900.0), 2, VPC), ((1500.0, -30.0, 40.0), 2, 8),
          ((0.0, 0.0, 0.0), 1, 32)]


@pytest.mark.parametrize("cam,mode,vpc", SCENES)
def test_model_matches_oracle(cam, mode, vpc):
    """The kernels' formulation, host by host: the leaves' order (by their
    vertex positions) and the triangles, in order."""
    chunks, offs, seams = scene(cam, mode=mode, vpc=vpc)
    check_model(chunks, offs, seams, vpc)


def check_model(chunks, offs, seams, vpc):
    hosts = list(range(len(chunks)))
    v, t, counts = O.seam_generate(chunks, offs, seams, vpc, ROOT_MIN, ROOT_SIZE, hosts)
    vo = to = 0
    checked = 0
    for h in hosts:
        nv, nt = counts[h]
        leaves = SM.gather(chunks, offs, seams, vpc, ROOT_MIN, ROOT_SIZE, h)
        if leaves:
            order, tris = SM.contour(chunks[h][0], chunks[h][1], [(m, s, c) for m, s, c, _ in leaves])
        else:
            order, tris = [], []
        if not tris:
            assert nt == 0
            continue
        assert nv == len(order) and nt == len(tris), h
        pos = seams[[leaves[i][3] for i in order]][:, 4:7].view(np.float32)
        assert np.array_equal(v[vo:vo + nv, :3], pos), h
        assert np.array_equal(t[to:to + nt], np.array(tris, np.int32)), h
        vo += nv
        to += nt
        checked += 1
    assert checked >= 5
    return checked
