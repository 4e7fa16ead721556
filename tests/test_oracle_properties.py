"""Self-consistency of the oracle's integer stages, checked by independent
numpy restatements of FindFieldEdges (density_field.cl:41-76),
FindActiveVoxels (octree.cl:142-201) and GenerateMesh (octree.cl:385-442)."""
import numpy as np
import pytest

import oracle_lib as O

AIR = 201


@pytest.fixture(scope="module", autouse=True)
def seed():
    O.set_seed(1)


def shift_of(vpc):
    return int(np.log2(vpc)) + 1


def field(ch, vpc):
    fd = vpc + 2
    return ch.materials().reshape(fd, fd, fd)  # [z, y, x]


def numpy_edges(m, vpc):
    hd, sh = vpc + 1, shift_of(vpc)
    solid = m != AIR
    keys = []
    for z in range(hd):
        for y in range(hd):
            for x in range(hd):
                for a, (dx, dy, dz) in enumerate(((1, 0, 0), (0, 1, 0), (0, 0, 1))):
                    if solid[z, y, x] != solid[z + dz, y + dy, x + dx]:
                        keys.append(((x | (y << sh) | (z << 2 * sh)) << 2) | a)
    return np.asarray(keys, np.int32)


CORNERS = [(0, 0, 0), (0, 0, 1), (0, 1, 0), (0, 1, 1), (1, 0, 0), (1, 0, 1), (1, 1, 0), (1, 1, 1)]
EDGE_MAP = [(0, 4), (1, 5), (2, 6), (3, 7), (0, 2), (1, 3), (4, 6), (5, 7), (0, 1), (2, 3), (4, 5), (6, 7)]


def code_for(x, y, z, depth):
    code = 1
    for d in range(depth - 1, -1, -1):
        code = (code << 3) | (((x >> d) & 1) << 2) | (((y >> d) & 1) << 1) | ((z >> d) & 1)
    return code


@pytest.mark.parametrize("mode,vpc", [(1, 16), (1, 32), (0, 16), (2, 16)])
def test_edges_and_voxels_independent(mode, vpc):
    mn = (0, 0, 0) if mode == 0 else (0, 128, 0)
    ch = O.OracleChunk(O.density(mode=mode), mn, 4 * vpc, vpc=vpc)
    m = field(ch, vpc)
    assert np.array_equal(ch.edge_keys(), numpy_edges(m, vpc))
    depth = int(np.log2(vpc))
    codes, edges, corners_l = [], [], []
    for z in range(vpc):
        for y in range(vpc):
            for x in range(vpc):
                c = 0
                for i, (ox, oy, oz) in enumerate(CORNERS):
                    c |= int(m[z + oz, y + oy, x + ox] != AIR) << i
                if c in (0, 255):
                    continue
                codes.append(code_for(x, y, z, depth))
                e = 0
                for i, (a, b) in enumerate(EDGE_MAP):
                    e |= int(((c >> a) & 1) != ((c >> b) & 1)) << i
                edges.append(e)
                corners_l.append(c)
    assert np.array_equal(ch.node_codes(), np.asarray(codes, np.uint32))
    assert np.array_equal(ch.node_edges(), np.asarray(edges, np.int32))
    assert np.array_equal(ch.node_materials() & 0xFF, np.asarray(corners_l, np.int32))


@pytest.mark.parametrize("vpc", [16, 32])
def test_mesh_topology(vpc):
    ch = O.OracleChunk(O.density(mode=1), (0, 128, 0), 4 * vpc, vpc=vpc)
    tris = ch.triangles()
    nv = ch.count(O.ORC_NODE_CODES)
    assert tris.size and tris.min() >= 0 and tris.max() < nv
    assert ch.mesh_vertex_count() == nv
    # each quad = 2 triangles sharing the diagonal (octree.cl:357-362)
    q = tris.reshape(-1, 6)
    assert np.all(q[:, 0] == q[:, 3])
    v = ch.vertices()
    assert np.isfinite(v).all()
    # unclamped QEF solutions stay within two voxels of their leaf cube
    # (world units, LOD0: 4 per voxel)
    codes = ch.node_codes()
    depth = int(np.log2(vpc))
    pos = np.zeros((codes.size, 3), np.int64)
    for i, c in enumerate(codes.tolist()):
        for d in range(depth):
            b = (c >> (3 * d)) & 7
            pos[i] += np.array([(b >> 2) & 1, (b >> 1) & 1, b & 1]) << d
    world = pos * 4 + np.array([0, 128, 0])
    assert np.all(v[:, :3] >= world - 8.0) and np.all(v[:, :3] <= world + 12.0)


def test_empty_and_full_chunks():
    d = O.density(mode=1)
    high = O.OracleChunk(d, (0, 4096, 0), 64, vpc=16)   # far above the surface: all air
    assert high.count(O.ORC_EDGE_KEYS) == 0 and high.count(O.ORC_NODE_CODES) == 0
    low = O.OracleChunk(d, (0, -4096, 0), 64, vpc=16)   # far below: all solid
    assert low.count(O.ORC_EDGE_KEYS) == 0 and low.mesh_vertex_count() == 0


def test_csg_subtract_sphere_creates_and_prunes():
    d = O.density(mode=1)
    # sphere centred on the surface region of the chunk at (0, 128, 0) size 64
    base = O.OracleChunk(d, (0, 128, 0), 64, vpc=16)
    op = (1, 1, AIR, 0.0, (8.0, 40.0, 8.0), (5.0, 5.0, 5.0))
    ch = O.OracleChunk(d, (0, 128, 0), 64, vpc=16, ops=[op])
    mats = ch.materials()
    assert (mats == AIR).sum() >= (base.materials() == AIR).sum()
    plain = set(ch.plain_edge_keys().tolist())
    final = ch.edge_keys().tolist()
    created = ch.created_edge_keys().tolist()
    assert len(set(final)) == len(final)
    assert set(created) <= set(final)
    kept = [k for k in final if k not in set(created)]
    assert set(kept) <= plain
    # the final edge set is exactly the sign changes of the final materials
    # inside the hermite grid, plus created edges on the field border
    vpc, sh = 16, shift_of(16)
    m = mats.reshape(18, 18, 18)
    inside = set(numpy_edges(m, vpc).tolist())
    border = {k for k in final if max((k >> 2) & 31, (k >> (2 + sh)) & 31, (k >> (2 + 2 * sh)) & 31) > vpc}
    assert set(final) - border == inside


def test_op_bounds_and_overlap():
    lo, hi = O.op_bounds((1, 1, AIR, 0.0, (10.5, 20.5, -3.5), (3.0, 3.0, 3.0)))
    # CalcCSGOperationBounds: half = int(3 * 4) + 2 = 14, origin = int((o - 0.5) * 4)
    assert lo == [40 - 14, 80 - 14, -16 - 14] and hi == [40 + 14, 80 + 14, -16 + 14]
