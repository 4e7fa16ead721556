"""Properties of the oracle's bottom-up octree simplification (CPU only).

The simplification is not in the reference, so nothing there pins it; these
tests check it against an independent float64 re-derivation of each collapsed
node's QEF error from the chunk's hermite data, and against the structural
properties dual contouring on a collapsed octree must keep.
"""
from collections import Counter

import numpy as np
import pytest

import oracle_lib as O

EDGE_MAP = [(0, 4), (1, 5), (2, 6), (3, 7), (0, 2), (1, 3), (4, 6), (5, 7), (0, 1), (2, 3), (4, 5), (6, 7)]
CHILD = [((i >> 2) & 1, (i >> 1) & 1, i & 1) for i in range(8)]


def positions(codes, depth):
    p = np.zeros((codes.size, 3), np.int64)
    c = codes.astype(np.int64)
    for i in range(depth):
        b = c & 7
        c >>= 3
        p[:, 0] |= ((b >> 2) & 1) << i
        p[:, 1] |= ((b >> 1) & 1) << i
        p[:, 2] |= (b & 1) << i
    return p


def chunk(mode, mn, vpc=64):
    O.set_seed(1)
    return O.OracleChunk(O.density(mode=mode), mn, 4 * vpc, vpc=vpc)


CASES = [(1, (0, 128, 0), 64), (2, (0, 0, 0), 64), (2, (128, 0, 256), 32)]


def undirected_edges(tris):
    c = Counter()
    for t in tris:
        for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
            c[(min(a, b), max(a, b))] += 1
    return c


@pytest.mark.parametrize("mode,mn,vpc", CASES)
def test_structure(mode, mn, vpc):
    ch = chunk(mode, mn, vpc)
    V = ch.count(O.ORC_NODE_CODES)
    plain_boundary = sum(1 for v in undirected_edges(ch.triangles()).values() if v == 1)
    depth = vpc.bit_length() - 1
    pos = positions(ch.node_codes(), depth)
    seam = ((pos == 0) | (pos == vpc - 1)).any(axis=1)
    last = None
    for thr in (0.0, 0.05, 1.0, 1e9):
        ch.simplify(thr)
        tris = ch.simp_triangles()
        verts = ch.simp_vertices()
        reps = ch.simp_reps()
        level, anchor = reps >> 20, reps & 0xFFFFF
        assert reps.size == V
        # seam voxels never collapse, anchors are the first leaf below their node
        assert (level[seam] == 0).all() and (anchor[seam] == np.arange(V)[seam]).all()
        assert (anchor <= np.arange(V)).all()
        assert verts.shape[0] == np.count_nonzero(anchor == np.arange(V))
        if tris.size:
            assert tris.min() >= 0 and tris.max() < verts.shape[0]
            assert (tris[:, 0] != tris[:, 1]).all() and (tris[:, 1] != tris[:, 2]).all() and (tris[:, 0] != tris[:, 2]).all()
        # the open border of the chunk's mesh is the seam voxels' and is kept
        assert sum(1 for v in undirected_edges(tris).values() if v == 1) == plain_boundary
        # leaves of one representative share its node
        for lv in range(1, depth + 1):
            sel = level == lv
            if sel.any():
                node = pos[sel] >> lv
                first = pos[anchor[sel]] >> lv
                assert (node == first).all()
        if last is not None:
            assert verts.shape[0] <= last
        last = verts.shape[0]
    assert last < V  # something collapsed at the largest threshold


def test_threshold_zero_keeps_leaf_vertices():
    ch = chunk(1, (0, 128, 0))
    plain = ch.vertices()[:ch.mesh_vertex_count()]
    ch.simplify(0.0)
    reps = ch.simp_reps()
    keep = (reps >> 20) == 0
    verts = ch.simp_vertices()
    # leaf representatives carry the unsimplified vertex bit for bit
    anchors = np.flatnonzero((reps & 0xFFFFF) == np.arange(reps.size))
    leaf_rows = np.flatnonzero(keep[anchors])
    assert np.array_equal(verts[leaf_rows].view(np.int32), plain[anchors[leaf_rows]].view(np.int32))


@pytest.mark.parametrize("mode,mn,vpc", CASES[:2])
@pytest.mark.parametrize("thr", [0.05, 1.0])
def test_error_bound_float64(mode, mn, vpc, thr):
    """Each collapsed node's vertex, re-checked in float64 against all the
    edge crossings below it: sum (n.(x - p))^2 <= threshold."""
    ch = chunk(mode, mn, vpc)
    depth = vpc.bit_length() - 1
    shift = depth + 1
    keys, info = ch.edge_keys(), ch.edge_info().astype(np.float64)
    index = {int(k): i for i, k in enumerate(keys)}
    pos = positions(ch.node_codes(), depth)
    edges = ch.node_edges()
    ch.simplify(thr)
    reps = ch.simp_reps()
    level, anchor = reps >> 20, reps & 0xFFFFF
    verts = ch.simp_vertices()
    vindex = np.cumsum(anchor == np.arange(reps.size)) - 1
    checked = 0
    for a in np.unique(anchor[level > 0]):
        members = np.flatnonzero(anchor == a)
        lv = int(level[members[0]])
        origin = (pos[a] >> lv) << lv
        x_world = verts[vindex[a], :3].astype(np.float64)
        x = (x_world - np.array(mn, np.float64)) / 4.0 - origin  # voxel units, node frame (sampleScale 1)
        err = 0.0
        for v in members:
            for e, (c0, c1) in enumerate(EDGE_MAP):
                if not (edges[v] >> e) & 1:
                    continue
                o0, o1 = np.array(CHILD[c0]), np.array(CHILD[c1])
                q = pos[v] + o0
                key = ((int(q[0]) | (int(q[1]) << shift) | (int(q[2]) << (2 * shift))) << 2) | (e // 4)
                if key not in index:
                    continue
                nx, ny, nz, t = info[index[key]]
                p = (pos[v] - origin) + o0 + (o1 - o0) * np.float32(t)
                err += (nx * (x[0] - p[0]) + ny * (x[1] - p[1]) + nz * (x[2] - p[2])) ** 2
        assert err <= thr * (1 + 1e-3) + 1e-4, (a, lv, err)
        assert (x >= -1e-4).all() and (x <= (1 << lv) + 1e-4).all()
        checked += 1
    assert checked > 0
