"""The oracle's clipmap chunk lists (CPU only).

SelectActiveClipmapNodes / FindNodesInsideAABB / processCSGOperationsImpl
(leven/src/clipmap.cpp:1056-1128, 1571-1607, 1647-1673) ship no known answers
and clipmap.cpp does not compile without the engine's renderer and physics, so
the oracle's restatement is checked here against a second, independent
restatement (leven_gb300.workloads, float64 distances) and against brute-force
enumeration of the octree's nodes ("parity unpinned" against the reference
itself).
"""
import itertools

import numpy as np
import pytest

import oracle_lib as O
from leven_gb300 import workloads as W

ROOT_MIN = (-16384, -16384, -16384)
ROOT_SIZE = 1 << 15


def all_nodes(root_min, root_size, max_size):
    """Every node of the complete octree no larger than max_size."""
    size = W.CLIPMAP_LEAF_SIZE
    while size <= min(root_size, max_size):
        per = root_size // size
        for i, j, k in itertools.product(range(per), repeat=3):
            yield (root_min[0] + i * size, root_min[1] + j * size, root_min[2] + k * size, size)
        size *= 2


def edge_cameras(rng, n):
    """Cameras on the leaf lattice and at exact active distances from it."""
    out = []
    for _ in range(n):
        base = rng.integers(-40, 40, 3) * 256
        off = rng.choice([0.0, 128.0, 384.0, 896.0, 1408.0, 1920.0, 3456.0, -384.0, 0.5, -0.25], 3)
        out.append((base + off).astype(np.float32))
    return out


def test_select_matches_second_restatement():
    rng = np.random.default_rng(7)
    cams = [rng.uniform(-20000, 20000, 3).astype(np.float32) for _ in range(60)] + edge_cameras(rng, 60)
    for cam in cams:
        a = O.clipmap_select(cam, ROOT_MIN, ROOT_SIZE)
        b = W.select_clipmap_nodes(ROOT_MIN, ROOT_SIZE, tuple(float(x) for x in cam))
        assert np.array_equal(a, np.array([[*m, s] for m, s in b], np.int32).reshape(-1, 4)), cam


@pytest.mark.parametrize("root_size", [256, 2048, 8192, 1 << 15, 1 << 16])
def test_select_covers_the_root_once(root_size):
    """The selected nodes tile the root: disjoint, volumes summing to the root's."""
    rng = np.random.default_rng(root_size)
    root_min = (-(root_size // 2), 0, -(root_size // 4))
    for _ in range(8):
        cam = rng.uniform(-root_size, root_size, 3).astype(np.float32)
        nodes = O.clipmap_select(cam, root_min, root_size).astype(np.int64)
        assert (nodes[:, 3] ** 3).sum() == root_size ** 3
        # pre-order of a tiling: strictly increasing Morton order of the first leaves
        leaf = (nodes[:, :3] - np.array(root_min)) // W.CLIPMAP_LEAF_SIZE
        keys = [morton(p) for p in leaf]
        assert keys == sorted(keys) and len(set(keys)) == len(keys)


def morton(p):
    code = 0
    for bit in range(20, -1, -1):
        code = (code << 3) | (((int(p[0]) >> bit) & 1) << 2) | (((int(p[1]) >> bit) & 1) << 1) | ((int(p[2]) >> bit) & 1)
    return code


def test_select_lod_distances():
    """Every selected node of LOD l > 0 lies at least LOD_ACTIVE_DISTANCES[l] away."""
    rng = np.random.default_rng(3)
    for _ in range(20):
        cam = rng.uniform(-8000, 8000, 3).astype(np.float32)
        for x, y, z, s in O.clipmap_select(cam, ROOT_MIN, ROOT_SIZE):
            lod = int(s // W.CLIPMAP_LEAF_SIZE).bit_length() - 1
            assert W.distance_to_node((x, y, z), s, cam.astype(np.float64)) >= W.LOD_ACTIVE_DISTANCES[lod] - 1e-3


def brute_overlap(box_lo, box_hi, root_min, root_size):
    out = set()
    for x, y, z, s in all_nodes(root_min, root_size, W.LOD_MAX_NODE_SIZE):
        apart = (box_hi[0] < x or box_hi[1] < y or box_hi[2] < z or box_lo[0] > x + s or box_lo[1] > y + s or
                 box_lo[2] > z + s)
        if not apart:
            out.add((x, y, z, s))
    return out


def is_post_order(nodes):
    """Every node comes after all of its listed descendants."""
    pos = {tuple(n): i for i, n in enumerate(nodes)}
    for i, (x, y, z, s) in enumerate(nodes):
        if s == W.CLIPMAP_LEAF_SIZE:
            continue
        h = s // 2
        for c in range(8):
            ch = (x + ((c >> 2) & 1) * h, y + ((c >> 1) & 1) * h, z + (c & 1) * h, h)
            if ch in pos and pos[ch] > i:
                return False
    return True


def test_nodes_in_aabb_matches_brute_force():
    root_min, root_size = (-4096, -4096, -4096), 8192  # 32^3 leaves: enumerable
    rng = np.random.default_rng(11)
    for _ in range(12):
        lo = rng.integers(-5000, 4000, 3)
        hi = lo + rng.integers(0, 3000, 3)
        got = O.clipmap_nodes_in_aabb(lo, hi, root_min, root_size)
        assert set(map(tuple, got.tolist())) == brute_overlap(lo, hi, root_min, root_size)
        assert len(got) == len(set(map(tuple, got.tolist())))
        assert is_post_order([tuple(n) for n in got.tolist()])


def random_ops(rng, n, spread=900.0, rmax=40.0):
    ops = []
    for _ in range(n):
        o = rng.uniform(-spread, spread, 3)
        d = rng.uniform(1.0, rmax, 3)
        ops.append((int(rng.integers(0, 2)), int(rng.integers(0, 2)), 1, float(rng.uniform(0, 3)), tuple(o), tuple(d)))
    return ops


@pytest.mark.parametrize("n_ops", [1, 5, 32])
def test_touched_is_the_union_of_the_per_op_walks(n_ops):
    """processCSGOperationsImpl's touch set: the union of FindNodesInsideAABB
    over the operations' CalcCSGOperationBounds, each node once."""
    rng = np.random.default_rng(n_ops)
    ops = random_ops(rng, n_ops)
    got = O.clipmap_touched(ops, ROOT_MIN, ROOT_SIZE)
    union = set()
    for op in ops:
        lo, hi = O.op_bounds(op)
        union |= set(map(tuple, O.clipmap_nodes_in_aabb(lo, hi, ROOT_MIN, ROOT_SIZE).tolist()))
    assert set(map(tuple, got.tolist())) == union
    assert len(got) == len(union)
    assert is_post_order([tuple(n) for n in got.tolist()])


def test_touched_empty_and_outside():
    assert O.clipmap_touched([], ROOT_MIN, ROOT_SIZE).shape == (0, 4)
    far = [(0, 1, 1, 0.0, (1e6, 1e6, 1e6), (4.0, 4.0, 4.0))]
    assert O.clipmap_touched(far, ROOT_MIN, ROOT_SIZE).shape == (0, 4)
