"""The edge-collapse simplification (ngMeshSimplifier, ng_mesh_simplify.cpp:
441-540) on the CPU: the oracle's restatement, and the random edge draws the
GPU takes from a precomputed std::mt19937(42) stream.

The reference ships no simplifier fixtures, its QEF uses _mm_rsqrt_ps (whose
result differs between x86 implementations) and its draws depend on the
standard library it was built with, so parity is pinned here to libstdc++'s
own uniform_int_distribution and otherwise "unpinned" against the reference.
"""
import numpy as np
import pytest

import oracle_lib as O
from leven_gb300 import workloads as W


def raw_stream(n):
    g = W.MT19937(42)
    return np.array([g.u32() for _ in range(n)], np.uint64)


@pytest.mark.parametrize("hi", [0, 1, 2, 6, 99, 1000, 4095, 4096, 12345, 65535, 99991, (1 << 20) + 7,
                                (1 << 31) - 2])
def test_draws_match_libstdcxx(hi):
    """Lemire's method over the raw stream (the kernel's formulation): keep a
    raw value when the low half of raw * range is at least (2^32 - range) mod
    range, and return the high half."""
    n = 2000
    rng = hi + 1
    raw = raw_stream(3 * n)
    prod = raw * np.uint64(rng)
    low = prod & np.uint64(0xFFFFFFFF)
    threshold = np.uint64(((1 << 32) - rng) % rng)
    kept = (prod >> np.uint64(32))[low >= threshold][:n]
    assert np.array_equal(kept.astype(np.int64), O.uniform_draws(hi, n).astype(np.int64))


@pytest.fixture(scope="module")
def meshes():
    O.set_seed(1)
    out = []
    for mode, mn, size, vpc in [(1, (0, 128, 0), 256, 64), (2, (0, 0, 0), 256, 64), (2, (512, -512, 0), 512, 32),
                                (1, (0, 0, 256), 256, 16)]:
        ch = O.OracleChunk(O.density(mode=mode), mn, size, vpc=vpc)
        nv = ch.mesh_vertex_count()
        out.append((mn, size, ch.vertices()[:nv].copy(), ch.triangles().copy()))
    return out


def test_simplified_meshes_are_valid(meshes):
    for mn, size, v, t in meshes:
        sv, st = O.mesh_collapse(v, t, O.node_offset(mn, size), O.simplify_options(size))
        if len(t) >= 100 and len(v) >= 100:
            assert len(st) < len(t)
        assert len(st) and st.min() >= 0 and st.max() < len(sv)
        assert not ((st[:, 0] == st[:, 1]) | (st[:, 0] == st[:, 2]) | (st[:, 1] == st[:, 2])).any()
        used = np.zeros(len(sv), bool)
        used[st.ravel()] = True
        assert used.all()  # CompactVertices keeps only referenced vertices
        assert np.isfinite(sv).all() and (sv[:, 3] == 1.0).all()


def test_small_meshes_unchanged(meshes):
    mn, size, v, t = meshes[0]
    sv, st = O.mesh_collapse(v[:99], t[:50], O.node_offset(mn, size), O.simplify_options(size))
    assert np.array_equal(sv, v[:99]) and np.array_equal(st, t[:50])


def test_no_iterations_roundtrips_offset(meshes):
    """max_iterations 0: only the offset round trip and the vertex compaction."""
    mn, size, v, t = meshes[0]
    opt = O.simplify_options(size)
    opt[1] = 0
    sv, st = O.mesh_collapse(v, t, O.node_offset(mn, size), opt)
    assert len(st) == len(t)
    off = O.node_offset(mn, size)
    assert np.allclose(sv[:, :3], v[np.unique(t)][:, :3], atol=1e-4)
    assert np.array_equal(sv[:, :3], (v[np.unique(t)][:, :3] - off[:3]) + off[:3])
