"""The FLOP figures of the bench's FP32 roofline against the oracle's own
operation count (orc_flop_counts: the restated density and edge arithmetic
run on a counting scalar; add, sub, mul, div, sqrt and floor count 1, an fma
counts 2, compares, min / max and abs are free, every simplex corner is
taken, as the branch-free kernels compute them)."""
import bench
import oracle_lib as O


def test_height_and_cave_terms():
    h, p, *_ = O.flop_counts(O.density(mode=1))
    assert (h, p) == (bench.FLOP_HEIGHT8, 2)
    h, p, *_ = O.flop_counts(O.density(mode=2))
    assert (h, p) == (bench.FLOP_HEIGHT8, 2 + bench.FLOP_CAVES6)


def test_edge_arithmetic():
    # the oracle's FindEdgeIntersectionInfo evaluates every one of its 23
    # density samples in full, height term included
    for mode in (1, 2):
        h, p, ex, ey, ez = O.flop_counts(O.density(mode=mode))
        assert ex == ey == ez == 23 * (h + p) + bench.FLOP_EDGE_EXTRA


def test_kernel_edge_work_follows_the_count():
    h, p = bench.density_flops(type("W", (), {"density": {"mode": 2, "octaves2": 8, "octaves3": 6}}))
    xz, y = bench.hermite_edge_flops(h, p)
    full = O.flop_counts(O.density(mode=2))[2]
    # the kernel skips only height terms: 4 of an x / z edge's 23, 19 of a y edge's
    assert full - xz == 4 * h and full - y == 19 * h
