"""The FP32 leaf solve against its FP64 restatement (the oracle's qef64_solve).

qef_solve (qef.cl:239-256) is an FP32 ATA / ATb Jacobi-SVD pseudo-inverse
with mass-point bias.  The oracle repeats it in double from the same crossing
points and normals; the distance between the two vertices, in the chunk's
voxels, is the FP32 solve's error.  The CUDA leaves reproduce the oracle's
FP32 vertices bit for bit (tests/test_gpu_parity.py), so the bound holds for
them too; tests/test_gpu_workloads.py checks the GPU's vertices directly.
"""
import numpy as np
import pytest

import oracle_lib as O
from leven_gb300 import workloads as W

# max |x_fp32 - x_fp64| over every leaf checked, in voxels of its chunk
QEF_FP64_BOUND = 1e-3


def chunk_errors(mode, mn, size, ops=()):
    O.set_seed(1)
    ch = O.OracleChunk(O.density(mode=mode), mn, size, vpc=64, ops=[op.as_tuple() for op in ops])
    return ch.qef_fp64_error_voxels(), ch


@pytest.mark.parametrize("mode,mn,size", [(1, (0, 128, 0), 256), (2, (0, 0, 0), 256),
                                          (2, (1024, -1024, 0), 1024), (1, (-2048, -2048, 4096), 4096)])
def test_fp32_solve_within_bound_of_fp64(mode, mn, size):
    err, ch = chunk_errors(mode, mn, size)
    assert err.size > 0
    assert err.max() <= QEF_FP64_BOUND, err.max()
    assert err.mean() <= 1e-4
    # the FP64 record carries each leaf's crossing count (1..12)
    n = ch.positions_f64()[:, 3]
    assert n.min() >= 1 and n.max() <= 12


def test_fp64_solve_with_csg():
    wl = W.tiled_csg(2, 2, 2, n_ops=12, seed=3)
    worst = 0.0
    for mn, size in wl.chunks:
        err, _ = chunk_errors(1, mn, size, W.ops_for_chunk(wl.ops, mn, size))
        if err.size:
            worst = max(worst, float(err.max()))
    assert worst <= QEF_FP64_BOUND
