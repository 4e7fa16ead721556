"""lvn_meshgen_generate_chunks_async / lvn_meshgen_wait: two contexts with a
batch in flight each, writing pinned host arrays, give byte for byte the
synchronous call's meshes; a second batch on a busy context is refused."""
import ctypes as C

import numpy as np
import pytest

from leven_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def host_out(lvn, torch, cap_v, cap_t, cap_s, results):
    hv = torch.zeros(cap_v * 12, dtype=torch.float32).pin_memory()
    ht = torch.zeros(cap_t * 3, dtype=torch.int32).pin_memory()
    hs = torch.zeros(cap_s * 12, dtype=torch.int32).pin_memory()
    bo = lvn.BatchOut(lvn.LVN_MEMORY_HOST, hv.data_ptr(), cap_v, 0, ht.data_ptr(), cap_t, 0, hs.data_ptr(), cap_s, 0,
                      C.cast(results, C.POINTER(lvn.ChunkResult)))
    return bo, (hv, ht, hs)


@pytest.mark.parametrize("host_writes,order", [(1, 0), (0, 0), (0, 1), (1, 1)])
def test_two_batches_in_flight_match_the_synchronous_call(lvn_gpu, host_writes, order):
    """host_writes 1: the kernels write the pinned arrays; 0: device pools and
    a copy-engine transfer (LVN_OPT_HOST_WRITES).  order 1: both contexts'
    kernels in the device-wide order (LVN_OPT_COMPUTE_ORDER)."""
    torch = pytest.importorskip("torch")
    lvn = lvn_gpu
    wl = W.tiled_csg(4, 2, 4, n_ops=16, seed=11)
    lvn.set_density(**wl.density)
    lvn.clear_csg_operations()
    for op in wl.ops:
        lvn.store_csg_operation(lvn.make_op(op.type, op.brush_shape, op.material, op.origin, op.dimensions))
    halves = [wl.chunks[:16], wl.chunks[16:]]
    ref = lvn.MeshGen(64)
    ctx = [lvn.MeshGen(64), lvn.MeshGen(64)]
    try:
        ref.set_option(lvn.LVN_OPT_CACHE, 0)
        want = [ref.generate_chunks(h) for h in halves]
        keep = []
        for k, h in enumerate(halves):
            ctx[k].set_option(lvn.LVN_OPT_CACHE, 0)
            ctx[k].set_option(lvn.LVN_OPT_HOST_WRITES, host_writes)
            ctx[k].set_option(lvn.LVN_OPT_COMPUTE_ORDER, order)
        for rnd in range(2):  # two rounds, so each context runs a second batch after its wait
            outs = []
            for k, h in enumerate(halves):
                n = len(h)
                descs = (lvn.ChunkDesc * n)(*[lvn.ChunkDesc((C.c_int32 * 3)(*mn), s) for mn, s in h])
                results = (lvn.ChunkResult * n)()
                V, T, S, _ = want[k]
                bo, arrays = host_out(lvn, torch, V.shape[0] + 8, T.shape[0] + 8, S.shape[0] + 8, results)
                keep.append((descs, results, bo, arrays))
                assert ctx[k].generate_chunks_async_raw(descs, n, bo) == 0
                if rnd == 0 and k == 0:
                    assert ctx[0].generate_chunks_async_raw(descs, n, bo) == lvn.LVN_ERR_INVALID
                outs.append((bo, arrays, results, n))
            for k, (bo, arrays, results, n) in enumerate(outs):
                assert ctx[k].wait() == 0
                V, T, S, res = want[k]
                hv, ht, hs = arrays
                assert (bo.total_vertices, bo.total_triangles, bo.total_seams) == (V.shape[0], T.shape[0], S.shape[0])
                assert np.array_equal(hv.numpy().reshape(-1, 12)[:V.shape[0]].view(np.int32), V.view(np.int32))
                assert np.array_equal(ht.numpy().reshape(-1, 3)[:T.shape[0]], T)
                assert np.array_equal(hs.numpy().reshape(-1, 12)[:S.shape[0]], S)
                got = np.ctypeslib.as_array(C.cast(results, C.POINTER(C.c_int32)), shape=(n, 8))
                assert np.array_equal(got, res)
        assert ctx[0].wait() == 0  # nothing in flight
        # a context closed while it was the last in the order leaves the order
        # empty; the next ordered batch waits on nothing
        ctx[1].close()
        V, T, S, res = ctx[0].generate_chunks(halves[0])
        assert np.array_equal(V.view(np.int32), want[0][0].view(np.int32))
    finally:
        ref.close()
        for c in ctx:
            c.close()
        lvn.clear_csg_operations()
