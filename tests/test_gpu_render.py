"""Device-resident render meshes (the headless stand-in for the engine's GL
upload, render_mesh.cpp:94-138): a batch's chunk meshes gathered into a pool
in one launch read back byte for byte; empty meshes get no render mesh;
freed ranges are reused; exhaustion takes nothing."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def device_batch(lvn, chunks):
    import torch

    lvn.clear_csg_operations()
    lvn.set_density(mode=lvn.LVN_DENSITY_FBM2D)
    g = lvn.MeshGen(64)
    hv, ht, _, hres = g.generate_chunks(chunks)  # host reference
    cap_v, cap_t, cap_s = len(hv) + 64, len(ht) + 64, 1 << 16
    dv = torch.empty((cap_v, 12), dtype=torch.float32, device="cuda")
    dt = torch.empty((cap_t, 3), dtype=torch.int32, device="cuda")
    ds = torch.empty((cap_s, 12), dtype=torch.int32, device="cuda")
    n = len(chunks)
    descs = (lvn.ChunkDesc * n)()
    for i, (mn, size) in enumerate(chunks):
        descs[i] = lvn.ChunkDesc((C.c_int32 * 3)(*mn), size)
    results = (lvn.ChunkResult * n)()
    bo = lvn.BatchOut(lvn.LVN_MEMORY_DEVICE, dv.data_ptr(), cap_v, 0, dt.data_ptr(), cap_t, 0, ds.data_ptr(), cap_s, 0,
                      C.cast(results, C.POINTER(lvn.ChunkResult)))
    assert g.generate_chunks_raw(descs, n, bo) == 0
    torch.cuda.synchronize()
    g.close()
    return bo, (dv, dt, ds, results), hv, ht, hres


def test_batch_into_pool(lvn_gpu):
    lvn = lvn_gpu
    chunks = [((x * 256, 128, z * 256), 256) for x in range(3) for z in range(2)] + [((0, 4096, 0), 256)]  # last: empty
    bo, keep, hv, ht, hres = device_batch(lvn, chunks)
    pool = lvn.RenderPool(1 << 20, 1 << 21, 64)
    try:
        pos = np.array([[mn[0] + 128.0, mn[1] + 128.0, mn[2] + 128.0] for mn, _ in chunks], np.float32)
        handles = pool.from_batch(bo, len(chunks), pos)
        has = hres[:, 3] > 0  # a chunk without triangles gets no render mesh
        assert handles[-1] == -1 and np.array_equal(handles >= 0, has) and has.sum() >= 4
        for c, h in enumerate(handles):
            if h < 0:
                continue
            vo, nv, to, nt = hres[c, :4]
            v, t = pool.download(h)
            assert np.array_equal(v.view(np.int32), hv[vo:vo + nv].view(np.int32))
            assert np.array_equal(t, ht[to:to + nt])
            view = pool.view(h)
            assert view.num_vertices == nv and view.num_triangles == nt and view.vertices
            assert tuple(view.position) == tuple(pos[c])
        used_v, used_t, meshes = pool.usage()
        assert meshes == has.sum() and used_v == hres[has, 1].sum() and used_t == hres[has, 3].sum()
        # free two, upload one from the host into the freed ranges
        live = np.flatnonzero(has)
        pool.free(handles[live[0]])
        pool.free(handles[live[1]])
        vo, nv, to, nt = hres[live[0], :4]
        h = pool.upload(hv[vo:vo + nv], ht[to:to + nt], pos[live[0]])
        v, t = pool.download(h)
        assert np.array_equal(v.view(np.int32), hv[vo:vo + nv].view(np.int32)) and np.array_equal(t, ht[to:to + nt])
        assert pool.upload(hv[:10], np.zeros((0, 3), np.int32)) == -1  # no triangles, no render mesh
        stale = [x for x in (handles[live[0]], handles[live[1]]) if x != h]
        assert len(stale) == 1  # the upload reused one of the two freed handles
        with pytest.raises(lvn.LvnError):
            pool.free(stale[0])  # already freed
    finally:
        pool.close()


def test_pool_exhaustion_takes_nothing(lvn_gpu):
    lvn = lvn_gpu
    chunks = [((x * 256, 128, 0), 256) for x in range(4)]
    bo, keep, hv, ht, hres = device_batch(lvn, chunks)
    has = hres[:, 3] > 0
    pool = lvn.RenderPool(int(hres[has, 1].sum()) - 1, 1 << 20, 16)  # one vertex short
    try:
        with pytest.raises(lvn.LvnError):
            pool.from_batch(bo, len(chunks))
        assert pool.usage() == (0, 0, 0)
        last = np.flatnonzero(has)[-1]
        handles = pool.from_batch(bo, int(last))  # the chunks before the last one with triangles fit
        assert np.array_equal(handles >= 0, has[:last])
    finally:
        pool.close()
