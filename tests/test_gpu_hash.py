"""The device cuckoo hash (Cuckoo_InsertKeys / Cuckoo_Find, cuckoo.cl:26-104)
on the reference's own golden key sets, a forced stash, the reference's stash
lookup, and the host-side failure paths of the meshing calls.

The reference's only golden data on the hot path are the twelve octree-key
sets of its cuckoo test (leven/src/test_cuckoo.cpp:120-179: every key
inserts, every key is found with its value).  They go through the same
cuckoo_insert and HashView::find that the meshing stages run, via the
lvn_debug_cuckoo test hook.

Failure injection is host-side (lvn_debug_inject_fault): an allocation that
reports out-of-memory and a degenerate hash family; no GPU fault is made.
"""
import pathlib

import numpy as np
import pytest

import oracle_lib as O
from leven_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).with_name("golden") / "octree_keys.npz"
EMPTY = np.uint64(0xFFFFFFFFFFFFFFFF)


def fixture_sets():
    data = np.load(GOLDEN)
    return {k: data[k] for k in data.files}


def entries(table):
    """(key, value) pairs held in a table + stash dump."""
    t = table[table != EMPTY]
    return set(zip((t & np.uint64(0xFFFFFFFF)).astype(np.int64).tolist(), (t >> np.uint64(32)).astype(np.int64).tolist()))


@pytest.mark.parametrize("name", sorted(fixture_sets()))
def test_octree_key_fixture_on_device_hash(lvn_gpu, name):
    """test_cuckoo.cpp:120-179 on the device table: every key inserts and is
    found with its index; the table and stash hold exactly the (key, index)
    pairs; the table size is FindNextPrime(max(2048, 2n)) as the oracle's."""
    lvn = lvn_gpu
    keys = fixture_sets()[name]
    vals, info, table = lvn.debug_cuckoo(keys, with_table=True)
    prime, stash_used, draws, failed = info
    assert failed == 0 and draws >= 1
    assert prime == O.find_next_prime(max(2048, 2 * keys.size))
    assert np.array_equal(vals, np.arange(keys.size, dtype=np.uint32)), "a key not found with its index"
    assert entries(table) == set(zip(keys.astype(np.int64).tolist(), range(keys.size)))
    # a second build (new parameter draws) gives the same answers
    vals2, _, _ = lvn.debug_cuckoo(keys)
    assert np.array_equal(vals2, np.arange(keys.size, dtype=np.uint32))


def test_forced_stash_and_reference_stash_lookup(lvn_gpu):
    """A table smaller than the key count sends keys to the 101-entry stash:
    this library's lookup finds them (the stash probe reads the stash), while
    the reference's Cuckoo_Find as written (cuckoo.cl:93-101, the probe reads
    data[h]) misses exactly the stashed keys."""
    lvn = lvn_gpu
    sets = fixture_sets()
    keys = sets[sorted(sets)[0]][:12].copy()
    prime = 11  # 12 keys in 11 slots: at least one key is stashed
    vals, info, table = lvn.debug_cuckoo(keys, prime=prime, with_table=True)
    assert info[0] == prime and info[1] == 1 and info[3] == 0, info
    assert np.array_equal(vals, np.arange(keys.size, dtype=np.uint32))
    stash = table[prime:]
    stashed = {k for k, _ in entries(stash)}
    assert len(stashed) >= keys.size - prime
    assert entries(table) == set(zip(keys.astype(np.int64).tolist(), range(keys.size)))
    # the reference's lookup on a fresh table: stashed keys are lost
    rvals, rinfo, rtable = lvn.debug_cuckoo(keys, prime=prime, reference_find=True, with_table=True)
    assert rinfo[1] == 1 and rinfo[3] == 0
    rstashed = {k for k, _ in entries(rtable[prime:])}
    for i, k in enumerate(keys.tolist()):
        if k in rstashed:
            assert rvals[i] == 0xFFFFFFFF, "the reference's stash probe cannot see the stash"
        else:
            assert rvals[i] == i


def test_debug_cuckoo_rejects_bad_arguments(lvn_gpu):
    lvn = lvn_gpu
    with pytest.raises(lvn.LvnError):
        lvn.debug_cuckoo(np.zeros(0, np.uint32))
    with pytest.raises(lvn.LvnError):
        lvn.debug_cuckoo(np.arange(4, dtype=np.uint32), prime=1)


def test_injected_hash_family_fails_after_bounded_retries(lvn_gpu):
    """A parameter family under which no table holds three keys: the meshing
    call gives up with LVN_ERR_HASH after its bounded retries (the reference
    retries without bound, compute_cuckoo.cpp:86-132), and the next call with
    normal draws meshes the chunk as the oracle does."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    lvn.clear_csg_operations()
    mg = lvn.MeshGen(64)
    try:
        mg.set_option(lvn.LVN_OPT_CACHE, 0)
        lvn.inject_fault(lvn.LVN_FAULT_HASH_FAMILY, 1000)
        with pytest.raises(lvn.LvnError) as e:
            mg.generate_chunk_mesh((0, 128, 0), 256)
        assert e.value.code == lvn.LVN_ERR_HASH
        with pytest.raises(lvn.LvnError) as e:
            lvn.debug_cuckoo(np.arange(1, 64, dtype=np.uint32))
        assert e.value.code == lvn.LVN_ERR_HASH
        lvn.inject_fault(lvn.LVN_FAULT_NONE, 0)
        mesh = mg.generate_chunk_mesh((0, 128, 0), 256)
        O.set_seed(1)
        ref = O.OracleChunk(O.density(mode=1), (0, 128, 0), 256, vpc=64)
        assert np.array_equal(mesh.triangles, ref.triangles())
    finally:
        lvn.inject_fault(lvn.LVN_FAULT_NONE, 0)
        mg.close()


def test_injected_allocation_failure(lvn_gpu):
    """A device allocation that fails as cudaMalloc's out-of-memory does: the
    batch call returns LVN_ERR_OUT_OF_MEMORY, and the same context meshes the
    batch correctly once allocations succeed again."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    lvn.clear_csg_operations()
    chunks = [((0, 128, 0), 256), ((256, 128, 0), 256)]
    mg = lvn.MeshGen(64)
    try:
        mg.set_option(lvn.LVN_OPT_CACHE, 0)
        lvn.inject_fault(lvn.LVN_FAULT_DEVICE_ALLOC, 1)
        with pytest.raises(lvn.LvnError) as e:
            mg.generate_chunks(chunks)
        assert e.value.code == lvn.LVN_ERR_OUT_OF_MEMORY
        lvn.inject_fault(lvn.LVN_FAULT_NONE, 0)
        V, T, S, res = mg.generate_chunks(chunks)
        O.set_seed(1)
        for c, (mn, size) in enumerate(chunks):
            ref = O.OracleChunk(O.density(mode=1), mn, size, vpc=64)
            r = res[c]
            assert np.array_equal(T[r[2]:r[2] + r[3]], ref.triangles())
    finally:
        lvn.inject_fault(lvn.LVN_FAULT_NONE, 0)
        mg.close()


def test_device_table_repair(lvn_gpu):
    """A failed cuckoo insert is repaired inside the batch: with every host
    draw of parameters degenerate (no table holds three keys) and the batch's
    device-side repair left its own draws, each chunk's edge and leaf tables
    are rebuilt on the device, and the meshes equal the oracle's bit for bit,
    through the batch call and the single-chunk call.  Without the repair the
    call could only end in LVN_ERR_HASH (previous test)."""
    lvn = lvn_gpu
    lvn.set_density(**W.FBM2D)
    lvn.clear_csg_operations()
    chunks = [((0, 128, 0), 256), ((256, 128, 0), 256), ((0, -128, 256), 256), ((256, 0, 256), 256)]
    mg = lvn.MeshGen(64)
    try:
        mg.set_option(lvn.LVN_OPT_CACHE, 0)
        lvn.inject_fault(lvn.LVN_FAULT_HASH_FAMILY_HOST, 1 << 20)
        V, T, S, res = mg.generate_chunks(chunks)
        one = mg.generate_chunk_mesh(chunks[0][0], chunks[0][1])
        lvn.inject_fault(lvn.LVN_FAULT_NONE, 0)
        O.set_seed(1)
        for c, (mn, size) in enumerate(chunks):
            ref = O.OracleChunk(O.density(mode=1), mn, size, vpc=64)
            r = res[c]
            nv = ref.mesh_vertex_count()
            assert r[1] == nv > 0
            assert np.array_equal(V[r[0]:r[0] + nv].view(np.int32), ref.vertices()[:nv].view(np.int32)), c
            assert np.array_equal(T[r[2]:r[2] + r[3]], ref.triangles()), c
            assert np.array_equal(S[r[4]:r[4] + r[5]][:, :4], ref.seams()[:, :4]), c
            if c == 0:
                assert np.array_equal(one.triangles, ref.triangles())
    finally:
        lvn.inject_fault(lvn.LVN_FAULT_NONE, 0)
        mg.close()
