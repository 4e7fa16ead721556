"""The oracle pinned against the reference's own known answers.

The reference's tests hold golden data only for the hash table
(leven/src/test_cuckoo.cpp:120-179, twelve octree-key fixtures) and for
RemoveDuplicates (test_compute.cpp:46-68).  FindNextPrime is pinned against
the reference's own primes.cpp compiled by oracle/Makefile where the
reference tree is mounted.
"""
import ctypes as C
import pathlib

import numpy as np
import pytest

import oracle_lib as O

GOLDEN = pathlib.Path(__file__).with_name("golden") / "octree_keys.npz"


def fixture_sets():
    data = np.load(GOLDEN)
    return {k: data[k] for k in data.files}


def test_fixture_inventory():
    sets = fixture_sets()
    assert len(sets) == 12
    assert sum(v.size for v in sets.values()) == 139943
    for name, keys in sets.items():
        assert 11000 < keys.size < 12300, name
        assert np.unique(keys).size == keys.size, f"{name} holds duplicate keys"


@pytest.mark.parametrize("name", sorted(fixture_sets()))
def test_cuckoo_octree_fixture(name):
    """test_cuckoo.cpp:120-179: every key inserts and is found with its value."""
    keys = np.ascontiguousarray(fixture_sets()[name], dtype=np.uint32)
    L = O.lib()
    retries = C.c_int32(0)
    h = L.orc_cuckoo_build(keys.ctypes.data, keys.size, 5489, C.byref(retries))
    try:
        assert L.orc_cuckoo_prime(h) == O.find_next_prime(max(2048, 2 * keys.size))
        val = C.c_uint32(0)
        for i, k in enumerate(keys.tolist()):
            assert L.orc_cuckoo_find(h, k, C.byref(val)) == 1, hex(k)
            assert val.value == i
        # keys that are not in the set are not found
        absent = np.setdiff1d(np.arange(1, 5000, dtype=np.uint32) * 7919, keys)[:200]
        for k in absent.tolist():
            assert L.orc_cuckoo_find(h, k, C.byref(val)) == 0
    finally:
        L.orc_cuckoo_free(h)


def duplicate_data(keys, seed):
    """gen_duplicate_data.py logic: each line of eight keys repeated 1-5 times."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(0, keys.size, 8):
        out.extend([keys[i:i + 8]] * int(rng.integers(1, 6)))
    return np.concatenate(out).astype(np.int32)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_remove_duplicates_fixture(seed):
    """test_compute.cpp:46-68: RemoveDuplicates of the duplicated OCTREE_KEYS_3
    equals OCTREE_KEYS_3 as a sorted set."""
    keys = fixture_sets()["OCTREE_KEYS_3"].astype(np.int32)
    dup = duplicate_data(keys, seed)
    assert dup.size > keys.size
    uniq = O.remove_duplicates(dup)
    assert uniq.size == keys.size
    assert np.array_equal(np.sort(uniq), np.sort(keys))


def test_remove_duplicates_edge_cases():
    assert O.remove_duplicates(np.zeros(0, np.int32)).size == 0
    assert O.remove_duplicates(np.full(1000, 7, np.int32)).tolist() == [7]
    v = np.arange(5000, dtype=np.int32)
    assert np.array_equal(np.sort(O.remove_duplicates(np.concatenate([v, v[::-1]]))), v)


@pytest.fixture(scope="module")
def ref_lib():
    if not O.REF_SO.exists():
        pytest.skip("reference harness not built here (needs the reference tree)")
    L = C.CDLL(str(O.REF_SO))
    L.ref_find_next_prime.argtypes = [C.c_int]
    L.ref_cuckoo_octree_keys.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    return L


def test_find_next_prime_matches_reference(ref_lib):
    ns = list(range(0, 5000)) + list(range(5000, 2_000_000, 997)) + [2048, 4096, 823875 * 2, 262144 * 2]
    for n in ns:
        assert O.find_next_prime(n) == ref_lib.ref_find_next_prime(n), n


@pytest.mark.parametrize("name", sorted(fixture_sets()))
def test_reference_cpu_cuckoo_on_fixture(ref_lib, name):
    """The reference's own CuckooHashTable (cuckoo.h) passes its fixture test
    here, so the fixtures are read correctly."""
    keys = np.ascontiguousarray(fixture_sets()[name], dtype=np.uint32)
    found, all42 = C.c_int(0), C.c_int(0)
    inserted = ref_lib.ref_cuckoo_octree_keys(keys.ctypes.data, keys.size, C.byref(found), C.byref(all42))
    assert inserted == keys.size and found.value == keys.size and all42.value == 1
