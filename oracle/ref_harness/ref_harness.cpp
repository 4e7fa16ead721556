// C entry points over the reference's own CPU code (primes.cpp, cuckoo.h),
// compiled from the reference tree by oracle/Makefile.  Used only by tests to
// pin the oracle's FindNextPrime restatement and to run the reference's
// CuckooHashTable on its own octree-key fixtures.
#include <stdint.h>
#define LVN_ASSERT(x) ((void)0)
#include "cuckoo.h"

extern "C" {

int ref_find_next_prime(int n) { return FindNextPrime(n); }

// test_cuckoo.cpp:120-179 "CuckooHashTable (Octree data)": insert every key
// with value 42, then look every key up.  Returns inserted count; *found and
// *all42 report the lookup pass.
int ref_cuckoo_octree_keys(const uint32_t* keys, int n, int* found, int* all42) {
    CuckooHashTable table(n);
    int inserted = 0;
    for (int i = 0; i < n; i++)
        if (table.insert(keys[i], 42)) inserted++;
    int f = 0, ok = 1;
    for (int i = 0; i < n; i++) {
        uint32_t v = ~0u;
        if (table.find(keys[i], &v)) f++;
        ok = ok && v == 42;
    }
    *found = f;
    *all42 = ok;
    return inserted;
}

}
