"""Generates the committed golden fixtures from the reference's test data.

Reads the twelve octree-key fixtures that the reference's cuckoo tests use
(leven/src/testdata/octree_keys_*.cpp, consumed by test_cuckoo.cpp:120-179)
and writes them, unchanged, to tests/golden/octree_keys.npz as uint32 arrays
without the ~0 terminator.  Run it where the reference tree is mounted, with
the reference checkout's root as the argument:

    python tests/golden/make_golden.py <reference checkout>
"""
import pathlib
import re
import sys

import numpy as np


def main(ref_root: str) -> None:
    src = pathlib.Path(ref_root) / "leven" / "src" / "testdata"
    out = {}
    for path in sorted(src.glob("octree_keys_*.cpp")):
        text = path.read_text()
        name = re.search(r"OCTREE_KEYS_(\d+)", text).group(0)
        body = text[text.index("{") + 1: text.rindex("}")]
        assert body.rstrip().endswith("~0"), path  # the ~0 terminator
        vals = [int(v, 16) for v in re.findall(r"0x[0-9a-fA-F]+", body)]
        out[name] = np.asarray(vals, dtype=np.uint32)
    dst = pathlib.Path(__file__).with_name("octree_keys.npz")
    np.savez_compressed(dst, **out)
    print(f"wrote {dst} ({len(out)} sets, {sum(v.size for v in out.values())} keys)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout root>")
    main(sys.argv[1])
