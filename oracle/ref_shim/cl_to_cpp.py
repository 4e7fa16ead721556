"""Build step of the reference harness (test infrastructure): makes the
reference's OpenCL C sources compilable as C++ against cl_shim.h.

The one OpenCL C construct C++ cannot parse is the vector literal
`(float3)(a, b, c)` (C++ reads it as a cast of a comma expression).  This
rewrites each vector literal `(TYPEn)(` as the constructor call `TYPEn(` and
writes the result under the output directory, keeping file names, so that the
sources' own `#include "cl/..."` lines resolve there.  Nothing else changes.
The output is a build product (oracle/_ref/, git-ignored); the reference's
sources are read where they lie.

    python oracle/ref_shim/cl_to_cpp.py <reference cl directory> <output cl directory>
"""
import pathlib
import re
import sys

VECTOR_LITERAL = re.compile(r"\(\s*((?:u?char|u?short|u?int|u?long|float|double)(?:2|3|4|8|16))\s*\)\s*\(")


def convert(text: str) -> str:
    return VECTOR_LITERAL.sub(lambda m: m.group(1) + "(", text)


def main(src: str, dst: str) -> None:
    out = pathlib.Path(dst)
    out.mkdir(parents=True, exist_ok=True)
    for path in sorted(pathlib.Path(src).iterdir()):
        if path.suffix in (".cl", ".glsl"):
            (out / path.name).write_text(convert(path.read_text()))


if __name__ == "__main__":
    if len(sys.argv) != 3:
        sys.exit("usage: cl_to_cpp.py <reference cl directory> <output cl directory>")
    main(sys.argv[1], sys.argv[2])
