"""The C-ABI library loads and exports every entry point include/lvn.h
declares; host-side argument checks work without a GPU (no compute calls)."""
import ctypes as C
import pathlib
import re

import pytest

import leven_gb300 as lvn

ROOT = pathlib.Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from leven_gb300 import build

    build.build()
    return lvn.lib()


def header_functions():
    text = (ROOT / "include" / "lvn.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lvn_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(lvn.EXPORTS) == names


def test_constants_match_header():
    """Every option, fault and memory-kind constant the Python binding defines
    has the value include/lvn.h gives it, and every option the header
    declares is bound."""
    text = (ROOT / "include" / "lvn.h").read_text()
    defines = {k: int(v) for k, v in re.findall(r"#define\s+(LVN_[A-Z0-9_]+)\s+(-?\d+)\b", text)}
    bound = {k: getattr(lvn, k) for k in defines if hasattr(lvn, k)}
    assert bound and all(bound[k] == defines[k] for k in bound), {k: (bound[k], defines[k]) for k in bound}
    missing = [k for k in defines if k.startswith(("LVN_OPT_", "LVN_FAULT_", "LVN_MEMORY_")) and k not in bound]
    assert not missing, missing


def test_struct_layouts():
    # byte-identical to CSGOperationInfo, MeshVertex, MeshTriangle, SeamNodeInfo
    assert C.sizeof(lvn.CsgOp) == 48
    assert C.sizeof(lvn.ChunkDesc) == 16
    assert C.sizeof(lvn.ChunkResult) == 32


def test_error_strings(lib):
    assert lvn.error_string(0) == "LVN_OK"
    assert lvn.error_string(-100) == "LVN_ERR_CAPACITY"
    assert lvn.error_string(-99999) == "LVN_ERR_CUDA"


def test_host_checks_without_device(lib):
    # before lvn_initialise nothing computes
    assert lib.lvn_meshgen_create(64) is None
    mn = (C.c_int32 * 3)(0, 0, 0)
    out = lvn.BatchOut()
    assert lib.lvn_meshgen_generate_chunks(None, None, 0, C.byref(out)) in (-101, -30)
    # operation bounds are host logic (CalcCSGOperationBounds, clipmap.cpp:1638-1643)
    op = lvn.make_op(1, 1, 201, (10.5, 20.5, -3.5), (3.0, 3.0, 3.0))
    lo, hi = lvn.csg_operation_bounds(op)
    assert lo == [26, 66, -30] and hi == [54, 94, -2]
    assert lib.lvn_store_csg_operation(C.byref(lvn.make_op(2, 0, 1, (0, 0, 0), (1, 1, 1))), mn, mn) == -30
    assert lib.lvn_store_csg_operation(C.byref(lvn.make_op(0, 0, 300, (0, 0, 0), (1, 1, 1))), mn, mn) == -30
    assert lib.lvn_clear_csg_operations() == 0
    p = lvn.DensityParams(7, 8, 0.1, 2.0, 0.5, 48.0, 6, 0.1, 2.0, 0.5, 12.0)
    assert lib.lvn_set_density(C.byref(p)) == -30


def test_workload_generator():
    from leven_gb300 import workloads as W

    # std::mt19937 default seed: the 10000th output is 4123659995
    rng = W.MT19937(5489)
    for _ in range(9999):
        rng.u32()
    assert rng.u32() == 4123659995
    wl = W.tiled_csg()
    assert len(wl.chunks) == 128 and len(wl.ops) == 32
    kinds = {(o.type, o.brush_shape) for o in wl.ops}
    assert kinds == {(1, 1), (0, 0)}
    for o in wl.ops:
        assert 0 <= o.origin[0] < 512 and -64 <= o.origin[1] < 64 and 0 <= o.origin[2] < 512
        assert all(2 <= d <= 12 for d in o.dimensions)
    assert W.op_bounds(W.Op(1, 1, 201, (10.5, 20.5, -3.5), (3.0, 3.0, 3.0))) == ([26, 66, -30], [54, 94, -2])


def test_headers_compile_and_link(tmp_path):
    """include/lvn.h as C and include/lvn_compute.hpp as C++ compile against
    liblvn.so; calls that need no device run."""
    import pathlib
    import shutil
    import subprocess

    import leven_gb300 as lvn

    root = pathlib.Path(__file__).resolve().parents[1]
    lib = lvn.LIB_PATH
    lvn.lib()
    if not shutil.which("gcc") or not shutil.which("g++"):
        pytest.skip("no host compiler")
    c_src = tmp_path / "abi.c"
    c_src.write_text(r'''
#include "lvn.h"
#include <stdio.h>
#include <string.h>
int main(void) {
    lvn_simplify_options o;
    lvn_simplify_options_default(&o);
    if (o.max_iterations != 10 || o.edge_fraction != 0.125f) return 1;
    if (strcmp(lvn_error_string(LVN_ERR_DEVICE_STATUS), "LVN_ERR_DEVICE_STATUS")) return 2;
    if (sizeof(lvn_mesh_vertex) != 48 || sizeof(lvn_seam_node) != 48 || sizeof(lvn_csg_op) != 48 ||
        sizeof(lvn_mesh_triangle) != 12 || sizeof(lvn_chunk_desc) != 16 || sizeof(lvn_chunk_result) != 32)
        return 3;
    int32_t n = 0;
    if (lvn_clipmap_select(0, -1, 0, 0, 0, 0, &n) != LVN_ERR_INVALID) return 4;
    if (lvn_render_pool_create(0, 0, 0) != 0) return 5;
    puts("c ok");
    return 0;
}
''')
    cpp_src = tmp_path / "facade.cpp"
    cpp_src.write_text(r'''
#include "lvn_compute.hpp"
#include <cstdio>
int main() {
    lvn_simplify_options o;
    lvn_simplify_options_default(&o);
    LvnMeshBuffer mesh;
    ngMeshSimplifier(&mesh, {0.f, 0.f, 0.f, 0.f}, o);  // no triangles: nothing to do
    std::vector<lvn_chunk_desc> nodes;
    if (SelectActiveClipmapNodes({0.f, 0.f, 0.f}, {0, 0, 0}, 100, nodes) != LVN_ERR_INVALID) return 1;
    std::puts(GetCLErrorString(LVN_ERR_CAPACITY));
    return 0;
}
''')
    for cc, src, std in (("gcc", c_src, "-std=c11"), ("g++", cpp_src, "-std=c++17")):
        exe = tmp_path / (src.stem + ".bin")
        subprocess.run([cc, std, "-I", str(root / "include"), str(src), str(lib), f"-Wl,-rpath,{lib.parent}", "-o",
                        str(exe)], check=True)
        out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
        assert out.returncode == 0, (src.name, out.returncode, out.stderr)
