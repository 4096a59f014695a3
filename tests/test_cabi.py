"""The C-ABI library loads and exports every function include/meshode.h
declares (no compute: this runs without a GPU)."""
import ctypes
import os
import re

from meshode_gb300 import _lib as L
from meshode_gb300 import build as B

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "meshode.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:[A-Za-z_][A-Za-z0-9_]*[\s*]+)+(mo_[A-Za-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_builds_and_exports_header_symbols():
    B.build()
    lib = ctypes.CDLL(L.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(declared_functions()) == set(L.exported_symbols())


def test_struct_layout_matches_library():
    B.build()
    a, b = ctypes.c_size_t(), ctypes.c_size_t()
    L.call("mo_abi_sizes", ctypes.byref(a), ctypes.byref(b))
    assert a.value == ctypes.sizeof(L.MoPair)
    assert b.value == ctypes.sizeof(L.MoTile)


def test_host_side_queries_without_gpu():
    B.build()
    lib = L.lib()
    assert lib.mo_version() >= 100
    assert lib.mo_grid_bytes(64, L.MO_LAYOUT_LINEAR) == 64 ** 3 * 4
    assert lib.mo_grid_bytes(64, L.MO_LAYOUT_CELL) == 63 ** 3 * 32
    assert lib.mo_grid_bytes(64, 7) == 0
    assert lib.mo_edge_count(10, L.MO_EDGES_FACES) == 30
    assert lib.mo_edge_count(10, L.MO_EDGES_LIST) == 10
    assert lib.mo_edge_count(10, 5) == -1
    assert lib.mo_df_method_for(20, 64) == L.MO_DF_BRUTE
    assert lib.mo_df_method_for(1_310_720, 256) == L.MO_DF_LBVH
    assert lib.mo_df_build_scratch_bytes(1000, 2000, 64, L.MO_DF_LBVH) > 2000 * 64
    assert lib.mo_edge_csr_bytes(100, 50, L.MO_EDGES_FACES) >= 4 * (101 + 4 * 150)


def test_argument_errors_are_reported_without_gpu():
    B.build()
    lib = L.lib()
    rc = lib.mo_dfloss_forward(None, 10, None, 64, L.MO_LAYOUT_LINEAR, None, None)
    assert rc == L.MO_ERR_INVALID
    assert b"null" in lib.mo_last_error()
    rc = lib.mo_dfloss_backward(None, 10, None, 1, L.MO_LAYOUT_LINEAR, None, None)
    assert rc == L.MO_ERR_INVALID and b"resolution" in lib.mo_last_error()
    rc = lib.mo_df_build(None, 0, None, 0, 64, None, 0, None, 0, None, None, None)
    assert rc == L.MO_ERR_INVALID
    rc = lib.mo_edge_offsets(None, 10, None, 5, 9, None, None)
    assert rc == L.MO_ERR_INVALID and b"kind" in lib.mo_last_error()


STRUCTS = {"MoPair": L.MoPair, "MoTile": L.MoTile, "MoDfOptions": L.MoDfOptions,
           "MoPoolConfig": L.MoPoolConfig, "MoRequest": L.MoRequest, "MoPoolStats": L.MoPoolStats}


def test_struct_offsets_match_c_compiler(tmp_path):
    """Every field offset and struct size of the ctypes mirror equals what a C
    compiler makes of include/meshode.h."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "meshode.h"', "int main(void) {"]
    for name, cls in STRUCTS.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for fname, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, fname, name, fname))
    lines.append("return 0; }")
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "abi"
    subprocess.run([cc, "-std=c99", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                         check=True).stdout.splitlines())
    for name, cls in STRUCTS.items():
        assert int(out[name]) == ctypes.sizeof(cls), name
        for fname, _ in cls._fields_:
            assert int(out["%s.%s" % (name, fname)]) == getattr(cls, fname).offset, (name, fname)


def test_pool_argument_errors_without_gpu():
    B.build()
    lib = L.lib()
    assert lib.mo_pool_create(None, None) == L.MO_ERR_INVALID
    cfg = L.MoPoolConfig(max_pairs=0, max_tiles=10, group_steps=5)
    out = ctypes.c_void_p()
    assert lib.mo_pool_create(ctypes.byref(cfg), ctypes.byref(out)) == L.MO_ERR_INVALID
    assert b"sizes" in lib.mo_last_error() and not out.value
    cfg = L.MoPoolConfig(max_pairs=4, max_tiles=10, group_steps=5, layout=9)
    assert lib.mo_pool_create(ctypes.byref(cfg), ctypes.byref(out)) == L.MO_ERR_INVALID
    assert b"layout" in lib.mo_last_error()
    req = L.MoRequest()
    nid = ctypes.c_int64()
    assert lib.mo_pool_submit(None, ctypes.byref(req), ctypes.byref(nid)) == L.MO_ERR_INVALID
    assert lib.mo_pool_progress(None, 0, None) == L.MO_ERR_INVALID
    assert lib.mo_pool_destroy(None) == L.MO_OK
    cfg = L.MoPoolConfig(max_pairs=4, max_tiles=10, group_steps=5, df_mode=7)
    assert lib.mo_pool_create(ctypes.byref(cfg), ctypes.byref(out)) == L.MO_ERR_INVALID
    assert b"df_mode" in lib.mo_last_error()
    assert lib.mo_pool_fill_totals(None, None) == L.MO_ERR_INVALID


def test_distance_field_entry_points_check_arguments_without_gpu():
    """The tree-only build, the on-demand fills and the packet shapes are
    checked on the host before anything runs."""
    B.build()
    lib = L.lib()
    assert lib.mo_df_tree_bytes(0) == 0
    assert lib.mo_df_tree_bytes(3) == 16 * (16 + 8 * 2)  # 15 triangle float4 padded to 16, two 128 B nodes
    assert lib.mo_df_tree_scratch_bytes(-1, 3) == 0
    assert lib.mo_df_tree_build(None, 10, None, 4, None, None, 0, None, None, None) == L.MO_ERR_INVALID
    assert b"null" in lib.mo_last_error()
    # child ids are index << 3 | bucket size: at most 2^27 triangles in a tree
    assert lib.mo_df_tree_build(None, 10, None, (1 << 27) + 1, None, None, 0, None, None, None) == L.MO_ERR_INVALID
    assert b"too large" in lib.mo_last_error()
    opt = L.MoDfOptions(L.MO_DF_LBVH, L.MO_PACKET_4x4x2, 0.0)
    dummy = (ctypes.c_double * 4)()  # never read: the size is refused first
    p = ctypes.cast(dummy, ctypes.c_void_p)
    rc = lib.mo_df_build_ex(p, 10, p, (1 << 27) + 1, 64, p, ctypes.byref(opt), None, 0, p, None, None)
    assert rc == L.MO_ERR_INVALID and b"too large for the LBVH" in lib.mo_last_error()
    assert lib.mo_df_lazy_bytes(1) == 0 and lib.mo_df_lazy_bytes(L.MO_DF_LAZY_MAX_N + 1) == 0
    assert lib.mo_df_lazy_seed(None, 0, None, -1, None, None, None, 0, None) == L.MO_ERR_INVALID
    assert lib.mo_df_lazy_seed(None, 0, None, 0, None, None, None, 0, None) == L.MO_OK  # nothing to seed
    assert lib.mo_df_lazy_fill(None, None, None, None, -1, None, None) == L.MO_ERR_INVALID
    assert lib.mo_df_lazy_fill(None, None, None, None, 1 << 28, None, None) == L.MO_ERR_INVALID
    opt = L.MoDfOptions(L.MO_DF_LBVH, L.MO_PACKET_2x4x4_TRI2 + 1, 0.0)
    rc = lib.mo_df_build_ex(None, 10, None, 4, 64, None, ctypes.byref(opt), None, 0, None, None, None)
    assert rc == L.MO_ERR_INVALID and b"packet" in lib.mo_last_error()
    assert lib.mo_fused_step_on_demand(None, None, None, 4, 0, None, 0, None) == L.MO_ERR_INVALID


def test_noalloc_capacity_matches_documented_figure():
    """The header documents that mo_df_build_noalloc's fixed array holds
    targets of up to 20,000 triangles with up to 10,000 vertices; the
    library's own scratch planner must agree, so the figure cannot drift."""
    B.build()
    lib = L.lib()
    cap = lib.mo_df_noalloc_scratch_capacity()
    src = open(HEADER).read()
    assert "20,000" in src and "10,000 vertices" in src
    assert lib.mo_df_method_for(20_000, 64) == L.MO_DF_LBVH
    for N in (32, 64, 128, 256):
        m = lib.mo_df_method_for(20_000, N)
        assert lib.mo_df_build_scratch_bytes(10_000, 20_000, N, m) <= cap
        # about 5% more triangles no longer fit
        m = lib.mo_df_method_for(21_000, N)
        assert lib.mo_df_build_scratch_bytes(10_000, 21_000, N, m) > cap
