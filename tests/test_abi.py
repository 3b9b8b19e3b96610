"""The C-ABI library builds, loads, and exports every function the public
header declares.  No compute call is made (CPU machines have no GPU)."""
import re
from pathlib import Path

from page_rank_gb300 import native

HEADER = Path(__file__).resolve().parents[1] / "include" / "graph_link_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(gl_[a-z0-9_]+)\s*\(", text, re.M)
    return sorted(set(names))


def test_header_declares_functions():
    names = declared_functions()
    assert "gl_pbr_spmm" in names and "gl_ppr_step" in names and "gl_pbr_build_fill" in names


def test_library_exports_every_declared_symbol():
    lib = native.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    assert sorted(native.exported_symbols()) == declared_functions()


def test_version_and_error_text():
    lib = native.lib()
    assert lib.gl_version() >= 100
    assert isinstance(lib.gl_last_error(), bytes)


def test_workspace_query_is_host_only():
    lib = native.lib()
    assert lib.gl_pbr_build_workspace_bytes(1000, 1000, 5000, 8, 8) > 0
    assert lib.gl_pbr_build_workspace_bytes(-1, 10, 10, 2, 2) < 0


def test_edge_and_topk_workspace_queries_are_host_only():
    lib = native.lib()
    assert lib.gl_edges_workspace_bytes(1000, 5000) > 0
    assert lib.gl_edges_workspace_bytes(0, 0) > 0
    assert lib.gl_edges_workspace_bytes(-1, 10) < 0
    assert lib.gl_edges_workspace_bytes(10, 1 << 40) < 0
    assert lib.gl_topk_workspace_bytes(1 << 20, 64, 100) > 0
    assert lib.gl_topk_workspace_bytes(100, 4, native.GL_TOPK_MAX + 1) < 0
    assert lib.gl_topk_workspace_bytes(-5, 4, 10) < 0


def _desc(block, rows=16):
    d = native.PbrMatrixDesc()
    d.rows, d.cols = rows, rows
    d.block_rows = d.block_cols = block
    d.value_type = native.GL_F32
    return d


def test_argument_errors_need_no_gpu():
    """Argument checks run before any CUDA call, return the documented status
    and the reference's message, and map to ValueError."""
    import ctypes

    import pytest
    lib = native.lib()
    rc = lib.gl_pbr_spmm(_desc(3), None, None, 1, 4, None, 0, None)
    assert rc == native.GL_ERR_UNSUPPORTED_BLOCK
    assert lib.gl_last_error().decode() == ("Unsupported block size for PBR SpMM. "
                                            "Only 2x2, 4x4, and 8x8 are supported.")   # pbr_kernel.cu:392
    with pytest.raises(ValueError):
        native.check(rc)
    assert lib.gl_pbr_spmm_static(_desc(5), None, None, 1, 4, None) == native.GL_ERR_UNSUPPORTED_BLOCK
    assert lib.gl_pbr_spmm(None, None, None, 1, 4, None, 0, None) == native.GL_ERR_INVALID_ARGUMENT
    assert lib.gl_pbr_spmm(_desc(4), None, None, 1, -1, None, 0, None) == native.GL_ERR_INVALID_ARGUMENT
    assert lib.gl_pbr_spmm(_desc(4, rows=0), None, None, 1, 4, None, 0, None) == native.GL_OK   # nothing to do
    assert lib.gl_pbr_validate(None, None, None) == native.GL_ERR_INVALID_ARGUMENT
    nnz = ctypes.c_int64(0)
    assert lib.gl_edges_to_transition(-1, 0, None, None, None, 1, None, None, None, None,
                                      ctypes.addressof(nnz), None, 0, None) == native.GL_ERR_INVALID_ARGUMENT
    assert lib.gl_topk_columns(None, 10, 4, None, 4, native.GL_TOPK_MAX + 1, None, None, None, 0,
                               None) == native.GL_ERR_INVALID_ARGUMENT
    assert lib.gl_topk_columns(None, 10, 4, None, 0, 5, None, None, None, 0, None) == native.GL_OK
    counts = native.BuildCounts()
    # 2^30 stripes of 8 rows: beyond the builder's int32 stripe lists
    assert lib.gl_pbr_build_count(None, None, native.GL_I64, 1 << 33, 1 << 33, 0, 8, 8, 8, None, 0, counts,
                                  None) == native.GL_ERR_INVALID_ARGUMENT
    assert "stripes" in lib.gl_last_error().decode()
    assert lib.gl_pbr_build_count(None, None, native.GL_I32, 16, 16, 0, 9, 9, 1, None, 0, counts,
                                  None) == native.GL_ERR_INVALID_ARGUMENT   # 81 bits per block


def test_descriptor_size_matches_the_library():
    """The ctypes descriptors here and in the reference-side binding stub
    have the library's sizeof(gl_pbr_matrix)."""
    import ctypes
    import importlib.util
    import pathlib
    lib = native.lib()
    assert lib.gl_pbr_matrix_bytes() == ctypes.sizeof(native.PbrMatrixDesc)
    stub = pathlib.Path(__file__).with_name("ref_binding_stub.py").read_text()
    ns: dict = {}
    src = stub.split("_lib = ctypes.CDLL")[0] + "\n_P, _I32, _I64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64\n"
    cls = stub[stub.index("class _Pbr"):stub.index("_lib.gl_pbr_stripe_index")]
    exec(src + cls, ns)
    assert ctypes.sizeof(ns["_Pbr"]) == lib.gl_pbr_matrix_bytes()


def test_every_ctypes_struct_matches_the_library():
    import ctypes
    lib = native.lib()
    pairs = {"gl_pbr_matrix": native.PbrMatrixDesc, "gl_pbr_build_counts": native.BuildCounts,
             "gl_teleport": native.TeleportDesc, "gl_ppr_step_params": native.PprStepParams,
             "gl_ppr_run_result": native.PprRunResult}
    for name, cls in pairs.items():
        assert lib.gl_struct_bytes(name.encode()) == ctypes.sizeof(cls), name
    assert lib.gl_struct_bytes(b"no_such_struct") == -1
