"""Build and load the native library ``libgl_gb300.so`` (CUDA, sm_103a).

The library exports the C ABI declared in ``include/graph_link_gb300.h``.
Everything above it in this package talks to it through :mod:`ctypes`
(``ctypes`` drops the GIL for the duration of each call).

There is deliberately no fallback: if the library cannot be loaded, or no
CUDA device is visible, the calls raise.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
import threading
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
LIB_DIR = PKG_DIR / "_lib"
LIB_PATH = LIB_DIR / "libgl_gb300.so"
OBJ_DIR = LIB_DIR / "obj"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE), "-I", str(CSRC)]

GL_TOPK_MAX = 2048
GL_OK = 0
GL_ERR_INVALID_ARGUMENT = 1
GL_ERR_UNSUPPORTED_BLOCK = 2
GL_ERR_OOM = 3
GL_ERR_CUDA = 4
GL_ERR_TIMEOUT = 5
GL_ERR_NONCANONICAL = 6
GL_ERR_WORKSPACE = 7
GL_I32, GL_I64 = 0, 1
GL_F32, GL_F64 = 0, 1
GL_PPR_STOP_ALL, GL_PPR_STOP_PER_COLUMN = 0, 1
GL_DANGLING_TO_TELEPORT, GL_DANGLING_UNIFORM = 0, 1
GL_SPMM_STATIC_SCRATCH_BYTES = 16 * 1024 * 1024
GL_MLP_MAX_IN, GL_MLP_HIDDEN = 16, 128


def _nvcc() -> str:
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda_home) / "bin" / "nvcc"
    return str(cand) if cand.is_file() else "nvcc"


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.is_file():
        return True
    deps = [src, *CSRC.glob("*.cuh"), *INCLUDE.glob("*.h")]
    return obj.stat().st_mtime < max(d.stat().st_mtime for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every ``csrc/*.cu`` for sm_103a (in parallel) and link the .so."""
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for src in sources():
        obj = OBJ_DIR / (src.stem + ".o")
        if force or _stale(obj, src):
            jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
        return obj

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(compile_one, jobs))
    objs = [OBJ_DIR / (s.stem + ".o") for s in sources()]
    if force or jobs or not LIB_PATH.is_file():
        tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-cudart", "shared", *map(str, objs), "-o", str(tmp)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class GLError(RuntimeError):
    """A native call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class GLValueError(GLError, ValueError):
    """Status that the reference reports as a ValueError / invalid_argument."""


_lib = None
_lock = threading.Lock()

_c = ctypes
_vp = _c.c_void_p
_i32 = _c.c_int32
_i64 = _c.c_int64


class PbrMatrixDesc(_c.Structure):
    _fields_ = [("rows", _i64), ("cols", _i64), ("block_rows", _i32), ("block_cols", _i32),
                ("num_blocks", _i64), ("packed_nnz", _i64), ("remainder_nnz", _i64),
                ("value_type", _i32),
                ("block_codes", _vp), ("block_coords", _vp), ("block_offsets", _vp),
                ("block_data", _vp), ("remainder_indptr", _vp), ("remainder_col_ind", _vp),
                ("remainder_data", _vp), ("stripe_block_ptr", _vp),
                ("num_heavy", _i32), ("num_pieces", _i32), ("piece_work", _i32), ("column_tile", _i32),
                ("lane_split", _i32),
                ("heavy_of", _vp), ("heavy_stripe", _vp), ("heavy_first", _vp), ("piece_heavy", _vp),
                ("kernel", _i32), ("piece_range", _vp)]


class BuildCounts(_c.Structure):
    _fields_ = [("num_blocks", _i64), ("packed_nnz", _i64), ("remainder_nnz", _i64),
                ("max_stripe_blocks", _i64), ("distinct_blocks", _i64)]


class TeleportDesc(_c.Structure):
    _fields_ = [("stripe_ptr", _vp), ("row", _vp), ("col", _vp), ("weight", _vp),
                ("num_entries", _i64)]


class PprStepParams(_c.Structure):
    _fields_ = [("alpha", _c.c_double), ("tol", _c.c_double), ("stop_mode", _i32),
                ("max_iterations", _i32), ("step_in_chunk", _i32), ("chunk_base", _vp),
                ("residual_hist", _vp), ("dangling_hist", _vp), ("dangling_bitmap", _vp),
                ("dangling_target", _i32), ("column_alpha", _vp), ("column_tol", _vp)]


class PprRunResult(_c.Structure):
    _fields_ = [("iterations", _i32), ("converged", _i32), ("result_in_x1", _i32)]


# name -> (restype, argtypes)
_SIGS = {
    "gl_last_error": (_c.c_char_p, []),
    "gl_version": (_c.c_int, []),
    "gl_pbr_matrix_bytes": (_i64, []),
    "gl_struct_bytes": (_i64, [_c.c_char_p]),
    "gl_edges_workspace_bytes": (_i64, [_i64, _i64]),
    "gl_edges_to_transition": (_c.c_int, [_i64, _i64, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _i64,
                                          _vp]),
    "gl_pbr_build_workspace_bytes": (_i64, [_i64, _i64, _i64, _i32, _i32]),
    "gl_pbr_build_count": (_c.c_int, [_vp, _vp, _i32, _i64, _i64, _i64, _i32, _i32, _i32, _vp, _i64,
                                      _c.POINTER(BuildCounts), _vp]),
    "gl_pbr_build_fill": (_c.c_int, [_vp, _vp, _vp, _i32, _i32, _i64, _i64, _i64, _i32, _i32, _i32, _vp,
                                     _i64, _c.POINTER(BuildCounts), _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                     _vp, _vp]),
    "gl_pbr_stripe_index": (_c.c_int, [_vp, _i64, _i64, _i32, _vp, _vp, _vp]),
    "gl_pbr_validate": (_c.c_int, [_c.POINTER(PbrMatrixDesc), _vp, _vp]),
    "gl_pbr_schedule_elems": (_i64, [_c.POINTER(PbrMatrixDesc), _i32]),
    "gl_pbr_schedule_build": (_c.c_int, [_c.POINTER(PbrMatrixDesc), _i32, _vp, _i64, _vp]),
    "gl_pbr_spmm_workspace_bytes": (_i64, [_c.POINTER(PbrMatrixDesc), _i64, _i64]),
    "gl_pbr_spmm": (_c.c_int, [_c.POINTER(PbrMatrixDesc), _vp, _vp, _i64, _i64, _vp, _i64, _vp]),
    "gl_pbr_spmm_static": (_c.c_int, [_c.POINTER(PbrMatrixDesc), _vp, _vp, _i64, _i64, _vp]),
    "gl_spmm_workspace_error": (_c.c_int, [_vp, _vp]),
    "gl_pbr_to_csr_workspace_bytes": (_i64, [_c.POINTER(PbrMatrixDesc)]),
    "gl_pbr_to_csr": (_c.c_int, [_c.POINTER(PbrMatrixDesc), _vp, _vp, _vp, _vp, _i64, _vp]),
    "gl_pbr_block_patterns_workspace_bytes": (_i64, [_i64]),
    "gl_pbr_block_patterns": (_c.c_int, [_vp, _i64, _i64, _vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "gl_ppr_teleport_index": (_c.c_int, [_i64, _i32, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp,
                                         _vp]),
    "gl_ppr_init": (_c.c_int, [_c.POINTER(TeleportDesc), _i64, _i64, _i32, _vp, _vp, _vp, _vp]),
    "gl_ppr_dangling_mass": (_c.c_int, [_vp, _i64, _i64, _i32, _vp, _vp, _vp]),
    "gl_ppr_step": (_c.c_int, [_c.POINTER(PbrMatrixDesc), _c.POINTER(TeleportDesc), _vp, _vp, _i64,
                               _c.POINTER(PprStepParams), _vp, _i64, _vp]),
    "gl_counter_add": (_c.c_int, [_vp, _i32, _vp]),
    "gl_ppr_run": (_c.c_int, [_c.POINTER(PbrMatrixDesc), _c.POINTER(TeleportDesc), _vp, _vp, _i64,
                              _c.POINTER(PprStepParams), _i32, _i32, _vp, _i64, _vp,
                              _c.POINTER(PprRunResult), _vp]),
    "gl_topk_workspace_bytes": (_i64, [_i64, _i64, _i32]),
    "gl_topk_columns": (_c.c_int, [_vp, _i64, _i64, _vp, _i64, _i32, _vp, _vp, _vp, _i64, _vp]),
    "gl_mlp_forward": (_c.c_int, [_vp, _i64, _i32, _vp, _vp, _vp, _c.c_float, _vp, _vp]),
    "gl_mlp_backward": (_c.c_int, [_vp, _vp, _i64, _i32, _vp, _vp, _vp, _c.c_float, _vp, _vp, _vp]),
    "gl_mlp_adam": (_c.c_int, [_vp, _vp, _vp, _vp, _i64, _c.c_float, _c.c_float, _c.c_float, _c.c_float,
                               _c.c_float, _i32, _vp, _vp, _i32, _vp]),
    "gl_window_blocks": (_c.c_int, [_vp, _vp, _vp, _i64, _c.c_float, _vp, _vp]),
    "gl_window_invert": (_c.c_int, [_vp, _i64, _vp, _vp]),
    "gl_window_apply": (_c.c_int, [_vp, _i64, _i32, _vp, _c.c_float, _vp, _vp, _c.c_float, _i32, _vp, _vp]),
    "gl_window_finalize_workspace_bytes": (_i64, [_i64, _i32]),
    "gl_window_finalize": (_c.c_int, [_vp, _i64, _i32, _vp, _vp, _vp, _i64, _vp]),
    "gl_cold_residual": (_c.c_int, [_vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i32, _c.c_float, _vp, _vp]),
}


def exported_symbols() -> list[str]:
    return list(_SIGS)


def lib():
    """Load (building first if needed) the native library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.is_file():
                build()
            handle = ctypes.CDLL(str(LIB_PATH))
            for name, (res, args) in _SIGS.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def check(rc: int) -> None:
    """Raise the Python error that matches a native status code."""
    if rc == GL_OK:
        return
    msg = (lib().gl_last_error() or b"").decode(errors="replace") or f"status {rc}"
    if rc in (GL_ERR_INVALID_ARGUMENT, GL_ERR_UNSUPPORTED_BLOCK, GL_ERR_NONCANONICAL):
        raise GLValueError(rc, msg)
    if rc == GL_ERR_OOM:
        raise GLError(rc, "out of device memory: " + msg)
    raise GLError(rc, msg)
