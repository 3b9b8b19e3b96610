"""The ctypes binding a maintainer of the reference package would add
(as graph_link/gb300.py) so that its pbr_batched_matmul_cuda
(Backend/graph_link/__init__.py:88-101) runs the fused sm_103a SpMM on the
tensors the reference's PBRMatrix.to() registers.  Kept here, byte for byte
as published, so the GPU tests can load it against this library.
"""
# graph_link/gb300.py  (new file in the reference package)
import ctypes, os, torch

_lib = ctypes.CDLL(os.environ.get("GL_GB300_LIB", "libgl_gb300.so"))
_P, _I32, _I64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64

class _Pbr(ctypes.Structure):
    _fields_ = [("rows", _I64), ("cols", _I64), ("block_rows", _I32), ("block_cols", _I32),
                ("num_blocks", _I64), ("packed_nnz", _I64), ("remainder_nnz", _I64),
                ("value_type", _I32)] + \
               [(n, _P) for n in ("block_codes", "block_coords", "block_offsets", "block_data",
                                  "remainder_indptr", "remainder_col_ind", "remainder_data",
                                  "stripe_block_ptr")] + \
               [(n, _I32) for n in ("num_heavy", "num_pieces", "piece_work", "column_tile",
                                    "lane_split")] + \
               [(n, _P) for n in ("heavy_of", "heavy_stripe", "heavy_first", "piece_heavy")] + \
               [("kernel", _I32), ("piece_range", _P)]     # gl_pbr_matrix as of ABI 101 (gl_version())

_lib.gl_pbr_stripe_index.argtypes = [_P, _I64, _I64, _I32, _P, _P, _P]
_lib.gl_pbr_validate.argtypes = [ctypes.POINTER(_Pbr), _P, _P]
_lib.gl_pbr_schedule_elems.argtypes = [ctypes.POINTER(_Pbr), _I32]
_lib.gl_pbr_schedule_elems.restype = _I64
_lib.gl_pbr_schedule_build.argtypes = [ctypes.POINTER(_Pbr), _I32, _P, _I64, _P]
_lib.gl_pbr_spmm_static.argtypes = [ctypes.POINTER(_Pbr), _P, _P, _I64, _I64, _P]
_lib.gl_last_error.restype = ctypes.c_char_p
_lib.gl_pbr_matrix_bytes.restype = _I64
if _lib.gl_pbr_matrix_bytes() != ctypes.sizeof(_Pbr):      # a descriptor of another ABI version
    raise ImportError(f"gl_pbr_matrix is {_lib.gl_pbr_matrix_bytes()} bytes in the library, "
                      f"{ctypes.sizeof(_Pbr)} here")

def _check(rc):
    if rc == 2: raise ValueError(_lib.gl_last_error().decode())     # reference's message
    if rc: raise RuntimeError(_lib.gl_last_error().decode())

def _descriptor(pbr, meta, dtype, stream):
    """One-time per matrix (after .to('cuda')): stripe index + load-balance
    schedule, kept in meta next to the reference's own device tensors."""
    if "gb300_desc" in meta and meta["gb300_dtype"] == dtype:
        return meta["gb300_desc"]
    dev = meta["codes"].device
    ns = -(-pbr.rows // pbr.block_rows)
    meta["stripe_ptr"] = torch.empty(ns + 1, dtype=torch.int32, device=dev)
    flag = torch.empty(1, dtype=torch.int32, device=dev)
    _check(_lib.gl_pbr_stripe_index(meta["coords"].data_ptr(), meta["codes"].numel(), pbr.rows,
                                    pbr.block_rows, meta["stripe_ptr"].data_ptr(), flag.data_ptr(),
                                    stream))
    ptr = lambda k: meta[k].data_ptr() if meta[k].numel() else None
    d = _Pbr(pbr.rows, pbr.cols, pbr.block_rows, pbr.block_cols, meta["codes"].numel(),
             meta["data"].numel(), meta["rem_col_ind"].numel(), 0 if dtype == torch.float32 else 1,
             *[ptr(k) for k in ("codes", "coords", "offsets", "data", "rem_indptr", "rem_col_ind",
                                "rem_vals", "stripe_ptr")])
    _check(_lib.gl_pbr_validate(ctypes.byref(d), flag.data_ptr(), stream))   # arrays from the host builder
    elems = _lib.gl_pbr_schedule_elems(ctypes.byref(d), 0)
    meta["gb300_sched"] = torch.empty(max(elems, 1), dtype=torch.int32, device=dev)
    _check(_lib.gl_pbr_schedule_build(ctypes.byref(d), 0, meta["gb300_sched"].data_ptr(), elems, stream))
    meta["gb300_desc"], meta["gb300_dtype"] = d, dtype
    return d

def pbr_spmm_gb300(pbr, meta, x):            # meta = get_pbr_gpu_meta(pbr)
    stream = torch.cuda.current_stream().cuda_stream
    d = _descriptor(pbr, meta, x.dtype, stream)
    x3 = (x.unsqueeze(0) if x.dim() == 2 else x).contiguous()
    y = torch.empty((x3.shape[0], pbr.rows, x3.shape[2]), dtype=x.dtype, device=x.device)
    _check(_lib.gl_pbr_spmm_static(ctypes.byref(d), x3.data_ptr(), y.data_ptr(), x3.shape[0],
                                   x3.shape[2], stream))
    return y
