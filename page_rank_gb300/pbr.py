"""PBR (packed block representation) matrices built on the GPU.

:class:`PBRMatrix` mirrors the reference's bound ``pbr_matrix_t`` classes
(``Backend/graph_link/bindings/bindings.cpp:9-50``): the same read-only
attributes (numpy arrays, fetched lazily from device memory), the same
methods, and the four class names ``PBRMatrix{Int32,Int64}{Float,Double}``
that the reference's pybind overloads produce for the four index/value type
combinations.

:func:`build_pbr_device` runs the device builder (``gl_pbr_build_count`` then
``gl_pbr_build_fill``) on a CSR that already lives in device memory and
returns the PBR arrays as device tensors.
"""
from __future__ import annotations

import copy
import enum
from dataclasses import dataclass

import numpy as np
import torch

from . import native
from .trace import nvtx_range


class DataOrder(enum.IntEnum):
    """Value order inside a block (``pbr_matrix.hpp:91-96``); the builder
    always produces BLOCK_ROW_MAJOR."""

    BLOCK_ROW_MAJOR = 0
    BLOCK_COLUMN_MAJOR = 1
    INTERLEAVED_ROW_MAJOR = 2
    INTERLEAVED_COLUMN_MAJOR = 3


_TORCH_OF = {np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64,
             np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None or t.numel() == 0 else t.data_ptr()


def _stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


@dataclass
class DeviceBuild:
    """Device tensors produced by the builder (index dtype follows the input)."""

    codes: torch.Tensor        # int64 (raw 64-bit masks)
    coords: torch.Tensor       # [2 * nb] index dtype
    offsets: torch.Tensor      # [nb + 1] index dtype
    data: torch.Tensor         # [packed] value dtype
    rem_indptr: torch.Tensor   # [rows + 1] index dtype
    rem_col_ind: torch.Tensor  # [rem] index dtype
    rem_vals: torch.Tensor     # [rem] value dtype
    stripe_ptr: torch.Tensor   # [ceil(rows / block_rows) + 1] int32
    counts: dict
    trusted: bool = True       # False: arrays from outside the builder, checked on .to()


def build_pbr_device(indptr: torch.Tensor, indices: torch.Tensor, data: torch.Tensor,
                     rows: int, cols: int, block_rows: int, block_cols: int,
                     min_nnz_per_block: int) -> DeviceBuild:
    """Build PBR arrays from a canonical device CSR with the GPU builder (with
    the CSR's device current, whose stream the builder's kernels run on)."""
    if indptr.device.type != "cuda":
        raise RuntimeError("build_pbr_device needs CSR tensors in CUDA memory")
    with torch.cuda.device(indptr.device), nvtx_range(f"pbr.build {block_rows}x{block_cols}"):
        return _build_pbr_device(indptr, indices, data, rows, cols, block_rows, block_cols, min_nnz_per_block)


def _build_pbr_device(indptr: torch.Tensor, indices: torch.Tensor, data: torch.Tensor,
                      rows: int, cols: int, block_rows: int, block_cols: int,
                      min_nnz_per_block: int) -> DeviceBuild:
    dev = indptr.device
    if dev.type != "cuda":
        raise RuntimeError("build_pbr_device needs CSR tensors in CUDA memory")
    itype = indptr.dtype
    if itype not in (torch.int32, torch.int64) or indices.dtype != itype:
        raise TypeError("indptr / indices must share an int32 or int64 dtype")
    if data.dtype not in (torch.float32, torch.float64):
        raise TypeError("data must be float32 or float64")
    L = native.lib()
    gl_itype = native.GL_I32 if itype == torch.int32 else native.GL_I64
    gl_vtype = native.GL_F32 if data.dtype == torch.float32 else native.GL_F64
    nnz = int(indices.numel())
    ws_bytes = int(L.gl_pbr_build_workspace_bytes(rows, cols, nnz, block_rows, block_cols))
    if ws_bytes < 0:
        raise ValueError("invalid matrix / block sizes")
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    stream = _stream_handle(dev)
    counts = native.BuildCounts()
    native.check(L.gl_pbr_build_count(_ptr(indptr), _ptr(indices), gl_itype, rows, cols, nnz,
                                      block_rows, block_cols, int(min_nnz_per_block),
                                      ws.data_ptr(), ws_bytes, counts, stream))
    nb, packed, rem = counts.num_blocks, counts.packed_nnz, counts.remainder_nnz
    nstripes = -(-rows // block_rows)
    out = DeviceBuild(
        codes=torch.empty(nb, dtype=torch.int64, device=dev),
        coords=torch.empty(2 * nb, dtype=itype, device=dev),
        offsets=torch.empty(nb + 1, dtype=itype, device=dev),
        data=torch.empty(packed, dtype=data.dtype, device=dev),
        rem_indptr=torch.empty(rows + 1, dtype=itype, device=dev),
        rem_col_ind=torch.empty(rem, dtype=itype, device=dev),
        rem_vals=torch.empty(rem, dtype=data.dtype, device=dev),
        stripe_ptr=torch.empty(nstripes + 1, dtype=torch.int32, device=dev),
        counts={"num_blocks": nb, "packed_nnz": packed, "remainder_nnz": rem,
                "max_stripe_blocks": counts.max_stripe_blocks,
                "distinct_blocks": counts.distinct_blocks},
    )
    native.check(L.gl_pbr_build_fill(
        _ptr(indptr), _ptr(indices), _ptr(data), gl_itype, gl_vtype, rows, cols, nnz,
        block_rows, block_cols, int(min_nnz_per_block), ws.data_ptr(), ws_bytes, counts,
        _ptr(out.codes), _ptr(out.coords), out.offsets.data_ptr(), _ptr(out.data),
        out.rem_indptr.data_ptr(), _ptr(out.rem_col_ind), _ptr(out.rem_vals),
        out.stripe_ptr.data_ptr(), stream))
    return out


def stripe_index(coords_i32: torch.Tensor, rows: int, block_rows: int) -> torch.Tensor:
    """stripe_block_ptr for PBR arrays not produced by the device builder."""
    dev = coords_i32.device
    nb = coords_i32.numel() // 2
    ptr = torch.empty(-(-rows // block_rows) + 1, dtype=torch.int32, device=dev)
    flag = torch.empty(1, dtype=torch.int32, device=dev)
    native.check(native.lib().gl_pbr_stripe_index(_ptr(coords_i32), nb, rows, block_rows,
                                                   ptr.data_ptr(), flag.data_ptr(),
                                                   _stream_handle(dev)))
    return ptr


class PBRMatrix:
    """A PBR matrix; see the module docstring.

    ``data_order`` is always ``DataOrder.BLOCK_ROW_MAJOR`` (the only order the
    reference builder emits, ``pbr_matrix.cpp:473``).
    """

    _index_dtype = np.int32
    _value_dtype = np.float32

    def __init__(self, rows: int, cols: int, block_rows: int, block_cols: int, total_nnz: int,
                 build: DeviceBuild):
        self.rows = int(rows)
        self.cols = int(cols)
        self.block_rows = int(block_rows)
        self.block_cols = int(block_cols)
        self.total_nnz = int(total_nnz)
        self.data_order = DataOrder.BLOCK_ROW_MAJOR
        self._build = build
        self._host: dict[str, np.ndarray] = {}

    # -- read-only arrays (bindings.cpp:17-45) --------------------------------
    def _fetch(self, name: str, tensor: torch.Tensor, np_dtype) -> np.ndarray:
        arr = self._host.get(name)
        if arr is None:
            arr = tensor.detach().cpu().numpy().astype(np_dtype, copy=False)
            arr.setflags(write=False)
            self._host[name] = arr
        return arr

    @property
    def block_codes(self) -> np.ndarray:
        arr = self._host.get("block_codes")
        if arr is None:
            arr = self._build.codes.cpu().numpy().view(np.uint64)
            arr.setflags(write=False)
            self._host["block_codes"] = arr
        return arr

    @property
    def block_coords(self) -> np.ndarray:
        return self._fetch("block_coords", self._build.coords, self._index_dtype)

    @property
    def block_offsets(self) -> np.ndarray:
        return self._fetch("block_offsets", self._build.offsets, self._index_dtype)

    @property
    def block_data(self) -> np.ndarray:
        return self._fetch("block_data", self._build.data, self._value_dtype)

    @property
    def remainder_indptr(self) -> np.ndarray:
        return self._fetch("remainder_indptr", self._build.rem_indptr, self._index_dtype)

    @property
    def remainder_col_ind(self) -> np.ndarray:
        return self._fetch("remainder_col_ind", self._build.rem_col_ind, self._index_dtype)

    @property
    def remainder_data(self) -> np.ndarray:
        return self._fetch("remainder_data", self._build.rem_vals, self._value_dtype)

    # -- methods (bindings.cpp:47-50) -----------------------------------------
    def accounted_blocks(self) -> int:
        return int(self._build.codes.numel())

    def compressed_nnz(self) -> int:
        return int(self._build.data.numel())

    def remainder_nnz(self) -> int:
        return int(self._build.rem_col_ind.numel())

    def __copy__(self):
        new = object.__new__(type(self))
        new.__dict__.update(self.__dict__)
        new._host = dict(self._host)
        return new

    def __repr__(self) -> str:
        return (f"{type(self).__name__}(rows={self.rows}, cols={self.cols}, "
                f"block={self.block_rows}x{self.block_cols}, blocks={self.accounted_blocks()}, "
                f"packed={self.compressed_nnz()}, remainder={self.remainder_nnz()})")

    def to(self, device="cuda"):
        """Out-of-place device move with the reference's semantics
        (``graph_link/__init__.py:17-56``): returns ``self`` when already on
        ``device``, otherwise a copy registered with GPU metadata.  The arrays
        already live in device memory, so moving to CUDA uploads nothing; the
        index arrays are narrowed to int32 as the reference does."""
        from .graph_link import pbr_registry as reg

        target = "cpu" if device is None else str(torch.device(device))
        existing = reg.get_pbr_gpu_meta(self)
        current = str(existing["codes"].device) if existing else "cpu"
        if current == target:
            return self
        new = copy.copy(self)
        if target != "cpu":
            dev = torch.device(target)
            if dev.type != "cuda":
                raise ValueError(f"unsupported device {device!r}")
            b = self._build
            meta = {
                "codes": b.codes.to(dev),
                "coords": b.coords.to(dev, torch.int32),
                "offsets": b.offsets.to(dev, torch.int32),
                "data": b.data.to(dev),
                "rem_indptr": b.rem_indptr.to(dev, torch.int32),
                "rem_col_ind": b.rem_col_ind.to(dev, torch.int32),
                "rem_vals": b.rem_vals.to(dev),
                "stripe_ptr": b.stripe_ptr.to(dev),
            }
            if not b.trusted:   # e.g. read from a file: check before any kernel reads them
                validate_arrays(meta, self.rows, self.cols, self.block_rows, self.block_cols)
            reg.set_pbr_gpu_meta(new, meta)
        return new


class PBRMatrixInt32Float(PBRMatrix):
    _index_dtype, _value_dtype = np.int32, np.float32


class PBRMatrixInt64Float(PBRMatrix):
    _index_dtype, _value_dtype = np.int64, np.float32


class PBRMatrixInt32Double(PBRMatrix):
    _index_dtype, _value_dtype = np.int32, np.float64


class PBRMatrixInt64Double(PBRMatrix):
    _index_dtype, _value_dtype = np.int64, np.float64


_CLASS_OF = {(torch.int32, torch.float32): PBRMatrixInt32Float,
             (torch.int64, torch.float32): PBRMatrixInt64Float,
             (torch.int32, torch.float64): PBRMatrixInt32Double,
             (torch.int64, torch.float64): PBRMatrixInt64Double}


def pbr_from_device_csr(indptr: torch.Tensor, indices: torch.Tensor, data: torch.Tensor,
                        rows: int, cols: int, block_rows: int, block_cols: int,
                        min_nnz_per_block: int) -> PBRMatrix:
    build = build_pbr_device(indptr, indices, data, rows, cols, block_rows, block_cols,
                             min_nnz_per_block)
    cls = _CLASS_OF[(indptr.dtype, data.dtype)]
    return cls(rows, cols, block_rows, block_cols, int(indices.numel()), build)


SCHED_FIELDS = ("num_heavy", "num_pieces", "piece_work", "heavy_of", "heavy_stripe", "heavy_first",
                "piece_heavy", "piece_range")


def matrix_desc(meta: dict, rows: int, cols: int, block_rows: int, block_cols: int
                ) -> native.PbrMatrixDesc:
    """C descriptor for a registered (int32-index) device matrix, including its
    load-balance schedule (built on first use and kept in ``meta``)."""
    d = _array_desc(meta, rows, cols, block_rows, block_cols)
    sched = meta.get("schedule")
    if sched is None and block_rows == block_cols and block_rows in (2, 4, 8) and rows > 0:
        sched = build_schedule(d, meta["stripe_ptr"].device, int(meta.get("piece_work", 0)))
        meta["schedule"] = sched
    if sched is not None:
        for f in SCHED_FIELDS:
            setattr(d, f, sched[f])
    return d


def device_to_csr(pbr: "PBRMatrix", device=None) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """CSR of a PBR matrix computed on the device (``gl_pbr_to_csr``): int32
    indptr / indices and values of the matrix's value type, rows sorted by
    column (the reference's ``pbr_to_csr``, ``pbr_matrix.cpp:289-338``)."""
    from .graph_link import pbr_registry as reg

    dev = torch.device(device) if device is not None else pbr._build.codes.device
    if dev.type != "cuda":
        raise RuntimeError("device_to_csr needs a CUDA device")
    mat = pbr.to(dev)
    meta = reg.get_pbr_gpu_meta(mat)
    d = _array_desc(meta, pbr.rows, pbr.cols, pbr.block_rows, pbr.block_cols)
    L = native.lib()
    nbytes = int(L.gl_pbr_to_csr_workspace_bytes(d))
    if nbytes < 0:
        raise ValueError("matrix too large for an int32 CSR")
    nnz = int(d.packed_nnz + d.remainder_nnz)
    with torch.cuda.device(dev):
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        indptr = torch.empty(pbr.rows + 1, dtype=torch.int32, device=dev)
        indices = torch.empty(nnz, dtype=torch.int32, device=dev)
        data = torch.empty(nnz, dtype=meta["data"].dtype, device=dev)
        native.check(L.gl_pbr_to_csr(d, indptr.data_ptr(), _ptr(indices), _ptr(data), ws.data_ptr(), nbytes,
                                     _stream_handle(dev)))
    return indptr, indices, data


def block_patterns(codes: torch.Tensor, min_nnz_coverage: int) -> tuple[np.ndarray, np.ndarray, dict]:
    """Distinct block codes (ascending, uint64), their occurrence counts and
    the coverage-rule totals, counted on the device
    (``gl_pbr_block_patterns``)."""
    dev = codes.device
    nb = int(codes.numel())
    L = native.lib()
    nbytes = int(L.gl_pbr_block_patterns_workspace_bytes(nb))
    if nbytes < 0:
        raise ValueError("too many blocks")
    with torch.cuda.device(dev):
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        uniq = torch.empty(max(nb, 1), dtype=torch.int64, device=dev)
        counts = torch.empty(max(nb, 1), dtype=torch.int64, device=dev)
        small = torch.zeros(5, dtype=torch.int64, device=dev)    # [num_unique, totals[4]]
        native.check(L.gl_pbr_block_patterns(_ptr(codes.contiguous()), nb, int(min_nnz_coverage),
                                             uniq.data_ptr(), counts.data_ptr(), small.data_ptr(),
                                             small[1:].data_ptr(), ws.data_ptr(), nbytes, _stream_handle(dev)))
        sm = small.cpu().numpy()
    u = int(sm[0])
    totals = {"accounted_nnz": int(sm[1]), "remainder_nnz": int(sm[2]), "accounted_patterns": int(sm[3]),
              "accounted_blocks": int(sm[4])}
    return uniq[:u].cpu().numpy().view(np.uint64), counts[:u].cpu().numpy(), totals


def validate_arrays(meta: dict, rows: int, cols: int, block_rows: int, block_cols: int) -> None:
    """``gl_pbr_validate`` on device PBR arrays that did not come from this
    library's builder; raises ``ValueError`` naming the first broken
    property (offsets vs bit counts, coordinates, bits past the edge,
    remainder pointers / columns, stripe pointers)."""
    d = _array_desc(meta, rows, cols, block_rows, block_cols)
    dev = meta["rem_indptr"].device
    flag = torch.empty(1, dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        native.check(native.lib().gl_pbr_validate(d, flag.data_ptr(), torch.cuda.current_stream(dev).cuda_stream))


def _array_desc(meta: dict, rows: int, cols: int, block_rows: int, block_cols: int) -> native.PbrMatrixDesc:
    d = native.PbrMatrixDesc()
    d.rows, d.cols = rows, cols
    d.block_rows, d.block_cols = block_rows, block_cols
    d.num_blocks = meta["codes"].numel()
    d.packed_nnz = meta["data"].numel()
    d.remainder_nnz = meta["rem_col_ind"].numel()
    d.value_type = native.GL_F32 if meta["data"].dtype == torch.float32 else native.GL_F64
    d.block_codes = _ptr(meta["codes"])
    d.block_coords = _ptr(meta["coords"])
    d.block_offsets = _ptr(meta["offsets"])
    d.block_data = _ptr(meta["data"])
    d.remainder_indptr = _ptr(meta["rem_indptr"])
    d.remainder_col_ind = _ptr(meta["rem_col_ind"])
    d.remainder_data = _ptr(meta["rem_vals"])
    d.stripe_block_ptr = _ptr(meta["stripe_ptr"])
    d.column_tile = int(meta.get("column_tile", 0))
    d.lane_split = int(meta.get("lane_split", 0))
    d.kernel = int(meta.get("kernel", 0))
    return d


def build_schedule(d: native.PbrMatrixDesc, device, piece_work: int = 0) -> dict:
    L = native.lib()
    elems = int(L.gl_pbr_schedule_elems(d, piece_work))
    buf = torch.empty(max(elems, 1), dtype=torch.int32, device=device)
    with torch.cuda.device(device):
        native.check(L.gl_pbr_schedule_build(d, piece_work, buf.data_ptr(), elems,
                                             torch.cuda.current_stream(device).cuda_stream))
    sched = {f: getattr(d, f) for f in SCHED_FIELDS}
    sched["buffer"] = buf          # keeps the device arrays alive
    return sched


def spmm_workspace(meta: dict, desc: native.PbrMatrixDesc, batch: int, K: int, device) -> torch.Tensor | None:
    """Zero-filled workspace for gl_pbr_spmm / gl_ppr_step, cached per shape
    and stream (a workspace must not be used by two launches at once)."""
    nbytes = int(native.lib().gl_pbr_spmm_workspace_bytes(desc, batch, K))
    if nbytes <= 0:
        return None
    key = (batch, K, torch.cuda.current_stream(device).cuda_stream)
    cache = meta.setdefault("ws_cache", {})
    ws = cache.get(key)
    if ws is None or ws.numel() < nbytes:
        ws = torch.zeros(nbytes, dtype=torch.uint8, device=device)
        cache[key] = ws
    return ws
