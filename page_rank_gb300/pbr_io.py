"""On-disk PBR matrices: a prebuilt graph is loaded by a serving process
without rebuilding it.

The reference has no file format for PBR matrices (it rebuilds on every
request).  This one stores exactly the seven arrays of a PBR matrix
(``bindings.cpp:9-50``) so a loaded matrix is bit-identical to the saved one:

    bytes 0..7    magic ``b"GLPBR\\x00\\x01\\x00"`` (format version 1)
    bytes 8..15   little-endian uint64: length H of the header
    bytes 16..    H bytes of UTF-8 JSON: rows, cols, block_rows, block_cols,
                  total_nnz, index_dtype, value_dtype and, per array, its
                  name, dtype, element count, byte offset and CRC-32
    then          the arrays, little-endian, each at a 64-byte aligned offset

Reading checks the magic, the version, every array's bounds and checksum,
and the structural invariants a builder guarantees (offsets, indptr,
coordinates on the block grid); a file that fails any of them raises
``ValueError`` before anything reaches the GPU.
"""
from __future__ import annotations

import json
import zlib
from pathlib import Path

import numpy as np
import torch

MAGIC = b"GLPBR\x00\x01\x00"
ALIGN = 64
ARRAYS = ("block_codes", "block_coords", "block_offsets", "block_data", "remainder_indptr",
          "remainder_col_ind", "remainder_data")


def _kind(name: str) -> str:
    if name == "block_codes":
        return "uint64"
    if name in ("block_data", "remainder_data"):
        return "value"
    return "index"


def write_pbr_arrays(path, meta: dict, arrays: dict) -> None:
    """Write a PBR file from host arrays (``meta``: rows, cols, block_rows,
    block_cols, total_nnz)."""
    itype = np.dtype(arrays["block_coords"].dtype)
    vtype = np.dtype(arrays["block_data"].dtype)
    if itype not in (np.dtype(np.int32), np.dtype(np.int64)) or vtype not in (np.dtype(np.float32),
                                                                                np.dtype(np.float64)):
        raise TypeError("index arrays must be int32 / int64 and values float32 / float64")
    blobs, entries, off = [], [], 0
    for name in ARRAYS:
        want = {"uint64": np.dtype("<u8"), "index": itype.newbyteorder("<"),
                "value": vtype.newbyteorder("<")}[_kind(name)]
        a = np.ascontiguousarray(np.asarray(arrays[name]).astype(want, copy=False))
        raw = a.tobytes()
        entries.append({"name": name, "dtype": want.str, "count": int(a.size), "offset": off,
                        "crc32": zlib.crc32(raw)})
        blobs.append(raw)
        off += (len(raw) + ALIGN - 1) // ALIGN * ALIGN
    header = {"rows": int(meta["rows"]), "cols": int(meta["cols"]), "block_rows": int(meta["block_rows"]),
              "block_cols": int(meta["block_cols"]), "total_nnz": int(meta["total_nnz"]),
              "index_dtype": itype.name, "value_dtype": vtype.name, "arrays": entries}
    hb = json.dumps(header, sort_keys=True).encode()
    base = (16 + len(hb) + ALIGN - 1) // ALIGN * ALIGN
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(len(hb).to_bytes(8, "little"))
        f.write(hb)
        f.write(b"\0" * (base - 16 - len(hb)))
        for e, raw in zip(entries, blobs):
            f.seek(base + e["offset"])
            f.write(raw)
        f.truncate(base + off)   # zero padding up to the end of the last (aligned) array


def read_pbr_arrays(path) -> tuple[dict, dict]:
    """(meta, arrays) of a PBR file, fully validated; host memory only."""
    data = Path(path).read_bytes()
    if len(data) < 16 or data[:8] != MAGIC:
        raise ValueError("not a PBR file (bad magic or unsupported version)")
    hlen = int.from_bytes(data[8:16], "little")
    if hlen <= 0 or 16 + hlen > len(data):
        raise ValueError("PBR file header is truncated")
    try:
        header = json.loads(data[16:16 + hlen].decode())
        base = (16 + hlen + ALIGN - 1) // ALIGN * ALIGN
        meta = {k: int(header[k]) for k in ("rows", "cols", "block_rows", "block_cols", "total_nnz")}
        entries = {e["name"]: e for e in header["arrays"]}
    except (ValueError, KeyError, TypeError) as exc:
        raise ValueError(f"PBR file header is malformed: {exc}") from None
    if set(entries) != set(ARRAYS):
        raise ValueError("PBR file does not hold the seven PBR arrays")
    arrays = {}
    for name in ARRAYS:
        e = entries[name]
        dt = np.dtype(e["dtype"])
        start, count = base + int(e["offset"]), int(e["count"])
        if count < 0 or int(e["offset"]) < 0 or start + count * dt.itemsize > len(data):
            raise ValueError(f"PBR array {name} lies outside the file")
        raw = data[start:start + count * dt.itemsize]
        if zlib.crc32(raw) != int(e["crc32"]):
            raise ValueError(f"PBR array {name} fails its checksum")
        arrays[name] = np.frombuffer(raw, dtype=dt).astype(dt.newbyteorder("="), copy=True)
    _validate(meta, arrays)
    return meta, arrays


def _validate(meta: dict, a: dict) -> None:
    rows, cols, br, bc = meta["rows"], meta["cols"], meta["block_rows"], meta["block_cols"]
    if rows < 0 or cols < 0 or br < 1 or bc < 1 or br * bc > 64:
        raise ValueError("PBR file has invalid sizes")
    nb = a["block_codes"].size
    off, rp = a["block_offsets"], a["remainder_indptr"]

    def fail(msg):
        raise ValueError("PBR file is inconsistent: " + msg)

    if a["block_coords"].size != 2 * nb or off.size != nb + 1:
        fail("block arrays disagree on the block count")
    if nb and (off[0] != 0 or np.any(np.diff(off) < 0) or off[-1] != a["block_data"].size):
        fail("block_offsets")
    table = np.array([bin(i).count("1") for i in range(256)], dtype=np.int64)
    pops = table[a["block_codes"].view(np.uint8).reshape(-1, 8)].sum(axis=1) if nb else np.zeros(0, np.int64)
    if nb and np.any(np.diff(off) != pops):
        fail("block_offsets do not match the block codes")
    if rp.size != rows + 1 or rp[0] != 0 or np.any(np.diff(rp) < 0) or rp[-1] != a["remainder_col_ind"].size:
        fail("remainder_indptr")
    if a["remainder_data"].size != a["remainder_col_ind"].size:
        fail("remainder arrays disagree")
    rc = a["remainder_col_ind"]
    if rc.size and (rc.min() < 0 or rc.max() >= cols):
        fail("remainder column out of range")
    co = a["block_coords"].reshape(-1, 2) if nb else np.zeros((0, 2), np.int64)
    if nb and (np.any(co[:, 0] % br) or np.any(co[:, 1] % bc) or co[:, 0].min() < 0 or co[:, 0].max() >= rows
               or co[:, 1].min() < 0 or co[:, 1].max() >= cols):
        fail("block coordinates off the block grid")
    if a["block_data"].size + rc.size != meta["total_nnz"]:
        fail("total_nnz")


def save_pbr(pbr, path) -> None:
    """Write a PBRMatrix (as returned by ``graph_link.csr_to_pbr``)."""
    write_pbr_arrays(path, {"rows": pbr.rows, "cols": pbr.cols, "block_rows": pbr.block_rows,
                            "block_cols": pbr.block_cols, "total_nnz": pbr.total_nnz},
                     {name: getattr(pbr, name) for name in ARRAYS})


def load_pbr(path, device=None):
    """Read a PBR file into a PBRMatrix whose arrays live on ``device``
    (default: the current CUDA device); call ``.to('cuda')`` as for a built
    matrix.  The blocks must be stored stripe-major, as every builder emits
    them (checked on the device); ``.to('cuda')`` also runs the device
    consistency check (``gl_pbr_validate``) before any kernel reads them."""
    from .pbr import _CLASS_OF, DeviceBuild, stripe_index

    meta, a = read_pbr_arrays(path)
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    itype = torch.int32 if a["block_coords"].dtype == np.int32 else torch.int64
    vtype = torch.float32 if a["block_data"].dtype == np.float32 else torch.float64
    t = {k: torch.from_numpy(v) for k, v in a.items()}
    coords = t["block_coords"].to(dev)
    build = DeviceBuild(
        codes=torch.from_numpy(a["block_codes"].view(np.int64)).to(dev),
        coords=coords, offsets=t["block_offsets"].to(dev), data=t["block_data"].to(dev),
        rem_indptr=t["remainder_indptr"].to(dev), rem_col_ind=t["remainder_col_ind"].to(dev),
        rem_vals=t["remainder_data"].to(dev),
        stripe_ptr=stripe_index(coords.to(torch.int32), meta["rows"], meta["block_rows"]),
        counts={"num_blocks": int(a["block_codes"].size), "packed_nnz": int(a["block_data"].size),
                "remainder_nnz": int(a["remainder_col_ind"].size)},
        trusted=False)
    cls = _CLASS_OF[(itype, vtype)]
    return cls(meta["rows"], meta["cols"], meta["block_rows"], meta["block_cols"], meta["total_nnz"], build)
