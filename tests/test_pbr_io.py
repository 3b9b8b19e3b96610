"""On-disk PBR files: exact round trip of the seven arrays, and rejection
of damaged or inconsistent files (host-side; no GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from page_rank_gb300.pbr_io import ARRAYS, read_pbr_arrays, write_pbr_arrays


def _arrays(seed=0, itype=np.int32, vtype=np.float32, bs=4, mn=2):
    A = sp.random(300, 280, density=0.05, format="csr", dtype=vtype, random_state=seed)
    A = sp.csr_matrix((A.data, A.indices.astype(itype), A.indptr.astype(itype)), shape=A.shape)
    arr = oracle.csr_to_pbr(A.indptr, A.indices, A.data, 300, 280, bs, bs, mn)
    meta = {"rows": 300, "cols": 280, "block_rows": bs, "block_cols": bs, "total_nnz": int(A.nnz)}
    return meta, {k: arr[k] for k in ARRAYS}


@pytest.mark.parametrize("itype,vtype", [(np.int32, np.float32), (np.int64, np.float64)])
def test_round_trip_is_exact(tmp_path, itype, vtype):
    meta, arrays = _arrays(1, itype, vtype)
    path = tmp_path / "g.pbr"
    write_pbr_arrays(path, meta, arrays)
    m2, a2 = read_pbr_arrays(path)
    assert m2 == meta
    for k in ARRAYS:
        assert a2[k].dtype == np.asarray(arrays[k]).dtype or k == "block_codes"
        assert np.array_equal(a2[k].view(np.uint64) if k == "block_codes" else a2[k],
                              np.asarray(arrays[k]).view(np.uint64) if k == "block_codes" else arrays[k])


def test_empty_matrix_round_trip(tmp_path):
    meta = {"rows": 5, "cols": 7, "block_rows": 2, "block_cols": 2, "total_nnz": 0}
    arrays = {"block_codes": np.zeros(0, np.uint64), "block_coords": np.zeros(0, np.int32),
              "block_offsets": np.zeros(1, np.int32), "block_data": np.zeros(0, np.float32),
              "remainder_indptr": np.zeros(6, np.int32), "remainder_col_ind": np.zeros(0, np.int32),
              "remainder_data": np.zeros(0, np.float32)}
    write_pbr_arrays(tmp_path / "e.pbr", meta, arrays)
    m2, a2 = read_pbr_arrays(tmp_path / "e.pbr")
    assert m2 == meta and a2["remainder_indptr"].size == 6


def test_damaged_files_are_rejected(tmp_path):
    meta, arrays = _arrays(2)
    path = tmp_path / "g.pbr"
    write_pbr_arrays(path, meta, arrays)
    raw = bytearray(path.read_bytes())
    bad = tmp_path / "bad.pbr"
    bad.write_bytes(b"XXXXXXXX" + bytes(raw[8:]))
    with pytest.raises(ValueError, match="magic"):
        read_pbr_arrays(bad)
    flipped = bytearray(raw)
    flipped[-70] ^= 0x40                      # inside the last array
    bad.write_bytes(bytes(flipped))
    with pytest.raises(ValueError, match="checksum"):
        read_pbr_arrays(bad)
    bad.write_bytes(bytes(raw[: len(raw) // 2]))
    with pytest.raises(ValueError, match="outside the file|truncated"):
        read_pbr_arrays(bad)


def test_inconsistent_arrays_are_rejected(tmp_path):
    meta, arrays = _arrays(3)
    path = tmp_path / "g.pbr"
    off = np.array(arrays["block_offsets"]).copy()
    off[1] += 1
    with pytest.raises(ValueError, match="block_offsets"):
        write_pbr_arrays(path, meta, {**arrays, "block_offsets": off})
        read_pbr_arrays(path)
    rc = np.array(arrays["remainder_col_ind"]).copy()
    rc[0] = 280
    write_pbr_arrays(path, meta, {**arrays, "remainder_col_ind": rc})
    with pytest.raises(ValueError, match="out of range"):
        read_pbr_arrays(path)
    write_pbr_arrays(path, {**meta, "total_nnz": meta["total_nnz"] + 1}, arrays)
    with pytest.raises(ValueError, match="total_nnz"):
        read_pbr_arrays(path)
