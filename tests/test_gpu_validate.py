"""gl_pbr_validate: PBR arrays from outside the device builder are checked
before any kernel reads them.  Each corrupted copy below is only validated
(never handed to the SpMM); the original passes.  GPU only."""
import numpy as np
import pytest
import torch

from tests._cases import random_csr

pytestmark = pytest.mark.gpu


def _matrix(n):
    """A random matrix with a kept block in the last column block."""
    import scipy.sparse as sp
    A = random_csr(n, 0.06, seed=9).tolil()
    A[0, n - 3:] = 1.0
    A[1, n - 3:] = 1.0
    return sp.csr_matrix(A, dtype=np.float32)


def _meta(device, n=200, bs=4):
    from page_rank_gb300 import graph_link as gl
    A = _matrix(n)
    p = gl.csr_to_pbr(A, bs, bs, 2).to(device)
    meta = gl.get_pbr_gpu_meta(p)
    keep = ("codes", "coords", "offsets", "data", "rem_indptr", "rem_col_ind", "rem_vals", "stripe_ptr")
    return {k: meta[k].clone() for k in keep}, n, bs


def _check(meta, n, bs):
    from page_rank_gb300.pbr import validate_arrays
    validate_arrays(meta, n, n, bs, bs)


def test_valid_arrays_pass(device):
    meta, n, bs = _meta(device)
    _check(meta, n, bs)


@pytest.mark.parametrize("what,match", [
    ("offsets", "bit counts"),
    ("coords_off_grid", "block grid"),
    ("coords_outside", "block grid"),
    ("bit_past_edge", "past the matrix edge"),
    ("rem_indptr", "row pointer"),
    ("rem_col", "column index"),
    ("stripe_ptr", "stripe by stripe"),
])
def test_corrupted_arrays_rejected(what, match, device):
    meta, n, bs = _meta(device, n=203, bs=4)   # 203 rows / columns: a ragged last stripe
    if what == "offsets":
        meta["offsets"][3] += 1
    elif what == "coords_off_grid":
        meta["coords"][1] += 1
    elif what == "coords_outside":
        meta["coords"][0] = n + 4
    elif what == "bit_past_edge":
        # a block in the last column block gets a bit in column 203 (past 202)
        co = meta["coords"].view(-1, 2).cpu().numpy()
        b = int(np.nonzero(co[:, 1] == 200)[0][0])
        meta["codes"][b] |= 1 << 3          # row 0, column 200 + 3
        meta["offsets"][b + 1:] += 1          # keep offsets consistent with the bit counts
        k = int(meta["offsets"][b])
        meta["data"] = torch.cat([meta["data"][:k], meta["data"][:1], meta["data"][k:]])
    elif what == "rem_indptr":
        meta["rem_indptr"][5] = meta["rem_indptr"][6] + 1
    elif what == "rem_col":
        meta["rem_col_ind"][0] = n
    elif what == "stripe_ptr":
        meta["stripe_ptr"][1] += 1
    with pytest.raises(ValueError, match=match):
        _check(meta, n, bs)


def test_loaded_file_is_checked(tmp_path, device):
    """A file whose arrays pass the host checks but have a bit past the
    matrix edge is refused when moved to the GPU."""
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300.pbr_io import read_pbr_arrays, write_pbr_arrays
    p = gl.csr_to_pbr(_matrix(203), 4, 4, 2)
    f = tmp_path / "m.pbr"
    gl.save_pbr(p, f)
    meta, arrays = read_pbr_arrays(f)
    co = arrays["block_coords"].reshape(-1, 2)
    b = int(np.nonzero(co[:, 1] == 200)[0][0])
    codes = arrays["block_codes"].copy()
    codes[b] |= np.uint64(1 << 3)
    arrays["block_codes"] = codes
    offs = arrays["block_offsets"].copy()
    offs[b + 1:] += 1
    arrays["block_offsets"] = offs
    data = arrays["block_data"]
    k = int(offs[b])
    arrays["block_data"] = np.insert(data, k, np.float32(0.5))
    meta["total_nnz"] += 1
    write_pbr_arrays(f, meta, arrays)
    q = gl.load_pbr(f)
    with pytest.raises(ValueError, match="past the matrix edge"):
        q.to(device)
