"""A PBR matrix saved to disk and loaded back is bit-identical and gives
the same SpMM result, bit for bit."""
import numpy as np
import pytest
import torch

from tests._cases import PBR_KEYS, random_csr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bs,mn", [(8, 8), (4, 2), (2, 1)])
def test_save_load_round_trip(tmp_path, bs, mn, device):
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300.pbr_io import load_pbr, save_pbr
    A = random_csr(700, 0.03)
    p = gl.csr_to_pbr(A, bs, bs, mn)
    save_pbr(p, tmp_path / "m.pbr")
    q = load_pbr(tmp_path / "m.pbr", device)
    assert type(q) is type(p) and q.total_nnz == p.total_nnz
    for k in PBR_KEYS:
        a, b = getattr(p, k), getattr(q, k)
        assert a.dtype == b.dtype and np.array_equal(a, b), k
    X = torch.rand((700, 64), device=device)
    y1 = gl.pbr_matmul(p.to(device), X)
    y2 = gl.pbr_matmul(q.to(device), X)
    assert torch.equal(y1, y2)
