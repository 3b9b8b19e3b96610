"""Device top-k of PPR columns (``gl_topk_columns``) against the oracle
(``oracle/topk.py``), bit for bit: values and rows.  GPU only."""
import numpy as np
import pytest
import torch

from oracle import topk as ot

pytestmark = pytest.mark.gpu


def _check(X, k, columns=None):
    from page_rank_gb300.topk import topk_columns
    Xd = torch.from_numpy(X).cuda()
    v, r = topk_columns(Xd, k, columns)
    wv, wr = ot.topk_columns(X, k, columns)
    assert np.array_equal(r.cpu().numpy(), wr)
    assert np.array_equal(v.cpu().numpy().view(np.uint32), wv.view(np.uint32))


@pytest.mark.parametrize("n,K,k,seed", [(1, 1, 1, 0), (10, 3, 4, 1), (1000, 33, 100, 2), (5000, 64, 1, 3),
                                        (70000, 7, 2048, 4), (300000, 40, 50, 5), (17, 5, 40, 6)])
def test_random(n, K, k, seed):
    rng = np.random.default_rng(seed)
    X = (rng.random((n, K)) ** 4).astype(np.float32)
    _check(X, k)


def test_ties_zeros_and_signs():
    rng = np.random.default_rng(9)
    n, K = 20000, 37
    X = rng.choice(np.array([0.0, 1.0, 2.0, -1.0, -0.0, 0.5], np.float32), size=(n, K))
    X[:, 3] = 0.0                       # a column of zeros: ties to the lowest rows
    X[:5, 4] = np.array([3, 1, 3, 2, 3], np.float32)
    X[5:, 4] = 0.0
    for k in (1, 7, 100, 1000):
        _check(X, k)


def test_selected_columns_and_strided_rows():
    rng = np.random.default_rng(12)
    X = rng.random((40000, 256)).astype(np.float32)
    _check(X, 64, columns=[255, 0, 17, 17, 100])
    from page_rank_gb300.topk import topk_columns
    Xd = torch.from_numpy(X).cuda()
    sub = Xd[:, 10:20]                 # row stride 256, 10 columns
    v, r = topk_columns(sub, 8)
    wv, wr = ot.topk_columns(X[:, 10:20], 8)
    assert np.array_equal(r.cpu().numpy(), wr) and np.array_equal(v.cpu().numpy(), wv)


def test_ppr_column_top_nodes():
    """The top nodes of real PPR columns (the serving use): same as sorting
    the full vectors on the host."""
    from page_rank_gb300 import synth
    from page_rank_gb300.engine import PPREngine
    from page_rank_gb300.topk import topk_columns
    g = synth.cluster_rmat_graph(log2n=14, seed=3)
    eng = PPREngine(g.A, block_size=8, min_nnz_per_block=8, dangling=g.dangling)
    sets = [np.array([5]), np.array([1, 900, 4000]), np.array([77])]
    res = eng.solve(sets, alpha=0.85, tol=1e-6)
    v, r = topk_columns(res.X, 25)
    X = res.X.cpu().numpy()
    wv, wr = ot.topk_columns(X, 25)
    assert np.array_equal(r.cpu().numpy(), wr) and np.array_equal(v.cpu().numpy(), wv)


def test_k_zero_and_bounds():
    from page_rank_gb300.topk import topk_columns
    Xd = torch.rand((100, 4), device="cuda")
    v, r = topk_columns(Xd, 0)
    assert v.shape == (4, 0)
    with pytest.raises(ValueError):
        topk_columns(Xd, 4096)
    with pytest.raises(ValueError):
        topk_columns(Xd, 3, columns=[4])
