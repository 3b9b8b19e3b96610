"""Device edge list -> transition matrix (``gl_edges_to_transition``) against
the reference service's own output (golden fixtures) and the oracle
(``oracle/edges.py``), bit for bit, plus the resident-graph reuse of the
request path.  GPU only."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import edges as oe
from tests._cases import load_edge_cases, without_dense_columns

pytestmark = pytest.mark.gpu
CASES = load_edge_cases()


def _device(n, s, t, w, normalize=True):
    from page_rank_gb300.transition import device_transition
    ip, ix, dv, dg = device_transition(n, s, t, w, torch.device("cuda", 0), normalize=normalize)
    return ip.cpu().numpy(), ix.cpu().numpy(), dv.cpu().numpy(), dg.cpu().numpy()


def _same(got, want_ptr, want_idx, want_val, ctx):
    ip, ix, dv = got[:3]
    assert np.array_equal(ip, np.asarray(want_ptr)), ctx
    assert np.array_equal(ix, np.asarray(want_idx)), ctx
    assert np.array_equal(dv.view(np.uint32), np.asarray(want_val, np.float32).view(np.uint32)), ctx


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_matches_reference_golden(case):
    name, n, s, t, w, A, An = case
    got = _device(n, s, t, w)
    dangling = np.asarray(A.tocsc().sum(axis=0)).ravel() == 0 if n else np.zeros(0, bool)
    assert np.array_equal(got[3], dangling), name
    want = without_dense_columns(An, dangling)
    _same(got, want.indptr, want.indices, want.data, name)
    raw = _device(n, s, t, w, normalize=False)
    A.sort_indices()
    _same(raw, A.indptr, A.indices, A.data, name + " (no normalize)")
    assert not raw[3].any()


@pytest.mark.parametrize("seed,n,m,dups", [(0, 1, 50, 0), (1, 7, 200, 3), (2, 300, 5000, 0),
                                           (3, 4096, 60000, 2), (4, 100000, 400000, 1),
                                           (5, 70000, 9000, 0)])
def test_matches_oracle_seeded(seed, n, m, dups):
    """Random edge lists with invalid edges and duplicates (equal weights, so
    every duplicate order gives the same sums, or distinct weights when
    dups == 1, i.e. at most two copies of a pair)."""
    rng = np.random.default_rng(seed)
    s = rng.integers(-3, n + 3, m)
    t = rng.integers(-3, n + 3, m)
    if dups == 1:
        key = np.unique(np.stack([s, t], 1), axis=0, return_index=True)[1]
        key.sort()
        s, t = s[key], t[key]
        again = rng.random(s.size) < 0.3
        s, t = np.concatenate([s, s[again]]), np.concatenate([t, t[again]])
        w = rng.random(s.size) * 4 + 1e-4
        w[rng.random(s.size) < 0.02] = -1.0
    else:
        w = rng.choice([1.0, 1.0, 0.5, 0.0, np.nan, 3.0], m)
        if dups:
            s[: m // 4] = s[0]   # one hub source: a long column (pairwise recursion)
            t[: m // 4] = rng.integers(0, n, m // 4)
    got = _device(n, s, t, w)
    ip, ix, dv, dg = oe.transition_from_edges(n, s, t, w)
    _same(got, ip, ix, dv, f"seed {seed}")
    assert np.array_equal(got[3], dg)


def test_hub_column_long_pairwise():
    """A column of 300 000 entries with distinct weights: the column sum runs
    through many levels of the pairwise recursion."""
    rng = np.random.default_rng(11)
    n = 400000
    t = rng.permutation(n)[:300000]
    s = np.full(t.size, 17)
    w = rng.random(t.size) * 10 + 1e-3
    got = _device(n, s, t, w)
    ip, ix, dv, dg = oe.transition_from_edges(n, s, t, w)
    _same(got, ip, ix, dv, "hub")
    assert np.array_equal(got[3], dg)


def test_large_against_host_path():
    """2^20 nodes, 8M edges (at most two copies of a pair): the device result
    equals the host path (scipy construction + the reference's normalize
    arithmetic) bit for bit; every non-dangling column sums to 1 within FP32."""
    from page_rank_gb300.transition import edge_list_csr, normalize_columns
    rng = np.random.default_rng(7)
    n, m = 1 << 20, 8 << 20
    s = rng.integers(0, n, m)
    t = (s + rng.integers(-5000, 5000, m)) % n
    order = np.argsort(s * n + t, kind="stable")        # drop third copies of a pair
    k = (s * n + t)[order]
    first = np.r_[0, np.flatnonzero(k[1:] != k[:-1]) + 1]
    rank = np.arange(m) - np.repeat(first, np.diff(np.r_[first, m]))
    keep = np.sort(order[rank < 2])
    s, t = s[keep], t[keep]
    w = rng.random(s.size) + 0.01
    got = _device(n, s, t, w)
    A_norm, dangling = normalize_columns(edge_list_csr(n, s, t, w))
    _same(got, A_norm.indptr, A_norm.indices, A_norm.data, "2^20")
    assert np.array_equal(got[3], dangling)
    col = np.bincount(got[1], weights=got[2].astype(np.float64), minlength=n)
    assert np.abs(col[~dangling] - 1).max() < 1e-5


def test_empty_and_rejected():
    from page_rank_gb300.transition import device_transition
    ip, ix, dv, dg = _device(0, np.zeros(0), np.zeros(0), np.zeros(0))
    assert ip.tolist() == [0] and ix.size == 0 and dg.size == 0
    ip, ix, dv, dg = _device(3, np.zeros(0), np.zeros(0), np.zeros(0))
    assert ip.tolist() == [0, 0, 0, 0] and dg.all()
    with pytest.raises(ValueError):
        device_transition(3, np.zeros(2), np.zeros(3), np.zeros(2), torch.device("cuda", 0))


def test_request_graphs_stay_resident():
    """Two requests over the same edge list build the PBR matrix once; a
    different edge list builds its own."""
    from page_rank_gb300 import transition as tr
    tr.clear_resident_graphs()
    ids = [str(i) for i in range(40)]
    index_of = {x: i for i, x in enumerate(ids)}
    rng = np.random.default_rng(5)
    src = [str(x) for x in rng.integers(0, 40, 150)]
    dst = [str(x) for x in rng.integers(0, 40, 150)]
    w = [1.0] * 150
    a = tr.solve_edge_list_request(ids, index_of, src, dst, w, [0], 0.85, 100, 1e-7)
    first = list(tr._resident.values())[0][0]
    b = tr.solve_edge_list_request(ids, index_of, src, dst, w, [3], 0.85, 100, 1e-7)
    assert len(tr._resident) == 1 and list(tr._resident.values())[0][0] is first
    assert a["iterations"] > 0 and b["iterations"] > 0
    tr.solve_edge_list_request(ids, index_of, src[:-1], dst[:-1], w[:-1], [0], 0.85, 100, 1e-7)
    assert len(tr._resident) == 2
    tr.clear_resident_graphs()
