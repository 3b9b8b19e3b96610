"""Format tools beyond the hot path: pbr_to_csr (including the partial last
stripe the reference rejects), pbr_analyze_csr, the autotuner."""
import numpy as np
import pytest
import scipy.sparse as sp

from tests._cases import random_csr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,bs", [(64, 4), (101, 8), (37, 2)])
def test_pbr_to_csr_roundtrip(n, bs, device):
    from page_rank_gb300 import graph_link as gl
    A = random_csr(n, 0.1)
    p = gl.csr_to_pbr(A, bs, bs, 2)
    indptr = np.zeros(n + 1, np.int32)
    indices = np.zeros(A.nnz, np.int32)
    data = np.zeros(A.nnz, np.float32)
    gl.pbr_to_csr(p, indptr, indices, data)
    assert np.array_equal(indptr, A.indptr) and np.array_equal(indices, A.indices)
    assert np.array_equal(data, A.data)


def test_pbr_analyze_csr_counts(device):
    from page_rank_gb300 import graph_link as gl
    A = random_csr(256, 0.05)
    st = gl.pbr_analyze_csr(A, 4, 4, min_nnz_coverage=10)
    assert st["accounted_nnz"] + st["remainder_nnz"] == A.nnz
    assert sum(st["patterns"].values()) >= st["accounted_blocks"]
    pops = {c: bin(c).count("1") for c in st["patterns"]}
    covered = sum(n * pops[c] for c, n in st["patterns"].items() if n * pops[c] >= 10)
    assert covered == st["accounted_nnz"]


def test_autotuner_picks_a_measured_candidate(device):
    from page_rank_gb300 import synth
    from page_rank_gb300.autotune import autotune
    g = synth.cluster_zipf_graph(log2n=12, mean_degree=10.0, seed=8)
    r = autotune(g.A, 32, device=device, candidates=[(2, 2, 0), (4, 4, 0), (8, 8, 0)], steps=2)
    assert (r.block_size, r.min_nnz, r.column_tile) in [(b, m, t) for b, m, t, *_ in r.table]
    assert r.ms_per_step == pytest.approx(min(row[3] for row in r.table), abs=1e-3)
