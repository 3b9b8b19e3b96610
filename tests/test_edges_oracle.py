"""The edge list -> transition matrix oracle (``oracle/edges.py``) against
the reference service's own output (golden fixtures written by
tests/golden/make_golden.py from ``app.py:111-131`` and the reference
``normalize_transition_matrix``), and its restated numpy pairwise sum
against numpy itself.  CPU only."""
import numpy as np
import pytest

from oracle import edges as oe
from tests._cases import load_edge_cases, without_dense_columns

CASES = load_edge_cases()


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_edge_matrix_matches_reference(case):
    name, n, s, t, w, A, An = case
    indptr, indices, data = oe.edges_to_csr(n, s, t, w)
    A.sort_indices()
    assert np.array_equal(indptr, A.indptr) and np.array_equal(indices, A.indices)
    assert np.array_equal(data.view(np.uint32), A.data.astype(np.float32).view(np.uint32))


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_transition_matches_reference(case):
    name, n, s, t, w, A, An = case
    indptr, indices, data, dangling = oe.transition_from_edges(n, s, t, w)
    colsum = np.asarray(A.tocsc().sum(axis=0)).ravel() if n else np.zeros(0)
    assert np.array_equal(dangling, colsum == 0)
    want = without_dense_columns(An, dangling)
    assert np.array_equal(indptr, want.indptr) and np.array_equal(indices, want.indices)
    assert np.array_equal(data.view(np.uint32), want.data.astype(np.float32).view(np.uint32))


def test_pairwise_sum_is_numpys():
    """first + pairwise(rest) == np.add.reduceat on one segment, for lengths
    across every branch (< 8, <= 128, recursive splits)."""
    rng = np.random.default_rng(3)
    for length in list(range(1, 140)) + [255, 256, 257, 1000, 1031, 4099]:
        a = (rng.random(length) * rng.choice([1e-3, 1.0, 1e3], length)).astype(np.float32)
        want = np.add.reduceat(a, [0])[0]
        assert oe.column_sum_f32(a) == want, length


def test_duplicates_summed_in_input_order():
    w = np.array([1e8, 3.0, 3.0, 3.0])
    indptr, indices, data = oe.edges_to_csr(2, [0] * 4, [1] * 4, w)
    acc = np.float32(1e8)
    for x in w[1:]:
        acc = np.float32(acc + np.float32(x))
    assert indices.tolist() == [0] and data[0] == acc
