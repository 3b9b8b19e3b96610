"""Pin the oracle: the restated builder against the reference builder compiled
from its own sources (oracle/_ref), on randomized matrices.  CPU only; skipped
where the reference checkout / build is absent (e.g. on GPU machines)."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from oracle import ref_build
from tests._cases import PBR_KEYS, assert_pbr_equal

core = ref_build.load_reference_core()
pytestmark = pytest.mark.skipif(core is None, reason="reference builder not built (oracle/_ref)")


def _ref(A, br, bc, mn):
    p = core.csr_to_pbr(A.indptr, A.indices, A.data, A.shape[0], A.shape[1], br, bc, mn)
    d = {k: np.asarray(getattr(p, k)) for k in PBR_KEYS}
    d["total_nnz"] = p.total_nnz
    return d


@pytest.mark.parametrize("seed", range(12))
def test_random_matrices(seed):
    rng = np.random.default_rng(seed)
    for _ in range(15):
        n = int(rng.integers(1, 300))
        m = int(rng.integers(1, 300))
        dens = float(rng.choice([0.01, 0.05, 0.2, 0.5]))
        A = sp.random(n, m, density=dens, format="csr", dtype=np.float32,
                      random_state=int(rng.integers(1 << 30)))
        br = int(rng.choice([1, 2, 3, 4, 8]))
        bc = int(rng.choice([1, 2, 4, 8])) if rng.random() < 0.3 else br
        mn = int(rng.integers(0, 10))
        if rng.random() < 0.3:
            A = A.astype(np.float64)
        if rng.random() < 0.3:
            A = sp.csr_matrix((A.data, A.indices.astype(np.int64), A.indptr.astype(np.int64)), shape=A.shape)
        got = oracle.csr_to_pbr(A.indptr, A.indices, A.data, n, m, br, bc, mn)
        want = _ref(A, br, bc, mn)
        assert got["total_nnz"] == want["total_nnz"]
        assert_pbr_equal(got, want, f"seed={seed} n={n} m={m} b={br}x{bc} min={mn}")


def test_int32_key_truncation():
    """Block indices above 2**31 wrap in the int32-keyed map; order must follow."""
    n = 150000
    r = np.random.default_rng(5)
    k = 300000
    A = sp.csr_matrix((r.random(k).astype(np.float32), (r.integers(0, n, k), r.integers(0, n, k))),
                      shape=(n, n))
    got = oracle.csr_to_pbr(A.indptr, A.indices, A.data, n, n, 2, 2, 1)
    assert_pbr_equal(got, _ref(A, 2, 2, 1), "truncation")


def test_unsorted_and_duplicate_input():
    """Non-canonical CSR: the restatement follows the reference even where the
    reference pairs values with the wrong bits."""
    indptr = np.array([0, 3, 5, 5, 7], np.int32)
    indices = np.array([3, 1, 0, 2, 2, 1, 0], np.int32)
    data = np.arange(1, 8, dtype=np.float32)
    for mn in (0, 2, 5):
        got = oracle.csr_to_pbr(indptr, indices, data, 4, 4, 2, 2, mn)
        p = core.csr_to_pbr(indptr, indices, data, 4, 4, 2, 2, mn)
        want = {k: np.asarray(getattr(p, k)) for k in PBR_KEYS}
        assert_pbr_equal(got, want, f"noncanonical min={mn}")
