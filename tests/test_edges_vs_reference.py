"""Pin the edge-list oracle against the reference's own normalize function
(run from the reference checkout) on randomized edge lists.  CPU only;
skipped where the reference checkout is absent (e.g. on GPU machines).

The reference's matrix step (``Backend/server/app.py:111-131``) is restated
in ``tests/golden/make_golden.py:reference_edge_matrix``; the edge lists keep
every duplicate sum independent of scipy's unstable per-row sort (at most
two copies of a pair with distinct weights, or equal weights)."""
import sys

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import edges as oe
from oracle import ref_build
from tests._cases import GOLDEN, without_dense_columns

pytestmark = pytest.mark.skipif(not ref_build.reference_present(), reason="reference checkout absent")


def _reference():
    sys.path.insert(0, str(GOLDEN))
    import make_golden
    return make_golden.reference_edge_matrix, make_golden._reference_normalize()


@pytest.mark.parametrize("seed", range(10))
def test_random_edge_lists(seed):
    edge_matrix, normalize = _reference()
    rng = np.random.default_rng(100 + seed)
    for _ in range(6):
        n = int(rng.integers(1, 400))
        m = int(rng.integers(0, 5000))
        s = rng.integers(-2, n, m)
        t = rng.integers(-2, n, m)
        if rng.random() < 0.5:      # equal weights: any duplicate count
            w = rng.choice([1.0, 1.0, 0.0, -2.0, np.nan], m)
        else:                       # distinct weights, at most two copies of a pair
            key = np.unique(np.stack([s, t], 1), axis=0, return_index=True)[1]
            key.sort()
            s, t = s[key], t[key]
            again = rng.random(s.size) < 0.3
            s, t = np.concatenate([s, s[again]]), np.concatenate([t, t[again]])
            w = rng.random(s.size) * 3 + 1e-3
            w[rng.random(s.size) < 0.05] = -1.0
        A = edge_matrix(n, s, t, w)
        An = normalize(A)
        ip, ix, dv, dg = oe.transition_from_edges(n, s, t, w)
        colsum = np.asarray(A.tocsc().sum(axis=0)).ravel()
        assert np.array_equal(dg, colsum == 0)
        want = without_dense_columns(An, dg)
        assert np.array_equal(ip, want.indptr) and np.array_equal(ix, want.indices)
        assert np.array_equal(dv.view(np.uint32), want.data.astype(np.float32).view(np.uint32))
