"""The window-solve warm start's FP64 oracle on the CPU: the series it
truncates converges to the exact PPR vector, start vectors are probability
vectors, the cold residual is one power step, and on the cluster / Zipf
graph class the start cuts the power iterations by more than 1.5x."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import ppr as oppr
from oracle import window_start as ows


def _graph(log2n=11, seed=3):
    from page_rank_gb300 import synth
    g = synth.cluster_zipf_graph(log2n=log2n, mean_degree=20.0, seed=seed)
    assert not g.dangling.any()
    return g.A.astype(np.float64).tocsr()


def _power_iterations(A, X0, V, alpha, thr, maxit=2000):
    X = X0.copy()
    done = np.zeros(X.shape[1], dtype=int)
    for t in range(maxit):
        Xn = alpha * (A @ X) + (1 - alpha) * V
        upd = np.abs(Xn - X).sum(axis=0)
        X = Xn
        newly = (upd < thr) & (done == 0)
        done[newly] = t + 1
        if (done > 0).all():
            break
    return done, X


def test_blocks_hold_the_in_window_entries():
    A = _graph(10)
    B = ows.window_blocks(A, 0.85)
    n = A.shape[0]
    dense = np.eye(n) - 0.85 * A.toarray()
    for w in range(0, n // 64, 5):
        assert np.allclose(B[w], dense[w * 64:(w + 1) * 64, w * 64:(w + 1) * 64])
    # column diagonal dominance: Gauss-Jordan needs no pivoting
    diag = np.abs(np.einsum("wii->wi", B))
    off = np.abs(B).sum(axis=1) - diag
    assert (diag > off).all()


def test_ragged_last_window_is_identity_past_n():
    A = sp.random(1000, 1000, density=0.01, random_state=1, format="csr")
    A = sp.csr_matrix(A / np.maximum(A.sum(axis=0), 1e-30))
    B = ows.window_blocks(A, 0.9)
    assert B.shape == (16, 64, 64)
    tail = 1000 - 15 * 64
    assert np.array_equal(B[15, tail:, tail:], np.eye(64 - tail))
    assert not B[15, tail:, :tail].any() and not B[15, :tail, tail:].any()


def test_series_converges_to_the_exact_vector():
    A = _graph(10)
    n = A.shape[0]
    sets = [np.array([3]), np.array([100, 700, 701]), np.arange(0, 1024, 37)]
    V = oppr.teleport_matrix(n, sets)
    exact = spla.spsolve(sp.identity(n, format="csc") - 0.85 * A.tocsc(), 0.15 * V)
    prev = None
    for L in (0, 2, 4, 40):
        nf = ows.near_field(A, V, 0.85, L)
        assert (nf >= -1e-15).all()
        err = np.abs(nf - exact).sum(axis=0).max()
        if prev is not None:
            assert err < prev
        prev = err
    assert prev < 1e-9


def test_start_is_a_probability_vector():
    A = _graph(10)
    n = A.shape[0]
    V = oppr.teleport_matrix(n, [np.array([5, 9]), np.array([1000])])
    shape = np.full(n, 1.0 / n)
    for L in (0, 1, 3):
        x0 = ows.window_start(A, V, 0.85, L, shape)
        assert np.allclose(x0.sum(axis=0), 1.0)
        assert (x0 >= 0).all()


def test_cold_residual_is_one_power_step():
    from page_rank_gb300 import synth
    g = synth.cluster_zipf_graph(log2n=10, mean_degree=8.0, seed=7)
    A = g.A.astype(np.float64).tocsr().tolil()
    A[:, 11] = 0                                        # a dangling seed
    A = A.tocsr()
    A.eliminate_zeros()
    dangling = np.asarray(A.sum(axis=0)).ravel() == 0
    n = A.shape[0]
    sets = [np.array([11]), np.array([11, 12, 13]), np.array([64, 65, 66, 67])]
    V = oppr.teleport_matrix(n, sets)
    r = ows.cold_residual(A, V, 0.85, dangling)
    d = V[dangling].sum(axis=0)
    step = 0.85 * (A @ V) + (0.15 + 0.85 * d)[None, :] * V
    assert np.allclose(r, np.abs(step - V).sum(axis=0), rtol=1e-12)


def test_start_cuts_iterations_on_the_cluster_zipf_class():
    A = _graph(12)
    n = A.shape[0]
    alpha = 0.85
    thr = 1e-6 * (1 - alpha) / alpha
    from page_rank_gb300 import synth
    sets = synth.seed_sets(n, 8, 1, 32, seed=11)
    V = oppr.teleport_matrix(n, sets)
    u = np.full((n, 1), 1.0 / n)
    _, pr = _power_iterations(A, u, u, alpha, 1e-14)
    near_u = ows.near_field(A, u, alpha, 3)[:, 0]
    far_u = np.maximum(pr[:, 0] - near_u, 0)
    far_u /= far_u.sum()
    cold, Xc = _power_iterations(A, V, V, alpha, thr)
    warm, Xw = _power_iterations(A, ows.window_start(A, V, alpha, 3, far_u), V, alpha, thr)
    assert cold.mean() / warm.mean() >= 1.5, (cold.mean(), warm.mean())
    assert np.abs(Xc - Xw).sum(axis=0).max() < 2e-6
