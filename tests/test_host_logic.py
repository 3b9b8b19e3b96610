"""Host-side logic that needs no GPU: normalize_transition_matrix against the
reference's own output (golden), the sparse normalization used in-kernel,
dtype dispatch, error behaviour without a device, synthetic generators."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from tests._cases import GOLDEN


def test_normalize_matches_reference_golden():
    from page_rank_gb300 import graph_link as gl
    z = np.load(GOLDEN / "normalize_cases.npz")
    for i in range(int(z["count"])):
        k = f"c{i}"
        A = sp.csr_matrix((z[f"{k}/data"], z[f"{k}/indices"], z[f"{k}/indptr"]), shape=tuple(z[f"{k}/shape"]))
        out = gl.normalize_transition_matrix(A)
        assert np.array_equal(out.indptr, z[f"{k}/out_indptr"])
        assert np.array_equal(out.indices, z[f"{k}/out_indices"])
        assert np.array_equal(out.data.view(np.uint8), z[f"{k}/out_data"].view(np.uint8))


def test_sparse_normalization_agrees_off_dangling_columns():
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300.transition import normalize_columns
    z = np.load(GOLDEN / "normalize_cases.npz")
    A = sp.csr_matrix((z["c0/data"], z["c0/indices"], z["c0/indptr"]), shape=tuple(z["c0/shape"]))
    dense = gl.normalize_transition_matrix(A).toarray()
    sparse, dmask = normalize_columns(A)
    s = sparse.toarray()
    assert np.array_equal(s[:, ~dmask], dense[:, ~dmask])
    assert (s[:, dmask] == 0).all() and np.allclose(dense[:, dmask], 1.0 / A.shape[0])


def test_pybind_overload_order_dtype_dispatch():
    from page_rank_gb300.graph_link import _dtypes
    i32, i64 = np.zeros(1, np.int32), np.zeros(1, np.int64)
    f32, f64 = np.zeros(1, np.float32), np.zeros(1, np.float64)
    assert _dtypes(i32, i32, f32) == (np.int32, np.float32)
    assert _dtypes(i64, i64, f32) == (np.int64, np.float32)
    assert _dtypes(i32, i32, f64) == (np.int32, np.float64)
    assert _dtypes(i64, i32, f64) == (np.int64, np.float64)


def test_builder_needs_a_device_and_rejects_bad_types():
    from page_rank_gb300 import graph_link as gl
    A = sp.random(8, 8, density=0.3, format="csr", dtype=np.float32, random_state=0)
    with pytest.raises(TypeError):
        gl.csr_to_pbr(A.toarray())
    with pytest.raises(TypeError):
        gl.csr_to_pbr(A, min_nnz_per_block=256)
    if not torch.cuda.is_available():
        with pytest.raises(RuntimeError):
            gl.csr_to_pbr(A)


def test_cpu_matmul_raises_like_reference():
    from page_rank_gb300 import graph_link as gl
    with pytest.raises(TypeError):
        gl.pbr_batched_matmul_cpu(None, torch.zeros(2, 2))


def test_synthetic_generators_are_column_stochastic_and_seeded():
    from page_rank_gb300 import synth
    for g in (synth.sbm_graph(8, 16, 0.3, 0.01, seed=1),
              synth.cluster_rmat_graph(log2n=10, seed=2),
              synth.cluster_zipf_graph(log2n=10, mean_degree=6.0, seed=3)):
        cs = np.asarray(g.A.sum(axis=0)).ravel()
        assert np.allclose(cs[~g.dangling], 1.0, atol=1e-5)
        assert (cs[g.dangling] == 0).all()
        assert g.A.has_canonical_format
    a = synth.cluster_zipf_graph(log2n=10, mean_degree=6.0, seed=3).A
    b = synth.cluster_zipf_graph(log2n=10, mean_degree=6.0, seed=3).A
    assert (a != b).nnz == 0
    sets = synth.seed_sets(100, 10, 1, 32, seed=4)
    assert all(1 <= len(s) <= 32 and len(np.unique(s)) == len(s) for s in sets)


def test_certified_tolerance():
    from page_rank_gb300.engine import certified_tolerance
    assert certified_tolerance(1e-6, 0.85) == pytest.approx(1e-6 * 0.15 / 0.85)


def test_topk_oracle_matches_numpy_sort():
    """The top-k oracle is numpy's descending sort for distinct values and
    takes the lowest rows among equal values."""
    from oracle import topk as ot
    rng = np.random.default_rng(0)
    X = rng.random((500, 3)).astype(np.float32)
    v, r = ot.topk_columns(X, 10)
    for c in range(3):
        order = np.argsort(-X[:, c], kind="stable")[:10]
        assert np.array_equal(r[c], order) and np.array_equal(v[c], X[order, c])
    Z = np.zeros((6, 1), np.float32)
    Z[4, 0] = 1.0
    v, r = ot.topk_columns(Z, 3)
    assert r[0].tolist() == [4, 0, 1]
    v, r = ot.topk_columns(Z, 8)
    assert r[0].tolist()[-2:] == [-1, -1] and np.isneginf(v[0, -1])


def test_dangling_bitmap_matches_host_packing():
    """The device-side dangling bitmap of the request path packs bits like
    the engine's host helper (bit j % 32 of word j // 32)."""
    from page_rank_gb300.engine import _bitmap_from_mask
    from page_rank_gb300.transition import dangling_bitmap
    rng = np.random.default_rng(2)
    for n in (1, 31, 32, 33, 100, 1000):
        m = rng.random(n) < 0.5
        m[-1] = True
        assert torch.equal(dangling_bitmap(torch.from_numpy(m)), _bitmap_from_mask(m, "cpu"))


def test_warm_start_gate_keeps_prediction_only_when_it_pays():
    """The gate predicts until it has a measurement, then only while the
    estimated saving (iterations x seconds per column-iteration) beats the
    prediction's cost, probing again every probe_every batches."""
    import numpy as np
    from page_rank_gb300.warmstart import WarmStartGate
    g = WarmStartGate(probe_every=4, rate=0.5, smoothing=0.0)
    assert g.want_prediction()                                   # nothing measured yet
    # residual 8x smaller: log(8) / log(2) = 3 iterations saved per column,
    # each worth 1 ms per column, against 5 ms of prediction per column
    g.record(pred_seconds=0.010, step_seconds=0.002, columns=2, r_warm=np.array([1.0, 1.0]),
             r_cold=np.array([8.0, 8.0]))
    assert abs(g.saved_iters - 3.0) < 1e-12
    decisions = [g.want_prediction() for _ in range(6)]          # calls 2..7: only call 4 probes
    assert decisions == [False, False, True, False, False, False]
    # a cheap prediction pays: 3 x 1 ms > 0.5 ms
    g.record(pred_seconds=0.001, step_seconds=0.002, columns=2, r_warm=np.array([1.0, 1.0]),
             r_cold=np.array([8.0, 8.0]))
    assert g.want_prediction()
    # a start that is no better than the cold one saves nothing
    g2 = WarmStartGate(smoothing=0.0)
    g2.record(0.001, 0.002, 1, np.array([2.0]), np.array([1.0]))
    assert g2.saved_iters == 0.0 and not g2.want_prediction()


def test_cpulist_parsing():
    from page_rank_gb300.hostmem import _parse_cpulist, restore_cpus
    assert _parse_cpulist("0-3,8,10-11\n") == [0, 1, 2, 3, 8, 10, 11]
    assert _parse_cpulist("") == []
    restore_cpus({"bound": False})          # nothing recorded: no change


def test_seed_set_index_matches_per_set_unique():
    """The engine's host seed-set index: distinct seeds per set in increasing
    order, weight = multiplicity / set size (duplicates merge)."""
    import numpy as np
    from page_rank_gb300.engine import seed_set_index
    rng = np.random.default_rng(3)
    sets = [rng.integers(0, 50, rng.integers(1, 30)) for _ in range(100)] + [np.array([7, 7, 7]), np.arange(5)]
    ptr, rows, w = seed_set_index(sets)
    assert ptr.dtype == np.int32 and rows.dtype == np.int32 and w.dtype == np.float32
    for k, s in enumerate(sets):
        u, c = np.unique(s, return_counts=True)
        assert np.array_equal(rows[ptr[k]:ptr[k + 1]], u)
        assert np.allclose(w[ptr[k]:ptr[k + 1]], c / c.sum())
    e_ptr, e_rows, e_w = seed_set_index([])
    assert e_ptr.tolist() == [0] and e_rows.size == 0 and e_w.size == 0
