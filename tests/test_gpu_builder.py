"""GPU builder parity: bit-exact against the oracle (and the reference's
golden output), including the order of blocks inside each stripe."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from tests._cases import PBR_KEYS, assert_pbr_equal, load_builder_cases

pytestmark = pytest.mark.gpu

CASES = load_builder_cases()


def _gpu(A, br, bc, mn):
    from page_rank_gb300 import graph_link as gl
    p = gl.csr_to_pbr(A, block_rows=br, block_cols=bc, min_nnz_per_block=mn)
    d = {k: getattr(p, k) for k in PBR_KEYS}
    d["total_nnz"] = p.total_nnz
    return p, d


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_builder_matches_reference_golden(case, device):
    name, A, br, bc, mn, ref = case
    p, got = _gpu(A, br, bc, mn)
    assert got["total_nnz"] == ref["total_nnz"]
    assert_pbr_equal(got, ref, name)
    expect_cls = {(np.dtype(np.int32), np.dtype(np.float32)): "PBRMatrixInt32Float",
                  (np.dtype(np.int64), np.dtype(np.float32)): "PBRMatrixInt64Float",
                  (np.dtype(np.int32), np.dtype(np.float64)): "PBRMatrixInt32Double",
                  (np.dtype(np.int64), np.dtype(np.float64)): "PBRMatrixInt64Double"}
    assert type(p).__name__ == expect_cls[(A.indices.dtype, A.data.dtype)]


@pytest.mark.parametrize("seed", range(8))
def test_builder_random_vs_oracle(seed, device):
    rng = np.random.default_rng(1000 + seed)
    for _ in range(10):
        n = int(rng.integers(1, 2000))
        m = int(rng.integers(1, 2000))
        dens = float(rng.choice([0.002, 0.01, 0.05, 0.2]))
        A = sp.random(n, m, density=dens, format="csr", dtype=np.float32,
                      random_state=int(rng.integers(1 << 30)))
        br = int(rng.choice([1, 2, 3, 4, 8]))
        bc = br if rng.random() < 0.7 else int(rng.choice([1, 2, 4, 8]))
        mn = int(rng.integers(0, 12))
        if rng.random() < 0.25:
            A = A.astype(np.float64)
        if rng.random() < 0.25:
            A = sp.csr_matrix((A.data, A.indices.astype(np.int64), A.indptr.astype(np.int64)), shape=A.shape)
        want = oracle.csr_to_pbr(A.indptr, A.indices, A.data, n, m, br, bc, mn)
        _, got = _gpu(A, br, bc, mn)
        assert_pbr_equal(got, want, f"n={n} m={m} b={br}x{bc} min={mn}")


def test_builder_int32_key_truncation(device):
    n = 150000
    r = np.random.default_rng(5)
    k = 300000
    A = sp.csr_matrix((r.random(k).astype(np.float32), (r.integers(0, n, k), r.integers(0, n, k))),
                      shape=(n, n))
    for br, mn in ((2, 1), (4, 2)):
        want = oracle.csr_to_pbr(A.indptr, A.indices, A.data, n, n, br, br, mn)
        _, got = _gpu(A, br, br, mn)
        assert_pbr_equal(got, want, f"truncation b={br}")


def test_builder_rehash_within_and_across_stripes(device):
    """Stripes with many distinct blocks (the map grows mid-stripe) followed
    by small ones (it keeps its buckets)."""
    rng = np.random.default_rng(9)
    dense = sp.random(24, 20000, density=0.3, format="csr", dtype=np.float32, random_state=1)
    sparse = sp.random(200, 20000, density=0.001, format="csr", dtype=np.float32, random_state=2)
    A = sp.vstack([sparse, dense, sparse]).tocsr()
    for br in (2, 8):
        want = oracle.csr_to_pbr(A.indptr, A.indices, A.data, A.shape[0], A.shape[1], br, br, 1)
        _, got = _gpu(A, br, br, 1)
        assert_pbr_equal(got, want, f"rehash b={br}")


def test_builder_rejects_bad_input(device):
    from page_rank_gb300 import graph_link as gl
    A = sp.random(16, 16, density=0.3, format="csr", dtype=np.float32, random_state=0)
    with pytest.raises(ValueError):
        gl.csr_to_pbr(A, block_rows=9, block_cols=9)   # 81 bits > 64
    with pytest.raises(TypeError):
        gl.csr_to_pbr(A, min_nnz_per_block=300)
    with pytest.raises(TypeError):
        gl.csr_to_pbr(A.toarray())


def test_noncanonical_input_is_canonicalized(device):
    from page_rank_gb300 import graph_link as gl
    indptr = np.array([0, 3, 5, 5, 7], np.int32)
    indices = np.array([3, 1, 0, 2, 2, 1, 0], np.int32)
    data = np.arange(1, 8, dtype=np.float32)
    A = sp.csr_matrix((data, indices, indptr), shape=(4, 4))
    C = A.copy()
    C.sum_duplicates()
    want = oracle.csr_to_pbr(C.indptr, C.indices, C.data, 4, 4, 2, 2, 2)
    _, got = _gpu(A, 2, 2, 2)
    assert_pbr_equal(got, want, "canonicalized")


def test_builder_hub_stripes_vs_oracle(device):
    """Clustered R-MAT graph whose hub rows put hundreds to thousands of
    distinct blocks into one stripe (the one-CTA ordering path, with rehashes
    inside the stripe), several block shapes."""
    from page_rank_gb300 import synth
    g = synth.cluster_rmat_graph(log2n=15, cluster=64, mean_degree=16, p_intra=0.7, seed=4)
    A = g.A
    n = A.shape[0]
    rows = np.repeat(np.arange(n), np.diff(A.indptr))
    key = (rows // 8).astype(np.int64) * (n // 8 + 1) + A.indices // 8
    distinct = np.bincount(np.unique(key) // (n // 8 + 1))
    assert distinct.max() > 1000 and (distinct > 64).sum() > 300
    for br, mn in ((8, 8), (4, 2), (2, 1)):
        want = oracle.csr_to_pbr(A.indptr, A.indices, A.data, n, A.shape[1], br, br, mn)
        _, got = _gpu(A, br, br, mn)
        assert_pbr_equal(got, want, f"hub b={br} min={mn}")


@pytest.mark.parametrize("br,bc,mn", [(6, 10, 2), (12, 5, 3), (16, 4, 4), (32, 2, 2)])
def test_builder_tall_blocks_vs_oracle(br, bc, mn, device):
    """Block heights that give a stripe 8, 16 or 32 lanes in the count pass
    (four, two or one stripe per warp), on the hub graph, so short stripes,
    long ones and hub stripes all occur."""
    from page_rank_gb300 import synth
    g = synth.cluster_rmat_graph(log2n=14, cluster=64, mean_degree=16, p_intra=0.7, seed=6)
    A = g.A
    n = A.shape[0]
    want = oracle.csr_to_pbr(A.indptr, A.indices, A.data, n, A.shape[1], br, bc, mn)
    _, got = _gpu(A, br, bc, mn)
    assert_pbr_equal(got, want, f"tall b={br}x{bc} min={mn}")


@pytest.mark.parametrize("rows_per_stripe", [2, 8])
def test_builder_validation_in_long_stripes(rows_per_stripe, device):
    """Out-of-range, unsorted and duplicate columns inside stripes long
    enough for the CTA-parallel count are rejected with the same statuses
    as in short ones."""
    import torch

    from page_rank_gb300 import native
    from page_rank_gb300.pbr import build_pbr_device
    dense = sp.random(16, 30000, density=0.3, format="csr", dtype=np.float32, random_state=3)
    dense.sort_indices()
    ip = torch.from_numpy(dense.indptr.astype(np.int32)).to(device)
    dv = torch.from_numpy(dense.data).to(device)
    good = dense.indices.astype(np.int32)
    assert np.diff(dense.indptr).max() * rows_per_stripe > 4096   # a hub stripe, counted by a CTA
    build_pbr_device(ip, torch.from_numpy(good).to(device), dv, 16, 30000, rows_per_stripe, rows_per_stripe, 1)
    k = int(dense.indptr[3]) + 100           # an entry in the middle of row 3
    bad_range = good.copy()
    bad_range[k] = 30000 + 5
    with pytest.raises(native.GLValueError, match="out of range"):
        build_pbr_device(ip, torch.from_numpy(bad_range).to(device), dv, 16, 30000, rows_per_stripe,
                         rows_per_stripe, 1)
    for bad in (good.copy(), good.copy()):
        bad[k], bad[k + 1] = bad[k + 1], bad[k]
        break
    unsorted = bad
    dup = good.copy()
    dup[k + 1] = dup[k]
    for arr in (unsorted, dup):
        with pytest.raises(native.GLError) as ei:
            build_pbr_device(ip, torch.from_numpy(arr).to(device), dv, 16, 30000, rows_per_stripe,
                             rows_per_stripe, 1)
        assert ei.value.code == native.GL_ERR_NONCANONICAL


def test_fill_repeated_after_one_count(device):
    """gl_pbr_build_fill run twice after one gl_pbr_build_count on the same
    workspace writes the same arrays both times: the fill resets the
    counters its kernels draw stripes from (short stripes, long ones in
    shared and in global scratch)."""
    import torch

    from page_rank_gb300 import native, synth
    from page_rank_gb300.pbr import _stream_handle
    g = synth.cluster_rmat_graph(log2n=13, cluster=64, mean_degree=16, p_intra=0.7, seed=8)
    A = g.A
    n, nnz = A.shape[0], A.nnz
    ip = torch.from_numpy(A.indptr.astype(np.int32)).to(device)
    ix = torch.from_numpy(A.indices.astype(np.int32)).to(device)
    dv = torch.from_numpy(A.data.astype(np.float32)).to(device)
    L = native.lib()
    ws_bytes = int(L.gl_pbr_build_workspace_bytes(n, n, nnz, 8, 8))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=device)
    stream = _stream_handle(device)
    counts = native.BuildCounts()
    native.check(L.gl_pbr_build_count(ip.data_ptr(), ix.data_ptr(), native.GL_I32, n, n, nnz, 8, 8, 8,
                                      ws.data_ptr(), ws_bytes, counts, stream))
    assert counts.max_stripe_blocks > 64
    want = oracle.csr_to_pbr(A.indptr, A.indices, A.data, n, n, 8, 8, 8)
    nb, packed, rem = counts.num_blocks, counts.packed_nnz, counts.remainder_nnz
    for _ in range(2):
        out = {"block_codes": torch.empty(nb, dtype=torch.int64, device=device),
               "block_coords": torch.empty(2 * nb, dtype=torch.int32, device=device),
               "block_offsets": torch.empty(nb + 1, dtype=torch.int32, device=device),
               "block_data": torch.empty(packed, dtype=torch.float32, device=device),
               "remainder_indptr": torch.empty(n + 1, dtype=torch.int32, device=device),
               "remainder_col_ind": torch.empty(rem, dtype=torch.int32, device=device),
               "remainder_data": torch.empty(rem, dtype=torch.float32, device=device)}
        sp_ptr = torch.empty(-(-n // 8) + 1, dtype=torch.int32, device=device)
        native.check(L.gl_pbr_build_fill(
            ip.data_ptr(), ix.data_ptr(), dv.data_ptr(), native.GL_I32, native.GL_F32, n, n, nnz, 8, 8, 8,
            ws.data_ptr(), ws_bytes, counts, *(out[k].data_ptr() for k in PBR_KEYS), sp_ptr.data_ptr(), stream))
        torch.cuda.synchronize(device)
        got = {k: v.cpu().numpy() for k, v in out.items()}
        got["block_codes"] = got["block_codes"].view(np.uint64)
        assert_pbr_equal(got, want, "repeated fill")
