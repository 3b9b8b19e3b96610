"""Format tools beyond the hot path: pbr_to_csr (including the partial last
stripe the reference rejects), pbr_analyze_csr, the autotuner."""
import numpy as np
import pytest
import scipy.sparse as sp

from tests._cases import GOLDEN, load_builder_cases, random_csr

pytestmark = pytest.mark.gpu


def _gold():
    z = np.load(GOLDEN / "pbr_to_csr_cases.npz")
    return {str(n): (z[f"{n}/out_indptr"], z[f"{n}/out_indices"], z[f"{n}/out_data"]) for n in z["names"]}


CASES = load_builder_cases()


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_device_pbr_to_csr_matches_reference_golden(case, device):
    """gl_pbr_to_csr on the device build of each builder case: bit-exact
    against the reference pbr_to_csr's output (pbr_matrix.cpp:289-338), and
    for ragged last stripes (where the reference throws) against the input."""
    from page_rank_gb300 import graph_link as gl
    name, A, br, bc, mn, ref = case
    gold = _gold()
    p = gl.csr_to_pbr(A, br, bc, mn)
    indptr = np.zeros(A.shape[0] + 1, A.indptr.dtype)
    indices = np.zeros(A.nnz, A.indices.dtype)
    data = np.zeros(A.nnz, A.data.dtype)
    gl.pbr_to_csr(p, indptr, indices, data)
    want = gold.get(name, (A.indptr, A.indices, A.data))
    assert np.array_equal(indptr, want[0]) and np.array_equal(indices, want[1]), name
    assert np.array_equal(data.view(np.uint8), want[2].view(np.uint8)), name


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


@pytest.mark.parametrize("bs,dtype", [(8, np.float32), (4, np.float64), (2, np.float32)])
def test_device_pbr_to_csr_large_clustered_graph(bs, dtype, device):
    """A 2^16-node clustered R-MAT graph (hub stripes cut into pieces by the
    SpMM schedule, tens of thousands of blocks per stripe pattern) round trips
    through the device build and gl_pbr_to_csr, into torch outputs too."""
    import torch
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300 import synth
    A = synth.cluster_rmat_graph(log2n=16, seed=4).A.astype(dtype)
    p = gl.csr_to_pbr(A, bs, bs, bs)
    ip = torch.zeros(A.shape[0] + 1, dtype=torch.int64, device=device)
    ix = torch.zeros(A.nnz, dtype=torch.int64, device=device)
    dv = torch.zeros(A.nnz, dtype=torch.float32 if dtype == np.float32 else torch.float64, device=device)
    gl.pbr_to_csr(p, ip, ix, dv)
    assert np.array_equal(ip.cpu().numpy(), A.indptr) and np.array_equal(ix.cpu().numpy(), A.indices)
    assert np.array_equal(dv.cpu().numpy(), A.data)


def test_pbr_analyze_csr_counts(device):
    from page_rank_gb300 import graph_link as gl
    A = random_csr(256, 0.05)
    st = gl.pbr_analyze_csr(A, 4, 4, min_nnz_coverage=10)
    assert st["accounted_nnz"] + st["remainder_nnz"] == A.nnz
    assert sum(st["patterns"].values()) >= st["accounted_blocks"]
    pops = {c: bin(c).count("1") for c in st["patterns"]}
    covered = sum(n * pops[c] for c, n in st["patterns"].items() if n * pops[c] >= 10)
    assert covered == st["accounted_nnz"]


@pytest.mark.parametrize("bs,cov", [(8, 1), (8, 1000), (4, 50), (2, 7)])
def test_device_block_patterns_against_numpy(bs, cov, device):
    """gl_pbr_block_patterns against numpy's unique on the same codes (codes
    with bit 63 set included) and the coverage rule's totals."""
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300 import synth
    from page_rank_gb300.pbr import block_patterns
    A = synth.cluster_rmat_graph(log2n=15, seed=6).A
    p = gl.csr_to_pbr(A, bs, bs, 0)
    codes = np.asarray(p.block_codes, dtype=np.uint64)
    u_np, c_np = np.unique(codes, return_counts=True)
    u, c, tot = block_patterns(p._build.codes, cov)
    assert np.array_equal(u, u_np) and np.array_equal(c, c_np)
    pops = np.array([bin(int(x)).count("1") for x in u_np], dtype=np.int64)
    cover = pops * c_np
    keep = cover >= cov
    assert tot == {"accounted_nnz": int(cover[keep].sum()), "remainder_nnz": int(cover[~keep].sum()),
                   "accounted_patterns": int(keep.sum()), "accounted_blocks": int(c_np[keep].sum())}
    if bs == 8:
        assert (u_np >> np.uint64(63)).any()      # the sort handles the sign bit of the high word


def test_autotuner_picks_a_measured_candidate(device):
    from page_rank_gb300 import synth
    from page_rank_gb300.autotune import autotune
    g = synth.cluster_zipf_graph(log2n=12, mean_degree=10.0, seed=8)
    r = autotune(g.A, 32, device=device, candidates=[(2, 2, 0), (4, 4, 0), (8, 8, 0)], steps=2)
    assert (r.block_size, r.min_nnz, r.column_tile) in [(b, m, t) for b, m, t, *_ in r.table]
    assert r.ms_per_step == pytest.approx(min(row[3] for row in r.table), abs=1e-3)
