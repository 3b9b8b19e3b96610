"""The oracle's restated builder against the reference builder's own output
(golden fixtures written by tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

import oracle
from tests._cases import GOLDEN, assert_pbr_equal, load_builder_cases

CASES = load_builder_cases()


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_reference_golden(case):
    name, A, br, bc, mn, ref = case
    got = oracle.csr_to_pbr(A.indptr, A.indices, A.data, A.shape[0], A.shape[1], br, bc, mn)
    assert got["total_nnz"] == ref["total_nnz"]
    assert_pbr_equal(got, ref, name)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_golden_invariants(case):
    """Content invariants of the reference format: offsets advance by popcount,
    kept blocks meet min_nnz, packed + remainder == nnz, remainder rows sorted."""
    name, A, br, bc, mn, ref = case
    codes = ref["block_codes"].astype(np.uint64)
    pops = np.array([bin(int(c)).count("1") for c in codes], dtype=np.int64)
    assert np.array_equal(np.diff(ref["block_offsets"].astype(np.int64)), pops)
    assert (pops >= mn).all()
    assert len(ref["block_data"]) + len(ref["remainder_data"]) == A.nnz
    ip = ref["remainder_indptr"].astype(np.int64)
    for r in range(A.shape[0]):
        row = ref["remainder_col_ind"][ip[r]:ip[r + 1]]
        assert np.all(np.diff(row) > 0)


def test_oracle_pbr_expands_to_input():
    """PBR -> COO recovers the CSR exactly (the reference's pbr_to_csr
    contract, pbr_matrix.cpp:289-338)."""
    for name, A, br, bc, mn, ref in CASES:
        pbr = dict(ref, rows=A.shape[0], cols=A.shape[1], block_rows=br, block_cols=bc)
        indptr, indices, vals = oracle.pbr_to_csr(pbr)
        assert np.array_equal(indptr, A.indptr.astype(indptr.dtype)), name
        assert np.array_equal(indices, A.indices.astype(indices.dtype)), name
        assert np.array_equal(vals, A.data), name


def _pbr_to_csr_golden():
    z = np.load(GOLDEN / "pbr_to_csr_cases.npz")
    return {str(n): (z[f"{n}/out_indptr"], z[f"{n}/out_indices"], z[f"{n}/out_data"]) for n in z["names"]}


def test_reference_pbr_to_csr_golden_pinned():
    """The reference pbr_to_csr's output (golden) is the input CSR of every
    case it accepts, and the oracle's expansion agrees with it bit for bit."""
    gold = _pbr_to_csr_golden()
    assert len(gold) >= 10
    for name, A, br, bc, mn, ref in CASES:
        if name not in gold:
            assert A.shape[0] % br != 0, name     # only ragged cases are left out
            continue
        gip, gix, gdv = gold[name]
        assert np.array_equal(gip, A.indptr) and np.array_equal(gix, A.indices), name
        assert np.array_equal(gdv.view(np.uint8), A.data.view(np.uint8)), name
        pbr = dict(ref, rows=A.shape[0], cols=A.shape[1], block_rows=br, block_cols=bc)
        indptr, indices, vals = oracle.pbr_to_csr(pbr)
        assert np.array_equal(indptr, gip.astype(indptr.dtype)) and np.array_equal(indices, gix), name
        assert np.array_equal(vals, gdv), name


def test_bucket_chain_shape():
    ch = oracle.bucket_chain(362, 5000)
    assert ch[0, 0] == 0 and ch[0, 1] >= 362
    # every growth happens when the count passes the previous bucket count
    for (c0, b0), (c1, b1) in zip(ch[:-1], ch[1:]):
        assert c1 == b0 + 1 and b1 > b0
