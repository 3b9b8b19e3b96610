"""The window kernel (64-row windows, diagonal X tile staged in shared memory
by bulk asynchronous copies) against the FP64 product and the stripe kernel.

Both kernels sit behind gl_pbr_spmm; the descriptor's ``kernel`` field picks
one.  Shapes cover every block size, one and several column tiles, partial
tiles, batches, rectangular matrices (windows past the last X row),
row counts that are not multiples of the window or block size, heavy
stripes cut into pieces, an empty matrix, determinism and the workspace's
error word."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle.spmm import spmm_csr_fp64
from tests._cases import random_csr

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


def _run(A, X, block, min_nnz, kernel, device, piece_work=None):
    """Y of gl_pbr_spmm with the given kernel; checks the error word."""
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300 import native
    from page_rank_gb300.pbr import matrix_desc, spmm_workspace
    rows, cols = A.shape
    pbr = gl.csr_to_pbr(A, block_rows=block, block_cols=block, min_nnz_per_block=min_nnz).to(device)
    meta = gl.get_pbr_gpu_meta(pbr)
    if piece_work is not None:
        meta["piece_work"] = piece_work
    desc = matrix_desc(meta, rows, cols, block, block)
    desc.kernel = kernel
    Xd = torch.from_numpy(np.ascontiguousarray(X)).to(device)
    B = 1 if X.ndim == 2 else X.shape[0]
    F = X.shape[-1]
    Y = torch.full((B, rows, F) if X.ndim == 3 else (rows, F), float("nan"), device=device)
    ws = spmm_workspace(meta, desc, B, F, device)
    L = native.lib()
    st = torch.cuda.current_stream(device).cuda_stream
    native.check(L.gl_pbr_spmm(desc, Xd.data_ptr(), Y.data_ptr(), B, F, ws.data_ptr(), ws.numel(), st))
    assert L.gl_spmm_workspace_error(ws.data_ptr(), st) == 0, L.gl_last_error()
    return Y.cpu().numpy(), desc


def _check(Y, Yref):
    Y = np.asarray(Y, dtype=np.float64)
    assert Y.shape == Yref.shape
    assert np.isfinite(Y).all()
    err = np.abs(Y - Yref)
    assert err.max(initial=0.0) <= 1e-4
    rel = err / np.maximum(np.abs(Yref), 1e-30)
    assert rel[np.abs(Yref) > 1e-30].max(initial=0.0) <= REL_TOL, rel.max()


def _cluster_graph(log2n, seed=5):
    from page_rank_gb300 import synth
    return synth.cluster_rmat_graph(log2n=log2n, cluster=64, mean_degree=16, p_intra=0.7, seed=seed).A


@pytest.mark.parametrize("block", [2, 4, 8])
@pytest.mark.parametrize("F", [64, 68, 128, 200, 256])
def test_window_kernel_clustered_graph(block, F, device):
    A = _cluster_graph(14)
    X = np.random.default_rng(F).random((A.shape[1], F)).astype(np.float32)
    ref = spmm_csr_fp64(A, X)
    Yw, desc = _run(A, X, block, block, 2, device)
    assert desc.num_pieces > 0
    _check(Yw, ref)
    Ys, _ = _run(A, X, block, block, 1, device)
    _check(Ys, ref)


@pytest.mark.parametrize("piece_work", [32, 64, 192])
def test_window_kernel_small_pieces(piece_work, device):
    A = _cluster_graph(13, seed=9)
    X = np.random.default_rng(2).random((A.shape[1], 64)).astype(np.float32)
    Y, desc = _run(A, X, 8, 8, 2, device, piece_work=piece_work)
    assert desc.num_pieces > 0
    _check(Y, spmm_csr_fp64(A, X))


def test_window_kernel_batch(device):
    A = _cluster_graph(12)
    X = np.random.default_rng(3).random((3, A.shape[1], 64)).astype(np.float32)
    Y, _ = _run(A, X, 8, 8, 2, device)
    _check(Y, spmm_csr_fp64(A, X))


@pytest.mark.parametrize("shape", [(1000, 150), (100, 3000), (1000, 1000), (37, 64), (2100, 2100)])
@pytest.mark.parametrize("block", [4, 8])
def test_window_kernel_ragged_and_rectangular(shape, block, device):
    rows, cols = shape
    A = random_csr(rows, 0.02, seed=rows + cols, m=cols).tolil()
    rng = np.random.default_rng(1)
    for r in range(0, rows, 7):            # some near-diagonal structure as well
        c = min(cols - 1, r + int(rng.integers(0, 5)))
        A[r, c] = 0.5
    A = sp.csr_matrix(A, dtype=np.float32)
    X = rng.random((cols, 64)).astype(np.float32)
    Y, _ = _run(A, X, block, 2, 2, device)
    _check(Y, spmm_csr_fp64(A, X))


@pytest.mark.parametrize("F", [64, 256])
def test_window_kernel_hub_row_and_column(F, device):
    rng = np.random.default_rng(5)
    n = 3000
    A = random_csr(n, 0.004, seed=11).tolil()
    A[17, :] = (rng.random(n) < 0.6).astype(np.float32) * rng.random(n).astype(np.float32)
    A[:, 40] = (rng.random((n, 1)) < 0.3).astype(np.float32)
    A = sp.csr_matrix(A, dtype=np.float32)
    A.eliminate_zeros()
    X = rng.random((n, F)).astype(np.float32)
    Y, desc = _run(A, X, 8, 2, 2, device)
    assert desc.num_pieces > 0
    _check(Y, spmm_csr_fp64(A, X))
    Y2, _ = _run(A, X, 8, 2, 2, device)
    assert np.array_equal(Y, Y2)           # deterministic


def test_window_kernel_empty_matrix(device):
    A = sp.csr_matrix((300, 300), dtype=np.float32)
    X = np.random.default_rng(0).random((300, 64)).astype(np.float32)
    Y, _ = _run(A, X, 8, 8, 2, device)
    assert np.array_equal(Y, np.zeros_like(Y))
