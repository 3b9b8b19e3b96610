"""Fused PBR + CSR-remainder SpMM against the FP64 oracle.

Mirrors the reference grid (Tests/test_spmm.py:37-88: atol 1e-4) and adds the
relative bound Y vs scipy FP64 <= 1e-5 (nonnegative inputs, so no
cancellation), 3-D batches, FP64 matrices and empty edge cases."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle.spmm import spmm_csr_fp64
from tests._cases import random_csr, random_x

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


def _gl():
    from page_rank_gb300 import graph_link
    return graph_link


def _check(Y, Yref):
    Y = np.asarray(Y, dtype=np.float64)
    assert Y.shape == Yref.shape
    assert np.allclose(Y, Yref, atol=1e-4), f"max abs diff {np.abs(Y - Yref).max():.3e}"
    scale = np.maximum(np.abs(Yref), 1e-30)
    rel = (np.abs(Y - Yref) / scale)[np.abs(Yref) > 1e-30]
    assert rel.size == 0 or rel.max() <= REL_TOL, f"max rel err {rel.max():.3e}"


@pytest.mark.parametrize("N", [64, 128, 1024])
@pytest.mark.parametrize("num_features", [8, 64, 256])
@pytest.mark.parametrize("density", [0.05, 0.15])
@pytest.mark.parametrize("block_size", [2, 4, 8])
@pytest.mark.parametrize("min_nnz", [1, 4])
def test_spmm_accuracy(N, num_features, density, block_size, min_nnz, device):
    A = random_csr(N, density)
    X = random_x(N, num_features)
    pbr = _gl().csr_to_pbr(A, block_rows=block_size, block_cols=block_size,
                           min_nnz_per_block=min_nnz).to(device)
    Y = _gl().pbr_matmul(pbr, torch.from_numpy(X).to(device)).cpu().numpy()
    _check(Y, spmm_csr_fp64(A, X))


@pytest.mark.parametrize("num_features", [1, 2, 3, 5, 6, 7, 9, 12, 17, 33, 65, 130])
@pytest.mark.parametrize("block_size", [2, 4, 8])
@pytest.mark.parametrize("min_nnz", [1, 4])
def test_spmm_odd_feature_counts(num_features, block_size, min_nnz, device):
    A = random_csr(128, 0.1)
    X = random_x(128, num_features)
    pbr = _gl().csr_to_pbr(A, block_rows=block_size, block_cols=block_size,
                           min_nnz_per_block=min_nnz).to(device)
    Y = _gl().pbr_matmul(pbr, torch.from_numpy(X).to(device)).cpu().numpy()
    _check(Y, spmm_csr_fp64(A, X))


@pytest.mark.parametrize("block_size", [2, 4, 8])
def test_spmm_batched_3d_and_ragged_rows(block_size, device):
    A = random_csr(203, 0.08, m=203)
    rng = np.random.default_rng(3)
    X = rng.random((3, 203, 40)).astype(np.float32)
    pbr = _gl().csr_to_pbr(A, block_rows=block_size, block_cols=block_size, min_nnz_per_block=2).to(device)
    Y = _gl().pbr_matmul(pbr, torch.from_numpy(X).to(device)).cpu().numpy()
    _check(Y, spmm_csr_fp64(A, X))


@pytest.mark.parametrize("F", [1, 3, 16, 20, 64, 100])
def test_spmm_float64(F, device):
    A = random_csr(300, 0.05, dtype=np.float64)
    X = np.random.default_rng(1).random((300, F))
    pbr = _gl().csr_to_pbr(A, block_rows=4, block_cols=4, min_nnz_per_block=2).to(device)
    Y = _gl().pbr_matmul(pbr, torch.from_numpy(X).to(device)).cpu().numpy()
    assert np.allclose(Y, spmm_csr_fp64(A, X), rtol=1e-12, atol=1e-12)


def test_spmm_rectangular(device):
    A = random_csr(96, 0.1, m=160)
    X = random_x(160, 64)
    pbr = _gl().csr_to_pbr(A, block_rows=8, block_cols=8, min_nnz_per_block=3).to(device)
    Y = _gl().pbr_matmul(pbr, torch.from_numpy(X).to(device)).cpu().numpy()
    _check(Y, spmm_csr_fp64(A, X))


def test_spmm_empty_matrix_and_all_remainder(device):
    gl = _gl()
    A = sp.csr_matrix((64, 64), dtype=np.float32)
    pbr = gl.csr_to_pbr(A, 4, 4, 1).to(device)
    X = torch.rand(64, 16, device=device)
    assert torch.count_nonzero(gl.pbr_matmul(pbr, X)) == 0
    B = random_csr(64, 0.1)
    pbr = gl.csr_to_pbr(B, 8, 8, 65).to(device)    # nothing packs: all remainder
    assert pbr.accounted_blocks() == 0
    Xn = random_x(64, 16)
    _check(gl.pbr_matmul(pbr, torch.from_numpy(Xn).to(device)).cpu().numpy(), spmm_csr_fp64(B, Xn))


def test_spmm_reference_uploaded_arrays(device):
    """A matrix whose arrays came from elsewhere (the oracle builder, standing
    in for the reference's host builder) works after the stripe index is
    derived on the device."""
    import oracle
    from page_rank_gb300 import pbr as pbrmod
    from page_rank_gb300 import native
    A = random_csr(256, 0.05)
    o = oracle.csr_to_pbr(A.indptr, A.indices, A.data, 256, 256, 4, 4, 2)
    meta = {
        "codes": torch.from_numpy(o["block_codes"].view(np.int64)).to(device),
        "coords": torch.from_numpy(o["block_coords"]).to(device),
        "offsets": torch.from_numpy(o["block_offsets"]).to(device),
        "data": torch.from_numpy(o["block_data"]).to(device),
        "rem_indptr": torch.from_numpy(o["remainder_indptr"]).to(device),
        "rem_col_ind": torch.from_numpy(o["remainder_col_ind"]).to(device),
        "rem_vals": torch.from_numpy(o["remainder_data"]).to(device),
    }
    meta["stripe_ptr"] = pbrmod.stripe_index(meta["coords"], 256, 4)
    X = random_x(256, 32)
    Xt = torch.from_numpy(X).to(device)
    Y = torch.empty(256, 32, device=device)
    desc = pbrmod.matrix_desc(meta, 256, 256, 4, 4)
    ws = pbrmod.spmm_workspace(meta, desc, 1, 32, device)
    native.check(native.lib().gl_pbr_spmm(desc, Xt.data_ptr(), Y.data_ptr(), 1, 32,
                                          ws.data_ptr() if ws is not None else None,
                                          ws.numel() if ws is not None else 0,
                                          torch.cuda.current_stream().cuda_stream))
    _check(Y.cpu().numpy(), spmm_csr_fp64(A, X))


def test_spmm_unsupported_block_and_errors(device):
    gl = _gl()
    A = random_csr(64, 0.1)
    pbr = gl.csr_to_pbr(A, block_rows=3, block_cols=3, min_nnz_per_block=1).to(device)
    with pytest.raises(ValueError, match="Only 2x2, 4x4, and 8x8"):
        gl.pbr_matmul(pbr, torch.rand(64, 4, device=device))
    pbr_host = gl.csr_to_pbr(A, 2, 2, 1)
    with pytest.raises(RuntimeError, match="not on GPU"):
        gl.pbr_batched_matmul_cuda(pbr_host, torch.rand(64, 4, device=device))
    with pytest.raises(TypeError):
        gl.pbr_matmul(pbr_host, torch.rand(64, 4))
    with pytest.raises(ValueError):
        gl.pbr_matmul(pbr_host.to(device), torch.rand(63, 4, device=device))


def test_to_semantics(device):
    gl = _gl()
    A = random_csr(64, 0.1)
    p = gl.csr_to_pbr(A)
    assert gl.get_pbr_gpu_meta(p) is None
    q = p.to("cuda")
    assert q is not p and gl.get_pbr_gpu_meta(q) is not None
    # the reference compares str(torch.device(...)): "cuda:0" matches the
    # tensors' device, bare "cuda" does not and yields a fresh copy
    assert q.to("cuda:0") is q
    assert q.to("cuda") is not q
    c = q.to("cpu")
    assert gl.get_pbr_gpu_meta(c) is None
    gl.clear_pbr_gpu_meta(q)
    assert gl.get_pbr_gpu_meta(q) is None


def test_host_batches_pipeline(device):
    """spmm_host_batches: host batches in, host results out, copies overlapped."""
    from page_rank_gb300.streaming import spmm_host_batches
    gl = _gl()
    A = random_csr(512, 0.05)
    pbr = gl.csr_to_pbr(A, 8, 8, 4).to(device)
    xs = [torch.from_numpy(random_x(512, 64, seed=s)).pin_memory() for s in range(5)]
    ys = [torch.empty(512, 64).pin_memory() for _ in range(5)]
    spmm_host_batches(pbr, xs, ys)
    torch.cuda.synchronize()
    for x, y in zip(xs, ys):
        _check(y.numpy(), spmm_csr_fp64(A, x.numpy()))


@pytest.mark.parametrize("F", [1, 129, 256, 300, 520])
@pytest.mark.parametrize("block_size", [4, 8])
def test_spmm_multi_tile_with_heavy_stripes(F, block_size, device):
    """Several column tiles per stripe (one decoded list consumed once per
    tile, or decoded again when a stripe's rows do not fit it) together with
    heavy stripes cut into pieces: a hub row and a hub column."""
    rng = np.random.default_rng(5)
    n = 3000
    A = random_csr(n, 0.004, seed=11).tolil()
    A[17, :] = (rng.random(n) < 0.6).astype(np.float32) * rng.random(n).astype(np.float32)
    A[:, 40] = (rng.random((n, 1)) < 0.3).astype(np.float32)
    A = sp.csr_matrix(A, dtype=np.float32)
    A.eliminate_zeros()
    X = random_x(n, F, seed=3)
    pbr = _gl().csr_to_pbr(A, block_rows=block_size, block_cols=block_size, min_nnz_per_block=2).to(device)
    Xd = torch.from_numpy(X).to(device)
    Y = _gl().pbr_matmul(pbr, Xd).cpu().numpy()
    _check(Y, spmm_csr_fp64(A, X))
    Y2 = _gl().pbr_matmul(pbr, Xd).cpu().numpy()   # the workspace is left clean for the next call
    assert np.array_equal(Y, Y2)


@pytest.mark.parametrize("F", [2, 5, 16])
def test_spmm_float64_heavy_stripes_one_column_tiles(F, device):
    """FP64 with fewer than 17 columns runs one column per tile (list-free
    path, X read with the row stride F) including heavy stripes."""
    rng = np.random.default_rng(8)
    n = 2500
    A = random_csr(n, 0.004, dtype=np.float64, seed=4).tolil()
    A[9, :] = (rng.random(n) < 0.5) * rng.random(n)
    A = sp.csr_matrix(A, dtype=np.float64)
    A.eliminate_zeros()
    X = rng.random((n, F))
    pbr = _gl().csr_to_pbr(A, block_rows=8, block_cols=8, min_nnz_per_block=2).to(device)
    Y = _gl().pbr_matmul(pbr, torch.from_numpy(X).to(device)).cpu().numpy()
    assert np.allclose(Y, spmm_csr_fp64(A, X), rtol=1e-12, atol=1e-12)


@pytest.mark.skipif(not torch.cuda.is_available() or torch.cuda.device_count() < 2,
                    reason="needs two visible GPUs")
def test_spmm_wide_tiles_on_a_second_device():
    """The per-device launch attributes: a 128-column FP32 SpMM (dynamic
    shared memory above the 48 KiB default) on device 1 after device 0."""
    gl = _gl()
    A = random_csr(2048, 0.01, seed=21)
    X = random_x(2048, 128, seed=3)
    Yref = spmm_csr_fp64(A, X)
    for dev in ("cuda:0", "cuda:1"):
        pbr = gl.csr_to_pbr(A, block_rows=8, block_cols=8, min_nnz_per_block=2).to(dev)
        Y = gl.pbr_matmul(pbr, torch.from_numpy(X).to(dev)).cpu().numpy()
        _check(Y, Yref)


def test_spmm_from_two_host_threads(device):
    """Two host threads launching wide SpMMs on their own streams at once
    (the HTTP server's thread pool does this): both results exact."""
    import threading
    gl = _gl()
    A = random_csr(4096, 0.004, seed=22)
    X = random_x(4096, 128, seed=4)
    Yref = spmm_csr_fp64(A, X)
    pbr = gl.csr_to_pbr(A, block_rows=8, block_cols=8, min_nnz_per_block=2).to(device)
    Xd = torch.from_numpy(X).to(device)
    out, errors = {}, []

    def work(k):
        try:
            idx = torch.device(device).index
            torch.cuda.set_device(idx if idx is not None else torch.cuda.current_device())
            s = torch.cuda.Stream(device)
            with torch.cuda.stream(s):
                ys = [gl.pbr_matmul(pbr, Xd) for _ in range(4)]
            s.synchronize()
            out[k] = [y.cpu().numpy() for y in ys]
        except BaseException as exc:        # surfaced below
            errors.append(exc)

    ts = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(120)
    assert not errors, errors
    for k in range(2):
        for Y in out[k]:
            _check(Y, Yref)
