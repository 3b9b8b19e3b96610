"""gl_pbr_spmm_static — the SpMM entry point that allocates nothing.

Some callers cannot allocate device memory at the moment they call the
SpMM: a host program that owns all device memory through its own allocator
and hands this library only X and Y, or a latency-critical loop that must
not wait on cudaMalloc / cudaFree.  For them the heavy-stripe scratch lives
in a fixed static device array.  This test calls that entry point through
the C ABI twice in a row and checks both results against gl_pbr_spmm (the
entry point with a caller-provided workspace) within the SpMM tolerance used
by the other tests; it also checks that an oversized request is refused
before anything runs.  It lives in its own file, collected last, and builds
everything it needs itself, so it runs alone or after the other tests."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


def _matrix(device, dtype=np.float32, piece_work=64):
    from page_rank_gb300 import synth
    from page_rank_gb300 import graph_link as gl
    g = synth.cluster_rmat_graph(log2n=14, cluster=64, mean_degree=16, p_intra=0.7, seed=5)
    A = g.A.astype(dtype)
    pbr = gl.csr_to_pbr(A, block_rows=8, block_cols=8, min_nnz_per_block=8).to(device)
    meta = gl.get_pbr_gpu_meta(pbr)
    meta["piece_work"] = piece_work  # small pieces: many heavy stripes use the scratch
    return A, pbr, meta


def _fitting_matrix(device, dtype, batch, features):
    """The case with the smallest pieces whose scratch fits the static array
    (FP64 and batches need more scratch per piece)."""
    from page_rank_gb300 import native
    from page_rank_gb300.pbr import matrix_desc
    L = native.lib()
    for pw in (64, 128, 256):
        A, pbr, meta = _matrix(device, dtype, pw)
        desc = matrix_desc(meta, A.shape[0], A.shape[1], 8, 8)
        if max(int(L.gl_pbr_spmm_workspace_bytes(desc, batch, F)) for F in features) \
                <= native.GL_SPMM_STATIC_SCRATCH_BYTES:
            return A, pbr, meta, desc
    raise AssertionError("no piece size fits the static scratch")


@pytest.mark.parametrize("dtype,batch", [(np.float32, 1), (np.float32, 2), (np.float64, 1), (np.float64, 2)])
def test_static_scratch_spmm_matches_workspace_spmm(device, dtype, batch):
    from page_rank_gb300 import native
    from page_rank_gb300.pbr import spmm_workspace
    A, pbr, meta, desc = _fitting_matrix(device, dtype, batch, (64, 7))
    n = A.shape[0]
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    assert desc.num_pieces > 0, "the case must exercise the heavy-stripe scratch"
    L = native.lib()
    st = torch.cuda.current_stream(device).cuda_stream
    for F in (64, 7):
        X = torch.rand((batch, n, F), device=device, dtype=tdt,
                       generator=torch.Generator(device=device).manual_seed(F))
        need = int(L.gl_pbr_spmm_workspace_bytes(desc, batch, F))
        assert 0 < need <= native.GL_SPMM_STATIC_SCRATCH_BYTES
        ws = spmm_workspace(meta, desc, batch, F, device)
        Y_ref = torch.empty((batch, n, F), device=device, dtype=tdt)
        native.check(L.gl_pbr_spmm(desc, X.data_ptr(), Y_ref.data_ptr(), batch, F, ws.data_ptr(), ws.numel(), st))
        for _ in range(2):                      # two calls in a row share the static array
            Y = torch.full((batch, n, F), float("nan"), device=device, dtype=tdt)
            native.check(L.gl_pbr_spmm_static(desc, X.data_ptr(), Y.data_ptr(), batch, F, st))
            torch.cuda.synchronize(device)
            ref = Y_ref.double()
            err = (Y.double() - ref).abs()
            assert torch.isfinite(Y).all()
            assert float(err.max()) <= 1e-4
            assert float((err / ref.abs().clamp_min(1e-30)).max()) <= REL_TOL
        # and both agree with the FP64 product, batch by batch
        A64 = A.astype(np.float64)
        for b in range(batch):
            Y64 = torch.from_numpy(np.asarray(A64 @ X[b].double().cpu().numpy())).to(device)
            assert float(((Y[b].double() - Y64).abs() / Y64.abs().clamp_min(1e-30)).max()) <= REL_TOL


def test_static_scratch_rejects_oversized_requests(device):
    from page_rank_gb300 import native
    from page_rank_gb300.pbr import matrix_desc
    A, pbr, meta = _matrix(device)
    n = A.shape[0]
    desc = matrix_desc(meta, n, n, 8, 8)
    L = native.lib()
    F = 1 << 20                               # needs far more than the static scratch
    assert int(L.gl_pbr_spmm_workspace_bytes(desc, 1, F)) > native.GL_SPMM_STATIC_SCRATCH_BYTES
    dummy = torch.empty(1, device=device)
    rc = L.gl_pbr_spmm_static(desc, dummy.data_ptr(), dummy.data_ptr(), 1, F,
                              torch.cuda.current_stream(device).cuda_stream)
    assert rc == native.GL_ERR_WORKSPACE
    assert b"static scratch" in L.gl_last_error()
