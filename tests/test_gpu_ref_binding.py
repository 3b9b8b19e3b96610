"""The reference-side ctypes binding (tests/ref_binding_stub.py) run against
this library: the reference's pbr_batched_matmul_cuda body replaced by
pbr_spmm_gb300 must give the CSR product for 2-D and 3-D inputs, FP32 and
FP64, and raise the reference's ValueError for an unsupported block size."""
import importlib.util
import os
import pathlib

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle.spmm import spmm_csr_fp64
from page_rank_gb300 import graph_link as gl
from page_rank_gb300 import native

pytestmark = pytest.mark.gpu


def _stub():
    native.lib()
    os.environ["GL_GB300_LIB"] = str(native.LIB_PATH)
    path = pathlib.Path(__file__).with_name("ref_binding_stub.py")
    spec = importlib.util.spec_from_file_location("ref_binding_stub", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _matrix(n, dtype, seed):
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=12.0 / n, format="csr", random_state=rng, dtype=np.float64)
    A = A + sp.eye(n, format="csr")
    hub = sp.csr_matrix((rng.random(3000), (np.full(3000, 7), rng.integers(0, n, 3000))), shape=(n, n))
    A = (A + hub).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    return A.astype(dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("bs,min_nnz", [(8, 4), (4, 2)])
def test_stub_spmm(dtype, bs, min_nnz):
    mod = _stub()
    dev = torch.device("cuda", 0)
    A = _matrix(5000, dtype, 3)
    pbr = gl.csr_to_pbr(A, bs, bs, min_nnz).to(dev)
    meta = dict(gl.get_pbr_gpu_meta(pbr))
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    for shape in ((5000, 33), (2, 5000, 16)):
        x = torch.rand(shape, dtype=tdt, device=dev)
        y = mod.pbr_spmm_gb300(pbr, meta, x)
        torch.cuda.synchronize()
        xs = x.cpu().numpy().reshape(-1, 5000, shape[-1])
        ys = y.cpu().numpy().reshape(-1, 5000, shape[-1])
        for b in range(xs.shape[0]):
            ref = spmm_csr_fp64(A, xs[b])
            rel = np.abs(ys[b] - ref).max() / np.abs(ref).max()
            assert rel < (1e-5 if dtype == np.float32 else 1e-12)


def test_stub_unsupported_block():
    mod = _stub()
    dev = torch.device("cuda", 0)
    A = _matrix(600, np.float32, 4)
    pbr = gl.csr_to_pbr(A, 3, 3, 2).to(dev)
    meta = dict(gl.get_pbr_gpu_meta(pbr))
    with pytest.raises(ValueError, match="Unsupported block size"):
        mod.pbr_spmm_gb300(pbr, meta, torch.rand((600, 4), device=dev))
