"""The HTTP contract of POST /api/ppr and GET /api/health.

CPU: contract and error paths through FastAPI's TestClient (skipped where
FastAPI is absent).  GPU: the request body solved on the device against the
FP64 oracle of the reference's semantics (dense uniform dangling columns,
one column per seed, mean)."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import ppr as oppr


def _app():
    pytest.importorskip("fastapi")
    from page_rank_gb300.server import app as mod
    return mod


def _post(mod, body):
    """Call the POST /api/ppr handler the way FastAPI would (validated model);
    returns (status, json)."""
    from fastapi import HTTPException
    try:
        return 200, mod.run_ppr(mod.PPRRequest(**body))
    except HTTPException as e:
        return e.status_code, {"detail": e.detail}


def _request(seeds=("a",)):
    nodes = [{"id": x} for x in "abcdef"]
    edges = [{"source": "a", "target": "b"}, {"source": "b", "target": "c", "weight": 2.0},
             {"source": "c", "target": "a"}, {"source": "d", "target": "a"},
             {"source": "e", "target": "f", "weight": -1.0}, {"source": "a", "target": "zz"}]
    return {"graph": {"nodes": nodes, "edges": edges, "warnings": []},
            "params": {"alpha": 0.85, "maxIter": 100, "tolerance": 1e-6, "topX": 3, "seeds": list(seeds)}}


def test_routes_registered():
    mod = _app()
    paths = {(r.path, tuple(sorted(getattr(r, "methods", []) or []))) for r in mod.app.routes}
    assert ("/api/health", ("GET",)) in paths
    assert ("/api/ppr", ("POST",)) in paths


def test_health_contract():
    import torch
    body = _app().health()
    assert set(body) == {"status", "cuda", "device"} and body["status"] == "ok"
    assert body["cuda"] == torch.cuda.is_available()


def test_errors_contract():
    import torch
    mod = _app()
    if not torch.cuda.is_available():
        assert _post(mod, _request())[0] == 503
        return
    bad = _request()
    bad["graph"]["nodes"] = []
    assert _post(mod, bad)[0] == 422
    assert _post(mod, _request(seeds=("nope",)))[0] == 422
    code, body = _post(mod, _request())
    assert code == 200
    assert set(body) == {"ranks", "iterations", "converged", "convergenceHistory", "degrees"}


@pytest.mark.gpu
def test_request_solution_matches_reference_semantics(device):
    from page_rank_gb300 import graph_link as gl
    from page_rank_gb300.transition import solve_edge_list_request
    req = _request(seeds=("a", "d"))
    ids = [n["id"] for n in req["graph"]["nodes"]]
    index_of = {x: i for i, x in enumerate(ids)}
    src = [e["source"] for e in req["graph"]["edges"]]
    dst = [e["target"] for e in req["graph"]["edges"]]
    w = [e.get("weight", 1.0) for e in req["graph"]["edges"]]
    out = solve_edge_list_request(ids, index_of, src, dst, w, [0, 3], 0.85, 300, 1e-7)
    # reference semantics on the host in FP64
    rows, cols, vals = [], [], []
    for s, t, x in zip(src, dst, w):
        if s in index_of and t in index_of and x > 0:
            rows.append(index_of[t]); cols.append(index_of[s]); vals.append(x)
    A = sp.csr_matrix((np.array(vals, np.float32), (rows, cols)), shape=(6, 6))
    dense = gl.normalize_transition_matrix(A)
    X = oppr.direct_solve_fp64(dense, oppr.teleport_matrix(6, [[0], [3]]), 0.85)
    r = X.mean(axis=1)
    r /= r.sum()
    assert np.abs(out["ranks"] - r).sum() < 1e-6
    assert out["converged"]
    assert out["out_deg"]["a"] == 2.0 and out["in_deg"]["a"] == 2.0 and out["in_deg"]["f"] == 1.0
