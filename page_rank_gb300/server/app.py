"""FastAPI service with the reference's HTTP contract.

Same routes, request / response JSON and error codes as the reference
service (``Backend/server/app.py:41-160``, wire types in
``Frontend/src/lib/ppr/types.ts:5-40``):

* ``GET /api/health`` -> ``{status, cuda, device}``
* ``POST /api/ppr`` with ``{graph: {nodes, edges, format?, warnings}, params:
  {alpha, maxIter, tolerance, topX, seeds}}`` -> ``{ranks, iterations,
  converged, convergenceHistory, degrees: {in, out}}``; 503 without CUDA,
  422 for an empty graph or when no seed names a node.

Differences in *how*, not *what*: the edge list becomes a CSR with numpy
(no per-edge Python loops), dangling sources keep empty columns and their
mass is spread uniformly inside the fused kernel (the reference stores a
dense 1/N column per dangling node, same fixed point), and the power
iteration is the fused GPU step.  One column per seed, stop when the largest
per-column L1 change < tolerance, then the mean over columns renormalized —
as the reference does.
"""
from __future__ import annotations

import numpy as np
import torch
from fastapi import FastAPI, HTTPException
from fastapi.middleware.cors import CORSMiddleware
from pydantic import BaseModel, Field

from ..transition import solve_edge_list_request

app = FastAPI(title="PPR Analyzer backend (GB300)", version="1.0")
app.add_middleware(CORSMiddleware, allow_origins=["*"], allow_methods=["*"], allow_headers=["*"])


class GraphNode(BaseModel):
    id: str


class GraphEdge(BaseModel):
    source: str
    target: str
    weight: float = 1.0


class Graph(BaseModel):
    nodes: list[GraphNode]
    edges: list[GraphEdge]
    format: str | None = None
    warnings: list[str] = Field(default_factory=list)


class PPRParams(BaseModel):
    alpha: float = 0.85
    maxIter: int = 100
    tolerance: float = 1e-6
    topX: int = 10
    seeds: list[str] = Field(default_factory=list)


class PPRRequest(BaseModel):
    graph: Graph
    params: PPRParams


@app.get("/api/health")
def health() -> dict:
    cuda = torch.cuda.is_available()
    return {"status": "ok", "cuda": cuda, "device": torch.cuda.get_device_name(0) if cuda else None}


@app.post("/api/ppr")
def run_ppr(req: PPRRequest) -> dict:
    if not torch.cuda.is_available():
        raise HTTPException(status_code=503, detail="CUDA device not available on the server.")
    g, p = req.graph, req.params
    ids = [n.id for n in g.nodes]
    if not ids:
        raise HTTPException(status_code=422, detail="Graph has no nodes.")
    index_of = {nid: i for i, nid in enumerate(ids)}
    seed_idx = [index_of[s] for s in p.seeds if s in index_of]
    if not seed_idx:
        raise HTTPException(status_code=422, detail="Personalized PageRank requires at least one seed node.")
    src = [e.source for e in g.edges]
    dst = [e.target for e in g.edges]
    w = np.asarray([e.weight for e in g.edges], dtype=np.float64)
    out = solve_edge_list_request(ids, index_of, src, dst, w, seed_idx, p.alpha, p.maxIter, p.tolerance)
    r = out["ranks"]
    return {
        "ranks": {ids[i]: float(r[i]) for i in range(len(ids))},
        "iterations": int(out["iterations"]),
        "converged": bool(out["converged"]),
        "convergenceHistory": [float(h) for h in out["history"]],
        "degrees": {"in": out["in_deg"], "out": out["out_deg"]},
    }
