"""GPU metadata registry for PBR matrices.

Same contract as the reference registry (``graph_link/pbr_registry.py:1-31``):
metadata is keyed by ``id(pbr_mat)``, purged by a ``weakref.finalize`` when
the matrix dies, and a size check drops entries whose id was recycled.  The
table is guarded by a lock because the serving layer calls in from several
threads (the reference's plain dict is not thread-safe).
"""
from __future__ import annotations

import threading
import weakref

_PBR_GPU_CACHE: dict[int, dict] = {}
_LOCK = threading.Lock()


def get_pbr_gpu_meta(pbr_mat):
    obj_id = id(pbr_mat)
    with _LOCK:
        meta = _PBR_GPU_CACHE.get(obj_id)
        if meta is not None and meta["rem_indptr"].numel() != pbr_mat.rows + 1:
            del _PBR_GPU_CACHE[obj_id]
            return None
        return meta


def set_pbr_gpu_meta(pbr_mat, meta_dict):
    obj_id = id(pbr_mat)
    with _LOCK:
        _PBR_GPU_CACHE[obj_id] = meta_dict
    try:
        weakref.finalize(pbr_mat, _pop, obj_id)
    except TypeError:
        pass


def _pop(obj_id):
    with _LOCK:
        _PBR_GPU_CACHE.pop(obj_id, None)


def clear_pbr_gpu_meta(pbr_mat):
    _pop(id(pbr_mat))
