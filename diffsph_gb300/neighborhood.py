"""Drop-in for the reference neighbor search (src/diffSPH/v2/modules/neighborhood.py).

``neighborSearch`` keeps the reference signature and return value
``(datastructure, neighborDict)``; the pairs come from the sm_103a cell-grid search of
libsph103.so (sph_neighbor_count / sph_neighbor_fill), which applies the reference's exact
fp32 filter, so the pair set equals the reference's. The reference reuses a Verlet
candidate list between calls (``priorState``, ``neighborDatastructure``); this search is
exact on every call, so those arguments are accepted and only echoed back.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .solver import _f, _stream, domain_struct


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def exact_pairs(x_query, x_ref, h_ref, config, compute_kernels=True, count_only=False):
    """Exact scatter-mode pairs (|x_i - x_j| <= h_j, the reference's fp32 test).

    Returns (i, j, q, xhat, h_j, W, gradW, counts, offsets) as CUDA tensors; rows sorted by
    i, columns by j (original indices)."""
    lib = _lib.load()
    xq = torch.as_tensor(x_query).to("cuda", torch.float32).contiguous()
    xr = torch.as_tensor(x_ref).to("cuda", torch.float32).contiguous()
    hr = torch.as_tensor(h_ref).to("cuda", torch.float32).contiguous()
    nq, nr = xq.shape[0], xr.shape[0]
    dom = domain_struct(config)
    hmax = float(hr.max()) if nr else 1.0
    nbytes = ctypes.c_size_t()
    _lib.check("sph_neighbor_workspace_bytes",
               lib.sph_neighbor_workspace_bytes(nq, nr, ctypes.byref(dom), hmax, ctypes.byref(nbytes)))
    ws = torch.empty(int(nbytes.value) + 256, dtype=torch.uint8, device="cuda")
    wsp = (ws.data_ptr() + 255) & ~255
    counts = torch.empty(nq, dtype=torch.int32, device="cuda")
    offsets = torch.empty(nq + 1, dtype=torch.int64, device="cuda")
    st = _stream()
    _lib.check("sph_neighbor_count", lib.sph_neighbor_count(
        _ptr(xq), nq, _ptr(xr), _ptr(hr), nr, ctypes.byref(dom), hmax, ctypes.c_void_p(wsp), nbytes.value,
        _ptr(counts), _ptr(offsets), st))
    npairs = int(offsets[-1].item())
    if count_only:
        return counts, offsets
    i = torch.empty(npairs, dtype=torch.int64, device="cuda")
    j = torch.empty(npairs, dtype=torch.int64, device="cuda")
    q = torch.empty(npairs, device="cuda")
    xh = torch.empty(npairs, 2, device="cuda")
    hp = torch.empty(npairs, device="cuda")
    W = torch.empty(npairs, device="cuda") if compute_kernels else None
    G = torch.empty(npairs, 2, device="cuda") if compute_kernels else None
    _lib.check("sph_neighbor_fill", lib.sph_neighbor_fill(
        _ptr(xq), nq, _ptr(xr), _ptr(hr), nr, ctypes.byref(dom), hmax, ctypes.c_void_p(wsp), nbytes.value,
        _ptr(offsets), npairs, _ptr(i), _ptr(j), _ptr(q), _ptr(xh), _ptr(hp), _ptr(W), _ptr(G), st))
    return i, j, q, xh, hp, W, G, counts, offsets


def neighborSearch(queryState, referenceState, config, computeKernels=True, priorState=None,
                   neighborDatastructure=None, verbose=False):
    """Same contract as neighborhood.py:491-593 (scatter mode, h_ij = h_j)."""
    i, j, q, xh, hp, W, G, counts, offsets = exact_pairs(
        queryState["positions"], referenceState["positions"], referenceState["supports"], config, computeKernels)
    numNeighbors = counts
    neighborOffsets = offsets[:-1].to(torch.int32)
    nb = {
        "indices": (i, j), "fullIndices": (i, j), "distances": q, "vectors": xh, "supports": hp,
        "initialPositions": (queryState["positions"], referenceState["positions"]),
        "numNeighbors": numNeighbors, "neighborOffsets": neighborOffsets,
        "fullNumNeighbors": numNeighbors, "fullNeighborOffsets": neighborOffsets,
    }
    if computeKernels:
        nb["kernels"] = W
        nb["gradients"] = G
    ds = neighborDatastructure if neighborDatastructure is not None else {
        "referencePositions": referenceState["positions"], "referenceSupports": referenceState["supports"],
        "sortIndex": torch.arange(torch.as_tensor(referenceState["positions"]).shape[0]),
    }
    return ds, nb
