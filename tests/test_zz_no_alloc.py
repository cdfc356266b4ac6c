"""co_collision_noalloc: the pair sum for callers that cannot allocate device
memory (for example a host whose own memory pool owns the GPU, or one that must
not allocate between time steps). Its scratch is a fixed __device__ array shared
by every call, so this checks calls in a row -- each one after the previous
call has left its partial sums in the array -- against the library's context
entry point co_collision on the same inputs, with the FP64 tolerance of the
other parity tests (1e-12 normwise relative). The sizes cover one slice pair
(2048, 4096), eight slices with a short last tile (1000) and the largest
allowed N with a short last slice (32768). It also checks that a repeated call
leaves the device's free memory unchanged, that NaN inputs come back as
CO_ERR_NONFINITE, and the size limit. Kept in a file of its own that pytest
collects last."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_markers, uniform_bp

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def _inputs(om, N, seed):
    v, w = gaussian_markers(N, 1.0, 0.5, seed=seed)
    v[0] = (7.0, 0.0)                          # one marker outside the domain
    f = om.l2_project(v, w)
    G = om.compute_G(v, om.mass_solve(om.compute_r(f)))
    return v, w, G


def _dev(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).to(dev)  # (2, N) == N x 2


def test_noalloc_matches_context_entry_point(built_lib, collops_mod, oracle_mod):
    import torch

    lib = collops_mod.load_library()
    dev = torch.device("cuda", 0)
    bp = uniform_bp(-6.0, 6.0, 16)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    om = oracle_mod.OracleMesh(bp, bp, 6)
    # the larger calls first, then smaller ones on top of their leftovers
    for N, seed in ((32768, 20), (4096, 21), (1000, 23), (2048, 22)):
        v, w, G = _inputs(om, N, seed)
        ref = np.zeros((N, 2), order="F")
        collops_mod.compute_collision_gpu(ws, ref, v, w, G)
        v_t, G_t = _dev(v, dev), _dev(G, dev)
        w_t = torch.from_numpy(w).to(dev)
        outs = []
        for rep in range(2):
            out_t = torch.full((2, N), np.nan, dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            st = lib.co_collision_noalloc(v_t.data_ptr(), w_t.data_ptr(), G_t.data_ptr(),
                                          out_t.data_ptr(), N, bp[0], bp[-1], bp[0], bp[-1],
                                          None)
            assert st == 0
            torch.cuda.synchronize()
            if rep == 1:
                # a repeated call allocates nothing on the device
                assert torch.cuda.mem_get_info()[0] == free0
            outs.append(out_t.cpu().numpy().T)
        for got in outs:
            assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < TOL64
            assert np.all(got[0] == 0.0)
        assert np.array_equal(outs[0], outs[1])
    ws.close()


def test_noalloc_rejects_nonfinite(built_lib, collops_mod, oracle_mod):
    import torch

    lib = collops_mod.load_library()
    dev = torch.device("cuda", 0)
    bp = uniform_bp(-6.0, 6.0, 16)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    N = 1000
    v, w, G = _inputs(om, N, 24)
    G[17, 1] = np.nan
    v_t, G_t = _dev(v, dev), _dev(G, dev)
    w_t = torch.from_numpy(w).to(dev)
    out_t = torch.full((2, N), 3.0, dtype=torch.float64, device=dev)
    st = lib.co_collision_noalloc(v_t.data_ptr(), w_t.data_ptr(), G_t.data_ptr(),
                                  out_t.data_ptr(), N, bp[0], bp[-1], bp[0], bp[-1], None)
    assert st == 4                                  # CO_ERR_NONFINITE
    torch.cuda.synchronize()
    assert bool((out_t == 3.0).all())               # dot_v untouched


def test_noalloc_rejects_oversize(built_lib, collops_mod):
    lib = collops_mod.load_library()
    assert lib.co_collision_noalloc(None, None, None, None, 32769, -6.0, 6.0, -6.0, 6.0,
                                    None) == 1      # NULL pointers first
    import torch
    x = torch.zeros(2, dtype=torch.float64, device="cuda")
    p = x.data_ptr()
    assert lib.co_collision_noalloc(p, p, p, p, 32769, -6.0, 6.0, -6.0, 6.0, None) == 8
    assert b"32768" in lib.co_strerror(8)
