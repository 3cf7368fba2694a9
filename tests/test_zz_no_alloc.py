"""The allocation-free TV entry point, called through the C ABI.

``sci_tv_chambolle_noalloc`` serves callers that cannot allocate device
memory (a framework that owns every device byte through its own pool, a
plug-in that only receives its input and output buffers): its scratch is a
fixed array inside the library.  This test checks it against the regular
``sci_tv_chambolle`` (caller-provided workspace) on the same input, twice
in a row -- the second call reuses the array the first call left behind --
and that a request beyond the array's limit is refused.  The file sorts
last so that a run stopping at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest
import torch

import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import _dev, _lib

pytestmark = pytest.mark.gpu

ATOL = 2e-5  # the TV tests' per-pixel tolerance


def _frames(F, H, W, seed):
    x = sci.datasets.video_scene(H, W, F, seed=seed)
    return _dev.planar(x)


def _regular(f, weight, K, eps=2e-4):
    nf, H, W = f.shape
    u = torch.empty_like(f)
    steps = torch.zeros(nf, dtype=torch.int32, device=f.device)
    n = ctypes.c_size_t()
    _lib.call("sci_tv_workspace_bytes", nf, H, W, K, ctypes.byref(n))
    ws = torch.empty(n.value, dtype=torch.uint8, device=f.device)
    _lib.call("sci_tv_chambolle", f.data_ptr(), u.data_ptr(), None, nf, H, W, weight, eps, K,
              steps.data_ptr(), None, ws.data_ptr(), n.value, _dev.stream_handle())
    return u, steps


def _noalloc(f, weight, K, eps=2e-4):
    nf, H, W = f.shape
    u = torch.empty_like(f)
    steps = torch.zeros(nf, dtype=torch.int32, device=f.device)
    _lib.call("sci_tv_chambolle_noalloc", f.data_ptr(), u.data_ptr(), None, nf, H, W, weight,
              eps, K, steps.data_ptr(), _dev.stream_handle())
    return u, steps


def test_noalloc_matches_workspace_variant_twice():
    f = _frames(6, 300, 260, seed=21)
    ref, ref_steps = _regular(f, 0.1, 5)
    for _ in range(2):
        u, steps = _noalloc(f, 0.1, 5)
        torch.cuda.synchronize()
        assert float((u - ref).abs().max()) < ATOL
        assert torch.equal(steps, ref_steps)
    # a stop-test case: the energy sums must start from zero on every call
    g = _frames(8, 72, 80, seed=5)
    ref, ref_steps = _regular(g, 0.2, 5, eps=0.05)
    for _ in range(2):
        u, steps = _noalloc(g, 0.2, 5, eps=0.05)
        torch.cuda.synchronize()
        assert float((u - ref).abs().max()) < ATOL
        assert torch.equal(steps, ref_steps)


def test_noalloc_edge_of_its_scratch():
    """742 frames at n_iter_max 5 fill the 64 KiB scratch exactly and run
    (matching the workspace variant); 743 are refused."""
    n = ctypes.c_size_t()
    _lib.call("sci_tv_workspace_bytes", 742, 32, 32, 5, ctypes.byref(n))
    assert n.value <= 64 * 1024
    _lib.call("sci_tv_workspace_bytes", 743, 32, 32, 5, ctypes.byref(n))
    assert n.value > 64 * 1024
    f = _frames(742, 32, 32, seed=3)
    ref, ref_steps = _regular(f, 0.15, 5, eps=0.02)
    u, steps = _noalloc(f, 0.15, 5, eps=0.02)
    torch.cuda.synchronize()
    assert float((u - ref).abs().max()) < ATOL
    assert torch.equal(steps, ref_steps)
    L = _lib.load()
    g = torch.zeros((743, 32, 32), dtype=torch.float32, device=f.device)
    v = torch.empty_like(g)
    assert L.sci_tv_chambolle_noalloc(g.data_ptr(), v.data_ptr(), None, 743, 32, 32, 0.15, 0.02,
                                      5, None, _dev.stream_handle()) == -1
    assert "scratch" in _lib.last_error()


def test_noalloc_rejects_requests_beyond_its_scratch():
    L = _lib.load()
    f = _frames(1, 16, 16, seed=1)
    u = torch.empty_like(f)
    s = _dev.stream_handle()
    assert L.sci_tv_chambolle_noalloc(f.data_ptr(), u.data_ptr(), None, 1, 16, 16, 0.1, 2e-4, 6,
                                      None, s) == -1
    assert "limit of 5" in _lib.last_error()
    assert L.sci_tv_chambolle_noalloc(f.data_ptr(), u.data_ptr(), None, 778, 16, 16, 0.1, 2e-4,
                                      5, None, s) == -1
    assert "scratch" in _lib.last_error()
