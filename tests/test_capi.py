"""C-ABI library: loads, exports every declared symbol, validates arguments
(all without touching a GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import _lib, _dev

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(REPO, "include", "sci_gb300.h")).read()
    return sorted(set(re.findall(r"^int\s+(sci_\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def L():
    sci.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(L):
    declared = header_symbols()
    assert len(declared) >= 14
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(_lib.exported_symbols()) == declared


def test_version_and_error_buffer(L):
    assert L.sci_version() >= 100
    buf = ctypes.create_string_buffer(8)
    n = L.sci_last_error(buf, len(buf))
    assert n >= 0


def test_argument_checks_return_codes_without_gpu(L):
    s = None
    assert L.sci_A(None, None, None, 8, 16, 16, s) == -1
    assert "null pointer" in _lib.last_error()
    assert L.sci_A(None, None, None, 0, 16, 16, s) == -1
    assert "invalid sizes" in _lib.last_error()
    assert L.sci_pack_mask(1, 1, 1, 33, 4, 4, s) == -1
    assert "B=33" in _lib.last_error()
    # proj_gap with accelerate but no y1
    assert L.sci_proj_gap(1, 1, None, 1, None, 1, 2, ctypes.c_float(1.0), 1, 8, 4, 4, s) == -1
    assert "y1" in _lib.last_error()
    # aliasing is rejected
    assert L.sci_proj_gap(1, 1, None, 1, 1, 1, 1, ctypes.c_float(1.0), 1, 8, 4, 4, s) == -1
    # TV: weight must be positive; workspace must be large enough
    n = ctypes.c_size_t()
    assert L.sci_tv_workspace_bytes(4, 64, 64, 5, ctypes.byref(n)) == 0 and n.value > 0
    assert L.sci_tv_chambolle(1, 2, None, 4, 64, 64, ctypes.c_float(0.0), ctypes.c_float(2e-4),
                              5, None, None, 3, n.value, s) == -1
    assert "weight" in _lib.last_error()
    assert L.sci_tv_chambolle(1, 2, None, 4, 64, 64, ctypes.c_float(0.1), ctypes.c_float(2e-4),
                              5, None, None, 3, n.value - 1, s) == -1
    assert "workspace" in _lib.last_error()


def test_workspace_sizes_scale():
    L = _lib.load()
    n5, n30 = ctypes.c_size_t(), ctypes.c_size_t()
    L.sci_tv_workspace_bytes(24, 2048, 2048, 5, ctypes.byref(n5))
    L.sci_tv_workspace_bytes(24, 2048, 2048, 30, ctypes.byref(n30))
    # a single pass keeps p on chip: only energies and flags
    assert n5.value < 1 << 16
    # multi-pass runs carry p (2 planes, two buffers) through the workspace
    assert n30.value >= 2 * 2 * 24 * 2048 * 2048 * 4
    o = _lib.SolveOpts()
    o.tv_iter_max = 5
    nb = ctypes.c_size_t()
    assert L.sci_solver_workspace_bytes(24, 2048, 2048, ctypes.byref(o), ctypes.byref(nb)) == 0
    # ADMM keeps theta, v and two b buffers: 4 stacks
    assert nb.value >= 4 * 24 * 2048 * 2048 * 4


def test_schedule_and_layout_helpers():
    assert np.array_equal(_dev.schedule(0.5, 3), np.full(3, 0.5, np.float32))
    assert _dev.schedule([1, 2, 3], 3).dtype == np.float32
    with pytest.raises(ValueError):
        _dev.schedule([1, 2], 3)
    from sci_algorithms_gb300.pnp_sci_algo import _total_iters, _check_plugin, _flip
    assert _total_iters(50, None) == 50
    assert _total_iters([10, 10, 5], [1, 2, 3]) == 25
    _check_plugin("ffdnet")  # the CNN denoisers run with a model= network
    _check_plugin("fastdvdnet")
    with pytest.raises(ValueError):
        _check_plugin("wavelet")
    _check_plugin("tv", "ATV_ClipA")  # the MATLAB twin's TV names are accepted
    with pytest.raises(ValueError):
        _check_plugin("tv", "ATV_ClipC")
    assert _flip("updown", 1) and not _flip("updown", 0)
    assert _flip("downup", 0) and not _flip("plain", 1)


def test_unsupported_projmeth_raises():
    with pytest.raises(ValueError):
        sci.admmdenoise_cacti(np.zeros((4, 4, 1)), np.zeros((4, 4, 2)), None, None,
                              projmeth="ista")


def test_no_gpu_fails_loudly(monkeypatch):
    import torch
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(RuntimeError, match="CUDA GPU"):
        sci.A_(np.zeros((4, 4, 2)), np.ones((4, 4, 2)))


def test_argument_checks_of_the_wider_entry_points(L):
    """Argument errors of the spectral, batched, unrolled, MATLAB-TV, metrics
    and CNN entry points return -1 with a message before any device work
    (no GPU needed)."""
    s = None
    n = ctypes.c_size_t()
    # spectral: step must be >= 1; null buffers
    assert L.sci_cassi_workspace_bytes(28, 256, 256, 0, 5, ctypes.byref(n)) == -1
    assert "step" in _lib.last_error()
    o = _lib.SolveOpts()
    o.iters, o.tv_iter_max = 4, 5
    assert L.sci_cassi_gap_tv(None, 1, 1, 1, 1, 28, 256, 256, 2, ctypes.byref(o), 1, 1, s) == -1
    assert "null" in _lib.last_error()
    # batched: 1..256 items, tv_iter_max in [2, 5]
    items = (_lib.BatchItem * 1)()
    assert L.sci_batch_workspace_bytes(items, 0, 5, ctypes.byref(n)) == -1
    assert "items" in _lib.last_error()
    assert L.sci_batch_workspace_bytes(items, 1, 9, ctypes.byref(n)) == -1
    assert "tv_iter_max" in _lib.last_error()
    # unrolled: tv_iters in [2, 5], K >= 1
    assert L.sci_unrolled_workspace_bytes(16, 8, 256, 256, 20, 7, ctypes.byref(n)) == -1
    assert "tv_iters" in _lib.last_error()
    assert L.sci_unrolled_workspace_bytes(16, 8, 256, 256, 0, 5, ctypes.byref(n)) == -1
    # MATLAB TVs: unknown kind, aliasing input and output
    assert L.sci_tv_matlab(99, 1, 2, 4, 64, 64, ctypes.c_float(0.1), 5, None, 0, s) == -1
    assert "kind" in _lib.last_error()
    assert L.sci_tv_matlab(1, 1, 1, 4, 64, 64, ctypes.c_float(0.1), 5, None, 0, s) == -1
    # per-frame metrics: frames of at least 7 x 7
    assert L.sci_frame_metrics(1, 2, 4, 5, 64, 1.0, 3, 4, s) == -1
    assert "7 x 7" in _lib.last_error()
    # CNN first layer: null input
    assert L.sci_cnn_conv_thin(None, 16, 32, 48, 8, 64, 64, 96, 1, s) == -1
    assert "null" in _lib.last_error()
    # DenBlock tail: null input, odd padded size, padding as large as the source
    assert L.sci_cnn_den_tail(None, 16, 32, 48, 64, 0, 80, 4, 64, 64, 0, 2, 64, 64, 64, 64, 0,
                              96, s) == -1
    assert "null" in _lib.last_error()
    assert L.sci_cnn_den_tail(16, 32, 48, 64, 80, 0, 96, 4, 63, 63, 0, 2, 63, 64, 63, 63, 0,
                              112, s) == -1
    assert "even" in _lib.last_error()
    assert L.sci_cnn_den_tail(16, 32, 48, 64, 80, 0, 96, 4, 32, 32, 0, 2, 64, 64, 64, 64, 0,
                              112, s) == -1
    assert "padding" in _lib.last_error()
    assert L.sci_cnn_den_tail(16, 32, 48, 64, 80, 0, 96, 4, 64, 64, 3, 2, 64, 64, 64, 64, 0,
                              112, s) == -1
    assert "frames" in _lib.last_error()


def test_noalloc_scratch_limit_is_as_documented(L):
    """The allocation-free TV's fixed 64 KiB scratch holds the workspace of
    742 frames at n_iter_max = 5 and not of 743 (sci_gb300.h)."""
    n = ctypes.c_size_t()
    assert L.sci_tv_workspace_bytes(742, 64, 64, 5, ctypes.byref(n)) == 0 and n.value <= 64 * 1024
    assert L.sci_tv_workspace_bytes(743, 64, 64, 5, ctypes.byref(n)) == 0 and n.value > 64 * 1024
