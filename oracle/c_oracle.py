"""ctypes front end of the C oracle (``oracle/csrc/sci_oracle.c``).

TEST INFRASTRUCTURE ONLY (see that file's header).  Arrays are float64 in
the planar layout B x H x W; helpers convert from the reference layout
H x W x B.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsci_oracle.so")
_lib = None

_d = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.c_int64


def build():
    """Compile the C oracle with the committed Makefile."""
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile")],
                   check=True, cwd=HERE)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_A.argtypes = [_d, _d, _d, _i64, _i64, _i64]
        L.orc_At.argtypes = [_d, _d, _d, _i64, _i64, _i64]
        L.orc_tv_chambolle.argtypes = [_d, _d, _i64, _i64, _i64, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int), _d]
        L.orc_gap_tv.argtypes = [_d, _d, _d, _d, _i64, _i64, _i64, ctypes.c_int,
                                 _d, _d, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                 _d, _d]
        L.orc_admm_tv.argtypes = [_d, _d, _d, _d, _i64, _i64, _i64, ctypes.c_int,
                                  _d, _d, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_double, _d, _d]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_d) if a is not None else None


def planar(a):
    """H x W x B -> contiguous float64 B x H x W."""
    return np.ascontiguousarray(np.moveaxis(np.asarray(a, dtype=np.float64), -1, 0))


def unplanar(a):
    return np.ascontiguousarray(np.moveaxis(a, 0, -1))


def tv_chambolle(stack_bhw, weight, n_iter_max, eps=2e-4):
    """Per-frame TV of a planar float64 stack; returns (u, steps, energies)."""
    f = np.ascontiguousarray(stack_bhw, dtype=np.float64)
    nf, H, W = f.shape
    u = np.empty_like(f)
    steps = np.zeros(nf, dtype=np.int32)
    en = np.empty((nf, n_iter_max), dtype=np.float64)
    lib().orc_tv_chambolle(_p(f), _p(u), nf, H, W, float(weight), float(eps),
                           int(n_iter_max),
                           steps.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(en))
    return u, steps, en


def _schedule(v, n):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (n,)))


def gap_tv(y, phi_bhw, phisum, x0_bhw, iters, lambdas=1.0, weights=0.1,
           tv_iter_max=5, eps=2e-4, accelerate=True, orig_bhw=None):
    """GAP-TV on planar float64 arrays; returns (x, psnr_all or None)."""
    phi = np.ascontiguousarray(phi_bhw, dtype=np.float64)
    B, H, W = phi.shape
    x = np.array(x0_bhw, dtype=np.float64, order="C", copy=True)
    y = np.ascontiguousarray(y, dtype=np.float64)
    ps = np.ascontiguousarray(phisum, dtype=np.float64)
    lam = _schedule(lambdas, iters)
    wts = _schedule(weights, iters)
    orig = None if orig_bhw is None else np.ascontiguousarray(orig_bhw, dtype=np.float64)
    pa = np.empty(iters) if orig is not None else None
    lib().orc_gap_tv(_p(y), _p(phi), _p(ps), _p(x), B, H, W, int(iters), _p(lam),
                     _p(wts), int(tv_iter_max), float(eps), int(bool(accelerate)),
                     _p(orig), _p(pa))
    return x, pa


def admm_tv(y, phi_bhw, phisum, x0_bhw, iters, lambdas=1.0, weights=0.1,
            gamma=0.01, tv_iter_max=5, eps=2e-4, orig_bhw=None):
    """ADMM-TV on planar float64 arrays; returns (x, psnr_all or None)."""
    phi = np.ascontiguousarray(phi_bhw, dtype=np.float64)
    B, H, W = phi.shape
    x = np.array(x0_bhw, dtype=np.float64, order="C", copy=True)
    y = np.ascontiguousarray(y, dtype=np.float64)
    ps = np.ascontiguousarray(phisum, dtype=np.float64)
    lam = _schedule(lambdas, iters)
    wts = _schedule(weights, iters)
    orig = None if orig_bhw is None else np.ascontiguousarray(orig_bhw, dtype=np.float64)
    pa = np.empty(iters) if orig is not None else None
    lib().orc_admm_tv(_p(y), _p(phi), _p(ps), _p(x), B, H, W, int(iters), _p(lam),
                      _p(wts), float(gamma), int(tv_iter_max), float(eps),
                      _p(orig), _p(pa))
    return x, pa
