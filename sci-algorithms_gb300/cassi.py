"""Spectral SCI (CASSI): coded aperture + dispersion operators and GAP-TV.

A single H x W aperture ``phi`` codes every band; band b of the H x W x L
cube lands on the H x (W + step (L-1)) detector shifted by ``step * b``
pixels along W.  The reference's Python path has no spectral operator; its
MATLAB CASSI test (``DeSCI/test_desci_cassi.m:58-62``) uses the same model
with a pre-shifted mask and ``Phisum = sum(mask.^2, 3)``.  ``CassiOperator``
provides the (A, At) callables; ``gap_denoise`` in this package recognises
them and runs the native loop (``sci_cassi_gap_tv``).
"""
import ctypes
import math

import numpy as np
import torch

from . import _dev
from ._lib import SolveOpts, call


class CassiOperator:
    def __init__(self, aperture, L, step=2):
        self.dev = _dev.device()
        self.phi = _dev.plane(aperture, self.dev)
        self.H, self.W = self.phi.shape
        self.L, self.step = int(L), int(step)
        if self.step < 1:
            raise ValueError("step must be >= 1")
        self.Wd = self.W + self.step * (self.L - 1)
        self.B = self.L
        self.phisum = torch.empty((self.H, self.Wd), dtype=torch.float32, device=self.dev)
        call("sci_cassi_phisum", self.phi.data_ptr(), self.phisum.data_ptr(), self.L, self.H,
             self.W, self.step, 1, _dev.stream_handle())

    def forward(self, x):
        """H x W x L cube -> H x Wd detector image."""
        xp = _dev.planar(x, self.dev)
        if tuple(xp.shape) != (self.L, self.H, self.W):
            raise ValueError("cube shape mismatch")
        y = torch.empty((self.H, self.Wd), dtype=torch.float32, device=self.dev)
        call("sci_cassi_A", xp.data_ptr(), self.phi.data_ptr(), y.data_ptr(), self.L, self.H,
             self.W, self.step, _dev.stream_handle())
        return _dev.unplane(y, x)

    def adjoint(self, y):
        """H x Wd detector image -> H x W x L cube."""
        yp = _dev.plane(y, self.dev)
        if tuple(yp.shape) != (self.H, self.Wd):
            raise ValueError("detector shape mismatch")
        x = torch.empty((self.L, self.H, self.W), dtype=torch.float32, device=self.dev)
        call("sci_cassi_At", yp.data_ptr(), self.phi.data_ptr(), x.data_ptr(), self.L, self.H,
             self.W, self.step, _dev.stream_handle())
        return _dev.unplanar(x, y)

    __call__ = forward


def make_cassi_ops(aperture, L, step=2):
    op = CassiOperator(aperture, L, step)
    return op.forward, op.adjoint


class CassiSolver:
    """GAP-TV on one CASSI measurement (native loop)."""

    def __init__(self, op, iters=80, lambdas=1.0, tv_weight=0.1, tv_iter_max=5, eps=2e-4,
                 accelerate=True, use_graph=True):
        self.op = op
        self.iters = int(iters)
        self._lam = _dev.schedule(lambdas, self.iters)
        self._w = _dev.schedule(tv_weight, self.iters)
        o = self.opts = SolveOpts()
        o.iters = self.iters
        o.lambdas = self._lam.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        o.weights = self._w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        o.tv_iter_max = int(tv_iter_max)
        o.eps = float(eps)
        o.accelerate = 1 if accelerate else 0
        o.use_graph = 1 if use_graph else 0
        n = ctypes.c_size_t()
        call("sci_cassi_workspace_bytes", op.L, op.H, op.W, op.step, int(tv_iter_max),
             ctypes.byref(n))
        self.ws = _dev.workspace(n.value, op.dev)
        self.x = torch.empty((op.L, op.H, op.W), dtype=torch.float32, device=op.dev)
        self.sqerr = torch.zeros(self.iters, dtype=torch.float64, device=op.dev)

    def run(self, y, x0=None, phisum=None, orig=None):
        op = self.op
        if x0 is None:
            x0 = self.x
            call("sci_cassi_At", y.data_ptr(), op.phi.data_ptr(), x0.data_ptr(), op.L, op.H,
                 op.W, op.step, _dev.stream_handle())
        o = self.opts
        o.orig = None if orig is None else orig.data_ptr()
        o.sqerr = None if orig is None else self.sqerr.data_ptr()
        ps = op.phisum if phisum is None else phisum
        call("sci_cassi_gap_tv", y.data_ptr(), op.phi.data_ptr(), ps.data_ptr(), x0.data_ptr(),
             self.x.data_ptr(), op.L, op.H, op.W, op.step, ctypes.byref(o), self.ws.data_ptr(),
             self.ws.numel(), _dev.stream_handle())
        return self.x

    def psnr_all(self):
        n = self.op.L * self.op.H * self.op.W
        return [100 if s == 0 else 20 * math.log10(1.0 / math.sqrt(s / n))
                for s in self.sqerr.tolist()]
