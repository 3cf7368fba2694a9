"""Device-resident GAP-TV / ADMM-TV solver over the native C-ABI loop.

``Solver`` owns the workspace for one (B, H, W) problem and one option set
and calls ``sci_gap_tv`` / ``sci_admm_tv``, which enqueue (and, by default,
replay as one cached CUDA graph) every iteration of
``gap_denoise`` / ``admm_denoise`` (``PnP_SCI/python/pnp_sci_algo.py:536-864``).
``Solver.run_host`` is the end-to-end entry: pinned host inputs in, host
result out; ``Solver.run_host_many`` pipelines a sequence of measurements
(the copy-out of one overlaps the solve of the next).
"""
import ctypes
import math

import numpy as np
import torch

from . import _dev
from ._lib import SolveOpts, call
from .tv import TVM, tvm_kind


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if a is not None else None


class Solver:
    """One reconstruction problem: mask operator, iteration count, schedules."""

    def __init__(self, op, projmeth="gap", iters=50, lambdas=1.0, tv_weight=0.1,
                 tv_iter_max=5, eps=2e-4, accelerate=True, gamma=0.01, gammas=None,
                 use_graph=True, use_bits=True, tvm="tv_chambolle", resid_norm=False):
        if projmeth not in ("gap", "admm"):
            raise ValueError("Unsupported projection method %s" % projmeth)
        self.op = op
        self.admm = projmeth == "admm"
        self.B, self.H, self.W = op.B, op.H, op.W
        self.iters = int(iters)
        self._lam = _dev.schedule(lambdas, self.iters)
        self._w = _dev.schedule(tv_weight, self.iters)
        self._g = None if gammas is None else _dev.schedule(gammas, self.iters)
        if np.any(self._w <= 0):
            raise ValueError("tv_weight must be > 0")
        self.bits = op.bits if use_bits else None
        self.opts = SolveOpts()
        o = self.opts
        o.iters = self.iters
        o.lambdas = _fptr(self._lam)
        o.weights = _fptr(self._w)
        # tvm: the scikit-image Chambolle TV, or a MATLAB-twin denoiser with
        # gapdenoise.m's iteration count (tv_iter_max does not apply to it)
        o.tvm = tvm_kind(tvm)
        o.tv_iter_max = int(tv_iter_max) if o.tvm == 0 else TVM[tvm][2]
        o.eps = float(eps)
        o.accelerate = 1 if accelerate else 0
        o.gamma = float(gamma)
        o.gammas = _fptr(self._g)
        o.orig = None
        o.sqerr = None
        o.tv_steps = None
        o.use_graph = 1 if use_graph else 0
        # FP64 ||r_k||^2 of every iteration's projection residual, on the
        # device (see resid_norms)
        self.resid_norm = (torch.zeros(self.iters, dtype=torch.float64, device=op.dev)
                           if resid_norm else None)
        o.resid_norm = self.resid_norm.data_ptr() if resid_norm else None
        n = ctypes.c_size_t()
        call("sci_solver_workspace_bytes", self.B, self.H, self.W, ctypes.byref(o),
             ctypes.byref(n))
        self.ws = _dev.workspace(n.value, op.dev)
        self.x = torch.empty((self.B, self.H, self.W), dtype=torch.float32, device=op.dev)
        self.sqerr = None
        self.tv_steps = None
        self._y_dev = None  # run_host's device copy of the measurement

    def run(self, y, x0=None, phisum=None, orig=None, tv_steps=False, out=None):
        """Solve on the device.  y: (H, W) float32 CUDA; x0: (B, H, W) or None
        (At(y)); orig: (B, H, W) for the per-iteration PSNR.  Returns x
        (B, H, W), which is ``out`` (or the solver's own buffer)."""
        op = self.op
        if x0 is None:
            x0 = self.x if out is None else out
            call("sci_At", y.data_ptr(), op.phi.data_ptr(), x0.data_ptr(), self.B, self.H,
                 self.W, _dev.stream_handle())
        x = self.x if out is None else out
        o = self.opts
        if orig is not None:
            if self.sqerr is None:
                self.sqerr = torch.zeros(self.iters, dtype=torch.float64, device=op.dev)
            o.orig, o.sqerr = orig.data_ptr(), self.sqerr.data_ptr()
        else:
            o.orig, o.sqerr = None, None
        if tv_steps:
            if self.tv_steps is None:
                self.tv_steps = torch.zeros((self.iters, self.B), dtype=torch.int32, device=op.dev)
            o.tv_steps = self.tv_steps.data_ptr()
        else:
            o.tv_steps = None
        ps = op.phisum if phisum is None else phisum
        fn = "sci_admm_tv" if self.admm else "sci_gap_tv"
        call(fn, y.data_ptr(), None if self.bits is not None else op.phi.data_ptr(),
             _dev.ptr(self.bits), ps.data_ptr(), x0.data_ptr(), x.data_ptr(), self.B, self.H,
             self.W, ctypes.byref(o), self.ws.data_ptr(), self.ws.numel(), _dev.stream_handle())
        return x

    def resid_norms(self):
        """||r_k||^2 per iteration of the last run (float64 numpy): the
        squared L2 norm of the projection residual r = (y1 - A x) / Phi_sum
        (GAP_acc), (y - A x) / Phi_sum (GAP) or (y - A(theta + b)) /
        (Phi_sum + gamma) (ADMM), summed in FP64 on the GPU.  Needs
        ``resid_norm=True`` at construction."""
        if self.resid_norm is None:
            raise ValueError("Solver(..., resid_norm=True) records the residual norms")
        return self.resid_norm.cpu().numpy()

    def psnr_all(self):
        """Per-iteration PSNR of the last run with ``orig`` (utils.py:28-36)."""
        n = self.B * self.H * self.W
        out = []
        for s in self.sqerr.tolist():
            mse = s / n
            out.append(100 if mse == 0 else 20 * math.log10(1.0 / math.sqrt(mse)))
        return out

    def run_host_many(self, y_hosts, x_hosts):
        """End to end over a sequence of measurements (the frame-block loop of
        ``admmdenoise_cacti``): each pinned host measurement (H, W) is solved
        on the current stream while, on a second stream, the previous result
        is copied back into its pinned ``x_hosts[k]`` (B, H, W) and the
        measurement after next is copied in.  Two device result slots and two
        measurement slots alternate; a result slot is reused only after its
        copy-out has finished, a measurement slot only after the solve that
        read it.  Returns when every result is on the host."""
        if len(y_hosts) != len(x_hosts):
            raise ValueError("one host result buffer per measurement")
        dev = self.op.dev
        if getattr(self, "_slots", None) is None:
            self._slots = [torch.empty((self.B, self.H, self.W), dtype=torch.float32, device=dev)
                           for _ in range(2)]
            self._y_slots = [torch.empty((self.H, self.W), dtype=torch.float32, device=dev)
                             for _ in range(2)]
            self._copy_stream = torch.cuda.Stream(device=dev)
        main = torch.cuda.current_stream()
        copy = self._copy_stream
        n = len(y_hosts)
        freed = [None, None]  # events: copy-out of each result slot finished
        ready = [None, None]  # events: copy-in of each measurement slot finished
        read = [None, None]   # events: the solve reading each measurement slot finished
        copy.wait_stream(main)  # the slots may still be in use by earlier work

        def copy_in(k):
            s = k % 2
            with torch.cuda.stream(copy):
                if read[s] is not None:
                    copy.wait_event(read[s])
                self._y_slots[s].copy_(y_hosts[k], non_blocking=True)
                ready[s] = torch.cuda.Event()
                ready[s].record(copy)

        for k in range(min(n, 2)):
            copy_in(k)
        x = None
        for k in range(n):
            s = k % 2
            if freed[s] is not None:
                main.wait_event(freed[s])
            main.wait_event(ready[s])
            x = self.run(self._y_slots[s], out=self._slots[s])
            solved = torch.cuda.Event()
            solved.record(main)
            read[s] = solved
            copy.wait_event(solved)
            with torch.cuda.stream(copy):
                x_hosts[k].copy_(x, non_blocking=True)
            freed[s] = torch.cuda.Event()
            freed[s].record(copy)
            if k + 2 < n:
                copy_in(k + 2)
        copy.synchronize()
        main.synchronize()
        return x_hosts

    def run_host(self, y_host, x_host=None):
        """End to end: copy a pinned host measurement (H, W) in, solve, copy
        the result (B, H, W) back into pinned ``x_host`` (allocated if None)."""
        # a buffer of the solver's own, so that every call replays the same
        # cached graph (its key holds the device pointers)
        if self._y_dev is None:
            self._y_dev = torch.empty((self.H, self.W), dtype=torch.float32, device=self.op.dev)
        y = self._y_dev
        y.copy_(y_host, non_blocking=True)
        x = self.run(y)
        if x_host is None:
            x_host = torch.empty(x.shape, dtype=torch.float32, pin_memory=True)
        x_host.copy_(x, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return x_host
