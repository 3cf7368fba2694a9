"""Batched GAP-TV: many measurements of uneven H x W x B solved together.

``BatchSolver`` builds one device item table for a list of measurements
(each with its own binary mask, packed to one word per pixel) and calls
``sci_batch_gap_tv``: persistent launches over a device work queue run the
projection tiles, TV work items and stop tests of every item, each task
waiting only for earlier tasks of its own item, and the whole loop is
captured once into a CUDA graph.  ``autotune=True`` lets
``sci_batch_autotune`` pick each shape's TV column width and row-chunk
height, and the iterations per persistent launch, by timing them on the
items' data.  Each item's result equals a single-measurement
``gap_denoise`` (``PnP_SCI/python/pnp_sci_algo.py:536``) with
x0 = At(y / Phi_sum).
"""
import ctypes

import torch

from . import _dev
from ._lib import BatchItem, call
from .utils import MaskOperator


class BatchSolver:
    def __init__(self, meas_list, mask_list, iters=50, lam=1.0, tv_weight=0.1, tv_iter_max=5,
                 eps=2e-4, accelerate=True, autotune=True, use_graph=True):
        if len(meas_list) != len(mask_list) or not meas_list:
            raise ValueError("need one mask per measurement")
        self.dev = _dev.device()
        self.iters, self.K, self.eps = int(iters), int(tv_iter_max), float(eps)
        self.accelerate, self.use_graph = int(bool(accelerate)), int(bool(use_graph))
        self.ops, self.ys, self.xs = [], [], []
        n = len(meas_list)
        self.items = (BatchItem * n)()
        for i, (y, m) in enumerate(zip(meas_list, mask_list)):
            op = MaskOperator(m)
            if op.bits is None:
                raise ValueError("item %d: the batched solver needs a binary mask with B <= 32" % i)
            yd = _dev.plane(y, self.dev)
            x = torch.empty((op.B, op.H, op.W), dtype=torch.float32, device=self.dev)
            self.ops.append(op)
            self.ys.append(yd)
            self.xs.append(x)
            it = self.items[i]
            it.y, it.mask_bits, it.phisum, it.x = (yd.data_ptr(), op.bits.data_ptr(),
                                                   op.phisum.data_ptr(), x.data_ptr())
            it.B, it.H, it.W = op.B, op.H, op.W
            it.lam, it.tv_weight, it.R, it.cpl = float(lam), float(tv_weight), 0, 0
        nb = ctypes.c_size_t()
        call("sci_batch_workspace_bytes", self.items, n, self.K, ctypes.byref(nb))
        self.ws = _dev.workspace(nb.value, self.dev)
        # iterations per persistent launch of the work queue (0: all)
        self.iters_per_launch = 0
        if autotune:
            self._call(0, 1, graph=False)  # x = x0, a realistic input to time on
            ipl = ctypes.c_int(0)
            call("sci_batch_autotune", self.items, n, self.iters, self.K, self.eps,
                 self.accelerate, ctypes.byref(ipl), self.ws.data_ptr(), self.ws.numel(),
                 _dev.stream_handle())
            self.iters_per_launch = ipl.value

    def _call(self, iters, init_x0, graph):
        call("sci_batch_gap_tv", self.items, len(self.xs), iters, self.K, self.eps,
             self.accelerate, init_x0, int(graph), int(self.iters_per_launch),
             self.ws.data_ptr(), self.ws.numel(), _dev.stream_handle())

    def chunk_rows(self):
        return [self.items[i].R for i in range(len(self.xs))]

    def columns_per_lane(self):
        return [self.items[i].cpl or 4 for i in range(len(self.xs))]

    def run(self, x0=None):
        """Solve all items; returns the list of (B, H, W) results (device
        tensors owned by the solver).  x0: optional list of start points."""
        if x0 is not None:
            for x, v in zip(self.xs, x0):
                x.copy_(v)
        self._call(self.iters, 1 if x0 is None else 0, self.use_graph)
        return self.xs
