"""Mask operators and metrics: the reference's ``utils.py`` plug-in surface.

``A_`` / ``At_`` / ``psnr`` keep the names and argument meaning of
``PnP_SCI/python/utils.py:10-36``.  ``MaskOperator`` is the device-resident
form of the ``A = lambda x: A_(x, mask)`` / ``At = lambda y: At_(y, mask)``
closures the reference drivers build (``pnp_sci_test_orig.py:147-148``):
its bound methods are callables with the same behaviour, and the solvers
recognise them and run the fused native loop.
"""
import math

import numpy as np
import torch

from . import _dev
from ._lib import call


class MaskOperator:
    """Snapshot forward model y = sum_b mask_b * x_b for one coded mask.

    Holds the mask on the GPU in planar float32 (B x H x W), its guarded
    frame sum (zeros replaced by 1, ``pnp_sci_algo.py:491-492``) and, for a
    binary mask with B <= 32, the mask packed to one 32-bit word per pixel,
    which the projection kernels read instead of the float planes.
    """

    def __init__(self, mask, pack=True):
        self.dev = _dev.device()
        self.phi = _dev.planar(mask, self.dev)
        self.B, self.H, self.W = self.phi.shape
        s = _dev.stream_handle()
        self.phisum = torch.empty((self.H, self.W), dtype=torch.float32, device=self.dev)
        call("sci_phisum", self.phi.data_ptr(), self.phisum.data_ptr(), self.B, self.H,
             self.W, 1, s)
        self.bits = None
        if pack and self.B <= 32:
            bits = torch.empty((self.H, self.W), dtype=torch.int32, device=self.dev)
            flag = torch.zeros(1, dtype=torch.int32, device=self.dev)
            call("sci_pack_mask", self.phi.data_ptr(), bits.data_ptr(), flag.data_ptr(),
                 self.B, self.H, self.W, s)
            if int(flag.item()) == 0:
                self.bits = bits

    # -- the two plug-in callables ----------------------------------------
    def forward(self, x):
        """A(x): H x W x B -> H x W  (``utils.py:10-15``)."""
        xp = _dev.planar(x, self.dev)
        self._check(xp)
        y = torch.empty((self.H, self.W), dtype=torch.float32, device=self.dev)
        call("sci_A", xp.data_ptr(), self.phi.data_ptr(), y.data_ptr(), self.B, self.H,
             self.W, _dev.stream_handle())
        return _dev.unplane(y, x)

    def adjoint(self, y):
        """At(y): H x W -> H x W x B  (``utils.py:17-26``)."""
        yp = _dev.plane(y, self.dev)
        if tuple(yp.shape) != (self.H, self.W):
            raise ValueError("measurement shape %s != mask %s" % (tuple(yp.shape), (self.H, self.W)))
        x = torch.empty((self.B, self.H, self.W), dtype=torch.float32, device=self.dev)
        call("sci_At", yp.data_ptr(), self.phi.data_ptr(), x.data_ptr(), self.B, self.H,
             self.W, _dev.stream_handle())
        return _dev.unplanar(x, y)

    __call__ = forward

    def _check(self, xp):
        if tuple(xp.shape) != (self.B, self.H, self.W):
            raise ValueError("stack shape (B,H,W)=%s != mask %s"
                             % (tuple(xp.shape), (self.B, self.H, self.W)))


def make_ops(mask, pack=True):
    """(A, At) callables bound to ``mask`` -- the reference's
    ``A = lambda x: A_(x, mask); At = lambda y: At_(y, mask)``."""
    op = MaskOperator(mask, pack=pack)
    return op.forward, op.adjoint


def operator_of(A, At):
    """The native operator (MaskOperator, CassiOperator) behind (A, At) if
    both are the forward / adjoint bound methods of the same object."""
    oa = getattr(A, "__self__", None)
    ot = getattr(At, "__self__", None)
    if oa is None or oa is not ot:
        return None
    cls = type(oa)
    if getattr(A, "__func__", None) is getattr(cls, "forward", None) and \
            getattr(At, "__func__", None) is getattr(cls, "adjoint", None) and \
            hasattr(oa, "phisum"):
        return oa
    return None


def A_(x, Phi):
    """Forward model (``PnP_SCI/python/utils.py:10-15``), on the GPU.

    x, Phi: H x W x B (numpy or torch); returns H x W (float32; numpy in ->
    numpy out, torch in -> CUDA tensor out).
    """
    phi = _dev.planar(Phi)
    xp = _dev.planar(x)
    if xp.shape != phi.shape:
        raise ValueError("x %s and Phi %s differ" % (tuple(xp.shape), tuple(phi.shape)))
    B, H, W = phi.shape
    y = torch.empty((H, W), dtype=torch.float32, device=phi.device)
    call("sci_A", xp.data_ptr(), phi.data_ptr(), y.data_ptr(), B, H, W, _dev.stream_handle())
    return _dev.unplane(y, x)


def At_(y, Phi):
    """Transpose of the forward model (``PnP_SCI/python/utils.py:17-26``)."""
    phi = _dev.planar(Phi)
    B, H, W = phi.shape
    yp = _dev.plane(y, phi.device)
    if tuple(yp.shape) != (H, W):
        raise ValueError("y %s and Phi %s differ" % (tuple(yp.shape), (H, W)))
    x = torch.empty((B, H, W), dtype=torch.float32, device=phi.device)
    call("sci_At", yp.data_ptr(), phi.data_ptr(), x.data_ptr(), B, H, W, _dev.stream_handle())
    return _dev.unplanar(x, y)


def sum_sq_err(a_planar, b_planar):
    """sum (a - b)^2 in float64 on the GPU (both contiguous float32)."""
    out = torch.zeros(1, dtype=torch.float64, device=a_planar.device)
    call("sci_sqerr_accum", a_planar.data_ptr(), b_planar.data_ptr(), a_planar.numel(),
         out.data_ptr(), _dev.stream_handle())
    return float(out.item())


def psnr_from_mse(mse):
    """``utils.py:28-36``: 100 when equal, else 20 log10(1 / sqrt(MSE))."""
    if mse == 0:
        return 100
    return 20 * math.log10(1.0 / math.sqrt(mse))


def _flat(a, dev):
    if _dev.is_torch(a):
        return a.to(device=dev, dtype=torch.float32).contiguous().reshape(-1)
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev).reshape(-1)


def psnr(ref, img):
    """Peak signal-to-noise ratio with peak 1 (``PnP_SCI/python/utils.py:28-36``)."""
    dev = _dev.device()
    a, b = _flat(ref, dev), _flat(img, dev)
    if np.shape(ref) != np.shape(img):
        raise ValueError("shapes differ: %s vs %s" % (np.shape(ref), np.shape(img)))
    return psnr_from_mse(sum_sq_err(a, b) / a.numel())
