"""Chambolle TV denoiser: the ``denoise_tv_chambolle`` plug-in, on the GPU.

Same call as the scikit-image function the reference uses
(``PnP_SCI/python/pnp_sci_algo.py:650``, ``:812-813``):
``denoise_tv_chambolle(image, weight, eps=2e-4, n_iter_max=200,
multichannel=False)``.  With ``multichannel=True`` every slice
``image[..., c]`` is an independent 2-D image (an H x W x B frame stack);
without it the image must be 2-D.  Arithmetic is float32 on the device;
numpy input returns numpy in the input's float dtype.
"""
import ctypes

import numpy as np
import torch

from . import _dev
from ._lib import call


def tv_workspace(nframes, H, W, n_iter_max, dev=None):
    n = ctypes.c_size_t()
    call("sci_tv_workspace_bytes", nframes, H, W, int(n_iter_max), ctypes.byref(n))
    return _dev.workspace(n.value, dev)


def tv_frames(f, weight, n_iter_max=200, eps=2e-4, u=None, resid=None, steps=None,
              energy=None, workspace=None):
    """TV of a planar (nframes, H, W) contiguous float32 CUDA tensor.

    Returns u (allocated unless given).  ``resid`` receives u - f,
    ``steps`` (int32[nframes]) the executed Chambolle steps per frame,
    ``energy`` (float64[nframes, n_iter_max, 2]) the per-step sums.
    """
    if f.dim() != 3 or f.dtype != torch.float32 or not f.is_cuda or not f.is_contiguous():
        raise ValueError("tv_frames expects a contiguous float32 CUDA tensor (F, H, W)")
    nf, H, W = f.shape
    if u is None:
        u = torch.empty_like(f)
    if workspace is None:
        workspace = tv_workspace(nf, H, W, n_iter_max, f.device)
    call("sci_tv_chambolle", f.data_ptr(), u.data_ptr(), _dev.ptr(resid), nf, H, W,
         float(weight), float(eps), int(n_iter_max), _dev.ptr(steps), _dev.ptr(energy),
         workspace.data_ptr(), workspace.numel(), _dev.stream_handle())
    return u


def denoise_tv_chambolle(image, weight=0.1, eps=2.e-4, n_iter_max=200, multichannel=False):
    """Per-frame Chambolle TV (scikit-image 0.16 semantics) on the GPU."""
    if not _dev.is_torch(image):
        image_np = np.asarray(image)
        if image_np.dtype.kind != 'f':
            raise TypeError("denoise_tv_chambolle takes floating-point images")
    nd = image.dim() if _dev.is_torch(image) else np.ndim(image)
    if multichannel:
        if nd != 3:
            raise ValueError("multichannel=True expects an H x W x C stack")
        f = _dev.planar(image)
        u = tv_frames(f, weight, n_iter_max, eps)
        out = _dev.unplanar(u, image)
    else:
        if nd != 2:
            raise NotImplementedError("only 2-D images (or multichannel stacks) are supported")
        f = _dev.plane(image).unsqueeze(0)
        u = tv_frames(f, weight, n_iter_max, eps)[0]
        out = _dev.unplane(u, image)
    if not _dev.is_torch(image):
        out = out.astype(np.asarray(image).dtype, copy=False)
    return out


# ------------------------------------------------- MATLAB-twin TV denoisers
# gapdenoise.m:92-112: tvm name -> (kind of sci_tv_matlab, the file's
# parameter as a function of tvweight, iterations)
TVM = {
    "ATV_ClipA": (1, lambda w: w, 5),
    "ATV_ClipB": (2, lambda w: w, 5),
    "ATV_cham": (3, lambda w: 1.0 / w, 5),
    "ATV_FGP": (4, lambda w: w, 2),
    "ITV2D_cham": (5, lambda w: 1.0 / w, 5),
    "ITV2D_FGP": (6, lambda w: w, 2),
    "ITV3D_cham": (7, lambda w: 1.0 / w, 5),
    "ITV3D_FGP": (8, lambda w: w, 2),
}


def tvm_kind(tvm):
    """The sci_tv_matlab kind of a tvm name ('tv_chambolle' -> 0)."""
    if tvm == "tv_chambolle":
        return 0
    if tvm not in TVM:
        raise ValueError("Unsupported TV denoiser {}!".format(tvm))
    return TVM[tvm][0]


def tv_matlab_workspace(kind, nframes, H, W, iters, dev=None):
    n = ctypes.c_size_t()
    call("sci_tv_matlab_workspace_bytes", int(kind), nframes, H, W, int(iters), ctypes.byref(n))
    return _dev.workspace(n.value, dev)


def tv_matlab_frames(f, tvm, lam, iters, u=None, workspace=None):
    """A MATLAB-twin denoiser (tvm name or kind) with the file's own
    parameters on a planar (nframes, H, W) float32 CUDA tensor."""
    if f.dim() != 3 or f.dtype != torch.float32 or not f.is_cuda or not f.is_contiguous():
        raise ValueError("tv_matlab_frames expects a contiguous float32 CUDA tensor (F, H, W)")
    kind = tvm if isinstance(tvm, int) else tvm_kind(tvm)
    nf, H, W = f.shape
    if u is None:
        u = torch.empty_like(f)
    if workspace is None:
        workspace = tv_matlab_workspace(kind, nf, H, W, iters, f.device)
    call("sci_tv_matlab", kind, f.data_ptr(), u.data_ptr(), nf, H, W, float(lam), int(iters),
         workspace.data_ptr(), workspace.numel(), _dev.stream_handle())
    return u


def denoise_tv_matlab(v, tvm, tvweight):
    """The denoising step of gapdenoise.m:92-112 for `tvm` on an H x W x B
    stack (numpy or torch), with gapdenoise's parameters and iteration
    counts."""
    tvm_kind(tvm)  # ValueError for an unknown name
    kind, param, iters = TVM[tvm]
    f = _dev.planar(v)
    out = _dev.unplanar(tv_matlab_frames(f, kind, param(float(tvweight)), iters), v)
    if not _dev.is_torch(v):
        out = out.astype(np.asarray(v).dtype, copy=False)
    return out
