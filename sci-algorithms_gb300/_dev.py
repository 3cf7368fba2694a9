"""Device plumbing: layout conversion at the boundary, streams, workspaces.

The reference keeps frame stacks as numpy H x W x B (frames last,
``PnP_SCI/python/utils.py:15,26``); the kernels use planar B x H x W
(frame-major, W fastest) so that rows are contiguous for 16-byte loads and
stencil tiles.  Conversion happens once per call here.  PyTorch provides
device memory and the current stream only; all arithmetic is done by the
library's kernels.
"""
import numpy as np
import torch


def device():
    if not torch.cuda.is_available():
        raise RuntimeError("sci_algorithms_gb300 needs a CUDA GPU (sm_103a); none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def stream_handle():
    return torch.cuda.current_stream().cuda_stream


def is_torch(a):
    return isinstance(a, torch.Tensor)


def ptr(t):
    return None if t is None else t.data_ptr()


def planar(a, dev=None):
    """H x W x B (numpy or torch) -> contiguous float32 B x H x W on the GPU.

    A torch tensor that already is a frames-last view of a planar buffer
    (``t.permute(1, 2, 0)`` of a contiguous B x H x W tensor) is used without
    a copy.
    """
    dev = dev or device()
    if is_torch(a):
        if a.dim() != 3:
            raise ValueError("expected an H x W x B stack, got shape %s" % (tuple(a.shape),))
        t = a.to(device=dev, dtype=torch.float32)
        p = t.permute(2, 0, 1)
        return p if p.is_contiguous() else p.contiguous()
    a = np.asarray(a)
    if a.ndim != 3:
        raise ValueError("expected an H x W x B stack, got shape %s" % (a.shape,))
    h = np.ascontiguousarray(np.moveaxis(a, -1, 0), dtype=np.float32)
    return torch.from_numpy(h).to(dev)


def plane(a, dev=None):
    """H x W map (numpy or torch) -> contiguous float32 on the GPU."""
    dev = dev or device()
    if is_torch(a):
        if a.dim() != 2:
            raise ValueError("expected an H x W map, got shape %s" % (tuple(a.shape),))
        return a.to(device=dev, dtype=torch.float32).contiguous()
    a = np.asarray(a)
    if a.ndim != 2:
        raise ValueError("expected an H x W map, got shape %s" % (a.shape,))
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


def stack(a, dev=None):
    """An H x W x F array (numpy or torch) as a float32 tensor on the GPU,
    in its own layout: numpy input crosses to the device once in its own
    dtype and is converted there (a host-side float64 -> float32 pass over
    a multi-GB ground truth costs more than the larger copy)."""
    dev = dev or device()
    if is_torch(a):
        return a.to(device=dev, dtype=torch.float32)
    a = np.asarray(a)
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float32)
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev).to(torch.float32)


def unplanar(p, like):
    """B x H x W device tensor -> H x W x B in the kind of ``like``.

    torch in -> torch view on the device (no copy); numpy in -> float32 numpy.
    """
    v = p.permute(1, 2, 0)
    if is_torch(like):
        return v
    return v.contiguous().cpu().numpy()


def unplane(t, like):
    if is_torch(like):
        return t
    return t.cpu().numpy()


def schedule(v, n):
    """Scalar or per-iteration sequence -> float32 numpy array of length n."""
    a = np.asarray(v, dtype=np.float32)
    if a.ndim == 0:
        return np.full(n, float(a), dtype=np.float32)
    if a.shape != (n,):
        raise ValueError("schedule of length %d expected, got %s" % (n, a.shape))
    return np.ascontiguousarray(a)


def workspace(nbytes, dev=None):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=dev or device())
