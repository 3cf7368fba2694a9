"""ctypes binding of ``libsci_gb300.so`` (declared in ``include/sci_gb300.h``).

The library is the only compute path: if it is missing or fails to load,
every operation raises -- there is no CPU or eager fallback.
"""
import ctypes
import os

from . import buildlib as _build

c_i64 = ctypes.c_int64
c_f = ctypes.c_float
c_vp = ctypes.c_void_p
c_sz = ctypes.c_size_t

SCI_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "unsupported",
          -4: "workspace", -5: "device-side timeout"}


class SciError(RuntimeError):
    """A negative status from the C ABI, with the library's message."""

    def __init__(self, fn, code, msg):
        super().__init__("%s failed (%d: %s): %s" % (fn, code, ERRORS.get(code, "?"), msg))
        self.code = code


class SolveOpts(ctypes.Structure):
    """``sci_solve_opts`` of include/sci_gb300.h."""
    _fields_ = [("iters", ctypes.c_int),
                ("lambdas", ctypes.POINTER(c_f)),
                ("weights", ctypes.POINTER(c_f)),
                ("tv_iter_max", ctypes.c_int),
                ("eps", c_f),
                ("accelerate", ctypes.c_int),
                ("gamma", c_f),
                ("gammas", ctypes.POINTER(c_f)),
                ("orig", c_vp),
                ("sqerr", c_vp),
                ("tv_steps", c_vp),
                ("use_graph", ctypes.c_int),
                ("tvm", ctypes.c_int),
                ("resid_norm", c_vp)]


class BatchItem(ctypes.Structure):
    """``sci_batch_item`` of include/sci_gb300.h."""
    _fields_ = [("y", c_vp), ("mask_bits", c_vp), ("phisum", c_vp), ("x", c_vp),
                ("B", c_i64), ("H", c_i64), ("W", c_i64), ("lam", c_f), ("tv_weight", c_f),
                ("R", ctypes.c_int), ("cpl", ctypes.c_int)]


# name -> argtypes (all functions return int status)
_SIGS = {
    "sci_version": [],
    "sci_last_error": [ctypes.c_char_p, c_sz],
    "sci_device_status": [ctypes.POINTER(ctypes.c_uint), ctypes.c_int],
    "sci_selftest_bounded_wait": [ctypes.c_uint, c_vp],
    "sci_A": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_vp],
    "sci_At": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_vp],
    "sci_phisum": [c_vp, c_vp, c_i64, c_i64, c_i64, ctypes.c_int, c_vp],
    "sci_pack_mask": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_vp],
    "sci_proj_gap": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_f, ctypes.c_int,
                     c_i64, c_i64, c_i64, c_vp],
    "sci_gap_residual": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, ctypes.c_int, c_i64, c_i64,
                         c_i64, c_vp],
    "sci_proj_admm": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_f, c_f,
                      c_i64, c_i64, c_i64, c_vp],
    "sci_tv_workspace_bytes": [c_i64, c_i64, c_i64, ctypes.c_int, ctypes.POINTER(c_sz)],
    "sci_tv_chambolle": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_f, c_f, ctypes.c_int,
                         c_vp, c_vp, c_vp, c_sz, c_vp],
    "sci_tv_chambolle_noalloc": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_f, c_f,
                                 ctypes.c_int, c_vp, c_vp],
    "sci_tv_matlab_workspace_bytes": [ctypes.c_int, c_i64, c_i64, c_i64, ctypes.c_int,
                                      ctypes.POINTER(c_sz)],
    "sci_tv_matlab": [ctypes.c_int, c_vp, c_vp, c_i64, c_i64, c_i64, c_f, ctypes.c_int, c_vp,
                      c_sz, c_vp],
    "sci_sqerr_accum": [c_vp, c_vp, c_i64, c_vp, c_vp],
    "sci_frame_metrics": [c_vp, c_vp, c_i64, c_i64, c_i64, ctypes.c_double, c_vp, c_vp, c_vp],
    "sci_solver_workspace_bytes": [c_i64, c_i64, c_i64, ctypes.POINTER(SolveOpts),
                                   ctypes.POINTER(c_sz)],
    "sci_gap_tv": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_i64,
                   ctypes.POINTER(SolveOpts), c_vp, c_sz, c_vp],
    "sci_admm_tv": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_i64,
                    ctypes.POINTER(SolveOpts), c_vp, c_sz, c_vp],
    "sci_cassi_A": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, ctypes.c_int, c_vp],
    "sci_cassi_At": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, ctypes.c_int, c_vp],
    "sci_cassi_phisum": [c_vp, c_vp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int, c_vp],
    "sci_cassi_workspace_bytes": [c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(c_sz)],
    "sci_cassi_gap_tv": [c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, ctypes.c_int,
                         ctypes.POINTER(SolveOpts), c_vp, c_sz, c_vp],
    "sci_batch_workspace_bytes": [ctypes.POINTER(BatchItem), ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(c_sz)],
    "sci_batch_autotune": [ctypes.POINTER(BatchItem), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                           c_f, ctypes.c_int, ctypes.POINTER(ctypes.c_int), c_vp, c_sz, c_vp],
    "sci_batch_selftest_queue_wait": [ctypes.c_uint, c_vp, c_sz, c_vp],
    "sci_batch_gap_tv": [ctypes.POINTER(BatchItem), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                         c_f, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_vp, c_sz,
                         c_vp],
    "sci_cnn_ffdnet_pack": [c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, ctypes.c_int, c_vp],
    "sci_cnn_ffdnet_unpack_sub": [c_vp, c_vp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, c_vp, c_vp],
    "sci_cnn_window": [c_vp, c_i64, c_i64, c_i64, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp,
                       ctypes.c_int, c_vp],
    "sci_cnn_center_sub": [c_vp, c_i64, c_i64, c_i64, c_i64, c_i64, c_vp, ctypes.c_int,
                           ctypes.c_int, c_i64, c_i64, c_i64, c_i64, ctypes.c_int, c_vp, c_vp],
    "sci_cnn_shuffle_add": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_vp],
    "sci_cnn_shuffle_add_f32": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_vp],
    "sci_cnn_conv_thin": [c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, ctypes.c_int,
                          ctypes.c_int, c_vp],
    "sci_cnn_den_tail": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64,
                         c_i64, c_i64, c_i64, c_i64, c_i64, ctypes.c_int, c_vp, c_vp],
    "sci_unrolled_workspace_bytes": [c_i64, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(c_sz)],
    "sci_unrolled_fwd": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, ctypes.c_int,
                         ctypes.c_int, c_f, c_vp, c_vp, c_vp, c_sz, c_vp],
    "sci_unrolled_bwd": [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, ctypes.c_int,
                         ctypes.c_int, c_f, c_f, c_vp, c_vp, c_vp, c_sz, c_vp],
}

_lib = None


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path) or (build_if_missing and not _build.up_to_date()):
        if not build_if_missing:
            raise RuntimeError("libsci_gb300.so is not built (%s); run build()" % path)
        _build.build()
    L = ctypes.CDLL(path)
    for name, argt in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = argt
        fn.restype = ctypes.c_int
    _lib = L
    return L


def exported_symbols():
    return sorted(_SIGS)


def last_error():
    L = load()
    buf = ctypes.create_string_buffer(1024)
    L.sci_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def call(name, *args):
    """Call ``name`` and raise SciError on a negative status."""
    L = load()
    rc = getattr(L, name)(*args)
    if rc != SCI_OK:
        raise SciError(name, rc, last_error())
    return rc
