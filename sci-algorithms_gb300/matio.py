"""MATLAB data in and out, as the reference's test scripts do it (host side).

* ``load_cacti`` -- ``orig`` / ``mask`` from two .mat files
  (``PnP_SCI/python/pnp_sci_test_orig.py:94-110``): v7.2 and older through
  ``scipy.io.loadmat``; v7.3 (HDF5) through h5py, transposed from MATLAB's
  column-major order (``(2, 1, 0)`` for a stack).  Both come back float32.
* ``cacti_measurements`` -- ``meas[..., i] = sum_b orig[..., i*B + b] *
  mask[..., b]`` per block of B frames (``:112-123``), plus the optional
  Gaussian noise of ``:127-129``.
* ``save_results`` -- the result file of ``utils.py:98-125``
  (``vdenoise``, ``orig``, PSNR/SSIM lists, timing, frame range, ``Cr``).

h5py is optional: without it a v7.3 file raises ``ImportError``.
"""
import os

import numpy as np
import scipy.io as sio
from scipy.io.matlab import matfile_version


def mat_version(path):
    """(major, minor) of a .mat file: (1, 0) for v5 - v7.2, (2, 0) for v7.3."""
    return matfile_version(path, appendmat=True)


def load_mat_array(path, key):
    """One variable of a .mat file as a numpy array in MATLAB's index order
    (a v7.3 dataset is transposed back from HDF5's row-major view)."""
    if mat_version(path)[0] < 2:
        return np.array(sio.loadmat(path)[key])
    try:
        import h5py
    except ImportError as e:  # pragma: no cover - depends on the environment
        raise ImportError("reading a MATLAB v7.3 (HDF5) .mat file needs h5py") from e
    with h5py.File(path, "r") as f:
        a = np.array(f[key])
    return a.transpose(tuple(range(a.ndim))[::-1])


def load_cacti(origpath, maskpath):
    """``orig`` and ``mask`` (H x W x F, H x W x B) as float32, like
    pnp_sci_test_orig.py:94-110."""
    orig = np.float32(load_mat_array(origpath, "orig"))
    mask = np.float32(load_mat_array(maskpath, "mask"))
    return orig, mask


def cacti_measurements(orig, mask, gaussian_noise_level=0.0, seed=None):
    """Coded measurements of consecutive blocks of B frames
    (pnp_sci_test_orig.py:112-123), float64 H x W x (F // B), with
    N(0, level^2) noise added when ``gaussian_noise_level`` > 0 (:127-129;
    the reference draws from numpy's global generator, here a seeded one)."""
    nmask = mask.shape[2]
    norig = orig.shape[2]
    meas = np.zeros([orig.shape[0], orig.shape[1], norig // nmask])
    for i in range(norig // nmask):
        meas[:, :, i] = np.sum(orig[:, :, i * nmask:(i + 1) * nmask] * mask, 2)
    if gaussian_noise_level:
        rng = np.random.default_rng(seed)
        meas = meas + rng.standard_normal(meas.shape) * gaussian_noise_level
    return meas


def save_results(savedmatdir, save_name, vdenoise, tdenoise, iframe, nframe, Cr, orig=None,
                 psnr_denoise=None, ssim_denoise=None, psnrall_denoise=None, **kwargs):
    """Writes ``{save_name}_kmeas{iframe}_{iframe+nframe-1}.mat`` with the
    fields of utils.py:98-125; returns its path."""
    os.makedirs(savedmatdir, exist_ok=True)
    path = os.path.join(savedmatdir, "{}_kmeas{:d}_{:d}.mat".format(save_name, iframe,
                                                                    iframe + nframe - 1))
    rec = {"vdenoise": np.asarray(vdenoise), "tdenoise": tdenoise, "iframe": iframe,
           "nframe": nframe, "Cr": Cr}
    if orig is not None:
        rec.update({"orig": np.asarray(orig), "psnr_denoise": psnr_denoise,
                    "ssim_denoise": ssim_denoise, "psnrall_denoise": psnrall_denoise,
                    "psnr_mean": float(np.mean(psnr_denoise))})
    rec.update(kwargs)
    sio.savemat(path, rec)
    return path
