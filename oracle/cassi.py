"""CPU oracle: spectral (CASSI) operators, restated in numpy.

TEST INFRASTRUCTURE ONLY (checker for the CUDA CASSI path).

The reference's Python path has no spectral operator.  The model follows
its MATLAB CASSI test (``DeSCI/test_desci_cassi.m:58-62``: forward with a
shifted mask, ``Phisum = sum(mask.^2, 3)`` with zeros replaced by 1) in the
form of a single coded aperture followed by a dispersion of ``step`` pixels
per band along W:

    y[h, w + step b] += phi[h, w] x[h, w, b]          (H x W x L -> H x Wd)
    x[h, w, b]        = phi[h, w] y[h, w + step b]    (adjoint)

The GAP-TV loop is the reference's own (``oracle.reference_port.gap_denoise``,
a bit-exact port of ``pnp_sci_algo.py:536-706``) with these closures.
Parity status: the operators are restated (no reference implementation
exists to pin them); the loop is pinned.
"""
import numpy as np


def detector_width(W, L, step):
    return W + step * (L - 1)


def cassi_A(x, phi, step=2):
    H, W, L = x.shape
    y = np.zeros((H, detector_width(W, L, step)), dtype=np.result_type(x, phi))
    for b in range(L):
        y[:, step * b:step * b + W] += phi * x[:, :, b]
    return y


def cassi_At(y, phi, L, step=2):
    H, W = phi.shape
    x = np.empty((H, W, L), dtype=np.result_type(y, phi))
    for b in range(L):
        x[:, :, b] = phi * y[:, step * b:step * b + W]
    return x


def cassi_phisum(phi, L, step=2):
    H, W = phi.shape
    s = np.zeros((H, detector_width(W, L, step)), dtype=np.float64)
    for b in range(L):
        s[:, step * b:step * b + W] += phi * phi
    s[s == 0] = 1
    return s
