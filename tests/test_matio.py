"""MATLAB .mat IO of the reference's scripts (pnp_sci_test_orig.py:94-123,
utils.py:98-125), on CPU."""
import numpy as np
import pytest
import scipy.io as sio

from sci_algorithms_gb300 import matio


def test_v5_roundtrip_and_measurements(tmp_path):
    rng = np.random.default_rng(0)
    orig = rng.random((12, 16, 8))
    mask = (rng.random((12, 16, 4)) < 0.5).astype(np.uint8)
    sio.savemat(tmp_path / "orig.mat", {"orig": orig})
    sio.savemat(tmp_path / "mask.mat", {"mask": mask})
    assert matio.mat_version(str(tmp_path / "mask.mat"))[0] == 1
    o, m = matio.load_cacti(str(tmp_path / "orig.mat"), str(tmp_path / "mask"))
    assert o.dtype == np.float32 and m.dtype == np.float32
    assert np.array_equal(o, orig.astype(np.float32)) and np.array_equal(m, mask)
    meas = matio.cacti_measurements(o, m)
    assert meas.shape == (12, 16, 2)
    assert np.allclose(meas[..., 1], np.sum(o[..., 4:] * m, axis=2))
    noisy = matio.cacti_measurements(o, m, gaussian_noise_level=5, seed=1)
    assert 3 < np.std(noisy - meas) < 7


def test_save_results_fields(tmp_path):
    v = np.zeros((4, 5, 3), np.float32)
    p = matio.save_results(str(tmp_path / "savedmat"), "kobe_gaptv", v, 1.5, 0, 2, 8, orig=v,
                           psnr_denoise=[30.0, 31.0], ssim_denoise=[0.9, 0.95],
                           psnrall_denoise=[[1.0, 2.0]], projmeth="gap")
    assert p.endswith("kobe_gaptv_kmeas0_1.mat")
    r = sio.loadmat(p)
    assert r["vdenoise"].shape == (4, 5, 3)
    assert float(r["psnr_mean"].squeeze()) == 30.5 and str(r["projmeth"][0]) == "gap"
    q = matio.save_results(str(tmp_path / "savedmat"), "x", v, 1.0, 3, 1, 8)
    assert "orig" not in sio.loadmat(q)


def test_v73_header_is_detected(tmp_path):
    """A v7.3 file (HDF5 with MATLAB's 512-byte header) goes to h5py."""
    hdr = b"MATLAB 7.3 MAT-file, Platform: GLNXA64".ljust(116, b" ") + b"\0" * 8
    hdr += b"\x00\x02" + b"IM"
    (tmp_path / "v73.mat").write_bytes(hdr + b"\0" * 400)
    assert matio.mat_version(str(tmp_path / "v73.mat"))[0] == 2
    try:
        import h5py  # noqa: F401
    except ImportError:
        with pytest.raises(ImportError, match="h5py"):
            matio.load_mat_array(str(tmp_path / "v73.mat"), "mask")
