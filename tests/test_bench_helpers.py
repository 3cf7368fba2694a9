"""bench.py's host-side helpers: the parity figures it reports per
configuration and the CPU description of its baseline (no GPU needed)."""
import math

import numpy as np

import bench


def test_psnr_frames_is_the_mean_of_per_frame_psnr():
    rng = np.random.default_rng(0)
    orig = rng.random((3, 16, 20))
    x = orig + 0.01 * rng.standard_normal(orig.shape)
    want = np.mean([10 * math.log10(1.0 / np.mean((x[b] - orig[b]) ** 2)) for b in range(3)])
    assert abs(bench._psnr_frames(x, orig) - want) < 1e-12
    # float32 input is compared in float64
    assert abs(bench._psnr_frames(x.astype(np.float32), orig) - want) < 1e-3


def test_parity_of_identical_and_perturbed_results():
    rng = np.random.default_rng(1)
    orig = rng.random((2, 8, 8))
    ref = orig + 0.05 * rng.standard_normal(orig.shape)
    r = bench._parity(ref.copy(), ref, orig)
    assert r["rel_l2"] == 0.0 and r["delta_psnr_db"] == 0.0
    assert r["psnr_db"] == r["psnr_oracle_db"]
    x = ref * (1 + 1e-6)
    r = bench._parity(x, ref, orig)
    assert abs(r["rel_l2"] - 1e-6) < 1e-9
    assert abs(r["delta_psnr_db"] - (r["psnr_db"] - r["psnr_oracle_db"])) < 1e-15


def test_host_info_names_cores_and_model():
    h = bench.host_info()
    assert isinstance(h["host_cores"], int) and h["host_cores"] >= 1
    assert isinstance(h["cpu_model"], str) and h["cpu_model"]
    assert h["arch"]
