"""The CNN restatement (oracle/cnn.py) against the reference's own FFDNet /
FastDVDnet code run on seeded weights (tests/golden/make_golden_cnn.py),
and the loops around it against the reference's joint and PnP drivers."""
import json

import numpy as np
import pytest

from oracle import cnn as ocnn
from oracle import reference_port as port

# the reference computes in float32, the restatement in float64
TOL = 2e-5


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def params(g):
    layout = list(zip([str(k) for k in g["keys"]], map(tuple, json.loads(str(g["shapes"])))))
    return ocnn.as_float64(ocnn.seeded_state_dict(layout, int(g["seed"])))


@pytest.mark.parametrize("case,layout", [("cnn_ffdnet", ocnn.ffdnet_layout(1)),
                                         ("cnn_ffdnet_rgb", ocnn.ffdnet_layout(3)),
                                         ("cnn_fastdvdnet", ocnn.fastdvdnet_layout(1))])
def test_checkpoint_layouts_match_reference(golden, case, layout):
    g = golden(case)
    assert [k for k, _ in layout] == [str(k) for k in g["keys"]]
    assert [list(s) for _, s in layout] == json.loads(str(g["shapes"]))


def test_ffdnet_video_denoiser(golden):
    g = golden("cnn_ffdnet")
    x = ocnn.ffdnet_vdenoiser(g["v"], float(g["sigma"]), params(g))
    assert rel(x, g["x"]) < TOL
    with pytest.raises(ValueError):
        ocnn.ffdnet_vdenoiser(g["v"][:-1], 0.1, params(g))


def test_ffdnet_rgb_forward(golden):
    g = golden("cnn_ffdnet_rgb")
    noise = ocnn.ffdnet_forward(params(g), g["x"].astype(np.float64), g["sigma"], C=3)
    assert rel(noise, g["noise"]) < TOL


@pytest.mark.parametrize("case", ["cnn_fastdvdnet", "cnn_fastdvdnet_pad"])
def test_fastdvdnet_denoiser(golden, case):
    g = golden(case)
    x = ocnn.fastdvdnet_denoiser(g["v"], float(g["sigma"]), params(g))
    assert rel(x, g["x"]) < TOL


def test_space_depth_round_trip():
    x = np.random.default_rng(0).random((2, 3, 6, 8))
    assert np.array_equal(ocnn.depth_to_space(ocnn.space_to_depth(x)), x)


@pytest.mark.parametrize("projmeth", ["gap", "admm"])
def test_joint_loops_with_cnn(golden, projmeth):
    g = golden("cnn_joint_" + projmeth)
    p = params(golden("cnn_ffdnet" if projmeth == "gap" else "cnn_fastdvdnet"))
    if projmeth == "gap":
        def cnn(x, nsig, model=None):
            return ocnn.ffdnet_vdenoiser(x, nsig, p)
    else:
        def cnn(x, nsig, model=None):
            return ocnn.fastdvdnet_denoiser(x, nsig, p)
    mask = g["mask"]
    x_, _t, psnr_, ssim_, psnrall_ = port.joint_admmdenoise_cacti(
        g["meas"], mask, lambda x: port.A_(x, mask), lambda y: port.At_(y, mask), cnn,
        projmeth=projmeth, orig=g["orig"], denoiser=str(g["denoiser"]),
        **json.loads(str(g["args_json"])))
    assert rel(x_, g["x"]) < 1e-4
    assert np.max(np.abs(np.array(psnrall_) - g["psnrall"])) < 1e-3


@pytest.mark.parametrize("projmeth", ["gap", "admm"])
def test_pnp_loops_with_cnn(golden, projmeth):
    g = golden("cnn_pnp_" + projmeth)
    p = params(golden("cnn_ffdnet" if projmeth == "gap" else "cnn_fastdvdnet"))
    mask = g["mask"]
    x_, _t, psnr_, ssim_, psnrall_ = port.admmdenoise_cacti(
        g["meas"], mask, lambda x: port.A_(x, mask), lambda y: port.At_(y, mask),
        projmeth=projmeth, orig=g["orig"], denoiser=str(g["denoiser"]), model=p,
        **json.loads(str(g["args_json"])))
    assert rel(x_, g["x"]) < 1e-4
    assert np.max(np.abs(np.array(psnrall_) - g["psnrall"])) < 1e-3
