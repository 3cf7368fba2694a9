"""FFDNet / FastDVDnet module definitions and the reference checkpoint
layout, on the CPU: the networks' own PyTorch forward (the layer stack the
GPU engine folds and batches) against the reference's outputs for seeded
weights, and the checkpoint name translation both ways."""
import json

import numpy as np
import pytest
import torch

from oracle import cnn as ocnn
import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import cnn


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def ref_sd(g, prefix=""):
    layout = list(zip([str(k) for k in g["keys"]], map(tuple, json.loads(str(g["shapes"])))))
    sd = ocnn.seeded_state_dict(layout, int(g["seed"]))
    return {prefix + k: torch.from_numpy(np.asarray(v)) for k, v in sd.items()}


def test_ffdnet_forward_matches_reference(golden):
    g = golden("cnn_ffdnet")
    net = cnn.load_reference_state_dict(sci.FFDNet(1), ref_sd(g, "module.")).double().eval()
    v = torch.from_numpy(g["v"]).permute(2, 0, 1)[:, None]
    with torch.no_grad():
        noise = net(v, torch.full((v.shape[0],), float(g["sigma"]), dtype=torch.float64))
    x = (v - noise)[:, 0].permute(1, 2, 0).numpy()
    assert rel(x, g["x"]) < 2e-5


def test_ffdnet_rgb_forward_matches_reference(golden):
    g = golden("cnn_ffdnet_rgb")
    net = cnn.load_reference_state_dict(sci.FFDNet(3), ref_sd(g)).double().eval()
    with torch.no_grad():
        noise = net(torch.from_numpy(g["x"]).double(), torch.from_numpy(g["sigma"]).double())
    assert rel(noise.numpy(), g["noise"]) < 2e-5


def test_fastdvdnet_forward_matches_reference(golden):
    g = golden("cnn_fastdvdnet")
    net = cnn.load_reference_state_dict(sci.FastDVDnet(5, 1), ref_sd(g)).double().eval()
    v = np.moveaxis(g["v"].astype(np.float64), -1, 0)  # F x H x W
    Fn, H, W = v.shape
    nmap = torch.full((1, 1, H, W), float(g["sigma"]), dtype=torch.float64)
    out = np.empty_like(v)
    with torch.no_grad():
        for f in range(Fn):
            win = torch.from_numpy(v[[(f + k - 2) % Fn for k in range(5)]])[None]
            out[f] = net(win, nmap)[0, 0].numpy()
    assert rel(np.moveaxis(out, 0, -1), g["x"]) < 2e-5


@pytest.mark.parametrize("make,case", [(lambda: sci.FFDNet(1), "cnn_ffdnet"),
                                       (lambda: sci.FFDNet(3), "cnn_ffdnet_rgb"),
                                       (lambda: sci.FastDVDnet(5, 1), "cnn_fastdvdnet")])
def test_checkpoint_names_round_trip(golden, make, case):
    g = golden(case)
    net = make()
    assert sorted(net.reference_names()) == sorted(str(k) for k in g["keys"])
    sd = ref_sd(g)
    cnn.load_reference_state_dict(net, sd)
    back = cnn.reference_state_dict(net)
    assert sorted(back) == sorted(sd)
    for k in sd:
        assert torch.equal(back[k], sd[k])


def test_checkpoint_mismatch_raises(golden):
    sd = ref_sd(golden("cnn_ffdnet"))
    with pytest.raises(KeyError):
        cnn.load_reference_state_dict(sci.FastDVDnet(5, 1), sd)
    sd.pop(next(iter(sd)))
    with pytest.raises(KeyError):
        cnn.load_reference_state_dict(sci.FFDNet(1), sd)


def test_checkpoint_file(golden, tmp_path):
    sd = ref_sd(golden("cnn_ffdnet"), "module.")
    path = tmp_path / "net_gray.pth"
    torch.save(sd, path)
    net = cnn.load_checkpoint(sci.FFDNet(1), str(path))
    assert torch.equal(net.convs[0].weight, sd["module.intermediate_dncnn.itermediate_dncnn.0.weight"])


def test_fold_matches_batchnorm():
    torch.manual_seed(0)
    conv = torch.nn.Conv2d(8, 16, 3, padding=1, bias=False).double()
    bn = torch.nn.BatchNorm2d(16).double().eval()
    bn.running_mean.normal_()
    bn.running_var.uniform_(0.5, 2)
    bn.weight.data.uniform_(0.5, 1.5)
    bn.bias.data.normal_()
    x = torch.randn(2, 8, 9, 11, dtype=torch.float64)
    w, b = cnn._fold(conv, bn, torch.float64)
    ref = bn(conv(x))
    got = torch.nn.functional.conv2d(x, w, b, padding=1)
    assert torch.allclose(got, ref, rtol=1e-5, atol=1e-5)


def test_dense_groups_equals_grouped():
    torch.manual_seed(1)
    w = torch.randn(90, 2, 3, 3, dtype=torch.float64)
    x = torch.randn(1, 6, 8, 8, dtype=torch.float64)
    d = cnn._dense_groups(w, 3, 6)
    a = torch.nn.functional.conv2d(x, w, padding=1, groups=3)
    b = torch.nn.functional.conv2d(x, d, padding=1)
    assert torch.allclose(a, b, rtol=1e-12, atol=1e-12)
