"""GPU FFDNet / FastDVDnet denoisers (cnn.CnnEngine: folded batch norm,
batched frames, the sci_cnn_* glue kernels, CUDA graphs) against the
reference's own outputs for seeded weights (tests/golden/cnn_*.npz) and
against the oracle restatement where the reference cannot run (odd sizes,
padded multi-frame sequences); and the PnP / joint loops with real networks
against the reference's drivers."""
import ctypes
import json

import numpy as np
import pytest
import torch

from oracle import cnn as ocnn
import sci_algorithms_gb300 as sci
from sci_algorithms_gb300 import cnn
from sci_algorithms_gb300._lib import call

pytestmark = pytest.mark.gpu

# relative error of the estimated noise (output - input) per precision
NOISE_TOL = {"fp32": 1e-4, "tf32": 1e-2, "bf16": 5e-2}


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def ref_sd(g):
    layout = list(zip([str(k) for k in g["keys"]], map(tuple, json.loads(str(g["shapes"])))))
    sd = ocnn.seeded_state_dict(layout, int(g["seed"]))
    return {k: torch.from_numpy(np.asarray(v)) for k, v in sd.items()}


def ffdnet(golden):
    return cnn.load_reference_state_dict(sci.FFDNet(1), ref_sd(golden("cnn_ffdnet"))).eval()


def fastdvdnet(golden):
    g = golden("cnn_fastdvdnet")
    return cnn.load_reference_state_dict(sci.FastDVDnet(5, 1), ref_sd(g)).eval()


def noise_rel(out, v, ref):
    out, v, ref = (np.asarray(a, np.float64) for a in (out, v, ref))
    return np.linalg.norm(out - ref) / np.linalg.norm(v - ref)


@pytest.mark.parametrize("precision", ["fp32", "tf32", "bf16"])
def test_ffdnet_vdenoiser(golden, precision):
    g = golden("cnn_ffdnet")
    x = sci.ffdnet_vdenoiser(g["v"], float(g["sigma"]), model=ffdnet(golden),
                             precision=precision)
    assert x.shape == g["v"].shape and x.dtype == np.float32
    assert noise_rel(x, g["v"], g["x"]) < NOISE_TOL[precision]


@pytest.mark.parametrize("case", ["cnn_fastdvdnet", "cnn_fastdvdnet_pad"])
@pytest.mark.parametrize("precision", ["fp32", "tf32", "bf16"])
def test_fastdvdnet_denoiser(golden, case, precision):
    g = golden(case)
    x = sci.fastdvdnet_denoiser(g["v"], float(g["sigma"]), model=fastdvdnet(golden), gray=True,
                                precision=precision)
    assert x.shape == g["v"].shape
    assert noise_rel(x, g["v"], g["x"]) < NOISE_TOL[precision]


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_fastdvdnet_chunks_and_eager_agree(golden, precision):
    """Frame chunks of 1, 2 and 3 centres and the eager (non-graph) run give
    the graph's result."""
    g = golden("cnn_fastdvdnet")
    net = fastdvdnet(golden)
    x = torch.from_numpy(np.moveaxis(g["v"], -1, 0).copy()).float().cuda()
    full = cnn.CnnEngine(net, "fastdvdnet", precision)(x, 0.1)
    for per in (1, 2, 3):
        eng = cnn.CnnEngine(net, "fastdvdnet", precision, graphs=False)
        eng.chunk_bytes = per * eng._bytes_per_frame(24, 32)
        got = eng(x, 0.1)
        assert torch.allclose(got, full, rtol=0, atol=2e-5 if precision == "fp32" else 2e-2)


def test_graph_replay_takes_new_sigma_and_clip(golden):
    g = golden("cnn_ffdnet")
    net = ffdnet(golden)
    x = torch.from_numpy(np.moveaxis(g["v"], -1, 0).copy()).float().cuda()
    eng = cnn.CnnEngine(net, "ffdnet", "fp32")
    eager = cnn.CnnEngine(net, "ffdnet", "fp32", graphs=False)
    a = eng(x, 0.05)
    b = eng(x, 0.2)
    assert torch.allclose(a, eager(x, 0.05), atol=1e-6)
    assert torch.allclose(b, eager(x, 0.2), atol=1e-6)
    assert not torch.allclose(a, b)
    c = eng(x, 0.2, clip=True)
    assert torch.equal(c, b.clamp(0, 1))


def test_parameter_change_refolds(golden):
    net = ffdnet(golden).cuda()
    g = golden("cnn_ffdnet")
    x = torch.from_numpy(np.moveaxis(g["v"], -1, 0).copy()).float().cuda()
    eng = cnn.CnnEngine(net, "ffdnet", "fp32")
    a = eng(x, 0.1)
    with torch.no_grad():
        net.convs[-1].weight.mul_(2.0)
    b = eng(x, 0.1)
    assert not torch.allclose(a, b)
    assert torch.allclose(x - b, 2 * (x - a), rtol=1e-4, atol=1e-5)


def test_ffdnet_odd_sizes_against_oracle(golden):
    """Odd frames repeat the last row / column (the reference fails on them)."""
    g = golden("cnn_ffdnet")
    v = g["v"][:-1, :-3]  # 23 x 29
    x = sci.ffdnet_vdenoiser(v, 0.1, model=ffdnet(golden), precision="fp32")
    vp = np.pad(v, ((0, 1), (0, 1), (0, 0)), mode="edge")
    p = ocnn.as_float64(ocnn.seeded_state_dict(ocnn.ffdnet_layout(1), int(g["seed"])))
    ref = ocnn.ffdnet_vdenoiser(vp, 0.1, p)[:-1, :-1]
    assert noise_rel(x, v, ref) < 1e-4


def test_fastdvdnet_padded_sequence_against_oracle(golden):
    """Several frames of a size that needs padding (the reference re-pads
    its noise map per frame and fails; the oracle pads each window)."""
    g = golden("cnn_fastdvdnet")
    v = np.asarray(g["v"][:22, :30, :5], np.float32).copy()
    x = sci.fastdvdnet_denoiser(v, 0.1, model=fastdvdnet(golden), gray=True, precision="fp32")
    p = ocnn.as_float64(ocnn.seeded_state_dict(ocnn.fastdvdnet_layout(1), int(g["seed"])))
    ref = ocnn.fastdvdnet_denoiser(v, 0.1, p)
    assert noise_rel(x, v, ref) < 1e-4


def _tree(sd):
    """A module tree with the given (dotted) parameter names, standing in for
    a network built by the reference's own classes."""
    root = torch.nn.Module()
    for k, v in sd.items():
        parts = k.split(".")
        m = root
        for p in parts[:-1]:
            if not hasattr(m, p):
                m.add_module(p, torch.nn.Module())
            m = getattr(m, p)
        m.register_buffer(parts[-1], v.clone())
    return root


def test_reference_built_model_is_converted(golden):
    g = golden("cnn_ffdnet")
    foreign = torch.nn.DataParallel(_tree(ref_sd(g)))
    x = sci.ffdnet_vdenoiser(g["v"], float(g["sigma"]), model=foreign, precision="fp32")
    assert noise_rel(x, g["v"], g["x"]) < 1e-4
    # a later change of the foreign network's weights reaches the converted copy
    last = foreign.module.intermediate_dncnn.itermediate_dncnn
    getattr(last, str(2 + 3 * 13)).weight.mul_(2.0)
    x2 = sci.ffdnet_vdenoiser(g["v"], float(g["sigma"]), model=foreign, precision="fp32")
    assert np.allclose(g["v"] - x2, 2 * (g["v"] - x), rtol=1e-3, atol=1e-5)
    with pytest.raises(ValueError):
        sci.ffdnet_vdenoiser(g["v"], 0.1, model=None)


def test_torch_inputs_stay_on_device(golden):
    g = golden("cnn_fastdvdnet")
    v = torch.from_numpy(g["v"]).cuda()
    x = sci.fastdvdnet_denoiser(v, float(g["sigma"]), model=fastdvdnet(golden), gray=True,
                                precision="fp32")
    assert x.is_cuda and noise_rel(x.cpu().numpy(), g["v"], g["x"]) < 1e-4


@pytest.mark.parametrize("projmeth", ["gap", "admm"])
def test_joint_loops_with_networks(golden, projmeth):
    g = golden("cnn_joint_" + projmeth)
    net = ffdnet(golden) if projmeth == "gap" else fastdvdnet(golden)
    A, At = sci.make_ops(g["mask"])
    x_, _t, psnr_, ssim_, psnrall_ = sci.joint_admmdenoise_cacti(
        g["meas"], g["mask"], A, At, projmeth=projmeth, orig=g["orig"],
        denoiser=str(g["denoiser"]), model=net, precision="fp32",
        **json.loads(str(g["args_json"])))
    assert rel(x_, g["x"]) < 1e-4
    assert np.max(np.abs(np.array(psnr_) - g["psnr"])) < 1e-2
    assert np.max(np.abs(np.array(psnrall_) - g["psnrall"])) < 1e-2


@pytest.mark.parametrize("projmeth", ["gap", "admm"])
def test_pnp_cnn_loops(golden, projmeth):
    g = golden("cnn_pnp_" + projmeth)
    net = ffdnet(golden) if projmeth == "gap" else fastdvdnet(golden)
    A, At = sci.make_ops(g["mask"])
    x_, _t, psnr_, ssim_, psnrall_ = sci.admmdenoise_cacti(
        g["meas"], g["mask"], A, At, projmeth=projmeth, orig=g["orig"],
        denoiser=str(g["denoiser"]), model=net, precision="fp32",
        **json.loads(str(g["args_json"])))
    assert rel(x_, g["x"]) < 1e-4
    assert np.max(np.abs(np.array(psnrall_) - g["psnrall"])) < 1e-2


def test_bf16_joint_loop_close(golden):
    """The bf16 network inside the joint ADMM loop stays near the float32
    reference run (PSNR within 0.05 dB)."""
    g = golden("cnn_joint_admm")
    A, At = sci.make_ops(g["mask"])
    out = sci.joint_admmdenoise_cacti(
        g["meas"], g["mask"], A, At, projmeth="admm", orig=g["orig"],
        denoiser=str(g["denoiser"]), model=fastdvdnet(golden), precision="bf16",
        **json.loads(str(g["args_json"])))
    assert np.max(np.abs(np.array(out[2]) - g["psnr"])) < 0.05


@pytest.mark.parametrize("N,shape", [(96, (2, 37, 53)), (64, (1, 8, 16)), (96, (3, 200, 300)),
                                     (64, (2, 130, 71))])
def test_tcgen05_thin_conv_matches_cudnn(N, shape):
    """sci_cnn_conv_thin (tcgen05, TMEM accumulator) against cuDNN's
    convolution of the same bfloat16 operands: both accumulate in float32
    and round to bfloat16, so they agree to a bfloat16 rounding step."""
    torch.manual_seed(N + shape[1])
    n, H, W = shape
    x = torch.randn(n, 8, H, W, device="cuda").to(torch.bfloat16)
    x = x.contiguous(memory_format=torch.channels_last)
    w = (torch.randn(N, 8, 3, 3, device="cuda") * 0.2).to(torch.bfloat16)
    b = torch.randn(N, device="cuda").to(torch.bfloat16)
    ref = torch.relu(torch.nn.functional.conv2d(x.float(), w.float(), b.float(), padding=1))
    got = cnn.conv_thin(x, cnn._pack_thin(w, b)).float()
    assert got.shape == ref.shape
    err = (got - ref).abs()
    assert float(err.max()) <= 2 ** -7 * float(ref.abs().max()) + 1e-3
    assert float(err.mean()) < 4e-3 * float(ref.abs().mean()) + 1e-4
    got_lin = cnn.conv_thin(x, cnn._pack_thin(w, b), relu=False).float()
    lin = torch.nn.functional.conv2d(x.float(), w.float(), b.float(), padding=1)
    assert float((got_lin - lin).abs().max()) <= 2 ** -7 * float(lin.abs().max()) + 1e-3
    v = ctypes.c_uint(0)
    call("sci_device_status", ctypes.byref(v), 1)
    assert v.value == 0


def test_tc_and_cudnn_first_layers_agree(golden, monkeypatch):
    g = golden("cnn_fastdvdnet")
    net = fastdvdnet(golden)
    x = torch.from_numpy(np.moveaxis(g["v"], -1, 0).copy()).float().cuda()
    a = cnn.CnnEngine(net, "fastdvdnet", "bf16", graphs=False)
    assert a.tc
    monkeypatch.setenv("SCI_CNN_TC", "0")
    b = cnn.CnnEngine(net, "fastdvdnet", "bf16", graphs=False)
    assert not b.tc
    ra, rb = a(x, 0.1), b(x, 0.1)
    assert float((ra - rb).abs().max()) < 2e-2


@pytest.mark.parametrize("kind", ["ffdnet", "fastdvdnet"])
def test_bf16_tensor_core_path_on_odd_sizes(golden, kind):
    """bf16 engine (tcgen05 first layer, NHWC8 glue kernels, shuffle-add) on
    sizes that need padding (FastDVDnet: reflect to multiples of 4; FFDNet:
    odd sizes repeat the last row / column) against the float64 oracle."""
    g = golden("cnn_ffdnet" if kind == "ffdnet" else "cnn_fastdvdnet")
    v = np.asarray(g["v"], np.float32)
    if kind == "ffdnet":
        v = v[:-1, :-3]  # 23 x 29 x 3
        x = sci.ffdnet_vdenoiser(v, 0.1, model=ffdnet(golden), precision="bf16")
        vp = np.pad(v, ((0, 1), (0, 1), (0, 0)), mode="edge")
        p = ocnn.as_float64(ocnn.seeded_state_dict(ocnn.ffdnet_layout(1), int(g["seed"])))
        ref = ocnn.ffdnet_vdenoiser(vp, 0.1, p)[:-1, :-1]
    else:
        v = v[:22, :30, :5].copy()
        x = sci.fastdvdnet_denoiser(v, 0.1, model=fastdvdnet(golden), gray=True,
                                    precision="bf16")
        p = ocnn.as_float64(ocnn.seeded_state_dict(ocnn.fastdvdnet_layout(1), int(g["seed"])))
        ref = ocnn.fastdvdnet_denoiser(v, 0.1, p)
    assert x.shape == v.shape
    assert noise_rel(x, v, ref) < NOISE_TOL["bf16"]


def den_tail_ref(x0, u1, w0, b0, w1, src, first, Hs, Ws, Ho, Wo, clip):
    """DenBlock tail in float64 from the same bfloat16 operands, rounding h
    and o0 to bfloat16 where the kernel stores them."""
    import torch.nn.functional as F
    n, Hp, Wp, _ = x0.shape
    u = u1.double().reshape(n, Hp // 2, Wp // 2, 2, 2, 32).permute(0, 1, 3, 2, 4, 5)
    h = (x0.float() + u.reshape(n, Hp, Wp, 32).float()).to(torch.bfloat16).double()
    h = h.permute(0, 3, 1, 2)
    o0 = F.relu(F.conv2d(h, w0.double().reshape(32, 3, 3, 32).permute(0, 3, 1, 2), b0.double(),
                         padding=1))
    o0 = o0.to(torch.bfloat16).double()
    e = F.conv2d(o0, w1.double().reshape(1, 3, 3, 32).permute(0, 3, 1, 2), padding=1)[:, 0]
    cen = src[first:first + n].double()
    cen = F.pad(cen[:, None], (0, Wp - Ws, 0, Hp - Hs), mode="reflect")[:, 0]
    out = (cen - e)[:, :Ho, :Wo]
    return out.clamp(0, 1) if clip else out


@pytest.mark.parametrize("count,Hs,Ws,Hp,Wp,Ho,Wo,clip", [
    (2, 10, 258, 12, 260, 12, 260, 0),   # three strips, the last one partial; reflect rows / cols
    (1, 7, 130, 8, 132, 7, 130, 1),      # cropped and clipped
    (3, 24, 32, 24, 32, 24, 32, 0),      # narrower than one strip
    (2, 200, 300, 200, 300, 197, 299, 0),
])
def test_den_tail_matches_reference(count, Hs, Ws, Hp, Wp, Ho, Wo, clip):
    """sci_cnn_den_tail (shuffle + add, two tcgen05 convolutions, centre -
    output) against the float64 restatement of the same bfloat16 operands."""
    torch.manual_seed(Hp * 1000 + Wp)
    dev = torch.device("cuda")
    x0 = torch.randn(count, Hp, Wp, 32, device=dev).to(torch.bfloat16)
    u1 = torch.randn(count, Hp // 2, Wp // 2, 128, device=dev).to(torch.bfloat16)
    w0 = (torch.randn(32, 288, device=dev) / 12).to(torch.bfloat16).contiguous()
    b0 = torch.randn(32, device=dev) * 0.1
    w1 = (torch.randn(288, device=dev) / 12).to(torch.bfloat16).contiguous()
    first = 1
    src = torch.rand(first + count + 1, Hs, Ws, device=dev)
    out = torch.full((count, Ho, Wo), float("nan"), device=dev)
    call("sci_cnn_den_tail", x0.data_ptr(), u1.data_ptr(), w0.data_ptr(), b0.data_ptr(),
         w1.data_ptr(), None, src.data_ptr(), src.shape[0], Hs, Ws, first, count, Hp, Wp, Ho, Wo,
         clip, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    ref = den_tail_ref(x0.cpu(), u1.cpu(), w0.cpu(), b0.cpu(), w1.cpu(), src.cpu(), first, Hs,
                       Ws, Ho, Wo, clip)
    got = out.cpu().double()
    assert not torch.isnan(got).any()
    err = (got - ref).abs()
    # an o0 value that rounds to the neighbouring bfloat16 (float32 sums in
    # another order) moves e by about 2^-8 of one product
    assert float(err.max()) < 5e-3
    assert float(err.mean()) < 2e-4
    v = ctypes.c_uint(0)
    call("sci_device_status", ctypes.byref(v), 1)
    assert v.value == 0


def test_fused_tail_and_unfused_agree(golden, monkeypatch):
    """The bf16 FastDVDnet engine with the fused DenBlock tail against the
    same engine running it as shuffle-add, two cuDNN convolutions and the
    centre subtraction, on frames that need padding and three strips; both
    against the float64 oracle."""
    g = golden("cnn_fastdvdnet")
    net = fastdvdnet(golden)
    rng = np.random.default_rng(5)
    v = rng.random((38, 259, 5)).astype(np.float32)  # padded to 40 x 260: three strips
    a = cnn.CnnEngine(net, "fastdvdnet", "bf16", graphs=False)
    assert a.tail
    monkeypatch.setenv("SCI_CNN_TAIL", "0")
    b = cnn.CnnEngine(net, "fastdvdnet", "bf16", graphs=False)
    assert not b.tail
    x = torch.from_numpy(np.moveaxis(v, -1, 0).copy()).cuda()
    ra, rb = a(x, 0.1), b(x, 0.1)
    d = (ra - rb).abs()
    # bf16 networks: the unfused path rounds the output filter's result to
    # bfloat16 before the subtraction, and the first stage's difference
    # moves roundings of the second stage's inputs
    assert float(d.max()) < 2e-2 and float(d.mean()) < 3e-3
    p = ocnn.as_float64(ocnn.seeded_state_dict(ocnn.fastdvdnet_layout(1), int(g["seed"])))
    ref = ocnn.fastdvdnet_denoiser(v, 0.1, p)
    na = noise_rel(np.moveaxis(ra.cpu().numpy(), 0, -1), v, ref)
    nb = noise_rel(np.moveaxis(rb.cpu().numpy(), 0, -1), v, ref)
    assert na < NOISE_TOL["bf16"] and na < 1.1 * nb
