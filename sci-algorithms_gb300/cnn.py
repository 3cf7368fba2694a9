"""FFDNet and FastDVDnet denoisers for the CNN stages of the PnP and joint
TV + CNN loops (``PnP_SCI/python/packages/ffdnet``, ``packages/fastdvdnet``).

* ``FFDNet`` / ``FastDVDnet``: the networks with the reference's layer
  sizes and forward semantics (``ffdnet/models.py:60-105``,
  ``fastdvdnet/models.py:13-253``).  Their parameters load from the
  reference's checkpoints (``load_reference_state_dict``: the reference's
  ``state_dict`` names, with or without DataParallel's ``module.``), and a
  model built by the reference's own classes is converted on first use.
* ``ffdnet_vdenoiser`` / ``fastdvdnet_denoiser``: the reference's wrapper
  functions (``test_ffdnet_ipol.py:99-178``, ``test_fastdvdnet.py:144-201``)
  on the GPU.

Execution (``CnnEngine``) is laid out for one GB300 rather than as the
reference's per-frame loops:

* every frame of a stack goes through one batched network call (FFDNet's
  per-frame loop, FastDVDnet's per-frame window loop);
* FastDVDnet's first-stage denoiser is evaluated once per centre frame and
  shared by the three output frames whose windows contain it (the reference
  evaluates it three times per output frame) -- the same arithmetic, a
  third of the first-stage work;
* inference batch norm is folded into the preceding convolution; ReLU is
  fused into the convolution where cuDNN offers it;
* input and output tensors are built by this library's kernels
  (``sci_cnn_*``: 2 x 2 space-to-depth with the noise map, the circular
  frame window with reflect padding, and the final subtraction / crop /
  [0, 1] clip) straight from the planar frame stack;
* activations are channels-last (NHWC) with channel counts padded to
  multiples of 8 (cuDNN's NHWC kernels run TF32 about 5x faster than NCHW
  on GB300); ``precision``: 'fp32' (IEEE convolutions), 'tf32' (cuDNN's
  default, what the reference's GPU run computes in) or 'bf16' (bfloat16
  tensor-core convolutions, the first layer by this library's tcgen05
  kernel); frames are float32 in and out;
* each (frames, H, W) shape is captured once as a CUDA graph and replayed.

The trained weights are not part of the reference tree (git-LFS pointers),
so none ship here: pass ``model`` built from a checkpoint.
"""
import os
import weakref

import torch
import torch.nn as nn
import torch.nn.functional as F

from . import _dev
from ._lib import call

NCHW_F32 = 0  # SCI_CNN_NCHW_F32
NHWC8_BF16 = 1  # SCI_CNN_NHWC8_BF16
NHWC8_F32 = 2  # SCI_CNN_NHWC8_F32
PRECISIONS = ("fp32", "tf32", "bf16")
_default_precision = "tf32"


def set_default_precision(p):
    """Precision of CNN denoiser calls that do not name one."""
    global _default_precision
    if p not in PRECISIONS:
        raise ValueError("precision must be one of %s" % (PRECISIONS,))
    _default_precision = p


def _conv(cin, cout, stride=1, groups=1):
    return nn.Conv2d(cin, cout, 3, stride=stride, padding=1, groups=groups, bias=False)


# ----------------------------------------------------------------- FFDNet
class FFDNet(nn.Module):
    """FFDNet: 2 x 2 space-to-depth plus a noise-level map, a conv-BN-ReLU
    stack (gray: 15 layers of 64 features; RGB: 12 of 96) and
    depth-to-space; ``forward(x, noise_sigma)`` returns the estimated
    noise of x (N, C, H, W) like ``models.py:90-105``."""

    def __init__(self, num_input_channels=1):
        super().__init__()
        if num_input_channels not in (1, 3):
            raise ValueError("FFDNet takes 1 or 3 channels")
        C = num_input_channels
        self.num_input_channels = C
        self.feats, self.depth = (64, 15) if C == 1 else (96, 12)
        f = self.feats
        self.convs = nn.ModuleList([_conv(5 * C, f)] + [_conv(f, f) for _ in range(self.depth - 2)]
                                   + [_conv(f, 4 * C)])
        self.norms = nn.ModuleList([nn.BatchNorm2d(f) for _ in range(self.depth - 2)])

    def forward(self, x, noise_sigma):
        N, C, H, W = x.shape
        nmap = noise_sigma.reshape(N, 1, 1, 1).to(x.dtype).expand(N, C, H // 2, W // 2)
        h = torch.cat([nmap, F.pixel_unshuffle(x, 2)], dim=1)
        h = F.relu(self.convs[0](h))
        for conv, bn in zip(self.convs[1:-1], self.norms):
            h = F.relu(bn(conv(h)))
        return F.pixel_shuffle(self.convs[-1](h), 2)

    def reference_names(self):
        """{reference checkpoint name: own name} (models.py layer indices)."""
        pre = "intermediate_dncnn.itermediate_dncnn."
        m = {pre + "0.weight": "convs.0.weight"}
        for l in range(self.depth - 2):
            k = 2 + 3 * l
            m[pre + "%d.weight" % k] = "convs.%d.weight" % (l + 1)
            for s in ("weight", "bias", "running_mean", "running_var", "num_batches_tracked"):
                m[pre + "%d.%s" % (k + 1, s)] = "norms.%d.%s" % (l, s)
        m[pre + "%d.weight" % (2 + 3 * (self.depth - 2))] = "convs.%d.weight" % (self.depth - 1)
        return m


# ------------------------------------------------------------- FastDVDnet
# (own layer name, reference module path, has batch norm) of one DenBlock,
# in the reference's registration order
_DEN_LAYERS = [
    ("in0", "inc.convblock.0", "inc.convblock.1"),
    ("in1", "inc.convblock.3", "inc.convblock.4"),
    ("d0a", "downc0.convblock.0", "downc0.convblock.1"),
    ("d0b", "downc0.convblock.3.convblock.0", "downc0.convblock.3.convblock.1"),
    ("d0c", "downc0.convblock.3.convblock.3", "downc0.convblock.3.convblock.4"),
    ("d1a", "downc1.convblock.0", "downc1.convblock.1"),
    ("d1b", "downc1.convblock.3.convblock.0", "downc1.convblock.3.convblock.1"),
    ("d1c", "downc1.convblock.3.convblock.3", "downc1.convblock.3.convblock.4"),
    ("u2a", "upc2.convblock.0.convblock.0", "upc2.convblock.0.convblock.1"),
    ("u2b", "upc2.convblock.0.convblock.3", "upc2.convblock.0.convblock.4"),
    ("u2c", "upc2.convblock.1", None),
    ("u1a", "upc1.convblock.0.convblock.0", "upc1.convblock.0.convblock.1"),
    ("u1b", "upc1.convblock.0.convblock.3", "upc1.convblock.0.convblock.4"),
    ("u1c", "upc1.convblock.1", None),
    ("o0", "outc.convblock.0", "outc.convblock.1"),
    ("o1", "outc.convblock.3", None),
]


class DenBlock(nn.Module):
    """One FastDVDnet denoising block: three frames and their noise maps ->
    a U-Net of 32 / 64 / 128 features -> the centre frame minus the
    output (``models.py:150-206``)."""

    def __init__(self, num_color_channels=1):
        super().__init__()
        C = num_color_channels
        shapes = {"in0": (3 * (C + 1), 90, 1, 3), "in1": (90, 32, 1, 1),
                  "d0a": (32, 64, 2, 1), "d0b": (64, 64, 1, 1), "d0c": (64, 64, 1, 1),
                  "d1a": (64, 128, 2, 1), "d1b": (128, 128, 1, 1), "d1c": (128, 128, 1, 1),
                  "u2a": (128, 128, 1, 1), "u2b": (128, 128, 1, 1), "u2c": (128, 256, 1, 1),
                  "u1a": (64, 64, 1, 1), "u1b": (64, 64, 1, 1), "u1c": (64, 128, 1, 1),
                  "o0": (32, 32, 1, 1), "o1": (32, C, 1, 1)}
        self.conv = nn.ModuleDict()
        self.bn = nn.ModuleDict()
        for name, _, bn in _DEN_LAYERS:
            cin, cout, stride, groups = shapes[name]
            self.conv[name] = _conv(cin, cout, stride, groups)
            if bn is not None:
                self.bn[name] = nn.BatchNorm2d(cout)

    def _cbr(self, name, x):
        return F.relu(self.bn[name](self.conv[name](x)))

    def forward(self, in0, in1, in2, noise_map):
        x0 = self._cbr("in0", torch.cat([in0, noise_map, in1, noise_map, in2, noise_map], 1))
        x0 = self._cbr("in1", x0)
        x1 = self._cbr("d0c", self._cbr("d0b", self._cbr("d0a", x0)))
        x2 = self._cbr("d1c", self._cbr("d1b", self._cbr("d1a", x1)))
        x2 = F.pixel_shuffle(self.conv["u2c"](self._cbr("u2b", self._cbr("u2a", x2))), 2)
        x1 = F.pixel_shuffle(self.conv["u1c"](self._cbr("u1b", self._cbr("u1a", x1 + x2))), 2)
        x = self.conv["o1"](self._cbr("o0", x0 + x1))
        return in1 - x


class FastDVDnet(nn.Module):
    """FastDVDnet: two stages of DenBlocks over a 5-frame window
    (``models.py:208-253``); ``forward(x, noise_map)`` takes x
    (N, 5C, H, W), H and W multiples of 4, and returns (N, C, H, W)."""

    def __init__(self, num_input_frames=5, num_color_channels=3):
        super().__init__()
        if num_input_frames != 5:
            raise ValueError("FastDVDnet takes a 5-frame window")
        self.num_input_frames = num_input_frames
        self.num_color_channels = num_color_channels
        self.temp1 = DenBlock(num_color_channels)
        self.temp2 = DenBlock(num_color_channels)

    def forward(self, x, noise_map):
        C = self.num_color_channels
        f = [x[:, m * C:(m + 1) * C] for m in range(5)]
        x20 = self.temp1(f[0], f[1], f[2], noise_map)
        x21 = self.temp1(f[1], f[2], f[3], noise_map)
        x22 = self.temp1(f[2], f[3], f[4], noise_map)
        return self.temp2(x20, x21, x22, noise_map)

    def reference_names(self):
        m = {}
        for t in ("temp1", "temp2"):
            for name, cpath, bpath in _DEN_LAYERS:
                m["%s.%s.weight" % (t, cpath)] = "%s.conv.%s.weight" % (t, name)
                if bpath is not None:
                    for s in ("weight", "bias", "running_mean", "running_var",
                              "num_batches_tracked"):
                        m["%s.%s.%s" % (t, bpath, s)] = "%s.bn.%s.%s" % (t, name, s)
        return m


# ------------------------------------------------------ checkpoint format
def _strip(sd):
    return {(k[7:] if k.startswith("module.") else k): v for k, v in sd.items()}


def load_reference_state_dict(model, state_dict):
    """Load a checkpoint in the reference's layout (its modules'
    ``state_dict`` names, optionally DataParallel-prefixed) into ``model``."""
    sd = _strip(state_dict)
    names = model.reference_names()
    missing = sorted(set(names) - set(sd))
    extra = sorted(set(sd) - set(names))
    if missing or extra:
        raise KeyError("checkpoint does not match %s: missing %s, unexpected %s"
                       % (type(model).__name__, missing[:4], extra[:4]))
    own = {names[k]: v for k, v in sd.items()}
    model.load_state_dict(own, strict=True)
    return model


def reference_state_dict(model):
    """``model``'s parameters under the reference's checkpoint names."""
    inv = {v: k for k, v in model.reference_names().items()}
    return {inv[k]: v for k, v in model.state_dict().items()}


def load_checkpoint(model, path):
    """Read a reference checkpoint file (``torch.save`` of a state dict)."""
    return load_reference_state_dict(model, torch.load(path, map_location="cpu"))


_converted = weakref.WeakKeyDictionary()


def as_native(model, kind):
    """This module's network for ``model``: itself, or a converted copy of
    a network built by the reference's own classes (cached per model)."""
    if isinstance(model, nn.DataParallel):
        model = model.module
    if isinstance(model, (FFDNet, FastDVDnet)):
        return model
    if not isinstance(model, nn.Module):
        raise TypeError("model must be an FFDNet / FastDVDnet network, got %s"
                        % type(model).__name__)
    # the converted copy follows later changes of the foreign network's
    # parameters (their version counters)
    versions = tuple(t._version for t in list(model.parameters()) + list(model.buffers()))
    hit = _converted.get(model)
    if hit is not None and hit[1] == versions:
        return hit[0]
    sd = _strip(model.state_dict())
    if kind == "ffdnet":
        w = sd.get("intermediate_dncnn.itermediate_dncnn.0.weight")
        if w is None:
            raise TypeError("model is not an FFDNet")
        net = FFDNet(w.shape[1] // 5)
    else:
        w = sd.get("temp1.inc.convblock.0.weight")
        if w is None:
            raise TypeError("model is not a FastDVDnet")
        net = FastDVDnet(5, w.shape[1] - 1)
    if hit is not None:  # reload into the same copy, so that its engines refold
        net = hit[0]
    load_reference_state_dict(net, sd)
    net.eval()
    _converted[model] = (net, versions)
    return net


# ---------------------------------------------------------------- engine
class _Prec:
    """cuDNN's TF32 switch for the duration of a call (restored after)."""

    def __init__(self, precision):
        self.tf32 = precision == "tf32"

    def __enter__(self):
        self.saved = (torch.backends.cudnn.allow_tf32, torch.backends.cudnn.benchmark)
        torch.backends.cudnn.allow_tf32 = self.tf32
        torch.backends.cudnn.benchmark = True

    def __exit__(self, *exc):
        torch.backends.cudnn.allow_tf32, torch.backends.cudnn.benchmark = self.saved


def _pad8(n):
    return (n + 7) // 8 * 8


def _fold(conv, bn, dtype, cin_pad=None, cout_pad=None, cl=False):
    """(weight, bias) of conv followed by inference batch norm; bias None
    for a convolution without batch norm (the networks' convolutions have
    no bias of their own)."""
    w = conv.weight.detach().float()
    cout = w.shape[0]
    b = None
    if bn is not None:
        s = bn.weight.detach().float() / torch.sqrt(bn.running_var.detach().float() + bn.eps)
        b = bn.bias.detach().float() - bn.running_mean.detach().float() * s
        w = w * s[:, None, None, None]
    if cin_pad is not None and cin_pad > w.shape[1]:
        w = F.pad(w, (0, 0, 0, 0, 0, cin_pad - w.shape[1]))
    if cout_pad is not None and cout_pad > cout:
        w = F.pad(w, (0, 0, 0, 0, 0, 0, 0, cout_pad - cout))
        if b is not None:
            b = F.pad(b, (0, cout_pad - cout))
    w = w.to(dtype)
    if cl:
        w = w.contiguous(memory_format=torch.channels_last)
    return w, (None if b is None else b.to(dtype))


def _subpixel_major(w):
    """Output channels c*4 + k of an upsampling convolution (PixelShuffle(2)
    order) reordered to k*C + c, so that each sub-pixel's C channels are one
    contiguous vector for sci_cnn_shuffle_add."""
    C = w.shape[0] // 4
    perm = torch.tensor([c * 4 + k for k in range(4) for c in range(C)], device=w.device)
    return w[perm]


def _dense_groups(w, groups, cin_total):
    """Grouped (Cout, Cin/g, 3, 3) weight as an equivalent dense one."""
    cout, cg = w.shape[0], w.shape[1]
    og = cout // groups
    d = torch.zeros(cout, cin_total, 3, 3, dtype=w.dtype, device=w.device)
    for g in range(groups):
        d[g * og:(g + 1) * og, g * cg:(g + 1) * cg] = w[g * og:(g + 1) * og]
    return d


def _pack_thin(w, b):
    """(N, 8, 3, 3) weights -> the N x 80 bfloat16 rows of sci_cnn_conv_thin
    (k = (3 dy + dx) * 8 + c, k >= 72 zero); bias as float32."""
    N = w.shape[0]
    wp = torch.zeros(N, 80, dtype=torch.bfloat16, device=w.device)
    wp[:, :72] = w.float().permute(0, 2, 3, 1).reshape(N, 72).to(torch.bfloat16)
    bias = b.float() if b is not None else torch.zeros(N, device=w.device)
    return wp.contiguous(), bias.contiguous()


def conv_thin(x, packed, relu=True):
    """sci_cnn_conv_thin on a bfloat16 NHWC8 tensor given as its
    channels-last (n, 8, H, W) view; returns the (n, N, H, W) channels-last
    view of the NHWC output."""
    wp, bias = packed
    n, c8, H, W = x.shape
    xn = x.permute(0, 2, 3, 1)
    if c8 != 8 or x.dtype != torch.bfloat16 or not xn.is_contiguous():
        raise ValueError("conv_thin takes a bfloat16 NHWC8 tensor")
    N = wp.shape[0]
    out = torch.empty((n, H, W, N), dtype=torch.bfloat16, device=x.device)
    call("sci_cnn_conv_thin", xn.data_ptr(), wp.data_ptr(), bias.data_ptr(), out.data_ptr(), n,
         H, W, N, int(relu), _dev.stream_handle())
    return out.permute(0, 3, 1, 2)


_fused_relu_ok = {}


def _conv_act(h, w, b, stride=1, groups=1, relu=True, tf32=False):
    """3 x 3 convolution + bias (+ ReLU) through cuDNN's fused
    convolution-bias-activation op; without bias or ReLU, the plain cuDNN
    convolution (aten's generic path picks slower kernels for bfloat16
    NHWC)."""
    if not relu and b is None:
        return torch.cudnn_convolution(h, w, (1, 1), (stride, stride), (1, 1), groups, True,
                                       False, tf32)
    key = (h.dtype, h.is_contiguous(memory_format=torch.channels_last), groups)
    if relu and _fused_relu_ok.get(key, True):
        try:
            return torch.cudnn_convolution_relu(h, w, b, (stride, stride), (1, 1), (1, 1), groups)
        except (RuntimeError, NotImplementedError):
            _fused_relu_ok[key] = False
    out = F.conv2d(h, w, b, stride, 1, 1, groups)
    return F.relu_(out) if relu else out


class CnnEngine:
    """Inference of one FFDNet / FastDVDnet on planar frame stacks.

    ``engine(x, sigma, clip=False)``: x (frames, H, W) float32 CUDA,
    returns the denoised stack (frames, H, W), clipped to [0, 1] when
    ``clip``.  FFDNet denoises frame by frame (batched); FastDVDnet uses the
    circular 5-frame window of the reference's sequence denoiser.
    """

    def __init__(self, model, kind, precision=None, graphs=True, chunk_bytes=24 << 30):
        self.kind = kind
        self.net = as_native(model, kind)
        self.precision = precision or _default_precision
        if self.precision not in PRECISIONS:
            raise ValueError("precision must be one of %s" % (PRECISIONS,))
        self.bf16 = self.precision == "bf16"
        # channels-last everywhere (cuDNN's NHWC kernels: TF32 about 5x its
        # NCHW rate on GB300); NHWC8 frames in / out of the glue kernels
        self.dtype = torch.bfloat16 if self.bf16 else torch.float32
        self.layout = NHWC8_BF16 if self.bf16 else NHWC8_F32
        # first layer on the tensor cores by this library's tcgen05 kernel
        # (bf16 only; SCI_CNN_TC=0 leaves it to cuDNN)
        self.tc = self.bf16 and os.environ.get("SCI_CNN_TC", "1") != "0"
        # FastDVDnet's DenBlock tail (full-resolution shuffle + add, the two
        # output convolutions, centre - output) in one tcgen05 kernel
        # (bf16 only; SCI_CNN_TAIL=0 runs it as shuffle-add, two cuDNN
        # convolutions and the centre subtraction)
        self.tail = self.tc and os.environ.get("SCI_CNN_TAIL", "1") != "0"
        self.graphs = graphs
        self.chunk_bytes = chunk_bytes
        self.dev = _dev.device()
        self.sigma = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self._versions = None
        self._graphs = {}
        self._fold()

    # -- parameters --------------------------------------------------------
    def _param_versions(self):
        return tuple(t._version for t in list(self.net.parameters()) + list(self.net.buffers()))

    def _fold(self):
        """Folded, channel-padded weights in the execution dtype, NHWC."""
        net = self.net.to(self.dev).eval()
        dt = self.dtype
        if self.kind == "ffdnet":
            if net.num_input_channels != 1:
                raise ValueError("the frame-stack engine runs the grayscale FFDNet")
            layers = []
            for i, conv in enumerate(net.convs):
                bn = net.norms[i - 1] if 0 < i < len(net.convs) - 1 else None
                cin_pad = 8 if i == 0 else None                    # NHWC8 input
                cout_pad = 8 if i == len(net.convs) - 1 else None  # 4 -> 8 outputs
                layers.append(_fold(conv, bn, dt, cin_pad, cout_pad, cl=True))
            self.layers = layers
            self.first_tc = _pack_thin(*layers[0]) if self.tc else None
        else:
            if net.num_color_channels != 1:
                raise ValueError("the frame-stack engine runs the grayscale FastDVDnet")
            self.blocks = []
            for blk in (net.temp1, net.temp2):
                p = {}
                for name, _, bpath in _DEN_LAYERS:
                    conv = blk.conv[name]
                    bn = blk.bn[name] if bpath is not None else None
                    if name == "in0":
                        # the 3-group input convolution as one dense 8 -> 96
                        # filter on the NHWC8 window (channels 6, 7 and
                        # outputs 90..95 zero)
                        w, b = _fold(conv, bn, torch.float32)
                        w = F.pad(_dense_groups(w, 3, 6), (0, 0, 0, 0, 0, 2))
                        w = F.pad(w, (0, 0, 0, 0, 0, 0, 0, 6))
                        b = F.pad(b, (0, 6))
                        p[name] = (w.to(dt).contiguous(memory_format=torch.channels_last),
                                   b.to(dt))
                        if self.tc:
                            p["in0_tc"] = _pack_thin(*p[name])
                    elif name == "in1":
                        p[name] = _fold(conv, bn, dt, cin_pad=96, cl=True)
                    elif name == "o1":
                        p[name] = _fold(conv, bn, dt, cout_pad=8, cl=True)
                        if self.tail:
                            w1 = p[name][0][0].permute(1, 2, 0).reshape(-1).contiguous()
                            p["tail_o1"] = (w1, None)
                    elif name in ("u2c", "u1c"):
                        w, b = _fold(conv, bn, dt)
                        p[name] = (_subpixel_major(w).contiguous(
                            memory_format=torch.channels_last), b)
                    else:
                        p[name] = _fold(conv, bn, dt, cl=True)
                        if name == "o0" and self.tail:
                            w0, b0 = p[name]
                            p["tail_o0"] = (w0.permute(0, 2, 3, 1).reshape(32, 288).contiguous(),
                                            b0.float().contiguous())
                self.blocks.append(p)
        self._versions = self._param_versions()
        self._graphs.clear()

    def _nhwc(self, n, H, W, C, dev):
        """An NHWC tensor (n, H, W, C) of the execution dtype."""
        return torch.empty((n, H, W, C), dtype=self.dtype, device=dev)

    @staticmethod
    def _dense(t):
        """The NHWC storage of a channels-last (n, C, H, W) view."""
        n = t.permute(0, 2, 3, 1)
        return n if n.is_contiguous() else n.contiguous()

    # -- FFDNet ------------------------------------------------------------
    def _ffdnet(self, x, out, clip):
        Fn, H, W = x.shape
        H2, W2 = (H + 1) // 2, (W + 1) // 2
        s = _dev.stream_handle()
        h = self._nhwc(Fn, H2, W2, 8, x.device)
        call("sci_cnn_ffdnet_pack", x.data_ptr(), Fn, H, W, self.sigma.data_ptr(), h.data_ptr(),
             self.layout, s)
        h = h.permute(0, 3, 1, 2)  # channels-last view
        L = self.layers
        tf32 = self.precision == "tf32"
        for i, (w, b) in enumerate(L):
            if i == 0 and self.tc:
                h = conv_thin(h, self.first_tc)
            else:
                h = _conv_act(h, w, b, relu=i < len(L) - 1, tf32=tf32)
        noise = self._dense(h)
        call("sci_cnn_ffdnet_unpack_sub", x.data_ptr(), noise.data_ptr(), Fn, H, W, self.layout,
             noise.shape[-1], int(clip), out.data_ptr(), s)

    # -- FastDVDnet ----------------------------------------------------------
    def _denblock(self, p, win, src, Hs, Ws, first, count, Hp, Wp, Ho, Wo, clip, out):
        """DenBlock on a prepared window tensor, then out = centre - DenBlock
        (cropped to Ho x Wo, clipped when `clip`)."""
        tf = self.precision == "tf32"

        def c(x, name, stride=1, relu=True):
            w, b = p[name]
            return _conv_act(x, w, b, stride, 1, relu, tf)

        x0 = c(conv_thin(win, p["in0_tc"]) if self.tc else c(win, "in0"), "in1")
        x1 = c(c(c(x0, "d0a", 2), "d0b"), "d0c")
        x2 = c(c(c(x1, "d1a", 2), "d1b"), "d1c")
        u2 = c(c(c(x2, "u2a"), "u2b"), "u2c", relu=False)
        x1 = self._shuffle_add(x1, u2)
        u1 = c(c(c(x1, "u1a"), "u1b"), "u1c", relu=False)
        if self.tail:
            x0n, u1n = self._dense(x0), self._dense(u1)
            (w0, b0), (w1, _) = p["tail_o0"], p["tail_o1"]
            call("sci_cnn_den_tail", x0n.data_ptr(), u1n.data_ptr(), w0.data_ptr(),
                 b0.data_ptr(), w1.data_ptr(), None, src.data_ptr(), src.shape[0], Hs, Ws, first,
                 count, Hp, Wp, Ho, Wo, int(clip), out.data_ptr(), _dev.stream_handle())
            return
        r = c(c(self._shuffle_add(x0, u1), "o0"), "o1", relu=False)
        self._center_sub(src, Hs, Ws, first, count, r, Hp, Wp, Ho, Wo, clip, out)

    def _shuffle_add(self, a, u):
        """a + PixelShuffle(2)(u) on NHWC tensors (u's channels in
        sub-pixel-major order), by sci_cnn_shuffle_add(_f32)."""
        N, C, H2, W2 = a.shape
        an, un = self._dense(a), self._dense(u)
        out = self._nhwc(N, H2, W2, C, a.device)
        fn = "sci_cnn_shuffle_add" if self.bf16 else "sci_cnn_shuffle_add_f32"
        call(fn, an.data_ptr(), un.data_ptr(), out.data_ptr(), N, H2 // 2, W2 // 2, C,
             _dev.stream_handle())
        return out.permute(0, 3, 1, 2)

    def _window(self, src, Hs, Ws, Hp, Wp, first, count):
        w = self._nhwc(count, Hp, Wp, 8, src.device)
        call("sci_cnn_window", src.data_ptr(), src.shape[0], Hs, Ws, Hp, Wp, first, count,
             self.sigma.data_ptr(), w.data_ptr(), self.layout, _dev.stream_handle())
        return w.permute(0, 3, 1, 2)  # channels-last view

    def _center_sub(self, src, Hs, Ws, first, count, r, Hp, Wp, Ho, Wo, clip, out):
        rr = self._dense(r)
        call("sci_cnn_center_sub", src.data_ptr(), src.shape[0], Hs, Ws, first, count,
             rr.data_ptr(), self.layout, rr.shape[-1], Hp, Wp, Ho, Wo, int(clip),
             out.data_ptr(), _dev.stream_handle())

    def _fastdvdnet(self, x, out, clip):
        if self.net.num_color_channels != 1:
            raise ValueError("the frame-stack engine runs the grayscale FastDVDnet")
        Fn, H, W = x.shape
        Hp, Wp = H + (-H) % 4, W + (-W) % 4
        if (Hp > H and Hp - H >= H) or (Wp > W and Wp - W >= W):
            raise ValueError("FastDVDnet's reflect padding needs frames of at least 4 x 4")
        step = max(1, min(Fn, self.chunk_bytes // self._bytes_per_frame(Hp, Wp)))
        # first stage, once per centre frame g: T[g] = x[g] - DenBlock1(x[g-1], x[g],
        # x[g+1]) at the padded size; output frame f's three first-stage
        # results are then T[f-1], T[f], T[f+1]
        T = torch.empty((Fn, Hp, Wp), device=x.device)
        for a in range(0, Fn, step):
            n = min(step, Fn - a)
            self._denblock(self.blocks[0], self._window(x, H, W, Hp, Wp, a, n), x, H, W, a, n,
                           Hp, Wp, Hp, Wp, False, T[a:a + n])
        # second stage over the windows of T, cropped back to H x W
        for a in range(0, Fn, step):
            n = min(step, Fn - a)
            self._denblock(self.blocks[1], self._window(T, Hp, Wp, Hp, Wp, a, n), T, Hp, Wp, a,
                           n, Hp, Wp, H, W, clip, out[a:a + n])

    def _bytes_per_frame(self, Hp, Wp):
        # live activations of one DenBlock call at full resolution (~4
        # tensors of 96 channels) plus the half / quarter levels
        e = 2 if self.bf16 else 4  # activations of the execution dtype
        return int(Hp * Wp * e * (4 * 96 + 2 * 64 + 2 * 32)) + 1

    # -- call ---------------------------------------------------------------
    def run(self, x, out, clip=False):
        """Eager run into ``out`` (no graph)."""
        if self._param_versions() != self._versions:
            self._fold()
        with _Prec(self.precision), torch.no_grad():
            if self.kind == "ffdnet":
                self._ffdnet(x, out, clip)
            else:
                self._fastdvdnet(x, out, clip)
        return out

    def __call__(self, x, sigma, clip=False):
        x = x.contiguous()
        if x.dim() != 3 or x.dtype != torch.float32 or not x.is_cuda:
            raise ValueError("expected a (frames, H, W) float32 CUDA stack")
        self.sigma.fill_(float(sigma))
        if not self.graphs:
            return self.run(x, torch.empty_like(x), clip)
        if self._param_versions() != self._versions:
            self._fold()
        key = (tuple(x.shape), bool(clip))
        g = self._graphs.get(key)
        if g is None:
            g = self._capture(x, clip)
            self._graphs[key] = g
        graph, xin, xout = g
        xin.copy_(x)
        graph.replay()
        return xout.clone()

    def _capture(self, x, clip):
        xin = x.clone()
        xout = torch.empty_like(x)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(2):  # cuDNN algorithm selection and workspaces
                self.run(xin, xout, clip)
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            self.run(xin, xout, clip)
        return graph, xin, xout


_engines = weakref.WeakKeyDictionary()


def engine_for(model, kind, precision=None):
    """The cached CnnEngine of ``model`` for this precision."""
    prec = precision or _default_precision
    net = as_native(model, kind)
    per = _engines.setdefault(net, {})
    e = per.get(prec)
    if e is None:
        e = CnnEngine(net, kind, prec)
        per[prec] = e
    return e


def conv_flops(model, kind, nframes, H, W):
    """Multiply-add FLOPs (2 per MAC) of one denoiser call on nframes H x W
    frames, counted on the network's own layer shapes (grouped convolution
    at its group size, no channel padding).  FastDVDnet counts the
    2 * nframes DenBlock evaluations the engine runs (the reference's
    per-frame loop runs 4 * nframes)."""
    net = as_native(model, kind)

    def conv(c, h, w):
        k = c.weight.shape
        return 2.0 * k[0] * k[1] * k[2] * k[3] * h * w

    if kind == "ffdnet":
        h, w = (H + 1) // 2, (W + 1) // 2
        return nframes * sum(conv(c, h, w) for c in net.convs)
    Hp, Wp = H + (-H) % 4, W + (-W) % 4
    level = {"in0": 1, "in1": 1, "d0a": 2, "d0b": 2, "d0c": 2, "d1a": 4, "d1b": 4, "d1c": 4,
             "u2a": 4, "u2b": 4, "u2c": 4, "u1a": 2, "u1b": 2, "u1c": 2, "o0": 1, "o1": 1}
    per = sum(conv(net.temp1.conv[n], Hp // s, Wp // s) for n, s in level.items())
    return 2 * nframes * per


# ------------------------------------------------- the reference's wrappers
def _check_model(model, name):
    if model is None:
        raise ValueError("%s: pass model= (the trained weights are not part of the reference "
                         "tree; build FFDNet / FastDVDnet and load_checkpoint)" % name)


def ffdnet_vdenoiser(vnoisy, sigma, model=None, useGPU=True, precision=None, clip=False):
    """``test_ffdnet_ipol.py:99-178``: every frame of vnoisy (H x W x F,
    numpy or torch) minus FFDNet's estimated noise at level sigma.  Runs on
    the GPU whatever ``useGPU`` says; numpy in -> float32 numpy out, torch
    in -> CUDA tensor out.  Odd sizes repeat the last row / column (the
    reference fails on them)."""
    _check_model(model, "ffdnet_vdenoiser")
    shape = tuple(vnoisy.shape)
    v = vnoisy.reshape(shape[0], shape[1], -1)
    x = _dev.planar(v)
    y = engine_for(model, "ffdnet", precision)(x, sigma, clip)
    out = _dev.unplanar(y, vnoisy)
    return out.reshape(shape)


def fastdvdnet_denoiser(vnoisy, sigma, model=None, useGPU=True, gray=False, precision=None,
                        clip=False):
    """``test_fastdvdnet.py:144-201``: FastDVDnet over the frames of vnoisy
    (H x W x F gray, ``gray=True``; the colour form H x W x F x 3 runs the
    colour network frame by frame in PyTorch), each frame from the 5-frame
    window around it (indices modulo F), reflect-padded to multiples of 4
    (the reference re-pads its noise map every frame and so fails on more
    than one padded frame; here every frame is padded alike)."""
    _check_model(model, "fastdvdnet_denoiser")
    if not gray:
        return _fastdvdnet_color(vnoisy, sigma, model, precision)
    x = _dev.planar(vnoisy)
    y = engine_for(model, "fastdvdnet", precision)(x, sigma, clip)
    return _dev.unplanar(y, vnoisy)


def _fastdvdnet_color(vnoisy, sigma, model, precision):
    net = as_native(model, "fastdvdnet").to(_dev.device()).eval()
    t = vnoisy if _dev.is_torch(vnoisy) else torch.from_numpy(vnoisy)
    seq = t.to(_dev.device(), torch.float32).permute(2, 3, 0, 1).contiguous()  # F C H W
    N, C, H, W = seq.shape
    hp, wp = (-H) % 4, (-W) % 4
    nmap = F.pad(torch.full((1, 1, H, W), float(sigma), device=seq.device), (0, wp, 0, hp),
                 mode="reflect")
    out = torch.empty_like(seq)
    with _Prec(precision or _default_precision), torch.no_grad():
        for f in range(N):
            idx = torch.tensor([(f + k - 2) % N for k in range(5)], device=seq.device)
            win = F.pad(seq[idx].reshape(1, 5 * C, H, W), (0, wp, 0, hp), mode="reflect")
            out[f] = net(win, nmap)[0, :, :H, :W]
    res = out.permute(2, 3, 0, 1)
    return res if _dev.is_torch(vnoisy) else res.contiguous().cpu().numpy()
