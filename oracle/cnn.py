"""CPU restatement of the CNN denoisers of the joint / PnP loops (test
infrastructure: only tests and the golden generator use it).

Float64 numpy forward passes of

* FFDNet (``PnP_SCI/python/packages/ffdnet/models.py:26-105``,
  ``functions.py:17-58``) and its frame-wise video wrapper
  ``ffdnet_vdenoiser`` (``packages/ffdnet/test_ffdnet_ipol.py:99-178``);
* FastDVDnet (``packages/fastdvdnet/models.py:13-253``) and its sequence
  wrapper ``fastdvdnet_denoiser`` -> ``fastdvdnet_seqdenoise``
  (``test_fastdvdnet.py:144-201``, ``fastdvdnet.py:86-143``).

Parameters are a dict keyed like the reference's checkpoints (the
``state_dict`` names of its modules, without the ``module.`` prefix of
DataParallel).  ``ffdnet_layout`` / ``fastdvdnet_layout`` restate those
names and shapes; ``seeded_state_dict`` fills a layout deterministically
(the networks' trained weights are not in the reference tree).  The
golden fixtures ``tests/golden/cnn_*.npz`` hold the reference's own
outputs for such weights; ``tests/test_oracle_cnn.py`` pins this file to
them.
"""
import numpy as np

BN_EPS = 1e-5


# ------------------------------------------------------------- primitives
def conv3x3(x, w, stride=1, groups=1):
    """3 x 3 convolution, zero padding 1, no bias.  x: (N, Cin, H, W);
    w: (Cout, Cin / groups, 3, 3)."""
    N, Cin, H, W = x.shape
    Cout = w.shape[0]
    cg, og = Cin // groups, Cout // groups
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    Ho = (H - 1) // stride + 1
    Wo = (W - 1) // stride + 1
    out = np.zeros((N, Cout, Ho, Wo))
    for g in range(groups):
        xs = xp[:, g * cg:(g + 1) * cg]
        wg = w[g * og:(g + 1) * og]
        for di in range(3):
            for dj in range(3):
                patch = xs[:, :, di:di + stride * (Ho - 1) + 1:stride,
                           dj:dj + stride * (Wo - 1) + 1:stride]
                out[:, g * og:(g + 1) * og] += np.einsum("ncij,oc->noij", patch,
                                                         wg[:, :, di, dj])
    return out


def batchnorm(x, p, name):
    """Inference batch normalisation with the running statistics."""
    s = p[name + ".weight"] / np.sqrt(p[name + ".running_var"] + BN_EPS)
    return (x - p[name + ".running_mean"][:, None, None]) * s[:, None, None] + \
        p[name + ".bias"][:, None, None]


def relu(x):
    return np.maximum(x, 0.0)


def space_to_depth(x):
    """(N, C, H, W) -> (N, 4C, H/2, W/2); channel 4c + 2i + j holds the
    pixels at offset (i, j) of the 2 x 2 cells (``functions.py:45-52``)."""
    N, C, H, W = x.shape
    out = np.empty((N, 4 * C, H // 2, W // 2))
    for c in range(C):
        for i in range(2):
            for j in range(2):
                out[:, 4 * c + 2 * i + j] = x[:, c, i::2, j::2]
    return out


def depth_to_space(x):
    """Inverse of space_to_depth (``functions.py:60-93``, and PixelShuffle(2))."""
    N, C4, h, w = x.shape
    C = C4 // 4
    out = np.empty((N, C, 2 * h, 2 * w))
    for c in range(C):
        for i in range(2):
            for j in range(2):
                out[:, c, i::2, j::2] = x[:, 4 * c + 2 * i + j]
    return out


# ----------------------------------------------------------------- FFDNet
def _ffdnet_dims(C):
    if C == 1:
        return 64, 15
    if C == 3:
        return 96, 12
    raise ValueError("FFDNet takes 1 or 3 channels")


def ffdnet_layout(C=1):
    """(name, shape) of FFDNet's parameters and buffers, in checkpoint order."""
    feats, depth = _ffdnet_dims(C)
    pre = "intermediate_dncnn.itermediate_dncnn."
    out = [(pre + "0.weight", (feats, 5 * C, 3, 3))]
    for l in range(depth - 2):
        k = 2 + 3 * l
        out.append((pre + "%d.weight" % k, (feats, feats, 3, 3)))
        for s in ("weight", "bias", "running_mean", "running_var", "num_batches_tracked"):
            out.append((pre + "%d.%s" % (k + 1, s), () if s == "num_batches_tracked" else (feats,)))
    out.append((pre + "%d.weight" % (2 + 3 * (depth - 2)), (4 * C, feats, 3, 3)))
    return out


def ffdnet_forward(p, x, sigma, C=1):
    """FFDNet.forward (models.py:90-105): the estimated noise of x
    (N, C, H, W), H and W even, for noise levels sigma (N,)."""
    feats, depth = _ffdnet_dims(C)
    N, _, H, W = x.shape
    nmap = np.broadcast_to(np.asarray(sigma, np.float64).reshape(N, 1, 1, 1),
                           (N, C, H // 2, W // 2))
    h = np.concatenate([nmap, space_to_depth(x)], axis=1)
    pre = "intermediate_dncnn.itermediate_dncnn."
    h = relu(conv3x3(h, p[pre + "0.weight"]))
    for l in range(depth - 2):
        k = 2 + 3 * l
        h = relu(batchnorm(conv3x3(h, p[pre + "%d.weight" % k]), p, pre + "%d" % (k + 1)))
    h = conv3x3(h, p[pre + "%d.weight" % (2 + 3 * (depth - 2))])
    return depth_to_space(h)


def ffdnet_vdenoiser(v, sigma, p):
    """test_ffdnet_ipol.py:99-178: every frame of v (H x W x F) minus its
    estimated noise at level sigma."""
    v = np.asarray(v, np.float64)
    H, W = v.shape[:2]
    if H % 2 or W % 2:
        raise ValueError("FFDNet needs even frame sizes")
    frames = np.moveaxis(v.reshape(H, W, -1), -1, 0)[:, None]
    noise = ffdnet_forward(p, frames, np.full(frames.shape[0], float(sigma)))
    return np.moveaxis((frames - noise)[:, 0], 0, -1).reshape(v.shape)


# ------------------------------------------------------------- FastDVDnet
def _cv(prefix, cin, cout):
    """CvBlock (models.py:13-27): two (conv, bn) pairs."""
    return [(prefix + "0", "conv", (cout, cin, 3, 3)), (prefix + "1", "bn", cout),
            (prefix + "3", "conv", (cout, cout, 3, 3)), (prefix + "4", "bn", cout)]


def _denblock_layers(C):
    """(module path, kind, shape / width) of DenBlock (models.py:150-206)."""
    # the input convolution has 3 groups, each (frame, noise map) -> 30
    L = [("inc.convblock.0", "conv", (90, C + 1, 3, 3)),
          ("inc.convblock.1", "bn", 90), ("inc.convblock.3", "conv", (32, 90, 3, 3)),
          ("inc.convblock.4", "bn", 32)]
    for name, cin, cout in (("downc0", 32, 64), ("downc1", 64, 128)):
        L += [(name + ".convblock.0", "conv", (cout, cin, 3, 3)),
              (name + ".convblock.1", "bn", cout)]
        L += _cv(name + ".convblock.3.convblock.", cout, cout)
    for name, cin, cout in (("upc2", 128, 64), ("upc1", 64, 32)):
        L += _cv(name + ".convblock.0.convblock.", cin, cin)
        L += [(name + ".convblock.1", "conv", (4 * cout, cin, 3, 3))]
    L += [("outc.convblock.0", "conv", (32, 32, 3, 3)), ("outc.convblock.1", "bn", 32),
          ("outc.convblock.3", "conv", (C, 32, 3, 3))]
    return L


def fastdvdnet_layout(C=1):
    """(name, shape) of FastDVDnet's parameters and buffers, in checkpoint order."""
    out = []
    for t in ("temp1.", "temp2."):
        for path, kind, shp in _denblock_layers(C):
            if kind == "conv":
                out.append((t + path + ".weight", shp))
            else:
                for s in ("weight", "bias", "running_mean", "running_var",
                          "num_batches_tracked"):
                    out.append((t + path + "." + s, () if s == "num_batches_tracked" else (shp,)))
    return out


def _denblock(p, t, in0, in1, in2, nmap):
    """DenBlock.forward (models.py:195-206)."""
    def conv(path, x, stride=1, groups=1):
        return conv3x3(x, p[t + path + ".weight"], stride, groups)

    def bnr(path, x):
        return relu(batchnorm(x, p, t + path))

    def cvblock(pre, x):
        x = bnr(pre + "1", conv(pre + "0", x))
        return bnr(pre + "4", conv(pre + "3", x))

    x = np.concatenate([in0, nmap, in1, nmap, in2, nmap], axis=1)
    x0 = bnr("inc.convblock.1", conv("inc.convblock.0", x, groups=3))
    x0 = bnr("inc.convblock.4", conv("inc.convblock.3", x0))
    x1 = bnr("downc0.convblock.1", conv("downc0.convblock.0", x0, stride=2))
    x1 = cvblock("downc0.convblock.3.convblock.", x1)
    x2 = bnr("downc1.convblock.1", conv("downc1.convblock.0", x1, stride=2))
    x2 = cvblock("downc1.convblock.3.convblock.", x2)
    x2 = depth_to_space(conv("upc2.convblock.1", cvblock("upc2.convblock.0.convblock.", x2)))
    x1 = depth_to_space(conv("upc1.convblock.1",
                             cvblock("upc1.convblock.0.convblock.", x1 + x2)))
    x = bnr("outc.convblock.1", conv("outc.convblock.0", x0 + x1))
    x = conv("outc.convblock.3", x)
    return in1 - x


def fastdvdnet_forward(p, x, nmap, C=1):
    """FastDVDnet.forward (models.py:231-249): x (N, 5C, H, W), H and W
    multiples of 4; nmap (N, 1, H, W)."""
    fr = [x[:, m * C:(m + 1) * C] for m in range(5)]
    x20 = _denblock(p, "temp1.", fr[0], fr[1], fr[2], nmap)
    x21 = _denblock(p, "temp1.", fr[1], fr[2], fr[3], nmap)
    x22 = _denblock(p, "temp1.", fr[2], fr[3], fr[4], nmap)
    return _denblock(p, "temp2.", x20, x21, x22, nmap)


def _reflect_pad(x, hp, wp):
    return np.pad(x, ((0, 0), (0, 0), (0, hp), (0, wp)), mode="reflect")


def fastdvdnet_denoiser(v, sigma, p, gray=True):
    """test_fastdvdnet.py:144-201 with fastdvdnet_seqdenoise
    (fastdvdnet.py:86-143): frame f is denoised from frames f-2..f+2
    (indices modulo the frame count), each window reflect-padded to
    multiples of 4 and cropped back.  v: H x W x F (gray)."""
    if not gray:
        raise ValueError("the oracle restates the grayscale path")
    v = np.asarray(v, np.float64)
    H, W, F = v.shape
    seq = np.moveaxis(v, -1, 0)[:, None]  # F x 1 x H x W
    hp, wp = (-H) % 4, (-W) % 4
    nmap = _reflect_pad(np.full((1, 1, H, W), float(sigma)), hp, wp)
    out = np.empty_like(seq)
    for f in range(F):
        idx = [(f + k - 2) % F for k in range(5)]
        win = _reflect_pad(seq[idx].reshape(1, 5, H, W), hp, wp)
        den = fastdvdnet_forward(p, win, nmap)
        out[f] = den[:, :, :H, :W]
    return np.moveaxis(out[:, 0], 0, -1)


# ------------------------------------------------------- seeded parameters
def seeded_state_dict(layout, seed, last_scale=0.1):
    """Deterministic parameters for a checkpoint layout (numpy PCG64, the
    same stream on every platform): convolution weights He-normal
    (std sqrt(2 / fan_in)), the last convolution of each network scaled by
    ``last_scale``; batch-norm weight U(0.8, 1.2), bias and running mean
    N(0, 0.05^2), running variance U(0.5, 1.5); num_batches_tracked 0."""
    rng = np.random.default_rng(seed)
    conv_names = [k for k, s in layout if len(s) == 4]
    last = {conv_names[-1]}
    if any(k.startswith("temp1.") for k in conv_names):
        last = {max((k for k in conv_names if k.startswith(t)), key=conv_names.index)
                for t in ("temp1.", "temp2.")}
    out = {}
    for k, s in layout:
        if k.endswith("num_batches_tracked"):
            out[k] = np.zeros((), np.int64)
        elif len(s) == 4:
            fan_in = s[1] * s[2] * s[3]
            w = rng.standard_normal(s) * np.sqrt(2.0 / fan_in)
            out[k] = (w * (last_scale if k in last else 1.0)).astype(np.float32)
        elif k.endswith(".weight"):
            out[k] = rng.uniform(0.8, 1.2, s).astype(np.float32)
        elif k.endswith(".running_var"):
            out[k] = rng.uniform(0.5, 1.5, s).astype(np.float32)
        else:
            out[k] = (rng.standard_normal(s) * 0.05).astype(np.float32)
    return out


def as_float64(sd):
    return {k: np.asarray(v, np.float64) for k, v in sd.items()}
