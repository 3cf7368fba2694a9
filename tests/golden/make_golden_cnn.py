"""Generate the CNN-denoiser golden fixtures from the reference itself.

Run in a checkout where the reference tree is available::

    python tests/golden/make_golden_cnn.py /path/to/SCI-algorithms

It imports the reference's own FFDNet and FastDVDnet packages
(``PnP_SCI/python/packages/ffdnet`` and ``packages/fastdvdnet``: models,
layers, ``ffdnet_vdenoiser``, ``fastdvdnet_denoiser``) and its joint and
PnP drivers (``joint_pnp_sci_algo.py``, ``pnp_sci_algo.py``).  Absent
third-party imports get stand-ins: ``cv2``, ``matplotlib``,
``tensorboardX``, ``colour_demosaicing`` (never called here) and
``skimage`` (the Chambolle TV and the metrics are the oracle
restatements).  The networks' trained weights are not in the reference
tree, so every network is filled by ``oracle.cnn.seeded_state_dict`` from
a seed.  The reference's wrappers run on the CPU here (``useGPU=False``
bound in; the drivers call them with the default ``useGPU=True``), in the
float32 of their own code.

Fixtures: ``cnn_ffdnet``, ``cnn_ffdnet_rgb``, ``cnn_fastdvdnet``,
``cnn_fastdvdnet_pad``, ``cnn_joint_gap``, ``cnn_joint_admm``,
``cnn_pnp_gap``, ``cnn_pnp_admm``.
"""
import functools
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import cnn as ocnn  # noqa: E402
from oracle import reference_port as port  # noqa: E402
from oracle.tv_chambolle import denoise_tv_chambolle  # noqa: E402
import sci_algorithms_gb300.datasets as ds  # noqa: E402


def _absent(*_a, **_k):
    raise NotImplementedError("stand-in for a package absent here")


def _install_stand_ins():
    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    sk = mod("skimage", __version__="0.16.2")
    sk.restoration = mod("skimage.restoration", denoise_tv_chambolle=denoise_tv_chambolle,
                         denoise_bilateral=_absent, denoise_wavelet=_absent,
                         estimate_sigma=_absent, denoise_tv_bregman=_absent)
    sk.measure = mod("skimage.measure", compare_psnr=port.compare_psnr,
                     compare_ssim=port.compare_ssim)
    sk.measure.simple_metrics = mod("skimage.measure.simple_metrics",
                                    compare_psnr=port.compare_psnr)
    sk.io = mod("skimage.io", imread=_absent)
    mod("cv2")
    mod("tensorboardX", SummaryWriter=_absent)
    mpl = mod("matplotlib")
    mpl.pyplot = mod("matplotlib.pyplot")
    mod("packages.colour_demosaicing").__path__ = []
    mod("packages.colour_demosaicing.bayer", demosaicing_CFA_Bayer_Menon2007=_absent)


def load_reference(ref_root):
    _install_stand_ins()
    sys.dont_write_bytecode = True
    src = os.path.join(ref_root, "PnP_SCI", "python")
    sys.path.insert(0, src)
    try:
        from packages.ffdnet import models as ffd_models
        from packages.ffdnet import test_ffdnet_ipol as ffd_test
        from packages.fastdvdnet import models as dvd_models
        from packages.fastdvdnet import test_fastdvdnet as dvd_test
        import joint_pnp_sci_algo as joint
        import pnp_sci_algo as algo
    finally:
        sys.path.remove(src)
    # the drivers call the wrappers with useGPU=True; this machine is CPU-only
    ffd = functools.partial(ffd_test.ffdnet_vdenoiser, useGPU=False)
    dvd = functools.partial(dvd_test.fastdvdnet_denoiser, useGPU=False)
    for m in (joint, algo):
        m.ffdnet_vdenoiser = ffd
        m.fastdvdnet_denoiser = dvd
    return ffd_models, dvd_models, ffd, dvd, joint, algo


def seeded(net, seed):
    """Fill a reference module with oracle.cnn.seeded_state_dict weights and
    return (layout names, layout shapes)."""
    import torch
    sd = net.state_dict()
    layout = [(k, tuple(v.shape)) for k, v in sd.items()]
    vals = ocnn.seeded_state_dict(layout, seed)
    net.load_state_dict({k: torch.from_numpy(np.asarray(v)) for k, v in vals.items()})
    net.eval()
    return np.array([k for k, _ in layout]), np.array(json.dumps([list(s) for _, s in layout]))


def noisy_video(H, W, F, seed, sigma):
    v = ds.video_scene(H, W, F, seed=seed)
    return v + np.random.default_rng(seed + 1).standard_normal(v.shape) * sigma


def main(ref_root):
    import torch
    torch.set_num_threads(8)
    ffd_models, dvd_models, ffdnet_vdenoiser, fastdvdnet_denoiser, joint, algo = \
        load_reference(ref_root)
    A_, At_ = port.A_, port.At_
    out = {}

    # --- FFDNet gray: frame-wise video wrapper
    net = ffd_models.FFDNet(num_input_channels=1)
    keys, shapes = seeded(net, 101)
    v = noisy_video(24, 32, 3, 110, 0.05)
    out["cnn_ffdnet"] = dict(v=v, sigma=0.1, x=ffdnet_vdenoiser(v, 0.1, net), seed=101,
                             keys=keys, shapes=shapes)
    ffdnet_gray = net

    # --- FFDNet RGB: the network's forward (estimated noise)
    net = ffd_models.FFDNet(num_input_channels=3)
    keys, shapes = seeded(net, 102)
    xin = np.random.default_rng(111).random((2, 3, 16, 20)).astype(np.float32)
    sig = np.array([0.05, 0.2], np.float32)
    with torch.no_grad():
        noise = net(torch.from_numpy(xin), torch.from_numpy(sig)).numpy()
    out["cnn_ffdnet_rgb"] = dict(x=xin, sigma=sig, noise=noise, seed=102, keys=keys,
                                 shapes=shapes)

    # --- FastDVDnet gray: sequence wrapper (sizes multiples of 4, and one
    # padded single frame -- the wrapper re-pads its noise map every frame,
    # so padded sizes only run for one frame)
    net = dvd_models.FastDVDnet(num_input_frames=5, num_color_channels=1)
    keys, shapes = seeded(net, 103)
    v = noisy_video(24, 32, 7, 112, 0.05).astype(np.float32)
    out["cnn_fastdvdnet"] = dict(v=v, sigma=0.1, x=fastdvdnet_denoiser(v, 0.1, net, gray=True),
                                 seed=103, keys=keys, shapes=shapes)
    v = noisy_video(22, 30, 1, 113, 0.05).astype(np.float32)
    out["cnn_fastdvdnet_pad"] = dict(v=v, sigma=0.08,
                                     x=fastdvdnet_denoiser(v, 0.08, net, gray=True),
                                     seed=103, keys=keys, shapes=shapes)
    fastdvd_gray = net

    # --- joint TV + CNN loops with the seeded networks
    orig = ds.video_scene(24, 32, 8, seed=120)
    mask = ds.bernoulli_mask(24, 32, 8, seed=121)
    meas = np.sum(orig * mask, axis=2)[..., None]
    A = lambda xx: A_(xx, mask)  # noqa: E731
    At = lambda yy: At_(yy, mask)  # noqa: E731
    for projmeth, den, net, seed in (("gap", "tv+ffdnet", ffdnet_gray, 101),
                                     ("admm", "tv+fastdvdnet", fastdvd_gray, 103)):
        args = dict(_lambda=1, tv_weight=0.1, tv_iter_max=5, sigma1=[None],
                    sigma2=[0.1, 0.05], iter_max1=3, iter_max2=[2, 1])
        if projmeth == "gap":
            args["accelerate"] = True
        else:
            args["gamma"] = 0.02
        x_, _t, psnr_, ssim_, psnrall_ = joint.joint_admmdenoise_cacti(
            meas, mask, A, At, projmeth=projmeth, orig=orig, denoiser=den, model=net, **args)
        out["cnn_joint_" + projmeth] = dict(
            meas=meas, mask=mask, orig=orig, x=np.asarray(x_, np.float64),
            psnr=np.array(psnr_), ssim=np.array(ssim_), psnrall=np.array(psnrall_),
            denoiser=den, seed=seed, args_json=np.array(json.dumps(args)))
        print("joint", projmeth, den, np.round(np.mean(psnr_), 3))

    # --- PnP-FFDNet / PnP-FastDVDnet (pnp_sci_algo.py gap_denoise /
    # admm_denoise with the CNN as the denoiser), staged sigma
    for projmeth, den, net, seed in (("gap", "ffdnet", ffdnet_gray, 101),
                                     ("admm", "fastdvdnet", fastdvd_gray, 103)):
        args = dict(_lambda=1, sigma=[0.2, 0.1], iter_max=[2, 2])
        if projmeth == "gap":
            args["accelerate"] = True
        else:
            args["gamma"] = 0.02
        x_, _t, psnr_, ssim_, psnrall_ = algo.admmdenoise_cacti(
            meas, mask, A, At, projmeth=projmeth, orig=orig, denoiser=den, model=net, **args)
        out["cnn_pnp_" + projmeth] = dict(
            meas=meas, mask=mask, orig=orig, x=np.asarray(x_, np.float64),
            psnr=np.array(psnr_), ssim=np.array(ssim_), psnrall=np.array(psnrall_),
            denoiser=den, seed=seed, args_json=np.array(json.dumps(args)))
        print("pnp", projmeth, den, np.round(np.mean(psnr_), 3))

    for name, rec in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    print("wrote", sorted(out))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SCI_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT  (or set SCI_REFERENCE_ROOT): the root of the "
                 "reference checkout, the directory holding PnP_SCI/" % sys.argv[0])
    main(root)
