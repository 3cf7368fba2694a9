"""Generate the golden fixtures in this directory from the reference itself.

Run in a checkout where the reference tree is available::

    python tests/golden/make_golden.py /path/to/SCI-algorithms

It imports the reference's own ``PnP_SCI/python/utils.py`` and
``PnP_SCI/python/pnp_sci_algo.py``.  Their third-party imports are absent
here, so stand-in modules are registered first:

* ``skimage`` (reported as 0.16.2, the release the import code implies)
  whose ``restoration.denoise_tv_chambolle`` is the oracle restatement
  ``oracle.tv_chambolle.denoise_tv_chambolle`` and whose
  ``measure.compare_psnr`` / ``compare_ssim`` are the oracle restatements;
* ``cv2``, ``matplotlib``, the ``packages.ffdnet`` / ``fastdvdnet`` /
  ``colour_demosaicing`` denoisers (never called on the TV path).

Everything else -- ``A_``, ``At_``, ``psnr``, ``gap_denoise``,
``admm_denoise``, ``admmdenoise_cacti``, ``ADMM_TV_rec``,
``gap_denoise_bayer`` and the joint TV + CNN loops of
``joint_pnp_sci_algo.py`` (with a box-blur stand-in for the CNN) -- is the
reference's code, run on the seeded inputs below in float64.  Each fixture
stores the inputs and the reference's outputs; ``tests/test_oracle.py``
checks ``oracle.reference_port`` against them bit for bit, and the GPU tests
compare the CUDA path against them within the FP32 tolerance.
"""
import hashlib
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import reference_port as port  # noqa: E402
from oracle.tv_chambolle import denoise_tv_chambolle  # noqa: E402
import sci_algorithms_gb300.datasets as ds  # noqa: E402


def _not_on_tv_path(*_a, **_k):
    raise NotImplementedError("stand-in: not on the TV path")


# the stand-in CNN of the joint fixtures (a 3 x 3 box blur; the FFDNet /
# FastDVDnet weights are not in the reference tree)
cnn_stand_in = port.cnn_stand_in


def _install_stand_ins():
    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    sk = mod("skimage", __version__="0.16.2")
    sk.restoration = mod("skimage.restoration",
                         denoise_tv_chambolle=denoise_tv_chambolle,
                         denoise_bilateral=_not_on_tv_path,
                         denoise_wavelet=_not_on_tv_path,
                         estimate_sigma=_not_on_tv_path,
                         denoise_tv_bregman=_not_on_tv_path)
    sk.measure = mod("skimage.measure", compare_psnr=port.compare_psnr,
                     compare_ssim=port.compare_ssim)
    mod("cv2")
    mpl = mod("matplotlib")
    mpl.pyplot = mod("matplotlib.pyplot")
    pk = mod("packages")
    pk.__path__ = []
    mod("packages.ffdnet").__path__ = []
    # the CNN denoisers: the box-blur stand-in (used by the joint loops only)
    mod("packages.ffdnet.test_ffdnet_ipol", ffdnet_vdenoiser=cnn_stand_in,
        ffdnet_rgb_denoise=_not_on_tv_path)
    mod("packages.fastdvdnet").__path__ = []
    mod("packages.fastdvdnet.test_fastdvdnet", fastdvdnet_denoiser=cnn_stand_in)
    mod("packages.colour_demosaicing").__path__ = []
    mod("packages.colour_demosaicing.bayer",
        demosaicing_CFA_Bayer_Menon2007=_not_on_tv_path)


def load_reference(ref_root):
    """Import the reference's utils / pnp_sci_algo modules (read-only)."""
    _install_stand_ins()
    sys.dont_write_bytecode = True
    src = os.path.join(ref_root, "PnP_SCI", "python")
    for name in ("utils", "pnp_sci_algo", "joint_pnp_sci_algo"):
        sys.modules.pop(name, None)
    sys.path.insert(0, src)
    try:
        import utils as ref_utils  # noqa: F401
        import pnp_sci_algo as ref_algo
        import joint_pnp_sci_algo as ref_joint
    finally:
        sys.path.remove(src)
    return ref_utils, ref_algo, ref_joint


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def small_video(H, W, B, seed, p=0.5):
    orig = ds.video_scene(H, W, B, seed=seed)
    mask = ds.bernoulli_mask(H, W, B, p=p, seed=seed + 1)
    return orig, mask


def main(ref_root):
    ref_utils, ref, joint = load_reference(ref_root)
    A_, At_ = ref_utils.A_, ref_utils.At_
    out = {}

    # --- operators (utils.py:10-36) ---------------------------------------
    rng = np.random.default_rng(7)
    x = rng.standard_normal((13, 21, 6))
    phi = rng.random((13, 21, 6))
    y = rng.standard_normal((13, 21))
    out["ops"] = dict(x=x, phi=phi, y=y, A=A_(x, phi), At=At_(y, phi),
                      psnr=np.float64(ref_utils.psnr(x, x + 0.01 * y[..., None])),
                      psnr_equal=np.float64(ref_utils.psnr(x, x)))

    # --- GAP / ADMM through the frame-block driver (pnp_sci_algo.py:479) --
    def run_cacti(tag, H, W, B, nframe, projmeth, seed, MAXB=1., v0=False,
                  maskdirection='plain', iframe=0, p=0.5, **args):
        orig, mask = small_video(H, W, B * (nframe + iframe), seed, p=p)
        mask = mask[..., :B]
        orig = orig * MAXB
        meas = np.stack([np.sum(orig[..., k * B:(k + 1) * B] * mask, axis=2)
                         for k in range(nframe + iframe)], axis=2)
        A = lambda xx: A_(xx, mask)  # noqa: E731  (pnp_sci_test_orig.py:147)
        At = lambda yy: At_(yy, mask)  # noqa: E731
        v0_arr = None
        if v0:
            msum = np.sum(mask, axis=2)
            msum[msum == 0] = 1
            v0_arr = np.concatenate([At_(meas[..., k + iframe] / MAXB / msum, mask)
                                     for k in range(nframe)], axis=2)
        x_, t_, psnr_, ssim_, psnrall_ = ref.admmdenoise_cacti(
            meas, mask, A, At, projmeth=projmeth, v0=v0_arr, orig=orig,
            iframe=iframe, nframe=nframe, MAXB=MAXB, maskdirection=maskdirection,
            **args)
        rec = dict(meas=meas, mask=mask, orig=orig, x=x_.astype(np.float64),
                   psnr=np.array(psnr_), ssim=np.array(ssim_),
                   psnrall=np.array(psnrall_), projmeth=projmeth, nframe=nframe,
                   iframe=iframe, MAXB=MAXB, maskdirection=maskdirection,
                   has_v0=v0)
        if v0_arr is not None:
            rec["v0"] = v0_arr
        rec["args_json"] = np.array(json.dumps(args))
        out[tag] = rec
        print(tag, "psnr", np.round(np.mean(psnr_), 3), "x digest", digest(x_)[:12])

    run_cacti("gap_acc", 24, 32, 8, 1, 'gap', seed=10, _lambda=1, accelerate=True,
              denoiser='tv', iter_max=12, tv_weight=0.1, tv_iter_max=5)
    run_cacti("gap_plain", 20, 28, 6, 1, 'gap', seed=20, _lambda=0.8, accelerate=False,
              denoiser='tv', iter_max=[4, 3], sigma=[None, None], tv_weight=0.15,
              tv_iter_max=3)
    run_cacti("gap_tv30", 24, 24, 4, 1, 'gap', seed=30, _lambda=1, accelerate=True,
              denoiser='tv', iter_max=5, tv_weight=0.2, tv_iter_max=30)
    run_cacti("admm", 24, 32, 8, 1, 'admm', seed=40, _lambda=1, gamma=0.01,
              denoiser='tv', iter_max=10, tv_weight=0.1, tv_iter_max=5)
    run_cacti("gap_updown", 16, 24, 4, 3, 'gap', seed=50, MAXB=255., v0=True,
              maskdirection='updown', iframe=1, _lambda=1, accelerate=True,
              denoiser='tv', iter_max=6, tv_weight=0.1, tv_iter_max=5)
    run_cacti("admm_downup", 16, 24, 4, 2, 'admm', seed=60, MAXB=255., v0=True,
              maskdirection='downup', _lambda=1, gamma=0.05,
              denoiser='tv', iter_max=6, tv_weight=0.1, tv_iter_max=4)

    # --- config 0: 256 x 256 x 8, 40 GAP-acc iterations, x0 = At(y/Phisum)
    orig, mask, meas = ds.config0()
    msum = np.sum(mask, axis=2)
    msum[msum == 0] = 1
    v0 = At_(meas / msum, mask)
    A = lambda xx: A_(xx, mask)  # noqa: E731
    At = lambda yy: At_(yy, mask)  # noqa: E731
    x_, _, psnr_, ssim_, psnrall_ = ref.admmdenoise_cacti(
        meas[..., None], mask, A, At, projmeth='gap', v0=v0, orig=orig,
        _lambda=1, accelerate=True, denoiser='tv', iter_max=40,
        tv_weight=0.1, tv_iter_max=5)
    # x_ is float32 (pnp_sci_algo.py:494); the float64 result is kept by
    # calling gap_denoise directly as well
    x64, psnr64, ssim64, psnrall64 = ref.gap_denoise(
        meas, msum, A, At, _lambda=1, accelerate=True, denoiser='tv',
        iter_max=40, tv_weight=0.1, tv_iter_max=5, x0=v0, X_orig=orig)
    out["config0"] = dict(x_digest=np.array(digest(x64)), x_f32=x_,
                          psnr=np.array(psnr64), ssim=np.array(ssim64),
                          psnrall=np.array(psnrall64),
                          orig_digest=np.array(digest(orig)),
                          mask_digest=np.array(digest(mask)),
                          meas_digest=np.array(digest(meas)))
    print("config0 psnr", np.mean(psnr64), "ssim", np.mean(ssim64))

    # --- legacy annealed ADMM loop (pnp_sci_algo.py:884-907) --------------
    orig, mask = small_video(20, 20, 4, seed=70)
    meas = np.sum(orig * mask, axis=2)
    msum = np.sum(mask, axis=2)
    msum[msum == 0] = 1
    v = ref.ADMM_TV_rec(meas, mask, A_, At_, msum, 6, 1.0, 0.1, 20, 20, 4, 0.01, orig)
    g = ref.GAP_TV_rec(meas, mask, A_, At_, msum, 5, 1.0, 0.1, 20, 20, 4, orig)
    out["legacy"] = dict(meas=meas, mask=mask, orig=orig, admm=v, gap=g)

    # --- Bayer GAP-TV (pnp_sci_algo.py:20-265): an RGGB mosaic measured
    # through a full-resolution mask; four sub-lattice problems
    orig, mask = small_video(24, 32, 6, seed=80)
    meas = np.sum(orig * mask, axis=2)
    for acc in (True, False):
        xb, psnr_, ssim_, psnrall_ = ref.gap_denoise_bayer(
            meas, mask, _lambda=1, accelerate=acc, denoiser='tv', iter_max=8,
            tv_weight=0.1, tv_iter_max=5, X_orig=orig)
        out["bayer_gap" + ("_acc" if acc else "")] = dict(
            meas=meas, mask=mask, orig=orig, x=np.asarray(xb, np.float64),
            psnr=np.array(psnr_), ssim=np.array(ssim_), psnrall=np.array(psnrall_),
            accelerate=acc)
    # admm_denoise_bayer (:268-476) reads `ball` before assigning it (:400)
    # and raises; its restatement in the oracle starts the multiplier at 0.
    try:
        ref.admm_denoise_bayer(meas, mask, iter_max=1, X_orig=orig)
        raise RuntimeError("admm_denoise_bayer ran; regenerate its fixture")
    except NameError:
        pass

    # --- joint TV + CNN loops (joint_pnp_sci_algo.py): the CNN denoisers
    # are the box-blur stand-in (their weights are not in the tree)
    jorig, jmask = small_video(24, 32, 8, seed=90)
    jmeas = np.sum(jorig * jmask, axis=2)[..., None]
    A = lambda xx: A_(xx, jmask)  # noqa: E731
    At = lambda yy: At_(yy, jmask)  # noqa: E731
    for projmeth, den in (("gap", "tv+ffdnet"), ("admm", "tv+fastdvdnet")):
        args = dict(_lambda=1, tv_weight=0.1, tv_iter_max=5, sigma1=[None], sigma2=[0.05],
                    iter_max1=5, iter_max2=4)
        if projmeth == "gap":
            args["accelerate"] = True
        else:
            args["gamma"] = 0.02
        x_, t_, psnr_, ssim_, psnrall_ = joint.joint_admmdenoise_cacti(
            jmeas, jmask, A, At, projmeth=projmeth, orig=jorig, denoiser=den, **args)
        out["joint_" + projmeth] = dict(meas=jmeas, mask=jmask, orig=jorig,
                                        x=x_.astype(np.float64), psnr=np.array(psnr_),
                                        ssim=np.array(ssim_), psnrall=np.array(psnrall_),
                                        denoiser=den, args_json=np.array(json.dumps(args)))
        print("joint", projmeth, "psnr", np.round(np.mean(psnr_), 3))

    for name, rec in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    print("wrote", sorted(out))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SCI_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT  (or set SCI_REFERENCE_ROOT): the root of the "
                 "reference checkout, the directory holding PnP_SCI/" % sys.argv[0])
    main(root)
