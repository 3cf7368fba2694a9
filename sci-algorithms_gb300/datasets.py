"""Seeded synthetic inputs standing in for the reference's benchmark data.

The reference's videos and masks (kobe32, traffic, bm_256_10f, the
large-scale sets; ``PnP_SCI/python/pnp_sci_test_orig.py:94-110``) are not
available, so every measurement here is built from seeded generators with
the shapes and value ranges of the workloads this project is measured on:

* ``video_scene``: per frame, a background of six random 2-D sinusoids
  plus five Gaussian blobs (sigma 8-20 px) moving linearly 2-4 px per
  frame, min-max normalised over the clip to [0, 1];
* ``bernoulli_mask``: i.i.d. binary coded-aperture masks;
* ``spectral_cube``: a CASSI cube whose every 16 x 16 region carries a
  spectrum made of three random Gaussian peaks.

All arrays are float64 in the reference layout H x W x B (frames last).
Seeds follow a fixed convention: scene 0, mask 1, noise 2.
"""
import numpy as np


def video_scene(H, W, B, seed=0):
    """Smooth moving scene, H x W x B float64 in [0, 1]."""
    rng = np.random.default_rng(seed)
    yy = np.arange(H, dtype=np.float64)
    xx = np.arange(W, dtype=np.float64)
    # six plane waves: cos(kx x + ky y + phase) = cos(a)cos(b) - sin(a)sin(b)
    waves = []
    for _ in range(6):
        cycles = rng.uniform(2.0, 16.0)
        theta = rng.uniform(0.0, np.pi)
        k = 2.0 * np.pi * cycles / max(H, W)
        kx, ky = k * np.cos(theta), k * np.sin(theta)
        phase = rng.uniform(0.0, 2.0 * np.pi)
        amp = rng.uniform(0.2, 1.0)
        drift = rng.uniform(-0.3, 0.3)  # phase drift per frame
        waves.append((kx, ky, phase, amp, drift))
    blobs = []
    for _ in range(5):
        sig = rng.uniform(8.0, 20.0)
        cy, cx = rng.uniform(0.15, 0.85) * H, rng.uniform(0.15, 0.85) * W
        speed = rng.uniform(2.0, 4.0)
        ang = rng.uniform(0.0, 2.0 * np.pi)
        amp = rng.uniform(0.6, 1.6)
        blobs.append((sig, cy, cx, speed * np.sin(ang), speed * np.cos(ang), amp))
    out = np.empty((H, W, B), dtype=np.float64)
    for t in range(B):
        fr = np.zeros((H, W), dtype=np.float64)
        for kx, ky, phase, amp, drift in waves:
            a = kx * xx
            b = ky * yy + phase + drift * t
            fr += amp * (np.outer(np.cos(b), np.cos(a)) - np.outer(np.sin(b), np.sin(a)))
        for sig, cy, cx, vy, vx, amp in blobs:
            gy = np.exp(-0.5 * ((yy - (cy + vy * t)) / sig) ** 2)
            gx = np.exp(-0.5 * ((xx - (cx + vx * t)) / sig) ** 2)
            fr += amp * np.outer(gy, gx)
        out[:, :, t] = fr
    lo, hi = out.min(), out.max()
    out -= lo
    out /= (hi - lo)
    return out


def bernoulli_mask(H, W, B, p=0.5, seed=1):
    """Binary coded-aperture masks, H x W x B float64 in {0, 1}."""
    rng = np.random.default_rng(seed)
    return (rng.random((H, W, B)) < p).astype(np.float64)


def measure(orig, mask, noise_rel=0.0, seed=2):
    """Snapshot y = sum_b mask_b * orig_b (+ Gaussian noise sigma = rel*max y).

    Same forward model as the reference drivers
    (``PnP_SCI/python/pnp_sci_test_orig.py:113-118``, noise ``:128``), but
    seeded.
    """
    y = np.sum(orig * mask, axis=2)
    if noise_rel > 0:
        rng = np.random.default_rng(seed)
        y = y + rng.standard_normal(y.shape) * (noise_rel * y.max())
    return y


def spectral_cube(H=256, W=256, L=28, region=16, seed=0):
    """CASSI test cube H x W x L in [0, 1]: 3 Gaussian spectral peaks per
    ``region`` x ``region`` block, bilinearly blended between blocks so the
    cube is spatially smooth."""
    rng = np.random.default_rng(seed)
    gh, gw = -(-H // region) + 1, -(-W // region) + 1
    lam = np.arange(L, dtype=np.float64)
    spec = np.zeros((gh, gw, L))
    for _ in range(3):
        c = rng.uniform(0, L - 1, size=(gh, gw, 1))
        s = rng.uniform(1.5, 5.0, size=(gh, gw, 1))
        a = rng.uniform(0.3, 1.0, size=(gh, gw, 1))
        spec += a * np.exp(-0.5 * ((lam - c) / s) ** 2)
    ty = np.arange(H) / region
    tx = np.arange(W) / region
    iy, ix = np.floor(ty).astype(int), np.floor(tx).astype(int)
    fy, fx = (ty - iy)[:, None, None], (tx - ix)[None, :, None]
    cube = ((1 - fy) * (1 - fx) * spec[iy][:, ix] + (1 - fy) * fx * spec[iy][:, ix + 1]
            + fy * (1 - fx) * spec[iy + 1][:, ix] + fy * fx * spec[iy + 1][:, ix + 1])
    cube -= cube.min()
    cube /= cube.max()
    return cube


def video_config(H, W, B, p=0.5, noise_rel=0.0, seeds=(0, 1, 2)):
    """(orig, mask, meas) for one video-SCI measurement."""
    orig = video_scene(H, W, B, seed=seeds[0])
    mask = bernoulli_mask(H, W, B, p=p, seed=seeds[1])
    meas = measure(orig, mask, noise_rel=noise_rel, seed=seeds[2])
    return orig, mask, meas


def config0():
    """256 x 256 x 8, Bernoulli(0.5), noise-free (CPU-runnable case)."""
    return video_config(256, 256, 8)


def config1():
    """2048 x 2048 x 24, Bernoulli(0.5), noise sigma = 0.01 max(y)."""
    return video_config(2048, 2048, 24, noise_rel=0.01)


def batch_config(n=64, seed=0, sizes=(128, 256, 512, 1024), frames=(8, 16, 24, 32)):
    """Uneven batch: item i has H = W drawn from ``sizes``, B from ``frames``,
    its own Bernoulli(p) mask with p ~ U[0.3, 0.7], the video scene generator
    and no noise; seeds (1000+i, 1000+i+1, 1000+i+2).  Yields
    (orig, mask, meas) one item at a time (the largest is 1024^2 x 32)."""
    rng = np.random.default_rng(seed)
    shapes = [(int(rng.choice(sizes)), int(rng.choice(frames)), float(rng.uniform(0.3, 0.7)))
              for _ in range(n)]
    for i, (s, b, p) in enumerate(shapes):
        yield video_config(s, s, b, p=p, seeds=(1000 + i, 1000 + i + 1, 1000 + i + 2))


def batch_shapes(n=64, seed=0, sizes=(128, 256, 512, 1024), frames=(8, 16, 24, 32)):
    """The (H, W, B, p) of ``batch_config`` without generating the data."""
    rng = np.random.default_rng(seed)
    return [(s, s, b, p) for s, b, p in
            ((int(rng.choice(sizes)), int(rng.choice(frames)), float(rng.uniform(0.3, 0.7)))
             for _ in range(n))]
