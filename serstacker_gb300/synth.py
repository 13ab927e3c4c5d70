"""Seeded synthetic planetary scenes for the registration + stacking workloads.

The reference ships no sample sequences, so every workload is generated here:
a Gaussian-blurred disk with sinusoidal latitude bands on a black background,
rendered analytically (no interpolation error) through a known per-frame warp,
with Poisson shot noise and Gaussian read noise.

Ground truth convention (the ECC one): frame f is rendered so that
``frame_f(W_f(x)) == scene(x)``, i.e. the registration of frame f against the
noiseless reference must return the warp ``W_f``.

Two back ends share the formulas: numpy (small cases, tests) and torch (the
full-size bench workloads, generated on the device).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Scene:
    width: int
    height: int
    radius: float
    edge_sigma: float = 2.0
    band_amp: float = 0.2
    band_period: float = 24.0
    peak: float = 200.0

    @property
    def center(self):
        return (self.width - 1) / 2.0, (self.height - 1) / 2.0


def scene_config0() -> Scene:
    return Scene(640, 480, 180.0)


def scene_config1() -> Scene:
    return Scene(1280, 960, 360.0)


def scene_bayer() -> Scene:
    """Raw 12-bit RGGB mosaic scene: the config-0 scene scaled to 3096x2080
    (disk radius and band period scaled by the width ratio), peak 1500 ADU."""
    f = 3096 / 640.0
    return Scene(3096, 2080, 180.0 * f, edge_sigma=2.0 * f, band_period=24.0 * f, peak=1500.0)


# RGGB cell gains (R, G / G, B) applied to the mosaic: the channels differ in level
BAYER_GAINS = ((1.0, 0.7), (0.7, 0.45))


def _erfc_np(x):
    from scipy.special import erfc
    return erfc(x)


def render_np(sc: Scene, X, Y, blur: float = 0.0):
    """Scene radiance at coordinates (X, Y) (float64 arrays), extra blur sigma."""
    cx, cy = sc.center
    s = math.sqrt(sc.edge_sigma ** 2 + blur ** 2)
    r = np.hypot(X - cx, Y - cy)
    disk = 0.5 * _erfc_np((r - sc.radius) / (math.sqrt(2.0) * s))
    amp = sc.band_amp * math.exp(-2.0 * math.pi ** 2 * (sc.edge_sigma ** 2 + blur ** 2) / sc.band_period ** 2)
    bands = 1.0 + amp * np.sin(2.0 * math.pi * (Y - cy) / sc.band_period)
    return sc.peak * disk * bands / (1.0 + sc.band_amp)


def reference_np(sc: Scene):
    y, x = np.mgrid[0:sc.height, 0:sc.width].astype(np.float64)
    return render_np(sc, x, y)


def homography_from_state(motion: int, state) -> np.ndarray:
    """3x3 matrix of W(x; state) for translation/euclidean/affine/homography."""
    s = np.asarray(state, np.float64)
    if motion == 0:
        return np.array([[1, 0, s[0]], [0, 1, s[1]], [0, 0, 1.0]])
    if motion in (1, 2):
        ca, sa, sc, cx, cy = math.cos(s[2]), math.sin(s[2]), s[3], s[4], s[5]
        return np.array([[sc * ca, -sc * sa, s[0] - sc * ca * cx + sc * sa * cy],
                         [sc * sa, sc * ca, s[1] - sc * sa * cx - sc * ca * cy], [0, 0, 1.0]])
    if motion == 3:
        return np.array([[s[0], s[1], s[2]], [s[3], s[4], s[5]], [0, 0, 1.0]])
    if motion in (4, 7):
        return np.array([[s[0], s[1], s[2]], [s[3], s[4], s[5]], [s[6], s[7], 1.0]])
    raise ValueError("not a projective motion model")


def render_frame_np(sc: Scene, H: np.ndarray, blur: float = 0.0):
    """frame(x') = scene(W^-1(x')) for the projective warp matrix H."""
    Hi = np.linalg.inv(H)
    y, x = np.mgrid[0:sc.height, 0:sc.width].astype(np.float64)
    w = Hi[2, 0] * x + Hi[2, 1] * y + Hi[2, 2]
    X = (Hi[0, 0] * x + Hi[0, 1] * y + Hi[0, 2]) / w
    Y = (Hi[1, 0] * x + Hi[1, 1] * y + Hi[1, 2]) / w
    return render_np(sc, X, Y, blur)


def add_noise_np(rng, img, read_sigma=2.0, gain=1.0, maxval=255):
    counts = rng.poisson(np.clip(img, 0, None)).astype(np.float64)
    counts += rng.normal(0.0, read_sigma, size=img.shape)
    return np.clip(np.rint(counts * gain), 0, maxval)


def random_warps(rng, n: int, kind: str):
    """Per-frame true warps as 3x3 matrices.

    config0: euclidean about (0,0): tx,ty ~ U(-8,8), theta ~ N(0, 0.5 deg)
    config1: homography: the config0 euclidean part, scale 1+U(-0.005,0.005),
             projective terms U(-2e-6, 2e-6) per pixel
    translation: tx,ty ~ U(-8,8) only
    """
    Hs = np.zeros((n, 3, 3))
    for i in range(n):
        tx, ty = rng.uniform(-8, 8, size=2)
        if kind == "translation":
            Hs[i] = np.array([[1.0, 0, tx], [0, 1.0, ty], [0, 0, 1.0]])
            continue
        th = math.radians(rng.normal(0.0, 0.5))
        c, s = math.cos(th), math.sin(th)
        H = np.array([[c, -s, tx], [s, c, ty], [0, 0, 1.0]])
        if kind == "config1":
            k = 1.0 + rng.uniform(-0.005, 0.005)
            H[:2, :2] *= k
            H[2, 0], H[2, 1] = rng.uniform(-2e-6, 2e-6, size=2)
        Hs[i] = H
    return Hs


def make_sequence_np(sc: Scene, n: int, seed: int, kind: str = "config0", dtype=np.uint8, gain=1.0,
                     blur_range=None, read_sigma=2.0):
    """Seeded frames (n, H, W) of ``dtype`` + true warps (n, 3, 3) + per-frame blur."""
    rng = np.random.default_rng(seed)
    Hs = random_warps(rng, n, kind)
    blurs = np.zeros(n) if blur_range is None else rng.uniform(blur_range[0], blur_range[1], size=n)
    maxval = np.iinfo(dtype).max
    frames = np.empty((n, sc.height, sc.width), dtype)
    for i in range(n):
        img = render_frame_np(sc, Hs[i], blurs[i])
        frames[i] = add_noise_np(rng, img, read_sigma, gain, maxval).astype(dtype)
    return frames, Hs, blurs


# --------------------------------------------------------------------------- torch back end

def make_sequence_torch(sc: Scene, n: int, seed: int, kind: str = "config1", gain: float = 64.0,
                        blur_range=(0.8, 2.5), read_sigma: float = 2.0, device="cuda", chunk: int = 64,
                        cell_gains=None, maxval: int = 65535):
    """Full-size sequences generated on the device (bench workloads).

    Same formulas as the numpy back end. ``cell_gains`` (2x2) multiplies the
    radiance per mosaic cell before the noise (raw Bayer frames); counts are
    clipped to [0, maxval]. Returns (frames as an int32 tensor holding the
    unsigned values, warps (n, 3, 3) float64 numpy, blurs numpy).
    """
    import torch
    rng = np.random.default_rng(seed)
    Hs = random_warps(rng, n, kind)
    blurs = rng.uniform(blur_range[0], blur_range[1], size=n) if blur_range else np.zeros(n)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    cx, cy = sc.center
    ys, xs = torch.meshgrid(torch.arange(sc.height, device=device, dtype=torch.float64),
                            torch.arange(sc.width, device=device, dtype=torch.float64), indexing="ij")
    out = torch.empty((n, sc.height, sc.width), dtype=torch.int32, device=device)
    for b0 in range(0, n, chunk):
        b1 = min(n, b0 + chunk)
        Hi = torch.as_tensor(np.linalg.inv(Hs[b0:b1]), device=device)
        bl = torch.as_tensor(blurs[b0:b1], device=device).view(-1, 1, 1)
        w = Hi[:, 2, 0, None, None] * xs + Hi[:, 2, 1, None, None] * ys + Hi[:, 2, 2, None, None]
        X = (Hi[:, 0, 0, None, None] * xs + Hi[:, 0, 1, None, None] * ys + Hi[:, 0, 2, None, None]) / w
        Y = (Hi[:, 1, 0, None, None] * xs + Hi[:, 1, 1, None, None] * ys + Hi[:, 1, 2, None, None]) / w
        s = torch.sqrt(sc.edge_sigma ** 2 + bl ** 2)
        r = torch.hypot(X - cx, Y - cy)
        disk = 0.5 * torch.special.erfc((r - sc.radius) / (math.sqrt(2.0) * s))
        amp = sc.band_amp * torch.exp(-2.0 * math.pi ** 2 * (sc.edge_sigma ** 2 + bl ** 2) / sc.band_period ** 2)
        bands = 1.0 + amp * torch.sin(2.0 * math.pi * (Y - cy) / sc.band_period)
        img = sc.peak * disk * bands / (1.0 + sc.band_amp)
        if cell_gains is not None:
            cg = torch.as_tensor(np.asarray(cell_gains, np.float64), device=device)
            img = img * cg.repeat(sc.height // 2 + 1, sc.width // 2 + 1)[:sc.height, :sc.width]
        counts = torch.poisson(img.clamp_min(0), generator=g)
        counts = counts + read_sigma * torch.randn(counts.shape, generator=g, device=device, dtype=counts.dtype)
        out[b0:b1] = torch.clamp(torch.round(counts * gain), 0, maxval).to(torch.int32)
        del w, X, Y, r, disk, bands, img, counts
    return out, Hs, blurs
