"""Seeded synthetic speckle image pairs with a known imposed displacement field.

The reference's own benchmark images are not distributed with it, so the
workloads are synthetic stand-ins with the shapes and value distributions of
the benchmark configurations:

* a reference image of Gaussian speckles (radius 2-4 px, peak 40-200 gray
  levels) on a background of 20 gray levels, clipped to [0, 255] and rounded;
* a target image obtained by warping the (unquantised) reference with an
  imposed displacement field u(X), v(X): every target pixel x' is mapped back to
  the reference point X that solves X + u(X) = x' (inverse mapping, so the
  imposed field is the one IC-GN recovers at reference POIs), the reference is
  sampled there with bicubic (Catmull-Rom, a = -1/2) interpolation, Gaussian
  noise of sigma 2 gray levels is added, and the result is clipped and rounded.

Everything is numpy and deterministic for a given seed.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Callable, Tuple

import numpy as np

Field = Callable[[np.ndarray, np.ndarray], Tuple[np.ndarray, np.ndarray]]


@dataclasses.dataclass
class SpecklePair:
    ref: np.ndarray          # uint8 [H, W]
    tar: np.ndarray          # uint8 [H, W]
    field: Field             # (X, Y) -> (u, v) imposed at reference coordinates
    grad: Callable[[np.ndarray, np.ndarray], Tuple[np.ndarray, ...]]  # -> (ux, uy, vx, vy)
    description: str


def speckle_intensity(h: int, w: int, n_speckles: int, rng: np.random.Generator,
                      radius=(2.0, 4.0), peak=(40.0, 200.0), background=20.0) -> np.ndarray:
    """Float intensity of `n_speckles` Gaussian speckles I = A exp(-d^2 / R^2)."""
    img = np.full(h * w, background, dtype=np.float64)
    cy = rng.uniform(-4, h + 4, n_speckles)
    cx = rng.uniform(-4, w + 4, n_speckles)
    rad = rng.uniform(radius[0], radius[1], n_speckles)
    amp = rng.uniform(peak[0], peak[1], n_speckles)
    half = int(math.ceil(3 * radius[1]))
    off = np.arange(-half, half + 1)
    chunk = 4096
    for s in range(0, n_speckles, chunk):
        e = min(s + chunk, n_speckles)
        iy = np.floor(cy[s:e]).astype(np.int64)[:, None, None] + off[None, :, None]
        ix = np.floor(cx[s:e]).astype(np.int64)[:, None, None] + off[None, None, :]
        d2 = (iy - cy[s:e, None, None]) ** 2 + (ix - cx[s:e, None, None]) ** 2
        val = amp[s:e, None, None] * np.exp(-d2 / rad[s:e, None, None] ** 2)
        ok = (iy >= 0) & (iy < h) & (ix >= 0) & (ix < w)
        idx = (iy * w + ix)[ok]
        img += np.bincount(idx, weights=val[ok], minlength=h * w)
    return img.reshape(h, w)


def _catmull_rom_weights(t: np.ndarray):
    t2 = t * t
    t3 = t2 * t
    w0 = -0.5 * t3 + t2 - 0.5 * t
    w1 = 1.5 * t3 - 2.5 * t2 + 1.0
    w2 = -1.5 * t3 + 2.0 * t2 + 0.5 * t
    w3 = 0.5 * t3 - 0.5 * t2
    return (w0, w1, w2, w3)


def bicubic_sample(img: np.ndarray, X: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """Catmull-Rom bicubic sample of `img` at (X, Y), edge-clamped."""
    h, w = img.shape
    x0 = np.floor(X).astype(np.int64)
    y0 = np.floor(Y).astype(np.int64)
    wx = _catmull_rom_weights(X - x0)
    wy = _catmull_rom_weights(Y - y0)
    out = np.zeros(X.shape, dtype=np.float64)
    for a in range(4):
        yy = np.clip(y0 + a - 1, 0, h - 1)
        row = np.zeros(X.shape, dtype=np.float64)
        for b in range(4):
            xx = np.clip(x0 + b - 1, 0, w - 1)
            row += wx[b] * img[yy, xx]
        out += wy[a] * row
    return out


def _inverse_map(field: Field, h: int, w: int, iters: int = 30):
    """Solve X + u(X) = x' for every target pixel x' by fixed-point iteration."""
    yp, xp = np.mgrid[0:h, 0:w].astype(np.float64)
    X, Y = xp.copy(), yp.copy()
    for _ in range(iters):
        u, v = field(X, Y)
        X = xp - u
        Y = yp - v
    return X, Y


def make_pair(h: int, w: int, n_speckles: int, field: Field, grad, seed: int, noise_sigma: float = 2.0,
              description: str = "") -> SpecklePair:
    rng = np.random.default_rng(seed)
    intensity = speckle_intensity(h, w, n_speckles, rng)
    ref = np.clip(np.rint(intensity), 0, 255).astype(np.uint8)
    X, Y = _inverse_map(field, h, w)
    tar_f = bicubic_sample(intensity, X, Y) + rng.normal(0.0, noise_sigma, (h, w))
    tar = np.clip(np.rint(tar_f), 0, 255).astype(np.uint8)
    return SpecklePair(ref=ref, tar=tar, field=field, grad=grad, description=description)


def affine_field(u0, v0, ux, uy, vx, vy, cx, cy):
    def field(X, Y):
        dx, dy = X - cx, Y - cy
        return u0 + ux * dx + uy * dy, v0 + vx * dx + vy * dy

    def grad(X, Y):
        one = np.ones_like(np.asarray(X, dtype=np.float64))
        return ux * one, uy * one, vx * one, vy * one

    return field, grad


def sinusoid_field(au, lu, bu, av, lv, bv):
    """u = au sin(2 pi X / lu) + bu, v = av cos(2 pi Y / lv) + bv."""
    def field(X, Y):
        return au * np.sin(2 * np.pi * X / lu) + bu, av * np.cos(2 * np.pi * Y / lv) + bv

    def grad(X, Y):
        X = np.asarray(X, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        z = np.zeros_like(X)
        return (au * 2 * np.pi / lu * np.cos(2 * np.pi * X / lu), z, z,
                -av * 2 * np.pi / lv * np.sin(2 * np.pi * Y / lv))

    return field, grad


# ---------------------------------------------------------------------------
# Benchmark workloads.  Geometry: the ROI leaves a one-pixel image border, which
# the reference's gradient and LUT precompute require (TW_utils.cpp:254-257,
# :615-619).

@dataclasses.dataclass
class Geometry:
    img_w: int
    img_h: int
    start_x: int
    start_y: int
    roi_w: int
    roi_h: int
    subset_r: int
    grid: int
    margin: int
    max_iter: int = 20
    delta_p: float = 0.001
    subset_ry: int = 0  # subset half height when it differs from subset_r (0: square)


def plain_512(seed: int = 2024) -> Tuple[SpecklePair, Geometry]:
    """512x512 pair, uniform affine field, 33x33 subsets at step 10, margin 20."""
    field, grad = affine_field(2.3, -1.7, 0.002, 0.00025, 0.00025, -0.001, 256.0, 256.0)
    pair = make_pair(512, 512, 6000, field, grad, seed, description="512x512 affine speckle pair")
    return pair, Geometry(512, 512, 1, 1, 510, 510, 16, 10, 20)


def scale_2048(seed: int = 7) -> Tuple[SpecklePair, Geometry]:
    """2048x2048 pair, sinusoidal field, 41x41 subsets at step 5, margin 20."""
    field, grad = sinusoid_field(3.0, 1024.0, 1.5, 2.0, 768.0, -0.8)
    pair = make_pair(2048, 2048, 100_000, field, grad, seed, description="2048x2048 sinusoid speckle pair")
    return pair, Geometry(2048, 2048, 1, 1, 2046, 2046, 20, 5, 20)


def small_case(h: int = 160, w: int = 192, r: int = 10, grid: int = 7, seed: int = 11,
               u0: float = 1.6, v0: float = -2.4) -> Tuple[SpecklePair, Geometry]:
    """A small affine case that the oracle finishes in well under a second."""
    n = int(6000 * h * w / (512 * 512))
    field, grad = affine_field(u0, v0, 0.004, -0.002, 0.003, -0.0035, w / 2, h / 2)
    pair = make_pair(h, w, n, field, grad, seed, description=f"{w}x{h} affine speckle pair")
    return pair, Geometry(w, h, 1, 1, w - 2, h - 2, r, grid, 12)


def stripe_pair(h: int = 150, w: int = 170, period: int = 8, y_amp: float = 1.5, shift=(3, 2), seed: int = 5,
                noise_sigma: float = 2.0) -> Tuple[np.ndarray, np.ndarray]:
    """A low-texture pair with a broad, periodic correlation surface:
    vertical stripes of `period` px (amplitude 50 around 128) with a weak
    vertical texture of amplitude `y_amp`, the target shifted by an integer
    `shift` (dx, dy), noise sigma `noise_sigma`.  In a window whose width is a
    multiple of the period nearly every vertical shift at every period
    multiple correlates within 0.01 ZNCC of the peak (about 200 shifts per
    40 x 40 window at y_amp 1.5, 40 to 80 at y_amp 8)."""
    rng = np.random.default_rng(seed)
    H, W = h + 40, w + 40
    x = np.arange(W)[None, :]
    y = np.arange(H)[:, None]
    base = 128 + 50.0 * np.sin(2 * np.pi * x / period) + y_amp * np.sin(2 * np.pi * y / 37.0) * np.cos(
        2 * np.pi * x / 53.0)
    base = np.broadcast_to(base, (H, W))
    dx, dy = shift
    ref = base[20:20 + h, 20:20 + w] + rng.normal(0, noise_sigma, (h, w))
    tar = base[20 - dy:20 - dy + h, 20 - dx:20 - dx + w] + rng.normal(0, noise_sigma, (h, w))
    return (np.clip(np.rint(ref), 0, 255).astype(np.uint8), np.clip(np.rint(tar), 0, 255).astype(np.uint8))


def camera_sequence(w: int, h: int, frames: int = 3, seed: int = 31, r: int = 15, grid: int = 8,
                    margin: int = 20):
    """A simulated camera: one reference and `frames` targets under a linear
    ramp of strain (up to 1 % at the last frame) plus a drift of 0.5 px per
    frame, speckle density as in the 512x512 case.  Returns (ref, targets,
    Geometry) with 31x31 subsets at step 8 by default."""
    rng_seed = seed
    n = int(6000 * h * w / (512 * 512))
    rng = np.random.default_rng(rng_seed)
    intensity = speckle_intensity(h, w, n, rng)
    ref = np.clip(np.rint(intensity), 0, 255).astype(np.uint8)
    tars = []
    yp, xp = np.meshgrid(np.arange(h, dtype=np.float64), np.arange(w, dtype=np.float64), indexing="ij")
    cx, cy = w / 2, h / 2
    for k in range(1, frames + 1):
        s = 0.01 * k / frames
        u0, v0, ux, vy = 0.5 * k, -0.35 * k, s, -0.6 * s
        # inverse of the affine map X + u(X) = x' in closed form
        X = cx + (xp - cx - u0) / (1.0 + ux)
        Y = cy + (yp - cy - v0) / (1.0 + vy)
        tar_f = bicubic_sample(intensity, X, Y) + rng.normal(0.0, 2.0, (h, w))
        tars.append(np.clip(np.rint(tar_f), 0, 255).astype(np.uint8))
    return ref, tars, Geometry(w, h, 1, 1, w - 2, h - 2, r, grid, margin)
