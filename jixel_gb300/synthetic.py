"""Seeded synthetic test images for the VarDCT front end workloads.

No public benchmark set ships with the reference encoder, so every workload is
drawn from one generator (numpy PCG64): low-frequency cosine gradients,
Gaussian noise, hard-edged rectangles (axis-aligned or 45 degrees), an 8-px
checker patch and, for the large workloads, a 1/f^2 band-limited texture.
"""
from __future__ import annotations

import numpy as np


def _texture(rng: np.random.Generator, h: int, w: int) -> np.ndarray:
    """1/f^2-spectrum noise normalised to [0, 255] per channel."""
    try:
        from scipy import fft as _fft
        irfft2 = lambda a, s: _fft.irfft2(a, s=s, workers=-1)  # noqa: E731
    except ImportError:  # pragma: no cover
        irfft2 = lambda a, s: np.fft.irfft2(a, s=s)  # noqa: E731
    fy = np.fft.fftfreq(h).astype(np.float32)[:, None]
    fx = np.fft.rfftfreq(w).astype(np.float32)[None, :]
    f2 = fx * fx + fy * fy
    f2[0, 0] = 1.0
    amp = (1.0 / np.sqrt(f2)).astype(np.float32)
    amp[0, 0] = 0.0
    out = np.empty((h, w, 3), np.float32)
    for c in range(3):
        phase = rng.uniform(0, 2 * np.pi, size=amp.shape).astype(np.float32)
        spec = (amp * np.cos(phase)) + 1j * (amp * np.sin(phase))
        t = irfft2(spec.astype(np.complex64), (h, w)).astype(np.float32)
        t -= t.min()
        t *= 255.0 / max(float(t.max()), 1e-6)
        out[..., c] = t
    return out


def generate(width: int, height: int, seed: int, *, noise_sigma: float = 6.0,
             rectangles: int = 20, texture_weight: float = 0.0, sixteen_bit: bool = False,
             alpha: bool = False) -> np.ndarray:
    """Return an (h, w, 3|4) uint8 sRGB image, or uint16 linear with ``sixteen_bit``."""
    rng = np.random.Generator(np.random.PCG64(seed))
    yy = np.arange(height, dtype=np.float32)[:, None]
    xx = np.arange(width, dtype=np.float32)[None, :]
    img = np.full((height, width, 3), 128.0, np.float32)
    for _ in range(3):
        cycles = rng.uniform(0.5, 3.0)
        theta = rng.uniform(0, np.pi)
        phase = rng.uniform(0, 2 * np.pi)
        u = (xx * np.cos(theta) / width + yy * np.sin(theta) / height) * cycles * 2 * np.pi
        wave = np.cos(u + phase)
        img += (40.0 * wave)[..., None] * rng.uniform(-1, 1, size=3).astype(np.float32)
    if texture_weight > 0:
        img = (1 - texture_weight) * img + texture_weight * _texture(rng, height, width)
    img += rng.normal(0, noise_sigma, size=img.shape).astype(np.float32)
    side_lo, side_hi = 0.02 * min(width, height), 0.25 * min(width, height)
    for _ in range(rectangles):
        cw = rng.uniform(side_lo, side_hi)
        chh = rng.uniform(side_lo, side_hi)
        cx = rng.uniform(0, width)
        cy = rng.uniform(0, height)
        fill = rng.uniform(0, 255, size=3).astype(np.float32)
        if rng.uniform() < 0.5:
            x0, x1 = int(max(cx - cw / 2, 0)), int(min(cx + cw / 2, width))
            y0, y1 = int(max(cy - chh / 2, 0)), int(min(cy + chh / 2, height))
            img[y0:y1, x0:x1] = fill
        else:
            # 45-degree rotated rectangle, evaluated on its bounding box only
            r = (cw + chh) / (2 * np.sqrt(2)) + 1
            x0, x1 = int(max(cx - r, 0)), int(min(cx + r + 1, width))
            y0, y1 = int(max(cy - r, 0)), int(min(cy + r + 1, height))
            if x1 <= x0 or y1 <= y0:
                continue
            sx = xx[:, x0:x1] - cx
            sy = yy[y0:y1, :] - cy
            u = (sx + sy) / np.sqrt(2)
            v = (sx - sy) / np.sqrt(2)
            m = (np.abs(u) <= cw / 2) & (np.abs(v) <= chh / 2)
            img[y0:y1, x0:x1][m] = fill
    # one 64x64 checker of 8-px squares, 0/255
    cs = min(64, width, height)
    ox = int(rng.integers(0, max(width - cs, 0) + 1))
    oy = int(rng.integers(0, max(height - cs, 0) + 1))
    cy_, cx_ = np.mgrid[0:cs, 0:cs]
    checker = (((cy_ // 8) + (cx_ // 8)) % 2 * 255).astype(np.float32)
    img[oy:oy + cs, ox:ox + cs] = checker[..., None]
    img = np.clip(img, 0, 255)
    if sixteen_bit:
        out = np.clip(img / 255.0 * 65535.0, 0, 65535).astype(np.uint16)
    else:
        out = np.rint(img).astype(np.uint8)
    if alpha:
        # smooth radial ramp, minus fully transparent discs covering ~10 % of
        # the area (disc radii 2 px .. 6 % of the short side)
        r = np.hypot((xx - width / 2) / max(width, 1), (yy - height / 2) / max(height, 1))
        a = np.clip(1.0 - r * 1.4, 0, 1)
        hole = np.zeros((height, width), bool)
        target = 0.10 * width * height
        covered = 0
        for _ in range(10000):
            if covered >= target:
                break
            hx, hy = rng.uniform(0, width), rng.uniform(0, height)
            rad = rng.uniform(2, max(3.0, 0.06 * min(width, height)))
            x0, x1 = int(max(hx - rad, 0)), int(min(hx + rad + 1, width))
            y0, y1 = int(max(hy - rad, 0)), int(min(hy + rad + 1, height))
            if x0 >= x1 or y0 >= y1:
                continue
            sub = (xx[:, x0:x1] - hx) ** 2 + (yy[y0:y1, :] - hy) ** 2 <= rad * rad
            view = hole[y0:y1, x0:x1]
            covered += int(np.count_nonzero(sub & ~view))
            view |= sub
        a[hole] = 0.0
        amax = 65535 if sixteen_bit else 255
        a_ch = (a * amax).astype(out.dtype)[..., None]
        out = np.concatenate([out, a_ch], axis=2)
    return np.ascontiguousarray(out)


def config1_image() -> np.ndarray:
    """512x512 RGB8, seed 1 (the plain CPU-runnable workload)."""
    return generate(512, 512, 1)


def config2_image(width: int = 3840, height: int = 2160) -> np.ndarray:
    """3840x2160 RGB8, seed 2: noise 4, 200 rectangles, 30 % 1/f^2 texture."""
    return generate(width, height, 2, noise_sigma=4.0, rectangles=200, texture_weight=0.3)


def config4_image(width: int = 1920, height: int = 1080) -> np.ndarray:
    """1920x1080 RGB8 from the 3840x2160 generator, seed 4 (the refinement
    workload: 240 x 135 blocks)."""
    return generate(width, height, 4, noise_sigma=4.0, rectangles=200, texture_weight=0.3)


def config5_image(size: int = 8192) -> np.ndarray:
    """size x size RGB 16-bit linear, seed 5: 50 % 1/f^2 texture."""
    return generate(size, size, 5, sixteen_bit=True, texture_weight=0.5)


def config3_batch(count: int = 256, seed0: int = 3000):
    """Log-uniform sizes 64x64..2048x1536; odd indices carry alpha."""
    out = []
    for i in range(count):
        rng = np.random.Generator(np.random.PCG64(seed0 + i))
        w = int(round(np.exp(rng.uniform(np.log(64), np.log(2048)))))
        h = int(round(np.exp(rng.uniform(np.log(64), np.log(1536)))))
        out.append(generate(w, h, seed0 + i, alpha=bool(i % 2)))
    return out
