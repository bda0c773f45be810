"""CPU restatement of the decoder's edge-preserving filter (test infrastructure).

Follows the reference's own coordinate oracle for `Epf::apply`
(src/epf_filter/tests.rs:33-127, `reference_stage` / `reference`): per pixel
the block's inverse sigma (1 / min(quant_mul / sigma_quant * sharpness / 7,
-1e-4)), the border SAD multiplier on block edges, patch or single-pixel
SADs of channel-weighted absolute differences over mirrored coordinates,
weights max(sad * inv + 1, 0) (zero for unfiltered blocks) and the weighted
mean, stage by stage (src/epf_filter.rs:213-263, :320-350).  numpy float32
with the reference's operation order: products and sums round separately.
Only the tests use it, as the checker of the CUDA EPF.
"""
import numpy as np

F = np.float32
SAD_MUL = F(1.65)
MIN_SIGMA = F(-3.905243)
# (dx, dy) directions and neighbours (direction, along), src/epf_filter.rs:219-263
STAGES = {
    0: ([(1, 0), (2, 0), (0, 1), (0, 2), (1, 1), (-1, 1)],
        [(3, 0), (4, 0), (2, 0), (5, 0), (1, 0), (0, 0), (0, 1), (1, 1), (5, 1), (2, 1), (4, 1), (3, 1)], True),
    1: ([(1, 0), (0, 1)], [(1, 0), (0, 0), (0, 1), (1, 1)], True),
    2: ([(1, 0), (0, 1)], [(1, 0), (0, 0), (0, 1), (1, 1)], False),
}


def mirror(i: int, n: int) -> int:
    """src/epf_filter.rs:150-160."""
    while i < 0 or i >= n:
        i = -i - 1 if i < 0 else 2 * n - 1 - i
    return i


def f16(v: float) -> F:
    """A LoopFilter field read back through F16."""
    return F(np.float16(F(v)))


def _stage(img: np.ndarray, sigma_quant: np.ndarray, quant_mul, sharpness, stage, sm, border_mul, cs):
    _, h, w = img.shape
    xb = (w + 7) // 8
    yy, xx = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    quant = sigma_quant.reshape(-1)[(yy // 8) * xb + xx // 8].astype(F)
    with np.errstate(divide="ignore", invalid="ignore"):
        m = (F(quant_mul) / quant) * (F(sharpness) / F(7.0))
        m = np.where(np.isnan(m), F(-1e-4), np.minimum(m, F(-1e-4))).astype(F)
        s = (F(1.0) / m).astype(F)
    keep = (s >= MIN_SIGMA).astype(F)
    border = (yy % 8 == 0) | (yy % 8 == 7) | (xx % 8 == 0) | (xx % 8 == 7)
    smb = np.where(border, F(sm) * F(border_mul), F(sm)).astype(F)
    inv = np.where(s >= MIN_SIGMA, s * smb, F(0.0)).astype(F)
    mx = {d: np.array([mirror(x + d, w) for x in range(w)]) for d in range(-4, 5)}
    my = {d: np.array([mirror(y + d, h) for y in range(h)]) for d in range(-4, 5)}

    def sample(c, ox, oy):  # the plane c at (x + ox, y + oy), mirrored
        return img[c][my[oy]][:, mx[ox]]

    def diff(ox, oy, dx, dy):  # difference(x + ox, y + oy, dx, dy)
        r = F(0.0)
        for c in range(3):
            r = (r + np.abs(sample(c, ox, oy) - sample(c, ox + dx, oy + dy)) * F(cs[c])).astype(F)
        return r

    dirs, neighbors, patch = STAGES[stage]
    total = np.ones((h, w), F)
    acc = [img[c].astype(F).copy() for c in range(3)]
    for d, along in neighbors:
        dx, dy = dirs[d]
        sx, sy = (0, 0) if along else (-dx, -dy)
        if patch:
            sad = ((diff(sx, sy, dx, dy) + (diff(sx - 1, sy, dx, dy) + diff(sx + 1, sy, dx, dy))) +
                   (diff(sx, sy - 1, dx, dy) + diff(sx, sy + 1, dx, dy))).astype(F)
        else:
            sad = diff(sx, sy, dx, dy)
        weight = (np.maximum(sad * inv + F(1.0), F(0.0)) * keep).astype(F)
        total = (total + weight).astype(F)
        nx, ny = (dx, dy) if along else (sx, sy)
        for c in range(3):
            acc[c] = (acc[c] + weight * sample(c, nx, ny)).astype(F)
    inv_sum = (F(1.0) / total).astype(F)
    return np.stack([(a * inv_sum).astype(F) for a in acc])


def epf(img, sigma_quant, iters, quant_mul, pass0, pass2, border_mul, channel_scale, sharpness):
    """`reference` (src/epf_filter/tests.rs:101-127): the stages in order."""
    out = np.asarray(img, F).copy()
    if iters == 0 or sharpness == 0:
        return out
    if iters >= 3:
        out = _stage(out, sigma_quant, quant_mul, sharpness, 0, SAD_MUL * F(pass0), border_mul, channel_scale)
    out = _stage(out, sigma_quant, quant_mul, sharpness, 1, SAD_MUL, border_mul, channel_scale)
    if iters >= 2:
        out = _stage(out, sigma_quant, quant_mul, sharpness, 2, SAD_MUL * F(pass2), border_mul, channel_scale)
    return out
