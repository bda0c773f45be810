"""CPU restatement of the reference's six-term luma proxy (test infrastructure).

The reference scores a decoded XYB Y plane against the source's with
`LumaProxy` (src/epf_proxy.rs:132-214): structure terms at half and quarter
resolution over reflected 5x5 box moments (src/epf_proxy/box_filter.rs:84-240)
and adjacent-gradient terms at full resolution (src/epf_proxy.rs:216-247),
weighted by six frozen weights.  This module restates the scalar path in
numpy float32 with the reference's operation order: the running-sum box
filter, the pooled sums in raster order (a sequential float32 sum, which
np.cumsum computes), and the same expression trees.  Only the tests use it,
as the checker of the CUDA proxy.
"""
import numpy as np

F = np.float32
# src/epf_proxy.rs:186-193
WEIGHTS = np.array([109.4163228369586, 4.685925102200196, 2.491781270704224, 2.167275675983448,
                    4.55227651921194, 2.847714678987977], dtype=np.float32)


def mirror(i: int, n: int) -> int:
    """src/epf_proxy.rs:17-28 (one reflection with the edge repeated)."""
    if 0 <= i < n:
        return i
    i = i % (2 * n)
    return i if i < n else 2 * n - i - 1


def half(src: np.ndarray, bias: bool) -> np.ndarray:
    """`half` / `half_y` (src/epf_proxy/row_kernels.rs:60-71): 2x2 means,
    +0.01 on each tap for the luma pyramid's first level."""
    h, w = src.shape
    a = src[: 2 * (h // 2), : 2 * (w // 2)].astype(F)
    t00, t01 = a[0::2, 0::2], a[0::2, 1::2]
    t10, t11 = a[1::2, 0::2], a[1::2, 1::2]
    if bias:
        b = F(0.01)
        t00, t01, t10, t11 = t00 + b, t01 + b, t10 + b, t11 + b
    return (F(0.25) * (((t00 + t10) + t01) + t11)).astype(F)


def _sequential(values: np.ndarray) -> F:
    """The float32 sum of `values` in order, from 0."""
    v = np.ascontiguousarray(values, dtype=F).ravel()
    return F(0.0) if v.size == 0 else np.cumsum(v, dtype=F)[-1]


def box_moments(test: np.ndarray, ref: np.ndarray | None = None):
    """Reflected 5x5 box means of test, test^2 and (with `ref`) ref * test:
    the vertical running sums of `Scratch::run` (box_filter.rs:84-171,
    accumulate / step :191-226) then the horizontal one (`horizontal_scalar`,
    :228-240), each scaled by 0.2."""
    h, w = test.shape
    t = test.astype(F)
    r = ref.astype(F) if ref is not None else None
    rows = lambda y: mirror(y, h)  # noqa: E731
    count = 3 if r is not None else 2
    sums = [np.full(w, F(-0.0), F) for _ in range(count)]
    for y in range(-2, 3):
        v = t[rows(y)]
        sums[0] = sums[0] + v
        sums[1] = sums[1] + v * v
        if r is not None:
            sums[2] = sums[2] + r[rows(y)] * v
    vert = [np.zeros((h, w), F) for _ in range(count)]
    for y in range(h):
        for c in range(count):
            vert[c][y] = sums[c] * F(0.2)
        if y + 1 < h:
            a, b = t[rows(y + 3)], t[rows(y - 2)]
            sums[0] = sums[0] + (a - b)
            sums[1] = sums[1] + (a * a - b * b)
            if r is not None:
                sums[2] = sums[2] + (r[rows(y + 3)] * a - r[rows(y - 2)] * b)
    out = []
    cols = lambda x: mirror(x, w)  # noqa: E731
    for c in range(count):
        src = vert[c]
        s = np.zeros(h, F)
        for x in range(-2, 3):
            s = s + src[:, cols(x)]
        dst = np.zeros((h, w), F)
        for x in range(w):
            dst[:, x] = s * F(0.2)
            if x + 1 < w:
                s = s + (src[:, cols(x + 3)] - src[:, cols(x - 2)])
        out.append(dst)
    return out


def original_box5(src: np.ndarray) -> np.ndarray:
    """The reference's independent full-plane box filter (box_filter.rs:466-490)."""
    h, w = src.shape
    s_ = src.astype(F)
    tmp = np.zeros((h, w), F)
    sum_ = np.zeros(w, F)
    for y in range(-2, 3):
        sum_ = sum_ + s_[mirror(y, h)]
    for y in range(h):
        tmp[y] = sum_ * F(0.2)
        sum_ = sum_ + (s_[mirror(y + 3, h)] - s_[mirror(y - 2, h)])
    dst = np.zeros((h, w), F)
    sum_ = np.zeros(h, F)
    for x in range(-2, 3):
        sum_ = sum_ + tmp[:, mirror(x, w)]
    for x in range(w):
        dst[:, x] = sum_ * F(0.2)
        sum_ = sum_ + (tmp[:, mirror(x + 3, w)] - tmp[:, mirror(x - 2, w)])
    return dst


class Scale:
    """A pyramid level of the source (src/epf_proxy.rs:62-130)."""

    def __init__(self, values: np.ndarray):
        self.values = values.astype(F)
        mean, square = box_moments(self.values)
        self.mean = mean
        self.variance = np.maximum(square - mean * mean, F(0.0))  # row_kernels.rs:81-85

    def compare(self, test: np.ndarray):
        """[mean s, (mean s^4)^(1/4)] of the per-pixel structure loss
        (`pool`, row_kernels.rs:86-103)."""
        mean, square, cross = box_moments(test, self.values)
        a, b = self.mean, mean
        var = np.maximum(square - b * b, F(0.0))
        cov = np.where((self.variance == 0) | (var == 0), F(0.0), cross - a * b).astype(F)
        d = a - b
        s = np.maximum(F(1.0) - (F(1.0) - d * d) * (F(2.0) * cov + F(0.0009)) /
                       (self.variance + var + F(0.0009)), F(0.0)).astype(F)
        n = F(test.size)
        total = _sequential(s)
        fourth = _sequential(((s * s) * s) * s)
        return [F(total / n), F(np.sqrt(np.sqrt(F(fourth / n))))]


def gradients(source: np.ndarray, test: np.ndarray):
    """Error, excess and fourth-power pools of the horizontal, then the
    vertical neighbour differences (src/epf_proxy.rs:216-247,
    row_kernels.rs:104-115)."""
    s, t = source.astype(F), test.astype(F)
    ah, bh = s[:, 1:] - s[:, :-1], t[:, 1:] - t[:, :-1]
    av, bv = s[1:, :] - s[:-1, :], t[1:, :] - t[:-1, :]
    a = np.concatenate([ah.ravel(), av.ravel()])
    b = np.concatenate([bh.ravel(), bv.ravel()])
    err = np.abs(b - a)
    exc = np.maximum(np.abs(b) - np.abs(a), F(0.0))
    loss = np.maximum(np.abs(a) - np.abs(b), F(0.0))
    return [_sequential(err), _sequential(exc), _sequential(((loss * loss) * loss) * loss)]


class LumaProxy:
    """`LumaProxy::new` / `compare` (src/epf_proxy.rs:148-214)."""

    def __init__(self, y: np.ndarray):
        h, w = y.shape
        assert w >= 4 and h >= 4
        self.source = y.astype(F)
        hy = half(self.source, True)
        self.half = Scale(hy)
        self.quarter = Scale(half(hy, False))

    def compare(self, y: np.ndarray):
        h, w = y.shape
        hy = half(y, True)
        hs = self.half.compare(hy)
        qs = self.quarter.compare(half(hy, False))
        error, excess, loss4 = gradients(self.source, y)
        n = F(h * (w - 1) + (h - 1) * w)
        terms = np.array([qs[0], hs[0], hs[1], error / n, excess / n,
                          np.sqrt(np.sqrt(F(loss4 / n)))], dtype=F)
        score = F(0.0)
        for v, wt in zip(terms, WEIGHTS):
            score = F(score + F(v * wt))
        return score, terms
