"""Quant-field refinement: the forward model, its hand-written adjoint and the
optimiser, against an FP64 PyTorch restatement of the same model.

The library has no counterpart in the reference (which computes no
gradients); what can be pinned is (1) the model's levels at theta = 0 are the
front end's own levels, bit for bit; (2) its loss and its gradient match an
FP64 autograd model of the same straight-through quantiser and of the
decoder's EPF with its weights held (levels and weights frozen to the
kernel's, so both sides round alike); (3) that FP64 model's gradient is
the derivative of the frozen-offset surrogate, checked by central
differences; (4) Adam steps lower the true (rounded) loss; (5) a pass with a
caller's field equals the plain pass when the field is the adaptive one.
"""
import numpy as np
import pytest

import jixel_gb300 as J
from jixel_gb300 import synthetic

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

OPSIN_INVERSE = np.array([[11.031567, -9.866944, -0.16462299],
                          [-3.2541473, 4.4187703, -0.16462299],
                          [-3.6588514, 2.712923, 1.9459282]])
OPSIN_BIAS, NEG_BIAS_CBRT = 0.0037930734, -0.1559542
BIAS_ONE = np.array([1.0 - 0.05465007330715401, 1.0 - 0.07005449891748593, 1.0 - 0.049935103337343655])
C1, C2 = 1e-4, 9e-4
EPF_STAGES = {  # (dx, dy) directions and neighbours (direction, along), the decoder's order
    0: ([(1, 0), (2, 0), (0, 1), (0, 2), (1, 1), (-1, 1)],
        [(3, 0), (4, 0), (2, 0), (5, 0), (1, 0), (0, 0), (0, 1), (1, 1), (5, 1), (2, 1), (4, 1), (3, 1)], True),
    1: ([(1, 0), (0, 1)], [(1, 0), (0, 0), (0, 1), (1, 1)], True),
    2: ([(1, 0), (0, 1)], [(1, 0), (0, 0), (0, 1), (1, 1)], False),
}
EPF_INV_SIGMA_NUM, EPF_MIN_SIGMA = -1.1715729, -3.905243
PROXY_WEIGHTS = [109.4163228369586, 4.685925102200196, 2.491781270704224, 2.167275675983448,
                 4.55227651921194, 2.847714678987977]


def proxy_mirror(i, n):
    if 0 <= i < n:
        return i
    i %= 2 * n
    return i if i < n else 2 * n - i - 1


def proxy_half(t, bias):
    h2, w2 = t.shape[0] // 2, t.shape[1] // 2
    a = t[: 2 * h2, : 2 * w2]
    b = 0.01 if bias else 0.0
    t00, t01, t10, t11 = a[0::2, 0::2] + b, a[0::2, 1::2] + b, a[1::2, 0::2] + b, a[1::2, 1::2] + b
    return 0.25 * (((t00 + t10) + t01) + t11)


def proxy_box(t):
    """The reflected 5x5 box mean (direct sums)."""
    h, w = t.shape
    ys = torch.tensor([[proxy_mirror(y + d, h) for d in range(-2, 3)] for y in range(h)])
    xs = torch.tensor([[proxy_mirror(x + d, w) for d in range(-2, 3)] for x in range(w)])
    v = t[ys].sum(1) * 0.2          # (h, w)
    return v[:, xs].sum(2) * 0.2    # (h, w)


def proxy_level(ref, test):
    a, vr = proxy_box(ref), torch.clamp(proxy_box(ref * ref) - proxy_box(ref) ** 2, min=0.0)
    b, sq, cross = proxy_box(test), proxy_box(test * test), proxy_box(ref * test)
    var = torch.clamp(sq - b * b, min=0.0)
    cov = torch.where((vr == 0) | (var == 0), torch.zeros_like(var), cross - a * b)
    s = torch.clamp(1.0 - (1.0 - (a - b) ** 2) * (2.0 * cov + 0.0009) / (vr + var + 0.0009), min=0.0)
    return s.mean(), (s ** 4).mean() ** 0.25


def luma_proxy(src, y):
    """The reference's six-term luma proxy in FP64 (src/epf_proxy.rs:132-214)."""
    hs, hy = proxy_half(src, True), proxy_half(y, True)
    qs, qy = proxy_half(hs, False), proxy_half(hy, False)
    h_mean, h_fourth = proxy_level(hs, hy)
    q_mean, _ = proxy_level(qs, qy)
    a = torch.cat([(src[:, 1:] - src[:, :-1]).reshape(-1), (src[1:] - src[:-1]).reshape(-1)])
    b = torch.cat([(y[:, 1:] - y[:, :-1]).reshape(-1), (y[1:] - y[:-1]).reshape(-1)])
    n = a.numel()
    err = (b - a).abs().sum() / n
    exc = torch.clamp(b.abs() - a.abs(), min=0.0).sum() / n
    l4 = (torch.clamp(a.abs() - b.abs(), min=0.0) ** 4).sum() / n
    terms = [q_mean, h_mean, h_fourth, err, exc, l4 ** 0.25]
    return sum(w * t for w, t in zip(PROXY_WEIGHTS, terms))


def mirror(i, n):
    while i < 0 or i >= n:
        i = -i - 1 if i < 0 else 2 * n - 1 - i
    return i


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


def ultrafast(d):
    return J.EncodeConfig(distance=d, speed=J.Speed.ULTRA_FAST)


class Fp64Model:
    """The refinement model in FP64 with levels frozen at `q0` (the kernel's
    levels at theta0): quantiser inputs u become q0 + (u - u(theta0)), so the
    value at theta0 is the rounded model and the derivative is the
    straight-through one."""

    def __init__(self, ctx, res, w, h):
        m = ctx.refine_model()
        xb, yb = ctx._refine_blocks
        self.w, self.h, self.xb, self.yb = w, h, xb, yb
        d = torch.float64
        self.scale = m["scale"]
        self.qm = torch.tensor(m["qm_mul"], dtype=d)
        self.mat = torch.tensor(m["matrix"], dtype=d)
        self.inv = torch.tensor(m["inv_matrix"], dtype=d)
        self.coef = torch.tensor(m["coef"], dtype=d)
        self.M = torch.tensor(m["inverse"], dtype=d)
        self.dc = torch.tensor(m["dc"], dtype=d)  # (nb, 3) decoded DC
        self.epf = m["epf"]
        pad = 8  # mirrored coordinates for offsets up to +-8
        self.mx = torch.tensor([mirror(i, w) for i in range(-pad, w + pad)])
        self.my = torch.tensor([mirror(i, h) for i in range(-pad, h + pad)])
        self.pad = pad
        thr = m["thresholds"]
        z = np.zeros((3, 64))
        for i in range(64):  # the zero region's edge per coefficient
            t = thr[:, (2 if i >> 3 >= 4 else 0) + (1 if i & 7 >= 4 else 0)]
            z[:, i] = np.maximum(t, 0.5)
        self.zero_edge = torch.tensor(z, dtype=d)
        self.qf = torch.tensor(res.quant_field.reshape(-1).astype(np.float64))
        by, bx = np.divmod(np.arange(xb * yb), xb)
        tiles = (by >> 3, bx >> 3)
        self.xf = torch.tensor(res.ytox[tiles].astype(np.float64) / 84.0)
        self.bf = torch.tensor(1.0 + res.ytob[tiles].astype(np.float64) / 84.0)
        self.src_y = torch.tensor(res.xyb[1].astype(np.float64))
        self.weights = (1.0, 0.0)  # ssim, proxy
        self.src = [self._linear(torch.tensor(res.xyb.astype(np.float64)))]
        for _ in range(2):
            self.src.append(self._down(self.src[-1]))

    @staticmethod
    def _linear(xyb):
        x, y, b = xyb[0], xyb[1], xyb[2]
        t = torch.stack([y + x, y - x, b])
        m = (t - NEG_BIAS_CBRT) ** 3 - OPSIN_BIAS
        return torch.einsum("jk,khw->jhw", torch.tensor(OPSIN_INVERSE), m)

    @staticmethod
    def _down(p):
        h2, w2 = p.shape[1] // 2, p.shape[2] // 2
        q = p[:, : 2 * h2, : 2 * w2]
        return 0.25 * (q[:, 0::2, 0::2] + q[:, 0::2, 1::2] + q[:, 1::2, 0::2] + q[:, 1::2, 1::2])

    @staticmethod
    def _blur(p):
        k = torch.tensor([1.0, 4.0, 6.0, 4.0, 1.0], dtype=p.dtype) / 16.0
        c = p.shape[0]
        x = torch.nn.functional.conv2d(p[None], k.view(1, 1, 1, 5).repeat(c, 1, 1, 1), padding=(0, 2),
                                       groups=c)
        x = torch.nn.functional.conv2d(x, k.view(1, 1, 5, 1).repeat(c, 1, 1, 1), padding=(2, 0), groups=c)
        return x[0]

    def _ssim_loss(self, a, b):
        m1, m2 = self._blur(a), self._blur(b)
        s11, s22, s12 = self._blur(a * a), self._blur(b * b), self._blur(a * b)
        v1, v2, c12 = s11 - m1 * m1, s22 - m2 * m2, s12 - m1 * m2
        ssim = (2 * m1 * m2 + C1) * (2 * c12 + C2) / ((m1 * m1 + m2 * m2 + C1) * (v1 + v2 + C2))
        return (1.0 - ssim).mean()

    def _inputs(self, s, q0, offset):
        """The three quantiser inputs at s: Y, then X and B after CfL from the
        dequantised Y (at the frozen levels, or at q0 itself for offset None)."""
        uy = self.inv[1] * (s * self.qm[1])[:, None] * self.coef[:, 1]
        yst = q0[:, 1] if offset is None else uy + offset[1]
        yh = self._bias(1, q0[:, 1], yst) * self.mat[1] / s[:, None]
        u = {1: uy}
        for c, f in ((0, self.xf), (2, self.bf)):
            v = self.coef[:, c] - f[:, None] * yh
            u[c] = self.inv[c] * (s * self.qm[c])[:, None] * v
        return u, yh

    def _shift(self, img, ox, oy):
        """img at (x + ox, y + oy) through the mirrored borders."""
        ys = self.my[torch.arange(self.h) + oy + self.pad]
        xs = self.mx[torch.arange(self.w) + ox + self.pad]
        return img[:, ys][:, :, xs]

    def _epf_weights(self, img, theta):
        """One stage's weights at a fixed input: per stage (normalised
        neighbour weights, centre weight), computed from the values given
        (the decoder's Epf::apply); the caller holds them fixed."""
        e = self.epf
        q = self.qf * torch.exp(theta)
        sq = e["quant_scale"] * q * EPF_INV_SIGMA_NUM
        sigma = 1.0 / torch.clamp((e["quant_mul"] / sq) * e["lut"], max=-1e-4)
        sig = sigma.view(self.yb, self.xb).repeat_interleave(8, 0).repeat_interleave(8, 1)[: self.h, : self.w]
        yy, xx = torch.meshgrid(torch.arange(self.h), torch.arange(self.w), indexing="ij")
        border = ((yy % 8 == 0) | (yy % 8 == 7) | (xx % 8 == 0) | (xx % 8 == 7))
        cs = torch.tensor(e["channel_scale"], dtype=torch.float64)
        out = []
        for stage, sm in e["stages"]:
            dirs, neighbors, patch = EPF_STAGES[stage]
            inv = sig * torch.where(border, torch.tensor(sm * e["border"], dtype=torch.float64),
                                    torch.tensor(sm, dtype=torch.float64))

            def diff(sx, sy, dx, dy):
                a, b = self._shift(img, sx, sy), self._shift(img, sx + dx, sy + dy)
                return ((a - b).abs() * cs[:, None, None]).sum(0)

            ws = []
            for d, along in neighbors:
                dx, dy = dirs[d]
                sx, sy = (0, 0) if along else (-dx, -dy)
                if patch:
                    sad = sum(diff(sx + ax, sy + ay, dx, dy) for ax, ay in ((0, 0), (-1, 0), (1, 0), (0, -1), (0, 1)))
                else:
                    sad = diff(sx, sy, dx, dy)
                ws.append(torch.clamp(sad * inv + 1.0, min=0.0))
            wsum = 1.0 + sum(ws)
            filtered = sig >= EPF_MIN_SIGMA
            norm = [torch.where(filtered, wk / wsum, torch.zeros_like(wk)) for wk in ws]
            centre = torch.where(filtered, 1.0 / wsum, torch.ones_like(wsum))
            out.append((norm, centre))
            img = self._epf_apply(img, stage, (norm, centre))
        return out

    def _epf_apply(self, img, stage, weights):
        dirs, neighbors, _ = EPF_STAGES[stage]
        norm, centre = weights
        acc = img * centre
        for (d, along), wk in zip(neighbors, norm):
            dx, dy = dirs[d]
            acc = acc + wk * (self._shift(img, dx, dy) if along else self._shift(img, -dx, -dy))
        return acc

    def _decode(self, theta, q0, offset):
        """The decoded coefficients (nb, 3, 64) and the model bits at theta."""
        nz = q0 != 0
        s = self.scale * self.qf * torch.exp(theta)
        u, yh = self._inputs(s, q0, offset)
        chat = []
        bits = torch.zeros((), dtype=torch.float64)
        for c in range(3):
            ust = u[c] + offset[c]
            if c == 1:
                hat = yh
            else:
                f = self.xf if c == 0 else self.bf
                hat = self._bias(c, q0[:, c], ust) * self.mat[c] / (s * self.qm[c])[:, None] + f[:, None] * yh
            hat = torch.cat([self.dc[:, c:c + 1], hat[:, 1:]], dim=1)  # the DC slot: decoded DC
            chat.append(hat)
            a = torch.where(nz[:, c], ust.abs(), torch.zeros_like(ust))
            zero = 2.6 * (u[c].abs() / self.zero_edge[c]) ** 4  # a zero level: its unrounded input
            term = torch.where(nz[:, c], 1.6 + torch.log2(1.0 + a), zero)
            bits = bits + term[:, 1:].sum()
        return torch.stack(chat, dim=1), bits

    def loss(self, theta, theta0, q0, lam):
        """(loss, distortion, bits) at theta with levels (and the EPF's
        weights) frozen at theta0."""
        q0 = torch.tensor(q0, dtype=torch.float64)  # (nb, 3, 64)
        with torch.no_grad():
            u0, _ = self._inputs(self.scale * self.qf * torch.exp(theta0), q0, None)
        offset = {c: q0[:, c] - u0[c] for c in range(3)}
        chat, bits = self._decode(theta, q0, offset)
        img = self.planes(chat)
        if self.epf["stages"]:
            with torch.no_grad():
                frozen = self._epf_weights(self.planes(self._decode(theta0, q0, offset)[0]), theta0)
            for (stage, _), wts in zip(self.epf["stages"], frozen):
                img = self._epf_apply(img, stage, wts)
        self.decoded = img
        ws, wp = self.weights
        dist = torch.zeros((), dtype=torch.float64)
        if ws > 0:
            rec = [self._linear(img)]
            for _ in range(2):
                rec.append(self._down(rec[-1]))
            dist = dist + ws * sum(self._ssim_loss(a, b) for a, b in zip(self.src, rec)) / 3.0
        if wp > 0:
            dist = dist + wp * luma_proxy(self.src_y, img[1])
        return dist + lam * bits / (self.w * self.h), dist, bits

    def planes(self, chat):
        """The w x h XYB planes of (nb, 3, 64) coefficients through M."""
        pix = chat @ self.M.T  # (nb, 3, 64), pixel p = row * 8 + col
        planes = pix.view(self.yb, self.xb, 3, 8, 8).permute(2, 0, 3, 1, 4).reshape(3, self.yb * 8, self.xb * 8)
        return planes[:, : self.h, : self.w]

    @staticmethod
    def _bias(c, q, ust):
        one = torch.sign(q) * BIAS_ONE[c]
        safe = torch.where(q.abs() >= 2, ust, torch.ones_like(ust))
        big = safe - 0.145 / safe
        return torch.where(q == 0, torch.zeros_like(ust), torch.where(q.abs() == 1, one, big))


def begin(ctx, w, h, seed, d=1.0):
    img = synthetic.generate(w, h, seed)
    res = ctx.frontend(img, ultrafast(d), xyb=True)
    xb, yb = ctx.refine_begin()
    assert (xb, yb) == ((w + 7) // 8, (h + 7) // 8)
    return img, res


@pytest.mark.parametrize("w,h,seed,d", [(70, 54, 11, 1.0), (256, 192, 12, 2.0), (33, 17, 13, 0.5)])
def test_levels_at_zero_are_the_front_ends(ctx, w, h, seed, d):
    img, res = begin(ctx, w, h, seed, d)
    nb = res.quant_field.size
    theta = torch.zeros(nb, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the library runs on its own stream
    _, lv = ctx.refine_eval(0.0, theta.data_ptr(), levels=True)
    got = lv.reshape(res.coefficients.shape)  # both in raw order
    want = res.coefficients.copy()
    got[..., 0] = want[..., 0] = 0  # the DC slot is not modelled
    bad = np.argwhere(got != want)
    assert bad.size == 0, (f"{len(bad)} levels differ (per channel {np.bincount(bad[:, 2], minlength=3)}, "
                           f"{np.count_nonzero(want)} non-zero), first {bad[:4].tolist()}, "
                           f"got {got[tuple(bad[0][:3])][:8]} want {want[tuple(bad[0][:3])][:8]}")


def test_decoded_frame_is_the_models(ctx):
    # jxg_refine_decoded: the FP64 model's decoded planes, within FP32, at
    # theta = 0 and at a random theta; and close to the source at d 1
    img, res = begin(ctx, 70, 54, 17, 1.0)
    nb = res.quant_field.size
    model = Fp64Model(ctx, res, 70, 54)
    for spread in (0.0, 0.3):
        th = np.random.default_rng(17).normal(0.0, spread, nb).astype(np.float32)
        ctx.refine_theta(th.reshape(res.quant_field.shape))
        dec = ctx.refine_decoded()
        _, lv = ctx.refine_eval(0.0, levels=True)
        t64 = torch.tensor(th.astype(np.float64))
        model.loss(t64, t64, lv, 0.0)
        want = model.decoded.numpy()
        assert dec.shape == (3, 54, 70)
        assert np.abs(dec - want).max() <= 2e-5 * max(1.0, np.abs(want).max()), np.abs(dec - want).max()
    ctx.refine_theta(np.zeros(res.quant_field.shape, np.float32))
    err = ctx.refine_decoded() - res.xyb
    assert np.sqrt(np.mean(err[1] ** 2)) < 0.02


def test_decoded_dc_is_the_dequantised_dc_levels(ctx):
    img, res = begin(ctx, 96, 72, 16)
    m = ctx.refine_model()
    dc = m["dc"].reshape(res.quant_field.shape + (3,))
    q = res.quant_dc.astype(np.float64)  # (3, yb, xb): X, Y, B
    # the DC step per channel from the Y plane's levels: decoded / level
    nz = q[1] != 0
    step_y = dc[..., 1][nz] / q[1][nz]
    assert np.allclose(step_y, step_y[0], rtol=1e-6)
    # within half a step of the source block means (the rounding of the levels)
    src = m["coef"][:, :, 0].reshape(dc.shape)
    assert np.all(np.abs(src[..., 1] - dc[..., 1]) <= 0.5 * abs(step_y[0]) * (1 + 1e-5))
    # X and B: their own levels plus the luma levels' chroma-from-luma share
    for c in (0, 2):
        nzc = q[c] != 0
        if nzc.any():
            step = (dc[..., c] * 1.0)[nzc & (q[1] == 0)] / q[c][nzc & (q[1] == 0)]
            if step.size:
                assert np.allclose(step, step[0], rtol=1e-6)


@pytest.mark.parametrize("w,h,seed", [(70, 54, 14), (256, 192, 15)])
def test_inverse_reproduces_the_source(ctx, w, h, seed):
    # the source coefficients through the model's inverse transform give the
    # pass's XYB planes back: coefficient layout, transform and crop agree
    img, res = begin(ctx, w, h, seed)
    model = Fp64Model(ctx, res, w, h)
    back = model.planes(model.coef).numpy()
    err = np.abs(back - res.xyb).max()
    assert err <= 1e-5 * max(1.0, np.abs(res.xyb).max()), err


def fp64_check(ctx, w, h, seed, lam, spread, d=1.0, weights=(1.0, 0.0)):
    img, res = begin(ctx, w, h, seed, d)
    ctx.refine_weights(*weights)
    nb = res.quant_field.size
    rng = np.random.default_rng(seed)
    th = rng.normal(0.0, spread, nb).astype(np.float32)
    theta = torch.tensor(th, device="cuda")
    grad = torch.zeros(nb, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    (loss, dist, bits), lv = ctx.refine_eval(lam, theta.data_ptr(), grad.data_ptr(), levels=True)
    g_gpu = grad.cpu().numpy().astype(np.float64)
    model = Fp64Model(ctx, res, w, h)
    model.weights = weights
    t64 = torch.tensor(th.astype(np.float64), requires_grad=True)
    l64, d64, b64 = model.loss(t64, t64.detach().clone(), lv, lam)
    l64.backward()
    g_ref = t64.grad.numpy()
    # FP32 against FP64: the rate within 1e-4 relative; the distortion within
    # 5e-4 relative plus 2e-6 (SSIM's FP32 variances cancel where the
    # decoded image is close to the source, as at d 0.5), 2e-3 with the luma
    # proxy (its box moments follow the reference's FP32 running sums, whose
    # variances cancel the same way)
    rel = 2e-3 if weights[1] > 0 else 5e-4
    assert abs(bits - b64.item()) <= 1e-4 * max(b64.item(), 1.0), (bits, b64.item())
    assert abs(dist - d64.item()) <= rel * d64.item() + 2e-6, (dist, d64.item())
    assert abs(loss - l64.item()) <= rel * l64.item() + 2e-6, (loss, l64.item())
    # the adjoint: per block, within 1e-3 of the largest gradient (1e-2 with
    # the luma proxy: its pool's partials are taken at the FP32 running-sum
    # moments, whose variances carry the cancellation above)
    tol = (1e-2 if weights[1] > 0 else 1e-3) * np.abs(g_ref).max()
    err = np.abs(g_gpu - g_ref)
    assert err.max() <= tol, (err.max(), tol, int(err.argmax()))
    ctx.refine_weights()
    return model, t64.detach(), lv, g_ref, lam


@pytest.mark.parametrize("w,h,seed,lam,spread,d", [(70, 54, 21, 0.002, 0.3, 1.0), (200, 136, 22, 0.01, 0.1, 1.0),
                                                    (72, 64, 23, 0.002, 0.2, 3.0), (45, 37, 24, 0.005, 0.2, 0.5)])
def test_loss_and_gradient_match_fp64(ctx, w, h, seed, lam, spread, d):
    # d 1.0: one EPF stage; d 3.0: three (pass-0 scale signalled); d 0.5: none
    fp64_check(ctx, w, h, seed, lam, spread, d)
    stages = len(ctx.refine_model()["epf"]["stages"])
    assert stages == {1.0: 1, 3.0: 3, 0.5: 0}[d]


@pytest.mark.parametrize("d,weights", [(1.0, (0.0, 1.0)), (3.0, (0.5, 0.2))])
def test_luma_proxy_loss_and_gradient_match_fp64(ctx, d, weights):
    # the proxy alone, and mixed with 1 - SSIM, through the EPF
    fp64_check(ctx, 80, 60, 25, 0.002, 0.2, d, weights)


def test_luma_proxy_matches_the_oracle(ctx):
    # the device proxy of the decoded Y plane against the restated reference
    # (float32, the reference's sum order) of the FP64 model's decoded plane:
    # within 2e-3 relative (the device decodes in FP32, which the moments'
    # variance cancellation amplifies, and pools in parallel)
    from oracle import luma_proxy as LP
    img, res = begin(ctx, 96, 72, 26, 1.0)
    nb = res.quant_field.size
    th = np.random.default_rng(26).normal(0.0, 0.2, nb).astype(np.float32)
    theta = torch.tensor(th, device="cuda")
    torch.cuda.synchronize()
    ctx.refine_weights(0.0, 1.0)
    try:
        (loss, dist, _), lv = ctx.refine_eval(0.0, theta.data_ptr(), levels=True)
    finally:
        ctx.refine_weights()
    model = Fp64Model(ctx, res, 96, 72)
    model.weights = (0.0, 1.0)
    t64 = torch.tensor(th.astype(np.float64))
    model.loss(t64, t64, lv, 0.0)
    y = model.decoded[1].numpy().astype(np.float32)
    want, _ = LP.LumaProxy(res.xyb[1].astype(np.float32)).compare(y)
    assert abs(dist - float(want)) <= 2e-3 * float(want), (dist, float(want))
    assert loss == dist


def test_fp64_gradient_is_the_surrogates_derivative(ctx):
    # central differences of the frozen-offset surrogate on 64 random blocks
    model, th, lv, g_ref, lam = fp64_check(ctx, 72, 68, 31, 0.002, 0.3, 3.0)  # three EPF stages
    step = 1e-5
    for b in np.random.default_rng(44).choice(th.numel(), 64, replace=False):
        e = torch.zeros_like(th)
        e[b] = step
        hi = model.loss(th + e, th, lv, lam)[0].item()
        lo = model.loss(th - e, th, lv, lam)[0].item()
        fd = (hi - lo) / (2 * step)
        assert abs(fd - g_ref[b]) <= 1e-6 + 1e-4 * abs(g_ref[b]), (b, fd, g_ref[b])


def test_adam_steps_lower_the_rounded_loss(ctx):
    img, res = begin(ctx, 256, 192, 41, 1.0)
    field, history, final = ctx.refine(steps=8, rate_lambda=0.002, learning_rate=0.05)
    assert final[0] < history[0][0], (history[0], final)
    losses = [h[0] for h in history] + [final[0]]
    assert all(b <= a for a, b in zip(losses, losses[1:])), losses  # the monotone driver
    theta = ctx.refine_theta()
    q = res.quant_field.astype(np.float64)
    v = q * np.exp(theta.astype(np.float64))
    assert np.all(v >= 1.0 - 1e-3) and np.all(v <= 255.0 + 1e-3)
    want = np.clip(np.rint(res.quant_field.astype(np.float32) * np.exp(theta)), 1, 255)
    assert np.abs(field.astype(np.int32) - want.astype(np.int32)).max() <= 1  # expf vs numpy exp
    # setting theta back to zero restores the starting loss
    ctx.refine_theta(np.zeros_like(theta))
    again, _ = ctx.refine_eval(0.002)
    assert again == history[0]


def test_pass_with_the_adaptive_field_is_the_plain_pass(ctx):
    img = synthetic.generate(300, 200, 51)
    plain = ctx.frontend(img, ultrafast(1.0))
    got = ctx.frontend_with_field(img, ultrafast(1.0), plain.quant_field)
    for k in ("quant_field", "ytox", "ytob", "quant_dc", "coefficients", "num_nzeros", "tokens",
              "group_offsets", "histograms"):
        assert np.array_equal(getattr(got, k), getattr(plain, k)), k
    assert got.params == plain.params


def test_pass_with_a_refined_field(ctx):
    img, res = begin(ctx, 256, 192, 61, 1.0)
    field, _, _ = ctx.refine(steps=4)
    got = ctx.frontend_with_field(img, ultrafast(1.0), field)
    assert np.array_equal(got.quant_field, field)
    # the refined field was taken from a copy: refinement state survives the pass
    again = ctx.refine_field()
    assert np.array_equal(again, field)


def test_ac_bits_estimate_counts_symbols_and_raw_bits(ctx):
    img = synthetic.generate(128, 96, 81)
    res = ctx.frontend(img, ultrafast(1.0))
    h = res.histograms.astype(np.float64)
    ent = 0.0
    for row in h[h.sum(axis=1) > 0]:
        p = row[row > 0] / row.sum()
        ent -= float((row[row > 0] * np.log2(p)).sum())
    raw = sum(int(np.floor(np.log2(v))) - 2 for v in res.tokens[:, 1] if v >= 16)
    assert abs(J.ac_bits_estimate(res) - (ent + raw)) <= 1e-6 * (ent + raw)
    assert res.histograms.sum() == len(res.tokens)


def test_encode_frontend_with_refinement():
    # the one-shot path: a refined field, then the frame coded with it
    img = synthetic.generate(160, 120, 91)
    cfg = ultrafast(1.0)
    plain = J.encode_frontend(img, cfg)
    refined = J.encode_frontend(img, cfg, refine_steps=4)
    assert refined.quant_field.shape == plain.quant_field.shape
    assert not np.array_equal(refined.quant_field, plain.quant_field)
    assert refined.params["num_tokens"] > 0
    with pytest.raises(J.EncodeError):
        J.encode_frontend(img, J.EncodeConfig(distance=3.0, speed=J.Speed.FASTEST), refine_steps=2)


def test_refinement_errors(ctx):
    img = synthetic.generate(64, 64, 71)
    with pytest.raises(J.EncodeError):
        ctx.frontend_with_field(img, J.EncodeConfig(distance=2.0, speed=J.Speed.FASTEST),
                                np.ones((8, 8), np.uint8))
    with pytest.raises(J.EncodeError):
        ctx.frontend_with_field(img, ultrafast(1.0), np.ones((4, 4), np.uint8))
    fresh = J.FrontendContext(0)
    try:
        with pytest.raises(J.EncodeError):
            fresh.refine_begin()
        ctx.frontend(img, J.EncodeConfig(distance=3.0, speed=J.Speed.FASTEST))
        with pytest.raises(J.EncodeError):
            ctx.refine_begin()  # a searched frame is not all DCT8
    finally:
        fresh.close()
