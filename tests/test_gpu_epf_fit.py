"""The EPF fit operator (jxg_op_epf_fit) against its restatement
(oracle/epf_fit.py: choose and fit over oracle/epf.py and
oracle/luma_proxy.py), on the reference's own fit scene
(src/epf_filter.rs:880-900, without its additive layer) and noisy
reconstructions at several distances."""
import numpy as np
import pytest

import jixel_gb300 as J
from oracle import epf_fit as EF

pytestmark = pytest.mark.gpu
F = np.float32


@pytest.fixture(scope="module")
def ctx():
    c = J.FrontendContext(0)
    yield c
    c.close()


def additive_scene():
    w, h = 32, 24
    x, y = np.arange(w)[None, :], np.arange(h)[:, None]
    value = (F(0.2) + F(0.003) * ((x * 7 + y * 3) % 23).astype(F)).astype(F)
    recon = np.zeros((3, h, w), F)
    recon[1] = value + F(0.004) * ((x + y) % 3).astype(F)
    recon[2] = value
    sq = np.full(((w + 7) // 8) * ((h + 7) // 8), F(-1.0))
    return value, recon, sq


def noisy_scene(w, h, seed, noise):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    src = np.stack([F(0.01) * np.sin(xx / 5.0), F(0.3) + F(0.2) * np.sin(xx / 9.0 + yy / 7.0),
                    F(0.3) + F(0.1) * np.cos(yy / 6.0)]).astype(F)
    recon = (src + rng.normal(0, noise, src.shape)).astype(F)
    nb = ((w + 7) // 8) * ((h + 7) // 8)
    sq = (F(-0.2) - rng.uniform(0, 1.5, nb)).astype(F)
    return src[1], recon, sq


def check(ctx, source_y, recon, sq, distance, baseline):
    got, score = ctx.epf_fit(source_y, recon, sq, distance, baseline)
    want, want_score = EF.fit(source_y, recon, sq, distance, EF.Choice(*baseline))
    assert (got[0], got[2], got[3]) == (want.iters, want.pass0, want.sharpness), (got, want)
    if want.quant_mul is None:
        assert got[1] is None
    else:
        assert abs(got[1] - want.quant_mul) <= 1e-5 * want.quant_mul, (got, want)
    assert abs(score - float(want_score)) <= 1e-4 * float(want_score), (score, want_score)


def test_fit_on_the_reference_scene(ctx):
    source_y, recon, sq = additive_scene()
    check(ctx, source_y, recon, sq, 2.0, (2, None, None, 5))


@pytest.mark.parametrize("distance,noise,seed", [(1.0, 0.004, 1), (2.35, 0.01, 2), (5.0, 0.03, 3)])
def test_fit_on_noisy_reconstructions(ctx, distance, noise, seed):
    source_y, recon, sq = noisy_scene(72, 56, seed, noise)
    check(ctx, source_y, recon, sq, distance, (2, None, None, 7))


def test_fit_rejects_bad_arguments(ctx):
    source_y, recon, sq = additive_scene()
    with pytest.raises(J.EncodeError):
        ctx.epf_fit(source_y, recon, sq, 0.0)
    with pytest.raises(J.EncodeError):
        ctx.epf_fit(source_y, recon, sq, 1.0, (4, None, None, 7))
