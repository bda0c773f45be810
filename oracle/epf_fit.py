"""CPU restatement of the encoder's EPF fit (test infrastructure).

`fit` (src/epf_filter.rs:807-873) renders candidate loop-filter settings
over a reconstruction with `Epf::apply` and ranks them by the luma proxy of
the filtered Y plane against the source's; `choose` (:599-671) picks the
candidates: the baseline, no filtering, four shape pilots at the centre
strength 2 / distance, the best pilot's two endpoints and the vertex of a
log-quadratic through them.  float32 arithmetic as the reference's.  Only
the tests use it, as the checker of the device fit.
"""
from dataclasses import dataclass

import numpy as np

from . import epf as E
from . import luma_proxy as LP

F = np.float32


@dataclass(frozen=True)
class Choice:
    """`Choice` (src/epf_filter.rs:577-594)."""
    iters: int
    quant_mul: float | None
    pass0: float | None
    sharpness: int

    @staticmethod
    def candidate(iters, strength, pass0):
        return Choice(iters, float(F(F(0.46) * F(strength))), pass0, 7)


def loop_filter(choice: Choice):
    """LoopFilter::new(iters, pass0, quant_mul, None) (src/epf_filter.rs:56-85):
    (quant_mul, pass0, pass2, border) with a signalled bundle read back
    through F16."""
    s = choice.pass0 if choice.pass0 is not None else (0.9 if choice.quant_mul is not None else None)
    if s is None:
        return F(0.46), F(0.9), F(6.5), F(2.0 / 3.0)
    q = choice.quant_mul if choice.quant_mul is not None else 0.46
    return E.f16(q), E.f16(s), E.f16(6.5), E.f16(2.0 / 3.0)


def choose(distance, baseline: Choice, score):
    """`choose` (src/epf_filter.rs:599-671)."""
    rows = []

    def trial(choice):
        for r in rows:
            if r[0] == choice:
                return r
        loss = F(score(choice))
        result = (choice, loss if np.isfinite(loss) else F(np.inf))
        rows.append(result)
        return result

    trial(baseline)
    trial(Choice(0, None, None, baseline.sharpness))
    d = F(distance)
    center = F(min(max(F(2.0) / d, F(0.0625)), F(4.0)))
    pilots = [trial(Choice.candidate(it, center, p0)) for it, p0 in ((1, None), (2, None), (3, 0.9), (3, 3.6))]
    pilot, middle = min(pilots, key=lambda r: r[1])  # the first of equal minima
    lo = F(max(center / F(2.0), F(0.0625)))
    hi = F(min(center * F(2.0), F(4.0)))
    low = trial(Choice.candidate(pilot.iters, lo, pilot.pass0))[1]
    high = trial(Choice.candidate(pilot.iters, hi, pilot.pass0))[1]
    if lo < center < hi:
        x0, x1, x2 = np.log2(lo), np.log2(center), np.log2(hi)
        with np.errstate(invalid="ignore"):  # infinite scores give NaN, as in f32
            a = F((F(middle - low) / F(x1 - x0) - F(high - middle) / F(x2 - x1)) / F(x0 - x2))
            b = F(F(middle - low) / F(x1 - x0) - F(a * F(x0 + x1)))
        if a > F(1e-12):
            v = F(min(max(F(-b / F(F(2.0) * a)), x0), x2))
            trial(Choice.candidate(pilot.iters, F(np.power(F(2.0), v)), pilot.pass0))
    return min(rows, key=lambda r: r[1])[0]


def fit(source_y, recon, sigma_quant, distance, baseline: Choice, channel_scale=(40.0, 5.0, 3.5)):
    """`fit` without overlay layers: (choice, its score)."""
    proxy = LP.LumaProxy(np.asarray(source_y, F))
    scores = {}

    def score(choice):
        q, p0, p2, border = loop_filter(choice)
        out = E.epf(recon, sigma_quant, choice.iters, q, p0, p2, border, channel_scale, choice.sharpness)
        s = proxy.compare(out[1])[0]
        scores[choice] = s
        return s

    best = choose(distance, baseline, score)
    return best, scores[best]
