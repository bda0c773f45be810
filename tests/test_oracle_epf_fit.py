"""The EPF fit's candidate search (oracle/epf_fit.py) against the
reference's own `choose` test (src/epf_filter.rs:1159-1173)."""
import numpy as np

from oracle import epf_fit as EF


def test_baseline_survives_ties_and_nonfinite_candidates():
    baseline = EF.Choice(2, None, None, 5)
    assert EF.choose(24.0, baseline, lambda c: 1.0) == baseline
    assert EF.choose(1.0, baseline, lambda c: 1.0 if c == baseline else float("nan")) == baseline


def test_search_visits_the_pilots_and_the_vertex():
    seen = []

    def score(c):
        seen.append(c)
        # a bowl in log strength, lowest for the two-stage pilot
        s = (c.quant_mul or 0.46) / 0.46
        return (np.log2(s) - 0.3) ** 2 + (0.0 if c.iters == 2 else 0.5)

    best = EF.choose(1.0, EF.Choice(1, None, None, 7), score)
    assert best.iters == 2
    assert len(seen) == len(set(seen)) == 9  # baseline, off, 4 pilots, 2 endpoints, the vertex
    assert abs(np.log2(best.quant_mul / 0.46) - 0.3) < 0.05
