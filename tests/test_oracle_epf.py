"""The EPF restatement (oracle/epf.py): the cases the reference's oracle
settles without filtering (src/epf_filter/tests.rs:101-104, :59-66)."""
import numpy as np

from oracle import epf as E

F = np.float32


def test_no_stages_or_no_sharpness_return_the_image():
    img = np.random.default_rng(1).uniform(0, 1, (3, 12, 10)).astype(F)
    sq = np.full(4, -1.0, F)
    for iters, sharp in ((0, 7), (2, 0)):
        assert np.array_equal(E.epf(img, sq, iters, 0.46, 0.9, 6.5, 2 / 3, [40, 5, 3.5], sharp), img)


def test_unfiltered_blocks_keep_their_pixels_exactly():
    # a sigma_quant of 0 gives 1 / -1e-4, below MIN_SIGMA: the block is left alone
    # small noise, so that the filtered blocks' weights are well above zero
    img = (F(0.5) + np.random.default_rng(2).uniform(0, 0.002, (3, 16, 16))).astype(F)
    sq = np.array([0.0, -1.0, 0.0, -1.0], F)
    one = E._stage(img, sq, 0.46, 7, 1, E.SAD_MUL, 2 / 3, [40, 5, 3.5])
    assert np.array_equal(one[:, :8, :8], img[:, :8, :8])
    assert np.array_equal(one[:, 8:, :8], img[:, 8:, :8])
    assert not np.array_equal(one[:, :8, 8:], img[:, :8, 8:])
