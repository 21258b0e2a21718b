"""Host parts of the per-detector and reconstruction API: the SNR container
(base.py:108-148) and the tabulated-density sampler
(bilby/core/prior/interpolated.py:10-160)."""
import numpy as np
import pytest

from bilby_gb300.likelihood import GravitationalWaveTransient
from bilby_gb300.prior import Interped


def test_calculated_snrs_sum_and_array_identity():
    S = GravitationalWaveTransient._CalculatedSNRs
    a = S(d_inner_h=1 + 2j, optimal_snr_squared=4.0, complex_matched_filter_snr=0.5j)
    b = S(d_inner_h=3 - 1j, optimal_snr_squared=5.0, d_inner_h_array=np.array([1.0, 2.0]))
    c = a + b
    assert c.d_inner_h == 4 + 1j and c.optimal_snr_squared == 9.0
    np.testing.assert_array_equal(c.d_inner_h_array, [1.0, 2.0])  # None + array = array
    assert c.optimal_snr_squared_array is None
    assert a.d_inner_h == 1 + 2j  # + leaves its operands alone
    c += b
    np.testing.assert_array_equal(c.d_inner_h_array, [2.0, 4.0])
    assert c.snrs_as_sample["optimal_snr"] == pytest.approx(np.sqrt(14.0))
    total = S()
    for s in (a, b):
        total += s
    assert total.d_inner_h == 4 + 1j


def test_interped_inverse_cdf_of_a_linear_density():
    x = np.linspace(0.0, 1.0, 2001)
    p = Interped(x, 2 * x)
    u = np.array([0.0, 0.01, 0.25, 0.5, 0.81, 1.0])
    np.testing.assert_allclose(p.rescale(u), np.sqrt(u), atol=2e-4)
    assert p.prob(0.5) == pytest.approx(1.0)
    assert p.prob(1.5) == 0.0


def test_interped_regrids_and_narrows_like_the_reference():
    # uneven abscissae are re-gridded evenly between the limits; a narrowed
    # maximum renormalises on the narrower interval
    x = np.array([0.0, 0.1, 0.5, 2.0])
    p = Interped(x, np.ones(4), maximum=1.0)
    assert p.minimum == 0.0 and p.maximum == 1.0
    np.testing.assert_allclose(p.xx, np.linspace(0.0, 1.0, 4))
    assert p.rescale(0.5) == pytest.approx(0.5)


def test_interped_sample_uses_the_shared_generator():
    from bilby_gb300 import random as grandom
    x = np.linspace(-1.0, 1.0, 101)
    p = Interped(x, np.exp(-x ** 2))
    grandom.seed(11)
    a = p.sample()
    u = np.random.default_rng(11).uniform(0, 1)
    assert a == pytest.approx(p.rescale(u), abs=0)
    assert p.sample(3, random_state=5).shape == (3,)
