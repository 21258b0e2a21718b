"""The prior distributions the marginalised likelihood needs, for use without
bilby installed (bilby/core/prior/analytical.py:78-265); bilby's own priors
are accepted as well (anything with ``prob``, ``rescale``, ``minimum``,
``maximum``)."""
from __future__ import annotations

import numpy as np


class Prior:
    def __init__(self, minimum=-np.inf, maximum=np.inf, name=None, latex_label=None, unit=None, boundary=None):
        self.minimum, self.maximum = minimum, maximum
        self.name, self.latex_label, self.unit, self.boundary = name, latex_label, unit, boundary

    is_fixed = False

    def is_in_prior_range(self, val):
        return (val >= self.minimum) & (val <= self.maximum)


class Uniform(Prior):
    def rescale(self, val):
        return self.minimum + val * (self.maximum - self.minimum)

    def prob(self, val):
        """analytical.py:231-242."""
        return ((val >= self.minimum) & (val <= self.maximum)) / (self.maximum - self.minimum)


class PowerLaw(Prior):
    def __init__(self, alpha, minimum, maximum, **kwargs):
        super().__init__(minimum, maximum, **kwargs)
        self.alpha = alpha

    def rescale(self, val):
        """analytical.py:104-123."""
        if self.alpha == -1:
            return self.minimum * np.exp(val * np.log(self.maximum / self.minimum))
        return (self.minimum ** (1 + self.alpha) + val * (self.maximum ** (1 + self.alpha)
                                                          - self.minimum ** (1 + self.alpha))) ** (1. / (1 + self.alpha))

    def prob(self, val):
        """analytical.py:125-141."""
        if self.alpha == -1:
            return np.nan_to_num(1 / val / np.log(self.maximum / self.minimum)) * self.is_in_prior_range(val)
        return np.nan_to_num(val ** self.alpha * (1 + self.alpha) / (self.maximum ** (1 + self.alpha)
                                                                      - self.minimum ** (1 + self.alpha))) \
            * self.is_in_prior_range(val)


class DeltaFunction(Prior):
    def __init__(self, peak, **kwargs):
        super().__init__(peak, peak, **kwargs)
        self.peak = peak

    is_fixed = True

    def rescale(self, val):
        return self.peak * val ** 0

    def prob(self, val):
        return np.where(val == self.peak, np.inf, 0.0)


class LogUniform(PowerLaw):
    """analytical.py:265-290: a power law with alpha = -1."""

    def __init__(self, minimum, maximum, **kwargs):
        super().__init__(-1, minimum, maximum, **kwargs)


class Sine(Prior):
    """analytical.py:450-507: p(x) proportional to sin x on [0, pi] by default."""

    def __init__(self, minimum=0.0, maximum=np.pi, **kwargs):
        super().__init__(minimum, maximum, **kwargs)

    def rescale(self, val):
        norm = 1 / (np.cos(self.minimum) - np.cos(self.maximum))
        return np.arccos(np.cos(self.minimum) - val / norm)

    def prob(self, val):
        return np.sin(val) / 2 * self.is_in_prior_range(val)


class Cosine(Prior):
    """analytical.py:390-447: p(x) proportional to cos x on [-pi/2, pi/2] by default."""

    def __init__(self, minimum=-np.pi / 2, maximum=np.pi / 2, **kwargs):
        super().__init__(minimum, maximum, **kwargs)

    def rescale(self, val):
        norm = 1 / (np.sin(self.maximum) - np.sin(self.minimum))
        return np.arcsin(val / norm + np.sin(self.minimum))

    def prob(self, val):
        return np.cos(val) / 2 * self.is_in_prior_range(val)


class Gaussian(Prior):
    """analytical.py:510-576."""

    def __init__(self, mu, sigma, **kwargs):
        super().__init__(-np.inf, np.inf, **kwargs)
        self.mu, self.sigma = mu, sigma

    def rescale(self, val):
        from scipy.special import erfinv
        return self.mu + erfinv(2 * val - 1) * 2 ** 0.5 * self.sigma

    def prob(self, val):
        return np.exp(-(self.mu - val) ** 2 / (2 * self.sigma ** 2)) / (2 * np.pi) ** 0.5 / self.sigma
