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
