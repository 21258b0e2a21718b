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


class TruncatedGaussian(Prior):
    """A Gaussian of mean mu and width sigma restricted to [minimum, maximum]
    (analytical.py:583-640)."""

    def __init__(self, mu, sigma, minimum, maximum, **kwargs):
        super().__init__(minimum, maximum, **kwargs)
        self.mu, self.sigma = mu, sigma

    @property
    def normalisation(self):
        from scipy.special import erf
        return (erf((self.maximum - self.mu) / 2 ** 0.5 / self.sigma)
                - erf((self.minimum - self.mu) / 2 ** 0.5 / self.sigma)) / 2

    def rescale(self, val):
        from scipy.special import erf, erfinv
        return erfinv(2 * val * self.normalisation + erf((self.minimum - self.mu) / 2 ** 0.5 / self.sigma)) \
            * 2 ** 0.5 * self.sigma + self.mu

    def prob(self, val):
        return np.exp(-(self.mu - val) ** 2 / (2 * self.sigma ** 2)) / (2 * np.pi) ** 0.5 / self.sigma \
            / self.normalisation * self.is_in_prior_range(val)


class Interped(Prior):
    """A density tabulated at points ``xx`` (bilby/core/prior/interpolated.py:10-160):
    linear interpolation of ``yy`` onto an evenly spaced grid of the same
    length between ``minimum`` and ``maximum`` (the extent of ``xx`` unless
    narrowed), normalised by the trapezoid rule; ``rescale`` is the linear
    interpolation of the inverse of the cumulative trapezoid, whose last value
    is set to exactly one."""

    def __init__(self, xx, yy, minimum=np.nan, maximum=np.nan, **kwargs):
        from scipy.interpolate import interp1d
        xx = np.asarray(xx, dtype=np.float64)
        yy = np.asarray(yy, dtype=np.float64)
        self.min_limit, self.max_limit = float(np.min(xx)), float(np.max(xx))
        minimum = float(np.nanmax(np.array((self.min_limit, minimum))))
        maximum = float(np.nanmin(np.array((self.max_limit, maximum))))
        super().__init__(minimum, maximum, **kwargs)
        full = interp1d(x=xx, y=yy, bounds_error=False, fill_value=0)
        self.xx = np.linspace(minimum, maximum, len(xx))
        self.yy = full(self.xx)
        self._tabulate()

    def _tabulate(self):
        from scipy.integrate import cumulative_trapezoid, trapezoid
        from scipy.interpolate import interp1d
        self.yy = self.yy / trapezoid(self.yy, self.xx)
        self.YY = cumulative_trapezoid(self.yy, self.xx, initial=0)
        self.YY[-1] = 1
        self._pdf = interp1d(x=self.xx, y=self.yy, bounds_error=False, fill_value=0)
        self._inverse_cdf = interp1d(x=self.YY, y=self.xx, bounds_error=True)

    def prob(self, val):
        return self._pdf(val)[()]

    def rescale(self, val):
        return self._inverse_cdf(val)[()]

    def sample(self, size=None, *, random_state=None):
        """One uniform draw per sample from the shared generator (or
        ``random_state``), rescaled (bilby/core/prior/base.py:143-165)."""
        from .random import resolve
        rng = resolve(random_state)
        if isinstance(size, (int, np.integer)):
            size = (size,)
        return self.rescale(rng.uniform(low=0, high=1, size=size))
