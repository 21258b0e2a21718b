"""Global seeded random generator, as bilby/core/utils/random.py:64-159 keeps
one: ``seed(s)`` replaces the shared numpy Generator; the noise draws of the
detector module use it, so a seed gives the reference's noise realisation."""
from __future__ import annotations

import numpy as np


class Generator:
    rng = np.random.default_rng()


def seed(s):
    Generator.rng = np.random.default_rng(s)


def resolve(random_state=None):
    if random_state is None:
        return Generator.rng
    if isinstance(random_state, np.random.Generator):
        return random_state
    return np.random.default_rng(random_state)
