"""Seeded analyses for the oracle, built the way the reference builds them.

TEST INFRASTRUCTURE ONLY.  Regenerates, with :mod:`oracle.restate`, the data
the reference generates for a workload of ``bilby_gb300.workloads``:
``bilby.core.utils.random.seed(seed)`` then
``InterferometerList(names).set_strain_data_from_power_spectral_densities``
(bilby/gw/detector/networks.py:87-110, one noise draw per detector in list
order from the shared generator) and one injection
(bilby/gw/detector/interferometer.py:412-510).
"""
from __future__ import annotations

import os

import numpy as np

from . import restate as R
from .taylorf2 import taylorf2_aligned

_CURVES = None

SG_ARGS = ("hrss", "Q", "frequency")
TF2_ARGS = ("mass_1", "mass_2", "chi_1", "chi_2", "luminosity_distance", "theta_jn", "phase")


def noise_curves():
    """(frequency, value) tables of the bundled sensitivity curves."""
    global _CURVES
    if _CURVES is None:
        path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "bilby_gb300", "noise_curves.npz")
        z = np.load(path)
        _CURVES = {stem: (z[stem + "_frequency"], z[stem + "_value"])
                   for stem in ("aLIGO_O4_high_asd", "AdV_psd")}
    return _CURVES


def source_for(model, minimum_frequency=20.0):
    """A callable (frequency_array, **params) -> polarisations, taking only
    the arguments the source model declares (waveform_generator.py:260-269)."""
    if model == "sinegaussian":
        def f(freq, **p):
            return R.sinegaussian(freq, **{k: p[k] for k in SG_ARGS})
    else:
        def f(freq, **p):
            return taylorf2_aligned(freq, **{k: p[k] for k in TF2_ARGS}, minimum_frequency=minimum_frequency)
    return f


def build_detectors(names, sampling_frequency, duration, start_time, seed, minimum_frequency=20.0):
    rng = np.random.default_rng(seed)
    curves = noise_curves()
    return [R.make_detector(n, sampling_frequency, duration, start_time, rng, curves,
                            minimum_frequency=minimum_frequency) for n in names]


def build_workload(w, inject=True):
    """Detectors of workload ``w`` (``bilby_gb300.workloads.Workload``), with
    the workload's injection added."""
    dets = build_detectors(w.detectors, w.sampling_frequency, w.duration, w.start_time, w.seed)
    if inject:
        src = source_for(w.model, w.minimum_frequency)
        pols = src(dets[0].frequency, **w.injection)
        for d in dets:
            R.inject(d, pols, w.injection)
    return dets


def strain_checksum(dets):
    return np.array([[np.sum(np.abs(d.masked_strain) ** 2) * 1e42, np.sum(d.masked_strain.real) * 1e21]
                     for d in dets])
