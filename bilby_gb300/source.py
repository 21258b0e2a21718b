"""Frequency-domain source models with bilby's source-model signature.

Passing one of these (or ``bilby.gw.source.sinegaussian``) to a
``WaveformGenerator`` selects the matching fused CUDA likelihood kernel.
Called directly (e.g. by ``inject_signal``), they evaluate the polarisations
with the float64 GPU kernel and return numpy arrays.
"""
from __future__ import annotations

import numpy as np

from . import _capi
from .analysis import params_block


def sinegaussian(frequency_array, hrss, Q, frequency, **kwargs):
    """Sine-Gaussian burst (bilby/gw/source.py:1153-1209)."""
    p = params_block(dict(hrss=hrss, Q=Q, frequency=frequency))[:, 0]
    plus, cross = _capi.source_polarizations(_capi.MODEL_SINEGAUSSIAN, np.asarray(frequency_array), p)
    return {"plus": plus, "cross": cross}


def taylorf2_aligned(frequency_array, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase,
                     **kwargs):
    """3.5PN aligned-spin TaylorF2 inspiral (restricted, Newtonian amplitude).

    h_+ = A(f) (1 + cos^2 theta_jn)/2 e^{-i Psi(f)}, h_x = -i A(f) cos theta_jn e^{-i Psi(f)},
    A(f) = sqrt(5/24) pi^(-2/3) (G Mc/c^3)^(5/6) f^(-7/6) c / d_L,
    Psi(f) = -2 phase - pi/4 + 3/(128 eta v^5) sum_k (a_k + l_k ln v) v^k, v = (pi G M f / c^3)^(1/3),
    non-zero for minimum_frequency <= f < f_ISCO.  Phase coefficients: arXiv:0907.0700 Eq. (3.18)
    (non-spinning), arXiv:0810.5336, arXiv:1303.7412, arXiv:1601.05588 (aligned spins, chi_s/chi_a form).
    ``minimum_frequency`` (default 20 Hz) is a waveform argument.
    """
    p = params_block(dict(mass_1=mass_1, mass_2=mass_2, chi_1=chi_1, chi_2=chi_2,
                          luminosity_distance=luminosity_distance, theta_jn=theta_jn, phase=phase))[:, 0]
    plus, cross = _capi.source_polarizations(_capi.MODEL_TAYLORF2, np.asarray(frequency_array), p,
                                             kwargs.get("minimum_frequency", 20.0))
    return {"plus": plus, "cross": cross}


def taylorf2_aligned_relative_binning(frequency_array, mass_1, mass_2, chi_1, chi_2, luminosity_distance,
                                      theta_jn, phase, **kwargs):
    """``taylorf2_aligned`` with bilby's relative-binning source convention
    (bilby/gw/source.py:724-761): ``fiducial=1`` evaluates on the full grid,
    otherwise on the ``frequency_bin_edges`` waveform argument."""
    fiducial = kwargs.pop("fiducial", 0)
    edges = kwargs.pop("frequency_bin_edges", None)
    grid = frequency_array if (fiducial == 1 or edges is None) else edges
    return taylorf2_aligned(grid, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase, **kwargs)


def taylorf2_aligned_frequency_sequence(frequency_array, mass_1, mass_2, chi_1, chi_2, luminosity_distance,
                                        theta_jn, phase, **kwargs):
    """``taylorf2_aligned`` on the ``frequencies`` waveform argument, the
    convention of bilby's frequency-sequence source models used by the
    multi-banded likelihood (bilby/gw/likelihood/multiband.py:451-481)."""
    frequencies = kwargs.pop("frequencies", None)
    grid = frequency_array if frequencies is None else frequencies
    return taylorf2_aligned(grid, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase, **kwargs)


def taylorf2_aligned_roq(frequency_array, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase,
                         **kwargs):
    """``taylorf2_aligned`` with bilby's ROQ source convention
    (bilby/gw/source.py:802-900): {"linear": ..., "quadratic": ...} at the
    frequency nodes of the waveform arguments."""
    if "frequency_nodes" in kwargs:
        nodes = kwargs.pop("frequency_nodes")
        li, qi = kwargs.pop("linear_indices"), kwargs.pop("quadratic_indices")
        pols = taylorf2_aligned(nodes, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase, **kwargs)
        return {"linear": {m: v[li] for m, v in pols.items()}, "quadratic": {m: v[qi] for m, v in pols.items()}}
    fl, fq = kwargs.pop("frequency_nodes_linear"), kwargs.pop("frequency_nodes_quadratic")
    return {"linear": taylorf2_aligned(fl, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase,
                                       **kwargs),
            "quadratic": taylorf2_aligned(fq, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase,
                                          **kwargs)}


def model_of(source_model) -> str:
    """Which fused kernel serves ``source_model`` ('sinegaussian' | 'taylorf2').

    Raises NotImplementedError for any other model: there is no CPU fallback.
    """
    name = getattr(source_model, "__name__", "")
    module = getattr(source_model, "__module__", "") or ""
    if source_model is sinegaussian or (name == "sinegaussian" and module.endswith("gw.source")):
        return "sinegaussian"
    if source_model in (taylorf2_aligned, taylorf2_aligned_relative_binning, taylorf2_aligned_frequency_sequence,
                        taylorf2_aligned_roq) \
            or name in ("taylorf2_aligned", "taylorf2_aligned_relative_binning", "taylorf2_aligned_frequency_sequence",
                        "taylorf2_aligned_roq"):
        return "taylorf2"
    raise NotImplementedError(
        f"source model {module}.{name} has no GPU kernel (supported: sinegaussian, taylorf2_aligned)")
