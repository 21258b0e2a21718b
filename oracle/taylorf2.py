"""numpy transcription of a 3.5PN aligned-spin TaylorF2 inspiral, written
from the published post-Newtonian formulae.

TEST INFRASTRUCTURE ONLY (the checker for the CUDA TaylorF2 kernels).  It has
bilby's source-model signature, so it plugs into the reference's
``WaveformGenerator`` / ``GravitationalWaveTransient`` as
``frequency_domain_source_model`` exactly like ``bilby.gw.source.sinegaussian``
(bilby/gw/source.py:1153-1209).  In bilby, TaylorF2 itself is reached through
lalsimulation (bilby/gw/source.py:552-690 -> bilby/gw/utils.py:642-686), an
external C library that is not part of the reference tree and not installed
here; parity of this model against lalsimulation is therefore unpinned.

Model definition (Fourier convention of bilby: h(f) = int h(t) e^{-2 pi i f t}):

    h_+(f) = A(f) (1 + cos^2 theta_jn) / 2 * exp(-i Psi(f))
    h_x(f) = -i A(f) cos theta_jn * exp(-i Psi(f))
    A(f)   = sqrt(5/24) pi^(-2/3) (G Mc / c^3)^(5/6) f^(-7/6) c / d_L
    Psi(f) = -2 phase - pi/4 + 3 / (128 eta v^5) * sum_k (a_k + l_k ln v) v^k
    v      = (pi G M f / c^3)^(1/3)

non-zero for minimum_frequency <= f < f_ISCO = 1 / (6^(3/2) pi G M / c^3);
coalescence time 0 (the detector response applies the geocentre time).

Phase coefficients a_k, l_k (eta = m1 m2 / M^2, delta = (m1 - m2) / M,
chi_s = (chi_1 + chi_2) / 2, chi_a = (chi_1 - chi_2) / 2):

* non-spinning 0PN..3.5PN: Buonanno, Iyer, Ochsner, Pan & Sathyaprakash,
  Phys. Rev. D 80, 084043 (2009), arXiv:0907.0700, Eq. (3.18) (with the
  2.5PN constant ln v_LSO dropped, and ln(4v) split into ln 4 + ln v);
* spin-orbit 1.5PN and 2.5PN and spin-spin 2PN: Arun, Buonanno, Faye &
  Ochsner, Phys. Rev. D 79, 104023 (2009), arXiv:0810.5336, with black-hole
  quadrupole (kappa = 1) in the chi_s / chi_a form;
* spin-orbit 3PN and 3.5PN: Bohe, Marsat, Faye & Blanchet, Class. Quantum
  Grav. 30, 135009 (2013), arXiv:1303.7412; spin-spin 3PN: Mishra, Kela,
  Arun & Faye, Phys. Rev. D 93, 084054 (2016), arXiv:1601.05588.
"""
from __future__ import annotations

import numpy as np

MTSUN_SI = 4.925490947641267e-06      # G M_sun / c^3 in seconds
PC_SI = 3.085677581491367e16          # parsec in metres
C_SI = 299792458.0
GAMMA_E = 0.5772156649015329


def phase_coefficients(mass_1, mass_2, chi_1, chi_2):
    """Return (a[0..7], l[0..7]) for the bracket sum of Psi (float64 scalars)."""
    m = mass_1 + mass_2
    eta = mass_1 * mass_2 / (m * m)
    delta = (mass_1 - mass_2) / m
    chi_s = 0.5 * (chi_1 + chi_2)
    chi_a = 0.5 * (chi_1 - chi_2)
    pi = np.pi
    a = np.zeros(8)
    l = np.zeros(8)
    a[0] = 1.0
    a[2] = 3715.0 / 756.0 + 55.0 * eta / 9.0
    a[3] = (-16.0 * pi + 113.0 / 3.0 * delta * chi_a
            + (113.0 / 3.0 - 76.0 * eta / 3.0) * chi_s)
    a[4] = (15293365.0 / 508032.0 + 27145.0 * eta / 504.0 + 3085.0 * eta * eta / 72.0
            + (-405.0 / 8.0 + 200.0 * eta) * chi_a * chi_a
            - 405.0 / 4.0 * delta * chi_s * chi_a
            + (-405.0 / 8.0 + 5.0 * eta / 2.0) * chi_s * chi_s)
    gamma = ((732985.0 / 2268.0 - 24260.0 * eta / 81.0 - 340.0 * eta * eta / 9.0) * chi_s
             + (732985.0 / 2268.0 + 140.0 * eta / 9.0) * delta * chi_a)
    c5 = pi * (38645.0 / 756.0 - 65.0 * eta / 9.0) - gamma
    a[5] = c5
    l[5] = 3.0 * c5
    a[6] = (11583231236531.0 / 4694215680.0 - 640.0 * pi * pi / 3.0 - 6848.0 * GAMMA_E / 21.0
            - 6848.0 / 21.0 * np.log(4.0)
            + eta * (-15737765635.0 / 3048192.0 + 2255.0 * pi * pi / 12.0)
            + 76055.0 * eta * eta / 1728.0 - 127825.0 * eta ** 3 / 1296.0
            + pi * (2270.0 / 3.0 * delta * chi_a + (2270.0 / 3.0 - 520.0 * eta) * chi_s)
            + (75515.0 / 144.0 - 8225.0 * eta / 18.0) * delta * chi_s * chi_a
            + (75515.0 / 288.0 - 263245.0 * eta / 252.0 - 480.0 * eta * eta) * chi_a * chi_a
            + (75515.0 / 288.0 - 232415.0 * eta / 504.0 + 1255.0 * eta * eta / 9.0) * chi_s * chi_s)
    l[6] = -6848.0 / 21.0
    a[7] = (pi * (77096675.0 / 254016.0 + 378515.0 * eta / 1512.0 - 74045.0 * eta * eta / 756.0)
            + (-25150083775.0 / 3048192.0 + 10566655595.0 * eta / 762048.0
               - 1042165.0 * eta * eta / 3024.0 + 5345.0 * eta ** 3 / 36.0) * chi_s
            + delta * (-25150083775.0 / 3048192.0 + 26804935.0 * eta / 6048.0
                       - 1985.0 * eta * eta / 48.0) * chi_a)
    return a, l


def isco_frequency(mass_1, mass_2):
    """f_ISCO = 1 / (6 sqrt(6) pi G M / c^3): written with sqrt so that every
    IEEE-754 implementation rounds it identically."""
    m_sec = (mass_1 + mass_2) * MTSUN_SI
    return 1.0 / (6.0 * np.sqrt(6.0) * np.pi * m_sec)


def amplitude_prefactor(mass_1, mass_2, luminosity_distance):
    """sqrt(5/24) pi^(-2/3) Mc^(5/6) c / d_L (Mc in s, d_L in m); multiply by f^(-7/6)."""
    m = mass_1 + mass_2
    eta = mass_1 * mass_2 / (m * m)
    mc_sec = eta ** 0.6 * m * MTSUN_SI
    d_m = luminosity_distance * 1e6 * PC_SI
    return np.sqrt(5.0 / 24.0) * np.pi ** (-2.0 / 3.0) * mc_sec ** (5.0 / 6.0) * C_SI / d_m


def taylorf2_aligned(frequency_array, mass_1, mass_2, chi_1, chi_2, luminosity_distance,
                     theta_jn, phase, **kwargs):
    """Frequency-domain polarisations {"plus", "cross"} (complex128).

    ``minimum_frequency`` (default 20 Hz) arrives through the generator's
    ``waveform_arguments``, as for bilby's lalsimulation models.
    """
    minimum_frequency = kwargs.get("minimum_frequency", 20.0)
    f = np.asarray(frequency_array, dtype=np.float64)
    m_sec = (mass_1 + mass_2) * MTSUN_SI
    eta = mass_1 * mass_2 / (mass_1 + mass_2) ** 2
    a, l = phase_coefficients(mass_1, mass_2, chi_1, chi_2)
    f_isco = isco_frequency(mass_1, mass_2)
    band = (f >= minimum_frequency) & (f < f_isco)
    fb = f[band]
    v = np.cbrt(np.pi * m_sec * fb)
    lnv = np.log(v)
    s = np.zeros_like(fb)
    vk = np.ones_like(fb)
    for k in range(8):
        s = s + (a[k] + l[k] * lnv) * vk
        vk = vk * v
    psi = -2.0 * phase - np.pi / 4 + 3.0 / (128.0 * eta) * s / v ** 5
    amp = amplitude_prefactor(mass_1, mass_2, luminosity_distance) * fb ** (-7.0 / 6.0)
    ci = np.cos(theta_jn)
    e = np.exp(-1j * psi)
    plus = np.zeros(f.shape, dtype=np.complex128)
    cross = np.zeros(f.shape, dtype=np.complex128)
    plus[band] = amp * (1.0 + ci * ci) / 2.0 * e
    cross[band] = -1j * amp * ci * e
    return {"plus": plus, "cross": cross}


def taylorf2_aligned_relative_binning(frequency_array, mass_1, mass_2, chi_1, chi_2, luminosity_distance,
                                      theta_jn, phase, **kwargs):
    """The same model with the relative-binning source convention of bilby
    (bilby/gw/source.py:724-761): ``fiducial=1`` evaluates on the full grid,
    otherwise on ``frequency_bin_edges`` from the waveform arguments."""
    fiducial = kwargs.pop("fiducial", 0)
    edges = kwargs.pop("frequency_bin_edges", None)
    if fiducial == 1 or edges is None:
        return taylorf2_aligned(frequency_array, mass_1, mass_2, chi_1, chi_2, luminosity_distance,
                                theta_jn, phase, **kwargs)
    return taylorf2_aligned(edges, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase, **kwargs)


def taylorf2_aligned_frequency_sequence(frequency_array, mass_1, mass_2, chi_1, chi_2, luminosity_distance,
                                        theta_jn, phase, **kwargs):
    """The same model on the ``frequencies`` waveform argument, the convention
    of bilby's frequency-sequence source models used by the multi-banded
    likelihood (bilby/gw/source.py, ``binary_black_hole_frequency_sequence``;
    bilby/gw/likelihood/multiband.py:437-439)."""
    frequencies = kwargs.pop("frequencies")
    return taylorf2_aligned(frequencies, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase,
                            **kwargs)


def taylorf2_aligned_roq(frequency_array, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase,
                         **kwargs):
    """The same model with the ROQ source convention of bilby
    (bilby/gw/source.py:802-900): polarisations at the linear and quadratic
    frequency nodes, {"linear": {...}, "quadratic": {...}}."""
    if "frequency_nodes" in kwargs:
        nodes = kwargs.pop("frequency_nodes")
        li = kwargs.pop("linear_indices")
        qi = kwargs.pop("quadratic_indices")
        pols = taylorf2_aligned(nodes, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase,
                                **kwargs)
        return {"linear": {m: v[li] for m, v in pols.items()}, "quadratic": {m: v[qi] for m, v in pols.items()}}
    fl = kwargs.pop("frequency_nodes_linear")
    fq = kwargs.pop("frequency_nodes_quadratic")
    return {"linear": taylorf2_aligned(fl, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase,
                                       **kwargs),
            "quadratic": taylorf2_aligned(fq, mass_1, mass_2, chi_1, chi_2, luminosity_distance, theta_jn, phase,
                                          **kwargs)}
