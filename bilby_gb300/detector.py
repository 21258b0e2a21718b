"""Detector-side inputs of the likelihood, usable without bilby installed.

A minimal mirror of the parts of bilby's detector package that the
likelihood reads (``bilby/gw/detector/{interferometer,psd,strain_data,
networks,geometry}.py``): detector geometry, PSD from the bundled curves,
seeded Gaussian noise, the frequency mask, and signal injection (projected on
the GPU).  The drop-in likelihood also accepts bilby's own
``Interferometer`` / ``InterferometerList`` objects directly.
"""
from __future__ import annotations

import os

import numpy as np
from scipy.interpolate import interp1d

from . import random as gwl_random

# Detector constants of bilby/gw/detector/detectors/{H1,L1,V1}.interferometer
# (LIGO-T980044-10, LIGO-P1200087-v42): degrees, metres; arm tilts in radians.
DETECTORS = {
    "H1": dict(latitude=46 + 27. / 60 + 18.528 / 3600, longitude=-(119 + 24. / 60 + 27.5657 / 3600),
               elevation=142.554, xarm_azimuth=125.9994, yarm_azimuth=215.9994, xarm_tilt=-6.195e-4,
               yarm_tilt=1.25e-5, length=4, curve=("aLIGO_O4_high_asd", "asd")),
    "L1": dict(latitude=30 + 33. / 60 + 46.4196 / 3600, longitude=-(90 + 46. / 60 + 27.2654 / 3600),
               elevation=-6.574, xarm_azimuth=197.7165, yarm_azimuth=287.7165, xarm_tilt=-3.121e-4,
               yarm_tilt=-6.107e-4, length=4, curve=("aLIGO_O4_high_asd", "asd")),
    "V1": dict(latitude=43 + 37. / 60 + 53.0921 / 3600, longitude=10 + 30. / 60 + 16.1878 / 3600,
               elevation=51.884, xarm_azimuth=70.5674, yarm_azimuth=160.5674, xarm_tilt=0.0, yarm_tilt=0.0,
               length=3, curve=("AdV_psd", "psd")),
}

_CURVES = None


def noise_curve(stem: str):
    """(frequency, value) of a bundled curve: ``aLIGO_O4_high_asd`` or ``AdV_psd``."""
    global _CURVES
    if _CURVES is None:
        z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "noise_curves.npz"))
        _CURVES = {k: z[k] for k in z.files}
    try:
        return _CURVES[stem + "_frequency"], _CURVES[stem + "_value"]
    except KeyError:
        raise ValueError(f"noise curve {stem} is not bundled (available: aLIGO_O4_high_asd, AdV_psd)") from None


# ---------------------------------------------------------------------------
# geometry (bilby/gw/detector/geometry.py:201-300, bilby/gw/geometry.py:51-115,
# bilby/gw/utils.py:59-88)
# ---------------------------------------------------------------------------
def vertex_position_geocentric(latitude, longitude, elevation):
    a, b = 6378137.0, 6356752.314
    radius = a ** 2 * (a ** 2 * np.cos(latitude) ** 2 + b ** 2 * np.sin(latitude) ** 2) ** (-0.5)
    return np.array([(radius + elevation) * np.cos(latitude) * np.cos(longitude),
                     (radius + elevation) * np.cos(latitude) * np.sin(longitude),
                     ((b / a) ** 2 * radius + elevation) * np.sin(latitude)])


def arm_vector(tilt, azimuth, longitude, latitude):
    e_long = np.array([-np.sin(longitude), np.cos(longitude), 0.0])
    e_lat = np.array([-np.sin(latitude) * np.cos(longitude), -np.sin(latitude) * np.sin(longitude),
                      np.cos(latitude)])
    e_h = np.array([np.cos(latitude) * np.cos(longitude), np.cos(latitude) * np.sin(longitude), np.sin(latitude)])
    return (np.cos(tilt) * np.cos(azimuth) * e_long + np.cos(tilt) * np.sin(azimuth) * e_lat
            + np.sin(tilt) * e_h)


class InterferometerGeometry:
    def __init__(self, latitude, longitude, elevation, xarm_azimuth, yarm_azimuth, xarm_tilt=0.0, yarm_tilt=0.0,
                 length=4):
        self.latitude, self.longitude, self.elevation = latitude, longitude, elevation
        self.xarm_azimuth, self.yarm_azimuth = xarm_azimuth, yarm_azimuth
        self.xarm_tilt, self.yarm_tilt, self.length = xarm_tilt, yarm_tilt, length
        lat, lon = np.radians(latitude), np.radians(longitude)
        self.vertex = vertex_position_geocentric(lat, lon, elevation)
        self.x = arm_vector(xarm_tilt, np.radians(xarm_azimuth), lon, lat)
        self.y = arm_vector(yarm_tilt, np.radians(yarm_azimuth), lon, lat)
        self.detector_tensor = (np.outer(self.x, self.x) - np.outer(self.y, self.y)) / 2


# ---------------------------------------------------------------------------
# PSD (bilby/gw/detector/psd.py:13-393)
# ---------------------------------------------------------------------------
class PowerSpectralDensity:
    def __init__(self, frequency_array=None, psd_array=None, asd_array=None, psd_file=None, asd_file=None):
        if asd_file is not None:
            f, v = noise_curve(os.path.splitext(os.path.basename(asd_file))[0])
            self.frequency_array, self.psd_array = f, v ** 2
        elif psd_file is not None:
            f, v = noise_curve(os.path.splitext(os.path.basename(psd_file))[0])
            self.frequency_array, self.psd_array = f, v
        elif psd_array is not None:
            self.frequency_array, self.psd_array = np.asarray(frequency_array), np.asarray(psd_array)
        elif asd_array is not None:
            self.frequency_array, self.psd_array = np.asarray(frequency_array), np.asarray(asd_array) ** 2
        else:
            raise ValueError("a PSD needs arrays or a bundled curve name")
        # psd.py:236-244: linear in the PSD, +inf outside the table
        self._interp = interp1d(self.frequency_array, self.psd_array, bounds_error=False, fill_value=np.inf)

    def get_power_spectral_density_array(self, frequency_array):
        return self._interp(frequency_array)

    def get_amplitude_spectral_density_array(self, frequency_array):
        return self._interp(frequency_array) ** 0.5

    def get_noise_realisation(self, number_of_samples, duration, *, random_state=None):
        """psd.py:350-376 + core/utils/series.py:161-198."""
        rng = gwl_random.resolve(random_state)
        freqs = np.arange(number_of_samples) / duration
        re1, im1 = rng.normal(0, 0.5 * duration ** 0.5, (2, len(freqs)))
        white = re1 + 1j * im1
        white[0] = 0
        white[-1] = 0
        with np.errstate(invalid="ignore"):
            strain = self._interp(freqs) ** 0.5 * white
        oob = (freqs < self.frequency_array.min()) | (freqs > self.frequency_array.max())
        strain[oob] = 0j
        return np.nan_to_num(strain), freqs


# ---------------------------------------------------------------------------
# strain data (bilby/gw/detector/strain_data.py)
# ---------------------------------------------------------------------------
class InterferometerStrainData:
    def __init__(self, minimum_frequency=20.0, maximum_frequency=2048.0):
        self.minimum_frequency = minimum_frequency
        self._maximum_frequency = maximum_frequency
        self.sampling_frequency = None
        self.duration = None
        self.start_time = 0.0
        self.frequency_array = None
        self._strain = None
        self.window_factor = 1

    @property
    def maximum_frequency(self):
        if self.sampling_frequency is not None:
            return min(self._maximum_frequency, self.sampling_frequency / 2)
        return self._maximum_frequency

    @maximum_frequency.setter
    def maximum_frequency(self, value):
        self._maximum_frequency = value

    def _grid(self, sampling_frequency, duration, start_time):
        self.sampling_frequency = float(sampling_frequency)
        self.duration = float(duration)
        self.start_time = float(start_time)
        n_samples = np.round(duration * sampling_frequency)
        self.frequency_array = np.linspace(0, sampling_frequency / 2, num=int(np.round(n_samples / 2) + 1))

    @property
    def frequency_mask(self):
        f = self.frequency_array
        return (f >= self.minimum_frequency) & (f <= self.maximum_frequency)

    @property
    def frequency_domain_strain(self):
        return self._strain * self.frequency_mask

    @frequency_domain_strain.setter
    def frequency_domain_strain(self, value):
        if len(value) != len(self.frequency_array):
            raise ValueError("The frequency_array and the set strain have different lengths")
        self._strain = np.asarray(value, dtype=np.complex128)

    def set_from_power_spectral_density(self, psd, sampling_frequency, duration, start_time=0, *,
                                        random_state=None):
        self._grid(sampling_frequency, duration, start_time)
        self._strain, _ = psd.get_noise_realisation(len(self.frequency_array), self.duration,
                                                    random_state=random_state)

    def set_from_frequency_domain_strain(self, frequency_domain_strain, sampling_frequency, duration, start_time=0):
        self._grid(sampling_frequency, duration, start_time)
        self.frequency_domain_strain = frequency_domain_strain

    def set_from_zero_noise(self, sampling_frequency, duration, start_time=0):
        self._grid(sampling_frequency, duration, start_time)
        self._strain = np.zeros(len(self.frequency_array), dtype=np.complex128)


# ---------------------------------------------------------------------------
# interferometer (bilby/gw/detector/interferometer.py)
# ---------------------------------------------------------------------------
class Interferometer:
    def __init__(self, name, power_spectral_density, minimum_frequency, maximum_frequency, length, latitude,
                 longitude, elevation, xarm_azimuth, yarm_azimuth, xarm_tilt=0.0, yarm_tilt=0.0,
                 calibration_model=None):
        self.name = name
        self.geometry = InterferometerGeometry(latitude, longitude, elevation, xarm_azimuth, yarm_azimuth,
                                               xarm_tilt, yarm_tilt, length)
        self.power_spectral_density = power_spectral_density
        self.strain_data = InterferometerStrainData(minimum_frequency, maximum_frequency)
        self.calibration_model = calibration_model
        self.meta_data = dict()

    minimum_frequency = property(lambda self: self.strain_data.minimum_frequency)
    maximum_frequency = property(lambda self: self.strain_data.maximum_frequency)
    frequency_domain_strain = property(lambda self: self.strain_data.frequency_domain_strain)

    # noise-weighted inner products over the masked band (interferometer.py:607-679,
    # gw/utils.py:118-190): host utilities on arrays the caller already holds
    def _weighted(self, aa, bb):
        m = self.frequency_mask
        return 4 / self.duration * np.sum(np.conj(aa[m]) * bb[m] / self.power_spectral_density_array[m])

    def inner_product(self, signal):
        return self._weighted(signal, self.frequency_domain_strain)

    def optimal_snr_squared(self, signal):
        return self._weighted(signal, signal).real

    def template_template_inner_product(self, signal_1, signal_2):
        return self._weighted(signal_1, signal_2)

    def matched_filter_snr(self, signal):
        return self.inner_product(signal) / self.optimal_snr_squared(signal) ** 0.5

    frequency_array = property(lambda self: self.strain_data.frequency_array)
    frequency_mask = property(lambda self: self.strain_data.frequency_mask)
    sampling_frequency = property(lambda self: self.strain_data.sampling_frequency)
    duration = property(lambda self: self.strain_data.duration)
    start_time = property(lambda self: self.strain_data.start_time)

    @property
    def power_spectral_density_array(self):
        # interferometer.py:551-564 (window correction 1 unless the legacy normalisation is requested)
        corr = self.strain_data.window_factor if os.environ.get(
            "BILBY_INCORRECT_PSD_NORMALIZATION", "FALSE").upper() in ("TRUE", "T", "1", "YES") else 1
        return self.power_spectral_density.get_power_spectral_density_array(self.frequency_array) * corr

    def set_strain_data_from_power_spectral_density(self, sampling_frequency, duration, start_time=0, *,
                                                    random_state=None):
        self.strain_data.set_from_power_spectral_density(self.power_spectral_density, sampling_frequency,
                                                         duration, start_time, random_state=random_state)

    def get_detector_response(self, waveform_polarizations, parameters):
        """interferometer.py:303-368, evaluated by the float64 GPU kernel."""
        from . import _capi
        from .analysis import params_block
        return _capi.detector_response(self.name, self.geometry.vertex, self.geometry.detector_tensor,
                                       self.strain_data.start_time, self.frequency_mask, self.frequency_array,
                                       waveform_polarizations["plus"], waveform_polarizations["cross"],
                                       params_block(parameters)[:, 0])

    def inject_signal(self, parameters, injection_polarizations=None, waveform_generator=None, raise_error=True):
        """interferometer.py:412-510: the masked strain plus the projected signal."""
        if injection_polarizations is None:
            if waveform_generator is None:
                raise ValueError("inject_signal needs one of waveform_generator or injection_polarizations.")
            injection_polarizations = waveform_generator.frequency_domain_strain(parameters)
        signal = self.get_detector_response(injection_polarizations, parameters)
        self.strain_data.frequency_domain_strain = self.strain_data.frequency_domain_strain + signal
        # interferometer.py:512-516 (read by the ROQ time resolution)
        self.meta_data["optimal_SNR"] = self.optimal_snr_squared(signal).real ** 0.5
        self.meta_data["matched_filter_SNR"] = self.matched_filter_snr(signal)
        self.meta_data["parameters"] = parameters
        return injection_polarizations


def get_empty_interferometer(name):
    if name not in DETECTORS:
        raise ValueError(f"interferometer {name} is not known (available: {sorted(DETECTORS)})")
    d = dict(DETECTORS[name])
    stem, kind = d.pop("curve")
    psd = PowerSpectralDensity(asd_file=stem) if kind == "asd" else PowerSpectralDensity(psd_file=stem)
    return Interferometer(name, psd, 20.0, 2048.0, **d)


class InterferometerList(list):
    """bilby/gw/detector/networks.py:13-353 (the parts the likelihood uses)."""

    def __init__(self, interferometers):
        super().__init__()
        if isinstance(interferometers, str):
            raise TypeError("Input must not be a string")
        for ifo in interferometers:
            self.append(get_empty_interferometer(ifo) if isinstance(ifo, str) else ifo)

    def set_strain_data_from_power_spectral_densities(self, sampling_frequency, duration, start_time=0, *,
                                                      random_state=None):
        for ifo in self:
            ifo.set_strain_data_from_power_spectral_density(sampling_frequency, duration, start_time,
                                                            random_state=random_state)

    def inject_signal(self, parameters=None, injection_polarizations=None, waveform_generator=None,
                      raise_error=True):
        if injection_polarizations is None:
            injection_polarizations = waveform_generator.frequency_domain_strain(parameters)
        for ifo in self:
            ifo.inject_signal(parameters, injection_polarizations=injection_polarizations)
        return injection_polarizations

    def _common(self, attr):
        vals = [getattr(ifo.strain_data, attr) for ifo in self]
        if any(v != vals[0] for v in vals):
            raise ValueError(f"The {attr} of all interferometers are not the same")
        return vals[0]

    start_time = property(lambda self: self._common("start_time"))
    duration = property(lambda self: self._common("duration"))
    sampling_frequency = property(lambda self: self._common("sampling_frequency"))
    frequency_array = property(lambda self: self[0].strain_data.frequency_array)

    @property
    def meta_data(self):
        return {ifo.name: dict(ifo.meta_data, minimum_frequency=ifo.minimum_frequency,
                               maximum_frequency=ifo.maximum_frequency) for ifo in self}
