"""CPU restatement (numpy, float64/complex128) of bilby's gravitational-wave
transient likelihood hot path.

TEST INFRASTRUCTURE ONLY.  This module is the *checker*: the GPU tests,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` call it to compute the expected answer or to time the
reference algorithm on host cores.  The library (``bilby_gb300``) never
imports it.

Every function restates one piece of the reference and cites the file:line
(paths inside the bilby project) that it follows.  It is pinned against the
reference itself by ``tests/test_oracle_vs_reference.py`` (run where the
reference tree is importable) and against committed golden values in
``tests/golden/`` (the reference's own known answer
``noise_log_likelihood == -4014.1787704539474`` from
``test/gw/likelihood_test.py:195-201`` among them).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
from scipy.interpolate import RectBivariateSpline, interp1d
from scipy.special import i0e, logsumexp

# ---------------------------------------------------------------------------
# time: GPS -> GMST                                  bilby/gw/time.py:63-192
# ---------------------------------------------------------------------------
JULIAN_GPS_EPOCH = 1721013.5           # time.py:70
EPOCH_J2000_0_JD = 2451545.0           # time.py:71
DAYS_PER_CENTURY = 36525.0             # time.py:72
SECONDS_PER_DAY = 86400.0              # time.py:73
LEAP_SECONDS = np.array([              # time.py:74-93 (GPS seconds of each leap)
    46828800, 78364801, 109900802, 173059203, 252028804, 315187205, 346723206,
    393984007, 425520008, 457056009, 504489610, 551750411, 599184012, 820108813,
    914803214, 1025136015, 1119744016, 1167264017], dtype=np.float64)


def n_leap_seconds(gps):
    """Number of leap seconds strictly before ``gps`` (time.py:168-192)."""
    gps = np.asarray(gps, dtype=np.float64)
    return np.sum(gps[..., None] > LEAP_SECONDS, axis=-1)


def julian_day_of_gps_second(gps_int):
    """Julian day of the barebones UTC datetime built by ``gps_time_to_utc``.

    ``gps_time_to_utc`` (time.py:96-111) returns ``GPS_EPOCH + datetime(second=
    gps - n_leap)``; the datetime ``julian_day`` property (time.py:57-66) then
    adds ``second / 86400`` to the day number of 1980-01-06.
    """
    year, month, day = 1980, 1, 6
    day_number = (367 * year - 7 * (year + (month + 9) // 12) // 4
                  + 275 * month // 9 + day)
    second = np.asarray(gps_int, dtype=np.float64) - n_leap_seconds(gps_int)
    return day_number + second / SECONDS_PER_DAY + JULIAN_GPS_EPOCH


def greenwich_mean_sidereal_time(gps):
    """GMST in radians, unreduced (time.py:114-165 with zero equation of equinoxes)."""
    gps = np.asarray(gps, dtype=np.float64)
    jd = julian_day_of_gps_second(gps // 1)
    t_hi = (jd - EPOCH_J2000_0_JD) / DAYS_PER_CENTURY
    t_lo = (gps % 1) / (DAYS_PER_CENTURY * SECONDS_PER_DAY)
    t = t_hi + t_lo
    st = 0.0 + (-6.2e-6 * t + 0.093104) * t ** 2 + 67310.54841
    st = st + 8640184.812866 * t_lo
    st = st + 3155760000.0 * t_lo
    st = st + 8640184.812866 * t_hi
    st = st + 3155760000.0 * t_hi
    return st * 2 * np.pi / SECONDS_PER_DAY


# ---------------------------------------------------------------------------
# detector geometry                  bilby/gw/geometry.py, bilby/gw/utils.py:59-88
# ---------------------------------------------------------------------------
def vertex_position_geocentric(latitude, longitude, elevation):
    """utils.py:59-88 (WGS-84 ellipsoid)."""
    a = 6378137.0
    b = 6356752.314
    radius = a ** 2 * (a ** 2 * np.cos(latitude) ** 2 + b ** 2 * np.sin(latitude) ** 2) ** (-0.5)
    x = (radius + elevation) * np.cos(latitude) * np.cos(longitude)
    y = (radius + elevation) * np.cos(latitude) * np.sin(longitude)
    z = ((b / a) ** 2 * radius + elevation) * np.sin(latitude)
    return np.array([x, y, z])


def arm_unit_vector(tilt, azimuth, longitude, latitude):
    """geometry.py:51-93 (calculate_arm)."""
    e_long = np.array([-np.sin(longitude), np.cos(longitude), 0.0])
    e_lat = np.array([-np.sin(latitude) * np.cos(longitude),
                      -np.sin(latitude) * np.sin(longitude), np.cos(latitude)])
    e_h = np.array([np.cos(latitude) * np.cos(longitude),
                    np.cos(latitude) * np.sin(longitude), np.sin(latitude)])
    return (np.cos(tilt) * np.cos(azimuth) * e_long
            + np.cos(tilt) * np.sin(azimuth) * e_lat + np.sin(tilt) * e_h)


def detector_tensor(x, y):
    """geometry.py:96-115."""
    return (np.outer(x, x) - np.outer(y, y)) / 2


def polarization_tensor(ra, dec, gps, psi, mode):
    """geometry.py:118-186 (plus / cross only; the hot path uses these two)."""
    gmst = greenwich_mean_sidereal_time(gps) % (2 * np.pi)
    phi = ra - gmst
    theta = np.pi / 2 - dec
    u = np.array([np.cos(phi) * np.cos(theta), np.cos(theta) * np.sin(phi), -np.sin(theta)])
    v = np.array([-np.sin(phi), np.cos(phi), 0.0])
    m = -u * np.sin(psi) - v * np.cos(psi)
    n = -u * np.cos(psi) + v * np.sin(psi)
    if mode == "plus":
        return np.outer(m, m) - np.outer(n, n)
    if mode == "cross":
        return np.outer(m, n) + np.outer(n, m)
    raise ValueError(mode)


def antenna_response(tensor, ra, dec, gps, psi, mode):
    """interferometer.py:267-301 + geometry.py:261-279 (einsum ij,ij)."""
    return np.einsum("ij,ij->", tensor, polarization_tensor(ra, dec, gps, psi, mode))


def time_delay_from_geocenter(vertex, ra, dec, gps):
    """geometry.py:282-343."""
    gmst = greenwich_mean_sidereal_time(gps) % (2 * np.pi)
    phi = ra - gmst
    theta = np.pi / 2 - dec
    omega = np.array([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)])
    return omega @ (np.zeros(3) - vertex) / 299792458.0


# ---------------------------------------------------------------------------
# detector descriptions: constants from bilby/gw/detector/detectors/*.interferometer
# ---------------------------------------------------------------------------
DETECTORS = {
    # H1.interferometer:5-14
    "H1": dict(latitude=46 + 27. / 60 + 18.528 / 3600, longitude=-(119 + 24. / 60 + 27.5657 / 3600),
               elevation=142.554, xarm_azimuth=125.9994, yarm_azimuth=215.9994,
               xarm_tilt=-6.195e-4, yarm_tilt=1.25e-5, curve="aLIGO_O4_high_asd", curve_kind="asd"),
    # L1.interferometer:5-14
    "L1": dict(latitude=30 + 33. / 60 + 46.4196 / 3600, longitude=-(90 + 46. / 60 + 27.2654 / 3600),
               elevation=-6.574, xarm_azimuth=197.7165, yarm_azimuth=287.7165,
               xarm_tilt=-3.121e-4, yarm_tilt=-6.107e-4, curve="aLIGO_O4_high_asd", curve_kind="asd"),
    # V1.interferometer:5-13 (arm tilts default to 0)
    "V1": dict(latitude=43 + 37. / 60 + 53.0921 / 3600, longitude=10 + 30. / 60 + 16.1878 / 3600,
               elevation=51.884, xarm_azimuth=70.5674, yarm_azimuth=160.5674,
               xarm_tilt=0.0, yarm_tilt=0.0, curve="AdV_psd", curve_kind="psd"),
}


def detector_geometry(name):
    """Vertex and detector tensor as ``InterferometerGeometry`` computes them
    (bilby/gw/detector/geometry.py:201-270; angles in degrees -> radians)."""
    d = DETECTORS[name]
    lat, lon = np.radians(d["latitude"]), np.radians(d["longitude"])
    x = arm_unit_vector(d["xarm_tilt"], np.radians(d["xarm_azimuth"]), lon, lat)
    y = arm_unit_vector(d["yarm_tilt"], np.radians(d["yarm_azimuth"]), lon, lat)
    return vertex_position_geocentric(lat, lon, d["elevation"]), detector_tensor(x, y)


# ---------------------------------------------------------------------------
# PSD and seeded noise           bilby/gw/detector/psd.py, core/utils/series.py
# ---------------------------------------------------------------------------
def psd_interpolant(table_frequency, table_psd):
    """psd.py:236-244: linear interpolation of the PSD, +inf outside the table."""
    return interp1d(table_frequency, table_psd, bounds_error=False, fill_value=np.inf)


def frequency_array(sampling_frequency, duration):
    """core/utils/series.py:115-134."""
    n_samples = np.round(duration * sampling_frequency)
    n_freq = int(np.round(n_samples / 2) + 1)
    return np.linspace(0, sampling_frequency / 2, num=n_freq)


def noise_realisation(rng, table_frequency, table_psd, n_freq, duration):
    """psd.py:350-376 + core/utils/series.py:161-198.

    ``rng`` is the shared numpy Generator (bilby's global ``random.rng``).
    """
    freqs = np.arange(n_freq) / duration
    norm1 = 0.5 * duration ** 0.5
    re1, im1 = rng.normal(0, norm1, (2, len(freqs)))
    white = re1 + 1j * im1
    white[0] = 0
    white[-1] = 0
    with np.errstate(invalid="ignore"):
        strain = psd_interpolant(table_frequency, table_psd)(freqs) ** 0.5 * white
    oob = (freqs < table_frequency.min()) | (freqs > table_frequency.max())
    strain[oob] = 0j
    return np.nan_to_num(strain)


@dataclass
class Detector:
    """What the likelihood reads from one ``Interferometer``."""
    name: str
    frequency: np.ndarray          # interferometer.frequency_array
    strain: np.ndarray             # unmasked frequency-domain strain
    psd: np.ndarray                # power_spectral_density_array
    mask: np.ndarray               # strain_data.frequency_mask
    vertex: np.ndarray
    tensor: np.ndarray
    duration: float
    start_time: float

    @property
    def masked_strain(self):
        """strain_data.py:213-233: the strain is multiplied by the mask on access."""
        return self.strain * self.mask


def make_detector(name, sampling_frequency, duration, start_time, rng, curves,
                  minimum_frequency=20.0, maximum_frequency=2048.0):
    """A seeded ``Interferometer`` as ``set_strain_data_from_power_spectral_density``
    builds it (interferometer.py:157-175, strain_data.py:627-662)."""
    d = DETECTORS[name]
    tf, tv = curves[d["curve"]]
    table_psd = tv ** 2 if d["curve_kind"] == "asd" else tv
    freq = frequency_array(sampling_frequency, duration)
    strain = noise_realisation(rng, tf, table_psd, len(freq), duration)
    psd = psd_interpolant(tf, table_psd)(freq)
    fmax = min(maximum_frequency, sampling_frequency / 2)  # strain_data.py:103-110
    mask = (freq >= minimum_frequency) & (freq <= fmax)    # strain_data.py:143-159
    vertex, tensor = detector_geometry(name)
    return Detector(name, freq, strain, psd, mask, vertex, tensor, float(duration), float(start_time))


# ---------------------------------------------------------------------------
# source models
# ---------------------------------------------------------------------------
def sinegaussian(frequency_array, hrss, Q, frequency, **kwargs):
    """bilby/gw/source.py:1153-1209 (same operations, same order)."""
    tau = Q / (2.0 ** 0.5 * np.pi * frequency)
    temp = Q / (4.0 * np.pi ** 0.5 * frequency)
    fm = frequency_array - frequency
    fp = frequency_array + frequency
    negative_term = np.exp(-fm ** 2 * np.pi ** 2 * tau ** 2)
    positive_term = np.exp(-fp ** 2 * np.pi ** 2 * tau ** 2)
    h_plus = hrss * np.pi ** 0.5 * tau / 2 * (negative_term + positive_term) / (temp * (1 + np.exp(-Q ** 2))) ** 0.5
    h_cross = -1j * hrss * np.pi ** 0.5 * tau / 2 * (negative_term - positive_term) / (temp * (1 - np.exp(-Q ** 2))) ** 0.5
    return {"plus": h_plus, "cross": h_cross}


# ---------------------------------------------------------------------------
# detector projection and inner products
# ---------------------------------------------------------------------------
def detector_response(det: Detector, pols, ra, dec, geocent_time, psi):
    """interferometer.py:303-368 (identity calibration)."""
    signal = 0
    for mode, h in pols.items():
        F = antenna_response(det.tensor, ra, dec, geocent_time, psi, mode)
        signal = signal + h * det.mask * F
    shift = time_delay_from_geocenter(det.vertex, ra, dec, geocent_time)
    dt_geocent = geocent_time - det.start_time
    dt = dt_geocent + shift
    return signal * np.exp(-1j * 2 * np.pi * dt * det.frequency)


def inject(det: Detector, pols, params):
    """interferometer.py:412-510: ``strain_data.frequency_domain_strain +=
    signal`` goes through the masking getter, so the stored strain becomes
    ``strain * mask + signal``."""
    signal = detector_response(det, pols, params["ra"], params["dec"], params["geocent_time"], params["psi"])
    det.strain = det.strain * det.mask + signal


def noise_weighted_inner_product(aa, bb, psd, duration):
    """utils.py:118-138."""
    return 4 / duration * np.sum(aa.conj() * bb / psd)


def noise_log_likelihood(dets):
    """likelihood/base.py:402-411."""
    log_l = 0.0
    for d in dets:
        m = d.mask
        log_l -= abs(noise_weighted_inner_product(d.masked_strain[m], d.masked_strain[m], d.psd[m], d.duration) / 2)
    return float(log_l)


def ln_i0(x):
    """utils.py:1006-1022."""
    return np.log(i0e(x)) + np.abs(x)


# ---------------------------------------------------------------------------
# marginalisation setup        likelihood/base.py:183-223, 875-934, 994-1035
# ---------------------------------------------------------------------------
@dataclass
class Marginalization:
    time: bool = False
    phase: bool = False
    distance: bool = False
    jitter_time: bool = True
    # time
    times: np.ndarray | None = None
    delta_tc: float = 0.0
    t_min: float = 0.0
    t_max: float = 0.0
    # distance
    ref_dist: float = 0.0
    table: np.ndarray | None = None
    spline: object = None
    distance_array: np.ndarray | None = None
    distance_prior_array: np.ndarray | None = None
    extra: dict = field(default_factory=dict)


def setup_time_marginalization(m: Marginalization, start_time, duration, sampling_frequency, t_min, t_max):
    """base.py:1027-1035: times spaced 2/fs, first sample dropped."""
    m.delta_tc = 2 / sampling_frequency
    m.times = start_time + np.linspace(0, duration, int(duration / 2 * sampling_frequency + 1))[1:]
    m.t_min, m.t_max = t_min, t_max


def d_inner_h_ref_axis(n, phase_marginalization):
    """base.py:904-914."""
    if phase_marginalization:
        return np.logspace(-5, 10, n)
    n_negative = n // 2
    n_positive = n - n_negative
    return np.hstack((-np.logspace(3, -3, n_negative), np.logspace(-3, 10, n_positive)))


def optimal_snr_squared_ref_axis(n):
    """base.py:899-902."""
    return np.logspace(-5, 10, n)


def create_distance_lookup_table(distance_array, prior_array, ref_dist, phase_marginalization):
    """base.py:994-1018 (vectorised over the d_inner_h axis, same arithmetic)."""
    table = np.zeros((400, 800))
    delta_distance = distance_array[1] - distance_array[0]
    scaling = ref_dist / distance_array
    dh_full = np.outer(d_inner_h_ref_axis(800, phase_marginalization), scaling)
    hh_full = np.outer(optimal_snr_squared_ref_axis(400), scaling ** 2)
    if phase_marginalization:
        dh_full = ln_i0(abs(dh_full))
    prior_term = prior_array * delta_distance
    for ii in range(400):
        table[ii] = logsumexp(dh_full - hh_full[ii] / 2, b=prior_term, axis=-1)
    log_norm = logsumexp(0 / distance_array, b=prior_array * delta_distance)
    return table - log_norm


def setup_distance_marginalization(m: Marginalization, distance_array, prior_array, ref_dist, table=None):
    """base.py:207-223 and 916-934; the spline is scipy's interpolating
    bicubic RectBivariateSpline, -inf outside its box (core/utils/calculus.py:221-262)."""
    m.distance_array = distance_array
    m.distance_prior_array = prior_array
    m.ref_dist = ref_dist
    if table is None:
        table = create_distance_lookup_table(distance_array, prior_array, ref_dist, m.phase)
    m.table = table
    x = d_inner_h_ref_axis(table.shape[1], m.phase)
    y = optimal_snr_squared_ref_axis(table.shape[0])
    m.spline = RectBivariateSpline(x, y, table.T, kx=3, ky=3, s=0)
    m.extra["bbox"] = (x.min(), x.max(), y.min(), y.max())


def interp_distance(m: Marginalization, dh, hh):
    dh = np.atleast_1d(np.asarray(dh, dtype=np.float64))
    hh = np.broadcast_to(np.atleast_1d(np.asarray(hh, dtype=np.float64)), dh.shape)
    out = m.spline(dh, hh, grid=False)
    xmin, xmax, ymin, ymax = m.extra["bbox"]
    bad = (dh < xmin) | (dh > xmax) | (hh < ymin) | (hh > ymax)
    out = np.asarray(out, dtype=np.float64)
    out[bad] = -np.inf
    return out


# ---------------------------------------------------------------------------
# the likelihood ratio
# ---------------------------------------------------------------------------
def snrs(det: Detector, pols, params, time_marginalization=False):
    """base.py:260-354 (no calibration marginalisation)."""
    signal = detector_response(det, pols, params["ra"], params["dec"], params["geocent_time"], params["psi"])
    m = det.mask
    d = det.masked_strain
    d_inner_h = noise_weighted_inner_product(signal[m], d[m], det.psd[m], det.duration)
    hh = noise_weighted_inner_product(signal[m], signal[m], det.psd[m], det.duration).real
    dh_array = None
    if time_marginalization:
        dh_array = 4 / det.duration * np.fft.fft(signal[0:-1] * d.conj()[0:-1] / det.psd[0:-1])
    return d_inner_h, hh, dh_array


def log_likelihood_ratio(dets, source, params, marg: Marginalization | None = None, prior_geocent=None):
    """base.py:419-477, 775-820.

    ``source`` maps (frequency_array, **params) -> {"plus","cross"} and is
    evaluated on the first detector's grid (the WaveformGenerator grid).
    ``prior_geocent`` is a callable giving the geocent_time prior density.
    """
    marg = marg or Marginalization()
    params = dict(params)
    pols = source(dets[0].frequency, **params)
    if marg.time and marg.jitter_time:
        params["geocent_time"] = params["geocent_time"] + params["time_jitter"]
    dh = 0j
    hh = 0.0
    dh_arr = None
    for det in dets:
        a, b, c = snrs(det, pols, params, marg.time)
        dh = dh + a
        hh = hh + b
        if c is not None:
            dh_arr = c if dh_arr is None else dh_arr + c
    return _combine(dh, hh, dh_arr, params, marg, prior_geocent)


def _distance(marg, dh, hh, params):
    """base.py:775-784 and _setup_rho base.py:879-885."""
    hh_ref = hh * params["luminosity_distance"] ** 2 / marg.ref_dist ** 2.
    dh_ref = dh * params["luminosity_distance"] / marg.ref_dist
    dh_ref = abs(dh_ref) if marg.phase else dh_ref.real
    return interp_distance(marg, dh_ref, hh_ref)


def _combine(dh, hh, dh_arr, params, marg: Marginalization, prior_geocent):
    if marg.time:
        times = marg.times
        if marg.jitter_time:
            times = marg.times + params["time_jitter"]
        tmask = (times >= marg.t_min) & (times <= marg.t_max)
        times = times[tmask]
        arr = dh_arr[tmask]
        prior = prior_geocent(times) * marg.delta_tc
        if marg.distance:
            l_tc = _distance(marg, arr, hh, params)
        elif marg.phase:
            l_tc = ln_i0(abs(arr)) - hh / 2
        else:
            l_tc = arr.real - hh / 2
        return float(logsumexp(l_tc, b=prior))
    if marg.distance:
        return float(_distance(marg, np.atleast_1d(dh), hh, params)[0])
    if marg.phase:
        return float(ln_i0(abs(dh)) - hh / 2)
    return float(np.real(dh) - hh / 2)


def plain_terms(dets, source, params):
    """(Re<d|h>, <h|h>) summed over detectors: the two terms of the plain lnL."""
    pols = source(dets[0].frequency, **params)
    dh, hh = 0j, 0.0
    for det in dets:
        a, b, _ = snrs(det, pols, params)
        dh += a
        hh += b
    return dh, hh


def parity_scale(dh, hh):
    """Scale used to turn the absolute lnL difference into a relative one."""
    return max(1.0, abs(np.real(dh)), abs(hh) / 2)


def gps_split(x):
    return math.floor(x), x - math.floor(x)
