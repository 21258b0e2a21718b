"""Host-side sky-frame conversions of ``get_sky_frame_parameters``
(bilby/gw/likelihood/base.py:1091-1137): detector-frame zenith/azimuth to
ra/dec (bilby/gw/utils.py:232-256, bilby/gw/geometry.py:185-232, 346-377,
bilby/core/utils/conversion.py:27-30) and a detector's arrival time to the
geocentre time (geometry.py:282-343).  Vectorised float64 numpy: these run
once per point as parameter preparation, before the GPU launch."""
from __future__ import annotations

import numpy as np

_LEAP = np.array([46828800, 78364801, 109900802, 173059203, 252028804, 315187205, 346723206, 393984007,
                  425520008, 457056009, 504489610, 551750411, 599184012, 820108813, 914803214, 1025136015,
                  1119744016, 1167264017], dtype=np.float64)


def greenwich_mean_sidereal_time(gps):
    """bilby/gw/time.py:114-165 (radians, unreduced)."""
    gps = np.asarray(gps, dtype=np.float64)
    gi = gps // 1
    nleap = np.sum(gi[..., None] > _LEAP, axis=-1)
    jd = 723231 + (gi - nleap) / 86400.0 + 1721013.5
    t_hi = (jd - 2451545.0) / 36525.0
    t_lo = (gps % 1) / (36525.0 * 86400.0)
    t = t_hi + t_lo
    st = 0.0 + (-6.2e-6 * t + 0.093104) * t ** 2 + 67310.54841
    st = st + 8640184.812866 * t_lo
    st = st + 3155760000.0 * t_lo
    st = st + 8640184.812866 * t_hi
    st = st + 3155760000.0 * t_hi
    return st * 2 * np.pi / 86400.0


def time_delay_from_geocenter(vertex, ra, dec, gps):
    gmst = greenwich_mean_sidereal_time(gps) % (2 * np.pi)
    phi = np.asarray(ra) - gmst
    theta = np.pi / 2 - np.asarray(dec)
    omega = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)])
    return np.tensordot(np.zeros(3) - np.asarray(vertex), omega, axes=(0, 0)) / 299792458.0


def rotation_matrix_from_delta(delta_x):
    """geometry.py:185-232."""
    delta_x = delta_x / (delta_x ** 2).sum() ** 0.5
    alpha = np.arctan2(-delta_x[1] * delta_x[2], delta_x[0])
    beta = np.arccos(delta_x[2])
    gamma = np.arctan2(delta_x[1], delta_x[0])
    r1 = np.array([[np.cos(alpha), -np.sin(alpha), 0], [np.sin(alpha), np.cos(alpha), 0], [0, 0, 1]])
    r2 = np.array([[np.cos(beta), 0, np.sin(beta)], [0, 1, 0], [-np.sin(beta), 0, np.cos(beta)]])
    r3 = np.array([[np.cos(gamma), -np.sin(gamma), 0], [np.sin(gamma), np.cos(gamma), 0], [0, 0, 1]])
    return r3 @ r2 @ r1


class ReferenceFrame:
    """The detector-pair frame of ``reference_frame`` (base.py:1062-1089)."""

    def __init__(self, frame):
        from .detector import get_empty_interferometer
        if isinstance(frame, str):
            names = [frame[:2], frame[2:4]]
            ifos = [get_empty_interferometer(n) for n in names]
        else:
            ifos = list(frame)[:2]
            ifos = [get_empty_interferometer(i) if isinstance(i, str) else i for i in ifos]
        self.ifos = ifos
        self.delta_x = np.asarray(ifos[0].geometry.vertex) - np.asarray(ifos[1].geometry.vertex)
        self.rotation = rotation_matrix_from_delta(self.delta_x)

    def zenith_azimuth_to_ra_dec(self, zenith, azimuth, geocent_time):
        zenith, azimuth = np.asarray(zenith, dtype=np.float64), np.asarray(azimuth, dtype=np.float64)
        omega_prime = np.stack([np.sin(zenith) * np.cos(azimuth), np.sin(zenith) * np.sin(azimuth), np.cos(zenith)])
        omega = np.tensordot(self.rotation, omega_prime, axes=(1, 0))
        theta = np.arccos(omega[2])
        phi = np.arctan2(omega[1], omega[0]) % (2 * np.pi)
        gmst = greenwich_mean_sidereal_time(geocent_time)
        ra = (phi + gmst) % (2 * np.pi)
        dec = np.pi / 2 - theta
        return ra, dec
