"""Drop-in GPU ``MBGravitationalWaveTransient`` (multi-banded likelihood).

Same constructor and methods as
``bilby.gw.likelihood.MBGravitationalWaveTransient``
(bilby/gw/likelihood/multiband.py:18-844, after Morisaki, arXiv:2104.07813).
The set-up -- frequency bands from the 0PN time to merger, the banded
frequencies, smoothing windows, and the linear coefficients (FFT down-sampling
of d/S) and quadratic coefficients (linear interpolation of |h|^2) -- runs once
on the host in float64.  Every likelihood evaluation then runs on the GPU: one
warp per parameter point evaluates the model at the banded frequencies and
contracts it with the coefficients (``k_multiband``, behind
``gwl_set_multiband`` in include/gwlnl.h).

With time marginalisation (multiband.py:714-726, 792-800) the float64
time-marginalised kernel scatters the banded strain times the linear
coefficients to the full-resolution grid, transforms it and marginalises
over time (``gwl_set_multiband_time_marginalization``).

With ``linear_interpolation=False`` <h|h> is the reference's IFFT-FFT sum
(multiband.py:613-650, 760-779): band 0 by direct weights, each later band b
by an inverse FFT of sqrt(w) h over M_b samples, zero-padding to 2 M_b and an
FFT weighted by the band's truncated inverse-PSD spectrum I_b.  Its even bins
equal the banded values themselves, so their weights join the quadratic
coefficients; the odd bins run on the GPU as one packed complex transform
per point, detector pair and band (``k_mb_hh_fft``, behind
``gwl_set_multiband_ifft_fft``).

Weights files need h5py, as in the reference.
"""
from __future__ import annotations

import logging
import math
import numbers

import numpy as np

from .likelihood import GravitationalWaveTransient

logger = logging.getLogger("bilby")

# bilby/core/utils/constants.py
SPEED_OF_LIGHT = 299792458.0
SOLAR_MASS = 1.988409870698050731911960804878414216e30
RADIUS_OF_EARTH = 6378136.6
GRAVITATIONAL_CONSTANT = 6.6743e-11

WEIGHT_KEYS = ["reference_chirp_mass", "highest_mode", "linear_interpolation", "accuracy_factor", "time_offset",
               "delta_f_end", "maximum_banding_frequency", "minimum_banding_duration", "durations", "fb_dfb", "Nbs",
               "Mbs", "Ks_Ke", "banded_frequency_points", "start_end_idxs", "unique_to_original_frequencies",
               "linear_coeffs", "quadratic_coeffs"]


def _power_of_two_at_least(x):
    """The smallest power of two >= x (bilby/core/utils/calculus.py:302-314)."""
    return 2 ** math.ceil(np.log2(x))


def scatter_lists(full_index, start_end_idxs, n):
    """For each full-resolution index k < n, the banded points scattered
    there by multiband.py:794-798 (``full_d_h[idx[band]] += values[band]``,
    band by band), as (index_start [n + 1], source): source codes j >= 0
    contribute; within one band a later point at the same index replaces an
    earlier one (numpy's buffered indexed +=), and the replaced point j is
    listed as -j - 1 (it still enters <h|h>).  Across bands the values add, in
    band order."""
    full = np.asarray(full_index, dtype=np.int64)
    if full.size and (full.min() < 0 or full.max() >= n):
        raise ValueError("a banded frequency maps outside the time-marginalisation FFT")
    code = np.arange(len(full), dtype=np.int64)
    for s0, e0 in np.asarray(start_end_idxs):
        seg = full[s0:e0 + 1]
        _, last = np.unique(seg[::-1], return_index=True)
        keep = np.zeros(len(seg), dtype=bool)
        keep[len(seg) - 1 - last] = True
        code[s0:e0 + 1][~keep] = -code[s0:e0 + 1][~keep] - 1
    order = np.argsort(full, kind="stable")
    ptr = np.zeros(n + 1, dtype=np.int64)
    ptr[1:] = np.cumsum(np.bincount(full, minlength=n))
    return ptr.astype(np.int32), code[order].astype(np.int32)


class MBGravitationalWaveTransient(GravitationalWaveTransient):
    """Multi-banded likelihood on the GPU (bilby/gw/likelihood/multiband.py:99-130)."""

    def __init__(self, interferometers, waveform_generator, reference_chirp_mass=None, highest_mode=2,
                 linear_interpolation=True, accuracy_factor=5, time_offset=None, delta_f_end=None,
                 maximum_banding_frequency=None, minimum_banding_duration=0., weights=None,
                 distance_marginalization=False, phase_marginalization=False, priors=None,
                 time_marginalization=False, jitter_time=True, distance_marginalization_lookup_table=None,
                 reference_frame="sky", time_reference="geocenter", precision="fp64"):
        self._mb = None
        self._mb_fft = None
        self._mb_tm = None
        super().__init__(interferometers, waveform_generator, priors=priors,
                         time_marginalization=time_marginalization,
                         distance_marginalization=distance_marginalization,
                         phase_marginalization=phase_marginalization,
                         distance_marginalization_lookup_table=distance_marginalization_lookup_table,
                         jitter_time=jitter_time, reference_frame=reference_frame, time_reference=time_reference,
                         precision=precision)
        if weights is None:
            self.reference_chirp_mass = reference_chirp_mass
            self.highest_mode = highest_mode
            self.linear_interpolation = linear_interpolation
            self.accuracy_factor = accuracy_factor
            self.time_offset = time_offset
            self.delta_f_end = delta_f_end
            self.maximum_banding_frequency = maximum_banding_frequency
            self.minimum_banding_duration = minimum_banding_duration
            self.setup_multibanding()
        else:
            if isinstance(weights, str):
                import h5py  # as in the reference; not needed for dict weights
                from bilby.core.utils import recursively_load_dict_contents_from_group  # type: ignore
                with h5py.File(weights, "r") as f:
                    weights = recursively_load_dict_contents_from_group(f, "/")
            self.setup_multibanding_from_weights(weights)
        if self.time_marginalization:
            self._setup_time_marginalization_multiband()
        self._upload()

    # ------------------------------------------------------------------
    # parameters of the banding (multiband.py:133-318)
    # ------------------------------------------------------------------
    @property
    def _ifo_duration(self):
        return float(self.interferometers[0].strain_data.duration)

    @property
    def _ifo_start_time(self):
        return float(self.interferometers[0].strain_data.start_time)

    @property
    def reference_chirp_mass(self):
        return self._reference_chirp_mass

    @reference_chirp_mass.setter
    def reference_chirp_mass(self, value):
        if isinstance(value, numbers.Number):
            self._reference_chirp_mass = value
            return
        minimum = getattr(self.priors, "minimum_chirp_mass", None) if self.priors is not None else None
        if minimum is None:
            raise TypeError("reference_chirp_mass is needed: the priors do not give a minimum chirp mass")
        self._reference_chirp_mass = minimum

    @property
    def reference_chirp_mass_in_second(self):
        return GRAVITATIONAL_CONSTANT * self._reference_chirp_mass * SOLAR_MASS / SPEED_OF_LIGHT ** 3.

    @property
    def highest_mode(self):
        return self._highest_mode

    @highest_mode.setter
    def highest_mode(self, value):
        if not isinstance(value, numbers.Number):
            raise TypeError("highest_mode must be a number")
        self._highest_mode = value

    @property
    def linear_interpolation(self):
        return self._linear_interpolation

    @linear_interpolation.setter
    def linear_interpolation(self, value):
        if not isinstance(value, (bool, np.bool_)):
            raise TypeError("linear_interpolation must be a bool")
        self._linear_interpolation = value

    @property
    def accuracy_factor(self):
        return self._accuracy_factor

    @accuracy_factor.setter
    def accuracy_factor(self, value):
        if not isinstance(value, numbers.Number):
            raise TypeError("accuracy_factor must be a number")
        self._accuracy_factor = value

    def _time_safety(self):
        return RADIUS_OF_EARTH / SPEED_OF_LIGHT * (1 if self.time_reference == "geocent" else 2)

    @property
    def time_offset(self):
        return self._time_offset

    @time_offset.setter
    def time_offset(self, value):
        key = self.time_reference + "_time"
        if value is not None:
            if not isinstance(value, numbers.Number):
                raise TypeError("time_offset must be a number")
            self._time_offset = value
        elif self.priors is not None and key in self.priors and hasattr(self.priors[key], "minimum"):
            self._time_offset = (self._ifo_start_time + self._ifo_duration - self.priors[key].minimum
                                 + self._time_safety())
        else:
            self._time_offset = 2.12
            logger.warning(f"time offset can not be inferred. Use the standard time offset of {self._time_offset} "
                           "seconds.")

    @property
    def delta_f_end(self):
        return self._delta_f_end

    @delta_f_end.setter
    def delta_f_end(self, value):
        key = self.time_reference + "_time"
        if value is not None:
            if not isinstance(value, numbers.Number):
                raise TypeError("delta_f_end must be a number")
            self._delta_f_end = value
        elif self.priors is not None and key in self.priors and hasattr(self.priors[key], "maximum"):
            self._delta_f_end = 100 / (self._ifo_start_time + self._ifo_duration - self.priors[key].maximum
                                       - self._time_safety())
        else:
            self._delta_f_end = 53.
            logger.warning(f"delta_f_end can not be inferred. Use the standard delta_f_end of {self._delta_f_end} Hz.")

    @property
    def maximum_banding_frequency(self):
        return self._maximum_banding_frequency

    @maximum_banding_frequency.setter
    def maximum_banding_frequency(self, value):
        # where f - 1/sqrt(-dtau/df) stops increasing (0PN)
        fmax = ((15 / 968) ** (3 / 5) * (self.highest_mode / (2 * np.pi)) ** (8 / 5)
                / self.reference_chirp_mass_in_second)
        if value is not None:
            if not isinstance(value, numbers.Number):
                raise TypeError("maximum_banding_frequency must be a number")
            if value < fmax:
                fmax = value
            else:
                logger.warning(f"The input maximum_banding_frequency is too large. It is set to be {fmax} Hz.")
        self._maximum_banding_frequency = fmax

    @property
    def minimum_banding_duration(self):
        return self._minimum_banding_duration

    @minimum_banding_duration.setter
    def minimum_banding_duration(self, value):
        if not isinstance(value, numbers.Number):
            raise TypeError("minimum_banding_duration must be a number")
        self._minimum_banding_duration = value

    @property
    def minimum_frequency(self):
        return np.min([i.minimum_frequency for i in self.interferometers])

    @property
    def maximum_frequency(self):
        return np.max([i.maximum_frequency for i in self.interferometers])

    @property
    def number_of_bands(self):
        return len(self.durations)

    # ------------------------------------------------------------------
    # set-up (host, float64)
    # ------------------------------------------------------------------
    def setup_multibanding(self):
        """multiband.py:317-326."""
        self._setup_frequency_bands()
        self._setup_integers()
        self._setup_waveform_frequency_points()
        self._setup_linear_coefficients()
        if self.linear_interpolation:
            self._setup_quadratic_coefficients_linear_interp()
        else:
            self._setup_quadratic_coefficients_ifft_fft()

    def _tau(self, f):
        """0PN time to merger (multiband.py:328-344)."""
        mc = self.reference_chirp_mass_in_second
        return 5 / 256 * mc * (np.pi * mc * (2 * f / self.highest_mode)) ** (-8 / 3)

    def _dtaudf(self, f):
        """Its frequency derivative (multiband.py:346-365)."""
        mc = self.reference_chirp_mass_in_second
        return -5 / 96 * mc * (np.pi * mc * (2 * f / self.highest_mode)) ** (-8. / 3.) / f

    def _find_starting_frequency(self, duration, fnow):
        """Bisection for the next band's start, conditions (10) and (51) of
        arXiv:2104.07813 (multiband.py:367-401)."""
        def above(f):
            cond1 = (duration - self.time_offset - self._tau(f)
                     - self.accuracy_factor * np.sqrt(-self._dtaudf(f))) > 0
            cond2 = f - 1. / np.sqrt(-self._dtaudf(f)) - fnow > 0
            return cond1 and cond2
        lo, hi = fnow, self.maximum_banding_frequency
        if not above(hi):
            return None, None
        while hi - lo > 1e-2 / duration:
            f = (lo + hi) / 2.
            if above(f):
                hi = f
            else:
                lo = f
        return f, 1. / np.sqrt(-self._dtaudf(f))

    def _setup_frequency_bands(self):
        """Durations T, T/2, T/4, ... and (start, smoothing scale) of each band
        (multiband.py:403-427)."""
        durations = [self._ifo_duration]
        fb = [[self.minimum_frequency, 0.]]
        dnext = self._ifo_duration / 2
        while dnext > max(self.time_offset, self.minimum_banding_duration):
            fnext, dfnext = self._find_starting_frequency(dnext, fb[-1][0])
            if fnext is not None and fnext < min(self.maximum_frequency, self.maximum_banding_frequency):
                durations.append(dnext)
                fb.append([fnext, dfnext])
                dnext /= 2
            else:
                break
        fb.append([self.maximum_frequency + self.delta_f_end, self.delta_f_end])
        self.durations = np.array(durations)
        self.fb_dfb = np.array(fb)

    def _setup_integers(self):
        """N^(b), M^(b) and the index range [K_s, K_e] of each band (multiband.py:429-449)."""
        T = self._ifo_duration
        nbs, mbs, ks_ke = [], [], []
        for b in range(self.number_of_bands):
            d = self.durations[b]
            fnow, dfnow = self.fb_dfb[b]
            fnext = self.fb_dfb[b + 1][0]
            nb = max(_power_of_two_at_least(2. * (fnext * T + 1.)), 2 ** b)
            nbs.append(nb)
            mbs.append(nb // 2 ** b)
            ks_ke.append([math.ceil((fnow - dfnow) * d), math.floor(fnext * d)])
        self.Nbs = np.array(nbs, dtype=int)
        self.Mbs = np.array(mbs, dtype=int)
        self.Ks_Ke = np.array(ks_ke)

    def _setup_waveform_frequency_points(self):
        """The banded frequencies k / T^(b), K_s <= k <= K_e, band after band
        (multiband.py:451-481)."""
        pts, se = [], []
        start = 0
        for b in range(self.number_of_bands):
            ks, ke = self.Ks_Ke[b]
            pts.append(np.arange(ks, ke + 1) / self.durations[b])
            se.append([start, start + ke - ks])
            start += ke - ks + 1
        self.banded_frequency_points = np.concatenate(pts)
        self.start_end_idxs = np.array(se)
        unique, inverse = np.unique(self.banded_frequency_points, return_inverse=True)
        self.waveform_generator.waveform_arguments["frequencies"] = unique
        self.unique_to_original_frequencies = inverse

    def _window(self, delta_f, start_idx, length, b):
        """Smoothing window of band b on the grid (start_idx + j) delta_f
        (multiband.py:483-528): cosine ramps over [f_b - df_b, f_b] and
        [f_{b+1} - df_{b+1}, f_{b+1}], one in between."""
        fnow, dfnow = self.fb_dfb[b]
        fnext, dfnext = self.fb_dfb[b + 1]
        w = np.zeros(length)
        up0 = int(np.clip(math.floor((fnow - dfnow) / delta_f) - start_idx + 1, 0, length))
        one0 = int(np.clip(math.ceil(fnow / delta_f) - start_idx, 0, length))
        down0 = int(np.clip(math.floor((fnext - dfnext) / delta_f) - start_idx + 1, 0, length))
        down1 = int(np.clip(math.ceil(fnext / delta_f) - start_idx, 0, length))
        w[one0:down0] = 1.
        if up0 < one0:
            f = (np.arange(up0, one0) + start_idx) * delta_f
            w[up0:one0] = (1. + np.cos(np.pi * (f - fnow) / dfnow)) / 2.
        if down0 < down1:
            f = (np.arange(down0, down1) + start_idx) * delta_f
            w[down0:down1] = (1. - np.cos(np.pi * (f - fnext) / dfnext)) / 2.
        return w

    def _setup_linear_coefficients(self):
        """(4 / T^(b)) w conj(d~^(b)) with d~^(b) the masked d/S down-sampled to
        band b by an inverse FFT, truncation to the last M^(b) samples and an
        FFT (multiband.py:530-550)."""
        N = self.Nbs[-1]
        self.linear_coeffs = dict()
        for ifo in self.interferometers:
            mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
            d_over_s = np.zeros(N // 2 + 1, dtype=complex)
            n = min(len(mask), len(d_over_s))
            src = np.zeros(len(mask), dtype=complex)
            src[mask] = (np.asarray(ifo.strain_data.frequency_domain_strain)[mask]
                         / np.asarray(ifo.power_spectral_density_array)[mask])
            d_over_s[:n] = src[:n]
            parts = []
            for b in range(self.number_of_bands):
                ks, ke = self.Ks_Ke[b]
                w = self._window(1. / self.durations[b], ks, ke - ks + 1, b)
                band = np.copy(d_over_s[:int(self.Nbs[b] / 2 + 1)])
                band[-1] = 0.
                td = np.fft.irfft(band)[-self.Mbs[b]:]
                parts.append((4. / self.durations[b]) * w * np.conj(np.fft.rfft(td)[ks:ke + 1]))
            self.linear_coeffs[ifo.name] = np.concatenate(parts)

    def _setup_quadratic_coefficients_linear_interp(self):
        """Weights of |h(f_k)|^2 such that linear interpolation of |h|^2 between
        banded frequencies, times w/S, summed over the original grid gives
        <h|h> (multiband.py:552-601).  Each interval's grid points are summed
        as one segment."""
        T = float(self._ifo_duration)
        self.quadratic_coeffs = dict((ifo.name, []) for ifo in self.interferometers)
        for b in range(self.number_of_bands):
            s, e = self.start_end_idxs[b]
            fk = self.banded_frequency_points[s:e + 1]
            pref = 4 * self.durations[b] / T
            fnow, dfnow = self.fb_dfb[b]
            fnext = self.fb_dfb[b + 1][0]
            i0 = math.ceil((fnow - dfnow) * T)
            w = self._window(1 / T, i0, math.floor(fnext * T) - i0 + 1, b)
            nk = len(fk)
            # grid-index range of each interval [f_k, f_{k+1}]
            lo = np.ceil(T * fk[:-1]).astype(np.int64)
            hi = np.ceil(T * fk[1:]).astype(np.int64) - 1
            for ifo in self.interferometers:
                psd = np.asarray(ifo.power_spectral_density_array)
                i1 = min(i0 + len(w) - 1, len(psd) - 1)
                m = np.asarray(ifo.strain_data.frequency_mask[i0:i1 + 1], dtype=bool)
                wp = np.zeros(i1 + 1 - i0)
                wp[m] = 1. / psd[i0:i1 + 1][m]
                wp *= w[:len(wp)]
                a = np.maximum(lo, i0)
                a[0] = i0
                z = np.minimum(hi, i1)
                z[-1] = i1
                coeffs = np.zeros(nk)
                grid = np.arange(i0, i1 + 1) / T
                for k in range(nk - 1):
                    if z[k] < a[k]:
                        continue
                    seg = wp[a[k] - i0:z[k] - i0 + 1]
                    f = grid[a[k] - i0:z[k] - i0 + 1]
                    coeffs[k] += pref * np.sum((fk[k + 1] - f) * seg)
                    coeffs[k + 1] += pref * np.sum((f - fk[k]) * seg)
                self.quadratic_coeffs[ifo.name].append(coeffs)
        for name in self.quadratic_coeffs:
            self.quadratic_coeffs[name] = np.concatenate(self.quadratic_coeffs[name])

    def _setup_quadratic_coefficients_ifft_fft(self):
        """multiband.py:613-650: per band the zero-padded length
        Nhat_b = min(2 M_b, N_b) and duration That_b = T Nhat_b / N_b, and per
        detector I_b = rfft of the inverse PSD's inverse FFT at N_b samples
        truncated to lags |n| <= Nhat_b / 2 (wrapped to Nhat_b samples); the
        band windows and their square roots."""
        N = int(self.Nbs[-1])
        nhat = [min(2 * int(mb), int(nb)) for mb, nb in zip(self.Mbs, self.Nbs)]
        self.Tbhats = [self._ifo_duration * nh / int(nb) for nb, nh in zip(self.Nbs, nhat)]
        self.Ibcs = dict((ifo.name, []) for ifo in self.interferometers)
        self.hbcs = dict((ifo.name, []) for ifo in self.interferometers)
        self.wths = dict((ifo.name, []) for ifo in self.interferometers)
        for ifo in self.interferometers:
            psd = np.asarray(ifo.power_spectral_density_array)
            mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
            inv = np.zeros(N // 2 + 1)
            n = min(len(psd), len(inv))
            m = mask[:n]
            inv[:n][m] = 1.0 / psd[:n][m]
            for b in range(self.number_of_bands):
                imb = np.fft.irfft(inv[:int(self.Nbs[b]) // 2 + 1])
                h = nhat[b] // 2
                self.Ibcs[ifo.name].append(np.fft.rfft(np.concatenate([imb[:h + 1], imb[len(imb) - (nhat[b] - h - 1):]])))
                self.hbcs[ifo.name].append(np.zeros(nhat[b]))
                self.wths[ifo.name].append(np.zeros(int(self.Mbs[b]) // 2 + 1, dtype=complex))
        ws = []
        for b in range(self.number_of_bands):
            ks, ke = self.Ks_Ke[b]
            ws.append(self._window(1. / self.durations[b], ks, ke - ks + 1, b))
        self.windows = np.concatenate(ws)
        self.square_root_windows = np.sqrt(self.windows)

    def _ifft_fft_tables(self):
        """The GPU form of the IFFT-FFT <h|h> (multiband.py:760-779): the
        quadratic coefficients [n_det, K] (band 0: (4/T) mask w / S; band
        b >= 1: the even bins, (4/That_b) w_k Re I_b[2 m_k] at grid index
        m_k = K_s + k - k_b), and per band b >= 1 K_s, M_b, 4 / That_b and the
        odd-bin weights Re I_b[2j + 1], j < M_b / 2."""
        T = float(self._ifo_duration)
        nb = self.number_of_bands
        quad = np.zeros((len(self.interferometers), len(self.banded_frequency_points)))
        odd = [[] for _ in self.interferometers]
        ks_out, m_out, scale = np.zeros(nb, dtype=np.int32), np.zeros(nb, dtype=np.int32), np.zeros(nb)
        for b in range(nb):
            ks, ke = (int(x) for x in self.Ks_Ke[b])
            s, e = (int(x) for x in self.start_end_idxs[b])
            w = np.asarray(self.windows[s:e + 1])
            for q, ifo in enumerate(self.interferometers):
                if b == 0:
                    psd = np.asarray(ifo.power_spectral_density_array)
                    mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
                    with np.errstate(divide="ignore", invalid="ignore"):
                        quad[q, s:e + 1] = (4. / T) * mask[ks:ke + 1] * w / psd[ks:ke + 1]
                else:
                    ibc = np.asarray(self.Ibcs[ifo.name][b]).real
                    quad[q, s:e + 1] = (4. / self.Tbhats[b]) * w * ibc[2 * np.arange(ks, ke + 1)]
                    odd[q].append(ibc[1::2][:int(self.Mbs[b]) // 2])
            if b > 0:
                mb = int(self.Mbs[b])
                if 2 * mb != min(2 * mb, int(self.Nbs[b])) or ks < 1 or ke >= mb // 2:
                    raise ValueError(f"band {b}: the IFFT-FFT <h|h> needs Nhat = 2 M and 1 <= K_s <= K_e < M / 2")
                ks_out[b], m_out[b], scale[b] = ks, mb, 4. / self.Tbhats[b]
        odd = np.stack([np.concatenate(o) if o else np.zeros(0) for o in odd])
        return quad, (ks_out, m_out, scale, np.asarray(self.square_root_windows, dtype=np.float64), odd)

    @property
    def weights(self):
        """multiband.py:652-671."""
        keys = WEIGHT_KEYS if self.linear_interpolation else [k for k in WEIGHT_KEYS if k != "quadratic_coeffs"]
        out = {key: getattr(self, key) for key in keys}
        out["waveform_frequencies"] = self.waveform_generator.waveform_arguments["frequencies"]
        if not self.linear_interpolation:
            for key in ("Tbhats", "windows", "square_root_windows"):
                out[key] = getattr(self, key)
            for key in ("wths", "hbcs", "Ibcs"):
                out[key] = {name: dict((str(b), v) for b, v in enumerate(data))
                            for name, data in getattr(self, key).items()}
        return out

    def setup_multibanding_from_weights(self, weights):
        """multiband.py:687-712."""
        weights = dict(weights)
        self.reference_chirp_mass = weights.pop("reference_chirp_mass")
        for key, value in weights.items():
            if key == "waveform_frequencies":
                self.waveform_generator.waveform_arguments["frequencies"] = value
            elif key in ("wths", "hbcs", "Ibcs"):
                setattr(self, key, {name: [data[str(b)] for b in range(len(data))] for name, data in value.items()})
            elif key in ("highest_mode", "linear_interpolation", "accuracy_factor", "time_offset", "delta_f_end",
                         "maximum_banding_frequency", "minimum_banding_duration"):
                setattr(self, "_" + key, value)
            else:
                setattr(self, key, value)

    def _setup_time_marginalization_multiband(self):
        """multiband.py:714-726: an FFT of length Nbs[-1] / 2 on the time
        grid start + j T / N, the banded points' full-resolution indices, and
        the antenna patterns fixed at the middle of the geocent_time prior
        (set on the interferometers, as the reference does)."""
        n = int(self.Nbs[-1]) // 2
        self._delta_tc = self.durations[0] / n
        self._times = self._ifo_start_time + np.arange(n) * self._delta_tc
        self.time_prior_array = self.priors["geocent_time"].prob(self._times) * self._delta_tc
        self._full_to_multiband = [int(f * self.durations[0]) for f in self.banded_frequency_points]
        tp = self.priors["geocent_time"]
        self._beam_pattern_reference_time = (tp.minimum + tp.maximum) / 2
        for ifo in self.interferometers:
            ifo.reference_time = self._beam_pattern_reference_time
        ptr, src = scatter_lists(self._full_to_multiband, self.start_end_idxs, n)
        self._mb_tm = (n, ptr, src, float(self._delta_tc), float(self._beam_pattern_reference_time))

    def _detector_analysis(self, interferometer):
        """A one-detector analysis with this detector's coefficients (and the
        time-marginalisation tables): calculate_snrs then gives the
        multi-banded inner products of multiband.py:728-807."""
        name = interferometer.name
        an = self._detector_analyses.get(name)
        if an is None:
            names = [ifo.name for ifo in self.interferometers]
            if name not in names:
                raise ValueError(f"interferometer {name} is not part of this likelihood")
            k = names.index(name)
            an = self._new_analysis([self.interferometers[k]])
            if self.time_marginalization:
                tp = self.priors["geocent_time"]
                an.set_time_marginalization(True, False, tp.minimum, tp.maximum)
            freqs, lin, quad, band_start, band_df = self._mb
            an.set_multiband(True, freqs, lin[k:k + 1], quad[k:k + 1], band_start, band_df)
            if self._mb_fft is not None:
                ks, m, scale, sw, odd = self._mb_fft
                an.set_multiband_ifft_fft(True, ks, m, scale, sw, odd[k:k + 1])
            if self._mb_tm is not None:
                an.set_multiband_time_marginalization(*self._mb_tm)
            self._detector_analyses[name] = an
        return an

    def generate_time_sample_from_marginalized_likelihood(self, signal_polarizations=None, *, parameters):
        """multiband.py:822-855: a draw from the time posterior on the
        marginalisation grid, from the GPU's <d|h>(t) summed over detectors,
        with numpy's global generator as the reference uses."""
        parameters.update(self.get_sky_frame_parameters(parameters))
        total = self._CalculatedSNRs()
        for ifo in self.interferometers:
            total += self.calculate_snrs(signal_polarizations, ifo, parameters=parameters)
        d_inner_h, h_inner_h = total.d_inner_h_array, total.optimal_snr_squared
        if self.distance_marginalization:
            lnl_t = self.distance_marginalized_likelihood(d_inner_h, h_inner_h, parameters=parameters)
        elif self.phase_marginalization:
            lnl_t = self.phase_marginalized_likelihood(d_inner_h, h_inner_h)
        else:
            lnl_t = d_inner_h.real - h_inner_h / 2
        times = self._times
        if self.jitter_time:
            times = times + parameters["time_jitter"]
        post = np.exp(lnl_t - np.max(lnl_t)) * self.priors["geocent_time"].prob(times)
        post /= np.sum(post)
        return np.random.choice(times, p=post)

    def _upload(self):
        names = [ifo.name for ifo in self.interferometers]
        lin = np.stack([np.asarray(self.linear_coeffs[n]) for n in names])
        if self.linear_interpolation:
            quad = np.stack([np.asarray(self.quadratic_coeffs[n]) for n in names])
            self._mb_fft = None
        else:
            quad, self._mb_fft = self._ifft_fft_tables()
        band_start = np.append(np.asarray(self.start_end_idxs)[:, 0], np.asarray(self.start_end_idxs)[-1, 1] + 1)
        self._mb = (np.asarray(self.banded_frequency_points, dtype=np.float64), lin, quad, band_start,
                    1.0 / np.asarray(self.durations, dtype=np.float64))
        self._set_bands(self.analysis)

    def _set_bands(self, an):
        an.set_multiband(True, *self._mb)
        if self._mb_fft is not None:
            an.set_multiband_ifft_fft(True, *self._mb_fft)
        if self._mb_tm is not None:
            an.set_multiband_time_marginalization(*self._mb_tm)

    def _build_analysis(self):
        super()._build_analysis()
        if getattr(self, "_mb", None) is not None:
            self._set_bands(self._analysis)
