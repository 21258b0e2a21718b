"""Drop-in GPU ``ROQGravitationalWaveTransient`` (reduced-order quadrature).

Same constructor as ``bilby.gw.likelihood.ROQGravitationalWaveTransient``
(bilby/gw/likelihood/roq.py:14-215) for one linear and one quadratic basis.
The weights -- time-dependent linear weights by inverse FFTs of d/S times each
basis element, quadratic weights from 1/S (roq.py:736-1007) -- are computed
once on the host in float64, or taken from a weights dictionary; every
likelihood evaluation then runs on the GPU: one warp per parameter point
evaluates the model at the frequency nodes, contracts it with the weights of
the five time samples around each detector's arrival time and interpolates
(``k_roq``, behind ``gwl_set_roq`` in include/gwlnl.h).

With time marginalisation (roq.py:320-331, 535-541, 604-651) one CTA per
point contracts the weight rows its detector times read, interpolates <d|h>
at every sample of the marginalisation grid and marginalises
(``k_roq_time_marg``, behind ``gwl_set_roq_time_marginalization``).

Not built: several bases selected by prior ranges and multi-banded ROQ
weights (NotImplementedError); hdf5 files need h5py, as in the reference.
"""
from __future__ import annotations

import logging

import numpy as np

from .likelihood import GravitationalWaveTransient

logger = logging.getLogger("bilby")

SPEED_OF_LIGHT = 299792458.0
RADIUS_OF_EARTH = 6378136.6


class BilbyROQParamsRangeError(Exception):
    """roq.py:1274 (a prior or data setting outside the basis' validity)."""


class ROQGravitationalWaveTransient(GravitationalWaveTransient):
    """ROQ likelihood on the GPU (bilby/gw/likelihood/roq.py:112-213)."""

    def __init__(self, interferometers, waveform_generator, priors, weights=None, linear_matrix=None,
                 quadratic_matrix=None, roq_params=None, roq_params_check=True, roq_scale_factor=1,
                 distance_marginalization=False, phase_marginalization=False, time_marginalization=False,
                 jitter_time=True, delta_tc=None, distance_marginalization_lookup_table=None, reference_frame="sky",
                 time_reference="geocenter", parameter_conversion=None, precision="fp64"):
        self._roq = None
        self._roq_tm = None
        self._delta_tc_request = delta_tc
        super().__init__(interferometers, waveform_generator, priors=priors,
                         time_marginalization=time_marginalization,
                         distance_marginalization=distance_marginalization,
                         phase_marginalization=phase_marginalization,
                         distance_marginalization_lookup_table=distance_marginalization_lookup_table,
                         jitter_time=jitter_time, reference_frame=reference_frame, time_reference=time_reference,
                         precision=precision)
        self.roq_params_check = roq_params_check
        self.roq_scale_factor = roq_scale_factor
        self.parameter_conversion = parameter_conversion
        if isinstance(roq_params, str):
            self.roq_params_file = roq_params
            self.roq_params = np.genfromtxt(roq_params, names=True)
        elif roq_params is None or isinstance(roq_params, np.ndarray):
            self.roq_params = roq_params
        else:
            raise TypeError("roq_params should be array or str")
        if isinstance(weights, dict):
            self.weights = weights
        elif isinstance(weights, str):
            self.weights = self.load_weights(weights)
        else:
            linear = self._parse_basis(linear_matrix, "linear")
            quadratic = self._parse_basis(quadratic_matrix, "quadratic")
            if self.roq_params is not None:
                for ifo in self.interferometers:
                    self.perform_roq_params_check(ifo)
            self.weights = dict()
            self._set_weights(linear, quadratic)
        for basis_type in ("linear", "quadratic"):
            if len(self.weights[f"{self.interferometers[0].name}_{basis_type}"]) != 1:
                raise NotImplementedError("several ROQ bases (selected by prior ranges) have no GPU kernel")
            key = f"frequency_nodes_{basis_type}"
            args = self.waveform_generator.waveform_arguments
            if key not in self.weights and key not in args:
                raise AttributeError(f"{key} should be contained in weights or waveform arguments.")
            if key not in args:
                args[key] = self.weights[key][0]
            elif key not in self.weights:
                self.weights[key] = [args[key]]
        self.number_of_bases_linear = 1
        self.number_of_bases_quadratic = 1
        self._upload()

    # ------------------------------------------------------------------
    # basis and weights (host, float64)
    # ------------------------------------------------------------------
    @staticmethod
    def _parse_basis(basis, basis_type):
        """roq.py:333-366: an array (n_frequencies x n_basis) or a .npy file
        (n_basis x n_frequencies) -> {basis_<type>: {"0": {"basis": n_basis x n_frequencies}}}."""
        if isinstance(basis, str):
            fmt = basis.split(".")[-1]
            if fmt == "npy":
                return {f"basis_{basis_type}": {"0": {"basis": np.load(basis)}}}
            if fmt == "hdf5":
                raise NotImplementedError("hdf5 ROQ bases need h5py and prior-range selection")
            raise IOError(f"Format {fmt} not recognized.")
        if isinstance(basis, np.ndarray):
            return {f"basis_{basis_type}": {"0": {"basis": basis.T}}}
        raise TypeError("basis needs to be str or np.ndarray")

    def load_weights(self, filename):
        """Weights saved as .npz (roq.py:1107-1163)."""
        if not filename.endswith(".npz"):
            raise NotImplementedError("only .npz weights are supported without h5py")
        loaded = dict(np.load(filename, allow_pickle=True))
        return {k: (v.tolist() if v.dtype == object else v) for k, v in loaded.items()}

    def perform_roq_params_check(self, ifo=None):
        """roq.py:653-734: the data and priors must lie inside the basis' validity."""
        if self.roq_params_check is False:
            logger.warning("No ROQ params checking performed")
            return
        p = self.roq_params
        fmin = p["flow"] * self.roq_scale_factor
        fmax = p["fhigh"] * self.roq_scale_factor
        seglen = p["seglen"] / self.roq_scale_factor
        names = p.dtype.names or ()
        if float(ifo.maximum_frequency) > fmax:
            raise BilbyROQParamsRangeError(f"Requested maximum frequency {ifo.maximum_frequency} larger than ROQ "
                                           f"basis fhigh {fmax}")
        if float(ifo.minimum_frequency) < fmin:
            raise BilbyROQParamsRangeError(f"Requested minimum frequency {ifo.minimum_frequency} lower than ROQ "
                                           f"basis flow {fmin}")
        if float(ifo.strain_data.duration) != seglen:
            raise BilbyROQParamsRangeError(f"Requested duration differs from ROQ basis seglen {seglen}")
        if self.priors is not None and "chirp_mass" in self.priors:
            if "chirpmassmin" in names and self.priors["chirp_mass"].minimum < p["chirpmassmin"] / self.roq_scale_factor:
                raise BilbyROQParamsRangeError("Prior minimum chirp mass below the ROQ basis bound")
            if "chirpmassmax" in names and self.priors["chirp_mass"].maximum > p["chirpmassmax"] / self.roq_scale_factor:
                raise BilbyROQParamsRangeError("Prior maximum chirp mass above the ROQ basis bound")

    def _get_time_resolution(self):
        """roq.py:1165-1231: 1/5 of 1/f_high with f_high from the SNR-scaled
        third frequency moment of the (last) detector's PSD, then rounded so
        that the segment holds a power of two of samples."""
        from scipy.integrate import simpson

        def calc_fhigh(freq, psd, scaling=20.):
            i1 = simpson(y=np.power(freq, -7. / 3) / psd, x=freq)
            f3 = simpson(y=np.power(freq, 2. / 3.) / (psd * i1), x=freq)
            return scaling * f3 ** (1 / 3)

        snr_sq = 0
        for ifo in self.interferometers:
            meta = getattr(ifo, "meta_data", None) or {}
            snr_sq += max(10, meta.get("optimal_SNR", 30)) ** 2
        mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
        psd = np.asarray(ifo.power_spectral_density_array)[mask]
        freq = np.asarray(ifo.strain_data.frequency_array)[mask]
        fhigh = calc_fhigh(freq, psd, scaling=(np.pi ** 2 * snr_sq / 6) ** (1 / 3))
        delta_t = fhigh ** -1 / 5
        duration = float(self.interferometers[0].strain_data.duration)
        n = max(duration / delta_t, float(self.interferometers[0].strain_data.frequency_array[-1]) * duration + 1)
        n = int(2 ** np.ceil(np.log2(n)))
        return duration / n

    def _set_weights(self, linear_matrix, quadratic_matrix):
        """roq.py:736-1005 for one basis of each kind, no multi-banding."""
        ifos = self.interferometers
        duration = float(ifos[0].strain_data.duration)
        start_time = float(ifos[0].strain_data.start_time)
        time_space = self._get_time_resolution()
        n_time = int(duration / time_space)
        crossing = 2 * RADIUS_OF_EARTH / SPEED_OF_LIGHT + 5 * time_space
        tp = self.priors[f"{self.time_reference}_time"]
        start_idx = max(0, int(np.floor((tp.minimum - crossing - start_time) / time_space)))
        end_idx = min(n_time - 1, int(np.ceil((tp.maximum + crossing - start_time) / time_space)))
        self.weights["time_samples"] = np.arange(start_idx, end_idx + 1) * float(time_space)
        lin = np.asarray(linear_matrix["basis_linear"]["0"]["basis"])
        quad = np.asarray(quadratic_matrix["basis_quadratic"]["0"]["basis"]).real
        for key, matrix in (("linear", linear_matrix), ("quadratic", quadratic_matrix)):
            node = matrix[f"basis_{key}"]["0"]
            if "frequency_nodes" in node:
                self.weights[f"frequency_nodes_{key}"] = [np.asarray(node["frequency_nodes"]) * self.roq_scale_factor]
        for ifo in ifos:
            mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
            fm = np.asarray(ifo.strain_data.frequency_array)[mask]
            if self.roq_params is not None:
                fmax = self.roq_params["fhigh"] * self.roq_scale_factor
                seglen = self.roq_params["seglen"] / self.roq_scale_factor
                roq_f = np.linspace(0, fmax, int(np.round(fmax * seglen)) + 1)
                roq_f = roq_f[roq_f >= self.roq_params["flow"] * self.roq_scale_factor]
                _, ifo_idxs, roq_idxs = np.intersect1d(fm, roq_f, return_indices=True)
            else:
                roq_idxs = np.arange(lin.shape[1], dtype=int)
                ifo_idxs = np.arange(int(mask.sum()))
                if len(ifo_idxs) != len(roq_idxs):
                    raise ValueError(f"Mismatch between ROQ basis and frequency array for {ifo.name}")
            nonzero = ifo_idxs + int(ifo.minimum_frequency * duration)
            d_over_s = (np.asarray(ifo.strain_data.frequency_domain_strain)[mask][ifo_idxs]
                        / np.asarray(ifo.power_spectral_density_array)[mask][ifo_idxs])
            rows = []
            for c0 in range(0, lin.shape[0], 16):  # inverse FFTs of 16 basis elements at a time
                block = np.zeros((min(16, lin.shape[0] - c0), n_time), dtype=complex)
                block[:, nonzero] = d_over_s * np.conj(lin[c0:c0 + 16][:, roq_idxs])
                rows.append(np.fft.ifft(block, axis=1)[:, start_idx:end_idx + 1])
            w = np.concatenate(rows).T * (4. * n_time / duration)
            self.weights[ifo.name + "_linear"] = [w]
            inv_psd = 1 / np.asarray(ifo.power_spectral_density_array)[mask][ifo_idxs]
            self.weights[ifo.name + "_quadratic"] = [4. / duration * quad[:, roq_idxs] @ inv_psd]

    def _setup_time_marginalization(self):
        """roq.py:320-331: delta_tc from the constructor or the ROQ time
        resolution, shrunk so that it divides the geocent_time prior; the
        samples sit at the middles of the intervals; the antenna patterns and
        delays are taken at the prior's mid time."""
        tp = self.priors["geocent_time"]
        if type(tp).__name__ != "Uniform":
            raise NotImplementedError("time marginalisation on the GPU needs a Uniform geocent_time prior")
        delta_tc = self._delta_tc_request
        if delta_tc is None:
            delta_tc = self._get_time_resolution()
        tcmin, tcmax = tp.minimum, tp.maximum
        n = int(np.ceil((tcmax - tcmin) / delta_tc))
        self._delta_tc = (tcmax - tcmin) / n
        self._times = tcmin + self._delta_tc / 2. + np.arange(n) * self._delta_tc
        self._beam_pattern_reference_time = (tcmin + tcmax) / 2.
        self.time_prior_array = tp.prob(self._times) * self._delta_tc

    def _detector_analysis(self, interferometer):
        """A one-detector analysis with this detector's weights (and the
        marginalisation grid): calculate_snrs then gives the ROQ inner
        products of roq.py:467-541, with the five-sample <d|h>(t) series under
        time marginalisation."""
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
                an.set_time_marginalization(True, self.jitter_time, tp.minimum, tp.maximum)
            fl, fq, start, dt, wl, wq = self._roq
            an.set_roq(True, fl, fq, start, dt, wl[k:k + 1], wq[k:k + 1])
            if self._roq_tm is not None:
                an.set_roq_time_marginalization(*self._roq_tm)
            self._detector_analyses[name] = an
        return an

    def _snr_block(self, parameters):
        """As the base class's, but the time jitter is kept: the ROQ time
        series adds it to the detector times itself (roq.py:535-539)."""
        from .analysis import params_block
        converted, _ = self.waveform_generator.parameter_conversion(dict(parameters))
        converted["time_jitter"] = parameters.get("time_jitter", 0.0) if self.time_marginalization else 0.0
        return params_block(converted, 1)

    def generate_time_sample_from_marginalized_likelihood(self, signal_polarizations=None, *, parameters):
        """roq.py:1238-1271: a draw from the time posterior on the
        marginalisation grid, from the GPU's <d|h>(t) summed over detectors,
        with the package's shared generator."""
        from .random import Generator
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
        post = np.exp(np.asarray(lnl_t - np.max(lnl_t))) * np.asarray(self.priors["geocent_time"].prob(times))
        post /= np.sum(post)
        return Generator.rng.choice(times, p=post)

    def _upload(self):
        ts = np.asarray(self.weights["time_samples"], dtype=np.float64)
        dt = float(ts[1] - ts[0])
        start = int(np.round(ts[0] / dt))
        # the device rebuilds time sample k as (start + k) * dt, the grid of roq.py:765
        if not np.array_equal(ts, np.arange(start, start + len(ts)) * dt):
            raise ValueError("ROQ time samples must be the grid (start + k) * dt")
        names = [ifo.name for ifo in self.interferometers]
        wl = np.stack([np.asarray(self.weights[n + "_linear"][0]) for n in names])
        wq = np.stack([np.asarray(self.weights[n + "_quadratic"][0]).real for n in names])
        self._roq = (np.asarray(self.weights["frequency_nodes_linear"][0], dtype=np.float64),
                     np.asarray(self.weights["frequency_nodes_quadratic"][0], dtype=np.float64), start, dt, wl, wq)
        if self.time_marginalization:
            self._roq_tm = (np.asarray(self._times, dtype=np.float64), float(self._delta_tc),
                            float(self._beam_pattern_reference_time))
        self._set_weights_on(self.analysis)

    def _set_weights_on(self, an):
        an.set_roq(True, *self._roq)
        if self._roq_tm is not None:
            an.set_roq_time_marginalization(*self._roq_tm)

    def _build_analysis(self):
        super()._build_analysis()
        if getattr(self, "_roq", None) is not None:
            self._set_weights_on(self._analysis)
