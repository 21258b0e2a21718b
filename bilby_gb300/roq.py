"""Drop-in GPU ``ROQGravitationalWaveTransient`` (reduced-order quadrature).

Same constructor as ``bilby.gw.likelihood.ROQGravitationalWaveTransient``
(bilby/gw/likelihood/roq.py:14-215).
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

Several linear and quadratic bases (roq.py:193-460): a weights dictionary
(or .npz file) with one weight array per basis, the frequency nodes of each
and their prior ranges; each point takes the first basis of each kind whose
prior ranges hold its parameters, as the reference's _update_basis does.
Every pair of bases a batch uses gets its own device-resident analysis (the
same data, that pair's nodes and weights); a batch is grouped by pair,
evaluated pair by pair and put back in order.

Bases come as arrays, .npy files, or a mapping laid out as an ROQ basis file
(``basis_<type>``, and optionally ``prior_range_<type>``,
``multiband_<type>``, ``durations_s_<type>``,
``start_end_frequency_bins_<type>``): bases outside the prior are dropped
(roq.py:368-400, 771-791), and a multi-banded basis gets its weights from the
band-wise down-sampled data and inverse PSD (roq.py:920-974, 1007-1055).
Basis files themselves need h5py, as in the reference.
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
        name0 = self.interferometers[0].name
        self.number_of_bases_linear = len(self.weights[f"{name0}_linear"])
        self.number_of_bases_quadratic = len(self.weights[f"{name0}_quadratic"])
        self._cache = dict(parameters=None, basis_number_linear=0, basis_number_quadratic=0)
        for basis_type in ("linear", "quadratic"):
            if getattr(self, f"number_of_bases_{basis_type}") > 1:
                self._verify_numbers_of_prior_ranges_and_frequency_nodes(basis_type)
            else:
                self._check_frequency_nodes_exist_for_single_basis(basis_type)
            self._verify_prior_ranges(basis_type)
        self._basis_analyses = {}
        self._upload()

    # ------------------------------------------------------------------
    # several bases (roq.py:193-460)
    # ------------------------------------------------------------------
    @property
    def multiple_bases(self) -> bool:
        return self.number_of_bases_linear > 1 or self.number_of_bases_quadratic > 1

    def _verify_numbers_of_prior_ranges_and_frequency_nodes(self, basis_type):
        """roq.py:216-247."""
        n = getattr(self, f"number_of_bases_{basis_type}")
        key = f"prior_range_{basis_type}"
        if key not in self.weights:
            raise AttributeError(f'For the use of multiple {basis_type} ROQ bases, weights should contain "{key}".')
        for param_name, ranges in self.weights[key].items():
            if len(ranges) != n:
                raise ValueError(f'The number of prior ranges for "{param_name}" does not match the number of '
                                 f'{basis_type} bases')
        key = f"frequency_nodes_{basis_type}"
        if key not in self.weights:
            raise AttributeError(f'For the use of multiple {basis_type} ROQ bases, weights should contain "{key}".')
        if len(self.weights[key]) != n:
            raise ValueError(f"The number of arrays of frequency nodes does not match the number of {basis_type} bases")

    def _verify_prior_ranges(self, basis_type):
        """roq.py:249-276: the prior must lie inside the union of the ranges."""
        key = f"prior_range_{basis_type}"
        if key not in self.weights or self.priors is None:
            return
        for param_name, ranges in self.weights[key].items():
            if param_name not in self.priors:
                continue
            ranges = np.asarray(ranges, dtype=np.float64)
            prior = self.priors[param_name]
            if prior.minimum < np.min(ranges[:, 0]):
                raise BilbyROQParamsRangeError(f"Prior minimum of {param_name} {prior.minimum} less than ROQ basis "
                                               f"bound {np.min(ranges[:, 0])}")
            if prior.maximum > np.max(ranges[:, 1]):
                raise BilbyROQParamsRangeError(f"Prior maximum of {param_name} {prior.maximum} greater than ROQ "
                                               f"basis bound {np.max(ranges[:, 1])}")

    def _check_frequency_nodes_exist_for_single_basis(self, basis_type):
        """roq.py:278-296."""
        key = f"frequency_nodes_{basis_type}"
        args = self.waveform_generator.waveform_arguments
        if key not in self.weights and key not in args:
            raise AttributeError(f"{key} should be contained in weights or waveform arguments.")
        if key not in args:
            args[key] = self.weights[key][0]
        elif key not in self.weights:
            self.weights[key] = [args[key]]

    def basis_numbers(self, parameters):
        """The (linear, quadratic) basis of each point, vectorised
        (roq.py:398-431): after the ROQ's own parameter_conversion, the first
        basis whose prior range holds every ranged parameter the point has;
        IndexError when none does, as in the reference."""
        p = dict(parameters)
        if self.parameter_conversion is not None:
            p = self.parameter_conversion(p)
        sizes = [np.size(v) for v in p.values() if not isinstance(v, str)]
        n_points = max(sizes) if sizes else 1
        out = []
        for basis_type in ("linear", "quadratic"):
            n = getattr(self, f"number_of_bases_{basis_type}")
            if n == 1:
                out.append(np.zeros(n_points, dtype=np.int64))
                continue
            ok = np.ones((n, n_points), dtype=bool)
            for name, ranges in self.weights[f"prior_range_{basis_type}"].items():
                if name not in p:
                    continue
                r = np.asarray(ranges, dtype=np.float64)
                v = np.broadcast_to(np.asarray(p[name], dtype=np.float64), (n_points,))
                ok &= (r[:, :1] <= v) & (r[:, 1:2] >= v)
            if not ok.any(axis=0).all():
                raise IndexError(f"a point lies in no {basis_type} ROQ basis' prior range")
            out.append(np.argmax(ok, axis=0).astype(np.int64))
        return out[0], out[1]

    def _update_basis(self, parameters):
        """roq.py:398-431 for one point: the cache the per-detector methods read."""
        il, iq = self.basis_numbers(parameters)
        self._cache.update(parameters=dict(parameters), basis_number_linear=int(il[0]),
                           basis_number_quadratic=int(iq[0]))

    @property
    def basis_number_linear(self):
        return self._cache["basis_number_linear"] if self.number_of_bases_linear > 1 else 0

    @property
    def basis_number_quadratic(self):
        return self._cache["basis_number_quadratic"] if self.number_of_bases_quadratic > 1 else 0

    def _analysis_for(self, il, iq):
        """The device analysis of the pair (linear basis il, quadratic basis iq)."""
        if (il, iq) == (0, 0):
            return self.analysis
        an = self._basis_analyses.get((il, iq))
        if an is None:
            an = self._new_analysis(self.interferometers)
            self._configure_analysis(an)
            an.set_roq(True, *self._roq_for(il, iq))
            if self._roq_tm is not None:
                an.set_roq_time_marginalization(*self._roq_tm)
            self._basis_analyses[(il, iq)] = an
        return an

    def log_likelihood_ratio(self, parameters):
        """roq.py:461-463: select the bases, then the likelihood."""
        if not self.multiple_bases:
            return super().log_likelihood_ratio(parameters)
        import copy
        from .analysis import params_block
        self._update_basis(parameters)
        an = self._analysis_for(self._cache["basis_number_linear"], self._cache["basis_number_quadratic"])
        block = params_block(self._prepare(copy.deepcopy(parameters)), 1)
        return float(an.log_likelihood_ratio_host(block, self.precision)[0])

    def log_likelihood_ratio_batch(self, parameters, precision=None, out=None):
        """A batch grouped by basis pair (numpy arrays or CUDA tensors)."""
        if not self.multiple_bases:
            return super().log_likelihood_ratio_batch(parameters, precision, out)
        precision = precision or self.precision
        first = next(iter(parameters.values()))
        cuda = hasattr(first, "is_cuda") and first.is_cuda
        host = {k: (v.detach().cpu().numpy() if cuda else np.asarray(v, dtype=np.float64))
                for k, v in parameters.items()}
        n = len(np.atleast_1d(host[next(iter(host))]))
        il, iq = self.basis_numbers(host)
        if cuda:
            import torch
            res = out if out is not None else torch.empty(n, dtype=torch.float64, device=first.device)
        else:
            res = np.empty(n)
        for pair in sorted(set(zip(il.tolist(), iq.tolist()))):
            idx = np.nonzero((il == pair[0]) & (iq == pair[1]))[0]
            if cuda:
                import torch
                ti = torch.from_numpy(idx).to(first.device)
                sub = {k: (v[ti] if v.ndim and v.shape[0] == n else v) for k, v in parameters.items()}
                res[ti] = self._batch_on(self._analysis_for(*pair), sub, precision)
            else:
                sub = {k: (v[idx] if np.ndim(v) and len(v) == n else v) for k, v in host.items()}
                res[idx] = self._batch_on(self._analysis_for(*pair), sub, precision)
        return res

    # ------------------------------------------------------------------
    # basis and weights (host, float64)
    # ------------------------------------------------------------------
    @staticmethod
    def _parse_basis(basis, basis_type):
        """roq.py:333-366: an array (n_frequencies x n_basis) or a .npy file
        (n_basis x n_frequencies) -> {basis_<type>: {"0": {"basis": n_basis x n_frequencies}}}.
        A mapping with the layout of a basis file (what h5py would open) is
        taken as it is."""
        if hasattr(basis, "keys") and not isinstance(basis, np.ndarray):
            if f"basis_{basis_type}" not in basis:
                raise ValueError(f"a {basis_type} basis mapping needs the key basis_{basis_type}")
            return basis
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

    def _select_prior_ranges(self, prior_ranges):
        """roq.py:368-400: the bases whose prior ranges meet the priors."""
        names = list(prior_ranges)
        n = len(prior_ranges[names[0]])
        keep = np.ones(n, dtype=bool)
        for name in names:
            if self.priors is None or name not in self.priors:
                continue
            pr = np.asarray(prior_ranges[name])
            keep &= (pr[:, 1] >= self.priors[name].minimum) & (pr[:, 0] <= self.priors[name].maximum)
        idx = np.arange(n)[keep]
        return idx, {name: np.asarray(prior_ranges[name])[idx] for name in names}

    def _set_weights(self, linear_matrix, quadratic_matrix):
        """roq.py:736-847: the time grid, the bases inside the prior and their
        frequency nodes, then the linear and quadratic weights of each basis
        (multi-banded or on the data's own frequencies)."""
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
        selected = {}
        for key, matrix in (("linear", linear_matrix), ("quadratic", quadratic_matrix)):
            pr_key = f"prior_range_{key}"
            if pr_key in matrix:
                ranges = {}
                for name in matrix[pr_key]:
                    attrs = getattr(matrix[pr_key][name], "attrs", {})
                    power = attrs["roq_scale_power"] if "roq_scale_power" in attrs else None
                    scale = self.roq_scale_factor ** power if power is not None else 1.
                    ranges[name] = np.asarray(matrix[pr_key][name][()]) * scale
                idx, sel = self._select_prior_ranges(ranges)
                if len(idx) == 0:
                    raise BilbyROQParamsRangeError(f"There are no {key} ROQ bases within the prior range.")
                self.weights[pr_key] = sel
                selected[key] = [int(i) for i in idx]
            else:
                selected[key] = [0]
            if "frequency_nodes" in matrix[f"basis_{key}"][str(selected[key][0])]:
                self.weights[f"frequency_nodes_{key}"] = [
                    np.asarray(matrix[f"basis_{key}"][str(i)]["frequency_nodes"][()]) * self.roq_scale_factor
                    for i in selected[key]]
        mb_lin = bool(np.asarray(linear_matrix["multiband_linear"][()])) if "multiband_linear" in linear_matrix \
            else False
        mb_quad = bool(np.asarray(quadratic_matrix["multiband_quadratic"][()])) \
            if "multiband_quadratic" in quadratic_matrix else False
        idxs = None
        if not (mb_lin and mb_quad):
            n_basis_f = np.asarray(linear_matrix["basis_linear"][str(selected["linear"][0])]["basis"]).shape[1]
            idxs = {ifo.name: self._overlap_indices(ifo, n_basis_f) for ifo in ifos}
        if mb_lin:
            self._set_weights_linear_multiband(linear_matrix, selected["linear"])
        else:
            self._set_weights_linear(linear_matrix, selected["linear"], idxs, n_time, start_idx, end_idx)
        if mb_quad:
            self._set_weights_quadratic_multiband(quadratic_matrix, selected["quadratic"])
        else:
            self._set_weights_quadratic(quadratic_matrix, selected["quadratic"], idxs)

    def _overlap_indices(self, ifo, n_basis_frequencies):
        """roq.py:802-837: (indices into the data's masked frequencies, indices
        into the basis' frequencies) of the frequencies both share."""
        mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
        fm = np.asarray(ifo.strain_data.frequency_array)[mask]
        if self.roq_params is not None:
            fmax = self.roq_params["fhigh"] * self.roq_scale_factor
            seglen = self.roq_params["seglen"] / self.roq_scale_factor
            roq_f = np.linspace(0, fmax, int(np.round(fmax * seglen)) + 1)
            roq_f = roq_f[roq_f >= self.roq_params["flow"] * self.roq_scale_factor]
            _, ifo_idxs, roq_idxs = np.intersect1d(fm, roq_f, return_indices=True)
        else:
            roq_idxs = np.arange(n_basis_frequencies, dtype=int)
            ifo_idxs = np.arange(int(mask.sum()))
            if len(ifo_idxs) != len(roq_idxs):
                raise ValueError(f"Mismatch between ROQ basis and frequency array for {ifo.name}")
        return ifo_idxs, roq_idxs

    def _set_weights_linear(self, linear_matrix, basis_idxs, idxs, n_time, start_idx, end_idx):
        """roq.py:849-918: per basis and detector, the inverse FFT of d/S times
        each conjugated basis element, kept on the time grid."""
        duration = float(self.interferometers[0].strain_data.duration)
        for ifo in self.interferometers:
            self.weights[ifo.name + "_linear"] = []
        for i in basis_idxs:
            lin = np.asarray(linear_matrix["basis_linear"][str(i)]["basis"][()])
            for ifo in self.interferometers:
                ifo_idxs, roq_idxs = idxs[ifo.name]
                mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
                nonzero = ifo_idxs + int(ifo.minimum_frequency * duration)
                d_over_s = (np.asarray(ifo.strain_data.frequency_domain_strain)[mask][ifo_idxs]
                            / np.asarray(ifo.power_spectral_density_array)[mask][ifo_idxs])
                rows = []
                for c0 in range(0, lin.shape[0], 16):  # inverse FFTs of 16 basis elements at a time
                    block = np.zeros((min(16, lin.shape[0] - c0), n_time), dtype=complex)
                    block[:, nonzero] = d_over_s * np.conj(lin[c0:c0 + 16][:, roq_idxs])
                    rows.append(np.fft.ifft(block, axis=1)[:, start_idx:end_idx + 1])
                self.weights[ifo.name + "_linear"].append(np.concatenate(rows).T * (4. * n_time / duration))

    def _set_weights_quadratic(self, quadratic_matrix, basis_idxs, idxs):
        """roq.py:976-1005: (4/T) basis times 1/S per basis and detector."""
        for ifo in self.interferometers:
            self.weights[ifo.name + "_quadratic"] = []
        for i in basis_idxs:
            quad = np.asarray(quadratic_matrix["basis_quadratic"][str(i)]["basis"][()]).real
            for ifo in self.interferometers:
                ifo_idxs, roq_idxs = idxs[ifo.name]
                mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
                inv_psd = 1 / np.asarray(ifo.power_spectral_density_array)[mask][ifo_idxs]
                self.weights[ifo.name + "_quadratic"].append(
                    4. / float(ifo.strain_data.duration) * quad[:, roq_idxs] @ inv_psd)

    @staticmethod
    def _band_layout(matrix, basis_type, scale):
        tbs = np.asarray(matrix[f"durations_s_{basis_type}"][()], dtype=np.float64) / scale
        se = np.asarray(matrix[f"start_end_frequency_bins_{basis_type}"][()]).astype(np.int64)
        return tbs, se, int(np.sum(se[:, 1] - se[:, 0] + 1)), float(np.max(se[:, 1] / tbs))

    def _set_weights_linear_multiband(self, linear_matrix, basis_idxs):
        """roq.py:920-974: d/S (zero outside the mask) up to the basis' top
        frequency to the time domain, each band's last 2 f_high T_b samples
        back to its frequencies k / T_b, times (4 / T_b) exp(2 pi i f (t - T +
        T_b)) on the time grid; the weights are the conjugated basis times
        that, per detector."""
        tbs, se, dim, fhigh = self._band_layout(linear_matrix, "linear", self.roq_scale_factor)
        ts = np.asarray(self.weights["time_samples"], dtype=np.float64)
        for ifo in self.interferometers:
            self.weights[ifo.name + "_linear"] = []
        bases = [np.asarray(linear_matrix["basis_linear"][str(i)]["basis"][()]) for i in basis_idxs]
        for ifo in self.interferometers:
            T = float(ifo.strain_data.duration)
            mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
            strain = np.asarray(ifo.strain_data.frequency_domain_strain)
            psd = np.asarray(ifo.power_spectral_density_array)
            data = np.zeros(int(fhigh * T) + 1, dtype=complex)
            data[np.arange(len(strain))[mask]] = strain[mask] / psd[mask]
            td = np.fft.irfft(data)
            shifted = np.zeros((dim, len(ts)), dtype=complex)
            off = 0
            for b, tb in enumerate(tbs):
                s0, e0 = (int(x) for x in se[b])
                fs = np.arange(s0, e0 + 1) / tb
                db = np.fft.rfft(td[-int(2. * fhigh * tb):])[s0:e0 + 1]
                shifted[off:off + e0 - s0 + 1] = 4. / tb * db[:, None] * np.exp(
                    2. * np.pi * 1j * fs[:, None] * (ts[None, :] - T + tb))
                off += e0 - s0 + 1
            for basis in bases:
                self.weights[ifo.name + "_linear"].append((basis.conj() @ shifted).T)
            del shifted

    def _set_weights_quadratic_multiband(self, quadratic_matrix, basis_idxs):
        """roq.py:1007-1055: 1/S (zero outside the mask) up to the basis' top
        frequency to the time domain, truncated to lags |n| < f_high T_b and
        back to each band's frequencies, times 4 / T_b; the weights are the
        basis times that, per detector."""
        tbs, se, dim, fhigh = self._band_layout(quadratic_matrix, "quadratic", self.roq_scale_factor)
        for ifo in self.interferometers:
            self.weights[ifo.name + "_quadratic"] = []
        bases = [np.asarray(quadratic_matrix["basis_quadratic"][str(i)]["basis"][()]).real for i in basis_idxs]
        for ifo in self.interferometers:
            T = float(ifo.strain_data.duration)
            mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
            psd = np.asarray(ifo.power_spectral_density_array)
            inv = np.zeros(int(fhigh * T) + 1)
            inv[np.arange(len(psd))[mask]] = 1. / psd[mask]
            td = np.fft.irfft(inv)
            v = np.zeros(dim)
            off = 0
            for b, tb in enumerate(tbs):
                s0, e0 = (int(x) for x in se[b])
                h = int(fhigh * tb)
                v[off:off + e0 - s0 + 1] = 4. / tb * np.fft.rfft(np.concatenate([td[:h], td[-h:]]))[s0:e0 + 1].real
                off += e0 - s0 + 1
            for basis in bases:
                self.weights[ifo.name + "_quadratic"].append(basis @ v)

    def _setup_time_marginalization(self):
        """roq.py:320-331: delta_tc from the constructor or the ROQ time
        resolution, shrunk so that it divides the geocent_time prior; the
        samples sit at the middles of the intervals; the antenna patterns and
        delays are taken at the prior's mid time."""
        tp = self.priors["geocent_time"]
        if not (np.isfinite(tp.minimum) and np.isfinite(tp.maximum)):
            raise ValueError("ROQ time marginalisation needs a geocent_time prior with finite bounds")
        delta_tc = self._delta_tc_request
        if delta_tc is None:
            delta_tc = self._get_time_resolution()
        tcmin, tcmax = tp.minimum, tp.maximum
        n = int(np.ceil((tcmax - tcmin) / delta_tc))
        self._delta_tc = (tcmax - tcmin) / n
        self._times = tcmin + self._delta_tc / 2. + np.arange(n) * self._delta_tc
        self._beam_pattern_reference_time = (tcmin + tcmax) / 2.
        self.time_prior_array = tp.prob(self._times) * self._delta_tc
        from .likelihood import time_prior_table
        self._time_prior_table = time_prior_table(tp, tcmin, tcmax, self._delta_tc)

    def _detector_analysis(self, interferometer):
        """A one-detector analysis with this detector's weights (and the
        marginalisation grid): calculate_snrs then gives the ROQ inner
        products of roq.py:467-541, with the five-sample <d|h>(t) series under
        time marginalisation."""
        name = interferometer.name
        pair = (self.basis_number_linear, self.basis_number_quadratic)  # the reference's cached bases
        an = self._detector_analyses.get((name, pair))
        if an is None:
            names = [ifo.name for ifo in self.interferometers]
            if name not in names:
                raise ValueError(f"interferometer {name} is not part of this likelihood")
            k = names.index(name)
            an = self._new_analysis([self.interferometers[k]])
            if self.time_marginalization:
                tp = self.priors["geocent_time"]
                an.set_time_marginalization(True, self.jitter_time, tp.minimum, tp.maximum)
            fl, fq, start, dt, wl, wq = self._roq_for(*pair)
            an.set_roq(True, fl, fq, start, dt, wl[k:k + 1], wq[k:k + 1])
            if self._roq_tm is not None:
                an.set_roq_time_marginalization(*self._roq_tm)
            self._detector_analyses[(name, pair)] = an
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
        self._roq_grid = (start, dt)
        self._roq = self._roq_for(0, 0)
        if self.time_marginalization:
            self._roq_tm = (np.asarray(self._times, dtype=np.float64), float(self._delta_tc),
                            float(self._beam_pattern_reference_time))
        self._set_weights_on(self.analysis)

    def __getstate__(self):
        state = super().__getstate__()
        state["_basis_analyses"] = {}
        return state

    def _roq_for(self, il, iq):
        """gwl_set_roq arguments of the pair (linear basis il, quadratic basis iq)."""
        start, dt = self._roq_grid
        names = [ifo.name for ifo in self.interferometers]
        wl = np.stack([np.asarray(self.weights[n + "_linear"][il]) for n in names])
        wq = np.stack([np.asarray(self.weights[n + "_quadratic"][iq]).real for n in names])
        return (np.asarray(self.weights["frequency_nodes_linear"][il], dtype=np.float64),
                np.asarray(self.weights["frequency_nodes_quadratic"][iq], dtype=np.float64), start, dt, wl, wq)

    def _set_weights_on(self, an):
        an.set_roq(True, *self._roq)
        if self._roq_tm is not None:
            an.set_roq_time_marginalization(*self._roq_tm)

    def _build_analysis(self):
        super()._build_analysis()
        if getattr(self, "_roq", None) is not None:
            self._set_weights_on(self._analysis)
