"""Drop-in GPU ``RelativeBinningGravitationalWaveTransient``.

Same constructor and methods as
``bilby.gw.likelihood.RelativeBinningGravitationalWaveTransient``
(bilby/gw/likelihood/relative.py:14-452, after Zackay, Dai & Venumadhav,
arXiv:1806.08792).  The set-up -- the fiducial responses (evaluated by the
float64 GPU source and response kernels), the bins and the per-bin summary
data -- runs once on the host in float64; every likelihood evaluation then
runs on the GPU: one warp per parameter point evaluates the model at the bin
edges, forms the ratio to the fiducial response and sums the summary data
(``k_relbin``, behind ``gwl_set_relative_binning`` in include/gwlnl.h).

With time marginalisation (relative.py:380-420) the float64
time-marginalised kernel rebuilds the piecewise-linear full-grid waveform
from the edge ratios, transforms it against the data and marginalises over
time with <h|h> from the summary data
(``gwl_set_relative_binning_time_weights``).
"""
from __future__ import annotations

import logging

import numpy as np

from . import _capi
from .analysis import params_block
from .likelihood import GravitationalWaveTransient

logger = logging.getLogger("bilby")

GAMMA = np.array([-5 / 3, -2 / 3, 1, 5 / 3, 7 / 3])  # relative.py:146


class RelativeBinningGravitationalWaveTransient(GravitationalWaveTransient):
    """Relative-binning likelihood on the GPU (bilby/gw/likelihood/relative.py:14-140)."""

    def __init__(self, interferometers, waveform_generator, fiducial_parameters=None, parameter_bounds=None,
                 maximization_kwargs=None, update_fiducial_parameters=False, distance_marginalization=False,
                 time_marginalization=False, phase_marginalization=False, priors=None,
                 distance_marginalization_lookup_table=None, jitter_time=True, reference_frame="sky",
                 time_reference="geocenter", chi=1, epsilon=0.5, precision="fp64"):
        self._rb = None
        self._rb_time_weights = None
        super().__init__(interferometers, waveform_generator, distance_marginalization=distance_marginalization,
                         time_marginalization=time_marginalization,
                         phase_marginalization=phase_marginalization, priors=priors,
                         distance_marginalization_lookup_table=distance_marginalization_lookup_table,
                         jitter_time=jitter_time, reference_frame=reference_frame, time_reference=time_reference,
                         precision=precision)
        if fiducial_parameters is None:
            logger.info("Drawing fiducial parameters from prior.")
            fiducial_parameters = priors.sample()
        self.fiducial_parameters = dict(fiducial_parameters)
        self._unset_fiducial()
        if self.time_marginalization:  # relative.py:139-140
            self.fiducial_parameters["geocent_time"] = self._start_time
        if self.distance_marginalization:
            self.fiducial_parameters["luminosity_distance"] = self._ref_dist
        if self.phase_marginalization:
            self.fiducial_parameters["phase"] = 0.0
        self.chi = chi
        self.epsilon = epsilon
        self.gamma = GAMMA
        self.maximum_frequency = waveform_generator.frequency_array[-1]
        self.fiducial_polarizations = None
        self.per_detector_fiducial_waveforms = dict()
        self.per_detector_fiducial_waveform_points = dict()
        self.set_fiducial_waveforms(self.fiducial_parameters)
        self.setup_bins()
        self.compute_summary_data()
        self._upload()
        if update_fiducial_parameters:
            self.parameters_to_be_updated = [
                key for key in priors
                if not (isinstance(priors[key], (float, int)) or getattr(priors[key], "is_fixed", False)
                        or type(priors[key]).__name__ == "Constraint")]
            if parameter_bounds is None:
                self.parameter_bounds = self.get_bounds_from_priors(priors)
            else:
                self.parameter_bounds = self.get_parameter_list_from_dictionary(parameter_bounds)
            self.fiducial_parameters = self.find_maximum_likelihood_parameters(
                self.parameter_bounds, maximization_kwargs=maximization_kwargs)

    def __repr__(self):
        return (f"{self.__class__.__name__}(interferometers={[i.name for i in self.interferometers]},\n\t"
                f"waveform_generator={self.waveform_generator},\n\tfiducial_parameters={self.fiducial_parameters},")

    # ------------------------------------------------------------------
    # set-up (host, float64)
    # ------------------------------------------------------------------
    def _set_fiducial(self):
        """relative.py:428-438."""
        self.waveform_generator.waveform_arguments["fiducial"] = 1
        cache = getattr(self.waveform_generator, "_cache", None)
        if isinstance(cache, dict):
            cache["parameters"] = None

    def _unset_fiducial(self):
        """relative.py:440-452."""
        self.waveform_generator.waveform_arguments["fiducial"] = 0
        cache = getattr(self.waveform_generator, "_cache", None)
        if isinstance(cache, dict):
            cache["parameters"] = None

    def set_fiducial_waveforms(self, parameters):
        """relative.py:232-254: the fiducial response of every detector on the
        full grid (float64 GPU kernels), zero above the fiducial's last non-zero
        frequency."""
        p = dict(parameters)
        p.update(self.get_sky_frame_parameters(p))
        block = params_block(self._prepare({k: np.atleast_1d(np.asarray(v, dtype=np.float64))
                                            for k, v in p.items()}), 1)[:, 0]
        freq = np.asarray(self.interferometers[0].strain_data.frequency_array, dtype=np.float64)
        fmin = self.waveform_generator.waveform_arguments.get("minimum_frequency", 20.0)
        plus, cross = _capi.source_polarizations(self.analysis.model_id, freq, block, fmin)
        self.fiducial_polarizations = {"plus": plus, "cross": cross}
        nz = np.where(plus != 0j)[0]
        if len(nz) == 0:
            raise ValueError(f"Cannot compute fiducial waveforms for {parameters}")
        self.maximum_frequency = freq[nz[-1]]
        for ifo in self.interferometers:
            geom = ifo.geometry
            wf = _capi.detector_response(ifo.name, geom.vertex, geom.detector_tensor, ifo.strain_data.start_time,
                                         np.asarray(ifo.strain_data.frequency_mask, dtype=bool), freq, plus, cross,
                                         block)
            wf = wf * (freq <= self.maximum_frequency)
            self.per_detector_fiducial_waveforms[ifo.name] = wf

    def setup_bins(self):
        """relative.py:178-230: bin edges where the differential phase of the
        power laws f^gamma grows by epsilon (vectorised search)."""
        f = np.asarray(self.waveform_generator.frequency_array, dtype=np.float64)
        fmax, fmin = f[0], f[-1]
        for ifo in self.interferometers:
            fmax = max(fmax, ifo.maximum_frequency)
            fmin = min(fmin, ifo.minimum_frequency)
        fmax = min(fmax, self.maximum_frequency)
        useful = f[(f >= fmin) & (f <= fmax)]
        g = self.gamma[:, np.newaxis]
        d_alpha = self.chi * 2 * np.pi / np.abs((fmin ** g) * np.heaviside(-g, 1) - (fmax ** g) * np.heaviside(g, 1))
        d_phi = np.sum(np.sign(g) * d_alpha * useful ** g, axis=0)
        d_phi_from_start = d_phi - d_phi[0]
        n = int(d_phi_from_start[-1] // self.epsilon)
        targets = (np.arange(n + 1) / n) * d_phi_from_start[-1]
        # the first index reaching each target; d_phi grows monotonically
        idx = np.unique(np.searchsorted(d_phi_from_start, targets, side="left"))
        self.bin_freqs = useful[idx]
        self.bin_inds = np.searchsorted(f, self.bin_freqs, side="left").astype(int)
        self.bin_sizes = np.diff(self.bin_inds)
        self.bin_sizes[-1] += 1
        self.number_of_bins = len(self.bin_inds) - 1
        self.waveform_generator.waveform_arguments["frequency_bin_edges"] = self.bin_freqs
        self.bin_widths = self.bin_freqs[1:] - self.bin_freqs[:-1]
        self.bin_centers = (self.bin_freqs[1:] + self.bin_freqs[:-1]) / 2
        for ifo in self.interferometers:
            self.per_detector_fiducial_waveform_points[ifo.name] = (
                self.per_detector_fiducial_waveforms[ifo.name][self.bin_inds])
        logger.debug(f"Set up {self.number_of_bins} bins between {fmin} Hz and {fmax} Hz")

    def compute_summary_data(self):
        """relative.py:319-363: per bin and detector a0 = <h0|d>, a1 = <h0|d df>,
        b0 = <h0|h0>, b1 = <h0|h0 df> on the masked grid, df from the bin
        centre, as segment sums."""
        summary = dict()
        for ifo in self.interferometers:
            mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool)
            mf = np.asarray(ifo.strain_data.frequency_array)[mask]
            inds = np.searchsorted(mf, self.bin_freqs, side="left")
            if np.any(inds >= len(mf)) or np.any(mf[np.minimum(inds, len(mf) - 1)] != self.bin_freqs):
                raise ValueError(f"{ifo.name}: a bin edge lies outside the detector's frequency mask")
            if inds[-1] < len(mf) - 1:
                inds[-1] += 1
            strain = np.asarray(ifo.strain_data.frequency_domain_strain)[mask]
            h0 = np.asarray(self.per_detector_fiducial_waveforms[ifo.name])[mask]
            psd = np.asarray(ifo.power_spectral_density_array)[mask]
            norm = 4 / ifo.strain_data.duration
            centre = (mf[inds[:-1]] + mf[inds[1:]]) / 2
            lo, hi = inds[0], inds[-1]
            df = mf[lo:hi] - np.repeat(centre, np.diff(inds))
            x = (h0.conj() * strain / psd)[lo:hi]
            y = (h0.conj() * h0 / psd)[lo:hi]
            starts = inds[:-1] - lo
            a0 = norm * np.add.reduceat(x, starts)
            a1 = norm * np.add.reduceat(x * df, starts)
            b0 = norm * np.add.reduceat(y, starts)
            b1 = norm * np.add.reduceat(y * df, starts)
            summary[ifo.name] = (a0, a1, b0, b1)
        self.summary_data = summary

    def _upload(self):
        """Edges, 1 / h0 at the edges and the summary data to the device."""
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = np.stack([1.0 / self.per_detector_fiducial_waveform_points[ifo.name]
                            for ifo in self.interferometers])
        sm = np.stack([np.stack([a0.real, a0.imag, a1.real, a1.imag, b0.real, b1.real], axis=-1)
                       for a0, a1, b0, b1 in (self.summary_data[ifo.name] for ifo in self.interferometers)])
        self._rb = (np.asarray(self.bin_inds, dtype=np.int64), inv, sm)
        self._rb_time_weights = self._time_weights() if self.time_marginalization else None
        self._set_bins(self.analysis)

    def _time_weights(self):
        """4/T h0_d conj(d) / S on the full grid, zero outside the mask and
        outside the first and last bin edges (relative.py:380-420 before the
        per-point ratio)."""
        out = []
        k0, k1 = int(self.bin_inds[0]), int(self.bin_inds[-1])
        for ifo in self.interferometers:
            mask = np.asarray(ifo.strain_data.frequency_mask, dtype=bool).copy()
            mask[:k0] = False
            mask[k1 + 1:] = False
            w = np.zeros(len(mask), dtype=np.complex128)
            h0 = np.asarray(self.per_detector_fiducial_waveforms[ifo.name])
            d = np.asarray(ifo.strain_data.frequency_domain_strain)
            psd = np.asarray(ifo.power_spectral_density_array)
            w[mask] = 4 / ifo.strain_data.duration * h0[mask] * np.conj(d[mask]) / psd[mask]
            out.append(w)
        return np.stack(out)

    def _set_bins(self, an):
        an.set_relative_binning(True, *self._rb)
        if self._rb_time_weights is not None:
            an.set_relative_binning_time_weights(self._rb_time_weights)

    def _build_analysis(self):
        super()._build_analysis()
        if getattr(self, "_rb", None) is not None:
            self._set_bins(self._analysis)

    def _detector_analysis(self, interferometer):
        """A one-detector analysis with this detector's bins, 1 / h0 at the
        edges, summary data (and time weights): calculate_snrs then gives the
        relative-binning inner products of relative.py:398-420."""
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
            idx, inv, sm = self._rb
            an.set_relative_binning(True, idx, inv[k:k + 1], sm[k:k + 1])
            if self._rb_time_weights is not None:
                an.set_relative_binning_time_weights(self._rb_time_weights[k:k + 1])
            self._detector_analyses[name] = an
        return an

    def _compute_full_waveform(self, signal_polarizations, interferometer, parameters):
        """relative.py:365-396: the fiducial response times the piecewise-linear
        ratio r0_b + r1_b (f - f_b) on the grid between the first and last
        edges.  The model and its response at the edges come from the float64
        GPU kernels (explicit frequencies, no mask)."""
        name = interferometer.name
        block = self._snr_block(parameters)[:, 0]
        fmin = self.waveform_generator.waveform_arguments.get("minimum_frequency", 20.0)
        edges = np.asarray(self.bin_freqs, dtype=np.float64)
        plus, cross = _capi.source_polarizations(self.analysis.model_id, edges, block, fmin)
        geom = interferometer.geometry
        strain = _capi.detector_response(name, geom.vertex, geom.detector_tensor,
                                         interferometer.strain_data.start_time, np.ones(len(edges), dtype=bool),
                                         edges, plus, cross, block)
        ratio = strain / self.per_detector_fiducial_waveform_points[name]
        r0 = (ratio[1:] + ratio[:-1]) / 2
        r1 = (ratio[1:] - ratio[:-1]) / self.bin_widths
        idxs = slice(int(self.bin_inds[0]), int(self.bin_inds[-1]) + 1)
        f = np.asarray(interferometer.frequency_array)
        full = np.zeros(len(f), dtype=complex)
        full[idxs] = (np.repeat(r0, self.bin_sizes)
                      + np.repeat(r1, self.bin_sizes) * (f[idxs] - np.repeat(self.bin_centers, self.bin_sizes)))
        return self.per_detector_fiducial_waveforms[name] * full

    # ------------------------------------------------------------------
    # fiducial optimisation (relative.py:256-317)
    # ------------------------------------------------------------------
    def find_maximum_likelihood_parameters(self, parameter_bounds, iterations=5, maximization_kwargs=None):
        """scipy differential evolution over the free parameters, with whole
        populations evaluated as one GPU batch (``vectorized``), re-binning
        about each new optimum until the fiducial lnL gains less than 0.1."""
        from scipy.optimize import differential_evolution
        maximization_kwargs = dict(maximization_kwargs or {})
        keys = self.parameters_to_be_updated
        x0 = self.get_parameter_list_from_dictionary(self.fiducial_parameters)
        old = self.log_likelihood_ratio(self.fiducial_parameters)
        updated = dict(self.fiducial_parameters)

        def objective(x):
            x = np.atleast_2d(np.asarray(x, dtype=np.float64).T).T  # (n_params, S)
            batch = {k: np.full(x.shape[1], float(v)) for k, v in self.fiducial_parameters.items()}
            for j, k in enumerate(keys):
                batch[k] = x[j]
            return -np.asarray(self.log_likelihood_ratio_batch(batch))

        for it in range(iterations):
            out = differential_evolution(objective, bounds=parameter_bounds, x0=x0, vectorized=True,
                                         updating="deferred", **maximization_kwargs)
            x0 = out["x"]
            updated = dict(self.fiducial_parameters)
            updated.update(self.get_parameter_dictionary_from_list(x0))
            self.set_fiducial_waveforms(updated)
            self.setup_bins()
            self.compute_summary_data()
            self._upload()
            new = self.log_likelihood_ratio(updated)
            if new - old < 0.1:
                break
            old = new
        return updated

    def get_parameter_dictionary_from_list(self, parameter_list):
        d = dict(zip(self.parameters_to_be_updated, parameter_list))
        for key in set(self.fiducial_parameters) - set(self.parameters_to_be_updated):
            d[key] = self.fiducial_parameters[key]
        return d

    def get_parameter_list_from_dictionary(self, parameter_dict):
        return [parameter_dict[k] for k in self.parameters_to_be_updated]

    def get_bounds_from_priors(self, priors):
        return [[priors[k].minimum, priors[k].maximum] for k in self.parameters_to_be_updated]
