"""Drop-in GPU ``GravitationalWaveTransient``.

Same constructor, parameter dictionary and methods as
``bilby.gw.likelihood.GravitationalWaveTransient``
(bilby/gw/likelihood/base.py:18-1183): ``log_likelihood_ratio(parameters)``,
``noise_log_likelihood()``, ``log_likelihood(parameters)``, the
marginalisation flags, the mutation of the caller's ``priors`` dictionary for
marginalised parameters, ``marginalized_parameters`` and ``meta_data``.  The
likelihood itself is evaluated by the fused CUDA kernels behind the C ABI
(include/gwlnl.h); there is no CPU fallback.

Extensions: ``log_likelihood_ratio_batch(params)`` evaluates a whole batch
(numpy arrays -> numpy, or CUDA tensors -> CUDA tensor on the current stream),
and ``precision`` selects the plain float64 kernels ("fp64", the default and
the drop-in) or the mixed-precision kernels ("mixed").
"""
from __future__ import annotations

import copy
import logging
import os

import numpy as np

from . import _capi
from .analysis import Analysis, DetectorData, params_block
from .source import model_of

logger = logging.getLogger("bilby")

try:  # subclass bilby's Likelihood where bilby is importable (samplers check isinstance)
    from bilby.core.likelihood import Likelihood as _Base  # type: ignore
except Exception:  # pragma: no cover - bilby absent
    class _Base:
        def __init__(self):
            self._meta_data = None
            self._marginalized_parameters = []

        def __repr__(self):
            return self.__class__.__name__

        @property
        def marginalized_parameters(self):
            return self._marginalized_parameters


def _prior_attr(prior, name):
    return getattr(prior, name, None)


def _is_fixed(prior):
    return bool(getattr(prior, "is_fixed", False)) or isinstance(prior, (int, float))


N_DISTANCE_GRID = 10000  # base.py:210-212


def d_inner_h_ref_axis(n, phase_marginalization):
    """base.py:904-914."""
    if phase_marginalization:
        return np.logspace(-5, 10, n)
    n_negative = n // 2
    return np.hstack((-np.logspace(3, -3, n_negative), np.logspace(-3, 10, n - n_negative)))


def optimal_snr_squared_ref_axis(n):
    """base.py:899-902."""
    return np.logspace(-5, 10, n)


class GravitationalWaveTransient(_Base):
    """GPU drop-in for bilby's GravitationalWaveTransient (sine-Gaussian and
    aligned-spin TaylorF2 source models, identity calibration)."""

    def __init__(self, interferometers, waveform_generator, time_marginalization=False,
                 distance_marginalization=False, phase_marginalization=False, calibration_marginalization=False,
                 priors=None, distance_marginalization_lookup_table=None, calibration_lookup_table=None,
                 number_of_response_curves=1000, starting_index=0, jitter_time=True, reference_frame="sky",
                 time_reference="geocenter", precision="fp64"):
        super().__init__()
        if not hasattr(self, "_marginalized_parameters"):
            self._marginalized_parameters = []
        if calibration_marginalization:
            raise NotImplementedError("calibration marginalisation has no GPU kernel")
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = precision
        self.waveform_generator = waveform_generator
        self.interferometers = list(interferometers)
        self.time_marginalization = time_marginalization
        self.distance_marginalization = distance_marginalization
        self.phase_marginalization = phase_marginalization
        self.calibration_marginalization = False
        self.priors = priors
        self._check_set_duration_and_sampling_frequency_of_waveform_generator()
        self._noise_log_likelihood_value = None
        self.jitter_time = jitter_time
        self.reference_frame = reference_frame
        self._model = model_of(waveform_generator.frequency_domain_source_model)
        self._frame = None
        if reference_frame != "sky":
            from .frames import ReferenceFrame
            self._frame = ReferenceFrame(reference_frame)
        if "geocent" not in time_reference:
            self.time_reference = time_reference
            from .detector import get_empty_interferometer
            self.reference_ifo = get_empty_interferometer(time_reference)
            if self.time_marginalization:
                logger.info("Cannot marginalise over non-geocenter time.")
                self.time_marginalization = False
                self.jitter_time = False
        else:
            self.time_reference = "geocent"
            self.reference_ifo = None
        for ifo in self.interferometers:
            cal = getattr(ifo, "calibration_model", None)
            if cal is not None and type(cal).__name__ != "Recalibrate":
                raise NotImplementedError(f"{ifo.name}: only the identity calibration model is supported")

        if self.time_marginalization:
            self._check_marginalized_prior_is_set("geocent_time")
            self._setup_time_marginalization()
            priors["geocent_time"] = float(self._start_time)
            if self.jitter_time:
                priors["time_jitter"] = self._jitter_prior()
            self._marginalized_parameters.append("geocent_time")
        elif self.jitter_time:
            self.jitter_time = False
        if self.phase_marginalization:
            self._check_marginalized_prior_is_set("phase")
            priors["phase"] = float(0)
            self._marginalized_parameters.append("phase")
        if self.distance_marginalization:
            self._lookup_table_filename = None
            self._check_marginalized_prior_is_set("luminosity_distance")
            dprior = self.priors["luminosity_distance"]
            self._distance_array = np.linspace(dprior.minimum, dprior.maximum, int(N_DISTANCE_GRID))
            self.distance_prior_array = np.array([dprior.prob(d) for d in self._distance_array])
            self._ref_dist = dprior.rescale(0.5)
            self._setup_distance_marginalization(distance_marginalization_lookup_table)
            for key in ("redshift", "comoving_distance"):
                if key in priors:
                    del priors[key]
            priors["luminosity_distance"] = float(self._ref_dist)
            self._marginalized_parameters.append("luminosity_distance")
        self._analysis = None
        self._build_analysis()

    # ------------------------------------------------------------------
    # set-up
    # ------------------------------------------------------------------
    def _check_set_duration_and_sampling_frequency_of_waveform_generator(self):
        """base.py:239-258."""
        for attribute in ("duration", "sampling_frequency", "start_time"):
            ifo_attr = getattr(self.interferometers[0].strain_data, attribute)
            for ifo in self.interferometers[1:]:
                if getattr(ifo.strain_data, attribute) != ifo_attr:
                    raise ValueError(f"The {attribute} of all interferometers are not the same")
            setattr(self.waveform_generator, attribute, ifo_attr)

    @property
    def _start_time(self):
        return self.interferometers[0].strain_data.start_time

    @property
    def priors(self):
        return self._prior

    @priors.setter
    def priors(self, priors):
        if priors is not None:
            self._prior = priors.copy()
        elif any([self.time_marginalization, self.phase_marginalization, self.distance_marginalization]):
            raise ValueError("You can't use a marginalized likelihood without specifying a priors")
        else:
            self._prior = None

    def _check_marginalized_prior_is_set(self, key):
        """base.py:356-400 (defaults for missing time / phase priors)."""
        if key in self.priors and _is_fixed(self.priors[key]):
            raise ValueError(f"Cannot use marginalized likelihood for {key}: prior is fixed")
        if key not in self.priors or not hasattr(self.priors[key], "prob"):
            from .prior import Uniform
            if key == "geocent_time":
                logger.warning("Prior not provided for geocent time, using the full segment.")
                self.priors[key] = Uniform(self._start_time, self._start_time + self.interferometers[0].duration)
            elif key == "phase":
                logger.warning("Prior not provided for phase, using the BBH default.")
                self.priors[key] = Uniform(0, 2 * np.pi, boundary="periodic")
            else:
                raise ValueError(f"A prior for {key} is required to marginalise over it")

    def _jitter_prior(self):
        from .prior import Uniform
        try:
            from bilby.core.prior import Uniform as BUniform  # type: ignore
            return BUniform(minimum=-self._delta_tc / 2, maximum=self._delta_tc / 2, boundary="periodic",
                            name="time_jitter", latex_label="$t_j$")
        except Exception:
            return Uniform(-self._delta_tc / 2, self._delta_tc / 2, boundary="periodic", name="time_jitter")

    def _setup_time_marginalization(self):
        """base.py:1027-1035; the GPU path needs a Uniform geocent_time prior."""
        fs = self.waveform_generator.sampling_frequency
        self._delta_tc = 2 / fs
        duration = self.interferometers[0].duration
        self._times = self._start_time + np.linspace(0, duration, int(duration / 2 * fs + 1))[1:]
        tp = self.priors["geocent_time"]
        if type(tp).__name__ != "Uniform":
            raise NotImplementedError("time marginalisation on the GPU needs a Uniform geocent_time prior")
        self.time_prior_array = tp.prob(self._times) * self._delta_tc

    def _setup_distance_marginalization(self, lookup_table=None):
        """base.py:916-992: load a matching cached table or build it (on the GPU)."""
        if isinstance(lookup_table, str) or lookup_table is None:
            self.cached_lookup_table_filename = lookup_table
            lookup_table = self.load_lookup_table(self.cached_lookup_table_filename)
        if isinstance(lookup_table, dict) and self._test_cached_lookup_table(lookup_table)[0]:
            self._dist_margd_loglikelihood_array = np.asarray(lookup_table["lookup_table"])
        else:
            self._create_lookup_table()
        from scipy.interpolate import RectBivariateSpline
        x = self._d_inner_h_ref_array
        y = self._optimal_snr_squared_ref_array
        spline = RectBivariateSpline(x, y, self._dist_margd_loglikelihood_array.T, kx=3, ky=3, s=0)
        self._spline_tck = spline.tck
        self._spline_bbox = np.array([min(x), max(x), min(y), max(y)])

    @property
    def _optimal_snr_squared_ref_array(self):
        return optimal_snr_squared_ref_axis(self._dist_margd_loglikelihood_array.shape[0])

    @property
    def _d_inner_h_ref_array(self):
        return d_inner_h_ref_axis(self._dist_margd_loglikelihood_array.shape[1], self.phase_marginalization)

    @property
    def _delta_distance(self):
        return self._distance_array[1] - self._distance_array[0]

    @property
    def cached_lookup_table_filename(self):
        if self._lookup_table_filename is None:
            self._lookup_table_filename = ".distance_marginalization_lookup.npz"
        return self._lookup_table_filename

    @cached_lookup_table_filename.setter
    def cached_lookup_table_filename(self, filename):
        if isinstance(filename, str) and filename[-4:] != ".npz":
            filename += ".npz"
        self._lookup_table_filename = filename

    def load_lookup_table(self, filename):
        if os.path.exists(filename):
            try:
                loaded = dict(np.load(filename))
            except Exception as e:  # a corrupt cache is rebuilt
                logger.warning(e)
                return None
            match, failure = self._test_cached_lookup_table(loaded)
            if match:
                logger.info(f"Loaded distance marginalisation lookup table from {filename}.")
                return loaded
            logger.info(f"Loaded distance marginalisation lookup table does not match for {failure}.")
        return None

    def cache_lookup_table(self):
        np.savez(self.cached_lookup_table_filename, distance_array=self._distance_array,
                 prior_array=self.distance_prior_array, lookup_table=self._dist_margd_loglikelihood_array,
                 reference_distance=self._ref_dist, phase_marginalization=self.phase_marginalization)

    def _test_cached_lookup_table(self, loaded_file):
        pairs = dict(distance_array=self._distance_array, prior_array=self.distance_prior_array,
                     reference_distance=self._ref_dist, phase_marginalization=self.phase_marginalization)
        for key, value in pairs.items():
            if key not in loaded_file:
                return False, key
            if not np.allclose(np.atleast_1d(loaded_file[key]), np.atleast_1d(value), rtol=1e-15):
                return False, key
        return True, None

    def _create_lookup_table(self):
        """base.py:994-1018, built by a float64 GPU kernel."""
        logger.info("Building lookup table for distance marginalisation.")
        self._dist_margd_loglikelihood_array = _capi.distance_lookup_table(
            self._distance_array, self.distance_prior_array, float(self._ref_dist), self.phase_marginalization)
        self.cache_lookup_table()

    def _build_analysis(self):
        ifos = self.interferometers
        freq = np.asarray(ifos[0].strain_data.frequency_array, dtype=np.float64)
        dets = []
        for ifo in ifos:
            geom = ifo.geometry
            dets.append(DetectorData(ifo.name, np.asarray(geom.vertex, dtype=np.float64),
                                     np.asarray(geom.detector_tensor, dtype=np.float64),
                                     float(ifo.strain_data.start_time),
                                     np.asarray(ifo.strain_data.frequency_domain_strain, dtype=np.complex128),
                                     np.asarray(ifo.power_spectral_density_array, dtype=np.float64),
                                     np.asarray(ifo.strain_data.frequency_mask, dtype=bool)))
        fmin = self.waveform_generator.waveform_arguments.get("minimum_frequency", 20.0)
        an = Analysis(self._model, freq, dets, float(ifos[0].strain_data.duration),
                      float(ifos[0].strain_data.sampling_frequency), fmin)
        if self.time_marginalization:
            tp = self.priors["geocent_time"]
            an.set_time_marginalization(True, self.jitter_time, tp.minimum, tp.maximum)
        if self.phase_marginalization:
            an.set_phase_marginalization(True)
        if self.distance_marginalization:
            tx, ty, c = self._spline_tck
            an.set_distance_marginalization(True, tx, ty, c, self._spline_bbox, self._ref_dist)
        self._analysis = an

    # ------------------------------------------------------------------
    # pickling: the device handle is rebuilt in the receiving process
    # ------------------------------------------------------------------
    def __getstate__(self):
        state = self.__dict__.copy()
        state["_analysis"] = None
        return state

    def __setstate__(self, state):
        self.__dict__.update(state)

    @property
    def analysis(self) -> Analysis:
        if self._analysis is None:
            self._build_analysis()
        return self._analysis

    # ------------------------------------------------------------------
    # the likelihood
    # ------------------------------------------------------------------
    def noise_log_likelihood(self):
        """base.py:413-417 (computed once per analysis when it is created)."""
        if self._noise_log_likelihood_value is None:
            self._noise_log_likelihood_value = self.analysis.noise_log_likelihood()
        return self._noise_log_likelihood_value

    def get_sky_frame_parameters(self, parameters):
        """base.py:1091-1137, vectorised."""
        time = parameters.get(f"{self.time_reference}_time", None)
        if self._frame is not None:
            try:
                ra, dec = self._frame.zenith_azimuth_to_ra_dec(parameters["zenith"], parameters["azimuth"], time)
            except KeyError:
                if "ra" in parameters and "dec" in parameters:
                    ra, dec = parameters["ra"], parameters["dec"]
                else:
                    raise
        else:
            ra, dec = parameters["ra"], parameters["dec"]
        if "geocent" not in self.time_reference and f"{self.time_reference}_time" in parameters:
            from .frames import time_delay_from_geocenter
            geocent_time = time - time_delay_from_geocenter(self.reference_ifo.geometry.vertex, ra, dec, time)
        else:
            geocent_time = parameters["geocent_time"]
        return dict(ra=ra, dec=dec, geocent_time=geocent_time)

    def _prepare(self, parameters: dict) -> dict:
        p = dict(parameters)
        p.update(self.get_sky_frame_parameters(p))
        converted, _ = self.waveform_generator.parameter_conversion(dict(p))
        if self.time_marginalization and self.jitter_time:
            converted["time_jitter"] = p.get("time_jitter", 0.0)
        return converted

    def log_likelihood_ratio(self, parameters):
        """base.py:419-446 for one point: a batch of size one on the GPU."""
        parameters = copy.deepcopy(parameters)
        block = params_block(self._prepare(parameters), 1)
        return float(self.analysis.log_likelihood_ratio_host(block, self.precision)[0])

    def log_likelihood(self, parameters):
        return self.log_likelihood_ratio(parameters) + self.noise_log_likelihood()

    def log_likelihood_ratio_batch(self, parameters, precision=None, out=None):
        """Evaluate a batch.  ``parameters`` maps names to equal-length numpy
        arrays (result: numpy float64) or to CUDA tensors (result: a CUDA
        float64 tensor, computed asynchronously on torch's current stream)."""
        precision = precision or self.precision
        first = next(iter(parameters.values()))
        if hasattr(first, "is_cuda") and first.is_cuda:
            import torch
            n = int(first.shape[0])
            p = {k: v for k, v in parameters.items()}
            host_keys = [k for k in p if not (hasattr(p[k], "is_cuda") and p[k].is_cuda)]
            if host_keys:
                raise ValueError(f"all batch parameters must be CUDA tensors (host: {host_keys})")
            conv = self._prepare(p)
            block = torch.zeros((_capi.NPARAM, n), dtype=torch.float64, device=first.device)
            for key, slot in _capi.SLOT.items():
                if key in conv and conv[key] is not None:
                    v = conv[key]
                    block[slot] = v.to(torch.float64) if hasattr(v, "to") else float(v)
            res = out if out is not None else torch.empty(n, dtype=torch.float64, device=first.device)
            stream = torch.cuda.current_stream(first.device).cuda_stream
            self.analysis.log_likelihood_ratio_device(block.data_ptr(), n, res.data_ptr(), precision, stream)
            return res
        arrays = {k: np.asarray(v, dtype=np.float64) for k, v in parameters.items()}
        return self.analysis.log_likelihood_ratio_staged(self._prepare(arrays), precision)

    def log_likelihood_ratio_from_unit_cube(self, unit, device_priors, precision=None, out=None):
        """lnL ratios of a batch given as unit-cube samples: ``unit`` is a CUDA
        float64 tensor [len(device_priors.keys), B]; the priors' inverse CDFs and
        the mass / inclination conversions run on the device
        (``bilby_gb300.priors_device.DevicePriors``), then the likelihood, all
        on torch's current stream with no host work per point.  Needs the sky
        frame and geocentre time (no detector-frame sampling)."""
        import torch
        if self._frame is not None or self.time_reference != "geocent":
            raise NotImplementedError("unit-cube batches need reference_frame='sky' and geocentre time")
        block = device_priors.rescale(unit)
        n = block.shape[1]
        res = out if out is not None else torch.empty(n, dtype=torch.float64, device=block.device)
        stream = torch.cuda.current_stream(block.device).cuda_stream
        self.analysis.log_likelihood_ratio_device(block.data_ptr(), n, res.data_ptr(), precision or self.precision,
                                                  stream)
        return res

    def autotune(self, parameters) -> tuple[int, float]:
        """Choose the mixed kernel's launch shape for batches like ``parameters``
        (a mapping of names to equal-length arrays): returns the chosen
        split-K depth and the milliseconds of one launch sequence at that depth."""
        import torch
        arrays = {k: np.asarray(v, dtype=np.float64) for k, v in parameters.items()}
        block = torch.from_numpy(params_block(self._prepare(arrays))).cuda()
        res = self.analysis.autotune(block.data_ptr(), block.shape[1], torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        return res

    # ------------------------------------------------------------------
    def __repr__(self):
        return (f"{self.__class__.__name__}(interferometers={[i.name for i in self.interferometers]},\n\t"
                f"waveform_generator={self.waveform_generator},\n\ttime_marginalization={self.time_marginalization}, "
                f"distance_marginalization={self.distance_marginalization}, phase_marginalization="
                f"{self.phase_marginalization}, calibration_marginalization=False, priors={self.priors})")

    @property
    def meta_data(self):
        wfg = self.waveform_generator
        return dict(
            interferometers={ifo.name: dict(minimum_frequency=ifo.strain_data.minimum_frequency,
                                            maximum_frequency=ifo.strain_data.maximum_frequency)
                             for ifo in self.interferometers},
            time_marginalization=self.time_marginalization, phase_marginalization=self.phase_marginalization,
            distance_marginalization=self.distance_marginalization, calibration_marginalization=False,
            waveform_generator_class=wfg.__class__, waveform_arguments=wfg.waveform_arguments,
            frequency_domain_source_model=wfg.frequency_domain_source_model,
            time_domain_source_model=getattr(wfg, "time_domain_source_model", None),
            parameter_conversion=wfg.parameter_conversion, sampling_frequency=wfg.sampling_frequency,
            duration=wfg.duration, start_time=wfg.start_time, time_reference=self.time_reference,
            reference_frame=self.reference_frame if isinstance(self.reference_frame, str) else "".join(
                i.name for i in self.reference_frame),
            lal_version="N/A", lalsimulation_version="N/A", precision=self.precision, backend="gwlnl-sm_103a")
