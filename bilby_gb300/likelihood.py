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

# parameters the fused kernels read for each source model: the source model's
# own arguments (bilby/gw/source.py:1153 for the sine-Gaussian) and the
# projection's sky position, polarisation angle and time (interferometer.py:303-368)
_PROJECTION = ("ra", "dec", "psi", "geocent_time")
REQUIRED_PARAMETERS = {
    "sinegaussian": ("hrss", "Q", "frequency") + _PROJECTION,
    "taylorf2": ("mass_1", "mass_2", "chi_1", "chi_2", "luminosity_distance", "theta_jn", "phase") + _PROJECTION,
}


def time_prior_table(prior, t_lo, t_hi, delta_tc):
    """The density of a geocent_time prior for the time-marginalised kernels:
    ``(density, t0, h)`` on the nodes t0 + g h, g < len(density), that lie in
    [max(prior.minimum, t_lo), min(prior.maximum, t_hi)].  h is the power of
    two at most delta_tc / 8 and t0 a multiple of it, so every node time is
    exact in float64 and the kernels' 4-node interpolation reads a time on a
    node exactly; Lagrange interpolation at spacing delta_tc / 8 leaves a
    relative error of order (h / width)^4 for a prior of that width.  Returns
    None for a Uniform prior (a constant weight)."""
    if type(prior).__name__ == "Uniform":
        return None
    lo = max(float(prior.minimum), float(t_lo))
    hi = min(float(prior.maximum), float(t_hi))
    h = 2.0 ** np.floor(np.log2(delta_tc / 8))
    t0 = np.ceil(lo / h) * h
    n = int(np.floor((hi - t0) / h)) + 1
    if n < 4:
        raise ValueError("the geocent_time prior's support is narrower than four table nodes")
    grid = t0 + h * np.arange(n)
    density = np.asarray(prior.prob(grid), dtype=np.float64)
    return np.nan_to_num(density, nan=0.0, posinf=0.0, neginf=0.0), float(t0), float(h)


def d_inner_h_ref_axis(n, phase_marginalization):
    """base.py:904-914."""
    if phase_marginalization:
        return np.logspace(-5, 10, n)
    n_negative = n // 2
    return np.hstack((-np.logspace(3, -3, n_negative), np.logspace(-3, 10, n - n_negative)))


def optimal_snr_squared_ref_axis(n):
    """base.py:899-902."""
    return np.logspace(-5, 10, n)


class ParameterPreparer:
    """The preparation of a sampler's parameter dictionary that precedes the
    likelihood kernels (base.py:419-446): the sky frame
    (``get_sky_frame_parameters``, base.py:1091-1137), the waveform
    generator's ``parameter_conversion`` (waveform_generator.py:260-269) and
    the time jitter of time marginalisation (base.py:427-428).  Raises
    ``KeyError`` when a parameter the source model or the projection needs is
    missing after conversion, as the reference's source-model call does."""

    def __init__(self, model, parameter_conversion, frame=None, time_reference="geocent", reference_vertex=None,
                 jitter=False):
        self.model = model
        self.parameter_conversion = parameter_conversion
        self.frame = frame
        self.time_reference = time_reference
        self.reference_vertex = reference_vertex
        self.jitter = jitter

    def sky_frame(self, parameters):
        time = parameters.get(f"{self.time_reference}_time", None)
        if self.frame is not None:
            try:
                ra, dec = self.frame.zenith_azimuth_to_ra_dec(parameters["zenith"], parameters["azimuth"], time)
            except KeyError:
                if "ra" in parameters and "dec" in parameters:
                    ra, dec = parameters["ra"], parameters["dec"]
                else:
                    raise
        else:
            ra, dec = parameters["ra"], parameters["dec"]
        if "geocent" not in self.time_reference and f"{self.time_reference}_time" in parameters:
            from .frames import time_delay_from_geocenter
            geocent_time = time - time_delay_from_geocenter(self.reference_vertex, ra, dec, time)
        else:
            geocent_time = parameters["geocent_time"]
        return dict(ra=ra, dec=dec, geocent_time=geocent_time)

    def prepare(self, parameters: dict) -> dict:
        p = dict(parameters)
        p.update(self.sky_frame(p))
        converted, _ = self.parameter_conversion(dict(p))
        if self.jitter:
            converted["time_jitter"] = p.get("time_jitter", 0.0)
        missing = [k for k in REQUIRED_PARAMETERS[self.model] if converted.get(k) is None]
        if missing:
            raise KeyError(f"parameters missing after conversion: {missing}")
        return converted

    def block(self, parameters) -> np.ndarray:
        """The [NPARAM, B] float64 block of a dictionary of scalars or
        equal-length arrays; the caller's dictionary is not modified."""
        arrays = {k: (np.asarray(v, dtype=np.float64) if not isinstance(v, str) else v)
                  for k, v in copy.deepcopy(dict(parameters)).items()}
        return params_block(self.prepare(arrays))


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
        self._detector_analyses = {}
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
        """base.py:1027-1035, with the prior's density tabulated for the kernels
        when the geocent_time prior is not Uniform (``time_prior_table``)."""
        fs = self.waveform_generator.sampling_frequency
        self._delta_tc = 2 / fs
        duration = self.interferometers[0].duration
        self._times = self._start_time + np.linspace(0, duration, int(duration / 2 * fs + 1))[1:]
        tp = self.priors["geocent_time"]
        self.time_prior_array = tp.prob(self._times) * self._delta_tc
        self._time_prior_table = time_prior_table(tp, self._start_time - self._delta_tc,
                                                  self._start_time + duration + self._delta_tc, self._delta_tc)

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

    @staticmethod
    def _detector_data(ifo) -> DetectorData:
        geom = ifo.geometry
        return DetectorData(ifo.name, np.asarray(geom.vertex, dtype=np.float64),
                            np.asarray(geom.detector_tensor, dtype=np.float64), float(ifo.strain_data.start_time),
                            np.asarray(ifo.strain_data.frequency_domain_strain, dtype=np.complex128),
                            np.asarray(ifo.power_spectral_density_array, dtype=np.float64),
                            np.asarray(ifo.strain_data.frequency_mask, dtype=bool))

    def _new_analysis(self, ifos) -> Analysis:
        freq = np.asarray(ifos[0].strain_data.frequency_array, dtype=np.float64)
        fmin = self.waveform_generator.waveform_arguments.get("minimum_frequency", 20.0)
        return Analysis(self._model, freq, [self._detector_data(ifo) for ifo in ifos],
                        float(ifos[0].strain_data.duration), float(ifos[0].strain_data.sampling_frequency), fmin)

    def _build_analysis(self):
        an = self._new_analysis(self.interferometers)
        self._configure_analysis(an)
        self._analysis = an

    def _configure_analysis(self, an):
        """The marginalisation settings of this likelihood on a device analysis."""
        if self.time_marginalization:
            tp = self.priors["geocent_time"]
            an.set_time_marginalization(True, self.jitter_time, tp.minimum, tp.maximum)
            table = getattr(self, "_time_prior_table", None)
            if table is not None:
                an.set_time_prior(*table)
        if self.phase_marginalization:
            an.set_phase_marginalization(True)
        if self.distance_marginalization:
            tx, ty, c = self._spline_tck
            an.set_distance_marginalization(True, tx, ty, c, self._spline_bbox, self._ref_dist)
            # E[d_ref / d] under any distance posterior is at most d_ref / d_min
            an.set_distance_slope(max(1.0, float(self._ref_dist) / float(self._distance_array[0])))

    # ------------------------------------------------------------------
    # pickling: the device handle is rebuilt in the receiving process
    # ------------------------------------------------------------------
    def __getstate__(self):
        state = self.__dict__.copy()
        state["_analysis"] = None
        state["_detector_analyses"] = {}
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

    @property
    def preparer(self) -> "ParameterPreparer":
        """What ``log_likelihood_ratio`` does to a parameter dictionary before
        the kernels read it, as a small picklable object (the serving client
        runs it in the sampler's process)."""
        vertex = None if self.reference_ifo is None else np.asarray(self.reference_ifo.geometry.vertex, dtype=np.float64)
        return ParameterPreparer(self._model, self.waveform_generator.parameter_conversion, self._frame,
                                 self.time_reference, vertex, self.time_marginalization and self.jitter_time)

    def get_sky_frame_parameters(self, parameters):
        """base.py:1091-1137, vectorised."""
        return self.preparer.sky_frame(parameters)

    def _prepare(self, parameters: dict) -> dict:
        return self.preparer.prepare(parameters)

    def parameters_block(self, parameters) -> np.ndarray:
        """The [NPARAM, B] float64 block the kernels read, from a sampler's
        parameter dictionary (scalars or equal-length arrays), after the same
        preparation as ``log_likelihood_ratio``.  The caller's dictionary is
        not modified."""
        return self.preparer.block(parameters)

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
        return self._batch_on(self.analysis, parameters, precision or self.precision, out)

    def _batch_on(self, analysis, parameters, precision, out=None):
        """``log_likelihood_ratio_batch`` on a given device analysis."""
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
            analysis.log_likelihood_ratio_device(block.data_ptr(), n, res.data_ptr(), precision, stream)
            return res
        arrays = {k: np.asarray(v, dtype=np.float64) for k, v in parameters.items()}
        return analysis.log_likelihood_ratio_staged(self._prepare(arrays), precision)

    def log_likelihood_ratio_from_unit_cube(self, unit, device_priors, precision=None, out=None):
        """lnL ratios of a batch given as unit-cube samples: ``unit`` is a CUDA
        float64 tensor [len(device_priors.keys), B]; the priors' inverse CDFs and
        the mass / inclination conversions run on the device
        (``bilby_gb300.priors_device.DevicePriors``), then the likelihood, all
        on torch's current stream with no host work per point.  With a
        detector-pair reference frame or a detector time reference the priors'
        zenith / azimuth and ``<detector>_time`` columns become ra / dec and
        geocent_time on the device, as get_sky_frame_parameters does
        (base.py:1091-1137)."""
        import torch
        rotation = None if self._frame is None else np.asarray(self._frame.rotation, dtype=np.float64)
        vertex = None if self.reference_ifo is None else np.asarray(self.reference_ifo.geometry.vertex,
                                                                    dtype=np.float64)
        device_priors.set_frame(rotation, vertex)
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
    # per-detector quantities and posterior reconstruction
    # (base.py:108-148, 260-354, 448-770)
    # ------------------------------------------------------------------
    class _CalculatedSNRs:
        """The inner products of one detector, or their sum over detectors
        (``+`` / ``+=``): base.py:108-148."""
        __slots__ = ("d_inner_h", "optimal_snr_squared", "complex_matched_filter_snr", "d_inner_h_array",
                     "optimal_snr_squared_array")

        def __init__(self, d_inner_h=0j, optimal_snr_squared=0, complex_matched_filter_snr=0j, d_inner_h_array=None,
                     optimal_snr_squared_array=None):
            self.d_inner_h = d_inner_h
            self.optimal_snr_squared = optimal_snr_squared
            self.complex_matched_filter_snr = complex_matched_filter_snr
            self.d_inner_h_array = d_inner_h_array
            self.optimal_snr_squared_array = optimal_snr_squared_array

        def __add__(self, other):
            new = copy.deepcopy(self)
            new += other
            return new

        def __iadd__(self, other):
            # None is the identity of the array slots
            for key in self.__slots__:
                mine, theirs = getattr(self, key), getattr(other, key)
                if mine is None:
                    setattr(self, key, theirs)
                elif theirs is not None:
                    setattr(self, key, mine + theirs)
            return self

        def __repr__(self):
            return (f"_CalculatedSNRs(d_inner_h={self.d_inner_h}, optimal_snr_squared={self.optimal_snr_squared}, "
                    f"complex_matched_filter_snr={self.complex_matched_filter_snr})")

        @property
        def snrs_as_sample(self) -> dict:
            return {"matched_filter_snr": self.complex_matched_filter_snr,
                    "optimal_snr": self.optimal_snr_squared.real ** 0.5}

    def _detector_analysis(self, interferometer) -> Analysis:
        """A device-resident analysis of one detector of this likelihood (built
        on first use), with time marginalisation configured so that the
        float64 transform <d|h>(t) is available."""
        name = interferometer.name
        an = self._detector_analyses.get(name)
        if an is None:
            matches = [ifo for ifo in self.interferometers if ifo.name == name]
            if not matches:
                raise ValueError(f"interferometer {name} is not part of this likelihood")
            an = self._new_analysis(matches[:1])
            if self.time_marginalization:
                tp = self.priors["geocent_time"]
                an.set_time_marginalization(True, False, tp.minimum, tp.maximum)
            self._detector_analyses[name] = an
        return an

    def _snr_block(self, parameters) -> np.ndarray:
        """The parameter block of ``parameters`` as given: sky position, psi and
        geocent_time (already jittered by the caller, as in base.py:427-428)
        are used as they are; the source parameters pass through the waveform
        generator's conversion."""
        converted, _ = self.waveform_generator.parameter_conversion(dict(parameters))
        converted["time_jitter"] = 0.0
        return params_block(converted, 1)

    def calculate_snrs(self, waveform_polarizations, interferometer, *, return_array=True, parameters):
        """The inner products of ``interferometer`` at ``parameters``
        (base.py:260-354): <d|h>, <h|h>, the complex matched-filter SNR and,
        with time marginalisation and ``return_array``, the transform
        d_inner_h_array[j] = 4/T FFT(h conj(d) / S)[j] over the FFT length
        n_frequencies - 1.  All are evaluated in float64 by the fused GPU
        kernels, which generate the source model of this likelihood's waveform
        generator at ``parameters``; ``waveform_polarizations`` (that model at
        the same parameters, in the reference's call) is accepted for the
        reference's signature and not read."""
        an = self._detector_analysis(interferometer)
        block = self._snr_block(parameters)
        dh, hh = an.inner_products_host(block, "fp64")
        # numpy scalars: <h|h> = 0 gives an infinite or NaN matched-filter SNR, as in the reference
        d_inner_h, optimal_snr_squared = np.complex128(dh[0]), np.float64(hh[0])
        d_inner_h_array = None
        if return_array and self.time_marginalization:
            series, _ = an.time_series_host(block)
            d_inner_h_array = series[0]
        with np.errstate(divide="ignore", invalid="ignore"):
            mf = d_inner_h / optimal_snr_squared ** 0.5
        return self._CalculatedSNRs(d_inner_h=d_inner_h, optimal_snr_squared=optimal_snr_squared,
                                    complex_matched_filter_snr=mf, d_inner_h_array=d_inner_h_array)

    def _setup_rho(self, d_inner_h, optimal_snr_squared, parameters):
        """base.py:879-885."""
        scale = parameters["luminosity_distance"] / self._ref_dist
        return d_inner_h * scale, np.real(optimal_snr_squared) * scale ** 2

    def distance_marginalized_likelihood(self, d_inner_h, h_inner_h, *, parameters):
        """base.py:775-784: the lookup table's bicubic spline (the kernels' own
        float64 evaluator, run on the host), -inf outside its box."""
        dh_ref, hh_ref = self._setup_rho(d_inner_h, h_inner_h, parameters)
        dh_ref = np.abs(dh_ref) if self.phase_marginalization else np.real(dh_ref)
        tx, ty, c = self._spline_tck
        x = np.atleast_1d(np.asarray(dh_ref, dtype=np.float64))
        y = np.broadcast_to(np.asarray(hh_ref, dtype=np.float64), x.shape)
        out = _capi.host_bicubic(x, y, tx, ty, c, self._spline_bbox)
        return float(out[0]) if np.ndim(dh_ref) == 0 else out

    def phase_marginalized_likelihood(self, d_inner_h, h_inner_h):
        """base.py:786-792: ln I0(|<d|h>|) - <h|h> / 2."""
        x = np.atleast_1d(np.abs(np.asarray(d_inner_h))).astype(np.float64)
        out = _capi.host_ln_i0(x) - np.real(h_inner_h) / 2
        return float(out[0]) if np.ndim(d_inner_h) == 0 else out

    def time_marginalized_likelihood(self, d_inner_h_tc_array, h_inner_h, *, parameters):
        """base.py:794-820: logsumexp over the time samples inside the
        geocent_time prior, weighted by prior(t) * delta_tc."""
        from scipy.special import logsumexp
        times = self._times
        if self.jitter_time:
            times = self._times + parameters["time_jitter"]
        tp = self.priors["geocent_time"]
        keep = (times >= tp.minimum) & (times <= tp.maximum)
        times = times[keep]
        series = np.asarray(d_inner_h_tc_array)[keep]
        weights = tp.prob(times) * self._delta_tc
        if self.distance_marginalization:
            lnl_t = self.distance_marginalized_likelihood(series, h_inner_h, parameters=parameters)
        elif self.phase_marginalization:
            lnl_t = self.phase_marginalized_likelihood(series, h_inner_h)
        else:
            lnl_t = series.real - np.real(h_inner_h) / 2
        return logsumexp(lnl_t, b=weights)

    def compute_log_likelihood_from_snrs(self, total_snrs, parameters):
        """base.py:448-477 on the host, from inner products already computed
        (by ``calculate_snrs``)."""
        if self.time_marginalization:
            return self.time_marginalized_likelihood(total_snrs.d_inner_h_array, total_snrs.optimal_snr_squared,
                                                     parameters=parameters)
        if self.distance_marginalization:
            return self.distance_marginalized_likelihood(total_snrs.d_inner_h, total_snrs.optimal_snr_squared,
                                                         parameters=parameters)
        if self.phase_marginalization:
            return self.phase_marginalized_likelihood(total_snrs.d_inner_h, total_snrs.optimal_snr_squared)
        return np.real(total_snrs.d_inner_h) - total_snrs.optimal_snr_squared / 2

    def compute_per_detector_log_likelihood(self, parameters):
        """base.py:479-499: adds ``<ifo>_log_likelihood`` to ``parameters`` (in
        place) for every detector and returns a copy."""
        parameters.update(self.get_sky_frame_parameters(parameters))
        if self.time_marginalization and self.jitter_time:
            parameters["geocent_time"] += parameters["time_jitter"]
        for ifo in self.interferometers:
            snrs = self.calculate_snrs(None, ifo, parameters=parameters)
            parameters[f"{ifo.name}_log_likelihood"] = self.compute_log_likelihood_from_snrs(snrs, parameters)
        if self.time_marginalization and self.jitter_time:
            parameters["geocent_time"] -= parameters["time_jitter"]
        return parameters.copy()

    def _calculate_inner_products(self, signal_polarizations, parameters):
        """base.py:707-716: <d|h> and <h|h> summed over detectors."""
        total = self._CalculatedSNRs()
        for ifo in self.interferometers:
            total += self.calculate_snrs(signal_polarizations, ifo, return_array=False, parameters=parameters)
        return total.d_inner_h, total.optimal_snr_squared

    def generate_posterior_sample_from_marginalized_likelihood(self, parameters):
        """base.py:502-541: draw the marginalised parameters (time, then
        distance, then phase) from their conditional posteriors at
        ``parameters``, with the package's shared random generator."""
        if len(self._marginalized_parameters) == 0:
            return parameters
        if self.time_marginalization:
            parameters["geocent_time"] = self.generate_time_sample_from_marginalized_likelihood(
                parameters=parameters)
        if self.distance_marginalization:
            parameters["luminosity_distance"] = self.generate_distance_sample_from_marginalized_likelihood(
                parameters=parameters)
        if self.phase_marginalization:
            parameters["phase"] = self.generate_phase_sample_from_marginalized_likelihood(parameters=parameters)
        return parameters.copy()

    def generate_time_sample_from_marginalized_likelihood(self, signal_polarizations=None, *, parameters):
        """base.py:577-653: the time posterior on a 16384 Hz grid.  The
        detector responses come from the GPU (the source and response
        kernels); the zero-padded transform and the draw are host work, as in
        the reference."""
        from .prior import Interped
        parameters.update(self.get_sky_frame_parameters(parameters))
        if self.jitter_time:
            parameters["geocent_time"] += parameters["time_jitter"]
        if signal_polarizations is None:
            signal_polarizations = self.waveform_generator.frequency_domain_strain(parameters)
        fs_up = 16384
        wfg = self.waveform_generator
        n_up = int(wfg.duration * fs_up)
        t0 = parameters["geocent_time"] - wfg.start_time  # core/utils/series.py:91-112
        times = np.linspace(t0, wfg.duration + t0 - 1 / fs_up, num=n_up)
        times = times % wfg.duration + wfg.start_time
        tp = self.priors["geocent_time"]
        in_prior = (times >= tp.minimum) & (times < tp.maximum)
        times = times[in_prior]
        d_inner_h = np.zeros(len(times), dtype=complex)
        psd = np.ones(n_up)
        signal_long = np.zeros(n_up, dtype=complex)
        data = np.zeros(n_up, dtype=complex)
        h_inner_h = np.zeros(1)
        for ifo in self.interferometers:
            n_ifo = len(ifo.frequency_domain_strain)
            mask = ifo.frequency_mask
            signal = self._compute_full_waveform(signal_polarizations, ifo, parameters)
            signal_long[:n_ifo] = signal
            data[:n_ifo] = np.conj(ifo.frequency_domain_strain)
            psd[:n_ifo][mask] = ifo.power_spectral_density_array[mask]
            d_inner_h += np.fft.fft(signal_long * data / psd)[in_prior]
            h_inner_h += ifo.optimal_snr_squared(signal=signal).real
        if self.distance_marginalization:
            lnl_t = self.distance_marginalized_likelihood(d_inner_h, h_inner_h, parameters=parameters)
        elif self.phase_marginalization:
            lnl_t = self.phase_marginalized_likelihood(d_inner_h, h_inner_h)
        else:
            lnl_t = d_inner_h.real - h_inner_h.real / 2
        post = np.exp(lnl_t - np.max(lnl_t)) * tp.prob(times)
        keep = post > np.max(post) / 1000
        if np.sum(keep) < 3:
            keep[1:-1] = keep[1:-1] | keep[2:] | keep[:-2]
        return Interped(times[keep], post[keep]).sample()

    def _compute_full_waveform(self, signal_polarizations, interferometer, parameters):
        """base.py:718-732: the detector response on the full grid (the GPU's
        response kernel for this package's interferometers)."""
        return interferometer.get_detector_response(signal_polarizations, parameters)

    def generate_distance_sample_from_marginalized_likelihood(self, signal_polarizations=None, *, parameters):
        """base.py:655-705: the distance posterior on the lookup table's
        distance grid."""
        from .prior import Interped
        parameters.update(self.get_sky_frame_parameters(parameters))
        d_inner_h, h_inner_h = self._calculate_inner_products(signal_polarizations, parameters)
        ratio = parameters["luminosity_distance"] / self._distance_array
        dh = d_inner_h * ratio
        hh = h_inner_h * ratio ** 2
        if self.phase_marginalization:
            lnl_d = self.phase_marginalized_likelihood(dh, hh)
        else:
            lnl_d = dh.real - hh.real / 2
        post = np.exp(lnl_d - np.max(lnl_d)) * self.distance_prior_array
        new_distance = Interped(self._distance_array, post).sample()
        if signal_polarizations is not None:  # base.py:1061-1063: rescaled in place
            for mode in signal_polarizations:
                signal_polarizations[mode] *= self._ref_dist / new_distance
        return new_distance

    def generate_phase_sample_from_marginalized_likelihood(self, signal_polarizations=None, *, parameters):
        """base.py:734-770: the phase posterior on 101 phases in [0, 2 pi],
        for a signal whose phase enters as exp(-2 i phase)."""
        from .prior import Interped
        parameters.update(self.get_sky_frame_parameters(parameters))
        d_inner_h, h_inner_h = self._calculate_inner_products(signal_polarizations, parameters)
        phases = np.linspace(0, 2 * np.pi, 101)
        log_post = (d_inner_h * np.exp(-2j * phases) - h_inner_h / 2).real
        post = np.exp(log_post - np.max(log_post))
        return Interped(phases, post).sample()

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
