"""Prior rescaling and parameter conversion on the device, for the batch path.

``DevicePriors(priors, keys)`` compiles a prior dictionary (bilby's priors or
this package's mirrors) into a ``gwl_priors`` program: each sampled key reads
one column of a unit-cube tensor and applies its inverse CDF; fixed priors
become constants; chirp mass / total mass with mass ratio become the
component masses, and cos_theta_jn becomes theta_jn
(bilby/core/prior/dict.py PriorDict.rescale, bilby/gw/conversion.py:182-283),
and with a frame set (``set_frame``) zenith / azimuth and a detector's arrival
time become ra / dec and geocent_time (bilby/gw/likelihood/base.py:1091-1137).
``rescale(unit)`` then maps a [len(keys), B] CUDA float64 tensor to the
[NPARAM, B] parameter block in one launch, so a sampler's unit-cube batch
goes to the likelihood without host work per point
(``GravitationalWaveTransient.log_likelihood_ratio_from_unit_cube``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi

PRIOR_DELTA, PRIOR_UNIFORM, PRIOR_POWERLAW, PRIOR_SINE, PRIOR_COSINE = 0, 1, 2, 3, 4
PRIOR_GAUSSIAN, PRIOR_TRUNCATED_GAUSSIAN, PRIOR_TABLE_LINEAR, PRIOR_TABLE_BSPLINE = 5, 6, 7, 8
TARGETS_EXTRA = {"chirp_mass": 100, "mass_ratio": 101, "total_mass": 102, "cos_theta_jn": 103, "zenith": 104,
                 "azimuth": 105}
TARGET_DETECTOR_TIME = 106  # "<detector>_time": the arrival time at the likelihood's reference detector


class GwlPrior(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("target", ctypes.c_int32), ("column", ctypes.c_int32),
                ("table_n", ctypes.c_int32), ("p", ctypes.c_double * 4),
                ("table_x", ctypes.POINTER(ctypes.c_double)), ("table_y", ctypes.POINTER(ctypes.c_double))]


def _fixed(prior):
    return isinstance(prior, (int, float)) or type(prior).__name__ == "DeltaFunction" or bool(
        getattr(prior, "is_fixed", False))


def compile_prior(prior):
    """(kind, parameters, table_x, table_y) of one prior, by its class."""
    name = type(prior).__name__
    if isinstance(prior, (int, float)):
        return PRIOR_DELTA, [float(prior)], None, None
    if name == "DeltaFunction":
        return PRIOR_DELTA, [float(prior.peak)], None, None
    if name == "Uniform":
        return PRIOR_UNIFORM, [prior.minimum, prior.maximum], None, None
    if name in ("PowerLaw", "LogUniform", "UniformInComponentsChirpMass"):
        alpha = -1.0 if name == "LogUniform" else float(prior.alpha)
        return PRIOR_POWERLAW, [alpha, prior.minimum, prior.maximum], None, None
    if name == "Sine":
        return PRIOR_SINE, [prior.minimum, prior.maximum], None, None
    if name == "Cosine":
        return PRIOR_COSINE, [prior.minimum, prior.maximum], None, None
    if name in ("Gaussian", "Normal"):
        return PRIOR_GAUSSIAN, [prior.mu, prior.sigma], None, None
    if name in ("TruncatedGaussian", "TruncatedNormal", "HalfGaussian", "HalfNormal"):
        return PRIOR_TRUNCATED_GAUSSIAN, [prior.mu, prior.sigma, prior.minimum, prior.normalisation], None, None
    if name == "UniformInComponentsMassRatio":
        icdf = prior.icdf
        spline = icdf._spline  # scipy interp1d(kind="cubic"): the interpolating B-spline
        t = np.ascontiguousarray(spline.t, dtype=np.float64)
        c = np.ascontiguousarray(np.ravel(spline.c), dtype=np.float64)
        if spline.k != 3 or len(c) != len(t) - 4:
            raise NotImplementedError("mass-ratio prior: unexpected inverse-CDF spline")
        lo, hi = icdf.fill_value if isinstance(icdf.fill_value, tuple) else (prior.minimum, prior.maximum)
        return (PRIOR_TABLE_BSPLINE, [float(np.ravel(lo)[0]), float(np.ravel(hi)[0]),
                                      1.0 if getattr(prior, "equal_mass", False) else 0.0, float(icdf.x[-1])], t, c)
    if hasattr(prior, "YY") and hasattr(prior, "xx"):  # Interped, AlignedSpin, FromFile, ...
        return (PRIOR_TABLE_LINEAR, [0.0, 0.0, 0.0, 0.0], np.ascontiguousarray(prior.YY, dtype=np.float64),
                np.ascontiguousarray(prior.xx, dtype=np.float64))
    raise NotImplementedError(f"prior {name} has no device inverse CDF")


def compile_program(priors, keys):
    """The program of ``priors`` for unit-cube columns ``keys``: a list of
    (kind, target, column, parameters[4], table_x, table_y)."""
    program = []
    for key, prior in priors.items():
        if type(prior).__name__ == "Constraint":
            continue
        if key in _capi.SLOT:
            target = _capi.SLOT[key]
        elif key in TARGETS_EXTRA:
            target = TARGETS_EXTRA[key]
        elif key.endswith("_time"):
            target = TARGET_DETECTOR_TIME
        else:
            raise NotImplementedError(f"no device conversion for parameter {key}")
        if key in keys:
            column = keys.index(key)
        elif _fixed(prior):
            column = -1
        else:
            raise ValueError(f"{key} has a non-fixed prior but no unit-cube column")
        kind, p, tx, ty = compile_prior(prior)
        program.append((kind, target, column, list(p) + [0.0] * (4 - len(p)), tx, ty))
    missing = [k for k in keys if k not in priors]
    if missing:
        raise ValueError(f"keys without priors: {missing}")
    return program


class DevicePriors:
    """A compiled prior program (gwl_priors)."""

    def __init__(self, priors=None, keys=None, program=None):
        self._lib = _capi.load()
        if program is None:
            if keys is None:
                keys = [k for k, v in priors.items() if not _fixed(v) and type(v).__name__ != "Constraint"]
            program = compile_program(priors, list(keys))
        self.keys = list(keys)
        entries, self._keep = [], []
        for kind, target, column, p, tx, ty in program:
            e = GwlPrior()
            e.kind, e.target, e.column = int(kind), int(target), int(column)
            for q, v in enumerate(p[:4]):
                e.p[q] = float(v)
            if tx is not None:
                tx = np.ascontiguousarray(tx, dtype=np.float64)
                ty = np.ascontiguousarray(ty, dtype=np.float64)
                self._keep += [tx, ty]
                e.table_n = len(tx)
                e.table_x = _capi.dptr(tx)
                e.table_y = _capi.dptr(ty)
            entries.append(e)
        arr = (GwlPrior * len(entries))(*entries)
        h = ctypes.c_void_p()
        _capi.check(self._lib.gwl_priors_create(arr, len(entries), ctypes.byref(h)), "gwl_priors_create")
        self._h = h

    def rescale(self, unit, out=None, stream=None):
        """unit: CUDA float64 [len(keys), B] -> [NPARAM, B] parameter block (asynchronous on ``stream``)."""
        import torch
        if unit.dtype != torch.float64 or not unit.is_cuda or unit.dim() != 2 or unit.shape[0] != len(self.keys):
            raise ValueError("unit must be a CUDA float64 tensor of shape (len(keys), B)")
        unit = unit.contiguous()
        B = unit.shape[1]
        if out is None:
            out = torch.zeros((_capi.NPARAM, B), dtype=torch.float64, device=unit.device)
        if stream is None:
            stream = torch.cuda.current_stream(unit.device)
        _capi.check(self._lib.gwl_priors_rescale(self._h, ctypes.c_void_p(unit.data_ptr()), int(B),
                                                 ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream)),
                    "gwl_priors_rescale")
        return out

    def set_frame(self, rotation=None, vertex=None):
        """Detector-frame conversion (``gwl_priors_set_frame``): the 3x3 rotation
        of the detector-pair frame and the reference detector's vertex; None
        clears either."""
        r = None if rotation is None else np.ascontiguousarray(rotation, dtype=np.float64).reshape(9)
        v = None if vertex is None else np.ascontiguousarray(vertex, dtype=np.float64).reshape(3)
        self._frame_keep = (r, v)
        _capi.check(self._lib.gwl_priors_set_frame(self._h, None if r is None else _capi.dptr(r),
                                                   None if v is None else _capi.dptr(v)), "gwl_priors_set_frame")

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.gwl_priors_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
