"""ctypes binding of the C ABI in ``include/gwlnl.h`` (``libgwlnl.so``).

There is no CPU fallback: if the shared library is missing or cannot be
loaded, every entry point raises.  Build the library with
``python -m bilby_gb300._build`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _build

GWL_OK = 0
GWL_ERR_ARGUMENT = 1
GWL_ERR_CUDA = 2
GWL_ERR_MEMORY = 3
GWL_ERR_UNSUPPORTED = 4
GWL_ERR_TIMEOUT = 5
GWL_ERR_STATE = 6
GWL_ERR_CHECK = 7

MODEL_SINEGAUSSIAN = 1
MODEL_TAYLORF2 = 2
PRECISION_FP64 = 0
PRECISION_MIXED = 1
MAX_DETECTORS = 4

# slots of the [GWL_NPARAM][B] parameter block (gwl_param in gwlnl.h)
PARAM_SLOTS = ("ra", "dec", "psi", "geocent_time", "time_jitter", "hrss", "Q", "frequency",
               "mass_1", "mass_2", "chi_1", "chi_2", "luminosity_distance", "theta_jn", "phase")
NPARAM = len(PARAM_SLOTS)
SLOT = {k: i for i, k in enumerate(PARAM_SLOTS)}

c_double_p = ctypes.POINTER(ctypes.c_double)
c_uint8_p = ctypes.POINTER(ctypes.c_uint8)


class GwlDetector(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 8), ("vertex", ctypes.c_double * 3), ("tensor", ctypes.c_double * 9),
                ("start_time", ctypes.c_double), ("strain", c_double_p), ("psd", c_double_p), ("mask", c_uint8_p)]


class GwlAnalysisDesc(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("n_detectors", ctypes.c_int32), ("n_bins", ctypes.c_int64),
                ("duration", ctypes.c_double), ("sampling_frequency", ctypes.c_double),
                ("minimum_frequency", ctypes.c_double), ("frequency", c_double_p),
                ("detectors", ctypes.POINTER(GwlDetector))]


class GwlBatchItem(ctypes.Structure):
    _fields_ = [("analysis", ctypes.c_void_p), ("params", ctypes.c_void_p), ("B", ctypes.c_int64),
                ("out", ctypes.c_void_p)]


# every symbol include/gwlnl.h declares, with (restype, argtypes)
SIGNATURES = {
    "gwl_analysis_create": (ctypes.c_int, [ctypes.POINTER(GwlAnalysisDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "gwl_analysis_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gwl_analysis_resident_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "gwl_noise_log_likelihood": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "gwl_set_time_marginalization": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                    ctypes.c_double]),
    "gwl_set_time_prior": (ctypes.c_int, [ctypes.c_void_p, c_double_p, ctypes.c_int64, ctypes.c_double,
                                          ctypes.c_double]),
    "gwl_set_phase_marginalization": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gwl_set_distance_marginalization": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, c_double_p, ctypes.c_int32,
                                                        c_double_p, ctypes.c_int32, c_double_p, c_double_p,
                                                        ctypes.c_double]),
    "gwl_eval_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.c_void_p]),
    "gwl_eval_host": (ctypes.c_int, [ctypes.c_void_p, c_double_p, ctypes.c_int64, ctypes.c_int32, c_double_p]),
    "gwl_eval_device_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                               ctypes.c_void_p]),
    "gwl_noalloc_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "gwl_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                                 ctypes.POINTER(ctypes.c_int)]),
    "gwl_inject_device_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gwl_inner_products_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "gwl_time_series_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p]),
    "gwl_source_polarizations": (ctypes.c_int, [ctypes.c_int32, c_double_p, ctypes.c_int64, c_double_p,
                                                ctypes.c_double, c_double_p, c_double_p]),
    "gwl_detector_response": (ctypes.c_int, [ctypes.POINTER(GwlDetector), c_double_p, ctypes.c_int64, c_double_p,
                                             c_double_p, c_double_p, c_double_p]),
    "gwl_distance_lookup_table": (ctypes.c_int, [c_double_p, c_double_p, ctypes.c_int32, ctypes.c_double,
                                                 c_double_p, ctypes.c_int32, c_double_p, ctypes.c_int32,
                                                 ctypes.c_int, c_double_p]),
    "gwl_host_math": (ctypes.c_int, [ctypes.c_int, c_double_p, c_double_p, ctypes.c_int64, c_double_p,
                                     ctypes.c_int32, c_double_p, ctypes.c_int32, c_double_p, c_double_p, c_double_p]),
    "gwl_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gwl_profile_last_kernel_ms": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "gwl_set_roq_time_marginalization": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, c_double_p,
                                                       ctypes.c_double, ctypes.c_double]),
    "gwl_set_multiband_time_marginalization": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                                             ctypes.c_void_p, ctypes.c_double, ctypes.c_double]),
    "gwl_set_relative_binning_time_weights": (ctypes.c_int, [ctypes.c_void_p, c_double_p]),
    "gwl_set_relative_binning": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int32,
                                                ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_double)]),
    "gwl_set_multiband_ifft_fft": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                  c_double_p, c_double_p, c_double_p]),
    "gwl_set_multiband": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                         ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                         ctypes.POINTER(ctypes.c_double)]),
    "gwl_set_roq": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                   ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.c_int64, ctypes.c_int64,
                                   ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(ctypes.c_double)]),
    "gwl_priors_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "gwl_priors_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gwl_priors_rescale": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "gwl_priors_set_frame": (ctypes.c_int, [ctypes.c_void_p, c_double_p, c_double_p]),
    "gwl_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                    ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)]),
    "gwl_get_chunks_per_group": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    "gwl_set_chunks_per_group": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "gwl_set_refinement": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "gwl_host_buffers": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                                        ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]),
    "gwl_eval_host_staged": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32]),
    "gwl_get_refinement": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "gwl_last_refined": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "gwl_batcher_last_refined": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "gwl_batcher_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p)]),
    "gwl_batcher_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gwl_batcher_use_graphs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gwl_batcher_eval": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(GwlBatchItem), ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_void_p]),
    "gwl_batcher_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "gwl_last_error": (ctypes.c_char_p, []),
    "gwl_version": (ctypes.c_char_p, []),
    "gwl_set_distance_slope": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "gwl_trace_push": (ctypes.c_int, [ctypes.c_char_p]),
    "gwl_trace_pop": (ctypes.c_int, []),
}

_LIB = None
_LOCK = threading.Lock()


def library_path() -> str:
    """``libgwlnl.so``, or the index-checked debug build ``libgwlnl_check.so``
    when the environment sets ``GWL_CHECKED=1``."""
    return _build.CHECKED_LIB_PATH if os.environ.get("GWL_CHECKED") == "1" else _build.LIB_PATH


def load():
    """Load ``libgwlnl.so`` (raises if it has not been built)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"bilby_gb300 CUDA library not found at {path}; build it with `python -m bilby_gb300._build`. "
                "There is no CPU fallback.")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def check(status: int, what: str = ""):
    if status == GWL_OK:
        return
    msg = load().gwl_last_error().decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if status == GWL_ERR_ARGUMENT:
        raise ValueError(text)
    if status == GWL_ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    if status == GWL_ERR_MEMORY:
        raise MemoryError(text)
    if status == GWL_ERR_TIMEOUT:
        raise TimeoutError(text)
    raise RuntimeError(f"gwlnl error {status}: {text}")


def dptr(a: np.ndarray):
    return a.ctypes.data_as(c_double_p)


def source_polarizations(model: int, frequency, params: np.ndarray, minimum_frequency: float = 20.0):
    """Float64 polarisations of one point, evaluated on the GPU."""
    f = np.ascontiguousarray(frequency, dtype=np.float64)
    p = np.ascontiguousarray(params, dtype=np.float64)
    plus = np.empty(2 * len(f))
    cross = np.empty(2 * len(f))
    check(load().gwl_source_polarizations(model, dptr(f), len(f), dptr(p), float(minimum_frequency),
                                          dptr(plus), dptr(cross)), "gwl_source_polarizations")
    return plus.view(np.complex128), cross.view(np.complex128)


def make_detector_struct(name, vertex, tensor, start_time, strain=None, psd=None, mask=None, keep=None):
    d = GwlDetector()
    d.name = name.encode()[:7]
    for i in range(3):
        d.vertex[i] = float(vertex[i])
    t = np.asarray(tensor, dtype=np.float64).reshape(9)
    for i in range(9):
        d.tensor[i] = float(t[i])
    d.start_time = float(start_time)
    if strain is not None:
        s = np.ascontiguousarray(np.asarray(strain, dtype=np.complex128)).view(np.float64)
        d.strain = dptr(s)
        keep.append(s)
    if psd is not None:
        p = np.ascontiguousarray(psd, dtype=np.float64)
        d.psd = dptr(p)
        keep.append(p)
    if mask is not None:
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        d.mask = m.ctypes.data_as(c_uint8_p)
        keep.append(m)
    return d


def detector_response(name, vertex, tensor, start_time, mask, frequency, plus, cross, params):
    keep = []
    det = make_detector_struct(name, vertex, tensor, start_time, mask=mask, keep=keep)
    f = np.ascontiguousarray(frequency, dtype=np.float64)
    pl = np.ascontiguousarray(plus, dtype=np.complex128).view(np.float64)
    cr = np.ascontiguousarray(cross, dtype=np.complex128).view(np.float64)
    p = np.ascontiguousarray(params, dtype=np.float64)
    out = np.empty(2 * len(f))
    check(load().gwl_detector_response(ctypes.byref(det), dptr(f), len(f), dptr(pl), dptr(cr), dptr(p), dptr(out)),
          "gwl_detector_response")
    return out.view(np.complex128)


def distance_lookup_table(distance, prior, ref_dist, phase_marginalization, n_hh=400, n_dh=800):
    """The 400 x 800 distance-marginalisation table (base.py:994-1018), built on the GPU."""
    from .likelihood import d_inner_h_ref_axis, optimal_snr_squared_ref_axis
    d = np.ascontiguousarray(distance, dtype=np.float64)
    p = np.ascontiguousarray(prior, dtype=np.float64)
    dh = np.ascontiguousarray(d_inner_h_ref_axis(n_dh, phase_marginalization))
    hh = np.ascontiguousarray(optimal_snr_squared_ref_axis(n_hh))
    out = np.empty((n_hh, n_dh), dtype=np.float64)
    check(load().gwl_distance_lookup_table(dptr(d), dptr(p), len(d), float(ref_dist), dptr(dh), n_dh, dptr(hh), n_hh,
                                           int(bool(phase_marginalization)), dptr(out)), "gwl_distance_lookup_table")
    return out


def host_ln_i0(x):
    """ln I0 evaluated by the library's host build of its device function (no GPU needed)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    check(load().gwl_host_math(0, dptr(x), None, x.size, None, 0, None, 0, None, None, dptr(out)), "gwl_host_math")
    return out


def host_bicubic(x, y, tx, ty, c, bbox):
    """The library's bicubic spline evaluated on the host (no GPU needed)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    tx = np.ascontiguousarray(tx, dtype=np.float64)
    ty = np.ascontiguousarray(ty, dtype=np.float64)
    c = np.ascontiguousarray(c, dtype=np.float64)
    bb = np.ascontiguousarray(bbox, dtype=np.float64)
    out = np.empty_like(x)
    check(load().gwl_host_math(1, dptr(x), dptr(y), x.size, dptr(tx), len(tx), dptr(ty), len(ty), dptr(c), dptr(bb),
                               dptr(out)), "gwl_host_math")
    return out
