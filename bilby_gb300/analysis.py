"""Python owner of one device-resident analysis handle (``gwl_analysis``).

An :class:`Analysis` is built from plain arrays (what bilby's
``Interferometer`` objects expose) and evaluates ``log_likelihood_ratio``
for batches of parameter points through the C ABI.  The likelihood class in
:mod:`bilby_gb300.likelihood` and the serving loop in
:mod:`bilby_gb300.serving` sit on top of it.
"""
from __future__ import annotations

import ctypes
import threading
from dataclasses import dataclass

import numpy as np

from . import _capi

PRECISIONS = {"fp64": _capi.PRECISION_FP64, "mixed": _capi.PRECISION_MIXED}


@dataclass
class DetectorData:
    """The per-detector inputs of the likelihood (one ``Interferometer``)."""
    name: str
    vertex: np.ndarray        # geometry.vertex (m)
    tensor: np.ndarray        # geometry.detector_tensor (3x3)
    start_time: float         # strain_data.start_time
    strain: np.ndarray        # masked frequency_domain_strain (complex128)
    psd: np.ndarray           # power_spectral_density_array
    mask: np.ndarray          # frequency_mask (bool)


def params_block(params: dict, n: int | None = None) -> np.ndarray:
    """Pack a dict of scalars / arrays into the [NPARAM, B] float64 block.
    Slots the model does not use may be absent (filled with zeros)."""
    if n is None:
        n = 1
        for v in params.values():
            s = np.shape(v)
            if len(s):
                n = max(n, s[0])
    block = np.zeros((_capi.NPARAM, n), dtype=np.float64)
    for key, slot in _capi.SLOT.items():
        if key in params and params[key] is not None:
            block[slot] = np.broadcast_to(np.asarray(params[key], dtype=np.float64), (n,))
    return block


class Analysis:
    """A device-resident analysis: data, PSD, geometry and derived tables."""

    def __init__(self, model: str, frequency: np.ndarray, detectors: list[DetectorData], duration: float,
                 sampling_frequency: float, minimum_frequency: float = 20.0):
        self._lib = _capi.load()
        self._staged_lock = threading.Lock()
        self.model = model
        self.model_id = {"sinegaussian": _capi.MODEL_SINEGAUSSIAN, "taylorf2": _capi.MODEL_TAYLORF2}[model]
        self.n_detectors = len(detectors)
        if not 1 <= self.n_detectors <= _capi.MAX_DETECTORS:
            raise ValueError(f"between 1 and {_capi.MAX_DETECTORS} detectors are supported")
        self.frequency = np.ascontiguousarray(frequency, dtype=np.float64)
        self.n_bins = len(self.frequency)
        self.duration = float(duration)
        self.sampling_frequency = float(sampling_frequency)
        keep: list = []
        arr = (_capi.GwlDetector * self.n_detectors)()
        for i, d in enumerate(detectors):
            if len(d.strain) != self.n_bins or len(d.psd) != self.n_bins or len(d.mask) != self.n_bins:
                raise ValueError(f"detector {d.name}: strain/psd/mask length differs from the frequency array")
            arr[i] = _capi.make_detector_struct(d.name, d.vertex, d.tensor, d.start_time, d.strain, d.psd,
                                                d.mask, keep)
        desc = _capi.GwlAnalysisDesc()
        desc.model = self.model_id
        desc.n_detectors = self.n_detectors
        desc.n_bins = self.n_bins
        desc.duration = self.duration
        desc.sampling_frequency = self.sampling_frequency
        desc.minimum_frequency = float(minimum_frequency)
        desc.frequency = _capi.dptr(self.frequency)
        desc.detectors = arr
        handle = ctypes.c_void_p()
        _capi.check(self._lib.gwl_analysis_create(ctypes.byref(desc), ctypes.byref(handle)), "gwl_analysis_create")
        self._h = handle
        self._host_out = None
        self.time_marginalization = False
        self.phase_marginalization = False
        self.distance_marginalization = False

    # -- configuration -----------------------------------------------------
    def set_time_marginalization(self, enable: bool, jitter: bool, t_min: float, t_max: float):
        _capi.check(self._lib.gwl_set_time_marginalization(self._h, int(enable), int(jitter), float(t_min),
                                                           float(t_max)), "gwl_set_time_marginalization")
        self.time_marginalization = bool(enable)

    def set_time_prior(self, density=None, t0: float = 0.0, h: float = 1.0):
        """A geocent_time prior other than Uniform (``gwl_set_time_prior``):
        its density on the nodes t0 + g h; None returns to Uniform."""
        if density is None:
            _capi.check(self._lib.gwl_set_time_prior(self._h, None, 0, 0.0, 1.0), "gwl_set_time_prior")
            return
        d = np.ascontiguousarray(density, dtype=np.float64)
        _capi.check(self._lib.gwl_set_time_prior(self._h, _capi.dptr(d), len(d), float(t0), float(h)),
                    "gwl_set_time_prior")

    def set_phase_marginalization(self, enable: bool):
        _capi.check(self._lib.gwl_set_phase_marginalization(self._h, int(enable)), "gwl_set_phase_marginalization")
        self.phase_marginalization = bool(enable)

    def set_distance_slope(self, max_slope: float):
        """The bound d_ref / d_min on the distance-marginalised lnL's slope in
        <d|h>, by which the mixed kernels scale their error bounds."""
        _capi.check(self._lib.gwl_set_distance_slope(self._h, float(max_slope)), "gwl_set_distance_slope")

    def set_distance_marginalization(self, enable: bool, tx=None, ty=None, coeffs=None, bbox=None,
                                     reference_distance=0.0):
        if not enable:
            _capi.check(self._lib.gwl_set_distance_marginalization(self._h, 0, None, 0, None, 0, None, None, 0.0))
            self.distance_marginalization = False
            return
        tx = np.ascontiguousarray(tx, dtype=np.float64)
        ty = np.ascontiguousarray(ty, dtype=np.float64)
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        bb = np.ascontiguousarray(bbox, dtype=np.float64)
        if c.size != (len(tx) - 4) * (len(ty) - 4):
            raise ValueError("spline coefficient count does not match the knot vectors")
        _capi.check(self._lib.gwl_set_distance_marginalization(
            self._h, 1, _capi.dptr(tx), len(tx), _capi.dptr(ty), len(ty), _capi.dptr(c), _capi.dptr(bb),
            float(reference_distance)), "gwl_set_distance_marginalization")
        self.distance_marginalization = True

    def set_relative_binning(self, enable: bool, edge_index=None, h0_inverse=None, summary=None):
        """Relative binning: ``edge_index`` [n_edges] increasing grid indices,
        ``h0_inverse`` [n_det, n_edges] complex 1 / h0 at the edges,
        ``summary`` [n_det, n_edges - 1, 6] (a0 re, a0 im, a1 re, a1 im, b0, b1)."""
        if not enable:
            _capi.check(self._lib.gwl_set_relative_binning(self._h, 0, 0, None, None, None),
                        "gwl_set_relative_binning")
            self.relative_binning = False
            return
        idx = np.ascontiguousarray(edge_index, dtype=np.int64)
        h = np.ascontiguousarray(np.asarray(h0_inverse, dtype=np.complex128).view(np.float64))
        sm = np.ascontiguousarray(summary, dtype=np.float64)
        if h.size != 2 * self.n_detectors * len(idx) or sm.size != 6 * self.n_detectors * (len(idx) - 1):
            raise ValueError("relative-binning arrays do not match the detectors and bin edges")
        _capi.check(self._lib.gwl_set_relative_binning(
            self._h, 1, len(idx), idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _capi.dptr(h),
            _capi.dptr(sm)), "gwl_set_relative_binning")
        self.relative_binning = True

    def set_relative_binning_time_weights(self, weights):
        """``weights`` [n_det, n_bins] complex: 4/T h0_d conj(d) / S on the full
        grid, for relative binning with time marginalisation."""
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.complex128).view(np.float64))
        if w.size != 2 * self.n_detectors * self.n_bins:
            raise ValueError("time weights must have shape (n_detectors, n_bins)")
        _capi.check(self._lib.gwl_set_relative_binning_time_weights(self._h, _capi.dptr(w)),
                    "gwl_set_relative_binning_time_weights")

    def set_roq_time_marginalization(self, times, delta_tc: float, antenna_time: float):
        """ROQ with time marginalisation: the marginalisation grid ``times``
        (absolute, increasing), its spacing and the antenna time."""
        t = np.ascontiguousarray(times, dtype=np.float64)
        _capi.check(self._lib.gwl_set_roq_time_marginalization(self._h, len(t), _capi.dptr(t), float(delta_tc),
                                                               float(antenna_time)),
                    "gwl_set_roq_time_marginalization")
        self.time_fft_length = len(t)  # the length of its <d|h>(t) series

    def set_multiband_time_marginalization(self, n_fft: int, index_start, source, delta_tc: float,
                                           antenna_time: float):
        """Multi-banding with time marginalisation: for each full-resolution
        index k < n_fft, ``source[index_start[k]:index_start[k + 1]]`` are the
        banded points scattered there (a negative code -j - 1: point j, in
        <h|h> only)."""
        ptr = np.ascontiguousarray(index_start, dtype=np.int32)
        src = np.ascontiguousarray(source, dtype=np.int32)
        if len(ptr) != n_fft + 1:
            raise ValueError("index_start must have n_fft + 1 entries")
        _capi.check(self._lib.gwl_set_multiband_time_marginalization(
            self._h, int(n_fft), ptr.ctypes.data_as(ctypes.c_void_p), src.ctypes.data_as(ctypes.c_void_p),
            float(delta_tc), float(antenna_time)), "gwl_set_multiband_time_marginalization")
        self.time_fft_length = int(n_fft)

    def set_multiband(self, enable: bool, frequencies=None, linear=None, quadratic=None, band_start=None,
                      band_df=None):
        """Multi-banding: ``frequencies`` [K] banded frequencies, ``linear``
        [n_det, K] complex and ``quadratic`` [n_det, K] real coefficients;
        band b holds frequencies [band_start[b], band_start[b + 1]) spaced by
        band_df[b]."""
        if not enable:
            _capi.check(self._lib.gwl_set_multiband(self._h, 0, 0, None, None, None, 0, None, None),
                        "gwl_set_multiband")
            self.multiband = False
            return
        f = np.ascontiguousarray(frequencies, dtype=np.float64)
        lin = np.ascontiguousarray(np.asarray(linear, dtype=np.complex128).view(np.float64))
        quad = np.ascontiguousarray(quadratic, dtype=np.float64)
        if lin.size != 2 * self.n_detectors * len(f) or quad.size != self.n_detectors * len(f):
            raise ValueError("multi-banding coefficients do not match the detectors and banded frequencies")
        bs = np.ascontiguousarray(band_start, dtype=np.int64)
        bd = np.ascontiguousarray(band_df, dtype=np.float64)
        if len(bs) != len(bd) + 1:
            raise ValueError("band_start needs one more entry than band_df")
        _capi.check(self._lib.gwl_set_multiband(self._h, 1, len(f), _capi.dptr(f), _capi.dptr(lin),
                                                _capi.dptr(quad), len(bd),
                                                bs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _capi.dptr(bd)),
                    "gwl_set_multiband")
        self.multiband = True

    def set_multiband_ifft_fft(self, enable: bool, ks=None, m=None, scale=None, sqrt_window=None,
                               odd_weights=None):
        """Multi-banding with the IFFT-FFT <h|h>, after :meth:`set_multiband`:
        per band b >= 1 the transform length ``m[b]`` (``m[0] = 0``), its first
        bin ``ks[b]``, ``scale[b] = 4 / That_b``; ``sqrt_window`` [K] the
        roots of the band windows; ``odd_weights`` [n_det, sum_b m[b] / 2]
        the odd-bin weights Re I_b[2j + 1], band after band."""
        if not enable:
            _capi.check(self._lib.gwl_set_multiband_ifft_fft(self._h, 0, None, None, None, None, None),
                        "gwl_set_multiband_ifft_fft")
            return
        ks = np.ascontiguousarray(ks, dtype=np.int32)
        m = np.ascontiguousarray(m, dtype=np.int32)
        sc = np.ascontiguousarray(scale, dtype=np.float64)
        sw = np.ascontiguousarray(sqrt_window, dtype=np.float64)
        od = np.ascontiguousarray(odd_weights, dtype=np.float64)
        n_odd = int(np.sum(m[1:] // 2))
        if len(ks) != len(m) or len(sc) != len(m) or od.size != self.n_detectors * n_odd:
            raise ValueError("IFFT-FFT tables do not match the bands and detectors")
        _capi.check(self._lib.gwl_set_multiband_ifft_fft(
            self._h, 1, ks.ctypes.data_as(ctypes.c_void_p), m.ctypes.data_as(ctypes.c_void_p), _capi.dptr(sc),
            _capi.dptr(sw), _capi.dptr(od)), "gwl_set_multiband_ifft_fft")

    def set_roq(self, enable: bool, nodes_linear=None, nodes_quadratic=None, time_start_index=0, time_step=0.0,
                linear_weights=None, quadratic_weights=None):
        """Reduced-order quadrature: ``linear_weights`` [n_det, n_time,
        n_linear] complex on the time grid (time_start_index + k) time_step,
        ``quadratic_weights`` [n_det, n_quadratic] real."""
        if not enable:
            _capi.check(self._lib.gwl_set_roq(self._h, 0, 0, None, 0, None, 0, 0, 0.0, None, None), "gwl_set_roq")
            self.roq = False
            return
        fl = np.ascontiguousarray(nodes_linear, dtype=np.float64)
        fq = np.ascontiguousarray(nodes_quadratic, dtype=np.float64)
        wl = np.ascontiguousarray(np.asarray(linear_weights, dtype=np.complex128))
        wq = np.ascontiguousarray(quadratic_weights, dtype=np.float64)
        if wl.ndim != 3 or wl.shape[0] != self.n_detectors or wl.shape[2] != len(fl) or \
                wq.shape != (self.n_detectors, len(fq)):
            raise ValueError("ROQ weights do not match the detectors and nodes")
        wlf = wl.view(np.float64)
        _capi.check(self._lib.gwl_set_roq(self._h, 1, len(fl), _capi.dptr(fl), len(fq), _capi.dptr(fq),
                                          wl.shape[1], int(time_start_index), float(time_step), _capi.dptr(wlf),
                                          _capi.dptr(wq)), "gwl_set_roq")
        self.roq = True

    # -- queries -----------------------------------------------------------
    def noise_log_likelihood(self) -> float:
        out = ctypes.c_double()
        _capi.check(self._lib.gwl_noise_log_likelihood(self._h, ctypes.byref(out)), "gwl_noise_log_likelihood")
        return out.value

    def resident_bytes(self) -> int:
        out = ctypes.c_size_t()
        _capi.check(self._lib.gwl_analysis_resident_bytes(self._h, ctypes.byref(out)))
        return int(out.value)

    def log_likelihood_ratio_host(self, block: np.ndarray, precision: str = "fp64") -> np.ndarray:
        """Host parameter block [NPARAM, B] -> host float64 [B] (synchronous)."""
        block = np.ascontiguousarray(block, dtype=np.float64)
        if block.ndim != 2 or block.shape[0] != _capi.NPARAM:
            raise ValueError("parameter block must have shape (NPARAM, B)")
        B = block.shape[1]
        out = np.empty(B, dtype=np.float64)
        _capi.check(self._lib.gwl_eval_host(self._h, _capi.dptr(block), B, PRECISIONS[precision], _capi.dptr(out)),
                    "gwl_eval_host")
        return out

    def log_likelihood_ratio_staged(self, params: dict, precision: str = "fp64") -> np.ndarray:
        """Like log_likelihood_ratio_host for a dict of equal-length arrays, with the
        parameter block written straight into the library's pinned staging
        buffer (gwl_host_buffers / gwl_eval_host_staged): no block allocation
        and no host copies inside the library."""
        n = 1
        for v in params.values():
            sh = np.shape(v)
            if len(sh):
                n = max(n, sh[0])
        with self._staged_lock:  # the staging buffer is shared by the calls on this analysis
            return self._staged(params, n, precision)

    def _staged(self, params: dict, n: int, precision: str) -> np.ndarray:
        pp = ctypes.POINTER(ctypes.c_double)()
        po = ctypes.POINTER(ctypes.c_double)()
        _capi.check(self._lib.gwl_host_buffers(self._h, int(n), ctypes.byref(pp), ctypes.byref(po)), "gwl_host_buffers")
        key = (ctypes.addressof(pp.contents), ctypes.addressof(po.contents), n)
        if getattr(self, "_staged_key", None) != key:
            self._staged_block = np.ctypeslib.as_array(pp, shape=(_capi.NPARAM * n,)).reshape(_capi.NPARAM, n)
            self._staged_out = np.ctypeslib.as_array(po, shape=(n,))
            self._staged_key = key
        block = self._staged_block
        for key_, slot in _capi.SLOT.items():
            v = params.get(key_)
            if v is None:
                block[slot] = 0.0
            else:
                block[slot] = v
        _capi.check(self._lib.gwl_eval_host_staged(self._h, int(n), PRECISIONS[precision]), "gwl_eval_host_staged")
        return self._staged_out.copy()

    def log_likelihood_ratio_device(self, block_ptr: int, B: int, out_ptr: int, precision: str = "fp64",
                                    stream: int = 0):
        """Device pointers in / out, asynchronous on ``stream`` (a cudaStream_t as int)."""
        _capi.check(self._lib.gwl_eval_device(self._h, ctypes.c_void_p(block_ptr), int(B), PRECISIONS[precision],
                                              ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream)),
                    "gwl_eval_device")

    def inner_products_device(self, block_ptr: int, B: int, dh_ptr: int, hh_ptr: int, precision: str = "fp64",
                              stream: int = 0):
        _capi.check(self._lib.gwl_inner_products_device(
            self._h, ctypes.c_void_p(block_ptr), int(B), PRECISIONS[precision], ctypes.c_void_p(dh_ptr),
            ctypes.c_void_p(hh_ptr), ctypes.c_void_p(stream)), "gwl_inner_products_device")

    def time_series_device(self, block_ptr: int, B: int, series_ptr: int, hh_ptr: int, stream: int = 0):
        """The float64 <d|h>(t) transform of every point ([B, 2 (n_bins - 1)]
        doubles) and <h|h> ([B]), device pointers, asynchronous on ``stream``."""
        _capi.check(self._lib.gwl_time_series_device(self._h, ctypes.c_void_p(block_ptr), int(B),
                                                     ctypes.c_void_p(series_ptr), ctypes.c_void_p(hh_ptr),
                                                     ctypes.c_void_p(stream)), "gwl_time_series_device")

    def inner_products_host(self, block: np.ndarray, precision: str = "fp64") -> tuple[np.ndarray, np.ndarray]:
        """Host parameter block [NPARAM, B] -> (complex <d|h> [B], <h|h> [B]),
        evaluated by the fused kernels (synchronous)."""
        import torch
        block = np.ascontiguousarray(block, dtype=np.float64)
        B = block.shape[1]
        dev = torch.from_numpy(block).cuda()
        dh = torch.empty((B, 2), dtype=torch.float64, device=dev.device)
        hh = torch.empty(B, dtype=torch.float64, device=dev.device)
        stream = torch.cuda.current_stream(dev.device)
        self.inner_products_device(dev.data_ptr(), B, dh.data_ptr(), hh.data_ptr(), precision, stream.cuda_stream)
        stream.synchronize()
        dh = dh.cpu().numpy()
        return dh[:, 0] + 1j * dh[:, 1], hh.cpu().numpy()

    def time_series_host(self, block: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """Host parameter block [NPARAM, B] -> (complex <d|h>(t) [B, n_bins - 1],
        <h|h> [B]) from the float64 time-marginalisation kernel (synchronous)."""
        import torch
        block = np.ascontiguousarray(block, dtype=np.float64)
        B, L = block.shape[1], getattr(self, "time_fft_length", self.n_bins - 1)
        dev = torch.from_numpy(block).cuda()
        series = torch.empty((B, L, 2), dtype=torch.float64, device=dev.device)
        hh = torch.empty(B, dtype=torch.float64, device=dev.device)
        stream = torch.cuda.current_stream(dev.device)
        self.time_series_device(dev.data_ptr(), B, series.data_ptr(), hh.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        s = series.cpu().numpy()
        return s[..., 0] + 1j * s[..., 1], hh.cpu().numpy()

    def set_profiling(self, enable: bool):
        _capi.check(self._lib.gwl_set_profiling(self._h, int(enable)), "gwl_set_profiling")

    def last_kernel_ms(self) -> float:
        ms = ctypes.c_float()
        _capi.check(self._lib.gwl_profile_last_kernel_ms(self._h, ctypes.byref(ms)), "gwl_profile_last_kernel_ms")
        return float(ms.value)

    # -- launch-shape tuning ---------------------------------------------------
    def autotune(self, block_ptr: int, B: int, stream: int = 0) -> tuple[int, float]:
        """Pick the split-K depth of the mixed TaylorF2 kernel by timing each
        candidate on B device points (block [NPARAM, B] at ``block_ptr``);
        returns (chunks per group, ms of the launch sequence at that depth)."""
        c = ctypes.c_int32()
        ms = ctypes.c_double()
        _capi.check(self._lib.gwl_autotune(self._h, ctypes.c_void_p(block_ptr), int(B), ctypes.c_void_p(stream),
                                           ctypes.byref(c), ctypes.byref(ms)), "gwl_autotune")
        return int(c.value), float(ms.value)

    @property
    def chunks_per_group(self) -> int:
        c = ctypes.c_int32()
        _capi.check(self._lib.gwl_get_chunks_per_group(self._h, ctypes.byref(c)), "gwl_get_chunks_per_group")
        return int(c.value)

    @chunks_per_group.setter
    def chunks_per_group(self, value: int):
        _capi.check(self._lib.gwl_set_chunks_per_group(self._h, int(value)), "gwl_set_chunks_per_group")

    @property
    def refinement_tolerance(self) -> float:
        """Error control of the mixed-precision TaylorF2 result: points whose
        |Delta lnL| bound exceeds this are recomputed with error-free sums
        (gwl_set_refinement); <= 0 turns it off."""
        t = ctypes.c_double()
        _capi.check(self._lib.gwl_get_refinement(self._h, ctypes.byref(t)), "gwl_get_refinement")
        return float(t.value)

    @refinement_tolerance.setter
    def refinement_tolerance(self, value: float):
        _capi.check(self._lib.gwl_set_refinement(self._h, float(value)), "gwl_set_refinement")

    def last_refined(self, stream: int = 0) -> int:
        """Points refined by the last mixed-precision evaluation (waits for ``stream``)."""
        n = ctypes.c_int64()
        _capi.check(self._lib.gwl_last_refined(self._h, ctypes.c_void_p(stream), ctypes.byref(n)), "gwl_last_refined")
        return int(n.value)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.gwl_analysis_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
