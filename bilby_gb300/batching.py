"""Several analyses in one launch: Python owner of a ``gwl_batcher``.

A batch is a list of (analysis, parameter block, result buffer) items of
uneven sizes; the batcher evaluates them with one persistent launch per
detector count (mixed-precision TaylorF2) and can replay the launch sequence
of a repeated batch shape from a captured CUDA graph.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from .analysis import PRECISIONS, Analysis


class Batcher:
    def __init__(self, use_graphs: bool = False):
        self._lib = _capi.load()
        h = ctypes.c_void_p()
        _capi.check(self._lib.gwl_batcher_create(ctypes.byref(h)), "gwl_batcher_create")
        self._h = h
        self.use_graphs(use_graphs)

    def use_graphs(self, enable: bool):
        _capi.check(self._lib.gwl_batcher_use_graphs(self._h, int(enable)), "gwl_batcher_use_graphs")
        self.graphs = bool(enable)

    def eval_device(self, items, precision: str = "mixed", stream: int = 0):
        """items: [(Analysis, block_ptr, B, out_ptr)] with device pointers; asynchronous on ``stream``."""
        arr = (_capi.GwlBatchItem * len(items))()
        for q, (an, block_ptr, B, out_ptr) in enumerate(items):
            if not isinstance(an, Analysis):
                raise TypeError("batch items must reference bilby_gb300.analysis.Analysis objects")
            arr[q].analysis = an._h.value
            arr[q].params = block_ptr
            arr[q].B = int(B)
            arr[q].out = out_ptr
        _capi.check(self._lib.gwl_batcher_eval(self._h, arr, len(items), PRECISIONS[precision],
                                               ctypes.c_void_p(stream)), "gwl_batcher_eval")

    def eval_tensors(self, items, precision: str = "mixed", stream=None):
        """items: [(Analysis, block [NPARAM, B] CUDA float64 tensor)] -> list of CUDA result tensors."""
        import torch
        if stream is None:
            stream = torch.cuda.current_stream()
        outs, raw = [], []
        for an, block in items:
            if block.dtype != torch.float64 or not block.is_cuda or block.shape[0] != _capi.NPARAM:
                raise ValueError("parameter blocks must be CUDA float64 tensors of shape (NPARAM, B)")
            block = block.contiguous()
            out = torch.empty(block.shape[1], dtype=torch.float64, device=block.device)
            outs.append(out)
            raw.append((an, block.data_ptr(), block.shape[1], out.data_ptr()))
        self.eval_device(raw, precision, stream.cuda_stream)
        return outs

    def eval_host(self, items, precision: str = "mixed"):
        """items: [(Analysis, numpy block [NPARAM, B])] -> list of numpy results (synchronous)."""
        import torch
        dev = [(an, torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).cuda()) for an, b in items]
        outs = self.eval_tensors(dev, precision)
        torch.cuda.current_stream().synchronize()
        self.check()
        return [o.cpu().numpy() for o in outs]

    def check(self):
        st = ctypes.c_int()
        _capi.check(self._lib.gwl_batcher_status(self._h, ctypes.byref(st)), "gwl_batcher_status")
        if st.value:
            raise TimeoutError("a bounded device wait gave up during a batched evaluation")

    def last_refined(self, stream: int = 0) -> int:
        """Points the last batched launch refined (see Analysis.refinement_tolerance); waits for ``stream``."""
        n = ctypes.c_int64()
        _capi.check(self._lib.gwl_batcher_last_refined(self._h, ctypes.c_void_p(stream), ctypes.byref(n)),
                    "gwl_batcher_last_refined")
        return int(n.value)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.gwl_batcher_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
