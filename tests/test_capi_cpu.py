"""The C-ABI library on the CPU: it loads, exports every symbol that
include/gwlnl.h declares, and its host build of the shared float64 math
(ln I0, bicubic spline) is right.  No compute call needs a GPU here."""
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT
from bilby_gb300 import _build, _capi


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _capi.load()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "gwlnl.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(gwl_\w+)\(", text, flags=re.M)))


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
        assert name in _capi.SIGNATURES, f"{name} has no ctypes signature"


def test_version_and_errors(lib):
    assert b"sm_103a" in lib.gwl_version()
    with pytest.raises(ValueError):
        _capi.check(lib.gwl_analysis_create(None, None), "create")
    assert b"null" in lib.gwl_last_error()


def test_host_ln_i0_matches_scipy(lib):
    """The reference bar (test/gw/utils_test.py:349-352) and large arguments."""
    from scipy.special import i0, i0e
    x = np.linspace(-10, 10, 101)
    assert np.max(np.abs(_capi.host_ln_i0(x) - np.log(i0(x)))) < 1e-10
    x = np.logspace(-5, 10, 400)
    ref = np.log(i0e(x)) + x
    assert np.max(np.abs(_capi.host_ln_i0(x) - ref) / np.maximum(1, ref)) < 1e-14


def test_host_bicubic_matches_scipy_spline(lib):
    """The de Boor evaluation against scipy's RectBivariateSpline (s=0, k=3)
    on the reference's table axes, with -inf outside the box."""
    from scipy.interpolate import RectBivariateSpline
    from bilby_gb300.likelihood import d_inner_h_ref_axis, optimal_snr_squared_ref_axis
    rng = np.random.default_rng(2)
    x = d_inner_h_ref_axis(800, False)
    y = optimal_snr_squared_ref_axis(400)
    table = np.add.outer(np.log1p(np.abs(y)) * -0.3, np.tanh(x / 50.0) * 7) + rng.normal(0, 1e-3, (400, 800))
    spline = RectBivariateSpline(x, y, table.T, kx=3, ky=3, s=0)
    tx, ty, c = spline.tck
    bbox = np.array([x.min(), x.max(), y.min(), y.max()])
    qx = np.concatenate([rng.uniform(-1000, 1e4, 500), x[::37], [x.min(), x.max(), -2000.0, 2e10]])
    qy = np.concatenate([10 ** rng.uniform(-5, 10, 500), y[::18][:len(x[::37])], [y.min(), y.max(), 1.0, 1.0]])
    got = _capi.host_bicubic(qx, qy, tx, ty, c, bbox)
    ref = spline(qx, qy, grid=False)
    inside = (qx >= bbox[0]) & (qx <= bbox[1]) & (qy >= bbox[2]) & (qy <= bbox[3])
    assert np.allclose(got[inside], ref[inside], rtol=1e-12, atol=1e-12)
    assert np.all(np.isneginf(got[~inside]))


def test_no_cpu_fallback_when_library_missing(monkeypatch, tmp_path):
    """The product path fails loudly without the CUDA library."""
    monkeypatch.setattr(_capi, "_LIB", None)
    monkeypatch.setattr(_build, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _capi.load()


CACHE_PROBE = r"""
#include <cstdio>
#include "gwl_device_cache.h"
int main() {
  gwl::PerDeviceCache<long> cache;
  int made = 0;
  long v = 0;
  auto make = [&](long* out) { *out = 1000 + (++made); return 0; };
  // the same FFT length on two devices gives two entries
  if (cache.get(0, 16384, &v, make) || v != 1001) return 1;
  if (cache.get(1, 16384, &v, make) || v != 1002) return 2;
  if (cache.get(0, 16384, &v, make) || v != 1001) return 3;   // found, not remade
  if (cache.get(1, 16384, &v, make) || v != 1002) return 4;
  if (cache.get(0, 8192, &v, make) || v != 1003) return 5;
  // a failed make keeps nothing and is retried on the next lookup
  if (cache.get(2, 16384, &v, [](long*) { return 7; }) != 7) return 6;
  if (cache.get(2, 16384, &v, make) || v != 1004) return 7;
  if (made != 4 || cache.size() != 4) return 8;
  std::puts("ok");
  return 0;
}
"""


def test_twiddle_tables_are_keyed_by_device_and_length(tmp_path):
    """The process-wide cache of the FFT twiddle tables keys on (device,
    length): the host logic, compiled with g++ against the library's header."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "probe.cpp"
    src.write_text(CACHE_PROBE)
    exe = tmp_path / "probe"
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "bilby_gb300", "csrc"), str(src), "-o",
                    str(exe), "-pthread"], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 0 and res.stdout.strip() == "ok", (res.returncode, res.stdout)


def test_trace_ranges_need_no_profiler(lib):
    """The NVTX entry points are no-ops without a profiler attached (no GPU
    needed) and balance."""
    for name in (b"admission", b"launch"):
        assert lib.gwl_trace_push(name) == _capi.GWL_OK
        assert lib.gwl_trace_pop() == _capi.GWL_OK
