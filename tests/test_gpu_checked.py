"""The index-checked debug build (``-DGWL_CHECK``, ``libgwlnl_check.so``).

Its kernels test the indices they read from host-built tables (the
multi-banding scatter lists, the relative-binning bin map, the IFFT-FFT
transform bins) before each access; a failed test records a status that the
next host evaluation returns as GWL_ERR_CHECK, and the access is skipped.
Here the variant is built, the parity tests of those table-driven paths run
against it in a child process (``GWL_CHECKED=1``) and pass unchanged, and a
check status in the status word surfaces once as GWL_ERR_CHECK and then
clears.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from tests.conftest import ROOT
from tests.gpu_helpers import device_analysis, draw_points, params_block, small_workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked_lib(gpu):
    from bilby_gb300 import _build
    return _build.build(checked=True)


def test_table_driven_parity_tests_pass_on_the_checked_build(checked_lib):
    env = dict(os.environ, GWL_CHECKED="1")
    probe = subprocess.run([sys.executable, "-c", "from bilby_gb300 import _capi; print(_capi.library_path())"],
                           cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert probe.returncode == 0 and probe.stdout.strip().endswith("libgwlnl_check.so"), probe.stdout + probe.stderr
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
                        "tests/test_gpu_multiband.py", "tests/test_gpu_relbin.py"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-4000:]


def test_check_status_surfaces_once_then_clears(gpu):
    from bilby_gb300 import _capi
    from oracle import data as OD
    w = small_workload("tf2_128s", duration=8.0, sampling_frequency=2048.0,
                       injection=dict(small_workload("tf2_128s").injection, geocent_time=1126259640.0 + 6.0))
    dets = OD.build_workload(w)
    an = device_analysis(dets, "taylorf2", w)
    block = params_block(draw_points(w, 64, np.random.default_rng(5)))
    good = an.log_likelihood_ratio_host(block, "fp64")
    _capi.check(_capi.load().gwl_inject_device_status(an._h, 3), "inject")
    with pytest.raises(RuntimeError, match="index check"):
        an.log_likelihood_ratio_host(block, "fp64")
    assert np.array_equal(an.log_likelihood_ratio_host(block, "fp64"), good)
    an.close()
