"""The oracle against the reference itself, imported in place (runs only
where the reference source tree is available; skipped elsewhere)."""
import numpy as np
import pytest

from oracle import ref_harness

pytestmark = [pytest.mark.reference,
              pytest.mark.skipif(not ref_harness.reference_available(), reason="reference tree not available")]


@pytest.fixture(scope="module")
def bilby():
    return ref_harness.import_bilby()


def test_gmst_antenna_delay(bilby):
    from oracle import restate as R
    rng = np.random.default_rng(0)
    ifo = bilby.gw.detector.get_empty_interferometer("L1")
    v, t = R.detector_geometry("L1")
    assert np.allclose(ifo.geometry.vertex, v, rtol=1e-13, atol=0)
    assert np.allclose(ifo.geometry.detector_tensor, t, rtol=1e-14, atol=1e-16)
    for _ in range(20):
        gps = 1126259640.0 + rng.uniform(0, 1e6)
        ra, dec, psi = rng.uniform(0, 2 * np.pi), np.arcsin(rng.uniform(-1, 1)), rng.uniform(0, np.pi)
        assert R.greenwich_mean_sidereal_time(gps) == bilby.gw.time.greenwich_mean_sidereal_time(gps)
        for mode in ("plus", "cross"):
            assert R.antenna_response(t, ra, dec, gps, psi, mode) == pytest.approx(
                ifo.antenna_response(ra, dec, gps, psi, mode), rel=1e-13, abs=1e-15)
        assert R.time_delay_from_geocenter(v, ra, dec, gps) == pytest.approx(
            ifo.time_delay_from_geocenter(ra, dec, gps), rel=1e-13, abs=1e-18)


def test_host_frames_match_reference(bilby):
    """bilby_gb300.frames (host parameter preparation) vs the reference."""
    from bilby_gb300 import frames
    rng = np.random.default_rng(1)
    ifos = bilby.gw.detector.InterferometerList(["H1", "L1"])
    frame = frames.ReferenceFrame("H1L1")
    for _ in range(10):
        z, a = np.arccos(rng.uniform(-1, 1)), rng.uniform(0, 2 * np.pi)
        gps = 1126259642.4 + rng.uniform(-1, 1)
        ra, dec = bilby.gw.utils.zenith_azimuth_to_ra_dec(z, a, gps, ifos)
        ra2, dec2 = frame.zenith_azimuth_to_ra_dec(z, a, gps)
        assert ra2 == pytest.approx(ra, abs=1e-12) and dec2 == pytest.approx(dec, abs=1e-12)
        dt = ifos[0].time_delay_from_geocenter(ra, dec, gps)
        assert frames.time_delay_from_geocenter(ifos[0].geometry.vertex, ra, dec, gps) == pytest.approx(dt, abs=1e-17)


def test_sinegaussian_source_is_bilbys(bilby):
    from oracle import restate as R
    f = np.linspace(0, 1024, 4097)
    for q in (3.0, 9.0, 29.0):
        ref = bilby.gw.source.sinegaussian(f, 1e-22, q, 150.0)
        got = R.sinegaussian(f, 1e-22, q, 150.0)
        assert np.array_equal(ref["plus"], got["plus"]) and np.array_equal(ref["cross"], got["cross"])
