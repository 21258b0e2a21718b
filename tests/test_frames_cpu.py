"""Sky-frame parameters (bilby/gw/likelihood/base.py:1091-1137) of the drop-in
likelihood against the reference's own get_sky_frame_parameters
(tests/golden/sky_frames.npz): detector-pair frames (zenith/azimuth -> ra/dec)
and detector time references (t_ifo -> geocent_time).  Host code, no GPU."""
import numpy as np
import pytest

from tests.conftest import golden

CASES = [("H1L1", "geocent"), ("H1L1", "H1"), ("sky", "L1"), ("L1V1", "V1")]


def frame_object(frame, tref):
    """The likelihood's parameter preparation for a sky frame and time reference."""
    from bilby_gb300.detector import get_empty_interferometer
    from bilby_gb300.frames import ReferenceFrame
    from bilby_gb300.likelihood import ParameterPreparer
    f = None if frame == "sky" else ReferenceFrame(frame)
    if "geocent" in tref:
        return ParameterPreparer("taylorf2", None, f, "geocent", None)
    return ParameterPreparer("taylorf2", None, f, tref, get_empty_interferometer(tref).geometry.vertex)


@pytest.mark.parametrize("q", range(len(CASES)))
def test_sky_frame_parameters_match_the_reference(q):
    z = golden("sky_frames")
    frame, tref = CASES[q]
    like = frame_object(frame, tref)
    key = "geocent_time" if "geocent" in tref else f"{tref}_time"
    p = dict(zenith=z["p_zenith"], azimuth=z["p_azimuth"], ra=z["p_ra"], dec=z["p_dec"])
    p[key] = z["p_t"]
    got = like.sky_frame(p)
    ref = z[f"frame_{q}"]
    assert np.allclose(np.asarray(got["ra"]), ref[:, 0], rtol=0, atol=1e-12)
    assert np.allclose(np.asarray(got["dec"]), ref[:, 1], rtol=0, atol=1e-12)
    assert np.allclose(np.asarray(got["geocent_time"]), ref[:, 2], rtol=0, atol=1e-9)
