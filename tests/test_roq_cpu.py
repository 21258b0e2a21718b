"""The host construction of the GPU ROQ likelihood's weights
(bilby/gw/likelihood/roq.py:736-1005: time grid, linear weights by inverse
FFTs, quadratic weights) reproduces the reference's weights for the same
seeded synthetic basis (tests/golden/tf2_marg_8s_2k_roq.npz), and for a
multi-banded basis (tests/golden/tf2_marg_8s_2k_roq_multiband.npz); bases
outside the prior are dropped.  No GPU."""
import numpy as np
import pytest

from tests.conftest import golden
from oracle import data as OD
from oracle import restate as R
from oracle import roq_basis
from bilby_gb300.workloads import WORKLOADS


class _StrainData:
    def __init__(self, det):
        self.frequency_array = det.frequency
        self.frequency_mask = det.mask
        self.frequency_domain_strain = det.masked_strain
        self.duration = det.duration
        self.start_time = det.start_time


class _Ifo:
    def __init__(self, det, snr):
        self.name = det.name
        self.strain_data = _StrainData(det)
        self.power_spectral_density_array = det.psd
        self.minimum_frequency = 20.0
        self.maximum_frequency = 1024.0
        self.meta_data = {"optimal_SNR": snr}


class _Uniform:
    def __init__(self, lo, hi):
        self.minimum, self.maximum = lo, hi


def _host_likelihood():
    """The product's ROQ class with the oracle's data of tf2_marg_8s_2k and
    its time prior, ready for _set_weights (no GPU)."""
    from bilby_gb300.roq import ROQGravitationalWaveTransient
    w = WORKLOADS["tf2_marg_8s_2k"]
    dets = OD.build_workload(w)
    src = OD.source_for(w.model, w.minimum_frequency)
    pols = src(dets[0].frequency, **w.injection)
    ifos = []
    for d in dets:
        s = R.detector_response(d, pols, w.injection["ra"], w.injection["dec"], w.injection["geocent_time"],
                                w.injection["psi"])
        m = d.mask
        snr = np.sqrt(R.noise_weighted_inner_product(s[m], s[m], d.psd[m], d.duration).real)
        ifos.append(_Ifo(d, snr))
    like = object.__new__(ROQGravitationalWaveTransient)
    like.interferometers = ifos
    tc = w.injection["geocent_time"]
    like._prior = {"geocent_time": _Uniform(tc - 0.1, tc + 0.1)}
    like.time_reference = "geocent"
    like.roq_params = None
    like.roq_scale_factor = 1
    like.weights = {}
    return like, w, dets, ifos


def _check_weights(like, ifos, z):
    ts = like.weights["time_samples"]
    t0, dt, n = z["roq_time_meta"]
    assert len(ts) == int(n) and ts[0] == t0 and ts[1] - ts[0] == dt
    for q, ifo in enumerate(ifos):
        lin = like.weights[ifo.name + "_linear"][0][z[f"roq_linear_rows_{q}"]]
        ref = z[f"roq_linear_{q}"]
        assert np.max(np.abs(lin - ref)) <= 1e-10 * np.max(np.abs(ref))
        quad = like.weights[ifo.name + "_quadratic"][0]
        assert np.max(np.abs(quad - z[f"roq_quadratic_{q}"])) <= 1e-12 * np.max(np.abs(quad))


def test_multiband_weights_match_the_reference():
    """A multi-banded basis (three bands of 8, 4 and 2 s) through
    _set_weights_linear_multiband / _set_weights_quadratic_multiband
    (roq.py:920-974, 1007-1055) gives the reference's weights."""
    like, w, dets, ifos = _host_likelihood()
    lin, quad = roq_basis.build_multiband(minimum_frequency=w.minimum_frequency)
    like._set_weights(like._parse_basis(lin, "linear"), like._parse_basis(quad, "quadratic"))
    assert np.array_equal(like.weights["frequency_nodes_linear"][0], lin["basis_linear"]["0"]["frequency_nodes"])
    _check_weights(like, ifos, golden("tf2_marg_8s_2k_roq_multiband"))


def test_weights_match_the_reference():
    like, w, dets, ifos = _host_likelihood()
    fm = dets[0].frequency[dets[0].mask]
    nl, bl, nq, bq = roq_basis.build(fm, minimum_frequency=w.minimum_frequency)
    like._set_weights(like._parse_basis(bl.T, "linear"), like._parse_basis(bq.T, "quadratic"))
    _check_weights(like, ifos, golden("tf2_marg_8s_2k_roq"))


def test_bases_outside_the_prior_are_dropped():
    """roq.py:368-400, 771-791: with prior ranges in the basis mapping only
    the bases whose ranges meet the priors are built, their ranges and nodes
    kept in that order; none inside raises."""
    from bilby_gb300.roq import BilbyROQParamsRangeError
    like, w, dets, ifos = _host_likelihood()
    fm = dets[0].frequency[dets[0].mask]
    _, bl, _, bq = roq_basis.build(fm, n_linear=4, n_quadratic=2, n_train=20, minimum_frequency=w.minimum_frequency)
    lin = {"basis_linear": {str(i): {"basis": bl * (i + 1), "frequency_nodes": fm[:4] + i} for i in range(3)},
           "prior_range_linear": {"chirp_mass": np.array([[5., 10.], [10., 20.], [20., 40.]])}}
    quad = {"basis_quadratic": {"0": {"basis": bq, "frequency_nodes": fm[:2]}}}
    like._prior["chirp_mass"] = _Uniform(12.0, 30.0)
    like._set_weights(like._parse_basis(lin, "linear"), like._parse_basis(quad, "quadratic"))
    assert np.array_equal(like.weights["prior_range_linear"]["chirp_mass"], [[10., 20.], [20., 40.]])
    assert [float(n[0]) for n in like.weights["frequency_nodes_linear"]] == [fm[0] + 1, fm[0] + 2]
    for ifo in ifos:
        a, b = like.weights[ifo.name + "_linear"]
        np.testing.assert_allclose(b, a * 1.5, rtol=1e-12)
    like._prior["chirp_mass"] = _Uniform(50.0, 60.0)
    like.weights = {}
    with pytest.raises(BilbyROQParamsRangeError):
        like._set_weights(like._parse_basis(lin, "linear"), like._parse_basis(quad, "quadratic"))


def _reference_update_basis(weights, n_bases, basis_type, parameters):
    """roq.py:398-431 restated for one point: the first basis whose range
    holds every ranged parameter the point has."""
    if n_bases == 1:
        return 0
    ok = np.ones(n_bases, dtype=bool)
    for name, ranges in weights[f"prior_range_{basis_type}"].items():
        if name not in parameters:
            continue
        ok *= (ranges[:, 0] <= parameters[name]) * (ranges[:, 1] >= parameters[name])
    return np.arange(n_bases)[ok][0]


def test_basis_selection_matches_the_reference_rule():
    """Vectorised basis selection of the multi-basis ROQ likelihood against
    the reference's per-point rule, with a second ranged parameter that some
    points lack, and IndexError for a point outside every range."""
    import pytest
    from bilby_gb300.roq import ROQGravitationalWaveTransient
    like = object.__new__(ROQGravitationalWaveTransient)
    like.parameter_conversion = None
    like.number_of_bases_linear, like.number_of_bases_quadratic = 3, 2
    like.weights = {
        "prior_range_linear": {"chirp_mass": np.array([[5.0, 12.0], [10.0, 20.0], [18.0, 40.0]]),
                               "mass_ratio": np.array([[0.1, 1.0], [0.5, 1.0], [0.1, 1.0]])},
        "prior_range_quadratic": {"chirp_mass": np.array([[5.0, 15.0], [14.0, 40.0]])}}
    rng = np.random.default_rng(3)
    p = {"chirp_mass": rng.uniform(5.0, 40.0, 600), "mass_ratio": rng.uniform(0.1, 1.0, 600)}
    ref, keep = [], []
    for i in range(600):
        q = {k: v[i] for k, v in p.items()}
        try:
            ref.append((_reference_update_basis(like.weights, 3, "linear", q),
                        _reference_update_basis(like.weights, 2, "quadratic", q)))
            keep.append(i)
        except IndexError:  # in no linear basis' range (chirp mass 12-18, mass ratio below 0.5)
            pass
    assert 300 < len(keep) < 600
    il, iq = like.basis_numbers({k: v[keep] for k, v in p.items()})
    assert list(zip(il.tolist(), iq.tolist())) == [(int(a), int(b)) for a, b in ref]
    assert {int(a) for a, _ in ref} == {0, 1, 2}
    il, _ = like.basis_numbers({"chirp_mass": np.array([11.0, 19.0])})   # no mass_ratio: not ranged
    assert list(il) == [0, 1]
    with pytest.raises(IndexError):
        like.basis_numbers({"chirp_mass": np.array([50.0])})
