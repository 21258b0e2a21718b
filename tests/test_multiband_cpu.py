"""Multi-banding without a GPU: the oracle's per-evaluation restatement on the
reference's own bands and coefficients reproduces the reference's lnL, and the
product's host set-up (bands, banded frequencies, linear and quadratic
coefficients; bilby/gw/likelihood/multiband.py:317-601) reproduces the
reference's arrays on the same data (tests/golden/tf2_128s_multiband.npz)."""
import numpy as np
import pytest

from tests.conftest import golden
from oracle import data as OD
from oracle import multiband as MB
from oracle import restate as R
from bilby_gb300.workloads import WORKLOADS, point


@pytest.fixture(scope="module")
def mb():
    w = WORKLOADS["tf2_128s"]
    dets = OD.build_workload(w)
    z = golden("tf2_128s_multiband")
    weights = {k[3:]: z[k] for k in z.files if k.startswith("mb_")}
    return w, dets, z, weights


@pytest.mark.parametrize("combo", ["none", "p"])
def test_oracle_reproduces_the_reference(mb, combo):
    w, dets, z, weights = mb
    assert np.allclose(OD.strain_checksum(dets), z["checksum"], rtol=1e-14, atol=0)
    src = OD.source_for(w.model, w.minimum_frequency)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    marg = R.Marginalization(phase="p" in combo)
    got = []
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if "p" in combo:
            q["phase"] = 0.0
        got.append(MB.log_likelihood_ratio(dets, src, weights, q, marg))
    ref = z["lnl_" + combo]
    assert np.all(np.abs(np.array(got) - ref) <= 1e-10 * np.maximum(1.0, np.abs(ref)))


class _StrainData:
    def __init__(self, det, fmin=20.0, fmax=2048.0):
        self.frequency_array = det.frequency
        self.frequency_mask = det.mask
        self.frequency_domain_strain = det.masked_strain
        self.duration = det.duration
        self.start_time = det.start_time
        self.minimum_frequency = fmin
        self.maximum_frequency = fmax


class _Ifo:
    def __init__(self, det):
        self.name = det.name
        self.strain_data = _StrainData(det)
        self.power_spectral_density_array = det.psd
        self.minimum_frequency = 20.0
        self.maximum_frequency = 2048.0


class _Gen:
    def __init__(self):
        self.waveform_arguments = {}


def test_host_setup_reproduces_the_reference(mb):
    from bilby_gb300.multiband import MBGravitationalWaveTransient
    w, dets, z, weights = mb
    like = object.__new__(MBGravitationalWaveTransient)
    like.interferometers = [_Ifo(d) for d in dets]
    like.waveform_generator = _Gen()
    like._prior = None
    like.time_reference = "geocent"
    like.reference_chirp_mass = 0.87
    like.highest_mode = 2
    like.linear_interpolation = True
    like.accuracy_factor = 5
    like.time_offset = None
    like.delta_f_end = None
    like.maximum_banding_frequency = None
    like.minimum_banding_duration = 0.
    like.setup_multibanding()
    assert like.time_offset == weights["time_offset"] and like.delta_f_end == weights["delta_f_end"]
    assert like.maximum_banding_frequency == weights["maximum_banding_frequency"]
    for key in ("durations", "fb_dfb", "Nbs", "Mbs", "Ks_Ke", "banded_frequency_points", "start_end_idxs",
                "unique_to_original_frequencies"):
        assert np.array_equal(np.asarray(getattr(like, key)), weights[key]), key
    assert np.array_equal(like.waveform_generator.waveform_arguments["frequencies"], weights["waveform_frequencies"])
    for q, d in enumerate(dets):
        lin, ref = like.linear_coeffs[d.name], weights[f"linear_coeffs_{q}"]
        assert np.max(np.abs(lin - ref)) <= 1e-12 * np.max(np.abs(ref))
        quad, ref = like.quadratic_coeffs[d.name], weights[f"quadratic_coeffs_{q}"]
        assert np.max(np.abs(quad - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_scatter_lists_reproduce_numpy_indexed_add():
    """The scatter lists of the time-marginalised multi-banding give, for
    random values, what multiband.py:794-798's band-by-band indexed += gives,
    duplicates within and across bands included."""
    from bilby_gb300.multiband import scatter_lists
    rng = np.random.default_rng(4)
    n = 64
    full = np.concatenate([rng.integers(0, 20, 30), rng.integers(10, 40, 25), rng.integers(30, 64, 40)])
    bands = np.array([[0, 29], [30, 54], [55, 94]])
    values = rng.standard_normal(len(full)) + 1j * rng.standard_normal(len(full))
    ref = np.zeros(n, dtype=complex)
    for s0, e0 in bands:
        ref[full[s0:e0 + 1]] += values[s0:e0 + 1]
    ptr, src = scatter_lists(full, bands, n)
    got = np.zeros(n, dtype=complex)
    for k in range(n):
        for c in src[ptr[k]:ptr[k + 1]]:
            if c >= 0:
                got[k] += values[c]
    np.testing.assert_allclose(got, ref, rtol=1e-14, atol=1e-14)
    # every banded point listed exactly once (replaced ones as -j - 1)
    decoded = np.where(src >= 0, src, -src - 1)
    assert np.array_equal(np.sort(decoded), np.arange(len(full)))


# ---------------------------------------------------------------------------
# the IFFT-FFT <h|h> (linear_interpolation=False, multiband.py:613-650, 760-779)
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def ifft_like(mb):
    from bilby_gb300.multiband import MBGravitationalWaveTransient
    w, dets, z, weights = mb
    like = object.__new__(MBGravitationalWaveTransient)
    like.interferometers = [_Ifo(d) for d in dets]
    like.waveform_generator = _Gen()
    like._prior = None
    like.time_reference = "geocent"
    like.reference_chirp_mass = 0.87
    like.highest_mode = 2
    like.linear_interpolation = False
    like.accuracy_factor = 5
    like.time_offset = None
    like.delta_f_end = None
    like.maximum_banding_frequency = None
    like.minimum_banding_duration = 0.
    like.setup_multibanding()
    return like


def _tables(like, dets):
    t = {key: getattr(like, key) for key in ("Ks_Ke", "start_end_idxs", "Mbs", "Tbhats", "windows",
                                             "square_root_windows")}
    t["duration"] = float(like.durations[0])
    for q, d in enumerate(dets):
        t[f"Ibcs_{q}"] = like.Ibcs[d.name]
    return t


def test_ifft_host_tables_reproduce_the_reference(mb, ifft_like):
    """Tbhats, the windows and every 61st entry of each detector's per-band
    I_b match the reference's _setup_quadratic_coefficients_ifft_fft."""
    w, dets, _, weights = mb
    z = golden("tf2_128s_multiband_ifft")
    assert len(ifft_like.banded_frequency_points) == int(z["mb_n_banded"])
    np.testing.assert_allclose(ifft_like.Tbhats, z["mb_Tbhats"], rtol=1e-15, atol=0)
    assert abs(np.sum(ifft_like.windows) - float(z["mb_windows_sum"])) <= 1e-12 * float(z["mb_windows_sum"])
    stride = int(z["ibc_stride"])
    for q, d in enumerate(dets):
        for b in range(len(ifft_like.Mbs)):
            ref = z[f"mb_Ibcs_{q}_{b}"]
            got = np.asarray(ifft_like.Ibcs[d.name][b])[::stride]
            assert len(got) == len(ref)
            assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref)), (q, b)


@pytest.mark.parametrize("combo", ["none", "p"])
def test_oracle_ifft_reproduces_the_reference(mb, ifft_like, combo):
    """The oracle's IFFT-FFT restatement on the product's host tables gives the
    reference's lnL ratios (tests/golden/tf2_128s_multiband_ifft.npz)."""
    w, dets, _, weights = mb
    z = golden("tf2_128s_multiband_ifft")
    src = OD.source_for(w.model, w.minimum_frequency)
    tables = _tables(ifft_like, dets)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    marg = R.Marginalization(phase="p" in combo)
    got = []
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if "p" in combo:
            q["phase"] = 0.0
        got.append(MB.log_likelihood_ratio_ifft_fft(dets, src, weights, tables, q, marg))
    ref = z["lnl_" + combo]
    assert np.all(np.abs(np.array(got) - ref) <= 1e-10 * np.maximum(1.0, np.abs(ref))), np.array(got) - ref


def _odd_bins_packed(strains, b, ks, m, sqrtw, s0, n):
    """The odd-bin sums sum_j |Z_j|^2 (as weights per detector) the way the
    CUDA kernel forms them: two detectors packed in one complex transform,
    inverse DFT, times exp(-i pi n / M) / M, DFT, separation by the conjugate
    symmetry of a real sequence's odd-frequency DFT.  Returns |Z_d,j|^2."""
    out = []
    for d1 in range(0, len(strains), 2):
        w1 = sqrtw[s0:s0 + n] * strains[d1][s0:s0 + n]
        w2 = sqrtw[s0:s0 + n] * strains[d1 + 1][s0:s0 + n] if d1 + 1 < len(strains) else np.zeros(n, complex)
        c = np.zeros(m, dtype=complex)
        idx = ks + np.arange(n)
        c[idx] = w1 + 1j * w2
        c[m - idx] = np.conj(w1) + 1j * np.conj(w2)
        y = np.fft.ifft(c)
        f = np.fft.fft(y * np.exp(-1j * np.pi * np.arange(m) / m))
        j = np.arange(m // 2)
        r = np.conj(f[m - 1 - j])
        out.append(np.abs((f[j] + r) / 2) ** 2)
        if d1 + 1 < len(strains):
            out.append(np.abs((f[j] - r) / 2j) ** 2)
    return out


def test_ifft_decomposition_matches_the_direct_sum(mb, ifft_like):
    """The GPU's form of the IFFT-FFT <h|h> -- even bins folded into the
    quadratic coefficients, odd bins by the packed two-detector transform --
    equals the reference's sum on random banded strains, detector by
    detector."""
    w, dets, _, weights = mb
    quad, (ks, m, scale, sw, odd) = ifft_like._ifft_fft_tables()
    tables = _tables(ifft_like, dets)
    rng = np.random.default_rng(11)
    K = len(ifft_like.banded_frequency_points)
    f = np.asarray(ifft_like.banded_frequency_points)
    amp = 1e-23 * (f / 100.0) ** (-7.0 / 6.0)
    strains = [amp * (rng.standard_normal(K) + 1j * rng.standard_normal(K)) for _ in dets]
    got = [float(quad[q] @ np.abs(strains[q]) ** 2) for q in range(len(dets))]
    off = 0
    for b in range(1, len(m)):
        s0, e0 = (int(x) for x in ifft_like.start_end_idxs[b])
        z2 = _odd_bins_packed(strains, b, int(ks[b]), int(m[b]), sw, s0, e0 - s0 + 1)
        for q in range(len(dets)):
            got[q] += scale[b] * float(z2[q] @ odd[q][off:off + int(m[b]) // 2])
        off += int(m[b]) // 2
    for q, det in enumerate(dets):
        ref = MB.hh_ifft_fft(strains[q], q, det, tables)
        assert abs(got[q] - ref) <= 1e-12 * abs(ref), (q, got[q], ref)
