"""Generate the golden fixtures in this directory (and the packaged detector
noise-curve tables) by running the reference bilby, imported in place from
its source tree, on the seeded workloads of ``bilby_gb300.workloads``.

Run from the repository root, where the reference tree is available:

    python tests/golden/make_golden.py            # everything
    python tests/golden/make_golden.py --quick    # skip the marginalised cases

Outputs
-------
``bilby_gb300/noise_curves.npz``
    The two bundled sensitivity curves the workloads use
    (bilby/gw/detector/noise_curves/aLIGO_O4_high_asd.txt and AdV_psd.txt),
    as float64 (frequency, value) arrays.
``tests/golden/known_answer.json``
    The reference's own known answer for H1, 4 s at 2048 Hz, seed 500
    (test/gw/likelihood_test.py:195-201), recomputed by the reference here.
``tests/golden/<workload>.npz``
    Prior draws and the reference's ``log_likelihood_ratio`` for each draw,
    the reference's ``noise_log_likelihood``, and a checksum of the strain it
    generated, so a test can check that the oracle regenerates the same data.
``tests/golden/tf2_marg_8s_2k.npz``, ``tests/golden/tf2_marg_8s.npz``
    Prior draws of the marginalised TaylorF2 workloads at 8 s and 2048 Hz
    (FFT length 8192) and 4096 Hz (FFT length 16384) and the reference's
    ``log_likelihood_ratio`` under each of the seven combinations of time,
    phase and distance marginalisation.
``tests/golden/tf2_marg_6s_2k.npz``
    The same seven combinations on a 6 s segment at 2048 Hz, whose FFT length
    (6144 = 3 x 2048) is not a power of two.
``tests/golden/tf2_marg_8s_2k_time_prior.npz``
    The reference's time-marginalised lnL under a TruncatedGaussian
    geocent_time prior (time, time+phase, time+distance, all three).
``tests/golden/tf2_128s_multiband.npz``
    The reference's ``MBGravitationalWaveTransient`` on tf2_128s (reference
    chirp mass 0.87, linear-interpolation <h|h>): its bands, banded
    frequencies, linear and quadratic coefficients and lnL ratios without
    marginalisation, with phase, with distance, with time, and with time,
    phase and distance marginalisation.
``tests/golden/tf2_128s_multiband_ifft.npz``
    The same likelihood with the IFFT-FFT <h|h> (``linear_interpolation=False``):
    lnL ratios without marginalisation, with phase, with time, and with time,
    phase and distance marginalisation, its Tbhats, the sum of its windows and
    a strided sample of each detector's per-band Ibcs.
``tests/golden/tf2_marg_8s_2k_roq.npz``
    The reference's ``ROQGravitationalWaveTransient`` on tf2_marg_8s_2k with the
    seeded synthetic basis of ``oracle/roq_basis.py``: its time grid, the rows
    of the linear weights the stored points read, the quadratic weights, the
    frequency nodes, and lnL ratios without marginalisation, with phase, with
    distance, with time, and with time, phase and distance marginalisation
    (with the time grid's spacing and length).
``tests/golden/tf2_marg_8s_2k_roq_multibasis.npz``
    The reference's ROQ likelihood with two linear and two quadratic seeded
    synthetic bases selected per point by chirp-mass ranges (a weights
    dictionary merged from single-basis weights): the sampler-style draws,
    the basis pair the reference selected for each, and its lnL ratios
    without and with time marginalisation.
``tests/golden/tf2_marg_8s_2k_roq_multiband.npz``
    The reference's ROQ weights built from a seeded multi-banded basis
    (``oracle/roq_basis.build_multiband``: three bands of 8, 4 and 2 s) -- the
    rows of the linear weights the stored points read and the quadratic
    weights -- and its lnL ratios without marginalisation, with time, and with
    time, phase and distance marginalisation.
``tests/golden/priors.npz``
    The reference's ``PriorDict.rescale`` of fixed unit-cube samples for the
    GW prior kinds the device rescaler supports, followed by
    ``convert_to_lal_binary_black_hole_parameters``.
``tests/golden/sky_frames.npz``
    The reference's ``get_sky_frame_parameters`` (base.py:1091-1137) for
    detector-pair frames and detector time references on random points.
``tests/golden/tf2_marg_8s_2k_snrs.npz``
    The reference's ``calculate_snrs`` per detector (<d|h>, <h|h>, matched-
    filter SNR; with time marginalisation the d_inner_h_array inside the
    prior window, its sum and power), ``compute_per_detector_log_likelihood``
    without and with marginalisation, and the draws of
    ``generate_posterior_sample_from_marginalized_likelihood`` with the
    shared generator seeded per point.
``tests/golden/tf2_128s_fast_snrs.npz``
    ``calculate_snrs`` and ``compute_per_detector_log_likelihood`` of the
    reference's relative-binning and multi-banded likelihoods, without and
    with time marginalisation.
``tests/golden/tf2_marg_8s_2k_roq_snrs.npz``
    The same for the reference's ROQ likelihood (seeded synthetic basis),
    with the time draw under time marginalisation.
``tests/golden/sg_4s_marg.npz``
    The reference's time- and time+phase-marginalised likelihood for the
    sine-Gaussian workload.
``tests/golden/tf2_128s_relbin.npz``
    The reference's ``RelativeBinningGravitationalWaveTransient`` on tf2_128s
    (fiducial = the injection): its bin edges, summary data and lnL ratios
    without marginalisation, with phase, with distance, with time, and with
    time, phase and distance marginalisation.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_harness  # noqa: E402
from oracle.taylorf2 import (taylorf2_aligned, taylorf2_aligned_frequency_sequence,  # noqa: E402
                             taylorf2_aligned_relative_binning, taylorf2_aligned_roq)
from bilby_gb300.workloads import WORKLOADS, DISTANCE_PRIOR, draw_points, point  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def export_noise_curves():
    out = {}
    for stem in ("aLIGO_O4_high_asd", "AdV_psd"):
        tab = np.genfromtxt(ref_harness.asd_file_path(stem + ".txt")).T
        out[stem + "_frequency"] = tab[0].astype(np.float64)
        out[stem + "_value"] = tab[1].astype(np.float64)
    np.savez_compressed(os.path.join(ROOT, "bilby_gb300", "noise_curves.npz"), **out)


def build_reference(bilby, w, source):
    bilby.core.utils.random.seed(w.seed)
    ifos = bilby.gw.detector.InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(
        sampling_frequency=w.sampling_frequency, duration=w.duration, start_time=w.start_time)
    wfg = bilby.gw.waveform_generator.WaveformGenerator(
        duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
        frequency_domain_source_model=source,
        waveform_arguments=dict(minimum_frequency=w.minimum_frequency) if w.model == "taylorf2" else {})
    # InterferometerList.inject_signal without its signal-duration check, which
    # needs lalsimulation (interferometer.py:370-410); the injection itself is
    # interferometer.py:493-510.
    pols = wfg.frequency_domain_strain(dict(w.injection))
    for ifo in ifos:
        ifo.inject_signal_from_waveform_polarizations(parameters=dict(w.injection), injection_polarizations=pols)
    return ifos, wfg


def strain_checksum(ifos):
    return np.array([[np.sum(np.abs(ifo.strain_data.frequency_domain_strain) ** 2) * 1e42,
                      np.sum(ifo.strain_data.frequency_domain_strain.real) * 1e21]
                     for ifo in ifos])


def make_priors(bilby, w, time=False, phase=False, distance=False):
    priors = bilby.core.prior.PriorDict()
    tc = w.injection["geocent_time"]
    if time:
        priors["geocent_time"] = bilby.core.prior.Uniform(tc - 0.1, tc + 0.1, name="geocent_time")
    if phase:
        priors["phase"] = bilby.core.prior.Uniform(0, 2 * np.pi, name="phase", boundary="periodic")
    if distance:
        priors["luminosity_distance"] = bilby.core.prior.PowerLaw(
            DISTANCE_PRIOR["alpha"], DISTANCE_PRIOR["minimum"], DISTANCE_PRIOR["maximum"],
            name="luminosity_distance")
    return priors


def run_plain(bilby, name, n_fixed, n_random):
    w = WORKLOADS[name]
    source = bilby.gw.source.sinegaussian if w.model == "sinegaussian" else taylorf2_aligned
    ifos, wfg = build_reference(bilby, w, source)
    like = bilby.gw.likelihood.GravitationalWaveTransient(interferometers=ifos, waveform_generator=wfg)
    rng = np.random.default_rng(w.draw_seed)
    pf = draw_points(w, n_fixed, rng, fixed_extrinsic=True)
    pr = draw_points(w, n_random, rng, fixed_extrinsic=False)
    params = {k: np.concatenate([pf[k], pr[k]]) for k in pf}
    n = n_fixed + n_random
    t0 = time.perf_counter()
    lnl = np.array([like.log_likelihood_ratio(point(params, i)) for i in range(n)])
    dt = (time.perf_counter() - t0) / n
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), lnl=lnl,
                        noise_lnl=float(like.noise_log_likelihood()),
                        checksum=strain_checksum(ifos), **{"p_" + k: v for k, v in params.items()})
    print(f"{name}: {n} points, {dt * 1e3:.2f} ms/eval in the reference, noise lnL {like.noise_log_likelihood()}")


MARG_COMBOS = ["t", "p", "d", "tp", "td", "pd", "tpd"]


def run_marginalised(bilby, name, n_points):
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed)
    params = draw_points(w, n_points, rng, fixed_extrinsic=False)
    params["time_jitter"] = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n_points)
    out = {"p_" + k: v for k, v in params.items()}
    for combo in MARG_COMBOS:
        ifos, wfg = build_reference(bilby, w, taylorf2_aligned)
        t, p, d = "t" in combo, "p" in combo, "d" in combo
        priors = make_priors(bilby, w, t, p, d)
        like = bilby.gw.likelihood.GravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, priors=priors,
            time_marginalization=t, phase_marginalization=p, distance_marginalization=d)
        t0 = time.perf_counter()
        vals = []
        for i in range(n_points):
            q = point(params, i)
            if t:
                q["geocent_time"] = float(priors["geocent_time"])
            if p:
                q["phase"] = 0.0
            if d:
                q["luminosity_distance"] = float(priors["luminosity_distance"])
            if not t:
                q.pop("time_jitter")
            vals.append(like.log_likelihood_ratio(q))
        out["lnl_" + combo] = np.array(vals)
        print(f"{name}[{combo}]: {(time.perf_counter() - t0) / n_points * 1e3:.2f} ms/eval")
        if combo == "tpd":
            out["noise_lnl"] = float(like.noise_log_likelihood())
            out["checksum"] = strain_checksum(ifos)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


RELBIN_COMBOS = ["none", "p", "d"]
RELBIN_TIME_COMBOS = ["t", "tpd"]


def run_relbin(bilby, name, n_fixed, n_random):
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 1)
    pf = draw_points(w, n_fixed, rng, fixed_extrinsic=True)
    pr = draw_points(w, n_random, rng, fixed_extrinsic=False)
    params = {k: np.concatenate([pf[k], pr[k]]) for k in pf}
    n = n_fixed + n_random
    # drawn after the points, so that the points do not depend on it
    jitter = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n)
    out = {"p_" + k: v for k, v in params.items()}
    out["time_jitter"] = jitter
    for combo in RELBIN_COMBOS + RELBIN_TIME_COMBOS:
        ifos, _ = build_reference(bilby, w, taylorf2_aligned)
        wfg = bilby.gw.waveform_generator.WaveformGenerator(
            duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
            frequency_domain_source_model=taylorf2_aligned_relative_binning,
            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
        t, p, d = "t" in combo, "p" in combo, "d" in combo
        priors = make_priors(bilby, w, t, p, d)
        # with time marginalisation and jitter the reference's constructor
        # evaluates the fiducial point, which then needs a time_jitter entry
        fiducial = dict(w.injection, time_jitter=0.0) if t else dict(w.injection)
        like = bilby.gw.likelihood.RelativeBinningGravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, fiducial_parameters=fiducial,
            priors=priors if (t or p or d) else None, time_marginalization=t, phase_marginalization=p,
            distance_marginalization=d)
        t0 = time.perf_counter()
        vals = []
        for i in range(n):
            q = point(params, i)
            if t:
                q["geocent_time"] = float(priors["geocent_time"])
                q["time_jitter"] = float(jitter[i])
            if p:
                q["phase"] = 0.0
            if d:
                q["luminosity_distance"] = float(priors["luminosity_distance"])
            vals.append(like.log_likelihood_ratio(q))
        out["lnl_" + combo] = np.array(vals)
        print(f"{name} relbin[{combo}]: {like.number_of_bins} bins, "
              f"{(time.perf_counter() - t0) / n * 1e3:.2f} ms/eval")
        if combo == "none":
            out["bin_inds"] = like.bin_inds
            out["bin_freqs"] = like.bin_freqs
            for q, ifo in enumerate(ifos):
                a0, a1, b0, b1 = like.summary_data[ifo.name]
                out[f"summary_{q}"] = np.stack([a0, a1, b0, b1])
            out["checksum"] = strain_checksum(ifos)
    np.savez_compressed(os.path.join(HERE, f"{name}_relbin.npz"), **out)


MB_KEYS = ["durations", "fb_dfb", "Nbs", "Mbs", "Ks_Ke", "banded_frequency_points", "start_end_idxs",
           "unique_to_original_frequencies"]


def run_multiband(bilby, name, n_fixed, n_random, reference_chirp_mass=0.87):
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 2)
    pf = draw_points(w, n_fixed, rng, fixed_extrinsic=True)
    pr = draw_points(w, n_random, rng, fixed_extrinsic=False)
    params = {k: np.concatenate([pf[k], pr[k]]) for k in pf}
    n = n_fixed + n_random
    # drawn after the points, so that the points do not depend on it
    jitter = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n)
    out = {"p_" + k: v for k, v in params.items()}
    out["time_jitter"] = jitter
    for combo in RELBIN_COMBOS + RELBIN_TIME_COMBOS:
        ifos, _ = build_reference(bilby, w, taylorf2_aligned)
        wfg = bilby.gw.waveform_generator.WaveformGenerator(
            duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
            frequency_domain_source_model=taylorf2_aligned_frequency_sequence,
            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
        t, p, d = "t" in combo, "p" in combo, "d" in combo
        priors = make_priors(bilby, w, t, p, d)
        like = bilby.gw.likelihood.MBGravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, reference_chirp_mass=reference_chirp_mass,
            priors=priors if (t or p or d) else None, time_marginalization=t, phase_marginalization=p,
            distance_marginalization=d)
        t0 = time.perf_counter()
        vals = []
        for i in range(n):
            q = point(params, i)
            if t:
                q["geocent_time"] = float(priors["geocent_time"])
                q["time_jitter"] = float(jitter[i])
            if p:
                q["phase"] = 0.0
            if d:
                q["luminosity_distance"] = float(priors["luminosity_distance"])
            vals.append(like.log_likelihood_ratio(q))
        out["lnl_" + combo] = np.array(vals)
        print(f"{name} multiband[{combo}]: {len(like.banded_frequency_points)} banded points, "
              f"{(time.perf_counter() - t0) / n * 1e3:.2f} ms/eval")
        if combo == "none":
            for key in MB_KEYS:
                out["mb_" + key] = np.asarray(getattr(like, key))
            for key in ("time_offset", "delta_f_end", "maximum_banding_frequency"):
                out["mb_" + key] = float(getattr(like, key))
            out["mb_waveform_frequencies"] = np.asarray(wfg.waveform_arguments["frequencies"])
            for q, ifo in enumerate(ifos):
                out[f"mb_linear_coeffs_{q}"] = np.asarray(like.linear_coeffs[ifo.name])
                out[f"mb_quadratic_coeffs_{q}"] = np.asarray(like.quadratic_coeffs[ifo.name])
            out["checksum"] = strain_checksum(ifos)
    np.savez_compressed(os.path.join(HERE, f"{name}_multiband.npz"), **out)


MB_IFFT_COMBOS = ["none", "p", "t", "tpd"]


def run_multiband_ifft(bilby, name, n_fixed, n_random, reference_chirp_mass=0.87, stride=61):
    """The reference's MBGravitationalWaveTransient with the IFFT-FFT <h|h>
    (linear_interpolation=False, multiband.py:613-650, 760-779): lnL ratios
    under four marginalisation combinations, its Tbhats, its windows' sum and
    every ``stride``-th entry of each detector's per-band Ibcs (the full
    arrays are 1.4 MB)."""
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 5)
    pf = draw_points(w, n_fixed, rng, fixed_extrinsic=True)
    pr = draw_points(w, n_random, rng, fixed_extrinsic=False)
    params = {k: np.concatenate([pf[k], pr[k]]) for k in pf}
    n = n_fixed + n_random
    jitter = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n)
    out = {"p_" + k: v for k, v in params.items()}
    out["time_jitter"] = jitter
    for combo in MB_IFFT_COMBOS:
        ifos, _ = build_reference(bilby, w, taylorf2_aligned)
        wfg = bilby.gw.waveform_generator.WaveformGenerator(
            duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
            frequency_domain_source_model=taylorf2_aligned_frequency_sequence,
            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
        t, p, d = "t" in combo, "p" in combo, "d" in combo
        priors = make_priors(bilby, w, t, p, d)
        like = bilby.gw.likelihood.MBGravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, reference_chirp_mass=reference_chirp_mass,
            priors=priors if (t or p or d) else None, time_marginalization=t, phase_marginalization=p,
            distance_marginalization=d, linear_interpolation=False)
        t0 = time.perf_counter()
        vals = []
        for i in range(n):
            q = point(params, i)
            if t:
                q["geocent_time"] = float(priors["geocent_time"])
                q["time_jitter"] = float(jitter[i])
            if p:
                q["phase"] = 0.0
            if d:
                q["luminosity_distance"] = float(priors["luminosity_distance"])
            vals.append(like.log_likelihood_ratio(q))
        out["lnl_" + combo] = np.array(vals)
        print(f"{name} multiband IFFT-FFT[{combo}]: {(time.perf_counter() - t0) / n * 1e3:.2f} ms/eval")
        if combo == "none":
            out["mb_Tbhats"] = np.asarray(like.Tbhats, dtype=np.float64)
            out["mb_windows_sum"] = float(np.sum(like.windows))
            out["mb_n_banded"] = len(like.banded_frequency_points)
            out["ibc_stride"] = stride
            for q, ifo in enumerate(ifos):
                for b, ibc in enumerate(like.Ibcs[ifo.name]):
                    out[f"mb_Ibcs_{q}_{b}"] = np.asarray(ibc)[::stride]
            out["checksum"] = strain_checksum(ifos)
    np.savez_compressed(os.path.join(HERE, f"{name}_multiband_ifft.npz"), **out)


def run_roq(bilby, name="tf2_marg_8s_2k", n_fixed=8, n_random=8):
    from oracle import roq_basis
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 3)
    pf = draw_points(w, n_fixed, rng, fixed_extrinsic=True)
    pr = draw_points(w, n_random, rng, fixed_extrinsic=False)
    params = {k: np.concatenate([pf[k], pr[k]]) for k in pf}
    params.pop("time_jitter", None)
    n = n_fixed + n_random
    # drawn after the points, so that the points do not depend on it
    jitter = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n)
    out = {"p_" + k: v for k, v in params.items()}
    out["time_jitter"] = jitter
    for combo in RELBIN_COMBOS + RELBIN_TIME_COMBOS:
        ifos, _ = build_reference(bilby, w, taylorf2_aligned)
        fm = ifos[0].frequency_array[ifos[0].frequency_mask]
        nl, bl, nq, bq = roq_basis.build(fm, minimum_frequency=w.minimum_frequency)
        wfg = bilby.gw.waveform_generator.WaveformGenerator(
            duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
            frequency_domain_source_model=taylorf2_aligned_roq,
            waveform_arguments=dict(minimum_frequency=w.minimum_frequency, frequency_nodes_linear=nl,
                                    frequency_nodes_quadratic=nq))
        t, p, d = "t" in combo, "p" in combo, "d" in combo
        priors = make_priors(bilby, w, True, p, d)
        like = bilby.gw.likelihood.ROQGravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, priors=priors, linear_matrix=bl.T,
            quadratic_matrix=bq.T, time_marginalization=t, phase_marginalization=p, distance_marginalization=d)
        if t:
            out["roq_tm_delta_tc_" + combo] = float(like._delta_tc)
            out["roq_tm_n_times_" + combo] = len(like._times)
        t0 = time.perf_counter()
        vals = []
        for i in range(n):
            q = point(params, i)
            if t:
                q["geocent_time"] = float(priors["geocent_time"])
                q["time_jitter"] = float(jitter[i])
            if p:
                q["phase"] = 0.0
            if d:
                q["luminosity_distance"] = float(priors["luminosity_distance"])
            vals.append(like.log_likelihood_ratio(q))
        out["lnl_" + combo] = np.array(vals)
        print(f"{name} roq[{combo}]: {len(nl)} linear / {len(nq)} quadratic nodes, "
              f"{(time.perf_counter() - t0) / n * 1e3:.2f} ms/eval")
        if combo == "none":
            ts = np.asarray(like.weights["time_samples"])
            out["roq_time_meta"] = np.array([ts[0], ts[1] - ts[0], len(ts)])
            out["roq_nodes_linear"] = nl
            out["roq_nodes_quadratic"] = nq
            # only the rows of the linear weights these points read (five
            # time samples per point and detector): the whole table is MBs
            for q, ifo in enumerate(ifos):
                rows = set()
                for i in range(n):
                    pt = point(params, i)
                    dt = ifo.time_delay_from_geocenter(pt["ra"], pt["dec"], pt["geocent_time"])
                    t_ifo = pt["geocent_time"] - ifo.strain_data.start_time + dt
                    c = int(np.floor((t_ifo - ts[0]) / (ts[1] - ts[0])))
                    rows.update(min(max(c + k, 0), len(ts) - 1) for k in range(-2, 3))
                rows = np.array(sorted(rows))
                out[f"roq_linear_rows_{q}"] = rows
                out[f"roq_linear_{q}"] = np.asarray(like.weights[ifo.name + "_linear"][0])[rows]
                out[f"roq_quadratic_{q}"] = np.asarray(like.weights[ifo.name + "_quadratic"][0])
            out["checksum"] = strain_checksum(ifos)
    np.savez_compressed(os.path.join(HERE, f"{name}_roq.npz"), **out)


def run_roq_multiband(bilby, name="tf2_marg_8s_2k", n_fixed=6, n_random=6):
    """The reference's ROQ likelihood with a seeded multi-banded basis
    (roq.py:793-1055, _set_weights_linear_multiband and
    _set_weights_quadratic_multiband; oracle/roq_basis.build_multiband).  The
    reference reads such a basis from an hdf5 file only, so its _set_weights
    runs here on the basis dictionary, and a likelihood built from the
    resulting weights gives the lnL ratios without marginalisation, with
    time, and with time, phase and distance marginalisation."""
    from oracle import roq_basis
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 7)
    pf = draw_points(w, n_fixed, rng, fixed_extrinsic=True)
    pr = draw_points(w, n_random, rng, fixed_extrinsic=False)
    params = {k: np.concatenate([pf[k], pr[k]]) for k in pf}
    params.pop("time_jitter", None)
    n = n_fixed + n_random
    jitter = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n)
    out = {"p_" + k: v for k, v in params.items()}
    out["time_jitter"] = jitter
    lin, quad = roq_basis.build_multiband(minimum_frequency=w.minimum_frequency)
    nl = lin["basis_linear"]["0"]["frequency_nodes"]
    nq = quad["basis_quadratic"]["0"]["frequency_nodes"]
    weights = None
    for combo in ("none", "t", "tpd"):
        ifos, _ = build_reference(bilby, w, taylorf2_aligned)
        wfg = bilby.gw.waveform_generator.WaveformGenerator(
            duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
            frequency_domain_source_model=taylorf2_aligned_roq,
            waveform_arguments=dict(minimum_frequency=w.minimum_frequency, frequency_nodes_linear=nl,
                                    frequency_nodes_quadratic=nq))
        t, p, d = "t" in combo, "p" in combo, "d" in combo
        priors = make_priors(bilby, w, True, p, d)
        if weights is None:
            fm = ifos[0].frequency_array[ifos[0].frequency_mask]
            _, bl0, _, bq0 = roq_basis.build(fm, n_linear=4, n_quadratic=2, n_train=20,
                                             minimum_frequency=w.minimum_frequency)
            seed_like = bilby.gw.likelihood.ROQGravitationalWaveTransient(
                interferometers=ifos, waveform_generator=wfg, priors=priors, linear_matrix=bl0.T,
                quadratic_matrix=bq0.T)
            seed_like.weights = dict()
            seed_like._set_weights(linear_matrix=lin, quadratic_matrix=quad)
            weights = seed_like.weights
        like = bilby.gw.likelihood.ROQGravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, priors=priors, weights=weights,
            time_marginalization=t, phase_marginalization=p, distance_marginalization=d)
        vals = []
        for i in range(n):
            q = point(params, i)
            if t:
                q["geocent_time"] = float(priors["geocent_time"])
                q["time_jitter"] = float(jitter[i])
            if p:
                q["phase"] = 0.0
            if d:
                q["luminosity_distance"] = float(priors["luminosity_distance"])
            vals.append(like.log_likelihood_ratio(q))
        out["lnl_" + combo] = np.array(vals)
        print(f"{name} multi-banded roq[{combo}]: {out['lnl_' + combo][:4]}")
        if combo == "none":
            ts = np.asarray(weights["time_samples"])
            out["roq_time_meta"] = np.array([ts[0], ts[1] - ts[0], len(ts)])
            for q, ifo in enumerate(ifos):
                rows = set()
                for i in range(n):
                    pt = point(params, i)
                    dt = ifo.time_delay_from_geocenter(pt["ra"], pt["dec"], pt["geocent_time"])
                    c = int(np.floor((pt["geocent_time"] - ifo.strain_data.start_time + dt - ts[0]) / (ts[1] - ts[0])))
                    rows.update(min(max(c + k, 0), len(ts) - 1) for k in range(-2, 3))
                rows = np.array(sorted(rows))
                out[f"roq_linear_rows_{q}"] = rows
                out[f"roq_linear_{q}"] = np.asarray(weights[ifo.name + "_linear"][0])[rows]
                out[f"roq_quadratic_{q}"] = np.asarray(weights[ifo.name + "_quadratic"][0])
            out["checksum"] = strain_checksum(ifos)
    np.savez_compressed(os.path.join(HERE, f"{name}_roq_multiband.npz"), **out)


# two seeded synthetic bases over overlapping chirp-mass ranges; the
# quadratic ranges differ from the linear ones, so that points take every
# (linear, quadratic) pair of bases
ROQ_BASES = [dict(seed=2024, mass_range=(10.0, 25.0)), dict(seed=2031, mass_range=(20.0, 40.0))]
ROQ_PRIOR_RANGE_LINEAR = np.array([[8.0, 21.0], [19.0, 35.0]])
ROQ_PRIOR_RANGE_QUADRATIC = np.array([[8.0, 25.0], [23.0, 35.0]])


def merge_roq_weights(single, prior_range_linear, prior_range_quadratic):
    """One weights dictionary with several bases (roq.py:193-260) from the
    weights of single-basis likelihoods on the same data: the per-detector
    weight lists and the frequency-node lists concatenated, the time samples
    shared, and the chirp-mass prior range of each basis."""
    out = {"time_samples": np.asarray(single[0]["time_samples"])}
    for key in single[0]:
        if key.endswith("_linear") or key.endswith("_quadratic"):
            out[key] = [np.asarray(w[key][0]) for w in single]
    out["prior_range_linear"] = {"chirp_mass": np.asarray(prior_range_linear)}
    out["prior_range_quadratic"] = {"chirp_mass": np.asarray(prior_range_quadratic)}
    return out


def roq_multibasis_points(w, n, seed):
    """Sampler-style draws for the two-basis ROQ: chirp mass U[9, 34], mass
    ratio U[0.4, 1], the workload's other parameters."""
    rng = np.random.default_rng(seed)
    p = draw_points(w, n, rng, fixed_extrinsic=False)
    p.pop("mass_1")
    p.pop("mass_2")
    p["chirp_mass"] = rng.uniform(9.0, 34.0, n)
    p["mass_ratio"] = rng.uniform(0.4, 1.0, n)
    p["time_jitter"] = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n)
    return p


def run_roq_multibasis(bilby, name="tf2_marg_8s_2k", n_points=24):
    """The reference's ROQGravitationalWaveTransient with two linear and two
    quadratic bases selected per point by chirp-mass ranges (roq.py:193-460),
    given as a weights dictionary, without and with time marginalisation:
    the basis numbers it selected and its lnL ratios."""
    from oracle import roq_basis
    w = WORKLOADS[name]
    params = roq_multibasis_points(w, n_points, w.draw_seed + 23)
    out = {"p_" + k: v for k, v in params.items()}
    for combo in ("none", "t"):
        t = combo == "t"
        single = []
        for b in ROQ_BASES:
            ifos, _ = build_reference(bilby, w, taylorf2_aligned)
            fm = ifos[0].frequency_array[ifos[0].frequency_mask]
            nl, bl, nq, bq = roq_basis.build(fm, minimum_frequency=w.minimum_frequency, seed=b["seed"],
                                            mass_range=b["mass_range"])
            wfg = bilby.gw.waveform_generator.WaveformGenerator(
                duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                frequency_domain_source_model=taylorf2_aligned_roq,
                waveform_arguments=dict(minimum_frequency=w.minimum_frequency, frequency_nodes_linear=nl,
                                        frequency_nodes_quadratic=nq))
            one = bilby.gw.likelihood.ROQGravitationalWaveTransient(
                interferometers=ifos, waveform_generator=wfg, priors=make_priors(bilby, w, True),
                linear_matrix=bl.T, quadratic_matrix=bq.T)
            single.append(dict(one.weights, frequency_nodes_linear=[nl], frequency_nodes_quadratic=[nq]))
        weights = merge_roq_weights(single, ROQ_PRIOR_RANGE_LINEAR, ROQ_PRIOR_RANGE_QUADRATIC)
        ifos, _ = build_reference(bilby, w, taylorf2_aligned)
        wfg = bilby.gw.waveform_generator.WaveformGenerator(
            duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
            frequency_domain_source_model=taylorf2_aligned_roq,
            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
        priors = make_priors(bilby, w, True)
        priors["chirp_mass"] = bilby.core.prior.Uniform(9.0, 34.0, name="chirp_mass")
        like = bilby.gw.likelihood.ROQGravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, priors=priors, weights=weights, time_marginalization=t)
        vals, bl_, bq_ = [], [], []
        for i in range(n_points):
            q = point(params, i)
            if t:
                q["geocent_time"] = float(priors["geocent_time"])
            else:
                q.pop("time_jitter")
            vals.append(like.log_likelihood_ratio(q))
            bl_.append(like.basis_number_linear)
            bq_.append(like.basis_number_quadratic)
        out["lnl_" + combo] = np.array(vals)
        out["basis_linear_" + combo] = np.array(bl_)
        out["basis_quadratic_" + combo] = np.array(bq_)
        print(f"{name} roq two bases [{combo}]: basis pairs {sorted(set(zip(bl_, bq_)))}")
    np.savez_compressed(os.path.join(HERE, f"{name}_roq_multibasis.npz"), **out)


def run_priors(bilby, n=256):
    from bilby.core.prior import (Cosine, Gaussian, LogUniform, PowerLaw, PriorDict, Sine, TruncatedGaussian,
                                  Uniform)
    from bilby.gw.conversion import convert_to_lal_binary_black_hole_parameters
    from bilby.gw.prior import AlignedSpin, UniformInComponentsChirpMass, UniformInComponentsMassRatio
    tc = WORKLOADS["tf2_128s"].injection["geocent_time"]
    cases = {
        "a": dict(chirp_mass=UniformInComponentsChirpMass(0.87, 1.74), mass_ratio=UniformInComponentsMassRatio(0.5, 1.0),
                  chi_1=AlignedSpin(a_prior=Uniform(0, 0.05)), chi_2=Uniform(-0.05, 0.05),
                  luminosity_distance=PowerLaw(2, 20, 200), dec=Cosine(), ra=Uniform(0, 2 * np.pi),
                  theta_jn=Sine(), psi=Uniform(0, np.pi), phase=Uniform(0, 2 * np.pi),
                  geocent_time=Uniform(tc - 0.1, tc + 0.1), hrss=LogUniform(1e-23, 1e-21), Q=Gaussian(10, 2),
                  frequency=TruncatedGaussian(200, 50, 50, 500)),
        "b": dict(chirp_mass=UniformInComponentsChirpMass(5, 30),
                  mass_ratio=UniformInComponentsMassRatio(0.125, 1.0, equal_mass=True),
                  cos_theta_jn=Uniform(-1, 1), luminosity_distance=PowerLaw(-1, 100, 1000)),
    }
    rng = np.random.default_rng(99)
    out = {}
    for name, d in cases.items():
        priors = PriorDict(d)
        keys = list(priors.keys())
        u = rng.uniform(size=(len(keys), n))
        vals = priors.rescale(keys, u)
        params = {k: np.asarray(v, dtype=np.float64) for k, v in zip(keys, vals)}
        conv, _ = convert_to_lal_binary_black_hole_parameters(dict(params))
        out[f"{name}_keys"] = np.array(keys)
        out[f"{name}_unit"] = u
        # the device program compiled from the reference's own prior objects
        from bilby_gb300.priors_device import compile_program
        prog = compile_program(priors, keys)
        out[f"{name}_prog_head"] = np.array([[k, t, c] for k, t, c, _, _, _ in prog], dtype=np.int64)
        out[f"{name}_prog_p"] = np.array([pp for _, _, _, pp, _, _ in prog], dtype=np.float64)
        for j, (_, _, _, _, tx, ty) in enumerate(prog):
            if tx is not None:
                out[f"{name}_prog_tx_{j}"] = tx
                out[f"{name}_prog_ty_{j}"] = ty
        for k in keys:
            out[f"{name}_v_{k}"] = params[k]
        for k in ("mass_1", "mass_2", "theta_jn"):
            if k in conv:
                out[f"{name}_c_{k}"] = np.asarray(conv[k], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "priors.npz"), **out)
    print("priors", {k: len(v) for k, v in cases.items()})


FRAME_CASES = [("H1L1", "geocent"), ("H1L1", "H1"), ("sky", "L1"), ("L1V1", "V1")]


def run_frames(bilby, n=16):
    w = WORKLOADS["sg_4s"]
    rng = np.random.default_rng(77)
    out = {}
    pts = dict(zenith=np.arccos(rng.uniform(-1, 1, n)), azimuth=rng.uniform(0, 2 * np.pi, n),
               ra=rng.uniform(0, 2 * np.pi, n), dec=np.arcsin(rng.uniform(-1, 1, n)),
               t=w.start_time + rng.uniform(0.5, 3.5, n))
    out.update({"p_" + k: v for k, v in pts.items()})
    for q, (frame, tref) in enumerate(FRAME_CASES):
        ifos, wfg = build_reference(bilby, w, bilby.gw.source.sinegaussian)
        like = bilby.gw.likelihood.GravitationalWaveTransient(interferometers=ifos, waveform_generator=wfg,
                                                              reference_frame=frame, time_reference=tref)
        key = "geocent_time" if "geocent" in tref else f"{tref}_time"
        res = np.zeros((n, 3))
        for i in range(n):
            par = dict(zenith=pts["zenith"][i], azimuth=pts["azimuth"][i], ra=pts["ra"][i], dec=pts["dec"][i])
            par[key] = pts["t"][i]
            r = like.get_sky_frame_parameters(par)
            res[i] = [r["ra"], r["dec"], r["geocent_time"]]
        out[f"frame_{q}"] = res
    np.savez_compressed(os.path.join(HERE, "sky_frames.npz"), **out)
    print("sky frames", len(FRAME_CASES), "cases")


RECON_COMBOS = ["t", "d", "p", "tpd"]
RECON_SEED = 4321


def run_snrs(bilby, name="tf2_marg_8s_2k", n_points=3):
    """The per-detector inner products (base.py:260-354), per-detector
    likelihoods (base.py:479-499) and posterior reconstruction draws
    (base.py:502-770) of the reference, on points of the marginalised
    workload.  The time series d_inner_h_array is stored inside the
    geocent_time prior window only, with its full-length sum and power."""
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 7)
    params = draw_points(w, n_points, rng, fixed_extrinsic=False)
    params["time_jitter"] = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n_points)
    out = {"p_" + k: v for k, v in params.items()}
    # plain likelihood: calculate_snrs and per-detector lnL
    ifos, wfg = build_reference(bilby, w, taylorf2_aligned)
    like = bilby.gw.likelihood.GravitationalWaveTransient(interferometers=ifos, waveform_generator=wfg)
    names = [ifo.name for ifo in ifos]
    dh = np.zeros((n_points, len(ifos)), complex)
    hh = np.zeros((n_points, len(ifos)))
    mf = np.zeros((n_points, len(ifos)), complex)
    per_det = np.zeros((n_points, len(ifos)))
    for i in range(n_points):
        q = point(params, i)
        q.pop("time_jitter")
        pols = wfg.frequency_domain_strain(dict(q))
        for k, ifo in enumerate(ifos):
            s = like.calculate_snrs(pols, ifo, parameters=dict(q))
            dh[i, k], hh[i, k], mf[i, k] = s.d_inner_h, s.optimal_snr_squared, s.complex_matched_filter_snr
        res = like.compute_per_detector_log_likelihood(dict(q))
        per_det[i] = [res[f"{n}_log_likelihood"] for n in names]
    out.update(snr_dh=dh, snr_hh=hh, snr_mf=mf, per_det_lnl=per_det)
    # marginalised likelihoods: per-detector lnL, the time series, reconstruction
    for combo in RECON_COMBOS:
        ifos, wfg = build_reference(bilby, w, taylorf2_aligned)
        t, p, d = "t" in combo, "p" in combo, "d" in combo
        priors = make_priors(bilby, w, t, p, d)
        like = bilby.gw.likelihood.GravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, priors=priors,
            time_marginalization=t, phase_marginalization=p, distance_marginalization=d)
        per_det = np.zeros((n_points, len(ifos)))
        draws = np.zeros((n_points, 3))
        for i in range(n_points):
            q = point(params, i)
            if t:
                q["geocent_time"] = float(priors["geocent_time"])
            else:
                q.pop("time_jitter")
            if p:
                q["phase"] = 0.0
            if d:
                q["luminosity_distance"] = float(priors["luminosity_distance"])
            res = like.compute_per_detector_log_likelihood(dict(q))
            per_det[i] = [res[f"{n}_log_likelihood"] for n in names]
            if combo == "t":
                qq = dict(q)
                qq["geocent_time"] += qq["time_jitter"]
                pols = wfg.frequency_domain_strain(dict(qq))
                win = None
                for k, ifo in enumerate(ifos):
                    s = like.calculate_snrs(pols, ifo, parameters=dict(qq))
                    arr = s.d_inner_h_array
                    times = like._times + qq["time_jitter"]
                    tp = like.priors["geocent_time"]
                    idx = np.nonzero((times >= tp.minimum) & (times <= tp.maximum))[0]
                    if win is None:
                        win = np.zeros((len(ifos), len(idx)), complex)
                        out[f"series_idx_{i}"] = idx
                    win[k] = arr[idx]
                    out.setdefault("series_sum", np.zeros((n_points, len(ifos)), complex))[i, k] = arr.sum()
                    out.setdefault("series_power", np.zeros((n_points, len(ifos))))[i, k] = np.sum(np.abs(arr) ** 2)
                out[f"series_{i}"] = win
            bilby.core.utils.random.seed(RECON_SEED + i)
            sample = like.generate_posterior_sample_from_marginalized_likelihood(dict(q))
            draws[i] = [sample["geocent_time"], sample["luminosity_distance"], sample["phase"]]
        out["per_det_lnl_" + combo] = per_det
        out["recon_" + combo] = draws
        print(f"{name}[{combo}]: per-detector lnL and reconstruction draws done")
    out["detectors"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, f"{name}_snrs.npz"), **out)


def run_fast_snrs(bilby, name="tf2_128s", n_points=2):
    """calculate_snrs and compute_per_detector_log_likelihood of the
    reference's relative-binning and multi-banded likelihoods, without and
    with time marginalisation (the d_inner_h_array inside the prior window,
    its sum and power)."""
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 11)
    params = draw_points(w, n_points, rng, fixed_extrinsic=False)
    params["time_jitter"] = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n_points)
    out = {"p_" + k: v for k, v in params.items()}
    for kind in ("relbin", "multiband"):
        for combo in ("none", "t"):
            ifos, _ = build_reference(bilby, w, taylorf2_aligned)
            t = combo == "t"
            priors = make_priors(bilby, w, t, False, False)
            if kind == "relbin":
                wfg = bilby.gw.waveform_generator.WaveformGenerator(
                    duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                    frequency_domain_source_model=taylorf2_aligned_relative_binning,
                    waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
                fiducial = dict(w.injection, time_jitter=0.0) if t else dict(w.injection)
                like = bilby.gw.likelihood.RelativeBinningGravitationalWaveTransient(
                    interferometers=ifos, waveform_generator=wfg, fiducial_parameters=fiducial,
                    priors=priors if t else None, time_marginalization=t)
            else:
                wfg = bilby.gw.waveform_generator.WaveformGenerator(
                    duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                    frequency_domain_source_model=taylorf2_aligned_frequency_sequence,
                    waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
                like = bilby.gw.likelihood.MBGravitationalWaveTransient(
                    interferometers=ifos, waveform_generator=wfg, reference_chirp_mass=0.87,
                    priors=priors if t else None, time_marginalization=t)
            key = f"{kind}_{combo}"
            dh = np.zeros((n_points, len(ifos)), complex)
            hh = np.zeros((n_points, len(ifos)))
            per_det = np.zeros((n_points, len(ifos)))
            for i in range(n_points):
                q = point(params, i)
                if t:
                    q["geocent_time"] = float(priors["geocent_time"]) + q["time_jitter"]
                else:
                    q.pop("time_jitter")
                pols = wfg.frequency_domain_strain(dict(q))
                for k, ifo in enumerate(ifos):
                    snr = like.calculate_snrs(pols, ifo, parameters=dict(q))
                    dh[i, k], hh[i, k] = snr.d_inner_h, snr.optimal_snr_squared
                    if t:
                        arr = np.asarray(snr.d_inner_h_array)
                        times = like._times + q["time_jitter"]
                        tp = like.priors["geocent_time"]
                        idx = np.nonzero((times >= tp.minimum) & (times <= tp.maximum))[0]
                        out[f"{key}_series_idx_{i}_{k}"] = idx
                        out[f"{key}_series_{i}_{k}"] = arr[idx]
                        out[f"{key}_series_len"] = len(arr)
                        out.setdefault(f"{key}_series_sum", np.zeros((n_points, len(ifos)), complex))[i, k] = arr.sum()
                        out.setdefault(f"{key}_series_power", np.zeros((n_points, len(ifos))))[i, k] = \
                            np.sum(np.abs(arr) ** 2)
                qq = dict(q)
                if t:
                    qq["geocent_time"] -= qq["time_jitter"]
                res = like.compute_per_detector_log_likelihood(dict(qq))
                per_det[i] = [res[f"{ifo.name}_log_likelihood"] for ifo in ifos]
                if t and kind == "multiband":  # multiband.py:822-855 draws with numpy's global generator
                    np.random.seed(RECON_SEED + i)
                    out.setdefault(f"{key}_time_draw", np.zeros(n_points))[i] = \
                        like.generate_time_sample_from_marginalized_likelihood(parameters=dict(qq))
                if t and kind == "relbin":  # base.py:577-653 with the piecewise waveform, bilby's generator
                    bilby.core.utils.random.seed(RECON_SEED + i)
                    out.setdefault(f"{key}_time_draw", np.zeros(n_points))[i] = \
                        like.generate_time_sample_from_marginalized_likelihood(parameters=dict(qq))
            out[f"{key}_dh"] = dh
            out[f"{key}_hh"] = hh
            out[f"{key}_per_det_lnl"] = per_det
            print(f"{name} {key}: per-detector SNRs done")
    np.savez_compressed(os.path.join(HERE, f"{name}_fast_snrs.npz"), **out)


def run_roq_snrs(bilby, name="tf2_marg_8s_2k", n_points=2):
    """calculate_snrs, compute_per_detector_log_likelihood and (with time
    marginalisation) the time draw of the reference's ROQ likelihood with the
    seeded synthetic basis of oracle/roq_basis.py; the d_inner_h_array is
    stored for its first 400 samples, with its sum and power."""
    from oracle import roq_basis
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 13)
    params = draw_points(w, n_points, rng, fixed_extrinsic=False)
    params["time_jitter"] = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n_points)
    out = {"p_" + k: v for k, v in params.items()}
    for combo in ("none", "t"):
        ifos, _ = build_reference(bilby, w, taylorf2_aligned)
        fm = ifos[0].frequency_array[ifos[0].frequency_mask]
        nl, bl, nq, bq = roq_basis.build(fm, minimum_frequency=w.minimum_frequency)
        wfg = bilby.gw.waveform_generator.WaveformGenerator(
            duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
            frequency_domain_source_model=taylorf2_aligned_roq,
            waveform_arguments=dict(minimum_frequency=w.minimum_frequency, frequency_nodes_linear=nl,
                                    frequency_nodes_quadratic=nq))
        t = combo == "t"
        priors = make_priors(bilby, w, True, False, False)
        like = bilby.gw.likelihood.ROQGravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, priors=priors, linear_matrix=bl.T,
            quadratic_matrix=bq.T, time_marginalization=t)
        key = f"roq_{combo}"
        dh = np.zeros((n_points, len(ifos)), complex)
        hh = np.zeros((n_points, len(ifos)))
        per_det = np.zeros((n_points, len(ifos)))
        for i in range(n_points):
            q = point(params, i)
            if t:
                q["geocent_time"] = float(priors["geocent_time"])
            else:
                q.pop("time_jitter")
            pols = wfg.frequency_domain_strain(dict(q))
            for k, ifo in enumerate(ifos):
                snr = like.calculate_snrs(pols, ifo, parameters=dict(q))
                dh[i, k], hh[i, k] = snr.d_inner_h, snr.optimal_snr_squared
                if t:
                    arr = np.asarray(snr.d_inner_h_array)
                    out[f"{key}_series_{i}_{k}"] = arr[:400]
                    out[f"{key}_series_len"] = len(arr)
                    out.setdefault(f"{key}_series_sum", np.zeros((n_points, len(ifos)), complex))[i, k] = arr.sum()
                    out.setdefault(f"{key}_series_power", np.zeros((n_points, len(ifos))))[i, k] = \
                        np.sum(np.abs(arr) ** 2)
            res = like.compute_per_detector_log_likelihood(dict(q))
            per_det[i] = [res[f"{ifo.name}_log_likelihood"] for ifo in ifos]
            if t:  # roq.py:1238-1271 draws with bilby's generator
                bilby.core.utils.random.seed(RECON_SEED + i)
                out.setdefault(f"{key}_time_draw", np.zeros(n_points))[i] = \
                    like.generate_time_sample_from_marginalized_likelihood(parameters=dict(q))
        out[f"{key}_dh"] = dh
        out[f"{key}_hh"] = hh
        out[f"{key}_per_det_lnl"] = per_det
        print(f"{name} {key}: per-detector SNRs done")
    np.savez_compressed(os.path.join(HERE, f"{name}_roq_snrs.npz"), **out)


def run_sg_marginalised(bilby, name="sg_4s", n_points=16):
    """The reference's time- and time+phase-marginalised likelihood for the
    sine-Gaussian burst (no distance parameter, so no distance
    marginalisation)."""
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 17)
    params = draw_points(w, n_points, rng, fixed_extrinsic=False)
    params["time_jitter"] = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n_points)
    out = {"p_" + k: v for k, v in params.items()}
    for combo in ("t", "tp"):
        ifos, wfg = build_reference(bilby, w, bilby.gw.source.sinegaussian)
        priors = make_priors(bilby, w, True, "p" in combo, False)
        like = bilby.gw.likelihood.GravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, priors=priors, time_marginalization=True,
            phase_marginalization="p" in combo)
        vals = []
        for i in range(n_points):
            q = point(params, i)
            q["geocent_time"] = float(priors["geocent_time"])
            if "p" in combo:
                q["phase"] = 0.0
            vals.append(like.log_likelihood_ratio(q))
        out["lnl_" + combo] = np.array(vals)
        print(f"{name}[{combo}] done")
    np.savez_compressed(os.path.join(HERE, f"{name}_marg.npz"), **out)


TIME_PRIOR = dict(mu_offset=0.02, sigma=0.04)   # TruncatedGaussian on geocent_time, within t_inj +- 0.1 s


def run_time_prior(bilby, name="tf2_marg_8s_2k", n_points=8):
    """The reference's time-marginalised likelihood under a geocent_time prior
    other than Uniform: TruncatedGaussian(mu = t_inj + 0.02, sigma = 0.04,
    t_inj -+ 0.1), with time, time+phase, time+distance and all three."""
    w = WORKLOADS[name]
    rng = np.random.default_rng(w.draw_seed + 19)
    params = draw_points(w, n_points, rng, fixed_extrinsic=False)
    params["time_jitter"] = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n_points)
    out = {"p_" + k: v for k, v in params.items()}
    tc = w.injection["geocent_time"]
    for combo in ("t", "tp", "td", "tpd"):
        ifos, wfg = build_reference(bilby, w, taylorf2_aligned)
        priors = make_priors(bilby, w, True, "p" in combo, "d" in combo)
        priors["geocent_time"] = bilby.core.prior.TruncatedGaussian(
            mu=tc + TIME_PRIOR["mu_offset"], sigma=TIME_PRIOR["sigma"], minimum=tc - 0.1, maximum=tc + 0.1,
            name="geocent_time")
        like = bilby.gw.likelihood.GravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, priors=priors, time_marginalization=True,
            phase_marginalization="p" in combo, distance_marginalization="d" in combo)
        vals = []
        for i in range(n_points):
            q = point(params, i)
            q["geocent_time"] = float(priors["geocent_time"])
            if "p" in combo:
                q["phase"] = 0.0
            if "d" in combo:
                q["luminosity_distance"] = float(priors["luminosity_distance"])
            vals.append(like.log_likelihood_ratio(q))
        out["lnl_" + combo] = np.array(vals)
        print(f"{name} time prior [{combo}] done")
    np.savez_compressed(os.path.join(HERE, f"{name}_time_prior.npz"), **out)


def known_answer(bilby):
    """test/gw/likelihood_test.py:143-201 (noise lnL only; the lnL value
    there needs IMRPhenomPv2 from lalsimulation)."""
    bilby.core.utils.random.seed(500)
    ifos = bilby.gw.detector.InterferometerList(["H1"])
    ifos.set_strain_data_from_power_spectral_densities(sampling_frequency=2048.0, duration=4.0)
    wfg = bilby.gw.waveform_generator.WaveformGenerator(
        duration=4.0, sampling_frequency=2048.0, frequency_domain_source_model=bilby.gw.source.sinegaussian)
    like = bilby.gw.likelihood.GravitationalWaveTransient(interferometers=ifos, waveform_generator=wfg)
    nll = float(like.noise_log_likelihood())
    with open(os.path.join(HERE, "known_answer.json"), "w") as f:
        json.dump({"H1_seed500_4s_2048Hz_noise_log_likelihood": nll,
                   "reference_test_value": -4014.1787704539474}, f, indent=1)
    print("known answer", nll)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--relbin-only", action="store_true")
    ap.add_argument("--multiband-only", action="store_true")
    ap.add_argument("--multiband-ifft-only", action="store_true")
    ap.add_argument("--frames-only", action="store_true")
    ap.add_argument("--priors-only", action="store_true")
    ap.add_argument("--roq-only", action="store_true")
    ap.add_argument("--snrs-only", action="store_true")
    ap.add_argument("--marg-only", action="store_true")
    ap.add_argument("--time-prior-only", action="store_true")
    ap.add_argument("--roq-multibasis-only", action="store_true")
    ap.add_argument("--roq-multiband-only", action="store_true")
    args = ap.parse_args()
    bilby = ref_harness.import_bilby()
    if args.roq_multiband_only:
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            try:
                run_roq_multiband(bilby)
            finally:
                os.chdir(cwd)
        return
    if args.roq_multibasis_only or args.time_prior_only:
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            try:
                if args.time_prior_only:
                    run_time_prior(bilby)
                    run_marginalised(bilby, "tf2_marg_6s_2k", 8)
                if args.roq_multibasis_only:
                    run_roq_multibasis(bilby)
            finally:
                os.chdir(cwd)
        return
    if args.marg_only:
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            try:
                run_marginalised(bilby, "tf2_marg_8s_2k", 8)
                run_marginalised(bilby, "tf2_marg_8s", 16)
            finally:
                os.chdir(cwd)
        return
    if args.snrs_only:
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            try:
                run_snrs(bilby)
                run_fast_snrs(bilby)
                run_roq_snrs(bilby)
                run_sg_marginalised(bilby)
            finally:
                os.chdir(cwd)
        return
    if args.roq_only:
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            try:
                run_roq(bilby)
            finally:
                os.chdir(cwd)
        return
    if args.priors_only:
        run_priors(bilby)
        return
    if args.frames_only:
        run_frames(bilby)
        return
    if args.multiband_ifft_only:
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            try:
                run_multiband_ifft(bilby, "tf2_128s", 4, 4)
            finally:
                os.chdir(cwd)
        return
    if args.multiband_only:
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            try:
                run_multiband(bilby, "tf2_128s", 8, 8)
            finally:
                os.chdir(cwd)
        return
    if args.relbin_only:
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            try:
                run_relbin(bilby, "tf2_128s", 8, 8)
            finally:
                os.chdir(cwd)
        return
    export_noise_curves()
    known_answer(bilby)
    run_plain(bilby, "sg_4s", 32, 32)
    run_frames(bilby)
    run_plain(bilby, "tf2_128s", 4, 4)
    if not args.quick:
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)  # the reference caches its distance table in the working directory
            try:
                run_marginalised(bilby, "tf2_marg_8s_2k", 8)
                run_marginalised(bilby, "tf2_marg_8s", 16)
                run_marginalised(bilby, "tf2_marg_6s_2k", 8)
                run_time_prior(bilby)
                run_relbin(bilby, "tf2_128s", 8, 8)
                run_multiband(bilby, "tf2_128s", 8, 8)
                run_multiband_ifft(bilby, "tf2_128s", 4, 4)
                run_roq(bilby)
                run_roq_multibasis(bilby)
                run_roq_multiband(bilby)
                run_snrs(bilby)
                run_fast_snrs(bilby)
                run_roq_snrs(bilby)
                run_sg_marginalised(bilby)
            finally:
                os.chdir(cwd)


if __name__ == "__main__":
    main()
