"""Seeded synthetic workloads for the GW-transient likelihood.

There is no public benchmark suite for this path: every workload is
synthetic, built the way bilby builds an injection study (seeded Gaussian
noise coloured by a bundled detector PSD, one injected signal), with the
shapes and prior ranges of the configurations the benchmark is quoted on:

``sg_4s``      sine-Gaussian burst, H1+L1, 4 s at 2048 Hz (4097 bins), f_min 20 Hz,
               hrss log-uniform [1e-23, 1e-21], Q U[3, 30], f0 U[50, 500] Hz; plain lnL.
``tf2_128s``   3.5PN aligned-spin TaylorF2, H1/L1/V1, 128 s at 4096 Hz (262145 bins),
               m1, m2 U[1, 2] Msun, chi U[-0.05, 0.05]; 4096 points per launch.
``tf2_marg_8s`` TaylorF2 m1, m2 U[10, 40] Msun, H1+L1, 8 s at 4096 Hz (16385 bins,
               FFT length 16384), time + phase + distance marginalisation; 8192 points.
``tf2_marg_8s_2k`` the same at 2048 Hz (8193 bins, FFT length 8192).
``tf2_marg_6s_2k`` the same for a 6 s segment at 2048 Hz (6145 bins, FFT length
               6144 = 3 x 2048, not a power of two).

Prior draws for the extrinsic parameters: ra U[0, 2 pi), dec = arcsin U[-1, 1],
psi U[0, pi), geocent_time U[t_inj - 0.1, t_inj + 0.1]; theta_jn = arccos U[-1, 1],
phase U[0, 2 pi), luminosity_distance U[20, 200] Mpc (TaylorF2 plain).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

START_TIME = 1126259640.0


@dataclass(frozen=True)
class Workload:
    name: str
    model: str                       # "sinegaussian" | "taylorf2"
    detectors: tuple
    sampling_frequency: float
    duration: float
    seed: int                        # noise seed (bilby.core.utils.random.seed)
    draw_seed: int                   # prior-draw seed (numpy default_rng)
    batch: int                       # points per launch
    injection: dict = field(default_factory=dict)
    time_marginalization: bool = False
    phase_marginalization: bool = False
    distance_marginalization: bool = False
    minimum_frequency: float = 20.0
    start_time: float = START_TIME
    mass_range: tuple = (10.0, 40.0)   # component masses (Msun) of the TaylorF2 prior draws

    @property
    def n_bins(self) -> int:
        return int(round(self.duration * self.sampling_frequency / 2)) + 1


_SKY = dict(ra=1.375, dec=-1.2108, psi=2.659)

WORKLOADS = {
    "sg_4s": Workload(
        "sg_4s", "sinegaussian", ("H1", "L1"), 2048.0, 4.0, seed=1, draw_seed=2, batch=10000,
        injection=dict(hrss=1e-22, Q=9.0, frequency=200.0, geocent_time=START_TIME + 2.0, **_SKY)),
    "tf2_128s": Workload(
        "tf2_128s", "taylorf2", ("H1", "L1", "V1"), 4096.0, 128.0, seed=3, draw_seed=3, batch=4096,
        injection=dict(mass_1=1.5, mass_2=1.3, chi_1=0.02, chi_2=-0.01, luminosity_distance=100.0,
                       theta_jn=0.4, phase=1.3, geocent_time=START_TIME + 124.0, **_SKY), mass_range=(1.0, 2.0)),
    "tf2_marg_8s": Workload(
        "tf2_marg_8s", "taylorf2", ("H1", "L1"), 4096.0, 8.0, seed=4, draw_seed=4, batch=8192,
        injection=dict(mass_1=30.0, mass_2=25.0, chi_1=0.02, chi_2=-0.01, luminosity_distance=800.0,
                       theta_jn=0.4, phase=1.3, geocent_time=START_TIME + 6.0, **_SKY),
        time_marginalization=True, phase_marginalization=True, distance_marginalization=True),
    "tf2_marg_8s_2k": Workload(
        "tf2_marg_8s_2k", "taylorf2", ("H1", "L1"), 2048.0, 8.0, seed=4, draw_seed=4, batch=8192,
        injection=dict(mass_1=30.0, mass_2=25.0, chi_1=0.02, chi_2=-0.01, luminosity_distance=800.0,
                       theta_jn=0.4, phase=1.3, geocent_time=START_TIME + 6.0, **_SKY),
        time_marginalization=True, phase_marginalization=True, distance_marginalization=True),
    "tf2_marg_6s_2k": Workload(
        "tf2_marg_6s_2k", "taylorf2", ("H1", "L1"), 2048.0, 6.0, seed=4, draw_seed=6, batch=8192,
        injection=dict(mass_1=30.0, mass_2=25.0, chi_1=0.02, chi_2=-0.01, luminosity_distance=800.0,
                       theta_jn=0.4, phase=1.3, geocent_time=START_TIME + 4.0, **_SKY),
        time_marginalization=True, phase_marginalization=True, distance_marginalization=True),
}

# distance prior of the marginalised workloads: PowerLaw(alpha=2, 100, 5000) Mpc
DISTANCE_PRIOR = dict(alpha=2.0, minimum=100.0, maximum=5000.0)


def draw_points(w: Workload, n: int, rng=None, fixed_extrinsic: bool = False) -> dict:
    """Draw ``n`` prior points for workload ``w`` as a dict of float64 arrays."""
    rng = np.random.default_rng(w.draw_seed) if rng is None else rng
    inj = w.injection
    out: dict = {}
    if w.model == "sinegaussian":
        out["hrss"] = 10 ** rng.uniform(-23, -21, n)
        out["Q"] = rng.uniform(3, 30, n)
        out["frequency"] = rng.uniform(50, 500, n)
    else:
        lo, hi = w.mass_range
        m1 = rng.uniform(lo, hi, n)
        m2 = rng.uniform(lo, hi, n)
        out["mass_1"] = np.maximum(m1, m2)
        out["mass_2"] = np.minimum(m1, m2)
        out["chi_1"] = rng.uniform(-0.05, 0.05, n)
        out["chi_2"] = rng.uniform(-0.05, 0.05, n)
        if w.distance_marginalization:
            out["luminosity_distance"] = rng.uniform(DISTANCE_PRIOR["minimum"], DISTANCE_PRIOR["maximum"], n)
        else:
            out["luminosity_distance"] = rng.uniform(20, 200, n)
        out["theta_jn"] = np.arccos(rng.uniform(-1, 1, n))
        out["phase"] = rng.uniform(0, 2 * np.pi, n)
    if fixed_extrinsic:
        for k in ("ra", "dec", "psi", "geocent_time"):
            out[k] = np.full(n, inj[k])
    else:
        out["ra"] = rng.uniform(0, 2 * np.pi, n)
        out["dec"] = np.arcsin(rng.uniform(-1, 1, n))
        out["psi"] = rng.uniform(0, np.pi, n)
        out["geocent_time"] = inj["geocent_time"] + rng.uniform(-0.1, 0.1, n)
    if w.time_marginalization:
        out["time_jitter"] = rng.uniform(-1.0 / w.sampling_frequency, 1.0 / w.sampling_frequency, n)
    return out


def point(params: dict, i: int) -> dict:
    """The ``i``-th point of a batch as a plain dict of Python floats."""
    return {k: float(v[i]) for k, v in params.items()}


# Mixed-duration TaylorF2 analyses (uneven batching): component-mass ranges
# whose inspirals from 20 Hz fit the segment, with the segment's injection.
_MASS_BY_DURATION = {4: (10.0, 40.0), 8: (10.0, 40.0), 16: (5.0, 10.0), 32: (2.5, 5.0), 64: (1.5, 3.0),
                     128: (1.0, 2.0)}


def uneven_analyses(n: int = 64, seed: int = 5) -> list:
    """``n`` TaylorF2 analyses: duration U{4,8,16,32,64,128} s, sampling rate
    U{2048, 4096} Hz, 2 or 3 detectors, batch log-uniform in [256, 4096]."""
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        T = float(rng.choice([4, 8, 16, 32, 64, 128]))
        fs = float(rng.choice([2048, 4096]))
        D = int(rng.choice([2, 3]))
        B = int(round(np.exp(rng.uniform(np.log(256), np.log(4096)))))
        lo, hi = _MASS_BY_DURATION[int(T)]
        m1, m2 = sorted(rng.uniform(lo, hi, 2))[::-1]
        inj = dict(mass_1=m1, mass_2=m2, chi_1=0.01, chi_2=-0.01, luminosity_distance=float(rng.uniform(100, 400)),
                   theta_jn=0.4, phase=1.3, geocent_time=START_TIME + T - 2.0, **_SKY)
        out.append(Workload(f"uneven_{q}", "taylorf2", ("H1", "L1", "V1")[:D], fs, T, seed=1000 + q,
                            draw_seed=2000 + q, batch=B, injection=inj, mass_range=(lo, hi)))
    return out
