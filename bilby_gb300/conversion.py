"""Host-side parameter conversion (bilby/gw/conversion.py:182-283 and the mass
helpers it calls, :849-989, :1826-1990), vectorised over numpy arrays so that a
batch of points converts in one call.  Redshift / comoving-distance inputs
need a cosmology and are not supported here: pass ``luminosity_distance``."""
from __future__ import annotations

import numpy as np


def _xp(x):
    """numpy, or torch for a torch tensor (CUDA batches convert on the device)."""
    if hasattr(x, "is_cuda"):
        import torch
        return torch
    return np


def _component_masses(p):
    """generate_component_masses (conversion.py:1826-1990), detector frame."""
    out = dict(p)
    if "mass_1" in p and "mass_2" in p:
        return out
    q = out.get("mass_ratio")
    if q is None and "symmetric_mass_ratio" in out:
        temp = 1 / out["symmetric_mass_ratio"] / 2 - 1
        q = temp - (temp ** 2 - 1) ** 0.5
    if "mass_1" in out:
        if "total_mass" in out:
            out["mass_2"] = out["total_mass"] - out["mass_1"]
        elif q is not None:
            out["mass_2"] = q * out["mass_1"]
        return out
    if "mass_2" in out:
        if "total_mass" in out:
            out["mass_1"] = out["total_mass"] - out["mass_2"]
        elif q is not None:
            out["mass_1"] = out["mass_2"] / q
        return out
    if "total_mass" in out:
        if q is None and "chirp_mass" in out:
            eta = (out["chirp_mass"] / out["total_mass"]) ** (5 / 3)
            temp = 1 / eta / 2 - 1
            q = temp - (temp ** 2 - 1) ** 0.5
        if q is None:
            return out
        total = out["total_mass"]
    elif "chirp_mass" in out and q is not None:
        total = out["chirp_mass"] * (1 + q) ** 1.2 / q ** 0.6   # conversion.py:987-989
    else:
        return out
    out["mass_ratio"] = q
    out["mass_1"] = total / (1 + q)                              # conversion.py:849-870
    out["mass_2"] = out["mass_1"] * q
    return out


def convert_to_lal_binary_black_hole_parameters(parameters):
    """Returns (converted parameters, added keys) like the reference."""
    converted = dict(parameters)
    original = list(converted.keys())
    if "luminosity_distance" not in original and ("redshift" in original or "comoving_distance" in original):
        raise NotImplementedError("redshift / comoving-distance inputs need a cosmology: pass luminosity_distance")
    converted = _component_masses(converted)
    for idx in ("1", "2"):
        key = f"chi_{idx}"
        if key in original and f"a_{idx}" not in original:
            converted[f"a_{idx}"] = abs(converted[key])
            converted[f"cos_tilt_{idx}"] = _xp(converted[key]).sign(converted[key])
    for key in ("phi_jl", "phi_12"):
        converted.setdefault(key, 0.0)
    for angle in ("tilt_1", "tilt_2", "theta_jn"):
        if f"cos_{angle}" in converted:
            with np.errstate(invalid="ignore"):
                converted[angle] = _xp(converted[f"cos_{angle}"]).arccos(converted[f"cos_{angle}"])
    if "delta_phase" in converted:
        with np.errstate(invalid="ignore"):
            xp = _xp(converted["delta_phase"])
            converted["phase"] = xp.remainder(converted["delta_phase"] - xp.sign(xp.cos(converted["theta_jn"]))
                                              * converted["psi"], 2 * np.pi)
    added = [k for k in converted if k not in original]
    return converted, added
