"""Host-side particle sampling through the native sampler (emoo_generate_host,
or any function of its signature, such as the CPU oracle's copy orc_generate).

The arrays are bit-identical on every platform (the sampler uses only
separately rounded basic operations). For a Poisson start with all-periodic
field boundaries the reference removes each species' mean velocity
(Particle_Handler::zeroAvgChargeAndVelocity_,
src/particles/particle_handler.cpp:379-444); the mean is taken here with
math.fsum (correctly rounded, so platform independent).
"""
import ctypes as C
import math

import numpy as np

from . import abi
from .configs import Config, gen_params


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def sample_species(cfg: Config, si: int, first: int = 0, n: int = None, generate=None):
    """Returns dict of float64 arrays x, y, z, vx, vy, vz, gamma for species si.
    generate: a ctypes function with emoo_generate_host's signature (default:
    the library's)."""
    if n is None:
        n = cfg.count(cfg.species[si]) - first
    g = gen_params(cfg, si)
    out = {k: np.empty(n, dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz", "gamma")}
    fn = generate or abi.lib().emoo_generate_host
    abi.check(fn(C.byref(g), first, n, _ptr(out["x"]), _ptr(out["y"]), _ptr(out["z"]),
                 _ptr(out["vx"]), _ptr(out["vy"]), _ptr(out["vz"]), _ptr(out["gamma"])), "generate particles")
    return out


def zero_mean(parts):
    n = len(parts["vx"])
    if n == 0:
        return parts
    for k in ("vx", "vy", "vz"):
        m = math.fsum(parts[k].tolist()) / n
        parts[k] = parts[k] - m
    return parts


def sample_all(cfg: Config, generate=None):
    """List (per species) of particle dicts, with the mean-velocity removal
    applied when the reference would apply it."""
    res = []
    zm = cfg.want_zero_mean()
    for si in range(len(cfg.species)):
        p = sample_species(cfg, si, generate=generate)
        if zm:
            p = zero_mean(p)
        res.append(p)
    return res
