"""Named parity cases shared by the golden-vector generator and the tests.

Each case is a small configuration (fast on every backend) exercising one
part of the reference's behaviour; `summary` cases are full-size runs of
which only reductions are stored.
"""
import math
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))

from apc_524_project_gb300 import configs  # noqa: E402

W = configs.Wave

# name -> (config factory, dt, steps, bit_exact_vs_reference)
CASES = {
    "periodic_poisson": (lambda: configs.tiny("periodic_poisson"), 0.45, 12, True),
    "rel_const": (lambda: configs.tiny("rel_const", relativity=1, init="constant", B0=(0.1, 0.2, 0.3),
                                       E0=(0.01, 0.0, 0.02), vth=0.15), 0.4, 12, True),
    "reflect_ext": (lambda: configs.tiny(
        "reflect_ext", relativity=1, init="constant",
        part_bc=("reflecting", "reflecting", "periodic", "periodic", "periodic", "periodic"),
        field_bc=("external", "external", "periodic", "periodic", "periodic", "periodic"),
        waves=[W(-1, 2, 0.05, 0.8, 30.0, 0.3, 1.0), W(-1, 3, 0.02, 0.5, 0.0, 0.0, 0.0),
               W(1, 2, 0.01, 1.1, 45.0, 0.5, 0.5)], vth=0.2, B0=(0.0, 0.0, 0.05)), 0.4, 12, True),
    "aniso_poisson": (lambda: configs.tiny("aniso_poisson", n=(5, 6, 7), dx=(0.7, 1.3, 0.5), init="poisson",
                                           vth=0.01), 0.4, 8, True),
    "aniso_const": (lambda: configs.tiny("aniso_const", n=(5, 6, 7), dx=(0.7, 1.3, 0.5), init="constant",
                                         B0=(0.02, 0.0, 0.01)), 0.4, 12, True),
    "sorted_test": (lambda: configs.tiny("sorted_test", nstep_sort=3, test_species=True), 0.4, 12, False),
    "es_poisson": (lambda: _es(), 0.4, 8, True),
}

SUMMARY_CASES = {
    # the 32^3 Langmuir workload, full size (524,288 particles). The
    # reference's scheme is unstable on it: by step 49 a particle crosses more
    # than a box length in one step and the reference aborts on its own
    # assertion (src/boundaries/b_particles/bc_p_periodic.cpp:59), so the
    # stored horizon is 40 steps.
    "langmuir32": (configs.langmuir32, 0.5, 40),
}


def _es():
    c = configs.tiny("es_poisson", vth=0.05)
    c.electrostatic = 1
    return c


def make(name):
    f, dt, steps, exact = CASES[name]
    return f(), dt, steps, exact


def pusher_inputs(n=16, seed=3):
    """Deterministic single-particle states and fields for the pusher cases:
    state = {x, y, z, vx, vy, vz, gamma, q, m}, field = {e1, e2, e3, b1, b2, b3}."""
    import numpy as np
    rng = np.random.default_rng(seed)
    st = np.zeros((n, 9))
    st[:, 0:3] = rng.uniform(-2, 2, (n, 3))
    st[:, 3:6] = rng.uniform(-0.4, 0.4, (n, 3))
    v2 = np.sum(st[:, 3:6] ** 2, axis=1)
    st[:, 6] = np.sqrt(1.0 - v2)
    st[:, 7] = rng.choice([-1.0, 1.0, 2.0], n) * rng.uniform(0.5, 2.0, n)
    st[:, 8] = rng.uniform(0.5, 3.0, n)
    fl = rng.uniform(-1.0, 1.0, (n, 6))
    return st, fl


def edge_particles(cfg):
    """Particles on cell faces and exactly on the domain faces (x == x0 and
    x == x0 + L), at rest, for the cell-index edge cases."""
    import numpy as np
    L = cfg.L
    xs = [0.0, L[0], L[0] * (1 - 1e-16), 1.0, cfg.dx[0] * 2.5, L[0] - cfg.dx[0]]
    pts = []
    for a in xs:
        for b in (0.0, L[1], 0.5 * cfg.dx[1]):
            pts.append((a, b, 0.5 * L[2]))
    pts = np.array(pts)
    n = len(pts)
    return {"x": pts[:, 0].copy(), "y": pts[:, 1].copy(), "z": pts[:, 2].copy(), "vx": np.zeros(n),
            "vy": np.zeros(n), "vz": np.zeros(n), "gamma": np.zeros(n)}


_ = math
