"""Shared test helpers: run a golden case on a backend and compare results."""
import os

import numpy as np

from apc_524_project_gb300 import configs, loading
from backends import by_id, rel_l2
from golden import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = list(range(13))


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def load_case_particles(b, cfg):
    parts = loading.sample_all(cfg)
    nid = 0
    for si, p in enumerate(parts):
        n = len(p["x"])
        b.add_species(si, p, ids=np.arange(nid, nid + n))
        nid += n
    return parts


def run_cpu_case(B, name):
    """Runs golden case `name` on a CPU backend class (oracle or reference)."""
    cfg, dt, steps, exact = cases.make(name)
    info = configs.input_info(cfg)
    b = B(info, dt)
    parts = load_case_particles(b, cfg)
    b.init_fields()
    out = {"init_fields": {i: b.get_field(i) for i in FIELDS}}
    pf = b.particle_fields()
    ids = b.particles()["id"]
    out["init_particle_fields"] = pf[np.argsort(ids)]
    counts, hist = [], []
    for ti in range(steps):
        c, h = b.step(ti)
        counts.append(c)
        if h is not None:
            hist.append(h)
    out["particles"] = by_id(b.particles())
    out["fields"] = {i: b.get_field(i) for i in FIELDS}
    out["counts"] = np.array(counts, dtype=np.int64)
    out["history"] = np.array(hist)
    out["parts_in"] = parts
    b.close()
    return out


def total_mass(info, parts):
    return sum(info.mass_ratio[si] * len(p["x"]) for si, p in enumerate(parts))


def history_close(a, b, rtol, mass):
    """History rows agree: t loosely (the reference prints it with 6 digits),
    energies to rtol, and each momentum to rtol times the row's momentum
    scale sqrt(2 * KE * total mass) >= sum m|v| / sqrt(3) (the momenta are
    sums of terms that cancel, so their own size is no scale)."""
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    if a.size == 0:
        return
    np.testing.assert_allclose(a[:, 0], b[:, 0], rtol=1e-5, atol=1e-12)
    for r in range(a.shape[0]):
        scale = np.sqrt(2.0 * abs(b[r, 4]) * mass) * np.sqrt(3.0)
        np.testing.assert_allclose(a[r, 1:4], b[r, 1:4], rtol=0, atol=rtol * scale + 1e-300)
    np.testing.assert_allclose(a[:, 4:], b[:, 4:], rtol=rtol, atol=1e-300)


__all__ = ["load_golden", "run_cpu_case", "history_close", "rel_l2", "FIELDS", "cases"]
