"""Generates the golden fixtures in this directory from the compiled reference.

Run in a checkout that has the reference sources (it builds oracle/_ref from
them first):

    python tests/golden/gen_golden.py

Every case feeds the reference serial build (driven through
oracle/ref/ref_harness.cpp) the particles of the seeded sampler and records
what the reference produces. Nothing here runs on the product.
"""
import hashlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from apc_524_project_gb300 import abi, configs, loading  # noqa: E402
from backends import RefBackend, by_id  # noqa: E402
from golden import cases  # noqa: E402

FIELDS = list(range(13))


def particles_hash(parts):
    h = hashlib.sha256()
    for p in parts:
        for k in ("x", "y", "z", "vx", "vy", "vz", "gamma"):
            h.update(np.ascontiguousarray(p[k]).tobytes())
    return h.hexdigest()


def load(b, parts):
    nid = 0
    for si, p in enumerate(parts):
        n = len(p["x"])
        b.add_species(si, p, ids=np.arange(nid, nid + n))
        nid += n


def gen_case(name):
    cfg, dt, steps, exact = cases.make(name)
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    b = RefBackend(info, dt)
    load(b, parts)
    b.init_fields()
    out = {"sample_sha256": np.array(particles_hash(parts))}
    init_f = {i: b.get_field(i) for i in FIELDS}
    for i in FIELDS:
        out[f"init_field_{i}"] = init_f[i]
    pf = b.particle_fields()
    ids = b.particles()["id"]
    o = np.argsort(ids)
    out["init_particle_fields"] = pf[o]
    counts, hist = [], []
    for ti in range(steps):
        c, h = b.step(ti)
        counts.append(c)
        if h is not None:
            hist.append(h)
    p = by_id(b.particles())
    for k in ("x", "y", "z", "vx", "vy", "vz", "gamma", "type", "id"):
        out[f"final_{k}"] = p[k]
    for i in FIELDS:
        out[f"final_field_{i}"] = b.get_field(i)
    out["counts"] = np.array(counts, dtype=np.int64)
    out["history"] = np.array(hist)
    out["time"] = np.array(RefBackend.lib().refh_time())
    b.close()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def gen_edges():
    cfg = configs.tiny("edges", init="constant", E0=(0.01, 0.02, -0.01), B0=(0.0, 0.0, 0.1))
    info = configs.input_info(cfg)
    p = cases.edge_particles(cfg)
    b = RefBackend(info, 0.4)
    b.add_species(0, p, ids=np.arange(len(p["x"])))
    cid = np.array([b.cell_id(x, y, z) for x, y, z in zip(p["x"], p["y"], p["z"])], dtype=np.int64)
    b.init_fields()
    pf = b.particle_fields()
    b.deposit(True)
    fields = {f"field_{i}": b.get_field(i) for i in (abi.JX, abi.JY, abi.JZ, abi.RHO)}
    b.close()
    np.savez_compressed(os.path.join(HERE, "edges.npz"), cell_id=cid, particle_fields=pf, **fields)


def gen_sort_order():
    """The reference's particle order after one SortParticles on the
    sorted_test particles (after the field start): ids, species and cell keys
    (Grid::getCellID) in storage order."""
    cfg, dt, steps, exact = cases.make("sorted_test")
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    b = RefBackend(info, dt)
    load(b, parts)
    b.init_fields()
    b.sort()
    p = b.particles()
    keys = np.array([b.cell_id(x, y, z) for x, y, z in zip(p["x"], p["y"], p["z"])], dtype=np.int64)
    b.close()
    np.savez_compressed(os.path.join(HERE, "sort_order.npz"), sample_sha256=np.array(particles_hash(parts)),
                        id=np.asarray(p["id"], dtype=np.int64), type=np.asarray(p["type"], dtype=np.int32),
                        key=keys)


def gen_pusher():
    st, fl = cases.pusher_inputs()
    out = {}
    for rel in (0, 1):
        res = np.array([RefBackend.pusher_steps(rel, st[i], fl[i], 0.05, 40) for i in range(len(st))])
        out[f"rel{rel}"] = res
    np.savez_compressed(os.path.join(HERE, "pusher.npz"), state=st, field=fl, **out)


def gen_summary(name):
    factory, dt, steps = cases.SUMMARY_CASES[name]
    cfg = factory()
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    b = RefBackend(info, dt)
    load(b, parts)
    b.init_fields()
    rng = np.random.default_rng(99)
    npts = int(np.prod([v + 3 for v in cfg.n]))
    probe = rng.choice(npts, 256, replace=False)
    out = {"sample_sha256": np.array(particles_hash(parts)), "probe": probe}

    def snap(tag):
        for i in FIELDS:
            f = b.get_field(i).ravel()
            out[f"{tag}_norm_{i}"] = np.array(np.sqrt(np.sum(f * f)))
            out[f"{tag}_probe_{i}"] = f[probe]

    snap("init")
    counts, hist = [], []
    for ti in range(steps):
        c, h = b.step(ti)
        counts.append(c)
        if h is not None:
            hist.append(h)
    snap("final")
    p = by_id(b.particles())
    out["final_moments"] = np.array([np.sum(p["x"]), np.sum(p["vx"] ** 2 + p["vy"] ** 2 + p["vz"] ** 2),
                                     np.sum(p["y"]), np.sum(p["z"])])
    out["counts"] = np.array(counts, dtype=np.int64)
    out["history"] = np.array(hist)
    b.close()
    np.savez_compressed(os.path.join(HERE, f"summary_{name}.npz"), **out)


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), "-s"], check=True)
    # the sampler lives in the product library (host code only)
    sys.path.insert(0, ROOT)
    import __graft_entry__  # noqa: F401  (build() compiles libemoo.so)
    __graft_entry__.build()
    which = sys.argv[1:] or (list(cases.CASES) + ["edges", "pusher", "sort_order"] +
                             [f"summary:{k}" for k in cases.SUMMARY_CASES])
    for w in which:
        print("generating", w, flush=True)
        if w == "edges":
            gen_edges()
        elif w == "pusher":
            gen_pusher()
        elif w == "sort_order":
            gen_sort_order()
        elif w.startswith("summary:"):
            gen_summary(w.split(":", 1)[1])
        else:
            gen_case(w)


if __name__ == "__main__":
    main()
