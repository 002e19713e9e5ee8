"""The CPU oracle against the golden vectors recorded from the compiled
reference (tests/golden/gen_golden.py). This pins the oracle: where the
reference's order of operations is fixed (no sort in the run) the oracle must
reproduce it bit for bit; with sorting, only the summation order of the
current differs and the tolerance below applies."""
import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading
from backends import OracleBackend
from golden import cases
from helpers import FIELDS, history_close, load_golden, rel_l2, run_cpu_case, total_mass
from golden.gen_golden import particles_hash

SORTED_RTOL = 1e-12  # relative L2, sorted runs (summation order of J differs)


@pytest.mark.parametrize("name", list(cases.CASES))
def test_oracle_matches_reference_golden(name):
    g = load_golden(name)
    cfg, dt, steps, exact = cases.make(name)
    out = run_cpu_case(OracleBackend, name)
    # the seeded sampler reproduces the recorded inputs
    assert particles_hash(out["parts_in"]) == str(g["sample_sha256"])
    np.testing.assert_array_equal(out["counts"], g["counts"])
    info = configs.input_info(cfg)
    mass = total_mass(info, out["parts_in"])
    if exact:
        for i in FIELDS:
            np.testing.assert_array_equal(out["init_fields"][i], g[f"init_field_{i}"], err_msg=f"init field {i}")
            np.testing.assert_array_equal(out["fields"][i], g[f"final_field_{i}"], err_msg=f"final field {i}")
        np.testing.assert_array_equal(out["init_particle_fields"], g["init_particle_fields"])
        for k in ("x", "y", "z", "vx", "vy", "vz", "gamma", "type", "id"):
            np.testing.assert_array_equal(out["particles"][k], g[f"final_{k}"], err_msg=k)
        # the reference prints history with 16 significant digits
        history_close(out["history"], g["history"], 1e-15, mass)
    else:
        for i in FIELDS:
            assert rel_l2(out["fields"][i], g[f"final_field_{i}"]) < SORTED_RTOL, i
        for k in ("x", "y", "z", "vx", "vy", "vz"):
            assert rel_l2(out["particles"][k], g[f"final_{k}"]) < SORTED_RTOL, k
        np.testing.assert_array_equal(out["particles"]["id"], g["final_id"])
        history_close(out["history"], g["history"], 1e-12, mass)


def test_oracle_pushers_match_reference():
    g = load_golden("pusher")
    for rel in (0, 1):
        res = np.array([OracleBackend.pusher_steps(rel, g["state"][i], g["field"][i], 0.05, 40)
                        for i in range(len(g["state"]))])
        np.testing.assert_array_equal(res, g[f"rel{rel}"])


def test_oracle_edge_positions():
    """Particles exactly on cell faces and on the domain faces (x == x0 + L
    lands in the ghost cell n+1, as getCellID's truncation gives)."""
    g = load_golden("edges")
    cfg = configs.tiny("edges", init="constant", E0=(0.01, 0.02, -0.01), B0=(0.0, 0.0, 0.1))
    info = configs.input_info(cfg)
    p = cases.edge_particles(cfg)
    b = OracleBackend(info, 0.4)
    b.add_species(0, p, ids=np.arange(len(p["x"])))
    cid = np.array([b.cell_id(x, y, z) for x, y, z in zip(p["x"], p["y"], p["z"])])
    np.testing.assert_array_equal(cid, g["cell_id"])
    b.init_fields()
    b.interpolate()
    np.testing.assert_array_equal(b.particle_fields(), g["particle_fields"])
    b.deposit(True)
    for i in (abi.JX, abi.JY, abi.JZ, abi.RHO):
        np.testing.assert_array_equal(b.get_field(i), g[f"field_{i}"])


def test_oracle_langmuir32_summary():
    """Full-size 32^3 Langmuir run (524,288 particles, Poisson start) against
    the reference's recorded reductions over the horizon it completes."""
    g = load_golden("summary_langmuir32")
    factory, dt, steps = cases.SUMMARY_CASES["langmuir32"]
    cfg = factory()
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    assert particles_hash(parts) == str(g["sample_sha256"])
    b = OracleBackend(info, dt)
    nid = 0
    for si, p in enumerate(parts):
        b.add_species(si, p, ids=np.arange(nid, nid + len(p["x"])))
        nid += len(p["x"])
    b.init_fields()
    probe = g["probe"]
    for i in FIELDS:
        f = b.get_field(i).ravel()
        np.testing.assert_array_equal(f[probe], g[f"init_probe_{i}"])
    counts, hist = [], []
    for ti in range(steps):
        c, h = b.step(ti)
        counts.append(c)
        if h is not None:
            hist.append(h)
    np.testing.assert_array_equal(np.array(counts), g["counts"])
    for i in FIELDS:
        f = b.get_field(i).ravel()
        np.testing.assert_array_equal(f[probe], g[f"final_probe_{i}"])
        assert float(np.sqrt(np.sum(f * f))) == float(g[f"final_norm_{i}"])
    history_close(np.array(hist), g["history"], 1e-15, total_mass(info, parts))
    b.close()


def test_oracle_sampler_equals_the_library_sampler():
    """The CPU legs generate particles with the oracle's copy of the sampler
    (orc_generate); it produces the library's arrays bit for bit."""
    cfg = configs.thermal256(8)
    for si in range(len(cfg.species)):
        a = loading.sample_species(cfg, si)
        b = loading.sample_species(cfg, si, generate=OracleBackend.generator())
        for k in a:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
