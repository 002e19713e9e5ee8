"""FP64 GPU form against the CPU oracle and the reference's golden vectors.

Tolerances (stated per the parity contract):
  * integer work - cell indices, crossing counts per side, the stable sort
    permutation, Jacobi iteration counts - must match exactly;
  * per-particle arithmetic (gather, push, boundaries), the Yee update, ghost
    fills, folds and the Jacobi solve are bit-exact on identical inputs (same
    order of operations, no fused multiply-add);
  * anything downstream of the current deposit differs only by the order in
    which particle contributions are summed: relative L2 <= FP64_RTOL after a
    multi-step run, <= DEPOSIT_RTOL for a single deposit.
"""
import ctypes as C

import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading
from backends import GpuBackend, OracleBackend, by_id, rel_l2
from golden import cases
from golden.gen_golden import particles_hash
from helpers import FIELDS, history_close, load_golden, total_mass

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9      # fields and particles after a multi-step run
DEPOSIT_RTOL = 1e-13  # one deposit: summation order only
HIST_RTOL = 1e-9


def _load(b, parts):
    nid = 0
    for si, p in enumerate(parts):
        n = len(p["x"])
        b.add_species(si, p, ids=np.arange(nid, nid + n))
        nid += n


def _pair(cfg, dt, load=True):
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    g = GpuBackend(info, dt)
    o = OracleBackend(info, dt)
    if load:
        _load(g, parts)
        _load(o, parts)
    return g, o, parts, info


def _random_fields(shape, seed, scale=0.1):
    rng = np.random.default_rng(seed)
    return {i: rng.uniform(-scale, scale, shape) for i in FIELDS}


@pytest.mark.parametrize("name", list(cases.CASES))
def test_time_loop_matches_oracle_and_reference(name):
    cfg, dt, steps, exact = cases.make(name)
    g, o, parts, info = _pair(cfg, dt)
    rg, itg = g.init_fields()
    ro, ito = o.init_fields()
    assert rg == ro and itg == ito, (rg, ro, itg, ito)
    for i in FIELDS:  # Poisson start on identical rho/J order -> exact up to the deposit order
        assert rel_l2(g.get_field(i), o.get_field(i)) <= DEPOSIT_RTOL * 10, i
    hist_o, counts_g = [], []
    for ti in range(steps):
        cg = g.step(1)
        co, h = o.step(ti)
        assert cg == co, f"step {ti}: crossings {cg} vs {co}"
        counts_g.append(cg)
        if h is not None:
            hist_o.append(h)
    pg, po = by_id(g.particles()), by_id(o.particles())
    np.testing.assert_array_equal(pg["id"], po["id"])
    np.testing.assert_array_equal(pg["type"], po["type"])
    for k in ("x", "y", "z", "vx", "vy", "vz", "gamma"):
        assert rel_l2(pg[k], po[k]) <= FP64_RTOL, (k, rel_l2(pg[k], po[k]))
    for i in FIELDS:
        assert rel_l2(g.get_field(i), o.get_field(i)) <= FP64_RTOL, (i, rel_l2(g.get_field(i), o.get_field(i)))
    mass = total_mass(info, parts)
    history_close(g.history_rows(), np.array(hist_o), HIST_RTOL, mass)
    # and directly against the reference's recorded end state
    gold = load_golden(name)
    np.testing.assert_array_equal(np.array(counts_g), gold["counts"])
    for i in FIELDS:
        assert rel_l2(g.get_field(i), gold[f"final_field_{i}"]) <= FP64_RTOL, i
    g.close()
    o.close()


def test_yee_ghost_fold_bit_exact():
    cfg = configs.tiny("yee", n=(6, 5, 7), dx=(0.7, 1.3, 0.5), init="constant")
    g, o, parts, info = _pair(cfg, 0.3, load=False)
    f = _random_fields(g.shape, 11)
    for i in FIELDS:
        g.set_field(i, f[i])
        o.set_field(i, f[i])
    for b in (g, o):
        b.execute_bc(abi.SEND_JRHO)
        b.evolve(False)
        b.execute_bc(abi.SEND_EB)
        b.evolve(False)  # second swap of the B roles
        b.execute_bc(abi.SEND_EB)
        b.evolve(True)
        b.execute_bc(abi.EX)
    for i in FIELDS:
        np.testing.assert_array_equal(g.get_field(i), o.get_field(i), err_msg=abi.FIELD_NAMES[i])


def test_external_light_bc_bit_exact():
    W = configs.Wave
    cfg = configs.tiny("light", init="constant", E0=(0.0, 0.01, 0.0), B0=(0.0, 0.0, 0.02),
                       part_bc=("reflecting", "reflecting", "periodic", "periodic", "reflecting", "reflecting"),
                       field_bc=("external", "external", "periodic", "periodic", "external", "external"),
                       waves=[W(-1, 2, 0.5, 0.4, 20.0, 0.2, 2.0), W(3, 1, 0.1, 0.9, 0.0, 0.0, 0.0)])
    g, o, parts, info = _pair(cfg, 0.35)
    g.init_fields()
    o.init_fields()
    for ti in range(6):
        g.step(1)
        o.step(ti)
    for i in range(6):
        assert rel_l2(g.get_field(i), o.get_field(i)) <= FP64_RTOL, i


def test_gather_push_bc_bit_exact():
    cfg = configs.tiny("unit", relativity=1, init="constant", vth=0.1,
                       part_bc=("reflecting", "reflecting", "periodic", "periodic", "periodic", "periodic"),
                       field_bc=("external", "external", "periodic", "periodic", "periodic", "periodic"))
    g, o, parts, info = _pair(cfg, 0.4)
    f = _random_fields(g.shape, 5, scale=0.3)
    for i in FIELDS:
        g.set_field(i, f[i])
        o.set_field(i, f[i])
    g.interpolate()
    o.interpolate()
    np.testing.assert_array_equal(g.particle_fields(), o.particle_fields())
    g.push()
    o.push()
    pg, po = by_id(g.particles()), by_id(o.particles())
    for k in ("x", "y", "z", "vx", "vy", "vz", "gamma"):
        np.testing.assert_array_equal(pg[k], po[k], err_msg=k)
    cg = g.particle_bc()
    co = o.particle_bc()
    assert cg == co
    pg, po = by_id(g.particles()), by_id(o.particles())
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_array_equal(pg[k], po[k], err_msg=k)


def test_deposit_matches_oracle():
    cfg = configs.tiny("dep", n=(8, 7, 6), dx=(1.0, 0.5, 2.0), ppc=6, init="constant", test_species=True)
    g, o, parts, info = _pair(cfg, 0.4)
    g.deposit(True)
    o.deposit(True)
    for i in (abi.JX, abi.JY, abi.JZ, abi.RHO):
        assert rel_l2(g.get_field(i), o.get_field(i)) <= DEPOSIT_RTOL, i


def test_poisson_bit_exact_and_iteration_counts():
    cfg = configs.tiny("pois", n=(8, 6, 10), init="poisson",
                       field_bc=("external", "external", "periodic", "periodic", "periodic", "periodic"),
                       part_bc=("reflecting", "reflecting", "periodic", "periodic", "periodic", "periodic"))
    cfg.bound_phi = (0.0, 0.02, 0.0, 0.0, 0.0, 0.0)
    cfg.bound_A = ((0.0,) * 6, (0.0, 1.2, 0.0, 0.0, 0.0, 0.0), (0.0,) * 6)
    g, o, parts, info = _pair(cfg, 0.4, load=False)
    rng = np.random.default_rng(2)
    rho = rng.normal(0, 1e-3, g.shape)
    for b in (g, o):
        b.set_field(abi.RHO, rho)
        b.set_field(abi.JY, rho * 0.1)
    rg, itg = g.poisson_init()
    ro, ito = o.initialize_fields_only()
    assert itg == ito and rg == ro, (itg, ito, rg, ro)
    for i in list(range(13)) + [abi.PHI1, abi.PHI2, abi.AY1, abi.AY2]:
        np.testing.assert_array_equal(g.get_field(i), o.get_field(i), err_msg=abi.FIELD_NAMES[i])


def test_stable_sort_permutation_matches_oracle():
    cfg = configs.tiny("sort", n=(7, 6, 5), ppc=9, init="constant")
    g, o, parts, info = _pair(cfg, 0.4)
    g.sort()
    o.sort()
    pg, po = g.particles(), o.particles()
    np.testing.assert_array_equal(pg["id"], po["id"])
    np.testing.assert_array_equal(pg["x"], po["x"])
    keys = [g.cell_id(x, y, z) for x, y, z in zip(pg["x"], pg["y"], pg["z"])]
    t = pg["type"]
    assert all((t[i], keys[i]) <= (t[i + 1], keys[i + 1]) for i in range(len(keys) - 1))


def test_sort_matches_the_references_order():
    """The reference sorts all particles together, descending by cell, with
    an unstable std::sort (src/particles/particle_utils.hpp:31-51); the GPU
    sorts each species ascending and stably. After the same field start, per
    species the GPU's key sequence is the reference's reversed, each cell
    holds the same particles in both, and within a cell the GPU keeps the
    load order (tests/golden/sort_order.npz, recorded from the reference)."""
    gold = load_golden("sort_order")
    cfg, dt, steps, _ = cases.make("sorted_test")
    g, o, parts, info = _pair(cfg, dt)
    assert particles_hash(parts) == str(gold["sample_sha256"])
    g.init_fields()
    g.sort()
    pg = g.particles()
    keys = np.array([g.cell_id(x, y, z) for x, y, z in zip(pg["x"], pg["y"], pg["z"])])
    for s in range(len(parts)):
        mine = pg["type"] == s
        ref = gold["type"] == s
        np.testing.assert_array_equal(keys[mine], gold["key"][ref][::-1])
        for k in np.unique(keys[mine]):
            ids_gpu = pg["id"][mine][keys[mine] == k]
            ids_ref = np.sort(gold["id"][ref][gold["key"][ref] == k])
            np.testing.assert_array_equal(ids_gpu, ids_ref)  # stable: load order = ascending id
    g.close()
    o.close()


# The 32^3 Langmuir run on the reference's scheme: its gather is
# discontinuous at cell faces (ghost-offset vertex), so a particle that lands
# within rounding distance of a face in one run and across it in the other
# changes its cell's force by O(1) for a step. The GPU sums the current with
# FP64 atomics (another order than the reference's particle vector), and over
# 40 steps of this growing mode that moves single probe points by up to ~5e-8
# relative while every crossing count stays exact. Measured on the GB300: field
# norms within 4.3e-11, the probe vectors within 2.9e-9 in relative L2. The
# bars: counts exact, norms and history FP64_RTOL, the probe vector
# LANGMUIR_PROBE_RTOL in relative L2.
LANGMUIR_PROBE_RTOL = 2e-8


def test_langmuir32_full_size_matches_the_reference():
    """The baseline's CPU-runnable case at full size on the GPU: 32^3 cells,
    524,288 particles, Jacobi Poisson start, the FP64 form over the 40 steps
    the reference completes (tests/golden/summary_langmuir32.npz, recorded from
    the compiled reference). Crossing counts per step are exact; field norms
    and the history rows agree to FP64_RTOL, the 256 probe points of every
    field to LANGMUIR_PROBE_RTOL in relative L2."""
    gold = load_golden("summary_langmuir32")
    factory, dt, steps = cases.SUMMARY_CASES["langmuir32"]
    cfg = factory()
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    assert particles_hash(parts) == str(gold["sample_sha256"])
    g = GpuBackend(info, dt)
    _load(g, parts)
    g.init_fields()
    probe = gold["probe"]
    worst = {}

    def close(tag, probe_rtol):
        for i in FIELDS:
            f = g.get_field(i).ravel()
            norm = float(np.sqrt(np.sum(f * f)))
            ref_norm = float(gold[f"{tag}_norm_{i}"])
            dn = abs(norm - ref_norm) / max(ref_norm, 1e-300)
            dp = rel_l2(f[probe], gold[f"{tag}_probe_{i}"])
            worst[tag] = max(worst.get(tag, (0.0, 0.0)), (dn, dp))
            assert dn <= FP64_RTOL, (tag, i, dn)
            assert dp <= probe_rtol, (tag, i, dp)

    close("init", FP64_RTOL)
    counts = np.array([g.step(1) for _ in range(steps)], dtype=np.int64)
    np.testing.assert_array_equal(counts, gold["counts"])
    close("final", LANGMUIR_PROBE_RTOL)
    history_close(g.history_rows(), gold["history"], HIST_RTOL, total_mass(info, parts))
    p = by_id(g.particles())
    mom = np.array([np.sum(p["x"]), np.sum(p["vx"] ** 2 + p["vy"] ** 2 + p["vz"] ** 2), np.sum(p["y"]),
                    np.sum(p["z"])])
    np.testing.assert_allclose(mom, gold["final_moments"], rtol=FP64_RTOL)
    assert g.check() == abi.OK
    g.close()
    print("langmuir32 vs reference (norm rel diff, probe rel L2):", worst)


def test_device_loader_matches_host_sampler():
    cfg = configs.tiny("load", n=(10, 9, 8), ppc=5, relativity=1, init="constant", vth=0.2)
    info = configs.input_info(cfg)
    g = GpuBackend(info, 0.4, track_ids=1)
    gp = configs.gen_params(cfg, 1)
    n = cfg.count(cfg.species[1])
    abi.check(g.L.emoo_load_generated(g.h, C.byref(gp), n))
    host = loading.sample_species(cfg, 1)
    p = g.particles()
    for k in ("x", "y", "z", "vx", "vy", "vz", "gamma"):
        np.testing.assert_array_equal(p[k][p["type"] == 1], host[k], err_msg=k)


def test_gauss_residual_and_history_match_oracle():
    cfg, dt, steps, _ = cases.make("periodic_poisson")
    g, o, parts, info = _pair(cfg, dt)
    g.init_fields()
    o.init_fields()
    rg, ro = g.gauss_residual(), o.gauss_residual()
    assert abs(rg[0] - ro[0]) <= 1e-12 * max(1.0, abs(ro[0])) and abs(rg[1] - ro[1]) <= 1e-10 * max(1.0, ro[1])
    hg = g.history()
    ho = o.history(0.0)
    history_close(np.array([hg]), np.array([ho]), 1e-12, total_mass(info, parts))


def test_out_of_grid_particle_is_reported_not_faulted():
    """A particle far outside the grid is caught by the kernels' own bounds
    check (the reference asserts in getCellID, src/grid/oGrid.cpp:212): the
    call returns EMOO_ERR_BOUNDS and the handle stays usable."""
    cfg = configs.tiny("oob", init="constant")
    info = configs.input_info(cfg)
    g = GpuBackend(info, 0.4)
    p = {k: np.array([-100.0, 1.5]) for k in ("x", "y", "z")}
    p.update({k: np.zeros(2) for k in ("vx", "vy", "vz", "gamma")})
    g.add_species(0, p)
    rc = g.L.emoo_interpolate(g.h)
    assert rc == abi.ERR_BOUNDS
    assert g.L.emoo_check(g.h) == abi.OK
    g.close()
