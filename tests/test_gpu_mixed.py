"""Mixed-precision form against the FP64 form (and so against the reference).

The mixed form is the same algorithm in FP32 with split-precision positions;
its error is stated against the FP64 GPU form:
  * initial state: positions to FP32 offset precision, fields <= 1e-7;
  * a stable run (the external-wave, reflecting case): relative L2 of E, B,
    J, rho <= MIXED_RTOL after 12 steps, crossing counts identical;
  * runs where the scheme itself amplifies perturbations: the mixed error
    after N steps stays within ENSEMBLE_FACTOR times the spread of an FP64
    ensemble perturbed after every step by the mixed form's own one-step
    rounding (emoo_perturb; the amplitude measured, a few FP32 ulps): what
    FP32 rounding alone does to this loop, measured instead of assumed
    (apc_524_project_gb300/precision.py);
    the thermal plasma of the 256^3 benchmark, scaled to 24^3, is checked
    that way over 100 steps in tests/test_mixed_error.py;
  * the fixed-point current makes runs bit-reproducible.
"""
import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading
from backends import GpuBackend, by_id, rel_l2
from golden import cases

pytestmark = pytest.mark.gpu

MIXED_RTOL = 2e-6
# The mixed error may be at most this many times the largest distance of the
# FP64 ensemble's members from the unperturbed FP64 run. These are the
# reference policy's tiny golden cases, where the gather jumps at cell faces
# and the FP32 current sum's rounding enters E within the same step (the
# ensemble perturbs the state between steps): measured on the GB300 the mixed
# distance is 0.4-2.2 times the largest member's. The benchmark's thermal
# plasma under the corrected policy meets 2x with room to spare
# (tests/test_mixed_error.py).
ENSEMBLE_FACTOR = 3.0
ENSEMBLE_MEMBERS = 6
FP32_ROUNDING = 2.0 ** -24


def _load(b, parts):
    nid = 0
    for si, p in enumerate(parts):
        n = len(p["x"])
        b.add_species(si, p, ids=np.arange(nid, nid + n))
        nid += n


INIT_FIELDS = (abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ, abi.BX_TM1, abi.BY_TM1, abi.BZ_TM1)


def _run(cfg, dt, steps, precision, perturb_seed=None, start_fields=None, rel=FP32_ROUNDING):
    """Runs cfg for `steps` steps; perturb_seed: after every step perturb the
    FP64 state by relative amplitude rel (emoo_perturb) with that seed;
    start_fields: E, B, B_tm1 to start from instead of the handle's own field
    start (returned as out["start"])."""
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    b = GpuBackend(info, dt, precision=precision)
    _load(b, parts)
    b.init_fields()
    if start_fields is not None:
        for i, a in start_fields.items():
            b.set_field(i, a)
    start = {i: b.get_field(i) for i in INIT_FIELDS}
    counts = np.zeros(6, dtype=np.int64)
    if perturb_seed is not None:  # the mixed form rounds the state it loads, too
        abi.check(b.L.emoo_perturb(b.h, perturb_seed * 1000003 + steps + 7, rel))
    for t in range(steps):
        counts += np.array(b.step(1))
        if perturb_seed is not None:
            abi.check(b.L.emoo_perturb(b.h, perturb_seed * 1000003 + t, rel))
    out = {i: b.get_field(i) for i in (abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ, abi.JX, abi.RHO)}
    out["p"] = by_id(b.particles())
    out["counts"] = counts
    out["hist"] = b.history_rows()
    out["start"] = start
    assert b.check() == abi.OK
    b.close()
    return out


def test_mixed_initial_state_matches_fp64():
    cfg, dt, _, _ = cases.make("rel_const")
    m = _run(cfg, dt, 0, abi.MIXED)
    f = _run(cfg, dt, 0, abi.FP64)
    for k in ("x", "y", "z"):
        assert rel_l2(m["p"][k], f["p"][k]) < 1e-7
    for k in ("vx", "vy", "vz", "gamma"):
        assert rel_l2(m["p"][k], f["p"][k]) < 1e-7
    for i in (abi.EX, abi.BZ):
        assert rel_l2(m[i], f[i]) < 1e-7


def test_mixed_stable_case_within_fp32_tolerance():
    cfg, dt, steps, _ = cases.make("reflect_ext")
    m = _run(cfg, dt, steps, abi.MIXED)
    f = _run(cfg, dt, steps, abi.FP64)
    np.testing.assert_array_equal(m["counts"], f["counts"])
    for i in (abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ, abi.JX, abi.RHO):
        assert rel_l2(m[i], f[i]) <= MIXED_RTOL, (abi.FIELD_NAMES[i], rel_l2(m[i], f[i]))
    np.testing.assert_allclose(m["hist"][:, 4:], f["hist"][:, 4:], rtol=1e-6)


def _one_step_rounding(cfg, dt, start_fields):
    """The mixed form's rounding in one step: RMS relative velocity difference
    against the FP64 form from the same particles and fields, times sqrt(3)
    (the amplitude of uniform noise with that RMS), at least 2^-24."""
    f = _run(cfg, dt, 1, abi.FP64)
    m = _run(cfg, dt, 1, abi.MIXED, start_fields=start_fields)
    vf = np.stack([f["p"][k] for k in ("vx", "vy", "vz")], axis=1)
    vm = np.stack([m["p"][k] for k in ("vx", "vy", "vz")], axis=1)
    nf = np.linalg.norm(vf, axis=1)
    r = np.linalg.norm(vm - vf, axis=1)[nf > 0] / nf[nf > 0]
    return max(FP32_ROUNDING, float(np.sqrt(3.0 * np.mean(r * r))))


@pytest.mark.parametrize("name", ["periodic_poisson", "aniso_const", "sorted_test"])
def test_mixed_error_within_its_rounding_spread(name):
    """On the golden cases (reference policy, 8-12 steps), started from the
    FP64 form's field start, the mixed form's distance from the FP64 form is
    at most ENSEMBLE_FACTOR times the largest distance of FP64 runs perturbed
    after every step by the mixed form's own one-step rounding (measured, a
    few FP32 ulps): on these small cases a few particles that end a step
    within rounding of a cell face, where the reference's gather jumps,
    decide the distance, so the largest member is the yardstick. (Each
    form's own Jacobi start on a periodic grid drifts in
    the potential's mean, by an amount set by its deposit's rounding, which
    AToB turns into a uniform B: a difference of the field start, stated
    apart, not of the loop.)"""
    cfg, dt, steps, _ = cases.make(name)
    f = _run(cfg, dt, steps, abi.FP64)
    m = _run(cfg, dt, steps, abi.MIXED, start_fields=f["start"])
    rel = _one_step_rounding(cfg, dt, f["start"])
    assert rel < 1e-5, rel
    ens = [_run(cfg, dt, steps, abi.FP64, perturb_seed=k + 1, rel=rel) for k in range(ENSEMBLE_MEMBERS)]
    phys = tuple(slice(1, v + 1) for v in cfg.n)
    for i in (abi.EX, abi.BY, abi.JX):
        err = rel_l2(m[i][phys], f[i][phys])
        spread = [rel_l2(e[i][phys], f[i][phys]) for e in ens]
        assert err <= ENSEMBLE_FACTOR * max(spread), (abi.FIELD_NAMES[i], err, spread, rel)


def test_mixed_divergence_starts_at_a_cell_face():
    """The reference's gather is discontinuous across cell faces (its vertex
    carries the ghost offset, so the weights jump from (1, 0) to (2, -1) at a
    face). A particle that ends a step within an FP32 offset ulp of a face can
    sit on different sides of it in the two forms, and its force then differs
    by O(1). In this seeded case that happens at step 7: the first particle
    whose velocity departs by more than 1e-4 was within 2^-22 cells of a face
    before that step, and every particle agreed to 1e-6 until then."""
    cfg, dt, steps, _ = cases.make("rel_const")
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    bs = []
    for prec in (abi.MIXED, abi.FP64):
        b = GpuBackend(info, dt, precision=prec)
        _load(b, parts)
        b.init_fields()
        bs.append(b)
    m, f = bs
    found = False
    for ti in range(steps):
        before = by_id(f.particles())
        bm = by_id(m.particles())
        m.step(1)
        f.step(1)
        pm, pf = by_id(m.particles()), by_id(f.particles())
        dv = sum(np.abs(pm[k] - pf[k]) for k in ("vx", "vy", "vz"))
        if dv.max() > 1e-4:
            k = int(np.argmax(dv))
            near = min(min(abs(before[c][k] - round(before[c][k])), abs(bm[c][k] - round(bm[c][k])))
                       for c in ("x", "y", "z"))
            assert near < 2.0 ** -22, near
            found = True
            break
        assert dv.max() < 1e-6
    assert found
    for b in bs:
        b.close()


def test_mixed_runs_are_bit_reproducible():
    cfg = configs.tiny("repro", n=(10, 8, 6), ppc=6, relativity=1, init="constant", B0=(0.0, 0.05, 0.0),
                       nstep_sort=4)
    a = _run(cfg, 0.45, 9, abi.MIXED)
    b = _run(cfg, 0.45, 9, abi.MIXED)
    for i in (abi.EX, abi.BY, abi.JX, abi.RHO):
        np.testing.assert_array_equal(a[i], b[i])
    for k in ("x", "vx"):
        np.testing.assert_array_equal(a["p"][k], b["p"][k])


def test_mixed_sort_keeps_particles_and_orders_cells():
    cfg = configs.tiny("msort", n=(9, 7, 5), ppc=7, relativity=1, init="constant", test_species=True)
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    b = GpuBackend(info, 0.4, precision=abi.MIXED)
    _load(b, parts)
    b.step(2)
    before = by_id(b.particles())
    b.sort()
    after = b.particles()
    assert len(after["id"]) == len(before["id"])
    for s in range(len(cfg.species)):
        sel = after["type"] == s
        keys = np.array([b.cell_id(x, y, z) for x, y, z in zip(after["x"][sel], after["y"][sel], after["z"][sel])])
        assert np.all(np.diff(keys) >= 0)
    a = by_id(after)
    for k in ("x", "vx"):
        np.testing.assert_array_equal(a[k], before[k])
    b.step(3)
    assert b.check() == abi.OK
    b.close()


def test_mixed_device_loader_and_readback():
    cfg = configs.tiny("mload", n=(12, 10, 8), ppc=4, relativity=1, init="constant", vth=0.2)
    info = configs.input_info(cfg)
    import ctypes as C

    b = GpuBackend(info, 0.4, precision=abi.MIXED)
    for si in range(len(cfg.species)):
        g = configs.gen_params(cfg, si)
        abi.check(b.L.emoo_load_generated(b.h, C.byref(g), cfg.count(cfg.species[si])))
    p = b.particles()
    for si in range(len(cfg.species)):
        host = loading.sample_species(cfg, si)
        sel = p["type"] == si
        np.testing.assert_allclose(p["x"][sel], host["x"], rtol=0, atol=1e-6)
        np.testing.assert_allclose(p["vx"][sel], host["vx"], rtol=1e-7, atol=1e-12)
        np.testing.assert_allclose(p["gamma"][sel], host["gamma"], rtol=1e-7)
    b.close()


@pytest.mark.parametrize("policy", [abi.POLICY_REFERENCE, abi.POLICY_CORRECTED])
def test_mixed_interpolate_matches_fp64(policy):
    """emoo_interpolate (Particle_Handler::InterpolateEB) in the mixed form:
    each particle's E and B from the interpolation pack against the FP64
    form's gather, after the field start (FP32 fields and offsets). Both
    start from the multigrid solve: the reference's periodic Jacobi drifts in
    the potentials' mean by J's mean per sweep, AToB (which takes Bx from Az
    and Ay together) turns that into a uniform B offset, and the two forms'
    deposits leave J means that differ at rounding level."""
    cfg, dt, _, _ = cases.make("periodic_poisson")
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    out = {}
    for prec in (abi.FP64, abi.MIXED):
        b = GpuBackend(info, dt, precision=prec, policy=policy, poisson_solver=abi.POISSON_MULTIGRID,
                       poisson_rtol=1e-12)
        _load(b, parts)
        b.init_fields()
        abi.check(b.L.emoo_interpolate(b.h), "emoo_interpolate")
        out[prec] = (b.particle_fields(), b.particles()["id"])  # both in device (load) order
        b.close()
    (ff, idf), (fm, idm) = out[abi.FP64], out[abi.MIXED]
    np.testing.assert_array_equal(idf, idm)
    for q in range(6):
        assert rel_l2(fm[:, q], ff[:, q]) <= 1e-5, (q, rel_l2(fm[:, q], ff[:, q]))


@pytest.mark.parametrize("name", ["reflect_ext", "periodic_poisson"])
def test_mixed_unfused_sequence_equals_the_fused_step(name):
    """The mixed form's unfused call sequence - emoo_interpolate
    (InterpolateEB), emoo_push (Push), emoo_apply_particle_bc (the six sides)
    - moves every particle exactly as one fused emoo_step does (no sort in
    that step), with the same crossing counts."""
    cfg, dt, _, _ = cases.make(name)
    cfg.nstep_sort = 0
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    a = GpuBackend(info, dt, precision=abi.MIXED)
    b = GpuBackend(info, dt, precision=abi.MIXED)
    for g in (a, b):
        _load(g, parts)
        g.init_fields()
    a.interpolate()
    a.push()
    ca = a.particle_bc()
    cb = b.step(1)
    assert list(ca) == list(cb)
    pa, pb = by_id(a.particles()), by_id(b.particles())
    for k in ("x", "y", "z", "vx", "vy", "vz", "gamma"):
        np.testing.assert_array_equal(pa[k], pb[k], err_msg=k)
    a.close()
    b.close()
