"""Differentiation of the FP64 loop under the corrected policy (emoo_ad_run
with POLICY_CORRECTED; no reference counterpart).

The corrected step's transposes: the charge-conserving current of each move
(ad_math.cuh vb_eval / vb_rev) and its exit piece at absorbing walls, the
whole-range periodic folds and ghost copies, the mirror fold at reflecting
walls, and the plane sets between the Yee halves and after them. Cases: the
small laser case of tests/test_gpu_adjoint.py with reflecting, absorbing
and mixed (reflecting left, absorbing right) x walls, and a fully periodic
thermal box differentiated with respect to the particle velocities.

  * the adjoint gradient is the transpose of the tangent (dot-product test);
  * the tangent equals central finite differences of the primal objective;
  * each wave parameter's adjoint derivative equals its central difference;
  * the checkpoint spacing does not change the gradient;
  * the primal objective run equals the handle's own emoo_step loop;
  * the mixed form's adjoint (FP32) gives the FP64 form's gradients to FP32
    accuracy, on the small laser case with each kind of wall and on the
    scaled laser-plasma workload (absorbing walls, shaped pulse).
As for the reference policy, cells and boundary events are held at the
primal run's; the perturbations are small enough that none changes between
the finite-difference evaluations at these sizes."""
import dataclasses

import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs
from apc_524_project_gb300.differentiate import Problem

pytestmark = pytest.mark.gpu

FD_RTOL = 1e-5
DOT_RTOL = 1e-9


def fd_rounding(objective, h):
    """The central difference's own rounding: the two objectives carry a
    few ulps of rounding each (the FP64 deposit's atomics sum in a varying
    order), divided by 2h. It matters only where the derivative is tiny."""
    return 8 * np.finfo(float).eps * abs(objective) / h


WALLS = {
    "reflecting": ("reflecting", "reflecting"),
    "absorbing": ("absorbing", "absorbing"),
    "mixed": ("reflecting", "absorbing"),
}


def _laser(walls="reflecting", every=4):
    cfg = configs.laser64(n=(16, 8, 8), steps=24, ppc=2, wavelength=8.0, fwhm_steps=8)
    cfg = dataclasses.replace(cfg, part_bc=WALLS[walls] + ("periodic",) * 4)
    return Problem(cfg, nsteps=24, slab=(2, 8), checkpoint_every=every, policy=abi.POLICY_CORRECTED)


def _thermal(every=5):
    cfg = configs.tiny("adj_periodic", n=(8, 6, 5), dx=(0.9, 1.1, 0.8), relativity=1, init="constant", vth=0.2,
                       steps=15, dt=0.3)
    return Problem(cfg, nsteps=15, slab=(1, 6), checkpoint_every=every, policy=abi.POLICY_CORRECTED)


def _direction(P, seed, with_theta=True, vscale=1e-3):
    rng = np.random.default_rng(seed)
    dth = rng.uniform(-1, 1, P.theta0.shape) if with_theta else np.zeros(P.theta0.shape)
    if with_theta and dth.size:
        dth[1::2] *= 10.0  # phase in degrees
    ddv = vscale * rng.uniform(-1, 1, (3, P.np))
    return dth, ddv


def _dot(P, seed, with_theta=True):
    g = P.gradient()
    dth, ddv = _direction(P, seed, with_theta)
    t = P.tangent(dth, ddv)
    assert np.isclose(t["objective"], g["objective"], rtol=1e-12)
    adj = float(np.dot(g["grad_theta"], dth) + np.sum(g["grad_v"] * ddv))
    assert abs(adj - t["tangent"]) <= DOT_RTOL * abs(t["tangent"]), (adj, t["tangent"])


def _fd(P, seed, with_theta=True):
    dth, ddv = _direction(P, seed, with_theta)
    t = P.tangent(dth, ddv)["tangent"]
    h = 1e-6
    lp = P.objective(P.theta0 + h * dth, h * ddv)
    lm = P.objective(P.theta0 - h * dth, -h * ddv)
    fd = (lp - lm) / (2 * h)
    assert abs(fd - t) <= FD_RTOL * abs(t) + fd_rounding(lp, h), (fd, t)


@pytest.mark.parametrize("walls", sorted(WALLS))
def test_adjoint_is_transpose_of_tangent(walls):
    P = _laser(walls)
    for seed in (1, 2):
        _dot(P, seed)


@pytest.mark.parametrize("walls", sorted(WALLS))
@pytest.mark.parametrize("with_theta", [True, False])
def test_tangent_matches_central_differences(walls, with_theta):
    _fd(_laser(walls), 3, with_theta)


@pytest.mark.parametrize("walls", sorted(WALLS))
def test_wave_gradient_matches_central_differences(walls):
    P = _laser(walls)
    g = P.gradient()["grad_theta"]
    for k, step in ((0, 1e-6), (1, 1e-4)):  # amplitude, phase (degrees)
        th = P.theta0.copy()
        th[k] += step
        lp = P.objective(th)
        th[k] -= 2 * step
        lm = P.objective(th)
        fd = (lp - lm) / (2 * step)
        assert abs(fd - g[k]) <= FD_RTOL * abs(g[k]), (k, fd, g[k])


def test_periodic_box_velocity_gradient():
    P = _thermal()
    _dot(P, 4, with_theta=False)
    _fd(P, 5, with_theta=False)


def test_absorbing_walls_remove_particles_in_the_differentiated_run():
    """The absorbing case differentiates through removals: some particles
    leave through the walls within the 24 steps."""
    from backends import GpuBackend

    P = _laser("absorbing")
    g = GpuBackend(configs.input_info(P.cfg), P.cfg.dt, policy=abi.POLICY_CORRECTED)
    for si, p in enumerate(P.parts):
        g.add_species(si, p)
    g.init_fields()
    c = np.array(g.step(P.nsteps))
    g.close()
    assert c[0] + c[1] > 0, c


@pytest.mark.parametrize("case", ["reflecting", "periodic"])
def test_checkpoint_spacing_does_not_change_the_gradient(case):
    if case == "periodic":
        a, b = _thermal(every=5).gradient(), _thermal(every=15).gradient()
    else:
        a, b = _laser(every=4).gradient(), _laser(every=24).gradient()
    if a["grad_theta"].size:
        np.testing.assert_allclose(a["grad_theta"], b["grad_theta"], rtol=1e-10)
    scale = np.abs(b["grad_v"]).max()
    assert scale > 0
    assert np.abs(a["grad_v"] - b["grad_v"]).max() <= 1e-10 * scale


def test_primal_run_is_the_time_loop():
    """emoo_ad_run's primal steps are emoo_step's corrected steps."""
    from backends import GpuBackend

    P = _laser()
    obj = P.objective()
    g = GpuBackend(configs.input_info(P.cfg), P.cfg.dt, policy=abi.POLICY_CORRECTED)
    nid = 0
    for si, p in enumerate(P.parts):
        g.add_species(si, p, ids=np.arange(nid, nid + len(p["x"])))
        nid += len(p["x"])
    g.init_fields()
    g.step(P.nsteps)
    lo, hi = P.slab[0] + 1, P.slab[1] + 1
    n = P.cfg.n
    e = 0.0
    for fid in (abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ):
        f = g.get_field(fid)[lo:hi, 1:n[1] + 1, 1:n[2] + 1]
        e += float(np.sum(f * f))
    vol = P.cfg.dx[0] * P.cfg.dx[1] * P.cfg.dx[2]
    g.close()
    assert abs(0.5 * vol * e - obj) <= 1e-12 * obj


# ---- the mixed-precision adjoint under the corrected policy -------------------

MIXED_GRAD_RTOL = 2e-3  # mixed-form gradient against the FP64 form's (FP32 forward and adjoint)


def _small_laser_plasma(steps=30):
    """The laser-plasma workload scaled down (40 x 16^2 cells, absorbing x
    walls, shaped pulse with a 16-coefficient envelope, plasma from x = 8)."""
    return configs.laser512(n=(40, 16, 16), steps=steps, ppc=2, wavelength=8.0, fwhm_steps=6, waist=5.0,
                            plasma_x0=8.0, vth=0.02, seed=11)


@pytest.mark.parametrize("objective", ["kinetic", "field"])
def test_mixed_adjoint_matches_fp64_gradient(objective):
    """The mixed form's run (FP32 state, checkpoints and adjoint) under the
    corrected policy gives the FP64 form's objective and gradients to FP32
    accuracy on the small laser-plasma case, and recomputes every step's
    cells exactly."""
    cfg = _small_laser_plasma()
    kw = dict(nsteps=30, slab=(8, 16), checkpoint_every=6, objective=objective, species=0,
              policy=abi.POLICY_CORRECTED)
    f = Problem(cfg, **kw).gradient()
    m = Problem(cfg, precision=abi.MIXED, **kw).gradient()
    assert m["cell_mismatch"] == 0
    assert abs(m["objective"] - f["objective"]) <= 1e-4 * abs(f["objective"])
    gf, gm = f["grad_theta"], m["grad_theta"]
    err = np.linalg.norm(gm - gf) / np.linalg.norm(gf)
    assert err <= MIXED_GRAD_RTOL, (err, gf[:6], gm[:6])
    vf, vm = f["grad_v"], m["grad_v"]
    assert np.linalg.norm(vm - vf) / np.linalg.norm(vf) <= 10 * MIXED_GRAD_RTOL


@pytest.mark.parametrize("walls", sorted(WALLS))
def test_mixed_adjoint_matches_fp64_on_the_laser_case(walls):
    """The small laser case with each kind of wall: the mixed form's wave and
    velocity gradients against the FP64 form's."""
    P = _laser(walls)
    f = P.gradient()
    m = Problem(P.cfg, nsteps=24, slab=(2, 8), checkpoint_every=4, policy=abi.POLICY_CORRECTED,
                precision=abi.MIXED, parts=P.parts).gradient()
    assert m["cell_mismatch"] == 0
    assert abs(m["objective"] - f["objective"]) <= 1e-4 * abs(f["objective"])
    gf, gm = f["grad_theta"], m["grad_theta"]
    assert np.linalg.norm(gm - gf) / np.linalg.norm(gf) <= MIXED_GRAD_RTOL, (gf, gm)
    vf, vm = f["grad_v"], m["grad_v"]
    assert np.linalg.norm(vm - vf) / np.linalg.norm(vf) <= 10 * MIXED_GRAD_RTOL


def test_mixed_adjoint_checkpoint_spacing():
    cfg = _small_laser_plasma()
    kw = dict(nsteps=30, slab=(8, 16), objective="kinetic", species=0, policy=abi.POLICY_CORRECTED,
              precision=abi.MIXED)
    a = Problem(cfg, checkpoint_every=5, **kw).gradient()
    b = Problem(cfg, checkpoint_every=30, **kw).gradient()
    # same forward and reverse arithmetic; only the FP32 atomics' order differs
    assert np.linalg.norm(a["grad_theta"] - b["grad_theta"]) <= 1e-4 * np.linalg.norm(b["grad_theta"])
