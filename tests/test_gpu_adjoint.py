"""Differentiation of the FP64 loop (emoo_ad_run) on a small laser case: a
wave injected at x-left into a plasma with reflecting x walls, objective the
field energy of an x slab after 24 steps.

  * the adjoint gradient is the transpose of the tangent-linear derivative:
    <grad, d> equals the tangent along d (dot-product test);
  * the tangent equals central finite differences of the primal objective
    (FD_RTOL), for a direction over all parameters and over the velocities
    alone;
  * each wave parameter's adjoint derivative equals its central difference;
  * the primal objective run equals the handle's own emoo_step loop.
The step is differentiated with the particles' cells and boundary events
held fixed; the perturbations are small enough that no particle changes
cell or boundary event between the FD evaluations at these sizes."""
import numpy as np
import pytest

from apc_524_project_gb300 import configs
from apc_524_project_gb300.differentiate import Problem

pytestmark = pytest.mark.gpu

FD_RTOL = 1e-5      # tangent / adjoint against central differences
DOT_RTOL = 1e-9     # adjoint against tangent (same discrete derivative)


def fd_rounding(objective, h):
    """The central difference's own rounding: the two objectives carry a
    few ulps of rounding each (the FP64 deposit's atomics sum in a varying
    order), divided by 2h. It matters only where the derivative is tiny."""
    return 8 * np.finfo(float).eps * abs(objective) / h


def _problem(every=4):
    cfg = configs.laser64(n=(16, 8, 8), steps=24, ppc=2, wavelength=8.0, fwhm_steps=8)
    return Problem(cfg, nsteps=24, slab=(2, 8), checkpoint_every=every)


def _direction(P, seed, with_theta=True, vscale=1e-3):
    rng = np.random.default_rng(seed)
    dth = rng.uniform(-1, 1, P.theta0.shape) if with_theta else np.zeros(P.theta0.shape)
    if with_theta:
        dth[1::2] *= 10.0  # phase in degrees
    ddv = vscale * rng.uniform(-1, 1, (3, P.np))
    return dth, ddv


def test_objective_depends_on_the_wave():
    P = _problem()
    base = P.objective()
    assert base > 0
    th = P.theta0.copy()
    th[0] *= 0.5
    assert abs(P.objective(th) - base) > 1e-3 * base


def test_adjoint_is_transpose_of_tangent():
    P = _problem()
    g = P.gradient()
    for seed in (1, 2):
        dth, ddv = _direction(P, seed)
        t = P.tangent(dth, ddv)
        assert np.isclose(t["objective"], g["objective"], rtol=1e-12)
        adj = float(np.dot(g["grad_theta"], dth) + np.sum(g["grad_v"] * ddv))
        assert abs(adj - t["tangent"]) <= DOT_RTOL * abs(t["tangent"]), (adj, t["tangent"])


@pytest.mark.parametrize("with_theta", [True, False])
def test_tangent_matches_central_differences(with_theta):
    P = _problem()
    dth, ddv = _direction(P, 3, with_theta)
    t = P.tangent(dth, ddv)["tangent"]
    h = 1e-6
    lp = P.objective(P.theta0 + h * dth, h * ddv)
    lm = P.objective(P.theta0 - h * dth, -h * ddv)
    fd = (lp - lm) / (2 * h)
    assert abs(fd - t) <= FD_RTOL * abs(t) + fd_rounding(lp, h), (fd, t)


def test_wave_gradient_matches_central_differences():
    P = _problem()
    g = P.gradient()["grad_theta"]
    for k, step in ((0, 1e-6), (1, 1e-4)):  # amplitude, phase (degrees)
        th = P.theta0.copy()
        th[k] += step
        lp = P.objective(th)
        th[k] -= 2 * step
        lm = P.objective(th)
        fd = (lp - lm) / (2 * step)
        assert abs(fd - g[k]) <= FD_RTOL * abs(g[k]), (k, fd, g[k])


def test_checkpoint_spacing_does_not_change_the_gradient():
    a = _problem(every=4).gradient()
    b = _problem(every=24).gradient()
    np.testing.assert_allclose(a["grad_theta"], b["grad_theta"], rtol=1e-10)
    scale = np.abs(b["grad_v"]).max()
    assert np.abs(a["grad_v"] - b["grad_v"]).max() <= 1e-10 * scale


def test_primal_run_is_the_time_loop():
    """emoo_ad_run's primal steps are emoo_step's steps (no sort here)."""
    from apc_524_project_gb300 import abi
    from backends import GpuBackend

    P = _problem()
    obj = P.objective()
    g = GpuBackend(configs.input_info(P.cfg), P.cfg.dt)
    nid = 0
    for si, p in enumerate(P.parts):
        g.add_species(si, p, ids=np.arange(nid, nid + len(p["x"])))
        nid += len(p["x"])
    g.init_fields()
    g.step(P.nsteps)
    lo, hi = P.slab[0] + 1, P.slab[1] + 1
    n = P.cfg.n
    e = 0.0
    # after an even number of steps the B role is the B slot
    for fid in (abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ):
        f = g.get_field(fid)[lo:hi, 1:n[1] + 1, 1:n[2] + 1]
        e += float(np.sum(f * f))
    vol = P.cfg.dx[0] * P.cfg.dx[1] * P.cfg.dx[2]
    g.close()
    assert abs(0.5 * vol * e - obj) <= 1e-12 * obj


@pytest.mark.parametrize("policy", ["reference", "corrected"])
def test_every_particle_gets_its_gradient(policy):
    """More particles than one thread per particle of a capped grid would
    reach (2,654,208 > 152 x 64 x 256): with the kinetic energy of all
    particles as the objective, every particle's velocity gradient is
    nonzero, the last loaded ones included, and a velocity-direction tangent
    equals the adjoint's inner product."""
    from apc_524_project_gb300 import abi

    cfg = configs.tiny("many", n=(48, 48, 48), ppc=12, relativity=1, init="constant", vth=0.05, steps=2, dt=0.3)
    pol = abi.POLICY_CORRECTED if policy == "corrected" else abi.POLICY_REFERENCE
    P = Problem(cfg, nsteps=2, slab=(0, 48), checkpoint_every=2, objective="kinetic", policy=pol)
    assert P.np > 152 * 64 * 256
    g = P.gradient()
    gv = g["grad_v"]
    assert np.all(np.abs(gv).sum(axis=0) > 0)
    rng = np.random.default_rng(9)
    ddv = 1e-3 * rng.uniform(-1, 1, (3, P.np))
    t = P.tangent(np.zeros(P.theta0.shape), ddv)["tangent"]
    adj = float(np.sum(gv * ddv))
    assert abs(adj - t) <= DOT_RTOL * abs(t), (adj, t)
