"""Known answers of the loop's physics, the kind the reference's unit tests
check (test/test_src/oGrid_unittests.cc:130-193 for the Yee plane wave,
test/test_src/particles_unittests.cc:34-84 for gyration and the light-speed
bound), stated here from the discrete equations themselves:

* Yee plane wave: Ey = sin(k x - w t), Bz in step, propagating along x in a
  periodic vacuum box; the discrete dispersion sin(w dt / 2) = (dt / dx)
  sin(k dx / 2) fixes w, and with B started half a step ahead of E the
  update reproduces the travelling wave to rounding (the reference's own
  test allows 7e-2 with a continuum w). This holds for the corrected
  policy only: the reference's update reads a stale E ghost at the periodic
  wrap (src/grid/oGrid.cpp:15-66 refreshes none between its two halves),
  which breaks the time centring there.
* Boris gyration in a uniform B: each step rotates v by
  theta = 2 atan(q_p |B|) about B, |v| is kept, and the positions are the
  vertices of a polygon inscribed in the circle of radius
  R = dt |v| / (2 sin(theta / 2)).
* The relativistic (Vay) pusher in a strong E: the speed approaches c = 1
  from below and never reaches it."""
import math

import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs
from backends import OracleBackend

UNIT_ACC = 0.58668774  # src/globals.hpp:12


def _plane_wave_fields(n, dx, dt, kmode):
    k = 2.0 * math.pi * kmode / (n[0] * dx[0])
    w = 2.0 / dt * math.asin(dt / dx[0] * math.sin(k * dx[0] / 2.0))
    shape = tuple(v + 3 for v in n)
    ey = np.zeros(shape)
    bz = np.zeros(shape)
    for i in range(n[0] + 3):
        ey[i, :, :] = math.sin(k * i * dx[0])                      # Ey at x_i, t = 0
        bz[i, :, :] = math.sin(k * (i + 0.5) * dx[0] - w * dt / 2)  # Bz at x_{i+1/2}, t = +dt/2
    return k, w, ey, bz


def _wave_case():
    n, dx, dt = (32, 4, 4), (1.0, 1.0, 1.0), 0.5
    cfg = configs.tiny("wave", n=n, dx=dx, init="constant", steps=40, dt=dt)
    return cfg, n, dx, dt


def _run_wave(b, cfg, n, dx, dt, step):
    k, w, ey, bz = _plane_wave_fields(n, dx, dt, 2)
    b.set_field(abi.EY, ey)
    b.set_field(abi.BZ, bz)
    b.execute_bc(abi.SEND_EB)
    for s in range(cfg.steps):
        step(s)
    got = b.get_field(abi.EY)[1:n[0] + 1, 2, 2]
    x = np.arange(1, n[0] + 1) * dx[0]
    want = np.sin(k * x - w * cfg.steps * dt)
    return np.abs(got - want).max()


def test_oracle_yee_plane_wave_follows_the_discrete_dispersion():
    cfg, n, dx, dt = _wave_case()
    o = OracleBackend(configs.input_info(cfg), dt)
    o.set_policy(abi.POLICY_CORRECTED)
    o.set_time(0.0, dt)
    assert _run_wave(o, cfg, n, dx, dt, o.step) <= 1e-12
    o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_gpu_yee_plane_wave_follows_the_discrete_dispersion(precision):
    from backends import GpuBackend

    cfg, n, dx, dt = _wave_case()
    g = GpuBackend(configs.input_info(cfg), dt, precision=precision, capacity=1,
                   policy=abi.POLICY_CORRECTED)
    err = _run_wave(g, cfg, n, dx, dt, lambda s: g.step(1))
    assert err <= (1e-12 if precision == abi.FP64 else 1e-5), err
    g.close()


def _gyration_case():
    q, m, dt, b = -1.0, 1.0, 0.05, 0.8
    qp = (0.5 * dt * q) / m * UNIT_ACC
    theta = 2.0 * math.atan(abs(qp) * b)
    return q, m, dt, b, theta


def test_oracle_boris_gyration_radius_and_speed():
    q, m, dt, b, theta = _gyration_case()
    v0 = np.array([0.03, 0.01, 0.0])
    state = np.array([0.0, 0.0, 0.0, *v0, 0.0, q, m])
    field = np.array([0.0, 0.0, 0.0, 0.0, 0.0, b])
    pts = []
    s = state
    for _ in range(40):
        s = OracleBackend.pusher_steps(0, s, field, dt, 1)
        pts.append(s[:2].copy())
    pts = np.array(pts)
    speed = np.linalg.norm(s[3:6])
    assert abs(speed - np.linalg.norm(v0)) <= 1e-14
    R = dt * np.linalg.norm(v0) / (2.0 * math.sin(theta / 2.0))
    # the circle through the points: least-squares centre, then every radius
    A = np.c_[2 * pts, np.ones(len(pts))]
    cx, cy, _ = np.linalg.lstsq(A, (pts ** 2).sum(1), rcond=None)[0]
    radii = np.hypot(pts[:, 0] - cx, pts[:, 1] - cy)
    assert np.abs(radii - R).max() <= 1e-10 * R
    # the velocity turned by 40 theta about z (the sense set by the sign of q B)
    ang = math.atan2(s[4], s[3]) - math.atan2(v0[1], v0[0])
    turn = (ang - 40 * theta * np.sign(-q * b) + math.pi) % (2 * math.pi) - math.pi
    assert abs(turn) <= 1e-10


def test_oracle_relativistic_speed_stays_below_c():
    state = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, -1.0, 1.0])
    field = np.array([5.0, 0.0, 0.0, 0.0, 0.0, 0.0])
    s = OracleBackend.pusher_steps(1, state, field, 0.5, 400)
    v = np.linalg.norm(s[3:6])
    assert 0.999 < v < 1.0
