"""The corrected-physics policy (no reference counterpart): the cell's own
lower corner as gather / deposit vertex, the Villasenor-Buneman
charge-conserving current, ghost copies and folds over the whole range of
every component; periodic boundaries here (walls: tests/test_corrected_walls.py).

CPU (oracle): the discrete continuity equation rho(t + dt) - rho(t) + dt div J
= 0 holds at every point to rounding, so the Gauss-law residual div E - 4 pi
rho keeps its initial value step after step.
GPU: the FP64 form against the oracle, and the residual's conservation."""
import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading
from backends import OracleBackend, by_id, rel_l2

FP64_RTOL = 1e-9


def _cfg(relativity=1, n=(6, 5, 4), dx=(0.9, 1.2, 0.7), steps=6, vth=0.15, nstep_sort=0):
    return configs.tiny("corr", n=n, dx=dx, relativity=relativity, init="poisson", vth=vth, steps=steps,
                        nstep_sort=nstep_sort, dt=0.3)


def _load(b, parts):
    nid = 0
    for si, p in enumerate(parts):
        b.add_species(si, p, ids=np.arange(nid, nid + len(p["x"])))
        nid += len(p["x"])


def _periodic(f, n):
    """The ghost planes 0 and n+1 set to their periodic images n and 1 (a fold
    leaves J's ghost planes holding their own deposits only)."""
    g = f.copy()
    for d in range(3):
        src, dst = [slice(None)] * 3, [slice(None)] * 3
        src[d], dst[d] = n[d], 0
        g[tuple(dst)] = g[tuple(src)]
        src[d], dst[d] = 1, n[d] + 1
        g[tuple(dst)] = g[tuple(src)]
    return g


def _div(f, dx, n):
    """Backward-difference divergence at the physical points, periodic."""
    Ex, Ey, Ez = (_periodic(a, n) for a in f)
    P = (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))
    return ((Ex[P] - Ex[0:n[0], 1:n[1] + 1, 1:n[2] + 1]) / dx[0] + (Ey[P] - Ey[1:n[0] + 1, 0:n[1], 1:n[2] + 1]) / dx[1]
            + (Ez[P] - Ez[1:n[0] + 1, 1:n[1] + 1, 0:n[2]]) / dx[2])


def _oracle(cfg, policy=1):
    o = OracleBackend(configs.input_info(cfg), cfg.dt)
    o.set_policy(policy)
    _load(o, loading.sample_all(cfg))
    return o


@pytest.mark.parametrize("relativity", [0, 1])
def test_oracle_continuity_and_gauss_law(relativity):
    cfg = _cfg(relativity)
    n = cfg.n
    o = _oracle(cfg)
    o.init_fields()
    P = (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))
    rho0 = o.get_field(abi.RHO)[P].copy()
    res0 = _div([o.get_field(i) for i in (abi.EX, abi.EY, abi.EZ)], cfg.dx, n) - 4 * np.pi * rho0
    scale = np.abs(rho0).max()
    for ti in range(cfg.steps):
        o.step(ti)
        rho1 = o.get_field(abi.RHO)[P]
        divj = _div([o.get_field(i) for i in (abi.JX, abi.JY, abi.JZ)], cfg.dx, n)
        cont = (rho1 - rho0) + cfg.dt * divj
        assert np.abs(cont).max() <= 1e-12 * scale, (ti, np.abs(cont).max(), scale)
        rho0 = rho1.copy()
    res = _div([o.get_field(i) for i in (abi.EX, abi.EY, abi.EZ)], cfg.dx, n) - 4 * np.pi * rho0
    assert np.abs(res - res0).max() <= 1e-10 * 4 * np.pi * scale
    o.close()


def test_reference_policy_does_not_conserve_charge():
    """The reference's deposit (ghost-offset vertex, current at the new
    position) breaks the continuity equation: what the corrected policy fixes."""
    cfg = _cfg(1)
    n = cfg.n
    o = _oracle(cfg, policy=0)
    o.init_fields()
    P = (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))
    rho0 = o.get_field(abi.RHO)[P].copy()
    o.step(0)
    rho1 = o.get_field(abi.RHO)[P]
    divj = _div([o.get_field(i) for i in (abi.JX, abi.JY, abi.JZ)], cfg.dx, n)
    assert np.abs(rho1 - rho0 + cfg.dt * divj).max() > 1e-3 * np.abs(rho0).max()
    o.close()


# ---- GPU -------------------------------------------------------------------

def _gpu(cfg, precision=abi.FP64, policy=abi.POLICY_CORRECTED, poisson_solver=abi.POISSON_JACOBI):
    from backends import GpuBackend

    g = GpuBackend(configs.input_info(cfg), cfg.dt, precision=precision, policy=policy, poisson_solver=poisson_solver,
                   poisson_rtol=1e-12)
    _load(g, loading.sample_all(cfg))
    return g


@pytest.mark.gpu
@pytest.mark.parametrize("relativity", [0, 1])
def test_gpu_corrected_policy_matches_oracle(relativity):
    cfg = _cfg(relativity, nstep_sort=3)
    g = _gpu(cfg)
    o = _oracle(cfg)
    rg, _ = g.init_fields()
    ro, _ = o.init_fields()
    assert rg == ro
    for ti in range(cfg.steps):
        assert g.step(1) == o.step(ti)[0], ti
    for i in range(13):
        assert rel_l2(g.get_field(i), o.get_field(i)) <= FP64_RTOL, abi.FIELD_NAMES[i]
    pg, po = by_id(g.particles()), by_id(o.particles())
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert rel_l2(pg[k], po[k]) <= FP64_RTOL, k
    g.close()
    o.close()


@pytest.mark.gpu
def test_gpu_corrected_policy_keeps_gauss_law():
    cfg = _cfg(1, n=(8, 6, 5), steps=10)
    n = cfg.n
    g = _gpu(cfg)
    g.init_fields()
    P = (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))

    def residual():
        return _div([g.get_field(i) for i in (abi.EX, abi.EY, abi.EZ)], cfg.dx, n) - 4 * np.pi * g.get_field(abi.RHO)[P]

    r0 = residual()
    scale = 4 * np.pi * np.abs(g.get_field(abi.RHO)[P]).max()
    g.step(cfg.steps)
    assert np.abs(residual() - r0).max() <= 1e-10 * scale
    g.close()


@pytest.mark.gpu
def test_gpu_corrected_policy_refuses_what_it_does_not_cover():
    """Both forms take the policy; a dimension that is neither periodic
    (particle and field sides) nor walled (reflecting or absorbing particle
    sides, external field sides) is refused, and so is the adjoint run."""
    _gpu(_cfg(1), precision=abi.MIXED).close()  # both forms take it
    half = configs.tiny("half", part_bc=("periodic",) * 6,
                        field_bc=("external", "external", "periodic", "periodic", "periodic", "periodic"),
                        init="constant")
    with pytest.raises(Exception):
        _gpu(half)


@pytest.mark.gpu
@pytest.mark.parametrize("dt,precision", [(0.125, abi.FP64), (0.5, abi.FP64), (0.5, abi.MIXED)])
def test_gpu_corrected_policy_is_stable_where_the_reference_is_not(dt, precision):
    """Thermal plasma 16^3, 2 x 16 ppc, v_th 0.1c, 600 steps: the reference's
    arithmetic heats the plasma (total energy grows several-fold at dt 0.125,
    without bound at dt 0.5); the corrected policy keeps it within a few per
    cent at both, in both forms."""
    from backends import GpuBackend

    cfg = configs.thermal256(16)
    cfg.dt = dt

    def history(policy):
        g = GpuBackend(configs.input_info(cfg), cfg.dt, policy=policy, track_ids=0, precision=precision)
        for si, p in enumerate(loading.sample_all(cfg)):
            g.add_species(si, p)
        g.init_fields()
        g.step(600)
        rows = g.history_rows()
        g.close()
        return rows[:, 7] / rows[0, 7]

    ref, cor = history(abi.POLICY_REFERENCE), history(abi.POLICY_CORRECTED)
    assert not ref[-1] <= 2.0, ref[-1]  # in FP32 the blow-up can overflow to NaN
    assert np.abs(cor - 1.0).max() < 0.1, np.abs(cor - 1.0).max()


def _vacuum(backend_factory, policy, n=12, dt=0.5, steps=400):
    """Field energy after `steps` vacuum steps over its initial value, from
    seeded random E and B (both B roles) on a periodic n^3 grid of unit
    cells. dt 0.5 is inside the 3-D Courant limit 1 / sqrt(3)."""
    cfg = configs.tiny("vacuum", n=(n, n, n), dx=(1.0, 1.0, 1.0), init="constant", steps=steps, dt=dt)
    b = backend_factory(cfg, policy)
    rng = np.random.default_rng(7)
    P = (slice(1, n + 1),) * 3
    for fid in (abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ, abi.BX_TM1, abi.BY_TM1, abi.BZ_TM1):
        f = np.zeros(b.get_field(fid).shape)
        f[P] = rng.normal(0.0, 1e-3, (n, n, n))
        b.set_field(fid, f)
    b.execute_bc(abi.SEND_EB)

    def energy():
        return sum(float(np.sum(b.get_field(i)[P] ** 2)) for i in range(6))

    e0 = energy()
    b.run(steps)
    e1 = energy()
    b.close()
    return e1 / e0


def _oracle_vacuum(cfg, policy):
    o = OracleBackend(configs.input_info(cfg), cfg.dt)
    o.set_policy(policy)
    o.set_time(0.0, cfg.dt)  # the step length the field start leaves

    def run(steps):
        for ti in range(steps):
            o.step(ti)

    o.run = run
    return o


def test_oracle_vacuum_yee_is_time_centred_under_the_corrected_policy():
    """The reference refreshes E's periodic ghosts only after the B half, so
    B at the high faces sees the previous step's E: the leapfrog is not
    time-centred at the wrap and vacuum fields grow without bound at dt 0.5.
    The corrected policy refreshes them between the halves; the energy then
    stays bounded (the discrete Yee energy oscillates, it is not exactly
    E^2 + B^2)."""
    assert _vacuum(_oracle_vacuum, 0) > 1e6
    assert _vacuum(_oracle_vacuum, 1) < 2.0


def _gpu_vacuum(cfg, policy):
    from backends import GpuBackend

    g = GpuBackend(configs.input_info(cfg), cfg.dt, policy=policy, track_ids=0)
    g.run = g.step
    return g


@pytest.mark.gpu
def test_gpu_vacuum_yee_is_time_centred_under_the_corrected_policy():
    ref = _vacuum(_gpu_vacuum, abi.POLICY_REFERENCE)
    cor = _vacuum(_gpu_vacuum, abi.POLICY_CORRECTED)
    assert ref > 1e6, ref
    assert cor < 2.0, cor
    assert abs(cor - _vacuum(_oracle_vacuum, 1)) <= 1e-9 * cor


# ---- the mixed form under the corrected policy ---------------------------------

MIXED_CORR_RTOL = 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("relativity", [0, 1])
def test_gpu_mixed_corrected_policy_matches_fp64(relativity):
    """The mixed form (FP32 positions, momenta and fields, fixed-point J)
    against the FP64 form under the corrected policy: with the continuous
    true-vertex gather there is no face discontinuity to amplify FP32
    rounding, so after 6 steps (a sort every 3) the fields and particles agree
    to FP32 precision and the crossing counts exactly. Both start from the
    multigrid solve: the FP32 deposit leaves rho's mean at FP32 rounding
    rather than zero, and on a periodic grid the reference's Jacobi then
    drifts by that much per sweep and misses its absolute stop test (E is
    unaffected); the multigrid removes the mean."""
    cfg = _cfg(relativity, nstep_sort=3)
    mg = abi.POISSON_MULTIGRID
    g, m = _gpu(cfg, poisson_solver=mg), _gpu(cfg, precision=abi.MIXED, poisson_solver=mg)
    assert g.init_fields()[0] == m.init_fields()[0] == 0
    for ti in range(cfg.steps):
        assert g.step(1) == m.step(1), ti
    n = cfg.n
    P = (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))
    for i in (abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ):
        assert rel_l2(m.get_field(i), g.get_field(i)) <= MIXED_CORR_RTOL, (abi.FIELD_NAMES[i],
                                                                            rel_l2(m.get_field(i), g.get_field(i)))
    # J and rho at the physical points: after the fold the ghost planes hold
    # leftovers nothing reads, and the two forms leave different ones (FP64
    # deposits into unwrapped cells -1..n, the mixed form wraps first)
    for i in (abi.JX, abi.JY, abi.JZ, abi.RHO):
        a, b = m.get_field(i)[P], g.get_field(i)[P]
        assert rel_l2(a, b) <= MIXED_CORR_RTOL, (abi.FIELD_NAMES[i], rel_l2(a, b))
    pg, pm = by_id(g.particles()), by_id(m.particles())
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert rel_l2(pm[k], pg[k]) <= MIXED_CORR_RTOL, k
    g.close()
    m.close()


@pytest.mark.gpu
def test_gpu_mixed_corrected_policy_conserves_charge():
    """The mixed form's FP32 Villasenor-Buneman current: rho(t + dt) - rho(t)
    + dt div J = 0 to FP32 rounding of the path (the fixed-point quantum is
    2^-32 of the largest charge), step after step, crossings included."""
    cfg = _cfg(1, n=(8, 6, 5), steps=8)
    n = cfg.n
    m = _gpu(cfg, precision=abi.MIXED, poisson_solver=abi.POISSON_MULTIGRID)
    assert m.init_fields()[0] == 0
    P = (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))
    rho0 = m.get_field(abi.RHO)[P].copy()
    scale = np.abs(rho0).max()
    crossed = 0
    for ti in range(cfg.steps):
        crossed += sum(m.step(1))
        rho1 = m.get_field(abi.RHO)[P]
        divj = _div([m.get_field(i) for i in (abi.JX, abi.JY, abi.JZ)], cfg.dx, n)
        cont = (rho1 - rho0) + cfg.dt * divj
        assert np.abs(cont).max() <= 1e-5 * scale, (ti, np.abs(cont).max(), scale)
        rho0 = rho1.copy()
    assert crossed > 0
    m.close()


def _full_ghosts(f, n):
    """Periodic ghost planes 0, n+1, n+2 from n, 1, 2, dimension by dimension
    over the whole range (the corrected policy's fill)."""
    for d in range(3):
        def pl(i):
            s = [slice(None)] * 3
            s[d] = i
            return tuple(s)
        f[pl(0)] = f[pl(n[d])]
        f[pl(n[d] + 1)] = f[pl(1)]
        f[pl(n[d] + 2)] = f[pl(2)]


def test_oracle_corrected_yee_matches_an_independent_leapfrog():
    """The oracle's corrected vacuum Yee update against a numpy leapfrog of
    the same stencils (src/grid/oGrid.cpp:15-60, B <-> B_tm1 role swap): E
    from the previous B with backward differences, E's periodic ghosts
    refreshed, then B from the new E with forward differences, all ghosts
    refreshed after the step. 20 steps on an anisotropic grid."""
    n, dx, dt = (6, 5, 4), (0.9, 1.2, 0.7), 0.3
    cfg = configs.tiny("yee", n=n, dx=dx, init="constant", steps=20, dt=dt)
    o = OracleBackend(configs.input_info(cfg), dt)
    o.set_policy(1)
    o.set_time(0.0, dt)
    rng = np.random.default_rng(11)
    P = (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))
    shape = o.get_field(abi.EX).shape
    init = {}
    for fid in (abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ, abi.BX_TM1, abi.BY_TM1, abi.BZ_TM1):
        f = np.zeros(shape)
        f[P] = rng.normal(0.0, 1e-3, n)
        init[fid] = f
        o.set_field(fid, f)
    o.execute_bc(abi.SEND_EB)
    E = [init[f].copy() for f in (abi.EX, abi.EY, abi.EZ)]
    B = [init[f].copy() for f in (abi.BX, abi.BY, abi.BZ)]
    for f in E + B:
        _full_ghosts(f, n)

    def sh(f, d, s):  # f at (index + s) along d, over the physical points
        sl = list(P)
        sl[d] = slice(1 + s, n[d] + 1 + s)
        return f[tuple(sl)]

    for ti in range(cfg.steps):
        T = B
        Ex, Ey, Ez = E
        Tx, Ty, Tz = T
        ex = Ex[P] - dt * ((sh(Ty, 2, 0) - sh(Ty, 2, -1)) / dx[2] - (sh(Tz, 1, 0) - sh(Tz, 1, -1)) / dx[1])
        ey = Ey[P] - dt * ((sh(Tz, 0, 0) - sh(Tz, 0, -1)) / dx[0] - (sh(Tx, 2, 0) - sh(Tx, 2, -1)) / dx[2])
        ez = Ez[P] - dt * ((sh(Tx, 1, 0) - sh(Tx, 1, -1)) / dx[1] - (sh(Ty, 0, 0) - sh(Ty, 0, -1)) / dx[0])
        Ex[P], Ey[P], Ez[P] = ex, ey, ez
        for f in E:
            _full_ghosts(f, n)
        Bn = [np.zeros(shape) for _ in range(3)]
        Bn[0][P] = Tx[P] + dt * ((sh(Ey, 2, 1) - sh(Ey, 2, 0)) / dx[2] - (sh(Ez, 1, 1) - sh(Ez, 1, 0)) / dx[1])
        Bn[1][P] = Ty[P] + dt * ((sh(Ez, 0, 1) - sh(Ez, 0, 0)) / dx[0] - (sh(Ex, 2, 1) - sh(Ex, 2, 0)) / dx[2])
        Bn[2][P] = Tz[P] + dt * ((sh(Ex, 1, 1) - sh(Ex, 1, 0)) / dx[1] - (sh(Ey, 0, 1) - sh(Ey, 0, 0)) / dx[0])
        for f in Bn:
            _full_ghosts(f, n)
        B = Bn
        o.step(ti)
    for c, fid in enumerate((abi.EX, abi.EY, abi.EZ)):
        got = o.get_field(fid)
        assert np.abs(got[P] - E[c][P]).max() <= 1e-12 * np.abs(E[c][P]).max(), abi.FIELD_NAMES[fid]
    o.close()
