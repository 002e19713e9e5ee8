"""The multigrid field start (EMOO_POISSON_MULTIGRID, no reference
counterpart) against the oracle's exact solve of the same discrete system.

The discrete problem is the fixed point of the reference's Jacobi iteration
(src/poisson/poisson.cpp:216-241): at every unknown point the 7-point
Laplacian of phi (A) equals -4 pi rho (J), periodic dimensions wrapping and
external ones holding the PoissonBC planes 1 and n + 1
(src/poisson/poissonBC.cpp:67-80).

CPU: the oracle's conjugate-gradient solve meets those equations to rounding,
agrees with an FFT solution of the periodic problem, and with the reference's
Jacobi result where that iteration converges (an external x dimension);
on a periodic grid with an even side the Jacobi result keeps the
odd-even mode, which the exact solution does not have.
GPU: the multigrid against the oracle on periodic, external and mixed boxes
(odd sides included, which take the Jacobi smoother), the mixed form, the
cycle counts, a 128 x 64 x 64 box against an FFT solution, and the
refusals."""
import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading
from backends import OracleBackend, rel_l2

FOUR_PI = 4.0 * np.pi
P = lambda n: (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))  # noqa: E731


def _box(n, field_bc=("periodic",) * 6, dx=(1.0, 1.0, 1.0), bound_phi=None, bound_A=None):
    part_bc = tuple("periodic" if b == "periodic" else "reflecting" for b in field_bc)
    cfg = configs.tiny("pois", n=n, dx=dx, init="poisson", field_bc=field_bc, part_bc=part_bc)
    if bound_phi is not None:
        cfg.bound_phi = bound_phi
    if bound_A is not None:
        cfg.bound_A = bound_A
    return cfg


def _sources(shape, seed=3):
    """Seeded rho and J (reference units) with a nonzero mean in rho."""
    rng = np.random.default_rng(seed)
    rho = rng.normal(0.0, 1e-3, shape) + 2e-4
    J = [rng.normal(0.0, 5e-4, shape) for _ in range(3)]
    return rho, J


def _set_sources(b, rho, J):
    b.set_field(abi.RHO, rho)
    for q in range(3):
        b.set_field(abi.JX + q, J[q])


def _residual(u, R, cfg):
    """max |Laplacian(u) - (-4 pi R)| over the unknowns, from the slot
    arrays (ghost and boundary planes as the boundary fill left them), and
    the size of the equation's terms there, max |4 pi R| + max |u| 2 sum 1/h^2
    (the rounding scale of the stencil); with every dimension periodic, R
    less its mean (the solvable part)."""
    n = cfg.n
    lo = [1 if cfg.field_bc[2 * d] == "periodic" else 2 for d in range(3)]
    sl = tuple(slice(lo[d], n[d] + 1) for d in range(3))
    if all(b == "periodic" for b in cfg.field_bc):
        R = R - R[sl].mean()
    lap = np.zeros_like(u[sl])
    for d in range(3):
        dn = list(sl)
        up = list(sl)
        dn[d] = slice(lo[d] - 1, n[d])
        up[d] = slice(lo[d] + 1, n[d] + 2)
        lap += (u[tuple(dn)] + u[tuple(up)] - 2.0 * u[sl]) / cfg.dx[d] ** 2
    terms = np.abs(FOUR_PI * R[sl]).max() + np.abs(u).max() * 2.0 * sum(1.0 / h ** 2 for h in cfg.dx)
    return np.abs(lap + FOUR_PI * R[sl]).max(), terms


def _fft_solution(R, cfg):
    """The periodic problem solved by FFT: mean-free right side, mean-free
    solution, over the physical points."""
    n = cfg.n
    f = -FOUR_PI * R[P(n)]
    f = f - f.mean()
    lam = np.zeros(n)
    for d in range(3):
        k = np.arange(n[d])
        ld = (2.0 * np.cos(2.0 * np.pi * k / n[d]) - 2.0) / cfg.dx[d] ** 2
        sh = [1, 1, 1]
        sh[d] = n[d]
        lam = lam + ld.reshape(sh)
    fh = np.fft.fftn(f)
    lam[0, 0, 0] = 1.0
    uh = fh / lam
    uh[0, 0, 0] = 0.0
    return np.real(np.fft.ifftn(uh))


def _oracle(cfg, solver, rtol=1e-13):
    o = OracleBackend(configs.input_info(cfg), 0.4)
    if solver:
        o.set_poisson_solver(1, rtol)
    return o


SLOTS = (abi.PHI1, abi.AX1, abi.AY1, abi.AZ1)
SOURCES = (abi.RHO, abi.JX, abi.JY, abi.JZ)


@pytest.mark.parametrize("bc", ["periodic", "external_x", "external_all"])
def test_oracle_exact_solve_meets_the_discrete_equations(bc):
    fb = {"periodic": ("periodic",) * 6,
          "external_x": ("external", "external") + ("periodic",) * 4,
          "external_all": ("external",) * 6}[bc]
    cfg = _box((8, 6, 5), fb, dx=(1.0, 0.5, 2.0), bound_phi=(0.1, -0.2, 0.05, 0.0, 0.3, 0.1),
               bound_A=((0.0, 0.2, 0.0, 0.0, 0.0, 0.0), (0.0,) * 6, (0.1,) * 6))
    o = _oracle(cfg, 1)
    shape = o.get_field(abi.RHO).shape
    rho, J = _sources(shape)
    if bc != "periodic":
        rho = rho - 2e-4
    _set_sources(o, rho, J)
    rc, it = o.initialize_fields_only()
    assert rc == 0, rc
    for s, r in zip(SLOTS, SOURCES):
        res, scale = _residual(o.get_field(s), o.get_field(r), cfg)
        assert res <= 1e-11 * scale, (abi.FIELD_NAMES[s], res, scale)
    np.testing.assert_array_equal(o.get_field(abi.PHI1), o.get_field(abi.PHI2))
    o.close()


def test_oracle_exact_solve_without_unknowns():
    """An external dimension of one cell leaves no unknown point: the
    potentials are the PoissonBC planes (E itself is then rewritten by the
    external-field fill, plane 1 being a boundary plane too)."""
    fb = ("external", "external") + ("periodic",) * 4
    cfg = _box((1, 6, 4), fb, bound_phi=(0.1, -0.2, 0.0, 0.0, 0.0, 0.0))
    o = _oracle(cfg, 1)
    rho, J = _sources(o.get_field(abi.RHO).shape)
    _set_sources(o, rho, J)
    rc, it = o.initialize_fields_only()
    assert rc == 0 and it == [0, 0, 0, 0]
    phi = o.get_field(abi.PHI1)
    assert np.all(phi[1] == 0.1) and np.all(phi[2] == -0.2)
    np.testing.assert_array_equal(o.get_field(abi.PHI2), phi)
    o.close()


def test_oracle_exact_solve_matches_fft_on_a_periodic_box():
    cfg = _box((8, 6, 10), dx=(1.0, 0.5, 2.0))
    o = _oracle(cfg, 1)
    rho, J = _sources(o.get_field(abi.RHO).shape)
    _set_sources(o, rho, J)
    assert o.initialize_fields_only()[0] == 0
    for s, r in zip(SLOTS, SOURCES):
        want = _fft_solution(o.get_field(r), cfg)
        got = o.get_field(s)[P(cfg.n)]
        assert np.abs(got - want).max() <= 1e-11 * np.abs(want).max(), abi.FIELD_NAMES[s]
    o.close()


def test_oracle_exact_solve_matches_converged_jacobi():
    """With an external x dimension the reference's Jacobi meets its stop
    test; its result and the exact solution then agree to what that test
    leaves: it stops once no point moves by 1e-9 of the boundary values'
    range (1.2e-9 for A here) in a sweep, some 40 sweeps' worth of such
    moves short of the fixed point, so within 2e-7 absolute."""
    fb = ("external", "external") + ("periodic",) * 4
    cfg = _box((8, 6, 10), fb, bound_phi=(0.0, 0.02, 0.0, 0.0, 0.0, 0.0),
               bound_A=((0.0,) * 6, (0.0, 1.2, 0.0, 0.0, 0.0, 0.0), (0.0,) * 6))
    oj, oe = _oracle(cfg, 0), _oracle(cfg, 1)
    rho, J = _sources(oj.get_field(abi.RHO).shape)
    rho = rho - 2e-4
    for o in (oj, oe):
        _set_sources(o, rho, J)
    rj, itj = oj.initialize_fields_only()
    re_, ite = oe.initialize_fields_only()
    assert rj == 0 and re_ == 0 and max(itj) < 10000
    for i in (abi.PHI1, abi.AX1, abi.AY1, abi.AZ1, abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ):
        assert np.abs(oe.get_field(i) - oj.get_field(i)).max() <= 2e-7, abi.FIELD_NAMES[i]
    assert max(ite) < min(itj) / 4  # conjugate gradients against Jacobi sweeps
    oj.close()
    oe.close()


def test_periodic_even_jacobi_keeps_the_odd_even_mode():
    """On a periodic grid with even sides the Jacobi iteration's odd-even
    mode has eigenvalue -1: after the 10000-iteration cap it is still
    there, so E differs from the exact solution's by more than rounding."""
    cfg = _box((6, 6, 4))
    oj, oe = _oracle(cfg, 0), _oracle(cfg, 1)
    rho, J = _sources(oj.get_field(abi.RHO).shape)
    for o in (oj, oe):
        _set_sources(o, rho, J)
    rj, itj = oj.initialize_fields_only()
    assert rj == -3 and itj[0] == 10000
    assert oe.initialize_fields_only()[0] == 0
    assert rel_l2(oj.get_field(abi.EX), oe.get_field(abi.EX)) > 1e-3
    oj.close()
    oe.close()


# ---- GPU -------------------------------------------------------------------

def _gpu(cfg, precision=abi.FP64, rtol=1e-12):
    from backends import GpuBackend

    return GpuBackend(configs.input_info(cfg), 0.4, precision=precision, poisson_solver=abi.POISSON_MULTIGRID,
                      poisson_rtol=rtol)


# The odd periodic case smooths by damped Jacobi, and its spacings differ by
# 4x (a 16x ratio of the stencil's weights), which point smoothers handle
# slowly: about 0.7 per cycle. The others converge at about 0.2 or better.
CYCLE_CAP = {"periodic_odd": 100}
CASES = {
    "periodic_16": ((16, 16, 16), ("periodic",) * 6, (1.0, 1.0, 1.0)),
    "periodic_odd": ((6, 5, 4), ("periodic",) * 6, (1.0, 0.5, 2.0)),
    "external_x": ((16, 12, 8), ("external", "external") + ("periodic",) * 4, (1.0, 1.0, 1.0)),
    "external_all": ((12, 10, 9), ("external",) * 6, (0.7, 1.0, 1.3)),
    "periodic_x_external_yz": ((32, 8, 8), ("periodic", "periodic") + ("external",) * 4, (1.0, 1.0, 1.0)),
    # degenerate: no unknowns at all (the boundary planes are the solution),
    # and the smallest periodic grid (one level, every neighbour a wrap)
    "external_x_one_cell": ((1, 6, 4), ("external", "external") + ("periodic",) * 4, (1.0, 1.0, 1.0)),
    "periodic_2": ((2, 2, 2), ("periodic",) * 6, (1.0, 1.0, 1.0)),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_multigrid_matches_oracle(case):
    n, fb, dx = CASES[case]
    cfg = _box(n, fb, dx=dx, bound_phi=(0.1, -0.2, 0.05, 0.0, 0.3, 0.1),
               bound_A=((0.0, 0.2, 0.0, 0.0, 0.0, 0.0), (0.0,) * 6, (0.1,) * 6))
    g, o = _gpu(cfg), _oracle(cfg, 1)
    rho, J = _sources(g.shape)
    if "external" in case:
        rho = rho - 2e-4
    for b in (g, o):
        _set_sources(b, rho, J)
    rg, itg = g.poisson_init()
    ro, _ = o.initialize_fields_only()
    assert rg == 0 and ro == 0, (rg, ro)
    assert max(itg) <= CYCLE_CAP.get(case, 40), itg
    unknowns = all(n[d] >= (1 if fb[2 * d] == "periodic" else 2) for d in range(3))
    for s, r in zip(SLOTS, SOURCES):
        if not unknowns:
            break
        res, scale = _residual(g.get_field(s), g.get_field(r), cfg)
        assert res <= 1e-11 * scale, (abi.FIELD_NAMES[s], res, scale)
    for i in list(range(13)) + [abi.PHI1, abi.PHI2, abi.AX1, abi.AY1, abi.AZ1]:
        a, b = g.get_field(i), o.get_field(i)
        if np.abs(b).max() == 0.0:
            assert np.abs(a).max() == 0.0, abi.FIELD_NAMES[i]
        else:
            assert rel_l2(a, b) <= 1e-9, (abi.FIELD_NAMES[i], rel_l2(a, b))
    g.close()
    o.close()


@pytest.mark.gpu
def test_gpu_multigrid_langmuir_start_and_mixed_form():
    """The 32^3 Langmuir start with particles: FP64 multigrid against the
    oracle's exact solve, few cycles, and the mixed form's fields equal to
    the FP64 form's (it solves on the same FP64 slots)."""
    from backends import GpuBackend

    cfg = configs.langmuir32()
    parts = loading.sample_all(cfg)
    info = configs.input_info(cfg)
    g = GpuBackend(info, cfg.dt, poisson_solver=abi.POISSON_MULTIGRID, poisson_rtol=1e-12)
    m = GpuBackend(info, cfg.dt, precision=abi.MIXED, poisson_solver=abi.POISSON_MULTIGRID, poisson_rtol=1e-12)
    o = OracleBackend(info, cfg.dt)
    o.set_poisson_solver(1, 1e-13)
    for si, p in enumerate(parts):
        for b in (g, m, o):
            b.add_species(si, p)
    rg, itg = g.init_fields()
    rm, itm = m.init_fields()
    ro, _ = o.init_fields()
    assert rg == rm == ro == 0 and itg == itm and max(itg) <= 20, (rg, rm, ro, itg, itm)
    for i in (abi.EX, abi.EY, abi.EZ, abi.PHI1):
        assert rel_l2(g.get_field(i), o.get_field(i)) <= 1e-9, abi.FIELD_NAMES[i]
    for i in (abi.EX, abi.EY, abi.EZ):
        assert rel_l2(m.get_field(i), g.get_field(i)) <= 1e-6, abi.FIELD_NAMES[i]
    for b in (g, m, o):
        b.close()


@pytest.mark.gpu
def test_gpu_multigrid_large_box_against_fft():
    """128 x 64 x 64 periodic, default tolerance: against an FFT solution."""
    cfg = _box((128, 64, 64))
    g = _gpu(cfg, rtol=1e-10)
    rho, J = _sources(g.shape)
    _set_sources(g, rho, J)
    rc, it = g.poisson_init()
    assert rc == 0 and max(it) <= 20, (rc, it)
    for s, r in ((abi.PHI1, abi.RHO), (abi.AZ1, abi.JZ)):
        want = _fft_solution(g.get_field(r), cfg)
        got = g.get_field(s)[P(cfg.n)]
        assert np.abs(got - want).max() <= 1e-7 * np.abs(want).max(), abi.FIELD_NAMES[s]
    g.close()


@pytest.mark.gpu
def test_gpu_multigrid_refusals():
    from backends import GpuBackend

    cfg = _box((8, 8, 8))
    with pytest.raises(abi.EmooError):
        GpuBackend(configs.input_info(cfg), 0.4, poisson_solver=7)
    mixed_sides = _box((8, 8, 8), ("external", "periodic") + ("periodic",) * 4)
    with pytest.raises(abi.EmooError):
        GpuBackend(configs.input_info(mixed_sides), 0.4, poisson_solver=abi.POISSON_MULTIGRID)


def test_oracle_exact_solve_matches_a_sparse_direct_solve():
    """Every side external, anisotropic cells: the oracle's conjugate-gradient
    solve against scipy's sparse direct solve of the same equations (unknowns
    2..n per dimension, the PoissonBC planes 1 and n + 1 moved to the right
    side)."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    cfg = _box((7, 6, 5), ("external",) * 6, dx=(0.7, 1.1, 1.6), bound_phi=(0.3, -0.1, 0.2, 0.05, -0.2, 0.15))
    o = _oracle(cfg, 1)
    rho, J = _sources(o.get_field(abi.RHO).shape)
    _set_sources(o, rho - 2e-4, J)
    assert o.initialize_fields_only()[0] == 0
    u = o.get_field(abi.PHI1)
    n = cfg.n
    m = [n[d] - 1 for d in range(3)]          # unknowns 2..n
    N = m[0] * m[1] * m[2]
    idx = lambda a, b, c: (a * m[1] + b) * m[2] + c  # noqa: E731
    rows, cols, vals = [], [], []
    rhs = np.zeros(N)
    R = o.get_field(abi.RHO)
    for a in range(m[0]):
        for b in range(m[1]):
            for c in range(m[2]):
                i, j, k = a + 2, b + 2, c + 2
                r = idx(a, b, c)
                rhs[r] = -FOUR_PI * R[i, j, k]
                diag = 0.0
                for d, (di, dj, dk) in enumerate(((1, 0, 0), (0, 1, 0), (0, 0, 1))):
                    w = 1.0 / cfg.dx[d] ** 2
                    diag -= 2 * w
                    for sgn in (-1, 1):
                        ii, jj, kk = i + sgn * di, j + sgn * dj, k + sgn * dk
                        aa, bb, cc = ii - 2, jj - 2, kk - 2
                        if 0 <= aa < m[0] and 0 <= bb < m[1] and 0 <= cc < m[2]:
                            rows.append(r), cols.append(idx(aa, bb, cc)), vals.append(w)
                        else:  # a boundary plane value, as the fill left it
                            rhs[r] -= w * u[ii, jj, kk]
                rows.append(r), cols.append(r), vals.append(diag)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(N, N))
    x = spl.spsolve(A, rhs)
    got = u[2:n[0] + 1, 2:n[1] + 1, 2:n[2] + 1].reshape(-1)
    assert np.abs(got - x).max() <= 1e-11 * np.abs(x).max()
    o.close()
