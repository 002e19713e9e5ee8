"""Two-stream workload (counter-streaming beams over an immobile neutralising
background, seeded B noise): the build's own features with no reference
counterpart, checked against the oracle's restatement of them.

  * the oracle's background makes the deposited charge neutral on average
    (CPU);
  * the FP64 GPU form matches the oracle step by step (crossings exact,
    fields and particles within FP64_RTOL, summation order only);
  * the mixed form stays within its FP32 bars against the FP64 form.
"""
import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading
from backends import GpuBackend, OracleBackend, by_id, rel_l2
from helpers import FIELDS

FP64_RTOL = 1e-9
SMALL = (12, 6, 6)
STEPS = 12


def _load(b, parts):
    nid = 0
    for si, p in enumerate(parts):
        n = len(p["x"])
        b.add_species(si, p, ids=np.arange(nid, nid + n))
        nid += n


def _noise(b, cfg):
    f = configs.b_noise_fields(cfg)
    for c in range(3):
        b.set_field(abi.BX + c, f[c])
        b.set_field(abi.BX_TM1 + c, f[c])


def _oracle(cfg, parts):
    info = configs.input_info(cfg)
    o = OracleBackend(info, cfg.dt)
    o.set_rho_background(configs.rho_background(cfg))
    _load(o, parts)
    o.init_fields()  # constant start (E0, B0 = 0); sets the step's time and dt
    _noise(o, cfg)
    # the reference pushes with the fields cached by InterpolateEB; the GPU
    # gathers at the push, so the cache must see the noise too
    o.interpolate()
    return o


def _gpu(cfg, parts, prec):
    g = GpuBackend(configs.input_info(cfg), cfg.dt, precision=prec, rho_background=configs.rho_background(cfg))
    _load(g, parts)
    g.init_fields()
    _noise(g, cfg)
    return g


def test_background_neutralises_the_deposit():
    cfg = configs.twostream(SMALL, STEPS)
    parts = loading.sample_all(cfg)
    bg = configs.rho_background(cfg)
    assert bg > 0
    rho = []
    for v in (0.0, bg):
        o = _oracle(cfg, parts)
        o.set_rho_background(v)
        o.deposit(1)
        o.execute_bc(abi.SEND_JRHO)
        rho.append(o.get_field(abi.RHO))
        o.close()
    phys = (slice(1, SMALL[0] + 1), slice(1, SMALL[1] + 1), slice(1, SMALL[2] + 1))
    d = rho[1] - rho[0]
    np.testing.assert_allclose(d[phys], bg, rtol=1e-12)
    d[phys] = 0.0
    assert not d.any()
    # the electrons' mean charge is -bg up to what the reference's fold leaves
    # in the edge ghosts (it folds the physical transverse range only)
    assert abs(rho[1][phys].mean()) < 0.05 * bg


@pytest.mark.gpu
def test_fp64_matches_oracle():
    cfg = configs.twostream(SMALL, STEPS)
    parts = loading.sample_all(cfg)
    o = _oracle(cfg, parts)
    g = _gpu(cfg, parts, abi.FP64)
    for ti in range(STEPS):
        cg = g.step(1)
        co, _ = o.step(ti)
        assert cg == co, (ti, cg, co)
    pg, po = by_id(g.particles()), by_id(o.particles())
    for k in ("x", "y", "z", "vx", "vy", "vz", "gamma"):
        assert rel_l2(pg[k], po[k]) <= FP64_RTOL, (k, rel_l2(pg[k], po[k]))
    for i in FIELDS:
        assert rel_l2(g.get_field(i), o.get_field(i)) <= FP64_RTOL, (abi.FIELD_NAMES[i], rel_l2(g.get_field(i), o.get_field(i)))
    g.close()
    o.close()


@pytest.mark.gpu
def test_mixed_within_fp32_bars():
    cfg = configs.twostream(SMALL, STEPS)
    parts = loading.sample_all(cfg)
    out = {}
    for prec in (abi.FP64, abi.MIXED):
        g = _gpu(cfg, parts, prec)
        g.step(STEPS)
        out[prec] = {i: g.get_field(i) for i in (abi.EX, abi.BY, abi.JX, abi.RHO)}
        g.close()
    # the beams are stable over 12 steps at this size: FP32 rounding only.
    # rho is dominated by the exactly cancelling background, so it is
    # compared against the deposited part (the background's magnitude)
    bg = configs.rho_background(cfg)
    for i in (abi.EX, abi.BY, abi.JX):
        assert rel_l2(out[abi.MIXED][i], out[abi.FP64][i]) <= 2e-5, (abi.FIELD_NAMES[i],)
    drho = out[abi.MIXED][abi.RHO] - out[abi.FP64][abi.RHO]
    assert np.sqrt(np.mean(drho ** 2)) <= 1e-6 * bg
