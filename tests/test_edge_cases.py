"""Empty and ragged particle sets through the whole loop.

* No particles at all (both forms, both policies): the loop runs as a vacuum
  field solver, the readback returns nothing, history rows are written, and
  the host-resident mode takes an empty species without arrays.
* Ragged species: 1, 0, 37 and 1000 particles (counts that fill no warp or
  block evenly), FP64 against the oracle over steps with a sort, and the
  mixed form's host-resident path against its round trip."""
import ctypes as C

import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading
from backends import OracleBackend, by_id, rel_l2

pytestmark = pytest.mark.gpu
_D = C.POINTER(C.c_double)
KEYS = ("x", "y", "z", "vx", "vy", "vz", "gamma")


def _cfg(policy, relativity=1):
    cfg = configs.tiny("edge", n=(6, 5, 4), relativity=relativity, init="constant", nstep_sort=3, steps=7,
                       E0=(1e-3, 0.0, 0.0), B0=(0.0, 0.0, 2e-3))
    return cfg


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
@pytest.mark.parametrize("policy", [abi.POLICY_REFERENCE, abi.POLICY_CORRECTED])
def test_no_particles(precision, policy):
    from backends import GpuBackend

    cfg = _cfg(policy)
    g = GpuBackend(configs.input_info(cfg), cfg.dt, precision=precision, policy=policy, capacity=1)
    assert g.init_fields()[0] == abi.OK
    for _ in range(cfg.steps):
        assert g.step(1) == [0] * 6
    assert g.num_particles() == 0
    assert g.history_rows().shape[0] >= 1
    for f in (abi.JX, abi.JY, abi.JZ, abi.RHO):
        assert np.abs(g.get_field(f)).max() == 0.0
    assert np.isfinite(g.get_field(abi.EX)).all()
    if precision == abi.MIXED:
        L = abi.lib()
        for s in range(len(cfg.species)):
            abi.check(L.emoo_attach_particles(g.h, s, 0, *([None] * 7)))
        cnt = (C.c_int64 * 6)()
        abi.check(L.emoo_step(g.h, 3, cnt))
        abi.check(L.emoo_detach_particles(g.h))
    g.close()


def _ragged(cfg, counts, seed=5):
    parts = loading.sample_all(cfg)
    out = []
    rng = np.random.default_rng(seed)
    for s, n in enumerate(counts):
        p = parts[s % len(parts)]
        idx = rng.choice(len(p["x"]), size=n, replace=n > len(p["x"]))
        out.append({k: np.ascontiguousarray(p[k][idx]) for k in KEYS})
    return out


def _cfg4(relativity):
    cfg = configs.tiny("ragged", n=(6, 5, 4), relativity=relativity, init="poisson", nstep_sort=3, steps=7)
    cfg.species = cfg.species + [configs.Species("e2", -1.0, 1.0, 1, 0.1), configs.Species("i2", 1.0, 40.0, 1, 0.02)]
    return cfg


@pytest.mark.parametrize("relativity", [0, 1])
def test_ragged_species_fp64_matches_oracle(relativity):
    from backends import GpuBackend

    cfg = _cfg4(relativity)
    parts = _ragged(cfg, [1, 0, 37, 1000])
    info = configs.input_info(cfg)
    info.nspecies = 4
    g = GpuBackend(info, cfg.dt, capacity=1038)
    o = OracleBackend(info, cfg.dt)
    nid = 0
    for s, p in enumerate(parts):
        ids = np.arange(nid, nid + len(p["x"]))
        nid += len(p["x"])
        if len(p["x"]):
            g.add_species(s, p, ids=ids)
            o.add_species(s, p, ids=ids)
    assert g.init_fields()[0] == o.init_fields()[0]
    for ti in range(cfg.steps):
        assert g.step(1) == o.step(ti)[0], ti
    for f in (abi.EX, abi.EY, abi.BZ, abi.JX, abi.RHO):
        assert rel_l2(g.get_field(f), o.get_field(f)) <= 1e-9, abi.FIELD_NAMES[f]
    pg, po = by_id(g.particles()), by_id(o.particles())
    for k in ("x", "vx", "vz"):
        assert rel_l2(pg[k], po[k]) <= 1e-9, k
    g.close()
    o.close()


def test_ragged_species_host_resident_equals_round_trip():
    from backends import GpuBackend

    cfg = _cfg4(1)
    parts = _ragged(cfg, [1, 0, 37, 1000])
    info = configs.input_info(cfg)
    info.nspecies = 4
    L = abi.lib()
    hs = []
    for _ in range(2):
        g = GpuBackend(info, cfg.dt, precision=abi.MIXED, capacity=1038, track_ids=0)
        for s, p in enumerate(parts):
            if len(p["x"]):
                g.add_species(s, p)
        g.init_fields()
        hs.append(g)
    A, B = hs

    def arrays(h):
        out = []
        for s in range(4):
            n = C.c_int64()
            abi.check(L.emoo_num_particles(h, s, C.byref(n)))
            a = {k: np.zeros(n.value) for k in KEYS}
            m = C.c_int64()
            abi.check(L.emoo_get_particles(h, s, n.value, *[a[k].ctypes.data_as(_D) for k in KEYS], None,
                                           C.byref(m)))
            out.append(a)
        return out

    ra, rb = arrays(A.h), arrays(B.h)
    cnt = (C.c_int64 * 6)()
    for _ in range(cfg.steps):
        for s in range(4):
            abi.check(L.emoo_set_particles(A.h, s, len(ra[s]["x"]), *[ra[s][k].ctypes.data_as(_D) for k in KEYS]))
        abi.check(L.emoo_step(A.h, 1, cnt))
        ra = arrays(A.h)
    for s in range(4):
        ptr = [rb[s][k].ctypes.data_as(_D) for k in KEYS] if len(rb[s]["x"]) else [None] * 7
        abi.check(L.emoo_attach_particles(B.h, s, len(rb[s]["x"]), *ptr))
    abi.check(L.emoo_step(B.h, cfg.steps, cnt))
    for s in range(4):
        for k in KEYS:
            assert np.array_equal(ra[s][k], rb[s][k], equal_nan=True), (s, k)
    assert np.array_equal(A.get_field(abi.EX), B.get_field(abi.EX))
    A.close()
    B.close()


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_sort_keys_beyond_32_bits_are_refused(precision):
    """Four species on a 1024^3 grid need sort keys (species * cells + cell)
    of more than 32 bits: the handle is refused before its grid is allocated."""
    L = abi.lib()

    def create(nspec):
        cfg = configs.tiny("wide", n=(1024, 1024, 1024))
        cfg.species = (cfg.species * 2)[:nspec]
        info = configs.input_info(cfg)
        info.nspecies = nspec
        o = abi.Opts()
        L.emoo_default_opts(C.byref(o))
        o.precision = precision
        h = C.c_void_p()
        rc = L.emoo_create(C.byref(info), C.byref(o), C.byref(h))
        return rc, h

    rc, h = create(4)
    assert rc == abi.ERR_UNSUPPORTED and not h.value
