"""Host-resident particles (emoo_attach_particles): emoo_step streams the
caller's FP64 arrays through the fused kernel, and its result must equal,
bit for bit, emoo_set_particles + emoo_step(1) + emoo_get_particles per step
on the same arrays - particles, fields, crossing counts and history rows -
across steps that sort, write a history row or make the first push (those
run on the device store between an upload and a readback)."""
import ctypes as C

import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading

KEYS = ("x", "y", "z", "vx", "vy", "vz", "gamma")
_D = C.POINTER(C.c_double)


def _arrays(L, h, nspec):
    out = []
    for s in range(nspec):
        n = C.c_int64()
        abi.check(L.emoo_num_particles(h, s, C.byref(n)))
        a = {k: np.zeros(n.value) for k in KEYS}
        m = C.c_int64()
        abi.check(L.emoo_get_particles(h, s, n.value, *[a[k].ctypes.data_as(_D) for k in KEYS], None, C.byref(m)))
        out.append(a)
    return out


def _handle(cfg, policy):
    from backends import GpuBackend

    g = GpuBackend(configs.input_info(cfg), cfg.dt, precision=abi.MIXED, policy=policy, track_ids=0)
    for si, p in enumerate(loading.sample_all(cfg)):
        g.add_species(si, p)
    assert g.init_fields()[0] in (abi.OK, abi.ERR_NOT_CONVERGED)
    return g


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("relativity,policy", [(1, abi.POLICY_REFERENCE), (0, abi.POLICY_REFERENCE),
                                                (1, abi.POLICY_CORRECTED)])
def test_host_resident_steps_equal_the_round_trip(relativity, policy):
    cfg = configs.tiny("hostres", n=(8, 6, 5), relativity=relativity, init="poisson", nstep_sort=4, steps=14,
                       vth=0.15, dt=0.4)
    L = abi.lib()
    A, B = _handle(cfg, policy), _handle(cfg, policy)
    nspec = len(cfg.species)
    ra, rb = _arrays(L, A.h, nspec), _arrays(L, B.h, nspec)
    for s in range(nspec):
        for k in KEYS:
            assert _same(ra[s][k], rb[s][k])
    # A: the round trip, one step at a time
    counts_a = np.zeros(6, dtype=np.int64)
    cnt = (C.c_int64 * 6)()
    for _ in range(cfg.steps):
        for s in range(nspec):
            abi.check(L.emoo_set_particles(A.h, s, len(ra[s]["x"]), *[ra[s][k].ctypes.data_as(_D) for k in KEYS]))
        abi.check(L.emoo_step(A.h, 1, cnt))
        counts_a += np.array(cnt[:])
        ra = _arrays(L, A.h, nspec)
    # B: host-resident, the same steps in two calls
    for s in range(nspec):
        abi.check(L.emoo_attach_particles(B.h, s, len(rb[s]["x"]), *[rb[s][k].ctypes.data_as(_D) for k in KEYS]))
    counts_b = np.zeros(6, dtype=np.int64)
    for k in (5, cfg.steps - 5):
        abi.check(L.emoo_step(B.h, k, cnt))
        counts_b += np.array(cnt[:])
    np.testing.assert_array_equal(counts_a, counts_b)
    for s in range(nspec):
        for k in KEYS:
            assert _same(ra[s][k], rb[s][k]), (s, k, np.abs(ra[s][k] - rb[s][k]).max())
    for f in (abi.EX, abi.EY, abi.EZ, abi.BX, abi.BY, abi.BZ, abi.JX, abi.JY, abi.JZ, abi.RHO):
        assert _same(A.get_field(f), B.get_field(f)), abi.FIELD_NAMES[f]
    np.testing.assert_array_equal(A.history_rows(), B.history_rows())
    # readback while attached copies the arrays; detaching keeps their state
    rb2 = _arrays(L, B.h, nspec)
    abi.check(L.emoo_detach_particles(B.h))
    rb3 = _arrays(L, B.h, nspec)
    for s in range(nspec):
        for k in KEYS:
            assert _same(rb2[s][k], rb[s][k]) and _same(rb3[s][k], ra[s][k])
    A.close()
    B.close()


@pytest.mark.gpu
def test_host_resident_refusals():
    L = abi.lib()
    cfg = configs.tiny("hostref", n=(6, 5, 4), relativity=1, init="constant")
    g = _handle(cfg, abi.POLICY_REFERENCE)
    r = _arrays(L, g.h, len(cfg.species))
    n0 = len(r[0]["x"])
    ptr = [r[0][k].ctypes.data_as(_D) for k in KEYS]
    assert L.emoo_attach_particles(g.h, 0, n0 + 1, *ptr) == abi.ERR_ARG          # wrong count
    assert L.emoo_attach_particles(g.h, 0, n0, *ptr[:6], None) == abi.ERR_ARG    # relativistic needs gamma
    for s in range(len(cfg.species)):
        abi.check(L.emoo_attach_particles(g.h, s, len(r[s]["x"]), *[r[s][k].ctypes.data_as(_D) for k in KEYS]))
    assert L.emoo_sort(g.h) == abi.ERR_STATE
    assert L.emoo_set_particles(g.h, 0, n0, *ptr) == abi.ERR_STATE
    abi.check(L.emoo_detach_particles(g.h))
    abi.check(L.emoo_sort(g.h))
    g.close()
    walls = configs.tiny("hostwall", n=(6, 5, 4), init="constant",
                         part_bc=("absorbing", "absorbing") + ("periodic",) * 4,
                         field_bc=("external", "external") + ("periodic",) * 4)
    w = _handle(walls, abi.POLICY_REFERENCE)
    rw = _arrays(L, w.h, len(walls.species))
    assert L.emoo_attach_particles(w.h, 0, len(rw[0]["x"]), *[rw[0][k].ctypes.data_as(_D) for k in KEYS]) == \
        abi.ERR_UNSUPPORTED
    w.close()
