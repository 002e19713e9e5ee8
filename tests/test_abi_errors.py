"""Refused calls on a live handle: each entry point answers bad arguments
with its documented status, and the handle keeps its particles and steps on.

The reference's own interfaces assert or throw on such calls
(Particle_Handler, Grid::getFieldPtr, Input::readinfo); across the C ABI they
become status codes. Every case here is caught on the host, so no kernel sees
the bad argument; both forms."""
import ctypes as C

import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading

pytestmark = pytest.mark.gpu
_D = C.POINTER(C.c_double)


def _handle(precision):
    from backends import GpuBackend

    cfg = configs.tiny("abi_errors", n=(6, 5, 4), relativity=1, init="constant", nstep_sort=3, steps=4)
    g = GpuBackend(configs.input_info(cfg), cfg.dt, precision=precision, track_ids=0)
    for si, p in enumerate(loading.sample_all(cfg)):
        g.add_species(si, p)
    g.init_fields()
    return g


def _ptr(a):
    return a.ctypes.data_as(_D)


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_refused_calls_leave_the_handle_usable(precision):
    g = _handle(precision)
    L, h, ns = g.L, g.h, g.nspec
    n0 = C.c_int64()
    abi.check(L.emoo_num_particles(h, -1, C.byref(n0)))
    counts = [g.num_particles(s) for s in range(ns)]
    a = np.zeros(max(counts) + 1)
    six = [_ptr(a)] * 6

    # particles in
    assert L.emoo_load_particles(h, -1, 1, *six, None, None) == abi.ERR_ARG
    assert L.emoo_load_particles(h, ns, 1, *six, None, None) == abi.ERR_ARG
    assert L.emoo_load_particles(h, 0, -1, *six, None, None) == abi.ERR_ARG
    assert L.emoo_load_particles(h, 0, 1, None, *six[1:], None, None) == abi.ERR_ARG
    assert L.emoo_load_generated(h, None, 1) == abi.ERR_ARG

    # particles out
    got = C.c_int64()
    assert L.emoo_num_particles(h, 0, None) == abi.ERR_ARG
    assert L.emoo_num_particles(h, ns, C.byref(got)) == abi.ERR_ARG
    assert L.emoo_get_particles(h, ns, len(a), *six, None, None, C.byref(got)) == abi.ERR_ARG
    assert L.emoo_get_particles(h, 0, counts[0] - 1, *six, None, None, C.byref(got)) == abi.ERR_ARG
    assert L.emoo_get_particles(h, 0, len(a), *six, None, None, None) == abi.ERR_ARG
    ids = np.zeros(len(a), dtype=np.int64)
    assert L.emoo_get_particles(h, 0, len(a), *six, None, ids.ctypes.data_as(C.POINTER(C.c_int64)),
                                C.byref(got)) == abi.ERR_STATE  # ids were not tracked
    assert L.emoo_get_particle_fields(h, 0, len(a), *six, C.byref(got)) == abi.ERR_STATE  # no interpolation yet

    # fields
    f = np.zeros(g.shape)
    assert L.emoo_get_field(h, -1, _ptr(f)) == abi.ERR_ARG
    assert L.emoo_get_field(h, abi.NFIELDS, _ptr(f)) == abi.ERR_ARG
    assert L.emoo_get_field(h, abi.EX, None) == abi.ERR_ARG
    assert L.emoo_set_field(h, abi.NFIELDS, _ptr(f)) == abi.ERR_ARG
    assert L.emoo_set_field(h, abi.EX, None) == abi.ERR_ARG

    # waves (this case injects none)
    w = np.ones(1)
    assert L.emoo_set_waves(h, 1, _ptr(w), _ptr(w)) == abi.ERR_ARG
    assert L.emoo_set_wave_shape(h, 0, None) == abi.ERR_ARG

    # loop and diagnostics
    assert L.emoo_step(h, -1, None) == abi.ERR_ARG
    assert L.emoo_history(h, None) == abi.ERR_ARG
    rows = np.zeros(8)
    nr = C.c_int()
    assert L.emoo_history_rows(h, -1, _ptr(rows), C.byref(nr)) == abi.ERR_ARG
    assert L.emoo_history_rows(h, 1, _ptr(rows), None) == abi.ERR_ARG
    assert L.emoo_gauss_residual(h, None) == abi.ERR_ARG
    assert L.emoo_cell_id(h, 0.5, 0.5, 0.5, None) == abi.ERR_ARG
    if precision == abi.FP64:
        assert L.emoo_perturb(h, 1, 1.5) == abi.ERR_ARG
    else:
        assert L.emoo_perturb(h, 1, 1e-7) == abi.ERR_UNSUPPORTED

    # nothing changed, and the handle still steps
    assert [g.num_particles(s) for s in range(ns)] == counts
    c = g.step(4)
    assert len(c) == 6
    abi.check(L.emoo_check(h), "device error word")
    n1 = C.c_int64()
    abi.check(L.emoo_num_particles(h, -1, C.byref(n1)))
    assert n1.value == n0.value
    assert np.isfinite(g.get_field(abi.EX)).all()
    g.close()
