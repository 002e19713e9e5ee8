"""Output files: the field time series (the reference's Hdf5IO datasets as raw
files, src/IO/hdf5io.cpp) and restart files (no reference counterpart).

CPU: the reader against a directory written by numpy in the documented
layout. GPU: the writer against emoo_get_field (physical points, the
reference's coordinate offsets, B averaged with B_tm1 as Grid::AvgB does);
continuing from a restart reproduces the uninterrupted run (bit for bit in
the mixed form, whose deposit is order-fixed; to the FP64 deposit's
summation-order bar in the FP64 form); a restart refuses a handle of another
grid."""
import ctypes as C
import os

import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading
from apc_524_project_gb300.fieldio import NAMES, read_fields


def test_reader_layout(tmp_path):
    n, nt = (3, 4, 5), 2
    t = np.array([0.0, 0.5])
    t.astype("<f8").tofile(tmp_path / "time.f64")
    rng = np.random.default_rng(1)
    ref = {}
    for name in ("Ex", "rho"):
        snaps = rng.normal(size=(nt,) + n)
        snaps.astype("<f8").tofile(tmp_path / f"{name}.f64")
        np.concatenate([np.arange(n[0]) + 0.5, np.arange(n[1]), np.arange(n[2])]).astype("<f8").tofile(
            tmp_path / f"{name}.xyz")
        ref[name] = snaps
    tt, f = read_fields(str(tmp_path), n)
    np.testing.assert_array_equal(tt, t)
    assert set(f) == {"Ex", "rho"}
    for name, snaps in ref.items():
        data, (x, y, z) = f[name]
        assert data.shape == n + (nt,)  # the reference dataset's dims [nx][ny][nz][time]
        np.testing.assert_array_equal(data[..., 1], snaps[1])
        np.testing.assert_array_equal(x, np.arange(n[0]) + 0.5)


# ---- GPU -----------------------------------------------------------------

def _loaded(cfg, precision, parts):
    from backends import GpuBackend

    g = GpuBackend(configs.input_info(cfg), cfg.dt, precision=precision)
    nid = 0
    for si, p in enumerate(parts):
        g.add_species(si, p, ids=np.arange(nid, nid + len(p["x"])))
        nid += len(p["x"])
    g.init_fields()
    return g


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_field_writer_matches_the_grid(tmp_path, precision):
    cfg = configs.tiny("io", n=(6, 5, 4), dx=(0.7, 1.3, 0.5), relativity=1, init="constant", vth=0.1)
    g = _loaded(cfg, precision, loading.sample_all(cfg))
    d = str(tmp_path / "fields")
    snaps = []
    for k in range(3):
        abi.check(g.L.emoo_write_fields(g.h, d.encode(), abi.FIELDS_ALL))
        snaps.append({i: g.get_field(i) for i in range(13)})
        g.step(2)
    t, f = read_fields(d, cfg.n)
    assert len(t) == 3 and t[0] == 0.0 and np.all(np.diff(t) > 0)
    ids = {"Ex": 0, "Ey": 1, "Ez": 2, "Jx": 6, "Jy": 7, "Jz": 8, "rho": 9}
    n = cfg.n
    phys = (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))
    for name in NAMES:
        data, (x, y, z) = f[name]
        for k in range(3):
            if name in ids:
                want = snaps[k][ids[name]][phys]
            else:
                c = "xyz".index(name[1])
                want = ((snaps[k][abi.BX + c] + snaps[k][abi.BX_TM1 + c]) / 2)[phys]
            np.testing.assert_array_equal(data[..., k], want, err_msg=name)
        # coordinates: xyz0 + d (i - 1), + d/2 along an E / J component's axis
        # and across a B component's two others
        off = {"E": lambda a, c: a == c, "J": lambda a, c: a == c, "B": lambda a, c: a != c}
        for a, v in enumerate((x, y, z)):
            half = name != "rho" and off[name[0]](a, "xyz".index(name[1]))
            np.testing.assert_allclose(v, cfg.dx[a] * (np.arange(n[a]) + (0.5 if half else 0.0)), rtol=0,
                                       atol=1e-12)
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_restart_continues_the_run(tmp_path, precision):
    from backends import by_id, rel_l2

    cfg = configs.tiny("rst", n=(8, 6, 5), relativity=1, init="constant", vth=0.12, nstep_sort=3, ppc=4,
                       part_bc=("reflecting", "reflecting", "periodic", "periodic", "periodic", "periodic"),
                       field_bc=("external", "external", "periodic", "periodic", "periodic", "periodic"),
                       waves=[configs.Wave(-1, 2, 0.3, 0.8, 0.0, 0.3, 1.0)])
    parts = loading.sample_all(cfg)
    a = _loaded(cfg, precision, parts)
    a.step(5)
    path = str(tmp_path / "state.rst")
    abi.check(a.L.emoo_write_restart(a.h, path.encode()), "emoo_write_restart")
    a.step(7)
    b = _loaded(cfg, precision, parts)  # same input and options, other state
    b.step(1)
    abi.check(b.L.emoo_read_restart(b.h, path.encode()), "emoo_read_restart")
    b.step(7)
    bar = 0.0 if precision == abi.MIXED else 1e-12
    for i in range(13):
        fa, fb = a.get_field(i), b.get_field(i)
        if bar == 0.0:
            np.testing.assert_array_equal(fa, fb, err_msg=abi.FIELD_NAMES[i])
        else:
            assert rel_l2(fb, fa) <= bar, i
    pa, pb = by_id(a.particles()), by_id(b.particles())
    np.testing.assert_array_equal(pa["id"], pb["id"])
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        if bar == 0.0:
            np.testing.assert_array_equal(pa[k], pb[k], err_msg=k)
        else:
            assert rel_l2(pb[k], pa[k]) <= bar, k
    np.testing.assert_allclose(np.array(b.history_rows()), np.array(a.history_rows()), rtol=1e-12)
    a.close()
    b.close()


@pytest.mark.gpu
def test_restart_refuses_another_grid(tmp_path):
    cfg = configs.tiny("rst2", n=(6, 5, 4), init="constant")
    a = _loaded(cfg, abi.MIXED, loading.sample_all(cfg))
    path = str(tmp_path / "s.rst")
    abi.check(a.L.emoo_write_restart(a.h, path.encode()))
    other = configs.tiny("rst3", n=(6, 5, 5), init="constant")
    b = _loaded(other, abi.MIXED, loading.sample_all(other))
    assert b.L.emoo_read_restart(b.h, path.encode()) == abi.ERR_STATE
    c = _loaded(cfg, abi.FP64, loading.sample_all(cfg))
    assert c.L.emoo_read_restart(c.h, path.encode()) == abi.ERR_STATE
    for h in (a, b, c):
        h.close()
