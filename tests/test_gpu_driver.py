"""The reference-style C++ driver (emoopic_gpu, built on include/emoopic.hpp)
run on an input.txt, against the CPU oracle fed the same particles: the
history.dat it writes matches the oracle's history rows."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from apc_524_project_gb300 import abi, build_native
from backends import OracleBackend
from helpers import history_close

pytestmark = pytest.mark.gpu

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
UNIT_VTH = 0.002232


def reference_load(info, seed=12345):
    """Particles as Particle_Handler::Load in emoopic.hpp makes them."""
    npart = info.nparticles_tot  # the one domain holds them all (Domain, src/domain/domain.cpp:100)
    counts = [0] * info.nspecies
    ispec, cden = 0, info.dens_frac[0]
    for ip in range(npart):
        if ip >= cden * npart:
            ispec += 1
            cden += info.dens_frac[ispec]
        counts[ispec] += 1
    zero_mean = info.fields_init == b"poisson" and all(
        bytes(info.fields_bound[i]).rstrip(b"\0") == b"periodic" for i in range(6))
    parts = []
    for s in range(info.nspecies):
        g = abi.GenParams()
        g.seed = seed
        g.species = s
        g.relativistic_gamma = 1
        vth = UNIT_VTH * np.sqrt(info.temp[s] / info.mass_ratio[s])
        for d in range(3):
            g.x0[d] = info.xyz0[d]
            g.L[d] = info.Lxyz[d]
            g.vth[d] = vth
        n = counts[s]
        p = {k: np.empty(n) for k in ("x", "y", "z", "vx", "vy", "vz", "gamma")}
        abi.check(abi.lib().emoo_generate_host(C.byref(g), 0, n, *[p[k].ctypes.data_as(C.POINTER(C.c_double))
                                                                    for k in ("x", "y", "z", "vx", "vy", "vz",
                                                                              "gamma")]))
        if zero_mean:
            for k in ("vx", "vy", "vz"):
                m = 0.0
                for a in p[k].tolist():  # sequential sum, as the driver's loader
                    m += a
                m /= n
                p[k] = p[k] - m
        parts.append(p)
    return parts


@pytest.mark.parametrize("flags", [[], ["--multigrid"], ["--corrected"]])
def test_driver_history_matches_oracle(tmp_path, flags):
    """With --multigrid the driver starts from the multigrid solve (to its
    default 1e-10 residual) and the oracle from its exact solve; the fields
    then agree to about 1e-9, so the history to 1e-7. With --corrected both
    run the corrected-physics policy."""
    multigrid = "--multigrid" in flags
    build_native.build()
    src = os.path.join(DATA, "driver_small.txt")
    inp = tmp_path / "input.txt"
    shutil.copy(src, inp)
    cmd = [build_native.DRIVER, str(inp)] + flags
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = np.loadtxt(tmp_path / "history.dat", skiprows=1, ndmin=2)
    info = abi.InputInfo()
    assert abi.lib().emoo_read_input(src.encode(), C.byref(info)) == abi.OK
    assert abi.lib().emoo_process_info(C.byref(info)) == abi.OK
    dx = min(info.Lxyz[d] / info.nCell[d] for d in range(3))
    dt = dx / 100.0
    parts = reference_load(info)
    o = OracleBackend(info, dt)
    if multigrid:
        o.set_poisson_solver(1)
    if "--corrected" in flags:
        o.set_policy(1)
    nid = 0
    for s, p in enumerate(parts):
        o.add_species(s, p, ids=np.arange(nid, nid + len(p["x"])))
        nid += len(p["x"])
    o.init_fields()
    hist = []
    for ti in range(info.nt):
        c, h = o.step(ti)
        if h is not None:
            hist.append(h)
    mass = sum(info.mass_ratio[s] * len(p["x"]) for s, p in enumerate(parts))
    assert rows.shape == (len(hist), 8)
    history_close(rows, np.array(hist), 1e-7 if multigrid else 1e-9, mass)
