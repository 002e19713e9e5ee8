"""The C ABI library (no GPU work): it loads, exports every function
include/emoo.h declares, its config struct is binary-identical to the
reference's Input_Info_t, and host-only entry points behave."""
import ctypes as C
import os
import re

import numpy as np

from apc_524_project_gb300 import abi, configs, loading

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-zA-Z_][\w \*]*?\b(emoo_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = abi.lib()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_prototypes_cover_header():
    assert set(declared_functions()) == set(abi.PROTOTYPES)


def test_input_info_layout_is_the_references():
    # sizeof(Input_Info_t) of the reference built for LP64 (x86-64 / aarch64)
    assert C.sizeof(abi.InputInfo) == 4056
    assert abi.InputInfo.nparticles_tot.offset == 464
    assert abi.InputInfo.t0.offset == 480
    assert abi.InputInfo.fields_bound.offset == 4056 - 6 * 64


def test_strerror_and_default_opts():
    L = abi.lib()
    assert L.emoo_strerror(0) == b"ok"
    assert L.emoo_strerror(abi.ERR_NOT_CONVERGED).startswith(b"Poisson solve did not converge")
    o = abi.Opts()
    assert L.emoo_default_opts(C.byref(o)) == 0
    assert o.precision == abi.FP64 and o.deposit_rho == 1 and o.history_every == 10
    assert o.poisson_solver == abi.POISSON_JACOBI and o.poisson_rtol == 1e-10
    assert L.emoo_default_opts(None) == abi.ERR_ARG


def test_bad_arguments_are_rejected_without_device_work():
    L = abi.lib()
    h = C.c_void_p()
    assert L.emoo_create(None, None, C.byref(h)) == abi.ERR_ARG
    info = configs.input_info(configs.tiny())
    info.parts_bound[0] = info.parts_bound[0].__class__.from_buffer_copy(b"bogus" + b"\0" * 59)
    assert L.emoo_create(C.byref(info), None, C.byref(h)) == abi.ERR_INPUT
    info = configs.input_info(configs.tiny())
    info.nCell[1] = 0
    assert L.emoo_create(C.byref(info), None, C.byref(h)) == abi.ERR_ARG
    assert L.emoo_destroy(None) == abi.ERR_ARG


def test_host_sampler_is_deterministic_and_maxwellian():
    cfg = configs.tiny(n=(16, 16, 16), ppc=8, vth=0.1)
    a = loading.sample_species(cfg, 0)
    b = loading.sample_species(cfg, 0)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    # sub-ranges reproduce the same stream elements
    c = loading.sample_species(cfg, 0, first=100, n=50)
    np.testing.assert_array_equal(c["vx"], a["vx"][100:150])
    v = np.concatenate([a["vx"], a["vy"], a["vz"]])
    assert abs(np.mean(v)) < 5 * 0.1 / np.sqrt(v.size)
    assert abs(np.std(v) / 0.1 - 1) < 0.03
    L = cfg.L
    assert a["x"].min() >= 0 and a["x"].max() < L[0]
    # density modulation 1 + 0.2 cos(2 pi x / L): first Fourier moment 0.1
    m1 = np.mean(np.cos(2 * np.pi * a["x"] / L[0]))
    assert abs(m1 - 0.1) < 0.02
