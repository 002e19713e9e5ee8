"""Uniform test-side view of three implementations of the same loop:

  RefBackend     the compiled reference serial build (oracle/_ref, built here
                 from the reference's own sources; absent on GPU machines)
  OracleBackend  the CPU restatement in oracle/ (plain C, FP64)
  GpuBackend     the product: libemoo.so through its C ABI

All three take the same Input_Info_t, the same particle arrays and expose
fields in the reference layout ((n+3)^3, C order) and particles with their
species and id, so parity tests compare like with like.
"""
import ctypes as C
import os

import numpy as np

from apc_524_project_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libemoo_ref.so")
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "liboracle.so")

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_L = C.POINTER(C.c_long)


def dptr(a):
    return a.ctypes.data_as(_D)


def _load_cpu_lib(path, prefix):
    L = C.CDLL(path)
    P = C.c_void_p

    def f(name, res, args):
        fn = getattr(L, prefix + name)
        fn.restype = res
        fn.argtypes = args

    f("create", P, [C.POINTER(abi.InputInfo), C.c_double, C.c_double] + ([C.c_char_p] if prefix == "refh_" else []))
    f("destroy", None, [P])
    f("npoints", C.c_long, [P])
    f("add_particles", C.c_int, [P, C.c_long, _D, _D, _D, _D, _D, _D, _D, _I, _L])
    f("num_particles", C.c_long, [P])
    f("get_particles", C.c_int, [P, _D, _D, _D, _D, _D, _D, _D, _I, _L])
    f("get_particle_fields", C.c_int, [P, _D, _D, _D, _D, _D, _D])
    f("get_field", C.c_int, [P, C.c_int, _D])
    f("set_field", C.c_int, [P, C.c_int, _D])
    f("cell_id", C.c_int, [P, C.c_double, C.c_double, C.c_double])
    f("sort", C.c_int, [P])
    f("push", C.c_int, [P])
    f("particle_bc", C.c_int, [P, _L])
    f("clear_ghosts", C.c_int, [P])
    f("deposit", C.c_int, [P, C.c_int])
    f("execute_bc", C.c_int, [P, C.c_int])
    f("evolve", C.c_int, [P, C.c_int])
    f("interpolate", C.c_int, [P])
    f("step", C.c_int, [P, C.c_int, _L, _D, _I])
    f("pusher_steps", C.c_int, [C.c_int, _D, _D, C.c_double, C.c_long])
    f("history", C.c_int, [P, C.c_double, _D])
    if prefix == "refh_":
        f("init_fields", C.c_int, [P])
        f("initialize_fields_only", C.c_int, [P])
        f("set_time", None, [P, C.c_double, C.c_double])
        f("time", C.c_double, [])
    else:
        f("init_fields", C.c_int, [P, _I])
        f("initialize_fields_only", C.c_int, [P, _I])
        f("set_time", None, [P, C.c_double, C.c_double])
        f("time", C.c_double, [P])
        f("gauss_residual", C.c_int, [P, _D])
        f("set_rho_background", None, [P, C.c_double])
        f("set_wave_shape", C.c_int, [P, C.c_int, C.POINTER(abi.WaveShape)])
        f("set_rho_background_xmin", None, [P, C.c_double])
        f("set_policy", C.c_int, [P, C.c_int])
        f("set_poisson_solver", C.c_int, [P, C.c_int, C.c_double])
    return L


class CpuBackend:
    prefix = None
    path = None
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(cls.path):
                raise FileNotFoundError(cls.path)
            cls._lib = _load_cpu_lib(cls.path, cls.prefix)
        return cls._lib

    @classmethod
    def available(cls):
        return os.path.exists(cls.path)

    def _f(self, name):
        return getattr(self.lib(), self.prefix + name)

    def __init__(self, info, dt, t0=0.0, tmpdir="/tmp"):
        self.info = info
        self.dt = dt
        self.n = [info.nCell[d] for d in range(3)]
        self.shape = tuple(v + 3 for v in self.n)
        args = [C.byref(info), dt, t0]
        if self.prefix == "refh_":
            args.append(tmpdir.encode())
        self.h = self._f("create")(*args)
        if not self.h:
            raise RuntimeError("create failed")

    def close(self):
        if self.h:
            self._f("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_species(self, si, p, ids=None):
        n = len(p["x"])
        typ = np.full(n, si, dtype=np.int32)
        if ids is None:
            ids = np.arange(self.num_particles(), self.num_particles() + n, dtype=np.int64)
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        arr = [np.ascontiguousarray(p[k], dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz", "gamma")]
        rc = self._f("add_particles")(self.h, n, *[dptr(a) for a in arr], typ.ctypes.data_as(_I),
                                      ids.ctypes.data_as(_L))
        assert rc == 0

    def num_particles(self):
        return int(self._f("num_particles")(self.h))

    def particles(self):
        n = self.num_particles()
        out = {k: np.empty(n) for k in ("x", "y", "z", "vx", "vy", "vz", "gamma")}
        out["type"] = np.empty(n, dtype=np.int32)
        out["id"] = np.empty(n, dtype=np.int64)
        self._f("get_particles")(self.h, *[dptr(out[k]) for k in ("x", "y", "z", "vx", "vy", "vz", "gamma")],
                                 out["type"].ctypes.data_as(_I), out["id"].ctypes.data_as(_L))
        return out

    def particle_fields(self):
        n = self.num_particles()
        f = [np.empty(n) for _ in range(6)]
        self._f("get_particle_fields")(self.h, *[dptr(a) for a in f])
        return np.stack(f, axis=1)

    def get_field(self, fid):
        a = np.empty(self.shape)
        assert self._f("get_field")(self.h, fid, dptr(a)) == 0
        return a

    def set_field(self, fid, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.shape)
        assert self._f("set_field")(self.h, fid, dptr(a)) == 0

    def cell_id(self, x, y, z):
        return int(self._f("cell_id")(self.h, x, y, z))

    def init_fields(self):
        if self.prefix == "refh_":
            return self._f("init_fields")(self.h), None
        it = (C.c_int * 4)()
        rc = self._f("init_fields")(self.h, it)
        return rc, list(it)

    def initialize_fields_only(self):
        if self.prefix == "refh_":
            return self._f("initialize_fields_only")(self.h), None
        it = (C.c_int * 4)()
        rc = self._f("initialize_fields_only")(self.h, it)
        return rc, list(it)

    def set_time(self, t, dtp):
        self._f("set_time")(self.h, t, dtp)

    def sort(self):
        self._f("sort")(self.h)

    def push(self):
        self._f("push")(self.h)

    def particle_bc(self):
        c = (C.c_long * 6)()
        self._f("particle_bc")(self.h, c)
        self._f("clear_ghosts")(self.h)
        return list(c)

    def deposit(self, with_rho=True):
        self._f("deposit")(self.h, 1 if with_rho else 0)

    def execute_bc(self, sid):
        self._f("execute_bc")(self.h, sid)

    def evolve(self, es=False):
        self._f("evolve")(self.h, 1 if es else 0)

    def interpolate(self):
        self._f("interpolate")(self.h)

    def step(self, ti):
        c = (C.c_long * 6)()
        hist = (C.c_double * 8)()
        w = C.c_int(0)
        self._f("step")(self.h, ti, c, hist, C.byref(w))
        return list(c), (list(hist) if w.value else None)

    def history(self, t):
        out = (C.c_double * 8)()
        assert self._f("history")(self.h, t, out) == 0
        return list(out)

    @classmethod
    def pusher_steps(cls, relativistic, state, field, dt, nsteps):
        st = np.ascontiguousarray(state, dtype=np.float64).copy()
        fl = np.ascontiguousarray(field, dtype=np.float64)
        getattr(cls.lib(), cls.prefix + "pusher_steps")(1 if relativistic else 0, dptr(st), dptr(fl), dt, nsteps)
        return st


class RefBackend(CpuBackend):
    prefix = "refh_"
    path = REF_LIB


class OracleBackend(CpuBackend):
    @classmethod
    def generator(cls):
        """The oracle's copy of the seeded sampler (orc_generate), for
        loading.sample_species(generate=...) without the product library."""
        fn = cls.lib().orc_generate
        fn.restype = C.c_int
        fn.argtypes = [C.POINTER(abi.GenParams), C.c_int64, C.c_int64, _D, _D, _D, _D, _D, _D, _D]
        return fn

    prefix = "orc_"
    path = ORACLE_LIB

    def gauss_residual(self):
        out = (C.c_double * 2)()
        self._f("gauss_residual")(self.h, out)
        return list(out)

    def set_rho_background(self, v, xmin=None):
        self._f("set_rho_background")(self.h, C.c_double(v))
        if xmin is not None:
            self._f("set_rho_background_xmin")(self.h, C.c_double(xmin))

    def set_wave_shape(self, w, shape):
        rc = self._f("set_wave_shape")(self.h, w, C.byref(shape) if shape is not None else None)
        if rc != 0:
            raise ValueError("orc_set_wave_shape refused the shape")

    def set_policy(self, policy):
        if self._f("set_policy")(self.h, policy) != 0:
            raise ValueError("orc_set_policy refused the policy")

    def set_poisson_solver(self, solver, rtol=1e-13):
        if self._f("set_poisson_solver")(self.h, solver, rtol) != 0:
            raise ValueError("orc_set_poisson_solver refused the solver")


class GpuBackend:
    """The product, through include/emoo.h."""

    def __init__(self, info, dt, t0=0.0, precision=abi.FP64, capacity=0, track_ids=1, device=0, rho_background=0.0,
                 rho_background_xmin=None, policy=abi.POLICY_REFERENCE, poisson_solver=abi.POISSON_JACOBI,
                 poisson_rtol=None):
        self.L = abi.lib()
        self.info = info
        self.n = [info.nCell[d] for d in range(3)]
        self.shape = tuple(v + 3 for v in self.n)
        o = abi.Opts()
        self.L.emoo_default_opts(C.byref(o))
        o.precision = precision
        o.dt = dt
        o.capacity = capacity
        o.track_ids = track_ids
        o.device = device
        o.rho_background = rho_background
        if rho_background_xmin is not None:
            o.rho_background_xmin = rho_background_xmin
        o.policy = policy
        o.poisson_solver = poisson_solver
        if poisson_rtol is not None:
            o.poisson_rtol = poisson_rtol
        h = C.c_void_p()
        abi.check(self.L.emoo_create(C.byref(info), C.byref(o), C.byref(h)), "emoo_create")
        self.h = h
        self.nspec = info.nspecies

    def close(self):
        if self.h:
            self.L.emoo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_species(self, si, p, ids=None):
        n = len(p["x"])
        arr = [np.ascontiguousarray(p[k], dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz", "gamma")]
        idp = None
        if ids is not None:
            ids = np.ascontiguousarray(ids, dtype=np.int64)
            idp = ids.ctypes.data_as(C.POINTER(C.c_int64))
        abi.check(self.L.emoo_load_particles(self.h, si, n, *[dptr(a) for a in arr], idp), "emoo_load_particles")

    def num_particles(self, species=-1):
        n = C.c_int64()
        abi.check(self.L.emoo_num_particles(self.h, species, C.byref(n)))
        return n.value

    def particles(self):
        parts = []
        for s in range(self.nspec):
            n = self.num_particles(s)
            out = {k: np.empty(n) for k in ("x", "y", "z", "vx", "vy", "vz", "gamma")}
            out["id"] = np.empty(n, dtype=np.int64)
            got = C.c_int64()
            abi.check(self.L.emoo_get_particles(self.h, s, n, *[dptr(out[k]) for k in
                                                                ("x", "y", "z", "vx", "vy", "vz", "gamma")],
                                                out["id"].ctypes.data_as(C.POINTER(C.c_int64)), C.byref(got)))
            out["type"] = np.full(n, s, dtype=np.int32)
            parts.append(out)
        return {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}

    def particle_fields(self):
        cols = []
        for s in range(self.nspec):
            n = self.num_particles(s)
            f = [np.empty(n) for _ in range(6)]
            got = C.c_int64()
            abi.check(self.L.emoo_get_particle_fields(self.h, s, n, *[dptr(a) for a in f], C.byref(got)))
            cols.append(np.stack(f, axis=1))
        return np.concatenate(cols, axis=0)

    def get_field(self, fid):
        a = np.empty(self.shape)
        abi.check(self.L.emoo_get_field(self.h, fid, dptr(a)), "emoo_get_field")
        return a

    def set_field(self, fid, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.shape)
        abi.check(self.L.emoo_set_field(self.h, fid, dptr(a)), "emoo_set_field")

    def cell_id(self, x, y, z):
        c = C.c_int()
        abi.check(self.L.emoo_cell_id(self.h, x, y, z, C.byref(c)))
        return c.value

    def set_wave_shape(self, w, shape):
        abi.check(self.L.emoo_set_wave_shape(self.h, w, C.byref(shape) if shape is not None else None),
                  "emoo_set_wave_shape")

    def init_fields(self):
        it = (C.c_int * 4)()
        rc = self.L.emoo_init_fields(self.h, it)
        return rc, list(it)

    def poisson_init(self):
        it = (C.c_int * 4)()
        rc = self.L.emoo_poisson_init(self.h, it)
        return rc, list(it)

    def sort(self):
        abi.check(self.L.emoo_sort(self.h), "emoo_sort")

    def interpolate(self):
        abi.check(self.L.emoo_interpolate(self.h), "emoo_interpolate")

    def push(self):
        abi.check(self.L.emoo_push(self.h), "emoo_push")

    def particle_bc(self):
        c = (C.c_int64 * 6)()
        abi.check(self.L.emoo_apply_particle_bc(self.h, c), "emoo_apply_particle_bc")
        return list(c)

    def deposit(self, with_rho=True):
        abi.check(self.L.emoo_deposit(self.h, 1 if with_rho else 0), "emoo_deposit")

    def execute_bc(self, sid):
        abi.check(self.L.emoo_execute_bc(self.h, sid), "emoo_execute_bc")

    def evolve(self, es=False):
        abi.check(self.L.emoo_evolve_fields(self.h, 1 if es else 0), "emoo_evolve_fields")

    def step(self, nsteps=1):
        c = (C.c_int64 * 6)()
        abi.check(self.L.emoo_step(self.h, nsteps, c), "emoo_step")
        return list(c)

    def history(self):
        out = (C.c_double * 8)()
        abi.check(self.L.emoo_history(self.h, out))
        return list(out)

    def history_rows(self):
        n = C.c_int()
        self.L.emoo_history_rows(self.h, 0, None, C.byref(n))
        rows = np.empty((n.value, 8))
        if n.value:
            self.L.emoo_history_rows(self.h, n.value, dptr(rows), C.byref(n))
        return rows

    def gauss_residual(self):
        out = (C.c_double * 2)()
        abi.check(self.L.emoo_gauss_residual(self.h, out))
        return list(out)

    def check(self):
        return self.L.emoo_check(self.h)


def by_id(parts):
    """Particle arrays reordered by id (the three implementations order
    particles differently)."""
    o = np.argsort(parts["id"], kind="stable")
    return {k: v[o] for k, v in parts.items()}


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.sqrt(np.sum(b * b))
    num = np.sqrt(np.sum((a - b) ** 2))
    if den == 0.0:
        return float(num)
    return float(num / den)
