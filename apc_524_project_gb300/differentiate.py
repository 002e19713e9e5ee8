"""Differentiation of the time loop: a thin harness over emoo_ad_run.

A Problem holds a workload and its initial particles. Every evaluation
builds a fresh handle (FP64, or the mixed-precision form: objective and
adjoint only; the reference policy or, FP64 only, the corrected one), loads
the particles with the velocity perturbation dv added (gamma kept), sets
the wave amplitudes and phases and the wave shapes (with the envelope
coefficients from theta), starts the fields and runs emoo_ad_run:

  * objective(theta, dv)            the objective alone (the primal loop)
  * tangent(theta, dv, dtheta, ddv) the objective's derivative along a direction
  * gradient(theta, dv)             the objective and its adjoint gradient

theta = (amp_0, phase_0 [degrees], amp_1, phase_1, ...), followed, when a
wave has a sine-series envelope, by 16 envelope coefficients per wave;
dv has shape (3, N) in the particles' load order. The objective is the
field energy of the x slab `slab` (cells), or with objective="kinetic" the
kinetic energy of the particles of `species` (-1: all) in that x range.
PicObjective wraps gradient() as a torch.autograd.Function for optimisation
loops; the C++ driver reaches the same kernels through include/emoo.h."""
import ctypes as C

import numpy as np

from . import abi, configs, loading


class Problem:
    def __init__(self, cfg, nsteps=None, slab=(48, 56), checkpoint_every=16, parts=None, objective="field",
                 species=-1, precision=abi.FP64, policy=abi.POLICY_REFERENCE):
        self.cfg = cfg
        self.policy = policy
        self.info0 = configs.input_info(cfg)
        self.nsteps = cfg.steps if nsteps is None else nsteps
        self.slab = slab
        self.every = checkpoint_every
        self.kind = {"field": abi.AD_OBJ_FIELD, "kinetic": abi.AD_OBJ_KINETIC}[objective]
        self.species = species
        self.precision = precision
        self.parts = parts if parts is not None else loading.sample_all(cfg)
        self.np = sum(len(p["x"]) for p in self.parts)
        nw = len(cfg.waves)
        self.series = any(w.shape is not None and len(w.shape.coef) > 0 for w in cfg.waves)
        th = [v for w in cfg.waves for v in (w.amp, w.phase_deg)]
        if self.series:
            for w in cfg.waves:
                c = list(w.shape.coef) if w.shape is not None else []
                th += c + [0.0] * (abi.NCOEF - len(c))
        self.theta0 = np.array(th, dtype=np.float64)
        self.ntheta = len(th)
        self.nwaves = nw

    # ---- one run on a fresh handle
    def _run(self, mode, theta, dv, dtheta=None, ddv=None, want_grad=False):
        L = abi.lib()
        info = configs.input_info(self.cfg)
        o = abi.Opts()
        L.emoo_default_opts(C.byref(o))
        o.precision = self.precision
        o.policy = self.policy
        o.dt = self.cfg.dt
        o.capacity = self.np
        o.rho_background = configs.rho_background(self.cfg)
        xmin = configs.rho_background_xmin(self.cfg)
        if xmin is not None:
            o.rho_background_xmin = xmin
        h = C.c_void_p()
        abi.check(L.emoo_create(C.byref(info), C.byref(o), C.byref(h)), "emoo_create")
        try:
            off = 0
            for si, p in enumerate(self.parts):
                n = len(p["x"])
                arr = {k: np.ascontiguousarray(p[k], dtype=np.float64) for k in ("x", "y", "z", "vx", "vy", "vz")}
                if dv is not None:
                    for a, k in enumerate(("vx", "vy", "vz")):
                        arr[k] = arr[k] + dv[a, off:off + n]
                g = np.ascontiguousarray(p.get("gamma", np.zeros(n)), dtype=np.float64)
                ptr = [arr[k].ctypes.data_as(C.POINTER(C.c_double)) for k in ("x", "y", "z", "vx", "vy", "vz")]
                abi.check(L.emoo_load_particles(h, si, n, *ptr, g.ctypes.data_as(C.POINTER(C.c_double)), None),
                          "emoo_load_particles")
                off += n
            nw = len(self.cfg.waves)
            if nw:
                th = np.asarray(theta, dtype=np.float64)
                amp = np.ascontiguousarray(th[0:2 * nw:2])
                pha = np.ascontiguousarray(th[1:2 * nw:2])
                abi.check(L.emoo_set_waves(h, nw, amp.ctypes.data_as(C.POINTER(C.c_double)),
                                           pha.ctypes.data_as(C.POINTER(C.c_double))), "emoo_set_waves")
                for w, wv in enumerate(self.cfg.waves):
                    if wv.shape is None:
                        continue
                    coef = None
                    if self.series and len(wv.shape.coef):
                        base = 2 * nw + abi.NCOEF * w
                        coef = th[base:base + len(wv.shape.coef)]
                    shape = configs.wave_shape(self.cfg, w, coef)
                    abi.check(L.emoo_set_wave_shape(h, w, C.byref(shape)), "emoo_set_wave_shape")
            assert L.emoo_ad_nparams(h) == self.ntheta
            it = (C.c_int * 4)()
            abi.check(L.emoo_init_fields(h, it), "emoo_init_fields")
            spec = abi.AdSpec(self.nsteps, self.every, self.slab[0], self.slab[1], self.kind, self.species)
            res = abi.AdResult()
            dp = C.POINTER(C.c_double)
            dth = ddvp = None
            if dtheta is not None:
                dth_arr = np.ascontiguousarray(dtheta, dtype=np.float64)
                dth = dth_arr.ctypes.data_as(dp)
            if ddv is not None:
                ddv_arr = np.ascontiguousarray(ddv, dtype=np.float64).reshape(3, self.np)
                ddvp = ddv_arr.ctypes.data_as(dp)
            gth = np.zeros(max(1, self.ntheta))
            gv = np.zeros((3, self.np))
            abi.check(L.emoo_ad_run(h, C.byref(spec), mode, dth, ddvp, C.byref(res),
                                    gth.ctypes.data_as(dp) if want_grad else None,
                                    gv.ctypes.data_as(dp) if want_grad else None), "emoo_ad_run")
            out = {"objective": res.objective, "tangent": res.tangent, "forward_ms": res.forward_ms,
                   "recompute_ms": res.recompute_ms, "reverse_ms": res.reverse_ms}
            if self.precision == abi.MIXED and mode == abi.AD_ADJOINT:
                st = abi.Stats()
                abi.check(L.emoo_get_stats(h, C.byref(st)), "emoo_get_stats")
                out["cell_mismatch"] = st.ad_cell_mismatch
            if want_grad:
                out["grad_theta"] = gth[:self.ntheta]
                out["grad_v"] = gv
            return out
        finally:
            L.emoo_destroy(h)

    def objective(self, theta=None, dv=None):
        return self._run(abi.AD_FORWARD, self.theta0 if theta is None else theta, dv)["objective"]

    def tangent(self, dtheta, ddv, theta=None, dv=None):
        return self._run(abi.AD_TANGENT, self.theta0 if theta is None else theta, dv, dtheta, ddv)

    def gradient(self, theta=None, dv=None):
        return self._run(abi.AD_ADJOINT, self.theta0 if theta is None else theta, dv, want_grad=True)


def pic_objective():
    """The torch.autograd.Function (built on first use: torch is optional
    for the rest of the package)."""
    import torch

    class PicObjective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, dv, problem):
            r = problem.gradient(theta.detach().cpu().numpy().astype(np.float64),
                                 dv.detach().cpu().numpy().astype(np.float64))
            ctx.save_for_backward(torch.as_tensor(r["grad_theta"], dtype=theta.dtype),
                                  torch.as_tensor(r["grad_v"], dtype=dv.dtype))
            return torch.tensor(r["objective"], dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            gth, gv = ctx.saved_tensors
            return g * gth, g * gv, None

    return PicObjective
