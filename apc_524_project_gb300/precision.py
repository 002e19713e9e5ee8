"""The mixed form's error, stated against the FP64 form.

The mixed form is the FP64 form's algorithm with FP32 state and arithmetic,
so what it has to show is that its results differ from the FP64 form's by
what FP32 rounding alone does to this loop - not by a fault. On a thermal
plasma that is not a fixed number: particle orbits separate from any
perturbation, and any two runs drift apart as the run goes on (the FP64
form reacts the same way to a change in the last bits). The bar is
therefore measured, not assumed: an ensemble of FP64 runs, each perturbed
after every step at the size of the mixed form's rounding (emoo_perturb: a
relative amount on every velocity component and field value, that fraction
of a cell on every position component), shows how far rounding of that size
moves the result at each step; the mixed form's distance from the
unperturbed FP64 run is stated next to that spread.

The size of that perturbation is the mixed form's own rounding per step,
measured: calibrate() runs one step of both forms from the same state and
takes the RMS relative difference of the particles' velocities (the push is a
few dozen FP32 operations with hardware reciprocal square roots, so the
mixed form errs by a few ulps a step, not by one); the perturbation
amplitude is sqrt(3) times that (uniform noise in [-1, 1) has RMS 1/sqrt(3)),
and never below 2^-24.

measure() returns, at each checkpoint step, the relative L2 distance of E, B
and J between the mixed and the FP64 run, the ensemble members' mean and
largest distance from the FP64 run, and the ratio of the mixed distance to
the largest (the mixed run is one more sample of rounding of that size; a
few particles that end a step within rounding of a cell face can dominate
a small case, so the largest member is the yardstick); and, from the history rows and the Gauss-law
residual, the field energy, kinetic energy, total energy and residual norm
of every run, each observable's mixed-vs-FP64 relative difference with the
ensemble's, and each form's total-energy drift.
"""
import ctypes as C

import numpy as np

from . import abi, configs

FP32_ROUNDING = 2.0 ** -24


def _handle(cfg, precision, policy, device, poisson_solver=0, track_ids=0):
    L = abi.lib()
    info = configs.input_info(cfg)
    o = abi.Opts()
    L.emoo_default_opts(C.byref(o))
    o.precision = precision
    o.policy = policy
    o.poisson_solver = poisson_solver
    o.dt = cfg.dt
    o.capacity = cfg.total_particles()
    o.track_ids = track_ids
    o.device = device
    o.rho_background = configs.rho_background(cfg)
    h = C.c_void_p()
    abi.check(L.emoo_create(C.byref(info), C.byref(o), C.byref(h)), "emoo_create")
    for si in range(len(cfg.species)):
        g = configs.gen_params(cfg, si)
        abi.check(L.emoo_load_generated(h, C.byref(g), cfg.count(cfg.species[si])), "emoo_load_generated")
    it = (C.c_int * 4)()
    rc = L.emoo_init_fields(h, it)
    if rc not in (abi.OK, abi.ERR_NOT_CONVERGED):
        abi.check(rc, "emoo_init_fields")
    return h


_GROUPS = {"E": (abi.EX, abi.EY, abi.EZ), "B": (abi.BX, abi.BY, abi.BZ), "J": (abi.JX, abi.JY, abi.JZ)}


def _snapshot(h, shape):
    """E, B and J over the physical points (the ghost planes hold copies, or
    after a fold whatever each form's deposit left there, which the loop does
    not read), the Gauss-law residual norm and the history row's energies."""
    L = abi.lib()
    out = {}
    phys = tuple(slice(1, m - 2) for m in shape)
    for name, ids in _GROUPS.items():
        parts = []
        for i in ids:
            a = np.empty(shape)
            abi.check(L.emoo_get_field(h, i, a.ctypes.data_as(C.POINTER(C.c_double))), "emoo_get_field")
            parts.append(a[phys].ravel())
        out[name] = np.concatenate(parts)
    r = (C.c_double * 2)()
    abi.check(L.emoo_gauss_residual(h, r), "emoo_gauss_residual")
    out["gauss_l2"] = float(r[1])
    row = (C.c_double * 8)()
    abi.check(L.emoo_history(h, row), "emoo_history")
    out["field_energy"] = float(row[5] + row[6])
    out["kinetic_energy"] = float(row[4])
    out["total_energy"] = float(row[7])
    return out


def _run(cfg, precision, policy, steps_at, device, perturb_seed=None, rel=FP32_ROUNDING):
    L = abi.lib()
    h = _handle(cfg, precision, policy, device)
    shape = tuple(v + 3 for v in cfg.n)
    snaps = {0: _snapshot(h, shape)}
    cnt = (C.c_int64 * 6)()
    if perturb_seed is not None:  # the mixed form rounds the state it loads, too
        abi.check(L.emoo_perturb(h, perturb_seed * 1000003, rel), "emoo_perturb")
    for t in range(1, max(steps_at) + 1):
        abi.check(L.emoo_step(h, 1, cnt), "emoo_step")
        if perturb_seed is not None:
            abi.check(L.emoo_perturb(h, perturb_seed * 1000003 + t, rel), "emoo_perturb")
        if t in steps_at:
            snaps[t] = _snapshot(h, shape)
    abi.check(L.emoo_check(h), "device error word")
    abi.check(L.emoo_destroy(h))
    return snaps


def _velocities_by_id(h, nspec):
    L = abi.lib()
    P = C.POINTER(C.c_double)
    vs, idl = [], []
    for sp in range(nspec):
        n = C.c_int64()
        abi.check(L.emoo_num_particles(h, sp, C.byref(n)))
        out = {k: np.empty(n.value) for k in ("x", "y", "z", "vx", "vy", "vz", "g")}
        ids = np.empty(n.value, dtype=np.int64)
        got = C.c_int64()
        abi.check(L.emoo_get_particles(h, sp, n.value, *(out[k].ctypes.data_as(P) for k in
                                                          ("x", "y", "z", "vx", "vy", "vz", "g")),
                                       ids.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(got)), "emoo_get_particles")
        vs.append(np.stack([out["vx"], out["vy"], out["vz"]], axis=1))
        idl.append(ids)
    v, ids = np.concatenate(vs), np.concatenate(idl)
    return v[np.argsort(ids)]


def calibrate(cfg, policy=1, device=0):
    """The mixed form's rounding per step, measured: RMS over particles of
    |v_mixed - v_fp64| / |v_fp64| after one step from the same particles
    and field start. Returns the ensemble perturbation amplitude
    max(2^-24, sqrt(3) RMS)."""
    L = abi.lib()
    vs = []
    for prec in (abi.FP64, abi.MIXED):
        h = _handle(cfg, prec, policy, device, track_ids=1)
        cnt = (C.c_int64 * 6)()
        abi.check(L.emoo_step(h, 1, cnt), "emoo_step")
        vs.append(_velocities_by_id(h, len(cfg.species)))
        abi.check(L.emoo_destroy(h))
    f, m = vs
    nf = np.sqrt(np.sum(f * f, axis=1))
    ok = nf > 0
    r = np.sqrt(np.sum((m - f) ** 2, axis=1))[ok] / nf[ok]
    rms = float(np.sqrt(np.mean(r * r))) if r.size else 0.0
    return max(FP32_ROUNDING, float(np.sqrt(3.0)) * rms)


def rel_l2(a, b):
    d = float(np.sqrt(np.sum((a - b) ** 2)))
    n = float(np.sqrt(np.sum(b * b)))
    return d / n if n > 0 else d


def measure(cfg, steps_at=(10, 50, 100), members=6, policy=1, device=0, rel=None):
    """Mixed and FP64 runs of cfg from the same particles and field start,
    plus `members` FP64 runs perturbed after every step by emoo_perturb(rel)
    (rel None: calibrate()); policy: abi.POLICY_CORRECTED (1) by default, the
    scheme that stays stable over the run (the reference policy's field
    energy grows without bound)."""
    steps_at = tuple(sorted(steps_at))
    if rel is None:
        rel = calibrate(cfg, policy, device)
    ref = _run(cfg, abi.FP64, policy, steps_at, device)
    mix = _run(cfg, abi.MIXED, policy, steps_at, device)
    ens = [_run(cfg, abi.FP64, policy, steps_at, device, perturb_seed=k + 1, rel=rel) for k in range(members)]
    out = {"steps": list(steps_at), "members": members, "perturbation": rel, "fields": {}, "observables": {}}
    for t in steps_at:
        row = {}
        for name in _GROUPS:
            err = rel_l2(mix[t][name], ref[t][name])
            d = [rel_l2(e[t][name], ref[t][name]) for e in ens]
            row[name] = {"mixed": err, "spread_mean": float(np.mean(d)), "spread_max": float(np.max(d)),
                         "ratio": err / float(np.max(d)) if np.max(d) > 0 else None}
        out["fields"][str(t)] = row
        obs = {}
        for name in ("field_energy", "kinetic_energy", "total_energy", "gauss_l2"):
            r = ref[t][name]
            dm = abs(mix[t][name] - r) / abs(r) if r else abs(mix[t][name])
            de = float(np.mean([abs(e[t][name] - r) / abs(r) if r else abs(e[t][name]) for e in ens]))
            obs[name] = {"fp64": r, "mixed": mix[t][name], "rel_diff": dm, "spread": de}
        out["observables"][str(t)] = obs
    t0, t1, tl = 0, steps_at[0], steps_at[-1]

    def drift(s, a):
        return abs(s[tl]["total_energy"] - s[a]["total_energy"]) / abs(s[a]["total_energy"])

    out["energy_drift"] = {
        "fp64_from_0": drift(ref, t0), "mixed_from_0": drift(mix, t0),
        f"fp64_from_{t1}": drift(ref, t1), f"mixed_from_{t1}": drift(mix, t1),
    }
    return out


def drift_vs_debye(cfg, omegas=(0.5, 0.2, 0.1), steps=100, start=10, policy=1, device=0):
    """Total-energy drift of cfg over steps start..steps in both forms at each
    plasma frequency in `omegas` (the electron Debye length in cells is
    v_th / omega_pe / dx). A drift that falls as lambda_D/dx grows, equally in
    both forms, is the explicit scheme's grid heating, not the form's rounding."""
    import dataclasses

    L = abi.lib()
    cnt = (C.c_int64 * 6)()
    vth, dx = cfg.species[0].vth, min(cfg.dx)
    rows = []
    for w in omegas:
        c = dataclasses.replace(cfg, omega_pe=w)
        row = {"omega_pe": w, "lambda_D_over_dx": vth / w / dx}
        for prec, name in ((abi.FP64, "fp64"), (abi.MIXED, "mixed")):
            h = _handle(c, prec, policy, device)
            tot = {}
            for t in range(steps + 1):
                if t in (0, start, steps):
                    r = (C.c_double * 8)()
                    abi.check(L.emoo_history(h, r), "emoo_history")
                    tot[t] = float(r[7])
                if t < steps:
                    abi.check(L.emoo_step(h, 1, cnt), "emoo_step")
            abi.check(L.emoo_check(h), "device error word")
            abi.check(L.emoo_destroy(h))
            row[f"{name}_from_{start}"] = abs(tot[steps] - tot[start]) / abs(tot[start])
            row[f"{name}_from_0"] = abs(tot[steps] - tot[0]) / abs(tot[0])
        rows.append(row)
    return rows
