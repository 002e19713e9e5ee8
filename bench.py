"""Throughput of the PIC time loop on the thermal-plasma workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the project's plain-vs-mixed configuration): periodic 256^3 cells,
dx = 1, dt = 0.5, electrons + ions (mass ratio 1836), 16 particles per cell
per species = 536,870,912 particles, Maxwellian with electron v_th = 0.1c,
relativistic Boris push, linear weights, particles re-sorted by cell every 20
steps. One step = one pass of the loop (sort at its cadence, history every 10
steps, fused gather+push+boundary+deposit, fold, Yee E/B update, ghost fill)
over every particle. `value` is particle-steps/s of the mixed-precision form
with the state resident in HBM; the FP64 form is timed beside it; `e2e` runs
the same steps through the C ABI with the particle state in host memory
(uploaded and read back every step).

--impl reference times the reference algorithm on the host cores: the CPU
restatement of the reference serial loop (oracle/, FP64, one process per
core, each on an independent 32^3 x 32 ppc box - the reference's own MPI
decomposition with its communication left out).
"""
import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0
METRIC = "particle-steps/s/GPU"
UNIT = "particle-steps/s"


# Host link, both directions at once (a kernel reading and writing pinned host
# memory concurrently), measured on these GB300 nodes: 167 GB/s each way.
HOST_LINK_DUPLEX_GBS = 334.0


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-laser512", action="store_true")
    ap.add_argument("--no-poisson", action="store_true")
    ap.add_argument("--no-corrected", action="store_true")
    ap.add_argument("--no-mixed-error", action="store_true")
    ap.add_argument("--no-full-run", action="store_true")
    ap.add_argument("--no-cadence", action="store_true")
    ap.add_argument("--only", choices=["poisson", "twostream", "adjoint", "mixed_error"], default=None,
                    help="run one side measurement alone and print its JSON line")
    ap.add_argument("--ad-policy", choices=["reference", "corrected"], default="corrected",
                    help="--only adjoint: the policy differentiated")
    ap.add_argument("--ad-steps", type=int, default=128, help="--only adjoint: the horizon")
    ap.add_argument("--cpu-procs", type=int, default=0)
    ap.add_argument("--cpu-steps", type=int, default=6)
    return ap.parse_args()


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def _traffic_per_unit():
    """DRAM bytes per particle of the fused kernel from the committed ncu
    summary (profiles/fused_mixed_thermal.json), if present."""
    p = os.path.join(ROOT, "profiles", "fused_mixed_thermal.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return None
    return None


def workload(size):
    from apc_524_project_gb300 import configs

    cfg = configs.thermal256(size)
    return cfg


def workload_desc(cfg):
    n = cfg.n
    return (f"thermal plasma {n[0]}x{n[1]}x{n[2]} cells, 2 species x 16 ppc = {cfg.total_particles():,} particles, "
            f"relativistic Boris, dt {cfg.dt}, sort every {cfg.nstep_sort}")


# ------------------------------------------------------------------ clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ GPU arms

def _make_handle(cfg, precision, capacity, device, poisson_solver=0, policy=0):
    from apc_524_project_gb300 import abi, configs

    L = abi.lib()
    info = configs.input_info(cfg)
    o = abi.Opts()
    L.emoo_default_opts(C.byref(o))
    o.precision = precision
    o.poisson_solver = poisson_solver
    o.policy = policy
    o.dt = cfg.dt
    o.capacity = capacity
    o.track_ids = 0
    o.device = device
    o.rho_background = configs.rho_background(cfg)
    xmin = configs.rho_background_xmin(cfg)
    if xmin is not None:
        o.rho_background_xmin = xmin
    h = C.c_void_p()
    abi.check(L.emoo_create(C.byref(info), C.byref(o), C.byref(h)), "emoo_create")
    for w in range(len(cfg.waves)):
        shape = configs.wave_shape(cfg, w)
        if shape is not None:
            abi.check(L.emoo_set_wave_shape(h, w, C.byref(shape)), "emoo_set_wave_shape")
    for si in range(len(cfg.species)):
        g = configs.gen_params(cfg, si)
        abi.check(L.emoo_load_generated(h, C.byref(g), cfg.count(cfg.species[si])), "emoo_load_generated")
    it = (C.c_int * 4)()
    rc = L.emoo_init_fields(h, it)
    if rc not in (abi.OK, abi.ERR_NOT_CONVERGED):
        abi.check(rc, "emoo_init_fields")
    return h


def _stream_of(h):
    import torch
    from apc_524_project_gb300 import abi

    s = C.c_void_p()
    abi.check(abi.lib().emoo_get_stream(h, C.byref(s)))
    return torch.cuda.ExternalStream(s.value)


def _timed_steps(h, steps, dist_barrier):
    """CUDA-event time of `steps` loop steps on the handle's stream."""
    import torch
    from apc_524_project_gb300 import abi

    L = abi.lib()
    st = _stream_of(h)
    dist_barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    cnt = (C.c_int64 * 6)()
    abi.check(L.emoo_step(h, steps, cnt), "emoo_step")
    e1.record(st)
    torch.cuda.synchronize()
    dist_barrier()
    return e0.elapsed_time(e1) / 1e3


def run_gpu_arm(args, rank, world, dist_barrier, dist_max):
    import torch
    from apc_524_project_gb300 import abi

    L = abi.lib()
    device = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(device)
    cfg = workload(args.size)
    N = cfg.total_particles()
    res = {}

    # ---- mixed form: the headline
    h = _make_handle(cfg, abi.MIXED, N, device)
    cnt = (C.c_int64 * 6)()
    for _ in range(args.warmup):
        abi.check(L.emoo_step(h, 1, cnt), "emoo_step")
    torch.cuda.synchronize()
    stats0 = abi.Stats()
    abi.check(L.emoo_set_profiling(h, 1))
    abi.check(L.emoo_get_stats(h, C.byref(stats0)))
    clk = ClockSampler(device)
    clk.start()
    t = _timed_steps(h, args.steps, dist_barrier)
    clocks = clk.stop()
    t = dist_max(t)
    stats = abi.Stats()
    abi.check(L.emoo_get_stats(h, C.byref(stats)))
    launches = int(stats.launches - stats0.launches)
    fused_ms = stats.timed_ms / max(1, stats.timed_launches)
    res["mixed"] = {"t": t, "fused_ms": fused_ms, "launches": launches, "clocks": clocks}

    # ---- one stable sort of the drifted particle state (part of the loop
    # every nstep_sort steps; timed alone here to show its share): the steps
    # up to the next sort first, so that the store has drifted as long as the
    # loop's own sort sees it. Reading rho first deposits the charge density
    # the steps left pending, which emoo_sort would otherwise do before
    # sorting (the loop's own sort does not).
    import numpy as np

    if cfg.nstep_sort > 0:
        more = (-(args.warmup + args.steps)) % cfg.nstep_sort
        if more:
            abi.check(L.emoo_step(h, more, cnt), "emoo_step")
        res["sort_drift_steps"] = cfg.nstep_sort
    rho = np.empty(tuple(v + 3 for v in cfg.n))
    abi.check(L.emoo_get_field(h, abi.RHO, rho.ctypes.data_as(C.POINTER(C.c_double))), "emoo_get_field")
    st = _stream_of(h)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    abi.check(L.emoo_sort(h), "emoo_sort")
    e1.record(st)
    torch.cuda.synchronize()
    res["sort_ms"] = e0.elapsed_time(e1)

    # ---- e2e through the C ABI with host-resident particle state
    if not args.no_e2e:
        res["e2e"] = _e2e(h, cfg, args.e2e_steps, dist_barrier, dist_max)
    abi.check(L.emoo_destroy(h))
    torch.cuda.synchronize()

    # ---- FP64 form
    if not args.no_fp64:
        h = _make_handle(cfg, abi.FP64, N, device)
        for _ in range(min(args.warmup, 2)):
            abi.check(L.emoo_step(h, 1, cnt), "emoo_step")
        abi.check(L.emoo_set_profiling(h, 1))
        t64 = dist_max(_timed_steps(h, args.fp64_steps, dist_barrier))
        s64 = abi.Stats()
        abi.check(L.emoo_get_stats(h, C.byref(s64)))
        res["fp64"] = {"t": t64, "fused_ms": s64.timed_ms / max(1, s64.timed_launches)}
        abi.check(L.emoo_destroy(h))

    # ---- differentiation: adjoint against forward cost on the laser workload
    if not args.no_adjoint:
        res["adjoint"] = adjoint_arm()
    if not args.no_laser512:
        res["laser512"] = laser512_arm(device)
    if not args.no_corrected:
        res["corrected"] = corrected_arm(cfg, args, device)
    if not args.no_cadence:
        res["sort_cadence"] = cadence_arm(cfg, device)
    if not args.no_poisson:
        res["poisson"] = poisson_arm(device)
    if not args.no_mixed_error:
        res["mixed_error"] = mixed_error_arm(device)
    return cfg, res


def mixed_error_arm(device, n=64, members=6):
    """The mixed form's error against the FP64 form on the benchmark's physics
    (thermal plasma, 32 particles per cell, v_th 0.1c, dt 0.5) at n^3 cells,
    100 steps under the corrected policy, next to the distances of an FP64
    ensemble perturbed after every step by the mixed form's measured one-step
    rounding."""
    from apc_524_project_gb300 import abi, configs, precision

    cfg = configs.thermal256(n=n)
    t0 = time.perf_counter()
    r = precision.measure(cfg, steps_at=(10, 50, 100), members=members, policy=abi.POLICY_CORRECTED, device=device)
    r["workload"] = (f"thermal plasma {n}^3 cells, {cfg.total_particles():,} particles (2 species x 16 ppc), "
                     "v_th 0.1c, relativistic, dt 0.5, sort every 20, corrected policy, 100 steps")
    # the drift at the workload's density (lambda_D = 0.2 dx) next to thinner plasmas
    r["drift_vs_debye"] = precision.drift_vs_debye(cfg, omegas=(0.5, 0.2, 0.1), policy=abi.POLICY_CORRECTED,
                                                   device=device)
    r["seconds"] = time.perf_counter() - t0
    worst = max(v["mixed"] for row in r["fields"].values() for v in row.values())
    worst_ratio = max(v["ratio"] or 0.0 for row in r["fields"].values() for v in row.values())
    worst_obs = max(o["rel_diff"] for row in r["observables"].values()
                    for k, o in row.items() if k in ("field_energy", "kinetic_energy", "gauss_l2"))
    r["summary"] = {
        "max_rel_l2_EBJ": worst, "max_ratio_to_largest_ensemble_member": worst_ratio,
        "max_observable_rel_diff": worst_obs,
        "target_rel_l2_1e-4_after_100_steps": worst <= 1e-4,
        "target_observables_1e-4": worst_obs <= 1e-4,
        "target_energy_drift_1e-3": r["energy_drift"]["mixed_from_10"] <= 1e-3,
        "target_energy_drift_1e-3_at_lambda_D_dx": r["drift_vs_debye"][-1]["mixed_from_10"] <= 1e-3,
    }
    return r


def corrected_arm(cfg, args, device):
    """The same workload and form under the corrected-physics policy (true
    vertex, charge-conserving Villasenor-Buneman current, time-centred Yee at
    the periodic wrap): loop throughput and the fused kernel's mean time."""
    from apc_524_project_gb300 import abi

    L = abi.lib()
    N = cfg.total_particles()
    h = _make_handle(cfg, abi.MIXED, N, device, policy=abi.POLICY_CORRECTED)
    cnt = (C.c_int64 * 6)()
    for _ in range(args.warmup):
        abi.check(L.emoo_step(h, 1, cnt), "emoo_step")
    abi.check(L.emoo_set_profiling(h, 1))
    t = _timed_steps(h, args.steps, lambda: None)
    st = abi.Stats()
    abi.check(L.emoo_get_stats(h, C.byref(st)))
    abi.check(L.emoo_destroy(h))
    out = {"policy": "corrected", "form": "mixed", "value": N * args.steps / t, "unit": UNIT,
           "ms_per_step": t / args.steps * 1e3, "fused_kernel_ms": st.timed_ms / max(1, st.timed_launches)}
    if not args.no_full_run:
        out["full_run"] = full_run(cfg, device)
    return out


def cadence_arm(cfg, device, cadences=(10, 14, 20), steps=140):
    """The benchmark's workload at other sort cadences (the input's nstep_sort;
    the headline keeps the configured 20): loop throughput over `steps` steps,
    a whole number of intervals at each cadence, under the corrected policy
    (over this many steps the reference policy's field energy grows, and its
    particles speed up with it). A sort costs a pass over the store; the fused
    kernel slows between sorts as particles leave their sorted cells."""
    import dataclasses

    import torch
    from apc_524_project_gb300 import abi

    L = abi.lib()
    N = cfg.total_particles()
    cnt = (C.c_int64 * 6)()
    out = {"workload": "the benchmark's workload, mixed form, corrected policy", "steps": steps}
    for T in cadences:
        h = _make_handle(dataclasses.replace(cfg, nstep_sort=T), abi.MIXED, N, device, policy=abi.POLICY_CORRECTED)
        abi.check(L.emoo_step(h, 1, cnt), "emoo_step")  # the first push, after the load's sort
        st = _stream_of(h)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        abi.check(L.emoo_step(h, steps, cnt), "emoo_step")
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        abi.check(L.emoo_destroy(h))
        out[str(T)] = {"value": N * steps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / steps}
    return out


def _history(h):
    from apc_524_project_gb300 import abi

    n = C.c_int()
    abi.check(abi.lib().emoo_history_rows(h, 0, None, C.byref(n)))
    rows = (C.c_double * (8 * max(1, n.value)))()
    abi.check(abi.lib().emoo_history_rows(h, n.value, rows, C.byref(n)))
    return [list(rows[8 * i:8 * i + 8]) for i in range(n.value)]


def full_run(cfg, device):
    """The whole configured run (200 steps: 10 sorts, 20 history rows) in the
    mixed form, timed end to end on the device, under the corrected policy
    (charge-conserving, time-centred: the stable scheme), with the total
    energy's drift from its history rows; and the same run under the
    reference policy, untimed, to record where its energy departs."""
    import torch
    from apc_524_project_gb300 import abi

    L = abi.lib()
    N = cfg.total_particles()
    cnt = (C.c_int64 * 6)()
    res = {"steps": cfg.steps}
    for policy, name in ((abi.POLICY_CORRECTED, "corrected"), (abi.POLICY_REFERENCE, "reference")):
        h = _make_handle(cfg, abi.MIXED, N, device, policy=policy)
        st = _stream_of(h)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        rc = L.emoo_step(h, cfg.steps, cnt)
        e1.record(st)
        torch.cuda.synchronize()
        rows = _history(h)
        abi.check(L.emoo_destroy(h))
        tot = [r[7] for r in rows]
        r = {"rc": rc, "history_rows": len(rows), "total_energy_first": tot[0] if tot else None,
             "total_energy_last": tot[-1] if tot else None}
        if policy == abi.POLICY_CORRECTED:
            t = e0.elapsed_time(e1) / 1e3
            r.update({"value": N * cfg.steps / t, "unit": UNIT, "seconds": t,
                      "drift_from_step_10": abs(tot[-1] - tot[1]) / abs(tot[1]) if len(tot) > 1 else None})
        else:
            grow = [i * 10 for i, v in enumerate(tot) if not (abs(v) <= 2.0 * abs(tot[1]))] if len(tot) > 1 else []
            r["first_step_beyond_2x_step_10_energy"] = grow[0] if grow else None
        res[name] = r
    return res


def twostream_arm(device, steps=1000, every=10, policy=1):
    """The two-stream workload at its configured size (256 x 128^2 cells,
    134,217,728 electrons in two beams drifting at +-0.3c, immobile ions,
    seeded 1e-4 B noise, dt 0.45, 1000 steps, sort every 20) in both forms
    under the corrected policy (the reference policy's field solver is
    unstable at this dt): loop throughput of each, and every `every` steps
    the FP64 history row (energies, momenta) and Gauss-law residual of each
    form with the mixed form's relative L2 distance from the FP64 form in E
    and B over the physical points."""
    import numpy as np
    import torch
    from apc_524_project_gb300 import abi, configs

    L = abi.lib()
    cfg = configs.twostream(steps=steps)
    N = cfg.total_particles()
    shape = tuple(v + 3 for v in cfg.n)
    phys = tuple(slice(1, v + 1) for v in cfg.n)
    noise = configs.b_noise_fields(cfg)
    hs = {}
    for prec, name in ((abi.FP64, "fp64"), (abi.MIXED, "mixed")):
        h = _make_handle(cfg, prec, N, device, policy=policy)
        for c in range(3):
            for base in (abi.BX, abi.BX_TM1):
                abi.check(L.emoo_set_field(h, base + c, noise[c].ctypes.data_as(C.POINTER(C.c_double))))
        hs[name] = h
    out = {"workload": (f"two-stream 256x128x128 cells, {N:,} electrons (2 beams x 16 ppc, drift +-0.3c, v_th "
                        "0.02c), immobile ions, B noise 1e-4, dt 0.45, relativistic, sort every 20"),
           "policy": "corrected" if policy else "reference", "steps": steps, "rows": []}
    times = {"fp64": 0.0, "mixed": 0.0}
    cnt = (C.c_int64 * 6)()

    def fields(h, ids):
        a = np.empty(shape)
        res = []
        for i in ids:
            abi.check(L.emoo_get_field(h, i, a.ctypes.data_as(C.POINTER(C.c_double))))
            res.append(a[phys].copy())
        return np.concatenate([r.ravel() for r in res])

    for t0 in range(0, steps, every):
        row = {"step": t0 + every}
        for name, h in hs.items():
            st = _stream_of(h)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            abi.check(L.emoo_step(h, every, cnt), "emoo_step")
            e1.record(st)
            torch.cuda.synchronize()
            times[name] += e0.elapsed_time(e1) / 1e3
            hist = (C.c_double * 8)()
            abi.check(L.emoo_history(h, hist))
            gr = (C.c_double * 2)()
            abi.check(L.emoo_gauss_residual(h, gr))
            row[name] = {"history": list(hist), "gauss_max": gr[0], "gauss_l2": gr[1]}
        if (t0 + every) % 100 == 0:
            for grp, ids in (("E", (abi.EX, abi.EY, abi.EZ)), ("B", (abi.BX, abi.BY, abi.BZ))):
                f, m = fields(hs["fp64"], ids), fields(hs["mixed"], ids)
                row[f"mixed_rel_l2_{grp}"] = float(np.linalg.norm(m - f) / max(np.linalg.norm(f), 1e-300))
        out["rows"].append(row)
    for name, h in hs.items():
        out[name] = {"value": N * steps / times[name], "unit": UNIT, "seconds": times[name]}
        abi.check(L.emoo_destroy(h))
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def _poisson_solve_ms(L, h, reps):
    """Wall time of emoo_poisson_init (synchronous; the four solves, phiToE,
    AToB and the E/B fill) on the fields the handle holds, best of reps."""
    from apc_524_project_gb300 import abi

    it = (C.c_int * 4)()
    best, rc = None, None
    for _ in range(reps):
        t0 = time.perf_counter()
        rc = L.emoo_poisson_init(h, it)
        t = time.perf_counter() - t0
        if rc not in (abi.OK, abi.ERR_NOT_CONVERGED):
            abi.check(rc, "emoo_poisson_init")
        best = t if best is None else min(best, t)
    return best * 1e3, list(it), rc == abi.OK


def poisson_arm(device):
    """The field start (four Poisson solves, phiToE, AToB): the reference's
    Jacobi iteration against the multigrid solve of the same discrete
    equations, both on the GPU in FP64. (1) The Langmuir workload's start,
    32^3 periodic, rho and J deposited from its 524,288 particles: the Jacobi
    runs into its 10000-sweep cap (the odd-even mode of an even periodic grid
    never decays); E then differs from the exact solution by that mode.
    (2) A periodic box of the laser-plasma size, 512 x 128 x 128 cells,
    seeded rho and J (mean-free noise)."""
    import numpy as np
    import torch
    from apc_524_project_gb300 import abi, configs

    L = abi.lib()
    out = {}
    n = (512, 128, 128)
    big = configs.tiny("poisson512", n=n, init="poisson", ppc=1)
    info = configs.input_info(big)
    shape = tuple(v + 3 for v in n)
    rng = np.random.default_rng(5)
    src = {abi.RHO: rng.normal(0.0, 1e-3, shape)}
    for q in range(3):
        src[abi.JX + q] = rng.normal(0.0, 5e-4, shape)
    box = {"workload": "periodic 512x128x128 cells, seeded rho and J"}
    for solver, name in ((abi.POISSON_MULTIGRID, "multigrid"), (abi.POISSON_JACOBI, "jacobi")):
        o = abi.Opts()
        L.emoo_default_opts(C.byref(o))
        o.device = device
        o.capacity = 1
        o.track_ids = 0
        o.poisson_solver = solver
        h = C.c_void_p()
        abi.check(L.emoo_create(C.byref(info), C.byref(o), C.byref(h)), "emoo_create")
        for fid, a in src.items():
            abi.check(L.emoo_set_field(h, fid, a.ctypes.data_as(C.POINTER(C.c_double))), "emoo_set_field")
        ms, it, ok = _poisson_solve_ms(L, h, 1 if solver == abi.POISSON_JACOBI else 3)
        box[name] = {"ms": ms, "iterations" if solver == abi.POISSON_JACOBI else "v_cycles": it, "converged": ok}
        abi.check(L.emoo_destroy(h))
        torch.cuda.synchronize()
    box["speedup"] = box["jacobi"]["ms"] / box["multigrid"]["ms"]
    out["box512x128x128"] = box
    cfg = configs.langmuir32()
    N = cfg.total_particles()
    ex = {}
    lang = {"workload": "Langmuir 32^3 periodic field start, rho/J from 524,288 particles"}
    for solver, name in ((abi.POISSON_JACOBI, "jacobi"), (abi.POISSON_MULTIGRID, "multigrid")):
        h = _make_handle(cfg, abi.FP64, N, device, poisson_solver=solver)
        ms, it, ok = _poisson_solve_ms(L, h, 1 if solver == abi.POISSON_JACOBI else 3)
        lang[name] = {"ms": ms, "iterations" if solver == abi.POISSON_JACOBI else "v_cycles": it, "converged": ok}
        a = np.zeros(tuple(v + 3 for v in cfg.n))
        abi.check(L.emoo_get_field(h, abi.EX, a.ctypes.data_as(C.POINTER(C.c_double))), "emoo_get_field")
        ex[name] = a
        abi.check(L.emoo_destroy(h))
    lang["speedup"] = lang["jacobi"]["ms"] / lang["multigrid"]["ms"]
    lang["ex_rel_l2_jacobi_vs_multigrid"] = float(np.linalg.norm(ex["jacobi"] - ex["multigrid"]) /
                                                  np.linalg.norm(ex["multigrid"]))
    out["langmuir32"] = lang
    return out


def laser512_arm(device, steps=20, warmup=3, fp64_steps=3, ad_every=23):
    """The laser-plasma workload at full size (512 x 128^2 cells, 117,440,512
    electrons, shaped pulse, absorbing x walls, sort every 20 steps): loop
    throughput of the mixed form (both policies) and the FP64 form, and the
    mixed-precision adjoint with respect to the 16 envelope coefficients
    after 512 steps, checkpoints every 23 steps (sqrt(512); 47 mixed snapshots
    of 3.6 GB), under the corrected policy: the named objective (electron
    kinetic energy at x in [448, 512)) and one the pulse reaches (x in
    [64, 192)); the latter also under the reference policy, whose field
    energy diverges on this workload (the final field energy of each run is
    recorded). Check: on the workload scaled to 40 x 16^2 cells (30 steps,
    objective x in [8, 16)), the mixed adjoint's derivative for envelope
    coefficient 1 against a central difference of two FP64 primal runs, under
    the corrected policy."""
    import torch
    from apc_524_project_gb300 import abi, configs
    from apc_524_project_gb300.differentiate import Problem

    L = abi.lib()
    cfg = configs.laser512()
    N = cfg.total_particles()
    out = {"workload": "laser-plasma 512x128x128 cells, 117,440,512 electrons from x = 64 at 0.01 n_c, a0 = 1 "
                       "pulse with waist 30 and a 16-coefficient sine envelope, absorbing x, sort every 20"}
    cnt = (C.c_int64 * 6)()
    n = C.c_int64()
    corr, ref = abi.POLICY_CORRECTED, abi.POLICY_REFERENCE
    for prec, name, k, pol in ((abi.MIXED, "mixed", steps, ref), (abi.FP64, "fp64", fp64_steps, ref),
                               (abi.MIXED, "mixed_corrected", steps, corr)):
        h = _make_handle(cfg, prec, N, device, policy=pol)
        for _ in range(warmup if prec == abi.MIXED else 1):
            abi.check(L.emoo_step(h, 1, cnt), "emoo_step")
        t = _timed_steps(h, k, lambda: None)
        abi.check(L.emoo_num_particles(h, -1, C.byref(n)), "emoo_num_particles")
        out[name] = {"value": n.value * k / t, "unit": UNIT, "steps": k, "ms_per_step": t / k * 1e3,
                     "particles": n.value, "policy": "corrected" if pol == corr else "reference"}
        abi.check(L.emoo_destroy(h))
        torch.cuda.synchronize()
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]

    def adjoint(slab, pol):
        h = _make_handle(cfg, abi.MIXED, N, device, policy=pol)
        nth = L.emoo_ad_nparams(h)
        spec = abi.AdSpec(cfg.steps, ad_every, slab[0], slab[1], abi.AD_OBJ_KINETIC, 0)
        res = abi.AdResult()
        g = (C.c_double * nth)()
        abi.check(L.emoo_ad_run(h, C.byref(spec), abi.AD_ADJOINT, None, None, C.byref(res), g, None), "emoo_ad_run")
        st = abi.Stats()
        abi.check(L.emoo_get_stats(h, C.byref(st)), "emoo_get_stats")
        row = (C.c_double * 8)()
        abi.check(L.emoo_history(h, row), "emoo_history")
        abi.check(L.emoo_destroy(h))
        coef = list(g)[2:]
        return {"form": "mixed", "policy": "corrected" if pol == corr else "reference", "steps": cfg.steps,
                "checkpoint_every": ad_every,
                "objective": f"electron kinetic energy, x in [{slab[0]}, {slab[1]})", "value": res.objective,
                "forward_ms": res.forward_ms, "recompute_ms": res.recompute_ms, "reverse_ms": res.reverse_ms,
                "adjoint_over_forward": (res.recompute_ms + res.reverse_ms) / res.forward_ms,
                "max_abs_coef_gradient": max(abs(v) for v in coef), "coef_gradient_l2": math.sqrt(sum(v * v for v in coef)),
                "cell_mismatch": st.ad_cell_mismatch, "final_field_energy": row[5] + row[6]}

    named = adjoint((448, 512), corr)
    small = configs.laser512(n=(40, 16, 16), steps=30, ppc=2, wavelength=8.0, fwhm_steps=6, waist=5.0,
                             plasma_x0=8.0, vth=0.02, seed=11)
    kw = dict(nsteps=30, slab=(8, 16), checkpoint_every=6, objective="kinetic", species=0, policy=corr)
    gm = Problem(small, precision=abi.MIXED, **kw).gradient()["grad_theta"]
    P = Problem(small, **kw)
    k = 2  # envelope coefficient 1
    hstep = 1e-6
    th = P.theta0.copy()
    th[k] += hstep
    lp = P.objective(th)
    th[k] -= 2 * hstep
    lm = P.objective(th)
    fd = (lp - lm) / (2 * hstep)
    # the named objective lies outside the pulse's light cone (0.45 x 512 =
    # 230 cells < 448): its gradient is 0 by causality, so this measures the
    # cost of the reverse pass on a vacuous gradient; the reachable range
    # [64, 192) (the plasma the pulse crosses) carries a nonzero one
    named["note"] = ("cost measurement: the objective range lies beyond the pulse's light cone, the gradient is "
                     "exactly 0 by causality")
    out["adjoint"] = named
    out["adjoint"]["fd_check"] = {"case": "laser-plasma 40x16x16, 2 ppc, 30 steps, kinetic energy x in [8, 16), "
                                          "d objective / d envelope coefficient 1, corrected policy",
                                  "mixed_adjoint": float(gm[k]), "fp64_central_difference": fd,
                                  "rel_err": abs(fd - gm[k]) / abs(fd)}
    out["adjoint_reachable"] = adjoint((64, 192), corr)
    out["adjoint_reachable_reference_policy"] = adjoint((64, 192), ref)
    out["adjoint_reachable_reference_policy"]["note"] = (
        "the reference scheme's field energy diverges on this workload (final_field_energy against the corrected "
        "run's): its gradient is that of a diverging run")
    return out


def adjoint_arm():
    """Differentiation of the FP64 loop. Cost: the laser workload at full size
    (64^3, 2 x 8 ppc, 128 steps, objective the slab x in [48, 56),
    checkpoints every 16 steps): one adjoint run (forward with checkpoints,
    then recompute + reverse per segment) against its forward. Check: on a
    16 x 8 x 8 laser case of 24 steps, where no particle changes cell within
    the difference step, the amplitude derivative against a central
    difference of two primal runs."""
    from apc_524_project_gb300 import configs
    from apc_524_project_gb300.differentiate import Problem

    P = Problem(configs.laser64(), nsteps=128, slab=(48, 56), checkpoint_every=16)
    P.gradient()  # warm-up (allocations, first launches)
    g = P.gradient()
    fwd = g["forward_ms"]
    S = Problem(configs.laser64(n=(16, 8, 8), steps=24, ppc=2, wavelength=8.0, fwhm_steps=8), nsteps=24,
                slab=(2, 8), checkpoint_every=4)
    gs = S.gradient()["grad_theta"][0]
    h = 1e-6 * S.theta0[0]
    th = S.theta0.copy()
    th[0] += h
    lp = S.objective(th)
    th[0] -= 2 * h
    lm = S.objective(th)
    fd = (lp - lm) / (2 * h)
    return {"workload": "laser plane wave into plasma, 64^3 cells, 2 x 8 ppc = 4,194,304 particles, 128 steps, "
                        "FP64, checkpoints every 16 steps",
            "forward_ms": fwd, "recompute_ms": g["recompute_ms"], "reverse_ms": g["reverse_ms"],
            "adjoint_over_forward": (g["recompute_ms"] + g["reverse_ms"]) / fwd,
            "fd_check": {"case": "laser 16x8x8, 2 x 2 ppc, 24 steps, d objective / d amplitude",
                         "adjoint": float(gs), "central_difference": fd, "rel_err": abs(fd - gs) / abs(fd)},
            "corrected": adjoint_corrected_arm()}


def adjoint_corrected_arm(hs=(1e-4, 1e-6, 1e-8), h_check=1e-6):
    """The differentiation workload at full size under the corrected policy
    (64^3, 2 x 8 ppc, 128 steps, slab x in [48, 56), checkpoints every 16,
    FP64): one adjoint run for the cost, its amplitude and phase derivatives
    against central differences of two primal runs with step h_check (the
    workload's h = 1e-6; the amplitude's step relative to its value, the
    phase's in degrees) and at the other steps `hs`, and the velocity
    gradient along a seeded direction of per-particle perturbations (sigma
    1e-3 c) against the central difference of the objective along it (the
    1e-3 target is the amplitude's and the phase's; the velocity direction is
    reported beside it at every step)."""
    import numpy as np
    from apc_524_project_gb300 import abi, configs
    from apc_524_project_gb300.differentiate import Problem

    P = Problem(configs.laser64(), nsteps=128, slab=(48, 56), checkpoint_every=16, policy=abi.POLICY_CORRECTED)
    P.gradient()  # warm-up
    g = P.gradient()
    fwd = g["forward_ms"]
    out = {"workload": "laser plane wave into plasma, 64^3 cells, 2 x 8 ppc = 4,194,304 particles, 128 steps, "
                       "FP64, corrected policy, checkpoints every 16 steps",
           "objective": g["objective"], "forward_ms": fwd, "recompute_ms": g["recompute_ms"],
           "reverse_ms": g["reverse_ms"], "adjoint_over_forward": (g["recompute_ms"] + g["reverse_ms"]) / fwd,
           "fd": {}}
    worst = 0.0
    for k, name, scale in ((0, "amplitude", P.theta0[0]), (1, "phase_deg", 1.0)):
        adj = float(g["grad_theta"][k])
        rows = []
        for hr in sorted(set(hs) | {h_check}, reverse=True):
            h = hr * scale
            th = P.theta0.copy()
            th[k] += h
            lp = P.objective(th)
            th[k] -= 2 * h
            lm = P.objective(th)
            fd = (lp - lm) / (2 * h)
            rows.append({"h": h, "central_difference": fd, "rel_err": abs(fd - adj) / abs(adj)})
            if hr == h_check:
                worst = max(worst, abs(fd - adj) / abs(adj))
        out["fd"][name] = {"adjoint": adj, "steps": rows}
    rng = np.random.default_rng(20240707)
    ddv = 1e-3 * rng.standard_normal((3, P.np))
    adj = float(np.sum(g["grad_v"] * ddv))
    rows = []
    for h in sorted(set(hs) | {h_check}, reverse=True):
        fd = (P.objective(None, h * ddv) - P.objective(None, -h * ddv)) / (2 * h)
        rows.append({"h": h, "central_difference": fd, "rel_err": abs(fd - adj) / abs(adj)})
    out["fd"]["velocity_direction"] = {
        "adjoint": adj, "steps": rows,
        "note": "a step moves all 4.2 M particles; at h = 1e-6 (1e-9 c each) about one crosses a cell face in the "
                "128 steps and its jump dominates the quotient; at h = 1e-8 none does"}
    out["max_rel_err_amplitude_phase_at_h_check"] = worst
    out["target_within_1e-3"] = worst <= 1e-3
    out["target_ratio_le_4"] = out["adjoint_over_forward"] <= 4.0
    return out


def _e2e(h, cfg, steps, dist_barrier, dist_max, roundtrip_steps=2):
    """The particle state in FP64 host arrays (pinned), every step crossing
    the host link both ways. Headline: the arrays attached
    (emoo_attach_particles) and `steps` loop steps in one emoo_step call,
    which streams them through the fused kernel in place (a history step also
    leaves the pre-push state in the device store for the moments); the step
    that sorts (every 20) runs as an upload, a device step and a readback -
    20 steps hold one sort and two history rows. Beside it: the per-step round trip emoo_set_particles +
    emoo_step(1) + emoo_get_particles, which gives bit-identical results."""
    import numpy as np
    import torch
    from apc_524_project_gb300 import abi

    L = abi.lib()
    keys = ("x", "y", "z", "vx", "vy", "vz", "gamma")
    bufs, pinned = [], True
    for si in range(len(cfg.species)):
        n = C.c_int64()
        abi.check(L.emoo_num_particles(h, si, C.byref(n)))
        d = {}
        for k in keys:
            try:
                d[k] = torch.empty(n.value, dtype=torch.float64, pin_memory=True).numpy()
            except Exception:
                d[k] = np.empty(n.value, dtype=np.float64)
                pinned = False
        bufs.append((n.value, d))

    def ptrs(d):
        return [d[k].ctypes.data_as(C.POINTER(C.c_double)) for k in keys]

    def get_all():
        got = C.c_int64()
        for si, (n, d) in enumerate(bufs):
            abi.check(L.emoo_get_particles(h, si, n, *ptrs(d), None, C.byref(got)), "emoo_get_particles")

    def set_all():
        for si, (n, d) in enumerate(bufs):
            abi.check(L.emoo_set_particles(h, si, n, *ptrs(d)), "emoo_set_particles")

    cnt = (C.c_int64 * 6)()
    get_all()
    set_all()
    abi.check(L.emoo_step(h, 1, cnt))
    get_all()
    dist_barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(roundtrip_steps):
        set_all()
        abi.check(L.emoo_step(h, 1, cnt))
        get_all()
    torch.cuda.synchronize()
    t_rt = dist_max(time.perf_counter() - t0)
    for si, (n, d) in enumerate(bufs):
        abi.check(L.emoo_attach_particles(h, si, n, *ptrs(d)), "emoo_attach_particles")
    abi.check(L.emoo_step(h, 1, cnt))  # warm-up: the first attached step re-uploads once
    dist_barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    abi.check(L.emoo_step(h, steps, cnt), "emoo_step")
    torch.cuda.synchronize()
    t = dist_max(time.perf_counter() - t0)
    abi.check(L.emoo_detach_particles(h))
    nbytes = sum(n for n, _ in bufs) * 8 * len(keys)
    return {"t": t, "steps": steps, "h2d": nbytes, "d2h": nbytes, "pinned": pinned, "t_roundtrip": t_rt,
            "roundtrip_steps": roundtrip_steps}


# ------------------------------------------------------------------ CPU arms

def _cpu_replica(args):
    """One process: the oracle on an independent 32^3 x 32 ppc relativistic
    thermal box; returns (particles, steps, seconds)."""
    size, steps, warm, seed = args
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    from apc_524_project_gb300 import configs, loading
    from backends import OracleBackend

    cfg = configs.thermal256(size)
    cfg.seed = seed
    info = configs.input_info(cfg)
    b = OracleBackend(info, cfg.dt)
    n = 0
    gen = OracleBackend.generator()  # the oracle's sampler: this leg loads no product library
    for si in range(len(cfg.species)):
        p = loading.sample_species(cfg, si, generate=gen)
        b.add_species(si, p, ids=np.arange(n, n + len(p["x"])))
        n += len(p["x"])
    b.init_fields()
    for ti in range(warm):  # warm-up steps (step 0 sorts)
        b.step(ti)
    t0 = time.perf_counter()
    for ti in range(warm, warm + steps):
        b.step(ti)
    t = time.perf_counter() - t0
    b.close()
    return n, steps, t


def cpu_baseline(procs, steps, warm=1, size=32):
    import multiprocessing as mp

    procs = procs or min(os.cpu_count() or 1, 16)
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        t0 = time.perf_counter()
        out = pool.map(_cpu_replica, [(size, steps, warm, 1000 + i) for i in range(procs)])
        wall = time.perf_counter() - t0
    tmax = max(o[2] for o in out)
    total = sum(o[0] * o[1] for o in out)
    n_each = out[0][0]
    return {
        "value": total / tmax,
        "unit": UNIT,
        "cores": procs,
        "kind": "port",
        "sample": (f"{procs} independent {size}^3-cell x 32 ppc relativistic thermal boxes ({n_each:,} particles "
                   f"each), {steps} timed steps each after {warm} warm-up step(s), FP64 CPU restatement of the "
                   f"reference loop, one process per core; wall {wall:.1f} s"),
        "seconds": tmax,
    }


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = workload(args.size)
    cb = cpu_baseline(args.cpu_procs, args.steps, warm=max(1, args.warmup))
    v = cb["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["seconds"] / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc(cfg), "form": "reference CPU loop (FP64)",
                   "sample": cb["sample"]},
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = _args()
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.only == "poisson":
        res = poisson_arm(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"metric": "field start (four Poisson solves + phiToE + AToB), multigrid",
                          "value": res["box512x128x128"]["multigrid"]["ms"], "unit": "ms",
                          "higher_is_better": False, "dtype": "f64 (FP32 V-cycles)", "data": "synthetic",
                          "config": {"workload": res["box512x128x128"]["workload"]}, "poisson": res}), flush=True)
        return
    if args.only == "twostream":
        res = twostream_arm(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"metric": "particle-steps/s, two-stream at configured size, mixed and FP64 forms",
                          "value": res["mixed"]["value"], "unit": UNIT, "higher_is_better": True,
                          "dtype": "f32 (mixed) / f64", "data": "synthetic", "config": {"workload": res["workload"]},
                          "twostream": res}), flush=True)
        return
    if args.only == "mixed_error":
        res = mixed_error_arm(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"metric": "mixed form's error against FP64 after 100 steps (max rel L2 of E, B, J)",
                          "value": res["summary"]["max_rel_l2_EBJ"], "unit": "rel L2", "higher_is_better": False,
                          "dtype": "f32 (mixed) / f64", "data": "synthetic", "config": {"workload": res["workload"]},
                          "mixed_error": res}), flush=True)
        return
    if args.only == "adjoint":
        # one gradient of the 64^3 laser workload (FP64), timed by emoo_ad_run's events
        from apc_524_project_gb300 import abi, configs
        from apc_524_project_gb300.differentiate import Problem

        pol = abi.POLICY_CORRECTED if args.ad_policy == "corrected" else abi.POLICY_REFERENCE
        P = Problem(configs.laser64(), nsteps=args.ad_steps, slab=(48, 56), checkpoint_every=16, policy=pol)
        g = P.gradient()
        ratio = (g["recompute_ms"] + g["reverse_ms"]) / g["forward_ms"]
        print(json.dumps({"metric": "adjoint / forward cost, laser 64^3 FP64", "value": ratio, "unit": "ratio",
                          "higher_is_better": False, "dtype": "f64", "data": "synthetic",
                          "config": {"workload": f"laser 64^3, 4,194,304 particles, {args.ad_steps} steps, "
                                                 f"{args.ad_policy} policy, checkpoints every 16"},
                          "forward_ms": g["forward_ms"], "recompute_ms": g["recompute_ms"],
                          "reverse_ms": g["reverse_ms"], "objective": g["objective"]}), flush=True)
        return
    from apc_524_project_gb300 import replicas

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    cb = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # before the first GPU call (the pool is spawned, but keep it first)
        cb = cpu_baseline(args.cpu_procs, args.cpu_steps)
    import torch  # noqa: F401

    world, rank, barrier, dmax, close = replicas.comm("nccl", int(os.environ.get("LOCAL_RANK", "0")))
    cfg, res = run_gpu_arm(args, rank, world, barrier, dmax)
    close()
    if rank != 0:
        return
    N = cfg.total_particles()
    m = res["mixed"]
    value = replicas.job_throughput(N, args.steps, world, m["t"])
    peak, peak_kind = _peaks()
    cells = cfg.n[0] * cfg.n[1] * cfg.n[2]
    # algorithmic bytes of one fused-kernel launch: every particle's 28-byte
    # state read and written, plus per cell the 9 FP32 field words gathered and
    # the 4 int64 J/rho words deposited
    alg_bytes = N * 56 + cells * (9 * 4 + 4 * 8)
    achieved = alg_bytes / (m["fused_ms"] / 1e3) / 1e9
    tr = _traffic_per_unit()
    traffic = None
    if tr and "dram_bytes_per_particle" in tr:
        traffic = tr["dram_bytes_per_particle"] * N
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": m["t"] / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_desc(cfg), "form": "mixed (int32 cell + FP32 offset, FP32 u and fields, "
                                                          "int64 fixed-point J/rho)",
                   "particles": N,
                   "l2": f"inputs larger than L2 ({N * 28 / 1e9:.1f} GB particle state per GPU, 129 MB L2), no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "kernel": "k_fused_m (gather+push+BC+deposit)",
                     "kernel_ms": m["fused_ms"], "algorithmic_bytes": alg_bytes},
        "gpu_launches": m["launches"],
        "clocks": m["clocks"],
        "sort_ms": res.get("sort_ms"),
        "sort_drift_steps": res.get("sort_drift_steps"),
    }
    if "fp64" in res:
        f = res["fp64"]
        v64 = N * args.fp64_steps * world / f["t"]
        # the FP64 form's push by operation count: about 70 FP64 operations per particle
        # for the relativistic (Vay) pusher, 30 for Boris, with the square roots and
        # divisions counted apart (2 and 4 for Vay, 0 and 1 for Boris)
        rel = cfg.relativity != 0
        ops, sq, dv = (70, 2, 4) if rel else (30, 0, 1)
        line["fp64"] = {"value": v64, "unit": UNIT, "steps": args.fp64_steps,
                        "ms_per_step": f["t"] / args.fp64_steps * 1e3, "fused_kernel_ms": f["fused_ms"],
                        "mixed_over_fp64": value / v64,
                        "push_flops": {"fp64_ops_per_particle": ops, "sqrt_per_particle": sq, "div_per_particle": dv,
                                       "achieved_gflops": N * ops / (f["fused_ms"] / 1e3) / 1e9,
                                       "bound": "FP64 pipe (the form keeps the reference's operation order, "
                                                "no FMA, IEEE divisions and square roots)"}}
    if "adjoint" in res:
        line["adjoint"] = res["adjoint"]
    if "laser512" in res:
        line["laser512"] = res["laser512"]
    if "poisson" in res:
        line["poisson"] = res["poisson"]
    if "corrected" in res:
        line["corrected"] = res["corrected"]
    if "sort_cadence" in res:
        line["sort_cadence"] = res["sort_cadence"]
    if "mixed_error" in res:
        line["mixed_error"] = res["mixed_error"]
    if "e2e" in res:
        e = res["e2e"]
        line["e2e"] = {"value": N * e["steps"] * world / e["t"], "unit": UNIT, "h2d_bytes_per_step": e["h2d"],
                       "d2h_bytes_per_step": e["d2h"], "steps": e["steps"], "pinned": e["pinned"],
                       "ms_per_step": e["t"] / e["steps"] * 1e3,
                       "path": "FP64 host arrays attached (emoo_attach_particles), emoo_step streams them through "
                               "the GPU every step; the sort step as upload + step + readback",
                       # the bound: both link directions at once, 167 GB/s each way measured on these nodes
                       # by a kernel reading and writing pinned host memory
                       "host_link": {"achieved_gbs": (e["h2d"] + e["d2h"]) * e["steps"] / e["t"] / 1e9,
                                     "peak_gbs": HOST_LINK_DUPLEX_GBS,
                                     "frac": (e["h2d"] + e["d2h"]) * e["steps"] / e["t"] / 1e9 / HOST_LINK_DUPLEX_GBS},
                       "roundtrip": {"value": N * e["roundtrip_steps"] * world / e["t_roundtrip"], "unit": UNIT,
                                     "ms_per_step": e["t_roundtrip"] / e["roundtrip_steps"] * 1e3,
                                     "path": "emoo_set_particles + emoo_step(1) + emoo_get_particles per step"}}
    if cb:
        line["cpu_baseline"] = cb
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
