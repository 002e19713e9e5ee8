"""The mixed form's error on the thermal-plasma benchmark's physics, stated
against the FP64 form (apc_524_project_gb300/precision.py).

Workload: the 256^3 thermal plasma (electrons and ions, 16 particles per
cell each, electron v_th = 0.1c, relativistic push, dt = 0.5, sort every 20
steps) scaled to 24^3 cells, under the corrected policy (the scheme that
stays stable over the run), 100 steps. Checks at steps 10, 50 and 100:
  * E, B and J of the mixed run are within ENSEMBLE_FACTOR times the largest
    distance of six FP64 runs perturbed after every step by the mixed form's
    own one-step rounding (measured);
  * the field energy, kinetic energy and Gauss-law residual norm of the mixed
    run are within OBS_RTOL of the FP64 run's.
"""
import pytest

from apc_524_project_gb300 import abi, configs, precision

pytestmark = pytest.mark.gpu

ENSEMBLE_FACTOR = 2.0
OBS_RTOL = 1e-4


def test_mixed_error_on_the_thermal_plasma():
    cfg = configs.thermal256(n=24)
    r = precision.measure(cfg, steps_at=(10, 50, 100), members=6, policy=abi.POLICY_CORRECTED)
    print("thermal 24^3 mixed vs FP64:", r)
    for t, row in r["fields"].items():
        for name, v in row.items():
            assert v["mixed"] <= ENSEMBLE_FACTOR * v["spread_max"], (t, name, v)
    for t, obs in r["observables"].items():
        for name in ("field_energy", "kinetic_energy", "gauss_l2"):
            assert obs[name]["rel_diff"] <= OBS_RTOL, (t, name, obs[name])
