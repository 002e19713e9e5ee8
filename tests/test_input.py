"""The input.txt reader (emoo_read_input / emoo_parse_input) and
emoo_process_info against the reference's parsing rules
(src/IO/readinfo.cpp, src/IO/check.cpp). Host only, no GPU."""
import ctypes as C
import os

import pytest

from apc_524_project_gb300 import abi

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


def parse(text):
    info = abi.InputInfo()
    rc = abi.lib().emoo_parse_input(text.encode(), C.byref(info))
    return rc, info, abi.lib().emoo_input_message().decode()


def test_read_full_file():
    info = abi.InputInfo()
    rc = abi.lib().emoo_read_input(os.path.join(DATA, "langmuir_small.txt").encode(), C.byref(info))
    assert rc == abi.OK, abi.lib().emoo_input_message()
    assert list(info.nCell) == [8, 6, 4] and list(info.Lxyz) == [8.0, 6.0, 4.0]
    assert list(info.nProc) == [1, 1, 1]
    assert info.nt == 25 and info.t0 == 0.5 and info.nstep_sort == 5
    assert info.nparticles_tot == 3000000000
    assert info.relativity == 1 and info.nspecies == 2
    assert list(info.mass_ratio[:2]) == [1.0, 100.0] and list(info.charge_ratio[:2]) == [-1.0, 1.0]
    assert list(info.isTestParticle[:2]) == [0, 1]
    assert list(info.dens_frac[:2]) == [3.0, 1.0] and list(info.temp[:2]) == [2.5, 0.5]
    assert info.fields_init == b"poisson" and info.electrostatic == 0
    assert list(info.B0) == [0.0, 0.0, 0.5] and list(info.E0) == [0.1, 0.0, 0.0]
    assert [bytes(info.parts_bound[i]).rstrip(b"\0") for i in range(6)][:2] == [b"reflecting", b"reflecting"]
    assert bytes(info.fields_bound[0]).rstrip(b"\0") == b"external"
    assert info.nwaves == 2 and list(info.inSide[:2]) == [-1, 1] and list(info.inPolE[:2]) == [2, 3]
    assert list(info.peakamps[:2]) == [0.01, 0.02] and list(info.delays[:2]) == [4.0, 0.0]
    assert info.bound_phi[1] == 0.5 and info.bound_Ay[1] == 0.2
    assert info.nstep_fields == 5 and info.nstep_parts == 3 and info.output_pCount == 4
    assert info.which_fields == 1 and info.nstep_restart == 100


MIN = """domain: { nCell = [4]; Lxyz = [2.0]; }
runtime: { nTimesteps = 3; }
initialization: { particles: { nParticles_tot = 64; relativity = 0; nspecies = 1;
   mass_ratio = 1.0; charge_ratio = -1.0; temperature = 0.1; }
   fields: { electrostatic = 0; init = "constant"; %s } }
diagnostics: { particles: { output_pCount = 0; } }
"""


def test_defaults_and_scalar_forms():
    rc, info, msg = parse(MIN % 'E0 = [1.0, 2.0, 3.0]; B0 = [4.0, 5.0, 6.0];')
    assert rc == abi.OK, msg
    assert list(info.nCell) == [4, 4, 4] and list(info.Lxyz) == [2.0, 2.0, 2.0]  # 1-element arrays broadcast
    assert info.dens_frac[0] == 1.0 and info.isTestParticle[0] == 0
    assert info.nstep_sort == 100 and info.nstep_fields == 10 and info.which_fields == -1
    assert all(bytes(info.parts_bound[i]).rstrip(b"\0") == b"periodic" for i in range(6))
    assert info.nwaves == 0 and info.t0 == 0.0


def test_missing_e0_resets_b0_like_the_reference():
    rc, info, msg = parse(MIN % 'B0 = [4.0, 5.0, 6.0];')
    assert rc == abi.OK
    assert list(info.B0) == [0.0, 0.0, 0.0]  # src/IO/readinfo.cpp:467


@pytest.mark.parametrize("drop,err", [("relativity = 0;", "relativity"), ("nTimesteps = 3;", "nTimesteps"),
                                      ("output_pCount = 0;", "output_pCount"), ('init = "constant";', "init")])
def test_required_settings(drop, err):
    rc, info, msg = parse((MIN % "").replace(drop, ""))
    assert rc == abi.ERR_INPUT
    assert err in msg or "initialization method" in msg


def test_syntax_errors_report_the_line():
    rc, info, msg = parse("domain: { nCell = [4, 4 }\n")
    assert rc == abi.ERR_INPUT and "line" in msg
    rc, info, msg = parse('runtime: { x = "unterminated }')
    assert rc == abi.ERR_INPUT


def test_species_array_length_mismatch():
    text = (MIN % "").replace("nspecies = 1;", "nspecies = 2;")
    rc, info, msg = parse(text)
    assert rc == abi.ERR_INPUT and "mass_ratio" in msg


def test_process_info_scales_super_particles():
    info = abi.InputInfo()
    assert abi.lib().emoo_read_input(os.path.join(DATA, "langmuir_small.txt").encode(), C.byref(info)) == abi.OK
    assert abi.lib().emoo_process_info(C.byref(info)) == abi.OK
    n0 = 3000000000 / (8.0 * 6.0 * 4.0)
    ratio = 2.0 / n0
    assert info.super_ratio == pytest.approx(ratio)
    assert info.dens_frac[0] == pytest.approx(0.75) and info.dens_frac[1] == pytest.approx(0.25)
    assert info.mass_ratio[1] == pytest.approx(100.0 * ratio)
    assert info.charge_ratio[0] == pytest.approx(-ratio)
    assert info.temp[0] == pytest.approx(2.5 * ratio)
    assert info.nparticles_domain == 0  # set by the Domain (src/domain/domain.cpp:100), not ProcessInfo


def test_process_info_rejects_inconsistent_boundaries():
    rc, info, msg = parse(MIN % "")
    info.parts_bound[0] = info.parts_bound[0].__class__.from_buffer_copy(b"reflecting" + b"\0" * 54)
    assert abi.lib().emoo_process_info(C.byref(info)) == abi.ERR_INPUT
