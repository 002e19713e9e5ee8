"""emoo_read_input + emoo_process_info against the reference's own reader.

The reference's Input::readinfo (src/IO/readinfo.cpp:18-733) and
Input::ProcessInfo (src/IO/check.cpp:12-147) are compiled from its sources,
with libconfig 1.5 compiled from the tarball it ships, into
oracle/_ref/libemoo_refinput.so (oracle/ref/Makefile). Each input file below
is read by both; the two Input_Info_t structs must be equal byte for byte,
before and after ProcessInfo, and a file one reader refuses the other must
refuse too. Host only; skipped where the reference build is absent.

Only inputs on which the reference returns are used: it terminates the
process on a missing relativity / electrostatic / output_pCount (it catches
those exceptions by pointer) and on a setting of a type libconfig cannot
convert, which emoo_read_input reports as EMOO_ERR_INPUT instead
(tests/test_input.py).
"""
import ctypes as C
import os

import pytest

from apc_524_project_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libemoo_refinput.so")
DATA = os.path.join(ROOT, "tests", "data")

pytestmark = pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference input reader not built here")

_REF = None


def ref():
    global _REF
    if _REF is None:
        L = C.CDLL(REF_LIB)
        L.refi_read_input.argtypes = [C.c_char_p, C.POINTER(abi.InputInfo)]
        L.refi_process_info.argtypes = [C.POINTER(abi.InputInfo)]
        assert L.refi_sizeof_input_info() == C.sizeof(abi.InputInfo)
        _REF = L
    return _REF


BASE = """# {title}
domain:
{{
  nCell = {ncell}
  {nproc}
  xyz0 = {xyz0}
  Lxyz = {lxyz}
}}
runtime: {{ nTimesteps = {nt}; {runtime} }}
initialization:
{{
  {restart}
  particles:
  {{
    nParticles_tot = {npart}
    {dens_phys}
    relativity = {rel}
    nspecies = {nspec}
    mass_ratio = {mass}
    charge_ratio = {charge}
    temperature = {temp}
    {extra_species}
  }}
  fields: {{ electrostatic = {es}; init = "{init}"; {fields} }}
}}
boundary:
{{
  {pbound}
  {fbound}
}}
diagnostics:
{{
  {diag}
  particles: {{ output_pCount = {pcount}; }}
}}
"""

DEFAULTS = dict(title="case", ncell="[8, 6, 4]", nproc="", xyz0="[0.0, 0.0, 0.0]", lxyz="[8.0, 6.0, 4.0]", nt=10,
                runtime="", restart="", npart=768, dens_phys="", rel=0, nspec=2, mass="[1.0, 1836.0]",
                charge="[-1.0, 1.0]", temp="[0.5, 0.5]", extra_species="dens_frac = [1.0, 1.0]", es=0, init="poisson", fields="",
                pbound="", fbound="", diag="", pcount=0)

WAVES = """fields:
  {
    conditions = ["external", "external", "periodic", "periodic", "periodic", "periodic"]
    external:
    {
      nwaves = 2
      inSide = [-1, 1]
      inPolE = [2, 3]
      peakamps = [0.01, 0.02]
      omegas = [0.8, 1.1]
      phases = [30.0, 0.0]
      invWidths = [0.3, 0.5]
      delays = [4.0, 0.0]
      poisson:
      {
        bound_phi = [0.0, 0.5, 0.0, 0.0, 0.0, 0.0]
        bound_Ax = [0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
        bound_Ay = [0.0, 0.2, 0.0, 0.0, 0.0, 0.0]
        bound_Az = [0.1, 0.0, 0.0, 0.0, 0.0, 0.0]
      }
    }
  }"""

CASES = {
    "defaults": {},
    "scalar_domain": dict(ncell="[16]", lxyz="[4.0]", xyz0="[1.0]"),
    "one_species_scalars": dict(nspec=1, mass="1.0", charge="-1.0", temp="0.25", extra_species="dens_frac = 1.0"),
    "three_species": dict(nspec=3, mass="[1.0, 100.0, 1836.0]", charge="[-1.0, 1.0, 1.0]", temp="[1.0, 0.5, 0.2]",
                          extra_species="dens_frac = [2.0, 1.0, 1.0]\n    isTestParticle = [0, 1, 0]"),
    "runtime_options": dict(runtime="startTime = 2.5; debug = 1; nstep_sort = 7;", restart="restart = 1",
                            dens_phys="dens_phys = 3.5e10"),
    "relativistic_constant": dict(rel=1, init="constant",
                                  fields="B0 = [0.0, 0.1, 0.2]; E0 = [0.01, 0.0, 0.0];"),
    "b0_without_e0": dict(init="constant", fields="B0 = [0.0, 0.1, 0.2];"),
    "short_field_vectors": dict(init="constant", fields="B0 = [0.3]; E0 = [0.2];"),
    "electrostatic": dict(es=1),
    "int64_particles": dict(npart="3000000000L"),
    "float_particles": dict(npart="1.5e9"),
    "hex_and_ints_as_doubles": dict(nt="0x1A", lxyz="[8, 6, 4]", temp="[1, 2]"),
    "walls": dict(pbound='particles: { conditions = ["reflecting", "reflecting", "periodic", "periodic", '
                         '"periodic", "periodic"]; }'),
    "external_waves": dict(pbound='particles: { conditions = ["reflecting", "reflecting", "periodic", "periodic", '
                                  '"periodic", "periodic"]; }', fbound=WAVES),
    "diagnostics": dict(diag="nstep_fields = 5; nstep_parts = 3; nstep_restart = 50;\n  fields: { which_fields = 1; }",
                        pcount=4),
    "syntax_variants": dict(title="comments // and /* */ and : separators",
                            runtime="startTime : 0.5, /* block */ nstep_sort = 3 // trailing\n",
                            fields='E0 = [0.0, 0.0, 0.0]; B0 = [0.0, 0.0, 0.0];'),
    "decomposition_adjusted": dict(nproc="nProc = [1, 1, 1]", ncell="[9, 6, 4]", lxyz="[9.0, 6.0, 4.0]"),
    # refused by both
    "mixed_type_array": dict(charge="[-1.0, 1]"),
    "no_timesteps": dict(nt='0; } runtime2: { x = 1'),
    "bad_species_count": dict(nspec=0),
    "wrong_length_bounds": dict(pbound='particles: { conditions = ["periodic", "periodic"]; }'),
    "mass_length_mismatch": dict(mass="[1.0]"),
    "syntax_error": dict(ncell="[8, 6, 4"),
    "int_overflow_particles": dict(npart="3000000000"),
}


def text_of(name):
    kw = dict(DEFAULTS)
    kw.update(CASES[name])
    t = BASE.format(**kw)
    if name == "no_timesteps":
        t = t.replace("nTimesteps = 0;", "")
    return t


def read_both(path):
    a, b = abi.InputInfo(), abi.InputInfo()
    ra = ref().refi_read_input(path.encode(), C.byref(a))
    rb = abi.lib().emoo_read_input(path.encode(), C.byref(b))
    return ra, a, rb, b


def differing_fields(a, b):
    out = []
    for name, _ in abi.InputInfo._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if hasattr(va, "_length_"):
            same = bytes(va) == bytes(vb) if hasattr(va, "_type_") or True else va == vb
        else:
            same = va == vb
        if not same:
            out.append(name)
    return out


def compare(path):
    ra, a, rb, b = read_both(path)
    assert (ra == 0) == (rb == abi.OK), (ra, rb, abi.lib().emoo_input_message())
    if ra != 0:
        return False
    assert bytes(a) == bytes(b), differing_fields(a, b)
    pa = ref().refi_process_info(C.byref(a))
    pb = abi.lib().emoo_process_info(C.byref(b))
    assert (pa == 0) == (pb == abi.OK), (pa, pb)
    assert bytes(a) == bytes(b), differing_fields(a, b)
    return True


@pytest.mark.parametrize("name", sorted(CASES))
def test_reader_equals_the_reference(tmp_path, name):
    p = tmp_path / f"{name}.txt"
    p.write_text(text_of(name))
    accepted = compare(str(p))
    refused = {"mixed_type_array", "no_timesteps", "bad_species_count", "wrong_length_bounds",
               "mass_length_mismatch", "syntax_error", "int_overflow_particles"}
    assert accepted == (name not in refused)


@pytest.mark.parametrize("fname", ["langmuir_small.txt", "driver_small.txt"])
def test_data_files_equal_the_reference(fname):
    assert compare(os.path.join(DATA, fname))
