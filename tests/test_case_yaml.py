"""The case reader (charm_case_read_yaml): task.yaml into charm_gpu_config_t.

It restates the reference's charm_init_context_yaml (src/charm_init_yaml.cpp:
333-428) and the model initialisers, which need yaml-cpp.  Checked here: a
case written out as YAML in every style the reference's files use reads back
into the same configuration the Python harness builds for it; every error of
the reference's reader is an error here (never a silently different case);
the reference's own sample case file reads into its stated values.
"""
import ctypes as C
import os
import subprocess
import tempfile

import pytest

from charm_3d_gb300 import abi
from charm_3d_gb300.case import Case

from .common import small_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def case_yaml(case: Case, regions=None, flow_style: bool = False) -> str:
    """A task.yaml of the reference's format for `case`."""
    out = ["method: CHARM_3D", "version: 0.1.2   # the file format", "control:"]
    c = ["  FLUX_TYPE: " + case.flux, "  LIMITER: " + case.limiter, f"  MAX_ERROR: {case.max_err!r}",
         f"  REFINE_PERIOD: {case.refine_period}", "  REPARTITION_PERIOD: 10", f"  MIN_LEVEL: {case.min_level}",
         f"  MAX_LEVEL: {case.max_level}", f"  CFL: {case.cfl!r}", f"  TAU: {case.tau!r}   # step", "  TMAX: 50",
         "  FILE_OUTPUT_STEP: 100", "  LOG_OUTPUT_STEP: 10"]
    if flow_style:
        c.append(f"  MODEL: {{name: {case.model}, use_visc: {case.use_visc}, use_diffusion: {case.use_diff}, "
                 f"t_ref: {case.t_ref!r}}}")
    else:
        c += ["  MODEL:", f"    name: {case.model}", f"    use_visc: {case.use_visc}",
              f"    use_diffusion: {case.use_diff}", f"    t_ref: {case.t_ref!r}"]
    out += c
    out += ["mesh:", "  files_type: gmsh_msh", "  name: 'box mesh.msh'", "components:"]
    for i, k in enumerate(case.components):
        cp = ", ".join(repr(x) for x in k.cp)
        out += ["  -", f"    id: {i}", f'    name: "{k.name}"', f"    cp_type: {k.cp_type}",
                f"    kp_type: {k.kp_type}", f"    ml_type: {k.ml_type}", f"    M: {k.m!r}", f"    Cp: [{cp}]",
                f"    KP0: {k.kp0!r}", f"    ML0: {k.ml0!r}", f"    T0: {k.t0!r}", f"    TS: {k.ts!r}",
                f"    Sig: {k.sig!r}", f"    ek: {k.ek!r}", f"    h0: {k.h0!r}"]
    out += ["materials:", "  - id: 0", "    name: MIXTURE", f"    eof_type: {case.eos}   # IDEAL, MIX"]
    out += ["regions:"]
    for r in regions or [("R0", case.grav)]:
        name, g = r
        comps = ", ".join(f"{{id: {i}, concentration: {1.0 if i == 0 else 0.0}}}" for i in range(case.n_comp))
        out += [f"  - id: 0", f"    name: {name}", "    cell_type: 0", "    material_id: 0",
                f"    components: [{comps}]", "    parameters:", "      V: {x: 1.5, y: 0, z: -2}", "      T: 300",
                "      P: 101325.0", f"      G: {{x: {g[0]!r}, y: {g[1]!r}, z: {g[2]!r}}}"]
    out += ["boundaries:"]
    for b in case.boundaries:
        out += [f"  - name: {b.name}", f"    type: {b.type}"]
        p = b.params
        if b.type == "BOUND_INLET":
            out += ["    parameters:", f"      V: {{x: {p[0]!r}, y: {p[1]!r}, z: {p[2]!r}}}", f"      T: {p[3]!r}",
                    f"      P: {p[4]!r}"]
        elif b.type == "BOUND_WALL_NO_SLIP":
            out += ["    parameters:", f"      T: {p[0]!r}"]
        elif b.type == "BOUND_MASS_FLOW":
            cs = ", ".join(repr(x) for x in p[7:7 + case.n_comp])
            out += ["    parameters:", f"      M: {p[0]!r}", f"      P: {p[1]!r}", f"      T: {p[2]!r}",
                    f"      CosX: {p[3]!r}", f"      CosY: {p[4]!r}", f"      CosZ: {p[5]!r}",
                    f"      components: [{cs}]"]
    if case.reactions:
        out += ["reactions:"]
        for r in case.reactions:
            left = [x for x in r.left if x >= 0]
            right = [x for x in r.right if x >= 0]
            out += [f"  - {{a: {r.a!r}, e: {r.e!r}, n: {r.n!r}, left: {left}, right: {right}}}"]
    return "\n".join(out) + "\n"


def _fields(cfg) -> dict:
    """Every field of a charm_gpu_config_t as nested Python values."""
    def conv(v):
        if isinstance(v, C.Array):
            return [conv(x) for x in v]
        if isinstance(v, C.Structure):
            return {n: conv(getattr(v, n)) for n, _ in v._fields_}
        return v
    d = conv(cfg)
    d["comp"] = d["comp"][:cfg.n_comp]
    d["bnd"] = d["bnd"][:cfg.n_bnd]
    d["react"] = d["react"][:cfg.n_react]
    return d


def _cases():
    ns = small_case("walls", "HLLC", "BJ", level=2)
    react = small_case("react", "LF", "BJ", level=2)
    react.components[1].cp_type = "POLYNOM"
    react.components[1].cp = (1850.0, 0.25, -1e-4)
    react.components[0].kp_type = react.components[0].ml_type = "SATHERLAND"
    mf = small_case("massflow", "GODUNOV", "NONE", level=2)
    b = mf.boundaries[0]
    b.params = b.params[:6] + (b.params[1],) + b.params[7:]   # the file's P is also the stored pressure
    euler = small_case("random", "CD", "NONE", level=2, model="EULER")
    euler.grav = (0.0, 0.0, -9.81)
    return {"ns_walls": ns, "ns_react_mix": react, "mass_flow": mf, "euler_gravity": euler}


@pytest.mark.parametrize("name", list(_cases()))
@pytest.mark.parametrize("flow_style", [False, True])
def test_case_file_reads_into_the_harness_configuration(name, flow_style):
    case = _cases()[name]
    got = abi.read_case_yaml(text=case_yaml(case, flow_style=flow_style))
    want = case.config()
    if case.model == "EULER":     # charm_model_euler_init reads no MODEL keys
        want.t_ref = 0.0
    assert _fields(got.cfg) == _fields(want)
    assert got.mesh_type == b"gmsh_msh" and got.mesh_name == b"box mesh.msh"
    assert [got.bnd_name[i].value for i in range(got.cfg.n_bnd)] == [b.name.encode() for b in case.boundaries]
    assert got.tmax == 50.0 and got.file_output_step == 100 and got.refine_period == case.refine_period
    assert got.n_reg == 1 and list(got.reg[0].v) == [1.5, 0.0, -2.0] and got.reg[0].p == 101325.0


def test_case_file_from_disk_and_region_gravity():
    case = _cases()["ns_walls"]
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "task.yaml")
        with open(path, "w") as fh:
            fh.write(case_yaml(case, regions=[("A", (0.0, 0.0, -1.0)), ("B", (0.0, 0.0, -1.0))]))
        got = abi.read_case_yaml(path)
        assert got.n_reg == 2 and list(got.cfg.grav) == [0.0, 0.0, -1.0]
        with open(path, "w") as fh:
            fh.write(case_yaml(case, regions=[("A", (0.0, 0.0, -1.0)), ("B", (0.0, 0.0, 0.0))]))
        with pytest.raises(abi.CharmGpuError) as e:
            abi.read_case_yaml(path)
        assert e.value.code == abi.ENOTSUP
    with pytest.raises(abi.CharmGpuError) as e:
        abi.read_case_yaml("/nonexistent/task.yaml")
    assert e.value.code == abi.EINVAL


BASE = case_yaml(_cases()["mass_flow"])


@pytest.mark.parametrize("old,new,code,msg", [
    ("method: CHARM_3D", "method: CHARM_2D", abi.EINVAL, b"Method name"),
    ("version: 0.1.2", "version: 0.1.0", abi.EINVAL, b"version"),
    ("FLUX_TYPE: GODUNOV", "FLUX_TYPE: ROE", abi.EINVAL, b"Unknown flux type"),
    ("LIMITER: NONE", "LIMITER: WENO", abi.EINVAL, b"Unknown limiter"),
    ("  TAU:", "  TAUX:", abi.EINVAL, b"'TAU' missing"),
    ("eof_type: IDEAL", "eof_type: TABLE", abi.ENOTSUP, b"TABLE"),
    ("eof_type: IDEAL", "eof_type: VDW", abi.EINVAL, b"unknown EOS"),
    ("type: BOUND_OUTLET", "type: BOUND_PERIODIC", abi.EINVAL, b"unknown boundary type"),
    ("components: [1.0]", "components: [0.5, 0.5]", abi.EINVAL, b"Too many components"),
    ("components: [1.0]", "components: []", abi.EINVAL, b"Too few components"),
    ("concentration: 1.0", "concentration: 1.1", abi.EINVAL, b"Sum of concentrations"),
    ("cp_type: CONST", "cp_type: TABLE", abi.EINVAL, b"Unknown Cp type"),
    ("    M: 0.02869409", "    M: heavy", abi.EINVAL, b"'M' missing or not a number"),
    ("  FLUX_TYPE:", "\tFLUX_TYPE:", abi.EINVAL, b"tab"),
    ("  LIMITER: NONE", "   LIMITER: NONE", abi.EINVAL, b"indentation"),
    ("  LIMITER: NONE", "  LIMITER: NONE\n  LIMITER: BJ", abi.EINVAL, b"duplicate key"),
    ("name: MF", "name: &a MF", abi.EINVAL, b"anchors"),
    ("  FLUX_TYPE: GODUNOV", "  FLUX_TYPE: [GODUNOV", abi.EINVAL, b"expected ','"),
    ("name: 'box mesh.msh'", "name: 'box mesh.msh", abi.EINVAL, b"unterminated"),
])
def test_case_file_errors_like_the_reference(old, new, code, msg):
    assert old in BASE, old
    with pytest.raises(abi.CharmGpuError) as e:
        abi.read_case_yaml(text=BASE.replace(old, new, 1))
    assert e.value.code == code
    assert msg in abi.load().charm_gpu_last_error(), abi.load().charm_gpu_last_error()


def test_concentration_sum_check_is_the_references():
    """The reference tests fabs(sum) - 1 > 1e-12 (src/charm_init_yaml.cpp:249):
    a sum above 1 is an error, a sum below 1 passes; the same here."""
    got = abi.read_case_yaml(text=BASE.replace("concentration: 1.0", "concentration: 0.9", 1))
    assert got.reg[0].c[0] == 0.9


def test_reaction_component_checks():
    text = case_yaml(_cases()["ns_react_mix"])
    assert abi.read_case_yaml(text=text).cfg.n_react == 1
    for bad, msg in (("left: [2]", b"Wrong component number"), ("left: [0, 1, 1, 0]", b"More than 3")):
        with pytest.raises(abi.CharmGpuError):
            abi.read_case_yaml(text=text.replace("left: [0]", bad, 1))
        assert msg in abi.load().charm_gpu_last_error()


def test_case_struct_size_matches_the_header():
    """sizeof(charm_case_t) from the C compiler equals the ctypes mirror."""
    src = '#include <stdio.h>\n#include "charm_gpu.h"\nint main(void){printf("%zu", sizeof(charm_case_t));return 0;}\n'
    with tempfile.TemporaryDirectory() as d:
        c, exe = os.path.join(d, "s.c"), os.path.join(d, "s")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        size = int(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    assert size == C.sizeof(abi.CaseFile)


@pytest.mark.reference
def test_reference_sample_case_file():
    """The reference's own sample case (samples/klin_amr/task.yaml) reads
    into the values it states (comments with non-ASCII text included)."""
    from oracle.build_ref import reference_root
    ref = reference_root()
    sample = os.path.join(ref, "samples", "klin_amr", "task.yaml") if ref else ""
    if not os.path.exists(sample):
        pytest.skip("reference checkout not present")
    got = abi.read_case_yaml(sample)
    c = got.cfg
    assert (c.flux, c.limiter, c.model, c.eos) == (abi.FLUX["HLLC"], abi.LIMITER["BJ"], abi.MODEL["EULER"],
                                                   abi.EOS["IDEAL"])
    assert (c.tau, c.cfl, got.tmax, got.max_error) == (1.0e-2, 0.1, 50.0, 0.01)
    assert (got.refine_period, got.min_level, got.max_level, got.file_output_step) == (10, 0, 1, 100)
    assert got.mesh_type == b"gmsh_msh" and got.mesh_name == b"klin.msh"
    assert c.n_comp == 1 and c.comp[0].m == 0.02869409 and list(c.comp[0].cp[:c.comp[0].n_cp]) == [1014.16]
    assert c.comp[0].h0 == -8.386329e+4 and got.comp_name[0].value == b"AIR"
    names = [got.bnd_name[i].value for i in range(c.n_bnd)]
    assert names == [b"BACK", b"FRONT", b"LEFT", b"RIGHT", b"TOP", b"BOTTOM"]
    assert [c.bnd[i].type for i in range(c.n_bnd)] == [abi.BND[t] for t in (
        "BOUND_WALL_SLIP", "BOUND_WALL_SLIP", "BOUND_INLET", "BOUND_OUTLET", "BOUND_WALL_SLIP", "BOUND_WALL_SLIP")]
    assert list(c.bnd[2].params[:5]) == [697.7082, 0.0, 0.0, 300.0, 101325.0]
    assert got.n_reg == 1 and got.reg[0].name == b"KLIN" and got.reg[0].p == 101325.0 and got.reg[0].c[0] == 1.0
