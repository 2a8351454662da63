"""The drop-in on the GPU: the reference's own time loop stepping through the
GPU model plugin.

oracle/_ref/libcharm_ref_plugin.so is the reference's C sources built with
the plugin (charm_3d_gb300/csrc/plugin/charm_model_gpu.c) and linked to
libcharm_gpu.so.  ref_run is the loop of charm_timesteps
(src/charm_timesteps.c:32-47) calling ctx->timestep_single_fn; after
ref_plugin_use_gpu that is charm_model_gpu_timestep_single, which flattens
the forest through p4est_iterate, uploads it, steps on the GPU and, every
REFINE_PERIOD steps, brings the state back for the reference's own
charm_adapt.  The reference's own model (libcharm_ref.so, the CPU
timestep_single_fn) from the same state is the comparison, at the drop-in's
bar of 1e-12 relative L2.

Needs the reference checkout (to build oracle/_ref) and a GPU.
"""
import numpy as np
import pytest

from charm_3d_gb300 import abi, synthetic
from charm_3d_gb300.solver import Forest
from oracle.ref import RefSolver

from .common import rel_l2, small_case
from .golden_cases import HEX_AMR_STEPS, hex_case

pytestmark = [pytest.mark.gpu, pytest.mark.reference]
TOL = 1e-12


def _u0(case):
    """The seeded state on the leaves in the forest's order (the order of
    the reference build's quadrants)."""
    return case.initial_state(Forest(case).flatten().center)


def _cpu(case, u0, steps, hexmesh=None, variant="ref"):
    """The reference's own model; variant "patched" where hanging faces meet
    the limiter (its species slots filled, as the GPU limiter does)."""
    ref = RefSolver(case, variant, hexmesh=hexmesh)
    ref.set_state(u0)
    ref.run(steps)
    return ref.get_state(), ref.leaves()


def _plugin(case, u0, steps, precision="FP64", hexmesh=None):
    ref = RefSolver(case, "plugin", hexmesh=hexmesh)
    ref.set_state(u0)
    ref.plugin_use_gpu(abi.PRECISION[precision])
    ref.run(steps)
    assert ref.plugin_finish() == 0
    return ref.get_state(), ref.leaves()


def test_plugin_config1_sod_every_step_matches_reference():
    """Config 1 (Sod tube, level 4, LF, BJ, outlet boundaries), all 100
    steps: each step from the plugin's previous state, once through the
    plugin on the GPU and once through the reference's own model.  (End
    states of separate 100-step runs differ by limiter switches that a
    1e-12 perturbation already flips, in the reference itself.)"""
    case = synthetic("sod")
    u = _u0(case)
    worst = 0.0
    for n in range(case.steps):
        want, _ = _cpu(case, u, 1)
        got, _ = _plugin(case, u, 1)
        worst = max(worst, rel_l2(got, want))
        u = got
    assert worst <= TOL


@pytest.mark.parametrize("kind,flux,lim,model", [("walls", "HLLC", "BJ", "NS"), ("random", "LF", "NONE", "EULER"),
                                                 ("mix2", "HLLC", "BJ", "NS")])
def test_plugin_steps_match_reference(kind, flux, lim, model):
    case = small_case(kind, flux, lim, model=model)
    u0 = _u0(case)
    want, lw = _cpu(case, u0, 3)
    got, lg = _plugin(case, u0, 3)
    assert np.array_equal(lw, lg)
    assert rel_l2(got, want) < TOL


def test_plugin_adapt_every_period_matches_reference():
    """REFINE_PERIOD 2 on the Sod tube (LF, BJ): the plugin brings the state
    back, runs the reference's charm_adapt on the CPU, flattens the new
    forest (hanging faces) and uploads it; the same leaves and states as the
    reference's own loop."""
    case = small_case("sod", "LF", "BJ", level=3)
    case.min_level, case.max_level, case.refine_period, case.max_err = 3, 4, 2, 0.05
    u0 = _u0(case)
    want, lw = _cpu(case, u0, 6, variant="patched")
    got, lg = _plugin(case, u0, 6)
    assert len(lw) > 8 ** 3, "the run refined"
    assert np.array_equal(lw, lg)
    assert rel_l2(got, want) < TOL


def test_plugin_general_hexahedra_match_reference():
    """The reference's sample geometry (ramp channel, trees in random
    orientations, Euler, HLLC, BJ): the plugin takes the forest to the
    general-hexahedron kernels."""
    case, _, _, u0, hexmesh = hex_case("hex_ramp_hllc_bj")
    want, _ = _cpu(case, u0, 5, hexmesh)
    got, _ = _plugin(case, u0, 5, hexmesh=hexmesh)
    assert rel_l2(got, want) < TOL


def test_plugin_sample_case_amr_on_hexahedra_matches_reference():
    """The sample case's AMR controls (MAX_ERROR 0.01, MAX_LEVEL 1,
    REFINE_PERIOD 10) on the ramp: adapts by the reference's charm_adapt
    between GPU steps on general hexahedra with mortars."""
    case, _, _, u0, hexmesh = hex_case("hex_ramp_amr")
    case.max_err, case.min_level, case.max_level, case.refine_period = 0.01, 0, 1, 10
    want, lw = _cpu(case, u0, HEX_AMR_STEPS, hexmesh, variant="patched")
    got, lg = _plugin(case, u0, HEX_AMR_STEPS, hexmesh=hexmesh)
    assert (lw[:, 4] == 1).any(), "the shock off the ramp refines"
    assert np.array_equal(lw, lg)
    assert rel_l2(got, want) < TOL


def test_plugin_mixed_precision_within_its_bar():
    """NS_GPU_MIXED through the plugin: within the mixed form's 1e-6."""
    case = small_case("walls", "HLLC", "BJ")
    u0 = _u0(case)
    want, _ = _cpu(case, u0, 3)
    got, _ = _plugin(case, u0, 3, precision="MIXED")
    err = rel_l2(got, want)
    assert 0.0 < err < 1e-6
