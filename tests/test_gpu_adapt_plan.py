"""Adapt with the state on the device: charm_gpu_density_means feeds the
host's plan (charm_host_forest_adapt_plan) and charm_gpu_adapt_upload
carries the device state through it.  The result must equal the host path
(adapt_state on the downloaded state, then upload and set_state) bit for bit
in FP64, and equal the mixed form's own host path; over several adapt and
step rounds that refine, coarsen and balance."""
import numpy as np
import pytest

from charm_3d_gb300.solver import Forest, Solver

from .common import amr_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,prec", [("sod", "FP64"), ("random", "FP64"), ("mix2", "FP64"), ("sod", "MIXED"),
                                       ("random", "MIXED")])
def test_device_adapt_matches_host_adapt(kind, prec):
    case = amr_case(kind, level=2, max_level=4, max_err=0.05 if kind == "sod" else 0.3)
    case.precision = prec
    fh, fd = Forest(case), Forest(case)
    mesh = fh.flatten()
    u0 = case.initial_state(mesh.center)
    gh, gd = Solver(case), Solver(case)
    for g in (gh, gd):
        g.upload(mesh)
        g.set_state(u0)
    for rnd in range(4):
        for g in (gh, gd):
            g.run(2, case.tau)
        # host path: download, project on the host, upload
        _, grad = gh.refine_flags(case.max_err)
        u = fh.adapt_state(grad, case.max_err, case.min_level, case.max_level, case.n_comp, gh.get_state())
        mh = fh.flatten()
        gh.upload(mh)
        gh.set_state(u)
        # device path
        _, grad_d = gd.refine_flags(case.max_err)
        assert np.array_equal(grad, grad_d)
        rho = gd.density_means()
        n, plan = fd.adapt_plan(grad_d, rho, case.max_err, case.min_level, case.max_level)
        md = fd.flatten()
        gd.adapt_upload(plan, md)
        assert n == mh.n_elem == md.n_elem
        assert np.array_equal(mh.level, md.level)
        a, b = gd.get_state(), gh.get_state()
        assert np.array_equal(a, b), f"round {rnd}"
    for g in (gh, gd):
        g.close()


def test_adapt_upload_rejects_a_foreign_plan():
    case = amr_case("sod", level=2, max_level=4)
    f = Forest(case)
    mesh = f.flatten()
    g = Solver(case)
    g.upload(mesh)
    g.set_state(case.initial_state(mesh.center))
    _, grad = g.refine_flags(case.max_err)
    n, plan = f.adapt_plan(grad, g.density_means(), case.max_err, case.min_level, case.max_level)
    m2 = f.flatten()
    g.adapt_upload(plan, m2)             # consistent: accepted
    from charm_3d_gb300.abi import CharmGpuError
    with pytest.raises(CharmGpuError):   # the plan's input is the old mesh, not the uploaded one
        g.adapt_upload(plan, m2)
    g.close()
