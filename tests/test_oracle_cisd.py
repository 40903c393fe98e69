"""CISD oracle vs golden vectors produced by the reference's own CISD modules."""
import numpy as np
import pytest

from oracle import cisd_oracle as co
from tests.conftest import load_golden

TOL = 1e-11


@pytest.fixture(params=["cisd_small", "cisd_n20"])
def cg(request):
    return load_golden(request.param)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_cisd_overlap(cg):
    tr = co.CisdTrial(cg["ci1"], cg["ci2"])
    assert _rel(co.overlap(cg["walkers"], tr), cg["overlap"]) < TOL
    assert _rel(co.overlap(cg["walkers"], tr), cg["overlap_meas"]) < TOL


def test_cisd_force_bias(cg):
    tr = co.CisdTrial(cg["ci1"], cg["ci2"])
    assert _rel(co.force_bias(cg["walkers"], tr, cg["chol"]), cg["force_bias"]) < TOL


def test_cisd_energy(cg):
    tr = co.CisdTrial(cg["ci1"], cg["ci2"])
    e = co.energy(cg["walkers"], tr, float(cg["h0"]), cg["h1"], cg["chol"])
    assert _rel(e, cg["energy"]) < TOL


def test_cisd_rdm1(cg):
    tr = co.CisdTrial(cg["ci1"], cg["ci2"])
    g = co.rdm1(cg["walkers"], tr)
    assert _rel(g, cg["rdm1"][:, 0]) < TOL
    assert np.array_equal(cg["rdm1"][:, 0], cg["rdm1"][:, 1])


def test_cisd_model_step_runs_through_the_generic_oracle_step():
    """The CISD model plugs into the generic oracle step: with zero CI
    amplitudes the CISD trial is the reference determinant, so the step equals
    the RHF-trial step on the same walkers and fields."""
    from oracle import afqmc_oracle as ao
    from trot_gb300 import synthetic

    cs = synthetic.make_cisd_system(10, 3, 12, seed=4, h0=0.3)
    tr = co.CisdTrial(np.zeros_like(cs.ci1), np.zeros_like(cs.ci2))
    mo = np.eye(10)[:, :3]
    dm = np.stack([mo @ mo.T, mo @ mo.T])
    prop = ao.build_prop_ctx(cs.h0, cs.h1, cs.chol, dm, 0.01)
    model_c = co.CisdModel(tr, cs.h0, cs.h1, cs.chol, prop)
    model_r = ao.Model("rhf_r", cs.h0, mo, ao.build_rhf_meas_ctx(cs.h1, cs.chol, mo), prop)
    w = synthetic.perturbed_walkers(mo, 4, 0.1, 9)
    x = np.random.default_rng(3).standard_normal((4, 12))
    ov = model_r.overlap(w)
    st = ao.State(w, np.ones(4), ov, 0.1, 0.1)
    p = ao.Params(dt=0.01)
    a = ao.afqmc_step(st, model_c, p, x)
    b = ao.afqmc_step(st, model_r, p, x)
    assert _rel(a.walkers, b.walkers) < 1e-13
    assert _rel(a.weights, b.weights) < 1e-12
    assert _rel(model_c.energy(w), model_r.energy(w)) < 1e-12
