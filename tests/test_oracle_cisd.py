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
