"""Pin the CPU oracle to golden vectors produced by the reference's own code
(tests/golden/make_golden.py runs trot's modules unmodified)."""
import numpy as np
import pytest

from oracle import afqmc_oracle as orc
from oracle import afqmc_oracle as ao
from tests.conftest import load_golden
from tests.golden_model import model_from_golden, rel_err, state_from_golden, walkers_from_golden

TOL = 1e-11


def test_prop_ctx(golden):
    m = model_from_golden(golden)
    assert rel_err(m.prop.mf_shifts, golden["mf_shifts"]) < TOL
    h0p = complex(golden["h0_prop"])
    assert h0p.imag == 0.0
    assert abs(m.prop.h0_prop - h0p.real) < TOL * max(1, abs(h0p.real))
    assert rel_err(m.prop.exp_h1_half, golden["exp_h1_half"]) < TOL


def test_overlap_force_bias_energy(golden):
    m = model_from_golden(golden)
    w = walkers_from_golden(golden)
    assert rel_err(m.overlap(w), golden["overlap"]) < TOL
    assert rel_err(m.force_bias(w), golden["force_bias"]) < TOL
    assert rel_err(m.energy(w), golden["energy"]) < TOL


def test_trotter(golden):
    m = model_from_golden(golden)
    w = walkers_from_golden(golden)
    out = m.trotter(w, golden["trotter_fields"], 6)
    if m.kind == "rhf_r":
        assert rel_err(out, golden["trotter_out"]) < TOL
    else:
        assert rel_err(out[0], golden["trotter_out_u"]) < TOL
        assert rel_err(out[1], golden["trotter_out_d"]) < TOL


def _check_state(st, golden, prefix, kind):
    w = walkers_from_golden(golden, prefix)
    if kind == "rhf_r":
        assert rel_err(st.walkers, w) < TOL
    else:
        assert rel_err(st.walkers[0], w[0]) < TOL
        assert rel_err(st.walkers[1], w[1]) < TOL
    assert rel_err(st.weights, golden[prefix + "weights"]) < TOL
    assert rel_err(st.overlaps, golden[prefix + "overlaps"]) < TOL
    assert abs(st.pop_control_ene_shift - float(golden[prefix + "shift"])) < 1e-9
    assert abs(st.e_estimate - float(golden[prefix + "e_estimate"])) < 1e-9
    assert st.node_encounters == int(golden[prefix + "nodes"])


def test_step(golden):
    m = model_from_golden(golden)
    params = orc.Params(dt=float(golden["dt"]))
    st = orc.afqmc_step(state_from_golden(golden), m, params, golden["step_fields"][0])
    _check_state(st, golden, "step1_", m.kind)


def test_block(golden):
    m = model_from_golden(golden)
    params = orc.Params(dt=float(golden["dt"]))
    st, e_block, w_sum = orc.block(state_from_golden(golden), m, params, golden["step_fields"],
                                   float(golden["zeta"]))
    _check_state(st, golden, "block_", m.kind)
    assert abs(e_block - float(golden["block_energy"])) < 1e-9 * max(1, abs(e_block))
    assert abs(w_sum - float(golden["block_weight"])) < 1e-12 * max(1, w_sum)


def test_block_rdm1(golden):
    """The block's rdm1 observable (weighted average of rdm1_kernel_rw / _uw)."""
    m = model_from_golden(golden)
    params = orc.Params(dt=float(golden["dt"]))
    _, _, _, rdm1 = orc.block(state_from_golden(golden), m, params, golden["step_fields"], float(golden["zeta"]),
                              rdm1=True)
    assert rel_err(rdm1, golden["block_rdm1"]) < 1e-11


def test_qr_and_sr(golden):
    m = model_from_golden(golden)
    w = walkers_from_golden(golden)
    q, norm = orc.orthogonalize(w, m.walker_kind)
    if m.kind == "rhf_r":
        assert rel_err(q, golden["qr_out"]) < 1e-12
    else:
        assert rel_err(q[0], golden["qr_out_u"]) < 1e-12
        assert rel_err(q[1], golden["qr_out_d"]) < 1e-12
    assert rel_err(norm, golden["qr_norm"]) < 1e-12
    sr_w = golden["sr_weights_in"]
    idx = orc.sr_indices(sr_w, float(golden["sr_zeta"]), sr_w.shape[0])
    np.testing.assert_array_equal(idx, golden["sr_idx"])
    _, wn, _ = orc.stochastic_reconfiguration(w, sr_w, float(golden["sr_zeta"]), m.walker_kind)
    np.testing.assert_array_equal(wn, golden["sr_weights_out"])


def test_init_walkers(golden):
    m = model_from_golden(golden)
    mo_a, mo_b = golden["mo_a"], golden["mo_b"]
    rdm1 = np.stack([mo_a @ mo_a.T, mo_b @ mo_b.T])
    na, nb = mo_a.shape[1], mo_b.shape[1]
    iw = orc.init_walkers(m.walker_kind, rdm1, na, nb, 2)
    # eigenvectors are unique up to sign: compare the projectors w w^H
    if m.kind == "rhf_r":
        pairs = [(iw, golden["init_walkers"])]
    else:
        pairs = [(iw[0], golden["init_walkers_u"]), (iw[1], golden["init_walkers_d"])]
    for a, b in pairs:
        pa = a @ np.conj(np.swapaxes(a, -1, -2))
        pb = b @ np.conj(np.swapaxes(b, -1, -2))
        assert rel_err(pa, pb) < 1e-10


@pytest.mark.parametrize("name", ["fp_rhf_r", "fp_uhf_u"])
def test_oracle_free_projection_step(name):
    _rel = rel_err
    """afqmc_step_fp, qr_norm and multiply_constants vs the reference's own
    free-projection modules (trot/prop/afqmc_fp.py, trot/walkers.py:182-227)."""
    g = load_golden(name)
    kind = str(g["kind"])
    wk = "restricted" if kind == "rhf_r" else "unrestricted"
    w = g["walkers"] if kind == "rhf_r" else (g["walkers_u"], g["walkers_d"])
    mo = g["mo_a"] if kind != "uhf_u" else (g["mo_a"], g["mo_b"])
    tmo = g["mo_a"] if kind == "rhf_r" else mo
    if kind == "uhf_u":
        dm = np.stack([g["mo_a"] @ g["mo_a"].T, g["mo_b"] @ g["mo_b"].T])
    else:
        dm = np.stack([g["mo_a"] @ g["mo_a"].T] * 2)
    prop = ao.build_prop_ctx(float(g["h0"]), g["h1"], g["chol"], dm, float(g["dt"]))
    prop = ao.PropCtx(prop.dt, prop.sqrt_dt, prop.exp_h1_half, prop.mf_shifts, prop.h0_prop + float(g["ene0"]),
                      prop.chol_flat, prop.norb)
    assert abs(prop.h0_prop - float(np.real(g["h0_prop"]))) <= 1e-12 * abs(prop.h0_prop)
    model = ao.Model(kind, float(g["h0"]), tmo, None, prop)
    st = ao.State(w, g["weights"], np.ones(len(g["weights"]), complex), 0.0, 0.0)
    out = ao.afqmc_step_fp(st, model, g["fields"], float(g["zeta"]))
    assert _rel(out.weights, g["out_weights"]) < 1e-11
    if kind == "rhf_r":
        assert _rel(out.walkers, g["out_walkers"]) < 1e-11
        assert _rel(ao.multiply_constants(w, g["mc_constants"], wk), g["mc_out"]) < 1e-14
    else:
        assert _rel(out.walkers[0], g["out_walkers_u"]) < 1e-11
        assert _rel(out.walkers[1], g["out_walkers_d"]) < 1e-11
        mc = ao.multiply_constants(w, g["mc_constants"], wk)
        assert _rel(mc[0], g["mc_out_u"]) < 1e-14 and _rel(mc[1], g["mc_out_d"]) < 1e-14
    assert _rel(ao.qr_norm(w, wk), g["qr_norm"]) < 1e-12
