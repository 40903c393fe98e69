"""Generate golden vectors by running the reference's own trot modules.

Run in a container that has the trot sources (argument 1, or the TROT_REFERENCE
environment variable; required) but no jax: ``_jaxshim`` supplies numpy-backed jax names, and
the reference functions (trot/meas/{rhf,uhf}.py, trot/trial/{rhf,uhf}.py,
trot/prop/{afqmc,chol_afqmc_ops,blocks}.py, trot/walkers.py) run unmodified.
Fields and SR zeta are injected. Outputs go to tests/golden/*.npz next to this
script; the tests read only those files (the reference is not needed at test
time).

    python tests/golden/make_golden.py /path/to/trot [fp|cisd]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import _jaxshim  # noqa: E402

_jaxshim.install()
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TROT_REFERENCE", "")
if not REF or not os.path.isdir(os.path.join(REF, "trot")):
    sys.exit("usage: make_golden.py /path/to/trot [fp|cisd]  (the directory that holds the trot package; "
             "or set TROT_REFERENCE)")
sys.path.insert(0, REF)

from trot.core.system import System  # noqa: E402
from trot.ham.chol import HamChol  # noqa: E402
from trot.meas import rhf as mrhf  # noqa: E402
from trot.meas import uhf as muhf  # noqa: E402
from trot.prop import blocks  # noqa: E402
from trot.prop.afqmc import make_prop_ops  # noqa: E402
from trot.prop.chol_afqmc_ops import _build_prop_ctx, make_trotter_ops  # noqa: E402
from trot.prop.types import PropState, QmcParams  # noqa: E402
from trot.trial import rhf as trhf  # noqa: E402
from trot.trial import uhf as tuhf  # noqa: E402
from trot import walkers as wk  # noqa: E402

from trot_gb300 import synthetic  # noqa: E402
from trot.meas import cisd as mcisd  # noqa: E402
from trot.trial import cisd as tcisd  # noqa: E402

INJ = _jaxshim.INJECT


def _vm(fn, *args):
    return np.asarray(_jaxshim.vmap(fn, in_axes=(0,) + (None,) * (len(args) - 1))(*args))


def case(name, norb, nelec, nchol, n_walkers, kind, dt=0.01, n_steps=3, h0=0.7, seed=0):
    ss = synthetic.make_system(norb, nelec, nchol, decay=30.0, seed=seed, h0=h0)
    ham = HamChol(h0=np.asarray(h0), h1=ss.h1, chol=ss.chol, basis="restricted")
    walker_kind = "restricted" if kind == "rhf_r" else "unrestricted"
    sysm = System(norb=norb, nelec=nelec, walker_kind=walker_kind)
    rng = np.random.default_rng(seed + 100)
    out = dict(h0=h0, h1=ss.h1, chol=ss.chol, mo_a=ss.mo_a, mo_b=ss.mo_b, dt=dt,
               kind=np.array(kind))
    if kind == "uhf_u":
        trial = tuhf.UhfTrial(ss.mo_a, ss.mo_b)
        meas_ops = muhf.make_uhf_meas_ops(sysm)
        trial_ops = tuhf.make_uhf_trial_ops(sysm)
    else:
        trial = trhf.RhfTrial(ss.mo_a)
        meas_ops = mrhf.make_rhf_meas_ops(sysm)
        trial_ops = trhf.make_rhf_trial_ops(sysm)
    meas_ctx = meas_ops.build_meas_ctx(ham, trial)
    rdm1 = trial_ops.get_rdm1(trial)
    prop_ctx = _build_prop_ctx(ham, rdm1, dt)
    out.update(mf_shifts=prop_ctx.mf_shifts, h0_prop=prop_ctx.h0_prop,
               exp_h1_half=prop_ctx.exp_h1_half)

    if kind == "rhf_r":
        w = synthetic.perturbed_walkers(ss.mo_a, n_walkers, 0.15, seed + 1)
        walkers = w
        out.update(walkers=w)
    else:
        wu = synthetic.perturbed_walkers(ss.mo_a, n_walkers, 0.15, seed + 1)
        wd = synthetic.perturbed_walkers(ss.mo_b, n_walkers, 0.15, seed + 2)
        walkers = (wu, wd)
        out.update(walkers_u=wu, walkers_d=wd)

    fb_k = meas_ops.require_kernel("force_bias")
    e_k = meas_ops.require_kernel("energy")
    vm = _jaxshim.vmap
    out["overlap"] = np.asarray(vm(meas_ops.overlap, in_axes=(0, None))(walkers, trial))
    out["force_bias"] = np.asarray(vm(fb_k, in_axes=(0, None, None, None))(walkers, ham, meas_ctx, trial))
    out["energy"] = np.asarray(vm(e_k, in_axes=(0, None, None, None))(walkers, ham, meas_ctx, trial))

    # Trotter action with given complex shifted fields
    xs = rng.normal(size=(n_walkers, nchol)) + 0.3j * rng.normal(size=(n_walkers, nchol))
    trot = make_trotter_ops("restricted", walker_kind)
    wt = vm(trot.apply_trotter, in_axes=(0, 0, None, None))(walkers, xs, prop_ctx, 6)
    out["trotter_fields"] = xs
    if kind == "rhf_r":
        out["trotter_out"] = np.asarray(wt)
    else:
        out["trotter_out_u"], out["trotter_out_d"] = np.asarray(wt[0]), np.asarray(wt[1])

    # one phaseless step and one block with injected fields / zeta
    params = QmcParams(dt=dt, n_chunks=1, n_exp_terms=6, n_prop_steps=n_steps,
                       n_walkers=n_walkers, seed=0)
    prop_ops = make_prop_ops("restricted", walker_kind)
    weights = 0.5 + rng.uniform(size=n_walkers)
    state = PropState(walkers=walkers, weights=weights, overlaps=out["overlap"],
                      rng_key=np.array([0, 0], np.uint32), pop_control_ene_shift=np.asarray(-0.3 + h0),
                      e_estimate=np.asarray(float(np.real(out["energy"][0]))),
                      node_encounters=np.asarray(0))
    out.update(state_weights=weights, state_shift=float(state.pop_control_ene_shift),
               state_e_estimate=float(state.e_estimate))
    step_fields = rng.standard_normal((n_steps, n_walkers, nchol))
    out["step_fields"] = step_fields
    INJ.clear()
    INJ.append(step_fields[0])
    s1 = prop_ops.step(state, params=params, ham_data=ham, trial_data=trial, trial_ops=trial_ops,
                       meas_ops=meas_ops, meas_ctx=meas_ctx, prop_ctx=prop_ctx)
    _save_state(out, "step1_", s1, kind)

    zeta = float(rng.uniform())
    out["zeta"] = zeta
    INJ.clear()
    for k in range(n_steps):
        INJ.append(step_fields[k])
    INJ.append(np.asarray(zeta))
    sb, obs = blocks.block(state, sys=sysm, params=params, ham_data=ham, trial_data=trial,
                           trial_ops=trial_ops, meas_ops=meas_ops, meas_ctx=meas_ctx,
                           prop_ops=prop_ops, prop_ctx=prop_ctx)
    assert not INJ
    _save_state(out, "block_", sb, kind)
    out["block_energy"] = float(obs.scalars["energy"])
    out["block_weight"] = float(obs.scalars["weight"])
    # the same block with the rdm1 observable (weighted average of rdm1_kernel_* over the walkers)
    for k in range(n_steps):
        INJ.append(step_fields[k])
    INJ.append(np.asarray(zeta))
    _, obs_r = blocks.block(state, sys=sysm, params=params, ham_data=ham, trial_data=trial,
                            trial_ops=trial_ops, meas_ops=meas_ops, meas_ctx=meas_ctx,
                            prop_ops=prop_ops, prop_ctx=prop_ctx, observable_names=("rdm1",))
    assert not INJ
    out["block_rdm1"] = np.asarray(obs_r.observables["rdm1"])

    # QR with phase convention, SR alone
    q, norm = wk.orthogonalize(walkers, walker_kind)
    if kind == "rhf_r":
        out["qr_out"] = np.asarray(q)
    else:
        out["qr_out_u"], out["qr_out_d"] = np.asarray(q[0]), np.asarray(q[1])
    out["qr_norm"] = np.asarray(norm)
    sr_w = rng.uniform(size=n_walkers) * (rng.uniform(size=n_walkers) > 0.2)
    sr_zeta = float(rng.uniform())
    w_sr, weights_sr = wk.stochastic_reconfiguration(walkers, sr_w, sr_zeta, walker_kind)
    out.update(sr_weights_in=sr_w, sr_zeta=sr_zeta, sr_weights_out=np.asarray(weights_sr),
               sr_idx=np.asarray(wk._sr_indices(sr_w, sr_zeta, n_walkers)))
    # initial walkers (natural orbitals of the trial density)
    iw = wk.init_walkers(sysm, rdm1, 2)
    if kind == "rhf_r":
        out["init_walkers"] = np.asarray(iw)
    else:
        out["init_walkers_u"], out["init_walkers_d"] = np.asarray(iw[0]), np.asarray(iw[1])
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in out.items()})
    print(f"wrote {path}: {os.path.getsize(path) / 1e3:.0f} kB")


def _save_state(out, prefix, st, kind):
    if kind == "rhf_r":
        out[prefix + "walkers"] = np.asarray(st.walkers)
    else:
        out[prefix + "walkers_u"] = np.asarray(st.walkers[0])
        out[prefix + "walkers_d"] = np.asarray(st.walkers[1])
    out[prefix + "weights"] = np.asarray(st.weights)
    out[prefix + "overlaps"] = np.asarray(st.overlaps)
    out[prefix + "shift"] = float(st.pop_control_ene_shift)
    out[prefix + "e_estimate"] = float(st.e_estimate)
    out[prefix + "nodes"] = int(st.node_encounters)


def fp_case(name, norb, nelec, nchol, n_walkers, kind, dt=0.02, ene0=-1.3, seed=3, h0=0.5):
    """One free-projection step (trot/prop/afqmc_fp.py) with injected fields and zeta."""
    from trot.prop.afqmc_fp import make_prop_ops_fp
    from trot.prop.types import QmcParamsFp

    ss = synthetic.make_system(norb, nelec, nchol, decay=30.0, seed=seed, h0=h0)
    ham = HamChol(h0=np.asarray(h0), h1=ss.h1, chol=ss.chol, basis="restricted")
    walker_kind = "restricted" if kind == "rhf_r" else "unrestricted"
    sysm = System(norb=norb, nelec=nelec, walker_kind=walker_kind)
    if kind == "uhf_u":
        trial, trial_ops = tuhf.UhfTrial(ss.mo_a, ss.mo_b), tuhf.make_uhf_trial_ops(sysm)
    else:
        trial, trial_ops = trhf.RhfTrial(ss.mo_a), trhf.make_rhf_trial_ops(sysm)
    params = QmcParamsFp(dt=dt, n_walkers=n_walkers, ene0=ene0, n_exp_terms=6, seed=0)
    prop_ops = make_prop_ops_fp("restricted", walker_kind, sysm)
    rdm1 = trial_ops.get_rdm1(trial)
    ctx = prop_ops.build_prop_ctx(ham, rdm1, params)
    rng = np.random.default_rng(seed + 7)
    wu = synthetic.perturbed_walkers(ss.mo_a, n_walkers, 0.2, seed + 1)
    wd = synthetic.perturbed_walkers(ss.mo_b, n_walkers, 0.2, seed + 2)
    walkers = wu if kind == "rhf_r" else (wu, wd)
    weights = 0.5 + rng.uniform(size=n_walkers)
    fields = rng.standard_normal((n_walkers, nchol))
    zeta = float(rng.uniform())
    state = PropState(walkers=walkers, weights=weights, overlaps=np.ones(n_walkers, np.complex128),
                      rng_key=np.array([0, 0], np.uint32), pop_control_ene_shift=np.asarray(0.0),
                      e_estimate=np.asarray(0.0), node_encounters=np.asarray(0))
    INJ.clear()
    INJ.append(fields)
    INJ.append(np.asarray(zeta))
    out_state = prop_ops.step(state, params=params, ham_data=ham, trial_data=trial, trial_ops=trial_ops,
                              meas_ops=None, meas_ctx=None, prop_ctx=ctx)
    assert not INJ
    out = dict(h0=h0, h1=ss.h1, chol=ss.chol, mo_a=ss.mo_a, mo_b=ss.mo_b, dt=dt, ene0=ene0, kind=np.array(kind),
               fields=fields, zeta=zeta, weights=weights, h0_prop=np.asarray(ctx.h0_prop),
               out_weights=np.asarray(out_state.weights))
    if kind == "rhf_r":
        out.update(walkers=wu, out_walkers=np.asarray(out_state.walkers))
    else:
        out.update(walkers_u=wu, walkers_d=wd, out_walkers_u=np.asarray(out_state.walkers[0]),
                   out_walkers_d=np.asarray(out_state.walkers[1]))
    out["qr_norm"] = np.asarray(wk.qr_norm(walkers, walker_kind))
    consts = np.exp(0.3j * rng.standard_normal(n_walkers) + 0.1 * rng.standard_normal(n_walkers))
    mc = wk.multiply_constants(walkers, consts, walker_kind)
    out["mc_constants"] = consts
    if kind == "rhf_r":
        out["mc_out"] = np.asarray(mc)
    else:
        out["mc_out_u"], out["mc_out_d"] = np.asarray(mc[0]), np.asarray(mc[1])
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in out.items()})
    print(f"wrote {path}: {os.path.getsize(path) / 1e3:.0f} kB")


def cisd_case(name, norb, nocc, nchol, n_walkers, seed=0, h0=0.4, noise=0.1):
    cs = synthetic.make_cisd_system(norb, nocc, nchol, decay=30.0, seed=seed, h0=h0)
    ham = HamChol(h0=np.asarray(h0), h1=cs.h1, chol=cs.chol, basis="restricted")
    sysm = System(norb=norb, nelec=(nocc, nocc), walker_kind="restricted")
    trial = tcisd.CisdTrial(ci1=cs.ci1, ci2=cs.ci2)
    meas_ops = mcisd.make_cisd_meas_ops(sysm, memory_mode="high", mixed_precision=False, testing=True)
    trial_ops = tcisd.make_cisd_trial_ops(sysm)
    meas_ctx = meas_ops.build_meas_ctx(ham, trial)
    ref = np.eye(norb)[:, :nocc]
    w = synthetic.perturbed_walkers(ref, n_walkers, noise, seed + 5)
    vm = _jaxshim.vmap
    out = dict(h0=h0, h1=cs.h1, chol=cs.chol, ci1=cs.ci1, ci2=cs.ci2, walkers=w)
    out["overlap"] = np.asarray(vm(trial_ops.overlap, in_axes=(0, None))(w, trial))
    out["overlap_meas"] = np.asarray(vm(meas_ops.overlap, in_axes=(0, None))(w, trial))
    out["force_bias"] = np.asarray(vm(meas_ops.require_kernel("force_bias"), in_axes=(0, None, None, None))(
        w, ham, meas_ctx, trial))
    out["energy"] = np.asarray(vm(meas_ops.require_kernel("energy"), in_axes=(0, None, None, None))(
        w, ham, meas_ctx, trial))
    out["rdm1"] = np.asarray(vm(meas_ops.require_observable("rdm1"), in_axes=(0, None, None, None))(
        w, ham, meas_ctx, trial))
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in out.items()})
    print(f"wrote {path}: {os.path.getsize(path) / 1e3:.0f} kB")


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "fp":
        fp_case("fp_rhf_r", norb=10, nelec=(3, 3), nchol=16, n_walkers=6, kind="rhf_r")
        fp_case("fp_uhf_u", norb=11, nelec=(4, 2), nchol=18, n_walkers=5, kind="uhf_u")
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == "cisd":
        cisd_case("cisd_small", norb=12, nocc=3, nchol=20, n_walkers=4)
        cisd_case("cisd_n20", norb=20, nocc=5, nchol=50, n_walkers=3, seed=1)
        sys.exit(0)
    cisd_case("cisd_small", norb=12, nocc=3, nchol=20, n_walkers=4)
    cisd_case("cisd_n20", norb=20, nocc=5, nchol=50, n_walkers=3, seed=1)
    fp_case("fp_rhf_r", norb=10, nelec=(3, 3), nchol=16, n_walkers=6, kind="rhf_r")
    fp_case("fp_uhf_u", norb=11, nelec=(4, 2), nchol=18, n_walkers=5, kind="uhf_u")
    case("rhf_r_small", norb=10, nelec=(3, 3), nchol=16, n_walkers=5, kind="rhf_r")
    case("rhf_u_small", norb=9, nelec=(3, 3), nchol=14, n_walkers=4, kind="rhf_u")
    case("uhf_u_small", norb=11, nelec=(4, 2), nchol=18, n_walkers=5, kind="uhf_u")
    case("rhf_r_n24", norb=24, nelec=(5, 5), nchol=120, n_walkers=4, kind="rhf_r", dt=0.005,
         n_steps=2)
    case("uhf_u_n20", norb=20, nelec=(5, 3), nchol=60, n_walkers=4, kind="uhf_u", dt=0.005,
         n_steps=2)
