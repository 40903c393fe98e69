"""Walker-steps/s of the phaseless-AFQMC hot path (prop + E_L every step).

Default workload: UHF trial, N=120 orbitals, (12, 10) electrons, G=600
Cholesky vectors (decay length 150), 1024 walkers, dt=0.005, QR + block tail
(overlaps, block energy, SR) every 10 steps; seeded synthetic Hamiltonian.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
                    [--impl ours|reference] [--config NAME]

Prints one JSON line (rank 0).  Under torchrun with N > 1 every rank runs an
independent replica of the workload (the path does not shard), the timed
region is bracketed by barriers, and the max time over ranks is used.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "walker-steps/s (prop+E_L), mixed vs FP64 on 1 GB300 at |ΔE_L|≤1e-5 Ha"
UNIT = "walker-steps/s"


def flops_per_walker_step(N, na, nb, G, nterms=6):
    """Algorithmic flops of one walker-step (reference contraction order;
    complex x real = 4 flop per MAC, complex x complex = 8)."""
    ns, sq = na + nb, na * na + nb * nb
    d = {
        "green": 4 * N * sq + 8 * sq * N,
        "force_bias": 4 * G * ns * N,
        "vhs": 4 * G * N * N,
        "taylor": nterms * 8 * N * N * ns,
        "onebody": 2 * 4 * N * N * ns,
        "overlap": 4 * N * sq + 6 * (na ** 3 + nb ** 3),
        "exchange": 4 * G * sq * N,
        "energy_rest": 8 * G * sq + 8 * ns * N,
    }
    return d


def flops_per_walker_step_cisd(N, n, G, nterms=6):
    """Algorithmic flops of one CISD walker-step (trot/meas/cisd.py:608-769 contraction
    order: the two l2ci2 quadratic forms, glgp, gl, lci2_green, ... plus the propagation)."""
    v = N - n
    nv = n * v
    d = {
        "l2ci2": 2 * 4 * G * nv * nv,
        "glgp": 8 * G * n * N * v,
        "gl": 4 * G * n * N * N,
        "lci2_green": 4 * G * n * N * N,
        "lg1": 4 * G * n * n * N,
        "chol_contract": 3 * 4 * G * N * N,
        "ci2g": 2 * 4 * nv * nv,
        "mats": 2 * 8 * N * N * n,
        "vhs": 4 * G * N * N,
        "taylor": nterms * 8 * N * N * n,
        "onebody": 2 * 4 * N * N * n,
    }
    return d


# DRAM bytes per launch of the dominant kernel, measured by ncu on the named workload (one counter
# pass; command and numbers in profiles/exchange_exact_tc_uhf_n120_w256.md, full-size launch)
NCU_DRAM_BYTES = {("cfg2_uhf_n120", "mixed", "exchange_exact_tc"): ((41.464 + 0.320) + (39.818 + 0.017)) / 2 * 1e6}


def exchange_tensor_flops(cfg, W):
    """FP16 tensor flops the exact-digit exchange kernel issues per launch (mean over spins):
    per (128-row Cholesky tile, walker tile of P columns) the 15 digit products t + u <= 4 of
    128 x P x 128, issued as five MMAs per K16 step with the Green's-function planes stacked
    along N (P = 48; 32 for n_pad = 16; n_pad = 4, 8, 12 or 16)."""
    N, (na, nb), G = cfg["norb"], cfg["nelec"], cfg["nchol"]
    spins = [na] if cfg["kind"] == "rhf_r" else [na, nb]
    tot = 0
    for n in spins:
        n_pad = 4 if n <= 4 else 8 if n <= 8 else 12 if n <= 12 else 16
        P = 32 if n_pad == 16 else 48
        wb = P // (2 * n_pad)
        gb = max(1, 128 // n)
        tot += 15 * 2 * 128 * P * 128 * ((W + wb - 1) // wb) * ((G + gb - 1) // gb)
    return tot / len(spins)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------
def build_workload(cfg, precision):
    import torch

    import trot_gb300 as tg
    from trot_gb300 import synthetic

    N, (na, nb), G, W = cfg["norb"], cfg["nelec"], cfg["nchol"], cfg["n_walkers"]
    kind = cfg["kind"]
    if kind == "cisd":
        return build_workload_cisd(cfg, precision)
    ss = synthetic.make_system(N, (na, nb), G, decay=cfg["decay"], seed=0, h0=0.0)
    wk = "restricted" if kind == "rhf_r" else "unrestricted"
    sysm = tg.System(norb=N, nelec=(na, nb), walker_kind=wk)
    ham = tg.HamChol(h0=ss.h0, h1=ss.h1, chol=ss.chol)
    params = tg.QmcParams(dt=cfg["dt"], n_walkers=W, n_prop_steps=cfg["qr_every"], seed=1234)
    mixed = precision == "mixed"
    if kind == "uhf_u":
        trial = tg.UhfTrial(ss.mo_a, ss.mo_b)
        trial_ops, meas_ops = tg.make_uhf_trial_ops(sysm), tg.make_uhf_meas_ops(sysm, mixed_precision=mixed)
    else:
        trial = tg.RhfTrial(ss.mo_a)
        trial_ops = tg.make_rhf_trial_ops(sysm)
        meas_ops = tg.make_rhf_meas_ops(sysm, mixed_precision=mixed)
    meas_ctx = meas_ops.build_meas_ctx(ham, trial)
    prop_ops = tg.make_prop_ops("restricted", wk, mixed_precision=(precision == "mixed"))
    prop_ctx = prop_ops.build_prop_ctx(ham, trial_ops.get_rdm1(trial), params)
    state = prop_ops.init_prop_state(sys=sysm, ham_data=ham, trial_ops=trial_ops, trial_data=trial,
                                     meas_ops=meas_ops, params=params)
    e = torch.empty(W, dtype=torch.complex128, device="cuda")
    return dict(tg=tg, ss=ss, sys=sysm, ham=ham, params=params, trial=trial, trial_ops=trial_ops,
                meas_ops=meas_ops, meas_ctx=meas_ctx, prop_ops=prop_ops, prop_ctx=prop_ctx, state=state, e=e,
                W=W, N=N, na=na, nb=nb, G=G, qr_every=cfg["qr_every"], kind=kind)


def build_workload_cisd(cfg, precision):
    """CISD trial (N, nocc, G) with restricted walkers; "mixed" = the reference's
    default CISD dtypes (tensor-core l2ci2, FP32 gl) and tensor-core propagation,
    "fp64" = testing=True and FP64 propagation."""
    import torch

    import trot_gb300 as tg
    from trot_gb300 import synthetic

    N, (n, _), G, W = cfg["norb"], cfg["nelec"], cfg["nchol"], cfg["n_walkers"]
    cs = synthetic.make_cisd_system(N, n, G, decay=cfg["decay"], seed=0, h0=0.0)
    sysm = tg.System(norb=N, nelec=(n, n), walker_kind="restricted")
    ham = tg.HamChol(h0=cs.h0, h1=cs.h1, chol=cs.chol)
    params = tg.QmcParams(dt=cfg["dt"], n_walkers=W, n_prop_steps=cfg["qr_every"], seed=1234)
    trial = tg.CisdTrial(cs.ci1, cs.ci2)
    trial_ops = tg.make_cisd_trial_ops(sysm)
    if precision == "mixed":
        meas_ops = tg.make_cisd_meas_ops(sysm)
    else:
        meas_ops = tg.make_cisd_meas_ops(sysm, mixed_precision=False, testing=True)
    meas_ctx = meas_ops.build_meas_ctx(ham, trial)
    prop_ops = tg.make_prop_ops("restricted", "restricted", mixed_precision=(precision == "mixed"))
    prop_ctx = prop_ops.build_prop_ctx(ham, trial_ops.get_rdm1(trial), params)
    state = prop_ops.init_prop_state(sys=sysm, ham_data=ham, trial_ops=trial_ops, trial_data=trial,
                                     meas_ops=meas_ops, params=params)
    e = torch.empty(W, dtype=torch.complex128, device="cuda")
    return dict(tg=tg, ss=cs, sys=sysm, ham=ham, params=params, trial=trial, trial_ops=trial_ops,
                meas_ops=meas_ops, meas_ctx=meas_ctx, prop_ops=prop_ops, prop_ctx=prop_ctx, state=state, e=e,
                W=W, N=N, na=n, nb=n, G=G, qr_every=cfg["qr_every"], kind="cisd")


def run_steps(wl, nsteps, k0=0, fields_host=None, pinned_e=None):
    """nsteps walker-steps (prop + E_L each step) plus the block tail every
    qr_every steps.  With fields_host/pinned_e the fields come from pinned host
    memory and each step's energies are copied back (end-to-end mode)."""
    import torch

    tg = wl["tg"]
    st = wl["state"]
    for k in range(k0, k0 + nsteps):
        fields = None
        if fields_host is not None:
            fields = fields_host[k % fields_host.shape[0]].to("cuda", non_blocking=True)
        st = wl["prop_ops"].step(st, params=wl["params"], ham_data=wl["ham"], trial_data=wl["trial"],
                                 trial_ops=wl["trial_ops"], meas_ops=wl["meas_ops"], meas_ctx=wl["meas_ctx"],
                                 prop_ctx=wl["prop_ctx"], fields=fields, energy_out=wl["e"])
        if pinned_e is not None:
            pinned_e.copy_(wl["e"], non_blocking=True)
        if (k + 1) % wl["qr_every"] == 0:
            st = block_tail(wl, st)
    wl["state"] = st


def block_tail(wl, st):
    """QR, overlaps, block energy + EMA, SR (trot/prop/blocks.py:230-281)."""
    import torch

    tg = wl["tg"]
    from trot_gb300 import _lib, native, rng

    walkers = tg.walkers.orthonormalize_(st.walkers, wl["sys"].walker_kind)
    e = wl["meas_ops"].kernels["energy"](walkers, wl["ham"], wl["meas_ctx"], wl["trial"])
    obs = wl.setdefault("obs", torch.empty(2, dtype=torch.float64, device="cuda"))
    _lib.call("trot_block_energy", wl["W"], e.data_ptr(), st.weights.data_ptr(), st.scalars.data_ptr(),
              float(wl["params"].dt), float(wl["params"].shift_ema), obs.data_ptr(), native.stream_ptr())
    zeta = rng.uniform(st.rng_key, 1)
    w_sr, weights_sr = tg.walkers.stochastic_reconfiguration(walkers, st.weights, zeta, wl["sys"].walker_kind)
    ov_sr = wl["meas_ops"].overlap(w_sr, wl["trial"])
    return st._replace(walkers=w_sr, weights=weights_sr, overlaps=ov_sr)


def perturbed_trial_walkers(wl, noise, seed=21):
    """W walkers = trial orbitals + complex Gaussian noise (the parity tests' recipe)."""
    import torch

    from trot_gb300 import synthetic

    W, N = wl["W"], wl["N"]
    if wl["kind"] == "cisd":
        return torch.as_tensor(synthetic.perturbed_walkers(np.eye(N)[:, :wl["na"]], W, noise, seed)).cuda()
    wa = torch.as_tensor(synthetic.perturbed_walkers(wl["ss"].mo_a, W, noise, seed)).cuda()
    if wl["kind"] == "rhf_r":
        return wa
    return wa, torch.as_tensor(synthetic.perturbed_walkers(wl["ss"].mo_b, W, noise, seed + 1)).cuda()


def fp64_self_noise(wl, m64, mc64, walkers, d, e64, emx, k=4, seed=3):
    """For the k walkers with the largest mixed-vs-FP64 difference: a second FP64
    evaluation of E_L on w U (U a random unitary per spin and walker; E_L is
    invariant under w -> w A for any invertible A), whose difference from the
    first estimates FP64's own rounding noise on that walker, plus its weight."""
    import torch

    idx = torch.argsort(d, descending=True)[:k]
    g = torch.Generator().manual_seed(seed)

    def rot(w):
        n = w.shape[2]
        z = torch.randn((len(idx), n, n), generator=g, dtype=torch.complex128)
        q, _ = torch.linalg.qr(z)
        return torch.matmul(w[idx], q.to(w.device)).contiguous()

    wsub = tuple(rot(w) for w in walkers) if isinstance(walkers, tuple) else rot(walkers)
    e64u = m64.kernels["energy"](wsub, wl["ham"], mc64, wl["trial"])
    wts = wl["state"].weights
    return [{"abs_dE_L_Ha": float(d[i]), "abs_E_L_Ha": float(e64[i].abs()),
             "fp64_self_noise_Ha": float((e64u[j] - e64[i]).abs()), "weight": float(wts[i])}
            for j, i in enumerate(idx.tolist())]


def max_over_ranks(x: float, world: int, device="cuda") -> float:
    """Largest value of ``x`` over the ranks of the process group (the job's
    time is its slowest replica's); ``x`` itself when running alone."""
    if world <= 1:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job throughput: the units all replicas processed over the slowest time."""
    return units_per_rank * world / seconds


def flush_l2(buf):
    buf.add_(1.0)


def cpu_port_rate(cfg, W_sample, steps, threads=None, min_seconds=0.0, max_steps=64):
    """Oracle (numpy complex128) walker-steps/s on a bounded sample of the
    workload: W_sample walkers, at least ``steps`` steps and at least
    ``min_seconds`` of work (capped at ``max_steps``)."""
    from oracle import afqmc_oracle as orc
    from trot_gb300 import synthetic

    N, (na, nb), G = cfg["norb"], cfg["nelec"], cfg["nchol"]
    kind = cfg["kind"]
    if kind == "cisd":
        from oracle import cisd_oracle as co

        ss = synthetic.make_cisd_system(N, na, G, decay=cfg["decay"], seed=0, h0=0.0)
        mo = np.eye(N)[:, :na]
        prop = orc.build_prop_ctx(ss.h0, ss.h1, ss.chol, np.stack([mo @ mo.T] * 2), cfg["dt"])
        m = co.CisdModel(co.CisdTrial(ss.ci1, ss.ci2), ss.h0, ss.h1, ss.chol, prop)
        w = synthetic.perturbed_walkers(mo, W_sample, 0.0)
    elif kind == "uhf_u":
        ss = synthetic.make_system(N, (na, nb), G, decay=cfg["decay"], seed=0, h0=0.0)
        prop = orc.build_prop_ctx(ss.h0, ss.h1, ss.chol, ss.rdm1(), cfg["dt"])
        m = orc.Model(kind, ss.h0, (ss.mo_a, ss.mo_b), orc.build_uhf_meas_ctx(ss.h1, ss.chol, ss.mo_a, ss.mo_b), prop)
        w = (synthetic.perturbed_walkers(ss.mo_a, W_sample, 0.0), synthetic.perturbed_walkers(ss.mo_b, W_sample, 0.0))
    else:
        ss = synthetic.make_system(N, (na, nb), G, decay=cfg["decay"], seed=0, h0=0.0)
        prop = orc.build_prop_ctx(ss.h0, ss.h1, ss.chol, ss.rdm1(), cfg["dt"])
        m = orc.Model(kind, ss.h0, ss.mo_a, orc.build_rhf_meas_ctx(ss.h1, ss.chol, ss.mo_a), prop)
        w = synthetic.perturbed_walkers(ss.mo_a, W_sample, 0.0)
    fields = synthetic.fields(W_sample, G, 2, seed=9)
    params = orc.Params(dt=cfg["dt"])
    st = orc.State(w, np.ones(W_sample), m.overlap(w), 0.0, 0.0, 0)
    m.energy(w)  # warm-up
    st = orc.afqmc_step(st, m, params, fields[0])
    t0 = time.perf_counter()
    k = 0
    while k < steps or (time.perf_counter() - t0 < min_seconds and k < max_steps):
        m.energy(st.walkers)
        st = orc.afqmc_step(st, m, params, fields[k % 2])
        k += 1
    dt = time.perf_counter() - t0
    return W_sample * k / dt, dt, k


def adjoint_leg(chol_scale=0.1, seed=11, n_steps=None):
    """Energy gradient through a whole run on the config-3 shapes (RHF trial, N=80, n=10,
    G=400, W=512, dt=0.01, 200 steps, checkpoints / blocks of 20 steps): one forward run,
    one forward + adjoint run, and central finite differences of the forward along a
    symmetric one-body perturbation O ~ N(0, 0.1) (lambda = +-1e-4, same fields).  The
    Cholesky vectors of the recipe are scaled by ``chol_scale``: unscaled, every walker
    weight of this recipe hits the floor / cap within two steps and the mixed energy is
    undefined (0 / 0); the work per step does not depend on the values."""
    import torch

    import trot_gb300 as tg
    from trot_gb300 import adjoint, synthetic

    cfg = synthetic.CONFIGS["cfg3_rhf_n80"]
    N, (n, _), G, W, T, spb, dt = (cfg["norb"], cfg["nelec"], cfg["nchol"], cfg["n_walkers"], cfg["n_steps"],
                                   cfg["qr_every"], cfg["dt"])
    if n_steps:
        T = int(n_steps)
    h0, h1, chol = synthetic.hamiltonian(N, G, cfg["decay"], seed, 0.0)
    chol = chol * chol_scale
    mo = synthetic.scf(h1, chol, n, n, 30)[0]
    fields = torch.as_tensor(np.random.default_rng(seed + 1).standard_normal((T, W, G))).cuda()
    params = tg.QmcParams(dt=dt, n_exp_terms=6, n_prop_steps=spb, n_walkers=W)
    trial = tg.RhfTrial(mo)
    one = adjoint.as_problem(h0, chol, trial, params, fields[:, :1].contiguous(), steps_per_block=spb)
    e0 = float(adjoint.LocalEnergy.apply(one.walkers0, torch.empty(0, dtype=torch.complex128, device="cuda"),
                                         torch.as_tensor(h1).cuda(), one)[0])
    prob = adjoint.as_problem(h0, chol, trial, params, fields, e_estimate0=e0, steps_per_block=spb)
    adjoint.energy(h1, prob)  # warm-up (first launches, workspaces)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J = adjoint.energy(h1, prob)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    _, g = adjoint.energy_and_grad(h1, prob)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    O = np.random.default_rng(9).normal(scale=0.1, size=h1.shape)
    O = 0.5 * (O + O.T)
    eps = 1e-4
    fd = (adjoint.energy(h1 + eps * O, prob) - adjoint.energy(h1 - eps * O, prob)) / (2 * eps)
    ad = float(torch.sum(g.cpu() * torch.as_tensor(O)))
    return {"workload": f"rhf_r N={N} n={n} G={G} W={W} dt={dt} {T} steps, blocks/checkpoints of {spb}, "
                        f"Cholesky x{chol_scale}, SR off, FP64",
            "objective": "sum_b sum_w wt E~ / sum_b sum_w wt (block energies after QR, clamp, e_estimate EMA)",
            "mixed_energy": J, "forward_s": t1 - t0, "forward_and_adjoint_s": t2 - t1,
            "dJ_dlambda_adjoint": ad, "dJ_dlambda_fd": fd, "rel_diff_vs_fd": abs(ad - fd) / max(abs(fd), 1e-300),
            "fd_lambda": eps}


def _block_energy_host(e, weights, e_ref, dt):
    """Block energy of trot/prop/blocks.py:236-251 on host arrays: non-finite or
    outlying (|E - e_ref| > sqrt(2/dt)) energies replaced by e_ref, non-finite
    walkers' weights zeroed, weighted mean (e_ref when the weights sum to 0)."""
    e = np.real(e)
    with np.errstate(invalid="ignore"):
        bad = ~np.isfinite(e)
        e = np.where(bad | (np.abs(e - e_ref) > np.sqrt(2.0 / dt)), e_ref, e)
    w = np.where(bad, 0.0, weights)
    ws = float(np.sum(w))
    return e_ref if ws == 0 else float(np.sum(w * e) / ws)


def precision_leg(chol_scale=0.1, n_steps=200, seed=5):
    """Mixed vs FP64 along whole trajectories on the headline workload's shapes
    (UHF N=120 (12,10) G=600 W=1024 dt=0.005, QR + block tail every 10 steps):
    the mixed run, and an FP64 run, from the same initial walkers with identical
    fields (seeded on the device per step), identical SR zeta per block and the mixed
    run's SR selections.
    Reports per-walker |dE_L| between the mixed and the FP64 local energy of the
    mixed run's walkers at every step (identical walkers), the block energies of
    the mixed run computed from mixed and from FP64 local energies of the same
    walkers and weights (clamp of trot/prop/blocks.py:236-251), and the block
    energies of the independent FP64 run.  The Cholesky vectors of the recipe are
    scaled by ``chol_scale``: unscaled, every walker weight hits the floor / cap
    within a few steps (block energies would be the clamp value); at x0.1 the
    population stays alive for the whole run."""
    import torch

    import trot_gb300 as tg
    from trot_gb300 import _lib, native, synthetic

    cfg = synthetic.CONFIGS["cfg2_uhf_n120"]
    N, (na, nb), G, W, dt, qr = (cfg["norb"], cfg["nelec"], cfg["nchol"], cfg["n_walkers"], cfg["dt"],
                                 cfg["qr_every"])
    h0, h1, chol = synthetic.hamiltonian(N, G, cfg["decay"], 0, 0.0)
    chol = chol * chol_scale
    ca, cb = synthetic.scf(h1, chol, na, nb, 30)
    sysm = tg.System(norb=N, nelec=(na, nb), walker_kind="unrestricted")
    ham = tg.HamChol(h0=h0, h1=h1, chol=chol)
    trial = tg.UhfTrial(ca, cb)
    params = tg.QmcParams(dt=dt, n_walkers=W, n_prop_steps=qr, seed=1234)
    trial_ops = tg.make_uhf_trial_ops(sysm)

    def setup(mixed):
        meas = tg.make_uhf_meas_ops(sysm, mixed_precision=mixed)
        mctx = meas.build_meas_ctx(ham, trial)
        pops = tg.make_prop_ops("restricted", "unrestricted", mixed_precision=mixed)
        pctx = pops.build_prop_ctx(ham, trial_ops.get_rdm1(trial), params)
        st = pops.init_prop_state(sys=sysm, ham_data=ham, trial_ops=trial_ops, trial_data=trial, meas_ops=meas,
                                  params=params)
        return dict(meas=meas, mctx=mctx, pops=pops, pctx=pctx, st=st)

    runs = {"mixed": setup(True), "fp64": setup(False), "fp64u": setup(False)}
    # control: an FP64 run from w U (a random unitary U per walker and spin), mathematically the
    # same trajectory (G, E_L, force bias, overlap ratios and weights are invariant under w -> w U)
    # with different rounding: its block energies against the plain FP64 run measure how far FP64
    # trajectories themselves drift apart
    gu = torch.Generator().manual_seed(seed + 17)

    def _unitary(w):
        z = torch.randn((w.shape[0], w.shape[2], w.shape[2]), generator=gu, dtype=torch.complex128)
        return torch.matmul(w, torch.linalg.qr(z)[0].to(w.device)).contiguous()

    st_u = runs["fp64u"]["st"]
    wu_rot = tuple(_unitary(w) for w in st_u.walkers)
    runs["fp64u"]["st"] = st_u._replace(walkers=wu_rot, overlaps=runs["fp64u"]["meas"].overlap(wu_rot, trial))
    obs = torch.empty(2, dtype=torch.float64, device="cuda")
    gen = torch.Generator(device="cuda")
    zetas = np.random.default_rng(seed).uniform(size=n_steps // qr)
    e_mx = torch.empty(W, dtype=torch.complex128, device="cuda")
    d_steps, e_abs = [], []
    blk = {"mixed_from_mixed_E": [], "mixed_from_fp64_E": [], "fp64_run": [], "fp64u_run": []}
    t0 = time.perf_counter()
    for b in range(n_steps // qr):
        for k in range(qr):
            gen.manual_seed(seed * 1000003 + b * qr + k)
            x = torch.randn((W, G), generator=gen, dtype=torch.float64, device="cuda")
            r = runs["mixed"]
            e64 = runs["fp64"]["meas"].kernels["energy"](r["st"].walkers, ham, runs["fp64"]["mctx"], trial)
            r["st"] = r["pops"].step(r["st"], params=params, ham_data=ham, trial_data=trial, trial_ops=trial_ops,
                                     meas_ops=r["meas"], meas_ctx=r["mctx"], prop_ctx=r["pctx"], fields=x,
                                     energy_out=e_mx)
            d_steps.append((e_mx - e64).abs().cpu().numpy())
            e_abs.append(e64.abs().cpu().numpy())
            for name in ("fp64", "fp64u"):
                f = runs[name]
                f["st"] = f["pops"].step(f["st"], params=params, ham_data=ham, trial_data=trial, trial_ops=trial_ops,
                                         meas_ops=f["meas"], meas_ctx=f["mctx"], prop_ctx=f["pctx"], fields=x)
        for name, r in runs.items():
            st = r["st"]
            walkers = tg.walkers.orthonormalize_(st.walkers, "unrestricted")
            e = r["meas"].kernels["energy"](walkers, ham, r["mctx"], trial)
            e_ref = float(st.e_estimate)
            wts = st.weights.cpu().numpy()
            if name == "mixed":
                e_other = runs["fp64"]["meas"].kernels["energy"](walkers, ham, runs["fp64"]["mctx"], trial)
                blk["mixed_from_mixed_E"].append(_block_energy_host(e.cpu().numpy(), wts, e_ref, dt))
                blk["mixed_from_fp64_E"].append(_block_energy_host(e_other.cpu().numpy(), wts, e_ref, dt))
            _lib.call("trot_block_energy", W, e.data_ptr(), st.weights.data_ptr(), st.scalars.data_ptr(), float(dt),
                      float(params.shift_ema), obs.data_ptr(), native.stream_ptr())
            if name in ("fp64", "fp64u"):
                blk[name + "_run"].append(float(obs[0]))
            if name == "mixed":
                w_sr, wts_sr = tg.walkers.stochastic_reconfiguration(walkers, st.weights, float(zetas[b]),
                                                                     "unrestricted")
                mixed_weights = st.weights.clone()
            else:
                # the FP64 run resamples with the mixed run's selections (same comb over the mixed
                # weights), so both trajectories keep the same walker lineage; its weights are reset
                # to the mean of its own weights
                w_sr, _ = tg.walkers.stochastic_reconfiguration(walkers, mixed_weights, float(zetas[b]),
                                                                "unrestricted")
                wts_sr = torch.full_like(st.weights, float(st.weights.abs().mean()))
            r["st"] = st._replace(walkers=w_sr, weights=wts_sr, overlaps=r["meas"].overlap(w_sr, trial))
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    d = np.concatenate(d_steps)
    ea = np.concatenate(e_abs)
    bm, bf, b64, b64u = (np.array(blk[k]) for k in ("mixed_from_mixed_E", "mixed_from_fp64_E", "fp64_run",
                                                    "fp64u_run"))
    wm = runs["mixed"]["st"].walkers[0].cpu().numpy()
    wf = runs["fp64"]["st"].walkers[0].cpu().numpy()
    return {
        "workload": f"uhf_u N={N} nelec=({na},{nb}) G={G} W={W} dt={dt}, {n_steps} steps, QR + block tail every "
                    f"{qr}, Cholesky x{chol_scale}, identical device-seeded fields, SR zeta and SR selections in "
                    f"both runs",
        "per_walker_identical_walkers": {"max_abs_dE_L_Ha": float(np.nanmax(d)),
                                         "p99_abs_dE_L_Ha": float(np.nanquantile(d, 0.99)),
                                         "median_abs_dE_L_Ha": float(np.nanmedian(d)),
                                         "max_abs_E_L_Ha": float(np.nanmax(ea)), "samples": int(d.size),
                                         "on": "every step, the mixed run's incoming walkers: mixed E_L (from the "
                                               "step) vs the FP64 E_L kernel"},
        "block_energy_diff_mHa": 1e3 * abs(float(np.mean(bm)) - float(np.mean(bf))),
        "max_block_energy_diff_mHa": 1e3 * float(np.max(np.abs(bm - bf))),
        "block_energy_note": "block energies of the mixed run from mixed vs FP64 local energies of the same "
                             "walkers and weights, averaged over the blocks",
        "block_average_mixed_Ha": float(np.mean(bm)),
        "fp64_run_block_average_Ha": float(np.mean(b64)),
        "fp64_run_block_energy_diff_mHa": 1e3 * abs(float(np.mean(bm)) - float(np.mean(b64))),
        "fp64_run_block_energy_diff_stderr_mHa": 1e3 * float(np.std(bm - b64, ddof=1) / np.sqrt(len(bm))),
        "fp64_run_block_energy_diffs_mHa": [round(1e3 * float(x), 6) for x in (bm - b64)],
        "fp64_run_max_block_energy_diff_mHa": 1e3 * float(np.max(np.abs(bm - b64))),
        "fp64_run_note": "block energies of an independent FP64 run (same fields, zeta and SR selections) "
                         "against the mixed run's, averaged over the blocks",
        "fp64_control_block_energy_diff_mHa": 1e3 * abs(float(np.mean(b64u)) - float(np.mean(b64))),
        "fp64_control_block_energy_diff_stderr_mHa": 1e3 * float(np.std(b64u - b64, ddof=1) / np.sqrt(len(b64))),
        "fp64_control_block_energy_diffs_mHa": [round(1e3 * float(x), 6) for x in (b64u - b64)],
        "fp64_control_note": "the same comparison between two FP64 runs of the same trajectory (the second from "
                             "w U, U a random unitary per walker and spin: identical in exact arithmetic): the "
                             "trajectory-noise floor of FP64 itself",
        "fp64_run_final_walker_rel_diff": float(np.max(np.abs(wm - wf)) / max(np.max(np.abs(wf)), 1e-300)),
        "alive_walkers_end": int((runs["mixed"]["st"].weights > 0).sum().item()),
        "seconds": secs,
    }


def fragments_leg(n_steps=10, warmup=3, n_walkers=128, n_fragments=24):
    """The batched uneven-fragment workload (24 LNO-style RHF fragments, N ~ U[30, 160],
    nocc = round(0.12 N), G = 4 N, 128 walkers each): one phaseless step + local energy
    of every fragment per step, each fragment on its own stream, the whole batch captured
    as one CUDA graph and replayed; the tensor-core path for fragments with N <= 128 and
    nocc <= 16 (the mixed batch), the FP64 kernels for all of them (the FP64 batch).
    Per-walker |dE_L| mixed vs FP64 on identical walkers near the trial, per mixed fragment."""
    import torch

    from trot_gb300 import fragments as fr
    from trot_gb300 import synthetic
    from trot_gb300.meas import make_rhf_meas_ops

    sizes = fr.lno_fragment_sizes(n_fragments)
    out = {"workload": f"{n_fragments} RHF fragments, N ~ U[30, 160] (seeded draw), nocc = round(0.12 N), "
                       f"G = 4 N, W = {n_walkers} each, dt = 0.005, one graph replay per step",
           "sizes_N": [int(sz[0]) for sz in sizes]}
    for mixed in (True, False):
        t0 = time.perf_counter()
        batch = fr.FragmentBatch([fr.make_fragment(N, n, G, n_walkers, seed=k, mixed=mixed)
                                  for k, (N, n, G) in enumerate(sizes)])
        t_build = time.perf_counter() - t0
        for _ in range(warmup):
            batch.step()
        batch.capture()
        batch.step()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(n_steps):
            batch.step()
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        leg = {"value": batch.walker_steps_per_step * n_steps / (ms / 1e3), "unit": "walker-steps/s",
               "ms_per_step": ms / n_steps, "steps": n_steps, "setup_s": t_build,
               "tensor_core_fragments": int(sum(f.mixed for f in batch.fragments))}
        if mixed:
            worst = 0.0
            for f in batch.fragments:
                if not f.mixed:
                    continue
                m64 = make_rhf_meas_ops(f.sys)
                mc64 = m64.build_meas_ctx(f.ham, f.trial)
                w = torch.as_tensor(synthetic.perturbed_walkers(f.trial.mo_coeff.cpu().numpy(), 16, 0.1, 3)).cuda()
                e64 = m64.kernels["energy"](w, f.ham, mc64, f.trial)
                emx = f.meas_ops.kernels["energy"](w, f.ham, f.meas_ctx, f.trial)
                worst = max(worst, float((emx - e64).abs().max()))
            leg["precision_check"] = {"max_abs_dE_L_Ha": worst,
                                      "on": "16 walkers near the trial (noise 0.1) per tensor-core fragment"}
        out["mixed" if mixed else "fp64"] = leg
        del batch
        torch.cuda.empty_cache()
    out["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def staged_load_leg(norb=256, nchol=2000, reps=3):
    """Staged-input cache -> HBM: a (nchol, norb, norb) float64 Cholesky tensor (1.05 GB at the
    defaults) written with staging.dump, then read back with staging.load(device=cuda)
    (positioned reads into two pinned buffers, copies to HBM on a side stream) and, for
    comparison, with a host load followed by one pageable host->device copy. The file sits
    in the page cache after the write, so this measures the host side of the loader, not
    the disk."""
    import tempfile

    import torch

    from trot_gb300 import staging

    rng = np.random.default_rng(4)
    chol = rng.standard_normal((nchol, norb, norb))
    h1 = rng.standard_normal((norb, norb))
    mo = np.linalg.qr(rng.standard_normal((norb, norb)))[0]
    ham = staging.HamInput(h0=0.0, h1=h1, chol=chol, nelec=(8, 8), norb=norb, chol_cut=1e-5, frozen=0,
                           source_kind="mf", basis="restricted")
    st = staging.StagedInputs(ham=ham, trial=staging.TrialInput(kind="rhf", data={"mo": mo}, frozen=0,
                                                                source_kind="mf"),
                              meta={"format_version": 1})
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "staged.h5")
        t0 = time.perf_counter()
        staging.dump(st, path)
        t_dump = time.perf_counter() - t0
        dev_s, host_s = [], []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            d = staging.load(path, device="cuda")
            torch.cuda.synchronize()
            dev_s.append(time.perf_counter() - t0)
            ok = bool(torch.equal(d.ham.chol[-1].cpu(), torch.from_numpy(chol[-1])))
            del d
            t0 = time.perf_counter()
            h = staging.load(path)
            c = torch.from_numpy(h.ham.chol).cuda()
            torch.cuda.synchronize()
            host_s.append(time.perf_counter() - t0)
            del h, c
    nbytes = chol.nbytes
    return {"workload": f"staged-input cache, chol ({nchol}, {norb}, {norb}) f64 = {nbytes / 1e9:.2f} GB "
                        "(file in the page cache)",
            "dump_s": t_dump, "device_load_s": float(np.median(dev_s)),
            "device_load_GBps": nbytes / float(np.median(dev_s)) / 1e9,
            "host_load_then_copy_s": float(np.median(host_s)),
            "host_load_then_copy_GBps": nbytes / float(np.median(host_s)) / 1e9,
            "device_copy_matches_file": ok}


def cisd_leg(steps=10, warmup=3, fp64_steps=2):
    """Config 4 (CISD trial, N=60, 8+8 electrons, G=300, W=256) beside the headline: mixed
    (the reference's default CISD dtypes, tensor-core propagation) and FP64 walker-steps/s
    with E_L each step, timed with CUDA events like the headline, and the mixed-vs-FP64
    E_L difference on walkers near the trial. Errors are recorded, not raised."""
    import torch

    from trot_gb300.synthetic import CONFIGS

    cfg = CONFIGS["cfg4_cisd_n60"]
    W = cfg["n_walkers"]
    out = {"workload": f"cisd N={cfg['norb']} nocc={cfg['nelec'][0]} G={cfg['nchol']} W={W} dt={cfg['dt']} "
                       f"qr/sr every {cfg['qr_every']}, prop + E_L each step"}
    try:
        for prec, n in (("mixed", steps), ("fp64", fp64_steps)):
            wl = build_workload(cfg, prec)
            run_steps(wl, warmup)
            torch.cuda.synchronize()
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record()
            run_steps(wl, n, k0=warmup)
            a1.record()
            torch.cuda.synchronize()
            ms = a0.elapsed_time(a1)
            out[prec] = {"value": W * n / (ms / 1e3), "unit": UNIT, "steps": n, "ms_per_step": ms / n}
            if prec == "mixed":
                import trot_gb300 as tg

                m64 = tg.make_cisd_meas_ops(wl["sys"], mixed_precision=False, testing=True)
                mc64 = m64.build_meas_ctx(wl["ham"], wl["trial"])
                near = {}
                for noise in (0.05, 0.3):
                    wn = perturbed_trial_walkers(wl, noise)
                    a64 = m64.kernels["energy"](wn, wl["ham"], mc64, wl["trial"])
                    amx = wl["meas_ops"].kernels["energy"](wn, wl["ham"], wl["meas_ctx"], wl["trial"])
                    dd = (amx - a64).abs()
                    near[f"noise_{noise}"] = {"max_abs_dE_L_Ha": float(dd.max()),
                                              "max_abs_E_L_Ha": float(a64.abs().max())}
                out["precision_near_trial"] = near
            del wl
        out["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    except Exception as exc:  # the headline line must still print
        out["error"] = f"{type(exc).__name__}: {exc}"
    return out


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--fp64-steps", type=int, default=3, help="steps of the FP64 path timed for the comparison")
    ap.add_argument("--config", default="cfg2_uhf_n120")
    ap.add_argument("--cpu-sample", type=int, default=0, help="walkers in the CPU baseline sample (0 = auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the config-3 energy-gradient leg")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the config-3 energy-gradient leg and print its JSON (for profiling)")
    ap.add_argument("--adjoint-steps", type=int, default=0,
                    help="steps of the energy-gradient leg (default: the config's 200)")
    ap.add_argument("--no-precision-leg", action="store_true",
                    help="skip the 200-step mixed-vs-FP64 trajectory comparison")
    ap.add_argument("--precision-only", action="store_true",
                    help="run only the mixed-vs-FP64 trajectory comparison and print its JSON")
    ap.add_argument("--no-fragments", action="store_true", help="skip the 24-fragment batch leg")
    ap.add_argument("--no-staged", action="store_true", help="skip the staged-input cache -> HBM leg")
    ap.add_argument("--no-cisd", action="store_true", help="skip the CISD (config 4) leg")
    ap.add_argument("--staged-only", action="store_true", help="run only the staged-input cache -> HBM leg")
    ap.add_argument("--fragments-only", action="store_true",
                    help="run only the 24-fragment batch leg and print its JSON")
    ap.add_argument("--profile-run", action="store_true",
                    help="timed steps only (no e2e, FP64 comparison, precision check or CPU baseline): "
                         "for profiler launch lists")
    args = ap.parse_args()

    from trot_gb300 import synthetic

    cfg = dict(synthetic.CONFIGS[args.config])
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    N, (na, nb), G, W = cfg["norb"], cfg["nelec"], cfg["nchol"], cfg["n_walkers"]
    fl = flops_per_walker_step_cisd(N, na, G) if cfg["kind"] == "cisd" else flops_per_walker_step(N, na, nb, G)
    nspin = 1 if cfg["kind"] in ("rhf_r", "cisd") else 2
    config = {"workload": f"{cfg['kind']} N={N} nelec=({na},{nb}) G={G} W={W} dt={cfg['dt']} "
                          f"qr/sr every {cfg['qr_every']}", "walkers": W, "norb": N, "nelec": [na, nb],
              "nchol": G, "trial": cfg["kind"], "seed": 0}

    if args.impl == "reference":
        if rank != 0:
            return
        cores = cpu_cores()
        sample = args.cpu_sample or 64
        rates, secs, ks = [], 0.0, 0
        for _ in range(max(1, min(3, args.steps // 10))):
            r, sec, k = cpu_port_rate(cfg, sample, 2, min_seconds=10.0)
            rates.append(r)
            secs += sec
            ks += k
        v = statistics.median(rates)
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": True, "dtype": "c128", "data": "synthetic",
                "config": config, "vs_baseline": None,
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": f"{sample} walkers x {ks} steps total (prop + E_L) in {len(rates)} "
                                           f"timed runs of >= 10 s, numpy complex128 oracle port, median; "
                                           f"{secs:.1f} s of CPU work"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch

    if world > 1:
        import torch.distributed as dist

        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from trot_gb300 import _lib

    if args.adjoint_only:
        if rank == 0:
            print(json.dumps({"adjoint": adjoint_leg(n_steps=args.adjoint_steps)}), flush=True)
        return
    if args.fragments_only:
        if rank == 0:
            print(json.dumps({"fragments": fragments_leg()}), flush=True)
        return
    if args.staged_only:
        if rank == 0:
            print(json.dumps({"staged_load": staged_load_leg()}), flush=True)
        return
    if args.precision_only:
        if rank == 0:
            print(json.dumps({"precision_trajectory": precision_leg()}), flush=True)
        return
    wl = build_workload(cfg, args.precision)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    # warm-up: W steps, then one untimed block tail (QR, energy, SR) so the
    # tail's one-time work (first launches, workspace growth) is outside the timed region
    run_steps(wl, args.warmup)
    wl["state"] = block_tail(wl, wl["state"])
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # timed region: K steps, device-timed with CUDA events on torch's stream
    _lib.profile_enable(64 * (args.steps + 8))
    flush_l2(flush)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        run_steps(wl, args.steps, k0=args.warmup)
        ev1.record()
        torch.cuda.synchronize()
        barrier()
    ms = ev0.elapsed_time(ev1)
    prof = _lib.profile_collect()
    n_launches = _lib.profile_launch_count()
    _lib.profile_enable(0)
    ms = max_over_ranks(ms, world)
    value = job_rate(W * args.steps, world, ms / 1e3)

    if args.profile_run:
        if rank == 0:
            print(json.dumps({"profile_run": True, "ms_per_step": ms / args.steps,
                              "kernels": {k: v for k, v in prof.items()}}), flush=True)
        return
    # end to end through the public API: host fields in, energies out, every step
    k_e2e = max(4, args.steps // 2)
    fields_host = torch.from_numpy(synthetic.fields(W, G, 4, seed=77)).pin_memory()
    pinned_e = torch.empty(W, dtype=torch.complex128).pin_memory()
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run_steps(wl, k_e2e, k0=args.warmup + args.steps, fields_host=fields_host, pinned_e=pinned_e)
    torch.cuda.synchronize()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world)
    e2e = {"value": job_rate(W * k_e2e, world, e2e_s), "unit": UNIT, "h2d_bytes_per_step": W * G * 8,
           "d2h_bytes_per_step": W * 16, "steps": k_e2e}
    # precision: mixed vs FP64 local energy on the run's own (identical) walkers
    precision_info = None
    fp64 = None
    if args.precision == "mixed":
        import trot_gb300 as tg

        st = wl["state"]
        mc64 = wl["meas_ctx"]
        if wl["kind"] == "uhf_u":
            m64 = tg.make_uhf_meas_ops(wl["sys"])
        elif wl["kind"] == "cisd":
            m64 = tg.make_cisd_meas_ops(wl["sys"], mixed_precision=False, testing=True)
            mc64 = m64.build_meas_ctx(wl["ham"], wl["trial"])
        else:
            m64 = tg.make_rhf_meas_ops(wl["sys"])
        e64 = m64.kernels["energy"](st.walkers, wl["ham"], mc64, wl["trial"])
        emx = wl["meas_ops"].kernels["energy"](st.walkers, wl["ham"], wl["meas_ctx"], wl["trial"])
        d = (emx - e64).abs()
        live = st.weights > 0
        precision_info = {
            "max_abs_dE_L_Ha": float(d.max()),
            "on": "every walker of the benchmark after warm-up + timed + e2e steps, mixed vs FP64 E_L kernel on "
                  "identical walkers (replaced by the 200-step trajectory leg below when it runs)",
            "bench_walkers": {"max_abs_dE_L_Ha": float(d.max()), "median_abs_dE_L_Ha": float(d.median()),
                              "max_abs_E_L_Ha": float(e64.abs().max()), "walkers": W,
                              "live_walkers": int(live.sum()), "above_1e-5": int((d > 1e-5).sum()),
                              "note": "the recipe's walkers decay within a few steps (weights at 0, |E_L| up to "
                                      "~1e7 Ha, where FP64's own rounding noise reaches 1e-4 Ha; see 'worst')"},
        }
        if wl["kind"] != "cisd":
            precision_info["bench_walkers"]["worst"] = fp64_self_noise(wl, m64, mc64, st.walkers, d, e64, emx)
        # the seeded recipe's population decays within a few steps (|E_L| up to ~1e6 Ha), so the
        # same comparison is also made on walkers near the trial, where E_L is physical
        near = {}
        for noise in (0.05, 0.3):
            wn = perturbed_trial_walkers(wl, noise)
            a64 = m64.kernels["energy"](wn, wl["ham"], mc64, wl["trial"])
            amx = wl["meas_ops"].kernels["energy"](wn, wl["ham"], wl["meas_ctx"], wl["trial"])
            dd = (amx - a64).abs()
            near[f"noise_{noise}"] = {"max_abs_dE_L_Ha": float(dd.max()), "median_abs_dE_L_Ha": float(dd.median()),
                                      "max_abs_E_L_Ha": float(a64.abs().max())}
        precision_info["near_trial_walkers"] = near
        # FP64 path on the same workload, same device, a few steps
        wl64 = build_workload(cfg, "fp64")
        run_steps(wl64, 1)
        torch.cuda.synchronize()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record()
        run_steps(wl64, args.fp64_steps, k0=1)
        a1.record()
        torch.cuda.synchronize()
        ms64 = a0.elapsed_time(a1)
        fp64 = {"value": W * args.fp64_steps / (ms64 / 1e3), "unit": UNIT, "steps": args.fp64_steps,
                "ms_per_step": ms64 / args.fp64_steps}
        del wl64
    if rank != 0:
        return

    peaks, peak_src = load_peaks()
    launches = n_launches  # every kernel of the library launched in the timed region (timed or not)
    # roofline of the dominant kernel
    top = max(prof.items(), key=lambda kv: kv[1][0]) if prof else ("none", (0.0, 1))
    tname, (tms, tcnt) = top
    # algorithmic flops per walker of one launch: the exchange kernel runs once per spin
    if cfg["kind"] == "cisd":
        v_ = N - na
        fl_map = {"cisd_gamma": fl["gl"] + fl["lci2_green"] + fl["glgp"] + fl["lg1"],
                  "cisd_l2ci2": 4 * G * (na * v_) ** 2,  # one quadratic form with the combined ci2m
                  "cisd_chol_gemm": 4 * G * na * N, "cisd_ci2g": 4 * (na * v_) ** 2, "vhs": fl["vhs"],
                  "trotter": fl["taylor"] + fl["onebody"]}
    else:
        fl_map = {"vhs": fl["vhs"], "exchange_exact": (fl["exchange"] + fl["force_bias"]) / nspin,
                  "exchange": fl["exchange"], "trotter": fl["taylor"] + fl["onebody"] + fl["overlap"],
                  "force_bias": fl["force_bias"], "green": fl["green"]}
    kfl = next((v for k, v in fl_map.items() if tname.startswith(k)), sum(fl.values()))
    per_launch_s = tms / max(tcnt, 1) / 1e3
    achieved_tflops = kfl * W / per_launch_s / 1e12 if per_launch_s > 0 else 0.0
    peak = peaks["bf16_tflops"]
    roofline = {"bound": "tensor", "kernel": tname, "achieved": achieved_tflops, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved_tflops / peak, "peak_source": f"{peak_src} bf16 dense (MEASURED_PEAKS.json)",
                "traffic": NCU_DRAM_BYTES.get((args.config, args.precision, tname)),
                "algorithmic_flops_per_launch": kfl * W,
                "note": "fp64 kernels run on the FP64 pipe; the bf16 tensor peak is the denominator the contract names"}
    if tname == "exchange_exact_tc":
        # the exact-slice kernel executes 15 BF16 products per output tile on top of the
        # algorithmic (FP64-equivalent) contraction: tensor work actually issued per launch
        ex = exchange_tensor_flops(cfg, W)
        roofline["executed_bf16_flops_per_launch"] = ex
        roofline["executed_bf16_tflops"] = ex / per_launch_s / 1e12
        roofline["executed_frac"] = ex / per_launch_s / 1e12 / peak
        roofline["traffic_note"] = ("DRAM bytes per launch (mean of the two spin launches) measured by ncu on this "
                                    "workload: profiles/exchange_exact_tc_uhf_n120_w256.md")
    step_flops = sum(fl.values()) * W
    kernels = {k: {"ms_total": round(v[0], 4), "launches": v[1], "ms_per_launch": round(v[0] / max(v[1], 1), 5)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128" if args.precision == "fp64" else "mixed(bf16/fp32 tc, f64)",
            "precision": args.precision, "data": "synthetic (seeded recipe)",
            "config": dict(config, l2="per-step working set > L2 (129 MB); L2 flushed before the timed region",
                           parallelism="replicas" if world > 1 else "1 GPU"),
            "clocks": clk.summary(), "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
            "step_tflops": step_flops / (ms / args.steps / 1e3) / 1e12, "kernels": kernels}
    if fp64 is not None:
        line["fp64_path"] = fp64
        line["speedup_vs_fp64"] = value / fp64["value"]
    if precision_info is not None:
        line["precision_check"] = precision_info
    if args.precision == "mixed" and not args.no_precision_leg and rank == 0 and world == 1 \
            and args.config == "cfg2_uhf_n120":
        traj = precision_leg()
        line["precision_trajectory"] = traj
        if precision_info is not None:
            # the headline precision statement: a population that stays alive (Cholesky x0.1), every
            # walker at every step, and the block energies of an independent FP64 run
            pw = traj["per_walker_identical_walkers"]
            precision_info["max_abs_dE_L_Ha"] = pw["max_abs_dE_L_Ha"]
            precision_info["block_energy_diff_mHa"] = traj["fp64_run_block_energy_diff_mHa"]
            precision_info["block_energy_diff_stderr_mHa"] = traj["fp64_run_block_energy_diff_stderr_mHa"]
            precision_info["fp64_control_block_energy_diff_mHa"] = traj["fp64_control_block_energy_diff_mHa"]
            precision_info["on"] = ("200-step trajectory on the headline shapes with live walkers (Cholesky x0.1): "
                                    f"{pw['samples']} per-walker samples of mixed vs FP64 E_L on identical walkers; "
                                    "block energies of an independent FP64 run with the same fields, zeta and SR "
                                    "selections (precision_trajectory)")
    if not args.no_adjoint and rank == 0 and world == 1:
        line["adjoint"] = adjoint_leg(n_steps=args.adjoint_steps)
    if not args.no_fragments and rank == 0 and world == 1 and args.config == "cfg2_uhf_n120":
        line["fragments"] = fragments_leg()
    if not args.no_staged and rank == 0 and world == 1 and args.config == "cfg2_uhf_n120":
        line["staged_load"] = staged_load_leg()
    if not args.no_cisd and rank == 0 and world == 1 and args.config == "cfg2_uhf_n120":
        line["cisd"] = cisd_leg()
    if not args.no_cpu_baseline:
        sample = args.cpu_sample or 64
        r, secs, ks = cpu_port_rate(cfg, sample, 2, min_seconds=10.0)
        line["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": cpu_cores(), "kind": "port",
                                "sample": f"{sample} walkers x {ks} steps (prop + E_L) of the same workload, numpy "
                                          f"complex128 oracle port (BLAS on all cores), {secs:.1f} s"}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
