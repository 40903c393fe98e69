"""trot_gb300: GB300-native (sm_103a) phaseless-AFQMC hot path with trot's
prop / meas / trial / walker call signatures.

All compute runs in ``lib/libtrot_gb300.so`` (hand-written CUDA behind the C
ABI of ``include/trot_gb300.h``); importing the package does not touch the GPU.
"""
from . import _lib, h5file, rng, staging, synthetic
from .blocks import BlockObs, block
from .core import (HamChol, MeasOps, PropOps, PropState, QmcParams, QmcParamsBase, QmcParamsFp, System,
                   TrialOps, k_energy, k_force_bias)
from .meas import (RhfMeasCtx, UhfMeasCtx, build_rhf_meas_ctx, build_uhf_meas_ctx, make_rhf_meas_ops,
                   make_uhf_meas_ops)
from .prop import CholAfqmcCtx, afqmc_step, init_prop_state, make_prop_ops, make_trotter_ops
from .trial import RhfTrial, UhfTrial, get_rdm1, make_rhf_trial_ops, make_uhf_trial_ops
from . import walkers
from .cisd import CisdMeasCtx, CisdTrial, make_cisd_meas_ops, make_cisd_trial_ops
from .prop_fp import afqmc_step_fp, make_prop_ops_fp

__all__ = [
    "HamChol", "MeasOps", "PropOps", "PropState", "QmcParams", "QmcParamsBase", "System", "TrialOps",
    "k_energy", "k_force_bias", "RhfMeasCtx", "UhfMeasCtx", "build_rhf_meas_ctx", "build_uhf_meas_ctx",
    "make_rhf_meas_ops", "make_uhf_meas_ops", "CholAfqmcCtx", "afqmc_step", "init_prop_state", "make_prop_ops",
    "make_trotter_ops", "RhfTrial", "UhfTrial", "get_rdm1", "make_rhf_trial_ops", "make_uhf_trial_ops",
    "walkers", "rng", "synthetic", "staging", "h5file", "block", "BlockObs", "CisdTrial", "CisdMeasCtx", "make_cisd_meas_ops",
    "make_cisd_trial_ops", "QmcParamsFp", "afqmc_step_fp", "make_prop_ops_fp",
]
