"""The Levy 'indep' path at scale (inverse-CDF marks, the shared small-jump
Brownian motion) and the exact-jumps MLMC preset of the reference's
LevyRainbowMLMC problem (sde_mc/problem.py:93-106): MLMC agrees with the plain
estimator at the finest level, and the GPU agrees with the oracle's own run
of the same model on the host."""
import math

import pytest
import torch

import sde_mc_gb300 as sm
from sde_mc_gb300 import kernels as K
from sde_mc_gb300.lowering import lower

pytestmark = pytest.mark.gpu


def levy_rainbow(steps, exact_jumps, seed=1):
    # LevyRainbow.default_params: c-=1, c+=1, alpha=0.5, mu=2, r=0.02, sigma=0.3, f=0.2, eps=0.001, d=2, T=3
    lev = sm.ExpExampleLevy(1, 1, 0.5, 2, 0.02, 0.3, 0.2, 0.001, 2)
    sde = sm.LevySde(lev, torch.ones(2))
    solver = sm.JumpEulerSolver(sde, 3, steps, exact_jumps=exact_jumps, seed=seed)
    return solver, sm.Rainbow(1.0), sm.ConstantShortRate(0.02)


def test_levy_plain_at_scale_matches_oracle(oracle_mod):
    solver, payoff, disc = levy_rainbow(64, False)
    st = sm.mc_simple(1 << 22, solver, payoff, disc, bs=1 << 22, payoff_time='adapted')
    inst = lower(solver, payoff, disc, num_paths=1 << 15, path_offset=1 << 40)
    out, _, rc = oracle_mod.price(inst)
    assert rc == 0
    se_cpu = math.sqrt(out[4] / out[2])
    assert abs(st.sample_mean - out[3]) < 3 * math.hypot(st.sample_std, se_cpu)
    # the same paths on the GPU and on the host: per-path transforms agree to ~1e-5
    g = K.price(inst).cpu().tolist()
    assert g[3] == pytest.approx(out[3], rel=1e-4)


def test_levy_mlmc_exact_jumps_preset():
    solver, payoff, disc = levy_rainbow(64, True, seed=3)
    levels = [4, 8, 16, 32, 64]
    plain = sm.mc_simple(1 << 21, solver, payoff, disc, bs=1 << 21, payoff_time='adapted')
    eps = 5e-3 * plain.sample_mean
    trials = sm.get_optimal_trials(1 << 13, levels, eps, solver, payoff, disc)
    ml = sm.mc_multilevel(trials, levels, solver, payoff, disc)
    assert abs(ml.sample_mean - plain.sample_mean) < 3 * math.hypot(ml.sample_std, plain.sample_std)
    assert 1.96 * ml.sample_std < 2 * eps
