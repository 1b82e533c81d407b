"""GPU estimators through the reference's public API: prices agree with the
FP64 closed forms and with the reference's own estimates within 3 standard
errors, and the drop-in return layouts match the reference's."""
import math

import numpy as np
import pytest
import torch

import sde_mc_gb300 as sm
from oracle import oracle
from tests.cases import gbm_uniform, indep2d, merton1d, merton2d_corr

pytestmark = pytest.mark.gpu


def test_c1_merton_price(kat, ref_stats):
    solver, payoff, disc = merton1d(100)
    st = sm.mc_simple(1 << 22, solver, payoff, disc, bs=1 << 22, payoff_time='adapted')
    exact = kat["merton_call"][1][1]
    # Euler bias at 100 jump-adapted steps was measured below 1e-4 (rel 4e-4 +- 6e-4)
    assert abs(st.sample_mean - exact) < 3 * st.sample_std + 1e-4
    r = ref_stats["c1_fp32_2p18"]
    assert abs(st.sample_mean - r["mean"]) < 3 * math.hypot(st.sample_std, r["se"])
    assert st.num_trials == 1 << 22 and st.time_elapsed > 0


def test_c1_unbatched_layout(ref_stats):
    solver, payoff, disc = merton1d(100)
    st = sm.mc_simple(4096, solver, payoff, disc, payoff_time='adapted')
    normals, time_paths, left, total, jumps = st.normals
    assert st.paths.shape == (4096, total + 1, 1)
    assert normals.shape == (4096, 100 + solver.max_jumps, 1)
    assert time_paths.shape == (4096, 101 + solver.max_jumps, 1)
    assert left.shape == jumps.shape == (4096, 101 + solver.max_jumps, 1)
    assert torch.all(time_paths[:, total] == 1.0)
    p = st.payoffs.double()
    assert st.sample_mean == pytest.approx(float(p.mean()), rel=1e-12)
    assert st.sample_std == pytest.approx(float(p.std() / 64.0), rel=1e-9)
    # the payoff is the discounted call on the terminal column
    x_t = st.paths[:, -1, 0]
    np.testing.assert_allclose(st.payoffs.cpu().numpy(),
                               (torch.clamp(x_t - 1.0, min=0) * math.exp(-0.02)).cpu().numpy(), rtol=1e-6, atol=1e-7)
    r = ref_stats["c1_fp32_2p16"]
    assert abs(st.sample_mean - r["mean"]) < 3 * math.hypot(st.sample_std, r["se"])


def test_terminal_payoff_time_reads_nominal_column():
    solver, payoff, disc = merton1d(100)
    st = sm.mc_simple(2048, solver, payoff, disc, payoff_time='terminal')
    x = st.paths[:, 100, 0]
    np.testing.assert_allclose(st.payoffs.cpu().numpy(),
                               (torch.clamp(x - 1.0, min=0) * np.float32(math.exp(-0.02))).cpu().numpy(),
                               rtol=1e-6, atol=1e-7)
    # batched K1 with the same paths gives the same mean
    s2 = sm.JumpEulerSolver(solver.sde, 1.0, 100, seed=solver.seed)
    b = sm.mc_simple(2048, s2, payoff, disc, bs=2048, payoff_time='terminal')
    assert b.sample_mean == pytest.approx(st.sample_mean, rel=1e-6)


def test_c2_rainbow_plain(ref_stats):
    solver, payoff, disc = indep2d(256)
    st = sm.mc_simple(1 << 20, solver, payoff, disc, bs=1 << 16, payoff_time='adapted')
    r = ref_stats["c2_plain_2p16"]
    assert abs(st.sample_mean - r["mean"]) < 3 * math.hypot(st.sample_std, r["se"])


def test_c2_mlmc(ref_stats):
    solver, payoff, disc = indep2d(256)
    levels = [4, 8, 16, 32, 64]
    st = sm.mc_multilevel([1 << 18] * 5, levels, solver, payoff, disc)
    r = ref_stats["c2_mlmc_l0_4"]
    assert abs(st.sample_mean - r["mean"]) < 3 * math.hypot(st.sample_std, r["se"])
    from sde_mc_gb300.mlmc import level_estimates
    est = level_estimates([1 << 18] * 5, levels, solver, payoff, disc)
    for (m, v), ref in zip(est[1:], ref_stats["c2_mlmc_level_stats"]):
        se = math.sqrt(v / (1 << 18) + ref["var"] / ref["n"])
        assert abs(m - ref["mean"]) < 3.5 * se
        assert v == pytest.approx(ref["var"], rel=0.3)
    cursor = solver.path_cursor
    trials = sm.get_optimal_trials(1 << 14, levels, 1e-3, solver, payoff, disc)
    assert len(trials) == 5 and all(isinstance(t, int) and t > 0 for t in trials)
    assert trials[0] > trials[-1]
    # as the reference, the call leaves the solver at the coarsest level (sde_mc/mlmc.py:82)
    assert solver.num_steps == levels[0]
    # the allocation of the pilot's own level variances, against the oracle's
    # FP64 restatement of Giles' formula (the reference rounds in float32)
    after = solver.path_cursor
    solver.path_cursor = cursor  # the pilot's own paths again
    pilot = level_estimates([1 << 14] * 5, levels, solver, payoff, disc)
    assert solver.path_cursor == after
    var = [v for _, v in pilot]
    ora = oracle.optimal_trials(var, levels, solver.time_interval, 1e-3)
    assert np.all(np.abs(np.asarray(trials) - ora) <= np.maximum(1, 1e-5 * ora)), (trials, ora)


def test_solver_layouts_match_reference():
    g = sm.Gbm(0.02, 0.2, torch.tensor([1., 2.]), dim=2)
    paths, normals = sm.EulerSolver(g, 3, 10).solve(bs=4, return_normals=True)
    assert paths.shape == (4, 11, 2) and normals.shape == (4, 10, 2)
    assert not torch.isnan(paths).any()
    st = sm.mc_simple(100, sm.EulerSolver(g, 3, 10), sm.EuroCall(1), sm.ConstantShortRate(0.02))
    assert st.paths.shape == (100, 11, 2) and st.sample_std > 0
    m = sm.Merton(0.02, 0.3, 2, -0.05, 0.3, torch.tensor([1.]), dim=1)
    paths, (normals, time_paths, left, total, jumps) = sm.JumpEulerSolver(m, 3, 10).solve(8)
    assert paths.shape == (8, total + 1, 1)
    for t in (normals, time_paths, left, jumps):
        assert not torch.isnan(t).any()
    (pf, pc), _ = sm.JumpEulerSolver(m, 3, 10).multilevel_solve(16, (20, 10))
    # (bs, total_steps_coarse + 1, dim): every coarse step of the batch
    assert pf.shape == pc.shape and pf.shape[0] == 16 and pf.shape[1] >= 11 and pf.shape[2] == 1
    dg = sm.DoubleGbm(0.02, 0.1, 0.2, torch.ones(2), 2)
    p, n = sm.EulerSolver(dg, 1.0, 8).solve(5)
    assert p.shape == (5, 9, 2) and n.shape == (5, 8, 2, 2)


def test_stream_advances_and_reseeds():
    solver, payoff, disc = merton1d(50)
    a = sm.mc_simple(10000, solver, payoff, disc, bs=10000, payoff_time='adapted').sample_mean
    b = sm.mc_simple(10000, solver, payoff, disc, bs=10000, payoff_time='adapted').sample_mean
    assert a != b
    s2 = sm.JumpEulerSolver(solver.sde, 1.0, 50, seed=solver.seed)
    assert sm.mc_simple(10000, s2, payoff, disc, bs=10000, payoff_time='adapted').sample_mean == a


def test_uniform_grid_gbm(ref_stats):
    g = sm.Gbm(0.02, 0.2, torch.tensor([1.]), 1)
    st = sm.mc_simple(1 << 20, sm.EulerSolver(g, 1.0, 50, seed=6), sm.EuroCall(1.0), sm.ConstantShortRate(0.02),
                      bs=1 << 20)
    r = ref_stats["gbm1d_uniform_2p16"]
    assert abs(st.sample_mean - r["mean"]) < 3 * math.hypot(st.sample_std, r["se"])
    assert abs(st.sample_mean - r["oracle"]) < 3 * st.sample_std + 2e-4


def test_run_mc_reaches_tolerance():
    solver, payoff, disc = merton1d(100)

    class P:
        pass
    prob = P()
    prob.solver, prob.payoff, prob.discounter = solver, payoff, disc
    st = sm.run_mc(prob, 1e-3, bs=1e5, init_trials=1e5)
    assert 1.96 * st.sample_std < 1.1e-3


def test_terminal_cv_reduces_variance():
    solver, payoff, disc = merton1d(100)
    plain = sm.mc_simple(1 << 16, solver, payoff, disc, bs=1 << 16, payoff_time='adapted')
    cv = sm.mc_terminal_cv(1 << 16, solver, payoff, disc, bs=1 << 14)
    assert cv.sample_std < plain.sample_std
    assert abs(cv.sample_mean - plain.sample_mean) < 3 * math.hypot(cv.sample_std, plain.sample_std)
