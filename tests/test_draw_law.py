"""The law of the counter-based draws.

The kernels take their normals, jump gaps, marks and asset picks from
Philox4x32-10 streams where the reference calls torch's generator
(``sample_corr_normals``, ``sample_jump_times``, ``sample_one_jump``,
sde_mc/solvers.py:51-56, 143-148; ``Sde.sample_jumps``, sde_mc/sde.py:325-326;
``LevySde.sample_jumps``, sde_mc/levy.py:85-87).  The GPU parity tests show
that a kernel's exported draws are the oracle's transforms of the same Philox
words; these tests show, on the host, that those transforms have the
reference's distributions: standard normals without correlation across
steps, components or paths, exponential gaps at the model's rate, marks
with the model's mark law and asset picks in proportion to the per-asset
rates.  The seeds are fixed, so the statistics are deterministic."""
import numpy as np
import pytest
import torch
from scipy import stats

import sde_mc_gb300 as sm
from tests.cases import basket, indep2d, inst_for, levy2d, merton1d, zdim


def _normals(O, inst, paths, steps):
    return np.stack([O.native_normals(inst, p, steps, zdim(inst)) for p in range(paths)])


@pytest.mark.parametrize("factory,paths,steps", [(lambda: merton1d(64), 3000, 64),
                                                 (lambda: indep2d(64), 1500, 64),
                                                 (lambda: basket(5, 32), 1000, 32),
                                                 (lambda: basket(8, 16), 1000, 16)])
def test_normals_are_independent_standard_normals(factory, paths, steps, oracle_mod):
    z = _normals(oracle_mod, inst_for(factory(), seed=11), paths, steps).astype(np.float64)  # (paths, steps, ZD)
    n = z.size
    assert abs(z.mean()) < 5 / np.sqrt(n)
    assert abs(z.var() - 1.0) < 5 * np.sqrt(2.0 / n)
    assert stats.kstest(z.ravel(), "norm").pvalue > 1e-4
    # fourth moment of a normal: 3
    assert abs((z ** 4).mean() - 3.0) < 5 * np.sqrt(96.0 / n)
    # no correlation between consecutive steps, between components, between neighbouring paths
    tol = 5 / np.sqrt(paths * (steps - 1) * z.shape[2])
    assert abs(np.mean(z[:, 1:, :] * z[:, :-1, :])) < tol
    if z.shape[2] > 1:
        c = np.corrcoef(z.reshape(-1, z.shape[2]).T)
        off = c[~np.eye(z.shape[2], dtype=bool)]
        assert np.abs(off).max() < 5 / np.sqrt(paths * steps)
    assert abs(np.mean(z[1:] * z[:-1])) < 5 / np.sqrt((paths - 1) * steps * z.shape[2])


def test_different_seeds_streams_and_paths_give_different_draws(oracle_mod):
    O = oracle_mod
    a = inst_for(merton1d(16), seed=1)
    b = inst_for(merton1d(16), seed=2)
    za, zb = O.native_normals(a, 0, 16, 1), O.native_normals(b, 0, 16, 1)
    assert not np.array_equal(za, zb)
    assert not np.array_equal(O.native_normals(a, 0, 16, 1), O.native_normals(a, 1, 16, 1))
    a.stream_id = 5
    assert not np.array_equal(za, O.native_normals(a, 0, 16, 1))
    a.stream_id = 0
    # path_offset shifts the path index: path p of offset 0 is path p - off of offset off
    c = inst_for(merton1d(16), seed=1, path_offset=7)
    np.testing.assert_array_equal(O.native_normals(a, 9, 16, 1), O.native_normals(c, 2, 16, 1))


def test_steps_read_the_normal_stream_densely_or_by_whole_blocks(oracle_mod):
    """A path's diffusion normals come four per Philox block, the blocks the
    same for every dimension (the counter is block, path, stream; the key the
    seed).  Steps of 1, 2, 3, 5 or 6 normals read the stream densely (step k
    takes normals k ZD .. k ZD + ZD - 1); steps of 4 or 8 take whole blocks;
    a step of 7 takes the first seven normals of its two blocks.  The
    stream itself is the whole-block sequence at d = 4."""
    O = oracle_mod
    S = 24
    stream = {p: O.native_normals(inst_for(basket(4, 16), seed=11), p, 2 * S, 4).ravel() for p in (0, 5)}
    for d in range(1, 9):
        inst = inst_for(basket(d, 16), seed=11)
        for p in (0, 5):
            z = O.native_normals(inst, p, S, d)
            if d == 7:
                want = stream[p][:8 * S].reshape(S, 8)[:, :7]
            else:
                want = stream[p][:d * S].reshape(S, d)
            np.testing.assert_array_equal(z, want, err_msg="d=%d path %d" % (d, p))


def _jumps(O, inst, paths, n):
    out = [O.native_jumps(inst, p, n) for p in range(paths)]
    jt = np.stack([o[0] for o in out]).astype(np.float64)
    jm = np.stack([o[1] for o in out]).astype(np.float64)
    js = np.stack([o[2] for o in out])
    return jt, jm, js


def test_merton_gaps_and_marks(oracle_mod):
    inst = inst_for(merton1d(16), seed=3)
    jt, jm, _ = _jumps(oracle_mod, inst, 2000, 8)
    gaps = np.diff(np.concatenate([np.zeros((jt.shape[0], 1)), jt], 1), axis=1).ravel()
    rate = float(inst.rate)
    assert rate == pytest.approx(2.0)
    assert stats.kstest(gaps, stats.expon(0, 1 / rate).cdf).pvalue > 1e-4
    assert np.all(np.diff(jt, axis=1) > 0)
    # exp(N(alpha, gamma)) - 1, alpha -0.1, gamma 0.2
    logj = np.log1p(jm.ravel())
    assert stats.kstest(logj, stats.norm(-0.1, 0.2).cdf).pvalue > 1e-4
    # the gaps and the marks of one jump are independent
    assert abs(np.corrcoef(gaps, logj)[0, 1]) < 5 / np.sqrt(gaps.size)


def test_per_asset_jumps_pick_assets_by_rate(oracle_mod):
    case = indep2d(16)
    inst = inst_for(case, seed=4)
    jt, jm, js = _jumps(oracle_mod, inst, 2000, 8)
    # IndependentJumpsMerton with rates (1, 1): total rate 2, each asset half the jumps
    assert float(inst.rate) == pytest.approx(2.0)
    counts = np.bincount(js.ravel(), minlength=2)
    assert stats.chisquare(counts, [js.size / 2] * 2).pvalue > 1e-4
    gaps = np.diff(np.concatenate([np.zeros((jt.shape[0], 1)), jt], 1), axis=1).ravel()
    assert stats.kstest(gaps, stats.expon(0, 0.5).cdf).pvalue > 1e-4
    assert stats.kstest(np.log1p(jm.ravel()), stats.norm(-0.05, 0.15).cdf).pvalue > 1e-4

    # unequal rates: picks in proportion
    m = sm.IndependentJumpsMerton(0.02, torch.tensor([0.2, 0.3, 0.25]), [0.5, 1.0, 2.5], -0.05, 0.15,
                                  torch.ones(3), 3)
    inst3 = inst_for((sm.JumpEulerSolver(m, 1.0, 16), sm.Rainbow(1.0), sm.ConstantShortRate(0.02)), seed=5)
    _, _, js3 = _jumps(oracle_mod, inst3, 2000, 8)
    counts = np.bincount(js3.ravel(), minlength=3)
    assert stats.chisquare(counts, js3.size * np.array([0.5, 1.0, 2.5]) / 4.0).pvalue > 1e-4


def test_levy_marks_follow_the_truncated_jump_measure(oracle_mod):
    solver, _, _ = levy2d(16)
    inst = inst_for((solver, sm.Rainbow(1.0), sm.ConstantShortRate(0.02)), seed=6)
    _, jm, _ = _jumps(oracle_mod, inst, 2000, 8)
    x = jm.ravel()
    ic = solver.sde.levy.icdf
    assert np.all(np.abs(x) >= ic.eps * (1 - 1e-5))
    # CDF of the marks: the inverse of the inverse CDF on a fine float64 grid of y
    y = torch.linspace(1e-7, 1 - 1e-7, 400001, dtype=torch.float64)
    xs = ic(y).numpy()
    order = np.argsort(xs)
    cdf = lambda v: np.interp(v, xs[order], y.numpy()[order])
    assert stats.kstest(x, cdf).pvalue > 1e-4
    # both signs, in the proportion of the measure's mass (c_minus = c_plus: symmetric)
    assert abs(np.mean(x > 0) - 0.5) < 5 * np.sqrt(0.25 / x.size)
