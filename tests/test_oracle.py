"""The oracle pinned against the reference: known-answer values and the draws
and outputs recorded from the reference's own solver runs (tests/golden)."""
import math

import numpy as np
import pytest
import torch

import sde_mc_gb300 as sm
from tests.cases import FIXTURE_CASES, asian_merton, heston, indep2d, inst_for, levy2d, loggbm_uniform, merton1d
from tests.conftest import load_npz


def test_philox_known_answers(oracle_mod):
    # Random123's published Philox4x32-10 known-answer vectors (Salmon et al., SC'11)
    import ctypes
    lib = oracle_mod.load()
    # counter = (block, c1, c2, c3): reproduce through the seed/stream/path mapping
    # ctr (0,0,0,0) key (0,0)
    out = oracle_mod.philox(0, 0, 0, 0, 0, 1)[0]
    assert [int(v) for v in out] == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    # ctr all ones, key all ones: block=0xffffffff, path lo=0xffffffff,
    # c2 = path_hi(0xffff) | tag 0xffff << 16, stream=0xffffffff
    out = oracle_mod.philox(0xFFFFFFFFFFFFFFFF, 0xFFFFFFFF, 0xFFFF, 0x0000FFFFFFFFFFFF, 0xFFFFFFFF, 1)[0]
    assert [int(v) for v in out] == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    out = oracle_mod.philox(0x299f31d0a4093822, 0x03707344, 0x1319, 0x8a2e85a308d3, 0x243f6a88, 1)[0]
    assert [int(v) for v in out] == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_closed_forms(oracle_mod, kat):
    args, v = kat["bs_call"]
    assert oracle_mod.bs_call(*args) == pytest.approx(v, rel=1e-12)
    args, v = kat["bs_binary_aon"]
    assert oracle_mod.bs_binary_aon(*args) == pytest.approx(v, rel=1e-9)
    for args, v in kat["merton_call"]:
        assert oracle_mod.merton_call(*args) == pytest.approx(v, rel=1e-12)
    args, v = kat["bs_digital_call"]
    assert oracle_mod.bs_digital_call(*args) == pytest.approx(v, rel=1e-10)
    args, v = kat["bs_asian_call"]
    assert oracle_mod.bs_asian_call(*args) == pytest.approx(v, rel=1e-12)
    assert oracle_mod.merton_call(1, 1, 3, 0.02, 0.3, -0.05, 0.3, 2) == pytest.approx(0.36328189504657027, rel=1e-12)


def test_mc_estimates(oracle_mod, kat):
    s = np.array(kat["mc_estimates"]["sample"], np.float64)
    m, v = oracle_mod.mc_estimates(s.sum(), (s * s).sum(), len(s))
    assert m == pytest.approx(kat["mc_estimates"]["mean"], rel=1e-6)
    assert v == pytest.approx(kat["mc_estimates"]["var"], rel=1e-6)


def _replay(oracle_mod, name):
    fx = load_npz(name)
    inst = inst_for(FIXTURE_CASES[name](), num_paths=int(fx["bs"]))
    if inst.grid == 1:
        out = oracle_mod.replay(inst, fx["dw"])
    else:
        out = oracle_mod.replay(inst, fx["dw"], fx["jump_times"], fx["marks"], fx.get("asset"))
    return fx, inst, out


@pytest.mark.parametrize("name", ["replay_merton1d", "replay_merton2d_corr", "replay_merton2d_exact",
                                  "replay_indep2d", "replay_gbm_uniform", "replay_asian_merton",
                                  "replay_loggbm_uniform", "replay_doublegbm_uniform"])
def test_replay_bit_exact_vs_reference(oracle_mod, name):
    """Recorded reference draws through the oracle's loop give the reference's
    paths, time grid, left limits, jump marks and payoffs bit for bit."""
    fx, inst, out = _replay(oracle_mod, name)
    assert out["rc"] == 0
    S = fx["paths"].shape[1] - 1
    np.testing.assert_array_equal(out["paths"][:, :S + 1], fx["paths"])
    if "time" in fx:
        np.testing.assert_array_equal(out["time"], fx["time"])
        np.testing.assert_array_equal(out["left"], fx["left"])
        np.testing.assert_array_equal(out["jumps"], expected_jump_paths(fx))
        assert int(out["steps"].max()) == int(fx["S"])
    if "payoffs" in fx:
        np.testing.assert_array_equal(out["payoffs"], fx["payoffs"])


def sqrt_tie_distance(v):
    """How far sqrt(v) (v float32) lies from the midpoint between its two
    neighbouring float32 values, in units of their spacing (0 = a tie)."""
    v = np.asarray(v, np.float32)
    exact = np.sqrt(v.astype(np.float64))
    lo = np.sqrt(v).astype(np.float32)
    lo = np.where(lo.astype(np.float64) > exact, np.nextafter(lo, np.float32(0)), lo)
    hi = np.nextafter(lo, np.float32(np.inf))
    frac = (exact - lo.astype(np.float64)) / (hi.astype(np.float64) - lo.astype(np.float64))
    return np.abs(frac - 0.5)


def heston_sqrt_inputs(x, dw1, inst):
    """The two square-root arguments of one Heston step from state x:
    v (the price diffusion) and b b - 4 a c (solve_quadratic), in the
    reference's float32 order (sde_mc/sde.py:275-279, helpers.py:46-47)."""
    f = np.float32
    v, h = x[..., 1].astype(f), f(inst.h)
    kap, kth, xi, xi2 = (f(inst.mark_p[i]) for i in range(4))
    a = f(-1) - kap * h
    b = xi * dw1.astype(f)
    c = (v + kth * h) - (f(0.5) * h) * xi2
    return v, (b * b) - (f(4) * a) * c


def test_replay_heston_vs_reference(oracle_mod):
    """Heston's implicit variance step (sde_mc/schemes.py:16-22).  The oracle
    and the kernels take correctly rounded square roots; the fixture was
    recorded with torch's x86 CPU sqrt, which rounds a near-tie the other way
    now and then.  So: one step of the oracle from every recorded state gives
    the recorded next state bit for bit except where a square-root argument
    sits within 1% of a rounding tie, and the whole trajectories agree to
    float32 rounding."""
    fx, inst, out = _replay(oracle_mod, "replay_heston")
    assert out["rc"] == 0
    P, dw = fx["paths"], fx["dw"]
    np.testing.assert_allclose(out["paths"], P, rtol=2e-6, atol=1e-9)
    np.testing.assert_allclose(out["payoffs"], fx["payoffs"], rtol=2e-6, atol=1e-9)
    assert np.mean(out["paths"] == P) > 0.99
    bs, S = dw.shape[0], dw.shape[1]
    one = inst_for(FIXTURE_CASES["replay_heston"](), num_paths=1)
    one.num_steps = 1
    mism, ties = 0, 0
    for p in range(bs):
        for k in range(S):
            for i in range(2):
                one.x0[i] = float(P[p, k, i])
            o = oracle_mod.replay(one, dw[p:p + 1, k:k + 1])
            assert o["rc"] == 0
            if not np.array_equal(o["paths"][0, 1], P[p, k + 1]):
                mism += 1
                v, disc = heston_sqrt_inputs(P[p, k], dw[p, k, 1], inst)
                near = min(sqrt_tie_distance(v), sqrt_tie_distance(disc))
                assert near < 0.01, (p, k, o["paths"][0, 1], P[p, k + 1], near)
                np.testing.assert_allclose(o["paths"][0, 1], P[p, k + 1], rtol=1e-6)
    assert mism <= 4


def expected_jump_paths(fx):
    """The per-asset adapter stores its encoded mark 10k + (1 + Y) in every
    column; the kernels store Y in asset k's column only.  Decode with the
    adapter's own float32 operations."""
    if "asset" not in fx:
        return fx["jumps"]
    m = fx["jumps"][..., 0].astype(np.float32)
    k = np.floor(m / np.float32(10.0))
    y = (m - np.float32(10.0) * k - np.float32(1.0)).astype(np.float32)
    out = np.zeros_like(fx["jumps"])
    for i in range(out.shape[-1]):
        out[..., i] = np.where((m != 0) & (k == i), y, np.float32(0.0))
    return out


def test_replay_levy_within_tolerance(oracle_mod):
    """The Levy drift folds -f*gamma into one coefficient, so it is 1e-5-close,
    not bit-exact; the time grid (pure float adds/mins) is still exact."""
    fx, inst, out = _replay(oracle_mod, "replay_levy2d")
    assert out["rc"] == 0
    np.testing.assert_array_equal(out["time"], fx["time"])
    np.testing.assert_allclose(out["paths"], fx["paths"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(out["payoffs"], fx["payoffs"], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("name,factory,levels", [("mlmc_merton1d", lambda: merton1d(4), (8, 4)),
                                                 ("mlmc_indep2d", lambda: indep2d(8), (16, 8)),
                                                 ("mlmc_asian_merton", lambda: asian_merton(4), (8, 4))])
def test_mlmc_replay_bit_exact(oracle_mod, name, factory, levels):
    fx = load_npz(name)
    inst = inst_for(factory(), num_paths=int(fx["bs"]), steps=levels[1])
    out = oracle_mod.mlmc_replay(inst, levels[0] // levels[1], float(fx["h_fine"]), float(fx["h_coarse"]),
                                 fx["dw"], fx["marks"].shape[1], fx["jump_times"], fx["marks"], fx.get("asset"))
    assert out["rc"] == 0
    np.testing.assert_array_equal(out["xf"], fx["xf"])
    np.testing.assert_array_equal(out["xc"], fx["xc"])


def test_mlmc_replay_levy_exact_jumps(oracle_mod):
    """The LevyRainbowMLMC coupling (sde_mc/problem.py:93-106): 2-D Levy
    'indep' model, exact_jumps=True, factor 2.  Within 1e-5 as the Levy
    replay (the drift folds -f*gamma into one coefficient); most paths are
    bit-exact."""
    fx = load_npz("mlmc_levy2d_exact")
    lev = sm.ExpExampleLevy(1, 1, 0.5, 2, 0.02, 0.2, 0.2, 0.2, 2)
    solver = sm.JumpEulerSolver(sm.LevySde(lev, torch.ones(2)), 1.0, 4, exact_jumps=True)
    inst = inst_for((solver, sm.Rainbow(1.0), sm.ConstantShortRate(0.02)), num_paths=int(fx["bs"]), steps=4)
    assert inst.exact_jumps == 1 and int(fx["max_jumps"]) == solver.max_jumps
    out = oracle_mod.mlmc_replay(inst, 2, float(fx["h_fine"]), float(fx["h_coarse"]), fx["dw"],
                                 fx["marks"].shape[1], fx["jump_times"], fx["marks"])
    assert out["rc"] == 0
    for k in ("xf", "xc"):
        np.testing.assert_allclose(out[k], fx[k], rtol=1e-5, atol=1e-6)
        assert np.mean(np.all(out[k] == fx[k], axis=1)) > 0.8


@pytest.mark.parametrize("name,levels,exact", [("mlmc_heston", (8, 4), False), ("mlmc_heston_f4", (16, 4), True)])
def test_mlmc_replay_heston(oracle_mod, name, levels, exact):
    """Coupled fine/coarse Heston levels (DiffusionSolver.multilevel_solve,
    sde_mc/solvers.py:90-119): the coarse step takes the fine increments'
    sum in the reference's order.  Bit-exact except where torch's x86 CPU
    sqrt rounded a near-tie the other way (one path of 32 in the (8, 4)
    fixture); those agree to float32 rounding."""
    from tests.cases import heston
    fx = load_npz(name)
    inst = inst_for(heston(levels[1]), num_paths=int(fx["bs"]), steps=levels[1])
    out = oracle_mod.mlmc_replay(inst, levels[0] // levels[1], float(fx["h_fine"]), float(fx["h_coarse"]),
                                 fx["dw"], levels[1])
    assert out["rc"] == 0
    np.testing.assert_array_equal(out["xc"], fx["xc"])
    if exact:
        np.testing.assert_array_equal(out["xf"], fx["xf"])
    else:
        np.testing.assert_allclose(out["xf"], fx["xf"], rtol=2e-6)
        assert np.all(out["xf"] == fx["xf"], axis=1).sum() >= int(fx["bs"]) - 1


def test_cv_mlp_grads_and_adam(oracle_mod):
    """Hand-written backprop of Var(payoff + sum e^{-rt} f . dW) and one Adam
    step agree with torch autograd + torch.optim.Adam run by the reference."""
    fx = load_npz("cv_mlp")
    params = [fx["p0_%d" % i].astype(np.float64) for i in range(8)]
    loss, gamma, grads = oracle_mod.cv_loss_and_grads(params, fx["f_in"].astype(np.float64),
                                                      fx["normals"].astype(np.float64),
                                                      fx["time"][..., 0].astype(np.float64),
                                                      fx["payoffs"].astype(np.float64), float(fx["r"]))
    assert loss == pytest.approx(float(fx["loss"]), rel=1e-4)
    np.testing.assert_allclose(gamma, fx["gamma"], rtol=1e-4, atol=1e-6)
    for i in range(8):
        np.testing.assert_allclose(grads[i], fx["grad_%d" % i], rtol=2e-3, atol=1e-7)
    new, _ = oracle_mod.adam_step(params, grads, lr=1e-3)
    for i in range(8):
        np.testing.assert_allclose(new[i], fx["p1_%d" % i], rtol=1e-5, atol=1e-6)


def test_cv_mixed_precision_restatement_vs_reference(oracle_mod):
    """The BF16 precision policy of the network kernels, restated on the CPU,
    stays within BF16 noise of the reference's FP32 network: outputs within 2%
    of their largest magnitude, every gradient within 2% in relative norm."""
    fx = load_npz("cv_mlp")
    p0 = [fx["p0_%d" % i] for i in range(8)]
    n, S, d = fx["normals"].shape
    out, _ = oracle_mod.mlp_forward_mixed(p0, fx["time"].reshape(-1), fx["paths"].reshape(-1, d))
    assert np.abs(out - fx["f_out"]).max() <= 2e-2 * np.abs(fx["f_out"]).max()
    gam, fo = oracle_mod.cv_gamma_mixed(p0, fx["time"][..., 0], fx["paths"], fx["normals"], fx["payoffs"],
                                        float(fx["r"]))
    scale = np.abs(fx["normals"] * fo).sum((1, 2))
    assert (np.abs(gam - fx["gamma"]) <= 1e-2 * scale + 1e-6).all()
    grads = oracle_mod.cv_grads_mixed(p0, fx["time"][..., 0], fx["paths"], fx["normals"], fx["gamma"],
                                      float(fx["r"]))
    for i in range(8):
        ref = fx["grad_%d" % i]
        assert np.linalg.norm(grads[i] - ref) <= 2e-2 * np.linalg.norm(ref), i
    # bf16_round: ties to even, exact values unchanged
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5], np.float32)
    np.testing.assert_array_equal(oracle_mod.bf16_round(v), [1.0, 1.0, 1.0 + 2 ** -6, 1.0, -2.5])


def test_native_price_vs_merton_closed_form(oracle_mod, kat, ref_stats):
    """The oracle's own Philox draws through the reference loop price the 1D Merton call
    within 3 standard errors of the Merton series and of the reference's run."""
    case = merton1d(100)
    inst = inst_for(case, num_paths=1 << 17, seed=11)
    out, _, rc = oracle_mod.price(inst)
    assert rc == 0
    mean, var = out[3], out[4]
    se = math.sqrt(var / out[2])
    exact = kat["merton_call"][1][1]
    assert abs(mean - exact) < 3 * se + 1e-4  # Euler bias at 100 steps is below 1e-4
    r = ref_stats["c1_fp32_2p18"]
    assert abs(mean - r["mean"]) < 3 * math.hypot(se, r["se"])


def test_native_price_c2_vs_reference(oracle_mod, ref_stats):
    inst = inst_for(indep2d(256), num_paths=1 << 15, seed=5)
    out, _, rc = oracle_mod.price(inst)
    assert rc == 0
    se = math.sqrt(out[4] / out[2])
    r = ref_stats["c2_plain_2p16"]
    assert abs(out[3] - r["mean"]) < 3 * math.hypot(se, r["se"])


@pytest.mark.parametrize("name,factory", [("heston_64_2p16", lambda: heston(64)),
                                          ("asian_merton_20_2p16", lambda: asian_merton(20)),
                                          ("levy2d_16_2p16", lambda: levy2d(16)),
                                          ("loggbm_16_2p16", lambda: loggbm_uniform(16))])
def test_native_price_vs_reference_estimates(oracle_mod, ref_stats, name, factory):
    """The oracle's own Philox run of each model kind against the reference's
    mc_simple estimate of the same problem (independent draws): within 3
    combined standard errors."""
    inst = inst_for(factory(), num_paths=1 << 16, seed=8)
    out, _, rc = oracle_mod.price(inst)
    assert rc == 0 and out[2] == 1 << 16
    se = math.sqrt(out[4] / out[2])
    r = ref_stats[name]
    assert abs(out[3] - r["mean"]) < 3 * math.hypot(se, r["se"]), (out[3], r["mean"], se, r["se"])


def test_mlmc_level_statistics_vs_reference(oracle_mod, ref_stats):
    """The oracle's coupled levels of the 2D rainbow (its own Philox draws)
    against the reference's multilevel_solve statistics at the same levels:
    the mean of P_f - P_c within 3.5 combined SE, its variance within 30%."""
    for ref in ref_stats["c2_mlmc_level_stats"]:
        fine, coarse = ref["levels"]
        inst = inst_for(indep2d(coarse), num_paths=1 << 14, seed=12, steps=coarse)
        hf = float(np.float32(1.0) / np.float32(fine))
        hc = float(np.float32(fine // coarse) * np.float32(hf))
        out, rc = oracle_mod.mlmc_level(inst, fine // coarse, hf, hc)
        assert rc == 0 and out[2] == 1 << 14
        n = out[2]
        mean = out[0] / n
        var = (out[1] - out[0] ** 2 / n) / (n - 1)
        se = math.sqrt(var / n + ref["var"] / ref["n"])
        assert abs(mean - ref["mean"]) < 3.5 * se, (fine, coarse, mean, ref["mean"], se)
        assert var == pytest.approx(ref["var"], rel=0.3)


def test_chunk_reduce_matches_fp64_sum(oracle_mod):
    rng = np.random.default_rng(0)
    v = rng.random(1000).astype(np.float32)
    out = oracle_mod.chunk_reduce(v)
    assert out[2] == 1000
    assert out[0] == pytest.approx(float(v.astype(np.float64).sum()), rel=1e-6)
    assert out[3] == pytest.approx(float(v.mean()), rel=1e-6)


def test_cv_with_jump_integrand_restatement(oracle_mod):
    """Both integrands of the reference's adapted control variate (f on the
    Brownian increments, g on the marks minus lambda E[J] h): the oracle's
    Gamma sums, loss and gradients of both networks equal what the reference's
    own apply/train functions produced (fixture)."""
    fx = load_npz("cv_mlp_jumps")
    pf = [fx["p0f_%d" % i].astype(np.float64) for i in range(8)]
    pg = [fx["p0g_%d" % i].astype(np.float64) for i in range(8)]
    t = fx["time"][..., 0]
    mult = oracle_mod.cv_jump_multipliers(t, fx["jumps"], fx["lam_kappa"])
    loss, gamma, gf, gg = oracle_mod.cv2_loss_and_grads(pf, pg, t, fx["paths"], fx["left"], fx["normals"], mult,
                                                        fx["payoffs"], float(fx["r"]))
    assert loss == pytest.approx(float(fx["loss"]), rel=1e-5)
    assert gamma.sum() == pytest.approx(float(fx["sum"]), rel=1e-5)
    assert (gamma * gamma).sum() == pytest.approx(float(fx["sum_sq"]), rel=1e-5)
    for i in range(8):
        np.testing.assert_allclose(gf[i], fx["gradf_%d" % i], rtol=2e-3, atol=1e-6)
        np.testing.assert_allclose(gg[i], fx["gradg_%d" % i], rtol=2e-3, atol=1e-6)


def test_heston_closed_form_limits(oracle_mod):
    """The Fourier-inversion Heston call (the independent check of the Heston
    kernels) reduces to Black-Scholes when the variance is constant (v0 =
    theta, vol of vol -> 0), decreases in the strike and stays inside the
    no-arbitrage bounds."""
    bs = oracle_mod.bs_call(1.0, 1.0, 1.0, 0.02, 0.2)
    assert oracle_mod.heston_call(1.0, 0.04, 1.0, 1.0, 0.02, 2.0, 0.04, 1e-4, -0.7) == pytest.approx(bs, rel=1e-6)
    prices = [oracle_mod.heston_call(1.0, 0.04, k, 1.0, 0.02, 2.0, 0.04, 0.3, -0.7) for k in (0.8, 0.9, 1.0, 1.1)]
    assert all(a > b for a, b in zip(prices, prices[1:]))
    for k, c in zip((0.8, 0.9, 1.0, 1.1), prices):
        assert max(0.0, 1.0 - k * math.exp(-0.02)) < c < 1.0
