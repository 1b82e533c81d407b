"""GPU parity of the path kernels (all calls go through the C ABI).

* K3 replay on draws recorded from the reference reproduces the reference's
  paths, time grid, left limits, marks and payoffs bit for bit (Levy: 1e-5).
* K4 with its raw draws exported is re-run step by step by the CPU oracle:
  every stored tensor matches bit for bit; the raw normals and jump stream
  match the oracle's own Philox + libm transforms within 2e-5.
* K1's per-path payoffs equal K4's bit for bit, its FP64 sums equal the
  oracle's restatement of the reduction order bit for bit, and they do not
  change with the launch shape.
"""
import math

import numpy as np
import pytest
import torch

import sde_mc_gb300 as sm
from sde_mc_gb300 import _native as N
from sde_mc_gb300 import kernels as K
from tests.cases import (FIXTURE_CASES, asian_merton, basket, double_gbm, gbm_uniform, heston, indep2d, inst_for,
                         levy2d, levy2d_exact, merton1d, merton2d_corr, zdim)
from tests.conftest import load_npz
from tests.test_oracle import expected_jump_paths

pytestmark = pytest.mark.gpu


def np_(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("name", list(FIXTURE_CASES))
def test_replay_matches_reference(name, oracle_mod):
    fx = load_npz(name)
    inst = inst_for(FIXTURE_CASES[name](), num_paths=int(fx["bs"]))
    dw = torch.from_numpy(fx["dw"])
    if inst.grid == N.GRID_UNIFORM:
        out = K.replay(inst, dw)
    else:
        asset = torch.from_numpy(fx["asset"]) if "asset" in fx else None
        out = K.replay(inst, dw, torch.from_numpy(fx["jump_times"]), torch.from_numpy(fx["marks"]), asset)
    assert int(out["status"].item()) == 0
    paths = np_(out["paths"])
    S = fx["paths"].shape[1] - 1
    if name == "replay_levy2d":
        np.testing.assert_array_equal(np_(out["time"]), fx["time"])
        np.testing.assert_allclose(paths, fx["paths"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(np_(out["payoffs"]), fx["payoffs"], rtol=1e-5, atol=1e-6)
    elif name == "replay_heston":
        # correctly rounded sqrt here, torch's x86 CPU sqrt in the fixture:
        # near-tie roundings differ (pinned step by step in test_oracle.py)
        np.testing.assert_allclose(paths, fx["paths"], rtol=2e-6, atol=1e-9)
        np.testing.assert_allclose(np_(out["payoffs"]), fx["payoffs"], rtol=2e-6, atol=1e-9)
    else:
        np.testing.assert_array_equal(paths[:, :S + 1], fx["paths"])
        if "time" in fx:
            np.testing.assert_array_equal(np_(out["time"]), fx["time"])
            np.testing.assert_array_equal(np_(out["left"]), fx["left"])
            np.testing.assert_array_equal(np_(out["jumps"]), expected_jump_paths(fx))
            np.testing.assert_array_equal(np_(out["payoffs"]), fx["payoffs"])
            assert int(np_(out["steps"]).max()) == int(fx["S"])
    # and the GPU agrees with the oracle's replay bit for bit
    ref = oracle_mod.replay(inst, fx["dw"], fx.get("jump_times") if inst.grid == 0 else None,
                            fx.get("marks") if inst.grid == 0 else None, fx.get("asset"))
    np.testing.assert_array_equal(paths, ref["paths"])
    if inst.payoff_log:
        # Option.log: CUDA's expf and libm's expf may round the last bit apart
        # (1.2e-7 at exp(x) ~ 1, which max(exp(x) - K, 0) keeps as an absolute error)
        np.testing.assert_allclose(np_(out["payoffs"]), ref["payoffs"], rtol=1e-6, atol=1e-6)
    else:
        np.testing.assert_array_equal(np_(out["payoffs"]), ref["payoffs"])


@pytest.mark.parametrize("name,factory,levels", [("mlmc_merton1d", lambda: merton1d(4), (8, 4)),
                                                 ("mlmc_indep2d", lambda: indep2d(8), (16, 8))])
def test_mlmc_replay_matches_reference(name, factory, levels):
    fx = load_npz(name)
    inst = inst_for(factory(), num_paths=int(fx["bs"]), steps=levels[1])
    asset = torch.from_numpy(fx["asset"]) if "asset" in fx else None
    out = K.mlmc_replay(inst, levels[0], levels[1], float(fx["h_fine"]), float(fx["h_coarse"]),
                        torch.from_numpy(fx["dw"]), fx["marks"].shape[1], torch.from_numpy(fx["jump_times"]),
                        torch.from_numpy(fx["marks"]), asset)
    assert int(out["status"].item()) == 0
    np.testing.assert_array_equal(np_(out["xf"]), fx["xf"])
    np.testing.assert_array_equal(np_(out["xc"]), fx["xc"])


@pytest.mark.parametrize("name,factory,levels,exact", [
    ("mlmc_asian_merton", lambda: asian_merton(4), (8, 4), True),
    ("mlmc_levy2d_exact", lambda: levy2d_exact(4), (8, 4), False)])
def test_mlmc_replay_asian_and_levy_exact_jumps(name, factory, levels, exact, oracle_mod):
    """K2 on the last two couplings recorded from the reference: the Asian
    wrapper around Merton (sde_mc/sde.py:378-406) and the LevyRainbowMLMC
    preset (Levy 'indep', exact_jumps=True, factor 2; sde_mc/problem.py:93-106,
    coupling loop sde_mc/solvers.py:228-307).  GPU == oracle bit for bit; the
    Asian coupling also == the reference's recorded states bit for bit, the
    Levy one within 1e-5 (its drift folds -f*gamma into one coefficient)."""
    fx = load_npz(name)
    inst = inst_for(factory(), num_paths=int(fx["bs"]), steps=levels[1])
    asset = torch.from_numpy(fx["asset"]) if "asset" in fx else None
    out = K.mlmc_replay(inst, levels[0], levels[1], float(fx["h_fine"]), float(fx["h_coarse"]),
                        torch.from_numpy(fx["dw"]), fx["marks"].shape[1], torch.from_numpy(fx["jump_times"]),
                        torch.from_numpy(fx["marks"]), asset)
    assert int(out["status"].item()) == 0
    ref = oracle_mod.mlmc_replay(inst, levels[0] // levels[1], float(fx["h_fine"]), float(fx["h_coarse"]),
                                 fx["dw"], fx["marks"].shape[1], fx["jump_times"], fx["marks"], fx.get("asset"))
    for k in ("xf", "xc"):
        np.testing.assert_array_equal(np_(out[k]), ref[k])
        if exact:
            np.testing.assert_array_equal(np_(out[k]), fx[k])
        else:
            np.testing.assert_allclose(np_(out[k]), fx[k], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("name,factory,levels", [("mlmc_cols_merton1d", lambda: merton1d(4), (8, 4)),
                                                 ("mlmc_cols_indep2d", lambda: indep2d(8), (16, 8)),
                                                 ("mlmc_cols_gbm_uniform", lambda: gbm_uniform(4), (8, 4))])
def test_mlmc_columns_match_reference(name, factory, levels):
    """Every column multilevel_solve returns, replayed from the reference's own
    draws: the jump-adapted grid's fine and coarse states after each coarse
    step up to the batch's last (sde_mc/solvers.py:228-307), and the uniform
    grid's every fine and coarse state (:90-119) — bit for bit."""
    fx = load_npz(name)
    inst = inst_for(factory(), num_paths=int(fx["bs"]), steps=levels[1])
    hf, hc = float(fx["h_fine"]), float(fx["h_coarse"])
    if inst.grid == N.GRID_UNIFORM:
        cols = (levels[0] + 1, levels[1] + 1)
        out = K.mlmc_replay(inst, levels[0], levels[1], hf, hc, torch.from_numpy(fx["normals"]), levels[1], cols=cols)
        total = None
    else:
        c = levels[1] + int(fx["max_jumps"]) + 1
        asset = torch.from_numpy(fx["asset"]) if "asset" in fx else None
        out = K.mlmc_replay(inst, levels[0], levels[1], hf, hc, torch.from_numpy(fx["dw"]), fx["marks"].shape[1],
                            torch.from_numpy(fx["jump_times"]), torch.from_numpy(fx["marks"]), asset, cols=(c, c))
        total = int(np_(out["steps"]).max())
        assert total + 1 == fx["paths_fine"].shape[1]
    assert int(out["status"].item()) == 0
    pf, pc = np_(out["paths_fine"]), np_(out["paths_coarse"])
    if total is not None:
        pf, pc = pf[:, :total + 1], pc[:, :total + 1]
    np.testing.assert_array_equal(pf, fx["paths_fine"])
    np.testing.assert_array_equal(pc, fx["paths_coarse"])


@pytest.mark.parametrize("factory,levels", [(lambda: indep2d(8), (16, 8)), (lambda: merton2d_corr(6), (12, 6)),
                                            (lambda: gbm_uniform(6), (24, 6)), (lambda: heston(4), (16, 4))])
def test_multilevel_solve_returns_every_column(factory, levels):
    """multilevel_solve's drop-in shapes and contents on the kernels' own
    draws: the first column is the initial state, the last the terminal states
    the estimators' level kernels compute (bit for bit); on the jump-adapted
    grid the batch has total_steps_coarse + 1 columns with finished paths
    frozen; on the uniform grid fine + 1 and coarse + 1 columns and the fine
    increments, whose sums drive the coarse steps."""
    solver = factory()[0]
    bs = 300
    cursor = solver.path_cursor
    (pf, pc), nz = solver.multilevel_solve(bs, levels)
    solver.path_cursor = cursor  # the same paths again
    d = solver.sde.dim
    x0 = torch.as_tensor(solver.sde.init_value, dtype=torch.float32).reshape(1, d).expand(bs, d)
    np.testing.assert_array_equal(np_(pf[:, 0]), np_(x0))
    np.testing.assert_array_equal(np_(pc[:, 0]), np_(x0))
    (tf, tc), _ = solver.multilevel_terminals(bs, levels)
    np.testing.assert_array_equal(np_(pf[:, -1]), np_(tf[:, -1]))
    np.testing.assert_array_equal(np_(pc[:, -1]), np_(tc[:, -1]))
    if solver.has_jumps:
        assert nz is None and pf.shape == pc.shape and pf.shape[0] == bs and pf.shape[2] == d
        assert pf.shape[1] >= levels[1] + 1
    else:
        assert pf.shape == (bs, levels[0] + 1, d) and pc.shape == (bs, levels[1] + 1, d)
        assert tuple(nz.shape[:3]) == (bs, levels[0], d)
        assert torch.isfinite(nz).all() and np_(nz).std() > 0


@pytest.mark.parametrize("name,levels", [("mlmc_heston", (8, 4)), ("mlmc_heston_f4", (16, 4))])
def test_mlmc_replay_heston(name, levels, oracle_mod):
    """K2's uniform-grid coupled Heston levels equal the oracle's bit for bit
    (which pins them to the reference, test_oracle.py)."""
    fx = load_npz(name)
    inst = inst_for(heston(levels[1]), num_paths=int(fx["bs"]), steps=levels[1])
    out = K.mlmc_replay(inst, levels[0], levels[1], float(fx["h_fine"]), float(fx["h_coarse"]),
                        torch.from_numpy(fx["dw"]), levels[1])
    assert int(out["status"].item()) == 0
    ref = oracle_mod.mlmc_replay(inst, levels[0] // levels[1], float(fx["h_fine"]), float(fx["h_coarse"]),
                                 fx["dw"], levels[1])
    np.testing.assert_array_equal(np_(out["xf"]), ref["xf"])
    np.testing.assert_array_equal(np_(out["xc"]), ref["xc"])
    np.testing.assert_array_equal(np_(out["xc"]), fx["xc"])


def test_philox_bit_exact(oracle_mod):
    for seed, stream, tag, path, first in [(0, 0, 0, 0, 0), (1, 3, 1, 12345, 7), (2 ** 63 + 5, 9, 0, 2 ** 40 + 3, 1000),
                                           (0xFFFFFFFFFFFFFFFF, 0xFFFFFFFF, 0xFFFF, 2 ** 48 - 1, 0xFFFFFF00)]:
        g = np_(K.philox(seed, stream, tag, path, first, 64)).view(np.uint32)
        c = oracle_mod.philox(seed, stream, tag, path, first, 64)
        np.testing.assert_array_equal(g, c)


EXPORT_CASES = {
    "merton1d": lambda: merton1d(100),
    "merton2d_corr": lambda: merton2d_corr(50),
    "merton2d_exact": lambda: merton2d_corr(20, exact=True),
    "indep2d": lambda: indep2d(64),
    "levy2d": lambda: levy2d(16),
    "gbm_uniform": lambda: gbm_uniform(12),
    "basket3": lambda: basket(3, 32),
    "basket5": lambda: basket(5, 24),
    "basket8": lambda: basket(8, 16),
    "double_gbm": lambda: double_gbm(3, 10),
    "heston": lambda: heston(24),
    "asian_merton": lambda: asian_merton(20),
    # the remaining payoff branches of the kernels' payoff() (sde_mc/options.py:179-321)
    "put1d": lambda: _with_payoff(merton1d(60), sm.EuroPut(1.05)),
    "binary_aon1d": lambda: _with_payoff(merton1d(60), sm.BinaryAoN(1.0)),
    "digital1d": lambda: _with_payoff(merton1d(60), sm.Digital(0.95)),
    "bestof3": lambda: _with_payoff(basket(3, 32), sm.BestOf(1.1)),
    "basket4_geometric": lambda: _with_payoff(basket(4, 24), sm.Basket(1.0, average_type="geometric")),
    "heston_rainbow": lambda: _with_payoff(heston(24), sm.HestonRainbow(1.0)),
}
# payoffs through CUDA's logf/expf, which may round the last bit apart from libm's
LIBM_PAYOFFS = {"basket4_geometric"}


def _with_payoff(case, payoff):
    return case[0], payoff, case[2]


def _export(name, n=1000, seed=77):
    case = EXPORT_CASES[name]()
    solver = case[0]
    inst = inst_for(case, num_paths=n, seed=seed, path_offset=12345)
    if inst.grid == N.GRID_ADAPTED:
        S = solver.num_steps + solver.max_jumps + 40
        jcap = solver.max_jumps + 40
    else:
        S, jcap = solver.num_steps, 0
    out = K.materialise(inst, S, export_draws=True, jcap=jcap)
    assert int(out["status"].item()) == 0
    return inst, S, jcap, out


@pytest.mark.parametrize("name", list(EXPORT_CASES))
def test_materialise_matches_oracle_step_by_step(name, oracle_mod):
    inst, S, jcap, out = _export(name)
    g = {k: np_(v) for k, v in out.items()}
    ref = oracle_mod.from_export(inst, g["z"], S, g.get("jt"), g.get("jm"), g.get("jsel"), exact=False)
    assert ref["rc"] == 0
    np.testing.assert_array_equal(g["steps"], ref["steps"])
    for key in ("paths", "left", "time", "jumps", "normals"):
        np.testing.assert_array_equal(g[key], ref[key], err_msg=key)
    if name in LIBM_PAYOFFS:
        np.testing.assert_allclose(g["payoffs"], ref["payoffs"], rtol=1e-6, atol=1e-6)
    else:
        np.testing.assert_array_equal(g["payoffs"], ref["payoffs"])
    assert np.count_nonzero(g["payoffs"]) > 0


@pytest.mark.parametrize("name", list(EXPORT_CASES))
def test_tiled_stores_equal_per_lane_stores(name):
    """K4 writes through shared-memory tiles (coalesced segments) unless the
    raw draws are exported; both give the same AdaptedPathData bits, with the
    step cap odd, exact and short of the loop (overflow)."""
    case = EXPORT_CASES[name]()
    solver = case[0]
    base = solver.num_steps + solver.max_jumps + 3 if is_adapted(case) else solver.num_steps
    for S, n in ((base, 777), (base + 5, 130), (max(solver.num_steps // 2, 1), 64)):
        if not is_adapted(case) and S < solver.num_steps:
            continue
        inst = inst_for(case, num_paths=n, seed=19, path_offset=3)
        a = K.materialise(inst, S)
        b = K.materialise(inst, S, export_draws=True, jcap=0)
        for key in ("paths", "left", "time", "jumps", "normals", "payoffs", "steps", "status"):
            np.testing.assert_array_equal(np_(a[key]), np_(b[key]), err_msg="%s S=%d" % (key, S))


def is_adapted(case):
    return hasattr(case[0], "max_jumps")


@pytest.mark.parametrize("name", ["merton1d", "indep2d", "levy2d", "basket5", "double_gbm", "heston"])
def test_native_draws_match_oracle_transforms(name, oracle_mod):
    """Philox words are bit-exact (above); the MUFU-based Box-Muller and the
    jump-stream transforms agree with the oracle's libm versions to 2e-5."""
    inst, S, jcap, out = _export(name, n=64)
    z = np_(out["z"])
    steps = np_(out["steps"])
    for p in range(0, 64, 9):
        zo = oracle_mod.native_normals(inst, p, int(steps[p]), zdim(inst))
        np.testing.assert_allclose(z[p, :steps[p]], zo, rtol=2e-5, atol=2e-5)
        if jcap:
            jt, jm, js = oracle_mod.native_jumps(inst, p, jcap)
            np.testing.assert_allclose(np_(out["jt"])[p], jt, rtol=2e-6)
            np.testing.assert_allclose(np_(out["jm"])[p], jm, rtol=2e-5, atol=2e-6)
            np.testing.assert_array_equal(np_(out["jsel"])[p], js)


@pytest.mark.parametrize("name", ["merton1d", "merton2d_corr", "indep2d", "levy2d", "gbm_uniform", "basket8",
                                  "heston", "asian_merton"])
def test_fused_price_matches_materialised_and_reduction(name, oracle_mod):
    case = EXPORT_CASES[name]()
    n = 5000
    inst = inst_for(case, num_paths=n, seed=31, path_offset=999)
    pay = torch.empty(n, dtype=torch.float32, device="cuda")
    res = np_(K.price(inst, payoffs=pay))
    assert res[5] == 0
    solver = case[0]
    S = solver.num_steps + solver.max_jumps + 40 if inst.grid == N.GRID_ADAPTED else solver.num_steps
    m = K.materialise(inst, S, want=("payoffs", "steps"))
    np.testing.assert_array_equal(np_(pay), np_(m["payoffs"]))
    red = oracle_mod.chunk_reduce(np_(pay))
    np.testing.assert_array_equal(res[:5], red)


def test_price_invariant_to_launch_shape():
    inst = inst_for(indep2d(64), num_paths=100_000, seed=3)
    base = np_(K.price(inst))
    for bt, cps, il in [(32, 1, 1), (64, 3, 1), (256, 2, 1), (128, 0, 0), (96, 5, 1), (128, 0, 2), (64, 3, 2),
                        (256, 1, 2)]:
        cfg = N.SdemcCfg(block_threads=bt, ctas_per_sm=cps, interleave=il)
        np.testing.assert_array_equal(np_(K.price(inst, cfg=cfg)), base)


@pytest.mark.parametrize("name", ["merton1d", "merton2d_exact", "indep2d", "gbm_uniform", "basket5", "double_gbm",
                                  "heston", "asian_merton"])
def test_two_paths_per_lane_is_bit_identical(name):
    """Paths-per-thread tiling (cfg.interleave = 2, simulate2) gives every path
    the bits of the one-path loop: payoffs and sums, odd chunk counts included."""
    case = EXPORT_CASES[name]()
    for n in (32 * 7 + 5, 20000):
        inst = inst_for(case, num_paths=n, seed=13, path_offset=77)
        p1 = torch.empty(n, dtype=torch.float32, device="cuda")
        p2 = torch.empty(n, dtype=torch.float32, device="cuda")
        r1 = np_(K.price(inst, payoffs=p1))
        r2 = np_(K.price(inst, cfg=N.SdemcCfg(interleave=2), payoffs=p2))
        np.testing.assert_array_equal(np_(p1), np_(p2))
        np.testing.assert_array_equal(r1, r2)
    inst.flags |= N.INST_PAYOFF_AT_NOMINAL_STEP
    np.testing.assert_array_equal(np_(K.price(inst)), np_(K.price(inst, cfg=N.SdemcCfg(interleave=2))))
    ex = N.SdemcCfg(flags=N.CFG_EXACT_EULER)
    ex2 = N.SdemcCfg(flags=N.CFG_EXACT_EULER, interleave=2)
    np.testing.assert_array_equal(np_(K.price(inst, cfg=ex)), np_(K.price(inst, cfg=ex2)))


def test_exact_euler_variant_replays_reference_order(oracle_mod):
    """The cfg flag that selects the reference's unfused Euler order gives the
    same bits as the oracle's exact-mode re-run of the exported draws."""
    inst, S, jcap, out = _export("merton1d", n=512)
    g = {k: np_(v) for k, v in out.items()}
    ref = oracle_mod.from_export(inst, g["z"], S, g["jt"], g["jm"], g["jsel"], exact=True)
    pay = torch.empty(512, dtype=torch.float32, device="cuda")
    K.price(inst, cfg=N.SdemcCfg(flags=N.CFG_EXACT_EULER), payoffs=pay)
    np.testing.assert_array_equal(np_(pay), ref["payoffs"])


def test_overflow_is_reported_not_written():
    solver, payoff, disc = merton1d(100)
    inst = inst_for((solver, payoff, disc), num_paths=256, seed=1)
    out = K.materialise(inst, 50)  # storage for 50 steps: every path needs ~100
    assert int(out["status"].item()) == N.EOVERFLOW


def test_empty_and_ragged_sizes():
    for n in [0, 1, 31, 127, 129, 1000]:
        inst = inst_for(merton1d(10), num_paths=n, seed=2)
        r = np_(K.price(inst))
        assert r[2] == n and r[5] == 0
        if n:
            m = K.materialise(inst, 40, want=("payoffs",))
            pay = torch.empty(max(n, 1), dtype=torch.float32, device="cuda")
            K.price(inst, payoffs=pay)
            np.testing.assert_array_equal(np_(pay)[:n], np_(m["payoffs"]))


def test_path_offset_continues_the_stream():
    """Two launches over [0, n) and [n, 2n) give the payoffs of one launch over [0, 2n)."""
    n = 4096
    a = torch.empty(2 * n, dtype=torch.float32, device="cuda")
    b = torch.empty(n, dtype=torch.float32, device="cuda")
    c = torch.empty(n, dtype=torch.float32, device="cuda")
    K.price(inst_for(indep2d(32), num_paths=2 * n, seed=9, path_offset=0), payoffs=a)
    K.price(inst_for(indep2d(32), num_paths=n, seed=9, path_offset=0), payoffs=b)
    K.price(inst_for(indep2d(32), num_paths=n, seed=9, path_offset=n), payoffs=c)
    np.testing.assert_array_equal(np_(a), np.concatenate([np_(b), np_(c)]))
