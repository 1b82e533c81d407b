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

from sde_mc_gb300 import _native as N
from sde_mc_gb300 import kernels as K
from tests.cases import (FIXTURE_CASES, asian_merton, basket, double_gbm, gbm_uniform, heston, indep2d, inst_for,
                         levy2d, merton1d, merton2d_corr, zdim)
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
}


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
    for key in ("paths", "left", "time", "jumps", "normals", "payoffs"):
        np.testing.assert_array_equal(g[key], ref[key], err_msg=key)


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
