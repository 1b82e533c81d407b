"""torch.ops.sdemc.* run the same kernels as the Python wrappers: identical
bits on the same inputs."""
import numpy as np
import pytest
import torch

import sde_mc_gb300 as sm
from sde_mc_gb300 import kernels as K
from sde_mc_gb300 import torch_ops as T
from sde_mc_gb300 import varred as V
from sde_mc_gb300.lowering import lower
from sde_mc_gb300.solvers import level_steps
from tests.cases import indep2d

pytestmark = pytest.mark.gpu


def test_price_and_mlmc_ops_match_wrappers():
    solver, payoff, disc = indep2d(32)
    inst = lower(solver, payoff, disc, num_paths=10_000, path_offset=5)
    a = torch.ops.sdemc.price(T.inst_tensor(inst))
    b = K.price(inst)
    torch.testing.assert_close(a, b, rtol=0, atol=0)
    a2 = torch.ops.sdemc.price(T.inst_tensor(inst), 64)
    torch.testing.assert_close(a2, b, rtol=0, atol=0)
    hf, hc = level_steps(solver, 16, 8)
    lv = lower(solver, payoff, disc, num_paths=8192, num_steps=8)
    torch.testing.assert_close(torch.ops.sdemc.mlmc_level(T.inst_tensor(lv), 16, 8, hf, hc),
                               K.mlmc_level(lv, 16, 8, hf, hc), rtol=0, atol=0)
    w = torch.ops.sdemc.philox(7, 3, 0, 11, 0, 4)
    torch.testing.assert_close(w, K.philox(7, 3, 0, 11, 0, 4), rtol=0, atol=0)


def test_cv_ops_match_wrappers():
    solver, payoff, disc = indep2d(16, seed=3)
    dl = sm.simulate_adapted_data(256, solver, payoff, disc, bs=256, inference=True)
    data = V.CvData.from_dataset(dl.dataset, solver, torch.device("cuda"))
    torch.manual_seed(1)
    f = sm.Mlp(3, [64, 64, 64], 2, batch_norm=False, batch_norm_init=False)
    cv = V.GpuCv(f, 2, torch.device("cuda"))
    idx = torch.randperm(data.n, device="cuda")[:128]
    g_ref = cv.forward(data, 0.02, idx=idx).clone()
    g_op = torch.ops.sdemc.cv_forward(cv.params, data.time, data.paths, data.normals, data.payoffs, idx, 0.02)
    torch.testing.assert_close(g_op, g_ref, rtol=0, atol=0)
    gr_ref = cv.backward(data, 0.02, g_ref, idx=idx).clone()
    gr_op = torch.ops.sdemc.cv_backward(cv.params, data.time, data.paths, data.normals, g_op, idx, 0.02)
    torch.testing.assert_close(gr_op, gr_ref, rtol=0, atol=0)
    p, m, v = cv.params.clone(), torch.zeros_like(cv.params), torch.zeros_like(cv.params)
    torch.ops.sdemc.adam_step(p, gr_op, m, v, 1, 1e-3, 0.9, 0.999, 1e-8)
    cv.grad.copy_(gr_op)
    cv.adam(1e-3)
    torch.testing.assert_close(p, cv.params, rtol=0, atol=0)
    with pytest.raises(ValueError):
        torch.ops.sdemc.cv_forward(cv.params.double(), data.time, data.paths, data.normals, data.payoffs, None,
                                   0.02)


def test_store_fp64_and_tensor_core_ops_match_wrappers():
    from tests.cases import FIXTURE_CASES, inst_for
    from tests.conftest import load_npz
    solver, payoff, disc = indep2d(24)
    inst = lower(solver, payoff, disc, num_paths=777, path_offset=9)
    torch.testing.assert_close(torch.ops.sdemc.price_f64(T.inst_tensor(inst)), K.price_f64(inst), rtol=0, atol=0)
    S = solver.num_steps + solver.max_jumps
    outs = torch.ops.sdemc.materialise(T.inst_tensor(inst), S)
    ref = K.materialise(inst, S)
    for t, key in zip(outs, ("paths", "left", "time", "jumps", "normals", "payoffs", "steps", "status")):
        torch.testing.assert_close(t, ref[key], rtol=0, atol=0)
    fx = load_npz("replay_merton1d")
    ri = inst_for(FIXTURE_CASES["replay_merton1d"](), num_paths=int(fx["bs"]))
    args = [torch.from_numpy(fx[k]).cuda() for k in ("dw", "jump_times", "marks")]
    r_op = torch.ops.sdemc.replay(T.inst_tensor(ri), args[0], args[1], args[2], None)
    r_ref = K.replay(ri, *args)
    for t, key in zip(r_op, ("paths", "left", "time", "jumps", "payoffs", "steps", "status")):
        torch.testing.assert_close(t, r_ref[key], rtol=0, atol=0)
    # K7 and K6 on tcgen05
    torch.manual_seed(2)
    f = sm.Mlp(3, [64, 64, 64], 2, batch_norm=False, batch_norm_init=False)
    cv = V.GpuCv(f, 2, torch.device("cuda"))
    pi = lower(solver, payoff, disc, num_paths=4096, path_offset=3)
    torch.testing.assert_close(torch.ops.sdemc.price_cv(T.inst_tensor(pi), cv.params, 0.02),
                               K.price_cv(pi, cv.params, 0.02), rtol=0, atol=0)
    dl = sm.simulate_adapted_data(256, solver, payoff, disc, bs=256, inference=True)
    data = V.CvData.from_dataset(dl.dataset, solver, torch.device("cuda"))
    g = cv.forward(data, 0.02)
    gr_ref = cv.backward_tc(data, 0.02, g).clone()
    gr_op = torch.ops.sdemc.cv_backward_tc(cv.params, data.time, data.paths, data.normals, g, None, 0.02)
    torch.testing.assert_close(gr_op, gr_ref, rtol=0, atol=0)
