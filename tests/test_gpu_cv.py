"""Control-variate network kernels (K5 forward, K6 backward, Adam) against the
CPU oracle and the reference's own network, and what the trained network
gains over the plain estimator.

Tolerances: against the oracle's restatement of the kernels' precision policy
(FP32 layers 1 and 4, BF16 64x64 layers with FP32 accumulation) the kernels
agree to accumulation-order noise — outputs within 1e-3 of their largest
magnitude, gradients within 3e-3 in relative norm.  Against the reference's
FP32 network (fixtures recorded from sde_mc) they agree to BF16 noise: 2% on
the Brownian-integrand fixture, 6% on the two-network fixture (where the BF16
policy itself, restated on the CPU, is up to 4.3% off in relative norm).
"""
import math

import numpy as np
import pytest
import torch

import sde_mc_gb300 as sm
from sde_mc_gb300 import varred as V
from tests.cases import indep2d, merton1d
from tests.conftest import load_npz

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda", 0)


def _fixture():
    fx = load_npz("cv_mlp")
    n, S, d = fx["normals"].shape
    t = torch.from_numpy(fx["time"][..., 0])
    x = torch.from_numpy(fx["paths"])
    # the kernels read (n, S+1) time and (n, S+1, d) paths: append a column
    t_full = torch.cat([t, torch.ones(n, 1)], 1)
    x_full = torch.cat([x, x[:, -1:]], 1)
    data = V.CvData(t_full, x_full, torch.from_numpy(fx["normals"]), torch.from_numpy(fx["payoffs"]), DEV)
    params = [fx["p0_%d" % i] for i in range(8)]
    return fx, data, params


def _net(d, params=None, seed=0):
    torch.manual_seed(seed)
    f = sm.Mlp(d + 1, [64, 64, 64], d, batch_norm=False, batch_norm_init=False)
    if params is not None:
        f.load_flat_params(torch.cat([torch.from_numpy(p).reshape(-1) for p in params]))
    return f


def test_forward_matches_oracle_and_reference(oracle_mod):
    fx, data, params = _fixture()
    n, S, d = fx["normals"].shape
    cv = V.GpuCv(_net(d, params), d, DEV)
    fout = torch.empty((n, S, d), dtype=torch.float32, device=DEV)
    gamma = cv.forward(data, float(fx["r"]), fout=fout)
    fo = fout.cpu().numpy().reshape(n * S, d)
    mixed, _ = oracle_mod.mlp_forward_mixed(params, fx["time"].reshape(-1), fx["paths"].reshape(-1, d))
    big = np.abs(mixed).max()
    assert np.abs(fo - mixed).max() <= 1e-3 * big
    assert np.abs(fo - fx["f_out"]).max() <= 2e-2 * np.abs(fx["f_out"]).max()
    gm, fom = oracle_mod.cv_gamma_mixed(params, fx["time"][..., 0], fx["paths"], fx["normals"], fx["payoffs"],
                                        float(fx["r"]))
    scale = np.abs(fx["normals"] * fom).sum((1, 2))
    g = gamma.cpu().numpy().astype(np.float64)
    assert (np.abs(g - gm) <= 1e-3 * scale + 1e-6).all()
    assert (np.abs(g - fx["gamma"]) <= 1e-2 * scale + 1e-6).all()


def test_backward_matches_oracle_and_reference(oracle_mod):
    fx, data, params = _fixture()
    n, S, d = fx["normals"].shape
    cv = V.GpuCv(_net(d, params), d, DEV)
    gamma = torch.from_numpy(fx["gamma"]).to(DEV)
    grad = cv.backward(data, float(fx["r"]), gamma).cpu().numpy()
    mixed = oracle_mod.cv_grads_mixed(params, fx["time"][..., 0], fx["paths"], fx["normals"], fx["gamma"],
                                      float(fx["r"]))
    off = 0
    for i in range(8):
        m = mixed[i].reshape(-1)
        g = grad[off:off + m.size]
        off += m.size
        assert np.linalg.norm(g - m) <= 3e-3 * np.linalg.norm(m) + 1e-9, ("oracle", i)
        ref = fx["grad_%d" % i].reshape(-1)
        assert np.linalg.norm(g - ref) <= 2e-2 * np.linalg.norm(ref) + 1e-9, ("reference", i)
    assert off == grad.size
    # deterministic: a second call gives the same bits
    grad2 = cv.backward(data, float(fx["r"]), gamma).cpu().numpy()
    np.testing.assert_array_equal(grad, grad2)


def test_adam_step_matches_reference():
    fx, data, params = _fixture()
    d = fx["normals"].shape[2]
    cv = V.GpuCv(_net(d, params), d, DEV)
    cv.grad.copy_(torch.cat([torch.from_numpy(fx["grad_%d" % i]).reshape(-1) for i in range(8)]).to(DEV))
    cv.adam(lr=1e-3)
    new = cv.params.cpu().numpy()
    ref = np.concatenate([fx["p1_%d" % i].reshape(-1) for i in range(8)])
    np.testing.assert_allclose(new, ref, rtol=1e-6, atol=1e-7)


def test_one_dimensional_network_and_index_gather(oracle_mod):
    """d = 1 network on materialised Merton paths; a gather through an index
    equals the forward on the gathered rows."""
    solver, payoff, disc = merton1d(24, seed=7)
    dl = sm.simulate_adapted_data(512, solver, payoff, disc, bs=512, inference=True)
    data = V.CvData.from_dataset(dl.dataset, solver, DEV)
    f = _net(1, seed=3)
    cv = V.GpuCv(f, 1, DEV)
    fout = torch.empty((data.n, data.steps, 1), dtype=torch.float32, device=DEV)
    gamma = cv.forward(data, 0.02, fout=fout)
    params = [p.detach().numpy() for lin in f.linears() for p in (lin.weight, lin.bias)]
    S = data.steps
    tt = data.time[:, :S].cpu().numpy()
    xx = data.paths[:, :S].cpu().numpy()
    gm, fom = oracle_mod.cv_gamma_mixed(params, tt, xx, data.normals.cpu().numpy(), data.payoffs.cpu().numpy(), 0.02)
    assert np.abs(fout.cpu().numpy() - fom).max() <= 1e-3 * np.abs(fom).max()
    scale = np.abs(data.normals.cpu().numpy() * fom).sum((1, 2))
    assert (np.abs(gamma.cpu().numpy() - gm) <= 1e-3 * scale + 1e-6).all()
    idx = torch.randperm(data.n, device=DEV)[:100]
    g_idx = cv.forward(data, 0.02, idx=idx)
    torch.testing.assert_close(g_idx, gamma[idx], rtol=0, atol=0)
    # backward through the index equals backward on the gathered dataset
    sub = V.CvData(data.time[idx], data.paths[idx], data.normals[idx], data.payoffs[idx], DEV)
    g1 = cv.backward(data, 0.02, g_idx, idx=idx).clone()
    g2 = cv.backward(sub, 0.02, g_idx).clone()
    torch.testing.assert_close(g1, g2, rtol=0, atol=0)


def test_training_reduces_variance_without_bias():
    """The learned-CV set-up at reduced size: the rainbow on two assets with
    independent per-asset jumps.  Train on paths the solver generates, then
    price fresh paths with and without the control variate: the variance
    falls and the two means agree within 3 standard errors."""
    solver, payoff, disc = indep2d(32, seed=11)
    f = _net(2, seed=5)
    opt = torch.optim.Adam(f.parameters(), lr=1e-3)
    dl = sm.simulate_adapted_data(1 << 16, solver, payoff, disc, bs=1024)
    losses = sm.train_adapted_control_variates([f, sm.ZeroFunction(2)], opt, dl, solver, disc, epochs=4,
                                               print_losses=False)
    assert losses[-1] < losses[0]
    # the trained weights were written back to the torch module
    assert torch.equal(f.flat_params(DEV), f._sdemc_gpu.params)
    solver.seed = 99
    st_cv = sm.mc_apply_cvs([f, sm.ZeroFunction(2)], solver, 1 << 16, payoff, disc, sim_bs=1 << 15, bs=1024)
    st_plain = sm.mc_simple(1 << 16, solver, payoff, disc, bs=1 << 16, payoff_time='adapted')
    vrf = (st_plain.sample_std / st_cv.sample_std) ** 2
    assert vrf > 2.0, vrf
    assert abs(st_cv.sample_mean - st_plain.sample_mean) < 3 * math.hypot(st_cv.sample_std, st_plain.sample_std)


@pytest.mark.parametrize("jumps", [False, True])
def test_graph_epochs_equal_step_by_step_training(monkeypatch, jumps):
    """Epochs replayed from a captured CUDA graph (Adam's bias corrections
    read from a device table) give the bits of the step-by-step epochs:
    losses, weights and Adam moments, for f alone and for f and g."""
    from tests.cases import merton2d_corr
    solver, payoff, disc = merton2d_corr(32, seed=13) if jumps else indep2d(32, seed=11)
    dl = sm.simulate_adapted_data(1 << 14, solver, payoff, disc, bs=1024)
    runs = []
    for graph in (False, True):
        monkeypatch.setattr(V, "TRAIN_GRAPH", graph)
        f = _net(2, seed=5)
        g = _net(2, seed=7) if jumps else sm.ZeroFunction(2)
        params = list(f.parameters()) + (list(g.parameters()) if jumps else [])
        opt = torch.optim.Adam(params, lr=1e-3)
        torch.manual_seed(123)
        losses = sm.train_adapted_control_variates([f, g], opt, dl, solver, disc, epochs=3, print_losses=False)
        nets = [f] + ([g] if jumps else [])
        runs.append((losses, [torch.cat([n._sdemc_gpu.params, n._sdemc_gpu.m, n._sdemc_gpu.v]).cpu() for n in nets],
                     [n._sdemc_gpu.step_count for n in nets]))
    assert runs[0][0] == runs[1][0]
    assert runs[0][2] == runs[1][2] == [3 * (1 << 14) // 1024] * len(runs[0][2])
    for a, b in zip(runs[0][1], runs[1][1]):
        assert torch.equal(a, b)


def test_unsupported_models_raise():
    solver, payoff, disc = indep2d(8)
    dl = sm.simulate_adapted_data(64, solver, payoff, disc, bs=64, inference=True)
    g = sm.Mlp(3, [64, 64, 64], 2)  # batch norm: no kernel
    with pytest.raises(NotImplementedError):
        sm.apply_adapted_control_variates([_net(2), g], dl, solver, disc)
    with pytest.raises(NotImplementedError):
        sm.apply_adapted_control_variates([sm.Mlp(3, [32, 32], 2, batch_norm=False, batch_norm_init=False),
                                           sm.ZeroFunction(2)], dl, solver, disc)


def _jump_fixture():
    fx = load_npz("cv_mlp_jumps")
    n, S, d = fx["normals"].shape
    t = torch.from_numpy(fx["time"][..., 0])
    t_full = torch.cat([t, torch.ones(n, 1)], 1)

    def pad(a):
        a = torch.from_numpy(a)
        return torch.cat([a, a[:, -1:]], 1)
    from oracle import oracle
    mult = oracle.cv_jump_multipliers(fx["time"][..., 0], fx["jumps"], fx["lam_kappa"]).astype(np.float32)
    data_f = V.CvData(t_full, pad(fx["paths"]), torch.from_numpy(fx["normals"]), torch.from_numpy(fx["payoffs"]), DEV)
    data_g = V.CvData(t_full, pad(fx["left"]), torch.from_numpy(mult), torch.zeros(n), DEV)
    pf = [fx["p0f_%d" % i] for i in range(8)]
    pg = [fx["p0g_%d" % i] for i in range(8)]
    return fx, data_f, data_g, pf, pg, mult


def test_jump_integrand_matches_reference(oracle_mod):
    """f and g together (two kernel passes, one Gamma): the sums, the loss and
    both networks' gradients agree with the reference's own apply/train run
    within BF16 noise, and with the oracle's precision-policy restatement to
    accumulation noise."""
    fx, data_f, data_g, pf, pg, mult = _jump_fixture()
    r = float(fx["r"])
    cf = V.GpuCv(_net(2, pf), 2, DEV)
    cg = V.GpuCv(_net(2, pg), 2, DEV)
    gamma = V.gamma_gpu([cf, cg], [data_f, data_g], r)
    g64 = gamma.double()
    assert float(g64.sum()) == pytest.approx(float(fx["sum"]), rel=2e-3)
    assert float(g64.var()) == pytest.approx(float(fx["loss"]), rel=2e-2)
    grad_f = cf.backward(data_f, r, gamma).cpu().numpy()
    grad_g = cg.backward(data_g, r, gamma).cpu().numpy()
    t = fx["time"][..., 0]
    gm = gamma.cpu().numpy().astype(np.float64)
    mixed_f = oracle_mod.cv_grads_mixed(pf, t, fx["paths"], fx["normals"], gm, r)
    mixed_g = oracle_mod.cv_grads_mixed(pg, t, fx["left"], mult, gm, r)
    for name, grad, mixed in (("f", grad_f, mixed_f), ("g", grad_g, mixed_g)):
        off = 0
        for i in range(8):
            m = mixed[i].reshape(-1)
            gi = grad[off:off + m.size]
            off += m.size
            assert np.linalg.norm(gi - m) <= 3e-3 * np.linalg.norm(m) + 1e-9, ("oracle", name, i)
            ref = fx["grad%s_%d" % (name, i)].reshape(-1)
            # the BF16 policy itself (oracle restatement) is up to 4.3% off the
            # reference's FP32 gradients of f's first layers on this fixture
            assert np.linalg.norm(gi - ref) <= 6e-2 * np.linalg.norm(ref) + 1e-9, ("reference", name, i)


def test_training_with_jump_integrand():
    """Merton 2D with common jumps: training f and g through the reference's
    API on solver paths lowers the loss, and the estimate on fresh paths
    agrees with the plain estimator within 3 standard errors."""
    from tests.cases import merton2d_corr
    solver, payoff, disc = merton2d_corr(32, seed=13)
    f, g = _net(2, seed=6), _net(2, seed=7)
    opt = torch.optim.Adam(list(f.parameters()) + list(g.parameters()), lr=1e-3)
    dl = sm.simulate_adapted_data(1 << 15, solver, payoff, disc, bs=1024)
    losses = sm.train_adapted_control_variates([f, g], opt, dl, solver, disc, epochs=4, print_losses=False)
    assert losses[-1] < losses[0]
    assert torch.equal(g.flat_params(DEV), g._sdemc_gpu.params)
    st_cv = sm.mc_apply_cvs([f, g], solver, 1 << 15, payoff, disc, sim_bs=1 << 15, bs=1024)
    st_plain = sm.mc_simple(1 << 16, solver, payoff, disc, bs=1 << 16, payoff_time='adapted')
    assert st_cv.sample_std < st_plain.sample_std * math.sqrt(2)
    assert abs(st_cv.sample_mean - st_plain.sample_mean) < 3 * math.hypot(st_cv.sample_std, st_plain.sample_std)


def test_mc_adaptive_cv_trains_coarse_and_prices_fine(oracle_mod):
    """mc_adaptive_cv (sde_mc/mc.py:245-326): trains the integrand network on a
    coarse grid, prices fresh paths on the fine grid with the control variate,
    and returns MCStatistics of the fine run; its mean agrees with the plain
    estimator on the same grid within 3 standard errors and with the Merton
    series within 3 standard errors plus the Euler bias."""
    solver, payoff, disc = merton1d(64, seed=21)
    f = _net(1, seed=3)
    opt = torch.optim.Adam(f.parameters(), lr=1e-3)
    st = sm.mc_adaptive_cv([f, sm.ZeroFunction(1)], opt, solver, (1 << 15, 1 << 17), (16, 64), payoff, disc,
                           sim_bs=(1 << 15, 1 << 17), bs=(1024, 1024), epochs=3, print_losses=False)
    assert isinstance(st, sm.MCStatistics)
    assert st.num_trials == 1 << 17 and solver.num_steps == 64
    assert st.time_elapsed > 0 and st.sample_std > 0
    solver.seed = 5
    plain = sm.mc_simple(1 << 21, solver, payoff, disc, bs=1 << 21, payoff_time='adapted')
    assert abs(st.sample_mean - plain.sample_mean) < 3 * math.hypot(st.sample_std, plain.sample_std)
    # the network pays: the control-variate run's standard error beats the
    # plain estimator's at the same path count
    assert st.sample_std < plain.sample_std * math.sqrt((1 << 21) / (1 << 17))
    exact = oracle_mod.merton_call(1.0, 1.0, 1.0, 0.02, 0.2, -0.1, 0.2, 2.0)
    assert abs(st.sample_mean - exact) < 3 * st.sample_std + 3e-4


def test_run_cv_mc_sizes_the_run_for_the_tolerance(oracle_mod):
    """run_cv_mc (sde_mc/mc.py:443-467) on the MertonEuroCall preset: trains on
    a grid step_factor times coarser, restores the step count, sizes the run
    from a control-variate pilot for a 95% half-width eps (a multiple of
    nn_bs), and returns (MCStatistics, train time, test time)."""
    problem = sm.MertonEuroCall.default_params(48, 'cuda')
    f = _net(1, seed=8)
    opt = torch.optim.Adam(f.parameters(), lr=1e-3)
    eps = 2e-3
    st, train_t, test_t = sm.run_cv_mc(problem, [f, sm.ZeroFunction(1)], opt, eps, 1 << 15, step_factor=4,
                                       sim_bs=1 << 16, train_bs=1024, nn_bs=1024, epochs=3, print_losses=False,
                                       init_trials=1 << 15)
    assert isinstance(st, sm.MCStatistics) and train_t > 0 and test_t > 0
    assert problem.solver.num_steps == 48
    assert st.num_trials % 1024 == 0
    assert 1.96 * st.sample_std <= eps * 1.15
    plain = sm.mc_simple(1 << 22, problem.solver, problem.payoff, problem.discounter, bs=1 << 22,
                         payoff_time='adapted')
    assert abs(st.sample_mean - plain.sample_mean) < 3 * math.hypot(st.sample_std, plain.sample_std)
    exact = oracle_mod.merton_call(1.0, 1.0, 3.0, 0.02, 0.2, -0.05, 0.3, 1.0)
    assert abs(st.sample_mean - exact) < 3 * st.sample_std + 5e-3
