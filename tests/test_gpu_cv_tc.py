"""K5 and K6 on tcgen05 (tensor-memory accumulators) against the mma.sync
kernels and the oracle's precision-policy restatement: both round the same
BF16 operands, so Gamma and the gradients agree to accumulation-order noise."""
import numpy as np
import pytest
import torch

import sde_mc_gb300 as sm
from sde_mc_gb300 import varred as V
from tests.cases import indep2d, merton1d
from tests.test_gpu_cv import DEV, _fixture, _net

pytestmark = pytest.mark.gpu


def test_tc_forward_matches_fixture_and_oracle(oracle_mod):
    fx, data, params = _fixture()
    n, S, d = fx["normals"].shape
    cv = V.GpuCv(_net(d, params), d, DEV)
    g_tc = cv.forward_tc(data, float(fx["r"]))
    assert int(cv._tc_status.item()) == 0
    g_mma = cv.forward(data, float(fx["r"]))
    gm, fom = oracle_mod.cv_gamma_mixed(params, fx["time"][..., 0], fx["paths"], fx["normals"], fx["payoffs"],
                                        float(fx["r"]))
    scale = np.abs(fx["normals"] * fom).sum((1, 2))
    g = g_tc.cpu().numpy().astype(np.float64)
    assert (np.abs(g - gm) <= 1e-3 * scale + 1e-6).all()
    assert (np.abs(g - g_mma.cpu().numpy()) <= 1e-3 * scale + 1e-6).all()


@pytest.mark.parametrize("d", [1, 2])
def test_tc_forward_large_batch_and_index(d):
    solver, payoff, disc = (merton1d(40, seed=4) if d == 1 else indep2d(40, seed=4))
    dl = sm.simulate_adapted_data(5000, solver, payoff, disc, bs=5000, inference=True)
    data = V.CvData.from_dataset(dl.dataset, solver, DEV)
    cv = V.GpuCv(_net(d, seed=9), d, DEV)
    g_tc = cv.forward_tc(data, 0.02)
    assert int(cv._tc_status.item()) == 0
    g_mma = cv.forward(data, 0.02)
    scale = (data.normals.abs().sum((1, 2)) * 0.2 + 1e-3)
    assert ((g_tc - g_mma).abs() <= 2e-3 * scale + 1e-5).all()
    idx = torch.randperm(data.n, device=DEV)[:777]
    g_idx = cv.forward_tc(data, 0.02, idx=idx)
    torch.testing.assert_close(g_idx, g_tc[idx], rtol=0, atol=0)


def _layer_norms(g, ref_layers):
    off, out = 0, []
    for m in ref_layers:
        m = np.asarray(m).reshape(-1)
        out.append((np.linalg.norm(g[off:off + m.size] - m), np.linalg.norm(m)))
        off += m.size
    assert off == g.size
    return out


def test_tc_backward_matches_oracle_and_mma(oracle_mod):
    fx, data, params = _fixture()
    n, S, d = fx["normals"].shape
    cv = V.GpuCv(_net(d, params), d, DEV)
    gamma = torch.from_numpy(fx["gamma"]).to(DEV)
    g_tc = cv.backward_tc(data, float(fx["r"]), gamma).cpu().numpy().copy()
    assert int(cv._bwd_status.item()) == 0
    g_mma = cv.backward(data, float(fx["r"]), gamma).cpu().numpy().copy()
    mixed = oracle_mod.cv_grads_mixed(params, fx["time"][..., 0], fx["paths"], fx["normals"], fx["gamma"],
                                      float(fx["r"]))
    for i, (e, m) in enumerate(_layer_norms(g_tc, mixed)):
        assert e <= 5e-3 * m + 1e-9, ("oracle", i, e / m)
    sizes = [np.asarray(m).size for m in mixed]
    split = np.split(g_mma, np.cumsum(sizes)[:-1])
    for i, (e, m) in enumerate(_layer_norms(g_tc, split)):
        assert e <= 5e-3 * m + 1e-9, ("mma.sync", i, e / m)
    g2 = cv.backward_tc(data, float(fx["r"]), gamma).cpu().numpy()
    np.testing.assert_array_equal(g_tc, g2)


@pytest.mark.parametrize("d", [1, 2])
def test_tc_backward_large_batch_and_index(d):
    solver, payoff, disc = (merton1d(40, seed=6) if d == 1 else indep2d(40, seed=6))
    dl = sm.simulate_adapted_data(20000, solver, payoff, disc, bs=20000, inference=True)
    data = V.CvData.from_dataset(dl.dataset, solver, DEV)
    cv = V.GpuCv(_net(d, seed=11), d, DEV)
    idx = torch.randperm(data.n, device=DEV)[:4096]
    gamma = cv.forward(data, 0.02, idx)
    g_tc = cv.backward_tc(data, 0.02, gamma, idx).cpu().numpy().copy()
    assert int(cv._bwd_status.item()) == 0
    g_mma = cv.backward(data, 0.02, gamma, idx).cpu().numpy().copy()
    # parameter layout: W1, b1, W2, b2, W3, b3, W4, b4
    IN, H = d + 1, 64
    sizes = [H * IN, H, H * H, H, H * H, H, d * H, d]
    parts = np.split(g_mma, np.cumsum(sizes)[:-1])
    for i, (e, m) in enumerate(_layer_norms(g_tc, parts)):
        assert e <= 5e-3 * m + 1e-9, (i, e / m)


def test_tc_backward_small_batches_match_mma():
    """Minibatches smaller than a 128-path group and step counts shorter than
    one 32-step range: padded rows contribute nothing."""
    fx, data, params = _fixture()
    n, S, d = fx["normals"].shape
    cv = V.GpuCv(_net(d, params), d, DEV)
    for m in (1, 3, 127, 129):
        idx = torch.arange(m, device=DEV) % n
        gamma = cv.forward(data, float(fx["r"]), idx)
        g_tc = cv.backward_tc(data, float(fx["r"]), gamma, idx).cpu().numpy().copy()
        assert int(cv._bwd_status.item()) == 0
        g_mma = cv.backward(data, float(fx["r"]), gamma, idx).cpu().numpy().copy()
        assert np.isfinite(g_tc).all()
        assert np.linalg.norm(g_tc - g_mma) <= 5e-3 * np.linalg.norm(g_mma) + 1e-9, m
