"""K5 on tcgen05 (tensor-memory accumulators) against the mma.sync kernel and
the oracle's precision-policy restatement: both round the same BF16
operands, so Gamma agrees to accumulation-order noise."""
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
