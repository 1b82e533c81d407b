"""K7 (paths + payoff + learned control variate in one pass) against K1 and
against materialise + K5 on tcgen05: the same paths give the same bits."""
import math

import numpy as np
import pytest
import torch

import sde_mc_gb300 as sm
from sde_mc_gb300 import kernels as K
from sde_mc_gb300 import varred as V
from sde_mc_gb300.lowering import lower
from tests.cases import indep2d, merton1d
from tests.test_gpu_cv import DEV, _net

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("d", [1, 2])
def test_fused_cv_equals_materialised_tc_and_k1(d, oracle_mod):
    solver, payoff, disc = (merton1d(40, seed=21) if d == 1 else indep2d(40, seed=21))
    n = 5000 + 17
    f = _net(d, seed=4)
    cv = V.GpuCv(f, d, DEV)
    inst = lower(solver, payoff, disc, num_paths=n, path_offset=123)
    gam = torch.empty(n, dtype=torch.float32, device=DEV)
    out = K.price_cv(inst, cv.params, 0.02, gamma=gam).cpu().tolist()
    assert out[7] == 0 and out[2] == n
    # the plain sums are K1's, bit for bit
    k1 = K.price(inst).cpu().tolist()
    assert out[3] == k1[0] and out[4] == k1[1]
    # Gamma per path equals the tcgen05 forward on the materialised paths
    cap = solver.num_steps + solver.max_jumps
    m = K.materialise(inst, cap)
    total = int(m["steps"].max().item())
    data = V.CvData(m["time"][:, :total + 1], m["paths"][:, :total + 1], m["normals"][:, :total].contiguous(),
                    m["payoffs"], DEV)
    g_tc = cv.forward_tc(data, 0.02)
    assert int(cv._tc_status.item()) == 0
    torch.testing.assert_close(gam, g_tc, rtol=0, atol=0)
    # the Gamma sums: the oracle's restatement of the chunk reduction order
    ref = oracle_mod.chunk_reduce(gam.cpu().numpy())
    assert out[0] == ref[0] and out[1] == ref[1] and out[2] == ref[2]


def test_mc_apply_cvs_uses_the_fused_kernel():
    """mc_apply_cvs on a supported model prices with K7 and agrees with the
    materialised route on the same fresh paths."""
    solver, payoff, disc = indep2d(32, seed=31)
    f = _net(2, seed=8)
    models = [f, sm.ZeroFunction(2)]
    assert V.fused_supported(models, solver, disc)
    start = solver.path_cursor
    st = sm.mc_apply_cvs(models, solver, 1 << 15, payoff, disc, sim_bs=1 << 15, bs=1024)
    solver.path_cursor = start
    dl = sm.simulate_adapted_data(1 << 15, solver, payoff, disc, bs=1024, inference=True)
    s1, s2 = sm.apply_adapted_control_variates(models, dl, solver, disc)
    n = 1 << 15
    mean = float(s1) / n
    # same per-path Gamma; K7 sums 32-path chunks in FP32 before FP64
    assert st.sample_mean == pytest.approx(mean, rel=1e-8)
