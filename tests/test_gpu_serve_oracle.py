"""The served control variate against the oracle (the headline estimator).

Three layers, each through the C ABI:
  1. path by path: the server kernels' per-path code (sdemc_serve_cv_paths)
     exports its draws and the integrand weights of every 4-step block; the
     oracle re-runs each path from those draws and, with the same weights,
     gives the same payoff and the same 2d + 1 regressors bit for bit; every
     weight the GPU evaluated agrees with the oracle's evaluation at the same
     state within the propagated error bound of CUDA's intrinsics;
  2. independently: the oracle's own weights give regressors that agree with
     the GPU's to single-precision accuracy;
  3. the request: a pricing server run of the same request gives the pilot
     mean and standard error, the control-variate coefficients, the
     variance-reduction factor, the main-run size and the final mean and
     standard error that the oracle's restatement of the server (pilot sums
     in the kernels' reduction order, slice accumulation, the regression and
     find_num_trials, sde_mc/mc.py:418-427) computes from the per-path values,
     bit for bit.
Cases: d = 1, 2, 3, 6, 8; common and per-asset jumps; call, put, digital,
rainbow, basket and best-of payoffs; a pilot that is not a whole number of
32-path chunks; slices small enough that each phase spans several."""
import numpy as np
import pytest

from oracle import oracle
from sde_mc_gb300 import kernels as K
from sde_mc_gb300 import serve
from tests.cases import inst_for, served_cv_cases

pytestmark = pytest.mark.gpu

CASES = served_cv_cases()
SLICE_WORK = 1 << 18
PILOT = {"call1d": 4096 + 17, "put1d": 1 << 13, "digital1d": 1 << 13}


def _inst(name, n=None):
    return inst_for(CASES[name], num_paths=n or PILOT.get(name, 1 << 12), seed=11, path_offset=0)


def _caps(inst):
    S = int(inst.num_steps) + 64
    return S, 64, S // 4 + 2


@pytest.mark.parametrize("name", sorted(CASES))
def test_paths_and_regressors_match_the_oracle(name):
    inst = _inst(name, 1500)
    S, jcap, wcap = _caps(inst)
    g = {k: v.cpu().numpy() for k, v in K.serve_cv_paths(inst, steps_cap=S, jcap=jcap, wcap=wcap).items()}
    assert int(g["status"][0]) == 0
    cw = oracle.serve_cv_weights(inst)
    assert bytes(cw) == bytes(K.serve_cv_weights(inst))
    pay, reg, rc, ws = oracle.serve_cv_from_export(inst, cw, g["z"], g["jt"], g["jm"], g["jsel"], g["wg"])
    assert rc == 0
    np.testing.assert_array_equal(pay, g["payoff"])
    np.testing.assert_array_equal(reg, g["reg"])
    # the GPU's weights vs the oracle's evaluation at the same block-start states
    assert ws[2] >= 1500
    assert ws[0] <= 1.0 and ws[1] <= 1.0, ws
    # the oracle's own weights: the regressors agree to single precision
    _, reg_o, rc, _ = oracle.serve_cv_from_export(inst, cw, g["z"], g["jt"], g["jm"], g["jsel"])
    assert rc == 0
    scale = np.abs(g["reg"]).max(axis=0) + 1e-30
    err = np.abs(reg_o - g["reg"]) / scale
    assert np.median(err) < 1e-6 and np.quantile(err, 0.999) < 1e-4, (np.median(err), err.max())


@pytest.mark.parametrize("name", sorted(CASES))
def test_served_request_equals_the_oracle_restatement(name):
    inst = _inst(name)
    rel = 3e-3
    with serve.Server(max_slots=4, mem_budget=1 << 30, slice_work=SLICE_WORK) as srv:
        srv.submit_inst(inst.copy(), rel, "linear_cv", tag=1)
        (r,) = srv.wait(1)
    r.raise_for_status()
    R = 2 * inst.dim + 1
    sl = oracle.serve_slice_paths(inst, SLICE_WORK)
    # pilot: the GPU's per-path values, the kernels' chunk rows, the slices
    p = K.serve_cv_paths(inst)
    pv, y = p["payoff"].cpu().numpy(), p["reg"].cpu().numpy()
    fit = oracle.serve_fit(oracle.serve_slices(oracle.serve_rows(pv, y), sl), R, rel)
    assert r.pilot_paths == inst.num_paths
    assert r.pilot_mean == fit["pilot_mean"] and r.pilot_se == fit["pilot_se"]
    assert r.estimator == fit["est"] and r.vrf == fit["vrf"]
    np.testing.assert_array_equal(np.asarray(r.beta, np.float32), fit["beta"])
    assert r.main_paths == fit["main_paths"]
    if name != "digital1d":
        assert r.estimator == serve.EST_LINEAR_CV and r.vrf > 1.5
    # main run: fresh paths after the pilot's, P - beta . r (P alone without the CV)
    m = inst.copy()
    m.path_offset = inst.path_offset + inst.num_paths
    m.num_paths = r.main_paths
    q = K.serve_cv_paths(m)
    rows = oracle.serve_rows(q["payoff"].cpu().numpy(), q["reg"].cpu().numpy(), beta=np.asarray(r.beta, np.float32))
    mean, se = oracle.serve_main(oracle.serve_slices(rows, sl))
    assert r.mean == mean and r.se == se
    assert max(inst.num_paths, r.main_paths) > sl  # a phase spanning several slices
