"""Host-side checks of the served control variate's restatement: the
library's weight derivation equals the oracle's bit for bit (no GPU call:
sdemc_serve_cv_weights is host code), and the oracle's restated regression
recovers known coefficients."""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from sde_mc_gb300 import _native as N
from tests.cases import inst_for, served_cv_cases


@pytest.mark.parametrize("name", sorted(served_cv_cases()))
def test_library_weights_equal_the_oracle(name):
    inst = inst_for(served_cv_cases()[name], num_paths=1024)
    lib = N.load()
    cw = N.SdemcCvWeights()
    assert lib.sdemc_serve_cv_weights(ctypes.byref(inst), ctypes.byref(cw)) == N.OK
    ref = oracle.serve_cv_weights(inst)
    assert ctypes.sizeof(cw) == ctypes.sizeof(ref)
    assert ctypes.string_at(ctypes.byref(cw), ctypes.sizeof(cw)) == ctypes.string_at(ctypes.byref(ref),
                                                                                   ctypes.sizeof(ref))
    d = inst.dim
    jumps = inst.rate > 0
    assert cw.jumps == int(jumps)
    if jumps:
        assert all(cw.comp[i] != 0 and cw.inv_comp[i] == np.float32(1.0 / np.float64(cw.comp[i])) for i in range(d))
    assert cw.wkind == {"put1d": 2, "digital1d": 0}.get(name, 1)


def test_weights_reject_a_bad_descriptor():
    inst = inst_for(served_cv_cases()["call1d"], num_paths=16)
    inst.dim = 0
    assert N.load().sdemc_serve_cv_weights(ctypes.byref(inst), ctypes.byref(N.SdemcCvWeights())) == N.EINVAL


def test_restated_regression_recovers_known_coefficients():
    """Payoffs P = 1 + 2 y0 - 0.5 y1 + small noise: the pilot rows, the
    slice accumulation and the regression give beta close to (2, -0.5, 0)."""
    rng = np.random.default_rng(3)
    n, R = 5000, 3
    y = rng.standard_normal((n, R)).astype(np.float32)
    pv = (1.0 + 2.0 * y[:, 0] - 0.5 * y[:, 1] + 0.01 * rng.standard_normal(n)).astype(np.float32)
    rows = oracle.serve_rows(pv, y)
    assert rows.shape == ((n + 31) // 32, 3 + 2 * R + R * (R + 1) // 2)
    acc = oracle.serve_slices(rows, 1024)
    assert acc[2] == n
    np.testing.assert_allclose(acc[0], pv.astype(np.float64).sum(), rtol=1e-5)
    fit = oracle.serve_fit(acc, R, rel_target=1e-2)
    assert fit["est"] == 1 and fit["vrf"] > 1000
    np.testing.assert_allclose(fit["beta"][:R], [2.0, -0.5, 0.0], atol=2e-3)
    # the main run's sums of P - beta . r: its mean is P's mean minus beta . mean(r)
    acc_m = oracle.serve_slices(oracle.serve_rows(pv, y, beta=fit["beta"]), 1024)
    mean, se = oracle.serve_main(acc_m)
    assert abs(mean - 1.0) < 5e-3 and se < 1e-3


def test_slice_sizes_follow_the_server_rule():
    inst = inst_for(served_cv_cases()["basket6"], num_paths=1024)
    cost = (inst.num_steps + inst.rate * inst.T) * inst.dim
    assert oracle.serve_slice_paths(inst, 1 << 20) == (int(np.ceil((1 << 20) / cost)) + 31) // 32 * 32
    assert oracle.serve_slice_paths(inst, 1 << 40) == 1 << 18
    assert oracle.serve_slice_paths(inst, 1) == 1 << 10
