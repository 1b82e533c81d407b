"""K11, the FP64 reference run: on the same paths as the FP32 pricer (same
Philox words) the two means differ by far less than the statistical error,
and the FP64 mean agrees with the closed forms."""
import math

import pytest

from sde_mc_gb300 import kernels as K
from sde_mc_gb300.lowering import lower
from tests.cases import basket, gbm_uniform, heston, indep2d, inst_for, levy2d, merton1d

pytestmark = pytest.mark.gpu


def _pair(case, n, seed=5, offset=0):
    inst = inst_for(case, num_paths=n, seed=seed, path_offset=offset)
    f32 = K.price(inst).cpu().tolist()
    f64 = K.price_f64(inst).cpu().tolist()
    assert f32[5] == 0 and f64[5] == 0 and f64[2] == n
    return f32, f64


@pytest.mark.parametrize("factory", [lambda: merton1d(100), lambda: indep2d(64), lambda: basket(8, 32),
                                     lambda: gbm_uniform(12), lambda: heston(24)])
def test_fp32_and_fp64_agree_on_the_same_paths(factory):
    f32, f64 = _pair(factory(), 1 << 18)
    se = math.sqrt(f64[4] / f64[2])
    # FP32 rounding and the float32 grid's isclose test move the mean by a
    # few 1e-6 relative; the statistical error at 2^18 paths is ~1e-3
    assert abs(f32[3] - f64[3]) < 0.02 * se, (f32[3], f64[3], se)
    assert f32[4] == pytest.approx(f64[4], rel=1e-3)


def test_fp64_merton_matches_series(oracle_mod):
    f32, f64 = _pair(merton1d(100), 1 << 22)
    se = math.sqrt(f64[4] / f64[2])
    exact = oracle_mod.merton_call(1.0, 1.0, 1.0, 0.02, 0.2, -0.1, 0.2, 2.0)
    assert abs(f64[3] - exact) < 4 * se, (f64[3], exact, se)


def test_fp64_heston_and_gbm_match_closed_forms(oracle_mod):
    _, f64 = _pair(heston(256), 1 << 22)
    se = math.sqrt(f64[4] / f64[2])
    exact = oracle_mod.heston_call(1.0, 0.04, 1.0, 1.0, 0.02, 2.0, 0.04, 0.3, -0.7)
    assert abs(f64[3] - exact) < 4 * se + 0.04 / 256, (f64[3], exact, se)
    _, g64 = _pair(gbm_uniform(64), 1 << 22)
    se = math.sqrt(g64[4] / g64[2])
    exact = oracle_mod.bs_call(1.0, 1.0, 1.0, 0.02, 0.2)
    assert abs(g64[3] - exact) < 4 * se + 0.02 / 64, (g64[3], exact, se)


def test_fp64_is_deterministic_and_rejects_unsupported():
    inst = inst_for(indep2d(32), num_paths=100_003, seed=9)
    a = K.price_f64(inst).cpu().tolist()
    b = K.price_f64(inst).cpu().tolist()
    assert a == b
    with pytest.raises(Exception):
        K.price_f64(inst_for(levy2d(8), num_paths=64))


def test_fp64_empty_and_ragged_sizes():
    for n in (0, 1, 31, 33, 1000):
        inst = inst_for(merton1d(10), num_paths=n, seed=4)
        a = K.price(inst).cpu().tolist()
        b = K.price_f64(inst).cpu().tolist()
        assert b[5] == 0 and b[2] == n == a[2]
        if n > 1:
            assert abs(a[3] - b[3]) <= 1e-4 * abs(b[3]) + 1e-7
