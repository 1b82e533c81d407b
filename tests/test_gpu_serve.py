"""Pricing server (K9): results equal the single-instance kernels on the same
paths, are bit-identical alone and in a mix, the linear control variate is
unbiased and cuts the variance, and admission respects the memory budget."""
import math

import numpy as np
import pytest
import torch

from sde_mc_gb300 import kernels as K
from sde_mc_gb300 import serve, workloads
from sde_mc_gb300.lowering import lower

pytestmark = pytest.mark.gpu


def _req(idx, rng_seed=0):
    rng = np.random.default_rng(rng_seed + 1000 * idx)
    return workloads.basket_instance(idx, *workloads.draw_basket_params(rng))


def _submit(srv, m, rel, est, tag=None, pilot=None):
    return srv.submit(m.solver, m.payoff, m.discounter, rel_target=rel, pilot_paths=pilot or m.paths,
                      estimator=est, tag=m.idx if tag is None else tag, stream_id=m.idx)


def test_plain_request_equals_k1_on_the_same_paths():
    m = workloads.basket_instance(3, 2, 64, 4096 + 17, 1.0, [0.2, 0.3], 1.0)
    with serve.Server(max_slots=8, mem_budget=1 << 30) as srv:
        _submit(srv, m, 1e-2, "plain")
        (r,) = srv.wait(1)
    r.raise_for_status()
    assert r.estimator == serve.EST_PLAIN and r.pilot_paths == 4096 + 17
    pilot = K.price(lower(m.solver, m.payoff, m.discounter, num_paths=r.pilot_paths, path_offset=0,
                          stream_id=m.idx)).cpu().tolist()
    assert r.pilot_mean == pytest.approx(pilot[3], rel=1e-12)
    assert r.pilot_se == pytest.approx(math.sqrt(pilot[4] / pilot[2]), rel=1e-9)
    # find_num_trials: ceil((1.96 * se / eps)^2 * n0) with eps = rel * |price|
    eps = 1e-2 * abs(pilot[3])
    assert r.main_paths == max(64, math.ceil(1.96 ** 2 * pilot[4] / eps ** 2))
    main = K.price(lower(m.solver, m.payoff, m.discounter, num_paths=r.main_paths, path_offset=r.pilot_paths,
                         stream_id=m.idx)).cpu().tolist()
    assert r.mean == pytest.approx(main[3], rel=1e-12)
    assert r.se == pytest.approx(math.sqrt(main[4] / main[2]), rel=1e-9)
    assert r.t_arrive_ns <= r.t_admit_ns <= r.t_done_ns


def test_result_is_the_same_alone_and_in_a_mix():
    probes = [_req(i) for i in (1, 2, 3)]
    alone = {}
    with serve.Server(max_slots=16, mem_budget=2 << 30) as srv:
        for m in probes:
            _submit(srv, m, 3e-3, "linear_cv")
            (r,) = srv.wait(1)
            alone[r.tag] = r.raise_for_status().key()
    mix = [_req(i) for i in range(4, 40)]
    with serve.Server(max_slots=64, mem_budget=4 << 30, tick_work=1 << 30, side_streams=4) as srv:
        order = mix[:10] + probes[:1] + mix[10:25] + probes[1:] + mix[25:]
        for m in order:
            if m in probes:
                _submit(srv, m, 3e-3, "linear_cv")
            else:
                _submit(srv, m, 1e-2 if m.idx % 2 else 3e-3, "linear_cv" if m.idx % 3 else "plain")
        res = {r.tag: r for r in srv.wait(len(order))}
        st = srv.stats()
    for m in probes:
        assert res[m.idx].key() == alone[m.idx], m.idx
    assert st["completed"] == len(order) and st["active"] == 0 and st["pending"] == 0
    assert st["ticks"] > 1 and st["busy_s"] > 0


def test_requests_of_one_seed_and_of_several_give_the_same_bits():
    """A d = 5 or 6 control-variate class whose requests share a seed takes the
    Philox round keys as launch constants; with requests of other seeds in the
    class it derives them per chunk.  A request's result is the same either
    way."""
    probes = [workloads.basket_instance(i, d, 48, 4096 + 33 * i, 1.0, [0.2 + 0.02 * j for j in range(d)], 1.0)
              for i, d in ((1, 5), (2, 6))]
    # small slices (the same in both servers: slices are a function of the
    # request and the slice size) spread every phase over several ticks, so
    # the probes' slices share class kernels with requests of other seeds
    slice_work = 1 << 18
    alone = {}
    with serve.Server(max_slots=8, mem_budget=1 << 30, slice_work=slice_work) as srv:
        for m in probes:
            _submit(srv, m, 3e-3, "linear_cv")
            (r,) = srv.wait(1)
            alone[r.tag] = r.raise_for_status().key()
    others = [workloads.basket_instance(10 + k, 5 + k % 2, 48, 4096, 1.05, [0.25] * (5 + k % 2), 1.5, seed=1000 + k)
              for k in range(6)]
    with serve.Server(max_slots=16, mem_budget=2 << 30, slice_work=slice_work) as srv:
        for m in others + probes:
            _submit(srv, m, 3e-3, "linear_cv")
        res = {r.tag: r for r in srv.wait(len(probes) + len(others))}
    for m in probes:
        assert res[m.idx].key() == alone[m.idx], m.idx
    assert all(res[m.idx].status == 0 for m in others)


def test_linear_cv_is_unbiased_and_reduces_variance():
    m = workloads.basket_instance(11, 2, 128, 1 << 14, 1.0, [0.2, 0.3], 1.0)
    with serve.Server(max_slots=4, mem_budget=1 << 30) as srv:
        _submit(srv, m, 2e-3, "plain", tag=1)
        _submit(srv, m, 2e-3, "linear_cv", tag=2)
        res = {r.tag: r.raise_for_status() for r in srv.wait(2)}
    plain, cv = res[1], res[2]
    assert cv.estimator == serve.EST_LINEAR_CV and cv.vrf > 3.0
    # the same pilot paths, so the same pilot estimate
    assert cv.pilot_mean == pytest.approx(plain.pilot_mean, rel=1e-12)
    assert cv.main_paths < plain.main_paths
    # both reach the target, and agree within 3 standard errors
    for r in (plain, cv):
        assert 1.96 * r.se <= 2e-3 * abs(r.mean) * 1.15
    assert abs(cv.mean - plain.mean) < 3 * math.hypot(cv.se, plain.se)
    # the realised variance ratio is close to the pilot's estimate
    realised = (plain.se ** 2 * plain.main_paths) / (cv.se ** 2 * cv.main_paths)
    assert realised == pytest.approx(cv.vrf, rel=0.3)


def test_memory_budget_limits_admission():
    reqs = [_req(i, rng_seed=5) for i in range(12)]
    with serve.Server(max_slots=64, mem_budget=1 << 30) as srv:
        fixed = srv.stats()["mem_in_use"]  # slot table and tick buffers of 64 slots
    # room for the chunk partials of one full slice in every tick buffer plus
    # the request state of only a few requests at a time
    budget = fixed + (64 << 20)
    with serve.Server(max_slots=64, mem_budget=budget, side_streams=0) as srv:
        for m in reqs:
            _submit(srv, m, 1e-2, "linear_cv")
        res = srv.wait(len(reqs))
        st = srv.stats()
    assert all(r.status == 0 for r in res)
    assert fixed < st["mem_peak"] <= budget
    assert st["completed"] == st["admitted"] == len(reqs)


def test_invalid_requests_are_refused():
    m = _req(0)
    with serve.Server(max_slots=4, mem_budget=1 << 30) as srv:
        with pytest.raises(ValueError):
            srv.submit(m.solver, m.payoff, m.discounter, rel_target=0.0, pilot_paths=1024)
        with pytest.raises(ValueError):
            srv.submit(m.solver, m.payoff, m.discounter, rel_target=1e-2, pilot_paths=1)
        assert srv.poll() == []


def _case(name):
    import sde_mc_gb300 as sm
    if name == "rainbow2d_indep_jumps":
        solver, payoff, disc = workloads.rainbow2d(64)
        return solver, payoff, disc
    if name == "basket6":
        m = workloads.basket_instance(0, 6, 48, 1, 1.05, [0.15, 0.2, 0.25, 0.3, 0.35, 0.4], 2.0)
        return m.solver, m.payoff, m.discounter
    if name == "put1d":
        m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
        return sm.JumpEulerSolver(m, 1.0, 50), sm.EuroPut(1.0), sm.ConstantShortRate(0.02)
    if name == "digital1d":
        m = sm.Merton(0.02, 0.2, 2.0, -0.1, 0.2, torch.tensor([1.]), dim=1)
        return sm.JumpEulerSolver(m, 1.0, 50), sm.Digital(1.0), sm.ConstantShortRate(0.02)
    raise KeyError(name)


@pytest.mark.parametrize("name", ["rainbow2d_indep_jumps", "basket6", "put1d", "digital1d"])
def test_control_variate_has_zero_mean(name):
    """The control variate's regressors are martingale integrals, so the
    served CV estimate agrees with a large plain run within 3 standard errors
    for per-asset jumps, common jumps, puts and unweighted payoffs."""
    solver, payoff, disc = _case(name)
    with serve.Server(max_slots=4, mem_budget=1 << 30) as srv:
        srv.submit(solver, payoff, disc, rel_target=2e-3, pilot_paths=1 << 14, estimator="linear_cv", tag=1,
                   stream_id=77)
        (r,) = srv.wait(1)
    r.raise_for_status()
    ref = K.price(lower(solver, payoff, disc, num_paths=1 << 23, path_offset=1 << 30, stream_id=78)).cpu().tolist()
    se_ref = math.sqrt(ref[4] / ref[2])
    assert abs(r.mean - ref[3]) < 3 * math.hypot(r.se, se_ref), (r, ref[3], se_ref)
    if name != "digital1d":
        assert r.estimator == serve.EST_LINEAR_CV and r.vrf > 2.0, r
