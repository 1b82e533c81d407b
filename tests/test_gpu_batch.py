"""K8 batched pricing: every instance of a heterogeneous batch gets the bits it
gets when priced alone (sdemc_price), whatever the launch shape, side
streams, or CUDA-graph replay; overflow is reported per instance."""
import numpy as np
import pytest
import torch

from sde_mc_gb300 import _native as N
from sde_mc_gb300 import batch as B
from sde_mc_gb300 import kernels as K
from sde_mc_gb300 import workloads
from tests.cases import basket, gbm_uniform, indep2d, inst_for, levy2d, merton1d

pytestmark = pytest.mark.gpu


def small_mix(n=40, scale=0.05):
    mix = workloads.basket_mix(n)
    for m in mix:  # keep the test quick: a few thousand paths each
        m.paths = max(1, int(m.paths * scale))
    return mix


def alone(insts):
    return np.stack([K.price(i).cpu().numpy() for i in insts])


def test_batch_equals_alone_bit_for_bit():
    insts = B.lower_mix(small_mix())
    ref = alone(insts)
    plan = B.BatchPlan(insts)
    got = plan.run().cpu().numpy()
    np.testing.assert_array_equal(got, ref)
    assert np.all(got[:, 5] == 0)


def test_batch_mixed_models_and_shapes():
    cases = [merton1d(50), indep2d(64), levy2d(16), gbm_uniform(12), basket(3, 32), basket(8, 16)]
    insts = []
    for k, c in enumerate(cases):
        for n in (1, 33, 1000):
            insts.append(inst_for(c, num_paths=n, seed=3 + k, path_offset=17 * n))
    ins0 = inst_for(merton1d(50), num_paths=0, seed=1)
    insts.append(ins0)
    ref = alone(insts)
    plan = B.BatchPlan(insts)
    for bt, ns in [(128, 0), (64, 3), (256, 8), (32, 1)]:
        plan.set_config(bt, ns)
        np.testing.assert_array_equal(plan.run().cpu().numpy(), ref)


def test_batch_class_with_one_seed_and_with_several():
    """A class whose instances share a seed takes the Philox round keys as
    launch constants, a class with several seeds derives them per instance:
    both give every instance the bits it gets alone."""
    same = [inst_for(merton1d(40), num_paths=n, seed=5, path_offset=3 * n) for n in (64, 1000, 4097)]
    mixed = [inst_for(merton1d(40), num_paths=n, seed=s, path_offset=0) for n, s in ((64, 5), (1000, 6), (4097, 2 ** 40 + 7))]
    for insts in (same, mixed):
        plan = B.BatchPlan(insts)
        np.testing.assert_array_equal(plan.run().cpu().numpy(), alone(insts))
        assert plan.header.n_class == 1


def test_batch_graph_replay_with_new_offsets():
    mix = small_mix(24)
    insts = B.lower_mix(mix)
    plan = B.BatchPlan(insts)
    plan.set_config(128, 4)
    plan.run()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.upload()
        plan.launch()
    for step in range(3):
        offs = [(step + 1) * 1_000_000 + 7 * i for i in range(len(insts))]
        plan.set_path_offsets(offs)
        g.replay()
        got = plan.out[:plan.n].cpu().numpy()
        ref = alone(B.lower_mix(mix, path_offsets=offs))
        np.testing.assert_array_equal(got, ref)


def test_batch_reports_overflow_per_instance():
    ok = inst_for(merton1d(50), num_paths=100, seed=1)
    bad = inst_for(merton1d(50), num_paths=100, seed=1)
    # gaps drawn at 5e7/yr while the iteration cap is sized for 5000/yr: every
    # path hits the cap, which must end the loop and flag this instance only
    bad.rate = 5000.0
    bad.inv_rate = 2e-8
    bad.num_steps = 1
    plan = B.BatchPlan([ok, bad])
    got = plan.run().cpu().numpy()
    assert got[0, 5] == 0
    assert got[1, 5] == N.EOVERFLOW


@pytest.mark.parametrize("bt", [64, 128, 256])
def test_two_paths_per_lane_batch_is_bit_identical(bt):
    """Paths-per-thread tiling in K8 (both chunks of a pair in one instance
    step together; pairs across an instance boundary run one after the
    other): every instance's result equals pricing it alone."""
    insts = B.lower_mix(small_mix(24))
    ref = alone(insts)
    plan = B.BatchPlan(insts)
    nc = plan.header.n_class
    for il in ([2] * nc, [1 + (j % 2) for j in range(nc)]):
        plan.set_config(bt, 2, il)
        np.testing.assert_array_equal(plan.run().cpu().numpy(), ref)
    with pytest.raises(ValueError):
        plan.set_config(bt, 2, [2] * (nc + 1))


def test_batch_overflow_with_two_paths_per_lane():
    ok = inst_for(merton1d(50), num_paths=1000, seed=1)
    bad = inst_for(merton1d(50), num_paths=1000, seed=1)
    bad.rate = 5000.0
    bad.inv_rate = 2e-8
    bad.num_steps = 1
    plan = B.BatchPlan([ok, bad, ok])
    plan.set_config(128, 0, [2] * plan.header.n_class)
    got = plan.run().cpu().numpy()
    assert got[0, 5] == 0 and got[2, 5] == 0
    assert got[1, 5] == N.EOVERFLOW


def test_autotune_choice_gives_same_bits(tmp_path, monkeypatch):
    monkeypatch.setenv("SDEMC_CACHE_DIR", str(tmp_path))
    insts = B.lower_mix(small_mix(16))
    ref = alone(insts)
    plan = B.BatchPlan(insts)
    entry = B.autotune(plan, repeats=1)
    assert len(entry["tried"]) == len(B.CANDIDATES)
    np.testing.assert_array_equal(plan.run().cpu().numpy(), ref)
    plan2 = B.BatchPlan(insts)
    assert B.autotune(plan2)["choice"] == entry["choice"]  # served from the cache
