"""Host logic of the estimators against the reference's own arithmetic:
Giles' MLMC allocation (get_optimal_trials, sde_mc/mlmc.py:77-97) on level
samples whose allocation the reference itself computed (recorded by
tests/golden/make_golden.py through a stand-in solver)."""
import numpy as np
import torch

from oracle import oracle
from sde_mc_gb300.mlmc import optimal_trials_from_variances
from tests.conftest import load_json


def test_allocation_equals_the_reference_on_the_same_variances():
    for case in load_json("optimal_trials"):
        # the reference's variance of each level's samples: torch.var in float32
        var = [float(torch.tensor(np.asarray(s, np.float32)).var()) for s in case["samples"]]
        got = optimal_trials_from_variances(var, case["levels"], case["T"], case["eps"])
        assert got == case["trials"]
        # the reference leaves the solver at the coarsest level
        assert case["num_steps_after"] == case["levels"][0]


def test_oracle_allocation_agrees_to_rounding():
    """The oracle's FP64 restatement of the same formula: within one path per
    level (the reference rounds its float32 product up)."""
    for case in load_json("optimal_trials"):
        var = [float(np.var(np.asarray(s, np.float64), ddof=1)) for s in case["samples"]]
        ref = np.asarray(case["trials"], np.int64)
        got = oracle.optimal_trials(var, case["levels"], case["T"], case["eps"])
        assert np.all(np.abs(got - ref) <= np.maximum(1, 1e-5 * ref)), (got, ref)
