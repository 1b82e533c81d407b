"""Synthetic workloads of the benchmark configurations (no dataset exists for
this path; instances are drawn from seeded generators with the stated laws).

* :func:`rainbow2d` — call on the max of two Merton assets with
  independent per-asset jumps.
* :func:`basket_mix` — 512 correlated d-dimensional Merton basket
  calls, d ~ U{1..8}, steps = round(exp(U(ln 32, ln 512))), paths =
  round(2^U(12, 18)), K ~ U(0.8, 1.2), sigma_i ~ U(0.1, 0.4), rate ~
  U(0.5, 3), drawn in that order per instance from numpy's default_rng(seed);
  fixed rho = 0.3 pairwise, log-jumps N(-0.1, 0.2), S0 = 1, r = 0.02, T = 1.
  Each instance prices on its own RNG stream (stream id = instance index).
"""
import math

import numpy as np
import torch

from .helpers import get_corr_matrix
from .options import Basket, ConstantShortRate, Rainbow
from .sde import IndependentJumpsMerton, Merton
from .solvers import JumpEulerSolver


def rainbow2d(steps=256, seed=1, device="cuda"):
    corr = get_corr_matrix([0.5])
    sde = IndependentJumpsMerton(0.02, torch.tensor([0.2, 0.3]), [1.0, 1.0], -0.05, 0.15, torch.ones(2), 2,
                                 corr_matrix=corr)
    return JumpEulerSolver(sde, 1.0, steps, seed=seed, device=device), Rainbow(1.0), ConstantShortRate(0.02)


class MixInstance:
    """One pricing request of the mix: solver, payoff, discounter, paths and
    its stream id; `cost` is paths x (steps + rate) x d (relative work)."""

    def __init__(self, idx, solver, payoff, discounter, paths, stream_id):
        self.idx, self.solver, self.payoff, self.discounter = idx, solver, payoff, discounter
        self.paths, self.stream_id = int(paths), int(stream_id)

    @property
    def dim(self):
        return self.solver.sde.dim

    @property
    def cost(self):
        rate = float(torch.as_tensor(self.solver.sde.jump_rate()).sum())
        return self.paths * (self.solver.num_steps + rate) * self.dim


def draw_basket_params(rng):
    d = int(rng.integers(1, 9))
    steps = int(round(math.exp(rng.uniform(math.log(32), math.log(512)))))
    paths = int(round(2 ** rng.uniform(12, 18)))
    strike = float(rng.uniform(0.8, 1.2))
    sigmas = [float(rng.uniform(0.1, 0.4)) for _ in range(d)]
    rate = float(rng.uniform(0.5, 3.0))
    return d, steps, paths, strike, sigmas, rate


def basket_instance(idx, d, steps, paths, strike, sigmas, rate, seed=1, device="cuda"):
    corr = get_corr_matrix([0.3] * (d * (d - 1) // 2)) if d > 1 else None
    sde = Merton(0.02, torch.tensor(sigmas), rate, -0.1, 0.2, torch.ones(d), dim=d, corr_matrix=corr)
    solver = JumpEulerSolver(sde, 1.0, steps, seed=seed, device=device)
    return MixInstance(idx, solver, Basket(strike), ConstantShortRate(0.02), paths, stream_id=idx)


def basket_mix(n=512, rng_seed=0, seed=1, device="cuda"):
    rng = np.random.default_rng(rng_seed)
    return [basket_instance(i, *draw_basket_params(rng), seed=seed, device=device) for i in range(n)]
