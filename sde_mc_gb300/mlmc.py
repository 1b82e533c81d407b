"""Multilevel Monte Carlo with the reference's interface (sde_mc/mlmc.py:7-101).

Level 0 is one fused pricing launch (K1) at levels[0] steps; every finer level
is one coupled launch (K2) whose fine and coarse paths share increments and
marks in the same thread.  Level sums come back in FP64.
"""
import math
import time

import torch

from . import kernels as K
from . import _native as N
from .mc import MCStatistics, finish_stats
from .solvers import level_steps


def _level0(solver, payoff, discounter, n, steps):
    inst = solver.lower(payoff, discounter, num_paths=int(n), num_steps=steps)
    return K.price(inst)


def _level(solver, payoff, discounter, n, fine, coarse):
    inst = solver.lower(payoff, discounter, num_paths=int(n), num_steps=coarse)
    hf, hc = level_steps(solver, fine, coarse)
    return K.mlmc_level(inst, fine, coarse, hf, hc)


def level_estimates(trials, levels, solver, payoff, discounter):
    """Launch every level, then read back (mean, var) per level in FP64.  A
    level allotted no paths (Giles' allocation gives N_l = 0 when the pilot
    saw V_l = 0, e.g. fine and coarse grids made only of jump times) is not
    launched and contributes (0, 0)."""
    outs = [_level0(solver, payoff, discounter, trials[0], levels[0]) if trials[0] > 0 else None]
    for i in range(1, len(levels)):
        outs.append(_level(solver, payoff, discounter, trials[i], levels[i], levels[i - 1]) if trials[i] > 0
                    else None)
    est = []
    for i, o in enumerate(outs):
        if o is None:
            est.append((0.0, 0.0))
            continue
        r = o.cpu().tolist()
        if i == 0:
            N.status_error(r[5], "mc_multilevel level 0")
            est.append((r[3], r[4]))
        else:
            N.status_error(r[7], "mc_multilevel level %d" % i)
            est.append((r[5], r[6]))
    return est


def mc_multilevel(trials, levels, solver, payoff, discounter, bs=None):
    """sum_l E[P_l - P_{l-1}] with sd = sqrt(sum_l V_l / N_l)."""
    start = time.time()
    trials = [int(t) for t in trials]
    est = level_estimates(trials, levels, solver, payoff, discounter)
    mean = sum(m for m, _ in est)
    sd = math.sqrt(sum(v / n for (_, v), n in zip(est, trials) if n > 0))
    return MCStatistics(mean, sd, time.time() - start, trials[-1])


def optimal_trials_from_variances(level_vars, levels, time_interval, epsilon):
    """Giles' allocation N_l = (1.96/eps)^2 sqrt(V_l h_l) sum_k sqrt(V_k / h_k),
    h_l = T / levels[l], in float32 exactly as the reference evaluates it
    (sde_mc/mlmc.py:92-96), rounded up."""
    var = torch.as_tensor(level_vars, dtype=torch.float64).to(torch.float32)
    h = time_interval / torch.tensor(levels)
    total = (var / h).sqrt().sum()
    opt = (1.96 ** 2 / (epsilon * epsilon)) * (var * h).sqrt() * total
    return opt.ceil().long().tolist()


def get_optimal_trials(trials, levels, epsilon, solver, payoff, discounter):
    """Giles' allocation from a pilot of ``trials`` paths per level
    (sde_mc/mlmc.py:77-97).  As the reference does, it leaves the solver's
    num_steps at levels[0]."""
    solver.num_steps = levels[0]
    est = level_estimates([int(trials)] * len(levels), levels, solver, payoff, discounter)
    return optimal_trials_from_variances([v for _, v in est], levels, solver.time_interval, epsilon)


def mlmc_bs_from_trials(trials, levels, max_mem=5 * 10 ** 8, dim=1, max_jumps=0):
    return torch.minimum(max_mem / (dim * (torch.tensor(levels) + max_jumps)), torch.as_tensor(trials)).ceil().long()
