"""Monte Carlo estimators with the reference's interface (sde_mc/mc.py:13-472).

``mc_simple`` with a batch size runs the fused pricing kernel (K1): one launch
simulates every path in registers and returns FP64 (sum, sum_sq, n); nothing
path-shaped touches HBM.  Without a batch size it materialises paths (K4), as
the reference does, so ``.paths``, ``.payoffs`` and ``.normals`` are filled.
The learned control-variate estimators live in :mod:`sde_mc_gb300.varred`.
"""
import math
import time

import numpy as np
import torch

from . import _native as N
from . import kernels as K
from .helpers import sample_cov
from .lowering import is_jump_solver
from .options import ConstantShortRate


class MCStatistics:
    """Result record: sample mean, standard error, wall time and trial count
    (plus paths, payoffs and the solver's auxiliary output when materialised)."""

    def __init__(self, sample_mean, sample_std, time_elapsed, num_trials, paths=None, payoffs=None,
                 normals=None):
        self.sample_mean = sample_mean.item() if torch.is_tensor(sample_mean) else float(sample_mean)
        self.sample_std = sample_std.item() if torch.is_tensor(sample_std) else float(sample_std)
        self.time_elapsed = time_elapsed
        self.num_trials = num_trials
        self.paths = paths
        self.payoffs = payoffs
        self.normals = normals

    def __str__(self):
        return 'Mean: {:.6f}  +/- {:.6f}    Time taken (s): {:.2f}    N: {:.2E}'.format(
            self.sample_mean, self.sample_std * 1.96, self.time_elapsed, self.num_trials)


def _payoff_flags(solver, payoff_time):
    if payoff_time not in ('terminal', 'adapted'):
        raise ValueError("payoff_time must be 'terminal' or 'adapted', got %r" % (payoff_time,))
    if payoff_time == 'terminal' and is_jump_solver(solver):
        return 1  # SDEMC_INST_PAYOFF_AT_NOMINAL_STEP
    return 0


def price_stats(solver, payoff, discounter, num_trials, payoff_time='adapted', cfg=None, payoffs=None,
                path_offset=None):
    """Launch K1 for ``num_trials`` fresh paths; returns the FP64 result tensor
    (sum, sum_sq, n, mean, var, status) on the device, unsynchronised."""
    inst = solver.lower(payoff, discounter, num_paths=int(num_trials), path_offset=path_offset)
    inst.flags |= _payoff_flags(solver, payoff_time)
    return K.price(inst, cfg=cfg, payoffs=payoffs)


def finish_stats(res, what="mc_simple"):
    """Host side of K1's output: check the status, return (mean, se, n)."""
    r = res.cpu().tolist()
    N.status_error(r[5], what)
    n = r[2]
    se = math.sqrt(max(r[4], 0.0) / n) if n > 1 else float('nan')
    return r[3], se, n


def materialise_with_payoffs(solver, num_trials, payoff, discounter, payoff_time):
    """K4 run that also evaluates the payoff in-kernel.  Returns (paths, aux,
    payoffs) laid out as the reference's solve() output."""
    n = int(num_trials)
    inst = solver.lower(payoff, discounter, num_paths=n)
    inst.flags |= _payoff_flags(solver, payoff_time)
    if is_jump_solver(solver):
        cap = solver.num_steps + solver.max_jumps
        out = K.materialise(inst, cap)
        st = int(out["status"].item())
        N.status_error(st, "mc_simple")
        total = int(out["steps"].max().item()) if n > 0 else 0
        T = float(solver.time_interval)
        time_p = out["time"].unsqueeze(-1)
        time_p[:, total + 1:] = T
        out["left"][:, total + 1:] = 0.0
        out["jumps"][:, total + 1:] = 0.0
        out["normals"][:, total:] = 0.0
        aux = (solver._out(out["normals"]), solver._out(time_p), solver._out(out["left"]), total,
               solver._out(out["jumps"]))
        return solver._out(out["paths"][:, :total + 1]), aux, out["payoffs"]
    out = K.materialise(inst, solver.num_steps, want=("paths", "normals", "payoffs", "steps"))
    N.status_error(out["status"].item(), "mc_simple")
    return solver._out(out["paths"]), solver._out(out["normals"]), out["payoffs"]


def mc_simple(num_trials, sde_solver, payoff, discounter=None, bs=None, return_normals=False,
              payoff_time='terminal'):
    """Plain Monte Carlo price of payoff(X_T) * discounter(T).

    ``payoff_time='adapted'`` uses each path's terminal state; 'terminal' keeps
    the reference's reading of storage column num_steps, which for a jump
    solver is the state after num_steps steps (sde_mc/mc.py:84-92)."""
    if discounter is None:
        discounter = ConstantShortRate(r=0.0)
    num_trials = int(num_trials)
    start = time.time()
    if not bs:
        paths, aux, payoffs = materialise_with_payoffs(sde_solver, num_trials, payoff, discounter, payoff_time)
        p64 = payoffs.double()
        mn = p64.mean()
        sd = p64.std() / np.sqrt(num_trials)
        tt = time.time() - start
        return MCStatistics(mn, sd, tt, num_trials, paths, sde_solver._out(payoffs), aux)
    res = price_stats(sde_solver, payoff, discounter, num_trials, payoff_time)
    mean, se, _ = finish_stats(res)
    return MCStatistics(mean, se, time.time() - start, num_trials)


def mc_terminal_cv(num_trials, sde_solver, payoff, discounter=None, bs=None, return_normals=False):
    """Terminal-value control variate: payoff - b (disc X_T^0 - X_0^0), with b
    estimated by regression (on the first batch when ``bs`` is given)."""
    if discounter is None:
        discounter = ConstantShortRate(r=0.0)
    num_trials = int(num_trials)
    start = time.time()
    disc = float(discounter(sde_solver.time_interval))
    x00 = float(torch.as_tensor(sde_solver.sde.init_value).reshape(-1)[0])
    chunks = [num_trials] if not bs else [min(int(bs), num_trials - i) for i in range(0, num_trials, int(bs))]
    b = None
    s = s2 = 0.0
    last = None
    for n in chunks:
        paths, aux, payoffs = materialise_with_payoffs(sde_solver, n, payoff, discounter, 'adapted')
        spots = paths[:, -1].to(payoffs.device)
        cv = disc * spots[:, 0] - x00
        if b is None:
            b = sample_cov(cv, payoffs) / cv.var()
        y = (payoffs - b * cv).double()
        s += float(y.sum())
        s2 += float((y * y).sum())
        last = (paths, payoffs, aux)
    mn = s / num_trials
    sd = math.sqrt(max(s2 / num_trials - mn * mn, 0.0) * num_trials / (num_trials - 1)) / math.sqrt(num_trials)
    if not bs:
        return MCStatistics(mn, sd, time.time() - start, num_trials, last[0], last[1], last[2])
    return MCStatistics(mn, sd, time.time() - start, num_trials)


def find_num_trials(problem, eps, models=None, init_trials=1e5, bs=1e5):
    """Trials needed for a 95% half-width of ``eps`` from a pilot run."""
    payoff_time = 'adapted' if problem.solver.has_jumps else 'terminal'
    if models is None:
        stats = mc_simple(init_trials, problem.solver, problem.payoff, problem.discounter, bs,
                          payoff_time=payoff_time)
    else:
        from .varred import mc_apply_cvs
        stats = mc_apply_cvs(models, problem.solver, init_trials, problem.payoff, problem.discounter, bs)
    ratio = (stats.sample_std * 1.96 / eps) ** 2
    return int(np.ceil(ratio * init_trials))


def find_num_trials_terminal_cv(problem, eps, init_trials, bs):
    stats = mc_terminal_cv(init_trials, problem.solver, problem.payoff, problem.discounter, bs)
    return int(np.ceil((stats.sample_std * 1.96 / eps) ** 2 * init_trials))


def run_mc(problem, eps, bs=1e5, init_trials=1e5):
    trials = find_num_trials(problem, eps, None, init_trials, bs)
    payoff_time = 'adapted' if problem.solver.has_jumps else 'terminal'
    return mc_simple(trials, problem.solver, problem.payoff, problem.discounter, bs=bs, payoff_time=payoff_time)


def run_mc_terminal_cv(problem, eps, bs=1e5, init_trials=1e5):
    trials = find_num_trials_terminal_cv(problem, eps, init_trials, bs)
    return mc_terminal_cv(trials, problem.solver, problem.payoff, problem.discounter, bs=bs)
