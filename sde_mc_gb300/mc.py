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
from scipy.stats import poisson  # noqa: F401  (re-exported as in sde_mc)
from torch.utils.data import DataLoader  # noqa: F401  (re-exported as in sde_mc)

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


# ---------------------------------------------------- learned control variates
def simulate_data(trials, solver, payoff, discounter, bs=1000, inference=False):
    """Materialise paths, payoffs and normals into a DataLoader (diffusion
    solvers; sde_mc/mc.py:378-388)."""
    from torch.utils.data import DataLoader
    from .nets import NormalPathData
    if inference:
        assert not trials % bs, 'Batch size should partition total trials evenly'
    stats = mc_simple(trials, solver, payoff, discounter, return_normals=True)
    dset = NormalPathData(stats.paths, stats.payoffs, stats.normals)
    return DataLoader(dset, batch_size=int(bs), shuffle=not inference, drop_last=not inference)


def simulate_adapted_data(trials, solver, payoff, discounter, bs=1000, inference=False):
    """Materialise jump-adapted paths into AdaptedPathData (sde_mc/mc.py:391-398);
    tensors stay on the GPU for the control-variate kernels."""
    from torch.utils.data import DataLoader
    from .nets import AdaptedPathData
    if not is_jump_solver(solver):
        raise ValueError("simulate_adapted_data needs a jump solver")
    paths, aux, payoffs = materialise_with_payoffs(solver, int(trials), payoff, discounter, 'adapted')
    normals, time_paths, left, total, jumps = aux
    S = total
    dset = AdaptedPathData(paths[:, :S + 1].contiguous(), payoffs, normals[:, :S].contiguous(),
                           left[:, :S + 1], time_paths[:, :S + 1].contiguous(), jumps[:, :S + 1], S)
    return DataLoader(dset, batch_size=int(bs), shuffle=not inference, drop_last=not inference)


def sim_train_control_variates(models, opt, solver, trials, payoff, discounter, sim_bs, bs, epochs=10,
                               print_losses=True, tol=0, early_stopping=None):
    from .varred import train_adapted_control_variates, train_diffusion_control_variate
    if solver.has_jumps:
        dl = simulate_adapted_data(trials, solver, payoff, discounter, bs=bs)
        return train_adapted_control_variates(models, opt, dl, solver, discounter, epochs, print_losses, tol,
                                              early_stopping)
    dl = simulate_data(trials, solver, payoff, discounter, bs=bs)
    return train_diffusion_control_variate(models, opt, dl, solver, discounter, epochs, print_losses, tol,
                                           early_stopping)[1]


def mc_apply_cvs(models, solver, trials, payoff, discounter, sim_bs=1e5, bs=1000, tol=0):
    """Plain estimate of Gamma = payoff + control variate over fresh paths
    (sde_mc/mc.py:195-242)."""
    from .helpers import mc_estimates
    from .varred import (apply_adapted_control_variates, apply_diffusion_control_variate, fused_cv_stats,
                         fused_supported)
    start = time.time()
    trials = int(trials)
    if solver.has_jumps and fused_supported(models, solver, discounter, tol):
        # K7: the same fresh paths, simulated and evaluated in one pass
        r = fused_cv_stats(models, solver, payoff, discounter, trials).cpu().tolist()
        N.status_error(r[7], "mc_apply_cvs")
        return MCStatistics(r[5], math.sqrt(max(r[6], 0.0)) / math.sqrt(trials), time.time() - start, trials)
    s = s2 = 0.0
    left = trials
    while left > 0:
        n = int(min(sim_bs, left))
        left -= n
        if solver.has_jumps:
            dl = simulate_adapted_data(n, solver, payoff, discounter, bs=bs, inference=True)
            a, b = apply_adapted_control_variates(models, dl, solver, discounter, tol)
        else:
            dl = simulate_data(n, solver, payoff, discounter, bs=n, inference=True)
            a, b = apply_diffusion_control_variate(models, dl, solver, discounter, tol)
        s += float(a)
        s2 += float(b)
    mn, var = mc_estimates(s, s2, trials)
    return MCStatistics(mn, math.sqrt(max(var, 0.0)) / math.sqrt(trials), time.time() - start, trials)


def mc_adaptive_cv(models, opt, solver, trials, steps, payoff, discounter, sim_bs=(1e4, 1e4), bs=(1000, 1000),
                   epochs=10, print_losses=True, pre_trained=False, tol=0, early_stopping=None):
    """Train on a coarse grid, then estimate with the control variate on the
    fine grid (sde_mc/mc.py:245-326)."""
    from .varred import train_adapted_control_variates
    train_trials, test_trials = trials
    train_steps, test_steps = steps
    train_bs, test_bs = bs
    train_sim_bs, test_sim_bs = sim_bs
    solver.num_steps = train_steps
    if early_stopping is not None:
        early_stopping.batch_size = bs[1]
    t0 = time.time()
    if not pre_trained:
        dl = simulate_adapted_data(train_trials, solver, payoff, discounter, bs=train_bs)
        train_adapted_control_variates(models, opt, dl, solver, discounter, epochs, print_losses, tol,
                                       early_stopping=early_stopping)
    train_time = time.time() - t0
    solver.num_steps = test_steps
    st = mc_apply_cvs(models, solver, test_trials, payoff, discounter, test_sim_bs, test_bs, tol)
    st.time_elapsed += train_time
    return st


def mc_control_variates(models, opt, solver, trials, steps, payoff, discounter, sim_bs=(1e5, 1e5),
                        bs=(1000, 1000), epochs=10, print_losses=True, tol=0, early_stopping=None):
    """Diffusion-solver variant of mc_adaptive_cv (sde_mc/mc.py:126-192)."""
    assert not solver.has_jumps
    train_trials, test_trials = trials
    train_steps, test_steps = steps
    train_bs, test_bs = bs
    train_sim_bs, test_sim_bs = sim_bs
    solver.num_steps = train_steps
    if early_stopping is not None:
        early_stopping.batch_size = bs[1]
    t0 = time.time()
    sim_train_control_variates(models, opt, solver, train_trials, payoff, discounter, train_sim_bs, train_bs, epochs,
                               print_losses, tol, early_stopping)
    t1 = time.time()
    solver.num_steps = test_steps
    st = mc_apply_cvs(models, solver, test_trials, payoff, discounter, test_sim_bs, test_bs, tol)
    st.time_elapsed += t1 - t0
    return st


def sample_batch_cost(solver, option, discounter, models, trials, bs, nn_bs):
    out = mc_apply_cvs(models, solver, trials, option, discounter, bs, nn_bs)
    return out.time_elapsed / (trials / nn_bs)


def run_cv_mc(problem, models, opt, eps, train_size, step_factor=30, sim_bs=1e5, train_bs=1e3, nn_bs=1e3, epochs=10,
              early_stopping=False, print_losses=True, init_trials=1e5):
    """Train on a grid step_factor times coarser, size the run for a 95%
    half-width eps from a pilot, then estimate with the control variate
    (sde_mc/mc.py:443-467)."""
    from .helpers import ceil_mult
    from .varred import EarlyStopping
    es = None
    if early_stopping:
        cost_batch = sample_batch_cost(problem.solver, problem.payoff, problem.discounter, models, sim_bs, sim_bs,
                                       nn_bs)
        es = EarlyStopping(eps, 1.96, cost_batch, 1)
        es.batch_size = nn_bs
    steps = problem.solver.num_steps
    problem.solver.num_steps = int(np.ceil(steps / step_factor))
    t0 = time.time()
    sim_train_control_variates(models, opt, problem.solver, train_size, problem.payoff, problem.discounter, sim_bs,
                               train_bs, epochs, print_losses, 0, es)
    train_time = time.time() - t0
    problem.solver.num_steps = steps
    trials = ceil_mult(find_num_trials(problem, eps, models, init_trials, sim_bs), nn_bs)
    st = mc_apply_cvs(models, problem.solver, trials, problem.payoff, problem.discounter, sim_bs, nn_bs)
    test_time = st.time_elapsed
    st.time_elapsed += train_time
    return st, train_time, test_time
